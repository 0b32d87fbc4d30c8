"""Build a flattened LBA design from a ggdmcModel-style specification.

ggdmcModel::BuildModel(p_map, match_map, factors, constants, accumulators)
(used by every fixture generator, e.g. tests/testthat/Group1/data/
6_lba_Bv_model.r:28-39 and README.md:31-42) names parameters and cells by
these rules, which the fixtures' model objects show:

* a cell is one combination of factor levels plus a response, named
  ``level1.level2....response``; cells are sorted by name;
* parameter ``q`` mapped to factors ``(F1, F2, ...)`` is named
  ``q.levelF1.levelF2...`` in p_map order; ``"1"`` means no factors; the
  match factor ``M`` contributes ``true`` when the accumulator is the one
  match_map pairs with the stimulus level, else ``false``;
* free parameters (``pnames``) are the sorted names minus the constants.

This mirrors those rules so synthetic workloads and tests can build designs
without R.  Names sort by code point, which equals R's order for the ASCII
and CJK labels the fixtures use.
"""

from __future__ import annotations

import itertools

import numpy as np

from .dmi import DDM_KINDS, LBA_KINDS, MODEL_DDM, MODEL_LBA, FlatModel


def _param_name(q, facs, levels, acc, match_factor, match_map):
    parts = [q]
    for f in facs:
        if f == "1":
            continue
        if f == "M":
            stim = levels[match_factor]
            parts.append("true" if match_map[stim] == acc else "false")
        else:
            parts.append(levels[f])
    return ".".join(parts)


def build_lba_model(p_map: dict, match_map: dict, factors: dict, constants: dict,
                    accumulators: list) -> FlatModel:
    """p_map: kind -> list of factor names ("1", "M" allowed);
    match_map: {"M": {stimulus_level: accumulator}}; factors: name -> levels."""
    mm = match_map.get("M", {})
    match_factor = None
    for f, levs in factors.items():
        if mm and set(mm).issubset(set(levs)):
            match_factor = f
            break
    fnames = list(factors)
    combos = [dict(zip(fnames, c)) for c in itertools.product(*[factors[f] for f in fnames])]
    # every parameter name that appears anywhere
    all_names = set()
    table = {}
    for lv in combos:
        for acc in accumulators:
            for q in LBA_KINDS:
                facs = p_map.get(q, ["1"])
                if isinstance(facs, str):
                    facs = [facs]
                name = _param_name(q, facs, lv, acc, match_factor, mm)
                table[(tuple(lv[f] for f in fnames), acc, q)] = name
                all_names.add(name)
    const_names = sorted(constants)
    pnames = sorted(n for n in all_names if n not in constants)
    cells = []
    for lv in combos:
        for r in accumulators:
            cells.append((".".join([lv[f] for f in fnames] + [r]), lv, r))
    cells.sort(key=lambda c: c[0])
    K = len(accumulators)
    src = np.zeros((len(cells), K, len(LBA_KINDS)), np.int32)
    resp = np.zeros(len(cells), np.int32)
    for ci, (cname, lv, r) in enumerate(cells):
        resp[ci] = accumulators.index(r)
        key = tuple(lv[f] for f in fnames)
        for k, acc in enumerate(accumulators):
            for qi, q in enumerate(LBA_KINDS):
                name = table[(key, acc, q)]
                src[ci, k, qi] = pnames.index(name) if name in pnames \
                    else -1 - const_names.index(name)
    return FlatModel(MODEL_LBA, pnames, list(accumulators), [c[0] for c in cells],
                     np.array([float(constants[c]) for c in const_names]), const_names,
                     src, resp)


def design_rows(model: FlatModel):
    """Distinct stimulus conditions: cell-name prefixes without the response,
    each with the cell index of every response."""
    rows = {}
    for ci, name in enumerate(model.cell_names):
        prefix = name.rsplit(".", 1)[0]
        rows.setdefault(prefix, {})[model.accumulators[model.resp[ci]]] = ci
    return [(p, [d[a] for a in model.accumulators]) for p, d in sorted(rows.items())]


# --------------------------------------------------------- reference designs
def design_bv13() -> FlatModel:
    """The 13-parameter B x v design of lba_data6 / README.md:31-42:
    2 accumulators, S x COLOR x NOISE (12 conditions, 24 cells)."""
    return build_lba_model(
        p_map={"A": ["1"], "B": ["S", "COLOR"], "t0": ["1"], "mean_v": ["NOISE", "M"],
               "sd_v": ["M"], "st0": ["1"]},
        match_map={"M": {"left": "z_key", "right": "x_key"}},
        factors={"S": ["left", "right"], "COLOR": ["red", "blue"],
                 "NOISE": ["high", "moderate", "low"]},
        constants={"st0": 0.0, "sd_v.false": 1.0},
        accumulators=["z_key", "x_key"])


def design_t0_17() -> FlatModel:
    """The 17-parameter, 4-accumulator design of lba_data5
    (5_lba_t0_model.r:24-31) with ASCII labels: mean_v by S x M, t0 by
    HANDEDNESS x MOTOR_SKILL (24 conditions, 96 cells)."""
    return build_lba_model(
        p_map={"A": ["1"], "B": ["1"], "mean_v": ["S", "M"], "sd_v": ["M"], "st0": ["1"],
               "t0": ["HANDEDNESS", "MOTOR_SKILL"]},
        match_map={"M": {"red": "east", "yellow": "south", "blue": "west", "green": "north"}},
        factors={"S": ["red", "yellow", "blue", "green"],
                 "HANDEDNESS": ["left_hander", "right_hander"],
                 "MOTOR_SKILL": ["excellent", "good", "poor"]},
        constants={"st0": 0.0, "sd_v.false": 1.0},
        accumulators=["east", "south", "west", "north"])


# README.md:78-88 / 6_lba_Bv_model.r:41-65 population and p_vector values
BV13_POP_MEAN = {
    "A": 0.25, "B.left.red": 2.33, "B.right.red": 2.13, "B.left.blue": 2.55,
    "B.right.blue": 2.35, "t0": 0.05, "mean_v.high.true": 2.1, "mean_v.moderate.true": 3.1,
    "mean_v.low.true": 4.1, "mean_v.high.false": 1.82, "mean_v.moderate.false": 1.70,
    "mean_v.low.false": 1.5, "sd_v.true": 0.2}
BV13_POP_SCALE = {
    "A": 0.2, "B.left.red": .23, "B.right.red": .23, "B.left.blue": .255, "B.right.blue": .235,
    "t0": 0.05, "mean_v.high.true": .25, "mean_v.moderate.true": .35, "mean_v.low.true": .45,
    "mean_v.high.false": .182, "mean_v.moderate.false": .170, "mean_v.low.false": .15,
    "sd_v.true": 0.2}

# 5_lba_t0_model.r:33-45 values, relabelled
T0_17_P = {
    "A": 0.25, "B": 1.33,
    "t0.left_hander.excellent": 0.11, "t0.right_hander.excellent": 0.01,
    "t0.left_hander.good": 0.12, "t0.right_hander.good": 0.02,
    "t0.left_hander.poor": 0.13, "t0.right_hander.poor": 0.03,
    "mean_v.red.true": 2.5, "mean_v.yellow.true": 2.7, "mean_v.blue.true": 2.9,
    "mean_v.green.true": 3.1, "mean_v.red.false": 1.24, "mean_v.yellow.false": 1.52,
    "mean_v.blue.false": 1.44, "mean_v.green.false": 1.72, "sd_v.true": 0.2}


def design_ddm9() -> FlatModel:
    """Ratcliff diffusion design with 9 parameters: a, v per stimulus (2
    levels), z, d, sz, sv, t0, st0 (z and sz relative to a).  Two responses:
    r1 is the lower boundary, r2 the upper; cells are stimulus x response."""
    pnames = ["a", "v.s1", "v.s2", "z", "d", "sz", "sv", "t0", "st0"]
    accs = ["r1", "r2"]
    cells = [f"{st}.{rsp}" for st in ("s1", "s2") for rsp in accs]
    src = np.zeros((len(cells), 2, len(DDM_KINDS)), np.int32)
    for c, name in enumerate(cells):
        st = name.split(".")[0]
        src[c, :, :] = [pnames.index(k) for k in ("a", f"v.{st}", "z", "d", "sz", "sv", "t0", "st0")]
    resp = np.array([accs.index(n.split(".")[1]) for n in cells], np.int32)
    return FlatModel(MODEL_DDM, pnames, accs, cells, np.zeros(0), [], src, resp, DDM_KINDS)


# population values of the diffusion design (rtdists-style magnitudes)
DDM9_P = {"a": 1.0, "v.s1": -1.5, "v.s2": 1.5, "z": 0.5, "d": 0.02, "sz": 0.2, "sv": 0.5,
          "t0": 0.3, "st0": 0.15}


def vector(model: FlatModel, values: dict) -> np.ndarray:
    return np.array([values[n] for n in model.pnames], np.float64)
