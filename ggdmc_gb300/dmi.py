"""Flat, device-ready form of ggdmc's model / data-model-instance (DMI) objects.

ggdmc describes a design with an S4 ``model`` (ggdmcModel::BuildModel) and
binds data to it in an S4 ``dmi`` (ggdmcModel::BuildDMI).  The fields this
module consumes are the ones the reference's likelihood reads through
``new_likelihood(dmi)`` (src/de2R.cpp:13, src/de2R.cpp:129):

* ``model@model_boolean[ncell, npxc, K]`` -- which parameter-by-condition name
  applies to accumulator ``k`` in cell ``c`` (column-major logical array);
* ``model@parameter_x_condition_names`` / ``model@pnames`` / ``model@constants``
  -- the names behind the middle axis, the free-parameter order of theta, and
  the fixed values;
* ``dmi@data`` -- a named list of RT vectors, one per non-empty cell;
* ``dmi@node_1_index[ncell, K]`` -- a permutation of the accumulators per cell
  with the responding accumulator first (0-based).

The flat form replaces the boolean cube by one integer per (cell, accumulator,
parameter kind): ``src >= 0`` indexes theta, ``src < 0`` is ``-1 - j`` into the
constants vector.  Trials are laid out subject-major with a per-trial cell
index, which is what the CUDA kernels stage into shared memory.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .rda import RS4, RList, RVector

# Parameter kinds of the LBA accumulator, in the order the kernels read them.
LBA_KINDS = ("A", "B", "mean_v", "sd_v", "t0", "st0")
# Parameter kinds of the Ratcliff diffusion model.
DDM_KINDS = ("a", "v", "z", "d", "sz", "sv", "t0", "st0")

MODEL_LBA = 0
MODEL_DDM = 1


@dataclass
class FlatModel:
    """A design, flattened: what the C-ABI's ``ggdmc_model`` struct carries."""
    model_type: int                 # MODEL_LBA or MODEL_DDM
    pnames: list                    # free-parameter names, theta order
    accumulators: list              # accumulator / response names
    cell_names: list                # all cells, the model's order
    constants: np.ndarray           # float64 [n_const]
    const_names: list
    param_src: np.ndarray           # int32 [n_cell, K, n_kind]
    resp: np.ndarray                # int32 [n_cell]: responding accumulator
    kinds: tuple = LBA_KINDS

    @property
    def n_par(self) -> int:
        return len(self.pnames)

    @property
    def n_cell(self) -> int:
        return len(self.cell_names)

    @property
    def n_acc(self) -> int:
        return len(self.accumulators)

    def cell_values(self, theta: np.ndarray) -> np.ndarray:
        """float64 [n_cell, K, n_kind]: each parameter kind resolved for theta."""
        theta = np.asarray(theta, dtype=np.float64)
        src = self.param_src
        out = np.where(src >= 0, theta[np.clip(src, 0, None)],
                       self.constants[np.clip(-1 - src, 0, None)] if len(self.constants)
                       else 0.0)
        return out


@dataclass
class SubjectData:
    """Trials of one subject: RT in seconds and the cell each trial belongs to."""
    rt: np.ndarray                  # float64 [N]
    cell: np.ndarray                # int32 [N], index into FlatModel.cell_names
    name: str = ""


@dataclass
class SubjectBatch:
    """All subjects packed back to back (the HBM layout the kernels read)."""
    rt: np.ndarray                  # float64 [sum N_s]
    cell: np.ndarray                # int32 [sum N_s]
    offsets: np.ndarray             # int64 [S + 1]
    names: list = field(default_factory=list)

    @property
    def n_subject(self) -> int:
        return len(self.offsets) - 1

    @property
    def counts(self) -> np.ndarray:
        return np.diff(self.offsets)

    @staticmethod
    def pack(subjects) -> "SubjectBatch":
        offs = np.zeros(len(subjects) + 1, dtype=np.int64)
        offs[1:] = np.cumsum([len(s.rt) for s in subjects])
        rt = np.concatenate([np.asarray(s.rt, np.float64) for s in subjects]) \
            if subjects else np.zeros(0)
        cell = np.concatenate([np.asarray(s.cell, np.int32) for s in subjects]) \
            if subjects else np.zeros(0, np.int32)
        return SubjectBatch(rt, cell, offs, [s.name for s in subjects])

    def subject(self, s: int) -> SubjectData:
        a, b = self.offsets[s], self.offsets[s + 1]
        return SubjectData(self.rt[a:b], self.cell[a:b],
                           self.names[s] if s < len(self.names) else "")


def _strs(v) -> list:
    if v is None:
        return []
    if isinstance(v, RVector):
        return [str(x) for x in v.data]
    return [str(x) for x in v]


def model_from_s4(model: RS4, node_1_index=None) -> FlatModel:
    """Flatten an S4 ``model`` (plus a DMI's ``node_1_index``) to a FlatModel."""
    mtype = str(model["type"].data[0]) if isinstance(model["type"], RVector) else "lba"
    kinds = DDM_KINDS if mtype in ("ddm", "diffusion", "rd") else LBA_KINDS
    mb = model["model_boolean"].array()           # [ncell, npxc, K]
    pxc = _strs(model["parameter_x_condition_names"])
    pnames = _strs(model["pnames"])
    cvec = model["constants"]
    if isinstance(cvec, RVector):
        const_names = cvec.names or []
        constants = np.asarray(cvec.data, np.float64)
    else:
        const_names, constants = [], np.zeros(0)
    cells = _strs(model["cell_names"])
    accs = _strs(model["accumulators"])
    ncell, npxc, K = mb.shape
    src = np.full((ncell, K, len(kinds)), np.iinfo(np.int32).min, dtype=np.int32)
    for j, name in enumerate(pxc):
        kind = name.split(".")[0]
        if kind not in kinds:
            raise ValueError(f"unknown parameter kind {kind!r} in {name!r}")
        q = kinds.index(kind)
        if name in pnames:
            code = pnames.index(name)
        elif name in const_names:
            code = -1 - const_names.index(name)
        else:
            raise ValueError(f"{name!r} is neither free nor constant")
        for c in range(ncell):
            for k in range(K):
                if mb[c, j, k]:
                    src[c, k, q] = code
    if (src == np.iinfo(np.int32).min).any():
        raise ValueError("model_boolean leaves a (cell, accumulator, kind) unset")
    if node_1_index is not None:
        n1 = np.asarray(node_1_index, dtype=np.int64)
        resp = n1[:, 0].astype(np.int32)
    else:
        resp = np.array([accs.index(c.split(".")[-1]) for c in cells], np.int32)
    return FlatModel(MODEL_DDM if kinds is DDM_KINDS else MODEL_LBA, pnames, accs,
                     cells, constants, list(const_names), src, resp, kinds)


def subject_from_dmi(dmi: RS4, model: FlatModel, name: str = "") -> SubjectData:
    """Trials of one S4 ``dmi``: ``dmi@data`` cells in list order, RTs as stored."""
    data = dmi["data"]
    rts, cells = [], []
    for cname, vec in zip(data.names, data.items):
        ci = model.cell_names.index(cname)
        r = np.asarray(vec.data, np.float64)
        rts.append(r)
        cells.append(np.full(len(r), ci, np.int32))
    rt = np.concatenate(rts) if rts else np.zeros(0)
    cell = np.concatenate(cells) if cells else np.zeros(0, np.int32)
    return SubjectData(rt, cell, name)


def model_from_dmi(dmi: RS4) -> FlatModel:
    n1 = dmi["node_1_index"]
    n1 = n1.array() if isinstance(n1, RVector) else None
    return model_from_s4(dmi["model"], n1)


def prior_table(p_prior: RList) -> np.ndarray:
    """float64 [P, 6] = (p0, p1, lower, upper, dist_id, log_p) per parameter.

    This is ggdmcPrior's per-parameter list as the reference hands it to
    ``prior::new_prior`` (src/de2R.cpp:12,34-35,127-128); dist_id 1 is the
    truncated normal and 6 the uniform.
    """
    rows = []
    for item in p_prior.items:
        vals = {k: (float(v.data[0]) if isinstance(v, RVector) and len(v.data) else np.nan)
                for k, v in zip(item.names, item.items)}
        lo = vals.get("lower", np.nan)
        hi = vals.get("upper", np.nan)
        rows.append([vals["p0"], vals["p1"],
                     -np.inf if np.isnan(lo) else lo,
                     np.inf if np.isnan(hi) else hi,
                     vals["dist_id"], vals.get("log_p", 1.0)])
    return np.asarray(rows, np.float64)
