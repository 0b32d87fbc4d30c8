"""Host logic: design builder, DMI flattening, canonical draws, ABI layout."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_fixture
from ggdmc_gb300 import abi
from ggdmc_gb300.design import build_lba_model, design_bv13, design_t0_17


def test_design_bv13_matches_fixture6():
    z, model, *_ = load_fixture(6)
    m = design_bv13()
    assert m.pnames == model.pnames and m.cell_names == model.cell_names
    assert np.array_equal(m.param_src, model.param_src) and np.array_equal(m.resp, model.resp)


def test_design_t0_matches_fixture5_structure():
    z, model, *_ = load_fixture(5)
    cjk = build_lba_model(
        p_map={"A": ["1"], "B": ["1"], "mean_v": ["S", "M"], "sd_v": ["M"], "st0": ["1"],
               "t0": ["HANDEDNESS", "MOTOR_SKILL"]},
        match_map={"M": {"紅": "反應東", "黃": "反應南", "藍": "反應西", "綠": "反應北"}},
        factors={"S": ["紅", "黃", "藍", "綠"], "HANDEDNESS": ["left_hander", "right_hander"],
                 "MOTOR_SKILL": ["excellent", "good", "poor"]},
        constants={"st0": 0, "sd_v.false": 1}, accumulators=["反應東", "反應南", "反應西", "反應北"])
    assert cjk.pnames == model.pnames and cjk.cell_names == model.cell_names
    assert np.array_equal(cjk.param_src, model.param_src)
    m = design_t0_17()
    assert m.n_par == 17 and m.n_acc == 4 and m.n_cell == 96


def test_philox_known_answers(oracle):
    # Random123 Philox4x32-10 known-answer vectors
    kat = [([0, 0, 0, 0], 0, 0, [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
           ([0xffffffff] * 4, 0xffffffff, 0xffffffff,
            [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
           ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], 0xa4093822, 0x299f31d0,
            [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1])]
    for ctr, k0, k1, want in kat:
        a = (C.c_uint32 * 4)(*ctr)
        oracle.lib().oracle_philox(a, k0, k1)
        assert list(a) == want


def test_uniforms_in_open_unit_interval(oracle):
    u = np.array([oracle.uniform(123, 1, l, 0, s) for l in range(3) for s in range(200)])
    assert np.all((u > 0) & (u < 1))
    assert abs(u.mean() - 0.5) < 0.05


def test_draw_layout_python_matches_c(oracle):
    from ggdmc_gb300 import build, gpu
    build.build()
    L = gpu.lib()   # ggdmc_draw_layout touches no device
    for hier in (0, 1):
        for hb, pb in ((0, 0), (1, 0), (0, 1), (1, 1)):
            cfg = abi.DEConfigPy(nchain=39, nparameter=26 if hier else 13, nmc=11, thin=3,
                                 is_hblocked=bool(hb), is_pblocked=bool(pb))
            out = [C.c_int64() for _ in range(4)]
            cc = cfg.to_c()
            assert L.ggdmc_draw_layout(C.byref(cc), 5, hier, *[C.byref(o) for o in out]) == 0
            ni, npass, ns = abi.draw_layout(cfg, 5, bool(hier))
            assert (out[0].value, out[1].value, out[2].value) == (ni, npass, ns)
            assert out[3].value == ni * 5 * npass * ns


def test_library_exports_every_declared_symbol():
    from ggdmc_gb300 import build
    lib_path = build.build()
    declared = set()
    for name in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if name.endswith(".h"):
            header = open(os.path.join(ROOT, "include", name)).read()
            declared |= set(re.findall(r"\b(ggdmc_[a-z0-9_]+)\s*\(", header))
    declared -= {"ggdmc_status"}
    lib = C.CDLL(lib_path)
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, missing
    assert len(declared) >= 21


def test_error_paths_without_device():
    # argument checks run before any CUDA call
    from ggdmc_gb300 import gpu
    L = gpu.lib()
    cfg = abi.DEConfigPy(nchain=2, nparameter=13).to_c()
    n = C.c_int64()
    assert L.ggdmc_draw_layout(C.byref(cfg), 1, 0, C.byref(n), None, None, None) == abi.GGDMC_ERR_ARG
    assert b"three or more chains" in L.ggdmc_last_error()


def test_dmi_flatten_roundtrip():
    z, model, sub, pop = load_fixture(6)
    assert pop.n_subject == 32 and pop.counts.sum() == len(pop.rt)
    cv = model.cell_values(z["sub_theta"][0])
    assert cv.shape == (model.n_cell, 2, 6)
    # the responding accumulator is node 1: its mean_v is the cell's match/mismatch rate
    assert set(np.unique(model.resp)) == {0, 1}


def test_rda_reader_on_reference_fixture():
    # GGDMC_REFERENCE names a checkout of the reference package (the fixture
    # files are read from it); the test is skipped without one
    ref = os.environ.get("GGDMC_REFERENCE")
    if not ref:
        pytest.skip("GGDMC_REFERENCE is not set")
    path = os.path.join(ref, "tests/testthat/Group1/data/lba_data6.rda")
    if not os.path.exists(path):
        pytest.skip("reference checkout not present")
    from ggdmc_gb300.dmi import model_from_dmi
    from ggdmc_gb300.rda import load_rda
    d = load_rda(path)
    m = model_from_dmi(d["sub_dmis"][0])
    assert m.pnames == design_bv13().pnames
