"""The plain-C conversions of include/ggdmc_dmi.h (what the .Call shim uses)
against ggdmc_gb300/dmi.py and the golden vectors, on the raw S4 slots of the
reference's own fixtures (tests/golden/dmi_raw_fx*.npz: model_boolean as R
stores it, column-major, the parameter and cell names, the data list and the
prior list).  No GPU is needed: the converters are host code in the library.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN
from ggdmc_gb300 import abi
from ggdmc_gb300.dmi import LBA_KINDS

P_I32 = C.POINTER(C.c_int32)
P_DBL = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def lib():
    from ggdmc_gb300 import build
    L = C.CDLL(build.build())
    L.ggdmc_dmi_n_kind.restype = C.c_int32
    L.ggdmc_dmi_param_src.argtypes = [C.c_int32, P_I32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                      C.c_int32, C.c_void_p, C.c_int32, P_I32]
    L.ggdmc_dmi_responders.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, P_I32]
    L.ggdmc_dmi_trials.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, P_I32, C.c_int32, P_DBL,
                                   P_I32, C.c_int64, C.POINTER(C.c_int64)]
    L.ggdmc_prior_row.argtypes = [C.c_void_p, P_DBL, C.c_int32, P_DBL]
    L.ggdmc_transpose.argtypes = [P_DBL, C.c_int32, C.c_int32, P_DBL]
    return L


def cstrs(names):
    arr = (C.c_char_p * len(names))(*[str(n).encode() for n in names])
    return arr


def raw(fx):
    return dict(np.load(os.path.join(GOLDEN, f"dmi_raw_fx{fx}.npz")))


@pytest.mark.parametrize("fx", [3, 6])
def test_param_src_and_responders_match_dmi_py_and_golden(lib, fx):
    from conftest import load_fixture
    z, model, _, _ = load_fixture(fx)
    r = raw(fx)
    ncell, npxc, K = (int(x) for x in r["model_boolean_dim"])
    mb = np.ascontiguousarray(r["model_boolean"], np.int32)
    out = np.zeros((ncell, K, len(LBA_KINDS)), np.int32)
    st = lib.ggdmc_dmi_param_src(abi.MODEL_LBA, mb.ctypes.data_as(P_I32), ncell, npxc, K, cstrs(r["pxc_names"]),
                                 cstrs(r["pnames"]), len(r["pnames"]), cstrs(r["const_names"]),
                                 len(r["const_names"]), out.ctypes.data_as(P_I32))
    assert st == 0
    np.testing.assert_array_equal(out, model.param_src)          # dmi.py's flattening
    np.testing.assert_array_equal(out, z["param_src"])           # the golden vectors
    resp = np.zeros(ncell, np.int32)
    assert lib.ggdmc_dmi_responders(cstrs(r["cell_names"]), ncell, cstrs(r["accumulators"]), K,
                                    resp.ctypes.data_as(P_I32)) == 0
    np.testing.assert_array_equal(resp, z["resp"])


@pytest.mark.parametrize("fx", [3, 6])
def test_trials_in_list_order(lib, fx):
    from conftest import load_fixture
    z, model, sub, _ = load_fixture(fx)
    r = raw(fx)
    names, lens, rts = r["data_names"], r["data_len"].astype(np.int32), r["data_rt"]
    offs = np.concatenate([[0], np.cumsum(lens)])
    vecs = [np.ascontiguousarray(rts[offs[i]:offs[i + 1]]) for i in range(len(lens))]
    ptrs = (P_DBL * len(vecs))(*[v.ctypes.data_as(P_DBL) for v in vecs])
    n = C.c_int64()
    cells = cstrs(r["cell_names"])
    assert lib.ggdmc_dmi_trials(cells, len(r["cell_names"]), cstrs(names), ptrs, lens.ctypes.data_as(P_I32),
                                len(lens), None, None, 0, C.byref(n)) == 0
    assert n.value == len(sub.rt)
    rt = np.zeros(n.value)
    cell = np.zeros(n.value, np.int32)
    assert lib.ggdmc_dmi_trials(cells, len(r["cell_names"]), cstrs(names), ptrs, lens.ctypes.data_as(P_I32),
                                len(lens), rt.ctypes.data_as(P_DBL), cell.ctypes.data_as(P_I32), n.value,
                                C.byref(n)) == 0
    np.testing.assert_array_equal(rt, sub.rt)
    np.testing.assert_array_equal(cell, sub.cell)
    # a data cell the model does not have is an error
    bad = np.array(list(names[:-1]) + ["no.such.cell"])
    assert lib.ggdmc_dmi_trials(cells, len(r["cell_names"]), cstrs(bad), ptrs, lens.ctypes.data_as(P_I32),
                                len(lens), rt.ctypes.data_as(P_DBL), cell.ctypes.data_as(P_I32), n.value,
                                C.byref(n)) == abi.GGDMC_ERR_ARG


@pytest.mark.parametrize("fx", [3, 6])
def test_prior_rows(lib, fx):
    from conftest import load_fixture
    z, *_ = load_fixture(fx)
    r = raw(fx)
    for j in range(r["prior_fields"].shape[0]):
        row = np.zeros(6)
        vals = np.ascontiguousarray(r["prior_values"][j])
        assert lib.ggdmc_prior_row(cstrs(r["prior_fields"][j]), vals.ctypes.data_as(P_DBL), len(vals),
                                   row.ctypes.data_as(P_DBL)) == 0
        np.testing.assert_array_equal(row, z["sub_prior"][j])
    # NA bounds are open; a missing dist_id is an error
    row = np.zeros(6)
    vals = np.array([0.5, 2.0, np.nan, np.nan, 1.0])
    assert lib.ggdmc_prior_row(cstrs(["p0", "p1", "lower", "upper", "dist_id"]), vals.ctypes.data_as(P_DBL), 5,
                               row.ctypes.data_as(P_DBL)) == 0
    np.testing.assert_array_equal(row, [0.5, 2.0, -np.inf, np.inf, 1.0, 1.0])
    assert lib.ggdmc_prior_row(cstrs(["p0", "p1"]), vals.ctypes.data_as(P_DBL), 2,
                               row.ctypes.data_as(P_DBL)) == abi.GGDMC_ERR_ARG


def test_param_src_rejects_unknown_names(lib):
    mb = np.ones(2 * 1 * 2, np.int32)
    out = np.zeros((2, 2, 6), np.int32)
    args = (abi.MODEL_LBA, mb.ctypes.data_as(P_I32), 2, 1, 2)
    assert lib.ggdmc_dmi_param_src(*args, cstrs(["zz.x"]), cstrs(["zz.x"]), 1, None, 0,
                                   out.ctypes.data_as(P_I32)) == abi.GGDMC_ERR_ARG     # unknown kind
    assert lib.ggdmc_dmi_param_src(*args, cstrs(["A"]), cstrs(["B"]), 1, None, 0,
                                   out.ctypes.data_as(P_I32)) == abi.GGDMC_ERR_ARG     # not free, not constant
    assert lib.ggdmc_dmi_param_src(*args, cstrs(["A"]), cstrs(["A"]), 1, None, 0,
                                   out.ctypes.data_as(P_I32)) == abi.GGDMC_ERR_ARG     # kinds left unset


def test_transpose_hyper_matrix(lib):
    x = np.arange(12, dtype=np.float64).reshape(3, 4)              # [n_row, P] as numpy rows
    colmajor = np.ascontiguousarray(x.T).ravel()                    # how R stores it
    out = np.zeros(12)
    assert lib.ggdmc_transpose(colmajor.ctypes.data_as(P_DBL), 3, 4, out.ctypes.data_as(P_DBL)) == 0
    np.testing.assert_array_equal(out.reshape(3, 4), x)


def test_r_shim_compiles_against_the_r_api_declarations(tmp_path):
    """The .Call shim needs R's headers, which are not installed here.  It is
    compiled (syntax and types only) against tests/rshim_stub/, a header that
    declares the R C API entry points the shim uses with R's signatures."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    root = os.path.dirname(os.path.dirname(GOLDEN))
    shim = os.path.join(root, "ggdmc_gb300", "rshim", "ggdmc_gpu_shim.c")
    # (DL_FUNC) casts in the registration table are R's idiom: -Wno-cast-function-type
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-Wno-cast-function-type", "-fsyntax-only",
           "-I", os.path.join(root, "tests", "rshim_stub"), "-I", os.path.join(root, "include"), shim]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
