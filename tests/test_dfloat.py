"""Accuracy of two host/device headers, compiled here for the host:
the double-float FP32 arithmetic (ggdmc_gb300/csrc/dfloat.h) that forms the
per-proposal constants of the FP32 trial density -- Phi(v/s), its
complement, the quotients s / (A Phi) and Phi(-k) / Phi(k) and log g -- and
the F quantile (ggdmc_gb300/csrc/fquantile.h) of the PSRF upper bound.

The headers are compiled for the host (tests/dfloat_check/dfloat_check.cpp,
g++ without FP contraction, which keeps the error-free transformations
exact) and checked against 40-digit mpmath on the split inputs, over the
ranges the density uses: |v/s| <= 11 (Phi(v/s) >= 1e-28; a smaller value
sends the proposal to FP64), results above 1e-30.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")
mp.mp.dps = 40
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
P = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    so = str(tmp_path_factory.mktemp("dfc") / "dfc.so")
    cmd = ["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-I", os.path.join(ROOT, "ggdmc_gb300", "csrc"),
           os.path.join(ROOT, "tests", "dfloat_check", "dfloat_check.cpp"), "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return C.CDLL(so)


def call(lib, f, *args, nout=1):
    n = len(args[0])
    outs = [np.zeros(n) for _ in range(nout)]
    getattr(lib, f)(*[a.ctypes.data_as(P) for a in args], *[o.ctypes.data_as(P) for o in outs], C.c_int(n))
    return outs


def split(x):
    """x as the double-float code sees it (hi + lo of FP32 parts)."""
    h = x.astype(np.float32).astype(np.float64)
    return h + (x - h).astype(np.float32).astype(np.float64)


def ref(f, *xs):
    return np.array([float(f(*[mp.mpf(float(v)) for v in t])) for t in zip(*xs)])


def rel(y, r):
    return np.max(np.abs(y - r) / np.abs(r))


rng = np.random.default_rng(7)


def test_phi_pair_1e10(lib):
    k = split(rng.uniform(-11, 11, 1500))
    k[:4] = [0.0, 1e-9, -1e-9, 11.0]
    pk, pnk = call(lib, "dfc_phi_pair", k, nout=2)
    assert rel(pk, ref(mp.ncdf, k)) < 2e-10
    assert rel(pnk, ref(lambda v: mp.ncdf(-v), k)) < 2e-10


def test_exp_log(lib):
    x = split(-rng.uniform(0, 68, 1000))               # results above 3e-30
    assert rel(call(lib, "dfc_exp", x)[0], ref(mp.exp, x)) < 1e-12
    x = split(np.exp(rng.uniform(-60, 60, 1000)))
    x[:3] = [1.0, 1.0 + 2.0 ** -22, 1.4142135]
    y = call(lib, "dfc_log", x)[0]
    assert np.max(np.abs(y - ref(mp.log, x))) < 5e-11   # log g enters sums as an absolute term


def test_products_and_quotients(lib):
    a = split(rng.uniform(-10, 10, 1000))
    b = split(np.exp(rng.uniform(-8, 8, 1000)))
    assert rel(call(lib, "dfc_div", a, b)[0], ref(lambda u, v: u / v, a, b)) < 5e-14
    assert rel(call(lib, "dfc_mul", a, b)[0], ref(lambda u, v: u * v, a, b)) < 5e-14
    c = split(-a * (1 + 2.0 ** -30))
    s = call(lib, "dfc_add", a, c)[0]
    assert rel(s, ref(lambda u, v: u + v, a, c)) < 1e-6        # cancellation keeps the low parts


def test_f_quantile_against_scipy(lib):
    """fquantile.h's qf (the PSRF upper bound's F quantile) against scipy,
    second degrees of freedom from 0.5 to 1e9 (the range scipy resolves to
    1e-11)."""
    fdist = pytest.importorskip("scipy.stats").f
    lib.fqc_quantile.argtypes = [P, P, P, P, C.c_int]
    n = 1200
    p = rng.choice([0.975, 0.95, 0.5, 0.025, 0.999], n)
    d1 = np.exp(rng.uniform(0.0, np.log(500.0), n))
    d2 = np.exp(rng.uniform(np.log(0.5), np.log(1e9), n))
    d1[:4], d2[:4] = [1.0, 2.0, 50.0, 1.0], [1.0, 3.0, 5e4, 1e9]
    y = np.zeros(n)
    lib.fqc_quantile(p.ctypes.data_as(P), d1.ctypes.data_as(P), d2.ctypes.data_as(P), y.ctypes.data_as(P), n)
    np.testing.assert_allclose(y, fdist.ppf(p, d1, d2), rtol=5e-11)


def test_f_cdf_large_second_df(lib):
    """For d2 up to 1e12 (scipy loses digits there) the quantile is checked
    by its 40-digit CDF: I_x(d1/2, d2/2) at the returned F equals p."""
    lib.fqc_quantile.argtypes = [P, P, P, P, C.c_int]
    p = np.array([0.975, 0.95, 0.999, 0.5])
    d1 = np.array([1.2, 36.0, 4.0, 100.0])
    d2 = np.array([2e11, 6e11, 1e12, 3e10])
    y = np.zeros(4)
    lib.fqc_quantile(p.ctypes.data_as(P), d1.ctypes.data_as(P), d2.ctypes.data_as(P), y.ctypes.data_as(P), 4)
    for pi, a, b, f in zip(p, d1, d2, y):
        u = mp.mpf(float(a)) * mp.mpf(float(f))
        cdf = mp.betainc(mp.mpf(float(a)) / 2, mp.mpf(float(b)) / 2, 0, u / (u + mp.mpf(float(b))), regularized=True)
        assert abs(float(cdf) - pi) < 1e-12
