"""The FP32 LBA trial density of ggdmc_gb300/csrc/device_common.cuh compiled
for the host (the CUDA intrinsics it uses replaced by host arithmetic,
tests/density_check/host_shim.h) against the FP64 oracle, trial by trial:
which trials the FP32 form takes and how close it is, on the benchmark
design near its generating values, on the reference fixture's start
samples, and on trials far too fast for the winner (the floor taken by the
bound on the winner's bracket).  No GPU: the device's approximate divide and
exponentials become host libm forms, so the values are within the same
tolerances, not the same bits.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from ggdmc_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "ggdmc_gb300", "csrc")
CUDA_INC = "/usr/local/cuda/include"


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA_INC, "vector_types.h")):
        pytest.skip("g++ or the CUDA headers (vector types) not available")
    d = tmp_path_factory.mktemp("dc32")
    src = open(os.path.join(CSRC, "device_common.cuh")).read()
    src = src.replace("#include <cuda_runtime.h>", '#include "host_shim.h"')
    src = src.replace("__device__ __forceinline__", "static inline")
    (d / "device_common_host.h").write_text(src)
    shutil.copy(os.path.join(ROOT, "tests", "density_check", "host_shim.h"), d / "host_shim.h")
    so = str(d / "dc32.so")
    cmd = ["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC", "-I", str(d), "-I", CSRC,
           "-I", CUDA_INC, os.path.join(ROOT, "tests", "density_check", "density_check.cpp"), "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    L = C.CDLL(so)
    L.dc_trial.argtypes = [C.c_double, C.c_double, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.dc_ddm.argtypes = [C.c_double, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double)]
    return L


def fp32_trials(L, model, rt, cell, theta):
    """Per trial: code (0 FP32, 1 FP64 form, 2 proposal in FP64) and value."""
    ps = model.param_src

    def val(src):
        return theta[src] if src >= 0 else model.constants[-1 - src]

    codes, vals = np.zeros(len(rt), int), np.full(len(rt), np.nan)
    out = C.c_double()
    for i in range(len(rt)):
        c = int(cell[i])
        win = int(model.resp[c])
        order = [win] + [k for k in range(model.n_acc) if k != win]
        abvs = np.array([[val(ps[c, k, q]) for q in range(4)] for k in order], np.float64).ravel()
        codes[i] = L.dc_trial(float(rt[i]), float(val(ps[c, win, 4])), model.n_acc,
                              abvs.ctypes.data_as(C.POINTER(C.c_double)), C.byref(out))
        if codes[i] == 0:
            vals[i] = out.value
    return codes, vals


def compare(L, oracle, model, batch, thetas, subjects):
    """Per-trial errors of the FP32 trials, the declined share, and each sum's
    error (the sum formed as the sampler forms it, declined trials in FP64)
    over the bound the FP32 form is built to: 1e-6 of the sum, or of
    1.2 sqrt(N) + 0.03 N for a sum nearer zero (the likelihood API refines
    those in FP64)."""
    errs, declined, n, rels = [], 0, 0, []
    for s in subjects:
        a, b = batch.offsets[s], batch.offsets[s + 1]
        for th in thetas[s]:
            codes, v = fp32_trials(L, model, batch.rt[a:b], batch.cell[a:b], th)
            _, want = oracle.sumloglike(model, batch.rt[a:b], batch.cell[a:b], th, per_trial=True)
            ok = codes == 0
            errs.append(v[ok] - want[ok])
            declined += int((~ok).sum())
            n += len(codes)
            tot = np.where(ok, v, want).sum()
            N = len(codes)
            rels.append(abs(tot - want.sum()) / max(abs(want.sum()), 1.2 * np.sqrt(N) + 0.03 * N))
    return np.concatenate(errs), declined / n, np.array(rels)


def near_truth(w, n, rng, spread):
    th = w.theta_true[:, None, :] * (1 + spread * rng.standard_normal((w.theta_true.shape[0], n,
                                                                       w.theta_true.shape[1])))
    return np.abs(th)


@pytest.mark.parametrize("spread,max_declined", [(0.05, 0.01), (0.2, 0.08)])
def test_benchmark_design_near_truth(lib, oracle, spread, max_declined):
    # at a 20% spread a few parameter vectors (drift rates over 40 standard
    # deviations) leave a third of their trials to the FP64 form
    w = synth.uneven_lba_256(n_subject=6, n_lo=100, n_hi=400)
    th = near_truth(w, 3, np.random.default_rng(4), spread)
    err, dec, rel = compare(lib, oracle, w.model, w.batch, th, range(6))
    assert dec < max_declined
    assert np.abs(err).max() <= 2e-5 and np.median(np.abs(err)) <= 2e-7 and abs(err.mean()) <= 2e-8
    assert rel.max() <= 1e-6


def test_fixture_start_samples(lib, oracle):
    """lba_data6's own start samples (prior draws far from the data, t0 above
    most responses): most trials at the floor, few left to FP64."""
    from bench import FX6
    w = synth.fixture_lba_768(FX6, hierarchical=True)
    th = w.start_theta[:, ::8]
    err, dec, rel = compare(lib, oracle, w.model, w.batch, th, range(3))
    assert dec < 0.02
    assert np.abs(err).max() <= 2e-5 and rel.max() <= 1e-6


def test_responses_far_too_fast_take_the_floor(lib, oracle):
    """t0 at the 60% quantile of the responses: the trials before it take the
    reference's floor, and those just after it (both of the winner's z beyond
    13) the floor by the bound on its bracket, in FP32, matching the oracle."""
    from ggdmc_gb300.design import T0_17_P, design_t0_17, vector
    model = design_t0_17()
    th = vector(model, T0_17_P)
    sub = synth.simulate_subject(model, th, 1500, np.random.default_rng(21), "1")
    late = th.copy()
    for j, nm in enumerate(model.pnames):
        if nm.startswith("t0"):
            late[j] = np.quantile(sub.rt, 0.6)
    codes, v = fp32_trials(lib, model, sub.rt, sub.cell, late)
    _, want = oracle.sumloglike(model, sub.rt, sub.cell, late, per_trial=True)
    q = np.quantile(sub.rt, 0.6)
    fast = (sub.rt > q + 1e-3) & (sub.rt < q + 0.05)
    assert fast.sum() > 20 and np.mean(codes[fast] == 0) >= 0.95
    assert np.all(np.abs(v[codes == 0] - want[codes == 0]) <= 2e-5)
    assert (codes != 0).mean() < 0.01


def test_diffusion_fp32_density(lib, oracle):
    """The diffusion model's FP32 density (Navarro-Fuss series, the sz / st0
    midpoint rule) against the oracle's FP64 one on its benchmark design near
    the generating values: per trial within 5e-5 (median 1e-6), few trials
    left to FP64."""
    w = synth.hier_ddm_64(n_subject=3, n=200, dt=1e-3)
    m = w.model
    rng = np.random.default_rng(6)
    out = C.c_double()
    errs, declined, n = [], 0, 0
    for s in range(3):
        a, b = w.batch.offsets[s], w.batch.offsets[s + 1]
        for _ in range(2):
            th = w.theta_true[s] * (1 + 0.05 * rng.standard_normal(m.n_par))
            signed = np.array([nm.startswith("v.") for nm in m.pnames])
            th = np.where(signed, th, np.abs(th))

            def val(src):
                return th[src] if src >= 0 else m.constants[-1 - src]

            for i in range(a, b):
                c = int(w.batch.cell[i])
                wb = int(m.resp[c])
                cv = np.array([[val(m.param_src[c, k, q]) for q in range(8)] for k in range(2)], np.float64)
                v8 = np.ascontiguousarray(cv[wb])
                code = lib.dc_ddm(float(w.batch.rt[i]), v8.ctypes.data_as(C.POINTER(C.c_double)), wb,
                                  C.byref(out))
                n += 1
                if code:
                    declined += 1
                    continue
                errs.append(out.value - np.log(oracle.ddm_dens(float(w.batch.rt[i]), cv, wb)))
    err = np.abs(np.array(errs))
    assert declined / n < 0.02
    assert err.max() <= 5e-5 and np.median(err) <= 1e-6
