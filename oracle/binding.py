"""ctypes binding of the CPU oracle (oracle/libggdmc_oracle.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker of the CUDA library.  The product
package (ggdmc_gb300/) never imports this module.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from ggdmc_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libggdmc_oracle.so")            # parity build
FAST_PATH = os.path.join(HERE, "libggdmc_oracle_fast.so")      # timed CPU baseline

_libs = {}
_use_fast = False


def build(force: bool = False) -> str:
    """Compile both oracle builds with the Makefile (gcc, a few seconds)."""
    src = os.path.getmtime(os.path.join(HERE, "ggdmc_oracle.c"))
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < src for p in (LIB_PATH, FAST_PATH)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def use_build(fast: bool) -> None:
    """Route the functions below to the -O3 build (the timed CPU baseline)
    or back to the parity build (the default; every parity check uses it)."""
    global _use_fast
    _use_fast = bool(fast)


def lib():
    path = FAST_PATH if _use_fast else LIB_PATH
    L = _libs.get(path)
    if L is None:
        build()
        L = C.CDLL(path)
        P = C.POINTER
        L.oracle_uniform.restype = C.c_double
        L.oracle_uniform.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_int64, C.c_int64]
        L.oracle_sumloglike.restype = C.c_double
        L.oracle_sumloglike.argtypes = [P(abi.Model), P(C.c_double), P(C.c_int32), C.c_int64,
                                        P(C.c_double), P(C.c_double)]
        L.oracle_loglik.argtypes = [P(abi.Model), P(abi.Data), P(C.c_double), C.c_int32,
                                    P(C.c_double)]
        L.oracle_logprior.argtypes = [P(abi.Prior), P(C.c_double), C.c_int32, P(C.c_double)]
        L.oracle_loghlike.argtypes = [P(abi.Prior), P(C.c_double), P(C.c_double), C.c_int32,
                                      C.c_int32, P(C.c_double)]
        L.oracle_tnorm_logpdf.restype = C.c_double
        L.oracle_tnorm_logpdf.argtypes = [C.c_double] * 5
        L.oracle_lba_dens.restype = C.c_double
        L.oracle_lba_dens.argtypes = [C.c_double, P(C.c_double), C.c_int, C.c_int]
        L.oracle_initialise.restype = C.c_int
        L.oracle_initialise.argtypes = [P(abi.Model), P(abi.Data), P(abi.Prior), P(abi.Prior), C.c_int32,
                                        C.c_int32, C.c_uint64, P(abi.ChainState), P(abi.ChainState)]
        L.oracle_ddm_dens.restype = C.c_double
        L.oracle_ddm_dens.argtypes = [C.c_double, P(C.c_double), C.c_int]
        L.oracle_run_subject.argtypes = [P(abi.DEConfig), P(abi.Model), P(abi.Data),
                                         P(abi.Prior), P(abi.ChainState), P(C.c_double),
                                         P(abi.Samples), P(abi.RunStats)]
        L.oracle_run_subjects.argtypes = L.oracle_run_subject.argtypes
        L.oracle_run_hyper.argtypes = [P(abi.DEConfig), P(C.c_double), C.c_int32, P(abi.Prior),
                                       P(abi.Prior), P(abi.ChainState), P(C.c_double),
                                       P(abi.Samples), P(abi.RunStats)]
        L.oracle_run.argtypes = [P(abi.DEConfig), P(abi.Model), P(abi.Data), P(abi.Prior),
                                 P(abi.Prior), P(abi.ChainState), P(abi.ChainState),
                                 P(C.c_double), P(abi.Samples), P(abi.Samples),
                                 P(abi.RunStats)]
        _libs[path] = L
    return L


def uniform(seed, it, level, pass_, slot) -> float:
    return lib().oracle_uniform(seed, it, level, pass_, slot)


def sumloglike(model, rt, cell, theta, per_trial=False):
    m = abi.Marshal()
    cm = m.model(model)
    rt = m.keep(np.ascontiguousarray(rt, np.float64))
    cell = m.keep(np.ascontiguousarray(cell, np.int32))
    th = m.keep(np.ascontiguousarray(theta, np.float64))
    pt = m.keep(np.zeros(max(len(rt), 1))) if per_trial else None
    s = lib().oracle_sumloglike(C.byref(cm), abi.dptr(rt), abi.i32ptr(cell), len(rt),
                                abi.dptr(th), abi.dptr(pt) if per_trial else None)
    return (s, pt[:len(rt)].copy()) if per_trial else s


def initialise(model, batch, p_table, h_table, nchain, max_attempts, seed):
    """Start states by rejection from the priors (initialise_theta /
    initialise_phi): ((theta [S][C][P], lp, ll), phi (theta, lp, ll) or None)."""
    m = abi.Marshal()
    cm, cd, cp = m.model(model), m.data(batch), m.prior(p_table)
    ch = m.prior(h_table) if h_table is not None else None
    S, P = batch.n_subject, model.n_par
    st, th, lp, ll = m.states(np.zeros((S, nchain, P)), np.zeros((S, nchain)), np.zeros((S, nchain)))
    pst = None
    if h_table is not None:
        pst, pth, plp, pll = m.states(np.zeros((1, nchain, h_table.shape[0])), np.zeros((1, nchain)),
                                      np.zeros((1, nchain)))
    L = lib()
    s = L.oracle_initialise(C.byref(cm), C.byref(cd), C.byref(cp), C.byref(ch) if ch is not None else None,
                            nchain, max_attempts, C.c_uint64(seed), st, pst)
    if s != 0:
        raise RuntimeError(f"oracle_initialise failed with status {s}")
    return (th, lp, ll), ((pth[0], plp[0], pll[0]) if h_table is not None else None)


def ddm_dens(rt, cv, w):
    """Diffusion density of one trial: cv [2][8] (a, v, z, d, sz, sv, t0,
    st0) per boundary, w = 0 lower, 1 upper (floored at 1e-10)."""
    cv = np.ascontiguousarray(cv, np.float64).reshape(-1)
    return lib().oracle_ddm_dens(float(rt), abi.dptr(cv), int(w))


def loglik(model, batch, theta):
    """theta [S][n][P] -> [S][n]."""
    m = abi.Marshal()
    cm, cd = m.model(model), m.data(batch)
    th = m.keep(np.ascontiguousarray(theta, np.float64))
    out = np.zeros(th.shape[:2])
    lib().oracle_loglik(C.byref(cm), C.byref(cd), abi.dptr(th), th.shape[1], abi.dptr(out))
    return out


def logprior(table, theta):
    m = abi.Marshal()
    p = m.prior(table)
    th = m.keep(np.ascontiguousarray(np.atleast_2d(theta), np.float64))
    out = np.zeros(th.shape[0])
    lib().oracle_logprior(C.byref(p), abi.dptr(th), th.shape[0], abi.dptr(out))
    return out


def loghlike(p_table, phi, subj_theta):
    """phi [n][2P]; subj_theta [S][n][P] -> [n]."""
    m = abi.Marshal()
    p = m.prior(p_table)
    ph = m.keep(np.ascontiguousarray(phi, np.float64))
    st = m.keep(np.ascontiguousarray(subj_theta, np.float64))
    out = np.zeros(ph.shape[0])
    lib().oracle_loghlike(C.byref(p), abi.dptr(ph), abi.dptr(st), st.shape[0], ph.shape[0],
                          abi.dptr(out))
    return out


def _draw_ptr(m, draws):
    if draws is None:
        return None
    d = m.keep(np.ascontiguousarray(draws, np.float64))
    return abi.dptr(d)


def run_subjects(cfg: abi.DEConfigPy, model, batch, p_table, theta, lp, ll, draws=None):
    """Independent subject-level fits (run_subject per subject).  theta [F][C][P]."""
    m = abi.Marshal()
    cc, cm, cd, cp = cfg.to_c(), m.model(model), m.data(batch), m.prior(p_table)
    st, th, lpa, lla = m.states(theta, lp, ll)
    so, sth, slp, sll = m.samples(batch.n_subject, cfg.nmc, cfg.nchain, model.n_par)
    stats = abi.RunStats()
    fn = lib().oracle_run_subject if batch.n_subject == 1 else lib().oracle_run_subjects
    rc = fn(C.byref(cc), C.byref(cm), C.byref(cd), C.byref(cp), st, _draw_ptr(m, draws), so,
            C.byref(stats))
    if rc != 0:
        raise RuntimeError(f"oracle run failed: {abi.STATUS_NAMES.get(rc, rc)}")
    return dict(theta=th, lp=lpa, ll=lla, s_theta=sth, s_lp=slp, s_ll=sll, stats=stats)


def run_hyper(cfg, hyper_rows, p_table, h_table, theta, lp, ll, draws=None):
    m = abi.Marshal()
    cc, cp, ch = cfg.to_c(), m.prior(p_table), m.prior(h_table)
    rows = m.keep(np.ascontiguousarray(hyper_rows, np.float64))
    st, th, lpa, lla = m.states(theta[None], lp[None], ll[None])
    so, sth, slp, sll = m.samples(1, cfg.nmc, cfg.nchain, h_table.shape[0])
    stats = abi.RunStats()
    rc = lib().oracle_run_hyper(C.byref(cc), abi.dptr(rows), rows.shape[0], C.byref(cp),
                                C.byref(ch), st, _draw_ptr(m, draws), so, C.byref(stats))
    if rc != 0:
        raise RuntimeError(f"oracle run_hyper failed: {abi.STATUS_NAMES.get(rc, rc)}")
    return dict(theta=th[0], lp=lpa[0], ll=lla[0], s_theta=sth[0], s_lp=slp[0], s_ll=sll[0],
                stats=stats)


def run(cfg, model, batch, p_table, h_table, phi, subj, draws=None):
    """Hierarchical run.  phi = (theta [C][2P], lp, ll); subj = (theta [S][C][P], lp, ll)."""
    m = abi.Marshal()
    cc, cm, cd = cfg.to_c(), m.model(model), m.data(batch)
    cp, ch = m.prior(p_table), m.prior(h_table)
    pst, pth, plp, pll = m.states(phi[0][None], phi[1][None], phi[2][None])
    sst, sth, slp, sll = m.states(*subj)
    pso, psth, pslp, psll = m.samples(1, cfg.nmc, cfg.nchain, h_table.shape[0])
    sso, ssth, sslp, ssll = m.samples(batch.n_subject, cfg.nmc, cfg.nchain, model.n_par)
    stats = abi.RunStats()
    rc = lib().oracle_run(C.byref(cc), C.byref(cm), C.byref(cd), C.byref(cp), C.byref(ch),
                          pst, sst, _draw_ptr(m, draws), pso, sso, C.byref(stats))
    if rc != 0:
        raise RuntimeError(f"oracle run failed: {abi.STATUS_NAMES.get(rc, rc)}")
    return dict(phi=(pth[0], plp[0], pll[0]), subj=(sth, slp, sll),
                phi_s=(psth[0], pslp[0], psll[0]), subj_s=(ssth, sslp, ssll), stats=stats)
