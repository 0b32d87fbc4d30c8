"""ctypes binding of libggdmc_gpu.so (the C ABI of include/ggdmc_gpu.h).

There is no CPU fallback: if the library is missing, or no GPU is present,
every call raises.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi
from .build import LIB

_lib = None


class GGDMCError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def lib():
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise RuntimeError(f"{LIB} is missing: build it with ggdmc_gb300.build.build()")
    L = C.CDLL(LIB)
    P = C.POINTER
    St = C.c_int
    L.ggdmc_last_error.restype = C.c_char_p
    L.ggdmc_version.restype = C.c_char_p
    L.ggdmc_draw_layout.restype = St
    L.ggdmc_draw_layout.argtypes = [P(abi.DEConfig), C.c_int32, C.c_int32, P(C.c_int64),
                                    P(C.c_int64), P(C.c_int64), P(C.c_int64)]
    L.ggdmc_create.restype = St
    L.ggdmc_create.argtypes = [P(abi.Model), P(abi.Data), P(C.c_void_p)]
    L.ggdmc_destroy.restype = St
    L.ggdmc_destroy.argtypes = [C.c_void_p]
    L.ggdmc_loglik.restype = St
    L.ggdmc_loglik.argtypes = [C.c_void_p, P(C.c_double), C.c_int32, C.c_int32, P(C.c_double)]
    L.ggdmc_loglik_device.restype = St
    L.ggdmc_loglik_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p,
                                      C.c_void_p]
    L.ggdmc_trial_logdens.restype = St
    L.ggdmc_trial_logdens.argtypes = [C.c_void_p, P(C.c_double), C.c_int32, P(C.c_double)]
    L.ggdmc_logprior.restype = St
    L.ggdmc_logprior.argtypes = [P(abi.Prior), P(C.c_double), C.c_int32, P(C.c_double)]
    L.ggdmc_logprior_noalloc.restype = St
    L.ggdmc_logprior_noalloc.argtypes = [P(abi.Prior), P(C.c_double), C.c_int32, P(C.c_double)]
    L.ggdmc_initialise.restype = St
    L.ggdmc_initialise.argtypes = [C.c_void_p, P(abi.Prior), P(abi.Prior), C.c_int32, C.c_int32,
                                   C.c_uint64, C.c_int32, P(abi.ChainState), P(abi.ChainState)]
    L.ggdmc_handle_summary.restype = St
    L.ggdmc_handle_summary.argtypes = [C.c_void_p, C.c_int32] + [P(C.c_double)] * 6
    L.ggdmc_handle_diagnostics.restype = St
    L.ggdmc_handle_diagnostics.argtypes = [C.c_void_p, C.c_int32, C.c_int32, P(C.c_double), C.c_int32,
                                           C.c_double, C.c_int32, P(abi.Diag), P(abi.Diag)]
    L.ggdmc_loghlike.restype = St
    L.ggdmc_loghlike.argtypes = [P(abi.Prior), P(C.c_double), P(C.c_double), C.c_int32,
                                 C.c_int32, P(C.c_double)]
    run_args = [P(abi.DEConfig), P(abi.Model), P(abi.Data), P(abi.Prior), P(abi.ChainState),
                P(C.c_double), P(abi.Samples), P(abi.RunStats)]
    L.ggdmc_run_subject.restype = St
    L.ggdmc_run_subject.argtypes = run_args
    L.ggdmc_run_subjects.restype = St
    L.ggdmc_run_subjects.argtypes = run_args
    L.ggdmc_run_hyper.restype = St
    L.ggdmc_run_hyper.argtypes = [P(abi.DEConfig), P(C.c_double), C.c_int32, P(abi.Prior),
                                  P(abi.Prior), P(abi.ChainState), P(C.c_double), P(abi.Samples),
                                  P(abi.RunStats)]
    L.ggdmc_run.restype = St
    L.ggdmc_run.argtypes = [P(abi.DEConfig), P(abi.Model), P(abi.Data), P(abi.Prior),
                            P(abi.Prior), P(abi.ChainState), P(abi.ChainState), P(C.c_double),
                            P(abi.Samples), P(abi.Samples), P(abi.RunStats)]
    L.ggdmc_handle_run.restype = St
    L.ggdmc_handle_run.argtypes = [C.c_void_p, P(abi.DEConfig), P(abi.Prior), P(abi.Prior),
                                   P(abi.ChainState), P(abi.ChainState), P(C.c_double),
                                   P(abi.Samples), P(abi.Samples), P(abi.RunStats)]
    L.ggdmc_rebuild_posterior.restype = St
    L.ggdmc_rebuild_posterior.argtypes = [P(abi.Samples), C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                          P(abi.Samples)]
    L.ggdmc_tune_key.restype = St
    L.ggdmc_tune_key.argtypes = [P(abi.Model), P(abi.Data), C.c_int32, C.c_int32, C.c_char_p, C.c_int32]
    L.ggdmc_tune_lookup.restype = St
    L.ggdmc_tune_lookup.argtypes = [C.c_char_p, C.c_char_p, P(abi.Tuning)]
    L.ggdmc_tune_store.restype = St
    L.ggdmc_tune_store.argtypes = [C.c_char_p, C.c_char_p, P(abi.Tuning)]
    L.ggdmc_handle_set_tuning.restype = St
    L.ggdmc_handle_set_tuning.argtypes = [C.c_void_p, P(abi.Tuning)]
    L.ggdmc_autotune.restype = St
    L.ggdmc_autotune.argtypes = [C.c_void_p, P(abi.DEConfig), P(abi.Prior), P(abi.Prior), P(abi.ChainState),
                                 P(abi.ChainState), C.c_int32, C.c_char_p, P(abi.Tuning)]
    L.ggdmc_probe_peaks.restype = St
    L.ggdmc_probe_peaks.argtypes = [P(C.c_double), P(C.c_double)]
    _lib = L
    return L


def check(status: int):
    if status != 0:
        raise GGDMCError(status, lib().ggdmc_last_error().decode(errors="replace"))


def probe_peaks():
    """(FP32 TFLOP/s, MUFU tera-ops/s) measured on this GPU."""
    a, b = C.c_double(), C.c_double()
    check(lib().ggdmc_probe_peaks(C.byref(a), C.byref(b)))
    return a.value, b.value


def version() -> str:
    return lib().ggdmc_version().decode()


def _draw_ptr(m, draws):
    if draws is None:
        return None
    d = m.keep(np.ascontiguousarray(draws, np.float64))
    return abi.dptr(d)


def stats_dict(st: abi.RunStats) -> dict:
    return {k: (float(getattr(st, k)) if k.endswith("_ms") else int(getattr(st, k)))
            for k, _ in abi.RunStats._fields_}


class Handle:
    """Design + trials resident on the GPU (ggdmc_create / ggdmc_destroy)."""

    def __init__(self, model, batch):
        self._m = abi.Marshal()
        self.model = model
        self.batch = batch
        cm, cd = self._m.model(model), self._m.data(batch)
        h = C.c_void_p()
        check(lib().ggdmc_create(C.byref(cm), C.byref(cd), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().ggdmc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def loglik(self, theta, precision=abi.FP64):
        """theta [S][n][P] -> per-subject log-likelihood sums [S][n]."""
        th = np.ascontiguousarray(theta, np.float64)
        out = np.zeros(th.shape[:2])
        check(lib().ggdmc_loglik(self.h, abi.dptr(th), th.shape[1], precision, abi.dptr(out)))
        return out

    def loglik_device(self, d_theta_ptr: int, n_theta: int, d_out_ptr: int, precision=abi.MIXED,
                      stream: int = 0):
        check(lib().ggdmc_loglik_device(self.h, C.c_void_p(d_theta_ptr), n_theta, precision,
                                        C.c_void_p(d_out_ptr), C.c_void_p(stream)))

    def initialise(self, p_table, h_table=None, nchain=3, max_attempts=200, seed=0,
                   precision=abi.FP64):
        """Start states drawn from the priors (initialise_theta / _phi):
        ((theta [S][C][P], lp, ll), phi (theta [C][2P], lp, ll) or None)."""
        m = abi.Marshal()
        cp = m.prior(p_table)
        ch = m.prior(h_table) if h_table is not None else None
        S, P = self.batch.n_subject, self.model.n_par
        st, th, lp, ll = m.states(np.zeros((S, nchain, P)), np.zeros((S, nchain)), np.zeros((S, nchain)))
        pst = None
        if h_table is not None:
            pst, pth, plp, pll = m.states(np.zeros((1, nchain, 2 * P)), np.zeros((1, nchain)),
                                          np.zeros((1, nchain)))
        check(lib().ggdmc_initialise(self.h, C.byref(cp), C.byref(ch) if ch is not None else None,
                                     nchain, max_attempts, C.c_uint64(seed), precision, st, pst))
        return (th, lp, ll), ((pth[0], plp[0], pll[0]) if h_table is not None else None)

    def summary(self, start=0, phi=False):
        """Posterior mean, sd and PSRF (coda's form) of the last run's samples,
        computed on the device: {"subj": (mean, sd, psrf) [S][P], "phi": ... [2P]}."""
        S, P = self.batch.n_subject, self.model.n_par
        m, s, r = (np.zeros((S, P)) for _ in range(3))
        pm, ps, pr = (np.zeros(2 * P) for _ in range(3))
        ptr = lambda a: abi.dptr(a) if phi else None
        check(lib().ggdmc_handle_summary(self.h, start, abi.dptr(m), abi.dptr(s), abi.dptr(r),
                                         ptr(pm), ptr(ps), ptr(pr)))
        out = {"subj": (m, s, r)}
        if phi:
            out["phi"] = (pm, ps, pr)
        return out

    def diagnostics(self, start=0, end=0, probs=(0.05, 0.5, 0.975), conf=0.95, form=abi.PSRF_REFERENCE,
                    phi=False):
        """summary + gelman of the last run's samples, on the device
        (ggdmc_handle_diagnostics): {"subj": {...} [S][P], "phi": {...} [2P]}
        with mean, sd, naive_se, ts_se, quantiles [..][n_prob], psrf [..][2]."""
        pr = np.ascontiguousarray(probs, np.float64)
        levels = [("subj", self.batch.n_subject, self.model.n_par)]
        if phi:
            levels.append(("phi", 1, 2 * self.model.n_par))
        outs, structs = {}, []
        for name, L, P in levels:
            o = {k: np.full((L, P), np.nan) for k in ("mean", "sd", "naive_se", "ts_se")}
            o["quantiles"] = np.full((L, P, len(pr)), np.nan)
            o["psrf"] = np.full((L, P, 2), np.nan)
            outs[name] = o
            structs.append(abi.Diag(*[abi.dptr(o[k]) for k in ("mean", "sd", "naive_se", "ts_se", "quantiles",
                                                                "psrf")]))
        ph = C.byref(structs[1]) if phi else None
        check(lib().ggdmc_handle_diagnostics(self.h, start, end, abi.dptr(pr) if len(pr) else None, len(pr),
                                             conf, form, C.byref(structs[0]), ph))
        if phi:
            outs["phi"] = {k: v[0] for k, v in outs["phi"].items()}
        return outs

    def set_tuning(self, tuning=None):
        """Launch settings for this handle's runs (dict of ggdmc_tuning fields,
        0 = built-in choice; None clears them)."""
        t = abi.Tuning(**(tuning or {})) if tuning is not None else None
        check(lib().ggdmc_handle_set_tuning(self.h, C.byref(t) if t is not None else None))

    def autotune(self, cfg, p_table, theta, lp, ll, h_table=None, phi=None, n_probe=5, cache_path=None):
        """ggdmc_autotune: the cached or freshly timed settings for runs like
        cfg from these start states (not changed); the handle keeps them."""
        m = abi.Marshal()
        cc, cp = cfg.to_c(), m.prior(p_table)
        ch = m.prior(h_table) if h_table is not None else None
        st, *_ = m.states(theta, lp, ll)
        pst = m.states(phi[0][None], phi[1][None], phi[2][None])[0] if phi is not None else None
        out = abi.Tuning()
        check(lib().ggdmc_autotune(self.h, C.byref(cc), C.byref(cp), C.byref(ch) if ch is not None else None,
                                   pst, st, n_probe, cache_path.encode() if cache_path else None, C.byref(out)))
        return out.as_dict()

    def trial_logdens(self, theta, precision=abi.FP64):
        """theta [S][P] -> per-trial log densities [N]."""
        th = np.ascontiguousarray(theta, np.float64)
        out = np.zeros(max(len(self.batch.rt), 1))
        check(lib().ggdmc_trial_logdens(self.h, abi.dptr(th), precision, abi.dptr(out)))
        return out[:len(self.batch.rt)]

    def run(self, cfg: abi.DEConfigPy, p_table, theta, lp, ll, draws=None, h_table=None,
            phi=None):
        """Subject fits (phi None) or a hierarchical run on the resident data."""
        m = abi.Marshal()
        cc, cp = cfg.to_c(), m.prior(p_table)
        ch = m.prior(h_table) if h_table is not None else None
        st, th, lpa, lla = m.states(theta, lp, ll)
        S = self.batch.n_subject
        so, sth, slp, sll = m.samples(S, cfg.nmc, cfg.nchain, self.model.n_par)
        pst = pso = None
        if phi is not None:
            pst, pth, plp, pll = m.states(phi[0][None], phi[1][None], phi[2][None])
            pso, psth, pslp, psll = m.samples(1, cfg.nmc, cfg.nchain, h_table.shape[0])
        stats = abi.RunStats()
        check(lib().ggdmc_handle_run(self.h, C.byref(cc), C.byref(cp),
                                     C.byref(ch) if ch is not None else None, pst, st,
                                     _draw_ptr(m, draws), pso, so, C.byref(stats)))
        out = dict(theta=th, lp=lpa, ll=lla, s_theta=sth, s_lp=slp, s_ll=sll,
                   stats=stats_dict(stats))
        if phi is not None:
            out.update(phi=(pth[0], plp[0], pll[0]), phi_s=(psth[0], pslp[0], psll[0]))
        return out


def run_subjects(cfg, model, batch, p_table, theta, lp, ll, draws=None):
    """ggdmc_run_subject(s): independent subject fits through the one-shot C ABI."""
    m = abi.Marshal()
    cc, cm, cd, cp = cfg.to_c(), m.model(model), m.data(batch), m.prior(p_table)
    st, th, lpa, lla = m.states(theta, lp, ll)
    so, sth, slp, sll = m.samples(batch.n_subject, cfg.nmc, cfg.nchain, model.n_par)
    stats = abi.RunStats()
    fn = lib().ggdmc_run_subject if batch.n_subject == 1 else lib().ggdmc_run_subjects
    check(fn(C.byref(cc), C.byref(cm), C.byref(cd), C.byref(cp), st, _draw_ptr(m, draws), so,
             C.byref(stats)))
    return dict(theta=th, lp=lpa, ll=lla, s_theta=sth, s_lp=slp, s_ll=sll,
                stats=stats_dict(stats))


def run_hyper(cfg, hyper_rows, p_table, h_table, theta, lp, ll, draws=None):
    m = abi.Marshal()
    cc, cp, ch = cfg.to_c(), m.prior(p_table), m.prior(h_table)
    rows = m.keep(np.ascontiguousarray(hyper_rows, np.float64))
    st, th, lpa, lla = m.states(theta[None], lp[None], ll[None])
    so, sth, slp, sll = m.samples(1, cfg.nmc, cfg.nchain, h_table.shape[0])
    stats = abi.RunStats()
    check(lib().ggdmc_run_hyper(C.byref(cc), abi.dptr(rows), rows.shape[0], C.byref(cp),
                                C.byref(ch), st, _draw_ptr(m, draws), so, C.byref(stats)))
    return dict(theta=th[0], lp=lpa[0], ll=lla[0], s_theta=sth[0], s_lp=slp[0], s_ll=sll[0],
                stats=stats_dict(stats))


def run(cfg, model, batch, p_table, h_table, phi, subj, draws=None):
    """ggdmc_run: hierarchical DE-MCMC through the one-shot C ABI."""
    m = abi.Marshal()
    cc, cm, cd = cfg.to_c(), m.model(model), m.data(batch)
    cp, ch = m.prior(p_table), m.prior(h_table)
    pst, pth, plp, pll = m.states(phi[0][None], phi[1][None], phi[2][None])
    sst, sth, slp, sll = m.states(*subj)
    pso, psth, pslp, psll = m.samples(1, cfg.nmc, cfg.nchain, h_table.shape[0])
    sso, ssth, sslp, ssll = m.samples(batch.n_subject, cfg.nmc, cfg.nchain, model.n_par)
    stats = abi.RunStats()
    check(lib().ggdmc_run(C.byref(cc), C.byref(cm), C.byref(cd), C.byref(cp), C.byref(ch), pst,
                          sst, _draw_ptr(m, draws), pso, sso, C.byref(stats)))
    return dict(phi=(pth[0], plp[0], pll[0]), subj=(sth, slp, sll),
                phi_s=(psth[0], pslp[0], psll[0]), subj_s=(ssth, sslp, ssll),
                stats=stats_dict(stats))


def logprior(p_table, theta):
    m = abi.Marshal()
    p = m.prior(p_table)
    th = m.keep(np.ascontiguousarray(np.atleast_2d(theta), np.float64))
    out = np.zeros(th.shape[0])
    check(lib().ggdmc_logprior(C.byref(p), abi.dptr(th), th.shape[0], abi.dptr(out)))
    return out


def logprior_noalloc(p_table, theta):
    """logprior through the entry point that stages in a fixed device array."""
    m = abi.Marshal()
    p = m.prior(p_table)
    th = m.keep(np.ascontiguousarray(np.atleast_2d(theta), np.float64))
    out = np.zeros(th.shape[0])
    check(lib().ggdmc_logprior_noalloc(C.byref(p), abi.dptr(th), th.shape[0], abi.dptr(out)))
    return out


def loghlike(p_table, phi, subj_theta):
    m = abi.Marshal()
    p = m.prior(p_table)
    ph = m.keep(np.ascontiguousarray(phi, np.float64))
    st = m.keep(np.ascontiguousarray(subj_theta, np.float64))
    out = np.zeros(ph.shape[0])
    check(lib().ggdmc_loghlike(C.byref(p), abi.dptr(ph), abi.dptr(st), st.shape[0], ph.shape[0],
                               abi.dptr(out)))
    return out


def rebuild_posterior(fits):
    """RebuildPosterior / RebuildHyper (R/parallel_helper.R:62-109) through
    ggdmc_rebuild_posterior: fits is a list of (theta [nmc][C][P], lp [nmc][C],
    ll [nmc][C]) sample sets of one level (for example the levels of a
    run_subjects call on one subject's data replicated, or the phi samples of
    several hierarchical runs).  Returns (theta [nmc*C][F][P], lp, ll [nmc*C][F])
    in the reference's merged order.  Host code only: needs no GPU."""
    fits = [tuple(np.ascontiguousarray(a, np.float64) for a in f) for f in fits]
    nmc, nchain, npar = fits[0][0].shape
    for th, lp, ll in fits:
        if th.shape != (nmc, nchain, npar) or lp.shape != (nmc, nchain) or ll.shape != (nmc, nchain):
            raise ValueError("every fit needs theta [nmc][nchain][npar] and lp, ll [nmc][nchain] of one shape")
    F = len(fits)
    arr = (abi.Samples * F)(*[abi.Samples(abi.dptr(th), abi.dptr(lp), abi.dptr(ll)) for th, lp, ll in fits])
    th = np.zeros((nmc * nchain, F, npar))
    lp = np.zeros((nmc * nchain, F))
    ll = np.zeros((nmc * nchain, F))
    out = abi.Samples(abi.dptr(th), abi.dptr(lp), abi.dptr(ll))
    check(lib().ggdmc_rebuild_posterior(arr, F, nmc, nchain, npar, C.byref(out)))
    return th, lp, ll


def rebuild_posteriors(runs):
    """RebuildPosteriors (R/parallel_helper.R:162-208): the subject samples of
    several hierarchical runs (each a gpu.run result) merged per subject."""
    S = runs[0]["subj_s"][0].shape[0]
    return [rebuild_posterior([tuple(x[s] for x in r["subj_s"]) for r in runs]) for s in range(S)]


def tune_key(model, batch, nchain, hierarchical):
    """The autotuner's cache key of a design and data shape (ggdmc_tune_key); host only."""
    m = abi.Marshal()
    buf = C.create_string_buffer(512)
    check(lib().ggdmc_tune_key(C.byref(m.model(model)), C.byref(m.data(batch)), nchain, int(hierarchical), buf, 512))
    return buf.value.decode()


def tune_lookup(key, cache_path=None):
    """Cached settings of a key (process cache, then the file), or None."""
    out = abi.Tuning()
    st = lib().ggdmc_tune_lookup(key.encode(), cache_path.encode() if cache_path else None, C.byref(out))
    return out.as_dict() if st == 0 else None


def tune_store(key, tuning, cache_path=None):
    t = abi.Tuning(**tuning)
    check(lib().ggdmc_tune_store(key.encode(), cache_path.encode() if cache_path else None, C.byref(t)))
