"""GPU parity of the diffusion model (Navarro-Fuss with sz / sv / st0
variability) against the CPU oracle, through the C ABI.

Tolerances:
* FP64: per-subject sums and per-trial log densities within 1e-12 relative
  of the oracle; chain states after a run bit-identical.
* MIXED: per trial within 5e-5 absolute (median 1e-6); per-subject sums
  within 1e-6 of sum_i |log d_i|.
"""
import numpy as np
import pytest

from ggdmc_gb300 import abi, gpu, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from ggdmc_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def work():
    # coarser Euler step than the 1e-4 s of the full config: parity does not
    # depend on how the RTs were made
    return synth.hier_ddm_64(n_subject=10, n=160, dt=1e-3)


def near_truth(w, n, seed, spread=0.05):
    rng = np.random.default_rng(seed)
    th = w.theta_true[:, None, :] * (1 + spread * rng.standard_normal(
        (w.theta_true.shape[0], n, w.theta_true.shape[1])))
    signed = np.array([nm.startswith("v.") for nm in w.model.pnames])
    return np.where(signed, th, np.abs(th))


def test_ddm_fp64_matches_oracle(oracle, work):
    w = work
    theta = near_truth(w, 3, 1)
    h = gpu.Handle(w.model, w.batch)
    got = h.loglik(theta, abi.FP64)
    want = oracle.loglik(w.model, w.batch, theta)
    np.testing.assert_allclose(got, want, rtol=1e-12)
    per = h.trial_logdens(theta[:, 0, :], abi.FP64)
    want_t = np.concatenate([oracle.sumloglike(w.model, w.batch.subject(s).rt, w.batch.subject(s).cell,
                                               theta[s, 0], per_trial=True)[1]
                             for s in range(w.batch.n_subject)])
    np.testing.assert_allclose(per, want_t, rtol=1e-12, atol=1e-13)


def test_ddm_mixed_close_to_oracle(oracle, work):
    w = work
    theta = near_truth(w, 2, 2)
    h = gpu.Handle(w.model, w.batch)
    per = h.trial_logdens(theta[:, 0, :], abi.MIXED)
    want_t = np.concatenate([oracle.sumloglike(w.model, w.batch.subject(s).rt, w.batch.subject(s).cell,
                                               theta[s, 0], per_trial=True)[1]
                             for s in range(w.batch.n_subject)])
    err = np.abs(per - want_t)
    assert err.max() <= 5e-5, err.max()
    assert np.median(err) <= 1e-6, np.median(err)
    mixed = h.loglik(theta, abi.MIXED)
    want = oracle.loglik(w.model, w.batch, theta)
    scale = np.zeros_like(want)
    for s in range(w.batch.n_subject):
        sd = w.batch.subject(s)
        for j in range(theta.shape[1]):
            scale[s, j] = np.abs(oracle.sumloglike(w.model, sd.rt, sd.cell, theta[s, j],
                                                   per_trial=True)[1]).sum()
    assert np.all(np.abs(mixed - want) / scale <= 1e-6)


def test_ddm_run_subjects_fp64_bit_exact(oracle, work):
    w = work
    S, C, P = 3, 27, w.model.n_par
    from ggdmc_gb300.dmi import SubjectBatch
    batch = SubjectBatch(w.batch.rt[: w.batch.offsets[S]], w.batch.cell[: w.batch.offsets[S]],
                         w.batch.offsets[: S + 1])
    th = near_truth(w, C, 3)[:S]
    lp = np.stack([oracle.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = oracle.loglik(w.model, batch, th)
    cfg = abi.DEConfigPy(nchain=C, nparameter=P, nmc=4, thin=1, sub_migration_prob=0.2, seed=31)
    g = gpu.run_subjects(cfg, w.model, batch, w.p_prior, th, lp, ll)
    o = oracle.run_subjects(cfg, w.model, batch, w.p_prior, th, lp, ll)
    assert np.array_equal(g["theta"], o["theta"])
    np.testing.assert_allclose(g["ll"], o["ll"], rtol=1e-12)
    assert g["stats"]["accepts"] == o["stats"].accepts > 0


def test_ddm_hierarchical_fp64_bit_exact(oracle, work):
    w = work
    C, P = 27, w.model.n_par
    rng = np.random.default_rng(7)
    th, phi = synth.start_states(w, C, rng)
    S = w.batch.n_subject
    lp = np.stack([oracle.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = oracle.loglik(w.model, w.batch, th)
    plp = oracle.logprior(w.h_prior, phi)
    pll = oracle.loghlike(w.p_prior, phi, th)
    cfg = abi.DEConfigPy(nchain=C, nparameter=2 * P, nmc=3, thin=1, pop_migration_prob=0.1,
                         sub_migration_prob=0.1, seed=5)
    g = gpu.run(cfg, w.model, w.batch, w.p_prior, w.h_prior, (phi, plp, pll), (th, lp, ll))
    o = oracle.run(cfg, w.model, w.batch, w.p_prior, w.h_prior, (phi, plp, pll), (th, lp, ll))
    assert np.array_equal(g["phi"][0], o["phi"][0])
    assert np.array_equal(g["subj"][0], o["subj"][0])
    np.testing.assert_allclose(g["subj"][2], o["subj"][2], rtol=1e-12)


def test_ddm_mixed_same_decisions_under_both_schedules(monkeypatch, work):
    # the ordered resolve (512-thread blocks) and the fused schedule take the
    # same decisions on the diffusion model; its per-trial FP32 values may
    # round differently in the two kernels (the compiler contracts its
    # products and sums per kernel), so the sums agree to ~1e-6
    w = work
    S, C, P = w.batch.n_subject, 27, w.model.n_par
    h = gpu.Handle(w.model, w.batch)
    th = near_truth(w, C, 5)
    lp = np.stack([gpu.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = h.loglik(th, abi.MIXED_SUMS)
    cfg = abi.DEConfigPy(nchain=C, nparameter=P, nmc=6, thin=1, sub_migration_prob=0.2, seed=13,
                         precision=abi.MIXED)
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("GGDMC_FUSED", mode)
        out[mode] = h.run(cfg, w.p_prior, th, lp, ll)
    a, b = out["0"], out["1"]
    np.testing.assert_array_equal(a["theta"], b["theta"])
    np.testing.assert_array_equal(a["s_theta"], b["s_theta"])
    np.testing.assert_allclose(a["ll"], b["ll"], rtol=0, atol=1e-5)
    assert a["stats"]["accepts"] == b["stats"]["accepts"] > 0
