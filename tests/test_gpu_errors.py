"""Failure handling on the GPU without a fault: a run whose device work
outlasts GGDMC_TIMEOUT_S returns GGDMC_ERR_TIMEOUT (the host stops waiting;
the device finishes its work), and the same handle then runs normally."""
import numpy as np
import pytest

from ggdmc_gb300 import abi, gpu, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from ggdmc_gb300 import build
    build.build()


def test_deadline_returns_timeout_and_handle_recovers(oracle, monkeypatch):
    w = synth.uneven_lba_256(n_subject=24)
    h = gpu.Handle(w.model, w.batch)
    rng = np.random.default_rng(2)
    th, phi = synth.start_states(w, w.nchain, rng)
    S = w.batch.n_subject
    lp = np.stack([gpu.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = h.loglik(th, abi.FP64)
    plp = gpu.logprior(w.h_prior, phi)
    pll = gpu.loghlike(w.p_prior, phi, th)
    cfg = abi.DEConfigPy(nchain=w.nchain, nparameter=2 * w.model.n_par, nmc=60, thin=1, seed=3)
    monkeypatch.setenv("GGDMC_TIMEOUT_S", "1e-7")
    with pytest.raises(gpu.GGDMCError, match="TIMEOUT"):
        h.run(cfg, w.p_prior, th, lp, ll, h_table=w.h_prior, phi=(phi, plp, pll))
    monkeypatch.delenv("GGDMC_TIMEOUT_S")
    short = abi.DEConfigPy(nchain=w.nchain, nparameter=2 * w.model.n_par, nmc=3, thin=1, seed=3,
                           precision=abi.FP64)
    out = h.run(short, w.p_prior, th, lp, ll, h_table=w.h_prior, phi=(phi, plp, pll))
    want = oracle.run(short, w.model, w.batch, w.p_prior, w.h_prior, (phi, plp, pll), (th, lp, ll))
    assert np.array_equal(out["theta"], want["subj"][0])
    assert np.array_equal(out["phi"][0], want["phi"][0])


def test_device_wait_gives_up_and_handle_recovers(oracle, monkeypatch):
    """The fused schedule's idle CTAs poll for work with a limit.  One fit of
    6000 trials among 300 fits of 20-40: the other CTAs finish their fits and
    wait while it is resolved; with the limit at 0 polls they give up at once,
    the kernel sets the run's status and returns (no GPU wait is left
    running), the host reports GGDMC_ERR_TIMEOUT, and the same handle then
    reproduces the oracle."""
    from ggdmc_gb300.dmi import SubjectBatch
    monkeypatch.setenv("GGDMC_FUSED", "1")
    w = synth.many_fits_1024(n_fit=300, n_lo=20, n_hi=40)
    long_fit = synth.simulate_subject(w.model, w.theta_true[0], 6000, np.random.default_rng(1), "long")
    subs = [long_fit] + [w.batch.subject(f) for f in range(1, 300)]
    batch = SubjectBatch.pack(subs)
    C = 27
    th, _ = synth.start_states(w, C, np.random.default_rng(6))
    lp = np.stack([oracle.logprior(w.p_prior, th[f]) for f in range(batch.n_subject)])
    ll = oracle.loglik(w.model, batch, th)
    h = gpu.Handle(w.model, batch)
    cfg = abi.DEConfigPy(nchain=C, nparameter=w.model.n_par, nmc=6, thin=1, sub_migration_prob=0.06,
                         seed=9, precision=abi.FP64)
    monkeypatch.setenv("GGDMC_SPEC_IDLE_LIMIT", "0")
    with pytest.raises(gpu.GGDMCError, match="device-side wait gave up") as e:
        h.run(cfg, w.p_prior, th, lp, ll)
    assert e.value.status == abi.GGDMC_ERR_TIMEOUT
    monkeypatch.delenv("GGDMC_SPEC_IDLE_LIMIT")
    out = h.run(cfg, w.p_prior, th, lp, ll)
    want = oracle.run_subjects(cfg, w.model, batch, w.p_prior, th, lp, ll)
    assert np.array_equal(out["theta"], want["theta"])
    assert np.array_equal(out["s_theta"], want["s_theta"])
