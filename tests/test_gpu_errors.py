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
