"""ggdmc_handle_summary: posterior mean, sd and PSRF computed on the device
from the samples a run left there, against ggdmc_gb300.diagnostics on the
same samples copied to the host."""
import numpy as np
import pytest

from ggdmc_gb300 import abi, diagnostics, gpu, synth

pytestmark = pytest.mark.gpu
pytest.importorskip("scipy")


@pytest.fixture(scope="module", autouse=True)
def built():
    from ggdmc_gb300 import build
    build.build()


def test_device_summary_matches_host():
    w = synth.hier_lba_32(n_subject=4, n=200)
    h = gpu.Handle(w.model, w.batch)
    rng = np.random.default_rng(9)
    th, phi = synth.start_states(w, w.nchain, rng)
    S = w.batch.n_subject
    lp = np.stack([gpu.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = h.loglik(th, abi.FP64)
    plp = gpu.logprior(w.h_prior, phi)
    pll = gpu.loghlike(w.p_prior, phi, th)
    cfg = abi.DEConfigPy(nchain=w.nchain, nparameter=2 * w.model.n_par, nmc=150, thin=1,
                         precision=abi.MIXED, seed=4)
    out = h.run(cfg, w.p_prior, th, lp, ll, h_table=w.h_prior, phi=(phi, plp, pll))
    dev = h.summary(start=50, phi=True)
    for s in range(S):
        smp = out["s_theta"][s]
        host = diagnostics.summary(smp, start=50)
        g = diagnostics.gelman(smp, start=50, form="coda", multivariate=False)
        m, sd, r = (x[s] for x in dev["subj"])
        np.testing.assert_allclose(m, host["mean"], rtol=1e-11, atol=1e-12)
        np.testing.assert_allclose(sd, host["sd"], rtol=1e-9)
        np.testing.assert_allclose(r, g["psrf"][:, 0], rtol=1e-8)
    host = diagnostics.summary(out["phi_s"][0], start=50)
    g = diagnostics.gelman(out["phi_s"][0], start=50, form="coda", multivariate=False)
    np.testing.assert_allclose(dev["phi"][0], host["mean"], rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(dev["phi"][1], host["sd"], rtol=1e-9)
    np.testing.assert_allclose(dev["phi"][2], g["psrf"][:, 0], rtol=1e-8)


def test_summary_needs_a_run():
    w = synth.hier_lba_32(n_subject=2, n=50)
    h = gpu.Handle(w.model, w.batch)
    with pytest.raises(gpu.GGDMCError, match="ARG"):
        h.summary()
