"""ggdmc_handle_summary and ggdmc_handle_diagnostics: posterior summaries
and PSRFs computed on the device from the samples a run left there, against
ggdmc_gb300.diagnostics on the same samples copied to the host."""
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


@pytest.mark.parametrize("form", ["reference", "coda"])
def test_device_diagnostics_match_host(form):
    """ggdmc_handle_diagnostics (summary's Mean, SD, Naive SE, Time-series SE
    and quantiles; gelman's point estimate and upper C.I.) against the host
    restatements on the same samples, subject and phi levels."""
    w = synth.hier_lba_32(n_subject=3, n=150)
    h = gpu.Handle(w.model, w.batch)
    th, phi = synth.start_states(w, w.nchain, np.random.default_rng(11))
    S = w.batch.n_subject
    lp = np.stack([gpu.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = h.loglik(th, abi.FP64)
    plp = gpu.logprior(w.h_prior, phi)
    pll = gpu.loghlike(w.p_prior, phi, th)
    cfg = abi.DEConfigPy(nchain=w.nchain, nparameter=2 * w.model.n_par, nmc=240, thin=1,
                         precision=abi.MIXED, seed=5)
    out = h.run(cfg, w.p_prior, th, lp, ll, h_table=w.h_prior, phi=(phi, plp, pll))
    probs = (0.05, 0.5, 0.975)
    fcode = abi.PSRF_REFERENCE if form == "reference" else abi.PSRF_CODA
    dev = h.diagnostics(start=40, end=0, probs=probs, conf=0.95, form=fcode, phi=True)
    levels = [(dev["subj"], s, out["s_theta"][s]) for s in range(S)] + [(dev["phi"], None, out["phi_s"][0])]
    for d, s, smp in levels:
        pick = (lambda v: v[s]) if s is not None else (lambda v: v)
        host = diagnostics.summary(smp, start=40, probs=probs)
        g = diagnostics.gelman(smp, start=40, form=form, multivariate=False)
        np.testing.assert_allclose(pick(d["mean"]), host["mean"], rtol=1e-11, atol=1e-13)
        np.testing.assert_allclose(pick(d["sd"]), host["sd"], rtol=1e-9)
        np.testing.assert_allclose(pick(d["naive_se"]), host["naive_se"], rtol=1e-9)
        np.testing.assert_allclose(pick(d["ts_se"]), host["ts_se"], rtol=1e-7)
        np.testing.assert_array_equal(pick(d["quantiles"]), host["quantiles"].T)
        np.testing.assert_allclose(pick(d["psrf"]), g["psrf"], rtol=1e-8)


def test_diagnostics_argument_errors():
    w = synth.hier_lba_32(n_subject=2, n=60)
    h = gpu.Handle(w.model, w.batch)
    with pytest.raises(gpu.GGDMCError, match="ARG"):
        h.diagnostics()                                           # no run yet
    th, _ = synth.start_states(w, 3, np.random.default_rng(2))
    lp = np.stack([gpu.logprior(w.p_prior, th[s]) for s in range(2)])
    ll = h.loglik(th, abi.FP64)
    cfg = abi.DEConfigPy(nchain=3, nparameter=w.model.n_par, nmc=20, thin=1, seed=1)
    h.run(cfg, w.p_prior, th, lp, ll)
    with pytest.raises(gpu.GGDMCError, match="more than one element"):
        h.diagnostics(probs=(0.5,))
    with pytest.raises(gpu.GGDMCError, match="two or more iterations"):
        h.diagnostics(start=19)
    d = h.diagnostics(probs=())
    assert np.all(np.isfinite(d["subj"]["psrf"][..., 0]))
