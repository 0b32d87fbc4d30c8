"""Samples reach the caller's buffers while later sweeps run: after each
CUDA-graph replay the runtime copies the slots it stored, for every level,
into a page-locked stage and from there into the caller's arrays, and the
slots after the last whole replay are copied at the end.  Checked against
the oracle and against the same run with the L2-flush timing (which takes
no pipelined copies), over several replays, with thinning and with
iterations left over after the last replay."""
import numpy as np
import pytest

from conftest import load_fixture
from ggdmc_gb300 import abi, gpu, synth
from ggdmc_gb300.dmi import SubjectBatch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from ggdmc_gb300 import build
    build.build()


@pytest.mark.parametrize("nmc,thin,iters", [(30, 2, "8"), (25, 1, "3"), (9, 3, "4")])
def test_pipelined_subject_samples(oracle, monkeypatch, nmc, thin, iters):
    monkeypatch.setenv("GGDMC_GRAPH_ITERS", iters)
    w = synth.many_fits_1024(n_fit=12, n_lo=40, n_hi=200)
    C = 15
    th, _ = synth.start_states(w, C, np.random.default_rng(8))
    lp = np.stack([oracle.logprior(w.p_prior, th[f]) for f in range(12)])
    ll = oracle.loglik(w.model, w.batch, th)
    cfg = abi.DEConfigPy(nchain=C, nparameter=w.model.n_par, nmc=nmc, thin=thin,
                         sub_migration_prob=0.1, seed=21, precision=abi.FP64)
    g = gpu.run_subjects(cfg, w.model, w.batch, w.p_prior, th, lp, ll)
    o = oracle.run_subjects(cfg, w.model, w.batch, w.p_prior, th, lp, ll)
    assert np.array_equal(g["s_theta"], o["s_theta"])
    assert np.allclose(g["s_lp"], o["s_lp"], rtol=1e-12)
    assert np.allclose(g["s_ll"], o["s_ll"], rtol=1e-12)
    # the resident-data API with the L2-flush timing copies everything at the end
    h = gpu.Handle(w.model, w.batch)
    flushed = abi.DEConfigPy(nchain=C, nparameter=w.model.n_par, nmc=nmc, thin=thin,
                             sub_migration_prob=0.1, seed=21, precision=abi.FP64,
                             flags=abi.FLAG_L2_FLUSH)
    r = h.run(flushed, w.p_prior, th, lp, ll)
    assert np.array_equal(r["s_theta"], g["s_theta"])
    assert np.array_equal(r["s_ll"], g["s_ll"])


def test_pipelined_hierarchical_samples(oracle, monkeypatch):
    monkeypatch.setenv("GGDMC_GRAPH_ITERS", "4")
    z, model, _, pop = load_fixture(6)
    S, C = 6, 26
    batch = SubjectBatch(pop.rt[: pop.offsets[S]], pop.cell[: pop.offsets[S]],
                         pop.offsets[: S + 1])
    phi = (z["phi_theta"][:C], z["phi_lp"][:C], z["phi_ll"][:C])
    subj = (z["subj_theta"][:S, :C], z["subj_lp"][:S, :C], z["subj_ll"][:S, :C])
    cfg = abi.DEConfigPy(nchain=C, nparameter=2 * model.n_par, nmc=14, thin=1,
                         pop_migration_prob=0.2, sub_migration_prob=0.2, seed=5)
    g = gpu.run(cfg, model, batch, z["pop_p_prior"], z["pop_h_prior"], phi, subj)
    o = oracle.run(cfg, model, batch, z["pop_p_prior"], z["pop_h_prior"], phi, subj)
    assert np.array_equal(g["phi_s"][0], o["phi_s"][0])
    assert np.allclose(g["phi_s"][2], o["phi_s"][2], rtol=1e-12)
    assert np.array_equal(g["subj_s"][0], o["subj_s"][0])
    assert np.allclose(g["subj_s"][2], o["subj_s"][2], rtol=1e-12)
