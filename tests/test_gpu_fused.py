"""The subject pass fused with the next iteration's proposals (k_sub_step and
k_sub_spec_rest) against the oracle, through the C ABI.  The runtime takes
the fused schedule by itself for many independent fits (at least two waves
of levels per SM) and for hierarchical runs of more than one wave;
GGDMC_FUSED=1 forces it here on small cases, with
and without a phi level, in CUDA-graph replays and in the iterations
launched one by one after the last whole graph."""
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


def _fits(oracle, n_fit, C):
    w = synth.many_fits_1024(n_fit=n_fit, n_lo=50, n_hi=400)
    th, _ = synth.start_states(w, C, np.random.default_rng(5))
    lp = np.stack([oracle.logprior(w.p_prior, th[f]) for f in range(n_fit)])
    ll = oracle.loglik(w.model, w.batch, th)
    return w, th, lp, ll


@pytest.mark.parametrize("mig,iters", [(0.0, "8"), (0.25, "8"), (0.25, "3")])
def test_fused_subjects_bit_exact(oracle, monkeypatch, mig, iters):
    monkeypatch.setenv("GGDMC_FUSED", "1")
    monkeypatch.setenv("GGDMC_GRAPH_ITERS", iters)     # "3": 2 replays + 1 eager iteration
    w, th, lp, ll = _fits(oracle, 40, 27)
    cfg = abi.DEConfigPy(nchain=27, nparameter=w.model.n_par, nmc=8, thin=1,
                         sub_migration_prob=mig, seed=12, precision=abi.FP64)
    g = gpu.run_subjects(cfg, w.model, w.batch, w.p_prior, th, lp, ll)
    o = oracle.run_subjects(cfg, w.model, w.batch, w.p_prior, th, lp, ll)
    assert np.array_equal(g["theta"], o["theta"])
    assert np.array_equal(g["s_theta"], o["s_theta"])
    assert np.allclose(g["ll"], o["ll"], rtol=1e-12)
    assert g["stats"]["accepts"] == o["stats"].accepts > 0
    if mig:
        assert g["stats"]["migrations"] == o["stats"].migrations > 0


def test_fused_hierarchical_bit_exact(oracle, monkeypatch):
    monkeypatch.setenv("GGDMC_FUSED", "1")
    z, model, _, pop = load_fixture(6)
    S, C = 8, 26
    batch = SubjectBatch(pop.rt[: pop.offsets[S]], pop.cell[: pop.offsets[S]],
                         pop.offsets[: S + 1])
    phi = (z["phi_theta"][:C], z["phi_lp"][:C], z["phi_ll"][:C])
    subj = (z["subj_theta"][:S, :C], z["subj_lp"][:S, :C], z["subj_ll"][:S, :C])
    cfg = abi.DEConfigPy(nchain=C, nparameter=2 * model.n_par, nmc=6, thin=2,
                         pop_migration_prob=0.3, sub_migration_prob=0.3, seed=77)
    g = gpu.run(cfg, model, batch, z["pop_p_prior"], z["pop_h_prior"], phi, subj)
    o = oracle.run(cfg, model, batch, z["pop_p_prior"], z["pop_h_prior"], phi, subj)
    assert np.array_equal(g["phi"][0], o["phi"][0])
    assert np.array_equal(g["subj"][0], o["subj"][0])
    assert np.array_equal(g["phi_s"][0], o["phi_s"][0])
    assert np.allclose(g["subj"][2], o["subj"][2], rtol=1e-12)
    assert g["stats"]["accepts"] == o["stats"].accepts


def test_fused_and_unfused_agree_mixed(oracle, monkeypatch):
    # the same run on one handle under both schedules: the same decisions
    w, th, lp, ll = _fits(oracle, 48, 39)
    h = gpu.Handle(w.model, w.batch)
    cfg = abi.DEConfigPy(nchain=39, nparameter=w.model.n_par, nmc=12, thin=1,
                         sub_migration_prob=0.06, seed=3, precision=abi.MIXED)
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("GGDMC_FUSED", mode)
        out[mode] = h.run(cfg, w.p_prior, th, lp, ll)
    a, b = out["0"], out["1"]
    # a proposal's FP32 sum is an exact integer sum of its trials' terms, the
    # same bits in the 512-thread resolve blocks and the 128-thread
    # speculative ones: the two schedules give the same numbers
    for k in ("theta", "ll", "lp", "s_theta", "s_ll"):
        np.testing.assert_array_equal(a[k], b[k])
    for k in ("accepts", "trial_evals", "migrations", "proposals"):
        assert a["stats"][k] == b["stats"][k]


def test_fused_and_unfused_agree_mixed_hierarchical(monkeypatch):
    # hierarchical, many migrating subjects, few subjects per SM (so the
    # fused schedule's idle blocks help the migrating subjects' rounds)
    w = synth.uneven_lba_256(seed=5, n_subject=24, n_lo=150, n_hi=900)
    h = gpu.Handle(w.model, w.batch)
    S, P = w.batch.n_subject, w.model.n_par
    th, phi = synth.start_states(w, w.nchain, np.random.default_rng(8))
    lp = np.stack([gpu.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = h.loglik(th, abi.MIXED_SUMS)
    plp = gpu.logprior(w.h_prior, phi)
    pll = gpu.loghlike(w.p_prior, phi, th)
    cfg = abi.DEConfigPy(nchain=w.nchain, nparameter=2 * P, nmc=9, thin=1, pop_migration_prob=0.2,
                         sub_migration_prob=0.5, seed=19, precision=abi.MIXED)
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("GGDMC_FUSED", mode)
        out[mode] = h.run(cfg, w.p_prior, th, lp, ll, h_table=w.h_prior, phi=(phi, plp, pll))
    a, b = out["0"], out["1"]
    assert a["stats"]["migrations"] > 20
    for k in ("theta", "ll", "lp", "s_theta", "s_ll"):
        np.testing.assert_array_equal(a[k], b[k])
    for x, y in zip(a["phi_s"], b["phi_s"]):
        np.testing.assert_array_equal(x, y)
    for k in ("accepts", "migrations", "proposals"):
        assert a["stats"][k] == b["stats"][k]


@pytest.mark.parametrize("group", ["1", "2", "4"])
def test_spec_group_sizes_bit_exact(oracle, monkeypatch, group):
    # the number of proposals per speculative work item only regroups the
    # work: each proposal's trials are summed over the same thread partition
    monkeypatch.setenv("GGDMC_SPEC_GROUP", group)
    z, model, _, pop = load_fixture(6)
    S, C = 8, 26
    batch = SubjectBatch(pop.rt[: pop.offsets[S]], pop.cell[: pop.offsets[S]],
                         pop.offsets[: S + 1])
    phi = (z["phi_theta"][:C], z["phi_lp"][:C], z["phi_ll"][:C])
    subj = (z["subj_theta"][:S, :C], z["subj_lp"][:S, :C], z["subj_ll"][:S, :C])
    cfg = abi.DEConfigPy(nchain=C, nparameter=2 * model.n_par, nmc=4, thin=1,
                         pop_migration_prob=0.3, sub_migration_prob=0.3, seed=31)
    g = gpu.run(cfg, model, batch, z["pop_p_prior"], z["pop_h_prior"], phi, subj)
    o = oracle.run(cfg, model, batch, z["pop_p_prior"], z["pop_h_prior"], phi, subj)
    assert np.array_equal(g["subj"][0], o["subj"][0])
    assert np.array_equal(g["phi"][0], o["phi"][0])
    assert np.allclose(g["subj"][2], o["subj"][2], rtol=1e-12)
