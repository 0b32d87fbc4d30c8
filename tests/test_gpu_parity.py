"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle.

Tolerances:
* FP64 path: per-subject log-likelihood sums within 1e-12 relative of the
  oracle (1e-11 absolute for sums near zero, whose last bits depend on the
  summation order); chain states after a run bit-identical (same keyed draws,
  so the same partners, subsets and accept decisions).
* MIXED path (ggdmc_loglik): every per-subject sum within 1e-6 relative of
  the FP64 oracle, |mixed - fp64| <= 1e-6 |fp64|, on the data of all five
  workloads; per trial within 2e-5 absolute, median within 2e-7.
"""
import numpy as np
import pytest

from conftest import PINNED_LBA_FIXTURES, load_fixture
from ggdmc_gb300 import abi, gpu, synth
from ggdmc_gb300.dmi import SubjectBatch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from ggdmc_gb300 import build
    build.build()


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(np.asarray(b)), 1e-300)


@pytest.mark.parametrize("fx", PINNED_LBA_FIXTURES)
def test_fp64_loglik_matches_oracle_and_golden(oracle, fx):
    z, model, sub, pop = load_fixture(fx)
    h = gpu.Handle(model, pop)
    S = pop.n_subject
    got = h.loglik(z["subj_theta"][:S], abi.FP64)
    want = oracle.loglik(model, pop, z["subj_theta"][:S])
    assert np.all(rel(got, want) <= 1e-12), rel(got, want).max()
    assert np.all(rel(got, z["subj_ll"][:S]) <= 2e-9)
    hs = gpu.Handle(model, sub)
    got1 = hs.loglik(z["sub_theta"][None], abi.FP64)[0]
    assert np.all(rel(got1, z["sub_ll"]) <= 2e-9)


def test_fp64_per_trial_log_densities(oracle):
    z, model, _, pop = load_fixture(6)
    h = gpu.Handle(model, pop)
    S = pop.n_subject
    theta = z["subj_theta"][:S, 0]
    got = h.trial_logdens(theta, abi.FP64)
    for s in range(S):
        a, b = pop.offsets[s], pop.offsets[s + 1]
        _, want = oracle.sumloglike(model, pop.rt[a:b], pop.cell[a:b], theta[s], per_trial=True)
        assert np.allclose(got[a:b], want, rtol=1e-12, atol=1e-12)


def near_truth(w, n, rng, spread):
    th = w.theta_true[:, None, :] * (1 + spread * rng.standard_normal((w.theta_true.shape[0], n,
                                                                       w.theta_true.shape[1])))
    return np.abs(th)


def single_lba_768():
    from ggdmc_gb300.design import BV13_POP_MEAN, design_bv13, vector
    rng = np.random.default_rng(0)
    model = design_bv13()
    th = vector(model, BV13_POP_MEAN)
    sub = synth.simulate_subject(model, th, 768, rng, "1")
    return synth.Workload("single_lba_768", model, SubjectBatch.pack([sub]), th[None],
                          synth.unif_prior(model.n_par), None, None, None, 3 * model.n_par, False)


def many_fits_subset():
    # 96 fits of the many-fit design (trial counts U{200..5000} as in the full workload)
    return synth.many_fits_1024(n_fit=96)


WORKLOADS = {
    "single_lba_768": single_lba_768,
    "hier_lba_32": synth.hier_lba_32,
    "uneven_lba_256": synth.uneven_lba_256,
    "hier_ddm_64": synth.hier_ddm_64,
    "many_fits_1024": many_fits_subset,
}


@pytest.mark.parametrize("name", sorted(WORKLOADS))
def test_mixed_loglik_within_1e6_relative(oracle, name):
    """Chains scattered around the generating values (5% and 20%), as the
    benchmark starts: sums of either sign, some near zero."""
    w = WORKLOADS[name]()
    rng = np.random.default_rng(3)
    h = gpu.Handle(w.model, w.batch)
    for spread in (0.05, 0.2):
        theta = synth.start_states(w, min(w.nchain, 12), rng, spread=spread)[0]
        mixed = h.loglik(theta, abi.MIXED)
        want = oracle.loglik(w.model, w.batch, theta)
        err = np.abs(mixed - want)
        assert np.all(err <= 1e-6 * np.abs(want)), (spread, (err / np.abs(want)).max())
        fp64 = h.loglik(theta, abi.FP64)
        assert np.all(np.abs(fp64 - want) <= 1e-12 * np.abs(want) + 1e-11)


def test_mixed_trial_logdens_per_trial(oracle):
    # each FP32 trial density against the FP64 oracle
    w = synth.uneven_lba_256(n_subject=48)
    rng = np.random.default_rng(4)
    theta = near_truth(w, 1, rng, 0.05)[:, 0, :]
    h = gpu.Handle(w.model, w.batch)
    got = h.trial_logdens(theta, abi.MIXED)
    want = np.concatenate([
        oracle.sumloglike(w.model, w.batch.subject(s).rt, w.batch.subject(s).cell, theta[s],
                          per_trial=True)[1] for s in range(w.batch.n_subject)])
    err = np.abs(got - want)
    assert err.max() <= 2e-5, err.max()
    assert np.median(err) <= 2e-7, np.median(err)
    assert abs(np.mean(got - want)) <= 2e-8          # no bias that sums would accumulate


def test_mixed_loglik_fixtures_close(oracle):
    # prior draws of the fixtures: wild parameters, many FP64 re-evaluations
    for fx in (3, 6):
        z, model, _, pop = load_fixture(fx)
        h = gpu.Handle(model, pop)
        S = pop.n_subject
        mixed = h.loglik(z["subj_theta"][:S], abi.MIXED)
        want = oracle.loglik(model, pop, z["subj_theta"][:S])
        assert np.all(np.abs(mixed - want) <= 1e-6 * np.abs(want)), rel(mixed, want).max()


def test_mixed_small_start_point_range(oracle):
    """A start-point range A of 1e-6 .. 1e-2 (the sampler reaches it when A is
    weakly identified): the closed forms cancel there and the quadrature
    branch takes over."""
    w = synth.many_fits_1024(n_fit=8, n_lo=300, n_hi=600)
    rng = np.random.default_rng(8)
    theta = near_truth(w, 6, rng, 0.05)
    ia = w.model.pnames.index("A")
    theta[:, :, ia] = 10.0 ** rng.uniform(-6, -2, theta.shape[:2])
    h = gpu.Handle(w.model, w.batch)
    mixed = h.loglik(theta, abi.MIXED)
    want = oracle.loglik(w.model, w.batch, theta)
    assert np.all(np.abs(mixed - want) <= 1e-6 * np.abs(want)), rel(mixed, want).max()


def informative(z, C):
    idx = np.argsort(z["sub_ll"])[::-1][:C]
    return z["sub_theta"][idx].copy(), z["sub_lp"][idx].copy(), z["sub_ll"][idx].copy()


@pytest.mark.parametrize("mig,blocked", [(0.0, False), (0.3, False), (0.15, True)])
def test_run_subject_fp64_bit_exact(oracle, mig, blocked):
    z, model, sub, _ = load_fixture(6)
    th, lp, ll = informative(z, 39)
    cfg = abi.DEConfigPy(nchain=39, nparameter=model.n_par, nmc=6, thin=2,
                         sub_migration_prob=mig, is_pblocked=blocked, seed=2024)
    g = gpu.run_subjects(cfg, model, sub, z["sub_prior"], th[None], lp[None], ll[None])
    o = oracle.run_subjects(cfg, model, sub, z["sub_prior"], th[None], lp[None], ll[None])
    assert np.array_equal(g["theta"], o["theta"])
    assert np.array_equal(g["s_theta"], o["s_theta"])
    assert np.allclose(g["ll"], o["ll"], rtol=1e-12)
    assert np.allclose(g["s_lp"], o["s_lp"], rtol=1e-12)
    assert g["stats"]["accepts"] == o["stats"].accepts > 0
    assert g["stats"]["kernel_launches"] > 0


def test_run_subject_host_fed_draws(oracle):
    z, model, sub, _ = load_fixture(6)
    th, lp, ll = informative(z, 15)
    cfg = abi.DEConfigPy(nchain=15, nparameter=model.n_par, nmc=5, thin=1,
                         sub_migration_prob=0.25, seed=0)
    ni, npass, ns = abi.draw_layout(cfg, 1, False)
    draws = np.random.default_rng(11).random(ni * npass * ns)
    g = gpu.run_subjects(cfg, model, sub, z["sub_prior"], th[None], lp[None], ll[None], draws)
    o = oracle.run_subjects(cfg, model, sub, z["sub_prior"], th[None], lp[None], ll[None], draws)
    assert np.array_equal(g["theta"], o["theta"])


@pytest.mark.parametrize("pm,sm,hb,pb", [(0.0, 0.0, False, False), (0.3, 0.3, False, False),
                                         (0.2, 0.2, True, True)])
def test_run_hierarchical_fp64_bit_exact(oracle, pm, sm, hb, pb):
    z, model, _, pop = load_fixture(6)
    S, C = 8, 26
    batch = SubjectBatch(pop.rt[: pop.offsets[S]], pop.cell[: pop.offsets[S]],
                         pop.offsets[: S + 1])
    phi = (z["phi_theta"][:C], z["phi_lp"][:C], z["phi_ll"][:C])
    subj = (z["subj_theta"][:S, :C], z["subj_lp"][:S, :C], z["subj_ll"][:S, :C])
    cfg = abi.DEConfigPy(nchain=C, nparameter=2 * model.n_par, nmc=4, thin=1,
                         pop_migration_prob=pm, sub_migration_prob=sm, is_hblocked=hb,
                         is_pblocked=pb, seed=31)
    g = gpu.run(cfg, model, batch, z["pop_p_prior"], z["pop_h_prior"], phi, subj)
    o = oracle.run(cfg, model, batch, z["pop_p_prior"], z["pop_h_prior"], phi, subj)
    assert np.array_equal(g["phi"][0], o["phi"][0])
    assert np.allclose(g["phi"][2], o["phi"][2], rtol=1e-12)
    assert np.array_equal(g["subj"][0], o["subj"][0])
    assert np.allclose(g["subj"][2], o["subj"][2], rtol=1e-12)
    assert np.array_equal(g["phi_s"][0], o["phi_s"][0])
    assert g["stats"]["accepts"] == o["stats"].accepts


def test_run_hyper_fp64_bit_exact(oracle):
    z, model, _, _ = load_fixture(6)
    rows = z["subj_theta"][:, 0, :]        # a subject-by-parameter matrix
    C = 26
    theta = z["phi_theta"][:C]
    lp = oracle.logprior(z["pop_h_prior"], theta)
    ll = oracle.loghlike(z["pop_p_prior"], theta, np.repeat(rows[:, None, :], C, axis=1))
    cfg = abi.DEConfigPy(nchain=C, nparameter=2 * model.n_par, nmc=5, thin=1,
                         sub_migration_prob=0.2, seed=8)
    g = gpu.run_hyper(cfg, rows, z["pop_p_prior"], z["pop_h_prior"], theta, lp, ll)
    o = oracle.run_hyper(cfg, rows, z["pop_p_prior"], z["pop_h_prior"], theta, lp, ll)
    assert np.array_equal(g["theta"], o["theta"])
    assert np.allclose(g["ll"], o["ll"], rtol=1e-12)


def test_gpu_priors_match_oracle(oracle):
    for fx in (3, 6):
        z, *_ = load_fixture(fx)
        assert np.allclose(gpu.logprior(z["sub_prior"], z["sub_theta"]), z["sub_lp"], rtol=1e-12)
        got = gpu.loghlike(z["pop_p_prior"], z["phi_theta"], z["subj_theta"])
        assert np.allclose(got, z["phi_ll"], rtol=1e-12)


def test_many_fits_match_oracle(oracle):
    w = synth.many_fits_1024(n_fit=6, n_lo=50, n_hi=300)
    rng = np.random.default_rng(0)
    C = 39
    th, _ = synth.start_states(w, C, rng)
    lp = np.stack([oracle.logprior(w.p_prior, th[f]) for f in range(6)])
    ll = oracle.loglik(w.model, w.batch, th)
    cfg = abi.DEConfigPy(nchain=C, nparameter=w.model.n_par, nmc=4, thin=1,
                         sub_migration_prob=0.06, seed=4)
    g = gpu.run_subjects(cfg, w.model, w.batch, w.p_prior, th, lp, ll)
    o = oracle.run_subjects(cfg, w.model, w.batch, w.p_prior, th, lp, ll)
    assert np.array_equal(g["theta"], o["theta"])


def test_edge_empty_subject_and_floor(oracle):
    z, model, sub, _ = load_fixture(6)
    rt = np.concatenate([sub.rt[:10], sub.rt[:0], sub.rt[:5]])
    cell = np.concatenate([sub.cell[:10], sub.cell[:0], sub.cell[:5]])
    batch = SubjectBatch(rt, cell, np.array([0, 10, 10, 15], np.int64))
    h = gpu.Handle(model, batch)
    th = np.repeat(z["sub_theta"][None, :2], 3, axis=0)
    th[:, 1, model.pnames.index("t0")] = 50.0        # t0 beyond every RT: all floors
    got = h.loglik(th, abi.FP64)
    assert got[1, 0] == 0.0 and got[1, 1] == 0.0     # no trials, no log-likelihood
    assert np.allclose(got[0, 1], 10 * np.log(1e-10), rtol=1e-13)
    want = oracle.loglik(model, batch, th)
    assert np.allclose(got, want, rtol=1e-12)


def test_mixed_many_fallbacks_in_one_block(oracle):
    # one subject of 3000 trials with drift rates 8x the generating ones: the
    # responses are far too slow for them, so nearly every trial follows the
    # reference form's FP64 rounding (a winner bracket of differences of Phi
    # near 1, survivors of terms far above their size) and leaves the FP32
    # form, more than a block lists, so the block re-scans its trials; sums
    # still match the FP64 oracle.  And t0 above 60% of the RTs: those trials
    # take the reference's floor, the ones just after t0 (a response far too
    # fast for the winner) the floor by the bound on the bracket
    from ggdmc_gb300.design import T0_17_P, design_t0_17, vector
    rng = np.random.default_rng(21)
    model = design_t0_17()
    th = vector(model, T0_17_P)
    sub = synth.simulate_subject(model, th, 3000, rng, "1")
    batch = SubjectBatch.pack([sub])
    bad, late = th.copy(), th.copy()
    for j, nm in enumerate(model.pnames):
        if nm.startswith("mean_v"):
            bad[j] = 8.0 * th[j]
        if nm.startswith("t0"):
            late[j] = np.quantile(sub.rt, 0.6)
    theta = np.stack([th, bad, late])[None]            # [1][3][P]
    h = gpu.Handle(model, batch)
    want = oracle.loglik(model, batch, theta)
    mixed = h.loglik(theta, abi.MIXED)
    assert np.all(rel(mixed, want) <= 1e-6), rel(mixed, want)
    sums = h.loglik(theta, abi.MIXED_SUMS)
    assert rel(sums[0, 2], want[0, 2]) <= 1e-6
    run = h.run(abi.DEConfigPy(nchain=3, nparameter=model.n_par, nmc=2, thin=1, seed=1,
                               precision=abi.MIXED), synth.unif_prior(model.n_par, 0.0, 50.0),
                np.stack([bad] * 3)[None], np.zeros((1, 3)), h.loglik(np.stack([bad] * 3)[None], abi.MIXED))
    assert run["stats"]["fallbacks"] > 1024


def test_invalid_inputs_are_errors():
    z, model, sub, _ = load_fixture(6)
    bad = SubjectBatch(sub.rt[:5], np.full(5, model.n_cell + 3, np.int32), np.array([0, 5]))
    with pytest.raises(gpu.GGDMCError) as e:
        gpu.Handle(model, bad)
    assert e.value.status == abi.GGDMC_ERR_ARG
    cfg = abi.DEConfigPy(nchain=2, nparameter=model.n_par, nmc=2)
    th, lp, ll = informative(z, 2)
    with pytest.raises(gpu.GGDMCError):
        gpu.run_subjects(cfg, model, sub, z["sub_prior"], th[None], lp[None], ll[None])
    prior = z["sub_prior"].copy()
    prior[0, 4] = 3.0                                # unsupported dist_id
    cfg = abi.DEConfigPy(nchain=3, nparameter=model.n_par, nmc=2)
    th, lp, ll = informative(z, 3)
    with pytest.raises(gpu.GGDMCError):
        gpu.run_subjects(cfg, model, sub, prior, th[None], lp[None], ll[None])


def test_mixed_sums_are_the_sampler_sums_refined_only_near_zero():
    """GGDMC_MIXED_SUMS returns the FP32 sums as the sampler forms them;
    GGDMC_MIXED re-evaluates in FP64 only the sums whose FP32 error could
    reach 1e-6 of their size (|sum| < 1.2 sqrt(N) + 0.03 N): the others are
    the same numbers bit for bit, the refined ones are within 1e-12 of the
    FP64 sums."""
    w = synth.uneven_lba_256(n_subject=64)
    rng = np.random.default_rng(8)
    th = near_truth(w, 12, rng, 0.2)
    h = gpu.Handle(w.model, w.batch)
    sums = h.loglik(th, abi.MIXED_SUMS)
    refined = h.loglik(th, abi.MIXED)
    fp64 = h.loglik(th, abi.FP64)
    n = np.diff(w.batch.offsets)[:, None] * np.ones((1, th.shape[1]))
    near = np.abs(sums) < 1.2 * np.sqrt(n) + 0.03 * n
    assert near.any() and (~near).any()
    np.testing.assert_array_equal(refined[~near], sums[~near])
    np.testing.assert_allclose(refined[near], fp64[near], rtol=1e-12, atol=1e-11)
    assert np.all(rel(sums[~near], fp64[~near]) <= 1e-6)


@pytest.mark.parametrize("fused", ["0", "1"])
def test_sampler_sums_equal_the_api_sums(monkeypatch, fused):
    """A proposal's FP32 sum is an exact integer sum of per-trial terms, so it
    is the same number in every kernel that forms it: every log-likelihood a
    mixed run stores (the speculative evaluation, the resolve's
    re-evaluations, migration variants; with GGDMC_FUSED=1 the fused
    schedule) equals GGDMC_MIXED_SUMS of its theta bit for bit."""
    monkeypatch.setenv("GGDMC_FUSED", fused)
    w = synth.uneven_lba_256(n_subject=24, n_lo=40, n_hi=900)
    h = gpu.Handle(w.model, w.batch)
    S, C, P = w.batch.n_subject, 18, w.model.n_par
    th = near_truth(w, C, np.random.default_rng(21), 0.1)
    lp = np.stack([gpu.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = h.loglik(th, abi.MIXED_SUMS)
    cfg = abi.DEConfigPy(nchain=C, nparameter=P, nmc=7, thin=1, sub_migration_prob=0.3,
                         precision=abi.MIXED, seed=31)
    out = h.run(cfg, w.p_prior, th, lp, ll)
    st = out["stats"]
    assert st["reevaluations"] > 0 and st["migrations"] > 0 and st["accepts"] > 0
    smp = out["s_theta"].reshape(S, -1, P)                 # every stored sample
    np.testing.assert_array_equal(h.loglik(smp, abi.MIXED_SUMS), out["s_ll"].reshape(S, -1))
    np.testing.assert_array_equal(h.loglik(out["theta"], abi.MIXED_SUMS), out["ll"])
