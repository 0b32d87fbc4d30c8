"""FP64 chains on the full 256-subject workload, bit for bit against the oracle.

The workload is the one the benchmark times: 256 subjects with N_s ~
U{100..2000} (272,607 trials), the 17-parameter 4-accumulator LBA design, 51
chains, a phi level of 34 parameters and the start states the benchmark uses.
Each case runs 6 sweeps through the one-shot ``ggdmc_run`` and compares every
phi and subject chain, every stored sample and the accept count with the
oracle's sequential run (src/de.cpp:272-383) given the same keyed draws:

* migration at the workload's rates (0.05 phi, 0.06 subjects) and raised to
  0.3 for both levels, so that dozens of subjects migrate in one pass;
* the ordered resolve (GGDMC_FUSED=0) and the persistent fused schedule
  (GGDMC_FUSED=1, which the runtime picks by itself for this workload);
* host-fed draws (the canonical draw array of include/ggdmc_gpu.h) for
  ``ggdmc_run`` on the full workload and for ``ggdmc_run_hyper``.

The oracle runs (about 2 s per sweep each on one core) start in threads when
the module is collected, so they overlap the GPU cases.
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

from conftest import load_fixture
from ggdmc_gb300 import abi, gpu, synth

pytestmark = pytest.mark.gpu

NMC = 7                                     # 6 sweeps after the start slot
RATES = {"workload": (0.05, 0.06), "raised": (0.3, 0.3)}


def full_workload(oracle):
    w = synth.uneven_lba_256()
    th, phi = synth.start_states(w, w.nchain, np.random.default_rng(12))
    S = w.batch.n_subject
    lp = np.stack([oracle.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = oracle.loglik(w.model, w.batch, th)
    plp = oracle.logprior(w.h_prior, phi)
    pll = oracle.loghlike(w.p_prior, phi, th)
    return w, (phi, plp, pll), (th, lp, ll)


def cfg_of(w, rates, nmc=NMC, seed=2025):
    pm, sm = rates
    return abi.DEConfigPy(nchain=w.nchain, nparameter=2 * w.model.n_par, nmc=nmc, thin=1,
                          pop_migration_prob=pm, sub_migration_prob=sm, seed=seed,
                          precision=abi.FP64)


def host_draws(w, cfg, seed=17):
    ni, npass, ns = abi.draw_layout(cfg, w.batch.n_subject + 1, True)
    return np.random.default_rng(seed).random(ni * (w.batch.n_subject + 1) * npass * ns)


@pytest.fixture(scope="module")
def setup(oracle):
    from ggdmc_gb300 import build
    build.build()
    w, phi, subj = full_workload(oracle)
    pool = cf.ThreadPoolExecutor(max_workers=min(5, os.cpu_count() or 1))
    futs = {}
    for key, rates in RATES.items():
        cfg = cfg_of(w, rates)
        futs[key] = pool.submit(oracle.run, cfg, w.model, w.batch, w.p_prior, w.h_prior, phi, subj)
    dcfg = cfg_of(w, RATES["raised"], nmc=4, seed=0)
    draws = host_draws(w, dcfg)
    futs["draws"] = pool.submit(oracle.run, dcfg, w.model, w.batch, w.p_prior, w.h_prior, phi, subj,
                                draws)
    yield dict(w=w, phi=phi, subj=subj, futs=futs, dcfg=dcfg, draws=draws)
    pool.shutdown(wait=True)


# Log-likelihood sums: the GPU adds a subject's trial terms in a block
# reduction, the oracle in sequence, so a sum near zero (some subjects' sums
# are ~0.01) differs in its last bits; within 1e-12 relative or 1e-11 absolute.
LL_TOL = dict(rtol=1e-12, atol=1e-11)


def assert_same_run(g, o):
    assert np.array_equal(g["phi"][0], o["phi"][0])
    assert np.array_equal(g["subj"][0], o["subj"][0])
    assert np.array_equal(g["phi_s"][0], o["phi_s"][0])
    assert np.array_equal(g["subj_s"][0], o["subj_s"][0])
    np.testing.assert_allclose(g["subj"][2], o["subj"][2], **LL_TOL)
    np.testing.assert_allclose(g["phi"][2], o["phi"][2], **LL_TOL)
    np.testing.assert_allclose(g["subj_s"][1], o["subj_s"][1], **LL_TOL)
    np.testing.assert_allclose(g["subj_s"][2], o["subj_s"][2], **LL_TOL)
    assert g["stats"]["accepts"] == o["stats"].accepts > 0
    assert g["stats"]["migrations"] == o["stats"].migrations


@pytest.mark.parametrize("fused", ["0", "1"])
@pytest.mark.parametrize("rates", sorted(RATES))
def test_full_workload_fp64_bit_exact(setup, monkeypatch, rates, fused):
    monkeypatch.setenv("GGDMC_FUSED", fused)
    w = setup["w"]
    cfg = cfg_of(w, RATES[rates])
    g = gpu.run(cfg, w.model, w.batch, w.p_prior, w.h_prior, setup["phi"], setup["subj"])
    o = setup["futs"][rates].result()
    assert_same_run(g, o)
    if rates == "raised":
        # many subjects migrate in the same pass (256 x 6 passes at p = 0.3)
        assert o["stats"].migrations >= 300


def test_full_workload_host_fed_draws(setup):
    w = setup["w"]
    g = gpu.run(setup["dcfg"], w.model, w.batch, w.p_prior, w.h_prior, setup["phi"], setup["subj"],
                setup["draws"])
    assert_same_run(g, setup["futs"]["draws"].result())


def test_run_hyper_host_fed_draws(oracle):
    z, model, _, _ = load_fixture(6)
    rows = z["subj_theta"][:, 0, :]
    C = 26
    theta = z["phi_theta"][:C]
    lp = oracle.logprior(z["pop_h_prior"], theta)
    ll = oracle.loghlike(z["pop_p_prior"], theta, np.repeat(rows[:, None, :], C, axis=1))
    for blocked in (False, True):
        cfg = abi.DEConfigPy(nchain=C, nparameter=2 * model.n_par, nmc=10, thin=1,
                             sub_migration_prob=0.25, is_pblocked=blocked, seed=0)
        ni, npass, ns = abi.draw_layout(cfg, 1, False)
        draws = np.random.default_rng(23).random(ni * npass * ns)
        g = gpu.run_hyper(cfg, rows, z["pop_p_prior"], z["pop_h_prior"], theta, lp, ll, draws)
        o = oracle.run_hyper(cfg, rows, z["pop_p_prior"], z["pop_h_prior"], theta, lp, ll, draws)
        assert np.array_equal(g["theta"], o["theta"])
        assert np.array_equal(g["s_theta"], o["s_theta"])
        np.testing.assert_allclose(g["ll"], o["ll"], **LL_TOL)
        assert g["stats"]["accepts"] == o["stats"].accepts > 0


@pytest.mark.parametrize("blocked", [False, True])
def test_hierarchical_host_fed_draws_fixture(oracle, blocked):
    from ggdmc_gb300.dmi import SubjectBatch
    z, model, _, pop = load_fixture(6)
    S, C = 8, 26
    batch = SubjectBatch(pop.rt[: pop.offsets[S]], pop.cell[: pop.offsets[S]],
                         pop.offsets[: S + 1])
    phi = (z["phi_theta"][:C], z["phi_lp"][:C], z["phi_ll"][:C])
    subj = (z["subj_theta"][:S, :C], z["subj_lp"][:S, :C], z["subj_ll"][:S, :C])
    cfg = abi.DEConfigPy(nchain=C, nparameter=2 * model.n_par, nmc=4, thin=2,
                         pop_migration_prob=0.3, sub_migration_prob=0.3, is_hblocked=blocked,
                         is_pblocked=blocked, seed=0)
    ni, npass, ns = abi.draw_layout(cfg, S + 1, True)
    draws = np.random.default_rng(29).random(ni * (S + 1) * npass * ns)
    g = gpu.run(cfg, model, batch, z["pop_p_prior"], z["pop_h_prior"], phi, subj, draws)
    o = oracle.run(cfg, model, batch, z["pop_p_prior"], z["pop_h_prior"], phi, subj, draws)
    assert_same_run(g, o)
