"""The CPU oracle against the reference's own stored values (golden vectors).

The reference fixtures (tests/testthat/Group1/data/lba_data{0..6}.rda) hold
initial MCMC samples whose log-likelihoods and log priors were computed by
ggdmcLikelihood / ggdmcPrior.  These tests pin the oracle to them.
"""
import numpy as np
import pytest

from conftest import PINNED_LBA_FIXTURES, load_fixture


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


@pytest.mark.parametrize("fx", PINNED_LBA_FIXTURES)
def test_lba_single_subject_sums(oracle, fx):
    z, model, sub, _ = load_fixture(fx)
    got = oracle.loglik(model, sub, z["sub_theta"][None])[0]
    assert np.all(rel(got, z["sub_ll"]) <= 2e-9), rel(got, z["sub_ll"]).max()


@pytest.mark.parametrize("fx", PINNED_LBA_FIXTURES)
def test_lba_hierarchical_subject_sums(oracle, fx):
    z, model, _, pop = load_fixture(fx)
    S = pop.n_subject
    got = oracle.loglik(model, pop, z["subj_theta"][:S])
    r = rel(got, z["subj_ll"][:S])
    assert np.all(r <= 2e-9), (np.sum(r > 2e-9), r.max())


def test_floor_chains_give_n_log_1e10(oracle):
    # chains whose t0 exceeds every RT store exactly N log(1e-10)
    z, model, sub, _ = load_fixture(6)
    N = len(sub.rt)
    floor = np.isclose(z["sub_ll"], N * np.log(1e-10), rtol=1e-10, atol=0)
    assert floor.sum() > 0
    got = oracle.loglik(model, sub, z["sub_theta"][floor][None])[0]
    assert np.allclose(got, z["sub_ll"][floor], rtol=1e-10)


@pytest.mark.parametrize("fx", range(7))
def test_subject_priors(oracle, fx):
    z, *_ = load_fixture(fx)
    assert np.all(rel(oracle.logprior(z["sub_prior"], z["sub_theta"]), z["sub_lp"]) < 1e-12)
    for s in range(z["subj_theta"].shape[0]):
        got = oracle.logprior(z["pop_p_prior"], z["subj_theta"][s])
        assert np.all(rel(got, z["subj_lp"][s]) < 1e-12)


@pytest.mark.parametrize("fx", range(7))
def test_hyper_loglik_and_prior(oracle, fx):
    z, *_ = load_fixture(fx)
    got = oracle.loghlike(z["pop_p_prior"], z["phi_theta"], z["subj_theta"])
    assert np.all(rel(got, z["phi_ll"]) < 1e-12)
    assert np.all(rel(oracle.logprior(z["pop_h_prior"], z["phi_theta"]), z["phi_lp"]) < 1e-12)


def test_nonpositive_product_uses_dbl_epsilon(oracle):
    # A loser survivor that cancels to <= 0 gives DBL_EPSILON (R/phi.R:3-13);
    # fixture 6 has such pairs (differences of exactly log(eps/1e-10)).
    z, model, _, pop = load_fixture(6)
    s, per = oracle.sumloglike(model, pop.subject(0).rt, pop.subject(0).cell,
                               z["subj_theta"][0][0], per_trial=True)
    assert np.isfinite(s) and per.shape == pop.subject(0).rt.shape
    eps = np.finfo(float).eps
    cv = np.zeros((2, 6))
    cv[:, 0] = 0.3; cv[:, 1] = 1.0; cv[:, 2] = [3.0, 40.0]; cv[:, 3] = [1.0, 0.05]
    # the loser (v/s = 800) is certain to have finished: survivor cancels to <= 0
    import ctypes as C
    arr = (C.c_double * 12)(*cv.ravel())
    d = oracle.lib().oracle_lba_dens(2.0, arr, 2, 0)
    assert d == eps
