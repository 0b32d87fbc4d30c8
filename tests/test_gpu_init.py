"""ggdmc_initialise (initialise_theta / initialise_phi, R/phi.R:141-332)
against the oracle's restatement, through the C ABI.

The GPU draws through CUDA's normcdfinv, the oracle through bisection and
Newton on erfc, so the same keyed uniforms give starts equal to ~1e-12.
"""
import numpy as np
import pytest

from ggdmc_gb300 import abi, gpu, synth

pytestmark = pytest.mark.gpu
TOL = dict(rtol=1e-10, atol=1e-12)


@pytest.fixture(scope="module", autouse=True)
def built():
    from ggdmc_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def work():
    return synth.hier_lba_32(n_subject=3, n=120)


def test_subjects_and_phi_match_oracle(oracle, work):
    w = work
    h = gpu.Handle(w.model, w.batch)
    (th, lp, ll), ph = h.initialise(w.p_prior, w.h_prior, nchain=9, max_attempts=50, seed=7)
    (oth, olp, oll), oph = oracle.initialise(w.model, w.batch, w.p_prior, w.h_prior, 9, 50, 7)
    np.testing.assert_allclose(th, oth, **TOL)
    np.testing.assert_allclose(lp, olp, **TOL)
    np.testing.assert_allclose(ll, oll, **TOL)
    for a, b in zip(ph, oph):
        np.testing.assert_allclose(a, b, **TOL)
    assert np.isfinite(ll).all() and np.isfinite(ph[2]).all()


def test_unbounded_prior_matches_oracle(oracle, work):
    # A ~ tnorm(0.2, 0.5) on (-inf, inf): draws on both sides of zero (the
    # LBA density's floors keep every log-likelihood finite, so none is
    # rejected, as in the reference)
    w = work
    p = w.p_prior.copy()
    ia = w.model.pnames.index("A")
    p[ia] = [0.2, 0.5, -np.inf, np.inf, 1.0, 1.0]
    h = gpu.Handle(w.model, w.batch)
    (th, lp, ll), _ = h.initialise(p, None, nchain=16, max_attempts=60, seed=3)
    (oth, olp, oll), _ = oracle.initialise(w.model, w.batch, p, None, 16, 60, 3)
    np.testing.assert_allclose(th, oth, **TOL)
    np.testing.assert_allclose(ll, oll, **TOL)
    assert (th[:, :, ia] < 0).any() and np.isfinite(ll).all()


def test_uniform_draws_cover_the_prior(work):
    w = work
    P = w.model.n_par
    p = synth.unif_prior(P, 0.0, 4.0)
    h = gpu.Handle(w.model, w.batch)
    (th, lp, _), _ = h.initialise(p, None, nchain=400, max_attempts=20, seed=11)
    np.testing.assert_allclose(lp, -P * np.log(4.0), rtol=1e-12)
    x = th.reshape(-1, P)
    assert (x >= 0).all() and (x <= 4).all()
    assert np.all(np.abs(x.mean(axis=0) - 2.0) <= 5 * 4 / np.sqrt(12 * len(x)))


def test_no_valid_start_is_an_error(oracle, work):
    # a zero-width truncated normal: its log density is -inf for every draw
    w = work
    p = w.p_prior.copy()
    ia = w.model.pnames.index("A")
    p[ia] = [0.3, 0.0, 0.0, np.inf, 1.0, 1.0]
    h = gpu.Handle(w.model, w.batch)
    with pytest.raises(gpu.GGDMCError, match="NUMERIC|no start"):
        h.initialise(p, None, nchain=4, max_attempts=3, seed=1)
    with pytest.raises(RuntimeError):
        oracle.initialise(w.model, w.batch, p, None, 4, 3, 1)
