"""ggdmc_rebuild_posterior against a restatement of RebuildPosterior
(R/parallel_helper.R:62-83) that follows R's column-major operations step by
step: .GetParamArray re-dimensions each fit's theta [npar, nchain, nmc] to
[npar, nchain * nmc] (:15-55) and .get_likelihood_matrix stacks
as.vector(t(m)) of each fit's [nchain, nmc] matrix (:1-12).  Host code only.
"""
import numpy as np
import pytest

from ggdmc_gb300 import gpu


def r_rebuild(fits):
    """fits in R's layout: theta [npar, nchain, nmc], lp, ll [nchain, nmc]."""
    npar, nchain, nmc = fits[0][0].shape
    theta = np.empty((npar, len(fits), nchain * nmc))
    for i, (th, _, _) in enumerate(fits):
        theta[:, i, :] = th.reshape((npar, nchain * nmc), order="F")      # dim<- keeps R's order
    lp = np.stack([f[1].T.reshape(-1, order="F") for f in fits])          # rbind(as.vector(t(m)))
    ll = np.stack([f[2].T.reshape(-1, order="F") for f in fits])
    return theta, lp, ll


def as_r(theta, lp, ll):
    """C-ABI arrays [nmc][nchain][npar], [nmc][nchain] -> R's dimensions."""
    return theta.transpose(2, 1, 0), lp.T, ll.T


@pytest.mark.parametrize("F,nmc,C,P", [(4, 7, 3, 5), (1, 1, 1, 1), (3, 2, 9, 1)])
def test_merge_matches_r_layout(F, nmc, C, P):
    rng = np.random.default_rng(F * 100 + nmc)
    fits = [(rng.normal(size=(nmc, C, P)), rng.normal(size=(nmc, C)), rng.normal(size=(nmc, C)))
            for _ in range(F)]
    th, lp, ll = gpu.rebuild_posterior(fits)
    rt, rlp, rll = r_rebuild([as_r(*f) for f in fits])
    # ours [nmc'][F][P] and [nmc'][F] are R's [P, F, nmc'] and [F, nmc']
    np.testing.assert_array_equal(th.transpose(2, 1, 0), rt)
    np.testing.assert_array_equal(lp.T, rlp)
    np.testing.assert_array_equal(ll.T, rll)
    # theta sample j = m * C + c; lp sample j = c * nmc + m (the reference's two orders)
    m, c = nmc - 1, C - 1
    np.testing.assert_array_equal(th[m * C + c, F - 1], fits[F - 1][0][m, c])
    assert lp[c * nmc + m, F - 1] == fits[F - 1][1][m, c]


def test_merged_posterior_per_subject_and_errors():
    rng = np.random.default_rng(3)
    runs = [{"subj_s": (rng.normal(size=(2, 5, 4, 3)), rng.normal(size=(2, 5, 4)),
                        rng.normal(size=(2, 5, 4)))} for _ in range(3)]
    per = gpu.rebuild_posteriors(runs)
    assert len(per) == 2
    for s, (th, lp, ll) in enumerate(per):
        ref = r_rebuild([as_r(*(x[s] for x in r["subj_s"])) for r in runs])
        np.testing.assert_array_equal(th.transpose(2, 1, 0), ref[0])
        np.testing.assert_array_equal(ll.T, ref[2])
    with pytest.raises(ValueError):
        gpu.rebuild_posterior([(np.zeros((2, 3, 4)), np.zeros((2, 3)), np.zeros((2, 3))),
                               (np.zeros((2, 2, 4)), np.zeros((2, 2)), np.zeros((2, 2)))])
