"""Brooks-Gelman PSRF and summaries of ggdmc_gb300.diagnostics (CPU)."""
import numpy as np
import pytest

pytest.importorskip("scipy")
from ggdmc_gb300 import diagnostics  # noqa: E402


def test_psrf_near_one_for_exchangeable_chains():
    rng = np.random.default_rng(0)
    th = rng.standard_normal((2000, 8, 3)) * [1.0, 2.0, 0.5] + [0.0, 5.0, -1.0]
    g = diagnostics.gelman(th, form="coda")
    assert np.all(np.abs(g["psrf"][:, 0] - 1) < 0.01)
    assert np.all(g["psrf"][:, 1] >= g["psrf"][:, 0])
    assert abs(g["mpsrf"] - 1) < 0.02
    # the reference's form differs only in df_adj: same R2 estimate underneath
    r = diagnostics.gelman(th)
    assert np.all(r["psrf"][:, 0] >= 1.0) and r["mpsrf"] == g["mpsrf"]


def test_psrf_flags_separated_chains():
    rng = np.random.default_rng(1)
    th = rng.standard_normal((500, 6, 2))
    th[:, :3, 0] += 3.0                       # half the chains elsewhere in parameter 0
    g = diagnostics.gelman(th)
    assert g["psrf"][0, 0] > 1.5 and abs(g["psrf"][1, 0] - 1) < 0.05
    assert g["mpsrf"] > 1.5


def test_psrf_point_estimate_formula():
    # the point estimate sqrt(df_adj * ((n-1)/n + (1+1/m) B/(n W))) by hand, one parameter
    rng = np.random.default_rng(2)
    th = rng.standard_normal((300, 5, 1)) + rng.standard_normal((1, 5, 1)) * 0.2
    n, m = 300, 5
    x = th[:, :, 0]
    w = x.var(axis=0, ddof=1).mean()
    b = n * x.mean(axis=0).var(ddof=1)
    g = diagnostics.gelman(th, multivariate=False, form="coda")
    r2 = (n - 1) / n + (1 + 1 / m) * b / (n * w)
    # df_adj lies in (1, 3]; the point estimate must lie between sqrt(r2) and sqrt(3 r2)
    assert np.sqrt(r2) <= g["psrf"][0, 0] <= np.sqrt(3 * r2)
    # the reference's form is undefined for one parameter (R's var of one value is NA)
    assert np.isnan(diagnostics.gelman(th, multivariate=False)["psrf"][0, 0])


def test_summary_shapes_and_values():
    rng = np.random.default_rng(3)
    th = rng.normal(2.0, 0.5, (4000, 10, 2))
    s = diagnostics.summary(th, probs=(0.025, 0.25, 0.5, 0.75, 0.975))
    assert s["quantiles"].shape == (5, 2)
    np.testing.assert_allclose(s["mean"], 2.0, atol=0.01)
    np.testing.assert_allclose(s["sd"], 0.5, atol=0.01)
    np.testing.assert_allclose(s["quantiles"][2], 2.0, atol=0.02)
    assert np.all(s["se_mean"] < 0.01)


def test_rejects_two_chains():
    with pytest.raises(ValueError):
        diagnostics.gelman(np.zeros((10, 2, 1)))


def ar1(rng, n, phi, sigma=1.0):
    e = rng.standard_normal(n) * sigma
    x = np.zeros(n)
    for i in range(1, n):
        x[i] = phi * x[i - 1] + e[i]
    return x


def test_spectrum0_ar_of_ar1_chains():
    # an AR(1) chain x_t = phi x_{t-1} + e_t has spectral density at zero
    # sigma^2 / (1 - phi)^2; the Yule-Walker fit finds it within sampling error
    rng = np.random.default_rng(4)
    for phi in (0.0, 0.5, 0.8):
        x = ar1(rng, 20000, phi)
        spec, order = diagnostics.spectrum0_ar(x)
        assert abs(spec / (1.0 / (1 - phi) ** 2) - 1) < 0.15, (phi, spec, order)
    # a constant chain or a straight line: residual sd 0 -> spectrum 0
    assert diagnostics.spectrum0_ar(np.full(300, 0.7)) == (0.0, 0)
    assert diagnostics.spectrum0_ar(2.0 + 0.01 * np.arange(300.0)) == (0.0, 0)


def test_summary_se_formulas():
    rng = np.random.default_rng(5)
    th = np.stack([np.stack([ar1(rng, 3000, 0.6) + k for k in range(2)], axis=1) for _ in range(4)], axis=1)
    s = diagnostics.summary(th)
    niter, nchain = 3000, 4
    flat = th.reshape(-1, 2)
    np.testing.assert_allclose(s["naive_se"], np.sqrt(flat.var(axis=0, ddof=1) / niter * nchain), rtol=1e-12)
    spec = np.array([[diagnostics.spectrum0_ar(th[:, k, p])[0] for p in range(2)] for k in range(nchain)])
    np.testing.assert_allclose(s["ts_se"], np.sqrt(spec.mean(axis=0) / niter * nchain), rtol=1e-12)
    # autocorrelated chains: the time-series SE exceeds the naive one by about 1 / (1 - 0.6)
    assert np.all(s["ts_se"] / s["naive_se"] > 1.7)
    np.testing.assert_array_equal(s["probs"], [0.05, 0.5, 0.975])   # the reference's default


def test_quantile7_matches_r_type7():
    rng = np.random.default_rng(6)
    for n in (1, 2, 7, 1000):
        x = rng.normal(size=n)
        probs = [0.0, 0.05, 0.5, 0.975, 1.0]
        np.testing.assert_allclose(diagnostics.quantile7(x, probs), np.quantile(x, probs), rtol=1e-14, atol=1e-15)
    x = np.array([1.0, 1.0, 1.0, 2.0])
    assert diagnostics.quantile7(x, [0.5])[0] == 1.0                  # equal order statistics
