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
    s = diagnostics.summary(th)
    assert s["quantiles"].shape == (5, 2)
    np.testing.assert_allclose(s["mean"], 2.0, atol=0.01)
    np.testing.assert_allclose(s["sd"], 0.5, atol=0.01)
    np.testing.assert_allclose(s["quantiles"][2], 2.0, atol=0.02)
    assert np.all(s["se_mean"] < 0.01)


def test_rejects_two_chains():
    with pytest.raises(ValueError):
        diagnostics.gelman(np.zeros((10, 2, 1)))
