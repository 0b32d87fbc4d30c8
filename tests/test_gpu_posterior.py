"""Posterior summaries of the mixed-precision sampler against the FP64 one,
within Monte-Carlo error (GPU, through the C ABI).

Both samplers run the reference's DE-MCMC on the same subject (fixture
lba_data6, 13 parameters, U(0, 10) priors, 39 chains) from the same
start, with different draw streams. After burn-in:

* each run is converged (Brooks-Gelman PSRF, coda form, <= 1.2 per parameter);
* the two runs pooled are indistinguishable (PSRF over all 78 chains <= 1.1);
* posterior means agree within 5 Monte-Carlo standard errors;
* 2.5% and 97.5% quantiles agree within 15% of the 95% interval width.
"""
import numpy as np
import pytest

from conftest import load_fixture
from ggdmc_gb300 import abi, diagnostics, gpu

pytestmark = pytest.mark.gpu
pytest.importorskip("scipy")

NMC, BURN, C = 700, 200, 39


@pytest.fixture(scope="module", autouse=True)
def built():
    from ggdmc_gb300 import build
    build.build()


def run(precision, seed):
    z, model, sub, _ = load_fixture(6)
    idx = np.argsort(z["sub_ll"])[::-1][:C]
    th, lp, ll = z["sub_theta"][idx].copy(), z["sub_lp"][idx].copy(), z["sub_ll"][idx].copy()
    cfg = abi.DEConfigPy(nchain=C, nparameter=model.n_par, nmc=NMC, thin=1,
                         sub_migration_prob=0.06, precision=precision, seed=seed)
    out = gpu.run_subjects(cfg, model, sub, z["sub_prior"], th[None], lp[None], ll[None])
    return out["s_theta"][0]                  # [nmc][C][P]


@pytest.fixture(scope="module")
def chains():
    return run(abi.FP64, 101), run(abi.MIXED, 202)


def test_each_run_converged(chains):
    for th in chains:
        g = diagnostics.gelman(th, start=BURN, form="coda")
        assert np.all(g["psrf"][:, 0] <= 1.2), g["psrf"][:, 0]


def test_pooled_runs_indistinguishable(chains):
    pooled = np.concatenate(chains, axis=1)
    g = diagnostics.gelman(pooled, start=BURN, form="coda")
    assert np.all(g["psrf"][:, 0] <= 1.1), g["psrf"][:, 0]


def test_means_and_quantiles_within_mc_error(chains):
    a, b = (diagnostics.summary(th, start=BURN) for th in chains)
    se = np.sqrt(a["se_mean"] ** 2 + b["se_mean"] ** 2)
    assert np.all(np.abs(a["mean"] - b["mean"]) <= 5 * se), (a["mean"] - b["mean"]) / se
    width = a["quantiles"][-1] - a["quantiles"][0]
    for q in (0, -1):
        assert np.all(np.abs(a["quantiles"][q] - b["quantiles"][q]) <= 0.15 * width)
