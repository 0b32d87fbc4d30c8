"""Posterior summaries of the mixed-precision sampler against the FP64 one,
within Monte-Carlo error (GPU, through the C ABI).

DE-MCMC chains are coupled through crossover, so the Monte-Carlo error of a
run is measured across independent replicate runs. Setup:

* The subject of fixture lba_data6 (13 parameters, U(0, 10) priors, 39
  chains) is fitted R times in one `ggdmc_run_subjects` call. Each fit keys
  its own draws, so the fits are independent replicates.
* This is done once in FP64 and once in mixed precision.

For each parameter, after burn-in, the replicate means, 2.5% and 97.5%
quantiles of the two precisions must agree within 4.5 standard errors of
their difference, with the standard error estimated from the replicates'
spread. Every run must also be converged: Brooks-Gelman PSRF, coda form,
<= 1.2.
"""
import numpy as np
import pytest

from conftest import load_fixture
from ggdmc_gb300 import abi, diagnostics, gpu
from ggdmc_gb300.dmi import SubjectBatch

pytestmark = pytest.mark.gpu
pytest.importorskip("scipy")

R, NMC, THIN, BURN, C = 8, 1000, 2, 250, 39


@pytest.fixture(scope="module", autouse=True)
def built():
    from ggdmc_gb300 import build
    build.build()


def replicate_runs(precision, seed):
    z, model, sub, _ = load_fixture(6)
    idx = np.argsort(z["sub_ll"])[::-1][:C]
    th, lp, ll = z["sub_theta"][idx], z["sub_lp"][idx], z["sub_ll"][idx]
    batch = SubjectBatch.pack([sub.subject(0)] * R)
    cfg = abi.DEConfigPy(nchain=C, nparameter=model.n_par, nmc=NMC, thin=THIN,
                         sub_migration_prob=0.06, precision=precision, seed=seed)
    out = gpu.run_subjects(cfg, model, batch, z["sub_prior"], np.repeat(th[None], R, 0),
                           np.repeat(lp[None], R, 0), np.repeat(ll[None], R, 0))
    return out["s_theta"]                     # [R][nmc][C][P]


@pytest.fixture(scope="module")
def runs():
    return replicate_runs(abi.FP64, 101), replicate_runs(abi.MIXED, 202)


def test_every_replicate_converged(runs):
    for rep in runs:
        for th in rep:
            g = diagnostics.gelman(th, start=BURN, form="coda")
            assert np.all(g["psrf"][:, 0] <= 1.2), g["psrf"][:, 0]


def test_summaries_within_mc_error(runs):
    stats = []
    for rep in runs:
        s = [diagnostics.summary(th, start=BURN) for th in rep]
        stats.append({k: np.stack([x[k] for x in s]) for k in ("mean", "quantiles")})
    a, b = stats
    for key, pick in (("mean", lambda v: v), ("q025", lambda v: v[:, 0]), ("q975", lambda v: v[:, -1])):
        va = pick(a["mean" if key == "mean" else "quantiles"])
        vb = pick(b["mean" if key == "mean" else "quantiles"])
        se = np.sqrt(va.var(axis=0, ddof=1) / R + vb.var(axis=0, ddof=1) / R)
        zstat = np.abs(va.mean(axis=0) - vb.mean(axis=0)) / se
        assert np.all(zstat <= 4.5), (key, zstat)
