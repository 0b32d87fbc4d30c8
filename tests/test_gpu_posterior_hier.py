"""Posterior summaries of the mixed-precision sampler against the FP64 one in
a hierarchical fit, within Monte-Carlo error (GPU, through the C ABI).

Setup: 6 subjects of the 17-parameter 4-accumulator design of the benchmark
workload (N_s ~ U{150..300}), the population level with 34 parameters and 51
chains, started near the generating values. R independent runs (their own
draw seeds and start states, 3000 iterations kept every second) in FP64 and
R in mixed precision.

For each population parameter, after burn-in, the replicate means and 2.5% /
97.5% quantiles of the two precisions are compared by Welch's t statistic
(the standard error estimated from the replicates' spread), against the
t quantile of a family-wise level of 0.001 over the 102 comparisons
(Bonferroni); every run's population chains must be converged
(Brooks-Gelman PSRF, coda form, <= 1.2).
"""
import numpy as np
import pytest

from ggdmc_gb300 import abi, diagnostics, gpu, synth

pytestmark = pytest.mark.gpu
pytest.importorskip("scipy")

R, NMC, THIN, BURN = 8, 1500, 2, 500


@pytest.fixture(scope="module", autouse=True)
def built():
    from ggdmc_gb300 import build
    build.build()


def replicate_runs(precision, seed0):
    w = synth.uneven_lba_256(seed=3, n_subject=6, n_lo=150, n_hi=300)
    h = gpu.Handle(w.model, w.batch)
    S, P = w.batch.n_subject, w.model.n_par
    out = []
    for r in range(R):
        th, phi = synth.start_states(w, w.nchain, np.random.default_rng(seed0 + r))
        lp = np.stack([gpu.logprior(w.p_prior, th[s]) for s in range(S)])
        ll = h.loglik(th, abi.FP64)
        plp = gpu.logprior(w.h_prior, phi)
        pll = gpu.loghlike(w.p_prior, phi, th)
        cfg = abi.DEConfigPy(nchain=w.nchain, nparameter=2 * P, nmc=NMC, thin=THIN,
                             pop_migration_prob=0.05, sub_migration_prob=0.06,
                             precision=precision, seed=seed0 + r)
        o = h.run(cfg, w.p_prior, th, lp, ll, h_table=w.h_prior, phi=(phi, plp, pll))
        out.append(o["phi_s"][0])                      # [NMC][C][2P]
    return out


@pytest.fixture(scope="module")
def runs():
    return {"fp64": replicate_runs(abi.FP64, 100), "mixed": replicate_runs(abi.MIXED, 200)}


def test_population_chains_converged(runs):
    for name, reps in runs.items():
        for smp in reps:
            g = diagnostics.gelman(smp, start=BURN, form="coda", multivariate=False)
            assert np.all(g["psrf"][:, 0] <= 1.2), (name, g["psrf"][:, 0].max())


def test_population_summaries_within_mc_error(runs):
    from scipy.stats import t as tdist

    def stats(smp):
        x = smp[BURN:].reshape(-1, smp.shape[-1])
        return np.stack([x.mean(0), np.quantile(x, 0.025, axis=0), np.quantile(x, 0.975, axis=0)])

    a = np.stack([stats(s) for s in runs["fp64"]])      # [R][3][2P]
    b = np.stack([stats(s) for s in runs["mixed"]])
    va, vb = a.var(0, ddof=1) / R, b.var(0, ddof=1) / R
    se = np.sqrt(va + vb)
    tval = np.abs(b.mean(0) - a.mean(0)) / np.maximum(se, 1e-12 * np.abs(a.mean(0)) + 1e-300)
    df = (va + vb) ** 2 / (va ** 2 / (R - 1) + vb ** 2 / (R - 1) + 1e-300)   # Welch-Satterthwaite
    crit = tdist.ppf(1 - 0.001 / (2 * tval.size), np.maximum(df, 1.0))
    assert np.all(tval <= crit), (tval.max(), np.unravel_index((tval / crit).argmax(), tval.shape))
    # and most comparisons well inside the usual range
    assert np.mean(tval <= 3.0) >= 0.95
