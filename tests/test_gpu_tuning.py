"""Launch settings and the autotuner on the GPU: every setting the tuner
chooses between (the likelihood kernel variant, the speculative group size,
the migration steps per resolve round, the iterations per graph) gives the
same chains bit for bit, and a tuned handle runs exactly as an untuned one."""
import numpy as np
import pytest

from ggdmc_gb300 import abi, gpu, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    from ggdmc_gb300 import build
    build.build()
    # the 4-accumulator design (both likelihood kernel variants apply)
    w = synth.uneven_lba_256(n_subject=12, n_lo=100, n_hi=600)
    h = gpu.Handle(w.model, w.batch)
    th, phi = synth.start_states(w, w.nchain, np.random.default_rng(21))
    S = w.batch.n_subject
    lp = np.stack([gpu.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = h.loglik(th, abi.FP64)
    plp = gpu.logprior(w.h_prior, phi)
    pll = gpu.loghlike(w.p_prior, phi, th)
    return w, h, (th, lp, ll), (phi, plp, pll)


def run(case, precision, tuning=None, nmc=8):
    w, h, subj, phi = case
    cfg = abi.DEConfigPy(nchain=w.nchain, nparameter=2 * w.model.n_par, nmc=nmc, thin=1,
                         pop_migration_prob=0.2, sub_migration_prob=0.3, precision=precision, seed=17)
    h.set_tuning(tuning)
    out = h.run(cfg, w.p_prior, *subj, h_table=w.h_prior, phi=phi)
    h.set_tuning(None)
    return out


def same(a, b):
    for k in ("theta", "lp", "ll", "s_theta", "s_lp", "s_ll"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["phi_s"][0], b["phi_s"][0])
    # (the work done, trial_evals, depends on the migration steps per round)
    for k in ("accepts", "migrations", "proposals"):
        assert a["stats"][k] == b["stats"][k], k


@pytest.mark.parametrize("precision", [abi.MIXED, abi.FP64])
@pytest.mark.parametrize("setting", [dict(lik_variant=2), dict(spec_group=1), dict(spec_group=4),
                                     dict(mig_round=3), dict(mig_round=8), dict(graph_iters=3),
                                     dict(graph_iters=16)])
def test_settings_do_not_change_results(case, precision, setting):
    base = run(case, precision)
    assert base["stats"]["migrations"] > 0
    same(run(case, precision, setting), base)


def test_autotune_caches_and_keeps_results(case, tmp_path):
    w, h, subj, phi = case
    cfg = abi.DEConfigPy(nchain=w.nchain, nparameter=2 * w.model.n_par, nmc=8, thin=1,
                         pop_migration_prob=0.2, sub_migration_prob=0.3, precision=abi.MIXED, seed=17)
    base = run(case, abi.MIXED)
    path = str(tmp_path / "tune.txt")
    t = h.autotune(cfg, w.p_prior, *subj, h_table=w.h_prior, phi=phi, n_probe=3, cache_path=path)
    assert t["sweep_ms"] > 0 and t["spec_group"] in (0, 1, 2, 4)
    key = gpu.tune_key(w.model, w.batch, w.nchain, True)
    assert gpu.tune_lookup(key, path)["sweep_ms"] == t["sweep_ms"]
    # the tuned handle's run (settings kept by the handle) equals the untuned one
    out = h.run(cfg, w.p_prior, *subj, h_table=w.h_prior, phi=phi)
    same(out, base)
    # a second call finds the key cached and does not probe again
    assert h.autotune(cfg, w.p_prior, *subj, h_table=w.h_prior, phi=phi, n_probe=3) == t
    h.set_tuning(None)
