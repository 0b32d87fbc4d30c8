"""ggdmc_logprior_noalloc: sumlogprior staged in a fixed device array.

The GPU test compares it with ggdmc_logprior (which allocates per call) on
the same inputs, twice in a row, so a stale or shared staging area would
show; the size limit is checked on the host before any device work.  This
file is collected last so the fixed array has seen the other tests' calls.
"""
import numpy as np
import pytest

from conftest import load_fixture
from ggdmc_gb300 import gpu, synth

TOL = dict(rtol=1e-12, atol=0.0)   # same kernel either way; FP64 sums


def _inputs(fx, n, seed):
    z, *_ = load_fixture(fx)
    table = z["sub_prior"]
    rng = np.random.default_rng(seed)
    base = z["sub_theta"].reshape(-1, table.shape[0])
    theta = base[rng.integers(0, base.shape[0], n)] * rng.uniform(0.5, 1.5, (n, table.shape[0]))
    theta[::7, 0] = -1.0          # below a lower bound: -inf rows
    return table, theta


@pytest.mark.gpu
@pytest.mark.parametrize("fx", [3, 6])
def test_noalloc_matches_allocating_entry_point(fx):
    from ggdmc_gb300 import build
    build.build()
    for n, seed in ((1, 0), (2000, 1), (513, 2)):
        table, theta = _inputs(fx, n, seed)
        want = gpu.logprior(table, theta)
        first = gpu.logprior_noalloc(table, theta)
        second = gpu.logprior_noalloc(table, theta)
        np.testing.assert_allclose(first, want, **TOL)
        np.testing.assert_allclose(second, want, **TOL)
        assert np.isneginf(first[::7]).all()


@pytest.mark.gpu
def test_noalloc_tnorm_and_uniform_rows():
    from ggdmc_gb300 import build
    build.build()
    P = 17
    table = np.concatenate([synth.tnorm_prior(np.linspace(0.1, 2.0, 9), 1.5),
                            synth.unif_prior(P - 9, 0.0, 5.0)])
    rng = np.random.default_rng(3)
    theta = rng.uniform(0.0, 4.0, (4096, P))
    want = gpu.logprior(table, theta)
    for _ in range(2):
        np.testing.assert_allclose(gpu.logprior_noalloc(table, theta), want, **TOL)


def test_noalloc_rejects_sizes_beyond_the_fixed_array():
    from ggdmc_gb300 import build
    build.build()
    P = 17
    table = synth.unif_prior(P)
    theta = np.ones((10000, P))          # 1.36 MB of theta alone
    with pytest.raises(gpu.GGDMCError, match="limit is 1048576 bytes"):
        gpu.logprior_noalloc(table, theta)
