"""The autotuner's key and cache (ggdmc_tune_key / _lookup / _store): host
code, no GPU.  The key names the model type, accumulators, free parameters,
chains, the level layout and the histogram of subjects' trial counts in
powers of two, so that data sets of the same shape share tuned settings."""
import os

import numpy as np
import pytest

from ggdmc_gb300 import gpu, synth
from ggdmc_gb300.dmi import SubjectBatch


def batch_of(counts, seed=0):
    rng = np.random.default_rng(seed)
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    n = int(offs[-1])
    return SubjectBatch(rng.uniform(0.3, 1.5, n), rng.integers(0, 4, n).astype(np.int32), offs)


@pytest.fixture(scope="module")
def model():
    from ggdmc_gb300 import build
    build.build()
    return synth.uneven_lba_256().model


def test_key_names_the_shape(model):
    k = gpu.tune_key(model, batch_of([1000] * 8), 51, True)
    assert k.startswith("lba4.p17.c51.h.s3.")
    # trial counts in the same power-of-two bins, subject counts in the same bins: one key
    assert gpu.tune_key(model, batch_of([1010, 990, 1020, 1001, 1000, 1003, 1015, 999], 1), 51, True) == k
    # another chain count, level layout, bin or subject count: another key
    assert gpu.tune_key(model, batch_of([1000] * 8), 39, True) != k
    assert gpu.tune_key(model, batch_of([1000] * 8), 51, False) != k
    assert gpu.tune_key(model, batch_of([3000] * 8), 51, True) != k
    assert gpu.tune_key(model, batch_of([1000] * 16), 51, True) != k
    assert gpu.tune_key(model, batch_of([100, 2000] * 4), 51, True) != k


def test_cache_in_process_and_file(model, tmp_path):
    key = gpu.tune_key(model, batch_of([700] * 3), 26, False)
    assert gpu.tune_lookup(key) is None
    t = dict(spec_group=4, graph_iters=16, mig_round=3, lik_variant=2, sweep_ms=0.5)
    gpu.tune_store(key, t)
    assert gpu.tune_lookup(key) == t                       # process cache
    path = str(tmp_path / "tune.txt")
    # a key only in the file (another process stored it): the last line wins
    k2 = key + ".other"
    with open(path, "w") as f:
        f.write(f"{k2} 1 8 4 1 0.9\n")
        f.write(f"{k2} 2 4 6 2 0.7\n")
    assert gpu.tune_lookup(k2) is None
    got = gpu.tune_lookup(k2, path)
    assert got == dict(spec_group=2, graph_iters=4, mig_round=6, lik_variant=2, sweep_ms=0.7)
    assert gpu.tune_lookup(k2) == got                      # now in the process cache too
    # storing with a path appends a line another process can read
    k3 = key + ".third"
    gpu.tune_store(k3, t, path)
    with open(path) as f:
        assert f.read().splitlines()[-1].split()[:5] == [k3, "4", "16", "3", "2"]


def test_key_errors(model):
    from ggdmc_gb300 import abi
    import ctypes as C
    m = abi.Marshal()
    buf = C.create_string_buffer(8)
    st = gpu.lib().ggdmc_tune_key(C.byref(m.model(model)), C.byref(m.data(batch_of([10, 20]))), 3, 0, buf, 8)
    assert st == abi.GGDMC_ERR_ARG                          # buffer too small
    with pytest.raises(gpu.GGDMCError):
        gpu.tune_store("has space", dict(spec_group=1, graph_iters=1, mig_round=1, lik_variant=1, sweep_ms=0))
