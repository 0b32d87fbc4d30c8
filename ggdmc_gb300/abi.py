"""ctypes mirror of include/ggdmc_gpu.h and marshalling of numpy arrays into it.

Only plain C types cross the boundary: the same structs an R ``.Call`` shim
fills from S4 slots.  The helpers here keep the numpy buffers alive for as long
as the struct that points into them (``Marshal`` owns both).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

GGDMC_OK, GGDMC_ERR_ARG, GGDMC_ERR_CUDA, GGDMC_ERR_TIMEOUT, GGDMC_ERR_NUMERIC, \
    GGDMC_ERR_NOMEM = range(6)
STATUS_NAMES = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_TIMEOUT",
                4: "ERR_NUMERIC", 5: "ERR_NOMEM"}

MODEL_LBA, MODEL_DDM = 0, 1
FP64, MIXED, FP64_PLAIN, MIXED_SUMS = 0, 1, 2, 3
PRIOR_TNORM, PRIOR_UNIF = 1, 6
FLAG_L2_FLUSH = 1

_dp = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)


class Model(C.Structure):
    _fields_ = [("model_type", C.c_int32), ("n_par", C.c_int32), ("n_cell", C.c_int32),
                ("n_acc", C.c_int32), ("n_kind", C.c_int32), ("n_const", C.c_int32),
                ("param_src", _i32p), ("resp", _i32p), ("constants", _dp)]


class Data(C.Structure):
    _fields_ = [("n_subject", C.c_int32), ("offsets", _i64p), ("rt", _dp), ("cell", _i32p)]


class Prior(C.Structure):
    _fields_ = [("n_par", C.c_int32), ("table", _dp)]


class DEConfig(C.Structure):
    _fields_ = [("pop_migration_prob", C.c_double), ("sub_migration_prob", C.c_double),
                ("gamma_precursor", C.c_double), ("rp", C.c_double),
                ("is_hblocked", C.c_int32), ("is_pblocked", C.c_int32),
                ("nparameter", C.c_int32), ("nchain", C.c_int32),
                ("nmc", C.c_int32), ("thin", C.c_int32),
                ("precision", C.c_int32), ("flags", C.c_int32), ("seed", C.c_uint64)]


class ChainState(C.Structure):
    _fields_ = [("theta", _dp), ("lp", _dp), ("ll", _dp)]


class Samples(C.Structure):
    _fields_ = [("theta", _dp), ("lp", _dp), ("ll", _dp)]


class Diag(C.Structure):
    _fields_ = [("mean", _dp), ("sd", _dp), ("naive_se", _dp), ("ts_se", _dp), ("quantiles", _dp),
                ("psrf", _dp)]


PSRF_REFERENCE, PSRF_CODA = 0, 1


class Tuning(C.Structure):
    _fields_ = [("spec_group", C.c_int32), ("graph_iters", C.c_int32), ("mig_round", C.c_int32),
                ("lik_variant", C.c_int32), ("sweep_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class RunStats(C.Structure):
    _fields_ = [("proposals", C.c_int64), ("accepts", C.c_int64), ("migrations", C.c_int64),
                ("reevaluations", C.c_int64), ("kernel_launches", C.c_int64),
                ("trial_evals", C.c_int64), ("iterations", C.c_int64), ("sweep_ms", C.c_double),
                ("resolve_rounds", C.c_int64), ("variants", C.c_int64), ("fallbacks", C.c_int64),
                ("setup_ms", C.c_double), ("capture_ms", C.c_double), ("run_ms", C.c_double),
                ("copyout_ms", C.c_double)]


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def i32ptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_i32p)


def i64ptr(a: np.ndarray):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(_i64p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class Marshal:
    """Owns numpy buffers and the ctypes structs pointing into them."""

    def __init__(self):
        self._keep = []

    def keep(self, *arrs):
        self._keep.extend(arrs)
        return arrs[0] if len(arrs) == 1 else arrs

    def model(self, fm) -> Model:
        src = self.keep(_c(fm.param_src, np.int32))
        resp = self.keep(_c(fm.resp, np.int32))
        consts = self.keep(_c(fm.constants if len(fm.constants) else np.zeros(1), np.float64))
        return Model(fm.model_type, fm.n_par, fm.n_cell, fm.n_acc, src.shape[2],
                     len(fm.constants), i32ptr(src), i32ptr(resp), dptr(consts))

    def data(self, batch) -> Data:
        offs = self.keep(_c(batch.offsets, np.int64))
        rt = self.keep(_c(batch.rt if len(batch.rt) else np.zeros(1), np.float64))
        cell = self.keep(_c(batch.cell if len(batch.cell) else np.zeros(1), np.int32))
        return Data(len(offs) - 1, i64ptr(offs), dptr(rt), i32ptr(cell))

    def prior(self, table) -> Prior:
        t = self.keep(_c(table, np.float64))
        return Prior(t.shape[0], dptr(t))

    def states(self, theta, lp, ll):
        """theta [L][C][P], lp/ll [L][C] (copied; returns the arrays to read back)."""
        theta = self.keep(np.array(theta, dtype=np.float64, order="C", copy=True))
        lp = self.keep(np.array(lp, dtype=np.float64, order="C", copy=True))
        ll = self.keep(np.array(ll, dtype=np.float64, order="C", copy=True))
        arr = self.ptr_table(ChainState, theta, lp, ll)
        return arr, theta, lp, ll

    def samples(self, n_level, nmc, nchain, npar):
        # not pre-filled: a run that returns OK writes every slot (slot 0 is the
        # start state), and a failed run raises before they are read
        theta = self.keep(np.empty((n_level, nmc, nchain, npar)))
        lp = self.keep(np.empty((n_level, nmc, nchain)))
        ll = self.keep(np.empty((n_level, nmc, nchain)))
        arr = self.ptr_table(Samples, theta, lp, ll)
        return arr, theta, lp, ll

    def ptr_table(self, struct, *arrs):
        """An array of `struct` (all of whose fields are double pointers),
        entry i pointing at arrs[k][i]; built in one numpy pass."""
        n = arrs[0].shape[0]
        tab = np.empty((n, len(arrs)), dtype=np.uintp)
        idx = np.arange(n, dtype=np.uintp)
        for k, a in enumerate(arrs):
            tab[:, k] = np.uintp(a.ctypes.data) + idx * np.uintp(a.strides[0])
        self.keep(tab)
        return (struct * n).from_buffer(tab)


@dataclass
class DEConfigPy:
    """de_input + theta_input fields as Python values (R/model-class.R:1288-1313)."""
    nchain: int
    nparameter: int
    nmc: int = 2
    thin: int = 1
    pop_migration_prob: float = 0.0
    sub_migration_prob: float = 0.0
    gamma_precursor: float = 2.38
    rp: float = 0.001
    is_hblocked: bool = False
    is_pblocked: bool = False
    precision: int = FP64
    seed: int = 0
    flags: int = 0

    def to_c(self) -> DEConfig:
        return DEConfig(self.pop_migration_prob, self.sub_migration_prob, self.gamma_precursor,
                        self.rp, int(self.is_hblocked), int(self.is_pblocked),
                        self.nparameter, self.nchain, self.nmc, self.thin,
                        self.precision, self.flags, self.seed & 0xFFFFFFFFFFFFFFFF)


def draw_slots(nchain: int, nparameter: int) -> int:
    return 2 + nchain + nchain * (nparameter + 3)


def draw_layout(cfg: DEConfigPy, n_level: int, hierarchical: bool):
    """(n_iter, n_pass, n_slot): the canonical keyed draw extents."""
    if hierarchical:
        a = cfg.nparameter if cfg.is_hblocked else 1
        b = cfg.nparameter // 2 if cfg.is_pblocked else 1
        n_pass = max(a, b)
    else:
        n_pass = cfg.nparameter if cfg.is_pblocked else 1
    return (cfg.nmc - 1) * cfg.thin, n_pass, draw_slots(cfg.nchain, cfg.nparameter)
