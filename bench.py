"""Benchmark of the DE-MCMC hot path on one GB300.

Workload: the uneven 256-subject hierarchical LBA (N_s ~ U{100..2000}, the
17-parameter 4-accumulator design, 51 chains, theta ~ tnorm(pop, 10% CV)).
A step is one DE sweep: the phi level and every subject, all chains
(src/de.cpp:272-383).  Metric: DE sweeps/s (with trial-logL evals/s beside
it), batched mixed precision, exact reference chain order.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--no-cpu] [--profile]

--impl reference times the reference's algorithm on the host cores: the
CPU restatement in oracle/ (the reference itself needs R and packages that
are not installable here), one replica per host thread, as the reference's
own parallelism runs independent instances (R/sampling.R:13-121).
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from ggdmc_gb300 import abi, synth  # noqa: E402

WORKLOAD = "uneven_lba_256"
E2E_MAX_STEPS = 500                      # samples of every chain come back: 2.1 MB per sweep
PROFILE = os.path.join(ROOT, "profiles", "k_loglik_batch_uneven_lba_256.md")
K_ACC = 4
FLOPS_PER_EVAL = 17 * K_ACC + 2          # algorithmic flops of one LBA trial density
TRANS_PER_EVAL = 4 * K_ACC + 1           # Phi / phi / log evaluations


def max_over_ranks(x: float, device: str) -> float:
    """The largest x over the ranks of the default process group (the
    slowest replica sets the whole job's time)."""
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(steps: int, world: int, ms_max: float) -> float:
    """Sweeps/s of the whole job: every replica's steps over the slowest time."""
    return steps * world / (ms_max / 1e3)


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.rows = []
        if self.proc is None:
            return False
        time.sleep(0.3)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)
        return False

    def summary(self):
        rows = getattr(self, "rows", [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


FX6 = os.path.join(ROOT, "tests", "golden", "lba_fx6.npz")

WORKLOADS = {
    "uneven_lba_256": synth.uneven_lba_256,
    # the reference fixture lba_data6.rda's own data and start samples
    "single_lba_768": lambda: synth.fixture_lba_768(FX6, hierarchical=False),
    "hier_lba_32": lambda: synth.fixture_lba_768(FX6, hierarchical=True),
    "hier_ddm_64": synth.hier_ddm_64,
    "many_fits_1024": synth.many_fits_1024,
}


def make_workload(name=WORKLOAD):
    t = time.time()
    w = WORKLOADS[name]()
    log(f"workload {w.name}: {w.batch.n_subject} subjects, {len(w.batch.rt)} trials, "
        f"{w.nchain} chains ({time.time() - t:.1f}s to simulate)")
    return w


def start_state(w, gpu, h):
    rng = np.random.default_rng(12)
    C_ = w.nchain
    th, phi = synth.start_states(w, C_, rng)
    S = w.batch.n_subject
    lp = np.stack([gpu.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = h.loglik(th, abi.FP64)
    if phi is None:
        return None, (th, lp, ll)
    plp = gpu.logprior(w.h_prior, phi)
    pll = gpu.loghlike(w.p_prior, phi, th.transpose(0, 1, 2))
    return (phi, plp, pll), (th, lp, ll)


def cfg_for(w, steps, precision, flags=0, seed=2025):
    npar = 2 * w.model.n_par if w.hierarchical else w.model.n_par
    return abi.DEConfigPy(nchain=w.nchain, nparameter=npar, nmc=steps + 1, thin=1,
                          pop_migration_prob=0.05, sub_migration_prob=0.06, precision=precision,
                          seed=seed, flags=flags)


def measured_hbm_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


def profiled_traffic():
    """DRAM bytes per launch of the likelihood kernel from the committed ncu
    summary (dram__bytes_read.sum + dram__bytes_write.sum), or None."""
    try:
        with open(PROFILE) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return int(line.split(":")[1].strip())
    except OSError:
        pass
    return None


def loglik_roofline(w, h, n_launch=10, precision=abi.MIXED_SUMS):
    """Time the likelihood API's launches live (CUDA events on its stream):
    all subjects x 51 proposals per call, the k_sub_loglik work of one sweep,
    as k_batch_tables (the proposals' FP32 tables) then k_loglik_batch.
    MIXED_SUMS times these two alone (the sums the sampler uses); MIXED adds
    the likelihood API's FP64 pass over sums near zero."""
    import torch
    rng = np.random.default_rng(5)
    th, _ = synth.start_states(w, w.nchain, rng)
    d_th = torch.from_numpy(np.ascontiguousarray(th)).cuda()
    d_out = torch.empty((w.batch.n_subject, w.nchain), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(3):
        h.loglik_device(d_th.data_ptr(), w.nchain, d_out.data_ptr(), precision, stream.cuda_stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    times = []
    for i in range(n_launch):
        flush.fill_(i & 0xff)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.loglik_device(d_th.data_ptr(), w.nchain, d_out.data_ptr(), precision, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = float(np.median(times))
    evals = int(w.nchain * len(w.batch.rt))
    return ms, evals


def oracle_start(ob, w):
    """The benchmark's start state scored by the oracle (FP64)."""
    rng = np.random.default_rng(12)
    th, phi = synth.start_states(w, w.nchain, rng)
    S = w.batch.n_subject
    lp = np.stack([ob.logprior(w.p_prior, th[s]) for s in range(S)])
    ll = ob.loglik(w.model, w.batch, th)
    pst = None
    if phi is not None:
        pst = (phi, ob.logprior(w.h_prior, phi), ob.loghlike(w.p_prior, phi, th))
    return pst, (th, lp, ll)


def cpu_baseline(w, n_sweeps=1, threads=None):
    """The oracle's -O3 build on the host cores: one replica of n_sweeps
    sweeps of the full workload alone (the single-thread rate, as one
    reference instance runs), then `threads` replicas at once (all cores, as
    the reference's independent instances run); FP64, reference chain order."""
    from oracle import binding as ob
    ob.build()
    phi, subj = oracle_start(ob, w)
    cfg = cfg_for(w, n_sweeps, abi.FP64)
    threads = threads or os.cpu_count() or 1
    times = [0.0] * threads

    def one(k):
        c = abi.DEConfigPy(**{**cfg.__dict__, "seed": 1000 + k})
        t0 = time.perf_counter()
        if phi is not None:
            ob.run(c, w.model, w.batch, w.p_prior, w.h_prior, phi, subj)
        else:
            ob.run_subjects(c, w.model, w.batch, w.p_prior, *subj)
        times[k] = time.perf_counter() - t0

    ob.use_build(fast=True)
    try:
        one(0)
        single = times[0]
        ts = [threading.Thread(target=one, args=(k,)) for k in range(threads)]
        t0 = time.perf_counter()
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        wall = time.perf_counter() - t0
    finally:
        ob.use_build(fast=False)
    sweeps = threads * n_sweeps
    return {"value": sweeps / wall, "unit": "DE sweeps/s", "cores": threads, "kind": "port",
            "sample": f"{threads} concurrent replicas x {n_sweeps} sweep(s) of the full {w.name} "
                      f"workload (after one replica alone), oracle/ FP64 C restatement built -O3, "
                      f"one thread each",
            "single_thread_sweeps_per_s": n_sweeps / single,
            "wall_s": wall, "single_replica_s": single,
            "trial_logl_evals_per_s": sweeps * w.nchain * len(w.batch.rt) / wall}


def oracle_accuracy(w, h, theta):
    """Errors against the oracle (FP64) at the chain states theta [S][C][P]:
    every per-subject sum of the MIXED likelihood through ggdmc_loglik, and
    per trial through ggdmc_trial_logdens for each subject's first chain."""
    from oracle import binding as ob
    ob.build()
    mixed = h.loglik(theta, abi.MIXED)
    want = ob.loglik(w.model, w.batch, theta)
    t32 = h.trial_logdens(theta[:, 0], abi.MIXED)
    t64 = np.concatenate([ob.sumloglike(w.model, w.batch.subject(s).rt, w.batch.subject(s).cell,
                                        theta[s, 0], per_trial=True)[1] for s in range(w.batch.n_subject)])
    return {"max_rel_err_per_sum": float(np.max(np.abs(mixed - want) / np.abs(want))),
            "max_abs_err_per_sum": float(np.max(np.abs(mixed - want))),
            "max_abs_err_per_trial": float(np.max(np.abs(t32 - t64))),
            "median_abs_err_per_trial": float(np.median(np.abs(t32 - t64))),
            "mean_err_per_trial": float(np.mean(t32 - t64)),
            "sums": int(want.size), "trials": int(t64.size),
            "state": "the chains after the timed sweeps"}


def config_of(w, world=1):
    """The workload's description, the same in both arms' lines."""
    S, Cn, P = w.batch.n_subject, w.nchain, w.model.n_par
    c = {"workload": w.name, "subjects": S, "trials": int(len(w.batch.rt)),
         "accumulators": int(w.model.n_acc), "npar": P, "nphi": 2 * P if w.hierarchical else 0,
         "chains": Cn, "pop_migration_prob": 0.05 if w.hierarchical else 0.0, "sub_migration_prob": 0.06,
         "chain_order": "reference (in place, in order)",
         "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
         "l2": "flushed between sweeps (256 MB memset, excluded from the timing)"}
    if w.name == WORKLOAD:
        c["trials_per_subject"] = "U{100..2000}"
    return c


def run_ours(args):
    import torch
    from ggdmc_gb300 import build, gpu
    rank, world, local = dist_env()
    if world > 1:
        torch.distributed.init_process_group("nccl")
        torch.cuda.set_device(local)
    build.build()
    w = make_workload(args.workload)
    default = args.workload == WORKLOAD
    h = gpu.Handle(w.model, w.batch)
    phi, subj = start_state(w, gpu, h)
    peak_fp32, peak_mufu = gpu.probe_peaks()

    # the autotuner's settings for this design and data shape (cached in the
    # process; one-shot ggdmc_run calls of the same shape use them too)
    tuning = None
    if not args.no_tune:
        t0 = time.perf_counter()
        tuning = h.autotune(cfg_for(w, args.warmup, abi.MIXED, abi.FLAG_L2_FLUSH), w.p_prior, *subj,
                            h_table=w.h_prior, phi=phi, n_probe=4)
        tune_s = time.perf_counter() - t0

    # warm-up (also compiles nothing: the library is prebuilt)
    wu = cfg_for(w, args.warmup, abi.MIXED, abi.FLAG_L2_FLUSH)
    h.run(wu, w.p_prior, *subj, h_table=w.h_prior, phi=phi)   # (phi None: independent fits)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    cfg = cfg_for(w, args.steps, abi.MIXED, abi.FLAG_L2_FLUSH)
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        out = h.run(cfg, w.p_prior, *subj, h_table=w.h_prior, phi=phi)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    st = out["stats"]
    ms = st["sweep_ms"]
    tune_line = None
    if tuning is not None:
        # the same timed run under the built-in settings, for comparison
        h.set_tuning(None)
        dflt = h.run(cfg, w.p_prior, *subj, h_table=w.h_prior, phi=phi)["stats"]["sweep_ms"]
        h.set_tuning({k: v for k, v in tuning.items()})
        tune_line = dict(tuning, ms_per_step_tuned=round(ms / args.steps, 4),
                         ms_per_step_default=round(dflt / args.steps, 4), tune_s=round(tune_s, 2))
    if args.profile:
        lk_ms, lk_evals = loglik_roofline(w, h, n_launch=2)
        log(f"profile mode: {args.steps} sweeps in {ms:.3f} ms; likelihood launch {lk_ms:.3f} ms")
        return
    if world > 1:
        ms = max_over_ranks(ms, "cuda")
    sweeps_s = whole_job_rate(args.steps, 1, ms)
    evals_s = st["trial_evals"] / (st["sweep_ms"] / 1e3)

    # plain FP64 one-launch-per-subject form (the comparison the target names)
    n_plain = max(2, min(args.steps, 4))
    plain_sweeps_s = None
    if default:
        pl = h.run(cfg_for(w, n_plain, abi.FP64_PLAIN, abi.FLAG_L2_FLUSH), w.p_prior, *subj,
                   h_table=w.h_prior, phi=phi)["stats"]
        plain_sweeps_s = n_plain / (pl["sweep_ms"] / 1e3)
    fb = h.run(cfg_for(w, n_plain, abi.FP64, abi.FLAG_L2_FLUSH), w.p_prior, *subj,
               h_table=w.h_prior, phi=phi)["stats"]
    fp64_sweeps_s = n_plain / (fb["sweep_ms"] / 1e3)
    if not default:
        line = {"metric": "DE sweeps/s", "value": round(sweeps_s, 3), "unit": "DE sweeps/s",
                "workload": w.name, "subjects": w.batch.n_subject, "trials": int(len(w.batch.rt)),
                "chains": w.nchain, "hierarchical": w.hierarchical, "steps": args.steps,
                "ms_per_step": round(ms / args.steps, 4),
                "trial_logl_evals_per_s": round(evals_s, 1),
                "fp64_fallback_fraction": round(st["fallbacks"] / max(st["trial_evals"], 1), 6),
                "fp64_batched_sweeps_per_s": round(fp64_sweeps_s, 3),
                "acceptance": round(st["accepts"] / max(st["proposals"], 1), 4),
                "tuning": tune_line,
                "clocks": clk.summary()}
        line["config"] = config_of(w, world)
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline(w, 1)
            line["accuracy_vs_oracle"] = oracle_accuracy(w, h, out["theta"])
        print(json.dumps(line), flush=True)
        return

    # likelihood kernel roofline (live): the FP32 kernel alone, and the
    # likelihood API call with its FP64 pass over sums near zero beside it
    lk_ms, lk_evals = loglik_roofline(w, h)
    api_ms, _ = loglik_roofline(w, h, n_launch=3, precision=abi.MIXED)
    ach_tflops = lk_evals * FLOPS_PER_EVAL / (lk_ms * 1e-3) / 1e12
    ach_mufu = lk_evals * TRANS_PER_EVAL / (lk_ms * 1e-3) / 1e12
    # its algorithmic bytes: each trial (float2 time + uint16 cell) once, the
    # theta vectors and the per-(subject, proposal) sums
    S_, C_, P_ = w.batch.n_subject, w.nchain, w.model.n_par
    lk_bytes = len(w.batch.rt) * 10 + S_ * C_ * P_ * 8 + S_ * C_ * 8
    hbm_peak = measured_hbm_gbs()

    # end to end through the one-shot C ABI with host buffers: upload of the
    # trials and chain states, the sweeps, download of every sample
    e2e_steps = min(args.steps, E2E_MAX_STEPS)
    gpu.run(cfg_for(w, e2e_steps, abi.MIXED), w.model, w.batch, w.p_prior, w.h_prior, phi, subj)  # warm-up
    t0 = time.perf_counter()
    e2e = gpu.run(cfg_for(w, e2e_steps, abi.MIXED), w.model, w.batch, w.p_prior, w.h_prior,
                  phi, subj)
    e2e_s = time.perf_counter() - t0
    S, Cn, P = w.batch.n_subject, w.nchain, w.model.n_par
    h2d = (w.batch.rt.nbytes + w.batch.cell.nbytes + w.batch.offsets.nbytes
           + subj[0].nbytes + subj[1].nbytes + subj[2].nbytes
           + phi[0].nbytes + phi[1].nbytes + phi[2].nbytes)
    d2h = 8 * (S * (e2e_steps + 1) * Cn * (P + 2) + (e2e_steps + 1) * Cn * (2 * P + 2)
               + S * Cn * (P + 2) + Cn * (2 * P + 2))

    line = {
        "metric": "DE sweeps/s (trial-logL evals/s beside it), batched mixed FP32/FP64",
        "value": round(whole_job_rate(args.steps, world, ms), 3),
        "unit": "DE sweeps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic (seeded LBA race simulation of the named shapes)",
        "config": config_of(w, world),
        "trial_logl_evals_per_s": round(evals_s * world, 1),
        "fp64_fallback_fraction": round(st["fallbacks"] / max(st["trial_evals"], 1), 6),
        "fp64_plain_sweeps_per_s": round(plain_sweeps_s, 3),
        "fp64_batched_sweeps_per_s": round(fp64_sweeps_s, 3),
        "speedup_vs_fp64_plain": round(sweeps_s / plain_sweeps_s, 2),
        "reevaluations_per_sweep": round(st["reevaluations"] / args.steps, 2),
        "acceptance": round(st["accepts"] / max(st["proposals"], 1), 4),
        "gpu_launches": int(st["kernel_launches"]),
        "tuning": tune_line,
        "roofline": {"kernel": "loglik (k_batch_tables + k_loglik_batch, the k_sub_loglik body)",
                     "bound": "fp32", "achieved": round(ach_tflops, 3),
                     "peak": round(peak_fp32, 3), "unit": "TFLOP/s",
                     "frac": round(ach_tflops / peak_fp32, 4), "traffic": profiled_traffic(),
                     "flops_per_eval": FLOPS_PER_EVAL, "evals_per_launch": lk_evals,
                     "launch_ms": round(lk_ms, 4),
                     "loglik_api_ms_with_fp64_refinement": round(api_ms, 4),
                     "peak_source": "measured (ggdmc_probe_peaks FMA loop)",
                     "sfu": {"achieved_tops": round(ach_mufu, 4), "peak_tops": round(peak_mufu, 4),
                             "frac": round(ach_mufu / peak_mufu, 4),
                             "transcendentals_per_eval": TRANS_PER_EVAL},
                     "hbm_view": {"algorithmic_bytes": int(lk_bytes),
                                  "achieved_gbs": round(lk_bytes / (lk_ms * 1e-3) / 1e9, 2),
                                  "peak_gbs": hbm_peak,
                                  "frac": (round(lk_bytes / (lk_ms * 1e-3) / 1e9 / hbm_peak, 5)
                                           if hbm_peak else None),
                                  "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"}},
        "e2e": {"value": round(e2e_steps / e2e_s, 3), "unit": "DE sweeps/s",
                "h2d_bytes_per_step": int(h2d // e2e_steps), "d2h_bytes_per_step": int(d2h // e2e_steps),
                "steps": e2e_steps,
                "call": "ggdmc_run (one-shot C ABI: upload, sweeps, sample download; "
                        "one untimed call first)",
                # host wall-clock of the call's phases (ggdmc_run_stats) and the
                # Python marshalling around it
                "breakdown_ms": {"total": round(e2e_s * 1e3, 3),
                                 "create_upload": round(e2e["stats"]["setup_ms"], 3),
                                 "graph_capture": round(e2e["stats"]["capture_ms"], 3),
                                 "sweeps_and_sample_copies": round(e2e["stats"]["run_ms"], 3),
                                 "copy_out_release": round(e2e["stats"]["copyout_ms"], 3),
                                 "python": round(e2e_s * 1e3 - sum(e2e["stats"][k] for k in (
                                     "setup_ms", "capture_ms", "run_ms", "copyout_ms")), 3),
                                 "device_sweeps": round(e2e["stats"]["sweep_ms"], 3)}},
        "clocks": clk.summary(),
        "wall_s_timed_run": round(wall, 3),
    }
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(w, 1)
        line["accuracy_vs_oracle"] = oracle_accuracy(w, h, out["theta"])
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    w = make_workload()
    from oracle import binding as ob
    ob.build()
    threads = os.cpu_count() or 1
    # each step: one sweep per replica, all host threads
    vals = []
    t_all = time.perf_counter()
    for _ in range(max(1, min(args.steps, 2))):
        vals.append(cpu_baseline(w, 1, threads))
    wall = time.perf_counter() - t_all
    v = float(np.median([x["value"] for x in vals]))
    line = {
        "metric": "DE sweeps/s (trial-logL evals/s beside it), batched mixed FP32/FP64",
        "value": round(v, 4), "unit": "DE sweeps/s", "impl": "reference",
        "n_gpus": world, "steps": len(vals), "warmup": 0,
        "ms_per_step": round(1e3 / v, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(w, world),
        "trial_logl_evals_per_s": round(float(np.median([x["trial_logl_evals_per_s"] for x in vals])), 1),
        "cpu_baseline": {**vals[0], "value": round(v, 4)},
        "e2e": {"value": round(v, 4), "unit": "DE sweeps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "wall_s": round(wall, 2),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(WORKLOADS),
                    help="another configuration, reported in a reduced line (default: the "
                         "256-subject uneven workload of the contract line)")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (built-in launch settings)")
    ap.add_argument("--profile", action="store_true",
                    help="warm-up and timed sweeps only (for ncu launch lists and captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
