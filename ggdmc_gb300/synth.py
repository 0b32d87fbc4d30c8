"""Seeded synthetic LBA workloads of the shapes the reference's benchmarks name.

The race is simulated as the reference's fixture generators do with
lbaModel::simulate (e.g. tests/testthat/Group1/data/6_lba_Bv_model.r:91-92):
per trial and accumulator, start ~ U(0, A), drift ~ N(mean_v, sd_v) redrawn
until positive, finish = (A + B - start) / drift; RT = t0 + min(finish) and
the response is the argmin.  Subject parameters of hierarchical workloads
are drawn from truncated normals (lower 0) around a population vector.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .design import (BV13_POP_MEAN, BV13_POP_SCALE, DDM9_P, T0_17_P, design_bv13, design_ddm9,
                     design_rows,
                     design_t0_17, vector)
from .dmi import FlatModel, SubjectBatch, SubjectData

PRIOR_ROW_UNIF_0_10 = [0.0, 10.0, 0.0, 10.0, 6.0, 1.0]


def rtnorm(rng, mean, sd, lower=0.0, size=None):
    """Truncated normal draws (lower bound) by rejection."""
    mean = np.asarray(mean, float)
    sd = np.asarray(sd, float)
    out = rng.normal(mean, sd, size=size)
    bad = out <= lower
    while np.any(bad):
        out = np.where(bad, rng.normal(mean, sd, size=out.shape), out)
        bad = out <= lower
    return out


def simulate_subject(model: FlatModel, theta: np.ndarray, n: int, rng, name="") -> SubjectData:
    """n trials spread evenly over the design's stimulus conditions."""
    rows = design_rows(model)
    cv = model.cell_values(theta)            # [n_cell, K, 6]
    K = model.n_acc
    counts = np.full(len(rows), n // len(rows))
    counts[: n % len(rows)] += 1
    rts, cells = [], []
    for (prefix, cell_by_resp), m in zip(rows, counts):
        if m == 0:
            continue
        p = cv[cell_by_resp[0]]              # accumulator parameters do not depend on the response
        A, B, v, s, t0 = p[:, 0], p[:, 1], p[:, 2], p[:, 3], p[0, 4]
        start = rng.random((m, K)) * A
        drift = rng.normal(v, s, size=(m, K))
        bad = drift <= 0
        while np.any(bad):
            drift = np.where(bad, rng.normal(v, s, size=(m, K)), drift)
            bad = drift <= 0
        finish = (A + B - start) / drift
        w = np.argmin(finish, axis=1)
        rts.append(t0 + finish[np.arange(m), w])
        cells.append(np.array(cell_by_resp, np.int32)[w])
    rt = np.concatenate(rts)
    cell = np.concatenate(cells)
    order = np.argsort(cell, kind="stable")  # DMI layout: trials grouped by cell
    return SubjectData(rt[order], cell[order], name)


@dataclass
class Workload:
    name: str
    model: FlatModel
    batch: SubjectBatch
    theta_true: np.ndarray          # [S][P]
    p_prior: np.ndarray             # [P][6]
    h_prior: np.ndarray | None      # [2P][6]
    pop_mean: np.ndarray | None
    pop_scale: np.ndarray | None
    nchain: int
    hierarchical: bool
    # a stored start state (theta [S][C][P], phi [C][2P] or None), used
    # instead of chains scattered around theta_true
    start_theta: np.ndarray | None = None
    start_phi: np.ndarray | None = None


def unif_prior(P, lo=0.0, hi=10.0):
    return np.tile(np.array([lo, hi, lo, hi, 6.0, 1.0]), (P, 1))


def tnorm_prior(mu, sigma, lo=0.0, hi=np.inf):
    mu = np.asarray(mu, float)
    return np.stack([mu, np.broadcast_to(sigma, mu.shape), np.full_like(mu, lo),
                     np.full_like(mu, hi), np.full_like(mu, 1.0), np.ones_like(mu)], axis=1)


def uneven_lba_256(seed: int = 1, n_subject: int = 256, n_lo: int = 100, n_hi: int = 2000,
                   cv: float = 0.10) -> Workload:
    """256 subjects, N_s ~ U{100..2000}, the 17-parameter 4-accumulator design,
    subject theta ~ tnorm(pop, 10% CV, lower 0); hierarchical, 3 x npar chains."""
    rng = np.random.default_rng(seed)
    model = design_t0_17()
    pop = vector(model, T0_17_P)
    ns = rng.integers(n_lo, n_hi + 1, size=n_subject)
    thetas, subs = [], []
    for s in range(n_subject):
        th = rtnorm(rng, pop, cv * pop)
        thetas.append(th)
        subs.append(simulate_subject(model, th, int(ns[s]), rng, str(s + 1)))
    P = model.n_par
    return Workload("uneven_lba_256", model, SubjectBatch.pack(subs), np.array(thetas),
                    tnorm_prior(rng.random(P), 10.0),
                    unif_prior(2 * P), pop, cv * pop, 3 * P, True)


def hier_lba_32(seed: int = 0, n_subject: int = 32, n: int = 768) -> Workload:
    """32 subjects x 768 trials of the 13-parameter design, theta from the
    README's pop_mean / pop_scale truncated normals."""
    rng = np.random.default_rng(seed)
    model = design_bv13()
    mu, sc = vector(model, BV13_POP_MEAN), vector(model, BV13_POP_SCALE)
    thetas, subs = [], []
    for s in range(n_subject):
        th = rtnorm(rng, mu, sc)
        thetas.append(th)
        subs.append(simulate_subject(model, th, n, rng, str(s + 1)))
    P = model.n_par
    return Workload("hier_lba_32", model, SubjectBatch.pack(subs), np.array(thetas),
                    tnorm_prior(rng.random(P), 10.0), unif_prior(2 * P), mu, sc, 3 * P, True)


def many_fits_1024(seed: int = 4, n_fit: int = 1024, n_lo: int = 200, n_hi: int = 5000) -> Workload:
    """1024 independent single-subject fits of the 13-parameter design; theta
    from the 32-subject population, N ~ U{200..5000}; U(0,10) priors."""
    rng = np.random.default_rng(seed)
    model = design_bv13()
    mu, sc = vector(model, BV13_POP_MEAN), vector(model, BV13_POP_SCALE)
    ns = rng.integers(n_lo, n_hi + 1, size=n_fit)
    thetas, subs = [], []
    for s in range(n_fit):
        th = rtnorm(rng, mu, sc)
        thetas.append(th)
        subs.append(simulate_subject(model, th, int(ns[s]), rng, str(s + 1)))
    P = model.n_par
    return Workload("many_fits_1024", model, SubjectBatch.pack(subs), np.array(thetas),
                    unif_prior(P), None, None, None, 3 * P, False)


def simulate_ddm_batch(model: FlatModel, thetas: np.ndarray, ns, rng, dt: float = 1e-4,
                       tmax: float = 5.0) -> list:
    """Diffusion trials by Euler integration of the unit-variance Wiener
    process, every subject's trials advanced together: start a (z + sz (U -
    1/2)), drift ~ N(v, sv^2), absorbed at 0 (response r1) or a (r2);
    RT = decision time + t0 + st0 U, -d/2 for the upper response, +d/2 for
    the lower.  Stimuli are equally likely.  Trials still running at tmax
    are dropped."""
    stimuli = sorted({c.split(".")[0] for c in model.cell_names})
    kidx = {k: i for i, k in enumerate(model.kinds)}
    subj, stim, par = [], [], []
    for s, (th, n) in enumerate(zip(thetas, ns)):
        cv = model.cell_values(th)                      # [n_cell, 2, 8]
        st = rng.integers(0, len(stimuli), int(n))
        rows = np.array([model.cell_names.index(f"{stimuli[k]}.{model.accumulators[0]}") for k in st])
        subj.append(np.full(int(n), s))
        stim.append(st)
        par.append(cv[rows, 0, :])
    subj, stim, par = np.concatenate(subj), np.concatenate(stim), np.concatenate(par)
    g = lambda k: par[:, kidx[k]]
    a, v, z, d, sz, sv, t0, st0 = (g(k) for k in ("a", "v", "z", "d", "sz", "sv", "t0", "st0"))
    x = a * (z + sz * (rng.random(len(a)) - 0.5))
    drift = v + sv * rng.standard_normal(len(a))
    tdec = np.full(len(a), np.nan)
    resp = np.full(len(a), -1)
    act = np.arange(len(a))
    sq = np.sqrt(dt)
    for step in range(1, int(tmax / dt) + 1):
        x[act] += drift[act] * dt + sq * rng.standard_normal(len(act))
        lo, hi = x[act] <= 0.0, x[act] >= a[act]
        done = lo | hi
        if done.any():
            idx = act[done]
            tdec[idx] = step * dt
            resp[idx] = np.where(hi[done], 1, 0)
            act = act[~done]
        if len(act) == 0:
            break
    tnd = t0 + st0 * rng.random(len(a)) + np.where(resp == 1, -d / 2, d / 2)
    rt = tdec + tnd
    out = []
    for s in range(len(ns)):
        m = (subj == s) & (resp >= 0)
        cells = np.array([model.cell_names.index(f"{stimuli[k]}.{model.accumulators[r]}")
                          for k, r in zip(stim[m], resp[m])], np.int32)
        order = np.argsort(cells, kind="stable")           # cell-grouped, as dmi@data
        out.append(SubjectData(rt[m][order], cells[order], str(s + 1)))
    return out


def hier_ddm_64(seed: int = 3, n_subject: int = 64, n: int = 500, dt: float = 1e-4) -> Workload:
    """64 subjects x 500 diffusion trials (Euler, dt = 1e-4 s) of the
    9-parameter design; subject theta ~ N(pop, 10% CV), positive kinds
    truncated at 0; 27 chains (3 x npar)."""
    rng = np.random.default_rng(seed)
    model = design_ddm9()
    pop = vector(model, DDM9_P)
    sc = 0.1 * np.abs(pop)
    signed = np.array([nm.startswith("v.") for nm in model.pnames])
    thetas = []
    for _ in range(n_subject):
        th = pop + sc * rng.standard_normal(len(pop))
        th = np.where(signed, th, np.abs(th))
        thetas.append(th)
    thetas = np.array(thetas)
    subs = simulate_ddm_batch(model, thetas, [n] * n_subject, rng, dt)
    P = model.n_par
    lo = np.where(signed, -np.inf, 0.0)
    hi = np.array([1.0 if nm in ("z", "sz") else np.inf for nm in model.pnames])
    p_prior = np.stack([pop, np.full(P, 2.0), lo, hi, np.ones(P), np.ones(P)], axis=1)
    h_loc = np.stack([pop, np.full(P, 2.0), lo, hi, np.ones(P), np.ones(P)], axis=1)
    h_prior = np.concatenate([h_loc, unif_prior(P, 0.0, 5.0)])
    return Workload("hier_ddm_64", model, SubjectBatch.pack(subs), thetas, p_prior, h_prior,
                    pop, sc, 3 * P, True)


def start_states(w: Workload, nchain: int, rng, spread: float = 0.05):
    """Chains scattered around the generating values (theta [S][C][P] and,
    for hierarchical workloads, phi [C][2P]), or the workload's stored start
    state; lp / ll left for the caller."""
    if w.start_theta is not None:
        phi = w.start_phi[:nchain] if w.start_phi is not None else None
        return np.array(w.start_theta[:, :nchain]), (np.array(phi) if phi is not None else None)
    S, P = w.theta_true.shape
    th = w.theta_true[:, None, :] * (1.0 + spread * rng.standard_normal((S, nchain, P)))
    th = np.abs(th)
    phi = None
    if w.hierarchical:
        loc = w.pop_mean[None, :] * (1.0 + spread * rng.standard_normal((nchain, P)))
        sca = w.pop_scale[None, :] * (1.0 + spread * rng.standard_normal((nchain, P)))
        phi = np.concatenate([np.abs(loc), np.abs(sca)], axis=1)
    return th, phi


def fixture_lba_768(npz: str, hierarchical: bool, nchain: int = 39) -> Workload:
    """The reference fixture lba_data6.rda's own data (tests/golden/lba_fx6.npz):
    the 13-parameter, 2-accumulator design with 768 trials per subject, and
    its stored start samples.  Single subject: its sub_dmi, U(0, 10) priors
    and sub_samples; hierarchical: the 32 pop_dmis, pop_priors and the phi and
    subject chains of pop_samples (the first nchain of them)."""
    z = np.load(npz)
    model = FlatModel(0, list(z["pnames"]), list(z["accumulators"]), list(z["cell_names"]),
                      z["constants"], list(z["const_names"]), z["param_src"], z["resp"])
    if not hierarchical:
        batch = SubjectBatch(z["sub_rt"], z["sub_cell"], np.array([0, len(z["sub_rt"])], np.int64))
        th = z["sub_theta"][None, :nchain]
        return Workload("single_lba_768", model, batch, th[:, 0], z["sub_prior"], None, None, None,
                        nchain, False, start_theta=th)
    batch = SubjectBatch(z["pop_rt"], z["pop_cell"], z["pop_offsets"])
    th = z["subj_theta"][:, :nchain]
    return Workload("hier_lba_32", model, batch, th[:, 0], z["pop_p_prior"], z["pop_h_prior"], None, None,
                    nchain, True, start_theta=th, start_phi=z["phi_theta"][:nchain])
