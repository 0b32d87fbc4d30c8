"""The oracle's DE sampler against a second, independent restatement of
src/de.cpp written here in Python (both consume the same keyed draws).

Two restatements written apart agreeing on every accepted state is the check
that the oracle's chain order, migration cycle, refresh and draw keying follow
de.cpp; the GPU is then held to the oracle.
"""
import math

import numpy as np
import pytest
from scipy.special import erfc

from conftest import load_fixture
from ggdmc_gb300 import abi


class Draws:
    def __init__(self, oracle, seed, C, Pn):
        self.o, self.seed, self.C, self.Pn = oracle, seed, C, Pn

    def u(self, it, lev, p, slot):
        return self.o.uniform(self.seed, it, lev, p, slot)

    def base(self, i):
        return 2 + self.C + i * (self.Pn + 3)

    def partners(self, it, lev, p, i):
        C = self.C
        r0 = min(int(self.u(it, lev, p, self.base(i)) * (C - 1)), C - 2)
        r1 = min(int(self.u(it, lev, p, self.base(i) + 1) * (C - 2)), C - 3)
        others = [c for c in range(C) if c != i]
        a = others[r0]
        rest = [c for c in others if c != a]
        return a, rest[r1]

    def jitter(self, rp, it, lev, p, i, j):
        return -rp + (rp - (-rp)) * self.u(it, lev, p, self.base(i) + 2 + j)

    def accept(self, it, lev, p, i):
        return self.u(it, lev, p, self.base(i) + 2 + self.Pn)

    def subchains(self, it, lev, p):
        C = self.C
        n = min(max(int(math.ceil(C * self.u(it, lev, p, 1))), 2), C)
        perm = list(range(C))
        for j in range(n):
            q = min(j + int(self.u(it, lev, p, 2 + j) * (C - j)), C - 1)
            perm[j], perm[q] = perm[q], perm[j]
        return sorted(perm[:n])


def tnorm_lp(x, mu, sg, lo, hi):
    if x < lo or x > hi or not sg > 0:
        return -math.inf
    a, b = (lo - mu) / sg, (hi - mu) / sg
    if math.isinf(hi) and hi > 0:
        mass = 0.5 * erfc(a / math.sqrt(2))
    else:
        mass = 0.5 * erfc(-b / math.sqrt(2)) - 0.5 * erfc(-a / math.sqrt(2))
    z = (x - mu) / sg
    return -0.5 * z * z - 0.5 * math.log(2 * math.pi) - math.log(sg) - math.log(mass)


def prior_lp(table, x):
    s = 0.0
    for row, v in zip(table, x):
        if int(row[4]) == 1:
            s += tnorm_lp(v, row[0], row[1], row[2], row[3])
        else:
            s += -math.inf if (v < row[0] or v > row[1]) else -math.log(row[1] - row[0])
    return s


def prior_phi(table, phi, x):
    P = len(table)
    return sum(tnorm_lp(v, phi[j], phi[P + j], table[j][2], table[j][3]) for j, v in enumerate(x))


def mh(D, it, lev, p, step, tlp, tll, cur):
    d = (tlp + tll) - cur
    if math.isnan(d):
        return False                       # NaN ratio: rejected without a draw
    r = math.inf if d > 709.0 else math.exp(d)
    return D.accept(it, lev, p, step) < r


def run_chains_py(D, cfg, th, lp, ll, lik, prior, lev=0):
    gamma = cfg.gamma_precursor / math.sqrt(2.0 * cfg.nparameter)
    C, Pn = cfg.nchain, cfg.nparameter
    for it in range(1, (cfg.nmc - 1) * cfg.thin + 1):
        if D.u(it, lev, 0, 0) < cfg.sub_migration_prob:
            sub = D.subchains(it, lev, 0)
            for i, src in enumerate(sub):
                nxt = sub[0] if i + 1 == len(sub) else sub[i + 1]
                tmp = th[src].copy()
                for j in range(Pn):
                    tmp[j] += D.jitter(cfg.rp, it, lev, 0, i, j)
                tlp, tll = prior(tmp), lik(tmp)
                if mh(D, it, lev, 0, i, tlp, tll, lp[nxt] + ll[nxt]):
                    th[nxt], lp[nxt], ll[nxt] = tmp, tlp, tll
        else:
            passes = range(Pn) if cfg.is_pblocked else [None]
            for para in passes:
                p = 0 if para is None else para
                for i in range(C):
                    cur = ll[i] + lp[i]
                    tmp = th[i].copy()
                    a, b = D.partners(it, lev, p, i)
                    js = range(Pn) if para is None else [para]
                    for j in js:
                        tmp[j] += D.jitter(cfg.rp, it, lev, p, i, j) + gamma * (th[a][j] - th[b][j])
                    tlp, tll = prior(tmp), lik(tmp)
                    if mh(D, it, lev, p, i, tlp, tll, cur):
                        th[i], lp[i], ll[i] = tmp, tlp, tll
    return th, lp, ll


@pytest.mark.parametrize("mig,blocked", [(0.0, False), (0.4, False), (0.2, True)])
def test_run_subject_matches_python_restatement(oracle, mig, blocked):
    z, model, sub, _ = load_fixture(6)
    C = 12
    th0 = z["sub_theta"][:C].copy()
    good = np.argsort(z["sub_ll"])[::-1][:C]        # informative chains
    th0 = z["sub_theta"][good].copy()
    lp0, ll0 = z["sub_lp"][good].copy(), z["sub_ll"][good].copy()
    cfg = abi.DEConfigPy(nchain=C, nparameter=model.n_par, nmc=4, thin=2,
                         sub_migration_prob=mig, is_pblocked=blocked, seed=99)
    o = oracle.run_subjects(cfg, model, sub, z["sub_prior"], th0[None], lp0[None], ll0[None])
    D = Draws(oracle, cfg.seed, C, cfg.nparameter)
    lik = lambda t: oracle.sumloglike(model, sub.rt, sub.cell, t)
    prior = lambda t: prior_lp(z["sub_prior"], t)
    th, lp, ll = run_chains_py(D, cfg, [r.copy() for r in th0], list(lp0), list(ll0), lik, prior)
    assert np.array_equal(np.array(th), o["theta"][0])
    assert np.allclose(lp, o["lp"][0], rtol=1e-12) and np.allclose(ll, o["ll"][0], rtol=1e-12)
    assert o["stats"].proposals > 0


def run_hchains_py(D, cfg, phi, subs, liks, p_table, h_table):
    gamma = cfg.gamma_precursor / math.sqrt(2.0 * cfg.nparameter)
    C, Pn, half = cfg.nchain, cfg.nparameter, cfg.nparameter // 2
    pth, plp, pll = phi
    S = len(subs)

    def H(vec, chain):
        return sum(prior_phi(p_table, vec, subs[s][0][chain]) for s in range(S))

    for it in range(1, (cfg.nmc - 1) * cfg.thin + 1):
        ppasses = range(Pn) if cfg.is_hblocked else [None]
        for para in ppasses:
            p = 0 if para is None else para
            if D.u(it, 0, p, 0) < cfg.pop_migration_prob:
                sub = D.subchains(it, 0, p)
                for i, src in enumerate(sub):
                    nxt = sub[0] if i + 1 == len(sub) else sub[i + 1]
                    pll[src] = H(pth[src], src)
                    pll[nxt] = H(pth[nxt], nxt)
                    tmp = pth[src].copy()
                    for j in (range(Pn) if para is None else [para]):
                        tmp[j] += D.jitter(cfg.rp, it, 0, p, i, j)
                    tlp, tll = prior_lp(h_table, tmp), H(tmp, src)
                    if mh(D, it, 0, p, i, tlp, tll, plp[nxt] + pll[nxt]):
                        pth[nxt], plp[nxt], pll[nxt] = tmp, tlp, tll
            else:
                for i in range(C):
                    pll[i] = H(pth[i], i)
                    cur = pll[i] + plp[i]
                    tmp = pth[i].copy()
                    a, b = D.partners(it, 0, p, i)
                    for j in (range(Pn) if para is None else [para]):
                        tmp[j] += D.jitter(cfg.rp, it, 0, p, i, j) + gamma * (pth[a][j] - pth[b][j])
                    tlp, tll = prior_lp(h_table, tmp), H(tmp, i)
                    if mh(D, it, 0, p, i, tlp, tll, cur):
                        pth[i], plp[i], pll[i] = tmp, tlp, tll
        for s in range(S):
            th, lp, ll = subs[s]
            lev = 1 + s
            spasses = range(half) if cfg.is_pblocked else [None]
            for para in spasses:
                p = 0 if para is None else para
                if D.u(it, lev, p, 0) < cfg.sub_migration_prob:
                    sub = D.subchains(it, lev, p)
                    for i, src in enumerate(sub):
                        nxt = sub[0] if i + 1 == len(sub) else sub[i + 1]
                        tmp = th[src].copy()
                        for j in (range(half) if para is None else [para]):
                            tmp[j] += D.jitter(cfg.rp, it, lev, p, i, j)
                        tlp, tll = prior_phi(p_table, pth[src], tmp), liks[s](tmp)
                        if mh(D, it, lev, p, i, tlp, tll, lp[nxt] + ll[nxt]):
                            th[nxt], lp[nxt], ll[nxt] = tmp, tlp, tll
                else:
                    for i in range(C):
                        cur = ll[i] + lp[i]
                        tmp = th[i].copy()
                        a, b = D.partners(it, lev, p, i)
                        for j in (range(half) if para is None else [para]):
                            tmp[j] += D.jitter(cfg.rp, it, lev, p, i, j) + gamma * (th[a][j] - th[b][j])
                        tlp, tll = prior_phi(p_table, pth[i], tmp), liks[s](tmp)
                        if mh(D, it, lev, p, i, tlp, tll, cur):
                            th[i], lp[i], ll[i] = tmp, tlp, tll
    return phi, subs


@pytest.mark.parametrize("pm,sm,hb,pb", [(0.3, 0.3, False, False), (0.2, 0.2, True, True)])
def test_run_hierarchical_matches_python_restatement(oracle, pm, sm, hb, pb):
    z, model, _, pop = load_fixture(6)
    S, C = 3, 10
    batch = type(pop)(pop.rt[: pop.offsets[S]], pop.cell[: pop.offsets[S]], pop.offsets[: S + 1])
    phi = (z["phi_theta"][:C].copy(), z["phi_lp"][:C].copy(), z["phi_ll"][:C].copy())
    subj = (z["subj_theta"][:S, :C].copy(), z["subj_lp"][:S, :C].copy(),
            z["subj_ll"][:S, :C].copy())
    cfg = abi.DEConfigPy(nchain=C, nparameter=2 * model.n_par, nmc=3, thin=1,
                         pop_migration_prob=pm, sub_migration_prob=sm,
                         is_hblocked=hb, is_pblocked=pb, seed=5)
    o = oracle.run(cfg, model, batch, z["pop_p_prior"], z["pop_h_prior"], phi, subj)
    D = Draws(oracle, cfg.seed, C, cfg.nparameter)
    liks = [(lambda t, s=s: oracle.sumloglike(model, batch.subject(s).rt, batch.subject(s).cell, t))
            for s in range(S)]
    pphi = ([r.copy() for r in phi[0]], list(phi[1]), list(phi[2]))
    psub = [([r.copy() for r in subj[0][s]], list(subj[1][s]), list(subj[2][s])) for s in range(S)]
    pphi, psub = run_hchains_py(D, cfg, pphi, psub, liks, z["pop_p_prior"], z["pop_h_prior"])
    assert np.array_equal(np.array(pphi[0]), o["phi"][0])
    assert np.allclose(pphi[2], o["phi"][2], rtol=1e-12)
    for s in range(S):
        assert np.array_equal(np.array(psub[s][0]), o["subj"][0][s])
        assert np.allclose(psub[s][1], o["subj"][1][s], rtol=1e-12)


def test_samples_slot0_and_thinning(oracle):
    z, model, sub, _ = load_fixture(6)
    C = 6
    good = np.argsort(z["sub_ll"])[::-1][:C]
    th0, lp0, ll0 = z["sub_theta"][good], z["sub_lp"][good], z["sub_ll"][good]
    cfg = abi.DEConfigPy(nchain=C, nparameter=model.n_par, nmc=3, thin=2, seed=1)
    o = oracle.run_subjects(cfg, model, sub, z["sub_prior"], th0[None], lp0[None], ll0[None])
    assert np.array_equal(o["s_theta"][0, 0], th0)          # slot 0 = start state
    assert np.array_equal(o["s_theta"][0, -1], o["theta"][0])   # last slot = final state


def test_rejects_two_chains(oracle):
    z, model, sub, _ = load_fixture(6)
    cfg = abi.DEConfigPy(nchain=2, nparameter=model.n_par, nmc=2, seed=1)
    with pytest.raises(RuntimeError):
        oracle.run_subjects(cfg, model, sub, z["sub_prior"], z["sub_theta"][None, :2],
                            z["sub_lp"][None, :2], z["sub_ll"][None, :2])
