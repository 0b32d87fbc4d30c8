/*
 * ggdmc_oracle.c -- CPU ORACLE (test infrastructure, never the product).
 *
 * A plain-C, FP64, single-threaded restatement of ggdmc's DE-MCMC sampling
 * path, used only by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline as the checker the CUDA library is compared against.  Nothing in
 * ggdmc_gb300/ links or calls it.
 *
 * What it restates, and where from:
 *   - de_class (src/de.cpp:1-664 of the reference) line by line: chains are
 *     updated in place and in order, migration cycles through a sorted random
 *     subset, a NaN Metropolis ratio rejects (src/de.cpp:81-108), the phi
 *     level refreshes its hyper log-likelihood before each proposal
 *     (src/de.cpp:397-400,494-500), subject proposals in the hierarchical
 *     model take their prior from phi chain i (src/de.cpp:599-600,646-649).
 *   - the LBA per-trial density of the external ggdmcLikelihood package,
 *     restated from Brown & Heathcote (2008) with the truncated-positive drift
 *     normalisation, in the operation order and with the floors that the
 *     reference's stored log-likelihoods pin (fixtures lba_data2..6.rda):
 *     node-1 pdf floored at 1e-10, t <= 0 gives 1e-10, a non-positive product
 *     gives DBL_EPSILON (R/phi.R:3-13).
 *   - ggdmcPrior's truncated-normal (dist_id 1) and uniform (dist_id 6) log
 *     densities and the hyper sum sumloghlike (src/de.cpp:245-270).
 *   - the Navarro & Fuss (2009) diffusion first-passage density with
 *     sz / sv / st0 variability (ggdmcLikelihood's DDM; parity unpinned).
 *
 * Random draws: the reference calls R's RNG (Rf_runif, arma::shuffle), which
 * cannot run without R.  Both this oracle and the CUDA library instead read
 * uniforms keyed by (iteration, level, pass, slot) -- from a caller array or
 * from Philox4x32-10 (Salmon et al., SC'11) -- with the layout documented in
 * include/ggdmc_gpu.h.  Given the same draws, partner picks, migration
 * subsets and accept decisions are identical.
 *
 * Build: see oracle/Makefile (gcc -O2 -ffp-contract=off: no FMA contraction,
 * so x86 and Arm builds give the same bits).
 */
#define _GNU_SOURCE
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/ggdmc_gpu.h"

#define EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------ normals */
static double Phi(double z) { return 0.5 * erfc(-z * M_SQRT1_2); }
static double phi(double z) { return exp(-0.5 * z * z) * 0.39894228040143267794; }

/* ------------------------------------------------------------ LBA trial
 * cv: [K][6] resolved (A, B, mean_v, sd_v, t0, st0) of the trial's cell.
 * w : responding accumulator.  Returns the density (not its log). */
static double lba_dens(double rt, const double *cv, int K, int w)
{
    double t = rt - cv[w * 6 + 4];
    if (!(t > 0.0)) return 1e-10;
    double pdf = 0.0, surv = 1.0;
    for (int k = 0; k < K; ++k) {
        const double A = cv[k * 6 + 0], b = A + cv[k * 6 + 1];
        const double v = cv[k * 6 + 2], s = cv[k * 6 + 3];
        const double ts = t * s;
        const double chim = b - t * v, xx = chim - A;
        const double cz = chim / ts, czm = xx / ts;
        const double den = Phi(v / s);
        if (k == w) {
            double f = (v * (Phi(cz) - Phi(czm)) + s * (phi(czm) - phi(cz))) / A;
            pdf = f / den;
        } else {
            double F = 1.0 + (ts * (phi(czm) - phi(cz)) + xx * Phi(czm) - chim * Phi(cz)) / A;
            surv = surv * (1.0 - F / den);
        }
    }
    if (!(pdf > 1e-10)) pdf = 1e-10;
    double d = pdf * surv;
    if (!(d > 0.0)) d = DBL_EPSILON;
    return d;
}

/* ------------------------------------------------------------ DDM trial
 * Navarro & Fuss (2009) first-passage time density of the Wiener process at
 * the lower boundary, with the number of series terms chosen by their error
 * bounds; variability in start point (sz), drift (sv, closed form) and
 * non-decision time (st0) is integrated numerically with the midpoint rule
 * (DDM_NZ / DDM_NT nodes).  cv: [2][8] (a, v, z, d, sz, sv, t0, st0) of the
 * cell; w = 0 lower boundary, 1 upper. */
#define DDM_NZ 8
#define DDM_NT 8
#define DDM_EPS 1e-10

static double nf_density(double tt, double w, double eps)
{
    /* density of the standard Wiener FPT at the lower boundary, time tt
     * (scaled by a^2), relative start w in (0,1). */
    if (!(tt > 0.0)) return 0.0;
    double ks, kl;
    /* large-time term count */
    if (M_PI * tt * eps < 1.0) {
        kl = sqrt(-2.0 * log(M_PI * tt * eps) / (M_PI * M_PI * tt));
        double lb = 1.0 / (M_PI * sqrt(tt));
        if (kl < lb) kl = lb;
    } else {
        kl = 1.0 / (M_PI * sqrt(tt));
    }
    /* small-time term count */
    if (2.0 * sqrt(2.0 * M_PI * tt) * eps < 1.0) {
        ks = 2.0 + sqrt(-2.0 * tt * log(2.0 * sqrt(2.0 * M_PI * tt) * eps));
        double lb = sqrt(tt) + 1.0;
        if (ks < lb) ks = lb;
    } else {
        ks = 2.0;
    }
    double p = 0.0;
    if (ks < kl) {
        int K = (int)ceil(ks);
        for (int k = -((K - 1) / 2); k <= (K - 1) / 2; ++k) {
            double x = w + 2.0 * k;
            p += x * exp(-(x * x) / (2.0 * tt));
        }
        p /= sqrt(2.0 * M_PI * tt * tt * tt);
    } else {
        int K = (int)ceil(kl);
        for (int k = 1; k <= K; ++k)
            p += k * exp(-(k * k) * (M_PI * M_PI * tt / 2.0)) * sin(k * M_PI * w);
        p *= M_PI;
    }
    return p;
}

/* density at lower boundary with drift v ~ N(v, sv^2) integrated in closed
 * form, boundary a, absolute start z, decision time t */
static double ddm_fixed(double t, double a, double v, double z, double sv)
{
    if (!(t > 0.0)) return 0.0;
    double w = z / a;
    double g = nf_density(t / (a * a), w, DDM_EPS) / (a * a);
    double den = 1.0 + sv * sv * t;
    double e = (sv * sv * (a * w) * (a * w) - 2.0 * v * a * w - v * v * t) / (2.0 * den);
    return g * exp(e) / sqrt(den);
}

static double ddm_dens(double rt, const double *cv, int w)
{
    const double *p = cv + w * 8;
    double a = p[0], v = p[1], zr = p[2], d = p[3], sz = p[4], sv = p[5];
    double t0 = p[6], st0 = p[7];
    /* upper boundary: mirror drift and start point */
    double zrel = (w == 1) ? 1.0 - zr : zr;
    double vv = (w == 1) ? -v : v;
    /* response-specific non-decision time shift d (t0 +/- d/2) */
    double tshift = (w == 1) ? t0 - d / 2.0 : t0 + d / 2.0;
    int nz = (sz > 0.0) ? DDM_NZ : 1;
    int nt = (st0 > 0.0) ? DDM_NT : 1;
    double acc = 0.0;
    for (int it = 0; it < nt; ++it) {
        double tu = (nt > 1) ? tshift + st0 * ((it + 0.5) / nt) : tshift;
        double tt = rt - tu;
        if (!(tt > 0.0)) continue;
        for (int iz = 0; iz < nz; ++iz) {
            double zz = (nz > 1) ? zrel + sz * ((iz + 0.5) / nz - 0.5) : zrel;
            acc += ddm_fixed(tt, a, vv, zz * a, sv);
        }
    }
    double dens = acc / (double)(nz * nt);
    if (!(dens > 1e-10)) dens = 1e-10;
    return dens;
}

/* ------------------------------------------------------------ model */
static int model_cell_values(const ggdmc_model *m, const double *theta, double *cv)
{
    int n = m->n_cell * m->n_acc * m->n_kind;
    for (int i = 0; i < n; ++i) {
        int32_t s = m->param_src[i];
        cv[i] = (s >= 0) ? theta[s] : m->constants[-1 - s];
    }
    return n;
}

static double subject_sumloglike(const ggdmc_model *m, const double *rt, const int32_t *cell,
                                 int64_t n, const double *theta, double *cv, double *per_trial)
{
    model_cell_values(m, theta, cv);
    const int K = m->n_acc, NK = m->n_kind;
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        int c = cell[i];
        double d = (m->model_type == GGDMC_MODEL_LBA)
                       ? lba_dens(rt[i], cv + (size_t)c * K * NK, K, m->resp[c])
                       : ddm_dens(rt[i], cv + (size_t)c * K * NK, m->resp[c]);
        double ld = log(d);
        if (per_trial) per_trial[i] = ld;
        s += ld;
    }
    return s;
}

/* ------------------------------------------------------------ priors */
static double tnorm_logpdf(double x, double mu, double sigma, double lo, double hi)
{
    if (x < lo || x > hi) return -INFINITY;
    if (!(sigma > 0.0)) return -INFINITY;
    double z = (x - mu) / sigma;
    double a = (lo - mu) / sigma, b = (hi - mu) / sigma;
    double mass;
    if (isinf(hi) && hi > 0) mass = 0.5 * erfc(a * M_SQRT1_2);          /* 1 - Phi(a) */
    else if (isinf(lo) && lo < 0) mass = 0.5 * erfc(-b * M_SQRT1_2);   /* Phi(b)     */
    else mass = Phi(b) - Phi(a);
    return -0.5 * z * z - 0.91893853320467274178 - log(sigma) - log(mass);
}

static double prior_one(const double *row, double x)
{
    int id = (int)row[4];
    if (id == GGDMC_PRIOR_TNORM) return tnorm_logpdf(x, row[0], row[1], row[2], row[3]);
    /* uniform on [p0, p1] */
    if (x < row[0] || x > row[1]) return -INFINITY;
    return -log(row[1] - row[0]);
}

static double sumlogprior(const ggdmc_prior *p, const double *theta)
{
    double s = 0.0;
    for (int j = 0; j < p->n_par; ++j) s += prior_one(p->table + 6 * j, theta[j]);
    return s;
}

/* sumlogprior with p0/p1 replaced by the two halves of phi (src/de.cpp:250-251) */
static double sumlogprior_phi(const ggdmc_prior *p, const double *phi_v, const double *theta)
{
    double s = 0.0;
    const int P = p->n_par;
    for (int j = 0; j < P; ++j) {
        double row[6];
        memcpy(row, p->table + 6 * j, sizeof row);
        row[0] = phi_v[j];
        row[1] = phi_v[P + j];
        s += prior_one(row, theta[j]);
    }
    return s;
}

static int prior_supported(const ggdmc_prior *p)
{
    for (int j = 0; j < p->n_par; ++j) {
        int id = (int)p->table[6 * j + 4];
        if (id != GGDMC_PRIOR_TNORM && id != GGDMC_PRIOR_UNIF) return 0;
        if (p->table[6 * j + 5] == 0.0) return 0;
    }
    return 1;
}

/* ------------------------------------------------------------ draws */
static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}

typedef struct {
    const double *draws;
    uint64_t seed;
    int64_t n_level, n_pass, n_slot;
} draw_ctx;

static double U(const draw_ctx *d, int64_t iter, int64_t level, int64_t pass, int64_t slot)
{
    if (d->draws)
        return d->draws[(((iter - 1) * d->n_level + level) * d->n_pass + pass) * d->n_slot + slot];
    uint32_t c[4] = {(uint32_t)slot, (uint32_t)pass, (uint32_t)level, (uint32_t)iter};
    philox4x32_10(c, (uint32_t)d->seed, (uint32_t)(d->seed >> 32));
    uint64_t m = ((uint64_t)c[0] << 20) | (c[1] >> 12);       /* 52 bits */
    return ((double)m + 0.5) * 0x1p-52;
}

EXPORT double oracle_uniform(uint64_t seed, int64_t iter, int64_t level, int64_t pass, int64_t slot)
{
    draw_ctx d = {NULL, seed, 1, 1, 1};
    return U(&d, iter, level, pass, slot);
}

/* ------------------------------------------------------------ sampler */
typedef struct level_s level_t;
typedef double (*like_fn)(level_t *L, const double *theta, int chain_for_hyper);

typedef struct {
    const ggdmc_de_config *cfg;
    draw_ctx dc;
    double gamma;
    int C;
    int Pn;          /* de_input nparameter */
    int half;        /* Pn / 2 */
    ggdmc_run_stats st;
} de_t;

struct level_s {
    int npar;            /* length of this level's theta */
    int index;           /* draw level */
    double *theta, *lp, *ll;      /* current state [C][npar], [C], [C] */
    /* likelihood context */
    const ggdmc_model *model;
    const double *rt;
    const int32_t *cell;
    int64_t ntrial;
    double *cv;
    /* prior context */
    const ggdmc_prior *prior;        /* prior of this level                  */
    const double *prior_phi;         /* non-NULL: phi [C][2P] supplies p0/p1 */
    int prior_phi_npar;
    /* hyper likelihood context (phi level / hyper-only) */
    const ggdmc_prior *hyp_prior;    /* p_prior whose p0/p1 come from theta  */
    level_t *subjects;               /* phi level: the subject levels        */
    int n_subject;
    const double *hyper_rows;        /* hyper-only: data matrix [n_row][P]   */
    int n_row;
    /* storage */
    ggdmc_samples *out;
};

static double level_lp(level_t *L, const double *theta, int phi_chain)
{
    if (L->prior_phi)
        return sumlogprior_phi(L->prior, L->prior_phi + (size_t)phi_chain * L->prior_phi_npar, theta);
    return sumlogprior(L->prior, theta);
}

/* sumloghlike (src/de.cpp:245-270): sum over subjects of the log prior of
 * subject chain `chain` with p0/p1 = halves of phi. */
static double hyper_ll(level_t *L, const double *phi_v, int chain)
{
    double out = 0.0;
    if (L->subjects) {
        for (int s = 0; s < L->n_subject; ++s) {
            level_t *S = &L->subjects[s];
            out += sumlogprior_phi(L->hyp_prior, phi_v, S->theta + (size_t)chain * S->npar);
        }
    } else {
        for (int r = 0; r < L->n_row; ++r)
            out += sumlogprior_phi(L->hyp_prior, phi_v, L->hyper_rows + (size_t)r * L->hyp_prior->n_par);
    }
    return out;
}

static double level_ll(level_t *L, const double *theta, int chain)
{
    if (L->model)
        return subject_sumloglike(L->model, L->rt, L->cell, L->ntrial, theta, L->cv, NULL);
    return hyper_ll(L, theta, chain);
}

static void partners(const de_t *D, int64_t it, int lev, int pass, int i, int *a, int *b)
{
    const int C = D->C;
    int64_t base = 2 + C + (int64_t)i * (D->Pn + 3);
    double u0 = U(&D->dc, it, lev, pass, base + 0);
    double u1 = U(&D->dc, it, lev, pass, base + 1);
    int r0 = (int)(u0 * (double)(C - 1));
    if (r0 > C - 2) r0 = C - 2;
    int r1 = (int)(u1 * (double)(C - 2));
    if (r1 > C - 3) r1 = C - 3;
    int pa = (r0 < i) ? r0 : r0 + 1;
    int lo = pa < i ? pa : i, hi = pa < i ? i : pa;
    int pb = r1;
    if (pb >= lo) ++pb;
    if (pb >= hi) ++pb;
    *a = pa;
    *b = pb;
}

/* get_subchains (src/de.cpp:62-78): n = clamp(ceil(C*U), 2, C) chains drawn
 * without replacement, sorted ascending. */
static int subchains(const de_t *D, int64_t it, int lev, int pass, int *sub)
{
    const int C = D->C;
    double prop = U(&D->dc, it, lev, pass, 1);
    int n = (int)ceil((double)C * prop);
    if (n < 2) n = 2;
    if (n > C) n = C;
    int perm[4096];
    for (int j = 0; j < C; ++j) perm[j] = j;
    for (int j = 0; j < n; ++j) {
        int r = j + (int)(U(&D->dc, it, lev, pass, 2 + j) * (double)(C - j));
        if (r > C - 1) r = C - 1;
        int tmp = perm[j]; perm[j] = perm[r]; perm[r] = tmp;
    }
    for (int j = 0; j < n; ++j) sub[j] = perm[j];
    /* insertion sort */
    for (int j = 1; j < n; ++j) {
        int x = sub[j], q = j - 1;
        while (q >= 0 && sub[q] > x) { sub[q + 1] = sub[q]; --q; }
        sub[q + 1] = x;
    }
    return n;
}

static double jitter(const de_t *D, int64_t it, int lev, int pass, int step, int j)
{
    int64_t base = 2 + D->C + (int64_t)step * (D->Pn + 3);
    double lo = -D->cfg->rp, hi = D->cfg->rp;
    return lo + (hi - lo) * U(&D->dc, it, lev, pass, base + 2 + j);
}

static double accept_u(const de_t *D, int64_t it, int lev, int pass, int step)
{
    int64_t base = 2 + D->C + (int64_t)step * (D->Pn + 3);
    return U(&D->dc, it, lev, pass, base + 2 + D->Pn);
}

/* update_theta (src/de.cpp:81-108) */
static void metropolis(de_t *D, level_t *L, int dst, const double *tmp, double tmp_lp,
                       double tmp_ll, double cur, int64_t it, int pass, int step)
{
    double mh = exp((tmp_lp + tmp_ll) - cur);
    D->st.proposals++;
    if (isnan(mh)) return;
    if (accept_u(D, it, L->index, pass, step) < mh) {
        memcpy(L->theta + (size_t)dst * L->npar, tmp, sizeof(double) * L->npar);
        L->lp[dst] = tmp_lp;
        L->ll[dst] = tmp_ll;
        D->st.accepts++;
    }
}

/* crossover: subject-only / hyper-only (src/de.cpp:111-155), phi level
 * (src/de.cpp:385-465, refresh first) and subject-in-HB (src/de.cpp:567-613,
 * prior from phi chain i, nloop = half).  para < 0: all parameters. */
static void crossover(de_t *D, level_t *L, int64_t it, int pass, int para, int nloop, int refresh)
{
    const int C = D->C, P = L->npar;
    double tmp[1024];
    for (int i = 0; i < C; ++i) {
        if (refresh) L->ll[i] = hyper_ll(L, L->theta + (size_t)i * P, i);
        double cur = L->ll[i] + L->lp[i];
        memcpy(tmp, L->theta + (size_t)i * P, sizeof(double) * P);
        int a, b;
        partners(D, it, L->index, pass, i, &a, &b);
        const double *ta = L->theta + (size_t)a * P, *tb = L->theta + (size_t)b * P;
        if (para >= 0) {
            tmp[para] += jitter(D, it, L->index, pass, i, para) + D->gamma * (ta[para] - tb[para]);
        } else {
            for (int j = 0; j < nloop; ++j)
                tmp[j] += jitter(D, it, L->index, pass, i, j) + D->gamma * (ta[j] - tb[j]);
        }
        double tlp = level_lp(L, tmp, i);
        double tll = level_ll(L, tmp, i);
        metropolis(D, L, i, tmp, tlp, tll, cur, it, pass, i);
    }
}

/* migration: subject-only (src/de.cpp:157-199), phi level (src/de.cpp:467-565,
 * refreshing both chains), subject-in-HB (src/de.cpp:615-665). */
static void migration(de_t *D, level_t *L, int64_t it, int pass, int para, int nloop, int refresh)
{
    const int P = L->npar;
    int sub[4096];
    double tmp[1024];
    int n = subchains(D, it, L->index, pass, sub);
    D->st.migrations++;
    for (int i = 0; i < n; ++i) {
        int src = sub[i];
        int next = (i + 1 == n) ? sub[0] : sub[i + 1];
        if (refresh) {
            L->ll[src] = hyper_ll(L, L->theta + (size_t)src * P, src);
            L->ll[next] = hyper_ll(L, L->theta + (size_t)next * P, next);
        }
        memcpy(tmp, L->theta + (size_t)src * P, sizeof(double) * P);
        if (para >= 0) {
            tmp[para] += jitter(D, it, L->index, pass, i, para);
        } else {
            for (int j = 0; j < nloop; ++j) tmp[j] += jitter(D, it, L->index, pass, i, j);
        }
        double tlp = level_lp(L, tmp, src);
        double tll = level_ll(L, tmp, src);
        double cur = L->lp[next] + L->ll[next];
        metropolis(D, L, next, tmp, tlp, tll, cur, it, pass, i);
    }
}

static void store(const de_t *D, level_t *L, int64_t it)
{
    const ggdmc_de_config *c = D->cfg;
    if (!L->out || it % c->thin != 0) return;
    int64_t slot = it / c->thin;
    if (slot >= c->nmc) return;
    size_t C = (size_t)D->C, P = (size_t)L->npar;
    memcpy(L->out->theta + slot * C * P, L->theta, sizeof(double) * C * P);
    memcpy(L->out->lp + slot * C, L->lp, sizeof(double) * C);
    memcpy(L->out->ll + slot * C, L->ll, sizeof(double) * C);
}

static void store0(const de_t *D, level_t *L)
{
    if (!L->out) return;
    size_t C = (size_t)D->C, P = (size_t)L->npar;
    memcpy(L->out->theta, L->theta, sizeof(double) * C * P);
    memcpy(L->out->lp, L->lp, sizeof(double) * C);
    memcpy(L->out->ll, L->ll, sizeof(double) * C);
}

static int64_t n_iter_of(const ggdmc_de_config *c)
{
    return (int64_t)(c->nmc - 1) * c->thin;
}

EXPORT ggdmc_status oracle_draw_layout(const ggdmc_de_config *cfg, int32_t n_level,
                                       int32_t hierarchical, int64_t *n_iter, int64_t *n_pass,
                                       int64_t *n_slot, int64_t *total)
{
    int64_t np = 1;
    if (hierarchical) {
        int64_t a = cfg->is_hblocked ? cfg->nparameter : 1;
        int64_t b = cfg->is_pblocked ? cfg->nparameter / 2 : 1;
        np = a > b ? a : b;
    } else if (cfg->is_pblocked) {
        np = cfg->nparameter;
    }
    int64_t ni = n_iter_of(cfg);
    int64_t ns = GGDMC_DRAW_SLOTS(cfg->nchain, cfg->nparameter);
    if (n_iter) *n_iter = ni;
    if (n_pass) *n_pass = np;
    if (n_slot) *n_slot = ns;
    if (total) *total = ni * n_level * np * ns;
    return GGDMC_OK;
}

static int check_cfg(const ggdmc_de_config *cfg)
{
    if (!cfg || cfg->nchain <= 2 || cfg->nmc < 1 || cfg->thin < 1 || cfg->nparameter < 1) return 0;
    if (cfg->nchain > 4096 || cfg->nparameter > 1000) return 0;
    return 1;
}

static void de_init(de_t *D, const ggdmc_de_config *cfg, const double *draws, int n_level, int hier)
{
    memset(D, 0, sizeof *D);
    D->cfg = cfg;
    D->C = cfg->nchain;
    D->Pn = cfg->nparameter;
    D->half = cfg->nparameter / 2;
    D->gamma = cfg->gamma_precursor / sqrt(2.0 * cfg->nparameter);
    D->dc.draws = draws;
    D->dc.seed = cfg->seed;
    oracle_draw_layout(cfg, n_level, hier, NULL, &D->dc.n_pass, &D->dc.n_slot, NULL);
    D->dc.n_level = n_level;
}

/* run_chains (src/de.cpp:201-242) on level L */
static void run_chains(de_t *D, level_t *L)
{
    const ggdmc_de_config *c = D->cfg;
    store0(D, L);
    int64_t ni = n_iter_of(c);
    for (int64_t it = 1; it <= ni; ++it) {
        double u = U(&D->dc, it, L->index, 0, 0);
        if (u < c->sub_migration_prob) {
            migration(D, L, it, 0, -1, D->Pn, 0);
        } else if (c->is_pblocked) {
            for (int p = 0; p < D->Pn; ++p) crossover(D, L, it, p, p, D->Pn, 0);
        } else {
            crossover(D, L, it, 0, -1, D->Pn, 0);
        }
        store(D, L, it);
    }
}

static void fill_stats(const de_t *D, ggdmc_run_stats *stats)
{
    if (stats) *stats = D->st;
}

EXPORT ggdmc_status oracle_run_subject(const ggdmc_de_config *cfg, const ggdmc_model *model,
                                       const ggdmc_data *data, const ggdmc_prior *p_prior,
                                       ggdmc_chain_state *state, const double *draws,
                                       ggdmc_samples *out, ggdmc_run_stats *stats)
{
    if (!check_cfg(cfg) || !model || !data || data->n_subject != 1 || !prior_supported(p_prior))
        return GGDMC_ERR_ARG;
    de_t D;
    de_init(&D, cfg, draws, 1, 0);
    double *cv = malloc(sizeof(double) * model->n_cell * model->n_acc * model->n_kind);
    level_t L;
    memset(&L, 0, sizeof L);
    L.npar = model->n_par;
    L.index = 0;
    L.theta = state->theta; L.lp = state->lp; L.ll = state->ll;
    L.model = model;
    L.rt = data->rt + data->offsets[0];
    L.cell = data->cell + data->offsets[0];
    L.ntrial = data->offsets[1] - data->offsets[0];
    L.cv = cv;
    L.prior = p_prior;
    L.out = out;
    run_chains(&D, &L);
    free(cv);
    fill_stats(&D, stats);
    return GGDMC_OK;
}

EXPORT ggdmc_status oracle_run_subjects(const ggdmc_de_config *cfg, const ggdmc_model *model,
                                        const ggdmc_data *data, const ggdmc_prior *p_prior,
                                        ggdmc_chain_state *state, const double *draws,
                                        ggdmc_samples *out, ggdmc_run_stats *stats)
{
    if (!check_cfg(cfg) || !model || !data || !prior_supported(p_prior)) return GGDMC_ERR_ARG;
    de_t D;
    de_init(&D, cfg, draws, data->n_subject, 0);
    double *cv = malloc(sizeof(double) * model->n_cell * model->n_acc * model->n_kind);
    for (int f = 0; f < data->n_subject; ++f) {
        level_t L;
        memset(&L, 0, sizeof L);
        L.npar = model->n_par;
        L.index = f;
        L.theta = state[f].theta; L.lp = state[f].lp; L.ll = state[f].ll;
        L.model = model;
        L.rt = data->rt + data->offsets[f];
        L.cell = data->cell + data->offsets[f];
        L.ntrial = data->offsets[f + 1] - data->offsets[f];
        L.cv = cv;
        L.prior = p_prior;
        L.out = out ? &out[f] : NULL;
        run_chains(&D, &L);
    }
    free(cv);
    fill_stats(&D, stats);
    return GGDMC_OK;
}

EXPORT ggdmc_status oracle_run_hyper(const ggdmc_de_config *cfg, const double *hyper_data,
                                     int32_t n_row, const ggdmc_prior *p_prior,
                                     const ggdmc_prior *h_prior, ggdmc_chain_state *state,
                                     const double *draws, ggdmc_samples *out,
                                     ggdmc_run_stats *stats)
{
    if (!check_cfg(cfg) || !hyper_data || n_row < 1 || !prior_supported(p_prior) ||
        !prior_supported(h_prior) || h_prior->n_par != 2 * p_prior->n_par)
        return GGDMC_ERR_ARG;
    de_t D;
    de_init(&D, cfg, draws, 1, 0);
    level_t L;
    memset(&L, 0, sizeof L);
    L.npar = h_prior->n_par;
    L.index = 0;
    L.theta = state->theta; L.lp = state->lp; L.ll = state->ll;
    L.prior = h_prior;
    L.hyp_prior = p_prior;
    L.hyper_rows = hyper_data;
    L.n_row = n_row;
    L.out = out;
    run_chains(&D, &L);
    fill_stats(&D, stats);
    return GGDMC_OK;
}

/* run_hchains (src/de.cpp:272-383) */
EXPORT ggdmc_status oracle_run(const ggdmc_de_config *cfg, const ggdmc_model *model,
                               const ggdmc_data *data, const ggdmc_prior *p_prior,
                               const ggdmc_prior *h_prior, ggdmc_chain_state *phi_state,
                               ggdmc_chain_state *subj_state, const double *draws,
                               ggdmc_samples *phi_out, ggdmc_samples *subj_out,
                               ggdmc_run_stats *stats)
{
    if (!check_cfg(cfg) || !model || !data || data->n_subject < 1 || !prior_supported(p_prior) ||
        !prior_supported(h_prior) || p_prior->n_par != model->n_par ||
        h_prior->n_par != 2 * model->n_par)
        return GGDMC_ERR_ARG;
    const int S = data->n_subject;
    de_t D;
    de_init(&D, cfg, draws, S + 1, 1);
    double *cv = malloc(sizeof(double) * model->n_cell * model->n_acc * model->n_kind);
    level_t *subs = calloc((size_t)S, sizeof(level_t));
    level_t phi;
    memset(&phi, 0, sizeof phi);
    phi.npar = h_prior->n_par;
    phi.index = 0;
    phi.theta = phi_state->theta; phi.lp = phi_state->lp; phi.ll = phi_state->ll;
    phi.prior = h_prior;
    phi.hyp_prior = p_prior;
    phi.subjects = subs;
    phi.n_subject = S;
    phi.out = phi_out;
    for (int s = 0; s < S; ++s) {
        level_t *L = &subs[s];
        L->npar = model->n_par;
        L->index = 1 + s;
        L->theta = subj_state[s].theta; L->lp = subj_state[s].lp; L->ll = subj_state[s].ll;
        L->model = model;
        L->rt = data->rt + data->offsets[s];
        L->cell = data->cell + data->offsets[s];
        L->ntrial = data->offsets[s + 1] - data->offsets[s];
        L->cv = cv;
        L->prior = p_prior;
        L->prior_phi = phi_state->theta;
        L->prior_phi_npar = phi.npar;
        L->out = subj_out ? &subj_out[s] : NULL;
        store0(&D, L);
    }
    store0(&D, &phi);
    int64_t ni = n_iter_of(cfg);
    for (int64_t it = 1; it <= ni; ++it) {
        if (cfg->is_hblocked) {
            for (int p = 0; p < D.Pn; ++p) {
                if (U(&D.dc, it, 0, p, 0) < cfg->pop_migration_prob)
                    migration(&D, &phi, it, p, p, D.Pn, 1);
                else
                    crossover(&D, &phi, it, p, p, D.Pn, 1);
            }
        } else {
            if (U(&D.dc, it, 0, 0, 0) < cfg->pop_migration_prob)
                migration(&D, &phi, it, 0, -1, D.Pn, 1);
            else
                crossover(&D, &phi, it, 0, -1, D.Pn, 1);
        }
        for (int s = 0; s < S; ++s) {
            level_t *L = &subs[s];
            if (cfg->is_pblocked) {
                for (int p = 0; p < D.half; ++p) {
                    if (U(&D.dc, it, L->index, p, 0) < cfg->sub_migration_prob)
                        migration(&D, L, it, p, p, D.half, 0);
                    else
                        crossover(&D, L, it, p, p, D.half, 0);
                }
            } else {
                if (U(&D.dc, it, L->index, 0, 0) < cfg->sub_migration_prob)
                    migration(&D, L, it, 0, -1, D.half, 0);
                else
                    crossover(&D, L, it, 0, -1, D.half, 0);
            }
            store(&D, L, it);
        }
        store(&D, &phi, it);
    }
    free(subs);
    free(cv);
    fill_stats(&D, stats);
    return GGDMC_OK;
}

/* ------------------------------------------------------------ checkers */
EXPORT double oracle_sumloglike(const ggdmc_model *m, const double *rt, const int32_t *cell,
                                int64_t n, const double *theta, double *per_trial)
{
    double *cv = malloc(sizeof(double) * m->n_cell * m->n_acc * m->n_kind);
    double s = subject_sumloglike(m, rt, cell, n, theta, cv, per_trial);
    free(cv);
    return s;
}

EXPORT ggdmc_status oracle_loglik(const ggdmc_model *m, const ggdmc_data *data,
                                  const double *theta, int32_t n_theta, double *out)
{
    double *cv = malloc(sizeof(double) * m->n_cell * m->n_acc * m->n_kind);
    for (int s = 0; s < data->n_subject; ++s) {
        int64_t a = data->offsets[s], b = data->offsets[s + 1];
        for (int j = 0; j < n_theta; ++j)
            out[(size_t)s * n_theta + j] = subject_sumloglike(
                m, data->rt + a, data->cell + a, b - a,
                theta + ((size_t)s * n_theta + j) * m->n_par, cv, NULL);
    }
    free(cv);
    return GGDMC_OK;
}

EXPORT ggdmc_status oracle_logprior(const ggdmc_prior *p, const double *theta, int32_t n,
                                    double *out)
{
    for (int i = 0; i < n; ++i) out[i] = sumlogprior(p, theta + (size_t)i * p->n_par);
    return GGDMC_OK;
}

EXPORT ggdmc_status oracle_loghlike(const ggdmc_prior *p_prior, const double *phi_v,
                                    const double *subj_theta, int32_t n_subject, int32_t n,
                                    double *out)
{
    const int P = p_prior->n_par;
    for (int j = 0; j < n; ++j) {
        double s = 0.0;
        for (int q = 0; q < n_subject; ++q)
            s += sumlogprior_phi(p_prior, phi_v + (size_t)j * 2 * P,
                                 subj_theta + ((size_t)q * n + j) * P);
        out[j] = s;
    }
    return GGDMC_OK;
}

/* ------------------------------------------------------------ start states
 * initialise_theta / initialise_phi (R/phi.R:141-332): chain c of subject s
 * takes the first of max_attempts draws from p_prior whose prior and
 * likelihood are both finite; then each phi chain c the first draw from
 * h_prior whose prior and hyper log-likelihood against the subjects' chains
 * c are finite.  R draws with rprior; here draw j of attempt a of chain c at
 * level v (0 phi, 1 + s subject s) is the prior's inverse distribution
 * function at the keyed uniform (iteration 0, level v, pass a, slot
 * c * npar + j) -- iteration 0 is never used by the sampler. */
static double Phi_inv(double p)
{
    /* bisection to a bracket, then Newton on Phi (erfc-based) */
    double lo = -40.0, hi = 40.0, x = 0.0;
    for (int it = 0; it < 60; ++it) {
        x = 0.5 * (lo + hi);
        if (Phi(x) < p) lo = x; else hi = x;
    }
    for (int it = 0; it < 3; ++it) {
        double f = Phi(x) - p, d = exp(-0.5 * x * x) * 0.39894228040143267794;
        if (!(d > 0.0)) break;
        x -= f / d;
    }
    return x;
}

static double prior_draw(const double *row, double u)
{
    if ((int)row[4] == GGDMC_PRIOR_UNIF) return row[0] + u * (row[1] - row[0]);
    double mu = row[0], sg = row[1], lo = row[2], hi = row[3];
    double pa = isinf(lo) ? 0.0 : Phi((lo - mu) / sg), pb = isinf(hi) ? 1.0 : Phi((hi - mu) / sg);
    double x = mu + sg * Phi_inv(pa + u * (pb - pa));
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}

EXPORT ggdmc_status oracle_initialise(const ggdmc_model *m, const ggdmc_data *data,
                                      const ggdmc_prior *p_prior, const ggdmc_prior *h_prior,
                                      int32_t nchain, int32_t max_attempts, uint64_t seed,
                                      ggdmc_chain_state *subj, ggdmc_chain_state *phi)
{
    const int P = p_prior->n_par, S = data->n_subject;
    draw_ctx d = {NULL, seed, 1, 1, 1};
    double *cv = malloc(sizeof(double) * m->n_cell * m->n_acc * m->n_kind);
    double th[1024];
    for (int s = 0; s < S; ++s) {
        int64_t a0 = data->offsets[s], b0 = data->offsets[s + 1];
        for (int c = 0; c < nchain; ++c) {
            int ok = 0;
            for (int a = 0; a < max_attempts && !ok; ++a) {
                for (int j = 0; j < P; ++j)
                    th[j] = prior_draw(p_prior->table + 6 * j, U(&d, 0, 1 + s, a, (int64_t)c * P + j));
                double lp = sumlogprior(p_prior, th);
                double ll = isfinite(lp) ? subject_sumloglike(m, data->rt + a0, data->cell + a0, b0 - a0, th, cv, NULL)
                                         : -INFINITY;
                if (isfinite(lp) && isfinite(ll)) {
                    memcpy(subj[s].theta + (size_t)c * P, th, sizeof(double) * P);
                    subj[s].lp[c] = lp;
                    subj[s].ll[c] = ll;
                    ok = 1;
                }
            }
            if (!ok) { free(cv); return GGDMC_ERR_NUMERIC; }
        }
    }
    free(cv);
    if (!phi || !h_prior) return GGDMC_OK;
    const int H = h_prior->n_par;
    for (int c = 0; c < nchain; ++c) {
        int ok = 0;
        for (int a = 0; a < max_attempts && !ok; ++a) {
            for (int j = 0; j < H; ++j)
                th[j] = prior_draw(h_prior->table + 6 * j, U(&d, 0, 0, a, (int64_t)c * H + j));
            double lp = sumlogprior(h_prior, th);
            double ll = 0.0;
            for (int s = 0; s < S && isfinite(lp); ++s)
                ll += sumlogprior_phi(p_prior, th, subj[s].theta + (size_t)c * P);
            if (isfinite(lp) && isfinite(ll)) {
                memcpy(phi->theta + (size_t)c * H, th, sizeof(double) * H);
                phi->lp[c] = lp;
                phi->ll[c] = ll;
                ok = 1;
            }
        }
        if (!ok) return GGDMC_ERR_NUMERIC;
    }
    return GGDMC_OK;
}

EXPORT double oracle_tnorm_logpdf(double x, double mu, double sigma, double lo, double hi)
{
    return tnorm_logpdf(x, mu, sigma, lo, hi);
}

EXPORT double oracle_lba_dens(double rt, const double *cv, int K, int w)
{
    return lba_dens(rt, cv, K, w);
}

EXPORT double oracle_ddm_dens(double rt, const double *cv, int w)
{
    return ddm_dens(rt, cv, w);
}

/* raw Philox4x32-10 block, for known-answer tests */
EXPORT void oracle_philox(uint32_t *ctr, uint32_t k0, uint32_t k1)
{
    philox4x32_10(ctr, k0, k1);
}
