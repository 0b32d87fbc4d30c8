// sampler_kernels.cu -- DE-MCMC kernels for GB300 (sm_103a).
//
// One DE iteration of ggdmc's sampler (src/de.cpp) is a short launch
// sequence, captured into a CUDA graph by the host runtime:
//
//   phi level:  k_phi_propose -> k_phi_eval -> k_phi_resolve -> k_phi_tables
//   subjects:   k_sub_propose -> k_sub_loglik -> k_sub_resolve   (per pass)
//   k_store -> k_next_iter
//
// The reference updates chains in place and in order (src/de.cpp:111-155):
// chain i's partners may already have moved earlier in the same sweep.  The
// kernels keep exactly that semantics by speculation.  k_sub_propose builds
// every chain's proposal from the start-of-pass state and k_sub_loglik
// evaluates all of them at once (the hot path: each CTA evaluates up to four
// proposals of one subject, trials striped over its threads).  k_sub_resolve
// then walks each subject's steps in order on one CTA, taking Metropolis
// decisions from the speculative results for as long as a proposal is the
// one the sequential algorithm would have built, and re-proposes and
// re-evaluates the rest round by round.  Given the same draws the accepted
// states equal the sequential sampler's.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstdint>

#include "dfloat.h"
#include "sampler.cuh"

// k_sub_resolve's block: 512 threads, one CTA per SM (128 registers a thread;
// measured faster than 384 x 2 and 768 x 1 on the 256-subject workload)
#ifndef GGDMC_RESOLVE_THREADS
#define GGDMC_RESOLVE_THREADS 512
#endif
#ifndef GGDMC_RESOLVE_MINB
#define GGDMC_RESOLVE_MINB 1
#endif
// likelihood kernels: 6 blocks of 128 threads per SM (80 registers), which
// measured faster than 4 (128 registers) or 1
#ifndef GGDMC_LIK_MINB
#define GGDMC_LIK_MINB 6
#endif
// the 4-accumulator LBA instantiations of the speculative and batch
// likelihood kernels: 8 blocks per SM (64 registers) measured 8% faster on
// the batch kernel and 1% on the sweep; 2-accumulator designs and the
// diffusion model measured 2-10% slower at 8 than at 6
#ifndef GGDMC_LIK_MINB_LBA
#define GGDMC_LIK_MINB_LBA 8
#endif

namespace ggdmc {

constexpr int kLikThreads = 128;
constexpr int kResolveThreads = GGDMC_RESOLVE_THREADS;
// resolve migration levels first (1) or by trial count alone (0)
#ifndef GGDMC_MIG_FIRST
#define GGDMC_MIG_FIRST 1
#endif
constexpr int kPhiThreads = 256;
constexpr int kProposeThreads = 512;
// k_sub_step's claim counters (RunDev::ctl)
constexpr int kCtlResNext = 0, kCtlResDone = 1, kCtlEvents = 2, kCtlN = 3;
constexpr int kPhiProposeThreads = 1024;   // one CTA: a warp per phi chain's prior

// ------------------------------------------------------------- helpers
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ double block_sum(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = (lane < nw) ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[32] = v;
    }
    __syncthreads();
    const double out = red[32];
    __syncthreads();
    return out;
}

// Add one warp's integer partials (every lane's s, e, nf) to a proposal's
// shared-memory JobPart: a shuffle reduction, then one atomic per field from
// lane 0.  Integer addition is exact, so neither the lanes' nor the warps'
// order changes the result.  Warp-uniform call.
__device__ __forceinline__ void warp_flush(JobPart &p, long long s, int e, int nf)
{
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        e += __shfl_down_sync(0xffffffffu, e, o);
        nf += __shfl_down_sync(0xffffffffu, nf, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (s) atomicAdd(reinterpret_cast<unsigned long long *>(&p.s), (unsigned long long)s);
        if (e) atomicAdd(&p.e, e);
        if (nf) atomicAdd(&p.nf, nf);
    }
}

__device__ __forceinline__ double prior_term(const double *row, double x)
{
    const int id = (int)row[0];
    if (id == 1) {
        if (x < row[3] || x > row[4]) return -INFINITY;
        if (!(row[2] > 0.0)) return -INFINITY;
        const double z = (x - row[1]) / row[2];
        return -0.5 * z * z + row[5];
    }
    if (x < row[1] || x > row[2]) return -INFINITY;
    return row[5];
}

// Constant part of the truncated-normal log density:
// -log(sqrt(2 pi)) - log(sigma) - log(Phi(b) - Phi(a)).
__device__ __forceinline__ double tnorm_const(double mu, double sigma, double lo, double hi)
{
    if (!(sigma > 0.0)) return -INFINITY;
    const double a = (lo - mu) / sigma, b = (hi - mu) / sigma;
    double mass;
    if (isinf(hi) && hi > 0) mass = 0.5 * erfc(a * 0.70710678118654752440);
    else if (isinf(lo) && lo < 0) mass = 0.5 * erfc(-b * 0.70710678118654752440);
    else mass = Phi64(b) - Phi64(a);
    return -0.91893853320467274178 - log(sigma) - log(mass);
}

// The same constant in FP32 (MIXED): on this GPU an FP64 erfc costs about
// 4,300 cycles and an FP64 log about 2,000, and the constant is needed for
// every phi vector scored.  The relative error of the FP32 form is ~1e-7.
__device__ __forceinline__ double tnorm_const_mixed(double mu, double sigma, double lo, double hi)
{
    if (!(sigma > 0.0)) return -INFINITY;
    const float is = 1.f / (float)sigma;
    const float a = (float)(lo - mu) * is, b = (float)(hi - mu) * is;
    float mass;
    if (isinf(hi) && hi > 0) mass = 0.5f * erfcf(a * 0.70710678f);
    else if (isinf(lo) && lo < 0) mass = 0.5f * erfcf(-b * 0.70710678f);
    else mass = normcdff(b) - normcdff(a);
    return (double)(-0.918938533f - logf((float)sigma) - logf(mass));
}

__device__ __forceinline__ double tnorm_const_p(const RunDev &r, double mu, double sigma, double lo, double hi)
{
    return (r.prec == PREC_MIXED) ? tnorm_const_mixed(mu, sigma, lo, hi) : tnorm_const(mu, sigma, lo, hi);
}

// The phi level's prior (h_prior), the warp's lanes over the parameters;
// every lane gets the sum.
__device__ __forceinline__ double warp_phi_prior(const RunDev &r, const double *th)
{
    double s = 0.0;
    for (int j = threadIdx.x & 31; j < r.Pphi; j += 32) s += prior_term(r.hprior + kPriorRow * j, th[j]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    return __shfl_sync(0xffffffffu, s, 0);
}

// Metropolis test of update_theta (src/de.cpp:81-108): accept iff
// u < exp(d), d = log posterior difference; NaN rejects.  FP64 instructions
// are scarce on this GPU and this test sits on the serial decision path, so
// FP32 decides unless u lies within the FP32 error bound of exp(d): expf is
// within 2 ulp, rounding d to float moves exp(d) by at most |d| 2^-24
// relative and the two products round once more.  Only inside that band is
// the double exp evaluated, so the outcome equals u < exp(d) in FP64.
__device__ __forceinline__ bool mh_accept(double d, double u)
{
    if (isnan(d)) return false;
    if (d >= 0.0) return u < 1.0 || u < exp(d);
    if (d < -746.0) return u < 0.0;             // exp(d) underflows to +0
    if (d < -80.0) return u < exp(d);           // rare: exp(d) < 2e-35
    const float df = (float)d;
    const float e = expf(df);
    const float m = 1e-6f + fabsf(df) * 1.2e-7f;
    if (u < (double)(e * (1.f - m))) return true;
    if (u > (double)(e * (1.f + m))) return false;
    return u < exp(d);
}

// draw slots (include/ggdmc_gpu.h): base(step) = 2 + C + step*(Pn+3)
__device__ __forceinline__ int64_t step_base(const RunDev &r, int step)
{
    return 2 + (int64_t)r.C + (int64_t)step * (r.Pn + 3);
}

__device__ __forceinline__ double jitter_draw(const RunDev &r, int64_t it, int lev, int pass, int step,
                                              int j)
{
    const double lo = -r.rp, hi = r.rp;
    const double u = uniform(r.ds, it, lev, pass, step_base(r, step) + 2 + j);
    return __dadd_rn(lo, __dmul_rn(__dsub_rn(hi, lo), u));
}

__device__ __forceinline__ double accept_draw(const RunDev &r, int64_t it, int lev, int pass, int step)
{
    return uniform(r.ds, it, lev, pass, step_base(r, step) + 2 + r.Pn);
}

// get_chains (src/de.cpp:52-60): two distinct partners other than i
__device__ __forceinline__ void partners(const RunDev &r, int64_t it, int lev, int pass, int i,
                                         int &a, int &b)
{
    const int C = r.C;
    const int64_t base = step_base(r, i);
    const double u0 = uniform(r.ds, it, lev, pass, base);
    const double u1 = uniform(r.ds, it, lev, pass, base + 1);
    int r0 = (int)(u0 * (double)(C - 1));
    if (r0 > C - 2) r0 = C - 2;
    int r1 = (int)(u1 * (double)(C - 2));
    if (r1 > C - 3) r1 = C - 3;
    const int pa = (r0 < i) ? r0 : r0 + 1;
    const int lo = pa < i ? pa : i, hi = pa < i ? i : pa;
    int pb = r1;
    if (pb >= lo) ++pb;
    if (pb >= hi) ++pb;
    a = pa;
    b = pb;
}

// get_subchains (src/de.cpp:62-78) from uniforms u[1..C+1] drawn in
// parallel; single thread.
// Migration subset (src/de.cpp:62-78): n = ceil(C u1) clamped to [2, C]
// chains picked by a partial Fisher-Yates shuffle on the keyed uniforms
// (perm[0..n) after the call); subchains_sort then sorts them ascending.
__device__ int subchains_pick(int C, const double *u, int *perm)
{
    int n = (int)ceil((double)C * u[1]);
    if (n < 2) n = 2;
    if (n > C) n = C;
    for (int j = 0; j < C; ++j) perm[j] = j;
    for (int j = 0; j < n; ++j) {
        int q = j + (int)(u[2 + j] * (double)(C - j));
        if (q > C - 1) q = C - 1;
        const int t = perm[j]; perm[j] = perm[q]; perm[q] = t;
    }
    return n;
}

// sub = perm[0..n) in ascending order (the picks are distinct: each one's
// rank is the number of smaller picks).  All threads.
__device__ __forceinline__ void subchains_sort(const int *perm, int n, int *sub)
{
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const int x = perm[j];
        int rank = 0;
        for (int i = 0; i < n; ++i) rank += (perm[i] < x) ? 1 : 0;
        sub[rank] = x;
    }
    __syncthreads();
}

// one component of a crossover proposal (src/de.cpp:111-142):
// theta_i + (U(-rp,rp) + gamma (theta_a - theta_b))
__device__ __forceinline__ double cross_comp(double gamma, double ti, double ta, double tb, double jit)
{
    return __dadd_rn(ti, __dadd_rn(jit, __dmul_rn(gamma, __dsub_rn(ta, tb))));
}

__device__ __forceinline__ bool updated(int j, int para, int nloop)
{
    return (para >= 0) ? (j == para) : (j < nloop);
}

// --------------------------------------------------- subject likelihood
constexpr int kGroup = 4;   // proposals evaluated together per pass over the trials

struct SubSmem {
    double *theta;   // [kGroup][kMaxTheta]
    double *e64;     // n_ent * 5
    double *t064;    // n_t0
    double *red;     // kRedDoubles: block reductions
    Ent32 *e32;      // [kGroup][n_ent] FP32 trial constants of each proposal
    double *lg;      // [kGroup][n_ent] log g of each tuple (FP64)
    float2 *t032;    // [kGroup][n_t0]
    uint8_t *cent;   // n_cell * n_acc
    uint8_t *cw;     // n_cell
    uint8_t *ct0;    // n_cell
    int *flag;       // [kGroup] 1: FP32 form unusable for proposal g
    double *d64;     // [kGroup][n_dent][8] DDM entries (FP64)
    float *d32;      // [kGroup][n_dent][8] DDM entries (FP32; [3],[7] tshift hi, lo)
    int *fb;         // [kFbCap] trials whose FP32 form declined: trial << 2 | proposal
    int *fbn;        // their count
};

__host__ __device__ inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

constexpr int kFbCap = 1024;   // FP64 re-evaluations a block lists before re-scanning its trials
// block reductions: block_sum (33) or a group of kGroup (double, float pair,
// int) sums, 3 doubles per warp and proposal, plus the results
constexpr int kRedDoubles = 33 + kGroup * 32 * 3 + kGroup;

__host__ __device__ inline size_t sub_smem_layout(const DevModel &m, size_t off[16])
{
    size_t o = 0;
    off[0] = o; o += sizeof(double) * kMaxTheta * kGroup;
    off[1] = o; o += sizeof(double) * 5 * m.n_ent;
    off[2] = o; o += sizeof(double) * m.n_t0;
    off[3] = o; o += sizeof(double) * kRedDoubles;
    o = align_up(o, 16);
    off[4] = o; o += sizeof(Ent32) * m.n_ent * kGroup;
    off[5] = o; o += sizeof(double) * m.n_ent * kGroup;
    off[6] = o; o += sizeof(float2) * m.n_t0 * kGroup;
    off[7] = o; o += (size_t)m.n_cell * m.n_acc;
    off[8] = o; o += m.n_cell;
    off[9] = o; o += m.n_cell;
    o = align_up(o, 16);
    off[10] = o; o += sizeof(int) * kGroup;
    o = align_up(o, 16);
    off[11] = o; o += sizeof(double) * 8 * m.n_dent * kGroup;
    off[12] = o; o += sizeof(float) * 8 * m.n_dent * kGroup;
    o = align_up(o, 16);
    off[13] = o; o += sizeof(int) * kFbCap;
    off[14] = o; o += sizeof(int) * 4;
    return align_up(o, 16);
}

__host__ __device__ size_t sub_smem_bytes(const DevModel &m)
{
    size_t off[16];
    return sub_smem_layout(m, off);
}

__device__ SubSmem carve(char *base, const DevModel &m)
{
    size_t off[16];
    sub_smem_layout(m, off);
    SubSmem s;
    s.theta = (double *)(base + off[0]);
    s.e64 = (double *)(base + off[1]);
    s.t064 = (double *)(base + off[2]);
    s.red = (double *)(base + off[3]);
    s.e32 = (Ent32 *)(base + off[4]);
    s.lg = (double *)(base + off[5]);
    s.t032 = (float2 *)(base + off[6]);
    s.cent = (uint8_t *)(base + off[7]);
    s.cw = (uint8_t *)(base + off[8]);
    s.ct0 = (uint8_t *)(base + off[9]);
    s.flag = (int *)(base + off[10]);
    s.d64 = (double *)(base + off[11]);
    s.d32 = (float *)(base + off[12]);
    s.fb = (int *)(base + off[13]);
    s.fbn = (int *)(base + off[14]);
    return s;
}

__device__ void load_design(const RunDev &r, SubSmem &sm)
{
    const int n = r.m.n_cell * r.m.n_acc;
    for (int i = threadIdx.x; i < n; i += blockDim.x) sm.cent[i] = r.m.cell_ent[i];
    for (int i = threadIdx.x; i < r.m.n_cell; i += blockDim.x) {
        sm.cw[i] = r.m.cell_w[i];
        sm.ct0[i] = r.m.cell_t0[i];
    }
}

// FP64 tables of theta: (A, b, v, s, Phi(v/s)) per tuple, t0 per source.
__device__ void build_tables64(const RunDev &r, SubSmem &sm, const double *theta)
{
    for (int u = threadIdx.x; u < r.m.n_ent; u += blockDim.x) {
        const EntSrc es = r.m.ent_src[u];
        const double A = src_value(es.A, theta, r.m.consts);
        const double B = src_value(es.B, theta, r.m.consts);
        const double v = src_value(es.v, theta, r.m.consts);
        const double s = src_value(es.s, theta, r.m.consts);
        double *e = sm.e64 + 5 * u;
        e[0] = A; e[1] = A + B; e[2] = v; e[3] = s; e[4] = Phi64(v / s);
    }
    for (int q = threadIdx.x; q < r.m.n_t0; q += blockDim.x)
        sm.t064[q] = src_value(r.m.t0_src[q], theta, r.m.consts);
}

// FP32 trial constants of tuple u of theta (Ent32, device_common.cuh) and
// lg = log g, in double-float FP32 arithmetic (dfloat.h; about 1e-10
// relative, where FP64 erfc, log and divisions here cost the proposal kernel
// more than the rest of its work).  Returns false when the tuple is outside
// the FP32 form's domain (Phi(v/s) below 1e-30, or a constant not finite).
__device__ __forceinline__ bool entry32(const RunDev &r, const double *theta, int u, Ent32 &E, double &lg)
{
    const EntSrc es = r.m.ent_src[u];
    return lba_tuple32(src_value(es.A, theta, r.m.consts), src_value(es.B, theta, r.m.consts),
                       src_value(es.v, theta, r.m.consts), src_value(es.s, theta, r.m.consts), E, lg);
}

__device__ __forceinline__ float2 t0split(const RunDev &r, const double *theta, int q)
{
    const dfl t0 = df_from_double(src_value(r.m.t0_src[q], theta, r.m.consts));
    return make_float2(t0.h, t0.l);
}

// FP32 tables of proposal g from sm.theta[g] (sets sm.flag[g]).
__device__ void build_tables32(const RunDev &r, SubSmem &sm, int g)
{
    const int NE = r.m.n_ent, NT = r.m.n_t0;
    for (int u = threadIdx.x; u < NE; u += blockDim.x) {
        Ent32 E;
        double lg;
        if (!entry32(r, sm.theta + g * kMaxTheta, u, E, lg)) sm.flag[g] = 1;
        sm.e32[g * NE + u] = E;
        sm.lg[g * NE + u] = lg;
    }
    for (int q = threadIdx.x; q < NT; q += blockDim.x)
        sm.t032[g * NT + q] = t0split(r, sm.theta + g * kMaxTheta, q);
}

// Load proposal slot `slot` (theta and, in MIXED, its stored FP32 tables)
// as group member g.
// Global load; CO: through L2 only, for data another CTA of the running
// kernel wrote (published by a release/acquire pair on a flag).
template <bool CO, class T>
__device__ __forceinline__ T ldx(const T *p)
{
    if constexpr (CO) return __ldcg(p);
    else return *p;
}

template <bool CO = false>
__device__ void load_slot(const RunDev &r, size_t slot, SubSmem &sm, int g, bool mixed)
{
    const int NE = r.m.n_ent, NT = r.m.n_t0;
    for (int j = threadIdx.x; j < r.P; j += blockDim.x) sm.theta[g * kMaxTheta + j] = ldx<CO>(r.th_s + slot * r.P + j);
    if (!mixed) return;
    // the tables as float4 words: 3 per tuple
    const float4 *src = reinterpret_cast<const float4 *>(r.tab_e + slot * NE);
    float4 *dst = reinterpret_cast<float4 *>(sm.e32 + g * NE);
    for (int u = threadIdx.x; u < 3 * NE; u += blockDim.x) dst[u] = ldx<CO>(src + u);
    for (int u = threadIdx.x; u < NE; u += blockDim.x) sm.lg[g * NE + u] = ldx<CO>(r.tab_lg + slot * NE + u);
    for (int q = threadIdx.x; q < NT; q += blockDim.x) sm.t032[g * NT + q] = ldx<CO>(r.tab_t + slot * NT + q);
    if (threadIdx.x == 0) sm.flag[g] = ldx<CO>(r.tab_bad + slot);
}

// Trial log density of proposal g in FP64 (the reference form).
__device__ __forceinline__ double trial64(const RunDev &r, const SubSmem &sm, int64_t gi, int c, int K)
{
    int e8[kMaxAcc];
    for (int k = 0; k < K; ++k) e8[k] = sm.cent[c * K + k];
    return lba_logdens64(r.rt64[gi] - sm.t064[sm.ct0[c]], e8, K, sm.cw[c], sm.e64);
}

// Log-likelihood sums over trials [i0, i1) of subject level l for the ng
// (<= kGroup) proposals loaded in sm, on the whole CTA; out[g] valid on all
// threads.  MIXED: FP32 per trial, each trial's data read once for the whole
// group; FP64 tables are built only for a proposal some trial of which needs
// the FP64 form, and only those trials use it.
// DDM entries of proposal g from its theta (the responding boundary's
// mirrored values; see ddm_logdens64).
__device__ void ddm_build(const RunDev &r, SubSmem &sm, int g, const double *theta)
{
    const int ND = r.m.n_dent;
    for (int u = threadIdx.x; u < ND; u += blockDim.x) {
        const int32_t *q = r.m.ddm_src + 9 * u;
        double v8[8];
        for (int j = 0; j < 8; ++j) v8[j] = src_value(q[j], theta, r.m.consts);
        ddm_entry(v8, q[8] == 1, sm.d64 + 8 * (g * ND + u), sm.d32 + 8 * (g * ND + u));
    }
}

// group_loglik for the diffusion model, into parts[g] (valid on all threads
// on return).  MIXED: FP32 per trial with FP64 re-evaluation where
// ddm_logdens32 declines, each term added in 2^-32 fixed point (an exact
// integer sum, which no block size or grouping changes, as for the LBA);
// FP64: a plain FP64 sum.
__device__ void ddm_group_loglik(const RunDev &r, int l, int i0, int i1, SubSmem &sm, int ng, bool mixed,
                                 JobPart *parts)
{
    for (int g = 0; g < ng; ++g) ddm_build(r, sm, g, sm.theta + g * kMaxTheta);
    if (threadIdx.x < ng) parts[threadIdx.x] = JobPart{0, 0, 0, 0.0};
    __syncthreads();
    const int64_t base = r.offs[l] + i0;
    const int n = i1 - i0, K = r.m.n_acc, ND = r.m.n_dent;
    double acc[kGroup];
    long long fx[kGroup];
#pragma unroll
    for (int g = 0; g < kGroup; ++g) { acc[g] = 0.0; fx[g] = 0; }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int u = sm.cent[r.cell[base + i] * K];
        const float2 rt = r.rt32[base + i];
#pragma unroll
        for (int g = 0; g < kGroup; ++g) {
            if (g >= ng) break;
            float ld;
            if (!mixed) {
                acc[g] += ddm_logdens64(r.rt64[base + i], sm.d64 + 8 * (g * ND + u));
            } else if (ddm_logdens32(rt.x, rt.y, sm.d32 + 8 * (g * ND + u), ld)) {
                fx[g] += __float2ll_rn(ld * kFixScale);          // |ld| < 89
            } else {
                const double x = ddm_logdens64(r.rt64[base + i], sm.d64 + 8 * (g * ND + u));
                if (fabs(x) < 1073741824.0) fx[g] += __double2ll_rn(x * 4294967296.0);
                else acc[g] += x;
            }
        }
    }
    for (int g = 0; g < ng; ++g) {
        if (mixed) warp_flush(parts[g], fx[g], 0, 0);
        const double t = block_sum(acc[g], sm.red);   // its barriers also order the atomics
        if (threadIdx.x == 0) parts[g].f64 = t;
    }
    __syncthreads();
}

// group_loglik's per-proposal results and partial sums, in sm.red after the
// 33 doubles block_sum uses.
constexpr int kResOff = 40;
static_assert(kResOff + kGroup + kGroup * sizeof(JobPart) / sizeof(double) <= kRedDoubles,
              "sm.red holds block_sum's partials, the results and the job parts");
__device__ __forceinline__ double *group_res(const SubSmem &sm) { return sm.red + kResOff; }
__device__ __forceinline__ JobPart *job_parts(const SubSmem &sm)
{
    return reinterpret_cast<JobPart *>(sm.red + kResOff + kGroup);
}

// The FP32 pass of group_loglik over trials [base, base + n) for K
// accumulators (K = 0: the design's count at run time) and the ng proposals
// loaded in sm, into parts[g] (zeroed by the caller).  The work is split
// into chunks of 32 consecutive trials of one proposal, chunk c = g nch + j
// (nch chunks per proposal), and warp w takes chunks w, w + nw, ...: every
// warp is busy while there are chunks, whatever the number of proposals or
// trials.  Each trial adds its mantissa log in fixed point (lm 2^32 rounded
// to an integer; |lm| < 0.35, so it fits an int) and its binary exponent;
// a warp adds its partials to the proposal's JobPart when it moves on to the
// next proposal.  The sums are exact integers, so a proposal's result is
// the same for any block size, grouping or kernel.  A trial the FP32 form
// declines is listed for FP64.
template <int K>
__device__ __forceinline__ void lba_group_loop32(const RunDev &r, int64_t base, int n, const SubSmem &sm, int ng,
                                                 JobPart *parts)
{
    const int NE = r.m.n_ent, NT = r.m.n_t0, KR = r.m.n_acc;
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int nch = (n + 31) >> 5;
    if (nch == 0) return;
    int g = 0, j = threadIdx.x >> 5;                 // this warp's chunk (g, j), warp-uniform
    while (j >= nch && g < ng) { j -= nch; ++g; }
    long long s = 0;
    int e = 0, nf = 0;
#pragma unroll 1
    while (g < ng) {
        if (sm.flag[g] == 0) {
            const Ent32 *E = sm.e32 + g * NE;
            const float2 *T0 = sm.t032 + g * NT;
            const int i = (j << 5) + lane;
            if (i < n) {
                const int c = r.cell[base + i];
                const float2 rt = r.rt32[base + i];
                const float2 t0 = T0[sm.ct0[c]];
                int ex;
                float lm;
                bool good;
                if (t_before(rt, t0)) {
                    // the density floor as the winner's tuple stores it (its log g
                    // comes with the cell constant)
                    const Ent32 &W = E[sm.cent[c * KR]];
                    ex = (int)W.a.y;
                    lm = W.b.y;
                    good = true;
                } else if constexpr (K > 0) {
                    int ent[K];
#pragma unroll
                    for (int k = 0; k < K; ++k) ent[k] = sm.cent[c * K + k];
                    good = lba_ld32<K>(rt, t0, ent, E, ex, lm);
                } else {
                    good = lba_ld32_n(rt, t0, sm.cent + c * KR, KR, E, ex, lm);
                }
                if (good) {
                    s += (long long)__float2int_rn(lm * kFixScale);
                    e += ex;
                } else {
                    ++nf;
                    const int pos = atomicAdd(sm.fbn, 1);
                    if (pos < kFbCap) sm.fb[pos] = (i << 2) | g;
                }
            }
        }
        const int g0 = g;
        j += nw;
        while (j >= nch && g < ng) { j -= nch; ++g; }
        if (g != g0) {
            warp_flush(parts[g0], s, e, nf);
            s = 0;
            e = 0;
            nf = 0;
        }
    }
}

// MODEL: kAnyModel dispatches on the design's model type; kLbaOnly and
// kDdmOnly compile one density only (the per-model kernel instantiations),
// kLba4 only the 4-accumulator LBA loop.
constexpr int kAnyModel = 0, kLbaOnly = 1, kDdmOnly = 2, kLba4 = 3;

// Partial log-likelihood sums of trials [i0, i1) of subject level l for the
// ng (<= kGroup) proposals loaded in sm, on the whole CTA, into parts[g]
// (shared memory; valid on all threads on return).  MIXED LBA: the FP32
// pass (lba_group_loop32) adds each trial's binary exponent and fixed-point
// mantissa log to parts[g]; a trial's log density is log g_w + e ln 2 +
// log m, and log g_w is NOT included here (group_cell_const adds it once per
// cell).  FP64 tables are built only for a proposal some trial of which
// needs the FP64 form, and only those trials use it; their FP64 value, less
// log g_w, is added to parts[g].s in the same fixed point (a value of 2^30
// or more in magnitude, or not finite, to parts[g].f64).  A proposal outside
// the FP32 form's domain, FP64 and the diffusion model: parts[g].f64 only.
template <int MODEL = kAnyModel>
__device__ void group_chunk(const RunDev &r, int l, int i0, int i1, SubSmem &sm, int ng, bool mixed, JobPart *parts)
{
    const int64_t base = r.offs[l] + i0;
    const int n = i1 - i0;
    bool ddm = MODEL == kDdmOnly;
    if constexpr (MODEL == kAnyModel) ddm = r.m.model_type == kModelDdm;
    if (ddm) {
        ddm_group_loglik(r, l, i0, i1, sm, ng, mixed, parts);
        return;
    }
    const int K = r.m.n_acc;
    const int NE = r.m.n_ent, NT = r.m.n_t0;
    if (!mixed) {
        for (int g = 0; g < ng; ++g) {
            build_tables64(r, sm, sm.theta + g * kMaxTheta);
            __syncthreads();
            double acc = 0.0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) acc += trial64(r, sm, base + i, r.cell[base + i], K);
            const double tot = block_sum(acc, sm.red);
            if (threadIdx.x == 0) parts[g] = JobPart{0, 0, 0, tot};
        }
        __syncthreads();
        return;
    }
    if (threadIdx.x == 0) *sm.fbn = 0;
    if (threadIdx.x < ng) parts[threadIdx.x] = JobPart{0, 0, 0, 0.0};
    __syncthreads();
    switch (MODEL == kLba4 ? 4 : K) {
    case 2: if constexpr (MODEL != kLba4) lba_group_loop32<2>(r, base, n, sm, ng, parts); break;
    case 3: if constexpr (MODEL != kLba4) lba_group_loop32<3>(r, base, n, sm, ng, parts); break;
    case 4: lba_group_loop32<4>(r, base, n, sm, ng, parts); break;
    default: if constexpr (MODEL != kLba4) lba_group_loop32<0>(r, base, n, sm, ng, parts); break;
    }
    __syncthreads();
    bool anyfb = false;
    for (int g = 0; g < ng; ++g) anyfb |= parts[g].nf > 0 || sm.flag[g] != 0;
    if (!anyfb) return;
    // FP64 for the listed trials (log g_w taken back out: the cell constant
    // counts it for every trial), or for every trial of a proposal outside
    // the FP32 form's domain
    for (int g = 0; g < ng; ++g) {
        const bool usable = sm.flag[g] == 0;
        const int nfg = parts[g].nf;
        if (usable && nfg == 0) continue;           // uniform over the block
        build_tables64(r, sm, sm.theta + g * kMaxTheta);
        if (r.stats && threadIdx.x == 0)
            atomicAdd(&r.stats[ST_FALLBACKS], (unsigned long long)(usable ? nfg : n));
        __syncthreads();
        const int fbn = *sm.fbn;
        double acc = 0.0;
        auto add_fixed = [&](double x) {
            if (fabs(x) < 1073741824.0)
                atomicAdd(reinterpret_cast<unsigned long long *>(&parts[g].s),
                          (unsigned long long)__double2ll_rn(x * 4294967296.0));
            else
                acc += x;
        };
        if (!usable) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) acc += trial64(r, sm, base + i, r.cell[base + i], K);
        } else if (fbn <= kFbCap) {
            for (int q = threadIdx.x; q < fbn; q += blockDim.x) {
                const int e = sm.fb[q];
                if ((e & 3) != g) continue;
                const int i = e >> 2, c = r.cell[base + i];
                add_fixed(trial64(r, sm, base + i, c, K) - sm.lg[g * NE + sm.cent[c * K]]);
            }
        } else {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int c = r.cell[base + i];
                const float2 t0 = sm.t032[g * NT + sm.ct0[c]];
                int ex;
                float lm;
                if (t_before(r.rt32[base + i], t0) ||
                    lba_ld32_n(r.rt32[base + i], t0, sm.cent + c * K, K, sm.e32 + g * NE, ex, lm))
                    continue;
                add_fixed(trial64(r, sm, base + i, c, K) - sm.lg[g * NE + sm.cent[c * K]]);
            }
        }
        const double tot = block_sum(acc, sm.red);  // its barriers also order the atomics
        if (threadIdx.x == 0) parts[g].f64 += tot;
        __syncthreads();
    }
}

// The per-cell FP64 constant of a MIXED LBA proposal, on one warp (every
// lane gets it): sum over cells of n_c log g_w (lg [n_ent], the proposal's
// log g of each tuple).
__device__ __forceinline__ double group_cell_const(const RunDev &r, int l, const double *lg, const uint8_t *cent)
{
    const int lane = threadIdx.x & 31, K = r.m.n_acc;
    const int32_t *cnt = r.cell_cnt + (size_t)l * r.m.n_cell;
    double dc = 0.0;
    for (int c = lane; c < r.m.n_cell; c += 32) {
        const int nc = cnt[c];
        if (nc) dc = __fma_rn((double)nc, lg[cent[c * K]], dc);
    }
    for (int o = 16; o > 0; o >>= 1) dc += __shfl_down_sync(0xffffffffu, dc, o);
    return __shfl_sync(0xffffffffu, dc, 0);
}

// The sum of a proposal from its parts and its cell constant (dc = 0 where
// the FP32 form was not used).
__device__ __forceinline__ double part_total(const JobPart &p, double dc)
{
    // explicit roundings: the same value in every kernel that forms it
    return __dadd_rn(__dadd_rn(__dadd_rn(dc, __dmul_rn((double)p.s, kFixUnit)), __dmul_rn(kLn2, (double)p.e)),
                     p.f64);
}

// Log-likelihood sums of the subject's trials for the ng (<= kGroup)
// proposals loaded in sm, on the whole CTA; out[g] valid on all threads.
template <int MODEL = kAnyModel>
__device__ void group_loglik(const RunDev &r, int l, SubSmem &sm, int ng, bool mixed, double *out)
{
    const int n = (int)(r.offs[l + 1] - r.offs[l]);
    JobPart *parts = job_parts(sm);
    double *res = group_res(sm);
    group_chunk<MODEL>(r, l, 0, n, sm, ng, mixed, parts);
    bool lba = MODEL != kDdmOnly;
    if constexpr (MODEL == kAnyModel) lba = r.m.model_type != kModelDdm;
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int g = wid; g < ng; g += nw) {
        const double dc = (mixed && lba && sm.flag[g] == 0)
                              ? group_cell_const(r, l, sm.lg + g * r.m.n_ent, sm.cent) : 0.0;
        if ((threadIdx.x & 31) == 0) res[g] = part_total(parts[g], dc);
    }
    __syncthreads();
    for (int g = 0; g < ng; ++g) out[g] = res[g];
    __syncthreads();
}

// Evaluate the log-likelihoods of proposal slots `slots[0..m)` of level l on
// the whole CTA, kGroup at a time; results to ll_s (and to lls[k] when given).
template <bool CO = false, int MODEL = kAnyModel>
__device__ void eval_slots(const RunDev &r, int l, const int *slots, int m, SubSmem &sm, bool mixed,
                           double *lls_sm)
{
    const int N = (int)(r.offs[l + 1] - r.offs[l]);
    for (int g0 = 0; g0 < m; g0 += kGroup) {
        const int ng = min(kGroup, m - g0);
        for (int g = 0; g < ng; ++g) load_slot<CO>(r, (size_t)l * r.CS + slots[g0 + g], sm, g, mixed);
        __syncthreads();
        double out[kGroup];
        group_loglik<MODEL>(r, l, sm, ng, mixed, out);
        if (threadIdx.x == 0) {
            for (int g = 0; g < ng; ++g) {
                r.ll_s[(size_t)l * r.CS + slots[g0 + g]] = out[g];
                if (lls_sm) lls_sm[slots[g0 + g]] = out[g];
            }
            atomicAdd(&r.stats[ST_TRIALS], (unsigned long long)N * ng);
        }
        __syncthreads();
    }
}

// Store the FP32 tables of proposal slot `slot` from theta (threads of the
// CTA in parallel over (slot, entry) are the caller's; this is one entry).
// entry32 as a call: its double-float chain then takes no registers from the
// kernels that build tables beside other work (the ordered resolve: 5% of a
// sweep of the 256-subject workload)
__device__ __noinline__ bool entry32_call(const RunDev &r, const double *theta, int u, Ent32 &E, double &lg)
{
    return entry32(r, theta, u, E, lg);
}

__device__ __forceinline__ void store_entry(const RunDev &r, size_t slot, const double *theta, int u)
{
    const int NE = r.m.n_ent, NT = r.m.n_t0;
    if (u < NE) {
        Ent32 E;
        double lg;
        if (!entry32_call(r, theta, u, E, lg)) atomicOr(&r.tab_bad[slot], 1);
        r.tab_e[slot * NE + u] = E;
        r.tab_lg[slot * NE + u] = lg;
    } else {
        r.tab_t[slot * NT + (u - NE)] = t0split(r, theta, u - NE);
    }
}

// One prior term of subject parameter j (fixed table or the truncated
// normal of phi chain `owner`).
__device__ __forceinline__ double prior_j(const RunDev &r, double x, int j, int owner)
{
    if (r.prior) return prior_term(r.prior + kPriorRow * j, x);
    const double *pt = r.phi_tab + ((size_t)owner * r.P + j) * 3;   // (mu, 1/sigma, c)
    if (x < r.pp_bounds[2 * j] || x > r.pp_bounds[2 * j + 1] || !(pt[1] > 0.0)) return -INFINITY;
    const double z = (x - pt[0]) * pt[1];
    return -0.5 * z * z + pt[2];
}

// Log prior of theta on one warp (lanes over parameters, fixed-order sum).
__device__ __forceinline__ double warp_prior(const RunDev &r, const double *th, int owner)
{
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    for (int j = lane; j < r.P; j += 32) s += prior_j(r, th[j], j, owner);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    return __shfl_sync(0xffffffffu, s, 0);
}

// --------------------------------------------------------- subject kernels
// k_sub_propose: pass type, partners, stored draws and proposals of every
// chain of every subject level, with their log priors and FP32 tables.
// grid = S.
// In a hierarchical sweep the subject proposals are built while the phi
// level runs (defer_prior): the prior, the only term that reads phi, is
// scored after both, at the start of k_sub_resolve, and a proposal is
// evaluated when it lies in the prior's support, which does not depend on phi.
__device__ __forceinline__ bool in_support(const RunDev &r, const double *th)
{
    for (int j = 0; j < r.P; ++j)
        if (!(th[j] >= r.pp_bounds[2 * j] && th[j] <= r.pp_bounds[2 * j + 1])) return false;
    return true;
}

// Shared scratch of propose_level: (C + 2) uniforms (reused for the
// migration cascade, hence at least P), then four int arrays of C.
__host__ __device__ inline int prop_cap(int C, int P) { return (C + 2 > P) ? C + 2 : P; }
__host__ __device__ inline size_t prop_scratch_bytes(int C, int P)
{
    return sizeof(double) * (size_t)prop_cap(C, P) + sizeof(int) * 4 * (size_t)C;
}

// Pass type, partners, stored draws and proposals of subject level l for
// iteration `it` (the body of k_sub_propose; all threads of the CTA).
template <bool CO = false>
__device__ void propose_level(const RunDev &r, int l, int64_t it, int pass, bool defer_prior, char *scratch)
{
    __shared__ int s_type, s_n, s_para;
    const int lev = r.level0 + l;
    const int C = r.C, P = r.P, CS = r.CS;
    double *s_u = (double *)scratch;
    int *s_sub = (int *)(s_u + prop_cap(C, P));
    int *s_perm = s_sub + C;
    int *s_pa = s_perm + C;
    int *s_pb = s_pa + C;
    if (threadIdx.x == 0) {
        int type = PASS_CROSS, para = -1;
        if (r.loop == LOOP_HCHAINS) {
            const bool mig = uniform(r.ds, it, lev, pass, 0) < r.sub_mig;
            type = mig ? PASS_MIG : PASS_CROSS;
            para = r.sub_blocked ? pass : -1;
        } else if (pass == 0) {
            const bool mig = uniform(r.ds, it, lev, 0, 0) < r.sub_mig;
            r.migrated[l] = mig;
            type = mig ? PASS_MIG : PASS_CROSS;
            para = (!mig && r.sub_blocked) ? 0 : -1;
        } else {
            type = r.migrated[l] ? PASS_SKIP : PASS_CROSS;
            para = pass;
        }
        s_type = type;
        s_para = para;
    }
    __syncthreads();
    const int type = s_type, para = s_para;
    if (type == PASS_MIG) {
        for (int q = 1 + threadIdx.x; q < C + 2; q += blockDim.x) s_u[q] = uniform(r.ds, it, lev, pass, q);
        __syncthreads();
        if (threadIdx.x == 0) {
            s_n = subchains_pick(C, s_u, s_perm);
            atomicAdd(&r.stats[ST_MIGRATIONS], 1ull);
        }
        __syncthreads();
        subchains_sort(s_perm, s_n, s_sub);
    } else if (threadIdx.x == 0) {
        s_n = (type == PASS_SKIP) ? 0 : C;
    }
    __syncthreads();
    const int n = s_n;
    if (threadIdx.x == 0) {
        r.ptype[l] = type;
        r.nstep[l] = n;
        r.rs_para[l] = para;
    }
    if (n == 0) return;
    const int nloop = (r.loop == LOOP_HCHAINS) ? r.half : r.Pn;
    const double *th = r.th + (size_t)l * C * P;
    double *ths = r.th_s + (size_t)l * CS * P;
    double *jit = r.jit + (size_t)l * C * P;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        if (type == PASS_CROSS) {
            int a, b;
            partners(r, it, lev, pass, k, a, b);
            s_pa[k] = a;
            s_pb[k] = b;
            r.partner[((size_t)l * C + k) * 2] = a;
            r.partner[((size_t)l * C + k) * 2 + 1] = b;
        } else {
            r.sub[(size_t)l * C + k] = s_sub[k];
        }
        r.accu[(size_t)l * C + k] = accept_draw(r, it, lev, pass, k);
        r.tab_bad[(size_t)l * CS + k] = 0;
    }
    __syncthreads();
    // proposals, one thread per (step, parameter)
    for (int q = threadIdx.x; q < n * P; q += blockDim.x) {
        const int k = q / P, j = q % P;
        const int src = (type == PASS_CROSS) ? k : s_sub[k];
        const double ts = ldx<CO>(th + (size_t)src * P + j);
        double out = ts;
        if (updated(j, para, nloop)) {
            const double jv = jitter_draw(r, it, lev, pass, k, j);
            jit[(size_t)k * P + j] = jv;
            out = (type == PASS_CROSS)
                      ? cross_comp(r.gamma, ts, ldx<CO>(th + (size_t)s_pa[k] * P + j),
                                   ldx<CO>(th + (size_t)s_pb[k] * P + j), jv)
                      : __dadd_rn(ts, jv);
        }
        ths[(size_t)k * P + j] = out;
    }
    __syncthreads();
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (defer_prior) {
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            r.ll_s[(size_t)l * CS + k] = 0.0;
            r.need[(size_t)l * CS + k] = in_support(r, ths + (size_t)k * P) ? 1 : 0;
        }
    } else {
        for (int k = wid; k < n; k += nw) {
            const int owner = (type == PASS_CROSS) ? k : s_sub[k];
            const double lp = warp_prior(r, ths + (size_t)k * P, owner);
            if ((threadIdx.x & 31) == 0) {
                r.lp_s[(size_t)l * CS + k] = lp;
                r.ll_s[(size_t)l * CS + k] = 0.0;
                r.need[(size_t)l * CS + k] = (lp > -INFINITY) ? 1 : 0;
            }
        }
    }
    // migration: the cascade V_s = V_(s-1) + jit_s from V_0 = proposal 0, the
    // proposal step s gets when every step before it accepts (slots C + s)
    const int nv = (type == PASS_MIG) ? n : 0;
    for (int w = nv + threadIdx.x; w < C; w += blockDim.x) r.need[(size_t)l * CS + C + w] = 0;
    if (nv) {
        // the running sums in shared memory (s_u, whose draws are consumed),
        // then one parallel store; jit was written above by this block
        double *s_v = s_u;
        const int kCap = prop_cap(C, P);
        for (int w0 = 0; w0 < nv; w0 += kCap / P) {
            const int wn = min(nv - w0, kCap / P);
            __syncthreads();
            for (int q = threadIdx.x; q < wn * P; q += blockDim.x) s_v[q] = jit[(size_t)(w0 + q / P) * P + q % P];
            __syncthreads();
            for (int j = threadIdx.x; j < P; j += blockDim.x) {
                double v = (w0 == 0) ? ldx<CO>(th + (size_t)s_sub[0] * P + j) : ths[(size_t)(C + w0 - 1) * P + j];
                const bool up = updated(j, para, nloop);
                for (int w = 0; w < wn; ++w) {
                    if (up) v = __dadd_rn(v, s_v[w * P + j]);
                    s_v[w * P + j] = v;
                }
            }
            __syncthreads();
            for (int q = threadIdx.x; q < wn * P; q += blockDim.x)
                ths[(size_t)(C + w0 + q / P) * P + q % P] = s_v[q];
            __syncthreads();
        }
        for (int w = threadIdx.x; w < nv; w += blockDim.x) r.tab_bad[(size_t)l * CS + C + w] = 0;
        __syncthreads();
        if (defer_prior) {
            // V_0 equals proposal 0, already evaluated
            for (int w = threadIdx.x; w < nv; w += blockDim.x) {
                r.ll_s[(size_t)l * CS + C + w] = 0.0;
                r.need[(size_t)l * CS + C + w] =
                    (w > 0 && in_support(r, ths + (size_t)(C + w) * P)) ? 1 : 0;
            }
        } else {
            for (int w = wid; w < nv; w += nw) {
                // V_0 equals proposal 0, already evaluated
                const double lp = (w == 0) ? -INFINITY : warp_prior(r, ths + (size_t)(C + w) * P, s_sub[w]);
                if ((threadIdx.x & 31) == 0) {
                    r.lp_s[(size_t)l * CS + C + w] = lp;
                    r.ll_s[(size_t)l * CS + C + w] = 0.0;
                    r.need[(size_t)l * CS + C + w] = (lp > -INFINITY) ? 1 : 0;
                }
            }
        }
    }
    if (r.prec != PREC_MIXED) return;
    const int NU = r.m.n_ent + r.m.n_t0;
    for (int q = threadIdx.x; q < (n + nv) * NU; q += blockDim.x) {
        const int k0 = q / NU, u = q % NU;
        const int k = (k0 < n) ? k0 : C + (k0 - n);
        store_entry(r, (size_t)l * CS + k, ths + (size_t)k * P, u);
    }
}

// grid = S.  fused: a level k_sub_step already proposed for this iteration
// (ready[l] == iteration) is skipped, and a level proposed here gets its
// spec-item counter cleared and its ready stamp; block 0 also clears
// k_sub_step's claim counters.
__global__ void __launch_bounds__(kProposeThreads) k_sub_propose(RunDev r, int pass, int defer_prior, int fused)
{
    extern __shared__ __align__(16) char smem_raw[];
    const int l = blockIdx.x;
    const int it = *r.iter;
    if (fused) {
        if (l == 0 && threadIdx.x < kCtlN) r.ctl[threadIdx.x] = 0;
        if (r.ready[l] == it) return;
    }
    propose_level(r, l, it, pass, defer_prior != 0, smem_raw);
    if (fused && threadIdx.x == 0) {
        r.spec_cnt[l] = 0;
        r.ready[l] = it;
    }
}

// k_sub_loglik: the hot kernel.  One CTA per work item = up to kGroup
// proposals of one subject, items in descending trial-count order (longest
// first keeps the tail short).  item = level * CS + first slot.
template <int MINB, int MODEL>
__global__ void __launch_bounds__(kLikThreads, MINB) k_sub_loglik(RunDev r, const int32_t *items, int group)
{
    extern __shared__ __align__(16) char smem_raw[];
    __shared__ int s_slots[kGroup];
    __shared__ int s_m;
    const int32_t item = items[blockIdx.x];
    const int l = item / r.CS, k0 = item % r.CS;
    const int n = r.nstep[l];
    if (threadIdx.x == 0) {
        int m = 0;
        const int kend = (k0 < r.C) ? min(n, k0 + group) : min(r.C + n, k0 + group);
        for (int k = k0; k < kend; ++k)
            if (r.need[(size_t)l * r.CS + k]) s_slots[m++] = k;
        s_m = m;
    }
    __syncthreads();
    if (s_m == 0) return;
    SubSmem sm = carve(smem_raw, r.m);
    load_design(r, sm);
    eval_slots<false, MODEL>(r, l, s_slots, s_m, sm, r.prec == PREC_MIXED, nullptr);
}

// Spec item k of level l: the crossover steps [k g, k g + g) for k < ceil(C / g),
// then the migration cascade slots C + [..).  Writes the slots that need an
// evaluation to slots[] and returns their count (one thread).
template <bool CO>
__device__ int spec_item_slots(const RunDev &r, int l, int k, int group, int *slots)
{
    const int nic = (r.C + group - 1) / group;
    const int n = ldx<CO>(r.nstep + l);
    int k0, kend;
    if (k < nic) {
        k0 = k * group;
        kend = min(n, k0 + group);
    } else {
        k0 = r.C + (k - nic) * group;
        kend = min(r.C + n, k0 + group);
    }
    int m = 0;
    for (int q = k0; q < kend; ++q)
        if (ldx<CO>(r.need + (size_t)l * r.CS + q)) slots[m++] = q;
    return m;
}

// k_sub_spec_rest: the spec items k_sub_step left unclaimed.  blocks_per_level
// CTAs per level (levels largest first), each claiming items from the level's
// counter until none is left.
template <int MINB, int MODEL>
__global__ void __launch_bounds__(kLikThreads, MINB)
k_sub_spec_rest(RunDev r, int group, int blocks_per_level)
{
    extern __shared__ __align__(16) char smem_raw[];
    __shared__ int s_slots[kGroup];
    __shared__ int s_m, s_k;
    const int l = r.sub_order[blockIdx.x / blocks_per_level];
    const int n_item = 2 * ((r.C + group - 1) / group);
    SubSmem sm = carve(smem_raw, r.m);
    bool loaded = false;
    for (;;) {
        if (threadIdx.x == 0) {
            int k, m = 0;
            do {
                k = atomicAdd(r.spec_cnt + l, 1);
                if (k < n_item) m = spec_item_slots<false>(r, l, k, group, s_slots);
            } while (k < n_item && m == 0);
            s_k = k;
            s_m = m;
        }
        __syncthreads();
        if (s_k >= n_item) return;
        if (!loaded) {
            load_design(r, sm);
            loaded = true;
        }
        eval_slots<false, MODEL>(r, l, s_slots, s_m, sm, r.prec == PREC_MIXED, nullptr);
        __syncthreads();
    }
}

// Evaluate slots[0..m) of subject l over all its trials, kGroup at a time;
// out[slots[q] - out_off] and ll_s receive slot q's log-likelihood.
__device__ void eval_direct(const RunDev &r, int l, const int *slots, int m, SubSmem &sm, bool mixed,
                            double *out, int out_off)
{
    const int N = (int)(r.offs[l + 1] - r.offs[l]);
    for (int g0 = 0; g0 < m; g0 += kGroup) {
        const int ng = min(kGroup, m - g0);
        for (int g = 0; g < ng; ++g) load_slot(r, (size_t)l * r.CS + slots[g0 + g], sm, g, mixed);
        __syncthreads();
        double o[kGroup];
        group_loglik(r, l, sm, ng, mixed, o);
        if (threadIdx.x == 0) {
            for (int g = 0; g < ng; ++g) {
                out[slots[g0 + g] - out_off] = o[g];
                r.ll_s[(size_t)l * r.CS + slots[g0 + g]] = o[g];
            }
            atomicAdd(&r.stats[ST_TRIALS], (unsigned long long)N * ng);
        }
        __syncthreads();
    }
}

struct ResSmem {
    double *lp, *ll;        // [C] current state
    double *lps, *lls;      // [C] proposal values of each step
    double *cur;            // [C] migration: log posterior of each step's destination
    double *vlp, *vll;      // [C] migration variants
    double *accu;           // [C]
    int *pa, *pb;           // [C] partners (crossover) / pa = subset (migration)
    int *acc, *accslot;     // [C] accepted steps of a scan and the slot they used
    int *list;              // [C + kVariants] steps / slots to evaluate
    int *misc;              // 8
    int *vr, *vs;           // [kVariants] migration variant w: last rejected step (-1: none
                            // since the round began) and the step it serves
    int *warp;              // [33] per-warp counts of a block compaction
    int16_t *ver;           // [C]
    uint8_t *mod, *dec;     // [C] step outcome in the sweep, Metropolis outcome of its proposal
    uint8_t *cdec;          // [C] migration: outcome of the cascade value of step s
    uint8_t *vdec;          // [kVariants] migration: outcome of variant w
};

__host__ __device__ inline size_t res_layout(int C, size_t off[8])
{
    size_t o = 0;
    off[0] = o; o += sizeof(double) * 8 * (size_t)C;                     // lp .. accu
    off[1] = o; o += sizeof(int) * (4 * (size_t)C + C + kVariants + 8 + 2 * kVariants + 33);
    off[2] = o; o += sizeof(int16_t) * (size_t)C;
    off[3] = o; o += 3 * (size_t)C + kVariants;
    return align_up(o, 16);
}
__host__ __device__ inline size_t res_smem_bytes(int C)
{
    size_t off[8];
    return res_layout(C, off);
}
__device__ ResSmem carve_res(char *base, int C)
{
    size_t off[8];
    res_layout(C, off);
    ResSmem s;
    s.lp = (double *)(base + off[0]);
    s.ll = s.lp + C;
    s.lps = s.ll + C;
    s.lls = s.lps + C;
    s.cur = s.lls + C;
    s.accu = s.cur + C;
    s.vlp = s.accu + C;
    s.vll = s.vlp + C;
    s.pa = (int *)(base + off[1]);
    s.pb = s.pa + C;
    s.acc = s.pb + C;
    s.accslot = s.acc + C;
    s.list = s.accslot + C;
    s.misc = s.list + C + kVariants;
    s.vr = s.misc + 8;
    s.vs = s.vr + kVariants;
    s.warp = s.vs + kVariants;
    s.ver = (int16_t *)(base + off[2]);
    s.mod = (uint8_t *)(base + off[3]);
    s.dec = s.mod + C;
    s.cdec = s.dec + C;
    s.vdec = s.cdec + C;
    return s;
}

// Smallest i in [lo, hi) with pred(i), else hi.  All threads; every thread
// gets the result.
template <class F>
__device__ __forceinline__ int block_first(int lo, int hi, F pred, int *tmp)
{
    if (threadIdx.x == 0) *tmp = hi;
    __syncthreads();
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x)
        if (pred(i)) atomicMin(tmp, i);
    __syncthreads();
    const int r = *tmp;
    __syncthreads();
    return r;
}

// The i in [lo, hi) with pred(i), ascending, into out; returns their count.
// All threads (blockDim.x a multiple of 32, at most 1024).
template <class F>
__device__ __forceinline__ int block_compact(int lo, int hi, F pred, int *out, int *warp)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int total = 0;
    for (int b0 = lo; b0 < hi; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        const bool p = i < hi && pred(i);
        const unsigned m = __ballot_sync(0xffffffffu, p);
        if (lane == 0) warp[wid] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int w = 0; w < nw; ++w) {
                const int c = warp[w];
                warp[w] = acc;
                acc += c;
            }
            warp[32] = acc;
        }
        __syncthreads();
        if (p) out[total + warp[wid] + __popc(m & ((1u << lane) - 1u))] = i;
        total += warp[32];
        __syncthreads();
    }
    return total;
}

// The subject's jitter rows are staged in shared memory when they fit.
constexpr size_t kJitStage = 32768;
__host__ __device__ inline size_t jit_stage_bytes(int C, int P)
{
    const size_t b = (size_t)C * P * sizeof(double);
    return b <= kJitStage ? b : 0;
}

// Copy the rows of the steps accepted by the last scan into the state.
__device__ void write_accepts(const RunDev &r, int l, int type, int n, ResSmem &rs, int na)
{
    const int C = r.C, P = r.P;
    const size_t lc = (size_t)l * C, ls = (size_t)l * r.CS;
    for (int q = threadIdx.x; q < na * P; q += blockDim.x) {
        const int a = q / P, j = q % P;
        const int i = rs.acc[a];
        const int dst = (type == PASS_CROSS) ? i : ((i + 1 == n) ? rs.pa[0] : rs.pa[i + 1]);
        r.th[(lc + dst) * P + j] = r.th_s[(ls + rs.accslot[a]) * P + j];
    }
    for (int a = threadIdx.x; a < na; a += blockDim.x) {
        const int i = rs.acc[a];
        const int dst = (type == PASS_CROSS) ? i : ((i + 1 == n) ? rs.pa[0] : rs.pa[i + 1]);
        const int sl = rs.accslot[a];
        const double lpv = (sl < C) ? rs.lps[sl] : rs.vlp[sl - C];
        const double llv = (sl < C) ? rs.lls[sl] : rs.vll[sl - C];
        r.lp[lc + dst] = lpv;
        r.ll[lc + dst] = llv;
        rs.lp[dst] = lpv;
        rs.ll[dst] = llv;
    }
    if (threadIdx.x == 0 && na) atomicAdd(&r.stats[ST_ACCEPTS], (unsigned long long)na);
    __syncthreads();
}

// resolve_level: ordered decisions of one subject level (src/de.cpp:111-199,
// 567-665), by one CTA.  Decisions are taken from the speculative results
// while the proposal a step would get in sequence is the one evaluated; a
// crossover chain whose partner moved earlier in the sweep is re-proposed
// from the current state and re-evaluated with the other stale chains of its
// round.  Migration steps: the first round uses the start-of-pass proposals
// (valid after a rejection) and the cascade from step 0 (valid while every
// step accepts); later rounds evaluate the most likely values the next steps
// can need.
__device__ void resolve_level(const RunDev &r, int l, SubSmem &sm, char *smem_raw, bool score_priors)
{
    const int type = r.ptype[l];
    if (type == PASS_SKIP) return;
    const int n = r.nstep[l];
    const int C = r.C, P = r.P;
    const size_t lc = (size_t)l * C, ls = (size_t)l * r.CS;
    const bool mixed = r.prec == PREC_MIXED;
    ResSmem rs = carve_res(smem_raw + sub_smem_bytes(r.m), C);
    const unsigned long long t_beg = (threadIdx.x == 0) ? global_ns() : 0ull;
    if (score_priors) {
        // deferred priors of the pass's proposals (and migration cascade),
        // with the phi chains of this sweep: a warp per slot
        const int nv = (type == PASS_MIG) ? n : 0;
        const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int q = wid; q < n + nv; q += nw) {
            const int slot = (q < n) ? q : C + (q - n);
            const int k = (q < n) ? q : q - n;
            const int owner = (type == PASS_CROSS) ? k : r.sub[lc + k];
            const double lp = (slot == C) ? -INFINITY : warp_prior(r, r.th_s + (ls + slot) * P, owner);
            if ((threadIdx.x & 31) == 0) r.lp_s[ls + slot] = lp;
        }
        __syncthreads();
    }
    for (int k = threadIdx.x; k < C; k += blockDim.x) {
        rs.lp[k] = r.lp[lc + k];
        rs.ll[k] = r.ll[lc + k];
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        rs.lps[k] = r.lp_s[ls + k];
        rs.lls[k] = r.ll_s[ls + k];
        rs.accu[k] = r.accu[lc + k];
        rs.ver[k] = 0;
        rs.mod[k] = 0;
        if (type == PASS_CROSS) {
            rs.pa[k] = r.partner[(lc + k) * 2];
            rs.pb[k] = r.partner[(lc + k) * 2 + 1];
        } else {
            rs.pa[k] = r.sub[lc + k];
        }
    }
    __syncthreads();
    const int nloop = (r.loop == LOOP_HCHAINS) ? r.half : r.Pn;
    const int para = r.rs_para[l];
    const double *jit = r.jit + lc * P;
    if (jit_stage_bytes(C, P)) {
        double *js = (double *)(smem_raw + sub_smem_bytes(r.m) + res_smem_bytes(C));
        for (int q = threadIdx.x; q < C * P; q += blockDim.x) js[q] = jit[q];
        __syncthreads();
        jit = js;
    }
    const int ct = threadIdx.x, cstride = blockDim.x;
    // variants live in slots C + w, so at most C of them (CS = 2C)
    const int mig_round = min(max(r.mig_round, 1), min(kVariants, C));
    int rounds = 0, reevals = 0, variants = 0;
    int decided = 0;
    if (type == PASS_CROSS) {
        while (decided < n) {
            ++rounds;
            // Metropolis outcome of every undecided step: it depends only on
            // the step's own proposal and its own chain's current state.
            for (int k = decided + threadIdx.x; k < n; k += blockDim.x)
                rs.dec[k] = mh_accept((rs.lps[k] + rs.lls[k]) - (rs.ll[k] + rs.lp[k]), rs.accu[k]) ? 1 : 0;
            __syncthreads();
            // The decided prefix ends at the first step one of whose partners
            // moved after that step's proposal was made: a partner accepted in
            // an earlier round (mod) or earlier in this one (dec).
            const int dc = decided;
            const int d = block_first(dc, n, [&](int i) {
                const int a = rs.pa[i], b = rs.pb[i], v = rs.ver[i];
                const bool ma = a >= v && a < i && (a < dc ? rs.mod[a] : rs.dec[a]);
                const bool mb = b >= v && b < i && (b < dc ? rs.mod[b] : rs.dec[b]);
                return ma || mb;
            }, rs.misc + 6);
            for (int i = dc + threadIdx.x; i < d; i += blockDim.x) rs.mod[i] = rs.dec[i];
            const int na = block_compact(dc, d, [&](int i) { return rs.dec[i] != 0; }, rs.acc, rs.warp);
            for (int q = threadIdx.x; q < na; q += blockDim.x) rs.accslot[q] = rs.acc[q];
            __syncthreads();
            write_accepts(r, l, type, n, rs, na);
            decided = d;
            if (decided >= n) break;
            // stale chains: a partner in [ver, decided) moved
            const int m = block_compact(decided, n, [&](int k) {
                const int a = rs.pa[k], b = rs.pb[k], v = rs.ver[k];
                return (a >= v && a < decided && rs.mod[a]) || (b >= v && b < decided && rs.mod[b]);
            }, rs.list, rs.warp);
            for (int k = decided + threadIdx.x; k < n; k += blockDim.x) rs.ver[k] = (int16_t)decided;
            __syncthreads();
            reevals += m;
            for (int q = ct; q < m * P; q += cstride) {
                const int k = rs.list[q / P], j = q % P;
                const double tk = r.th[(lc + k) * P + j];
                r.th_s[(ls + k) * P + j] =
                    updated(j, para, nloop)
                        ? cross_comp(r.gamma, tk, r.th[(lc + rs.pa[k]) * P + j], r.th[(lc + rs.pb[k]) * P + j],
                                     jit[(size_t)k * P + j])
                        : tk;
            }
            for (int q = ct; q < m; q += cstride) r.tab_bad[ls + rs.list[q]] = 0;
            __syncthreads();
            const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
            for (int q = wid; q < m; q += nw) {
                const int k = rs.list[q];
                const double lp = warp_prior(r, r.th_s + (ls + k) * P, k);
                if ((threadIdx.x & 31) == 0) {
                    rs.lps[k] = lp;
                    rs.lls[k] = 0.0;
                    r.lp_s[ls + k] = lp;
                    r.ll_s[ls + k] = 0.0;
                }
            }
            if (mixed) {
                // from the block's last thread down, so the tables build on
                // other warps than the priors' (warps 0..m-1), at the same time
                const int NU = r.m.n_ent + r.m.n_t0;
                for (int q = cstride - 1 - ct; q < m * NU; q += cstride) {
                    const int k = rs.list[q / NU];
                    store_entry(r, ls + k, r.th_s + (ls + k) * P, q % NU);
                }
            }
            __syncthreads();
            // evaluate the re-proposed chains whose prior is finite
            const int e = block_compact(0, m, [&](int q) { return rs.lps[rs.list[q]] > -INFINITY; },
                                        rs.acc, rs.warp);
            if (e < m) {
                // through accslot (free until the next round's decisions): an
                // in-place gather could read an entry another warp has moved
                for (int q = threadIdx.x; q < e; q += blockDim.x) rs.accslot[q] = rs.list[rs.acc[q]];
                __syncthreads();
                for (int q = threadIdx.x; q < e; q += blockDim.x) rs.list[q] = rs.accslot[q];
                __syncthreads();
            }
            eval_direct(r, l, rs.list, e, sm, mixed, rs.lls, 0);
        }
    } else {
        // migration: cur[s] = log posterior of step s's destination, which
        // only step s itself can change
        for (int s = threadIdx.x; s < n; s += blockDim.x) {
            const int dst = (s + 1 == n) ? rs.pa[0] : rs.pa[s + 1];
            rs.cur[s] = rs.lp[dst] + rs.ll[dst];
        }
        __syncthreads();
        for (int w = threadIdx.x; w < n; w += blockDim.x) {
            rs.vlp[w] = r.lp_s[ls + C + w];
            rs.vll[w] = r.ll_s[ls + C + w];
        }
        __syncthreads();
        // Metropolis outcomes of every step's start-of-pass proposal and of
        // its cascade value (draw-free: the accept uniforms are fixed)
        for (int s = threadIdx.x; s < n; s += blockDim.x) {
            rs.dec[s] = mh_accept((rs.lps[s] + rs.lls[s]) - rs.cur[s], rs.accu[s]) ? 1 : 0;
            rs.cdec[s] = (s > 0 && mh_accept((rs.vlp[s] + rs.vll[s]) - rs.cur[s], rs.accu[s])) ? 1 : 0;
        }
        if (threadIdx.x == 0) rs.misc[5] = 0;   // accepted steps so far
        __syncthreads();
        while (decided < n) {
            ++rounds;
            const int d = decided;
            // Round d > 0 starts because step d-1 was accepted, so step d's
            // source moved.  The value step s needs is fixed by the last
            // rejected step r before it: the spec proposal of step r+1 plus
            // the jitters of steps r+2..s, or, with no reject since d, the
            // new source plus the jitters of d..s.  Evaluate the r.mig_round
            // most likely of these, scored with this pass's acceptance so far.
            if (d > 0) {
                if (threadIdx.x < 32) {
                    // candidate c < kVariants: the run value for step d + c
                    // (score a^c, 2 for c = 0); c >= kVariants: the value for
                    // step rj + 1 + k after a reject at rj = d + (c - kVariants) / 3,
                    // k = 1 + (c - kVariants) % 3 (score (1 - a) a^k 0.95^(rj - d));
                    // the mig_round best, ties to the lower c.  Scores are
                    // ranked as FP32 log2 values: they only choose which values
                    // are evaluated ahead, never a result.
                    const int c = threadIdx.x;
                    const float a = (rs.misc[5] + 1.f) / (d + 2.f);       // in (0, 1)
                    const float la = __log2f(a), lb = __log2f(1.f - a);
                    float sc = -INFINITY;
                    int vr = 0, vs = 0;
                    if (c < kVariants) {
                        if (d + c < n) {
                            sc = (c == 0) ? 1.f : (float)c * la;
                            vr = -1;
                            vs = d + c;
                        }
                    } else {
                        const int rj = d + (c - kVariants) / 3, k = 1 + (c - kVariants) % 3;
                        if (rj + 1 + k < n) {
                            sc = fmaf((float)(rj - d), -0.0740005815f, fmaf((float)k, la, lb));   // log2 0.95
                            vr = rj;
                            vs = rj + 1 + k;
                        }
                    }
                    int rank = 0;
                    for (int o = 0; o < 32; ++o) {
                        const float so = __shfl_sync(0xffffffffu, sc, o);
                        rank += (so > sc || (so == sc && o < c)) ? 1 : 0;
                    }
                    const bool valid = sc > -INFINITY;
                    if (valid && rank < mig_round) {
                        rs.vr[rank] = vr;
                        rs.vs[rank] = vs;
                    }
                    const int nvalid = __popc(__ballot_sync(0xffffffffu, valid));
                    if (c == 0) rs.misc[4] = min(mig_round, nvalid);
                }
                __syncthreads();
                const int nv = rs.misc[4];
                for (int q = ct; q < nv * P; q += cstride) {
                    const int w = q / P, j = q % P;
                    const int vr = rs.vr[w], vs = rs.vs[w];
                    double v = (vr < 0) ? r.th[(lc + rs.pa[d]) * P + j] : r.th_s[(ls + vr + 1) * P + j];
                    if (updated(j, para, nloop))
                        for (int t = (vr < 0) ? d : vr + 2; t <= vs; ++t) v = __dadd_rn(v, jit[(size_t)t * P + j]);
                    r.th_s[(ls + C + w) * P + j] = v;
                }
                for (int w = ct; w < nv; w += cstride) r.tab_bad[ls + C + w] = 0;
                __syncthreads();
                const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
                for (int w = wid; w < nv; w += nw) {
                    const double lp = warp_prior(r, r.th_s + (ls + C + w) * P, rs.pa[rs.vs[w]]);
                    if ((threadIdx.x & 31) == 0) {
                        rs.vlp[w] = lp;
                        rs.vll[w] = 0.0;
                    }
                }
                if (mixed) {
                    const int NU = r.m.n_ent + r.m.n_t0;              // beside the priors' warps
                    for (int q = cstride - 1 - ct; q < nv * NU; q += cstride) {
                        const int w = q / NU;
                        store_entry(r, ls + C + w, r.th_s + (ls + C + w) * P, q % NU);
                    }
                }
                __syncthreads();
                if (threadIdx.x == 0) {
                    int e = 0;
                    for (int w = 0; w < nv; ++w)
                        if (rs.vlp[w] > -INFINITY) rs.list[e++] = C + w;
                    rs.misc[3] = e;
                }
                __syncthreads();
                const int ne = rs.misc[3];
                variants += ne;
                if (ne) eval_direct(r, l, rs.list, ne, sm, mixed, rs.vll, C);
                for (int w = threadIdx.x; w < nv; w += blockDim.x)
                    rs.vdec[w] = mh_accept((rs.vlp[w] + rs.vll[w]) - rs.cur[rs.vs[w]], rs.accu[rs.vs[w]]) ? 1 : 0;
                __syncthreads();
            }
            if (threadIdx.x == 0) {
                // the steps in order, each with the outcome of the value it
                // needs, until one needs a value not evaluated yet
                const int nv = (d == 0) ? n : rs.misc[4];
                int s = d, na = 0, lastrej = -1, nacc = rs.misc[5];
                while (s < n) {
                    int slot = -1;
                    bool ok = false;
                    if (s > 0 && !rs.mod[s - 1]) {
                        slot = s;                    // source unchanged: the spec proposal
                        ok = rs.dec[s];
                    } else if (d == 0) {
                        if (s == 0) {
                            slot = 0;
                            ok = rs.dec[0];
                        } else if (lastrej < 0) {    // cascade from step 0
                            slot = C + s;
                            ok = rs.cdec[s];
                        }
                    } else {
                        for (int w = 0; w < nv; ++w)
                            if (rs.vs[w] == s && rs.vr[w] == lastrej) {
                                slot = C + w;
                                ok = rs.vdec[w];
                            }
                    }
                    if (slot < 0) break;
                    rs.mod[s] = ok ? 1 : 0;
                    if (ok) { rs.acc[na] = s; rs.accslot[na] = slot; ++na; ++nacc; }
                    else lastrej = s;
                    ++s;
                }
                rs.misc[0] = s;
                rs.misc[1] = na;
                rs.misc[5] = nacc;
            }
            __syncthreads();
            decided = rs.misc[0];
            write_accepts(r, l, type, n, rs, rs.misc[1]);
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        // this level's cost, for the order of the next sweep's crossover
        // levels: the mean of the last measurement and the one before
        if (type == PASS_CROSS) {
            const long long t = (long long)min(global_ns() - t_beg, 0x7fffffffull), o = r.lvl_ns[l];
            r.lvl_ns[l] = (int32_t)(o > 0 ? (o + t) / 2 : t);
        }
        atomicAdd(&r.stats[ST_PROPOSALS], (unsigned long long)n);
        atomicAdd(&r.stats[ST_REEVALS], (unsigned long long)reevals);
        atomicAdd(&r.stats[ST_VARIANTS], (unsigned long long)variants);
        atomicAdd(&r.stats[ST_ROUNDS], (unsigned long long)rounds);
    }
}

// The level at rank q of the order the resolve takes levels in: this pass's
// migration levels (the longest to resolve: a round per few steps) first,
// then the others, each group in res_order's order (k_level_order).  All
// threads; tmp holds 34 ints.
__device__ int mig_first_level(const RunDev &r, int q, int *tmp)
{
    const int S = r.S;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // number of migration levels
    int c = 0;
    for (int i = threadIdx.x; i < S; i += blockDim.x) c += r.ptype[r.res_order[i]] == PASS_MIG;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (threadIdx.x == 0) tmp[33] = 0;
    __syncthreads();
    if (lane == 0 && c) atomicAdd(tmp + 33, c);
    __syncthreads();
    const int nm = tmp[33];
    const bool want = q < nm;
    int rank = want ? q : q - nm;
    // the rank-th level (in sub_order) whose type matches, scanned a block at a time
    int found = -1;
    for (int b0 = 0; b0 < S && found < 0; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        const bool p = i < S && ((r.ptype[r.res_order[i]] == PASS_MIG) == want);
        const unsigned m = __ballot_sync(0xffffffffu, p);
        if (lane == 0) tmp[wid] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int w = 0; w < nw; ++w) { const int t = tmp[w]; tmp[w] = acc; acc += t; }
            tmp[32] = acc;
            tmp[33] = -1;
        }
        __syncthreads();
        const int before = tmp[wid] + __popc(m & ((1u << lane) - 1u));
        if (p && before == rank) tmp[33] = r.res_order[i];
        const int total = tmp[32];
        __syncthreads();
        found = tmp[33];
        rank -= total;
        __syncthreads();
    }
    return found;
}

// k_sub_resolve: one CTA per level of [level_begin, level_begin + n_level),
// block q taking the level at rank q of mig_first_level's order when every
// level runs (else index order), so the longest levels start in the first
// wave.
__global__ void __launch_bounds__(kResolveThreads, GGDMC_RESOLVE_MINB)
k_sub_resolve(RunDev r, int level_begin, int n_level, int ordered, int score_priors)
{
    extern __shared__ __align__(16) char smem_raw[];
    __shared__ int s_tmp[34];
    const int q = blockIdx.x;
    if (q >= n_level) return;
    SubSmem sm = carve(smem_raw, r.m);
    load_design(r, sm);
    const int l = (ordered == 1) ? mig_first_level(r, q, s_tmp)
                  : (ordered == 2) ? r.sub_order[q] : level_begin + q;
    __syncthreads();
    resolve_level(r, l, sm, smem_raw, score_priors != 0);
}

// k_sub_step: the subject pass of iteration t (= *iter) and the start of
// iteration t + 1's, on a persistent grid.  CTAs claim levels in res_order
// and resolve them; the CTA that resolved level l then builds l's proposals
// for t + 1 (they read only l's state) and publishes them (ready[l] = t + 1).
// Once every level is claimed, CTAs evaluate spec items of published levels
// while any level is still being resolved, and leave the rest to
// k_sub_spec_rest, which runs beside the phi level of t + 1.  An idle CTA
// polls one event counter (bumped by every publication and every resolved
// level); its waits are only for levels a running CTA holds, and bounded.
constexpr int kStatusSpecWait = 3;           // RunDev::status when an idle wait gave up

__device__ __forceinline__ int vload(const int32_t *p) { return *(const volatile int32_t *)p; }

__global__ void __launch_bounds__(kResolveThreads, GGDMC_RESOLVE_MINB)
k_sub_step(RunDev r, int score_priors, int defer_next, int group)
{
    extern __shared__ __align__(16) char smem_raw[];
    __shared__ int s_q, s_m, s_state;
    __shared__ int s_slots[kGroup];
    SubSmem sm = carve(smem_raw, r.m);
    load_design(r, sm);
    __syncthreads();
    const int it = *r.iter;
    const bool next = it < r.iter_end;
    // propose_level's scratch: the resolve's region, free once a level is decided
    char *scratch = smem_raw + sub_smem_bytes(r.m);
    for (;;) {
        if (threadIdx.x == 0) s_q = atomicAdd(r.ctl + kCtlResNext, 1);
        __syncthreads();
        const int q = s_q;
        __syncthreads();
        if (q >= r.S) break;
        const int l = r.res_order[q];
        resolve_level(r, l, sm, smem_raw, score_priors != 0);
        __syncthreads();
        if (next) {
            propose_level(r, l, it + 1, 0, defer_next != 0, scratch);
            __syncthreads();
            if (threadIdx.x == 0) {
                r.spec_cnt[l] = 0;
                __threadfence();
                atomicExch(r.ready + l, it + 1);
            }
        }
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(r.ctl + kCtlResDone, 1);
            atomicAdd(r.ctl + kCtlEvents, 1);
        }
    }
    if (!next) return;
    const bool mixed = r.prec == PREC_MIXED;
    const int n_item = 2 * ((r.C + group - 1) / group);
    int seen = -1;                 // event count of the last fruitless scan
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            // 0: every level resolved, 1: scan, 2: gave up waiting
            int st = 1;
            for (int idle = 0;; ++idle) {
                if (vload(r.ctl + kCtlResDone) >= r.S) { st = 0; break; }
                if (vload(r.ctl + kCtlEvents) != seen) break;
                if (idle > r.spec_idle_limit) {
                    atomicExch(r.status, kStatusSpecWait);
                    st = 2;
                    break;
                }
                __nanosleep(1000);
            }
            s_state = st;
            s_q = INT_MAX;
            s_m = 0;
        }
        __syncthreads();
        if (s_state != 1) break;
        const int ev = vload(r.ctl + kCtlEvents);        // before the scan
        // the first published level (largest first) with an unclaimed item
        for (int q = threadIdx.x; q < r.S; q += blockDim.x) {
            const int l = r.sub_order[q];
            if (vload(r.ready + l) == it + 1 && vload(r.spec_cnt + l) < n_item) atomicMin(&s_q, q);
        }
        __syncthreads();
        if (threadIdx.x == 0 && s_q != INT_MAX) {
            const int l = r.sub_order[s_q];
            if (vload(r.ready + l) == it + 1) {
                __threadfence();                      // acquire l's proposals
                // two items a claim where their proposals fit one group:
                // the resolve block's 16 warps then have twice the chunks
                const int take = (2 * group <= kGroup) ? 2 : 1;
                const int k = atomicAdd(r.spec_cnt + l, take);
                int mm = 0;
                for (int j = 0; j < take; ++j)
                    if (k + j < n_item) mm += spec_item_slots<true>(r, l, k + j, group, s_slots + mm);
                s_m = mm;
            }
        }
        __syncthreads();
        if (s_q == INT_MAX) {
            seen = ev;             // nothing to take: wait for the next event
            continue;
        }
        if (s_m > 0) eval_slots<true>(r, r.sub_order[s_q], s_slots, s_m, sm, mixed, nullptr);
    }
}

// ------------------------------------------------------------ phi level
// Hyper log-likelihood (sumloghlike, src/de.cpp:245-270) of phi vector `phv`
// (shared memory) against subject chain `chain`, or, for run_hyper, against
// the fixed data rows.  Every thread gets the sum.  MIXED: terms in FP32,
// sum in FP64.
__device__ double hyper_sum(const RunDev &r, const double *phv, int chain, double *cst, double *red)
{
    // cst[p] = constant of the log density, cst[P + p] = 1 / sigma
    const int P = r.Pphi / 2;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        cst[p] = tnorm_const_p(r, phv[p], phv[P + p], r.pp_bounds[2 * p], r.pp_bounds[2 * p + 1]);
        cst[P + p] = 1.0 / phv[P + p];
    }
    __syncthreads();
    const int nrow = r.hrows ? r.n_row : r.S;
    const bool fp32 = r.prec == PREC_MIXED;
    double acc = 0.0;
    float accf = 0.f;
    for (int idx = threadIdx.x; idx < nrow * P; idx += blockDim.x) {
        const int s = idx / P, p = idx % P;
        const double x = r.hrows ? r.hrows[(size_t)s * P + p]
                                 : r.th[((size_t)s * r.C + chain) * r.P + p];
        if (x < r.pp_bounds[2 * p] || x > r.pp_bounds[2 * p + 1] || !(phv[P + p] > 0.0)) {
            acc = -INFINITY;
        } else if (fp32) {
            const float z = (float)(x - phv[p]) * (float)cst[P + p];
            accf = fmaf(-0.5f * z, z, accf + (float)cst[p]);
        } else {
            const double z = (x - phv[p]) * cst[P + p];
            acc += -0.5 * z * z + cst[p];
        }
    }
    return block_sum(acc + (double)accf, red);
}

__global__ void __launch_bounds__(kPhiProposeThreads) k_phi_propose(RunDev r, int pass)
{
    __shared__ double s_u[kMaxChain + 2];
    __shared__ int s_sub[kMaxChain];
    __shared__ int s_perm[kMaxChain];
    __shared__ int s_pa[kMaxChain], s_pb[kMaxChain];
    __shared__ int s_type, s_n, s_para;
    const int64_t it = *r.iter;
    const int C = r.C, P = r.Pphi;
    if (threadIdx.x == 0) {
        int type = PASS_CROSS, para = -1;
        if (r.phi_loop == LOOP_HCHAINS) {
            const bool mig = uniform(r.ds, it, 0, pass, 0) < r.pop_mig;
            type = mig ? PASS_MIG : PASS_CROSS;
            para = r.phi_blocked ? pass : -1;
        } else if (pass == 0) {
            const bool mig = uniform(r.ds, it, 0, 0, 0) < r.sub_mig;
            r.pmigrated[0] = mig;
            type = mig ? PASS_MIG : PASS_CROSS;
            para = (!mig && r.phi_blocked) ? 0 : -1;
        } else {
            type = r.pmigrated[0] ? PASS_SKIP : PASS_CROSS;
            para = pass;
        }
        s_type = type;
        s_para = para;
    }
    __syncthreads();
    const int type = s_type, para = s_para;
    if (type == PASS_MIG) {
        for (int q = 1 + threadIdx.x; q < C + 2; q += blockDim.x) s_u[q] = uniform(r.ds, it, 0, pass, q);
        __syncthreads();
        if (threadIdx.x == 0) {
            s_n = subchains_pick(C, s_u, s_perm);
            atomicAdd(&r.stats[ST_MIGRATIONS], 1ull);
        }
        __syncthreads();
        subchains_sort(s_perm, s_n, s_sub);
    } else if (threadIdx.x == 0) {
        s_n = (type == PASS_SKIP) ? 0 : C;
    }
    __syncthreads();
    const int n = s_n;
    if (threadIdx.x == 0) {
        r.pptype[0] = type;
        r.pnstep[0] = n;
    }
    if (n == 0) return;
    const int nloop = r.Pn;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        if (type == PASS_CROSS) {
            int a, b;
            partners(r, it, 0, pass, k, a, b);
            s_pa[k] = a;
            s_pb[k] = b;
            r.ppartner[2 * k] = a;
            r.ppartner[2 * k + 1] = b;
        } else {
            r.psub[k] = s_sub[k];
        }
        r.paccu[k] = accept_draw(r, it, 0, pass, k);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < n * P; q += blockDim.x) {
        const int k = q / P, j = q % P;
        const int src = (type == PASS_CROSS) ? k : s_sub[k];
        const double ts = r.pth[(size_t)src * P + j];
        double out = ts;
        if (updated(j, para, nloop)) {
            const double jv = jitter_draw(r, it, 0, pass, k, j);
            r.pjit[(size_t)k * P + j] = jv;
            out = (type == PASS_CROSS)
                      ? cross_comp(r.gamma, ts, r.pth[(size_t)s_pa[k] * P + j],
                                   r.pth[(size_t)s_pb[k] * P + j], jv)
                      : __dadd_rn(ts, jv);
        }
        r.pth_s[(size_t)k * P + j] = out;
    }
    __syncthreads();
    for (int k = threadIdx.x >> 5; k < n; k += blockDim.x >> 5) {
        const double lp = warp_phi_prior(r, r.pth_s + (size_t)k * P);
        if ((threadIdx.x & 31) == 0) {
            r.plp_s[k] = lp;
            r.pll_s[k] = 0.0;
            r.pneed[k] = (lp > -INFINITY) ? 1 : 0;
        }
    }
}

// k_phi_eval: grid = 3*C; block (k, what): what 0 refresh of the step's
// source chain, 1 the proposal, 2 refresh of a migration's destination.
__global__ void __launch_bounds__(kPhiThreads) k_phi_eval(RunDev r)
{
    __shared__ double s_phi[kMaxTheta];
    __shared__ double s_cst[2 * kMaxTheta];
    __shared__ double s_red[33];
    const int k = blockIdx.x / 3, what = blockIdx.x % 3;
    const int type = r.pptype[0];
    if (type == PASS_SKIP || k >= r.pnstep[0]) return;
    const bool refresh = (r.phi_loop == LOOP_HCHAINS);
    const int P = r.Pphi;
    int chain;
    const double *vec;
    if (type == PASS_CROSS) {
        if (what == 2) return;
        if (what == 0 && !refresh) return;
        chain = k;
        vec = (what == 0) ? r.pth + (size_t)k * P : r.pth_s + (size_t)k * P;
    } else {
        const int src = r.psub[k];
        const int dst = (k + 1 == r.pnstep[0]) ? r.psub[0] : r.psub[k + 1];
        if (what != 1 && !refresh) return;
        chain = (what == 2) ? dst : src;
        vec = (what == 0) ? r.pth + (size_t)src * P
              : (what == 1) ? r.pth_s + (size_t)k * P : r.pth + (size_t)dst * P;
    }
    if (what == 1 && !r.pneed[k]) return;
    for (int j = threadIdx.x; j < P; j += blockDim.x) s_phi[j] = vec[j];
    __syncthreads();
    const double h = hyper_sum(r, s_phi, chain, s_cst, s_red);
    if (threadIdx.x == 0) {
        if (what == 0) r.pref_src[k] = h;
        else if (what == 1) r.pll_s[k] = h;
        else r.pref_next[k] = h;
    }
}

// Hyper log-likelihoods of m phi vectors at once.  A round re-scores only a
// few vectors, so every vector's subject x parameter terms are spread over
// the whole block (a handful of independent loads per thread) rather than a
// warp walking each subject's row in series; warp partials land in part[q][w]
// and are summed in warp order.  vecs[q] points to vector q, chains[q] is the
// subject chain it is scored against; cst holds 2 * m * P doubles, part
// m * 32 doubles, oos m ints.  Results to out[q].
__device__ void phi_batch_hyper(const RunDev &r, const double *const *vecs, const int *chains, int m,
                                double *cst, double *part, int *oos, double *out)
{
    const int P = r.Pphi / 2;
    for (int t = threadIdx.x; t < m * P; t += blockDim.x) {
        const int q = t / P, p = t % P;
        const double mu = vecs[q][p], sg = vecs[q][P + p];
        cst[2 * t] = tnorm_const_p(r, mu, sg, r.pp_bounds[2 * p], r.pp_bounds[2 * p + 1]);
        cst[2 * t + 1] = (sg > 0.0) ? 1.0 / sg : 0.0;
    }
    if (threadIdx.x < m) oos[threadIdx.x] = 0;
    __syncthreads();
    const int nrow = r.hrows ? r.n_row : r.S;
    const int nterm = nrow * P;
    const bool fp32 = r.prec == PREC_MIXED;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q = 0; q < m; ++q) {
        const double *v = vecs[q];
        const double *cq = cst + 2 * q * P;
        const size_t cbase = (size_t)chains[q] * r.P;
        bool bad = false;
        double acc = 0.0;
        float facc = 0.f;
        // loads first, eight per thread in flight, then branch-free terms
        constexpr int U = 8;
        for (int e0 = threadIdx.x; e0 < nterm; e0 += U * blockDim.x) {
            double x[U];
            int pp[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int e = e0 + u * blockDim.x;
                pp[u] = -1;
                x[u] = 0.0;
                if (e < nterm) {
                    const int sj = e / P;
                    pp[u] = e - sj * P;
                    x[u] = r.hrows ? r.hrows[e] : r.th[(size_t)sj * r.C * r.P + cbase + pp[u]];
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int p = pp[u];
                if (p < 0) continue;
                const double xv = x[u];
                bad |= (xv < r.pp_bounds[2 * p]) | (xv > r.pp_bounds[2 * p + 1]) | !(cq[2 * p + 1] > 0.0);
                if (fp32) {
                    const float z = (float)(xv - v[p]) * (float)cq[2 * p + 1];
                    facc += fmaf(-0.5f * z, z, (float)cq[2 * p]);
                } else {
                    const double z = (xv - v[p]) * cq[2 * p + 1];
                    acc += -0.5 * z * z + cq[2 * p];
                }
            }
        }
        acc += (double)facc;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        bad = __any_sync(0xffffffffu, bad);
        if (lane == 0) {
            part[q * 32 + wid] = acc;
            if (bad) oos[q] = 1;
        }
    }
    __syncthreads();
    if (threadIdx.x < m) {
        const int q = threadIdx.x;
        double sum = 0.0;
        for (int w = 0; w < nw; ++w) sum += part[q * 32 + w];
        out[q] = oos[q] ? -INFINITY : sum;
    }
    __syncthreads();
}

// k_phi_resolve: ordered decisions of the phi level (src/de.cpp:385-565;
// run_hyper's level follows src/de.cpp:111-199).  One CTA.
constexpr int kPhiResolveThreads = 1024;
constexpr int kPhiBatch = 16;       // phi vectors scored per batch

__global__ void __launch_bounds__(kPhiResolveThreads) k_phi_resolve(RunDev r, int pass)
{
    __shared__ double s_lps[kMaxChain], s_lls[kMaxChain], s_ref[kMaxChain];
    __shared__ uint8_t s_mod[kMaxChain], s_dec[kMaxChain];
    __shared__ int16_t s_ver[kMaxChain];
    __shared__ int s_list[kMaxChain], s_acc[kMaxChain];
    __shared__ int16_t s_pa[kMaxChain], s_pb[kMaxChain];
    __shared__ double s_cst[kPhiBatch * kMaxTheta];
    __shared__ const double *s_vecs[kPhiBatch];
    __shared__ int s_chains[kPhiBatch];
    __shared__ double s_out[kPhiBatch];
    __shared__ double s_part[kPhiBatch * 32];
    __shared__ int s_oos[kPhiBatch];
    __shared__ int s_misc[4];
    const int type = r.pptype[0];
    if (type == PASS_SKIP) return;
    const int C = r.C, P = r.Pphi;
    const int n = r.pnstep[0];
    const bool refresh = (r.phi_loop == LOOP_HCHAINS);
    const int nloop = r.Pn;
    int para;
    if (r.phi_loop == LOOP_HCHAINS) para = r.phi_blocked ? pass : -1;
    else para = (type == PASS_MIG) ? -1 : (r.phi_blocked ? pass : -1);
    int reevals = 0, accepts = 0;
    if (type == PASS_CROSS) {
        for (int k = threadIdx.x; k < C; k += blockDim.x) {
            s_pa[k] = (int16_t)r.ppartner[2 * k];
            s_pb[k] = (int16_t)r.ppartner[2 * k + 1];
            s_lps[k] = r.plp_s[k];
            s_lls[k] = r.pll_s[k];
            // the refreshed hyper log-likelihood of chain k (src/de.cpp:397-400)
            s_ref[k] = refresh ? r.pref_src[k] : r.pll[k];
            s_ver[k] = 0;
            s_mod[k] = 0;
        }
        __syncthreads();
        int decided = 0;
        while (decided < n) {
            for (int k = decided + threadIdx.x; k < n; k += blockDim.x)
                s_dec[k] = mh_accept((s_lps[k] + s_lls[k]) - (s_ref[k] + r.plp[k]), r.paccu[k]) ? 1 : 0;
            __syncthreads();
            if (threadIdx.x == 0) {
                int i = decided, na = 0;
                while (i < n) {
                    const int a = s_pa[i], b = s_pb[i], v = s_ver[i];
                    if ((a >= v && a < i && s_mod[a]) || (b >= v && b < i && s_mod[b])) break;
                    s_mod[i] = s_dec[i];
                    if (s_dec[i]) s_acc[na++] = i;
                    ++i;
                }
                s_misc[0] = i;
                s_misc[1] = na;
            }
            __syncthreads();
            const int d = s_misc[0], na = s_misc[1];
            accepts += na;
            // decided steps: the refresh is stored, an accept overwrites it
            for (int k = decided + threadIdx.x; k < d; k += blockDim.x) {
                r.pll[k] = s_mod[k] ? s_lls[k] : s_ref[k];
                if (s_mod[k]) r.plp[k] = s_lps[k];
            }
            for (int q = threadIdx.x; q < na * P; q += blockDim.x) {
                const int i = s_acc[q / P], j = q % P;
                r.pth[(size_t)i * P + j] = r.pth_s[(size_t)i * P + j];
            }
            decided = d;
            __syncthreads();
            if (decided >= n) break;
            if (threadIdx.x == 0) {
                int m = 0;
                for (int k = decided; k < n; ++k) {
                    const int a = s_pa[k], b = s_pb[k], v = s_ver[k];
                    if ((a >= v && a < decided && s_mod[a]) || (b >= v && b < decided && s_mod[b]))
                        s_list[m++] = k;
                    s_ver[k] = (int16_t)decided;
                }
                s_misc[2] = m;
            }
            __syncthreads();
            const int m = s_misc[2];
            reevals += m;
            for (int q = threadIdx.x; q < m * P; q += blockDim.x) {
                const int k = s_list[q / P], j = q % P;
                const double tk = r.pth[(size_t)k * P + j];
                r.pth_s[(size_t)k * P + j] =
                    updated(j, para, nloop)
                        ? cross_comp(r.gamma, tk, r.pth[(size_t)s_pa[k] * P + j],
                                     r.pth[(size_t)s_pb[k] * P + j], r.pjit[(size_t)k * P + j])
                        : tk;
            }
            __syncthreads();
            for (int q = threadIdx.x >> 5; q < m; q += blockDim.x >> 5) {
                const int k = s_list[q];
                const double lp = warp_phi_prior(r, r.pth_s + (size_t)k * P);
                if ((threadIdx.x & 31) == 0) {
                    s_lps[k] = lp;
                    s_lls[k] = 0.0;
                }
            }
            __syncthreads();
            for (int q0 = 0; q0 < m; q0 += kPhiBatch) {
                const int mb = min(kPhiBatch, m - q0);
                if (threadIdx.x < mb) {
                    const int k = s_list[q0 + threadIdx.x];
                    s_vecs[threadIdx.x] = r.pth_s + (size_t)k * P;
                    s_chains[threadIdx.x] = k;
                }
                __syncthreads();
                phi_batch_hyper(r, s_vecs, s_chains, mb, s_cst, s_part, s_oos, s_out);
                for (int q = threadIdx.x; q < mb; q += blockDim.x) {
                    const int k = s_list[q0 + q];
                    if (s_lps[k] > -INFINITY) s_lls[k] = s_out[q];
                }
                __syncthreads();
            }
            for (int q = threadIdx.x; q < m; q += blockDim.x) {
                const int k = s_list[q];
                r.plp_s[k] = s_lps[k];
                r.pll_s[k] = s_lls[k];
            }
            __syncthreads();
        }
    } else {
        // migration (pop_migration_prob per sweep): steps in order; a step
        // whose source was replaced by the previous step's accept is
        // re-proposed from it, and its source's refreshed value recomputed.
        if (threadIdx.x == 0) s_misc[0] = 0;
        __syncthreads();
        for (int i = 0; i < n; ++i) {
            const int src = r.psub[i];
            const int dst = (i + 1 == n) ? r.psub[0] : r.psub[i + 1];
            const bool stale = i > 0 && s_misc[0];
            if (stale) {
                for (int j = threadIdx.x; j < P; j += blockDim.x)
                    r.pth_s[(size_t)i * P + j] = updated(j, para, nloop)
                        ? __dadd_rn(r.pth[(size_t)src * P + j], r.pjit[(size_t)i * P + j])
                        : r.pth[(size_t)src * P + j];
                __syncthreads();
                if (threadIdx.x < 32) {
                    const double lp = warp_phi_prior(r, r.pth_s + (size_t)i * P);
                    if (threadIdx.x == 0) {
                        s_vecs[0] = r.pth_s + (size_t)i * P;
                        s_vecs[1] = r.pth + (size_t)src * P;
                        s_chains[0] = src;
                        s_chains[1] = src;
                        s_lps[0] = lp;
                    }
                }
                __syncthreads();
                phi_batch_hyper(r, s_vecs, s_chains, refresh ? 2 : 1, s_cst, s_part, s_oos, s_out);
                if (threadIdx.x == 0) {
                    r.plp_s[i] = s_lps[0];
                    r.pll_s[i] = (s_lps[0] > -INFINITY) ? s_out[0] : 0.0;
                    if (refresh) r.pref_src[i] = s_out[1];
                }
                ++reevals;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                if (refresh) {
                    r.pll[src] = r.pref_src[i];
                    r.pll[dst] = r.pref_next[i];
                }
                const double cur = r.plp[dst] + r.pll[dst];
                const bool ok = mh_accept((r.plp_s[i] + r.pll_s[i]) - cur, r.paccu[i]);
                if (ok) {
                    r.plp[dst] = r.plp_s[i];
                    r.pll[dst] = r.pll_s[i];
                    ++accepts;
                }
                s_misc[0] = ok ? 1 : 0;
            }
            __syncthreads();
            if (s_misc[0])
                for (int j = threadIdx.x; j < P; j += blockDim.x)
                    r.pth[(size_t)dst * P + j] = r.pth_s[(size_t)i * P + j];
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        atomicAdd(&r.stats[ST_PROPOSALS], (unsigned long long)n);
        atomicAdd(&r.stats[ST_ACCEPTS], (unsigned long long)accepts);
        atomicAdd(&r.stats[ST_REEVALS], (unsigned long long)reevals);
    }
}

// k_phi_tables: (mu, 1/sigma, c) of every phi chain for the subject priors.
__global__ void k_phi_tables(RunDev r)
{
    const int i = blockIdx.x;
    const int P = r.P;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        const double mu = r.pth[(size_t)i * r.Pphi + p];
        const double sg = r.pth[(size_t)i * r.Pphi + P + p];
        double *o = r.phi_tab + ((size_t)i * P + p) * 3;
        o[0] = mu;
        o[1] = (sg > 0.0) ? 1.0 / sg : 0.0;     // 0 marks an invalid scale
        o[2] = tnorm_const_p(r, mu, sg, r.pp_bounds[2 * p], r.pp_bounds[2 * p + 1]);
    }
}

// k_level_order: the order of the next subject pass's levels, by the
// duration of each level's last crossover resolve, longest first (levels not
// yet measured, and ties, in sub_order's order), so that a level slow for
// its trial count (many rounds, FP64 fallbacks) starts in the first wave.
// with_type (the fused schedule, whose pass types are final here): this
// pass's migration levels first, as k_sub_step claims levels in this order;
// otherwise k_sub_resolve puts them first itself (mig_first_level).  One
// block; a level's rank is the count of larger keys.  Runs beside the
// subject kernels (after the phi level), off the sweep's critical path.
constexpr int kOrderMax = 4096;
__global__ void k_level_order(RunDev r, int with_type)
{
    __shared__ unsigned long long key[kOrderMax];
    const int S = r.S;
    if (S > kOrderMax) return;                   // keep the order as it is
    for (int q = threadIdx.x; q < S; q += blockDim.x) {
        const int l = r.sub_order[q];
        const unsigned long long mig = (with_type && r.ptype[l] == PASS_MIG) ? 1ull : 0ull;
        key[q] = (mig << 62) | ((unsigned long long)(unsigned)max(r.lvl_ns[l], 0) << 20) |
                 (unsigned long long)(S - 1 - q);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < S; q += blockDim.x) {
        const unsigned long long k = key[q];
        int rank = 0;
        for (int j = 0; j < S; ++j) rank += key[j] > k ? 1 : 0;
        r.res_order[rank] = r.sub_order[q];
    }
}

// k_store: theta_class::store (thinned copy of the state into the samples).
__global__ void k_store(RunDev r)
{
    const int64_t it = *r.iter;
    if (it % r.thin != 0) return;
    const int64_t slot = it / r.thin;
    if (slot >= r.nmc) return;
    const int l = blockIdx.x;
    const size_t C = r.C;
    if (l < r.S) {
        const size_t P = r.P;
        double *dt = r.smp_th + ((size_t)l * r.nmc + slot) * C * P;
        const double *st = r.th + (size_t)l * C * P;
        for (size_t j = threadIdx.x; j < C * P; j += blockDim.x) dt[j] = st[j];
        for (size_t j = threadIdx.x; j < C; j += blockDim.x) {
            r.smp_lp[((size_t)l * r.nmc + slot) * C + j] = r.lp[(size_t)l * C + j];
            r.smp_ll[((size_t)l * r.nmc + slot) * C + j] = r.ll[(size_t)l * C + j];
        }
    } else if (r.Pphi > 0) {
        const size_t P = r.Pphi;
        for (size_t j = threadIdx.x; j < C * P; j += blockDim.x)
            r.psmp_th[slot * C * P + j] = r.pth[j];
        for (size_t j = threadIdx.x; j < C; j += blockDim.x) {
            r.psmp_lp[slot * C + j] = r.plp[j];
            r.psmp_ll[slot * C + j] = r.pll[j];
        }
    }
}

__global__ void k_next_iter(RunDev r)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *r.iter += 1;
}

// ------------------------------------------------- batch likelihood API
// theta [S][n_theta][P] -> out [S][n_theta]; grid = S * n_theta.
// k_batch_tables: the FP32 tables of every proposal of a likelihood batch,
// one thread per (proposal, tuple or t0 entry) over the whole GPU.  Built in
// each likelihood block instead, a proposal's tuples keep a few of the
// block's threads busy for the whole double-float chain while the others
// wait (about 15% of the likelihood kernel's time).  bad[] is zeroed first.
__global__ void k_batch_tables(RunDev r, const double *theta, int n_theta, BatchTables bt)
{
    const int NE = r.m.n_ent, NT = r.m.n_t0, NU = NE + NT;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)r.S * n_theta * NU) return;
    const size_t q = i / NU;
    const int u = (int)(i % NU);
    const double *th = theta + q * r.P;
    if (u < NE) {
        Ent32 E;
        double lg;
        if (!entry32(r, th, u, E, lg)) atomicOr(bt.bad + q, 1);
        bt.e[q * NE + u] = E;
        bt.lg[q * NE + u] = lg;
    } else {
        bt.t[q * NT + (u - NE)] = t0split(r, th, u - NE);
    }
}

template <int MINB, int MODEL>
__global__ void __launch_bounds__(kLikThreads, MINB) k_loglik_batch(RunDev r, const double *theta,
                                                                    int n_theta, double *out, BatchTables bt)
{
    extern __shared__ __align__(16) char smem_raw[];
    const int l = blockIdx.x / n_theta, k = blockIdx.x % n_theta;
    const size_t q = (size_t)l * n_theta + k;
    SubSmem sm = carve(smem_raw, r.m);
    const double *th = theta + q * r.P;
    for (int j = threadIdx.x; j < r.P; j += blockDim.x) sm.theta[j] = th[j];
    load_design(r, sm);
    const bool mixed = r.prec == PREC_MIXED;
    if (mixed && bt.e) {
        // the tables k_batch_tables built, as float4 words (3 per tuple)
        const int NE = r.m.n_ent, NT = r.m.n_t0;
        const float4 *src = reinterpret_cast<const float4 *>(bt.e + q * NE);
        float4 *dst = reinterpret_cast<float4 *>(sm.e32);
        for (int u = threadIdx.x; u < 3 * NE; u += blockDim.x) dst[u] = src[u];
        for (int u = threadIdx.x; u < NE; u += blockDim.x) sm.lg[u] = bt.lg[q * NE + u];
        for (int u = threadIdx.x; u < NT; u += blockDim.x) sm.t032[u] = bt.t[q * NT + u];
        if (threadIdx.x == 0) sm.flag[0] = bt.bad[q];
        __syncthreads();
    } else {
        if (threadIdx.x == 0) sm.flag[0] = 0;
        __syncthreads();
        if (mixed) build_tables32(r, sm, 0);
    }
    double ll[kGroup];
    group_loglik<MODEL>(r, l, sm, 1, mixed, ll);
    if (threadIdx.x == 0) out[(size_t)l * n_theta + k] = ll[0];
}

// ------------------------------------- FP64 refinement of sums near zero
// The FP32 form's error in a sum of N trial log densities is a random walk of
// about 1.5e-7 per trial plus a bias below 3e-8 per trial.  A sum whose size
// is below kRefSig sqrt(N) + kRefBias N could therefore be off by more than
// 1e-6 of itself; those sums are recomputed in FP64 (the reference form).
// Their trials are split into chunks of kRefChunk, claimed by a grid-stride
// loop over the whole GPU (a few sums of a few thousand trials would
// otherwise occupy a few SMs for their FP64 work), and each sum is the
// chunks' partial sums added in chunk order.
constexpr int kRefChunk = 256;
constexpr double kRefSig = 1.2, kRefBias = 0.03;

// one thread per (subject, theta) sum: claim its chunks, or base = -1
__global__ void k_refine_flag(RunDev r, const double *out, int n_theta, int32_t *count, int32_t *base,
                              int32_t *item)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= r.S * n_theta) return;
    const int l = q / n_theta;
    const int n = (int)(r.offs[l + 1] - r.offs[l]);
    const double T = kRefSig * sqrt((double)n) + kRefBias * n;
    int b = -1;
    if (n > 0 && !(fabs(out[q]) >= T)) {
        const int nc = (n + kRefChunk - 1) / kRefChunk;
        b = atomicAdd(count, nc);
        for (int c = 0; c < nc; ++c) item[b + c] = q;
    }
    base[q] = b;
}

// chunks of the claimed sums in FP64, grid-stride
__global__ void __launch_bounds__(kLikThreads) k_refine_eval(RunDev r, const double *theta, int n_theta,
                                                             const int32_t *count, const int32_t *base,
                                                             const int32_t *item, double *partial)
{
    extern __shared__ __align__(16) char smem_raw[];
    SubSmem sm = carve(smem_raw, r.m);
    load_design(r, sm);
    const int nw = *count;
    const int K = r.m.n_acc;
    const bool ddm = r.m.model_type == kModelDdm;
    for (int w = blockIdx.x; w < nw; w += gridDim.x) {
        const int q = item[w], c = w - base[q];
        const int l = q / n_theta;
        __syncthreads();                    // the previous item's tables are no longer read
        for (int j = threadIdx.x; j < r.P; j += blockDim.x) sm.theta[j] = theta[(size_t)q * r.P + j];
        __syncthreads();
        if (ddm) ddm_build(r, sm, 0, sm.theta);
        else build_tables64(r, sm, sm.theta);
        __syncthreads();
        const int64_t b0 = r.offs[l];
        const int n = (int)(r.offs[l + 1] - b0);
        const int i1 = min(n, (c + 1) * kRefChunk);
        double acc = 0.0;
        for (int i = c * kRefChunk + threadIdx.x; i < i1; i += blockDim.x) {
            const int cell = r.cell[b0 + i];
            acc += ddm ? ddm_logdens64(r.rt64[b0 + i], sm.d64 + 8 * sm.cent[cell * K])
                       : trial64(r, sm, b0 + i, cell, K);
        }
        const double s = block_sum(acc, sm.red);
        if (threadIdx.x == 0) partial[w] = s;
    }
}

// one thread per sum: the claimed sums' chunks added in order
__global__ void k_refine_sum(RunDev r, int n_theta, const int32_t *base, const double *partial, double *out)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= r.S * n_theta || base[q] < 0) return;
    const int l = q / n_theta;
    const int nc = ((int)(r.offs[l + 1] - r.offs[l]) + kRefChunk - 1) / kRefChunk;
    double s = 0.0;
    for (int c = 0; c < nc; ++c) s += partial[base[q] + c];
    out[q] = s;
}

// per-trial log densities of theta [S][P] -> out [N]; grid = S.
__global__ void __launch_bounds__(kLikThreads) k_trial_logdens(RunDev r, const double *theta,
                                                               double *out)
{
    extern __shared__ __align__(16) char smem_raw[];
    const int l = blockIdx.x;
    SubSmem sm = carve(smem_raw, r.m);
    for (int j = threadIdx.x; j < r.P; j += blockDim.x) sm.theta[j] = theta[(size_t)l * r.P + j];
    load_design(r, sm);
    if (threadIdx.x == 0) sm.flag[0] = 0;
    __syncthreads();
    const bool mixed = r.prec == PREC_MIXED;
    const int64_t base = r.offs[l];
    const int n = (int)(r.offs[l + 1] - base);
    const int K = r.m.n_acc;
    if (r.m.model_type == kModelDdm) {
        ddm_build(r, sm, 0, sm.theta);
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int u = sm.cent[r.cell[base + i] * K];
            const float2 rt = r.rt32[base + i];
            float ld;
            out[base + i] = (mixed && ddm_logdens32(rt.x, rt.y, sm.d32 + 8 * u, ld))
                                ? (double)ld
                                : ddm_logdens64(r.rt64[base + i], sm.d64 + 8 * u);
        }
        return;
    }
    if (mixed) build_tables32(r, sm, 0);
    build_tables64(r, sm, sm.theta);
    __syncthreads();
    const bool use32 = mixed && sm.flag[0] == 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int c = r.cell[base + i];
        if (use32) {
            int ex;
            float lm;
            if (lba_ld32_n(r.rt32[base + i], sm.t032[sm.ct0[c]], sm.cent + c * K, K, sm.e32, ex, lm)) {
                out[base + i] = sm.lg[sm.cent[c * K]] + kLn2 * (double)ex + (double)lm;
                continue;
            }
        }
        out[base + i] = trial64(r, sm, base + i, c, K);
    }
}

// sumlogprior of n vectors against fixed rows; one thread per vector.
// Start-state draws (initialise_theta / initialise_phi, R/phi.R:141-332):
// parameter j of chain c at level v0 + v is the prior's inverse distribution
// function at the keyed uniform (iteration 0, level v0 + v, pass = the pair's
// attempt, slot c * P + j), for the (level, chain) pairs not yet accepted.
// rows: the device prior rows (id, p0, p1, lower, upper, constant).
__device__ __forceinline__ double prior_draw(const double *row, double u)
{
    if ((int)row[0] != 1) return row[1] + u * (row[2] - row[1]);
    const double mu = row[1], sg = row[2], lo = row[3], hi = row[4];
    const double pa = isinf(lo) ? 0.0 : Phi64((lo - mu) / sg);
    const double pb = isinf(hi) ? 1.0 : Phi64((hi - mu) / sg);
    double x = mu + sg * normcdfinv(pa + u * (pb - pa));
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}

__global__ void k_init_draw(const double *rows, int P, int C, int level0, int n_level,
                            const int32_t *attempt, const uint8_t *done, uint64_t seed, double *theta)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n_level * C * P) return;
    const int j = (int)(idx % P);
    const int64_t lc = idx / P;
    if (done[lc]) return;
    const int c = (int)(lc % C), v = (int)(lc / C);
    const DrawSrc ds{nullptr, seed, 1, 1, 1};
    theta[idx] = prior_draw(rows + kPriorRow * j, uniform(ds, 0, level0 + v, attempt[lc], (int64_t)c * P + j));
}

__global__ void k_logprior(const double *rows, int P, const double *theta, int n, double *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int j = 0; j < P; ++j) s += prior_term(rows + kPriorRow * j, theta[(size_t)i * P + j]);
    out[i] = s;
}

// sumloghlike of phi [n][2P] against subject thetas [S][n][P]; one CTA per phi.
__global__ void __launch_bounds__(kPhiThreads) k_loghlike(RunDev r, const double *phi, double *out)
{
    __shared__ double s_phi[kMaxTheta];
    __shared__ double s_cst[2 * kMaxTheta];
    __shared__ double s_red[33];
    const int j = blockIdx.x;
    for (int q = threadIdx.x; q < r.Pphi; q += blockDim.x) s_phi[q] = phi[(size_t)j * r.Pphi + q];
    __syncthreads();
    const double h = hyper_sum(r, s_phi, j, s_cst, s_red);
    if (threadIdx.x == 0) out[j] = h;
}

// ------------------------------------------------------------ launchers
cudaError_t configure_kernels(const DevModel &m)
{
    const int bytes = (int)sub_smem_bytes(m);
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_sub_loglik<GGDMC_LIK_MINB_LBA, kLba4>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
        return e;
    if ((e = cudaFuncSetAttribute(k_sub_loglik<GGDMC_LIK_MINB, kLbaOnly>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
        return e;
    if ((e = cudaFuncSetAttribute(k_sub_loglik<GGDMC_LIK_MINB, kDdmOnly>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
        return e;
    if ((e = cudaFuncSetAttribute(k_sub_resolve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  bytes + (int)res_smem_bytes(kMaxChain) + (int)kJitStage)))
        return e;
    if ((e = cudaFuncSetAttribute(k_sub_spec_rest<GGDMC_LIK_MINB_LBA, kLba4>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
        return e;
    if ((e = cudaFuncSetAttribute(k_sub_spec_rest<GGDMC_LIK_MINB, kLbaOnly>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
        return e;
    if ((e = cudaFuncSetAttribute(k_sub_spec_rest<GGDMC_LIK_MINB, kDdmOnly>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
        return e;
    const size_t step_extra = std::max(res_smem_bytes(kMaxChain) + kJitStage, prop_scratch_bytes(kMaxChain, kMaxTheta));
    if ((e = cudaFuncSetAttribute(k_sub_step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  bytes + (int)step_extra)))
        return e;
    if ((e = cudaFuncSetAttribute(k_loglik_batch<GGDMC_LIK_MINB_LBA, kLba4>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
        return e;
    if ((e = cudaFuncSetAttribute(k_loglik_batch<GGDMC_LIK_MINB, kLbaOnly>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
        return e;
    if ((e = cudaFuncSetAttribute(k_loglik_batch<GGDMC_LIK_MINB, kDdmOnly>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)))
        return e;
    if ((e = cudaFuncSetAttribute(k_refine_eval, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes))) return e;
    return cudaFuncSetAttribute(k_trial_logdens, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t launch_sub_propose(const RunDev &r, int pass, bool defer_prior, bool fused, cudaStream_t st)
{
    k_sub_propose<<<r.S, kProposeThreads, prop_scratch_bytes(r.C, r.P), st>>>(r, pass, defer_prior ? 1 : 0,
                                                                            fused ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_sub_spec_rest(const RunDev &r, int group, cudaStream_t st)
{
    const int bpl = (r.C + group - 1) / group;
    const size_t smem = sub_smem_bytes(r.m);
    if (r.m.model_type == kModelDdm)
        k_sub_spec_rest<GGDMC_LIK_MINB, kDdmOnly><<<r.S * bpl, kLikThreads, smem, st>>>(r, group, bpl);
    else if (r.m.n_acc == 4 && r.lik_variant == 0)
        k_sub_spec_rest<GGDMC_LIK_MINB_LBA, kLba4><<<r.S * bpl, kLikThreads, smem, st>>>(r, group, bpl);
    else
        k_sub_spec_rest<GGDMC_LIK_MINB, kLbaOnly><<<r.S * bpl, kLikThreads, smem, st>>>(r, group, bpl);
    return cudaGetLastError();
}

cudaError_t launch_sub_step(const RunDev &r, bool score_priors, bool defer_next, int group, cudaStream_t st)
{
    const size_t smem = sub_smem_bytes(r.m) + std::max(res_smem_bytes(r.C) + jit_stage_bytes(r.C, r.P),
                                                       prop_scratch_bytes(r.C, r.P));
    // persistent: at most the CTAs that fit on the device at once
    thread_local size_t cached_smem = 0;
    thread_local int cached_grid = 0;
    if (cached_smem != smem) {
        int dev = 0, n_sm = 0, per_sm = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (!e) e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
        if (!e) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sub_step, kResolveThreads, smem);
        if (e) return e;
        cached_grid = std::max(1, n_sm * std::max(1, per_sm));
        cached_smem = smem;
    }
    const int grid = std::min(r.S, cached_grid);
    k_sub_step<<<grid, kResolveThreads, smem, st>>>(r, score_priors ? 1 : 0, defer_next ? 1 : 0, group);
    return cudaGetLastError();
}


cudaError_t launch_sub_loglik(const RunDev &r, const int32_t *items, int n_items, int group,
                              cudaStream_t st)
{
    const size_t smem = sub_smem_bytes(r.m);
    if (r.m.model_type == kModelDdm)
        k_sub_loglik<GGDMC_LIK_MINB, kDdmOnly><<<n_items, kLikThreads, smem, st>>>(r, items, group);
    else if (r.m.n_acc == 4 && r.lik_variant == 0)
        k_sub_loglik<GGDMC_LIK_MINB_LBA, kLba4><<<n_items, kLikThreads, smem, st>>>(r, items, group);
    else
        k_sub_loglik<GGDMC_LIK_MINB, kLbaOnly><<<n_items, kLikThreads, smem, st>>>(r, items, group);
    return cudaGetLastError();
}

cudaError_t launch_sub_resolve(const RunDev &r, int pass, int level_begin, int level_count,
                               bool score_priors, cudaStream_t st)
{
    (void)pass;
    // every subject at once: migration levels first, then the others in
    // res_order (by measured cost, else largest first), unless every level
    // starts in the first wave; a single subject keeps its index
    thread_local int n_sm = 0;
    if (!n_sm) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (!e) e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
        if (e) return e;
    }
    int ordered = 0;
    if (level_count == r.S && level_begin == 0) ordered = (GGDMC_MIG_FIRST && r.S > n_sm) ? 1 : 2;
    const size_t smem = sub_smem_bytes(r.m) + res_smem_bytes(r.C) + jit_stage_bytes(r.C, r.P);
    k_sub_resolve<<<level_count, kResolveThreads, smem, st>>>(r, level_begin, level_count, ordered,
                                                             score_priors ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_phi_tables(const RunDev &r, cudaStream_t st)
{
    k_phi_tables<<<r.C, 32, 0, st>>>(r);
    return cudaGetLastError();
}

cudaError_t launch_level_order(const RunDev &r, bool with_type, cudaStream_t st)
{
    k_level_order<<<1, 256, 0, st>>>(r, with_type ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_phi_propose(const RunDev &r, int pass, cudaStream_t st)
{
    k_phi_propose<<<1, kPhiProposeThreads, 0, st>>>(r, pass);
    return cudaGetLastError();
}

cudaError_t launch_phi_eval(const RunDev &r, cudaStream_t st)
{
    k_phi_eval<<<3 * r.C, kPhiThreads, 0, st>>>(r);
    return cudaGetLastError();
}

cudaError_t launch_phi_resolve(const RunDev &r, int pass, cudaStream_t st)
{
    k_phi_resolve<<<1, kPhiResolveThreads, 0, st>>>(r, pass);
    return cudaGetLastError();
}

cudaError_t launch_store(const RunDev &r, cudaStream_t st)
{
    k_store<<<r.S + (r.Pphi > 0 ? 1 : 0), 256, 0, st>>>(r);
    return cudaGetLastError();
}

cudaError_t launch_next_iter(const RunDev &r, cudaStream_t st)
{
    k_next_iter<<<1, 32, 0, st>>>(r);
    return cudaGetLastError();
}

cudaError_t launch_loglik_batch(const RunDev &r, const double *theta, int n_theta, double *out,
                                cudaStream_t st, const BatchTables *tabs)
{
    const size_t smem = sub_smem_bytes(r.m);
    BatchTables bt{nullptr, nullptr, nullptr, nullptr};
    if (tabs && r.prec == PREC_MIXED && r.m.model_type != kModelDdm) {
        bt = *tabs;
        cudaError_t e = cudaMemsetAsync(bt.bad, 0, sizeof(int32_t) * (size_t)r.S * n_theta, st);
        if (e) return e;
        const size_t n = (size_t)r.S * n_theta * (r.m.n_ent + r.m.n_t0);
        k_batch_tables<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(r, theta, n_theta, bt);
        if ((e = cudaGetLastError())) return e;
    }
    if (r.m.model_type == kModelDdm)
        k_loglik_batch<GGDMC_LIK_MINB, kDdmOnly><<<r.S * n_theta, kLikThreads, smem, st>>>(r, theta, n_theta, out, bt);
    else if (r.m.n_acc == 4)
        k_loglik_batch<GGDMC_LIK_MINB_LBA, kLba4><<<r.S * n_theta, kLikThreads, smem, st>>>(r, theta, n_theta, out, bt);
    else
        k_loglik_batch<GGDMC_LIK_MINB, kLbaOnly><<<r.S * n_theta, kLikThreads, smem, st>>>(r, theta, n_theta, out, bt);
    return cudaGetLastError();
}

size_t refine_capacity(const int64_t *h_offs, int S, int n_theta)
{
    size_t n = 0;
    for (int l = 0; l < S; ++l) n += (size_t)n_theta * (size_t)((h_offs[l + 1] - h_offs[l] + kRefChunk - 1) / kRefChunk);
    return n;
}

cudaError_t launch_refine(const RunDev &r, const double *theta, int n_theta, double *out, int32_t *count,
                          int32_t *base, int32_t *item, double *partial, int grid, cudaStream_t st)
{
    const int nq = r.S * n_theta;
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int32_t), st);
    if (e) return e;
    k_refine_flag<<<(nq + 255) / 256, 256, 0, st>>>(r, out, n_theta, count, base, item);
    if ((e = cudaGetLastError())) return e;
    k_refine_eval<<<grid, kLikThreads, sub_smem_bytes(r.m), st>>>(r, theta, n_theta, count, base, item, partial);
    if ((e = cudaGetLastError())) return e;
    k_refine_sum<<<(nq + 255) / 256, 256, 0, st>>>(r, n_theta, base, partial, out);
    return cudaGetLastError();
}

cudaError_t launch_trial_logdens(const RunDev &r, const double *theta, double *out, cudaStream_t st)
{
    k_trial_logdens<<<r.S, kLikThreads, sub_smem_bytes(r.m), st>>>(r, theta, out);
    return cudaGetLastError();
}

cudaError_t launch_init_draw(const double *rows, int P, int C, int level0, int n_level, const int32_t *attempt,
                             const uint8_t *done, uint64_t seed, double *theta, cudaStream_t st)
{
    const int64_t n = (int64_t)n_level * C * P;
    if (n == 0) return cudaSuccess;
    k_init_draw<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(rows, P, C, level0, n_level, attempt, done, seed, theta);
    return cudaGetLastError();
}

// Posterior summaries of stored samples (summary / gelman, R/model-class.R:
// 370-424, 1559-1690): level l's samples smp [l][nmc][C][P], iterations
// [start, nmc).  Phase 1: per (chain, parameter) the mean and variance
// (Welford, coalesced over the (chain, parameter) pairs of an iteration)
// into cs [l][C][P][2]; phase 2: per parameter the pooled mean and sd and
// the potential scale reduction factor's point estimate in Brooks & Gelman's
// form as coda computes it (chains as the replicates; needs C >= 2).
__global__ void k_summary(const double *smp, int nmc, int C, int P, int start, double *cs,
                          double *mean, double *sd, double *psrf)
{
    const int l = blockIdx.x;
    const int n = nmc - start;
    const double *x = smp + (size_t)l * nmc * C * P;
    double *stat = cs + (size_t)l * C * P * 2;
    for (int q = threadIdx.x; q < C * P; q += blockDim.x) {
        double m = 0.0, m2 = 0.0;
        for (int i = 0; i < n; ++i) {
            const double v = x[(size_t)(start + i) * C * P + q];
            const double dl = v - m;
            m += dl / (i + 1);
            m2 += dl * (v - m);
        }
        stat[2 * q] = m;
        stat[2 * q + 1] = (n > 1) ? m2 / (n - 1) : 0.0;
    }
    __syncthreads();
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        double mu = 0.0, w = 0.0;
        for (int c = 0; c < C; ++c) {
            mu += stat[2 * (c * P + p)];
            w += stat[2 * (c * P + p) + 1];
        }
        mu /= C;
        w /= C;
        double b = 0.0, vw = 0.0, m2bar = 0.0;
        for (int c = 0; c < C; ++c) {
            const double mc = stat[2 * (c * P + p)], sc = stat[2 * (c * P + p) + 1];
            b += (mc - mu) * (mc - mu);
            vw += (sc - w) * (sc - w);
            m2bar += mc * mc;
        }
        m2bar /= C;
        double cov_s_m = 0.0, cov_s_m2 = 0.0;
        for (int c = 0; c < C; ++c) {
            const double mc = stat[2 * (c * P + p)], sc = stat[2 * (c * P + p) + 1];
            cov_s_m += (sc - w) * (mc - mu);
            cov_s_m2 += (sc - w) * (mc * mc - m2bar);
        }
        const double varm = b / (C - 1);                  // var of the chain means
        b = n * varm;
        const double var_w = vw / (C - 1) / C;
        const double var_b = 2.0 * b * b / (C - 1);
        const double cov_wb = ((double)n / C) * (cov_s_m2 / (C - 1) - 2.0 * mu * cov_s_m / (C - 1));
        const double V = (n - 1.0) / n * w + (1.0 + 1.0 / C) / n * b;
        const double var_V = ((n - 1.0) * (n - 1.0) * var_w + (1.0 + 1.0 / C) * (1.0 + 1.0 / C) * var_b +
                              2.0 * (n - 1.0) * (1.0 + 1.0 / C) * cov_wb) / ((double)n * n);
        const double df_V = 2.0 * V * V / var_V;
        const double df_adj = (df_V + 3.0) / (df_V + 1.0);
        const double r2 = (n - 1.0) / n + (1.0 + 1.0 / C) / n * (b / w);
        // pooled over chains and iterations
        const double tot = (double)n * C;
        const double ss = (n - 1.0) * w * C + n * varm * (C - 1);
        mean[(size_t)l * P + p] = mu;
        sd[(size_t)l * P + p] = sqrt(ss / (tot - 1.0));
        psrf[(size_t)l * P + p] = sqrt(df_adj * r2);
    }
}

cudaError_t launch_summary(const double *smp, int L, int nmc, int C, int P, int start, double *cs,
                           double *mean, double *sd, double *psrf, cudaStream_t st)
{
    if (L < 1) return cudaSuccess;
    k_summary<<<L, 256, 0, st>>>(smp, nmc, C, P, start, cs, mean, sd, psrf);
    return cudaGetLastError();
}

// FP32 (hi, lo) split of each response time: hi = RT rounded to FP32, lo =
// the rest rounded to FP32 (as the host would form it).
__global__ void k_split_rt(const double *rt, int64_t n, float2 *out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = rt[i];
        const float hi = __double2float_rn(x);
        out[i] = make_float2(hi, __double2float_rn(x - (double)hi));
    }
}

cudaError_t launch_split_rt(const double *rt, int64_t n, float2 *out, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 4096);
    k_split_rt<<<(unsigned)blocks, 256, 0, st>>>(rt, n, out);
    return cudaGetLastError();
}

cudaError_t launch_logprior(const double *rows, int P, const double *theta, int n, double *out,
                            cudaStream_t st)
{
    k_logprior<<<(n + 127) / 128, 128, 0, st>>>(rows, P, theta, n, out);
    return cudaGetLastError();
}

cudaError_t launch_loghlike(const RunDev &r, const double *phi, double *out, cudaStream_t st)
{
    k_loghlike<<<r.C, kPhiThreads, 0, st>>>(r, phi, out);
    return cudaGetLastError();
}

}  // namespace ggdmc
