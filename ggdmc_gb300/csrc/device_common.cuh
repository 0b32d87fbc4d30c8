// device_common.cuh -- draws, normal functions and the per-trial LBA densities
// shared by the sampler kernels (sm_103a).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "model_tables.h"

namespace ggdmc {

// ----------------------------------------------------------------- draws
// Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11), counter = (slot, pass,
// level, iteration), key = seed.  The 52-bit uniform ((m + 0.5) * 2^-52) is
// exactly representable, so every consumer of a draw sees the same double.
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
        const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}

struct DrawSrc {
    const double *draws;   // host-fed canonical array, or nullptr
    uint64_t seed;
    int64_t n_level, n_pass, n_slot;
};

__device__ __forceinline__ double uniform(const DrawSrc &d, int64_t it, int64_t level,
                                          int64_t pass, int64_t slot)
{
    if (d.draws)
        return d.draws[(((it - 1) * d.n_level + level) * d.n_pass + pass) * d.n_slot + slot];
    uint32_t c[4] = {(uint32_t)slot, (uint32_t)pass, (uint32_t)level, (uint32_t)it};
    philox4x32_10(c, (uint32_t)d.seed, (uint32_t)(d.seed >> 32));
    const uint64_t m = ((uint64_t)c[0] << 20) | (c[1] >> 12);
    return __dmul_rn((double)m + 0.5, 0x1p-52);
}

// -------------------------------------------------------------- normals
__device__ __forceinline__ double Phi64(double z) { return 0.5 * erfc(-z * 0.70710678118654752440); }
__device__ __forceinline__ double phi64(double z) { return exp(-0.5 * z * z) * 0.39894228040143267794; }
// phi in FP32 with the square split exactly (z*z = h + l), so the exponent
// keeps full relative accuracy for large |z|: exp(-h/2) (1 - l/2).
__device__ __forceinline__ float phi32(float z)
{
    const float h = z * z, l = fmaf(z, z, -h);
    const float e = expf(-0.5f * h) * 0.398942280f;
    return fmaf(e, -0.5f * l, e);
}

// Mills ratio M(x) = Q(x)/phi(x), x >= 0: rational P4/Q5 fitted for minimax
// relative error on [0, 14] (fit_mills.py; 5.5e-9 exact, 3.2e-7 in FP32).
// Beyond 14, phi(x) underflows FP32, so the clamp does not change a product.
__device__ __forceinline__ float mills32(float x)
{
    x = fminf(x, 14.f);
    const float p = fmaf(fmaf(fmaf(fmaf(__int_as_float(0x3c2779df), x, __int_as_float(0x3dcf447b)), x,
                                   __int_as_float(0x3eea2de0)), x, __int_as_float(0x3f8c4b52)), x,
                         __int_as_float(0x3fa06c99));
    const float q = fmaf(fmaf(fmaf(fmaf(fmaf(__int_as_float(0x3c277955), x, __int_as_float(0x3dcf480d)), x,
                                        __int_as_float(0x3eef5540)), x, __int_as_float(0x3f99834b)), x,
                              __int_as_float(0x3fd61160)), x, 1.f);
    return __fdividef(p, q);
}

// Phi(x) from phx = phi(x): the lower tail phi(x) M(-x) for x < 0, else
// 1 - phi(x) M(x).
__device__ __forceinline__ float ncdf32(float x, float phx)
{
    const float t = phx * mills32(fabsf(x));
    return (x < 0.f) ? t : 1.f - t;
}

// ------------------------------------------------------ FP64 LBA trial
// The reference form (ggdmcLikelihood, restated): node-1 pdf floored at
// 1e-10, t <= 0 gives 1e-10, a non-positive product gives DBL_EPSILON.
// e64[u] = (A, b, v, s, Phi(v/s)) of unique accumulator tuple u.
__device__ __forceinline__ double lba_logdens64(double t, const int *ents, int K, int w,
                                                const double *e64)
{
    if (!(t > 0.0)) return -23.025850929940456840;   // log(1e-10)
    double pdf = 0.0, surv = 1.0;
    for (int k = 0; k < K; ++k) {
        const double *e = e64 + 5 * ents[k];
        const double A = e[0], b = e[1], v = e[2], s = e[3], den = e[4];
        const double ts = __dmul_rn(t, s);
        const double chim = __dsub_rn(b, __dmul_rn(t, v)), xx = __dsub_rn(chim, A);
        const double cz = __ddiv_rn(chim, ts), czm = __ddiv_rn(xx, ts);
        if (k == w) {
            const double f = __ddiv_rn(__dadd_rn(__dmul_rn(v, __dsub_rn(Phi64(cz), Phi64(czm))),
                                                 __dmul_rn(s, __dsub_rn(phi64(czm), phi64(cz)))), A);
            pdf = __ddiv_rn(f, den);
        } else {
            const double in = __dsub_rn(__dadd_rn(__dmul_rn(ts, __dsub_rn(phi64(czm), phi64(cz))),
                                                  __dmul_rn(xx, Phi64(czm))),
                                        __dmul_rn(chim, Phi64(cz)));
            const double F = __dadd_rn(1.0, __ddiv_rn(in, A));
            surv = __dmul_rn(surv, __dsub_rn(1.0, __ddiv_rn(F, den)));
        }
    }
    if (!(pdf > 1e-10)) pdf = 1e-10;
    double d = __dmul_rn(pdf, surv);
    if (!(d > 0.0)) d = 2.220446049250313080847e-16;
    return log(d);
}

// The winner's density in FP32.  When both normal arguments are >= 0 the
// density is a sum of same-sign upper-tail terms, each relative-accurate in
// FP32 (Mills-ratio tails), so a small density is exact enough; only one
// within 0.1% of the reference's 1e-10 floor is re-evaluated (the floor
// decision must agree), and one below is floored here.  Otherwise (a slow
// response) the two terms cancel to leading order and a density below 1e-8
// is re-evaluated in FP64.
__device__ __forceinline__ bool winner_pdf_usable(bool fast, float &pdf)
{
    if (!fast) return pdf >= 1e-8f;
    if (pdf > 1.001e-10f) return true;
    if (pdf < 0.999e-10f) {       // also 0 and underflowed tails
        pdf = 1e-10f;
        return true;
    }
    return false;                  // near the floor, or NaN
}

// ------------------------------------------------------ FP32 LBA trial
// e32a[u] = (beta = b/s, betam = (b-A)/s, kappa = v/s, cs = s/(A Phi(v/s)))
// e32b[u] = (cv = v/(A Phi(v/s)), q = Phi(-v/s)/Phi(v/s))
// z = beta/t - kappa.  Winner: pdf = cv*(Phi(cz)-Phi(czm)) + cs*(phi(czm)-phi(cz)),
// with the difference taken on the upper tail when czm >= 0.  Loser survivor:
// late (cz < 0) t*cs*(phi(cz)-phi(czm) + cz Phi(cz) - czm Phi(czm)) - q,
// early 1 - t*cs*(cz Q(cz) - czm Q(czm) + phi(czm) - phi(cz)).
// Returns false when the trial must be re-evaluated in FP64: a survivor in
// the range where either form loses digits, a pdf near the 1e-10 floor, a
// non-positive product or t below 1e-4 s.
__device__ __forceinline__ bool lba_logdens32(float t, const uint8_t *ents, int K, int w,
                                              const float4 *e32a, const float2 *e32b,
                                              float &ld)
{
    if (!(t > 1e-4f)) return false;
    const float it = __frcp_rn(t);
    float pdf;
    bool pdf_ok;
    {
        const float4 a = e32a[ents[w]];
        const float2 b = e32b[ents[w]];
        const float cz = fmaf(a.x, it, -a.z), czm = fmaf(a.y, it, -a.z);
        const float pz = phi32(cz), pm = phi32(czm);
        const bool fast = czm >= 0.f;
        const float sg = fast ? -1.f : 1.f;
        const float d = sg * (ncdf32(sg * cz, pz) - ncdf32(sg * czm, pm));
        pdf = fmaf(b.x, d, a.w * (pm - pz));
        pdf_ok = winner_pdf_usable(fast, pdf);
    }
    float surv = 1.f;
    bool bad = false;
    for (int j = 0; j < K - 1; ++j) {
        const int k = (j < w) ? j : j + 1;
        const float4 a = e32a[ents[k]];
        const float2 b = e32b[ents[k]];
        const float cz = fmaf(a.x, it, -a.z), czm = fmaf(a.y, it, -a.z);
        const float pz = phi32(cz), pm = phi32(czm);
        const bool late = cz < 0.f;
        const float sg = late ? 1.f : -1.f;
        const float br = fmaf(cz, ncdf32(sg * cz, pz), -czm * ncdf32(sg * czm, pm)) + sg * (pz - pm);
        const float tcs = t * a.w;
        const float S = late ? fmaf(tcs, br, -b.y) : fmaf(-tcs, br, 1.f);
        surv *= S;
        // Early, S = 1 - F cancels as F -> 1; late, S1/Phi(v/s) - q cancels as
        // S1 -> Phi(-v/s); below 1e-9 the reference's own FP64 form loses its
        // digits (it cancels to <= 0 and takes DBL_EPSILON), so follow it there.
        bad |= late ? !(S >= 1e-9f && S * 32.f >= b.y) : !(S >= 1e-2f);
    }
    const float d = pdf * surv;
    if (bad || !pdf_ok || !(d >= 1.2e-38f) || !(d < 3.0e38f)) return false;
    ld = __logf(d);
    return true;
}

// lba_logdens32 for a fixed accumulator count, with the cell's entry ids in
// registers, winner first (the host stores each cell's entries that way).
template <int K>
__device__ __forceinline__ bool lba_logdens32_k(float t, const int (&ent)[K], const float4 *e32a,
                                                const float2 *e32b, float &ld)
{
    if (!(t > 1e-4f)) return false;
    const float it = __frcp_rn(t);
    float pdf;
    bool pdf_ok;
    {
        const float4 a = e32a[ent[0]];
        const float2 b = e32b[ent[0]];
        const float cz = fmaf(a.x, it, -a.z), czm = fmaf(a.y, it, -a.z);
        const float pz = phi32(cz), pm = phi32(czm);
        const bool fast = czm >= 0.f;
        const float sg = fast ? -1.f : 1.f;
        const float d = sg * (ncdf32(sg * cz, pz) - ncdf32(sg * czm, pm));
        pdf = fmaf(b.x, d, a.w * (pm - pz));
        pdf_ok = winner_pdf_usable(fast, pdf);
    }
    float surv = 1.f;
    bool bad = false;
#pragma unroll
    for (int k = 1; k < K; ++k) {
        const float4 a = e32a[ent[k]];
        const float2 b = e32b[ent[k]];
        const float cz = fmaf(a.x, it, -a.z), czm = fmaf(a.y, it, -a.z);
        const float pz = phi32(cz), pm = phi32(czm);
        const bool late = cz < 0.f;
        const float sg = late ? 1.f : -1.f;
        const float br = fmaf(cz, ncdf32(sg * cz, pz), -czm * ncdf32(sg * czm, pm)) + sg * (pz - pm);
        const float tcs = t * a.w;
        const float S = late ? fmaf(tcs, br, -b.y) : fmaf(-tcs, br, 1.f);
        surv *= S;
        bad |= late ? !(S >= 1e-9f && S * 32.f >= b.y) : !(S >= 1e-2f);
    }
    const float d = pdf * surv;
    if (bad || !pdf_ok || !(d >= 1.2e-38f) || !(d < 3.0e38f)) return false;
    ld = __logf(d);
    return true;
}

// ------------------------------------------------------ DDM trial
// Navarro & Fuss (2009) first-passage density of the Wiener process at the
// lower boundary, with the series length chosen from its error bounds;
// drift variability sv integrated in closed form, start-point (sz) and
// non-decision-time (st0) variability by the midpoint rule on kDdmNz x kDdmNt
// nodes.  The entry of a (cell, proposal) holds the responding boundary's
// mirrored values: p[0] a, p[1] v (negated for the upper boundary), p[2] z/a
// (1 - z/a for the upper), p[3] the response's non-decision time
// (t0 - d/2 upper, t0 + d/2 lower), p[4] sz, p[5] sv, p[6] st0.
constexpr int kDdmNz = 8, kDdmNt = 8;
constexpr double kDdmEps = 1e-10;

__device__ __forceinline__ double nf_density64(double tt, double w)
{
    if (!(tt > 0.0)) return 0.0;
    const double pi = 3.14159265358979323846;
    double ks, kl;
    if (pi * tt * kDdmEps < 1.0) {
        kl = sqrt(-2.0 * log(pi * tt * kDdmEps) / (pi * pi * tt));
        const double lb = 1.0 / (pi * sqrt(tt));
        if (kl < lb) kl = lb;
    } else {
        kl = 1.0 / (pi * sqrt(tt));
    }
    if (2.0 * sqrt(2.0 * pi * tt) * kDdmEps < 1.0) {
        ks = 2.0 + sqrt(-2.0 * tt * log(2.0 * sqrt(2.0 * pi * tt) * kDdmEps));
        const double lb = sqrt(tt) + 1.0;
        if (ks < lb) ks = lb;
    } else {
        ks = 2.0;
    }
    double p = 0.0;
    if (ks < kl) {
        const int K = (int)ceil(ks);
        for (int k = -((K - 1) / 2); k <= (K - 1) / 2; ++k) {
            const double x = w + 2.0 * k;
            p += x * exp(-(x * x) / (2.0 * tt));
        }
        p /= sqrt(2.0 * pi * tt * tt * tt);
    } else {
        const int K = (int)ceil(kl);
        for (int k = 1; k <= K; ++k) p += k * exp(-(double)(k * k) * (pi * pi * tt / 2.0)) * sinpi(k * w);
        p *= pi;
    }
    return p;
}

__device__ __forceinline__ double ddm_fixed64(double t, double a, double v, double w, double sv)
{
    if (!(t > 0.0)) return 0.0;
    const double g = nf_density64(t / (a * a), w) / (a * a);
    const double den = 1.0 + sv * sv * t;
    const double e = (sv * sv * (a * w) * (a * w) - 2.0 * v * a * w - v * v * t) / (2.0 * den);
    return g * exp(e) / sqrt(den);
}

__device__ __forceinline__ double ddm_logdens64(double rt, const double *p)
{
    const double a = p[0], v = p[1], zr = p[2], tshift = p[3], sz = p[4], sv = p[5], st0 = p[6];
    const int nz = (sz > 0.0) ? kDdmNz : 1;
    const int nt = (st0 > 0.0) ? kDdmNt : 1;
    double acc = 0.0;
    for (int it = 0; it < nt; ++it) {
        const double tu = (nt > 1) ? tshift + st0 * ((it + 0.5) / nt) : tshift;
        const double tt = rt - tu;
        if (!(tt > 0.0)) continue;
        for (int iz = 0; iz < nz; ++iz) {
            const double zz = (nz > 1) ? zr + sz * ((iz + 0.5) / nz - 0.5) : zr;
            acc += ddm_fixed64(tt, a, v, zz, sv);
        }
    }
    double dens = acc / (double)(nz * nt);
    if (!(dens > 1e-10)) dens = 1e-10;
    return log(dens);
}

// FP32 form of the same density: the series lengths from the same bounds
// evaluated in FP32, the terms and the node sum in FP32.  The series choice,
// its length and the large-time exponentials depend on the decision time
// only, so they are formed once per non-decision-time node and shared by the
// start-point nodes.  Returns false (re-evaluate in FP64) below 1e-8, where
// the 1e-10 floor is near, or when a value is not finite.
struct Nf32 {
    bool small;          // small-time series
    int K;               // its length
    float i2t, norm;     // small time: 1 / (2 tt), (2 pi tt^3)^-1/2
    float ek[8];         // large time: k exp(-k^2 pi^2 tt / 2), k = 1..8
    float c;             // large time: pi^2 tt / 2 (terms past 8)
};

__device__ __forceinline__ void nf32_prepare(float tt, Nf32 &q)
{
    const float pi = 3.14159265f;
    const float ek = pi * tt * 1e-10f;
    const float kl = (ek < 1.f) ? fmaxf(sqrtf(-2.f * __logf(ek) / (pi * pi * tt)), 1.f / (pi * sqrtf(tt)))
                                : 1.f / (pi * sqrtf(tt));
    const float es = 2.f * sqrtf(2.f * pi * tt) * 1e-10f;
    const float ks = (es < 1.f) ? fmaxf(2.f + sqrtf(-2.f * tt * __logf(es)), sqrtf(tt) + 1.f) : 2.f;
    q.small = ks < kl;
    q.K = (int)ceilf(q.small ? ks : kl);
    q.i2t = 0.5f / tt;
    q.norm = rsqrtf(2.f * pi * tt * tt * tt);
    q.c = pi * pi * tt * 0.5f;
    if (!q.small) {
#pragma unroll
        for (int k = 1; k <= 8; ++k) q.ek[k - 1] = (float)k * expf(-(float)(k * k) * q.c);
    }
}

__device__ __forceinline__ float nf32_eval(const Nf32 &q, float w)
{
    float p = 0.f;
    if (q.small) {
        for (int k = -((q.K - 1) / 2); k <= (q.K - 1) / 2; ++k) {
            const float x = w + 2.f * k;
            p = fmaf(x, expf(-(x * x) * q.i2t), p);
        }
        return p * q.norm;
    }
#pragma unroll
    for (int k = 1; k <= 8; ++k)
        if (k <= q.K) p = fmaf(q.ek[k - 1], sinpif(k * w), p);
    for (int k = 9; k <= q.K; ++k) p = fmaf((float)k * expf(-(float)(k * k) * q.c), sinpif(k * w), p);
    return p * 3.14159265f;
}

__device__ __forceinline__ bool ddm_logdens32(float rt_hi, float rt_lo, const float *p, float &ld)
{
    const float a = p[0], v = p[1], zr = p[2], sz = p[4], sv = p[5], st0 = p[6];
    const float ia2 = 1.f / (a * a), sv2 = sv * sv;
    const int nz = (sz > 0.f) ? kDdmNz : 1;
    const int nt = (st0 > 0.f) ? kDdmNt : 1;
    float acc = 0.f;
    for (int it = 0; it < nt; ++it) {
        // decision time from the (hi, lo) split of rt and tshift (p[3], p[7])
        const float tu = (nt > 1) ? st0 * ((it + 0.5f) / nt) : 0.f;
        const float tt = ((rt_hi - p[3]) + (rt_lo - p[7])) - tu;
        if (!(tt > 0.f)) continue;
        const float den = fmaf(sv2, tt, 1.f);
        const float rden = rsqrtf(den), hden = 0.5f / den;
        Nf32 q;
        nf32_prepare(tt * ia2, q);
        float part = 0.f;
        for (int iz = 0; iz < nz; ++iz) {
            const float zz = (nz > 1) ? fmaf(sz, (iz + 0.5f) / nz - 0.5f, zr) : zr;
            const float g = nf32_eval(q, zz) * ia2;
            const float aw = a * zz;
            const float e = (fmaf(sv2 * aw, aw, -2.f * v * aw) - v * v * tt) * hden;
            part = fmaf(g, expf(e), part);
        }
        acc = fmaf(part, rden, acc);
    }
    const float dens = acc / (float)(nz * nt);
    if (!(dens >= 1e-8f) || !(dens < 3.0e38f)) return false;
    ld = __logf(dens);
    return true;
}

}  // namespace ggdmc
