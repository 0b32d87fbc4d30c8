// device_common.cuh -- draws, normal functions and the per-trial LBA densities
// shared by the sampler kernels (sm_103a).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "dfloat.h"
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

// ------------------------------------------------------ FP32 LBA trial
// The trial density d = pdf_w(t) prod_{k != w} S_k(t) of the reference form
// (lba_logdens64), evaluated in FP32 so that its log is within ~1e-7 of the
// FP64 value per trial with a bias below 1e-8, so that sums over thousands of
// trials stay within 1e-6 relative.  In terms of z = beta/t - kappa
// (beta = b/s, kappa = v/s), cz at b and czm at b - A, h = (cz - czm)/2 =
// A/(2 s t), m = (cz + czm)/2 and g = s/(A Phi(kappa)):
//
//   pdf_w = g * br,  br = kappa (Phi(cz) - Phi(czm)) + phi(czm) - phi(cz)
//                       = integral over [czm, cz] of (z + kappa) phi(z)
//   S_k   = 1 - g t int Q  (early, cz >= 0)  =  g t int Phi - q  (late, cz < 0)
//         = avg Phi - q avg Q over [czm, cz],  q = Phi(-kappa)/Phi(kappa)
//
// Where the interval is narrow (h max(1, |m|) < 1/8: small A or slow
// responses) the closed forms cancel, so the integrals are taken by 3-node
// Gauss-Legendre quadrature about m, whose truncation error is below 2e-9
// there.  Accuracy measures, each of which removed a measured bias:
//  - t = RT - t0, u = 1/t and the z values are double-float (hi + lo), so
//    exp(-z^2/2) keeps full accuracy out to the tails (its error is z dz);
//  - every per-proposal constant is formed in FP64 and kept as a hi + lo pair
//    where its rounding would scale all trials alike (beta, betam, kappa, hA,
//    g, q); log g of the winner enters the sum in FP64, once per cell;
//  - 1/sqrt(2 pi) is applied as a hi + lo pair, the Mills ratio's mean
//    relative bias (-1.45e-8 over [0, 14]) is removed, the quadrature weights
//    sum to 1 exactly;
//  - the log is split: d = m 2^e, e summed as an integer, log m from the
//    series 2 atanh((m-1)/(m+1)) on [sqrt(1/2), sqrt(2)).
// A trial is left to the FP64 form (returns false) where FP32 cannot follow
// the reference form: t < 1e-4; a winner bracket or survivor that cancels by
// more than 16x; a pdf within 0.1% of the reference's 1e-10 floor (below it
// the pdf is floored here); where the reference form's own FP64 rounding
// exceeds 1e-6 relative in the winner's bracket (it differences Phi values
// near 1) or 1e-8 in a survivor (terms much larger than the survivor), so
// that the value follows the reference; and a product outside the normal
// FP32 range.
//
// Per proposal and accumulator tuple (the host builds them in FP64):
struct Ent32 {
    float4 a;   // beta_h, fe, kappa_h, hA_h      hA = A / (2 s)
    float4 b;   // beta_l, flm, kappa_l, hA_l     (low parts); fe ln 2 + flm = log 1e-10 - log g,
                //                                 the floor of a trial before t0 (t_before)
    float4 c;   // g_h, g_l, q_h, q_l
};

// The FP32 tuple of an accumulator (A, B, v, s) in double-float (dfloat.h)
// and the FP64 log g; false: outside the FP32 form's domain (the proposal
// is evaluated in FP64).
__device__ __forceinline__ bool lba_tuple32(double A, double B, double v, double s, Ent32 &E, double &lg)
{
    const dfl Ad = df_from_double(A), Bd = df_from_double(B), sd = df_from_double(s);
    const dfl is = df_div(dfl{1.f, 0.f}, sd);
    const dfl kap = df_mul(df_from_double(v), is);
    dfl den, qt;                                    // Phi(kappa), Phi(-kappa)
    df_phi_pair(kap, den, qt);
    const dfl g = df_div(sd, df_mul(Ad, den)), q = df_div(qt, den);
    const dfl ab = df_mul(df_add(Ad, Bd), is), bs = df_mul(Bd, is), ha = df_mul_f(df_mul(Ad, is), 0.5f);
    // (FP32 tests of A and s: a value too small for FP32 goes to the FP64 form)
    const bool ok = Ad.h > 0.f && sd.h > 0.f && den.h > 1e-30f && isfinite(ab.h) && isfinite(bs.h) &&
                    isfinite(kap.h) && isfinite(g.h) && isfinite(q.h) && ha.h > 0.f && g.h > 0.f;
    const dfl lgd = ok ? df_log(g) : dfl{0.f, 0.f};
    lg = df_to_double(lgd);
    // the density floor of a trial before t0 in the trial form, less log g:
    // log 1e-10 - log g = fe ln 2 + flm (fe an integer, |flm| <= ln 2 / 2),
    // in double-float (log 1e-10 as hi + lo)
    const dfl fx = df_add(dfl{-23.025850296020508f, -6.339199671856477e-07f}, df_neg(lgd));
    const float fe = rintf(fx.h * 1.44269504088896341f);
    const dfl fl = df_add(fx, df_neg(df_mul_f(dfl{kDfLn2H, kDfLn2L}, fe)));
    E.a = make_float4(ab.h, fe, kap.h, ha.h);
    E.b = make_float4(ab.l, fl.h + fl.l, kap.l, ha.l);
    E.c = make_float4(g.h, g.l, q.h, q.l);
    return ok;
}

constexpr float kPhiC = 0.398942280401432678f;            // 1/sqrt(2 pi), hi
constexpr float kPhiCl = -1.13351701e-8f;                  // 1/sqrt(2 pi) - kPhiC
constexpr float kGlX1 = 0.774596669241483f;                // sqrt(3/5)
constexpr float kGlW1 = 0.277777791f;                      // 5/18 in FP32
constexpr float kGlW0 = 0.444444418f;                      // 1 - 2 kGlW1, exactly
constexpr float kGlMax = 0.125f;                           // h max(1,|m|) below: quadrature
constexpr float kAmp = 16.f;                               // cancellation allowed
constexpr float kMillsBias = 1.45e-8f;                     // mean relative bias removed
constexpr double kLn2 = 0.693147180559945309417;

// a - b as hi + lo (Knuth's two-sum)
__device__ __forceinline__ void two_diff(float a, float b, float &s, float &e)
{
    s = a - b;
    const float bb = s - a;
    e = (a - (s - bb)) - (b + bb);
}

// z = beta u - kappa in double-float (beta, u, kappa as hi + lo), normalised
__device__ __forceinline__ void zdf(float bh, float bl, float uh, float ul, float kh, float kl,
                                    float &zh, float &zl)
{
    const float p = bh * uh;
    float pe = fmaf(bh, uh, -p);
    pe = fmaf(bh, ul, pe);
    pe = fmaf(bl, uh, pe);
    float s, e;
    two_diff(p, kh, s, e);
    const float l = e + (pe - kl);
    zh = s + l;
    zl = l - (zh - s);
}

// czm = cz - 2h = betam u - kappa from cz and h = hA u (each hi + lo),
// normalised: betam = beta - 2 hA, so the second product is not needed
__device__ __forceinline__ void zlower(float czh, float czl, float h, float hc, float &zh, float &zl)
{
    float s, e;
    two_diff(czh, 2.f * h, s, e);
    const float l = e + (czl - 2.f * hc);
    zh = s + l;
    zl = l - (zh - s);
}

// phi(z) of a double-float z: exp(-zh^2/2) (1 - zh zl - (zh^2 - fl(zh^2))/2) / sqrt(2 pi)
__device__ __forceinline__ float phidf(float zh, float zl)
{
    const float hh = zh * zh, hl = fmaf(zh, zh, -hh);
    const float e0 = expf(-0.5f * hh);
    const float e = fmaf(e0, kPhiC, e0 * kPhiCl);
    return fmaf(e, fmaf(-zh, zl, -0.5f * hl), e);
}

// The normal tail beyond z (upper for z >= 0, lower for z < 0) from phi(z).
__device__ __forceinline__ float ntail(float z, float ph)
{
    const float m = mills32(fabsf(z));
    return ph * fmaf(m, kMillsBias, m);
}

// P = m 2^e with m in [sqrt(1/2), sqrt(2)); returns log m.  P > 0, normal.
__device__ __forceinline__ float log_split(float P, int &e)
{
    const unsigned bits = __float_as_uint(P);
    e = (int)(bits >> 23) - 127;
    float m = __uint_as_float((bits & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) {
        m *= 0.5f;
        ++e;
    }
    const float s = __fdividef(m - 1.f, m + 1.f), s2 = s * s;
    const float poly = fmaf(fmaf(fmaf(fmaf(2.f / 11.f, s2, 2.f / 9.f), s2, 2.f / 7.f), s2, 2.f / 5.f), s2,
                            2.f / 3.f);
    return fmaf(s * s2, poly, 2.f * s);
}

// Winner bracket br (pdf = g br) of one accumulator; false: FP64 form.
__device__ __forceinline__ bool winner_br(const Ent32 &P, float uh, float ul, float &br)
{
    float czh, czl, cmh, cml;
    zdf(P.a.x, P.b.x, uh, ul, P.a.z, P.b.z, czh, czl);
    const float h = P.a.w * uh, hc = fmaf(P.a.w, ul, P.b.w * uh);
    zlower(czh, czl, h, hc, cmh, cml);
    const float mh = czh - h, ml = (czl - hc) + ((czh - mh) - h);
    float ref;   // the reference form's FP64 rounding in its bracket
    if (h * fmaxf(1.f, fabsf(mh)) < kGlMax) {
        const float pm = phidf(mh, ml);
        const float hx = h * kGlX1, a = hx * mh, c = 0.5f * hx * hx;
        const float ep = expf(a - c), em = expf(-a - c);          // phi(m -/+ hx) / phi(m)
        const float mk = (mh + P.a.z) + (ml + P.b.z);            // m + kappa
        const float inner = fmaf(kGlW1, fmaf(mk + hx, em, (mk - hx) * ep), kGlW0 * mk);
        const float y = 2.f * pm * inner, x2 = fmaf(y, uh, y * ul);
        br = fmaf(P.a.w, x2, P.b.w * x2);
        const float phimax = (mh < -1.f) ? pm / -mh : 1.f;       // Phi(m) <= phi(m) / |m|
        ref = 1.1e-16f * (fabsf(P.a.z) * phimax + 2.f * pm);
        if (!(br > 0.f)) return false;
    } else {
        const float pz = phidf(czh, czl), pm = phidf(cmh, cml);
        const float tz = ntail(czh, pz), tm = ntail(cmh, pm);
        const bool fast = cmh >= 0.f;
        const float phimax = fast ? 1.f : ((czh < 0.f) ? tz : 1.f - tz);
        const float dP = fast ? tm - tz : phimax - tm, dp = pm - pz;
        br = fmaf(P.a.z, dP, fmaf(P.b.z, dP, dp));
        ref = 1.1e-16f * (fabsf(P.a.z) * phimax + pm + pz);
        // A response far too fast for the winner (both z beyond 13): phi
        // underflows FP32 there (phi(13) < 8.0e-38) and the bracket is at
        // most (|kappa| / czm + 1) phi(czm).  When that bound puts the pdf
        // below 1e-10, the reference's pdf (at most g phi(czm)) is floored
        // too, so the trial takes the floor here instead of the FP64 form.
        if (cmh > 13.f && P.c.x * fmaf(fabsf(P.a.z), 0.0769231f, 1.f) < 1.2e27f) {
            br = __fdividef(1e-10f, P.c.x);
            return true;
        }
        if (!(br > 0.f) || !(br * kAmp >= fabsf(P.a.z * dP) + fabsf(dp))) return false;
    }
    const float pdf = br * P.c.x;
    if (pdf < 0.999e-10f) {
        br = __fdividef(1e-10f, P.c.x);     // the reference's floor
        return true;
    }
    return pdf >= 1.001e-10f && br * 1e-6f >= ref;
}

// Survivor S of a losing accumulator; false: FP64 form.
__device__ __forceinline__ bool loser_s(const Ent32 &P, float th, float tl, float uh, float ul, float &S)
{
    float czh, czl, cmh, cml;
    zdf(P.a.x, P.b.x, uh, ul, P.a.z, P.b.z, czh, czl);
    const float h = P.a.w * uh, hc = fmaf(P.a.w, ul, P.b.w * uh);
    zlower(czh, czl, h, hc, cmh, cml);
    const float mh = czh - h, ml = (czl - hc) + ((czh - mh) - h);
    float terms;   // the reference's survivor sums terms of this size, scaled 1/(2h)
    bool ok;
    if (h * fmaxf(1.f, fabsf(mh)) < kGlMax) {
        const float p0 = phidf(mh, ml);
        const float hx = h * kGlX1, a = hx * mh, c = 0.5f * hx * hx;
        const float zp = mh + hx, zn = mh - hx;
        const float pp = p0 * expf(-a - c), pn = p0 * expf(a - c);
        const float t0 = ntail(mh, p0), tp = ntail(zp, pp), tn = ntail(zn, pn);
        const float P0 = (mh < 0.f) ? t0 : 1.f - t0, Q0 = (mh < 0.f) ? 1.f - t0 : t0;
        const float Pp = (zp < 0.f) ? tp : 1.f - tp, Qp = (zp < 0.f) ? 1.f - tp : tp;
        const float Pn = (zn < 0.f) ? tn : 1.f - tn, Qn = (zn < 0.f) ? 1.f - tn : tn;
        const float aP = fmaf(kGlW1, Pp + Pn, kGlW0 * P0), aQ = fmaf(kGlW1, Qp + Qn, kGlW0 * Q0);
        const float qa = P.c.z * aQ;
        S = fmaf(-P.c.z, aQ, aP) - P.c.w * aQ;
        ok = S > 0.f && S * kAmp >= qa;
        terms = 2.f * (fabsf(mh) * P0 + p0);
    } else {
        const float pz = phidf(czh, czl), pm = phidf(cmh, cml);
        const float tz = ntail(czh, pz), tm = ntail(cmh, pm);
        const bool late = czh < 0.f;
        // late: both tails are lower tails (Phi); early: Q(cz) = tz, Q(czm) by its sign
        const float Qm = (cmh < 0.f) ? 1.f - tm : tm;
        const float iX = late ? fmaf(czh, tz, -cmh * tm) + (pz - pm) : fmaf(czh, tz, -cmh * Qm) + (pm - pz);
        const float x = fmaf(th, iX, tl * iX);
        S = late ? fmaf(P.c.x, x, -P.c.z) + fmaf(P.c.y, x, -P.c.w) : fmaf(-P.c.x, x, fmaf(-P.c.y, x, 1.f));
        ok = late ? S * kAmp >= P.c.z : S >= 1.f / kAmp;
        const float Pz = late ? tz : 1.f - tz, Pm = (cmh < 0.f) ? tm : 1.f - tm;
        terms = fabsf(czh) * Pz + fabsf(cmh) * Pm + pm + pz;
    }
    const float ref = 1.1e-16f * (1.f + __fdividef(terms, 2.f * h)) * (1.f + P.c.z);
    return ok && S * 1e-8f >= ref;
}

// A trial whose response clearly precedes its non-decision time (t = RT - t0
// below -1e-5 s): the reference form gives it the density floor, log 1e-10
// (t <= 0).  Times within 1e-5 s of t0 are left to the FP64 form, which
// decides the sign exactly.
__device__ __forceinline__ bool t_before(float2 rt, float2 t0)
{
    return (rt.x - t0.x) + (rt.y - t0.y) < -1e-5f;
}

// Log density of one trial in FP32 for K accumulators, the cell's entry ids
// winner first: d = g_w * (m 2^e); returns e and log m (the caller adds
// log g_w in FP64).  rt, t0: (hi, lo) splits.  false: use the FP64 form.
template <int K>
__device__ __forceinline__ bool lba_ld32(float2 rt, float2 t0, const int (&ent)[K], const Ent32 *E, int &e,
                                         float &lm)
{
    float th, te;
    two_diff(rt.x, t0.x, th, te);
    const float tl = te + (rt.y - t0.y);
    if (!(th > 1e-4f)) return false;
    const float uh = __frcp_rn(th);
    const float ul = uh * fmaf(-tl, uh, fmaf(-th, uh, 1.f));
    float P;
    if (!winner_br(E[ent[0]], uh, ul, P)) return false;
#pragma unroll
    for (int k = 1; k < K; ++k) {
        float S;
        if (!loser_s(E[ent[k]], th, tl, uh, ul, S)) return false;
        P *= S;
    }
    if (!(P >= 1.2e-38f) || !(P < 3.0e38f)) return false;
    lm = log_split(P, e);
    return true;
}

// The same for a run-time accumulator count (<= kMaxAcc): ents winner first.
__device__ __forceinline__ bool lba_ld32_n(float2 rt, float2 t0, const uint8_t *ents, int K, const Ent32 *E,
                                           int &e, float &lm)
{
    float th, te;
    two_diff(rt.x, t0.x, th, te);
    const float tl = te + (rt.y - t0.y);
    if (!(th > 1e-4f)) return false;
    const float uh = __frcp_rn(th);
    const float ul = uh * fmaf(-tl, uh, fmaf(-th, uh, 1.f));
    float P;
    if (!winner_br(E[ents[0]], uh, ul, P)) return false;
    for (int k = 1; k < K; ++k) {
        float S;
        if (!loser_s(E[ents[k]], th, tl, uh, ul, S)) return false;
        P *= S;
    }
    if (!(P >= 1.2e-38f) || !(P < 3.0e38f)) return false;
    lm = log_split(P, e);
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

// The diffusion entry of a responding boundary from its (a, v, z, d, sz, sv,
// t0, st0): the upper boundary mirrored to the lower (v -> -v, z -> 1 - z),
// the boundary's shift t0 -/+ d/2, in FP64 (e) and FP32 (f; f[7] the low
// part of the shift).
__device__ __forceinline__ void ddm_entry(const double *v8, bool upper, double *e, float *f)
{
    e[0] = v8[0];
    e[1] = upper ? -v8[1] : v8[1];
    e[2] = upper ? 1.0 - v8[2] : v8[2];
    e[3] = upper ? v8[6] - v8[3] / 2.0 : v8[6] + v8[3] / 2.0;
    e[4] = v8[4];
    e[5] = v8[5];
    e[6] = v8[7];
    e[7] = 0.0;
    for (int j = 0; j < 7; ++j) f[j] = (float)e[j];
    f[7] = (float)(e[3] - (double)f[3]);
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
