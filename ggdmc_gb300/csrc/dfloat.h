// dfloat.h -- double-float arithmetic (a value as an unevaluated sum hi + lo
// of two FP32 numbers, about 48 significant bits) for the per-proposal
// constants of the FP32 trial density.
//
// On this GPU FP64 instructions issue at 1/64 of the FP32 rate, and the FP64
// special functions (erfc, log) cost hundreds of FP64 instructions each; the
// constants of every proposal and accumulator tuple (Phi(v/s), its log, a few
// quotients) built that way took the proposal kernel from 43 to 113 us per
// sweep of the 256-subject workload.  The same constants in double-float
// FP32 need about 500 FP32 instructions and are accurate to about 1e-10
// relative, far below the 1e-8 the trial sums need.
//
// The building blocks are the error-free transformations of Dekker (1971)
// and Knuth (TwoSum) with the fused multiply-add for the exact product
// error; exp by Cody-Waite reduction and a Taylor series, log by the series
// 2 atanh((m-1)/(m+1)), and the normal tail from a rational Mills ratio
// fitted by fit_mills_df.py.  Header-only and host/device, so the CPU tests
// run the same arithmetic.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define GG_HD __host__ __device__ __forceinline__
#else
#define GG_HD inline
#endif

namespace ggdmc {

struct dfl {
    float h, l;
};

GG_HD dfl df_make(float h, float l = 0.f) { return dfl{h, l}; }

// exact split of a double into hi + lo (to the FP32 resolution of lo).
// (An integer form of the split, without FP64 instructions, gave the same
// bits but made the sweep 0.6% slower: four FP64 operations per parameter
// cost less than its 64-bit integer sequence.)
GG_HD dfl df_from_double(double x)
{
    const float h = (float)x;
    return dfl{h, (float)(x - (double)h)};
}

GG_HD double df_to_double(dfl a) { return (double)a.h + (double)a.l; }

// s + e = a + b exactly (Knuth)
GG_HD dfl df_two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return dfl{s, (a - (s - bb)) + (b - bb)};
}

// s + e = a + b exactly, |a| >= |b| (Dekker)
GG_HD dfl df_fast_two_sum(float a, float b)
{
    const float s = a + b;
    return dfl{s, b - (s - a)};
}

GG_HD dfl df_add(dfl a, dfl b)
{
    dfl s = df_two_sum(a.h, b.h);
    const dfl t = df_two_sum(a.l, b.l);
    s.l += t.h;
    s = df_fast_two_sum(s.h, s.l);
    s.l += t.l;
    return df_fast_two_sum(s.h, s.l);
}

GG_HD dfl df_add_f(dfl a, float b)
{
    dfl s = df_two_sum(a.h, b);
    s.l += a.l;
    return df_fast_two_sum(s.h, s.l);
}

GG_HD dfl df_neg(dfl a) { return dfl{-a.h, -a.l}; }

GG_HD dfl df_mul(dfl a, dfl b)
{
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return df_fast_two_sum(p, e);
}

GG_HD dfl df_mul_f(dfl a, float b)
{
    const float p = a.h * b;
    const float e = fmaf(a.l, b, fmaf(a.h, b, -p));
    return df_fast_two_sum(p, e);
}

// 1 / x in FP32, correctly rounded (the quotients below only need it to a
// few ulps: each is corrected with an exact remainder)
GG_HD float df_rcp(float x)
{
#ifdef __CUDA_ARCH__
    return __frcp_rn(x);
#else
    return 1.f / x;
#endif
}

// a / b: three FP32 quotients from one reciprocal of b.h, each correcting
// the exact remainder of the ones before (a - b q1, then a - b (q1 + q2))
GG_HD dfl df_div(dfl a, dfl b)
{
    const float rb = df_rcp(b.h);
    const float q1 = a.h * rb;
    const dfl r = df_add(a, df_neg(df_mul_f(b, q1)));     // a - b q1
    const float q2 = r.h * rb;
    const dfl r2 = df_add(r, df_neg(df_mul_f(b, q2)));
    const float q3 = r2.h * rb;
    dfl q = df_fast_two_sum(q1, q2);
    return df_add_f(q, q3);
}

GG_HD dfl df_scale(dfl a, int k) { return dfl{ldexpf(a.h, k), ldexpf(a.l, k)}; }

// ln 2 and 1/sqrt(2 pi) as hi + lo
constexpr float kDfLn2H = 0.6931471824645996f, kDfLn2L = -1.9046542121259336e-09f;
constexpr float kDfRs2piH = 0.3989422917366028f, kDfRs2piL = -1.1335170135851058e-08f;

// exp(x), x <= 0 (results below ~1e-38 lose precision as FP32 denormals)
GG_HD dfl df_exp(dfl x)
{
    const float k = rintf(x.h * 1.44269504088896341f);
    // r = x - k ln2, |r| <= 0.35
    dfl r = df_add(x, df_neg(df_mul_f(dfl{kDfLn2H, kDfLn2L}, k)));
    // Taylor series of exp(r) to r^10 (remainder below 3e-13 relative)
    constexpr float c[11][2] = {{1.0f, 0.0f},
                                {1.0f, 0.0f},
                                {0.5f, 0.0f},
                                {0.1666666716337204f, -4.967053879312289e-09f},
                                {0.0416666679084301f, -1.2417634698280722e-09f},
                                {0.008333333767950535f, -4.34617203337595e-10f},
                                {0.0013888889225199819f, -3.3631094437103215e-11f},
                                {0.00019841270113829523f, -2.725596874933456e-12f},
                                {2.4801587642286904e-05f, -3.40699609366682e-13f},
                                {2.7557318844628753e-06f, 3.793571224297229e-14f},
                                {2.755731998149713e-07f, -7.575112209051195e-15f}};
    dfl p = dfl{c[10][0], c[10][1]};
#pragma unroll
    for (int i = 9; i >= 0; --i) p = df_add(df_mul(p, r), dfl{c[i][0], c[i][1]});
    return df_scale(p, (int)k);
}

// log(x), x > 0 and x.h a normal FP32 number
GG_HD dfl df_log(dfl x)
{
    uint32_t bits;
    std::memcpy(&bits, &x.h, 4);
    int e = (int)(bits >> 23) - 127;
    dfl m = df_scale(x, -e);                        // m.h in [1, 2)
    if (m.h > 1.41421356f) {
        m = df_scale(m, -1);
        ++e;
    }
    // s = (m - 1) / (m + 1), |s| <= 0.172; log m = 2 (s + s^3/3 + ... + s^11/11)
    const dfl s = df_div(df_add_f(m, -1.f), df_add_f(m, 1.f));
    const dfl s2 = df_mul(s, s);
    constexpr float c[6][2] = {{1.0f, 0.0f},
                               {0.3333333432674408f, -9.934107758624577e-09f},
                               {0.20000000298023224f, -2.9802322831784522e-09f},
                               {0.1428571492433548f, -6.38621200366174e-09f},
                               {0.1111111119389534f, -8.278422947149977e-10f},
                               {0.09090909361839294f, -2.709302115988521e-09f}};
    dfl p = dfl{c[5][0], c[5][1]};
#pragma unroll
    for (int i = 4; i >= 0; --i) p = df_add(df_mul(p, s2), dfl{c[i][0], c[i][1]});
    const dfl lm = df_mul_f(df_mul(p, s), 2.f);
    return df_add(df_mul_f(dfl{kDfLn2H, kDfLn2L}, (float)e), lm);
}

// Q(x) = phi(x) M(x), the upper normal tail at x >= 0, to ~2e-10 relative
// (for x > 14 the value is below 1e-42; it is returned approximately)
GG_HD dfl df_qtail(dfl x)
{
    // P8(t) / Q9(t), t = x / 14, as hi + lo pairs (fit_mills_df.py)
    constexpr float P[9][2] = {{1.2533141374588013f, 2.0971446801354432e-11f},
                               {12.299561500549316f, -1.8281421887422766e-07f},
                               {60.469947814941406f, 1.5834275473025627e-06f},
                               {142.44403076171875f, 1.7743705029715784e-06f},
                               {107.82442474365234f, -2.6871466616285034e-06f},
                               {-123.47360229492188f, 3.123592250631191e-06f},
                               {54.08159255981445f, 1.1189361259766883e-07f},
                               {-13.577574729919434f, -2.5557147864674334e-07f},
                               {1.6431769132614136f, 3.543528803717777e-09f}};
    constexpr float Q[10][2] = {{1.0f, 0.0f},
                                {20.9840145111084f, -4.120550443076354e-07f},
                                {184.64749145507812f, 5.019035597797483e-06f},
                                {849.6051635742188f, 1.4880830349284224e-05f},
                                {1992.9686279296875f, 5.9207883168710396e-05f},
                                {1504.1337890625f, -3.2472114980919287e-05f},
                                {-1721.3927001953125f, 1.1936158443859313e-05f},
                                {752.3377075195312f, 2.9810591513523832e-05f},
                                {-188.3076629638672f, 8.041967021199525e-07f},
                                {22.7136287689209f, 6.636840055307403e-08f}};
    const dfl xc = (x.h > 14.f) ? dfl{14.f, 0.f} : x;
    const dfl t = df_mul(xc, dfl{0.0714285746216774f, -3.19310600183087e-09f});   // x / 14
    // the two Horner chains are independent; unrolled, the tables become immediates
    dfl p = dfl{P[8][0], P[8][1]}, q = dfl{Q[9][0], Q[9][1]};
#pragma unroll
    for (int i = 8; i >= 0; --i) {
        if (i < 8) p = df_add(df_mul(p, t), dfl{P[i][0], P[i][1]});
        q = df_add(df_mul(q, t), dfl{Q[i][0], Q[i][1]});
    }
    const dfl mills = df_div(p, q);
    // phi(x) = exp(-x^2 / 2) / sqrt(2 pi), x^2 exactly as hi + lo
    const dfl x2 = df_mul(x, x);
    const dfl ph = df_mul(df_exp(df_mul_f(x2, -0.5f)), dfl{kDfRs2piH, kDfRs2piL});
    return df_mul(ph, mills);
}

// Phi(k) and Phi(-k), each with full relative accuracy
GG_HD void df_phi_pair(dfl k, dfl &pk, dfl &pnk)
{
    const bool neg = k.h < 0.f;
    const dfl tail = df_qtail(neg ? df_neg(k) : k);              // Q(|k|)
    const dfl rest = df_add_f(df_neg(tail), 1.f);                 // 1 - Q(|k|)
    pk = neg ? tail : rest;
    pnk = neg ? rest : tail;
}

}  // namespace ggdmc
