// diag_kernels.cu -- posterior diagnostics of stored samples on the device:
// summary (R/model-class.R:370-424) and gelman (R/model-class.R:1559-1690).
//
// The samples of L levels lie as smp [L][nmc][C][P] (R's posterior@theta
// [P, C, nmc] per level); iterations [start, start + n) are summarised.
//
//   k_diag_chain   per chain and parameter (a column of C*P): the mean, the
//                  variance and spectrum0_ar's spectral density at zero --
//                  the autocovariances of the demeaned chain up to lag
//                  kmax = min(n - 1, floor(10 log10 n)), the residual sd of
//                  the chain's linear trend, the Yule-Walker fits of orders
//                  0..kmax by the Durbin-Levinson recursion, the order of
//                  least AIC.  32 columns a CTA (one coalesced row segment),
//                  rows staged through shared memory, each warp owning every
//                  eighth lag.
//   k_diag_cov     per level and chain the P x P covariance of the chain's
//                  parameters (the reference's form of the PSRF needs all of
//                  W, the mean of these matrices).
//   k_diag_level   per level and parameter: the pooled mean, sd, Naive SE,
//                  Time-series SE and the PSRF with its upper confidence
//                  bound (fquantile.h's F quantile).
//   k_diag_quant   per level and parameter the quantiles of type 7 over all
//                  chains and iterations: the order statistics they need by
//                  an 8-pass radix select on the order-preserving 64-bit key
//                  of each double (one 256-bin histogram per wanted rank and
//                  pass, warp-aggregated shared-memory counts).
//
// Every sum runs in a fixed order, so results do not depend on scheduling.
#include <cmath>
#include <cstdint>

#include "fquantile.h"
#include "sampler.cuh"

namespace ggdmc {

namespace {

constexpr int kCols = 32;          // chain columns per CTA of k_diag_chain
constexpr int kDiagThreads = 256;  // 8 warps
constexpr int kTileRows = 64;
constexpr int kLagsPerWarp = kDiagMaxLag / 8 + 1;

__device__ __forceinline__ size_t row_off(int l, int nmc, int start, int i, int CP)
{
    return ((size_t)l * nmc + start + i) * CP;
}

__global__ void __launch_bounds__(kDiagThreads) k_diag_chain(const double *smp, int nmc, int C, int P, int start,
                                                             int n, int kmax, double *cstat)
{
    __shared__ double xs[kTileRows + kDiagMaxLag][kCols];
    __shared__ double red[8][kCols];
    double(*rr)[kCols] = xs;                      // the lag sums, once the tiles are done
    const int CP = C * P, l = blockIdx.y;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int q = blockIdx.x * kCols + lane;
    const bool valid = q < CP;
    // pass 1: the mean (warp w sums rows w, w + 8, ...)
    double s = 0.0;
    if (valid)
        for (int i = w; i < n; i += 8) s += smp[row_off(l, nmc, start, i, CP) + q];
    red[w][lane] = s;
    __syncthreads();
    double mean = 0.0;
    for (int k = 0; k < 8; ++k) mean += red[k][lane];
    mean /= n;
    __syncthreads();
    // pass 2: autocovariance sums sum_i x_i x_{i-k} of the demeaned chain,
    // and sum_i (i - (n-1)/2) x_i for the trend
    double acc[kLagsPerWarp];
#pragma unroll
    for (int m = 0; m < kLagsPerWarp; ++m) acc[m] = 0.0;
    double sxz = 0.0;
    const double zbar = 0.5 * (n - 1);
    for (int t0 = 0; t0 < n; t0 += kTileRows) {
        for (int j = w; j < kTileRows + kmax; j += 8) {
            const int i = t0 - kmax + j;
            xs[j][lane] = (valid && i >= 0 && i < n) ? smp[row_off(l, nmc, start, i, CP) + q] - mean : 0.0;
        }
        __syncthreads();
        const int rows = min(kTileRows, n - t0);
        for (int ii = 0; ii < rows; ++ii) {
            const double xi = xs[kmax + ii][lane];
            if ((ii & 7) == w) sxz += (t0 + ii - zbar) * xi;
#pragma unroll
            for (int m = 0; m < kLagsPerWarp; ++m) {
                const int k = w + 8 * m;
                if (k <= kmax) acc[m] += xi * xs[kmax + ii - k][lane];
            }
        }
        __syncthreads();
    }
    static_assert(kTileRows >= 1, "xs holds the kDiagMaxLag + 1 lag sums");
#pragma unroll
    for (int m = 0; m < kLagsPerWarp; ++m) {
        const int k = w + 8 * m;
        if (k <= kmax) rr[k][lane] = acc[m] / n;
    }
    red[w][lane] = sxz;
    __syncthreads();
    if (w != 0 || !valid) return;
    double z = 0.0;
    for (int k = 0; k < 8; ++k) z += red[k][lane];
    const double r0 = rr[0][lane];
    const double szz = (double)n * ((double)n * n - 1.0) / 12.0;
    const double rss = fmax(n * r0 - z * z / szz, 0.0);
    double spec;
    if (sqrt(rss / (n - 1)) <= 1.5e-8) {
        spec = 0.0;                               // all.equal(sd(residuals), 0)
    } else {
        double phi[kDiagMaxLag + 1], prev[kDiagMaxLag + 1];
        double v = r0, best_aic = n * log(r0), best_v = r0, best_sum = 0.0, sum = 0.0;
        int best = 0;
        for (int k = 1; k <= kmax; ++k) {
            double num = rr[k][lane];
            for (int j = 1; j < k; ++j) num -= prev[j] * rr[k - j][lane];
            const double a = num / v;
            for (int j = 1; j < k; ++j) phi[j] = prev[j] - a * prev[k - j];
            phi[k] = a;
            v *= 1.0 - a * a;
            sum = 0.0;
            for (int j = 1; j <= k; ++j) {
                prev[j] = phi[j];
                sum += phi[j];
            }
            const double aic = n * log(v) + 2.0 * k;
            if (aic < best_aic) {
                best_aic = aic;
                best = k;
                best_v = v;
                best_sum = sum;
            }
        }
        const double vp = best_v * n / (n - (best + 1.0));
        spec = vp / ((1.0 - best_sum) * (1.0 - best_sum));
    }
    double *o = cstat + ((size_t)l * CP + q) * 3;
    o[0] = mean;
    o[1] = n * r0 / (n - 1);
    o[2] = spec;
}

// covariance of chain c of level l (blockIdx.x = l * C + c) into wcov [L][C][P][P]
__global__ void __launch_bounds__(kDiagThreads) k_diag_cov(const double *smp, int nmc, int C, int P, int start,
                                                           int n, const double *cstat, double *wcov)
{
    constexpr int kRows = 32, kPer = (kDiagMaxPsrfPar * (kDiagMaxPsrfPar + 1) / 2 + kDiagThreads - 1) / kDiagThreads;
    __shared__ double xs[kRows][kDiagMaxPsrfPar];
    const int l = blockIdx.x / C, c = blockIdx.x % C, CP = C * P;
    const int ne = P * (P + 1) / 2;
    double acc[kPer];
    int ei[kPer], ej[kPer];
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
        acc[m] = 0.0;
        int e = threadIdx.x + m * kDiagThreads, i = 0;
        if (e < ne) {
            while (e >= P - i) {                  // entry e of the upper triangle, row by row
                e -= P - i;
                ++i;
            }
        }
        ei[m] = i;
        ej[m] = i + e;
    }
    for (int t0 = 0; t0 < n; t0 += kRows) {
        const int rows = min(kRows, n - t0);
        for (int u = threadIdx.x; u < rows * P; u += kDiagThreads) {
            const int r = u / P, p = u % P;
            xs[r][p] = smp[row_off(l, nmc, start, t0 + r, CP) + c * P + p] - cstat[((size_t)l * CP + c * P + p) * 3];
        }
        __syncthreads();
#pragma unroll
        for (int m = 0; m < kPer; ++m) {
            if (threadIdx.x + m * kDiagThreads >= ne) continue;
            double a = acc[m];
            for (int r = 0; r < rows; ++r) a += xs[r][ei[m]] * xs[r][ej[m]];
            acc[m] = a;
        }
        __syncthreads();
    }
    double *o = wcov + ((size_t)l * C + c) * P * P;
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
        if (threadIdx.x + m * kDiagThreads >= ne) continue;
        const double v = acc[m] / (n - 1);
        o[ei[m] * P + ej[m]] = v;
        o[ej[m] * P + ei[m]] = v;
    }
}

__global__ void k_diag_level(int C, int P, int n, const double *cstat, const double *wcov, double conf, int form,
                             double *mean, double *sd, double *nse, double *tse, double *psrf)
{
    const int l = blockIdx.x, CP = C * P;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        const double *cs = cstat + (size_t)l * CP * 3;
        double mu = 0.0, w = 0.0, sp = 0.0;
        for (int c = 0; c < C; ++c) {
            mu += cs[(c * P + p) * 3];
            w += cs[(c * P + p) * 3 + 1];
            sp += cs[(c * P + p) * 3 + 2];
        }
        mu /= C;
        w /= C;
        sp /= C;
        double bm = 0.0, vw = 0.0, m2bar = 0.0;
        for (int c = 0; c < C; ++c) {
            const double mc = cs[(c * P + p) * 3], vc = cs[(c * P + p) * 3 + 1];
            bm += (mc - mu) * (mc - mu);
            vw += (vc - w) * (vc - w);
            m2bar += mc * mc;
        }
        m2bar /= C;
        const size_t o = (size_t)l * P + p;
        // pooled over chains and iterations
        const double var = ((n - 1.0) * w * C + n * bm) / ((double)n * C - 1.0);
        if (mean) mean[o] = mu;
        if (sd) sd[o] = sqrt(var);
        if (nse) nse[o] = sqrt(var / n * C);           // the reference's formula
        if (tse) tse[o] = sqrt(sp / n * C);
        if (!psrf) continue;
        const double b = n * bm / (C - 1);             // n var(chain means)
        const double var_b = 2.0 * b * b / (C - 1);
        const double cf = 1.0 + 1.0 / C;
        double var_w, var_V;
        if (form == 0) {
            // reference: var of W's row p (W = mean of the chains' covariances) / C
            double rm = 0.0, rv = 0.0;
            for (int j = 0; j < P; ++j) {
                double wj = 0.0;
                for (int c = 0; c < C; ++c) wj += wcov[(((size_t)l * C + c) * P + p) * P + j];
                rm += wj / C;
            }
            rm /= P;
            for (int j = 0; j < P; ++j) {
                double wj = 0.0;
                for (int c = 0; c < C; ++c) wj += wcov[(((size_t)l * C + c) * P + p) * P + j];
                wj /= C;
                rv += (wj - rm) * (wj - rm);
            }
            var_w = (P > 1) ? rv / (P - 1) / C : NAN;
            var_V = ((n - 1.0) * (n - 1.0) * var_w + cf * cf * var_b) / ((double)n * n);
        } else {
            // coda (Brooks & Gelman 1998): var of the chains' variances and the W-B covariance
            double cov_s_m = 0.0, cov_s_m2 = 0.0;
            for (int c = 0; c < C; ++c) {
                const double mc = cs[(c * P + p) * 3], vc = cs[(c * P + p) * 3 + 1];
                cov_s_m += (vc - w) * (mc - mu);
                cov_s_m2 += (vc - w) * (mc * mc - m2bar);
            }
            var_w = vw / (C - 1) / C;
            const double cov_wb = ((double)n / C) * (cov_s_m2 / (C - 1) - 2.0 * mu * cov_s_m / (C - 1));
            var_V = ((n - 1.0) * (n - 1.0) * var_w + cf * cf * var_b + 2.0 * (n - 1.0) * cf * cov_wb) /
                    ((double)n * n);
        }
        const double V = (n - 1.0) / n * w + cf / n * b;
        const double df_V = 2.0 * V * V / var_V;
        const double df_adj = (df_V + 3.0) / (df_V + 1.0);
        const double r2_fixed = (n - 1.0) / n, r2_random = cf / n * (b / w);
        const double qf = f_quantile(0.5 * (1.0 + conf), C - 1.0, 2.0 * w * w / var_w);
        psrf[2 * o] = sqrt(df_adj * (r2_fixed + r2_random));
        psrf[2 * o + 1] = sqrt(df_adj * (r2_fixed + qf * r2_random));
    }
}

// order-preserving key of a double (NaN excluded): negative values reversed
__device__ __forceinline__ uint64_t dkey(double x)
{
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ double dval(uint64_t k)
{
    const uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// quantiles of type 7 of level l, parameter p (blockIdx.x = l * P + p) over
// the N = n C values; out [L][P][n_prob]
__global__ void __launch_bounds__(kDiagThreads) k_diag_quant(const double *smp, int nmc, int C, int P, int start,
                                                             int n, const double *probs, int n_prob, double *out)
{
    __shared__ unsigned hist[2 * kDiagMaxProb][256];
    __shared__ uint64_t prefix[2 * kDiagMaxProb];
    __shared__ long long rank[2 * kDiagMaxProb];
    const int l = blockIdx.x / P, p = blockIdx.x % P, CP = C * P;
    const long long N = (long long)n * C;
    const int nt = 2 * n_prob;
    if (threadIdx.x < nt) {
        const double h = (N - 1) * probs[threadIdx.x >> 1];
        const long long lo = (long long)floor(h);
        rank[threadIdx.x] = (threadIdx.x & 1) ? min(lo + 1, N - 1) : lo;
        prefix[threadIdx.x] = 0;
    }
    const double *base = smp + row_off(l, nmc, start, 0, CP) + p;
    const int lane = threadIdx.x & 31;
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = 56 - 8 * pass;
        for (int u = threadIdx.x; u < nt * 256; u += kDiagThreads) hist[u >> 8][u & 255] = 0;
        __syncthreads();
        // every lane of a warp runs the same trip count (the match needs all 32)
        for (long long e0 = (long long)(threadIdx.x - lane); e0 < N; e0 += kDiagThreads) {
            const long long e = e0 + lane;
            const bool in = e < N;
            const uint64_t key = in ? dkey(base[(size_t)e * P]) : 0;
            for (int t = 0; t < nt; ++t) {
                const bool hit = in && (pass == 0 || (key >> (shift + 8)) == (prefix[t] >> (shift + 8)));
                const int d = hit ? (int)((key >> shift) & 255) : -1;
                const unsigned grp = __match_any_sync(0xffffffffu, d);
                if (d >= 0 && lane == __ffs(grp) - 1) atomicAdd(&hist[t][d], (unsigned)__popc(grp));
            }
        }
        __syncthreads();
        if (threadIdx.x < nt) {
            const int t = threadIdx.x;
            long long r = rank[t], cum = 0;
            int d = 0;
            for (; d < 255; ++d) {
                if (cum + hist[t][d] > r) break;
                cum += hist[t][d];
            }
            rank[t] = r - cum;
            prefix[t] |= (uint64_t)d << shift;
        }
        __syncthreads();
    }
    if (threadIdx.x < n_prob) {
        const int i = threadIdx.x;
        const double h = (N - 1) * probs[i];
        const double g = h - floor(h);
        const double xlo = dval(prefix[2 * i]), xhi = dval(prefix[2 * i + 1]);
        // (1 - g) xlo + g xhi rounded term by term, as R and the host form it (no FMA)
        out[(size_t)blockIdx.x * n_prob + i] =
            (g == 0.0 || xhi == xlo) ? xlo : __dadd_rn(__dmul_rn(1.0 - g, xlo), __dmul_rn(g, xhi));
    }
}

}  // namespace

int diag_kmax(int n)
{
    const int k = (int)floor(10.0 * log10((double)n));
    return k < n - 1 ? k : n - 1;
}

cudaError_t launch_diagnostics(const double *smp, int L, int nmc, int C, int P, int start, int n, const double *probs,
                               int n_prob, double conf, int form, double *cstat, double *wcov, double *mean,
                               double *sd, double *nse, double *tse, double *quant, double *psrf, cudaStream_t st)
{
    if (L < 1) return cudaSuccess;
    const int kmax = diag_kmax(n);
    dim3 g1((unsigned)((C * P + kCols - 1) / kCols), (unsigned)L);
    k_diag_chain<<<g1, kDiagThreads, 0, st>>>(smp, nmc, C, P, start, n, kmax, cstat);
    if (psrf && form == 0) k_diag_cov<<<(unsigned)(L * C), kDiagThreads, 0, st>>>(smp, nmc, C, P, start, n, cstat, wcov);
    k_diag_level<<<(unsigned)L, 64, 0, st>>>(C, P, n, cstat, wcov, conf, form, mean, sd, nse, tse, psrf);
    if (quant && n_prob > 0)
        k_diag_quant<<<(unsigned)(L * P), kDiagThreads, 0, st>>>(smp, nmc, C, P, start, n, probs, n_prob, quant);
    return cudaGetLastError();
}

}  // namespace ggdmc
