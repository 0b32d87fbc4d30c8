// sampler.cuh -- device-side run description shared by the kernels and the
// host runtime.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "model_tables.h"

namespace ggdmc {

enum PassType : int32_t { PASS_CROSS = 0, PASS_MIG = 1, PASS_SKIP = 2 };
enum Prec : int32_t { PREC_FP64 = 0, PREC_MIXED = 1 };
// Which de.cpp loop the levels follow.
enum LoopKind : int32_t {
    LOOP_CHAINS = 0,   // run_chains (src/de.cpp:201-242): one selector per iteration
    LOOP_HCHAINS = 1   // run_hchains (src/de.cpp:272-383): a selector per pass
};

// Prior row: (dist_id, p0, p1, lower, upper, c) with c the constant part of
// the log density (truncated normal: -log(sqrt(2 pi)) - log(p1) - log(mass);
// uniform: -log(p1 - p0)).
constexpr int kPriorRow = 6;

enum StatIdx { ST_PROPOSALS = 0, ST_ACCEPTS, ST_MIGRATIONS, ST_REEVALS, ST_TRIALS, ST_ROUNDS,
               ST_VARIANTS, ST_FALLBACKS, ST_N };

// Migration steps evaluated ahead per in-CTA round under the assumption that
// the steps before them accept (a migration cascade carries one value
// forward); the first round's cascade is evaluated with the speculative
// proposals.
constexpr int kVariants = 8;


// Partial log-likelihood sums of one proposal over a subject's trials
// (group_chunk): the fixed-point sum (units of 2^-32) of the trials' mantissa
// logs and FP64 terms, their binary exponents, the trials left to FP64, and
// the FP64 sum of a proposal outside the FP32 form's domain.  Integer sums
// are exact, so the total does not depend on how trials map to threads.
struct JobPart {
    long long s;
    int32_t e, nf;
    double f64;
};
constexpr float kFixScale = 4294967296.f;                  // 2^32
constexpr double kFixUnit = 1.0 / 4294967296.0;            // 2^-32

struct RunDev {
    // ------------------------------------------------------------ shape
    int32_t C;            // chains
    int32_t P;            // subject-level theta length
    int32_t Pphi;         // phi-level theta length (0: no phi level)
    int32_t S;            // subject levels
    int32_t Pn;           // de_input nparameter (gamma, loop bound, draw stride)
    int32_t half;         // Pn / 2
    int32_t loop;         // LoopKind of the subject levels
    int32_t level0;       // draw level of subject level 0
    int32_t prec;         // Prec
    int32_t sub_blocked;  // is_pblocked
    int32_t phi_blocked;  // is_hblocked (phi of run) / is_pblocked (run_hyper)
    int32_t phi_loop;     // LoopKind of the phi level
    int32_t thin, nmc;
    double gamma, rp, sub_mig, pop_mig;
    DrawSrc ds;
    int32_t *iter;        // current iteration (device counter)

    // ------------------------------------------------------------ data
    DevModel m;
    const int64_t *offs;     // [S+1]
    const double *rt64;      // [N]
    const float2 *rt32;      // [N] (hi, lo)
    const uint16_t *cell;    // [N]

    // ----------------------------------------------------- subject levels
    double *th, *lp, *ll;          // [S][C][P], [S][C]
    double *th_s, *lp_s, *ll_s;    // [S][CS][P], [S][CS]: proposals by step, then variants
    int32_t *partner;              // [S][C][2]
    int8_t *need;                  // [S][CS]
    int32_t *ptype;                // [S]
    int32_t *nstep;                // [S]
    int32_t *sub;                  // [S][C]
    int32_t *migrated;             // [S] (LOOP_CHAINS: migration taken this iteration)
    double *jit;                   // [S][C][P] jitter draws of the pass (re-proposals reuse them)
    double *accu;                  // [S][C]    Metropolis accept uniforms of the pass
    int32_t *rs_para;              // [S] blocked parameter of the pass, -1 for all
    const int32_t *sub_order;      // [S] subjects by trial count, largest first
    int32_t *res_order;            // [S] the subject pass's level order (k_level_order)
    int32_t *lvl_ns;               // [S] duration of each level's last crossover resolve (ns)
    int32_t CS;                    // proposal slots per level: C speculative + C variants
    // FP32 tables of every proposal slot, built where the proposal is built
    Ent32 *tab_e;                  // [S*CS][n_ent] FP32 trial constants (device_common.cuh)
    double *tab_lg;                // [S*CS][n_ent] log g of each tuple
    float2 *tab_t;                 // [S*CS][n_t0]  t0 as (hi, lo)
    int32_t *tab_bad;              // [S*CS] 1: outside the FP32 form's domain
    const int32_t *cell_cnt;       // [S][n_cell] trials of each subject in each cell
    const double *prior;           // [P][kPriorRow] fixed subject prior (nullptr in HB)
    const double *pp_bounds;       // [P][2] p_prior (lower, upper) for HB / phi level
    double *phi_tab;               // [C][P][3] (mu, 1/sigma, c) of phi chain (HB)

    // ---------------------------------------------------------- phi level
    double *pth, *plp, *pll;       // [C][Pphi], [C]
    double *pth_s, *plp_s, *pll_s; // proposals
    double *pref_src, *pref_next;  // refreshed hyper log-likelihoods by step
    int32_t *ppartner;             // [C][2]
    int8_t *pneed;                 // [C]
    int32_t *pptype, *pnstep, *psub, *pmigrated;
    double *pjit, *paccu;          // [C][Pphi], [C]
    const double *hprior;          // [Pphi][kPriorRow]
    const double *hrows;           // run_hyper data [n_row][Pphi/2] (nullptr in HB)
    int32_t n_row;

    // ---------------------------------------------------------- samples
    double *smp_th, *smp_lp, *smp_ll;     // [S][nmc][C][P], [S][nmc][C]
    double *psmp_th, *psmp_lp, *psmp_ll;  // [nmc][C][Pphi], [nmc][C]

    // k_sub_step / k_sub_spec_rest (subject pass fused with the next
    // iteration's proposals)
    int32_t *ready;                // [S] iteration whose proposals level l holds
    int32_t *spec_cnt;             // [S] spec items of the level claimed so far
    int32_t *ctl;                  // [3] levels claimed / resolved this pass, events
    int32_t iter_end;              // last iteration of the run
    int32_t spec_idle_limit;       // polls (~1 us each) an idle k_sub_step CTA waits before giving up

    // launch settings (ggdmc_tuning): migration variants evaluated per
    // resolve round (1..kVariants), and the likelihood kernel of 4-accumulator
    // LBA designs (0: the 4-accumulator instantiation at 8 CTAs per SM, 1: the
    // generic one at 6); neither changes a result
    int32_t mig_round;
    int32_t lik_variant;

    unsigned long long *stats;     // [ST_N]
    int32_t *status;
};

// --------------------------------------------------------------- launchers
// (defined in sampler_kernels.cu)
cudaError_t launch_sub_propose(const RunDev &r, int pass, bool defer_prior, bool fused, cudaStream_t st);
cudaError_t launch_sub_spec_rest(const RunDev &r, int group, cudaStream_t st);
cudaError_t launch_sub_step(const RunDev &r, bool score_priors, bool defer_next, int group, cudaStream_t st);
cudaError_t launch_sub_loglik(const RunDev &r, const int32_t *items, int n_items, int group,
                              cudaStream_t st);
cudaError_t launch_sub_resolve(const RunDev &r, int pass, int level_begin, int level_count,
                               bool score_priors, cudaStream_t st);
cudaError_t launch_phi_tables(const RunDev &r, cudaStream_t st);
cudaError_t launch_level_order(const RunDev &r, bool with_type, cudaStream_t st);
cudaError_t launch_phi_propose(const RunDev &r, int pass, cudaStream_t st);
cudaError_t launch_phi_eval(const RunDev &r, cudaStream_t st);
cudaError_t launch_phi_resolve(const RunDev &r, int pass, cudaStream_t st);
cudaError_t launch_store(const RunDev &r, cudaStream_t st);
cudaError_t launch_next_iter(const RunDev &r, cudaStream_t st);
// The FP32 tables of the batch's proposals ([S * n_theta] proposals), built
// by a whole-GPU kernel before the likelihood kernel reads them (MIXED LBA);
// nullptr pointers: each likelihood block builds its proposal's own.
struct BatchTables {
    Ent32 *e;        // [S * n_theta][n_ent]
    double *lg;      // [S * n_theta][n_ent]
    float2 *t;       // [S * n_theta][n_t0]
    int32_t *bad;    // [S * n_theta]
};
cudaError_t launch_loglik_batch(const RunDev &r, const double *theta, int n_theta, double *out,
                                cudaStream_t st, const BatchTables *tabs = nullptr);
cudaError_t launch_trial_logdens(const RunDev &r, const double *theta, double *out,
                                 cudaStream_t st);
// FP64 refinement of the MIXED sums out [S][n_theta] near zero (theta as given
// to launch_loglik_batch); buffers sized by refine_capacity.
size_t refine_capacity(const int64_t *h_offs, int S, int n_theta);
cudaError_t launch_refine(const RunDev &r, const double *theta, int n_theta, double *out, int32_t *count,
                          int32_t *base, int32_t *item, double *partial, int grid, cudaStream_t st);
cudaError_t launch_init_draw(const double *rows, int P, int C, int level0, int n_level, const int32_t *attempt,
                             const uint8_t *done, uint64_t seed, double *theta, cudaStream_t st);
cudaError_t launch_summary(const double *smp, int L, int nmc, int C, int P, int start, double *cs,
                           double *mean, double *sd, double *psrf, cudaStream_t st);
// Posterior diagnostics (diag_kernels.cu) of samples smp [L][nmc][C][P],
// iterations [start, start + n): cstat [L][C*P][3] and (form 0 with psrf)
// wcov [L][C][P][P] are scratch; mean, sd, nse, tse [L][P], quant
// [L][P][n_prob] (probs on the device), psrf [L][P][2]; any output may be
// NULL.  form 0: the reference's PSRF, 1: coda's.
constexpr int kDiagMaxLag = 64;       // kmax = min(n - 1, floor(10 log10 n)) <= 64: n < 2.5e6
constexpr int kDiagMaxPsrfPar = 64;   // P of the reference's PSRF form (the P x P covariances)
constexpr int kDiagMaxProb = 16;
int diag_kmax(int n);
cudaError_t launch_diagnostics(const double *smp, int L, int nmc, int C, int P, int start, int n, const double *probs,
                               int n_prob, double conf, int form, double *cstat, double *wcov, double *mean,
                               double *sd, double *nse, double *tse, double *quant, double *psrf, cudaStream_t st);
cudaError_t launch_split_rt(const double *rt, int64_t n, float2 *out, cudaStream_t st);
cudaError_t launch_logprior(const double *rows, int P, const double *theta, int n, double *out,
                            cudaStream_t st);
cudaError_t launch_loghlike(const RunDev &r, const double *phi, double *out, cudaStream_t st);
__host__ __device__ size_t sub_smem_bytes(const DevModel &m);
cudaError_t configure_kernels(const DevModel &m);

}  // namespace ggdmc
