/*
 * ggdmc_gpu.h -- C ABI of the GB300 DE-MCMC sampler (ggdmc's sampling hot path).
 *
 * The reference crosses from R into C++ through three .Call entry points
 * registered in src/RcppExports.cpp:54-59:
 *
 *   _ggdmc_run_subject(config, dmi,  samples)  -> src/de2R.cpp:8-23
 *   _ggdmc_run_hyper  (config, dmi,  samples)  -> src/de2R.cpp:30-47
 *   _ggdmc_run        (config, dmis, samples)  -> src/de2R.cpp:123-171
 *
 * Each unpacks S4 slots into ggdmcHeaders objects, runs de_class
 * (run_chains / run_hchains, src/de.cpp) and wraps theta_class storage into S4
 * `posterior` objects (src/type_casting.h:10-25).  This header is the same
 * boundary with plain C types: a .Call shim (or ctypes / cffi) converts the S4
 * slots into the POD structs below, calls one function, and copies the sample
 * arrays back into `posterior` slots.  The array layouts equal R's
 * column-major ones, so that copy is a memcpy.
 *
 * All pointers are HOST pointers owned by the caller.  Functions return a
 * ggdmc_status (0 = success) and never abort; ggdmc_last_error() gives the
 * message of the calling thread's last failure.
 */
#ifndef GGDMC_GPU_H
#define GGDMC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef enum {
    GGDMC_OK = 0,
    GGDMC_ERR_ARG = 1,      /* invalid argument or unsupported model       */
    GGDMC_ERR_CUDA = 2,     /* a CUDA runtime call failed                   */
    GGDMC_ERR_TIMEOUT = 3,  /* the device did not finish within the limit   */
    GGDMC_ERR_NUMERIC = 4,  /* a device-side check flagged bad numerics     */
    GGDMC_ERR_NOMEM = 5     /* device or host allocation failed             */
} ggdmc_status;

/* ------------------------------------------------------- enumerations */
enum { GGDMC_MODEL_LBA = 0, GGDMC_MODEL_DDM = 1 };

/* Arithmetic of the likelihood kernels.
 *  FP64        -- every step in double; the parity path.
 *  MIXED       -- per-trial densities in FP32 with FP64 re-evaluation of the
 *                 trials whose FP32 form is ill-conditioned; per-chain sums,
 *                 priors and the Metropolis difference in FP64.
 *  FP64_PLAIN  -- double throughout, one launch per subject per pass: the
 *                 plain GPU form the batched kernels are measured against. */
enum { GGDMC_FP64 = 0, GGDMC_MIXED = 1, GGDMC_FP64_PLAIN = 2, GGDMC_MIXED_SUMS = 3 };

/* ggdmc_de_config.flags: flush L2 between iterations and report in
 * ggdmc_run_stats.sweep_ms only the iterations' own kernel time (benchmarks). */
#define GGDMC_FLAG_L2_FLUSH 1

/* Prior families, ggdmcPrior's dist_id codes (fixture lba_data*.rda). */
enum { GGDMC_PRIOR_TNORM = 1, GGDMC_PRIOR_UNIF = 6 };

/* Number of parameter kinds per accumulator (LBA: A, B, mean_v, sd_v, t0,
 * st0) and per response (DDM: a, v, z, d, sz, sv, t0, st0). */
#define GGDMC_LBA_NKIND 6
#define GGDMC_DDM_NKIND 8

/* ------------------------------------------------------------- structs */

/* A design, flattened from ggdmcModel's `model` + a DMI's node_1_index.
 * param_src[(c*n_acc + k)*n_kind + q] >= 0 indexes theta; < 0 is -1-j into
 * constants.  resp[c] is the responding accumulator (node 1) of cell c. */
typedef struct {
    int32_t model_type;        /* GGDMC_MODEL_LBA / GGDMC_MODEL_DDM */
    int32_t n_par;             /* free parameters per subject       */
    int32_t n_cell;
    int32_t n_acc;             /* LBA accumulators; DDM: 2 boundaries */
    int32_t n_kind;            /* GGDMC_LBA_NKIND / GGDMC_DDM_NKIND   */
    int32_t n_const;
    const int32_t *param_src;  /* [n_cell][n_acc][n_kind] */
    const int32_t *resp;       /* [n_cell]                */
    const double *constants;   /* [n_const]               */
} ggdmc_model;

/* Trials of n_subject subjects packed back to back (dmi@data, cell-grouped). */
typedef struct {
    int32_t n_subject;
    const int64_t *offsets;    /* [n_subject + 1]          */
    const double *rt;          /* [offsets[n_subject]] (s) */
    const int32_t *cell;       /* [offsets[n_subject]]     */
} ggdmc_data;

/* One ggdmcPrior p_prior / h_prior list: per parameter
 * (p0, p1, lower, upper, dist_id, log_p). */
typedef struct {
    int32_t n_par;
    const double *table;       /* [n_par][6] */
} ggdmc_prior;

/* de_input + theta_input (R/model-class.R:1288-1313, 36-57). */
typedef struct {
    double pop_migration_prob;
    double sub_migration_prob;
    double gamma_precursor;    /* 2.38 */
    double rp;                 /* 0.001 */
    int32_t is_hblocked;
    int32_t is_pblocked;
    int32_t nparameter;        /* de_input@nparameter: gamma = g0/sqrt(2*nparameter) */
    int32_t nchain;
    int32_t nmc;               /* stored samples, slot 0 = start state */
    int32_t thin;              /* iterations between stored samples    */
    int32_t precision;         /* GGDMC_FP64 / GGDMC_MIXED / GGDMC_FP64_PLAIN */
    int32_t flags;             /* GGDMC_FLAG_* bits, 0 by default */
    uint64_t seed;             /* key of the counter-based draw stream */
} ggdmc_de_config;

/* Current chain state of one level (theta_class m_used_theta/lp/ll). */
typedef struct {
    double *theta;             /* [nchain][npar] == R [npar, nchain] */
    double *lp;                /* [nchain] */
    double *ll;                /* [nchain] */
} ggdmc_chain_state;

/* Thinned samples of one level: posterior@theta, @summed_log_prior,
 * @log_likelihoods (R/phi.R:77-87).  The buffers fill while the run goes
 * on (a CUDA-graph replay's slots while the next replay runs); every slot is
 * written when the call returns GGDMC_OK.  Any pointer may be NULL. */
typedef struct {
    double *theta;             /* [nmc][nchain][npar] == R [npar, nchain, nmc] */
    double *lp;                /* [nmc][nchain]       == R [nchain, nmc]       */
    double *ll;                /* [nmc][nchain]                                */
} ggdmc_samples;

/* Acceptance counters of one run (reported, not needed for results). */
typedef struct {
    int64_t proposals;
    int64_t accepts;
    int64_t migrations;        /* migration passes taken      */
    int64_t reevaluations;     /* speculative re-evaluations  */
    int64_t kernel_launches;   /* kernels launched by the run */
    int64_t trial_evals;       /* per-trial densities evaluated */
    int64_t iterations;        /* DE iterations (sweeps) run    */
    double sweep_ms;           /* device time of the sweeps (CUDA events), ms */
    int64_t resolve_rounds;    /* ordered-decision rounds over all subject passes */
    int64_t variants;          /* migration steps evaluated ahead of their decision */
    int64_t fallbacks;         /* MIXED: trial densities re-evaluated in FP64 */
    /* host wall-clock of the call's phases, ms */
    double setup_ms;           /* handle creation and uploads (one-shot calls), run buffers, start state */
    double capture_ms;         /* CUDA graph capture and instantiation (or reuse of the handle's graph) */
    double run_ms;             /* graph replays, with the sample copies that overlap them */
    double copyout_ms;         /* final state, remaining samples, counters; handle release (one-shot) */
} ggdmc_run_stats;

typedef struct ggdmc_handle ggdmc_handle;

/* ------------------------------------------------------ canonical draws
 * Every uniform the sampler consumes is keyed by (iteration, level, pass,
 * slot).  level 0 is the single level of run_subject / run_hyper or the phi
 * level of run; level 1+s is subject s of run.  pass is 0, or the blocked
 * parameter index.  With draws == NULL the uniforms come from Philox4x32-10
 * keyed by cfg->seed; otherwise draws[] holds them at
 *   ((((iter-1)*n_level + level)*n_pass + pass)*n_slot + slot)
 * for iter = 1 .. n_iter.  ggdmc_draw_layout() returns the four extents.
 *
 * Within one (iter, level, pass), with C = nchain and Pn = cfg->nparameter:
 *   slot 0                    migration-vs-crossover selector
 *   slot 1                    migration subset proportion
 *   slot 2 .. C+1             migration subset picks (partial Fisher-Yates)
 *   base(i) = 2 + C + i*(Pn+3), chain i of a crossover / step i of a
 *   migration: base+0, base+1 partner picks; base+2+j jitter of parameter j;
 *   base+2+Pn the Metropolis accept uniform. */
#define GGDMC_DRAW_SLOTS(nchain, nparameter) \
    (2 + (int64_t)(nchain) + (int64_t)(nchain) * ((int64_t)(nparameter) + 3))
ggdmc_status ggdmc_draw_layout(const ggdmc_de_config *cfg, int32_t n_level,
                               int32_t hierarchical,
                               int64_t *n_iter, int64_t *n_pass,
                               int64_t *n_slot, int64_t *total);

/* ---------------------------------------------------- entry points */

/* run_subject (src/de2R.cpp:8-23, .Call _ggdmc_run_subject): DE-MCMC of one
 * subject; `state` is the start (slot 0) and receives the final state. */
ggdmc_status ggdmc_run_subject(const ggdmc_de_config *cfg,
                               const ggdmc_model *model,
                               const ggdmc_data *data,       /* n_subject == 1 */
                               const ggdmc_prior *p_prior,
                               ggdmc_chain_state *state,
                               const double *draws,          /* NULL: Philox */
                               ggdmc_samples *out,
                               ggdmc_run_stats *stats);      /* nullable */

/* run_hyper (src/de2R.cpp:30-47, .Call _ggdmc_run_hyper): phi-only DE-MCMC
 * whose likelihood is the truncated-normal density of a fixed subject-by-
 * parameter matrix (hyper_dmi@data, row-major [n_row][p_prior->n_par]). */
ggdmc_status ggdmc_run_hyper(const ggdmc_de_config *cfg,
                             const double *hyper_data, int32_t n_row,
                             const ggdmc_prior *p_prior,
                             const ggdmc_prior *h_prior,
                             ggdmc_chain_state *state,
                             const double *draws,
                             ggdmc_samples *out,
                             ggdmc_run_stats *stats);

/* run (src/de2R.cpp:123-171, .Call _ggdmc_run): hierarchical DE-MCMC,
 * phi level + data->n_subject subjects.  subj_state[s] / subj_out[s] per
 * subject. */
ggdmc_status ggdmc_run(const ggdmc_de_config *cfg,
                       const ggdmc_model *model,
                       const ggdmc_data *data,
                       const ggdmc_prior *p_prior,
                       const ggdmc_prior *h_prior,
                       ggdmc_chain_state *phi_state,
                       ggdmc_chain_state *subj_state,
                       const double *draws,
                       ggdmc_samples *phi_out,
                       ggdmc_samples *subj_out,
                       ggdmc_run_stats *stats);

/* Many independent run_subject fits in one launch sequence (the reference
 * runs them as separate R processes, R/sampling.R:13-121).  Fit f uses the
 * data of subject f, p_prior, state[f], out[f]; level f keys its draws. */
ggdmc_status ggdmc_run_subjects(const ggdmc_de_config *cfg,
                                const ggdmc_model *model,
                                const ggdmc_data *data,
                                const ggdmc_prior *p_prior,
                                ggdmc_chain_state *state,
                                const double *draws,
                                ggdmc_samples *out,
                                ggdmc_run_stats *stats);

/* ------------------------------------------------- resident handle API
 * Upload a design and its trials once; run repeatedly (RestartSampling).  */
ggdmc_status ggdmc_create(const ggdmc_model *model, const ggdmc_data *data,
                          ggdmc_handle **out);
ggdmc_status ggdmc_destroy(ggdmc_handle *h);

/* Per-subject log-likelihood sums of n_theta parameter vectors per subject:
 * theta [n_subject][n_theta][n_par] -> out [n_subject][n_theta].
 * This is LPtr->sumloglike (called at src/de.cpp:145,187,604,653) batched.
 * precision GGDMC_MIXED adds an FP64 pass over the sums whose FP32 error
 * could exceed 1e-6 of their size (|sum| < 1.2 sqrt(N) + 0.03 N for N
 * trials: sums near zero), so that every sum is within 1e-6 relative of the
 * FP64 one; GGDMC_MIXED_SUMS returns the FP32 sums as the sampler forms
 * them, without that pass (likelihood calls only). */
ggdmc_status ggdmc_loglik(ggdmc_handle *h, const double *theta, int32_t n_theta,
                          int32_t precision, double *out);

/* The same with theta and out already in device memory (CUDA pointers) and
 * the launch on `stream` (a cudaStream_t; NULL = the default stream).  The
 * handle keeps device buffers for the call (the proposals' FP32 tables at
 * MIXED and MIXED_SUMS, the FP64 pass's work at MIXED), grown as needed. */
ggdmc_status ggdmc_loglik_device(ggdmc_handle *h, const double *d_theta,
                                 int32_t n_theta, int32_t precision,
                                 double *d_out, void *stream);

/* Per-trial log densities of one parameter vector per subject (the terms
 * sumloglike adds): theta [n_subject][n_par] -> out [total trials]. */
ggdmc_status ggdmc_trial_logdens(ggdmc_handle *h, const double *theta,
                                 int32_t precision, double *out);

/* sumlogprior (ggdmcPrior, called at src/de.cpp:144,186,603,652):
 * theta [n][n_par] -> out [n]. */
ggdmc_status ggdmc_logprior(const ggdmc_prior *prior, const double *theta,
                            int32_t n, double *out);

/* sumlogprior as ggdmc_logprior, without allocating: no counterpart in the
 * reference.  Stages the prior rows, theta and the output in a fixed 1 MiB
 * device array (one per device) instead of cudaMalloc; nothing in it needs to
 * start at zero.  Sizes whose staging (each piece rounded up to 256 bytes)
 * exceeds 1 MiB return GGDMC_ERR_ARG before any device work.  Calls that
 * overlap on one device (two host threads) share the array and race.  The
 * first call on a device looks up the array's address, which may load the
 * module: make it outside any stream capture. */
ggdmc_status ggdmc_logprior_noalloc(const ggdmc_prior *prior, const double *theta,
                                    int32_t n, double *out);

/* sumloghlike (src/de.cpp:245-270): phi [n][2P], subject thetas
 * [n_subject][n][P] (chain j of every subject pairs with phi j) -> out [n]. */
ggdmc_status ggdmc_loghlike(const ggdmc_prior *p_prior, const double *phi,
                            const double *subj_theta, int32_t n_subject,
                            int32_t n, double *out);

/* initialise_theta / initialise_phi (R/phi.R:141-332): start states by
 * rejection from the priors.  Chain c of every subject takes the first of
 * max_attempts draws from p_prior with a finite prior and likelihood; with
 * h_prior (2 x n_par rows), each phi chain c then the first draw from h_prior
 * with a finite prior and hyper log-likelihood against the subjects' chains
 * c.  Draws are keyed by (seed, iteration 0, level, attempt, chain, parameter)
 * -- R's rprior stream cannot be reproduced -- and mapped through the prior's
 * inverse distribution function.  subj_state [n_subject] / phi_state receive
 * theta, lp and ll; GGDMC_ERR_NUMERIC if a chain found no start. */
ggdmc_status ggdmc_initialise(ggdmc_handle *h, const ggdmc_prior *p_prior,
                              const ggdmc_prior *h_prior, int32_t nchain,
                              int32_t max_attempts, uint64_t seed, int32_t precision,
                              ggdmc_chain_state *subj_state,
                              ggdmc_chain_state *phi_state);

/* summary / gelman (R/model-class.R:370-424, 1559-1690) of the samples the
 * last ggdmc_handle_run left on the device, without copying them: for
 * iterations [start, nmc), per subject and parameter the posterior mean, sd
 * and the potential scale reduction factor's point estimate (Brooks &
 * Gelman's form as coda's gelman.diag computes it).  mean, sd, psrf:
 * [n_subject][n_par]; phi_*: [2 n_par] of the phi level, or NULL. */
ggdmc_status ggdmc_handle_summary(ggdmc_handle *h, int32_t start, double *mean,
                                  double *sd, double *psrf, double *phi_mean,
                                  double *phi_sd, double *phi_psrf);

/* The full summary and gelman diagnostics of the samples the last
 * ggdmc_handle_run left on the device, computed there.  Per level (subject
 * or phi) and parameter, over the iterations [start, end) of every chain
 * (end <= 0: nmc; R's start is 1-based and its end inclusive):
 *   mean, sd    summary's "Mean" and "SD" over all chains and iterations
 *   naive_se    "Naive SE" = sqrt(var / niter * nchain), the reference's
 *               formula (R/model-class.R:410)
 *   ts_se       "Time-series SE" = sqrt(mean over chains of safespec0 /
 *               niter * nchain): spectrum0_ar's AR spectral density at zero
 *               (R/model-class.R:257-281; Yule-Walker, order by AIC up to
 *               min(n - 1, floor(10 log10 n)))
 *   quantiles   [n_prob] per parameter, of type 7 (matrixStats::rowQuantiles)
 *   psrf        [2] per parameter: gelman's "Point est." and "Upper C.I."
 *               at level conf (R/model-class.R:1590-1616, 1677-1683)
 * Each pointer may be NULL (not computed).  probs (host) default in R to
 * 0.05, 0.5, 0.975; n_prob is 0 or 2..16 ("prob must be more than one
 * element").  psrf_form GGDMC_PSRF_REFERENCE is the reference's own form
 * (the variance of each row of W stands for the variance of the chains'
 * variances, no W-B covariance term; NaN for one parameter; needs n_par <= 64
 * at that level), GGDMC_PSRF_CODA Brooks & Gelman's as coda computes it.
 * GGDMC_ERR_ARG without stored samples, for fewer than 2 iterations, more
 * than 2.5e6 iterations, psrf with fewer than 3 chains ("Minimum three
 * chains needed"), or conf outside (0, 1). */
#define GGDMC_PSRF_REFERENCE 0
#define GGDMC_PSRF_CODA 1
typedef struct {
    double *mean;              /* [n_level][n_par]         */
    double *sd;                /* [n_level][n_par]         */
    double *naive_se;          /* [n_level][n_par]         */
    double *ts_se;             /* [n_level][n_par]         */
    double *quantiles;         /* [n_level][n_par][n_prob] */
    double *psrf;              /* [n_level][n_par][2]      */
} ggdmc_diag;

ggdmc_status ggdmc_handle_diagnostics(ggdmc_handle *h, int32_t start, int32_t end,
                                      const double *probs, int32_t n_prob, double conf,
                                      int32_t psrf_form, ggdmc_diag *subj, ggdmc_diag *phi);

/* ------------------------------------------------------------ tuning
 * Launch settings of a handle's runs.  None of them changes a result: the
 * chains of a run are the same bit for bit under every setting.  0 in a
 * field means "the built-in choice"; the environment variables
 * GGDMC_SPEC_GROUP, GGDMC_GRAPH_ITERS, GGDMC_MIG_ROUND and GGDMC_LIK_VARIANT
 * override a handle's settings. */
typedef struct {
    int32_t spec_group;        /* proposals per speculative likelihood CTA: 1, 2 or 4        */
    int32_t graph_iters;       /* DE iterations per captured CUDA graph, 1..64              */
    int32_t mig_round;         /* migration steps evaluated ahead per resolve round, 1..8   */
    int32_t lik_variant;       /* 4-accumulator LBA: 1 = the 4-accumulator likelihood kernel
                                  (8 CTAs per SM), 2 = the generic one (6 CTAs per SM)      */
    double sweep_ms;           /* device time per sweep measured for the choice (output)   */
} ggdmc_tuning;

/* The autotuner's cache key of a design and data shape: model type,
 * accumulators, free parameters, chains, whether a phi level runs, and the
 * histogram of the subjects' trial counts in powers of two (each bin's count
 * rounded to a power of two, so that similar data sets share a key).
 * Writes a NUL-terminated key of at most key_len bytes.  Host only. */
ggdmc_status ggdmc_tune_key(const ggdmc_model *model, const ggdmc_data *data, int32_t nchain,
                            int32_t hierarchical, char *key, int32_t key_len);

/* The cached settings of a key: from this process's cache, else from the
 * text file cache_path (NULL: none; one "key spec_group graph_iters mig_round
 * lik_variant sweep_ms" line per entry, the last line of a key wins).
 * GGDMC_ERR_ARG when the key is not cached.  Host only. */
ggdmc_status ggdmc_tune_lookup(const char *key, const char *cache_path, ggdmc_tuning *out);

/* Put settings in this process's cache and, with cache_path, append them to
 * the file.  Host only. */
ggdmc_status ggdmc_tune_store(const char *key, const char *cache_path, const ggdmc_tuning *t);

/* Settings for the runs of a handle (NULL: the built-in choices). */
ggdmc_status ggdmc_handle_set_tuning(ggdmc_handle *h, const ggdmc_tuning *t);

/* Autotune a handle for runs like cfg (its chains, level layout and
 * precision): look the key up (cache_path as ggdmc_tune_lookup) and, when it
 * is not cached, time candidate settings on n_probe DE iterations each from
 * the given start states (which are not changed) -- the likelihood kernel
 * variant, the speculative group size, the migration steps per round and the
 * iterations per graph, one setting at a time from the built-in choice, by
 * CUDA events on the device -- and store the fastest.  The handle then runs
 * with it; *out (nullable) receives it. */
ggdmc_status ggdmc_autotune(ggdmc_handle *h, const ggdmc_de_config *cfg, const ggdmc_prior *p_prior,
                            const ggdmc_prior *h_prior, const ggdmc_chain_state *phi_state,
                            const ggdmc_chain_state *subj_state, int32_t n_probe,
                            const char *cache_path, ggdmc_tuning *out);

/* Run on a resident handle: level layout as ggdmc_run (phi_state == NULL
 * runs the subjects as independent fits, like ggdmc_run_subjects). */
ggdmc_status ggdmc_handle_run(ggdmc_handle *h, const ggdmc_de_config *cfg,
                              const ggdmc_prior *p_prior,
                              const ggdmc_prior *h_prior,
                              ggdmc_chain_state *phi_state,
                              ggdmc_chain_state *subj_state,
                              const double *draws,
                              ggdmc_samples *phi_out,
                              ggdmc_samples *subj_out,
                              ggdmc_run_stats *stats);

/* Measured throughput of this GPU's FP32 FMA pipe (TFLOP/s, 2 flops per
 * FMA) and MUFU unit (tera-ops/s of ex2.approx): the roofline denominators of
 * the likelihood kernel.  No counterpart in the reference (a measurement
 * utility of this library). */
ggdmc_status ggdmc_probe_peaks(double *fp32_tflops, double *mufu_tops);

/* Message of this thread's last failed call ("" if none). */
const char *ggdmc_last_error(void);

/* Library version string. */
const char *ggdmc_version(void);

#ifdef __cplusplus
}
#endif
#endif /* GGDMC_GPU_H */
