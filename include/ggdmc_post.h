/*
 * ggdmc_post.h -- host-side operations on stored samples (ggdmc_samples of
 * include/ggdmc_gpu.h).
 *
 * RebuildPosterior, RebuildHyper and RebuildPosteriors
 * (R/parallel_helper.R:62-109, 162-208) combine fits run as separate R
 * processes (one per core, R/sampling.R) into one posterior whose chains are
 * the fits.  On this GPU the fits of one design run as the levels of one
 * ggdmc_run_subjects / ggdmc_run call; ggdmc_rebuild_posterior merges their
 * ggdmc_samples in the reference's layout.
 */
#ifndef GGDMC_POST_H
#define GGDMC_POST_H

#include "ggdmc_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* RebuildPosterior (R/parallel_helper.R:62-83, with .GetParamArray at :15-55
 * and .get_likelihood_matrix at :1-12).  fits[n_fit], each nmc x nchain x
 * npar samples of one level, become one posterior of nchain' = n_fit chains
 * and nmc' = nmc * nchain samples:
 *   out->theta [nmc'][n_fit][npar]: sample j = m * nchain + c of chain f is
 *              fits[f].theta[m][c] (R: theta [npar, nchain, nmc] of a fit
 *              re-dimensioned to [npar, nchain * nmc]);
 *   out->lp, out->ll [nmc'][n_fit]: sample j = c * nmc + m of chain f is
 *              fits[f].lp[m][c] (R: as.vector(t(summed_log_prior)), which
 *              runs over iterations first -- a different order from theta's,
 *              kept as the reference has it).
 * RebuildHyper is the same merge of the fits' phi samples; RebuildPosteriors
 * is this merge for each subject.  start and thin are those of the first fit
 * (the caller keeps them).  Any out pointer may be NULL, and so may the
 * matching input pointers then.  GGDMC_ERR_ARG for a non-positive extent or
 * a missing input whose output is requested. */
ggdmc_status ggdmc_rebuild_posterior(const ggdmc_samples *fits, int32_t n_fit, int32_t nmc,
                                     int32_t nchain, int32_t npar, ggdmc_samples *out);

#ifdef __cplusplus
}
#endif

#endif /* GGDMC_POST_H */
