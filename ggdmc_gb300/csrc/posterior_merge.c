/*
 * posterior_merge.c -- ggdmc_rebuild_posterior (include/ggdmc_post.h): the
 * RebuildPosterior merge of R/parallel_helper.R:62-83 on flat arrays.
 *
 * The reference builds the merged theta by giving each fit's
 * [npar, nchain, nmc] array the dimensions [npar, nchain * nmc] and storing
 * it as chain f of a [npar, n_fit, nchain * nmc] array (.GetParamArray,
 * :15-55); in C order a fit's samples [nmc][nchain][npar] are already
 * [nmc * nchain][npar], so merged sample j of chain f is the fit's row j.
 * The log-prior and log-likelihood matrices [nchain, nmc] are transposed
 * before they are flattened (.get_likelihood_matrix, :1-12), so their merged
 * sample j = c * nmc + m is the fit's (m, c) entry.
 */
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include "../../include/ggdmc_post.h"

#define EXPORT __attribute__((visibility("default")))

static void merge_scalar(const ggdmc_samples *fits, int n_fit, int nmc, int nchain, int ll, double *out)
{
    for (int f = 0; f < n_fit; ++f) {
        const double *src = ll ? fits[f].ll : fits[f].lp;
        for (int c = 0; c < nchain; ++c)
            for (int m = 0; m < nmc; ++m)
                out[((size_t)c * nmc + m) * n_fit + f] = src[(size_t)m * nchain + c];
    }
}

EXPORT ggdmc_status ggdmc_rebuild_posterior(const ggdmc_samples *fits, int32_t n_fit, int32_t nmc,
                                            int32_t nchain, int32_t npar, ggdmc_samples *out)
{
    if (!fits || !out || n_fit < 1 || nmc < 1 || nchain < 1 || npar < 1) return GGDMC_ERR_ARG;
    for (int f = 0; f < n_fit; ++f)
        if ((out->theta && !fits[f].theta) || (out->lp && !fits[f].lp) || (out->ll && !fits[f].ll))
            return GGDMC_ERR_ARG;
    const size_t rows = (size_t)nmc * nchain;
    if (out->theta)
        for (int f = 0; f < n_fit; ++f)
            for (size_t j = 0; j < rows; ++j)
                memcpy(out->theta + (j * n_fit + f) * npar, fits[f].theta + j * npar, sizeof(double) * npar);
    if (out->lp) merge_scalar(fits, n_fit, nmc, nchain, 0, out->lp);
    if (out->ll) merge_scalar(fits, n_fit, nmc, nchain, 1, out->ll);
    return GGDMC_OK;
}
