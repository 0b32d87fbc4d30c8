/*
 * ggdmc_dmi.h -- conversions from ggdmc's R objects, read as flat arrays, to
 * the structs of ggdmc_gpu.h.
 *
 * In the reference these conversions happen inside Rcpp when a .Call entry
 * point starts (src/de2R.cpp:8-23, 30-47, 123-171): new_likelihood(dmi)
 * reads a data-model instance, prior::new_prior(priors@p_prior) the prior
 * list, new_DEInput / new_ThetaInput the sampler settings.  Here a .Call
 * shim (ggdmc_gb300/rshim/ggdmc_gpu_shim.c) reads the S4 slots with the R C
 * API -- R's logical, integer and double vectors are already flat and
 * column-major -- and passes them to these functions, which need neither R
 * nor a GPU.  All pointers are host pointers owned by the caller; strings
 * are NUL-terminated (CHAR(STRING_ELT(x, i)) in R's API).
 */
#ifndef GGDMC_DMI_H
#define GGDMC_DMI_H

#include "ggdmc_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Parameter kinds per accumulator of a model type (GGDMC_LBA_NKIND,
 * GGDMC_DDM_NKIND), or -1 for an unknown type. */
int32_t ggdmc_dmi_n_kind(int32_t model_type);

/* model@model_boolean -> ggdmc_model.param_src.  Replaces the design part of
 * new_likelihood(dmi) (src/de2R.cpp:13,129; the model object of
 * ggdmcModel::BuildModel).
 *   model_boolean  R logical array [n_cell, n_pxc, n_acc], column-major
 *                  (LOGICAL(slot)): TRUE where parameter-by-condition name j
 *                  applies to accumulator k in cell c
 *   pxc_names      model@parameter_x_condition_names [n_pxc]; the kind of a
 *                  name is its part before the first '.' (A, B, mean_v, sd_v,
 *                  t0, st0 for the LBA; a, v, z, d, sz, sv, t0, st0 for the
 *                  diffusion model)
 *   pnames         model@pnames [n_par] (theta order)
 *   const_names    names(model@constants) [n_const]
 *   param_src      out [n_cell][n_acc][n_kind]: the theta index, or -1 - j for
 *                  constant j
 * GGDMC_ERR_ARG for an unknown kind, a name that is neither free nor
 * constant, or a (cell, accumulator, kind) that no name covers. */
ggdmc_status ggdmc_dmi_param_src(int32_t model_type, const int32_t *model_boolean,
                                 int32_t n_cell, int32_t n_pxc, int32_t n_acc,
                                 const char *const *pxc_names,
                                 const char *const *pnames, int32_t n_par,
                                 const char *const *const_names, int32_t n_const,
                                 int32_t *param_src);

/* The responding accumulator of each cell (ggdmc_model.resp): the
 * accumulator named by the cell name's last '.'-separated field
 * ("left.blue.high.r1" -> "r1").  Cell names end in the response in every
 * ggdmcModel::BuildModel design; dmi@node_1_index is not in accumulator order
 * in the reference's own fixtures, so the name is the rule. */
ggdmc_status ggdmc_dmi_responders(const char *const *cell_names, int32_t n_cell,
                                  const char *const *accumulators, int32_t n_acc,
                                  int32_t *resp);

/* One subject's dmi@data -- a named list of RT vectors, one per non-empty
 * cell, in list order -- as trials with their cell index (the trial part of
 * new_likelihood(dmi)).  data_names[i] must be one of cell_names.  With rt
 * and cell both NULL only *n_trial is set (a size query); otherwise the
 * trials go to rt[0..n) / cell[0..n), capacity >= n. */
ggdmc_status ggdmc_dmi_trials(const char *const *cell_names, int32_t n_cell,
                              const char *const *data_names, const double *const *data_rt,
                              const int32_t *data_len, int32_t n_data, double *rt,
                              int32_t *cell, int64_t capacity, int64_t *n_trial);

/* One element of a ggdmcPrior p_prior / h_prior list -- a named numeric list
 * with p0, p1, lower, upper, dist_id, log_p -- as a ggdmc_prior table row
 * (replaces prior::new_prior, src/de2R.cpp:11-12,34-35,127-128).  A missing
 * or NA lower / upper bound is -Inf / +Inf; a missing log_p is 1 (TRUE);
 * p0, p1 and dist_id are required. */
ggdmc_status ggdmc_prior_row(const char *const *field_names, const double *field_values,
                             int32_t n_field, double *row /* [6] */);

/* in [n_row, n_col] column-major (an R matrix) -> out [n_row][n_col]
 * row-major: hyper_dmi@data, the subject-by-parameter matrix of run_hyper
 * (src/de2R.cpp:30-47), as ggdmc_run_hyper takes it. */
ggdmc_status ggdmc_transpose(const double *in, int32_t n_row, int32_t n_col, double *out);

#ifdef __cplusplus
}
#endif
#endif /* GGDMC_DMI_H */
