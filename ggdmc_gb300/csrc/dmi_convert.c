/*
 * dmi_convert.c -- the S4-to-POD conversions of the .Call boundary, in plain C
 * on flat arrays (declared in include/ggdmc_dmi.h).
 *
 * The reference turns its S4 objects into C++ objects inside Rcpp: a data-model
 * instance through new_likelihood(dmi) (src/de2R.cpp:13,129), the priors
 * through prior::new_prior(priors@p_prior) (src/de2R.cpp:11-12,34-35,127-128)
 * and the sampler settings through new_DEInput / new_ThetaInput
 * (src/de2R.cpp:15-16).  A .Call shim reads the S4 slots into C arrays (R's
 * logical, integer and double vectors are already flat, column-major) and
 * these functions build the structs of include/ggdmc_gpu.h from them.  They
 * need neither R nor a GPU, so they are tested on the CPU against
 * ggdmc_gb300/dmi.py.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include "../../include/ggdmc_dmi.h"

#define EXPORT __attribute__((visibility("default")))

static const char *const kLbaKinds[GGDMC_LBA_NKIND] = {"A", "B", "mean_v", "sd_v", "t0", "st0"};
static const char *const kDdmKinds[GGDMC_DDM_NKIND] = {"a", "v", "z", "d", "sz", "sv", "t0", "st0"};

/* Index of the parameter kind that prefixes `name` (the part before the
 * first '.'), or -1. */
static int kind_of(const char *name, const char *const *kinds, int n_kind)
{
    const char *dot = strchr(name, '.');
    const size_t len = dot ? (size_t)(dot - name) : strlen(name);
    for (int q = 0; q < n_kind; ++q)
        if (strlen(kinds[q]) == len && strncmp(kinds[q], name, len) == 0) return q;
    return -1;
}

static int find_name(const char *name, const char *const *names, int n)
{
    for (int i = 0; i < n; ++i)
        if (names[i] && strcmp(names[i], name) == 0) return i;
    return -1;
}

EXPORT int32_t ggdmc_dmi_n_kind(int32_t model_type)
{
    return model_type == GGDMC_MODEL_DDM ? GGDMC_DDM_NKIND
           : model_type == GGDMC_MODEL_LBA ? GGDMC_LBA_NKIND : -1;
}

EXPORT ggdmc_status ggdmc_dmi_param_src(int32_t model_type, const int32_t *model_boolean,
                                        int32_t n_cell, int32_t n_pxc, int32_t n_acc,
                                        const char *const *pxc_names,
                                        const char *const *pnames, int32_t n_par,
                                        const char *const *const_names, int32_t n_const,
                                        int32_t *param_src)
{
    const int n_kind = ggdmc_dmi_n_kind(model_type);
    if (n_kind < 0 || !model_boolean || !pxc_names || !param_src || n_cell < 1 || n_pxc < 1 ||
        n_acc < 1 || n_par < 0 || n_const < 0 || (n_par > 0 && !pnames) ||
        (n_const > 0 && !const_names))
        return GGDMC_ERR_ARG;
    const char *const *kinds = model_type == GGDMC_MODEL_DDM ? kDdmKinds : kLbaKinds;
    const size_t n_out = (size_t)n_cell * n_acc * n_kind;
    for (size_t i = 0; i < n_out; ++i) param_src[i] = INT32_MIN;
    for (int j = 0; j < n_pxc; ++j) {
        if (!pxc_names[j]) return GGDMC_ERR_ARG;
        const int q = kind_of(pxc_names[j], kinds, n_kind);
        if (q < 0) return GGDMC_ERR_ARG;                 /* unknown parameter kind */
        int code = find_name(pxc_names[j], pnames, n_par);
        if (code < 0) {
            const int k = find_name(pxc_names[j], const_names, n_const);
            if (k < 0) return GGDMC_ERR_ARG;              /* neither free nor constant */
            code = -1 - k;
        }
        for (int k = 0; k < n_acc; ++k)
            for (int c = 0; c < n_cell; ++c) {
                /* R logical array [ncell, npxc, K], column-major */
                const int32_t on = model_boolean[c + (size_t)n_cell * (j + (size_t)n_pxc * k)];
                if (on == 1) param_src[((size_t)c * n_acc + k) * n_kind + q] = code;
            }
    }
    for (size_t i = 0; i < n_out; ++i)
        if (param_src[i] == INT32_MIN) return GGDMC_ERR_ARG;   /* a (cell, acc, kind) unset */
    return GGDMC_OK;
}

EXPORT ggdmc_status ggdmc_dmi_responders(const char *const *cell_names, int32_t n_cell,
                                         const char *const *accumulators, int32_t n_acc,
                                         int32_t *resp)
{
    if (!cell_names || !accumulators || !resp || n_cell < 1 || n_acc < 1) return GGDMC_ERR_ARG;
    for (int c = 0; c < n_cell; ++c) {
        if (!cell_names[c]) return GGDMC_ERR_ARG;
        const char *dot = strrchr(cell_names[c], '.');
        const char *suffix = dot ? dot + 1 : cell_names[c];
        const int k = find_name(suffix, accumulators, n_acc);
        if (k < 0) return GGDMC_ERR_ARG;
        resp[c] = k;
    }
    return GGDMC_OK;
}

EXPORT ggdmc_status ggdmc_dmi_trials(const char *const *cell_names, int32_t n_cell,
                                     const char *const *data_names, const double *const *data_rt,
                                     const int32_t *data_len, int32_t n_data, double *rt,
                                     int32_t *cell, int64_t capacity, int64_t *n_trial)
{
    if (!cell_names || n_cell < 1 || n_data < 0 || !n_trial ||
        (n_data > 0 && (!data_names || !data_rt || !data_len)))
        return GGDMC_ERR_ARG;
    int64_t n = 0;
    for (int i = 0; i < n_data; ++i) {
        if (data_len[i] < 0 || (data_len[i] > 0 && !data_rt[i]) || !data_names[i])
            return GGDMC_ERR_ARG;
        n += data_len[i];
    }
    *n_trial = n;
    if (!rt && !cell) return GGDMC_OK;              /* size query */
    if (!rt || !cell || capacity < n) return GGDMC_ERR_ARG;
    int64_t o = 0;
    for (int i = 0; i < n_data; ++i) {
        const int c = find_name(data_names[i], cell_names, n_cell);
        if (c < 0) return GGDMC_ERR_ARG;               /* a data cell the model lacks */
        for (int32_t t = 0; t < data_len[i]; ++t, ++o) {
            rt[o] = data_rt[i][t];
            cell[o] = c;
        }
    }
    return GGDMC_OK;
}

EXPORT ggdmc_status ggdmc_prior_row(const char *const *field_names, const double *field_values,
                                    int32_t n_field, double *row)
{
    if (!field_names || !field_values || !row || n_field < 1) return GGDMC_ERR_ARG;
    static const char *const kField[6] = {"p0", "p1", "lower", "upper", "dist_id", "log_p"};
    /* a missing or NA bound is open; log_p defaults to TRUE */
    const double dflt[6] = {NAN, NAN, -INFINITY, INFINITY, NAN, 1.0};
    for (int q = 0; q < 6; ++q) {
        const int i = find_name(kField[q], field_names, n_field);
        double v = (i >= 0) ? field_values[i] : NAN;
        if (isnan(v)) v = dflt[q];
        if (isnan(v)) return GGDMC_ERR_ARG;             /* p0, p1 and dist_id are required */
        row[q] = v;
    }
    return GGDMC_OK;
}

EXPORT ggdmc_status ggdmc_transpose(const double *in, int32_t n_row, int32_t n_col, double *out)
{
    if (!in || !out || n_row < 0 || n_col < 0) return GGDMC_ERR_ARG;
    for (int32_t r = 0; r < n_row; ++r)
        for (int32_t c = 0; c < n_col; ++c) out[(size_t)r * n_col + c] = in[r + (size_t)n_row * c];
    return GGDMC_OK;
}
