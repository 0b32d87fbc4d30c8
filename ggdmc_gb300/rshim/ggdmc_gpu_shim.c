/*
 * ggdmc_gpu_shim.c -- the .Call shim that puts libggdmc_gpu.so behind ggdmc's
 * three sampling entry points.
 *
 * The reference registers (src/RcppExports.cpp:54-64):
 *
 *   _ggdmc_run_subject(config, dmi,  samples)  -> src/de2R.cpp:8-23
 *   _ggdmc_run_hyper  (config, dmi,  samples)  -> src/de2R.cpp:30-47
 *   _ggdmc_run        (config, dmis, samples)  -> src/de2R.cpp:123-171
 *
 * and this file defines the same three with the same arguments and results:
 * ggdmc_gpu_run_subject / ggdmc_gpu_run_hyper return an S4 `posterior`
 * (src/type_casting.h:10-25), ggdmc_gpu_run returns list(phi = posterior,
 * subject_theta = list(posterior, ...)) (src/de2R.cpp:158-170).  The R stubs
 * in R/RcppExports.R:6-8,12-14,81-83 change only their .Call target; the
 * callers (StartSampling, RestartSampling, R/sampling.R) are unchanged.
 *
 * It reads the S4 slots with the R C API and hands flat arrays to the
 * converters of ggdmc_dmi.h, calls one function of ggdmc_gpu.h, and lets the
 * library write the samples straight into the new posterior's arrays, whose
 * memory order ([npar, nchain, nmc] and [nchain, nmc], column-major) is the
 * library's.  Library errors become R errors, as END_RCPP turns the
 * reference's C++ exceptions into R errors (src/RcppExports.cpp:17-25).
 *
 * Build: compiled into the R package next to src/RcppExports.cpp, with
 * PKG_CPPFLAGS = -I<ggdmc_gb300>/include and PKG_LIBS = -L<ggdmc_gb300>
 * -lggdmc_gpu.  It needs R's headers, which this repository's build machines
 * do not have, so the library's build does not compile it.
 *
 * Precision: R option ggdmc_gpu_precision, "mixed" (default) or "fp64".
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <R.h>
#include <Rinternals.h>
#include <R_ext/Rdynload.h>

#include "ggdmc_dmi.h"
#include "ggdmc_gpu.h"

/* ------------------------------------------------------------ R helpers */
static SEXP slot(SEXP obj, const char *name) { return R_do_slot(obj, Rf_install(name)); }

/* obj@name <- value (value is protected while the symbol is looked up) */
static void set_slot(SEXP obj, const char *name, SEXP value)
{
    PROTECT(value);
    R_do_slot_assign(obj, Rf_install(name), value);
    UNPROTECT(1);
}

/* Element `name` of a named list, or R_NilValue. */
static SEXP elt(SEXP list, const char *name)
{
    SEXP nm = Rf_getAttrib(list, R_NamesSymbol);
    if (Rf_isNull(nm)) return R_NilValue;
    for (R_xlen_t i = 0; i < XLENGTH(list); ++i)
        if (strcmp(CHAR(STRING_ELT(nm, i)), name) == 0) return VECTOR_ELT(list, i);
    return R_NilValue;
}

/* A character vector as C strings (R_alloc: freed when the .Call returns). */
static const char **strings(SEXP x, int32_t *n)
{
    *n = Rf_isNull(x) ? 0 : (int32_t)XLENGTH(x);
    const char **out = (const char **)R_alloc((size_t)(*n > 0 ? *n : 1), sizeof(char *));
    for (int32_t i = 0; i < *n; ++i) out[i] = CHAR(STRING_ELT(x, i));
    return out;
}

static void lib_check(ggdmc_status s, const char *what)
{
    if (s != GGDMC_OK) Rf_error("ggdmc_gpu %s: %s", what, ggdmc_last_error());
}

static void conv_check(ggdmc_status s, const char *what)
{
    if (s != GGDMC_OK) Rf_error("ggdmc_gpu: cannot convert %s", what);
}

/* ------------------------------------------------------------ conversions */
/* dmi@model (+ the cell-name responder rule) -> ggdmc_model */
static void model_from_dmi(SEXP dmi, ggdmc_model *m)
{
    SEXP model = slot(dmi, "model");
    const char *type = CHAR(STRING_ELT(slot(model, "type"), 0));
    m->model_type = (strcmp(type, "ddm") == 0 || strcmp(type, "diffusion") == 0 ||
                     strcmp(type, "rd") == 0) ? GGDMC_MODEL_DDM : GGDMC_MODEL_LBA;
    m->n_kind = ggdmc_dmi_n_kind(m->model_type);
    SEXP mb = slot(model, "model_boolean");
    SEXP dim = Rf_getAttrib(mb, R_DimSymbol);
    if (Rf_length(dim) != 3) Rf_error("ggdmc_gpu: model_boolean is not a 3-way array");
    const int n_cell = INTEGER(dim)[0], n_pxc = INTEGER(dim)[1], n_acc = INTEGER(dim)[2];
    int32_t n_name, n_par, n_const, n_cellname, n_accname;
    const char **pxc = strings(slot(model, "parameter_x_condition_names"), &n_name);
    const char **pnames = strings(slot(model, "pnames"), &n_par);
    SEXP consts = PROTECT(Rf_coerceVector(slot(model, "constants"), REALSXP));
    const char **cnames = strings(Rf_getAttrib(consts, R_NamesSymbol), &n_const);
    const char **cells = strings(slot(model, "cell_names"), &n_cellname);
    const char **accs = strings(slot(model, "accumulators"), &n_accname);
    if (n_name != n_pxc || n_cellname != n_cell || n_accname != n_acc)
        Rf_error("ggdmc_gpu: model_boolean does not match the model's names");
    int32_t *src = (int32_t *)R_alloc((size_t)n_cell * n_acc * m->n_kind, sizeof(int32_t));
    conv_check(ggdmc_dmi_param_src(m->model_type, LOGICAL(mb), n_cell, n_pxc, n_acc, pxc, pnames,
                                   n_par, cnames, n_const, src), "model@model_boolean");
    int32_t *resp = (int32_t *)R_alloc((size_t)n_cell, sizeof(int32_t));
    conv_check(ggdmc_dmi_responders(cells, n_cell, accs, n_acc, resp), "model@cell_names");
    double *cv = (double *)R_alloc((size_t)(n_const > 0 ? n_const : 1), sizeof(double));
    for (int32_t j = 0; j < n_const; ++j) cv[j] = REAL(consts)[j];
    UNPROTECT(1);
    m->n_par = n_par;
    m->n_cell = n_cell;
    m->n_acc = n_acc;
    m->n_const = n_const;
    m->param_src = src;
    m->resp = resp;
    m->constants = cv;
}

/* dmi@data of every dmi in `dmis` (a list, or one S4 dmi) -> ggdmc_data */
static void data_from_dmis(SEXP dmis, SEXP model, ggdmc_data *d)
{
    const int one = Rf_isS4(dmis);
    const int S = one ? 1 : (int)XLENGTH(dmis);
    int32_t n_cell;
    const char **cells = strings(slot(model, "cell_names"), &n_cell);
    int64_t *offs = (int64_t *)R_alloc((size_t)S + 1, sizeof(int64_t));
    offs[0] = 0;
    for (int s = 0; s < S; ++s) {
        SEXP data = slot(one ? dmis : VECTOR_ELT(dmis, s), "data");
        int64_t n = 0;
        for (R_xlen_t i = 0; i < XLENGTH(data); ++i) n += XLENGTH(VECTOR_ELT(data, i));
        offs[s + 1] = offs[s] + n;
    }
    double *rt = (double *)R_alloc((size_t)(offs[S] > 0 ? offs[S] : 1), sizeof(double));
    int32_t *cell = (int32_t *)R_alloc((size_t)(offs[S] > 0 ? offs[S] : 1), sizeof(int32_t));
    for (int s = 0; s < S; ++s) {
        SEXP data = slot(one ? dmis : VECTOR_ELT(dmis, s), "data");
        int32_t n_data;
        const char **names = strings(Rf_getAttrib(data, R_NamesSymbol), &n_data);
        const double **vec = (const double **)R_alloc((size_t)(n_data > 0 ? n_data : 1), sizeof(double *));
        int32_t *len = (int32_t *)R_alloc((size_t)(n_data > 0 ? n_data : 1), sizeof(int32_t));
        for (int32_t i = 0; i < n_data; ++i) {
            SEXP v = VECTOR_ELT(data, i);
            vec[i] = REAL(v);
            len[i] = (int32_t)XLENGTH(v);
        }
        int64_t got = 0;
        conv_check(ggdmc_dmi_trials(cells, n_cell, names, vec, len, n_data, rt + offs[s], cell + offs[s],
                                    offs[s + 1] - offs[s], &got), "dmi@data");
    }
    d->n_subject = S;
    d->offsets = offs;
    d->rt = rt;
    d->cell = cell;
}

/* a ggdmcPrior list (one named list per parameter) -> ggdmc_prior */
static void prior_from_list(SEXP plist, ggdmc_prior *p)
{
    const int P = (int)XLENGTH(plist);
    double *table = (double *)R_alloc((size_t)P * 6, sizeof(double));
    for (int j = 0; j < P; ++j) {
        SEXP item = VECTOR_ELT(plist, j);
        int32_t nf;
        const char **fn = strings(Rf_getAttrib(item, R_NamesSymbol), &nf);
        double *fv = (double *)R_alloc((size_t)(nf > 0 ? nf : 1), sizeof(double));
        for (int32_t i = 0; i < nf; ++i) fv[i] = Rf_asReal(VECTOR_ELT(item, i));
        conv_check(ggdmc_prior_row(fn, fv, nf, table + 6 * (size_t)j), "a prior entry");
    }
    p->n_par = P;
    p->table = table;
}

/* config@de_input + config@theta_input (R/model-class.R:36-57, 1288-1313) */
static void config_from_s4(SEXP config, ggdmc_de_config *c)
{
    SEXP de = slot(config, "de_input"), ti = slot(config, "theta_input");
    memset(c, 0, sizeof *c);
    c->pop_migration_prob = Rf_asReal(slot(de, "pop_migration_prob"));
    c->sub_migration_prob = Rf_asReal(slot(de, "sub_migration_prob"));
    c->gamma_precursor = Rf_asReal(slot(de, "gamma_precursor"));
    c->rp = Rf_asReal(slot(de, "rp"));
    c->is_hblocked = Rf_asLogical(slot(de, "is_hblocked")) == TRUE;
    c->is_pblocked = Rf_asLogical(slot(de, "is_pblocked")) == TRUE;
    c->nparameter = Rf_asInteger(slot(de, "nparameter"));
    c->nchain = Rf_asInteger(slot(ti, "nchain"));
    c->nmc = Rf_asInteger(slot(ti, "nmc"));
    c->thin = Rf_asInteger(slot(ti, "thin"));
    c->seed = (uint64_t)(uint32_t)Rf_asInteger(slot(config, "seed"));
    c->precision = GGDMC_MIXED;
    SEXP opt = Rf_GetOption1(Rf_install("ggdmc_gpu_precision"));
    if (Rf_isString(opt) && strcmp(CHAR(STRING_ELT(opt, 0)), "fp64") == 0) c->precision = GGDMC_FP64;
}

/* The start state of a `samples` posterior: its last filled slice (slice 1
 * of a fresh initialise_theta / initialise_phi object, the last sample of a
 * previous run's posterior for RestartSampling). */
static void state_from_samples(SEXP samples, int P, int C, ggdmc_chain_state *st)
{
    SEXP th = slot(samples, "theta"), lp = slot(samples, "summed_log_prior"),
         ll = slot(samples, "log_likelihoods");
    const R_xlen_t per = (R_xlen_t)P * C;
    if (XLENGTH(th) < per || XLENGTH(th) % per != 0)
        Rf_error("ggdmc_gpu: samples@theta is not [npar, nchain, nmc] for this model");
    R_xlen_t k = XLENGTH(th) / per - 1;
    while (k > 0 && ISNAN(REAL(th)[per * k])) --k;
    st->theta = (double *)R_alloc((size_t)per, sizeof(double));
    st->lp = (double *)R_alloc((size_t)C, sizeof(double));
    st->ll = (double *)R_alloc((size_t)C, sizeof(double));
    memcpy(st->theta, REAL(th) + per * k, sizeof(double) * (size_t)per);
    memcpy(st->lp, REAL(lp) + (R_xlen_t)C * k, sizeof(double) * (size_t)C);
    memcpy(st->ll, REAL(ll) + (R_xlen_t)C * k, sizeof(double) * (size_t)C);
}

/* new_posterior (src/type_casting.h:10-25): a fresh S4 `posterior` whose
 * arrays the library fills.  Returned PROTECTed once. */
static SEXP new_posterior(int P, int C, const ggdmc_de_config *c, SEXP pnames, ggdmc_samples *smp)
{
    SEXP out = PROTECT(R_do_new_object(R_do_MAKE_CLASS("posterior")));
    SEXP th = PROTECT(Rf_alloc3DArray(REALSXP, P, C, c->nmc));
    SEXP lp = PROTECT(Rf_allocMatrix(REALSXP, C, c->nmc));
    SEXP ll = PROTECT(Rf_allocMatrix(REALSXP, C, c->nmc));
    set_slot(out, "theta", th);
    set_slot(out, "summed_log_prior", lp);
    set_slot(out, "log_likelihoods", ll);
    set_slot(out, "start", Rf_ScalarInteger(1));
    set_slot(out, "npar", Rf_ScalarInteger(P));
    set_slot(out, "pnames", pnames);
    set_slot(out, "nmc", Rf_ScalarInteger(c->nmc));
    set_slot(out, "thin", Rf_ScalarInteger(c->thin));
    set_slot(out, "nchain", Rf_ScalarInteger(C));
    smp->theta = REAL(th);
    smp->lp = REAL(lp);
    smp->ll = REAL(ll);
    UNPROTECT(4);
    return out;
}

/* ------------------------------------------------------------ entry points */
SEXP ggdmc_gpu_run_subject(SEXP config, SEXP dmi, SEXP samples)
{
    ggdmc_de_config cfg;
    ggdmc_model model;
    ggdmc_data data;
    ggdmc_prior prior;
    ggdmc_chain_state st;
    ggdmc_samples smp;
    config_from_s4(config, &cfg);
    model_from_dmi(dmi, &model);
    data_from_dmis(dmi, slot(dmi, "model"), &data);
    prior_from_list(slot(slot(config, "prior"), "p_prior"), &prior);
    state_from_samples(samples, model.n_par, cfg.nchain, &st);
    SEXP out = new_posterior(model.n_par, cfg.nchain, &cfg, slot(slot(config, "theta_input"), "pnames"), &smp);
    lib_check(ggdmc_run_subject(&cfg, &model, &data, &prior, &st, NULL, &smp, NULL), "run_subject");
    UNPROTECT(1);
    return out;
}

SEXP ggdmc_gpu_run_hyper(SEXP config, SEXP dmi, SEXP samples)
{
    ggdmc_de_config cfg;
    ggdmc_prior p_prior, h_prior;
    ggdmc_chain_state st;
    ggdmc_samples smp;
    config_from_s4(config, &cfg);
    SEXP priors = slot(config, "prior");
    prior_from_list(slot(priors, "p_prior"), &p_prior);
    prior_from_list(slot(priors, "h_prior"), &h_prior);
    /* hyper_dmi@data: the subject-by-parameter matrix [n_row, P] */
    SEXP x = PROTECT(Rf_coerceVector(slot(dmi, "data"), REALSXP));
    SEXP dim = Rf_getAttrib(slot(dmi, "data"), R_DimSymbol);
    if (Rf_length(dim) != 2 || INTEGER(dim)[1] != p_prior.n_par)
        Rf_error("ggdmc_gpu: hyper_dmi@data is not a [subject, parameter] matrix");
    const int n_row = INTEGER(dim)[0];
    double *rows = (double *)R_alloc((size_t)n_row * p_prior.n_par, sizeof(double));
    conv_check(ggdmc_transpose(REAL(x), n_row, p_prior.n_par, rows), "hyper_dmi@data");
    const int P = h_prior.n_par;
    state_from_samples(samples, P, cfg.nchain, &st);
    SEXP out = new_posterior(P, cfg.nchain, &cfg, slot(slot(config, "theta_input"), "pnames"), &smp);
    lib_check(ggdmc_run_hyper(&cfg, rows, n_row, &p_prior, &h_prior, &st, NULL, &smp, NULL), "run_hyper");
    UNPROTECT(2);
    return out;
}

SEXP ggdmc_gpu_run(SEXP config, SEXP dmis, SEXP samples)
{
    ggdmc_de_config cfg;
    ggdmc_model model;
    ggdmc_data data;
    ggdmc_prior p_prior, h_prior;
    ggdmc_chain_state phi_st;
    ggdmc_samples phi_smp;
    config_from_s4(config, &cfg);
    if (XLENGTH(dmis) < 1) Rf_error("ggdmc_gpu: dmis is empty");
    SEXP dmi0 = VECTOR_ELT(dmis, 0);
    model_from_dmi(dmi0, &model);
    data_from_dmis(dmis, slot(dmi0, "model"), &data);
    SEXP priors = slot(config, "prior");
    prior_from_list(slot(priors, "p_prior"), &p_prior);
    prior_from_list(slot(priors, "h_prior"), &h_prior);
    const int S = data.n_subject, C = cfg.nchain, P = model.n_par;

    SEXP subj_in = elt(samples, "subject_theta"), phi_in = elt(samples, "phi");
    if (Rf_isNull(subj_in) || Rf_isNull(phi_in) || XLENGTH(subj_in) != S)
        Rf_error("ggdmc_gpu: samples needs phi and one subject_theta per dmi");
    state_from_samples(phi_in, h_prior.n_par, C, &phi_st);
    ggdmc_chain_state *subj_st = (ggdmc_chain_state *)R_alloc((size_t)S, sizeof(ggdmc_chain_state));
    ggdmc_samples *subj_smp = (ggdmc_samples *)R_alloc((size_t)S, sizeof(ggdmc_samples));
    for (int s = 0; s < S; ++s) state_from_samples(VECTOR_ELT(subj_in, s), P, C, &subj_st[s]);

    /* the subjects' posteriors carry the model's free parameters
     * (src/de2R.cpp:135-136); phi's the config's theta_input */
    SEXP sub_pnames = slot(slot(dmi0, "model"), "pnames");
    SEXP theta_out = PROTECT(Rf_allocVector(VECSXP, S));
    for (int s = 0; s < S; ++s) {
        SET_VECTOR_ELT(theta_out, s, new_posterior(P, C, &cfg, sub_pnames, &subj_smp[s]));
        UNPROTECT(1);
    }
    SEXP phi_out = new_posterior(h_prior.n_par, C, &cfg, slot(slot(config, "theta_input"), "pnames"),
                                 &phi_smp);
    lib_check(ggdmc_run(&cfg, &model, &data, &p_prior, &h_prior, &phi_st, subj_st, NULL, &phi_smp,
                        subj_smp, NULL), "run");

    /* list(phi = posterior, subject_theta = list(...)) (src/de2R.cpp:158-170) */
    SEXP out = PROTECT(Rf_allocVector(VECSXP, 2));
    SEXP nm = PROTECT(Rf_allocVector(STRSXP, 2));
    SET_VECTOR_ELT(out, 0, phi_out);
    SET_VECTOR_ELT(out, 1, theta_out);
    SET_STRING_ELT(nm, 0, Rf_mkChar("phi"));
    SET_STRING_ELT(nm, 1, Rf_mkChar("subject_theta"));
    Rf_setAttrib(out, R_NamesSymbol, nm);
    UNPROTECT(4);
    return out;
}

/* ------------------------------------------------------------ registration */
static const R_CallMethodDef gpu_calls[] = {
    {"ggdmc_gpu_run_subject", (DL_FUNC)&ggdmc_gpu_run_subject, 3},
    {"ggdmc_gpu_run_hyper", (DL_FUNC)&ggdmc_gpu_run_hyper, 3},
    {"ggdmc_gpu_run", (DL_FUNC)&ggdmc_gpu_run, 3},
    {NULL, NULL, 0}};

/* Called from the package's R_init_ggdmc (src/RcppExports.cpp:61-64) beside
 * its own R_registerRoutines, or as R_init_<library> when the shim is built
 * as a library of its own. */
void ggdmc_gpu_register(DllInfo *dll) { R_registerRoutines(dll, NULL, gpu_calls, NULL, NULL); }
