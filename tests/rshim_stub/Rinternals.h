/* The subset of R's Rinternals.h API used by ggdmc_gb300/rshim/ggdmc_gpu_shim.c,
 * declared with R's signatures (see R.h here).  Test infrastructure only. */
#ifndef GGDMC_RSHIM_STUB_RINTERNALS_H
#define GGDMC_RSHIM_STUB_RINTERNALS_H
#include <math.h>
#include "R.h"
typedef struct SEXPREC *SEXP;
typedef ptrdiff_t R_xlen_t;
typedef unsigned int SEXPTYPE;
typedef enum { FALSE = 0, TRUE } Rboolean;
#define REALSXP 14
#define STRSXP 16
#define VECSXP 19
#define ISNAN(x) (isnan(x) != 0)
extern SEXP R_NilValue;
extern SEXP R_NamesSymbol;
extern SEXP R_DimSymbol;
SEXP Rf_install(const char *);
SEXP R_do_slot(SEXP obj, SEXP name);
SEXP R_do_slot_assign(SEXP obj, SEXP name, SEXP value);
SEXP R_do_MAKE_CLASS(const char *what);
SEXP R_do_new_object(SEXP class_def);
SEXP Rf_getAttrib(SEXP, SEXP);
SEXP Rf_setAttrib(SEXP, SEXP, SEXP);
Rboolean Rf_isNull(SEXP);
Rboolean Rf_isS4(SEXP);
Rboolean Rf_isString(SEXP);
R_xlen_t XLENGTH(SEXP x);
int Rf_length(SEXP);
SEXP VECTOR_ELT(SEXP x, R_xlen_t i);
SEXP SET_VECTOR_ELT(SEXP x, R_xlen_t i, SEXP v);
SEXP STRING_ELT(SEXP x, R_xlen_t i);
void SET_STRING_ELT(SEXP x, R_xlen_t i, SEXP v);
const char *CHAR(SEXP x);
SEXP Rf_mkChar(const char *);
double *REAL(SEXP x);
int *INTEGER(SEXP x);
int *LOGICAL(SEXP x);
double Rf_asReal(SEXP x);
int Rf_asInteger(SEXP x);
int Rf_asLogical(SEXP x);
SEXP Rf_coerceVector(SEXP, SEXPTYPE);
SEXP Rf_allocVector(SEXPTYPE, R_xlen_t);
SEXP Rf_allocMatrix(SEXPTYPE, int, int);
SEXP Rf_alloc3DArray(SEXPTYPE, int, int, int);
SEXP Rf_ScalarInteger(int);
SEXP Rf_GetOption1(SEXP);
SEXP Rf_protect(SEXP);
void Rf_unprotect(int);
#define PROTECT(s) Rf_protect(s)
#define UNPROTECT(n) Rf_unprotect(n)
#endif
