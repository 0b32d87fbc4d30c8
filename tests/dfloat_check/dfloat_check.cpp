// Host entry points over ggdmc_gb300/csrc/dfloat.h and fquantile.h for
// tests/test_dfloat.py and tests/test_diagnostics.py:
// each takes n doubles, splits them to hi + lo, applies one double-float
// function and writes the result back as a double.
#include "dfloat.h"

using namespace ggdmc;

extern "C" {
void dfc_exp(const double *x, double *y, int n)
{
    for (int i = 0; i < n; ++i) y[i] = df_to_double(df_exp(df_from_double(x[i])));
}
void dfc_log(const double *x, double *y, int n)
{
    for (int i = 0; i < n; ++i) y[i] = df_to_double(df_log(df_from_double(x[i])));
}
void dfc_qtail(const double *x, double *y, int n)
{
    for (int i = 0; i < n; ++i) y[i] = df_to_double(df_qtail(df_from_double(x[i])));
}
void dfc_phi_pair(const double *x, double *pk, double *pnk, int n)
{
    for (int i = 0; i < n; ++i) {
        dfl a, b;
        df_phi_pair(df_from_double(x[i]), a, b);
        pk[i] = df_to_double(a);
        pnk[i] = df_to_double(b);
    }
}
void dfc_div(const double *a, const double *b, double *y, int n)
{
    for (int i = 0; i < n; ++i) y[i] = df_to_double(df_div(df_from_double(a[i]), df_from_double(b[i])));
}
void dfc_mul(const double *a, const double *b, double *y, int n)
{
    for (int i = 0; i < n; ++i) y[i] = df_to_double(df_mul(df_from_double(a[i]), df_from_double(b[i])));
}
void dfc_add(const double *a, const double *b, double *y, int n)
{
    for (int i = 0; i < n; ++i) y[i] = df_to_double(df_add(df_from_double(a[i]), df_from_double(b[i])));
}
}

#include "fquantile.h"

extern "C" void fqc_quantile(const double *p, const double *d1, const double *d2, double *y, int n)
{
    for (int i = 0; i < n; ++i) y[i] = f_quantile(p[i], d1[i], d2[i]);
}
