/* Declarations of the R C API entry points the .Call shim uses, with R's
 * signatures, so that the shim can be compiled (syntax and types) where R's
 * own headers are not installed.  Test infrastructure only: nothing links it. */
#ifndef GGDMC_RSHIM_STUB_R_H
#define GGDMC_RSHIM_STUB_R_H
#include <stddef.h>
#include <stdint.h>
void Rf_error(const char *fmt, ...);
char *R_alloc(size_t n, int size);
#endif
