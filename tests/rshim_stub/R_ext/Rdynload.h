/* R's routine-registration declarations used by the shim (see ../R.h). */
#ifndef GGDMC_RSHIM_STUB_RDYNLOAD_H
#define GGDMC_RSHIM_STUB_RDYNLOAD_H
typedef void *(*DL_FUNC)(void);
typedef struct {
    const char *name;
    DL_FUNC fun;
    int numArgs;
} R_CallMethodDef;
typedef struct _DllInfo DllInfo;
int R_registerRoutines(DllInfo *info, const void *croutines, const R_CallMethodDef *callRoutines,
                       const void *fortranRoutines, const void *externalRoutines);
#endif
