// Host entry point over the FP32 LBA trial density of device_common.cuh
// (compiled for the host by tests/test_density32_host.py): one trial of an
// accumulator design given its tuples (A, B, v, s) winner first and t0.
#include "device_common_host.h"

using namespace ggdmc;

// 0: the FP32 form's log density in *logd; 1: the trial takes the FP64 form;
// 2: a tuple outside the FP32 form's domain (the proposal takes FP64)
extern "C" int dc_trial(double rt, double t0, int K, const double *abvs, double *logd)
{
    Ent32 E[8];
    double lgw = 0.0;
    for (int k = 0; k < K; ++k) {
        double lg;
        if (!lba_tuple32(abvs[4 * k], abvs[4 * k + 1], abvs[4 * k + 2], abvs[4 * k + 3], E[k], lg)) return 2;
        if (k == 0) lgw = lg;
    }
    const float rh = (float)rt, th = (float)t0;
    const float2 r2 = make_float2(rh, (float)(rt - (double)rh)), t2 = make_float2(th, (float)(t0 - (double)th));
    uint8_t ents[8] = {0, 1, 2, 3, 4, 5, 6, 7};
    int e;
    float lm;
    if (t_before(r2, t2)) {                  // the floor as the winner's tuple stores it
        *logd = lgw + (double)E[0].a.y * 0.6931471805599453 + (double)E[0].b.y;
        return 0;
    }
    if (!lba_ld32_n(r2, t2, ents, K, E, e, lm)) return 1;
    *logd = lgw + e * 0.6931471805599453 + (double)lm;
    return 0;
}

// One diffusion-model trial: the responding boundary's (a, v, z, d, sz, sv,
// t0, st0) and whether it is the upper one.  0: the FP32 form's log density
// in *logd; 1: the trial takes the FP64 form.
extern "C" int dc_ddm(double rt, const double *v8, int upper, double *logd)
{
    double e[8];
    float f[8];
    ddm_entry(v8, upper != 0, e, f);
    const float rh = (float)rt, rl = (float)(rt - (double)rh);
    float ld;
    if (!ddm_logdens32(rh, rl, f, ld)) return 1;
    *logd = ld;
    return 0;
}
