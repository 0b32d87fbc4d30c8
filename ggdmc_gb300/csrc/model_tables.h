// model_tables.h -- the flattened design as the kernels read it.
//
// ggdmc's model_boolean maps (cell, accumulator) to parameter names; most
// (cell, accumulator) pairs share the same (A, B, mean_v, sd_v) sources
// (fixture lba_data5: 96 cells x 4 accumulators use 8 distinct tuples).  The
// host therefore deduplicates them into "entries": per proposal the kernels
// resolve each entry once (A, b = A + B, v, s and the normalisation
// Phi(v/s)), and each trial only looks up the entry index of its cell and
// accumulator.
#pragma once
#include <cstdint>

namespace ggdmc {

constexpr int kMaxAcc = 8;        // accumulators per cell
constexpr int kMaxEnt = 255;      // distinct accumulator tuples (uint8 index)
constexpr int kMaxCell = 4096;
constexpr int kMaxPar = 64;       // subject-level parameters
constexpr int kMaxChain = 1024;
constexpr int kMaxTheta = 128;    // longest theta vector at any level (phi = 2P)

// Parameter source: >= 0 theta index, < 0 is -1-j into the constants.
struct EntSrc {
    int32_t A, B, v, s;
};

constexpr int kMaxT0 = 255;      // distinct t0 sources (uint8 index)
constexpr int kMaxDent = 255;    // distinct DDM tuples (uint8 index)
constexpr int kModelDdm = 1;

struct DevModel {
    int32_t model_type;     // 0 LBA, 1 DDM
    int32_t n_par;
    int32_t n_cell;
    int32_t n_acc;
    int32_t n_ent;          // distinct tuples
    int32_t n_const;
    int32_t n_t0;           // distinct t0 sources
    const EntSrc *ent_src;  // [n_ent]          (LBA)
    const uint8_t *cell_ent;// [n_cell][n_acc]  entry index
    const uint8_t *cell_w;  // [n_cell]         responding accumulator
    const uint8_t *cell_t0; // [n_cell]         index into t0_src
    const int32_t *t0_src;  // [n_t0]           source of each distinct t0
    int32_t n_dent;         // distinct DDM (parameter sources, boundary) tuples
    const int32_t *ddm_src; // [n_dent][9]      DDM: a, v, z, d, sz, sv, t0, st0 sources + boundary
    const double *consts;   // [n_const]
};

__host__ __device__ inline double src_value(int32_t src, const double *theta, const double *consts)
{
    return src >= 0 ? theta[src] : consts[-1 - src];
}

}  // namespace ggdmc
