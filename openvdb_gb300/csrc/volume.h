// Volume advection kernels: tools::VolumeAdvection (tools/VolumeAdvect.h)
// for FloatGrid volumes in a Vec3f velocity grid (dense box, trilinear
// BoxSampler, non-staggered), semi-Lagrangian with RK1-4, MacCormack and
// BFECC, CLAMP / REVERT limiters.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gbls_internal.cuh"

namespace gbls {

// A device tree sampled with ValueAccessor::getValue semantics: a leaf's
// voxel (active: its packed value; inactive: +-background by its sign bit),
// else the covering tile (+-background by the node tables).  slot == null:
// leaf i stores its values at [i * 512].
struct VolGrid {
    const uint64_t* keys;
    const int32_t* slot;
    int64_t nleaf;
    const uint64_t* amask;
    const uint64_t* smask;
    const float* vals;
    NodeTables nodes;
    float background;
};

// Linear maps index <-> world (uniform scale and translation):
// world = index * scale + t, index = (world - t) * inv (inv = 1 / scale).
struct VolMap {
    double scale, inv, t[3];
};

// The velocity grid: a dense box of Vec3f (background outside), its map,
// or a constant velocity (kind 0).
struct VolVelocity {
    int kind;                 // 0: constant, 1: dense box
    float constant[3];
    int origin[3], dims[3];
    const float* dense;       // [nx][ny][nz][3]
    float background[3];
    VolMap map;
};

// The output topology (the handle's current layout): every active voxel
// of every leaf gets a value.
struct VolOut {
    int64_t nleaf;
    const uint64_t* keys;
    const int32_t* slot;
    const uint64_t* amask;
};

enum { VOL_COMBINE_MAC = 0, VOL_COMBINE_BFECC = 1 };

struct VolRkArgs {
    VolOut out;
    float* dst;        // [slot * 512 + rank]
    VolGrid src;       // the grid sampled at the end of the characteristic
    VolMap map;        // the volume's map
    VolVelocity vel;
    float dt;          // RealT(-time_step) or its negation
    int order;         // 1..4
};

struct VolCombineArgs {
    VolOut out;
    float* out0;       // buffer 0 (read and written)
    const float* out1; // buffer 1
    VolGrid in;        // the input grid, looked up at each voxel
    int op;            // VOL_COMBINE_*
};

struct VolLimitArgs {
    VolOut out;
    float* vals;       // buffer 0, limited in place
    uint64_t* keep;    // [slot * 8]: active voxels that stay active
    VolGrid in;
    VolMap map;
    VolVelocity vel;
    float dt;
    int limiter;       // 0 none, 1 clamp, 2 revert (only when do_limit)
    int do_limit;
    float background;
};

// atomicMax of the Vec3f lengths of n dense velocities into *max_bits
// (float bits; non-negative floats order like their bits)
void launch_vol_max_speed(const float* dense, int64_t n, unsigned int* max_bits, cudaStream_t s);
void launch_vol_rk(const VolRkArgs& a, cudaStream_t s);
void launch_vol_combine(const VolCombineArgs& a, cudaStream_t s);
void launch_vol_limit(const VolLimitArgs& a, cudaStream_t s);

}  // namespace gbls
