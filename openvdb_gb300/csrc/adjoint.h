// Adjoint (reverse-mode) kernels of the advection hot path.
//
// The forward pass records a tape per CFL substep; the kernels below run the
// transposed Jacobians of the recorded operations with the topology, the
// upwind directions, the Godunov branches and the trim decisions held fixed
// as recorded; the time steps' dependence on the velocity is carried.  All
// adjoint arrays use "leaf-index" numbering: leaf l of a recorded list
// stores its packed values at [l*512 + rank].  Every sum runs in a fixed
// order (no floating-point atomics), so a backward sweep is deterministic.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gbls_internal.cuh"

namespace gbls {

// Gather slot-numbered state into leaf-index numbering.
void launch_tape_gather(int64_t n, const int32_t* slot, const uint64_t* am, const uint64_t* sm,
                        const float* vals, uint64_t* am_o, uint64_t* sm_o, float* vals_o, cudaStream_t s);
// Neighbour table in leaf-index numbering: inv[slot] = leaf, then remap.
void launch_nbr_to_index(int64_t n, const int32_t* slot, const int32_t* nbr, int32_t* inv, int64_t slot_cap,
                         int32_t* nbr_o, cudaStream_t s);
// Masks only (slot -> leaf index).
void launch_mask_gather(int64_t n, const int32_t* slot, const uint64_t* m, uint64_t* m_o, cudaStream_t s);

// The stage kernels write the transposed stencil sums of each leaf to
// part[leaf * 512 + voxel] (its own voxels, by position) and halo[(leaf * 6 +
// face) * 192 + ...] (the three-voxel slabs of its face neighbours);
// launch_adj_combine adds them into the packed adjoint in a fixed order.
struct AdjRkArgs {
    int64_t nleaf;
    const uint64_t* keys;
    const int32_t* nbr;
    Layout src;            // stage input phi (leaf-index numbering)
    const float* lam_out;  // adjoint of the stage output (same layout)
    float* part;           // beta (I - dt J)^T lam_out, own voxels
    float* halo;           // and face-neighbour slabs
    float alpha, beta, dt, gamma, invdx, t0;
    int backward;
    FieldParams field;
    float* dvel;           // DENSE field gradient [nx][ny][nz][3] (null: not wanted)
    double* dt_part;       // per leaf: += dL/d(dt) of the stage (null: not wanted)
};

// The voxel whose |v|^2 set a substep's time step: the first active voxel
// (canonical order) where |v|^2 equals the recorded maximum.
struct AdjArgmaxArgs {
    int64_t nleaf;
    const uint64_t* keys;
    const uint64_t* am;
    FieldParams field;
    float t0, maxv2;
    unsigned long long* argkey;  // leaf * 512 + voxel, minimised (preset to ~0)
    int64_t* argcell;            // out: the DENSE cell of that voxel (-1: none)
};

struct AdjNormArgs {
    int64_t nleaf;
    const int32_t* nbr;
    Layout src;              // renormalisation input (leaf-index numbering)
    const uint64_t* pmask;   // renormalised voxels
    const float* lam4;       // adjoint of the output, packed by pmask rank
    float* part;             // J^T lam4, own voxels
    float* halo;             // and face-neighbour slabs
    float gamma, mdt, invdx;
};

struct AdjCombineArgs {
    int64_t nleaf;
    const int32_t* nbr;      // face neighbours (leaf-index numbering)
    const uint64_t* am;      // active masks of the packed layout
    const float* part;
    const float* halo;
    float* lam;              // += part + neighbour halos (packed by am rank)
    const float* lam_out;    // with lam_phin: lam_phin += alpha lam_out
    float* lam_phin;
    float alpha;
};

struct AdjExpandArgs {
    int64_t nleaf;            // merged (dilated) list
    const uint64_t* pmask;    // renormalised voxels of each merged leaf
    const uint64_t* fin;      // voxels still active after trimming
    const int32_t* keep;      // 1 when the leaf survived the prune
    const int32_t* idx;       // its index in the next list
    const float* lam_next;    // adjoint on the next list (packed by fin rank)
    float* lam4;              // out: packed by pmask rank (0 on trimmed voxels)
};

struct AdjMapArgs {
    int64_t nleaf;             // pre-dilation list
    const uint64_t* keys;      // its keys
    const uint64_t* am;        // its masks
    const uint64_t* keys_m;    // merged list keys
    int64_t nleaf_m;
    const float* lam_m;        // adjoint on the merged list (same layout per leaf)
    float* lam;                // out
};

void launch_adj_rk(const AdjRkArgs& a, cudaStream_t s);
void launch_adj_norm(const AdjNormArgs& a, cudaStream_t s);
void launch_adj_combine(const AdjCombineArgs& a, cudaStream_t s);
void launch_adj_expand(const AdjExpandArgs& a, cudaStream_t s);
void launch_adj_map(const AdjMapArgs& a, cudaStream_t s);
void launch_adj_argmax(const AdjArgmaxArgs& a, cudaStream_t s);
// out = sum of part[0..n) in a fixed order (one CTA)
void launch_adj_dt_reduce(const double* part, int64_t n, double* out, cudaStream_t s);
// dvel[cell_k] += 2 mbar_k v[cell_k] for k = 0..n-1 in order (one thread):
// the velocity's part in the time steps, through |v|^2 at each step's maximum
void launch_adj_dt_scatter(int64_t n, const int64_t* cell, const float* mbar, const float* dense, float* dvel,
                           cudaStream_t s);

}  // namespace gbls
