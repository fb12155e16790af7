// Kernels of LevelSetFilter (tools/LevelSetFilter.h) on the device: one
// pass updates every active voxel from the staged 14^3 tile of its leaf
// (values of the previous pass), as the reference's Filter::cook does over
// its leaf buffers, and writes the result in the same packed layout:
//   LAPLACIAN  phi + dt * invdx2 * (sum of the six face neighbours - 6 phi)
//              (laplacianImpl :452-477, GradStencil::laplacian,
//              math/Stencils.h:1294-1299), dt = dx^2 / 6;
//   BOX        the mean of the 2w+1 values along one axis, summed in index
//              order and scaled by 1/(2w+1) (Filter::Avg :206-219, boxImpl
//              :327-349); w <= 3, the tile's halo;
//   OFFSET     phi + offset (offsetImpl :479-497).
#pragma once

#include "stencil_ops.cuh"

namespace gbls {

enum FilterOp { FILTER_LAPLACIAN = 0, FILTER_BOX = 1, FILTER_OFFSET = 2 };

struct FilterArgs {
    int64_t nleaf;
    const int32_t* slot;
    const int32_t* nbr;
    Layout src;
    float* out;
    float gamma;
    int op, axis, width;
    float frac;     // BOX: 1 / (2w + 1)
    float dt, invdx2;  // LAPLACIAN
    float offset;   // OFFSET
};

template <class A>
__global__ void __launch_bounds__(STENCIL_THREADS) filter_kernel(const FilterArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ uint16_t list[LEAF_VOX];
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    stage_masks(st, a.src, s, a.nbr + 6 * l, nullptr, nullptr);
    load_tile(tile, st, a.gamma);
    const int n = build_list(list, st.am[0]);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += STENCIL_THREADS) {
        const int v = list[i];
        const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
        const float c = tile[tile_index(x, y, z)];
        float r;
        if (a.op == FILTER_LAPLACIAN) {
            float sum = A::add(tile[tile_index(x - 1, y, z)], tile[tile_index(x + 1, y, z)]);
            sum = A::add(sum, tile[tile_index(x, y - 1, z)]);
            sum = A::add(sum, tile[tile_index(x, y + 1, z)]);
            sum = A::add(sum, tile[tile_index(x, y, z - 1)]);
            sum = A::add(sum, tile[tile_index(x, y, z + 1)]);
            const float lap = A::mul(a.invdx2, A::sub(sum, A::mul(6.0f, c)));
            r = A::add(c, A::mul(a.dt, lap));
        } else if (a.op == FILTER_BOX) {
            float sum = 0.0f;
            for (int k = -a.width; k <= a.width; ++k) {
                const int xx = x + (a.axis == 0 ? k : 0), yy = y + (a.axis == 1 ? k : 0),
                          zz = z + (a.axis == 2 ? k : 0);
                sum = A::add(sum, tile[tile_index(xx, yy, zz)]);
            }
            r = A::mul(sum, a.frac);
        } else {
            r = A::add(c, a.offset);
        }
        a.out[size_t(s) * LEAF_VOX + i] = r;
    }
}

}  // namespace gbls
