// tools::VolumeAdvection (tools/VolumeAdvect.h:336-560) on the device: the
// per-voxel passes of Advect::cook for FloatGrid volumes.  Every float
// operation is the reference's, with explicit round-to-nearest intrinsics
// (the unit is also built with -fmad=false): the characteristic is traced
// through VelocityIntegrator::rungeKutta (tools/VelocityFields.h:229-266)
// in a Vec3f velocity grid sampled by BoxSampler, and the volume is sampled
// by BoxSampler::sample (tools/Interpolation.h:714-781).
#include "volume.h"

namespace gbls {

namespace {

constexpr int VOL_THREADS = 64;

// ValueAccessor::getValue of the grid at index (x, y, z).
__device__ float vol_value(const VolGrid& g, int x, int y, int z) {
    if (x < -COORD_LIMIT || x >= COORD_LIMIT || y < -COORD_LIMIT || y >= COORD_LIMIT || z < -COORD_LIMIT ||
        z >= COORD_LIMIT)
        return g.background;
    const uint64_t key = leaf_key(x, y, z);
    const int64_t i = find_u64(g.keys, g.nleaf, key);
    if (i < 0) return tile_sign(g.nodes, key) ? -g.background : g.background;
    const size_t s = g.slot ? size_t(g.slot[i]) : size_t(i);
    const int v = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7);
    const int w = v >> 6, b = v & 63;
    const uint64_t m = g.amask[s * 8 + w];
    if ((m >> b) & 1) {
        int rank = __popcll(m & ((uint64_t(1) << b) - 1));
        for (int k = 0; k < w; ++k) rank += __popcll(g.amask[s * 8 + k]);
        return g.vals[s * LEAF_VOX + rank];
    }
    return ((g.smask[s * 8 + w] >> b) & 1) ? -g.background : g.background;
}

// BoxSampler's `a + ValueT((b - a) * weight)` (float difference, double
// product rounded to float, float sum).
__device__ __forceinline__ float lerp_box(float a, float b, double w) {
    return __fadd_rn(a, __double2float_rn(__dmul_rn(double(__fsub_rn(b, a)), w)));
}

// Coord::floor of an index-space position, within the key range.
__device__ __forceinline__ bool floor_coord(const double q[3], int i0[3], double uvw[3]) {
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double f = floor(q[a]);
        ok &= f > -double(COORD_LIMIT) && f < double(COORD_LIMIT);
        i0[a] = ok ? int(f) : 0;
        uvw[a] = __dsub_rn(q[a], double(i0[a]));
    }
    return ok;
}

// BoxSampler::getValues (tools/Interpolation.h:629-655) from the volume.
__device__ void box_values(const VolGrid& g, const int i0[3], float d[2][2][2]) {
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int z = 0; z < 2; ++z) d[x][y][z] = vol_value(g, i0[0] + x, i0[1] + y, i0[2] + z);
}

// BoxSampler::trilinearInterpolation (tools/Interpolation.h:714-741).
__device__ __forceinline__ float box_trilinear(const float d[2][2][2], const double uvw[3]) {
    return lerp_box(lerp_box(lerp_box(d[0][0][0], d[0][0][1], uvw[2]), lerp_box(d[0][1][0], d[0][1][1], uvw[2]),
                             uvw[1]),
                    lerp_box(lerp_box(d[1][0][0], d[1][0][1], uvw[2]), lerp_box(d[1][1][0], d[1][1][1], uvw[2]),
                             uvw[1]),
                    uvw[0]);
}

// map.worldToIndex / indexToWorld of a uniform scale + translation map.
__device__ __forceinline__ double to_index(const VolMap& m, double w, int a) {
    return __dmul_rn(__dsub_rn(w, m.t[a]), m.inv);
}
__device__ __forceinline__ double to_world(const VolMap& m, double i, int a) {
    return __dadd_rn(__dmul_rn(i, m.scale), m.t[a]);
}

// The velocity grid's value at index (i, j, k).
__device__ __forceinline__ void vel_value(const VolVelocity& v, int i, int j, int k, float out[3]) {
    const int a = i - v.origin[0], b = j - v.origin[1], c = k - v.origin[2];
    if (a >= 0 && b >= 0 && c >= 0 && a < v.dims[0] && b < v.dims[1] && c < v.dims[2]) {
        const float* p = v.dense + 3 * ((size_t(a) * v.dims[1] + b) * v.dims[2] + c);
        out[0] = __ldg(p); out[1] = __ldg(p + 1); out[2] = __ldg(p + 2);
    } else {
        out[0] = v.background[0]; out[1] = v.background[1]; out[2] = v.background[2];
    }
}

// VelocitySampler::sample (tools/VelocityFields.h:176-181): the velocity at
// the world position P (a Vec3f), through the velocity grid's worldToIndex
// and BoxSampler.
__device__ void vel_sample(const VolVelocity& v, const float P[3], float out[3]) {
    if (v.kind == 0) {
        out[0] = v.constant[0]; out[1] = v.constant[1]; out[2] = v.constant[2];
        return;
    }
    double q[3], uvw[3];
    int i0[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) q[a] = to_index(v.map, double(P[a]), a);
    if (!floor_coord(q, i0, uvw)) {
        out[0] = v.background[0]; out[1] = v.background[1]; out[2] = v.background[2];
        return;
    }
    float d[2][2][2][3];
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int z = 0; z < 2; ++z) vel_value(v, i0[0] + x, i0[1] + y, i0[2] + z, d[x][y][z]);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float a0 = lerp_box(lerp_box(d[0][0][0][c], d[0][0][1][c], uvw[2]),
                                  lerp_box(d[0][1][0][c], d[0][1][1][c], uvw[2]), uvw[1]);
        const float a1 = lerp_box(lerp_box(d[1][0][0][c], d[1][0][1][c], uvw[2]),
                                  lerp_box(d[1][1][0][c], d[1][1][1][c], uvw[2]), uvw[1]);
        out[c] = lerp_box(a0, a1, uvw[0]);
    }
}

// P + s * V component-wise (Vec3f arithmetic, s a float scalar).
__device__ __forceinline__ void axpy(const float P[3], float s, const float V[3], float out[3]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) out[c] = __fadd_rn(P[c], __fmul_rn(s, V[c]));
}

// VelocityIntegrator::rungeKutta<Order, Vec3d>(dt, world) (tools/VelocityFields.h:229-266).
__device__ void runge_kutta(const VolVelocity& v, int order, float dt, double w[3]) {
    float P[3] = {float(w[0]), float(w[1]), float(w[2])};
    float V0[3], V1[3], V2[3], V3[3], Q[3], D[3];
    vel_sample(v, P, V0);
    const float half_dt = __fmul_rn(0.5f, dt);
    if (order == 1) {
#pragma unroll
        for (int c = 0; c < 3; ++c) D[c] = __fmul_rn(dt, V0[c]);
    } else if (order == 2) {
        axpy(P, half_dt, V0, Q);
        vel_sample(v, Q, V1);
#pragma unroll
        for (int c = 0; c < 3; ++c) D[c] = __fmul_rn(dt, V1[c]);
    } else if (order == 3) {
        axpy(P, half_dt, V0, Q);
        vel_sample(v, Q, V1);
        float E[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) E[c] = __fsub_rn(__fmul_rn(2.0f, V1[c]), V0[c]);
        axpy(P, dt, E, Q);
        vel_sample(v, Q, V2);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float s = __fadd_rn(__fadd_rn(V0[c], __fmul_rn(4.0f, V1[c])), V2[c]);
            D[c] = __fmul_rn(__fmul_rn(dt, s), float(1.0 / 6.0));
        }
    } else {
        axpy(P, half_dt, V0, Q);
        vel_sample(v, Q, V1);
        axpy(P, half_dt, V1, Q);
        vel_sample(v, Q, V2);
        axpy(P, dt, V2, Q);
        vel_sample(v, Q, V3);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float s = __fadd_rn(__fadd_rn(V0[c], __fmul_rn(2.0f, __fadd_rn(V1[c], V2[c]))), V3[c]);
            D[c] = __fmul_rn(__fmul_rn(dt, s), float(1.0 / 6.0));
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) w[c] = __dadd_rn(w[c], double(D[c]));
}

// The index-space foot of the characteristic through voxel ijk.
__device__ __forceinline__ void trace(const VolMap& m, const VolVelocity& v, int order, float dt, int x, int y,
                                      int z, double q[3]) {
    double w[3] = {to_world(m, double(x), 0), to_world(m, double(y), 1), to_world(m, double(z), 2)};
    runge_kutta(v, order, dt, w);
#pragma unroll
    for (int a = 0; a < 3; ++a) q[a] = to_index(m, w[a], a);
}

// Rank of bit t of word w and the voxel offset: the output leaf's
// active voxels visited as thread t owning bit t of every word.
struct LeafWalk {
    uint64_t m[8];
    int pre[8];
};

__device__ __forceinline__ void leaf_walk(const VolOut& o, int64_t l, LeafWalk& lw) {
    const size_t s = size_t(o.slot[l]);
    int c = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
        lw.m[w] = o.amask[s * 8 + w];
        lw.pre[w] = c;
        c += __popcll(lw.m[w]);
    }
}

// Advect::rk (tools/VolumeAdvect.h:492-507).
__global__ void __launch_bounds__(VOL_THREADS) vol_rk_kernel(const VolRkArgs a) {
    const int64_t l = blockIdx.x;
    if (l >= a.out.nleaf) return;
    const int t = threadIdx.x;
    LeafWalk lw;
    leaf_walk(a.out, l, lw);
    int ox, oy, oz;
    key_origin(a.out.keys[l], ox, oy, oz);
    const size_t s = size_t(a.out.slot[l]);
    for (int w = 0; w < 8; ++w) {
        if (!((lw.m[w] >> t) & 1)) continue;
        const int v = (w << 6) | t;
        double q[3];
        trace(a.map, a.vel, a.order, a.dt, ox + (v >> 6), oy + ((v >> 3) & 7), oz + (v & 7), q);
        int i0[3];
        double uvw[3];
        float r = a.src.background;
        if (floor_coord(q, i0, uvw)) {
            float d[2][2][2];
            box_values(a.src, i0, d);
            r = box_trilinear(d, uvw);
        }
        a.dst[s * LEAF_VOX + lw.pre[w] + __popcll(lw.m[w] & ((uint64_t(1) << t) - 1))] = r;
    }
}

// Advect::mac and Advect::bfecc (tools/VolumeAdvect.h:432-490).
__global__ void __launch_bounds__(VOL_THREADS) vol_combine_kernel(const VolCombineArgs a) {
    const int64_t l = blockIdx.x;
    if (l >= a.out.nleaf) return;
    const int t = threadIdx.x;
    LeafWalk lw;
    leaf_walk(a.out, l, lw);
    int ox, oy, oz;
    key_origin(a.out.keys[l], ox, oy, oz);
    const size_t s = size_t(a.out.slot[l]);
    for (int w = 0; w < 8; ++w) {
        if (!((lw.m[w] >> t) & 1)) continue;
        const int v = (w << 6) | t;
        const size_t i = s * LEAF_VOX + lw.pre[w] + __popcll(lw.m[w] & ((uint64_t(1) << t) - 1));
        const float in0 = vol_value(a.in, ox + (v >> 6), oy + ((v >> 3) & 7), oz + (v & 7));
        if (a.op == VOL_COMBINE_MAC)
            a.out0[i] = __fadd_rn(a.out0[i], __fmul_rn(0.5f, __fsub_rn(in0, a.out1[i])));
        else
            a.out0[i] = __fmul_rn(0.5f, __fsub_rn(__fmul_rn(3.0f, in0), a.out1[i]));
    }
}

// Advect::limiter (tools/VolumeAdvect.h:508-560): the flux limiter of the
// second-order schemes, then voxels within Delta<float> of the background
// take the background and turn inactive.  keep receives the active voxels
// that stay active.
__global__ void __launch_bounds__(VOL_THREADS) vol_limit_kernel(const VolLimitArgs a) {
    const int64_t l = blockIdx.x;
    if (l >= a.out.nleaf) return;
    const int t = threadIdx.x;
    LeafWalk lw;
    leaf_walk(a.out, l, lw);
    int ox, oy, oz;
    key_origin(a.out.keys[l], ox, oy, oz);
    const size_t s = size_t(a.out.slot[l]);
    __shared__ uint32_t kept[8][2];
    for (int w = 0; w < 8; ++w) {
        bool on = (lw.m[w] >> t) & 1;
        if (on) {
            const int v = (w << 6) | t;
            const size_t i = s * LEAF_VOX + lw.pre[w] + __popcll(lw.m[w] & ((uint64_t(1) << t) - 1));
            float value = a.vals[i];
            if (a.do_limit) {
                double q[3];
                trace(a.map, a.vel, 1, a.dt, ox + (v >> 6), oy + ((v >> 3) & 7), oz + (v & 7), q);
                int i0[3];
                double uvw[3];
                float d[2][2][2];
                if (floor_coord(q, i0, uvw)) {
                    box_values(a.in, i0, d);
                } else {
                    for (int x = 0; x < 8; ++x) (&d[0][0][0])[x] = a.in.background;
                }
                // BoxSampler::extrema (tools/Interpolation.h:690-710), its visiting order
                float vmin = d[0][0][0], vmax = d[0][0][0];
                const float order8[7] = {d[0][0][1], d[0][1][0], d[0][1][1], d[1][0][0],
                                         d[1][0][1], d[1][1][0], d[1][1][1]};
#pragma unroll
                for (int k = 0; k < 7; ++k) {
                    vmin = vmin < order8[k] ? vmin : order8[k];
                    vmax = vmax < order8[k] ? order8[k] : vmax;
                }
                if (a.limiter == 1) {
                    value = value > vmin ? (value < vmax ? value : vmax) : vmin;  // math::Clamp
                } else if (value < vmin || value > vmax) {
                    value = box_trilinear(d, uvw);
                }
            }
            // math::isApproxEqual(value, background, Delta<float>::value())
            if (!(fabsf(__fsub_rn(value, a.background)) > 1e-5f)) {
                value = a.background;
                on = false;
            }
            a.vals[i] = value;
        }
        const uint32_t b = __ballot_sync(0xffffffffu, on);
        if ((t & 31) == 0) kept[w][t >> 5] = b;
    }
    __syncthreads();
    if (t < 8) a.keep[s * 8 + t] = uint64_t(kept[t][0]) | (uint64_t(kept[t][1]) << 32);
}

// max over a dense Vec3f box of Vec3f::length() (float squares and sums,
// the square root in double, rounded to float), as math::Extrema sees the
// velocity grid's values (tools/Statistics.h:225-227).
__global__ void vol_max_speed_kernel(const float* v, int64_t n, unsigned int* max_bits) {
    float m = 0.0f;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const float x = v[3 * i], y = v[3 * i + 1], z = v[3 * i + 2];
        const float s = __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
        m = fmaxf(m, __double2float_rn(__dsqrt_rn(double(s))));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(max_bits, __float_as_uint(m));
}

}  // namespace

void launch_vol_max_speed(const float* dense, int64_t n, unsigned int* max_bits, cudaStream_t s) {
    if (n > 0) vol_max_speed_kernel<<<256, 256, 0, s>>>(dense, n, max_bits);
}

void launch_vol_rk(const VolRkArgs& a, cudaStream_t s) {
    if (a.out.nleaf > 0) vol_rk_kernel<<<unsigned(a.out.nleaf), VOL_THREADS, 0, s>>>(a);
}
void launch_vol_combine(const VolCombineArgs& a, cudaStream_t s) {
    if (a.out.nleaf > 0) vol_combine_kernel<<<unsigned(a.out.nleaf), VOL_THREADS, 0, s>>>(a);
}
void launch_vol_limit(const VolLimitArgs& a, cudaStream_t s) {
    if (a.out.nleaf > 0) vol_limit_kernel<<<unsigned(a.out.nleaf), VOL_THREADS, 0, s>>>(a);
}

}  // namespace gbls
