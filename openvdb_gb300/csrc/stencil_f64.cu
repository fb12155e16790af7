// FP64 instance of the advection hot path: the FloatGrid scheme of
// LevelSetAdvection / LevelSetTracker with the level set's values and every
// value operation in double -- WENO5 (the reference formula with ValueType
// double), the RK stages, the Eikonal update and the trim thresholds -- while
// the scheme's constants keep their FloatGrid values (the band width, the RK
// weight 1/3 and the normaliser's time-step factor as floats, widened) and
// the velocities stay Vec3f samples.  It is the precision oracle of the FP32
// run, not the reference's DoubleGrid instantiation (whose constants are
// double).  The value buffers of a handle in this mode hold 512 doubles per
// slot; masks, staging records, topology and the velocity evaluation are the
// FP32 path's.  Compiled without contraction: every double operation rounds
// once, as the host's do.
#include "stencil_f64.h"

#include "stencil_ops.cuh"

namespace gbls {
namespace {

// math::WENO5 (math/FiniteDifference.h:301-321) with ValueType double:
// every literal and sub-expression in double, eps = 1e-6 * double(0.01f).
__device__ double weno5_d(double v1, double v2, double v3, double v4, double v5) {
    const double C = 13.0 / 12.0;
    const double eps = 1.0e-6 * static_cast<double>(0.01f);
    const double t1 = __dadd_rn(__dsub_rn(v1, __dmul_rn(2.0, v2)), v3);
    const double u1 = __dadd_rn(__dsub_rn(v1, __dmul_rn(4.0, v2)), __dmul_rn(3.0, v3));
    const double d1 = __dadd_rn(__dadd_rn(__dmul_rn(C, __dmul_rn(t1, t1)), __dmul_rn(0.25, __dmul_rn(u1, u1))), eps);
    const double A1 = __ddiv_rn(0.1, __dmul_rn(d1, d1));
    const double t2 = __dadd_rn(__dsub_rn(v2, __dmul_rn(2.0, v3)), v4);
    const double u2 = __dsub_rn(v2, v4);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(C, __dmul_rn(t2, t2)), __dmul_rn(0.25, __dmul_rn(u2, u2))), eps);
    const double A2 = __ddiv_rn(0.6, __dmul_rn(d2, d2));
    const double t3 = __dadd_rn(__dsub_rn(v3, __dmul_rn(2.0, v4)), v5);
    const double u3 = __dadd_rn(__dsub_rn(__dmul_rn(3.0, v3), __dmul_rn(4.0, v4)), v5);
    const double d3 = __dadd_rn(__dadd_rn(__dmul_rn(C, __dmul_rn(t3, t3)), __dmul_rn(0.25, __dmul_rn(u3, u3))), eps);
    const double A3 = __ddiv_rn(0.3, __dmul_rn(d3, d3));
    const double p1 = __dadd_rn(__dsub_rn(__dmul_rn(2.0, v1), __dmul_rn(7.0, v2)), __dmul_rn(11.0, v3));
    const double p2 = __dadd_rn(__dsub_rn(__dmul_rn(5.0, v3), v2), __dmul_rn(2.0, v4));
    const double p3 = __dsub_rn(__dadd_rn(__dmul_rn(2.0, v3), __dmul_rn(5.0, v4)), v5);
    const double num = __dadd_rn(__dadd_rn(__dmul_rn(A1, p1), __dmul_rn(A2, p2)), __dmul_rn(A3, p3));
    const double den = __dmul_rn(6.0, __dadd_rn(__dadd_rn(A1, A2), A3));
    return __ddiv_rn(num, den);
}

// The seven values S(-3..3) along one axis of the tile.
struct Line7d {
    double v[7];
};
__device__ __forceinline__ Line7d tile_line_d(const double* tile, int x, int y, int z, int axis) {
    Line7d L;
    const int stride = axis == 0 ? TILE_DIM * TILE_DIM : axis == 1 ? TILE_DIM : 1;
    const int c = tile_index(x, y, z);
#pragma unroll
    for (int k = 0; k < 7; ++k) L.v[k] = tile[c + (k - 3) * stride];
    return L;
}
// D1<FD_HJWENO5>: WENO5(S3-S2, S2-S1, S1-S0, S0-S-1, S-1-S-2)
__device__ __forceinline__ double hj_fd_d(const Line7d& L) {
    const double* s = L.v + 3;
    return weno5_d(__dsub_rn(s[3], s[2]), __dsub_rn(s[2], s[1]), __dsub_rn(s[1], s[0]), __dsub_rn(s[0], s[-1]),
                   __dsub_rn(s[-1], s[-2]));
}
// D1<BD_HJWENO5> = -FD on the mirrored stencil: -WENO5(S-3-S-2, ..., S1-S2)
__device__ __forceinline__ double hj_bd_d(const Line7d& L) {
    const double* s = L.v + 3;
    return -weno5_d(__dsub_rn(s[-3], s[-2]), __dsub_rn(s[-2], s[-1]), __dsub_rn(s[-1], s[0]), __dsub_rn(s[0], s[1]),
                    __dsub_rn(s[1], s[2]));
}

// Value of bit bb of a half-word record: the packed double, else
// +-gamma by the sign bit.
__device__ __forceinline__ double record_load_d(const uint4 q, int bb, const double* vb, double gamma) {
    const double inactive = ((q.y >> bb) & 1) ? -gamma : gamma;
    if ((q.x >> bb) & 1) return vb[q.w + q.z + uint32_t(__popc(q.x & ((1u << bb) - 1u)))];
    return inactive;
}

// load_tile for double values (the same records and voxel assignment).
__device__ inline void load_tile_d(double* tile, const LeafStage& st, double gamma) {
    const int t = threadIdx.x;
    const int a = t >> 3, c = t & 7, h = t >> 5, bt = t & 31;
    const double* vb = reinterpret_cast<const double*>(st.vb);
#pragma unroll
    for (int k = 0; k < 8; ++k) tile[tile_index(k, a, c)] = record_load_d(st.rec[0][2 * k + h], bt, vb, gamma);
    const uint4 qmy = st.rec[3][2 * a + 1], qpy = st.rec[4][2 * a];
    const uint4 qmz = st.rec[5][2 * a + (c >> 2)], qpz = st.rec[6][2 * a + (c >> 2)];
    const int zb = (c & 3) << 3;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        tile[tile_index(-3 + d, a, c)] = record_load_d(st.rec[1][2 * (5 + d) + h], bt, vb, gamma);
        tile[tile_index(8 + d, a, c)] = record_load_d(st.rec[2][2 * d + h], bt, vb, gamma);
        tile[tile_index(a, -3 + d, c)] = record_load_d(qmy, ((5 + d) << 3 | c) & 31, vb, gamma);
        tile[tile_index(a, 8 + d, c)] = record_load_d(qpy, (d << 3) | c, vb, gamma);
        tile[tile_index(a, c, -3 + d)] = record_load_d(qmz, zb | (5 + d), vb, gamma);
        tile[tile_index(a, c, 8 + d)] = record_load_d(qpz, zb | d, vb, gamma);
    }
}

// One TVD-RK stage (tools/LevelSetAdvect.h:543-572) with ValueType double:
//   a = phi_c - dt * ((v0 g0 + v1 g1) + v2 g2),  g = Vec3d(HJWENO5) * (1/dx)
//   out = N ? alpha*phin + (1 - alpha)*a : a
// dt is the double substep length (a.dt64); alpha the float constant of the
// stage, widened.
__global__ void __launch_bounds__(STENCIL_THREADS) rk_stage_f64_kernel(const RkArgs a) {
    __shared__ double tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ uint16_t list[LEAF_VOX];
    __shared__ FieldParams sf;
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    if (threadIdx.x == 0) sf = a.field;
    stage_masks(st, a.src, s, a.nbr + 6 * l, nullptr, nullptr);
    load_tile_d(tile, st, double(a.gamma));
    const int n = build_list(list, st.am[0]);
    __syncthreads();
    int ox, oy, oz;
    key_origin(a.keys[l], ox, oy, oz);
    const double* phin = reinterpret_cast<const double*>(a.phin);
    double* out = reinterpret_cast<double*>(a.out);
    const double dt = a.dt64, alpha = double(a.alpha), beta = __dsub_rn(1.0, alpha);
    for (int i = threadIdx.x; i < n; i += STENCIL_THREADS) {
        const int v = list[i];
        const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
        float vel[3];
        eval_field(sf, ox + x, oy + y, oz + z, a.t0, vel);
        if (a.backward) { vel[0] = -vel[0]; vel[1] = -vel[1]; vel[2] = -vel[2]; }
        double g[3];
#pragma unroll 1
        for (int ax = 0; ax < 3; ++ax) {
            const Line7d L = tile_line_d(tile, x, y, z, ax);
            const float va = ax == 0 ? vel[0] : ax == 1 ? vel[1] : vel[2];
            g[ax] = __dmul_rn(va < 0.0f ? hj_fd_d(L) : hj_bd_d(L), a.invdx);
        }
        const double dot = __dadd_rn(__dadd_rn(__dmul_rn(double(vel[0]), g[0]), __dmul_rn(double(vel[1]), g[1])),
                                     __dmul_rn(double(vel[2]), g[2]));
        const double r = __dsub_rn(tile[tile_index(x, y, z)], __dmul_rn(dt, dot));
        double o = r;
        if (a.has_phi) o = __dadd_rn(__dmul_rn(alpha, phin[size_t(s) * LEAF_VOX + i]), __dmul_rn(beta, r));
        out[size_t(s) * LEAF_VOX + i] = o;
    }
}

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }  // std::min

// One stage of Normalizer::euler (tools/LevelSetTracker.h:623-676) with
// ValueType double over the voxels of pmask (plus the carried active ones),
// optionally followed by Trim; output in the layout of the surviving
// active set.  The structure of normalize_kernel in double arithmetic:
// GodunovsNormSqrd of the six HJ-WENO5
// derivatives, v = phi0 / (sqrt(phi0^2 + G) + double(1e-8f)),
// phi0 - mDt * v * (sqrt(G) * invDx - 1).
__global__ void __launch_bounds__(STENCIL_THREADS) normalize_f64_kernel(const NormArgs a) {
    __shared__ double tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ double res[LEAF_VOX];
    __shared__ uint16_t list[LEAF_VOX];
    __shared__ uint8_t flag[LEAF_VOX];  // bit 0: active after the pass, bit 1: negative
    __shared__ uint64_t pm[8], um[8], fin[8], fsg[8], phm[8];
    __shared__ uint32_t half[2][2][8];
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    const int t = threadIdx.x;
    stage_masks(st, a.src, s, a.nbr + 6 * l, a.pmask, pm);
    if (t < 8) {
        um[t] = pm[t] | st.am[0][t];
        fin[t] = 0;
        fsg[t] = st.sm[0][t] & ~um[t];
        if (a.has_phi) phm[t] = a.phi.amask[size_t(s) * 8 + t];
    }
    const double g = double(a.gamma);
    load_tile_d(tile, st, g);
    __syncthreads();
    const int n = build_list(list, um);
    __syncthreads();
    const double mdt = a.mdt64, invdx = a.invdx64, alpha = double(a.alpha), beta = __dsub_rn(1.0, alpha);
    const double* phiv = reinterpret_cast<const double*>(a.phi.vals);
    for (int i = t; i < n; i += STENCIL_THREADS) {
        const int v = list[i];
        const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
        const double phi0 = tile[tile_index(x, y, z)];
        double val = phi0;
        const uint64_t bit = uint64_t(1) << (v & 63);
        if (!(pm[v >> 6] & bit)) {  // active voxel outside the processed set
            res[v] = val;
            flag[v] = uint8_t((a.carry ? 1 : 0) | (val < 0.0 ? 2 : 0));
            continue;
        }
        if (!a.copy_only) {
            double up[3], dn[3];
#pragma unroll 1
            for (int ax = 0; ax < 3; ++ax) {
                const Line7d L = tile_line_d(tile, x, y, z, ax);
                up[ax] = hj_fd_d(L);
                dn[ax] = hj_bd_d(L);
            }
            // GodunovsNormSqrd(phi0 > 0, down, up) (math/FiniteDifference.h:324-357)
            double nsq = 0.0;
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                double term;
                if (phi0 > 0.0) {
                    const double m = dmax(dn[ax], 0.0), p = dmin(up[ax], 0.0);
                    term = dmax(__dmul_rn(m, m), __dmul_rn(p, p));
                } else {
                    const double m = dmin(dn[ax], 0.0), p = dmax(up[ax], 0.0);
                    term = dmax(__dmul_rn(m, m), __dmul_rn(p, p));
                }
                nsq = ax == 0 ? term : __dadd_rn(nsq, term);
            }
            double w = __ddiv_rn(phi0, __dadd_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(phi0, phi0), nsq)), double(1e-8f)));
            w = __dsub_rn(phi0, __dmul_rn(__dmul_rn(mdt, w), __dsub_rn(__dmul_rn(__dsqrt_rn(nsq), invdx), 1.0)));
            if (a.has_phi) {
                const int wd = v >> 6, b = v & 63;
                double p;
                if ((phm[wd] >> b) & 1) {
                    int rank = __popcll(phm[wd] & (bit - 1));
                    for (int k = 0; k < wd; ++k) rank += __popcll(phm[k]);
                    p = phiv[size_t(s) * LEAF_VOX + rank];
                } else {
                    p = ((a.phi.smask[size_t(s) * 8 + wd] >> b) & 1) ? -g : g;
                }
                w = __dadd_rn(__dmul_rn(alpha, p), __dmul_rn(beta, w));
            }
            val = w;
        }
        bool act = true, neg = val < 0.0;
        if ((a.trim & 1) && val <= -g) { act = false; neg = true; }
        else if ((a.trim & 2) && val >= g) { act = false; neg = false; }
        res[v] = val;
        flag[v] = uint8_t((act ? 1 : 0) | (neg ? 2 : 0));
    }
    __syncthreads();
    {
        const int w = t >> 5, lane = t & 31;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int v = (k << 6) | t;
            const bool vis = (um[k] >> t) & 1;
            const uint8_t f = vis ? flag[v] : uint8_t(0);
            const uint32_t ba = __ballot_sync(0xffffffffu, f & 1);
            const uint32_t bn = __ballot_sync(0xffffffffu, (f >> 1) & 1);
            if (lane == 0) {
                half[0][w][k] = ba;
                half[1][w][k] = bn;
            }
        }
    }
    __syncthreads();
    if (t < 8) {
        fin[t] = uint64_t(half[0][0][t]) | (uint64_t(half[0][1][t]) << 32);
        fsg[t] |= uint64_t(half[1][0][t]) | (uint64_t(half[1][1][t]) << 32);
    }
    __syncthreads();
    double* out = reinterpret_cast<double*>(a.out_vals);
    const uint64_t low = (uint64_t(1) << t) - 1;
    int base = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint64_t w = fin[k];
        if ((w >> t) & 1) out[size_t(s) * LEAF_VOX + base + __popcll(w & low)] = res[(k << 6) | t];
        base += __popcll(w);
    }
    if (t < 8) {
        a.out_amask[size_t(s) * 8 + t] = fin[t];
        a.out_smask[size_t(s) * 8 + t] = fsg[t];
    }
    if (t == 0) {
        if (a.out_count) a.out_count[l] = base;
        if (a.acc) {
            int np = 0;
            for (int w = 0; w < 8; ++w) np += __popcll(pm[w]);
            atomicAdd(a.acc, (unsigned long long)np);
            atomicAdd(a.acc + 1, (unsigned long long)base);
        }
    }
}

__global__ void k_widen(const float* in, double* out, size_t n) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        out[i] = double(in[i]);
}
__global__ void k_narrow(const double* in, float* out, size_t n) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        out[i] = __double2float_rn(in[i]);
}

// The first active voxel (leaf order, then voxel order) whose Vec3f |v|^2
// equals the float maximum: key leaf * 512 + voxel, minimised.
__global__ void __launch_bounds__(64) k_argmax_f64(int64_t nleaf, const uint64_t* keys, const int32_t* slot,
                                                  const uint64_t* am, FieldParams f, float t0, float maxv2,
                                                  unsigned long long* argkey) {
    const int64_t l = blockIdx.x;
    if (l >= nleaf) return;
    int ox, oy, oz;
    key_origin(keys[l], ox, oy, oz);
    const int s = slot[l];
    for (int v = threadIdx.x; v < LEAF_VOX; v += blockDim.x) {
        if (!((am[size_t(s) * 8 + (v >> 6)] >> (v & 63)) & 1)) continue;
        float vel[3];
        eval_field(f, ox + (v >> 6), oy + ((v >> 3) & 7), oz + (v & 7), t0, vel);
        const float m = __fadd_rn(__fadd_rn(__fmul_rn(vel[0], vel[0]), __fmul_rn(vel[1], vel[1])),
                                  __fmul_rn(vel[2], vel[2]));
        if (m == maxv2) atomicMin(argkey, (unsigned long long)(l * LEAF_VOX + v));
    }
}
// |v|^2 of that voxel in double: (x*x + y*y) + z*z of the widened components.
__global__ void k_argmax_f64_value(const uint64_t* keys, FieldParams f, float t0, const unsigned long long* argkey,
                                   double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const unsigned long long k = *argkey;
    if (k == ~0ull) { *out = -1.0; return; }
    const int64_t l = int64_t(k / LEAF_VOX);
    const int v = int(k % LEAF_VOX);
    int ox, oy, oz;
    key_origin(keys[l], ox, oy, oz);
    float vel[3];
    eval_field(f, ox + (v >> 6), oy + ((v >> 3) & 7), oz + (v & 7), t0, vel);
    const double x = vel[0], y = vel[1], z = vel[2];
    *out = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

// Active values of leaves [0, n) in tree order into out[prefix[l] + rank].
__global__ void __launch_bounds__(64) k_gather_active_f64(int64_t n, const int32_t* slot, const uint64_t* am,
                                                         const int64_t* prefix, const double* vals, double* out) {
    const int64_t l = blockIdx.x;
    if (l >= n) return;
    const size_t s = size_t(slot[l]);
    int cnt = 0;
    for (int w = 0; w < 8; ++w) cnt += __popcll(am[s * 8 + w]);
    for (int r = threadIdx.x; r < cnt; r += blockDim.x) out[prefix[l] + r] = vals[s * LEAF_VOX + r];
}

}  // namespace

void launch_rk_f64(const RkArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    rk_stage_f64_kernel<<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

void launch_norm_f64(const NormArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    normalize_f64_kernel<<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

void launch_widen(const float* in, double* out, size_t n, cudaStream_t s) {
    if (n) k_widen<<<unsigned(std::min<size_t>((n + 255) / 256, 4096)), 256, 0, s>>>(in, out, n);
}
void launch_narrow(const double* in, float* out, size_t n, cudaStream_t s) {
    if (n) k_narrow<<<unsigned(std::min<size_t>((n + 255) / 256, 4096)), 256, 0, s>>>(in, out, n);
}

void launch_argmax_f64(int64_t nleaf, const uint64_t* keys, const int32_t* slot, const uint64_t* am,
                       const FieldParams& f, float t0, float maxv2, unsigned long long* argkey, double* out,
                       cudaStream_t s) {
    cudaMemsetAsync(argkey, 0xff, sizeof(unsigned long long), s);
    if (nleaf > 0) k_argmax_f64<<<unsigned(nleaf), 64, 0, s>>>(nleaf, keys, slot, am, f, t0, maxv2, argkey);
    k_argmax_f64_value<<<1, 32, 0, s>>>(keys, f, t0, argkey, out);
}

void launch_gather_active_f64(int64_t n, const int32_t* slot, const uint64_t* am, const int64_t* prefix,
                              const double* vals, double* out, cudaStream_t s) {
    if (n > 0) k_gather_active_f64<<<unsigned(n), 64, 0, s>>>(n, slot, am, prefix, vals, out);
}

}  // namespace gbls
