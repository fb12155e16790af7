// FAST-mode stencil kernels on voxel pairs with packed FP32x2 arithmetic
// (Blackwell FFMA2 / FADD2 / FMUL2): each thread evaluates the HJ-WENO5
// derivatives of two active voxels at once, halving the floating-point
// instruction count of the issue-bound stencil loop.  Same formulas as
// FastArith; staging (masks, 14^3 tile, voxel list) is shared with the
// scalar kernels.
#pragma once

#include "stencil_ops.cuh"

namespace gbls {

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.0f), a); }
// FastArith::weno5 on two lanes.
__device__ __forceinline__ float2 weno5x2(float2 v1, float2 v2, float2 v3, float2 v4, float2 v5) {
    const float2 C = f2(13.0f / 12.0f), Q = f2(0.25f), eps = f2(1.0e-8f);
    const float2 t1 = fma2(f2(-2.0f), v2, add2(v1, v3));
    const float2 u1 = fma2(f2(3.0f), v3, fma2(f2(-4.0f), v2, v1));
    const float2 t2 = fma2(f2(-2.0f), v3, add2(v2, v4));
    const float2 u2 = sub2(v2, v4);
    const float2 t3 = fma2(f2(-2.0f), v4, add2(v3, v5));
    const float2 u3 = fma2(f2(3.0f), v3, fma2(f2(-4.0f), v4, v5));
    const float2 d1 = fma2(mul2(C, t1), t1, fma2(mul2(Q, u1), u1, eps));
    const float2 d2 = fma2(mul2(C, t2), t2, fma2(mul2(Q, u2), u2, eps));
    const float2 d3 = fma2(mul2(C, t3), t3, fma2(mul2(Q, u3), u3, eps));
    const float2 q1 = mul2(d1, d1), q2 = mul2(d2, d2), q3 = mul2(d3, d3);
    const float2 A1 = mul2(f2(0.1f), mul2(q2, q3));
    const float2 A2 = mul2(f2(0.6f), mul2(q1, q3));
    const float2 A3 = mul2(f2(0.3f), mul2(q1, q2));
    const float2 p1 = fma2(f2(11.0f), v3, fma2(f2(-7.0f), v2, mul2(f2(2.0f), v1)));
    const float2 p2 = fma2(f2(2.0f), v4, fma2(f2(5.0f), v3, mul2(f2(-1.0f), v2)));
    const float2 p3 = fma2(f2(-1.0f), v5, fma2(f2(5.0f), v4, mul2(f2(2.0f), v3)));
    const float2 num = fma2(A3, p3, fma2(A2, p2, mul2(A1, p1)));
    const float2 den = mul2(f2(6.0f), add2(add2(A1, A2), A3));
    return make_float2(__fdividef(num.x, den.x), __fdividef(num.y, den.y));
}

struct Diff6x2 {
    float2 d[6];
};

__device__ __forceinline__ Diff6x2 line_diffs2(const float* tile, int c0, int c1, int stride) {
    float2 v[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) v[k] = make_float2(tile[c0 + (k - 3) * stride], tile[c1 + (k - 3) * stride]);
    Diff6x2 D;
#pragma unroll
    for (int k = 0; k < 6; ++k) D.d[k] = sub2(v[k + 1], v[k]);
    return D;
}

__device__ __forceinline__ float2 fd2(const Diff6x2& D) { return weno5x2(D.d[5], D.d[4], D.d[3], D.d[2], D.d[1]); }
__device__ __forceinline__ float2 bd2(const Diff6x2& D) { return weno5x2(D.d[0], D.d[1], D.d[2], D.d[3], D.d[4]); }

// FAST RK stage on voxel pairs (the semantics of rk_stage_kernel<FastArith>).
// The field is read through a pointer (the launch parameter, or a batch
// instance's entry) instead of a shared copy.  For the deformation field the
// leaf's factors are staged once: u = Xu[x] Yu[y] Zu[z], v = Xv[x] Yv[y] Zu[z],
// w = Xv[x] Yu[y] Zw[z] with Xu = 2 amp sin^2(pi x), Xv = -amp sin(2 pi x),
// Yu = sin(2 pi y), Yv = sin^2(pi y), Zu = sin(2 pi z), Zw = sin^2(pi z)
// (amp negated for backward time), so a voxel pair costs six packed products.
// At most 64 registers per thread keep 16 CTAs resident per SM.
__global__ void __launch_bounds__(STENCIL_THREADS, 16) rk_stage_kernel_x2(const __grid_constant__ RkArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ float vtab[6][8];
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    const uint64_t key = a.keys[l];
    float dt = a.dt, t0 = a.t0;
    const FieldParams* fp = &a.field;
    if (a.inst_run) {
        const uint32_t inst = key_instance(key);
        if (!a.inst_run[inst]) {
            if (a.copy_done) {
                int n = 0;
                for (int w = 0; w < 8; ++w) n += __popcll(a.src.amask[size_t(s) * 8 + w]);
                for (int i = threadIdx.x; i < n; i += STENCIL_THREADS)
                    a.out[size_t(s) * LEAF_VOX + i] = a.src.vals[size_t(s) * LEAF_VOX + i];
            }
            return;
        }
        dt = a.inst_dt[inst];
        t0 = a.inst_t0[inst];
        fp = a.inst_field + inst;
    }
    const FieldParams& sf = *fp;
    int ox, oy, oz;
    key_origin(key, ox, oy, oz);
    const bool tabbed = sf.kind == 2 && sf.tab && ox - sf.tab_lo >= 0 && oy - sf.tab_lo >= 0 &&
                        oz - sf.tab_lo >= 0 && ox + 8 - sf.tab_lo <= sf.tab_n &&
                        oy + 8 - sf.tab_lo <= sf.tab_n && oz + 8 - sf.tab_lo <= sf.tab_n;
    if (tabbed && threadIdx.x >= 40) {
        const int ax = (threadIdx.x - 40) >> 3, q = threadIdx.x & 7;
        const int o = (ax == 0 ? ox : ax == 1 ? oy : oz) + q - sf.tab_lo;
        const float sn = sf.tab[2 * o], s2 = sf.tab[2 * o + 1];
        const float amp = a.backward ? -sf.amp : sf.amp;
        if (ax == 0) {
            vtab[0][q] = 2.0f * amp * sn * sn;
            vtab[1][q] = -amp * s2;
        } else {
            vtab[2 * ax][q] = s2;
            vtab[2 * ax + 1][q] = sn * sn;
        }
    }
    stage_masks(st, a.src, s, a.nbr + 6 * l, nullptr, nullptr);
    load_tile(tile, st, a.gamma);
    __syncthreads();  // the staging records are dead: the voxel list reuses their storage
    uint16_t* list = reinterpret_cast<uint16_t*>(&st.rec[0][0]);
    const int n = build_list(list, st.am[0]);
    __syncthreads();
    const int npairs = (n + 1) >> 1;
    const float2 dt2 = f2(dt), invdx2 = f2(a.invdx_f);
    for (int p = threadIdx.x; p < npairs; p += STENCIL_THREADS) {
        const int i0 = 2 * p, i1 = min(2 * p + 1, n - 1);
        const int v0 = list[i0], v1 = list[i1];
        const int x0 = v0 >> 6, y0 = (v0 >> 3) & 7, z0 = v0 & 7;
        const int x1 = v1 >> 6, y1 = (v1 >> 3) & 7, z1 = v1 & 7;
        float ve0[3], ve1[3];
        if (tabbed) {
            const float2 xu = make_float2(vtab[0][x0], vtab[0][x1]), xv = make_float2(vtab[1][x0], vtab[1][x1]);
            const float2 yu = make_float2(vtab[2][y0], vtab[2][y1]), yv = make_float2(vtab[3][y0], vtab[3][y1]);
            const float2 zu = make_float2(vtab[4][z0], vtab[4][z1]), zw = make_float2(vtab[5][z0], vtab[5][z1]);
            const float2 u = mul2(mul2(xu, yu), zu), v = mul2(mul2(xv, yv), zu), w = mul2(mul2(xv, yu), zw);
            ve0[0] = u.x; ve1[0] = u.y;
            ve0[1] = v.x; ve1[1] = v.y;
            ve0[2] = w.x; ve1[2] = w.y;
        } else if (sf.kind == 4) {  // GBLS_FIELD_HOST_SAMPLED: ranks i0, i1 of leaf l
            const float* q0 = sf.sampled + 3 * (sf.prefix[l] + i0);
            const float* q1 = sf.sampled + 3 * (sf.prefix[l] + i1);
            for (int k = 0; k < 3; ++k) { ve0[k] = q0[k]; ve1[k] = q1[k]; }
            if (a.backward) {
                for (int k = 0; k < 3; ++k) { ve0[k] = -ve0[k]; ve1[k] = -ve1[k]; }
            }
        } else {
            eval_field(sf, ox + x0, oy + y0, oz + z0, t0, ve0);
            eval_field(sf, ox + x1, oy + y1, oz + z1, t0, ve1);
            if (a.backward) {
                for (int k = 0; k < 3; ++k) { ve0[k] = -ve0[k]; ve1[k] = -ve1[k]; }
            }
        }
        const int c0 = tile_index(x0, y0, z0), c1 = tile_index(x1, y1, z1);
        float2 dot = f2(0.0f);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int stride = ax == 0 ? TILE_DIM * TILE_DIM : ax == 1 ? TILE_DIM : 1;
            const Diff6x2 D = line_diffs2(tile, c0, c1, stride);
            float2 in[5];
            const bool f0 = ve0[ax] < 0.0f, f1 = ve1[ax] < 0.0f;
#pragma unroll
            for (int k = 0; k < 5; ++k)
                in[k] = make_float2(f0 ? D.d[5 - k].x : D.d[k].x, f1 ? D.d[5 - k].y : D.d[k].y);
            const float2 g = mul2(weno5x2(in[0], in[1], in[2], in[3], in[4]), invdx2);
            dot = fma2(make_float2(ve0[ax], ve1[ax]), g, dot);
        }
        const float2 c = make_float2(tile[c0], tile[c1]);
        float2 r = fma2(dot, make_float2(-dt2.x, -dt2.y), c);
        if (a.has_phi) {
            const float2 ph = make_float2(a.phin[size_t(s) * LEAF_VOX + i0], a.phin[size_t(s) * LEAF_VOX + i1]);
            r = fma2(f2(a.alpha), ph, mul2(f2(a.beta), r));
        }
        a.out[size_t(s) * LEAF_VOX + i0] = r.x;
        if (i1 != i0) a.out[size_t(s) * LEAF_VOX + i1] = r.y;
    }
}

// FAST renormalisation stage (RK1 form, no convex combination) on voxel
// pairs, with trimming: same semantics as normalize_kernel<FastArith> for
// has_phi == 0 and copy_only == 0.
__global__ void __launch_bounds__(STENCIL_THREADS, 16) normalize_kernel_x2(const __grid_constant__ NormArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ float res[LEAF_VOX];
    __shared__ uint64_t pm[8], um[8], fin[8], fsg[8];
    __shared__ uint32_t half[2][2][8];
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    const int t = threadIdx.x;
    const bool run = !a.inst_run || a.inst_run[key_instance(a.keys[l])];
    const int carry = run ? a.carry : 1;
    const int trim = run ? a.trim : 0;
    stage_masks(st, a.src, s, a.nbr + 6 * l, a.pmask, pm);
    if (t < 8) {
        if (!run) pm[t] = 0;
        um[t] = pm[t] | st.am[0][t];
        fin[t] = 0;
        fsg[t] = st.sm[0][t] & ~um[t];
    }
    load_tile(tile, st, a.gamma);
    __syncthreads();  // the staging records are dead: the voxel list reuses their storage
    uint16_t* list = reinterpret_cast<uint16_t*>(&st.rec[0][0]);
    const int n = build_list(list, um);
    __syncthreads();
    const float g = a.gamma;
    const int npairs = (n + 1) >> 1;
    for (int p = t; p < npairs; p += STENCIL_THREADS) {
        const int i0 = 2 * p, i1 = min(2 * p + 1, n - 1);
        const int v0 = list[i0], v1 = list[i1];
        const int c0 = tile_index(v0 >> 6, (v0 >> 3) & 7, v0 & 7), c1 = tile_index(v1 >> 6, (v1 >> 3) & 7, v1 & 7);
        const float2 phi0 = make_float2(tile[c0], tile[c1]);
        float2 nsq = f2(0.0f);
        const bool out0 = phi0.x > 0.0f, out1 = phi0.y > 0.0f;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int stride = ax == 0 ? TILE_DIM * TILE_DIM : ax == 1 ? TILE_DIM : 1;
            const Diff6x2 D = line_diffs2(tile, c0, c1, stride);
            const float2 up = fd2(D), dn = bd2(D);
            // GodunovsNormSqrd: outside max((max(dm,0))^2, (min(dp,0))^2),
            // inside max((min(dm,0))^2, (max(dp,0))^2)
            const float2 aa = make_float2(out0 ? fmaxf(dn.x, 0.0f) : fminf(dn.x, 0.0f),
                                          out1 ? fmaxf(dn.y, 0.0f) : fminf(dn.y, 0.0f));
            const float2 bb = make_float2(out0 ? fminf(up.x, 0.0f) : fmaxf(up.x, 0.0f),
                                          out1 ? fminf(up.y, 0.0f) : fmaxf(up.y, 0.0f));
            const float2 a2 = mul2(aa, aa), b2 = mul2(bb, bb);
            nsq = add2(nsq, make_float2(fmaxf(a2.x, b2.x), fmaxf(a2.y, b2.y)));
        }
        const float2 rr = fma2(phi0, phi0, nsq);
        const float2 r = make_float2(sqrtf(rr.x), sqrtf(rr.y));
        const float2 vv = make_float2(__fdividef(phi0.x, r.x + 1e-8f), __fdividef(phi0.y, r.y + 1e-8f));
        const float2 sg = make_float2(sqrtf(nsq.x), sqrtf(nsq.y));
        const float2 fac = fma2(sg, f2(a.invdx), f2(-1.0f));
        const float2 val2 = sub2(phi0, mul2(mul2(f2(a.mdt), vv), fac));
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            if (e == 1 && i1 == i0) break;
            const int v = e ? v1 : v0;
            const float ph = e ? phi0.y : phi0.x;
            float val = e ? val2.y : val2.x;
            // an active voxel outside the processed set keeps its value
            res[v] = ((pm[v >> 6] >> (v & 63)) & 1) ? val : ph;
        }
    }
    __syncthreads();
    {
        const int w = t >> 5, lane = t & 31;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int v = (k << 6) | t;
            const bool vis = (um[k] >> t) & 1;
            // the voxel's state after the pass from its result: processed
            // voxels are trimmed by the TrimMode bits, the others stay active
            // when `carry` is set
            uint8_t f = 0;
            if (vis) {
                const float val = res[v];
                bool act = true, neg = val < 0.0f;
                if ((pm[k] >> t) & 1) {
                    if ((trim & 1) && val <= -g) { act = false; neg = true; }
                    else if ((trim & 2) && val >= g) { act = false; neg = false; }
                } else {
                    act = carry != 0;
                }
                f = uint8_t((act ? 1 : 0) | (neg ? 2 : 0));
            }
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
    const uint64_t low = (uint64_t(1) << t) - 1;
    int base = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint64_t w = fin[k];
        if ((w >> t) & 1) a.out_vals[size_t(s) * LEAF_VOX + base + __popcll(w & low)] = res[(k << 6) | t];
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

}  // namespace gbls
