// PARITY-mode stencil kernels on voxel pairs with packed FP32x2 arithmetic.
//
// The same results as rk_stage_kernel<ParityArith> / normalize_kernel<
// ParityArith>, bit for bit: every float operation of the reference is one
// correctly rounded packed operation (add/sub/mul.rn.f32x2 in PTX, which
// ptxas never fuses into a multiply-add), and each HJ-WENO5 evaluates the
// double-typed weights of the reference as double words (weno_exact.h) for
// two voxels at once; a lane whose rounding that cannot decide takes the
// FP64 formula.  Staging (masks, 14^3 tile, voxel list) is the scalar
// kernels'.
#pragma once

#include "stencil_ops.cuh"

namespace gbls {

namespace xp {
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
using xw::add;
using xw::mul;
using xw::sub;

// ParityArith::weno5 on two lanes.
__device__ __forceinline__ float2 weno5(float2 v1, float2 v2, float2 v3, float2 v4, float2 v5) {
    float2 r;
    const unsigned ok = xw::weno5<float2>(v1, v2, v3, v4, v5, r);
    if (ok != 3u) {
        if (!(ok & 1u)) r.x = weno5_fp64(v1.x, v2.x, v3.x, v4.x, v5.x);
        if (!(ok & 2u)) r.y = weno5_fp64(v1.y, v2.y, v3.y, v4.y, v5.y);
    }
    return r;
}

// The six differences D_k = S(k-2) - S(k-3) of the lines through two voxels.
__device__ __forceinline__ void line_diffs(const float* tile, int c0, int c1, int stride, float2 D[6]) {
    float2 v[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) v[k] = make_float2(tile[c0 + (k - 3) * stride], tile[c1 + (k - 3) * stride]);
#pragma unroll
    for (int k = 0; k < 6; ++k) D[k] = sub(v[k + 1], v[k]);
}

// ParityArith::ijt on two lanes: identity for dx = 1.
__device__ __forceinline__ float2 ijt(float2 g, bool unit, double invdx) {
    if (unit) return g;
    return make_float2(ParityArith::ijt(g.x, invdx, 0.0f), ParityArith::ijt(g.y, invdx, 0.0f));
}

// std::max / std::min per lane
__device__ __forceinline__ float2 vmax(float2 a, float2 b) { return make_float2(ref_max(a.x, b.x), ref_max(a.y, b.y)); }
__device__ __forceinline__ float2 vmin(float2 a, float2 b) { return make_float2(ref_min(a.x, b.x), ref_min(a.y, b.y)); }
}  // namespace xp

// The RK stage of rk_stage_kernel<ParityArith> on voxel pairs (HJWENO5).
__global__ void __launch_bounds__(STENCIL_THREADS, 8) rk_stage_kernel_exact2(const __grid_constant__ RkArgs a) {
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
    // deformation field: the leaf's 8 sines per axis and function, staged once
    const bool tabbed = sf.kind == 2 && sf.tab && ox - sf.tab_lo >= 0 && oy - sf.tab_lo >= 0 &&
                        oz - sf.tab_lo >= 0 && ox + 8 - sf.tab_lo <= sf.tab_n &&
                        oy + 8 - sf.tab_lo <= sf.tab_n && oz + 8 - sf.tab_lo <= sf.tab_n;
    if (tabbed && threadIdx.x < 48) {
        const int ax = threadIdx.x >> 4, fn = (threadIdx.x >> 3) & 1, q = threadIdx.x & 7;
        const int o = ax == 0 ? ox : ax == 1 ? oy : oz;
        vtab[ax * 2 + fn][q] = sf.tab[2 * (o + q - sf.tab_lo) + fn];
    }
    stage_masks(st, a.src, s, a.nbr + 6 * l, nullptr, nullptr);
    load_tile(tile, st, a.gamma);
    __syncthreads();  // the staging records are dead: the voxel list reuses their storage
    uint16_t* list = reinterpret_cast<uint16_t*>(&st.rec[0][0]);
    const int n = build_list(list, st.am[0]);
    __syncthreads();
    const int npairs = (n + 1) >> 1;
    const bool unit = __double_as_longlong(a.invdx) == 0x3FF0000000000000ll;
    const float2 dt2 = xp::f2(dt);
    for (int p = threadIdx.x; p < npairs; p += STENCIL_THREADS) {
        const int i0 = 2 * p, i1 = min(2 * p + 1, n - 1);
        const int v0 = list[i0], v1 = list[i1];
        const int x0 = v0 >> 6, y0 = (v0 >> 3) & 7, z0 = v0 & 7;
        const int x1 = v1 >> 6, y1 = (v1 >> 3) & 7, z1 = v1 & 7;
        float2 ve[3];
        if (tabbed) {
            // gbls_deformation with the staged sines, the reference's order
            const float2 sx = make_float2(vtab[0][x0], vtab[0][x1]), s2x = make_float2(vtab[1][x0], vtab[1][x1]);
            const float2 sy = make_float2(vtab[2][y0], vtab[2][y1]), s2y = make_float2(vtab[3][y0], vtab[3][y1]);
            const float2 sz = make_float2(vtab[4][z0], vtab[4][z1]), s2z = make_float2(vtab[5][z0], vtab[5][z1]);
            const float2 amp = xp::f2(sf.amp);
            const float2 u = xp::mul(xp::mul(xp::mul(xp::mul(xp::f2(2.0f), sx), sx), s2y), s2z);
            const float2 w = xp::mul(xp::mul(xp::mul(s2x, sy), sy), s2z);
            const float2 q = xp::mul(xp::mul(xp::mul(s2x, s2y), sz), sz);
            ve[0] = xp::mul(u, amp);
            const float2 vw = xp::mul(w, amp), vq = xp::mul(q, amp);
            ve[1] = make_float2(-vw.x, -vw.y);
            ve[2] = make_float2(-vq.x, -vq.y);
        } else {
            float e0[3], e1[3];
            eval_field(sf, ox + x0, oy + y0, oz + z0, t0, e0);
            eval_field(sf, ox + x1, oy + y1, oz + z1, t0, e1);
            for (int k = 0; k < 3; ++k) ve[k] = make_float2(e0[k], e1[k]);
        }
        if (a.backward)
            for (int k = 0; k < 3; ++k) ve[k] = make_float2(-ve[k].x, -ve[k].y);
        const int c0 = tile_index(x0, y0, z0), c1 = tile_index(x1, y1, z1);
        float2 g[3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int stride = ax == 0 ? TILE_DIM * TILE_DIM : ax == 1 ? TILE_DIM : 1;
            float2 D[6];
            xp::line_diffs(tile, c0, c1, stride, D);
            float2 in[5];
            const bool f0 = ve[ax].x < 0.0f, f1 = ve[ax].y < 0.0f;
#pragma unroll
            for (int k = 0; k < 5; ++k)
                in[k] = make_float2(f0 ? D[5 - k].x : D[k].x, f1 ? D[5 - k].y : D[k].y);
            g[ax] = xp::ijt(xp::weno5(in[0], in[1], in[2], in[3], in[4]), unit, a.invdx);
        }
        const float2 dot = xp::add(xp::add(xp::mul(ve[0], g[0]), xp::mul(ve[1], g[1])), xp::mul(ve[2], g[2]));
        const float2 c = make_float2(tile[c0], tile[c1]);
        float2 r = xp::sub(c, xp::mul(dt2, dot));
        if (a.has_phi) {
            const float2 ph = make_float2(a.phin[size_t(s) * LEAF_VOX + i0], a.phin[size_t(s) * LEAF_VOX + i1]);
            r = xp::add(xp::mul(xp::f2(a.alpha), ph), xp::mul(xp::f2(a.beta), r));
        }
        a.out[size_t(s) * LEAF_VOX + i0] = r.x;
        if (i1 != i0) a.out[size_t(s) * LEAF_VOX + i1] = r.y;
    }
}

// The renormalisation stage of normalize_kernel<ParityArith> (RK1 form,
// has_phi == 0, copy_only == 0) on voxel pairs, with trimming.
__global__ void __launch_bounds__(STENCIL_THREADS, 8) normalize_kernel_exact2(const __grid_constant__ NormArgs a) {
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
        const bool out0 = phi0.x > 0.0f, out1 = phi0.y > 0.0f;
        float2 nsq = xp::f2(0.0f);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int stride = ax == 0 ? TILE_DIM * TILE_DIM : ax == 1 ? TILE_DIM : 1;
            float2 D[6];
            xp::line_diffs(tile, c0, c1, stride, D);
            const float2 up = xp::weno5(D[5], D[4], D[3], D[2], D[1]);   // FD
            const float2 dn = xp::weno5(D[0], D[1], D[2], D[3], D[4]);   // BD
            // GodunovsNormSqrd (math/FiniteDifference.h:324-357): outside
            // max((max(dm,0))^2, (min(dp,0))^2), inside max((min(dm,0))^2,
            // (max(dp,0))^2); terms summed in axis order
            const float2 z = xp::f2(0.0f);
            const float2 dmx = xp::vmax(dn, z), dmn = xp::vmin(dn, z), dpx = xp::vmax(up, z), dpn = xp::vmin(up, z);
            const float2 aa = make_float2(out0 ? dmx.x : dmn.x, out1 ? dmx.y : dmn.y);
            const float2 bb = make_float2(out0 ? dpn.x : dpx.x, out1 ? dpn.y : dpx.y);
            const float2 term = xp::vmax(xp::mul(aa, aa), xp::mul(bb, bb));
            nsq = ax == 0 ? term : xp::add(nsq, term);
        }
        // Normalizer::eval: phi0 - mDt * phi0/(sqrt(phi0^2 + G) + 1e-8) * (sqrt(G)/dx - 1)
        const float2 rr = xp::add(xp::mul(phi0, phi0), nsq);
        const float2 den = xp::add(make_float2(__fsqrt_rn(rr.x), __fsqrt_rn(rr.y)), xp::f2(1e-8f));
        const float2 vv = make_float2(__fdiv_rn(phi0.x, den.x), __fdiv_rn(phi0.y, den.y));
        const float2 sg = make_float2(__fsqrt_rn(nsq.x), __fsqrt_rn(nsq.y));
        const float2 fac = xp::sub(xp::mul(sg, xp::f2(a.invdx)), xp::f2(1.0f));
        const float2 val2 = xp::sub(phi0, xp::mul(xp::mul(xp::f2(a.mdt), vv), fac));
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            if (e == 1 && i1 == i0) break;
            const int v = e ? v1 : v0;
            const float ph = e ? phi0.y : phi0.x;
            // an active voxel outside the processed set keeps its value
            res[v] = ((pm[v >> 6] >> (v & 63)) & 1) ? (e ? val2.y : val2.x) : ph;
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
