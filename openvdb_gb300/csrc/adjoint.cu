// Adjoint kernels: transposed Jacobians of the recorded RK3-HJWENO5 stages
// (tools/LevelSetAdvect.h:543-572) and of the Godunov renormalisation
// (tools/LevelSetTracker.h:623-643), in FP32, with the branch structure of
// the forward pass (upwind direction from the velocity sign, Godunov term
// selection, trimming, topology) held fixed.
#include "adjoint.h"
#include "stencil_ops.cuh"

namespace gbls {

namespace {

// Gradient of Shu's WENO5 by reverse-mode differentiation, arranged so that
// FP32 keeps it accurate to a few ulps where the data are smooth.  Three
// things lose it otherwise: the smoothness indicators d_k are third
// differences of the level set, which differences of first differences D_k
// cancel to 1e-3 of |D| on a radius-40 sphere; the weight adjoints
// (p_k - 6W)/(6S) cancel p_k against the weighted mean; and unnormalised
// weights (gamma_k / d_k^2 products) overflow on flat lines.  So the caller
// passes E_a = v_{a+1} - v_a (second differences of the line, from
// error-free first differences), every indicator and every p_k - p_j is a
// short combination of them, and with the normalised weights w_k the
// adjoints are
//   dW/dp_k = w_k / 6,
//   dW/dd_k = 2 (sum_{j != k} w_j B_j) / d_k,  B_j = sum_i w_i (p_j - p_i) / 6.
// v1..v5: the operands (for the linear part p_k); E[0..3] = E_1..E_4.
__device__ __forceinline__ float weno5_grad(float v1, float v2, float v3, float v4, float v5, const float E[4],
                                            float g[5]) {
    const float C = 13.0f / 12.0f, eps = 1.0e-8f;
    const float E1 = E[0], E2 = E[1], E3 = E[2], E4 = E[3];
    const float t1 = E2 - E1, u1 = 3.0f * E2 - E1;
    const float t2 = E3 - E2, u2 = -(E2 + E3);
    const float t3 = E4 - E3, u3 = E4 - 3.0f * E3;
    const float p12 = -2.0f * E1 + 4.0f * E2 - 2.0f * E3;
    const float p13 = -2.0f * E1 + 5.0f * E2 - 4.0f * E3 + E4;
    const float p23 = E2 - 2.0f * E3 + E4;
    const float d1 = C * t1 * t1 + 0.25f * u1 * u1 + eps;
    const float d2 = C * t2 * t2 + 0.25f * u2 * u2 + eps;
    const float d3 = C * t3 * t3 + 0.25f * u3 * u3 + eps;
    const float a1 = 0.1f / (d1 * d1), a2 = 0.6f / (d2 * d2), a3 = 0.3f / (d3 * d3);
    const float rs = 1.0f / (a1 + a2 + a3);
    const float w1 = a1 * rs, w2 = a2 * rs, w3 = a3 * rs;
    const float p1 = 2.0f * v1 - 7.0f * v2 + 11.0f * v3;
    const float p2 = 5.0f * v3 - v2 + 2.0f * v4;
    const float p3 = 2.0f * v3 + 5.0f * v4 - v5;
    const float W = (w1 * p1 + w2 * p2 + w3 * p3) * (1.0f / 6.0f);
    const float B1 = (w2 * p12 + w3 * p13) * (1.0f / 6.0f);
    const float B2 = (w3 * p23 - w1 * p12) * (1.0f / 6.0f);
    const float B3 = -(w1 * p13 + w2 * p23) * (1.0f / 6.0f);
    const float d1b = 2.0f * (B2 * w2 + B3 * w3) / d1;
    const float d2b = 2.0f * (B1 * w1 + B3 * w3) / d2;
    const float d3b = 2.0f * (B1 * w1 + B2 * w2) / d3;
    const float p1b = w1 * (1.0f / 6.0f), p2b = w2 * (1.0f / 6.0f), p3b = w3 * (1.0f / 6.0f);
    const float t1b = d1b * 2.0f * C * t1, u1b = d1b * 0.5f * u1;
    const float t2b = d2b * 2.0f * C * t2, u2b = d2b * 0.5f * u2;
    const float t3b = d3b * 2.0f * C * t3, u3b = d3b * 0.5f * u3;
    g[0] = t1b + u1b + 2.0f * p1b;
    g[1] = -2.0f * t1b - 4.0f * u1b - 7.0f * p1b + t2b + u2b - p2b;
    g[2] = t1b + 3.0f * u1b + 11.0f * p1b - 2.0f * t2b + 5.0f * p2b + t3b + 3.0f * u3b + 2.0f * p3b;
    g[3] = t2b - u2b + 2.0f * p2b - 2.0f * t3b - 4.0f * u3b + 5.0f * p3b;
    g[4] = t3b + u3b - p3b;
    return W;
}

// a + b = s + e exactly (Knuth's TwoSum)
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
    const float s = a + b;
    const float ap = s - b;
    const float bp = s - ap;
    e = (a - ap) + (b - bp);
    return s;
}

// HJ-WENO5 derivative along one line and its gradient with respect to the
// seven line values S(-3..3): FD = W(D5..D1), BD = W(D0..D4), D_k = S_{k+1}-S_k.
// The second differences F_k = D_{k+1} - D_k come from the error-free D_k.
__device__ __forceinline__ float hj_grad(const Line7& L, bool fd, float dS[7]) {
    float D[6], Dl[6], F[5];
#pragma unroll
    for (int k = 0; k < 6; ++k) D[k] = two_sum(L.v[k + 1], -L.v[k], Dl[k]);
#pragma unroll
    for (int k = 0; k < 5; ++k) F[k] = (D[k + 1] - D[k]) + (Dl[k + 1] - Dl[k]);
    float g[5], dD[6] = {0, 0, 0, 0, 0, 0};
    float w;
    if (fd) {  // v = (D5, D4, D3, D2, D1): E_a = D_{5-a} - D_{6-a} = -F_{5-a}
        const float E[4] = {-F[4], -F[3], -F[2], -F[1]};
        w = weno5_grad(D[5], D[4], D[3], D[2], D[1], E, g);
        dD[5] = g[0]; dD[4] = g[1]; dD[3] = g[2]; dD[2] = g[3]; dD[1] = g[4];
    } else {  // v = (D0, ..., D4): E_a = F_{a-1}
        const float E[4] = {F[0], F[1], F[2], F[3]};
        w = weno5_grad(D[0], D[1], D[2], D[3], D[4], E, g);
#pragma unroll
        for (int k = 0; k < 5; ++k) dD[k] = g[k];
    }
#pragma unroll
    for (int j = 0; j < 7; ++j) dS[j] = (j > 0 ? dD[j - 1] : 0.0f) - (j < 6 ? dD[j] : 0.0f);
    return w;
}

// Shu's WENO5 value by the operations of weno5_grad's forward part.
__device__ __forceinline__ float weno5_val(float v1, float v2, float v3, float v4, float v5) {
    const float C = 13.0f / 12.0f, eps = 1.0e-8f;
    const float t1 = v1 - 2.0f * v2 + v3, u1 = v1 - 4.0f * v2 + 3.0f * v3;
    const float t2 = v2 - 2.0f * v3 + v4, u2 = v2 - v4;
    const float t3 = v3 - 2.0f * v4 + v5, u3 = 3.0f * v3 - 4.0f * v4 + v5;
    const float d1 = C * t1 * t1 + 0.25f * u1 * u1 + eps;
    const float d2 = C * t2 * t2 + 0.25f * u2 * u2 + eps;
    const float d3 = C * t3 * t3 + 0.25f * u3 * u3 + eps;
    const float q1 = d1 * d1, q2 = d2 * d2, q3 = d3 * d3;
    const float A1 = 0.1f * (q2 * q3), A2 = 0.6f * (q1 * q3), A3 = 0.3f * (q1 * q2);
    const float p1 = 2.0f * v1 - 7.0f * v2 + 11.0f * v3;
    const float p2 = 5.0f * v3 - v2 + 2.0f * v4;
    const float p3 = 2.0f * v3 + 5.0f * v4 - v5;
    const float S = A1 + A2 + A3;
    const float N = A1 * p1 + A2 * p2 + A3 * p3;
    return N / (6.0f * S);
}

__device__ __forceinline__ float hj_val(const Line7& L, bool fd) {
    float D[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) D[k] = L.v[k + 1] - L.v[k];
    return fd ? weno5_val(D[5], D[4], D[3], D[2], D[1]) : weno5_val(D[0], D[1], D[2], D[3], D[4]);
}

// Transposed stencil sums in a fixed order.  The stage kernels below hold
// one leaf per CTA and, axis by axis, the seven coefficients cf[k][q] =
// d out_q / d in_{q + (k-3) e_ax} * lam_out_q of every source voxel q in
// shared memory; each target point then sums its sources in k order.
// Targets inside the leaf accumulate in acc (and go to part[leaf][v]);
// targets in the three-voxel slabs of the six face neighbours go to the
// leaf's halo record, halo[(leaf * 6 + face) * 192 + d*64 + a*8 + c] with the
// slab point numbered as load_tile numbers it.  adj_combine_kernel then adds
// part and the neighbours' halo records into the packed adjoint, so no sum
// depends on the order in which CTAs run.
constexpr int HALO_FACE = 192;

__device__ __forceinline__ void gather_axis(int ax, const float (*cf)[LEAF_VOX], float* acc, float* halo, int64_t l) {
    const int t = threadIdx.x;
    const int stride = ax == 0 ? 64 : ax == 1 ? 8 : 1;
#pragma unroll 1
    for (int w = 0; w < 8; ++w) {
        const int v = 64 * w + t;
        const int pa = ax == 0 ? (v >> 6) : ax == 1 ? ((v >> 3) & 7) : (v & 7);
        float sum = 0.0f;
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            const int qa = pa - k + 3;
            if (qa >= 0 && qa < 8) sum += cf[k][v + (qa - pa) * stride];
        }
        acc[v] += sum;
    }
#pragma unroll 1
    for (int j = t; j < 2 * HALO_FACE; j += STENCIL_THREADS) {
        const int plus = j >= HALO_FACE ? 1 : 0;
        const int r = j - plus * HALO_FACE;
        const int d = r >> 6, aa = (r >> 3) & 7, cc = r & 7;
        const int pa = plus ? 8 + d : -3 + d;
        const int base = ax == 0 ? (aa << 3 | cc) : ax == 1 ? (aa << 6 | cc) : (aa << 6 | cc << 3);
        float sum = 0.0f;
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            const int qa = pa - k + 3;
            if (qa >= 0 && qa < 8) sum += cf[k][base + qa * stride];
        }
        halo[(size_t(l) * 6 + 2 * ax + plus) * HALO_FACE + r] = sum;
    }
}

// Rank of bit t in word w of mask m (pre: popcounts of the words before).
__device__ __forceinline__ int mask_rank(const uint64_t* m, const int* pre, int w, int t) {
    return pre[w] + __popcll(m[w] & ((uint64_t(1) << t) - 1));
}

__global__ void __launch_bounds__(STENCIL_THREADS) adj_rk_kernel(const AdjRkArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ float sv[3][LEAF_VOX];   // velocity as the stage used it, by position
    __shared__ float slo[LEAF_VOX];     // lam_out by position (0: inactive)
    __shared__ float cf[7][LEAF_VOX];
    __shared__ float acc[LEAF_VOX];
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    stage_masks(st, a.src, int(l), a.nbr + 6 * l, nullptr, nullptr);
    load_tile(tile, st, a.gamma);
    const int t = threadIdx.x;
    int pre[8];
    {
        int c = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) { pre[w] = c; c += __popcll(st.am[0][w]); }
    }
    int ox, oy, oz;
    key_origin(a.keys[l], ox, oy, oz);
#pragma unroll 1
    for (int w = 0; w < 8; ++w) {
        const int v = 64 * w + t;
        float lo = 0.0f;
        if ((st.am[0][w] >> t) & 1) lo = a.lam_out[size_t(l) * LEAF_VOX + mask_rank(st.am[0], pre, w, t)];
        float vel[3] = {0.0f, 0.0f, 0.0f};
        if (lo != 0.0f) {
            eval_field(a.field, ox + w, oy + (t >> 3), oz + (t & 7), a.t0, vel);
            if (a.backward) { vel[0] = -vel[0]; vel[1] = -vel[1]; vel[2] = -vel[2]; }
        }
        slo[v] = lo;
        acc[v] = a.beta * lo;
        sv[0][v] = vel[0];
        sv[1][v] = vel[1];
        sv[2][v] = vel[2];
    }
    __syncthreads();
    float gdt = 0.0f;  // this thread's part of dL/d(dt)
    const float sgn = a.backward ? -1.0f : 1.0f;
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
#pragma unroll 1
        for (int w = 0; w < 8; ++w) {
            const int v = 64 * w + t;
            const float lo = slo[v];
            if (lo == 0.0f) {
#pragma unroll
                for (int k = 0; k < 7; ++k) cf[k][v] = 0.0f;
                continue;
            }
            const int x = w, y = t >> 3, z = t & 7;
            const float va = sv[ax][v];
            float dS[7];
            const float wv = hj_grad(tile_line(tile, x, y, z, ax), va < 0.0f, dS);
            const float coef = -a.beta * a.dt * lo;
            const float c = coef * va * a.invdx;
#pragma unroll
            for (int k = 0; k < 7; ++k) cf[k][v] = c * dS[k];
            gdt -= a.beta * lo * va * (wv * a.invdx);
            if (a.dvel && a.field.kind == 1) {  // aligned dense velocity grid
                const int ia = ox + x - a.field.dense_origin[0], ja = oy + y - a.field.dense_origin[1],
                          ka = oz + z - a.field.dense_origin[2];
                if (ia >= 0 && ja >= 0 && ka >= 0 && ia < a.field.dense_dims[0] && ja < a.field.dense_dims[1] &&
                    ka < a.field.dense_dims[2]) {
                    // the voxel's own cell: no other thread of the launch writes it
                    float* p = a.dvel + 3 * ((size_t(ia) * a.field.dense_dims[1] + ja) * a.field.dense_dims[2] + ka);
                    p[ax] += sgn * (coef * wv * a.invdx);
                }
            }
        }
        __syncthreads();
        gather_axis(ax, cf, acc, a.halo, l);
        __syncthreads();
    }
#pragma unroll 1
    for (int w = 0; w < 8; ++w) a.part[size_t(l) * LEAF_VOX + 64 * w + t] = acc[64 * w + t];
    if (a.dt_part) {  // fixed-order block sum
        __shared__ double wsum[STENCIL_THREADS / 32];
        double d = gdt;
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        if ((t & 31) == 0) wsum[t >> 5] = d;
        __syncthreads();
        if (t == 0) {
            double s = 0.0;
            for (int k = 0; k < STENCIL_THREADS / 32; ++k) s += wsum[k];
            a.dt_part[l] += s;
        }
    }
}

__global__ void __launch_bounds__(STENCIL_THREADS) adj_norm_kernel(const AdjNormArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ uint64_t pm[8];
    __shared__ float scg[LEAF_VOX];       // lam4 * d phi4 / dG by position
    __shared__ float scoef[3][LEAF_VOX];  // d G / d (selected one-sided derivative), per axis
    __shared__ uint8_t sside[3][LEAF_VOX];  // 1: the upwind (FD) side was selected
    __shared__ float cf[7][LEAF_VOX];
    __shared__ float acc[LEAF_VOX];
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    stage_masks(st, a.src, int(l), a.nbr + 6 * l, a.pmask, pm);
    load_tile(tile, st, a.gamma);
    __syncthreads();
    const int t = threadIdx.x;
    int pre[8];
    {
        int c = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) { pre[w] = c; c += __popcll(pm[w]); }
    }
#pragma unroll 1
    for (int w = 0; w < 8; ++w) {
        const int v = 64 * w + t;
        const float lam = ((pm[w] >> t) & 1) ? a.lam4[size_t(l) * LEAF_VOX + mask_rank(pm, pre, w, t)] : 0.0f;
        acc[v] = 0.0f;
        scg[v] = 0.0f;
        scoef[0][v] = scoef[1][v] = scoef[2][v] = 0.0f;
        if (lam == 0.0f) continue;
        const int x = w, y = t >> 3, z = t & 7;
        const float phi0 = tile[tile_index(x, y, z)];
        const bool outside = phi0 > 0.0f;
        float G = 0.0f;
#pragma unroll 1
        for (int ax = 0; ax < 3; ++ax) {
            const Line7 L = tile_line(tile, x, y, z, ax);
            const float up = hj_val(L, true);
            const float dn = hj_val(L, false);
            float aa, bb;
            if (outside) { aa = fmaxf(dn, 0.0f); bb = fminf(up, 0.0f); }
            else { aa = fminf(dn, 0.0f); bb = fmaxf(up, 0.0f); }
            const bool take_b = aa * aa < bb * bb;
            G += take_b ? bb * bb : aa * aa;
            const bool dn_live = outside ? dn > 0.0f : dn < 0.0f;
            const bool up_live = outside ? up < 0.0f : up > 0.0f;
            scoef[ax][v] = take_b ? (up_live ? 2.0f * bb : 0.0f) : (dn_live ? 2.0f * aa : 0.0f);
            sside[ax][v] = take_b ? 1 : 0;
        }
        const float eps = 1e-8f;
        const float r = sqrtf(phi0 * phi0 + G);
        const float re = r + eps;
        const float s = phi0 / re;
        const float sg = sqrtf(G);
        const float fac = sg * a.invdx - 1.0f;
        const float ds_dphi = r > 0.0f ? (1.0f / re - phi0 * (phi0 / r) / (re * re)) : 1.0f / re;
        const float ds_dG = r > 0.0f ? -phi0 / (re * re) * (0.5f / r) : 0.0f;
        const float dphi4_dphi0 = 1.0f - a.mdt * ds_dphi * fac;
        const float dphi4_dG = -a.mdt * (ds_dG * fac + (sg > 0.0f ? s * a.invdx * 0.5f / sg : 0.0f));
        acc[v] = lam * dphi4_dphi0;
        scg[v] = lam * dphi4_dG;
    }
    __syncthreads();
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
#pragma unroll 1
        for (int w = 0; w < 8; ++w) {
            const int v = 64 * w + t;
            const float c = scg[v] * scoef[ax][v];
            if (c == 0.0f) {
#pragma unroll
                for (int k = 0; k < 7; ++k) cf[k][v] = 0.0f;
                continue;
            }
            float g[7];
            hj_grad(tile_line(tile, w, t >> 3, t & 7, ax), sside[ax][v] != 0, g);
#pragma unroll
            for (int k = 0; k < 7; ++k) cf[k][v] = c * g[k];
        }
        __syncthreads();
        gather_axis(ax, cf, acc, a.halo, l);
        __syncthreads();
    }
#pragma unroll 1
    for (int w = 0; w < 8; ++w) a.part[size_t(l) * LEAF_VOX + 64 * w + t] = acc[64 * w + t];
}

// lam[active voxel] += part + the face neighbours' halo records (fixed
// order: -x, +x, -y, +y, -z, +z); then lam_phin += alpha * lam_out.
__global__ void __launch_bounds__(64) adj_combine_kernel(const AdjCombineArgs a) {
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int t = threadIdx.x;
    int32_t nb[6];
#pragma unroll
    for (int f = 0; f < 6; ++f) nb[f] = a.nbr[6 * l + f];
    const int y = t >> 3, z = t & 7;
    int base = 0;
#pragma unroll 1
    for (int x = 0; x < 8; ++x) {
        const uint64_t m = a.am[size_t(l) * 8 + x];
        const int rank = base + __popcll(m & ((uint64_t(1) << t) - 1));
        base += __popcll(m);
        if (!((m >> t) & 1)) continue;
        float val = a.part[size_t(l) * LEAF_VOX + 64 * x + t];
        auto H = [&](int32_t n, int face, int d, int aa, int cc) {
            return a.halo[(size_t(n) * 6 + face) * HALO_FACE + d * 64 + aa * 8 + cc];
        };
        if (x < 3 && nb[0] >= 0) val += H(nb[0], 1, x, y, z);
        if (x >= 5 && nb[1] >= 0) val += H(nb[1], 0, x - 5, y, z);
        if (y < 3 && nb[2] >= 0) val += H(nb[2], 3, y, x, z);
        if (y >= 5 && nb[3] >= 0) val += H(nb[3], 2, y - 5, x, z);
        if (z < 3 && nb[4] >= 0) val += H(nb[4], 5, z, x, y);
        if (z >= 5 && nb[5] >= 0) val += H(nb[5], 4, z - 5, x, y);
        const size_t i = size_t(l) * LEAF_VOX + rank;
        a.lam[i] += val;
        if (a.lam_phin && a.alpha != 0.0f) a.lam_phin[i] += a.alpha * a.lam_out[i];
    }
}

__global__ void __launch_bounds__(64) adj_argmax_kernel(const AdjArgmaxArgs a) {
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int w = threadIdx.x >> 3, q = threadIdx.x & 7;  // word w, byte q
    const uint64_t bits = (a.am[size_t(l) * 8 + w] >> (8 * q)) & 0xffu;
    if (!bits) return;
    int ox, oy, oz;
    key_origin(a.keys[l], ox, oy, oz);
    for (int b = 0; b < 8; ++b) {
        if (!((bits >> b) & 1)) continue;
        const int v = 64 * w + 8 * q + b;
        float vel[3];
        eval_field(a.field, ox + (v >> 6), oy + ((v >> 3) & 7), oz + (v & 7), a.t0, vel);
        // |v|^2 as the CFL reduction forms it
        const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(vel[0], vel[0]), __fmul_rn(vel[1], vel[1])),
                                   __fmul_rn(vel[2], vel[2]));
        if (l2 == a.maxv2) {
            atomicMin(a.argkey, static_cast<unsigned long long>(l) * LEAF_VOX + unsigned(v));
            return;  // this thread's later voxels come after this one
        }
    }
}

__global__ void adj_argcell_kernel(const AdjArgmaxArgs a) {
    const unsigned long long k = *a.argkey;
    int64_t cell = -1;
    if (k != ~0ull && int64_t(k / LEAF_VOX) < a.nleaf) {
        const int64_t l = int64_t(k / LEAF_VOX);
        const int v = int(k % LEAF_VOX);
        int ox, oy, oz;
        key_origin(a.keys[l], ox, oy, oz);
        const FieldParams& f = a.field;
        const int i = ox + (v >> 6) - f.dense_origin[0], j = oy + ((v >> 3) & 7) - f.dense_origin[1],
                  kk = oz + (v & 7) - f.dense_origin[2];
        if (i >= 0 && j >= 0 && kk >= 0 && i < f.dense_dims[0] && j < f.dense_dims[1] && kk < f.dense_dims[2])
            cell = (int64_t(i) * f.dense_dims[1] + j) * f.dense_dims[2] + kk;
    }
    *a.argcell = cell;
}

__global__ void __launch_bounds__(1024) adj_dt_reduce_kernel(const double* part, int64_t n, double* out) {
    double d = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) d += part[i];
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    __shared__ double ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < 32; ++k) t += ws[k];
        *out = t;
    }
}

__global__ void adj_dt_scatter_kernel(int64_t n, const int64_t* cell, const float* mbar, const float* dense,
                                      float* dvel) {
    for (int64_t k = 0; k < n; ++k) {
        const int64_t c = cell[k];
        if (c < 0 || mbar[k] == 0.0f) continue;
        for (int e = 0; e < 3; ++e) dvel[3 * c + e] += 2.0f * mbar[k] * dense[3 * c + e];
    }
}

// lam4 over the renormalised voxels of each merged leaf: the next list's
// adjoint where the voxel survived trimming, 0 where it was trimmed.
__global__ void __launch_bounds__(64) adj_expand_kernel(const AdjExpandArgs a) {
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int t = threadIdx.x;
    const uint64_t low = (uint64_t(1) << t) - 1;
    const bool kept = a.keep[l] != 0;
    const int j = a.idx[l];
    int bp = 0, bf = 0;
    for (int k = 0; k < 8; ++k) {
        const uint64_t p = a.pmask[size_t(l) * 8 + k], f = a.fin[size_t(l) * 8 + k];
        if ((p >> t) & 1) {
            float val = 0.0f;
            if (kept && ((f >> t) & 1)) val = a.lam_next[size_t(j) * LEAF_VOX + bf + __popcll(f & low)];
            a.lam4[size_t(l) * LEAF_VOX + bp + __popcll(p & low)] = val;
        }
        bp += __popcll(p);
        bf += __popcll(f);
    }
}

__global__ void __launch_bounds__(64) adj_map_kernel(const AdjMapArgs a) {
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int64_t m = find_u64(a.keys_m, a.nleaf_m, a.keys[l]);
    int n = 0;
    for (int w = 0; w < 8; ++w) n += __popcll(a.am[size_t(l) * 8 + w]);
    for (int i = threadIdx.x; i < n; i += 64)
        a.lam[size_t(l) * LEAF_VOX + i] = m >= 0 ? a.lam_m[size_t(m) * LEAF_VOX + i] : 0.0f;
}

__global__ void k_tape_gather(int64_t n, const int32_t* slot, const uint64_t* am, const uint64_t* sm,
                              const float* vals, uint64_t* am_o, uint64_t* sm_o, float* vals_o) {
    const int64_t l = blockIdx.x;
    if (l >= n) return;
    const int s = slot[l];
    const int t = threadIdx.x;
    if (t < 8) {
        if (am_o) am_o[size_t(l) * 8 + t] = am[size_t(s) * 8 + t];
        if (sm_o) sm_o[size_t(l) * 8 + t] = sm[size_t(s) * 8 + t];
    }
    if (vals_o) {
        int cnt = 0;
        for (int w = 0; w < 8; ++w) cnt += __popcll(am[size_t(s) * 8 + w]);
        for (int i = t; i < cnt; i += blockDim.x) vals_o[size_t(l) * LEAF_VOX + i] = vals[size_t(s) * LEAF_VOX + i];
    }
}

__global__ void k_slot_inverse(int64_t n, const int32_t* slot, int32_t* inv) {
    const int64_t l = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (l < n) inv[slot[l]] = int32_t(l);
}

__global__ void k_nbr_remap(int64_t n, const int32_t* nbr, const int32_t* inv, int32_t* out) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n * 6) return;
    const int32_t s = nbr[i];
    out[i] = s >= 0 ? inv[s] : s;
}

inline unsigned nblk(int64_t n, int t) { return unsigned((n + t - 1) / t); }

}  // namespace

void launch_tape_gather(int64_t n, const int32_t* slot, const uint64_t* am, const uint64_t* sm, const float* vals,
                        uint64_t* am_o, uint64_t* sm_o, float* vals_o, cudaStream_t s) {
    if (n > 0) k_tape_gather<<<unsigned(n), 64, 0, s>>>(n, slot, am, sm, vals, am_o, sm_o, vals_o);
}

void launch_mask_gather(int64_t n, const int32_t* slot, const uint64_t* m, uint64_t* m_o, cudaStream_t s) {
    if (n > 0) k_tape_gather<<<unsigned(n), 64, 0, s>>>(n, slot, m, nullptr, nullptr, m_o, nullptr, nullptr);
}

void launch_nbr_to_index(int64_t n, const int32_t* slot, const int32_t* nbr, int32_t* inv, int64_t slot_cap,
                         int32_t* nbr_o, cudaStream_t s) {
    (void)slot_cap;
    if (n <= 0) return;
    k_slot_inverse<<<nblk(n, 256), 256, 0, s>>>(n, slot, inv);
    k_nbr_remap<<<nblk(n * 6, 256), 256, 0, s>>>(n, nbr, inv, nbr_o);
}

void launch_adj_rk(const AdjRkArgs& a, cudaStream_t s) {
    if (a.nleaf > 0) adj_rk_kernel<<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}
void launch_adj_norm(const AdjNormArgs& a, cudaStream_t s) {
    if (a.nleaf > 0) adj_norm_kernel<<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}
void launch_adj_combine(const AdjCombineArgs& a, cudaStream_t s) {
    if (a.nleaf > 0) adj_combine_kernel<<<unsigned(a.nleaf), 64, 0, s>>>(a);
}
void launch_adj_expand(const AdjExpandArgs& a, cudaStream_t s) {
    if (a.nleaf > 0) adj_expand_kernel<<<unsigned(a.nleaf), 64, 0, s>>>(a);
}
void launch_adj_map(const AdjMapArgs& a, cudaStream_t s) {
    if (a.nleaf > 0) adj_map_kernel<<<unsigned(a.nleaf), 64, 0, s>>>(a);
}
void launch_adj_argmax(const AdjArgmaxArgs& a, cudaStream_t s) {
    if (a.nleaf > 0) adj_argmax_kernel<<<unsigned(a.nleaf), 64, 0, s>>>(a);
    adj_argcell_kernel<<<1, 1, 0, s>>>(a);
}
void launch_adj_dt_reduce(const double* part, int64_t n, double* out, cudaStream_t s) {
    adj_dt_reduce_kernel<<<1, 1024, 0, s>>>(part, n, out);
}
void launch_adj_dt_scatter(int64_t n, const int64_t* cell, const float* mbar, const float* dense, float* dvel,
                           cudaStream_t s) {
    if (n > 0) adj_dt_scatter_kernel<<<1, 1, 0, s>>>(n, cell, mbar, dense, dvel);
}

}  // namespace gbls
