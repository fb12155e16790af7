// Adjoint kernels: transposed Jacobians of the recorded RK3-HJWENO5 stages
// (tools/LevelSetAdvect.h:543-572) and of the Godunov renormalisation
// (tools/LevelSetTracker.h:623-643), in FP32, with the branch structure of
// the forward pass (upwind direction from the velocity sign, Godunov term
// selection, trimming, topology) held fixed.
#include "adjoint.h"
#include "stencil_ops.cuh"

namespace gbls {

namespace {

// Shu's WENO5 (the FastArith formula, weights not rescaled) and its gradient
// g[k] = dW/dv_{k+1}, by reverse-mode differentiation of the expression.
__device__ __forceinline__ float weno5_grad(float v1, float v2, float v3, float v4, float v5, float g[5]) {
    const float C = 13.0f / 12.0f, eps = 1.0e-8f;
    const float t1 = v1 - 2.0f * v2 + v3, u1 = v1 - 4.0f * v2 + 3.0f * v3;
    const float t2 = v2 - 2.0f * v3 + v4, u2 = v2 - v4;
    const float t3 = v3 - 2.0f * v4 + v5, u3 = 3.0f * v3 - 4.0f * v4 + v5;
    const float d1 = C * t1 * t1 + 0.25f * u1 * u1 + eps;
    const float d2 = C * t2 * t2 + 0.25f * u2 * u2 + eps;
    const float d3 = C * t3 * t3 + 0.25f * u3 * u3 + eps;
    // scale the weights by d1^2 d2^2 d3^2 as the forward does (ratios unchanged)
    const float q1 = d1 * d1, q2 = d2 * d2, q3 = d3 * d3;
    const float A1 = 0.1f * (q2 * q3), A2 = 0.6f * (q1 * q3), A3 = 0.3f * (q1 * q2);
    const float p1 = 2.0f * v1 - 7.0f * v2 + 11.0f * v3;
    const float p2 = 5.0f * v3 - v2 + 2.0f * v4;
    const float p3 = 2.0f * v3 + 5.0f * v4 - v5;
    const float S = A1 + A2 + A3;
    const float N = A1 * p1 + A2 * p2 + A3 * p3;
    const float W = N / (6.0f * S);
    // reverse: W = N / (6 S)
    const float Nb = 1.0f / (6.0f * S);
    const float Sb = -W / S;
    const float A1b = Nb * p1 + Sb, A2b = Nb * p2 + Sb, A3b = Nb * p3 + Sb;
    const float p1b = Nb * A1, p2b = Nb * A2, p3b = Nb * A3;
    // A1 = 0.1 q2 q3 etc. with q_k = d_k^2
    const float q1b = A2b * 0.6f * q3 + A3b * 0.3f * q2;
    const float q2b = A1b * 0.1f * q3 + A3b * 0.3f * q1;
    const float q3b = A1b * 0.1f * q2 + A2b * 0.6f * q1;
    const float d1b = q1b * 2.0f * d1, d2b = q2b * 2.0f * d2, d3b = q3b * 2.0f * d3;
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

// HJ-WENO5 derivative along one line and its gradient with respect to the
// seven line values S(-3..3): FD = W(D5..D1), BD = W(D0..D4), D_k = S_{k+1}-S_k.
__device__ __forceinline__ float hj_grad(const Line7& L, bool fd, float dS[7]) {
    float D[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) D[k] = L.v[k + 1] - L.v[k];
    float g[5], dD[6] = {0, 0, 0, 0, 0, 0};
    float w;
    if (fd) {
        w = weno5_grad(D[5], D[4], D[3], D[2], D[1], g);
        dD[5] = g[0]; dD[4] = g[1]; dD[3] = g[2]; dD[2] = g[3]; dD[1] = g[4];
    } else {
        w = weno5_grad(D[0], D[1], D[2], D[3], D[4], g);
#pragma unroll
        for (int k = 0; k < 5; ++k) dD[k] = g[k];
    }
#pragma unroll
    for (int j = 0; j < 7; ++j) dS[j] = (j > 0 ? dD[j - 1] : 0.0f) - (j < 6 ? dD[j] : 0.0f);
    return w;
}

// lam[packed index of tile point (x,y,z)] += val when that point is an
// active voxel of the staged layout (inactive points and tiles are constants).
__device__ __forceinline__ void scatter_add(const LeafStage& st, float* lam, int x, int y, int z, float val) {
    int r = 0;
    if (x < 0) { r = 1; x += 8; }
    else if (x >= 8) { r = 2; x -= 8; }
    else if (y < 0) { r = 3; y += 8; }
    else if (y >= 8) { r = 4; y -= 8; }
    else if (z < 0) { r = 5; z += 8; }
    else if (z >= 8) { r = 6; z -= 8; }
    const int v = (x << 6) | (y << 3) | z;
    const uint4 q = st.rec[r][v >> 5];  // half word (v >> 6, (v >> 5) & 1)
    const int bb = v & 31;
    if (!((q.x >> bb) & 1)) return;
    const uint32_t rank = q.z + uint32_t(__popc(q.x & ((1u << bb) - 1u)));
    atomicAdd(lam + size_t(st.slot[r]) * LEAF_VOX + rank, val);
}

__device__ __forceinline__ void axis_point(int ax, int x, int y, int z, int k, int& px, int& py, int& pz) {
    px = x + (ax == 0 ? k : 0);
    py = y + (ax == 1 ? k : 0);
    pz = z + (ax == 2 ? k : 0);
}

__global__ void __launch_bounds__(STENCIL_THREADS) adj_rk_kernel(const AdjRkArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ uint16_t list[LEAF_VOX];
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    stage_masks(st, a.src, int(l), a.nbr + 6 * l, nullptr, nullptr);
    load_tile(tile, st, a.gamma);
    const int n = build_list(list, st.am[0]);
    __syncthreads();
    int ox, oy, oz;
    key_origin(a.keys[l], ox, oy, oz);
    for (int i = threadIdx.x; i < n; i += STENCIL_THREADS) {
        const float lo = a.lam_out[size_t(l) * LEAF_VOX + i];
        if (lo == 0.0f) continue;
        const int v = list[i];
        const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
        float vel[3];
        eval_field(a.field, ox + x, oy + y, oz + z, a.t0, vel);
        if (a.backward) { vel[0] = -vel[0]; vel[1] = -vel[1]; vel[2] = -vel[2]; }
        if (a.alpha != 0.0f) atomicAdd(a.lam_phin + size_t(l) * LEAF_VOX + i, a.alpha * lo);
        atomicAdd(a.lam_in + size_t(l) * LEAF_VOX + i, a.beta * lo);
        const float coef = -a.beta * a.dt * lo;
        float dv[3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const Line7 L = tile_line(tile, x, y, z, ax);
            float dS[7];
            const float w = hj_grad(L, vel[ax] < 0.0f, dS);
            dv[ax] = coef * w * a.invdx;
            const float c = coef * vel[ax] * a.invdx;
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                if (dS[k] == 0.0f) continue;
                int px, py, pz;
                axis_point(ax, x, y, z, k - 3, px, py, pz);
                scatter_add(st, a.lam_in, px, py, pz, c * dS[k]);
            }
        }
        if (a.dvel && a.field.kind == 1) {  // aligned dense velocity grid
            const int ia = ox + x - a.field.dense_origin[0], ja = oy + y - a.field.dense_origin[1],
                      ka = oz + z - a.field.dense_origin[2];
            if (ia >= 0 && ja >= 0 && ka >= 0 && ia < a.field.dense_dims[0] && ja < a.field.dense_dims[1] &&
                ka < a.field.dense_dims[2]) {
                float* p = a.dvel + 3 * ((size_t(ia) * a.field.dense_dims[1] + ja) * a.field.dense_dims[2] + ka);
                const float sgn = a.backward ? -1.0f : 1.0f;
                atomicAdd(p, sgn * dv[0]);
                atomicAdd(p + 1, sgn * dv[1]);
                atomicAdd(p + 2, sgn * dv[2]);
            }
        }
    }
}

__global__ void __launch_bounds__(STENCIL_THREADS) adj_norm_kernel(const AdjNormArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ uint16_t list[LEAF_VOX];
    __shared__ uint64_t pm[8];
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    stage_masks(st, a.src, int(l), a.nbr + 6 * l, a.pmask, pm);
    load_tile(tile, st, a.gamma);
    __syncthreads();
    const int n = build_list(list, pm);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += STENCIL_THREADS) {
        const float lam = a.lam4[size_t(l) * LEAF_VOX + i];
        if (lam == 0.0f) continue;
        const int v = list[i];
        const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
        const float phi0 = tile[tile_index(x, y, z)];
        const bool outside = phi0 > 0.0f;
        float G = 0.0f;
        float dtdn[3], dtup[3];
        float gu[3][7], gd[3][7];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const Line7 L = tile_line(tile, x, y, z, ax);
            const float up = hj_grad(L, true, gu[ax]);
            const float dn = hj_grad(L, false, gd[ax]);
            float aa, bb;
            if (outside) { aa = fmaxf(dn, 0.0f); bb = fminf(up, 0.0f); }
            else { aa = fminf(dn, 0.0f); bb = fmaxf(up, 0.0f); }
            const bool take_b = aa * aa < bb * bb;
            G += take_b ? bb * bb : aa * aa;
            const bool dn_live = outside ? dn > 0.0f : dn < 0.0f;
            const bool up_live = outside ? up < 0.0f : up > 0.0f;
            dtdn[ax] = (!take_b && dn_live) ? 2.0f * aa : 0.0f;
            dtup[ax] = (take_b && up_live) ? 2.0f * bb : 0.0f;
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
        float centre = lam * dphi4_dphi0;
        const float cg = lam * dphi4_dG;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const float c = cg * (dtdn[ax] * gd[ax][k] + dtup[ax] * gu[ax][k]);
                if (k == 3) { centre += c; continue; }
                if (c == 0.0f) continue;
                int px, py, pz;
                axis_point(ax, x, y, z, k - 3, px, py, pz);
                scatter_add(st, a.lam3, px, py, pz, c);
            }
        }
        scatter_add(st, a.lam3, x, y, z, centre);
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
void launch_adj_expand(const AdjExpandArgs& a, cudaStream_t s) {
    if (a.nleaf > 0) adj_expand_kernel<<<unsigned(a.nleaf), 64, 0, s>>>(a);
}
void launch_adj_map(const AdjMapArgs& a, cudaStream_t s) {
    if (a.nleaf > 0) adj_map_kernel<<<unsigned(a.nleaf), 64, 0, s>>>(a);
}

}  // namespace gbls
