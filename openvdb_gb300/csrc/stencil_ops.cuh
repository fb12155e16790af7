// Stencil arithmetic and the per-leaf kernels of the advection hot path.
//
// Included by two translation units with different arithmetic policies:
//   stencil_parity.cu  ParityArith: every operation of the reference,
//                      in its order and its types (FP64 WENO weights), with
//                      explicit round-to-nearest intrinsics so no operation
//                      can be contracted or reassociated.  Bit-identical to
//                      the reference CPU path compiled without contraction.
//   stencil_fast.cu    FastArith: FP32 throughout, contracted, one division
//                      per WENO5.
#pragma once

#include "gbls_internal.cuh"
#include "weno_exact.h"
#include "../../include/gbls_fields.h"

namespace gbls {

// ---- arithmetic policies ---------------------------------------------------

struct ParityArith {
    static constexpr bool kParity = true;
    __device__ __forceinline__ static float add(float a, float b) { return __fadd_rn(a, b); }
    __device__ __forceinline__ static float sub(float a, float b) { return __fsub_rn(a, b); }
    __device__ __forceinline__ static float mul(float a, float b) { return __fmul_rn(a, b); }
    __device__ __forceinline__ static float div(float a, float b) { return __fdiv_rn(a, b); }
    __device__ __forceinline__ static float sqrt(float a) { return __fsqrt_rn(a); }

    // math::WENO5<float> (math/FiniteDifference.h:301-321), scale2 = 0.01f.
    // Types follow the C++ expression: `2*v2`, `4*v2`, Pow2 of a float are
    // float; anything multiplied by a double literal or by C is double.
    __device__ static float weno5(float v1, float v2, float v3, float v4, float v5) {
        const double C = 13.0 / 12.0;
        const double eps = 1.0e-6 * static_cast<double>(0.01f);
        // A1 = 0.1/Pow2(C*Pow2(v1-2*v2+v3) + 0.25*Pow2(v1-4*v2+3.0*v3) + eps)
        const float t1 = __fadd_rn(__fsub_rn(v1, __fmul_rn(2.0f, v2)), v3);
        const double s1a = __dmul_rn(C, double(__fmul_rn(t1, t1)));
        const double u1 = __dadd_rn(double(__fsub_rn(v1, __fmul_rn(4.0f, v2))), __dmul_rn(3.0, double(v3)));
        const double s1b = __dmul_rn(0.25, __dmul_rn(u1, u1));
        const double d1 = __dadd_rn(__dadd_rn(s1a, s1b), eps);
        const double A1 = __ddiv_rn(0.1, __dmul_rn(d1, d1));
        // A2 = 0.6/Pow2(C*Pow2(v2-2*v3+v4) + 0.25*Pow2(v2-v4) + eps)
        const float t2 = __fadd_rn(__fsub_rn(v2, __fmul_rn(2.0f, v3)), v4);
        const double s2a = __dmul_rn(C, double(__fmul_rn(t2, t2)));
        const float u2 = __fsub_rn(v2, v4);
        const double s2b = __dmul_rn(0.25, double(__fmul_rn(u2, u2)));
        const double d2 = __dadd_rn(__dadd_rn(s2a, s2b), eps);
        const double A2 = __ddiv_rn(0.6, __dmul_rn(d2, d2));
        // A3 = 0.3/Pow2(C*Pow2(v3-2*v4+v5) + 0.25*Pow2(3.0*v3-4*v4+v5) + eps)
        const float t3 = __fadd_rn(__fsub_rn(v3, __fmul_rn(2.0f, v4)), v5);
        const double s3a = __dmul_rn(C, double(__fmul_rn(t3, t3)));
        const double u3 = __dadd_rn(__dsub_rn(__dmul_rn(3.0, double(v3)), double(__fmul_rn(4.0f, v4))),
                                    double(v5));
        const double s3b = __dmul_rn(0.25, __dmul_rn(u3, u3));
        const double d3 = __dadd_rn(__dadd_rn(s3a, s3b), eps);
        const double A3 = __ddiv_rn(0.3, __dmul_rn(d3, d3));
        // A1*(2v1-7v2+11v3) + A2*(5v3-v2+2v4) + A3*(2v3+5v4-v5)
        const double p1 = __dadd_rn(__dsub_rn(__dmul_rn(2.0, double(v1)), __dmul_rn(7.0, double(v2))),
                                    __dmul_rn(11.0, double(v3)));
        const double p2 = __dadd_rn(__dsub_rn(__dmul_rn(5.0, double(v3)), double(v2)),
                                    __dmul_rn(2.0, double(v4)));
        const double p3 = __dsub_rn(__dadd_rn(__dmul_rn(2.0, double(v3)), __dmul_rn(5.0, double(v4))),
                                    double(v5));
        const double num = __dadd_rn(__dadd_rn(__dmul_rn(A1, p1), __dmul_rn(A2, p2)), __dmul_rn(A3, p3));
        const double den = __dmul_rn(6.0, __dadd_rn(__dadd_rn(A1, A2), A3));
        return __double2float_rn(__ddiv_rn(double(__double2float_rn(num)), den));
    }

    // Vec3d(iGradient) -> map.applyIJT (x 1/dx in double) -> Vec3f
    // (math/Operators.h:838-845, math/Maps.h:767-771).
    __device__ __forceinline__ static float ijt(float g, double invdx, float) {
        return __double2float_rn(__dmul_rn(double(g), invdx));
    }
};

// ParityArith's results (bit-identical to the reference) on the FP32 pipes:
// WENO5 from the double-word evaluation of weno_exact.h, which decides the
// reference's float result in all but about one evaluation in 10^4; those
// take ParityArith's FP64 formula.  The float operations are ParityArith's.
static __device__ __noinline__ float weno5_fp64(float v1, float v2, float v3, float v4, float v5) {
    return ParityArith::weno5(v1, v2, v3, v4, v5);
}
static __device__ __noinline__ float ijt_fp64(float g, double invdx) { return ParityArith::ijt(g, invdx, 0.0f); }

struct ExactArith : ParityArith {
    __device__ __forceinline__ static float weno5(float v1, float v2, float v3, float v4, float v5) {
        float r;
        if (xw::weno5<float>(v1, v2, v3, v4, v5, r)) return r;
        return weno5_fp64(v1, v2, v3, v4, v5);
    }
    // applyIJT: with dx = 1 the double product is g itself; otherwise the
    // FP64 product, in a call the compiler cannot execute speculatively
    __device__ __forceinline__ static float ijt(float g, double invdx, float) {
        if (__double_as_longlong(invdx) == 0x3FF0000000000000ll) return g;
        return ijt_fp64(g, invdx);
    }
};

template <class A> struct IsExact { static constexpr bool value = false; };
template <> struct IsExact<ExactArith> { static constexpr bool value = true; };

struct FastArith {
    static constexpr bool kParity = false;
    __device__ __forceinline__ static float add(float a, float b) { return a + b; }
    __device__ __forceinline__ static float sub(float a, float b) { return a - b; }
    __device__ __forceinline__ static float mul(float a, float b) { return a * b; }
    __device__ __forceinline__ static float div(float a, float b) { return __fdividef(a, b); }
    __device__ __forceinline__ static float sqrt(float a) { return sqrtf(a); }

    // Shu's WENO5 in FP32.  The three weights share one reciprocal:
    // w_k = c_k / d_k^2 are scaled by d1^2 d2^2 d3^2 (d_k >= eps = 1e-8, so
    // the products stay above 1e-32, far from FP32 underflow).
    __device__ __forceinline__ static float weno5(float v1, float v2, float v3, float v4, float v5) {
        const float C = 13.0f / 12.0f;
        const float eps = 1.0e-8f;
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
        const float num = A1 * p1 + A2 * p2 + A3 * p3;
        const float den = 6.0f * (A1 + A2 + A3);
        return __fdividef(num, den);
    }

    __device__ __forceinline__ static float ijt(float g, double, float invdx) { return g * invdx; }
};

// ---- HJ-WENO5 one-sided derivatives on the staged tile --------------------
// D1<FD_HJWENO5> (math/FiniteDifference.h:1177-1274):
//   WENO5(S3-S2, S2-S1, S1-S0, S0-Sm1, Sm1-Sm2)
// D1<BD_HJWENO5> (:1381-1389 and its stencil form):
//   -WENO5(Sm3-Sm2, Sm2-Sm1, Sm1-S0, S0-S1, S1-S2)
template <class A>
__device__ __forceinline__ float hj_fd(float m2, float m1, float c, float p1, float p2, float p3) {
    return A::weno5(A::sub(p3, p2), A::sub(p2, p1), A::sub(p1, c), A::sub(c, m1), A::sub(m1, m2));
}
template <class A>
__device__ __forceinline__ float hj_bd(float m3, float m2, float m1, float c, float p1, float p2) {
    return -A::weno5(A::sub(m3, m2), A::sub(m2, m1), A::sub(m1, c), A::sub(c, p1), A::sub(p1, p2));
}

// The seven values along one axis around the centre, S(-3..3).
struct Line7 {
    float v[7];
};

__device__ __forceinline__ Line7 tile_line(const float* tile, int x, int y, int z, int axis) {
    Line7 L;
    const int stride = axis == 0 ? TILE_DIM * TILE_DIM : axis == 1 ? TILE_DIM : 1;
    const int c = tile_index(x, y, z);
#pragma unroll
    for (int k = 0; k < 7; ++k) L.v[k] = tile[c + (k - 3) * stride];
    return L;
}

// One-sided HJ-WENO5 derivatives from the six differences D_k = S(k-2) - S(k-3)
// of a line (k = 0..5): FD = WENO5(D5, D4, D3, D2, D1) is the reference's FD
// operand list; BD = -WENO5(-D0, ..., -D4) = WENO5(D0, ..., D4) because WENO5
// is odd in its arguments — exactly, operation by operation, in any IEEE
// rounding-to-nearest arithmetic (squares, products and sums change sign
// exactly).  Same operands and operations as hj_fd / hj_bd.
struct Diff6 {
    float d[6];
};
template <class A>
__device__ __forceinline__ Diff6 line_diffs(const Line7& L) {
    Diff6 D;
#pragma unroll
    for (int k = 0; k < 6; ++k) D.d[k] = A::sub(L.v[k + 1], L.v[k]);
    return D;
}
template <class A>
__device__ __forceinline__ float diff_fd(const Diff6& D) {
    return A::weno5(D.d[5], D.d[4], D.d[3], D.d[2], D.d[1]);
}
template <class A>
__device__ __forceinline__ float diff_bd(const Diff6& D) {
    return A::weno5(D.d[0], D.d[1], D.d[2], D.d[3], D.d[4]);
}
// V<0 ? FD : BD with one WENO5 evaluation on selected operands.
template <class A>
__device__ __forceinline__ float line_upwind(const Line7& L, bool fd) {
    const Diff6 D = line_diffs<A>(L);
    float in[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) in[k] = fd ? D.d[5 - k] : D.d[k];
    return A::weno5(in[0], in[1], in[2], in[3], in[4]);
}

template <class A>
__device__ __forceinline__ float line_fd(const Line7& L) {
    return hj_fd<A>(L.v[1], L.v[2], L.v[3], L.v[4], L.v[5], L.v[6]);
}
template <class A>
__device__ __forceinline__ float line_bd(const Line7& L) {
    return hj_bd<A>(L.v[0], L.v[1], L.v[2], L.v[3], L.v[4], L.v[5]);
}

// The other biased schemes (math/FiniteDifference.h D1<FD_1ST> .. D1<BD_WENO5>,
// :702-1375, selected by BIAS_SCHEME, math/Operators.h:139-186) from the
// values S(-3..3) of a line, operation by operation.  FD_3RD evaluates in
// double with explicit rounding.
__device__ __forceinline__ float fd3(float xp3, float xp2, float xp1, float xp0) {
    const double a = __dsub_rn(__ddiv_rn(double(xp3), 3.0), __dmul_rn(1.5, double(xp2)));
    const double b = __dadd_rn(a, __dmul_rn(3.0, double(xp1)));
    return __double2float_rn(__dsub_rn(b, __ddiv_rn(__dmul_rn(11.0, double(xp0)), 6.0)));
}
template <class A>
__device__ __forceinline__ float fd2(float xp2, float xp1, float xp0) {
    return A::sub(A::mul(2.0f, xp1), A::add(A::mul(0.5f, xp2), A::mul(1.5f, xp0)));
}
template <class A>
__device__ inline float scheme_fd(const Line7& L, int scheme) {
    const float* v = L.v;
    switch (scheme) {
    case 0: return A::sub(v[4], v[3]);                                   // FD_1ST
    case 1: return fd2<A>(v[5], v[4], v[3]);                             // FD_2ND
    case 2: return fd3(v[6], v[5], v[4], v[3]);                          // FD_3RD
    case 3: return A::sub(A::weno5(v[6], v[5], v[4], v[3], v[2]),       // FD_WENO5
                          A::weno5(v[5], v[4], v[3], v[2], v[1]));
    default: return diff_fd<A>(line_diffs<A>(L));                        // FD_HJWENO5
    }
}
template <class A>
__device__ inline float scheme_bd(const Line7& L, int scheme) {
    const float* v = L.v;
    switch (scheme) {
    case 0: return -A::sub(v[2], v[3]);                                  // BD_1ST = -FD_1ST(xm1, xm0)
    case 1: return -fd2<A>(v[1], v[2], v[3]);                            // BD_2ND
    case 2: return -fd3(v[0], v[1], v[2], v[3]);                         // BD_3RD
    case 3: return -A::sub(A::weno5(v[0], v[1], v[2], v[3], v[4]),      // BD_WENO5
                           A::weno5(v[1], v[2], v[3], v[4], v[5]));
    default: return diff_bd<A>(line_diffs<A>(L));                        // BD_HJWENO5
    }
}
// ISGradientBiased per axis: V < 0 ? FD : BD (math/Operators.h:195-226).
template <class A>
__device__ __forceinline__ float scheme_upwind(const Line7& L, bool fd, int scheme) {
    if (scheme == 4) return line_upwind<A>(L, fd);
    return fd ? scheme_fd<A>(L, scheme) : scheme_bd<A>(L, scheme);
}

// std::max / std::min as used by math::Max / math::Min.
__device__ __forceinline__ float ref_max(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float ref_min(float a, float b) { return (b < a) ? b : a; }

// math::GodunovsNormSqrd (math/FiniteDifference.h:324-357) with
// gradient_m = BD ("down"), gradient_p = FD ("up").
template <class A>
__device__ __forceinline__ float godunov(bool outside, const float* dm, const float* dp) {
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float term;
        if (outside) {
            const float a = ref_max(dm[k], 0.0f), b = ref_min(dp[k], 0.0f);
            term = ref_max(A::mul(a, a), A::mul(b, b));
        } else {
            const float a = ref_min(dm[k], 0.0f), b = ref_max(dp[k], 0.0f);
            term = ref_max(A::mul(a, a), A::mul(b, b));
        }
        acc = (k == 0) ? term : A::add(acc, term);
    }
    return acc;
}

// GodunovsNormSqrd (math/FiniteDifference.h:324-357) of the HJ-WENO5
// derivatives of every processed voxel of a leaf (the voxels of pm in
// `list`) into gsq[v] (v the voxel's position), evaluating only the
// derivatives whose value it uses: outside (phi0 > 0) a backward derivative
// known to be <= 0 enters as (max(dm,0))^2 = 0 and a forward one known to be
// >= 0 as (min(dp,0))^2 = 0, inside the mirror images, and a derivative that
// is a zero (five zero differences) adds +0; a derivative left out counts as
// 0, whose square is the same +0.  The signs come from xw::weno5_sign_pair.
// A warp that evaluates each voxel's derivatives in turn runs the union of
// its lanes' needs (about six WENO5 per voxel); here the
// derivatives a voxel needs become work items of a CTA-wide list, axis by
// axis, so every lane evaluates one needed WENO5 at a time.  An axis term
// max(a^2, b^2) is the maximum of its items' squares (+0 without items;
// non-negative floats order like their bits), kept in gsq as bits while the
// axis runs, and the terms are summed in axis order in registers (thread t
// owns list entries t + 64k).  The list of at most `cap` items lives in
// dead staging memory; more than cap/2 processed voxels run in two rounds.
// All threads call; starts and ends with a barrier.
__device__ inline void godunov_exact_leaf(const float* tile, const uint16_t* list, int n, const uint64_t* pm,
                                          float* gsq, uint16_t* queue, int cap, int* qn) {
    const int t = threadIdx.x;
    uint32_t* term = reinterpret_cast<uint32_t*>(gsq);
    int np = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) np += __popcll(pm[w]);
    const int rounds = 2 * np > cap ? 2 : 1;  // each half of the list holds at most 256 voxels
    const int mid = rounds == 2 ? n / 2 : n;
    if (t < 6) qn[t] = 0;
    __syncthreads();
    float acc[8];
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
#pragma unroll 1
        for (int r = 0; r < rounds; ++r) {
            const int lo = r == 0 ? 0 : mid, hi = r == 0 ? mid : n;
            int* cnt = qn + 2 * ax + r;
#pragma unroll 1
            for (int i = lo + t; i < hi; i += STAGE_THREADS) {
                const int v = list[i];
                if (!((pm[v >> 6] >> (v & 63)) & 1)) continue;
                const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
                const bool outside = tile[tile_index(x, y, z)] > 0.0f;
                const Diff6 D = line_diffs<ExactArith>(tile_line(tile, x, y, z, ax));
                int sb, sf;  // BD operands D0..D4, FD operands D5..D1
                xw::weno5_sign_pair(D.d[0], D.d[1], D.d[2], D.d[3], D.d[4], D.d[5], sb, sf);
                term[v] = 0u;
                // a derivative the norm clamps to zero, or a zero (flat line), adds nothing
                if (sb != 2 && (outside ? sb != -1 : sb != 1)) queue[atomicAdd(cnt, 1)] = uint16_t(v << 1);
                if (sf != 2 && (outside ? sf != 1 : sf != -1)) queue[atomicAdd(cnt, 1)] = uint16_t((v << 1) | 1);
            }
            __syncthreads();
            const int m = *cnt;
#pragma unroll 1
            for (int j = t; j < m; j += STAGE_THREADS) {
                const int e = queue[j];
                const int v = e >> 1;
                const bool fd = e & 1;
                const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
                const bool outside = tile[tile_index(x, y, z)] > 0.0f;
                const Diff6 D = line_diffs<ExactArith>(tile_line(tile, x, y, z, ax));
                float q[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) q[k] = fd ? D.d[5 - k] : D.d[k];  // FD: D5..D1, BD: D0..D4
                const float wv = ExactArith::weno5(q[0], q[1], q[2], q[3], q[4]);
                // dm enters as max(dm, 0) outside, min(dm, 0) inside; dp the other way
                const float c = fd ? (outside ? ref_min(wv, 0.0f) : ref_max(wv, 0.0f))
                                   : (outside ? ref_max(wv, 0.0f) : ref_min(wv, 0.0f));
                atomicMax(&term[v], __float_as_uint(ExactArith::mul(c, c)));
            }
            __syncthreads();
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int i = t + k * STAGE_THREADS;
            if (i < n) {
                const int v = list[i];
                if ((pm[v >> 6] >> (v & 63)) & 1) {
                    const float tv = __uint_as_float(term[v]);
                    acc[k] = ax == 0 ? tv : ExactArith::add(acc[k], tv);
                }
            }
        }
        __syncthreads();  // the next axis resets the terms
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int i = t + k * STAGE_THREADS;
        if (i < n) {
            const int v = list[i];
            if ((pm[v >> 6] >> (v & 63)) & 1) gsq[v] = acc[k];
        }
    }
    __syncthreads();
}

// ---- velocity --------------------------------------------------------------
// Value of the dense velocity grid at its index (a, b, c) (background outside).
__device__ __forceinline__ void dense_value(const FieldParams& f, int i, int j, int k, float out[3]) {
    const int a = i - f.dense_origin[0], b = j - f.dense_origin[1], c = k - f.dense_origin[2];
    if (a >= 0 && b >= 0 && c >= 0 && a < f.dense_dims[0] && b < f.dense_dims[1] && c < f.dense_dims[2]) {
        const float* p = f.dense + 3 * ((size_t(a) * f.dense_dims[1] + b) * f.dense_dims[2] + c);
        out[0] = __ldg(p); out[1] = __ldg(p + 1); out[2] = __ldg(p + 2);
    } else {
        out[0] = f.dense_background[0]; out[1] = f.dense_background[1]; out[2] = f.dense_background[2];
    }
}

// BoxSampler's `a + ValueT((b - a) * weight)` per component
// (tools/Interpolation.h:716-722): float difference, double product,
// rounded back to float, float sum.
__device__ __forceinline__ float box_lerp(float a, float b, double w) {
    return __fadd_rn(a, __double2float_rn(__dmul_rn(double(__fsub_rn(b, a)), w)));
}

// DiscreteField::operator()(xyz, t) at the world position of voxel ijk
// (map.applyMap, tools/LevelSetAdvect.h:482-483): worldToIndex into the
// velocity grid, then BoxSampler::sample (tools/Interpolation.h:714-762).
// Explicit round-to-nearest intrinsics keep it exact in every build unit.
__device__ inline void dense_trilinear(const FieldParams& f, int i, int j, int k, float out[3]) {
    const int ijk[3] = {i, j, k};
    int i0[3];
    double uvw[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double w = __dadd_rn(__dmul_rn(double(ijk[a]), f.ls_scale), f.ls_translation[a]);
        const double q = __dmul_rn(__dsub_rn(w, f.vel_translation[a]), f.vel_inv_scale);
        const double fl = floor(q);
        i0[a] = int(fl);
        uvw[a] = __dsub_rn(q, double(i0[a]));
    }
    float d[2][2][2][3];
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int z = 0; z < 2; ++z) dense_value(f, i0[0] + x, i0[1] + y, i0[2] + z, d[x][y][z]);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float a0 = box_lerp(box_lerp(d[0][0][0][c], d[0][0][1][c], uvw[2]),
                                  box_lerp(d[0][1][0][c], d[0][1][1][c], uvw[2]), uvw[1]);
        const float a1 = box_lerp(box_lerp(d[1][0][0][c], d[1][0][1][c], uvw[2]),
                                  box_lerp(d[1][1][0][c], d[1][1][1][c], uvw[2]), uvw[1]);
        out[c] = box_lerp(a0, a1, uvw[0]);
    }
}

__device__ __forceinline__ void eval_field(const FieldParams& f, int i, int j, int k, float t,
                                           float out[3]) {
    switch (f.kind) {
    case 0:  // GBLS_FIELD_CONSTANT
        out[0] = f.constant[0]; out[1] = f.constant[1]; out[2] = f.constant[2];
        break;
    case 1: {  // GBLS_FIELD_DENSE
        if (f.xform) {
            dense_trilinear(f, i, j, k, out);
        } else {  // aligned DiscreteField lookup
            dense_value(f, i, j, k, out);
        }
        break;
    }
    case 2: {  // GBLS_FIELD_DEFORMATION
        const unsigned ia = unsigned(i - f.tab_lo), ja = unsigned(j - f.tab_lo), ka = unsigned(k - f.tab_lo);
        if (f.tab && ia < unsigned(f.tab_n) && ja < unsigned(f.tab_n) && ka < unsigned(f.tab_n)) {
            // gbls_deformation with its sines read from the per-coordinate tables
            const float sx = f.tab[2 * ia], s2x = f.tab[2 * ia + 1];
            const float sy = f.tab[2 * ja], s2y = f.tab[2 * ja + 1];
            const float sz = f.tab[2 * ka], s2z = f.tab[2 * ka + 1];
            const float u = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(2.0f, sx), sx), s2y), s2z);
            const float v = __fmul_rn(__fmul_rn(__fmul_rn(s2x, sy), sy), s2z);
            const float w = __fmul_rn(__fmul_rn(__fmul_rn(s2x, s2y), sz), sz);
            out[0] = __fmul_rn(u, f.amp);
            out[1] = -__fmul_rn(v, f.amp);
            out[2] = -__fmul_rn(w, f.amp);
        } else {
            gbls_deformation(i, j, k, t, f.domain, f.period, f.scale, out);
        }
        break;
    }
    default:  // GBLS_FIELD_ROTATION
        gbls_rotation(i, j, k, f.constant, f.omega, f.center, out);
        break;
    }
}

// ---- kernel arguments -------------------------------------------------------
struct RkArgs {
    int spatial;           // BiasedGradientScheme (GBLS_*_BIAS)
    int64_t nleaf;
    const uint64_t* keys;
    const int32_t* slot;
    const int32_t* nbr;
    Layout src;            // stencil buffer (masks of the current active set)
    const float* phin;     // buffer of the convex combination (same layout)
    float* out;            // result buffer (same layout)
    float dt, alpha, beta, gamma, t0;
    int has_phi;           // Nominator != 0
    int backward;          // velocity negated (t0 > t1)
    double invdx;          // 1/dx (parity: applied in double like applyIJT)
    float invdx_f;         // 1/dx in float (fast)
    FieldParams field;
    // batches (null for a single level set): per-instance running flag, dt,
    // substep start time and velocity field; instance = key >> 54
    const uint8_t* inst_run;
    const float* inst_dt;
    const float* inst_t0;
    const FieldParams* inst_field;
    int copy_done;         // the stage's output becomes the result: copy finished instances
    double dt64;           // FP64 instance: the substep length in double
    int parts;             // CTAs per leaf (exact kernel; 0 or 1: one): CTA b takes leaf b / parts
                           // and every parts-th group of STENCIL_THREADS active voxels from b % parts
};

struct NormArgs {
    int spatial;            // tracker BiasedGradientScheme
    int64_t nleaf;
    const int32_t* slot;
    const int32_t* nbr;
    Layout src;             // stencil buffer and its layout
    Layout phi;             // convex-combination buffer and its layout
    const uint64_t* pmask;  // [slots*8] voxels to update
    float* out_vals;
    uint64_t* out_amask;
    uint64_t* out_smask;
    int32_t* out_count;     // [nleaf] active voxels after the pass
    float alpha, beta, gamma, mdt, invdx;
    int has_phi;
    int trim;               // TrimMode bits: 1 interior, 2 exterior
    int copy_only;          // 1: value = staged value (relayout / trim only)
    int carry;              // 1: active voxels outside pmask stay active unchanged
                            // 0: they become inactive (erosion relayout)
    unsigned long long* acc;  // [2] += voxels processed, voxels written (may be null)
    const uint64_t* keys;     // batches: leaf keys (instance = key >> 54)
    const uint8_t* inst_run;  // batches: finished instances are copied through
    double mdt64, invdx64;    // FP64 instance: mDt and 1/dx in double
};

struct CflArgs {
    int64_t nleaf;
    const uint64_t* keys;
    const int32_t* slot;
    const uint64_t* amask;
    float t0;
    FieldParams field;
    unsigned int* max_bits;  // float bits of max |v|^2 (values >= 0); [instances] for batches
    const unsigned long long* nleaf_dev;  // when set: the leaf count is min(nleaf, *nleaf_dev)
    float* part;             // single level set: per-leaf maxima [nleaf] (scratch)
    const uint8_t* inst_run;
    const float* inst_t0;
    const FieldParams* inst_field;
};

// ---- kernels ----------------------------------------------------------------
constexpr int STENCIL_THREADS = STAGE_THREADS;

// list[rank] = voxel for every set bit of m[8] (thread t handles bit t of
// each word); returns the number of set bits.
__device__ __forceinline__ int build_list(uint16_t* list, const uint64_t* m) {
    const int t = threadIdx.x;
    const uint64_t low = (uint64_t(1) << t) - 1;
    int base = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint64_t w = m[k];
        if ((w >> t) & 1) list[base + __popcll(w & low)] = uint16_t((k << 6) | t);
        base += __popcll(w);
    }
    return base;
}

// One TVD-RK stage of LevelSetAdvection::Advect::euler<N,D>
// (tools/LevelSetAdvect.h:543-572): for every active voxel
//   a = phi_c - dt * (v . GradientBiased<HJWENO5>(phi))
//   out = N ? alpha*phin + beta*a : a
// MINB: the minimum resident CTAs per SM the compiler must allow (register
// budget; 0 gives none), one of the launch shapes the autotuner chooses among.
template <class A, int MINB = 0>
__global__ void __launch_bounds__(STENCIL_THREADS, MINB) rk_stage_kernel(const RkArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ uint16_t list[LEAF_VOX];
    __shared__ float vtab[6][8];
    __shared__ FieldParams sf;
    const int parts = a.parts > 1 ? a.parts : 1;
    const int64_t l = parts > 1 ? int64_t(blockIdx.x) / parts : int64_t(blockIdx.x);
    const int part = parts > 1 ? int(blockIdx.x % unsigned(parts)) : 0;
    const int first = part * STENCIL_THREADS, stride = parts * STENCIL_THREADS;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    const uint64_t key = a.keys[l];
    float dt = a.dt, t0 = a.t0;
    if (a.inst_run) {
        const uint32_t inst = key_instance(key);
        if (!a.inst_run[inst]) {
            if (a.copy_done) {  // keep a finished instance's values in the result buffer
                int n = 0;
                for (int w = 0; w < 8; ++w) n += __popcll(a.src.amask[size_t(s) * 8 + w]);
                for (int i = first + threadIdx.x; i < n; i += stride)
                    a.out[size_t(s) * LEAF_VOX + i] = a.src.vals[size_t(s) * LEAF_VOX + i];
            }
            return;
        }
        dt = a.inst_dt[inst];
        t0 = a.inst_t0[inst];
        if (threadIdx.x == 0) sf = a.inst_field[inst];
    } else if (threadIdx.x == 0) {
        sf = a.field;
    }
    stage_masks(st, a.src, s, a.nbr + 6 * l, nullptr, nullptr);
    load_tile(tile, st, a.gamma);
    const int n = build_list(list, st.am[0]);
    __syncthreads();
    int ox, oy, oz;
    key_origin(key, ox, oy, oz);
    // deformation field: the leaf's 8 sines per axis and function, staged once
    const bool tabbed = sf.kind == 2 && sf.tab && ox - sf.tab_lo >= 0 && oy - sf.tab_lo >= 0 &&
                        oz - sf.tab_lo >= 0 && ox + 8 - sf.tab_lo <= sf.tab_n &&
                        oy + 8 - sf.tab_lo <= sf.tab_n && oz + 8 - sf.tab_lo <= sf.tab_n;
    if (tabbed) {
        if (threadIdx.x < 48) {
            const int ax = threadIdx.x >> 4, fn = (threadIdx.x >> 3) & 1, q = threadIdx.x & 7;
            const int o = ax == 0 ? ox : ax == 1 ? oy : oz;
            vtab[ax * 2 + fn][q] = sf.tab[2 * (o + q - sf.tab_lo) + fn];
        }
        __syncthreads();
    }
    for (int i = first + threadIdx.x; i < n; i += stride) {
        const int v = list[i];
        const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
        float vel[3];
        if (tabbed) {
            // gbls_deformation with the staged sines (same operations)
            const float sx = vtab[0][x], s2x = vtab[1][x], sy = vtab[2][y], s2y = vtab[3][y];
            const float sz = vtab[4][z], s2z = vtab[5][z];
            const float u = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(2.0f, sx), sx), s2y), s2z);
            const float w = __fmul_rn(__fmul_rn(__fmul_rn(s2x, sy), sy), s2z);
            const float q = __fmul_rn(__fmul_rn(__fmul_rn(s2x, s2y), sz), sz);
            vel[0] = __fmul_rn(u, sf.amp);
            vel[1] = -__fmul_rn(w, sf.amp);
            vel[2] = -__fmul_rn(q, sf.amp);
        } else if (sf.kind == 4) {  // GBLS_FIELD_HOST_SAMPLED: rank i of leaf l
            const float* q = sf.sampled + 3 * (sf.prefix[l] + i);
            vel[0] = q[0]; vel[1] = q[1]; vel[2] = q[2];
        } else {
            eval_field(sf, ox + x, oy + y, oz + z, t0, vel);
        }
        if (a.backward) { vel[0] = -vel[0]; vel[1] = -vel[1]; vel[2] = -vel[2]; }
        float dot = 0.0f;
        if (IsExact<A>::value && a.spatial == 4) {
            // one WENO5 call site in a loop that is not unrolled (instruction
            // cache); dot = (v0 g0 + v1 g1) + v2 g2 in that order
#pragma unroll 1
            for (int ax = 0; ax < 3; ++ax) {
                const float v = ax == 0 ? vel[0] : ax == 1 ? vel[1] : vel[2];
                const float g = A::ijt(line_upwind<A>(tile_line(tile, x, y, z, ax), v < 0.0f), a.invdx, a.invdx_f);
                const float m = A::mul(v, g);
                dot = ax == 0 ? m : A::add(dot, m);
            }
        } else {
            float g[3];
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                const Line7 L = tile_line(tile, x, y, z, ax);
                g[ax] = A::ijt(scheme_upwind<A>(L, vel[ax] < 0.0f, a.spatial), a.invdx, a.invdx_f);
            }
            dot = A::add(A::add(A::mul(vel[0], g[0]), A::mul(vel[1], g[1])), A::mul(vel[2], g[2]));
        }
        const float c = tile[tile_index(x, y, z)];
        const float r = A::sub(c, A::mul(dt, dot));
        float o = r;
        if (a.has_phi) {
            const float p = a.phin[size_t(s) * LEAF_VOX + i];
            o = A::add(A::mul(a.alpha, p), A::mul(a.beta, r));
        }
        a.out[size_t(s) * LEAF_VOX + i] = o;
    }
}

// One stage of LevelSetTracker::Normalizer::euler<N,D>
// (tools/LevelSetTracker.h:623-676) over the voxels of pmask (the masked
// form :661-670 when `carry` keeps the other active voxels), optionally
// followed by Trim (tools/LevelSetTracker.h:473-506), writing the result in
// the layout of the surviving active set.  Voxels visited: pmask | active.
template <class A, int MINB = 0>
__global__ void __launch_bounds__(STENCIL_THREADS, MINB) normalize_kernel(const NormArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ float res[LEAF_VOX];
    __shared__ uint16_t list[LEAF_VOX];
    __shared__ uint8_t flag[LEAF_VOX];  // bit 0: active after the pass, bit 1: negative
    __shared__ uint64_t pm[8], um[8], fin[8], fsg[8], phm[8];
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
        if (a.has_phi) phm[t] = a.phi.amask[size_t(s) * 8 + t];
    }
    load_tile(tile, st, a.gamma);
    __syncthreads();
    const int n = build_list(list, um);
    __syncthreads();
    const bool exact_hj = IsExact<A>::value && a.spatial == 4 && !a.copy_only;
    if constexpr (IsExact<A>::value) {
        // the Godunov norms first, into res (each voxel's own slot, which the
        // loop below reads before it writes the voxel's result there); the
        // work list reuses the staging records, dead once the tile is loaded
        __shared__ int gqn[6];
        if (exact_hj)
            godunov_exact_leaf(tile, list, n, pm, res, reinterpret_cast<uint16_t*>(&st.rec[0][0]),
                               int(sizeof(st.rec) / sizeof(uint16_t)), gqn);
    }
    const float g = a.gamma;
    for (int i = t; i < n; i += STENCIL_THREADS) {
        const int v = list[i];
        const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
        const float phi0 = tile[tile_index(x, y, z)];
        float val = phi0;
        const uint64_t bit = uint64_t(1) << (v & 63);
        if (!(pm[v >> 6] & bit)) {
            // active voxel outside the processed set
            res[v] = val;
            flag[v] = uint8_t((carry ? 1 : 0) | (val < 0.0f ? 2 : 0));
            continue;
        }
        if (!a.copy_only) {
            float nsq;
            if (exact_hj) {
                nsq = res[v];
            } else {
                float up[3], down[3];
#pragma unroll
                for (int ax = 0; ax < 3; ++ax) {
                    const Line7 L = tile_line(tile, x, y, z, ax);
                    up[ax] = scheme_fd<A>(L, a.spatial);
                    down[ax] = scheme_bd<A>(L, a.spatial);
                }
                nsq = godunov<A>(phi0 > 0.0f, down, up);
            }
            float vv = A::div(phi0, A::add(A::sqrt(A::add(A::mul(phi0, phi0), nsq)), 1e-8f));
            vv = A::sub(phi0, A::mul(A::mul(a.mdt, vv), A::sub(A::mul(A::sqrt(nsq), a.invdx), 1.0f)));
            if (a.has_phi) {
                const int w = v >> 6, b = v & 63;
                float p;
                if ((phm[w] >> b) & 1) {
                    int rank = __popcll(phm[w] & (bit - 1));
                    for (int k = 0; k < w; ++k) rank += __popcll(phm[k]);
                    p = a.phi.vals[size_t(s) * LEAF_VOX + rank];
                } else {
                    p = ((a.phi.smask[size_t(s) * 8 + w] >> b) & 1) ? -g : g;
                }
                vv = A::add(A::mul(a.alpha, p), A::mul(a.beta, vv));
            }
            val = vv;
        }
        bool act = true, neg = val < 0.0f;
        if ((trim & 1) && val <= -g) { act = false; neg = true; }
        else if ((trim & 2) && val >= g) { act = false; neg = false; }
        res[v] = val;
        flag[v] = uint8_t((act ? 1 : 0) | (neg ? 2 : 0));
    }
    __syncthreads();
    // gather the flags of the visited voxels into the output masks with ballots
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
    // packed output in the layout of fin: thread t writes bit t of each word
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

// Max of |v|^2 over the active voxels (LevelSetAdvection::Advect::sampleField,
// tools/LevelSetAdvect.h:447-455): Vec3f::lengthSqr in float, no contraction.
__global__ void cfl_max_kernel(const __grid_constant__ CflArgs a);

}  // namespace gbls
