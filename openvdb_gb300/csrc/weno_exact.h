// The reference's WENO5 (math/FiniteDifference.h:301-321) evaluated bit for
// bit without FP64 arithmetic on the fast path.
//
// The reference computes the weights in double from float differences and
// rounds twice: the numerator to float, then the quotient (in double) to
// float.  GB300 runs FP64 at a small fraction of its FP32 rate, so this
// header carries every double-typed quantity of the formula as a double-word
// float pair (hi + lo, about 48 significant bits; the error-free sum and
// product transformations and the double-word algorithms of Joldes, Muller
// and Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44(2), 2017: algorithms 4, 9, 12 and 17,
// and cascaded sums of error-free terms), together with an upper bound of
// its distance from the reference's double value.  When the interval of
// that width around the pair holds no float rounding boundary, the float
// the reference produces is known exactly; otherwise (about one evaluation
// in 5000) the caller evaluates the reference formula in FP64.  The
// float-typed sub-expressions of the reference (v1-2*v2+v3 and its square,
// v1-4*v2, v2-v4 and its square, 4*v4) are evaluated in float exactly as
// there.
//
// The evaluation is written once over a lane type: float (host and
// device) and, on the device, float2 with the packed FP32x2 operations
// (FADD2 / FMUL2 / FFMA2), which evaluate two voxels per instruction.
// Every add, multiply and fused multiply-add is correctly rounded, never
// contracted.  The reciprocal is the only operation that differs between
// host (correctly rounded) and device (the hardware approximation, within
// one ulp); it only seeds the divisions, whose error bound allows for it.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define GBLS_XHD __host__ __device__ __forceinline__
#define GBLS_XD __device__ __forceinline__
#else
#define GBLS_XHD inline
#endif

namespace gbls {
namespace xw {

// ---- float lanes --------------------------------------------------------
GBLS_XHD float add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
GBLS_XHD float sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
GBLS_XHD float mul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
GBLS_XHD float fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}
GBLS_XHD float rcp(float a) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
#else
    return 1.0f / a;
#endif
}
GBLS_XHD float neg(float a) { return -a; }
GBLS_XHD float vabs(float a) { return std::fabs(a); }
GBLS_XHD float splat(float c, float) { return c; }
GBLS_XHD uint32_t fbits(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}
GBLS_XHD float bitsf(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}

// ---- float2 lanes (device) ----------------------------------------------
// Packed FP32x2 instructions written as PTX with an explicit rounding
// modifier, which ptxas never fuses into a multiply-add: each operation is
// rounded once, as the reference's float operations are.
#if defined(__CUDACC__)
GBLS_XD unsigned long long as_b64(float2 a) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
GBLS_XD float2 as_f2(unsigned long long r) {
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
GBLS_XD float2 add(float2 a, float2 b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(as_b64(a)), "l"(as_b64(b)));
    return as_f2(r);
}
GBLS_XD float2 sub(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(as_b64(a)), "l"(as_b64(b)));
    return as_f2(r);
}
GBLS_XD float2 mul(float2 a, float2 b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(as_b64(a)), "l"(as_b64(b)));
    return as_f2(r);
}
GBLS_XD float2 fma(float2 a, float2 b, float2 c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(as_b64(a)), "l"(as_b64(b)), "l"(as_b64(c)));
    return as_f2(r);
}
GBLS_XD float2 rcp(float2 a) { return make_float2(rcp(a.x), rcp(a.y)); }
GBLS_XD float2 neg(float2 a) { return make_float2(-a.x, -a.y); }
GBLS_XD float2 vabs(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
GBLS_XD float2 splat(float c, float2) { return make_float2(c, c); }
#endif

// A double-word number h + l with |l| <= ulp(h)/2 (h = fl(h + l)).
template <class V>
struct DW {
    V h, l;
};

// Error-free transformations.
template <class V>
GBLS_XHD DW<V> two_sum(V a, V b) {
    const V s = add(a, b);
    const V bb = sub(s, a);
    return {s, add(sub(a, sub(s, bb)), sub(b, bb))};
}
template <class V>
GBLS_XHD DW<V> fast_two_sum(V a, V b) {  // |a| >= |b| or a == 0
    const V s = add(a, b);
    return {s, sub(b, sub(s, a))};
}
template <class V>
GBLS_XHD DW<V> two_prod(V a, V b) {
    const V p = mul(a, b);
    return {p, fma(a, b, neg(p))};
}

// Double-word operations; relative error bounds in units of u^2, u = 2^-24.
template <class V>
GBLS_XHD DW<V> dw_add_f(DW<V> x, V y) {  // algorithm 4: 2u^2
    const DW<V> s = two_sum(x.h, y);
    return fast_two_sum(s.h, add(x.l, s.l));
}
template <class V>
GBLS_XHD DW<V> dw_mul_f(DW<V> x, V y) {  // algorithm 9: 2u^2
    const DW<V> c = two_prod(x.h, y);
    return fast_two_sum(c.h, fma(x.l, y, c.l));
}
template <class V>
GBLS_XHD DW<V> dw_mul(DW<V> x, DW<V> y) {  // algorithm 12: 4u^2
    const DW<V> c = two_prod(x.h, y.h);
    const V t = fma(x.h, y.l, mul(x.l, y.l));
    return fast_two_sum(c.h, add(c.l, fma(x.l, y.h, t)));
}
// algorithm 17 with th = xh * r, r an approximate reciprocal of yh (within
// one ulp; th within two ulps of xh / yh, which the correction absorbs):
// 15u^2 + O(u^3)
template <class V>
GBLS_XHD DW<V> dw_div(DW<V> x, DW<V> y, V r) {
    const V th = mul(x.h, r);
    const DW<V> p = dw_mul_f(y, th);
    const V d = add(sub(x.h, p.h), sub(x.l, p.l));
    return fast_two_sum(th, mul(d, r));
}
// Sum of three double words by a cascade of two error-free sums of the high
// parts, the low parts and the sum errors added in float: absolute error
// within about 2u^2 (|a| + |b| + |c|).
template <class V>
GBLS_XHD DW<V> dw_sum3(DW<V> a, DW<V> b, DW<V> c) {
    const DW<V> s = two_sum(a.h, b.h);
    const DW<V> t = two_sum(s.h, c.h);
    const V low = add(add(add(a.l, b.l), c.l), add(s.l, t.l));
    return fast_two_sum(t.h, low);
}
template <class V>
GBLS_XHD DW<V> dw_scale(DW<V> x, V s) { return {mul(x.h, s), mul(x.l, s)}; }  // s a power of two

// Double constants of the formula as double-word pairs (hi = float(c),
// lo = float(c - hi), each within u^2 |c| of the double), evaluated by the
// compiler.
constexpr double kC = 13.0 / 12.0, kEps = 1.0e-6 * double(0.01f);
constexpr float kC_h = float(kC), kC_l = float(kC - double(kC_h));
constexpr float kEps_h = float(kEps), kEps_l = float(kEps - double(kEps_h));
constexpr float kG1_h = float(0.1), kG1_l = float(0.1 - double(kG1_h));
constexpr float kG2_h = float(0.6), kG2_l = float(0.6 - double(kG2_h));
constexpr float kG3_h = float(0.3), kG3_l = float(0.3 - double(kG3_h));
template <class V>
GBLS_XHD DW<V> dw_const(float h, float l, V like) {
    return {splat(h, like), splat(l, like)};
}

// The float that double value t rounds to, when every value within e of
// the pair t rounds to t.h.  t.h = fl(t.h + t.l), so t.h + t.l lies within
// half a float spacing of t.h; the condition |t.l| + e < half the spacing
// keeps the whole interval inside t.h's rounding interval, ties excluded.
// Half the spacing of a normal float of biased exponent E is 2^(E-151):
// the bits (E - 24) << 23.  Below a power of two the spacing halves, so
// there the smaller half-spacing applies.  Values below 2^-100 and
// non-finite values are left to the caller.
GBLS_XHD bool rounds_to_hi(float h, float l, float e) {
    const uint32_t b = fbits(h) & 0x7fffffffu;
    if (b < 0x0d800000u || b >= 0x7f800000u) return false;
    const uint32_t ex = b & 0x7f800000u;
    float hs = bitsf(ex - (24u << 23));
    if (b == ex) hs = mul(hs, 0.5f);  // a power of two
    return add(vabs(l), e) < hs;
}
// Lane masks (bit k for lane k).
GBLS_XHD unsigned round_mask(DW<float> t, float e) { return rounds_to_hi(t.h, t.l, e) ? 1u : 0u; }
GBLS_XHD unsigned zero_mask(float a, float b, float c, float d, float e) {
    return (a == 0.0f && b == 0.0f && c == 0.0f && d == 0.0f && e == 0.0f) ? 1u : 0u;
}
GBLS_XHD float select_lanes(unsigned m, float a, float b) { return (m & 1u) ? a : b; }
#if defined(__CUDACC__)
GBLS_XD unsigned round_mask(DW<float2> t, float2 e) {
    return (rounds_to_hi(t.h.x, t.l.x, e.x) ? 1u : 0u) | (rounds_to_hi(t.h.y, t.l.y, e.y) ? 2u : 0u);
}
GBLS_XD unsigned zero_mask(float2 a, float2 b, float2 c, float2 d, float2 e) {
    return zero_mask(a.x, b.x, c.x, d.x, e.x) | (zero_mask(a.y, b.y, c.y, d.y, e.y) << 1);
}
GBLS_XD float2 select_lanes(unsigned m, float2 a, float2 b) {  // lane k from a where bit k is set
    return make_float2((m & 1u) ? a.x : b.x, (m & 2u) ? a.y : b.y);
}
#endif

// WENO5 of the reference on every lane.  Returns the mask of lanes whose
// result `out` is the reference's float; the other lanes need the FP64
// formula.
template <class V>
GBLS_XHD unsigned weno5(V v1, V v2, V v3, V v4, V v5, V& out) {
    const V two = splat(2.0f, v1), four = splat(4.0f, v1), five = splat(5.0f, v1);
    const V zero = splat(0.0f, v1), quarter = splat(0.25f, v1);
    // float-typed sub-expressions, as the reference evaluates them
    const V t1 = add(sub(v1, mul(two, v2)), v3), pa1 = mul(t1, t1);
    const V t2 = add(sub(v2, mul(two, v3)), v4), pa2 = mul(t2, t2);
    const V t3 = add(sub(v3, mul(two, v4)), v5), pa3 = mul(t3, t3);
    const V w1 = sub(v1, mul(four, v2));
    const V u2 = sub(v2, v4), pb2 = mul(u2, u2);
    const V f4 = mul(four, v4);
    // u1 = double(w1) + 3.0*v3; u3 = (3.0*v3 - double(4*v4)) + v5 (double sums)
    const DW<V> v3x3 = two_prod(splat(3.0f, v1), v3);
    const DW<V> u1 = dw_add_f(v3x3, w1);
    const DW<V> i3 = dw_add_f(v3x3, neg(f4));
    const DW<V> u3 = dw_add_f(i3, v5);
    const DW<V> ub1 = dw_scale(dw_mul(u1, u1), quarter), ub3 = dw_scale(dw_mul(u3, u3), quarter);
    // d = (C*pa + 0.25*pb) + eps, every term >= 0
    const DW<V> C = dw_const(kC_h, kC_l, v1), EPS = dw_const(kEps_h, kEps_l, v1);
    const DW<V> d1 = dw_sum3(dw_mul_f(C, pa1), ub1, EPS);
    const DW<V> d2 = dw_sum3(dw_mul_f(C, pa2), DW<V>{mul(quarter, pb2), zero}, EPS);
    const DW<V> d3 = dw_sum3(dw_mul_f(C, pa3), ub3, EPS);
    const DW<V> D1 = dw_mul(d1, d1), D2 = dw_mul(d2, d2), D3 = dw_mul(d3, d3);
    const V r1 = rcp(D1.h), r2 = rcp(D2.h), r3 = rcp(D3.h);
    const DW<V> A1 = dw_div(dw_const(kG1_h, kG1_l, v1), D1, r1);
    const DW<V> A2 = dw_div(dw_const(kG2_h, kG2_l, v1), D2, r2);
    const DW<V> A3 = dw_div(dw_const(kG3_h, kG3_l, v1), D3, r3);
    // p1 = (2v1 - 7v2) + 11v3, p2 = (5v3 - v2) + 2v4, p3 = (2v3 + 5v4) - v5;
    // each product is exact in double and as a pair
    const DW<V> p1 = dw_sum3(two_prod(splat(-7.0f, v1), v2), DW<V>{mul(two, v1), zero},
                             two_prod(splat(11.0f, v1), v3));
    const DW<V> p2 = dw_sum3(two_prod(five, v3), DW<V>{neg(v2), zero}, DW<V>{mul(two, v4), zero});
    const DW<V> p3 = dw_sum3(two_prod(five, v4), DW<V>{mul(two, v3), zero}, DW<V>{neg(v5), zero});
    const DW<V> num = dw_sum3(dw_mul(A1, p1), dw_mul(A2, p2), dw_mul(A3, p3));

    // Error bound of num against the reference's double.  Relative error of
    // A_k: 2^-40 covers the double-word chain and the reference's own
    // roundings (about 2^-42.4 and 2^-49).  An error du in u moves d by
    // 0.25*2|u|du, and A by twice that relative to d: for u1 (one sum, du
    // within 2^-46 |u1|) and for the |u3| part of u3 that stays below
    // 2^-43 because d >= 0.25 u^2; the inner sum of u3, 3v3 - 4v4, errs by
    // up to 2^-46 of its own magnitude, which can exceed |u3| by far, so
    // A3 takes 2^-45 |u3| |3v3 - 4v4| / d3 more (a factor of two spare).
    // p_k: the reference's products are exact, its two sums err by up to
    // 2^-52 of T_k = sum of |terms|, the cascade by 2^-47 T_k; the sum of
    // the products A_k p_k (cascade) by 2^-46 of S = sum |A_k p_k|, which
    // the 2^-40 terms cover.  The total, doubled, is e_num.
    const V q3 = mul(mul(mul(vabs(u3.h), vabs(i3.h)), splat(0x1p-45f, v1)), mul(d3.h, r3));
    const V e40 = splat(0x1p-40f, v1), e46 = splat(0x1p-46f, v1);
    const V e3 = add(e40, q3);
    const V T1 = add(add(vabs(mul(two, v1)), vabs(mul(splat(7.0f, v1), v2))), vabs(mul(splat(11.0f, v1), v3)));
    const V T2 = add(add(vabs(mul(five, v3)), vabs(v2)), vabs(mul(two, v4)));
    const V T3 = add(add(vabs(mul(two, v3)), vabs(mul(five, v4))), vabs(v5));
    const V a1 = vabs(A1.h), a2 = vabs(A2.h), a3 = vabs(A3.h);
    const V s1 = fma(vabs(p1.h), e40, mul(T1, e46));
    const V s2 = fma(vabs(p2.h), e40, mul(T2, e46));
    const V s3 = fma(vabs(p3.h), e3, mul(T3, e46));
    const V e_num = mul(two, fma(a1, s1, fma(a2, s2, mul(a3, s3))));
    unsigned ok = round_mask(num, e_num);
    const V F = num.h;  // static_cast<float>(num)

    // den = 6 * ((A1 + A2) + A3), positive; its relative uncertainty is the
    // A_k's weighted by A_k / sum, plus the sums and the product
    const V six = splat(6.0f, v1);
    const DW<V> den = dw_mul_f(dw_sum3(A1, A2, A3), six);
    const V rd = rcp(den.h);
    const V e42 = splat(0x1p-42f, v1);
    const V e_den = add(mul(fma(a1, e40, fma(a2, e40, mul(a3, e3))), mul(six, rd)), e42);
    const DW<V> q = dw_div(DW<V>{F, zero}, den, rd);
    const V e_q = mul(mul(two, vabs(q.h)), add(e_den, e42));
    ok &= round_mask(q, e_q);
    out = q.h;
    // five zero operands: the reference's result is the signed zero of
    // ((A1 p1 + A2 p2) + A3 p3) with every A_k > 0; the same IEEE sign
    // rules give it in float
    const unsigned z = zero_mask(v1, v2, v3, v4, v5);
    if (z) {
        const V z1 = add(sub(mul(two, v1), mul(splat(7.0f, v1), v2)), mul(splat(11.0f, v1), v3));
        const V z2 = add(sub(mul(five, v3), v2), mul(two, v4));
        const V z3 = sub(add(mul(two, v3), mul(five, v4)), v5);
        out = select_lanes(z, add(add(z1, z2), z3), out);
        ok |= z;
    }
    return ok;
}

// Vec3d(g) * invdx (double) rounded to float (GradientBiased's applyIJT,
// math/Operators.h:838-845) for a float lane, or false when undecided.
GBLS_XHD bool ijt(float g, DW<float> invdx, float& out) {
    if (g == 0.0f) {
        out = g;
        return true;
    }
    const DW<float> p = dw_mul_f(invdx, g);
    if (!rounds_to_hi(p.h, p.l, mul(vabs(p.h), 0x1p-44f))) return false;
    out = p.h;
    return true;
}

}  // namespace xw
}  // namespace gbls
