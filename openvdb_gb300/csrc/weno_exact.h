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
// double-word arithmetic", ACM TOMS 44(2), 2017: algorithms 4, 9, 10 and 17,
// a squaring without the low parts' square, and cascaded sums of error-free
// terms), together with an upper bound of
// its distance from the reference's double value.  When the interval of
// that width around the pair holds no float rounding boundary, the float
// the reference produces is known exactly; otherwise (about one evaluation
// in 5000) the caller evaluates the reference formula in FP64.  The
// float-typed sub-expressions of the reference (v1-2*v2+v3 and its square,
// v1-4*v2, v2-v4 and its square, 4*v4) are evaluated in float exactly as
// there.
//
// Host and device evaluate the same operations: every add, multiply and
// fused multiply-add is correctly rounded and never contracted (explicit
// round-to-nearest intrinsics on the device, -ffp-contract=off on the
// host).  The reciprocal is the only operation that differs between host
// (correctly rounded) and device (the hardware approximation, within one
// ulp); it only seeds the divisions, whose error bound allows for it.  The
// evaluation is written over a lane type V (float here), the form a
// vectorised variant would take.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define GBLS_XHD __host__ __device__ __forceinline__
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
// The same pair before the final normalisation (|l| within about 2u |h|).
template <class V>
GBLS_XHD DW<V> dw_mul_f_un(DW<V> x, V y) {
    const DW<V> c = two_prod(x.h, y);
    return {c.h, fma(x.l, y, c.l)};
}
// x^2: h^2 = p + e exactly; t = fl(2hl + e) errs by at most u|2hl + e| <=
// 3u^2 h^2, the dropped l^2 is at most u^2 h^2, and |t| <= |p| makes the
// final sum exact: 4u^2
template <class V>
GBLS_XHD DW<V> dw_sqr(DW<V> x) {
    const DW<V> c = two_prod(x.h, x.h);
    return fast_two_sum(c.h, fma(x.h, add(x.l, x.l), c.l));
}
// x^2 / 4 as (x/2)^2, the halving exact: the same bound
template <class V>
GBLS_XHD DW<V> dw_sqr_quarter(DW<V> x) {
    const V hh = mul(x.h, splat(0.5f, x.h));
    const DW<V> c = two_prod(hh, hh);
    return fast_two_sum(c.h, fma(hh, x.l, c.l));
}
// algorithm 10 (no low-part product): about 7u^2, before the final
// normalisation (|l| within a few u |h|)
template <class V>
GBLS_XHD DW<V> dw_mul_lite_un(DW<V> x, DW<V> y) {
    const DW<V> c = two_prod(x.h, y.h);
    return {c.h, add(c.l, fma(x.l, y.h, mul(x.h, y.l)))};
}
// Algorithm 17 with th = xh * r, r an approximate reciprocal of yh (within
// one ulp; th within two ulps of xh / yh, which the correction absorbs):
// 15u^2 + O(u^3), returned before its final normalisation: the pair
// (th, d r) holds the value the normalised pair would, with |d r| up to
// about 8u |th| (th within two ulps of xh / yh, and x, y within u of their
// high parts), for callers that tolerate that.
// The product y th enters unnormalised: p.h = fl(yh th) is within a few
// ulps of xh, so xh - p.h stays exact (Sterbenz), and the low part is
// subtracted on its own.
template <class V>
GBLS_XHD DW<V> dw_div_un(DW<V> x, DW<V> y, V r) {
    const V th = mul(x.h, r);
    const DW<V> p = dw_mul_f_un(y, th);
    return {th, mul(add(sub(x.h, p.h), sub(x.l, p.l)), r)};
}
// Algorithm 17 (normalised) for a float numerator (x.l = 0), the same way.
template <class V>
GBLS_XHD DW<V> dw_div_f(V x, DW<V> y, V r) {
    const V th = mul(x, r);
    const DW<V> p = dw_mul_f_un(y, th);
    return fast_two_sum(th, mul(sub(sub(x, p.h), p.l), r));
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
// The cascade before the final normalisation (|l| within a few u |h| when
// the terms have one sign).
template <class V>
GBLS_XHD DW<V> dw_sum3_un(DW<V> a, DW<V> b, DW<V> c) {
    const DW<V> s = two_sum(a.h, b.h);
    const DW<V> t = two_sum(s.h, c.h);
    return {t.h, add(add(add(a.l, b.l), c.l), add(s.l, t.l))};
}
// The same cascade with float terms (low parts zero, not added).
template <class V>
GBLS_XHD DW<V> dw_sum3_f(DW<V> a, V b, DW<V> c) {
    const DW<V> s = two_sum(a.h, b);
    const DW<V> t = two_sum(s.h, c.h);
    return fast_two_sum(t.h, add(add(a.l, c.l), add(s.l, t.l)));
}
template <class V>
GBLS_XHD DW<V> dw_sum3_ff(DW<V> a, V b, V c) {
    const DW<V> s = two_sum(a.h, b);
    const DW<V> t = two_sum(s.h, c);
    return fast_two_sum(t.h, add(a.l, add(s.l, t.l)));
}

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
GBLS_XHD unsigned zero_mask(float a) { return a == 0.0f ? 1u : 0u; }
GBLS_XHD unsigned below_mask(float a, float b) { return a < b ? 1u : 0u; }
GBLS_XHD float vmax(float a, float b) { return a < b ? b : a; }
GBLS_XHD float select_lanes(unsigned m, float a, float b) { return (m & 1u) ? a : b; }

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
    // u3 by error-free sums: u3 = us.h + ub.h + ub.l + ua.l exactly, so the
    // pair (us.h + ub.h) is exact when ua.l and ub.l vanish.  When moreover the
    // nonzero terms 3v3, 4v4, v5 lie within 2^20 of one another, both of the
    // reference's double sums are exact (47 bits at most), so the pair is
    // the reference's u3 itself.
    const DW<V> i3 = two_sum(v3x3.h, neg(f4));
    const DW<V> us = two_sum(i3.h, v5);
    const DW<V> ua = two_sum(i3.l, v3x3.l);
    const DW<V> ub = two_sum(ua.h, us.l);
    const DW<V> u3 = two_sum(us.h, ub.h);
    const V m3a = vabs(v3x3.h), m3b = vabs(f4), m3c = vabs(v5);
    const V big = fmaxf(fmaxf(m3a, m3b), m3c);
    const V inf = splat(__builtin_huge_valf(), v1);
    const V small = fminf(fminf(m3a > 0.0f ? m3a : inf, m3b > 0.0f ? m3b : inf), m3c > 0.0f ? m3c : inf);
    const bool u3_exact = ua.l == 0.0f && ub.l == 0.0f && !(big > mul(small, splat(0x1p20f, v1)));
    const DW<V> ub1 = dw_sqr_quarter(u1), ub3 = dw_sqr_quarter(u3);
    // d = (C*pa + 0.25*pb) + eps, every term >= 0
    const DW<V> C = dw_const(kC_h, kC_l, v1), EPS = dw_const(kEps_h, kEps_l, v1);
    // (the products enter the cascades unnormalised: their low parts are
    // added on their own, and every term is >= 0)
    const DW<V> d1 = dw_sum3(dw_mul_f_un(C, pa1), ub1, EPS);
    const DW<V> d2 = dw_sum3_f(dw_mul_f_un(C, pa2), mul(quarter, pb2), EPS);
    const DW<V> d3 = dw_sum3(dw_mul_f_un(C, pa3), ub3, EPS);
    const DW<V> D1 = dw_sqr(d1), D2 = dw_sqr(d2), D3 = dw_sqr(d3);
    const V r1 = rcp(D1.h), r2 = rcp(D2.h), r3 = rcp(D3.h);
    // the weights stay unnormalised: they enter only products and sums
    const DW<V> A1 = dw_div_un(dw_const(kG1_h, kG1_l, v1), D1, r1);
    const DW<V> A2 = dw_div_un(dw_const(kG2_h, kG2_l, v1), D2, r2);
    const DW<V> A3 = dw_div_un(dw_const(kG3_h, kG3_l, v1), D3, r3);
    // p1 = (2v1 - 7v2) + 11v3, p2 = (5v3 - v2) + 2v4, p3 = (2v3 + 5v4) - v5;
    // each product is exact in double and as a pair
    const DW<V> p1 = dw_sum3_f(two_prod(splat(-7.0f, v1), v2), mul(two, v1), two_prod(splat(11.0f, v1), v3));
    const DW<V> p2 = dw_sum3_ff(two_prod(five, v3), neg(v2), mul(two, v4));
    const DW<V> p3 = dw_sum3_ff(two_prod(five, v4), mul(two, v3), neg(v5));
    const DW<V> num = dw_sum3(dw_mul_lite_un(A1, p1), dw_mul_lite_un(A2, p2), dw_mul_lite_un(A3, p3));

    // Error bound of num against the reference's double.  Relative error of
    // A_k: 2^-40 covers the double-word chain (u1 2u^2; its quarter square
    // 8u^2; d_k, a cascade of non-negative terms with unnormalised products,
    // 13u^2; D_k 30u^2; the division 15u^2 more: about 46u^2 = 2^-42.5) and
    // the reference's own roundings (about 2^-49).  An error du in u moves d by
    // 0.25*2|u|du, and A by twice that relative to d: for u1 (one sum, du
    // within 2^-46 |u1|) that stays below 2^-43 because d >= 0.25 u^2.
    // u3 is exact on both sides in the common case (u3_exact); otherwise
    // the reference's inner sum 3v3 - 4v4 and ours err by up to 2^-46 of
    // its magnitude, which can exceed |u3| by far, so A3 takes
    // 2^-45 |u3| |3v3 - 4v4| / d3 more (a factor of two spare).
    // p_k: the reference's products are exact, its two sums err by up to
    // 2^-52 of T_k = sum of |terms|, the cascade by 2^-47 T_k; the sum of
    // the products A_k p_k by 2^-44.2 of S = sum |A_k p_k| (14u^2, the
    // weights' low parts up to 8u of their high parts) and their cascade,
    // with unnormalised terms, by 2^-44.7 S, which the 2^-40 terms cover.
    // The total, doubled, is e_num.
    const V q3 = u3_exact ? zero : mul(mul(mul(vabs(u3.h), vabs(i3.h)), splat(0x1p-45f, v1)), mul(d3.h, r3));
    const V e40 = splat(0x1p-40f, v1), e46 = splat(0x1p-46f, v1);
    const V e3 = add(e40, q3);
    // (fused sums: within 2u of the exact T_k, which the doubling covers)
    const V T1 = fma(splat(11.0f, v1), vabs(v3), fma(splat(7.0f, v1), vabs(v2), add(vabs(v1), vabs(v1))));
    const V T2 = fma(two, vabs(v4), fma(five, vabs(v3), vabs(v2)));
    const V T3 = fma(five, vabs(v4), fma(two, vabs(v3), vabs(v5)));
    const V a1 = vabs(A1.h), a2 = vabs(A2.h), a3 = vabs(A3.h);
    const V s1 = fma(vabs(p1.h), e40, mul(T1, e46));
    const V s2 = fma(vabs(p2.h), e40, mul(T2, e46));
    const V s3 = fma(vabs(p3.h), e3, mul(T3, e46));
    const V e_num = mul(two, fma(a1, s1, fma(a2, s2, mul(a3, s3))));
    // Range: the bounds above are relative ones, which hold while the
    // weights and their low parts are normal floats.  D_k < 2^96 keeps A_k
    // above 2^-100 and its low part above 2^-124 (and the reciprocal seeds
    // normal); larger D_k (differences above about 2^20) are left to FP64.
    unsigned ok = round_mask(num, e_num) & below_mask(vmax(vmax(D1.h, D2.h), D3.h), splat(0x1p96f, v1));
    const V F = num.h;  // static_cast<float>(num)

    // den = 6 * ((A1 + A2) + A3), positive; its relative uncertainty is the
    // A_k's weighted by A_k / sum, plus the sums and the product
    const V six = splat(6.0f, v1);
    const DW<V> den = dw_mul_f_un(dw_sum3_un(A1, A2, A3), six);
    const V rd = rcp(den.h);
    const V e42 = splat(0x1p-42f, v1);
    const V e_den = add(mul(fma(a1, e40, fma(a2, e40, mul(a3, e3))), mul(six, rd)), e42);
    const DW<V> q = dw_div_f(F, den, rd);
    const V e_q = mul(mul(two, vabs(q.h)), add(e_den, e42));
    ok &= round_mask(q, e_q);
    out = q.h;
    // five zero operands (T1 = T3 = 0: sums of non-negative terms vanish
    // only when every term does): the reference's result is the signed
    // zero of ((A1 p1 + A2 p2) + A3 p3) with every A_k > 0; the same IEEE
    // sign rules give it in float
    const unsigned z = zero_mask(add(T1, T3));
    if (z) {
        const V z1 = add(sub(mul(two, v1), mul(splat(7.0f, v1), v2)), mul(splat(11.0f, v1), v3));
        const V z2 = add(sub(mul(five, v3), v2), mul(two, v4));
        const V z3 = sub(add(mul(two, v3), mul(five, v4)), v5);
        out = select_lanes(z, add(add(z1, z2), z3), out);
        ok |= z;
    }
    return ok;
}

// The sign of WENO5's result from its three candidate sums when they agree.
// The result is ((A1 p1 + A2 p2) + A3 p3) / (6 (A1 + A2 + A3)) with every
// A_k > 0 (and both roundings to float keep the sign), so when no p_k is
// negative the result is >= 0 (a zero of either sign included), and when
// no p_k is positive it is <= 0.  Each p_k is estimated in float by two
// fused multiply-adds, within 2u T_k of the exact sum (T_k = sum of
// |terms|), so an estimate beyond 4u T_k has the exact sum's sign; T_k = 0
// makes p_k exactly zero.  Returns +1 (result >= 0 for certain), -1
// (result <= 0 for certain), 2 (five zero operands: the result is a zero)
// or 0 (undecided).
// One candidate sum's estimate e and its T (T_k by fused multiply-adds:
// within 3u of the exact sums, so 4u T_k still exceeds the estimates' 2u
// error bound).
struct SignTerm {
    float e, t;
};
GBLS_XHD SignTerm sign_p1(float v1, float v2, float v3) {  // 2v1 - 7v2 + 11v3
    return {fma(11.0f, v3, fma(-7.0f, v2, mul(2.0f, v1))), fma(11.0f, vabs(v3), fma(7.0f, vabs(v2), mul(2.0f, vabs(v1))))};
}
GBLS_XHD SignTerm sign_p2(float v2, float v3, float v4) {  // 5v3 - v2 + 2v4
    return {fma(2.0f, v4, fma(5.0f, v3, -v2)), fma(5.0f, vabs(v3), fma(2.0f, vabs(v4), vabs(v2)))};
}
GBLS_XHD SignTerm sign_p3(float v3, float v4, float v5) {  // 2v3 + 5v4 - v5
    return {fma(-1.0f, v5, fma(5.0f, v4, mul(2.0f, v3))), fma(5.0f, vabs(v4), fma(2.0f, vabs(v3), vabs(v5)))};
}
GBLS_XHD int sign_of(SignTerm a, SignTerm b, SignTerm c) {
    const float m1 = mul(a.t, 0x1p-22f), m2 = mul(b.t, 0x1p-22f), m3 = mul(c.t, 0x1p-22f);
    const bool z1 = a.t == 0.0f, z2 = b.t == 0.0f, z3 = c.t == 0.0f;
    if (z1 && z2 && z3) return 2;
    const bool nonneg = (z1 || a.e > m1) && (z2 || b.e > m2) && (z3 || c.e > m3);
    const bool nonpos = (z1 || a.e < -m1) && (z2 || b.e < -m2) && (z3 || c.e < -m3);
    return nonneg ? 1 : nonpos ? -1 : 0;
}
GBLS_XHD int weno5_sign(float v1, float v2, float v3, float v4, float v5) {
    return sign_of(sign_p1(v1, v2, v3), sign_p2(v2, v3, v4), sign_p3(v3, v4, v5));
}
// weno5_sign of a line's backward operands (d0, d1, d2, d3, d4) and forward
// operands (d5, d4, d3, d2, d1) together.  The backward operands' second and
// third candidate sums, -d1 + 5d2 + 2d3 and 2d2 + 5d3 - d4, are the forward
// operands' third and second, so four estimates serve both (any estimate
// within 2u T of its sum certifies the same way).
GBLS_XHD void weno5_sign_pair(float d0, float d1, float d2, float d3, float d4, float d5, int& sb, int& sf) {
    const SignTerm y = sign_p2(d1, d2, d3), x = sign_p3(d2, d3, d4);
    sb = sign_of(sign_p1(d0, d1, d2), y, x);
    sf = sign_of(sign_p1(d5, d4, d3), x, y);
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
