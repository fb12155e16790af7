/*
 * gbls_fields.h -- analytic velocity fields shared by host and device code.
 *
 * The reference's advection takes any velocity functor evaluated at integer
 * voxel coordinates (tools/LevelSetAdvect.h:32-52, sample<Aligned> :472-493);
 * tools/VelocityFields.h:101-141 (EnrightField) and the vdb_tool LeVeque
 * functor (openvdb_cmd/vdb_tool/include/Tool.h:3436-3485) use std::sin.
 * std::sin and CUDA's sinf round differently, so a field evaluated on both
 * sides would break bit-parity.  The fields below therefore use a sin(pi x)
 * written here from its Taylor series (Horner form, reduced to
 * |pi r| <= pi/4) with only IEEE float add/multiply/divide/rint.  Every
 * operation is spelled out in a fixed order, so the host (compiled with
 * -ffp-contract=off, as all host code of this project is) and the device
 * (which uses the non-contracting __fadd_rn/__fmul_rn intrinsics) return the
 * same bits.  Accuracy: |error| < 2e-7 absolute on [-1, 1].
 */
#ifndef GBLS_FIELDS_H
#define GBLS_FIELDS_H

#include <math.h>

#if defined(__CUDACC__)
#define GBLS_HD __host__ __device__ __forceinline__
#else
#define GBLS_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define GBLS_FADD(a, b) __fadd_rn((a), (b))
#define GBLS_FSUB(a, b) __fsub_rn((a), (b))
#define GBLS_FMUL(a, b) __fmul_rn((a), (b))
#define GBLS_FDIV(a, b) __fdiv_rn((a), (b))
#else
#define GBLS_FADD(a, b) ((a) + (b))
#define GBLS_FSUB(a, b) ((a) - (b))
#define GBLS_FMUL(a, b) ((a) * (b))
#define GBLS_FDIV(a, b) ((a) / (b))
#endif

/* Taylor coefficients of sin(pi r) and cos(pi r) in powers of r. */
#define GBLS_S1 3.14159265358979323846f
#define GBLS_S3 -5.16771278004997003135f
#define GBLS_S5 2.55016403987734548746f
#define GBLS_S7 -0.59926452932079207689f
#define GBLS_S9 0.08214588661112822880f
#define GBLS_C2 -4.93480220054467930942f
#define GBLS_C4 4.05871212641676821814f
#define GBLS_C6 -1.33526276885458949614f
#define GBLS_C8 0.23533063035889320454f
#define GBLS_C10 -0.02580689139001406950f

GBLS_HD float gbls_sinpi_poly(float r) {
    const float r2 = GBLS_FMUL(r, r);
    float p = GBLS_S9;
    p = GBLS_FADD(GBLS_FMUL(p, r2), GBLS_S7);
    p = GBLS_FADD(GBLS_FMUL(p, r2), GBLS_S5);
    p = GBLS_FADD(GBLS_FMUL(p, r2), GBLS_S3);
    p = GBLS_FADD(GBLS_FMUL(p, r2), GBLS_S1);
    return GBLS_FMUL(p, r);
}

GBLS_HD float gbls_cospi_poly(float r) {
    const float r2 = GBLS_FMUL(r, r);
    float p = GBLS_C10;
    p = GBLS_FADD(GBLS_FMUL(p, r2), GBLS_C8);
    p = GBLS_FADD(GBLS_FMUL(p, r2), GBLS_C6);
    p = GBLS_FADD(GBLS_FMUL(p, r2), GBLS_C4);
    p = GBLS_FADD(GBLS_FMUL(p, r2), GBLS_C2);
    return GBLS_FADD(GBLS_FMUL(p, r2), 1.0f);
}

/* sin(pi x): x = q/2 + r with q = rint(2x), |r| <= 1/4 (both steps exact). */
GBLS_HD float gbls_sinpi(float x) {
    const float q = rintf(GBLS_FMUL(x, 2.0f));
    const float r = GBLS_FSUB(x, GBLS_FMUL(q, 0.5f));
    const int iq = ((int)q) & 3;
    if (iq == 0) return gbls_sinpi_poly(r);
    if (iq == 1) return gbls_cospi_poly(r);
    if (iq == 2) return -gbls_sinpi_poly(r);
    return -gbls_cospi_poly(r);
}

GBLS_HD float gbls_cospi(float x) {
    const float q = rintf(GBLS_FMUL(x, 2.0f));
    const float r = GBLS_FSUB(x, GBLS_FMUL(q, 0.5f));
    const int iq = ((int)q) & 3;
    if (iq == 0) return gbls_cospi_poly(r);
    if (iq == 1) return -gbls_sinpi_poly(r);
    if (iq == 2) return -gbls_cospi_poly(r);
    return gbls_sinpi_poly(r);
}

/* LeVeque's deformation field on the unit cube mapped to `domain` voxels,
 * modulated by cos(pi t / period) and scaled by `scale` voxels per time unit:
 *   u =  2 sin^2(pi x) sin(2 pi y) sin(2 pi z)
 *   v = -  sin(2 pi x) sin^2(pi y) sin(2 pi z)
 *   w = -  sin(2 pi x) sin(2 pi y) sin^2(pi z),   x = i/domain, ...         */
GBLS_HD void gbls_deformation(int i, int j, int k, float t, float domain, float period,
                              float scale, float out[3]) {
    const float x = GBLS_FDIV((float)i, domain);
    const float y = GBLS_FDIV((float)j, domain);
    const float z = GBLS_FDIV((float)k, domain);
    const float sx = gbls_sinpi(x), sy = gbls_sinpi(y), sz = gbls_sinpi(z);
    const float s2x = gbls_sinpi(GBLS_FMUL(x, 2.0f));
    const float s2y = gbls_sinpi(GBLS_FMUL(y, 2.0f));
    const float s2z = gbls_sinpi(GBLS_FMUL(z, 2.0f));
    const float amp = GBLS_FMUL(gbls_cospi(GBLS_FDIV(t, period)), scale);
    const float u = GBLS_FMUL(GBLS_FMUL(GBLS_FMUL(GBLS_FMUL(2.0f, sx), sx), s2y), s2z);
    const float v = GBLS_FMUL(GBLS_FMUL(GBLS_FMUL(s2x, sy), sy), s2z);
    const float w = GBLS_FMUL(GBLS_FMUL(GBLS_FMUL(s2x, s2y), sz), sz);
    out[0] = GBLS_FMUL(u, amp);
    out[1] = -GBLS_FMUL(v, amp);
    out[2] = -GBLS_FMUL(w, amp);
}

/* Rigid motion: constant + omega x (ijk - center). */
GBLS_HD void gbls_rotation(int i, int j, int k, const float c[3], const float omega[3],
                           const float center[3], float out[3]) {
    const float dx = GBLS_FSUB((float)i, center[0]);
    const float dy = GBLS_FSUB((float)j, center[1]);
    const float dz = GBLS_FSUB((float)k, center[2]);
    out[0] = GBLS_FADD(c[0], GBLS_FSUB(GBLS_FMUL(omega[1], dz), GBLS_FMUL(omega[2], dy)));
    out[1] = GBLS_FADD(c[1], GBLS_FSUB(GBLS_FMUL(omega[2], dx), GBLS_FMUL(omega[0], dz)));
    out[2] = GBLS_FADD(c[2], GBLS_FSUB(GBLS_FMUL(omega[0], dy), GBLS_FMUL(omega[1], dx)));
}

#if !defined(__CUDA_ARCH__)
/* tools::EnrightField<float>::operator()(xyz, time) (tools/VelocityFields.h:
 * 126-141): the reference's own formula with the C library's sinf / cosf, on
 * the host only (the device's sinf rounds differently), so fields of this
 * kind reach the device through GBLS_FIELD_HOST_SAMPLED.  xyz is the world
 * position in double, as the reference's map.applyMap returns it. */
static inline void gbls_enright(double x, double y, double z, float time, float out[3]) {
    const float pi = (float)3.141592653589793238462643383279502884e+00;
    const float phase = pi / 3.0f;
    const float Px = pi * (float)x, Py = pi * (float)y, Pz = pi * (float)z;
    const float tr = cosf(time * phase);
    const float a = sinf(2.0f * Py);
    const float b = -sinf(2.0f * Px);
    const float c = sinf(2.0f * Pz);
    const float sx = sinf(Px), sy = sinf(Py), sz = sinf(Pz);
    out[0] = tr * (2.0f * (sx * sx) * a * c);
    out[1] = tr * (b * (sy * sy) * c);
    out[2] = tr * (b * a * (sz * sz));
}
#endif

#endif /* GBLS_FIELDS_H */
