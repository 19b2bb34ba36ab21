// Device-side building blocks: shape functions, fixed-point accumulation,
// small 3x3 algebra and the constitutive updates.
#pragma once

#include <cstring>

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "mpm_internal.cuh"

namespace mpm {

// ---------------------------------------------------------------------------
// Shape functions.  Per direction the same closed forms as MakSf
// (module/shape_function.cpp:39-105): the linear hat 1 - |x - x_i|/dx with
// gradient +-1/dx, and the open-knot quadratic B-spline with its boundary
// pieces.  Tensor product ordering: x fastest, then y, then z
// (module/shape_function.cpp:107-110).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float rdiv(float a, float b, float inv_b) { return a * inv_b; }
__device__ __forceinline__ double rdiv(double a, double b, double) { return a / b; }

template <typename R, int O>
struct Axis {
    R w[O + 1];
    R dw[O + 1];
};

template <typename R>
__device__ __forceinline__ void axis_linear(R x, R xmin, R dx, R inv_dx, int ie, Axis<R, 1> &a) {
#pragma unroll
    for (int k = 0; k < 2; k++) {
        R xy = xmin + dx * (R)(ie + k);
        R r = x - xy;
        a.w[k] = (R)1 - rdiv(fabs(r), dx, inv_dx);
        // dN/dx by node: -1/dx for the lower node, +1/dx for the upper one.
        // MakSf (module/shape_function.cpp:39-50) takes the sign of r, which is
        // the same for a point inside the element; where rounding puts x on a
        // node plane beyond the element's end (common in FP32) the sign test
        // would give both nodes -1/dx.
        a.dw[k] = k == 0 ? -inv_dx : inv_dx;
    }
}

template <typename R>
__device__ __forceinline__ void axis_quadratic(R x, R xmin, R dx, R inv_dx, int ie, int nnc, Axis<R, 2> &a) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        int ncxy = ie + k;
        R xy = xmin + dx * (R)(ncxy - 2);
        R h = rdiv(x - xy, dx, inv_dx);
        R s1, s2, s3, d1, d2;
        if (ncxy == 0) {
            h -= (R)2;
            s1 = 1; s2 = -2; s3 = 1; d1 = 2; d2 = -2;
        } else if (ncxy == 1) {
            h -= (R)1;
            if (h <= (R)1) { s1 = -1.5; s2 = 2; s3 = 0; d1 = -3; d2 = 2; }
            else { s1 = 0.5; s2 = -2; s3 = 2; d1 = 1; d2 = -2; }
        } else if (ncxy == nnc - 1) {
            s1 = 1; s2 = 0; s3 = 0; d1 = 2; d2 = 0;
        } else if (ncxy == nnc - 2) {
            if (h <= (R)1) { s1 = 0.5; s2 = 0; s3 = 0; d1 = 1; d2 = 0; }
            else { s1 = -1.5; s2 = 4; s3 = -2; d1 = -3; d2 = 4; }
        } else {
            if (h <= (R)1) { s1 = 0.5; s2 = 0; s3 = 0; d1 = 1; d2 = 0; }
            else if (h <= (R)2) { s1 = -1; s2 = 3; s3 = -1.5; d1 = -2; d2 = 3; }
            else { s1 = 0.5; s2 = -3; s3 = 4.5; d1 = 1; d2 = -3; }
        }
        a.w[k] = (s1 * h + s2) * h + s3;
        a.dw[k] = rdiv(d1 * h + d2, dx, inv_dx);
    }
}

// Geometry as seen by a kernel, in the kernel's precision.
template <typename R>
struct KGeom {
    R xmin[3], dx[3], inv_dx[3];
    int nel[3], nnc[3], ntile[3];
    int nodec;
};

template <typename R, int O>
__device__ __forceinline__ void axis_eval(R x, const KGeom<R> &g, int d, int ie, Axis<R, O> &a);

template <>
__device__ __forceinline__ void axis_eval<float, 1>(float x, const KGeom<float> &g, int d, int ie, Axis<float, 1> &a) {
    axis_linear<float>(x, g.xmin[d], g.dx[d], g.inv_dx[d], ie, a);
}
template <>
__device__ __forceinline__ void axis_eval<double, 1>(double x, const KGeom<double> &g, int d, int ie,
                                                     Axis<double, 1> &a) {
    axis_linear<double>(x, g.xmin[d], g.dx[d], g.inv_dx[d], ie, a);
}
template <>
__device__ __forceinline__ void axis_eval<float, 2>(float x, const KGeom<float> &g, int d, int ie, Axis<float, 2> &a) {
    axis_quadratic<float>(x, g.xmin[d], g.dx[d], g.inv_dx[d], ie, g.nnc[d], a);
}
template <>
__device__ __forceinline__ void axis_eval<double, 2>(double x, const KGeom<double> &g, int d, int ie,
                                                     Axis<double, 2> &a) {
    axis_quadratic<double>(x, g.xmin[d], g.dx[d], g.inv_dx[d], ie, g.nnc[d], a);
}

// Element index of a point (MeshPointLinklist, module/material_point.cpp:59-65).
// Out-of-grid points are clamped and reported through *oob.
__device__ __forceinline__ float cell_coord(float x, const KGeom<float> &g, int d) {
    return (x - g.xmin[d]) * g.inv_dx[d];
}
__device__ __forceinline__ double cell_coord(double x, const KGeom<double> &g, int d) {
    return (x - g.xmin[d]) / g.dx[d];   // the reference's floor((x - xmin) / dx) in FP64
}

template <typename R>
__device__ __forceinline__ int cell_of(R x, const KGeom<R> &g, int d, bool &oob) {
    R t = cell_coord(x, g, d);
    int c = (int)floor(t);
    if (!(t >= (R)0) || c >= g.nel[d]) {   // also catches NaN
        oob = true;
        c = c < 0 || !(t >= (R)0) ? 0 : g.nel[d] - 1;
    }
    return c;
}

// ---------------------------------------------------------------------------
// Fixed-point accumulation.  Every contribution c is scaled by 2^e and
// rounded to an int64; the sums are exact integers, so the result does not
// depend on the order in which particles are visited.
// ---------------------------------------------------------------------------
// 2^e for |e| <= 240 (double) and |e| <= 120 (float), built from the
// exponent bits: exact, and cheap on a part whose FP64 library calls are slow
__host__ __device__ inline double pow2d(int e) {
    const unsigned long long b = (unsigned long long)(e + 1023) << 52;
    double d;
    memcpy(&d, &b, sizeof(d));
    return d;
}
__host__ __device__ inline float pow2f(int e) {
    const unsigned b = (unsigned)(e + 127) << 23;
    float f;
    memcpy(&f, &b, sizeof(f));
    return f;
}

__host__ __device__ inline Fix make_fix(double bound) {
    int e = 0;
    if (bound > 0.0 && bound < 1.0e300) {
        // k with bound < 2^k <= 2 bound (frexp's exponent), from the exponent
        // bits of a normal number; subnormal bounds take frexp
        unsigned long long bits;
        memcpy(&bits, &bound, sizeof(bits));
        const int ex = (int)((bits >> 52) & 0x7FF);
        int k;
        if (ex != 0) k = ex - 1022;
        else frexp(bound, &k);
        e = 62 - k;         // |sum| <= bound * 2^e < 2^62
    }
    if (e > 240) e = 240;
    if (e < -240) e = -240;
    Fix f;
    f.sd = pow2d(e);
    f.inv = pow2d(-e);
    f.s1 = pow2f(e / 2);
    f.s2 = pow2f(e - e / 2);
    f.i1 = pow2f(-(e / 2));
    f.i2 = pow2f(-(e - e / 2));
    return f;
}

__device__ __forceinline__ long long fx(float c, const Fix &f) { return __float2ll_rn((c * f.s1) * f.s2); }
__device__ __forceinline__ long long fx(double c, const Fix &f) { return __double2ll_rn(c * f.sd); }
// fixed point back to the working precision
__device__ __forceinline__ float unfx(long long q, const Fix &f, float) { return (__ll2float_rn(q) * f.i1) * f.i2; }
__device__ __forceinline__ double unfx(long long q, const Fix &f, double) { return (double)q * f.inv; }

__device__ __forceinline__ void atomic_add_i64(unsigned long long *p, long long v) {
    atomicAdd(p, (unsigned long long)v);
}

__device__ __forceinline__ float bits_f(unsigned int u) { return __uint_as_float(u); }
__device__ __forceinline__ void atomic_max_pos(unsigned int *slot, float v) {
    // v >= 0 (or NaN, mapped to +inf so that the caller's bounds stay safe)
    if (!(v >= 0.0f)) v = INFINITY;
    atomicMax(slot, __float_as_uint(v));
}

// ---------------------------------------------------------------------------
// Constitutive updates (module/solid/constitutive_model.cpp).
// D = dt * sum(dN (x) v) is the velocity-gradient increment, i.e. the
// reference's delta_def_grad minus the identity.
// ---------------------------------------------------------------------------
// MatLinElast (constitutive_model.cpp:16-60): incremental, engineering shear.
// Hardware reciprocal (rcp.approx: one MUFU operation, deterministic, within
// about an ulp of 1/x).  The FP32 path uses it where an IEEE division would
// cost a slow-path sequence per particle: the normalisation of gathers by
// their weight sum and the material constants; FP64 keeps 1.0 / x.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
template <typename R>
__device__ __forceinline__ R recip(R x) {
    if constexpr (sizeof(R) == 4) return rcp_approx(x);
    else return (R)1 / x;
}

template <typename R>
__device__ __forceinline__ void lin_elast_update(R *s, const R D[3][3], R E, R nu) {
    const R rd = recip<R>(((R)1 - (R)2 * nu) * ((R)1 + nu));   // one division
    const R C0 = E * ((R)1 - nu) * rd;
    const R C1 = E * nu * rd;
    const R C2 = (R)0.5 * E * ((R)1 - (R)2 * nu) * rd;
    R e0 = D[0][0], e1 = D[1][1], e2 = D[2][2];
    R e3 = D[1][2] + D[2][1], e4 = D[2][0] + D[0][2], e5 = D[0][1] + D[1][0];
    s[0] += C0 * e0 + C1 * e1 + C1 * e2;
    s[1] += C1 * e0 + C0 * e1 + C1 * e2;
    s[2] += C1 * e0 + C1 * e1 + C0 * e2;
    s[3] += C2 * e3;
    s[4] += C2 * e4;
    s[5] += C2 * e5;
}

// MatNeoHookean (constitutive_model.cpp:62-125), stress part.
// One division for the Lame constants and one for 1/J: FP64 divisions are
// expensive on this part (tens of FP64-pipe operations each).  Returns
// log(J) for callers that need it again (the tangent of the implicit solid).
template <typename R>
__device__ __forceinline__ R neo_hookean_stress(R *s, const R F[3][3], R jac, R E, R nu) {
    const R rd = (R)1 / (((R)1 + nu) * ((R)1 - (R)2 * nu));
    const R lmd = nu * E * rd;
    const R mu = (R)0.5 * E * ((R)1 - (R)2 * nu) * rd;
    const R lnj = log(jac);
    const R ij = (R)1 / jac;
    R be[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) be[i][j] = F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2];
    s[0] = (mu * (be[0][0] - (R)1) + lmd * lnj) * ij;
    s[1] = (mu * (be[1][1] - (R)1) + lmd * lnj) * ij;
    s[2] = (mu * (be[2][2] - (R)1) + lmd * lnj) * ij;
    s[3] = (mu * be[1][2]) * ij;
    s[4] = (mu * be[0][2]) * ij;
    s[5] = (mu * be[0][1]) * ij;
    return lnj;
}

// The same stress from the displacement gradient H = F - I and jm1 = J - 1,
// used by the FP32 path, which stores H: be - I = H + H^T + H H^T keeps the
// small strain out of the rounding of F F^T.
__device__ __forceinline__ void neo_hookean_stress_h(float *s, const float H[3][3], float jm1, float E, float nu) {
    const float rd = rcp_approx((1.0f + nu) * (1.0f - 2.0f * nu));
    const float lmd = nu * E * rd;
    const float mu = 0.5f * E * (1.0f - 2.0f * nu) * rd;
    const float lnj = log1pf(jm1);
    const float J = 1.0f + jm1;
    const float ij = rcp_approx(J);
    float bm[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            bm[i][j] = H[i][j] + H[j][i] + H[i][0] * H[j][0] + H[i][1] * H[j][1] + H[i][2] * H[j][2];
    s[0] = (mu * bm[0][0] + lmd * lnj) * ij;
    s[1] = (mu * bm[1][1] + lmd * lnj) * ij;
    s[2] = (mu * bm[2][2] + lmd * lnj) * ij;
    s[3] = (mu * bm[1][2]) * ij;
    s[4] = (mu * bm[0][2]) * ij;
    s[5] = (mu * bm[0][1]) * ij;
}

// F-bar form of MatNeoHookean (constitutive_model.cpp:62-120 with
// jac_bar = det_def_grad_bar): ln of J-bar in the volumetric term, the
// division by the plain J.  FP64 on F, FP32 on H = F - I with J - 1 values.
template <typename R>
__device__ __forceinline__ void neo_hookean_stress_bar(R *s, const R F[3][3], R jac, R jac_bar, R E, R nu) {
    const R rd = (R)1 / (((R)1 + nu) * ((R)1 - (R)2 * nu));
    const R lmd = nu * E * rd;
    const R mu = (R)0.5 * E * ((R)1 - (R)2 * nu) * rd;
    const R lnj = log(jac_bar);
    const R ij = (R)1 / jac;
    R be[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) be[i][j] = F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2];
    s[0] = (mu * (be[0][0] - (R)1) + lmd * lnj) * ij;
    s[1] = (mu * (be[1][1] - (R)1) + lmd * lnj) * ij;
    s[2] = (mu * (be[2][2] - (R)1) + lmd * lnj) * ij;
    s[3] = (mu * be[1][2]) * ij;
    s[4] = (mu * be[0][2]) * ij;
    s[5] = (mu * be[0][1]) * ij;
}

__device__ __forceinline__ void neo_hookean_stress_h_bar(float *s, const float H[3][3], float jm1, float jbm1, float E,
                                                         float nu) {
    const float rd = rcp_approx((1.0f + nu) * (1.0f - 2.0f * nu));
    const float lmd = nu * E * rd;
    const float mu = 0.5f * E * (1.0f - 2.0f * nu) * rd;
    const float lnj = log1pf(jbm1);
    const float ij = rcp_approx(1.0f + jm1);
    float bm[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            bm[i][j] = H[i][j] + H[j][i] + H[i][0] * H[j][0] + H[i][1] * H[j][1] + H[i][2] * H[j][2];
    s[0] = (mu * bm[0][0] + lmd * lnj) * ij;
    s[1] = (mu * bm[1][1] + lmd * lnj) * ij;
    s[2] = (mu * bm[2][2] + lmd * lnj) * ij;
    s[3] = (mu * bm[1][2]) * ij;
    s[4] = (mu * bm[0][2]) * ij;
    s[5] = (mu * bm[0][1]) * ij;
}

// MatStVk (constitutive_model.cpp:122-185), stress part: with b = F F^T and
// tr E = (tr b - 3) / 2, sigma = (mu b^2 + (lambda tr E - mu) b) / J.
template <typename R>
__device__ __forceinline__ void stvk_stress(R *s, const R F[3][3], R jac, R E, R nu) {
    const R rd = (R)1 / (((R)1 + nu) * ((R)1 - (R)2 * nu));
    const R lmd = nu * E * rd;
    const R mu = (R)0.5 * E * ((R)1 - (R)2 * nu) * rd;
    R be[3][3], b2[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) be[i][j] = F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) b2[i][j] = be[i][0] * be[0][j] + be[i][1] * be[1][j] + be[i][2] * be[2][j];
    const R tre = (R)0.5 * (be[0][0] + be[1][1] + be[2][2] - (R)3);
    const R ij = (R)1 / jac;
    const R cb = lmd * tre - mu;
    s[0] = (mu * b2[0][0] + cb * be[0][0]) * ij;
    s[1] = (mu * b2[1][1] + cb * be[1][1]) * ij;
    s[2] = (mu * b2[2][2] + cb * be[2][2]) * ij;
    s[3] = (mu * b2[1][2] + cb * be[1][2]) * ij;
    s[4] = (mu * b2[0][2] + cb * be[0][2]) * ij;
    s[5] = (mu * b2[0][1] + cb * be[0][1]) * ij;
}

// The same from H = F - I (FP32 path): with m = b - I = H + H^T + H H^T,
// mu b^2 + (lambda trE - mu) b = lambda trE (I + m) + mu (m + m^2), trE = tr m / 2,
// free of the cancellation of numbers near 1.
__device__ __forceinline__ void stvk_stress_h(float *s, const float H[3][3], float jm1, float E, float nu) {
    const float rd = rcp_approx((1.0f + nu) * (1.0f - 2.0f * nu));
    const float lmd = nu * E * rd;
    const float mu = 0.5f * E * (1.0f - 2.0f * nu) * rd;
    float m[3][3], m2[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) m[i][j] = H[i][j] + H[j][i] + H[i][0] * H[j][0] + H[i][1] * H[j][1] + H[i][2] * H[j][2];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) m2[i][j] = m[i][0] * m[0][j] + m[i][1] * m[1][j] + m[i][2] * m[2][j];
    const float lt = lmd * 0.5f * (m[0][0] + m[1][1] + m[2][2]);
    const float ij = rcp_approx(1.0f + jm1);
    s[0] = (lt * (1.0f + m[0][0]) + mu * (m[0][0] + m2[0][0])) * ij;
    s[1] = (lt * (1.0f + m[1][1]) + mu * (m[1][1] + m2[1][1])) * ij;
    s[2] = (lt * (1.0f + m[2][2]) + mu * (m[2][2] + m2[2][2])) * ij;
    s[3] = (lt * m[1][2] + mu * (m[1][2] + m2[1][2])) * ij;
    s[4] = (lt * m[0][2] + mu * (m[0][2] + m2[0][2])) * ij;
    s[5] = (lt * m[0][1] + mu * (m[0][1] + m2[0][1])) * ij;
}

// MatMooneyRivlin (constitutive_model.cpp:187-285), stress part; mat_prop =
// {c1, c2, bulk}.  With b = J^(-2/3) F F^T, I1 = tr b, I2 = (I1^2 - tr b^2) / 2:
// sigma = 2 ((c1 + c2 I1) b - c2 b^2) / J + (bulk ln J / J - 2 (c1 I1 + 2 c2 I2) / (3 J)) I.
template <typename R>
__device__ __forceinline__ void mooney_rivlin_stress(R *s, const R F[3][3], R jac, R c1, R c2, R bulk) {
    const R k = (R)1 / cbrt(jac);
    R be[3][3], b2[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            be[i][j] = (k * F[i][0]) * (k * F[j][0]) + (k * F[i][1]) * (k * F[j][1]) + (k * F[i][2]) * (k * F[j][2]);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) b2[i][j] = be[i][0] * be[0][j] + be[i][1] * be[1][j] + be[i][2] * be[2][j];
    const R i1 = be[0][0] + be[1][1] + be[2][2];
    const R i2 = (R)0.5 * (i1 * i1 - (b2[0][0] + b2[1][1] + b2[2][2]));
    const R ij = (R)1 / jac;
    const R hp = bulk * log(jac) * ij;
    const R dg = hp - (R)2 / (R)3 * ij * (c1 * i1 + (R)2 * c2 * i2);
    const R ca = (R)2 * (c1 + c2 * i1) * ij, cb = (R)2 * c2 * ij;
    s[0] = ca * be[0][0] - cb * b2[0][0] + dg;
    s[1] = ca * be[1][1] - cb * b2[1][1] + dg;
    s[2] = ca * be[2][2] - cb * b2[2][2] + dg;
    s[3] = ca * be[1][2] - cb * b2[1][2];
    s[4] = ca * be[0][2] - cb * b2[0][2];
    s[5] = ca * be[0][1] - cb * b2[0][1];
}

// The same from H = F - I (FP32 path).  With B = b - I = (J^(-2/3) - 1) I +
// J^(-2/3) m, m = H + H^T + H H^T, the stress is
//   2/J [ (c2 trB - (c1 trB + 4 c2 trB + c2 (trB)^2 - c2 tr B^2) / 3) I
//         + (c1 + c2 + c2 trB) B - c2 B^2 ] + bulk ln(J) / J I,
// which is the expression above with the parts that cancel at small strain
// taken out exactly.
__device__ __forceinline__ void mooney_rivlin_stress_h(float *s, const float H[3][3], float jm1, float c1, float c2,
                                                       float bulk) {
    const float lj = log1pf(jm1);
    const float km1 = expm1f(-(2.0f / 3.0f) * lj);   // J^(-2/3) - 1
    const float k = 1.0f + km1;
    float B[3][3], B2[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const float m = H[i][j] + H[j][i] + H[i][0] * H[j][0] + H[i][1] * H[j][1] + H[i][2] * H[j][2];
            B[i][j] = k * m + (i == j ? km1 : 0.0f);
        }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) B2[i][j] = B[i][0] * B[0][j] + B[i][1] * B[1][j] + B[i][2] * B[2][j];
    const float tb = B[0][0] + B[1][1] + B[2][2];
    const float tb2 = B2[0][0] + B2[1][1] + B2[2][2];
    const float ij = rcp_approx(1.0f + jm1);
    const float dg = 2.0f * ij * (c2 * tb - (c1 * tb + 4.0f * c2 * tb + c2 * tb * tb - c2 * tb2) / 3.0f) +
                     bulk * lj * ij;
    const float ca = 2.0f * ij * (c1 + c2 + c2 * tb), cb = 2.0f * ij * c2;
    s[0] = ca * B[0][0] - cb * B2[0][0] + dg;
    s[1] = ca * B[1][1] - cb * B2[1][1] + dg;
    s[2] = ca * B[2][2] - cb * B2[2][2] + dg;
    s[3] = ca * B[1][2] - cb * B2[1][2];
    s[4] = ca * B[0][2] - cb * B2[0][2];
    s[5] = ca * B[0][1] - cb * B2[0][1];
}

// Weakly compressible Newtonian fluid (material model 4, no counterpart in the
// reference): Tait equation of state p = (rho0 c0^2 / gamma) ((rho / rho0)^gamma - 1)
// with rho = rho0 / J, and sigma = -p I + 2 mu dev(D), D = sym(grad v).
// `inc` is the step increment dF - I = dt grad v; mat_prop = {c0, gamma, mu}.
// (rho/rho0)^gamma - 1 = expm1(-gamma log1p(J - 1)) keeps the small volume
// change out of the rounding of numbers near 1.
template <typename R>
__device__ __forceinline__ void tait_stress(R *s, const R inc[3][3], R jm1, R rho0, R c0, R gam, R mu, R inv_dt) {
    R pr;
    if constexpr (sizeof(R) == 8) pr = rho0 * c0 * c0 / gam * expm1(-gam * log1p(jm1));
    else pr = rho0 * c0 * c0 * rcp_approx(gam) * expm1f(-gam * log1pf(jm1));
    const R d0 = inc[0][0] * inv_dt, d1 = inc[1][1] * inv_dt, d2 = inc[2][2] * inv_dt;
    const R tr3 = (d0 + d1 + d2) * ((R)1 / (R)3);
    s[0] = -pr + (R)2 * mu * (d0 - tr3);
    s[1] = -pr + (R)2 * mu * (d1 - tr3);
    s[2] = -pr + (R)2 * mu * (d2 - tr3);
    s[3] = mu * (inc[1][2] + inc[2][1]) * inv_dt;
    s[4] = mu * (inc[0][2] + inc[2][0]) * inv_dt;
    s[5] = mu * (inc[0][1] + inc[1][0]) * inv_dt;
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start before its predecessor in the stream has finished;
// pdl_wait blocks until the predecessor has completed and its memory is
// visible (a no-op for an ordinary launch), pdl_trigger lets the next kernel
// of the stream be scheduled once every CTA of this one has started.  Every
// kernel launched that way calls pdl_wait before touching global memory.
// The step kernels do not trigger early: their persistent grids are sized to
// the SMs, and successor CTAs placed on the first SMs to drain unbalanced
// them (a step 463.5 -> 489 us at 4.1M particles).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// det(I + H) - 1 in FP64 for a row-major H[9] (host and device)
__host__ __device__ inline double det_ipm1_d(const double *H) {
    const double tr = H[0] + H[4] + H[8];
    const double m2 = H[0] * H[4] + H[0] * H[8] + H[4] * H[8] - H[1] * H[3] - H[2] * H[6] - H[5] * H[7];
    const double d = H[0] * (H[4] * H[8] - H[5] * H[7]) + H[1] * (H[5] * H[6] - H[3] * H[8]) +
                     H[2] * (H[3] * H[7] - H[4] * H[6]);
    return tr + m2 + d;
}

// det(I + H) - 1 without forming I + H
__device__ __forceinline__ float det_ipm1(const float H[3][3]) {
    const float tr = H[0][0] + H[1][1] + H[2][2];
    const float m2 = H[0][0] * H[1][1] + H[0][0] * H[2][2] + H[1][1] * H[2][2] - H[0][1] * H[1][0] -
                     H[0][2] * H[2][0] - H[1][2] * H[2][1];
    const float d = H[0][0] * (H[1][1] * H[2][2] - H[1][2] * H[2][1]) + H[0][1] * (H[1][2] * H[2][0] - H[1][0] * H[2][2]) +
                    H[0][2] * (H[1][0] * H[2][1] - H[1][1] * H[2][0]);
    return tr + m2 + d;
}

// ---------------------------------------------------------------------------
// Bulk asynchronous copies (TMA, 1-D) into shared memory, completed on an
// mbarrier.  Addresses must be 16-byte aligned and sizes multiples of 16.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: false when the phase did not complete within `limit` polls
// or `limit_ns` of wall time (one second by default), whichever comes first
// (try_wait may suspend the thread for a system-dependent time, so the poll
// count alone does not bound the time).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity, unsigned limit,
                                                  unsigned long long limit_ns = 1000000000ull) {
    const unsigned long long t0 = global_ns();
    for (unsigned i = 0; i < limit; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 255u) == 255u && global_ns() - t0 > limit_ns) return false;
    }
    return false;
}

template <typename R>
__device__ __forceinline__ R det3(const R a[3][3]) {
    return a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) + a[0][1] * (a[1][2] * a[2][0] - a[1][0] * a[2][2]) +
           a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
}

}  // namespace mpm
