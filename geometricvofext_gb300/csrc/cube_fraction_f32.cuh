// Volume fraction of a cube below a plane, in FP32 (Scardovelli & Zaleski,
// J. Comput. Phys. 164 (2000) 228-237), for the learned form's fallback
// test: how well a plane through the cell reproduces the volume fractions
// of the neighbouring cells.
//
// In the unit cube [0,1]^3 the part below sum m_i u_i = a, with m1 <= m2 <=
// m3, sum m_i = 1.  Each region is written so that no term divides a large
// cube by a small m1 (the forms of the FP64 box solve of the mixed forms).
#pragma once

#include <cuda_runtime.h>

#include <cmath>

namespace simplic {

constexpr float kCubeMinM = 1e-4f;  // smaller plane coefficients are raised to this

// Sorted coefficients and the reciprocals the fraction uses.
struct CubeCoef {
    float m1, m2, m3;
    float k1;   // 1 / (6 m1 m2 m3)
    float k2;   // 1 / (6 m2 m3)
    float im3;  // 1 / m3
};

// Coefficients of the normal (nx, ny, nz): m_i = |n_i| / sum |n_j| raised to
// kCubeMinM and renormalised, returned unsorted (with the normal's signs) in
// p; false for a zero normal.
__host__ __device__ __forceinline__ bool cubeCoefficientsF(float nx, float ny, float nz, CubeCoef& c, float3& p) {
    float a = fabsf(nx), b = fabsf(ny), d = fabsf(nz);
    const float M = a + b + d;
    if (!(M > 0.f)) return false;
    const float iM = 1.f / M;
    a = fmaxf(a * iM, kCubeMinM);
    b = fmaxf(b * iM, kCubeMinM);
    d = fmaxf(d * iM, kCubeMinM);
    const float s = 1.f / (a + b + d);
    a *= s;
    b *= s;
    d *= s;
    p = make_float3(copysignf(a, nx), copysignf(b, ny), copysignf(d, nz));
    c.m1 = fminf(a, fminf(b, d));
    c.m3 = fmaxf(a, fmaxf(b, d));
    c.m2 = fmaxf(fminf(a, b), fminf(fmaxf(a, b), d));  // the median
    c.k2 = 1.f / (6.f * c.m2 * c.m3);
    c.k1 = c.k2 / c.m1;
    c.im3 = 1.f / c.m3;
    return true;
}

// F(a) for a in [0, 1] (clamped outside); dF = dF/da.
__host__ __device__ __forceinline__ float cubeFractionF(float a, const CubeCoef& c, float& dF) {
    dF = 0.f;
    if (a <= 0.f) return 0.f;
    if (a >= 1.f) return 1.f;
    const bool flip = a > 0.5f;
    if (flip) a = 1.f - a;
    float F;
    if (a < c.m1) {
        F = a * a * a * c.k1;
        dF = 3.f * a * a * c.k1;
    } else if (c.m3 >= c.m1 + c.m2 && a >= c.m1 + c.m2) {
        F = (a - 0.5f * (c.m1 + c.m2)) * c.im3;
        dF = c.im3;
    } else {
        F = (3.f * a * a - 3.f * a * c.m1 + c.m1 * c.m1) * c.k2;
        dF = (6.f * a - 3.f * c.m1) * c.k2;
        if (a > c.m2) {
            const float t = a - c.m2;
            F -= t * t * t * c.k1;
            dF -= 3.f * t * t * c.k1;
        }
        if (a > c.m3) {
            const float t = a - c.m3;
            F -= t * t * t * c.k1;
            dF -= 3.f * t * t * c.k1;
        }
    }
    return flip ? 1.f - F : F;
}

// a with F(a) = v: closed forms in the corner (cube root), edge
// (quadratic) and slab (linear) regions, else Newton inside the bracket of
// the region (dF/da is the section area), safeguarded by bisection; F is
// symmetric, F(1 - a) = 1 - F(a).
__host__ __device__ __forceinline__ float cubeInverseF(float v, const CubeCoef& c) {
    if (v <= 0.f) return 0.f;
    if (v >= 1.f) return 1.f;
    const bool flip = v > 0.5f;
    if (flip) v = 1.f - v;
    float a;
    const float v1 = c.m1 * c.m1 * c.m1 * c.k1;              // F(m1)
    const float v2 = v1 + 0.5f * (c.m2 - c.m1) * c.im3;      // F(m2)
    if (v <= v1) {
        a = cbrtf(v / c.k1);
    } else if (v <= v2) {
        a = (3.f * c.m1 + sqrtf(fmaxf(12.f * v / c.k2 - 3.f * c.m1 * c.m1, 0.f))) * (1.f / 6.f);
    } else if (c.m3 >= c.m1 + c.m2 && v >= 0.5f * (c.m1 + c.m2) * c.im3) {
        a = c.m3 * v + 0.5f * (c.m1 + c.m2);
    } else {
        float lo = c.m2, hi = 0.5f;
        a = 0.5f * (lo + hi);
        for (int it = 0; it < 16; ++it) {
            float d;
            const float r = cubeFractionF(a, c, d) - v;
            if (r > 0.f)
                hi = a;
            else
                lo = a;
            float an = d > 1e-6f ? a - r / d : 0.5f * (lo + hi);
            if (!(an > lo && an < hi)) an = 0.5f * (lo + hi);
            const bool done = fabsf(an - a) < 1e-7f;
            a = an;
            if (done) break;
        }
    }
    return flip ? 1.f - a : a;
}

// Fraction of the unit square below q1 v1 + q2 v2 = b (q1, q2 > 0): a
// corner triangle, a trapezoid, or the square less the opposite triangle.
__host__ __device__ __forceinline__ float squareFractionF(float b, float q1, float q2) {
    const float lo = fminf(q1, q2), hi = fmaxf(q1, q2), s = lo + hi;
    if (b <= 0.f) return 0.f;
    if (b >= s) return 1.f;
    if (b < lo) return b * b / (2.f * lo * hi);
    if (b <= hi) return (b - 0.5f * lo) / hi;
    const float t = s - b;
    return 1.f - t * t / (2.f * lo * hi);
}

// The part below the plane of the face x_axis = sigma / 2 (sigma = +-1) of
// the cube [-1/2, 1/2]^3 cut by the plane p.x + 1/2 = a in the frame of
// cubeFractionF (p: the signed coefficients cubeCoefficientsF returns); the
// same face seen as the other side's face takes sigma of the other side.
__host__ __device__ __forceinline__ float cubeFaceFractionF(float a, float3 p, int axis, float sigma) {
    const float pa = axis == 0 ? p.x : (axis == 1 ? p.y : p.z);
    const float q1 = fabsf(axis == 0 ? p.y : p.x), q2 = fabsf(axis == 2 ? p.y : p.z);
    const float u = (sigma * pa > 0.f) ? 1.f : 0.f;  // the face's coordinate in the reflected frame
    return squareFractionF(a - fabsf(pa) * u, q1, q2);
}

}  // namespace simplic
