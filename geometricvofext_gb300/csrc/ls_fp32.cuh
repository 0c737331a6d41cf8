// FP32 least-squares normal of a neighbourhood (the polyDegree1 fit of
// reconstruction.C:85-141 in single precision), shared by the mixed form's
// normal kernel and the learned form's network inputs.
#pragma once

#include <cuda_runtime.h>

namespace simplic {

// Gaussian elimination with partial pivoting of a 4x4 system; false when
// singular.
__device__ __forceinline__ bool solve4f(float (&A)[4][4], float (&b)[4], float (&x)[4]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int p = k;
        float best = fabsf(A[k][k]);
#pragma unroll
        for (int i = k + 1; i < 4; ++i)
            if (fabsf(A[i][k]) > best) {
                best = fabsf(A[i][k]);
                p = i;
            }
        if (!(best > 1e-30f)) return false;
#pragma unroll
        for (int i = k + 1; i < 4; ++i) {
            if (i != p) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float t = A[k][j];
                A[k][j] = A[i][j];
                A[i][j] = t;
            }
            const float t = b[k];
            b[k] = b[i];
            b[i] = t;
        }
        const float inv = 1.0f / A[k][k];
#pragma unroll
        for (int i = k + 1; i < 4; ++i) {
            const float f = A[i][k] * inv;
#pragma unroll
            for (int j = k; j < 4; ++j) A[i][j] -= f * A[k][j];
            b[i] -= f * b[k];
        }
    }
#pragma unroll
    for (int i = 3; i >= 0; --i) {
        float s = b[i];
#pragma unroll
        for (int j = i + 1; j < 4; ++j) s -= A[i][j] * x[j];
        x[i] = s / A[i][i];
    }
    return true;
}

// Accumulates one neighbour (offset t, value v relative to the centre's)
// into the normal equations of a + g.t.
__device__ __forceinline__ void lsAccumulate(float (&A)[4][4], float (&b)[4], float t1, float t2, float t3, float v) {
    A[0][0] += 1.f;
    A[0][1] += t1;
    A[0][2] += t2;
    A[0][3] += t3;
    A[1][1] += t1 * t1;
    A[1][2] += t1 * t2;
    A[1][3] += t1 * t3;
    A[2][2] += t2 * t2;
    A[2][3] += t2 * t3;
    A[3][3] += t3 * t3;
    b[0] += v;
    b[1] += t1 * v;
    b[2] += t2 * v;
    b[3] += t3 * v;
}

// -grad / |grad| from the accumulated system (zero vector when singular or
// flat).
__device__ __forceinline__ float3 lsNormal(float (&A)[4][4], float (&b)[4]) {
    A[1][0] = A[0][1];
    A[2][0] = A[0][2];
    A[3][0] = A[0][3];
    A[2][1] = A[1][2];
    A[3][1] = A[1][3];
    A[3][2] = A[2][3];
    float x[4];
    float3 n = make_float3(0.f, 0.f, 0.f);
    if (solve4f(A, b, x)) {
        const float g2 = x[1] * x[1] + x[2] * x[2] + x[3] * x[3];
        if (g2 > 0.f) {
            const float r = -rsqrtf(g2);
            n = make_float3(x[1] * r, x[2] * r, x[3] * r);
        }
    }
    return n;
}

}  // namespace simplic
