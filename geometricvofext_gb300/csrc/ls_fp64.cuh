// FP64 least-squares gradient of a cell field over the cell-point-cell
// stencil (OpenFOAM leastSquareGrad<scalar>("polyDegree1") as the reference
// calls it, reconstruction.C:85-141 and 144-190), restated: the unweighted
// fit a0 + g.(x - x_c) over the cell and its stencil cells in ascending id
// order, normal equations summed in that order, Gaussian elimination with
// partial pivoting (first maximum on ties); a singular system gives g = 0.
// Translation units that use it for the plain form are built with
// -fmad=false.
#pragma once

#include "simplic_device.cuh"

namespace simplic {

__device__ __forceinline__ d3 lsGradient4(const double (&Ain)[4][4], const double (&bin)[4]) {
    double A[4][4], b[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        b[i] = bin[i];
#pragma unroll
        for (int j = 0; j < 4; ++j) A[i][j] = Ain[i][j];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int p = k;
        double best = fabs(A[k][k]);
#pragma unroll
        for (int i = k + 1; i < 4; ++i)
            if (fabs(A[i][k]) > best) {
                best = fabs(A[i][k]);
                p = i;
            }
        if (!(best > kVSMALL)) return mk(0, 0, 0);
        if (p != k) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                // select-based swap keeps the arrays in registers
                double tk = A[k][j], tp = A[p][j];
#pragma unroll
                for (int r = k + 1; r < 4; ++r)
                    if (r == p) tp = A[r][j];
                A[k][j] = tp;
#pragma unroll
                for (int r = k + 1; r < 4; ++r)
                    if (r == p) A[r][j] = tk;
            }
            double tk = b[k], tp = b[k];
#pragma unroll
            for (int r = k + 1; r < 4; ++r)
                if (r == p) tp = b[r];
            b[k] = tp;
#pragma unroll
            for (int r = k + 1; r < 4; ++r)
                if (r == p) b[r] = tk;
        }
#pragma unroll
        for (int i = k + 1; i < 4; ++i) {
            const double f = A[i][k] / A[k][k];
#pragma unroll
            for (int j = k; j < 4; ++j) A[i][j] = A[i][j] - f * A[k][j];
            b[i] = b[i] - f * b[k];
        }
    }
    double x[4];
#pragma unroll
    for (int i = 3; i >= 0; --i) {
        double s = b[i];
#pragma unroll
        for (int j = i + 1; j < 4; ++j) s = s - A[i][j] * x[j];
        x[i] = s / A[i][i];
    }
    return mk(x[1], x[2], x[3]);
}

// The gradient of `field` at cell c (the cell itself first, then its
// stencil row).
__device__ __forceinline__ d3 lsGradientField(const DevMesh& m, int c, const double* __restrict__ field,
                                              uint32_t& err) {
    const int32_t* st;
    const int ns = stencilOf(m, c, st, err);
    const d3 Cc = ld3(m.C, c);
    double A[4][4] = {{0}}, b[4] = {0, 0, 0, 0};
    for (int s = -1; s < ns; ++s) {
        const int x = (s < 0) ? c : st[s];
        const d3 dx = ld3(m.C, x) - Cc;
        const double v = field[x];
        const double t1 = dx.x, t2 = dx.y, t3 = dx.z;
        // A[i][j] += t_i t_j, b_i += t_i v with t_0 = 1 (1*x is exact);
        // A is symmetric bit for bit, so only the upper triangle is summed
        A[0][0] += 1.0;
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
    A[1][0] = A[0][1];
    A[2][0] = A[0][2];
    A[3][0] = A[0][3];
    A[2][1] = A[1][2];
    A[3][1] = A[1][3];
    A[3][2] = A[2][3];
    return lsGradient4(A, b);
}

}  // namespace simplic
