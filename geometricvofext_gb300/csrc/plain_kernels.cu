// Plain FP64 SimPLIC kernels (built with -fmad=false: bit-exact to the CPU
// restatement of the reference).
//
//  K1 scanMixed          reconstruction::initialize      reconstruction.C:634-677
//  K2 lsNormal           calcInterfaceNFromIsoAlphaGrad  reconstruction.C:85-141
//  K3 planeSolve         cutCell::findSignedDistance     cutCell.C:611-799
//  K4 interfaceFlux      advection::timeIntegratedFlux   advection.C:85-221
//  K5 update             upwind dVf + surfaceIntegrate + alpha update
//                                                        advectionTemplates.C:371,399-406
//  K6 bound              limitFlux / boundFlux           advectionTemplates.C:118-349
//  K7 bruteForce         applyBruteForceBounding         advection.C:291-308
//  faceFlatness          reconstruction::updateFaceFlatness reconstruction.C:408-440
#include "plain_geom.cuh"
#include "simplic_kernels.h"

#include <cfloat>
#include <climits>

namespace simplic {

// ---------------------------------------------------------------------------
// K1: mixed-cell list (warp-aggregated append) and per-cell status bytes
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) kScanMixed(int nc, const double* __restrict__ alpha, double tol,
                                                  int8_t* __restrict__ status, int* __restrict__ mixed,
                                                  int* __restrict__ nMixed) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    bool isMixed = false;
    if (c < nc) {
        const double a = alpha[c];
        isMixed = (tol < a) && (a < 1.0 - tol);
        status[c] = isMixed ? kStPending : kStNotMixed;
    }
    const unsigned ball = __ballot_sync(0xffffffffu, isMixed);
    if (ball == 0) return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0) base = atomicAdd(nMixed, __popc(ball));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (isMixed) mixed[base + __popc(ball & ((1u << lane) - 1u))] = c;
}

// ---------------------------------------------------------------------------
// K2: least-squares normal (polyDegree1 fit over the cell-point-cell stencil)
// ---------------------------------------------------------------------------
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

// Stencil: the cell, then all other cells sharing a point with it, ascending.
__device__ __forceinline__ int buildStencil(const DevMesh& m, int c, int* st, uint32_t& err) {
    int n = 0;
    for (int k = m.cpOff[c]; k < m.cpOff[c + 1]; ++k) {
        const int p = m.cPts[k];
        for (int q = m.pcOff[p]; q < m.pcOff[p + 1]; ++q) {
            const int x = m.pCells[q];
            if (x == c) continue;
            int pos = n;
            while (pos > 0 && st[pos - 1] > x) --pos;
            if (pos > 0 && st[pos - 1] == x) continue;
            if (n >= kMaxStencil) {
                err |= kErrStencilOverflow;
                continue;
            }
            for (int r = n; r > pos; --r) st[r] = st[r - 1];
            st[pos] = x;
            ++n;
        }
    }
    return n;
}

__global__ void __launch_bounds__(128) kLsNormal(DevMesh m, const double* __restrict__ alpha,
                                                 const int* __restrict__ mixed, const int* __restrict__ nMixed,
                                                 double* __restrict__ nrm, uint32_t* __restrict__ errOut) {
    const int nm = *nMixed;
    uint32_t err = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nm; i += gridDim.x * blockDim.x) {
        const int c = mixed[i];
        int st[kMaxStencil];
        const int ns = buildStencil(m, c, st, err);
        const d3 Cc = ld3(m.C, c);
        double A[4][4] = {{0}}, b[4] = {0, 0, 0, 0};
        for (int s = -1; s < ns; ++s) {
            const int x = (s < 0) ? c : st[s];
            const d3 dx = ld3(m.C, x) - Cc;
            const double v = alpha[x];
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
        const d3 g = lsGradient4(A, b);
        const d3 n = (-1.0) * g;
        st3(nrm, i, n / (mag(n) + kSMALL));
    }
    if (err) atomicOr(errOut, err);
}

// ---------------------------------------------------------------------------
// K3: plane constant per mixed cell
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) kPlaneSolve(DevMesh m, const double* __restrict__ alpha,
                                                   const int* __restrict__ mixed, const int* __restrict__ nMixed,
                                                   const double* __restrict__ nrm, int8_t* __restrict__ mStatus,
                                                   int8_t* __restrict__ status, double* __restrict__ dOut,
                                                   double* __restrict__ icOut, double* __restrict__ isOut,
                                                   uint32_t* __restrict__ errOut) {
    const int nm = *nMixed;
    uint32_t err = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nm; i += gridDim.x * blockDim.x) {
        const int c = mixed[i];
        CellWS w;
        double d = 0.0;
        d3 ic = mk(0, 0, 0), is = mk(0, 0, 0);
        int st;
        if (!loadCell(m, c, w)) {
            err |= kErrSubFaceOverflow;
            st = 1;
        } else {
            st = findSignedDistance(w, alpha[c], ld3(nrm, i), d, ic, is, err);
        }
        mStatus[i] = int8_t(st);
        status[c] = int8_t(st);
        dOut[i] = d;
        st3(icOut, i, ic);
        st3(isOut, i, is);
    }
    if (err) atomicOr(errOut, err);
}

// ---------------------------------------------------------------------------
// K4: Simpson time-integrated flux through downwind faces of cut cells
// ---------------------------------------------------------------------------
__device__ __forceinline__ d3 pointValue(const DevMesh& m, int p, const double* U, const double* Ub) {
    const int b0 = m.pbOff[p], b1 = m.pbOff[p + 1];
    d3 r = mk(0, 0, 0);
    if (b1 > b0) {
        for (int k = b0; k < b1; ++k) {
            const int f = m.pbFaces[k];
            const d3 u = Ub ? ld3(Ub, f - m.nfi) : ld3(U, m.own[f]);
            r = r + m.pbW[k] * u;
        }
        return r;
    }
    for (int k = m.pcOff[p]; k < m.pcOff[p + 1]; ++k) r = r + m.pcW[k] * ld3(U, m.pCells[k]);
    return r;
}

// cell-point interpolation (the restatement documented in the oracle)
__device__ __forceinline__ d3 interpolateU(const DevMesh& m, int c, d3 x, const double* U, const double* Ub) {
    const d3 a = ld3(m.C, c);
    const d3 r = x - a;
    int bp0 = -1, bp1 = -1, bp2 = -1;
    double bw0 = 0, bw1 = 0, bw2 = 0, bw3 = 0, bestMin = -1e300;
    bool found = false;
    for (int k = m.cOff[c]; k < m.cOff[c + 1] && !found; ++k) {
        const int f = m.cFaces[k];
        const int q0 = m.fOff[f], n = m.fOff[f + 1] - q0;
        const int g0 = m.fPts[q0];
        const d3 e1 = ld3(m.pts, g0) - a;
        for (int i = 1; i + 1 < n; ++i) {
            const int gi = m.fPts[q0 + i], gj = m.fPts[q0 + i + 1];
            const d3 e2 = ld3(m.pts, gi) - a, e3 = ld3(m.pts, gj) - a;
            const double det = dot(e1, cross(e2, e3));
            if (!(fabs(det) > kVSMALL)) continue;
            const double w1 = dot(r, cross(e2, e3)) / det;
            const double w2 = dot(e1, cross(r, e3)) / det;
            const double w3 = dot(e1, cross(e2, r)) / det;
            const double w0 = ((1.0 - w1) - w2) - w3;
            const double mn = fmin(fmin(w0, w1), fmin(w2, w3));
            if (mn > bestMin || mn >= -1e-10) {
                bestMin = mn;
                bp0 = g0;
                bp1 = gi;
                bp2 = gj;
                bw0 = w0;
                bw1 = w1;
                bw2 = w2;
                bw3 = w3;
            }
            if (mn >= -1e-10) {
                found = true;
                break;
            }
        }
    }
    if (bp0 < 0) return ld3(U, c);
    d3 t = bw0 * ld3(U, c);
    t = t + bw1 * pointValue(m, bp0, U, Ub);
    t = t + bw2 * pointValue(m, bp1, U, Ub);
    t = t + bw3 * pointValue(m, bp2, U, Ub);
    return t;
}

__global__ void __launch_bounds__(128) kInterfaceFlux(DevMesh m, const int* __restrict__ mixed,
                                                      const int* __restrict__ nMixed,
                                                      const int8_t* __restrict__ mStatus,
                                                      const double* __restrict__ nrm, const double* __restrict__ dArr,
                                                      const double* __restrict__ icArr, const double* __restrict__ phi,
                                                      const double* __restrict__ U, const double* __restrict__ Ub,
                                                      double dt, double* __restrict__ dvfI,
                                                      uint8_t* __restrict__ cutMask) {
    const int nm = *nMixed;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nm; i += gridDim.x * blockDim.x) {
        if (mStatus[i] != 0) continue;
        const int c = mixed[i];
        const d3 n = ld3(nrm, i);
        const double d = dArr[i];
        const double Un0 = dot(interpolateU(m, c, ld3(icArr, i), U, Ub), n);
        for (int k = m.cOff[c]; k < m.cOff[c + 1]; ++k) {
            const int f = m.cFaces[k];
            const double ph = phi[f];
            bool down;
            if (f < m.nfi)
                down = (c == m.own[f]) ? (ph >= 0.0) : (ph < 0.0);
            else
                down = ph >= 0.0;
            if (!down) continue;
            dvfI[f] = timeIntegratedFaceFlux(m, f, n, d, Un0, dt, ph, m.magSf[f]);
            if (cutMask) cutMask[f] = 1;
        }
    }
}

// ---------------------------------------------------------------------------
// K5: upwind flux, interface overrides, surfaceIntegrate and alpha update
// ---------------------------------------------------------------------------
// dVf of one face before bounding: the Simpson value when the upwind cell is
// cut, else (phi * alpha_f) * dt with alpha_f = w (aP - aN) + aN, w = pos0(phi)
// (upwind weights through the linear interpolation formula); boundary faces
// use the boundary value of alpha.
__device__ __forceinline__ double baseDVf(const DevMesh& m, int f, double ph, const double* aCur,
                                          const int8_t* status, const double* dvfI, const double* alphaB, double dt) {
    if (f < m.nfi) {
        const int o = m.own[f], nb = m.nei[f];
        const int up = (ph >= 0.0) ? o : nb;
        if (status[up] == 0) return dvfI[f];
        const double w = pos0(ph);
        const double af = w * (aCur[o] - aCur[nb]) + aCur[nb];
        return ph * af * dt;
    }
    const int o = m.own[f];
    if (ph >= 0.0 && status[o] == 0) return dvfI[f];
    const double ab = alphaB ? alphaB[f - m.nfi] : aCur[o];
    return ph * ab * dt;
}

__global__ void __launch_bounds__(256) kUpdate(DevMesh m, const double* __restrict__ phi,
                                               const double* __restrict__ aCur, const double* __restrict__ aOld,
                                               double* __restrict__ aNew, const int8_t* __restrict__ status,
                                               const double* __restrict__ dvfI, const double* __restrict__ alphaB,
                                               const double* __restrict__ Sp, const double* __restrict__ Su,
                                               double dt, double rDeltaT, double* __restrict__ alphaPhi,
                                               double* __restrict__ blkMin, double* __restrict__ blkMax) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double an = 0.0;
    bool valid = c < m.nc;
    if (valid) {
        const int k0 = m.cOff[c], k1 = m.cOff[c + 1];
        const double ao = aOld[c];
        const double ac = aCur[c];
        // Empty neighbourhood: every dVf is a signed zero, surfaceIntegrate
        // gives +0 and ((ao*r) - 0*r)/r returns ao itself (bit for bit).
        bool quick = (Sp == nullptr) && (Su == nullptr) && (ao == 0.0) && (ac == 0.0);
        if (quick) {
            for (int k = k0; k < k1; ++k) {
                const int nb = m.cNbr[k];
                double ax;
                if (nb >= 0)
                    ax = aCur[nb];
                else
                    ax = alphaB ? alphaB[(m.cAsc[k] & 0x7fffffff) - m.nfi] : ac;
                if (ax != 0.0) {
                    quick = false;
                    break;
                }
            }
        }
        if (quick) {
            an = ao;
            for (int k = k0; k < k1; ++k) {
                const int fa = m.cAsc[k];
                if (fa < 0) continue;  // neighbour side: the owner writes the face
                alphaPhi[fa] = copysign(0.0, phi[fa]);
            }
        } else {
            double sum = 0.0;
            for (int k = k0; k < k1; ++k) {
                const int fa = m.cAsc[k];
                const int f = fa & 0x7fffffff;
                const double ph = phi[f];
                const double dv = baseDVf(m, f, ph, aCur, status, dvfI, alphaB, dt);
                if (fa >= 0) {
                    alphaPhi[f] = dv / dt;
                    sum += dv;
                } else {
                    sum -= dv;
                }
            }
            const double ivf = sum / m.V[c];
            double num = ao * rDeltaT;
            if (Su) num = num + Su[c];
            num = num - ivf * rDeltaT;
            const double den = Sp ? (rDeltaT - Sp[c]) : rDeltaT;
            an = num / den;
        }
        aNew[c] = an;
    }
    // block min / max of the new alpha for limitFlux's gMin / gMax
    double mn = valid ? an : DBL_MAX, mx = valid ? an : -DBL_MAX;
    for (int o = 16; o > 0; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    __shared__ double smn[8], smx[8];
    const int wid = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        smn[wid] = mn;
        smx[wid] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            mn = fmin(mn, smn[w]);
            mx = fmax(mx, smx[w]);
        }
        blkMin[blockIdx.x] = mn;
        blkMax[blockIdx.x] = mx;
    }
}

// ---------------------------------------------------------------------------
// K6: conservative bounding (limitFlux + boundFlux), one block.  The
// reference's cell loop is serial and order dependent (a cell reads the
// corrections written by earlier cells), so thread 0 runs it over the
// ascending candidate list; the block shares the reductions, candidate
// search, sorting and min/max refresh.
// ---------------------------------------------------------------------------
struct BoundScratch {
    int* cand;
    int candCap;
    double* corr;      // [nf], zero outside a pass
    double* dvfMod;    // [nf]
    int* modStamp;     // [nf]
    int* doneStamp;    // [nf]
    int* corrected;    // first-loop corrected faces of a pass
    int* written;      // every face written in a pass
    int listCap;
    int* modList;      // faces whose dVf changed this step
    int modCap;
    int* touched;      // cells whose alpha changed in a pass
    int touchedCap;
};

__device__ __forceinline__ bool overshoots(double a) { return a < -100.0 * kSMALL || a > 1.0 + 100.0 * kSMALL; }

__device__ double blockReduceMinMax(double& mn, double& mx) {
    __shared__ double smn[32], smx[32];
    for (int o = 16; o > 0; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        smn[wid] = mn;
        smx[wid] = mx;
    }
    __syncthreads();
    mn = smn[0];
    mx = smx[0];
    for (int w = 1; w < nw; ++w) {
        mn = fmin(mn, smn[w]);
        mx = fmax(mx, smx[w]);
    }
    __syncthreads();
    return mn;
}

__device__ __forceinline__ double curDVf(const DevMesh& m, int f, const double* phi, const double* aCur,
                                         const int8_t* status, const double* dvfI, const double* alphaB, double dt,
                                         const BoundScratch& s, int stamp) {
    if (s.modStamp[f] == stamp) return s.dvfMod[f];
    return baseDVf(m, f, phi[f], aCur, status, dvfI, alphaB, dt);
}

__device__ __forceinline__ bool inNeedBounding(const DevMesh& m, int c, const int8_t* status) {
    if (status[c] != kStNotMixed) return true;
    for (int k = m.cOff[c]; k < m.cOff[c + 1]; ++k) {
        const int nb = m.cNbr[k];
        if (nb >= 0 && status[nb] != kStNotMixed) return true;
    }
    return false;
}

__device__ void blockBitonicSort(int* a, int n) {
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (int i = n + threadIdx.x; i < n2; i += blockDim.x) a[i] = INT_MAX;
    __syncthreads();
    for (int k = 2; k <= n2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const int ai = a[i], al = a[l];
                    const bool up = (i & k) == 0;
                    if ((ai > al) == up) {
                        a[i] = al;
                        a[l] = ai;
                    }
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(1024) kBound(DevMesh m, const double* __restrict__ phi,
                                               const double* __restrict__ aCur, const double* __restrict__ aOld,
                                               double* __restrict__ aNew, const int8_t* __restrict__ status,
                                               const int* __restrict__ mixed, const int* __restrict__ nMixed,
                                               const double* __restrict__ dvfI, const double* __restrict__ alphaB,
                                               const double* __restrict__ Sp, const double* __restrict__ Su,
                                               double dt, double rDeltaT, int nAlphaBounds,
                                               double* __restrict__ blkMin, double* __restrict__ blkMax, int nBlk,
                                               int blkCells, double* __restrict__ alphaPhi, BoundScratch s,
                                               int stamp, int* __restrict__ info, uint32_t* __restrict__ errOut) {
    const double aTol = 100.0 * kSMALL;
    __shared__ int sCount, sMod, sOverflow, sTouched;
    double mn = DBL_MAX, mx = -DBL_MAX;
    for (int b = threadIdx.x; b < nBlk; b += blockDim.x) {
        mn = fmin(mn, blkMin[b]);
        mx = fmax(mx, blkMax[b]);
    }
    blockReduceMinMax(mn, mx);
    if (threadIdx.x == 0) {
        sCount = 0;
        sMod = 0;
        sOverflow = 0;
        info[0] = 0;  // passes
        info[1] = 0;  // most overshooting cells in a pass
    }
    __syncthreads();
    if (!(mx - 1.0 > aTol || mn < -aTol)) return;

    // candidates: overshooting cells among the mixed cells and their face
    // neighbours (extendMarkedCells, advection.C:54-82)
    const int nm = *nMixed;
    for (int i = threadIdx.x; i < nm; i += blockDim.x) {
        const int c = mixed[i];
        if (overshoots(aNew[c])) {
            const int p = atomicAdd(&sCount, 1);
            if (p < s.candCap) s.cand[p] = c;
        }
        for (int k = m.cOff[c]; k < m.cOff[c + 1]; ++k) {
            const int nb = m.cNbr[k];
            if (nb >= 0 && overshoots(aNew[nb])) {
                const int p = atomicAdd(&sCount, 1);
                if (p < s.candCap) s.cand[p] = nb;
            }
        }
    }
    __syncthreads();
    int nCand = sCount;
    if (nCand * 2 > s.candCap) {
        if (threadIdx.x == 0) atomicOr(errOut, (uint32_t)kErrBoundOverflow);
        return;
    }
    blockBitonicSort(s.cand, nCand);
    if (threadIdx.x == 0) {  // unique
        int w = 0;
        for (int i = 0; i < nCand; ++i)
            if (w == 0 || s.cand[w - 1] != s.cand[i]) s.cand[w++] = s.cand[i];
        sCount = w;
    }
    __syncthreads();
    nCand = sCount;

    for (int pass = 0; pass < nAlphaBounds; ++pass) {
        if (!(mx - 1.0 > aTol || mn < -aTol)) break;
        if (threadIdx.x == 0) {
            info[0] = pass + 1;
            int nCorr = 0, nWritten = 0, nBoundCells = 0, nT = 0;
            int ovf = 0;
            const int passStamp = stamp * 64 + pass + 1;
            for (int ci = 0; ci < nCand && !ovf; ++ci) {
                const int c = s.cand[ci];
                const double a = aNew[c];
                if (!(a < -aTol || a > 1.0 + aTol)) continue;
                ++nBoundCells;
                const double Vi = m.V[c];
                double alphaOvershoot = pos0(a - 1.0) * (a - 1.0) + neg0(a) * a;
                double fluid = alphaOvershoot * Vi;
                int nPass = 1;
                bool firstLoop = true;
                for (int iter = 0; iter < 10; ++iter) {
                    if (fabs(alphaOvershoot) < aTol || nPass == 0) break;
                    int pf[kMaxCellFaces];
                    double pphi[kMaxCellFaces], pmax[kMaxCellFaces];
                    int np = 0;
                    double dVftot = 0.0;
                    nPass = 0;
                    for (int k = m.cOff[c]; k < m.cOff[c + 1]; ++k) {
                        const int f = m.cFaces[k];
                        const double ph = phi[f];
                        const bool down = (m.own[f] == c) ? (ph >= 0) : (ph < 0);
                        if (!down) continue;
                        const double dVff = curDVf(m, f, phi, aCur, status, dvfI, alphaB, dt, s, stamp) + s.corr[f];
                        const double maxExtra = fabs(pos0(fluid) * ph * dt - dVff);
                        if (maxExtra / Vi > aTol && np < kMaxCellFaces) {
                            pf[np] = f;
                            pphi[np] = ph;
                            pmax[np] = maxExtra;
                            ++np;
                            dVftot += fabs(ph * dt);
                        }
                    }
                    for (int fi = 0; fi < np; ++fi) {
                        const int f = pf[fi];
                        double through = fabs(fluid) * fabs(pphi[fi] * dt) / dVftot;
                        nPass += int(pos0(pmax[fi] - through));
                        through = fmin(through, pmax[fi]);
                        double dVff = s.corr[f];
                        dVff += sgn(pphi[fi]) * sgn(fluid) * through;
                        s.corr[f] = dVff;
                        if (nWritten < s.listCap) s.written[nWritten++] = f;
                        else ovf = 1;
                        if (firstLoop) {
                            if (nCorr < s.listCap) s.corrected[nCorr++] = f;
                            else ovf = 1;
                        }
                    }
                    firstLoop = false;
                    double nf1 = 0.0, nf2 = 0.0;
                    for (int k = m.cOff[c]; k < m.cOff[c + 1]; ++k) {
                        const int f = m.cFaces[k];
                        const double v1 = curDVf(m, f, phi, aCur, status, dvfI, alphaB, dt, s, stamp);
                        if (m.own[f] == c) nf1 += v1;
                        else nf1 -= v1;
                    }
                    for (int k = m.cOff[c]; k < m.cOff[c + 1]; ++k) {
                        const int f = m.cFaces[k];
                        if (m.own[f] == c) nf2 += s.corr[f];
                        else nf2 -= s.corr[f];
                    }
                    double num = aOld[c] * rDeltaT;
                    if (Su) num = num + Su[c];
                    num = num - nf1 / Vi * rDeltaT;
                    num = num - nf2 / Vi * rDeltaT;
                    const double den = Sp ? (rDeltaT - Sp[c]) : rDeltaT;
                    const double a1New = num / den;
                    alphaOvershoot = pos0(a1New - 1.0) * (a1New - 1.0) + neg0(a1New) * a1New;
                    fluid = alphaOvershoot * Vi;
                }
            }
            if (nBoundCells > info[1]) info[1] = nBoundCells;
            // apply corrections (advectionTemplates.C:164-192)
            for (int i = 0; i < nCorr; ++i) {
                const int f = s.corrected[i];
                if (s.doneStamp[f] == passStamp) continue;
                s.doneStamp[f] = passStamp;
                const double cv = s.corr[f];
                const int o = m.own[f];
                aNew[o] -= cv / m.V[o];
                if (nT < s.touchedCap) s.touched[nT++] = o;
                else ovf = 1;
                if (f < m.nfi) {
                    const int nb = m.nei[f];
                    aNew[nb] += cv / m.V[nb];
                    if (nT < s.touchedCap) s.touched[nT++] = nb;
                    else ovf = 1;
                }
                const double nv = curDVf(m, f, phi, aCur, status, dvfI, alphaB, dt, s, stamp) + cv;
                if (s.modStamp[f] != stamp) {
                    if (sMod < s.modCap) s.modList[sMod++] = f;
                    else ovf = 1;
                }
                s.dvfMod[f] = nv;
                s.modStamp[f] = stamp;
            }
            for (int i = 0; i < nWritten; ++i) s.corr[s.written[i]] = 0.0;
            // touched cells that belong to the bounding set join the candidates
            for (int i = 0; i < nT && !ovf; ++i) {
                const int t = s.touched[i];
                int lo = 0, hi = nCand;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (s.cand[mid] < t) lo = mid + 1;
                    else hi = mid;
                }
                if (lo < nCand && s.cand[lo] == t) continue;
                if (!inNeedBounding(m, t, status)) continue;
                if (nCand >= s.candCap) {
                    ovf = 1;
                    break;
                }
                for (int r = nCand; r > lo; --r) s.cand[r] = s.cand[r - 1];
                s.cand[lo] = t;
                ++nCand;
            }
            sCount = nCand;
            sTouched = nT;
            sOverflow = ovf;
        }
        __syncthreads();
        nCand = sCount;
        if (sOverflow) {
            if (threadIdx.x == 0) atomicOr(errOut, (uint32_t)kErrBoundOverflow);
            return;
        }
        // refresh the min / max partials of blocks holding touched cells
        const int nT = sTouched;
        for (int i = threadIdx.x; i < nT; i += blockDim.x) {
            const int b = s.touched[i] / blkCells;
            double bmn = DBL_MAX, bmx = -DBL_MAX;
            const int e = min(m.nc, (b + 1) * blkCells);
            for (int c = b * blkCells; c < e; ++c) {
                bmn = fmin(bmn, aNew[c]);
                bmx = fmax(bmx, aNew[c]);
            }
            blkMin[b] = bmn;  // identical value from every thread touching b
            blkMax[b] = bmx;
        }
        __syncthreads();
        mn = DBL_MAX;
        mx = -DBL_MAX;
        for (int b = threadIdx.x; b < nBlk; b += blockDim.x) {
            mn = fmin(mn, blkMin[b]);
            mx = fmax(mx, blkMax[b]);
        }
        blockReduceMinMax(mn, mx);
    }
    __syncthreads();
    // alphaPhi = dVf / dt for faces changed by the bounding
    const int nMod = sMod;
    for (int i = threadIdx.x; i < nMod; i += blockDim.x) {
        const int f = s.modList[i];
        alphaPhi[f] = s.dvfMod[f] / dt;
    }
}

// ---------------------------------------------------------------------------
// K7: snapping and clipping
// ---------------------------------------------------------------------------
__global__ void kBruteForce(int nc, double* __restrict__ a, double snap, int clip) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double x = a[c];
    if (snap > 0.0) x = x * pos0(x - snap) * neg0(x - (1.0 - snap)) + pos0(x - (1.0 - snap));
    if (clip) x = fmin(1.0, fmax(0.0, x));
    a[c] = x;
}

// ---------------------------------------------------------------------------
// face flatness (one-time, reconstruction.C:408-440)
// ---------------------------------------------------------------------------
__global__ void kFaceFlatness(DevMesh m, const double* __restrict__ Sf, double* __restrict__ flat) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.nf) return;
    const int q0 = m.fOff[f], n = m.fOff[f + 1] - q0;
    const double magA = mag(ld3(Sf, f));
    double out = 1.0;
    if (n > 3 && magA > kROOTVSMALL) {
        const d3 fc = ld3(m.Cf, f);
        double sumA = 0.0;
        for (int i = 0; i < n; ++i) {
            const d3 th = ld3(m.pts, m.fPts[q0 + i]);
            const d3 nx = ld3(m.pts, m.fPts[q0 + (i + 1) % n]);
            sumA += mag(0.5 * cross(nx - th, fc - th));
        }
        out = magA / (sumA + kROOTVSMALL);
    }
    flat[f] = out;
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static int persistentGrid(int threads) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms * (threads >= 256 ? 4 : 8);
}

void launchScanMixed(const StepArgs& a, cudaStream_t st) {
    const int nb = (a.m.nc + 255) / 256;
    kScanMixed<<<nb, 256, 0, st>>>(a.m.nc, a.aCur, a.mixedTol, a.status, a.mixed, a.nMixed);
}

void launchLsNormal(const StepArgs& a, cudaStream_t st) {
    kLsNormal<<<persistentGrid(128), 128, 0, st>>>(a.m, a.aCur, a.mixed, a.nMixed, a.nrm, a.err);
}

void launchPlaneSolve(const StepArgs& a, cudaStream_t st) {
    kPlaneSolve<<<persistentGrid(128), 128, 0, st>>>(a.m, a.aCur, a.mixed, a.nMixed, a.nrm, a.mStatus, a.status,
                                                    a.dArr, a.icArr, a.isArr, a.err);
}

void launchInterfaceFlux(const StepArgs& a, cudaStream_t st) {
    kInterfaceFlux<<<persistentGrid(128), 128, 0, st>>>(a.m, a.mixed, a.nMixed, a.mStatus, a.nrm, a.dArr, a.icArr,
                                                       a.phi, a.U, a.Ub, a.dt, a.dvfI, a.cutMask);
}

void launchUpdate(const StepArgs& a, cudaStream_t st) {
    const int nb = (a.m.nc + 255) / 256;
    kUpdate<<<nb, 256, 0, st>>>(a.m, a.phi, a.aCur, a.aOld, a.aNew, a.status, a.dvfI, a.alphaB, a.Sp, a.Su, a.dt,
                                a.rDeltaT, a.alphaPhi, a.blkMin, a.blkMax);
}

void launchBound(const StepArgs& a, const BoundBuffers& b, cudaStream_t st) {
    BoundScratch s;
    s.cand = b.cand;
    s.candCap = b.candCap;
    s.corr = b.corr;
    s.dvfMod = b.dvfMod;
    s.modStamp = b.modStamp;
    s.doneStamp = b.doneStamp;
    s.corrected = b.corrected;
    s.written = b.written;
    s.listCap = b.listCap;
    s.modList = b.modList;
    s.modCap = b.modCap;
    s.touched = b.touched;
    s.touchedCap = b.touchedCap;
    const int nBlk = (a.m.nc + 255) / 256;
    kBound<<<1, 1024, 0, st>>>(a.m, a.phi, a.aCur, a.aOld, a.aNew, a.status, a.mixed, a.nMixed, a.dvfI, a.alphaB,
                               a.Sp, a.Su, a.dt, a.rDeltaT, a.nAlphaBounds, a.blkMin, a.blkMax, nBlk, 256,
                               a.alphaPhi, s, b.stamp, b.info, a.err);
}

void launchBruteForce(const StepArgs& a, cudaStream_t st) {
    if (!(a.snapTol > 0.0) && !a.clip) return;
    const int nb = (a.m.nc + 255) / 256;
    kBruteForce<<<nb, 256, 0, st>>>(a.m.nc, a.aNew, a.snapTol, a.clip);
}

void launchFaceFlatness(const DevMesh& m, const double* Sf, double* flat, cudaStream_t st) {
    kFaceFlatness<<<(m.nf + 255) / 256, 256, 0, st>>>(m, Sf, flat);
}

}  // namespace simplic
