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
// K3: plane constant per mixed cell (cutCell::findSignedDistance) in three
// phases.  The bracketing loop only compares the VOF at the vertex levels
// it visits, so (a) the VOF of every interior vertex level is computed in
// parallel, one thread per (cell, level); (b) the loop is replayed over
// those values and the 1/3 and 2/3 evaluations run as two threads per cell;
// (c) Newton on the cubic and the final cut, one thread per cell.  Every
// calcSubCell is the same computation as in the serial algorithm, so the
// results are identical to it.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void writePlane(const PlaneArgs& p, int i, int c, int st, double d, d3 ic, d3 is) {
    p.mStatus[i] = int8_t(st);
    p.status[c] = int8_t(st);
    p.dOut[i] = d;
    st3(p.icOut, i, ic);
    st3(p.isOut, i, is);
}

__global__ void __launch_bounds__(128) kPlaneLevels(DevMesh m, PlaneArgs p) {
    const int nm = *p.nMixed;
    uint32_t err = 0;
    const long long total = (long long)nm * kLvThreads;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = int(t / kLvThreads), j = int(t % kLvThreads);
        const int c = p.mixed[i];
        const int np = m.cpOff[c + 1] - m.cpOff[c];
        if (j + 1 > np - 2) continue;
        const d3 nI = ld3(p.nrm, i);
        if (mag(nI) < kTSMALL) continue;
        CellWS w;
        if (!loadCell(m, c, w)) {
            err |= kErrSubFaceOverflow;
            continue;
        }
        double vd[kMaxCellPts];
        int order[kMaxCellPts];
        vertexOrder(w, nI, vd, order);
        for (int k = j + 1; k <= np - 2; k += kLvThreads) {
            SubCell sc;
            calcSubCell(w, nI, vd[order[k]], sc, err);
            p.lvVof[size_t(i) * kLvSlots + (k - 1)] = sc.vof;
        }
    }
    if (err) atomicOr(p.err, err);
}

__global__ void __launch_bounds__(128) kPlaneThirds(DevMesh m, PlaneArgs p) {
    const int nm = *p.nMixed;
    uint32_t err = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 2LL * nm;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = int(t >> 1), q = int(t & 1);
        const int c = p.mixed[i];
        const double alphaI = p.alpha[c];
        const d3 nI = ld3(p.nrm, i);
        if (mag(nI) < kTSMALL) {  // cutCell.C:625-628: no plane is written
            if (q == 0) {
                writePlane(p, i, c, int(sgn(0.5 - alphaI)), 0.0, mk(0, 0, 0), mk(0, 0, 0));
                p.done[i] = 1;
            }
            continue;
        }
        CellWS w;
        if (!loadCell(m, c, w)) {
            err |= kErrSubFaceOverflow;
            if (q == 0) {
                writePlane(p, i, c, 1, 0.0, mk(0, 0, 0), mk(0, 0, 0));
                p.done[i] = 1;
            }
            continue;
        }
        double vd[kMaxCellPts];
        int order[kMaxCellPts];
        vertexOrder(w, nI, vd, order);
        const Bracket br = replayBracketing(vd, order, w.np, alphaI, p.lvVof + size_t(i) * kLvSlots);
        SubCell sc;
        if (br.exitLevel >= 0) {
            if (q == 0) {
                const double dm = vd[order[br.exitLevel]];
                calcSubCell(w, nI, dm, sc, err);
                writePlane(p, i, c, sc.status, dm, sc.ic, sc.is);
                p.done[i] = 1;
            }
            continue;
        }
        if (fabs(br.lowD - br.upD) < kTSMALL) {
            if (q == 0) {
                const double dm = 0.5 * (br.lowD + br.upD);
                calcSubCell(w, nI, dm, sc, err);
                writePlane(p, i, c, sc.status, dm, sc.ic, sc.is);
                p.done[i] = 1;
            }
            continue;
        }
        const double deltaDistance = (br.upD - br.lowD) / 3.0;
        const double dq = (q == 0) ? br.lowD + deltaDistance : br.lowD + 2.0 * deltaDistance;
        calcSubCell(w, nI, dq, sc, err);
        p.v13[2 * size_t(i) + q] = sc.vof;
        if (q == 0) p.done[i] = 0;
    }
    if (err) atomicOr(p.err, err);
}

__global__ void __launch_bounds__(128) kPlaneFinal(DevMesh m, PlaneArgs p) {
    const int nm = *p.nMixed;
    uint32_t err = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nm; i += gridDim.x * blockDim.x) {
        if (p.done[i]) continue;
        const int c = p.mixed[i];
        const double alphaI = p.alpha[c];
        const d3 nI = ld3(p.nrm, i);
        CellWS w;
        if (!loadCell(m, c, w)) {
            err |= kErrSubFaceOverflow;
            continue;
        }
        double vd[kMaxCellPts];
        int order[kMaxCellPts];
        vertexOrder(w, nI, vd, order);
        const Bracket br = replayBracketing(vd, order, w.np, alphaI, p.lvVof + size_t(i) * kLvSlots);
        const double d0 = cubicDistance(br, p.v13[2 * size_t(i)], p.v13[2 * size_t(i) + 1], alphaI);
        SubCell sc;
        calcSubCell(w, nI, d0, sc, err);
        writePlane(p, i, c, sc.status, d0, sc.ic, sc.is);
    }
    if (err) atomicOr(p.err, err);
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

// (a) interface speed Un0 = U(interface centre) . n of every cut cell
__global__ void __launch_bounds__(128) kInterfaceUn0(DevMesh m, const int* __restrict__ mixed,
                                                     const int* __restrict__ nMixed,
                                                     const int8_t* __restrict__ mStatus,
                                                     const double* __restrict__ nrm, const double* __restrict__ icArr,
                                                     const double* __restrict__ U, const double* __restrict__ Ub,
                                                     double* __restrict__ un0) {
    const int nm = *nMixed;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nm; i += gridDim.x * blockDim.x) {
        if (mStatus[i] != 0) continue;
        const int c = mixed[i];
        un0[i] = dot(interpolateU(m, c, ld3(icArr, i), U, Ub), ld3(nrm, i));
    }
}

// (b) one thread per (cut cell, face slot): Simpson flux of the downwind faces
__global__ void __launch_bounds__(128) kInterfaceFaces(DevMesh m, const int* __restrict__ mixed,
                                                       const int* __restrict__ nMixed,
                                                       const int8_t* __restrict__ mStatus,
                                                       const double* __restrict__ nrm, const double* __restrict__ dArr,
                                                       const double* __restrict__ un0, const double* __restrict__ phi,
                                                       double dt, double* __restrict__ dvfI,
                                                       uint8_t* __restrict__ cutMask) {
    const int nm = *nMixed;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)nm * kMaxCellFaces;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = int(t / kMaxCellFaces), k = int(t % kMaxCellFaces);
        if (mStatus[i] != 0) continue;
        const int c = mixed[i];
        const int k0 = m.cOff[c];
        if (k >= m.cOff[c + 1] - k0) continue;
        const int f = m.cFaces[k0 + k];
        const double ph = phi[f];
        bool down;
        if (f < m.nfi)
            down = (c == m.own[f]) ? (ph >= 0.0) : (ph < 0.0);
        else
            down = ph >= 0.0;
        if (!down) continue;
        dvfI[f] = timeIntegratedFaceFlux(m, f, ld3(nrm, i), dArr[i], un0[i], dt, ph, m.magSf[f]);
        if (cutMask) cutMask[f] = 1;
    }
}

// ---------------------------------------------------------------------------
// K5: upwind flux, interface overrides, surfaceIntegrate and alpha update
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) kUpdate(DevMesh m, const double* __restrict__ phi,
                                               const double* __restrict__ aCur, const double* __restrict__ aOld,
                                               double* __restrict__ aNew, const int8_t* __restrict__ status,
                                               const double* __restrict__ dvfI, const double* __restrict__ alphaB,
                                               const double* __restrict__ Sp, const double* __restrict__ Su,
                                               double dt, double rDeltaT, double* __restrict__ alphaPhi,
                                               double* __restrict__ blkMin, double* __restrict__ blkMax,
                                               int* __restrict__ ovList, int* __restrict__ ovCount, int ovCap) {
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
    // cells outside [-aTol, 1 + aTol] are the bounding kernel's candidates
    const double aTol = 100.0 * kSMALL;
    const bool ov = valid && (an < -aTol || an > 1.0 + aTol);
    const unsigned ball = __ballot_sync(0xffffffffu, ov);
    if (ball) {
        const int lane = threadIdx.x & 31;
        int base = 0;
        if (lane == 0) base = atomicAdd(ovCount, __popc(ball));
        base = __shfl_sync(0xffffffffu, base, 0);
        const int p = base + __popc(ball & ((1u << lane) - 1u));
        if (ov && p < ovCap) ovList[p] = c;
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

static PlaneArgs planeArgs(const StepArgs& a) {
    PlaneArgs p;
    p.alpha = a.aCur;
    p.mixed = a.mixed;
    p.nMixed = a.nMixed;
    p.nrm = a.nrm;
    p.mStatus = a.mStatus;
    p.status = a.status;
    p.dOut = a.dArr;
    p.icOut = a.icArr;
    p.isOut = a.isArr;
    p.lvVof = a.lvVof;
    p.v13 = a.v13;
    p.done = a.done;
    p.err = a.err;
    return p;
}

void launchPlaneLevels(const StepArgs& a, cudaStream_t st) {
    kPlaneLevels<<<persistentGrid(128) * 4, 128, 0, st>>>(a.m, planeArgs(a));
}

void launchPlaneThirds(const StepArgs& a, cudaStream_t st) {
    kPlaneThirds<<<persistentGrid(128) * 2, 128, 0, st>>>(a.m, planeArgs(a));
}

void launchPlaneFinal(const StepArgs& a, cudaStream_t st) {
    kPlaneFinal<<<persistentGrid(128), 128, 0, st>>>(a.m, planeArgs(a));
}

void launchInterfaceUn0(const StepArgs& a, cudaStream_t st) {
    kInterfaceUn0<<<persistentGrid(128), 128, 0, st>>>(a.m, a.mixed, a.nMixed, a.mStatus, a.nrm, a.icArr, a.U, a.Ub,
                                                      a.un0);
}

void launchInterfaceFaces(const StepArgs& a, cudaStream_t st) {
    kInterfaceFaces<<<persistentGrid(128) * 4, 128, 0, st>>>(a.m, a.mixed, a.nMixed, a.mStatus, a.nrm, a.dArr,
                                                            a.un0, a.phi, a.dt, a.dvfI, a.cutMask);
}

void launchUpdate(const StepArgs& a, cudaStream_t st) {
    const int nb = (a.m.nc + 255) / 256;
    kUpdate<<<nb, 256, 0, st>>>(a.m, a.phi, a.aCur, a.aOld, a.aNew, a.status, a.dvfI, a.alphaB, a.Sp, a.Su, a.dt,
                                a.rDeltaT, a.alphaPhi, a.blkMin, a.blkMax, a.ovList, a.ovCount, a.ovCap);
}

void launchBruteForce(const StepArgs& a, cudaStream_t st) {
    if (!(a.snapTol > 0.0) && !a.clip) return;
    const int nb = (a.m.nc + 255) / 256;
    kBruteForce<<<nb, 256, 0, st>>>(a.m.nc, a.aNew, a.snapTol, a.clip);
}

void launchFaceFlatness(const DevMesh& m, const double* Sf, double* flat, cudaStream_t st) {
    kFaceFlatness<<<(m.nf + 255) / 256, 256, 0, st>>>(m, Sf, flat);
}

// face::centre and face::areaNormal of every face (one-time): what
// calcSubFace returns for a fully submerged face (cutFace.C:184-185)
__global__ void kFaceFull(DevMesh m, double* __restrict__ fullC, double* __restrict__ fullA) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.nf) return;
    const int q0 = m.fOff[f], n = m.fOff[f + 1] - q0;
    d3 fp[kMaxFacePts];
    for (int i = 0; i < n; ++i) fp[i] = ld3(m.pts, m.fPts[q0 + i]);
    st3(fullC, f, faceCentreOF(fp, n));
    st3(fullA, f, faceAreaNormalOF(fp, n));
}

void launchFaceFull(const DevMesh& m, double* fullC, double* fullA, cudaStream_t st) {
    kFaceFull<<<(m.nf + 255) / 256, 256, 0, st>>>(m, fullC, fullA);
}

}  // namespace simplic
