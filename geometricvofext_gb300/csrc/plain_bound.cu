// Conservative bounding of the plain FP64 form: advection::limitFlux and
// advection::boundFlux (src/SimPLIC/advection/advectionTemplates.C:118-349)
// with extendMarkedCells / netFlux / setDownwindFaces (advection.C:54-82,
// 224-288).  Built with -fmad=false.
//
// The reference walks the bounding set in ascending cell order and a cell
// reads the flux corrections that earlier cells wrote during the same pass,
// so the loop is order dependent.  A cell only reads corrections on its own
// faces, and only the face-adjacent cells write those, so the result is the
// same as long as every cell runs after its earlier face-adjacent
// overshooting neighbours and before its later ones.  One block therefore:
//   1. takes the overshooting cells appended by the update kernel, keeps the
//      ones in the bounding set (mixed cells and their face neighbours) and
//      sorts them;
//   2. gives each a dependency level (1 + the deepest earlier face-adjacent
//      candidate) and runs the levels one after another, the cells of a
//      level in parallel;
//   3. applies the corrections to alpha per target cell in the reference's
//      list order (the order of the floating-point updates is kept);
//   4. refreshes the per-block min / max of alpha for the next pass test.
#include <cfloat>
#include <climits>

#include "plain_geom.cuh"
#include "simplic_kernels.h"

namespace simplic {

namespace {

constexpr double kATol = 100.0 * kSMALL;  // advectionTemplates.C:125,228

__device__ __forceinline__ bool overshoots(double a) { return a < -kATol || a > 1.0 + kATol; }

__device__ __forceinline__ double curDVf(const DevMesh& m, int f, const double* phi, const double* aCur,
                                         const int8_t* status, const double* dvfI, const double* alphaB, double dt,
                                         const BoundBuffers& s, int stamp) {
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

__device__ __forceinline__ int findSorted(const int* a, int n, int x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return (lo < n && a[lo] == x) ? lo : -1;
}

__device__ void blockMinMax(double& mn, double& mx) {
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
}

template <class K>
__device__ void blockBitonicSort(K* a, int n, K pad) {
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (int i = n + threadIdx.x; i < n2; i += blockDim.x) a[i] = pad;
    __syncthreads();
    for (int k = 2; k <= n2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const K ai = a[i], al = a[l];
                    if ((ai > al) == ((i & k) == 0)) {
                        a[i] = al;
                        a[l] = ai;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// The body of the reference's cell loop (advectionTemplates.C:245-347) for
// one overshooting cell.  Face data is read once: dVf does not change within
// a pass, and the corrections on this cell's faces were final once the
// earlier face-adjacent cells ran.  Writes the cell's corrections back and
// records its first-iteration ("corrected") faces.
__device__ void boundCell(const DevMesh& m, int c, const double* phi, const double* aCur, const double* aOld,
                          const double* aNew, const int8_t* status, const double* dvfI, const double* alphaB,
                          const double* Sp, const double* Su, double dt, double rDeltaT, const BoundBuffers& s,
                          int stamp, int ci) {
    const int k0 = m.cOff[c], nfc = m.cOff[c + 1] - k0;
    int F[kMaxCellFaces];
    bool own[kMaxCellFaces], down[kMaxCellFaces], wrote[kMaxCellFaces];
    double ph[kMaxCellFaces], dv[kMaxCellFaces], cr[kMaxCellFaces];
    double nf1 = 0.0;  // netFlux(c, dVf): the same every iteration
    for (int k = 0; k < nfc; ++k) {
        const int f = m.cFaces[k0 + k];
        F[k] = f;
        own[k] = m.own[f] == c;
        ph[k] = phi[f];
        dv[k] = curDVf(m, f, phi, aCur, status, dvfI, alphaB, dt, s, stamp);
        cr[k] = s.corr[f];
        down[k] = own[k] ? (ph[k] >= 0) : (ph[k] < 0);
        wrote[k] = false;
        if (own[k]) nf1 += dv[k];
        else nf1 -= dv[k];
    }
    const double a = aNew[c];
    const double Vi = m.V[c];
    double alphaOvershoot = pos0(a - 1.0) * (a - 1.0) + neg0(a) * a;
    double fluid = alphaOvershoot * Vi;
    int nPass = 1, nCorr = 0;
    bool firstLoop = true;
    int* corrOut = s.candCorr + size_t(ci) * kMaxCellFaces;
    for (int iter = 0; iter < 10; ++iter) {
        if (fabs(alphaOvershoot) < kATol || nPass == 0) break;
        int pk[kMaxCellFaces];
        double pmax[kMaxCellFaces];
        int np = 0;
        double dVftot = 0.0;
        nPass = 0;
        for (int k = 0; k < nfc; ++k) {
            if (!down[k]) continue;
            const double dVff = dv[k] + cr[k];
            const double maxExtra = fabs(pos0(fluid) * ph[k] * dt - dVff);
            if (maxExtra / Vi > kATol) {
                pk[np] = k;
                pmax[np] = maxExtra;
                ++np;
                dVftot += fabs(ph[k] * dt);
            }
        }
        for (int q = 0; q < np; ++q) {
            const int k = pk[q];
            double through = fabs(fluid) * fabs(ph[k] * dt) / dVftot;
            nPass += int(pos0(pmax[q] - through));
            through = fmin(through, pmax[q]);
            double dVff = cr[k];
            dVff += sgn(ph[k]) * sgn(fluid) * through;
            cr[k] = dVff;
            wrote[k] = true;
            if (firstLoop) corrOut[nCorr++] = F[k];
        }
        firstLoop = false;
        double nf2 = 0.0;
        for (int k = 0; k < nfc; ++k) {
            if (own[k]) nf2 += cr[k];
            else nf2 -= cr[k];
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
    int nW = 0;
    int* wOut = s.candWritten + size_t(ci) * kMaxCellFaces;
    for (int k = 0; k < nfc; ++k)
        if (wrote[k]) {
            s.corr[F[k]] = cr[k];
            wOut[nW++] = F[k];
        }
    s.candNCorr[ci] = nCorr;
    s.candNWritten[ci] = nW;
}

// Phase timers (SM clock cycles, summed by thread 0): 0 setup, 1 levels,
// 2 cell work, 3 apply, 4 min/max refresh, 5 candidate merge, 6 alphaPhi.
#define BOUND_TICK(k)                             \
    do {                                          \
        if (threadIdx.x == 0) {                   \
            const long long _t = clock64();       \
            s.prof[k] += _t - tp;                 \
            tp = _t;                              \
        }                                         \
    } while (0)

__global__ void __launch_bounds__(1024) kBound(StepArgs a, BoundBuffers s, int nBlk, int blkCells) {
    const DevMesh& m = a.m;
    __shared__ int sCount, sMaxLevel, sChanged, sOverflow, sList, sRec, sNBlk;
    long long tp = clock64();
    double mn = DBL_MAX, mx = -DBL_MAX;
    for (int b = threadIdx.x; b < nBlk; b += blockDim.x) {
        mn = fmin(mn, a.blkMin[b]);
        mx = fmax(mx, a.blkMax[b]);
    }
    blockMinMax(mn, mx);
    if (threadIdx.x == 0) {
        sCount = 0;
        sOverflow = 0;
        s.info[0] = 0;
        s.info[1] = 0;
        s.info[2] = 0;
    }
    __syncthreads();
    if (!(mx - 1.0 > kATol || mn < -kATol)) return;

    // 1. candidates: overshooting cells of the bounding set, ascending
    const int nOv = min(*s.ovCount, s.ovCap);
    if (*s.ovCount > s.ovCap || 2 * nOv > s.candCap) {
        if (threadIdx.x == 0) atomicOr(a.err, (uint32_t)kErrBoundOverflow);
        return;
    }
    for (int i = threadIdx.x; i < nOv; i += blockDim.x) {
        const int c = s.ovList[i];
        if (inNeedBounding(m, c, a.status)) {
            const int p = atomicAdd(&sCount, 1);
            s.cand[p] = c;
        }
    }
    __syncthreads();
    int nCand = sCount;
    blockBitonicSort(s.cand, nCand, INT_MAX);
    BOUND_TICK(0);

    for (int pass = 0; pass < a.nAlphaBounds; ++pass) {
        if (!(mx - 1.0 > kATol || mn < -kATol)) break;
        if (threadIdx.x == 0) s.info[0] = pass + 1;
        // 2a. active cells and their earlier active face neighbours
        for (int i = threadIdx.x; i < nCand; i += blockDim.x) {
            const int c = s.cand[i];
            const bool act = overshoots(a.aNew[c]);
            s.candLevel[i] = act ? 0 : -1;
            int nd = 0;
            if (act) {
                for (int k = m.cOff[c]; k < m.cOff[c + 1]; ++k) {
                    const int nb = m.cNbr[k];
                    if (nb < 0 || nb > c) continue;
                    const int j = findSorted(s.cand, i, nb);
                    if (j >= 0 && overshoots(a.aNew[nb])) s.candDeps[size_t(i) * kMaxCellFaces + nd++] = j;
                }
            }
            s.candNDeps[i] = nd;
            s.candNCorr[i] = 0;
            s.candNWritten[i] = 0;
        }
        __syncthreads();
        // 2b. longest-path levels by relaxation (levels only grow)
        for (;;) {
            if (threadIdx.x == 0) sChanged = 0;
            __syncthreads();
            for (int i = threadIdx.x; i < nCand; i += blockDim.x) {
                if (s.candLevel[i] < 0) continue;
                int L = 0;
                const int* d = s.candDeps + size_t(i) * kMaxCellFaces;
                for (int q = 0; q < s.candNDeps[i]; ++q) L = max(L, ((volatile int*)s.candLevel)[d[q]] + 1);
                if (L > s.candLevel[i]) {
                    s.candLevel[i] = L;
                    sChanged = 1;
                }
            }
            __syncthreads();
            const int changed = sChanged;
            __syncthreads();  // every thread has read the flag before it is reset
            if (!changed) break;
        }
        if (threadIdx.x == 0) sMaxLevel = -1;
        __syncthreads();
        int lmax = -1;
        for (int i = threadIdx.x; i < nCand; i += blockDim.x) lmax = max(lmax, s.candLevel[i]);
        atomicMax(&sMaxLevel, lmax);
        __syncthreads();
        BOUND_TICK(1);
        // 2c. the levels in order, the cells of a level in parallel
        const int maxL = sMaxLevel;
        for (int L = 0; L <= maxL; ++L) {
            for (int i = threadIdx.x; i < nCand; i += blockDim.x)
                if (s.candLevel[i] == L)
                    boundCell(m, s.cand[i], a.phi, a.aCur, a.aOld, a.aNew, a.status, a.dvfI, a.alphaB, a.Sp, a.Su,
                              a.dt, a.rDeltaT, s, s.stamp, i);
            __syncthreads();
        }
        BOUND_TICK(2);
        if (threadIdx.x == 0) {
            int n = 0;
            for (int i = 0; i < nCand; ++i) n += s.candLevel[i] >= 0;
            if (n > s.info[1]) s.info[1] = n;
            if (maxL + 1 > s.info[2]) s.info[2] = maxL + 1;
            // 3a. the corrected-face list in the reference's order: cells
            // ascending, each cell's first-iteration faces in its order
            int tot = 0;
            for (int i = 0; i < nCand; ++i) {
                s.candListOff[i] = tot;
                tot += s.candNCorr[i];
            }
            sList = tot;
            if (4 * tot + 4 > s.recCap) sOverflow = 1;
        }
        __syncthreads();
        if (sOverflow) {
            if (threadIdx.x == 0) atomicOr(a.err, (uint32_t)kErrBoundOverflow);
            return;
        }
        const int nList = sList;
        for (int i = threadIdx.x; i < nCand; i += blockDim.x) {
            const int o = s.candListOff[i];
            for (int q = 0; q < s.candNCorr[i]; ++q) s.list[o + q] = s.candCorr[size_t(i) * kMaxCellFaces + q];
        }
        __syncthreads();
        // 3b. alpha updates keyed (target cell, position in the list)
        if (threadIdx.x == 0) sRec = 0;
        __syncthreads();
        for (int e = threadIdx.x; e < nList; e += blockDim.x) {
            const int f = s.list[e];
            const int p = atomicAdd(&sRec, f < m.nfi ? 2 : 1);
            s.rec[p] = ((long long)m.own[f] << 22) | (long long)(2 * e);
            if (f < m.nfi) s.rec[p + 1] = ((long long)m.nei[f] << 22) | (long long)(2 * e + 1);
        }
        __syncthreads();
        const int nRec = sRec;
        blockBitonicSort(s.rec, nRec, (long long)LLONG_MAX);
        for (int r = threadIdx.x; r < nRec; r += blockDim.x) {
            const int t = int(s.rec[r] >> 22);
            if (r > 0 && int(s.rec[r - 1] >> 22) == t) continue;
            double at = a.aNew[t];
            const double Vt = m.V[t];
            for (int q = r; q < nRec && int(s.rec[q] >> 22) == t; ++q) {
                const int seq = int(s.rec[q] & ((1LL << 22) - 1));
                const double cv = s.corr[s.list[seq >> 1]];
                if (seq & 1) at += cv / Vt;
                else at -= cv / Vt;
            }
            a.aNew[t] = at;
        }
        // dVf of the corrected faces (each face appears once in the list)
        for (int e = threadIdx.x; e < nList; e += blockDim.x) {
            const int f = s.list[e];
            const double nv = curDVf(m, f, a.phi, a.aCur, a.status, a.dvfI, a.alphaB, a.dt, s, s.stamp) + s.corr[f];
            if (s.modStamp[f] != s.stamp) {
                const int p = atomicAdd(s.modCount, 1);
                if (p < s.modCap) s.modList[p] = f;
                else atomicOr(a.err, (uint32_t)kErrBoundOverflow);
            }
            s.dvfMod[f] = nv;
            s.modStamp[f] = s.stamp;
        }
        __syncthreads();
        // 3c. clear this pass's corrections
        for (int i = threadIdx.x; i < nCand; i += blockDim.x) {
            const int* w = s.candWritten + size_t(i) * kMaxCellFaces;
            for (int q = 0; q < s.candNWritten[i]; ++q) s.corr[w[q]] = 0.0;
        }
        // the min / max blocks holding touched cells (targets are sorted, so
        // a block starts where the block id of consecutive targets changes)
        if (threadIdx.x == 0) sNBlk = 0;
        __syncthreads();
        BOUND_TICK(3);
        for (int r = threadIdx.x; r < nRec; r += blockDim.x) {
            const int b = int(s.rec[r] >> 22) / blkCells;
            if (r > 0 && int(s.rec[r - 1] >> 22) / blkCells == b) continue;
            s.list[atomicAdd(&sNBlk, 1)] = b;  // the face list is no longer needed
        }
        __syncthreads();
        // 4. refresh those partials, one warp per block
        const int nTB = sNBlk;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nWarps = blockDim.x >> 5;
        for (int q = warp; q < nTB; q += nWarps) {
            const int b = s.list[q];
            double bmn = DBL_MAX, bmx = -DBL_MAX;
            const int e = min(m.nc, (b + 1) * blkCells);
            for (int c = b * blkCells + lane; c < e; c += 32) {
                const double v = a.aNew[c];
                bmn = fmin(bmn, v);
                bmx = fmax(bmx, v);
            }
            for (int o = 16; o > 0; o >>= 1) {
                bmn = fmin(bmn, __shfl_xor_sync(0xffffffffu, bmn, o));
                bmx = fmax(bmx, __shfl_xor_sync(0xffffffffu, bmx, o));
            }
            if (lane == 0) {
                a.blkMin[b] = bmn;
                a.blkMax[b] = bmx;
            }
        }
        __syncthreads();
        mn = DBL_MAX;
        mx = -DBL_MAX;
        for (int b = threadIdx.x; b < nBlk; b += blockDim.x) {
            mn = fmin(mn, a.blkMin[b]);
            mx = fmax(mx, a.blkMax[b]);
        }
        blockMinMax(mn, mx);
        BOUND_TICK(4);
        // 5. touched cells of the bounding set join the candidates
        if (threadIdx.x == 0) sCount = nCand;
        __syncthreads();
        for (int r = threadIdx.x; r < nRec; r += blockDim.x) {
            const int t = int(s.rec[r] >> 22);
            if (r > 0 && int(s.rec[r - 1] >> 22) == t) continue;
            if (findSorted(s.cand, nCand, t) >= 0 || !inNeedBounding(m, t, a.status)) continue;
            const int p = atomicAdd(&sCount, 1);
            if (2 * (p + 1) <= s.candCap) s.cand[p] = t;
            else sOverflow = 1;
        }
        __syncthreads();
        if (sOverflow) {
            if (threadIdx.x == 0) atomicOr(a.err, (uint32_t)kErrBoundOverflow);
            return;
        }
        nCand = sCount;
        blockBitonicSort(s.cand, nCand, INT_MAX);
        BOUND_TICK(5);
    }
    __syncthreads();
    // alphaPhi = dVf / dt of every face the bounding changed this step
    const int nMod = min(*s.modCount, s.modCap);
    for (int i = threadIdx.x; i < nMod; i += blockDim.x) {
        const int f = s.modList[i];
        a.alphaPhi[f] = s.dvfMod[f] / a.dt;
    }
    BOUND_TICK(6);
}

}  // namespace

void launchBound(const StepArgs& a, const BoundBuffers& b, cudaStream_t st) {
    const int nBlk = (a.m.nc + 255) / 256;
    kBound<<<1, 1024, 0, st>>>(a, b, nBlk, 256);
}

}  // namespace simplic
