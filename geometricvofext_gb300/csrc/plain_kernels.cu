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
#include "ls_fp64.cuh"
#include "plain_geom.cuh"
#include "simplic_kernels.h"

#include <cfloat>
#include <climits>
#include <cstring>
#include <mutex>

namespace simplic {

// ---------------------------------------------------------------------------
// K1: mixed-cell list (warp-aggregated append) and per-cell status bytes
// ---------------------------------------------------------------------------
// isAMixedCell (reconstruction.H:281-288): tol < a < 1 - tol.  Evaluated on
// the bit patterns: for 0 <= tol < 0.5 the signed 64-bit order of a double's
// bits matches its numeric order on [+0, +inf], negative values fail the
// first test and NaN fails the second, exactly as the double comparisons do
// -- and it keeps the narrow FP64 pipe out of this memory-bound scan.
__global__ void __launch_bounds__(256) kScanMixed(int nc, const double* __restrict__ alpha, long long tolBits,
                                                  long long oneMinusTolBits, int8_t* __restrict__ status,
                                                  int* __restrict__ mixed, int* __restrict__ nMixed,
                                                  uint32_t* __restrict__ err) {
    // four cells per thread: two 16-byte loads, one 4-byte status store
    const int c0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    unsigned flags = 0;
    bool bad = false;  // a NaN or an infinity (all exponent bits set)
    const auto nonFinite = [](long long v) { return (v & 0x7ff0000000000000LL) == 0x7ff0000000000000LL; };
    if (c0 + 3 < nc) {
        const double2 p = *reinterpret_cast<const double2*>(alpha + c0);
        const double2 q = *reinterpret_cast<const double2*>(alpha + c0 + 2);
        const long long v[4] = {bitsOf(p.x), bitsOf(p.y), bitsOf(q.x), bitsOf(q.y)};
        uint32_t st = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool mx = v[k] > tolBits && v[k] < oneMinusTolBits;
            flags |= unsigned(mx) << k;
            bad = bad || nonFinite(v[k]);
            st |= uint32_t(uint8_t(mx ? kStPending : kStNotMixed)) << (8 * k);
        }
        *reinterpret_cast<uint32_t*>(status + c0) = st;
    } else {
        for (int k = 0; k < 4 && c0 + k < nc; ++k) {
            const long long v = bitsOf(alpha[c0 + k]);
            const bool mx = v > tolBits && v < oneMinusTolBits;
            flags |= unsigned(mx) << k;
            bad = bad || nonFinite(v);
            status[c0 + k] = mx ? kStPending : kStNotMixed;
        }
    }
    // a non-finite alpha is reported (the reference would carry it into
    // every neighbour's flux without notice)
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(err, (uint32_t)kErrNonFinite);
    // the mixed cells in ascending order within each thread, one atomic per warp
    const int lane = threadIdx.x & 31;
    const int cnt = __popc(flags);
    int incl = cnt;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    if (total == 0) return;
    int base = 0;
    if (lane == 31) base = atomicAdd(nMixed, total);
    base = __shfl_sync(0xffffffffu, base, 31) + incl - cnt;
    for (int k = 0; k < 4; ++k)
        if ((flags >> k) & 1u) mixed[base++] = c0 + k;
}

// ---------------------------------------------------------------------------
// K2: least-squares normal (polyDegree1 fit over the cell-point-cell stencil)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) kLsNormal(DevMesh m, const double* __restrict__ alpha,
                                                 const int* __restrict__ mixed, const int* __restrict__ nMixed,
                                                 double* __restrict__ nrm, uint32_t* __restrict__ errOut) {
    const int nm = *nMixed;
    uint32_t err = 0;
    for (int i = spreadFirst(); i < nm; i += spreadStride()) {
        const int c = mixed[i];
        const d3 g = lsGradientField(m, c, alpha, err);
        const d3 n = (-1.0) * g;
        st3(nrm, i, n / (mag(n) + kSMALL));
    }
    if (err) atomicOr(errOut, err);
}

// ---------------------------------------------------------------------------
// K3: plane constant per mixed cell (cutCell::findSignedDistance), one
// thread per cell.  On this FP64-poor part the kernel is limited by the
// FP64 pipe, so the serial bracketing (the fewest cuts) with lanes kept
// busy inside calcSubCell beats spreading the vertex levels over threads.
// One instantiation per cell class (workspace caps K); a launch handles the
// mixed cells of its class.
// ---------------------------------------------------------------------------
// With SPLIT the workspace is the splitWarpedFace one (warped faces as
// triangle fans, the warped faces' centres among the vertex levels).
template <class K, bool SPLIT>
__global__ void __launch_bounds__(128) kPlaneSolve(DevMesh m, PlaneArgs p, int cls) {
    const int nm = *p.nMixed;
    uint32_t err = 0;
    const int mask = SPLIT ? m.splitClassMask : m.classMask;
    const uint8_t* cellCls = SPLIT ? m.splitClass : m.cellClass;
    for (int i = spreadFirst(); i < nm; i += spreadStride()) {
        const int c = p.mixed[i];
        if (mask != (1 << cls) && cellCls[c] != cls) continue;
        if (p.skip && p.skip[i]) continue;
        CellWS<K> w;
        double d = 0.0;
        d3 ic = mk(0, 0, 0), is = mk(0, 0, 0);
        int st;
        if (!(SPLIT ? loadCellSplit(m, c, w) : loadCell(m, c, w))) {
            err |= kErrSubFaceOverflow;
            st = 1;
        } else {
            st = findSignedDistance(w, p.alpha[c], ld3(p.nrm, i), d, ic, is, err);
        }
        p.mStatus[i] = int8_t(st);
        p.status[c] = int8_t(st);
        p.dOut[i] = d;
        st3(p.icOut, i, ic);
        st3(p.isOut, i, is);
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

// (a) interface speed Un0 = U(interface centre) . n of every cut cell, and
//     the list of its downwind faces (advection.C:131-174: phi >= 0 on an
//     owned face, phi < 0 on a neighboured one; boundary faces phi >= 0)
__global__ void __launch_bounds__(128) kInterfaceUn0(DevMesh m, const int* __restrict__ mixed,
                                                     const int* __restrict__ nMixed,
                                                     const int8_t* __restrict__ mStatus,
                                                     const double* __restrict__ nrm, const double* __restrict__ icArr,
                                                     const double* __restrict__ U, const double* __restrict__ Ub,
                                                     const double* __restrict__ phi, double* __restrict__ un0,
                                                     int2* __restrict__ dwList, int* __restrict__ dwCount) {
    const int nm = *nMixed;
    const int lane = threadIdx.x & 31;
    // uniform trip count per warp so the list append can use warp shuffles
    const int stride = spreadStride();
    const int nIter = (nm + stride - 1) / stride;
    for (int it = 0; it < nIter; ++it) {
        const int i = it * stride + spreadFirst();
        int nd = 0, k0 = 0;
        unsigned down = 0;  // bit j: the cell's j-th face (cells() order) is downwind
        if (i < nm && mStatus[i] == 0) {
            const int c = mixed[i];
            un0[i] = dot(interpolateU(m, c, ld3(icArr, i), U, Ub), ld3(nrm, i));
            k0 = m.cOff[c];
            down = downwindFaces(m, c, k0, m.cOff[c + 1], phi);
            nd = __popc(down);
        }
        // warp-aggregated append
        int incl = nd;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        int base = 0;
        if (lane == 31 && total) base = atomicAdd(dwCount, total);
        base = __shfl_sync(0xffffffffu, base, 31);
        int q = base + incl - nd;
        for (unsigned mm = down; mm; mm &= mm - 1u) dwList[q++] = make_int2(i, m.cFaces[k0 + __ffs(mm) - 1]);
    }
}

// (b) one thread per downwind face of a cut cell: Simpson flux
__global__ void __launch_bounds__(128) kInterfaceFaces(DevMesh m, const int2* __restrict__ dwList,
                                                       const int* __restrict__ dwCount,
                                                       const double* __restrict__ nrm, const double* __restrict__ dArr,
                                                       const double* __restrict__ un0, const double* __restrict__ phi,
                                                       double dt, double* __restrict__ dvfI,
                                                       uint8_t* __restrict__ cutMask) {
    const int n = *dwCount;
    for (int t = spreadFirst(); t < n; t += spreadStride()) {
        const int i = dwList[t].x, f = dwList[t].y;
        dvfI[f] = timeIntegratedFaceFlux(m, f, ld3(nrm, i), dArr[i], un0[i], dt, phi[f], m.magSf[f]);
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
                                               double dt, double rDeltaT, double rrDeltaT,
                                               double* __restrict__ alphaPhi,
                                               int* __restrict__ ovList, int* __restrict__ ovCount, int ovCap) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    bool ov = false, inSet = false;
    if (c < m.nc) {
        // The face-slot records: from the lattice formula for the interior
        // cells of a lattice mesh (no addressing read), else the first
        // kBatch from memory, loaded together so they are in flight at once;
        // slots of larger cells follow one by one from k0 + kBatch.  Unused
        // slots hold x = -2.
        constexpr int kBatch = 6;
        int2 sl[kBatch];
        int k0, k1;
        if (m.latNx && latticeSlotsFast(c, m.latNx, m.latNy, m.latNz, m.latDivLayer, m.latDivNx, sl)) {
            k0 = 0;
            k1 = kBatch;
        } else {
            k0 = m.uniformFaces ? c * m.uniformFaces : m.cOff[c];
            k1 = m.uniformFaces ? k0 + m.uniformFaces : m.cOff[c + 1];
#pragma unroll
            for (int j = 0; j < kBatch; ++j) sl[j] = (k0 + j < k1) ? m.cSlot[k0 + j] : make_int2(-2, 0);
        }
        // Every load the common case needs is issued before any is used, so
        // a cell costs one memory round trip: the alpha across each slot
        // (alpha_b on a boundary face when given), phi of the owned faces,
        // the cell's old and current alpha.
        double ax[kBatch];
        double pv[kBatch];
#pragma unroll
        for (int j = 0; j < kBatch; ++j) {
            ax[j] = 0.0;
            if (sl[j].x >= 0)
                ax[j] = aCur[sl[j].x];
            else if (sl[j].x == -1 && alphaB)
                ax[j] = alphaB[(sl[j].y & 0x7fffffff) - m.nfi];
            pv[j] = (sl[j].x != -2 && sl[j].y >= 0) ? phi[sl[j].y] : 0.0;
        }
        const double ao = aOld[c];
        const double ac = aCur[c];
#pragma unroll
        for (int j = 0; j < kBatch; ++j)
            if (sl[j].x == -1 && !alphaB) ax[j] = ac;  // zero-gradient boundary value
        // Empty neighbourhood: every dVf is a signed zero, surfaceIntegrate
        // gives +0 and ((ao*r) - 0*r)/r returns ao itself (bit for bit), and
        // alphaPhi = dVf/dt is a zero with the sign of phi.  The zero tests
        // and the sign are integer operations on the bit patterns, so empty
        // cells issue no FP64 instruction.
        const auto isZero = [](double x) { return (bitsOf(x) << 1) == 0; };
        const long long kSign = (long long)0x8000000000000000ULL;
        bool quick = (Sp == nullptr) && (Su == nullptr) && isZero(ao) && isZero(ac);
        if (quick) {
#pragma unroll
            for (int j = 0; j < kBatch; ++j) quick = quick && isZero(ax[j]);
            for (int k = k0 + kBatch; quick && k < k1; ++k) {
                const int2 s = m.cSlot[k];
                const double x = (s.x >= 0) ? aCur[s.x] : (alphaB ? alphaB[(s.y & 0x7fffffff) - m.nfi] : ac);
                quick = isZero(x);
            }
        }
        if (quick) {
            aNew[c] = ao;
            // owned faces only (the owner writes each face); an internal face's
            // alpha_f is +0, a boundary face's zero also carries alpha_b's sign
#pragma unroll
            for (int j = 0; j < kBatch; ++j) {
                if (sl[j].x == -2 || sl[j].y < 0) continue;
                long long sgnBits = bitsOf(pv[j]) & kSign;
                if (sl[j].x == -1) sgnBits ^= bitsOf(ax[j]) & kSign;
                alphaPhi[sl[j].y] = __longlong_as_double(sgnBits);
            }
            for (int k = k0 + kBatch; k < k1; ++k) {
                const int2 s = m.cSlot[k];
                if (s.y < 0) continue;
                long long sgnBits = bitsOf(phi[s.y]) & kSign;
                if (s.x < 0) sgnBits ^= bitsOf(alphaB ? alphaB[s.y - m.nfi] : ac) & kSign;
                alphaPhi[s.y] = __longlong_as_double(sgnBits);
            }
        } else {
            // surfaceIntegrate in ascending face order: the batch, then the rest
            double sum = 0.0;
            const auto add = [&](int fa) {
                const int f = fa & 0x7fffffff;
                const double ph = phi[f];
                double x;
                bool prod;
                const double dv = baseDVf(m, f, ph, aCur, status, dvfI, alphaB, dt, x, prod);
                if (fa >= 0) {
                    // dv / dt: from the product dv was made of when there is one
                    alphaPhi[f] = prod ? divOfProduct(dv, dt, rDeltaT, x) : divByRecip(dv, dt, rDeltaT);
                    sum += dv;
                } else {
                    sum -= dv;
                }
            };
#pragma unroll
            for (int j = 0; j < kBatch; ++j)
                if (sl[j].x != -2) add(sl[j].y);
            for (int k = k0 + kBatch; k < k1; ++k) add(m.cSlot[k].y);
            // the divisions through correctly rounded reciprocals (1/V per
            // cell, 1/dt and 1/(1/dt) per step): the same quotients
            const double ivf = divByRecip(sum, m.V[c], m.rV[c]);
            double num = ao * rDeltaT;
            if (Su) num = num + Su[c];
            num = num - ivf * rDeltaT;
            const double an = Sp ? num / (rDeltaT - Sp[c]) : divByRecip(num, rDeltaT, rrDeltaT);
            aNew[c] = an;
            // cells outside [-aTol, 1 + aTol] are the bounding candidates; the
            // count of them decides limitFlux's loop (advectionTemplates.C:146)
            // (on the bits: an < -aTol or an > 1 + aTol, NaN neither)
            const double aTol = 100.0 * kSMALL;
            const long long ba = bitsOf(an);
            const long long mag = ba & 0x7fffffffffffffffLL;
            ov = mag <= 0x7ff0000000000000LL && (ba < 0 ? mag > bitsOf(aTol) : ba > bitsOf(1.0 + aTol));
            // only cells of the bounding set (mixed cells and their face
            // neighbours, advection.C:54-82) are listed; every overshooting
            // cell is counted
            if (ov) {
                inSet = status[c] != kStNotMixed;
#pragma unroll
                for (int j = 0; j < kBatch; ++j) inSet = inSet || (sl[j].x >= 0 && status[sl[j].x] != kStNotMixed);
                for (int k = k0 + kBatch; k < k1 && !inSet; ++k) {
                    const int nb = m.cSlot[k].x;
                    inSet = nb >= 0 && status[nb] != kStNotMixed;
                }
            }
        }
    }
    const unsigned ball = __ballot_sync(0xffffffffu, ov);
    if (ball) {
        const int lane = threadIdx.x & 31;
        if (lane == 0) atomicAdd(ovCount, __popc(ball));  // [0] all overshooting cells
        const unsigned sball = __ballot_sync(0xffffffffu, inSet);
        int base = 0;
        if (lane == 0 && sball) base = atomicAdd(ovCount + 1, __popc(sball));  // [1] listed cells
        base = __shfl_sync(0xffffffffu, base, 0);
        const int p = base + __popc(sball & ((1u << lane) - 1u));
        if (inSet && p < ovCap) ovList[p] = c;
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
// A grid of exactly the blocks that are resident at once on all SMs (the
// occupancy of `kernel` at `threads` per block), looked up once per kernel
// and device.
template <class Kernel>
static int residentGrid(Kernel kernel, int threads) {
    struct Entry {
        const void* fn;
        int dev, threads, grid;
    };
    constexpr int kSlots = 32;
    static Entry cache[kSlots] = {};
    static std::mutex mu;
    int dev = 0;
    cudaGetDevice(&dev);
    const void* fn = reinterpret_cast<const void*>(kernel);
    std::lock_guard<std::mutex> lock(mu);
    for (int i = 0; i < kSlots && cache[i].fn; ++i)
        if (cache[i].fn == fn && cache[i].dev == dev && cache[i].threads == threads) return cache[i].grid;
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
    const int g = (sms > 0 ? sms : 1) * (per > 0 ? per : 1);
    for (int i = 0; i < kSlots; ++i)
        if (!cache[i].fn) {
            cache[i] = {fn, dev, threads, g};
            break;
        }
    return g;
}

void launchScanMixed(const StepArgs& a, cudaStream_t st) {
    const int nb = ((a.m.nc + 3) / 4 + 255) / 256;
    const double omt = 1.0 - a.mixedTol;
    long long tolBits, omtBits;
    std::memcpy(&tolBits, &a.mixedTol, sizeof(double));
    std::memcpy(&omtBits, &omt, sizeof(double));
    kScanMixed<<<nb, 256, 0, st>>>(a.m.nc, a.aCur, tolBits, omtBits, a.status, a.mixed, a.nMixed, a.err);
}

void launchLsNormal(const StepArgs& a, cudaStream_t st) {
    kLsNormal<<<residentGrid(kLsNormal, 128), 128, 0, st>>>(a.m, a.aCur, a.mixed, a.nMixed, a.nrm, a.err);
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
    p.err = a.err;
    p.skip = nullptr;
    return p;
}

void launchPlaneSolve(const StepArgs& a, cudaStream_t st) { launchPlaneSolveSkip(a, nullptr, st); }

void launchPlaneSolveSkip(const StepArgs& a, const uint8_t* skip, cudaStream_t st) {
    PlaneArgs p = planeArgs(a);
    p.skip = skip;
    if (a.m.splitClassMask) {
        const int mk = a.m.splitClassMask;
        if (mk & 1) kPlaneSolve<CapsHex, true><<<residentGrid(kPlaneSolve<CapsHex, true>, 128), 128, 0, st>>>(a.m, p, 0);
        if (mk & 2) kPlaneSolve<CapsPoly, true><<<residentGrid(kPlaneSolve<CapsPoly, true>, 128), 128, 0, st>>>(a.m, p, 1);
        if (mk & 4) kPlaneSolve<CapsBig, true><<<residentGrid(kPlaneSolve<CapsBig, true>, 128), 128, 0, st>>>(a.m, p, 2);
        return;
    }
    const int mk = a.m.classMask;
    if (mk & 1) kPlaneSolve<CapsHex, false><<<residentGrid(kPlaneSolve<CapsHex, false>, 128), 128, 0, st>>>(a.m, p, 0);
    if (mk & 2) kPlaneSolve<CapsPoly, false><<<residentGrid(kPlaneSolve<CapsPoly, false>, 128), 128, 0, st>>>(a.m, p, 1);
    if (mk & 4) kPlaneSolve<CapsBig, false><<<residentGrid(kPlaneSolve<CapsBig, false>, 128), 128, 0, st>>>(a.m, p, 2);
}

void launchInterfaceUn0(const StepArgs& a, cudaStream_t st) {
    kInterfaceUn0<<<residentGrid(kInterfaceUn0, 128), 128, 0, st>>>(a.m, a.mixed, a.nMixed, a.mStatus, a.nrm, a.icArr, a.U, a.Ub,
                                                      a.phi, a.un0, a.dwList, a.dwCount);
}

void launchInterfaceFaces(const StepArgs& a, cudaStream_t st) {
    kInterfaceFaces<<<residentGrid(kInterfaceFaces, 128), 128, 0, st>>>(a.m, a.dwList, a.dwCount, a.nrm, a.dArr, a.un0, a.phi,
                                                            a.dt, a.dvfI, a.cutMask);
}

void launchUpdate(const StepArgs& a, cudaStream_t st) {
    const int nb = (a.m.nc + 255) / 256;
    kUpdate<<<nb, 256, 0, st>>>(a.m, a.phi, a.aCur, a.aOld, a.aNew, a.status, a.dvfI, a.alphaB, a.Sp, a.Su, a.dt,
                                a.rDeltaT, a.rrDeltaT, a.alphaPhi, a.ovList, a.ovCount, a.ovCap);
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

// 1/V of every cell (correctly rounded; the divisor reciprocals of divByRecip)
__global__ void kRecipVolume(int nc, const double* __restrict__ V, double* __restrict__ rV) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nc) rV[c] = 1.0 / V[c];
}

void launchRecipVolume(const DevMesh& m, double* rV, cudaStream_t st) {
    kRecipVolume<<<(m.nc + 255) / 256, 256, 0, st>>>(m.nc, m.V, rV);
}

void launchFaceFull(const DevMesh& m, double* fullC, double* fullA, cudaStream_t st) {
    kFaceFull<<<(m.nf + 255) / 256, 256, 0, st>>>(m, fullC, fullA);
}

// LS stencils of all cells, once per mesh: row lengths (count = true), then
// the rows (count = false).  An overflowing row gets kMaxStencil entries and
// a -1 (the readers report the overflow when they use the row).
__global__ void __launch_bounds__(128) kStencilRows(DevMesh m, bool count, int* __restrict__ len,
                                                    const int* __restrict__ off, int* __restrict__ rows) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.nc; c += gridDim.x * blockDim.x) {
        int st[kMaxStencil];
        uint32_t err = 0;
        const int n = buildStencil(m, c, st, err);
        if (count) {
            len[c] = err ? n + 1 : n;
        } else {
            int* row = rows + off[c];
            for (int k = 0; k < n; ++k) row[k] = st[k];
            if (err) row[n] = -1;
        }
    }
}

void launchStencilRows(const DevMesh& m, bool count, int* len, const int* off, int* rows, cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    kStencilRows<<<sms * 16, 128, 0, st>>>(m, count, len, off, rows);
}

}  // namespace simplic
