// Conservative bounding of the plain FP64 form: advection::limitFlux and
// advection::boundFlux (src/SimPLIC/advection/advectionTemplates.C:118-349)
// with extendMarkedCells / netFlux / setDownwindFaces (advection.C:54-82,
// 224-288).  Built with -fmad=false.
//
// The reference walks the bounding set (mixed cells and their face
// neighbours) in ascending cell order, and a cell reads the flux corrections
// that earlier cells wrote during the same pass.  A cell only reads
// corrections on its own faces and only its face-adjacent cells write those,
// so the result is the same whenever every overshooting cell runs after its
// earlier face-adjacent overshooting neighbours and before its later ones.
// The kernel runs on every SM (cooperative launch, all blocks resident):
//   * candidates: the overshooting cells the update kernel listed, filtered to
//     the bounding set; their dependencies are found through per-cell stamps,
//     no sorting;
//   * waves: a cell runs once all its earlier neighbours have published
//     "done" (release / acquire), so chains also advance inside a wave;
//   * corrections are applied per target cell in the reference's list order
//     (key = cell * 16 + position among the cell's first-iteration faces);
//   * the pass test max(alpha) - 1 > aTol || min(alpha) < -aTol is exactly
//     "some cell of the mesh overshoots": an exact counter of overshooting
//     cells replaces the global min / max.
// Blocks meet at a grid barrier whose wait is bounded (a timeout sets an
// error bit); every loop is bounded and no block returns after the first
// barrier, so all blocks take the same decisions from values that are final
// when read.
#include <cfloat>
#include <climits>

#include "plain_geom.cuh"
#include "simplic_kernels.h"

namespace simplic {

namespace {

constexpr double kATol = 100.0 * kSMALL;  // advectionTemplates.C:125,228
constexpr long long kMaxSpins = 20000000;  // ~1-2 s with 64 ns sleeps
constexpr int kDepSpins = 400;             // ~0.1-0.3 ms wait for earlier neighbours

__device__ __forceinline__ bool overshoots(double a) { return a < -kATol || a > 1.0 + kATol; }

// List append with one atomic per group of converged lanes: thousands of
// cells appending to one counter otherwise queue up on a single address.
__device__ __forceinline__ int aggAppend(int* ctr) {
    const unsigned m = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(ctr, __popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}
__device__ __forceinline__ void aggAdd(int* ctr, int v) {
    const unsigned m = __activemask();
    const int total = __reduce_add_sync(m, v);
    if ((threadIdx.x & 31) == __ffs(m) - 1 && total) atomicAdd(ctr, total);
}

// A bounding list ran out of room: the error bit for the host, and which list
// in info[3] (the largest code seen).
enum : int { kOvfOvershootList = 1, kOvfWaves = 2, kOvfModList = 3, kOvfTouchedList = 4, kOvfCandidates = 5 };
__device__ __forceinline__ void boundOverflow(const StepArgs& a, const BoundBuffers& s, int code) {
    atomicOr(a.err, (uint32_t)kErrBoundOverflow);
    atomicMax(s.info + 3, code);
}

// "done" flag of an overshooting cell, stored with release semantics after
// the cell's corrections; readers poll it and then fence (acquire).
__device__ __forceinline__ void stRelease(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ double curDVf(const DevMesh& m, int f, const double* phi, const double* aCur,
                                         const int8_t* status, const double* dvfI, const double* alphaB, double dt,
                                         const BoundBuffers& s, int stamp) {
    if (s.modStamp[f] == stamp) return s.dvfMod[f];
    return baseDVf(m, f, phi[f], aCur, status, dvfI, alphaB, dt);
}

__device__ __forceinline__ bool inNeedBounding(const DevMesh& m, int c, const int8_t* status) {
    if (status[c] != kStNotMixed) return true;
    for (int k = m.cOff[c]; k < m.cOff[c + 1]; ++k) {
        const int nb = m.cSlot[k].x;
        if (nb >= 0 && status[nb] != kStNotMixed) return true;
    }
    return false;
}

// Grid-wide barrier for a cooperative launch.  Thread 0 of each block
// arrives on a counter; the last one resets it and advances the generation.
__device__ void gridBarrier(const BoundBuffers& s, uint32_t* err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = s.barGen;
        const unsigned g = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(s.barCount, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(s.barCount, 0u);
            __threadfence();
            atomicAdd((unsigned*)s.barGen, 1u);
        } else {
            long long spins = 0;
            // once any barrier has timed out the results are void: later
            // barriers stop waiting so the kernel ends promptly
            const long long limit = (*(volatile uint32_t*)err & kErrBarrierTimeout) ? 0 : kMaxSpins;
            while (*gen == g) {
                if (++spins > limit) {
                    atomicOr(err, (uint32_t)kErrBarrierTimeout);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// The body of the reference's cell loop (advectionTemplates.C:245-347) for
// one overshooting cell, run by a whole warp, lane k on face k of the cell.
// The corrections on this cell's faces are final (its earlier neighbours are
// done, its later ones have not started).  The per-face terms (with their
// divisions) run in parallel; every sum is still taken in face order through
// shuffles, so the result is bit for bit the serial loop's.  Fs / ph / dv are
// this lane's face record (face id with bit 31 on the neighbour side, phi,
// dVf; loaded before the wait), al and Vi the cell's alpha and volume.
// Writes the cell's corrections and records its first-iteration faces.
__device__ void boundCellWarp(int c, int ci, int nfc, int Fs, double ph, double dv, double al, double Vi,
                              const StepArgs& a, const BoundBuffers& s, int lane) {
    constexpr unsigned kAll = 0xffffffffu;
    const bool on = lane < nfc;
    const int F = Fs & 0x7fffffff;
    const int own = (on && Fs >= 0) ? 1 : 0;
    const double cr0 = on ? ((volatile double*)s.corr)[F] : 0.0;
    double cr = cr0;
    const bool down = on && (own ? (ph >= 0) : (ph < 0));
    bool wrote = false;
    double nf1 = 0.0;  // netFlux(c, dVf): the same every iteration
    for (int k = 0; k < nfc; ++k) {
        const double x = __shfl_sync(kAll, dv, k);
        if (__shfl_sync(kAll, own, k))
            nf1 += x;
        else
            nf1 -= x;
    }
    const double dt = a.dt, rDeltaT = a.rDeltaT;
    double alphaOvershoot = pos0(al - 1.0) * (al - 1.0) + neg0(al) * al;
    double fluid = alphaOvershoot * Vi;
    int nPass = 1, nCorr = 0;
    bool firstLoop = true;
    const size_t sb = size_t(ci) * kMaxCellFaces;
    const unsigned below = (1u << lane) - 1u;
    for (int iter = 0; iter < 10; ++iter) {
        if (fabs(alphaOvershoot) < kATol || nPass == 0) break;
        bool pass = false;
        double pmax = 0.0;
        if (down) {
            const double dVff = dv + cr;
            const double maxExtra = fabs(pos0(fluid) * ph * dt - dVff);
            if (maxExtra / Vi > kATol) {
                pass = true;
                pmax = maxExtra;
            }
        }
        const unsigned pm = __ballot_sync(kAll, pass);
        const double myFlux = fabs(ph * dt);
        double dVftot = 0.0;
        for (unsigned mm = pm; mm; mm &= mm - 1u) dVftot += __shfl_sync(kAll, myFlux, __ffs(mm) - 1);
        int passInc = 0;
        if (pass) {
            double through = fabs(fluid) * fabs(ph * dt) / dVftot;
            passInc = int(pos0(pmax - through));
            through = fmin(through, pmax);
            double dVff = cr;
            dVff += sgn(ph) * sgn(fluid) * through;
            cr = dVff;
            wrote = true;
            if (firstLoop) s.candCorr[sb + nCorr + __popc(pm & below)] = F;
        }
        nPass = __reduce_add_sync(kAll, passInc);
        if (firstLoop) nCorr += __popc(pm);
        firstLoop = false;
        double nf2 = 0.0;
        for (int k = 0; k < nfc; ++k) {
            const double x = __shfl_sync(kAll, cr, k);
            if (__shfl_sync(kAll, own, k))
                nf2 += x;
            else
                nf2 -= x;
        }
        double num = a.aOld[c] * rDeltaT;
        if (a.Su) num = num + a.Su[c];
        num = num - nf1 / Vi * rDeltaT;
        num = num - nf2 / Vi * rDeltaT;
        const double den = a.Sp ? (rDeltaT - a.Sp[c]) : rDeltaT;
        const double a1New = num / den;
        alphaOvershoot = pos0(a1New - 1.0) * (a1New - 1.0) + neg0(a1New) * a1New;
        fluid = alphaOvershoot * Vi;
    }
    const unsigned wm = __ballot_sync(kAll, wrote);
    if (wrote) {
        s.corr[F] = cr;
        s.candWritten[sb + __popc(wm & below)] = F;
    }
    if (lane == 0) {
        s.candNCorr[ci] = nCorr;
        s.candNWritten[ci] = __popc(wm);
    }
}

__global__ void __launch_bounds__(256) kBound(StepArgs a, BoundBuffers s) {
    const DevMesh& m = a.m;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nth = gridDim.x * blockDim.x;
    const int stamp = s.stamp;  // step stamp
    // Decisions before the first barrier read values no block modifies.
    const int ovCount = s.ovCount[0];  // overshooting cells of the whole mesh
    const int nList = s.ovCount[1];    // those of them in the bounding set
    // No overshooting cell, or none in the bounding set: no pass can change
    // anything (corrections only come from listed cells), so nothing to do.
    if (ovCount == 0 || nList == 0) return;
    if (nList > s.ovCap || 2 * nList > s.candCap) {
        if (tid == 0) boundOverflow(a, s, kOvfOvershootList);
        return;
    }
    // 1. candidates: the overshooting cells of the bounding set, as listed
    //    by the update
    for (int i = tid; i < nList; i += nth) {
        const int c = s.ovList[i];
        s.cand[i] = c;
        s.candIdx[c] = i;
        s.candMark[c] = stamp;
    }
    if (tid == 0) s.ctl[kCtlCand] = nList;
    gridBarrier(s, a.err);

    int over = ovCount;  // overshooting cells in the whole mesh
    for (int pass = 0; pass < a.nAlphaBounds && pass < kMaxBoundPasses; ++pass) {
        if (over == 0) break;
        const int passStamp = stamp * kMaxBoundPasses + pass + 1;
        const int nCand = ((volatile int*)s.ctl)[kCtlCand];
        if (tid == 0) s.info[0] = pass + 1;
        // 2. active cells (overshooting now) and their earlier active neighbours
        for (int i = tid; i < nCand; i += nth) {
            const int c = s.cand[i];
            const bool act = overshoots(a.aNew[c]);
            s.candActive[i] = act ? 1 : 0;
            s.candDone[i] = 0;
            s.candNCorr[i] = 0;
            s.candNWritten[i] = 0;
            int nd = 0;
            if (act) {
                s.actList[aggAppend(s.ctl + kCtlActive0 + pass)] = i;
                const int k0 = m.cOff[c], k1 = m.cOff[c + 1];
                for (int k = k0; k < k1; ++k) {
                    const int nb = m.cSlot[k].x;
                    if (nb < 0 || nb > c || s.candMark[nb] != stamp) continue;
                    if (overshoots(a.aNew[nb])) s.candDeps[size_t(i) * kMaxCellFaces + nd++] = s.candIdx[nb];
                }
                // the cell's faces in cells() order with phi and the dVf the
                // pass starts from (final here: earlier passes are complete)
                const size_t sb = size_t(i) * kMaxCellFaces;
                s.candNF[i] = k1 - k0;
                for (int k = 0; k < k1 - k0; ++k) {
                    const int f = m.cFaces[k0 + k];
                    s.candSlotF[sb + k] = (m.own[f] == c) ? f : int(unsigned(f) | 0x80000000u);
                    s.candSlotPh[sb + k] = a.phi[f];
                    s.candSlotDv[sb + k] = curDVf(m, f, a.phi, a.aCur, a.status, a.dvfI, a.alphaB, a.dt, s, stamp);
                }
            }
            s.candNDeps[i] = nd;
        }
        gridBarrier(s, a.err);
        // 3. waves: a cell runs once its earlier neighbours are done
        const int nAct = ((volatile int*)s.ctl)[kCtlActive0 + pass];
        // no listed cell overshoots: this and every later pass change nothing
        if (nAct == 0) break;
        // One warp per overshooting cell, run by its lane 0, so no warp
        // holds both a waiting and a working cell.  The cell's fixed data is
        // loaded first; then, with at most one cell per warp, the cell waits
        // (bounded) for its earlier neighbours instead of leaving them to the
        // next wave, so dependency chains run through inside one wave.  The
        // waits always end: dependencies point to smaller cell ids (no
        // cycle) and every block is resident; a cell whose neighbours are not
        // done within the limit runs in a later wave.  The flags are polled
        // with plain (volatile) loads and one acquire fence follows.
        const int lane = threadIdx.x & 31;
        const int gw = tid >> 5, nw = nth >> 5;
        const int depSpins = (nAct <= nw) ? kDepSpins : 0;
        int doneSoFar = 0;
        int w = 0;
        for (; w < kMaxBoundWaves && doneSoFar < nAct; ++w) {
            for (int q = gw; q < nAct; q += nw) {
                // warp per cell: lane k holds face k; lanes below the cell's
                // dependency count poll one neighbour each
                const int i = s.actList[q];
                if (((volatile int*)s.candDone)[i]) continue;  // same value on every lane
                const int c = s.cand[i];
                const size_t sb = size_t(i) * kMaxCellFaces;
                const int nfc = s.candNF[i];
                const int nd = s.candNDeps[i];
                int Fs = 0;
                double ph = 0.0, dv = 0.0;
                if (lane < nfc) {
                    Fs = s.candSlotF[sb + lane];
                    ph = s.candSlotPh[sb + lane];
                    dv = s.candSlotDv[sb + lane];
                }
                const int dep = lane < nd ? s.candDeps[sb + lane] : -1;
                const double al = a.aNew[c];  // updated only after the waves
                const double Vi = m.V[c];
                bool ready = false;
                for (int spin = 0;; ++spin) {
                    const bool mine = dep < 0 || ((volatile int*)s.candDone)[dep] != 0;
                    ready = __all_sync(0xffffffffu, mine);
                    if (ready || spin >= depSpins) break;
                    __nanosleep(128);
                }
                if (ready) {
                    asm volatile("fence.acq_rel.gpu;" ::: "memory");  // acquire the neighbours' corrections
                    boundCellWarp(c, i, nfc, Fs, ph, dv, al, Vi, a, s, lane);
                    __threadfence();  // every lane's corrections before the flag
                    __syncwarp();
                    if (lane == 0) {
                        stRelease(s.candDone + i, 1);  // release this cell's corrections
                        atomicAdd(s.ctl + kCtlWave0 + pass * kMaxBoundWaves + w, 1);
                    }
                }
                __syncwarp();
            }
            gridBarrier(s, a.err);
            doneSoFar += ((volatile int*)s.ctl)[kCtlWave0 + pass * kMaxBoundWaves + w];
            if (w == kMaxBoundWaves - 1 && doneSoFar < nAct && tid == 0) boundOverflow(a, s, kOvfWaves);
        }
        if (tid == 0 && w > s.info[2]) s.info[2] = w;
        // 4a. list keys of the corrected faces; new dVf of those faces
        for (int i = tid; i < nCand; i += nth) {
            if (!s.candActive[i]) continue;
            const int c = s.cand[i];
            const int* cf = s.candCorr + size_t(i) * kMaxCellFaces;
            for (int q = 0; q < s.candNCorr[i]; ++q) {
                const int f = cf[q];
                s.faceKey[f] = c * 16 + q;
                s.faceStamp[f] = passStamp;
                const double nv = curDVf(m, f, a.phi, a.aCur, a.status, a.dvfI, a.alphaB, a.dt, s, stamp) + s.corr[f];
                if (s.modStamp[f] != stamp) {
                    const int p = aggAppend(s.ctl + kCtlMod);
                    if (p < s.modCap) s.modList[p] = f;
                    else boundOverflow(a, s, kOvfModList);
                }
                s.dvfMod[f] = nv;
                s.modStamp[f] = stamp;
            }
        }
        gridBarrier(s, a.err);
        // 4b. alpha of every target cell, its updates in list order
        //     (advectionTemplates.C:164-192: own -= corr/V, nei += corr/V)
        for (int i = tid; i < nCand; i += nth) {
            if (!s.candActive[i]) continue;
            const int* cf = s.candCorr + size_t(i) * kMaxCellFaces;
            for (int q = 0; q < s.candNCorr[i]; ++q) {
                const int f = cf[q];
                for (int side = 0; side < (f < m.nfi ? 2 : 1); ++side) {
                    const int t = side == 0 ? m.own[f] : m.nei[f];
                    if (atomicExch(s.cellClaim + t, passStamp) == passStamp) continue;
                    int key[kMaxCellFaces];
                    int fk[kMaxCellFaces];
                    int ne = 0;
                    for (int k = m.cOff[t]; k < m.cOff[t + 1]; ++k) {
                        const int g = m.cFaces[k];
                        if (s.faceStamp[g] != passStamp) continue;
                        const int kk = s.faceKey[g];
                        int j = ne++;
                        while (j > 0 && key[j - 1] > kk) {
                            key[j] = key[j - 1];
                            fk[j] = fk[j - 1];
                            --j;
                        }
                        key[j] = kk;
                        fk[j] = g;
                    }
                    double at = a.aNew[t];
                    const bool before = overshoots(at);
                    const double Vt = m.V[t];
                    for (int e = 0; e < ne; ++e) {
                        const double cv = s.corr[fk[e]];
                        if (m.own[fk[e]] == t) at -= cv / Vt;
                        else at += cv / Vt;
                    }
                    a.aNew[t] = at;
                    const int dOver = int(overshoots(at)) - int(before);
                    aggAdd(s.ctl + kCtlOverDelta0 + pass, dOver);
                    const int p = aggAppend(s.ctl + kCtlTouched);
                    if (p < s.touchedCap) s.touched[p] = t;
                    else boundOverflow(a, s, kOvfTouchedList);
                }
            }
        }
        gridBarrier(s, a.err);
        // 5. clear this pass's corrections; touched cells of the bounding
        //    set join the candidates
        for (int i = tid; i < nCand; i += nth) {
            const int* w = s.candWritten + size_t(i) * kMaxCellFaces;
            for (int q = 0; q < s.candNWritten[i]; ++q) s.corr[w[q]] = 0.0;
        }
        const int nT = min(((volatile int*)s.ctl)[kCtlTouched], s.touchedCap);
        for (int r = tid; r < nT; r += nth) {
            const int t = s.touched[r];
            if (s.candMark[t] == stamp || !inNeedBounding(m, t, a.status)) continue;
            if (atomicExch(s.candMark + t, stamp) == stamp) continue;
            const int p = aggAppend(s.ctl + kCtlCand);
            if (2 * (p + 1) <= s.candCap) {
                s.cand[p] = t;
                s.candIdx[t] = p;
            } else {
                boundOverflow(a, s, kOvfCandidates);
            }
        }
        gridBarrier(s, a.err);
        over += ((volatile int*)s.ctl)[kCtlOverDelta0 + pass];
        if (tid == 0) {
            const int n = ((volatile int*)s.ctl)[kCtlActive0 + pass];
            if (n > s.info[1]) s.info[1] = n;
        }
        // the touched list restarts each pass; reset it behind one more
        // barrier so no block still reads it
        if (tid == 0) ((volatile int*)s.ctl)[kCtlTouched] = 0;
        gridBarrier(s, a.err);
    }
    // alphaPhi = dVf / dt of every face the bounding changed this step
    const int nMod = min(((volatile int*)s.ctl)[kCtlMod], s.modCap);
    for (int i = tid; i < nMod; i += nth) {
        const int f = s.modList[i];
        a.alphaPhi[f] = s.dvfMod[f] / a.dt;
    }
}

}  // namespace

cudaError_t launchBound(const StepArgs& a, const BoundBuffers& b, cudaStream_t st) {
    // all blocks must be resident at once for the grid barrier: one or two
    // blocks per SM, as the occupancy calculator allows
    int dev = 0, sms = 0, perSm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kBound, 256, 0);
    if (e != cudaSuccess) return e;
    if (perSm < 1) return cudaErrorCooperativeLaunchTooLarge;
    const int grid = sms * (perSm >= 2 ? 2 : 1);
    StepArgs aa = a;
    BoundBuffers bb = b;
    void* args[] = {&aa, &bb};
    return cudaLaunchCooperativeKernel((const void*)kBound, dim3(grid), dim3(256), args, 0, st);
}

}  // namespace simplic
