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
//   * dataflow: everything of a cell's loop that reads no correction is
//     computed for all overshooting cells at once; a cell then runs as soon
//     as the earlier neighbours it waits for have stored the corrections on
//     the faces it shares with them -- the one that completes it runs it
//     next in the same warp (chains run through in one warp) and a ready
//     queue feeds the idle warps -- and the corrected-face lists are built
//     afterwards, off the dependency chains;
//   * corrections are applied per target cell in the reference's list order
//     (key = cell * 32 + position among the cell's first-iteration faces);
//   * the pass test max(alpha) - 1 > aTol || min(alpha) < -aTol is exactly
//     "some cell of the mesh overshoots": an exact counter of overshooting
//     cells replaces the global min / max.
// Blocks meet at a grid barrier whose wait is bounded (a timeout sets an
// error bit and ends the blocks that see it); every loop and every wait of
// the dependency phase is bounded too, and no block returns after the first
// barrier unless a bounded wait ran out, so all blocks take the same
// decisions from values that are final when read.
#include <cfloat>
#include <climits>

#include "plain_geom.cuh"
#include "simplic_kernels.h"

namespace simplic {

namespace {

constexpr double kATol = 100.0 * kSMALL;  // advectionTemplates.C:125,228

__device__ __forceinline__ bool overshoots(double a) { return a < -kATol || a > 1.0 + kATol; }
__device__ __forceinline__ unsigned long long globalNs() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

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
// (code 2 is not produced: the dependency phase has no depth cap)
enum : int { kOvfOvershootList = 1, kOvfModList = 3, kOvfTouchedList = 4, kOvfCandidates = 5 };
__device__ __forceinline__ void boundOverflow(const StepArgs& a, const BoundBuffers& s, int code) {
    atomicOr(a.err, (uint32_t)kErrBoundOverflow);
    atomicMax(s.info + 3, code);
}

// A face whose correction a later cell of the pass waits for holds this
// NaN pattern (never produced by arithmetic here, which gives the canonical
// NaN) until the earlier cell stores the value.  The value is the flag: a
// 64-bit store is single-copy atomic, so no fence is needed on either side.
constexpr long long kCorrPending = (long long)0xfff4c0de0000f00dULL;
__device__ __forceinline__ long long ldRelaxed64(const double* p) {
    long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void stRelaxed64(double* p, double v) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}

__device__ __forceinline__ double curDVf(const DevMesh& m, int f, const double* phi, const double* aCur,
                                         const int8_t* status, const double* dvfI, const double* alphaB, double dt,
                                         const BoundBuffers& s, int stamp) {
    if (s.modStamp[f] == stamp) return s.dvfMod[f];
    return baseDVf(m, f, phi[f], aCur, status, dvfI, alphaB, dt);
}

// Grid-wide barrier for a cooperative launch.  Thread 0 of each block
// arrives on a counter that only grows (zeroed before every launch): the
// k-th barrier (k counted by every thread of the block, from 0) is complete
// when the counter reaches (k + 1) x blocks, and the block that brings it
// there advances the generation the others wait on.  The wait is bounded
// (s.spinLimit polls): a block that gives up sets the timeout bit and the
// barrier returns false to all its threads, and the kernel then ends that
// block at once -- nothing after a failed barrier may read what other blocks
// were to write before it.  The other blocks then give up at their next
// barrier, so the launch always ends.  s.barrierExtra (a test setting,
// normally 0) makes the barrier wait for arrivals that never come.
__device__ bool gridBarrier(const BoundBuffers& s, uint32_t* err, unsigned& k) {
    __shared__ int ok;
    __syncthreads();
    const unsigned target = (k + 1u) * (gridDim.x + unsigned(s.barrierExtra));
    ++k;
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned* gen = s.barGen;
        const unsigned g = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(s.barCount, 1u) + 1u;
        if (arrived == target) {
            atomicAdd((unsigned*)s.barGen, 1u);
        } else {
            long long spins = 0;
            while (*gen == g) {
                if (++spins > s.spinLimit) {
                    atomicOr(err, (uint32_t)kErrBarrierTimeout);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Exact tests on IEEE bit patterns, on the integer pipe (a double compare
// costs as much as a double add on this part).  NaN is neither >= 0 nor < 0.
__device__ __forceinline__ bool geZero(double x) {  // x >= 0 (true for -0)
    const long long b = bitsOf(x);
    return b >= 0 ? b <= 0x7ff0000000000000LL : (b << 1) == 0;
}
__device__ __forceinline__ bool ltZero(double x) {  // x < 0
    const long long b = bitsOf(x);
    return b < 0 && (b << 1) != 0 && (b & 0x7fffffffffffffffLL) <= 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool isZero(double x) { return (bitsOf(x) << 1) == 0; }
__device__ __forceinline__ bool absLess(double x, double t) {  // |x| < t, t > 0 finite
    return (bitsOf(x) & 0x7fffffffffffffffLL) < bitsOf(t);
}
// fmin of two non-negative, non-NaN values
__device__ __forceinline__ double minNonNeg(double x, double y) { return bitsOf(x) <= bitsOf(y) ? x : y; }
__device__ __forceinline__ int expField(double x) { return int((bitsOf(x) >> 52) & 0x7ff); }

constexpr double kHalfATol = 0.5 * kATol;
constexpr double kUnitHi = 1.0 + kHalfATol;

// The body of the reference's cell loop (advectionTemplates.C:245-347) for
// one overshooting cell, run by a whole warp, lane k on the cell's k-th face
// (cells() order).  The corrections on this cell's faces are final (its
// earlier neighbours are done, its later ones have not started).  Every
// value is computed by the reference's operations in the reference's order,
// sums in face order through shuffles, so the corrections are bit for bit
// the serial loop's.  The latency of a dependency chain is the sum of its
// cells' loops, and a double operation takes tens of cycles here, so:
//   * everything that does not read a correction is computed for every
//     overshooting cell before the dependency phase (BoundLane /
//     BoundCellConst, kept per face slot and per cell), including the first
//     iteration's passing faces and flux shares as they are when no
//     correction has arrived -- reused when the corrections leave them
//     unchanged;
//   * the test "maxExtra / V > aTol" is decided on the bits of maxExtra
//     against aTol V (1 +- 2^-40), with the division only inside that band;
//   * the loop test on the next alpha1New is first decided on a product
//     estimate with a proved error bound (< 2^-46 + 2^-48 when it is
//     used), with the two divisions only when the estimate cannot decide;
//   * zero terms are left out of the face sums (a sum started at +0 never
//     becomes -0, so adding a zero never changes it).
struct BoundLane {
    int F;                   // face id
    bool on, own, down;      // a face of the cell; owner side; flux leaves the cell
    bool phPos;              // phi >= 0
    double dv, phdt, aPhdt;  // dVf at the start of the pass, phi dt, |phi dt|
    bool pass0;              // passing in the first iteration when no correction arrives
    double maxExtra0, through0;
};
struct BoundCellConst {
    double Vi, rVi;        // cell volume, 1 / V
    double ov0, fluid0;    // alphaOvershoot and fluid of the first iteration
    double num1;           // alpha.oldTime * rDeltaT (+ Su) - netFlux(dVf) / V * rDeltaT
    double den, rden;      // rDeltaT (- Sp), 1 / den
    double g;              // (1 / V) rDeltaT
    double tolLo, tolHi;   // aTol V (1 -+ 2^-40)
    int eNum1, eRden;      // exponent fields of num1, rden
    unsigned pm0, ownMask; // first-iteration passing faces without corrections; owner-side faces
    int nfc, pad;          // faces of the cell
};
static_assert(sizeof(BoundCellConst) == kBoundCellConstBytes, "per-candidate constant record size");

// face-slot flags of an overshooting candidate
enum : uint8_t { kSlotOn = 1, kSlotOwn = 2, kSlotDown = 4, kSlotPhPos = 8, kSlotPass0 = 16, kSlotDep = 32 };

// maxExtra / V > aTol, maxExtra >= 0
__device__ __forceinline__ bool exceedsATol(double maxExtra, const BoundCellConst& kc) {
    const long long b = bitsOf(maxExtra);
    if (b > bitsOf(kc.tolHi) && b <= 0x7ff0000000000000LL) return true;
    if (b < bitsOf(kc.tolLo)) return false;
    return divByRecip(maxExtra, kc.Vi, kc.rVi) > kATol;
}

// The parts of the cell loop that read no correction, computed for every
// overshooting candidate before the dependency phase.  The cell's faces are
// on a group of lanes: lanes base .. base + 15 (two cells per warp) or the
// whole warp (base 0) when a cell of the mesh has more than 16 faces; gl is
// the lane's face, gbits the group's lane bits, nmax the most faces of a
// cell in the warp (every lane takes part in every shuffle).  The masks
// kept in kc are by face (bit k: face k).
__device__ __forceinline__ void boundCellPrep(int c, int nfc, int nmax, int base, unsigned gbits, int Fs, double ph,
                                              double dv, const DevMesh& m, const StepArgs& a, int gl, BoundLane& L,
                                              BoundCellConst& kc) {
    constexpr unsigned kAll = 0xffffffffu;
    L.on = gl < nfc;
    L.F = Fs & 0x7fffffff;
    L.own = L.on && Fs >= 0;
    L.phPos = geZero(ph);
    L.down = L.on && (L.own ? L.phPos : ltZero(ph));
    L.dv = dv;
    L.phdt = ph * a.dt;
    L.aPhdt = fabs(L.phdt);
    kc.ownMask = (__ballot_sync(kAll, L.own) >> base) & gbits;
    kc.nfc = nfc;
    kc.pad = 0;
    // netFlux(c, dVf) in face order: the same every iteration
    double nf1 = 0.0;
    for (int k = 0; k < nmax; ++k) {
        const double x = __shfl_sync(kAll, dv, base + k);
        if (k < nfc) {
            if ((kc.ownMask >> k) & 1u)
                nf1 += x;
            else
                nf1 -= x;
        }
    }
    const double al = a.aNew[c];  // updated only after the dependency phase
    kc.Vi = m.V[c];
    kc.rVi = m.rV[c];
    kc.ov0 = pos0(al - 1.0) * (al - 1.0) + neg0(al) * al;
    kc.fluid0 = kc.ov0 * kc.Vi;
    double num = a.aOld[c] * a.rDeltaT;
    if (a.Su) num = num + a.Su[c];
    kc.num1 = num - divByRecip(nf1, kc.Vi, kc.rVi) * a.rDeltaT;
    kc.den = a.Sp ? (a.rDeltaT - a.Sp[c]) : a.rDeltaT;
    kc.rden = 1.0 / kc.den;
    kc.g = kc.rVi * a.rDeltaT;  // (1 / V) rDeltaT
    // the band is relative: with a subnormal aTol V every test divides
    const double t = kATol * kc.Vi;
    const bool normal = expField(t) != 0;
    kc.tolLo = normal ? t * (1.0 - 0x1p-40) : 0.0;
    kc.tolHi = normal ? t * (1.0 + 0x1p-40) : __longlong_as_double(0x7ff0000000000000LL);
    kc.eNum1 = expField(kc.num1);
    kc.eRden = expField(kc.rden);
    // the first iteration with every correction zero
    L.pass0 = false;
    L.maxExtra0 = 0.0;
    if (L.down) {
        const double dVff = dv + 0.0;
        const double me = geZero(kc.fluid0) ? fabs(L.phdt - dVff) : fabs(dVff);
        if (exceedsATol(me, kc)) {
            L.pass0 = true;
            L.maxExtra0 = me;
        }
    }
    kc.pm0 = (__ballot_sync(kAll, L.pass0) >> base) & gbits;
    double dVftot = 0.0;
    for (int k = 0; k < nmax; ++k) {
        const double x = __shfl_sync(kAll, L.aPhdt, base + k);
        if ((kc.pm0 >> k) & 1u) dVftot += x;
    }
    L.through0 = L.pass0 ? fabs(kc.fluid0) * L.aPhdt / dVftot : 0.0;
}

// The loop itself, once the corrections it reads are final.  cr0 is the
// correction on this lane's face as the earlier overshooting cell across it
// left it -- read only when the face is downwind for that cell (hasDep),
// the only case in which it can write one; zero otherwise (a later
// neighbour writes only after this cell in the reference's order, an
// inactive one writes nothing).  Returns this lane's final correction;
// pmFirst gets the faces that pass in the first iteration.
__device__ __forceinline__ double boundCellLoop(bool hasDep, double cr0, const BoundLane& L,
                                                const BoundCellConst& kc, const StepArgs& a, int lane,
                                                unsigned& pmFirst) {
    constexpr unsigned kAll = 0xffffffffu;
    double cr = cr0;
    double ov = kc.ov0, fluid = kc.fluid0;
    int nPass = 1;
    pmFirst = 0;
    for (int iter = 0; iter < 10; ++iter) {
        if (absLess(ov, kATol) || nPass == 0) break;
        bool pass = false;
        double pmax = 0.0;
        if (iter == 0 && !hasDep) {
            pass = L.pass0;
            pmax = L.maxExtra0;
        } else if (L.down) {
            const double dVff = L.dv + cr;
            // fabs(pos0(fluid) phi dt - dVff): pos0 is 1 or 0, and 0 phi dt - dVff
            // is -dVff up to the sign of a zero
            const double me = geZero(fluid) ? fabs(L.phdt - dVff) : fabs(dVff);
            if (exceedsATol(me, kc)) {
                pass = true;
                pmax = me;
            }
        }
        const unsigned pm = __ballot_sync(kAll, pass);
        double through = 0.0;
        if (iter == 0 && pm == kc.pm0) {
            through = L.through0;  // the same faces, so the same dVftot
        } else {
            double dVftot = 0.0;
            for (unsigned mm = pm; mm; mm &= mm - 1u) dVftot += __shfl_sync(kAll, L.aPhdt, __ffs(mm) - 1);
            if (pass) through = fabs(fluid) * L.aPhdt / dVftot;
        }
        int passInc = 0;
        if (pass) {
            passInc = geZero(pmax - through) ? 1 : 0;  // pos0(maxExtra - through)
            through = minNonNeg(through, pmax);
            // sign(phi) sign(fluid) through is +-through exactly
            cr = cr + ((L.phPos == geZero(fluid)) ? through : -through);
        }
        nPass = __reduce_add_sync(kAll, passInc);
        if (iter == 0) pmFirst = pm;
        // the next test ends the loop without reading alpha1New
        if (nPass == 0 || iter == 9) break;
        double nf2 = 0.0;  // netFlux(c, dVfcorrectionValues), face order
        const unsigned nz = __ballot_sync(kAll, L.on && !isZero(cr));
        for (unsigned mm = nz; mm; mm &= mm - 1u) {
            const int k = __ffs(mm) - 1;
            const double x = __shfl_sync(kAll, cr, k);
            if ((kc.ownMask >> k) & 1u)
                nf2 += x;
            else
                nf2 -= x;
        }
        // estimate: |a1 - alpha1New| < 2^-48 (|num1| + |t2|) |rden| + 2^-50 (|a1| + 1),
        // and |a1| < 2 inside the window; with the exponent test that is
        // below 2^-46 + 2^-48, so |alphaOvershoot| < aTol / 2 + that < aTol
        const double t2 = nf2 * kc.g;
        const double a1 = (kc.num1 - t2) * kc.rden;
        const long long b1 = bitsOf(a1);
        const bool inWindow = b1 >= 0 ? b1 < bitsOf(kUnitHi) : (b1 & 0x7fffffffffffffffLL) < bitsOf(kHalfATol);
        if (inWindow && max(kc.eNum1, expField(t2)) + kc.eRden <= 2045) break;
        double num = kc.num1;
        num = num - divByRecip(nf2, kc.Vi, kc.rVi) * a.rDeltaT;
        const double a1New = divByRecip(num, kc.den, kc.rden);
        ov = pos0(a1New - 1.0) * (a1New - 1.0) + neg0(a1New) * a1New;
        fluid = ov * kc.Vi;
    }
    (void)lane;
    return cr;
}

// After the dependency phase, for one overshooting cell (a warp, lane k on
// face k): the faces that passed in its first iteration join the list of
// corrected faces (key cell * 32 + position, the reference's list order)
// with their new dVf, and the cells on both sides become targets of the
// pass.  No later cell changes the correction of such a face, as a face is
// downwind for one side only.
__device__ void boundCellLists(int i, const DevMesh& m, const StepArgs& a, const BoundBuffers& s, int lane,
                               int pass, int passStamp, int stamp) {
    constexpr unsigned kAll = 0xffffffffu;
    const unsigned below = (1u << lane) - 1u;
    const int c = s.cand[i];
    const unsigned pmFirst = s.candPm[i];
    const bool first = (pmFirst >> lane) & 1u;
    int f = 0, t0 = -1, t1 = -1, c0 = passStamp, c1 = passStamp;
    bool fresh = false;
    if (first) {
        f = s.slotF[size_t(i) * m.maxCellFaces + lane];
        const double cr = s.corr[f];
        t0 = m.own[f];
        t1 = f < m.nfi ? m.nei[f] : -1;
        c0 = atomicExch(s.cellClaim + t0, passStamp);
        if (t1 >= 0) c1 = atomicExch(s.cellClaim + t1, passStamp);
        s.faceKey[f] = unsigned(c) * 32u + unsigned(__popc(pmFirst & below));
        s.faceStamp[f] = passStamp;
        const double nv = curDVf(m, f, a.phi, a.aCur, a.status, a.dvfI, a.alphaB, a.dt, s, stamp) + cr;
        fresh = s.modStamp[f] != stamp;
        s.dvfMod[f] = nv;
        s.modStamp[f] = stamp;
    }
    const bool w0 = first && c0 != passStamp, w1 = first && c1 != passStamp;
    const unsigned bm = __ballot_sync(kAll, fresh), b0 = __ballot_sync(kAll, w0), b1 = __ballot_sync(kAll, w1);
    int mBase = 0, tBase = 0;
    if (lane == 0) {
        if (bm) mBase = atomicAdd(s.ctl + kCtlMod, __popc(bm));
        if (b0 | b1) tBase = atomicAdd(s.ctl + kCtlTouched0 + pass, __popc(b0) + __popc(b1));
    }
    mBase = __shfl_sync(kAll, mBase, 0);
    tBase = __shfl_sync(kAll, tBase, 0);
    if (fresh) {
        const int p = mBase + __popc(bm & below);
        if (p < s.modCap) s.modList[p] = f;
        else boundOverflow(a, s, kOvfModList);
    }
    const int p0 = tBase + __popc(b0 & below) + __popc(b1 & below);
    if (w0) {
        if (p0 < s.touchedCap) s.touched[p0] = t0;
        else boundOverflow(a, s, kOvfTouchedList);
    }
    if (w1) {
        const int p1 = p0 + (w0 ? 1 : 0);
        if (p1 < s.touchedCap) s.touched[p1] = t1;
        else boundOverflow(a, s, kOvfTouchedList);
    }
}

// ready-queue entries carry the pass stamp, so stale ones never match
__device__ __forceinline__ void stQueue(unsigned long long* p, int passStamp, int i) {
    const unsigned long long v = (static_cast<unsigned long long>(unsigned(passStamp)) << 32) | unsigned(i);
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ldQueue(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ldVol(const int* p) { return *(volatile const int*)p; }

__global__ void __launch_bounds__(256, 2) kBound(StepArgs a, BoundBuffers s) {
    constexpr unsigned kAll = 0xffffffffu;
    const DevMesh& m = a.m;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nth = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    const int gw = tid >> 5, nw = nth >> 5;
    const int stamp = s.stamp;  // step stamp
    unsigned barK = 0;          // grid barriers passed
    const bool clock0 = tid == 0;  // block 0 keeps the time profile
    const unsigned long long tStart = clock0 ? globalNs() : 0ull;
    unsigned long long tDep = 0ull;
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
    if (!gridBarrier(s, a.err, barK)) return;

    int over = ovCount;  // overshooting cells in the whole mesh
    for (int pass = 0; pass < a.nAlphaBounds && pass < kMaxBoundPasses; ++pass) {
        if (over == 0) break;
        const int passStamp = stamp * kMaxBoundPasses + pass + 1;
        const int nCand = ldVol(s.ctl + kCtlCand);
        if (tid == 0) s.info[0] = pass + 1;
        // 2. the overshooting candidates (a half-warp or a warp per candidate,
        //    lane k of it on the cell's k-th face in cells() order): per face
        //    the dVf the pass
        //    starts from (final here: earlier passes are complete), the
        //    earlier overshooting cell it waits for (when the face is
        //    downwind for that cell, the only case in which it writes a
        //    correction there) and the later one it releases; then the loop's
        //    parts that read no correction.  Cells that wait for nobody go to
        //    the ready queue.
        {
            // two candidates per warp (a half-warp each) while every cell has
            // at most 16 faces, else one
            const bool wide = m.maxCellFaces > 16;
            const int per = wide ? 1 : 2;
            const int base = wide ? 0 : (lane & 16), gl = lane - base;
            const unsigned gbits = wide ? 0xffffffffu : 0xffffu;
            for (int r0 = gw * per; r0 < nCand; r0 += nw * per) {
                const int i = r0 + (base >> 4);
                const bool valid = i < nCand;
                const int c = valid ? s.cand[i] : s.cand[r0];
                const bool act = valid && overshoots(a.aNew[c]);
                if (!__any_sync(kAll, act)) continue;  // the same on every lane
                const int k0 = m.cOff[c], nfc = act ? m.cOff[c + 1] - k0 : 0;
                const int nmax = __reduce_max_sync(kAll, nfc);
                int Fs = 0, succ = -1;
                bool dep = false;
                double ph = 0.0, dv = 0.0;
                if (gl < nfc) {
                    const int f = m.cFaces[k0 + gl];
                    const int o = m.own[f];
                    const bool own = o == c;
                    const int nb = own ? (f < m.nfi ? m.nei[f] : -1) : o;
                    Fs = own ? f : int(unsigned(f) | 0x80000000u);
                    ph = a.phi[f];
                    dv = curDVf(m, f, a.phi, a.aCur, a.status, a.dvfI, a.alphaB, a.dt, s, stamp);
                    if (nb >= 0 && s.candMark[nb] == stamp && overshoots(a.aNew[nb])) {
                        if (nb < c && (own ? ltZero(ph) : geZero(ph))) {
                            dep = true;
                            s.corr[f] = __longlong_as_double(kCorrPending);  // until the earlier cell stores it
                        } else if (nb > c && (own ? geZero(ph) : ltZero(ph))) {
                            succ = s.candIdx[nb];
                        }
                    }
                }
                BoundLane L;
                BoundCellConst k;
                boundCellPrep(c, nfc, nmax, base, gbits, Fs, ph, dv, m, a, gl, L, k);
                const unsigned depMask = (__ballot_sync(kAll, dep) >> base) & gbits;
                if (L.on) {
                    const size_t sl = size_t(i) * m.maxCellFaces + gl;
                    s.slotF[sl] = L.F;
                    s.slotFlags[sl] = uint8_t(kSlotOn | (L.own ? kSlotOwn : 0) | (L.down ? kSlotDown : 0) |
                                              (L.phPos ? kSlotPhPos : 0) | (L.pass0 ? kSlotPass0 : 0) |
                                              (dep ? kSlotDep : 0));
                    s.slotSucc[sl] = succ;
                    s.slotDv[sl] = L.dv;
                    s.slotPhdt[sl] = L.phdt;
                    s.slotMax0[sl] = L.maxExtra0;
                    s.slotThr0[sl] = L.through0;
                }
                if (gl == 0 && act) {
                    reinterpret_cast<BoundCellConst*>(s.candK)[i] = k;
                    s.candDepN[i] = __popc(depMask);
                    s.candPending[i] = __popc(depMask);
                    s.actList[atomicAdd(s.ctl + kCtlActive0 + pass, 1)] = i;
                    if (depMask == 0) stQueue(s.readyQ + atomicAdd(s.ctl + kCtlQTail0 + pass, 1), passStamp, i);
                }
            }
        }
        if (!gridBarrier(s, a.err, barK)) return;
        const int nAct = ldVol(s.ctl + kCtlActive0 + pass);
        // no listed cell overshoots: this and every later pass change nothing
        if (nAct == 0) break;
        // 3. dependencies as dataflow.  A cell runs once every earlier
        //    overshooting neighbour it waits for has stored its corrections:
        //    the neighbour that completes it (the last one to decrement its
        //    count, or its only one) runs it next in the same warp, so a chain
        //    runs through in one warp; the others it completes go to the ready
        //    queue, from which idle warps take cells until all are done.  The
        //    correction values are their own flags (a face holds the pending
        //    NaN until the earlier cell stores it; a 64-bit store is single-
        //    copy atomic), so a released cell needs no fence.  Every wait is
        //    bounded: one that runs out sets the timeout bit and the warp
        //    stops; the others then stop at their own limits.
        const unsigned long long td0 = clock0 ? globalNs() : 0ull;
        {
            int longest = 0;
            bool failed = false;
            while (!failed) {
                int h = 0;
                if (lane == 0) h = atomicAdd(s.ctl + kCtlQHead0 + pass, 1);
                h = __shfl_sync(kAll, h, 0);
                if (h >= nAct) break;  // more takers than cells: nothing left for this warp
                int i = -1;
                if (lane == 0) {
                    for (long long spin = 0;; ++spin) {
                        const unsigned long long e = ldQueue(s.readyQ + h);
                        if (unsigned(e >> 32) == unsigned(passStamp)) {
                            i = int(unsigned(e));
                            break;
                        }
                        if (ldVol(s.ctl + kCtlDone0 + pass) >= nAct) break;  // all done: entry h never comes
                        if (spin >= s.spinLimit) {
                            atomicOr(a.err, (uint32_t)kErrBarrierTimeout);
                            i = -2;
                            break;
                        }
                        __nanosleep(100);
                    }
                    if (i >= 0) atomicAdd(s.ctl + kCtlStarts0 + pass, 1);
                }
                i = __shfl_sync(kAll, i, 0);
                if (i == -2) failed = true;
                if (i < 0) break;
                for (int hop = 0; i >= 0; ++hop) {
                    const BoundCellConst k = reinterpret_cast<const BoundCellConst*>(s.candK)[i];
                    BoundLane L;
                    uint8_t fl = 0;
                    int succ = -1;
                    L.F = 0;
                    L.dv = L.phdt = L.maxExtra0 = L.through0 = 0.0;
                    if (lane < k.nfc) {
                        const size_t sl = size_t(i) * m.maxCellFaces + lane;
                        fl = s.slotFlags[sl];
                        L.F = s.slotF[sl];
                        succ = s.slotSucc[sl];
                        L.dv = s.slotDv[sl];
                        L.phdt = s.slotPhdt[sl];
                        L.maxExtra0 = s.slotMax0[sl];
                        L.through0 = s.slotThr0[sl];
                    }
                    L.on = fl & kSlotOn;
                    L.own = fl & kSlotOwn;
                    L.down = fl & kSlotDown;
                    L.phPos = fl & kSlotPhPos;
                    L.pass0 = fl & kSlotPass0;
                    L.aPhdt = fabs(L.phdt);
                    const bool hasDep = fl & kSlotDep;
                    // how many cells this lane's successor waits for (read
                    // ahead; final since the candidates phase)
                    const int sDepN = succ >= 0 ? s.candDepN[succ] : 0;
                    long long cv = 0;  // bits of +0
                    bool stuck = false;
                    if (hasDep) {
                        for (long long spin = 0;; ++spin) {
                            cv = ldRelaxed64(s.corr + L.F);
                            if (cv != kCorrPending) break;
                            if (spin >= s.spinLimit) {
                                atomicOr(a.err, (uint32_t)kErrBarrierTimeout);
                                stuck = true;
                                break;
                            }
                            __nanosleep(32);
                        }
                    }
                    if (__any_sync(kAll, stuck)) {
                        failed = true;
                        break;
                    }
                    unsigned pmFirst = 0;
                    const double cr = boundCellLoop(hasDep, __longlong_as_double(cv), L, k, a, lane, pmFirst);
                    // only downwind faces can carry this cell's corrections, and
                    // each face is downwind for one side only: the face's one writer
                    if (L.down)
                        stRelaxed64(s.corr + L.F,
                                    bitsOf(cr) == kCorrPending ? __longlong_as_double(0x7fffffffffffffffLL) : cr);
                    if (lane == 0) {
                        s.candPm[i] = pmFirst;
                        atomicAdd(s.ctl + kCtlDone0 + pass, 1);
                    }
                    __syncwarp();
                    // release the later cells across the downwind faces
                    const bool rel = succ >= 0 && (sDepN == 1 || atomicSub(s.candPending + succ, 1) == 1);
                    const unsigned rm = __ballot_sync(kAll, rel);
                    longest = max(longest, hop + 1);
                    if (!rm) break;
                    const unsigned rest = rm & (rm - 1u);
                    if (rest) {
                        int base = 0;
                        if (lane == 0) base = atomicAdd(s.ctl + kCtlQTail0 + pass, __popc(rest));
                        base = __shfl_sync(kAll, base, 0);
                        if ((rest >> lane) & 1u)
                            stQueue(s.readyQ + base + __popc(rest & ((1u << lane) - 1u)), passStamp, succ);
                    }
                    i = __shfl_sync(kAll, succ, __ffs(rm) - 1);
                }
            }
            if (lane == 0 && longest > 0) atomicMax(s.info + 4, longest);
        }
        if (!gridBarrier(s, a.err, barK)) return;
        // a bounded wait ran out (the timeout bit was set before any block
        // reached this barrier, so every block leaves here)
        if (*(volatile uint32_t*)a.err & kErrBarrierTimeout) return;
        if (clock0) tDep += globalNs() - td0;
        // 3b. the corrected-face list and the targets of every overshooting cell
        for (int q = gw; q < nAct; q += nw) boundCellLists(s.actList[q], m, a, s, lane, pass, passStamp, stamp);
        if (!gridBarrier(s, a.err, barK)) return;
        // 4. alpha of every target cell, its updates in list order
        //    (advectionTemplates.C:164-192: own -= corr/V, nei += corr/V).
        //    A half-warp per target, lane k on the target's k-th face; a
        //    corrected face's rank is the number of corrected faces of the
        //    cell with a smaller key, and the half-warp adds the terms up in
        //    rank order.  Targets of the bounding set join the candidates
        //    (extendMarkedCells).  Loops and shuffles run on the whole warp.
        const int nT = min(ldVol(s.ctl + kCtlTouched0 + pass), s.touchedCap);
        {
            // a half-warp per target while every cell has at most 16 faces,
            // else a whole warp
            const bool wide = m.maxCellFaces > 16;
            const int gsz = wide ? 32 : 16, per = wide ? 1 : 2;
            const int half = wide ? 0 : (lane & 16), hl = wide ? lane : (lane & 15);
            const unsigned hmask = wide ? 0xffffffffu : (0xffffu << half);
            for (int r0 = (tid >> 5) * per; r0 < nT; r0 += (nth >> 5) * per) {
                const int r = r0 + (half >> 4);
                const bool valid = r < nT;
                const int t = valid ? s.touched[r] : 0;
                bool hit = false, ownSide = false, nbMixed = false;
                unsigned key = 0xffffffffu;
                double term = 0.0, at = 0.0, Vt = 1.0, rVt = 1.0;
                if (valid) {
                    const int k0 = m.cOff[t];
                    at = a.aNew[t];
                    Vt = m.V[t];
                    rVt = m.rV[t];
                    if (hl < m.cOff[t + 1] - k0) {
                        const int g = m.cFaces[k0 + hl];
                        const int nb = m.cSlot[k0 + hl].x;
                        nbMixed = nb >= 0 && a.status[nb] != kStNotMixed;
                        if (s.faceStamp[g] == passStamp) {
                            hit = true;
                            key = s.faceKey[g];
                            ownSide = m.own[g] == t;
                            term = divByRecip(s.corr[g], Vt, rVt);
                        }
                    }
                }
                const unsigned hits = __ballot_sync(0xffffffffu, hit) & hmask;
                const bool need = (__ballot_sync(0xffffffffu, nbMixed) & hmask) != 0;
                int rank = 0;
                for (int j = 0; j < gsz; ++j) {
                    const unsigned kj = __shfl_sync(0xffffffffu, key, half + j);
                    if (((hits >> (half + j)) & 1u) && kj < key) ++rank;
                }
                const bool before = overshoots(at);
                for (int e = 0; e < m.maxCellFaces; ++e) {
                    const unsigned who = __ballot_sync(0xffffffffu, hit && rank == e) & hmask;
                    const int src = who ? __ffs(who) - 1 : lane;
                    const double x = __shfl_sync(0xffffffffu, term, src);
                    const bool o = __shfl_sync(0xffffffffu, ownSide, src);
                    if (who) {
                        if (o) at -= x;
                        else at += x;
                    }
                }
                if (valid && hl == 0) {
                    a.aNew[t] = at;
                    aggAdd(s.ctl + kCtlOverDelta0 + pass, int(overshoots(at)) - int(before));
                    const bool inSet = need || a.status[t] != kStNotMixed;
                    if (inSet && s.candMark[t] != stamp && atomicExch(s.candMark + t, stamp) != stamp) {
                        const int p = aggAppend(s.ctl + kCtlCand);
                        if (2 * (p + 1) <= s.candCap) {
                            s.cand[p] = t;
                            s.candIdx[t] = p;
                        } else {
                            boundOverflow(a, s, kOvfCandidates);
                        }
                    }
                }
            }
        }
        if (!gridBarrier(s, a.err, barK)) return;
        over += ldVol(s.ctl + kCtlOverDelta0 + pass);
        if (tid == 0) {
            if (nAct > s.info[1]) s.info[1] = nAct;
            const int starts = ldVol(s.ctl + kCtlStarts0 + pass);
            if (starts > s.info[2]) s.info[2] = starts;
            s.info[5] += nAct;
        }
    }
    // alphaPhi = dVf / dt of every face the bounding changed this step
    const int nMod = min(ldVol(s.ctl + kCtlMod), s.modCap);
    for (int i = tid; i < nMod; i += nth) {
        const int f = s.modList[i];
        a.alphaPhi[f] = s.dvfMod[f] / a.dt;
    }
    if (clock0) {
        s.info[6] = int(tDep / 1000ull);
        s.info[7] = int((globalNs() - tStart) / 1000ull);
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
