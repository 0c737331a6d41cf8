// Device-side types and the FP64 geometry primitives of the plain SimPLIC
// form.  Every expression is written in the evaluation order of the
// reference (OpenFOAM Vector algebra: dot = (x*x' + y*y') + z*z', cross by
// components); translation units that include this header for the plain
// form are compiled with -fmad=false so no multiply-add is fused and every
// result is the IEEE-754 double of the written expression.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace simplic {

// OpenFOAM double constants
constexpr double kSMALL = 1.0e-15;
constexpr double kVSMALL = 1.0e-300;
constexpr double kROOTVSMALL = 1.0e-150;
constexpr double kTSMALL = 10.0 * kSMALL;

// Static caps of a cell (checked when a mesh is uploaded): any polyhedron
// with at most 32 faces and 32 points whose faces have at most 8 points.
constexpr int kMaxCellFaces = 32;
constexpr int kMaxFacePts = 8;
constexpr int kMaxCellPts = 32;
constexpr int kMaxSubPts = 2 * kMaxFacePts;

// The per-cell workspaces of the cut-cell routines are sized per cell
// class, one kernel instantiation per class present in the mesh, so the
// common cells keep a small working set: hexahedra and smaller cells
// (tetrahedra, prisms, pyramids); polyhedra up to 12 faces / 16 points;
// any cell within the caps (refined-mesh transition cells, split faces).
template <int MF, int MP, int MFP, int ME>
struct CellCaps {
    static constexpr int kFaces = MF;    // faces of the cell
    static constexpr int kPts = MP;      // points of the cell
    static constexpr int kFacePts = MFP; // points of one face
    static constexpr int kEdge = ME;     // interface edge points (cut points of all faces)
    static constexpr int kSub = 2 * MFP; // points of one clipped face
};
using CapsHex = CellCaps<6, 8, 4, 24>;
using CapsPoly = CellCaps<12, 16, 8, 48>;
using CapsBig = CellCaps<kMaxCellFaces, kMaxCellPts, kMaxFacePts, 4 * kMaxCellFaces>;
constexpr int kNumCellClasses = 3;
constexpr int kMaxStencil = 96;
constexpr int kMaxStencilCand = 256;

// per-cell status byte
constexpr int8_t kStNotMixed = 2;
constexpr int8_t kStPending = -100;

// device error bits
enum : uint32_t {
    kErrSubFaceOverflow = 1u << 0,
    kErrEdgeOverflow = 1u << 1,
    kErrStencilOverflow = 1u << 2,
    kErrBoundOverflow = 1u << 3,
    kErrNonFinite = 1u << 4,
    kErrBarrierTimeout = 1u << 5,
};

struct d3 {
    double x, y, z;
};

__host__ __device__ __forceinline__ d3 mk(double a, double b, double c) { return d3{a, b, c}; }
__host__ __device__ __forceinline__ d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ d3 operator*(double s, d3 a) { return {s * a.x, s * a.y, s * a.z}; }
__host__ __device__ __forceinline__ d3 operator/(d3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
__host__ __device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ d3 cross(d3 a, d3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ __forceinline__ double mag(d3 a) { return sqrt(dot(a, a)); }
__host__ __device__ __forceinline__ double sgn(double s) { return (s >= 0.0) ? 1.0 : -1.0; }
__host__ __device__ __forceinline__ double pos0(double s) { return (s >= 0.0) ? 1.0 : 0.0; }
__host__ __device__ __forceinline__ double neg0(double s) { return (s <= 0.0) ? 1.0 : 0.0; }
__host__ __device__ __forceinline__ d3 ld3(const double* p, int64_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
__host__ __device__ __forceinline__ void st3(double* p, int64_t i, d3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}
// The IEEE bit pattern of x through an opaque move.  Tests written on the
// bits (zero, sign, ordered range) stay integer instructions this way; a
// plain reinterpretation lets the compiler turn e.g. "(bits << 1) == 0"
// back into a double comparison, and every double instruction -- compares
// included -- goes through the narrow FP64 pipe of this part.
__device__ __forceinline__ long long bitsOf(double x) {
    long long r;
    asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
    return r;
}

// a / b rounded to nearest, given y = RN(1/b): the product a y corrected
// twice by Newton steps with fused multiply-add residuals (Markstein,
// IBM J. Res. Develop. 34 (1990) 111-119: once q is within one ulp of a/b
// and y is the correctly rounded reciprocal, r = a - b q is exact in an FMA
// and RN(q + r y) is the correctly rounded quotient).  The first step turns
// RN(a y) (up to 1.5 ulp off) into a faithful quotient, the second rounds
// it correctly.  Valid while the operands and the quotient are normal and
// the residuals exact (the range below); other inputs (subnormals,
// infinities, NaN, extreme ratios) take the division itself.  With y computed once per divisor this
// is 1 multiply and 4 FMAs instead of a full division.
//
// The range (biased exponent fields): a and b in [64, 1980] and the
// quotient's exponent ea - eb + 1023 in [64, 1980].  Then y and every q are
// normal, b q never overflows, and the residual a - b q is exact: its last
// bit is at least 2^(ea - 1023 - 105) >= 2^-1064 (a multiple of ulp(b)
// ulp(q), where ulp(q) >= ulp(a / b) / 2), so the FMA returns it without
// rounding.  A zero a over a finite nonzero b is the signed zero itself.
__host__ __device__ __forceinline__ double divByRecip(double a, double b, double y) {
#ifdef __CUDA_ARCH__
    const long long ba = __double_as_longlong(a), bb = __double_as_longlong(b);
#else
    long long ba, bb;
    std::memcpy(&ba, &a, sizeof ba);
    std::memcpy(&bb, &b, sizeof bb);
#endif
    const int ea = int((ba >> 52) & 0x7ff), eb = int((bb >> 52) & 0x7ff);
    if ((ba << 1) == 0 && eb != 0 && eb != 0x7ff) {
        const long long z = (ba ^ bb) & (long long)0x8000000000000000ULL;
        double r;
#ifdef __CUDA_ARCH__
        r = __longlong_as_double(z);
#else
        std::memcpy(&r, &z, sizeof r);
#endif
        return r;
    }
    if (ea < 64 || ea > 1980 || eb < 64 || eb > 1980 || ea - eb < 64 - 1023 || ea - eb > 1980 - 1023) return a / b;
#ifdef __CUDA_ARCH__
    const double q0 = __dmul_rn(a, y);
    const double q1 = __fma_rn(__fma_rn(-b, q0, a), y, q0);
    return __fma_rn(__fma_rn(-b, q1, a), y, q1);
#else
    const double q0 = a * y;
    const double q1 = std::fma(std::fma(-b, q0, a), y, q0);
    return std::fma(std::fma(-b, q1, a), y, q1);
#endif
}

// RN(dv / dt) where dv = RN(x dt), given y = RN(1/dt): dv / dt = x (1 + e)
// with |e| <= 2^-53, so x is a faithful approximation of the quotient (one
// of the two doubles around it, also at a binade boundary), and one Newton
// correction with the exact FMA residual dv - dt x rounds it correctly
// (Markstein's theorem, as in divByRecip).  The same range as divByRecip
// (every value normal, the residual exact); outside it, divByRecip.
__host__ __device__ __forceinline__ double divOfProduct(double dv, double dt, double y, double x) {
#ifdef __CUDA_ARCH__
    const long long ba = __double_as_longlong(dv), bb = __double_as_longlong(dt);
#else
    long long ba, bb;
    std::memcpy(&ba, &dv, sizeof ba);
    std::memcpy(&bb, &dt, sizeof bb);
#endif
    const int ea = int((ba >> 52) & 0x7ff), eb = int((bb >> 52) & 0x7ff);
    if (ea < 64 || ea > 1980 || eb < 64 || eb > 1980 || ea - eb < 64 - 1023 || ea - eb > 1980 - 1023)
        return divByRecip(dv, dt, y);
#ifdef __CUDA_ARCH__
    return __fma_rn(__fma_rn(-dt, x, dv), y, x);
#else
    return std::fma(std::fma(-dt, x, dv), y, x);
#endif
}

// the sign bit of x (set for -0 and negative NaNs too)
__host__ __device__ __forceinline__ bool negSignBit(double x) {
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x) < 0;
#else
    long long b;
    std::memcpy(&b, &x, sizeof b);
    return b < 0;
#endif
}
// atan2(y, x) in radians from correctly rounded +, -, *, / and sqrt only, so
// the host and the device (built without contraction) give the same bits:
// octant reduction to t = min / max in [0, 1], three half-angle steps
// atan t = 2 atan(t / (1 + sqrt(1 + t^2))) down to t <= tan(pi / 32), the
// Taylor series of atan to t^19 (remainder below 1e-21 t), times 8; then
// pi/2 - a above the diagonal, pi - a for x < 0 and the sign of y.  Signed
// zeros and non-finite inputs follow C's atan2.  Within a few ulp of the
// C library's atan2.
__host__ __device__ inline double planeAngle(double y, double x) {
    const double kPi = 3.141592653589793116, kHalfPi = 1.570796326794896558;
    if (x != x || y != y) return x + y;
    const double ax = fabs(x), ay = fabs(y);
    const bool steep = ay > ax;
    const double hi = steep ? ay : ax, lo = steep ? ax : ay;
    double a;
    if (hi == 0.0) {
        a = 0.0;
    } else if (hi - hi != 0.0) {  // infinite
        a = (lo == hi) ? 0.785398163397448279 : 0.0;
        if (lo == hi) {
            a = negSignBit(x) ? kPi - a : a;
            return negSignBit(y) ? -a : a;
        }
    } else {
        double t = lo / hi;
        for (int k = 0; k < 3; ++k) t = t / (1.0 + sqrt(1.0 + t * t));
        const double t2 = t * t;
        double p = -1.0 / 19.0;
        p = p * t2 + 1.0 / 17.0;
        p = p * t2 - 1.0 / 15.0;
        p = p * t2 + 1.0 / 13.0;
        p = p * t2 - 1.0 / 11.0;
        p = p * t2 + 1.0 / 9.0;
        p = p * t2 - 1.0 / 7.0;
        p = p * t2 + 1.0 / 5.0;
        p = p * t2 - 1.0 / 3.0;
        a = 8.0 * (t + t * (t2 * p));
    }
    if (steep) a = kHalfPi - a;
    if (negSignBit(x)) a = kPi - a;
    return negSignBit(y) ? -a : a;
}

// Grid-stride loops over short work lists (the mixed cells, the downwind
// faces of cut cells) deal the items out in warp-sized chunks, one chunk to
// each block before any block gets a second: with a grid of resident
// blocks spread over all SMs, a list of a few hundred warps of work then
// lands on every SM instead of on the first blocks' SMs.
__device__ __forceinline__ int spreadFirst() {
    return ((threadIdx.x >> 5) * gridDim.x + blockIdx.x) * 32 + (threadIdx.x & 31);
}
__device__ __forceinline__ int spreadStride() { return gridDim.x * blockDim.x; }

// v / n for a small integer count n: a power of two divides exactly like a
// multiplication by its reciprocal, which is cheaper on the FP64 pipe.
__device__ __forceinline__ d3 divCount(d3 v, int n) {
    if (n == 4) return 0.25 * v;
    if (n == 8) return 0.125 * v;
    if (n == 2) return 0.5 * v;
    if (n == 1) return v;
    const double dn = double(n);
    return v / dn;
}

// Unsigned division by a divisor fixed at mesh upload, d >= 2: n / d =
// (t + ((n - t) >> 1)) >> (l - 1) with t = mulhi(n, m), l = ceil(log2 d),
// m = floor(2^32 (2^l - d) / d) + 1 (Granlund and Montgomery, "Division by
// invariant integers using multiplication", PLDI 1994, Figure 4.1), exact
// for every 32-bit n.
struct FastDiv {
    uint32_t mul;
    int32_t sh;
};
inline FastDiv makeFastDiv(uint32_t d) {
    int l = 0;
    while ((1ull << l) < d) ++l;
    const unsigned long long m = ((1ull << 32) * ((1ull << l) - d)) / d + 1ull;
    return FastDiv{uint32_t(m), l - 1};
}
__host__ __device__ __forceinline__ uint32_t fastDivide(uint32_t n, FastDiv f) {
#ifdef __CUDA_ARCH__
    const uint32_t t = __umulhi(n, f.mul);
#else
    const uint32_t t = uint32_t((static_cast<unsigned long long>(n) * f.mul) >> 32);
#endif
    return (t + ((n - t) >> 1)) >> f.sh;
}

// Mesh arrays resident in HBM (structure of arrays, CSR addressing).
struct DevMesh {
    int32_t np, nf, nfi, nc;
    int32_t uniformFaces;    // faces of every cell when all cells have the same count
                             // (then cOff[c] = c * uniformFaces), else 0
    FastDiv latDivLayer, latDivNx;  // division by nx ny and by nx (a lattice only)
    int32_t latNx, latNy, latNz;  // a single-block lattice (cell i + nx (j + ny k), internal
                                  // faces by owner, +x +y +z): the slot records of every
                                  // interior cell follow from latticeSlots; else 0
    const double* pts;       // [3 np]
    const int32_t* fOff;     // [nf+1]
    const int32_t* fPts;     // face point lists, stored order
    const int32_t* own;      // [nf]
    const int32_t* nei;      // [nfi]
    const double* C;         // [3 nc]
    const double* V;         // [nc]
    const double* rV;        // [nc] 1 / V, correctly rounded
    const double* Cf;        // [3 nf]
    const double* magSf;     // [nf]
    const double* flat;      // [nf] face flatness
    const int32_t* cOff;     // [nc+1] cells() CSR
    const int32_t* cFaces;   // owned faces ascending, then neighbour faces
    const int2* cSlot;       // the same faces ascending, one record per slot:
                             // x = cell across the face (-1 on boundary),
                             // y = face id, bit 31 set on the neighbour side
    const int32_t* cpOff;    // [nc+1] cellPoints CSR (ascending)
    const int32_t* cPts;
    const uint8_t* boxCorner;  // [nc] axis-aligned box cell: 0x40 | lowest corner << 3 | highest
                               // corner (indices into the cell's points), else 0
    const int32_t* pcOff;    // [np+1] pointCells CSR (ascending)
    const int32_t* pCells;
    const int32_t* stOff;    // [nc+1] LS stencil CSR (buildStencil, built once): the other
    const int32_t* stCells;  // cells sharing a point, ascending; a row longer than
                             // kMaxStencil marks an overflow (its extra entry is -1)
    const double* pcW;       // normalised inverse-distance weights
    const int32_t* pbOff;    // [np+1] boundary faces of boundary points
    const int32_t* pbFaces;
    const double* pbW;
    const double* fullC;     // [3 nf] face::centre of each face (for fully submerged faces)
    const double* fullA;     // [3 nf] face::areaNormal of each face
    const uint8_t* cellClass;  // [nc] 0 CapsHex, 1 CapsPoly, 2 CapsBig
    int32_t classMask;         // bit k: the mesh has cells of class k
    const uint8_t* splitClass; // [nc] class of the splitWarpedFace workspace (when enabled)
    int32_t splitClassMask;    // 0 unless splitWarpedFace
    int32_t maxCellFaces;      // most faces of a cell (row stride of per-face scratch)
};

// Faces and points of a cell's splitWarpedFace workspace (host and device).
__host__ __device__ __forceinline__ void splitCounts(int nFaces, int nPts, const int* faceSizes, const bool* warped,
                                                     int& outFaces, int& outPts) {
    outFaces = 0;
    outPts = nPts;
    for (int k = 0; k < nFaces; ++k) {
        if (warped[k]) {
            outFaces += faceSizes[k];
            outPts += 1;
        } else {
            outFaces += 1;
        }
    }
}

// Smallest class whose caps hold a cell, -1 beyond the caps.
__host__ __device__ __forceinline__ int cellClassOf(int nFaces, int nPts, int maxFacePts) {
    if (nFaces <= CapsHex::kFaces && nPts <= CapsHex::kPts && maxFacePts <= CapsHex::kFacePts) return 0;
    if (nFaces <= CapsPoly::kFaces && nPts <= CapsPoly::kPts && maxFacePts <= CapsPoly::kFacePts) return 1;
    if (nFaces <= CapsBig::kFaces && nPts <= CapsBig::kPts && maxFacePts <= CapsBig::kFacePts) return 2;
    return -1;
}

// LS stencil (zoneCPCStencil): the cell, then all other cells sharing a
// point with it, ascending.  Returns the number of other cells in st[].
// Built once per mesh into DevMesh::stOff / stCells; the kernels read that.
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

// The precomputed stencil of cell c: its first entry in *st, the count as
// return value (at most kMaxStencil; an overflow sets the error bit).
__device__ __forceinline__ int stencilOf(const DevMesh& m, int c, const int32_t*& st, uint32_t& err) {
    const int s0 = m.stOff[c];
    int n = m.stOff[c + 1] - s0;
    if (n > kMaxStencil) {
        err |= kErrStencilOverflow;
        n = kMaxStencil;
    }
    st = m.stCells + s0;
    return n;
}

// The six face-slot records (ascending face id: -z, -y, -x neighbour sides,
// then the owned +x, +y, +z) of cell c when it is interior to the lattice;
// false for a boundary cell.  For an interior cell every owner involved
// owns all three of its faces, so the owners c - 1, c - nx, c - nx ny start
// 3, 3 nx - 1 and 3 nx ny - nx - ny faces before c.
// The records of cell c = i + nx (j + ny k), p = i + nx j, when it is interior.
__host__ __device__ __forceinline__ bool latticeSlotsAt(int c, int i, int j, int k, int p, int nx, int ny, int nz,
                                                        int2 (&sl)[6]) {
    const int layer = nx * ny;
    if (i == 0 || j == 0 || k == 0 || i == nx - 1 || j == ny - 1 || k == nz - 1) return false;
    // internal faces owned by the cells before c (faces are ordered by
    // owner, each owner's +x, +y, +z in turn): +x faces, nx - 1 per earlier
    // row plus one per earlier cell of c's row; +y faces, nx (ny - 1) per
    // earlier layer plus one per earlier cell of c's layer; +z faces, one
    // per earlier cell (every earlier cell in c's row / layer / the mesh
    // owns that face because c is interior)
    const int b = (j + ny * k) * (nx - 1) + i + k * nx * (ny - 1) + p + c;
    const unsigned side = 0x80000000u;
    sl[0] = make_int2(c - layer, int(unsigned(b - (3 * layer - nx - ny) + 2) | side));
    sl[1] = make_int2(c - nx, int(unsigned(b - (3 * nx - 1) + 1) | side));
    sl[2] = make_int2(c - 1, int(unsigned(b - 3) | side));
    sl[3] = make_int2(c + 1, b);
    sl[4] = make_int2(c + nx, b + 1);
    sl[5] = make_int2(c + layer, b + 2);
    return true;
}
__host__ __device__ __forceinline__ bool latticeSlots(int c, int nx, int ny, int nz, int2 (&sl)[6]) {
    const int layer = nx * ny;
    const int k = c / layer, p = c - k * layer;
    const int j = p / nx, i = p - j * nx;
    return latticeSlotsAt(c, i, j, k, p, nx, ny, nz, sl);
}
// the same with the two divisions by multiplications (dLayer: nx ny, dNx: nx)
__host__ __device__ __forceinline__ bool latticeSlotsFast(int c, int nx, int ny, int nz, FastDiv dLayer, FastDiv dNx,
                                                          int2 (&sl)[6]) {
    const int k = int(fastDivide(uint32_t(c), dLayer)), p = c - k * (nx * ny);
    const int j = int(fastDivide(uint32_t(p), dNx)), i = p - j * nx;
    return latticeSlotsAt(c, i, j, k, p, nx, ny, nz, sl);
}

}  // namespace simplic
