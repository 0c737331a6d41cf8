// Learned-normal form: network inputs, training samples and the choice
// between the network's normal and the least-squares one.
//
// Input of the network for an interface cell c (128 features): slots 0..30
// hold (alpha_j - alpha_c, (C_j - C_c) / h) with h = V_c^(1/3) -- slot 0 is
// c itself with its own alpha, slots 1..30 the cells of c's point-neighbour
// stencil nearest to C_c (ties by cell id), zero-padded -- and slot 31 the
// FP32 least-squares normal of those cells and a zero.  The network
// corrects that normal: the interface normal (pointing out of the liquid,
// as the reference's -grad(alpha)) is normalise(n_ls + y[0:3]); y[3] is the
// signed distance of the plane from C_c in units of h, (d + n.C_c) / h.
//
// Training samples come from the method's own cut-cell volume routine
// (cutCell::calcSubCell, FP64): a random plane through a random point of a
// random cell gives every stencil cell its exact volume fraction; a random
// sphere (radius 2h..20h) gives every stencil cell the volume fraction of
// its tangent plane at the sphere point nearest to the cell centre (exact
// for the plane, second order in h / R for the sphere), with the sphere
// normal at the point nearest to C_c as the label.
#include <cuda_bf16.h>

#include "cube_fraction_f32.cuh"
#include "ls_fp32.cuh"
#include "plain_geom.cuh"
#include "simplic_kernels.h"

namespace simplic {

namespace {

constexpr int kSlots = 32;      // feature slots of 4 values
constexpr int kCellSlots = 31;  // the cell and its 30 nearest neighbours

__device__ __forceinline__ uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform01(uint64_t& s) {
    return double(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ d3 randomUnit(uint64_t& s) {
    const double z = 2.0 * uniform01(s) - 1.0;
    const double phi = 6.283185307179586 * uniform01(s);
    const double r = sqrt(fmax(0.0, 1.0 - z * z));
    return mk(r * cos(phi), r * sin(phi), z);
}

// The (up to) 30 stencil cells nearest to C_c, nearest first.  Distances are
// compared in FP32 relative to h^2, so cells at the same distance up to
// round-off (the face, edge and corner neighbours of a regular grid) tie
// exactly and keep ascending id order.
__device__ int nearestNeighbours(const DevMesh& m, int c, int* sel, uint32_t& err) {
    constexpr int kMax = kCellSlots - 1;
    const int32_t* st;
    const int ns = stencilOf(m, c, st, err);
    const d3 Cc = ld3(m.C, c);
    const float ih2 = 1.0f / float(cbrt(m.V[c]) * cbrt(m.V[c]));
    float dsel[kMax];
    int n = 0;
    for (int s = 0; s < ns; ++s) {
        const int x = st[s];
        const d3 dx = ld3(m.C, x) - Cc;
        // rounded to 1/1024 of h^2: round-off noise cannot reorder equal distances
        const float d2 = rintf(float(dot(dx, dx)) * ih2 * 1024.0f);
        if (n == kMax && !(d2 < dsel[n - 1])) continue;  // ascending ids: an equal distance keeps the earlier
        int j = (n < kMax) ? n++ : n - 1;
        while (j > 0 && dsel[j - 1] > d2) {
            dsel[j] = dsel[j - 1];
            sel[j] = sel[j - 1];
            --j;
        }
        dsel[j] = d2;
        sel[j] = x;
    }
    return n;
}

// The neighbourhood in the network's terms before rounding to BF16.
struct Neighbourhood {
    int n;                   // cells used, the centre included
    float a[kCellSlots];     // alpha_j - alpha_c (slot 0: alpha_c)
    float r[kCellSlots][3];  // (C_j - C_c) / h
};

__device__ void writeRow(__nv_bfloat16* row, const Neighbourhood& nb) {
    float A[4][4] = {{0.f}}, b[4] = {0.f, 0.f, 0.f, 0.f};
    lsAccumulate(A, b, 0.f, 0.f, 0.f, 0.f);
    for (int k = 1; k < nb.n; ++k) lsAccumulate(A, b, nb.r[k][0], nb.r[k][1], nb.r[k][2], nb.a[k]);
    const float3 ls = lsNormal(A, b);
    for (int k = 0; k < kCellSlots; ++k) {
        const bool on = k < nb.n;
        row[4 * k + 0] = __float2bfloat16_rn(on ? nb.a[k] : 0.f);
        row[4 * k + 1] = __float2bfloat16_rn(on ? nb.r[k][0] : 0.f);
        row[4 * k + 2] = __float2bfloat16_rn(on ? nb.r[k][1] : 0.f);
        row[4 * k + 3] = __float2bfloat16_rn(on ? nb.r[k][2] : 0.f);
    }
    row[4 * kCellSlots + 0] = __float2bfloat16_rn(ls.x);
    row[4 * kCellSlots + 1] = __float2bfloat16_rn(ls.y);
    row[4 * kCellSlots + 2] = __float2bfloat16_rn(ls.z);
    row[4 * kCellSlots + 3] = __float2bfloat16_rn(0.f);
}

template <class K>
__device__ double cellVofK(const DevMesh& m, int c, d3 n, double d, uint32_t& err) {
    CellWS<K> w;
    if (!loadCell(m, c, w)) {
        err |= kErrSubFaceOverflow;
        return 0.0;
    }
    SubCell sc;
    calcSubCell(w, n, d, sc, err);
    return sc.vof;
}

// The cut volume fraction with the workspace of the cell's class.
__device__ double cellVof(const DevMesh& m, int c, d3 n, double d, uint32_t& err) {
    const int cls = m.cellClass[c];
    if (cls == 0) return cellVofK<CapsHex>(m, c, n, d, err);
    if (cls == 1) return cellVofK<CapsPoly>(m, c, n, d, err);
    return cellVofK<CapsBig>(m, c, n, d, err);
}

__global__ void __launch_bounds__(128) kMakeSamples(DevMesh m, unsigned long long seed, int count, int spherePct,
                                                    __nv_bfloat16* __restrict__ X, float* __restrict__ T,
                                                    uint32_t* __restrict__ errOut) {
    uint32_t err = 0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < count; s += gridDim.x * blockDim.x) {
        uint64_t rs = seed ^ (0xD1B54A32D192ED03ull * uint64_t(s + 1));
        int c = 0;
        double h = 1.0;
        d3 Cc = mk(0, 0, 0), nC = mk(0, 0, 1), ctr = mk(0, 0, 0);
        double dC = 0.0, R = 0.0, aC = 0.0;
        bool sphere = false;
        for (int attempt = 0; attempt < 16; ++attempt) {
            c = int(splitmix64(rs) % uint64_t(m.nc));
            Cc = ld3(m.C, c);
            h = cbrt(m.V[c]);
            sphere = int(splitmix64(rs) % 100) < spherePct;
            const d3 q = Cc + h * mk(0.8 * (uniform01(rs) - 0.5), 0.8 * (uniform01(rs) - 0.5),
                                     0.8 * (uniform01(rs) - 0.5));
            const d3 e = randomUnit(rs);
            if (sphere) {
                R = h * 2.0 * pow(10.0, uniform01(rs));  // 2h .. 20h
                ctr = q - R * e;
                const d3 r = Cc - ctr;
                nC = (1.0 / mag(r)) * r;
                dC = -dot(nC, ctr + R * nC);
            } else {
                nC = e;
                dC = -dot(e, q);
            }
            aC = cellVof(m, c, nC, dC, err);
            if (aC > 1e-6 && aC < 1.0 - 1e-6) break;
        }
        int sel[kCellSlots - 1];
        const int nn = nearestNeighbours(m, c, sel, err);
        Neighbourhood nb;
        nb.n = nn + 1;
        nb.a[0] = float(aC);
        nb.r[0][0] = nb.r[0][1] = nb.r[0][2] = 0.f;
        for (int k = 0; k < nn; ++k) {
            const int j = sel[k];
            const d3 Cj = ld3(m.C, j);
            d3 nj = nC;
            double dj = dC;
            if (sphere) {
                const d3 r = Cj - ctr;
                nj = (1.0 / mag(r)) * r;
                dj = -dot(nj, ctr + R * nj);
            }
            const double aj = cellVof(m, j, nj, dj, err);
            const d3 rel = (1.0 / h) * (Cj - Cc);
            nb.a[k + 1] = float(aj - aC);
            nb.r[k + 1][0] = float(rel.x);
            nb.r[k + 1][1] = float(rel.y);
            nb.r[k + 1][2] = float(rel.z);
        }
        writeRow(X + size_t(s) * (4 * kSlots), nb);
        T[4 * size_t(s) + 0] = float(nC.x);
        T[4 * size_t(s) + 1] = float(nC.y);
        T[4 * size_t(s) + 2] = float(nC.z);
        T[4 * size_t(s) + 3] = float((dC + dot(nC, Cc)) / h);
    }
    if (err) atomicOr(errOut, err);
}

// float(x) rounded to nearest even, on the integer pipe: a conversion
// instruction from double goes through the FP64 pipe, which on this part
// issues a whole warp at a time at a small fraction of the FP32 rate.
// Subnormal results are rounded like the hardware's; a NaN input gives a NaN.
__device__ __forceinline__ float toFloatRn(double x) {
    const unsigned long long b = static_cast<unsigned long long>(bitsOf(x));
    const unsigned sign = unsigned(b >> 32) & 0x80000000u;
    const int e = int((b >> 52) & 0x7ff);
    if (e == 0x7ff) return __uint_as_float(sign | ((b << 12) ? 0x7fc00000u : 0x7f800000u));
    const int fe = e - 1023 + 127;  // biased float exponent
    if (fe >= 255) return __uint_as_float(sign | 0x7f800000u);
    // the 53-bit significand with its implicit bit (none for zero or subnormal doubles)
    unsigned long long sig = (b & 0xfffffffffffffull) | (e ? (1ull << 52) : 0ull);
    // bits to drop: 29 for a normal float, more below the normal range
    const int drop = fe >= 1 ? 29 : 29 + (1 - fe);
    if (drop > 54) return __uint_as_float(sign);  // below half the smallest subnormal
    const unsigned long long keep = sig >> drop;
    const unsigned long long rem = sig & ((1ull << drop) - 1ull);
    const unsigned long long half = 1ull << (drop - 1);
    unsigned long long r = keep + ((rem > half || (rem == half && (keep & 1ull))) ? 1ull : 0ull);
    // normal: the implicit bit carries into the exponent field; subnormal:
    // the exponent field is 0 and a carry into bit 23 makes the smallest normal
    const unsigned bits = fe >= 1 ? (unsigned(fe - 1) << 23) + unsigned(r) : unsigned(r);
    return __uint_as_float(sign | bits);
}

// Network input of every mixed cell (rows beyond maxRows are not written)
// and the FP32 least-squares normal of the same neighbourhood (the
// fallback normal of the learned form, for every mixed cell), one warp per
// cell.  Per stencil cell (one per lane) the only double operations are the
// centre offset C_j - C_c and alpha_j - alpha_c (rounded to float on the
// integer pipe); the squared distance and the scaled offsets are FP32
// products (explicitly rounded, no contraction).  A cell's slot is the
// number of stencil cells with a smaller (distance rounded to h^2/1024, id)
// key, the order of nearestNeighbours.  The cell constants (h) are computed
// for 32 cells at once, one per lane.  Lane k then writes slot k (one
// 8-byte store) and adds its share of the least-squares sums (summed
// across the warp).
constexpr int kGatherWarps = 4;
__global__ void __launch_bounds__(32 * kGatherWarps) kGatherFeaturesWarp(DevMesh m, const double* __restrict__ alpha,
                                                                         const int* __restrict__ mixed,
                                                                         const int* __restrict__ nMixed, int maxRows,
                                                                         __nv_bfloat16* __restrict__ X,
                                                                         float* __restrict__ Arows,
                                                                         double* __restrict__ nrm,
                                                                         uint32_t* __restrict__ errOut) {
    __shared__ unsigned long long sKey[kGatherWarps][kMaxStencil];
    __shared__ float4 sVal[kGatherWarps][kMaxStencil];  // (alpha_j - alpha_c, (C_j - C_c) / h)
    __shared__ int sSel[kGatherWarps][kCellSlots - 1];
    constexpr unsigned kAll = 0xffffffffu;
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long* key = sKey[wl];
    float4* val = sVal[wl];
    int* sel = sSel[wl];
    const int nm = *nMixed;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t err = 0;
    for (int b0 = w0; b0 < nm; b0 += 32 * nw) {
        // constants of this warp's next 32 cells, one per lane
        const int il = b0 + lane * nw;
        float ihL = 0.f, ih2L = 0.f;
        if (il < nm) {
            const double hc = cbrt(m.V[mixed[il]]);
            ihL = toFloatRn(1.0 / hc);
            ih2L = 1.0f / toFloatRn(hc * hc);
        }
        for (int j = 0; j < 32 && b0 + j * nw < nm; ++j) {
            const int i = b0 + j * nw;
            const float ih = __shfl_sync(kAll, ihL, j);
            const float ih2 = __shfl_sync(kAll, ih2L, j);
            const int c = mixed[i];
            const d3 Cc = ld3(m.C, c);
            const double ac = alpha[c];
            const int32_t* st;
            const int nU = stencilOf(m, c, st, err);
            for (int u = lane; u < nU; u += 32) {
                const int x = st[u];
                const d3 dx = ld3(m.C, x) - Cc;
                const float fx = toFloatRn(dx.x), fy = toFloatRn(dx.y), fz = toFloatRn(dx.z);
                const float q = __fadd_rn(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)), __fmul_rn(fz, fz));
                const float d2 = rintf(__fmul_rn(__fmul_rn(q, ih2), 1024.0f));
                key[u] = (static_cast<unsigned long long>(static_cast<unsigned>(d2)) << 32) | static_cast<unsigned>(x);
                val[u] = make_float4(toFloatRn(alpha[x] - ac), __fmul_rn(fx, ih), __fmul_rn(fy, ih), __fmul_rn(fz, ih));
            }
            __syncwarp();
            for (int u = lane; u < nU; u += 32) {
                const unsigned long long k = key[u];
                int rank = 0;
                for (int f = 0; f < nU; ++f) rank += key[f] < k ? 1 : 0;
                if (rank < kCellSlots - 1) sel[rank] = u;
            }
            __syncwarp();
            const int nn = min(nU, kCellSlots - 1);
            float4 v = make_float4(lane == 0 ? toFloatRn(ac) : 0.f, 0.f, 0.f, 0.f);
            if (lane >= 1 && lane <= nn) v = val[sel[lane - 1]];
            // least squares: the centre (zero offset, zero value) and slots 1..nn
            float A[4][4] = {{0.f}}, b[4] = {0.f, 0.f, 0.f, 0.f};
            if (lane <= nn) lsAccumulate(A, b, v.y, v.z, v.w, lane == 0 ? 0.f : v.x);
#pragma unroll
            for (int o = 16; o; o >>= 1) {
#pragma unroll
                for (int p = 0; p < 4; ++p)
#pragma unroll
                    for (int r = p; r < 4; ++r) A[p][r] += __shfl_xor_sync(kAll, A[p][r], o);
#pragma unroll
                for (int p = 0; p < 4; ++p) b[p] += __shfl_xor_sync(kAll, b[p], o);
            }
            const float3 ls = lsNormal(A, b);
            if (lane == 0) st3(nrm, i, mk(double(ls.x), double(ls.y), double(ls.z)));
            if (i < maxRows) {
                __nv_bfloat16 h4[4];
                if (lane < kCellSlots) {
                    h4[0] = __float2bfloat16_rn(v.x);
                    h4[1] = __float2bfloat16_rn(v.y);
                    h4[2] = __float2bfloat16_rn(v.z);
                    h4[3] = __float2bfloat16_rn(v.w);
                } else {
                    h4[0] = __float2bfloat16_rn(ls.x);
                    h4[1] = __float2bfloat16_rn(ls.y);
                    h4[2] = __float2bfloat16_rn(ls.z);
                    h4[3] = __float2bfloat16_rn(0.f);
                }
                uint2 w;
                memcpy(&w, h4, sizeof(w));
                reinterpret_cast<uint2*>(X + size_t(i) * (4 * kSlots))[lane] = w;
                Arows[size_t(i) * 32 + lane] = lane < kCellSlots ? v.x : 0.f;
            }
            __syncwarp();  // the shared lists are refilled for the next cell
        }
    }
    if (err) atomicOr(errOut, err);
}

// Local volume residual of normal n for one network row, summed across the
// warp (lane k on neighbour slot k, offset r in units of h, alpha aj): the
// plane with that normal cutting the cell's own volume fraction ac from a
// cube of the cell's size centred on the cell is laid through equal cubes
// centred on the neighbours; R = sum |fraction_j - alpha_j|.  The plane
// coefficients are raised to at least kCubeMinM of their sum.
// The cube model of one normal for one row: its coefficients and the plane
// constant that cuts the cell's own volume fraction from the cell's cube
// ([-1/2, 1/2]^3); computed once and shared by both measures.
struct CubePlane {
    CubeCoef c;
    float3 p;
    float a0;
    bool ok;
};
__device__ __forceinline__ CubePlane cubePlane(float nx, float ny, float nz, float ac) {
    CubePlane q;
    q.ok = cubeCoefficientsF(nx, ny, nz, q.c, q.p);
    q.a0 = q.ok ? cubeInverseF(ac, q.c) : 0.f;
    return q;
}

__device__ float localResidualWarp(const CubePlane& q, bool on, float rx, float ry, float rz, float aj) {
    if (!q.ok) return 3.0e38f;
    const CubeCoef& c = q.c;
    const float3& p = q.p;
    const float a0 = q.a0;
    float t = 0.f;
    if (on) {
        float d;
        t = fabsf(cubeFractionF(a0 - (p.x * rx + p.y * ry + p.z * rz), c, d) - aj);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// Face-flux mismatch of normal n for one network row, summed across the
// warp: on every face of the cell's cube with a face neighbour (a slot at
// offset +-1 along one axis), the part of the face below the cell's plane
// against the part below the neighbour's own plane (same normal, through
// the neighbour's cube at its volume fraction).  A plane that continues
// across the face gives equal parts; the sum of |difference| says how
// much the fluxes the two cells' planes imply through their shared faces
// disagree.  Zero where no slot is a face neighbour (non-hexahedral
// neighbourhoods).
__device__ float faceMismatchWarp(const CubePlane& q, bool on, float rx, float ry, float rz, float aj) {
    if (!q.ok) return 3.0e38f;
    const CubeCoef& c = q.c;
    const float3& p = q.p;
    float t = 0.f;
    const float ax = fabsf(rx), ay = fabsf(ry), az = fabsf(rz);
    const int axis = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    const float ra = axis == 0 ? rx : (axis == 1 ? ry : rz);
    const float rest = axis == 0 ? ay + az : (axis == 1 ? ax + az : ax + ay);
    if (on && fabsf(ra) > 0.75f && fabsf(ra) < 1.25f && rest < 0.25f) {
        const float sigma = ra > 0.f ? 1.f : -1.f;
        const float aj0 = cubeInverseF(aj, c);  // the neighbour's own plane
        t = fabsf(cubeFaceFractionF(q.a0, p, axis, sigma) - cubeFaceFractionF(aj0, p, axis, -sigma));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// The learned form's choice, one warp per network row.  The network's
// normal normalise(n_ls + y[0:3]) (n_ls from the row's input) replaces the
// least-squares normal unless it is degenerate, or raises the local volume
// residual or the face-flux mismatch above the least-squares normal's by
// more than gateTol.  (The network's fourth output, its estimate of the
// plane constant, is trained but not used: the plane solve takes the closed
// form on box cells and the reference's bracket elsewhere.)
__global__ void __launch_bounds__(128) kLearnedGate(const int* __restrict__ nMixed, int maxRows,
                                                    const __nv_bfloat16* __restrict__ X, const float* __restrict__ A,
                                                    const float* __restrict__ Y, int ldY, double* __restrict__ nrm,
                                                    float gateTol, int* __restrict__ nLearned) {
    const int lane = threadIdx.x & 31;
    const int rows = min(*nMixed, maxRows);
    const int nw = (gridDim.x * blockDim.x) >> 5;
    int used = 0;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < rows; i += nw) {
        // slot lane of the row: (alpha_j - alpha_c, offset / h) in BF16; slot 31 the LS normal
        const uint2 q = reinterpret_cast<const uint2*>(X + size_t(i) * (4 * kSlots))[lane];
        const float rx = __uint_as_float(q.x & 0xffff0000u), ry = __uint_as_float(q.y << 16),
                    rz = __uint_as_float(q.y & 0xffff0000u);
        const float ac = A[size_t(i) * 32];
        const float aj = ac + A[size_t(i) * 32 + lane];
        const bool on = lane >= 1 && lane < kCellSlots && (rx != 0.f || ry != 0.f || rz != 0.f);
        const float lsx = __shfl_sync(0xffffffffu, __uint_as_float(q.x << 16), 31);
        const float lsy = __shfl_sync(0xffffffffu, __uint_as_float(q.x & 0xffff0000u), 31);
        const float lsz = __shfl_sync(0xffffffffu, __uint_as_float(q.y << 16), 31);
        // FP32 throughout: a double operation here would be issued for the
        // whole warp, and the normal is only as precise as its BF16 input
        const float* y = Y + size_t(i) * ldY;
        const float vx = lsx + y[0], vy = lsy + y[1], vz = lsz + y[2];
        const float vn = sqrtf(vx * vx + vy * vy + vz * vz);
        if (vn > 1e-3f) {
            const float iv = 1.f / vn;
            const float nx = vx * iv, ny = vy * iv, nz = vz * iv;
            const float3 ls = make_float3(float(nrm[3 * size_t(i)]), float(nrm[3 * size_t(i) + 1]),
                                          float(nrm[3 * size_t(i) + 2]));
            const float lsMag2 = ls.x * ls.x + ls.y * ls.y + ls.z * ls.z;
            // Both measures are sums of magnitudes (>= 0), so a network normal
            // whose own measure is within gateTol passes its test without the
            // least-squares normal's; the face test only where the volume
            // test keeps the network's normal.  (The sums are the same on
            // every lane, so the branches are warp-uniform.)
            const CubePlane qN = cubePlane(nx, ny, nz, ac);
            const float rLearned = localResidualWarp(qN, on, rx, ry, rz, aj);
            bool keep = rLearned <= gateTol;
            if (!keep) {
                const float rLs = lsMag2 < 1e-28f
                                      ? 3.0e38f
                                      : localResidualWarp(cubePlane(ls.x, ls.y, ls.z, ac), on, rx, ry, rz, aj);
                keep = rLearned <= rLs + gateTol;
            }
            if (keep) {
                const float fLearned = faceMismatchWarp(qN, on, rx, ry, rz, aj);
                keep = fLearned <= gateTol;
                if (!keep) {
                    const float fLs = lsMag2 < 1e-28f
                                          ? 3.0e38f
                                          : faceMismatchWarp(cubePlane(ls.x, ls.y, ls.z, ac), on, rx, ry, rz, aj);
                    keep = fLearned <= fLs + gateTol;
                }
            }
            if (keep) {
                if (lane == 0) st3(nrm, i, mk(double(nx), double(ny), double(nz)));
                ++used;
            }
        }
    }
    if (lane == 0 && used) atomicAdd(nLearned, used);
}

}  // namespace

void launchMakeSamples(const DevMesh& m, unsigned long long seed, int count, int spherePct, void* X, float* T,
                       uint32_t* err, cudaStream_t st) {
    const int grid = (count + 127) / 128;
    kMakeSamples<<<grid, 128, 0, st>>>(m, seed, count, spherePct, static_cast<__nv_bfloat16*>(X), T, err);
}

void launchGatherFeatures(const StepArgs& a, int maxRows, void* X, float* A, cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    kGatherFeaturesWarp<<<sms * 8, 32 * kGatherWarps, 0, st>>>(a.m, a.aCur, a.mixed, a.nMixed, maxRows,
                                                               static_cast<__nv_bfloat16*>(X), A, a.nrm, a.err);
}

void launchLearnedGate(const StepArgs& a, int maxRows, const void* X, const float* A, const float* Y, int ldY,
                       float gateTol, int* nLearned, cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // a warp per row over 32 blocks per SM (the row's cube inverses iterate:
    // latency, hidden by more warps in flight)
    kLearnedGate<<<sms * 32, 128, 0, st>>>(a.nMixed, maxRows, static_cast<const __nv_bfloat16*>(X), A, Y, ldY, a.nrm,
                                          gateTol, nLearned);
}

}  // namespace simplic
