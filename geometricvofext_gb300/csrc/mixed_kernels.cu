// Mixed-precision SimPLIC kernels (built with fused multiply-add allowed).
//
// The mixed form changes the method's arithmetic, not its steps:
//   * interface normals: the same least-squares fit over the same stencil
//     (reconstruction.C:85-141) in FP32 on cell-centred coordinates scaled
//     by the cell size;
//   * plane constant: FP64.  An axis-aligned box cell takes the closed-form
//     plane constant of its cuboid (the cut volume inverted region by region,
//     checked against alpha); any other cell takes the reference's own steps
//     (cutCell.C:611-799: the bracket of two vertex levels, the cubic through
//     the 1/3 and 2/3 cuts, Newton on the cubic);
//   * Simpson fluxes: the clipped face areas of cutFace::timeIntegratedArea
//     (cutFace.C:392-506) in FP32 on face-local coordinates (points shifted
//     by the face centre, plane constant shifted with them), fan sums with
//     Kahan compensation, the smaller side of a cut face clipped; vertex
//     times in FP32, interval widths, the Simpson sum and dVf in FP64.
// The update and the bounding of the mixed form are the FP64 kernels of the
// plain form, so mass is conserved to FP64 round-off either way.
#include "ls_fp32.cuh"
#include "plain_geom.cuh"
#include "simplic_kernels.h"

#include <mutex>

namespace simplic {

namespace {

// ---------------------------------------------------------------------------
// FP32 vector helpers
// ---------------------------------------------------------------------------
struct v3f {
    float x, y, z;
};
__device__ __forceinline__ v3f fv(float a, float b, float c) { return v3f{a, b, c}; }
__device__ __forceinline__ v3f operator+(v3f a, v3f b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ v3f operator-(v3f a, v3f b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ v3f operator*(float s, v3f a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float dotf(v3f a, v3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ v3f crossf(v3f a, v3f b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float magf(v3f a) { return sqrtf(dotf(a, a)); }
__device__ __forceinline__ v3f toF(d3 a) { return {float(a.x), float(a.y), float(a.z)}; }

// Kahan-compensated vector sum
struct KahanV {
    v3f s{0.f, 0.f, 0.f}, c{0.f, 0.f, 0.f};
    __device__ __forceinline__ void add(v3f v) {
        const v3f y = v - c;
        const v3f t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// ---------------------------------------------------------------------------
// normals: FP32 least squares
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) kLsNormalMixed(DevMesh m, const double* __restrict__ alpha,
                                                      const int* __restrict__ mixed, const int* __restrict__ nMixed,
                                                      double* __restrict__ nrm, uint32_t* __restrict__ errOut) {
    const int nm = *nMixed;
    uint32_t err = 0;
    for (int i = spreadFirst(); i < nm; i += spreadStride()) {
        const int c = mixed[i];
        const int32_t* st;
        const int ns = stencilOf(m, c, st, err);
        const d3 Cc = ld3(m.C, c);
        const double ac = alpha[c];
        const float invH = rcbrtf(float(m.V[c]));
        float A[4][4] = {{0.f}}, b[4] = {0.f, 0.f, 0.f, 0.f};
        for (int s = -1; s < ns; ++s) {
            const int x = (s < 0) ? c : st[s];
            const d3 dx = ld3(m.C, x) - Cc;  // FP64 difference, then scaled to O(1) in FP32
            // alpha relative to the cell's own value (the fitted gradient does
            // not change): in a nearly full or nearly empty neighbourhood the
            // differences are tiny and would drown in FP32 rounding of
            // values near 1
            lsAccumulate(A, b, float(dx.x) * invH, float(dx.y) * invH, float(dx.z) * invH, float(alpha[x] - ac));
        }
        const float3 nf = lsNormal(A, b);
        const d3 n = mk(double(nf.x), double(nf.y), double(nf.z));
        st3(nrm, i, n);
    }
    if (err) atomicOr(errOut, err);
}

// ---------------------------------------------------------------------------
// plane constant of box cells: the closed form, checked on the box volume
// ---------------------------------------------------------------------------
// |VOF(d) - alpha| the closed form must reach: times a Courant number below
// one it stays under the bounding tolerance 1e-13, so a full neighbour of a
// cut cell does not overshoot through the solve
constexpr double kVolTol = 5e-14;

// Fraction of the unit cube below sum m_i x_i = a (Scardovelli & Zaleski,
// J. Comput. Phys. 164 (2000) 228-237: inclusion-exclusion over the cube
// corners) for m1 <= m2 <= m3, sum m_i = 1, a in [m1, 1/2], written so that
// no term divides a large cube by a small m1: the part of the m1 corner is
// expanded, (a^3 - (a - m1)^3) / m1 = 3a^2 - 3a m1 + m1^2.  k6 = 1/(6 m1 m2 m3).
__device__ __forceinline__ void cubeVolumeCubic(double a, double m1, double m2, double m3, double k6, double& v,
                                                double& dv) {
    v = (3.0 * a * a - 3.0 * a * m1 + m1 * m1) * (m1 * k6);
    dv = (6.0 * a - 3.0 * m1) * (m1 * k6);
    if (a > m2) {
        const double t = a - m2;
        v -= t * t * t * k6;
        dv -= 3.0 * t * t * k6;
    }
    if (a > m3) {
        const double t = a - m3;
        v -= t * t * t * k6;
        dv -= 3.0 * t * t * k6;
    }
    if (a > m1 + m2) {
        const double t = a - m1 - m2;
        v += t * t * t * k6;
        dv += 3.0 * t * t * k6;
    }
}

// a in [0, 1/2] with volume fraction v <= 1/2 below sum m_i x_i = a: closed
// form in the corner (cube root), edge (quadratic) and prism (linear)
// regions, Newton inside the bracket of a cubic region.
__device__ double cubeInverse(double v, double m1, double m2, double m3) {
    const double k6 = 1.0 / (6.0 * m1 * m2 * m3);
    const double v1 = m1 * m1 / (6.0 * m2 * m3);
    const double v2 = v1 + (m2 - m1) / (2.0 * m3);
    if (v <= v1) return cbrt(v / k6);
    if (v <= v2) return (3.0 * m1 + sqrt(fmax(72.0 * m2 * m3 * v - 3.0 * m1 * m1, 0.0))) / 6.0;
    double lo, hi, vlo, vhi;
    if (m3 >= m1 + m2) {
        const double v3 = (m1 + m2) / (2.0 * m3);
        if (v >= v3) return m3 * v + 0.5 * (m1 + m2);
        lo = m2, hi = m1 + m2, vlo = v2, vhi = v3;
    } else {
        double v3, dv3;
        cubeVolumeCubic(m3, m1, m2, m3, k6, v3, dv3);
        if (v <= v3)
            lo = m2, hi = m3, vlo = v2, vhi = v3;
        else
            lo = m3, hi = 0.5, vlo = v3, vhi = 0.5;
    }
    double a = (vhi > vlo) ? lo + (v - vlo) / (vhi - vlo) * (hi - lo) : 0.5 * (lo + hi);
    for (int it = 0; it < 12; ++it) {
        double q, dq;
        cubeVolumeCubic(a, m1, m2, m3, k6, q, dq);
        const double r = q - v;
        if (r > 0.0)
            hi = a;
        else
            lo = a;
        double an = (dq > 0.0) ? a - r / dq : 0.5 * (lo + hi);
        if (!(an >= lo && an <= hi)) an = 0.5 * (lo + hi);
        const bool done = fabs(an - a) <= 2e-16;
        a = an;
        if (done) break;
    }
    return a;
}

// Plane constant of the axis-aligned box [lo, hi] whose part n.x + d < 0 has
// volume fraction alpha (the exact plane constant of a box-shaped cell).
__device__ double cuboidPlaneConstant(d3 n, d3 lo, d3 hi, double alpha) {
    const double L[3] = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
    const double nn[3] = {n.x, n.y, n.z};
    double mm[3], M = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        mm[i] = fabs(nn[i]) * L[i];
        M += mm[i];
    }
    // corner where the local coordinates start: n.x = n.corner + sum mm_i x'_i
    const double corner = (n.x >= 0 ? n.x * lo.x : n.x * hi.x) + (n.y >= 0 ? n.y * lo.y : n.y * hi.y) +
                          (n.z >= 0 ? n.z * lo.z : n.z * hi.z);
    if (!(M > 0.0)) return -corner;
    double m[3] = {mm[0] / M, mm[1] / M, mm[2] / M};
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2 - i; ++j)
            if (m[j] > m[j + 1]) {
                const double t = m[j];
                m[j] = m[j + 1];
                m[j + 1] = t;
            }
    // keep every m_i away from zero (the box volume check decides whether the
    // plane is kept: where the clamp moves the cut volume past the check's
    // tolerance, the cell takes the general solve)
#pragma unroll
    for (int i = 0; i < 3; ++i) m[i] = fmax(m[i], 1e-9);
    const double sum = m[0] + m[1] + m[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) m[i] /= sum;
    const bool flip = alpha > 0.5;
    double a = cubeInverse(flip ? 1.0 - alpha : alpha, m[0], m[1], m[2]);
    if (flip) a = 1.0 - a;
    return -(a * sum * M + corner);
}

// Volume fraction F of the unit cube below sum m_i x_i = a (m1 <= m2 <= m3,
// sum 1, m1 >= kBoxMinM) and dF/da, piecewise after Scardovelli & Zaleski
// (2000) with every region written so that no term loses more than a few
// ulps: the corner terms of the edge and prism regions are bounded by
// m1^2 / (m2 m3), and the slab region (m3 >= m1 + m2) is linear.
constexpr double kBoxMinM = 1e-6;
__device__ void boxFraction(double a, double m1, double m2, double m3, double& F, double& dF) {
    const bool flip = a > 0.5;
    if (flip) a = 1.0 - a;
    if (a <= 0.0) {
        F = 0.0;
        dF = 0.0;
    } else if (a < m1) {
        const double k = 1.0 / (6.0 * m1 * m2 * m3);
        F = a * a * a * k;
        dF = 3.0 * a * a * k;
    } else if (m3 >= m1 + m2 && a >= m1 + m2) {
        F = (a - 0.5 * (m1 + m2)) / m3;
        dF = 1.0 / m3;
    } else {
        const double k2 = 1.0 / (6.0 * m2 * m3);
        F = (3.0 * a * a - 3.0 * a * m1 + m1 * m1) * k2;
        dF = (6.0 * a - 3.0 * m1) * k2;
        const double k = k2 / m1;
        if (a > m2) {
            const double t = a - m2;
            F -= t * t * t * k;
            dF -= 3.0 * t * t * k;
        }
        if (a > m3) {
            const double t = a - m3;
            F -= t * t * t * k;
            dF -= 3.0 * t * t * k;
        }
    }
    if (flip) F = 1.0 - F;
}

// The plane of an axis-aligned box cell in closed form: the plane constant
// from the cube inverse, accepted on the exact box volume by the same test
// as the Newton iteration; the interface centre as calcInterfaceCentreAndArea
// (cutCell.C:37-100) forms it -- triangles from the average of the cut-edge
// points over the segments the plane leaves on the cell's faces -- in FP32
// about the box centre; the area vector = section area x unit normal,
// oriented like the reference's (towards the interface centre).  Returns
// false, for the general path, when a normal component is nearly zero, the
// section is tiny or the volume test fails.
__device__ bool boxPlane(d3 n, d3 lo, d3 hi, double alpha, double V, double& d, d3& ic, d3& is) {
    const double L[3] = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
    const double nn[3] = {n.x, n.y, n.z};
    double m[3], M = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        m[i] = fabs(nn[i]) * L[i];
        M += m[i];
    }
    if (!(M > 0.0)) return false;
    const double corner = (n.x >= 0 ? n.x * lo.x : n.x * hi.x) + (n.y >= 0 ? n.y * lo.y : n.y * hi.y) +
                          (n.z >= 0 ? n.z * lo.z : n.z * hi.z);
#pragma unroll
    for (int i = 0; i < 3; ++i) m[i] /= M;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2 - i; ++j)
            if (m[j] > m[j + 1]) {
                const double t = m[j];
                m[j] = m[j + 1];
                m[j + 1] = t;
            }
    if (m[0] < kBoxMinM) return false;
    d = cuboidPlaneConstant(n, lo, hi, alpha);
    double F, dF;
    boxFraction(-(d + corner) / M, m[0], m[1], m[2], F, dF);
    const double Vbox = L[0] * L[1] * L[2];
    const double nMag = mag(n);
    const double S = Vbox * dF / M * nMag;  // section area: dVolume / d(distance)
    const double r = F * (Vbox / V) - alpha;
    if (!(S > 1e3 * kTSMALL)) return false;
    if (!(fabs(r) <= kVolTol || fabs(r) * V <= 8.0 * 2.3e-16 * fabs(d) * S)) return false;
    // the segments on the six faces, in coordinates about the box centre
    const d3 cen = mk(0.5 * (lo.x + hi.x), 0.5 * (lo.y + hi.y), 0.5 * (lo.z + hi.z));
    const v3f h = fv(float(0.5 * L[0]), float(0.5 * L[1]), float(0.5 * L[2]));
    const v3f nf = toF(n);
    const float dl = float(dot(n, cen) + d);
    v3f P[8];
    float s[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        P[i] = fv((i & 1) ? h.x : -h.x, (i & 2) ? h.y : -h.y, (i & 4) ? h.z : -h.z);
        s[i] = dotf(nf, P[i]) + dl;
    }
    // corners of the faces x = const, y = const, z = const in cyclic order
    constexpr int kCyc[3][4] = {{0, 2, 6, 4}, {0, 1, 5, 4}, {0, 1, 3, 2}};
    v3f seg[6][2];
    int nSeg = 0;
    v3f fc = fv(0.f, 0.f, 0.f);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            int np = 0;
            v3f q[2];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int i = kCyc[ax][e] | (side << ax), j = kCyc[ax][(e + 1) & 3] | (side << ax);
                if ((s[i] < 0.f) != (s[j] < 0.f) && np < 2) {
                    q[np++] = P[i] + (s[i] / (s[i] - s[j])) * (P[j] - P[i]);
                }
            }
            if (np == 2) {
                seg[nSeg][0] = q[0];
                seg[nSeg][1] = q[1];
                fc = fc + q[0] + q[1];
                ++nSeg;
            }
        }
    if (nSeg < 3) return false;
    fc = (1.f / float(2 * nSeg)) * fc;
    float sumA = 0.f;
    v3f sumAc = fv(0.f, 0.f, 0.f);
    for (int k = 0; k < nSeg; ++k) {
        const v3f a = seg[k][0], b = seg[k][1];
        const float ar = magf(crossf(b - a, fc - a));
        sumA += ar;
        sumAc = sumAc + ar * (a + b + fc);
    }
    if (!(sumA > 0.f)) return false;
    const v3f icl = (1.f / (3.f * sumA)) * sumAc;
    ic = mk(cen.x + double(icl.x), cen.y + double(icl.y), cen.z + double(icl.z));
    is = (S / nMag) * n;
    if (dot(is, ic) < 0.0) is = (-1.0) * is;
    return true;
}

// One instantiation per cell class (workspace caps K); a launch handles the
// mixed cells of its class.
template <class K>
__global__ void __launch_bounds__(128) kPlaneSolveMixed(DevMesh m, PlaneArgs p, int cls) {
    const int nm = *p.nMixed;
    uint32_t err = 0;
    for (int i = spreadFirst(); i < nm; i += spreadStride()) {
        const int c = p.mixed[i];
        if (m.classMask != (1 << cls) && m.cellClass[c] != cls) continue;
        CellWS<K> w;
        double d = 0.0;
        d3 ic = mk(0, 0, 0), is = mk(0, 0, 0);
        int st;
        const double alphaI = p.alpha[c];
        const d3 nI = ld3(p.nrm, i);
        const unsigned bx = m.boxCorner[c];
        if (bx && alphaI > 0.0 && alphaI < 1.0) {
            const int p0 = m.cpOff[c];
            const d3 lo = ld3(m.pts, m.cPts[p0 + ((bx >> 3) & 7)]), hi = ld3(m.pts, m.cPts[p0 + (bx & 7)]);
            if (boxPlane(nI, lo, hi, alphaI, m.V[c], d, ic, is)) {
                p.mStatus[i] = 0;
                p.status[c] = 0;
                p.dOut[i] = d;
                st3(p.icOut, i, ic);
                st3(p.isOut, i, is);
                continue;
            }
        }
        if (!loadCell(m, c, w)) {
            err |= kErrSubFaceOverflow;
            st = 1;
        } else if (mag(nI) < kTSMALL) {
            st = int(sgn(0.5 - alphaI));
        } else {
            st = findSignedDistance(w, alphaI, nI, d, ic, is, err);
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
// Simpson fluxes: FP32 clipping on face-local coordinates
// ---------------------------------------------------------------------------
// Below this |distance| a vertex counts as lying above the plane by that much
// (the role of the 1e-14 lift of the FP64 form; coordinates here are O(h)).
constexpr float kLiftF = 1e-30f;

__device__ __forceinline__ float liftedF(v3f p, v3f n, float d) {
    float di = dotf(p, n) + d;
    if (fabsf(di) < kLiftF) di = (di >= 0.f) ? di + kLiftF : di - kLiftF;
    return di;
}

// |area| of the part n.x + d < 0 of the polygon fp[0..n) (fan about the
// point average, compensated sums).  The side with fewer vertices is
// clipped in FP32 and the other side follows from the FP64 area of the whole
// face, so the error is relative to the smaller part: faces that are nearly
// fully submerged or nearly empty come out nearly exact, and a cell next to
// the interface does not leave [0, 1] through FP32 rounding.
__device__ double clippedAreaF(const v3f* fp, int n, v3f nrm, float d, double fullMag) {
    float dist[kMaxFacePts];
    int nSub = 0;
    for (int i = 0; i < n; ++i) {
        dist[i] = liftedF(fp[i], nrm, d);
        nSub += dist[i] < 0.f;
    }
    if (nSub == n) return fullMag;
    if (nSub == 0) return 0.0;
    const bool keepSub = 2 * nSub <= n;
    const auto kept = [&](int i) { return (dist[i] < 0.f) == keepSub; };
    int first = 0;
    while (first < n - 1 && !kept(first)) ++first;
    v3f sp[kMaxSubPts];
    int ns = 0;
    for (int k = first; k < first + n; ++k) {
        const int cur = k % n, nxt = (k + 1) % n;
        if (kept(cur)) sp[ns++] = fp[cur];
        if ((dist[cur] < 0.f) != (dist[nxt] < 0.f)) {
            const float wgt = dist[cur] / (dist[cur] - dist[nxt]);
            sp[ns++] = fp[cur] + wgt * (fp[nxt] - fp[cur]);
        }
    }
    float part;
    if (ns < 3) {
        // fewer than three points: a submerged polygon counts as the whole
        // face (cutFace.C:243-255), an empty remainder as nothing
        return fullMag;
    } else if (ns == 3) {
        part = 0.5f * magf(crossf(sp[1] - sp[0], sp[2] - sp[0]));
    } else {
        v3f fc = sp[0];
        for (int i = 1; i < ns; ++i) fc = fc + sp[i];
        fc = (1.0f / float(ns)) * fc;
        KahanV sum;
        for (int i = 0; i < ns; ++i) {
            const v3f nx = sp[(i + 1) % ns];
            sum.add(crossf(nx - sp[i], fc - sp[i]));
        }
        part = 0.5f * magf(sum.s);
    }
    return keepSub ? double(part) : fmax(fullMag - double(part), 0.0);
}

// cutFace::timeIntegratedArea with FP32 clipping and an FP64 Simpson sum
__device__ double timeIntegratedAreaF(const v3f* fp, int n, v3f nrm, float distance, const float* pTimes,
                                      float Un0, double dt, double magSf, double fullMag, float smallTime) {
    int order[kMaxFacePts];
    for (int i = 0; i < n; ++i) {
        int j = i;
        while (j > 0 && pTimes[order[j - 1]] > pTimes[i]) {
            order[j] = order[j - 1];
            --j;
        }
        order[j] = i;
    }
    // vertex times are FP32; every interval width is taken in FP64 (the
    // difference of two floats is exact in a double) against the FP64 step,
    // so the intervals cover [0, dt] exactly and a face submerged for the
    // whole step never carries more than the full flux -- the bounding would
    // read any excess as free capacity and push more through
    const double firstTime = pTimes[order[0]];
    const double lastTime = pTimes[order[n - 1]];
    const double pos = (Un0 >= 0.f) ? 1.0 : 0.0;
    if (lastTime <= 0.0) return magSf * dt * pos;
    if (firstTime >= dt) return magSf * dt * (1.0 - pos);
    double sortedTimes[kMaxFacePts + 2];
    int nT = 0;
    double tIntArea = 0.0, subAreaOld, prevTime;
    if (firstTime > 0.0) {
        subAreaOld = magSf * (1.0 - pos);
        tIntArea = subAreaOld * firstTime;
        sortedTimes[nT++] = firstTime;
        prevTime = firstTime;
    } else {
        sortedTimes[nT++] = 0.0;
        prevTime = 0.0;
        subAreaOld = clippedAreaF(fp, n, nrm, distance, fullMag);
    }
    for (int ti = 0; ti < n; ++ti) {
        const double timeI = pTimes[order[ti]];
        if (timeI > (prevTime + double(smallTime)) && timeI < dt) {
            sortedTimes[nT++] = timeI;
            prevTime = timeI;
        }
    }
    if (lastTime > dt)
        sortedTimes[nT++] = dt;
    else
        tIntArea += magSf * (dt - lastTime) * pos;
    for (int k = 0; k + 1 < nT; ++k) {
        const double tauOld = sortedTimes[k];
        const double tauNew = sortedTimes[k + 1];
        const double deltaTau = 0.5 * (tauNew - tauOld);
        const double subAreaNew = clippedAreaF(fp, n, nrm, distance - float(tauNew) * Un0, fullMag);
        const double subAreaMid = clippedAreaF(fp, n, nrm, distance - float(tauOld + deltaTau) * Un0, fullMag);
        tIntArea += (deltaTau / 3.0) * (subAreaOld + 4.0 * subAreaMid + subAreaNew);
        subAreaOld = subAreaNew;
    }
    return tIntArea;
}

// cutFace::timeIntegratedFaceFlux (cutFace.C:262-389) on face-local
// coordinates: points and plane shifted by the face centre, clipping in
// FP32, areas of whole faces and fan triangles in FP64.
__device__ double timeIntegratedFaceFluxF(const DevMesh& m, int f, d3 nrm, double distance, double Un0, double dt,
                                          double phi, double magSf) {
    if (fabs(phi) <= kTSMALL) return 0.0;
    const int q0 = m.fOff[f], n = m.fOff[f + 1] - q0;
    const d3 cf = ld3(m.Cf, f);
    d3 pd[kMaxFacePts];
    v3f fp[kMaxFacePts];
    for (int i = 0; i < n; ++i) {
        pd[i] = ld3(m.pts, m.fPts[q0 + i]) - cf;
        fp[i] = toF(pd[i]);
    }
    const v3f nF = toF(nrm);
    const float dF = float(dot(nrm, cf) + distance);  // plane constant in face-local coordinates
    const bool flat = m.flat[f] > (1.0 - kTSMALL);
    const bool moving = fabs(Un0 * dt) > kTSMALL;
    const float un = float(Un0);
    const float smallTime = moving ? 1e-6f * sqrtf(float(magSf)) / fabsf(un) : 0.f;
    float pTimes[kMaxFacePts];
    if (moving)
        for (int i = 0; i < n; ++i) {
            const float t = (dotf(fp[i], nF) + dF) / un;
            pTimes[i] = fabsf(t) < smallTime ? 0.f : t;
        }
    if (flat) {
        const double fullMag = mag(ld3(m.fullA, f));
        if (moving)
            return phi / magSf * timeIntegratedAreaF(fp, n, nF, dF, pTimes, un, dt, magSf, fullMag, smallTime);
        return phi * dt * clippedAreaF(fp, n, nF, dF, fullMag) / magSf;
    }
    // warped face: fan of triangles about the face centre, phi split by area
    v3f tri[3];
    float tt[3];
    tri[0] = fv(0.f, 0.f, 0.f);
    tt[0] = (moving && fabsf(dF / un) >= smallTime) ? dF / un : 0.f;
    double dVf = 0.0;
    for (int pi = 0; pi < n; ++pi) {
        const int pj = (pi + 1) % n;
        tri[1] = fp[pi];
        tri[2] = fp[pj];
        const double magTri = mag(0.5 * cross(pd[pi], pd[pj]));
        if (!(magTri > 0.0)) continue;
        const double phiTri = phi * magTri / magSf;
        if (moving) {
            tt[1] = pTimes[pi];
            tt[2] = pTimes[pj];
            dVf += phiTri / magTri * timeIntegratedAreaF(tri, 3, nF, dF, tt, un, dt, magTri, magTri, smallTime);
        } else {
            dVf += phiTri * dt * clippedAreaF(tri, 3, nF, dF, magTri) / magTri;
        }
    }
    return dVf;
}

__global__ void __launch_bounds__(128) kInterfaceFacesMixed(DevMesh m, const int2* __restrict__ dwList,
                                                            const int* __restrict__ dwCount,
                                                            const double* __restrict__ nrm,
                                                            const double* __restrict__ dArr,
                                                            const double* __restrict__ un0,
                                                            const double* __restrict__ phi, double dt,
                                                            double* __restrict__ dvfI, uint8_t* __restrict__ cutMask) {
    const int n = *dwCount;
    for (int t = spreadFirst(); t < n; t += spreadStride()) {
        const int i = dwList[t].x, f = dwList[t].y;
        dvfI[f] = timeIntegratedFaceFluxF(m, f, ld3(nrm, i), dArr[i], un0[i], dt, phi[f], m.magSf[f]);
        if (cutMask) cutMask[f] = 1;
    }
}

template <class Kernel>
int residentGridM(Kernel kernel, int threads) {
    struct Entry {
        const void* fn;
        int dev, grid;
    };
    static Entry cache[8] = {};
    static std::mutex mu;
    int dev = 0;
    cudaGetDevice(&dev);
    const void* fn = reinterpret_cast<const void*>(kernel);
    std::lock_guard<std::mutex> lock(mu);
    for (auto& e : cache)
        if (e.fn == fn && e.dev == dev) return e.grid;
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
    const int g = (sms > 0 ? sms : 1) * (per > 0 ? per : 1);
    for (auto& e : cache)
        if (!e.fn) {
            e = {fn, dev, g};
            break;
        }
    return g;
}

// ---------------------------------------------------------------------------
// Interface speed of the mixed forms: the cell-point interpolation of U at
// the interface centre (the tetrahedron search of the plain form) in FP32
// about the cell centre; U enters the Simpson time positions only.
// ---------------------------------------------------------------------------
__device__ __forceinline__ v3f pointValueF(const DevMesh& m, int p, const double* U, const double* Ub) {
    const int b0 = m.pbOff[p], b1 = m.pbOff[p + 1];
    v3f r = fv(0.f, 0.f, 0.f);
    if (b1 > b0) {
        for (int k = b0; k < b1; ++k) {
            const int f = m.pbFaces[k];
            const d3 u = Ub ? ld3(Ub, f - m.nfi) : ld3(U, m.own[f]);
            r = r + float(m.pbW[k]) * toF(u);
        }
        return r;
    }
    for (int k = m.pcOff[p]; k < m.pcOff[p + 1]; ++k) r = r + float(m.pcW[k]) * toF(ld3(U, m.pCells[k]));
    return r;
}

__device__ v3f interpolateUF(const DevMesh& m, int c, d3 x, const double* U, const double* Ub) {
    const d3 a = ld3(m.C, c);
    const v3f r = toF(x - a);
    int bp0 = -1, bp1 = -1, bp2 = -1;
    float bw0 = 0.f, bw1 = 0.f, bw2 = 0.f, bw3 = 0.f, bestMin = -3.0e38f;
    bool found = false;
    for (int k = m.cOff[c]; k < m.cOff[c + 1] && !found; ++k) {
        const int f = m.cFaces[k];
        const int q0 = m.fOff[f], n = m.fOff[f + 1] - q0;
        const int g0 = m.fPts[q0];
        const v3f e1 = toF(ld3(m.pts, g0) - a);
        for (int i = 1; i + 1 < n; ++i) {
            const int gi = m.fPts[q0 + i], gj = m.fPts[q0 + i + 1];
            const v3f e2 = toF(ld3(m.pts, gi) - a), e3 = toF(ld3(m.pts, gj) - a);
            const v3f c23 = crossf(e2, e3);
            const float det = dotf(e1, c23);
            if (!(fabsf(det) > 0.f)) continue;
            const float id = 1.f / det;
            const float w1 = dotf(r, c23) * id;
            const float w2 = dotf(e1, crossf(r, e3)) * id;
            const float w3 = dotf(e1, crossf(e2, r)) * id;
            const float w0 = ((1.f - w1) - w2) - w3;
            const float mn = fminf(fminf(w0, w1), fminf(w2, w3));
            // inside up to FP32 rounding of the weights
            const bool inside = mn >= -1e-6f;
            if (mn > bestMin || inside) {
                bestMin = mn;
                bp0 = g0;
                bp1 = gi;
                bp2 = gj;
                bw0 = w0;
                bw1 = w1;
                bw2 = w2;
                bw3 = w3;
            }
            if (inside) {
                found = true;
                break;
            }
        }
    }
    if (bp0 < 0) return toF(ld3(U, c));
    v3f t = bw0 * toF(ld3(U, c));
    t = t + bw1 * pointValueF(m, bp0, U, Ub);
    t = t + bw2 * pointValueF(m, bp1, U, Ub);
    t = t + bw3 * pointValueF(m, bp2, U, Ub);
    return t;
}

// Un0 of every cut cell and the list of its downwind faces (advection.C:
// 131-174), as the plain form's kernel, with the interpolation above.
__global__ void __launch_bounds__(128) kInterfaceUn0Mixed(DevMesh m, const int* __restrict__ mixed,
                                                          const int* __restrict__ nMixed,
                                                          const int8_t* __restrict__ mStatus,
                                                          const double* __restrict__ nrm,
                                                          const double* __restrict__ icArr,
                                                          const double* __restrict__ U, const double* __restrict__ Ub,
                                                          const double* __restrict__ phi, double* __restrict__ un0,
                                                          int2* __restrict__ dwList, int* __restrict__ dwCount) {
    const int nm = *nMixed;
    const int lane = threadIdx.x & 31;
    const int stride = spreadStride();
    const int nIter = (nm + stride - 1) / stride;
    for (int it = 0; it < nIter; ++it) {
        const int i = it * stride + spreadFirst();
        int nd = 0, k0 = 0;
        unsigned down = 0;  // bit j: the cell's j-th face (cells() order) is downwind
        if (i < nm && mStatus[i] == 0) {
            const int c = mixed[i];
            const v3f u = interpolateUF(m, c, ld3(icArr, i), U, Ub);
            const d3 n = ld3(nrm, i);
            un0[i] = double(u.x) * n.x + double(u.y) * n.y + double(u.z) * n.z;
            k0 = m.cOff[c];
            down = downwindFaces(m, c, k0, m.cOff[c + 1], phi);
            nd = __popc(down);
        }
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

}  // namespace

static void planeSolveMixedAll(const DevMesh& m, const PlaneArgs& p, cudaStream_t st) {
    if (m.classMask & 1)
        kPlaneSolveMixed<CapsHex><<<residentGridM(kPlaneSolveMixed<CapsHex>, 128), 128, 0, st>>>(m, p, 0);
    if (m.classMask & 2)
        kPlaneSolveMixed<CapsPoly><<<residentGridM(kPlaneSolveMixed<CapsPoly>, 128), 128, 0, st>>>(m, p, 1);
    if (m.classMask & 4)
        kPlaneSolveMixed<CapsBig><<<residentGridM(kPlaneSolveMixed<CapsBig>, 128), 128, 0, st>>>(m, p, 2);
}

void launchLsNormalMixed(const StepArgs& a, cudaStream_t st) {
    kLsNormalMixed<<<residentGridM(kLsNormalMixed, 128), 128, 0, st>>>(a.m, a.aCur, a.mixed, a.nMixed, a.nrm, a.err);
}

void launchPlaneSolveMixed(const StepArgs& a, cudaStream_t st) {
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
    planeSolveMixedAll(a.m, p, st);
}

void launchInterfaceUn0Mixed(const StepArgs& a, cudaStream_t st) {
    kInterfaceUn0Mixed<<<residentGridM(kInterfaceUn0Mixed, 128), 128, 0, st>>>(
        a.m, a.mixed, a.nMixed, a.mStatus, a.nrm, a.icArr, a.U, a.Ub, a.phi, a.un0, a.dwList, a.dwCount);
}

void launchInterfaceFacesMixed(const StepArgs& a, cudaStream_t st) {
    kInterfaceFacesMixed<<<residentGridM(kInterfaceFacesMixed, 128), 128, 0, st>>>(
        a.m, a.dwList, a.dwCount, a.nrm, a.dArr, a.un0, a.phi, a.dt, a.dvfI, a.cutMask);
}

}  // namespace simplic
