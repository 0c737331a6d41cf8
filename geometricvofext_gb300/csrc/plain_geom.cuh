// Plain-form (FP64, bit-exact) geometry of the SimPLIC step, device side.
//
// Restates, per thread:
//   cutFace::calcSubFace / calcSubFaceCentreAndArea   cutFace.C:37-96, 136-259
//   cutFace::timeIntegratedFaceFlux / Area            cutFace.C:262-506
//   cutCell::calcSubCell and helpers                  cutCell.C:37-137, 343-542
//   cutCell::findSignedDistance                       cutCell.C:611-799
// with the same floating-point operation order as the reference, so that a
// translation unit built with -fmad=false reproduces the CPU results bit for
// bit.  Work that does not change any result is skipped (sub-cell centres
// that only feed output, face areas of fully submerged faces that depend on
// the face alone and are computed once per cell).
#pragma once

#include "simplic_device.cuh"

namespace simplic {

// v / s for the three components: one division for 1/s, then the
// correctly rounded quotients through it (divByRecip), the same results.
__device__ __forceinline__ d3 divBy(d3 v, double s) {
    const double y = 1.0 / s;
    return mk(divByRecip(v.x, s, y), divByRecip(v.y, s, y), divByRecip(v.z, s, y));
}

// OpenFOAM face::centre (triangle direct; otherwise area-weighted fan about
// the point average, centre via sumAc / (3 sumA)).
__device__ __forceinline__ d3 faceCentreOF(const d3* p, int n) {
    if (n == 3) return (1.0 / 3.0) * ((p[0] + p[1]) + p[2]);
    d3 cp = p[0];
    for (int i = 1; i < n; ++i) cp = cp + p[i];
    cp = divCount(cp, n);
    double sumA = 0.0;
    d3 sumAc = mk(0, 0, 0);
    for (int i = 0; i < n; ++i) {
        const d3 nx = p[(i + 1) % n];
        const d3 ttc = (p[i] + nx) + cp;
        const double ta = mag(cross(p[i] - cp, nx - cp));
        sumA += ta;
        sumAc = sumAc + ta * ttc;
    }
    if (sumA > kVSMALL) return sumAc / (3.0 * sumA);
    return cp;
}

// OpenFOAM face::areaNormal (sum of 0.5 (b-a)^(c-a) over (p_i, p_i+1, centre)).
__device__ __forceinline__ d3 faceAreaNormalOF(const d3* p, int n) {
    if (n == 3) return 0.5 * cross(p[1] - p[0], p[2] - p[0]);
    d3 cp = p[0];
    for (int i = 1; i < n; ++i) cp = cp + p[i];
    cp = divCount(cp, n);
    d3 nrm = mk(0, 0, 0);
    for (int i = 0; i < n; ++i) {
        const d3 nx = (i < n - 1) ? p[i + 1] : p[0];
        nrm = nrm + 0.5 * cross(nx - p[i], cp - p[i]);
    }
    return nrm;
}

// calcSubFaceCentreAndArea (cutFace.C:37-96): centre and area of a polygon.
__device__ __forceinline__ void fanCentreArea(const d3* p, int n, d3& cen, d3& area) {
    if (n == 3) {
        cen = (1.0 / 3.0) * ((p[0] + p[1]) + p[2]);
        area = 0.5 * cross(p[1] - p[0], p[2] - p[0]);
        return;
    }
    d3 fc = p[0];
    for (int i = 1; i < n; ++i) fc = fc + p[i];
    fc = divCount(fc, n);
    d3 sumN = mk(0, 0, 0), sumAc = mk(0, 0, 0);
    double sumA = 0.0;
    for (int i = 0; i < n; ++i) {
        const d3 nx = p[(i + 1) % n];
        const d3 c = (p[i] + nx) + fc;
        const d3 nv = cross(nx - p[i], fc - p[i]);
        const double a = mag(nv);
        sumN = sumN + nv;
        sumA += a;
        sumAc = sumAc + a * c;
    }
    if (sumA < kROOTVSMALL) {
        cen = fc;
        area = mk(0, 0, 0);
    } else {
        cen = divBy((1.0 / 3.0) * sumAc, sumA);
        area = 0.5 * sumN;
    }
}

// Area vector only.  sumA < ROOTVSMALL is decided without the square roots
// when any fan triangle has |n|^2 >= 1e-299 (then sumA >= 1e-150 for sure);
// otherwise sumA is summed exactly as the reference does.
__device__ __forceinline__ d3 fanArea(const d3* p, int n) {
    if (n == 3) return 0.5 * cross(p[1] - p[0], p[2] - p[0]);
    d3 fc = p[0];
    for (int i = 1; i < n; ++i) fc = fc + p[i];
    fc = divCount(fc, n);
    d3 sumN = mk(0, 0, 0);
    double s2max = 0.0;
    for (int i = 0; i < n; ++i) {
        const d3 nx = p[(i + 1) % n];
        const d3 nv = cross(nx - p[i], fc - p[i]);
        sumN = sumN + nv;
        s2max = fmax(s2max, dot(nv, nv));
    }
    if (!(s2max >= 1e-299)) {
        double sumA = 0.0;
        for (int i = 0; i < n; ++i) {
            const d3 nx = p[(i + 1) % n];
            sumA += mag(cross(nx - p[i], fc - p[i]));
        }
        if (sumA < kROOTVSMALL) return mk(0, 0, 0);
    }
    return 0.5 * sumN;
}

// The TSMALL lift of cutFace.C:159-165: |di| < TSMALL and sgn(di) (+1 for
// -0) decided on the bits; the lift adds the same +-TSMALL.
__device__ __forceinline__ double liftedDistance(d3 p, d3 n, double d) {
    double di = dot(p, n) + d;
    const long long b = bitsOf(di);
    if ((b & 0x7fffffffffffffffLL) < bitsOf(kTSMALL)) {
        const bool pos = b >= 0 || (b << 1) == 0;  // di >= 0, -0 included
        di += pos ? kTSMALL : -kTSMALL;
    }
    return di;
}
// A lifted distance is below the plane (d < 0): at least TSMALL in
// magnitude, so the sign bit decides (NaN never).
__device__ __forceinline__ bool belowBits(double x) {
    const long long b = bitsOf(x);
    return b < 0 && (b & 0x7fffffffffffffffLL) <= 0x7ff0000000000000LL && (b << 1) != 0;
}
// dc * dn < 0 for two lifted distances: the product of two numbers of at
// least TSMALL in magnitude is not zero, so it is negative exactly when the
// signs differ (NaN never).
__device__ __forceinline__ bool crossesBits(double a, double b) {
    const long long ba = bitsOf(a), bb = bitsOf(b);
    const long long kMag = 0x7fffffffffffffffLL, kInf = 0x7ff0000000000000LL;
    return (ba ^ bb) < 0 && (ba & kMag) <= kInf && (bb & kMag) <= kInf && (ba << 1) != 0 && (bb << 1) != 0;
}

// One cut face of a cell clipped against the plane (the cut branch of
// calcSubFace, cutFace.C:198-257).  P: cell points, idx: the face's local
// point indices in stored order, dist: lifted distances of the cell points,
// subMask: bit i set when dist[i] < 0.  Returns 0 with the sub-face centre /
// area and the cut points appended to edge[], or -1 when fewer than three
// points remain (then the face counts as fully submerged).
template <class K>
__device__ __forceinline__ int clipCutFace(const d3* P, const uint8_t* idx, int n, const double* dist,
                                           unsigned subMask, d3& cen, d3& area, d3* edge, int& nEdge,
                                           uint32_t& err) {
    int first = 0;
    while (first < n - 1 && !((subMask >> idx[first]) & 1u)) ++first;
    // The edges the plane cuts, by position j in the walk from `first` (edge
    // first + j).  A convex face has two: their cut points are computed
    // first, on every lane of the warp at once (cells cut their faces at
    // different positions of the walk, which would otherwise serialise the
    // divisions); further cut points (warped faces) follow in the walk.
    unsigned cutE = 0;
    for (int j = 0; j < n; ++j) {
        const int cur = (first + j) % n, nxt = (first + j + 1) % n;
        if (crossesBits(dist[idx[cur]], dist[idx[nxt]])) cutE |= 1u << j;
    }
    const auto cutPoint = [&](int j) {
        const int cur = (first + j) % n, nxt = (first + j + 1) % n;
        const double dc = dist[idx[cur]], dn = dist[idx[nxt]];
        const double w = dc / (dc - dn);
        return P[idx[cur]] + w * (P[idx[nxt]] - P[idx[cur]]);
    };
    const int j1 = cutE ? __ffs(cutE) - 1 : 0;
    const unsigned rest = cutE & (cutE - 1u);
    const int j2 = rest ? __ffs(rest) - 1 : j1;
    const d3 c1 = cutPoint(j1), c2 = cutPoint(j2);
    d3 sp[K::kSub];
    int ns = 0;
    const int e0 = nEdge;
    for (int j = 0; j < n; ++j) {
        const int cur = (first + j) % n;
        if ((subMask >> idx[cur]) & 1u) sp[ns++] = P[idx[cur]];
        if ((cutE >> j) & 1u) {
            const d3 cp = (j == j1) ? c1 : (j == j2 ? c2 : cutPoint(j));
            sp[ns++] = cp;
            if (nEdge < K::kEdge) edge[nEdge++] = cp;
            else err |= kErrEdgeOverflow;
        }
    }
    if (ns >= 3) {
        fanCentreArea(sp, ns, cen, area);
        return 0;
    }
    nEdge = e0;  // fewer than 3 points: treated as fully submerged (cutFace.C:249-255)
    return -1;
}

// Per-thread copy of one cell (points ascending by id, faces in cells()
// order as local point indices), plus the face::centre / areaNormal of each
// face, which calcSubFace returns for fully submerged faces.  Sized by the
// caps K of the cell's class.
template <class K>
struct CellWS {
    int np, nf, cell;
    double V, rV;  // volume, 1 / V
    d3 C;
    d3 P[K::kPts];
    uint8_t fsz[K::kFaces];
    uint8_t fidx[K::kFaces][K::kFacePts];
    d3 fullC[K::kFaces], fullA[K::kFaces];
};

template <class K>
__device__ __forceinline__ bool loadCell(const DevMesh& m, int c, CellWS<K>& w) {
    w.cell = c;
    w.V = m.V[c];
    w.rV = m.rV[c];
    w.C = ld3(m.C, c);
    const int p0 = m.cpOff[c], np = m.cpOff[c + 1] - p0;
    const int f0 = m.cOff[c], nf = m.cOff[c + 1] - f0;
    if (np > K::kPts || nf > K::kFaces) return false;
    w.np = np;
    w.nf = nf;
    int gid[K::kPts];
    for (int i = 0; i < np; ++i) {
        gid[i] = m.cPts[p0 + i];
        w.P[i] = ld3(m.pts, gid[i]);
    }
    for (int k = 0; k < nf; ++k) {
        const int f = m.cFaces[f0 + k];
        const int q0 = m.fOff[f], n = m.fOff[f + 1] - q0;
        if (n > K::kFacePts) return false;
        w.fsz[k] = uint8_t(n);
        for (int i = 0; i < n; ++i) {
            const int g = m.fPts[q0 + i];
            int loc = 0;
            while (loc < np - 1 && gid[loc] != g) ++loc;
            w.fidx[k][i] = uint8_t(loc);
        }
        w.fullC[k] = ld3(m.fullC, f);
        w.fullA[k] = ld3(m.fullA, f);
    }
    return true;
}

// The workspace of a cell with splitWarpedFace (getLocalPointFieldAndFaceList,
// cutCell.C:140-236): the cell points, then the centre (mesh Cf) of every
// warped face (flatness <= 1 - 1e-14) in face order; flat faces keep their
// points, warped faces become the triangles (centre, p_i, p_i+1); on the
// neighbour side every local face is reversed with its first point kept
// (face::reverseFace).  The whole-face centre and area of each local face
// (calcSubFace's result for a fully submerged face) are face::centre /
// areaNormal of the local point list.  False when the split cell exceeds
// the caps K.
template <class K>
__device__ __forceinline__ bool loadCellSplit(const DevMesh& m, int c, CellWS<K>& w) {
    w.cell = c;
    w.V = m.V[c];
    w.rV = m.rV[c];
    w.C = ld3(m.C, c);
    const int p0 = m.cpOff[c], np = m.cpOff[c + 1] - p0;
    const int f0 = m.cOff[c], nfc = m.cOff[c + 1] - f0;
    if (np > K::kPts) return false;
    int gid[K::kPts];
    for (int i = 0; i < np; ++i) {
        gid[i] = m.cPts[p0 + i];
        w.P[i] = ld3(m.pts, gid[i]);
    }
    int npl = np, nf = 0;
    for (int k = 0; k < nfc; ++k) {
        const int f = m.cFaces[f0 + k];
        const int q0 = m.fOff[f], n = m.fOff[f + 1] - q0;
        if (n > kMaxFacePts) return false;
        uint8_t loc[kMaxFacePts];
        for (int i = 0; i < n; ++i) {
            const int g = m.fPts[q0 + i];
            int l = 0;
            while (l < np - 1 && gid[l] != g) ++l;
            loc[i] = uint8_t(l);
        }
        const bool owner = m.own[f] == c;
        d3 fp[kMaxFacePts];
        if (m.flat[f] > (1.0 - kTSMALL)) {
            if (nf >= K::kFaces || n > K::kFacePts) return false;
            for (int i = 0; i < n; ++i) {
                const int src = (owner || i == 0) ? i : n - i;  // reverseFace keeps the first point
                w.fidx[nf][i] = loc[src];
                fp[i] = w.P[loc[src]];
            }
            w.fsz[nf] = uint8_t(n);
            w.fullC[nf] = faceCentreOF(fp, n);
            w.fullA[nf] = faceAreaNormalOF(fp, n);
            ++nf;
        } else {
            if (npl >= K::kPts || nf + n > K::kFaces || K::kFacePts < 3) return false;
            const int ctr = npl++;
            w.P[ctr] = ld3(m.Cf, f);
            for (int i = 0; i < n; ++i) {
                const int a = loc[i], b = loc[(i + 1) % n];
                w.fidx[nf][0] = uint8_t(ctr);
                w.fidx[nf][1] = uint8_t(owner ? a : b);
                w.fidx[nf][2] = uint8_t(owner ? b : a);
                w.fsz[nf] = 3;
                fp[0] = w.P[ctr];
                fp[1] = w.P[w.fidx[nf][1]];
                fp[2] = w.P[w.fidx[nf][2]];
                w.fullC[nf] = faceCentreOF(fp, 3);
                w.fullA[nf] = faceAreaNormalOF(fp, 3);
                ++nf;
            }
        }
    }
    w.np = npl;
    w.nf = nf;
    return true;
}

// Vertex distances -n.x of the cell points and their stable descending
// order (cutCell.C:644-670).
template <class K>
__device__ __forceinline__ void vertexOrder(const CellWS<K>& w, d3 nI, double* vd, int* order) {
    const int np = w.np;
    for (int i = 0; i < np; ++i) vd[i] = -dot(nI, w.P[i]);
    for (int i = 0; i < np; ++i) {
        int j = i;
        while (j > 0 && vd[order[j - 1]] < vd[i]) {
            order[j] = order[j - 1];
            --j;
        }
        order[j] = i;
    }
}

// The bracket the bisection over vertex levels ends with (cutCell.C:682-719):
// plane constants and VOF of the two levels that enclose alpha.
struct Bracket {
    double lowD, upD, lowA, upA;
};

// Newton on the cubic through the bracket (cutCell.C:743-789); returns the
// plane constant.
__device__ __forceinline__ double cubicDistance(const Bracket& br, double v13, double v23, double alphaI) {
    const double alphaPrismatoid = br.upA - br.lowA;
    const double a13 = v13 - br.lowA;
    const double a23 = v23 - br.lowA;
    const double a = 13.5 * a13 - 13.5 * a23 + 4.5 * alphaPrismatoid;
    const double b = -22.5 * a13 + 18.0 * a23 - 4.5 * alphaPrismatoid;
    const double c = 9.0 * a13 - 4.5 * a23 + 1.0 * alphaPrismatoid;
    const double dd = br.lowA - alphaI;
    double lambda = 0.5;
    for (int iter = 0; iter < 100; ++iter) {
        const double l2 = lambda * lambda;
        const double func = a * (lambda * l2) + b * l2 + c * lambda + dd;
        const double funcPrime = 3.0 * a * l2 + 2.0 * b * lambda + c;
        const double lambdaNew = lambda - (func / funcPrime);
        if (fabs(lambdaNew - lambda) < kTSMALL) break;
        lambda = lambdaNew;
    }
    return br.lowD - lambda * (br.lowD - br.upD);
}

struct SubCell {
    int status;
    double vof;
    d3 ic, is;  // interface centre / area vector
};

// cutCell::calcSubCell (cutCell.C:343-542) without the sub-cell centre,
// which no caller of this routine uses.
template <class K>
static __device__ __noinline__ void calcSubCell(const CellWS<K>& w, d3 n, double d, SubCell& out, uint32_t& err) {
    double dist[K::kPts];
    unsigned subMask = 0;  // bit i: cell point i lies below the plane
    for (int i = 0; i < w.np; ++i) {
        dist[i] = liftedDistance(w.P[i], n, d);
        if (belowBits(dist[i])) subMask |= 1u << i;
    }
    // face classification from the point mask (calcSubFace's counting)
    int8_t fst[K::kFaces];
    int cutK[K::kFaces], nCut = 0;
    for (int k = 0; k < w.nf; ++k) {
        int cnt = 0;
        for (int i = 0; i < w.fsz[k]; ++i) cnt += (subMask >> w.fidx[k][i]) & 1u;
        fst[k] = int8_t(cnt == w.fsz[k] ? -1 : (cnt == 0 ? 1 : 0));
        if (cnt != 0 && cnt != w.fsz[k]) cutK[nCut++] = k;
    }
    // The cut faces are clipped as a compact list: the lanes of a warp (one
    // cell each) run their j-th cut face together instead of idling on the
    // faces other cells leave uncut.  Face order is kept for the sums below.
    d3 cenK[K::kFaces], areaK[K::kFaces];
    d3 edge[K::kEdge];
    int eStartK[K::kFaces], eCntK[K::kFaces], nEdge = 0;
    for (int j = 0; j < nCut; ++j) {
        const int k = cutK[j];
        const int e0 = nEdge;
        if (clipCutFace<K>(w.P, w.fidx[k], w.fsz[k], dist, subMask, cenK[k], areaK[k], edge, nEdge, err) == 0) {
            eStartK[k] = e0;
            eCntK[k] = nEdge - e0;
        } else {
            fst[k] = -1;
        }
    }
    // the sub-cell's faces in face order: the cut faces' sub-faces (fst 0)
    // and the fully submerged faces (fst -1), then the interface
    int ncut = 0;
    bool fullySub = true, fullyEmpty = true;
    int nSubFaces = 0;
    for (int k = 0; k < w.nf; ++k) {
        if (fst[k] == 0) {
            ++ncut;
            fullySub = false;
            fullyEmpty = false;
        } else if (fst[k] == -1) {
            ++ncut;
            fullyEmpty = false;
            ++nSubFaces;
        } else {
            fullySub = false;
        }
    }
    out.ic = mk(0, 0, 0);
    out.is = mk(0, 0, 0);
    if (!fullySub && !fullyEmpty) {
        // calcInterfaceCentreAndArea (cutCell.C:37-100)
        d3 fc = mk(0, 0, 0);
        for (int i = 0; i < nEdge; ++i) fc = fc + edge[i];
        if (nEdge > 0) fc = divCount(fc, nEdge);
        d3 sumN = mk(0, 0, 0), sumAc = mk(0, 0, 0);
        double sumA = 0.0;
        for (int k = 0; k < w.nf; ++k) {
            if (fst[k] != 0) continue;
            const d3* ep = edge + eStartK[k];
            for (int i = 0; i < eCntK[k] - 1; ++i) {
                const d3 nx = ep[i + 1];
                const d3 c = (ep[i] + nx) + fc;
                const d3 nv = cross(nx - ep[i], fc - ep[i]);
                const double a = mag(nv);
                sumN = sumN + sgn(dot(nv, sumN)) * nv;
                sumA += a;
                sumAc = sumAc + a * c;
            }
        }
        d3 ic, is;
        if (sumA < kROOTVSMALL) {
            ic = fc;
            is = mk(0, 0, 0);
        } else {
            ic = divBy((1.0 / 3.0) * sumAc, sumA);
            is = 0.5 * sumN;
        }
        // the sub-cell centre is still zero at this point in the reference
        if (dot(is, ic) < 0.0) is = (-1.0) * is;
        out.ic = ic;
        out.is = is;
        if (mag(is) < kTSMALL) {
            if (nSubFaces == 0) {
                out.status = 1;
                out.vof = 0.0;
            } else {
                out.status = -1;
                out.vof = 1.0;
            }
            return;
        }
        ++ncut;  // the interface closes the sub-cell
        // calcSubCellCentreAndVolume (cutCell.C:103-137), volume only
        d3 cEst = mk(0, 0, 0);
        for (int k = 0; k < w.nf; ++k) {
            if (fst[k] == 0) cEst = cEst + cenK[k];
            else if (fst[k] == -1) cEst = cEst + w.fullC[k];
        }
        cEst = cEst + ic;
        cEst = divCount(cEst, ncut);
        double vol = 0.0;
        for (int k = 0; k < w.nf; ++k) {
            if (fst[k] == 0) vol += fmax(fabs(dot(areaK[k], cenK[k] - cEst)), kVSMALL);
            else if (fst[k] == -1) vol += fmax(fabs(dot(w.fullA[k], w.fullC[k] - cEst)), kVSMALL);
        }
        vol += fmax(fabs(dot(is, ic - cEst)), kVSMALL);
        vol /= 3.0;
        out.status = 0;
        out.vof = divByRecip(vol, w.V, w.rV);  // vol / V
    } else if (fullyEmpty) {
        out.status = 1;
        out.vof = 0.0;
    } else {
        out.status = -1;
        out.vof = 1.0;
    }
}

// cutCell::findSignedDistance (cutCell.C:611-799), splitWarpedFace = false.
// d/ic/is are written exactly where the reference writes interfaceD/C/S.
template <class K>
__device__ __forceinline__ int findSignedDistance(const CellWS<K>& w, double alphaI, d3 nI, double& dOut, d3& icOut,
                                                  d3& isOut, uint32_t& err) {
    if (mag(nI) < kTSMALL) return int(sgn(0.5 - alphaI));
    const int np = w.np;
    double vd[K::kPts];
    int order[K::kPts];
    vertexOrder(w, nI, vd, order);
    Bracket br;
    br.lowD = vd[order[0]];
    br.upD = vd[order[np - 1]];
    br.lowA = 0.0;
    br.upA = 1.0;
    int lowLabel = 0, upLabel = np - 1;
    SubCell sc;
    while ((upLabel - lowLabel) > 1) {
        const int midLabel = (upLabel + lowLabel + 1) >> 1;
        const double midDistance = vd[order[midLabel]];
        calcSubCell(w, nI, midDistance, sc, err);
        const double midAlpha = sc.vof;
        if (fabs(midAlpha - alphaI) < kTSMALL) {
            dOut = midDistance;
            icOut = sc.ic;
            isOut = sc.is;
            return sc.status;
        }
        if (midAlpha > alphaI) {
            upLabel = midLabel;
            br.upD = midDistance;
            br.upA = midAlpha;
        } else {
            lowLabel = midLabel;
            br.lowD = midDistance;
            br.lowA = midAlpha;
        }
    }
    if (fabs(br.lowD - br.upD) < kTSMALL) {
        const double midDistance = 0.5 * (br.lowD + br.upD);
        calcSubCell(w, nI, midDistance, sc, err);
        dOut = midDistance;
        icOut = sc.ic;
        isOut = sc.is;
        return sc.status;
    }
    const double deltaDistance = (br.upD - br.lowD) / 3.0;
    calcSubCell(w, nI, br.lowD + deltaDistance, sc, err);
    const double v13 = sc.vof;
    calcSubCell(w, nI, br.lowD + 2.0 * deltaDistance, sc, err);
    const double v23 = sc.vof;
    const double distance0 = cubicDistance(br, v13, v23, alphaI);
    calcSubCell(w, nI, distance0, sc, err);
    dOut = distance0;
    icOut = sc.ic;
    isOut = sc.is;
    return sc.status;
}

// |area| of a face polygon clipped by the plane (calcSubFace then
// mag(subFaceArea)); fullMag is |face::areaNormal| of the whole face.
__device__ __forceinline__ double clippedFaceArea(const d3* fp, int n, d3 nrm, double d, double fullMag) {
    double dist[kMaxFacePts];
    int nSub = 0, first = -1;
    unsigned sub = 0;
    for (int i = 0; i < n; ++i) {
        dist[i] = liftedDistance(fp[i], nrm, d);
        if (belowBits(dist[i])) {
            ++nSub;
            sub |= 1u << i;
            if (first < 0) first = i;
        }
    }
    if (nSub == n) return fullMag;
    if (nSub == 0) return 0.0;
    // the cut edges by position in the walk from `first`; the first two cut
    // points on every lane at once (see clipCutFace)
    unsigned cutE = 0;
    for (int j = 0; j < n; ++j)
        if (crossesBits(dist[(first + j) % n], dist[(first + j + 1) % n])) cutE |= 1u << j;
    const auto cutPoint = [&](int j) {
        const int cur = (first + j) % n, nxt = (first + j + 1) % n;
        const double w = dist[cur] / (dist[cur] - dist[nxt]);
        return fp[cur] + w * (fp[nxt] - fp[cur]);
    };
    const int j1 = cutE ? __ffs(cutE) - 1 : 0;
    const unsigned rest = cutE & (cutE - 1u);
    const int j2 = rest ? __ffs(rest) - 1 : j1;
    const d3 c1 = cutPoint(j1), c2 = cutPoint(j2);
    d3 sp[kMaxSubPts];
    int ns = 0;
    for (int j = 0; j < n; ++j) {
        const int cur = (first + j) % n;
        if ((sub >> cur) & 1u) sp[ns++] = fp[cur];
        if ((cutE >> j) & 1u) sp[ns++] = (j == j1) ? c1 : (j == j2 ? c2 : cutPoint(j));
    }
    if (ns < 3) return fullMag;
    return mag(fanArea(sp, ns));
}

// cutFace::timeIntegratedArea (cutFace.C:392-506)
__device__ __forceinline__ double timeIntegratedArea(const d3* fp, int n, d3 nrm, double distance,
                                                     const double* pTimes, double Un0, double dt, double magSf,
                                                     double fullMag) {
    int order[kMaxFacePts];
    for (int i = 0; i < n; ++i) {  // stable ascending sort
        int j = i;
        while (j > 0 && pTimes[order[j - 1]] > pTimes[i]) {
            order[j] = order[j - 1];
            --j;
        }
        order[j] = i;
    }
    const double firstTime = pTimes[order[0]];
    const double lastTime = pTimes[order[n - 1]];
    if (lastTime <= 0.0) return magSf * dt * pos0(Un0);
    if (firstTime >= dt) return magSf * dt * (1.0 - pos0(Un0));
    double sortedTimes[kMaxFacePts + 2];
    int nT = 0;
    double tIntArea = 0.0, prevTime, subAreaOld;
    if (firstTime > 0.0) {
        subAreaOld = magSf * (1.0 - pos0(Un0));
        tIntArea = subAreaOld * firstTime;
        sortedTimes[nT++] = firstTime;
        prevTime = firstTime;
    } else {
        sortedTimes[nT++] = 0.0;
        prevTime = 0.0;
        subAreaOld = clippedFaceArea(fp, n, nrm, distance, fullMag);
    }
    const double smallTime = fmax(kTSMALL / fabs(Un0), kTSMALL);
    for (int ti = 0; ti < n; ++ti) {
        const double timeI = pTimes[order[ti]];
        if (timeI > (prevTime + smallTime) && timeI < dt) {
            sortedTimes[nT++] = timeI;
            prevTime = timeI;
        }
    }
    if (lastTime > dt)
        sortedTimes[nT++] = dt;
    else
        tIntArea += magSf * (dt - lastTime) * pos0(Un0);
    for (int k = 0; k + 1 < nT; ++k) {
        const double tauOld = sortedTimes[k];
        const double tauNew = sortedTimes[k + 1];
        const double deltaTau = 0.5 * (tauNew - tauOld);
        const double subAreaNew = clippedFaceArea(fp, n, nrm, distance - tauNew * Un0, fullMag);
        const double subAreaMid = clippedFaceArea(fp, n, nrm, distance - (tauOld + deltaTau) * Un0, fullMag);
        tIntArea += divByRecip(deltaTau, 3.0, 1.0 / 3.0) * (subAreaOld + 4.0 * subAreaMid + subAreaNew);
        subAreaOld = subAreaNew;
    }
    return tIntArea;
}

// cutFace::timeIntegratedFaceFlux (cutFace.C:262-389)
__device__ __forceinline__ double timeIntegratedFaceFlux(const DevMesh& m, int f, d3 nrm, double distance,
                                                         double Un0, double dt, double phi, double magSf) {
    if (fabs(phi) <= kTSMALL) return 0.0;
    const int q0 = m.fOff[f], n = m.fOff[f + 1] - q0;
    d3 fp[kMaxFacePts];
    for (int i = 0; i < n; ++i) fp[i] = ld3(m.pts, m.fPts[q0 + i]);
    const bool flat = m.flat[f] > (1.0 - kTSMALL);
    if (fabs(Un0 * dt) > kTSMALL) {
        double pTimes[kMaxFacePts];
        const double rUn0 = 1.0 / Un0;  // the arrival times share the divisor
        for (int i = 0; i < n; ++i) {
            const double t = divByRecip(dot(fp[i], nrm) + distance, Un0, rUn0);
            pTimes[i] = fabs(t) < kTSMALL ? 0.0 : t;
        }
        if (flat) {
            // |face::areaNormal| of the face: the per-face table holds the same bits
            const double fullMag = mag(ld3(m.fullA, f));
            return phi / magSf * timeIntegratedArea(fp, n, nrm, distance, pTimes, Un0, dt, magSf, fullMag);
        }
        d3 tri[3];
        double tt[3];
        tri[0] = ld3(m.Cf, f);
        const double t0 = divByRecip(dot(tri[0], nrm) + distance, Un0, rUn0);
        tt[0] = fabs(t0) < kTSMALL ? 0.0 : t0;
        double dVf = 0.0;
        for (int pi = 0; pi < n; ++pi) {
            tri[1] = fp[pi];
            tt[1] = pTimes[pi];
            tri[2] = fp[(pi + 1) % n];
            tt[2] = pTimes[(pi + 1) % n];
            const d3 triA = 0.5 * cross(tri[1] - tri[0], tri[2] - tri[0]);
            const double magSfTri = mag(triA);
            const double phiTri = phi * magSfTri / magSf;
            dVf += phiTri / magSfTri * timeIntegratedArea(tri, 3, nrm, distance, tt, Un0, dt, magSfTri, magSfTri);
        }
        return dVf;
    }
    if (flat) {
        const double fullMag = mag(ld3(m.fullA, f));
        const double alphaf = clippedFaceArea(fp, n, nrm, distance, fullMag) / magSf;
        return phi * dt * alphaf;
    }
    d3 tri[3];
    tri[0] = ld3(m.Cf, f);
    double dVf = 0.0;
    for (int pi = 0; pi < n; ++pi) {
        tri[1] = fp[pi];
        tri[2] = fp[(pi + 1) % n];
        const double magSfTri = mag(0.5 * cross(tri[1] - tri[0], tri[2] - tri[0]));
        const double phiTri = phi * magSfTri / magSf;
        const double alphafTri = clippedFaceArea(tri, 3, nrm, distance, magSfTri) / magSfTri;
        dVf += phiTri * dt * alphafTri;
    }
    return dVf;
}

// The downwind faces of cell c (advection.C:131-174: phi >= 0 on an owned
// face, phi < 0 on a neighboured one; boundary faces phi >= 0) as a mask of
// its cells() slots k0 .. k1 - 1 (at most 32).
__device__ __forceinline__ unsigned downwindFaces(const DevMesh& m, int c, int k0, int k1, const double* phi) {
    unsigned down = 0;
    for (int k = k0; k < k1; ++k) {
        const int f = m.cFaces[k];
        const double ph = phi[f];
        bool dn;
        if (f < m.nfi)
            dn = (c == m.own[f]) ? (ph >= 0.0) : (ph < 0.0);
        else
            dn = ph >= 0.0;
        if (dn) down |= 1u << (k - k0);
    }
    return down;
}

// x >= 0 on the bits of x (true for -0, false for NaN)
__device__ __forceinline__ bool nonNegBits(long long b) {
    return b >= 0 ? b <= 0x7ff0000000000000LL : (b << 1) == 0;
}

// The upwind face value w (aP - aN) + aN with w = pos0(phi) (the linear
// interpolation form of OpenFOAM's upwind scheme), without the multiply:
// w = 1 gives 1 x = x exactly; w = 0 gives 0 x + aN = aN exactly when aN is
// a nonzero finite number and x is finite, and +0 when aN is +0.  For w = 1,
// (aP - aN) + aN is aP itself when aN is +0 (aP not -0), when aP is +0 (the
// sum cancels to +0), or when aP and aN share sign and binade (Sterbenz: the
// difference is exact).  Other cases (a zero or non-finite value where the
// sign of a zero decides, or aP, aN of different binades) take the
// reference's arithmetic.  The tests are integer operations on the bits.
__device__ __forceinline__ double upwindAlpha(double ph, double aP, double aN) {
    const long long bp = bitsOf(ph), bP = bitsOf(aP), bN = bitsOf(aN);
    const long long kExp = 0x7ff0000000000000LL, kSign = (long long)0x8000000000000000ULL;
    const bool finite = (bP & kExp) != kExp && (bN & kExp) != kExp;
    if (nonNegBits(bp)) {
        if (finite && ((bN == 0 && bP != kSign) || bP == 0 ||
                       (((bP ^ bN) & (kSign | kExp)) == 0 && (bP & kExp) != 0)))
            return aP;
        return (aP - aN) + aN;
    }
    if (finite && (bN << 1) != 0) return aN;
    if (finite && bN == 0) return 0.0;  // (+0 or -0) + +0
    const double w = 0.0;
    return w * (aP - aN) + aN;
}

// (phi * alpha_f) * dt: a zero carrying the signs of phi and dt when alpha_f
// is +0 (phi and dt finite), one multiply less when alpha_f is 1.  x gets the
// product phi * alpha_f when the result is that product times dt (so that
// divOfProduct can give dVf / dt), and prod says so.
__device__ __forceinline__ double fluxDt(double ph, double af, double dt, double& x, bool& prod) {
    const long long ba = bitsOf(af), bp = bitsOf(ph), bd = bitsOf(dt);
    const long long kExp = 0x7ff0000000000000LL, kSign = (long long)0x8000000000000000ULL;
    if (ba == 0 && (bp & kExp) != kExp && (bd & kExp) != kExp) {
        prod = false;
        return __longlong_as_double((bp ^ bd) & kSign);
    }
    x = (ba == 0x3ff0000000000000LL) ? ph : ph * af;
    prod = true;
    return x * dt;
}

// dVf of one face before bounding: the Simpson value when the upwind cell is
// cut, else (phi * alpha_f) * dt with alpha_f = w (aP - aN) + aN, w = pos0(phi)
// (upwind weights through the linear interpolation formula); boundary faces
// use the boundary value of alpha.  x / prod as for fluxDt (prod false for a
// Simpson value).
__device__ __forceinline__ double baseDVf(const DevMesh& m, int f, double ph, const double* aCur,
                                          const int8_t* status, const double* dvfI, const double* alphaB, double dt,
                                          double& x, bool& prod) {
    const bool pos = nonNegBits(bitsOf(ph));
    prod = false;
    if (f < m.nfi) {
        const int o = m.own[f], nb = m.nei[f];
        const int up = pos ? o : nb;
        if (status[up] == 0) return dvfI[f];
        return fluxDt(ph, upwindAlpha(ph, aCur[o], aCur[nb]), dt, x, prod);
    }
    const int o = m.own[f];
    if (pos && status[o] == 0) return dvfI[f];
    const double ab = alphaB ? alphaB[f - m.nfi] : aCur[o];
    return fluxDt(ph, ab, dt, x, prod);
}
__device__ __forceinline__ double baseDVf(const DevMesh& m, int f, double ph, const double* aCur,
                                          const int8_t* status, const double* dvfI, const double* alphaB, double dt) {
    double x;
    bool prod;
    return baseDVf(m, f, ph, aCur, status, dvfI, alphaB, dt, x, prod);
}

}  // namespace simplic
