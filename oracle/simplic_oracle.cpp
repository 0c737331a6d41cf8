// SimPLIC CPU oracle -- TEST INFRASTRUCTURE ONLY (see simplic_oracle.h).
//
// Serial FP64 restatement of the reference SimPLIC step.  Each function
// cites the reference file:line it follows (paths inside
// daidezhi/geometricVofExt).  OpenFOAM library pieces the reference calls are
// restated from their published methods; the choices are stated in place.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fopenmp -fPIC -shared

#include "simplic_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <unordered_set>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// OpenFOAM double-precision constants (doubleScalar.H)
constexpr double SMALL = 1.0e-15;
constexpr double VSMALL = 1.0e-300;
constexpr double ROOTVSMALL = 1.0e-150;
constexpr double TSMALL = 10.0 * SMALL;  // cutFace.C:154, cutCell.C:355,618

struct vec {
    double x, y, z;
};
inline vec V3(double a, double b, double c) { return vec{a, b, c}; }
inline vec operator+(vec a, vec b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec operator-(vec a, vec b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec operator*(double s, vec a) { return {s * a.x, s * a.y, s * a.z}; }
inline vec operator/(vec a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline vec& operator+=(vec& a, vec b) { a = a + b; return a; }
// OpenFOAM Vector '&' and magSqr: (x*x + y*y) + z*z, left to right
inline double dot(vec a, vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// OpenFOAM Vector '^'
inline vec cross(vec a, vec b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double mag(vec a) { return std::sqrt(dot(a, a)); }
inline double sgn(double s) { return (s >= 0.0) ? 1.0 : -1.0; }  // Foam::sign
inline double pos0(double s) { return (s >= 0.0) ? 1.0 : 0.0; }
inline double neg0(double s) { return (s <= 0.0) ? 1.0 : 0.0; }
inline vec load(const double* p, int64_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
inline void store(double* p, int64_t i, vec v) { p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z; }

// OpenFOAM face::centre (face.C): triangle -> (1/3)(a+b+c); otherwise the
// area-weighted centroid of the fan about the point average.  Used by
// cutFace::calcSubFace for fully submerged faces (cutFace.C:184,253).
vec faceCentreOF(const vec* p, int n) {
    if (n == 3) return (1.0 / 3.0) * ((p[0] + p[1]) + p[2]);
    vec cp = p[0];
    for (int i = 1; i < n; ++i) cp += p[i];
    cp = cp / double(n);
    double sumA = 0.0;
    vec sumAc = V3(0, 0, 0);
    for (int i = 0; i < n; ++i) {
        const vec nx = p[(i + 1) % n];
        const vec ttc = (p[i] + nx) + cp;
        const double ta = mag(cross(p[i] - cp, nx - cp));
        sumA += ta;
        sumAc += ta * ttc;
    }
    if (sumA > VSMALL) return sumAc / (3.0 * sumA);
    return cp;
}

// OpenFOAM face::areaNormal (face.C): sum of 0.5*(b-a)^(c-a) over the fan
// triangles (p_i, p_i+1, centre), centre last.
vec faceAreaNormalOF(const vec* p, int n) {
    if (n == 3) return 0.5 * cross(p[1] - p[0], p[2] - p[0]);
    vec cp = p[0];
    for (int i = 1; i < n; ++i) cp += p[i];
    cp = cp / double(n);
    vec nrm = V3(0, 0, 0);
    for (int i = 0; i < n; ++i) {
        const vec nx = (i < n - 1) ? p[i + 1] : p[0];
        nrm += 0.5 * cross(nx - p[i], cp - p[i]);
    }
    return nrm;
}

// Stable ascending / descending argsort (Foam::sortedOrder is a stable sort).
void stableOrder(const std::vector<double>& v, std::vector<int>& order, bool descending) {
    order.resize(v.size());
    std::iota(order.begin(), order.end(), 0);
    if (descending)
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return v[a] > v[b]; });
    else
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return v[a] < v[b]; });
}

// ---------------------------------------------------------------------------
// cutFace (src/SimPLIC/cut/cutFace/cutFace.C)
// ---------------------------------------------------------------------------
struct CutFace {
    vec subFaceCentre{0, 0, 0};
    vec subFaceArea{0, 0, 0};
    std::vector<vec> subFacePoints;
    std::vector<vec> interfacePoints;
    std::vector<double> pointDistances;
    int faceStatus = -1;

    void clearStorage() {
        subFaceCentre = V3(0, 0, 0);
        subFaceArea = V3(0, 0, 0);
        subFacePoints.clear();
        interfacePoints.clear();
        pointDistances.clear();
        faceStatus = -1;
    }

    // cutFace.C:37-96
    void calcSubFaceCentreAndArea() {
        const int n = int(subFacePoints.size());
        const vec* p = subFacePoints.data();
        if (n == 3) {
            subFaceCentre = (1.0 / 3.0) * ((p[0] + p[1]) + p[2]);
            subFaceArea = 0.5 * cross(p[1] - p[0], p[2] - p[0]);
            return;
        }
        vec sumN = V3(0, 0, 0);
        double sumA = 0.0;
        vec sumAc = V3(0, 0, 0);
        vec fc = p[0];
        for (int i = 1; i < n; ++i) fc += p[i];
        fc = fc / double(n);
        for (int i = 0; i < n; ++i) {
            const vec nx = p[(i + 1) % n];
            const vec c = (p[i] + nx) + fc;
            const vec nv = cross(nx - p[i], fc - p[i]);
            const double a = mag(nv);
            sumN += nv;
            sumA += a;
            sumAc += a * c;
        }
        if (sumA < ROOTVSMALL) {
            subFaceCentre = fc;
            subFaceArea = V3(0, 0, 0);
        } else {
            subFaceCentre = ((1.0 / 3.0) * sumAc) / sumA;
            subFaceArea = 0.5 * sumN;
        }
    }

    // cutFace.C:136-259 -- submerged side is x.n + d < 0
    int calcSubFace(const vec* fPts, int n, vec normal, double distance) {
        clearStorage();
        int nSub = 0, first = -1;
        for (int i = 0; i < n; ++i) {
            double di = dot(fPts[i], normal) + distance;
            if (std::fabs(di) < TSMALL) di += sgn(di) * TSMALL;
            pointDistances.push_back(di);
            if (di < 0.0) {
                ++nSub;
                if (first == -1) first = i;
            }
        }
        if (nSub == n) {
            faceStatus = -1;
            subFaceCentre = faceCentreOF(fPts, n);
            subFaceArea = faceAreaNormalOF(fPts, n);
            return faceStatus;
        }
        if (nSub == 0) {
            faceStatus = 1;
            subFaceCentre = V3(0, 0, 0);
            subFaceArea = V3(0, 0, 0);
            return faceStatus;
        }
        faceStatus = 0;
        for (int i = first; i < first + n; ++i) {
            const int cur = i % n;
            const int nxt = (i + 1) % n;
            if (pointDistances[cur] < 0) subFacePoints.push_back(fPts[cur]);
            if (pointDistances[cur] * pointDistances[nxt] < 0) {
                const double w = pointDistances[cur] / (pointDistances[cur] - pointDistances[nxt]);
                const vec cp = fPts[cur] + w * (fPts[nxt] - fPts[cur]);
                subFacePoints.push_back(cp);
                interfacePoints.push_back(cp);
            }
        }
        if (subFacePoints.size() >= 3) {
            faceStatus = 0;
            calcSubFaceCentreAndArea();
        } else {
            faceStatus = -1;
            subFaceCentre = faceCentreOF(fPts, n);
            subFaceArea = faceAreaNormalOF(fPts, n);
        }
        return faceStatus;
    }

    // cutFace.C:392-506
    double timeIntegratedArea(const vec* fPts, int n, vec normal, double distance,
                              const std::vector<double>& pTimes, double Un0, double dt,
                              double magSf) {
        double tIntArea = 0.0;
        std::vector<int> order;
        stableOrder(pTimes, order, false);
        const double firstTime = pTimes[order.front()];
        const double lastTime = pTimes[order.back()];
        if (lastTime <= 0.0) return magSf * dt * pos0(Un0);
        if (firstTime >= dt) return magSf * dt * (1.0 - pos0(Un0));
        std::vector<double> sortedTimes;
        double prevTime = 0.0;
        double subAreaOld = 0.0, subAreaNew = 0.0, subAreaMid = 0.0;
        if (firstTime > 0.0) {
            subAreaOld = magSf * (1.0 - pos0(Un0));
            tIntArea = subAreaOld * firstTime;
            sortedTimes.push_back(firstTime);
            prevTime = firstTime;
        } else {
            sortedTimes.push_back(0.0);
            prevTime = 0.0;
            calcSubFace(fPts, n, normal, distance);
            subAreaOld = mag(subFaceArea);
        }
        const double smallTime = std::max(TSMALL / std::fabs(Un0), TSMALL);
        for (size_t ti = 0; ti < order.size(); ++ti) {
            const double timeI = pTimes[order[ti]];
            if (timeI > (prevTime + smallTime) && timeI < dt) {
                sortedTimes.push_back(timeI);
                prevTime = timeI;
            }
        }
        if (lastTime > dt)
            sortedTimes.push_back(dt);
        else
            tIntArea += magSf * (dt - lastTime) * pos0(Un0);
        for (int k = 0; k + 1 < int(sortedTimes.size()); ++k) {
            const double tauOld = sortedTimes[k];
            const double tauNew = sortedTimes[k + 1];
            const double deltaTau = 0.5 * (tauNew - tauOld);
            calcSubFace(fPts, n, normal, distance - tauNew * Un0);
            subAreaNew = mag(subFaceArea);
            calcSubFace(fPts, n, normal, distance - (tauOld + deltaTau) * Un0);
            subAreaMid = mag(subFaceArea);
            tIntArea += (deltaTau / 3.0) * (subAreaOld + 4.0 * subAreaMid + subAreaNew);
            subAreaOld = subAreaNew;
        }
        return tIntArea;
    }
};

// ---------------------------------------------------------------------------
// Mesh with derived addressing
// ---------------------------------------------------------------------------
struct Mesh {
    int np = 0, nf = 0, nfi = 0, nc = 0;
    std::vector<vec> points, C, Cf, Sf;
    std::vector<double> V, magSf;
    std::vector<int64_t> fOff;
    std::vector<int32_t> fPts, own, nei;
    // primitiveMesh::cells(): owned faces ascending, then neighbour faces
    std::vector<int64_t> cOff;
    std::vector<int32_t> cFaces;
    // primitiveMesh::cellPoints(): ascending point ids
    std::vector<int64_t> cpOff;
    std::vector<int32_t> cPts;
    // pointCells: ascending cell ids
    std::vector<int64_t> pcOff;
    std::vector<int32_t> pCells;
    // boundary point -> boundary faces (ascending); empty for interior points
    std::vector<int64_t> pbOff;
    std::vector<int32_t> pbFaces;
    std::vector<double> flatness;

    int faceSize(int f) const { return int(fOff[f + 1] - fOff[f]); }
    void facePts(int f, std::vector<vec>& out) const {
        out.clear();
        for (int64_t k = fOff[f]; k < fOff[f + 1]; ++k) out.push_back(points[fPts[k]]);
    }
    bool isInternal(int f) const { return f < nfi; }

    void build(const oracle_mesh* m) {
        np = m->n_points; nf = m->n_faces; nfi = m->n_internal_faces; nc = m->n_cells;
        points.resize(np);
        for (int i = 0; i < np; ++i) points[i] = load(m->points, i);
        fOff.resize(nf + 1);
        for (int i = 0; i <= nf; ++i) fOff[i] = m->face_offsets[i];
        fPts.assign(m->face_points, m->face_points + fOff[nf]);
        own.assign(m->owner, m->owner + nf);
        nei.assign(m->neighbour, m->neighbour + nfi);
        C.resize(nc); V.assign(m->cell_volumes, m->cell_volumes + nc);
        for (int i = 0; i < nc; ++i) C[i] = load(m->cell_centres, i);
        Cf.resize(nf); Sf.resize(nf);
        for (int i = 0; i < nf; ++i) { Cf[i] = load(m->face_centres, i); Sf[i] = load(m->face_areas, i); }
        magSf.assign(m->face_mag_areas, m->face_mag_areas + nf);

        // cells()
        std::vector<int64_t> nOwn(nc, 0), nNei(nc, 0);
        for (int f = 0; f < nf; ++f) nOwn[own[f]]++;
        for (int f = 0; f < nfi; ++f) nNei[nei[f]]++;
        cOff.assign(nc + 1, 0);
        for (int c = 0; c < nc; ++c) cOff[c + 1] = cOff[c] + nOwn[c] + nNei[c];
        cFaces.resize(cOff[nc]);
        std::vector<int64_t> fill(nc, 0);
        for (int f = 0; f < nf; ++f) { int c = own[f]; cFaces[cOff[c] + fill[c]++] = f; }
        for (int f = 0; f < nfi; ++f) { int c = nei[f]; cFaces[cOff[c] + fill[c]++] = f; }

        // pointCells by inverting cell -> point sets; cellPoints by inverting back
        std::vector<std::vector<int32_t>> pc(np);
        for (int c = 0; c < nc; ++c) {
            std::vector<int32_t> ps;
            for (int64_t k = cOff[c]; k < cOff[c + 1]; ++k) {
                int f = cFaces[k];
                for (int64_t q = fOff[f]; q < fOff[f + 1]; ++q) ps.push_back(fPts[q]);
            }
            std::sort(ps.begin(), ps.end());
            ps.erase(std::unique(ps.begin(), ps.end()), ps.end());
            for (int p : ps) pc[p].push_back(c);  // cells visited ascending
        }
        pcOff.assign(np + 1, 0);
        for (int p = 0; p < np; ++p) pcOff[p + 1] = pcOff[p] + int64_t(pc[p].size());
        pCells.resize(pcOff[np]);
        for (int p = 0; p < np; ++p) std::copy(pc[p].begin(), pc[p].end(), pCells.begin() + pcOff[p]);
        std::vector<std::vector<int32_t>> cp(nc);
        for (int p = 0; p < np; ++p)
            for (int64_t k = pcOff[p]; k < pcOff[p + 1]; ++k) cp[pCells[k]].push_back(p);
        cpOff.assign(nc + 1, 0);
        for (int c = 0; c < nc; ++c) cpOff[c + 1] = cpOff[c] + int64_t(cp[c].size());
        cPts.resize(cpOff[nc]);
        for (int c = 0; c < nc; ++c) std::copy(cp[c].begin(), cp[c].end(), cPts.begin() + cpOff[c]);

        // boundary point -> boundary faces
        std::vector<std::vector<int32_t>> pb(np);
        for (int f = nfi; f < nf; ++f)
            for (int64_t q = fOff[f]; q < fOff[f + 1]; ++q) pb[fPts[q]].push_back(f);
        pbOff.assign(np + 1, 0);
        for (int p = 0; p < np; ++p) pbOff[p + 1] = pbOff[p] + int64_t(pb[p].size());
        pbFaces.resize(pbOff[np]);
        for (int p = 0; p < np; ++p) std::copy(pb[p].begin(), pb[p].end(), pbFaces.begin() + pbOff[p]);

        // reconstruction::updateFaceFlatness (reconstruction.C:408-440)
        flatness.assign(nf, 1.0);
        for (int f = 0; f < nf; ++f) {
            const int n = faceSize(f);
            const double magA = mag(Sf[f]);
            if (n > 3 && magA > ROOTVSMALL) {
                const vec fc = Cf[f];
                double sumA = 0.0;
                for (int i = 0; i < n; ++i) {
                    const vec th = points[fPts[fOff[f] + i]];
                    const vec nx = points[fPts[fOff[f] + (i + 1) % n]];
                    const vec nv = 0.5 * cross(nx - th, fc - th);
                    sumA += mag(nv);
                }
                flatness[f] = magA / (sumA + ROOTVSMALL);
            }
        }
    }
};

// ---------------------------------------------------------------------------
// cutCell (src/SimPLIC/cut/cutCell/cutCell.C)
// ---------------------------------------------------------------------------
struct CutCell {
    const Mesh* mesh = nullptr;
    CutFace cutFace;
    // splitWarpedFace: the cell's faces as getLocalPointFieldAndFaceList
    // builds them (cutCell.C:140-236) -- flat faces in point order, warped
    // ones (flatness <= 1 - 1e-14) as triangles about the face centre, both
    // reversed (face::reverseFace, first point kept) on the neighbour side
    // -- and the cell points followed by the centres of the warped faces
    bool useLocal = false;
    std::vector<std::vector<vec>> localFaces;
    std::vector<vec> localPoints;

    void buildLocal(int cellI) {
        const Mesh& m = *mesh;
        localFaces.clear();
        localPoints.clear();
        for (int64_t k = m.cpOff[cellI]; k < m.cpOff[cellI + 1]; ++k) localPoints.push_back(m.points[m.cPts[k]]);
        std::vector<vec> P;
        for (int64_t k = m.cOff[cellI]; k < m.cOff[cellI + 1]; ++k) {
            const int f = m.cFaces[k];
            m.facePts(f, P);
            const int n = int(P.size());
            const bool owner = m.own[f] == cellI;
            if (m.flatness[f] > (1.0 - TSMALL)) {
                std::vector<vec> lf(P);
                if (!owner) std::reverse(lf.begin() + 1, lf.end());
                localFaces.push_back(lf);
            } else {
                const vec ctr = m.Cf[f];
                localPoints.push_back(ctr);
                for (int i = 0; i < n; ++i) {
                    const vec a = P[i], b = P[(i + 1) % n];
                    localFaces.push_back(owner ? std::vector<vec>{ctr, a, b} : std::vector<vec>{ctr, b, a});
                }
            }
        }
    }
    int cellStatus = -1;
    std::vector<vec> cutFaceCentres, cutFaceAreas;
    std::vector<std::vector<vec>> interfaceEdges;
    vec subCellCentre{0, 0, 0};
    double subCellVolume = -10, VOF = -10;
    vec interfaceCentre{0, 0, 0}, interfaceArea{0, 0, 0};
    std::vector<vec> fbuf;

    void clearStorage() {
        cellStatus = -1;
        cutFaceCentres.clear();
        cutFaceAreas.clear();
        interfaceEdges.clear();
        interfaceCentre = V3(0, 0, 0);
        interfaceArea = V3(0, 0, 0);
        subCellCentre = V3(0, 0, 0);
        subCellVolume = -10;
        VOF = -10;
    }

    // The angle of (x, y): the reference takes the C library's atan2, whose
    // last bits depend on the library.  Both this oracle and the GPU path
    // use this one instead, made of correctly rounded operations only, so
    // they agree bit for bit (it is within a few ulp of atan2; the angles
    // only order the points and drop copies within 1e-8, so the last bits
    // only decide which of two copies of one edge's cut point -- the same
    // point up to rounding, reached from its two faces -- is kept).  The
    // method: reduce to t = min(|x|,|y|) / max(|x|,|y|), apply the half-angle
    // identity atan t = 2 atan(t / (1 + sqrt(1 + t^2))) three times, sum the
    // Taylor series of atan to t^19 and multiply by 8, then unfold the octant.
    static double planeAngle(double y, double x) {
        const double kPi = 3.141592653589793116, kHalfPi = 1.570796326794896558;
        if (std::isnan(x) || std::isnan(y)) return x + y;
        const double ax = std::fabs(x), ay = std::fabs(y);
        const bool steep = ay > ax;
        const double hi = steep ? ay : ax, lo = steep ? ax : ay;
        double a;
        if (hi == 0.0) {
            a = 0.0;
        } else if (std::isinf(hi)) {
            if (lo == hi) {
                a = std::signbit(x) ? kPi - 0.785398163397448279 : 0.785398163397448279;
                return std::signbit(y) ? -a : a;
            }
            a = 0.0;
        } else {
            double t = lo / hi;
            for (int k = 0; k < 3; ++k) t = t / (1.0 + std::sqrt(1.0 + t * t));
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
        if (std::signbit(x)) a = kPi - a;
        return std::signbit(y) ? -a : a;
    }

    // cutCell::interfacePoints (cutCell.C:545-608): the interface polygon of
    // the last cut, its points ordered by angle about the interface centre
    // in the interface plane (Foam::sortedOrder: a stable ascending sort;
    // the angle from planeAngle, see above),
    // points whose angle is within 1e-8 of the previous sorted one dropped.
    // The frame: zhat along the interface area, xhat towards the first edge
    // point, both normalised with OpenFOAM's Vector::normalise (zero below
    // ROOTVSMALL).
    std::vector<vec> interfacePoints() const {
        std::vector<vec> out;
        if (cellStatus != 0) return out;
        const vec zhat = interfaceArea / mag(interfaceArea);
        vec xhat = interfaceEdges[0][0] - interfaceCentre;
        xhat = xhat - dot(xhat, zhat) * zhat;
        { const double s = mag(xhat); xhat = (s < ROOTVSMALL) ? V3(0, 0, 0) : xhat / s; }
        vec yhat = cross(zhat, xhat);
        { const double s = mag(yhat); yhat = (s < ROOTVSMALL) ? V3(0, 0, 0) : yhat / s; }
        std::vector<vec> pts;
        std::vector<double> ang;
        for (const auto& e : interfaceEdges)
            for (const vec& p : e) {
                pts.push_back(p);
                ang.push_back(planeAngle(dot(p - interfaceCentre, yhat), dot(p - interfaceCentre, xhat)));
            }
        std::vector<int> order(pts.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = int(i);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ang[a] < ang[b]; });
        out.push_back(pts[order[0]]);
        for (size_t i = 1; i < order.size(); ++i)
            if (std::fabs(ang[order[i]] - ang[order[i - 1]]) > 1e-8) out.push_back(pts[order[i]]);
        return out;
    }

    // cutCell.C:37-100.  subCellCentre is still zero here (cleared at the
    // start of calcSubCell), so the orientation test uses the origin.
    void calcInterfaceCentreAndArea() {
        vec fc = V3(0, 0, 0);
        int nEdge = 0;
        for (const auto& e : interfaceEdges)
            for (const vec& p : e) { fc += p; ++nEdge; }
        if (nEdge > 0) fc = fc / double(nEdge);
        vec sumN = V3(0, 0, 0);
        double sumA = 0.0;
        vec sumAc = V3(0, 0, 0);
        for (const auto& e : interfaceEdges) {
            const int n = int(e.size());
            for (int i = 0; i < n - 1; ++i) {
                const vec nx = e[i + 1];
                const vec c = (e[i] + nx) + fc;
                const vec nv = cross(nx - e[i], fc - e[i]);
                const double a = mag(nv);
                sumN += sgn(dot(nv, sumN)) * nv;
                sumA += a;
                sumAc += a * c;
            }
        }
        if (sumA < ROOTVSMALL) {
            interfaceCentre = fc;
            interfaceArea = V3(0, 0, 0);
        } else {
            interfaceCentre = ((1.0 / 3.0) * sumAc) / sumA;
            interfaceArea = 0.5 * sumN;
        }
        if (dot(interfaceArea, interfaceCentre - subCellCentre) < 0.0)
            interfaceArea = (-1.0) * interfaceArea;
    }

    // cutCell.C:103-137
    void calcSubCellCentreAndVolume() {
        subCellCentre = V3(0, 0, 0);
        subCellVolume = 0.0;
        vec cEst = V3(0, 0, 0);
        for (const vec& c : cutFaceCentres) cEst += c;
        cEst = cEst / double(cutFaceCentres.size());
        for (size_t i = 0; i < cutFaceCentres.size(); ++i) {
            const double pyr3 = std::max(std::fabs(dot(cutFaceAreas[i], cutFaceCentres[i] - cEst)), VSMALL);
            const vec pc = 0.75 * cutFaceCentres[i] + 0.25 * cEst;
            subCellCentre += pyr3 * pc;
            subCellVolume += pyr3;
        }
        subCellCentre = subCellCentre / subCellVolume;
        subCellVolume /= 3.0;
    }

    // cutCell.C:343-542 (non-split branch :425-485)
    int calcSubCell(int cellI, vec normal, double distance) {
        clearStorage();
        const Mesh& m = *mesh;
        bool fullySubmerged = true, fullyEmpty = true;
        int nSubmergedFaces = 0;
        const int64_t nFaces = useLocal ? int64_t(localFaces.size()) : m.cOff[cellI + 1] - m.cOff[cellI];
        for (int64_t k = 0; k < nFaces; ++k) {
            if (useLocal)
                fbuf = localFaces[k];
            else
                m.facePts(m.cFaces[m.cOff[cellI] + k], fbuf);
            const int st = cutFace.calcSubFace(fbuf.data(), int(fbuf.size()), normal, distance);
            if (st == 0) {
                cutFaceCentres.push_back(cutFace.subFaceCentre);
                cutFaceAreas.push_back(cutFace.subFaceArea);
                interfaceEdges.push_back(cutFace.interfacePoints);
                fullySubmerged = false;
                fullyEmpty = false;
            } else if (st == -1) {
                cutFaceCentres.push_back(cutFace.subFaceCentre);
                cutFaceAreas.push_back(cutFace.subFaceArea);
                fullyEmpty = false;
                ++nSubmergedFaces;
            } else {
                fullySubmerged = false;
            }
        }
        if (!fullySubmerged && !fullyEmpty) {
            cellStatus = 0;
            calcInterfaceCentreAndArea();
            if (mag(interfaceArea) < TSMALL) {
                if (nSubmergedFaces == 0) {
                    cellStatus = 1;
                    subCellCentre = V3(0, 0, 0);
                    subCellVolume = 0.0;
                    VOF = 0.0;
                } else {
                    cellStatus = -1;
                    subCellCentre = m.C[cellI];
                    subCellVolume = m.V[cellI];
                    VOF = 1.0;
                }
                return cellStatus;
            }
            cutFaceCentres.push_back(interfaceCentre);
            cutFaceAreas.push_back(interfaceArea);
            calcSubCellCentreAndVolume();
            VOF = subCellVolume / m.V[cellI];
        } else if (fullyEmpty) {
            cellStatus = 1;
            subCellCentre = V3(0, 0, 0);
            subCellVolume = 0.0;
            VOF = 0.0;
        } else {
            cellStatus = -1;
            subCellCentre = m.C[cellI];
            subCellVolume = m.V[cellI];
            VOF = 1.0;
        }
        return cellStatus;
    }

    // cutCell.C:611-799.  Returns the status; writes d/centre/area through
    // the out-pointers exactly where the reference writes interfaceD/C/S.
    int findSignedDistance(int cellI, double alphaI, vec normalI, double* dOut, vec* cOut, vec* sOut,
                           bool split = false) {
        if (mag(normalI) < TSMALL) return int(sgn(0.5 - alphaI));
        if (split) buildLocal(cellI);
        useLocal = split;
        const int st = findSignedDistanceImpl(cellI, alphaI, normalI, dOut, cOut, sOut);
        useLocal = false;
        return st;
    }

    int findSignedDistanceImpl(int cellI, double alphaI, vec normalI, double* dOut, vec* cOut, vec* sOut) {
        const Mesh& m = *mesh;
        const int nPoints = useLocal ? int(localPoints.size()) : int(m.cpOff[cellI + 1] - m.cpOff[cellI]);
        std::vector<double> vd(nPoints);
        for (int i = 0; i < nPoints; ++i)
            vd[i] = -dot(normalI, useLocal ? localPoints[i] : m.points[m.cPts[m.cpOff[cellI] + i]]);
        std::vector<int> order;
        stableOrder(vd, order, true);
        double lowDistance = vd[order.front()];
        double upDistance = vd[order.back()];
        int lowLabel = 0, upLabel = nPoints - 1;
        double lowAlpha = 0.0, upAlpha = 1.0;
        while ((upLabel - lowLabel) > 1) {
            const int midLabel = (upLabel + lowLabel + 1) / 2;  // round(0.5*(up+low))
            const double midDistance = vd[order[midLabel]];
            calcSubCell(cellI, normalI, midDistance);
            const double midAlpha = VOF;
            if (std::fabs(midAlpha - alphaI) < TSMALL) {
                *dOut = midDistance; *cOut = interfaceCentre; *sOut = interfaceArea;
                return cellStatus;
            }
            if (midAlpha > alphaI) {
                upLabel = midLabel; upDistance = midDistance; upAlpha = midAlpha;
            } else {
                lowLabel = midLabel; lowDistance = midDistance; lowAlpha = midAlpha;
            }
        }
        if (std::fabs(lowDistance - upDistance) < TSMALL) {
            const double midDistance = 0.5 * (lowDistance + upDistance);
            calcSubCell(cellI, normalI, midDistance);
            *dOut = midDistance; *cOut = interfaceCentre; *sOut = interfaceArea;
            return cellStatus;
        }
        const double alphaPrismatoid = upAlpha - lowAlpha;
        const double deltaDistance = (upDistance - lowDistance) / 3.0;
        const double d13 = lowDistance + deltaDistance;
        calcSubCell(cellI, normalI, d13);
        const double a13 = VOF - lowAlpha;
        const double d23 = lowDistance + 2.0 * deltaDistance;
        calcSubCell(cellI, normalI, d23);
        const double a23 = VOF - lowAlpha;
        const double a = 13.5 * a13 - 13.5 * a23 + 4.5 * alphaPrismatoid;
        const double b = -22.5 * a13 + 18.0 * a23 - 4.5 * alphaPrismatoid;
        const double c = 9.0 * a13 - 4.5 * a23 + 1.0 * alphaPrismatoid;
        const double d = lowAlpha - alphaI;
        double lambda = 0.5;
        for (int iter = 0; iter < 100; ++iter) {
            // pow3(l) = l*sqr(l), sqr(l) = l*l
            const double func = a * (lambda * (lambda * lambda)) + b * (lambda * lambda) + c * lambda + d;
            const double funcPrime = 3.0 * a * (lambda * lambda) + 2.0 * b * lambda + c;
            const double lambdaNew = lambda - (func / funcPrime);
            if (std::fabs(lambdaNew - lambda) < TSMALL) break;
            lambda = lambdaNew;
        }
        const double distance0 = lowDistance - lambda * (lowDistance - upDistance);
        calcSubCell(cellI, normalI, distance0);
        *dOut = distance0; *cOut = interfaceCentre; *sOut = interfaceArea;
        return cellStatus;
    }
};

// Least-squares gradient of polynomial degree 1 (OpenFOAM leastSquareGrad
// "polyDegree1", reconstruction.C:89,135): fit value = a0 + g.(x - x_c) over
// the stencil with unit weights; normal equations A = sum t t^T, b = sum t v
// with t = (1, dx, dy, dz), solved by Gaussian elimination with partial
// pivoting (first maximum on ties).  A singular system returns g = 0.
vec lsGradient(const std::vector<vec>& dx, const std::vector<double>& val) {
    double A[4][4] = {{0}}, b[4] = {0};
    for (size_t s = 0; s < dx.size(); ++s) {
        const double t[4] = {1.0, dx[s].x, dx[s].y, dx[s].z};
        for (int i = 0; i < 4; ++i) {
            for (int j = 0; j < 4; ++j) A[i][j] += t[i] * t[j];
            b[i] += t[i] * val[s];
        }
    }
    for (int k = 0; k < 4; ++k) {
        int p = k;
        double best = std::fabs(A[k][k]);
        for (int i = k + 1; i < 4; ++i)
            if (std::fabs(A[i][k]) > best) { best = std::fabs(A[i][k]); p = i; }
        if (!(best > VSMALL)) return V3(0, 0, 0);
        if (p != k) {
            for (int j = 0; j < 4; ++j) std::swap(A[k][j], A[p][j]);
            std::swap(b[k], b[p]);
        }
        for (int i = k + 1; i < 4; ++i) {
            const double f = A[i][k] / A[k][k];
            for (int j = k; j < 4; ++j) A[i][j] = A[i][j] - f * A[k][j];
            b[i] = b[i] - f * b[k];
        }
    }
    double x[4];
    for (int i = 3; i >= 0; --i) {
        double s = b[i];
        for (int j = i + 1; j < 4; ++j) s = s - A[i][j] * x[j];
        x[i] = s / A[i][i];
    }
    return V3(x[1], x[2], x[3]);
}

// ---------------------------------------------------------------------------
// The solver state (reconstruction + advection)
// ---------------------------------------------------------------------------
struct Oracle {
    Mesh m;
    oracle_controls ctrl{};
    // reconstruction state
    std::vector<int32_t> mixedCells, cellStatus;
    std::vector<vec> iN, iC, iS;
    std::vector<double> iD;
    // advection state
    std::vector<double> dVf, alphaPhi;
    std::vector<uint8_t> cutFaces;
    double tRecon = 0.0, tAdv = 0.0;
    int32_t nBoundPasses = 0;
    int32_t rdfIterations = 0;  // isoRDF iterations of the last reconstruct
    mutable int32_t maxBoundCells = 0;

    int nThreads() const { return ctrl.n_threads > 1 ? ctrl.n_threads : 1; }

    // LS stencil: the cell itself, then every other cell sharing a point with
    // it in ascending order (the zone cell-point-cell stencil of
    // reconstruction.C:97-131, with a fixed order).
    void stencil(int c, std::vector<int32_t>& s) const {
        s.clear();
        for (int64_t k = m.cpOff[c]; k < m.cpOff[c + 1]; ++k) {
            const int p = m.cPts[k];
            for (int64_t q = m.pcOff[p]; q < m.pcOff[p + 1]; ++q)
                if (m.pCells[q] != c) s.push_back(m.pCells[q]);
        }
        std::sort(s.begin(), s.end());
        s.erase(std::unique(s.begin(), s.end()), s.end());
        s.insert(s.begin(), c);
    }

    // reconstruction::reconstruct (reconstruction.C:680-722) with
    // initialize (:634-677) and calcInterfaceNFromIsoAlphaGrad (:85-141)
    void reconstruct(const double* alpha) {
        const auto t0 = std::chrono::steady_clock::now();
        const int nc = m.nc;
        mixedCells.clear();
        cellStatus.clear();
        iN.assign(nc, V3(0, 0, 0));
        iD.assign(nc, 0.0);
        iC.assign(nc, V3(0, 0, 0));
        iS.assign(nc, V3(0, 0, 0));
        const double tol = ctrl.mixed_cell_tol;
        for (int c = 0; c < nc; ++c)
            if (tol < alpha[c] && alpha[c] < 1.0 - tol) {
                mixedCells.push_back(c);
                cellStatus.push_back(-100);
            }
        if (!mixedCells.empty() && ctrl.orientation == 1) {
            orientIsoRDF(alpha);
        } else if (!mixedCells.empty()) {
            const int nm = int(mixedCells.size());
#pragma omp parallel num_threads(nThreads())
            {
                std::vector<int32_t> st;
                std::vector<vec> dx;
                std::vector<double> av;
#pragma omp for schedule(dynamic, 64)
                for (int i = 0; i < nm; ++i) {
                    const int c = mixedCells[i];
                    stencil(c, st);
                    dx.clear();
                    av.clear();
                    for (int s : st) { dx.push_back(m.C[s] - m.C[c]); av.push_back(alpha[s]); }
                    const vec g = lsGradient(dx, av);
                    const vec n = (-1.0) * g;
                    iN[c] = n / (mag(n) + SMALL);
                }
            }
            // interfaceNIn /= (mag + SMALL) applies to every cell; cells that are
            // not mixed hold 0/(0+SMALL) = 0.
#pragma omp parallel num_threads(nThreads())
            {
                CutCell cc;
                cc.mesh = &m;
#pragma omp for schedule(dynamic, 16)
                for (int i = 0; i < nm; ++i) {
                    const int c = mixedCells[i];
                    double d = iD[c];
                    vec ic = iC[c], is = iS[c];
                    cellStatus[i] = cc.findSignedDistance(c, alpha[c], iN[c], &d, &ic, &is, ctrl.split_warped_face != 0);
                    iD[c] = d; iC[c] = ic; iS[c] = is;
                }
            }
        }
        tRecon += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    // OpenFOAM Vector::normalise(tol), in place: zero below tol, else each
    // component divided by the magnitude.
    static vec& normaliseInPlace(vec& v, double tol) {
        const double s = mag(v);
        if (s < tol)
            v = V3(0, 0, 0);
        else
            v = v / s;
        return v;
    }

    // LS gradient of a cell field over the stencil of cell c
    // (reconstruction::isoInterfaceGrad, reconstruction.C:144-190).
    vec stencilGradient(int c, const double* field, std::vector<int32_t>& st, std::vector<vec>& dx,
                        std::vector<double>& av) const {
        stencil(c, st);
        dx.clear();
        av.clear();
        for (int s : st) { dx.push_back(m.C[s] - m.C[c]); av.push_back(field[s]); }
        return lsGradient(dx, av);
    }

    // calcInterfaceNFromIsoRDF (reconstruction.C:193-405).  The
    // reconstructed distance function is OpenFOAM v2312's
    // reconstructedDistanceFunction (transportModels/geometricVoF, linked in
    // by src/Allwmake:17-19; absent here), restated from its published
    // method (Scheufler & Roenby, J. Comput. Phys. 383 (2019) 1-23):
    //  * band = the mixed cells and every cell sharing a point with one
    //    (markCellsNearSurf with one ring);
    //  * a mixed cell with a nonzero normal n: RDF = (C_int - C) . n/|n|;
    //  * another band cell: the mean over its stencil cells j with a plane,
    //    RDF = sum_j w_j d_j / sum_j w_j, d_j = (C_int,j - C) . n_j,
    //    w_j = ((C_int,j - C)/|C_int,j - C| . n_j)^2 (1 where C_int,j = C),
    //    kept from the previous iteration when no stencil cell has a plane;
    //  * the RDF starts at zero every reconstruct; contact-angle corrections
    //    of the boundary (updateContactAngle) do nothing on walls without a
    //    contact-angle condition, the only walls here.
    // The residual sums run over the mixed cells in ascending cell order.
    void orientIsoRDF(const double* alpha) {
        const int nc = m.nc, nm = int(mixedCells.size());
        const double TSMALL = 10.0 * SMALL;
        std::vector<vec> grad(nm);
        std::vector<uint8_t> band(nc, 0);
        for (int i = 0; i < nm; ++i) {
            std::vector<int32_t> st;
            stencil(mixedCells[i], st);
            for (int x : st) band[x] = 1;
        }
        std::vector<int32_t> bandCells;
        for (int c = 0; c < nc; ++c)
            if (band[c]) bandCells.push_back(c);
#pragma omp parallel num_threads(nThreads())
        {
            std::vector<int32_t> st;
            std::vector<vec> dx;
            std::vector<double> av;
#pragma omp for schedule(dynamic, 64)
            for (int i = 0; i < nm; ++i) grad[i] = stencilGradient(mixedCells[i], alpha, st, dx, av);
        }
        std::vector<double> rdf(nc, 0.0);
        std::vector<uint8_t> tooCoarse(nm, 0);
        std::vector<double> res(nm), avgA(nm);
        const int iterations = ctrl.rdf_iterations;
        for (int iter = 0; iter < iterations; ++iter) {
            for (int i = 0; i < nm; ++i) iN[mixedCells[i]] = (-1.0) * normaliseInPlace(grad[i], SMALL);
#pragma omp parallel num_threads(nThreads())
            {
                CutCell cc;
                cc.mesh = &m;
#pragma omp for schedule(dynamic, 16)
                for (int i = 0; i < nm; ++i) {
                    if (tooCoarse[i]) continue;
                    const int c = mixedCells[i];
                    double d = iD[c];
                    vec ic = iC[c], is = iS[c];
                    cellStatus[i] = cc.findSignedDistance(c, alpha[c], iN[c], &d, &ic, &is, ctrl.split_warped_face != 0);
                    iD[c] = d; iC[c] = ic; iS[c] = is;
                }
            }
            // the distance function on the band (normals -interfaceN passed,
            // negated again inside)
            const int nb = int(bandCells.size());
#pragma omp parallel num_threads(nThreads())
            {
                std::vector<int32_t> st;
#pragma omp for schedule(dynamic, 256)
                for (int q = 0; q < nb; ++q) {
                    const int c = bandCells[q];
                    const vec normalC = (-1.0) * iN[c];
                    if (mag(normalC) != 0.0) {
                        const vec n = (-1.0) * normalC / mag(normalC);
                        rdf[c] = dot(iC[c] - m.C[c], n);
                        continue;
                    }
                    double averageDist = 0.0, avgWeight = 0.0;
                    const vec p = m.C[c];
                    stencil(c, st);
                    for (int g : st) {
                        vec n = (-1.0) * ((-1.0) * iN[g]);
                        if (mag(n) != 0.0) {
                            n = n / mag(n);
                            vec toSeg = iC[g] - p;
                            const double distToSurf = dot(toSeg, n);
                            double weight;
                            if (mag(toSeg) != 0.0) {
                                toSeg = toSeg / mag(toSeg);
                                const double w = std::fabs(dot(toSeg, n));
                                weight = w * w;
                            } else {
                                weight = 1.0;
                            }
                            averageDist += distToSurf * weight;
                            avgWeight += weight;
                        }
                    }
                    if (avgWeight != 0.0) rdf[c] = averageDist / avgWeight;
                }
            }
#pragma omp parallel num_threads(nThreads())
            {
                std::vector<int32_t> st;
                std::vector<vec> dx;
                std::vector<double> av;
#pragma omp for schedule(dynamic, 64)
                for (int i = 0; i < nm; ++i) {
                    const int c = mixedCells[i];
                    grad[i] = stencilGradient(c, rdf.data(), st, dx, av);
                    // the reference's zero-normal test normalises the new
                    // gradient in place when the cell's normal is not zero
                    if (!(mag(iN[c]) < TSMALL)) normaliseInPlace(grad[i], SMALL);
                    double avgDiff = 0.0, weight = 0.0;
                    const vec cellNormal = iN[c];
                    for (size_t j = 0; j < st.size(); ++j) {
                        const vec normal = iN[st[j]];
                        if (mag(normal) >= TSMALL && j != 0) {
                            const vec n = normal / mag(normal);
                            const double cosAngle = std::max(std::min(dot(cellNormal, n), 1.0), -1.0);
                            avgDiff += std::acos(cosAngle) * mag(normal);
                            weight += mag(normal);
                        }
                    }
                    avgDiff = (weight != 0.0) ? avgDiff / weight : 0.0;
                    const vec newCellNormal = (-1.0) * normaliseInPlace(grad[i], SMALL);
                    res[i] = 1.0 - dot(cellNormal, newCellNormal);
                    avgA[i] = avgDiff;
                }
            }
            int resCounter = 0;
            double avgRes = 0.0, avgNormRes = 0.0;
            for (int i = 0; i < nm; ++i) {
                if (avgA[i] > 0.26 && iter > 0) {
                    tooCoarse[i] = 1;
                } else {
                    avgRes += res[i];
                    const double discreteError = 0.01 * (avgA[i] * avgA[i]);
                    const double normRes = discreteError != 0.0 ? res[i] / std::max(discreteError, ctrl.rdf_tol)
                                                                : res[i] / ctrl.rdf_tol;
                    avgNormRes += normRes;
                    ++resCounter;
                }
            }
            if (resCounter == 0) {
                resCounter = 1;
                avgRes = 0.0;
                avgNormRes = 0.0;
            }
            rdfIterations = iter + 1;
            if (((avgNormRes / resCounter < ctrl.rdf_rel_tol || avgRes / resCounter < ctrl.rdf_tol) && iter >= 1) ||
                iter + 1 == iterations)
                break;
        }
    }

    // Cell-point interpolation of U at x inside cell c (OpenFOAM
    // interpolationCellPoint, advection.C:91,126), restated:
    //  * point value = inverse-distance weighted cell values (weights
    //    1/|p - C|, normalised by their sum, accumulated in ascending cell
    //    order); a point on the boundary uses the boundary face values with
    //    weights 1/|p - Cf| instead;
    //  * the cell is split into tets (cell centre, f[0], f[i], f[i+1]) over its
    //    faces in cells() order; the first tet whose barycentric weights are
    //    all >= -1e-10 is used, else the one with the largest minimum weight;
    //  * U(x) = w0 U_c + w1 U_f0 + w2 U_fi + w3 U_fi+1, summed in that order.
    vec pointValue(int p, const double* U, const double* Ub) const {
        const vec P = m.points[p];
        const int64_t b0 = m.pbOff[p], b1 = m.pbOff[p + 1];
        std::vector<double> w;
        double sumW = 0.0;
        if (b1 > b0) {
            for (int64_t k = b0; k < b1; ++k) {
                const double wi = 1.0 / mag(P - m.Cf[m.pbFaces[k]]);
                w.push_back(wi);
                sumW += wi;
            }
            vec r = V3(0, 0, 0);
            for (int64_t k = b0; k < b1; ++k) {
                const int f = m.pbFaces[k];
                const vec u = Ub ? load(Ub, f - m.nfi) : load(U, m.own[f]);
                r += (w[k - b0] / sumW) * u;
            }
            return r;
        }
        for (int64_t k = m.pcOff[p]; k < m.pcOff[p + 1]; ++k) {
            const double wi = 1.0 / mag(P - m.C[m.pCells[k]]);
            w.push_back(wi);
            sumW += wi;
        }
        vec r = V3(0, 0, 0);
        for (int64_t k = m.pcOff[p]; k < m.pcOff[p + 1]; ++k)
            r += (w[k - m.pcOff[p]] / sumW) * load(U, m.pCells[k]);
        return r;
    }

    vec interpolateU(int c, vec x, const double* U, const double* Ub) const {
        const vec a = m.C[c];
        const vec r = x - a;
        int bestP[3] = {-1, -1, -1};
        double bestW[4] = {0, 0, 0, 0};
        double bestMin = -1e300;
        bool found = false;
        for (int64_t k = m.cOff[c]; k < m.cOff[c + 1] && !found; ++k) {
            const int f = m.cFaces[k];
            const int n = m.faceSize(f);
            const int q0 = m.fPts[m.fOff[f]];
            for (int i = 1; i + 1 < n; ++i) {
                const int qi = m.fPts[m.fOff[f] + i];
                const int qj = m.fPts[m.fOff[f] + i + 1];
                const vec e1 = m.points[q0] - a, e2 = m.points[qi] - a, e3 = m.points[qj] - a;
                const double det = dot(e1, cross(e2, e3));
                if (!(std::fabs(det) > VSMALL)) continue;
                const double w1 = dot(r, cross(e2, e3)) / det;
                const double w2 = dot(e1, cross(r, e3)) / det;
                const double w3 = dot(e1, cross(e2, r)) / det;
                const double w0 = ((1.0 - w1) - w2) - w3;
                const double mn = std::min(std::min(w0, w1), std::min(w2, w3));
                if (mn > bestMin || mn >= -1e-10) {
                    bestMin = mn;
                    bestP[0] = q0; bestP[1] = qi; bestP[2] = qj;
                    bestW[0] = w0; bestW[1] = w1; bestW[2] = w2; bestW[3] = w3;
                }
                if (mn >= -1e-10) { found = true; break; }
            }
        }
        if (bestP[0] < 0) return load(U, c);
        vec t = bestW[0] * load(U, c);
        t += bestW[1] * pointValue(bestP[0], U, Ub);
        t += bestW[2] * pointValue(bestP[1], U, Ub);
        t += bestW[3] * pointValue(bestP[2], U, Ub);
        return t;
    }

    // cutFace::timeIntegratedFaceFlux (cutFace.C:262-389)
    double timeIntegratedFaceFlux(CutFace& cf, int faceI, vec normal, double distance, double Un0,
                                  double dt, double phi, double magSf) const {
        if (std::fabs(phi) <= TSMALL) return 0.0;
        std::vector<vec> fPts;
        m.facePts(faceI, fPts);
        const int nPoints = int(fPts.size());
        if (std::fabs(Un0 * dt) > TSMALL) {
            std::vector<double> pTimes(nPoints);
            for (int i = 0; i < nPoints; ++i) {
                const double t = (dot(fPts[i], normal) + distance) / Un0;
                pTimes[i] = std::fabs(t) < TSMALL ? 0.0 : t;
            }
            double dVfv = 0.0;
            if (m.flatness[faceI] > (1.0 - TSMALL)) {
                dVfv = phi / magSf * cf.timeIntegratedArea(fPts.data(), nPoints, normal, distance, pTimes, Un0, dt, magSf);
            } else {
                vec tri[3];
                std::vector<double> tt(3);
                tri[0] = m.Cf[faceI];
                const double t0 = (dot(tri[0], normal) + distance) / Un0;
                tt[0] = std::fabs(t0) < TSMALL ? 0.0 : t0;
                for (int pi = 0; pi < nPoints; ++pi) {
                    tri[1] = fPts[pi];
                    tt[1] = pTimes[pi];
                    tri[2] = fPts[(pi + 1) % nPoints];
                    tt[2] = pTimes[(pi + 1) % nPoints];
                    const double magSfTri = mag(0.5 * cross(tri[1] - tri[0], tri[2] - tri[0]));
                    const double phiTri = phi * magSfTri / magSf;
                    dVfv += phiTri / magSfTri * cf.timeIntegratedArea(tri, 3, normal, distance, tt, Un0, dt, magSfTri);
                }
            }
            return dVfv;
        }
        if (m.flatness[faceI] > (1.0 - TSMALL)) {
            cf.calcSubFace(fPts.data(), nPoints, normal, distance);
            const double alphaf = mag(cf.subFaceArea) / magSf;
            return phi * dt * alphaf;
        }
        vec tri[3];
        tri[0] = m.Cf[faceI];
        double dVfv = 0.0;
        for (int pi = 0; pi < nPoints; ++pi) {
            tri[1] = fPts[pi];
            tri[2] = fPts[(pi + 1) % nPoints];
            const double magSfTri = mag(0.5 * cross(tri[1] - tri[0], tri[2] - tri[0]));
            const double phiTri = phi * magSfTri / magSf;
            cf.calcSubFace(tri, 3, normal, distance);
            const double alphafTri = mag(cf.subFaceArea) / magSfTri;
            dVfv += phiTri * dt * alphafTri;
        }
        return dVfv;
    }

    // advection::timeIntegratedFlux (advection.C:85-221)
    void timeIntegratedFlux(const double* phi, const double* U, const double* Ub, double dt) {
        const int nm = int(mixedCells.size());
#pragma omp parallel num_threads(nThreads())
        {
            CutFace cf;
#pragma omp for schedule(dynamic, 16)
            for (int i = 0; i < nm; ++i) {
                if (cellStatus[i] != 0) continue;
                const int c = mixedCells[i];
                const vec n = iN[c];
                const double d = iD[c];
                const double Un0 = dot(interpolateU(c, iC[c], U, Ub), n);
                for (int64_t k = m.cOff[c]; k < m.cOff[c + 1]; ++k) {
                    const int f = m.cFaces[k];
                    bool down;
                    if (m.isInternal(f))
                        down = (c == m.own[f]) ? (phi[f] >= 0.0) : (phi[f] < 0.0);
                    else
                        down = phi[f] >= 0.0;  // boundary: owner only (:197)
                    if (!down) continue;
                    dVf[f] = timeIntegratedFaceFlux(cf, f, n, d, Un0, dt, phi[f], m.magSf[f]);
                    cutFaces[f] = 1;
                }
            }
        }
    }

    // advection::netFlux (advection.C:259-288)
    double netFlux(int c, const std::vector<double>& F) const {
        double dV = 0.0;
        for (int64_t k = m.cOff[c]; k < m.cOff[c + 1]; ++k) {
            const int f = m.cFaces[k];
            if (m.own[f] == c) dV += F[f];
            else dV -= F[f];
        }
        return dV;
    }

    // advection::boundFlux (advectionTemplates.C:218-349)
    void boundFlux(const std::vector<int32_t>& nextToInterface, const double* alpha,
                   const double* alphaOld, std::vector<double>& corr, std::vector<int32_t>& corrected,
                   const double* phi, double dt, const double* Sp, const double* Su) const {
        const double aTol = 100.0 * SMALL;
        const double rDeltaT = 1.0 / dt;
        corrected.clear();
        std::vector<int32_t> downwind, pass;
        std::vector<double> dVfmax, phis;
        int32_t nCells = 0;
        for (const int c : nextToInterface) {
            if (!(alpha[c] < -aTol || alpha[c] > 1.0 + aTol)) continue;
            ++nCells;
            if (nCells > maxBoundCells) maxBoundCells = nCells;
            const double Vi = m.V[c];
            double alphaOvershoot = pos0(alpha[c] - 1.0) * (alpha[c] - 1.0) + neg0(alpha[c]) * alpha[c];
            double fluidToPassOn = alphaOvershoot * Vi;
            int nFacesToPass = 1;
            bool firstLoop = true;
            for (int iter = 0; iter < 10; ++iter) {
                if (std::fabs(alphaOvershoot) < aTol || nFacesToPass == 0) break;
                pass.clear(); dVfmax.clear(); phis.clear();
                // setDownwindFaces (advection.C:224-256)
                downwind.clear();
                for (int64_t k = m.cOff[c]; k < m.cOff[c + 1]; ++k) {
                    const int f = m.cFaces[k];
                    const double ph = phi[f];
                    if (m.own[f] == c) { if (ph >= 0) downwind.push_back(f); }
                    else if (ph < 0) downwind.push_back(f);
                }
                double dVftot = 0.0;
                nFacesToPass = 0;
                for (const int f : downwind) {
                    const double phif = phi[f];
                    const double dVff = dVf[f] + corr[f];
                    const double maxExtra = std::fabs(pos0(fluidToPassOn) * phif * dt - dVff);
                    if (maxExtra / Vi > aTol) {
                        pass.push_back(f);
                        phis.push_back(phif);
                        dVfmax.push_back(maxExtra);
                        dVftot += std::fabs(phif * dt);
                    }
                }
                for (size_t fi = 0; fi < pass.size(); ++fi) {
                    const int f = pass[fi];
                    double through = std::fabs(fluidToPassOn) * std::fabs(phis[fi] * dt) / dVftot;
                    nFacesToPass += int(pos0(dVfmax[fi] - through));
                    through = std::min(through, dVfmax[fi]);
                    double dVff = corr[f];
                    dVff += sgn(phis[fi]) * sgn(fluidToPassOn) * through;
                    corr[f] = dVff;
                    if (firstLoop) corrected.push_back(f);
                }
                firstLoop = false;
                double num = alphaOld[c] * rDeltaT;
                if (Su) num = num + Su[c];
                num = num - netFlux(c, dVf) / Vi * rDeltaT;
                num = num - netFlux(c, corr) / Vi * rDeltaT;
                const double den = Sp ? (rDeltaT - Sp[c]) : rDeltaT;
                const double alpha1New = num / den;
                alphaOvershoot = pos0(alpha1New - 1.0) * (alpha1New - 1.0) + neg0(alpha1New) * alpha1New;
                fluidToPassOn = alphaOvershoot * Vi;
            }
        }
    }

    // advection::advect (advectionTemplates.C:352-418)
    void advect(double* alpha, const double* alphaOldIn, const double* phi, const double* U,
                const double* Ub, const double* alphaB, double dt, const double* Sp, const double* Su) {
        const auto t0 = std::chrono::steady_clock::now();
        const int nc = m.nc, nf = m.nf, nfi = m.nfi;
        std::vector<double> oldCopy;
        const double* alphaOld = alphaOldIn;
        if (!alphaOld) { oldCopy.assign(alpha, alpha + nc); alphaOld = oldCopy.data(); }
        const double rDeltaT = 1.0 / dt;
        // upwind flux: phi * (w*(aP - aN) + aN) * dt, w = pos0(phi)
        // (surfaceInterpolationScheme::interpolate with upwind weights);
        // boundary faces use the boundary value of alpha.
        dVf.assign(nf, 0.0);
        cutFaces.assign(nf, 0);
        for (int f = 0; f < nfi; ++f) {
            const double w = pos0(phi[f]);
            const double af = w * (alpha[m.own[f]] - alpha[m.nei[f]]) + alpha[m.nei[f]];
            dVf[f] = phi[f] * af * dt;
        }
        for (int f = nfi; f < nf; ++f) {
            const double ab = alphaB ? alphaB[f - nfi] : alpha[m.own[f]];
            dVf[f] = phi[f] * ab * dt;
        }
        timeIntegratedFlux(phi, U, Ub, dt);
        // fvc::surfaceIntegrate: owner += / neighbour -= over internal faces in
        // face order, boundary faces after, then divide by V
        std::vector<double> ivf(nc, 0.0);
        if (nThreads() == 1) {
            for (int f = 0; f < nfi; ++f) { ivf[m.own[f]] += dVf[f]; ivf[m.nei[f]] -= dVf[f]; }
            for (int f = nfi; f < nf; ++f) ivf[m.own[f]] += dVf[f];
        } else {
            // the same per-cell order: every cell's faces in ascending face id
#pragma omp parallel num_threads(nThreads())
            {
                std::vector<int32_t> fs;
#pragma omp for schedule(static)
                for (int c = 0; c < nc; ++c) {
                    fs.assign(m.cFaces.begin() + m.cOff[c], m.cFaces.begin() + m.cOff[c + 1]);
                    std::sort(fs.begin(), fs.end());
                    double s = 0.0;
                    for (int f : fs) { if (m.own[f] == c) s += dVf[f]; else s -= dVf[f]; }
                    ivf[c] = s;
                }
            }
        }
        for (int c = 0; c < nc; ++c) {
            ivf[c] = ivf[c] / m.V[c];
            double num = alphaOld[c] * rDeltaT;
            if (Su) num = num + Su[c];
            num = num - ivf[c] * rDeltaT;
            const double den = Sp ? (rDeltaT - Sp[c]) : rDeltaT;
            alpha[c] = num / den;
        }
        limitFlux(alpha, alphaOld, phi, dt, Sp, Su);
        applyBruteForceBounding(alpha);
        alphaPhi.resize(nf);
        for (int f = 0; f < nf; ++f) alphaPhi[f] = dVf[f] / dt;
        tAdv += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    // advection::limitFlux (advectionTemplates.C:118-215) with
    // extendMarkedCells (advection.C:54-82)
    void limitFlux(double* alpha, const double* alphaOld, const double* phi, double dt,
                   const double* Sp, const double* Su) {
        const double aTol = 100.0 * SMALL;
        const int nc = m.nc;
        double mx = alpha[0], mn = alpha[0];
        for (int c = 1; c < nc; ++c) { mx = std::max(mx, alpha[c]); mn = std::min(mn, alpha[c]); }
        double maxAlphaMinus1 = mx - 1.0, minAlpha = mn;
        std::vector<double> corr(m.nf, 0.0);
        std::vector<uint8_t> mark(nc, 0), fmark(m.nf, 0);
        for (int c : mixedCells) mark[c] = 1;
        for (int c = 0; c < nc; ++c)
            if (mark[c])
                for (int64_t k = m.cOff[c]; k < m.cOff[c + 1]; ++k) fmark[m.cFaces[k]] = 1;
        for (int f = 0; f < m.nfi; ++f)
            if (fmark[f]) { mark[m.own[f]] = 1; mark[m.nei[f]] = 1; }
        for (int f = m.nfi; f < m.nf; ++f)
            if (fmark[f]) mark[m.own[f]] = 1;
        std::vector<int32_t> need;
        for (int c = 0; c < nc; ++c) if (mark[c]) need.push_back(c);
        std::vector<int32_t> corrected;
        for (int n = 0; n < ctrl.n_alpha_bounds; ++n) {
            if (maxAlphaMinus1 > aTol || minAlpha < -aTol) {
                ++nBoundPasses;
                std::fill(corr.begin(), corr.end(), 0.0);
                boundFlux(need, alpha, alphaOld, corr, corrected, phi, dt, Sp, Su);
                std::unordered_set<int32_t> done;
                for (const int f : corrected) {
                    if (!done.insert(f).second) continue;
                    const int o = m.own[f];
                    alpha[o] -= corr[f] / m.V[o];
                    if (m.isInternal(f)) {
                        const int nb = m.nei[f];
                        alpha[nb] += corr[f] / m.V[nb];
                    }
                    dVf[f] = dVf[f] + corr[f];
                }
            } else {
                break;
            }
            mx = alpha[0]; mn = alpha[0];
            for (int c = 1; c < nc; ++c) { mx = std::max(mx, alpha[c]); mn = std::min(mn, alpha[c]); }
            maxAlphaMinus1 = mx - 1.0;
            minAlpha = mn;
        }
    }

    // advection::applyBruteForceBounding (advection.C:291-308)
    void applyBruteForceBounding(double* alpha) const {
        const double snap = ctrl.snap_tol;
        if (snap > 0.0)
            for (int c = 0; c < m.nc; ++c)
                alpha[c] = alpha[c] * pos0(alpha[c] - snap) * neg0(alpha[c] - (1.0 - snap)) + pos0(alpha[c] - (1.0 - snap));
        if (ctrl.clip)
            for (int c = 0; c < m.nc; ++c) alpha[c] = std::min(1.0, std::max(0.0, alpha[c]));
    }
};

}  // namespace

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
extern "C" {

double oracle_plane_angle(double y, double x) { return CutCell::planeAngle(y, x); }

void* oracle_create(const oracle_mesh* mesh, const oracle_controls* ctrl) {
    Oracle* o = new Oracle();
    o->ctrl = *ctrl;
    o->m.build(mesh);
    return o;
}

void oracle_destroy(void* h) { delete static_cast<Oracle*>(h); }

int oracle_reconstruct(void* h, const double* alpha) {
    static_cast<Oracle*>(h)->reconstruct(alpha);
    return 0;
}

int oracle_advect(void* h, double* alpha, const double* alpha_old, const double* phi, const double* U,
                  const double* U_boundary, const double* alpha_boundary, double dt, const double* Sp,
                  const double* Su) {
    static_cast<Oracle*>(h)->advect(alpha, alpha_old, phi, U, U_boundary, alpha_boundary, dt, Sp, Su);
    return 0;
}

int32_t oracle_n_mixed(void* h) { return int32_t(static_cast<Oracle*>(h)->mixedCells.size()); }

void oracle_get_mixed(void* h, int32_t* cells, int32_t* status) {
    Oracle* o = static_cast<Oracle*>(h);
    std::copy(o->mixedCells.begin(), o->mixedCells.end(), cells);
    std::copy(o->cellStatus.begin(), o->cellStatus.end(), status);
}

void oracle_get_interface(void* h, double* n, double* d, double* c, double* s) {
    Oracle* o = static_cast<Oracle*>(h);
    for (int i = 0; i < o->m.nc; ++i) {
        store(n, i, o->iN[i]);
        d[i] = o->iD[i];
        store(c, i, o->iC[i]);
        store(s, i, o->iS[i]);
    }
}

void oracle_get_alpha_phi(void* h, double* ap) {
    Oracle* o = static_cast<Oracle*>(h);
    std::copy(o->alphaPhi.begin(), o->alphaPhi.end(), ap);
}

void oracle_get_dvf(void* h, double* dvf) {
    Oracle* o = static_cast<Oracle*>(h);
    std::copy(o->dVf.begin(), o->dVf.end(), dvf);
}

void oracle_get_face_flatness(void* h, double* flat) {
    Oracle* o = static_cast<Oracle*>(h);
    std::copy(o->m.flatness.begin(), o->m.flatness.end(), flat);
}

void oracle_get_cut_faces(void* h, uint8_t* mask) {
    Oracle* o = static_cast<Oracle*>(h);
    std::copy(o->cutFaces.begin(), o->cutFaces.end(), mask);
}

int32_t oracle_rdf_iterations(void* h) { return static_cast<Oracle*>(h)->rdfIterations; }

void oracle_get_stats(void* h, double* times2, int32_t* n_bound) {
    Oracle* o = static_cast<Oracle*>(h);
    times2[0] = o->tRecon;
    times2[1] = o->tAdv;
    n_bound[0] = o->nBoundPasses;
    n_bound[1] = o->maxBoundCells;
}

int oracle_calc_sub_face(const double* pts, int32_t n, const double* normal, double distance,
                         double* centre, double* area) {
    CutFace cf;
    std::vector<vec> p(n);
    for (int i = 0; i < n; ++i) p[i] = load(pts, i);
    const int st = cf.calcSubFace(p.data(), n, load(normal, 0), distance);
    store(centre, 0, cf.subFaceCentre);
    store(area, 0, cf.subFaceArea);
    return st;
}

int oracle_map_alpha_field(void* h, double* alpha, const double* normal, const double* distance, double lower,
                           double upper) {
    // reconstruction::mapAlphaField (reconstruction.C:725-784): every cell
    // with lowerRefineLevel <= alpha <= upperRefineLevel gets the volume
    // fraction its (mapped) interface plane cuts from it
    Oracle* o = static_cast<Oracle*>(h);
    CutCell cc;
    cc.mesh = &o->m;
    for (int c = 0; c < o->m.nc; ++c) {
        if (alpha[c] >= lower && alpha[c] <= upper) {
            cc.calcSubCell(c, load(normal, c), distance[c]);
            alpha[c] = cc.VOF;
        }
    }
    return 0;
}

int oracle_interface_polygons(void* h, int32_t* n_polys, int32_t* n_points, int32_t* offsets, double* pts,
                              int32_t* cells) {
    // reconstruction::interface (reconstruction.C:787-835): the PLIC
    // polygon of every mixed cell whose plane cuts it, ascending in cell
    Oracle* o = static_cast<Oracle*>(h);
    std::vector<int32_t> order(o->mixedCells);
    std::sort(order.begin(), order.end());
    CutCell cc;
    cc.mesh = &o->m;
    int np = 0, nq = 0;
    for (int c : order) {
        if (cc.calcSubCell(c, o->iN[c], o->iD[c]) != 0) continue;
        const std::vector<vec> poly = cc.interfacePoints();
        if (offsets) offsets[nq] = np;
        if (cells) cells[nq] = c;
        for (const vec& p : poly) {
            if (pts) store(pts, np, p);
            ++np;
        }
        ++nq;
    }
    if (offsets) offsets[nq] = np;
    *n_polys = nq;
    *n_points = np;
    return 0;
}

int oracle_calc_sub_cell(void* h, int32_t cell, const double* normal, double distance, double* vof,
                         double* centre, double* area) {
    Oracle* o = static_cast<Oracle*>(h);
    CutCell cc;
    cc.mesh = &o->m;
    const int st = cc.calcSubCell(cell, load(normal, 0), distance);
    *vof = cc.VOF;
    store(centre, 0, cc.interfaceCentre);
    store(area, 0, cc.interfaceArea);
    return st;
}

int oracle_find_signed_distance(void* h, int32_t cell, double alpha, const double* normal, double* d,
                                double* centre, double* area) {
    Oracle* o = static_cast<Oracle*>(h);
    CutCell cc;
    cc.mesh = &o->m;
    vec c = load(centre, 0), s = load(area, 0);
    const int st = cc.findSignedDistance(cell, alpha, load(normal, 0), d, &c, &s);
    store(centre, 0, c);
    store(area, 0, s);
    return st;
}

double oracle_time_integrated_face_flux(void* h, int32_t face, const double* normal, double d, double Un0,
                                        double dt, double phi, double magSf) {
    Oracle* o = static_cast<Oracle*>(h);
    CutFace cf;
    return o->timeIntegratedFaceFlux(cf, face, load(normal, 0), d, Un0, dt, phi, magSf);
}

void oracle_interpolate_U(void* h, int32_t cell, const double* x, const double* U, const double* U_boundary,
                          double* out) {
    Oracle* o = static_cast<Oracle*>(h);
    store(out, 0, o->interpolateU(cell, load(x, 0), U, U_boundary));
}

}  // extern "C"
