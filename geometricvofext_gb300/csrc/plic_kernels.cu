// PLIC surface extraction of the plain FP64 form (built with -fmad=false):
// reconstruction::interface (reconstruction.C:787-835) with
// cutCell::interfacePoints (cutCell.C:545-608).
//
// For every mixed cell the cut of its plane (interfaceN, interfaceD) is
// recomputed (cutCell::calcSubCell, the plane solve's routine); when the
// plane cuts the cell (status 0) the cut points of its faces, in face
// order, are ordered by their angle about the interface centre in the
// interface plane and a point whose angle is within 1e-8 of the previous
// sorted one is dropped.  The angles come from planeAngle (an atan2 of
// correctly rounded operations only, within a few ulp of the C library's):
// a cut point shared by two faces appears twice with coordinates equal up
// to rounding, and which copy is kept depends on the last bits of the two
// angles, so those bits must not depend on a math library.  One
// thread per mixed cell, one instantiation per cell class; each cell
// writes its polygon to a fixed stride and the host gathers them in
// ascending cell order.
#include "plain_geom.cuh"
#include "simplic_kernels.h"

namespace simplic {

namespace {

template <class K>
__global__ void __launch_bounds__(128) kPlicPolygons(DevMesh m, const int* __restrict__ mixed,
                                                     const int* __restrict__ nMixed, const double* __restrict__ nrm,
                                                     const double* __restrict__ dArr, int cls, int stride,
                                                     double* __restrict__ pts, int* __restrict__ count,
                                                     uint32_t* __restrict__ errOut) {
    const int nm = *nMixed;
    uint32_t err = 0;
    for (int i = spreadFirst(); i < nm; i += spreadStride()) {
        const int c = mixed[i];
        if (m.classMask != (1 << cls) && m.cellClass[c] != cls) continue;
        count[i] = 0;
        CellWS<K> w;
        if (!loadCell(m, c, w)) {
            err |= kErrSubFaceOverflow;
            continue;
        }
        const d3 n = ld3(nrm, i);
        const double d = dArr[i];
        SubCell sc;
        calcSubCell(w, n, d, sc, err);
        if (sc.status != 0) continue;
        // the cut points of the faces in face order, as calcSubCell collects them
        double dist[K::kPts];
        unsigned subMask = 0;
        for (int q = 0; q < w.np; ++q) {
            dist[q] = liftedDistance(w.P[q], n, d);
            if (belowBits(dist[q])) subMask |= 1u << q;
        }
        d3 edge[K::kEdge];
        int nEdge = 0;
        for (int k = 0; k < w.nf; ++k) {
            int cnt = 0;
            for (int q = 0; q < w.fsz[k]; ++q) cnt += (subMask >> w.fidx[k][q]) & 1u;
            if (cnt == 0 || cnt == w.fsz[k]) continue;
            d3 cen, area;
            clipCutFace<K>(w.P, w.fidx[k], w.fsz[k], dist, subMask, cen, area, edge, nEdge, err);
        }
        if (nEdge == 0) continue;
        const d3 zhat = sc.is / mag(sc.is);
        d3 xhat = edge[0] - sc.ic;
        xhat = xhat - dot(xhat, zhat) * zhat;
        {
            const double s = mag(xhat);
            xhat = (s < kROOTVSMALL) ? mk(0, 0, 0) : xhat / s;
        }
        d3 yhat = cross(zhat, xhat);
        {
            const double s = mag(yhat);
            yhat = (s < kROOTVSMALL) ? mk(0, 0, 0) : yhat / s;
        }
        double ang[K::kEdge];
        int order[K::kEdge];
        for (int q = 0; q < nEdge; ++q) {
            const d3 r = edge[q] - sc.ic;
            ang[q] = planeAngle(dot(r, yhat), dot(r, xhat));
            int j = q;  // stable insertion sort, ascending
            while (j > 0 && ang[order[j - 1]] > ang[q]) {
                order[j] = order[j - 1];
                --j;
            }
            order[j] = q;
        }
        double* out = pts + 3 * size_t(i) * stride;
        int np = 0;
        for (int q = 0; q < nEdge; ++q) {
            if (q > 0 && !(fabs(ang[order[q]] - ang[order[q - 1]]) > 1e-8)) continue;
            if (np < stride) st3(out, np, edge[order[q]]);
            else err |= kErrEdgeOverflow;
            ++np;
        }
        count[i] = min(np, stride);
    }
    if (err) atomicOr(errOut, err);
}

// reconstruction::mapAlphaField (reconstruction.C:725-784): a cell whose
// alpha lies in [lower, upper] gets the volume fraction its interface plane
// (normal, distance: full cell fields, e.g. mapped from the parent cells of
// a refined mesh) cuts from it.
template <class K>
__global__ void __launch_bounds__(128) kMapAlpha(DevMesh m, double* __restrict__ alpha,
                                                 const double* __restrict__ normal,
                                                 const double* __restrict__ distance, double lower, double upper,
                                                 int cls, uint32_t* __restrict__ errOut) {
    uint32_t err = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.nc; c += gridDim.x * blockDim.x) {
        const double a = alpha[c];
        if (!(a >= lower && a <= upper)) continue;
        if (m.classMask != (1 << cls) && m.cellClass[c] != cls) continue;
        CellWS<K> w;
        if (!loadCell(m, c, w)) {
            err |= kErrSubFaceOverflow;
            continue;
        }
        SubCell sc;
        calcSubCell(w, ld3(normal, c), distance[c], sc, err);
        alpha[c] = sc.vof;
    }
    if (err) atomicOr(errOut, err);
}

template <class Kernel>
int residentBlocks(Kernel k) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, 128, 0);
    return (sms > 0 ? sms : 1) * (per > 0 ? per : 1);
}

}  // namespace

void launchPlicPolygons(const StepArgs& a, int stride, double* pts, int* count, cudaStream_t st) {
    const DevMesh& m = a.m;
    if (m.classMask & 1)
        kPlicPolygons<CapsHex><<<residentBlocks(kPlicPolygons<CapsHex>), 128, 0, st>>>(
            m, a.mixed, a.nMixed, a.nrm, a.dArr, 0, stride, pts, count, a.err);
    if (m.classMask & 2)
        kPlicPolygons<CapsPoly><<<residentBlocks(kPlicPolygons<CapsPoly>), 128, 0, st>>>(
            m, a.mixed, a.nMixed, a.nrm, a.dArr, 1, stride, pts, count, a.err);
    if (m.classMask & 4)
        kPlicPolygons<CapsBig><<<residentBlocks(kPlicPolygons<CapsBig>), 128, 0, st>>>(
            m, a.mixed, a.nMixed, a.nrm, a.dArr, 2, stride, pts, count, a.err);
}

void launchMapAlpha(const DevMesh& m, double* alpha, const double* normal, const double* distance, double lower,
                    double upper, uint32_t* err, cudaStream_t st) {
    if (m.classMask & 1)
        kMapAlpha<CapsHex><<<residentBlocks(kMapAlpha<CapsHex>), 128, 0, st>>>(m, alpha, normal, distance, lower,
                                                                              upper, 0, err);
    if (m.classMask & 2)
        kMapAlpha<CapsPoly><<<residentBlocks(kMapAlpha<CapsPoly>), 128, 0, st>>>(m, alpha, normal, distance, lower,
                                                                                upper, 1, err);
    if (m.classMask & 4)
        kMapAlpha<CapsBig><<<residentBlocks(kMapAlpha<CapsBig>), 128, 0, st>>>(m, alpha, normal, distance, lower,
                                                                              upper, 2, err);
}

}  // namespace simplic
