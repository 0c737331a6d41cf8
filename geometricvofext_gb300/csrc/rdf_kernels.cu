// isoRDF orientation of the plain FP64 form (built with -fmad=false):
// reconstruction::calcInterfaceNFromIsoRDF (reconstruction.C:193-405).
//
// The reference iterates: normals from a least-squares gradient, the plane
// solve (cutCell::findSignedDistance) of every mixed cell not marked too
// coarse, a reconstructed distance function (RDF) on the band of cells
// next to the interface, its least-squares gradient as the next normal,
// and a residual per mixed cell whose sums decide whether to stop.  The
// distance function is OpenFOAM v2312's reconstructedDistanceFunction
// (linked into the reference by src/Allwmake:17-19, absent here), restated
// from the published method (Scheufler & Roenby, J. Comput. Phys. 383
// (2019) 1-23) exactly as the CPU oracle restates it:
//   * band: the mixed cells and every cell sharing a point with one;
//   * a mixed cell with a nonzero normal n: RDF = (C_int - C) . n/|n|;
//   * any other band cell: sum_j w_j (C_int,j - C) . n_j / sum_j w_j over
//     its stencil cells j that carry a plane, w_j the squared cosine between
//     n_j and the direction to C_int,j (1 when C_int,j = C); a cell without
//     such a neighbour keeps its value (zero at the start of a reconstruct).
// Every kernel here is one thread per cell; the per-cell arithmetic is the
// oracle's, operation for operation.  The residual sums that decide the
// iteration count run on the host over the mixed cells in ascending order.
#include "ls_fp64.cuh"
#include "plain_geom.cuh"
#include "simplic_kernels.h"

namespace simplic {

namespace {

// OpenFOAM Vector::normalise(tol): zero below tol, else divided by |v|.
__device__ __forceinline__ d3 normaliseOF(d3 v, double tol) {
    const double s = mag(v);
    return (s < tol) ? mk(0, 0, 0) : v / s;
}

// The mixed position of cell x this reconstruct, or -1.
__device__ __forceinline__ int mixPos(const RdfBuffers& r, int x) {
    const int2 cm = r.cellMix[x];
    return cm.x == r.stamp ? cm.y : -1;
}

// Band, cell -> mixed position, and the alpha gradient of every mixed cell.
__global__ void __launch_bounds__(128) kRdfStart(DevMesh m, const double* __restrict__ alpha,
                                                 const int* __restrict__ mixed, const int* __restrict__ nMixed,
                                                 RdfBuffers r, uint32_t* __restrict__ errOut) {
    const int nm = *nMixed;
    uint32_t err = 0;
    for (int i = spreadFirst(); i < nm; i += spreadStride()) {
        const int c = mixed[i];
        r.cellMix[c] = make_int2(r.stamp, i);
        const int32_t* st;
        const int ns = stencilOf(m, c, st, err);
        for (int s = -1; s < ns; ++s) {
            const int x = (s < 0) ? c : st[s];
            if (atomicExch(r.bandStamp + x, r.stamp) != r.stamp) {
                r.rdf[x] = 0.0;
                r.bandList[atomicAdd(r.bandCount, 1)] = x;
            }
        }
        st3(r.grad, i, lsGradientField(m, c, alpha, err));
        r.tooCoarse[i] = 0;
    }
    if (err) atomicOr(errOut, err);
}

// interfaceN = -normalise(grad), the gradient normalised in place
// (reconstruction.C:240).
__global__ void __launch_bounds__(128) kRdfNormals(const int* __restrict__ nMixed, RdfBuffers r,
                                                   double* __restrict__ nrm) {
    const int nm = *nMixed;
    for (int i = spreadFirst(); i < nm; i += spreadStride()) {
        const d3 g = normaliseOF(ld3(r.grad, i), kSMALL);
        st3(r.grad, i, g);
        st3(nrm, i, (-1.0) * g);
    }
}

// constructRDF on the band (normals -interfaceN passed in, negated again).
__global__ void __launch_bounds__(128) kRdfConstruct(DevMesh m, RdfBuffers r, const double* __restrict__ nrm,
                                                     const double* __restrict__ icArr,
                                                     uint32_t* __restrict__ errOut) {
    const int nb = *r.bandCount;
    uint32_t err = 0;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nb; q += gridDim.x * blockDim.x) {
        const int c = r.bandList[q];
        const int ic = mixPos(r, c);
        if (ic >= 0) {
            const d3 normalC = (-1.0) * ld3(nrm, ic);
            if (mag(normalC) != 0.0) {
                const d3 n = ((-1.0) * normalC) / mag(normalC);
                r.rdf[c] = dot(ld3(icArr, ic) - ld3(m.C, c), n);
                continue;
            }
        }
        double averageDist = 0.0, avgWeight = 0.0;
        const d3 p = ld3(m.C, c);
        const int32_t* st;
        const int ns = stencilOf(m, c, st, err);
        for (int s = -1; s < ns; ++s) {
            const int g = (s < 0) ? c : st[s];
            const int ig = mixPos(r, g);
            if (ig < 0) continue;  // no plane: a zero normal
            d3 n = (-1.0) * ((-1.0) * ld3(nrm, ig));
            if (mag(n) != 0.0) {
                n = n / mag(n);
                d3 toSeg = ld3(icArr, ig) - p;
                const double distToSurf = dot(toSeg, n);
                double weight;
                if (mag(toSeg) != 0.0) {
                    toSeg = toSeg / mag(toSeg);
                    const double w = fabs(dot(toSeg, n));
                    weight = w * w;
                } else {
                    weight = 1.0;
                }
                averageDist += distToSurf * weight;
                avgWeight += weight;
            }
        }
        if (avgWeight != 0.0) r.rdf[c] = averageDist / avgWeight;
    }
    if (err) atomicOr(errOut, err);
}

// The gradient of the distance function and the residual of every mixed
// cell (reconstruction.C:264-332): the mean angle to the neighbours'
// normals (weighted by their magnitudes) and 1 - n . n_new.
__global__ void __launch_bounds__(128) kRdfResidual(DevMesh m, const int* __restrict__ mixed,
                                                    const int* __restrict__ nMixed, RdfBuffers r,
                                                    const double* __restrict__ nrm, uint32_t* __restrict__ errOut) {
    constexpr double kTSMALLr = kTSMALL;
    const int nm = *nMixed;
    uint32_t err = 0;
    for (int i = spreadFirst(); i < nm; i += spreadStride()) {
        const int c = mixed[i];
        d3 g = lsGradientField(m, c, r.rdf, err);
        const d3 cellNormal = ld3(nrm, i);
        // the reference's zero-normal test normalises the gradient in place
        // when the cell's own normal is not zero
        if (!(mag(cellNormal) < kTSMALLr)) g = normaliseOF(g, kSMALL);
        double avgDiff = 0.0, weight = 0.0;
        const int32_t* st;
        const int ns = stencilOf(m, c, st, err);
        for (int s = 0; s < ns; ++s) {  // stencil entries after the cell itself
            const int ig = mixPos(r, st[s]);
            if (ig < 0) continue;
            const d3 normal = ld3(nrm, ig);
            if (mag(normal) >= kTSMALLr) {
                const d3 n = normal / mag(normal);
                const double cosAngle = fmax(fmin(dot(cellNormal, n), 1.0), -1.0);
                avgDiff += acos(cosAngle) * mag(normal);
                weight += mag(normal);
            }
        }
        avgDiff = (weight != 0.0) ? avgDiff / weight : 0.0;
        g = normaliseOF(g, kSMALL);
        st3(r.grad, i, g);
        r.res[i] = 1.0 - dot(cellNormal, (-1.0) * g);
        r.avgA[i] = avgDiff;
    }
    if (err) atomicOr(errOut, err);
}

template <class Kernel>
int gridFor(Kernel k, int threads) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, threads, 0);
    return (sms > 0 ? sms : 1) * (per > 0 ? per : 1);
}

}  // namespace

void launchRdfStart(const StepArgs& a, const RdfBuffers& r, cudaStream_t st) {
    kRdfStart<<<gridFor(kRdfStart, 128), 128, 0, st>>>(a.m, a.aCur, a.mixed, a.nMixed, r, a.err);
}

void launchRdfNormals(const StepArgs& a, const RdfBuffers& r, cudaStream_t st) {
    kRdfNormals<<<gridFor(kRdfNormals, 128), 128, 0, st>>>(a.nMixed, r, a.nrm);
}

void launchRdfConstruct(const StepArgs& a, const RdfBuffers& r, cudaStream_t st) {
    kRdfConstruct<<<gridFor(kRdfConstruct, 128), 128, 0, st>>>(a.m, r, a.nrm, a.icArr, a.err);
}

void launchRdfResidual(const StepArgs& a, const RdfBuffers& r, cudaStream_t st) {
    kRdfResidual<<<gridFor(kRdfResidual, 128), 128, 0, st>>>(a.m, a.mixed, a.nMixed, r, a.nrm, a.err);
}

}  // namespace simplic
