// C ABI of the GB300 SimPLIC step: handle, one-time mesh upload, launches.
//
// The handle stands in for one reference solveVofEqu object
// (src/SimPLIC/solveVofEqu/solveVofEqu.C:55-107): it owns the
// reconstruction state (mixed cells, statuses, interface planes) and the
// advection state (Simpson face fluxes, alphaPhi, bounding scratch).  Host
// code here is built with -ffp-contract=off: the interpolation weights it
// precomputes are the same doubles as the CPU restatement's.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/simplic.h"
#include "../../include/simplic_mlp.h"
#include "simplic_kernels.h"

using namespace simplic;

namespace {

thread_local std::string g_createError;

constexpr int kMapTimer = 1000;  // event kind of simplic_map_alpha_field

struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    int kind = 0;  // 0 reconstruct, 1 advect; 2 + kernel id for kernel timing
};

enum KernelId {
    kKScan = 0,
    kKLs,
    kKPlane,
    kKFluxUn0,
    kKFluxFaces,
    kKUpdate,
    kKBound,
    kKBrute,
    kKFlat,
    kKFaceFull,
    kKNetInputs,
    kKNetwork,
    kKNetGate,
    kKRdf,
    kNumKernels
};
const char* const kKernelNames[kNumKernels] = {"scanMixed", "lsNormal",   "planeSolve",   "interfaceUn0",
                                               "interfaceFaces", "update", "bound",       "bruteForce",
                                               "faceFlatness", "faceFull", "netInputs", "network",
                                               "netGate", "isoRDF"};
static_assert(kNumKernels == SIMPLIC_N_KERNELS, "kernel table");

struct DeviceBuffers {
    std::vector<void*> owned;
    // test setting (SIMPLIC_TEST_FAIL_ALLOC_AFTER): the allocations left
    // before one fails as if the device were out of memory; -1 = never
    long long failAfter = -1;
    template <class T>
    T* alloc(size_t n) {
        void* p = nullptr;
        if (n == 0) n = 1;
        if (failAfter == 0) return nullptr;
        if (failAfter > 0) --failAfter;
        if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
        owned.push_back(p);
        return static_cast<T*>(p);
    }
    ~DeviceBuffers() {
        for (void* p : owned) cudaFree(p);
    }
};

}  // namespace

struct simplic_handle {
    simplic_controls ctrl{};
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    std::string err;
    DeviceBuffers mem;
    DevMesh m{};
    double* Sf = nullptr;
    // alpha
    double* aBuf[2] = {nullptr, nullptr};
    int cur = 0;
    double* aOldBuf = nullptr;
    bool haveAlpha = false, reconstructed = false;
    // reconstruction state
    int8_t* status = nullptr;
    int* mixed = nullptr;
    int* nMixed = nullptr;
    double* nrm = nullptr;
    int8_t* mStatus = nullptr;
    double* dArr = nullptr;
    double* icArr = nullptr;
    double* isArr = nullptr;
    // advection state
    double* dvfI = nullptr;
    double* alphaPhi = nullptr;
    uint8_t* cutMask = nullptr;
    double* un0 = nullptr;
    int2* dwList = nullptr;
    int* dwCount = nullptr;
    uint32_t* devErr = nullptr;
    BoundBuffers bb{};
    RdfBuffers rdf{};  // isoRDF orientation only
    int32_t lastRdfIterations = 0;
    // PLIC surface of the last reconstruct (built on the first request)
    uint64_t reconCount = 0, plicOf = ~uint64_t(0);
    double* plicPts = nullptr;
    int* plicCount = nullptr;
    int plicCap = 0;  // mixed cells the scratch holds
    std::vector<int32_t> plicOffsets, plicCells;
    std::vector<double> plicPoints;
    // host-input staging (allocated on first host-API advect)
    double* sPhi = nullptr;
    double* sU = nullptr;
    double* sUb = nullptr;
    double* sAlphaB = nullptr;
    double* sSp = nullptr;
    double* sSu = nullptr;
    double* scratchF = nullptr;  // [nf] for rho-phi on host arrays
    double* mapScratch = nullptr;  // [5 nc] alpha, normal, distance of a host-array mapAlphaField
    // learned-normal network (allocated by simplic_set_network)
    bool haveNet = false;
    int netRows = 0;               // rows of the network buffers (mixed cells evaluated)
    float netGateTol = 0.f;
    float* netA = nullptr;          // [netRows][32] FP32 alphas of the network's neighbourhoods
    float* netY = nullptr;          // [netRows][16] network outputs
    __nv_bfloat16* netW = nullptr;  // [4][128][128]
    float* netB = nullptr;          // [4][128]
    __nv_bfloat16* netX = nullptr;  // [netRows][128] network input
    int* nLearned = nullptr;
    // timers
    std::vector<EventPair> events;
    size_t eventsUsed = 0;
    double tRecon = 0.0, tAdv = 0.0, tMap = 0.0;
    bool kernelTiming = false;
    double kMs[kNumKernels] = {0};
    int64_t kLaunches[kNumKernels] = {0};
    int32_t lastNMixed = 0, lastPasses = 0, lastMaxBound = 0;
    int32_t nBoxCells = 0;  // axis-aligned box cells of the mesh
    int nb = 0, nfb = 0;
};

namespace {

int fail(simplic_handle* h, int code, const std::string& msg) {
    if (h)
        h->err = msg;
    else
        g_createError = msg;
    return code;
}

int cudaFail(simplic_handle* h, cudaError_t e, const char* what) {
    return fail(h, SIMPLIC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(h, expr)                                   \
    do {                                              \
        cudaError_t _e = (expr);                      \
        if (_e != cudaSuccess) return cudaFail(h, _e, #expr); \
    } while (0)

template <class T>
int upload(simplic_handle* h, T*& dst, const T* src, size_t n) {
    dst = h->mem.alloc<T>(n);
    if (!dst) return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (mesh upload)");
    if (n) CK(h, cudaMemcpy(dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return SIMPLIC_OK;
}

EventPair& nextEvents(simplic_handle* h, int kind) {
    if (h->eventsUsed == h->events.size()) {
        EventPair p;
        cudaEventCreate(&p.a);
        cudaEventCreate(&p.b);
        h->events.push_back(p);
    }
    EventPair& e = h->events[h->eventsUsed++];
    e.kind = kind;
    return e;
}

void collectTimers(simplic_handle* h) {
    for (size_t i = 0; i < h->eventsUsed; ++i) {
        float ms = 0.f;
        if (cudaEventSynchronize(h->events[i].b) == cudaSuccess &&
            cudaEventElapsedTime(&ms, h->events[i].a, h->events[i].b) == cudaSuccess) {
            const int k = h->events[i].kind;
            if (k == 0)
                h->tRecon += 1e-3 * ms;
            else if (k == 1)
                h->tAdv += 1e-3 * ms;
            else if (k == kMapTimer)
                h->tMap += 1e-3 * ms;
            else
                h->kMs[k - 2] += ms;
        }
    }
    h->eventsUsed = 0;
}

// Launch wrapper: counts launches and, when enabled, brackets the launch
// with an event pair.  Pending pairs are folded in at the start of a call
// once 4096 are queued, so the list stays bounded without a per-step
// synchronisation.
// nKernels: the kernels one call launches (counted in kLaunches)
template <class F>
void timedLaunch(simplic_handle* h, int kid, F&& launch, int nKernels = 1) {
    if (h->kernelTiming) {
        EventPair& e = nextEvents(h, 2 + kid);
        cudaEventRecord(e.a, h->stream);
        launch();
        cudaEventRecord(e.b, h->stream);
    } else {
        launch();
    }
    h->kLaunches[kid] += nKernels;
}

StepArgs baseArgs(simplic_handle* h) {
    StepArgs a{};
    a.m = h->m;
    a.mixedTol = h->ctrl.mixed_cell_tol;
    a.snapTol = h->ctrl.snap_tol;
    a.clip = h->ctrl.clip;
    a.nAlphaBounds = h->ctrl.n_alpha_bounds;
    a.status = h->status;
    a.mixed = h->mixed;
    a.nMixed = h->nMixed;
    a.nrm = h->nrm;
    a.mStatus = h->mStatus;
    a.dArr = h->dArr;
    a.icArr = h->icArr;
    a.isArr = h->isArr;
    a.dvfI = h->dvfI;
    a.alphaPhi = h->alphaPhi;
    a.cutMask = h->ctrl.record_cut_faces ? h->cutMask : nullptr;
    a.un0 = h->un0;
    a.dwList = h->dwList;
    a.dwCount = h->dwCount;
    a.ovList = h->bb.ovList;
    a.ovCount = h->bb.ovCount;
    a.ovCap = h->bb.ovCap;
    a.err = h->devErr;
    return a;
}

int checkDeviceErrors(simplic_handle* h) {
    uint32_t e = 0;
    CK(h, cudaMemcpyAsync(&e, h->devErr, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (e) {
        CK(h, cudaMemsetAsync(h->devErr, 0, sizeof(uint32_t), h->stream));
        std::string msg = "device error flags:";
        if (e & kErrSubFaceOverflow) msg += " cell-exceeds-caps";
        if (e & kErrEdgeOverflow) msg += " interface-edge-overflow";
        if (e & kErrStencilOverflow) msg += " stencil-overflow";
        if (e & kErrBoundOverflow) msg += " bounding-scratch-overflow";
        if (e & kErrNonFinite) msg += " non-finite-alpha";
        if (e & kErrBarrierTimeout) msg += " grid-barrier-timeout";
        return fail(h, SIMPLIC_ERR_DEVICE, msg);
    }
    return SIMPLIC_OK;
}

// -------------------------------------------------------------------------
// one-time mesh preprocessing (host) and upload
// -------------------------------------------------------------------------
inline d3 hld(const double* p, int64_t i) { return d3{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
inline double hmag(d3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// Host-side addressing built from the caller's mesh (validated on the way;
// no device call), then uploaded by uploadMesh.
struct HostMesh {
    std::vector<int32_t> cOff, cFaces, cpOff, cPts, pcOff, pCells, pbOff, pbFaces;
    std::vector<int2> cSlot;
    std::vector<uint8_t> boxCorner, cellClass;
    int32_t classMask = 0, maxCellFaces = 0;
    std::vector<double> pcW, pbW;
};

int prepareMesh(simplic_handle* h, const simplic_mesh_desc* d, HostMesh& hm) {
    const int np = d->n_points, nf = d->n_faces, nfi = d->n_internal_faces, nc = d->n_cells;
    // cells < 2^27: the bounding kernel keys corrected faces as cell * 32 + slot in 32 bits
    if (np <= 0 || nf <= 0 || nc <= 0 || nfi < 0 || nfi > nf || nc >= (1 << 27))
        return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "mesh sizes out of range");
    if (!d->points || !d->face_offsets || !d->face_points || !d->owner || (nfi && !d->neighbour) ||
        !d->cell_centres || !d->cell_volumes || !d->face_centres || !d->face_areas || !d->face_mag_areas)
        return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "mesh array pointer is NULL");
    const int32_t* fo = d->face_offsets;
    if (fo[0] != 0) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "face_offsets[0] != 0");
    for (int f = 0; f < nf; ++f) {
        const int n = fo[f + 1] - fo[f];
        if (n < 3) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "face with fewer than 3 points");
        if (n > kMaxFacePts) return fail(h, SIMPLIC_ERR_MESH_CAPS, "face exceeds kMaxFacePts points");
    }
    const int64_t nfp = fo[nf];
    for (int64_t k = 0; k < nfp; ++k)
        if (d->face_points[k] < 0 || d->face_points[k] >= np)
            return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "face point index out of range");
    for (int f = 0; f < nf; ++f)
        if (d->owner[f] < 0 || d->owner[f] >= nc) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "owner out of range");
    for (int f = 0; f < nfi; ++f)
        if (d->neighbour[f] < 0 || d->neighbour[f] >= nc || d->neighbour[f] == d->owner[f])
            return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "neighbour out of range");

    // cells(): owned faces ascending, then neighbour faces ascending
    std::vector<int32_t> nOwn(nc, 0), nNei(nc, 0);
    for (int f = 0; f < nf; ++f) nOwn[d->owner[f]]++;
    for (int f = 0; f < nfi; ++f) nNei[d->neighbour[f]]++;
    std::vector<int32_t> cOff(nc + 1, 0);
    for (int c = 0; c < nc; ++c) {
        const int k = nOwn[c] + nNei[c];
        if (k > kMaxCellFaces) return fail(h, SIMPLIC_ERR_MESH_CAPS, "cell exceeds kMaxCellFaces faces");
        if (k < 4) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "cell with fewer than 4 faces");
        cOff[c + 1] = cOff[c] + k;
    }
    const int64_t ncf = cOff[nc];
    std::vector<int32_t> cFaces(ncf), fill(nc, 0);
    for (int f = 0; f < nf; ++f) {
        const int c = d->owner[f];
        cFaces[cOff[c] + fill[c]++] = f;
    }
    for (int f = 0; f < nfi; ++f) {
        const int c = d->neighbour[f];
        cFaces[cOff[c] + fill[c]++] = f;
    }
    // ascending merge with the neighbour-side flag, and the cell across
    std::vector<int2> cSlot(ncf);
    for (int c = 0; c < nc; ++c) {
        int a = cOff[c], ae = cOff[c] + nOwn[c], b = ae, be = cOff[c + 1], w = cOff[c];
        while (a < ae || b < be) {
            const bool takeOwn = (b >= be) || (a < ae && cFaces[a] < cFaces[b]);
            const int f = takeOwn ? cFaces[a++] : cFaces[b++];
            cSlot[w].x = (f < nfi) ? (takeOwn ? d->neighbour[f] : d->owner[f]) : -1;
            cSlot[w].y = takeOwn ? f : int32_t(uint32_t(f) | 0x80000000u);
            ++w;
        }
    }
    // cellPoints ascending
    std::vector<int32_t> cpOff(nc + 1, 0), cPts;
    cPts.reserve(size_t(nc) * 8);
    std::vector<int32_t> tmp;
    for (int c = 0; c < nc; ++c) {
        tmp.clear();
        for (int k = cOff[c]; k < cOff[c + 1]; ++k) {
            const int f = cFaces[k];
            for (int q = fo[f]; q < fo[f + 1]; ++q) tmp.push_back(d->face_points[q]);
        }
        std::sort(tmp.begin(), tmp.end());
        tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
        if (int(tmp.size()) > kMaxCellPts) return fail(h, SIMPLIC_ERR_MESH_CAPS, "cell exceeds kMaxCellPts points");
        cPts.insert(cPts.end(), tmp.begin(), tmp.end());
        cpOff[c + 1] = int32_t(cPts.size());
    }
    // workspace class of every cell (its faces, points, largest face)
    hm.cellClass.assign(nc, 0);
    for (int c = 0; c < nc; ++c) {
        int mfp = 0;
        for (int k = cOff[c]; k < cOff[c + 1]; ++k) mfp = std::max(mfp, fo[cFaces[k] + 1] - fo[cFaces[k]]);
        const int nfc = cOff[c + 1] - cOff[c];
        const int cls = cellClassOf(nfc, cpOff[c + 1] - cpOff[c], mfp);
        if (cls < 0) return fail(h, SIMPLIC_ERR_MESH_CAPS, "cell exceeds the static caps");
        hm.cellClass[c] = uint8_t(cls);
        hm.classMask |= 1 << cls;
        hm.maxCellFaces = std::max(hm.maxCellFaces, nfc);
    }
    // axis-aligned box cells (eight points on the corners of their bounding
    // box, six faces): 0x40 | (lowest corner << 3) | highest corner, local
    // point indices; the mixed forms solve their planes in closed form
    std::vector<uint8_t> boxCorner(nc, 0);
    for (int c = 0; c < nc; ++c) {
        const int p0 = cpOff[c];
        if (cpOff[c + 1] - p0 != 8 || cOff[c + 1] - cOff[c] != 6) continue;
        double lo[3], hi[3];
        for (int k = 0; k < 3; ++k) lo[k] = hi[k] = d->points[3 * size_t(cPts[p0]) + k];
        for (int i = 1; i < 8; ++i)
            for (int k = 0; k < 3; ++k) {
                const double x = d->points[3 * size_t(cPts[p0 + i]) + k];
                lo[k] = std::min(lo[k], x);
                hi[k] = std::max(hi[k], x);
            }
        unsigned seen = 0;
        int iLo = -1, iHi = -1;
        bool ok = hi[0] > lo[0] && hi[1] > lo[1] && hi[2] > lo[2];
        for (int i = 0; ok && i < 8; ++i) {
            unsigned code = 0;
            for (int k = 0; k < 3; ++k) {
                const double x = d->points[3 * size_t(cPts[p0 + i]) + k];
                if (x == hi[k]) code |= 1u << k;
                else if (x != lo[k]) ok = false;
            }
            seen |= 1u << code;
            if (code == 0) iLo = i;
            if (code == 7) iHi = i;
        }
        if (ok && seen == 0xffu) {
            boxCorner[c] = uint8_t(0x40 | (iLo << 3) | iHi);
            ++h->nBoxCells;
        }
    }
    // pointCells (ascending cells) with normalised inverse-distance weights
    std::vector<int32_t> pcOff(np + 1, 0);
    for (size_t k = 0; k < cPts.size(); ++k) pcOff[cPts[k] + 1]++;
    for (int p = 0; p < np; ++p) pcOff[p + 1] += pcOff[p];
    std::vector<int32_t> pCells(cPts.size()), pf(np, 0);
    for (int c = 0; c < nc; ++c)
        for (int k = cpOff[c]; k < cpOff[c + 1]; ++k) {
            const int p = cPts[k];
            pCells[pcOff[p] + pf[p]++] = c;
        }
    std::vector<double> pcW(pCells.size());
    for (int p = 0; p < np; ++p) {
        const d3 P = hld(d->points, p);
        double sumW = 0.0;
        for (int k = pcOff[p]; k < pcOff[p + 1]; ++k) {
            const double w = 1.0 / hmag(P - hld(d->cell_centres, pCells[k]));
            pcW[k] = w;
            sumW += w;
        }
        for (int k = pcOff[p]; k < pcOff[p + 1]; ++k) pcW[k] = pcW[k] / sumW;
    }
    // boundary point -> boundary faces (ascending), weights 1/|p - Cf|
    std::vector<int32_t> pbOff(np + 1, 0);
    for (int f = nfi; f < nf; ++f)
        for (int q = fo[f]; q < fo[f + 1]; ++q) pbOff[d->face_points[q] + 1]++;
    for (int p = 0; p < np; ++p) pbOff[p + 1] += pbOff[p];
    std::vector<int32_t> pbFaces(pbOff[np]);
    std::fill(pf.begin(), pf.end(), 0);
    for (int f = nfi; f < nf; ++f)
        for (int q = fo[f]; q < fo[f + 1]; ++q) {
            const int p = d->face_points[q];
            pbFaces[pbOff[p] + pf[p]++] = f;
        }
    std::vector<double> pbW(pbFaces.size());
    for (int p = 0; p < np; ++p) {
        const d3 P = hld(d->points, p);
        double sumW = 0.0;
        for (int k = pbOff[p]; k < pbOff[p + 1]; ++k) {
            const double w = 1.0 / hmag(P - hld(d->face_centres, pbFaces[k]));
            pbW[k] = w;
            sumW += w;
        }
        for (int k = pbOff[p]; k < pbOff[p + 1]; ++k) pbW[k] = pbW[k] / sumW;
    }
    hm.cOff = std::move(cOff);
    hm.cFaces = std::move(cFaces);
    hm.cSlot = std::move(cSlot);
    hm.cpOff = std::move(cpOff);
    hm.cPts = std::move(cPts);
    hm.boxCorner = std::move(boxCorner);
    hm.pcOff = std::move(pcOff);
    hm.pCells = std::move(pCells);
    hm.pcW = std::move(pcW);
    hm.pbOff = std::move(pbOff);
    hm.pbFaces = std::move(pbFaces);
    hm.pbW = std::move(pbW);
    return SIMPLIC_OK;
}

int uploadMesh(simplic_handle* h, const simplic_mesh_desc* d, const HostMesh& hm) {
    const int np = d->n_points, nf = d->n_faces, nfi = d->n_internal_faces, nc = d->n_cells;
    const int32_t* fo = d->face_offsets;
    const int64_t nfp = fo[nf];
    const auto& cOff = hm.cOff;
    const auto& cFaces = hm.cFaces;
    const auto& cSlot = hm.cSlot;
    const auto& cpOff = hm.cpOff;
    const auto& cPts = hm.cPts;
    const auto& boxCorner = hm.boxCorner;
    const auto& pcOff = hm.pcOff;
    const auto& pCells = hm.pCells;
    const auto& pcW = hm.pcW;
    const auto& pbOff = hm.pbOff;
    const auto& pbFaces = hm.pbFaces;
    const auto& pbW = hm.pbW;
    DevMesh& m = h->m;
    m.np = np;
    m.nf = nf;
    m.nfi = nfi;
    m.nc = nc;
    int r;
    double* dp;
    int32_t* ip;
#define UP(field, T, src, n)                                      \
    if ((r = upload<T>(h, (T*&)(field), (src), (n))) != SIMPLIC_OK) return r;
    UP(dp, double, d->points, size_t(3) * np); m.pts = dp;
    UP(ip, int32_t, d->face_offsets, size_t(nf) + 1); m.fOff = ip;
    UP(ip, int32_t, d->face_points, size_t(nfp)); m.fPts = ip;
    UP(ip, int32_t, d->owner, size_t(nf)); m.own = ip;
    UP(ip, int32_t, d->neighbour, size_t(nfi)); m.nei = ip;
    UP(dp, double, d->cell_centres, size_t(3) * nc); m.C = dp;
    UP(dp, double, d->cell_volumes, size_t(nc)); m.V = dp;
    UP(dp, double, d->face_centres, size_t(3) * nf); m.Cf = dp;
    UP(dp, double, d->face_mag_areas, size_t(nf)); m.magSf = dp;
    UP(dp, double, d->face_areas, size_t(3) * nf); h->Sf = dp;
    UP(ip, int32_t, cOff.data(), cOff.size()); m.cOff = ip;
    m.uniformFaces = nc > 0 ? cOff[1] - cOff[0] : 0;
    for (int c = 1; c < nc && m.uniformFaces; ++c)
        if (cOff[c + 1] - cOff[c] != m.uniformFaces) m.uniformFaces = 0;
    // a single-block lattice: the dimensions from cell 0's owned neighbours
    // (+x = 1, +y = nx, +z = nx ny), accepted only if every interior cell's
    // slot records are those latticeSlots gives
    m.latNx = m.latNy = m.latNz = 0;
    m.latDivLayer = m.latDivNx = FastDiv{0u, 0};
    if (m.uniformFaces == 6 && nc >= 27) {
        int nb[6], nn = 0;
        for (int q = 0; q < 6; ++q)
            if (cSlot[q].x > 0 && cSlot[q].y >= 0) nb[nn++] = cSlot[q].x;
        if (nn == 3 && nb[0] == 1 && nb[1] > 2 && nb[2] % nb[1] == 0) {
            const int nx = nb[1], ny = nb[2] / nb[1];
            const int nz = (ny > 0 && nc % (nx * ny) == 0) ? nc / (nx * ny) : 0;
            bool ok = nz >= 3 && ny >= 3 && nx >= 3;
            // the device derives a cell's lattice position by multiplications
            // (latticeSlotsFast); every cell is checked with that same code
            const FastDiv dLayer = makeFastDiv(uint32_t(nx) * uint32_t(ny)), dNx = makeFastDiv(uint32_t(nx));
            for (int c = 0; ok && c < nc; ++c) {
                int2 sl[6], sr[6];
                const bool in = latticeSlotsFast(c, nx, ny, nz, dLayer, dNx, sl);
                ok = in == latticeSlots(c, nx, ny, nz, sr);
                if (!ok || !in) continue;
                for (int q = 0; q < 6 && ok; ++q) ok = sl[q].x == cSlot[6 * size_t(c) + q].x && sl[q].y == cSlot[6 * size_t(c) + q].y;
            }
            if (ok) {
                m.latNx = nx;
                m.latNy = ny;
                m.latNz = nz;
                m.latDivLayer = dLayer;
                m.latDivNx = dNx;
            }
        }
    }
    UP(ip, int32_t, cFaces.data(), cFaces.size()); m.cFaces = ip;
    {
        int2* sp = nullptr;
        UP(sp, int2, cSlot.data(), cSlot.size());
        m.cSlot = sp;
    }
    UP(ip, int32_t, cpOff.data(), cpOff.size()); m.cpOff = ip;
    {
        uint8_t* cp = nullptr;
        UP(cp, uint8_t, hm.cellClass.data(), hm.cellClass.size());
        m.cellClass = cp;
        m.classMask = hm.classMask;
        m.maxCellFaces = hm.maxCellFaces;
    }
    {
        uint8_t* bp = nullptr;
        UP(bp, uint8_t, boxCorner.data(), boxCorner.size());
        m.boxCorner = bp;
    }
    UP(ip, int32_t, cPts.data(), cPts.size()); m.cPts = ip;
    UP(ip, int32_t, pcOff.data(), pcOff.size()); m.pcOff = ip;
    UP(ip, int32_t, pCells.data(), pCells.size()); m.pCells = ip;
    UP(dp, double, pcW.data(), pcW.size()); m.pcW = dp;
    UP(ip, int32_t, pbOff.data(), pbOff.size()); m.pbOff = ip;
    UP(ip, int32_t, pbFaces.data(), pbFaces.size()); m.pbFaces = ip;
    UP(dp, double, pbW.data(), pbW.size()); m.pbW = dp;
#undef UP
    double* flat = h->mem.alloc<double>(nf);
    double* fullC = h->mem.alloc<double>(size_t(3) * nf);
    double* fullA = h->mem.alloc<double>(size_t(3) * nf);
    if (!flat || !fullC || !fullA) return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (face data)");
    m.flat = flat;
    m.fullC = fullC;
    m.fullA = fullA;
    {
        double* rV = h->mem.alloc<double>(nc);
        if (!rV) return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (reciprocal volumes)");
        m.rV = rV;
        launchRecipVolume(m, rV, h->stream);
    }
    timedLaunch(h, kKFlat, [&] { launchFaceFlatness(m, h->Sf, flat, h->stream); });
    timedLaunch(h, kKFaceFull, [&] { launchFaceFull(m, fullC, fullA, h->stream); });
    CK(h, cudaGetLastError());
    m.splitClass = nullptr;
    m.splitClassMask = 0;
    if (h->ctrl.split_warped_face) {
        // the workspace class of every cell with its warped faces fanned
        // (getLocalPointFieldAndFaceList, cutCell.C:140-236)
        std::vector<double> fl(nf);
        CK(h, cudaMemcpyAsync(fl.data(), flat, sizeof(double) * nf, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        std::vector<uint8_t> sc(nc);
        int sizes[kMaxCellFaces];
        bool warped[kMaxCellFaces];
        for (int c = 0; c < nc; ++c) {
            const int nfc = cOff[c + 1] - cOff[c];
            int mfp = 0;
            for (int k = 0; k < nfc; ++k) {
                const int f = cFaces[cOff[c] + k];
                sizes[k] = fo[f + 1] - fo[f];
                warped[k] = !(fl[f] > 1.0 - kTSMALL);
                mfp = std::max(mfp, warped[k] ? 3 : sizes[k]);
            }
            int sf = 0, sp = 0;
            splitCounts(nfc, cpOff[c + 1] - cpOff[c], sizes, warped, sf, sp);
            const int cls = cellClassOf(sf, sp, mfp);
            if (cls < 0) return fail(h, SIMPLIC_ERR_MESH_CAPS, "a cell with its warped faces split exceeds the static caps");
            sc[c] = uint8_t(cls);
            m.splitClassMask |= 1 << cls;
        }
        uint8_t* sp = nullptr;
        if ((r = upload<uint8_t>(h, sp, sc.data(), sc.size())) != SIMPLIC_OK) return r;
        m.splitClass = sp;
    }
    // LS stencils of all cells (read by the normal and network-input kernels)
    {
        int* len = h->mem.alloc<int>(size_t(nc));
        if (!len) return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (stencil lengths)");
        launchStencilRows(m, true, len, nullptr, nullptr, h->stream);
        CK(h, cudaGetLastError());
        std::vector<int32_t> stOff(size_t(nc) + 1, 0);
        CK(h, cudaMemcpyAsync(stOff.data() + 1, len, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        int64_t tot = 0;
        for (int c = 0; c < nc; ++c) {
            tot += stOff[c + 1];
            if (tot > INT32_MAX) return fail(h, SIMPLIC_ERR_MESH_CAPS, "LS stencils exceed 2^31 entries");
            stOff[c + 1] = int32_t(tot);
        }
        int32_t* off = nullptr;
        if ((r = upload<int32_t>(h, off, stOff.data(), stOff.size())) != SIMPLIC_OK) return r;
        int32_t* rows = h->mem.alloc<int32_t>(size_t(std::max<int64_t>(tot, 1)));
        if (!rows) return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (stencils)");
        launchStencilRows(m, false, nullptr, off, rows, h->stream);
        CK(h, cudaGetLastError());
        m.stOff = off;
        m.stCells = rows;
    }
    return SIMPLIC_OK;
}

int allocState(simplic_handle* h) {
    const int nc = h->m.nc, nf = h->m.nf;
    h->nb = (nc + 255) / 256;
    h->nfb = nf - h->m.nfi;
    auto& M = h->mem;
    h->aBuf[0] = M.alloc<double>(nc);
    h->aBuf[1] = M.alloc<double>(nc);
    h->aOldBuf = M.alloc<double>(nc);
    h->status = M.alloc<int8_t>(nc);
    h->mixed = M.alloc<int>(nc);
    h->nMixed = M.alloc<int>(1);
    h->nrm = M.alloc<double>(size_t(3) * nc);
    h->mStatus = M.alloc<int8_t>(nc);
    h->dArr = M.alloc<double>(nc);
    h->icArr = M.alloc<double>(size_t(3) * nc);
    h->isArr = M.alloc<double>(size_t(3) * nc);
    h->un0 = M.alloc<double>(nc);
    // every face is downwind of at most one cell: nf entries always suffice
    h->dwList = M.alloc<int2>(nf);
    h->dwCount = M.alloc<int>(1);
    if (!h->un0 || !h->dwList || !h->dwCount)
        return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (plane scratch)");
    h->dvfI = M.alloc<double>(nf);
    h->alphaPhi = M.alloc<double>(nf);
    h->cutMask = h->ctrl.record_cut_faces ? M.alloc<uint8_t>(nf) : nullptr;
    h->devErr = M.alloc<uint32_t>(1);
    BoundBuffers& b = h->bb;
    // overshooting cells per step are a small fraction of the interface
    // cells; the caps scale with the mesh (1/16 of the cells, at least 128k)
    // and an overflow is reported as a device error, never truncated
    b.ovCap = std::max(1 << 17, nc / 16);
    b.ovList = M.alloc<int>(b.ovCap);
    b.ovCount = M.alloc<int>(2);  // [0] overshooting cells, [1] listed (bounding-set) cells
    b.candCap = 2 * b.ovCap;
    b.cand = M.alloc<int>(b.candCap);
    b.candIdx = M.alloc<int>(nc);
    b.candMark = M.alloc<int>(nc);
    b.cellClaim = M.alloc<int>(nc);
    b.faceKey = M.alloc<unsigned>(nf);
    b.faceStamp = M.alloc<int>(nf);
    b.touchedCap = std::max(1 << 20, 4 * b.candCap);
    b.touched = M.alloc<int>(b.touchedCap);
    b.corr = M.alloc<double>(nf);
    b.dvfMod = M.alloc<double>(nf);
    b.modStamp = M.alloc<int>(nf);
    b.modCap = std::max(1 << 20, 4 * b.candCap);
    b.modList = M.alloc<int>(b.modCap);
    b.ctl = M.alloc<int>(kCtlSize);
    b.barCount = M.alloc<unsigned>(1);
    b.barGen = M.alloc<unsigned>(1);
    b.spinLimit = kBarrierSpins;
    b.barrierExtra = 0;
    // test setting: a grid barrier that waits for one block too many, so its
    // bounded wait runs out (polls: the value of the variable)
    if (const char* v = std::getenv("SIMPLIC_TEST_BARRIER_STALL")) {
        const long long spins = std::atoll(v);
        if (spins > 0) {
            b.barrierExtra = 1;
            b.spinLimit = spins;
        }
    }
    b.info = M.alloc<int>(8);
    b.actList = M.alloc<int>(b.candCap);
    {
        const size_t slots = size_t(b.candCap) * h->m.maxCellFaces;
        b.slotF = M.alloc<int>(slots);
        b.slotFlags = M.alloc<uint8_t>(slots);
        b.slotSucc = M.alloc<int>(slots);
        b.slotDv = M.alloc<double>(slots);
        b.slotPhdt = M.alloc<double>(slots);
        b.slotMax0 = M.alloc<double>(slots);
        b.slotThr0 = M.alloc<double>(slots);
    }
    b.candK = M.alloc<uint8_t>(size_t(b.candCap) * kBoundCellConstBytes);
    b.candDepN = M.alloc<int>(b.candCap);
    b.candPending = M.alloc<int>(b.candCap);
    b.candPm = M.alloc<unsigned>(b.candCap);
    b.readyQ = M.alloc<unsigned long long>(b.candCap);
    b.stamp = 0;
    for (void* p : {(void*)h->aBuf[0], (void*)h->aBuf[1], (void*)h->aOldBuf, (void*)h->status, (void*)h->mixed,
                    (void*)h->nMixed, (void*)h->nrm, (void*)h->mStatus, (void*)h->dArr, (void*)h->icArr,
                    (void*)h->isArr, (void*)h->dvfI, (void*)h->alphaPhi,
                    (void*)h->devErr, (void*)b.ovList, (void*)b.ovCount, (void*)b.cand, (void*)b.candIdx,
                    (void*)b.candMark, (void*)b.cellClaim, (void*)b.faceKey, (void*)b.faceStamp,
                    (void*)b.touched, (void*)b.corr, (void*)b.dvfMod, (void*)b.modStamp, (void*)b.modList,
                    (void*)b.ctl, (void*)b.barCount, (void*)b.barGen, (void*)b.info, (void*)b.actList,
                    (void*)b.slotF, (void*)b.slotFlags, (void*)b.slotSucc, (void*)b.slotDv, (void*)b.slotPhdt,
                    (void*)b.slotMax0, (void*)b.slotThr0, b.candK, (void*)b.candDepN, (void*)b.candPending,
                    (void*)b.candPm, (void*)b.readyQ})
        if (!p) return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (solver state)");
    if (h->ctrl.record_cut_faces && !h->cutMask) return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (cut mask)");
    CK(h, cudaMemsetAsync(h->nMixed, 0, sizeof(int), h->stream));
    CK(h, cudaMemsetAsync(h->devErr, 0, sizeof(uint32_t), h->stream));
    CK(h, cudaMemsetAsync(h->alphaPhi, 0, sizeof(double) * nf, h->stream));
    CK(h, cudaMemsetAsync(b.corr, 0, sizeof(double) * nf, h->stream));
    CK(h, cudaMemsetAsync(b.modStamp, 0xff, sizeof(int) * nf, h->stream));
    CK(h, cudaMemsetAsync(b.candMark, 0, sizeof(int) * nc, h->stream));
    CK(h, cudaMemsetAsync(b.cellClaim, 0, sizeof(int) * nc, h->stream));
    CK(h, cudaMemsetAsync(b.faceStamp, 0, sizeof(int) * nf, h->stream));
    CK(h, cudaMemsetAsync(b.readyQ, 0, sizeof(unsigned long long) * b.candCap, h->stream));
    CK(h, cudaMemsetAsync(b.barCount, 0, sizeof(unsigned), h->stream));
    CK(h, cudaMemsetAsync(b.barGen, 0, sizeof(unsigned), h->stream));
    CK(h, cudaMemsetAsync(b.info, 0, sizeof(int) * 8, h->stream));
    if (h->ctrl.orientation_method == SIMPLIC_ORIENTATION_ISO_RDF) {
        RdfBuffers& r = h->rdf;
        r.rdf = M.alloc<double>(nc);
        r.cellMix = M.alloc<int2>(nc);
        r.bandStamp = M.alloc<int>(nc);
        r.bandList = M.alloc<int>(nc);
        r.bandCount = M.alloc<int>(1);
        r.grad = M.alloc<double>(size_t(3) * nc);
        r.res = M.alloc<double>(nc);
        r.avgA = M.alloc<double>(nc);
        r.tooCoarse = M.alloc<uint8_t>(nc);
        r.stamp = 0;
        for (void* p : {(void*)r.rdf, (void*)r.cellMix, (void*)r.bandStamp, (void*)r.bandList, (void*)r.bandCount,
                        (void*)r.grad, (void*)r.res, (void*)r.avgA, (void*)r.tooCoarse})
            if (!p) return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (isoRDF buffers)");
        CK(h, cudaMemsetAsync(r.cellMix, 0, sizeof(int2) * nc, h->stream));
        CK(h, cudaMemsetAsync(r.bandStamp, 0, sizeof(int) * nc, h->stream));
    }
    return SIMPLIC_OK;
}

// calcInterfaceNFromIsoRDF (reconstruction.C:193-405): the device does the
// per-cell work; the stopping test -- sums over the mixed cells in
// ascending cell order, as the reference's loop adds them -- and the
// too-coarse flags are decided here, once per iteration.
int runIsoRDF(simplic_handle* h, const StepArgs& a) {
    RdfBuffers& r = h->rdf;
    r.stamp += 1;
    CK(h, cudaMemsetAsync(r.bandCount, 0, sizeof(int), h->stream));
    int32_t nm = 0;
    CK(h, cudaMemcpyAsync(&nm, h->nMixed, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    timedLaunch(h, kKRdf, [&] { launchRdfStart(a, r, h->stream); });
    CK(h, cudaStreamSynchronize(h->stream));
    h->lastRdfIterations = 0;
    if (nm == 0) return SIMPLIC_OK;
    std::vector<int32_t> cells(nm), order(nm);
    std::vector<double> res(nm), avgA(nm);
    std::vector<uint8_t> tooCoarse(nm, 0);
    CK(h, cudaMemcpyAsync(cells.data(), h->mixed, sizeof(int32_t) * nm, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    for (int i = 0; i < nm; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int x, int y) { return cells[x] < cells[y]; });
    const int iterations = h->ctrl.iso_rdf_iterations;
    for (int iter = 0; iter < iterations; ++iter) {
        timedLaunch(h, kKRdf, [&] { launchRdfNormals(a, r, h->stream); });
        timedLaunch(h, kKPlane, [&] { launchPlaneSolveSkip(a, r.tooCoarse, h->stream); });
        timedLaunch(h, kKRdf, [&] { launchRdfConstruct(a, r, h->stream); });
        timedLaunch(h, kKRdf, [&] { launchRdfResidual(a, r, h->stream); });
        CK(h, cudaGetLastError());
        CK(h, cudaMemcpyAsync(res.data(), r.res, sizeof(double) * nm, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaMemcpyAsync(avgA.data(), r.avgA, sizeof(double) * nm, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        int resCounter = 0;
        double avgRes = 0.0, avgNormRes = 0.0;
        bool changed = false;
        for (int q = 0; q < nm; ++q) {
            const int i = order[q];
            if (avgA[i] > 0.26 && iter > 0) {
                changed = changed || !tooCoarse[i];
                tooCoarse[i] = 1;
            } else {
                avgRes += res[i];
                const double discreteError = 0.01 * (avgA[i] * avgA[i]);
                const double normRes = discreteError != 0.0 ? res[i] / std::max(discreteError, h->ctrl.iso_rdf_tol)
                                                            : res[i] / h->ctrl.iso_rdf_tol;
                avgNormRes += normRes;
                ++resCounter;
            }
        }
        if (resCounter == 0) {
            resCounter = 1;
            avgRes = 0.0;
            avgNormRes = 0.0;
        }
        h->lastRdfIterations = iter + 1;
        if (((avgNormRes / resCounter < h->ctrl.iso_rdf_rel_tol || avgRes / resCounter < h->ctrl.iso_rdf_tol) &&
             iter >= 1) ||
            iter + 1 == iterations)
            break;
        if (changed)
            CK(h, cudaMemcpyAsync(r.tooCoarse, tooCoarse.data(), nm, cudaMemcpyHostToDevice, h->stream));
    }
    return SIMPLIC_OK;
}

int ensureStaging(simplic_handle* h) {
    if (h->sPhi) return SIMPLIC_OK;
    const int nc = h->m.nc, nf = h->m.nf;
    auto& M = h->mem;
    h->sPhi = M.alloc<double>(nf);
    h->sU = M.alloc<double>(size_t(3) * nc);
    h->sUb = M.alloc<double>(size_t(3) * std::max(1, h->nfb));
    h->sAlphaB = M.alloc<double>(std::max(1, h->nfb));
    h->sSp = M.alloc<double>(nc);
    h->sSu = M.alloc<double>(nc);
    if (!h->sPhi || !h->sU || !h->sUb || !h->sAlphaB || !h->sSp || !h->sSu)
        return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (input staging)");
    return SIMPLIC_OK;
}

// reconstruct on aBuf[cur] (device)
int runReconstruct(simplic_handle* h) {
    StepArgs a = baseArgs(h);
    a.aCur = h->aBuf[h->cur];
    if (h->eventsUsed >= 4096) collectTimers(h);
    const size_t evIdx = h->eventsUsed;
    nextEvents(h, 0);
    CK(h, cudaEventRecord(h->events[evIdx].a, h->stream));
    CK(h, cudaMemsetAsync(h->nMixed, 0, sizeof(int), h->stream));
    timedLaunch(h, kKScan, [&] { launchScanMixed(a, h->stream); });
    if (h->ctrl.precision == SIMPLIC_PRECISION_LEARNED) {
        if (!h->haveNet) return fail(h, SIMPLIC_ERR_STATE, "learned precision: no network loaded (simplic_set_network)");
        // the gather also writes the FP32 least-squares normal of the same
        // neighbourhood (the fallback), so no separate normal kernel runs
        cudaError_t ne = cudaSuccess;
        CK(h, cudaMemsetAsync(h->nLearned, 0, sizeof(int), h->stream));
        const int R = h->netRows;
        timedLaunch(h, kKNetInputs, [&] { launchGatherFeatures(a, R, h->netX, h->netA, h->stream); });
        timedLaunch(h, kKNetwork, [&] {
            ne = launchNetwork(h->netX, h->nMixed, R, h->netW, h->netB, h->netY, 16, h->devErr, h->stream);
        });
        timedLaunch(h, kKNetGate, [&] {
            launchLearnedGate(a, R, h->netX, h->netA, h->netY, 16, h->netGateTol, h->nLearned, h->stream);
        });
        CK(h, ne);
        timedLaunch(h, kKPlane, [&] { launchPlaneSolveMixed(a, h->stream); });
    } else if (h->ctrl.precision == SIMPLIC_PRECISION_MIXED) {
        timedLaunch(h, kKLs, [&] { launchLsNormalMixed(a, h->stream); });
        timedLaunch(h, kKPlane, [&] { launchPlaneSolveMixed(a, h->stream); });
    } else if (h->ctrl.orientation_method == SIMPLIC_ORIENTATION_ISO_RDF) {
        if (int r = runIsoRDF(h, a)) return r;
    } else {
        timedLaunch(h, kKLs, [&] { launchLsNormal(a, h->stream); });
        timedLaunch(h, kKPlane, [&] { launchPlaneSolve(a, h->stream); });
    }
    CK(h, cudaGetLastError());
    CK(h, cudaEventRecord(h->events[evIdx].b, h->stream));
    h->reconstructed = true;
    h->reconCount += 1;
    return SIMPLIC_OK;
}

// advect from aBuf[cur] into aBuf[1-cur]; in holds device pointers
int runAdvect(simplic_handle* h, const simplic_step_inputs* in, const double* aOld) {
    if (!h->reconstructed) return fail(h, SIMPLIC_ERR_STATE, "advect called before reconstruct");
    if (!(in->dt > 0.0) || !std::isfinite(in->dt)) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "dt must be > 0");
    if (!in->phi || !in->U) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "phi and U are required");
    StepArgs a = baseArgs(h);
    a.aCur = h->aBuf[h->cur];
    a.aOld = aOld ? aOld : h->aBuf[h->cur];
    a.aNew = h->aBuf[1 - h->cur];
    a.phi = in->phi;
    a.U = in->U;
    a.Ub = in->U_boundary;
    a.alphaB = in->alpha_boundary;
    a.Sp = in->Sp;
    a.Su = in->Su;
    a.dt = in->dt;
    a.rDeltaT = 1.0 / in->dt;
    a.rrDeltaT = 1.0 / a.rDeltaT;
    if (h->eventsUsed >= 4096) collectTimers(h);
    const size_t evIdx = h->eventsUsed;
    nextEvents(h, 1);
    CK(h, cudaEventRecord(h->events[evIdx].a, h->stream));
    if (a.cutMask) CK(h, cudaMemsetAsync(a.cutMask, 0, h->m.nf, h->stream));
    CK(h, cudaMemsetAsync(h->bb.ovCount, 0, 2 * sizeof(int), h->stream));
    CK(h, cudaMemsetAsync(h->dwCount, 0, sizeof(int), h->stream));
    CK(h, cudaMemsetAsync(h->bb.ctl, 0, sizeof(int) * kCtlSize, h->stream));
    CK(h, cudaMemsetAsync(h->bb.info, 0, sizeof(int) * 8, h->stream));
    // a barrier that timed out leaves its arrival count behind
    CK(h, cudaMemsetAsync(h->bb.barCount, 0, sizeof(unsigned), h->stream));
    if (h->ctrl.precision != SIMPLIC_PRECISION_PLAIN_FP64) {
        timedLaunch(h, kKFluxUn0, [&] { launchInterfaceUn0Mixed(a, h->stream); });
        timedLaunch(h, kKFluxFaces, [&] { launchInterfaceFacesMixed(a, h->stream); });
    } else {
        timedLaunch(h, kKFluxUn0, [&] { launchInterfaceUn0(a, h->stream); });
        timedLaunch(h, kKFluxFaces, [&] { launchInterfaceFaces(a, h->stream); });
    }
    timedLaunch(h, kKUpdate, [&] { launchUpdate(a, h->stream); });
    h->bb.stamp += 1;
    cudaError_t be = cudaSuccess;
    timedLaunch(h, kKBound, [&] { be = launchBound(a, h->bb, h->stream); });
    CK(h, be);
    if ((a.snapTol > 0.0) || a.clip) timedLaunch(h, kKBrute, [&] { launchBruteForce(a, h->stream); });
    CK(h, cudaGetLastError());
    CK(h, cudaEventRecord(h->events[evIdx].b, h->stream));
    h->cur = 1 - h->cur;
    h->reconstructed = false;
    return SIMPLIC_OK;
}

// The device address of a pinned (page-locked, mapped) host array, or NULL
// for pageable memory, which has to be copied.
const double* mappedHostPointer(const double* p) {
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (attr.type != cudaMemoryTypeHost || !attr.devicePointer) return nullptr;
    return static_cast<const double*>(attr.devicePointer);
}

int readStats(simplic_handle* h) {
    int32_t nm = 0, info[2] = {0, 0};
    CK(h, cudaMemcpyAsync(&nm, h->nMixed, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(info, h->bb.info, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->lastNMixed = nm;
    h->lastPasses = info[0];
    h->lastMaxBound = info[1];
    return SIMPLIC_OK;
}

}  // namespace

// Entry points without a handle report through simplic_last_error(NULL).
void simplic::setCreateError(const std::string& msg) { g_createError = msg; }

extern "C" {

void simplic_default_controls(simplic_controls* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->mixed_cell_tol = 1e-8;
    c->orientation_method = SIMPLIC_ORIENTATION_ISO_ALPHA_GRAD;
    c->split_warped_face = 0;
    c->n_alpha_bounds = 10;
    c->snap_tol = 0.0;
    c->clip = 1;
    c->write_plic_fields = 0;
    c->map_alpha_field = 0;
    c->precision = SIMPLIC_PRECISION_PLAIN_FP64;
    c->record_cut_faces = 0;
    c->iso_rdf_tol = 1e-6;
    c->iso_rdf_rel_tol = 0.1;
    c->iso_rdf_iterations = 5;
}

int simplic_create(const simplic_mesh_desc* mesh, const simplic_controls* controls, void* stream,
                   simplic_handle** out) {
    if (!out) return fail(nullptr, SIMPLIC_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!mesh) return fail(nullptr, SIMPLIC_ERR_INVALID_ARGUMENT, "mesh is NULL");
    simplic_controls ctrl;
    simplic_default_controls(&ctrl);
    if (controls) ctrl = *controls;
    if (ctrl.orientation_method != SIMPLIC_ORIENTATION_ISO_ALPHA_GRAD &&
        ctrl.orientation_method != SIMPLIC_ORIENTATION_ISO_RDF)
        return fail(nullptr, SIMPLIC_ERR_UNSUPPORTED,
                    "orientationMethod: isoAlphaGrad (LS) and isoRDF are implemented on the GPU");
    if (ctrl.orientation_method == SIMPLIC_ORIENTATION_ISO_RDF &&
        ctrl.precision != SIMPLIC_PRECISION_PLAIN_FP64)
        return fail(nullptr, SIMPLIC_ERR_UNSUPPORTED, "orientationMethod isoRDF needs the plain FP64 precision");
    if (ctrl.orientation_method == SIMPLIC_ORIENTATION_ISO_RDF &&
        (!(ctrl.iso_rdf_tol > 0.0) || !(ctrl.iso_rdf_rel_tol >= 0.0) || ctrl.iso_rdf_iterations < 1 ||
         ctrl.iso_rdf_iterations > 1000))
        return fail(nullptr, SIMPLIC_ERR_INVALID_ARGUMENT, "isoRDF controls out of range");
    if (ctrl.split_warped_face && ctrl.precision != SIMPLIC_PRECISION_PLAIN_FP64)
        return fail(nullptr, SIMPLIC_ERR_UNSUPPORTED, "splitWarpedFace needs the plain FP64 precision");
    if (ctrl.precision != SIMPLIC_PRECISION_PLAIN_FP64 && ctrl.precision != SIMPLIC_PRECISION_MIXED &&
        ctrl.precision != SIMPLIC_PRECISION_LEARNED)
        return fail(nullptr, SIMPLIC_ERR_INVALID_ARGUMENT, "unknown precision");
    if (!(ctrl.mixed_cell_tol >= 0.0 && ctrl.mixed_cell_tol < 0.5) || ctrl.n_alpha_bounds < 0 ||
        ctrl.n_alpha_bounds > kMaxBoundPasses)
        return fail(nullptr, SIMPLIC_ERR_INVALID_ARGUMENT, "controls out of range");
    std::unique_ptr<simplic_handle> h(new simplic_handle());
    h->ctrl = ctrl;
    if (const char* v = std::getenv("SIMPLIC_TEST_FAIL_ALLOC_AFTER")) h->mem.failAfter = std::atoll(v);
    // the mesh is checked and its addressing built on the host before any
    // device call, so a bad mesh is reported the same way with or without a GPU
    HostMesh hm;
    if (const int pr = prepareMesh(h.get(), mesh, hm)) {
        g_createError = h->err;
        return pr;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(nullptr, SIMPLIC_ERR_CUDA, "no CUDA device available");
    if (stream) {
        h->stream = static_cast<cudaStream_t>(stream);
    } else {
        if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
            return fail(nullptr, SIMPLIC_ERR_CUDA, "cudaStreamCreate failed");
        h->ownStream = true;
    }
    int r = uploadMesh(h.get(), mesh, hm);
    if (r == SIMPLIC_OK) r = allocState(h.get());
    if (r == SIMPLIC_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) {
        h->err = "mesh upload failed";
        r = SIMPLIC_ERR_CUDA;
    }
    if (r != SIMPLIC_OK) {
        g_createError = h->err;
        if (h->ownStream) cudaStreamDestroy(h->stream);
        return r;
    }
    *out = h.release();
    return SIMPLIC_OK;
}

int simplic_destroy(simplic_handle* h) {
    if (!h) return SIMPLIC_OK;
    cudaStreamSynchronize(h->stream);
    if (h->plicPts) cudaFree(h->plicPts);
    if (h->plicCount) cudaFree(h->plicCount);
    for (auto& e : h->events) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    const bool own = h->ownStream;
    cudaStream_t s = h->stream;
    delete h;
    if (own) cudaStreamDestroy(s);
    return SIMPLIC_OK;
}

const char* simplic_last_error(const simplic_handle* h) { return h ? h->err.c_str() : g_createError.c_str(); }

int simplic_set_alpha(simplic_handle* h, const double* alpha, int32_t mem) {
    if (!h || !alpha) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    CK(h, cudaMemcpyAsync(h->aBuf[h->cur], alpha, sizeof(double) * h->m.nc,
                          mem == SIMPLIC_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    h->haveAlpha = true;
    h->reconstructed = false;
    return SIMPLIC_OK;
}

int simplic_reconstruct_resident(simplic_handle* h) {
    if (!h) return SIMPLIC_ERR_INVALID_ARGUMENT;
    if (!h->haveAlpha) return fail(h, SIMPLIC_ERR_STATE, "no alpha loaded");
    return runReconstruct(h);
}

int simplic_advect_resident(simplic_handle* h, const simplic_step_inputs* in) {
    if (!h || !in) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    return runAdvect(h, in, nullptr);
}

const double* simplic_alpha_device(const simplic_handle* h) { return h ? h->aBuf[h->cur] : nullptr; }

int simplic_get_alpha(simplic_handle* h, double* out, int32_t mem) {
    if (!h || !out) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    CK(h, cudaMemcpyAsync(out, h->aBuf[h->cur], sizeof(double) * h->m.nc,
                          mem == SIMPLIC_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
    if (mem != SIMPLIC_MEM_DEVICE) CK(h, cudaStreamSynchronize(h->stream));
    return SIMPLIC_OK;
}

int simplic_synchronize(simplic_handle* h) {
    if (!h) return SIMPLIC_ERR_INVALID_ARGUMENT;
    CK(h, cudaStreamSynchronize(h->stream));
    return checkDeviceErrors(h);
}

int simplic_reconstruct(simplic_handle* h, const double* alpha) {
    if (!h || !alpha) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    int r = simplic_set_alpha(h, alpha, SIMPLIC_MEM_HOST);
    if (r) return r;
    if ((r = runReconstruct(h))) return r;
    return checkDeviceErrors(h);
}

int simplic_advect(simplic_handle* h, double* alpha, const double* alpha_old, const simplic_step_inputs* in) {
    if (!h || !alpha || !in) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!in->phi || !in->U) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "phi and U are required");
    int r = ensureStaging(h);
    if (r) return r;
    const int nc = h->m.nc, nf = h->m.nf, nfb = h->nfb;
    cudaStream_t s = h->stream;
    if (!(in->flags & SIMPLIC_ALPHA_UNCHANGED)) {
        const bool was = h->reconstructed;
        CK(h, cudaMemcpyAsync(h->aBuf[h->cur], alpha, sizeof(double) * nc, cudaMemcpyHostToDevice, s));
        h->reconstructed = was;
    }
    const double* aOld = nullptr;
    if (alpha_old) {
        CK(h, cudaMemcpyAsync(h->aOldBuf, alpha_old, sizeof(double) * nc, cudaMemcpyHostToDevice, s));
        aOld = h->aOldBuf;
    }
    simplic_step_inputs d = *in;
    CK(h, cudaMemcpyAsync(h->sPhi, in->phi, sizeof(double) * nf, cudaMemcpyHostToDevice, s));
    d.phi = h->sPhi;
    // U and U_boundary are read only around the interface (the velocity at
    // the interface centres of the cut cells): pinned host arrays are read
    // in place by those kernels, others are copied
    if (const double* du = mappedHostPointer(in->U)) {
        d.U = du;
    } else {
        CK(h, cudaMemcpyAsync(h->sU, in->U, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, s));
        d.U = h->sU;
    }
    if (in->U_boundary) {
        if (const double* db = mappedHostPointer(in->U_boundary)) {
            d.U_boundary = db;
        } else {
            CK(h, cudaMemcpyAsync(h->sUb, in->U_boundary, sizeof(double) * 3 * nfb, cudaMemcpyHostToDevice, s));
            d.U_boundary = h->sUb;
        }
    }
    if (in->alpha_boundary) {
        CK(h, cudaMemcpyAsync(h->sAlphaB, in->alpha_boundary, sizeof(double) * nfb, cudaMemcpyHostToDevice, s));
        d.alpha_boundary = h->sAlphaB;
    }
    if (in->Sp) {
        CK(h, cudaMemcpyAsync(h->sSp, in->Sp, sizeof(double) * nc, cudaMemcpyHostToDevice, s));
        d.Sp = h->sSp;
    }
    if (in->Su) {
        CK(h, cudaMemcpyAsync(h->sSu, in->Su, sizeof(double) * nc, cudaMemcpyHostToDevice, s));
        d.Su = h->sSu;
    }
    if ((r = runAdvect(h, &d, aOld))) return r;
    CK(h, cudaMemcpyAsync(alpha, h->aBuf[h->cur], sizeof(double) * nc, cudaMemcpyDeviceToHost, s));
    return checkDeviceErrors(h);
}

int simplic_get_mixed_cells(simplic_handle* h, int32_t* n, int32_t* cells, int32_t* status) {
    if (!h || !n) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    int r = readStats(h);
    if (r) return r;
    const int nm = h->lastNMixed;
    *n = nm;
    if (!cells && !status) return SIMPLIC_OK;
    std::vector<int32_t> c(nm);
    std::vector<int8_t> st(nm);
    if (nm) {
        CK(h, cudaMemcpyAsync(c.data(), h->mixed, sizeof(int32_t) * nm, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaMemcpyAsync(st.data(), h->mStatus, nm, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    std::vector<int32_t> order(nm);
    for (int i = 0; i < nm; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return c[a] < c[b]; });
    for (int i = 0; i < nm; ++i) {
        if (cells) cells[i] = c[order[i]];
        if (status) status[i] = st[order[i]];
    }
    return SIMPLIC_OK;
}

int simplic_get_interface(simplic_handle* h, double* n, double* d, double* c, double* s) {
    if (!h) return SIMPLIC_ERR_INVALID_ARGUMENT;
    int r = readStats(h);
    if (r) return r;
    const int nm = h->lastNMixed, nc = h->m.nc;
    std::vector<int32_t> cells(nm);
    std::vector<double> vn(3 * size_t(nm)), vd(nm), vc(3 * size_t(nm)), vs(3 * size_t(nm));
    if (nm) {
        CK(h, cudaMemcpyAsync(cells.data(), h->mixed, sizeof(int32_t) * nm, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaMemcpyAsync(vn.data(), h->nrm, sizeof(double) * 3 * nm, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaMemcpyAsync(vd.data(), h->dArr, sizeof(double) * nm, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaMemcpyAsync(vc.data(), h->icArr, sizeof(double) * 3 * nm, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaMemcpyAsync(vs.data(), h->isArr, sizeof(double) * 3 * nm, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    if (n) std::fill(n, n + 3 * size_t(nc), 0.0);
    if (d) std::fill(d, d + nc, 0.0);
    if (c) std::fill(c, c + 3 * size_t(nc), 0.0);
    if (s) std::fill(s, s + 3 * size_t(nc), 0.0);
    for (int i = 0; i < nm; ++i) {
        const int64_t cc = cells[i];
        for (int k = 0; k < 3; ++k) {
            if (n) n[3 * cc + k] = vn[3 * size_t(i) + k];
            if (c) c[3 * cc + k] = vc[3 * size_t(i) + k];
            if (s) s[3 * cc + k] = vs[3 * size_t(i) + k];
        }
        if (d) d[cc] = vd[i];
    }
    return SIMPLIC_OK;
}

int simplic_get_alpha_phi(simplic_handle* h, double* out, int32_t mem) {
    if (!h || !out) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    CK(h, cudaMemcpyAsync(out, h->alphaPhi, sizeof(double) * h->m.nf,
                          mem == SIMPLIC_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return SIMPLIC_OK;
}

}  // extern "C"

namespace {
__global__ void kRhoPhi(int nf, double a, double b, const double* __restrict__ aphi, const double* __restrict__ phi,
                        double* __restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < nf) out[f] = a * aphi[f] + b * phi[f];
}
}  // namespace

extern "C" {

int simplic_get_rho_phi(simplic_handle* h, double rho1, double rho2, const double* phi, double* out, int32_t mem) {
    if (!h || !phi || !out) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    const int nf = h->m.nf;
    const double* dPhi = phi;
    double* dOut = out;
    if (mem != SIMPLIC_MEM_DEVICE) {
        int r = ensureStaging(h);
        if (r) return r;
        if (!h->scratchF) {
            h->scratchF = h->mem.alloc<double>(nf);
            if (!h->scratchF) return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed");
        }
        CK(h, cudaMemcpyAsync(h->sPhi, phi, sizeof(double) * nf, cudaMemcpyHostToDevice, h->stream));
        dPhi = h->sPhi;
        dOut = h->scratchF;
    }
    kRhoPhi<<<(nf + 255) / 256, 256, 0, h->stream>>>(nf, rho1 - rho2, rho2, h->alphaPhi, dPhi, dOut);
    CK(h, cudaGetLastError());
    if (mem != SIMPLIC_MEM_DEVICE)
        CK(h, cudaMemcpyAsync(out, dOut, sizeof(double) * nf, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return SIMPLIC_OK;
}

int simplic_get_face_flatness(simplic_handle* h, double* out) {
    if (!h || !out) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    CK(h, cudaMemcpyAsync(out, h->m.flat, sizeof(double) * h->m.nf, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return SIMPLIC_OK;
}

int simplic_get_cut_faces(simplic_handle* h, uint8_t* mask) {
    if (!h || !mask) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!h->cutMask) return fail(h, SIMPLIC_ERR_STATE, "record_cut_faces was not enabled");
    CK(h, cudaMemcpyAsync(mask, h->cutMask, h->m.nf, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return SIMPLIC_OK;
}

int simplic_timers(simplic_handle* h, double* rec, double* adv, double* mapping) {
    if (!h) return SIMPLIC_ERR_INVALID_ARGUMENT;
    CK(h, cudaStreamSynchronize(h->stream));
    collectTimers(h);
    if (rec) *rec = h->tRecon;
    if (adv) *adv = h->tAdv;
    if (mapping) *mapping = h->tMap;
    return SIMPLIC_OK;
}

int simplic_set_kernel_timing(simplic_handle* h, int32_t enable) {
    if (!h) return SIMPLIC_ERR_INVALID_ARGUMENT;
    h->kernelTiming = enable != 0;
    return SIMPLIC_OK;
}

int simplic_kernel_times(simplic_handle* h, double* total_ms, int64_t* launches, const char** names) {
    if (!h) return SIMPLIC_ERR_INVALID_ARGUMENT;
    CK(h, cudaStreamSynchronize(h->stream));
    collectTimers(h);
    for (int k = 0; k < kNumKernels; ++k) {
        if (total_ms) total_ms[k] = h->kMs[k];
        if (launches) launches[k] = h->kLaunches[k];
        if (names) names[k] = kKernelNames[k];
    }
    return SIMPLIC_OK;
}

int simplic_reset_kernel_times(simplic_handle* h) {
    if (!h) return SIMPLIC_ERR_INVALID_ARGUMENT;
    CK(h, cudaStreamSynchronize(h->stream));
    collectTimers(h);
    for (int k = 0; k < kNumKernels; ++k) {
        h->kMs[k] = 0.0;
        h->kLaunches[k] = 0;
    }
    return SIMPLIC_OK;
}

int simplic_bound_info(simplic_handle* h, int32_t* info) {
    if (!h || !info) return SIMPLIC_ERR_INVALID_ARGUMENT;
    int32_t in[4];
    CK(h, cudaMemcpyAsync(in, h->bb.info, sizeof(in), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    for (int k = 0; k < 4; ++k) info[k] = in[k];
    return SIMPLIC_OK;
}

int simplic_bound_profile(simplic_handle* h, int32_t* info) {
    if (!h || !info) return SIMPLIC_ERR_INVALID_ARGUMENT;
    int32_t in[8];
    CK(h, cudaMemcpyAsync(in, h->bb.info, sizeof(in), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    for (int k = 0; k < 4; ++k) info[k] = in[4 + k];
    return SIMPLIC_OK;
}

int simplic_map_alpha_field(simplic_handle* h, double* alpha, const double* normal, const double* distance,
                            double lower, double upper, int32_t mem) {
    if (!h || !alpha || !normal || !distance) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    const int nc = h->m.nc;
    double *a = const_cast<double*>(alpha), *n = const_cast<double*>(normal), *d = const_cast<double*>(distance);
    if (mem != SIMPLIC_MEM_DEVICE) {
        // host arrays go through a device scratch of five cell fields
        if (!h->mapScratch) {
            h->mapScratch = h->mem.alloc<double>(size_t(5) * nc);
            if (!h->mapScratch) return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (map scratch)");
        }
        a = h->mapScratch;
        n = h->mapScratch + nc;
        d = h->mapScratch + 4 * size_t(nc);
        CK(h, cudaMemcpyAsync(a, alpha, sizeof(double) * nc, cudaMemcpyHostToDevice, h->stream));
        CK(h, cudaMemcpyAsync(n, normal, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, h->stream));
        CK(h, cudaMemcpyAsync(d, distance, sizeof(double) * nc, cudaMemcpyHostToDevice, h->stream));
    }
    if (h->eventsUsed >= 4096) collectTimers(h);
    const size_t evIdx = h->eventsUsed;
    nextEvents(h, kMapTimer);
    CK(h, cudaEventRecord(h->events[evIdx].a, h->stream));
    launchMapAlpha(h->m, a, n, d, lower, upper, h->devErr, h->stream);
    CK(h, cudaGetLastError());
    CK(h, cudaEventRecord(h->events[evIdx].b, h->stream));
    if (mem != SIMPLIC_MEM_DEVICE)
        CK(h, cudaMemcpyAsync(alpha, a, sizeof(double) * nc, cudaMemcpyDeviceToHost, h->stream));
    return checkDeviceErrors(h);
}

int simplic_get_interface_polygons(simplic_handle* h, int32_t* n_polys, int32_t* n_points, int32_t* offsets,
                                   double* points, int32_t* cells) {
    if (!h || !n_polys || !n_points) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    if (h->reconCount == 0) return fail(h, SIMPLIC_ERR_STATE, "no reconstruct yet");
    if (h->plicOf != h->reconCount) {
        int r = readStats(h);
        if (r) return r;
        const int nm = h->lastNMixed;
        constexpr int kStride = 64;
        if (nm > h->plicCap) {
            if (h->plicPts) cudaFree(h->plicPts);
            if (h->plicCount) cudaFree(h->plicCount);
            h->plicPts = nullptr;
            h->plicCount = nullptr;
            h->plicCap = 0;
            CK(h, cudaMalloc(&h->plicPts, sizeof(double) * 3 * kStride * size_t(nm)));
            CK(h, cudaMalloc(&h->plicCount, sizeof(int) * size_t(nm)));
            h->plicCap = nm;
        }
        std::vector<int32_t> cnt(nm), mcells(nm);
        std::vector<double> pts(size_t(nm) * 3 * kStride);
        if (nm) {
            StepArgs a = baseArgs(h);
            launchPlicPolygons(a, kStride, h->plicPts, h->plicCount, h->stream);
            CK(h, cudaGetLastError());
            CK(h, cudaMemcpyAsync(cnt.data(), h->plicCount, sizeof(int) * nm, cudaMemcpyDeviceToHost, h->stream));
            CK(h, cudaMemcpyAsync(mcells.data(), h->mixed, sizeof(int) * nm, cudaMemcpyDeviceToHost, h->stream));
            CK(h, cudaMemcpyAsync(pts.data(), h->plicPts, sizeof(double) * pts.size(), cudaMemcpyDeviceToHost,
                                  h->stream));
        }
        if ((r = checkDeviceErrors(h))) return r;
        std::vector<int32_t> order(nm);
        for (int i = 0; i < nm; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](int x, int y) { return mcells[x] < mcells[y]; });
        h->plicOffsets.assign(1, 0);
        h->plicCells.clear();
        h->plicPoints.clear();
        for (int i : order) {
            if (cnt[i] == 0) continue;
            h->plicCells.push_back(mcells[i]);
            h->plicPoints.insert(h->plicPoints.end(), pts.begin() + size_t(i) * 3 * kStride,
                                 pts.begin() + (size_t(i) * kStride + cnt[i]) * 3);
            h->plicOffsets.push_back(h->plicOffsets.back() + cnt[i]);
        }
        h->plicOf = h->reconCount;
    }
    *n_polys = int32_t(h->plicCells.size());
    *n_points = h->plicOffsets.back();
    if (offsets) std::copy(h->plicOffsets.begin(), h->plicOffsets.end(), offsets);
    if (points) std::copy(h->plicPoints.begin(), h->plicPoints.end(), points);
    if (cells) std::copy(h->plicCells.begin(), h->plicCells.end(), cells);
    return SIMPLIC_OK;
}

int simplic_rdf_iterations(simplic_handle* h, int32_t* n) {
    if (!h || !n) return SIMPLIC_ERR_INVALID_ARGUMENT;
    *n = h->lastRdfIterations;
    return SIMPLIC_OK;
}

int simplic_mesh_info(simplic_handle* h, int32_t* info) {
    if (!h || !info) return SIMPLIC_ERR_INVALID_ARGUMENT;
    info[0] = h->m.uniformFaces;
    info[1] = h->m.latNx;
    info[2] = h->m.latNy;
    info[3] = h->m.latNz;
    info[4] = h->nBoxCells;
    return SIMPLIC_OK;
}

int simplic_stats(simplic_handle* h, int32_t* n_mixed, int32_t* passes, int32_t* max_bound) {
    if (!h) return SIMPLIC_ERR_INVALID_ARGUMENT;
    int r = readStats(h);
    if (r) return r;
    if (n_mixed) *n_mixed = h->lastNMixed;
    if (passes) *passes = h->lastPasses;
    if (max_bound) *max_bound = h->lastMaxBound;
    return SIMPLIC_OK;
}

// --- learned-normal network (include/simplic_mlp.h) ---

int simplic_set_network(simplic_handle* h, const float* W, const float* b, float gate_tol) {
    if (!h || !W || !b) return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "NULL argument");
    const int nc = h->m.nc;
    if (!h->netW) {
        // rows of the network: the mixed cells of a step, up to 1/8 of the
        // mesh (at least 2^20); cells beyond keep their least-squares normal
        // rows for up to 1/32 of the cells (at least 2^18): interface cells are a
        // few percent at most; any beyond keep their least-squares normal
        const int rows = std::min(nc, std::max(1 << 18, nc / 32));
        h->netRows = rows;
        h->netW = h->mem.alloc<__nv_bfloat16>(size_t(4) * 128 * 128);
        h->netB = h->mem.alloc<float>(4 * 128);
        h->netX = h->mem.alloc<__nv_bfloat16>(size_t(rows) * 128);
        h->netA = h->mem.alloc<float>(size_t(rows) * 32);
        h->netY = h->mem.alloc<float>(size_t(rows) * 16);
        h->nLearned = h->mem.alloc<int>(1);
        if (!h->netW || !h->netB || !h->netX || !h->netA || !h->netY || !h->nLearned)
            return fail(h, SIMPLIC_ERR_CUDA, "cudaMalloc failed (network buffers)");
        CK(h, cudaMemsetAsync(h->nLearned, 0, sizeof(int), h->stream));
    }
    std::vector<__nv_bfloat16> wb(size_t(4) * 128 * 128);
    for (size_t i = 0; i < wb.size(); ++i) wb[i] = __float2bfloat16(W[i]);
    CK(h, cudaMemcpyAsync(h->netW, wb.data(), wb.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->netB, b, 4 * 128 * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->netGateTol = gate_tol;
    h->haveNet = true;
    return SIMPLIC_OK;
}

int simplic_network_stats(simplic_handle* h, int32_t* n_learned) {
    if (!h || !n_learned) return SIMPLIC_ERR_INVALID_ARGUMENT;
    *n_learned = 0;
    if (!h->nLearned) return SIMPLIC_OK;
    CK(h, cudaMemcpyAsync(n_learned, h->nLearned, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return SIMPLIC_OK;
}

int simplic_network_info(simplic_handle* h, int32_t* info) {
    if (!h || !info) return SIMPLIC_ERR_INVALID_ARGUMENT;
    int r = simplic_network_stats(h, &info[0]);
    if (r) return r;
    if ((r = readStats(h))) return r;
    info[1] = h->netRows;
    info[2] = h->haveNet ? std::max(0, h->lastNMixed - h->netRows) : 0;
    return SIMPLIC_OK;
}

int simplic_network_inputs(simplic_handle* h, int32_t max_rows, int32_t* rows, int32_t* cells, void* X, float* A) {
    if (!h || !rows || max_rows < 0 || (max_rows > 0 && (!X || !cells))) return SIMPLIC_ERR_INVALID_ARGUMENT;
    *rows = 0;
    if (!h->haveNet) return fail(h, SIMPLIC_ERR_STATE, "no network set");
    int r = readStats(h);
    if (r) return r;
    // rows exist for the first netRows entries of the (unordered) mixed list
    const int n = std::min(h->lastNMixed, h->netRows);
    std::vector<int32_t> c(n);
    std::vector<uint16_t> x(size_t(n) * 128);
    std::vector<float> al(A ? size_t(n) * 32 : 0);
    if (n > 0) {
        CK(h, cudaMemcpyAsync(c.data(), h->mixed, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaMemcpyAsync(x.data(), h->netX, x.size() * sizeof(uint16_t), cudaMemcpyDeviceToHost, h->stream));
        if (A) CK(h, cudaMemcpyAsync(al.data(), h->netA, al.size() * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    }
    CK(h, cudaStreamSynchronize(h->stream));
    std::vector<int32_t> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return c[a] < c[b]; });
    const int m = std::min(n, max_rows);
    for (int i = 0; i < m; ++i) {
        cells[i] = c[order[i]];
        std::memcpy(static_cast<uint16_t*>(X) + size_t(i) * 128, x.data() + size_t(order[i]) * 128,
                    128 * sizeof(uint16_t));
        if (A) std::memcpy(A + size_t(i) * 32, al.data() + size_t(order[i]) * 32, 32 * sizeof(float));
    }
    *rows = m;
    return SIMPLIC_OK;
}

int simplic_mlp_samples(simplic_handle* h, uint64_t seed, int32_t count, int32_t sphere_percent, void* X,
                        float* T) {
    if (!h || !X || !T || count <= 0 || sphere_percent < 0 || sphere_percent > 100)
        return fail(h, SIMPLIC_ERR_INVALID_ARGUMENT, "bad sample arguments");
    launchMakeSamples(h->m, seed, count, sphere_percent, X, T, h->devErr, h->stream);
    CK(h, cudaGetLastError());
    return SIMPLIC_OK;
}

}  // extern "C"
