// Launch interface between the C-ABI layer and the kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "simplic_device.cuh"

namespace simplic {

void setCreateError(const std::string& msg);

// Pointers of one reconstruct / advect call (device memory).
struct StepArgs {
    DevMesh m;
    // alpha
    const double* aCur;   // alpha used for classification and upwind fluxes
    const double* aOld;   // alpha.oldTime()
    double* aNew;         // output of advect
    // per-step inputs
    const double* phi;
    const double* U;
    const double* Ub;
    const double* alphaB;
    const double* Sp;
    const double* Su;
    double dt, rDeltaT;
    double rrDeltaT;      // 1 / rDeltaT (the reciprocal of the update's divisor)
    // controls
    double mixedTol, snapTol;
    int clip, nAlphaBounds;
    // reconstruction state (compact, indexed by position in the mixed list)
    int8_t* status;   // [nc]
    int* mixed;       // [nc]
    int* nMixed;      // [1]
    double* nrm;      // [3 nc]
    int8_t* mStatus;  // [nc]
    double* dArr;     // [nc]
    double* icArr;    // [3 nc]
    double* isArr;    // [3 nc]
    // advection state
    double* dvfI;       // [nf] Simpson dVf of faces downwind of cut cells
    double* alphaPhi;   // [nf]
    uint8_t* cutMask;   // [nf] optional record of Simpson faces
    double* un0;        // [nc] interface normal speed of cut cells
    int2* dwList;       // [nf] (mixed index, face) of every downwind face of a cut cell
    int* dwCount;
    int* ovList;        // cells the update left outside [-aTol, 1+aTol]
    int* ovCount;
    int ovCap;
    uint32_t* err;      // device error bits
};

// Polls of the bounding kernel's grid barrier before it gives up: about 1-2 s
// with 64 ns sleeps, far beyond any wait of a working launch.
constexpr long long kBarrierSpins = 20000000;

// Bounding kernel limits and the layout of its per-step control counters.
constexpr int kMaxBoundPasses = 64;   // nAlphaBounds cap
enum : int {
    kCtlCand = 0,     // candidates so far
    kCtlMod = 1,      // faces whose dVf the bounding changed
    kCtlActive0 = 4,  // [pass] overshooting candidates
    kCtlOverDelta0 = kCtlActive0 + kMaxBoundPasses,  // [pass] change of the overshoot count
    kCtlTouched0 = kCtlOverDelta0 + kMaxBoundPasses, // [pass] target cells of the pass
    kCtlQHead0 = kCtlTouched0 + kMaxBoundPasses,     // [pass] ready-queue entries taken
    kCtlQTail0 = kCtlQHead0 + kMaxBoundPasses,       // [pass] ready-queue entries written
    kCtlDone0 = kCtlQTail0 + kMaxBoundPasses,        // [pass] cells run
    kCtlStarts0 = kCtlDone0 + kMaxBoundPasses,       // [pass] chains started from the queue
    kCtlSize = kCtlStarts0 + kMaxBoundPasses,
};
constexpr int kBoundCellConstBytes = 104;  // per-candidate constants of the cell loop

// Scratch of the bounding kernel (per-candidate arrays have candCap rows,
// the per-face-slot ones maxCellFaces columns: slot i * maxCellFaces + k is
// the k-th face of candidate i in cells() order).
struct BoundBuffers {
    int* ovList;
    int* ovCount;
    int ovCap;
    int* cand;
    int candCap;
    int* candIdx;      // [nc] position of a candidate cell
    int* candMark;     // [nc] step stamp: cell is a candidate
    int* cellClaim;    // [nc] pass stamp: target already updated
    unsigned* faceKey; // [nf] list position key of a corrected face (cell * 32 + position)
    int* faceStamp;    // [nf] pass stamp of faceKey
    int* touched;
    int touchedCap;
    double* corr;      // [nf], zero outside a pass
    double* dvfMod;    // [nf] dVf of faces the bounding changed
    int* modStamp;     // [nf] step stamp of dvfMod
    int* modList;
    int modCap;
    int* ctl;          // [kCtlSize] counters, zeroed before every launch
    unsigned* barCount;    // zeroed before every launch
    unsigned* barGen;
    long long spinLimit;   // polls before a bounded wait gives up (kBarrierSpins)
    int barrierExtra;      // arrivals a barrier waits for beyond the grid (test setting; 0)
    int stamp;
    int* info;  // [0] passes run, [1] most cells bounded in a pass, [2] most chains started
                // from the ready queue in a pass, [3] overflow code, [4] most cells one warp
                // ran in a row along a chain, [5] cells run in all passes, [6] us in the
                // dependency phases, [7] us of the launch ([6], [7] on block 0's clock)
    // The overshooting candidates of the current pass with everything their
    // loop needs that reads no correction, computed before the dependency
    // phase (per face slot and per cell), the dependency counts and the
    // ready queue.
    int* actList;          // [candCap] overshooting candidates of the pass
    int* slotF;            // [slots] face id
    uint8_t* slotFlags;    // [slots] kSlot* bits
    int* slotSucc;         // [slots] later overshooting candidate across a downwind face, or -1
    double* slotDv;        // [slots] dVf at the start of the pass
    double* slotPhdt;      // [slots] phi dt
    double* slotMax0;      // [slots] first iteration without corrections: maxExtra
    double* slotThr0;      // [slots] ... and the flux share
    void* candK;           // [candCap * kBoundCellConstBytes] per-cell constants
    int* candDepN;         // [candCap] faces on which the cell waits for an earlier cell
    int* candPending;      // [candCap] of those, not yet published
    unsigned* candPm;      // [candCap] faces that pass in the loop's first iteration
    unsigned long long* readyQ;  // [candCap] (pass stamp << 32) | candidate
};

// arguments of the three plane-solve kernels
struct PlaneArgs {
    const double* alpha;
    const int* mixed;
    const int* nMixed;
    const double* nrm;
    int8_t* mStatus;
    int8_t* status;
    double* dOut;
    double* icOut;
    double* isOut;
    uint32_t* err;
    const uint8_t* skip;  // optional per mixed cell: nonzero keeps the previous plane (isoRDF)
};

// Buffers of the isoRDF orientation (reconstruction.C:193-405), allocated
// when a handle is created with that method.
struct RdfBuffers {
    double* rdf;        // [nc] reconstructed distance function
    int2* cellMix;      // [nc] (stamp, position in the mixed list) of a mixed cell
    int* bandStamp;     // [nc] stamp: the cell is in the band
    int* bandList;      // [nc] band cells
    int* bandCount;     // [1]
    double* grad;       // [3 nc] per mixed position: the gradient being iterated
    double* res;        // [nc] per mixed position: normal residual
    double* avgA;       // [nc] per mixed position: mean angle to the neighbours' normals
    uint8_t* tooCoarse; // [nc] per mixed position
    int stamp;
};

void launchScanMixed(const StepArgs& a, cudaStream_t st);
// isoRDF: band, cell -> mixed position map, alpha gradient (start); then per
// iteration: normals from the gradient, the plane solve of the cells not
// too coarse, the distance function on the band, its gradient and the
// residuals
void launchRdfStart(const StepArgs& a, const RdfBuffers& r, cudaStream_t st);
void launchRdfNormals(const StepArgs& a, const RdfBuffers& r, cudaStream_t st);
void launchPlaneSolveSkip(const StepArgs& a, const uint8_t* skip, cudaStream_t st);
void launchRdfConstruct(const StepArgs& a, const RdfBuffers& r, cudaStream_t st);
void launchRdfResidual(const StepArgs& a, const RdfBuffers& r, cudaStream_t st);
// PLIC polygon of every mixed cell: up to `stride` points at pts[3 stride i],
// count[i] points (0 where the plane does not cut the cell)
void launchPlicPolygons(const StepArgs& a, int stride, double* pts, int* count, cudaStream_t st);
// alpha = cut volume fraction of the given plane where lower <= alpha <= upper
void launchMapAlpha(const DevMesh& m, double* alpha, const double* normal, const double* distance, double lower,
                    double upper, uint32_t* err, cudaStream_t st);
void launchLsNormal(const StepArgs& a, cudaStream_t st);
void launchPlaneSolve(const StepArgs& a, cudaStream_t st);
void launchInterfaceUn0(const StepArgs& a, cudaStream_t st);
void launchInterfaceFaces(const StepArgs& a, cudaStream_t st);
void launchUpdate(const StepArgs& a, cudaStream_t st);
cudaError_t launchBound(const StepArgs& a, const BoundBuffers& b, cudaStream_t st);
void launchBruteForce(const StepArgs& a, cudaStream_t st);
void launchFaceFlatness(const DevMesh& m, const double* Sf, double* flat, cudaStream_t st);
void launchFaceFull(const DevMesh& m, double* fullC, double* fullA, cudaStream_t st);
void launchRecipVolume(const DevMesh& m, double* rV, cudaStream_t st);
// LS stencil rows of all cells: lengths (count) or the rows at off
void launchStencilRows(const DevMesh& m, bool count, int* len, const int* off, int* rows, cudaStream_t st);
// mixed-precision form (FP32 normals and Simpson clipping, FP64 volume matching)
void launchLsNormalMixed(const StepArgs& a, cudaStream_t st);
void launchPlaneSolveMixed(const StepArgs& a, cudaStream_t st);
void launchInterfaceUn0Mixed(const StepArgs& a, cudaStream_t st);
void launchInterfaceFacesMixed(const StepArgs& a, cudaStream_t st);
// learned-normal form (the mixed form with the network's normals)
void launchMakeSamples(const DevMesh& m, unsigned long long seed, int count, int spherePct, void* X, float* T,
                       uint32_t* err, cudaStream_t st);
// network inputs of the first maxRows mixed cells, their alphas in FP32
// (A: [row][32], alpha_c then alpha_j - alpha_c per slot), and the FP32
// least-squares normal of every mixed cell (written to a.nrm); the cells
// from maxRows on get no row
void launchGatherFeatures(const StepArgs& a, int maxRows, void* X, float* A, cudaStream_t st);
cudaError_t launchNetwork(const void* X, const int* Mdev, int maxRows, const void* W, const float* bias, float* Y,
                          int ldy, uint32_t* err, cudaStream_t st);
// the learned form's choice per network row: normalise(n_ls + y[0:3]) (n_ls
// from the row's input) unless degenerate or its local volume residual or
// face-flux mismatch exceeds the least-squares normal's by more than
// gateTol; nLearned counts the choices
void launchLearnedGate(const StepArgs& a, int maxRows, const void* X, const float* A, const float* Y, int ldY,
                       float gateTol, int* nLearned, cudaStream_t st);

}  // namespace simplic
