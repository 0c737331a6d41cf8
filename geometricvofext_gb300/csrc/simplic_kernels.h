// Launch interface between the C-ABI layer and the kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include "simplic_device.cuh"

namespace simplic {

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
    double* lvVof;      // [kLvSlots nc] VOF of the interior vertex levels
    double* v13;        // [2 nc] VOF at the 1/3 and 2/3 plane constants
    int8_t* done;       // [nc] plane found before the cubic step
    double* un0;        // [nc] interface normal speed of cut cells
    double* blkMin;     // [ceil(nc/256)]
    double* blkMax;
    int* ovList;        // cells the update left outside [-aTol, 1+aTol]
    int* ovCount;
    int ovCap;
    uint32_t* err;      // device error bits
};

// Scratch of the bounding kernel (per-candidate arrays have candCap rows,
// the per-face ones kMaxCellFaces columns).
struct BoundBuffers {
    int* ovList;
    int* ovCount;
    int ovCap;
    int* cand;
    int candCap;
    int* candLevel;
    int* candDeps;
    int* candNDeps;
    int* candCorr;
    int* candNCorr;
    int* candWritten;
    int* candNWritten;
    int* candListOff;
    int* list;
    long long* rec;
    int recCap;
    double* corr;      // [nf], zero outside a pass
    double* dvfMod;    // [nf] dVf of faces the bounding changed
    int* modStamp;     // [nf] step stamp of dvfMod
    int* modList;
    int* modCount;
    int modCap;
    int stamp;
    int* info;  // [0] passes run, [1] most cells bounded in a pass, [2] deepest level count
    long long* prof;  // [8] SM cycles per phase of the bounding kernel (summed)
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
    double* lvVof;
    double* v13;
    int8_t* done;
    uint32_t* err;
};

void launchScanMixed(const StepArgs& a, cudaStream_t st);
void launchLsNormal(const StepArgs& a, cudaStream_t st);
void launchPlaneLevels(const StepArgs& a, cudaStream_t st);
void launchPlaneThirds(const StepArgs& a, cudaStream_t st);
void launchPlaneFinal(const StepArgs& a, cudaStream_t st);
void launchInterfaceUn0(const StepArgs& a, cudaStream_t st);
void launchInterfaceFaces(const StepArgs& a, cudaStream_t st);
void launchUpdate(const StepArgs& a, cudaStream_t st);
void launchBound(const StepArgs& a, const BoundBuffers& b, cudaStream_t st);
void launchBruteForce(const StepArgs& a, cudaStream_t st);
void launchFaceFlatness(const DevMesh& m, const double* Sf, double* flat, cudaStream_t st);
void launchFaceFull(const DevMesh& m, double* fullC, double* fullA, cudaStream_t st);

}  // namespace simplic
