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
    double* blkMin;     // [ceil(nc/256)]
    double* blkMax;
    uint32_t* err;      // device error bits
};

struct BoundBuffers {
    int* cand;
    int candCap;
    double* corr;
    double* dvfMod;
    int* modStamp;
    int* doneStamp;
    int* corrected;
    int* written;
    int listCap;
    int* modList;
    int modCap;
    int* touched;
    int touchedCap;
    int stamp;
    int* info;  // [0] passes run, [1] most cells bounded in a pass
};

void launchScanMixed(const StepArgs& a, cudaStream_t st);
void launchLsNormal(const StepArgs& a, cudaStream_t st);
void launchPlaneSolve(const StepArgs& a, cudaStream_t st);
void launchInterfaceFlux(const StepArgs& a, cudaStream_t st);
void launchUpdate(const StepArgs& a, cudaStream_t st);
void launchBound(const StepArgs& a, const BoundBuffers& b, cudaStream_t st);
void launchBruteForce(const StepArgs& a, cudaStream_t st);
void launchFaceFlatness(const DevMesh& m, const double* Sf, double* flat, cudaStream_t st);

}  // namespace simplic
