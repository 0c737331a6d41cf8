// simplic_mixed_cells_noalloc: the mixed-cell scan of the reconstruction
// without any device allocation.
//
// Who needs it: callers that may not call cudaMalloc at the point where they
// want the interface cells -- a solver whose device memory is owned by its
// own pool or by a framework allocator (raw cudaMalloc would bypass the
// pool's accounting and can synchronise the device), or code running under
// a memory limit that the library's handle would break.  Such callers
// cannot create a simplic handle (it allocates the mesh and the step state),
// so this entry point takes plain device pointers and keeps its only scratch
// -- the per-tile counts of a stable, two-pass compaction -- in a
// fixed-size file-scope device array.
//
// Algorithm: the cells are split into tiles of kTileCells.  Pass 1 counts
// the mixed cells of each tile (alpha strictly inside (tol, 1 - tol), the
// test of reconstruction.C:689-700, done on the IEEE bit patterns like the
// handle's scan), pass 2 turns the counts into exclusive offsets in one
// block, pass 3 writes each tile's mixed cells at its offset.  The list
// comes out in ascending cell order, the order simplic_get_mixed_cells
// reports.  Every tile count that pass 2 reads was written by pass 1 of the
// same call, so no part of the scratch has to start at zero.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/simplic.h"

namespace simplic {
void setCreateError(const std::string& msg);
}

namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 8;
constexpr int kTileCells = kThreads * kCellsPerThread;  // 2048
constexpr int kMaxTiles = SIMPLIC_NOALLOC_MAX_CELLS / kTileCells;  // 65536 tiles, 256 KiB
constexpr int kScanThreads = 1024;
constexpr int kMaxDevices = 64;
static_assert(SIMPLIC_NOALLOC_MAX_CELLS % kTileCells == 0, "whole tiles");
static_assert(kMaxTiles % kScanThreads == 0, "scan split");

// Per-tile mixed-cell counts, then (after pass 2) per-tile output offsets.
// Shared by every call on a device and kept until the process exits.
static __device__ __align__(256) int32_t g_tileScratch[kMaxTiles];

__device__ __forceinline__ bool isMixedBits(double a, long long tolBits, long long omtBits) {
    const long long b = __double_as_longlong(a);
    return (b > tolBits) && (b < omtBits);
}

__global__ void __launch_bounds__(kThreads) kTileCount(int n, const double* __restrict__ alpha, long long tolBits,
                                                       long long omtBits, int32_t* __restrict__ tileCount) {
    __shared__ int warpSum[kThreads / 32];
    const int tile = blockIdx.x;
    const int base = tile * kTileCells;
    int cnt = 0;
#pragma unroll
    for (int k = 0; k < kCellsPerThread; ++k) {
        const int c = base + k * kThreads + threadIdx.x;
        if (c < n && isMixedBits(alpha[c], tolBits, omtBits)) ++cnt;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) warpSum[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < kThreads / 32; ++w) s += warpSum[w];
        tileCount[tile] = s;
    }
}

// One block: exclusive scan of nTiles counts in place; the total goes to
// *nMixed.  Each thread owns a contiguous run of kMaxTiles / kScanThreads
// entries at most.
__global__ void __launch_bounds__(kScanThreads) kTileScan(int nTiles, int32_t* __restrict__ tile,
                                                          int32_t* __restrict__ nMixed) {
    __shared__ int part[kScanThreads];
    const int per = (nTiles + kScanThreads - 1) / kScanThreads;
    const int lo = threadIdx.x * per;
    const int hi = min(lo + per, nTiles);
    int s = 0;
    for (int i = lo; i < hi; ++i) s += tile[i];
    part[threadIdx.x] = s;
    __syncthreads();
    // Hillis-Steele inclusive scan of the per-thread sums
    for (int o = 1; o < kScanThreads; o <<= 1) {
        const int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int run = part[threadIdx.x] - s;
    for (int i = lo; i < hi; ++i) {
        const int v = tile[i];
        tile[i] = run;
        run += v;
    }
    if (threadIdx.x == kScanThreads - 1) *nMixed = part[kScanThreads - 1];
}

__global__ void __launch_bounds__(kThreads) kTileScatter(int n, const double* __restrict__ alpha, long long tolBits,
                                                         long long omtBits, const int32_t* __restrict__ tileOffset,
                                                         int32_t* __restrict__ cells, int capacity) {
    __shared__ int warpCnt[kThreads / 32];
    const int tile = blockIdx.x;
    const int base = tile * kTileCells;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int run = tileOffset[tile];
#pragma unroll 1
    for (int k = 0; k < kCellsPerThread; ++k) {
        const int c = base + k * kThreads + threadIdx.x;
        const bool m = c < n && isMixedBits(alpha[c], tolBits, omtBits);
        const unsigned ball = __ballot_sync(0xffffffffu, m);
        if (lane == 0) warpCnt[warp] = __popc(ball);
        __syncthreads();
        int before = 0, total = 0;
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) {
            const int v = warpCnt[w];
            before += w < warp ? v : 0;
            total += v;
        }
        if (m) {
            const int slot = run + before + __popc(ball & ((1u << lane) - 1u));
            if (slot < capacity) cells[slot] = c;
        }
        run += total;
        __syncthreads();  // warpCnt is rewritten by the next k
    }
}

// Device address of the scratch array per device ordinal.  Stored only once
// a lookup has succeeded: a failed lookup (say, inside a stream capture)
// is retried by the next call instead of being remembered.
std::mutex g_setupMu;
int32_t* g_scratchPtr[kMaxDevices] = {};

int fail(int code, const std::string& msg) {
    simplic::setCreateError("simplic_mixed_cells_noalloc: " + msg);
    return code;
}

}  // namespace

extern "C" int simplic_mixed_cells_noalloc(const double* alpha, int32_t n_cells, double mixed_cell_tol,
                                           int32_t* cells, int32_t capacity, int32_t* n_mixed, void* stream) {
    if (n_cells < 0 || capacity < 0) return fail(SIMPLIC_ERR_INVALID_ARGUMENT, "negative size");
    if (n_cells > SIMPLIC_NOALLOC_MAX_CELLS)
        return fail(SIMPLIC_ERR_INVALID_ARGUMENT,
                    "n_cells = " + std::to_string(n_cells) + " exceeds the fixed scratch limit of " +
                        std::to_string(SIMPLIC_NOALLOC_MAX_CELLS) + " cells");
    if (!n_mixed || (n_cells > 0 && !alpha) || (capacity > 0 && !cells))
        return fail(SIMPLIC_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (!(mixed_cell_tol >= 0.0 && mixed_cell_tol < 0.5))
        return fail(SIMPLIC_ERR_INVALID_ARGUMENT, "mixed_cell_tol must lie in [0, 0.5)");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SIMPLIC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(SIMPLIC_ERR_UNSUPPORTED, "device ordinal beyond 63");
    // First successful call on this device: resolve the device address of
    // the scratch array (its host-side name is only a stand-in).
    int32_t* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setupMu);
        if (!g_scratchPtr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_tileScratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();  // the next call retries
                return fail(SIMPLIC_ERR_CUDA,
                            std::string("cudaGetSymbolAddress of the scratch array: ") + cudaGetErrorString(e));
            }
            g_scratchPtr[dev] = static_cast<int32_t*>(p);
        }
        scratch = g_scratchPtr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    if (n_cells == 0) {
        e = cudaMemsetAsync(n_mixed, 0, sizeof(int32_t), st);
        if (e != cudaSuccess) return fail(SIMPLIC_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
        return SIMPLIC_OK;
    }
    const double omt = 1.0 - mixed_cell_tol;
    long long tolBits, omtBits;
    std::memcpy(&tolBits, &mixed_cell_tol, sizeof(double));
    std::memcpy(&omtBits, &omt, sizeof(double));
    const int nTiles = (n_cells + kTileCells - 1) / kTileCells;
    kTileCount<<<nTiles, kThreads, 0, st>>>(n_cells, alpha, tolBits, omtBits, scratch);
    kTileScan<<<1, kScanThreads, 0, st>>>(nTiles, scratch, n_mixed);
    kTileScatter<<<nTiles, kThreads, 0, st>>>(n_cells, alpha, tolBits, omtBits, scratch, cells, capacity);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SIMPLIC_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return SIMPLIC_OK;
}
