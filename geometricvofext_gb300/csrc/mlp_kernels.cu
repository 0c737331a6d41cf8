// Dense layers of the learned-normal MLP on the 5th-generation tensor cores.
//
// One kernel, kGemmTN, computes D[M x N] = A[M x K] * B[N x K]^T with A and B
// in BF16 (K contiguous in memory for both), FP32 accumulation in tensor
// memory, and a fused epilogue.  Per CTA: one 128-row block of D and all N
// (<= 256) columns, over a range of K (gridDim.y splits K; the split-K
// epilogue adds into FP32 with atomics).  128 threads:
//   * all threads stage a 128 x 64 tile of A and an N x 64 tile of B into
//     shared memory in the canonical no-swizzle K-major layout (8 x 16-byte
//     core matrices; LBO = 128 B between K-adjacent, SBO = 1024 B between
//     row-adjacent core matrices);
//   * one elected thread issues four tcgen05.mma (K = 16 each,
//     kind::f16 with BF16 inputs, FP32 accumulator of 128 lanes x N columns
//     in TMEM) and tcgen05.commit to an mbarrier;
//   * after the last K tile each warp reads its 32 accumulator rows with
//     tcgen05.ld (32x32b) and runs the epilogue.
// Every wait on the mbarrier is bounded: on time-out the CTA sets an error
// flag and leaves after its outstanding MMAs have been waited for (bounded
// again) and its TMEM has been freed.
//
// The shapes of the network are small (128-wide layers, tens of thousands of
// rows per step), so the kernel favours simplicity over pipelining.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/simplic_mlp.h"

namespace simplic {
namespace {

constexpr int kTileM = 128;
constexpr int kTileK = 64;
constexpr int kThreads = 128;
constexpr long long kWaitLimit = 1ll << 22;  // try_wait polls (a few seconds at most)

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) of a K-major tile with kTileK columns in the
// no-swizzle canonical layout.
__device__ __forceinline__ uint32_t coreOffset(int r, int k) {
    return uint32_t((r >> 3) * 1024 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// tcgen05 shared-memory matrix descriptor: start address, leading (K) and
// stride (row) byte offsets, version bits 46-48 = 0b001, no swizzle.
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= uint64_t((addr >> 4) & 0x3FFF);
    d |= uint64_t((lbo >> 4) & 0x3FFF) << 16;
    d |= uint64_t((sbo >> 4) & 0x3FFF) << 32;
    d |= uint64_t(1) << 46;
    return d;
}

// Instruction descriptor of kind::f16: D = F32, A = B = BF16, both K-major,
// M = 128, N = n.
__host__ __device__ constexpr uint32_t instrDesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(kTileM >> 4) << 24);
}

__device__ __forceinline__ void mbarInit(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}

// Bounded wait for the completion of the phase with the given parity.
__device__ __forceinline__ bool mbarWait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smemAddr(bar);
    for (long long i = 0; i < kWaitLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// tanh form of GELU with the hardware tanh (tanh.approx.f32, relative error
// about 2^-11, far below the BF16 rounding of the activations); training
// and inference use the same function
__device__ __forceinline__ float tanhHw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float geluF(float z) {
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    return 0.5f * z * (1.f + tanhHw(k0 * (z + k1 * z * z * z)));
}
__device__ __forceinline__ float geluGradF(float z) {
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    const float u = k0 * (z + k1 * z * z * z);
    const float t = tanhHw(u);
    const float du = k0 * (1.f + 3.f * k1 * z * z);
    return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * du;
}

struct GemmArgs {
    const __nv_bfloat16* A;
    int lda;
    const __nv_bfloat16* B;
    int ldb;
    int M, N, K;
    int mode;
    float* D;  // FP32 output (modes STORE / BIAS / ATOMIC), or the pre-activation of GELU
    int ldd;
    const float* bias;   // [N]
    __nv_bfloat16* H;    // BF16 output (GELU, GELU_BACKWARD)
    int ldh;
    __nv_bfloat16* HT;   // optional transposed BF16 output [N][ldht]
    int ldht;
    const float* Zin;    // pre-activation for GELU_BACKWARD [M][ldz]
    int ldz;
    unsigned* err;
    const int* Mdev;     // optional row count on the device (at most M)
};

__global__ void __launch_bounds__(kThreads) kGemmTN(GemmArgs g) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sA = smem;                        // 128 x 64 bf16 = 16 KB
    uint8_t* sB = smem + kTileM * kTileK * 2;  // N x 64 bf16 <= 32 KB
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmemBase;
    __shared__ int failed;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // rows known only on the device: blocks past them leave before touching
    // tensor memory
    if (g.Mdev) {
        const int md = *g.Mdev;
        if (md < g.M) g.M = md;
    }
    if (int(blockIdx.x) * kTileM >= g.M) return;
    const int kPer = (g.K / kTileK + gridDim.y - 1) / gridDim.y * kTileK;
    const int kBeg = blockIdx.y * kPer;
    const int kEnd = min(g.K, kBeg + kPer);
    const int N = g.N;
    const uint32_t nCols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));

    if (tid == 0) {
        mbarInit(&bar, 1);
        failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(&tmemBase)),
                     "r"(nCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmemBase;
    const uint32_t idesc = instrDesc(N);

    uint32_t phase = 0;
    // row tiles blockIdx.x, blockIdx.x + gridDim.x, ...: a grid smaller than
    // the tile count keeps its tensor memory across tiles
    for (int tile = blockIdx.x; tile * kTileM < g.M && !failed; tile += gridDim.x) {
    const int m0 = tile * kTileM;
    int nIssued = 0;
    for (int k0 = kBeg; k0 < kEnd; k0 += kTileK) {
        // stage A (rows m0..m0+127) and B (rows 0..N-1), 8 bf16 = 16 B per load
        for (int v = tid; v < kTileM * (kTileK / 8); v += kThreads) {
            const int r = v / (kTileK / 8), kc = (v % (kTileK / 8)) * 8;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (m0 + r < g.M && k0 + kc < g.K)
                val = *reinterpret_cast<const uint4*>(g.A + size_t(m0 + r) * g.lda + k0 + kc);
            *reinterpret_cast<uint4*>(sA + coreOffset(r, kc)) = val;
        }
        for (int v = tid; v < N * (kTileK / 8); v += kThreads) {
            const int r = v / (kTileK / 8), kc = (v % (kTileK / 8)) * 8;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (k0 + kc < g.K) val = *reinterpret_cast<const uint4*>(g.B + size_t(r) * g.ldb + k0 + kc);
            *reinterpret_cast<uint4*>(sB + coreOffset(r, kc)) = val;
        }
        // the tensor core reads shared memory through the async proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int s = 0; s < kTileK / 16; ++s) {
                const uint64_t ad = smemDesc(smemAddr(sA) + s * 256, 128, 1024);
                const uint64_t bd = smemDesc(smemAddr(sB) + s * 256, 128, 1024);
                const uint32_t acc = (k0 > kBeg || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smemAddr(&bar))
                         : "memory");
        }
        ++nIssued;
        // the tiles are overwritten by the next iteration: wait for the MMAs
        if (!mbarWait(&bar, phase)) failed = 1;
        phase ^= 1u;
        __syncthreads();
        if (failed) break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (!failed && nIssued > 0) {
        // epilogue: warp w owns accumulator rows 32w .. 32w+31 (TMEM lanes)
        const int row = m0 + warp * 32 + lane;
        for (int c0 = 0; c0 < N; c0 += 8) {
            uint32_t r[8];
            const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row >= g.M) continue;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int col = c0 + j;
                if (col >= N) break;
                float acc = __uint_as_float(r[j]);
                switch (g.mode) {
                    case SIMPLIC_MLP_STORE:
                        g.D[size_t(row) * g.ldd + col] = acc;
                        break;
                    case SIMPLIC_MLP_ATOMIC:
                        atomicAdd(g.D + size_t(row) * g.ldd + col, acc);
                        break;
                    case SIMPLIC_MLP_BIAS:
                        g.D[size_t(row) * g.ldd + col] = acc + (g.bias ? g.bias[col] : 0.f);
                        break;
                    case SIMPLIC_MLP_BIAS_GELU: {
                        const float z = acc + (g.bias ? g.bias[col] : 0.f);
                        if (g.D) g.D[size_t(row) * g.ldd + col] = z;
                        const __nv_bfloat16 h = __float2bfloat16_rn(geluF(z));
                        g.H[size_t(row) * g.ldh + col] = h;
                        if (g.HT) g.HT[size_t(col) * g.ldht + row] = h;
                        break;
                    }
                    case SIMPLIC_MLP_GELU_BACKWARD: {
                        // dZ = dH * GELU'(Z)
                        const float dz = acc * geluGradF(g.Zin[size_t(row) * g.ldz + col]);
                        const __nv_bfloat16 h = __float2bfloat16_rn(dz);
                        g.H[size_t(row) * g.ldh + col] = h;
                        if (g.HT) g.HT[size_t(col) * g.ldht + row] = h;
                        break;
                    }
                    default:
                        break;
                }
            }
        }
    }
    // every warp has read its accumulator rows before the next tile's MMAs
    // overwrite them
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    }  // row tiles
    if (failed) {
        // give the MMAs still in flight a second bounded wait before the
        // tensor memory they write is released
        mbarWait(&bar, phase ^ 1u);
        if (tid == 0) atomicOr(g.err, 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(nCols) : "memory");
}

// ---------------------------------------------------------------------------
// The whole network in one kernel for inference: the weights of the four
// layers (three 128 x 128, the output layer's first 16 rows) and one 128-row
// activation tile stay in shared memory, the accumulator in TMEM; each
// layer is 8 MMAs (K = 16) from the activation tile, and its epilogue
// (bias, GELU, BF16) writes the next layer's input back into the same tile.
// Persistent over 128-row tiles; the row count is read on the device.
// ---------------------------------------------------------------------------
constexpr int kNetWidth = 128;
constexpr int kNetOut = 16;  // rows of the output layer evaluated (4 used)
constexpr uint32_t kNetSbo = (kNetWidth / 8) * 128;  // row-adjacent core matrices for K = 128

__device__ __forceinline__ uint32_t coreOffset128(int r, int k) {
    return uint32_t((r >> 3) * kNetSbo + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// rows x 128 BF16 from global memory into the core-matrix layout, 16 bytes
// per asynchronous copy, all in flight at once; rows from validRows on are
// zero-filled (nothing is read for them).
__device__ __forceinline__ void stageRows(uint8_t* dst, const __nv_bfloat16* src, int rows, int validRows, int tid) {
    for (int v = tid; v < rows * (kNetWidth / 8); v += kThreads) {
        const int r = v / (kNetWidth / 8), kc = (v % (kNetWidth / 8)) * 8;
        const bool ok = r < validRows;
        const __nv_bfloat16* g = src + size_t(ok ? r : 0) * kNetWidth + kc;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smemAddr(dst + coreOffset128(r, kc))),
                     "l"(g), "r"(ok ? 16u : 0u)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

__global__ void __launch_bounds__(kThreads) kMlpFused(const __nv_bfloat16* __restrict__ X, const int* __restrict__ Mdev,
                                                     int maxRows, const __nv_bfloat16* __restrict__ W,
                                                     const float* __restrict__ bias, float* __restrict__ Y, int ldy,
                                                     unsigned* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sW = smem;                                            // 3 x 32 KB + 4 KB
    uint8_t* sA = smem + 3 * kNetWidth * kNetWidth * 2 + kNetOut * kNetWidth * 2;  // 32 KB
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmemBase;
    __shared__ int failed;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int M = min(*Mdev, maxRows);
    if (int(blockIdx.x) * kTileM >= M) return;

    if (tid == 0) {
        mbarInit(&bar, 1);
        failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(&tmemBase)),
                     "r"(uint32_t(kNetWidth))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    for (int l = 0; l < 3; ++l)
        stageRows(sW + l * kNetWidth * kNetWidth * 2, W + size_t(l) * kNetWidth * kNetWidth, kNetWidth, kNetWidth, tid);
    stageRows(sW + 3 * kNetWidth * kNetWidth * 2, W + size_t(3) * kNetWidth * kNetWidth, kNetOut, kNetOut, tid);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmemBase;

    uint32_t phase = 0;
    for (int tile = blockIdx.x; tile * kTileM < M && !failed; tile += gridDim.x) {
        const int m0 = tile * kTileM;
        stageRows(sA, X + size_t(m0) * kNetWidth, kTileM, M - m0, tid);
        for (int l = 0; l < 4 && !failed; ++l) {
            const int N = (l < 3) ? kNetWidth : kNetOut;
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t wBase = smemAddr(sW + l * kNetWidth * kNetWidth * 2);
                const uint32_t idesc = instrDesc(N);
#pragma unroll
                for (int s = 0; s < kNetWidth / 16; ++s) {
                    const uint64_t ad = smemDesc(smemAddr(sA) + s * 256, 128, kNetSbo);
                    const uint64_t bd = smemDesc(wBase + s * 256, 128, kNetSbo);
                    const uint32_t acc = s > 0 ? 1u : 0u;
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                        : "memory");
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smemAddr(&bar))
                             : "memory");
            }
            if (!mbarWait(&bar, phase)) failed = 1;
            phase ^= 1u;
            __syncthreads();
            if (failed) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int rloc = warp * 32 + lane;
            const int row = m0 + rloc;
            // 32 columns per TMEM load (16 for the output layer), one wait each
            for (int c0 = 0; c0 < N; c0 += 32) {
                uint32_t r[32];
                const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0);
                const int nc = N - c0 < 32 ? N - c0 : 32;
                if (nc == 32)
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                        "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
                        "%30, %31}, [%32];"
                        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
                          "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                          "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                        : "r"(taddr)
                        : "memory");
                else
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                        "%12, %13, %14, %15}, [%16];"
                        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                          "=r"(r[14]), "=r"(r[15])
                        : "r"(taddr)
                        : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                const float* bl = bias + l * kNetWidth + c0;
                if (l < 3) {
                    // next layer's input, in place (this layer's MMAs are complete)
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        __align__(16) __nv_bfloat16 h[8];
#pragma unroll
                        for (int j = 0; j < 8; ++j)
                            h[j] = __float2bfloat16_rn(geluF(__uint_as_float(r[8 * q + j]) + bl[8 * q + j]));
                        *reinterpret_cast<uint4*>(sA + coreOffset128(rloc, c0 + 8 * q)) =
                            *reinterpret_cast<const uint4*>(h);
                    }
                } else if (row < M) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) Y[size_t(row) * ldy + c0 + j] = __uint_as_float(r[j]) + bl[j];
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        }
        __syncthreads();
    }
    if (failed) {
        mbarWait(&bar, phase ^ 1u);
        if (tid == 0) atomicOr(err, 1u);
    }

    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(uint32_t(kNetWidth))
                     : "memory");
}

}  // namespace

// The four layers of the network on the rows *Mdev (at most maxRows) of X:
// Y[:, 0:16] (FP32, leading dimension ldy) = output layer of the network.
cudaError_t launchNetwork(const void* X, const int* Mdev, int maxRows, const void* W, const float* bias, float* Y,
                          int ldy, uint32_t* err, cudaStream_t st) {
    const size_t smemBytes = size_t(3) * kNetWidth * kNetWidth * 2 + size_t(kNetOut) * kNetWidth * 2 +
                             size_t(kTileM) * kNetWidth * 2;
    // set on every launch: the attribute belongs to the current device, and
    // the call is cheap next to the launch
    cudaError_t e = cudaFuncSetAttribute(kMlpFused, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smemBytes));
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tiles = (maxRows + kTileM - 1) / kTileM;
    kMlpFused<<<tiles < sms ? tiles : sms, kThreads, smemBytes, st>>>(
        static_cast<const __nv_bfloat16*>(X), Mdev, maxRows, static_cast<const __nv_bfloat16*>(W), bias, Y, ldy,
        reinterpret_cast<unsigned*>(err));
    return cudaGetLastError();
}

}  // namespace simplic

using namespace simplic;

extern "C" int simplic_mlp_gemm(const void* A, int32_t lda, const void* B, int32_t ldb, int32_t M, int32_t N,
                                int32_t K, int32_t mode, float* D, int32_t ldd, const float* bias, void* H,
                                int32_t ldh, void* HT, int32_t ldht, const float* Zin, int32_t ldz, int32_t splitK,
                                uint32_t* err, void* stream) {
    if (!A || !B || !err || M <= 0 || N <= 0 || K <= 0) return 1;
    if (N % 16 != 0 || N > 256 || K % kTileK != 0 || lda % 8 != 0 || ldb % 8 != 0) return 1;
    if (splitK < 1) splitK = 1;
    if (splitK > K / kTileK) splitK = K / kTileK;
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return 1;
    if ((mode == SIMPLIC_MLP_BIAS_GELU || mode == SIMPLIC_MLP_GELU_BACKWARD) && !H) return 1;
    if (mode == SIMPLIC_MLP_GELU_BACKWARD && !Zin) return 1;
    if ((mode == SIMPLIC_MLP_STORE || mode == SIMPLIC_MLP_ATOMIC || mode == SIMPLIC_MLP_BIAS) && !D) return 1;
    if (mode != SIMPLIC_MLP_ATOMIC && splitK != 1) return 1;
    if (mode < SIMPLIC_MLP_STORE || mode > SIMPLIC_MLP_GELU_BACKWARD) return 1;
    GemmArgs g{static_cast<const __nv_bfloat16*>(A), lda, static_cast<const __nv_bfloat16*>(B), ldb, M, N, K, mode,
               D, ldd, bias, static_cast<__nv_bfloat16*>(H), ldh, static_cast<__nv_bfloat16*>(HT), ldht, Zin, ldz,
               err, nullptr};
    const size_t smemBytes = size_t(kTileM) * kTileK * 2 + size_t(N) * kTileK * 2;
    // set on every launch: the attribute belongs to the current device
    if (cudaFuncSetAttribute(kGemmTN, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(kTileM * kTileK * 2 + 256 * kTileK * 2)) != cudaSuccess)
        return 2;
    dim3 grid((M + kTileM - 1) / kTileM, splitK);
    kGemmTN<<<grid, kThreads, smemBytes, static_cast<cudaStream_t>(stream)>>>(g);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

extern "C" int simplic_mlp_forward(const void* X, const int32_t* M, int32_t maxRows, const void* W, const float* b,
                                   float* Y, int32_t ldy, uint32_t* err, void* stream) {
    if (!X || !M || !W || !b || !Y || !err || maxRows <= 0 || ldy < 16) return 1;
    if ((reinterpret_cast<uintptr_t>(X) | reinterpret_cast<uintptr_t>(W)) & 15) return 1;
    return launchNetwork(X, M, maxRows, W, b, Y, ldy, err, static_cast<cudaStream_t>(stream)) == cudaSuccess ? 0 : 2;
}
