/* Learned-normal network of the SimPLIC step: tensor-core primitives.
 *
 * These entry points have no counterpart in the reference, whose
 * reconstruction uses only least-squares or iso-surface normals.  They are
 * the building blocks with which the network that maps an interface cell's
 * neighbourhood (alpha and relative centroids of up to 32 cells, 128
 * features) to a unit normal and a plane constant is trained on the GPU and
 * evaluated inside the step.  All pointers are device pointers; every call
 * only enqueues work on `stream` (a cudaStream_t or NULL).  Return 0 on
 * success, 1 for invalid arguments, 2 for a CUDA launch error; device-side
 * failures (a bounded wait that timed out) set bit 0 of *err.
 */
#ifndef SIMPLIC_MLP_H
#define SIMPLIC_MLP_H

#include <stdint.h>

#include "simplic.h"

#ifdef __cplusplus
extern "C" {
#endif

/* epilogue of simplic_mlp_gemm */
#define SIMPLIC_MLP_STORE 0         /* D = A B^T (FP32) */
#define SIMPLIC_MLP_ATOMIC 1        /* D += A B^T (FP32 atomics; split-K allowed) */
#define SIMPLIC_MLP_BIAS 2          /* D = A B^T + bias (FP32) */
#define SIMPLIC_MLP_BIAS_GELU 3     /* Z = A B^T + bias -> D (optional); H = gelu(Z) (BF16), HT = H^T (optional) */
#define SIMPLIC_MLP_GELU_BACKWARD 4 /* H = (A B^T) * gelu'(Zin) (BF16), HT = H^T (optional) */

/* D[M x N] = A[M x K] B[N x K]^T with A, B BF16 row-major (K contiguous,
 * leading dimensions lda / ldb in elements, multiples of 8, 16-byte aligned
 * bases), FP32 accumulation in tensor memory (tcgen05.mma kind::f16).
 * N a multiple of 16 up to 256; K a multiple of 64; M any.  splitK > 1 only
 * with SIMPLIC_MLP_ATOMIC. */
int simplic_mlp_gemm(const void* A, int32_t lda, const void* B, int32_t ldb, int32_t M, int32_t N, int32_t K,
                     int32_t mode, float* D, int32_t ldd, const float* bias, void* H, int32_t ldh, void* HT,
                     int32_t ldht, const float* Zin, int32_t ldz, int32_t splitK, uint32_t* err, void* stream);

/* The whole network (inference) in one kernel: rows *M (device int, at most
 * maxRows) of X (BF16 [.][128]) through the four layers of W (BF16
 * [4][128][128]) and b (FP32 [4][128]); Y[row][0..15] (FP32, leading
 * dimension ldy >= 16) = the first 16 outputs.  Weights and the activation
 * tile stay in shared memory, accumulators in TMEM. */
int simplic_mlp_forward(const void* X, const int32_t* M, int32_t maxRows, const void* W, const float* b, float* Y,
                        int32_t ldy, uint32_t* err, void* stream);

/* Training samples on the handle's mesh (enqueued on the handle's stream):
 * count rows of network input X (BF16 [count][128]) and targets T (FP32
 * [count][4]: unit normal, (d + n.C) / h).  Each sample is a random plane
 * (or, for sphere_percent of them, a random sphere of radius 2h..20h)
 * through a random cell, the stencil's volume fractions from the cut-cell
 * routine of the step.  Deterministic in seed. */
int simplic_mlp_samples(simplic_handle* h, uint64_t seed, int32_t count, int32_t sphere_percent, void* X, float* T);

/* Network of the learned precision: W [4][128][128] (row = output unit,
 * K = input), b [4][128], FP32 host arrays (stored as BF16 / FP32).  A
 * cell keeps its least-squares normal when the network's normal is nearly
 * zero or raises the local volume residual above the least-squares
 * normal's by more than gate_tol.  The local volume residual of a normal
 * is sum_j |f_j - alpha_j| over the cell's network neighbourhood (its 30
 * nearest point neighbours): the plane with that normal which cuts the
 * cell's volume fraction from a cube of the cell's size centred on the
 * cell is laid through equal cubes centred on the neighbours, f_j being the
 * fractions it cuts from them (FP32). */
int simplic_set_network(simplic_handle* h, const float* W, const float* b, float gate_tol);
/* cells of the last reconstruct that took the network's normal */
int simplic_network_stats(simplic_handle* h, int32_t* n_learned);
/* info[3] of the last reconstruct: cells that took the network's normal,
 * the network's row capacity (max(2^18, cells / 32)), and the mixed cells
 * beyond that capacity, which get no network row and keep the FP32
 * least-squares normal */
int simplic_network_info(simplic_handle* h, int32_t* info);
/* the network inputs of the last reconstruct, ascending in cell: row i
 * (BF16 [128] in X) belongs to cells[i]; A (nullable, FP32 [32] per row)
 * receives the alphas the fallback test uses (alpha_c, then alpha_j -
 * alpha_c per neighbour slot); at most max_rows rows are copied to the
 * host buffers, *rows = the number copied */
int simplic_network_inputs(simplic_handle* h, int32_t max_rows, int32_t* rows, int32_t* cells, void* X, float* A);

#ifdef __cplusplus
}
#endif
#endif /* SIMPLIC_MLP_H */
