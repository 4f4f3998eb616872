// Instantiations and launch of the row-staged (bulk-copy) step kernel:
// D2Q9 and D3Q19, BGK / TRT / MRT, F32 and F16S storage, physics mode.
#include <cuda_runtime.h>

#include "lbm_step_tma.cuh"

namespace lbm {

using TmaKernel = void (*)(StepParams, TmaRows);

static TmaKernel tma_kernel(int q, int coll, int st) {
#define TMA_CASE(Q, C, S) \
    if (q == Q && coll == C && st == S) return step_kernel_tma<Q, C, S>;
    TMA_CASE(9, 1, 0) TMA_CASE(9, 2, 0) TMA_CASE(9, 3, 0) TMA_CASE(9, 1, 1) TMA_CASE(9, 2, 1) TMA_CASE(9, 3, 1)
    TMA_CASE(19, 1, 0) TMA_CASE(19, 2, 0) TMA_CASE(19, 3, 0) TMA_CASE(19, 1, 1) TMA_CASE(19, 2, 1)
    TMA_CASE(19, 3, 1)
#undef TMA_CASE
    return nullptr;
}

int tma_threads() { return TMA_THREADS; }
int tma_barrier_bytes() { return TMA_BARRIER_BYTES; }
unsigned tma_stage_size(int q, int nx, int elem) { return tma_stage_bytes(q, nx, elem); }

// Allow `smem` bytes of dynamic shared memory and report how many blocks of
// the kernel fit on one SM.  Returns a CUDA error code.
int tma_prepare(int q, int coll, int st, size_t smem, int *blocks_per_sm) {
    TmaKernel k = tma_kernel(q, coll, st);
    if (!k) return (int)cudaErrorInvalidDeviceFunction;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, TMA_THREADS, smem);
    return (int)e;
}

int launch_step_tma(int q, const StepParams &p, const TmaRows &rows, int coll, int st, int grid, size_t smem,
                    cudaStream_t s) {
    TmaKernel k = tma_kernel(q, coll, st);
    if (!k) return -1;
    k<<<grid, TMA_THREADS, smem, s>>>(p, rows);
    return 0;
}

}  // namespace lbm
