/*
 * Host shim for compiling the reference solver's CUDA kernel sources with g++.
 *
 * TEST INFRASTRUCTURE ONLY: this header is force-included (g++ -include) when
 * oracle/build_ref.sh compiles the reference's own GpuCollision.cu,
 * GpuStream.cu, GpuBoundaries.cu, GpuUpdateMacro.cu, GpuInit.cu and
 * CellFunctions.cu into oracle/_ref/.  The kernels are then executed one
 * emulated CUDA thread at a time by ref_harness.cpp.  Nothing in the product
 * links against the result.
 *
 * The built-in launch variables become thread-local globals that the harness
 * sets before each emulated thread; the CUDA memory qualifiers vanish; the
 * two runtime calls the reference's set-up code makes (cudaMemcpyToSymbol,
 * cudaMemcpy) become memcpy, because "device" memory is host memory here.
 */
#pragma once
#include <string.h>
#include <stddef.h>
#include <math.h>

struct shim_dim3 {
    unsigned x, y, z;
};
extern thread_local shim_dim3 blockIdx, threadIdx, blockDim, gridDim;

#define __global__
#define __device__
#define __host__
#define __constant__
#define cudaMemcpyToSymbol(sym, src, sz) memcpy((void *)&(sym), (const void *)(src), (sz))

enum shim_memcpy_kind {
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3
};
static inline int cudaMemcpy(void *dst, const void *src, size_t bytes, int) {
    memcpy(dst, src, bytes);
    return 0;
}

/*
 * 64-bit BC mask macros for the reference's 3D kernels.  The reference's own
 * include/BcMacros3D.h shifts the untyped constants BC3D_ALL (0x7) and
 * BC3D_WALL (0x1) as 32-bit ints, so BC3D_MASK(BC3D_ALL, dir) in
 * gpuBcSimpleWall3D (GpuBoundaries.cu:457-459) is undefined for directions
 * 11-18 and the host and device compilers resolve it differently.  Defining
 * the header guard here makes every 3D mask 64 bits wide with the same bit
 * layout (3 bits per link direction from bit 0, main type at bit 54, corner
 * 57, fluid 58), so the harness runs the kernels as their authors intended.
 */
#define BC_MACROS3D_H
#define BC3D_NONE 0x0ULL
#define BC3D_WALL 0x1ULL
#define BC3D_INLT 0x2ULL
#define BC3D_OUTL 0x3ULL
#define BC3D_CYCL 0x4ULL
#define BC3D_SYMP 0x5ULL
#define BC3D_ALL 0x7ULL
#define BC3D_MASK(type, dir) ((unsigned long long)(type) << (((dir)-1) * 3))
#define BC3D_WALL_1 (1ULL << 0)
#define BC3D_INLT_1 (2ULL << 0)
#define BC3D_OUTL_1 (3ULL << 0)
#define BC3D_CYCL_1 (4ULL << 0)
#define BC3D_SYMP_1 (5ULL << 0)
#define BC3D_1(i) ((unsigned long long)(i) << 0)
#define BC3D_WALL_2 (1ULL << 3)
#define BC3D_INLT_2 (2ULL << 3)
#define BC3D_OUTL_2 (3ULL << 3)
#define BC3D_CYCL_2 (4ULL << 3)
#define BC3D_SYMP_2 (5ULL << 3)
#define BC3D_2(i) ((unsigned long long)(i) << 3)
#define BC3D_WALL_3 (1ULL << 6)
#define BC3D_INLT_3 (2ULL << 6)
#define BC3D_OUTL_3 (3ULL << 6)
#define BC3D_CYCL_3 (4ULL << 6)
#define BC3D_SYMP_3 (5ULL << 6)
#define BC3D_3(i) ((unsigned long long)(i) << 6)
#define BC3D_WALL_4 (1ULL << 9)
#define BC3D_INLT_4 (2ULL << 9)
#define BC3D_OUTL_4 (3ULL << 9)
#define BC3D_CYCL_4 (4ULL << 9)
#define BC3D_SYMP_4 (5ULL << 9)
#define BC3D_4(i) ((unsigned long long)(i) << 9)
#define BC3D_WALL_5 (1ULL << 12)
#define BC3D_INLT_5 (2ULL << 12)
#define BC3D_OUTL_5 (3ULL << 12)
#define BC3D_CYCL_5 (4ULL << 12)
#define BC3D_SYMP_5 (5ULL << 12)
#define BC3D_5(i) ((unsigned long long)(i) << 12)
#define BC3D_WALL_6 (1ULL << 15)
#define BC3D_INLT_6 (2ULL << 15)
#define BC3D_OUTL_6 (3ULL << 15)
#define BC3D_CYCL_6 (4ULL << 15)
#define BC3D_SYMP_6 (5ULL << 15)
#define BC3D_6(i) ((unsigned long long)(i) << 15)
#define BC3D_WALL_7 (1ULL << 18)
#define BC3D_INLT_7 (2ULL << 18)
#define BC3D_OUTL_7 (3ULL << 18)
#define BC3D_CYCL_7 (4ULL << 18)
#define BC3D_SYMP_7 (5ULL << 18)
#define BC3D_7(i) ((unsigned long long)(i) << 18)
#define BC3D_WALL_8 (1ULL << 21)
#define BC3D_INLT_8 (2ULL << 21)
#define BC3D_OUTL_8 (3ULL << 21)
#define BC3D_CYCL_8 (4ULL << 21)
#define BC3D_SYMP_8 (5ULL << 21)
#define BC3D_8(i) ((unsigned long long)(i) << 21)
#define BC3D_WALL_9 (1ULL << 24)
#define BC3D_INLT_9 (2ULL << 24)
#define BC3D_OUTL_9 (3ULL << 24)
#define BC3D_CYCL_9 (4ULL << 24)
#define BC3D_SYMP_9 (5ULL << 24)
#define BC3D_9(i) ((unsigned long long)(i) << 24)
#define BC3D_WALL_10 (1ULL << 27)
#define BC3D_INLT_10 (2ULL << 27)
#define BC3D_OUTL_10 (3ULL << 27)
#define BC3D_CYCL_10 (4ULL << 27)
#define BC3D_SYMP_10 (5ULL << 27)
#define BC3D_10(i) ((unsigned long long)(i) << 27)
#define BC3D_WALL_11 (1ULL << 30)
#define BC3D_INLT_11 (2ULL << 30)
#define BC3D_OUTL_11 (3ULL << 30)
#define BC3D_CYCL_11 (4ULL << 30)
#define BC3D_SYMP_11 (5ULL << 30)
#define BC3D_11(i) ((unsigned long long)(i) << 30)
#define BC3D_WALL_12 (1ULL << 33)
#define BC3D_INLT_12 (2ULL << 33)
#define BC3D_OUTL_12 (3ULL << 33)
#define BC3D_CYCL_12 (4ULL << 33)
#define BC3D_SYMP_12 (5ULL << 33)
#define BC3D_12(i) ((unsigned long long)(i) << 33)
#define BC3D_WALL_13 (1ULL << 36)
#define BC3D_INLT_13 (2ULL << 36)
#define BC3D_OUTL_13 (3ULL << 36)
#define BC3D_CYCL_13 (4ULL << 36)
#define BC3D_SYMP_13 (5ULL << 36)
#define BC3D_13(i) ((unsigned long long)(i) << 36)
#define BC3D_WALL_14 (1ULL << 39)
#define BC3D_INLT_14 (2ULL << 39)
#define BC3D_OUTL_14 (3ULL << 39)
#define BC3D_CYCL_14 (4ULL << 39)
#define BC3D_SYMP_14 (5ULL << 39)
#define BC3D_14(i) ((unsigned long long)(i) << 39)
#define BC3D_WALL_15 (1ULL << 42)
#define BC3D_INLT_15 (2ULL << 42)
#define BC3D_OUTL_15 (3ULL << 42)
#define BC3D_CYCL_15 (4ULL << 42)
#define BC3D_SYMP_15 (5ULL << 42)
#define BC3D_15(i) ((unsigned long long)(i) << 42)
#define BC3D_WALL_16 (1ULL << 45)
#define BC3D_INLT_16 (2ULL << 45)
#define BC3D_OUTL_16 (3ULL << 45)
#define BC3D_CYCL_16 (4ULL << 45)
#define BC3D_SYMP_16 (5ULL << 45)
#define BC3D_16(i) ((unsigned long long)(i) << 45)
#define BC3D_WALL_17 (1ULL << 48)
#define BC3D_INLT_17 (2ULL << 48)
#define BC3D_OUTL_17 (3ULL << 48)
#define BC3D_CYCL_17 (4ULL << 48)
#define BC3D_SYMP_17 (5ULL << 48)
#define BC3D_17(i) ((unsigned long long)(i) << 48)
#define BC3D_WALL_18 (1ULL << 51)
#define BC3D_INLT_18 (2ULL << 51)
#define BC3D_OUTL_18 (3ULL << 51)
#define BC3D_CYCL_18 (4ULL << 51)
#define BC3D_SYMP_18 (5ULL << 51)
#define BC3D_18(i) ((unsigned long long)(i) << 51)
#define BC3D_WALL_B (1ULL << 54)
#define BC3D_INLT_B (2ULL << 54)
#define BC3D_OUTL_B (3ULL << 54)
#define BC3D_CYCL_B (4ULL << 54)
#define BC3D_SYMP_B (5ULL << 54)
#define BC3D_ALL_B (7ULL << 54)
#define BC3D_CORNER (1ULL << 57)
#define BC3D_FLUID (1ULL << 58)
#define BC3D_B(i) ((unsigned long long)(i) << 54)
#define BC3D_C(i) ((unsigned long long)(i) << 57)
#define BC3D_F(i) ((unsigned long long)(i) << 58)
