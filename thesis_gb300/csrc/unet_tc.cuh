// 3x3 convolution as an implicit GEMM on the fifth-generation tensor cores
// (tcgen05.mma, accumulator in tensor memory), for sm_100-class GPUs.
//
//   out[n, y, x0+m, co] = act(bias[co] + sum_{tap, ci} w[tap][co][ci] in[n, y+ky-1, x0+m+kx-1, ci])
//
// One CTA (4 warps) owns TC_M = 128 consecutive pixels of one image row: the
// GEMM's M.  N = COUT output channels (32, 64, 128 or 256), K = 9 taps x cin,
// taken CHUNK input channels at a time.  Per chunk the CTA stages in shared
// memory
//   A  the three input rows the taps read, 130 pixels (one-pixel halo) x
//      CHUNK channels, and
//   B  the weights of all nine taps for those channels, COUT x CHUNK each,
// both in the K-major "no swizzle" layout of the tensor cores' shared-memory
// descriptors: core matrices of 8 rows x 16 bytes (8 BF16 along K) stored as
// 128 contiguous bytes.  Rows (pixels, output channels) are 16 bytes apart,
// and the 8-channel groups of K are whole planes apart:
//   A byte (row r, group j, pixel p) = ((r * KG + j) * NP + p) * 16
//   B byte (tap t, group j, chan co) = ((t * KG + j) * COUT + co) * 16
// so a core matrix starts at any pixel, and the tap's x shift kx is a start
// address kx * 16 bytes further: one A stage serves all nine taps.  The
// descriptor's leading byte offset (between the two 8-channel groups of one
// K = 16 instruction) is a plane, NP * 16 or COUT * 16 bytes; its stride
// byte offset (between 8-row groups along M or N) is 128 bytes.
//
// One thread issues the chunk's 9 x CHUNK/16 MMAs (M = 128, N = COUT,
// K = 16, BF16 in, FP32 accumulate) and commits them to an mbarrier; every
// thread waits on it before the next chunk overwrites the stages.  The
// epilogue reads each warp's 32 TMEM lanes (its 32 pixels) 16 columns at a
// time, adds the bias, applies ReLU and stores BF16 (and FP32 if asked).
// Every wait is bounded: a wait that gives up sets *err, the CTA skips the
// rest of its MMAs, waits (bounded) for the ones in flight, frees its tensor
// memory and returns.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace unet_tc {

constexpr int TC_M = 128;             // pixels per CTA (GEMM rows)
constexpr int TC_NP = TC_M + 2;       // staged pixels per row (halo)
constexpr long long TC_SPIN = 1ll << 26;  // bounded mbarrier polls

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (all in 16-byte units), the fixed version field (bits 46-47 = 1),
// base offset 0 and layout type 0 (no swizzle).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A
// and B BF16 (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17,
// M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// true once phase `parity` of the barrier has completed; false after
// TC_SPIN polls
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (long long i = 0; i < TC_SPIN; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <int COUT, int CHUNK>
struct TcSmem {
    static constexpr int KG = CHUNK / 8;
    static constexpr int A_BYTES = 3 * KG * TC_NP * 16;
    static constexpr int B_BYTES = 9 * KG * COUT * 16;
    static constexpr int BYTES = A_BYTES + B_BYTES + 16;  // + mbarrier and TMEM address
};

template <int COUT, int CHUNK>
__global__ void __launch_bounds__(128, 1)
conv3x3_tc_kernel(const __nv_bfloat16 *__restrict__ in, int in_cs, int in_co, int cin,
                  const __nv_bfloat16 *__restrict__ w, const float *__restrict__ bias, __nv_bfloat16 *__restrict__ out,
                  int out_cs, int out_co, float *__restrict__ out32, int H, int W, int relu, int *err) {
    using SM = TcSmem<COUT, CHUNK>;
    constexpr int KG = SM::KG;
    constexpr uint32_t COLS = COUT < 32 ? 32 : COUT;  // TMEM columns (a power of two >= 32)
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *sA = smem, *sB = smem + SM::A_BYTES;
    uint64_t *mbar = (uint64_t *)(smem + SM::A_BYTES + SM::B_BYTES);
    uint32_t *tmem_slot = (uint32_t *)(mbar + 1);
    const int x0 = blockIdx.x * TC_M, y = blockIdx.y, n = blockIdx.z;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t mbar_a = smem_u32(mbar);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) mbar_init(mbar_a, 1);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    constexpr uint32_t IDESC = idesc_bf16(TC_M, COUT);
    bool ok = true;
    int chunks = 0;

    for (int c0 = 0; c0 < cin && ok; c0 += CHUNK) {
        const int kg = (cin - c0 >= CHUNK ? CHUNK : cin - c0) / 8;  // 8-channel groups in this chunk (even)
        if (chunks > 0) {
            // the previous chunk's MMAs read the stages: wait before overwriting
            if (!mbar_wait(mbar_a, (uint32_t)((chunks - 1) & 1))) ok = false;
            fence_after();
        }
        // every thread reaches this barrier, so a failed wait is seen by all
        if (!__syncthreads_and(ok ? 1 : 0)) {
            ok = false;
            break;
        }
        // A: three input rows, 130 pixels, kg groups of 8 channels
        for (int i = tid; i < 3 * kg * TC_NP; i += 128) {
            const int r = i / (kg * TC_NP), rem = i % (kg * TC_NP), j = rem / TC_NP, p = rem % TC_NP;
            const int gy = y + r - 1, gx = x0 + p - 1;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gy >= 0 && gy < H && gx >= 0 && gx < W)
                v = *(const uint4 *)(in + (((size_t)n * H + gy) * W + gx) * in_cs + in_co + c0 + 8 * j);
            *(uint4 *)(sA + ((size_t)(r * KG + j) * TC_NP + p) * 16) = v;
        }
        // B: nine taps x COUT output channels x kg groups
        for (int i = tid; i < 9 * kg * COUT; i += 128) {
            const int t = i / (kg * COUT), rem = i % (kg * COUT), j = rem / COUT, co = rem % COUT;
            const uint4 v = *(const uint4 *)(w + ((size_t)t * COUT + co) * cin + c0 + 8 * j);
            *(uint4 *)(sB + ((size_t)(t * KG + j) * COUT + co) * 16) = v;
        }
        fence_proxy_async();  // the stores above become visible to the tensor cores
        __syncthreads();
        if (tid == 0) {
            fence_after();
            const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
#pragma unroll 1
            for (int t = 0; t < 9; ++t) {
                const int ky = t / 3, kx = t % 3;
#pragma unroll 1
                for (int s = 0; s < kg / 2; ++s) {
                    const uint32_t aa = a0 + (uint32_t)(((ky * KG + 2 * s) * TC_NP + kx) * 16);
                    const uint32_t bb = b0 + (uint32_t)(((t * KG + 2 * s) * COUT) * 16);
                    mma_bf16(tmem, smem_desc(aa, TC_NP * 16, 128), smem_desc(bb, COUT * 16, 128), IDESC,
                             (c0 > 0 || t > 0 || s > 0) ? 1u : 0u);
                }
            }
            mma_commit(mbar_a);
        }
        ++chunks;
    }
    // the last chunk's MMAs (or, after a failure, whatever is in flight)
    if (chunks > 0 && !mbar_wait(mbar_a, (uint32_t)((chunks - 1) & 1))) ok = false;
    fence_after();
    if (!__syncthreads_and(ok ? 1 : 0)) ok = false;
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
    } else {
        const int p = warp * 32 + lane;  // TMEM lane = GEMM row = pixel
        const int x = x0 + p;
        const size_t pix = ((size_t)n * H + y) * W + x;
#pragma unroll 1
        for (int c = 0; c < COUT; c += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
            if (x < W) {
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    if (bias) v[i] += bias[c + i];
                    if (relu) v[i] = fmaxf(v[i], 0.f);
                }
                if (out) {
                    uint32_t pk[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
                        pk[i] = *(const uint32_t *)&h2;
                    }
                    uint4 *o = (uint4 *)(out + pix * out_cs + out_co + c);
                    o[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    o[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                }
                if (out32) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) out32[pix * COUT + c + i] = v[i];
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(COLS) : "memory");
}

}  // namespace unet_tc
