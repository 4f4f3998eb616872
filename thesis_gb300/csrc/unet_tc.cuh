// 3x3 convolutions of the warm-start U-Net on the fifth-generation tensor
// cores (tcgen05.mma, accumulators in tensor memory, operands staged by
// tensor copies), for sm_100-class GPUs.
//
// Forward and data gradient (conv3x3_tc_kernel):
//
//   out[n, y, x0+m, co] = act(bias[co] + sum_{tap, ci} w[tap][co][ci] in[n, y+ky-1, x0+m+kx-1, ci])
//
// A tile is TC_M = 128 consecutive pixels of one image row: the GEMM's M.
// N = COUT output channels (16, 32, 64 or 128), K = 9 taps x cin, taken CHUNK
// (16, 32 or 64) input channels at a time; a job is one (tile, chunk).  The
// kernel is persistent: CTA b walks tiles b, b + gridDim.x, ...  Shared
// memory holds
//   B  every weight of the layer (9 taps x cin x COUT), loaded once, in the
//      K-major no-swizzle layout: core matrices of 8 rows x 16 bytes stored
//      as 128 contiguous bytes, byte ((t * KGall + j) * COUT + co) * 16 for
//      tap t, 8-channel group j, output channel co;
//   A  NS stages of input rows: one tensor copy per job brings the three
//      rows the taps read, TC_BOX = 136 pixels from x0 - 1 (zero fill outside
//      the image) x CHUNK channels, as K-major rows of 2 x CHUNK bytes with
//      the tensor copy's 128-, 64- or 32-byte swizzle.
// The tap's x shift kx is a start address kx rows further inside the same
// staged row: the hardware applies the swizzle to absolute shared-memory
// address bits, so a start moved by whole rows (or by 32 bytes for the next
// K = 16) reads the right elements with the descriptor's base offset 0.
//
// Warp 4 (one thread) issues the copies and each job's 9 x CHUNK/16 MMAs
// (M = 128, N = COUT, K = 16, BF16 in, FP32 accumulate); warps 0-3 read
// finished tiles from NA tensor-memory accumulators (each warp its 32 lanes =
// 32 pixels), add the bias, apply ReLU and store BF16 (and FP32 if asked),
// while the next tiles accumulate.  Every wait is bounded: a wait that gives
// up sets *err, both roles stop, the copies and MMAs in flight finish, the
// tensor memory is freed and the kernel returns.
//
// Weight gradient (wgrad_tc_kernel): see its comment below.
#pragma once
#include <cuda.h>
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
// TC_SPIN polls, or as soon as *stop (when given) is set
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, volatile int *stop = nullptr) {
    for (long long i = 0; i < TC_SPIN; ++i) {
        if (stop && (i & 1023) == 1023 && *stop) return false;
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

// 16 bytes global -> shared without a register round trip; src_bytes 0
// writes zeros (the source is then not read)
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Swizzled K-major operand descriptor (tcgen05 layout types 2, 4, 6 for
// 128-, 64- and 32-byte rows): rows of ROWB bytes, 8-row groups 8 x ROWB
// bytes apart.  The hardware applies the swizzle to absolute shared-memory
// address bits, so a start address moved by whole rows (the tap shift) or by
// 32 bytes (the next K = 16) inside a swizzle atom reads the matching
// elements with base offset 0, as long as the tensor copy wrote the atoms at
// their absolute addresses.
template <int ROWB>
__device__ __forceinline__ uint64_t smem_desc_sw(uint32_t addr) {
    constexpr uint64_t layout = ROWB == 128 ? 2 : (ROWB == 64 ? 4 : 6);
    return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)((8 * ROWB) >> 4) << 32) | (1ull << 46) |
           (layout << 61);
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// Tiled tensor copy of a 4-D box (c, x, y, n) into shared memory, completing
// on mbar.  The innermost coordinate c is a multiple of 8 channels (16 bytes).
__device__ __forceinline__ void tma_load4(uint32_t dst, const void *tmap, int c, int x, int y, int n, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(tmap), "r"(c), "r"(x), "r"(y), "r"(n), "r"(mbar)
        : "memory");
}

constexpr int TC_BOX = 136;  // staged pixels per row: x0 - 1 .. x0 + 134, a whole number of swizzle atoms

template <int COUT, int CHUNK, int NS>
struct TcSmem {
    // tensor-memory accumulators: a tile's MMAs wait for the epilogue of the
    // tile NA before it, so NA tiles overlap one accumulator round trip
    // (commit, epilogue, release); NA x COUT columns
    static constexpr int NA = 4 * COUT <= 512 ? 4 : 2;
    static constexpr int ROWB = CHUNK * 2;
    static constexpr int A_STAGE = 3 * TC_BOX * ROWB;
    static constexpr size_t bytes(int cin) {
        return 1024 + NS * (size_t)A_STAGE + 18 * (size_t)cin * COUT + 4 * COUT + 8 * (2 * NS + 2 * NA) + 16;
    }
};

// Warp roles: warps 0-3 read the accumulators (each its 32 TMEM lanes) and
// store the outputs; one thread of warp 4 issues the tensor copies and the
// MMAs.  Barriers (all counts 1 except acc_empty, 4):
//   full[s]      stage s holds its job's rows (tensor-copy bytes)
//   empty[s]     the MMAs that read stage s are done (tcgen05.commit)
//   acc_full[a]  accumulator a holds a finished tile (tcgen05.commit)
//   acc_empty[a] the four epilogue warps have read accumulator a
template <int COUT, int CHUNK, int NS>
__global__ void __launch_bounds__(160, 1)
conv3x3_tc_kernel(const __grid_constant__ CUtensorMap tin, int cin, const __nv_bfloat16 *__restrict__ w,
                  const float *__restrict__ bias, __nv_bfloat16 *__restrict__ out, int out_cs, int out_co,
                  float *__restrict__ out32, int B, int H, int W, int relu, int *err) {
    static_assert(COUT % 16 == 0 && COUT <= 128 && (CHUNK == 16 || CHUNK == 32 || CHUNK == 64), "N, K chunk");
    static_assert(NS >= 2 && NS <= 4, "input stages");
    using SM = TcSmem<COUT, CHUNK, NS>;
    constexpr int ROWB = SM::ROWB, KG = CHUNK / 8;
    constexpr uint32_t A_STAGE = SM::A_STAGE;
    constexpr int NA = SM::NA;
    constexpr uint32_t COLS = NA * COUT < 32 ? 32 : NA * COUT;  // a power of two >= 32
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw), base = (raw + 1023u) & ~1023u;
    unsigned char *smem = smem_raw + (base - raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int KGall = cin / 8, nch = cin / CHUNK;
    const uint32_t b_base = base + NS * A_STAGE;
    float *sbias = (float *)(smem + NS * A_STAGE + (size_t)18 * cin * COUT);
    uint64_t *bars = (uint64_t *)(sbias + COUT);
    const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * NS, accf0 = empty0 + 8 * NS, acce0 = accf0 + 8 * NA;
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * NS + 2 * NA);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    const int xt = (W + TC_M - 1) / TC_M;
    const long long ntiles = (long long)B * H * xt;
    const long long my_tiles = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const long long jobs = my_tiles * nch;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int k = 0; k < NS; ++k) {
            mbar_init(full0 + 8 * k, 1);
            mbar_init(empty0 + 8 * k, 1);
        }
        for (int a = 0; a < NA; ++a) {
            mbar_init(accf0 + 8 * a, 1);
            mbar_init(acce0 + 8 * a, 4);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (tid < COUT) sbias[tid] = bias ? bias[tid] : 0.f;
    // every weight of the layer, no swizzle: byte ((t * KGall + j) * COUT + co) * 16
    for (int i = tid; i < 9 * KGall * COUT; i += 160) {
        const int tc = i / KGall, j = i % KGall, t = tc / COUT, co = tc % COUT;
        cp_async16(b_base + (uint32_t)(((t * KGall + j) * COUT + co) * 16), w + (size_t)i * 8, 16);
    }
    cp_async_commit();
    cp_async_wait<0>();
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    bool ok = true;

    if (warp == 4) {
        if (lane == 0) {
            constexpr uint32_t IDESC = idesc_bf16(TC_M, COUT);
            // the CTA's job j: tile blockIdx.x + (j / nch) gridDim.x, chunk j % nch
            auto load = [&](long long j) {
                const long long tile = blockIdx.x + (j / nch) * gridDim.x;
                const int xb = (int)(tile % xt);
                const long long ny = tile / xt;
                const uint32_t s = (uint32_t)(j % NS), fb = full0 + 8 * s;
                mbar_expect_tx(fb, A_STAGE);
                tma_load4(base + s * A_STAGE, &tin, (int)(j % nch) * CHUNK, xb * TC_M - 1, (int)(ny % H) - 1,
                          (int)(ny / H), fb);
            };
            long long issued = 0, committed = 0;
            for (; issued < jobs && issued < NS; ++issued) load(issued);
            for (long long j = 0; j < jobs && ok; ++j) {
                const long long k = j / nch;
                const int c = (int)(j % nch), s = (int)(j % NS), a = (int)(k % NA);
                if (!mbar_wait(full0 + 8 * s, (uint32_t)((j / NS) & 1), abort_flag)) ok = false;
                // the epilogue of tile k - NA has read accumulator a
                if (ok && c == 0 && k >= NA && !mbar_wait(acce0 + 8 * a, (uint32_t)((k / NA - 1) & 1), abort_flag))
                    ok = false;
                if (!ok || *abort_flag) {
                    ok = false;
                    break;
                }
                fence_after();
                const uint64_t da = smem_desc_sw<ROWB>(base + (uint32_t)s * A_STAGE);
                const uint64_t db = smem_desc(b_base + (uint32_t)(c * KG * COUT * 16), COUT * 16, 128);
                const uint32_t d = tmem + (uint32_t)(a * COUT);
#pragma unroll
                for (int t = 0; t < 9; ++t) {
#pragma unroll
                    for (int q = 0; q < KG / 2; ++q)
                        mma_bf16(d, da + (uint64_t)(((t / 3) * TC_BOX + t % 3) * ROWB / 16 + 2 * q),
                                 db + (uint64_t)((t * KGall + 2 * q) * COUT), IDESC,
                                 (c > 0 || t > 0 || q > 0) ? 1u : 0u);
                }
                mma_commit(empty0 + 8 * s);
                if (c == nch - 1) mma_commit(accf0 + 8 * a);
                committed = j + 1;
                // refill the stage of job j - 1, whose MMAs were issued before
                if (j >= 1 && issued < jobs) {
                    const long long jr = j - 1;
                    if (!mbar_wait(empty0 + 8 * (uint32_t)(jr % NS), (uint32_t)((jr / NS) & 1), abort_flag)) {
                        ok = false;
                        break;
                    }
                    load(issued++);
                }
            }
            if (!ok) {
                *abort_flag = 1;
                atomicExch(err, 1);
                // the tensor copies and MMAs in flight finish before the CTA
                // leaves: the last use of each stage, and the last commit
                // (MMAs complete in order)
                for (long long j = issued > NS ? issued - NS : 0; j < issued; ++j)
                    mbar_wait(full0 + 8 * (uint32_t)(j % NS), (uint32_t)((j / NS) & 1));
                if (committed > 0)
                    mbar_wait(empty0 + 8 * (uint32_t)((committed - 1) % NS), (uint32_t)(((committed - 1) / NS) & 1));
            }
        }
        __syncwarp();
    } else {
        // epilogue warps: tile k from accumulator k % NA
        for (long long k = 0; k < my_tiles; ++k) {
            const int a = (int)(k % NA);
            const bool got = mbar_wait(accf0 + 8 * a, (uint32_t)((k / NA) & 1), abort_flag);
            if (!__all_sync(0xffffffffu, got)) {
                ok = false;
                break;
            }
            fence_after();
            const long long tile = blockIdx.x + k * gridDim.x;
            const int xb = (int)(tile % xt);
            const long long ny = tile / xt;
            const int y = (int)(ny % H), n = (int)(ny / H);
            const int x = xb * TC_M + warp * 32 + lane;  // TMEM lane = GEMM row = pixel
            const size_t pix = ((size_t)n * H + y) * W + x;
            const uint32_t acc = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(a * COUT);
#pragma unroll 1
            for (int c = 0; c < COUT; c += 16) {
                float v[16];
                tmem_ld16(acc + (uint32_t)c, v);
                if (x < W) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        v[i] += sbias[c + i];
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
                        float4 *o = (float4 *)(out32 + pix * COUT + c);
#pragma unroll
                        for (int i = 0; i < 4; ++i)
                            o[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
                    }
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(acce0 + 8 * a);
        }
        if (!ok) {
            *abort_flag = 1;
            if (lane == 0) atomicExch(err, 1);
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(COLS) : "memory");
}

// dst[0..3] += (a, b, c, d) in one vector reduction; dst 16-byte aligned
__device__ __forceinline__ void red_add4(float *dst, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}

// Weight gradient on the tensor cores:
//
//   dw[ky][kx][co][ci] += sum_{n, y, x} dpre[n, y, x, co] in[n, y+ky-1, x+kx-1, ci]
//
// A job is one input row y and TC_M = 128 output pixels x0 .. x0+127: the
// GEMM's K.  Input row y meets output-gradient row y - ky + 1 in tap row ky.
// One tensor copy stages the output-gradient rows y-1, y, y+1 (128 pixels x
// CO channels each); the A operand stacks them along M as (row, co), so M
// row m holds channel m % CO of row y - 1 + m / CO, i.e. tap row
// ky = 2 - m / CO, in M_BLOCKS blocks of 128 (rows past 3 x CO read staging
// memory no result uses: the input row or the next stage).  A second copy
// stages the input row (TC_BOX pixels from x0 - 1) right after the three
// rows, for NC input channels: the B operand, whose tap shift
// kx is a start address kx pixel rows further.  Both operands are
// channel-contiguous per pixel, "MN-major" (the instruction descriptor's
// transpose bits), swizzled by their row bytes (2 x CO and 2 x NC): the
// leading byte offset steps between channel blocks along M (one staged row
// of 128 pixels), the stride byte offset between groups of 8 pixels along K.
// The accumulators D[block][kx] (128 lanes x NC columns) stay in tensor
// memory across all of a CTA's jobs and are added to dw at the end with
// 16-byte vector reductions (dw, cin and NC keep every group of four columns
// aligned); a layer wider than NC input channels is split over gridDim.y.
// One thread issues the copies (NS stages) and the MMAs; every wait is
// bounded.
template <int CO, int NC, int NS>
struct WgSmem {
    static constexpr int ROWB_A = CO * 2, ROWB_B = NC * 2;
    static constexpr int M_BLOCKS = 3 * CO > 128 ? 2 : 1;
    // The copy writes the three rows (A_ROWS bytes, a whole number of 1 KB
    // swizzle atoms) and B right after them; the MMAs of an M block read
    // 128 rows of CO channels from the stage start (A_SPAN bytes), so the
    // rows past 3 x CO fall on B or the next stage: in bounds, and they only
    // feed accumulator rows no result uses.  TAIL keeps the last stage's
    // span inside the allocation.
    static constexpr int A_ROWS = 3 * TC_M * ROWB_A;
    static constexpr int A_STAGE = A_ROWS;                        // offset of B in a stage
    static constexpr int A_SPAN = M_BLOCKS * 128 * TC_M * 2;
    static constexpr int B_STAGE = TC_BOX * ROWB_B;
    static constexpr int STAGE = (A_STAGE + B_STAGE + 1023) / 1024 * 1024;
    static constexpr int TAIL = A_SPAN > STAGE ? A_SPAN - STAGE : 0;
    static constexpr int BYTES = 1024 + NS * STAGE + TAIL + 16 * NS + 16;
    static constexpr int USED = M_BLOCKS * 3 * NC;
    static constexpr uint32_t COLS = USED <= 32 ? 32 : USED <= 64 ? 64 : USED <= 128 ? 128 : USED <= 256 ? 256 : 512;
};

// Swizzled MN-major operand descriptor: rows of ROWB bytes along K (one per
// pixel), lbo between channel blocks along M or N, 8-row groups 8 x ROWB
// bytes apart along K.
template <int ROWB>
__device__ __forceinline__ uint64_t smem_desc_sw_mn(uint32_t addr, uint32_t lbo) {
    constexpr uint64_t layout = ROWB == 128 ? 2 : (ROWB == 64 ? 4 : 6);
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((8 * ROWB) >> 4) << 32) | (1ull << 46) | (layout << 61);
}

template <int CO, int NC, int NS>
__global__ void __launch_bounds__(128, 1)
wgrad_tc_kernel(const __grid_constant__ CUtensorMap tdp, const __grid_constant__ CUtensorMap tin, int cin,
                float *__restrict__ dw, int B, int H, int W, int *err) {
    static_assert((CO == 16 || CO == 32 || CO == 64) && (NC == 16 || NC == 32 || NC == 64), "swizzle rows");
    using SM = WgSmem<CO, NC, NS>;
    constexpr int MB = SM::M_BLOCKS, ROWB_A = SM::ROWB_A, ROWB_B = SM::ROWB_B;
    constexpr uint32_t STAGE = SM::STAGE, A_STAGE = SM::A_STAGE, COLS = SM::COLS;
    static_assert(SM::USED <= 512, "accumulators fit in tensor memory");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw), base = (raw + 1023u) & ~1023u;
    unsigned char *smem = smem_raw + (base - raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ci0 = blockIdx.y * NC;
    uint64_t *bars = (uint64_t *)(smem + NS * STAGE + SM::TAIL);
    const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * NS;
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * NS);
    const int xt = (W + TC_M - 1) / TC_M;
    const long long units = (long long)B * H * xt;
    const long long jobs = units > blockIdx.x ? (units - 1 - blockIdx.x) / gridDim.x + 1 : 0;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int k = 0; k < NS; ++k) {
            mbar_init(full0 + 8 * k, 1);
            mbar_init(empty0 + 8 * k, 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    // kind::f16, BF16 operands, FP32 accumulator, A and B MN-major
    constexpr uint32_t IDESC = idesc_bf16(TC_M, NC) | (1u << 15) | (1u << 16);
    __shared__ int status;  // 1: every MMA committed and complete

    if (tid == 0) {
        bool ok = true;
        auto load = [&](long long j) {
            const long long unit = blockIdx.x + j * gridDim.x;
            const int xb = (int)(unit % xt);
            const long long ny = unit / xt;
            const int y = (int)(ny % H), n = (int)(ny / H);
            const uint32_t s = (uint32_t)(j % NS), fb = full0 + 8 * s, dst = base + s * STAGE;
            mbar_expect_tx(fb, SM::A_ROWS + SM::B_STAGE);
            tma_load4(dst, &tdp, 0, xb * TC_M, y - 1, n, fb);
            tma_load4(dst + A_STAGE, &tin, ci0, xb * TC_M - 1, y, n, fb);
        };
        long long issued = 0, committed = 0;
        for (; issued < jobs && issued < NS; ++issued) load(issued);
        for (long long j = 0; j < jobs; ++j) {
            const uint32_t s = (uint32_t)(j % NS);
            if (!mbar_wait(full0 + 8 * s, (uint32_t)((j / NS) & 1))) {
                ok = false;
                break;
            }
            fence_after();
            const uint32_t a0 = base + s * STAGE;
            const uint64_t da = smem_desc_sw_mn<ROWB_A>(a0, TC_M * ROWB_A);
            const uint64_t db = smem_desc_sw_mn<ROWB_B>(a0 + A_STAGE, TC_BOX * ROWB_B);
#pragma unroll
            for (int ks = 0; ks < TC_M / 16; ++ks) {
#pragma unroll
                for (int b = 0; b < MB; ++b) {
#pragma unroll
                    for (int kx = 0; kx < 3; ++kx)
                        mma_bf16(tmem + (uint32_t)((b * 3 + kx) * NC),
                                 da + (uint64_t)((b * 128 * TC_M * 2 + 16 * ks * ROWB_A) / 16),
                                 db + (uint64_t)((16 * ks + kx) * ROWB_B / 16), IDESC, (j > 0 || ks > 0) ? 1u : 0u);
                }
            }
            mma_commit(empty0 + 8 * s);
            committed = j + 1;
            if (j >= 1 && issued < jobs) {
                const long long jr = j - 1;
                if (!mbar_wait(empty0 + 8 * (uint32_t)(jr % NS), (uint32_t)((jr / NS) & 1))) {
                    ok = false;
                    break;
                }
                load(issued++);
            }
        }
        // the last commit covers every MMA (they complete in order); copies
        // still in flight after a failure land before the CTA leaves
        if (committed > 0 &&
            !mbar_wait(empty0 + 8 * (uint32_t)((committed - 1) % NS), (uint32_t)(((committed - 1) / NS) & 1)))
            ok = false;
        if (!ok) {
            for (long long j = issued > NS ? issued - NS : 0; j < issued; ++j)
                mbar_wait(full0 + 8 * (uint32_t)(j % NS), (uint32_t)((j / NS) & 1));
            atomicExch(err, 1);
        }
        status = ok && committed == jobs ? 1 : 0;
    }
    __syncthreads();
    if (status && jobs > 0) {
        fence_after();
#pragma unroll
        for (int b = 0; b < MB; ++b) {
            const int m = b * 128 + warp * 32 + lane;  // TMEM lane of this thread in block b
            const int ky = 2 - m / CO, co = m % CO;
#pragma unroll 1
            for (int kx = 0; kx < 3; ++kx) {
#pragma unroll 1
                for (int c = 0; c < NC; c += 16) {
                    float v[16];
                    tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)((b * 3 + kx) * NC + c), v);
                    if (ky >= 0) {
                        float *d = dw + ((size_t)(ky * 3 + kx) * CO + co) * cin + ci0 + c;
#pragma unroll
                        for (int i = 0; i < 16; i += 4) red_add4(d + i, v[i], v[i + 1], v[i + 2], v[i + 3]);
                    }
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
