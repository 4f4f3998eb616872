// Row-staged time step: a persistent kernel whose populations arrive in
// shared memory by bulk asynchronous copies (cp.async.bulk, the 1D form of
// the tensor-memory accelerator) instead of per-thread loads.
//
// Work unit: one x-row (y, z) of the lattice.  For a row the kernel needs,
// per direction d, the row (y - c_d.y, z - c_d.z) of array d (the pull
// source; the x shift is an index shift inside shared memory), the row's
// flag words, and, for the directions that some fluid node of the row cannot
// pull across (bounce-back), the row itself of array opp(d).  The host lists
// the rows that hold fluid nodes and, per row, which pull rows and which own
// rows are needed.
//
// One producer thread issues the copies of a row into a ring of stages and
// arms that stage's "full" mbarrier with the byte count; eight consumer warps
// wait on it, gather each node's populations from shared memory with the
// x shift, update the node (update_node: boundary conditions, moments,
// collision) and store the result to global memory with coalesced stores,
// then release the stage on its "empty" mbarrier.  Many rows are in flight
// per SM whatever the register count of the update, which is what keeps HBM
// busy: the per-thread-load kernels were bound by the loads a warp could
// keep outstanding.
//
// Physics mode only (the reference mode's wall copies need the pulled value
// itself, which this kernel provides too, but its 3D quirks are left to the
// one-node kernel).  Every wait is bounded: a wait that gives up sets
// *err, and the producer waits for the copies it issued before returning.
#pragma once
#include "lbm_step.cuh"

namespace lbm {

struct TmaRows {
    const int32_t *row;     // rows holding fluid nodes (y + ny z), in order
    const uint32_t *lmask;  // per listed row: directions whose pull row is copied
    const uint32_t *omask;  // per listed row: arrays whose own row is copied
    int nrows;
    int stages;
    unsigned int *err;      // non-zero after a wait gave up
};

constexpr int TMA_CONSUMER_WARPS = 8;
constexpr int TMA_CONSUMERS = TMA_CONSUMER_WARPS * 32;
constexpr int TMA_THREADS = TMA_CONSUMERS + 32;
constexpr int TMA_BARRIER_BYTES = 128;
constexpr long long TMA_WAIT_CYCLES = 4000000000LL;  // about 2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Wait for the phase of the given parity to complete; false if it did not
// within TMA_WAIT_CYCLES.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > TMA_WAIT_CYCLES) return false;
    return true;
}
// Global -> shared bulk copy; both addresses 16-byte aligned, bytes a
// multiple of 16.  Completion is counted on `bar`.
__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

// Bytes of one stage: flag words, Q pull rows, Q own rows.
__host__ __device__ constexpr uint32_t tma_stage_bytes(int q, int nx, int elem) {
    return (uint32_t)nx * 4u + 2u * (uint32_t)q * (uint32_t)nx * (uint32_t)elem;
}

template <int Q, int COLL, int ST>
__global__ void __launch_bounds__(TMA_THREADS) step_kernel_tma(const StepParams p, const TmaRows rows) {
    using S = Store<ST>;
    using T = typename S::T;
    using R = typename S::R;
    using L = Lat<Q>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int nst = rows.stages;
    const int nx = p.nx;
    const uint32_t rowb = (uint32_t)nx * (uint32_t)sizeof(T);
    const uint32_t stage_bytes = tma_stage_bytes(Q, nx, (int)sizeof(T));
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem);  // full[nst], empty[nst]
    unsigned char *stage0 = smem + TMA_BARRIER_BYTES;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < nst; ++s) {
            mbar_init(smem_addr(bars + s), 1);
            mbar_init(smem_addr(bars + nst + s), TMA_CONSUMER_WARPS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == TMA_CONSUMER_WARPS) {
        // ---- producer: one thread ----
        if (lane != 0) return;
        int issued = 0;
        for (int k = blockIdx.x; k < rows.nrows; k += gridDim.x, ++issued) {
            const int s = issued % nst;
            const uint32_t use = (uint32_t)(issued / nst);
            if (!mbar_wait(smem_addr(bars + nst + s), (use & 1u) ^ 1u)) {
                atomicExch(rows.err, 1u);
                break;
            }
            const int r = rows.row[k];
            const uint32_t lm = rows.lmask[k], om = rows.omask[k];
            const uint32_t full = smem_addr(bars + s);
            mbar_arrive_expect_tx(full, (uint32_t)nx * 4u + (uint32_t)(__popc(lm) + __popc(om)) * rowb);
            unsigned char *st = stage0 + (size_t)s * stage_bytes;
            bulk_copy_g2s(smem_addr(st), p.word + (size_t)r * nx, (uint32_t)nx * 4u, full);
            const int y = r % p.ny, z = r / p.ny;
            unsigned char *pull = st + (size_t)nx * 4;
#pragma unroll
            for (int d = 0; d < Q; ++d) {
                if (!((lm >> d) & 1u)) continue;
                int sy = y - L::cy(d), sz = z - L::cz(d);
                sy = sy < 0 ? sy + p.ny : (sy >= p.ny ? sy - p.ny : sy);
                sz = sz < 0 ? sz + p.nz : (sz >= p.nz ? sz - p.nz : sz);
                const size_t src_row = (size_t)sy + (size_t)p.ny * sz;
                bulk_copy_g2s(smem_addr(pull + (size_t)d * rowb), (const T *)p.fin[d] + src_row * p.pitch, rowb,
                              full);
            }
            unsigned char *own = pull + (size_t)Q * rowb;
#pragma unroll
            for (int e = 0; e < Q; ++e) {
                if (!((om >> e) & 1u)) continue;
                bulk_copy_g2s(smem_addr(own + (size_t)e * rowb), (const T *)p.fin[e] + (size_t)r * p.pitch, rowb,
                              full);
            }
        }
        // Copies still in flight must land before the block's shared memory
        // goes away: wait for the last armed phase of every stage.
        for (int s = 0; s < nst && s < issued; ++s) {
            const int last = ((issued - 1 - s) / nst) * nst + s;  // last use index armed on stage s
            if (!mbar_wait(smem_addr(bars + s), (uint32_t)(last / nst) & 1u)) atomicExch(rows.err, 3u);
        }
        return;
    }

    // ---- consumers: eight warps ----
    const int ct = threadIdx.x;
    int used = 0;
    for (int k = blockIdx.x; k < rows.nrows; k += gridDim.x, ++used) {
        const int s = used % nst;
        const uint32_t use = (uint32_t)(used / nst);
        // every lane waits; the warp leaves together if any lane gave up
        const bool ok = mbar_wait(smem_addr(bars + s), use & 1u);
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) atomicExch(rows.err, 2u);
            return;
        }
        const unsigned char *st = stage0 + (size_t)s * stage_bytes;
        const uint32_t *wrow = reinterpret_cast<const uint32_t *>(st);
        const T *pull = reinterpret_cast<const T *>(st + (size_t)nx * 4);
        const T *own = pull + (size_t)Q * nx;
        const int r = rows.row[k];
        for (int x = ct; x < nx; x += TMA_CONSUMERS) {
            const uint32_t w = wrow[x];
            const int node = r * nx + x;       // flag words and macroscopic fields
            const long long idx = (long long)r * p.pitch + x;  // populations
            if (!(w & W_FLUID)) {
                // solid nodes keep the zero encoding; writing it keeps the
                // warp's stores sector-complete
#pragma unroll
                for (int d = 0; d < Q; ++d) ((T *)p.fout[d])[idx] = S::encode((R)0, p.shift[d], p.scale);
                continue;
            }
            const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
            R f[Q];
#pragma unroll
            for (int d = 0; d < Q; ++d) {
                const int sx = L::cx(d) == 1 ? xm : (L::cx(d) == -1 ? xp : x);
                T v = pull[d * nx + sx];
                if (d != 0 && ((w >> d) & 1u)) v = own[L::opp(d) * nx + x];
                f[d] = S::decode(v, p.shift[d], p.inv_scale);
            }
            update_node<Q, COLL, ST, true, true, DynGeom>(f, w, node, p, DynGeom{p.nx, p.ny, p.nz, p.pitch});
#pragma unroll
            for (int d = 0; d < Q; ++d) S::store((T *)p.fout[d] + idx, f[d], p.shift[d], p.scale);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(bars + nst + s));
    }
}

}  // namespace lbm
