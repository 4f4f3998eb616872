// Batched independent domains: many lattices of uneven sizes (a sweep over
// geometry and Reynolds number) advanced together, one persistent launch per
// step over a packed tile table, with the step loop captured in a CUDA graph
// and per-domain FP64 residuals that retire converged domains from the table.
//
// The reference runs one lattice per process (Iterate2D/3D); this is the
// batched form of the same step (h_node: arithmetic in storage units, so a
// domain can reach a 1e-6 residual in FP32).  Every domain keeps its own row-layout
// population segment, flag words, macroscopic fields and boundary slots in
// shared device arrays, and its own StepParams record (four per domain:
// buffer parity x whether the step stores rho, u).  A tile is up to
// STEP_BLOCK consecutive nodes of one row of one domain; the kernel's blocks
// stride over the tile table, so small domains fill the GPU together instead
// of leaving it idle one launch at a time.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "lbm_flags.h"
#include "lbm_step_x2.cuh"
#include "thesis_lbm.h"

namespace lbm {

int launch_init_q9(const StepParams &p, const StepParams &o, int coll, int st, int phys, int eq, cudaStream_t s);
int launch_init_q19(const StepParams &p, const StepParams &o, int coll, int st, int phys, int eq, cudaStream_t s);
int launch_decode_q9(const StepParams &p, int st, double *out, long long n, cudaStream_t s);
int launch_decode_q19(const StepParams &p, int st, double *out, long long n, cudaStream_t s);

namespace {

// A tile is one warp's work: 32 consecutive nodes of BATCH_ROWS consecutive
// rows of one domain.  int4: x = domain, y = first row (y + ny z), z = first
// x, w = node index of (first x, first row) in the batch's macroscopic arrays.
constexpr int BATCH_WARPS = STEP_BLOCK / 32;
constexpr int BATCH_ROWS = 4;
constexpr int PARAM_WORDS = (int)(sizeof(StepParams) / 4);
static_assert(sizeof(StepParams) % 4 == 0, "StepParams is copied as 32-bit words");

// The warp's copy of its domain's step parameters, refreshed when the warp
// moves to a tile of another domain (tiles of a domain are contiguous).
__device__ __forceinline__ void batch_load_params(StepParams *dst, const StepParams *src) {
    const int lane = threadIdx.x & 31;
    const uint32_t *s = (const uint32_t *)src;
    uint32_t *d = (uint32_t *)dst;
    for (int k = lane; k < PARAM_WORDS; k += 32) d[k] = __ldg(s + k);
    __syncwarp();
}

template <int Q, int COLL, int ST, bool PHYS>
__global__ void __launch_bounds__(STEP_BLOCK)
batch_step_kernel(const StepParams *__restrict__ tab, const int4 *__restrict__ tiles, const int *__restrict__ count) {
    __shared__ StepParams sp[BATCH_WARPS];
    const int ntiles = *count;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    StepParams &p = sp[warp];
    int cur = -1;
    for (int t = blockIdx.x * BATCH_WARPS + warp; t < ntiles; t += gridDim.x * BATCH_WARPS) {
        const int4 tl = tiles[t];
        if (tl.x != cur) {
            __syncwarp();
            batch_load_params(&p, tab + tl.x);
            cur = tl.x;
        }
        const DynGeom g{p.nx, p.ny, p.nz, p.pitch};
        const int x = tl.z + lane;
        const int rows = g.ny * g.nz;
        const int r_end = min(tl.y + BATCH_ROWS, rows);
        const bool in_row = x < g.nx;
        // the next row's flag word is requested before the current row's update
        uint32_t w = in_row ? __ldg(p.word + x + g.nx * tl.y) : 0u;
#pragma unroll 1
        for (int r = tl.y; r < r_end; ++r) {
            const uint32_t wn = in_row && r + 1 < r_end ? __ldg(p.word + x + g.nx * (r + 1)) : 0u;
            h_node_w<Q, COLL, ST, PHYS, true, DynGeom, false, false>(p, g, x, r % g.ny, r / g.ny, w);
            w = wn;
        }
    }
}

// Per-tile FP64 partial sums of the velocity residual over fluid nodes:
// sum |u - u_prev|^2 and sum |u|^2; u_prev <- u.  Tiles of one domain are
// contiguous, so the per-domain totals (batch_residual_final) add partials in
// a fixed order: deterministic.
__global__ void __launch_bounds__(STEP_BLOCK)
batch_residual_partial(const StepParams *__restrict__ tab, const int4 *__restrict__ tiles,
                       const int *__restrict__ count, float *pu, double2 *partial) {
    const int ntiles = *count;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int t = blockIdx.x * BATCH_WARPS + warp; t < ntiles; t += gridDim.x * BATCH_WARPS) {
        const int4 tl = tiles[t];
        const StepParams &p = tab[tl.x];
        const int nx = p.nx, rows = p.ny * p.nz;
        const int x = tl.z + lane;
        const int r_end = min(tl.y + BATCH_ROWS, rows);
        double a = 0, b = 0;
        if (x < nx) {
            for (int r = tl.y; r < r_end; ++r) {
                const long long i = (long long)tl.w + (long long)(r - tl.y) * nx + lane;  // batch node index
                const int local = r * nx + x;
                if (p.word[local] & W_FLUID) {
                    const double u = p.ux[local], v = p.uy[local], w = p.uz[local];
                    const double du = u - pu[3 * i], dv = v - pu[3 * i + 1], dw = w - pu[3 * i + 2];
                    a += du * du + dv * dv + dw * dw;
                    b += u * u + v * v + w * w;
                    pu[3 * i] = (float)u;
                    pu[3 * i + 1] = (float)v;
                    pu[3 * i + 2] = (float)w;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
        if (lane == 0) partial[t] = make_double2(a, b);
    }
}

__global__ void batch_residual_final(const double2 *partial, const int2 *ranges, int ndom, double *res) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= ndom) return;
    const int2 r = ranges[d];
    if (r.y <= r.x) return;  // retired: keep its last residual
    double a = 0, b = 0;
    for (int t = r.x; t < r.y; ++t) {
        a += partial[t].x;
        b += partial[t].y;
    }
    res[d] = b > 0 ? sqrt(a) / sqrt(b) : (a > 0 ? INFINITY : 0.0);
    if (!isfinite(a) || !isfinite(b)) res[d] = NAN;
}

using BatchKernel = void (*)(const StepParams *, const int4 *, const int *);

BatchKernel batch_kernel(int q, int coll, int st, int phys) {
#define B_CASE(Q, C, S, P) \
    if (q == Q && coll == C && st == S && (phys != 0) == P) return batch_step_kernel<Q, C, S, P>;
    B_CASE(9, 1, 0, true) B_CASE(9, 2, 0, true) B_CASE(9, 3, 0, true)
    B_CASE(9, 1, 1, true) B_CASE(9, 2, 1, true) B_CASE(9, 3, 1, true)
    B_CASE(19, 1, 0, true) B_CASE(19, 2, 0, true) B_CASE(19, 3, 0, true)
    B_CASE(19, 1, 1, true) B_CASE(19, 2, 1, true) B_CASE(19, 3, 1, true)
#undef B_CASE
    return nullptr;
}

thread_local std::string g_batch_error;
int bfail(int code, const std::string &m) {
    g_batch_error = m;
    return code;
}

}  // namespace
}  // namespace lbm

using namespace lbm;

struct lbm_batch_s {
    int ndom = 0, q = 9, dims = 2, coll = 1, storage = 0;
    std::vector<int> n, m, h;
    std::vector<long long> node_off, pop_off, slot_off, fluid;
    long long total_nodes = 0, total_pop = 0, total_fluid = 0;
    std::vector<lbm_params> P;
    void *fbuf[2] = {nullptr, nullptr};
    uint32_t *word = nullptr;
    int32_t *slot = nullptr;
    unsigned long long *mask = nullptr;
    int32_t *kind = nullptr;
    double *uvw = nullptr;
    float *macro = nullptr;  // rho, ux, uy, uz: 4 x total_nodes
    float *pu = nullptr;     // previous velocity for residuals, 3 x total_nodes
    StepParams *tab = nullptr;  // [parity 0,1][write_macro 0,1][domain]
    int4 *tiles = nullptr;
    int *ntiles_d = nullptr;
    double2 *partial = nullptr;
    int2 *ranges_d = nullptr;
    double *res_d = nullptr;
    std::vector<int4> all_tiles;       // every tile of every domain, domain-major
    std::vector<int> dom_tile_begin;   // into all_tiles
    std::vector<char> active;
    int ntiles = 0;
    int cur = 0;                       // buffer holding the current state
    long long steps_done = 0;
    std::vector<long long> dom_steps;
    std::vector<int> dom_buf;          // buffer holding each domain's state
    std::vector<std::vector<long long>> slot_node;  // per domain: node of each boundary slot
    std::vector<double> residual;
    int grid = 0;
    BatchKernel kern = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t stepped = nullptr;  // after the last lbm_batch_step, on its stream
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0, graph_parity = -1;
    size_t elem = 4;
};

static void batch_free(lbm_batch_s *B) {
    if (!B) return;
    if (B->graph) cudaGraphExecDestroy(B->graph);
    void *ptrs[] = {B->fbuf[0], B->fbuf[1], B->word, B->slot, B->mask, B->kind, B->uvw, B->macro,
                    B->pu, B->tab, B->tiles, B->ntiles_d, B->partial, B->ranges_d, B->res_d};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (B->stepped) cudaEventDestroy(B->stepped);
    if (B->stream) cudaStreamDestroy(B->stream);
    delete B;
}

static StepParams batch_params(const lbm_batch_s *B, int d, int parity, int write_macro) {
    StepParams p;
    memset(&p, 0, sizeof(p));
    const int n = B->n[d], q = B->q;
    const size_t e = B->elem;
    for (int k = 0; k < q; ++k) {
        p.fin[k] = (const char *)B->fbuf[parity] + ((size_t)B->pop_off[d] + (size_t)k * n) * e;
        p.fout[k] = (char *)B->fbuf[1 - parity] + ((size_t)B->pop_off[d] + (size_t)k * n) * e;
    }
    const long long no = B->node_off[d], so = B->slot_off[d], T = B->total_nodes;
    p.word = B->word + no;
    p.slot = B->slot + no;
    p.bc_mask = B->mask + so;
    p.bc_kind = B->kind + so;
    p.bc_uvw = B->uvw + 3 * so;
    p.rho = B->macro + no;
    p.ux = B->macro + T + no;
    p.uy = B->macro + 2 * T + no;
    p.uz = B->macro + 3 * T + no;
    p.nx = n;
    p.ny = B->m[d];
    p.nz = B->h[d];
    p.pitch = q * n;
    p.write_macro = write_macro;
    const lbm_params &P = B->P[d];
    p.omega = 1.0 / (3.0 * P.viscosity + 0.5);
    p.omega_m = 8.0 * (2.0 - p.omega) / (8.0 - p.omega);
    p.gshift = B->dims == 3 ? P.g / p.omega : 0.0;
    p.rho_in = P.rho_in;
    p.rho_out = P.rho_out;
    p.rho0 = P.rho;
    p.scale = P.f16_scale > 0 ? (float)P.f16_scale : 1024.f;
    p.inv_scale = 1.0f / p.scale;
    // batches run in physics mode: F32 and F16S hold deviations from the rest state
    for (int k = 0; k < q; ++k) p.shift[k] = (float)rest_shift(q, B->coll, k);
    p.sigma = 1.f;
    p.outlet_profile = P.outlet_profile;
    p.update_inlet_outlet = P.update_inlet_outlet;
    p.init_rho = P.rho;
    p.init_ux = P.u;
    p.init_uy = P.v;
    p.init_uz = B->dims == 3 ? P.w : 0.0;
    return p;
}

// Upload the tiles of the active domains and their ranges.
static int batch_upload_tiles(lbm_batch_s *B) {
    std::vector<int4> t;
    std::vector<int2> ranges(B->ndom, make_int2(0, 0));
    for (int d = 0; d < B->ndom; ++d) {
        const int b = B->dom_tile_begin[d], e = B->dom_tile_begin[d + 1];
        ranges[d] = make_int2((int)t.size(), (int)t.size());
        if (!B->active[d]) continue;
        t.insert(t.end(), B->all_tiles.begin() + b, B->all_tiles.begin() + e);
        ranges[d].y = (int)t.size();
    }
    B->ntiles = (int)t.size();
    cudaError_t err = cudaSuccess;
    if (!t.empty())
        err = cudaMemcpyAsync(B->tiles, t.data(), sizeof(int4) * t.size(), cudaMemcpyHostToDevice, B->stream);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(B->ntiles_d, &B->ntiles, sizeof(int), cudaMemcpyHostToDevice, B->stream);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(B->ranges_d, ranges.data(), sizeof(int2) * B->ndom, cudaMemcpyHostToDevice, B->stream);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(B->stream, B->stepped, 0);
    if (err == cudaSuccess) err = cudaStreamSynchronize(B->stream);  // host vectors go out of scope
    return err == cudaSuccess ? LBM_OK : bfail(LBM_ERR_CUDA, std::string("tile upload: ") + cudaGetErrorString(err));
}

static cudaError_t batch_launch(lbm_batch_s *B, int parity, int write_macro, cudaStream_t s) {
    const StepParams *tab = B->tab + (size_t)(parity * 2 + write_macro) * B->ndom;
    void *args[] = {(void *)&tab, (void *)&B->tiles, (void *)&B->ntiles_d};
    return cudaLaunchKernel((const void *)B->kern, dim3((unsigned)B->grid), dim3(STEP_BLOCK), args, 0, s);
}

extern "C" {

const char *lbm_batch_last_error(void) { return g_batch_error.c_str(); }

int lbm_batch_create(const lbm_lattice_desc *const *lattices, const lbm_params *params, int count,
                     lbm_batch *out) {
    if (!lattices || !params || !out || count < 1) return bfail(LBM_ERR_INVALID, "null argument or empty batch");
    *out = nullptr;
    lbm_batch_s *B = new (std::nothrow) lbm_batch_s();
    if (!B) return bfail(LBM_ERR_NOMEM, "out of host memory");
    B->ndom = count;
    B->dims = lattices[0]->dims;
    B->q = B->dims == 2 ? 9 : 19;
    B->coll = params[0].collision_model;
    B->storage = params[0].storage;
    B->elem = B->storage == LBM_STORE_F32 ? 4 : (B->storage == LBM_STORE_F16S ? 2 : 8);
    B->kern = batch_kernel(B->q, B->coll, B->storage, params[0].mode == LBM_MODE_PHYSICS);
    if (!B->kern) {
        batch_free(B);
        return bfail(LBM_ERR_UNSUPPORTED, "batches run in physics mode with F32 or F16S storage");
    }
    std::vector<DeviceFlags> flags(count);
    for (int d = 0; d < count; ++d) {
        const lbm_lattice_desc &L = *lattices[d];
        const lbm_params &P = params[d];
        if (L.dims != B->dims || P.collision_model != B->coll || P.storage != B->storage ||
            P.mode != LBM_MODE_PHYSICS) {
            batch_free(B);
            return bfail(LBM_ERR_INVALID, "domains of a batch share dims, collision model, storage and mode");
        }
        if (!(P.viscosity > 0)) {
            batch_free(B);
            return bfail(LBM_ERR_INVALID, "viscosity must be positive");
        }
        RefMasks refm;
        std::string err;
        int rc = build_ref_masks(L, refm, err);
        if (!rc) rc = build_device_flags(L, P, refm, flags[d], err);
        if (!rc && std::any_of(flags[d].kind.begin(), flags[d].kind.end(), [](int k) { return (k & BCK_HE) != 0; })) {
            rc = LBM_ERR_UNSUPPORTED;
            err = "HEmodel outlets keep per-node state that batches do not carry";
        }
        if (rc) {
            batch_free(B);
            return bfail(rc, "domain " + std::to_string(d) + ": " + err);
        }
        const int h = L.dims == 2 ? 1 : L.h;
        B->n.push_back(L.n);
        B->m.push_back(L.m);
        B->h.push_back(h);
        B->P.push_back(P);
        const long long N = (long long)L.n * L.m * h;
        B->node_off.push_back(B->total_nodes);
        B->pop_off.push_back(B->total_pop);
        B->slot_off.push_back(d ? B->slot_off[d - 1] + (long long)flags[d - 1].slot_node.size() : 0);
        B->total_nodes += N;
        B->total_pop += ((long long)B->q * N + 63) / 64 * 64;
        long long fl = 0;
        for (long long i = 0; i < N; ++i) fl += L.node_type[i] & 1;
        B->fluid.push_back(fl);
        B->total_fluid += fl;
    }
    const long long nslots = B->slot_off[count - 1] + (long long)flags[count - 1].slot_node.size();
    // tiles, domain-major
    B->dom_tile_begin.push_back(0);
    for (int d = 0; d < count; ++d) {
        const int rows = B->m[d] * B->h[d];
        for (int r = 0; r < rows; ++r)
            if (r % BATCH_ROWS == 0)
                for (int x0 = 0; x0 < B->n[d]; x0 += 32)
                    B->all_tiles.push_back(make_int4(d, r, x0, (int)(B->node_off[d] + (long long)r * B->n[d] + x0)));
        B->dom_tile_begin.push_back((int)B->all_tiles.size());
    }
    if (B->total_nodes >= (1ll << 31)) {
        batch_free(B);
        return bfail(LBM_ERR_INVALID, "a batch holds fewer than 2^31 nodes");
    }
    B->active.assign(count, 1);
    B->dom_steps.assign(count, 0);
    B->dom_buf.assign(count, 0);
    B->residual.assign(count, INFINITY);
    const size_t T = (size_t)B->total_nodes, NT = B->all_tiles.size();
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes ? bytes : 16);
    };
    alloc(&B->fbuf[0], (size_t)B->total_pop * B->elem);
    alloc(&B->fbuf[1], (size_t)B->total_pop * B->elem);
    alloc((void **)&B->word, sizeof(uint32_t) * T);
    alloc((void **)&B->slot, sizeof(int32_t) * T);
    alloc((void **)&B->mask, sizeof(unsigned long long) * nslots);
    alloc((void **)&B->kind, sizeof(int32_t) * nslots);
    alloc((void **)&B->uvw, sizeof(double) * 3 * nslots);
    alloc((void **)&B->macro, sizeof(float) * 4 * T);
    alloc((void **)&B->pu, sizeof(float) * 3 * T);
    alloc((void **)&B->tab, sizeof(StepParams) * 4 * count);
    alloc((void **)&B->tiles, sizeof(int4) * NT);
    alloc((void **)&B->ntiles_d, sizeof(int));
    alloc((void **)&B->partial, sizeof(double2) * NT);
    alloc((void **)&B->ranges_d, sizeof(int2) * count);
    alloc((void **)&B->res_d, sizeof(double) * count);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B->stepped, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        batch_free(B);
        return bfail(LBM_ERR_NOMEM, std::string("allocation: ") + cudaGetErrorString(e));
    }
    // flags, slots (made batch-global), boundary data
    std::vector<uint32_t> word(T);
    std::vector<int32_t> slot(T);
    std::vector<unsigned long long> mask(nslots);
    std::vector<int32_t> kind(nslots);
    std::vector<double> uvw(3 * nslots);
    B->slot_node.resize(count);
    for (int d = 0; d < count; ++d) {
        const DeviceFlags &F = flags[d];
        B->slot_node[d] = F.slot_node;
        std::copy(F.word.begin(), F.word.end(), word.begin() + B->node_off[d]);
        std::copy(F.slot.begin(), F.slot.end(), slot.begin() + B->node_off[d]);  // slots stay domain-local
        for (size_t s = 0; s < F.slot_node.size(); ++s) {
            const size_t g = (size_t)B->slot_off[d] + s;
            mask[g] = F.mask[s];
            kind[g] = F.kind[s];
            uvw[3 * g] = B->P[d].u;
            uvw[3 * g + 1] = B->P[d].v;
            uvw[3 * g + 2] = B->P[d].w;
        }
    }
    e = cudaMemcpy(B->word, word.data(), sizeof(uint32_t) * T, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(B->slot, slot.data(), sizeof(int32_t) * T, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nslots) {
        e = cudaMemcpy(B->mask, mask.data(), sizeof(unsigned long long) * nslots, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(B->kind, kind.data(), sizeof(int32_t) * nslots, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(B->uvw, uvw.data(), sizeof(double) * 3 * nslots, cudaMemcpyHostToDevice);
    }
    std::vector<StepParams> tab(4 * (size_t)count);
    for (int par = 0; par < 2; ++par)
        for (int wm = 0; wm < 2; ++wm)
            for (int d = 0; d < count; ++d) tab[(size_t)(par * 2 + wm) * count + d] = batch_params(B, d, par, wm);
    if (e == cudaSuccess) e = cudaMemcpy(B->tab, tab.data(), sizeof(StepParams) * tab.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        batch_free(B);
        return bfail(LBM_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
    }
    int dev = 0, sms = 0, bps = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, B->kern, STEP_BLOCK, 0);
    B->grid = std::max(1, sms * std::max(bps, 1));
    int rc = batch_upload_tiles(B);
    if (rc) {
        batch_free(B);
        return rc;
    }
    *out = B;
    return LBM_OK;
}

int lbm_batch_init(lbm_batch B) {
    if (!B) return bfail(LBM_ERR_INVALID, "null batch");
    const size_t T = (size_t)B->total_nodes;
    cudaError_t e = cudaMemsetAsync(B->pu, 0, sizeof(float) * 3 * T, B->stream);
    for (int d = 0; d < B->ndom && e == cudaSuccess; ++d) {
        StepParams p = batch_params(B, d, 1, 0);        // writes buffer 0
        const StepParams o = batch_params(B, d, 0, 0);  // writes buffer 1
        p.init_from_arrays = 0;
        const int rc = B->q == 9 ? launch_init_q9(p, o, B->coll, B->storage, 1, 1, B->stream)
                                 : launch_init_q19(p, o, B->coll, B->storage, 1, 1, B->stream);
        if (rc) return bfail(LBM_ERR_UNSUPPORTED, "no init kernel for this configuration");
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
    if (e != cudaSuccess) return bfail(LBM_ERR_CUDA, std::string("init: ") + cudaGetErrorString(e));
    B->cur = 0;
    B->steps_done = 0;
    std::fill(B->dom_steps.begin(), B->dom_steps.end(), 0);
    std::fill(B->dom_buf.begin(), B->dom_buf.end(), 0);
    std::fill(B->active.begin(), B->active.end(), 1);
    std::fill(B->residual.begin(), B->residual.end(), INFINITY);
    return batch_upload_tiles(B);
}

// nsteps steps of every active domain; the last one stores rho, u when
// write_macro_last.  Long runs replay a captured graph of an even number of
// plain steps.
int lbm_batch_step(lbm_batch B, int nsteps, int write_macro_last, void *stream) {
    if (!B || nsteps < 0) return bfail(LBM_ERR_INVALID, "invalid argument");
    cudaStream_t s = stream ? (cudaStream_t)stream : B->stream;
    const int plain = write_macro_last && nsteps > 0 ? nsteps - 1 : nsteps;
    constexpr int G = 16;  // steps per graph replay (even: the buffer parity is unchanged)
    int done = 0;
    cudaError_t e = cudaSuccess;
    if (plain >= G) {
        if (!B->graph || B->graph_parity != B->cur) {
            if (B->graph) cudaGraphExecDestroy(B->graph);
            B->graph = nullptr;
            cudaGraph_t g;
            e = cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal);
            for (int k = 0; k < G && e == cudaSuccess; ++k) e = batch_launch(B, (B->cur + k) & 1, 0, B->stream);
            cudaError_t e2 = cudaStreamEndCapture(B->stream, &g);
            if (e == cudaSuccess) e = e2;
            if (e == cudaSuccess) {
                e = cudaGraphInstantiate(&B->graph, g, 0);
                cudaGraphDestroy(g);
            }
            B->graph_parity = B->cur;
        }
        for (; e == cudaSuccess && done + G <= plain; done += G) e = cudaGraphLaunch(B->graph, s);
    }
    for (; e == cudaSuccess && done < plain; ++done) {
        e = batch_launch(B, B->cur ^ (done & 1), 0, s);
    }
    int parity = B->cur ^ (plain & 1);
    if (e == cudaSuccess && nsteps > plain) {
        e = batch_launch(B, parity, 1, s);
        parity ^= 1;
    }
    if (e == cudaSuccess) e = cudaEventRecord(B->stepped, s);
    if (e != cudaSuccess) return bfail(LBM_ERR_CUDA, std::string("batch step: ") + cudaGetErrorString(e));
    B->cur = parity;
    B->steps_done += nsteps;
    for (int d = 0; d < B->ndom; ++d)
        if (B->active[d]) {
            B->dom_steps[d] += nsteps;
            B->dom_buf[d] = B->cur;
        }
    return LBM_OK;
}

// Per-domain FP64 velocity residual of the last stored fields against those
// of the previous call: sqrt(sum |u - u_prev|^2) / sqrt(sum |u|^2) over fluid
// nodes.  Retired domains keep their last value.
int lbm_batch_residuals(lbm_batch B, double *res) {
    if (!B || !res) return bfail(LBM_ERR_INVALID, "null argument");
    cudaStreamWaitEvent(B->stream, B->stepped, 0);
    batch_residual_partial<<<B->grid, STEP_BLOCK, 0, B->stream>>>(B->tab, B->tiles, B->ntiles_d, B->pu, B->partial);
    std::vector<double> r(B->residual);
    cudaError_t e = cudaMemcpyAsync(B->res_d, r.data(), sizeof(double) * B->ndom, cudaMemcpyHostToDevice, B->stream);
    batch_residual_final<<<(B->ndom + 127) / 128, 128, 0, B->stream>>>(B->partial, B->ranges_d, B->ndom, B->res_d);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(B->residual.data(), B->res_d, sizeof(double) * B->ndom, cudaMemcpyDeviceToHost, B->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
    if (e != cudaSuccess) return bfail(LBM_ERR_CUDA, std::string("batch residuals: ") + cudaGetErrorString(e));
    memcpy(res, B->residual.data(), sizeof(double) * B->ndom);
    for (int d = 0; d < B->ndom; ++d)
        if (B->active[d] && !(res[d] == res[d])) return bfail(LBM_DIVERGED, "domain " + std::to_string(d) + " diverged");
    return LBM_OK;
}

int lbm_batch_set_active(lbm_batch B, const int *active) {
    if (!B || !active) return bfail(LBM_ERR_INVALID, "null argument");
    cudaError_t e = cudaStreamWaitEvent(B->stream, B->stepped, 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
    for (int d = 0; d < B->ndom && e == cudaSuccess; ++d) {
        const bool on = active[d] != 0;
        // a domain that rejoins with its state in the other buffer is copied
        // to the buffer the next step reads
        if (on && !B->active[d] && B->dom_buf[d] != B->cur) {
            const size_t bytes = (size_t)B->q * B->n[d] * B->m[d] * B->h[d] * B->elem;
            const size_t off = (size_t)B->pop_off[d] * B->elem;
            e = cudaMemcpyAsync((char *)B->fbuf[B->cur] + off, (const char *)B->fbuf[B->cur ^ 1] + off, bytes,
                                cudaMemcpyDeviceToDevice, B->stream);
            B->dom_buf[d] = B->cur;
        }
        B->active[d] = on;
    }
    if (e != cudaSuccess) return bfail(LBM_ERR_CUDA, std::string("set_active: ") + cudaGetErrorString(e));
    return batch_upload_tiles(B);
}

int lbm_batch_run_to_tolerance(lbm_batch B, double tol, int check_every, long long max_steps, long long *steps,
                               double *res) {
    if (!B || check_every < 2 || !(tol > 0)) return bfail(LBM_ERR_INVALID, "invalid argument");
    std::vector<double> r(B->ndom);
    int rc = LBM_OK;
    bool first = true;
    while (B->ntiles > 0 && B->steps_done < max_steps) {
        if ((rc = lbm_batch_step(B, check_every, 1, nullptr))) break;
        rc = lbm_batch_residuals(B, r.data());
        if (rc == LBM_DIVERGED) break;
        if (rc) break;
        bool changed = false;
        if (!first)  // the first residual is against the zero field
            for (int d = 0; d < B->ndom; ++d)
                if (B->active[d] && r[d] < tol) {
                    B->active[d] = 0;
                    changed = true;
                }
        first = false;
        if (changed && (rc = batch_upload_tiles(B))) break;
    }
    if (steps) memcpy(steps, B->dom_steps.data(), sizeof(long long) * B->ndom);
    if (res) memcpy(res, B->residual.data(), sizeof(double) * B->ndom);
    return rc;
}

int lbm_batch_set_inlet_velocity(lbm_batch B, int d, const float *u, const float *v, const float *w) {
    if (!B || d < 0 || d >= B->ndom) return bfail(LBM_ERR_INVALID, "invalid domain");
    const std::vector<long long> &sn = B->slot_node[d];
    if (sn.empty()) return LBM_OK;
    std::vector<double> uvw(3 * sn.size());
    const lbm_params &P = B->P[d];
    for (size_t k = 0; k < sn.size(); ++k) {
        uvw[3 * k] = u ? u[sn[k]] : P.u;
        uvw[3 * k + 1] = v ? v[sn[k]] : P.v;
        uvw[3 * k + 2] = w ? w[sn[k]] : P.w;
    }
    cudaError_t e = cudaStreamSynchronize(B->stream);
    if (e == cudaSuccess)
        e = cudaMemcpy(B->uvw + 3 * B->slot_off[d], uvw.data(), sizeof(double) * uvw.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return bfail(LBM_ERR_CUDA, std::string("set_inlet_velocity: ") + cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_batch_init_fields(lbm_batch B, int d, const float *rho, const float *u, const float *v, const float *w) {
    if (!B || d < 0 || d >= B->ndom) return bfail(LBM_ERR_INVALID, "invalid domain");
    if (B->steps_done != 0 || B->cur != 0)
        return bfail(LBM_ERR_INVALID, "lbm_batch_init_fields must follow lbm_batch_init, before any step");
    const long long T = B->total_nodes, no = B->node_off[d];
    const size_t nn = (size_t)B->n[d] * B->m[d] * B->h[d];
    const float *src[4] = {rho, u, v, w};
    int mask = 0;
    cudaError_t e = cudaStreamSynchronize(B->stream);
    for (int k = 0; k < 4 && e == cudaSuccess; ++k)
        if (src[k]) {
            e = cudaMemcpy(B->macro + k * T + no, src[k], sizeof(float) * nn, cudaMemcpyHostToDevice);
            mask |= 1 << k;
        }
    if (e != cudaSuccess) return bfail(LBM_ERR_CUDA, std::string("init_fields: ") + cudaGetErrorString(e));
    StepParams p = batch_params(B, d, 1, 0);        // writes buffer 0
    const StepParams o = batch_params(B, d, 0, 0);  // writes buffer 1
    p.init_from_arrays = mask;
    const int rc = B->q == 9 ? launch_init_q9(p, o, B->coll, B->storage, 1, 1, B->stream)
                             : launch_init_q19(p, o, B->coll, B->storage, 1, 1, B->stream);
    if (rc) return bfail(LBM_ERR_UNSUPPORTED, "no init kernel for this configuration");
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
    if (e != cudaSuccess) return bfail(LBM_ERR_CUDA, std::string("init_fields: ") + cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_batch_get_macro(lbm_batch B, int d, float *rho, float *u, float *v, float *w) {
    if (!B || d < 0 || d >= B->ndom) return bfail(LBM_ERR_INVALID, "invalid domain");
    cudaError_t e = cudaStreamWaitEvent(B->stream, B->stepped, 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
    const size_t N = (size_t)B->n[d] * B->m[d] * B->h[d], T = (size_t)B->total_nodes, o = (size_t)B->node_off[d];
    float *dst[4] = {rho, u, v, w};
    for (int k = 0; k < 4 && e == cudaSuccess; ++k)
        if (dst[k]) e = cudaMemcpy(dst[k], B->macro + k * T + o, sizeof(float) * N, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? LBM_OK : bfail(LBM_ERR_CUDA, std::string("read-back: ") + cudaGetErrorString(e));
}

int lbm_batch_get_populations(lbm_batch B, int d, double *f) {
    if (!B || d < 0 || d >= B->ndom || !f) return bfail(LBM_ERR_INVALID, "invalid argument");
    const long long N = (long long)B->n[d] * B->m[d] * B->h[d];
    double *tmp = nullptr;
    cudaError_t e = cudaStreamWaitEvent(B->stream, B->stepped, 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
    if (e == cudaSuccess) e = cudaMalloc((void **)&tmp, sizeof(double) * B->q * N);
    if (e == cudaSuccess) {
        // a retired domain's state is in the buffer its last step wrote
        const int parity = B->dom_buf[d];
        const StepParams p = batch_params(B, d, parity, 0);
        if (B->q == 9) launch_decode_q9(p, B->storage, tmp, N, B->stream);
        else launch_decode_q19(p, B->storage, tmp, N, B->stream);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
        if (e == cudaSuccess) e = cudaMemcpy(f, tmp, sizeof(double) * B->q * N, cudaMemcpyDeviceToHost);
        cudaFree(tmp);
    }
    return e == cudaSuccess ? LBM_OK : bfail(LBM_ERR_CUDA, std::string("read-back: ") + cudaGetErrorString(e));
}

int lbm_batch_info(lbm_batch B, int *domains, long long *nodes, long long *fluid_nodes, int *active_tiles) {
    if (!B) return bfail(LBM_ERR_INVALID, "null batch");
    if (domains) *domains = B->ndom;
    if (nodes) *nodes = B->total_nodes;
    if (fluid_nodes) *fluid_nodes = B->total_fluid;
    if (active_tiles) *active_tiles = B->ntiles;
    return LBM_OK;
}

long long lbm_batch_active_fluid_nodes(lbm_batch B) {
    if (!B) return -1;
    long long s = 0;
    for (int d = 0; d < B->ndom; ++d)
        if (B->active[d]) s += B->fluid[d];
    return s;
}

void lbm_batch_destroy(lbm_batch B) {
    if (B && B->stream) {
        cudaStreamWaitEvent(B->stream, B->stepped, 0);
        cudaStreamSynchronize(B->stream);
    }
    batch_free(B);
}

}  // extern "C"
