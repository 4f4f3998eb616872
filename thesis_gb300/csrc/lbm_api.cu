// C ABI of the lattice-Boltzmann engine (include/thesis_lbm.h): handle
// lifetime, device allocation, initial collision, the step loop (with a
// captured two-step CUDA graph for short steps) and read-back.
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <string>
#include <vector>

#include "lbm_flags.h"
#include "lbm_jit.h"
#include "lbm_step_tma.cuh"

namespace lbm {
int launch_step_q9(const StepParams &p, int coll, int st, int phys, cudaStream_t s);
int launch_step_q19(const StepParams &p, int coll, int st, int phys, cudaStream_t s);
int launch_step_x2_q9(const StepParams &p, int coll, int st, int phys, cudaStream_t s);
int launch_step_x2_q19(const StepParams &p, int coll, int st, int phys, cudaStream_t s);
int launch_init_q9(const StepParams &p, const StepParams &o, int coll, int st, int phys, int eq, cudaStream_t s);
int launch_init_q19(const StepParams &p, const StepParams &o, int coll, int st, int phys, int eq, cudaStream_t s);
int launch_decode_q9(const StepParams &p, int st, double *out, long long n, cudaStream_t s);
int launch_decode_q19(const StepParams &p, int st, double *out, long long n, cudaStream_t s);
int launch_encode_q9(const StepParams &p, int st, const double *in, long long n, cudaStream_t s);
int launch_encode_q19(const StepParams &p, int st, const double *in, long long n, cudaStream_t s);
int launch_norms(const uint32_t *word, const float *rho, const float *ux, const float *uy,
                 const float *uz, float *pux, float *puy, float *puz, long long n,
                 double *partial, double *out, cudaStream_t s);
int norm_partial_count();
int launch_resid_l2_q9(const StepParams &p, int st, int phys, double *partial, double *out, cudaStream_t s);
int launch_resid_l2_q19(const StepParams &p, int st, int phys, double *partial, double *out, cudaStream_t s);
long long resid_l2_partials_q9(const StepParams &p);
int launch_momentum_exchange_q9(const StepParams &p, int st, const int *box, double *partial, double *out,
                                cudaStream_t s);
int launch_momentum_exchange_q19(const StepParams &p, int st, const int *box, double *partial, double *out,
                                 cudaStream_t s);
long long resid_l2_partials_q19(const StepParams &p);
int launch_fd_rel_q9(const StepParams &p, int st, int phys, float *fprev, float *ffirst, int first,
                     double *partial, double *out, cudaStream_t s);
int launch_fd_rel_q19(const StepParams &p, int st, int phys, float *fprev, float *ffirst, int first,
                      double *partial, double *out, cudaStream_t s);
int launch_macro_diff(const float *ux, const float *uy, const float *uz, const float *rho, float *pux, float *puy,
                      float *puz, float *prho, long long n, double *partial, double *out, cudaStream_t s);
int tma_prepare(int q, int coll, int st, size_t smem, int *blocks_per_sm);
int launch_step_tma(int q, const StepParams &p, const TmaRows &rows, int coll, int st, int grid, size_t smem,
                    cudaStream_t s);
unsigned tma_stage_size(int q, int nx, int elem);
}  // namespace lbm

using namespace lbm;

static thread_local std::string g_last_error;

static int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

#define CUDA_TRY(call)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return fail(LBM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct lbm_handle_s {
    int dims = 2, q = 9, n = 0, m = 0, h = 1;
    long long N = 0, stride = 0, fluid = 0;
    lbm_params P{};
    size_t elem = 4;
    void *fbuf[2] = {nullptr, nullptr};
    uint32_t *word = nullptr;
    int32_t *slot = nullptr;
    unsigned long long *mask = nullptr;
    int32_t *kind = nullptr;
    double *uvw = nullptr;
    float *rho = nullptr, *ux = nullptr, *uy = nullptr, *uz = nullptr;
    float *pux = nullptr, *puy = nullptr, *puz = nullptr;
    float *mdiff_prev = nullptr;  // u, v, w, rho at the last lbm_macro_diff (4 N floats)
    float *fd_snap = nullptr;     // FdRelDiff: f_prev, f_first (2 Q N floats, allocated on first use)
    bool fd_recorded = false;
    int zwalk_request = 0;        // THESIS_LBM_KERNEL=jithz<k>[b<block>][m<min blocks>][p]
    int hb_request = 0;           // ... p: predicated bounce-back loads
    int zp_request = 0;           // ... q: two z nodes at a time on packed FP32x2
    int block_request = 0, minb_request = 0;
    double *partial = nullptr, *norms = nullptr;
    int nslots = 0;
    std::vector<long long> slot_node;
    // reference curved walls: per slot Q link fractions on the device (null
    // for straight walls), the boundary nodes in ascending order (the
    // reference's collapsed order) and, per BC link, its node's place there
    double *bcq = nullptr;
    double *bc_macro = nullptr;  // HEmodel outlets: per slot rho, u, v, w of the previous step
    // reference-mode 2D: boundary nodes whose mask carries a boundary id
    // (bits 24-31), for the reference's drag/lift sums
    std::vector<long long> id_nodes;
    std::vector<unsigned char> id_bits;
    std::vector<long long> bc_nodes;
    std::vector<int> link_b;
    std::vector<unsigned char> link_dir;
    int cur = 0;
    cudaStream_t stream = nullptr;
    // recorded after the steps of every lbm_step, on the stream they ran on;
    // the handle's own stream waits for it before reductions and read-back
    cudaEvent_t stepped = nullptr;
    cudaGraphExec_t pair[2] = {nullptr, nullptr};
    int status = LBM_OK;
    bool initialised = false;
    bool pair_kernel = false;  // two nodes per thread (even nx, F32/F16S)
    bool tma_kernel = false;   // row-staged bulk-copy kernel
    bool jit_kernel = false;   // step kernel specialised for this lattice at run time
    std::string kernel_warning; // why the run-time build fell back to the compiled-in kernel
    cudaKernel_t jit_fn = nullptr;
    JitStepKey jit_key{};
    int32_t *tma_row = nullptr;
    uint32_t *tma_lmask = nullptr, *tma_omask = nullptr;
    unsigned int *tma_err = nullptr;
    int tma_nrows = 0, tma_stages = 0, tma_grid = 0;
    size_t tma_smem = 0;
    double omega = 1, omega_m = 1, gshift = 0;
    float scale = 1024.f;
};

static StepParams make_params(const lbm_handle_s *H, int from, int write_macro) {
    StepParams p;
    memset(&p, 0, sizeof(p));
    for (int d = 0; d < H->q; ++d) {
        // row layout: direction d of row r starts at (r * q + d) * n
        p.fin[d] = (const char *)H->fbuf[from] + (size_t)d * H->n * H->elem;
        p.fout[d] = (char *)H->fbuf[1 - from] + (size_t)d * H->n * H->elem;
    }
    p.word = H->word;
    p.slot = H->slot;
    p.bc_mask = H->mask;
    p.bc_kind = H->kind;
    p.bc_uvw = H->uvw;
    p.bc_q = H->bcq;
    p.bc_macro = H->bc_macro;
    p.rho = H->rho;
    p.ux = H->ux;
    p.uy = H->uy;
    p.uz = H->uz;
    p.nx = H->n;
    p.ny = H->m;
    p.nz = H->h;
    p.pitch = H->q * H->n;
    p.write_macro = write_macro;
    p.omega = H->omega;
    p.omega_m = H->omega_m;
    p.gshift = H->gshift;
    p.rho_in = H->P.rho_in;
    p.rho_out = H->P.rho_out;
    p.rho0 = H->P.rho;
    p.ref_hh = H->P.mode != LBM_MODE_PHYSICS && H->q == 19 && H->P.bc_wall_model == LBM_WALL_COMPLEX;
    p.scale = H->scale;
    p.inv_scale = 1.0f / H->scale;
    // populations stored as deviations from the rest state: F16S always, F32
    // in physics mode (moments then come from small numbers, without the
    // cancellation that limits an FP32 steady state to a ~1e-6 residual)
    const bool shifted = H->P.storage == LBM_STORE_F16S || H->P.storage == LBM_STORE_F16C ||
                         (H->P.storage == LBM_STORE_F32 && H->P.mode == LBM_MODE_PHYSICS);
    for (int d = 0; d < H->q; ++d) p.shift[d] = shifted ? (float)rest_shift(H->q, H->P.collision_model, d) : 0.0f;
    p.sigma = shifted ? 1.f : 0.f;
    p.outlet_profile = H->P.outlet_profile;
    p.update_inlet_outlet = H->P.update_inlet_outlet;
    return p;
}

static void free_handle(lbm_handle_s *H) {
    if (!H) return;
    for (int c = 0; c < 2; ++c)
        if (H->pair[c]) cudaGraphExecDestroy(H->pair[c]);
    void *ptrs[] = {H->fbuf[0], H->fbuf[1], H->word, H->slot, H->mask, H->kind, H->uvw,
                    H->rho, H->ux, H->uy, H->uz, H->pux, H->puy, H->puz, H->partial, H->norms,
                    H->tma_row, H->tma_lmask, H->tma_omask, H->tma_err, H->mdiff_prev, H->fd_snap,
                    H->bcq, H->bc_macro};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (H->stepped) cudaEventDestroy(H->stepped);
    if (H->stream) cudaStreamDestroy(H->stream);
    delete H;
}

// Per row (y + ny z) holding fluid nodes: the directions whose pull row the
// row-staged kernel must copy (those some fluid node of the row pulls across
// an open link) and the arrays whose own row it must copy (opp(d) for every
// d that some fluid node of the row cannot pull).
template <int Q>
static void tma_row_tables(const HostArray<uint32_t> &word, int nx, long long nrows_all,
                           std::vector<int32_t> &rows, std::vector<uint32_t> &lm, std::vector<uint32_t> &om) {
    using L = Lat<Q>;
    const uint32_t dirs = (1u << Q) - 1u;
    for (long long r = 0; r < nrows_all; ++r) {
        const uint32_t *w = word.data() + (size_t)r * nx;
        uint32_t any_blocked = 0, all_blocked = dirs;
        bool fluid = false;
        for (int x = 0; x < nx; ++x) {
            if (!(w[x] & W_FLUID)) continue;
            fluid = true;
            const uint32_t b = w[x] & dirs & ~1u;
            any_blocked |= b;
            all_blocked &= b;
        }
        if (!fluid) continue;
        uint32_t o = 0;
        for (int d = 1; d < Q; ++d)
            if ((any_blocked >> d) & 1u) o |= 1u << L::opp(d);
        rows.push_back((int32_t)r);
        lm.push_back(dirs & ~all_blocked);
        om.push_back(o);
    }
}

// Decide whether the row-staged kernel can run this lattice and set it up:
// physics mode, F32/F16S storage, rows a multiple of 16 bytes and at least
// two stages in shared memory.  Returns LBM_OK with H->tma_kernel false when
// it cannot.
static int setup_tma(lbm_handle_s *H, const HostArray<uint32_t> &word) {
    H->tma_kernel = false;
    if (H->P.mode != LBM_MODE_PHYSICS) return LBM_OK;
    if (H->P.storage != LBM_STORE_F32 && H->P.storage != LBM_STORE_F16S) return LBM_OK;
    if (((size_t)H->n * H->elem) % 16 != 0) return LBM_OK;
    int dev = 0, sms = 0, smem_sm = 0, smem_blk = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    CUDA_TRY(cudaDeviceGetAttribute(&smem_blk, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const long long stage = tma_stage_size(H->q, H->n, (int)H->elem);
    int stages = 0;
    for (int blocks = 2; blocks >= 1; --blocks) {
        const long long per_block = std::min<long long>(smem_blk, smem_sm / blocks - 1024);
        stages = (int)std::min<long long>(8, (per_block - TMA_BARRIER_BYTES) / stage);
        if (stages >= (blocks == 2 ? 3 : 2)) break;
    }
    if (stages < 2) return LBM_OK;
    std::vector<int32_t> rows;
    std::vector<uint32_t> lm, om;
    const long long nrows_all = (long long)H->m * H->h;
    if (H->q == 9) tma_row_tables<9>(word, H->n, nrows_all, rows, lm, om);
    else tma_row_tables<19>(word, H->n, nrows_all, rows, lm, om);
    if (rows.empty()) return LBM_OK;
    const size_t smem = TMA_BARRIER_BYTES + (size_t)stages * stage;
    int bps = 0;
    const int e = tma_prepare(H->q, H->P.collision_model, H->P.storage, smem, &bps);
    if (e != 0 || bps < 1) return LBM_OK;
    const size_t nr = rows.size();
    CUDA_TRY(cudaMalloc((void **)&H->tma_row, sizeof(int32_t) * nr));
    CUDA_TRY(cudaMalloc((void **)&H->tma_lmask, sizeof(uint32_t) * nr));
    CUDA_TRY(cudaMalloc((void **)&H->tma_omask, sizeof(uint32_t) * nr));
    CUDA_TRY(cudaMalloc((void **)&H->tma_err, sizeof(unsigned int)));
    CUDA_TRY(cudaMemcpy(H->tma_row, rows.data(), sizeof(int32_t) * nr, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(H->tma_lmask, lm.data(), sizeof(uint32_t) * nr, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(H->tma_omask, om.data(), sizeof(uint32_t) * nr, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(H->tma_err, 0, sizeof(unsigned int)));
    H->tma_nrows = (int)nr;
    H->tma_stages = stages;
    H->tma_smem = smem;
    H->tma_grid = (int)std::min<long long>((long long)nr, (long long)sms * bps);
    H->tma_kernel = true;
    return LBM_OK;
}

// True when some fluid node pulls across an out-of-domain link that is not
// blocked: the step must then wrap coordinates at the faces.
template <int Q>
static bool open_outside_links(const HostArray<uint32_t> &word, int n, int m, int h) {
    using L = Lat<Q>;
    for (int z = 0; z < h; ++z)
        for (int y = 0; y < m; ++y) {
            const bool face_row = y == 0 || y == m - 1 || z == 0 || z == h - 1;
            for (int x = 0; x < n; x = (face_row || x == n - 1) ? x + 1 : n - 1) {
                const uint32_t w = word[(size_t)x + (size_t)n * (y + (size_t)m * z)];
                if (!(w & W_FLUID)) continue;
                for (int d = 1; d < Q; ++d) {
                    const int sx = x - L::cx(d), sy = y - L::cy(d), sz = z - L::cz(d);
                    const bool outside = sx < 0 || sx >= n || sy < 0 || sy >= m || sz < 0 || sz >= h;
                    if (outside && !((w >> d) & 1u)) return true;
                }
            }
        }
    return false;
}

// Knobs of the specialised kernel chosen by lbm_autotune, remembered per
// lattice configuration for the rest of the process.
struct TunedKnobs {
    int block, hint;
    bool pred, pair;
    int minb;
    bool hspace;
    bool zpair;
    int zwalk;
};
static std::mutex g_tuned_mutex;
static std::map<std::string, TunedKnobs> g_tuned;

static std::string tune_key(const JitStepKey &k) {
    char b[160];
    snprintf(b, sizeof(b), "%d/%d/%d/%d/%d/%d/%d/%d", k.q, k.coll, k.storage, (int)k.phys, (int)k.wrap, k.nx,
             k.ny, k.nz);
    return b;
}

// Build the run-time specialised step kernel for this lattice.
static int setup_jit(lbm_handle_s *H, const HostArray<uint32_t> &word, bool pair, int hspace) {
    const bool periodic = H->P.mode == LBM_MODE_PHYSICS &&
                          (H->P.periodic[0] || H->P.periodic[1] || (H->dims == 3 && H->P.periodic[2]));
    const bool wrap = periodic || (H->q == 9 ? open_outside_links<9>(word, H->n, H->m, H->h)
                                             : open_outside_links<19>(word, H->n, H->m, H->h));
    JitStepKey k{H->q, H->P.collision_model, H->P.storage, H->P.mode == LBM_MODE_PHYSICS, wrap,
                 H->n, H->m, H->h, pair ? 64 : STEP_BLOCK, 0, false, false, pair};
    // storage-unit arithmetic by default in physics mode (accuracy of the
    // moments); reference mode keeps the f-space form of the reference
    k.hspace = !pair && (hspace > 0 || (hspace < 0 && H->P.mode == LBM_MODE_PHYSICS &&
                                        H->P.storage != LBM_STORE_F64));
    k.pred = k.hspace && hspace == 2;
    k.zwalk = k.hspace && H->zwalk_request > 1 ? H->zwalk_request : 1;
    if (k.hspace && H->block_request >= 32 && H->block_request <= 1024 && H->block_request % 32 == 0)
        k.block = H->block_request;
    if (k.hspace && H->minb_request > 1) k.minb = H->minb_request;
    if (k.hspace && H->hb_request) k.hint = 1;
    if (k.hspace && H->zp_request && k.zwalk > 1 && k.zwalk % 2 == 0) k.zpair = true;
    {
        std::lock_guard<std::mutex> lock(g_tuned_mutex);
        auto it = g_tuned.find(tune_key(k));
        // a two-node choice tuned on another lattice of this shape does not
        // carry over to boundaries only the one-node kernels apply
        if (it != g_tuned.end() && !pair && !(it->second.pair && one_node_boundaries(H->P, H->q))) {
            k.block = it->second.block;
            k.hint = it->second.hint;
            k.pred = it->second.pred;
            k.pair = it->second.pair;
            k.minb = it->second.minb;
            k.hspace = it->second.hspace;
            k.zwalk = it->second.zwalk;
            k.zpair = it->second.zpair;
        }
    }
    std::string err;
    if (jit_step_kernel(k, &H->jit_fn, err)) return fail(LBM_ERR_CUDA, "run-time kernel build: " + err);
    H->jit_key = k;
    H->jit_kernel = true;
    return LBM_OK;
}

// A bounded wait inside the row-staged kernel that gave up leaves a code in
// tma_err; report it once the stream is idle.
static int check_tma(lbm_handle_s *H) {
    if (!H->tma_kernel) return LBM_OK;
    unsigned int err = 0;
    CUDA_TRY(cudaMemcpy(&err, H->tma_err, sizeof(err), cudaMemcpyDeviceToHost));
    if (err) {
        H->status = LBM_ERR_CUDA;
        return fail(LBM_ERR_CUDA, "row-staged step: a shared-memory pipeline wait timed out (code " +
                                      std::to_string(err) + ")");
    }
    return LBM_OK;
}

extern "C" {

int lbm_version(void) { return 1; }

const char *lbm_last_error(void) { return g_last_error.c_str(); }

int lbm_create(const lbm_lattice_desc *L, const lbm_params *P, lbm_handle *out) {
    if (!L || !P || !out) return fail(LBM_ERR_INVALID, "null argument");
    *out = nullptr;
    if (L->dims != 2 && L->dims != 3) return fail(LBM_ERR_INVALID, "dims must be 2 or 3");
    const int h = L->dims == 2 ? 1 : L->h;
    if (L->n < 1 || L->m < 1 || h < 1 || !L->node_type)
        return fail(LBM_ERR_INVALID, "empty lattice");
    if (L->dims == 2 && (L->m > 65535)) return fail(LBM_ERR_INVALID, "m exceeds 65535");
    if (L->dims == 3 && (L->m > 65535 || h > 65535)) return fail(LBM_ERR_INVALID, "m or h exceeds 65535");
    const long long N = (long long)L->n * L->m * h;
    const int q = L->dims == 2 ? 9 : 19;
    // population offsets inside one z-plane (q * n * m elements) are 32-bit
    if ((long long)q * L->n * L->m >= (1ll << 31)) return fail(LBM_ERR_INVALID, "lattice plane too large");
    if (N >= (1ll << 31)) return fail(LBM_ERR_INVALID, "more than 2^31 nodes");
    if (L->num_conns > 0 && (!L->bc_i || !L->bc_j || !L->bc_dir || !L->bc_type || (L->dims == 3 && !L->bc_k)))
        return fail(LBM_ERR_INVALID, "missing BC columns");
    if (P->collision_model < LBM_BGKW || P->collision_model > LBM_MRT)
        return fail(LBM_ERR_INVALID, "unknown collision model");
    if (P->storage < LBM_STORE_F32 || P->storage > LBM_STORE_F16C)
        return fail(LBM_ERR_INVALID, "unknown storage");
    if (P->storage == LBM_STORE_F16C && P->mode != LBM_MODE_PHYSICS)
        return fail(LBM_ERR_UNSUPPORTED, "F16C storage runs in physics mode");
    if (P->mode != LBM_MODE_REFERENCE && P->mode != LBM_MODE_PHYSICS)
        return fail(LBM_ERR_INVALID, "unknown mode");
    if (!(P->viscosity > 0)) return fail(LBM_ERR_INVALID, "viscosity must be positive");
    if (P->mode == LBM_MODE_REFERENCE && L->dims == 3 && P->collision_model == LBM_TRT)
        return fail(LBM_ERR_UNSUPPORTED, "the reference has no 3D TRT (Iterate3D.cu:517-520)");

    RefMasks refm;
    DeviceFlags flags;
    std::string err;
    int rc = build_ref_masks(*L, refm, err);
    if (rc) return fail(rc, err);
    rc = build_device_flags(*L, *P, refm, flags, err);
    if (rc) return fail(rc, err);

    lbm_handle_s *H = new (std::nothrow) lbm_handle_s();
    if (!H) return fail(LBM_ERR_NOMEM, "out of host memory");
    H->dims = L->dims;
    H->q = q;
    H->n = L->n;
    H->m = L->m;
    H->h = h;
    H->N = N;
    H->stride = (N + 63) / 64 * 64;
    H->P = *P;
    H->elem = P->storage == LBM_STORE_F32 ? 4 : (P->storage == LBM_STORE_F64 ? 8 : 2);
    // F16C holds |f - shift| * scale below 2.  The D3Q19 MRT stores
    // deviations from its own rest state (4/21, 13/126, 1/63) while an
    // equilibrium start uses w (1/3, 1/18, 1/36): f0 starts 0.143 off, so its
    // default scale is 8; 256 elsewhere.
    const float f16c_scale = (L->dims == 3 && P->collision_model == LBM_MRT) ? 8.0f : 256.0f;
    H->scale = P->f16_scale > 0 ? (float)P->f16_scale : (P->storage == LBM_STORE_F16C ? f16c_scale : 1024.0f);
    // omega as the reference computes it (GpuInit.cu:102-103)
    H->omega = 1.0 / (3.0 * P->viscosity + 0.5);
    H->omega_m = 8.0 * (2.0 - H->omega) / (8.0 - H->omega);
    H->gshift = L->dims == 3 ? P->g / H->omega : 0.0;
    long long fl = 0;
    for (long long i = 0; i < N; ++i) fl += (L->node_type[i] & 1);
    H->fluid = fl;
    bool want_tma = false, want_jit = false, jit_required = false, jit_pair = false;
    int jit_hspace = -1;
    {
        // Default: the one-node kernel specialised at run time for this
        // lattice (all population offsets become immediates; fastest for
        // every storage), falling back to the compiled-in one-node kernel if
        // the run-time build is unavailable.  THESIS_LBM_KERNEL=scalar|pair|
        // tma|jit selects a variant explicitly (jit then fails loudly).
        const char *kv = getenv("THESIS_LBM_KERNEL");
        // the two-node kernels have no curved-wall or extrapolation-outlet path
        const bool can_pair = (L->n % 2 == 0) && (P->storage == LBM_STORE_F32 || P->storage == LBM_STORE_F16S) &&
                              !one_node_boundaries(*P, q);
        H->pair_kernel = kv && strcmp(kv, "pair") == 0 && can_pair;
        want_tma = kv && strcmp(kv, "tma") == 0;
        // jithz<k>[b<block>][m<min blocks>]: storage units walking k nodes along z
        int zw_env = 0, b_env = 0, m_env = 0;
        if (kv && strncmp(kv, "jithz", 5) == 0) {
            zw_env = atoi(kv + 5);
            if (const char *bp = strchr(kv, 'b')) b_env = atoi(bp + 1);
            if (const char *mp = strchr(kv + 5, 'm')) m_env = atoi(mp + 1);
            H->hb_request = strchr(kv + 5, 'p') ? 1 : 0;
            H->zp_request = strchr(kv + 5, 'q') ? 1 : 0;
        }
        H->block_request = b_env;
        H->minb_request = m_env;
        want_jit = !kv || !*kv || strcmp(kv, "jit") == 0 || strcmp(kv, "jit2") == 0 || strcmp(kv, "jith") == 0 ||
                   strcmp(kv, "jiths") == 0 || strcmp(kv, "jitf") == 0 || zw_env > 0;
        H->zwalk_request = zw_env;
        jit_required = kv && *kv && want_jit;
        jit_pair = kv && strcmp(kv, "jit2") == 0 && can_pair;
        jit_hspace = kv && (strcmp(kv, "jith") == 0 || zw_env > 0) ? 1
                     : kv && strcmp(kv, "jiths") == 0 ? 2  // storage units, speculative loads
                     : kv && strcmp(kv, "jitf") == 0  ? 0
                                                      : -1;
    }
    H->nslots = (int)flags.slot_node.size();
    H->slot_node = flags.slot_node;
    if (L->dims == 2)
        for (size_t b = 0; b < refm.bc_nodes.size(); ++b)
            if (((refm.mask[b] >> 24) & 0xFFull) && (L->node_type[refm.bc_nodes[b]] & 1)) {
                H->id_nodes.push_back(refm.bc_nodes[b]);
                H->id_bits.push_back((unsigned char)((refm.mask[b] >> 24) & 0xFFull));
            }
    if (want_tma) {
        rc = setup_tma(H, flags.word);
        if (rc) {
            free_handle(H);
            return rc;
        }
    }
    if (want_jit) {
        rc = setup_jit(H, flags.word, jit_pair, jit_hspace);
        const char *req = getenv("THESIS_LBM_REQUIRE_JIT");
        if (rc && (jit_required || (req && *req && strcmp(req, "0") != 0))) {
            free_handle(H);
            return rc;
        }
        if (rc) {
            // the default kernel could not be built (no NVRTC, or the toolkit
            // headers it compiles against are missing): keep the compiled-in
            // kernel, which is slower, and say so once per process on stderr
            // and per handle through lbm_kernel_warning
            H->kernel_warning = "run-time specialised step kernel unavailable, using the compiled-in kernel: " +
                                std::string(lbm_last_error());
            static std::once_flag warned;
            std::call_once(warned, [&] { fprintf(stderr, "thesis_lbm: %s\n", H->kernel_warning.c_str()); });
            rc = LBM_OK;
        }
    }

#define ALLOC(ptr, bytes)                                                               \
    do {                                                                                \
        cudaError_t e_ = cudaMalloc((void **)&(ptr), (bytes) > 0 ? (bytes) : 16);       \
        if (e_ != cudaSuccess) {                                                        \
            free_handle(H);                                                             \
            return fail(LBM_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e_)); \
        }                                                                               \
    } while (0)
    const size_t fbytes = (size_t)q * H->stride * H->elem;
    ALLOC(H->fbuf[0], fbytes);
    ALLOC(H->fbuf[1], fbytes);
    ALLOC(H->word, sizeof(uint32_t) * N);
    ALLOC(H->slot, sizeof(int32_t) * N);
    ALLOC(H->mask, sizeof(unsigned long long) * H->nslots);
    ALLOC(H->kind, sizeof(int32_t) * H->nslots);
    ALLOC(H->uvw, sizeof(double) * 3 * H->nslots);
    if (curved_walls(*P, q)) ALLOC(H->bcq, sizeof(double) * q * H->nslots);
    if (std::any_of(flags.kind.begin(), flags.kind.end(), [](int k) { return (k & BCK_HE) != 0; }))
        ALLOC(H->bc_macro, sizeof(double) * 4 * H->nslots);
    ALLOC(H->rho, sizeof(float) * N);
    ALLOC(H->ux, sizeof(float) * N);
    ALLOC(H->uy, sizeof(float) * N);
    ALLOC(H->uz, sizeof(float) * N);
    ALLOC(H->pux, sizeof(float) * N);
    ALLOC(H->puy, sizeof(float) * N);
    ALLOC(H->puz, sizeof(float) * N);
    ALLOC(H->partial, sizeof(double) * std::max(norm_partial_count(), 304 * 5));
    ALLOC(H->mdiff_prev, sizeof(float) * 4 * N);
    ALLOC(H->norms, sizeof(double) * LBM_NORMS);
#undef ALLOC
    cudaError_t e = cudaStreamCreateWithFlags(&H->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&H->stepped, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMemcpy(H->word, flags.word.data(), sizeof(uint32_t) * N, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(H->slot, flags.slot.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && H->nslots) {
        std::vector<unsigned long long> mk(flags.mask.begin(), flags.mask.end());
        e = cudaMemcpy(H->mask, mk.data(), sizeof(unsigned long long) * H->nslots, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(H->kind, flags.kind.data(), sizeof(int32_t) * H->nslots, cudaMemcpyHostToDevice);
        std::vector<double> uvw((size_t)3 * H->nslots);
        for (int s = 0; s < H->nslots; ++s) {
            uvw[3 * s] = P->u;
            uvw[3 * s + 1] = P->v;
            uvw[3 * s + 2] = P->w;
        }
        if (e == cudaSuccess)
            e = cudaMemcpy(H->uvw, uvw.data(), sizeof(double) * 3 * H->nslots, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && H->bcq) {
        // every link fraction starts at the reference's fill value 1/2
        // (Iterate.cu:277, Iterate3D.cu:364) until lbm_set_link_q
        H->bc_nodes = refm.bc_nodes;
        H->link_b.resize((size_t)L->num_conns);
        H->link_dir.resize((size_t)L->num_conns);
        for (int c = 0; c < L->num_conns; ++c) {
            const long long ind = L->bc_i[c] + (long long)L->n * (L->bc_j[c] + (long long)L->m * (L->dims == 3 ? L->bc_k[c] : 0));
            H->link_b[c] = (int)(std::lower_bound(H->bc_nodes.begin(), H->bc_nodes.end(), ind) - H->bc_nodes.begin());
            H->link_dir[c] = (unsigned char)L->bc_dir[c];
        }
        std::vector<double> qt((size_t)q * H->nslots, 0.5);
        if (H->nslots) e = cudaMemcpy(H->bcq, qt.data(), sizeof(double) * qt.size(), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemset(H->pux, 0, sizeof(float) * N);
    if (e == cudaSuccess) e = cudaMemset(H->puy, 0, sizeof(float) * N);
    if (e == cudaSuccess) e = cudaMemset(H->puz, 0, sizeof(float) * N);
    if (e != cudaSuccess) {
        free_handle(H);
        return fail(LBM_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
    }
    *out = H;
    return LBM_OK;
}

int lbm_set_inlet_velocity(lbm_handle H, const float *u, const float *v, const float *w) {
    if (!H) return fail(LBM_ERR_INVALID, "null handle");
    if (!H->nslots) return LBM_OK;
    std::vector<double> uvw((size_t)3 * H->nslots);
    for (int s = 0; s < H->nslots; ++s) {
        const long long node = H->slot_node[s];
        uvw[3 * s] = u ? (double)u[node] : H->P.u;
        uvw[3 * s + 1] = v ? (double)v[node] : H->P.v;
        uvw[3 * s + 2] = w ? (double)w[node] : H->P.w;
    }
    CUDA_TRY(cudaMemcpyAsync(H->uvw, uvw.data(), sizeof(double) * 3 * H->nslots, cudaMemcpyHostToDevice, H->stream));
    CUDA_TRY(cudaStreamSynchronize(H->stream));
    return LBM_OK;
}

int lbm_set_link_q(lbm_handle H, const double *q) {
    if (!H || !q) return fail(LBM_ERR_INVALID, "null argument");
    if (!H->bcq)
        return fail(LBM_ERR_UNSUPPORTED, "link fractions need reference-mode curved walls (LBM_CURVED with the "
                                         "simple wall model)");
    const int Q = H->q, D = Q - 1;
    const size_t nb = H->bc_nodes.size();
    // the reference's per-node table q[node * D + dir - 1], unset links 1/2
    // (initBoundaryConditions2D/3D, GpuInit.cu:1086-1088, :1203-1207)
    std::vector<double> tab(nb * D, 0.5);
    for (size_t c = 0; c < H->link_b.size(); ++c) {
        if (!std::isfinite(q[c])) return fail(LBM_ERR_INVALID, "link fraction " + std::to_string(c) + " is not finite");
        tab[(size_t)H->link_b[c] * D + H->link_dir[c] - 1] = q[c];
    }
    // per slot: the node's D entries, then the entry that follows them in the
    // collapsed table (collapseBc2D/3D): the next boundary node's first, and
    // past the last node (where the reference reads beyond its array) 1/2
    std::vector<double> qt((size_t)Q * H->nslots);
    for (int s = 0; s < H->nslots; ++s) {
        const size_t b = (size_t)(std::lower_bound(H->bc_nodes.begin(), H->bc_nodes.end(), H->slot_node[s]) -
                                  H->bc_nodes.begin());
        for (int j = 0; j < D; ++j) qt[(size_t)s * Q + j] = tab[b * D + j];
        qt[(size_t)s * Q + D] = b + 1 < nb ? tab[(b + 1) * D] : 0.5;
    }
    if (!H->nslots) return LBM_OK;
    CUDA_TRY(cudaStreamWaitEvent(H->stream, H->stepped, 0));
    CUDA_TRY(cudaMemcpyAsync(H->bcq, qt.data(), sizeof(double) * qt.size(), cudaMemcpyHostToDevice, H->stream));
    CUDA_TRY(cudaStreamSynchronize(H->stream));
    return LBM_OK;
}

int lbm_reference_drag_lift(lbm_handle H, int boundary_id, const float *node_x, const float *node_y, double *out) {
    if (!H || !out) return fail(LBM_ERR_INVALID, "null argument");
    out[0] = out[1] = 0.0;
    if (H->dims != 2 || boundary_id <= 0 || H->id_nodes.empty()) return LBM_OK;
    if (!node_x || !node_y) return fail(LBM_ERR_INVALID, "null coordinates");
    CUDA_TRY(cudaStreamWaitEvent(H->stream, H->stepped, 0));
    std::vector<float> rho((size_t)H->N);
    CUDA_TRY(cudaMemcpyAsync(rho.data(), H->rho, sizeof(float) * H->N, cudaMemcpyDeviceToHost, H->stream));
    CUDA_TRY(cudaStreamSynchronize(H->stream));
    // per node as gpuUpdateMacro2D stores it (FLOAT_TYPE of a double
    // product), summed in FP64
    for (size_t k = 0; k < H->id_nodes.size(); ++k) {
        if (H->id_bits[k] != (unsigned)boundary_id) continue;
        const long long i = H->id_nodes[k];
        const float r = rho[(size_t)i];
        out[0] += (double)(float)(0.33333333 * (double)r * (double)(20.0f - node_x[i]) * 0.2);
        out[1] += (double)(float)(0.33333333 * (double)r * (double)(20.0f - node_y[i]) * 0.2);
    }
    return LBM_OK;
}

int lbm_link_q(int dims, int n, int m, int h, int num_conns, const int *bc_i, const int *bc_j, const int *bc_k,
               const int *bc_dir, const float *bc_x, const float *bc_y, const float *bc_z, const float *node_x,
               const float *node_y, const float *node_z, double delta, double *q) {
    if (dims != 2 && dims != 3) return fail(LBM_ERR_INVALID, "dims must be 2 or 3");
    if (num_conns < 0 || (num_conns > 0 && (!bc_i || !bc_j || !bc_dir || !bc_x || !bc_y || !node_x || !node_y || !q)))
        return fail(LBM_ERR_INVALID, "null argument");
    if (dims == 3 && num_conns > 0 && (!bc_k || !bc_z || !node_z)) return fail(LBM_ERR_INVALID, "null argument");
    if (!(delta > 0)) return fail(LBM_ERR_INVALID, "grid spacing must be positive");
    const int Q = dims == 2 ? 9 : 19;
    const int hh = dims == 2 ? 1 : h;
    for (int c = 0; c < num_conns; ++c) {
        const int i = bc_i[c], j = bc_j[c], k = dims == 3 ? bc_k[c] : 0, d = bc_dir[c];
        if (i < 0 || i >= n || j < 0 || j >= m || k < 0 || k >= hh || d < 1 || d >= Q)
            return fail(LBM_ERR_INVALID, "BC link " + std::to_string(c) + " out of range");
        const long long ind = i + (long long)n * (j + (long long)m * k);
        const double dx = (double)bc_x[c] - node_x[ind], dy = (double)bc_y[c] - node_y[ind];
        const double dz = dims == 3 ? (double)bc_z[c] - node_z[ind] : 0.0;
        // |c_d|: 1 on the axes, sqrt(2) on the diagonals (qLat, GpuInit.cu:1063-1064, :1173-1176)
        const int cc = lattice_cx(Q, d) * lattice_cx(Q, d) + lattice_cy(Q, d) * lattice_cy(Q, d) +
                       lattice_cz(Q, d) * lattice_cz(Q, d);
        q[c] = std::sqrt(dx * dx + dy * dy + dz * dz) / (delta * std::sqrt((double)cc));
    }
    return LBM_OK;
}

static int upload_or_fill(float *dst, const float *src, float value, long long N, cudaStream_t s) {
    if (src) {
        CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(float) * N, cudaMemcpyHostToDevice, s));
        return cudaStreamSynchronize(s) == cudaSuccess ? LBM_OK : fail(LBM_ERR_CUDA, "sync");
    }
    std::vector<float> tmp((size_t)N, value);
    CUDA_TRY(cudaMemcpyAsync(dst, tmp.data(), sizeof(float) * N, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    return LBM_OK;
}

// HEmodel outlets start from the macroscopic fields of the initial state.
__global__ void init_bc_macro_kernel(const uint32_t *word, const int32_t *slot, const int32_t *kind,
                                     const float *rho, const float *ux, const float *uy, const float *uz,
                                     long long n, double *bc_macro) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !(word[i] & W_SPECIAL)) return;
    const int sl = slot[i];
    if (kind[sl] & BCK_HE) {
        bc_macro[4 * sl] = rho[i];
        bc_macro[4 * sl + 1] = ux[i];
        bc_macro[4 * sl + 2] = uy[i];
        bc_macro[4 * sl + 3] = uz[i];
    }
}

static int init_bc_macro(lbm_handle_s *H) {
    if (!H->bc_macro) return LBM_OK;
    const unsigned blocks = (unsigned)((H->N + 255) / 256);
    init_bc_macro_kernel<<<blocks, 256, 0, H->stream>>>(H->word, H->slot, H->kind, H->rho, H->ux, H->uy, H->uz,
                                                        H->N, H->bc_macro);
    CUDA_TRY(cudaGetLastError());
    return LBM_OK;
}

int lbm_init(lbm_handle H, const float *rho, const float *u, const float *v, const float *w) {
    if (!H) return fail(LBM_ERR_INVALID, "null handle");
    int rc;
    if ((rc = upload_or_fill(H->rho, rho, (float)H->P.rho, H->N, H->stream))) return rc;
    if ((rc = upload_or_fill(H->ux, u, (float)H->P.u, H->N, H->stream))) return rc;
    if ((rc = upload_or_fill(H->uy, v, (float)H->P.v, H->N, H->stream))) return rc;
    if ((rc = upload_or_fill(H->uz, w, H->dims == 3 ? (float)H->P.w : 0.0f, H->N, H->stream))) return rc;
    CUDA_TRY(cudaMemsetAsync(H->pux, 0, sizeof(float) * H->N, H->stream));
    CUDA_TRY(cudaMemsetAsync(H->puy, 0, sizeof(float) * H->N, H->stream));
    CUDA_TRY(cudaMemsetAsync(H->puz, 0, sizeof(float) * H->N, H->stream));
    H->fd_recorded = false;
    // MaxMacroDiff compares against the initial fields first (Iterate3D.cu:208-213)
    const size_t fb = sizeof(float) * (size_t)H->N;
    CUDA_TRY(cudaMemcpyAsync(H->mdiff_prev, H->ux, fb, cudaMemcpyDeviceToDevice, H->stream));
    CUDA_TRY(cudaMemcpyAsync(H->mdiff_prev + H->N, H->uy, fb, cudaMemcpyDeviceToDevice, H->stream));
    CUDA_TRY(cudaMemcpyAsync(H->mdiff_prev + 2 * H->N, H->uz, fb, cudaMemcpyDeviceToDevice, H->stream));
    CUDA_TRY(cudaMemcpyAsync(H->mdiff_prev + 3 * H->N, H->rho, fb, cudaMemcpyDeviceToDevice, H->stream));
    StepParams p = make_params(H, 1, 0);  // fout = buffer 0
    const StepParams o = make_params(H, 0, 0);  // fout = buffer 1
    p.init_rho = H->P.rho;
    p.init_ux = H->P.u;
    p.init_uy = H->P.v;
    p.init_uz = H->dims == 3 ? H->P.w : 0.0;
    p.init_from_arrays = (rho ? 1 : 0) | (u ? 2 : 0) | (v ? 4 : 0) | (w ? 8 : 0);
    const int phys = H->P.mode == LBM_MODE_PHYSICS;
    rc = H->q == 9 ? launch_init_q9(p, o, H->P.collision_model, H->P.storage, phys, H->P.init_equilibrium, H->stream)
                   : launch_init_q19(p, o, H->P.collision_model, H->P.storage, phys, H->P.init_equilibrium, H->stream);
    if (rc) return fail(LBM_ERR_UNSUPPORTED, "no kernel for this configuration");
    CUDA_TRY(cudaGetLastError());
    if ((rc = init_bc_macro(H))) return rc;
    CUDA_TRY(cudaStreamSynchronize(H->stream));
    H->cur = 0;
    H->initialised = true;
    H->status = LBM_OK;
    return LBM_OK;
}

static int launch(lbm_handle_s *H, int from, int write_macro, cudaStream_t s) {
    const StepParams p = make_params(H, from, write_macro);
    const int phys = H->P.mode == LBM_MODE_PHYSICS;
    int rc;
    if (H->jit_kernel) {
        const int bx = H->jit_key.block;
        const int units = H->jit_key.pair ? H->n / 2 : H->n;  // threads along x (h-space: one node each)
        const int zw = H->jit_key.hspace && H->jit_key.zwalk > 1 ? H->jit_key.zwalk : 1;
        const dim3 grid((unsigned)((units + bx - 1) / bx), (unsigned)H->m, (unsigned)((H->h + zw - 1) / zw));
        void *args[] = {(void *)&p};
        cudaError_t e = cudaLaunchKernel((const void *)H->jit_fn, grid, dim3((unsigned)bx), args, 0, s);
        return e == cudaSuccess ? LBM_OK : fail(LBM_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
    }
    if (H->tma_kernel) {
        TmaRows rows;
        rows.row = H->tma_row;
        rows.lmask = H->tma_lmask;
        rows.omask = H->tma_omask;
        rows.nrows = H->tma_nrows;
        rows.stages = H->tma_stages;
        rows.err = H->tma_err;
        rc = launch_step_tma(H->q, p, rows, H->P.collision_model, H->P.storage, H->tma_grid, H->tma_smem, s);
    } else if (H->pair_kernel)
        rc = H->q == 9 ? launch_step_x2_q9(p, H->P.collision_model, H->P.storage, phys, s)
                       : launch_step_x2_q19(p, H->P.collision_model, H->P.storage, phys, s);
    else
        rc = H->q == 9 ? launch_step_q9(p, H->P.collision_model, H->P.storage, phys, s)
                       : launch_step_q19(p, H->P.collision_model, H->P.storage, phys, s);
    return rc ? fail(LBM_ERR_UNSUPPORTED, "no kernel for this configuration") : LBM_OK;
}

// Two steps (from buffer c back to buffer c) captured once as a graph.
static int pair_graph(lbm_handle_s *H, int c) {
    if (H->pair[c]) return LBM_OK;
    cudaGraph_t g;
    CUDA_TRY(cudaStreamBeginCapture(H->stream, cudaStreamCaptureModeThreadLocal));
    int rc = launch(H, c, 0, H->stream);
    if (!rc) rc = launch(H, 1 - c, 0, H->stream);
    cudaError_t e = cudaStreamEndCapture(H->stream, &g);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&H->pair[c], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_step(lbm_handle H, int nsteps, int write_macro_last, void *stream) {
    if (!H) return fail(LBM_ERR_INVALID, "null handle");
    if (!H->initialised) return fail(LBM_ERR_INVALID, "lbm_init has not been called");
    if (nsteps < 0) return fail(LBM_ERR_INVALID, "negative step count");
    cudaStream_t s = stream ? (cudaStream_t)stream : H->stream;
    int plain = nsteps - (write_macro_last && nsteps > 0 ? 1 : 0);
    int rc;
    if (plain >= 8) {
        if ((rc = pair_graph(H, H->cur))) return rc;
        for (int i = 0; i + 1 < plain; i += 2) CUDA_TRY(cudaGraphLaunch(H->pair[H->cur], s));
        if (plain & 1) {
            if ((rc = launch(H, H->cur, 0, s))) return rc;
            H->cur ^= 1;
        }
    } else {
        for (int i = 0; i < plain; ++i) {
            if ((rc = launch(H, H->cur, 0, s))) return rc;
            H->cur ^= 1;
        }
    }
    if (nsteps > plain) {
        if ((rc = launch(H, H->cur, 1, s))) return rc;
        H->cur ^= 1;
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(H->stepped, s);
    if (e != cudaSuccess) {
        H->status = LBM_ERR_CUDA;
        return fail(LBM_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
    }
    return LBM_OK;
}

int lbm_get_macro(lbm_handle H, float *rho, float *u, float *v, float *w) {
    if (!H) return fail(LBM_ERR_INVALID, "null handle");
    CUDA_TRY(cudaDeviceSynchronize());
    if (int rc = check_tma(H)) return rc;
    const size_t b = sizeof(float) * H->N;
    if (rho) CUDA_TRY(cudaMemcpy(rho, H->rho, b, cudaMemcpyDeviceToHost));
    if (u) CUDA_TRY(cudaMemcpy(u, H->ux, b, cudaMemcpyDeviceToHost));
    if (v) CUDA_TRY(cudaMemcpy(v, H->uy, b, cudaMemcpyDeviceToHost));
    if (w) CUDA_TRY(cudaMemcpy(w, H->uz, b, cudaMemcpyDeviceToHost));
    return LBM_OK;
}

int lbm_get_populations(lbm_handle H, double *f) {
    if (!H || !f) return fail(LBM_ERR_INVALID, "null argument");
    CUDA_TRY(cudaDeviceSynchronize());
    if (int rc = check_tma(H)) return rc;
    double *tmp = nullptr;
    const size_t bytes = sizeof(double) * (size_t)H->q * H->N;
    CUDA_TRY(cudaMalloc((void **)&tmp, bytes));
    const StepParams p = make_params(H, H->cur, 0);
    if (H->q == 9)
        launch_decode_q9(p, H->P.storage, tmp, H->N, H->stream);
    else
        launch_decode_q19(p, H->P.storage, tmp, H->N, H->stream);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (e == cudaSuccess) e = cudaMemcpy(f, tmp, bytes, cudaMemcpyDeviceToHost);
    cudaFree(tmp);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("read-back: ") + cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_set_populations(lbm_handle H, const double *f) {
    if (!H || !f) return fail(LBM_ERR_INVALID, "null argument");
    CUDA_TRY(cudaStreamWaitEvent(H->stream, H->stepped, 0));
    // macroscopic fields as lbm_init leaves them (the params' constants);
    // the fluid nodes' values are rewritten by the next step that stores them
    int rc;
    if ((rc = upload_or_fill(H->rho, nullptr, (float)H->P.rho, H->N, H->stream))) return rc;
    if ((rc = upload_or_fill(H->ux, nullptr, (float)H->P.u, H->N, H->stream))) return rc;
    if ((rc = upload_or_fill(H->uy, nullptr, (float)H->P.v, H->N, H->stream))) return rc;
    if ((rc = upload_or_fill(H->uz, nullptr, H->dims == 3 ? (float)H->P.w : 0.0f, H->N, H->stream))) return rc;
    const size_t bytes = sizeof(double) * (size_t)H->q * H->N;
    double *tmp = nullptr;
    CUDA_TRY(cudaMallocAsync((void **)&tmp, bytes, H->stream));
    cudaError_t e = cudaMemcpyAsync(tmp, f, bytes, cudaMemcpyHostToDevice, H->stream);
    const StepParams p = make_params(H, H->cur, 0);
    if (e == cudaSuccess) {
        if (H->q == 9)
            launch_encode_q9(p, H->P.storage, tmp, H->N, H->stream);
        else
            launch_encode_q19(p, H->P.storage, tmp, H->N, H->stream);
        e = cudaGetLastError();
    }
    const size_t fb = sizeof(float) * (size_t)H->N;
    if (e == cudaSuccess) e = cudaMemsetAsync(H->pux, 0, fb, H->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(H->puy, 0, fb, H->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(H->puz, 0, fb, H->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(H->mdiff_prev, 0, 4 * fb, H->stream);
    if (e == cudaSuccess && init_bc_macro(H)) e = cudaErrorUnknown;
    cudaFreeAsync(tmp, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("set_populations: ") + cudaGetErrorString(e));
    H->initialised = true;
    H->fd_recorded = false;
    return LBM_OK;
}

// Raw storage state in the reference's SoA order: one 2D copy per direction
// between the row layout (direction d of row r at (r Q + d) n) and
// state[d N + node].
long long lbm_state_bytes(lbm_handle H) { return H ? (long long)H->q * H->N * (long long)H->elem : -1; }

static int state_copy(lbm_handle H, void *host, bool to_host) {
    CUDA_TRY(cudaStreamWaitEvent(H->stream, H->stepped, 0));
    const size_t e = H->elem, n = (size_t)H->n, rows = (size_t)H->m * H->h;
    char *dev = (char *)H->fbuf[H->cur];
    cudaError_t err = cudaSuccess;
    for (int d = 0; d < H->q && err == cudaSuccess; ++d) {
        char *h = (char *)host + (size_t)d * H->N * e;
        char *g = dev + (size_t)d * n * e;
        err = to_host ? cudaMemcpy2DAsync(h, n * e, g, (size_t)H->q * n * e, n * e, rows, cudaMemcpyDeviceToHost,
                                          H->stream)
                      : cudaMemcpy2DAsync(g, (size_t)H->q * n * e, h, n * e, n * e, rows, cudaMemcpyHostToDevice,
                                          H->stream);
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(H->stream);
    if (err != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("state copy: ") + cudaGetErrorString(err));
    return LBM_OK;
}

int lbm_get_state(lbm_handle H, void *state) {
    if (!H || !state) return fail(LBM_ERR_INVALID, "null argument");
    if (!H->initialised) return fail(LBM_ERR_INVALID, "lbm_init has not been called");
    return state_copy(H, state, true);
}

int lbm_set_state(lbm_handle H, const void *state) {
    if (!H || !state) return fail(LBM_ERR_INVALID, "null argument");
    int rc;
    if ((rc = upload_or_fill(H->rho, nullptr, (float)H->P.rho, H->N, H->stream))) return rc;
    if ((rc = upload_or_fill(H->ux, nullptr, (float)H->P.u, H->N, H->stream))) return rc;
    if ((rc = upload_or_fill(H->uy, nullptr, (float)H->P.v, H->N, H->stream))) return rc;
    if ((rc = upload_or_fill(H->uz, nullptr, H->dims == 3 ? (float)H->P.w : 0.0f, H->N, H->stream))) return rc;
    if ((rc = state_copy(H, const_cast<void *>(state), false))) return rc;
    const size_t fb = sizeof(float) * (size_t)H->N;
    CUDA_TRY(cudaMemsetAsync(H->pux, 0, fb, H->stream));
    CUDA_TRY(cudaMemsetAsync(H->puy, 0, fb, H->stream));
    CUDA_TRY(cudaMemsetAsync(H->puz, 0, fb, H->stream));
    CUDA_TRY(cudaMemsetAsync(H->mdiff_prev, 0, 4 * fb, H->stream));
    CUDA_TRY(cudaStreamSynchronize(H->stream));
    H->initialised = true;
    H->fd_recorded = false;
    return LBM_OK;
}

int lbm_macro_norms(lbm_handle H, double *out) {
    if (!H || !out) return fail(LBM_ERR_INVALID, "null argument");
    CUDA_TRY(cudaStreamWaitEvent(H->stream, H->stepped, 0));
    launch_norms(H->word, H->rho, H->ux, H->uy, H->uz, H->pux, H->puy, H->puz, H->N, H->partial,
                 H->norms, H->stream);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(out, H->norms, sizeof(double) * LBM_NORMS, cudaMemcpyDeviceToHost, H->stream));
    CUDA_TRY(cudaStreamSynchronize(H->stream));
    if (int rc = check_tma(H)) return rc;
    for (int k = 0; k < LBM_NORMS; ++k)
        if (!isfinite(out[k])) {
            H->status = LBM_DIVERGED;
            return fail(LBM_DIVERGED, "non-finite macroscopic field (divergence)");
        }
    return LBM_OK;
}

int lbm_residual_l2(lbm_handle H, double *out) {
    if (!H || !out) return fail(LBM_ERR_INVALID, "null argument");
    if (!H->initialised) return fail(LBM_ERR_INVALID, "lbm_init has not been called");
    CUDA_TRY(cudaStreamWaitEvent(H->stream, H->stepped, 0));
    const StepParams p = make_params(H, H->cur, 0);
    const long long nb = H->q == 9 ? resid_l2_partials_q9(p) : resid_l2_partials_q19(p);
    double *partial = nullptr;
    CUDA_TRY(cudaMallocAsync((void **)&partial, sizeof(double) * (nb + 1), H->stream));
    if (H->q == 9) launch_resid_l2_q9(p, H->P.storage, H->P.mode == LBM_MODE_PHYSICS, partial, partial + nb, H->stream);
    else launch_resid_l2_q19(p, H->P.storage, H->P.mode == LBM_MODE_PHYSICS, partial, partial + nb, H->stream);
    cudaError_t e = cudaGetLastError();
    double s = 0.0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&s, partial + nb, sizeof(double), cudaMemcpyDeviceToHost, H->stream);
    cudaFreeAsync(partial, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("L2 residual: ") + cudaGetErrorString(e));
    *out = sqrt(s);
    if (!(*out == *out)) {
        H->status = LBM_DIVERGED;
        return fail(LBM_DIVERGED, "non-finite populations (divergence)");
    }
    return LBM_OK;
}

int lbm_residual_fd_rel_diff(lbm_handle H, double *out) {
    if (!H || !out) return fail(LBM_ERR_INVALID, "null argument");
    if (!H->initialised) return fail(LBM_ERR_INVALID, "lbm_init has not been called");
    const size_t qn = (size_t)H->q * H->N;
    if (!H->fd_snap) CUDA_TRY(cudaMalloc((void **)&H->fd_snap, sizeof(float) * 2 * qn));
    CUDA_TRY(cudaStreamWaitEvent(H->stream, H->stepped, 0));
    const StepParams p = make_params(H, H->cur, 0);
    const long long nb = H->q == 9 ? resid_l2_partials_q9(p) : resid_l2_partials_q19(p);
    double *partial = nullptr;
    CUDA_TRY(cudaMallocAsync((void **)&partial, sizeof(double) * (2 * nb + 2), H->stream));
    const int first = H->fd_recorded ? 0 : 1;
    const int phys = H->P.mode == LBM_MODE_PHYSICS;
    if (H->q == 9)
        launch_fd_rel_q9(p, H->P.storage, phys, H->fd_snap, H->fd_snap + qn, first, partial, partial + 2 * nb,
                         H->stream);
    else
        launch_fd_rel_q19(p, H->P.storage, phys, H->fd_snap, H->fd_snap + qn, first, partial, partial + 2 * nb,
                          H->stream);
    cudaError_t e = cudaGetLastError();
    double r[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(r, partial + 2 * nb, sizeof(r), cudaMemcpyDeviceToHost, H->stream);
    cudaFreeAsync(partial, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("FdRelDiff residual: ") + cudaGetErrorString(e));
    H->fd_recorded = true;
    *out = first ? 0.0 : r[0];
    if (r[1] > 0) {
        H->status = LBM_DIVERGED;
        return fail(LBM_DIVERGED, "non-finite populations (divergence)");
    }
    return LBM_OK;
}

int lbm_momentum_exchange(lbm_handle H, const int *box, double *force) {
    if (!H || !box || !force) return fail(LBM_ERR_INVALID, "null argument");
    if (!H->initialised) return fail(LBM_ERR_INVALID, "lbm_init has not been called");
    if (H->P.mode != LBM_MODE_PHYSICS)
        return fail(LBM_ERR_UNSUPPORTED, "momentum exchange needs physics mode's half-way bounce-back");
    CUDA_TRY(cudaStreamWaitEvent(H->stream, H->stepped, 0));
    const StepParams p = make_params(H, H->cur, 0);
    const long long nb = H->q == 9 ? resid_l2_partials_q9(p) : resid_l2_partials_q19(p);
    double *partial = nullptr;
    CUDA_TRY(cudaMallocAsync((void **)&partial, sizeof(double) * (3 * nb + 3), H->stream));
    if (H->q == 9) launch_momentum_exchange_q9(p, H->P.storage, box, partial, partial + 3 * nb, H->stream);
    else launch_momentum_exchange_q19(p, H->P.storage, box, partial, partial + 3 * nb, H->stream);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(force, partial + 3 * nb, sizeof(double) * 3, cudaMemcpyDeviceToHost, H->stream);
    cudaFreeAsync(partial, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("momentum exchange: ") + cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_macro_diff(lbm_handle H, double *out) {
    if (!H || !out) return fail(LBM_ERR_INVALID, "null argument");
    CUDA_TRY(cudaStreamWaitEvent(H->stream, H->stepped, 0));
    const long long N = H->N;
    launch_macro_diff(H->ux, H->uy, H->uz, H->rho, H->mdiff_prev, H->mdiff_prev + N, H->mdiff_prev + 2 * N,
                      H->mdiff_prev + 3 * N, N, H->partial, H->norms, H->stream);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(out, H->norms, sizeof(double) * 5, cudaMemcpyDeviceToHost, H->stream));
    CUDA_TRY(cudaStreamSynchronize(H->stream));
    if (int rc = check_tma(H)) return rc;
    if (out[4] != 0.0) {
        H->status = LBM_DIVERGED;
        return fail(LBM_DIVERGED, "non-finite macroscopic field (divergence)");
    }
    return LBM_OK;
}

int lbm_build_flags(const lbm_lattice_desc *L, const lbm_params *P, uint64_t *mask, uint32_t *word,
                    int32_t *slot, int *num_bc_nodes) {
    if (!L || !P) return fail(LBM_ERR_INVALID, "null argument");
    RefMasks refm;
    DeviceFlags flags;
    std::string err;
    int rc = build_ref_masks(*L, refm, err);
    if (rc) return fail(rc, err);
    rc = build_device_flags(*L, *P, refm, flags, err);
    if (rc) return fail(rc, err);
    const size_t N = (size_t)L->n * L->m * (L->dims == 2 ? 1 : L->h);
    if (mask) {
        memset(mask, 0, sizeof(uint64_t) * N);
        for (size_t b = 0; b < refm.bc_nodes.size(); ++b) mask[refm.bc_nodes[b]] = refm.mask[b];
    }
    if (word) memcpy(word, flags.word.data(), sizeof(uint32_t) * N);
    if (slot) memcpy(slot, flags.slot.data(), sizeof(int32_t) * N);
    if (num_bc_nodes) *num_bc_nodes = (int)refm.bc_nodes.size();
    return LBM_OK;
}

int lbm_status(lbm_handle H) { return H ? H->status : LBM_ERR_INVALID; }

long long lbm_fluid_nodes(lbm_handle H) { return H ? H->fluid : -1; }

int lbm_kernel_variant(lbm_handle H) {
    return H ? (H->jit_kernel ? 4 : (H->tma_kernel ? 3 : (H->pair_kernel ? 2 : 1))) : -1;
}

const char *lbm_kernel_warning(lbm_handle H) { return H ? H->kernel_warning.c_str() : ""; }

int lbm_autotune(lbm_handle H, int trial_steps, int *block, int *hint, int *pred) {
    if (!H) return fail(LBM_ERR_INVALID, "null handle");
    if (!H->jit_kernel) return fail(LBM_ERR_UNSUPPORTED, "autotuning needs the run-time specialised kernel");
    if (trial_steps < 2) trial_steps = 2;
    // one node per thread in f space: block, load form, bounce-back form and a
    // register cap that buys occupancy; in storage units (h): block and
    // register cap; two nodes per thread (storage units): block and cap.
    // Physics-mode F32 keeps to the storage-unit kernels, whose moments come
    // from deviations: an f-space kernel would bring back the ~1e-6 residual
    // floor of cancelling FP32 sums.
    struct V {
        int block, hint, pred, pair, minb, hs, zw;
    };
    const bool fspace_ok = !(H->P.mode == LBM_MODE_PHYSICS &&
                             (H->P.storage == LBM_STORE_F32 || H->P.storage == LBM_STORE_F16C));
    const bool hs_ok = H->P.storage != LBM_STORE_F64;
    std::vector<V> vs;
    if (fspace_ok) {
        const V fv[] = {{128, 0, 0, 0, 1, 0, 1}, {128, 1, 0, 0, 1, 0, 1}, {128, 0, 1, 0, 1, 0, 1},
                        {128, 1, 1, 0, 1, 0, 1}, {256, 0, 0, 0, 1, 0, 1}, {256, 1, 1, 0, 1, 0, 1},
                        {128, 1, 1, 0, 12, 0, 1}};
        vs.insert(vs.end(), fv, fv + 7);
    }
    if (hs_ok) {
        // register caps of about 64, 48 and 40 per thread; pred = 1 loads the
        // pull and own values before the flag word arrives; zw > 1 walks zw
        // nodes along z per thread with the next flag word loaded ahead
        const V hv[] = {{128, 0, 0, 0, 1, 1, 1}, {128, 0, 0, 0, 10, 1, 1}, {128, 0, 0, 0, 12, 1, 1},
                        {256, 0, 0, 0, 1, 1, 1}, {256, 0, 0, 0, 5, 1, 1},  {128, 0, 1, 0, 1, 1, 1},
                        {128, 0, 1, 0, 10, 1, 1}};
        vs.insert(vs.end(), hv, hv + 7);
        if (H->h >= 16) {
            const V hz[] = {{128, 0, 0, 0, 10, 1, 2}, {128, 0, 0, 0, 10, 1, 4}, {128, 0, 0, 0, 10, 1, 8},
                            {128, 0, 0, 0, 10, 1, 16}, {128, 0, 0, 0, 11, 1, 4}, {256, 0, 0, 0, 5, 1, 4},
                            {64, 0, 0, 0, 20, 1, 4},   {64, 0, 0, 0, 20, 1, 8}, {128, 0, 0, 0, 12, 1, 8},
                            {256, 0, 0, 0, 5, 1, 8},
                            // hint 1 in storage units: predicated bounce-back loads
                            {64, 1, 0, 0, 20, 1, 8},   {64, 1, 0, 0, 20, 1, 4}, {128, 1, 0, 0, 10, 1, 8},
                            {128, 1, 0, 0, 12, 1, 8}};
            vs.insert(vs.end(), hz, hz + 14);
            // two z nodes at a time on FP32x2 (zw + 100 marks them below)
            const V zp[] = {{64, 0, 0, 0, 10, 1, 108}, {64, 0, 0, 0, 8, 1, 108}, {128, 0, 0, 0, 5, 1, 108},
                            {64, 1, 0, 0, 10, 1, 108}, {64, 0, 0, 0, 10, 1, 104}, {128, 0, 0, 0, 4, 1, 108}};
            vs.insert(vs.end(), zp, zp + 6);
        }
    }
    if (H->n % 2 == 0 && hs_ok && !one_node_boundaries(H->P, H->q)) {
        const V pv[] = {{64, 0, 0, 1, 1, 0, 1}, {128, 0, 0, 1, 1, 0, 1}, {64, 0, 0, 1, 12, 0, 1},
                        {128, 0, 0, 1, 6, 0, 1}};
        vs.insert(vs.end(), pv, pv + 4);
    }
    std::vector<JitStepKey> cand;
    for (const V &v : vs) {
        JitStepKey k = H->jit_key;
        k.block = v.block;
        k.hint = v.hint;
        k.pred = v.pred != 0;
        k.pair = v.pair != 0;
        k.minb = v.minb;
        k.hspace = v.hs != 0;
        k.zwalk = v.zw > 100 ? v.zw - 100 : v.zw;
        k.zpair = v.zw > 100;
        cand.push_back(k);
    }
    std::vector<cudaKernel_t> fn(cand.size(), nullptr);
    std::vector<std::string> errs(cand.size());
    {
        std::vector<std::thread> th;
        for (size_t i = 0; i < cand.size(); ++i)
            th.emplace_back([&, i] { jit_step_kernel(cand[i], &fn[i], errs[i]); });
        for (auto &t : th) t.join();
    }
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    const JitStepKey keep = H->jit_key;
    const cudaKernel_t keep_fn = H->jit_fn;
    // each candidate: the median of three windows of trial_steps steps; then
    // the three fastest again over three windows of 4 x trial_steps, so a
    // choice between close candidates does not rest on one short window
    auto time_candidate = [&](size_t i, int steps, float &med) -> int {
        H->jit_key = cand[i];
        H->jit_fn = fn[i];
        int rc = launch(H, H->cur, 0, H->stream);  // warm-up
        if (!rc) rc = launch(H, 1 - H->cur, 0, H->stream);
        float w[3];
        for (int r = 0; r < 3 && !rc; ++r) {
            if (cudaEventRecord(e0, H->stream) != cudaSuccess) return LBM_ERR_CUDA;
            for (int sI = 0; sI < steps && !rc; ++sI) rc = launch(H, (H->cur + sI) & 1, 0, H->stream);
            if (cudaEventRecord(e1, H->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&w[r], e0, e1) != cudaSuccess)
                return LBM_ERR_CUDA;
        }
        if (rc) return rc;
        std::sort(w, w + 3);
        med = w[1];
        return LBM_OK;
    };
    std::vector<std::pair<float, size_t>> order;
    for (size_t i = 0; i < cand.size(); ++i) {
        if (!fn[i]) continue;
        float ms = 0;
        if (time_candidate(i, trial_steps, ms) == LBM_OK) order.push_back({ms, i});
    }
    std::sort(order.begin(), order.end());
    float best = 1e30f;
    int best_i = -1;
    for (size_t r = 0; r < order.size() && r < 3; ++r) {
        float ms = 0;
        if (time_candidate(order[r].second, 4 * trial_steps, ms) == LBM_OK && ms < best) {
            best = ms;
            best_i = (int)order[r].second;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_i < 0) {
        H->jit_key = keep;
        H->jit_fn = keep_fn;
        return fail(LBM_ERR_CUDA, "autotune: no candidate ran: " + errs[0]);
    }
    H->jit_key = cand[best_i];
    H->jit_fn = fn[best_i];
    for (int c = 0; c < 2; ++c)
        if (H->pair[c]) {
            cudaGraphExecDestroy(H->pair[c]);
            H->pair[c] = nullptr;
        }
    {
        std::lock_guard<std::mutex> lock(g_tuned_mutex);
        g_tuned[tune_key(H->jit_key)] = TunedKnobs{H->jit_key.block, H->jit_key.hint, H->jit_key.pred,
                                                   H->jit_key.pair, H->jit_key.minb, H->jit_key.hspace,
                                                   H->jit_key.zpair, H->jit_key.zwalk};
    }
    H->initialised = false;  // the trial steps leave the populations undefined
    if (block) *block = H->jit_key.block;
    if (hint) *hint = H->jit_key.hint | (H->jit_key.hspace ? 2 : 0) | (H->jit_key.zwalk > 1 ? H->jit_key.zwalk << 2 : 0);
    if (pred)
        *pred = (H->jit_key.pred ? 1 : 0) | (H->jit_key.pair ? 2 : 0) | (H->jit_key.minb > 1 ? H->jit_key.minb << 2 : 0) |
                (H->jit_key.zpair ? 1 << 10 : 0);
    return LBM_OK;
}

int lbm_kernel_config(lbm_handle H, int *block, int *hint, int *pred) {
    if (!H) return fail(LBM_ERR_INVALID, "null handle");
    if (block) *block = H->jit_kernel ? H->jit_key.block : STEP_BLOCK;
    if (hint)
        *hint = H->jit_kernel ? H->jit_key.hint | (H->jit_key.hspace ? 2 : 0) |
                                    (H->jit_key.zwalk > 1 ? H->jit_key.zwalk << 2 : 0)
                              : 0;
    if (pred)
        *pred = H->jit_kernel ? (H->jit_key.pred ? 1 : 0) | (H->jit_key.pair ? 2 : 0) |
                                    (H->jit_key.minb > 1 ? H->jit_key.minb << 2 : 0) | (H->jit_key.zpair ? 1 << 10 : 0)
                              : 0;
    return LBM_OK;
}

int lbm_jit_check(int q, int coll, int storage, int phys, int wrap, int nx, int ny, int nz, int block, int hint,
                  int pred) {
    const int minb = (pred >> 2) & 255;
    JitStepKey k{q, coll, storage, phys != 0, wrap != 0, nx, ny, nz, block, hint & 1, (pred & 1) != 0, true,
                 (pred & 2) != 0, minb > 1 ? minb : 1};
    k.hspace = (hint & 2) != 0;
    k.zwalk = k.hspace && (hint >> 2) > 1 ? hint >> 2 : 1;
    k.zpair = k.hspace && ((pred >> 10) & 1) && k.zwalk % 2 == 0;
    std::string err;
    if (jit_step_kernel(k, nullptr, err)) return fail(LBM_ERR_CUDA, err);
    return LBM_OK;
}

int lbm_bytes_per_update(lbm_handle H) { return H ? (int)(2 * H->q * H->elem) : -1; }

void lbm_destroy(lbm_handle H) {
    if (H) cudaStreamSynchronize(H->stream);
    free_handle(H);
}

}  // extern "C"
