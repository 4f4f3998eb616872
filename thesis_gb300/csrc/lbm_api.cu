// C ABI of the lattice-Boltzmann engine (include/thesis_lbm.h): handle
// lifetime, device allocation, initial collision, the step loop (with a
// captured two-step CUDA graph for short steps) and read-back.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <new>
#include <string>
#include <vector>

#include "lbm_flags.h"
#include "lbm_step.cuh"

namespace lbm {
int launch_step_q9(const StepParams &p, int coll, int st, int phys, cudaStream_t s);
int launch_step_q19(const StepParams &p, int coll, int st, int phys, cudaStream_t s);
int launch_init_q9(const StepParams &p, const StepParams &o, int coll, int st, int phys, int eq, cudaStream_t s);
int launch_init_q19(const StepParams &p, const StepParams &o, int coll, int st, int phys, int eq, cudaStream_t s);
int launch_decode_q9(const StepParams &p, int st, double *out, long long n, cudaStream_t s);
int launch_decode_q19(const StepParams &p, int st, double *out, long long n, cudaStream_t s);
int launch_norms(const uint32_t *word, const float *rho, const float *ux, const float *uy,
                 const float *uz, float *pux, float *puy, float *puz, long long n,
                 double *partial, double *out, cudaStream_t s);
int norm_partial_count();
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
    double *partial = nullptr, *norms = nullptr;
    int nslots = 0;
    std::vector<long long> slot_node;
    int cur = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t pair[2] = {nullptr, nullptr};
    int status = LBM_OK;
    bool initialised = false;
    double omega = 1, omega_m = 1, gshift = 0;
    float scale = 1024.f;
};

static StepParams make_params(const lbm_handle_s *H, int from, int write_macro) {
    StepParams p;
    memset(&p, 0, sizeof(p));
    for (int d = 0; d < H->q; ++d) {
        p.fin[d] = (const char *)H->fbuf[from] + (size_t)d * H->stride * H->elem;
        p.fout[d] = (char *)H->fbuf[1 - from] + (size_t)d * H->stride * H->elem;
    }
    p.word = H->word;
    p.slot = H->slot;
    p.bc_mask = H->mask;
    p.bc_kind = H->kind;
    p.bc_uvw = H->uvw;
    p.rho = H->rho;
    p.ux = H->ux;
    p.uy = H->uy;
    p.uz = H->uz;
    p.nx = H->n;
    p.ny = H->m;
    p.nz = H->h;
    p.write_macro = write_macro;
    p.omega = H->omega;
    p.omega_m = H->omega_m;
    p.gshift = H->gshift;
    p.rho_in = H->P.rho_in;
    p.rho_out = H->P.rho_out;
    p.scale = H->scale;
    p.inv_scale = 1.0f / H->scale;
    p.outlet_profile = H->P.outlet_profile;
    p.update_inlet_outlet = H->P.update_inlet_outlet;
    return p;
}

static void free_handle(lbm_handle_s *H) {
    if (!H) return;
    for (int c = 0; c < 2; ++c)
        if (H->pair[c]) cudaGraphExecDestroy(H->pair[c]);
    void *ptrs[] = {H->fbuf[0], H->fbuf[1], H->word, H->slot, H->mask, H->kind, H->uvw,
                    H->rho, H->ux, H->uy, H->uz, H->pux, H->puy, H->puz, H->partial, H->norms};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (H->stream) cudaStreamDestroy(H->stream);
    delete H;
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
    if ((long long)q * N >= (1ll << 31) * 8ll) return fail(LBM_ERR_INVALID, "lattice too large");
    if (N >= (1ll << 31)) return fail(LBM_ERR_INVALID, "more than 2^31 nodes");
    if (L->num_conns > 0 && (!L->bc_i || !L->bc_j || !L->bc_dir || !L->bc_type || (L->dims == 3 && !L->bc_k)))
        return fail(LBM_ERR_INVALID, "missing BC columns");
    if (P->collision_model < LBM_BGKW || P->collision_model > LBM_MRT)
        return fail(LBM_ERR_INVALID, "unknown collision model");
    if (P->storage < LBM_STORE_F32 || P->storage > LBM_STORE_F64)
        return fail(LBM_ERR_INVALID, "unknown storage");
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
    H->elem = P->storage == LBM_STORE_F32 ? 4 : (P->storage == LBM_STORE_F16S ? 2 : 8);
    H->scale = P->f16_scale > 0 ? (float)P->f16_scale : 1024.0f;
    // omega as the reference computes it (GpuInit.cu:102-103)
    H->omega = 1.0 / (3.0 * P->viscosity + 0.5);
    H->omega_m = 8.0 * (2.0 - H->omega) / (8.0 - H->omega);
    H->gshift = L->dims == 3 ? P->g / H->omega : 0.0;
    long long fl = 0;
    for (long long i = 0; i < N; ++i) fl += (L->node_type[i] & 1);
    H->fluid = fl;
    H->nslots = (int)flags.slot_node.size();
    H->slot_node = flags.slot_node;

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
    ALLOC(H->rho, sizeof(float) * N);
    ALLOC(H->ux, sizeof(float) * N);
    ALLOC(H->uy, sizeof(float) * N);
    ALLOC(H->uz, sizeof(float) * N);
    ALLOC(H->pux, sizeof(float) * N);
    ALLOC(H->puy, sizeof(float) * N);
    ALLOC(H->puz, sizeof(float) * N);
    ALLOC(H->partial, sizeof(double) * norm_partial_count());
    ALLOC(H->norms, sizeof(double) * LBM_NORMS);
#undef ALLOC
    cudaError_t e = cudaStreamCreateWithFlags(&H->stream, cudaStreamNonBlocking);
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
    CUDA_TRY(cudaStreamSynchronize(H->stream));
    H->cur = 0;
    H->initialised = true;
    H->status = LBM_OK;
    return LBM_OK;
}

static int launch(lbm_handle_s *H, int from, int write_macro, cudaStream_t s) {
    const StepParams p = make_params(H, from, write_macro);
    const int phys = H->P.mode == LBM_MODE_PHYSICS;
    const int rc = H->q == 9 ? launch_step_q9(p, H->P.collision_model, H->P.storage, phys, s)
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
    if (e != cudaSuccess) {
        H->status = LBM_ERR_CUDA;
        return fail(LBM_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
    }
    return LBM_OK;
}

int lbm_get_macro(lbm_handle H, float *rho, float *u, float *v, float *w) {
    if (!H) return fail(LBM_ERR_INVALID, "null handle");
    CUDA_TRY(cudaDeviceSynchronize());
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

int lbm_macro_norms(lbm_handle H, double *out) {
    if (!H || !out) return fail(LBM_ERR_INVALID, "null argument");
    launch_norms(H->word, H->rho, H->ux, H->uy, H->uz, H->pux, H->puy, H->puz, H->N, H->partial,
                 H->norms, H->stream);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(out, H->norms, sizeof(double) * LBM_NORMS, cudaMemcpyDeviceToHost, H->stream));
    CUDA_TRY(cudaStreamSynchronize(H->stream));
    for (int k = 0; k < LBM_NORMS; ++k)
        if (!isfinite(out[k])) {
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
    const size_t N = refm.mask.size();
    if (mask) memcpy(mask, refm.mask.data(), sizeof(uint64_t) * N);
    if (word) memcpy(word, flags.word.data(), sizeof(uint32_t) * N);
    if (slot) memcpy(slot, flags.slot.data(), sizeof(int32_t) * N);
    if (num_bc_nodes) *num_bc_nodes = (int)refm.bc_nodes.size();
    return LBM_OK;
}

int lbm_status(lbm_handle H) { return H ? H->status : LBM_ERR_INVALID; }

long long lbm_fluid_nodes(lbm_handle H) { return H ? H->fluid : -1; }

int lbm_bytes_per_update(lbm_handle H) { return H ? (int)(2 * H->q * H->elem) : -1; }

void lbm_destroy(lbm_handle H) {
    if (H) cudaStreamSynchronize(H->stream);
    free_handle(H);
}

}  // extern "C"
