// The fused step, init, residual, force and encode/decode kernels' host
// launchers, written once for any lattice Q; lbm_kernels_q9.cu and
// lbm_kernels_q19.cu instantiate them for D2Q9 and D3Q19 (two translation
// units, so the two lattices compile in parallel) under the names the rest of
// the library calls (launch_step_q9, launch_step_q19, ...).
#pragma once
#include "lbm_step_x2.cuh"

namespace lbm {


inline dim3 node_grid(const StepParams &p) {
    return dim3((unsigned)((p.nx + STEP_BLOCK - 1) / STEP_BLOCK), (unsigned)p.ny, (unsigned)p.nz);
}

#define LBM_FOR_ALL(M)                                                                      \
    M(1, 0, false) M(1, 1, false) M(1, 2, false) M(2, 0, false) M(2, 1, false) M(2, 2, false) \
    M(3, 0, false) M(3, 1, false) M(3, 2, false) M(1, 0, true) M(1, 1, true) M(1, 2, true)   \
    M(2, 0, true) M(2, 1, true) M(2, 2, true) M(3, 0, true) M(3, 1, true) M(3, 2, true)   \
    M(1, 3, true) M(2, 3, true) M(3, 3, true)

template <int Q>
int launch_step_t(const StepParams &p, int coll, int st, int phys, cudaStream_t s) {
#define STEP_CASE(C, S, P)                                                         \
    if (coll == C && st == S && (phys != 0) == P) {                                \
        step_kernel<Q, C, S, P><<<node_grid(p), STEP_BLOCK, 0, s>>>(p);           \
        return 0;                                                                  \
    }
    LBM_FOR_ALL(STEP_CASE)
#undef STEP_CASE
    return -1;
}

inline dim3 pair_grid(const StepParams &p) {
    const int pairs = p.nx / 2;
    return dim3((unsigned)((pairs + X2_BLOCK - 1) / X2_BLOCK), (unsigned)p.ny, (unsigned)p.nz);
}

// Two-node kernel (F32 / F16S storage, even nx).
template <int Q>
int launch_step_x2_t(const StepParams &p, int coll, int st, int phys, cudaStream_t s) {
#define X2_CASE(C, S, P)                                                              \
    if (coll == C && st == S && (phys != 0) == P) {                                  \
        step_kernel_x2<Q, C, S, P><<<pair_grid(p), X2_BLOCK, 0, s>>>(p);           \
        return 0;                                                                     \
    }
    X2_CASE(1, 0, false) X2_CASE(1, 1, false) X2_CASE(2, 0, false) X2_CASE(2, 1, false)
    X2_CASE(3, 0, false) X2_CASE(3, 1, false) X2_CASE(1, 0, true) X2_CASE(1, 1, true)
    X2_CASE(2, 0, true) X2_CASE(2, 1, true) X2_CASE(3, 0, true) X2_CASE(3, 1, true)
#undef X2_CASE
    return -1;
}

template <int Q>
int launch_init_t(const StepParams &p, const StepParams &o, int coll, int st, int phys, int eq,
                    cudaStream_t s) {
#define INIT_CASE(C, S, P)                                                         \
    if (coll == C && st == S && (phys != 0) == P) {                                \
        init_kernel<Q, C, S, P><<<node_grid(p), STEP_BLOCK, 0, s>>>(p, o, eq);    \
        return 0;                                                                  \
    }
    LBM_FOR_ALL(INIT_CASE)
#undef INIT_CASE
    return -1;
}

// The reference's L2 residual: per-block partials, then their fixed-order sum.
template <int Q>
int launch_resid_l2_t(const StepParams &p, int st, int phys, double *partial, double *out, cudaStream_t s) {
    const dim3 grid = node_grid(p);
    const long long nb = (long long)grid.x * grid.y * grid.z;
#define R_CASE(S, P)                                                               \
    if (st == S && (phys != 0) == P) resid_l2_kernel<Q, S, P><<<grid, STEP_BLOCK, 0, s>>>(p, partial);
    R_CASE(0, false) R_CASE(1, false) R_CASE(2, false) R_CASE(0, true) R_CASE(1, true) R_CASE(2, true)
    R_CASE(3, true)
#undef R_CASE
    sum_partials_kernel<<<1, 1024, 0, s>>>(partial, nb, out);
    return 0;
}

template <int Q>
int launch_momentum_exchange_t(const StepParams &p, int st, const int *box, double *partial, double *out,
                                 cudaStream_t s) {
    const dim3 grid = node_grid(p);
    const long long nb = (long long)grid.x * grid.y * grid.z;
    const int4 lo = make_int4(box[0], box[2], box[4], 0), hi = make_int4(box[1], box[3], box[5], 0);
    if (st == LBM_STORE_F32) momentum_exchange_kernel<Q, LBM_STORE_F32><<<grid, STEP_BLOCK, 0, s>>>(p, lo, hi, partial, nb);
    else if (st == LBM_STORE_F16S) momentum_exchange_kernel<Q, LBM_STORE_F16S><<<grid, STEP_BLOCK, 0, s>>>(p, lo, hi, partial, nb);
    else if (st == LBM_STORE_F16C) momentum_exchange_kernel<Q, LBM_STORE_F16C><<<grid, STEP_BLOCK, 0, s>>>(p, lo, hi, partial, nb);
    else momentum_exchange_kernel<Q, LBM_STORE_F64><<<grid, STEP_BLOCK, 0, s>>>(p, lo, hi, partial, nb);
    for (int k = 0; k < 3; ++k) sum_partials_kernel<<<1, 1024, 0, s>>>(partial + k * nb, nb, out + k);
    return 0;
}

template <int Q>
int launch_fd_rel_t(const StepParams &p, int st, int phys, float *fprev, float *ffirst, int first,
                      double *partial, double *out, cudaStream_t s) {
    const dim3 grid = node_grid(p);
    const long long nb = (long long)grid.x * grid.y * grid.z;
#define F_CASE(S, P)                                                                                   \
    if (st == S && (phys != 0) == P)                                                                   \
        fd_rel_kernel<Q, S, P><<<grid, STEP_BLOCK, 0, s>>>(p, fprev, ffirst, first, partial, nb);
    F_CASE(0, false) F_CASE(1, false) F_CASE(2, false) F_CASE(0, true) F_CASE(1, true) F_CASE(2, true)
    F_CASE(3, true)
#undef F_CASE
    max_partials_kernel<<<1, 1024, 0, s>>>(partial, nb, out);
    return 0;
}

template <int Q>
long long resid_l2_partials_t(const StepParams &p) {
    const dim3 g = node_grid(p);
    return (long long)g.x * g.y * g.z;
}

template <int Q>
int launch_encode_t(const StepParams &p, int st, const double *in, long long n, cudaStream_t s) {
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (st == LBM_STORE_F32) encode_kernel<Q, LBM_STORE_F32><<<blocks, 256, 0, s>>>(p, in, n);
    else if (st == LBM_STORE_F16S) encode_kernel<Q, LBM_STORE_F16S><<<blocks, 256, 0, s>>>(p, in, n);
    else if (st == LBM_STORE_F16C) encode_kernel<Q, LBM_STORE_F16C><<<blocks, 256, 0, s>>>(p, in, n);
    else encode_kernel<Q, LBM_STORE_F64><<<blocks, 256, 0, s>>>(p, in, n);
    return 0;
}

template <int Q>
int launch_decode_t(const StepParams &p, int st, double *out, long long n, cudaStream_t s) {
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (st == LBM_STORE_F32) decode_kernel<Q, LBM_STORE_F32><<<blocks, 256, 0, s>>>(p, out, n);
    else if (st == LBM_STORE_F16S) decode_kernel<Q, LBM_STORE_F16S><<<blocks, 256, 0, s>>>(p, out, n);
    else if (st == LBM_STORE_F16C) decode_kernel<Q, LBM_STORE_F16C><<<blocks, 256, 0, s>>>(p, out, n);
    else decode_kernel<Q, LBM_STORE_F64><<<blocks, 256, 0, s>>>(p, out, n);
    return 0;
}


}  // namespace lbm

// Defines the launchers of lattice Q under their _q<Q> names.
#define LBM_DEFINE_LAUNCHERS(Q)                                                                              \
    namespace lbm {                                                                                          \
    int launch_step_q##Q(const StepParams &p, int coll, int st, int phys, cudaStream_t s) {                  \
        return launch_step_t<Q>(p, coll, st, phys, s);                                                       \
    }                                                                                                        \
    int launch_step_x2_q##Q(const StepParams &p, int coll, int st, int phys, cudaStream_t s) {               \
        return launch_step_x2_t<Q>(p, coll, st, phys, s);                                                    \
    }                                                                                                        \
    int launch_init_q##Q(const StepParams &p, const StepParams &o, int coll, int st, int phys, int eq,       \
                         cudaStream_t s) {                                                                   \
        return launch_init_t<Q>(p, o, coll, st, phys, eq, s);                                                \
    }                                                                                                        \
    int launch_resid_l2_q##Q(const StepParams &p, int st, int phys, double *partial, double *out,            \
                             cudaStream_t s) {                                                               \
        return launch_resid_l2_t<Q>(p, st, phys, partial, out, s);                                           \
    }                                                                                                        \
    int launch_momentum_exchange_q##Q(const StepParams &p, int st, const int *box, double *partial,          \
                                      double *out, cudaStream_t s) {                                         \
        return launch_momentum_exchange_t<Q>(p, st, box, partial, out, s);                                   \
    }                                                                                                        \
    int launch_fd_rel_q##Q(const StepParams &p, int st, int phys, float *fprev, float *ffirst, int first,   \
                           double *partial, double *out, cudaStream_t s) {                                   \
        return launch_fd_rel_t<Q>(p, st, phys, fprev, ffirst, first, partial, out, s);                       \
    }                                                                                                        \
    long long resid_l2_partials_q##Q(const StepParams &p) { return resid_l2_partials_t<Q>(p); }              \
    int launch_encode_q##Q(const StepParams &p, int st, const double *in, long long n, cudaStream_t s) {     \
        return launch_encode_t<Q>(p, st, in, n, s);                                                          \
    }                                                                                                        \
    int launch_decode_q##Q(const StepParams &p, int st, double *out, long long n, cudaStream_t s) {          \
        return launch_decode_t<Q>(p, st, out, n, s);                                                         \
    }                                                                                                        \
    }
