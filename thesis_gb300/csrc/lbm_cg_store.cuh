// Population storage of the colour-gradient paths (lbm_cg.cu, lbm_cg3.cuh).
//
// A node keeps two values per direction d in two slots, each a direction-major
// array (slot c of direction d at base + (c*Q + d)*N):
//   F32, F64  slot 0 the red population r_d, slot 1 the blue one b_d; the
//             arithmetic runs in the storage type (F64 is the FP64 run of the
//             same solver that the other storages are measured against);
//   F16S      slot 0 the summed population as a shifted FP16 deviation,
//             (r_d + b_d - w_d) * S; slot 1 the minority colour's fraction
//             of it as FP16, its sign bit naming the majority colour: +m for
//             b_d = m f_d (red majority), -m for r_d = m f_d (blue majority),
//             so -0 is pure blue and +0 pure red; the arithmetic runs in FP32.
// Every colour-gradient model here relaxes the summed population as one BGK
// fluid and only splits it by colour in the recolouring, so the summed value
// carries the flow (mass, momentum, pressure) and is stored the way the
// single-phase F16S storage is: as a small deviation from the rest state w_d
// (the rest weights phi_k + theta_k alpha equal w_d for alpha = 4/9), which
// keeps FP16's 11 significant bits on the deviation.  The colour split only
// sets where the interface is: stored as the minority fraction, a bulk phase
// stays exactly one colour and a small admixture keeps 11 significant bits
// of itself, where a stored difference r_d - b_d would carry an absolute
// error of 2^-12 |f_d| into the minority colour everywhere.
#pragma once
#include <cuda_fp16.h>

#include "lbm_device.cuh"

namespace lbm {

template <int ST> struct CgStore;

template <> struct CgStore<LBM_STORE_F32> {
    using T = float;
    using R = float;
    __device__ static __forceinline__ void load(const T *s0, const T *s1, R w, R, R &r, R &b) {
        r = __ldg(s0);
        b = __ldg(s1);
    }
    __device__ static __forceinline__ void store(T *s0, T *s1, R w, R, R r, R b) {
        *s0 = r;
        *s1 = b;
    }
};

template <> struct CgStore<LBM_STORE_F64> {
    using T = double;
    using R = double;
    __device__ static __forceinline__ void load(const T *s0, const T *s1, R w, R, R &r, R &b) {
        r = __ldg(s0);
        b = __ldg(s1);
    }
    __device__ static __forceinline__ void store(T *s0, T *s1, R w, R, R r, R b) {
        *s0 = r;
        *s1 = b;
    }
};

template <> struct CgStore<LBM_STORE_F16S> {
    using T = __half;
    using R = float;
    // inv_s = 1/S
    __device__ static __forceinline__ void load(const T *s0, const T *s1, R w, R inv_s, R &r, R &b) {
        const float f = fmaf(__half2float(__ldg(s0)), inv_s, w);
        const float m = __half2float(__ldg(s1));
        const float minor = fabsf(m) * f;
        if (signbit(m)) {
            r = minor;
            b = f - minor;
        } else {
            b = minor;
            r = f - minor;
        }
    }
    // s = S; a non-positive summed population (not met in a stable run)
    // keeps no colour split: it is stored as red
    __device__ static __forceinline__ void store(T *s0, T *s1, R w, R s, R r, R b) {
        const float f = r + b;
        *s0 = __float2half_rn((f - w) * s);
        float m = 0.f;
        if (f > 0.f) m = r >= b ? __fdividef(b, f) : copysignf(__fdividef(r, f), -1.f);
        *s1 = __float2half_rn(m);
    }
};

// Bytes of one stored value.
__host__ __device__ constexpr int cg_elem_bytes(int st) {
    return st == LBM_STORE_F64 ? 8 : (st == LBM_STORE_F16S ? 2 : 4);
}

}  // namespace lbm
