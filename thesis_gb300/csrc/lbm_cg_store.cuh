// Population storage of the colour-gradient paths (lbm_cg.cu, lbm_cg3.cuh).
//
// A node keeps two values per direction d in two slots, each a direction-major
// array (slot c of direction d at base + (c*Q + d)*N):
//   F32, F64  slot 0 the red population r_d, slot 1 the blue one b_d; the
//             arithmetic runs in the storage type (F64 is the FP64 run of the
//             same solver that the other storages are measured against);
//   F16S      slot 0 the summed population as a shifted FP16 deviation,
//             (r_d + b_d - w_d) * S; slot 1 the minority colour's fraction
//             mu of it, offset by 2^-8 and signed by the majority colour:
//             +(mu + 2^-8) for b_d = mu f_d (red majority), -(mu + 2^-8) for
//             r_d = mu f_d (blue majority).  The offset keeps slightly
//             negative minorities (recolouring can undershoot; -7e-4 f_d at
//             most in the perturbed-bubble tests) down to -2^-8 f_d; a pure
//             phase (mu = 0) stores exactly 2^-8.  The arithmetic runs in
//             FP32.
// Every colour-gradient model here relaxes the summed population as one BGK
// fluid and only splits it by colour in the recolouring, so the summed value
// carries the flow (mass, momentum, pressure) and is stored the way the
// single-phase F16S storage is: as a small deviation from the rest state w_d
// (the rest weights phi_k + theta_k alpha equal w_d for alpha = 4/9), which
// keeps FP16's 11 significant bits on the deviation.  The colour split only
// sets where the interface is: stored as the minority fraction next to
// 2^-8, a bulk phase stays exactly one colour and a small admixture is kept
// to 2^-19 f_d, where a stored difference r_d - b_d would carry an absolute
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
    static constexpr float OFF = 0.00390625f;  // offset of the stored minority fraction, 2^-8
    // inv_s = 1/S
    __device__ static __forceinline__ void load(const T *s0, const T *s1, R w, R inv_s, R &r, R &b) {
        const float f = fmaf(__half2float(__ldg(s0)), inv_s, w);
        const float m = __half2float(__ldg(s1));
        const float minor = (fabsf(m) - OFF) * f;
        if (signbit(m)) {
            r = minor;
            b = f - minor;
        } else {
            b = minor;
            r = f - minor;
        }
    }
    // s = S; a minority below -2^-8 of the sum is clamped there, and a
    // non-positive sum (not met in a stable run) is stored as red
    __device__ static __forceinline__ void store(T *s0, T *s1, R w, R s, R r, R b) {
        const float f = r + b;
        *s0 = __float2half_rn((f - w) * s);
        float m = OFF;
        if (f > 0.f) {
            const bool red = r >= b;
            const float mu = fmaxf(__fdividef(red ? b : r, f), -OFF * 0.99f);
            m = red ? mu + OFF : -(mu + OFF);
        }
        *s1 = __float2half_rn(m);
    }
};

// Bytes of one stored value.
__host__ __device__ constexpr int cg_elem_bytes(int st) {
    return st == LBM_STORE_F64 ? 8 : (st == LBM_STORE_F16S ? 2 : 4);
}

}  // namespace lbm
