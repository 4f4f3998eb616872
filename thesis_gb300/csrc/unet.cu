// U-Net warm start: BF16 tensor-core convolution kernels (forward, data
// gradient, weight gradient), the small kernels around them (pooling,
// upsampling, ReLU masks, loss, Adam) and the host side of the C ABI in
// include/thesis_unet.h.
//
// Tensors are NHWC BF16 with channel counts that are multiples of 16.  A 3x3
// convolution is an implicit GEMM: M = pixels, N = output channels, K = 9 taps
// x input channels, computed with mma.sync.m16n8k16 (BF16 in, FP32
// accumulate).  One block of 4 warps owns 64 consecutive pixels of one image
// row; the three input rows it needs (with a one-pixel halo) are staged in
// shared memory in chunks of 32 channels, the weights come through L1.  The
// data gradient is the same kernel run on the output gradient with the
// weights transposed (cin <-> cout) and flipped (tap -> 8 - tap).  The weight
// gradient is a GEMM over pixels (M = cout, N = cin, K = pixels): each block
// owns one tap, stages pixel-major tiles of the output gradient and of the
// shifted input row, and adds its FP32 partial sums atomically.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdio.h>
#include <math.h>
#include <stdlib.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <map>
#include <string>
#include <vector>

#include "thesis_lbm.h"
#include "thesis_unet.h"
#include "unet_tc.cuh"

namespace {

typedef __nv_bfloat16 bf16;

thread_local std::string g_unet_error;
int ufail(int code, const std::string &m) {
    g_unet_error = m;
    return code;
}

// ---------------------------------------------------------------------------
// Tensor-core primitive.  Fragment layout of m16n8k16 (g = lane / 4,
// t = lane % 4): A (16x16, row-major) registers hold (g, 2t..2t+1),
// (g+8, 2t..), (g, 2t+8..), (g+8, 2t+8..); B (16x8, K-major) holds
// (k = 2t..2t+1, n = g), (k = 2t+8.., n = g); C holds (g, 2t..2t+1),
// (g+8, 2t..2t+1).  The lower 16 bits of a register hold the lower index.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack2(const bf16 *lo, const bf16 *hi) {
    return (uint32_t)*(const uint16_t *)lo | ((uint32_t)*(const uint16_t *)hi << 16);
}

constexpr int TILE_X = 64;     // pixels per block (4 warps x 16)
constexpr int CHUNK = 32;      // input channels staged per pass
constexpr int SROW = 40;       // staged pixel pitch in bf16 (80 B: conflict-free fragment loads)

// out[n, y, x0+p, co] = act(bias[co] + sum_{tap, ci} w[tap][co][ci] in[n, y+ky-1, x0+p+kx-1, ci])
template <int COUT>
__global__ void __launch_bounds__(128) conv3x3_kernel(const bf16 *__restrict__ in, int in_cs, int in_co, int cin,
                                                      const bf16 *__restrict__ w, const float *__restrict__ bias,
                                                      bf16 *__restrict__ out, int out_cs, int out_co,
                                                      float *__restrict__ out32, int H, int W, int relu) {
    __shared__ __align__(16) bf16 s_in[3][TILE_X + 2][SROW];
    const int x0 = blockIdx.x * TILE_X, y = blockIdx.y, n = blockIdx.z;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    constexpr int NT = COUT / 8;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const int p0 = warp * 16 + g;  // this thread's A rows: pixels p0 and p0 + 8

    for (int c0 = 0; c0 < cin; c0 += CHUNK) {
        const int nvec = (cin - c0 >= CHUNK ? CHUNK : cin - c0) / 8;  // 16-byte vectors per pixel
        __syncthreads();
        for (int i = tid; i < 3 * (TILE_X + 2) * 4; i += 128) {
            const int r = i / ((TILE_X + 2) * 4), rem = i % ((TILE_X + 2) * 4), px = rem >> 2, v = rem & 3;
            const int gy = y + r - 1, gx = x0 + px - 1;
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if (v < nvec && gy >= 0 && gy < H && gx >= 0 && gx < W)
                val = *(const uint4 *)(in + (((size_t)n * H + gy) * W + gx) * in_cs + in_co + c0 + v * 8);
            *(uint4 *)&s_in[r][px][v * 8] = val;
        }
        __syncthreads();
#pragma unroll 1
        for (int tap = 0; tap < 9; ++tap) {
            const int ky = tap / 3, kx = tap % 3;
#pragma unroll
            for (int kk = 0; kk < 2; ++kk) {
                if (kk * 2 >= nvec) break;
                const int kc = kk * 16 + 2 * t;
                uint32_t a[4];
                a[0] = *(const uint32_t *)&s_in[ky][p0 + kx][kc];
                a[1] = *(const uint32_t *)&s_in[ky][p0 + 8 + kx][kc];
                a[2] = *(const uint32_t *)&s_in[ky][p0 + kx][kc + 8];
                a[3] = *(const uint32_t *)&s_in[ky][p0 + 8 + kx][kc + 8];
                const bf16 *wt = w + (size_t)tap * COUT * cin + c0 + kc;
#pragma unroll
                for (int j = 0; j < NT; ++j) {
                    const bf16 *wr = wt + (size_t)(j * 8 + g) * cin;
                    const uint32_t b0 = __ldg((const unsigned int *)wr);
                    const uint32_t b1 = __ldg((const unsigned int *)(wr + 8));
                    mma16816(acc[j], a, b0, b1);
                }
            }
        }
    }
    // epilogue: bias, ReLU, BF16 (and optionally FP32) store
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int x = x0 + p0 + 8 * h;
        if (x >= W) continue;
        const size_t pix = ((size_t)n * H + y) * W + x;
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const int co = j * 8 + 2 * t;
            float v0 = acc[j][2 * h], v1 = acc[j][2 * h + 1];
            if (bias) {
                v0 += bias[co];
                v1 += bias[co + 1];
            }
            if (relu) {
                v0 = fmaxf(v0, 0.f);
                v1 = fmaxf(v1, 0.f);
            }
            if (out) *(__nv_bfloat162 *)(out + pix * out_cs + out_co + co) = __floats2bfloat162_rn(v0, v1);
            if (out32) {
                out32[pix * COUT + co] = v0;
                out32[pix * COUT + co + 1] = v1;
            }
        }
    }
}

// dw[tap][co][ci] += sum_p dpre[p][co] in[p shifted by tap][ci]  (one tap per blockIdx.y)
template <int COUT, int CIN>
__global__ void __launch_bounds__(128) wgrad_kernel(const bf16 *__restrict__ dpre, const bf16 *__restrict__ in,
                                                    int in_cs, int in_co, float *__restrict__ dw, int B, int H,
                                                    int W) {
    constexpr int DP = TILE_X + 8;        // pixel pitch of the staged output gradient
    constexpr int IP = TILE_X + 2 + 8;    // pixel pitch of the staged input row
    __shared__ __align__(16) bf16 sD[COUT][DP];
    __shared__ __align__(16) bf16 sI[CIN][IP];
    constexpr int MT = COUT / 16, NTL = CIN / 8, TILES = MT * NTL;
    constexpr int PER = (TILES + 3) / 4;  // tiles per warp
    const int tap = blockIdx.y, ky = tap / 3, kx = tap % 3;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    float acc[PER][4];
#pragma unroll
    for (int i = 0; i < PER; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
    const int xt = (W + TILE_X - 1) / TILE_X;
    const long long rows = (long long)B * H * xt;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const int xi = (int)(r % xt);
        const long long ny = r / xt;
        const int y = (int)(ny % H), n = (int)(ny / H);
        const int x0 = xi * TILE_X;
        __syncthreads();
        // output gradient tile, transposed to [co][pixel]
        for (int i = tid; i < TILE_X * (COUT / 8); i += 128) {
            const int px = i / (COUT / 8), cv = i % (COUT / 8);
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if (x0 + px < W) val = *(const uint4 *)(dpre + (((size_t)n * H + y) * W + x0 + px) * COUT + cv * 8);
            const bf16 *e = (const bf16 *)&val;
#pragma unroll
            for (int k = 0; k < 8; ++k) sD[cv * 8 + k][px] = e[k];
        }
        // input row y + ky - 1, pixels x0 - 1 .. x0 + 64, transposed to [ci][pixel]
        const int gy = y + ky - 1;
        for (int i = tid; i < (TILE_X + 2) * (CIN / 8); i += 128) {
            const int px = i / (CIN / 8), cv = i % (CIN / 8);
            const int gx = x0 + px - 1;
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if (gy >= 0 && gy < H && gx >= 0 && gx < W)
                val = *(const uint4 *)(in + (((size_t)n * H + gy) * W + gx) * in_cs + in_co + cv * 8);
            const bf16 *e = (const bf16 *)&val;
#pragma unroll
            for (int k = 0; k < 8; ++k) sI[cv * 8 + k][px] = e[k];
        }
        __syncthreads();
#pragma unroll
        for (int k0 = 0; k0 < TILE_X; k0 += 16) {
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                const int tile = warp + 4 * i;
                if (tile >= TILES) break;
                const int co0 = (tile / NTL) * 16, ci0 = (tile % NTL) * 8;
                uint32_t a[4];
                const int kc = k0 + 2 * t;
                a[0] = *(const uint32_t *)&sD[co0 + g][kc];
                a[1] = *(const uint32_t *)&sD[co0 + g + 8][kc];
                a[2] = *(const uint32_t *)&sD[co0 + g][kc + 8];
                a[3] = *(const uint32_t *)&sD[co0 + g + 8][kc + 8];
                // output pixel p reads staged input pixel p + kx
                const bf16 *ir = &sI[ci0 + g][kc + kx];
                const uint32_t b0 = pack2(ir, ir + 1), b1 = pack2(ir + 8, ir + 9);
                mma16816(acc[i], a, b0, b1);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int tile = warp + 4 * i;
        if (tile >= TILES) break;
        const int co0 = (tile / NTL) * 16, ci0 = (tile % NTL) * 8;
        float *d = dw + ((size_t)tap * COUT + co0 + g) * CIN + ci0 + 2 * t;
        atomicAdd(d, acc[i][0]);
        atomicAdd(d + 1, acc[i][1]);
        atomicAdd(d + (size_t)8 * CIN, acc[i][2]);
        atomicAdd(d + (size_t)8 * CIN + 1, acc[i][3]);
    }
}

// Elementwise kernels work on 8 channels (16 bytes) per thread: every
// channel count, channel stride and channel offset of the activations is a
// multiple of 8, and the index arithmetic stays in 32 bits (a batch holds
// fewer than 2^31 channel groups; lbm_unet_create checks it).
struct V8 {
    float v[8];
};
__device__ __forceinline__ V8 ld8(const bf16 *p) {
    const uint4 r = __ldg((const uint4 *)p);
    const __nv_bfloat162 *h = (const __nv_bfloat162 *)&r;
    V8 o;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 f = __bfloat1622float2(h[k]);
        o.v[2 * k] = f.x;
        o.v[2 * k + 1] = f.y;
    }
    return o;
}
__device__ __forceinline__ void st8(bf16 *p, const V8 &a) {
    uint4 r;
    __nv_bfloat162 *h = (__nv_bfloat162 *)&r;
#pragma unroll
    for (int k = 0; k < 4; ++k) h[k] = __floats2bfloat162_rn(a.v[2 * k], a.v[2 * k + 1]);
    *(uint4 *)p = r;
}

// db[co] += sum_p dpre[p][co]: thread t sums channel group t % G of pixels
// t / G, t / G + 256 / G, ...; the block adds its partial sums per channel
__global__ void __launch_bounds__(256) bias_grad_kernel(const bf16 *__restrict__ dpre, int cout, int npix,
                                                        float *__restrict__ db) {
    __shared__ float part[256][9];
    const int G = cout / 8, t = threadIdx.x, v = t % G, sets = 256 / G;
    V8 s;
#pragma unroll
    for (int k = 0; k < 8; ++k) s.v[k] = 0.f;
    for (int p = blockIdx.x * sets + t / G; p < npix; p += gridDim.x * sets) {
        const V8 a = ld8(dpre + (size_t)p * cout + 8 * v);
#pragma unroll
        for (int k = 0; k < 8; ++k) s.v[k] += a.v[k];
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) part[t][k] = s.v[k];
    __syncthreads();
    if (t < cout) {
        float a = 0.f;
        for (int q = t / 8; q < 256; q += G) a += part[q][t % 8];
        atomicAdd(db + t, a);
    }
}

// 2x2 average pooling: out[n, y, x, c] = mean of in[n, 2y+i, 2x+j, c]
__global__ void pool_kernel(const bf16 *in, int in_cs, int in_co, bf16 *out, int C, int B, int Ho, int Wo) {
    const int G = C / 8, total = B * Ho * Wo * G;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int g = i % G, p = i / G, x = p % Wo, ny = p / Wo, y = ny % Ho, n = ny / Ho;
        const int Wi = 2 * Wo;
        const size_t b = (((size_t)n * 2 * Ho + 2 * y) * Wi + 2 * x) * in_cs + in_co + 8 * g;
        const V8 a = ld8(in + b), c = ld8(in + b + in_cs), d = ld8(in + b + (size_t)Wi * in_cs),
                 e = ld8(in + b + (size_t)Wi * in_cs + in_cs);
        V8 o;
#pragma unroll
        for (int k = 0; k < 8; ++k) o.v[k] = 0.25f * (a.v[k] + c.v[k] + d.v[k] + e.v[k]);
        st8(out + (size_t)i * 8, o);
    }
}

// nearest x2 upsampling into channels [out_co, out_co + C) of out
__global__ void up_kernel(const bf16 *in, int C, bf16 *out, int out_cs, int out_co, int B, int Ho, int Wo) {
    const int G = C / 8, total = B * Ho * Wo * G;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int g = i % G, p = i / G, x = p % Wo, ny = p / Wo, y = ny % Ho, n = ny / Ho;
        const int Hi = Ho / 2, Wi = Wo / 2;
        *(uint4 *)(out + (size_t)p * out_cs + out_co + 8 * g) =
            __ldg((const uint4 *)(in + (((size_t)n * Hi + y / 2) * Wi + x / 2) * C + 8 * g));
    }
}

// dpre[p][c] = g[p][c] * (act[p][c] > 0)
__global__ void relu_bwd_kernel(const bf16 *g, int g_cs, int g_co, const bf16 *act, int a_cs, int a_co, bf16 *dpre,
                                int C, int npix) {
    const int G = C / 8, total = npix * G;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int v = i % G, p = i / G;
        const V8 a = ld8(act + (size_t)p * a_cs + a_co + 8 * v);
        V8 o = ld8(g + (size_t)p * g_cs + g_co + 8 * v);
#pragma unroll
        for (int k = 0; k < 8; ++k) o.v[k] = a.v[k] > 0.f ? o.v[k] : 0.f;
        st8(dpre + (size_t)i * 8, o);
    }
}

// dpre = (pool gradient + skip gradient) masked by ReLU, at full resolution
__global__ void pool_skip_bwd_kernel(const bf16 *gpool, const bf16 *gskip, int s_cs, int s_co, const bf16 *act,
                                     int a_cs, int a_co, bf16 *dpre, int C, int B, int H, int W) {
    const int G = C / 8, total = B * H * W * G;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int v = i % G, p = i / G, x = p % W, ny = p / W, y = ny % H, n = ny / H;
        const V8 gp = ld8(gpool + (((size_t)n * (H / 2) + y / 2) * (W / 2) + x / 2) * C + 8 * v);
        const V8 gs = ld8(gskip + (size_t)p * s_cs + s_co + 8 * v);
        const V8 a = ld8(act + (size_t)p * a_cs + a_co + 8 * v);
        V8 o;
#pragma unroll
        for (int k = 0; k < 8; ++k) o.v[k] = a.v[k] > 0.f ? 0.25f * gp.v[k] + gs.v[k] : 0.f;
        st8(dpre + (size_t)i * 8, o);
    }
}

// dpre at low resolution = sum of the 2x2 upsampled gradient, masked by ReLU
__global__ void up_bwd_kernel(const bf16 *gup, int g_cs, int g_co, const bf16 *act, bf16 *dpre, int C, int B, int H,
                              int W) {
    const int G = C / 8, total = B * H * W * G;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int v = i % G, p = i / G, x = p % W, ny = p / W, y = ny % H, n = ny / H;
        const int W2 = 2 * W;
        const size_t b = (((size_t)n * 2 * H + 2 * y) * W2 + 2 * x) * g_cs + g_co + 8 * v;
        const V8 a = ld8(gup + b), c = ld8(gup + b + g_cs), d = ld8(gup + b + (size_t)W2 * g_cs),
                 e = ld8(gup + b + (size_t)W2 * g_cs + g_cs);
        const V8 m = ld8(act + (size_t)i * 8);
        V8 o;
#pragma unroll
        for (int k = 0; k < 8; ++k) o.v[k] = m.v[k] > 0.f ? a.v[k] + c.v[k] + d.v[k] + e.v[k] : 0.f;
        st8(dpre + (size_t)i * 8, o);
    }
}

// loss sums: sums[0] += sum_p w_p sum_{c<oc} (y - t)^2, sums[1] += sum_p w_p
__global__ void loss_kernel(const float *pred, int pc, const float *tgt, int oc, const float *wt, long long npix,
                            double *sums) {
    double a = 0, b = 0;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
        const float wp = wt[p];
        float e = 0.f;
        for (int c = 0; c < oc; ++c) {
            const float d = pred[p * pc + c] - tgt[p * oc + c];
            e += d * d;
        }
        a += (double)wp * e;
        b += wp;
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(sums, a);
        atomicAdd(sums + 1, b);
    }
}

// output gradient of the weighted MSE, BF16, pc channels (the unused ones 0)
__global__ void loss_grad_kernel(const float *pred, int pc, const float *tgt, int oc, const float *wt,
                                 int npix, const double *sums, bf16 *dout) {
    const float norm = sums[1] > 0 ? (float)(2.0 / (oc * sums[1])) : 0.f;
    const int G = pc / 8, total = npix * G;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int v = i % G, p = i / G;
        const float wp = norm * wt[p];
        V8 o;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int c = 8 * v + k;
            o.v[k] = c < oc ? wp * (pred[(size_t)i * 8 + k] - tgt[(size_t)p * oc + c]) : 0.f;
        }
        st8(dout + (size_t)i * 8, o);
    }
}

__global__ void adam_kernel(float *p, const float *g, float *m, float *v, long long n, float lr, float c1, float c2) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = 0.9f * m[i] + 0.1f * gi;
        const float vi = 0.999f * v[i] + 0.001f * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
    }
}

// BF16 copies of one layer's FP32 weights [9][cout][cin]: w and the data-
// gradient form wt[tap'][ci][co] = w[8 - tap'][co][ci]
__global__ void weights_kernel(const float *p, bf16 *w, bf16 *wt, int cout, int cin) {
    const int total = 9 * cout * cin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int ci = i % cin, co = (i / cin) % cout, tap = i / (cin * cout);
        const bf16 b = __float2bfloat16(p[i]);
        w[i] = b;
        wt[((size_t)(8 - tap) * cin + ci) * cout + co] = b;
    }
}

// float inputs [n][H][W][ic] -> BF16 [n][H][W][16], zero padded
__global__ void pack_input_kernel(const float *in, int ic, bf16 *out, long long npix) {
    const long long total = npix * 16;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % 16);
        const long long p = i / 16;
        out[i] = __float2bfloat16(c < ic ? in[p * ic + c] : 0.f);
    }
}

__global__ void unpack_output_kernel(const float *in, int pc, float *out, int oc, long long npix) {
    const long long total = npix * oc;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
        out[i] = in[(i / oc) * pc + i % oc];
}

int grid_for(long long n, int block = 256) {
    long long b = (n + block - 1) / block;
    return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct Act {  // a tensor of the network: NHWC, channel stride cs, first channel co
    bf16 *p = nullptr;
    int cs = 0, co = 0, C = 0, level = 0;
};

struct Layer {
    int cin, cout, relu;
    size_t w_off, b_off;  // into the FP32 parameter vector
    bf16 *w = nullptr, *wt = nullptr;
};

}  // namespace

struct lbm_unet_s {
    lbm_unet_config cfg;
    int levels = 3;
    int base = 16, cap = 64;   // channel widths c_l = min(base * 2^l, cap)
    bool tc = true;            // 3x3 convolutions with 16..128 outputs on tcgen05 (unet_tc.cuh)
    int sms = 1, smem_optin = 0;  // the device's SM count and opt-in shared memory per block
    size_t smem_per_sm = 0;       // shared memory per SM
    // tensor-core configuration per layer shape (+-(cout * 4096 + cin) for
    // convolutions / weight gradients): instance index and CTAs per SM
    std::map<int, std::pair<int, int>> tc_choice;
    int *tc_err = nullptr;     // set by a tensor-core kernel whose bounded wait gave up
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double last_ms = 0;
    std::vector<Layer> L;  // enc_a(l), enc_b(l) for l < levels; bottleneck a, b; dec_a(l), dec_b(l) for
                           // l = levels-1 .. 0; output
    long long nparams = 0;
    float *params = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    long long adam_t = 0;
    std::vector<void *> allocs;
    // activations per level and their gradients: e_a[l] first encoder conv,
    // cat[l] = [upsampled decoder input | second encoder conv (the skip)],
    // p[l] pooled (level l + 1), d_a[l] / d_b[l] decoder convs, ba / bb bottleneck
    Act x0, ba, bb, g_ba, g_bb;
    std::vector<Act> e_a, cat, p, d_a, d_b, g_e_a, g_cat, g_p, g_d_a, g_d_b;
    float *out32 = nullptr;     // [B][H][W][16] FP32 output
    bf16 *dout = nullptr;       // its gradient
    bf16 *dpre = nullptr;       // scratch: a layer's pre-activation gradient
    float *fin = nullptr, *fout = nullptr;  // host-format staging
    float *tgt = nullptr, *wt = nullptr;    // batch targets and weights
    double *sums = nullptr;
    // dataset
    int ds_count = 0;
    bf16 *ds_in = nullptr;
    float *ds_tgt = nullptr, *ds_wt = nullptr;
};

namespace {

int H_of(const lbm_unet_s *u, int level) { return u->cfg.height >> level; }
int W_of(const lbm_unet_s *u, int level) { return u->cfg.width >> level; }

// widths: c_l = min(base * 2^l, cap); the second decoder conv of level l
// outputs c_(l-1) (c_0 at level 0), which level l-1 upsamples into its
// concatenation; level levels-1 upsamples the bottleneck (c_levels)
int ch(const lbm_unet_s *u, int l) { return (u->base << l) < u->cap ? (u->base << l) : u->cap; }
int ch_dec_b(const lbm_unet_s *u, int l) { return l > 0 ? ch(u, l - 1) : ch(u, 0); }
int ch_up(const lbm_unet_s *u, int l) { return l == u->levels - 1 ? ch(u, u->levels) : ch(u, l); }
int enc_a(int l) { return 2 * l; }
int enc_b(int l) { return 2 * l + 1; }
int bott_a(const lbm_unet_s *u) { return 2 * u->levels; }
int bott_b(const lbm_unet_s *u) { return 2 * u->levels + 1; }
int dec_a(const lbm_unet_s *u, int l) { return 2 * u->levels + 2 + 2 * (u->levels - 1 - l); }
int dec_b(const lbm_unet_s *u, int l) { return dec_a(u, l) + 1; }
int out_layer(const lbm_unet_s *u) { return 4 * u->levels + 2; }

int alloc(lbm_unet_s *u, void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes > 0 ? bytes : 16);
    if (e != cudaSuccess) return ufail(LBM_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    u->allocs.push_back(*p);
    cudaMemsetAsync(*p, 0, bytes > 0 ? bytes : 16, u->stream);
    return LBM_OK;
}

int make_act(lbm_unet_s *u, Act &a, int C, int level) {
    a.C = C;
    a.cs = C;
    a.co = 0;
    a.level = level;
    const size_t n = (size_t)u->cfg.max_batch * H_of(u, level) * W_of(u, level) * C;
    return alloc(u, (void **)&a.p, n * sizeof(bf16));
}

Act view(const Act &a, int co, int C) {
    Act v = a;
    v.co = co;
    v.C = C;
    return v;
}

// Blocks of `threads` threads of a kernel that fit an SM by registers
// (65,536 per SM, allocated per thread in multiples of 8) and by threads;
// 1 when the attributes cannot be read.
int resident_by_registers(const void *kern, int threads) {
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, kern) != cudaSuccess || a.numRegs <= 0) return 1;
    const int regs = (a.numRegs + 7) / 8 * 8;
    const int by_regs = 65536 / (regs * ((threads + 31) / 32 * 32));
    return std::max(1, std::min(by_regs, 2048 / threads));
}

// The driver's tensor-map encoder, through the runtime (no -lcuda); looked
// up once per process (a function-local static is initialised thread-safely).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (PFN_cuTensorMapEncodeTiled_v12000)p;
        return nullptr;
    }();
    return fn;
}

// Tensor map of C channels of an NHWC BF16 tensor (channel stride cs, base
// at its first channel): dims (channel, x, y, image), boxes of box_c
// channels x box_x pixels x box_y rows, swizzled by the box's row bytes
// (128, 64 or 32: 64, 32 or 16 channels); out-of-image elements read zero.
bool nhwc_tensor_map(CUtensorMap *m, const bf16 *p, int C, int cs, int H, int W, int B, int box_c, int box_x,
                     int box_y) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t pcs = (cuuint64_t)cs * sizeof(bf16);
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {pcs, pcs * W, pcs * W * H};
    const cuuint32_t box[4] = {(cuuint32_t)box_c, (cuuint32_t)box_x, (cuuint32_t)box_y, 1}, es[4] = {1, 1, 1, 1};
    const CUtensorMapSwizzle sw = box_c == 64 ? CU_TENSOR_MAP_SWIZZLE_128B
                                              : (box_c == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)p, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the convolution's input rows: chunk channels x TC_BOX pixels x 3 rows
bool act_tensor_map(CUtensorMap *m, const Act &a, int cin, int chunk, int H, int W, int B) {
    return nhwc_tensor_map(m, a.p + a.co, cin, a.cs, H, W, B, chunk, unet_tc::TC_BOX, 3);
}

void conv(lbm_unet_s *u, const Layer &l, const Act &in, const Act &out, const float *bias, float *out32, int B,
          int level, bool transposed) {
    const int H = H_of(u, level), W = W_of(u, level);
    dim3 grid((W + TILE_X - 1) / TILE_X, H, B);
    const bf16 *w = transposed ? l.wt : l.w;
    const int cin = transposed ? l.cout : l.cin, cout = transposed ? l.cin : l.cout;
    const int relu = transposed ? 0 : l.relu;
    bf16 *op = out.p;
    if (u->tc && (cout == 16 || cout == 32 || cout == 64 || cout == 128) && cin % 16 == 0) {
        // persistent tensor-core kernel, the layer's weights resident in
        // shared memory, input rows by tensor copies.  Each CTA is one
        // pipeline whose jobs cost about the same whatever their size, and
        // which needs two copies in flight to hide their latency, so the
        // configuration (chunk of input channels, stages) maximises resident
        // CTAs x chunk x min(stages - 1, 2), then resident CTAs, chunk and
        // stages.  Measured on a
        // 16 x 256 x 1024 batch: for 16 input channels three CTAs of 4 stages
        // beat four of 2 stages 1.8x; for 32, three CTAs of 16-channel chunks
        // beat one CTA of 32-channel chunks 1.6x, and with 64 outputs two
        // CTAs of 2 stages beat one of 4 stages 1.3x; for 64, one CTA of one
        // 64-channel chunk beat two CTAs of four 16-channel chunks 1.1x
        const long long tiles = (long long)B * H * ((W + unet_tc::TC_M - 1) / unet_tc::TC_M);
        int best = -1, best_occ = 1, idx = 0;
        long long best_score = -1;
        const int key = cout * 4096 + cin;
        const bool cached = u->tc_choice.count(key) != 0;
        if (cached) {
            best = u->tc_choice[key].first;
            best_occ = u->tc_choice[key].second;
        }
#define TC_LIST(X)                                                                                              \
    X(16, 64, 3) X(16, 32, 3) X(16, 32, 2) X(16, 16, 4) X(16, 16, 2)                                            \
    X(32, 64, 3) X(32, 32, 4) X(32, 32, 3) X(32, 32, 2) X(32, 16, 4) X(32, 16, 2)                               \
    X(64, 64, 3) X(64, 64, 2) X(64, 32, 4) X(64, 32, 3) X(64, 32, 2) X(64, 16, 4) X(64, 16, 2)                  \
    X(128, 64, 3) X(128, 32, 3) X(128, 32, 2) X(128, 16, 4) X(128, 16, 2)
#define TC_EVAL(CO, CH, NS)                                                                                     \
    {                                                                                                           \
        using SM = unet_tc::TcSmem<CO, CH, NS>;                                                                 \
        const size_t bytes = SM::bytes(cin);                                                                    \
        if (cout == CO && cin % CH == 0 && bytes <= (size_t)u->smem_optin) {                                    \
            auto kern = unet_tc::conv3x3_tc_kernel<CO, CH, NS>;                                                 \
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);                \
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,                          \
                                 cudaSharedmemCarveoutMaxShared);                                               \
            const int occ = std::min(std::min((int)(u->smem_per_sm / (bytes + 1024)),                           \
                                              512 / std::max(32, SM::NA * CO)),                                 \
                                     resident_by_registers((const void *)kern, 160));                          \
            const long long score = (long long)occ * CH * std::min(NS - 1, 2) * 1024 + occ * 128 + CH + NS;   \
            if (occ >= 1 && score > best_score) {                                                               \
                best_score = score;                                                                             \
                best = idx;                                                                                     \
                best_occ = occ;                                                                                 \
            }                                                                                                   \
        }                                                                                                       \
        ++idx;                                                                                                  \
    }
#define TC_RUN(CO, CH, NS)                                                                                      \
    {                                                                                                           \
        if (idx == best) {                                                                                      \
            auto kern = unet_tc::conv3x3_tc_kernel<CO, CH, NS>;                                                 \
            const int bytes = (int)unet_tc::TcSmem<CO, CH, NS>::bytes(cin);                                     \
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);                     \
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,                          \
                                 cudaSharedmemCarveoutMaxShared);                                               \
            const long long g = (long long)u->sms * best_occ < tiles ? (long long)u->sms * best_occ : tiles;    \
            kern<<<(unsigned)g, 160, bytes, u->stream>>>(map, cin, w, bias, op, out.cs, out.co, out32, B, H, W,  \
                                                         relu, u->tc_err);                                      \
        }                                                                                                       \
        ++idx;                                                                                                  \
    }
        if (!cached) {
            TC_LIST(TC_EVAL)
            u->tc_choice[key] = std::make_pair(best, best_occ);
        }
        if (best >= 0) {
            int chunk = 0;
            idx = 0;
#define TC_CHUNK(CO, CH, NS)                                                                                    \
    {                                                                                                           \
        if (idx == best) chunk = CH;                                                                            \
        ++idx;                                                                                                  \
    }
            TC_LIST(TC_CHUNK)
            CUtensorMap map;
            if (act_tensor_map(&map, in, cin, chunk, H, W, B)) {
                idx = 0;
                TC_LIST(TC_RUN)
                return;
            }
            fprintf(stderr, "thesis_unet: tensor map encoding failed; convolutions fall back to mma.sync\n");
            u->tc = false;
        }
#undef TC_CHUNK
#undef TC_RUN
#undef TC_EVAL
#undef TC_LIST
    }
    switch (cout) {
    case 16: conv3x3_kernel<16><<<grid, 128, 0, u->stream>>>(in.p, in.cs, in.co, cin, w, bias, op, out.cs, out.co, out32, H, W, relu); break;
    case 32: conv3x3_kernel<32><<<grid, 128, 0, u->stream>>>(in.p, in.cs, in.co, cin, w, bias, op, out.cs, out.co, out32, H, W, relu); break;
    case 64: conv3x3_kernel<64><<<grid, 128, 0, u->stream>>>(in.p, in.cs, in.co, cin, w, bias, op, out.cs, out.co, out32, H, W, relu); break;
    case 128: conv3x3_kernel<128><<<grid, 128, 0, u->stream>>>(in.p, in.cs, in.co, cin, w, bias, op, out.cs, out.co, out32, H, W, relu); break;
    default: ufail(LBM_ERR_INVALID, "no convolution kernel for this width"); break;
    }
}

// persistent tensor-core weight gradient (unet_tc.cuh); false when the
// layer's shape has no instance
bool wgrad_tc(lbm_unet_s *u, const Layer &l, const Act &in, int B, int H, int W, float *dw) {
    const int nc = l.cin < 64 ? l.cin : 64;
    if (l.cin % nc) return false;
    const long long units = (long long)B * H * ((W + unet_tc::TC_M - 1) / unet_tc::TC_M);
    CUtensorMap tdp, tin;
    if (!nhwc_tensor_map(&tdp, u->dpre, l.cout, l.cout, H, W, B, l.cout, unet_tc::TC_M, 3) ||
        !nhwc_tensor_map(&tin, in.p + in.co, l.cin, in.cs, H, W, B, nc, unet_tc::TC_BOX, 1)) {
        fprintf(stderr, "thesis_unet: tensor map encoding failed; weight gradients fall back to mma.sync\n");
        u->tc = false;
        return false;
    }
    // the most resident CTAs, then the most stages
    int best = -1, best_occ = 1, idx = 0;
    long long best_score = -1;
    const int key = -(l.cout * 4096 + l.cin);
    const bool cached = u->tc_choice.count(key) != 0;
    if (cached) {
        best = u->tc_choice[key].first;
        best_occ = u->tc_choice[key].second;
    }
#define WG_LIST(X)                                                                                              \
    X(16, 16, 4) X(16, 16, 3) X(16, 16, 2) X(16, 32, 4) X(16, 32, 3) X(16, 32, 2) X(16, 64, 4) X(16, 64, 3)     \
    X(16, 64, 2) X(32, 16, 4) X(32, 16, 3) X(32, 16, 2) X(32, 32, 4) X(32, 32, 3) X(32, 32, 2) X(32, 64, 4)     \
    X(32, 64, 3) X(32, 64, 2) X(64, 16, 4) X(64, 16, 3) X(64, 16, 2) X(64, 32, 4) X(64, 32, 3) X(64, 32, 2)     \
    X(64, 64, 4) X(64, 64, 3) X(64, 64, 2)
#define WG_EVAL(CO, NC, NS)                                                                                     \
    {                                                                                                           \
        using SM = unet_tc::WgSmem<CO, NC, NS>;                                                                 \
        if (l.cout == CO && nc == NC && SM::BYTES <= u->smem_optin) {                                           \
            auto kern = unet_tc::wgrad_tc_kernel<CO, NC, NS>;                                                   \
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SM::BYTES);                  \
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,                          \
                                 cudaSharedmemCarveoutMaxShared);                                               \
            const int occ = std::min(std::min((int)(u->smem_per_sm / (SM::BYTES + 1024)), 512 / (int)SM::COLS),  \
                                     resident_by_registers((const void *)kern, 128));                          \
            const long long score = (long long)occ * 16 + NS;                                                  \
            if (occ >= 1 && score > best_score) {                                                               \
                best_score = score;                                                                             \
                best = idx;                                                                                     \
                best_occ = occ;                                                                                 \
            }                                                                                                   \
        }                                                                                                       \
        ++idx;                                                                                                  \
    }
#define WG_RUN(CO, NC, NS)                                                                                      \
    {                                                                                                           \
        if (idx == best) {                                                                                      \
            using SM = unet_tc::WgSmem<CO, NC, NS>;                                                             \
            auto kern = unet_tc::wgrad_tc_kernel<CO, NC, NS>;                                                   \
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SM::BYTES);                  \
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,                          \
                                 cudaSharedmemCarveoutMaxShared);                                               \
            const int split = l.cin / NC;                                                                       \
            long long g = ((long long)u->sms * best_occ + split - 1) / split;                                   \
            /* at least 8 rows per CTA: each CTA ends with 9 x CO x NC reductions */                            \
            g = g < (units + 7) / 8 ? g : (units + 7) / 8;                                                      \
            kern<<<dim3((unsigned)g, split), 128, SM::BYTES, u->stream>>>(tdp, tin, l.cin, dw, B, H, W,          \
                                                                          u->tc_err);                           \
        }                                                                                                       \
        ++idx;                                                                                                  \
    }
    if (!cached) {
        WG_LIST(WG_EVAL)
        u->tc_choice[key] = std::make_pair(best, best_occ);
    }
    if (best < 0) return false;
    idx = 0;
    WG_LIST(WG_RUN)
#undef WG_RUN
#undef WG_EVAL
#undef WG_LIST
    return true;
}

void wgrad(lbm_unet_s *u, const Layer &l, const Act &in, int B, int level) {
    const int H = H_of(u, level), W = W_of(u, level);
    const long long rows = (long long)B * H * ((W + TILE_X - 1) / TILE_X);
    dim3 grid((unsigned)(rows < 64 ? rows : 64), 9);
    float *dw = u->grad + l.w_off;
    const long long npix = (long long)B * H * W;
    if (u->tc && l.cin % 16 == 0 && wgrad_tc(u, l, in, B, H, W, dw)) {
        bias_grad_kernel<<<grid_for(npix * (l.cout / 8), 256), 256, 0, u->stream>>>(u->dpre, l.cout, (int)npix,
                                                                                 u->grad + l.b_off);
        return;
    }
#define WG(CO, CI)                                                                                            \
    if (l.cout == CO && l.cin == CI) {                                                                        \
        wgrad_kernel<CO, CI><<<grid, 128, 0, u->stream>>>(u->dpre, in.p, in.cs, in.co, dw, B, H, W);         \
    } else
    WG(16, 16) WG(32, 16) WG(32, 32) WG(64, 32) WG(64, 64) WG(64, 128) WG(32, 64) WG(16, 32) {
        ufail(LBM_ERR_INVALID, "no weight-gradient kernel for this layer shape");
    }
#undef WG
    bias_grad_kernel<<<grid_for(npix * (l.cout / 8), 256), 256, 0, u->stream>>>(u->dpre, l.cout, (int)npix,
                                                                                 u->grad + l.b_off);
}

void refresh_weights(lbm_unet_s *u) {
    for (const Layer &l : u->L)
        weights_kernel<<<grid_for(9LL * l.cout * l.cin), 256, 0, u->stream>>>(u->params + l.w_off, l.w, l.wt, l.cout,
                                                                               l.cin);
}

// forward pass on the batch in x0; FP32 output in out32
void forward(lbm_unet_s *u, int B) {
    auto &L = u->L;
    const float *P = u->params;
    const int NL = u->levels;
    auto cv = [&](int k, const Act &in, const Act &out, int lev, float *o32 = nullptr) {
        conv(u, L[k], in, out, P + L[k].b_off, o32, B, lev, false);
    };
    Act x = u->x0;
    for (int l = 0; l < NL; ++l) {
        cv(enc_a(l), x, u->e_a[l], l);
        const Act skip = view(u->cat[l], ch_up(u, l), ch(u, l));
        cv(enc_b(l), u->e_a[l], skip, l);
        const long long n = (long long)B * H_of(u, l + 1) * W_of(u, l + 1) * ch(u, l);
        pool_kernel<<<grid_for(n / 8), 256, 0, u->stream>>>(skip.p, skip.cs, skip.co, u->p[l].p, ch(u, l), B,
                                                          H_of(u, l + 1), W_of(u, l + 1));
        x = u->p[l];
    }
    cv(bott_a(u), x, u->ba, NL);
    cv(bott_b(u), u->ba, u->bb, NL);
    Act prev = u->bb;
    for (int l = NL - 1; l >= 0; --l) {
        const long long n = (long long)B * H_of(u, l) * W_of(u, l) * prev.C;
        up_kernel<<<grid_for(n / 8), 256, 0, u->stream>>>(prev.p, prev.C, u->cat[l].p, u->cat[l].cs, 0, B, H_of(u, l),
                                                        W_of(u, l));
        cv(dec_a(u, l), u->cat[l], u->d_a[l], l);
        cv(dec_b(u, l), u->d_a[l], u->d_b[l], l);
        prev = u->d_b[l];
    }
    Act none;
    cv(out_layer(u), u->d_b[0], none, 0, u->out32);
}

// backward pass from dout; parameter gradients accumulate into grad
void backward(lbm_unet_s *u, int B) {
    auto &L = u->L;
    const int NL = u->levels;
    auto npix = [&](int lev) { return (long long)B * H_of(u, lev) * W_of(u, lev); };
    auto dgrad = [&](int k, const Act &gin, int lev) {
        Act d;
        d.p = u->dpre;
        d.cs = L[k].cout;
        d.co = 0;
        d.C = L[k].cout;
        conv(u, L[k], d, gin, nullptr, nullptr, B, lev, true);
    };
    auto relu_bwd = [&](const Act &g, const Act &act, int C, int lev) {
        const long long n = npix(lev) * C;
        relu_bwd_kernel<<<grid_for(n / 8), 256, 0, u->stream>>>(g.p, g.cs, g.co, act.p, act.cs, act.co, u->dpre, C,
                                                                  (int)npix(lev));
    };
    auto pool_skip = [&](const Act &gpool, const Act &gskip, const Act &act, int C, int lev) {
        const long long n = npix(lev) * C;
        pool_skip_bwd_kernel<<<grid_for(n / 8), 256, 0, u->stream>>>(gpool.p, gskip.p, gskip.cs, gskip.co, act.p,
                                                                   act.cs, act.co, u->dpre, C, B, H_of(u, lev),
                                                                   W_of(u, lev));
    };
    auto up_bwd = [&](const Act &gup, const Act &act, int C, int lev) {
        const long long n = npix(lev) * C;
        up_bwd_kernel<<<grid_for(n / 8), 256, 0, u->stream>>>(gup.p, gup.cs, gup.co, act.p, u->dpre, C, B, H_of(u, lev),
                                                            W_of(u, lev));
    };
    // output layer: dpre = dout
    cudaMemcpyAsync(u->dpre, u->dout, sizeof(bf16) * npix(0) * 16, cudaMemcpyDeviceToDevice, u->stream);
    wgrad(u, L[out_layer(u)], u->d_b[0], B, 0);
    dgrad(out_layer(u), u->g_d_b[0], 0);
    // decoder, from level 0 up
    for (int l = 0; l < NL; ++l) {
        if (l == 0)
            relu_bwd(u->g_d_b[0], u->d_b[0], ch_dec_b(u, 0), 0);
        else  // d_b[l] was upsampled into the first channels of cat[l-1]
            up_bwd(view(u->g_cat[l - 1], 0, ch_dec_b(u, l)), u->d_b[l], ch_dec_b(u, l), l);
        wgrad(u, L[dec_b(u, l)], u->d_a[l], B, l);
        dgrad(dec_b(u, l), u->g_d_a[l], l);
        relu_bwd(u->g_d_a[l], u->d_a[l], ch(u, l), l);
        wgrad(u, L[dec_a(u, l)], u->cat[l], B, l);
        dgrad(dec_a(u, l), u->g_cat[l], l);
    }
    // bottleneck
    up_bwd(view(u->g_cat[NL - 1], 0, ch(u, NL)), u->bb, ch(u, NL), NL);
    wgrad(u, L[bott_b(u)], u->ba, B, NL);
    dgrad(bott_b(u), u->g_ba, NL);
    relu_bwd(u->g_ba, u->ba, ch(u, NL), NL);
    wgrad(u, L[bott_a(u)], u->p[NL - 1], B, NL);
    dgrad(bott_a(u), u->g_p[NL - 1], NL);
    // encoder, from the deepest level down
    for (int l = NL - 1; l >= 0; --l) {
        pool_skip(u->g_p[l], view(u->g_cat[l], ch_up(u, l), ch(u, l)), view(u->cat[l], ch_up(u, l), ch(u, l)), ch(u, l), l);
        wgrad(u, L[enc_b(l)], u->e_a[l], B, l);
        dgrad(enc_b(l), u->g_e_a[l], l);
        relu_bwd(u->g_e_a[l], u->e_a[l], ch(u, l), l);
        wgrad(u, L[enc_a(l)], l == 0 ? u->x0 : u->p[l - 1], B, l);
        if (l > 0) dgrad(enc_a(l), u->g_p[l - 1], l);
    }
}

// loss and output gradient of the batch whose targets and weights are in tgt, wt
void loss(lbm_unet_s *u, int B) {
    const long long np = (long long)B * u->cfg.height * u->cfg.width;
    cudaMemsetAsync(u->sums, 0, 2 * sizeof(double), u->stream);
    loss_kernel<<<grid_for(np), 256, 0, u->stream>>>(u->out32, 16, u->tgt, u->cfg.out_channels, u->wt, np, u->sums);
    loss_grad_kernel<<<grid_for(np * 2), 256, 0, u->stream>>>(u->out32, 16, u->tgt, u->cfg.out_channels, u->wt,
                                                               (int)np, u->sums, u->dout);
}

int gather_batch(lbm_unet_s *u, int batch, const int *idx) {
    if (batch < 1 || batch > u->cfg.max_batch) return ufail(LBM_ERR_INVALID, "batch outside 1..max_batch");
    if (!u->ds_count) return ufail(LBM_ERR_INVALID, "no dataset");
    const size_t hw = (size_t)u->cfg.height * u->cfg.width;
    const int oc = u->cfg.out_channels;
    for (int i = 0; i < batch; ++i) {
        if (idx[i] < 0 || idx[i] >= u->ds_count) return ufail(LBM_ERR_INVALID, "sample index out of range");
        cudaMemcpyAsync(u->x0.p + i * hw * 16, u->ds_in + (size_t)idx[i] * hw * 16, hw * 16 * sizeof(bf16),
                        cudaMemcpyDeviceToDevice, u->stream);
        cudaMemcpyAsync(u->tgt + i * hw * oc, u->ds_tgt + (size_t)idx[i] * hw * oc, hw * oc * sizeof(float),
                        cudaMemcpyDeviceToDevice, u->stream);
        cudaMemcpyAsync(u->wt + i * hw, u->ds_wt + (size_t)idx[i] * hw, hw * sizeof(float), cudaMemcpyDeviceToDevice,
                        u->stream);
    }
    return LBM_OK;
}

int finish(lbm_unet_s *u, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(u->stream);
    if (e != cudaSuccess) return ufail(LBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    if (u->tc_err) {
        int flag = 0;
        e = cudaMemcpy(&flag, u->tc_err, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return ufail(LBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
        if (flag) {
            cudaMemset(u->tc_err, 0, sizeof(int));
            return ufail(LBM_ERR_CUDA, std::string(what) + ": a tensor-core convolution's bounded wait gave up");
        }
    }
    return LBM_OK;
}

uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

extern "C" {

int lbm_unet_create(const lbm_unet_config *cfg, lbm_unet *out) {
    if (!cfg || !out) return ufail(LBM_ERR_INVALID, "null argument");
    *out = nullptr;
    const int NL = cfg->levels ? cfg->levels : 3;
    if (NL < 3 || NL > 5) return ufail(LBM_ERR_INVALID, "levels must be 3..5");
    const int mult = 1 << NL;
    if (cfg->height < mult || cfg->width < mult || cfg->height % mult || cfg->width % mult)
        return ufail(LBM_ERR_INVALID, "height and width must be positive multiples of 2^levels");
    if (cfg->in_channels < 1 || cfg->in_channels > 16 || cfg->out_channels < 1 || cfg->out_channels > 16)
        return ufail(LBM_ERR_INVALID, "in_channels and out_channels must be 1..16");
    if (cfg->max_batch < 1) return ufail(LBM_ERR_INVALID, "max_batch must be positive");
    // the elementwise kernels index 8-channel groups of a batch in 32 bits
    if ((long long)cfg->max_batch * cfg->height * cfg->width * 16 >= (1ll << 31))
        return ufail(LBM_ERR_INVALID, "max_batch x height x width must stay below 2^27 pixels");
    const int base = cfg->base_channels ? cfg->base_channels : 16, cap = cfg->max_channels ? cfg->max_channels : 64;
    if ((base != 16 && base != 32) || cap != 64)
        return ufail(LBM_ERR_INVALID, "base_channels must be 16 or 32 and max_channels 64");
    lbm_unet_s *u = new lbm_unet_s();
    u->cfg = *cfg;
    u->levels = NL;
    u->base = base;
    u->cap = cap;
    const char *tce = getenv("THESIS_UNET_TC");
    u->tc = !(tce && strcmp(tce, "0") == 0);
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&u->sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&u->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        int per_sm = 0;
        cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        u->smem_per_sm = per_sm > 0 ? (size_t)per_sm : (size_t)u->smem_optin;
        if (u->sms < 1) u->sms = 1;
    }
    if (cudaStreamCreateWithFlags(&u->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&u->e0) != cudaSuccess || cudaEventCreate(&u->e1) != cudaSuccess) {
        lbm_unet_destroy(u);
        return ufail(LBM_ERR_CUDA, "stream or event creation failed");
    }
    // layers (cin, cout, relu) in parameter order
    std::vector<std::array<int, 3>> spec;
    for (int l = 0; l < NL; ++l) {
        spec.push_back({l == 0 ? 16 : ch(u, l - 1), ch(u, l), 1});
        spec.push_back({ch(u, l), ch(u, l), 1});
    }
    spec.push_back({ch(u, NL - 1), ch(u, NL), 1});
    spec.push_back({ch(u, NL), ch(u, NL), 1});
    for (int l = NL - 1; l >= 0; --l) {
        spec.push_back({ch_up(u, l) + ch(u, l), ch(u, l), 1});
        spec.push_back({ch(u, l), ch_dec_b(u, l), 1});
    }
    spec.push_back({ch(u, 0), 16, 0});
    size_t off = 0;
    for (const auto &sp : spec) {
        Layer l;
        l.cin = sp[0];
        l.cout = sp[1];
        l.relu = sp[2];
        l.w_off = off;
        off += (size_t)9 * l.cin * l.cout;
        l.b_off = off;
        off += l.cout;
        u->L.push_back(l);
    }
    u->nparams = (long long)off;
    int rc = LBM_OK;
    rc = rc ? rc : alloc(u, (void **)&u->tc_err, sizeof(int));
    const size_t pb = sizeof(float) * off;
    rc = rc ? rc : alloc(u, (void **)&u->params, pb);
    rc = rc ? rc : alloc(u, (void **)&u->grad, pb);
    rc = rc ? rc : alloc(u, (void **)&u->adam_m, pb);
    rc = rc ? rc : alloc(u, (void **)&u->adam_v, pb);
    for (Layer &l : u->L) {
        rc = rc ? rc : alloc(u, (void **)&l.w, sizeof(bf16) * 9 * l.cin * l.cout);
        rc = rc ? rc : alloc(u, (void **)&l.wt, sizeof(bf16) * 9 * l.cin * l.cout);
    }
    for (auto *v : {&u->e_a, &u->cat, &u->p, &u->d_a, &u->d_b, &u->g_e_a, &u->g_cat, &u->g_p, &u->g_d_a, &u->g_d_b})
        v->resize(NL);
    rc = rc ? rc : make_act(u, u->x0, 16, 0);
    for (int l = 0; l < NL; ++l) {
        rc = rc ? rc : make_act(u, u->e_a[l], ch(u, l), l);
        rc = rc ? rc : make_act(u, u->cat[l], ch_up(u, l) + ch(u, l), l);
        rc = rc ? rc : make_act(u, u->p[l], ch(u, l), l + 1);
        rc = rc ? rc : make_act(u, u->d_a[l], ch(u, l), l);
        rc = rc ? rc : make_act(u, u->d_b[l], ch_dec_b(u, l), l);
        rc = rc ? rc : make_act(u, u->g_e_a[l], ch(u, l), l);
        rc = rc ? rc : make_act(u, u->g_cat[l], ch_up(u, l) + ch(u, l), l);
        rc = rc ? rc : make_act(u, u->g_p[l], ch(u, l), l + 1);
        rc = rc ? rc : make_act(u, u->g_d_a[l], ch(u, l), l);
        rc = rc ? rc : make_act(u, u->g_d_b[l], ch_dec_b(u, l), l);
    }
    rc = rc ? rc : make_act(u, u->ba, ch(u, NL), NL);
    rc = rc ? rc : make_act(u, u->bb, ch(u, NL), NL);
    rc = rc ? rc : make_act(u, u->g_ba, ch(u, NL), NL);
    rc = rc ? rc : make_act(u, u->g_bb, ch(u, NL), NL);
    const size_t np = (size_t)cfg->max_batch * cfg->height * cfg->width;
    rc = rc ? rc : alloc(u, (void **)&u->out32, np * 16 * sizeof(float));
    rc = rc ? rc : alloc(u, (void **)&u->dout, np * 16 * sizeof(bf16));
    // largest pre-activation gradient: the output layer's 16 channels at level
    // 0, or the widest level's channels (ch(l) on 4^-l of the pixels; base 32
    // puts 32 channels on level 0)
    size_t dpre_elems = np * 16;
    for (int l = 0; l <= NL; ++l)
        dpre_elems = std::max(dpre_elems, (size_t)ch(u, l) * cfg->max_batch * H_of(u, l) * W_of(u, l));
    rc = rc ? rc : alloc(u, (void **)&u->dpre, dpre_elems * sizeof(bf16));
    rc = rc ? rc : alloc(u, (void **)&u->fin, np * 16 * sizeof(float));
    rc = rc ? rc : alloc(u, (void **)&u->fout, np * 16 * sizeof(float));
    rc = rc ? rc : alloc(u, (void **)&u->tgt, np * 16 * sizeof(float));
    rc = rc ? rc : alloc(u, (void **)&u->wt, np * sizeof(float));
    rc = rc ? rc : alloc(u, (void **)&u->sums, 4 * sizeof(double));
    if (rc) {
        lbm_unet_destroy(u);
        return rc;
    }
    // He-normal initialisation over the real fan-in; padded input channels
    // and unused outputs start (and, without gradient, stay) at zero
    std::vector<float> p((size_t)off, 0.f);
    uint64_t s = cfg->seed * 0x2545F4914F6CDD1Dull + 1;
    for (int k = 0; k < (int)u->L.size(); ++k) {
        const Layer &l = u->L[k];
        const int cin_real = k == 0 ? cfg->in_channels : l.cin;
        const int cout_real = k == out_layer(u) ? cfg->out_channels : l.cout;
        const double sd = sqrt(2.0 / (9.0 * cin_real));
        for (int tap = 0; tap < 9; ++tap)
            for (int co = 0; co < l.cout; ++co)
                for (int ci = 0; ci < l.cin; ++ci) {
                    const double u1 = ((splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
                    const double u2 = ((splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
                    const double z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
                    if (ci < cin_real && co < cout_real)
                        p[l.w_off + ((size_t)tap * l.cout + co) * l.cin + ci] = (float)(sd * z);
                }
    }
    cudaMemcpyAsync(u->params, p.data(), pb, cudaMemcpyHostToDevice, u->stream);
    refresh_weights(u);
    rc = finish(u, "create");
    if (rc) {
        lbm_unet_destroy(u);
        return rc;
    }
    *out = u;
    return LBM_OK;
}

long long lbm_unet_param_count(lbm_unet u) { return u ? u->nparams : -1; }

int lbm_unet_get_params(lbm_unet u, float *params) {
    if (!u || !params) return ufail(LBM_ERR_INVALID, "null argument");
    cudaMemcpyAsync(params, u->params, sizeof(float) * u->nparams, cudaMemcpyDeviceToHost, u->stream);
    return finish(u, "get_params");
}

int lbm_unet_set_params(lbm_unet u, const float *params) {
    if (!u || !params) return ufail(LBM_ERR_INVALID, "null argument");
    cudaMemcpyAsync(u->params, params, sizeof(float) * u->nparams, cudaMemcpyHostToDevice, u->stream);
    cudaMemsetAsync(u->adam_m, 0, sizeof(float) * u->nparams, u->stream);
    cudaMemsetAsync(u->adam_v, 0, sizeof(float) * u->nparams, u->stream);
    u->adam_t = 0;
    refresh_weights(u);
    return finish(u, "set_params");
}

int lbm_unet_set_dataset(lbm_unet u, int count, const float *inputs, const float *targets, const float *weights) {
    if (!u || count < 1 || !inputs || !targets || !weights) return ufail(LBM_ERR_INVALID, "bad dataset arguments");
    const size_t hw = (size_t)u->cfg.height * u->cfg.width;
    const int ic = u->cfg.in_channels, oc = u->cfg.out_channels;
    cudaStreamSynchronize(u->stream);
    if (u->ds_in) cudaFree(u->ds_in);
    if (u->ds_tgt) cudaFree(u->ds_tgt);
    if (u->ds_wt) cudaFree(u->ds_wt);
    u->ds_in = nullptr;
    u->ds_tgt = u->ds_wt = nullptr;
    u->ds_count = 0;
    if (cudaMalloc((void **)&u->ds_in, (size_t)count * hw * 16 * sizeof(bf16)) != cudaSuccess ||
        cudaMalloc((void **)&u->ds_tgt, (size_t)count * hw * oc * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void **)&u->ds_wt, (size_t)count * hw * sizeof(float)) != cudaSuccess)
        return ufail(LBM_ERR_NOMEM, "dataset does not fit on the device");
    // inputs go through the float staging buffer, max_batch samples at a time
    for (int s0 = 0; s0 < count; s0 += u->cfg.max_batch) {
        const int k = count - s0 < u->cfg.max_batch ? count - s0 : u->cfg.max_batch;
        cudaMemcpyAsync(u->fin, inputs + (size_t)s0 * hw * ic, (size_t)k * hw * ic * sizeof(float),
                        cudaMemcpyHostToDevice, u->stream);
        pack_input_kernel<<<grid_for((long long)k * hw * 16), 256, 0, u->stream>>>(u->fin, ic, u->ds_in + (size_t)s0 * hw * 16,
                                                                                  (long long)k * hw);
        const int rc = finish(u, "set_dataset");
        if (rc) return rc;
    }
    cudaMemcpyAsync(u->ds_tgt, targets, (size_t)count * hw * oc * sizeof(float), cudaMemcpyHostToDevice, u->stream);
    cudaMemcpyAsync(u->ds_wt, weights, (size_t)count * hw * sizeof(float), cudaMemcpyHostToDevice, u->stream);
    const int rc = finish(u, "set_dataset");
    if (rc == LBM_OK) u->ds_count = count;
    return rc;
}

static int grad_pass(lbm_unet u, int batch, const int *idx, double *loss_out) {
    int rc = gather_batch(u, batch, idx);
    if (rc) return rc;
    cudaMemsetAsync(u->grad, 0, sizeof(float) * u->nparams, u->stream);
    forward(u, batch);
    loss(u, batch);
    backward(u, batch);
    if (loss_out) {
        double s[2];
        cudaMemcpyAsync(s, u->sums, sizeof(s), cudaMemcpyDeviceToHost, u->stream);
        rc = finish(u, "gradients");
        if (rc) return rc;
        *loss_out = s[1] > 0 ? s[0] / (u->cfg.out_channels * s[1]) : 0.0;
    }
    return LBM_OK;
}

int lbm_unet_train_step(lbm_unet u, int batch, const int *idx, float lr, double *loss_out) {
    if (!u || !idx) return ufail(LBM_ERR_INVALID, "null argument");
    cudaEventRecord(u->e0, u->stream);
    int rc = grad_pass(u, batch, idx, nullptr);
    if (rc) return rc;
    ++u->adam_t;
    const float c1 = (float)(1.0 / (1.0 - pow(0.9, (double)u->adam_t)));
    const float c2 = (float)(1.0 / (1.0 - pow(0.999, (double)u->adam_t)));
    adam_kernel<<<grid_for(u->nparams), 256, 0, u->stream>>>(u->params, u->grad, u->adam_m, u->adam_v, u->nparams, lr,
                                                              c1, c2);
    refresh_weights(u);
    cudaEventRecord(u->e1, u->stream);
    double s[2] = {0, 0};
    cudaMemcpyAsync(s, u->sums, sizeof(s), cudaMemcpyDeviceToHost, u->stream);
    rc = finish(u, "train_step");
    if (rc) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, u->e0, u->e1);
    u->last_ms = ms;
    const double l = s[1] > 0 ? s[0] / (u->cfg.out_channels * s[1]) : 0.0;
    if (loss_out) *loss_out = l;
    if (!isfinite(l)) return ufail(LBM_DIVERGED, "non-finite loss");
    return LBM_OK;
}

int lbm_unet_gradients(lbm_unet u, int batch, const int *idx, float *grad, double *loss_out) {
    if (!u || !idx || !grad) return ufail(LBM_ERR_INVALID, "null argument");
    int rc = grad_pass(u, batch, idx, loss_out);
    if (rc) return rc;
    cudaMemcpyAsync(grad, u->grad, sizeof(float) * u->nparams, cudaMemcpyDeviceToHost, u->stream);
    return finish(u, "gradients");
}

int lbm_unet_predict(lbm_unet u, int count, const float *inputs, float *outputs) {
    if (!u || !inputs || !outputs) return ufail(LBM_ERR_INVALID, "null argument");
    if (count < 1 || count > u->cfg.max_batch) return ufail(LBM_ERR_INVALID, "count outside 1..max_batch");
    const long long np = (long long)count * u->cfg.height * u->cfg.width;
    const int ic = u->cfg.in_channels, oc = u->cfg.out_channels;
    cudaMemcpyAsync(u->fin, inputs, sizeof(float) * np * ic, cudaMemcpyHostToDevice, u->stream);
    cudaEventRecord(u->e0, u->stream);
    pack_input_kernel<<<grid_for(np * 16), 256, 0, u->stream>>>(u->fin, ic, u->x0.p, np);
    forward(u, count);
    unpack_output_kernel<<<grid_for(np * oc), 256, 0, u->stream>>>(u->out32, 16, u->fout, oc, np);
    cudaEventRecord(u->e1, u->stream);
    cudaMemcpyAsync(outputs, u->fout, sizeof(float) * np * oc, cudaMemcpyDeviceToHost, u->stream);
    const int rc = finish(u, "predict");
    if (rc) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, u->e0, u->e1);
    u->last_ms = ms;
    return LBM_OK;
}

double lbm_unet_last_ms(lbm_unet u) { return u ? u->last_ms : -1.0; }

const char *lbm_unet_last_error(void) { return g_unet_error.c_str(); }

void lbm_unet_destroy(lbm_unet u) {
    if (!u) return;
    if (u->stream) cudaStreamSynchronize(u->stream);
    for (void *p : u->allocs) cudaFree(p);
    if (u->ds_in) cudaFree(u->ds_in);
    if (u->ds_tgt) cudaFree(u->ds_tgt);
    if (u->ds_wt) cudaFree(u->ds_wt);
    if (u->e0) cudaEventDestroy(u->e0);
    if (u->e1) cudaEventDestroy(u->e1);
    if (u->stream) cudaStreamDestroy(u->stream);
    delete u;
}

}  // extern "C"
