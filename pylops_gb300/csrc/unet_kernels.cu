// Memory-bound kernels of the U-Net image preconditioner; its convolutions
// run on the tcgen05 GEMM (gemm_tcgen05.cu).  Activations are NHWC (channel
// fastest).  A ks x ks convolution (ks = 1 or 3, zero padding ks/2, stride s)
//   y[b,ho,wo,co] = sum_{ky,kx,ci} W[co][(ky*ks+kx)*Cin+ci] x[b, ho*s+ky-pad, wo*s+kx-pad, ci]
// is lowered to three GEMMs:
//   forward          y    = col  . W^T      col  = unfold(x)        (P_out x Kpad)
//   weight gradient  dW   = g^T  . colT^T   colT = unfold(x)^T      (ks^2 Cin x P_out)
//   data gradient    dx   = gcol . Wt^T     gcol = unfold^T(g)      (P_in x Kg)
// where g = dy (.) relu'(y) and Wt[ci][(tap)*Cout+co] = W[co][tap*Cin+ci];
// unfold^T gathers, for every input pixel, the output-gradient pixels whose
// window covers it, so the data gradient is a plain GEMM (no scatter) and
// training is deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "kgb_internal.h"

namespace kgb {
namespace un {

typedef __nv_bfloat16 bf16;

int grid_for(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 16 * 152)); }

// two floats rounded to bf16 (round to nearest even), low half first
__device__ __forceinline__ uint32_t pack_bf16_pair(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Source pixel of destination pixel (hd, wd) for tap (ky, kx).  Forward
// unfold: hs = hd*s + ky - pad.  Transposed unfold: hd = hs*s + ky - pad.
template <bool TRANS>
__device__ __forceinline__ bool src_pixel(int hd, int wd, int ky, int kx, int s, int pad, int Hs, int Ws, int& hs,
                                          int& ws) {
    if (!TRANS) {
        hs = hd * s + ky - pad;
        ws = wd * s + kx - pad;
    } else {
        const int nh = hd + pad - ky, nw = wd + pad - kx;
        if (nh < 0 || nw < 0) return false;
        if (s == 2 && ((nh | nw) & 1)) return false;
        hs = s == 2 ? nh >> 1 : nh;
        ws = s == 2 ? nw >> 1 : nw;
    }
    return hs >= 0 && hs < Hs && ws >= 0 && ws < Ws;
}

// out[pd][(ky*ks+kx)*C + c] for pd over B x Hd x Wd, columns padded to Kpad.
// VEC: C % 8 == 0 and 8 channels (16 bytes) per thread.
template <bool TRANS, bool VEC, typename I>
__global__ void unfold_kernel(const bf16* __restrict__ src, bf16* __restrict__ out, int B, int Hs, int Ws, int C,
                              int Hd, int Wd, int ks, int s, int Kpad) {
    const int pad = ks >> 1;
    const int G = VEC ? 8 : 1;
    const I kunits = (I)(Kpad / G);
    const I total = (I)B * Hd * Wd * kunits;
    for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (I)gridDim.x * blockDim.x) {
        const int k = (int)(i % kunits) * G;
        const I p = i / kunits;
        const int wd = (int)(p % (I)Wd);
        const I t = p / (I)Wd;
        const int hd = (int)(t % (I)Hd);
        const int b = (int)(t / (I)Hd);
        const bf16* sp = nullptr;
        if (k < ks * ks * C) {
            const int tap = k / C, c = k - tap * C;
            const int ky = tap / ks, kx = tap - ky * ks;
            int hs, ws;
            if (src_pixel<TRANS>(hd, wd, ky, kx, s, pad, Hs, Ws, hs, ws))
                sp = src + (((int64_t)b * Hs + hs) * Ws + ws) * C + c;
        }
        if (VEC) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (sp) v = __ldg(reinterpret_cast<const uint4*>(sp));
            reinterpret_cast<uint4*>(out)[i] = v;
        } else {
            out[i] = sp ? sp[0] : __float2bfloat16(0.f);
        }
    }
}

// colT[(tap*C + c)][p] = x[pixel(p, tap), c]: 32 pixels x 32 channels per
// block through shared memory, coalesced on both sides.
__global__ void unfold_t_kernel(const bf16* __restrict__ x, bf16* __restrict__ colT, int B, int H, int W, int C,
                                int Ho, int Wo, int ks, int s, int64_t P) {
    __shared__ bf16 tile[32][34];
    const int pad = ks >> 1;
    const int64_t p0 = (int64_t)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    const int tap = blockIdx.z;
    const int ky = tap / ks, kx = tap - ky * ks;
    const int tx = threadIdx.x;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int64_t p = p0 + j;
        const int c = c0 + tx;
        bf16 v = __float2bfloat16(0.f);
        if (p < P && c < C) {
            const int wo = (int)(p % Wo);
            const int64_t t = p / Wo;
            const int ho = (int)(t % Ho);
            const int b = (int)(t / Ho);
            const int h = ho * s + ky - pad, w = wo * s + kx - pad;
            if (h >= 0 && h < H && w >= 0 && w < W) v = x[(((int64_t)b * H + h) * W + w) * C + c];
        }
        tile[j][tx] = v;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int c = c0 + j;
        const int64_t p = p0 + tx;
        if (c < C && p < P) colT[((int64_t)tap * C + c) * P + p] = tile[tx][j];
    }
}

// Vector form of unfold_t for C % 8 == 0 and P % 8 == 0: each thread moves
// an 8-pixel x 8-channel block of one tap (eight 16-byte loads, an 8 x 8
// transpose of 16-bit values in registers, eight 16-byte stores).
// Consecutive threads take the channel groups of consecutive pixel groups,
// so a warp's loads cover whole pixels and its stores runs of 8 pixels.
template <typename I>
__global__ void unfold_t_vec_kernel(const bf16* __restrict__ x, bf16* __restrict__ colT, int H, int W, int C, int Ho,
                                    int Wo, int ks, int s, int64_t P) {
    const int pad = ks >> 1;
    const I cgn = (I)(C >> 3);
    const I pgn = (I)(P >> 3);
    const I total = (I)(ks * ks) * cgn * pgn;
    // the 8 pixels of a group lie in one output row when Wo % 8 == 0
    const bool row8 = (Wo & 7) == 0;
    for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (I)gridDim.x * blockDim.x) {
        // channel group fastest: a warp loads whole pixels (contiguous
        // channel groups) and stores 8 runs of consecutive pixels per row
        const int cg = (int)(i % cgn);
        const I rest = i / cgn;
        const I pg = rest % pgn;
        const int tap = (int)(rest / pgn);
        const int ky = tap / ks, kx = tap - ky * ks;
        int wo0 = 0, ho0 = 0, b0 = 0;
        if (row8) {
            const I p0 = pg * 8;
            wo0 = (int)(p0 % (I)Wo);
            const I t = p0 / (I)Wo;
            ho0 = (int)(t % (I)Ho);
            b0 = (int)(t / (I)Ho);
        }
        uint32_t v[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            int wo = wo0 + j, ho = ho0, b = b0;
            if (!row8) {
                const I p = pg * 8 + j;
                wo = (int)(p % (I)Wo);
                const I t = p / (I)Wo;
                ho = (int)(t % (I)Ho);
                b = (int)(t / (I)Ho);
            }
            const int h = ho * s + ky - pad, w = wo * s + kx - pad;
            uint4 u = make_uint4(0, 0, 0, 0);
            if (h >= 0 && h < H && w >= 0 && w < W)
                u = __ldg(reinterpret_cast<const uint4*>(x + (((int64_t)b * H + h) * W + w) * C + cg * 8));
            v[j][0] = u.x;
            v[j][1] = u.y;
            v[j][2] = u.z;
            v[j][3] = u.w;
        }
        // channel k of pixel j is the (k & 1) half of word k >> 1 of v[j]
        bf16* dst = colT + ((int64_t)tap * C + cg * 8) * P + (int64_t)pg * 8;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t sel = (k & 1) ? 0x7632u : 0x5410u;  // high or low halves of two words
            uint4 o;
            o.x = __byte_perm(v[0][k >> 1], v[1][k >> 1], sel);
            o.y = __byte_perm(v[2][k >> 1], v[3][k >> 1], sel);
            o.z = __byte_perm(v[4][k >> 1], v[5][k >> 1], sel);
            o.w = __byte_perm(v[6][k >> 1], v[7][k >> 1], sel);
            *reinterpret_cast<uint4*>(dst + (int64_t)k * P) = o;
        }
    }
}

// unfold_t for narrow inputs (C < 32, where a 32 x 32 tile would leave
// most lanes idle): one thread per output element, pixels fastest.
template <typename I>
__global__ void unfold_t_small_kernel(const bf16* __restrict__ x, bf16* __restrict__ colT, int H, int W, int C, int Ho,
                                      int Wo, int ks, int s, int64_t P) {
    const int pad = ks >> 1;
    const I total = (I)(ks * ks * C) * (I)P;
    for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (I)gridDim.x * blockDim.x) {
        const I p = i % (I)P;
        const int k = (int)(i / (I)P);
        const int tap = k / C, c = k - tap * C;
        const int ky = tap / ks, kx = tap - ky * ks;
        const int wo = (int)(p % (I)Wo);
        const I t = p / (I)Wo;
        const int ho = (int)(t % (I)Ho);
        const int b = (int)(t / (I)Ho);
        const int h = ho * s + ky - pad, w = wo * s + kx - pad;
        colT[i] = (h >= 0 && h < H && w >= 0 && w < W) ? x[(((int64_t)b * H + h) * W + w) * C + c]
                                                       : __float2bfloat16(0.f);
    }
}

// Per-image-row transposes for the implicit weight gradient: for each of
// the R = B H image rows r, the W x C block src[r][w][c] (NHWC, C % 8 == 0)
// becomes dst[r][s][c][w] = src[r][w + s - 1][c] for s < 3 (shifts = 3:
// three copies shifted by -1, 0, +1 columns, zero outside the row, stacked
// per row so that the 3 C rows of one image row are contiguous) or
// dst[r][c][w] = src[r][w][c] (shifts = 1).  One block per (row, 64
// columns, 32 channels): the strip (with its one-column halo) is staged in
// shared memory by 16-byte loads along channels and written by 16-byte
// stores along columns.
__global__ void row_transpose_kernel(const bf16* __restrict__ src, bf16* __restrict__ dst, int64_t R, int W, int C,
                                     int shifts) {
    // channel-major staging [c - c0][w - (w0 + lo)], 33 words per row: the
    // scalar writes of the load phase and the reads of the store phase fall
    // in distinct banks across a warp
    __shared__ unsigned short tile[32][66];
    const int wb = (W + 63) / 64, cb = (C + 31) / 32;
    const int64_t items = R * wb * cb;
    const int lo = shifts == 3 ? -1 : 0;
    const int span = shifts == 3 ? 66 : 64;
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
        const int c0 = (int)(it % cb) * 32;
        const int64_t r1 = it / cb;
        const int w0 = (int)(r1 % wb) * 64;
        const int64_t r = r1 / wb;
        __syncthreads();
        // 8 channels (16 bytes) per load
        for (int e = threadIdx.x; e < span * 4; e += blockDim.x) {
            const int j = e >> 2, q = e & 3;
            const int w = w0 + lo + j, c = c0 + 8 * q;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (w >= 0 && w < W && c < C) v = __ldg(s4 + ((r * W + w) * C + c) / 8);
            const uint32_t wd[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int i = 0; i < 8; ++i) tile[8 * q + i][j] = (unsigned short)(wd[i >> 1] >> (16 * (i & 1)));
        }
        __syncthreads();
        // 8 columns (16 bytes) per store; a warp writes 4 channels x 64
        // columns, i.e. four whole 128-byte row segments
        for (int e = threadIdx.x; e < shifts * 32 * 8; e += blockDim.x) {
            const int w8 = e & 7, cc = (e >> 3) & 31, sh = e >> 8;
            const int c = c0 + cc, w = w0 + 8 * w8;
            if (c >= C || w >= W) continue;
            // staged column of output column w + k: (w + k + sh - 1) - (w0 - 1) = 8 w8 + k + sh
            // (shifts = 3), (w + k) - w0 = 8 w8 + k (shifts = 1); W % 8 == 0, so w + 8 <= W
            const unsigned short* t = &tile[cc][shifts == 3 ? 8 * w8 + sh : 8 * w8];
            uint4 o;
            o.x = (uint32_t)t[0] | ((uint32_t)t[1] << 16);
            o.y = (uint32_t)t[2] | ((uint32_t)t[3] << 16);
            o.z = (uint32_t)t[4] | ((uint32_t)t[5] << 16);
            o.w = (uint32_t)t[6] | ((uint32_t)t[7] << 16);
            *reinterpret_cast<uint4*>(dst + ((r * shifts + sh) * C + c) * W + w) = o;
        }
    }
}

// Column sums of a bf16 matrix g (rows x cols, cols % 8 == 0, cols <= 256),
// each row optionally weighted by wt[r] (bf16): the bias gradient straight
// from the NHWC output gradient, or (weighted) the weight gradient of a 1x1
// convolution to one channel.  Block k sums
// rows [k chunk, (k + 1) chunk): thread (phase, column group) adds 8
// columns (one 16-byte load) of rows r0 + phase, r0 + phase + nph, ... in
// order; the phases are added in order into work[k][c], and colsum_final
// adds the blocks in order, so the sums are deterministic.
constexpr int kColChunks = 1024;
__device__ __forceinline__ float bf16_bits(uint32_t h) { return __uint_as_float(h << 16); }

__global__ void __launch_bounds__(256) colsum_partial_kernel(const bf16* __restrict__ g, const bf16* __restrict__ wt,
                                                             float* __restrict__ work, int64_t rows, int cols) {
    __shared__ float part[8 * 256];
    const int ng = cols >> 3;                 // 16-byte column groups
    const int nph = blockDim.x / ng;          // row phases
    const int ph = threadIdx.x / ng, cg = threadIdx.x - ph * ng;
    const int64_t chunk = (rows + kColChunks - 1) / kColChunks;
    const int64_t r0 = (int64_t)blockIdx.x * chunk, r1 = min(rows, r0 + chunk);
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (ph < nph) {
        for (int64_t rr = r0 + ph; rr < r1; rr += nph) {
            const uint4 u = __ldg(reinterpret_cast<const uint4*>(g + rr * cols) + cg);
            const uint32_t wd[4] = {u.x, u.y, u.z, u.w};
            const float f = wt ? __bfloat162float(wt[rr]) : 1.f;
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[i] += f * bf16_bits((wd[i >> 1] >> (16 * (i & 1))) & 0xffffu);
        }
        for (int i = 0; i < 8; ++i) part[ph * cols + cg * 8 + i] = acc[i];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < cols; c += blockDim.x) {
        float sum = 0.f;
        for (int k = 0; k < nph; ++k) sum += part[k * cols + c];
        work[(int64_t)blockIdx.x * cols + c] = sum;
    }
}

// one warp per column: lane l adds blocks l, l + 32, ... in order, then a
// fixed butterfly over the lanes
__global__ void colsum_final_kernel(const float* __restrict__ work, float* __restrict__ out, int cols) {
    const int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (c >= cols) return;
    float acc = 0.f;
    for (int k = lane; k < kColChunks; k += 32) acc += work[(int64_t)k * cols + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) out[c] = acc;
}

// 1x1 convolution to one channel (the network's head): y[p] = b + sum_c
// w[c] x[p][c], x NHWC bf16 with C % 8 == 0, w bf16, fp32 accumulation.
__global__ void head_forward_kernel(const uint4* __restrict__ x, const bf16* __restrict__ w, const float* __restrict__ b,
                                    float* __restrict__ y, int64_t P, int C) {
    __shared__ float wsh[256];
    for (int c = threadIdx.x; c < C; c += blockDim.x) wsh[c] = __bfloat162float(w[c]);
    __syncthreads();
    const float bias = b ? b[0] : 0.f;
    const int G = C >> 3;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (int gI = 0; gI < G; ++gI) {
            const uint4 u = __ldg(x + p * G + gI);
            const uint32_t wd[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int i = 0; i < 8; ++i) acc += wsh[8 * gI + i] * bf16_bits((wd[i >> 1] >> (16 * (i & 1))) & 0xffffu);
        }
        y[p] = acc + bias;
    }
}

// Its data gradient: dx[p][c] = g[p] w[c] (float32), 4 channels per thread.
__global__ void head_dx_kernel(const bf16* __restrict__ g, const bf16* __restrict__ w, float4* __restrict__ dx,
                               int64_t P, int C) {
    __shared__ float wsh[256];
    for (int c = threadIdx.x; c < C; c += blockDim.x) wsh[c] = __bfloat162float(w[c]);
    __syncthreads();
    const int Q = C >> 2;
    const int64_t total = P * Q;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = i / Q;
        const int q = (int)(i - p * Q);
        const float gv = __bfloat162float(g[p]);
        dx[i] = make_float4(gv * wsh[4 * q], gv * wsh[4 * q + 1], gv * wsh[4 * q + 2], gv * wsh[4 * q + 3]);
    }
}

// 3x3 convolution of a one-channel image (the network's first layer), zero
// padding 1: y[p][n] = act(b[n] + sum_t w[n][t] x[p + off(t)]) as bf16, w
// bf16 with row stride kpad (tap t = 3 ky + kx), N % 8 == 0, N <= 128;
// fp32 accumulation, one pixel and 8 output channels per thread.
__global__ void conv_c1_kernel(const bf16* __restrict__ x, const bf16* __restrict__ w, const float* __restrict__ b,
                               uint4* __restrict__ y, int B, int H, int W, int N, int kpad, int relu) {
    // tap-major weights: the 8 output channels of one tap are two 16-byte loads
    __shared__ __align__(16) float wsh[9 * 128];
    __shared__ float bsh[128];
    for (int k = threadIdx.x; k < N * 9; k += blockDim.x)
        wsh[(k % 9) * 128 + k / 9] = __bfloat162float(w[(k / 9) * kpad + k % 9]);
    for (int k = threadIdx.x; k < N; k += blockDim.x) bsh[k] = b ? b[k] : 0.f;
    __syncthreads();
    // thread = (pixel, group of 8 output channels): consecutive threads
    // write consecutive 16-byte pieces of the NHWC output
    const int G = N >> 3;
    const int64_t T = (int64_t)B * H * W * G;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < T; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = i / G;
        const int n8 = (int)(i - p * G) * 8;
        const int wi = (int)(p % W);
        const int hi = (int)((p / W) % H);
        float v[9];
#pragma unroll
        for (int ky = 0; ky < 3; ++ky)
#pragma unroll
            for (int kx = 0; kx < 3; ++kx) {
                const int hh = hi + ky - 1, ww = wi + kx - 1;
                v[ky * 3 + kx] = (hh >= 0 && hh < H && ww >= 0 && ww < W)
                                     ? __bfloat162float(x[p + (int64_t)(ky - 1) * W + (kx - 1)])
                                     : 0.f;
            }
        float o[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) o[j] = bsh[n8 + j];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const float4 a = *reinterpret_cast<const float4*>(wsh + k * 128 + n8);
            const float4 c = *reinterpret_cast<const float4*>(wsh + k * 128 + n8 + 4);
            o[0] += a.x * v[k];
            o[1] += a.y * v[k];
            o[2] += a.z * v[k];
            o[3] += a.w * v[k];
            o[4] += c.x * v[k];
            o[5] += c.y * v[k];
            o[6] += c.z * v[k];
            o[7] += c.w * v[k];
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) o[j] = relu ? fmaxf(o[j], 0.f) : o[j];
        uint4 u;
        u.x = pack_bf16_pair(o[0], o[1]);
        u.y = pack_bf16_pair(o[2], o[3]);
        u.z = pack_bf16_pair(o[4], o[5]);
        u.w = pack_bf16_pair(o[6], o[7]);
        y[i] = u;
    }
}

// Its weight gradient: dW[n][t] = sum_p g[p][n] x[p + off(t)].  Block k
// takes image rows [k rpb, (k + 1) rpb); warp w of the block the rows k rpb
// + w, + 4, ...; lane l the output channels l, l + 32, ... (N <= 128) with
// nine tap accumulators each, walking the row kC1Span pixels at a time (the
// span's gradient values and its 3 x (kC1Span + 2) window of x loaded
// together, so the loads of a warp overlap).  The warps' sums are added in
// warp order into work[k][n * 9 + t];
// conv_c1_wgrad_final adds the blocks in a fixed order (warp per output).
constexpr int kC1Warps = 4;
constexpr int kC1Span = 8;  // pixels of a row whose loads are issued together
__global__ void __launch_bounds__(32 * kC1Warps) conv_c1_wgrad_partial_kernel(const bf16* __restrict__ x,
                                                                             const bf16* __restrict__ g,
                                                                             float* __restrict__ work, int B, int H,
                                                                             int W, int N) {
    __shared__ float red[kC1Warps][128 * 9];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t R = (int64_t)B * H;
    const int64_t rpb = (R + kColChunks - 1) / kColChunks;
    const int64_t r0 = (int64_t)blockIdx.x * rpb, r1 = min(R, r0 + rpb);
    const int ng = (N + 31) / 32;  // channel groups per lane (N <= 128)
    float acc[4][9];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int t = 0; t < 9; ++t) acc[q][t] = 0.f;
    for (int64_t r = r0 + warp; r < r1; r += kC1Warps) {
        const int h = (int)(r % H);
        const bf16* xr = x + r * W;  // row h of image r / H
        const bool up = h > 0, dn = h + 1 < H;
        auto xv = [&](int dy, int w) -> float {
            if (w < 0 || w >= W || (dy < 0 && !up) || (dy > 0 && !dn)) return 0.f;
            return __bfloat162float(xr[(int64_t)dy * W + w]);
        };
        // kC1Span pixels at a time: their gradients and the input window
        // xw[dy][c] = x at (h + dy - 1, w0 + c - 1) are loaded together
        // (independent loads in flight), then summed pixel by pixel
        for (int w0 = 0; w0 < W; w0 += kC1Span) {
            float gv[4][kC1Span];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int n = lane + 32 * q;
#pragma unroll
                for (int j = 0; j < kC1Span; ++j)
                    gv[q][j] = (q < ng && n < N && w0 + j < W) ? __bfloat162float(g[(r * W + w0 + j) * N + n]) : 0.f;
            }
            float xw[3][kC1Span + 2];
#pragma unroll
            for (int dy = 0; dy < 3; ++dy)
#pragma unroll
                for (int c = 0; c < kC1Span + 2; ++c) xw[dy][c] = xv(dy - 1, w0 + c - 1);
#pragma unroll
            for (int j = 0; j < kC1Span; ++j)
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (q < ng)
#pragma unroll
                        for (int dy = 0; dy < 3; ++dy)
#pragma unroll
                            for (int dx = 0; dx < 3; ++dx) acc[q][dy * 3 + dx] += gv[q][j] * xw[dy][j + dx];
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int n = lane + 32 * q;
        if (q < ng && n < N)
#pragma unroll
            for (int t = 0; t < 9; ++t) red[warp][n * 9 + t] = acc[q][t];
    }
    __syncthreads();
    for (int o = threadIdx.x; o < 9 * N; o += blockDim.x) {
        float sum = 0.f;
        for (int k = 0; k < kC1Warps; ++k) sum += red[k][o];
        work[(int64_t)blockIdx.x * 9 * N + o] = sum;
    }
}

// The same weight gradient, pixel-parallel: lane (slot, cg) of a warp takes
// output channels 8 cg .. 8 cg + 7 (one 16-byte load of g) of pixel slot of
// each group of 32 / G consecutive pixels (G = N / 8 lanes per pixel, so a
// warp reads 512 contiguous bytes per load), two groups per step.  Each
// lane sums its pixels in order, the slots sharing a channel group are
// combined by a fixed xor-shuffle tree, the warps in warp order into
// work[k][n * 9 + t].  Block k takes pixels [k ppb, (k + 1) ppb).
template <int G>
__global__ void __launch_bounds__(256) conv_c1_wgrad_px_kernel(const bf16* __restrict__ x, const uint4* __restrict__ g,
                                                               float* __restrict__ work, int B, int H, int W) {
    constexpr int PPW = 32 / G;  // pixels per warp and group
    constexpr int NW = 8;        // warps per block
    __shared__ float red[NW][9 * 8 * G];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int slot = lane / G, cg = lane - slot * G;
    const int64_t P = (int64_t)B * H * W;
    const int64_t ppb = (P + kColChunks - 1) / kColChunks;
    const int64_t p0 = (int64_t)blockIdx.x * ppb, p1 = min(P, p0 + ppb);
    float acc[8][9];
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int t = 0; t < 9; ++t) acc[j][t] = 0.f;
    constexpr int64_t kStep = (int64_t)NW * PPW;
    for (int64_t pb = p0 + warp * PPW + slot; pb < p1; pb += 2 * kStep) {
        uint4 gv[2];
        float xv[2][9];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int64_t p = pb + u * kStep;
            const bool in = p < p1;
            gv[u] = in ? __ldg(g + p * G + cg) : make_uint4(0u, 0u, 0u, 0u);
            const int w = in ? (int)(p % W) : 0;
            const int h = in ? (int)((p / W) % H) : 0;
#pragma unroll
            for (int dy = 0; dy < 3; ++dy)
#pragma unroll
                for (int dx = 0; dx < 3; ++dx) {
                    const int hh = h + dy - 1, ww = w + dx - 1;
                    xv[u][dy * 3 + dx] = (in && hh >= 0 && hh < H && ww >= 0 && ww < W)
                                             ? __bfloat162float(x[p + (int64_t)(dy - 1) * W + (dx - 1)])
                                             : 0.f;
                }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const uint32_t wd[4] = {gv[u].x, gv[u].y, gv[u].z, gv[u].w};
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float gf = __uint_as_float((wd[j >> 1] >> (16 * (j & 1))) << 16);
#pragma unroll
                for (int t = 0; t < 9; ++t) acc[j][t] += gf * xv[u][t];
            }
        }
    }
#pragma unroll
    for (int off = G; off < 32; off <<= 1)
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
            for (int t = 0; t < 9; ++t) acc[j][t] += __shfl_xor_sync(0xffffffffu, acc[j][t], off);
    if (slot == 0)
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
            for (int t = 0; t < 9; ++t) red[warp][(cg * 8 + j) * 9 + t] = acc[j][t];
    __syncthreads();
    for (int o = threadIdx.x; o < 9 * 8 * G; o += blockDim.x) {
        float sum = 0.f;
        for (int k = 0; k < NW; ++k) sum += red[k][o];
        work[(int64_t)blockIdx.x * 9 * 8 * G + o] = sum;
    }
}

__global__ void conv_c1_wgrad_final_kernel(const float* __restrict__ work, float* __restrict__ dW, int N, int kpad) {
    const int o = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (o >= 9 * N) return;
    float acc = 0.f;
    for (int k = lane; k < kColChunks; k += 32) acc += work[(int64_t)k * 9 * N + o];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (lane == 0) dW[(o / 9) * kpad + o % 9] = acc;
}

// out[c][r] = in[r][c]; rows x cols, in leading dimension ldi, out ldo.
template <typename TI, typename TO>
__global__ void transpose_kernel(const TI* __restrict__ in, TO* __restrict__ out, int64_t rows, int cols, int64_t ldi,
                                 int64_t ldo) {
    __shared__ float tile[32][33];
    const int64_t r0 = (int64_t)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int64_t r = r0 + j;
        const int c = c0 + threadIdx.x;
        tile[j][threadIdx.x] = (r < rows && c < cols) ? (float)in[r * ldi + c] : 0.f;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int c = c0 + j;
        const int64_t r = r0 + threadIdx.x;
        if (c < cols && r < rows) out[(int64_t)c * ldo + r] = (TO)tile[threadIdx.x][j];
    }
}

// bf16 weights for the forward (W, Cout x Kpad) and data-gradient (Wt,
// Cin x Kg) GEMMs from the float32 master weights.
__global__ void weights_kernel(const float* __restrict__ Wm, bf16* __restrict__ Wb, bf16* __restrict__ Wt, int Cout,
                               int Cin, int taps, int Kpad, int Kg) {
    const int64_t nW = (int64_t)Cout * Kpad, nT = Wt ? (int64_t)Cin * Kg : 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nW + nT; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < nW) {
            Wb[i] = __float2bfloat16(Wm[i]);
        } else {
            const int64_t j = i - nW;
            const int ci = (int)(j / Kg), q = (int)(j % Kg);
            float v = 0.f;
            if (q < taps * Cout) {
                const int tap = q / Cout, co = q - tap * Cout;
                v = Wm[(int64_t)co * Kpad + tap * Cin + ci];
            }
            Wt[j] = __float2bfloat16(v);
        }
    }
}

// bf16 weights of the implicit 3x3 convolutions: Wi (Cout x 9*Cpi) for the
// forward and Wti (Cin x 9*Cpo) for the data gradient, channel blocks
// padded to 64 (Cpi, Cpo) with zeros.
__global__ void weights_implicit_kernel(const float* __restrict__ Wm, bf16* __restrict__ Wi, bf16* __restrict__ Wti,
                                        int Cout, int Cin, int Kpad, int Cpi, int Cpo) {
    const int64_t nI = (int64_t)Cout * 9 * Cpi, nT = Wti ? (int64_t)Cin * 9 * Cpo : 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nI + nT; i += (int64_t)gridDim.x * blockDim.x) {
        float v = 0.f;
        if (i < nI) {
            const int co = (int)(i / (9 * Cpi));
            const int q = (int)(i - (int64_t)co * 9 * Cpi);
            const int tap = q / Cpi, c = q - tap * Cpi;
            if (c < Cin) v = Wm[(int64_t)co * Kpad + tap * Cin + c];
            Wi[i] = __float2bfloat16(v);
        } else {
            const int64_t j = i - nI;
            const int ci = (int)(j / (9 * Cpo));
            const int q = (int)(j - (int64_t)ci * 9 * Cpo);
            const int tap = q / Cpo, co = q - tap * Cpo;
            if (co < Cout) v = Wm[(int64_t)co * Kpad + tap * Cin + ci];
            Wti[j] = __float2bfloat16(v);
        }
    }
}

// vector form (n % 8 == 0, 16-byte aligned): 8 elements per iteration
__global__ void relu_grad_vec_kernel(const float4* __restrict__ dy, const uint4* __restrict__ y, uint4* __restrict__ g,
                                     int64_t n8, int relu) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = __ldg(dy + 2 * i), b = __ldg(dy + 2 * i + 1);
        float v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        if (relu) {
            const uint4 u = __ldg(y + i);
            const uint32_t wd[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (!(__uint_as_float((wd[k >> 1] >> (16 * (k & 1))) << 16) > 0.f)) v[k] = 0.f;
        }
        uint4 o;
        o.x = pack_bf16_pair(v[0], v[1]);
        o.y = pack_bf16_pair(v[2], v[3]);
        o.z = pack_bf16_pair(v[4], v[5]);
        o.w = pack_bf16_pair(v[6], v[7]);
        g[i] = o;
    }
}

// g = dy (.) (y > 0)  (relu) or dy, rounded to bf16
__global__ void relu_grad_kernel(const float* __restrict__ dy, const bf16* __restrict__ y, bf16* __restrict__ g,
                                 int64_t n, int relu) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float v = dy[i];
        if (relu && !(__bfloat162float(y[i]) > 0.f)) v = 0.f;
        g[i] = __float2bfloat16(v);
    }
}

// Row sums of a bf16 matrix (bias gradients from g^T) in two passes with a
// fixed order: block (r, k) sums chunk k of row r into work[r][k], then one
// thread per row adds the chunks in order.
constexpr int kRowChunks = 64;
__global__ void rowsum_partial_kernel(const bf16* __restrict__ in, float* __restrict__ work, int64_t cols) {
    const int r = blockIdx.x, k = blockIdx.y;
    const int64_t chunk = (cols + kRowChunks - 1) / kRowChunks;
    const int64_t c0 = (int64_t)k * chunk, c1 = min(cols, c0 + chunk);
    const bf16* row = in + (int64_t)r * cols;
    float acc = 0.f;
    for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) acc += __bfloat162float(row[c]);
    __shared__ float sh[256];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) work[r * kRowChunks + k] = sh[0];
}

__global__ void rowsum_final_kernel(const float* __restrict__ work, float* __restrict__ out, int rows) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    float acc = 0.f;
    for (int k = 0; k < kRowChunks; ++k) acc += work[r * kRowChunks + k];
    out[r] = acc;
}

// nearest x2 upsampling of x (B x H x W x C) into channels [coff, coff+C)
// of y (B x 2H x 2W x Ctot)
__global__ void upsample_kernel(const bf16* __restrict__ x, bf16* __restrict__ y, int B, int H, int W, int C, int Ctot,
                                int coff) {
    const int64_t total = (int64_t)B * 2 * H * 2 * W * C;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        int64_t t = i / C;
        const int w = (int)(t % (2 * W));
        t /= 2 * W;
        const int h = (int)(t % (2 * H));
        const int b = (int)(t / (2 * H));
        y[(((int64_t)b * 2 * H + h) * 2 * W + w) * Ctot + coff + c] = x[(((int64_t)b * H + h / 2) * W + w / 2) * C + c];
    }
}

// vector form (C, Ctot, coff multiples of 8, 16-byte aligned): 8 channels
// (16 bytes) per thread
template <typename I>
__global__ void upsample_vec_kernel(const uint4* __restrict__ x, uint4* __restrict__ y, int B, int H, int W, int C8,
                                    int Ctot8, int coff8) {
    const I total = (I)B * 2 * H * 2 * W * C8;
    for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (I)gridDim.x * blockDim.x) {
        const int c = (int)(i % (I)C8);
        I t = i / (I)C8;
        const int w = (int)(t % (I)(2 * W));
        t /= (I)(2 * W);
        const int h = (int)(t % (I)(2 * H));
        const int b = (int)(t / (I)(2 * H));
        y[(((int64_t)b * 2 * H + h) * 2 * W + w) * Ctot8 + coff8 + c] =
            __ldg(x + (((int64_t)b * H + h / 2) * W + w / 2) * C8 + c);
    }
}

// its gradient: dx[b,h,w,c] = sum of the 2x2 block of dy[..., coff + c]
template <typename I>
__global__ void upsample_grad_kernel(const float* __restrict__ dy, float* __restrict__ dx, int B, int H, int W, int C,
                                     int Ctot, int coff) {
    const I total = (I)B * H * W * C;
    for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (I)gridDim.x * blockDim.x) {
        const int c = (int)(i % (I)C);
        I t = i / (I)C;
        const int w = (int)(t % (I)W);
        t /= (I)W;
        const int h = (int)(t % (I)H);
        const int b = (int)(t / (I)H);
        const int64_t r0 = (((int64_t)b * 2 * H + 2 * h) * 2 * W + 2 * w) * Ctot + coff + c;
        const int64_t rs = (int64_t)2 * W * Ctot;
        dx[i] = (dy[r0] + dy[r0 + Ctot]) + (dy[r0 + rs] + dy[r0 + rs + Ctot]);
    }
}

// y[p][coff + c] = x[p][c]  (skip connection into the concatenation)
template <typename I>
__global__ void put_channels_kernel(const bf16* __restrict__ x, bf16* __restrict__ y, int64_t P, int C, int Ctot,
                                    int coff) {
    const I total = (I)P * (I)C;
    for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (I)gridDim.x * blockDim.x)
        y[(int64_t)(i / (I)C) * Ctot + coff + (int)(i % (I)C)] = x[i];
}

// y[p][c] (+)= x[p][coff + c]  (gradient of the skip connection)
template <typename I>
__global__ void take_channels_kernel(const float* __restrict__ x, float* __restrict__ y, int64_t P, int C, int Ctot,
                                     int coff, int accumulate) {
    const I total = (I)P * (I)C;
    for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (I)gridDim.x * blockDim.x) {
        const float v = x[(int64_t)(i / (I)C) * Ctot + coff + (int)(i % (I)C)];
        y[i] = accumulate ? y[i] + v : v;
    }
}

// x (float, B images of n values) * per-image scale -> bf16 (NHWC with C = 1)
__global__ void to_bf16_kernel(const float* __restrict__ x, bf16* __restrict__ y, int64_t n, int B,
                               const float* __restrict__ scale) {
    const int64_t total = n * B;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16(x[i] * (scale ? scale[i / n] : 1.f));
}

// Mean-squared error: grad = 2 (y - t) / n, per-block partial sums of
// (y - t)^2 in double, then one thread sums them in order.
constexpr int kMseBlocks = 304;
__global__ void mse_kernel(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ grad,
                           int64_t n, double* __restrict__ partials) {
    double acc = 0.0;
    const float sc = 2.f / (float)n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float d = y[i] - t[i];
        acc += (double)d * d;
        if (grad) grad[i] = sc * d;
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

__global__ void mse_final_kernel(const double* __restrict__ partials, int np, int64_t n, double* __restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < np; ++i) s += partials[i];
        out[0] = s / (double)n;
    }
}

// scale[b] = 1 / sqrt(mean over image b of x^2) (0 for an all-zero image);
// one block per image, fixed reduction order.  Each thread keeps a
// compensated (Kahan) float32 sum of its strided elements -- the float64
// pipe of this GPU runs at 1/64 of the float32 rate -- and the block adds
// the 512 per-thread sums in float64.
__global__ void image_rms_kernel(const float* __restrict__ x, int64_t n, float* __restrict__ scale) {
    const float* xb = x + (int64_t)blockIdx.x * n;
    float sum = 0.f, comp = 0.f;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const float v = xb[i];
        const float y = __fmul_rn(v, v) - comp;
        const float t = __fadd_rn(sum, y);
        comp = __fsub_rn(__fsub_rn(t, sum), y);
        sum = t;
    }
    __shared__ double sh[512];
    sh[threadIdx.x] = (double)sum - (double)comp;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) scale[blockIdx.x] = sh[0] > 0.0 ? (float)(1.0 / sqrt(sh[0] / (double)n)) : 0.f;
}

// Adam on float32 master weights (bias-corrected moments)
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

}  // namespace un
}  // namespace kgb

using namespace kgb;
using namespace kgb::un;

extern "C" {

int kgb_unet_unfold(const void* src, void* out, int B, int Hs, int Ws, int C, int Hd, int Wd, int ks, int stride,
                    int transposed, int Kpad, void* stream) {
    if (!src || !out || B <= 0 || Hs <= 0 || Ws <= 0 || C <= 0 || Hd <= 0 || Wd <= 0 || (ks != 1 && ks != 3) ||
        (stride != 1 && stride != 2) || Kpad < ks * ks * C || Kpad % 8)
        return set_error(KGB_ERR_VALUE, "unet_unfold: bad arguments");
    const bool vec = C % 8 == 0 && ((uintptr_t)src & 15) == 0 && ((uintptr_t)out & 15) == 0;
    const int64_t n = (int64_t)B * Hd * Wd * (vec ? Kpad / 8 : Kpad);
    cudaStream_t s = (cudaStream_t)stream;
    const bf16* x = (const bf16*)src;
    bf16* y = (bf16*)out;
    // 32-bit index arithmetic whenever the element count allows it
    const bool i32 = n < (int64_t)1 << 31;
#define KGB_UNFOLD(T, V)                                                                                    \
    (i32 ? unfold_kernel<T, V, uint32_t><<<grid_for(n), 256, 0, s>>>(x, y, B, Hs, Ws, C, Hd, Wd, ks, stride, Kpad) \
         : unfold_kernel<T, V, int64_t><<<grid_for(n), 256, 0, s>>>(x, y, B, Hs, Ws, C, Hd, Wd, ks, stride, Kpad))
    if (transposed) {
        if (vec) KGB_UNFOLD(true, true);
        else KGB_UNFOLD(true, false);
    } else {
        if (vec) KGB_UNFOLD(false, true);
        else KGB_UNFOLD(false, false);
    }
#undef KGB_UNFOLD
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_unfold_t(const void* x, void* colT, int B, int H, int W, int C, int ks, int stride, void* stream) {
    if (!x || !colT || B <= 0 || H <= 0 || W <= 0 || C <= 0 || (ks != 1 && ks != 3) || (stride != 1 && stride != 2))
        return set_error(KGB_ERR_VALUE, "unet_unfold_t: bad arguments");
    const int pad = ks >> 1;
    const int Ho = (H + 2 * pad - ks) / stride + 1, Wo = (W + 2 * pad - ks) / stride + 1;
    const int64_t P = (int64_t)B * Ho * Wo;
    if ((P + 31) / 32 > 0x7fffffffLL) return set_error(KGB_ERR_VALUE, "unet_unfold_t: too many pixels");
    if (C % 8 == 0 && P % 8 == 0 && ((uintptr_t)x & 15) == 0 && ((uintptr_t)colT & 15) == 0) {
        const int64_t n = (int64_t)ks * ks * (C / 8) * (P / 8);
        if (n < (int64_t)1 << 31)
            unfold_t_vec_kernel<uint32_t><<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((const bf16*)x, (bf16*)colT, H,
                                                                                        W, C, Ho, Wo, ks, stride, P);
        else
            unfold_t_vec_kernel<int64_t><<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((const bf16*)x, (bf16*)colT, H,
                                                                                       W, C, Ho, Wo, ks, stride, P);
    } else if (C < 32) {
        const int64_t n = (int64_t)ks * ks * C * P;
        if (n < (int64_t)1 << 31)
            unfold_t_small_kernel<uint32_t><<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(
                (const bf16*)x, (bf16*)colT, H, W, C, Ho, Wo, ks, stride, P);
        else
            unfold_t_small_kernel<int64_t><<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(
                (const bf16*)x, (bf16*)colT, H, W, C, Ho, Wo, ks, stride, P);
    } else {
        dim3 grid((unsigned)((P + 31) / 32), (unsigned)((C + 31) / 32), (unsigned)(ks * ks)), block(32, 8);
        unfold_t_kernel<<<grid, block, 0, (cudaStream_t)stream>>>((const bf16*)x, (bf16*)colT, B, H, W, C, Ho, Wo,
                                                                  ks, stride, P);
    }
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

// kind: 0 bf16 -> bf16, 1 float -> float
int kgb_unet_transpose(const void* in, void* out, int64_t rows, int cols, int64_t ldi, int64_t ldo, int kind,
                       void* stream) {
    if (!in || !out || rows <= 0 || cols <= 0 || ldi < cols || ldo < rows || (kind != 0 && kind != 1))
        return set_error(KGB_ERR_VALUE, "unet_transpose: bad arguments");
    if ((rows + 31) / 32 > 0x7fffffffLL) return set_error(KGB_ERR_VALUE, "unet_transpose: too many rows");
    dim3 grid((unsigned)((rows + 31) / 32), (unsigned)((cols + 31) / 32)), block(32, 8);
    cudaStream_t s = (cudaStream_t)stream;
    if (kind == 0)
        transpose_kernel<bf16, bf16><<<grid, block, 0, s>>>((const bf16*)in, (bf16*)out, rows, cols, ldi, ldo);
    else
        transpose_kernel<float, float><<<grid, block, 0, s>>>((const float*)in, (float*)out, rows, cols, ldi, ldo);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_weights(const float* Wm, void* Wb, void* Wt, int Cout, int Cin, int ks, int Kpad, int Kg, void* stream) {
    if (!Wm || !Wb || Cout <= 0 || Cin <= 0 || (ks != 1 && ks != 3) || Kpad < ks * ks * Cin ||
        (Wt && Kg < ks * ks * Cout))
        return set_error(KGB_ERR_VALUE, "unet_weights: bad arguments");
    const int64_t n = (int64_t)Cout * Kpad + (Wt ? (int64_t)Cin * Kg : 0);
    weights_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(Wm, (bf16*)Wb, (bf16*)Wt, Cout, Cin, ks * ks, Kpad,
                                                                  Kg);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_weights_implicit(const float* Wm, void* Wi, void* Wti, int Cout, int Cin, int Kpad, void* stream) {
    if (!Wm || !Wi || Cout <= 0 || Cin <= 0 || Kpad < 9 * Cin)
        return set_error(KGB_ERR_VALUE, "unet_weights_implicit: bad arguments");
    const int Cpi = (Cin + 63) / 64 * 64, Cpo = (Cout + 63) / 64 * 64;
    const int64_t n = (int64_t)Cout * 9 * Cpi + (Wti ? (int64_t)Cin * 9 * Cpo : 0);
    weights_implicit_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(Wm, (bf16*)Wi, (bf16*)Wti, Cout, Cin, Kpad,
                                                                           Cpi, Cpo);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_relu_grad(const float* dy, const void* y, void* g, int64_t n, int relu, void* stream) {
    if (!dy || !g || (relu && !y) || n <= 0) return set_error(KGB_ERR_VALUE, "unet_relu_grad: bad arguments");
    if (n % 8 == 0 && (((uintptr_t)dy | (uintptr_t)g | (relu ? (uintptr_t)y : 0)) & 15) == 0)
        relu_grad_vec_kernel<<<grid_for(n / 8), 256, 0, (cudaStream_t)stream>>>(
            (const float4*)dy, (const uint4*)y, (uint4*)g, n / 8, relu);
    else
        relu_grad_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(dy, (const bf16*)y, (bf16*)g, n, relu);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_rowsum(const void* in, float* out, int rows, int64_t cols, float* work, void* stream) {
    if (!in || !out || !work || rows <= 0 || cols <= 0) return set_error(KGB_ERR_VALUE, "unet_rowsum: bad arguments");
    dim3 grid((unsigned)rows, (unsigned)kRowChunks);
    rowsum_partial_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>((const bf16*)in, work, cols);
    rowsum_final_kernel<<<(rows + 127) / 128, 128, 0, (cudaStream_t)stream>>>(work, out, rows);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_upsample(const void* x, void* y, int B, int H, int W, int C, int Ctot, int coff, int grad, void* stream) {
    if (!x || !y || B <= 0 || H <= 0 || W <= 0 || C <= 0 || coff < 0 || coff + C > Ctot)
        return set_error(KGB_ERR_VALUE, "unet_upsample: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    if (grad) {
        const int64_t n = (int64_t)B * H * W * C;
        if (n < (int64_t)1 << 31)
            upsample_grad_kernel<uint32_t><<<grid_for(n), 256, 0, s>>>((const float*)x, (float*)y, B, H, W, C, Ctot, coff);
        else
            upsample_grad_kernel<int64_t><<<grid_for(n), 256, 0, s>>>((const float*)x, (float*)y, B, H, W, C, Ctot, coff);
    } else {
        if (C % 8 == 0 && Ctot % 8 == 0 && coff % 8 == 0 && (((uintptr_t)x | (uintptr_t)y) & 15) == 0) {
            const int64_t n = (int64_t)B * 4 * H * W * (C / 8);
            if (n < (int64_t)1 << 31)
                upsample_vec_kernel<uint32_t><<<grid_for(n), 256, 0, s>>>((const uint4*)x, (uint4*)y, B, H, W, C / 8,
                                                                          Ctot / 8, coff / 8);
            else
                upsample_vec_kernel<int64_t><<<grid_for(n), 256, 0, s>>>((const uint4*)x, (uint4*)y, B, H, W, C / 8,
                                                                         Ctot / 8, coff / 8);
        } else {
            const int64_t n = (int64_t)B * 4 * H * W * C;
            upsample_kernel<<<grid_for(n), 256, 0, s>>>((const bf16*)x, (bf16*)y, B, H, W, C, Ctot, coff);
        }
    }
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_channels(const void* x, void* y, int64_t P, int C, int Ctot, int coff, int take, int accumulate,
                      void* stream) {
    if (!x || !y || P <= 0 || C <= 0 || coff < 0 || coff + C > Ctot)
        return set_error(KGB_ERR_VALUE, "unet_channels: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const bool i32 = P * C < (int64_t)1 << 31;
    if (take && i32)
        take_channels_kernel<uint32_t><<<grid_for(P * C), 256, 0, s>>>((const float*)x, (float*)y, P, C, Ctot, coff,
                                                                       accumulate);
    else if (take)
        take_channels_kernel<int64_t><<<grid_for(P * C), 256, 0, s>>>((const float*)x, (float*)y, P, C, Ctot, coff,
                                                                      accumulate);
    else if (i32)
        put_channels_kernel<uint32_t><<<grid_for(P * C), 256, 0, s>>>((const bf16*)x, (bf16*)y, P, C, Ctot, coff);
    else
        put_channels_kernel<int64_t><<<grid_for(P * C), 256, 0, s>>>((const bf16*)x, (bf16*)y, P, C, Ctot, coff);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_to_bf16(const float* x, void* y, int64_t n, int B, const float* scale, void* stream) {
    if (!x || !y || n <= 0 || B <= 0) return set_error(KGB_ERR_VALUE, "unet_to_bf16: bad arguments");
    to_bf16_kernel<<<grid_for(n * B), 256, 0, (cudaStream_t)stream>>>(x, (bf16*)y, n, B, scale);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_row_transpose(const void* src, void* dst, int B, int H, int W, int C, int shifts, void* stream) {
    if (!src || !dst || B <= 0 || H <= 0 || W <= 0 || C <= 0 || C % 8 || W % 8 || (shifts != 1 && shifts != 3) ||
        (((uintptr_t)src | (uintptr_t)dst) & 15))
        return set_error(KGB_ERR_VALUE, "unet_row_transpose: bad arguments (C and W multiples of 8, 16-byte aligned)");
    const int64_t R = (int64_t)B * H;
    const int64_t items = R * ((W + 63) / 64) * ((C + 31) / 32);
    const int grid = (int)std::min<int64_t>(items, 16 * 152);
    row_transpose_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>((const bf16*)src, (bf16*)dst, R, W, C, shifts);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_colsum(const void* g, const void* wt, float* out, int64_t rows, int cols, float* work, void* stream) {
    if (!g || !out || !work || rows <= 0 || cols <= 0 || cols > 256 || cols % 8 || ((uintptr_t)g & 15))
        return set_error(KGB_ERR_VALUE, "unet_colsum: bad arguments (cols a multiple of 8 up to 256, g 16-byte aligned)");
    cudaStream_t s = (cudaStream_t)stream;
    // 256 threads: (256 / (cols / 8)) row phases x (cols / 8) column groups
    const int threads = (256 / (cols / 8)) * (cols / 8);
    colsum_partial_kernel<<<kColChunks, threads, 0, s>>>((const bf16*)g, (const bf16*)wt, work, rows, cols);
    KGB_CUDA_TRY(cudaGetLastError());
    colsum_final_kernel<<<(cols + 7) / 8, 256, 0, s>>>(work, out, cols);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_head_forward(const void* x, const void* w, const float* bias, float* y, int64_t P, int C, void* stream) {
    if (!x || !w || !y || P <= 0 || C <= 0 || C % 8 || C > 256 || ((uintptr_t)x & 15))
        return set_error(KGB_ERR_VALUE, "unet_head_forward: bad arguments");
    head_forward_kernel<<<grid_for(P), 256, 0, (cudaStream_t)stream>>>((const uint4*)x, (const bf16*)w, bias, y, P, C);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_head_dx(const void* g, const void* w, float* dx, int64_t P, int C, void* stream) {
    if (!g || !w || !dx || P <= 0 || C <= 0 || C % 4 || C > 256 || ((uintptr_t)dx & 15))
        return set_error(KGB_ERR_VALUE, "unet_head_dx: bad arguments");
    head_dx_kernel<<<grid_for(P * (C / 4)), 256, 0, (cudaStream_t)stream>>>((const bf16*)g, (const bf16*)w, (float4*)dx,
                                                                           P, C);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_conv3x3_c1(const void* x, const void* w, const void* bias, void* y, int B, int H, int W, int N, int kpad,
                        int relu, void* stream) {
    if (!x || !w || !y || B <= 0 || H <= 0 || W <= 0 || N <= 0 || N % 8 || N > 128 || kpad < 9 ||
        ((uintptr_t)y & 15))
        return set_error(KGB_ERR_VALUE, "unet_conv3x3_c1: bad arguments");
    const int64_t P = (int64_t)B * H * W;
    conv_c1_kernel<<<grid_for(P * (N / 8)), 256, 0, (cudaStream_t)stream>>>(
        (const bf16*)x, (const bf16*)w, (const float*)bias, (uint4*)y, B, H, W, N, kpad, relu);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_conv3x3_c1_wgrad(const void* x, const void* g, float* dW, int B, int H, int W, int N, int kpad,
                              float* work, void* stream) {
    if (!x || !g || !dW || !work || B <= 0 || H <= 0 || W <= 0 || N <= 0 || N > 128 || kpad < 9)
        return set_error(KGB_ERR_VALUE, "unet_conv3x3_c1_wgrad: bad arguments (N <= 128)");
    cudaStream_t s = (cudaStream_t)stream;
    const bool px = ((uintptr_t)g & 15) == 0;
    const bf16* xb = (const bf16*)x;
    const uint4* g4 = (const uint4*)g;
    if (px && N == 8)
        conv_c1_wgrad_px_kernel<1><<<kColChunks, 256, 0, s>>>(xb, g4, work, B, H, W);
    else if (px && N == 16)
        conv_c1_wgrad_px_kernel<2><<<kColChunks, 256, 0, s>>>(xb, g4, work, B, H, W);
    else if (px && N == 32)
        conv_c1_wgrad_px_kernel<4><<<kColChunks, 256, 0, s>>>(xb, g4, work, B, H, W);
    else if (px && N == 64)
        conv_c1_wgrad_px_kernel<8><<<kColChunks, 256, 0, s>>>(xb, g4, work, B, H, W);
    else
        conv_c1_wgrad_partial_kernel<<<kColChunks, 32 * kC1Warps, 0, s>>>(xb, (const bf16*)g, work, B, H, W, N);
    KGB_CUDA_TRY(cudaGetLastError());
    conv_c1_wgrad_final_kernel<<<(9 * N + 7) / 8, 256, 0, s>>>(work, dW, N, kpad);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_image_rms(const float* x, int64_t n, int B, float* scale, void* stream) {
    if (!x || !scale || n <= 0 || B <= 0) return set_error(KGB_ERR_VALUE, "unet_image_rms: bad arguments");
    image_rms_kernel<<<B, 512, 0, (cudaStream_t)stream>>>(x, n, scale);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_mse(const float* y, const float* t, float* grad, int64_t n, double* partials, double* loss,
                 void* stream) {
    if (!y || !t || !partials || !loss || n <= 0) return set_error(KGB_ERR_VALUE, "unet_mse: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    mse_kernel<<<kMseBlocks, 256, 0, s>>>(y, t, grad, n, partials);
    mse_final_kernel<<<1, 32, 0, s>>>(partials, kMseBlocks, n, loss);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_unet_adam(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps,
                  int step, void* stream) {
    if (!w || !g || !m || !v || n <= 0 || step < 1) return set_error(KGB_ERR_VALUE, "unet_adam: bad arguments");
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    adam_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

}  // extern "C"
