// Kirchhoff spreading (forward) and gathering (adjoint) kernels for sm_103a,
// and the wavelet convolution along time.
//
// Arithmetic follows pylops/waveeqprocessing/kirchhoff.py:728-1001:
//   t = ts + tr;  it = int(t/dt) (truncation);  w = t/dt - it;
//   valid iff 0 <= it < nt-1;
//   forward:  y[pair, it] += x*(1-w)*W;  y[pair, it+1] += x*w*W
//   adjoint:  img[ii] += (d[pair, it]*(1-w) + d[pair, it+1]*w)*W
// with W = 1 (kinematic) or the dynamic weight
//   W = 2 cos((a_s - a_r)/2) A_s A_r / v * taper_s * taper_r * offset_gate.
//
// Traveltimes are stored as 32-bit fixed-point sample counts, so t/dt of a
// source-receiver pair is one exact integer add: the integer part is a
// shift, the fraction a mask, and the index decision is the reference's
// float64 one except within 2^-frac_bits samples of a bin edge.
#include <cuda_runtime.h>

#include <algorithm>

#include "kgb_internal.h"

namespace kgb {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int kGatherThreads = 256;
constexpr int kGatherRC = 8;          // receivers held in registers per thread
constexpr int kSpreadThreads = 256;   // 8 warps, one trace per warp
constexpr int kNumSM = 152;

struct FixedPoint {
    int F;
    unsigned bias;   // 2^F - 1
    unsigned umax;   // nt*2^F - 1
    float scale;     // 2^-F
    __device__ __forceinline__ bool valid(int s) const { return (unsigned)s + bias < umax; }
    __device__ __forceinline__ int index(int s) const { return max(s, 0) >> F; }
    __device__ __forceinline__ float frac(int s, int it) const { return (float)(s - (it << F)) * scale; }
};

__host__ inline FixedPoint make_fp(int F, int nt) {
    FixedPoint fp;
    fp.F = F;
    fp.bias = (1u << F) - 1u;
    fp.umax = ((unsigned)nt << F) - 1u;
    fp.scale = 1.0f / (float)(1u << F);
    return fp;
}

// ---------------------------------------------------------------------------
// Adjoint: one thread per image point.  Each thread keeps kGatherRC receiver
// traveltimes (and weights) in registers and sweeps every source against
// them, so table reads are ~1/kGatherRC per pair-point and fully coalesced.
// The sum over traces has a fixed order per image point: the result is
// bit-identical run to run (no atomics).
// ---------------------------------------------------------------------------
template <bool DYN, bool GATE>
__global__ void __launch_bounds__(kGatherThreads)
gather_kernel(const KirchDev K, const FixedPoint fp, const float* __restrict__ d,
              float* __restrict__ out, int s_per_split) {
    const int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ii >= K.ni) return;
    const int s_begin = blockIdx.y * s_per_split;
    const int s_end = min(K.ns, s_begin + s_per_split);
    const int iz = (int)(ii % K.nz);
    const int nt = K.nt;
    float total = 0.f;
    for (int r0 = 0; r0 < K.nr; r0 += kGatherRC) {
        int trv[kGatherRC];
        float rcv[kGatherRC], rsv[kGatherRC];
#pragma unroll
        for (int r = 0; r < kGatherRC; ++r) {
            const int ir = r0 + r;
            trv[r] = 0;
            rcv[r] = 0.f;
            rsv[r] = 0.f;
            if (ir < K.nr) {
                trv[r] = __ldg(K.trq + (size_t)ir * K.ni + ii);
                if (DYN) {
                    rcv[r] = __ldg(K.wrc + (size_t)ir * K.ni + ii);
                    rsv[r] = __ldg(K.wrs + (size_t)ir * K.ni + ii);
                }
            }
        }
        const int nrc = min(kGatherRC, K.nr - r0);
        float chunk = 0.f;
        for (int is = s_begin; is < s_end; ++is) {
            const int ts = __ldg(K.tsq + (size_t)is * K.ni + ii);
            float sc = 0.f, ss = 0.f;
            if (DYN) {
                sc = __ldg(K.wsc + (size_t)is * K.ni + ii);
                ss = __ldg(K.wss + (size_t)is * K.ni + ii);
            }
            const size_t pair0 = (size_t)is * K.nr + r0;
            const float* drow = d + pair0 * nt;
#pragma unroll
            for (int r = 0; r < kGatherRC; ++r) {
                if (r < nrc) {
                    const int s = ts + trv[r];
                    if (fp.valid(s)) {
                        const int it = fp.index(s);
                        const float w = fp.frac(s, it);
                        const float* p = drow + (size_t)r * nt + it;
                        const float d0 = __ldg(p);
                        const float d1 = __ldg(p + 1);
                        float val = fmaf(w, d1 - d0, d0);
                        if (DYN) {
                            float wt = fmaf(sc, rcv[r], ss * rsv[r]);
                            if (GATE && iz < __ldg(K.izmin + pair0 + r)) wt = 0.f;
                            val *= wt;
                        }
                        chunk += val;
                    }
                }
            }
        }
        total += chunk;
    }
    if (DYN) total *= __ldg(K.vscale + ii);
    out[(size_t)blockIdx.y * K.ni + ii] = total;
}

// Fixed-order sum of the per-split partial images.
__global__ void sum_partials_kernel(const float* __restrict__ partial, float* __restrict__ img,
                                    int64_t ni, int nsplit) {
    for (int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ii < ni;
         ii += (int64_t)gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (int s = 0; s < nsplit; ++s) acc += partial[(size_t)s * ni + ii];
        img[ii] = acc;
    }
}

// ---------------------------------------------------------------------------
// Forward: one warp per trace (source-receiver pair) with a private trace in
// shared memory.  32 consecutive image points are processed per step; lanes
// whose contributions land in the same time bin are found with
// __match_any_sync and summed by the lowest lane of the bin in lane order
// (time-binned warp reduction), then the bin leaders update the shared
// trace in two conflict-free phases (sample it, then it+1).  No atomics: the
// result does not depend on scheduling.  The wavelet convolution is applied
// to the finished trace in shared memory and written once to HBM.
// ---------------------------------------------------------------------------
template <bool DYN, bool GATE>
__global__ void __launch_bounds__(kSpreadThreads)
spread_kernel(const KirchDev K, const FixedPoint fp, const float* __restrict__ m,
              float* __restrict__ y, const float* __restrict__ h, int L, int Lpad, int nt_pad,
              int fuse) {
    extern __shared__ float smem[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    float* hs = smem;
    float* trace = smem + Lpad + (size_t)warp * nt_pad;
    if (fuse) {
        for (int k = threadIdx.x; k < L; k += blockDim.x) hs[k] = h[k];
    }
    __syncthreads();
    const int64_t npair = (int64_t)K.ns * K.nr;
    const int64_t pair = (int64_t)blockIdx.x * nw + warp;
    if (pair >= npair) return;
    const int nt = K.nt;
    for (int n = lane; n < nt; n += 32) trace[n] = 0.f;
    __syncwarp();
    const int is = (int)(pair / K.nr);
    const int ir = (int)(pair - (int64_t)is * K.nr);
    const int32_t* __restrict__ tsrow = K.tsq + (size_t)is * K.ni;
    const int32_t* __restrict__ trrow = K.trq + (size_t)ir * K.ni;
    const int izmin = GATE ? __ldg(K.izmin + pair) : 0;
    const unsigned lower = (1u << lane) - 1u;
    for (int64_t base = 0; base < K.ni; base += 32) {
        const int64_t ii = base + lane;
        float v0 = 0.f, v1 = 0.f;
        int it = 0;
        bool valid = false;
        if (ii < K.ni) {
            const int s = __ldg(tsrow + ii) + __ldg(trrow + ii);
            if (fp.valid(s)) {
                it = fp.index(s);
                const float w = fp.frac(s, it);
                float val = __ldg(m + ii);
                if (DYN) {
                    float wt = fmaf(__ldg(K.wsc + (size_t)is * K.ni + ii), __ldg(K.wrc + (size_t)ir * K.ni + ii),
                                    __ldg(K.wss + (size_t)is * K.ni + ii) * __ldg(K.wrs + (size_t)ir * K.ni + ii));
                    wt *= __ldg(K.vscale + ii);
                    if (GATE && (int)(ii % K.nz) < izmin) wt = 0.f;
                    val *= wt;
                }
                v1 = val * w;
                v0 = val - v1;
                valid = true;
            }
        }
        if (__ballot_sync(FULL, valid) == 0u) continue;
        const unsigned key = valid ? (unsigned)it : (0x80000000u | (unsigned)lane);
        const unsigned peers = __match_any_sync(FULL, key);
        unsigned rest = peers & (peers - 1u);  // bin members after the lowest lane
        const int maxc = __reduce_max_sync(FULL, (unsigned)__popc(rest));
        float s0 = v0, s1 = v1;
        for (int k = 0; k < maxc; ++k) {
            const int src = rest ? (__ffs(rest) - 1) : lane;
            const float a0 = __shfl_sync(FULL, v0, src);
            const float a1 = __shfl_sync(FULL, v1, src);
            if (rest) {
                s0 += a0;
                s1 += a1;
                rest &= rest - 1u;
            }
        }
        const bool lead = valid && ((peers & lower) == 0u);
        if (lead) trace[it] += s0;
        __syncwarp();
        if (lead) trace[it + 1] += s1;
        __syncwarp();
    }
    float* __restrict__ yrow = y + pair * nt;
    if (fuse) {
        const int c = (L - 1) / 2;
        for (int n = lane; n < nt; n += 32) {
            const int kmin = max(0, n + c - (nt - 1));
            const int kmax = min(L - 1, n + c);
            float acc = 0.f;
            for (int k = kmin; k <= kmax; ++k) acc = fmaf(hs[k], trace[n + c - k], acc);
            yrow[n] = acc;
        }
    } else {
        for (int n = lane; n < nt; n += 32) yrow[n] = trace[n];
    }
}

// ---------------------------------------------------------------------------
// 'same'-mode FIR along time: y[n] = sum_k g[k] x[n + c - k], c = (L-1)/2.
// One block per trace (grid-stride), trace and taps staged in shared memory.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
wavelet_kernel(const float* __restrict__ x, float* __restrict__ y, int64_t ntr, int nt,
               const float* __restrict__ g, int L, int Lpad) {
    extern __shared__ float smem[];
    float* gs = smem;
    float* xs = smem + Lpad;
    for (int k = threadIdx.x; k < L; k += blockDim.x) gs[k] = g[k];
    const int c = (L - 1) / 2;
    for (int64_t tr = blockIdx.x; tr < ntr; tr += gridDim.x) {
        __syncthreads();
        const float* xrow = x + tr * nt;
        for (int n = threadIdx.x; n < nt; n += blockDim.x) xs[n] = xrow[n];
        __syncthreads();
        float* yrow = y + tr * nt;
        for (int n = threadIdx.x; n < nt; n += blockDim.x) {
            const int kmin = max(0, n + c - (nt - 1));
            const int kmax = min(L - 1, n + c);
            float acc = 0.f;
            for (int k = kmin; k <= kmax; ++k) acc = fmaf(gs[k], xs[n + c - k], acc);
            yrow[n] = acc;
        }
    }
}

int gather_splits(const KirchDev& K) {
    const int64_t blocks = (K.ni + kGatherThreads - 1) / kGatherThreads;
    const int64_t want = 2 * kNumSM;
    if (blocks >= want) return 1;
    int split = (int)std::min<int64_t>((want + blocks - 1) / blocks, (int64_t)K.ns);
    return std::max(split, 1);
}

}  // namespace

int64_t gather_partial_elems(const KirchDev& K) {
    const int split = gather_splits(K);
    return split > 1 ? (int64_t)split * K.ni : 0;
}

int launch_gather(const KirchDev& K, bool dynamic, bool gate, const float* d, float* img,
                  float* partial, int64_t partial_capacity, cudaStream_t stream) {
    if (K.ni <= 0 || K.ns <= 0 || K.nr <= 0) return KGB_OK;
    const FixedPoint fp = make_fp(K.frac_bits, K.nt);
    int split = gather_splits(K);
    int s_per = (K.ns + split - 1) / split;
    split = (K.ns + s_per - 1) / s_per;
    float* out = img;
    if (split > 1) {
        if (partial == nullptr || partial_capacity < (int64_t)split * K.ni)
            return set_error(KGB_ERR_STATE, "gather: partial-image scratch too small");
        out = partial;
    }
    dim3 grid((unsigned)((K.ni + kGatherThreads - 1) / kGatherThreads), (unsigned)split);
    if (dynamic) {
        if (gate) gather_kernel<true, true><<<grid, kGatherThreads, 0, stream>>>(K, fp, d, out, s_per);
        else gather_kernel<true, false><<<grid, kGatherThreads, 0, stream>>>(K, fp, d, out, s_per);
    } else {
        gather_kernel<false, false><<<grid, kGatherThreads, 0, stream>>>(K, fp, d, out, s_per);
    }
    KGB_CUDA_TRY(cudaGetLastError());
    if (split > 1) {
        const int blocks = (int)std::min<int64_t>((K.ni + 255) / 256, 4 * kNumSM);
        sum_partials_kernel<<<blocks, 256, 0, stream>>>(partial, img, K.ni, split);
        KGB_CUDA_TRY(cudaGetLastError());
    }
    return KGB_OK;
}

template <bool DYN, bool GATE>
static int spread_launch_t(const KirchDev& K, const FixedPoint& fp, const float* m, float* y,
                           const float* h, int L, bool fuse, cudaStream_t stream) {
    const int Lpad = fuse ? ((L + 3) & ~3) : 0;
    const int nt_pad = (K.nt + 3) & ~3;
    int warps = kSpreadThreads / 32;
    const size_t max_smem = 200 * 1024;
    while (warps > 1 && (size_t)(Lpad + warps * nt_pad) * sizeof(float) > max_smem) --warps;
    const size_t smem = (size_t)(Lpad + warps * nt_pad) * sizeof(float);
    if (smem > 227 * 1024)
        return set_error(KGB_ERR_NOT_IMPLEMENTED, "spread: nt=%d too long for one trace in shared memory", K.nt);
    auto kern = spread_kernel<DYN, GATE>;
    KGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t npair = (int64_t)K.ns * K.nr;
    const int64_t blocks = (npair + warps - 1) / warps;
    kern<<<(unsigned)blocks, warps * 32, smem, stream>>>(K, fp, m, y, h, L, Lpad, nt_pad, fuse ? 1 : 0);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_spread(const KirchDev& K, bool dynamic, bool gate, const float* m, float* y,
                  const float* h, int L, bool fuse_wavelet, cudaStream_t stream) {
    if (K.ns <= 0 || K.nr <= 0 || K.nt <= 0) return KGB_OK;
    const FixedPoint fp = make_fp(K.frac_bits, K.nt);
    if (dynamic) {
        if (gate) return spread_launch_t<true, true>(K, fp, m, y, h, L, fuse_wavelet, stream);
        return spread_launch_t<true, false>(K, fp, m, y, h, L, fuse_wavelet, stream);
    }
    return spread_launch_t<false, false>(K, fp, m, y, h, L, fuse_wavelet, stream);
}

int launch_wavelet(const float* x, float* y, int64_t ntr, int nt, const float* g, int L,
                   cudaStream_t stream) {
    if (ntr <= 0 || nt <= 0) return KGB_OK;
    const int Lpad = (L + 3) & ~3;
    const size_t smem = (size_t)(Lpad + nt) * sizeof(float);
    if (smem > 227 * 1024)
        return set_error(KGB_ERR_NOT_IMPLEMENTED, "wavelet: nt=%d too long for shared memory", nt);
    KGB_CUDA_TRY(cudaFuncSetAttribute(wavelet_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t blocks = std::min<int64_t>(ntr, 8 * kNumSM);
    wavelet_kernel<<<(unsigned)blocks, 256, smem, stream>>>(x, y, ntr, nt, g, L, Lpad);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

}  // namespace kgb
