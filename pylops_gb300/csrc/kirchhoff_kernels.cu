// Kirchhoff spreading (forward) and gathering (adjoint) kernels for sm_103a,
// and the wavelet convolution along time.
//
// Arithmetic follows pylops/waveeqprocessing/kirchhoff.py:728-1001:
//   t = ts + tr;  it = int(t/dt) (truncation);  w = t/dt - it;
//   valid iff 0 <= it < nt-1;
//   forward:  y[pair, it] += x*(1-w)*W;  y[pair, it+1] += x*w*W
//   adjoint:  img[ii] += (d[pair, it]*(1-w) + d[pair, it+1]*w)*W
// with W = 1 (kinematic) or the dynamic weight
//   W = 2 cos((a_s - a_r)/2) A_s A_r / v * taper_s * taper_r * offset_gate
//     = (2/v) * (wc_s wc_r + ws_s ws_r) * offset_gate,
//   wc = A taper cos(a/2), ws = A taper sin(a/2) (folded per table entry).
// A pair-point whose weight is exactly zero (outside the angle aperture)
// contributes exactly zero and is skipped before its data is touched.
//
// Traveltimes are stored as 32-bit fixed-point sample counts, so t/dt of a
// source-receiver pair is one exact integer add: the integer part is a
// shift, the fraction a mask, and the index decision is the reference's
// float64 one except within 2^-frac_bits samples of a bin edge.
//
// Both directions are deterministic: the adjoint sums each image point in a
// fixed order; the forward either accumulates exact 64-bit fixed point
// (integer additions commute) or bins contributions per warp in lane order.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <type_traits>
#include <vector>

#include "fir.cuh"
#include "fixed_acc.cuh"
#include "kgb_internal.h"
#include "tma.cuh"

namespace kgb {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int kGatherThreads = 256;
constexpr int kGatherRC = 4;        // receivers held in registers per thread
constexpr int kSpreadThreads = 512;
constexpr int kMaxSplit = 16;       // source splits of the gather (partial images)

int num_sms() {
    static int sms[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 148;
    if (!sms[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        sms[dev] = v > 0 ? v : 148;
    }
    return sms[dev];
}

// Fixed-point traveltime decoding.  s = ts + tr in units of 2^-F samples.
template <bool NONNEG>
struct FixedPoint {
    int F;
    unsigned bias;   // 2^F - 1 (general case)
    unsigned umax;   // NONNEG: (nt-1) 2^F; general: nt 2^F - 1
    unsigned fmask;  // 2^F - 1
    int fshift;      // 23 - F
    __device__ __forceinline__ bool valid(int s) const {
        return NONNEG ? ((unsigned)s < umax) : ((unsigned)s + bias < umax);
    }
    __device__ __forceinline__ int index(int s) const {
        return NONNEG ? (int)((unsigned)s >> F) : (max(s, 0) >> F);
    }
    // fraction w = t/dt - it; exact (F <= 22 bits)
    __device__ __forceinline__ float frac(int s, int it) const {
        if (NONNEG) {
            // 1.f + frac * 2^-F built directly in the mantissa, then minus 1
            return __int_as_float((((unsigned)s & fmask) << fshift) | 0x3f800000u) - 1.0f;
        }
        return (float)(s - (it << F)) * __int_as_float((127 - F) << 23);
    }
};

template <bool NONNEG>
FixedPoint<NONNEG> make_fp(int F, int nt) {
    FixedPoint<NONNEG> fp;
    fp.F = F;
    fp.bias = (1u << F) - 1u;
    fp.umax = NONNEG ? ((unsigned)(nt - 1) << F) : (((unsigned)nt << F) - 1u);
    fp.fmask = (1u << F) - 1u;
    fp.fshift = 23 - F;
    return fp;
}

// One table entry: traveltime (fixed point) and, in dynamic mode, weights.
struct Entry {
    int t;
    float c, s;
};

// STREAM: the record is read once per application (evict-first in L1 and
// L2, so the caches keep what is reused: data traces, model, re-read rows).
// HALF: bf16-weight records (8 bytes) from tab2 instead of tab.
template <bool DYN, bool STREAM = false, bool HALF = false>
__device__ __forceinline__ Entry load_entry(const int32_t* __restrict__ tq, const int4* __restrict__ tab,
                                            size_t idx, const int2* __restrict__ tab2 = nullptr) {
    Entry e;
    if (DYN && HALF) {
        // bf16 weights: one 8-byte record
        const int2 v = STREAM ? __ldcs(tab2 + idx) : __ldg(tab2 + idx);
        e.t = v.x;
        e.c = __uint_as_float((unsigned)v.y << 16);
        e.s = __uint_as_float((unsigned)v.y & 0xffff0000u);
    } else if (DYN) {
        const int4 v = STREAM ? __ldcs(tab + idx) : __ldg(tab + idx);
        e.t = v.x;
        e.c = __int_as_float(v.y);
        e.s = __int_as_float(v.z);
    } else {
        e.t = STREAM ? __ldcs(tq + idx) : __ldg(tq + idx);
        e.c = 1.f;
        e.s = 0.f;
    }
    return e;
}

__device__ __forceinline__ Entry zero_entry() {
    Entry e;
    e.t = 0;
    e.c = 0.f;
    e.s = 0.f;
    return e;
}

// Is depth iz inside a row's active range (packed lo | hi << 16) for this column?
__device__ __forceinline__ bool in_range(const uint32_t* __restrict__ rng, size_t idx, int iz) {
    const uint32_t v = __ldg(rng + idx);
    return iz >= (int)(v & 0xffffu) && iz < (int)(v >> 16);
}

// ---------------------------------------------------------------------------
// Adjoint: one thread per image point.  Each thread keeps kGatherRC receiver
// entries in registers and sweeps every source against them, so table reads
// are ~1/kGatherRC per pair-point and coalesced.  The correlated
// data is stored as interleaved pairs (d[it], d[it+1]) so one 8-byte load
// feeds the interpolation.  The sum over traces has a fixed order.  The
// loop is a chain of dependent loads (source record, then its data), so the
// kernel is sized for occupancy: four receivers per thread fit 32 registers
// and eight blocks (the SM's 64 warps) stay resident.
// ---------------------------------------------------------------------------
template <bool DYN, bool GATE, bool NONNEG, bool HALF = false>
__global__ void __launch_bounds__(kGatherThreads, 8)
gather_kernel(const KirchDev K, const FixedPoint<NONNEG> fp, const float2* __restrict__ d2,
              float* __restrict__ out, int r_per_split) {
    const int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    // lanes of this warp that stay (blockDim is a multiple of 32)
    const unsigned live = __ballot_sync(0xffffffffu, ii < K.ni);
    if (ii >= K.ni) return;
    // blockIdx.y selects a range of receivers: every split sweeps all sources,
    // which are re-streamed per receiver chunk anyway, so splitting adds no
    // table traffic
    const int s_begin = 0, s_end = K.ns;
    const int r_begin = blockIdx.y * r_per_split;
    const int r_end = min(K.nr, r_begin + r_per_split);
    int col = 0, iz = 0;  // depth column and depth (column counts fit in int)
    if (DYN || GATE) {
        col = (int)(ii / K.nz);
        iz = (int)(ii - (int64_t)col * K.nz);
    }
    const int ncol = (int)(K.ni / K.nz);
    const int nt = K.nt;
    // dynamic: which sources of this split are active at this image point
    // (sources beyond the first 64 of the split are always tested)
    unsigned long long smask = ~0ull;
    if (DYN) {
        smask = 0ull;
        for (int is = s_begin; is < min(s_end, s_begin + 64); ++is)
            if (in_range(K.srng, (size_t)is * ncol + col, iz)) smask |= 1ull << (is - s_begin);
    }
    float total = 0.f;
    for (int r0 = r_begin; r0 < r_end; r0 += kGatherRC) {
        // the warp skips the chunk when no receiver of the group of 8 that
        // holds it has a nonzero weight at any of the warp's points (a
        // warp-uniform branch; a per-thread one costs register spills)
        if (DYN && 8 % kGatherRC == 0 && K.grng &&
            !__any_sync(live, in_range(K.grng, (size_t)(r0 >> 3) * ncol + col, iz)))
            continue;
        Entry re[kGatherRC];
        const int nrc = min(kGatherRC, r_end - r0);
#pragma unroll
        for (int r = 0; r < kGatherRC; ++r) {
            re[r] = zero_entry();
            if (r < nrc) re[r] = load_entry<DYN, true, HALF>(K.trq, K.rtab, (size_t)(r0 + r) * K.ni + ii, K.rtab2);
        }
        float chunk = 0.f;
        for (int is = s_begin; is < s_end; ++is) {
            if (DYN) {
                const int k = is - s_begin;
                if (k < 64 ? !((smask >> k) & 1ull) : !in_range(K.srng, (size_t)is * ncol + col, iz)) continue;
            }
            const Entry se = load_entry<DYN, false, HALF>(K.tsq, K.stab, (size_t)is * K.ni + ii, K.stab2);
            if (DYN && se.c == 0.f && se.s == 0.f) continue;  // source outside the angle aperture
            const size_t pair0 = (size_t)is * K.nr + r0;
            const float2* __restrict__ drow = d2 + pair0 * nt;
#pragma unroll
            for (int r = 0; r < kGatherRC; ++r) {
                if (r < nrc) {
                    const int s = se.t + re[r].t;
                    float wt = 1.f;
                    if (DYN) {
                        wt = fmaf(se.c, re[r].c, se.s * re[r].s);
                        if (GATE && iz < __ldg(K.izmin + pair0 + r)) wt = 0.f;
                    }
                    if (fp.valid(s) && (!DYN || wt != 0.f)) {
                        const int it = fp.index(s);
                        const float w = fp.frac(s, it);
                        const float2 dd = __ldg(drow + ((size_t)r * nt + it));
                        const float val = fmaf(w, dd.y - dd.x, dd.x);
                        chunk = DYN ? fmaf(val, wt, chunk) : chunk + val;
                    }
                }
            }
        }
        total += chunk;
    }
    if (DYN) total *= __ldg(K.vscale + ii);
    out[(size_t)blockIdx.y * K.ni + ii] = total;
}

// ---------------------------------------------------------------------------
// Adjoint with the source records staged by TMA.  Same per-point arithmetic
// and summation order as gather_kernel (so the same bits), but the source
// record a thread needs at each step of its source loop is already in shared
// memory: the CTA's 256 image points' records of one source are one 4 KB
// (2 KB for bf16 weights) box of a 3-D bulk-tensor copy {record words,
// points, sources}, and kGatherStages boxes are in flight ahead of the
// consumers in a ring of full/empty mbarriers.  The dependent chain per
// source step becomes shared-memory record -> data load instead of global
// record -> data load.
//
// Work items are (source, receiver chunk) pairs in the order of
// gather_kernel's loops, skipping the sources and receiver groups that have
// zero weight at every point of the CTA (their contributions are exactly
// zero).  Thread 0 issues them: items 0..kGatherStages-1 up front, then item
// k + kGatherStages once all 8 warps released item k's stage; an item with
// source -1 ends the sequence.  Every wait is bounded; on a timeout the CTA
// records an error code in *err, stops, and thread 0 waits (bounded) for the
// copies it issued before the CTA exits.
// ---------------------------------------------------------------------------
constexpr int kGatherStages = 4;
constexpr int kGatherWarps = kGatherThreads / 32;
constexpr int kGatherTmaBlocks = 6;  // resident CTAs per SM the register budget is sized for

// Thread 0's producer state, in shared memory (it would otherwise take
// registers in every thread of the hot loop).
struct GatherProducer {
    int p_is, p_r0;          // last source issued, and its chunk
    int issued, consumed;    // items issued (the end marker included) and consumed by thread 0
    int stop;                // the end marker was issued
    unsigned smask[2];       // sources 0..63 with a nonzero weight at some point of the CTA
    unsigned gmask[2];       // receiver groups 0..63 of the split likewise
};

// The next (source, chunk) item that may have a nonzero weight, or src = -1.
__device__ __forceinline__ void gather_next_item(GatherProducer& P, int ns, int r_begin, int r_end, int g_begin,
                                                 bool groups, int& src, int& r0) {
    for (;;) {
        if (++P.p_is >= ns) {
            P.p_is = 0;
            P.p_r0 += kGatherRC;
        }
        if (P.p_r0 >= r_end) {
            src = -1;
            r0 = -1;
            return;
        }
        const int gi = (P.p_r0 >> 3) - g_begin;
        if (groups && gi < 64 && !((P.gmask[gi >> 5] >> (gi & 31)) & 1u)) {  // no point of the CTA in this group
            P.p_is = ns - 1;
            continue;
        }
        if (P.p_is < 64 && !((P.smask[P.p_is >> 5] >> (P.p_is & 31)) & 1u)) continue;  // zero at every point
        src = P.p_is;
        r0 = P.p_r0;
        return;
    }
}

template <bool GATE, bool NONNEG, bool HALF>
__global__ void __launch_bounds__(kGatherThreads, kGatherTmaBlocks)
gather_tma_kernel(const __grid_constant__ CUtensorMap smap, const KirchDev K, const FixedPoint<NONNEG> fp,
                  const float2* __restrict__ d2, float* __restrict__ out, int r_per_split, unsigned* __restrict__ err) {
    using Rec = typename std::conditional<HALF, int2, int4>::type;
    constexpr uint32_t kBox = kGatherThreads * sizeof(Rec);
    __shared__ __align__(128) Rec stage[kGatherStages][kGatherThreads];
    __shared__ __align__(8) unsigned long long full_bar[kGatherStages], empty_bar[kGatherStages];
    __shared__ int meta_src[kGatherStages], meta_r0[kGatherStages];
    __shared__ unsigned long long warp_groups[kGatherWarps];
    __shared__ GatherProducer P;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t ii = (int64_t)blockIdx.x * kGatherThreads + tid;
    const bool live = ii < K.ni;
    const int r_begin = blockIdx.y * r_per_split;
    const int r_end = min(K.nr, r_begin + r_per_split);
    const int64_t ncol = K.ni / K.nz;
    int col = 0, iz = 0;
    if (live) {
        col = (int)(ii / K.nz);
        iz = (int)(ii - (int64_t)col * K.nz);
    }
    const int nt = K.nt;
    const int g_begin = r_begin >> 3;
    if (tid == 0) {
        P.p_is = -1;
        P.p_r0 = r_begin;
        P.issued = P.consumed = P.stop = 0;
        P.smask[0] = P.smask[1] = P.gmask[0] = P.gmask[1] = 0u;
        for (int s = 0; s < kGatherStages; ++s) {
            tma::mbar_init(tma::smem_u32(&full_bar[s]), 1);
            tma::mbar_init(tma::smem_u32(&empty_bar[s]), kGatherWarps);
        }
        tma::mbar_fence_init();
    }
    __syncthreads();
    // sources 0..63 with a nonzero weight at this point
    unsigned long long smask = 0ull;
    if (live)
        for (int is = 0; is < min(K.ns, 64); ++is)
            if (in_range(K.srng, (size_t)is * ncol + col, iz)) smask |= 1ull << is;
    {
        // receiver groups of 8 (the first 64 of this split) with a nonzero
        // weight at some point of this warp; later groups are tested per chunk
        const int g_count = r_end > r_begin ? ((r_end - 1) >> 3) - g_begin + 1 : 0;
        unsigned long long wg = 0ull;
        if (K.grng)
            for (int g = 0; g < min(g_count, 64); ++g)
                if (__any_sync(FULL, live && in_range(K.grng, (size_t)(g_begin + g) * ncol + col, iz))) wg |= 1ull << g;
        const unsigned lo = __reduce_or_sync(FULL, (unsigned)smask);
        const unsigned hi = __reduce_or_sync(FULL, (unsigned)(smask >> 32));
        if (lane == 0) {
            warp_groups[warp] = wg;
            if (lo) atomicOr(&P.smask[0], lo);
            if (hi) atomicOr(&P.smask[1], hi);
            if ((unsigned)wg) atomicOr(&P.gmask[0], (unsigned)wg);
            if ((unsigned)(wg >> 32)) atomicOr(&P.gmask[1], (unsigned)(wg >> 32));
        }
    }
    __syncthreads();
    // thread 0: item j into stage j % kGatherStages
    auto issue = [&](int j) {
        const int s = j % kGatherStages;
        int src, r0;
        gather_next_item(P, K.ns, r_begin, r_end, g_begin, K.grng != nullptr, src, r0);
        meta_src[s] = src;
        meta_r0[s] = r0;
        const uint32_t fb = tma::smem_u32(&full_bar[s]);
        if (src < 0) {
            tma::mbar_arrive(fb);
            P.stop = 1;
        } else {
            tma::mbar_expect_tx(fb, kBox);
            const int64_t ii0 = (int64_t)blockIdx.x * kGatherThreads;
            tma::load_3d(tma::smem_u32(&stage[s][0]), &smap, fb, 0, HALF ? (int)(ii0 >> 1) : (int)ii0, src);
        }
        P.issued = j + 1;
    };
    if (tid == 0)
        for (int j = 0; j < kGatherStages && !P.stop; ++j) issue(j);
    Entry re[kGatherRC];
    int cur_r0 = -1;
    bool wact = false;
    float total = 0.f, chunk = 0.f;
    bool failed = false;
    for (int k = 0;; ++k) {
        const int s = k % kGatherStages;
        const uint32_t par = (uint32_t)(k / kGatherStages) & 1u;
        if (!tma::mbar_wait(tma::smem_u32(&full_bar[s]), par)) {
            atomicExch(err, 1u);
            failed = true;
            break;
        }
        if (tid == 0) P.consumed = k + 1;
        const int src = meta_src[s];
        const int r0 = meta_r0[s];
        if (src < 0) break;
        if (r0 != cur_r0) {
            if (wact) total += chunk;
            chunk = 0.f;
            cur_r0 = r0;
            const int gi = (r0 >> 3) - g_begin;
            wact = !K.grng ? true
                           : (gi < 64 ? ((warp_groups[warp] >> gi) & 1ull) != 0ull
                                      : __any_sync(FULL, live && in_range(K.grng, (size_t)(r0 >> 3) * ncol + col, iz)));
            if (wact && live) {
                const int nrc = min(kGatherRC, r_end - r0);
#pragma unroll
                for (int r = 0; r < kGatherRC; ++r) {
                    re[r] = zero_entry();
                    if (r < nrc) re[r] = load_entry<true, true, HALF>(K.trq, K.rtab, (size_t)(r0 + r) * K.ni + ii, K.rtab2);
                }
            }
        }
        if (wact && live &&
            (src < 64 ? ((smask >> src) & 1ull) != 0ull : in_range(K.srng, (size_t)src * ncol + col, iz))) {
            Entry se;
            if (HALF) {
                const int2 v = *reinterpret_cast<const int2*>(&stage[s][tid]);
                se.t = v.x;
                se.c = __uint_as_float((unsigned)v.y << 16);
                se.s = __uint_as_float((unsigned)v.y & 0xffff0000u);
            } else {
                const int4 v = *reinterpret_cast<const int4*>(&stage[s][tid]);
                se.t = v.x;
                se.c = __int_as_float(v.y);
                se.s = __int_as_float(v.z);
            }
            if (se.c != 0.f || se.s != 0.f) {
                const int nrc = min(kGatherRC, r_end - r0);
                const size_t pair0 = (size_t)src * K.nr + r0;
                const float2* __restrict__ drow = d2 + pair0 * nt;
#pragma unroll
                for (int r = 0; r < kGatherRC; ++r) {
                    if (r < nrc) {
                        const int sum = se.t + re[r].t;
                        float wt = fmaf(se.c, re[r].c, se.s * re[r].s);
                        if (GATE && iz < __ldg(K.izmin + pair0 + r)) wt = 0.f;
                        if (fp.valid(sum) && wt != 0.f) {
                            const int it = fp.index(sum);
                            const float w = fp.frac(sum, it);
                            const float2 dd = __ldg(drow + ((size_t)r * nt + it));
                            const float val = fmaf(w, dd.y - dd.x, dd.x);
                            chunk = fmaf(val, wt, chunk);
                        }
                    }
                }
            }
        }
        __syncwarp();
        if (lane == 0) tma::mbar_arrive(tma::smem_u32(&empty_bar[s]));
        if (tid == 0 && !P.stop) {
            // stage s is free once every warp released item k
            if (!tma::mbar_wait(tma::smem_u32(&empty_bar[s]), par)) {
                atomicExch(err, 2u);
                failed = true;
                break;
            }
            issue(k + kGatherStages);
        }
    }
    if (tid == 0) {
        // no copy of this CTA may still be in flight when it exits
        for (int j = P.consumed; j < P.issued; ++j)
            tma::mbar_wait(tma::smem_u32(&full_bar[j % kGatherStages]), (uint32_t)(j / kGatherStages) & 1u);
    }
    if (failed) return;
    if (wact) total += chunk;
    if (live) out[(size_t)blockIdx.y * K.ni + ii] = total * __ldg(K.vscale + ii);
}

// ---------------------------------------------------------------------------
// Adjoint with the next source record in flight (dynamic tables, at most 64
// sources).  Same sums in the same order as gather_kernel -- receiver chunks
// in order, within a chunk the sources with a nonzero weight at the point in
// increasing order -- so the image is the same bit for bit.  The active
// sources are walked through the point's bit mask, and the record of the
// next active source is loaded before the current one's data are read: the
// record load of step k+1 overlaps the data loads of step k instead of
// preceding them in one dependent chain.  Three more registers per thread
// cost resident warps (kGatherPfBlocks CTAs per SM).
// ---------------------------------------------------------------------------
constexpr int kGatherPfBlocks = 6;

template <bool GATE, bool NONNEG, bool HALF>
__global__ void __launch_bounds__(kGatherThreads, kGatherPfBlocks)
gather_pf_kernel(const KirchDev K, const FixedPoint<NONNEG> fp, const float2* __restrict__ d2,
                 float* __restrict__ out, int r_per_split) {
    const int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned live = __ballot_sync(0xffffffffu, ii < K.ni);
    if (ii >= K.ni) return;
    const int r_begin = blockIdx.y * r_per_split;
    const int r_end = min(K.nr, r_begin + r_per_split);
    const int col = (int)(ii / K.nz);
    const int iz = (int)(ii - (int64_t)col * K.nz);
    const int ncol = (int)(K.ni / K.nz);
    const int nt = K.nt;
    unsigned long long smask = 0ull;
    for (int is = 0; is < K.ns; ++is)
        if (in_range(K.srng, (size_t)is * ncol + col, iz)) smask |= 1ull << is;
    float total = 0.f;
    for (int r0 = r_begin; r0 < r_end; r0 += kGatherRC) {
        if (8 % kGatherRC == 0 && K.grng &&
            !__any_sync(live, in_range(K.grng, (size_t)(r0 >> 3) * ncol + col, iz)))
            continue;
        Entry re[kGatherRC];
        const int nrc = min(kGatherRC, r_end - r0);
#pragma unroll
        for (int r = 0; r < kGatherRC; ++r) {
            re[r] = zero_entry();
            if (r < nrc) re[r] = load_entry<true, true, HALF>(K.trq, K.rtab, (size_t)(r0 + r) * K.ni + ii, K.rtab2);
        }
        float chunk = 0.f;
        unsigned long long rem = smask;
        int cur = -1;
        Entry se = zero_entry();
        if (rem) {
            cur = __ffsll((long long)rem) - 1;
            rem &= rem - 1ull;
            se = load_entry<true, false, HALF>(K.tsq, K.stab, (size_t)cur * K.ni + ii, K.stab2);
        }
        while (cur >= 0) {
            int nxt = -1;
            Entry sn = zero_entry();
            if (rem) {  // the next active source's record, in flight while this one is used
                nxt = __ffsll((long long)rem) - 1;
                rem &= rem - 1ull;
                sn = load_entry<true, false, HALF>(K.tsq, K.stab, (size_t)nxt * K.ni + ii, K.stab2);
            }
            if (se.c != 0.f || se.s != 0.f) {
                const size_t pair0 = (size_t)cur * K.nr + r0;
                const float2* __restrict__ drow = d2 + pair0 * nt;
#pragma unroll
                for (int r = 0; r < kGatherRC; ++r) {
                    if (r < nrc) {
                        const int s = se.t + re[r].t;
                        float wt = fmaf(se.c, re[r].c, se.s * re[r].s);
                        if (GATE && iz < __ldg(K.izmin + pair0 + r)) wt = 0.f;
                        if (fp.valid(s) && wt != 0.f) {
                            const int it = fp.index(s);
                            const float w = fp.frac(s, it);
                            const float2 dd = __ldg(drow + ((size_t)r * nt + it));
                            const float val = fmaf(w, dd.y - dd.x, dd.x);
                            chunk = fmaf(val, wt, chunk);
                        }
                    }
                }
            }
            cur = nxt;
            se = sn;
        }
        total += chunk;
    }
    out[(size_t)blockIdx.y * K.ni + ii] = total * __ldg(K.vscale + ii);
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
// Forward.
// Prepass: mv = m * 2/v (dynamic) or m, and max |mv| for the fixed-point
// scale of the spreading kernel.
// ---------------------------------------------------------------------------
template <bool DYN>
__global__ void __launch_bounds__(256)
spread_prepass_kernel(const KirchDev K, const float* __restrict__ m) {
    __shared__ unsigned hist[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) hist[k] = 0u;
    __syncthreads();
    float amax = 0.f;
    for (int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ii < K.ni;
         ii += (int64_t)gridDim.x * blockDim.x) {
        float v = m[ii];
        if (DYN) v *= __ldg(K.vscale + ii);
        K.mv[ii] = v;
        amax = fmaxf(amax, fabsf(v));
        if (v != 0.f) atomicAdd(&hist[scale_bucket(v)], 1u);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(FULL, amax, o));
    if ((threadIdx.x & 31) == 0 && amax > 0.f) atomicMax(K.absmax, __float_as_uint(amax));
    __syncthreads();
    for (int k = threadIdx.x; k < 256; k += blockDim.x)
        if (hist[k]) atomicAdd(K.absmax + 2 + k, hist[k]);
}

// One block: the scale exponent from the scale block (fixed_choose_exponent).
__global__ void __launch_bounds__(256) spread_scale_kernel(const KirchDev K, float wfactor) {
    fixed_choose_exponent(K.absmax, K.ni, wfactor);
}

// Bound on |contribution| / |scaled model value| of the fixed-point spread:
// the largest weight, twice that on the general path, whose interpolation
// weight can be negative (|v (1 - w)| <= 2 |v| for -1 < w < 0).
__host__ __device__ __forceinline__ float spread_wfactor(float wmax, bool nonneg) { return nonneg ? wmax : 2.f * wmax; }

// Spreading, fixed-point variant: one CTA per (source, group of R receivers).
// A warp takes a depth column at a time and sweeps the depths where the
// source and at least one receiver of the group have a nonzero weight,
// loads the source-side entry once per point and, for each of its R traces,
// accumulates the two contributions v*(1-w), v*w into that trace's shared-
// memory time bins as 64-bit fixed point (each contribution scaled by a
// power of two chosen from a bound on |v|, rounded to an integer of at most
// kFixedBits bits plus sign and added exactly), so the trace is independent
// of the order in which threads arrive.  The finished traces are converted
// back to float, convolved with the wavelet in shared memory and written
// once.
//
// ACC selects how a bin adds:
//   kAccCarry  one returned 32-bit atomic per contribution plus a rare carry
//              (fixed_add), valid for any number of contributions per bin;
//   kAccSplit  two fire-and-forget 32-bit atomics (split_add), for operators
//              whose bins receive at most kSplitMaxCount contributions; wide
//              contributions go to the 64-bit global accumulator K.wacc;
//   kAccCount  no model: counts the contributions every bin can receive
//              (valid time, nonzero weight) and writes the largest count of
//              the CTA's bins to *K.count_out (atomicMax).
// kAccCarry and kAccSplit give bitwise identical traces.
constexpr int kAccCarry = 0, kAccSplit = 1, kAccCount = 2;

template <bool DYN, bool GATE, bool NONNEG, int R, bool HALF = false, int ACC = kAccCarry>
__global__ void __launch_bounds__(kSpreadThreads, 2)
spread_kernel(const KirchDev K, const FixedPoint<NONNEG> fp, float* __restrict__ y,
              const float* __restrict__ h, int L, int nt_pad, int fuse) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // R trace rows of 64-bit fixed-point bins (fixed_add layout)
    unsigned long long* acc = reinterpret_cast<unsigned long long*>(smem_raw);
    uint32_t* acc32 = reinterpret_cast<uint32_t*>(smem_raw);
    // the finished trace, zero-padded for fir_same, then the padded taps
    float* ftr = reinterpret_cast<float*>(acc + (size_t)R * nt_pad);
    float* hs = ftr + fir_span(L, K.nt);
    const int tid = threadIdx.x;
    const int nt = K.nt;
    const int ngroups = (K.nr + R - 1) / R;
    // source varies fastest across consecutive blocks: the CTAs resident at
    // one time share a few receiver groups (whose rows stay in L2) and sweep
    // the sources.
    const int is = blockIdx.x % K.ns;
    const int g = K.g0 + (int)(blockIdx.x / K.ns);
    if (g >= ngroups || g >= K.g1) return;
    const int r0 = g * R;
    const int nrr = min(R, K.nr - r0);
    __shared__ int wide_any;  // kAccSplit: a wide contribution went to K.wacc
    if (ACC == kAccCarry) fixed_clear(acc32, R, nt_pad, tid, blockDim.x);
    else split_clear(acc32, R, nt_pad, tid, blockDim.x);
    if (tid == 0) wide_any = 0;
    if (fuse && ACC != kAccCount) {
        for (int k = tid; k < fir_lpad(L); k += blockDim.x) hs[k] = k < L ? h[k] : 0.f;
        for (int k = tid; k < fir_span(L, K.nt); k += blockDim.x) ftr[k] = 0.f;
    }
    const int e = ACC == kAccCount ? 0 : (int)K.absmax[1];  // spread_scale_kernel
    const float S = ldexpf(1.f, e);
    // first depth of each receiver's gate, in shared memory (read as a warp
    // broadcast; held in registers it costs spills)
    __shared__ int izmin[R];
    if (tid < R) izmin[tid] = (GATE && tid < nrr) ? __ldg(K.izmin + (size_t)is * K.nr + r0 + tid) : 0;
    __syncthreads();
    const int64_t ncol = K.ni / K.nz;
    // one image point (index ii, depth izp in column colp, scaled value v);
    // FULL: all R receivers of the group exist (no per-receiver bounds)
    // WIDE: the point may give contributions of 2^31 or more (fixed_wide)
    auto point_t = [&](auto full, auto wide, int64_t ii, int64_t colp, int izp, float v) {
        constexpr bool FULL = decltype(full)::value;
        constexpr bool WIDE = decltype(wide)::value;
        const Entry se = load_entry<DYN, false, HALF>(K.tsq, K.stab, (size_t)is * K.ni + ii, K.stab2);
        if (DYN && se.c == 0.f && se.s == 0.f) return;  // source outside the angle aperture
        // all R receiver records in flight before any is used
        Entry re[R];
#pragma unroll
        for (int r = 0; r < R; ++r)
            re[r] = (FULL || r < nrr) ? load_entry<DYN, false, HALF>(K.trq, K.rtab, (size_t)(r0 + r) * K.ni + ii, K.rtab2)
                                      : zero_entry();
        if (WIDE && ACC == kAccSplit && !wide_any) wide_any = 1;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int s = se.t + re[r].t;
            float val = v;
            float wt = 1.f;
            if (DYN) {
                wt = fmaf(se.c, re[r].c, se.s * re[r].s);
                if (GATE && izp < izmin[r]) wt = 0.f;
                val *= wt;
            }
            // straight-line code: an invalid time or a missing receiver
            // gives zero contributions, which the adds skip
            const bool ok = (FULL || r < nrr) && fp.valid(s);
            const int it = fp.index(s);
            uint32_t* row = acc32 + (size_t)r * 2 * nt_pad;
            if (ACC == kAccCount) {
                if (ok && (!DYN || wt != 0.f)) {
                    atomicAdd(row + it, 1u);
                    atomicAdd(row + it + 1, 1u);
                }
                continue;
            }
            const float w = fp.frac(s, it);
            const float v1 = val * w;
            const float v0 = val - v1;
            if (WIDE && ACC == kAccSplit) {
                unsigned long long* wrow = K.wacc + ((size_t)is * K.nr + r0 + r) * nt;
                if (ok) {
                    split_add_wide(wrow, it, v0);
                    split_add_wide(wrow, it + 1, v1);
                }
            } else if (WIDE) {
                fixed_add_wide(row, nt_pad, it, ok ? v0 : 0.f);
                fixed_add_wide(row, nt_pad, it + 1, ok ? v1 : 0.f);
            } else if (ACC == kAccSplit) {
                split_add(row, nt_pad, it, ok ? __float2int_rn(v0) : 0);
                split_add(row, nt_pad, it + 1, ok ? __float2int_rn(v1) : 0);
            } else {
                fixed_add(row, nt_pad, it, ok ? __float2int_rn(v0) : 0);
                fixed_add(row, nt_pad, it + 1, ok ? __float2int_rn(v1) : 0);
            }
        }
    };
    auto point = [&](int64_t ii, int64_t colp, int izp, float v) {
        if (ACC != kAccCount && fixed_wide(v, spread_wfactor(K.wmax, NONNEG))) {
            if (nrr == R) point_t(std::true_type{}, std::true_type{}, ii, colp, izp, v);
            else point_t(std::false_type{}, std::true_type{}, ii, colp, izp, v);
        } else if (nrr == R) {
            point_t(std::true_type{}, std::false_type{}, ii, colp, izp, v);
        } else {
            point_t(std::false_type{}, std::false_type{}, ii, colp, izp, v);
        }
    };
    // scaled model value of point ii (every point counts as nonzero when counting)
    auto model = [&](int64_t ii) { return ACC == kAccCount ? 1.f : __ldg(K.mv + ii) * S; };
    if (DYN && R == 8 && K.grng) {
        // a warp per depth column, over the depths where both the source
        // and at least one receiver of this group of 8 have a nonzero weight
        const int lane = tid & 31;
        const int nw = blockDim.x >> 5;
        for (int64_t c = tid >> 5; c < ncol; c += nw) {
            const uint32_t a = __ldg(K.srng + (size_t)is * ncol + c);
            const uint32_t b = __ldg(K.grng + (size_t)g * ncol + c);
            const int lo = max((int)(a & 0xffffu), (int)(b & 0xffffu));
            const int hi = min((int)(a >> 16), (int)(b >> 16));
            for (int iz = lo + lane; iz < hi; iz += 32) {
                const int64_t ii = c * K.nz + iz;
                const float v = model(ii);
                if (v != 0.f) point(ii, c, iz, v);
            }
        }
    } else {
        // depth column and depth of this thread's point, advanced incrementally
        int64_t col = tid / K.nz;
        int iz = tid - (int)(col * K.nz);
        const int64_t stride_col = (int64_t)blockDim.x / K.nz;
        const int stride_iz = blockDim.x - (int)(stride_col * K.nz);
        for (int64_t ii = tid; ii < K.ni; ii += blockDim.x) {
            const int64_t colp = col;
            const int izp = iz;
            col += stride_col;
            iz += stride_iz;
            if (iz >= K.nz) {
                iz -= K.nz;
                ++col;
            }
            const float v = model(ii);
            if (v == 0.f) continue;  // zero model point: no contribution
            if (DYN && !in_range(K.srng, (size_t)is * ncol + colp, izp)) continue;  // source weight zero here
            point(ii, colp, izp, v);
        }
    }
    __syncthreads();
    if (ACC == kAccCount) {
        // the largest count of the CTA's bins (low plane of each row)
        unsigned mx = 0u;
        for (int r = 0; r < nrr; ++r)
            for (int n = tid; n < nt; n += blockDim.x) mx = max(mx, acc32[(size_t)r * 2 * nt_pad + n]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(FULL, mx, o));
        if ((tid & 31) == 0 && mx) atomicMax(K.count_out, mx);
        return;
    }
    const float invS = ldexpf(1.f, -e);
    const bool wide_rows = ACC == kAccSplit && wide_any;
    float* xt = fuse ? ftr + fir_q(L) : ftr;
    for (int r = 0; r < nrr; ++r) {
        const uint32_t* arow = acc32 + (size_t)r * 2 * nt_pad;
        unsigned long long* wrow = wide_rows ? K.wacc + ((size_t)is * K.nr + r0 + r) * nt : nullptr;
        for (int n = tid; n < nt; n += blockDim.x) {
            long long q;
            if (ACC == kAccSplit) {
                q = split_get(arow, nt_pad, n);
                if (wide_rows) {
                    // the wide part, read and cleared for the next application
                    q += (long long)wrow[n];
                    wrow[n] = 0ull;
                }
            } else {
                q = fixed_get(arow, nt_pad, n);
            }
            xt[n] = (float)q * invS;
        }
        __syncthreads();
        // the convolved trace goes to this receiver's accumulator row, which
        // is no longer needed (2 * nt_pad >= fir_out(nt) floats)
        const float* o = xt;
        if (fuse) {
            float* os = reinterpret_cast<float*>(acc32 + (size_t)r * 2 * nt_pad);
            fir_same(hs, ftr, os, L, nt, tid, blockDim.x);
            __syncthreads();
            o = os;
        }
        float* __restrict__ yrow = y + ((size_t)is * K.nr + r0 + r) * nt;
        for (int n = tid; n < nt; n += blockDim.x) __stcs(yrow + n, o[n]);
        __syncthreads();
    }
}

// Add one warp's contributions (lane: v0 at bin it, v1 at it + 1, if
// contrib) to a trace in shared memory, in a fixed order:
//  * bins strictly increasing over a run of consecutive lanes: straight
//    adds, bin it in one pass and it + 1 in the next;
//  * bins non-decreasing: lanes sharing a bin are contiguous; a segmented
//    warp scan (5 shuffle steps) sums each segment and its last lane adds;
//  * otherwise lanes sharing a bin are found with __match_any_sync and
//    summed by the bin's lowest lane in lane order.
__device__ __forceinline__ void warp_bin_add(float* trc, bool contrib, int it, float v0, float v1, int lane) {
    const unsigned cm = __ballot_sync(FULL, contrib);
    if (cm == 0u) return;
    if (!contrib) it = 0;
    const unsigned lower = (1u << lane) - 1u;
    const int first = __ffs(cm) - 1;
    const int last = 31 - __clz(cm);
    const unsigned sh = cm >> first;
    const bool run = (sh & (sh + 1u)) == 0u;
    const int prev_it = __shfl_up_sync(FULL, it, 1);
    const bool strict = !contrib || lane == first || it > prev_it;
    const bool nondec = !contrib || lane == first || it >= prev_it;
    if (run && __all_sync(FULL, strict)) {
        if (contrib) trc[it] += v0;
        __syncwarp();
        if (contrib) trc[it + 1] += v1;
        __syncwarp();
    } else if (run && __all_sync(FULL, nondec)) {
        const bool head = contrib && (lane == first || it != prev_it);
        const unsigned hm = __ballot_sync(FULL, head);
        const int start = 31 - __clz(hm & (lower | (1u << lane)));
        float s0 = v0, s1 = v1;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const float a0 = __shfl_up_sync(FULL, s0, off);
            const float a1 = __shfl_up_sync(FULL, s1, off);
            if (contrib && lane - off >= start) {
                s0 += a0;
                s1 += a1;
            }
        }
        const int next_it = __shfl_down_sync(FULL, it, 1);
        const bool tail = contrib && (lane == last || next_it != it);
        if (tail) trc[it] += s0;
        __syncwarp();
        if (tail) trc[it + 1] += s1;
        __syncwarp();
    } else {
        const unsigned key = contrib ? (unsigned)it : (0x80000000u | (unsigned)lane);
        const unsigned peers = __match_any_sync(FULL, key);
        unsigned rest = peers & (peers - 1u);
        const int maxc = __reduce_max_sync(FULL, (unsigned)__popc(rest));
        float s0 = v0, s1 = v1;
        for (int k = 0; k < maxc; ++k) {
            const int src = rest ? (__ffs(rest) - 1) : lane;
            const float b0 = __shfl_sync(FULL, v0, src);
            const float b1 = __shfl_sync(FULL, v1, src);
            if (rest) {
                s0 += b0;
                s1 += b1;
                rest &= rest - 1u;
            }
        }
        const bool lead = contrib && ((peers & lower) == 0u);
        if (lead) trc[it] += s0;
        __syncwarp();
        if (lead) trc[it + 1] += s1;
        __syncwarp();
    }
}

// Spreading, warp-binned variant: each warp owns RT traces (one source, RT
// receivers) in shared memory and walks the image one depth column at a time,
// 32 consecutive depths per step, lane = depth.  Down a column the time
// index of the contributing points normally increases strictly (always so
// inside an angle aperture below ~60 degrees, where the two-way vertical
// slowness exceeds one sample per cell); then the lanes' bins are distinct
// and the contributions are added directly, sample it in one pass and it+1
// in the next.  Otherwise lanes that share a bin are found with
// __match_any_sync and summed by the lowest lane of the bin in lane order.
// No atomics and a fixed summation order: deterministic.
template <bool DYN, bool GATE, bool NONNEG, int RT, bool HALF = false>
__global__ void __launch_bounds__(256)
spread_binned_kernel(const KirchDev K, const FixedPoint<NONNEG> fp, float* __restrict__ y,
                     const float* __restrict__ h, int L, int Lpad, int nt_pad, int fuse) {
    extern __shared__ __align__(16) float smem_f[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    float* hs = smem_f;
    float* traces = smem_f + Lpad + (size_t)warp * RT * nt_pad;
    if (fuse)
        for (int k = threadIdx.x; k < L; k += blockDim.x) hs[k] = h[k];
    __syncthreads();
    const int nt = K.nt;
    const int nz = K.nz;
    const int per_cta = nw * RT;
    const int ngroups = (K.nr + per_cta - 1) / per_cta;
    const int is = blockIdx.x % K.ns;
    const int g = blockIdx.x / K.ns;
    if (g >= ngroups) return;
    const int r0 = g * per_cta + warp * RT;
    const int nrr = max(0, min(RT, K.nr - r0));
    if (nrr == 0) return;
    for (int k = lane; k < RT * nt_pad; k += 32) traces[k] = 0.f;
    __syncwarp();
    int izmin[RT];
#pragma unroll
    for (int r = 0; r < RT; ++r) izmin[r] = (GATE && r < nrr) ? __ldg(K.izmin + (size_t)is * K.nr + r0 + r) : 0;
    const int64_t ncol = K.ni / nz;
    for (int64_t col = 0; col < ncol; ++col) {
        for (int iz0 = 0; iz0 < nz; iz0 += 32) {
            const int iz = iz0 + lane;
            const bool inb = iz < nz;
            const int64_t ii = col * nz + (inb ? iz : 0);
            float v = 0.f;
            Entry se;
            se.t = 0;
            se.c = se.s = 0.f;
            if (inb) {
                v = __ldg(K.mv + ii);
                if (DYN && !in_range(K.srng, (size_t)is * ncol + col, iz)) v = 0.f;
                if (v != 0.f) {
                    se = load_entry<DYN, false, HALF>(K.tsq, K.stab, (size_t)is * K.ni + ii, K.stab2);
                    if (DYN && se.c == 0.f && se.s == 0.f) v = 0.f;
                }
            }
            if (__ballot_sync(FULL, v != 0.f) == 0u) continue;
#pragma unroll
            for (int r = 0; r < RT; ++r) {
                if (r >= nrr) break;
                int s = 0;
                float val = 0.f;  // stays 0 for a receiver outside its active range
                if (inb && v != 0.f && (!DYN || in_range(K.rrng, (size_t)(r0 + r) * ncol + col, iz))) {
                    val = v;
                    const Entry re = load_entry<DYN, false, HALF>(K.trq, K.rtab, (size_t)(r0 + r) * K.ni + ii, K.rtab2);
                    s = se.t + re.t;
                    if (DYN) {
                        float wt = fmaf(se.c, re.c, se.s * re.s);
                        if (GATE && iz < izmin[r]) wt = 0.f;
                        val *= wt;
                    }
                }
                const bool tv = inb && val != 0.f && fp.valid(s);
                const int it = tv ? fp.index(s) : 0;
                float v0 = 0.f, v1 = 0.f;
                if (tv) {
                    const float w = fp.frac(s, it);
                    v1 = val * w;
                    v0 = val - v1;
                }
                warp_bin_add(traces + r * nt_pad, tv, it, v0, v1, lane);
            }
        }
    }
    const int c = (L - 1) / 2;
    for (int r = 0; r < nrr; ++r) {
        const float* tr = traces + r * nt_pad;
        float* __restrict__ yrow = y + ((size_t)is * K.nr + r0 + r) * nt;
        for (int n = lane; n < nt; n += 32) {
            float o;
            if (fuse) {
                const int kmin = max(0, n + c - (nt - 1));
                const int kmax = min(L - 1, n + c);
                o = 0.f;
                for (int k = kmin; k <= kmax; ++k) o = fmaf(hs[k], tr[n + c - k], o);
            } else {
                o = tr[n];
            }
            yrow[n] = o;
        }
    }
}

// ---------------------------------------------------------------------------
// 'same'-mode FIR along time: o[n] = sum_k g[k] x[n + c - k], c = (L-1)/2
// (fir_same).  One block per trace (grid-stride); taps and the zero-padded
// trace staged in shared memory, two trace buffers: the next trace's
// samples arrive by cp.async while the current one is filtered and
// written.  interleave = 1 writes (o[n], o[n+1]) pairs for the gather;
// g == nullptr copies the trace (o = x).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__global__ void __launch_bounds__(256)
wavelet_kernel(const float* __restrict__ x, float* __restrict__ y, int64_t ntr, int nt,
               const float* __restrict__ g, int L, int interleave) {
    extern __shared__ __align__(16) float smem[];
    const int Lp = fir_lpad(L);
    const int span = fir_span(L, nt);
    const int q = fir_q(L);
    float* gs = smem;
    float* xb0 = gs + Lp;
    float* xb1 = xb0 + span;
    float* os = xb1 + span;
    auto store = [&](int64_t tr) {
        if (interleave) {
            float2* yrow = reinterpret_cast<float2*>(y) + tr * nt;
            for (int n = threadIdx.x; n < nt; n += blockDim.x)
                yrow[n] = make_float2(os[n], n + 1 < nt ? os[n + 1] : 0.f);
        } else {
            float* yrow = y + tr * nt;
            for (int n = threadIdx.x; n < nt; n += blockDim.x) yrow[n] = os[n];
        }
    };
    if (!g) {
        // copy (no filter)
        for (int64_t tr = blockIdx.x; tr < ntr; tr += gridDim.x) {
            __syncthreads();
            const float* xrow = x + tr * nt;
            for (int n = threadIdx.x; n < nt; n += blockDim.x) os[n] = __ldcs(xrow + n);
            __syncthreads();
            store(tr);
        }
        return;
    }
    for (int k = threadIdx.x; k < Lp; k += blockDim.x) gs[k] = k < L ? g[k] : 0.f;
    for (int i = threadIdx.x; i < 2 * span; i += blockDim.x) xb0[i] = 0.f;
    __syncthreads();  // the zero padding is in place before the copies land
    auto stage = [&](int64_t tr, float* dst) {
        const float* xrow = x + tr * nt;
        for (int n = threadIdx.x; n < nt; n += blockDim.x) cp_async4(dst + q + n, xrow + n);
    };
    int64_t tr = blockIdx.x;
    if (tr < ntr) stage(tr, xb0);
    cp_async_commit();
    for (int it = 0; tr < ntr; ++it, tr += gridDim.x) {
        float* cur = (it & 1) ? xb1 : xb0;
        float* nxt = (it & 1) ? xb0 : xb1;
        // the next trace into the buffer filtered one iteration ago
        if (tr + gridDim.x < ntr) stage(tr + gridDim.x, nxt);
        cp_async_commit();
        cp_async_wait<1>();  // this thread's copies of the current trace landed
        __syncthreads();     // ... and every thread's
        fir_same(gs, cur, os, L, nt, threadIdx.x, blockDim.x);
        __syncthreads();
        store(tr);
    }
    cp_async_wait<0>();
}

// Dynamic-mode records {tq, wc, ws, 0}.
__global__ void pack_tables_kernel(const int32_t* __restrict__ tq, const float* __restrict__ wc,
                                   const float* __restrict__ ws, int4* __restrict__ tab, int64_t n) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        tab[k] = make_int4(tq[k], __float_as_int(wc[k]), __float_as_int(ws[k]), 0);
}

__global__ void pack_tables_bf16_kernel(const int32_t* __restrict__ tq, const float* __restrict__ wc,
                                        const float* __restrict__ ws, int2* __restrict__ tab, int64_t n) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(wc[k], ws[k]);  // .x = wc (low half), .y = ws
        tab[k] = make_int2(tq[k], *reinterpret_cast<const int*>(&h));
    }
}

// Union of the depth ranges of the receivers 8g .. 8g+7 for each column
// (empty ranges, lo = hi, do not widen it).
__global__ void group_range_kernel(const uint32_t* __restrict__ rrng, uint32_t* __restrict__ grng, int nr,
                                   int64_t ncol) {
    const int ng = (nr + 7) / 8;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < (int64_t)ng * ncol;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int g = (int)(k / ncol);
        const int64_t col = k - (int64_t)g * ncol;
        int lo = 1 << 30, hi = 0;
        for (int r = 8 * g; r < min(nr, 8 * g + 8); ++r) {
            const uint32_t v = rrng[(size_t)r * ncol + col];
            const int l = (int)(v & 0xffffu), h = (int)(v >> 16);
            if (h > l) {
                lo = min(lo, l);
                hi = max(hi, h);
            }
        }
        if (hi == 0) lo = 0;
        grng[k] = (uint32_t)lo | ((uint32_t)hi << 16);
    }
}

// Per (row, depth column): smallest and one-past-largest depth with a
// nonzero weight (lo = hi = 0 when the whole column is zero).
__global__ void range_kernel(const float* __restrict__ wc, const float* __restrict__ ws, uint32_t* __restrict__ rng,
                             int64_t nrows, int64_t ncol, int nz) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nrows * ncol;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = k / ncol, col = k - row * ncol;
        const size_t base = (size_t)row * ncol * nz + (size_t)col * nz;
        int lo = -1, hi = 0;
        for (int iz = 0; iz < nz; ++iz) {
            if (wc[base + iz] != 0.f || ws[base + iz] != 0.f) {
                if (lo < 0) lo = iz;
                hi = iz + 1;
            }
        }
        if (lo < 0) lo = hi = 0;
        rng[k] = (uint32_t)lo | ((uint32_t)hi << 16);
    }
}

// ---------------------------------------------------------------------------
// launch configuration
// ---------------------------------------------------------------------------
template <bool DYN, bool GATE, bool NONNEG, bool HALF = false>
int gather_blocks_per_sm() {
    static int cached = 0;
    if (!cached) {
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, gather_kernel<DYN, GATE, NONNEG, HALF>, kGatherThreads, 0);
        cached = nb > 0 ? nb : 1;
    }
    return cached;
}

// Number of receiver splits (ranges of whole register chunks) that keeps the
// last wave of the gather grid full.
int choose_split(int64_t blocks, int capacity, int nr) {
    int best = 1;
    double best_eff = 0.0;
    const int nchunks = (nr + kGatherRC - 1) / kGatherRC;
    const int maxs = std::min(kMaxSplit, nchunks);
    for (int s = 1; s <= maxs; ++s) {
        const int c_per = (nchunks + s - 1) / s;
        const int sp = (nchunks + c_per - 1) / c_per;
        const double waves = (double)(blocks * sp) / capacity;
        const double eff = waves / std::ceil(waves) * (waves >= 1.0 ? 1.0 : waves);
        if (eff > best_eff + 0.02) {
            best_eff = eff;
            best = sp;
        }
    }
    return best;
}

template <bool GATE, bool NONNEG, bool HALF>
int gather_tma_blocks_per_sm() {
    static int cached = 0;
    if (!cached) {
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, gather_tma_kernel<GATE, NONNEG, HALF>, kGatherThreads, 0);
        cached = nb > 0 ? nb : 1;
    }
    return cached;
}

// the staged (TMA) adjoint applies: dynamic tables with a record map
template <bool DYN>
bool gather_staged(const KirchDev& K) {
    return DYN && K.rec_map != nullptr && K.err != nullptr;
}

template <bool GATE, bool NONNEG, bool HALF>
int gather_pf_blocks_per_sm() {
    static int cached = 0;
    if (!cached) {
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, gather_pf_kernel<GATE, NONNEG, HALF>, kGatherThreads, 0);
        cached = nb > 0 ? nb : 1;
    }
    return cached;
}

// the adjoint with the next record in flight applies: dynamic tables, at most 64 sources
template <bool DYN>
bool gather_prefetch(const KirchDev& K) {
    return DYN && K.adjoint_variant == 1 && K.ns <= 64 && K.srng != nullptr;
}

template <bool DYN, bool GATE, bool NONNEG, bool HALF = false>
int gather_launch_t(const KirchDev& K, const float2* d2, float* img, float* partial, int64_t cap,
                    cudaStream_t stream) {
    const FixedPoint<NONNEG> fp = make_fp<NONNEG>(K.frac_bits, K.nt);
    const int64_t blocks = (K.ni + kGatherThreads - 1) / kGatherThreads;
    const bool staged = gather_staged<DYN>(K);
    const bool pf = !staged && gather_prefetch<DYN>(K);
    const int capacity = num_sms() * (staged ? gather_tma_blocks_per_sm<GATE, NONNEG, HALF>()
                                      : pf   ? gather_pf_blocks_per_sm<GATE, NONNEG, HALF>()
                                             : gather_blocks_per_sm<DYN, GATE, NONNEG, HALF>());
    int split = choose_split(blocks, capacity, K.nr);
    if (partial == nullptr || cap < (int64_t)split * K.ni) split = 1;
    const int nchunks = (K.nr + kGatherRC - 1) / kGatherRC;
    const int c_per = (nchunks + split - 1) / split;
    split = (nchunks + c_per - 1) / c_per;
    float* out = split > 1 ? partial : img;
    dim3 grid((unsigned)blocks, (unsigned)split);
    if (staged)
        gather_tma_kernel<GATE, NONNEG, HALF>
            <<<grid, kGatherThreads, 0, stream>>>(*K.rec_map, K, fp, d2, out, c_per * kGatherRC, K.err);
    else if (pf)
        gather_pf_kernel<GATE, NONNEG, HALF><<<grid, kGatherThreads, 0, stream>>>(K, fp, d2, out, c_per * kGatherRC);
    else
        gather_kernel<DYN, GATE, NONNEG, HALF><<<grid, kGatherThreads, 0, stream>>>(K, fp, d2, out, c_per * kGatherRC);
    KGB_CUDA_TRY(cudaGetLastError());
    if (split > 1) {
        const int nb = (int)std::min<int64_t>((K.ni + 255) / 256, 4 * num_sms());
        sum_partials_kernel<<<nb, 256, 0, stream>>>(partial, img, K.ni, split);
        KGB_CUDA_TRY(cudaGetLastError());
    }
    return KGB_OK;
}

struct SpreadShape {
    int R;
    size_t smem;
    int nt_pad;
};

// Receivers per CTA: as many as keep two CTAs per SM, fewer when the grid
// would not fill the GPU.
SpreadShape spread_shape(const KirchDev& K, int L) {
    SpreadShape sh;
    sh.nt_pad = (K.nt + 3) & ~3;
    const size_t fixed = (size_t)(fir_span(L, K.nt) + fir_lpad(L)) * sizeof(float);
    const size_t budget2 = 110 * 1024, budget1 = 220 * 1024;
    int R = 8;
    auto need = [&](int r) { return fixed + (size_t)r * sh.nt_pad * 8; };
    while (R > 1 && need(R) > budget2) R >>= 1;
    const int sms = num_sms();
    while (R > 1 && (int64_t)K.ns * ((K.nr + R - 1) / R) < 2 * sms) R >>= 1;
    if (need(R) > budget1) R = 0;
    sh.R = R;
    sh.smem = R ? need(R) : 0;
    return sh;
}

// wfactor: bound on |contribution| / |mv| (the largest weight; 2 for the
// single table's negative-time path)
template <bool DYN>
int launch_prepass(const KirchDev& K, const float* m, cudaStream_t stream, float wfactor) {
    KGB_CUDA_TRY(cudaMemsetAsync(K.absmax, 0, kScaleWords * sizeof(unsigned), stream));
    const int pb = (int)std::min<int64_t>((K.ni + 255) / 256, 4 * num_sms());
    spread_prepass_kernel<DYN><<<pb, 256, 0, stream>>>(K, m);
    spread_scale_kernel<<<1, 256, 0, stream>>>(K, wfactor);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

template <bool DYN, bool GATE, bool NONNEG, int R, bool HALF = false>
int spread_launch_r(const KirchDev& K, const float* m, float* y, const float* h, int L, bool fuse,
                    const SpreadShape& sh, cudaStream_t stream, bool prepare_only) {
    // split accumulation (R = 8 only): see spread_kernel
    constexpr int ACC2 = R == 8 ? kAccSplit : kAccCarry;
    const bool split = R == 8 && K.split_ok && K.wacc != nullptr && K.spread_variant != 3;
    auto kern = split ? spread_kernel<DYN, GATE, NONNEG, R, HALF, ACC2> : spread_kernel<DYN, GATE, NONNEG, R, HALF>;
    if (prepare_only) {
        KGB_CUDA_TRY(cudaFuncSetAttribute(spread_kernel<DYN, GATE, NONNEG, R, HALF>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem));
        if (R == 8) {
            KGB_CUDA_TRY(cudaFuncSetAttribute(spread_kernel<DYN, GATE, NONNEG, R, HALF, ACC2>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem));
            KGB_CUDA_TRY(cudaFuncSetAttribute(spread_kernel<DYN, GATE, NONNEG, R, HALF, kAccCount>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh.smem));
        }
        return KGB_OK;
    }
    if (K.prepass) {
        int rc = launch_prepass<DYN>(K, m, stream, spread_wfactor(K.wmax, NONNEG));
        if (rc) return rc;
    }
    const FixedPoint<NONNEG> fp = make_fp<NONNEG>(K.frac_bits, K.nt);
    const int ngroups = (K.nr + R - 1) / R;
    const int gn = std::min(ngroups, K.g1) - std::max(0, K.g0);
    if (gn <= 0) return KGB_OK;
    const int64_t blocks = (int64_t)K.ns * gn;
    kern<<<(unsigned)blocks, kSpreadThreads, sh.smem, stream>>>(K, fp, y, h, L, sh.nt_pad, fuse ? 1 : 0);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

// Warp-binned variant: RT traces per warp, 8 warps per CTA.
template <bool DYN, bool GATE, bool NONNEG, int RT, bool HALF = false>
int spread_binned_launch_r(const KirchDev& K, const float* m, float* y, const float* h, int L, bool fuse,
                           cudaStream_t stream, bool prepare_only) {
    auto kern = spread_binned_kernel<DYN, GATE, NONNEG, RT, HALF>;
    const int Lpad = (L + 3) & ~3;
    const int nt_pad = (K.nt + 3) & ~3;
    const int warps = 8;
    const size_t smem = (size_t)(Lpad + (size_t)warps * RT * nt_pad) * sizeof(float);
    if (smem > 227 * 1024)
        return set_error(KGB_ERR_NOT_IMPLEMENTED, "spread: nt=%d too long for the binned variant", K.nt);
    if (prepare_only) {
        KGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return KGB_OK;
    }
    int rc = launch_prepass<DYN>(K, m, stream, K.wmax);
    if (rc) return rc;
    const FixedPoint<NONNEG> fp = make_fp<NONNEG>(K.frac_bits, K.nt);
    const int per_cta = warps * RT;
    const int64_t blocks = (int64_t)K.ns * ((K.nr + per_cta - 1) / per_cta);
    kern<<<(unsigned)blocks, warps * 32, smem, stream>>>(K, fp, y, h, L, Lpad, nt_pad, fuse ? 1 : 0);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

template <bool DYN, bool GATE, bool NONNEG, bool HALF = false>
int spread_launch_t(const KirchDev& K, const float* m, float* y, const float* h, int L, bool fuse,
                    cudaStream_t stream, bool prepare_only) {
    const int Lpad = (L + 3) & ~3;
    const int nt_pad = (K.nt + 3) & ~3;
    const bool fits1 = (size_t)(Lpad + 8 * (size_t)nt_pad) * 4 <= 227 * 1024;
    const bool fits2 = (size_t)(Lpad + 16 * (size_t)nt_pad) * 4 <= 227 * 1024;
    int rc = KGB_OK;
    if (prepare_only) {
        if (fits1) rc = spread_binned_launch_r<DYN, GATE, NONNEG, 1, HALF>(K, m, y, h, L, fuse, stream, true);
        if (!rc && fits2) rc = spread_binned_launch_r<DYN, GATE, NONNEG, 2, HALF>(K, m, y, h, L, fuse, stream, true);
        if (rc) return rc;
    } else if (K.spread_variant == 2 && fits2) {
        return spread_binned_launch_r<DYN, GATE, NONNEG, 2, HALF>(K, m, y, h, L, fuse, stream, false);
    } else if (K.spread_variant == 1 && fits1) {
        return spread_binned_launch_r<DYN, GATE, NONNEG, 1, HALF>(K, m, y, h, L, fuse, stream, false);
    }
    const SpreadShape sh = spread_shape(K, L);
    switch (sh.R) {
        case 8: return spread_launch_r<DYN, GATE, NONNEG, 8, HALF>(K, m, y, h, L, fuse, sh, stream, prepare_only);
        case 4: return spread_launch_r<DYN, GATE, NONNEG, 4, HALF>(K, m, y, h, L, fuse, sh, stream, prepare_only);
        case 2: return spread_launch_r<DYN, GATE, NONNEG, 2, HALF>(K, m, y, h, L, fuse, sh, stream, prepare_only);
        case 1: return spread_launch_r<DYN, GATE, NONNEG, 1, HALF>(K, m, y, h, L, fuse, sh, stream, prepare_only);
        default:
            return set_error(KGB_ERR_NOT_IMPLEMENTED, "spread: nt=%d too long for one trace in shared memory", K.nt);
    }
}

template <bool DYN, bool GATE, bool HALF = false>
int spread_dispatch_nn(const KirchDev& K, const float* m, float* y, const float* h, int L, bool fuse,
                       cudaStream_t stream, bool prep) {
    if (K.nonneg) return spread_launch_t<DYN, GATE, true, HALF>(K, m, y, h, L, fuse, stream, prep);
    return spread_launch_t<DYN, GATE, false, HALF>(K, m, y, h, L, fuse, stream, prep);
}

int spread_dispatch(const KirchDev& K, bool dynamic, bool gate, const float* m, float* y, const float* h,
                    int L, bool fuse, cudaStream_t stream, bool prep) {
    if (dynamic && K.stab2) {
        if (gate) return spread_dispatch_nn<true, true, true>(K, m, y, h, L, fuse, stream, prep);
        return spread_dispatch_nn<true, false, true>(K, m, y, h, L, fuse, stream, prep);
    }
    if (dynamic) {
        if (gate) return spread_dispatch_nn<true, true>(K, m, y, h, L, fuse, stream, prep);
        return spread_dispatch_nn<true, false>(K, m, y, h, L, fuse, stream, prep);
    }
    return spread_dispatch_nn<false, false>(K, m, y, h, L, fuse, stream, prep);
}

template <bool DYN, bool GATE, bool NONNEG, bool HALF = false>
int spread_count_t(const KirchDev& K, int L, unsigned* count, cudaStream_t stream) {
    const SpreadShape sh = spread_shape(K, L);
    if (sh.R != 8) {  // the split kernels exist for groups of 8 receivers only
        KGB_CUDA_TRY(cudaMemsetAsync(count, 0xff, sizeof(unsigned), stream));
        return KGB_OK;
    }
    KirchDev Kc = K;
    Kc.count_out = count;
    const FixedPoint<NONNEG> fp = make_fp<NONNEG>(K.frac_bits, K.nt);
    const int64_t blocks = (int64_t)K.ns * ((K.nr + 7) / 8);
    spread_kernel<DYN, GATE, NONNEG, 8, HALF, kAccCount>
        <<<(unsigned)blocks, kSpreadThreads, sh.smem, stream>>>(Kc, fp, nullptr, nullptr, L, sh.nt_pad, 0);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

template <bool DYN, bool GATE, bool HALF = false>
int spread_count_nn(const KirchDev& K, int L, unsigned* count, cudaStream_t stream) {
    if (K.nonneg) return spread_count_t<DYN, GATE, true, HALF>(K, L, count, stream);
    return spread_count_t<DYN, GATE, false, HALF>(K, L, count, stream);
}

// ---------------------------------------------------------------------------
// Single traveltime table (kirchhoff.py:396-398, 684-725): one table entry
// per (image point, trace), t/dt = itrav + travd with itrav = int(t/dt).
// The table is the whole input of the operator (4 bytes per pair-point, read
// once per application), so both directions stream it from HBM with
// evict-first loads; they are HBM-bound by design.
// ---------------------------------------------------------------------------
template <bool FIXED>
__device__ __forceinline__ bool single_entry(const KirchDev& K, const FixedPoint<true>& fp, int q, float wf, int& it,
                                             float& w) {
    if (FIXED) {
        if (!fp.valid(q)) return false;
        it = fp.index(q);
        w = fp.frac(q, it);
        return true;
    }
    it = q;
    w = wf;
    return (unsigned)q < (unsigned)(K.nt - 1);
}

// Adjoint: one thread per image point, traces [t0, t1) of its split in
// order; four table entries in flight per thread.
template <bool FIXED>
__global__ void __launch_bounds__(256)
gather1_kernel(const KirchDev K, const FixedPoint<true> fp, const float2* __restrict__ d2, float* __restrict__ out,
               int tr_per_split) {
    const int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ii >= K.ni) return;
    const int nsnr = K.ns * K.nr;
    const int t0 = blockIdx.y * tr_per_split;
    const int t1 = min(nsnr, t0 + tr_per_split);
    const int32_t* __restrict__ tq = K.tq1 + ii;
    const float* __restrict__ tw = FIXED ? nullptr : K.tw1 + ii;
    float acc = 0.f;
    int tr = t0;
    for (; tr + 4 <= t1; tr += 4) {
        int q[4];
        float wf[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            q[u] = __ldcs(tq + (size_t)(tr + u) * K.ni);
            wf[u] = FIXED ? 0.f : __ldcs(tw + (size_t)(tr + u) * K.ni);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            int it;
            float w;
            if (single_entry<FIXED>(K, fp, q[u], wf[u], it, w)) {
                const float2 p = __ldg(d2 + (size_t)(tr + u) * K.nt + it);
                acc = fmaf(p.x, 1.f - w, acc);
                acc = fmaf(p.y, w, acc);
            }
        }
    }
    for (; tr < t1; ++tr) {
        int it;
        float w;
        const int q = __ldcs(tq + (size_t)tr * K.ni);
        const float wf = FIXED ? 0.f : __ldcs(tw + (size_t)tr * K.ni);
        if (single_entry<FIXED>(K, fp, q, wf, it, w)) {
            const float2 p = __ldg(d2 + (size_t)tr * K.nt + it);
            acc = fmaf(p.x, 1.f - w, acc);
            acc = fmaf(p.y, w, acc);
        }
    }
    out[(size_t)blockIdx.y * K.ni + ii] = acc;
}

// Adjoint, vector form (ni % 4 == 0): one thread per 4 consecutive image
// points, one 16-byte table load per trace, the next 4 traces' entries
// loaded while the current ones are used.  Same per-point summation order
// as gather1_kernel.
template <bool FIXED>
__device__ __forceinline__ void gather1_accumulate(const KirchDev& K, const FixedPoint<true>& fp,
                                                   const float2* __restrict__ drow, int q, float wf, float& acc) {
    int it;
    float w;
    if (single_entry<FIXED>(K, fp, q, wf, it, w)) {
        const float2 p = __ldg(drow + it);
        acc = fmaf(p.x, 1.f - w, acc);
        acc = fmaf(p.y, w, acc);
    }
}

template <bool FIXED>
__global__ void __launch_bounds__(256)
gather1_vec_kernel(const KirchDev K, const FixedPoint<true> fp, const float2* __restrict__ d2, float* __restrict__ out,
                   int tr_per_split) {
    const int64_t i4 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i4 * 4 >= K.ni) return;
    const int nsnr = K.ns * K.nr;
    const int t0 = blockIdx.y * tr_per_split;
    const int t1 = min(nsnr, t0 + tr_per_split);
    const int4* __restrict__ tq = reinterpret_cast<const int4*>(K.tq1) + i4;
    const float4* __restrict__ tw = FIXED ? nullptr : reinterpret_cast<const float4*>(K.tw1) + i4;
    const int64_t rs = K.ni / 4;  // row stride in 16-byte units
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    constexpr int U = 4;
    int4 qn[U];
    float4 wn[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const bool ok = t0 + u < t1;
        qn[u] = ok ? __ldcs(tq + (size_t)(t0 + u) * rs) : make_int4(-1, -1, -1, -1);
        wn[u] = (!FIXED && ok) ? __ldcs(tw + (size_t)(t0 + u) * rs) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int tr = t0; tr < t1; tr += U) {
        int4 q[U];
        float4 wf[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            q[u] = qn[u];
            wf[u] = wn[u];
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const bool ok = tr + U + u < t1;
            qn[u] = ok ? __ldcs(tq + (size_t)(tr + U + u) * rs) : make_int4(-1, -1, -1, -1);
            wn[u] = (!FIXED && ok) ? __ldcs(tw + (size_t)(tr + U + u) * rs) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (tr + u >= t1) break;
            const float2* drow = d2 + (size_t)(tr + u) * K.nt;
            gather1_accumulate<FIXED>(K, fp, drow, q[u].x, wf[u].x, a0);
            gather1_accumulate<FIXED>(K, fp, drow, q[u].y, wf[u].y, a1);
            gather1_accumulate<FIXED>(K, fp, drow, q[u].z, wf[u].z, a2);
            gather1_accumulate<FIXED>(K, fp, drow, q[u].w, wf[u].w, a3);
        }
    }
    reinterpret_cast<float4*>(out + (size_t)blockIdx.y * K.ni)[i4] = make_float4(a0, a1, a2, a3);
}

// Forward, warp-binned: one warp per trace walking the image one depth
// column at a time, 32 consecutive depths per step (lane = depth).  When
// the contributing lanes' time bins increase strictly (the usual case down a
// column) they add straight into the warp's shared-memory trace, bin it in
// one pass and it + 1 in the next; otherwise lanes sharing a bin are summed
// by the bin's lowest lane in lane order (__match_any_sync).  No atomics,
// fixed order: deterministic.  Each table entry is read once.
template <bool FIXED>
__global__ void __launch_bounds__(256)
spread1_binned_kernel(const KirchDev K, const FixedPoint<true> fp, const float* __restrict__ m, float* __restrict__ y,
                      const float* __restrict__ h, int L, int Lpad, int nt_pad, int fuse) {
    extern __shared__ __align__(16) float smem_f[];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    float* hs = smem_f;
    float* trc = smem_f + Lpad + (size_t)warp * nt_pad;
    if (fuse)
        for (int k = threadIdx.x; k < L; k += blockDim.x) hs[k] = h[k];
    __syncthreads();
    const int tr = blockIdx.x * nw + warp;
    if (tr >= K.ns * K.nr) return;
    const int nt = K.nt, nz = K.nz;
    for (int k = lane; k < nt_pad; k += 32) trc[k] = 0.f;
    __syncwarp();
    const int64_t ncol = K.ni / nz;
    const int cpc = (nz + 31) / 32;  // 32-depth chunks per column
    const int64_t nchunk = ncol * cpc;
    const int32_t* __restrict__ tq = K.tq1 + (size_t)tr * K.ni;
    const float* __restrict__ tw = FIXED ? nullptr : K.tw1 + (size_t)tr * K.ni;
    // U chunks per step, all their loads issued before any is used
    constexpr int U = 4;
    int64_t colg = 0;  // (column, chunk) of the group's first chunk, advanced without divisions
    int jg = 0;
    for (int64_t c0 = 0; c0 < nchunk; c0 += U) {
        float vv[U], ww[U];
        int qq[U];
        int64_t col = colg;
        int j = jg;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int iz = j * 32 + lane;
            const bool inb = c0 + u < nchunk && iz < nz;
            const int64_t ii = col * nz + iz;
            vv[u] = inb ? __ldg(m + ii) : 0.f;
            qq[u] = inb ? __ldcs(tq + ii) : -1;
            ww[u] = (!FIXED && inb) ? __ldcs(tw + ii) : 0.f;
            if (++j == cpc) {
                j = 0;
                ++col;
            }
        }
        colg = col;
        jg = j;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const float v = vv[u];
            int it = 0;
            float w = 0.f;
            const bool contrib = v != 0.f && single_entry<FIXED>(K, fp, qq[u], ww[u], it, w);
            float v0 = 0.f, v1 = 0.f;
            if (contrib) {
                v1 = v * w;
                v0 = v - v1;
            }
            warp_bin_add(trc, contrib, it, v0, v1, lane);
        }
    }
    const int c = (L - 1) / 2;
    float* __restrict__ yrow = y + (size_t)tr * nt;
    for (int n = lane; n < nt; n += 32) {
        float o;
        if (fuse) {
            const int kmin = max(0, n + c - (nt - 1));
            const int kmax = min(L - 1, n + c);
            o = 0.f;
            for (int k = kmin; k <= kmax; ++k) o = fmaf(hs[k], trc[n + c - k], o);
        } else {
            o = trc[n];
        }
        __stcs(yrow + n, o);
    }
}

// Forward: one CTA per R consecutive traces, the 64-bit fixed-point
// shared-memory accumulation of spread_kernel (order-independent, so
// deterministic), then the wavelet epilogue.
template <bool FIXED, int R>
__global__ void __launch_bounds__(kSpreadThreads, 2)
spread1_kernel(const KirchDev K, const FixedPoint<true> fp, float* __restrict__ y, const float* __restrict__ h, int L,
               int nt_pad, int fuse) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // R trace rows of 64-bit fixed-point bins (fixed_add layout)
    unsigned long long* acc = reinterpret_cast<unsigned long long*>(smem_raw);
    uint32_t* acc32 = reinterpret_cast<uint32_t*>(smem_raw);
    // the finished trace, zero-padded for fir_same, then the padded taps
    float* ftr = reinterpret_cast<float*>(acc + (size_t)R * nt_pad);
    float* hs = ftr + fir_span(L, K.nt);
    const int tid = threadIdx.x;
    const int nt = K.nt;
    const int nsnr = K.ns * K.nr;
    const int tr0 = blockIdx.x * R;
    if (tr0 >= nsnr) return;
    const int ntr = min(R, nsnr - tr0);
    fixed_clear(acc32, R, nt_pad, tid, blockDim.x);
    if (fuse) {
        for (int k = tid; k < fir_lpad(L); k += blockDim.x) hs[k] = k < L ? h[k] : 0.f;
        for (int k = tid; k < fir_span(L, K.nt); k += blockDim.x) ftr[k] = 0.f;
    }
    // |v (1 - w)| <= 2 |v| on the negative-time path: one bit of headroom
    const int e = (int)K.absmax[1];  // spread_scale_kernel
    const float S = ldexpf(1.f, e);
    __syncthreads();
    for (int64_t ii = tid; ii < K.ni; ii += blockDim.x) {
        const float v = __ldg(K.mv + ii) * S;
        if (v == 0.f) continue;
        const bool wide = fixed_wide(v, FIXED ? 1.f : 2.f);
        int q[R];
        float wf[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            q[r] = r < ntr ? __ldcs(K.tq1 + (size_t)(tr0 + r) * K.ni + ii) : -1;
            wf[r] = (!FIXED && r < ntr) ? __ldcs(K.tw1 + (size_t)(tr0 + r) * K.ni + ii) : 0.f;
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            int it;
            float w;
            if (r < ntr && single_entry<FIXED>(K, fp, q[r], wf[r], it, w)) {
                const float v1 = v * w;
                const float v0 = v - v1;
                uint32_t* row = acc32 + (size_t)r * 2 * nt_pad;
                if (wide) {
                    fixed_add_wide(row, nt_pad, it, v0);
                    fixed_add_wide(row, nt_pad, it + 1, v1);
                } else {
                    fixed_add(row, nt_pad, it, __float2int_rn(v0));
                    fixed_add(row, nt_pad, it + 1, __float2int_rn(v1));
                }
            }
        }
    }
    __syncthreads();
    const float invS = ldexpf(1.f, -e);
    float* xt = fuse ? ftr + fir_q(L) : ftr;
    for (int r = 0; r < ntr; ++r) {
        for (int n = tid; n < nt; n += blockDim.x) xt[n] = (float)fixed_get(acc32 + (size_t)r * 2 * nt_pad, nt_pad, n) * invS;
        __syncthreads();
        // convolved trace into this trace's spent accumulator row
        const float* o = xt;
        if (fuse) {
            float* os = reinterpret_cast<float*>(acc32 + (size_t)r * 2 * nt_pad);
            fir_same(hs, ftr, os, L, nt, tid, blockDim.x);
            __syncthreads();
            o = os;
        }
        float* __restrict__ yrow = y + (size_t)(tr0 + r) * nt;
        for (int n = tid; n < nt; n += blockDim.x) __stcs(yrow + n, o[n]);
        __syncthreads();
    }
}

template <bool FIXED, int R>
int spread1_launch_r(const KirchDev& K, const float* m, float* y, const float* h, int L, bool fuse, size_t smem,
                     int nt_pad, cudaStream_t stream, bool prepare_only) {
    auto kern = spread1_kernel<FIXED, R>;
    if (prepare_only) {
        KGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return KGB_OK;
    }
    int rc = launch_prepass<false>(K, m, stream, FIXED ? 1.f : 2.f);
    if (rc) return rc;
    const FixedPoint<true> fp = make_fp<true>(K.frac_bits, K.nt);
    const int64_t blocks = ((int64_t)K.ns * K.nr + R - 1) / R;
    kern<<<(unsigned)blocks, kSpreadThreads, smem, stream>>>(K, fp, y, h, L, nt_pad, fuse ? 1 : 0);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

template <bool FIXED>
int spread1_binned_launch(const KirchDev& K, const float* m, float* y, const float* h, int L, bool fuse,
                          cudaStream_t stream, bool prepare_only) {
    auto kern = spread1_binned_kernel<FIXED>;
    const int Lpad = (L + 3) & ~3;
    const int nt_pad = (K.nt + 3) & ~3;
    const int warps = 8;
    const size_t smem = (size_t)(Lpad + (size_t)warps * nt_pad) * sizeof(float);
    if (smem > 227 * 1024)
        return set_error(KGB_ERR_NOT_IMPLEMENTED, "spread: nt=%d too long for the binned variant", K.nt);
    if (prepare_only) {
        KGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return KGB_OK;
    }
    const FixedPoint<true> fp = make_fp<true>(K.frac_bits, K.nt);
    const int64_t blocks = ((int64_t)K.ns * K.nr + warps - 1) / warps;
    kern<<<(unsigned)blocks, warps * 32, smem, stream>>>(K, fp, m, y, h, L, Lpad, nt_pad, fuse ? 1 : 0);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

template <bool FIXED>
int spread1_dispatch_t(const KirchDev& K, const float* m, float* y, const float* h, int L, bool fuse,
                       cudaStream_t stream, bool prep) {
    const int Lpad = (L + 3) & ~3;
    const int nt_pad = (K.nt + 3) & ~3;
    const bool binned_fits = (size_t)(Lpad + 8 * (size_t)nt_pad) * 4 <= 227 * 1024;
    if (prep && binned_fits) {
        int rc = spread1_binned_launch<FIXED>(K, m, y, h, L, fuse, stream, true);
        if (rc) return rc;
    } else if (!prep && (K.spread_variant == 1 || K.spread_variant == 2) && binned_fits) {
        return spread1_binned_launch<FIXED>(K, m, y, h, L, fuse, stream, false);
    }
    const size_t fixed = (size_t)(fir_span(L, K.nt) + fir_lpad(L)) * sizeof(float);
    auto need = [&](int r) { return fixed + (size_t)r * nt_pad * 8; };
    int R = 8;
    while (R > 1 && need(R) > 110 * 1024) R >>= 1;
    while (R > 1 && ((int64_t)K.ns * K.nr + R - 1) / R < 2 * num_sms()) R >>= 1;
    if (need(R) > 220 * 1024)
        return set_error(KGB_ERR_NOT_IMPLEMENTED, "spread: nt=%d too long for one trace in shared memory", K.nt);
    if (prep) {  // every shape a later call may choose
        int rc = KGB_OK;
        for (int r : {8, 4, 2, 1}) {
            if (need(r) > 220 * 1024) continue;
            switch (r) {
                case 8: rc = spread1_launch_r<FIXED, 8>(K, m, y, h, L, fuse, need(8), nt_pad, stream, true); break;
                case 4: rc = spread1_launch_r<FIXED, 4>(K, m, y, h, L, fuse, need(4), nt_pad, stream, true); break;
                case 2: rc = spread1_launch_r<FIXED, 2>(K, m, y, h, L, fuse, need(2), nt_pad, stream, true); break;
                default: rc = spread1_launch_r<FIXED, 1>(K, m, y, h, L, fuse, need(1), nt_pad, stream, true);
            }
            if (rc) return rc;
        }
        return KGB_OK;
    }
    switch (R) {
        case 8: return spread1_launch_r<FIXED, 8>(K, m, y, h, L, fuse, need(8), nt_pad, stream, false);
        case 4: return spread1_launch_r<FIXED, 4>(K, m, y, h, L, fuse, need(4), nt_pad, stream, false);
        case 2: return spread1_launch_r<FIXED, 2>(K, m, y, h, L, fuse, need(2), nt_pad, stream, false);
        default: return spread1_launch_r<FIXED, 1>(K, m, y, h, L, fuse, need(1), nt_pad, stream, false);
    }
}

__global__ void sum_splits_kernel(const float* __restrict__ partial, float* __restrict__ img, int64_t ni, int nsplit) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ni; i += (int64_t)gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (int k = 0; k < nsplit; ++k) acc += partial[(size_t)k * ni + i];
        img[i] = acc;
    }
}

template <bool FIXED>
int gather1_launch_t(const KirchDev& K, const float2* d2, float* img, float* partial, int64_t cap,
                     cudaStream_t stream) {
    const FixedPoint<true> fp = make_fp<true>(K.frac_bits, K.nt);
    const int nsnr = K.ns * K.nr;
    // 4 points per thread: 16-byte table rows and float4 stores of the result
    // (the partial images are cudaMalloc'ed; the caller's image must be
    // 16-byte aligned for the unsplit case, else the scalar kernel runs)
    bool vec = K.ni % 4 == 0;
    const int64_t blocks = vec ? (K.ni / 4 + 255) / 256 : (K.ni + 255) / 256;
    // split over traces until two waves of 8 blocks per SM are resident
    int split = (int)std::max<int64_t>(1, (2 * 8 * (int64_t)num_sms() + blocks - 1) / blocks);
    split = std::min(split, std::max(1, nsnr / 64));
    if (partial == nullptr) split = 1;
    else split = (int)std::min<int64_t>(split, cap / K.ni);
    split = std::max(split, 1);
    const int per = (nsnr + split - 1) / split;
    split = (nsnr + per - 1) / per;
    float* out = split > 1 ? partial : img;
    if (((uintptr_t)out & 15) != 0) vec = false;
    dim3 grid((unsigned)(vec ? blocks : (K.ni + 255) / 256), (unsigned)split);
    if (vec) gather1_vec_kernel<FIXED><<<grid, 256, 0, stream>>>(K, fp, d2, out, per);
    else gather1_kernel<FIXED><<<grid, 256, 0, stream>>>(K, fp, d2, out, per);
    KGB_CUDA_TRY(cudaGetLastError());
    if (split > 1) {
        const int nb = (int)std::min<int64_t>((K.ni + 255) / 256, 4 * num_sms());
        sum_splits_kernel<<<nb, 256, 0, stream>>>(partial, img, K.ni, split);
        KGB_CUDA_TRY(cudaGetLastError());
    }
    return KGB_OK;
}

// taps, two padded trace buffers and the output trace
size_t wavelet_smem(int L, int nt) {
    return (size_t)(fir_lpad(L) + 2 * fir_span(L, nt) + fir_out(nt)) * sizeof(float);
}

int wavelet_threads(const float* g, int nt) {
    const int nblk = fir_out(nt) / kFirJ;
    return g ? std::min(256, (nblk + 31) / 32 * 32) : 256;
}

// Resident wavelet_kernel blocks per SM for a launch shape, cached: the
// operator's shapes are queried when its kernels are prepared, outside any
// stream capture.
int wavelet_blocks_per_sm(int threads, size_t smem) {
    struct Entry {
        int threads;
        size_t smem;
        int per_sm;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    std::lock_guard<std::mutex> lock(mu);
    for (const Entry& e : cache)
        if (e.threads == threads && e.smem == smem) return e.per_sm;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wavelet_kernel, threads, smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    cache.push_back({threads, smem, per_sm});
    return per_sm;
}

}  // namespace

int make_record_map(CUtensorMap* map, const void* records, int64_t ni, int ns, bool half) {
    tma::EncodeTiledFn fn = tma::encode_fn();
    if (!fn) return set_error(KGB_ERR_NOT_IMPLEMENTED, "record map: cuTensorMapEncodeTiled unavailable");
    // {4 words, points, sources} with one 16-byte record per point, or two
    // 8-byte bf16-weight records per 16 bytes; box: the records of one CTA's
    // kGatherThreads points of one source
    const int64_t per16 = half ? 2 : 1;
    if (!records || ni % per16 != 0 || ni / per16 > ((int64_t)1 << 31) - 1 || ns <= 0)
        return set_error(KGB_ERR_NOT_IMPLEMENTED, "record map: layout not supported");
    cuuint64_t dims[3] = {4, (cuuint64_t)(ni / per16), (cuuint64_t)ns};
    cuuint64_t strides[2] = {16, (cuuint64_t)ni * 16 / per16};
    cuuint32_t box[3] = {4, (cuuint32_t)(kGatherThreads / per16), 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<void*>(records), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(KGB_ERR_NOT_IMPLEMENTED, "record map rejected (CUresult %d)", (int)r);
    return KGB_OK;
}

int launch_spread_count(const KirchDev& K, bool dynamic, bool gate, int L, unsigned* count, cudaStream_t stream) {
    KGB_CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(unsigned), stream));
    if (K.ns <= 0 || K.nr <= 0 || K.tq1) return KGB_OK;
    if (dynamic && K.stab2) {
        if (gate) return spread_count_nn<true, true, true>(K, L, count, stream);
        return spread_count_nn<true, false, true>(K, L, count, stream);
    }
    if (dynamic) {
        if (gate) return spread_count_nn<true, true>(K, L, count, stream);
        return spread_count_nn<true, false>(K, L, count, stream);
    }
    return spread_count_nn<false, false>(K, L, count, stream);
}


int gather_nsplit(const KirchDev& K, bool dynamic, bool gate) {
    const int64_t blocks = (K.ni + kGatherThreads - 1) / kGatherThreads;
    int bps;
    if (dynamic && !gather_staged<true>(K) && gather_prefetch<true>(K)) {
        if (K.stab2)
            bps = gate ? (K.nonneg ? gather_pf_blocks_per_sm<true, true, true>() : gather_pf_blocks_per_sm<true, false, true>())
                       : (K.nonneg ? gather_pf_blocks_per_sm<false, true, true>() : gather_pf_blocks_per_sm<false, false, true>());
        else
            bps = gate ? (K.nonneg ? gather_pf_blocks_per_sm<true, true, false>() : gather_pf_blocks_per_sm<true, false, false>())
                       : (K.nonneg ? gather_pf_blocks_per_sm<false, true, false>() : gather_pf_blocks_per_sm<false, false, false>());
    } else if (dynamic && gather_staged<true>(K)) {
        if (K.stab2)
            bps = gate ? (K.nonneg ? gather_tma_blocks_per_sm<true, true, true>() : gather_tma_blocks_per_sm<true, false, true>())
                       : (K.nonneg ? gather_tma_blocks_per_sm<false, true, true>() : gather_tma_blocks_per_sm<false, false, true>());
        else
            bps = gate ? (K.nonneg ? gather_tma_blocks_per_sm<true, true, false>() : gather_tma_blocks_per_sm<true, false, false>())
                       : (K.nonneg ? gather_tma_blocks_per_sm<false, true, false>() : gather_tma_blocks_per_sm<false, false, false>());
    } else if (dynamic && K.stab2)
        bps = gate ? (K.nonneg ? gather_blocks_per_sm<true, true, true, true>() : gather_blocks_per_sm<true, true, false, true>())
                   : (K.nonneg ? gather_blocks_per_sm<true, false, true, true>() : gather_blocks_per_sm<true, false, false, true>());
    else if (dynamic) bps = gate ? (K.nonneg ? gather_blocks_per_sm<true, true, true>() : gather_blocks_per_sm<true, true, false>())
                            : (K.nonneg ? gather_blocks_per_sm<true, false, true>() : gather_blocks_per_sm<true, false, false>());
    else bps = K.nonneg ? gather_blocks_per_sm<false, false, true>() : gather_blocks_per_sm<false, false, false>();
    int split = choose_split(blocks, num_sms() * bps, K.nr);
    const int nchunks = (K.nr + kGatherRC - 1) / kGatherRC;
    const int c_per = (nchunks + split - 1) / split;
    return (nchunks + c_per - 1) / c_per;
}

int64_t gather_partial_elems(const KirchDev& K) {
    return (int64_t)std::min(kMaxSplit, (K.nr + kGatherRC - 1) / kGatherRC) * K.ni;
}

int launch_gather(const KirchDev& K, bool dynamic, bool gate, const float* d, float* img,
                  float* partial, int64_t cap, cudaStream_t stream) {
    if (K.ni <= 0 || K.ns <= 0 || K.nr <= 0) return KGB_OK;
    const float2* d2 = reinterpret_cast<const float2*>(d);
    if (K.tq1) {
        if (K.tw1) return gather1_launch_t<false>(K, d2, img, partial, cap, stream);
        return gather1_launch_t<true>(K, d2, img, partial, cap, stream);
    }
    if (dynamic && K.stab2) {
        if (gate) {
            if (K.nonneg) return gather_launch_t<true, true, true, true>(K, d2, img, partial, cap, stream);
            return gather_launch_t<true, true, false, true>(K, d2, img, partial, cap, stream);
        }
        if (K.nonneg) return gather_launch_t<true, false, true, true>(K, d2, img, partial, cap, stream);
        return gather_launch_t<true, false, false, true>(K, d2, img, partial, cap, stream);
    }
    if (dynamic) {
        if (gate) {
            if (K.nonneg) return gather_launch_t<true, true, true>(K, d2, img, partial, cap, stream);
            return gather_launch_t<true, true, false>(K, d2, img, partial, cap, stream);
        }
        if (K.nonneg) return gather_launch_t<true, false, true>(K, d2, img, partial, cap, stream);
        return gather_launch_t<true, false, false>(K, d2, img, partial, cap, stream);
    }
    if (K.nonneg) return gather_launch_t<false, false, true>(K, d2, img, partial, cap, stream);
    return gather_launch_t<false, false, false>(K, d2, img, partial, cap, stream);
}

int spread_group_size(const KirchDev& K, int L) {
    if (K.tq1 || K.spread_variant == 1 || K.spread_variant == 2 || K.ns <= 0 || K.nr <= 0 || K.nt <= 0) return 0;
    return spread_shape(K, L).R;
}

int launch_spread_prepass(const KirchDev& K, bool dynamic, const float* m, cudaStream_t stream) {
    const float wf = spread_wfactor(K.wmax, K.nonneg != 0);
    return dynamic ? launch_prepass<true>(K, m, stream, wf) : launch_prepass<false>(K, m, stream, wf);
}

int launch_spread(const KirchDev& K, bool dynamic, bool gate, const float* m, float* y,
                  const float* h, int L, bool fuse_wavelet, cudaStream_t stream) {
    if (K.ns <= 0 || K.nr <= 0 || K.nt <= 0) return KGB_OK;
    if (K.tq1) {
        if (K.tw1) return spread1_dispatch_t<false>(K, m, y, h, L, fuse_wavelet, stream, false);
        return spread1_dispatch_t<true>(K, m, y, h, L, fuse_wavelet, stream, false);
    }
    return spread_dispatch(K, dynamic, gate, m, y, h, L, fuse_wavelet, stream, false);
}

int prepare_kernels(const KirchDev& K0, int L) {
    int rc;
    KirchDev K = K0;
    for (int nn = 0; nn < 2; ++nn) {
        K.nonneg = nn;
        for (int dyn = 0; dyn < 2; ++dyn)
            for (int gate = 0; gate < 2; ++gate)
                if ((rc = spread_dispatch(K, dyn, gate, nullptr, nullptr, nullptr, L, true, nullptr, true))) return rc;
        // bf16-weight instantiations (dispatched on a non-null stab2; nothing is launched here)
        KirchDev Kh = K;
        Kh.stab2 = reinterpret_cast<const int2*>(&K);  // a non-null marker only
        for (int gate = 0; gate < 2; ++gate)
            if ((rc = spread_dispatch(Kh, 1, gate, nullptr, nullptr, nullptr, L, true, nullptr, true))) return rc;
    }
    if ((rc = spread1_dispatch_t<true>(K, nullptr, nullptr, nullptr, L, true, nullptr, true))) return rc;
    if ((rc = spread1_dispatch_t<false>(K, nullptr, nullptr, nullptr, L, true, nullptr, true))) return rc;
    const size_t smem = wavelet_smem(L, K.nt);
    if (smem <= 227 * 1024) {
        KGB_CUDA_TRY(cudaFuncSetAttribute(wavelet_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        // the launch shapes of the correlation (with the wavelet) and of the copy (without)
        wavelet_blocks_per_sm(wavelet_threads(&K.wmax, K.nt), smem);
        wavelet_blocks_per_sm(wavelet_threads(nullptr, K.nt), wavelet_smem(1, K.nt));
    }
    return KGB_OK;
}

int launch_wavelet(const float* x, float* y, int64_t ntr, int nt, const float* g, int L, int interleave,
                   cudaStream_t stream) {
    if (ntr <= 0 || nt <= 0) return KGB_OK;
    const size_t smem = wavelet_smem(L, nt);
    if (smem > 227 * 1024)
        return set_error(KGB_ERR_NOT_IMPLEMENTED, "wavelet: nt=%d too long for shared memory", nt);
    // threads: enough for the output blocks of one trace, whole warps;
    // blocks: as many as stay resident (one wave of the grid-stride loop)
    const int threads = wavelet_threads(g, nt);
    const int64_t blocks = std::min<int64_t>(ntr, (int64_t)wavelet_blocks_per_sm(threads, smem) * num_sms());
    wavelet_kernel<<<(unsigned)blocks, threads, smem, stream>>>(x, y, ntr, nt, g, L, interleave);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_pack_tables(const KirchDev& K, const float* wsc, const float* wss, const float* wrc,
                       const float* wrs, int4* stab, int4* rtab, uint32_t* srng, uint32_t* rrng,
                       cudaStream_t stream) {
    const int nb = 4 * num_sms();
    pack_tables_kernel<<<nb, 256, 0, stream>>>(K.tsq, wsc, wss, stab, (int64_t)K.ns * K.ni);
    pack_tables_kernel<<<nb, 256, 0, stream>>>(K.trq, wrc, wrs, rtab, (int64_t)K.nr * K.ni);
    const int64_t ncol = K.ni / K.nz;
    range_kernel<<<nb, 256, 0, stream>>>(wsc, wss, srng, K.ns, ncol, K.nz);
    range_kernel<<<nb, 256, 0, stream>>>(wrc, wrs, rrng, K.nr, ncol, K.nz);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_pack_tables_bf16(const KirchDev& K, const float* wsc, const float* wss, const float* wrc,
                            const float* wrs, int2* stab2, int2* rtab2, cudaStream_t stream) {
    const int nb = 4 * num_sms();
    pack_tables_bf16_kernel<<<nb, 256, 0, stream>>>(K.tsq, wsc, wss, stab2, (int64_t)K.ns * K.ni);
    pack_tables_bf16_kernel<<<nb, 256, 0, stream>>>(K.trq, wrc, wrs, rtab2, (int64_t)K.nr * K.ni);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_group_ranges(const uint32_t* rrng, uint32_t* grng, int nr, int64_t ncol, cudaStream_t stream) {
    group_range_kernel<<<4 * num_sms(), 256, 0, stream>>>(rrng, grng, nr, ncol);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

}  // namespace kgb
