// Batched Kirchhoff least-squares migration: many independent kinematic
// operators of different sizes applied, and solved with CGLS, together.
//
// The batch is the block-diagonal operator diag(K_1, ..., K_P) over the
// concatenated models and data.  Each application is one launch per kernel
// for the whole batch: the kernels walk a precomputed work list whose items
// are (problem, source, receiver group) for the forward, (problem, tile of
// image points) for the adjoint and (problem, trace) for the wavelet, so
// problems of any size share the GPU without a launch per problem.  CGLS
// (pylops/optimization/cls_basic.py:334-708) runs on every problem at once:
// per-problem float64 scalars, segmented deterministic reductions, and one
// iteration captured in a CUDA-graph WHILE node that loops until every
// problem has met its stopping rule or used its iterations.
//
// Arithmetic per problem is that of the single-operator kernels
// (kirchhoff_kernels.cu): fixed-point traveltimes, exact 64-bit fixed-point
// accumulation in the forward, fixed-order sums in the adjoint.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "fir.cuh"
#include "fixed_acc.cuh"
#include "dfacc.cuh"
#include "kgb_internal.h"

namespace kgb {
namespace bt {

constexpr int kRedThreads = 256;
constexpr int kTile = 256;      // image points per adjoint item

struct Prob {
    int ns, nr, nt, nz;
    int64_t ni;
    int F;           // fixed-point fraction bits
    int nonneg;
    int L;
    const int32_t* tsq;
    const int32_t* trq;
    const float* h;      // padded wavelet
    const float* hflip;  // reversed
    int64_t m_off;   // model offset in the concatenated model
    int64_t d_off;   // data offset in the concatenated data
    int64_t tr_off;  // first trace of this problem in the concatenated traces
};

struct SpreadItem {
    int p, is, g;
};
struct GatherItem {
    int p;
    int tile;
};
struct SegItem {  // a chunk of one problem's segment for the reductions
    int p;
    int64_t begin, end;
};

__device__ __forceinline__ bool fp_valid(int s, int F, int nt, int nonneg) {
    if (nonneg) return (unsigned)s < ((unsigned)(nt - 1) << F);
    return (unsigned)s + ((1u << F) - 1u) < (((unsigned)nt << F) - 1u);
}
__device__ __forceinline__ int fp_index(int s, int F, int nonneg) {
    return nonneg ? (int)((unsigned)s >> F) : (max(s, 0) >> F);
}
__device__ __forceinline__ float fp_frac(int s, int it, int F) {
    return (float)(s - (it << F)) * __int_as_float((127 - F) << 23);
}

// ---------------------------------------------------------------- forward
__global__ void __launch_bounds__(256)
absmax_kernel(const float* __restrict__ m, int64_t n, unsigned* __restrict__ out) {
    float a = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a = fmaxf(a, fabsf(m[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
    if ((threadIdx.x & 31) == 0 && a > 0.f) atomicMax(out, __float_as_uint(a));
}

// One CTA per item (problem, source, group of R receivers): the same
// fixed-point shared-memory accumulation and fused wavelet epilogue as the
// single-operator forward.
template <int R>
__global__ void __launch_bounds__(256)
batch_spread_kernel(const Prob* __restrict__ probs, const SpreadItem* __restrict__ items, const float* __restrict__ m,
                    float* __restrict__ y, const unsigned* __restrict__ absmax, int nt_pad_max,
                    int span_max) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const SpreadItem it_ = items[blockIdx.x];
    const Prob P = probs[it_.p];
    const int nt_pad = (P.nt + 3) & ~3;
    // R trace rows of 64-bit fixed-point bins (fixed_add layout)
    unsigned long long* acc = reinterpret_cast<unsigned long long*>(smem_raw);
    uint32_t* acc32 = reinterpret_cast<uint32_t*>(smem_raw);
    // the finished trace, zero-padded for fir_same, then the padded taps
    float* ftr = reinterpret_cast<float*>(acc + (size_t)R * nt_pad_max);
    float* hs = ftr + span_max;
    const int tid = threadIdx.x;
    const int r0 = it_.g * R;
    const int nrr = min(R, P.nr - r0);
    fixed_clear(acc32, R, nt_pad, tid, blockDim.x);
    for (int k = tid; k < fir_lpad(P.L); k += blockDim.x) hs[k] = k < P.L ? P.h[k] : 0.f;
    for (int k = tid; k < fir_span(P.L, P.nt); k += blockDim.x) ftr[k] = 0.f;
    const int e = fixed_scale_exponent(__uint_as_float(*absmax));
    const float S = ldexpf(1.f, e);
    __syncthreads();
    const float* __restrict__ mp = m + P.m_off;
    const int32_t* __restrict__ tsrow = P.tsq + (size_t)it_.is * P.ni;
    for (int64_t ii = tid; ii < P.ni; ii += blockDim.x) {
        const float v = __ldg(mp + ii) * S;
        if (v == 0.f) continue;
        const int ts = __ldg(tsrow + ii);
        int tr[R];
#pragma unroll
        for (int r = 0; r < R; ++r) tr[r] = r < nrr ? __ldg(P.trq + (size_t)(r0 + r) * P.ni + ii) : 0;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (r < nrr) {
                const int s = ts + tr[r];
                if (fp_valid(s, P.F, P.nt, P.nonneg)) {
                    const int t = fp_index(s, P.F, P.nonneg);
                    const float w = fp_frac(s, t, P.F);
                    const float v1 = v * w;
                    const float v0 = v - v1;
                    uint32_t* row = acc32 + (size_t)r * 2 * nt_pad;
                    fixed_add(row, nt_pad, t, __float2int_rn(v0));
                    fixed_add(row, nt_pad, t + 1, __float2int_rn(v1));
                }
            }
        }
    }
    __syncthreads();
    const float invS = ldexpf(1.f, -e);
    float* xt = ftr + fir_q(P.L);
    for (int r = 0; r < nrr; ++r) {
        for (int n = tid; n < P.nt; n += blockDim.x) xt[n] = (float)fixed_get(acc32 + (size_t)r * 2 * nt_pad, nt_pad, n) * invS;
        __syncthreads();
        // convolved trace into this receiver's spent accumulator row
        float* os = reinterpret_cast<float*>(acc32 + (size_t)r * 2 * nt_pad);
        fir_same(hs, ftr, os, P.L, P.nt, tid, blockDim.x);
        __syncthreads();
        float* __restrict__ yrow = y + P.d_off + ((size_t)it_.is * P.nr + r0 + r) * P.nt;
        for (int n = tid; n < P.nt; n += blockDim.x) yrow[n] = os[n];
        __syncthreads();
    }
}

// ---------------------------------------------------------------- adjoint
// Correlation with the reversed wavelet, one CTA per trace of the batch,
// written as interleaved pairs (d[t], d[t+1]) for the gather.
__global__ void __launch_bounds__(256)
batch_correlate_kernel(const Prob* __restrict__ probs, int nprob, const float* __restrict__ d, float2* __restrict__ dc,
                       int64_t ntraces, int span_max, int Lpad_max) {
    extern __shared__ __align__(16) float smem[];
    float* gs = smem;
    float* xp = smem + Lpad_max;  // zero-padded trace
    float* os = xp + span_max;
    for (int64_t tr = blockIdx.x; tr < ntraces; tr += gridDim.x) {
        // problem of this trace: binary search over the trace offsets
        int lo = 0, hi = nprob - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (probs[mid].tr_off <= tr) lo = mid;
            else hi = mid - 1;
        }
        const Prob& P = probs[lo];
        __syncthreads();
        for (int k = threadIdx.x; k < fir_lpad(P.L); k += blockDim.x) gs[k] = k < P.L ? P.hflip[k] : 0.f;
        const int64_t local = tr - P.tr_off;
        const float* xrow = d + P.d_off + local * P.nt;
        const int q = fir_q(P.L);
        for (int i = threadIdx.x; i < fir_span(P.L, P.nt); i += blockDim.x)
            xp[i] = (i >= q && i < q + P.nt) ? xrow[i - q] : 0.f;
        __syncthreads();
        fir_same(gs, xp, os, P.L, P.nt, threadIdx.x, blockDim.x);
        __syncthreads();
        float2* yrow = dc + P.d_off + local * P.nt;
        for (int n = threadIdx.x; n < P.nt; n += blockDim.x)
            yrow[n] = make_float2(os[n], n + 1 < P.nt ? os[n + 1] : 0.f);
    }
}

// Adjoint: one CTA per (problem, tile) item of the work list, one launch for
// the whole batch; a tile is kTile * PPT image points, each thread sums PPT
// of them (kTile apart) over all traces of its problem in a fixed order,
// with RC receiver traveltimes per point in registers.  (A persistent grid
// walking the list costs the loop's registers: ~200 bytes of spills at the
// 32-register budget that keeps the SM's 64 warps resident.)
// RC and PPT are chosen per batch by the autotuner (kgb_batch_set_gather):
// more points per thread put more independent record -> data load chains
// in flight per thread, more receivers in registers read the source
// traveltimes fewer times; both cost registers and so resident warps.
template <int RC, int PPT>
__global__ void __launch_bounds__(kTile, 8 / PPT)
batch_gather_kernel(const Prob* __restrict__ probs, const GatherItem* __restrict__ items, int nitems,
                    const float2* __restrict__ dc, float* __restrict__ img) {
    {
        const int item = blockIdx.x;
        if (item >= nitems) return;
        const GatherItem it_ = items[item];
        const Prob& P = probs[it_.p];
        const int ni = (int)P.ni, ns = P.ns, nr = P.nr, nt = P.nt, F = P.F, nonneg = P.nonneg;
        const int i0 = it_.tile * PPT * kTile + (int)threadIdx.x;  // first point of this thread (problem-local)
        if (i0 >= ni) return;
        const int32_t* __restrict__ tsq = P.tsq;
        const int32_t* __restrict__ trq = P.trq;
        const float2* __restrict__ d2 = dc + P.d_off;
        float total[PPT];
#pragma unroll
        for (int q = 0; q < PPT; ++q) total[q] = 0.f;
        for (int r0 = 0; r0 < nr; r0 += RC) {
            int tr[PPT][RC];
            const int nrc = min(RC, nr - r0);
#pragma unroll
            for (int q = 0; q < PPT; ++q)
#pragma unroll
                for (int r = 0; r < RC; ++r) {
                    const int ii = i0 + q * kTile;
                    tr[q][r] = (r < nrc && ii < ni) ? __ldg(trq + (size_t)(r0 + r) * ni + ii) : 0;
                }
            float chunk[PPT];
#pragma unroll
            for (int q = 0; q < PPT; ++q) chunk[q] = 0.f;
            for (int is = 0; is < ns; ++is) {
                const float2* __restrict__ drow = d2 + ((size_t)is * nr + r0) * nt;
#pragma unroll
                for (int q = 0; q < PPT; ++q) {
                    const int ii = i0 + q * kTile;
                    if (ii >= ni) continue;
                    const int ts = __ldg(tsq + (size_t)is * ni + ii);
#pragma unroll
                    for (int r = 0; r < RC; ++r) {
                        if (r < nrc) {
                            const int s = ts + tr[q][r];
                            if (fp_valid(s, F, nt, nonneg)) {
                                const int t = fp_index(s, F, nonneg);
                                const float w = fp_frac(s, t, F);
                                const float2 dd = __ldg(drow + ((size_t)r * nt + t));
                                chunk[q] += fmaf(w, dd.y - dd.x, dd.x);
                            }
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < PPT; ++q) total[q] += chunk[q];
        }
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            const int ii = i0 + q * kTile;
            if (ii < ni) img[P.m_off + ii] = total[q];
        }
    }
}

// ---------------------------------------------------------------- CGLS
struct CglsState {
    double kold, k, a, b, damp, dampsq, tol;
    int iiter, target, active;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ double block_sum(double v) {
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    if (warp == 0) v = warp_sum(v);
    __syncthreads();
    return v;
}

// op codes of the fused segmented vector kernel
enum SegOp {
    OP_SQ = 0,       // partial = sum a^2
    OP_X = 1,        // x += a_p c; partial = sum x^2
    OP_S = 2,        // s -= a_p q; partial = sum s^2
    OP_R = 3,        // r -= damp_p x; partial = sum r^2
    OP_C = 4,        // c = r + b_p c
};

__global__ void __launch_bounds__(kRedThreads)
seg_kernel(const SegItem* __restrict__ items, int op, float* __restrict__ u, const float* __restrict__ w,
           const CglsState* __restrict__ st, double* __restrict__ partials) {
    const SegItem it_ = items[blockIdx.x];
    const CglsState S = st[it_.p];
    DFAcc dacc;
    if (S.active) {
        const float a = (float)S.a, b = (float)S.b, dsq = (float)S.dampsq;
        for (int64_t i = it_.begin + threadIdx.x; i < it_.end; i += blockDim.x) {
            float v = u[i];
            switch (op) {
                case OP_X: v = v + a * w[i]; u[i] = v; break;
                case OP_S: v = v - a * w[i]; u[i] = v; break;
                case OP_R: v = v - dsq * w[i]; u[i] = v; break;
                case OP_C: v = w[i] + b * v; u[i] = v; break;
                default: break;
            }
            dacc.add_prod(v, v);
        }
    }
    if (op == OP_C) return;
    double acc = block_sum(dacc.value());
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// per-problem fixed-order sum of the item partials [first[p], first[p+1])
__device__ double prob_sum(const double* __restrict__ partials, const int* __restrict__ first, int p) {
    double s = 0.0;
    for (int k = first[p]; k < first[p + 1]; ++k) s += partials[k];
    return s;
}

// a = kold / (q.q + damp c.c)   (cls_basic.py:525-527)
__global__ void cgls_a_kernel(CglsState* st, int nprob, const double* pq, const int* fq, const double* pc,
                              const int* fc) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nprob || !st[p].active) return;
    const double qq = prob_sum(pq, fq, p), cc = prob_sum(pc, fc, p);
    st[p].a = st[p].kold / (qq + st[p].dampsq * cc);
}

// k = r.r, b = k/kold, cost histories (cls_basic.py:542-564)
__global__ void cgls_b_kernel(CglsState* st, int nprob, const double* pr, const int* fr, const double* ps,
                              const int* fs, const double* px, const int* fx, double* cost, double* cost1,
                              int cost_stride) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nprob || !st[p].active) return;
    const double k = prob_sum(pr, fr, p), ss = prob_sum(ps, fs, p), xx = prob_sum(px, fx, p);
    st[p].k = k;
    st[p].b = k / st[p].kold;
    const int i = st[p].iiter + 1;
    cost[(size_t)p * cost_stride + i] = sqrt(ss);
    cost1[(size_t)p * cost_stride + i] = sqrt(ss + st[p].dampsq * fabs(xx));
}

// kold = k; iteration count; stopping rule (cls_basic.py:599); then the
// graph condition: is any problem still active?
__global__ void __launch_bounds__(256)
cgls_tail_kernel(CglsState* st, int nprob, cudaGraphConditionalHandle h, int use_handle) {
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int p = threadIdx.x; p < nprob; p += blockDim.x) {
        CglsState S = st[p];
        if (S.active) {
            S.kold = S.k;
            S.iiter += 1;
            S.active = (S.iiter < S.target && S.kold > S.tol) ? 1 : 0;
            st[p] = S;
        }
        if (S.active) any = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0 && use_handle) cudaGraphSetConditional(h, any ? 1u : 0u);
}

// before a run: every problem may take niter more iterations
__global__ void cgls_target_kernel(CglsState* st, int nprob, int niter) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nprob) return;
    st[p].target = st[p].iiter + niter;
    st[p].active = (st[p].iiter < st[p].target && st[p].kold > st[p].tol) ? 1 : 0;
}

__global__ void __launch_bounds__(256)
cgls_cond_kernel(const CglsState* st, int nprob, cudaGraphConditionalHandle h) {
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int p = threadIdx.x; p < nprob; p += blockDim.x)
        if (st[p].active) any = 1;
    __syncthreads();
    if (threadIdx.x == 0) cudaGraphSetConditional(h, any ? 1u : 0u);
}

// setup: kold = c.c, cost[0] = ||s||, cost1[0] (x0 = 0)  (cls_basic.py:474-503)
__global__ void cgls_setup_kernel(CglsState* st, int nprob, const double* pc, const int* fc, const double* ps,
                                  const int* fs, double* cost, double* cost1, int cost_stride, double damp,
                                  double tol) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nprob) return;
    CglsState S;
    S.kold = fabs(prob_sum(pc, fc, p));
    S.k = 0.0;
    S.a = S.b = 0.0;
    S.damp = damp;
    S.dampsq = damp * damp;
    S.tol = tol;
    S.iiter = 0;
    S.target = 0;
    S.active = 1;  // the setup's sums run for every problem
    const double ss = prob_sum(ps, fs, p);
    cost[(size_t)p * cost_stride] = sqrt(ss);
    cost1[(size_t)p * cost_stride] = sqrt(ss);
    st[p] = S;
}

}  // namespace bt
}  // namespace kgb

using namespace kgb;
using namespace kgb::bt;

struct kgb_batch {
    std::vector<kgb_kirchhoff*> ops;
    int nprob = 0;
    int64_t nm = 0, nd = 0, ntraces = 0;
    int nt_pad_max = 0, Lpad_max = 0;  // Lpad_max: padded taps (fir_lpad)
    int span_max = 0, out_max = 0;     // padded trace and FIR output floats
    int R = 8;  // receivers per forward item (autotuned)
    Prob* d_probs = nullptr;
    SpreadItem* d_spread[4] = {nullptr, nullptr, nullptr, nullptr};  // R = 1, 2, 4, 8
    int n_spread[4] = {0, 0, 0, 0};
    // adjoint work lists for 1 and 2 image points per thread, and the
    // autotuned shape: receivers in registers (4 or 8), points per thread
    GatherItem* d_gather[2] = {nullptr, nullptr};
    int n_gather[2] = {0, 0};
    int grc = 8, gppt = 1;
    SegItem* d_mseg = nullptr;
    SegItem* d_dseg = nullptr;
    int n_mseg = 0, n_dseg = 0;
    int* d_fm = nullptr;  // first model item of each problem (nprob+1)
    int* d_fd = nullptr;
    float2* dc = nullptr;   // correlated data, interleaved
    unsigned* absmax = nullptr;
    // CGLS
    float *x = nullptr, *c = nullptr, *r = nullptr, *sv = nullptr, *q = nullptr;
    double* partials = nullptr;  // 5 arrays: q, c, x, s, r
    CglsState* st = nullptr;
    double *cost = nullptr, *cost1 = nullptr;
    int cost_stride = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphConditionalHandle handle = 0;
};

namespace {

int r_index(int R) { return R == 1 ? 0 : R == 2 ? 1 : R == 4 ? 2 : 3; }

size_t spread_smem(const kgb_batch* b, int R) {
    return (size_t)R * b->nt_pad_max * 8 + (size_t)(b->span_max + b->Lpad_max) * 4;
}

size_t correlate_smem(const kgb_batch* b) { return (size_t)(b->Lpad_max + b->span_max + b->out_max) * 4; }

int batch_forward(kgb_batch* b, const float* m, float* y, cudaStream_t s) {
    KGB_CUDA_TRY(cudaMemsetAsync(b->absmax, 0, sizeof(unsigned), s));
    absmax_kernel<<<4 * 152, 256, 0, s>>>(m, b->nm, b->absmax);
    const int ri = r_index(b->R);
    const size_t smem = spread_smem(b, b->R);
    switch (b->R) {
        case 1: batch_spread_kernel<1><<<b->n_spread[ri], 256, smem, s>>>(b->d_probs, b->d_spread[ri], m, y, b->absmax, b->nt_pad_max, b->span_max); break;
        case 2: batch_spread_kernel<2><<<b->n_spread[ri], 256, smem, s>>>(b->d_probs, b->d_spread[ri], m, y, b->absmax, b->nt_pad_max, b->span_max); break;
        case 4: batch_spread_kernel<4><<<b->n_spread[ri], 256, smem, s>>>(b->d_probs, b->d_spread[ri], m, y, b->absmax, b->nt_pad_max, b->span_max); break;
        default: batch_spread_kernel<8><<<b->n_spread[ri], 256, smem, s>>>(b->d_probs, b->d_spread[ri], m, y, b->absmax, b->nt_pad_max, b->span_max); break;
    }
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int batch_adjoint(kgb_batch* b, const float* d, float* img, cudaStream_t s) {
    const size_t smem = correlate_smem(b);
    const int64_t nb = std::min<int64_t>(b->ntraces, 8 * 152);
    batch_correlate_kernel<<<(unsigned)nb, 256, smem, s>>>(b->d_probs, b->nprob, d, b->dc, b->ntraces, b->span_max,
                                                          b->Lpad_max);
    const int k = (b->grc == 8 ? 2 : 0) + (b->gppt == 2 ? 1 : 0);
    const int n = b->n_gather[b->gppt - 1];
    const GatherItem* items = b->d_gather[b->gppt - 1];
    const int grid = std::max(1, n);
    switch (k) {
        case 0: batch_gather_kernel<4, 1><<<grid, kTile, 0, s>>>(b->d_probs, items, n, b->dc, img); break;
        case 1: batch_gather_kernel<4, 2><<<grid, kTile, 0, s>>>(b->d_probs, items, n, b->dc, img); break;
        case 2: batch_gather_kernel<8, 1><<<grid, kTile, 0, s>>>(b->d_probs, items, n, b->dc, img); break;
        default: batch_gather_kernel<8, 2><<<grid, kTile, 0, s>>>(b->d_probs, items, n, b->dc, img); break;
    }
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}


template <typename T>
int upload(T** dst, const std::vector<T>& v) {
    KGB_CUDA_TRY(cudaMalloc(dst, std::max<size_t>(1, v.size()) * sizeof(T)));
    if (!v.empty()) KGB_CUDA_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return KGB_OK;
}

// chunk each problem's segment of length len_p into items of at most `chunk`
void seg_items(const std::vector<int64_t>& off, const std::vector<int64_t>& len, int64_t chunk,
               std::vector<SegItem>& items, std::vector<int>& first) {
    first.assign(off.size() + 1, 0);
    for (size_t p = 0; p < off.size(); ++p) {
        first[p] = (int)items.size();
        for (int64_t b = 0; b < len[p]; b += chunk) items.push_back({(int)p, off[p] + b, off[p] + std::min(len[p], b + chunk)});
    }
    first[off.size()] = (int)items.size();
}

int enqueue_cgls_iteration(kgb_batch* b, cudaStream_t s, int use_handle) {
    double* Pq = b->partials;
    double* Pc = Pq + b->n_dseg;
    double* Px = Pc + b->n_mseg;
    double* Ps = Px + b->n_mseg;
    double* Pr = Ps + b->n_dseg;
    const int pb = (b->nprob + 127) / 128;
    seg_kernel<<<b->n_dseg, kRedThreads, 0, s>>>(b->d_dseg, OP_SQ, b->q, nullptr, b->st, Pq);
    seg_kernel<<<b->n_mseg, kRedThreads, 0, s>>>(b->d_mseg, OP_SQ, b->c, nullptr, b->st, Pc);
    cgls_a_kernel<<<pb, 128, 0, s>>>(b->st, b->nprob, Pq, b->d_fd, Pc, b->d_fm);
    seg_kernel<<<b->n_mseg, kRedThreads, 0, s>>>(b->d_mseg, OP_X, b->x, b->c, b->st, Px);
    seg_kernel<<<b->n_dseg, kRedThreads, 0, s>>>(b->d_dseg, OP_S, b->sv, b->q, b->st, Ps);
    int rc;
    if ((rc = batch_adjoint(b, b->sv, b->r, s))) return rc;
    seg_kernel<<<b->n_mseg, kRedThreads, 0, s>>>(b->d_mseg, OP_R, b->r, b->x, b->st, Pr);
    cgls_b_kernel<<<pb, 128, 0, s>>>(b->st, b->nprob, Pr, b->d_fm, Ps, b->d_fd, Px, b->d_fm, b->cost, b->cost1,
                                     b->cost_stride);
    seg_kernel<<<b->n_mseg, kRedThreads, 0, s>>>(b->d_mseg, OP_C, b->c, b->r, b->st, nullptr);
    if ((rc = batch_forward(b, b->c, b->q, s))) return rc;
    cgls_tail_kernel<<<1, 256, 0, s>>>(b->st, b->nprob, b->handle, use_handle);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int build_cgls_graph(kgb_batch* b, cudaStream_t s) {
    if (b->exec) return KGB_OK;
    cudaGraph_t g = nullptr;
    KGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(e, "batch: cudaGraphConditionalHandleCreate"); }
    b->handle = h;
    e = cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(e, "batch: capture init"); }
    cgls_cond_kernel<<<1, 256, 0, s>>>(b->st, b->nprob, h);
    cudaGraph_t tmp;
    e = cudaStreamEndCapture(s, &tmp);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(e, "batch: capture init end"); }
    cudaGraphNode_t init = nullptr;
    size_t nn = 1;
    e = cudaGraphGetNodes(g, &init, &nn);
    if (e != cudaSuccess || nn != 1) { cudaGraphDestroy(g); return set_error(KGB_ERR_CUDA, "batch: graph init node"); }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode;
    e = cudaGraphAddNode(&wnode, g, &init, nullptr, 1, &cp);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(e, "batch: cudaGraphAddNode(while)"); }
    e = cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(e, "batch: capture body"); }
    int rc = enqueue_cgls_iteration(b, s, 1);
    cudaGraph_t body;
    e = cudaStreamEndCapture(s, &body);
    if (rc) { cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(e, "batch: capture body end"); }
    e = cudaGraphInstantiate(&b->exec, g, 0);
    if (e != cudaSuccess) { cudaGraphDestroy(g); b->exec = nullptr; return cuda_error(e, "batch: instantiate"); }
    b->graph = g;
    return KGB_OK;
}

}  // namespace

extern "C" {

int kgb_batch_create(kgb_batch** out, kgb_kirchhoff* const* ops, int nops) {
    if (!out || !ops || nops <= 0) return set_error(KGB_ERR_VALUE, "batch_create: no operators");
    *out = nullptr;
    kgb_batch* b = new kgb_batch();
    b->nprob = nops;
    std::vector<Prob> probs(nops);
    std::vector<int64_t> moff(nops), mlen(nops), doff(nops), dlen(nops);
    for (int p = 0; p < nops; ++p) {
        kgb_kirchhoff* op = ops[p];
        if (!op || !op->trav_ready) { delete b; return set_error(KGB_ERR_STATE, "batch_create: operator %d has no tables", p); }
        if (op->dynamic) { delete b; return set_error(KGB_ERR_NOT_IMPLEMENTED, "batch_create: operator %d is dynamic; the batch runs kinematic operators", p); }
        b->ops.push_back(op);
        Prob& P = probs[p];
        P.ns = op->ns; P.nr = op->nr; P.nt = op->nt; P.nz = op->nz; P.ni = op->ni;
        P.F = op->frac_bits; P.nonneg = op->nonneg ? 1 : 0; P.L = op->L;
        P.tsq = op->tsq; P.trq = op->trq; P.h = op->h_dev; P.hflip = op->hflip_dev;
        P.m_off = b->nm; P.d_off = b->nd; P.tr_off = b->ntraces;
        moff[p] = b->nm; mlen[p] = op->ni; doff[p] = b->nd; dlen[p] = op->ndata();
        b->nm += op->ni;
        b->nd += op->ndata();
        b->ntraces += op->npair();
        b->nt_pad_max = std::max(b->nt_pad_max, (op->nt + 3) & ~3);
        b->Lpad_max = std::max(b->Lpad_max, fir_lpad(op->L));
        b->span_max = std::max(b->span_max, fir_span(op->L, op->nt));
        b->out_max = std::max(b->out_max, fir_out(op->nt));
    }
    int rc = KGB_OK;
    do {
        if ((rc = upload(&b->d_probs, probs))) break;
        const int Rs[4] = {1, 2, 4, 8};
        for (int k = 0; k < 4 && !rc; ++k) {
            std::vector<SpreadItem> items;
            for (int p = 0; p < nops; ++p) {
                const int ng = (probs[p].nr + Rs[k] - 1) / Rs[k];
                for (int g = 0; g < ng; ++g)
                    for (int is = 0; is < probs[p].ns; ++is) items.push_back({p, is, g});
            }
            b->n_spread[k] = (int)items.size();
            rc = upload(&b->d_spread[k], items);
        }
        if (rc) break;
        for (int ppt = 1; ppt <= 2 && !rc; ++ppt) {
            std::vector<GatherItem> gi;
            for (int p = 0; p < nops; ++p)
                for (int64_t t = 0; t * kTile * ppt < probs[p].ni; ++t) gi.push_back({p, (int)t});
            b->n_gather[ppt - 1] = (int)gi.size();
            rc = upload(&b->d_gather[ppt - 1], gi);
        }
        if (rc) break;
        std::vector<SegItem> ms, ds;
        std::vector<int> fm, fd;
        seg_items(moff, mlen, 8192, ms, fm);
        seg_items(doff, dlen, 65536, ds, fd);
        b->n_mseg = (int)ms.size();
        b->n_dseg = (int)ds.size();
        if ((rc = upload(&b->d_mseg, ms)) || (rc = upload(&b->d_dseg, ds)) || (rc = upload(&b->d_fm, fm)) ||
            (rc = upload(&b->d_fd, fd)))
            break;
        cudaError_t e = cudaMalloc(&b->dc, (size_t)b->nd * sizeof(float2));
        if (e == cudaSuccess) e = cudaMalloc(&b->absmax, sizeof(unsigned));
        if (e != cudaSuccess) { rc = cuda_error(e, "batch_create: scratch"); break; }
        const size_t smem8 = spread_smem(b, 8);
        if (smem8 > 227 * 1024) { rc = set_error(KGB_ERR_NOT_IMPLEMENTED, "batch_create: nt too long"); break; }
        KGB_CUDA_TRY(cudaFuncSetAttribute(batch_spread_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spread_smem(b, 1)));
        KGB_CUDA_TRY(cudaFuncSetAttribute(batch_spread_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spread_smem(b, 2)));
        KGB_CUDA_TRY(cudaFuncSetAttribute(batch_spread_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spread_smem(b, 4)));
        KGB_CUDA_TRY(cudaFuncSetAttribute(batch_spread_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem8));
        KGB_CUDA_TRY(cudaFuncSetAttribute(batch_correlate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)correlate_smem(b)));
    } while (0);
    if (rc) {
        kgb_batch_destroy(b);
        return rc;
    }
    *out = b;
    return KGB_OK;
}

int kgb_batch_destroy(kgb_batch* b) {
    if (!b) return KGB_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    void* ptrs[] = {b->d_probs, b->d_spread[0], b->d_spread[1], b->d_spread[2], b->d_spread[3], b->d_gather[0],
                    b->d_gather[1],
                    b->d_mseg, b->d_dseg, b->d_fm, b->d_fd, b->dc, b->absmax, b->x, b->c, b->r, b->sv, b->q,
                    b->partials, b->st, b->cost, b->cost1};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete b;
    return KGB_OK;
}

int kgb_batch_sizes(const kgb_batch* b, int64_t* sizes4) {
    if (!b || !sizes4) return set_error(KGB_ERR_VALUE, "batch_sizes: null pointer");
    sizes4[0] = b->nprob; sizes4[1] = b->nm; sizes4[2] = b->nd; sizes4[3] = b->R;
    return KGB_OK;
}

int kgb_batch_set_tile(kgb_batch* b, int receivers_per_item) {
    if (!b) return set_error(KGB_ERR_VALUE, "batch_set_tile: null batch");
    const int R = receivers_per_item;
    if (R != 1 && R != 2 && R != 4 && R != 8) return set_error(KGB_ERR_VALUE, "batch_set_tile: receivers per item must be 1, 2, 4 or 8");
    b->R = R;
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
    if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
    return KGB_OK;
}

int kgb_batch_set_gather(kgb_batch* b, int receivers_in_registers, int points_per_thread) {
    if (!b) return set_error(KGB_ERR_VALUE, "batch_set_gather: null batch");
    if ((receivers_in_registers != 4 && receivers_in_registers != 8) || (points_per_thread != 1 && points_per_thread != 2))
        return set_error(KGB_ERR_VALUE, "batch_set_gather: receivers in registers 4 or 8, points per thread 1 or 2");
    b->grc = receivers_in_registers;
    b->gppt = points_per_thread;
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
    if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
    return KGB_OK;
}

int kgb_batch_forward(kgb_batch* b, const float* m, float* d, void* stream) {
    if (!b || !m || !d) return set_error(KGB_ERR_VALUE, "batch_forward: null pointer");
    return batch_forward(b, m, d, (cudaStream_t)stream);
}

int kgb_batch_adjoint(kgb_batch* b, const float* d, float* m, void* stream) {
    if (!b || !m || !d) return set_error(KGB_ERR_VALUE, "batch_adjoint: null pointer");
    return batch_adjoint(b, d, m, (cudaStream_t)stream);
}

int kgb_batch_cgls(kgb_batch* b, const float* y, float* x_out, int niter, double damp, double tol, int use_graph,
                   double* cost_host, int* iiter_host, double* kold_host, void* stream_) {
    if (!b || !y || !x_out) return set_error(KGB_ERR_VALUE, "batch_cgls: null pointer");
    if (niter < 0) return set_error(KGB_ERR_VALUE, "batch_cgls: niter must be >= 0");
    cudaStream_t s = (cudaStream_t)stream_;
    cudaError_t e = cudaSuccess;
    auto A = [&](float** p, int64_t n) { if (!*p && e == cudaSuccess) e = cudaMalloc(p, (size_t)n * 4); };
    A(&b->x, b->nm); A(&b->c, b->nm); A(&b->r, b->nm); A(&b->sv, b->nd); A(&b->q, b->nd);
    if (!b->partials && e == cudaSuccess) e = cudaMalloc(&b->partials, (size_t)(2 * b->n_dseg + 3 * b->n_mseg) * 8);
    if (!b->st && e == cudaSuccess) e = cudaMalloc(&b->st, (size_t)b->nprob * sizeof(CglsState));
    if (b->cost_stride < niter + 1) {
        if (b->cost) { cudaFree(b->cost); cudaFree(b->cost1); b->cost = b->cost1 = nullptr; }
        b->cost_stride = niter + 1;
        if (e == cudaSuccess) e = cudaMalloc(&b->cost, (size_t)b->nprob * b->cost_stride * 8);
        if (e == cudaSuccess) e = cudaMalloc(&b->cost1, (size_t)b->nprob * b->cost_stride * 8);
        if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
        if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
    }
    if (e != cudaSuccess) return cuda_error(e, "batch_cgls: allocation");
    // setup (x0 = 0): s = y, c = K^H s, q = K c, kold = c.c
    KGB_CUDA_TRY(cudaMemsetAsync(b->x, 0, (size_t)b->nm * 4, s));
    KGB_CUDA_TRY(cudaMemcpyAsync(b->sv, y, (size_t)b->nd * 4, cudaMemcpyDeviceToDevice, s));
    int rc;
    if ((rc = batch_adjoint(b, b->sv, b->c, s))) return rc;
    if ((rc = batch_forward(b, b->c, b->q, s))) return rc;
    // plain sums of squares (all problems): mark every problem active for them
    double* Pc = b->partials + b->n_dseg;
    double* Ps = b->partials + b->n_dseg + 2 * b->n_mseg;
    {
        // a state with every problem active so seg_kernel runs
        std::vector<CglsState> init(b->nprob);
        for (auto& S : init) { S = CglsState{}; S.active = 1; }
        KGB_CUDA_TRY(cudaMemcpyAsync(b->st, init.data(), init.size() * sizeof(CglsState), cudaMemcpyHostToDevice, s));
        KGB_CUDA_TRY(cudaStreamSynchronize(s));
    }
    seg_kernel<<<b->n_mseg, kRedThreads, 0, s>>>(b->d_mseg, OP_SQ, b->c, nullptr, b->st, Pc);
    seg_kernel<<<b->n_dseg, kRedThreads, 0, s>>>(b->d_dseg, OP_SQ, b->sv, nullptr, b->st, Ps);
    const int pb = (b->nprob + 127) / 128;
    cgls_setup_kernel<<<pb, 128, 0, s>>>(b->st, b->nprob, Pc, b->d_fm, Ps, b->d_fd, b->cost, b->cost1, b->cost_stride,
                                         damp, tol);
    cgls_target_kernel<<<pb, 128, 0, s>>>(b->st, b->nprob, niter);
    KGB_CUDA_TRY(cudaGetLastError());
    if (use_graph && s != nullptr) {
        if ((rc = build_cgls_graph(b, s))) return rc;
        KGB_CUDA_TRY(cudaGraphLaunch(b->exec, s));
    } else {
        for (int k = 0; k < niter; ++k)
            if ((rc = enqueue_cgls_iteration(b, s, 0))) return rc;
    }
    KGB_CUDA_TRY(cudaMemcpyAsync(x_out, b->x, (size_t)b->nm * 4, cudaMemcpyDeviceToDevice, s));
    std::vector<CglsState> hs(b->nprob);
    KGB_CUDA_TRY(cudaMemcpyAsync(hs.data(), b->st, hs.size() * sizeof(CglsState), cudaMemcpyDeviceToHost, s));
    if (cost_host)  // host rows hold niter+1 values; device rows cost_stride >= niter+1
        KGB_CUDA_TRY(cudaMemcpy2DAsync(cost_host, (size_t)(niter + 1) * 8, b->cost, (size_t)b->cost_stride * 8,
                                       (size_t)(niter + 1) * 8, (size_t)b->nprob, cudaMemcpyDeviceToHost, s));
    KGB_CUDA_TRY(cudaStreamSynchronize(s));
    for (int p = 0; p < b->nprob; ++p) {
        if (iiter_host) iiter_host[p] = hs[p].iiter;
        if (kold_host) kold_host[p] = hs[p].kold;
    }
    return KGB_OK;
}

}  // extern "C"
