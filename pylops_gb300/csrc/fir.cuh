// 'same'-mode FIR along time on a trace staged in shared memory,
//   o[n] = sum_{k=0}^{L-1} g[k] x[n + c - k],  c = (L-1)/2,  n in [0, nt),
// the trace convolution of Kirchhoff (Convolve1D over the time axis,
// kirchhoff.py:407-408, 1093, 1099), with the wavelet padded on the host so
// that its centre sits at c.
//
// Register blocking: a thread produces kFirJ consecutive outputs and walks
// the taps kFirJ at a time, holding 2*kFirJ trace samples and kFirJ taps in
// registers, so one shared-memory word feeds kFirJ/2 FMAs instead of one
// word per FMA.  The trace sits zero-padded in shared memory (sample i at
// fir_q(L) + i, zeros elsewhere) and the taps are zero-padded to
// fir_lpad(L): no per-sample bounds.  Each output sums its taps in
// increasing k, and the padded terms add exact zeros, so o[n] equals the
// plain loop over k in [max(0, n+c-nt+1), min(L-1, n+c)] bit for bit.
#pragma once

namespace kgb {

constexpr int kFirJ = 8;

// taps rounded up to a multiple of kFirJ
__host__ __device__ __forceinline__ int fir_lpad(int L) { return (L + kFirJ - 1) / kFirJ * kFirJ; }
// position of sample 0 in the padded trace
__host__ __device__ __forceinline__ int fir_q(int L) { return fir_lpad(L) - 1 - (L - 1) / 2; }
// floats of the padded trace (a multiple of 4)
__host__ __device__ __forceinline__ int fir_span(int L, int nt) { return (fir_lpad(L) + nt + 8 + 3) & ~3; }
// floats of an output buffer fir_same may write (whole blocks of kFirJ)
__host__ __device__ __forceinline__ int fir_out(int nt) { return (nt + kFirJ - 1) / kFirJ * kFirJ; }

// gs: fir_lpad(L) taps, zero past L; xp: fir_span(L, nt) floats, zero
// outside [fir_q(L), fir_q(L) + nt); os: fir_out(nt) floats.  All three
// 16-byte aligned.  Threads t, t + nthreads, ... of the caller take the
// output blocks; no barrier inside.
__device__ __forceinline__ void fir_same(const float* __restrict__ gs, const float* __restrict__ xp,
                                         float* __restrict__ os, int L, int nt, int t, int nthreads) {
    const int Lp = fir_lpad(L);
    const int nblk = (nt + kFirJ - 1) / kFirJ;
    for (int b = t; b < nblk; b += nthreads) {
        const int n0 = b * kFirJ;
        float o[kFirJ];
#pragma unroll
        for (int j = 0; j < kFirJ; ++j) o[j] = 0.f;
        for (int k0 = 0; k0 < Lp; k0 += kFirJ) {
            // samples xp[Lp - 1 + n - k] for n = n0 + j, k = k0 + kk:
            // r[i] = xp[Lp - kFirJ + n0 - k0 + i], i = j - kk + kFirJ - 1
            const float4* xb = reinterpret_cast<const float4*>(xp + (Lp - kFirJ + n0 - k0));
            float r[2 * kFirJ];
#pragma unroll
            for (int v = 0; v < kFirJ / 2; ++v) {
                const float4 a = xb[v];
                r[4 * v] = a.x;
                r[4 * v + 1] = a.y;
                r[4 * v + 2] = a.z;
                r[4 * v + 3] = a.w;
            }
            float gk[kFirJ];
#pragma unroll
            for (int v = 0; v < kFirJ / 4; ++v) {
                const float4 a = reinterpret_cast<const float4*>(gs + k0)[v];
                gk[4 * v] = a.x;
                gk[4 * v + 1] = a.y;
                gk[4 * v + 2] = a.z;
                gk[4 * v + 3] = a.w;
            }
#pragma unroll
            for (int kk = 0; kk < kFirJ; ++kk)
#pragma unroll
                for (int j = 0; j < kFirJ; ++j) o[j] = fmaf(gk[kk], r[j - kk + kFirJ - 1], o[j]);
        }
#pragma unroll
        for (int v = 0; v < kFirJ / 4; ++v)
            reinterpret_cast<float4*>(os + n0)[v] = make_float4(o[4 * v], o[4 * v + 1], o[4 * v + 2], o[4 * v + 3]);
    }
}

}  // namespace kgb
