// 64-bit fixed-point trace accumulators in shared memory, added with one
// native 32-bit atomic per contribution.
//
// Each contribution is rounded to an integer x with |x| <= 2^kFixedBits
// (fixed_scale_exponent picks the power-of-two scale from a bound on the
// contributions).  A row of nt_pad bins occupies 2 * nt_pad 32-bit words:
// the low words of the bins in [0, nt_pad), the high words in
// [nt_pad, 2 * nt_pad); a bin holds 2^31 + (sum of its contributions) as a
// 64-bit two's-complement number.  fixed_add adds x to the low word and,
// from the value the atomic returns, the carry or borrow to the high word;
// starting the low words at 2^31 makes that second atomic rare (the running
// sum has to move 2^31 away from zero).  Every bin ends at the exact
// integer sum whatever the order of the atomics, so the traces are
// bitwise repeatable.  The rounding step is 2^-(kFixedBits+1) of the bound.
#pragma once

#include <stdint.h>

namespace kgb {

constexpr int kFixedBits = 30;
constexpr uint32_t kFixedBias = 0x80000000u;

// e with |v| 2^e < 2^kFixedBits for |v| <= amax
__device__ __forceinline__ int fixed_scale_exponent(float amax) {
    if (!(amax > 0.f)) return 0;
    int ex;
    frexpf(amax, &ex);  // amax < 2^ex
    return max(-126, min(kFixedBits - ex, 126));
}

// Set rows [0, nrows) of nt_pad bins to zero (low words at the bias).
__device__ __forceinline__ void fixed_clear(uint32_t* __restrict__ acc, int nrows, int nt_pad, int t, int nthreads) {
    uint2* a2 = reinterpret_cast<uint2*>(acc);  // nt_pad is a multiple of 4: a pair never straddles planes
    const int half = nt_pad / 2;
    for (int k = t; k < nrows * nt_pad; k += nthreads) {
        const bool lo = (k % nt_pad) < half;
        a2[k] = lo ? make_uint2(kFixedBias, kFixedBias) : make_uint2(0u, 0u);
    }
}

// x == 0 touches nothing (bin may then be out of range).
__device__ __forceinline__ void fixed_add(uint32_t* __restrict__ row, int nt_pad, int bin, int x) {
    if (x != 0) {
        const uint32_t old = atomicAdd(row + bin, (uint32_t)x);
        const uint32_t now = old + (uint32_t)x;
        // carry out of the low word, minus one for the sign extension of x
        const int hi = (now < old ? 1 : 0) - (x < 0 ? 1 : 0);
        if (hi) atomicAdd(row + nt_pad + bin, (uint32_t)hi);
    }
}

__device__ __forceinline__ long long fixed_get(const uint32_t* __restrict__ row, int nt_pad, int bin) {
    const unsigned long long u = ((unsigned long long)row[nt_pad + bin] << 32) | row[bin];
    return (long long)(u - kFixedBias);
}

}  // namespace kgb
