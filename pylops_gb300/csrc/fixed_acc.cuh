// 64-bit fixed-point trace accumulators in shared memory, added with one
// native 32-bit atomic per contribution.
//
// A row of nt_pad bins occupies 2 * nt_pad 32-bit words: the low words of
// the bins in [0, nt_pad), the high words in [nt_pad, 2 * nt_pad).  A bin
// holds 2^31 + (sum of its contributions) as a 64-bit two's-complement
// number.  fixed_add adds an integer x, |x| < 2^31, to the low word and,
// from the value the atomic returns, the carry or borrow to the high word --
// a second atomic that is skipped when that is zero, which is the rule
// (starting the low words at 2^31 makes a carry or borrow rare: the running
// sum has to move 2^31 away from zero).  fixed_add_wide does the same with
// the high 32 bits of a larger x added to the high word.  Every bin ends at the exact integer
// sum whatever the order of the atomics, so the traces are bitwise
// repeatable.
//
// The scale (a power of two) is chosen per application from the magnitudes
// of the model (fixed_choose_exponent): 99 % of the contributions round to
// at most kFixedBits bits plus sign -- a rounding step of 2^-(kFixedBits+1)
// of their bound -- and the image points that may give more, up to a bound
// that keeps every bin sum inside 62 bits, take fixed_add_wide exactly.  A few large model values
// therefore cost neither the precision of the others nor correctness.
#pragma once

#include <stdint.h>

namespace kgb {

constexpr int kFixedBits = 30;
constexpr uint32_t kFixedBias = 0x80000000u;

// Histogram bucket of a nonzero float: its biased exponent, so that
// |v| < 2^(bucket - 126).
__device__ __forceinline__ int scale_bucket(float v) { return (int)((__float_as_uint(v) >> 23) & 0xffu); }

// Run by one block of 256 threads.  blk: [0] bits of max |mv|, [1] output
// exponent e, [2, 258) histogram of scale_bucket(mv) over the nonzero mv;
// contributions are bounded by |mv| * wfactor.  e = min(e_fast, e_safe):
// e_fast puts 99 % of the contributions below 2^kFixedBits, e_safe keeps
// each contribution below 2^(61 - ceil(log2(ni + 1))) so that the 2 ni
// contributions a bin can receive sum inside int64.
__device__ __forceinline__ void fixed_choose_exponent(unsigned* blk, int64_t ni, float wfactor) {
    __shared__ unsigned cum[256];
    const int t = threadIdx.x;
    cum[t] = blk[2 + t];
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {  // inclusive prefix sum
        const unsigned a = t >= off ? cum[t - off] : 0u;
        __syncthreads();
        cum[t] += a;
        __syncthreads();
    }
    const unsigned total = cum[255];
    const unsigned need = total - total / 100u;
    __shared__ int b99;
    if (t == 0) b99 = 255;
    __syncthreads();
    if (total && cum[t] >= need && (t == 0 || cum[t - 1] < need)) b99 = t;
    __syncthreads();
    if (t != 0) return;
    const float amax = __uint_as_float(blk[0]);
    int e = 0;
    if (total && amax > 0.f && wfactor > 0.f) {
        int ew, eb;
        frexpf(wfactor, &ew);            // wfactor < 2^ew
        frexpf(amax * wfactor, &eb);     // every contribution < 2^eb
        int nb = 0;
        while (nb < 40 && ((int64_t)1 << nb) <= ni) ++nb;
        const int e_fast = kFixedBits - ((b99 - 126) + ew);
        const int e_safe = 61 - nb - eb;
        e = max(-126, min(min(e_fast, e_safe), 126));
    }
    blk[1] = (unsigned)e;
}

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

// Add x (|x| < 2^31) to bin `bin` of the row; x == 0 touches nothing (bin
// may then be out of range).
__device__ __forceinline__ void fixed_add(uint32_t* __restrict__ row, int nt_pad, int bin, int x) {
    if (x != 0) {
        const uint32_t old = atomicAdd(row + bin, (uint32_t)x);
        const uint32_t now = old + (uint32_t)x;
        // carry out of the low word, minus one for the sign extension of x
        const int hi = (now < old ? 1 : 0) - (x < 0 ? 1 : 0);
        if (hi) atomicAdd(row + nt_pad + bin, (uint32_t)hi);
    }
}

// The same for a scaled contribution v of any size the scale allows
// (|v| < 2^62), rounded to the nearest integer: the low 32 bits go to the
// low word, the high 32 bits plus the carry to the high word.
__device__ __forceinline__ void fixed_add_wide(uint32_t* __restrict__ row, int nt_pad, int bin, float v) {
    const long long x = __float2ll_rn(v);
    if (x == 0) return;
    const uint32_t lo = (uint32_t)x;
    int hi = (int)(x >> 32);
    const uint32_t old = atomicAdd(row + bin, lo);
    hi += (old + lo < old) ? 1 : 0;
    if (hi) atomicAdd(row + nt_pad + bin, (uint32_t)hi);
}

// Whether a point of scaled value v may give a contribution of 2^31 or more
// (|contribution| <= |v| * wfactor): such points take fixed_add_wide.
__device__ __forceinline__ bool fixed_wide(float v, float wfactor) { return fabsf(v) * wfactor >= 2147483520.f; }

__device__ __forceinline__ long long fixed_get(const uint32_t* __restrict__ row, int nt_pad, int bin) {
    const unsigned long long u = ((unsigned long long)row[nt_pad + bin] << 32) | row[bin];
    return (long long)(u - kFixedBias);
}

// ---------------------------------------------------------------------------
// Split accumulation: the same exact integer sums without returned atomics
// or carries, for traces whose bins provably receive at most
// kSplitMaxCount contributions each (counted once per operator when its
// tables are set, spread_count_kernel).
//
// Each bin keeps two 32-bit words, both cleared to 0:
//   L = sum of x           mod 2^32   (low plane, [0, nt_pad))
//   H = sum of floor(x/2^16) mod 2^32 (high plane, [nt_pad, 2 nt_pad))
// each added with one fire-and-forget shared atomic (the value is not read
// back).  With R = sum of (x mod 2^16), 0 <= R < count * 2^16 <= 2^32, so
// R = (L - 2^16 H) mod 2^32 exactly, and S = 2^16 H + R mod 2^48 is the
// exact sum when |S| < 2^47 -- true for at most kSplitMaxCount
// contributions of |x| < 2^31.  Larger contributions (the points the scale
// marks wide) are added exactly with 64-bit global atomics into a per-trace
// accumulator instead (split_add_wide).  Integer sums commute, so the
// result equals the carry scheme's bit for bit.
// ---------------------------------------------------------------------------
constexpr unsigned kSplitMaxCount = 65535u;

__device__ __forceinline__ void split_clear(uint32_t* __restrict__ acc, int nrows, int nt_pad, int t, int nthreads) {
    uint4* a4 = reinterpret_cast<uint4*>(acc);  // 2 nt_pad words per row, nt_pad a multiple of 4
    for (int k = t; k < nrows * nt_pad / 2; k += nthreads) a4[k] = make_uint4(0u, 0u, 0u, 0u);
}

// Add x (|x| < 2^31) to bin `bin`; x == 0 touches nothing.
__device__ __forceinline__ void split_add(uint32_t* __restrict__ row, int nt_pad, int bin, int x) {
    if (x != 0) {
        atomicAdd(row + bin, (uint32_t)x);
        atomicAdd(row + nt_pad + bin, (uint32_t)(x >> 16));
    }
}

// A wide contribution (scaled value v, |v| < 2^62, rounded to the nearest
// integer) into the trace's 64-bit global accumulator.
__device__ __forceinline__ void split_add_wide(unsigned long long* __restrict__ wrow, int bin, float v) {
    const long long x = __float2ll_rn(v);
    if (x != 0) atomicAdd(wrow + bin, (unsigned long long)x);
}

__device__ __forceinline__ long long split_get(const uint32_t* __restrict__ row, int nt_pad, int bin) {
    const uint32_t L = row[bin], H = row[nt_pad + bin];
    const uint32_t R = L - (H << 16);
    const unsigned long long u = ((unsigned long long)H << 16) + R;
    return (long long)(u << 16) >> 16;  // sign-extend the 48-bit sum
}

}  // namespace kgb
