// Double-float accumulation of float32 products on the float32 pipe.
//
// The solvers' dot products and norms run over float32 vectors of up to tens
// of millions of elements.  Converting every element to float64 puts the whole
// pass on the float64 pipe, which runs at 1/64 of the float32 rate on GB300.
// Here a thread keeps its running sum as hi + lo in float32: the rounding
// error of each product comes exactly from an fma, the error of each addition
// exactly from TwoSum (Knuth), and both go into lo, so the pair carries the
// sum to ~2^-48 relative -- float64 quality -- before it is handed to the
// float64 block and grid reductions (hi + lo as a double).  Products are
// formed in float32, so, as with the float32 norms of the reference, their
// magnitude must stay below ~3e38 (squares of |v| < 1.8e19).
#pragma once

namespace kgb {

struct DFAcc {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add_prod(float a, float b) {
        const float p = __fmul_rn(a, b);
        const float e = __fmaf_rn(a, b, -p);  // a b - p, exact
        const float s = __fadd_rn(hi, p);
        const float bb = __fsub_rn(s, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));  // hi + p - s, exact
        hi = s;
        lo = __fadd_rn(lo, __fadd_rn(err, e));
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

}  // namespace kgb
