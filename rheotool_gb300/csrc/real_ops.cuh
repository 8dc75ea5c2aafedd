// real_ops.cuh — explicitly rounded arithmetic for kernels templated on the
// real type.  The explicit forms keep the compiler from contracting or
// reordering, so two kernels that evaluate the same recurrence in the same
// order of operations give the same bits.
#pragma once

namespace rt {

__device__ __forceinline__ double r_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float r_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double r_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float r_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double r_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float r_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double r_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float r_div(float a, float b) { return __fdiv_rn(a, b); }

// Sums of FP32 vectors kept as an unevaluated pair hi + lo of FP32 numbers:
// each product split exactly by an FMA, each addition by Knuth's two-sum
// (the Dot2 algorithm of Ogita, Rump and Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26 (2005)).  The result carries about twice
// the FP32 precision, near an FP64 accumulation, with FP32 arithmetic only:
// GB300 runs FP64 at a small fraction of its FP32 rate, so a per-element FP64
// accumulation bounds a reduction that one CTA performs over a whole case.
// The products must stay in the FP32 range (|x y| < 3.4e38).
struct Acc2f {
    float hi = 0.0f, lo = 0.0f;
};
__device__ __forceinline__ void acc_add(Acc2f &a, float x) {
    const float s = __fadd_rn(a.hi, x);
    const float z = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, z)), __fsub_rn(x, z));
    a.hi = s;
    a.lo = __fadd_rn(a.lo, e);
}
__device__ __forceinline__ void acc_dot(Acc2f &a, float x, float y) {
    const float p = __fmul_rn(x, y);
    const float e = __fmaf_rn(x, y, -p);
    acc_add(a, p);
    a.lo = __fadd_rn(a.lo, e);
}
__device__ __forceinline__ double acc_value(const Acc2f &a) { return (double)a.hi + (double)a.lo; }

// the FP64 counterpart (FP64 vectors): a plain FP64 sum
struct Acc1d {
    double v = 0.0;
};
__device__ __forceinline__ void acc_add(Acc1d &a, double x) { a.v += x; }
__device__ __forceinline__ void acc_dot(Acc1d &a, double x, double y) { a.v += x * y; }
__device__ __forceinline__ double acc_value(const Acc1d &a) { return a.v; }

template <class V>
struct AccOf {
    using type = Acc1d;
};
template <>
struct AccOf<float> {
    using type = Acc2f;
};

}  // namespace rt
