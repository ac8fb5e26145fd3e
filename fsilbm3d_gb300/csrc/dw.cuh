// dw.cuh -- double-word ("float-float") arithmetic: a value is the unevaluated
// sum h + l of two FP32 numbers with |l| <= ulp(h), about 48 significant bits.
//
// GB300 issues FP64 at about 1/60 of its FP32 rate, so an FP64 collision is
// bound by the FP64 pipe at a fifth of the HBM roofline. The FSI_PREC_F64_DW
// form keeps the distributions in FP64 in HBM and computes the collision in
// double-word arithmetic on the FP32 pipe. Building blocks (all with
// round-to-nearest FP32 operations that the compiler may not contract):
//   Fast2Sum  -- Dekker, "A floating-point technique for extending the
//               available precision", Numer. Math. 18 (1971): s + t = a + b
//               exactly when |a| >= |b|.
//   TwoSum    -- Knuth, TAOCP vol. 2, 4.2.2: s + t = a + b exactly, any order.
//   addition  -- SloppyDWPlusDW (Joldes, Muller, Popescu, "Tight and rigorous
//               error bounds for basic building blocks of double-word
//               arithmetic", ACM TOMS 44 (2017), Algorithm 5): TwoSum of the
//               high parts, the low parts added, renormalised by Fast2Sum.
//               Its error is a few units of 2^-48 of the operands' magnitude,
//               which is the scale every quantity of the collision is judged on.
//   product   -- DWTimesDW3 (same paper, Algorithm 12) with fused
//               multiply-add for the exact product of the high parts.
//   reciprocal-- one Newton step r = y + y (1 - x y) from the FP32 reciprocal.
// FP64 -> double word is integer bit work (FP64 -> FP32 conversion runs on
// GB300's FP64 pipe, about 2 per clock per SM); double word -> FP64 is two
// exact FP32 -> FP64 conversions (about 20 per clock per SM) and one FP64
// addition per stored value, so that the step issues little FP64 work.
#pragma once
#include <cuda_runtime.h>

namespace fsi {

// Declared, never defined: the functions below are device arithmetic, and
// their host-compiled bodies only call this, so that host code using them
// fails to link (nvcc accepts a __device__ operator called from a host
// template without a diagnostic, and the call then ends the process at run
// time).
void dw_arithmetic_is_device_only();

struct dw {
    float h, l;
    __host__ __device__ constexpr dw() : h(0.0f), l(0.0f) {}
    // nearest pair of a double; folded at compile time for constants
    __host__ __device__ constexpr dw(double d) : h((float)d), l((float)(d - (double)(float)d)) {}
    __host__ __device__ constexpr dw(float hh, float ll, int) : h(hh), l(ll) {}
    __device__ explicit operator double() const;
};

__host__ __device__ __forceinline__ dw dw_fast2sum(float a, float b) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw();
#else
    const float s = __fadd_rn(a, b);
    const float z = __fsub_rn(s, a);
    return dw(s, __fsub_rn(b, z), 0);
#endif
}

__host__ __device__ __forceinline__ dw dw_two_sum(float a, float b) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw();
#else
    const float s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float ap = __fsub_rn(s, bp);
    const float db = __fsub_rn(b, bp), da = __fsub_rn(a, ap);
    return dw(s, __fadd_rn(da, db), 0);
#endif
}

__host__ __device__ __forceinline__ dw operator+(dw x, dw y) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw();
#else
    const dw s = dw_two_sum(x.h, y.h);
    const float v = __fadd_rn(x.l, y.l);
    return dw_fast2sum(s.h, __fadd_rn(s.l, v));
#endif
}
__host__ __device__ __forceinline__ dw operator-(dw x) { return dw(-x.h, -x.l, 0); }
__host__ __device__ __forceinline__ dw operator-(dw x, dw y) { return x + (-y); }
__host__ __device__ __forceinline__ dw operator*(dw x, dw y) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw();
#else
    const float ch = __fmul_rn(x.h, y.h);
    const float cl1 = __fmaf_rn(x.h, y.h, -ch);
    const float tl0 = __fmul_rn(x.l, y.l);
    const float tl1 = __fmaf_rn(x.h, y.l, tl0);
    const float cl2 = __fmaf_rn(x.l, y.h, tl1);
    return dw_fast2sum(ch, __fadd_rn(cl1, cl2));
#endif
}
__host__ __device__ __forceinline__ dw &operator+=(dw &x, dw y) { return x = x + y; }
__host__ __device__ __forceinline__ dw &operator-=(dw &x, dw y) { return x = x - y; }
__host__ __device__ __forceinline__ dw &operator*=(dw &x, dw y) { return x = x * y; }

// 1/x: the FP32 reciprocal y, then y + y (1 - x y) with x y formed exactly
// enough (its high part is within an ulp of 1, so 1 - h is exact)
__host__ __device__ __forceinline__ dw rcp(dw x) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw();
#else
    const float y = __frcp_rn(x.h);
    const float ph = __fmul_rn(x.h, y);
    const float pl = __fmaf_rn(x.l, y, __fmaf_rn(x.h, y, -ph));
    const float d = __fsub_rn(__fsub_rn(1.0f, ph), pl);
    return dw_fast2sum(y, __fmul_rn(y, d));
#endif
}

// FP64 bits -> double word, without FP64 instructions: the leading 24
// significant bits truncated into h (the exponent rebased from 1023 to 127),
// the remaining 29 bits rounded into l. Values below 2^-126 become 0 (l
// alone below 2^-74); values from 2^128 up are outside the form's range.
__host__ __device__ __forceinline__ dw dw_from_f64(double d) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw();
#else
    const unsigned lo = (unsigned)__double2loint(d), hi = (unsigned)__double2hiint(d);
    const unsigned e11 = (hi >> 20) & 0x7FFu;
    const unsigned sgn = hi & 0x80000000u;
    const unsigned hb = (__funnelshift_r(lo, hi, 29) - (896u << 23)) | sgn;
    const float r = __fmul_rn(__uint2float_rn(lo & 0x1FFFFFFFu), __uint_as_float((e11 - 948u) << 23));
    const float l = __uint_as_float(__float_as_uint(r) | sgn);
    return dw(e11 >= 897u ? __uint_as_float(hb) : 0.0f, e11 >= 949u ? l : 0.0f, 0);
#endif
}

// double word -> nearest FP64: the two parts converted exactly (FP32 -> FP64
// conversion is not an FP64-pipe instruction on GB300), one FP64 addition
__host__ __device__ __forceinline__ double dw_to_f64(dw x) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return double();
#else
    return __dadd_rn((double)x.h, (double)x.l);
#endif
}

__device__ __forceinline__ dw::operator double() const { return dw_to_f64(*this); }

}  // namespace fsi
