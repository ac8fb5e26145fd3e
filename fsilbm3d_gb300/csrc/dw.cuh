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
// Conversions between FP32 and FP64 run on GB300's FP64 pipe (about two per
// clock per SM), so both directions are integer bit work here: FP64 -> double
// word splits the significand, double word -> FP64 builds the two exact FP64
// parts and adds them with the one FP64 instruction per stored value.
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

// the exact FP64 value of an FP32 number by bit operations (subnormals -> 0):
// GB300 runs FP32 -> FP64 conversion on its FP64 pipe
__host__ __device__ __forceinline__ double f64_of_f32(float x) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return double();
#else
    const unsigned b = __float_as_uint(x);
    const unsigned sgn = b & 0x80000000u;
    const bool nz = (b & 0x7F800000u) != 0u;
    const unsigned hi = nz ? (((b & 0x7FFFFFFFu) >> 3) + (896u << 20)) | sgn : sgn;
    const unsigned lo = nz ? (b << 29) : 0u;
    return __hiloint2double((int)hi, (int)lo);
#endif
}

// double word -> nearest FP64: the two parts made exact FP64 numbers by bit
// operations, one FP64 addition (the only FP64-pipe instruction per value)
__host__ __device__ __forceinline__ double dw_to_f64(dw x) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return double();
#else
    return __dadd_rn(f64_of_f32(x.h), f64_of_f32(x.l));
#endif
}

__device__ __forceinline__ dw::operator double() const { return dw_to_f64(*this); }

}  // namespace fsi

// ---------------------------------------------------------------------------
// dw2: two double words side by side (the same quantity of two cells), every
// operation one packed FP32x2 instruction (FADD2 / FMUL2 / FFMA2) per step of
// the single algorithms above, so that two cells cost the issue slots of one.
// Subtraction is written out (TwoDiff) instead of adding a negated operand.
namespace fsi {

__device__ __forceinline__ float2 p2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, p2(-1.0f), a); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

struct dw2 {
    float2 h, l;
    __host__ __device__ constexpr dw2() : h{0.0f, 0.0f}, l{0.0f, 0.0f} {}
    __host__ __device__ constexpr dw2(double d)
        : h{(float)d, (float)d}, l{(float)(d - (double)(float)d), (float)(d - (double)(float)d)} {}
    __host__ __device__ constexpr dw2(float2 hh, float2 ll, int) : h(hh), l(ll) {}
};

__host__ __device__ __forceinline__ dw2 dw2_fast2sum(float2 a, float2 b) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw2();
#else
    const float2 s = padd(a, b);
    return dw2(s, psub(b, psub(s, a)), 0);
#endif
}

__host__ __device__ __forceinline__ dw2 operator+(dw2 x, dw2 y) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw2();
#else
    const float2 s = padd(x.h, y.h);
    const float2 bp = psub(s, x.h);
    const float2 ap = psub(s, bp);
    const float2 e = padd(psub(x.h, ap), psub(y.h, bp));
    return dw2_fast2sum(s, padd(e, padd(x.l, y.l)));
#endif
}
__host__ __device__ __forceinline__ dw2 operator-(dw2 x, dw2 y) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw2();
#else
    // TwoDiff(a, b) = TwoSum(a, -b) with the negation folded in
    const float2 s = psub(x.h, y.h);
    const float2 bp = psub(s, x.h);
    const float2 ap = psub(s, bp);
    const float2 e = psub(psub(x.h, ap), padd(y.h, bp));
    return dw2_fast2sum(s, padd(e, psub(x.l, y.l)));
#endif
}
__host__ __device__ __forceinline__ dw2 operator-(dw2 x) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw2();
#else
    return dw2(pmul(x.h, p2(-1.0f)), pmul(x.l, p2(-1.0f)), 0);
#endif
}
__host__ __device__ __forceinline__ dw2 operator*(dw2 x, dw2 y) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw2();
#else
    const float2 ch = pmul(x.h, y.h);
    const float2 cl1 = pfma(x.h, y.h, pmul(ch, p2(-1.0f)));
    const float2 cl2 = pfma(x.l, y.h, pfma(x.h, y.l, pmul(x.l, y.l)));
    return dw2_fast2sum(ch, padd(cl1, cl2));
#endif
}
__host__ __device__ __forceinline__ dw2 &operator+=(dw2 &x, dw2 y) { return x = x + y; }
__host__ __device__ __forceinline__ dw2 &operator-=(dw2 &x, dw2 y) { return x = x - y; }
__host__ __device__ __forceinline__ dw2 &operator*=(dw2 &x, dw2 y) { return x = x * y; }

__host__ __device__ __forceinline__ dw2 rcp(dw2 x) {
#ifndef __CUDA_ARCH__
    dw_arithmetic_is_device_only();
    return dw2();
#else
    const float2 y = make_float2(__frcp_rn(x.h.x), __frcp_rn(x.h.y));
    const float2 ph = pmul(x.h, y);
    const float2 pl = pfma(x.l, y, pfma(x.h, y, pmul(ph, p2(-1.0f))));
    const float2 d = psub(psub(p2(1.0f), ph), pl);
    return dw2_fast2sum(y, pmul(y, d));
#endif
}

}  // namespace fsi
