// k_fast.cu -- the throughput forms of the fused collide+stream step.
//
//  FSI_PREC_F64_FAST  FP64 storage of f, FP64 arithmetic regrouped around the
//                     nine opposite-direction pairs (ConstParams.f90:19-20)
//                     with fused multiply-add.
//  FSI_PREC_F64_DW    FP64 storage of f, the collision in double-word FP32
//                     arithmetic (dw.cuh) on the FP32 pipe; SRT and MRT.
//  FSI_PREC_F32/F16/BF16
//                     storage of the offsets g_i = f_i - w_i (w_i: lattice
//                     weights, ConstParams.f90:22-25) in FP32, FP16 or BF16;
//                     all arithmetic in FP32 on the offsets, so that the
//                     density enters as 1 + sum(g) and no precision is spent
//                     on the constant part of f.
//
// Physics and step order are those of the exact form (collision_ SRT/MRT
// with Guo forcing, FluidDomain.f90:1208-1238; streaming_ :1514-1625; the
// IB window and face hooks of k_f64_exact.cu); only rounding differs.
//
// This file is compiled once per storage form, with -DFSI_FAST_PREC=<form>
// (1..5: FSI_PREC_F64_FAST, F32, F16, BF16, F64_DW), so that the forms'
// kernels build in parallel. The F64_DW unit defines only the bulk step: its
// blocks use the F64_FAST unit for everything else (same FP64 storage). Each unit defines the launchers of fsi_kernels.h's
// FSI_FAST_API in namespace fsi::fast_p<form>; fast_route.cu forwards the
// public names to them.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <type_traits>

#include "bc_impl.cuh"
#include "dw.cuh"
#include "fsi_kernels.h"
#include "ib_impl.cuh"
#include "mlp_impl.cuh"
#include "../../include/fsi_gpu.h"

#ifndef FSI_FAST_PREC
#error "k_fast.cu is built once per storage form: -DFSI_FAST_PREC=1|2|3|4|5"
#endif
#if FSI_FAST_PREC < FSI_PREC_F64_FAST || FSI_FAST_PREC > FSI_PREC_F64_DW
#error "FSI_FAST_PREC must be FSI_PREC_F64_FAST, F32, F16, BF16 or F64_DW"
#endif
#define FSI_CAT2(a, b) a##b
#define FSI_CAT(a, b) FSI_CAT2(a, b)
#define FSI_FAST_NS FSI_CAT(fast_p, FSI_FAST_PREC)

namespace fsi {
namespace {

constexpr int TPB = 256;

template <int P> struct ST;
// internal: the double-word form with two cells per thread (dw2)
constexpr int PDW2 = 105;
template <> struct ST<PDW2> {
    using S = double; using C = dw2;
    static constexpr bool OFF = false;
};
template <> struct ST<FSI_PREC_F64_FAST> {
    using S = double; using C = double;
    static constexpr bool OFF = false;
    static __device__ __forceinline__ C dec(S s) { return s; }
    static __device__ __forceinline__ S enc(C c) { return c; }
};
template <> struct ST<FSI_PREC_F64_DW> {
    using S = double; using C = dw;
    static constexpr bool OFF = false;
    static __device__ __forceinline__ C dec(S s) { return dw_from_f64(s); }
    static __device__ __forceinline__ S enc(C c) { return dw_to_f64(c); }
};
template <> struct ST<FSI_PREC_F32> {
    using S = float; using C = float;
    static constexpr bool OFF = true;
    static __device__ __forceinline__ C dec(S s) { return s; }
    static __device__ __forceinline__ S enc(C c) { return c; }
};
template <> struct ST<FSI_PREC_F16> {
    using S = __half; using C = float;
    static constexpr bool OFF = true;
    static __device__ __forceinline__ C dec(S s) { return __half2float(s); }
    static __device__ __forceinline__ S enc(C c) { return __float2half_rn(c); }
};
template <> struct ST<FSI_PREC_BF16> {
    using S = __nv_bfloat16; using C = float;
    static constexpr bool OFF = true;
    static __device__ __forceinline__ C dec(S s) { return __bfloat162float(s); }
    static __device__ __forceinline__ S enc(C c) { return __float2bfloat16_rn(c); }
};

// accessor for the boundary kernels: FP64 distribution values in and out
template <int P> struct AccS {
    using T = ST<P>;
    static __device__ __forceinline__ double load(const void *f, long long i, int q) {
        double v = (double)T::dec(((const typename T::S *)f)[i]);
        return T::OFF ? v + wt_(q) : v;
    }
    static __device__ __forceinline__ void store(void *f, long long i, int q, double v) {
        ((typename T::S *)f)[i] = T::enc((typename T::C)(T::OFF ? v - wt_(q) : v));
    }
};

__device__ __forceinline__ long long cidx(int z, int y, int x, int Z, int Y) {
    return (long long)z + (long long)Z * ((long long)y + (long long)Y * (long long)x);
}

// 1/rho: IEEE in FP64; the hardware approximation (about 1 ulp) in FP32,
// where the stored form's rounding dominates
__device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
__device__ __forceinline__ float rcp(float x) { return __fdividef(1.0f, x); }

// +v, -v or the additive identity -0 for lattice component e
template <typename C> __device__ __forceinline__ C sel(int e, C v) { return e > 0 ? v : (e < 0 ? -v : C(-0.0)); }

// e_i . (v0, v1, v2) summing only the nonzero components (i is a constant
// after unrolling). Equal, bit for bit, to the three-term sum of sel():
// x + (-0) is x in IEEE arithmetic; the double-word type is spared the
// additions of zero.
template <typename C> __device__ __forceinline__ C eacc(bool set, int e, C acc, C v) {
    return set ? (e > 0 ? acc + v : acc - v) : sel(e, v);
}
template <typename C> __device__ __forceinline__ C edot3(int i, C v0, C v1, C v2) {
    C acc = C(-0.0);
    bool set = false;
    if (ex_(i) != 0) { acc = sel(ex_(i), v0); set = true; }
    if (ey_(i) != 0) { acc = eacc(set, ey_(i), acc, v1); set = true; }
    if (ez_(i) != 0) { acc = eacc(set, ez_(i), acc, v2); }
    return acc;
}

// offset equilibrium g_eq = w (rho - 1) + w rho (3 eu + 4.5 eu^2 - 1.5 u^2),
// k15 = 1.5 u^2 (the face kernels and the fused z faces)
__device__ __forceinline__ float geq_off(int q, float rho, float u0, float u1, float u2, float k15) {
    const float eu = (float)ex_(q) * u0 + (float)ey_(q) * u1 + (float)ez_(q) * u2;
    const float w = (float)wt_(q);
    return w * (rho - 1.0f) + (w * rho) * ((3.0f + 4.5f * eu) * eu - k15);
}
__device__ __forceinline__ float geq_zface(const StepArgs &a, int side, int q) { return a.zg[side][q]; }

// density (and its offset from 1) and velocity of one cell,
// calculate_macro_quantities_ (FluidDomain.f90:1136-1139) regrouped
template <int P>
__device__ __forceinline__ void macro_fast(const typename ST<P>::C g[Q], const typename ST<P>::C vf[3],
                                           typename ST<P>::C dh, typename ST<P>::C &rho, typename ST<P>::C &drho,
                                           typename ST<P>::C &u0, typename ST<P>::C &u1, typename ST<P>::C &u2) {
    using C = typename ST<P>::C;
    C s = g[0], jx = C(-0.0), jy = C(-0.0), jz = C(-0.0);
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const int i = pr_(k), o = opp_(i);
        const C sk = g[i] + g[o], dk = g[i] - g[o];
        s += sk;
        if (ex_(i) > 0) jx += dk; else if (ex_(i) < 0) jx -= dk;
        if (ey_(i) > 0) jy += dk; else if (ey_(i) < 0) jy -= dk;
        if (ez_(i) > 0) jz += dk; else if (ez_(i) < 0) jz -= dk;
    }
    if (ST<P>::OFF) { drho = s; rho = C(1) + s; }
    else { rho = s; drho = s - C(1); }
    const C inv = rcp(rho);
    const C h = C(0.5) * dh;
    u0 = (jx + h * vf[0]) * inv;
    u1 = (jy + h * vf[1]) * inv;
    u2 = (jz + h * vf[2]) * inv;
}

// SRT/BGK with Guo forcing (FluidDomain.f90:1218-1227) on pairs
template <int P, bool FORCED>
__device__ __forceinline__ void collide_srt(typename ST<P>::C g[Q], typename ST<P>::C rho, typename ST<P>::C drho,
                                            typename ST<P>::C u0, typename ST<P>::C u1, typename ST<P>::C u2,
                                            typename ST<P>::C F0, typename ST<P>::C F1, typename ST<P>::C F2,
                                            typename ST<P>::C om, typename ST<P>::C dh3) {
    using C = typename ST<P>::C;
    constexpr bool OFF = ST<P>::OFF;
    const C usq = u0 * u0 + u1 * u1 + u2 * u2;
    const C k15 = C(1.5) * usq;
    const C cf = (C(1) - C(0.5) * om) * dh3;
    C uF = C(0);
    if (FORCED) uF = u0 * F0 + u1 * F1 + u2 * F2;
    {
        const C w = C(wt_(0));
        const C eq = OFF ? w * (drho - rho * k15) : (w * rho) * (C(1) - k15);
        g[0] = g[0] + om * (eq - g[0]);
        if (FORCED) g[0] = g[0] - (cf * w) * uF;
    }
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const int i = pr_(k), o = opp_(i);
        const C w = C(wt_(i));
        const C eu = edot3(i, u0, u1, u2);
        const C wr = w * rho;
        const C sym = OFF ? w * drho + wr * (C(4.5) * eu * eu - k15) : wr * ((C(1) - k15) + C(4.5) * eu * eu);
        const C asym = (C(3) * wr) * eu;
        const C gi = g[i], go = g[o];
        C ni = gi + om * ((sym + asym) - gi);
        C no = go + om * ((sym - asym) - go);
        if (FORCED) {
            const C eF = edot3(i, F0, F1, F2);
            const C cw = cf * w;
            const C Fs = cw * (C(3) * eu * eF - uF), Fa = cw * eF;
            ni += Fs + Fa;
            no += Fs - Fa;
        }
        g[i] = ni;
        g[o] = no;
    }
}

// the MRT matrices in the arithmetic type; sd: S_k / |row k|^2 of their
// moment form (used when the host found one, MrtMats::diag)
template <typename C> struct MatsT { C mc[361]; C mf[361]; C sd[Q]; };

// internal model tag: MRT applied in moment space (the matrices have the
// moment form M_COLLID = M^-1 S M, M_FORCE = I - M_COLLID/2)
constexpr int CM_MRT_MOM = 103;

// MRT (FluidDomain.f90:1236-1238): g += M_COLLID (feq - f) + M_FORCE Flb
template <int P>
__device__ __forceinline__ void collide_mrt(typename ST<P>::C g[Q], typename ST<P>::C rho, typename ST<P>::C drho,
                                            typename ST<P>::C u0, typename ST<P>::C u1, typename ST<P>::C u2,
                                            typename ST<P>::C F0, typename ST<P>::C F1, typename ST<P>::C F2,
                                            bool forced, typename ST<P>::C dh3,
                                            const MatsT<typename ST<P>::C> &mm) {
    using C = typename ST<P>::C;
    constexpr bool OFF = ST<P>::OFF;
    const C usq = u0 * u0 + u1 * u1 + u2 * u2;
    const C k15 = C(1.5) * usq;
    C neq[Q], flb[Q];
    const C uF = u0 * F0 + u1 * F1 + u2 * F2;
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const C w = C(wt_(i));
        const C eu = edot3(i, u0, u1, u2);
        const C eq = OFF ? w * drho + (w * rho) * ((C(3) + C(4.5) * eu) * eu - k15)
                         : (w * rho) * ((C(1) - k15) + (C(3) + C(4.5) * eu) * eu);
        neq[i] = eq - g[i];
        const C eF = edot3(i, F0, F1, F2);
        flb[i] = (dh3 * w) * (eF - uF + C(3) * eu * eF);
    }
#pragma unroll
    for (int i = 0; i < Q; i++) {
        C s = g[i];
#pragma unroll
        for (int j = 0; j < Q; j++) s += mm.mc[i + Q * j] * neq[j];
        if (forced) {
#pragma unroll
            for (int j = 0; j < Q; j++) s += mm.mf[i + Q * j] * flb[j];
        }
        g[i] = s;
    }
}

// The D3Q19 moment transform (rows mrow_) for one cell in any arithmetic
// type, by velocity class: r0 the rest value, rs[k] = r_i + r_o and rd[k] =
// r_i - r_o for the nine pairs in pr_ order (x, y, z axes; diagonals (1,1,0),
// (-1,1,0), (1,0,1), (-1,0,1), (0,1,1), (0,-1,1)). t[k] = sd[k] m_k; the
// conserved moments 0, 3, 5, 7 are not formed (their rates are zero).
template <typename C>
__device__ __forceinline__ void mrt_forward_c(C r0, const C rs[9], const C rd[9], const C sd[Q], C t[Q]) {
    const C Ax = rs[0], Ay = rs[1], Az = rs[2];
    const C Dxy = rs[3] + rs[4], Dxz = rs[5] + rs[6], Dyz = rs[7] + rs[8];
    const C A = (Ax + Ay) + Az, D = (Dxy + Dxz) + Dyz;
    const C m1 = C(-30) * r0 + (C(-11) * A + C(8) * D);
    const C m2 = C(12) * r0 + (C(-4) * A + D);
    const C U = Ay + Az, V = C(-2) * Dyz + (Dxy + Dxz);
    const C m9 = C(2) * Ax + (V - U);
    const C m10 = C(-4) * Ax + (C(2) * U + V);
    const C W = Ay - Az, Xd = Dxy - Dxz;
    const C m11 = W + Xd;
    const C m12 = C(-2) * W + Xd;
    const C m13 = rs[3] - rs[4], m14 = rs[7] - rs[8], m15 = rs[5] - rs[6];
    const C p3 = rd[3] - rd[4], q3 = rd[3] + rd[4];
    const C p5 = rd[5] - rd[6], q5 = rd[5] + rd[6];
    const C p7 = rd[7] - rd[8], q7 = rd[7] + rd[8];
    const C m4 = C(-4) * rd[0] + (p3 + p5);
    const C m16 = p3 - p5;
    const C m6 = C(-4) * rd[1] + (q3 + p7);
    const C m17 = p7 - q3;
    const C m8 = C(-4) * rd[2] + (q5 + q7);
    const C m18 = q5 - q7;
    t[0] = t[3] = t[5] = t[7] = C(0);
    t[1] = sd[1] * m1; t[2] = sd[2] * m2; t[4] = sd[4] * m4; t[6] = sd[6] * m6; t[8] = sd[8] * m8;
    t[9] = sd[9] * m9; t[10] = sd[10] * m10; t[11] = sd[11] * m11; t[12] = sd[12] * m12;
    t[13] = sd[13] * m13; t[14] = sd[14] * m14; t[15] = sd[15] * m15;
    t[16] = sd[16] * m16; t[17] = sd[17] * m17; t[18] = sd[18] * m18;
}

// Delta = M^T t split by parity: Delta_0 = E0; for pair k with representative
// i: Delta_i = E[k] + O[k], Delta_opp(i) = E[k] - O[k]
template <typename C>
__device__ __forceinline__ void mrt_backward_c(const C t[Q], C &E0, C E[9], C O[9]) {
    E0 = C(-30) * t[1] + C(12) * t[2];
    const C Ca = C(-11) * t[1] + C(-4) * t[2];
    const C G = C(2) * t[10] - t[9];
    const C H = C(-2) * t[12] + t[11];
    E[0] = C(-2) * G + Ca;
    E[1] = (Ca + G) + H;
    E[2] = (Ca + G) - H;
    O[0] = C(-4) * t[4];
    O[1] = C(-4) * t[6];
    O[2] = C(-4) * t[8];
    const C Cd = C(8) * t[1] + t[2];
    const C J = t[9] + t[10], K = t[11] + t[12];
    const C L = Cd + J;
    const C b34 = L + K, b56 = L - K, b78 = C(-2) * J + Cd;
    E[3] = b34 + t[13]; E[4] = b34 - t[13];
    E[5] = b56 + t[15]; E[6] = b56 - t[15];
    E[7] = b78 + t[14]; E[8] = b78 - t[14];
    const C a = t[4] + t[16], b = t[6] - t[17];
    const C c = t[4] - t[16], d = t[8] + t[18];
    const C e = t[6] + t[17], f = t[8] - t[18];
    O[3] = a + b; O[4] = b - a;
    O[5] = c + d; O[6] = d - c;
    O[7] = e + f; O[8] = f - e;
}

// MRT (FluidDomain.f90:1236-1238) in moment space for one cell:
// g' = g + M^-1 S M (feq - g - Flb/2) + Flb, which is M_COLLID (feq - g) +
// M_FORCE Flb for M_COLLID = M^-1 S M and M_FORCE = I - M_COLLID/2
template <int P>
__device__ __forceinline__ void collide_mrt_mom(typename ST<P>::C g[Q], typename ST<P>::C rho,
                                                typename ST<P>::C drho, typename ST<P>::C u0,
                                                typename ST<P>::C u1, typename ST<P>::C u2,
                                                typename ST<P>::C F0, typename ST<P>::C F1,
                                                typename ST<P>::C F2, bool forced, typename ST<P>::C dh3,
                                                const typename ST<P>::C sd[Q]) {
    using C = typename ST<P>::C;
    constexpr bool OFF = ST<P>::OFF;
    const C k15 = C(1.5) * (u0 * u0 + u1 * u1 + u2 * u2);
    const C uF = u0 * F0 + u1 * F1 + u2 * F2;
    C flb[Q], r[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const C w = C(wt_(i));
        const C eu = edot3(i, u0, u1, u2);
        const C eq = OFF ? w * drho + (w * rho) * ((C(3) + C(4.5) * eu) * eu - k15)
                         : (w * rho) * ((C(1) - k15) + (C(3) + C(4.5) * eu) * eu);
        if (forced) {
            const C eF = edot3(i, F0, F1, F2);
            flb[i] = (dh3 * w) * ((eF - uF) + (C(3) * eu) * eF);
            r[i] = (eq - g[i]) - C(0.5) * flb[i];
        } else {
            flb[i] = C(0);
            r[i] = eq - g[i];
        }
    }
    C rs[9], rd[9], t[Q], E0, E[9], O[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const int i = pr_(k), o = opp_(i);
        rs[k] = r[i] + r[o];
        rd[k] = r[i] - r[o];
    }
    mrt_forward_c<C>(r[0], rs, rd, sd, t);
    mrt_backward_c<C>(t, E0, E, O);
    g[0] = g[0] + (E0 + flb[0]);
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const int i = pr_(k), o = opp_(i);
        g[i] = g[i] + ((E[k] + O[k]) + flb[i]);
        g[o] = g[o] + ((E[k] - O[k]) + flb[o]);
    }
}

// SRT/BGK without forcing, Omega folded into per-weight-class constants:
// per pair (i, opp) the post-collision values are
//   g_i' = (1-Om) g_i + S + A,  g_o' = (1-Om) g_o + S - A,
//   S = a_c + b_c (e.u)^2,  A = c_c (e.u),
// with a_c = Om w (rho (1 - 1.5 u^2)) [stored f] or Om w (drho - 1.5 rho u^2)
// [stored offsets], b_c = 4.5 Om w rho, c_c = 3 Om w rho.
template <int P>
__device__ __forceinline__ void collide_srt_free(typename ST<P>::C g[Q], typename ST<P>::C rho,
                                                 typename ST<P>::C drho, typename ST<P>::C u0,
                                                 typename ST<P>::C u1, typename ST<P>::C u2, typename ST<P>::C om) {
    using C = typename ST<P>::C;
    constexpr bool OFF = ST<P>::OFF;
    const C k15 = C(1.5) * (u0 * u0 + u1 * u1 + u2 * u2);
    const C omc = C(1) - om;
    const C base = OFF ? (drho - rho * k15) : rho * (C(1) - k15);
    const C orho = om * rho;
    // weight classes: 0 -> 1/3, 1 -> 1/18, 2 -> 1/36
    const C ac0 = (om * C(wt_(0))) * base;
    const C ac1 = (om * C(wt_(1))) * base, bc1 = C(4.5 * wt_(1)) * orho, cc1 = C(3.0 * wt_(1)) * orho;
    const C ac2 = (om * C(wt_(7))) * base, bc2 = C(4.5 * wt_(7)) * orho, cc2 = C(3.0 * wt_(7)) * orho;
    g[0] = omc * g[0] + ac0;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const int i = pr_(k), o = opp_(i);
        const bool cls1 = (i <= 6);
        const C eu = edot3(i, u0, u1, u2);
        const C Sm = (cls1 ? bc1 : bc2) * (eu * eu) + (cls1 ? ac1 : ac2);
        const C Am = (cls1 ? cc1 : cc2) * eu;
        const C gi = g[i], go = g[o];
        g[i] = omc * gi + (Sm + Am);
        g[o] = omc * go + (Sm - Am);
    }
}

// per-population element offsets, uniform across the grid: ld[i] = i*N
// (population stride) and st[i] = i*N + e_i.(1, Z, Z*Y) (the streaming
// displacement of an interior cell); the periodic wrap at the block faces is
// a per-thread correction added to the pointer
template <typename IT> struct Offs { IT ld[Q]; IT st[Q]; };

template <typename IT>
__device__ __forceinline__ IT wrap_corr(int e, IT cp, IT cm) { return e > 0 ? cp : (e < 0 ? cm : IT(0)); }

// per-launch scalars in the arithmetic type, converted on the host: GB300
// issues FP64 at a small fraction of the FP32 rate, so the FP32 kernels must
// not convert double parameters per thread
template <typename C> struct Scal { C om, dh, dh3, vf[3]; int forced; C om2, tau, nu, cles; };

// ---- TRT and the SRT collisions with a per-cell rate (LES) ----
// The rates follow smag / WALE / vrem (FluidDomain.f90:1265-1506) in the
// arithmetic type. WALE and Vreman scale their velocity-gradient tensors by
// the largest entry g before the products (OP is homogeneous of degree 1 in
// g), so that FP32 neither underflows nor overflows on quiet or violent
// flow; the fractional powers are written with square roots.

template <typename C>
__device__ __forceinline__ void neq_stress_c(const C neq[Q], C q[6]) {
    // fneq = -neq (FluidDomain.f90:1271-1276)
    q[0] = -(neq[1] + neq[2] + neq[7] + neq[8] + neq[9] + neq[10] + neq[11] + neq[12] + neq[13] + neq[14]);
    q[1] = -(neq[3] + neq[4] + neq[7] + neq[8] + neq[9] + neq[10] + neq[15] + neq[16] + neq[17] + neq[18]);
    q[2] = -(neq[5] + neq[6] + neq[11] + neq[12] + neq[13] + neq[14] + neq[15] + neq[16] + neq[17] + neq[18]);
    q[3] = -((neq[7] - neq[8]) - (neq[9] - neq[10]));
    q[4] = -((neq[11] - neq[12]) - (neq[13] - neq[14]));
    q[5] = -((neq[15] - neq[16]) - (neq[17] - neq[18]));
}

// the velocity field and tau_all of the per-cell-rate models in the
// arithmetic type: FP32 arrays for the offset forms (GB300 converts between
// FP64 and FP32 on its FP64 pipe), FP64 arrays for FSI_PREC_F64_FAST
template <int P> __device__ __forceinline__ typename ST<P>::C uval(const StepArgs &a, long long i) {
    if (ST<P>::OFF) return a.uf[i];
    else return (typename ST<P>::C)a.u[i];
}
template <int P> __device__ __forceinline__ typename ST<P>::C tau_get(const StepArgs &a, long long c) {
    if (ST<P>::OFF) return a.tauf_prev[c];
    else return (typename ST<P>::C)a.tau_all[c];
}
template <int P> __device__ __forceinline__ void tau_put(const StepArgs &a, long long c, typename ST<P>::C v) {
    if (ST<P>::OFF) a.tauf[c] = (float)v;
    else a.tau_all[c] = (double)v;
}

// center_diff / onesid_diff of velocity component k along axis d, times dh
template <int P>
__device__ __forceinline__ typename ST<P>::C les_diff_c(const StepArgs &a, int k, int d, int z, int y, int x,
                                                        long long c, typename ST<P>::C dh) {
    using C = typename ST<P>::C;
    const long long b = a.N * k + c;
    const int i = d == 0 ? x : (d == 1 ? y : z);
    const int D = d == 0 ? a.X : (d == 1 ? a.Y : a.Z);
    const long long s = d == 0 ? (long long)a.Z * a.Y : (d == 1 ? (long long)a.Z : 1LL);
    if (i > 0 && i < D - 1) return (uval<P>(a, b + s) - uval<P>(a, b - s)) * dh;
    const long long s1 = i == 0 ? s : -s;
    return ((C(4) * uval<P>(a, b + s1) - C(3) * uval<P>(a, b)) - uval<P>(a, b + 2 * s1)) * dh;
}

template <typename C> __device__ __forceinline__ C pw15(C x) { return x * sqrt(x); }
template <typename C> __device__ __forceinline__ C pw25(C x) { return (x * x) * sqrt(x); }
template <typename C> __device__ __forceinline__ C pw125(C x) { return x * sqrt(sqrt(x)); }

// WALE's relaxation time from S_ij (the strain rate of the non-equilibrium
// stress) and O12, O13, O23 (FluidDomain.f90:1337-1413), the tensors scaled by
// their largest entry before the products
template <typename C>
__device__ __forceinline__ C wale_tau(const Scal<C> &sc, C S11, C S22, C S33, C S12, C S13, C S23, C O12, C O13,
                                      C O23) {
    C g = fmax(fmax(fmax(fabs(S11), fabs(S22)), fmax(fabs(S33), fabs(S12))),
               fmax(fmax(fabs(S13), fabs(S23)), fmax(fmax(fabs(O12), fabs(O13)), fabs(O23))));
    C OP = C(0);
    if (g > C(0)) {
        const C ig = C(1) / g;
        S11 *= ig; S22 *= ig; S33 *= ig; S12 *= ig; S13 *= ig; S23 *= ig;
        O12 *= ig; O13 *= ig; O23 *= ig;
        const C S = S11 * S11 + S22 * S22 + S33 * S33 + C(2) * (S12 * S12 + S13 * S13 + S23 * S23);
        const C O = C(2) * (O12 * O12 + O23 * O23 + O13 * O13);
        const C a12 = O12 * O12, a13 = O13 * O13, a23 = O23 * O23;
        const C SO11 = -((S11 * S11 + S12 * S12 + S13 * S13) * (a12 + a13));
        const C SO22 = -((S12 * S12 + S22 * S22 + S23 * S23) * (a12 + a23));
        const C SO33 = -((S13 * S13 + S23 * S23 + S33 * S33) * (a13 + a23));
        const C SO12 = -((S11 * S12 + S12 * S22 + S13 * S23) * (O13 * O23));
        const C SO13 = (S11 * S13 + S12 * S23 + S13 * S33) * (O12 * O23);
        const C SO23 = -((S12 * S13 + S22 * S23 + S23 * S33) * (O12 * O13));
        const C SO = SO11 + SO22 + SO33 + C(2) * (SO12 + SO13 + SO23);
        const C SdSd = (S * S + O * O) * C(1.0 / 6.0) + C(2.0 / 3.0) * S * O + C(2) * SO;
        OP = g * (pw15(SdSd) / (pw25(S) + pw125(SdSd)));
        if (!(OP >= C(0)) || !isfinite(OP)) OP = C(0);
    }
    return (sc.nu + sc.cles * OP * sc.dh * sc.dh) / (sc.dh * C(1.0 / 3.0)) + C(0.5);
}

// The gradient pass of the fast forms (after the velocity pass): Vreman's
// relaxation time (vrem, FluidDomain.f90:1428-1506), or WALE's rotation-rate
// entries (:1341-1391), from the neighbours' velocity, one thread per cell.
template <int P, int MODEL>
__global__ void __launch_bounds__(256) k_les_grad(StepArgs a, Scal<typename ST<P>::C> sc) {
    using C = typename ST<P>::C;
    const int z = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, x = blockIdx.z;
    if (z >= a.Z) return;
    const long long c = cidx(z, y, x, a.Z, a.Y);
    if constexpr (MODEL == CM_WALE) {
        const C ox = C(0.5) * (les_diff_c<P>(a, 2, 1, z, y, x, c, sc.dh) - les_diff_c<P>(a, 1, 2, z, y, x, c, sc.dh));
        const C oy = C(0.5) * (les_diff_c<P>(a, 0, 2, z, y, x, c, sc.dh) - les_diff_c<P>(a, 2, 0, z, y, x, c, sc.dh));
        const C oz = C(0.5) * (les_diff_c<P>(a, 1, 0, z, y, x, c, sc.dh) - les_diff_c<P>(a, 0, 1, z, y, x, c, sc.dh));
        C *og = (C *)a.og;
        og[c] = C(-0.5) * oz;
        og[c + a.N] = C(0.5) * oy;
        og[c + 2 * a.N] = C(-0.5) * ox;
    } else {
        C m[3][3];
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int i = 0; i < 3; i++) m[i][j] = C(0.5) * les_diff_c<P>(a, i, j, z, y, x, c, sc.dh);
        C g = C(0);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) g = fmax(g, fabs(m[i][j]));
        C OP = C(0);
        if (g > C(0)) {
            const C ig = C(1) / g;
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) m[i][j] *= ig;
            const C r0 = m[0][0] * m[0][0] + m[0][1] * m[0][1] + m[0][2] * m[0][2];
            const C r1 = m[1][0] * m[1][0] + m[1][1] * m[1][1] + m[1][2] * m[1][2];
            const C r2 = m[2][0] * m[2][0] + m[2][1] * m[2][1] + m[2][2] * m[2][2];
            const C d01 = m[0][0] * m[1][0] + m[0][1] * m[1][1] + m[0][2] * m[1][2];
            const C d02 = m[0][0] * m[2][0] + m[0][1] * m[2][1] + m[0][2] * m[2][2];
            const C d12 = m[1][0] * m[2][0] + m[1][1] * m[2][1] + m[1][2] * m[2][2];
            const C bb = (r0 * r1 - d01 * d01) + (r0 * r2 - d02 * d02) + (r1 * r2 - d12 * d12);
            OP = g * sqrt(bb / (r0 + r1 + r2));
            if (!isfinite(OP)) OP = C(0);
        }
        tau_put<P>(a, c, (sc.nu + sc.cles * OP * sc.dh * sc.dh) / (sc.dh * C(1.0 / 3.0)) + C(0.5));
    }
}

template <int P, int MODEL>
__device__ __forceinline__ typename ST<P>::C les_rate_c(const StepArgs &a, const Scal<typename ST<P>::C> &sc,
                                                        const typename ST<P>::C neq[Q], typename ST<P>::C rho, int z,
                                                        int y, int x, long long c) {
    using C = typename ST<P>::C;
    C t;
    if (MODEL == CM_SMAG) {
        C q[6];
        neq_stress_c(neq, q);
        const C QQ = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + C(2) * (q[3] * q[3] + q[4] * q[4] + q[5] * q[5]);
        const C tau_t = sqrt(sc.tau * sc.tau + sc.cles * sqrt(QQ) / rho);
        tau_put<P>(a, c, C(0.5) * (sc.tau + tau_t));
        return C(2) / (sc.tau + tau_t);
    } else if (MODEL == CM_WALE) {
        C q[6];
        neq_stress_c(neq, q);
        const C k = -(C(1.5) * sc.dh) / (rho * tau_get<P>(a, c));
        const C *og = (const C *)a.og;
        t = wale_tau<C>(sc, k * q[0], k * q[1], k * q[2], k * q[3], k * q[4], k * q[5], og[c], og[c + a.N],
                        og[c + 2 * a.N]);
    } else {
        // Vreman: the gradient pass wrote tau_all
        return C(1) / tau_get<P>(a, c);
    }
    tau_put<P>(a, c, t);
    return C(1) / t;
}

// TRT (FluidDomain.f90:1228-1235) and the per-cell-rate SRT collisions
// (:1239-1262) with Guo forcing on one cell
template <int P, int MODEL>
__device__ __forceinline__ void collide_rate(typename ST<P>::C g[Q], typename ST<P>::C rho, typename ST<P>::C drho,
                                             typename ST<P>::C u0, typename ST<P>::C u1, typename ST<P>::C u2,
                                             typename ST<P>::C F0, typename ST<P>::C F1, typename ST<P>::C F2,
                                             const Scal<typename ST<P>::C> &sc, const StepArgs &a, int x, int y,
                                             int z, long long c) {
    using C = typename ST<P>::C;
    constexpr bool OFF = ST<P>::OFF;
    const C k15 = C(1.5) * (u0 * u0 + u1 * u1 + u2 * u2);
    const C uF = u0 * F0 + u1 * F1 + u2 * F2;
    C neq[Q], flb[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const C w = C(wt_(i));
        const C eu = edot3(i, u0, u1, u2);
        const C eq = OFF ? w * drho + (w * rho) * ((C(3) + C(4.5) * eu) * eu - k15)
                         : (w * rho) * ((C(1) - k15) + (C(3) + C(4.5) * eu) * eu);
        neq[i] = eq - g[i];
        const C eF = edot3(i, F0, F1, F2);
        flb[i] = (sc.dh3 * w) * (eF - uF + C(3) * eu * eF);
    }
    if (MODEL == CM_TRT) {
        const C om = sc.om, om2 = sc.om2;
        const C hp = C(0.5) * om, hm = C(0.5) * om2, fp = C(0.5) - C(0.25) * om, fm = C(0.5) - C(0.25) * om2;
        g[0] += om * neq[0] + (C(1) - C(0.5) * om) * flb[0];
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const int p = pr_(k), m = opp_(p);
            const C sp = hp * (neq[p] + neq[m]) + fp * (flb[p] + flb[m]);
            const C sm = hm * (neq[p] - neq[m]) + fm * (flb[p] - flb[m]);
            g[p] += sp + sm;
            g[m] += sp - sm;
        }
    } else {
        const C om = les_rate_c<P, MODEL>(a, sc, neq, rho, z, y, x, c);
        const C cf = C(1) - C(0.5) * om;
#pragma unroll
        for (int i = 0; i < Q; i++) g[i] += om * neq[i] + cf * flb[i];
    }
}

template <int P, int MODEL, bool HOOKS, typename IT>
__global__ void __launch_bounds__(TPB) k_step_fast(StepArgs a, MatsT<typename ST<P>::C> mm, Offs<IT> of,
                                                   Scal<typename ST<P>::C> sc) {
    using T = ST<P>;
    using S = typename T::S;
    using C = typename T::C;
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int x = blockIdx.z;
    if (z >= a.Z || y >= a.Y) return;
    const int X = a.X, Y = a.Y, Z = a.Z;
    const long long N = a.N;
    const IT c = (IT)z + (IT)Z * ((IT)y + (IT)Y * (IT)x);
    const S *__restrict__ sp = (const S *)a.src + c;
    // IT = int: the buffer spans less than 4 GiB and every access is a 32-bit
    // byte offset from its base (as in the paired kernel)
    constexpr bool U32 = sizeof(IT) == 4;

    C g[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) {
        if constexpr (U32)
            g[i] = T::dec(__ldcs((const S *)((const char *)a.src + (unsigned)(c + of.ld[i]) * (unsigned)sizeof(S))));
        else
            g[i] = T::dec(__ldcs(sp + of.ld[i]));
    }

    C rho, drho, u0, u1, u2, F0 = C(0), F1 = C(0), F2 = C(0);
    bool forced = false;
    const Win &w = a.win;
    if (HOOKS && x >= w.x0 && x <= w.x1 && y >= w.y0 && y <= w.y1 && z >= w.z0 && z <= w.z1) {
        long long wc = (long long)(z - w.z0) + (long long)w.WZ * ((long long)(y - w.y0) + (long long)w.WY * (x - w.x0));
        const double d = w.den[wc];
        if (T::OFF) { drho = (C)(d - 1.0); rho = C(1) + drho; }
        else { rho = (C)d; drho = rho - C(1); }
        u0 = (C)w.u[wc]; u1 = (C)w.u[wc + w.n]; u2 = (C)w.u[wc + 2 * w.n];
        F0 = (C)w.force[wc]; F1 = (C)w.force[wc + w.n]; F2 = (C)w.force[wc + 2 * w.n];
        forced = true;
    } else {
        macro_fast<P>(g, sc.vf, sc.dh, rho, drho, u0, u1, u2);
        F0 = sc.vf[0]; F1 = sc.vf[1]; F2 = sc.vf[2];
        forced = sc.forced != 0;
    }
    if (HOOKS && !(grad_model(MODEL) && !T::OFF) &&
        ((a.l2[0] && x == 1) || (a.l2[1] && x == X - 2) || (a.l2[2] && y == 1) || (a.l2[3] && y == Y - 2) ||
         (a.l2[4] && z == 1) || (a.l2[5] && z == Z - 2))) {
        a.den[c] = T::OFF ? 1.0 + (double)drho : (double)rho;
        a.u[c] = (double)u0; a.u[c + N] = (double)u1; a.u[c + 2 * N] = (double)u2;
    }
    const C om = sc.om, dh3 = sc.dh3;
    if constexpr (MODEL == CM_SRT) {
        if (forced) collide_srt<P, true>(g, rho, drho, u0, u1, u2, F0, F1, F2, om, dh3);
        else collide_srt_free<P>(g, rho, drho, u0, u1, u2, om);
    } else if constexpr (MODEL == CM_MRT) {
        collide_mrt<P>(g, rho, drho, u0, u1, u2, F0, F1, F2, forced, dh3, mm);
    } else if constexpr (MODEL == CM_MRT_MOM) {
        collide_mrt_mom<P>(g, rho, drho, u0, u1, u2, F0, F1, F2, forced, dh3, mm.sd);
    } else {
        collide_rate<P, MODEL>(g, rho, drho, u0, u1, u2, F0, F1, F2, sc, a, x, y, z, (long long)c);
    }

    if (HOOKS) {
        // halfwayBCset_ (FluidDomain.f90:567-614): post-collision faces as FP64 f
#define FSI_HW(K, COND, OFS)                                                       \
        if (a.hw[K] && (COND)) {                                                   \
            double *h = a.hw[K] + (long long)Q * (OFS);                            \
            _Pragma("unroll") for (int i = 0; i < Q; i++)                          \
                h[i] = T::OFF ? (double)g[i] + wt_(i) : (double)g[i];              \
        }
        FSI_HW(0, x == 0, z + (long long)Z * y)
        FSI_HW(1, x == X - 1, z + (long long)Z * y)
        FSI_HW(2, y == 0, z + (long long)Z * x)
        FSI_HW(3, y == Y - 1, z + (long long)Z * x)
        FSI_HW(4, z == 0, y + (long long)Y * x)
        FSI_HW(5, z == Z - 1, y + (long long)Y * x)
#undef FSI_HW
    }

    // push: destination = c + st[i] + wrap correction (periodic in all axes)
    const IT ZY = (IT)Z * (IT)Y, NN = (IT)N;
    const IT czp = (z == Z - 1) ? -(IT)Z : 0, czm = (z == 0) ? (IT)Z : 0;
    const IT cyp = (y == Y - 1) ? -ZY : 0, cym = (y == 0) ? ZY : 0;
    const IT cxp = (x == X - 1) ? -NN : 0, cxm = (x == 0) ? NN : 0;
    S *__restrict__ dp = (S *)a.dst + c;
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const IT corr = wrap_corr(ez_(i), czp, czm) + wrap_corr(ey_(i), cyp, cym) + wrap_corr(ex_(i), cxp, cxm);
        if constexpr (U32)
            __stcs((S *)((char *)a.dst + (unsigned)(c + corr + of.st[i]) * (unsigned)sizeof(S)), T::enc(g[i]));
        else
            __stcs((dp + corr) + of.st[i], T::enc(g[i]));
    }
}

#if FSI_FAST_PREC == FSI_PREC_F64_DW
// ---------------------------------------------------------------------------
// The double-word form's bulk step without hooks (no IB window, half-way or
// 102 faces) and with an even z extent: each thread takes the cells z, z+1
// (z even) in one dw2, so that every double-word operation serves two cells
// with packed FP32x2 instructions. Loads are 16-byte pairs of FP64; a
// population that streams along z lands on an odd offset and is stored as two
// FP64 values. Same physics and step as k_step_fast (push scheme, periodic
// wrap, uniform volume force).
// ---------------------------------------------------------------------------
constexpr int TPB_DW2 = 128;
struct SdT { dw2 sd[Q]; };

// resident CTAs per SM (the register budget), measured on GB300 (256^3 TGV):
// SRT 3 (165 registers, no spill); unforced MRT 4 (128 registers with about
// 450 bytes of spill: 6.7k MLUPS, against 6.3k at 2 CTAs with 244 registers
// and 6.1k at 3); forced MRT 2
#ifndef FSI_DW2_MINB_MRT
#define FSI_DW2_MINB_MRT 4
#endif
// FORCED (MRT): a nonzero volume force, compiled apart, so that the
// unforced step does not carry the forcing terms' registers
template <int MODEL, typename IT, bool FORCED>
__global__ void __launch_bounds__(TPB_DW2, MODEL == CM_SRT ? 3 : (FORCED ? 2 : FSI_DW2_MINB_MRT))
k_step_dw2(StepArgs a, Offs<IT> of, Scal<dw2> sc, SdT sdt) {
    const int zp = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int x = blockIdx.z;
    const int X = a.X, Y = a.Y, Z = a.Z;
    const int z = 2 * zp;
    if (z >= Z || y >= Y) return;
    const long long N = a.N;
    const IT c = (IT)z + (IT)Z * ((IT)y + (IT)Y * (IT)x);
    constexpr bool U32 = sizeof(IT) == 4;
    dw2 g[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) {
        double2 v;
        if constexpr (U32)
            v = __ldcs((const double2 *)((const char *)a.src + (unsigned)(c + of.ld[i]) * 8u));
        else
            v = __ldcs((const double2 *)((const double *)a.src + (c + of.ld[i])));
        const dw d0 = dw_from_f64(v.x), d1 = dw_from_f64(v.y);
        g[i] = dw2(make_float2(d0.h, d1.h), make_float2(d0.l, d1.l), 0);
    }
    dw2 rho, drho, u0, u1, u2;
    macro_fast<PDW2>(g, sc.vf, sc.dh, rho, drho, u0, u1, u2);
    if constexpr (MODEL == CM_SRT) {
        // (one SRT kernel with the forcing branch measured faster than two)
        if (sc.forced) collide_srt<PDW2, true>(g, rho, drho, u0, u1, u2, sc.vf[0], sc.vf[1], sc.vf[2], sc.om, sc.dh3);
        else collide_srt_free<PDW2>(g, rho, drho, u0, u1, u2, sc.om);
    } else {
        collide_mrt_mom<PDW2>(g, rho, drho, u0, u1, u2, sc.vf[0], sc.vf[1], sc.vf[2], FORCED, sc.dh3, sdt.sd);
    }
    // push: destination = c + st[i] + the periodic wrap of each cell
    const IT ZY = (IT)Z * (IT)Y, NN = (IT)N;
    const IT cyp = (y == Y - 1) ? -ZY : 0, cym = (y == 0) ? ZY : 0;
    const IT cxp = (x == X - 1) ? -NN : 0, cxm = (x == 0) ? NN : 0;
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const double d0 = dw_to_f64(dw(g[i].h.x, g[i].l.x, 0)), d1 = dw_to_f64(dw(g[i].h.y, g[i].l.y, 0));
        const IT cxy = wrap_corr(ey_(i), cyp, cym) + wrap_corr(ex_(i), cxp, cxm);
        const IT o = c + cxy + of.st[i];
        if (ez_(i) == 0) {
            if constexpr (U32) __stcs((double2 *)((char *)a.dst + (unsigned)o * 8u), make_double2(d0, d1));
            else __stcs((double2 *)((double *)a.dst + o), make_double2(d0, d1));
        } else {
            // cell z streams to z + ez, cell z+1 to z+1+ez; only z = 0 (ez < 0)
            // and z+1 = Z-1 (ez > 0) wrap
            const IT w0 = (ez_(i) < 0 && z == 0) ? (IT)Z : 0;
            const IT w1 = (ez_(i) > 0 && z + 1 == Z - 1) ? -(IT)Z : 0;
            if constexpr (U32) {
                __stcs((double *)((char *)a.dst + (unsigned)(o + w0) * 8u), d0);
                __stcs((double *)((char *)a.dst + (unsigned)(o + 1 + w1) * 8u), d1);
            } else {
                __stcs((double *)a.dst + (o + w0), d0);
                __stcs((double *)a.dst + (o + 1 + w1), d1);
            }
        }
    }
}

template <int MODEL, typename IT>
cudaError_t dw2_launch(const StepArgs &a, const MrtMats *mm, cudaStream_t st) {
    Offs<IT> of{};
    const long long ZY = (long long)a.Z * a.Y;
    for (int i = 0; i < Q; i++) {
        of.ld[i] = (IT)((long long)i * a.N);
        of.st[i] = (IT)((long long)i * a.N + ez_(i) + (long long)a.Z * ey_(i) + ZY * ex_(i));
    }
    const int Zp = a.Z / 2;
    int bz = Zp >= TPB_DW2 ? TPB_DW2 : ((Zp + 31) / 32) * 32;
    int by = TPB_DW2 / bz;
    if (by < 1) by = 1;
    dim3 blk(bz, by), grd((Zp + bz - 1) / bz, (a.Y + by - 1) / by, a.X);
    Scal<dw2> sc{};
    sc.om = dw2(a.omega);
    sc.dh = dw2(a.dh);
    sc.dh3 = dw2(3.0 * a.dh);
    for (int k = 0; k < 3; k++) sc.vf[k] = dw2(a.vf[k]);
    sc.forced = (a.vf[0] != 0.0 || a.vf[1] != 0.0 || a.vf[2] != 0.0) ? 1 : 0;
    SdT sdt{};
    for (int k = 0; k < Q; k++) sdt.sd[k] = dw2(mm->sd[k]);
    if (sc.forced && MODEL != CM_SRT) k_step_dw2<MODEL, IT, true><<<grd, blk, 0, st>>>(a, of, sc, sdt);
    else k_step_dw2<MODEL, IT, false><<<grd, blk, 0, st>>>(a, of, sc, sdt);
    return cudaGetLastError();
}
#endif

// ---------------------------------------------------------------------------
// Paired-cell form of the step for the offset storage forms (FP32, FP16,
// BF16), SRT or MRT, with or without the IB window and face hooks: each thread
// owns the two z-adjacent cells (z0, z0+1), z0 even. Loads and stores move
// both cells in one 32-bit (FP16/BF16) or 64-bit (FP32) access and all
// arithmetic runs on packed FP32x2 (fma.rn.f32x2, sm_100 and later), so one
// instruction serves both cells. A CTA holds whole z-rows; the +-z streaming
// shift goes through shared memory, the +-y/+-x shift moves whole rows.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 f2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.0f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return __fmul2_rn(a, f2(-1.0f)); }

template <int P> struct V2;
template <> struct V2<FSI_PREC_F32> {
    using S2 = float2; using S = float;
    static __device__ __forceinline__ float2 dec(S2 s) { return s; }
    static __device__ __forceinline__ S2 enc(float2 c) { return c; }
    static __device__ __forceinline__ S lo(S2 s) { return s.x; }
    static __device__ __forceinline__ S hi(S2 s) { return s.y; }
    static __device__ __forceinline__ S2 pack(S a, S b) { return make_float2(a, b); }
    static __device__ __forceinline__ float dec1(S s) { return s; }
    static __device__ __forceinline__ S enc1(float c) { return c; }
};
template <> struct V2<FSI_PREC_F16> {
    using S2 = __half2; using S = __half;
    static __device__ __forceinline__ float2 dec(S2 s) { return __half22float2(s); }
    static __device__ __forceinline__ S2 enc(float2 c) { return __float22half2_rn(c); }
    static __device__ __forceinline__ S lo(S2 s) { return __low2half(s); }
    static __device__ __forceinline__ S hi(S2 s) { return __high2half(s); }
    static __device__ __forceinline__ S2 pack(S a, S b) { return __halves2half2(a, b); }
    static __device__ __forceinline__ float dec1(S s) { return __half2float(s); }
    static __device__ __forceinline__ S enc1(float c) { return __float2half_rn(c); }
};
template <> struct V2<FSI_PREC_BF16> {
    using S2 = __nv_bfloat162; using S = __nv_bfloat16;
    static __device__ __forceinline__ float2 dec(S2 s) { return __bfloat1622float2(s); }
    static __device__ __forceinline__ S2 enc(float2 c) { return __float22bfloat162_rn(c); }
    static __device__ __forceinline__ S lo(S2 s) { return __low2bfloat16(s); }
    static __device__ __forceinline__ S hi(S2 s) { return __high2bfloat16(s); }
    static __device__ __forceinline__ S2 pack(S a, S b) { return __halves2bfloat162(a, b); }
    static __device__ __forceinline__ float dec1(S s) { return __bfloat162float(s); }
    static __device__ __forceinline__ S enc1(float c) { return __float2bfloat16_rn(c); }
};

// index of z-moving population i among the ten with ez != 0
__host__ __device__ constexpr int zslot_(int i) {
    return i == 5 ? 0 : i == 6 ? 1 : i == 11 ? 2 : i == 12 ? 3 : i == 13 ? 4 : i == 14 ? 5
         : i == 15 ? 6 : i == 16 ? 7 : i == 17 ? 8 : i == 18 ? 9 : -1;
}

// moment-space MRT: S_k / |row k|^2 for every moment (zero on conserved ones)
struct MrtS { float sd[Q]; };

// accumulator of integer-weighted terms; the weights are compile-time
// constants after unrolling, so zero terms vanish and +-1 become add/sub
struct Acc2 {
    float2 v;
    bool set;
};
__device__ __forceinline__ void acc_add(Acc2 &a, int c, float2 x) {
    if (c == 0) return;
    if (!a.set) {
        a.v = c == 1 ? x : (c == -1 ? neg2(x) : mul2(f2((float)c), x));
        a.set = true;
    } else {
        a.v = c == 1 ? add2(a.v, x) : (c == -1 ? sub2(a.v, x) : fma2(f2((float)c), x, a.v));
    }
}
__device__ __forceinline__ float2 acc_val(const Acc2 &a) { return a.set ? a.v : f2(0.0f); }

__device__ __forceinline__ float2 edot(int i, float2 v0, float2 v1, float2 v2) {
    Acc2 a{f2(0.0f), false};
    acc_add(a, ex_(i), v0);
    acc_add(a, ey_(i), v1);
    acc_add(a, ez_(i), v2);
    return acc_val(a);
}

__device__ __forceinline__ void setl(float2 &v, int l, float s) {
    if (l == 0) v.x = s;
    else v.y = s;
}
__device__ __forceinline__ float getl(float2 v, int l) { return l == 0 ? v.x : v.y; }

// density offset, density and momentum of two cells (offsets: rho = 1 + sum g)
__device__ __forceinline__ void macro2(const float2 g[Q], float2 &drho, float2 &rho, float2 &jx, float2 &jy,
                                       float2 &jz) {
    float2 s = g[0];
    jx = f2(0.f); jy = f2(0.f); jz = f2(0.f);
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const int i = pr_(k), o = opp_(i);
        const float2 sk = add2(g[i], g[o]), dk = sub2(g[i], g[o]);
        s = add2(s, sk);
        if (ex_(i)) jx = ex_(i) > 0 ? add2(jx, dk) : sub2(jx, dk);
        if (ey_(i)) jy = ey_(i) > 0 ? add2(jy, dk) : sub2(jy, dk);
        if (ez_(i)) jz = ez_(i) > 0 ? add2(jz, dk) : sub2(jz, dk);
    }
    drho = s;
    rho = add2(f2(1.0f), s);
}

// velocity with the half-force shift of Guo forcing (calculate_macro_quantities_)
template <bool FORCED>
__device__ __forceinline__ void vel2(float2 rho, float2 jx, float2 jy, float2 jz, float2 F0, float2 F1, float2 F2,
                                     float h, float2 &u0, float2 &u1, float2 &u2) {
    const float2 inv = make_float2(__fdividef(1.0f, rho.x), __fdividef(1.0f, rho.y));
    if (FORCED) {
        u0 = mul2(fma2(f2(h), F0, jx), inv);
        u1 = mul2(fma2(f2(h), F1, jy), inv);
        u2 = mul2(fma2(f2(h), F2, jz), inv);
    } else {
        u0 = mul2(jx, inv); u1 = mul2(jy, inv); u2 = mul2(jz, inv);
    }
}

// The moment transform of the D3Q19 basis (mrow_) written out by velocity
// class, for the pair layout of the paired kernels: r0 (rest), rs[k] = r_i +
// r_o and rd[k] = r_i - r_o for the nine pairs in pr_ order (x, y, z axes;
// diagonals (1,1,0), (-1,1,0), (1,0,1), (-1,0,1), (0,1,1), (0,-1,1)).
// Shared partial sums (axis / diagonal class sums and pair combinations)
// replace the direct 19-term rows: about 40 packed operations each way
// instead of about 80. The conserved moments 0, 3, 5, 7 are not formed.
// t[k] = sd[k] m_k (relaxation rate over |row k|^2).
__device__ __forceinline__ void mrt_forward(float2 r0, const float2 rs[9], const float2 rd[9], const MrtS &ms,
                                            float2 t[Q]) {
    // even moments from the pair sums
    const float2 Ax = rs[0], Ay = rs[1], Az = rs[2];
    const float2 Dxy = add2(rs[3], rs[4]), Dxz = add2(rs[5], rs[6]), Dyz = add2(rs[7], rs[8]);
    const float2 A = add2(add2(Ax, Ay), Az), D = add2(add2(Dxy, Dxz), Dyz);
    const float2 m1 = fma2(f2(-30.0f), r0, fma2(f2(-11.0f), A, mul2(f2(8.0f), D)));
    const float2 m2 = fma2(f2(12.0f), r0, fma2(f2(-4.0f), A, D));
    const float2 U = add2(Ay, Az), V = fma2(f2(-2.0f), Dyz, add2(Dxy, Dxz));
    const float2 m9 = fma2(f2(2.0f), Ax, sub2(V, U));
    const float2 m10 = fma2(f2(-4.0f), Ax, fma2(f2(2.0f), U, V));
    const float2 W = sub2(Ay, Az), Xd = sub2(Dxy, Dxz);
    const float2 m11 = add2(W, Xd);
    const float2 m12 = fma2(f2(-2.0f), W, Xd);
    const float2 m13 = sub2(rs[3], rs[4]), m14 = sub2(rs[7], rs[8]), m15 = sub2(rs[5], rs[6]);
    // odd moments from the pair differences
    const float2 p3 = sub2(rd[3], rd[4]), q3 = add2(rd[3], rd[4]);
    const float2 p5 = sub2(rd[5], rd[6]), q5 = add2(rd[5], rd[6]);
    const float2 p7 = sub2(rd[7], rd[8]), q7 = add2(rd[7], rd[8]);
    const float2 m4 = fma2(f2(-4.0f), rd[0], add2(p3, p5));
    const float2 m16 = sub2(p3, p5);
    const float2 m6 = fma2(f2(-4.0f), rd[1], add2(q3, p7));
    const float2 m17 = sub2(p7, q3);
    const float2 m8 = fma2(f2(-4.0f), rd[2], add2(q5, q7));
    const float2 m18 = sub2(q5, q7);
    t[0] = t[3] = t[5] = t[7] = f2(0.0f);
    t[1] = mul2(f2(ms.sd[1]), m1);
    t[2] = mul2(f2(ms.sd[2]), m2);
    t[4] = mul2(f2(ms.sd[4]), m4);
    t[6] = mul2(f2(ms.sd[6]), m6);
    t[8] = mul2(f2(ms.sd[8]), m8);
    t[9] = mul2(f2(ms.sd[9]), m9);
    t[10] = mul2(f2(ms.sd[10]), m10);
    t[11] = mul2(f2(ms.sd[11]), m11);
    t[12] = mul2(f2(ms.sd[12]), m12);
    t[13] = mul2(f2(ms.sd[13]), m13);
    t[14] = mul2(f2(ms.sd[14]), m14);
    t[15] = mul2(f2(ms.sd[15]), m15);
    t[16] = mul2(f2(ms.sd[16]), m16);
    t[17] = mul2(f2(ms.sd[17]), m17);
    t[18] = mul2(f2(ms.sd[18]), m18);
}

// Delta = M^T t split by parity: Delta_0 = E0; for pair k with representative
// i: Delta_i = E[k] + O[k], Delta_opp(i) = E[k] - O[k]
__device__ __forceinline__ void mrt_backward(const float2 t[Q], float2 &E0, float2 E[9], float2 O[9]) {
    E0 = fma2(f2(-30.0f), t[1], mul2(f2(12.0f), t[2]));
    // axes
    const float2 Ca = fma2(f2(-11.0f), t[1], mul2(f2(-4.0f), t[2]));
    const float2 G = fma2(f2(2.0f), t[10], neg2(t[9]));
    const float2 H = fma2(f2(-2.0f), t[12], t[11]);
    E[0] = fma2(f2(-2.0f), G, Ca);
    E[1] = add2(add2(Ca, G), H);
    E[2] = sub2(add2(Ca, G), H);
    O[0] = mul2(f2(-4.0f), t[4]);
    O[1] = mul2(f2(-4.0f), t[6]);
    O[2] = mul2(f2(-4.0f), t[8]);
    // diagonals
    const float2 Cd = fma2(f2(8.0f), t[1], t[2]);
    const float2 J = add2(t[9], t[10]), K = add2(t[11], t[12]);
    const float2 L = add2(Cd, J);
    const float2 b34 = add2(L, K), b56 = sub2(L, K), b78 = fma2(f2(-2.0f), J, Cd);
    E[3] = add2(b34, t[13]);
    E[4] = sub2(b34, t[13]);
    E[5] = add2(b56, t[15]);
    E[6] = sub2(b56, t[15]);
    E[7] = add2(b78, t[14]);
    E[8] = sub2(b78, t[14]);
    const float2 a = add2(t[4], t[16]), b = sub2(t[6], t[17]);
    const float2 c = sub2(t[4], t[16]), d = add2(t[8], t[18]);
    const float2 e = add2(t[6], t[17]), f = sub2(t[8], t[18]);
    O[3] = add2(a, b);
    O[4] = sub2(b, a);
    O[5] = add2(c, d);
    O[6] = sub2(d, c);
    O[7] = add2(e, f);
    O[8] = sub2(f, e);
}

// the collision of two cells (offset storage, FP32x2): SRT (FluidDomain.f90:
// 1218-1227, Omega folded per weight class) or MRT (:1236-1238) in moment
// space, g' = g + M^-1 S M (feq - g - Flb/2) + Flb, which is M_COLLID (feq - g)
// + M_FORCE Flb for M_FORCE = I - M_COLLID/2. Opposite velocities are handled
// as sums (even moments) and differences (odd moments). Each post-collision
// population goes to emit(i, value) as soon as it is known, so that the
// caller can store it at once. With KEEPG false the MRT form does not keep g
// past the moment transform (g = feq - Flb/2 - r is rebuilt from the sums it
// keeps); with KEEPG true it adds Delta + Flb to the g it kept.
template <int MODEL, bool FORCED, bool KEEPG, class EMIT>
__device__ __forceinline__ void collide_emit(const float2 g[Q], float2 rho, float2 drho, float2 u0, float2 u1,
                                             float2 u2, float2 F0, float2 F1, float2 F2, const Scal<float> &sc,
                                             const MrtS &ms, EMIT &&emit, float2 *tau_rel = nullptr,
                                             const float2 *les_in = nullptr) {
    const float om = sc.om;
    const float2 k15 = mul2(f2(1.5f), fma2(u0, u0, fma2(u1, u1, mul2(u2, u2))));
    float2 uF = f2(0.f);
    if (FORCED) uF = fma2(u0, F0, fma2(u1, F1, mul2(u2, F2)));
    const float w0 = (float)wt_(0), w1 = (float)wt_(1), w2 = (float)wt_(7);
    // per pair: fsum = feq_i + feq_o, fdif = feq_i - feq_o,
    // FS = (Flb_i + Flb_o)/2, FA = (Flb_i - Flb_o)/2
    auto pair_terms = [&](int i, float2 &fsum, float2 &fdif, float2 &FS, float2 &FA) {
        const float w = (float)wt_(i);
        const float2 eu = edot(i, u0, u1, u2);
        const float2 wr = mul2(f2(w), rho);
        fsum = mul2(f2(2.0f), fma2(f2(w), drho, mul2(wr, fma2(f2(4.5f), mul2(eu, eu), neg2(k15)))));
        fdif = mul2(mul2(f2(6.0f), wr), eu);
        if (FORCED) {
            const float2 eF = edot(i, F0, F1, F2);
            FS = mul2(f2(sc.dh3 * w), sub2(mul2(f2(3.0f), mul2(eu, eF)), uF));
            FA = mul2(f2(sc.dh3 * w), eF);
        } else {
            FS = f2(0.f);
            FA = f2(0.f);
        }
    };
    if (MODEL == CM_SMAG || MODEL == CM_VREM || MODEL == CM_WALE) {
        // SRT with a per-cell rate (FluidDomain.f90:1239-1262). Smagorinsky
        // (smag :1265-1281): the stress sums Q_ab = sum e_a e_b fneq_i take the
        // pair sums s = neq_i + neq_o only (fneq = -neq); *tau_rel receives
        // tau_all. Vreman: *tau_rel holds tau_all from the gradient pass.
        // WALE: the same stress sums give S_ij with the previous tau_all
        // (les_in[0]) and les_in[1..3] hold O12, O13, O23; *tau_rel receives
        // tau_all.
        float2 omv, cfv;
        if (MODEL == CM_VREM) {
#pragma unroll
            for (int l = 0; l < 2; l++) {
                setl(omv, l, 1.0f / getl(*tau_rel, l));
                setl(cfv, l, 1.0f - 0.5f * getl(omv, l));
            }
        } else {
        float2 q11 = f2(0.f), q22 = f2(0.f), q33 = f2(0.f), q12 = f2(0.f), q13 = f2(0.f), q23 = f2(0.f);
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const int i = pr_(k), o = opp_(i);
            float2 fsum, fdif, FS, FA;
            pair_terms(i, fsum, fdif, FS, FA);
            const float2 sv = sub2(add2(g[i], g[o]), fsum);  // fneq_i + fneq_o
            if (ex_(i)) q11 = add2(q11, sv);
            if (ey_(i)) q22 = add2(q22, sv);
            if (ez_(i)) q33 = add2(q33, sv);
            if (ex_(i) && ey_(i)) q12 = ex_(i) * ey_(i) > 0 ? add2(q12, sv) : sub2(q12, sv);
            if (ex_(i) && ez_(i)) q13 = ex_(i) * ez_(i) > 0 ? add2(q13, sv) : sub2(q13, sv);
            if (ey_(i) && ez_(i)) q23 = ey_(i) * ez_(i) > 0 ? add2(q23, sv) : sub2(q23, sv);
        }
        const float2 qq = fma2(q11, q11, fma2(q22, q22, fma2(q33, q33, mul2(f2(2.0f), fma2(q12, q12, fma2(q13, q13,
                                                                                                   mul2(q23, q23)))))));
        if (MODEL == CM_WALE) {
#pragma unroll
            for (int l = 0; l < 2; l++) {
                const float k = -(1.5f * sc.dh) / (getl(rho, l) * getl(les_in[0], l));
                const float t = wale_tau<float>(sc, k * getl(q11, l), k * getl(q22, l), k * getl(q33, l),
                                                k * getl(q12, l), k * getl(q13, l), k * getl(q23, l),
                                                getl(les_in[1], l), getl(les_in[2], l), getl(les_in[3], l));
                setl(omv, l, 1.0f / t);
                setl(cfv, l, 1.0f - 0.5f * getl(omv, l));
                if (tau_rel) setl(*tau_rel, l, t);
            }
        } else {
#pragma unroll
        for (int l = 0; l < 2; l++) {
            const float tau_t = sqrtf(sc.tau * sc.tau + sc.cles * sqrtf(getl(qq, l)) / getl(rho, l));
            setl(omv, l, 2.0f / (sc.tau + tau_t));
            setl(cfv, l, 1.0f - 0.5f * getl(omv, l));
            if (tau_rel) setl(*tau_rel, l, 0.5f * (sc.tau + tau_t));
        }
        }
        }
        const float2 feq0 = mul2(f2(w0), sub2(drho, mul2(rho, k15)));
        float2 n0 = fma2(omv, sub2(feq0, g[0]), g[0]);
        if (FORCED) n0 = sub2(n0, mul2(mul2(cfv, f2(sc.dh3 * w0)), uF));
        emit(0, n0);
        const float2 hov = mul2(f2(-0.5f), omv);
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const int i = pr_(k), o = opp_(i);
            float2 fsum, fdif, FS, FA;
            pair_terms(i, fsum, fdif, FS, FA);
            // neq_i,o = (-s_k +- d)/2, d = fdif - (g_i - g_o)
            const float2 dv = sub2(fdif, sub2(g[i], g[o]));
            float2 A = mul2(hov, sub2(add2(g[i], g[o]), fsum));  // Om (neq_i + neq_o)/2
            float2 B = mul2(mul2(f2(-1.0f), hov), dv);  // Om (neq_i - neq_o)/2
            if (FORCED) {
                A = fma2(cfv, FS, A);
                B = fma2(cfv, FA, B);
            }
            emit(i, add2(g[i], add2(A, B)));
            emit(o, add2(g[o], sub2(A, B)));
        }
    } else if (MODEL == CM_SRT || MODEL == CM_TRT) {
        // SRT, and TRT (FluidDomain.f90:1228-1235) in the same form: per pair
        //   g'_i = al g_i + be g_o + S + A,  g'_o = al g_o + be g_i + S - A,
        //   S = Om/2 (feq_i + feq_o), A = Om2/2 (feq_i - feq_o),
        //   al = 1 - (Om + Om2)/2, be = (Om2 - Om)/2  (SRT: Om2 = Om),
        // forcing (1 - Om/2)(Flb_i + Flb_o)/2 +- (1 - Om2/2)(Flb_i - Flb_o)/2
        constexpr bool TRT = MODEL == CM_TRT;
        const float oa = TRT ? sc.om2 : om;
        const float2 omc = f2(TRT ? 1.0f - 0.5f * (om + oa) : 1.0f - om);
        const float bet = TRT ? 0.5f * (oa - om) : 0.0f;
        const float2 base = sub2(drho, mul2(rho, k15));
        const float2 orho = mul2(f2(om), rho);
        const float2 arho = TRT ? mul2(f2(oa), rho) : orho;
        const float2 ac0 = mul2(f2(om * w0), base);
        const float2 ac1 = mul2(f2(om * w1), base), bc1 = mul2(f2(4.5f * w1), orho), cc1 = mul2(f2(3.0f * w1), arho);
        const float2 ac2 = mul2(f2(om * w2), base), bc2 = mul2(f2(4.5f * w2), orho), cc2 = mul2(f2(3.0f * w2), arho);
        const float cf = (1.0f - 0.5f * om) * sc.dh3;
        const float cfa = TRT ? (1.0f - 0.5f * oa) * sc.dh3 : cf;
        float2 n0 = fma2(TRT ? f2(1.0f - om) : omc, g[0], ac0);
        if (FORCED) n0 = sub2(n0, mul2(f2(cf * w0), uF));
        emit(0, n0);
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const int i = pr_(k), o = opp_(i);
            const bool cls1 = (i <= 6);
            const float2 eu = edot(i, u0, u1, u2);
            const float2 Sm = fma2(cls1 ? bc1 : bc2, mul2(eu, eu), cls1 ? ac1 : ac2);
            const float2 Am = mul2(cls1 ? cc1 : cc2, eu);
            float2 ni = fma2(omc, g[i], add2(Sm, Am));
            float2 no = fma2(omc, g[o], sub2(Sm, Am));
            if (TRT) {
                ni = fma2(f2(bet), g[o], ni);
                no = fma2(f2(bet), g[i], no);
            }
            if (FORCED) {
                const float2 eF = edot(i, F0, F1, F2);
                const float wc = cls1 ? w1 : w2;
                const float2 Fs = mul2(f2(cf * wc), sub2(mul2(f2(3.0f), mul2(eF, eu)), uF));
                const float2 Fa = mul2(f2(cfa * wc), eF);
                ni = add2(ni, add2(Fs, Fa));
                no = add2(no, sub2(Fs, Fa));
            }
            emit(i, ni);
            emit(o, no);
        }
    } else {
        const float dh3 = sc.dh3;
        const float2 feq0 = mul2(f2(w0), sub2(drho, mul2(rho, k15)));
        const float2 hf0 = FORCED ? mul2(f2(0.5f * dh3 * w0), uF) : f2(0.f);  // -Flb_0/2
        // r = feq - g - Flb/2: rest r0, pair sums rs = r_i + r_o, differences rd = r_i - r_o
        const float2 r0 = FORCED ? sub2(add2(feq0, hf0), g[0]) : sub2(feq0, g[0]);
        float2 rs[9], rd[9];
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const int i = pr_(k), o = opp_(i);
            float2 fsum, fdif, FS, FA;
            pair_terms(i, fsum, fdif, FS, FA);
            float2 sm = sub2(fsum, add2(g[i], g[o]));
            float2 dm = sub2(fdif, sub2(g[i], g[o]));
            if (FORCED) {
                sm = sub2(sm, FS);
                dm = sub2(dm, FA);
            }
            rs[k] = sm;
            rd[k] = dm;
        }
        float2 t[Q], E0, E[9], O[9];
        mrt_forward(r0, rs, rd, ms, t);
        mrt_backward(t, E0, E, O);
        if (KEEPG) {
            // g'_i = g_i + Delta_i + Flb_i
            float2 n0 = add2(g[0], E0);
            if (FORCED) n0 = fma2(f2(-2.0f), hf0, n0);
            emit(0, n0);
#pragma unroll
            for (int k = 0; k < 9; k++) {
                const int i = pr_(k), o = opp_(i);
                float2 ev = E[k], dv = O[k];
                if (FORCED) {
                    float2 fsum, fdif, FS, FA;
                    pair_terms(i, fsum, fdif, FS, FA);
                    ev = add2(ev, FS);
                    dv = add2(dv, FA);
                }
                emit(i, add2(g[i], add2(ev, dv)));
                emit(o, add2(g[o], sub2(ev, dv)));
            }
        } else {
            // g'_i = g_i + Delta_i + Flb_i with g_i = feq_i - Flb_i/2 - r_i:
            //   rest:  g'_0 = feq_0 + Flb_0/2 - r_0 + Delta_0
            //   pairs: g'_i,o = A +- B, A = (fsum + FS - rs)/2 + E, B = (fdif + FA - rd)/2 + O
            float2 n0 = add2(sub2(feq0, r0), E0);
            if (FORCED) n0 = sub2(n0, hf0);
            emit(0, n0);
#pragma unroll
            for (int k = 0; k < 9; k++) {
                const int i = pr_(k), o = opp_(i);
                float2 fsum, fdif, FS, FA;
                pair_terms(i, fsum, fdif, FS, FA);
                float2 A = fma2(f2(0.5f), sub2(fsum, rs[k]), E[k]);
                float2 B = fma2(f2(0.5f), sub2(fdif, rd[k]), O[k]);
                if (FORCED) {
                    A = fma2(f2(0.5f), FS, A);
                    B = fma2(f2(0.5f), FA, B);
                }
                emit(i, add2(A, B));
                emit(o, sub2(A, B));
            }
        }
    }
}

// collide_emit with the results written back into g
template <int MODEL, bool FORCED>
__device__ __forceinline__ void collide2(float2 g[Q], float2 rho, float2 drho, float2 u0, float2 u1, float2 u2,
                                         float2 F0, float2 F1, float2 F2, const Scal<float> &sc, const MrtS &ms,
                                         float2 *tau_rel = nullptr, const float2 *les_in = nullptr) {
    float2 out[Q];
    collide_emit<MODEL, FORCED, true>(g, rho, drho, u0, u1, u2, F0, F1, F2, sc, ms,
                                      [&](int i, float2 v) { out[i] = v; }, tau_rel, les_in);
#pragma unroll
    for (int i = 0; i < Q; i++) g[i] = out[i];
}

// resident CTAs per SM the paired bulk kernel is compiled for (its register
// budget), measured best on GB300: SRT 4 x 256 threads (<= 64 registers);
// MRT unforced FP16/BF16 3 (<= 85, a little spill), MRT forced or FP32 2
// threads per CTA of the paired bulk kernel (whole z-rows: at least Z/2).
// Measured on GB300 (FP16, 256^3 TGV): 128-thread CTAs beat 256-thread ones
// (MRT 58.7k -> 63.1k MLUPS, SRT 74.7k -> 76.0k): the z-shift barrier stalls
// fewer warps at a time.
#ifndef FSI_PAIR_THREADS
#define FSI_PAIR_THREADS 128
#endif
#ifndef FSI_PAIR_MINB_SRT
#define FSI_PAIR_MINB_SRT 4
#endif
#ifndef FSI_PAIR_MINB_MRT
#define FSI_PAIR_MINB_MRT 3
#endif
#ifndef FSI_PAIR_MINB_MRT_FORCED
#define FSI_PAIR_MINB_MRT_FORCED 2
#endif
template <int P, int MODEL, bool FORCED>
constexpr int pair_minb() {
    return (MODEL == CM_SRT || MODEL == CM_TRT)
               ? FSI_PAIR_MINB_SRT
               : ((FORCED || P == FSI_PREC_F32) ? FSI_PAIR_MINB_MRT_FORCED : FSI_PAIR_MINB_MRT);
}
// the same budgets for CTAs of FSI_PAIR_THREADS (the single-block kernel);
// MRT unforced FP16/BF16 at 128 threads: 5 CTAs (up to 102 registers) beat 6
// (85, spilling) and 4 (128): 256^3 TGV FP16 63.9k / 62.8k / 57.9k MLUPS
#ifndef FSI_PAIR_CTAS_MRT
#define FSI_PAIR_CTAS_MRT (FSI_PAIR_THREADS == 128 ? 5 : FSI_PAIR_MINB_MRT * 256 / FSI_PAIR_THREADS)
#endif
template <int P, int MODEL, bool FORCED, int T>
constexpr int pair_ctas() {
    return T != FSI_PAIR_THREADS ? pair_minb<P, MODEL, FORCED>() * 256 / T
           : (MODEL != CM_SRT && MODEL != CM_TRT && !FORCED && P != FSI_PREC_F32)
               ? FSI_PAIR_CTAS_MRT
               : pair_minb<P, MODEL, FORCED>() * 256 / T;
}

// The bulk step: every cell takes den/u from its own distributions and the
// uniform volume force vf. Cells of the IB window, half-way faces and 102
// planes are then corrected by the small kernels below, which read the same
// (unchanged) source buffer.
// One row group of the bulk step: thread (tz, ty) of the group owns the cells
// (2 tz, 2 tz + 1) of z-row y = y0 + ty in x-plane x; R rows per group; sm
// holds [10][R][Z] elements. Every thread of the CTA calls it (the ones
// outside the group with in_group false): it contains a CTA barrier.
// U32: every access as a 32-bit byte offset from the buffer's base (the
// buffer spans less than 4 GiB). Measured on GB300, FP16 256^3 TGV: SRT 75.7k
// -> 81.5k, MRT 63.9k -> 66.9k MLUPS against a 64-bit pointer plus a
// per-population element offset, which costs a 64-bit add per access.
template <int P, int MODEL, bool FORCED, bool U32 = true>
__device__ __forceinline__ void pair_body(const StepArgs &a, const Offs<int> &of, const Scal<float> &sc,
                                          const MrtS &ms, int tz, int ty, int R, int y, int x, bool in_group,
                                          typename V2<P>::S *sm) {
    using V = V2<P>;
    using S2 = typename V::S2;
    using S = typename V::S;
    const int Z = a.Z, Y = a.Y, X = a.X;
    const int z0 = 2 * tz;
    const bool active = in_group && (y < Y);
    const int c = z0 + Z * ((active ? y : 0) + Y * x);
    const int N = (int)a.N;

    float2 g[Q];
    if (active) {
        if constexpr (U32) {
            const char *sb = (const char *)a.src;
#pragma unroll
            for (int i = 0; i < Q; i++)
                g[i] = V::dec(__ldcs((const S2 *)(sb + (unsigned)(c + of.ld[i]) * (unsigned)sizeof(S))));
        } else {
            const S *sp = (const S *)a.src + c;
#pragma unroll
            for (int i = 0; i < Q; i++) g[i] = V::dec(__ldcs((const S2 *)(sp + of.ld[i])));
        }
    } else {
#pragma unroll
        for (int i = 0; i < Q; i++) g[i] = f2(0.0f);
    }
    float2 drho, rho, jx, jy, jz, u0, u1, u2;
    macro2(g, drho, rho, jx, jy, jz);
    const float2 F0 = f2(sc.vf[0]), F1 = f2(sc.vf[1]), F2 = f2(sc.vf[2]);
    vel2<FORCED>(rho, jx, jy, jz, F0, F1, F2, 0.5f * sc.dh, u0, u1, u2);

    // push; the destination row is (y+ey, x+ex) with periodic wrap. The nine
    // populations with ez = 0 are stored as soon as they are collided; the
    // ten z-moving ones go through shared memory for the +-z shift.
    const int ZY = Z * Y;
    const int cyp = (y == Y - 1) ? -ZY : 0, cym = (y == 0) ? ZY : 0;
    const int cxp = (x == X - 1) ? -N : 0, cxm = (x == 0) ? N : 0;
    S *dp = (S *)a.dst + c;
    auto corr = [&](int i) {
        return (ey_(i) > 0 ? cyp : (ey_(i) < 0 ? cym : 0)) + (ex_(i) > 0 ? cxp : (ex_(i) < 0 ? cxm : 0));
    };
    char *db = (char *)a.dst;
    auto dst_at = [&](int i) {
        if constexpr (U32) return (S2 *)(db + (unsigned)(c + corr(i) + of.st[i]) * (unsigned)sizeof(S));
        else return (S2 *)(dp + corr(i) + of.st[i]);
    };
    // destination cells z0, z0+1 on a z face the kernel writes itself
    const bool zf0 = a.zeq[0] && z0 == 0, zf1 = a.zeq[1] && z0 + 1 == Z - 1;
    auto emit = [&](int i, float2 v) {
        if (!active) return;
        if (ez_(i) == 0) {
            if (zf0) v.x = geq_zface(a, 0, i);
            if (zf1) v.y = geq_zface(a, 1, i);
            __stcs(dst_at(i), V::enc(v));
        } else {
            *(S2 *)(sm + (zslot_(i) * R + ty) * Z + z0) = V::enc(v);
        }
    };
    if (MODEL == CM_SRT || MODEL == CM_TRT) {
        // SRT, TRT: stored pair by pair, so that the 64-register budget holds
        collide_emit<MODEL, FORCED, false>(g, rho, drho, u0, u1, u2, F0, F1, F2, sc, ms, emit);
    } else if (MODEL == CM_SMAG || MODEL == CM_VREM || MODEL == CM_WALE) {
        // tau_all(z0, z0+1) with the populations (c is even: an aligned pair);
        // Smagorinsky and WALE write it, Vreman reads what the gradient pass
        // wrote; WALE reads the previous one and its rotation entries
        float2 tr = f2(sc.tau);
        float2 li[4] = {f2(sc.tau), f2(0.f), f2(0.f), f2(0.f)};
        if (MODEL == CM_VREM && active) tr = *(const float2 *)(a.tauf + c);
        if (MODEL == CM_WALE && active) {
            const float *og = (const float *)a.og;
            li[0] = *(const float2 *)(a.tauf_prev + c);
            li[1] = *(const float2 *)(og + c);
            li[2] = *(const float2 *)(og + c + N);
            li[3] = *(const float2 *)(og + c + 2 * N);
        }
        collide_emit<MODEL, FORCED, true>(g, rho, drho, u0, u1, u2, F0, F1, F2, sc, ms, emit, &tr, li);
        if (MODEL != CM_VREM && active) *(float2 *)(a.tauf + c) = tr;
    } else {
        // MRT: all 19 collided first, then stored under one branch
        collide2<MODEL, FORCED>(g, rho, drho, u0, u1, u2, F0, F1, F2, sc, ms);
        if (active) {
#pragma unroll
            for (int i = 0; i < Q; i++) {
                float2 v = g[i];
                if (ez_(i) == 0) {
                    if (zf0) v.x = geq_zface(a, 0, i);
                    if (zf1) v.y = geq_zface(a, 1, i);
                    __stcs(dst_at(i), V::enc(v));
                } else {
                    *(S2 *)(sm + (zslot_(i) * R + ty) * Z + z0) = V::enc(v);
                }
            }
        }
    }
    __syncthreads();
    if (!active) return;
    const int zl = (z0 == 0) ? Z - 1 : z0 - 1, zr = (z0 + 2 == Z) ? 0 : z0 + 2;
#pragma unroll
    for (int i = 0; i < Q; i++) {
        if (ez_(i) == 0) continue;
        const S *row = sm + (zslot_(i) * R + ty) * Z;
        // ez = +1: cells z0, z0+1 receive z0-1, z0; ez = -1: they receive z0+1, z0+2
        S lo = ez_(i) > 0 ? row[zl] : row[z0 + 1], hi = ez_(i) > 0 ? row[z0] : row[zr];
        if (zf0) lo = V::enc1(geq_zface(a, 0, i));
        if (zf1) hi = V::enc1(geq_zface(a, 1, i));
        __stcs(dst_at(i), V::pack(lo, hi));
    }
}


// T: the CTA size it is compiled for (FSI_PAIR_THREADS, or 256 for rows
// longer than FSI_PAIR_THREADS pairs)
template <int P, int MODEL, bool FORCED, int T, bool U32>
__global__ void __launch_bounds__(T, pair_ctas<P, MODEL, FORCED, T>())
k_step_pair(StepArgs a, Offs<int> of, Scal<float> sc, MrtS ms) {
    extern __shared__ unsigned char smraw[];
    const int R = blockDim.y;
    pair_body<P, MODEL, FORCED, U32>(a, of, sc, ms, threadIdx.x, threadIdx.y, R, blockIdx.y * R + threadIdx.y,
                                     blockIdx.z, true, (typename V2<P>::S *)smraw);
}

// ---------------------------------------------------------------------------
// Pipelined persistent form of the bulk step (Z a multiple of 8): each CTA
// walks row groups (R consecutive z-rows of one x-plane) with a stride of the
// grid, and keeps the next groups' 19 population rows in flight as 1-D bulk
// copies global -> shared (cp.async.bulk, completion on an mbarrier per
// stage), so that loads stream while the CTA collides. All waits are bounded:
// a wait that runs out sets bit 1 of the error word, waits (bounded) for the
// copies still in flight into this CTA and returns.
// ---------------------------------------------------------------------------
constexpr int PIPE_NS = 3;                 // stages
constexpr long long PIPE_WAIT = 1LL << 22;  // try_wait rounds before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_tx(uint64_t *b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(b))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t *b, unsigned parity) {
    for (long long k = 0; k < PIPE_WAIT; k++)
        if (mbar_try_wait(b, parity)) return true;
    return false;
}

struct PipeGeom {
    int R, ngy, G;  // rows per group, groups per x-plane, groups
};

// queue the bulk copies of group j into stage buffer st (19 contiguous runs of
// rows*Z elements, one per population)
template <typename S>
__device__ __forceinline__ void pipe_issue(const StepArgs &a, const PipeGeom &pg, int j, S *st, uint64_t *bar) {
    const int x = j / pg.ngy, y0 = (j % pg.ngy) * pg.R;
    const int rows = min(pg.R, a.Y - y0);
    const unsigned bytes = (unsigned)(rows * a.Z * (int)sizeof(S));
    const S *src = (const S *)a.src + (long long)a.Z * ((long long)y0 + (long long)a.Y * x);
    mbar_arrive_tx(bar, bytes * Q);
#pragma unroll 1
    for (int i = 0; i < Q; i++) bulk_g2s(st + (long long)i * pg.R * a.Z, src + a.N * i, bytes, bar);
}

template <int P, int MODEL, bool FORCED>
__global__ void __launch_bounds__(256, 2) k_step_pipe(StepArgs a, Offs<int> of, Scal<float> sc, MrtS ms, PipeGeom pg) {
    using V = V2<P>;
    using S2 = typename V::S2;
    using S = typename V::S;
    extern __shared__ __align__(128) unsigned char smraw[];
    const int Z = a.Z, Y = a.Y, X = a.X;
    const int tz = threadIdx.x, ty = threadIdx.y, R = pg.R;
    const int tid = ty * blockDim.x + tz;
    const int z0 = 2 * tz;
    const int RZ = R * Z;
    S *stage = (S *)smraw;                       // [NS][19][R*Z]
    S *zsm = stage + (long long)PIPE_NS * Q * RZ;  // [10][R][Z]
    uint64_t *bar = (uint64_t *)(((uintptr_t)(zsm + 10 * RZ) + 7) & ~(uintptr_t)7);
    const int N = (int)a.N;
    const int stride = gridDim.x;

    if (tid == 0) {
        for (int s = 0; s < PIPE_NS; s++) mbar_init(bar + s, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < PIPE_NS; s++) {
            const int j = blockIdx.x + s * stride;
            if (j < pg.G) pipe_issue(a, pg, j, stage + (long long)s * Q * RZ, bar + s);
        }
    }

    int it = 0;
    for (int j = blockIdx.x; j < pg.G; j += stride, it++) {
        const int s = it % PIPE_NS;
        const unsigned par = (unsigned)((it / PIPE_NS) & 1);
        const bool ok = mbar_wait(bar + s, par);
        if (!__syncthreads_and(ok)) {
            // drain: every copy queued for this CTA lands before it returns
            if (tid == 0) {
                atomicOr(a.kerr, 1);
                for (int k = 0; k < PIPE_NS; k++) {
                    const int jk = j + k * stride;
                    if (jk < pg.G) mbar_wait(bar + (it + k) % PIPE_NS, (unsigned)(((it + k) / PIPE_NS) & 1));
                }
            }
            return;
        }
        const int x = j / pg.ngy, y0 = (j % pg.ngy) * R;
        const int y = y0 + ty;
        const bool active = (y < Y);
        const S *sb = stage + (long long)s * Q * RZ + ty * Z + z0;
        float2 g[Q];
#pragma unroll
        for (int i = 0; i < Q; i++) g[i] = active ? V::dec(*(const S2 *)(sb + i * RZ)) : f2(0.0f);
        __syncthreads();  // stage s is read; zsm of the previous group is free
        if (tid == 0) {
            const int jn = j + PIPE_NS * stride;
            if (jn < pg.G) {
                fence_proxy_async();
                pipe_issue(a, pg, jn, stage + (long long)s * Q * RZ, bar + s);
            }
        }

        float2 drho, rho, jx, jy, jz, u0, u1, u2;
        macro2(g, drho, rho, jx, jy, jz);
        const float2 F0 = f2(sc.vf[0]), F1 = f2(sc.vf[1]), F2 = f2(sc.vf[2]);
        vel2<FORCED>(rho, jx, jy, jz, F0, F1, F2, 0.5f * sc.dh, u0, u1, u2);
        collide2<MODEL, FORCED>(g, rho, drho, u0, u1, u2, F0, F1, F2, sc, ms);

        if (active) {
#pragma unroll
            for (int i = 0; i < Q; i++)
                if (ez_(i) != 0) *(S2 *)(zsm + (zslot_(i) * R + ty) * Z + z0) = V::enc(g[i]);
        }
        __syncthreads();
        if (active) {
            const int c = z0 + Z * (y + Y * x);
            const int ZY = Z * Y;
            const int cyp = (y == Y - 1) ? -ZY : 0, cym = (y == 0) ? ZY : 0;
            const int cxp = (x == X - 1) ? -N : 0, cxm = (x == 0) ? N : 0;
            S *dp = (S *)a.dst + c;
            const int zl = (z0 == 0) ? Z - 1 : z0 - 1, zr = (z0 + 2 == Z) ? 0 : z0 + 2;
#pragma unroll
            for (int i = 0; i < Q; i++) {
                const int corr =
                    (ey_(i) > 0 ? cyp : (ey_(i) < 0 ? cym : 0)) + (ex_(i) > 0 ? cxp : (ex_(i) < 0 ? cxm : 0));
                S lo, hi;
                if (ez_(i) == 0) {
                    lo = V::lo(V::enc(g[i]));
                    hi = V::hi(V::enc(g[i]));
                } else {
                    const S *row = zsm + (zslot_(i) * R + ty) * Z;
                    lo = ez_(i) > 0 ? row[zl] : row[z0 + 1];
                    hi = ez_(i) > 0 ? row[z0] : row[zr];
                }
                if (a.zeq[0] && z0 == 0) lo = V::enc1(geq_zface(a, 0, i));
                if (a.zeq[1] && z0 + 1 == Z - 1) hi = V::enc1(geq_zface(a, 1, i));
                __stcs((S2 *)(dp + corr + of.st[i]), V::pack(lo, hi));
            }
        }
    }
}

template <int P>
size_t pipe_smem(int R, int Z) {
    using S = typename V2<P>::S;
    return (size_t)(PIPE_NS * Q + 10) * R * Z * sizeof(S) + 16 + 8 * PIPE_NS;
}

// persistent grid of the pipelined kernel: co-resident CTAs on this device
template <int P, int MODEL, bool FORCED>
cudaError_t pipe_run(const StepArgs &a, const Offs<int> &of, const Scal<float> &sc, const MrtS &ms, int tpr, int R,
                     cudaStream_t st) {
    auto kern = k_step_pipe<P, MODEL, FORCED>;
    const size_t smem = pipe_smem<P>(R, a.Z);
    static int grid_cache[64][2] = {};  // per device: grid, smem it was sized for
    static std::mutex grid_mu;          // callers on several host threads
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    int resident = 0;
    {
        std::lock_guard<std::mutex> lock(grid_mu);
        if (grid_cache[dev][1] != (int)smem) {
            e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            int nb = 0, sms = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, tpr * R, smem);
            if (e != cudaSuccess) return e;
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            if (nb < 1) return cudaErrorInvalidConfiguration;
            grid_cache[dev][0] = nb * sms;
            grid_cache[dev][1] = (int)smem;
        }
        resident = grid_cache[dev][0];
    }
    PipeGeom pg;
    pg.R = R;
    pg.ngy = (a.Y + R - 1) / R;
    pg.G = pg.ngy * a.X;
    const int grid = std::min(resident, pg.G);
    kern<<<grid, dim3(tpr, R), smem, st>>>(a, of, sc, ms, pg);
    return cudaGetLastError();
}

// cell (x, y, z) of window cell wc
__device__ __forceinline__ void win_cell(const Win &w, long long wc, int &x, int &y, int &z) {
    z = (int)(wc % w.WZ) + w.z0;
    const long long t = wc / w.WZ;
    y = (int)(t % w.WY) + w.y0;
    x = (int)(t / w.WY) + w.x0;
}

// One cell of a two-cell lane group, for the fix-up kernels: the 19 source
// populations, and the destination of each push with periodic wrap.
template <int P>
__device__ __forceinline__ void load_cell(const StepArgs &a, int x, int y, int z, float2 g[Q], int l) {
    using V = V2<P>;
    const typename V::S *src = (const typename V::S *)a.src;
    const long long c = (long long)z + (long long)a.Z * ((long long)y + (long long)a.Y * x);
#pragma unroll
    for (int i = 0; i < Q; i++) setl(g[i], l, V::dec1(src[c + a.N * i]));
}

template <int P>
__device__ __forceinline__ void push_cell(const StepArgs &a, int x, int y, int z, const float2 g[Q], int l) {
    using V = V2<P>;
    typename V::S *dst = (typename V::S *)a.dst;
#pragma unroll
    for (int i = 0; i < Q; i++) {
        int xd = x + ex_(i), yd = y + ey_(i), zd = z + ez_(i);
        xd = xd < 0 ? a.X - 1 : (xd == a.X ? 0 : xd);
        yd = yd < 0 ? a.Y - 1 : (yd == a.Y ? 0 : yd);
        zd = zd < 0 ? a.Z - 1 : (zd == a.Z ? 0 : zd);
        const long long cd = (long long)zd + (long long)a.Z * ((long long)yd + (long long)a.Y * xd);
        float v = getl(g[i], l);
        if (a.zeq[0] && zd == 0) v = geq_zface(a, 0, i);
        if (a.zeq[1] && zd == a.Z - 1) v = geq_zface(a, 1, i);
        dst[cd + a.N * i] = V::enc1(v);
    }
}

// the per-cell-rate inputs of two arbitrary cells (the fix-up kernels):
// Vreman's tau_all into tr; WALE's previous tau_all and rotation entries
template <int MODEL>
__device__ __forceinline__ void les_cells(const StepArgs &a, const int x[2], const int y[2], const int z[2],
                                          float2 &tr, float2 li[4]) {
    if constexpr (MODEL == CM_VREM || MODEL == CM_WALE) {
#pragma unroll
        for (int l = 0; l < 2; l++) {
            const long long c = (long long)z[l] + (long long)a.Z * ((long long)y[l] + (long long)a.Y * x[l]);
            if (MODEL == CM_VREM) {
                setl(tr, l, a.tauf[c]);
            } else {
                const float *og = (const float *)a.og;
                setl(li[0], l, a.tauf_prev[c]);
                setl(li[1], l, og[c]);
                setl(li[2], l, og[c + a.N]);
                setl(li[3], l, og[c + 2 * a.N]);
            }
        }
    }
}

// The IB window: its cells collide with the den/u/force of the IB stage and
// push again, replacing what the bulk step pushed for them. Two window cells
// per thread (any two: the lanes are independent).
template <int P, int MODEL>
__device__ __forceinline__ void win_fix_body(const StepArgs &a, const Scal<float> &sc, const MrtS &ms, long long w0) {
    const Win &w = a.win;
    if (w0 >= w.n) return;
    const bool two = w0 + 1 < w.n;
    int x[2], y[2], z[2];
    float2 g[Q], drho, rho, u0, u1, u2, F0, F1, F2;
#pragma unroll
    for (int l = 0; l < 2; l++) {
        const long long wc = (l == 1 && !two) ? w0 : w0 + l;
        win_cell(w, wc, x[l], y[l], z[l]);
        load_cell<P>(a, x[l], y[l], z[l], g, l);
        const float d = (float)(__ldcg(w.den + wc) - 1.0);
        setl(drho, l, d);
        setl(rho, l, 1.0f + d);
        setl(u0, l, (float)__ldcg(w.u + wc));
        setl(u1, l, (float)__ldcg(w.u + wc + w.n));
        setl(u2, l, (float)__ldcg(w.u + wc + 2 * w.n));
        setl(F0, l, (float)__ldcg(w.force + wc));
        setl(F1, l, (float)__ldcg(w.force + wc + w.n));
        setl(F2, l, (float)__ldcg(w.force + wc + 2 * w.n));
    }
    float2 tr = f2(sc.tau);
    float2 li[4] = {f2(sc.tau), f2(0.f), f2(0.f), f2(0.f)};
    les_cells<MODEL>(a, x, y, z, tr, li);
    collide2<MODEL, true>(g, rho, drho, u0, u1, u2, F0, F1, F2, sc, ms, &tr, li);
    push_cell<P>(a, x[0], y[0], z[0], g, 0);
    if (two) push_cell<P>(a, x[1], y[1], z[1], g, 1);
    if (MODEL == CM_SMAG || MODEL == CM_WALE) {
#pragma unroll
        for (int l = 0; l < 2; l++) {
            if (l == 1 && !two) break;
            a.tauf[(long long)z[l] + (long long)a.Z * ((long long)y[l] + (long long)a.Y * x[l])] = getl(tr, l);
        }
    }
}

template <int P, int MODEL>
__global__ void __launch_bounds__(128) k_win_fix(StepArgs a, Scal<float> sc, MrtS ms) {
    win_fix_body<P, MODEL>(a, sc, ms, 2 * (blockIdx.x * (long long)blockDim.x + threadIdx.x));
}

// Face hooks of one face k: the post-collision FP64 copy of a half-way face
// (halfwayBCset_, FluidDomain.f90:567-614) or den/u on the layer-2 plane of a
// 102 face. Cells of the IB window use the window's den/u/force, as the
// bulk and window kernels do. Two face cells per thread.
template <int P, int MODEL>
__global__ void __launch_bounds__(128) k_face_hook(StepArgs a, Scal<float> sc, MrtS ms, int k, int A, int B) {
    const long long n = (long long)A * B;
    const long long f0 = 2 * (blockIdx.x * (long long)blockDim.x + threadIdx.x);
    if (f0 >= n) return;
    const bool two = f0 + 1 < n;
    const bool hw = a.hw[k] != nullptr;
    const int ax = k >> 1;
    // face cell (ia, ib): ia runs along z (x/y faces) or y (z faces)
    int x[2], y[2], z[2];
    float2 g[Q], drho, rho, jx, jy, jz, u0, u1, u2;
    float2 F0 = f2(sc.vf[0]), F1 = f2(sc.vf[1]), F2 = f2(sc.vf[2]);
#pragma unroll
    for (int l = 0; l < 2; l++) {
        const long long fc = (l == 1 && !two) ? f0 : f0 + l;
        const int ia = (int)(fc % A), ib = (int)(fc / A);
        // the plane: the face itself (half-way copy) or layer 2 (102)
        const int lay = hw ? ((k & 1) ? (ax == 0 ? a.X : ax == 1 ? a.Y : a.Z) - 1 : 0)
                           : ((k & 1) ? (ax == 0 ? a.X : ax == 1 ? a.Y : a.Z) - 2 : 1);
        if (ax == 0) { x[l] = lay; y[l] = ib; z[l] = ia; }
        else if (ax == 1) { y[l] = lay; x[l] = ib; z[l] = ia; }
        else { z[l] = lay; x[l] = ib; y[l] = ia; }
        load_cell<P>(a, x[l], y[l], z[l], g, l);
    }
    macro2(g, drho, rho, jx, jy, jz);
    vel2<true>(rho, jx, jy, jz, F0, F1, F2, 0.5f * sc.dh, u0, u1, u2);
    const Win &w = a.win;
#pragma unroll
    for (int l = 0; l < 2; l++) {
        if (x[l] >= w.x0 && x[l] <= w.x1 && y[l] >= w.y0 && y[l] <= w.y1 && z[l] >= w.z0 && z[l] <= w.z1) {
            const long long wc = (long long)(z[l] - w.z0) +
                                 (long long)w.WZ * ((long long)(y[l] - w.y0) + (long long)w.WY * (x[l] - w.x0));
            const float d = (float)(__ldcg(w.den + wc) - 1.0);
            setl(drho, l, d);
            setl(rho, l, 1.0f + d);
            setl(u0, l, (float)__ldcg(w.u + wc));
            setl(u1, l, (float)__ldcg(w.u + wc + w.n));
            setl(u2, l, (float)__ldcg(w.u + wc + 2 * w.n));
            setl(F0, l, (float)__ldcg(w.force + wc));
            setl(F1, l, (float)__ldcg(w.force + wc + w.n));
            setl(F2, l, (float)__ldcg(w.force + wc + 2 * w.n));
        }
    }
    if (!hw) {
#pragma unroll
        for (int l = 0; l < 2; l++) {
            if (l == 1 && !two) break;
            const long long c = (long long)z[l] + (long long)a.Z * ((long long)y[l] + (long long)a.Y * x[l]);
            a.den[c] = 1.0 + (double)getl(drho, l);
            a.u[c] = getl(u0, l);
            a.u[c + a.N] = getl(u1, l);
            a.u[c + 2 * a.N] = getl(u2, l);
        }
        return;
    }
    float2 tr = f2(sc.tau);
    float2 li[4] = {f2(sc.tau), f2(0.f), f2(0.f), f2(0.f)};
    les_cells<MODEL>(a, x, y, z, tr, li);
    collide2<MODEL, true>(g, rho, drho, u0, u1, u2, F0, F1, F2, sc, ms, MODEL == CM_VREM ? &tr : nullptr, li);
#pragma unroll
    for (int l = 0; l < 2; l++) {
        if (l == 1 && !two) break;
        const long long fc = f0 + l;
        double *h = a.hw[k] + (long long)Q * fc;
#pragma unroll
        for (int i = 0; i < Q; i++) h[i] = (double)getl(g[i], l) + wt_(i);
    }
}

template <int P, int MODEL>
cudaError_t pair_launch(const StepArgs &a, const MrtMats *mm, bool hooks, cudaStream_t st) {
    Offs<int> of{};
    const long long ZY = (long long)a.Z * a.Y;
    for (int i = 0; i < Q; i++) {
        of.ld[i] = (int)((long long)i * a.N);
        // no z term: the z shift happens in shared memory
        of.st[i] = (int)((long long)i * a.N + (long long)a.Z * ey_(i) + ZY * ex_(i));
    }
    Scal<float> sc{};
    sc.om = (float)a.omega;
    sc.dh = (float)a.dh;
    sc.dh3 = 3.0f * (float)a.dh;
    for (int k = 0; k < 3; k++) sc.vf[k] = (float)a.vf[k];
    sc.forced = (a.vf[0] != 0.0 || a.vf[1] != 0.0 || a.vf[2] != 0.0) ? 1 : 0;
    sc.om2 = (float)a.omega2;
    sc.tau = (float)a.tau;
    sc.nu = (float)a.nu;
    sc.cles = (float)a.cles;
    MrtS ms{};
    if (MODEL == 3)
        for (int k = 0; k < Q; k++) ms.sd[k] = (float)mm->sd[k];
    const int tpr = a.Z / 2;
    // rows of more than FSI_PAIR_THREADS pairs take the 256-thread build;
    // 32-bit byte offsets while the buffer spans less than 4 GiB
    const bool big = tpr > FSI_PAIR_THREADS;
    const bool u32 = (unsigned long long)Q * a.N * sizeof(typename V2<P>::S) < (1ULL << 32);
    const int R = std::max(1, (big ? 256 : FSI_PAIR_THREADS) / tpr);
    dim3 blk(tpr, R), grd(1, (a.Y + R - 1) / R, a.X);
    size_t smem = (size_t)10 * R * a.Z * sizeof(typename V2<P>::S);
    // the pipelined persistent form (on request, SRT and MRT; it needs
    // 16-byte aligned population rows) or the paired form
    const bool pipe = a.variant == 2 && a.Z % 8 == 0 && (MODEL == CM_SRT || MODEL == CM_MRT);
    if (pipe) {
        if constexpr (MODEL == CM_SRT || MODEL == CM_MRT) {
            cudaError_t e = sc.forced ? pipe_run<P, MODEL, true>(a, of, sc, ms, tpr, R, st)
                                      : pipe_run<P, MODEL, false>(a, of, sc, ms, tpr, R, st);
            if (e != cudaSuccess) return e;
        }
    } else if (sc.forced) {
        if (big) k_step_pair<P, MODEL, true, 256, false><<<grd, blk, smem, st>>>(a, of, sc, ms);
        else if (u32) k_step_pair<P, MODEL, true, FSI_PAIR_THREADS, true><<<grd, blk, smem, st>>>(a, of, sc, ms);
        else k_step_pair<P, MODEL, true, FSI_PAIR_THREADS, false><<<grd, blk, smem, st>>>(a, of, sc, ms);
    } else {
        if (big) k_step_pair<P, MODEL, false, 256, false><<<grd, blk, smem, st>>>(a, of, sc, ms);
        else if (u32) k_step_pair<P, MODEL, false, FSI_PAIR_THREADS, true><<<grd, blk, smem, st>>>(a, of, sc, ms);
        else k_step_pair<P, MODEL, false, FSI_PAIR_THREADS, false><<<grd, blk, smem, st>>>(a, of, sc, ms);
    }
    // what needs the IB stage's window waits for it
    if (a.join) {
        cudaError_t e = cudaStreamWaitEvent(st, (cudaEvent_t)a.join, 0);
        if (e != cudaSuccess) return e;
    }
    // the face hooks read the source buffer, which the bulk step leaves as is
    if (hooks) {
        for (int k = 0; k < 6; k++) {
            if (!a.hw[k] && !a.l2[k]) continue;
            const int ax = k >> 1;
            const int A = ax == 2 ? a.Y : a.Z, B = ax == 0 ? a.Y : a.X;
            const long long n = (long long)A * B;
            k_face_hook<P, MODEL><<<(unsigned)((n + 255) / 256), 128, 0, st>>>(a, sc, ms, k, A, B);
        }
    }
    if (a.win.x1 >= a.win.x0 && a.win.n > 0)
        k_win_fix<P, MODEL><<<(unsigned)((a.win.n + 255) / 256), 128, 0, st>>>(a, sc, ms);
    return cudaGetLastError();
}

template <int P>
__global__ void k_macro_fast(const void *__restrict__ fs, double *den, double *u, int Y, int Z, long long N, double dh,
                             double vf0, double vf1, double vf2) {
    using T = ST<P>;
    using C = typename T::C;
    int z = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, x = blockIdx.z;
    if (z >= Z) return;
    long long c = cidx(z, y, x, Z, Y);
    const typename T::S *src = (const typename T::S *)fs;
    C g[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) g[i] = T::dec(src[c + N * i]);
    const C vf[3] = {(C)vf0, (C)vf1, (C)vf2};
    C rho, drho, u0, u1, u2;
    macro_fast<P>(g, vf, (C)dh, rho, drho, u0, u1, u2);
    den[c] = T::OFF ? 1.0 + (double)drho : (double)rho;
    u[c] = u0; u[c + N] = u1; u[c + 2 * N] = u2;
}

// den/uuu of every cell as the collision sees them (IB window cells from the
// IB stage), before the step of a model that reads neighbour velocities
template <int P>
__global__ void k_step_macro_fast(StepArgs a, Scal<typename ST<P>::C> sc) {
    using T = ST<P>;
    using C = typename T::C;
    const int z = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, x = blockIdx.z;
    if (z >= a.Z) return;
    const long long c = cidx(z, y, x, a.Z, a.Y), N = a.N;
    const Win &w = a.win;
    if (x >= w.x0 && x <= w.x1 && y >= w.y0 && y <= w.y1 && z >= w.z0 && z <= w.z1) {
        long long wc = (long long)(z - w.z0) + (long long)w.WZ * ((long long)(y - w.y0) + (long long)w.WY * (x - w.x0));
        const double d = w.den[wc];
        // the values the step kernel converts them to
        C rho, drho;
        if (T::OFF) { drho = (C)(d - 1.0); rho = C(1) + drho; }
        else { rho = (C)d; drho = rho - C(1); }
        if (T::OFF) {
            a.uf[c] = (C)w.u[wc]; a.uf[c + N] = (C)w.u[wc + w.n]; a.uf[c + 2 * N] = (C)w.u[wc + 2 * w.n];
        } else {
            a.den[c] = (double)rho;
            a.u[c] = (C)w.u[wc]; a.u[c + N] = (C)w.u[wc + w.n]; a.u[c + 2 * N] = (C)w.u[wc + 2 * w.n];
        }
        (void)drho;
        return;
    }
    const typename T::S *src = (const typename T::S *)a.src;
    C g[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) g[i] = T::dec(src[c + N * i]);
    C rho, drho, u0, u1, u2;
    macro_fast<P>(g, sc.vf, sc.dh, rho, drho, u0, u1, u2);
    if (T::OFF) {
        a.uf[c] = u0; a.uf[c + N] = u1; a.uf[c + 2 * N] = u2;
    } else {
        a.den[c] = (double)rho;
        a.u[c] = u0; a.u[c + N] = u1; a.u[c + 2 * N] = u2;
    }
}

template <int P>
__global__ void k_win_macro_fast(const void *__restrict__ fs, double *wden, double *wu, IbGeom g, long long N,
                                 long long Nw, double vf0, double vf1, double vf2) {
    using T = ST<P>;
    using C = typename T::C;
    long long wc = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (wc >= Nw) return;
    int wz = (int)(wc % g.WZ);
    long long t = wc / g.WZ;
    int wy = (int)(t % g.WY), wx = (int)(t / g.WY);
    long long c = cidx(wz + g.wz0, wy + g.wy0, wx + g.wx0, g.Z, g.Y);
    const typename T::S *src = (const typename T::S *)fs;
    C gl[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) gl[i] = T::dec(src[c + N * i]);
    const C vf[3] = {(C)vf0, (C)vf1, (C)vf2};
    C rho, drho, u0, u1, u2;
    macro_fast<P>(gl, vf, (C)g.dh, rho, drho, u0, u1, u2);
    wden[wc] = T::OFF ? 1.0 + (double)drho : (double)rho;
    wu[wc] = u0; wu[wc + Nw] = u1; wu[wc + 2 * Nw] = u2;
}

// ---------------------------------------------------------------------------
// Immersed boundary for the fast forms: the whole of calculate_interaction_force
// (Solidbody.f90:869-918) in one persistent cooperative launch. Phases are
// separated by a grid barrier; a warp serves one marker (two stencil points per
// lane, shuffle reduction); the velocity correction and the spreading scatter
// with FP64 atomics, so sums are not in the reference's order (the exact form
// keeps that order). Data written inside the launch are read through L2
// (__ldcg): L1 is not coherent across SMs.
// ---------------------------------------------------------------------------

// grid barrier with an iteration limit. The arrival counter (status[2])
// only grows, from launch to launch: the k-th barrier of a launch waits for
// base + k * nblk arrivals (base: the counter at launch, which the host keeps
// from the previous launch's status), one release-add and acquire polls of a
// single word. On timeout the status gets bit 8 and the CTA returns false;
// the other CTAs then time out at their next barrier.
__device__ __forceinline__ bool gbar(int *status, unsigned nblk, unsigned &target) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned *cnt = (unsigned *)(status + 2);
        target += nblk;
        unsigned v;
        asm volatile("atom.add.release.gpu.u32 %0, [%1], 1;" : "=r"(v) : "l"(cnt) : "memory");
        v += 1u;
        int good = 1;
        for (long long it = 0; (int)(v - target) < 0; it++) {
            if (it > (1LL << 21)) {
                atomicOr(status, 8);
                good = 0;
                break;
            }
            asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(v) : "l"(cnt) : "memory");
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// The IB stage of one block, by nth threads (tid = 0..nth-1, tid = CTA *
// blockDim.x + thread) that meet at bar(): the whole grid of a cooperative
// launch (k_ib_coop, grid barrier) or one cluster (k_ib_cluster, k_ib_batch).
//
// The penalty loop runs one barrier per stage (a stage = one body in one
// iteration, Solidbody.f90:893-906): stage s interpolates the window velocity
// V_s = P_s + D_{s-1} and scatters its velocity corrections into D_s, where
// P_s (two ping-pong buffers) holds V_{s-1} and D (three rotating slots) the
// corrections of one stage each. The stage's owner pass writes P_{s+1} =
// P_s + D_{s-1} and clears D_{s-2}, the slot that D_{s+1} reuses. No stage
// writes what it reads, so the interpolation and the correction of a stage
// need no barrier between them.
//
// Arithmetic of the loop (R): FP32 for the offset forms, whose distributions
// carry FP32 arithmetic (GB300 runs FP64 at a small fraction of the FP32
// rate, and every FP64 warp instruction of a phase is on its critical path);
// FP64 for the FP64-storage forms. With R = FP32 the two P buffers live in
// wu2 and the correction slots, the spreading sums and the Lagrangian-force
// sums in dlt, w64 and fet (each sized for FP64); the window's den, u and
// force (read by the step's window fix-up) and the Lagrangian force stay FP64.
template <int P, class BAR>
__device__ __forceinline__ void ib_body(const IbCoop &a, long long tid, long long nth, BAR &&bar) {
    using T = ST<P>;
    using C = typename T::C;
    constexpr bool F32IB = std::is_same<C, float>::value;
    using R = typename std::conditional<F32IB, float, double>::type;
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // warps numbered across the CTAs first (warp w of CTA b is w * nblk + b),
    // so that the few warps that hold markers are spread over all the CTAs'
    // SMs; window cells (own) go to the CTAs' last threads first, which hold
    // no marker unless the markers fill the grid
    const long long bd = blockDim.x, nblk = nth / bd, t = tid % bd;
    const long long gw = (t >> 5) * nblk + tid / bd, nw = nth >> 5;
    const long long own = (bd - 1 - t) * nblk + tid / bd;
    const IbGeom &g = a.g;
    const long long Nw = a.Nw;
    R *const P0 = F32IB ? (R *)a.wu2 : (R *)a.wu;
    R *const P1 = F32IB ? (R *)a.wu2 + 3 * Nw : (R *)a.wu2;
    R *const D = (R *)a.dlt;
    float *const Sp = (float *)a.dlt + 9 * Nw;  // R = FP32: spreading sums (3 Nw)
    R *const W64 = (R *)a.w64;
    float *const efs = (float *)a.fet;          // R = FP32: Lagrangian-force sums (3 Mtot)
    // a group of IB_GL lanes serves one marker, IB_PTS of its 64 stencil
    // points each: point p = gl + IB_GL j has z offset gl & 3, y offset
    // ((gl >> 2) & 1) + 2 (j & 1) and x offset j >> 1
    constexpr int IB_GL = 8, IB_PTS = 64 / IB_GL, IB_MPW = 32 / IB_GL;
    const int sub = lane / IB_GL, gl = lane % IB_GL;

    // calculate_macro_quantities_ and the force reset + add_volume_force_ on
    // the window; the correction slots (and spreading sums) cleared
    const C vf[3] = {(C)a.vf[0], (C)a.vf[1], (C)a.vf[2]};
    for (long long wc = own; wc < Nw; wc += nth) {
        const int wz = (int)(wc % g.WZ);
        const long long r = wc / g.WZ;
        const int wy = (int)(r % g.WY), wx = (int)(r / g.WY);
        const long long c = cidx(wz + g.wz0, wy + g.wy0, wx + g.wx0, g.Z, g.Y);
        const typename T::S *src = (const typename T::S *)a.f;
        C fl[Q];
#pragma unroll
        for (int i = 0; i < Q; i++) fl[i] = T::dec(src[c + a.N * i]);
        C rho, drho, u0, u1, u2;
        macro_fast<P>(fl, vf, (C)g.dh, rho, drho, u0, u1, u2);
        a.wden[wc] = T::OFF ? 1.0 + (double)drho : (double)rho;
        P0[wc] = (R)u0; P0[wc + Nw] = (R)u1; P0[wc + 2 * Nw] = (R)u2;
        a.wforce[wc] = a.vf[0]; a.wforce[wc + Nw] = a.vf[1]; a.wforce[wc + 2 * Nw] = a.vf[2];
#pragma unroll
        for (int k = 0; k < 9; k++) D[wc + k * Nw] = (R)0;
        if (F32IB) {
#pragma unroll
            for (int k = 0; k < 3; k++) Sp[wc + k * Nw] = 0.0f;
        }
    }
    // UpdateElmtInterp_ and v_Eforce = 0 (Solidbody.f90:886-889): the group
    // forms the stencil and writes the window cell and the weight product
    // rx ry rz of each of its 64 points, which every phase below reads
    // instead of forming them again. The registers rwc/rwt (and the marker's
    // velocity ub and area ar) hold those of marker cm, the last marker this
    // lane group read.
    long long cm = -1;
    int rwc[IB_PTS];
    R rwt[IB_PTS];
    R ub[3] = {(R)0, (R)0, (R)0}, ar = (R)0;
    for (long long mb = gw * IB_MPW; mb < a.Mtot; mb += nw * IB_MPW) {
        const long long m = mb + sub;
        const bool act = m < a.Mtot;
        int b = 0;
        if (act)
            while (b + 1 < a.nb && m >= a.offs[b + 1]) b++;
        int e[12];
        float w[12];
        const long long mm = act ? m : 0;
        const int st = ib_stencil_group(a.xyz + 3LL * a.offs[b], a.xyz + 3 * mm, g, gl, act, e, w);
        if (st && gl == 0) atomicOr(a.status, st);
        if (act) {
#pragma unroll
            for (int k = 0; k < 12; k++)
                if (k % IB_GL == gl) { a.ei[12 * m + k] = (int16_t)e[k]; a.ew[12 * m + k] = w[k]; }
            const int zi = gl & 3, yi = (gl >> 2) & 1;
            const int ez = zi == 0 ? e[8] : (zi == 1 ? e[9] : (zi == 2 ? e[10] : e[11]));
            const float wz = zi == 0 ? w[8] : (zi == 1 ? w[9] : (zi == 2 ? w[10] : w[11]));
            const int ey0 = yi ? e[5] : e[4], ey1 = yi ? e[7] : e[6];
            const float wy0 = yi ? w[5] : w[4], wy1 = yi ? w[7] : w[6];
            const long long cz = (long long)(ez - 1 - g.wz0);
#pragma unroll
            for (int j = 0; j < IB_PTS; j++) {
                const int ey = (j & 1) ? ey1 : ey0;
                const float wy = (j & 1) ? wy1 : wy0;
                rwc[j] = (int)(cz + (long long)g.WZ * ((long long)(ey - 1 - g.wy0) +
                                                       (long long)g.WY * (long long)(e[j >> 1] - 1 - g.wx0)));
                rwt[j] = ((R)w[j >> 1] * (R)wy) * (R)wz;
                a.c64[64 * m + gl + IB_GL * j] = rwc[j];
                W64[64 * m + gl + IB_GL * j] = rwt[j];
            }
#pragma unroll
            for (int k = 0; k < 3; k++) ub[k] = (R)a.vel[3 * m + k];
            ar = (R)a.area[m];
            cm = m;
            if (gl < 3) {
                // a seeded start keeps the caller's initial force
                if (!a.seed) a.eforce[3 * m + gl] = 0.0;
                if (F32IB) efs[3 * m + gl] = a.seed ? (float)a.eforce[3 * m + gl] : 0.0f;
            }
        }
    }
    for (long long i = tid; i < a.ntol; i += nth) a.tol_acc[i] = 0.0;
    if (!bar()) return;
    if (*(volatile int *)a.status & 3) return;
    // the points, velocity and area of marker m in the registers
    auto points = [&](long long m) {
        if (m == cm) return;
#pragma unroll
        for (int j = 0; j < IB_PTS; j++) {
            rwc[j] = __ldcg(a.c64 + 64 * m + gl + IB_GL * j);
            rwt[j] = __ldcg(W64 + 64 * m + gl + IB_GL * j);
        }
#pragma unroll
        for (int k = 0; k < 3; k++) ub[k] = (R)a.vel[3 * m + k];
        ar = (R)a.area[m];
        cm = m;
    };

    // learned warm start (no counterpart in the reference): features of every
    // marker from the uncorrected window velocity; with a network, its
    // predicted force becomes the first correction (into D_{-1}, the slot the
    // first stage reads), applied to all bodies at once, and the penalty loop
    // below continues from it
    // seeded start (no counterpart in the reference): the caller's force
    // (3,Mtot) in eforce becomes the first correction, as the network's
    // prediction does below
    if (a.seed) {
        for (long long m = gw; m < a.Mtot; m += nw) {
            const R f0 = (R)(a.eforce[3 * m] * a.invh3p), f1 = (R)(a.eforce[3 * m + 1] * a.invh3p),
                    f2 = (R)(a.eforce[3 * m + 2] * a.invh3p);
            R *Dm = D + 6 * Nw;
            for (int p = lane; p < 64; p += 32) {
                const long long wc = __ldcg(a.c64 + 64 * m + p);
                const R wt = __ldcg(W64 + 64 * m + p);
                atomicAdd(Dm + wc, -(f0 * wt));
                atomicAdd(Dm + wc + Nw, -(f1 * wt));
                atomicAdd(Dm + wc + 2 * Nw, -(f2 * wt));
            }
        }
        if (!bar()) return;
    }
    if (a.mlp || a.feat) {
        const float iU = (float)(1.0 / a.Uref);
        for (long long m = gw; m < a.Mtot; m += nw) {
            double v0 = 0.0, v1 = 0.0, v2 = 0.0;
            for (int p = lane; p < 64; p += 32) {
                const long long wc = __ldcg(a.c64 + 64 * m + p);
                const double wt = (double)__ldcg(W64 + 64 * m + p);
                v0 += (double)__ldcg(P0 + wc) * wt;
                v1 += (double)__ldcg(P0 + wc + Nw) * wt;
                v2 += (double)__ldcg(P0 + wc + 2 * Nw) * wt;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                v0 += __shfl_xor_sync(FULL, v0, o);
                v1 += __shfl_xor_sync(FULL, v1, o);
                v2 += __shfl_xor_sync(FULL, v2, o);
            }
            float x[MLP_IN];
            x[0] = (float)(a.vel[3 * m] - v0) * iU;
            x[1] = (float)(a.vel[3 * m + 1] - v1) * iU;
            x[2] = (float)(a.vel[3 * m + 2] - v2) * iU;
#pragma unroll
            for (int k = 0; k < 3; k++) x[3 + k] = (float)a.vel[3 * m + k] * iU;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                x[6 + k] = a.aux ? (float)a.aux[6 * m + k] * iU : 0.0f;
                x[9 + k] = a.aux ? (float)a.aux[6 * m + 3 + k] : 0.0f;
            }
            if (a.feat) {
#pragma unroll
                for (int k = 0; k < MLP_IN; k++)
                    if (lane == k) a.feat[MLP_IN * m + k] = x[k];
            }
            if (a.mlp) {
                float y[MLP_OUT];
                mlp_forward_warp(a.mlp, a.mlp_nrm, x, lane, y);
                const double sc = a.area[m] * a.Uref;
                double F[3];
#pragma unroll
                for (int k = 0; k < 3; k++) F[k] = (double)__shfl_sync(FULL, y[k], 0) * sc;
                if (lane == 0) {
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        a.eforce[3 * m + k] = F[k];
                        if (F32IB) efs[3 * m + k] = (float)F[k];
                    }
                }
                const R f0 = (R)(F[0] * a.invh3p), f1 = (R)(F[1] * a.invh3p), f2 = (R)(F[2] * a.invh3p);
                R *Dm = D + 6 * Nw;
                for (int p = lane; p < 64; p += 32) {
                    const long long wc = __ldcg(a.c64 + 64 * m + p);
                    const R wt = __ldcg(W64 + 64 * m + p);
                    atomicAdd(Dm + wc, -(f0 * wt));
                    atomicAdd(Dm + wc + Nw, -(f1 * wt));
                    atomicAdd(Dm + wc + 2 * Nw, -(f2 * wt));
                }
            }
        }
        if (a.mlp && !bar()) return;
    }

    // the PenaltyForce_ loop, Solidbody.f90:893-906 (bodies one after another,
    // one stage each); in the last iteration the cap allows, each stage also
    // spreads its markers' final force (FluidVolumeForce_, Solidbody.f90:968-977)
    const R ih3p = (R)a.invh3p, ih3s = (R)a.invh3s;
    const float stopf = (float)(a.dtol * a.dsumU);  // R = FP32: the residual test tol > dtol M U
    int it = 0;
    long long s = 0;
    double dmax = 1e10;
    R tol = (R)0;
    bool stop = !(dmax > a.dtol), nan = false;
    // the residual test of iteration it - 1 (tol_acc complete after the
    // barrier); false: the loop stops
    auto test = [&](R tl) {
        tol = tl;
        if (!isfinite(tol)) {
            nan = true;
            return false;
        }
        if (F32IB) {
            stop = !((float)tol > stopf);
        } else {
            dmax = (double)tol / a.dsumU;
            stop = !(dmax > a.dtol);
        }
        return !stop;
    };
    while (it < a.ntol && !stop) {
        const bool last = it == a.ntol - 1;
        for (int b = 0; b < a.nb; b++, s++) {
            const R *Pk = (s & 1) ? P1 : P0;
            R *Pn = (s & 1) ? P0 : P1;
            const R *Dr = D + 3 * Nw * ((s + 2) % 3);
            R *Dw = D + 3 * Nw * (s % 3);
            R *Dz = D + 3 * Nw * ((s + 1) % 3);
            const int m0 = a.offs[b], m1 = a.offs[b + 1];
            // the first stage of an iteration reads the previous iteration's
            // residual beside its own loads (its first window cell and
            // marker) and writes nothing before the test
            bool decided = !(b == 0 && it > 0);
            R tprev = (R)0;
            if (!decided) tprev = F32IB ? (R)__ldcg((const float *)a.tol_acc + it - 1) : (R)__ldcg(a.tol_acc + it - 1);
            R ow[3] = {(R)0, (R)0, (R)0};
            if (own < Nw) {
#pragma unroll
                for (int k = 0; k < 3; k++) ow[k] = __ldcg(Pk + own + k * Nw) + __ldcg(Dr + own + k * Nw);
            }
            bool go = true;
            for (long long mb = m0 + gw * IB_MPW; mb < m1; mb += nw * IB_MPW) {
                const long long m = mb + sub;
                const bool act = m < m1;
                R v0 = (R)0, v1 = (R)0, v2 = (R)0, ef[3] = {(R)0, (R)0, (R)0};
                if (act) {
                    points(m);
#pragma unroll
                    for (int k = 0; k < 3; k++) ef[k] = F32IB ? (R)__ldcg(efs + 3 * m + k) : (R)__ldcg(a.eforce + 3 * m + k);
#pragma unroll
                    for (int j = 0; j < IB_PTS; j++) {
                        const long long c = rwc[j];
                        const R wt = rwt[j];
                        v0 += (__ldcg(Pk + c) + __ldcg(Dr + c)) * wt;
                        v1 += (__ldcg(Pk + c + Nw) + __ldcg(Dr + c + Nw)) * wt;
                        v2 += (__ldcg(Pk + c + 2 * Nw) + __ldcg(Dr + c + 2 * Nw)) * wt;
                    }
                }
#pragma unroll
                for (int o = IB_GL / 2; o > 0; o >>= 1) {
                    v0 += __shfl_xor_sync(FULL, v0, o);
                    v1 += __shfl_xor_sync(FULL, v1, o);
                    v2 += __shfl_xor_sync(FULL, v2, o);
                }
                if (!decided) {
                    decided = true;
                    if (!test(tprev)) {
                        go = false;
                        break;
                    }
                }
                R tsum = (R)0;
                if (act) {
                    const R d0 = ub[0] - v0, d1 = ub[1] - v1, d2 = ub[2] - v2;
                    const R F0 = d0 * ar, F1 = d1 * ar, F2 = d2 * ar;
                    const R e0 = ef[0] + F0, e1 = ef[1] + F1, e2 = ef[2] + F2;
                    tsum = (fabs(d0) + fabs(d1)) + fabs(d2);
                    if (gl == 0) {
                        if (F32IB) {
                            efs[3 * m] = (float)e0; efs[3 * m + 1] = (float)e1; efs[3 * m + 2] = (float)e2;
                        } else {
                            a.eforce[3 * m] = (double)e0; a.eforce[3 * m + 1] = (double)e1;
                            a.eforce[3 * m + 2] = (double)e2;
                        }
                    }
                    // the velocity correction of the support (Solidbody.f90:1034-1048)
                    const R f0 = F0 * ih3p, f1 = F1 * ih3p, f2 = F2 * ih3p;
#pragma unroll
                    for (int j = 0; j < IB_PTS; j++) {
                        const long long c = rwc[j];
                        const R wt = rwt[j];
                        atomicAdd(Dw + c, -(f0 * wt));
                        atomicAdd(Dw + c + Nw, -(f1 * wt));
                        atomicAdd(Dw + c + 2 * Nw, -(f2 * wt));
                    }
                    if (last) {
                        const R s0 = e0 * ih3s, s1 = e1 * ih3s, s2 = e2 * ih3s;
                        if (F32IB) {
                            if (gl < 3) a.eforce[3 * m + gl] = (double)(gl == 0 ? e0 : (gl == 1 ? e1 : e2));
#pragma unroll
                            for (int j = 0; j < IB_PTS; j++) {
                                const long long c = rwc[j];
                                const float wt = (float)rwt[j];
                                atomicAdd(Sp + c, -((float)s0 * wt));
                                atomicAdd(Sp + c + Nw, -((float)s1 * wt));
                                atomicAdd(Sp + c + 2 * Nw, -((float)s2 * wt));
                            }
                        } else {
#pragma unroll
                            for (int j = 0; j < IB_PTS; j++) {
                                const long long c = rwc[j];
                                const double wt = (double)rwt[j];
                                atomicAdd(a.wforce + c, -((double)s0 * wt));
                                atomicAdd(a.wforce + c + Nw, -((double)s1 * wt));
                                atomicAdd(a.wforce + c + 2 * Nw, -((double)s2 * wt));
                            }
                        }
                    }
                }
                // the residual sum: one term per marker (its group's first
                // lane), one atomic per warp
                if (gl != 0) tsum = (R)0;
#pragma unroll
                for (int o = IB_GL; o < 32; o <<= 1) tsum += __shfl_xor_sync(FULL, tsum, o);
                if (lane == 0) {
                    if (F32IB) atomicAdd((float *)a.tol_acc + it, (float)tsum);
                    else atomicAdd(a.tol_acc + it, (double)tsum);
                }
            }
            if (go && !decided) go = test(tprev);
            if (nan) {
                if (tid == 0) atomicOr(a.status, 4);
                return;
            }
            if (!go) break;
            // owner pass: P_{s+1} = P_s + D_{s-1}, D_{s-2} cleared
            for (long long wc = own; wc < Nw; wc += nth) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    Pn[wc + k * Nw] = wc == own ? ow[k] : __ldcg(Pk + wc + k * Nw) + __ldcg(Dr + wc + k * Nw);
                    Dz[wc + k * Nw] = (R)0;
                }
            }
            if (!bar()) return;
        }
        if (stop) break;
        it = it + 1;
    }
    // the residual of the last iteration the cap allowed (a stop by the test
    // has read it already)
    if (!stop && it > 0) {
        if (!test(F32IB ? (R)__ldcg((const float *)a.tol_acc + it - 1) : (R)__ldcg(a.tol_acc + it - 1))) {
            if (nan) {
                if (tid == 0) atomicOr(a.status, 4);
                return;
            }
        }
    }
    const bool spread_done = a.ntol > 0 && it == a.ntol;
    // the window velocity after the loop, V_s = P_s + D_{s-1}, into wu (the
    // window fix-up of the fluid step reads it); with R = FP32 also the
    // spreading sums onto the window force
    {
        const R *Pk = (s & 1) ? P1 : P0;
        const R *Dr = D + 3 * Nw * ((s + 2) % 3);
        for (long long wc = own; wc < Nw; wc += nth) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                a.wu[wc + k * Nw] = (double)(__ldcg(Pk + wc + k * Nw) + __ldcg(Dr + wc + k * Nw));
                if (F32IB && spread_done) a.wforce[wc + k * Nw] += (double)__ldcg(Sp + wc + k * Nw);
            }
        }
    }
    // FluidVolumeForce_ spreading (Solidbody.f90:968-977) onto vf, where the
    // loop stopped before its last iteration
    if (!spread_done) {
        for (long long m = gw * IB_MPW + sub; m < a.Mtot; m += nw * IB_MPW) {
            points(m);
            double ef[3];
#pragma unroll
            for (int k = 0; k < 3; k++) ef[k] = F32IB ? (double)__ldcg(efs + 3 * m + k) : __ldcg(a.eforce + 3 * m + k);
            if (F32IB && gl < 3) a.eforce[3 * m + gl] = gl == 0 ? ef[0] : (gl == 1 ? ef[1] : ef[2]);
            const double f0 = ef[0] * a.invh3s, f1 = ef[1] * a.invh3s, f2 = ef[2] * a.invh3s;
#pragma unroll
            for (int j = 0; j < IB_PTS; j++) {
                const long long c = rwc[j];
                const double wt = (double)rwt[j];
                atomicAdd(a.wforce + c, -(f0 * wt));
                atomicAdd(a.wforce + c + Nw, -(f1 * wt));
                atomicAdd(a.wforce + c + 2 * Nw, -(f2 * wt));
            }
        }
    }
    if (tid == 0) {
        a.status[1] = it;
        *a.res = F32IB ? (it > 0 ? (double)tol / a.dsumU : dmax) : dmax;
    }
}

template <int P>
__global__ void __launch_bounds__(256) k_ib_coop(IbCoop a) {
    const unsigned nblk = gridDim.x;
    unsigned target = a.bar_base;
    ib_body<P>(a, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x,
               [&]() { return gbar(a.status, nblk, target); });
}

// the IB stage of many blocks, one thread-block cluster of IB_CLUSTER CTAs
// per block; the cluster barrier (release/acquire at cluster scope, with a
// device fence for the global-memory atomics) separates the phases
constexpr int IB_CLUSTER = 8;

__device__ __forceinline__ void cluster_barrier() {
    __threadfence();
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// the IB stage of one block on one cluster (so that it can run beside the
// bulk step: a cluster needs no grid-wide co-residency)
template <int P>
__global__ void __cluster_dims__(IB_CLUSTER, 1, 1) __launch_bounds__(512) k_ib_cluster(IbCoop a) {
    if (a.Mtot <= 0) return;
    ib_body<P>(a, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)IB_CLUSTER * blockDim.x, []() {
        cluster_barrier();
        return true;
    });
}

template <int P>
__global__ void __cluster_dims__(IB_CLUSTER, 1, 1) __launch_bounds__(512) k_ib_batch(const IbCoop *__restrict__ cases,
                                                                                      int n) {
    const int c = blockIdx.x / IB_CLUSTER, rank = blockIdx.x % IB_CLUSTER;
    if (c >= n) return;  // whole clusters only: the grid is n * IB_CLUSTER
    const IbCoop &a = cases[c];
    if (a.Mtot <= 0) return;
    ib_body<P>(a, (long long)rank * blockDim.x + threadIdx.x, (long long)IB_CLUSTER * blockDim.x, []() {
        cluster_barrier();
        return true;
    });
}

template <int P>
__global__ void k_to_store(const double *__restrict__ f, void *fs, long long N) {
    using T = ST<P>;
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= N * Q) return;
    int q = (int)(i / N);
    double v = f[i];
    ((typename T::S *)fs)[i] = T::enc((typename T::C)(T::OFF ? v - wt_(q) : v));
}

template <int P>
__global__ void k_from_store(const void *__restrict__ fs, double *f, long long N) {
    using T = ST<P>;
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= N * Q) return;
    int q = (int)(i / N);
    double v = (double)T::dec(((const typename T::S *)fs)[i]);
    f[i] = T::OFF ? v + wt_(q) : v;
}

template <int P, int MODEL, bool HOOKS, typename IT>
cudaError_t step_launch(const StepArgs &a, const MatsT<typename ST<P>::C> &m, cudaStream_t st) {
    Offs<IT> of{};
    const long long ZY = (long long)a.Z * a.Y;
    for (int i = 0; i < Q; i++) {
        of.ld[i] = (IT)((long long)i * a.N);
        of.st[i] = (IT)((long long)i * a.N + ez_(i) + (long long)a.Z * ey_(i) + ZY * ex_(i));
    }
    int bz = a.Z >= 128 ? 128 : ((a.Z + 31) / 32) * 32;
    int by = TPB / bz;
    if (by < 1) by = 1;
    dim3 blk(bz, by), grd((a.Z + bz - 1) / bz, (a.Y + by - 1) / by, a.X);
    using C = typename ST<P>::C;
    Scal<C> sc{};
    sc.om = (C)a.omega;
    sc.dh = (C)a.dh;
    // (host code: the double-word type's arithmetic is device-only, so its
    // scalars are formed in FP64 and converted once)
    if constexpr (P == FSI_PREC_F64_DW) sc.dh3 = (C)(3.0 * a.dh);
    else sc.dh3 = (C)3 * (C)a.dh;
    for (int k = 0; k < 3; k++) sc.vf[k] = (C)a.vf[k];
    sc.forced = (a.vf[0] != 0.0 || a.vf[1] != 0.0 || a.vf[2] != 0.0) ? 1 : 0;
    sc.om2 = (C)a.omega2;
    sc.tau = (C)a.tau;
    sc.nu = (C)a.nu;
    sc.cles = (C)a.cles;
    k_step_fast<P, MODEL, HOOKS, IT><<<grd, blk, 0, st>>>(a, m, of, sc);
    return cudaGetLastError();
}

template <int P, int MODEL>
cudaError_t step_inst(const StepArgs &a, const MrtMats *mm, cudaStream_t st) {
    using C = typename ST<P>::C;
    // the one-cell kernels' matrices in the arithmetic type, formed only for
    // them (the paired kernels take the rates alone, every step)
    auto mats = [&]() {
        MatsT<C> m{};
        if (MODEL == 3) {
            for (int i = 0; i < 361; i++) { m.mc[i] = (C)mm->mc[i]; m.mf[i] = (C)mm->mf[i]; }
            for (int k = 0; k < Q; k++) m.sd[k] = (C)mm->sd[k];
        }
        return m;
    };
    // the hook-free variant serves blocks without IB window, half-way faces
    // and non-equilibrium extrapolation faces
    bool hooks = a.win.x1 >= a.win.x0;
    for (int k = 0; k < 6; k++) hooks = hooks || a.hw[k] != nullptr || a.l2[k] != 0;
    // 32-bit byte offsets while all 19 populations span less than 4 GiB
    const bool small = (unsigned long long)Q * a.N * sizeof(typename ST<P>::S) < (1ULL << 32);
    if constexpr (P == FSI_PREC_F64_DW) {
        // double-word arithmetic: SRT, and MRT in moment space only; two
        // cells per thread when the block needs no hooks and z is even
#if FSI_FAST_PREC == FSI_PREC_F64_DW
        if constexpr (MODEL == CM_SRT || MODEL == CM_MRT) {
            if (!hooks && a.Z % 2 == 0 && (MODEL == CM_SRT || mm->diag)) {
                constexpr int MM = MODEL == CM_MRT ? CM_MRT_MOM : MODEL;
                return small ? dw2_launch<MM, int>(a, mm, st) : dw2_launch<MM, long long>(a, mm, st);
            }
        }
#endif
        if constexpr (MODEL == CM_SRT) {
            if (small) return hooks ? step_launch<P, MODEL, true, int>(a, mats(), st) : step_launch<P, MODEL, false, int>(a, mats(), st);
            return hooks ? step_launch<P, MODEL, true, long long>(a, mats(), st)
                         : step_launch<P, MODEL, false, long long>(a, mats(), st);
        } else if constexpr (MODEL == CM_MRT) {
            if (!mm->diag) return cudaErrorInvalidValue;
            if (small)
                return hooks ? step_launch<P, CM_MRT_MOM, true, int>(a, mats(), st)
                             : step_launch<P, CM_MRT_MOM, false, int>(a, mats(), st);
            return hooks ? step_launch<P, CM_MRT_MOM, true, long long>(a, mats(), st)
                         : step_launch<P, CM_MRT_MOM, false, long long>(a, mats(), st);
        } else {
            return cudaErrorInvalidValue;
        }
    } else {
    if (step_fast_paired(a, mm, P, MODEL))
        return pair_launch<P == FSI_PREC_F64_FAST ? FSI_PREC_F32 : P, MODEL>(a, mm, hooks, st);
    if (MODEL == CM_MRT && mm->diag) {
        // moment space: about 80 operations for the transform each way
        // instead of two dense 19x19 products
        constexpr int MM = MODEL == CM_MRT ? CM_MRT_MOM : MODEL;
        if (small) return hooks ? step_launch<P, MM, true, int>(a, mats(), st) : step_launch<P, MM, false, int>(a, mats(), st);
        return hooks ? step_launch<P, MM, true, long long>(a, mats(), st) : step_launch<P, MM, false, long long>(a, mats(), st);
    }
    if (small) return hooks ? step_launch<P, MODEL, true, int>(a, mats(), st) : step_launch<P, MODEL, false, int>(a, mats(), st);
    return hooks ? step_launch<P, MODEL, true, long long>(a, mats(), st) : step_launch<P, MODEL, false, long long>(a, mats(), st);
    }
}

// Face kernels of the offset storage forms (FP32, FP16, BF16): the codes of
// bc_apply with FP32 arithmetic on the offsets g = f - w_i, one launch per
// face in the reference order (edge and corner cells keep the value of the
// last face that writes them). Face velocities are evaluated in FP64 (a few
// operations per cell) and the rest in FP32.
template <int P, int FACE>
__device__ __forceinline__ void bc_off_body(const BcArgs &a, int fa, int fb) {
    using T = ST<P>;
    using S = typename T::S;
    const int A = (FACE < 4) ? a.Z : a.Y;
    const int B = (FACE < 2) ? a.Y : a.X;
    if (fa >= A || fb >= B) return;
    if (FACE < 4 && (fa < a.zlo || fa > a.zhi)) return;
    S *f = (S *)a.f;
    const long long N = a.N;
    const long long c1 = face_cell(a, fa, fb, 0);
    auto ld = [&](long long c, int q) { return (float)T::dec(f[c + N * q]); };
    auto stq = [&](long long c, int q, float g) { f[c + N * q] = T::enc(g); };
    auto geq = [](int q, float rho, float u0, float u1, float u2, float k15) {
        return geq_off(q, rho, u0, u1, u2, k15);
    };
    switch (a.code) {
    case BC_EQ: {
        if (a.uni) {
            // a uniform face: its populations from the host (no per-cell
            // FP64 velocity, which GB300 issues at a small fraction of FP32)
#pragma unroll
            for (int i = 0; i < Q; i++) stq(c1, i, a.gq[i]);
            break;
        }
        double v[3];
        face_vel(a, fa, fb, false, v);
        const float u0 = (float)v[0], u1 = (float)v[1], u2 = (float)v[2];
        const float k15 = 1.5f * (u0 * u0 + u1 * u1 + u2 * u2), rho = (float)a.denIn;
#pragma unroll
        for (int i = 0; i < Q; i++) stq(c1, i, geq(i, rho, u0, u1, u2, k15));
    } break;
    case BC_NEQ: {
        const long long c2 = face_cell(a, fa, fb, 1);
        double v[3];
        face_vel(a, fa, fb, false, v);
        const float u0 = (float)v[0], u1 = (float)v[1], u2 = (float)v[2];
        const float k15 = 1.5f * (u0 * u0 + u1 * u1 + u2 * u2), rho = (float)a.denIn;
        const float w0 = (float)a.u[c2], w1 = (float)a.u[c2 + N], w2 = (float)a.u[c2 + 2 * N];
        const float d2 = (float)a.den[c2];
        const float k15b = 1.5f * (w0 * w0 + w1 * w1 + w2 * w2);
#pragma unroll
        for (int j = 0; j < 5; j++) {
            const int q = inc_(FACE, j);
            stq(c1, q, geq(q, rho, u0, u1, u2, k15) + (ld(c2, q) - geq(q, d2, w0, w1, w2, k15b)));
        }
    } break;
    case BC_EXT1: {
        const long long c2 = face_cell(a, fa, fb, 1);
#pragma unroll
        for (int j = 0; j < 5; j++) { const int q = inc_(FACE, j); f[c1 + N * q] = f[c2 + N * q]; }
    } break;
    case BC_EXT2: {
        const long long c2 = face_cell(a, fa, fb, 1), c3 = face_cell(a, fa, fb, 2);
        // 2 f2 - f3 = w + (2 g2 - g3): the offsets extrapolate the same way
#pragma unroll
        for (int j = 0; j < 5; j++) {
            const int q = inc_(FACE, j);
            stq(c1, q, 2.0f * ld(c2, q) - ld(c3, q));
        }
    } break;
    case BC_WALL: {
        S t[5];
#pragma unroll
        for (int j = 0; j < 5; j++) t[j] = f[c1 + N * opp_(inc_(FACE, j))];
#pragma unroll
        for (int j = 0; j < 5; j++) f[c1 + N * inc_(FACE, j)] = t[j];
    } break;
    case BC_WALL_HW: {
        const double *h = a.hw + (long long)Q * ((long long)fa + (long long)(FACE < 4 ? a.Z : a.Y) * fb);
#pragma unroll
        for (int j = 0; j < 5; j++) {
            const int q = inc_(FACE, j);
            stq(c1, q, (float)(h[opp_(q)] - wt_(q)));
        }
    } break;
    case BC_MWALL:
    case BC_MWALL_HW: {
        const bool half = (a.code == BC_MWALL_HW);
        double v[3];
        face_vel(a, fa, fb, half, v);
        const double *h = a.hw + (long long)Q * ((long long)fa + (long long)(FACE < 4 ? a.Z : a.Y) * fb);
        float t[5];
#pragma unroll
        for (int j = 0; j < 5; j++) {
            const int q = inc_(FACE, j);
            const float eu = (float)(ex_(q) * v[0] + ey_(q) * v[1] + ez_(q) * v[2]);
            // f_q = f_opp + 6 w denIn (e.u); the weights of q and opp(q) agree
            const float gin = half ? (float)(h[opp_(q)] - wt_(q)) : ld(c1, opp_(q));
            t[j] = gin + (6.0f * (float)wt_(q) * (float)a.denIn) * eu;
        }
#pragma unroll
        for (int j = 0; j < 5; j++) stq(c1, inc_(FACE, j), t[j]);
    } break;
    case BC_SYMMETRIC: {
        S t[5];
#pragma unroll
        for (int j = 0; j < 5; j++) t[j] = f[c1 + N * mir_(FACE, j)];
#pragma unroll
        for (int j = 0; j < 5; j++) f[c1 + N * inc_(FACE, j)] = t[j];
    } break;
    default:
        break;
    }
}

template <int P, int FACE>
__global__ void __launch_bounds__(256) k_bc_off(BcArgs a) {
    bc_off_body<P, FACE>(a, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}

// the two faces of one axis in one launch (blockIdx.z: 0 the low face, 1 the
// high one); the host pairs them only when the axis is long enough that
// neither face reads a cell the other writes
template <int P, int AX>
__global__ void __launch_bounds__(256) k_bc_off_pair(BcArgs lo, BcArgs hi) {
    const int fa = blockIdx.x * blockDim.x + threadIdx.x, fb = blockIdx.y * blockDim.y + threadIdx.y;
    if (blockIdx.z == 0) bc_off_body<P, 2 * AX>(lo, fa, fb);
    else bc_off_body<P, 2 * AX + 1>(hi, fa, fb);
}

// face FACE of many blocks, blockIdx.z = block (code BC_FLUID: nothing to do)
template <int P, int FACE>
__global__ void __launch_bounds__(256) k_bc_off_batch(const BcArgs *__restrict__ bcs, int n) {
    if ((int)blockIdx.z >= n) return;
    const BcArgs &a = bcs[blockIdx.z];
    if (a.code == BC_FLUID) return;
    bc_off_body<P, FACE>(a, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}

// ---------------------------------------------------------------------------
// Many blocks in one launch: CTA j takes global row group j, finds its block
// in the case table (sorted by first group), copies the block's step
// arguments into shared memory with the offsets and collision constants the
// single-block launcher passes as kernel parameters, and runs pair_body.
// The per-block values are the same as the single-block path's, so a batch
// step equals stepping each block alone.
// ---------------------------------------------------------------------------
struct BatchCta {
    StepArgs a;
    Offs<int> of;
    Scal<float> sc;
    MrtS ms;
    int R, tpr, x, yb;
};

__device__ __forceinline__ void batch_prologue(const BatchCase *__restrict__ cases, const int *__restrict__ gcase,
                                               int j, BatchCta &cta) {
    const BatchCase &C = cases[gcase[j]];
    // the step arguments, word by word
    const int nw = (int)(sizeof(StepArgs) / 4);
    for (int k = threadIdx.x; k < nw; k += blockDim.x) ((int *)&cta.a)[k] = ((const int *)&C.a)[k];
    const int t = threadIdx.x;
    if (t < Q) {
        const long long ZY = (long long)C.a.Z * C.a.Y;
        cta.of.ld[t] = (int)((long long)t * C.a.N);
        cta.of.st[t] = (int)((long long)t * C.a.N + (long long)C.a.Z * ey_(t) + ZY * ex_(t));
        cta.ms.sd[t] = C.sd[t];
    }
    if (t == 0) {
        cta.sc.om = (float)C.a.omega;
        cta.sc.dh = (float)C.a.dh;
        cta.sc.dh3 = 3.0f * (float)C.a.dh;
        for (int k = 0; k < 3; k++) cta.sc.vf[k] = (float)C.a.vf[k];
        cta.sc.forced = (C.a.vf[0] != 0.0 || C.a.vf[1] != 0.0 || C.a.vf[2] != 0.0) ? 1 : 0;
        cta.sc.om2 = (float)C.a.omega2;
        cta.sc.tau = (float)C.a.tau;
        cta.sc.nu = (float)C.a.nu;
        cta.sc.cles = (float)C.a.cles;
        cta.R = C.R;
        cta.tpr = C.tpr;
        const int jj = j - C.g0;
        cta.x = jj / C.ngy;
        cta.yb = jj % C.ngy;
    }
    __syncthreads();
}

template <int P, int MODEL, bool FORCED, int T>
__global__ void __launch_bounds__(T, T == 512 ? 1 : pair_ctas<P, MODEL, FORCED, T>())
k_step_batch(const BatchCase *__restrict__ cases, const int *__restrict__ gcase) {
    using S = typename V2<P>::S;
    __shared__ BatchCta cta;
    __shared__ S rows[10 * 2 * T];  // [10][R][Z], R*Z <= 2T
    batch_prologue(cases, gcase, blockIdx.x, cta);
    const int t = threadIdx.x;
    const int tz = t % cta.tpr, ty = t / cta.tpr;
    pair_body<P, MODEL, FORCED, true>(cta.a, cta.of, cta.sc, cta.ms, tz, ty, cta.R, cta.yb * cta.R + ty, cta.x,
                                      ty < cta.R, rows);
}

// the IB-window fix-up of every block: blockIdx.y = block
template <int P, int MODEL>
__global__ void __launch_bounds__(128) k_win_fix_batch(const BatchCase *__restrict__ cases, int n) {
    if ((int)blockIdx.y >= n) return;
    const BatchCase &C = cases[blockIdx.y];
    if (C.a.win.x1 < C.a.win.x0 || C.a.win.n <= 0) return;
    Scal<float> sc{};
    sc.om = (float)C.a.omega;
    sc.dh = (float)C.a.dh;
    sc.dh3 = 3.0f * (float)C.a.dh;
    sc.om2 = (float)C.a.omega2;
    sc.tau = (float)C.a.tau;
    sc.nu = (float)C.a.nu;
    sc.cles = (float)C.a.cles;
    MrtS ms;
#pragma unroll
    for (int k = 0; k < Q; k++) ms.sd[k] = C.sd[k];
    win_fix_body<P, MODEL>(C.a, sc, ms, 2 * (blockIdx.x * (long long)blockDim.x + threadIdx.x));
}

template <int P, int MODEL, bool FORCED>
cudaError_t batch_step_inst(const BatchCase *d, const int *gcase, int n, int G, int threads, long long wmax,
                            cudaStream_t st) {
    switch (threads) {
    case 128: k_step_batch<P, MODEL, FORCED, 128><<<G, 128, 0, st>>>(d, gcase); break;
    case 512: k_step_batch<P, MODEL, FORCED, 512><<<G, 512, 0, st>>>(d, gcase); break;
    default: k_step_batch<P, MODEL, FORCED, 256><<<G, 256, 0, st>>>(d, gcase); break;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || wmax <= 0) return e;
    k_win_fix_batch<P, MODEL><<<dim3((unsigned)((wmax + 255) / 256), n), 128, 0, st>>>(d, n);
    return cudaGetLastError();
}

template <int P, int MODEL>
cudaError_t batch_winfix_inst(const BatchCase *d, int n, long long wmax, cudaStream_t st) {
    if (wmax <= 0) return cudaSuccess;
    k_win_fix_batch<P, MODEL><<<dim3((unsigned)((wmax + 255) / 256), n), 128, 0, st>>>(d, n);
    return cudaGetLastError();
}

template <int P>
cudaError_t bc_inst(const BcArgs &a, cudaStream_t st) {
    const int A = (a.face < 4) ? a.Z : a.Y;
    const int B = (a.face < 2) ? a.Y : a.X;
    dim3 blk(64, 4), grd((A + 63) / 64, (B + 3) / 4);
    if (P == FSI_PREC_F64_FAST) {
        switch (a.face) {
        case 0: k_bc<AccS<P>, 0><<<grd, blk, 0, st>>>(a); break;
        case 1: k_bc<AccS<P>, 1><<<grd, blk, 0, st>>>(a); break;
        case 2: k_bc<AccS<P>, 2><<<grd, blk, 0, st>>>(a); break;
        case 3: k_bc<AccS<P>, 3><<<grd, blk, 0, st>>>(a); break;
        case 4: k_bc<AccS<P>, 4><<<grd, blk, 0, st>>>(a); break;
        default: k_bc<AccS<P>, 5><<<grd, blk, 0, st>>>(a); break;
        }
        return cudaGetLastError();
    }
    constexpr int PO = P == FSI_PREC_F64_FAST ? FSI_PREC_F32 : P;
    switch (a.face) {
    case 0: k_bc_off<PO, 0><<<grd, blk, 0, st>>>(a); break;
    case 1: k_bc_off<PO, 1><<<grd, blk, 0, st>>>(a); break;
    case 2: k_bc_off<PO, 2><<<grd, blk, 0, st>>>(a); break;
    case 3: k_bc_off<PO, 3><<<grd, blk, 0, st>>>(a); break;
    case 4: k_bc_off<PO, 4><<<grd, blk, 0, st>>>(a); break;
    default: k_bc_off<PO, 5><<<grd, blk, 0, st>>>(a); break;
    }
    return cudaGetLastError();
}

}  // namespace

namespace FSI_FAST_NS {

// the body with PP = this unit's storage form; any other form is refused
#define FSI_DISPATCH(prec, ...)                                 \
    if ((prec) != FSI_FAST_PREC) return cudaErrorInvalidValue; \
    { constexpr int PP = FSI_FAST_PREC; __VA_ARGS__; }

bool step_fast_paired(const StepArgs &a, const MrtMats *mm, int prec, int model) {
    const bool small = (long long)Q * a.N < (1LL << 31) - 1;
    return prec != FSI_PREC_F64_FAST && prec != FSI_PREC_F64_DW &&
           (model == CM_SRT || model == CM_TRT || model == CM_SMAG || model == CM_VREM || model == CM_WALE ||
            (model == CM_MRT && mm->diag)) && small &&
           a.Z % 2 == 0 && a.Z <= 512;
}

cudaError_t launch_step_fast(const StepArgs &a, const MrtMats *mm, int prec, int model, cudaStream_t st) {
    switch (model) {
    case CM_MRT: { FSI_DISPATCH(prec, return (step_inst<PP, CM_MRT>(a, mm, st))) }
    case CM_TRT: { FSI_DISPATCH(prec, return (step_inst<PP, CM_TRT>(a, mm, st))) }
    case CM_SMAG: { FSI_DISPATCH(prec, return (step_inst<PP, CM_SMAG>(a, mm, st))) }
    case CM_WALE: { FSI_DISPATCH(prec, return (step_inst<PP, CM_WALE>(a, mm, st))) }
    case CM_VREM: { FSI_DISPATCH(prec, return (step_inst<PP, CM_VREM>(a, mm, st))) }
    default: { FSI_DISPATCH(prec, return (step_inst<PP, CM_SRT>(a, mm, st))) }
    }
}

#if FSI_FAST_PREC != FSI_PREC_F64_DW
// (the double-word unit defines the bulk step only)
cudaError_t launch_step_macro_fast(const StepArgs &a, int prec, cudaStream_t st) {
    int bz = a.Z >= 256 ? 256 : ((a.Z + 31) / 32) * 32;
    dim3 g((a.Z + bz - 1) / bz, a.Y, a.X);
    FSI_DISPATCH(prec, {
        using CC = typename ST<PP>::C;
        Scal<CC> sc{};
        sc.dh = (CC)a.dh;
        for (int k = 0; k < 3; k++) sc.vf[k] = (CC)a.vf[k];
        sc.nu = (CC)a.nu;
        sc.cles = (CC)a.cles;
        k_step_macro_fast<PP><<<g, bz, 0, st>>>(a, sc);
        if (a.og) k_les_grad<PP, CM_WALE><<<g, bz, 0, st>>>(a, sc);
        else k_les_grad<PP, CM_VREM><<<g, bz, 0, st>>>(a, sc);
        return cudaGetLastError();
    })
}

cudaError_t launch_bc_fast(const BcArgs &a, int prec, cudaStream_t st) {
    FSI_DISPATCH(prec, return bc_inst<PP>(a, st))
}


// the same for the kernels of the offset forms alone
#if FSI_FAST_PREC == FSI_PREC_F64_FAST
#define FSI_DISPATCH_OFF(prec, ...) return cudaErrorInvalidValue;
#else
#define FSI_DISPATCH_OFF(prec, ...) FSI_DISPATCH(prec, __VA_ARGS__)
#endif

cudaError_t launch_bc_pair_fast(const BcArgs &lo, const BcArgs &hi, int prec, cudaStream_t st) {
    const int ax = lo.face >> 1;
    const int A = (ax < 2) ? lo.Z : lo.Y;
    const int B = (ax == 0) ? lo.Y : lo.X;
    dim3 blk(64, 4), grd((A + 63) / 64, (B + 3) / 4, 2);
    switch (prec) {
    case FSI_PREC_F32: case FSI_PREC_F16: case FSI_PREC_BF16: break;
    default: return cudaErrorInvalidValue;
    }
    FSI_DISPATCH_OFF(prec, {
        if (ax == 0) k_bc_off_pair<PP, 0><<<grd, blk, 0, st>>>(lo, hi);
        else if (ax == 1) k_bc_off_pair<PP, 1><<<grd, blk, 0, st>>>(lo, hi);
        else k_bc_off_pair<PP, 2><<<grd, blk, 0, st>>>(lo, hi);
        return cudaGetLastError();
    })
}

cudaError_t launch_batch_step(const BatchCase *d_cases, const int *d_gcase, int n, int G, int threads, long long wmax,
                              int prec, int model, bool forced, cudaStream_t st) {
    if (n <= 0 || G <= 0) return cudaSuccess;
#define FSI_BATCH_MODEL(M)                                                                                      \
    if (model == M) {                                                                                           \
        if (forced) { FSI_DISPATCH_OFF(prec, return (batch_step_inst<PP, M, true>(d_cases, d_gcase, n, G, threads, wmax, st))) } \
        FSI_DISPATCH_OFF(prec, return (batch_step_inst<PP, M, false>(d_cases, d_gcase, n, G, threads, wmax, st)))   \
    }
    FSI_BATCH_MODEL(CM_MRT)
    FSI_BATCH_MODEL(CM_TRT)
    FSI_BATCH_MODEL(CM_SMAG)
    FSI_BATCH_MODEL(CM_SRT)
#undef FSI_BATCH_MODEL
    return cudaErrorInvalidValue;
}

cudaError_t launch_batch_winfix(const BatchCase *d_cases, int n, long long wmax, int prec, int model, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    switch (model) {
    case CM_MRT: { FSI_DISPATCH_OFF(prec, return (batch_winfix_inst<PP, CM_MRT>(d_cases, n, wmax, st))) }
    case CM_TRT: { FSI_DISPATCH_OFF(prec, return (batch_winfix_inst<PP, CM_TRT>(d_cases, n, wmax, st))) }
    case CM_SMAG: { FSI_DISPATCH_OFF(prec, return (batch_winfix_inst<PP, CM_SMAG>(d_cases, n, wmax, st))) }
    default: { FSI_DISPATCH_OFF(prec, return (batch_winfix_inst<PP, CM_SRT>(d_cases, n, wmax, st))) }
    }
}

cudaError_t launch_batch_bc(const BcArgs *d_bcs, int n, int face, int Amax, int Bmax, int prec, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    dim3 blk(64, 4), grd((Amax + 63) / 64, (Bmax + 3) / 4, n);
    FSI_DISPATCH_OFF(prec, switch (face) {
        case 0: k_bc_off_batch<PP, 0><<<grd, blk, 0, st>>>(d_bcs, n); break;
        case 1: k_bc_off_batch<PP, 1><<<grd, blk, 0, st>>>(d_bcs, n); break;
        case 2: k_bc_off_batch<PP, 2><<<grd, blk, 0, st>>>(d_bcs, n); break;
        case 3: k_bc_off_batch<PP, 3><<<grd, blk, 0, st>>>(d_bcs, n); break;
        case 4: k_bc_off_batch<PP, 4><<<grd, blk, 0, st>>>(d_bcs, n); break;
        default: k_bc_off_batch<PP, 5><<<grd, blk, 0, st>>>(d_bcs, n); break;
    } return cudaGetLastError())
}

cudaError_t launch_ib_cluster(const IbCoop &a, int prec, cudaStream_t st) {
    FSI_DISPATCH_OFF(prec, k_ib_cluster<PP><<<IB_CLUSTER, 512, 0, st>>>(a); return cudaGetLastError())
}

cudaError_t launch_batch_ib(const IbCoop *d_ib, int n, int threads, int prec, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    FSI_DISPATCH_OFF(prec, k_ib_batch<PP><<<n * IB_CLUSTER, threads, 0, st>>>(d_ib, n); return cudaGetLastError())
}

cudaError_t launch_convert_to_store(const double *f64, void *fs, long long N, int prec, cudaStream_t st) {
    long long n = N * Q;
    unsigned nb = (unsigned)((n + 255) / 256);
    FSI_DISPATCH(prec, k_to_store<PP><<<nb, 256, 0, st>>>(f64, fs, N); return cudaGetLastError())
}

cudaError_t launch_convert_from_store(const void *fs, double *f64, long long N, int prec, cudaStream_t st) {
    long long n = N * Q;
    unsigned nb = (unsigned)((n + 255) / 256);
    FSI_DISPATCH(prec, k_from_store<PP><<<nb, 256, 0, st>>>(fs, f64, N); return cudaGetLastError())
}

cudaError_t launch_macro_fast(const void *fs, int prec, double *den, double *u, int X, int Y, int Z, double dh,
                              const double vf[3], cudaStream_t st) {
    int bz = Z >= 256 ? 256 : ((Z + 31) / 32) * 32;
    dim3 g((Z + bz - 1) / bz, Y, X);
    long long N = (long long)X * Y * Z;
    FSI_DISPATCH(prec, k_macro_fast<PP><<<g, bz, 0, st>>>(fs, den, u, Y, Z, N, dh, vf[0], vf[1], vf[2]);
                 return cudaGetLastError())
}

cudaError_t launch_ib_coop(const IbCoop &a, int prec, int grid, cudaStream_t st) {
    void *args[] = {(void *)&a};
    FSI_DISPATCH(prec, return cudaLaunchCooperativeKernel((void *)k_ib_coop<PP>, grid, 256, args, 0, st))
}

int ib_coop_grid(int prec) {
    int dev = 0, sms = 0, nb = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (prec != FSI_FAST_PREC) return 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_ib_coop<FSI_FAST_PREC>, 256, 0);
    return e == cudaSuccess ? nb * sms : 0;
}

cudaError_t launch_win_macro_fast(const void *fs, int prec, double *wden, double *wu, const IbGeom &g, long long N,
                                  const double vf[3], cudaStream_t st) {
    long long Nw = (long long)(g.wx1 - g.wx0 + 1) * g.WY * g.WZ;
    if (Nw <= 0) return cudaSuccess;
    unsigned nb = (unsigned)((Nw + 255) / 256);
    FSI_DISPATCH(prec, k_win_macro_fast<PP><<<nb, 256, 0, st>>>(fs, wden, wu, g, N, Nw, vf[0], vf[1], vf[2]);
                 return cudaGetLastError())
}

#endif  // FSI_FAST_PREC != FSI_PREC_F64_DW

}  // namespace FSI_FAST_NS
}  // namespace fsi
