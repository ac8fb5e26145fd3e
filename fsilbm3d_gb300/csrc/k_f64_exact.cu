// k_f64_exact.cu -- FP64 kernels in the reference's floating-point operation
// order. This translation unit is compiled with -fmad=false: no multiply-add
// is fused, every expression is evaluated left to right as gfortran does on a
// target without FMA, and sums run sequentially in index order. Results are
// therefore bitwise equal to an FP64 CPU run of the same order.
//
// Kernels: equilibrium initialisation, macroscopic fields, the fused
// collide+stream step (SRT and MRT), face boundary conditions, the half-way
// face copy, the immersed-boundary stencil / penalty / spreading, and the
// block-refinement face exchange.
#include "fsi_kernels.h"
#include "bc_impl.cuh"
#include "ib_impl.cuh"
#include "store_acc.cuh"

#include <math.h>

namespace fsi {

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ long long cidx(int z, int y, int x, int Z, int Y) {
    return (long long)z + (long long)Z * ((long long)y + (long long)Y * (long long)x);
}

// calculate_macro_quantities_ for one cell, FluidDomain.f90:1136-1139
__device__ __forceinline__ void macro_cell(const double f[Q], const double vf[3], double dh,
                                           double &den, double &u0, double &u1, double &u2) {
    double s = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
#pragma unroll
    for (int i = 0; i < Q; i++) s += f[i];
#pragma unroll
    for (int i = 0; i < Q; i++) sx += f[i] * (double)ex_(i);
#pragma unroll
    for (int i = 0; i < Q; i++) sy += f[i] * (double)ey_(i);
#pragma unroll
    for (int i = 0; i < Q; i++) sz += f[i] * (double)ez_(i);
    den = s;
    u0 = (sx + (0.5 * vf[0]) * dh) / den;
    u1 = (sy + (0.5 * vf[1]) * dh) / den;
    u2 = (sz + (0.5 * vf[2]) * dh) / den;
}

// ------------------------------------------------- per-cell relaxation (LES)

// the non-equilibrium stress sums of smag and WALE (FluidDomain.f90:1271-1276)
// from fneq = -fEq
__device__ __forceinline__ void neq_stress(const double fEq[Q], double q[6]) {
    double fn[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) fn[i] = -fEq[i];
    q[0] = fn[1] + fn[2] + fn[7] + fn[8] + fn[9] + fn[10] + fn[11] + fn[12] + fn[13] + fn[14];
    q[1] = fn[3] + fn[4] + fn[7] + fn[8] + fn[9] + fn[10] + fn[15] + fn[16] + fn[17] + fn[18];
    q[2] = fn[5] + fn[6] + fn[11] + fn[12] + fn[13] + fn[14] + fn[15] + fn[16] + fn[17] + fn[18];
    q[3] = fn[7] - fn[8] - fn[9] + fn[10];
    q[4] = fn[11] - fn[12] - fn[13] + fn[14];
    q[5] = fn[15] - fn[16] - fn[17] + fn[18];
}

// center_diff / onesid_diff with the interior / first / last cell branches of
// WALE and vrem (FluidDomain.f90:1343-1388, 1425-1491): the derivative of
// velocity component k along axis d (0 x, 1 y, 2 z), times the reference's
// invdh = dh
__device__ __forceinline__ double les_diff(const StepArgs &a, int k, int d, int z, int y, int x, long long c) {
    const double *__restrict__ u = a.u + a.N * k;
    const int i = d == 0 ? x : (d == 1 ? y : z);
    const int D = d == 0 ? a.X : (d == 1 ? a.Y : a.Z);
    const long long s = d == 0 ? (long long)a.Z * a.Y : (d == 1 ? (long long)a.Z : 1LL);
    if (i > 0 && i < D - 1) return (u[c + s] - u[c - s]) * a.dh;
    if (i == 0) return ((-(3.0 * u[c]) + 4.0 * u[c + s]) - u[c + 2 * s]) * a.dh;
    return ((-(3.0 * u[c]) + 4.0 * u[c - s]) - u[c - 2 * s]) * a.dh;
}

// smag, FluidDomain.f90:1265-1281
__device__ __forceinline__ double les_smag(const StepArgs &a, const double fEq[Q], double rho, long long c) {
    double q[6];
    neq_stress(fEq, q);
    const double QQ = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + 2.0 * (q[3] * q[3] + q[4] * q[4] + q[5] * q[5]);
    const double tau_t = sqrt(a.tau * a.tau + a.cles * sqrt(QQ) / rho);
    a.tau_all[c] = 0.5 * (a.tau + tau_t);
    return 2.0 / (a.tau + tau_t);
}

// WALE, FluidDomain.f90:1304-1416 (the reference's 0.0d0 terms only change
// the sign of a zero sum, which reaches no output)
__device__ double les_wale(const StepArgs &a, const double fEq[Q], double rho, int z, int y, int x, long long c) {
    double q[6];
    neq_stress(fEq, q);
    const double invdh = a.dh, tau_ = a.tau_all[c];
    const double S11 = -(1.5 * invdh * q[0] / (rho * tau_));
    const double S22 = -(1.5 * invdh * q[1] / (rho * tau_));
    const double S33 = -(1.5 * invdh * q[2] / (rho * tau_));
    const double S12 = -(1.5 * invdh * q[3] / (rho * tau_));
    const double S13 = -(1.5 * invdh * q[4] / (rho * tau_));
    const double S23 = -(1.5 * invdh * q[5] / (rho * tau_));
    const double S = S11 * S11 + S22 * S22 + S33 * S33 + 2.0 * (S12 * S12 + S13 * S13 + S23 * S23);
    double ox = les_diff(a, 2, 1, z, y, x, c);
    ox = 0.5 * (ox - les_diff(a, 1, 2, z, y, x, c));
    double oy = les_diff(a, 0, 2, z, y, x, c);
    oy = 0.5 * (oy - les_diff(a, 2, 0, z, y, x, c));
    double oz = les_diff(a, 1, 0, z, y, x, c);
    oz = 0.5 * (oz - les_diff(a, 0, 1, z, y, x, c));
    const double O12 = -(0.5 * oz), O13 = 0.5 * oy, O23 = -(0.5 * ox);
    const double O = 2.0 * (O12 * O12 + O23 * O23 + O13 * O13);
    const double SO11 = -(S11 * S11 * O12 * O12 + S11 * S11 * O13 * O13 + S12 * S12 * O12 * O12 +
                          S12 * S12 * O13 * O13 + S13 * S13 * O12 * O12 + S13 * S13 * O13 * O13);
    const double SO22 = -(S12 * S12 * O12 * O12 + S12 * S12 * O23 * O23 + S22 * S22 * O12 * O12 +
                          S22 * S22 * O23 * O23 + S23 * S23 * O12 * O12 + S23 * S23 * O23 * O23);
    const double SO33 = -(S13 * S13 * O13 * O13 + S13 * S13 * O23 * O23 + S23 * S23 * O13 * O13 +
                          S23 * S23 * O23 * O23 + S33 * S33 * O13 * O13 + S33 * S33 * O23 * O23);
    const double SO12 = -(S11 * S12 * O13 * O23 + S12 * S22 * O13 * O23 + S13 * S23 * O13 * O23);
    const double SO13 = (S11 * S13 * O12 * O23 + S12 * S23 * O12 * O23 + S13 * S33 * O12 * O23);
    const double SO23 = -(S12 * S13 * O12 * O13 + S22 * S23 * O12 * O13 + S23 * S33 * O12 * O13);
    const double SO = SO11 + SO22 + SO33 + 2.0 * (SO12 + SO13 + SO23);
    const double SdSd = (S * S + O * O) / 6.0 + 2.0 * S * O / 3.0 + 2.0 * SO;
    double OP = pow(SdSd, 1.5) / (pow(S, 2.5) + pow(SdSd, 1.25));
    if (!isfinite(OP) || OP < 0.0) OP = 0.0;
    const double t = (a.nu + a.cles * OP * a.dh * a.dh) / (a.dh * (1.0 / 3.0)) + 0.5;
    a.tau_all[c] = t;
    return 1.0 / t;
}

// vrem, FluidDomain.f90:1428-1506; a[i][j] = half the derivative of
// component i along axis j
__device__ double les_vrem(const StepArgs &a, int z, int y, int x, long long c) {
    double g[3][3], b[3][3];
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++) g[i][j] = 0.5 * les_diff(a, i, j, z, y, x, c);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) b[i][j] = g[i][j] * g[i][j];
    const double aa = b[0][0] + b[0][1] + b[0][2] + b[1][0] + b[1][1] + b[1][2] + b[2][0] + b[2][1] + b[2][2];
    const double r0 = b[0][0] + b[0][1] + b[0][2], r1 = b[1][0] + b[1][1] + b[1][2], r2 = b[2][0] + b[2][1] + b[2][2];
    const double d01 = g[0][0] * g[1][0] + g[0][1] * g[1][1] + g[0][2] * g[1][2];
    const double d02 = g[0][0] * g[2][0] + g[0][1] * g[2][1] + g[0][2] * g[2][2];
    const double d12 = g[1][0] * g[2][0] + g[1][1] * g[2][1] + g[1][2] * g[2][2];
    const double bb = r0 * r1 - d01 * d01 + r0 * r2 - d02 * d02 + r1 * r2 - d12 * d12;
    double OP = sqrt(bb / aa);
    if (!isfinite(OP)) OP = 0.0;
    const double t = (a.nu + a.cles * OP * a.dh * a.dh) / (a.dh * (1.0 / 3.0)) + 0.5;
    a.tau_all[c] = t;
    return 1.0 / t;
}

// ---------------------------------------------------------------- init/macro

__global__ void k_init(double *f, double *den, double *u, int X, int Y, int Z, double dh, double xmin,
                       double ymin, double zmin, double denIn, Vel vel, long long N) {
    int z = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, x = blockIdx.z;
    if (z >= Z) return;
    long long c = cidx(z, y, x, Z, Y);
    double xc = xmin + dh * (double)x, yc = ymin + dh * (double)y, zc = zmin + dh * (double)z;
    double v[3];
    eval_vel(vel, zc, yc, xc, v);
    den[c] = denIn;
    u[c] = v[0];
    u[c + N] = v[1];
    u[c + 2 * N] = v[2];
    double uSqr = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
#pragma unroll
    for (int i = 0; i < Q; i++) f[c + N * i] = feq_dist(i, denIn, v, uSqr);
}

__global__ void k_macro(const double *__restrict__ f, double *den, double *u, int Y, int Z, long long N,
                        double dh, double vf0, double vf1, double vf2) {
    int z = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, x = blockIdx.z;
    if (z >= Z) return;
    long long c = cidx(z, y, x, Z, Y);
    double fl[Q], vf[3] = {vf0, vf1, vf2};
#pragma unroll
    for (int i = 0; i < Q; i++) fl[i] = f[c + N * i];
    double d, u0, u1, u2;
    macro_cell(fl, vf, dh, d, u0, u1, u2);
    den[c] = d;
    u[c] = u0;
    u[c + N] = u1;
    u[c + 2 * N] = u2;
}

// den/uuu of every cell as the collision sees them (calculate_macro_quantities_,
// then the IB stage's values inside its window), written before the step of a
// model that reads its neighbours' velocity (WALE, Vreman)
__global__ void k_step_macro(StepArgs a) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, x = blockIdx.z;
    if (z >= a.Z) return;
    const long long c = cidx(z, y, x, a.Z, a.Y);
    const Win &w = a.win;
    double d, u0, u1, u2;
    if (x >= w.x0 && x <= w.x1 && y >= w.y0 && y <= w.y1 && z >= w.z0 && z <= w.z1) {
        long long wc = (long long)(z - w.z0) + (long long)w.WZ * ((long long)(y - w.y0) + (long long)w.WY * (x - w.x0));
        d = w.den[wc];
        u0 = w.u[wc]; u1 = w.u[wc + w.n]; u2 = w.u[wc + 2 * w.n];
    } else {
        const double *__restrict__ f = (const double *)a.src;
        double fl[Q];
#pragma unroll
        for (int i = 0; i < Q; i++) fl[i] = f[c + a.N * i];
        macro_cell(fl, a.vf, a.dh, d, u0, u1, u2);
    }
    a.den[c] = d;
    a.u[c] = u0;
    a.u[c + a.N] = u1;
    a.u[c + 2 * a.N] = u2;
}

// ------------------------------------------------------------ collide+stream
// One thread per cell. Reads the 19 populations of its cell, collides them
// (collision_, FluidDomain.f90:1208-1238) and pushes each post-collision
// population to the neighbour it streams to (streaming_, :1514-1625, periodic
// wrap on all axes). The destination buffer then holds the reference's
// post-streaming state, on which the face kernels act.
template <int MODEL>
__global__ void __launch_bounds__(TPB) k_step_exact(StepArgs a, MrtMats mm) {
    int z = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    int x = blockIdx.z;
    if (z >= a.Z || y >= a.Y) return;
    const int X = a.X, Y = a.Y, Z = a.Z;
    const long long N = a.N;
    const long long c = cidx(z, y, x, Z, Y);
    const double *__restrict__ src = (const double *)a.src;
    double *__restrict__ dst = (double *)a.dst;

    double f[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) f[i] = src[c + N * i];

    double den, u0, u1, u2, F0, F1, F2;
    const Win &w = a.win;
    if (x >= w.x0 && x <= w.x1 && y >= w.y0 && y <= w.y1 && z >= w.z0 && z <= w.z1) {
        long long wc = (long long)(z - w.z0) + (long long)w.WZ * ((long long)(y - w.y0) + (long long)w.WY * (x - w.x0));
        den = w.den[wc];
        u0 = w.u[wc]; u1 = w.u[wc + w.n]; u2 = w.u[wc + 2 * w.n];
        F0 = w.force[wc]; F1 = w.force[wc + w.n]; F2 = w.force[wc + 2 * w.n];
    } else {
        macro_cell(f, a.vf, a.dh, den, u0, u1, u2);
        // ResetVolumeForce_ then add_volume_force_: 0 + vf
        F0 = 0.0 + a.vf[0]; F1 = 0.0 + a.vf[1]; F2 = 0.0 + a.vf[2];
    }
    // den/uuu of layer 2 feed the non-equilibrium extrapolation (code 102);
    // the models that read neighbour velocities had them written beforehand
    if (!grad_model(MODEL) &&
        ((a.l2[0] && x == 1) || (a.l2[1] && x == X - 2) || (a.l2[2] && y == 1) || (a.l2[3] && y == Y - 2) ||
         (a.l2[4] && z == 1) || (a.l2[5] && z == Z - 2))) {
        a.den[c] = den;
        a.u[c] = u0; a.u[c + N] = u1; a.u[c + 2 * N] = u2;
    }

    const double uSqr = (u0 * u0 + u1 * u1) + u2 * u2;
    const double dt3 = 3.0 * a.dh;
    double fo[Q];
    if (MODEL == CM_SRT) {
        const double om = a.omega;
#pragma unroll
        for (int i = 0; i < Q; i++) {
            const double ex = ex_(i), ey = ey_(i), ez = ez_(i);
            double uxyz = (u0 * ex + u1 * ey) + u2 * ez;
            double fEq = ((wt_(i) * den) * ((1.0 - 1.5 * uSqr) + uxyz * (3.0 + 4.5 * uxyz))) - f[i];
            double Flb = (dt3 * wt_(i)) * (((((ex - u0) + (3.0 * uxyz) * ex) * F0) +
                                            (((ey - u1) + (3.0 * uxyz) * ey) * F1)) +
                                           (((ez - u2) + (3.0 * uxyz) * ez) * F2));
            fo[i] = (f[i] + om * fEq) + (1.0 - 0.5 * om) * Flb;
        }
    } else {
        double fEq[Q], Flb[Q];
#pragma unroll
        for (int i = 0; i < Q; i++) {
            const double ex = ex_(i), ey = ey_(i), ez = ez_(i);
            double uxyz = (u0 * ex + u1 * ey) + u2 * ez;
            fEq[i] = ((wt_(i) * den) * ((1.0 - 1.5 * uSqr) + uxyz * (3.0 + 4.5 * uxyz))) - f[i];
            Flb[i] = (dt3 * wt_(i)) * (((((ex - u0) + (3.0 * uxyz) * ex) * F0) +
                                        (((ey - u1) + (3.0 * uxyz) * ey) * F1)) +
                                       (((ez - u2) + (3.0 * uxyz) * ez) * F2));
        }
        if (MODEL == CM_MRT) {
#pragma unroll
            for (int i = 0; i < Q; i++) {
                double s1 = 0.0, s2 = 0.0;
#pragma unroll
                for (int j = 0; j < Q; j++) s1 += mm.mc[i + Q * j] * fEq[j];
#pragma unroll
                for (int j = 0; j < Q; j++) s2 += mm.mf[i + Q * j] * Flb[j];
                fo[i] = (f[i] + s1) + s2;
            }
        } else if (MODEL == CM_TRT) {
            // TRT collision, FluidDomain.f90:1228-1235
            const double om = a.omega, om2 = a.omega2;
            fo[0] = f[0] + (om * fEq[0] + (1.0 - 0.5 * om) * Flb[0]);
#pragma unroll
            for (int k = 0; k < 9; k++) {
                const int p = pr_(k), m = opp_(p);
                const double sp = 0.5 * om * (fEq[p] + fEq[m]) + (0.5 - 0.25 * om) * (Flb[p] + Flb[m]);
                const double sm = 0.5 * om2 * (fEq[p] - fEq[m]) + (0.5 - 0.25 * om2) * (Flb[p] - Flb[m]);
                fo[p] = f[p] + (sp + sm);
                fo[m] = f[m] + (sp - sm);
            }
        } else {
            // SRT with a per-cell rate, FluidDomain.f90:1239-1262
            const double om = MODEL == CM_SMAG ? les_smag(a, fEq, den, c)
                            : MODEL == CM_WALE ? les_wale(a, fEq, den, z, y, x, c)
                                               : les_vrem(a, z, y, x, c);
#pragma unroll
            for (int i = 0; i < Q; i++) fo[i] = (f[i] + om * fEq[i]) + (1.0 - 0.5 * om) * Flb[i];
        }
    }

    // halfwayBCset_ (FluidDomain.f90:567-614): keep post-collision faces
    if (a.hw[0] && x == 0) { double *h = a.hw[0] + (long long)Q * (z + (long long)Z * y);
#pragma unroll
        for (int i = 0; i < Q; i++) h[i] = fo[i]; }
    if (a.hw[1] && x == X - 1) { double *h = a.hw[1] + (long long)Q * (z + (long long)Z * y);
#pragma unroll
        for (int i = 0; i < Q; i++) h[i] = fo[i]; }
    if (a.hw[2] && y == 0) { double *h = a.hw[2] + (long long)Q * (z + (long long)Z * x);
#pragma unroll
        for (int i = 0; i < Q; i++) h[i] = fo[i]; }
    if (a.hw[3] && y == Y - 1) { double *h = a.hw[3] + (long long)Q * (z + (long long)Z * x);
#pragma unroll
        for (int i = 0; i < Q; i++) h[i] = fo[i]; }
    if (a.hw[4] && z == 0) { double *h = a.hw[4] + (long long)Q * (y + (long long)Y * x);
#pragma unroll
        for (int i = 0; i < Q; i++) h[i] = fo[i]; }
    if (a.hw[5] && z == Z - 1) { double *h = a.hw[5] + (long long)Q * (y + (long long)Y * x);
#pragma unroll
        for (int i = 0; i < Q; i++) h[i] = fo[i]; }

    // push to the streaming destination
    const int zp = (z + 1 == Z) ? 0 : z + 1, zm = (z == 0) ? Z - 1 : z - 1;
    const int yp = (y + 1 == Y) ? 0 : y + 1, ym = (y == 0) ? Y - 1 : y - 1;
    const int xp = (x + 1 == X) ? 0 : x + 1, xm = (x == 0) ? X - 1 : x - 1;
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const int zd = ez_(i) > 0 ? zp : (ez_(i) < 0 ? zm : z);
        const int yd = ey_(i) > 0 ? yp : (ey_(i) < 0 ? ym : y);
        const int xd = ex_(i) > 0 ? xp : (ex_(i) < 0 ? xm : x);
        dst[cidx(zd, yd, xd, Z, Y) + N * i] = fo[i];
    }
}

__global__ void k_halfway(const double *__restrict__ f, double *hw, int X, int Y, int Z, int face) {
    const int ax = face >> 1, side = face & 1;
    const int A = (ax < 2) ? Z : Y, B = (ax == 0) ? Y : X;
    int fa = blockIdx.x * blockDim.x + threadIdx.x, fb = blockIdx.y;
    if (fa >= A || fb >= B) return;
    long long c;
    if (ax == 0) c = cidx(fa, fb, side ? X - 1 : 0, Z, Y);
    else if (ax == 1) c = cidx(fa, side ? Y - 1 : 0, fb, Z, Y);
    else c = cidx(side ? Z - 1 : 0, fa, fb, Z, Y);
    long long N = (long long)X * Y * Z;
    double *h = hw + (long long)Q * ((long long)fa + (long long)A * fb);
    for (int i = 0; i < Q; i++) h[i] = f[c + N * i];
}

// ------------------------------------------------------ immersed boundary

__global__ void k_win_macro(const double *__restrict__ f, double *wden, double *wu, IbGeom g, long long N,
                            long long Nw, double vf0, double vf1, double vf2) {
    long long wc = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (wc >= Nw) return;
    int wz = (int)(wc % g.WZ);
    long long t = wc / g.WZ;
    int wy = (int)(t % g.WY), wx = (int)(t / g.WY);
    long long c = cidx(wz + g.wz0, wy + g.wy0, wx + g.wx0, g.Z, g.Y);
    double fl[Q], vf[3] = {vf0, vf1, vf2};
#pragma unroll
    for (int i = 0; i < Q; i++) fl[i] = f[c + N * i];
    double d, u0, u1, u2;
    macro_cell(fl, vf, g.dh, d, u0, u1, u2);
    wden[wc] = d;
    wu[wc] = u0; wu[wc + Nw] = u1; wu[wc + 2 * Nw] = u2;
}

// UpdateElmtInterp_, Solidbody.f90:760-807. One thread per marker; the
// stencil origin comes from the first marker of the marker's body.
// Out-of-window indices come back clamped into the window so that no later
// kernel reads outside it; the host reports the error and stops.
__global__ void k_ib_stencil(const double *__restrict__ xyz, const int *__restrict__ offs, int nb, int Mtot,
                             IbGeom g, int16_t *ei, float *ew, int *err) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= Mtot) return;
    int b = 0;
    while (b + 1 < nb && m >= offs[b + 1]) b++;
    const int st = ib_stencil_one(xyz + 3LL * offs[b], xyz + 3LL * m, g, ei + 12LL * m, ew + 12LL * m);
    if (st) atomicOr(err, st);
}

// window cell of stencil entry e = marker*64 + (x*16 + y*4 + z)
__device__ __forceinline__ long long entry_cell(const int16_t *ei, const IbGeom &g, long long e) {
    long long m = e >> 6;
    int p = (int)(e & 63);
    const int16_t *s = ei + 12 * m;
    int xi = s[p >> 4] - 1, yi = s[4 + ((p >> 2) & 3)] - 1, zi = s[8 + (p & 3)] - 1;
    return (long long)(zi - g.wz0) + (long long)g.WZ * ((long long)(yi - g.wy0) + (long long)g.WY * (xi - g.wx0));
}

__global__ void k_ib_count(const int16_t *ei, long long E, IbGeom g, int *cnt) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= E) return;
    atomicAdd(cnt + entry_cell(ei, g, e), 1);
}

// exclusive scan of cnt[0..n) into start[0..n], one block
__global__ void k_scan(const int *cnt, int *start, long long n) {
    __shared__ int sh[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long long base = 0; base < n; base += 1024) {
        long long i = base + threadIdx.x;
        int v = (i < n) ? cnt[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            int t = (threadIdx.x >= off) ? sh[threadIdx.x - off] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < n) start[i] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += sh[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) start[n] = carry;
}

__global__ void k_ib_fill(const int16_t *ei, long long E, IbGeom g, const int *start, int *fillc, int *list) {
    long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= E) return;
    long long wc = entry_cell(ei, g, e);
    int slot = start[wc] + atomicAdd(fillc + wc, 1);
    list[slot] = (int)e;
}

// order each cell's entries by entry id: (body, marker, x, y, z) -- the
// reference's serial scatter order (Solidbody.f90:1034-1048, 938-977)
__global__ void k_ib_sort(const int *start, int *list, long long Nw) {
    long long wc = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (wc >= Nw) return;
    int s0 = start[wc], s1 = start[wc + 1];
    for (int i = s0 + 1; i < s1; i++) {
        int v = list[i], j = i - 1;
        while (j >= s0 && list[j] > v) { list[j + 1] = list[j]; j--; }
        list[j + 1] = v;
    }
}

// PenaltyForce_ interpolation part, Solidbody.f90:1001-1026
__global__ void k_ib_interp(const int16_t *__restrict__ ei, const float *__restrict__ ew,
                            const double *__restrict__ vel, const double *__restrict__ area,
                            const double *__restrict__ wu, IbGeom g, long long Nw, int m0, int m1,
                            double invh3, double *eforce, double *fet, double *tolm) {
    int m = m0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= m1) return;
    const int16_t *s = ei + 12LL * m;
    const float *w = ew + 12LL * m;
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
    for (int x = 0; x < 4; x++) {
        const double rx = (double)w[x];
        const long long cx = (long long)(s[x] - 1 - g.wx0);
        for (int y = 0; y < 4; y++) {
            const double ry = (double)w[4 + y];
            const long long cy = (long long)(s[4 + y] - 1 - g.wy0);
#pragma unroll
            for (int z = 0; z < 4; z++) {
                const double rz = (double)w[8 + z];
                const long long wc = (long long)(s[8 + z] - 1 - g.wz0) + (long long)g.WZ * (cy + (long long)g.WY * cx);
                v0 = v0 + ((wu[wc] * rx) * ry) * rz;
                v1 = v1 + ((wu[wc + Nw] * rx) * ry) * rz;
                v2 = v2 + ((wu[wc + 2 * Nw] * rx) * ry) * rz;
            }
        }
    }
    v0 = vel[3LL * m] - v0;
    v1 = vel[3LL * m + 1] - v1;
    v2 = vel[3LL * m + 2] - v2;
    const double ar = area[m];
    const double F0 = v0 * ar, F1 = v1 * ar, F2 = v2 * ar;
    tolm[m] = (fabs(v0) + fabs(v1)) + fabs(v2);
    eforce[3LL * m] = eforce[3LL * m] + F0;
    eforce[3LL * m + 1] = eforce[3LL * m + 1] + F1;
    eforce[3LL * m + 2] = eforce[3LL * m + 2] + F2;
    fet[3LL * m] = F0 * invh3;
    fet[3LL * m + 1] = F1 * invh3;
    fet[3LL * m + 2] = F2 * invh3;
}

// deterministic fixed-order sum of tolm[m0..m1)
__global__ void k_ib_reduce(const double *tolm, int m0, int m1, double *out) {
    __shared__ double sh[256];
    double s = 0.0;
    for (int m = m0 + threadIdx.x; m < m1; m += 256) s = s + tolm[m];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < off) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// PenaltyForce_ velocity correction, Solidbody.f90:1034-1048, as a gather:
// each window cell applies its entries of markers [m0,m1) in entry order
__global__ void k_ib_correct(const float *__restrict__ ew, const int *__restrict__ start,
                             const int *__restrict__ list, long long Nw, int m0, int m1,
                             const double *__restrict__ fet, double *wu) {
    long long wc = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (wc >= Nw) return;
    int s0 = start[wc], s1 = start[wc + 1];
    if (s0 == s1) return;
    double u0 = wu[wc], u1 = wu[wc + Nw], u2 = wu[wc + 2 * Nw];
    bool touched = false;
    for (int s = s0; s < s1; s++) {
        int e = list[s];
        int m = e >> 6, p = e & 63;
        if (m < m0 || m >= m1) continue;
        const float *w = ew + 12LL * m;
        const double rx = (double)w[p >> 4], ry = (double)w[4 + ((p >> 2) & 3)], rz = (double)w[8 + (p & 3)];
        u0 = u0 - ((fet[3LL * m] * rx) * ry) * rz;
        u1 = u1 - ((fet[3LL * m + 1] * rx) * ry) * rz;
        u2 = u2 - ((fet[3LL * m + 2] * rx) * ry) * rz;
        touched = true;
    }
    if (touched) { wu[wc] = u0; wu[wc + Nw] = u1; wu[wc + 2 * Nw] = u2; }
}

// FluidVolumeForce_ spreading (Solidbody.f90:968-977) onto a zeroed force,
// then add_volume_force_ (FluidDomain.f90:1182-1193)
__global__ void k_ib_spread(const float *__restrict__ ew, const int *__restrict__ start,
                            const int *__restrict__ list, long long Nw, const double *__restrict__ eforce,
                            double invh3, double vf0, double vf1, double vf2, double *wforce) {
    long long wc = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (wc >= Nw) return;
    int s0 = start[wc], s1 = start[wc + 1];
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int s = s0; s < s1; s++) {
        int e = list[s];
        int m = e >> 6, p = e & 63;
        const float *w = ew + 12LL * m;
        const double rx = (double)w[p >> 4], ry = (double)w[4 + ((p >> 2) & 3)], rz = (double)w[8 + (p & 3)];
        const double f0 = eforce[3LL * m] * invh3, f1 = eforce[3LL * m + 1] * invh3, f2 = eforce[3LL * m + 2] * invh3;
        a0 = a0 + (-(((f0 * rx) * ry) * rz));
        a1 = a1 + (-(((f1 * rx) * ry) * rz));
        a2 = a2 + (-(((f2 * rx) * ry) * rz));
    }
    wforce[wc] = a0 + vf0;
    wforce[wc + Nw] = a1 + vf1;
    wforce[wc + 2 * Nw] = a2 + vf2;
}

// ---------------------------------------------------------------- outputs
// write_flow_ (FluidDomain.f90:1651-1663), outputtype 1: the FP32 output
// fields over the block minus `off` cells on every side, (z,y,x,k) order:
// p = Cs2 (den - denIn) and u/Uref, rounded from FP64 as the reference's
// real(4) OUTtmp
__global__ void k_pack_flow(const double *__restrict__ den, const double *__restrict__ u, long long N, int X, int Y,
                            int Z, int off, double denIn, double invUref, float *out) {
    const int nz = Z - 2 * off, ny = Y - 2 * off, nx = X - 2 * off;
    const long long n = (long long)nz * ny * nx;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int zz = (int)(i % nz);
    const long long t = i / nz;
    const int yy = (int)(t % ny), xx = (int)(t / ny);
    const long long c = cidx(zz + off, yy + off, xx + off, Z, Y);
    const double Cs2 = 1.0 / 3.0;  // ConstParams.f90:39
    out[i] = (float)(Cs2 * (den[c] - denIn));
    out[i + n] = (float)(u[c] * invUref);
    out[i + 2 * n] = (float)(u[c + N] * invUref);
    out[i + 3 * n] = (float)(u[c + 2 * N] * invUref);
}

// write_fluid_flux (FluidDomain.f90:2019-2056): the x-flux through the
// planes x = 1, (xDim+1)/2 and xDim (1-based), one thread per plane summing
// in the reference's loop order (z outer, y inner) with its trapezoid weights
__global__ void k_flux(const double *__restrict__ den, const double *__restrict__ u, long long N, int X, int Y, int Z,
                       double dh, double *flux) {
    const int p = threadIdx.x;
    if (p >= 3) return;
    const int x = p == 0 ? 0 : (p == 1 ? (X + 1) / 2 - 1 : X - 1);
    double s = 0.0;
    for (int k = 0; k < Z; k++) {
        const double wz = (k == 0 || k == Z - 1) ? 0.5 : 1.0;
        for (int j = 0; j < Y; j++) {
            const double wy = (j == 0 || j == Y - 1) ? 0.5 : 1.0;
            const long long c = cidx(k, j, x, Z, Y);
            s = s + ((((u[c] * den[c]) * dh) * dh) * wy) * wz;
        }
    }
    flux[p] = s;
}

// grid_value_interpolation (Util.f90:123-158): trilinear velocity at probe
// points, one thread per probe and component; points on the last grid plane
// take their upper neighbour as the same plane (its weight is zero)
__global__ void k_probes(const double *__restrict__ u, long long N, int X, int Y, int Z, double dh, double xmin,
                         double ymin, double zmin, int n, const double *__restrict__ xyz, double invUref, double *out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * n) return;
    const int i = t / 3, comp = t % 3;
    const double cx = xyz[3 * i], cy = xyz[3 * i + 1], cz = xyz[3 * i + 2];
    int x1 = (int)floor((cx - xmin) / dh + 1.0), y1 = (int)floor((cy - ymin) / dh + 1.0),
        z1 = (int)floor((cz - zmin) / dh + 1.0);
    int x2 = x1 + 1, y2 = y1 + 1, z2 = z1 + 1;
    const double dx1 = cx - (xmin + dh * (double)(x1 - 1));
    const double dy1 = cy - (ymin + dh * (double)(y1 - 1));
    const double dz1 = cz - (zmin + dh * (double)(z1 - 1));
    const double dx2 = dh - dx1, dy2 = dh - dy1, dz2 = dh - dz1;
    x2 = x2 > X ? X : x2;
    y2 = y2 > Y ? Y : y2;
    z2 = z2 > Z ? Z : z2;
    const double coffe = 1.0 / ((dh * dh) * dh);
    const double c1 = ((dx2 * dy2) * dz2) * coffe, c2 = ((dx2 * dy2) * dz1) * coffe, c3 = ((dx2 * dy1) * dz2) * coffe,
                 c4 = ((dx1 * dy2) * dz2) * coffe, c5 = ((dx2 * dy1) * dz1) * coffe, c6 = ((dx1 * dy2) * dz1) * coffe,
                 c7 = ((dx1 * dy1) * dz2) * coffe, c8 = ((dx1 * dy1) * dz1) * coffe;
    const double *v = u + N * comp;
    auto at = [&](int z, int y, int x) { return v[cidx(z - 1, y - 1, x - 1, Z, Y)]; };
    const double val = ((((((c1 * at(z1, y1, x1) + c2 * at(z2, y1, x1)) + c3 * at(z1, y2, x1)) + c4 * at(z1, y1, x2)) +
                          c5 * at(z2, y2, x1)) + c6 * at(z2, y1, x2)) + c7 * at(z1, y2, x2)) + c8 * at(z2, y2, x2);
    out[t] = val * invUref;
}

// ------------------------------------------------------- block refinement
// The face kernels check every global index against its buffer; the first
// out-of-range access is recorded in err (code, index low, index high) and
// skipped, and the host turns it into FSI_E_RANGE.
__device__ __forceinline__ void rec_err(int *err, int code, long long idx) {
    if (atomicCAS(err, 0, code) == 0) {
        err[1] = (int)(idx & 0xffffffffLL);
        err[2] = (int)(idx >> 32);
    }
}

// extract_interpolate_layer for one son face (LBMBlockComm.f90:354-369):
// buf(e, a, b) = father fIn on the face plane; buft = father tau
template <int P>
__global__ void k_pair_extract(const void *__restrict__ ff, int FY, int FZ, long long NF, TauSrc tf, PairGeom p,
                               int face, double *buf, double *buft, int A, int B, int *err) {
    int a = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (a >= A || b >= B) return;
    int ax = face >> 1, xF, yF, zF;
    if (ax == 0) { xF = p.f[face]; yF = b + p.f[2]; zF = a + p.f[4]; }
    else if (ax == 1) { yF = p.f[face]; xF = b + p.f[0]; zF = a + p.f[4]; }
    else { zF = p.f[face]; xF = b + p.f[0]; yF = a + p.f[2]; }
    long long c = cidx(zF - 1, yF - 1, xF - 1, FZ, FY);
    long long o = (long long)a + (long long)A * b;
    if (c < 0 || c >= NF) { rec_err(err, 4, c); return; }
    for (int e = 0; e < Q; e++) buf[e + Q * o] = FAcc<P>::load(ff, c + NF * e, e);
    buft[o] = tf.at(c);
}

template <typename T>
__global__ void k_fill(T *p, long long n, T v) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

__global__ void k_pair_average(double *b1, const double *b2, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) b1[i] = 0.5 * (b1[i] + b2[i]);
}

// fIn_GridTransform, LBMBlockComm.f90:958-979
__device__ __forceinline__ void grid_transform(double fin[Q], double coeff, const double vf[3], double dh) {
    double den, u0, u1, u2;
    macro_cell(fin, vf, dh, den, u0, u1, u2);
    double uSqr = (u0 * u0 + u1 * u1) + u2 * u2;
#pragma unroll
    for (int i = 0; i < Q; i++) {
        double uxyz = (u0 * (double)ex_(i) + u1 * (double)ey_(i)) + u2 * (double)ez_(i);
        double fEq = (wt_(i) * den) * ((1.0 - 1.5 * uSqr) + uxyz * (3.0 + 4.5 * uxyz));
        fin[i] = fEq + coeff * (fin[i] - fEq);
    }
}

// interpolate_fIn / interpolate_tau (LBMBlockComm.f90:808-956), one thread
// per population q (nq threads), the reference's loop sequence per thread.
// fF(nq,bF,aF) -> fS(nq,bS,aS).
struct Checked {
    double *p;
    long long n;
    int *err;
    int code;
    __device__ double &at(long long i) {
        if (i < 0 || i >= n) { rec_err(err, code, i); return dummy; }
        return p[i];
    }
    double dummy;
};

__global__ void k_pair_interp(int nq, int bF, const double *__restrict__ fFp, long long nF, int bS, int aS,
                              double *fSp, long long nS, int scheme, int *err) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    Checked cF{const_cast<double *>(fFp), nF, err, 1, 0.0};
    Checked cS{fSp, nS, err, 2, 0.0};
#define FF(b_, a_) cF.at(q + (long long)nq * (((b_) - 1) + (long long)bF * ((a_) - 1)))
#define FS(b_, a_) cS.at(q + (long long)nq * (((b_) - 1) + (long long)bS * ((a_) - 1)))
    int r1 = 0, r2 = 0, bSt = bS, aSt = aS;
    if (bS % 2 == 0) { bSt = bS - 1; r2 = 1; }
    if (aS % 2 == 0) { aSt = aS - 1; r1 = 1; }
    if (scheme == 2) {
        for (int b = 1; b <= bSt; b += 2) {
            int b1 = b / 2 + 1;
            for (int a = 1; a <= aSt; a += 2) {
                int a1 = a / 2 + 1;
                FS(b, a) = FF(b1, a1);
                if (b == 1) FS(b + 1, a) = (0.375 * FF(b1, a1) + 0.75 * FF(b1 + 1, a1)) - 0.125 * FF(b1 + 2, a1);
                else if (b == bSt - 2) FS(b + 1, a) = (0.375 * FF(b1 + 1, a1) + 0.75 * FF(b1, a1)) - 0.125 * FF(b1 - 1, a1);
                else if (b != bSt)
                    FS(b + 1, a) = (((-(0.0625 * FF(b1 - 1, a1))) + 0.5625 * FF(b1, a1)) + 0.5625 * FF(b1 + 1, a1)) - 0.0625 * FF(b1 + 2, a1);
            }
        }
        for (int b = 1; b <= bSt; b++)
            for (int a = 2; a <= aSt; a += 2) {
                if (a == 2) FS(b, a) = (0.375 * FS(b, a - 1) + 0.75 * FS(b, a + 1)) - 0.125 * FS(b, a + 3);
                else if (a == aSt - 1) FS(b, a) = (0.375 * FS(b, a + 1) + 0.75 * FS(b, a - 1)) - 0.125 * FS(b, a - 3);
                else FS(b, a) = (((-(0.0625 * FS(b, a - 3))) + 0.5625 * FS(b, a - 1)) + 0.5625 * FS(b, a + 1)) - 0.0625 * FS(b, a + 3);
            }
        if (r2)
            for (int a = 1; a <= aSt; a++)
                FS(bSt + 1, a) = (((-(0.0625 * FS(bSt - 2, a))) + 0.5625 * FS(bSt, a)) + 0.5625 * FS(1, a)) - 0.0625 * FS(3, a);
        if (r1) {
            for (int b = 1; b <= bSt; b++)
                FS(b, aSt + 1) = (((-(0.0625 * FS(b, aSt - 2))) + 0.5625 * FS(b, aSt)) + 0.5625 * FS(b, 1)) - 0.0625 * FS(b, 3);
            if (r2)
                FS(bSt + 1, aSt + 1) = (((-(0.0625 * FS(bSt + 1, aSt - 2))) + 0.5625 * FS(bSt + 1, aSt)) + 0.5625 * FS(bSt + 1, 1)) - 0.0625 * FS(bSt + 1, 3);
        }
    } else {
        for (int b = 1; b <= bSt; b += 2) {
            int b1 = b / 2 + 1;
            for (int a = 1; a <= aSt; a += 2) {
                int a1 = a / 2 + 1;
                FS(b, a) = FF(b1, a1);
                if (b < bSt) FS(b + 1, a) = (FF(b1, a1) + FF(b1 + 1, a1)) * 0.5;
            }
        }
        for (int b = 1; b <= bSt; b++)
            for (int a = 2; a <= aSt; a += 2) FS(b, a) = (FS(b, a - 1) + FS(b, a + 1)) * 0.5;
        if (r2)
            for (int a = 1; a <= aSt; a++) FS(bSt + 1, a) = (FS(bSt, a) + FS(1, a)) * 0.5;
        if (r1) {
            for (int b = 1; b <= bSt; b++) FS(b, aSt + 1) = (FS(b, aSt) + FS(b, 1)) * 0.5;
            if (r2) FS(bSt + 1, aSt + 1) = (FS(bSt + 1, aSt) + FS(bSt + 1, 1)) * 0.5;
        }
    }
#undef FF
#undef FS
}

// interpolation_father_to_son apply step (LBMBlockComm.f90:685-693)
template <int P>
__global__ void k_pair_f2s_apply(void *fs, int SY, int SZ, long long NS, TauSrc ts, PairGeom p, int face,
                                 const double *tf, const double *tt, int AS, int BS, double vf0, double vf1,
                                 double vf2, double dh, int *err) {
    int a = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (a >= AS || b >= BS) return;
    int ax = face >> 1, xS, yS, zS;
    if (ax == 0) { xS = p.s[face]; yS = b + 1; zS = a + 1; }
    else if (ax == 1) { yS = p.s[face]; xS = b + 1; zS = a + 1; }
    else { zS = p.s[face]; xS = b + 1; yS = a + 1; }
    long long c = cidx(zS - 1, yS - 1, xS - 1, SZ, SY);
    long long o = (long long)a + (long long)AS * b;
    if (c < 0 || c >= NS) { rec_err(err, 3, c); return; }
    double coeff = (ts.at(c) / tt[o]) / 2.0;
    double fin[Q], vf[3] = {vf0, vf1, vf2};
    for (int e = 0; e < Q; e++) fin[e] = tf[Q * o + e];
    grid_transform(fin, coeff, vf, dh);
    for (int e = 0; e < Q; e++) FAcc<P>::store(fs, c + NS * e, e, fin[e]);
}

// deliver_son_to_father for one face (LBMBlockComm.f90:555-570 and siblings)
template <int P>
__global__ void k_pair_s2f(void *ff, int FY, int FZ, long long NF, TauSrc tf, const void *__restrict__ fs, int SY,
                           int SZ, long long NS, TauSrc ts, PairGeom p, int face, int n1, int n2,
                           double vf0, double vf1, double vf2, double dh, int *err) {
    int i1 = blockIdx.x * blockDim.x + threadIdx.x, i2 = blockIdx.y;
    if (i1 >= n2 || i2 >= n1) return;
    int ax = face >> 1;
    int o1 = (ax == 0) ? 1 : 0, o2 = (ax == 2) ? 1 : 2;
    int S[3], F[3];
    S[ax] = p.si[face]; F[ax] = p.fi[face];
    int v1 = p.si[2 * o1] + 2 * i2, v2 = p.si[2 * o2] + 2 * i1;
    S[o1] = v1; F[o1] = (v1 - p.si[2 * o1]) / 2 + p.fi[2 * o1];
    S[o2] = v2; F[o2] = (v2 - p.si[2 * o2]) / 2 + p.fi[2 * o2];
    long long cs = cidx(S[2] - 1, S[1] - 1, S[0] - 1, SZ, SY);
    long long cf = cidx(F[2] - 1, F[1] - 1, F[0] - 1, FZ, FY);
    if (cs < 0 || cs >= NS) { rec_err(err, 5, cs); return; }
    if (cf < 0 || cf >= NF) { rec_err(err, 6, cf); return; }
    double coeff = (tf.at(cf) / ts.at(cs)) * 2.0;
    double t[Q], vf[3] = {vf0, vf1, vf2};
    for (int e = 0; e < Q; e++) t[e] = FAcc<P>::load(fs, cs + NS * e, e);
    grid_transform(t, coeff, vf, dh);
    for (int e = 0; e < Q; e++) FAcc<P>::store(ff, cf + NF * e, e, t[e]);
}

// check_is_continue's trilinear re-grid (FluidDomain.f90:170-226): each
// cell takes the first file block (in search order) that contains it and
// blends its 8 surrounding nodes in the reference's order; cells outside
// every file block keep their values
__global__ void k_regrid(double *__restrict__ f, int X, int Y, int Z, double dh, double xmin, double ymin,
                         double zmin, const RegridSrc *__restrict__ src, int nsrc, int *err) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, x = blockIdx.z;
    if (z >= Z) return;
    const double xc = xmin + (double)x * dh, yc = ymin + (double)y * dh, zc = zmin + (double)z * dh;
    const long long N = (long long)X * Y * Z, c = cidx(z, y, x, Z, Y);
    for (int j = 0; j < nsrc; j++) {
        const RegridSrc o = src[j];
        if (!(zc >= o.zmin && zc <= o.zmx && yc >= o.ymin && yc <= o.ymx && xc >= o.xmin && xc <= o.xmx)) continue;
        double c1 = (xc - o.xmin) / o.dh, c2 = (yc - o.ymin) / o.dh, c3 = (zc - o.zmin) / o.dh;
        int i1 = (int)floor(c1), i3 = (int)floor(c2), i5 = (int)floor(c3);
        if (i1 == o.X - 1) i1 = i1 - 1;
        if (i3 == o.Y - 1) i3 = i3 - 1;
        if (i5 == o.Z - 1) i5 = i5 - 1;
        if (i1 < 0 || i1 + 1 >= o.X || i3 < 0 || i3 + 1 >= o.Y || i5 < 0 || i5 + 1 >= o.Z) {
            rec_err(err, 7, c);
            return;
        }
        c1 = c1 - (double)i1;
        c2 = c2 - (double)i3;
        c3 = c3 - (double)i5;
        const long long no = (long long)o.X * o.Y * o.Z;
        const long long a000 = cidx(i5, i3, i1, o.Z, o.Y), a001 = cidx(i5, i3, i1 + 1, o.Z, o.Y);
        const long long a010 = cidx(i5, i3 + 1, i1, o.Z, o.Y), a011 = cidx(i5, i3 + 1, i1 + 1, o.Z, o.Y);
        const long long a100 = cidx(i5 + 1, i3, i1, o.Z, o.Y), a101 = cidx(i5 + 1, i3, i1 + 1, o.Z, o.Y);
        const long long a110 = cidx(i5 + 1, i3 + 1, i1, o.Z, o.Y), a111 = cidx(i5 + 1, i3 + 1, i1 + 1, o.Z, o.Y);
        for (int q = 0; q < Q; q++) {
            const double *__restrict__ g = o.f + no * q;
            f[c + N * q] = g[a000] * (1.0 - c3) * (1.0 - c2) * (1.0 - c1) + g[a001] * (1.0 - c3) * (1.0 - c2) * c1 +
                           g[a010] * (1.0 - c3) * c2 * (1.0 - c1) + g[a011] * (1.0 - c3) * c2 * c1 +
                           g[a100] * c3 * (1.0 - c2) * (1.0 - c1) + g[a101] * c3 * (1.0 - c2) * c1 +
                           g[a110] * c3 * c2 * (1.0 - c1) + g[a111] * c3 * c2 * c1;
        }
        return;
    }
}

inline dim3 zgrid(int Z, int Y, int X, int &bz) {
    bz = Z >= 256 ? 256 : ((Z + 31) / 32) * 32;
    return dim3((Z + bz - 1) / bz, Y, X);
}

}  // namespace

// ----------------------------------------------------------------- launchers

cudaError_t launch_init_f64(double *f, double *den, double *u, int X, int Y, int Z, double dh, double xmin,
                            double ymin, double zmin, double denIn, const Vel &vel, double blktime,
                            cudaStream_t st) {
    (void)blktime;
    int bz;
    dim3 g = zgrid(Z, Y, X, bz);
    k_init<<<g, bz, 0, st>>>(f, den, u, X, Y, Z, dh, xmin, ymin, zmin, denIn, vel, (long long)X * Y * Z);
    return cudaGetLastError();
}

cudaError_t launch_macro_f64(const double *f, double *den, double *u, int X, int Y, int Z, double dh,
                             const double vf[3], cudaStream_t st) {
    int bz;
    dim3 g = zgrid(Z, Y, X, bz);
    k_macro<<<g, bz, 0, st>>>(f, den, u, Y, Z, (long long)X * Y * Z, dh, vf[0], vf[1], vf[2]);
    return cudaGetLastError();
}

cudaError_t launch_step_macro_f64(const StepArgs &a, cudaStream_t st) {
    int bz;
    dim3 g = zgrid(a.Z, a.Y, a.X, bz);
    k_step_macro<<<g, bz, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_step_f64_exact(const StepArgs &a, const MrtMats *mm, int model, cudaStream_t st) {
    int bz = a.Z >= 128 ? 128 : ((a.Z + 31) / 32) * 32;
    int by = TPB / bz;
    if (by < 1) by = 1;
    dim3 blk(bz, by), grd((a.Z + bz - 1) / bz, (a.Y + by - 1) / by, a.X);
    switch (model) {
    case CM_MRT: k_step_exact<CM_MRT><<<grd, blk, 0, st>>>(a, *mm); break;
    case CM_TRT: k_step_exact<CM_TRT><<<grd, blk, 0, st>>>(a, MrtMats{}); break;
    case CM_SMAG: k_step_exact<CM_SMAG><<<grd, blk, 0, st>>>(a, MrtMats{}); break;
    case CM_WALE: k_step_exact<CM_WALE><<<grd, blk, 0, st>>>(a, MrtMats{}); break;
    case CM_VREM: k_step_exact<CM_VREM><<<grd, blk, 0, st>>>(a, MrtMats{}); break;
    default: k_step_exact<CM_SRT><<<grd, blk, 0, st>>>(a, MrtMats{}); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_bc_f64(const BcArgs &a, cudaStream_t st) {
    const int A = (a.face < 4) ? a.Z : a.Y;
    const int B = (a.face < 2) ? a.Y : a.X;
    dim3 blk(64, 4), grd((A + 63) / 64, (B + 3) / 4);
    switch (a.face) {
    case 0: k_bc<AccF64, 0><<<grd, blk, 0, st>>>(a); break;
    case 1: k_bc<AccF64, 1><<<grd, blk, 0, st>>>(a); break;
    case 2: k_bc<AccF64, 2><<<grd, blk, 0, st>>>(a); break;
    case 3: k_bc<AccF64, 3><<<grd, blk, 0, st>>>(a); break;
    case 4: k_bc<AccF64, 4><<<grd, blk, 0, st>>>(a); break;
    default: k_bc<AccF64, 5><<<grd, blk, 0, st>>>(a); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_halfway_f64(const double *f, double *hw, int X, int Y, int Z, int face, cudaStream_t st) {
    const int ax = face >> 1;
    const int A = (ax < 2) ? Z : Y, B = (ax == 0) ? Y : X;
    k_halfway<<<dim3((A + 127) / 128, B), 128, 0, st>>>(f, hw, X, Y, Z, face);
    return cudaGetLastError();
}

cudaError_t launch_win_macro_f64(const void *f, int prec, double *wden, double *wu, const IbGeom &g, long long N,
                                 const double vf[3], cudaStream_t st) {
    (void)prec;
    long long Nw = (long long)(g.wx1 - g.wx0 + 1) * g.WY * g.WZ;
    if (Nw <= 0) return cudaSuccess;
    k_win_macro<<<(unsigned)((Nw + 255) / 256), 256, 0, st>>>((const double *)f, wden, wu, g, N, Nw, vf[0], vf[1], vf[2]);
    return cudaGetLastError();
}

cudaError_t launch_ib_stencil(const double *xyz, const int *offs, int nb, int Mtot, const IbGeom &g, int16_t *ei,
                              float *ew, int *err, cudaStream_t st) {
    if (Mtot <= 0) return cudaSuccess;
    k_ib_stencil<<<(Mtot + 127) / 128, 128, 0, st>>>(xyz, offs, nb, Mtot, g, ei, ew, err);
    return cudaGetLastError();
}

cudaError_t launch_ib_csr(const int16_t *ei, int Mtot, const IbGeom &g, long long Nw, int *cnt, int *start,
                          int *fillc, int *list, cudaStream_t st) {
    long long E = (long long)Mtot * 64;
    cudaError_t e;
    if ((e = cudaMemsetAsync(cnt, 0, sizeof(int) * Nw, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(fillc, 0, sizeof(int) * Nw, st)) != cudaSuccess) return e;
    if (E == 0) return cudaMemsetAsync(start, 0, sizeof(int) * (Nw + 1), st);
    k_ib_count<<<(unsigned)((E + 255) / 256), 256, 0, st>>>(ei, E, g, cnt);
    k_scan<<<1, 1024, 0, st>>>(cnt, start, Nw);
    k_ib_fill<<<(unsigned)((E + 255) / 256), 256, 0, st>>>(ei, E, g, start, fillc, list);
    k_ib_sort<<<(unsigned)((Nw + 255) / 256), 256, 0, st>>>(start, list, Nw);
    return cudaGetLastError();
}

cudaError_t launch_ib_interp(const int16_t *ei, const float *ew, const double *vel, const double *area,
                             const double *wu, const IbGeom &g, int m0, int m1, double invh3, double *eforce,
                             double *fet, double *tolm, cudaStream_t st) {
    int n = m1 - m0;
    if (n <= 0) return cudaSuccess;
    long long Nw = (long long)(g.wx1 - g.wx0 + 1) * g.WY * g.WZ;
    k_ib_interp<<<(n + 63) / 64, 64, 0, st>>>(ei, ew, vel, area, wu, g, Nw, m0, m1, invh3, eforce, fet, tolm);
    return cudaGetLastError();
}

cudaError_t launch_ib_reduce(const double *tolm, int m0, int m1, double *out, cudaStream_t st) {
    k_ib_reduce<<<1, 256, 0, st>>>(tolm, m0, m1, out);
    return cudaGetLastError();
}

cudaError_t launch_ib_correct(const float *ew, const int *start, const int *list, long long Nw, int m0, int m1,
                              const double *fet, double *wu, cudaStream_t st) {
    if (Nw <= 0) return cudaSuccess;
    k_ib_correct<<<(unsigned)((Nw + 127) / 128), 128, 0, st>>>(ew, start, list, Nw, m0, m1, fet, wu);
    return cudaGetLastError();
}

cudaError_t launch_ib_spread(const float *ew, const int *start, const int *list, long long Nw, const double *eforce,
                             double invh3, const double vf[3], double *wforce, cudaStream_t st) {
    if (Nw <= 0) return cudaSuccess;
    k_ib_spread<<<(unsigned)((Nw + 127) / 128), 128, 0, st>>>(ew, start, list, Nw, eforce, invh3, vf[0], vf[1],
                                                               vf[2], wforce);
    return cudaGetLastError();
}

cudaError_t launch_pack_flow(const double *den, const double *u, int X, int Y, int Z, int off, double denIn,
                             double Uref, float *out, cudaStream_t st) {
    const long long n = (long long)(Z - 2 * off) * (Y - 2 * off) * (X - 2 * off);
    if (n <= 0) return cudaSuccess;
    k_pack_flow<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(den, u, (long long)X * Y * Z, X, Y, Z, off, denIn,
                                                             1.0 / Uref, out);
    return cudaGetLastError();
}

cudaError_t launch_flux(const double *den, const double *u, int X, int Y, int Z, double dh, double *flux,
                        cudaStream_t st) {
    k_flux<<<1, 32, 0, st>>>(den, u, (long long)X * Y * Z, X, Y, Z, dh, flux);
    return cudaGetLastError();
}

cudaError_t launch_probes(const double *u, int X, int Y, int Z, double dh, double xmin, double ymin, double zmin, int n,
                          const double *xyz, double Uref, double *out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_probes<<<(3 * n + 127) / 128, 128, 0, st>>>(u, (long long)X * Y * Z, X, Y, Z, dh, xmin, ymin, zmin, n, xyz,
                                                  1.0 / Uref, out);
    return cudaGetLastError();
}

#define FSI_PAIR_DISPATCH(prec, ...)                                                      \
    switch (prec) {                                                                       \
    case FSI_PREC_F64: { constexpr int PP = FSI_PREC_F64; __VA_ARGS__; } break;           \
    case FSI_PREC_F64_FAST: { constexpr int PP = FSI_PREC_F64_FAST; __VA_ARGS__; } break; \
    case FSI_PREC_F32: { constexpr int PP = FSI_PREC_F32; __VA_ARGS__; } break;           \
    case FSI_PREC_F16: { constexpr int PP = FSI_PREC_F16; __VA_ARGS__; } break;           \
    case FSI_PREC_BF16: { constexpr int PP = FSI_PREC_BF16; __VA_ARGS__; } break;         \
    default: return cudaErrorInvalidValue;                                                \
    }

cudaError_t launch_pair_extract(const void *ff, int prec, int FX, int FY, int FZ, TauSrc tf, const PairGeom &p,
                                int face, double *buf, double *buft, int *err, cudaStream_t st) {
    int ax = face >> 1, A, B;
    if (ax == 0) { A = p.zDimF; B = p.yDimF; }
    else if (ax == 1) { A = p.zDimF; B = p.xDimF; }
    else { A = p.yDimF; B = p.xDimF; }
    FSI_PAIR_DISPATCH(prec, k_pair_extract<PP><<<dim3((A + 63) / 64, B), 64, 0, st>>>(
                                ff, FY, FZ, (long long)FX * FY * FZ, tf, p, face, buf, buft, A, B, err))
    return cudaGetLastError();
}

cudaError_t launch_regrid_f64(double *f, int X, int Y, int Z, double dh, double xmin, double ymin, double zmin,
                              const RegridSrc *src, int nsrc, int *err, cudaStream_t st) {
    int bz;
    dim3 g = zgrid(Z, Y, X, bz);
    k_regrid<<<g, bz, 0, st>>>(f, X, Y, Z, dh, xmin, ymin, zmin, src, nsrc, err);
    return cudaGetLastError();
}

cudaError_t launch_fill_f64(double *p, long long n, double v, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_fill<double><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p, n, v);
    return cudaGetLastError();
}

cudaError_t launch_fill_f32(float *p, long long n, float v, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_fill<float><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p, n, v);
    return cudaGetLastError();
}

cudaError_t launch_pair_average(double *b1, const double *b2, long long n, cudaStream_t st) {
    k_pair_average<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(b1, b2, n);
    return cudaGetLastError();
}

cudaError_t launch_pair_f2s(void *fs, int prec, int SX, int SY, int SZ, TauSrc ts, const PairGeom &p, int face,
                            const double *buf, const double *buft, int scheme, double *scratch_f, double *scratch_t,
                            long long scratch_cells, const double vf[3], double dh, int *err, cudaStream_t st) {
    int ax = face >> 1, AF, BF, AS, BS;
    if (ax == 0) { AF = p.zDimF; BF = p.yDimF; AS = p.zDimS; BS = p.yDimS; }
    else if (ax == 1) { AF = p.zDimF; BF = p.xDimF; AS = p.zDimS; BS = p.xDimS; }
    else { AF = p.yDimF; BF = p.xDimF; AS = p.yDimS; BS = p.xDimS; }
    const long long nF = (long long)AF * BF;
    // the interpolation is bounded by this face's own cells, not by the
    // scratch's capacity: a read past the face is reported, never served from
    // what an earlier (larger) face left in the scratch
    const long long nS = (long long)AS * BS;
    if (nS > scratch_cells) return cudaErrorInvalidValue;
    k_pair_interp<<<1, 32, 0, st>>>(Q, AF, buf, Q * nF, AS, BS, scratch_f, Q * nS, scheme, err);
    k_pair_interp<<<1, 32, 0, st>>>(1, AF, buft, nF, AS, BS, scratch_t, nS, 1, err);
    FSI_PAIR_DISPATCH(prec, k_pair_f2s_apply<PP><<<dim3((AS + 63) / 64, BS), 64, 0, st>>>(
                                fs, SY, SZ, (long long)SX * SY * SZ, ts, p, face, scratch_f, scratch_t, AS, BS, vf[0],
                                vf[1], vf[2], dh, err))
    return cudaGetLastError();
}

cudaError_t launch_pair_s2f(void *ff, int prec, int FX, int FY, int FZ, TauSrc tf, const void *fs, int SX, int SY,
                            int SZ, TauSrc ts, const PairGeom &p, int face, const double vf[3], double dh, int *err,
                            cudaStream_t st) {
    int ax = face >> 1;
    int o1 = (ax == 0) ? 1 : 0, o2 = (ax == 2) ? 1 : 2;
    // Fortran DO trip count of si(lo),si(hi),2: zero when hi < lo
    int n1 = (p.si[2 * o1 + 1] >= p.si[2 * o1]) ? (p.si[2 * o1 + 1] - p.si[2 * o1]) / 2 + 1 : 0;
    int n2 = (p.si[2 * o2 + 1] >= p.si[2 * o2]) ? (p.si[2 * o2 + 1] - p.si[2 * o2]) / 2 + 1 : 0;
    if (n1 <= 0 || n2 <= 0) return cudaSuccess;
    FSI_PAIR_DISPATCH(prec, k_pair_s2f<PP><<<dim3((n2 + 63) / 64, n1), 64, 0, st>>>(
                                ff, FY, FZ, (long long)FX * FY * FZ, tf, fs, SY, SZ, (long long)SX * SY * SZ, ts, p, face,
                                n1, n2, vf[0], vf[1], vf[2], dh, err))
    return cudaGetLastError();
}

}  // namespace fsi
