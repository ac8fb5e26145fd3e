// bc_impl.cuh -- device code of the face boundary conditions and the
// equilibrium helpers, shared by the exact and the fast translation units.
// Storage access goes through an accessor ACC with
//   static double load(const void *f, long long idx, int q)
//   static void   store(void *f, long long idx, int q, double v)
// that converts between the stored form and the FP64 distribution value.
#pragma once
#include "fsi_common.cuh"

namespace fsi {
// internal linkage: each translation unit compiles its own copy with its
// own floating-point flags
namespace {

__device__ __forceinline__ long long bc_cidx(int z, int y, int x, int Z, int Y) {
    return (long long)z + (long long)Z * ((long long)y + (long long)Y * (long long)x);
}

// FP64 storage, the distribution itself
struct AccF64 {
    static __device__ __forceinline__ double load(const void *f, long long i, int q) { return ((const double *)f)[i]; (void)q; }
    static __device__ __forceinline__ void store(void *f, long long i, int q, double v) { ((double *)f)[i] = v; (void)q; }
};

// evaluate_velocity, FluidDomain.f90:1791-1824
__device__ __forceinline__ void eval_vel(const Vel &v, double zc, double yc, double xc, double out[3]) {
    if (v.kind == 0) {
        out[0] = ((v.vin[0] + 0.0 * v.sr[0]) + yc * v.sr[1]) + zc * v.sr[2];
        out[1] = ((v.vin[1] + xc * v.sr[0]) + 0.0 * v.sr[1]) + zc * v.sr[2];
        out[2] = ((v.vin[2] + xc * v.sr[0]) + yc * v.sr[1]) + 0.0 * v.sr[2];
    } else {
        out[0] = v.osc[0];
        out[1] = v.osc[1];
        out[2] = v.osc[2];
    }
}

// calculate_distribution_funcion, FluidDomain.f90:1827-1834
__device__ __forceinline__ double feq_dist(int i, double density, const double v[3], double uSqr) {
    double uxyz = (v[0] * (double)ex_(i) + v[1] * (double)ey_(i)) + v[2] * (double)ez_(i);
    return (wt_(i) * density) * ((((1.0 + 3.0 * uxyz) + (4.5 * uxyz) * uxyz) - 1.5 * uSqr));
}

// -------------------------------------------------------- boundary faces
// set_boundary_conditions_ for one face, FluidDomain.f90:616-1126. One thread
// per face cell; faces run one launch after another in the reference order.
__device__ __forceinline__ long long face_cell(const BcArgs &a, int fa, int fb, int l) {
    const int ax = a.face >> 1, side = a.face & 1;
    if (ax == 0) return bc_cidx(fa, fb, side ? a.X - 1 - l : l, a.Z, a.Y);
    if (ax == 1) return bc_cidx(fa, side ? a.Y - 1 - l : l, fb, a.Z, a.Y);
    return bc_cidx(side ? a.Z - 1 - l : l, fa, fb, a.Z, a.Y);
}

__device__ __forceinline__ void face_vel(const BcArgs &a, int fa, int fb, bool half, double v[3]) {
    const int ax = a.face >> 1, side = a.face & 1;
    double xc, yc, zc;
    if (ax == 0) {
        zc = a.zmin + a.dh * (double)fa; yc = a.ymin + a.dh * (double)fb;
        xc = side ? (half ? a.xmax + a.dh * 0.5 : a.xmax) : (half ? a.xmin - a.dh * 0.5 : a.xmin);
    } else if (ax == 1) {
        zc = a.zmin + a.dh * (double)fa; xc = a.xmin + a.dh * (double)fb;
        yc = side ? (half ? a.ymax + a.dh * 0.5 : a.ymax) : (half ? a.ymin - a.dh * 0.5 : a.ymin);
    } else {
        yc = a.ymin + a.dh * (double)fa; xc = a.xmin + a.dh * (double)fb;
        zc = side ? (half ? a.zmax + a.dh * 0.5 : a.zmax) : (half ? a.zmin - a.dh * 0.5 : a.zmin);
    }
    eval_vel(a.vel, zc, yc, xc, v);
}

template <class ACC, int FACE>
__device__ __forceinline__ void bc_apply(const BcArgs &a, int fa, int fb) {
    void *f = a.f;
    const long long N = a.N;
    const long long c1 = face_cell(a, fa, fb, 0);
    switch (a.code) {
    case BC_EQ: {
        double v[3];
        face_vel(a, fa, fb, false, v);
        double uSqr = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
#pragma unroll
        for (int i = 0; i < Q; i++) ACC::store(f, c1 + N * (i), i, feq_dist(i, a.denIn, v, uSqr));
    } break;
    case BC_NEQ: {
        const long long c2 = face_cell(a, fa, fb, 1);
        double v[3], u2[3];
        face_vel(a, fa, fb, false, v);
        double uSqr = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
        u2[0] = a.u[c2]; u2[1] = a.u[c2 + N]; u2[2] = a.u[c2 + 2 * N];
        double d2 = a.den[c2];
        double uSqr2 = (u2[0] * u2[0] + u2[1] * u2[1]) + u2[2] * u2[2];
#pragma unroll
        for (int j = 0; j < 5; j++) {
            const int q = inc_(FACE, j);
            ACC::store(f, c1 + N * (q), q, feq_dist(q, a.denIn, v, uSqr) + (ACC::load(f, c2 + N * (q), q) - feq_dist(q, d2, u2, uSqr2)));
        }
    } break;
    case BC_EXT1: {
        const long long c2 = face_cell(a, fa, fb, 1);
#pragma unroll
        for (int j = 0; j < 5; j++) { const int q = inc_(FACE, j); ACC::store(f, c1 + N * (q), q, ACC::load(f, c2 + N * (q), q)); }
    } break;
    case BC_EXT2: {
        const long long c2 = face_cell(a, fa, fb, 1), c3 = face_cell(a, fa, fb, 2);
#pragma unroll
        for (int j = 0; j < 5; j++) {
            const int q = inc_(FACE, j);
            ACC::store(f, c1 + N * (q), q, 2.0 * ACC::load(f, c2 + N * (q), q) - ACC::load(f, c3 + N * (q), q));
        }
    } break;
    case BC_WALL: {
        double t[5];
#pragma unroll
        for (int j = 0; j < 5; j++) t[j] = ACC::load(f, c1 + N * (opp_(inc_(FACE, j))), opp_(inc_(FACE, j)));
#pragma unroll
        for (int j = 0; j < 5; j++) ACC::store(f, c1 + N * (inc_(FACE, j)), inc_(FACE, j), t[j]);
    } break;
    case BC_WALL_HW: {
        const double *h = a.hw + (long long)Q * ((long long)fa + (long long)(FACE < 2 ? a.Z : (FACE < 4 ? a.Z : a.Y)) * fb);
#pragma unroll
        for (int j = 0; j < 5; j++) ACC::store(f, c1 + N * (inc_(FACE, j)), inc_(FACE, j), h[opp_(inc_(FACE, j))]);
    } break;
    case BC_MWALL:
    case BC_MWALL_HW: {
        const bool half = (a.code == BC_MWALL_HW);
        double v[3];
        face_vel(a, fa, fb, half, v);
        const double *h = a.hw + (long long)Q * ((long long)fa + (long long)(FACE < 2 ? a.Z : (FACE < 4 ? a.Z : a.Y)) * fb);
        double t[5];
#pragma unroll
        for (int j = 0; j < 5; j++) {
            const int q = inc_(FACE, j);
            double uxyz = (v[0] * (double)ex_(q) + v[1] * (double)ey_(q)) + v[2] * (double)ez_(q);
            double din = half ? h[opp_(q)] : ACC::load(f, c1 + N * (opp_(q)), opp_(q));
            t[j] = din + (((2.0 * wt_(q)) * a.denIn) * uxyz) * 3.0;
        }
#pragma unroll
        for (int j = 0; j < 5; j++) ACC::store(f, c1 + N * (inc_(FACE, j)), inc_(FACE, j), t[j]);
    } break;
    case BC_SYMMETRIC: {
        double t[5];
#pragma unroll
        for (int j = 0; j < 5; j++) t[j] = ACC::load(f, c1 + N * (mir_(FACE, j)), mir_(FACE, j));
#pragma unroll
        for (int j = 0; j < 5; j++) ACC::store(f, c1 + N * (inc_(FACE, j)), inc_(FACE, j), t[j]);
    } break;
    default:
        break;
    }
}

template <class ACC, int FACE>
__global__ void k_bc(BcArgs a) {
    const int A = (FACE < 4) ? a.Z : a.Y;
    const int B = (FACE < 2) ? a.Y : a.X;
    int fa = blockIdx.x * blockDim.x + threadIdx.x;
    int fb = blockIdx.y * blockDim.y + threadIdx.y;
    if (fa >= A || fb >= B) return;
    if (FACE < 4 && (fa < a.zlo || fa > a.zhi)) return;
    bc_apply<ACC, FACE>(a, fa, fb);
}

}  // namespace
}  // namespace fsi
