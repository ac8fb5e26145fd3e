// ib_impl.cuh -- the immersed-boundary stencil of one marker
// (UpdateElmtInterp_, Solidbody.f90:760-867), shared by the exact and the
// fast translation units. Every floating-point operation is an explicit
// round-to-nearest intrinsic, so both units produce the same int16 indices and
// FP32 weights whatever their contraction flags.
#pragma once
#include "fsi_kernels.h"

namespace fsi {
namespace {

// Phi, Solidbody.f90:822-833
__device__ __forceinline__ double ib_phi4(double x) {
    const double r = fabs(x);
    if (r < 1.0)
        return __dmul_rn(__dadd_rn(__dsub_rn(3.0, __dmul_rn(2.0, r)),
                                   __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(__dmul_rn(4.0, r), __dsub_rn(1.0, r))))),
                         0.125);
    if (r < 2.0)
        return __dmul_rn(__dsub_rn(__dsub_rn(5.0, __dmul_rn(2.0, r)),
                                   __dsqrt_rn(__dadd_rn(-7.0, __dmul_rn(__dmul_rn(4.0, r), __dsub_rn(3.0, r))))),
                         0.125);
    return 0.0;
}

// trimedindex, Solidbody.f90:834-866 (1-based); false if out of range
__device__ __forceinline__ bool ib_trimed(int i, int dim, int out[4], int lo, int hi) {
    bool ok = true;
#pragma unroll
    for (int k = -1; k <= 2; k++) {
        int v = i + k;
        if (v < 1) {
            if (lo == BC_PERIODIC) v = v + dim;
            else if ((lo == BC_SYMMETRIC || lo == BC_WALL) && v == 0) v = 2;
            else if (lo == BC_WALL_HW && v == 0) v = 1;
            else { ok = false; v = 1; }
        } else if (v > dim) {
            if (hi == BC_PERIODIC) v = v - dim;
            else if ((hi == BC_SYMMETRIC || hi == BC_WALL) && v == dim + 1) v = dim - 1;
            else if (hi == BC_WALL_HW && v == dim + 1) v = dim;
            else { ok = false; v = dim; }
        }
        out[k + 1] = v;
    }
    return ok;
}

// stencil of marker p with the origin rule of the body whose first marker is
// p0 (Solidbody.f90:771-804); writes 12 indices and 12 weights. Returns a
// status: bit 0 index outside the block, bit 1 outside the IB window
// (indices are then clamped into the window).
__device__ __forceinline__ int ib_stencil_one(const double *p0, const double *p, const IbGeom &g, int16_t *e,
                                              float *w) {
    const double invdh = __ddiv_rn(1.0, g.dh);
    const double mins[3] = {g.xmin, g.ymin, g.zmin};
    int idx[3][4];
    double det[3];
    int st = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        int i0 = (int)floor(__dmul_rn(__dsub_rn(p0[a], mins[a]), invdh));
        const double x0 = __dadd_rn(mins[a], __dmul_rn((double)i0, g.dh));
        i0 = i0 + 1;
        const double o = __dmul_rn(__dsub_rn(p[a], x0), invdh);
        int i = (int)floor(o);
        det[a] = __dsub_rn(o, (double)i);
        i += i0;
        const int dim = a == 0 ? g.X : (a == 1 ? g.Y : g.Z);
        if (!ib_trimed(i, dim, idx[a], g.bc[2 * a], g.bc[2 * a + 1])) st |= 1;
    }
    const int lo[3] = {g.wx0, g.wy0, g.wz0}, hi[3] = {g.wx1, g.wy1, g.wz1};
    bool inwin = true;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int t = 0; t < 4; t++) inwin = inwin && (idx[a][t] - 1 >= lo[a]) && (idx[a][t] - 1 <= hi[a]);
    if (!inwin) st |= 2;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int t = 0; t < 4; t++) {
            e[4 * a + t] = (int16_t)(inwin ? idx[a][t] : lo[a] + 1);
            w[4 * a + t] = (float)ib_phi4(__dsub_rn((double)(t - 1), det[a]));
        }
    return st;
}

}  // namespace
}  // namespace fsi
