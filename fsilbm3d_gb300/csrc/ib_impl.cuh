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

// the same Phi with both branches' operands formed and one square root: the
// same operations on the same operands (so the same value), without the
// divergent second square root when the lanes of a warp fall in different
// branches
__device__ __forceinline__ double ib_phi4_sel(double x) {
    const double r = fabs(x);
    const bool near = r < 1.0;
    const double a = near ? __dsub_rn(3.0, __dmul_rn(2.0, r)) : __dsub_rn(5.0, __dmul_rn(2.0, r));
    const double q = near ? __dadd_rn(1.0, __dmul_rn(__dmul_rn(4.0, r), __dsub_rn(1.0, r)))
                          : __dadd_rn(-7.0, __dmul_rn(__dmul_rn(4.0, r), __dsub_rn(3.0, r)));
    const double sq = __dsqrt_rn(near || r < 2.0 ? q : 0.0);
    const double v = near ? __dadd_rn(a, sq) : __dsub_rn(a, sq);
    return r < 2.0 ? __dmul_rn(v, 0.125) : 0.0;
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
    const double invdh = g.invdh;
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

// The same stencil (the same operations, so the same indices and weights)
// formed by the 8 lanes of a group that serves one marker, one FP64 code path
// per group instead of one per marker: lanes 0-2 form the base index and the
// offset of axes 0-2, lanes 0-7 the weights of axes 0 and 1, lanes 0-3 those
// of axis 2; every lane of the group gets all 12. All 32 lanes of the warp
// call it (act false: a group without a marker).
__device__ __forceinline__ int ib_stencil_group(const double *p0, const double *p, const IbGeom &g, int gl, bool act,
                                                int e[12], float w[12]) {
    constexpr unsigned FULL = 0xffffffffu;
    int ib = 0;
    double det = 0.0;
    if (act && gl < 3) {
        const double mn = gl == 0 ? g.xmin : (gl == 1 ? g.ymin : g.zmin);
        int i0 = (int)floor(__dmul_rn(__dsub_rn(p0[gl], mn), g.invdh));
        const double x0 = __dadd_rn(mn, __dmul_rn((double)i0, g.dh));
        i0 = i0 + 1;
        const double o = __dmul_rn(__dsub_rn(p[gl], x0), g.invdh);
        const int i = (int)floor(o);
        det = __dsub_rn(o, (double)i);
        ib = i + i0;
    }
    int ia[3];
    double da[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        ia[a] = __shfl_sync(FULL, ib, a, 8);
        da[a] = __shfl_sync(FULL, det, a, 8);
    }
    int idx[3][4];
    int st = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int dim = a == 0 ? g.X : (a == 1 ? g.Y : g.Z);
        if (!ib_trimed(ia[a], dim, idx[a], g.bc[2 * a], g.bc[2 * a + 1])) st |= 1;
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
        for (int t = 0; t < 4; t++) e[4 * a + t] = inwin ? idx[a][t] : lo[a] + 1;
    float wa = 0.0f, wb = 0.0f;
    if (act) wa = (float)ib_phi4_sel(__dsub_rn((double)((gl & 3) - 1), (gl >> 2) ? da[1] : da[0]));
    if (act && gl < 4) wb = (float)ib_phi4_sel(__dsub_rn((double)(gl - 1), da[2]));
#pragma unroll
    for (int k = 0; k < 8; k++) w[k] = __shfl_sync(FULL, wa, k, 8);
#pragma unroll
    for (int k = 0; k < 4; k++) w[8 + k] = __shfl_sync(FULL, wb, k, 8);
    return act ? st : 0;
}

}  // namespace
}  // namespace fsi
