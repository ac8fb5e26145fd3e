// fast_route.cu -- the public launchers of the throughput forms.
//
// k_fast.cu is compiled once per storage form into namespace fsi::fast_p<form>
// (fsi_kernels.h, FSI_FAST_API); each name below forwards a call to the unit
// of its `prec` and refuses any other form the way the units do
// (cudaErrorInvalidValue, 0 or false).
#include "fsi_kernels.h"
#include "../../include/fsi_gpu.h"

namespace fsi {

#define FSI_ROUTE(prec, refused, CALL)                 \
    switch (prec) {                                    \
    case FSI_PREC_F64_FAST: return fast_p1::CALL;      \
    case FSI_PREC_F32: return fast_p2::CALL;           \
    case FSI_PREC_F16: return fast_p3::CALL;           \
    case FSI_PREC_BF16: return fast_p4::CALL;          \
    default: return refused;                           \
    }

// the bulk step also serves the double-word form, whose blocks otherwise run
// on the FP64 units (the host passes FSI_PREC_F64_DW to these two only)
#define FSI_ROUTE_STEP(prec, refused, CALL)            \
    switch (prec) {                                    \
    case FSI_PREC_F64_FAST: return fast_p1::CALL;      \
    case FSI_PREC_F32: return fast_p2::CALL;           \
    case FSI_PREC_F16: return fast_p3::CALL;           \
    case FSI_PREC_BF16: return fast_p4::CALL;          \
    case FSI_PREC_F64_DW: return fast_p5::CALL;        \
    default: return refused;                           \
    }

bool step_fast_paired(const StepArgs &a, const MrtMats *mm, int prec, int model) {
    FSI_ROUTE_STEP(prec, false, step_fast_paired(a, mm, prec, model))
}

cudaError_t launch_step_fast(const StepArgs &a, const MrtMats *mm, int prec, int model, cudaStream_t st) {
    FSI_ROUTE_STEP(prec, cudaErrorInvalidValue, launch_step_fast(a, mm, prec, model, st))
}

cudaError_t launch_step_macro_fast(const StepArgs &a, int prec, cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_step_macro_fast(a, prec, st))
}

cudaError_t launch_bc_fast(const BcArgs &a, int prec, cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_bc_fast(a, prec, st))
}

cudaError_t launch_bc_pair_fast(const BcArgs &lo, const BcArgs &hi, int prec, cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_bc_pair_fast(lo, hi, prec, st))
}

cudaError_t launch_convert_to_store(const double *f64, void *fs, long long N, int prec, cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_convert_to_store(f64, fs, N, prec, st))
}

cudaError_t launch_convert_from_store(const void *fs, double *f64, long long N, int prec, cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_convert_from_store(fs, f64, N, prec, st))
}

cudaError_t launch_macro_fast(const void *fs, int prec, double *den, double *u, int X, int Y, int Z, double dh,
                              const double vf[3], cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_macro_fast(fs, prec, den, u, X, Y, Z, dh, vf, st))
}

cudaError_t launch_win_macro_fast(const void *fs, int prec, double *wden, double *wu, const IbGeom &g, long long N,
                                  const double vf[3], cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_win_macro_fast(fs, prec, wden, wu, g, N, vf, st))
}

cudaError_t launch_ib_coop(const IbCoop &a, int prec, int grid, cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_ib_coop(a, prec, grid, st))
}

cudaError_t launch_ib_cluster(const IbCoop &a, int prec, cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_ib_cluster(a, prec, st))
}

int ib_coop_grid(int prec) { FSI_ROUTE(prec, 0, ib_coop_grid(prec)) }

cudaError_t launch_batch_step(const BatchCase *d_cases, const int *d_gcase, int n, int G, int threads, long long wmax,
                              int prec, int model, bool forced, cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue,
              launch_batch_step(d_cases, d_gcase, n, G, threads, wmax, prec, model, forced, st))
}

cudaError_t launch_batch_winfix(const BatchCase *d_cases, int n, long long wmax, int prec, int model, cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_batch_winfix(d_cases, n, wmax, prec, model, st))
}

cudaError_t launch_batch_bc(const BcArgs *d_bcs, int n, int face, int Amax, int Bmax, int prec, cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_batch_bc(d_bcs, n, face, Amax, Bmax, prec, st))
}

cudaError_t launch_batch_ib(const IbCoop *d_ib, int n, int threads, int prec, cudaStream_t st) {
    FSI_ROUTE(prec, cudaErrorInvalidValue, launch_batch_ib(d_ib, n, threads, prec, st))
}

}  // namespace fsi
