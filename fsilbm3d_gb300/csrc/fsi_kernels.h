// fsi_kernels.h -- host-side launchers of the CUDA kernels of libfsi_gpu.
// Each launcher enqueues on `st` and returns the launch status.
#pragma once
#include "fsi_common.cuh"
#include "store_acc.cuh"

namespace fsi {

// ---- exact FP64 translation unit (k_f64_exact.cu, built with -fmad=false) ----
cudaError_t launch_init_f64(double *f, double *den, double *u, int X, int Y, int Z,
                            double dh, double xmin, double ymin, double zmin,
                            double denIn, const Vel &vel, double blktime, cudaStream_t st);
cudaError_t launch_macro_f64(const double *f, double *den, double *u, int X, int Y, int Z,
                             double dh, const double vf[3], cudaStream_t st);
cudaError_t launch_step_f64_exact(const StepArgs &a, const MrtMats *mm, int model, cudaStream_t st);
// den/u of every cell as the collision sees them (IB window cells from the IB
// stage), written to a.den/a.u before the step of a model that reads its
// neighbours' velocity (grad_model)
cudaError_t launch_step_macro_f64(const StepArgs &a, cudaStream_t st);
cudaError_t launch_bc_f64(const BcArgs &a, cudaStream_t st);
cudaError_t launch_halfway_f64(const double *f, double *hw, int X, int Y, int Z, int face,
                               cudaStream_t st);

// IB (exact order)
struct IbGeom {
    int X, Y, Z;
    double dh, xmin, ymin, zmin;
    double invdh;  // 1 / dh, correctly rounded (formed on the host)
    int bc[6];
    int wx0, wx1, wy0, wy1, wz0, wz1, WY, WZ;
};
cudaError_t launch_win_macro_f64(const void *f, int prec, double *wden, double *wu,
                                 const IbGeom &g, long long N, const double vf[3], cudaStream_t st);
cudaError_t launch_ib_stencil(const double *xyz, const int *offs, int nb, int Mtot, const IbGeom &g,
                              int16_t *ei, float *ew, int *err, cudaStream_t st);
cudaError_t launch_ib_csr(const int16_t *ei, int Mtot, const IbGeom &g, long long Nw,
                          int *cnt, int *start, int *fillc, int *list, cudaStream_t st);
cudaError_t launch_ib_interp(const int16_t *ei, const float *ew, const double *vel, const double *area,
                             const double *wu, const IbGeom &g, int m0, int m1, double invh3,
                             double *eforce, double *fet, double *tolm, cudaStream_t st);
cudaError_t launch_ib_reduce(const double *tolm, int m0, int m1, double *out, cudaStream_t st);
cudaError_t launch_ib_correct(const float *ew, const int *start, const int *list, long long Nw,
                              int m0, int m1, const double *fet, double *wu, cudaStream_t st);
cudaError_t launch_ib_spread(const float *ew, const int *start, const int *list, long long Nw,
                             const double *eforce, double invh3, const double vf[3],
                             double *wforce, cudaStream_t st);

// One persistent cooperative launch for the whole IB solve of the fast forms
// (k_fast.cu): window macro, stencil, the penalty loop with its residual test
// on the device, spreading. status[0]: 1 stencil outside the block, 2 outside
// the window, 4 non-finite residual, 8 a grid barrier timed out;
// status[1]: iterations; status[2..3]: barrier count and generation.
struct IbCoop {
    IbGeom g;
    long long N, Nw;
    const void *f;
    double vf[3];
    int nb, Mtot;
    const int *offs;
    const double *xyz, *vel, *area;
    int16_t *ei;
    float *ew;
    // per marker and stencil point (64 each): window cell and weight product
    // rx ry rz, formed once per solve with the stencil
    int *c64;
    double *w64;
    double *eforce, *fet;
    double *wden, *wu, *wforce;
    // the fast forms' penalty loop: the second window-velocity buffer (3 Nw)
    // and three slots of velocity corrections (9 Nw)
    double *wu2, *dlt;
    int ntol;
    double dtol, dsumU, invh3p, invh3s;
    double *tol_acc;  // ntol sums
    int *status;
    double *res;
    // learned warm start (all null: the reference's loop alone)
    const float *mlp, *mlp_nrm;  // perceptron parameters and statistics, or null
    const double *aux;           // (6,Mtot): acceleration, normal; or null
    float *feat;                 // (12,Mtot) features out, or null
    double Uref;
    int seed;                    // 1: eforce holds the caller's initial force
    unsigned bar_base;           // the grid barrier's arrival counter (status[2]) at launch
};

// ---- output packing (k_f64_exact.cu, reference operation order) ----
cudaError_t launch_pack_flow(const double *den, const double *u, int X, int Y, int Z, int off, double denIn,
                             double Uref, float *out, cudaStream_t st);
cudaError_t launch_flux(const double *den, const double *u, int X, int Y, int Z, double dh, double *flux,
                        cudaStream_t st);
cudaError_t launch_probes(const double *u, int X, int Y, int Z, double dh, double xmin, double ymin, double zmin, int n,
                          const double *xyz, double Uref, double *out, cudaStream_t st);

// ---- continue-file re-grid (k_f64_exact.cu, check_is_continue,
// FluidDomain.f90:170-226): one file block, its upper corner precomputed ----
struct RegridSrc {
    double xmin, ymin, zmin, dh, xmx, ymx, zmx;
    int X, Y, Z;
    const double *f;  // fIn(z,y,x,0:18) on the device
};
// fIn (FP64, N = X*Y*Z cells) of a block at (xmin, ymin, zmin) with spacing dh
// from the file blocks src[0..nsrc) in search order; err: first bad index
cudaError_t launch_regrid_f64(double *f, int X, int Y, int Z, double dh, double xmin, double ymin, double zmin,
                              const RegridSrc *src, int nsrc, int *err, cudaStream_t st);

// ---- block refinement (k_f64_exact.cu) ----
struct PairGeom {
    int sds[6], s[6], f[6], si[6], fi[6];
    int xDimS, xDimF, yDimS, yDimF, zDimS, zDimF;
};
// the face exchange of block refinement on any storage form `prec` (father
// and son alike); tau per cell from TauSrc (store_acc.cuh)
cudaError_t launch_pair_extract(const void *ff, int prec, int FX, int FY, int FZ, TauSrc tf, const PairGeom &p,
                                int face, double *buf, double *buft, int *err, cudaStream_t st);
cudaError_t launch_pair_average(double *b1, const double *b2, long long n, cudaStream_t st);
cudaError_t launch_fill_f64(double *p, long long n, double v, cudaStream_t st);
cudaError_t launch_fill_f32(float *p, long long n, float v, cudaStream_t st);
cudaError_t launch_pair_f2s(void *fs, int prec, int SX, int SY, int SZ, TauSrc ts, const PairGeom &p, int face,
                            const double *buf, const double *buft, int scheme, double *scratch_f, double *scratch_t,
                            long long scratch_cells, const double vf[3], double dh, int *err, cudaStream_t st);
cudaError_t launch_pair_s2f(void *ff, int prec, int FX, int FY, int FZ, TauSrc tf, const void *fs, int SX, int SY,
                            int SZ, TauSrc ts, const PairGeom &p, int face, const double vf[3], double dh, int *err,
                            cudaStream_t st);

// ---- the throughput forms (k_fast.cu, built once per storage form) ----
// Many blocks stepped together (offset forms, paired kernels): one entry per
// block with its step arguments (src/dst of this step, window, z faces), the
// MRT rates S_k/|row k|^2, and its row groups: tpr = zDim/2 pairs per z-row,
// R rows per group, ngy groups per x-plane, g0 = first global group.
struct BatchCase {
    StepArgs a;
    float sd[19];
    int tpr, R, ngy, g0;
};
// thread counts the batched bulk kernel is built for (the autotuner's choices)
constexpr int BATCH_THREADS[3] = {256, 512, 128};

// Every launcher of k_fast.cu takes the storage form `prec` and returns
// cudaErrorInvalidValue (0 / false for the two queries) for a form it does not
// serve. k_fast.cu is compiled once per form (FSI_PREC_F64_FAST, F32, F16,
// BF16) into namespace fast_p<prec>; fast_route.cu defines the names below in
// namespace fsi and forwards each call to the unit of its form.
//
//  step_fast_paired        true when launch_step_fast runs the paired kernels
//                          (which can write 101 z faces)
//  launch_step_fast        the fused collide+stream step of one block
//  launch_step_macro_fast  den/u (FP32 `uf`) of every cell as the collision
//                          sees them, then the LES gradient pass (WALE, Vreman)
//  launch_bc_fast          one face
//  launch_bc_pair_fast     both faces of one axis in one launch (offset forms;
//                          faces that share no cell they read or write)
//  launch_convert_to_store / launch_convert_from_store   FP64 <-> storage form
//  launch_macro_fast       den/u of the whole block (output)
//  launch_win_macro_fast   den/u of the IB window
//  launch_ib_coop          the IB solve as one cooperative launch of `grid` CTAs
//  launch_ib_cluster       the same on one thread-block cluster, which may run
//                          beside other kernels (offset forms)
//  ib_coop_grid            co-resident CTAs (256 threads) on this device, 0 on error
//  launch_batch_step       the bulk step of every block (G groups in all,
//                          gcase[j] = block of group j) with CTAs of `threads`;
//                          then the IB-window fix-up of every block (wmax >=
//                          each block's window cells)
//  launch_batch_winfix     the IB-window fix-up alone (after the bulk step and
//                          the IB stage)
//  launch_batch_bc         face k of every block (bcs: n entries for this face;
//                          code BC_FLUID = none)
//  launch_batch_ib         the IB stage of every block, one CTA per block
#define FSI_FAST_API                                                                                             \
    bool step_fast_paired(const StepArgs &a, const MrtMats *mm, int prec, int model);                           \
    cudaError_t launch_step_fast(const StepArgs &a, const MrtMats *mm, int prec, int model, cudaStream_t st);    \
    cudaError_t launch_step_macro_fast(const StepArgs &a, int prec, cudaStream_t st);                            \
    cudaError_t launch_bc_fast(const BcArgs &a, int prec, cudaStream_t st);                                      \
    cudaError_t launch_bc_pair_fast(const BcArgs &lo, const BcArgs &hi, int prec, cudaStream_t st);              \
    cudaError_t launch_convert_to_store(const double *f64, void *fs, long long N, int prec, cudaStream_t st);    \
    cudaError_t launch_convert_from_store(const void *fs, double *f64, long long N, int prec, cudaStream_t st);  \
    cudaError_t launch_macro_fast(const void *fs, int prec, double *den, double *u, int X, int Y, int Z,         \
                                  double dh, const double vf[3], cudaStream_t st);                               \
    cudaError_t launch_win_macro_fast(const void *fs, int prec, double *wden, double *wu, const IbGeom &g,       \
                                      long long N, const double vf[3], cudaStream_t st);                         \
    cudaError_t launch_ib_coop(const IbCoop &a, int prec, int grid, cudaStream_t st);                            \
    cudaError_t launch_ib_cluster(const IbCoop &a, int prec, cudaStream_t st);                                   \
    int ib_coop_grid(int prec);                                                                                  \
    cudaError_t launch_batch_step(const BatchCase *d_cases, const int *d_gcase, int n, int G, int threads,       \
                                  long long wmax, int prec, int model, bool forced, cudaStream_t st);            \
    cudaError_t launch_batch_winfix(const BatchCase *d_cases, int n, long long wmax, int prec, int model,        \
                                    cudaStream_t st);                                                            \
    cudaError_t launch_batch_bc(const BcArgs *d_bcs, int n, int face, int Amax, int Bmax, int prec,              \
                                cudaStream_t st);                                                                \
    cudaError_t launch_batch_ib(const IbCoop *d_ib, int n, int threads, int prec, cudaStream_t st);

FSI_FAST_API
namespace fast_p1 { FSI_FAST_API }  // FSI_PREC_F64_FAST
namespace fast_p2 { FSI_FAST_API }  // FSI_PREC_F32
namespace fast_p3 { FSI_FAST_API }  // FSI_PREC_F16
namespace fast_p4 { FSI_FAST_API }  // FSI_PREC_BF16
namespace fast_p5 {                   // FSI_PREC_F64_DW: the bulk step only
bool step_fast_paired(const StepArgs &a, const MrtMats *mm, int prec, int model);
cudaError_t launch_step_fast(const StepArgs &a, const MrtMats *mm, int prec, int model, cudaStream_t st);
}

// ---- warm-start perceptron (k_mlp.cu) ----
cudaError_t launch_mlp_forward(const float *P, const float *nrm, const float *X, float *Y, int n, cudaStream_t st);
cudaError_t launch_mlp_grad(const float *P, const float *nrm, const float *X, const float *Y, const int *perm,
                            long long b0, int nb, int batch_total, float *grad, float *loss, cudaStream_t st);
cudaError_t launch_mlp_adam(float *P, float *grad, float *m, float *v, float lr, int step, cudaStream_t st);

}  // namespace fsi
