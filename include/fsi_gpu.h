/*
 * fsi_gpu.h -- C-ABI of the GB300 (sm_103a) implementation of FSILBM3D's
 * per-time-step hot path: D3Q19 collide-stream, face boundary conditions,
 * block-refinement face exchange and immersed-boundary coupling.
 *
 * The reference has no plugin or FFI layer: its hot path is a set of
 * Fortran type-bound procedures called from the tree recursion in
 * LBMBlockComm.f90:279-338. Each entry point below replaces the body of one
 * or more of those procedures; the comment on each names the reference
 * routine (file:line) it stands in for. A Fortran host binds these through
 * an ISO_C_BINDING interface module; any C, C++ or Python (ctypes) host can
 * call them directly.
 *
 * Conventions
 *  - Every function returns FSI_OK (0) or a negative FSI_E_* code; the
 *    message of the last failure on the calling thread is available from
 *    fsi_last_error(). No function calls exit(), abort() or a device trap:
 *    where the reference stops (e.g. Solidbody.f90:1028-1031 on NaN,
 *    FluidDomain.f90:704 on an unknown boundary code) the call returns an
 *    error code and the caller decides.
 *  - Host arrays are plain pointers in the reference's Fortran layout:
 *    fIn(z,y,x,0:18), uuu(z,y,x,1:3), den(z,y,x) column-major, marker arrays
 *    (3,M) column-major. Indices are 0-based in C; the stencil indices
 *    returned by fsi_ib_get_stencil keep the reference's 1-based values.
 *  - Calls are synchronous at the ABI level unless stated otherwise; a
 *    handle is used by one host thread at a time.
 *  - Device memory is owned by the handle; host memory by the caller.
 */
#ifndef FSI_GPU_H
#define FSI_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSI_OK         0
#define FSI_E_ARG     -1   /* invalid argument or unsupported option        */
#define FSI_E_CUDA    -2   /* CUDA runtime error                            */
#define FSI_E_NAN     -3   /* non-finite IB residual (Solidbody.f90:1028)   */
#define FSI_E_TIMEOUT -4   /* a bounded device wait ran out                 */
#define FSI_E_BC      -5   /* unknown boundary code (FluidDomain.f90:704)   */
#define FSI_E_RANGE   -6   /* IB stencil leaves the block (Solidbody.f90:850) */
#define FSI_E_STATE   -7   /* call order violated                           */

/* Storage / arithmetic forms of the distributions. */
#define FSI_PREC_F64       0  /* FP64 storage, FP64 arithmetic in the reference's
                                 operation order (no fused multiply-add): bitwise
                                 equal to an FP64 CPU run of the same order     */
#define FSI_PREC_F64_FAST  1  /* FP64 storage and arithmetic, regrouped with FMA */
#define FSI_PREC_F32       2  /* FP32 storage of f - w_i, FP32 arithmetic        */
#define FSI_PREC_F16       3  /* FP16 storage of f - w_i, FP32 arithmetic        */
#define FSI_PREC_BF16      4  /* BF16 storage of f - w_i, FP32 arithmetic        */
#define FSI_PREC_F64_DW    5  /* FP64 storage; the collide-stream step in double-word
                                 FP32 arithmetic (pairs of FP32 values, about 48
                                 significant bits) on the FP32 pipe; SRT and MRT
                                 (moment form); everything else as FSI_PREC_F64_FAST */

typedef struct fsi_block *fsi_block_t;

/* Parameters of one LBM block: LBMBlock (FluidDomain.f90:17-56), the block
 * section of inFlow.dat (FluidDomain.f90:61-108) and the flow conditions the
 * hot path reads (FlowCondition.f90:11-26). */
typedef struct {
    int    xDim, yDim, zDim;
    double dh, xmin, ymin, zmin;
    int    bndConds[6];      /* x-, x+, y-, y+, z-, z+ codes (ConstParams.f90:31-34) */
    int    iCollidModel;     /* 1 SRT/BGK, 2 TRT, 3 MRT, 11 SRT + Smagorinsky,
                                14 SRT + WALE, 15 SRT + Vreman (FluidDomain.f90:1225-1262);
                                12 (RBGK) and 13 (ELBM) are refused: the reference
                                reads an uninitialised rate / array there */
    double nu;               /* flow%nu; tau = nu/(dh/3) + 1/2 (FluidDomain.f90:452) */
    const double *m_collid;  /* optional 19x19 column-major M_COLLID (NULL: built here) */
    const double *m_force;   /* optional 19x19 column-major M_FORCE  (NULL: built here) */
    int    precision;        /* FSI_PREC_* */
    double denIn;
    double uvwIn[3];
    double shearRateIn[3];
    int    velocityKind;     /* 0 shear profile, 2 oscillatory (FluidDomain.f90:1791-1824) */
    double params[10];       /* params(1:10) of the block line (FluidDomain.f90:84);
                                params[0] = the TRT magic parameter Lambda of
                                calculate_TRT_params (FluidDomain.f90:458-464) */
} fsi_block_desc;

/* message of the last error on this thread ("" if none); returns its length */
int fsi_last_error(char *buf, int len);

/* library and device information: sm count, arch, build flags */
int fsi_device_info(int *sm_count, int *cc_major, int *cc_minor);

/* allocate_fluid_ + calculate_SRT/MRT_params (FluidDomain.f90:378-522) */
int fsi_block_create(fsi_block_t *out, const fsi_block_desc *desc);
int fsi_block_destroy(fsi_block_t h);

/* tau, Omega and the MRT matrices in use (FluidDomain.f90:450-522) */
int fsi_block_get_params(fsi_block_t h, double *tau, double *omega,
                         double *m_collid, double *m_force);

/* Omega2 of the TRT model (FluidDomain.f90:458-464; 0 for other models) */
int fsi_block_get_omega2(fsi_block_t h, double *omega2);

/* tau_all(z,y,x) (FluidDomain.f90:35): the per-cell relaxation time that the
 * Smagorinsky, WALE and Vreman collisions write every step (and WALE reads);
 * tau everywhere for the other models. N doubles in (z,y,x) order. */
int fsi_block_get_tau_all(fsi_block_t h, double *tau_all);

/* copy fIn(z,y,x,0:18) between host and device (write_continue_/read_continue_,
 * FluidDomain.f90:1770-1789, keep this exact layout) */
int fsi_block_upload_f(fsi_block_t h, const double *fIn);
int fsi_block_download_f(fsi_block_t h, double *fIn);

/* Continue files (restart). fsi_continue_write: write_continue_blocks and
 * write_continue_ (FluidDomain.f90:266-281, 1770-1777): int32 n, int32 step,
 * real8 time, then per block real8 xmin, ymin, zmin, dh, int32 xDim, yDim,
 * zDim and real8 fIn(z,y,x,0:18), stream access in native byte order (the
 * reference's ./DatContinue/continue<time> file). fsi_continue_read:
 * check_is_continue (FluidDomain.f90:127-236): the fIn of each of the n
 * blocks is re-gridded on the GPU from the file's blocks by trilinear
 * interpolation, each cell from the first file block containing it in the
 * reference's dh order; cells outside every file block keep their values.
 * step and time receive the file's. FSI_E_ARG for a short or malformed file. */
int fsi_continue_write(const char *path, const fsi_block_t *blocks, int n, int step, double time);
int fsi_continue_read(const char *path, const fsi_block_t *blocks, int n, int *step, double *time);

/* initialise_flow: den = denIn, uuu = inflow profile, fIn = feq (FluidDomain.f90:524-544) */
int fsi_block_initialise(fsi_block_t h, double time);

/* set_boundary_conditions_ on the current state (FluidDomain.f90:616-1126);
 * the first call marks half-way faces ready without applying them, as the
 * reference's allocate-on-first-call does (FluidDomain.f90:660-662) */
int fsi_block_set_boundary_conditions(fsi_block_t h, double blktime);

/* calculate_macro_quantities_ over the whole block (FluidDomain.f90:1128-1145);
 * den (N) and uuu (3N) are written to the host if non-NULL */
int fsi_block_macro(fsi_block_t h, const double vf[3], double *den, double *uuu);

/* Output packing on the GPU (the outputs of main.f90:107-141), each from the
 * macro quantities of the current state with volume force vf:
 * write_flow_ (FluidDomain.f90:1628-1663, outputtype 1): out (z,y,x,k), the
 * block minus `offset` cells (offsetOutput) on each side, k = p, u, v, w as
 * FP32: p = (den - denIn)/3, u/Uref. */
int fsi_block_pack_flow(fsi_block_t h, const double vf[3], double denIn, double Uref, int offset,
                        float *out);
/* write_fluid_flux (FluidDomain.f90:2019-2056): x-fluxes through the planes
 * x = 1, (xDim+1)/2, xDim, divided by denIn*Uref*(zmax-zmin)*(ymax-ymin) */
int fsi_block_flux(fsi_block_t h, const double vf[3], double denIn, double Uref, double flux[3]);
/* write_fluid_information probes (FlowCondition.f90:195-223 with
 * grid_value_interpolation, Util.f90:123-158): trilinear velocity / Uref at
 * n points xyz (3,n) into uvw (3,n); a point outside the block returns
 * FSI_E_RANGE (the reference stops) */
int fsi_block_probes(fsi_block_t h, const double vf[3], int n, const double *xyz, double Uref, double *uvw);

/* The fluid part of one time step, LBMBlockComm.f90:288-303:
 * add_volume_force_ (FluidDomain.f90:1182), collision_ (:1208),
 * halfwayBCset_ (:567), streaming_ (:1514), set_boundary_conditions_ (:616).
 * macro (:1128) and ResetVolumeForce_ (:1195) are folded in: cells outside
 * the IB window take den/u from their own distributions and force = vf;
 * cells inside take the IB-corrected values from the last fsi_ib_solve.
 * The one asynchronous call: it reads no host memory after its arguments,
 * so it returns once the step is queued on the block's stream; every call
 * that hands data back to the host waits for it (a kernel fault of the step
 * is reported by that next call). */
int fsi_block_step(fsi_block_t h, const double vf[3], double blktime);

/* run nsteps of fsi_block_step with constant vf and blktime advanced by dh per
 * step, launched from a captured CUDA graph; *ms = device time (CUDA events) */
int fsi_block_run(fsi_block_t h, const double vf[3], double blktime0, int nsteps, float *ms);

/* No counterpart in the reference: the bulk step kernel of the offset forms
 * (FSI_PREC_F32/F16/BF16): the paired form (one group of z-rows per CTA,
 * FSI_KERNEL_AUTO) or the pipelined persistent form (bulk copies into shared
 * memory, zDim a multiple of 8). Both compute the same values, bitwise. The
 * FP64 forms ignore it. */
#define FSI_KERNEL_AUTO      0
#define FSI_KERNEL_PAIRED    1
#define FSI_KERNEL_PIPELINED 2
int fsi_block_set_kernel(fsi_block_t h, int kernel);

/* No counterpart in the reference: how fsi_block_ib_step runs the IB stage
 * of the fast forms. FSI_IB_GRID: one cooperative launch over the GPU, then
 * the fluid step. FSI_IB_OVERLAP: the same cooperative launch on a second,
 * high-priority stream beside the bulk step (both only read the state), the
 * IB-window fix-up and face hooks after both. FSI_IB_CLUSTER: as OVERLAP with
 * the IB stage on one thread-block cluster. FSI_IB_AUTO: OVERLAP for the
 * offset forms when the paired kernels run the step, else GRID. Same
 * stopping rule and results to rounding (their sums are atomics, in any
 * order). FSI_IB_GATHER: the kernels FSI_PREC_F64 uses (each window cell
 * gathers its stencil entries in the reference's serial order, FP64; the
 * residual test on the host between iterations), on the fast forms' window
 * velocity: the same force from run to run, for comparisons. */
#define FSI_IB_AUTO    0
#define FSI_IB_GRID    1
#define FSI_IB_CLUSTER 2
#define FSI_IB_OVERLAP 3
#define FSI_IB_GATHER  4
int fsi_block_set_ib_mode(fsi_block_t h, int mode);

/* No counterpart in the reference: device time of the work a host loop
 * queues on the block's stream. stop = 0 records the start mark; stop = 1
 * records the end mark, waits for it and sets *ms to the time between. */
int fsi_block_timer(fsi_block_t h, int stop, float *ms);

/* Immersed boundary (Solidbody.f90:869-1049). Bodies are stored back to back:
 * marker m of body b is global marker offs[b]+m, offs = prefix sums of M. */
int fsi_ib_set_bodies(fsi_block_t h, int nbodies, const int *M, const int bc[6]);

/* One call per time step (FSInteraction_force -> calculate_interaction_force,
 * Solidbody.f90:589-918, for a block's carried bodies): UpdateElmtInterp_
 * (:760), macro and force reset in the IB window, the PenaltyForce_ loop
 * (:893-906, at most ntol iterations, stop when residual <= dtol) and the
 * spreading of FluidVolumeForce_ (:968-977), then add_volume_force_.
 * xyz/vel (3,Mtot), area (Mtot) in; eforce (3,Mtot) out (v_Eforce, FP64);
 * iters and residual out (both may be NULL). */
int fsi_ib_solve(fsi_block_t h, const double *xyz, const double *vel, const double *area,
                 const double vf[3], double denIn, double dt, double Uref,
                 int ntol, double dtol, double *eforce, int *iters, double *residual);

/* fsi_ib_solve followed by fsi_block_step(h, vf, blktime), the order of one
 * step in LBMBlockComm.f90:279-305. For the fast forms the fluid step is
 * queued behind the IB stage on the block's stream and the call returns as
 * soon as the Lagrangian force has reached the host, while the step runs;
 * the IB window of this solve is used by that step only. (If the IB stage
 * fails, the step has been queued on its result: the state must be discarded
 * with the error.) FSI_PREC_F64 runs the two calls one after the other. */
int fsi_block_ib_step(fsi_block_t h, const double *xyz, const double *vel, const double *area,
                      const double vf[3], double denIn, double dt, double Uref, int ntol,
                      double dtol, double blktime, double *eforce, int *iters, double *residual);

/* fsi_block_ib_step in two calls (no counterpart in the reference): the
 * first queues the IB stage and the fluid step and returns at once (the
 * marker arrays may be reused on return); the second waits for the IB stage
 * and returns its force, iteration count and residual (errors of the IB
 * stage come back here). A host with prescribed body motion can prepare the
 * next step's markers in between. While a step is pending, the IB calls of
 * the block (fsi_ib_solve*, fsi_block_ib_step*, fsi_ib_set_bodies) return
 * FSI_E_STATE; the other calls queue behind it on the block's stream.
 * fsi_block_ib_wait without a pending step returns FSI_E_STATE. */
int fsi_block_ib_step_async(fsi_block_t h, const double *xyz, const double *vel, const double *area,
                            const double vf[3], double denIn, double dt, double Uref, int ntol,
                            double dtol, double blktime);
int fsi_block_ib_wait(fsi_block_t h, double *eforce, int *iters, double *residual);

/* the stencil of the last fsi_ib_solve: v_Ei (12,Mtot) 1-based, v_Ew (12,Mtot) */
int fsi_ib_get_stencil(fsi_block_t h, int16_t *ei, float *ew);

/* the IB window of the last fsi_ib_solve (0-based inclusive x0,x1,y0,y1,z0,z1) */
int fsi_ib_get_window(fsi_block_t h, int box[6]);

/* Learned warm start of the penalty loop. No counterpart in the reference:
 * its loop (Solidbody.f90:893-906) starts every time step from v_Eforce = 0.
 * A 12 -> 64 -> 64 -> 3 perceptron (tanh hidden layers, FP32) maps the
 * features of one marker to its converged Lagrangian force; the prediction
 * is applied as a first velocity correction and the unchanged loop then runs
 * to the same ntol/dtol test, so the warm start changes how many iterations
 * are needed, not the stopping rule.
 *
 * Features of marker m, in this order (velocities divided by Uref):
 *   0-2  U_body - u_interp of the uncorrected field
 *   3-5  U_body
 *   6-8  body acceleration (aux), divided by Uref
 *   9-11 surface normal (aux)
 * Target: the converged v_Eforce of the marker divided by (area * Uref).
 * Inputs are standardised with (x - mean)/std and outputs de-standardised,
 * from FSI_MLP_NNORM statistics: mean_in[12], std_in[12], mean_out[3],
 * std_out[3]. Parameters, one FP32 array of FSI_MLP_NPARAM: W1[64][12],
 * b1[64], W2[64][64], b2[64], W3[3][64], b3[3] (row = output unit). */
#define FSI_MLP_IN     12
#define FSI_MLP_OUT    3
#define FSI_MLP_NPARAM 5187
#define FSI_MLP_NNORM  30
typedef struct fsi_mlp *fsi_mlp_t;
/* Glorot-uniform weights from seed, zero biases, identity statistics, on the
 * current device */
int fsi_mlp_create(fsi_mlp_t *out, unsigned long long seed);
int fsi_mlp_destroy(fsi_mlp_t m);
/* n must be FSI_MLP_NPARAM; set_params also clears the Adam moments */
int fsi_mlp_set_params(fsi_mlp_t m, const float *params, int n);
int fsi_mlp_get_params(fsi_mlp_t m, float *params, int n);
/* the FSI_MLP_NNORM statistics; deviations must be positive */
int fsi_mlp_set_norm(fsi_mlp_t m, const float *norm);
/* y (3,n) = network(x (12,n)), de-standardised */
int fsi_mlp_forward(fsi_mlp_t m, const float *x, int n, float *y);
/* gradient (FSI_MLP_NPARAM) and value of the loss
 * L = sum over the n samples and 3 outputs of (yn - tn)^2 / (3n),
 * yn and tn the standardised prediction and target */
int fsi_mlp_grad(fsi_mlp_t m, const float *x, const float *y, int n, float *grad, float *loss);
/* epochs of Adam (beta 0.9/0.999, eps 1e-8) over shuffled mini-batches of
 * batch samples; loss_per_epoch (epochs, may be NULL) receives the mean
 * mini-batch loss of each epoch. The Adam moments persist across calls. */
int fsi_mlp_train(fsi_mlp_t m, const float *x, const float *y, int n, int epochs, int batch, float lr,
                  unsigned long long seed, float *loss_per_epoch);
/* fsi_ib_solve for the fast forms (FSI_PREC_F64 returns FSI_E_ARG) with
 * aux (6,Mtot) = acceleration, normal per marker (NULL: zeros); warm (NULL:
 * the reference's loop from zero force); features (12,Mtot) out (NULL: not
 * written) -- with warm NULL and ntol large, the features and the returned
 * eforce are a training pair. */
int fsi_ib_solve_warm(fsi_block_t h, const double *xyz, const double *vel, const double *area,
                      const double *aux, const double vf[3], double denIn, double dt, double Uref,
                      int ntol, double dtol, fsi_mlp_t warm, float *features, double *eforce,
                      int *iters, double *residual);

/* Seeded start of the penalty loop (fast forms only). No counterpart in the
 * reference, whose loop starts every time step from v_Eforce = 0: guess
 * (3,Mtot) is applied as the first velocity correction and becomes the
 * starting v_Eforce, e.g. the previous time step's converged force; the
 * unchanged loop then runs to the same ntol/dtol test. A zero guess gives
 * the result of fsi_ib_solve. FSI_E_NAN for a non-finite guess. */
int fsi_ib_solve_seeded(fsi_block_t h, const double *xyz, const double *vel, const double *area,
                        const double *guess, const double vf[3], double denIn, double dt, double Uref,
                        int ntol, double dtol, double *eforce, int *iters, double *residual);

/* No counterpart in the reference: many independent blocks stepped together
 * (a parameter sweep of cases on one GPU). The blocks keep their handles and
 * state; while batched they are stepped only through fsi_batch_ib_step (the
 * other block calls stay valid between batch steps). Requirements: offset
 * storage (FSI_PREC_F32/F16/BF16, the same for all), one collision model,
 * even zDim up to 1024 with a moment-form MRT matrix, bodies already set
 * (zero bodies allowed), no face of code 0, 1, 102, 203 or 204. */
typedef struct fsi_batch *fsi_batch_t;
int fsi_batch_create(fsi_batch_t *out, int nblocks, const fsi_block_t *blocks);
int fsi_batch_destroy(fsi_batch_t b);
/* One time step of every block: the IB stage (fsi_ib_solve) then the fluid
 * step (fsi_block_step), as fsi_block_ib_step does for one block. Markers of
 * all blocks are packed in block order: xyz, vel (3, sum Mtot), area (sum
 * Mtot), eforce (3, sum Mtot) out; vf (3, n), denIn, dt, Uref, blktime (n);
 * iters, residual (n) out (may be NULL). The device work of the step is one
 * CUDA graph: an upload of every block's tables and markers, the IB stage of
 * all blocks (one 8-CTA cluster per block), the bulk step of all blocks,
 * their IB-window fix-ups, one launch per face index and one download.
 * FSI_E_STATE when a block's bodies changed (fsi_ib_set_bodies) after
 * fsi_batch_create. */
int fsi_batch_ib_step(fsi_batch_t b, const double *xyz, const double *vel, const double *area,
                      const double *vf, const double *denIn, const double *dt, const double *Uref,
                      int ntol, double dtol, const double *blktime, double *eforce, int *iters,
                      double *residual);
/* Autotuner: times the bulk step of all blocks in each form it can take
 * (reps launches each, reading the current state and writing the spare
 * buffer, so the state does not change) and keeps the fastest: the one
 * table-driven kernel over every block's row groups at each CTA size it is
 * built for (*threads = 128, 256, 512), or every block's own single-block
 * bulk kernel, launched side by side inside the step's graph (*threads = 0). */
int fsi_batch_tune(fsi_batch_t b, int reps, int *threads, float *ms_per_step);
/* the bulk step's form by hand: 128, 256 or 512 (the table-driven kernel's
 * CTA size) or 0 (each block's own kernel) */
int fsi_batch_set_threads(fsi_batch_t b, int threads);

/* Block refinement, LBMBlockComm.f90:340-979. A pair links a father and a
 * son block; the son's faces with code 0 (BCfluid) receive father data. */
typedef struct fsi_pair *fsi_pair_t;
/* build_blocks_comunication for one pair (LBMBlockComm.f90:42-92);
 * scheme = flow%interpolateScheme (1 linear, 2 third/fourth order) */
int fsi_pair_create(fsi_pair_t *out, fsi_block_t father, fsi_block_t son, int scheme);
int fsi_pair_destroy(fsi_pair_t p);
/* extract_interpolate_layer for this pair, time level 1 or 2 (LBMBlockComm.f90:340-505) */
int fsi_pair_extract(fsi_pair_t p, int time_level);
/* interpolation_father_to_son (LBMBlockComm.f90:655-806); vf = father volume force */
int fsi_pair_father_to_son(fsi_pair_t p, int n_timeStep, const double vf[3]);
/* deliver_son_to_father (LBMBlockComm.f90:546-653); vf = son volume force */
int fsi_pair_son_to_father(fsi_pair_t p, const double vf[3]);

/* No counterpart in the reference. fsi_pair_father_to_son for callers that
 * cannot allocate device memory once their time loop runs -- a host that
 * budgets all GPU memory at start-up, or one that may not call cudaMalloc
 * from its stepping code -- since fsi_pair_father_to_son interpolates the
 * father's face into scratch planes that fsi_pair_create allocated. This
 * variant allocates nothing: its scratch is one file-scope device array of
 * FSI_STATIC_FACE_CELLS son face cells (20 doubles each, 10 MiB). The array
 * is placed on a device, and its device address looked up
 * (cudaGetSymbolAddress), by the first fsi_pair_create on that device, so
 * the memory is taken at set-up and held until the process exits; the static
 * calls themselves take none. Create pairs before any stream capture. Faces
 * larger than FSI_STATIC_FACE_CELLS return FSI_E_ARG. All calls share the one
 * array and each call leaves its last contents there (every element a call
 * reads lies inside its own face and is written by that call first, so
 * nothing needs clearing; a stencil that would read past the face returns
 * FSI_E_RANGE, as in fsi_pair_father_to_son): calls that overlap on the GPU,
 * from different threads or streams, race. Same arguments and results as
 * fsi_pair_father_to_son. */
#define FSI_STATIC_FACE_CELLS 65536
int fsi_pair_father_to_son_static(fsi_pair_t p, int n_timeStep, const double vf[3]);

#ifdef __cplusplus
}
#endif
#endif /* FSI_GPU_H */
