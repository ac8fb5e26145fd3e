/*
 * fsi_oracle.h -- CPU FP64 restatement of FSILBM3D's per-time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the oracle the CUDA path is tested against:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it. The product (libfsi_gpu.so) never links or calls it.
 *
 * Parity status: UNPINNED against the Fortran reference itself. No Fortran
 * compiler exists where this project is built or run, and the reference
 * ships no tests, fixtures or example inputs. The restatement is checked by
 * analytic known-answer tests (tests/test_oracle_kat.py) and by committed
 * golden vectors that it generated (tests/golden/), which pin it against
 * accidental change.
 *
 * Every routine follows the reference loop by loop, in the reference's
 * floating-point operation order (left-to-right evaluation, sequential SUM
 * and MATMUL accumulation). Build with -ffp-contract=off so that no
 * multiply-add is fused, as gfortran does on x86-64 without -march.
 *
 * Array layout is the reference's column-major fIn(z,y,x,q): the linear
 * index of (z,y,x,q) (0-based) is z + Z*(y + Y*(x + X*q)).
 */
#ifndef FSI_ORACLE_H
#define FSI_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Flow conditions used inside the hot path (FlowCondition.f90:11-26). */
typedef struct {
    double denIn;
    double uvwIn[3];
    double shearRateIn[3];
    int    velocityKind;          /* 0 shear, 2 oscillatory */
    int    interpolateScheme;     /* 1 linear, 2 third/fourth order */
    double volumeForceIn[3];
    double volumeForceAmp, volumeForceFreq, volumeForcePhi;
    double nu;
} or_flow;

/* One LBM block (FluidDomain.f90:17-56). Arrays are owned by the caller. */
typedef struct {
    int    X, Y, Z;
    double dh, xmin, ymin, zmin, xmax, ymax, zmax;
    int    bnd[6];
    int    periodic[3];
    int    model;                 /* iCollidModel: 1 SRT, 2 TRT, 3 MRT, 11 SRT+Smagorinsky,
                                     14 SRT+WALE, 15 SRT+Vreman (12, 13 not restated) */
    double tau, omega;
    double mc[361], mf[361];      /* M_COLLID, M_FORCE, column-major (i + 19*j) */
    double volumeForce[3];
    double blktime;
    double *f;                    /* 19*N */
    double *u;                    /* 3*N   uuu(z,y,x,1:3) */
    double *den;                  /* N */
    double *force;                /* 3*N */
    double *tau_all;              /* N   (may be NULL: constant tau; required by 11, 14, 15) */
    double *hw[6];                /* half-way face copies, 19*face each (may be NULL) */
    int    hw_ready[6];           /* 0 until the first set_boundary_conditions call */
    double params[10];            /* params(1:10) of the block (FluidDomain.f90:84);
                                     params[0] = TRT magic parameter Lambda */
    double omega2;                /* TRT antisymmetric rate (FluidDomain.f90:458-464) */
    double nu;                    /* flow%nu, read by the WALE and Vreman models */
} or_block;

/* One immersed body (Solidbody.f90:25-68), markers stored as (3,M). */
typedef struct {
    int      M;
    double  *xyz;                 /* v_Exyz(3,M)   */
    double  *vel;                 /* v_Evel(3,M)   */
    double  *area;                /* v_Ea(M)       */
    double  *eforce;              /* v_Eforce(3,M) */
    int16_t *ei;                  /* v_Ei(12,M), 1-based indices */
    float   *ew;                  /* v_Ew(12,M)  */
} or_body;

/* ConstParams / FluidDomain helpers */
void   or_evaluate_velocity(const or_flow *fl, double time, double zc, double yc, double xc, double out[3]);
void   or_feq_dist(double density, const double vel[3], double out[19]);
void   or_mrt_matrices(double omega, double mc[361], double mf[361]);
void   or_block_setup(or_block *b, const or_flow *fl);
void   or_initialise_flow(or_block *b, const or_flow *fl, double time);
void   or_init_tgv(or_block *b, double u0, double rho0);

/* the per-step routines */
void   or_update_volume_force(or_block *b, const or_flow *fl);
void   or_macro(or_block *b);
void   or_reset_force(or_block *b);
void   or_add_force(or_block *b);
void   or_collide(or_block *b);
void   or_halfway_set(or_block *b);
void   or_stream(or_block *b, double *tmp);
int    or_set_bc(or_block *b, const or_flow *fl);

/* immersed boundary */
int    or_ib_stencil(or_body *bd, const or_block *b);
void   or_ib_penalty(or_body *bd, int nb, or_block *b, double denIn, double dt, double Uref,
                     int ntol, double dtol, int *iters, double *residual);
void   or_ib_spread(or_body *bd, int nb, or_block *b);

/* one whole step of a single block (LBMBlockComm.f90:279-318 without sons) */
int    or_step(or_block *b, const or_flow *fl, or_body *bd, int nb, double Uref,
               int ntol, double dtol, double *tmp, int *iters, double *residual);

/* continue-file re-grid (check_is_continue, FluidDomain.f90:127-236): the
 * reference's order of the file's blocks (sortdh, 0-based), and the fIn of
 * block b from the file's blocks old[0..nold) (X, Y, Z, dh, xmin, ymin, zmin
 * and f used); cells outside every file block keep their values */
void   or_continue_order(int nold, const double *dh, int *order);
void   or_continue_regrid(or_block *b, int nold, const or_block *old, const int *order);

/* field statistics (FluidDomain.f90:1739-1768) */
void   or_field_stat(const or_block *b, double Uref, double l2[3], double linf[3]);

/* block refinement communication (LBMBlockComm.f90:340-979) */
typedef struct {
    int sds[6], s[6], f[6], si[6], fi[6];
    int xDimS, xDimF, yDimS, yDimF, zDimS, zDimF;
} or_pair;
void   or_build_pair(const or_block *fa, const or_block *so, or_pair *p);
void   or_extract_layer(const or_block *fa, const or_block *so, const or_pair *p, int time,
                        double *buf_f[6][2], double *buf_tau[6][2]);
void   or_interp_f2s(or_block *so, const or_block *fa, const or_pair *p, int n_timeStep,
                     double *buf_f[6][2], double *buf_tau[6][2], int scheme);
void   or_deliver_s2f(or_block *fa, const or_block *so, const or_pair *p);
void   or_grid_transform(double fin[19], double coeff, const double vf[3], double dh);

#ifdef __cplusplus
}
#endif
#endif
