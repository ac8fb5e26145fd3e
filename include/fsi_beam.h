/*
 * fsi_beam.h -- C-ABI of the host-side structural solver of a flexible body:
 * the co-rotational 3-D Timoshenko beam of SolidSolver.f90 (Newmark-beta time
 * integration, full Newton-Raphson iteration, matrix-free block-Jacobi
 * preconditioned conjugate gradients) and the plate's immersed-boundary
 * markers and beam load of Solidbody.f90.
 *
 * This is host code (FP64, no device work): the reference's host keeps it
 * in Fortran and hands only the Lagrangian force to and the marker positions
 * from the GPU step (fsi_block_ib_step in fsi_gpu.h). It is a restatement of
 * that Fortran in the reference's operation order, for hosts without the
 * Fortran program, and the structural half of the coupled flexible-plate
 * runs. Every function returns FSI_OK (0) or a negative FSI_E_* code of
 * fsi_gpu.h with a message from fsi_last_error(); where the reference stops
 * (CG breakdown, Beam_CheckCGBreakdown, SolidSolver.f90:2281-2302; a missing
 * section of the mesh file) the call returns an error instead.
 *
 * Arrays are column-major as in the reference: xyz (8,nND), material
 * (8,nMT), boundary (6,nND), elements (6,nEL) = i, j, k, TYPE, MAT, Nspan
 * (1-based node and material numbers), node fields (6,nND), marker fields
 * (3,M).
 */
#ifndef FSI_BEAM_H
#define FSI_BEAM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fsi_beam *fsi_beam_t;

/* Set_SolidSolver_Params (SolidSolver.f90:1249-1264), from the SolidBody
 * section of inFlow.dat (Solidbody.f90:100-115) */
typedef struct {
    double dampK, dampM;            /* stiffness- and mass-proportional damping */
    double GeoGamma;                /* scale of the geometric stiffness         */
    double NewmarkGamma, NewmarkBeta;
    double dtolFEM;                 /* Newton-Raphson stop: max squared increment */
    int    ntolFEM;                 /* Newton-Raphson iteration limit           */
    int    isKB;                    /* 0: EmR/tcR given, 1: KB/KS given, else the file's materials */
    double g[3];                    /* gravity                                  */
} fsi_beam_params;

/* Beam_SetSolver (SolidSolver.f90:1219-1248): one body of a group, angles and
 * phases in degrees as read from inFlow.dat (Solidbody.f90:116-160) */
typedef struct {
    int    iBodyModel;              /* 1 rigid (prescribed), 2 elastic          */
    int    isMotionGiven[6];        /* prescribed DOFs of constrained nodes     */
    double denR, psR, EmR, tcR, KB, KS;
    double Freq, St;
    double XYZo[3], initXYZVel[3], XYZAmpl[3], XYZPhi[3];
    double AoAo[3], AoAAmpl[3], AoAPhi[3];
} fsi_beam_body;

/* Beam_ReadBuild (SolidSolver.f90:1270-1399) on the parsed mesh arrays:
 * elements built, Beam_cptAsfac (*Asfac = summed element lengths, *Lchod)
 * and Beam_adjustBC applied. Segment_Build's opposite span directions
 * return FSI_E_ARG (the reference stops). */
int fsi_beam_create(fsi_beam_t *out, const fsi_beam_params *solver, const fsi_beam_body *body, int nND, int nEL,
                    int nMT, const double *xyz, const double *material, const int *boundary, const int *elements,
                    double *Asfac, double *Lchod);
int fsi_beam_destroy(fsi_beam_t b);

/* Beam_calculate_angle_material (SolidSolver.f90:1533-1616): degrees to
 * radians, section properties from EmR/tcR (isKB 0) or KB/KS (isKB 1);
 * *uMax updated in place, *Lthck out */
int fsi_beam_set_material(fsi_beam_t b, double Lref, double Uref, double denIn, const double uvwIn[3], double *uMax,
                          double *Lthck);

/* Beam_Initialise (SolidSolver.f90:1401-1446) and PlateBuild_
 * (Solidbody.f90:1051-1071); *M = markers of the plate (sum of Nspan) */
int fsi_beam_initialise(fsi_beam_t b, double time, int *M);

/* PlateUpdatePosVelArea_ (Solidbody.f90:604-646): marker positions, velocities
 * (element mid-point + spin of the span offset) and areas (times
 * -2 alpha denIn) from the current beam state; xyz, vel (3,M), area (M) */
int fsi_beam_markers(fsi_beam_t b, double alpha, double denIn, double *xyz, double *vel, double *area);

/* The beam load of FluidVolumeForce_ (Solidbody.f90:946-967): lodFlow = 0,
 * then each marker's Lagrangian force (3,M) and its moment about the element
 * centre, half to each element node; xyz (3,M) = the markers the force was
 * computed on */
int fsi_beam_load(fsi_beam_t b, const double *xyz, const double *eforce);

/* Beam_structure (SolidSolver.f90:1820-1877): prescribed motion (iBodyModel 1)
 * or one Newmark step by Newton-Raphson (iBodyModel 2) for sub-step isubstep
 * of the fluid step ending at `time`; iters (Newton-Raphson iterations,
 * FishInfo(2)) and dnorm (FishInfo(3)) out (may be NULL) */
int fsi_beam_structure(fsi_beam_t b, double time, int isubstep, double deltat, double subdeltat, int *iters,
                       double *dnorm);

/* Node positions, displacements, velocities, accelerations (6,nND) and the
 * fluid load lodFlow (6 nND); any pointer may be NULL */
int fsi_beam_state(fsi_beam_t b, double *pos, double *dsp, double *vel, double *acc, double *lodFlow);

/* nND, nEL and the reference point XYZ of the body (any pointer may be NULL) */
int fsi_beam_info(fsi_beam_t b, int *nND, int *nEL, double XYZ[3]);

#ifdef __cplusplus
}
#endif
#endif /* FSI_BEAM_H */
