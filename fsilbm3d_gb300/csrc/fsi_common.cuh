// fsi_common.cuh -- D3Q19 lattice tables and kernel argument structs shared
// by the CUDA translation units of libfsi_gpu.
//
// Lattice: ConstParams.f90:9-34 (directions ee, opposites oppo, weights wt,
// boundary codes). Distribution layout on the device is the reference's
// Fortran fIn(z,y,x,0:18): element (z,y,x,q) at z + Z*(y + Y*(x + X*q)).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fsi {

constexpr int Q = 19;

__host__ __device__ constexpr int ex_(int i) {
    return (i == 1 || i == 7 || i == 9 || i == 11 || i == 13) ? 1
         : (i == 2 || i == 8 || i == 10 || i == 12 || i == 14) ? -1 : 0;
}
__host__ __device__ constexpr int ey_(int i) {
    return (i == 3 || i == 7 || i == 8 || i == 15 || i == 17) ? 1
         : (i == 4 || i == 9 || i == 10 || i == 16 || i == 18) ? -1 : 0;
}
__host__ __device__ constexpr int ez_(int i) {
    return (i == 5 || i == 11 || i == 12 || i == 15 || i == 16) ? 1
         : (i == 6 || i == 13 || i == 14 || i == 17 || i == 18) ? -1 : 0;
}
__host__ __device__ constexpr int opp_(int i) {
    return i == 0 ? 0 : ((i <= 6) ? ((i % 2) ? i + 1 : i - 1)
                                  : (i <= 10 ? 17 - i : (i <= 14 ? 25 - i : 33 - i)));
}
// weights as exact binary64 values of 1/3, 1/18, 1/36
__host__ __device__ constexpr double wt_(int i) {
    return i == 0 ? 1.0 / 3.0 : (i <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
}

// representatives of the nine opposite pairs (positivedirs, ConstParams.f90:19);
// opp_ of them gives negativedirs (ConstParams.f90:20) in the same order
__host__ __device__ constexpr int pr_(int k) {
    return k == 0 ? 1 : k == 1 ? 3 : k == 2 ? 5 : k == 3 ? 7 : k == 4 ? 8 : k == 5 ? 11 : k == 6 ? 12 : k == 7 ? 15 : 16;
}

// collision models (iCollidModel, FluidDomain.f90:1225-1262)
enum : int { CM_SRT = 1, CM_TRT = 2, CM_MRT = 3, CM_SMAG = 11, CM_WALE = 14, CM_VREM = 15 };
__host__ __device__ constexpr bool les_model(int m) { return m == CM_SMAG || m == CM_WALE || m == CM_VREM; }
// models that read the neighbours' velocity
__host__ __device__ constexpr bool grad_model(int m) { return m == CM_WALE || m == CM_VREM; }

// incoming population sets per face (x-, x+, y-, y+, z-, z+), FluidDomain.f90:645-1065
__host__ __device__ constexpr int inc_(int k, int j) {
    return k == 0 ? (j == 0 ? 1 : j == 1 ? 7 : j == 2 ? 9 : j == 3 ? 11 : 13)
         : k == 1 ? (j == 0 ? 2 : j == 1 ? 8 : j == 2 ? 10 : j == 3 ? 12 : 14)
         : k == 2 ? (j == 0 ? 3 : j == 1 ? 7 : j == 2 ? 8 : j == 3 ? 15 : 17)
         : k == 3 ? (j == 0 ? 4 : j == 1 ? 9 : j == 2 ? 10 : j == 3 ? 16 : 18)
         : k == 4 ? (j == 0 ? 5 : j == 1 ? 11 : j == 2 ? 12 : j == 3 ? 15 : 16)
                  : (j == 0 ? 6 : j == 1 ? 13 : j == 2 ? 14 : j == 3 ? 17 : 18);
}
// the symmetric (302) source of incoming population j of face k: the mirror
// across the face normal (FluidDomain.f90:697,781,865,949,1033,1117)
// (the incoming set of the opposite face, in the same order)
__host__ __device__ constexpr int mir_(int k, int j) { return inc_(k ^ 1, j); }

// The moment basis of calculate_MRT_params (FluidDomain.f90:466-522): row k
// of M at velocity i. Every entry is an integer.
__host__ __device__ constexpr int mrow_(int k, int i) {
    const int x = ex_(i), y = ey_(i), z = ez_(i);
    const int e2 = x * x + y * y + z * z;
    return k == 0 ? 1
         : k == 1 ? 19 * e2 - 30
         : k == 2 ? (21 * e2 * e2 - 53 * e2 + 24) / 2
         : k == 3 ? x : k == 4 ? (5 * e2 - 9) * x
         : k == 5 ? y : k == 6 ? (5 * e2 - 9) * y
         : k == 7 ? z : k == 8 ? (5 * e2 - 9) * z
         : k == 9 ? 3 * x * x - e2
         : k == 10 ? (3 * e2 - 5) * (3 * x * x - e2)
         : k == 11 ? y * y - z * z
         : k == 12 ? (3 * e2 - 5) * (y * y - z * z)
         : k == 13 ? x * y : k == 14 ? y * z : k == 15 ? z * x
         : k == 16 ? (y * y - z * z) * x
         : k == 17 ? (z * z - x * x) * y
         : (x * x - y * y) * z;
}
// rows odd in e: opposite velocities carry opposite entries
__host__ __device__ constexpr bool modd_(int k) { return (k >= 3 && k <= 8) || k >= 16; }

// boundary codes, ConstParams.f90:31-34
enum : int {
    BC_EQ = 101, BC_NEQ = 102, BC_EXT1 = 103, BC_EXT2 = 104,
    BC_WALL = 201, BC_MWALL = 202, BC_WALL_HW = 203, BC_MWALL_HW = 204,
    BC_PERIODIC = 301, BC_SYMMETRIC = 302, BC_FLUID = 0, BC_FLUID_FATHER = 1
};

// inflow-velocity model of evaluate_velocity (FluidDomain.f90:1791-1824).
// kind 0: shear profile evaluated per point; kind 2: spatially uniform value
// osc (computed on the host with the host cos()).
struct Vel {
    int kind;
    double vin[3];
    double sr[3];
    double osc[3];
};

// IB window: the box of cells whose den/u/force come from the IB stage
struct Win {
    int x0, x1, y0, y1, z0, z1;   // inclusive, 0-based; x1 < x0 means empty
    int WY, WZ;
    long long n;
    const double *den;  // n
    const double *u;    // 3n
    const double *force;// 3n
};

// MRT matrices passed by value (kernel parameter space, uniform reads)
struct MrtMats {
    double mc[361];       // M_COLLID, column-major
    double mf[361];       // M_FORCE
    // M_COLLID = M^-1 S M with S diagonal, zero on the conserved moments
    // 0, 3, 5, 7, and M_FORCE = I - M_COLLID/2: then sd[k] = S_k / |row k|^2
    // and the moment-space kernels apply the collision; else diag = 0
    int diag;
    double sd[19];
};

struct StepArgs {
    const void *src;
    void *dst;
    int X, Y, Z;
    long long N;
    double dh, omega;
    double vf[3];
    Win win;
    double *hw[6];        // half-way face copies (19 per face cell), NULL = off
    double *den;          // full-size den/u, written on layer-2 planes of 102 faces
    double *u;
    int l2[6];            // 1 if face k has code 102
    int *kerr;            // error word of the pipelined kernel (bit 1: a bounded wait ran out)
    int variant;          // bulk kernel of the offset forms: 0 auto, 1 paired, 2 pipelined
    // z- / z+ faces of code 101 with a uniform face velocity, written by the
    // paired step kernels themselves: zg holds the 19 offset equilibrium
    // populations g = feq(denIn, u_face) - w of the face; set only when the
    // host leaves those faces out of the face kernels
    int zeq[2];
    float zg[2][19];
    // host only: an event the window fix-up and face hooks wait for (the IB
    // stage running beside the bulk step on another stream), or null
    void *join;
    // TRT (iCollidModel 2): the antisymmetric rate Omega2. The SRT collisions
    // with a per-cell rate (11 Smagorinsky, 14 WALE, 15 Vreman): tau, flow%nu,
    // the model constant and tau_all(z,y,x), which WALE also reads. WALE and
    // Vreman read the velocity of each cell and its neighbours from u above,
    // written for every cell by a macro pass before the step.
    double omega2, tau, nu, cles;
    double *tau_all;
    // the offset storage forms keep that velocity field and tau_all in FP32
    // (uf: 3N, tauf: N) and use them instead of u and tau_all
    float *uf, *tauf;
    // fast forms, WALE: the rotation-rate entries O12, O13, O23 of every cell
    // (3N, the arithmetic type), written by the gradient pass before the step
    void *og;
    // offset forms: the tau_all the step reads (WALE reads the previous
    // step's and writes tauf; the others read and write the same array)
    float *tauf_prev;
};

struct BcArgs {
    void *f;
    int X, Y, Z;
    long long N;
    int face;             // 0..5
    int code;
    double dh, xmin, ymin, zmin, xmax, ymax, zmax;
    double denIn;
    Vel vel;
    const double *hw;     // half-way copy of this face
    const double *den;    // full-size den/u (102)
    const double *u;
    int zlo, zhi;         // x/y faces: the z range they act on (the z faces the
                          // step kernel wrote are left to it)
    // offset forms, code 101 with a face velocity uniform over the face: the
    // face's 19 offset equilibrium populations, formed on the host in FP64
    int uni;
    float gq[19];
};

}  // namespace fsi
