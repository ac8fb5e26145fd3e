/*
 * fsi_oracle.c -- CPU FP64 restatement of FSILBM3D's per-time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA path is tested against, never shipped or
 * called by the product. See fsi_oracle.h for the parity status (unpinned
 * against the Fortran itself; pinned by analytic known-answer tests and by
 * committed golden vectors).
 *
 * Each routine cites the reference file:line it restates and keeps the
 * reference's operation order. Build: gcc -O2 -ffp-contract=off -fopenmp.
 */
#include "fsi_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define Q 19
#define PI 3.141592653589793

/* ConstParams.f90:11-25 */
static const int EX[Q] = {0, 1,-1, 0, 0, 0, 0, 1,-1, 1,-1, 1,-1, 1,-1, 0, 0, 0, 0};
static const int EY[Q] = {0, 0, 0, 1,-1, 0, 0, 1, 1,-1,-1, 0, 0, 0, 0, 1,-1, 1,-1};
static const int EZ[Q] = {0, 0, 0, 0, 0, 1,-1, 0, 0, 0, 0, 1, 1,-1,-1, 1, 1,-1,-1};
static const int OPPO[Q] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
static const double WT[Q] = {
    1.0/3.0, 1.0/18.0, 1.0/18.0, 1.0/18.0, 1.0/18.0, 1.0/18.0, 1.0/18.0,
    1.0/36.0, 1.0/36.0, 1.0/36.0, 1.0/36.0, 1.0/36.0, 1.0/36.0,
    1.0/36.0, 1.0/36.0, 1.0/36.0, 1.0/36.0, 1.0/36.0, 1.0/36.0};
/* ConstParams.f90:28 */
static const double S0 = 0.0, S1 = 1.19, S2 = 1.4, S4 = 1.2, S10 = 1.4, S16 = 1.98;
static const double CS2 = 1.0/3.0;

/* incoming populations per face, FluidDomain.f90:645,729,813,897,981,1065 */
static const int INC[6][5] = {
    {1, 7, 9, 11, 13}, {2, 8, 10, 12, 14},
    {3, 7, 8, 15, 17}, {4, 9, 10, 16, 18},
    {5, 11, 12, 15, 16}, {6, 13, 14, 17, 18}};
/* sources of the symmetric (302) copy, FluidDomain.f90:697,781,865,949,1033,1117 */
static const int MIR[6][5] = {
    {2, 8, 10, 12, 14}, {1, 7, 9, 11, 13},
    {4, 9, 10, 16, 18}, {3, 7, 8, 15, 17},
    {6, 13, 14, 17, 18}, {5, 11, 12, 15, 16}};

static inline size_t ncell(const or_block *b) { return (size_t)b->X * b->Y * b->Z; }
static inline size_t cidx(const or_block *b, int z, int y, int x) {
    return (size_t)z + (size_t)b->Z * ((size_t)y + (size_t)b->Y * (size_t)x);
}

/* FluidDomain.f90:1791-1824 */
void or_evaluate_velocity(const or_flow *fl, double time, double zc, double yc, double xc, double out[3]) {
    const double *vi = fl->uvwIn, *sr = fl->shearRateIn;
    if (fl->velocityKind == 0) {
        out[0] = ((vi[0] + 0.0 * sr[0]) + yc * sr[1]) + zc * sr[2];
        out[1] = ((vi[1] + xc * sr[0]) + 0.0 * sr[1]) + zc * sr[2];
        out[2] = ((vi[2] + xc * sr[0]) + yc * sr[1]) + 0.0 * sr[2];
    } else {
        double amp = sr[0], freq = sr[1], phi = sr[2];
        out[0] = vi[0] + amp * cos(((2.0 * PI) * freq) * time + (phi / 180.0) * PI);
        out[1] = vi[1];
        out[2] = vi[2];
    }
}

/* calculate_distribution_funcion, FluidDomain.f90:1827-1834 */
void or_feq_dist(double density, const double v[3], double out[Q]) {
    double uSqr = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
    for (int i = 0; i < Q; i++) {
        double uxyz = (v[0] * (double)EX[i] + v[1] * (double)EY[i]) + v[2] * (double)EZ[i];
        out[i] = (WT[i] * density) * ((((1.0 + 3.0 * uxyz) + (4.5 * uxyz) * uxyz) - 1.5 * uSqr));
    }
}

/* evaluate_moving_wall, FluidDomain.f90:1837-1843 */
static void moving_wall(double density, const double v[3], const double *din, size_t stride, double out[Q]) {
    for (int i = 0; i < Q; i++) {
        double uxyz = (v[0] * (double)EX[i] + v[1] * (double)EY[i]) + v[2] * (double)EZ[i];
        out[i] = din[stride * OPPO[i]] + (((2.0 * WT[i]) * density) * uxyz) * 3.0;
    }
}

/* calculate_MRT_params, FluidDomain.f90:466-522 (sequential-k matrix products) */
void or_mrt_matrices(double omega, double mc[361], double mf[361]) {
    double Mm[Q][Q], Mi[Q][Q], MM[Q][Q], T[Q][Q], S[Q];
    for (int I = 0; I < Q; I++) {
        double e2 = (double)(EX[I] * EX[I] + EY[I] * EY[I] + EZ[I] * EZ[I]);
        double ex = EX[I], ey = EY[I], ez = EZ[I];
        Mm[0][I] = 1.0;
        Mm[1][I] = 19.0 * e2 - 30.0;
        Mm[2][I] = (21.0 * e2 * e2 - 53.0 * e2 + 24.0) / 2.0;
        Mm[3][I] = ex; Mm[5][I] = ey; Mm[7][I] = ez;
        Mm[4][I] = (5.0 * e2 - 9.0) * ex;
        Mm[6][I] = (5.0 * e2 - 9.0) * ey;
        Mm[8][I] = (5.0 * e2 - 9.0) * ez;
        Mm[9][I] = 3.0 * ex * ex - e2;
        Mm[10][I] = (3.0 * e2 - 5.0) * (3.0 * ex * ex - e2);
        Mm[11][I] = ey * ey - ez * ez;
        Mm[12][I] = (3.0 * e2 - 5.0) * (ey * ey - ez * ez);
        Mm[13][I] = ex * ey;
        Mm[14][I] = ey * ez;
        Mm[15][I] = ez * ex;
        Mm[16][I] = (ey * ey - ez * ez) * ex;
        Mm[17][I] = (ez * ez - ex * ex) * ey;
        Mm[18][I] = (ex * ex - ey * ey) * ez;
    }
    for (int i = 0; i < Q; i++)
        for (int j = 0; j < Q; j++) Mi[i][j] = Mm[j][i];
    for (int i = 0; i < Q; i++)
        for (int j = 0; j < Q; j++) {
            double s = 0.0;
            for (int k = 0; k < Q; k++) s += Mm[i][k] * Mi[k][j];
            MM[i][j] = s;
        }
    for (int I = 0; I < Q; I++)
        for (int r = 0; r < Q; r++) Mi[r][I] = Mi[r][I] / MM[I][I];
    double Sv[Q] = {S0, S1, S2, S0, S4, S0, S4, S0, S4, omega, S10, omega, S10, omega, omega, omega, S16, S16, S16};
    for (int i = 0; i < Q; i++) S[i] = Sv[i];
    for (int i = 0; i < Q; i++)
        for (int j = 0; j < Q; j++) {
            double s = 0.0;
            for (int k = 0; k < Q; k++) s += Mi[i][k] * (k == j ? S[k] : 0.0);
            T[i][j] = s;
        }
    for (int i = 0; i < Q; i++)
        for (int j = 0; j < Q; j++) {
            double s = 0.0;
            for (int k = 0; k < Q; k++) s += T[i][k] * Mm[k][j];
            mc[i + Q * j] = s;
        }
    for (int i = 0; i < Q; i++)
        for (int j = 0; j < Q; j++) mf[i + Q * j] = (i == j ? 1.0 : 0.0) - 0.5 * mc[i + Q * j];
}

/* read_fuild_blocks / check_periodic_boundary_ / calculate_SRT_params,
 * FluidDomain.f90:94-125, 450-456 */
void or_block_setup(or_block *b, const or_flow *fl) {
    for (int i = 0; i < 3; i++) {
        b->periodic[i] = (b->bnd[2 * i] == 301 || b->bnd[2 * i + 1] == 301) ? 1 : 0;
    }
    b->xmax = b->xmin + b->dh * (double)(b->X - 1);
    b->ymax = b->ymin + b->dh * (double)(b->Y - 1);
    b->zmax = b->zmin + b->dh * (double)(b->Z - 1);
    if (b->periodic[0]) b->xmax = b->xmax + b->dh;
    if (b->periodic[1]) b->ymax = b->ymax + b->dh;
    if (b->periodic[2]) b->zmax = b->zmax + b->dh;
    b->tau = fl->nu / (b->dh * CS2) + 0.5;
    b->omega = 1.0 / b->tau;
    if (b->tau_all) {
        size_t n = ncell(b);
        for (size_t i = 0; i < n; i++) b->tau_all[i] = b->tau;
    }
    if (b->model == 3) or_mrt_matrices(b->omega, b->mc, b->mf);
    /* calculate_TRT_params, FluidDomain.f90:458-464 */
    b->omega2 = 0.0;
    if (b->model == 2) {
        double tmp = (b->params[0] * 4.0 - 1.0) * b->omega + 2.0;
        b->omega2 = (2.0 * (2.0 - b->omega)) / tmp;
    }
    b->nu = fl->nu;
    for (int k = 0; k < 6; k++) b->hw_ready[k] = 0;
}

/* initialise_flow, FluidDomain.f90:524-544 */
void or_initialise_flow(or_block *b, const or_flow *fl, double time) {
    size_t n = ncell(b);
    b->blktime = time;
    for (int x = 0; x < b->X; x++) {
        double xc = b->xmin + b->dh * (double)x;
        for (int y = 0; y < b->Y; y++) {
            double yc = b->ymin + b->dh * (double)y;
            for (int z = 0; z < b->Z; z++) {
                double zc = b->zmin + b->dh * (double)z;
                size_t c = cidx(b, z, y, x);
                double v[3], fe[Q];
                b->den[c] = fl->denIn;
                or_evaluate_velocity(fl, b->blktime, zc, yc, xc, v);
                b->u[c] = v[0]; b->u[c + n] = v[1]; b->u[c + 2 * n] = v[2];
                or_feq_dist(b->den[c], v, fe);
                for (int q = 0; q < Q; q++) b->f[c + n * q] = fe[q];
            }
        }
    }
}

/* Taylor-Green vortex initial condition. Not in the reference: a build
 * addition for the periodic throughput case (u0 sin x cos y cos z, ...). */
void or_init_tgv(or_block *b, double u0, double rho0) {
    size_t n = ncell(b);
    double kx = 2.0 * PI / (double)b->X, ky = 2.0 * PI / (double)b->Y, kz = 2.0 * PI / (double)b->Z;
    for (int x = 0; x < b->X; x++)
        for (int y = 0; y < b->Y; y++)
            for (int z = 0; z < b->Z; z++) {
                double X = kx * (double)x, Y = ky * (double)y, Z = kz * (double)z;
                double v[3], fe[Q];
                v[0] = u0 * sin(X) * cos(Y) * cos(Z);
                v[1] = -u0 * cos(X) * sin(Y) * cos(Z);
                v[2] = 0.0;
                double p = rho0 * u0 * u0 / 16.0 * (cos(2.0 * X) + cos(2.0 * Y)) * (cos(2.0 * Z) + 2.0);
                double rho = rho0 + 3.0 * p;
                size_t c = cidx(b, z, y, x);
                b->den[c] = rho;
                b->u[c] = v[0]; b->u[c + n] = v[1]; b->u[c + 2 * n] = v[2];
                or_feq_dist(rho, v, fe);
                for (int q = 0; q < Q; q++) b->f[c + n * q] = fe[q];
            }
}

/* update_volume_force_, FluidDomain.f90:1174-1180 */
void or_update_volume_force(or_block *b, const or_flow *fl) {
    b->volumeForce[0] = fl->volumeForceIn[0] +
        fl->volumeForceAmp * sin(((2.0 * PI) * fl->volumeForceFreq) * b->blktime + (fl->volumeForcePhi / 180.0) * PI);
    b->volumeForce[1] = fl->volumeForceIn[1];
    b->volumeForce[2] = fl->volumeForceIn[2];
}

/* calculate_macro_quantities_, FluidDomain.f90:1128-1145 */
void or_macro(or_block *b) {
    size_t n = ncell(b);
    const double *vf = b->volumeForce;
    #pragma omp parallel for schedule(static)
    for (int x = 0; x < b->X; x++)
        for (int y = 0; y < b->Y; y++)
            for (int z = 0; z < b->Z; z++) {
                size_t c = cidx(b, z, y, x);
                double s = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
                for (int q = 0; q < Q; q++) s += b->f[c + n * q];
                for (int q = 0; q < Q; q++) sx += b->f[c + n * q] * (double)EX[q];
                for (int q = 0; q < Q; q++) sy += b->f[c + n * q] * (double)EY[q];
                for (int q = 0; q < Q; q++) sz += b->f[c + n * q] * (double)EZ[q];
                b->den[c] = s;
                b->u[c] = (sx + (0.5 * vf[0]) * b->dh) / b->den[c];
                b->u[c + n] = (sy + (0.5 * vf[1]) * b->dh) / b->den[c];
                b->u[c + 2 * n] = (sz + (0.5 * vf[2]) * b->dh) / b->den[c];
            }
}

/* ResetVolumeForce_ / add_volume_force_, FluidDomain.f90:1182-1206: x-slabs
 * shared among the threads as the reference's OpenMP loops share them */
void or_reset_force(or_block *b) {
    size_t n = ncell(b), slab = (size_t)b->Y * b->Z;
    #pragma omp parallel for schedule(static)
    for (int x = 0; x < b->X; x++)
        for (int k = 0; k < 3; k++) memset(b->force + n * k + slab * x, 0, sizeof(double) * slab);
}
void or_add_force(or_block *b) {
    size_t n = ncell(b), slab = (size_t)b->Y * b->Z;
    const double *vf = b->volumeForce;
    #pragma omp parallel for schedule(static)
    for (int x = 0; x < b->X; x++)
        for (int k = 0; k < 3; k++) {
            double *f = b->force + n * k + slab * x;
            for (size_t i = 0; i < slab; i++) f[i] = f[i] + vf[k];
        }
}

/* ConstParams.f90:19-20: the TRT population pairs */
static const int POSD[9] = {1, 3, 5, 7, 8, 11, 12, 15, 16};
static const int NEGD[9] = {2, 4, 6, 10, 9, 14, 13, 18, 17};

/* ConstParams.f90:40-45, each product rounded in turn as the parameter
 * expressions are evaluated */
static double les_const(int model) {
    const double Csmag = 0.17, CWALE = 0.50;
    if (model == 11) return ((2.0 * Csmag) * Csmag) * sqrt(2.0) * 9.0;
    if (model == 14) return CWALE * CWALE;
    return (2.5 * Csmag) * Csmag;
}

/* the non-equilibrium stress sums of smag/WALE (FluidDomain.f90:1271-1276) */
static void neq_stress(const double fn[Q], double q[6]) {
    q[0] = fn[1] + fn[2] + fn[7] + fn[8] + fn[9] + fn[10] + fn[11] + fn[12] + fn[13] + fn[14];
    q[1] = fn[3] + fn[4] + fn[7] + fn[8] + fn[9] + fn[10] + fn[15] + fn[16] + fn[17] + fn[18];
    q[2] = fn[5] + fn[6] + fn[11] + fn[12] + fn[13] + fn[14] + fn[15] + fn[16] + fn[17] + fn[18];
    q[3] = fn[7] - fn[8] - fn[9] + fn[10];
    q[4] = fn[11] - fn[12] - fn[13] + fn[14];
    q[5] = fn[15] - fn[16] - fn[17] + fn[18];
}

/* smag, FluidDomain.f90:1265-1281 */
static double les_smag(const or_block *b, const double fEq[Q], double rho, size_t c) {
    double fn[Q], q[6];
    for (int i = 0; i < Q; i++) fn[i] = -fEq[i];
    neq_stress(fn, q);
    double QQ = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + 2.0 * (q[3] * q[3] + q[4] * q[4] + q[5] * q[5]);
    double tau_t = sqrt(b->tau * b->tau + les_const(11) * sqrt(QQ) / rho);
    b->tau_all[c] = 0.5 * (b->tau + tau_t);
    return 2.0 / (b->tau + tau_t);
}

/* center_diff / onesid_diff and the interior / first / last branch of
 * WALE and vrem (FluidDomain.f90:1343-1388, 1425-1471, 1482-1491):
 * derivative of velocity component k along axis d at cell (z,y,x). The
 * reference multiplies by its invdh = dh. */
static double les_diff(const or_block *b, int k, int d, int z, int y, int x) {
    size_t n = ncell(b);
    const double *u = b->u + n * k;
    int p[3] = {x, y, z}, D[3] = {b->X, b->Y, b->Z};
    int i = p[d];
    size_t s = (d == 0) ? (size_t)b->Z * b->Y : (d == 1 ? (size_t)b->Z : 1);
    size_t c = cidx(b, z, y, x);
    double inv = b->dh;
    if (i > 0 && i < D[d] - 1) return (u[c + s] - u[c - s]) * inv;
    if (i == 0) return ((-(3.0 * u[c]) + 4.0 * u[c + s]) - u[c + 2 * s]) * inv;
    return ((-(3.0 * u[c]) + 4.0 * u[c - s]) - u[c - 2 * s]) * inv;
}

/* WALE, FluidDomain.f90:1304-1416 */
static double les_wale(const or_block *b, const double fEq[Q], double rho, int z, int y, int x, size_t c) {
    double fn[Q], q[6];
    for (int i = 0; i < Q; i++) fn[i] = -fEq[i];
    neq_stress(fn, q);
    double invdh = b->dh, tau_ = b->tau_all[c];
    double S11 = -(1.5 * invdh * q[0] / (rho * tau_));
    double S22 = -(1.5 * invdh * q[1] / (rho * tau_));
    double S33 = -(1.5 * invdh * q[2] / (rho * tau_));
    double S12 = -(1.5 * invdh * q[3] / (rho * tau_));
    double S13 = -(1.5 * invdh * q[4] / (rho * tau_));
    double S23 = -(1.5 * invdh * q[5] / (rho * tau_));
    double S = S11 * S11 + S22 * S22 + S33 * S33 + 2.0 * (S12 * S12 + S13 * S13 + S23 * S23);
    double ox = les_diff(b, 2, 1, z, y, x);
    ox = 0.5 * (ox - les_diff(b, 1, 2, z, y, x));
    double oy = les_diff(b, 0, 2, z, y, x);
    oy = 0.5 * (oy - les_diff(b, 2, 0, z, y, x));
    double oz = les_diff(b, 1, 0, z, y, x);
    oz = 0.5 * (oz - les_diff(b, 0, 1, z, y, x));
    double O12 = -(0.5 * oz), O13 = 0.5 * oy, O23 = -(0.5 * ox);
    double O = 2.0 * (O12 * O12 + O23 * O23 + O13 * O13);
    /* the reference's 0.0d0 terms change nothing but the sign of a zero sum,
     * which reaches no output (a zero SdSd gives OP = 0 either way) */
    double SO11 = -(S11 * S11 * O12 * O12 + S11 * S11 * O13 * O13 + S12 * S12 * O12 * O12 +
                    S12 * S12 * O13 * O13 + S13 * S13 * O12 * O12 + S13 * S13 * O13 * O13);
    double SO22 = -(S12 * S12 * O12 * O12 + S12 * S12 * O23 * O23 + S22 * S22 * O12 * O12 +
                    S22 * S22 * O23 * O23 + S23 * S23 * O12 * O12 + S23 * S23 * O23 * O23);
    double SO33 = -(S13 * S13 * O13 * O13 + S13 * S13 * O23 * O23 + S23 * S23 * O13 * O13 +
                    S23 * S23 * O23 * O23 + S33 * S33 * O13 * O13 + S33 * S33 * O23 * O23);
    double SO12 = -(S11 * S12 * O13 * O23 + S12 * S22 * O13 * O23 + S13 * S23 * O13 * O23);
    double SO13 = (S11 * S13 * O12 * O23 + S12 * S23 * O12 * O23 + S13 * S33 * O12 * O23);
    double SO23 = -(S12 * S13 * O12 * O13 + S22 * S23 * O12 * O13 + S23 * S33 * O12 * O13);
    double SO = SO11 + SO22 + SO33 + 2.0 * (SO12 + SO13 + SO23);
    double SdSd = (S * S + O * O) / 6.0 + 2.0 * S * O / 3.0 + 2.0 * SO;
    double OP = pow(SdSd, 1.5) / (pow(S, 2.5) + pow(SdSd, 1.25));
    if (!isfinite(OP) || OP < 0.0) OP = 0.0;
    double t = (b->nu + les_const(14) * OP * b->dh * b->dh) / (b->dh * CS2) + 0.5;
    b->tau_all[c] = t;
    return 1.0 / t;
}

/* vrem, FluidDomain.f90:1428-1506 */
static double les_vrem(const or_block *b, int z, int y, int x, size_t c) {
    double a[3][3];  /* a[i][j]: derivative of component i along axis j, halved */
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) a[i][j] = 0.5 * les_diff(b, i, j, z, y, x);
    double bq[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) bq[i][j] = a[i][j] * a[i][j];
    double aa = bq[0][0] + bq[0][1] + bq[0][2] + bq[1][0] + bq[1][1] + bq[1][2] + bq[2][0] + bq[2][1] + bq[2][2];
    double r0 = bq[0][0] + bq[0][1] + bq[0][2], r1 = bq[1][0] + bq[1][1] + bq[1][2], r2 = bq[2][0] + bq[2][1] + bq[2][2];
    double d01 = a[0][0] * a[1][0] + a[0][1] * a[1][1] + a[0][2] * a[1][2];
    double d02 = a[0][0] * a[2][0] + a[0][1] * a[2][1] + a[0][2] * a[2][2];
    double d12 = a[1][0] * a[2][0] + a[1][1] * a[2][1] + a[1][2] * a[2][2];
    double bb = r0 * r1 - d01 * d01 + r0 * r2 - d02 * d02 + r1 * r2 - d12 * d12;
    double OP = sqrt(bb / aa);
    if (!isfinite(OP)) OP = 0.0;
    double t = (b->nu + les_const(15) * OP * b->dh * b->dh) / (b->dh * CS2) + 0.5;
    b->tau_all[c] = t;
    return 1.0 / t;
}

/* collision_, FluidDomain.f90:1208-1262: SRT (1), TRT (2), MRT (3) and the
 * SRT collisions with a per-cell rate: Smagorinsky (11), WALE (14), Vreman
 * (15). RBGK (12) reads an uninitialised rate and ELBM (13) an uninitialised
 * array (x3), so neither has a defined result to restate. */
void or_collide(or_block *b) {
    size_t n = ncell(b);
    double dt3 = 3.0 * b->dh;
    #pragma omp parallel for schedule(static)
    for (int x = 0; x < b->X; x++)
        for (int y = 0; y < b->Y; y++)
            for (int z = 0; z < b->Z; z++) {
                size_t c = cidx(b, z, y, x);
                double u0 = b->u[c], u1 = b->u[c + n], u2 = b->u[c + 2 * n];
                double F0 = b->force[c], F1 = b->force[c + n], F2 = b->force[c + 2 * n];
                double den = b->den[c];
                double uSqr = (u0 * u0 + u1 * u1) + u2 * u2;
                double fEq[Q], Flb[Q];
                for (int i = 0; i < Q; i++) {
                    double ex = EX[i], ey = EY[i], ez = EZ[i];
                    double uxyz = (u0 * ex + u1 * ey) + u2 * ez;
                    fEq[i] = ((WT[i] * den) * ((1.0 - 1.5 * uSqr) + uxyz * (3.0 + 4.5 * uxyz))) - b->f[c + n * i];
                    Flb[i] = (dt3 * WT[i]) * (((((ex - u0) + (3.0 * uxyz) * ex) * F0) +
                                                (((ey - u1) + (3.0 * uxyz) * ey) * F1)) +
                                               (((ez - u2) + (3.0 * uxyz) * ez) * F2));
                }
                if (b->model == 1) {
                    for (int i = 0; i < Q; i++)
                        b->f[c + n * i] = (b->f[c + n * i] + b->omega * fEq[i]) + (1.0 - 0.5 * b->omega) * Flb[i];
                } else if (b->model == 3) {
                    for (int i = 0; i < Q; i++) {
                        double a = 0.0, bb = 0.0;
                        for (int j = 0; j < Q; j++) a += b->mc[i + Q * j] * fEq[j];
                        for (int j = 0; j < Q; j++) bb += b->mf[i + Q * j] * Flb[j];
                        b->f[c + n * i] = (b->f[c + n * i] + a) + bb;
                    }
                } else if (b->model == 2) {
                    const double om = b->omega, om2 = b->omega2;
                    double d[Q];
                    d[0] = om * fEq[0] + (1.0 - 0.5 * om) * Flb[0];
                    for (int k = 0; k < 9; k++) {
                        int p = POSD[k], m = NEGD[k];
                        double sp = 0.5 * om * (fEq[p] + fEq[m]) + (0.5 - 0.25 * om) * (Flb[p] + Flb[m]);
                        double sm = 0.5 * om2 * (fEq[p] - fEq[m]) + (0.5 - 0.25 * om2) * (Flb[p] - Flb[m]);
                        d[p] = sp + sm;
                        d[m] = sp - sm;
                    }
                    for (int i = 0; i < Q; i++) b->f[c + n * i] = b->f[c + n * i] + d[i];
                } else if (b->model == 11 || b->model == 14 || b->model == 15) {
                    double om = (b->model == 11) ? les_smag(b, fEq, den, c)
                              : (b->model == 14) ? les_wale(b, fEq, den, z, y, x, c)
                              : les_vrem(b, z, y, x, c);
                    for (int i = 0; i < Q; i++)
                        b->f[c + n * i] = (b->f[c + n * i] + om * fEq[i]) + (1.0 - 0.5 * om) * Flb[i];
                }
            }
}

/* face geometry helpers: face k = 2*axis + side */
static int face_dims(const or_block *b, int k, int *A, int *B) {
    int ax = k / 2;
    if (ax == 0) { *A = b->Z; *B = b->Y; }
    else if (ax == 1) { *A = b->Z; *B = b->X; }
    else { *A = b->Y; *B = b->X; }
    return ax;
}
/* cell (z,y,x) of face k at face-plane coordinates (a,b) and layer l (0 = boundary) */
static size_t face_cell(const or_block *b, int k, int a, int bb, int l) {
    int ax = k / 2, side = k % 2;
    if (ax == 0) { int x = side ? b->X - 1 - l : l; return cidx(b, a, bb, x); }
    if (ax == 1) { int y = side ? b->Y - 1 - l : l; return cidx(b, a, y, bb); }
    { int z = side ? b->Z - 1 - l : l; return cidx(b, z, a, bb); }
}

/* halfwayBCset_, FluidDomain.f90:567-614 */
void or_halfway_set(or_block *b) {
    size_t n = ncell(b);
    for (int k = 0; k < 6; k++) {
        if (!(b->bnd[k] == 203 || b->bnd[k] == 204) || !b->hw[k]) continue;
        int A, B;
        face_dims(b, k, &A, &B);
        for (int bb = 0; bb < B; bb++)
            for (int a = 0; a < A; a++) {
                size_t c = face_cell(b, k, a, bb, 0);
                double *h = b->hw[k] + (size_t)Q * ((size_t)a + (size_t)A * bb);
                for (int q = 0; q < Q; q++) h[q] = b->f[c + n * q];
            }
    }
}

/* streaming_, FluidDomain.f90:1514-1625: every population shifts by e_i with
 * periodic wrap in all three axes. A pull copy through tmp and back moves the
 * same values as the reference's in-place cyclic shifts, with the same two
 * passes over each moving population, shared among the threads by x-slabs as
 * the reference's OpenMP loops are; the rest population (q = 0) stays. */
void or_stream(or_block *b, double *tmp) {
    size_t n = ncell(b), slab = (size_t)b->Y * b->Z;
    int X = b->X, Y = b->Y, Z = b->Z;
    for (int q = 1; q < Q; q++) {
        #pragma omp parallel for schedule(static)
        for (int x = 0; x < X; x++) {
            int xs = (x - EX[q] + X) % X;
            for (int y = 0; y < Y; y++) {
                int ys = (y - EY[q] + Y) % Y;
                for (int z = 0; z < Z; z++) {
                    int zs = (z - EZ[q] + Z) % Z;
                    tmp[cidx(b, z, y, x) + n * q] = b->f[cidx(b, zs, ys, xs) + n * q];
                }
            }
        }
        #pragma omp parallel for schedule(static)
        for (int x = 0; x < X; x++)
            memcpy(b->f + n * q + slab * x, tmp + n * q + slab * x, sizeof(double) * slab);
    }
}

/* velocity point of face cell (a,b) of face k, shifted outward by `off` */
static void face_velocity(const or_block *b, const or_flow *fl, int k, int a, int bb, double off, double v[3]) {
    int ax = k / 2, side = k % 2;
    double sgn = side ? 1.0 : -1.0;
    if (ax == 0) {
        double zc = b->zmin + b->dh * (double)a, yc = b->ymin + b->dh * (double)bb;
        double xc = side ? b->xmax : b->xmin;
        if (off != 0.0) xc = side ? b->xmax + b->dh * 0.5 : b->xmin - b->dh * 0.5;
        or_evaluate_velocity(fl, b->blktime, zc, yc, xc, v);
    } else if (ax == 1) {
        double zc = b->zmin + b->dh * (double)a, xc = b->xmin + b->dh * (double)bb;
        double yc = side ? b->ymax : b->ymin;
        if (off != 0.0) yc = side ? b->ymax + b->dh * 0.5 : b->ymin - b->dh * 0.5;
        or_evaluate_velocity(fl, b->blktime, zc, yc, xc, v);
    } else {
        double yc = b->ymin + b->dh * (double)a, xc = b->xmin + b->dh * (double)bb;
        double zc = side ? b->zmax : b->zmin;
        if (off != 0.0) zc = side ? b->zmax + b->dh * 0.5 : b->zmin - b->dh * 0.5;
        or_evaluate_velocity(fl, b->blktime, zc, yc, xc, v);
    }
    (void)sgn;
}

/* set_boundary_conditions_, FluidDomain.f90:616-1126: faces x-, x+, y-, y+,
 * z-, z+ in that order, so edges and corners keep the last writer. */
int or_set_bc(or_block *b, const or_flow *fl) {
    size_t n = ncell(b);
    for (int k = 0; k < 6; k++) {
        int code = b->bnd[k];
        int A, B;
        face_dims(b, k, &A, &B);
        if (code == 301 || code == 0 || code == 1) continue;
        if (code == 203 || code == 204) {
            if (!b->hw_ready[k]) { b->hw_ready[k] = 1; continue; }
        }
        if (!(code == 101 || code == 102 || code == 103 || code == 104 || code == 201 ||
              code == 202 || code == 203 || code == 204 || code == 302))
            return -1;
        for (int bb = 0; bb < B; bb++)
            for (int a = 0; a < A; a++) {
                size_t c1 = face_cell(b, k, a, bb, 0);
                double *f1 = b->f + c1;
                if (code == 101) {
                    double v[3], fe[Q];
                    face_velocity(b, fl, k, a, bb, 0.0, v);
                    or_feq_dist(fl->denIn, v, fe);
                    for (int q = 0; q < Q; q++) f1[n * q] = fe[q];
                } else if (code == 102) {
                    size_t c2 = face_cell(b, k, a, bb, 1);
                    double v[3], fe[Q], fi[Q], u2[3];
                    face_velocity(b, fl, k, a, bb, 0.0, v);
                    or_feq_dist(fl->denIn, v, fe);
                    u2[0] = b->u[c2]; u2[1] = b->u[c2 + n]; u2[2] = b->u[c2 + 2 * n];
                    or_feq_dist(b->den[c2], u2, fi);
                    for (int j = 0; j < 5; j++) {
                        int q = INC[k][j];
                        f1[n * q] = fe[q] + (b->f[c2 + n * q] - fi[q]);
                    }
                } else if (code == 103) {
                    size_t c2 = face_cell(b, k, a, bb, 1);
                    for (int j = 0; j < 5; j++) { int q = INC[k][j]; f1[n * q] = b->f[c2 + n * q]; }
                } else if (code == 104) {
                    size_t c2 = face_cell(b, k, a, bb, 1), c3 = face_cell(b, k, a, bb, 2);
                    for (int j = 0; j < 5; j++) {
                        int q = INC[k][j];
                        f1[n * q] = 2.0 * b->f[c2 + n * q] - b->f[c3 + n * q];
                    }
                } else if (code == 201) {
                    double t[5];
                    for (int j = 0; j < 5; j++) t[j] = f1[n * OPPO[INC[k][j]]];
                    for (int j = 0; j < 5; j++) f1[n * INC[k][j]] = t[j];
                } else if (code == 203) {
                    const double *h = b->hw[k] + (size_t)Q * ((size_t)a + (size_t)A * bb);
                    for (int j = 0; j < 5; j++) f1[n * INC[k][j]] = h[OPPO[INC[k][j]]];
                } else if (code == 202) {
                    double v[3], ft[Q];
                    face_velocity(b, fl, k, a, bb, 0.0, v);
                    moving_wall(fl->denIn, v, f1, n, ft);
                    for (int j = 0; j < 5; j++) f1[n * INC[k][j]] = ft[INC[k][j]];
                } else if (code == 204) {
                    double v[3], ft[Q];
                    const double *h = b->hw[k] + (size_t)Q * ((size_t)a + (size_t)A * bb);
                    face_velocity(b, fl, k, a, bb, 1.0, v);
                    moving_wall(fl->denIn, v, h, 1, ft);
                    for (int j = 0; j < 5; j++) f1[n * INC[k][j]] = ft[INC[k][j]];
                } else if (code == 302) {
                    double t[5];
                    for (int j = 0; j < 5; j++) t[j] = f1[n * MIR[k][j]];
                    for (int j = 0; j < 5; j++) f1[n * INC[k][j]] = t[j];
                }
            }
    }
    return 0;
}

/* ---------------------------------------------------------------------------
 * Immersed boundary: UpdateElmtInterp_, PenaltyForce_, FluidVolumeForce_
 * (Solidbody.f90:760-1049) and the loop of calculate_interaction_force
 * (Solidbody.f90:869-918).
 * ------------------------------------------------------------------------- */

/* Phi, Solidbody.f90:822-833 */
static double phi4(double x) {
    double r = fabs(x);
    if (r < 1.0) return ((3.0 - 2.0 * r) + sqrt(1.0 + (4.0 * r) * (1.0 - r))) * 0.125;
    if (r < 2.0) return ((5.0 - 2.0 * r) - sqrt(-7.0 + (4.0 * r) * (3.0 - r))) * 0.125;
    return 0.0;
}

/* trimedindex, Solidbody.f90:834-866 (1-based indices) */
static int trimed(int i, int dim, int out[4], int bclo, int bchi) {
    for (int k = -1; k <= 2; k++) {
        int v = i + k;
        if (v < 1) {
            if (bclo == 301) v = v + dim;
            else if ((bclo == 302 || bclo == 201) && v == 0) v = 2;
            else if (bclo == 203 && v == 0) v = 1;
            else return -1;
        } else if (v > dim) {
            if (bchi == 301) v = v - dim;
            else if ((bchi == 302 || bchi == 201) && v == dim + 1) v = dim - 1;
            else if (bchi == 203 && v == dim + 1) v = dim;
            else return -1;
        }
        out[k + 1] = v;
    }
    return 0;
}

/* UpdateElmtInterp_, Solidbody.f90:760-807 */
int or_ib_stencil(or_body *bd, const or_block *b) {
    double invdh = 1.0 / b->dh;
    const double *p = bd->xyz;
    int i0 = (int)floor((p[0] - b->xmin) * invdh);
    double x0 = b->xmin + (double)i0 * b->dh;
    i0 = i0 + 1;
    int j0 = (int)floor((p[1] - b->ymin) * invdh);
    double y0 = b->ymin + (double)j0 * b->dh;
    j0 = j0 + 1;
    int k0 = (int)floor((p[2] - b->zmin) * invdh);
    double z0 = b->zmin + (double)k0 * b->dh;
    k0 = k0 + 1;
    for (int m = 0; m < bd->M; m++) {
        double ox = (p[3 * m] - x0) * invdh, oy = (p[3 * m + 1] - y0) * invdh, oz = (p[3 * m + 2] - z0) * invdh;
        int i = (int)floor(ox), j = (int)floor(oy), k = (int)floor(oz);
        double detx = ox - (double)i, dety = oy - (double)j, detz = oz - (double)k;
        i += i0; j += j0; k += k0;
        int ix[4], jy[4], kz[4];
        if (trimed(i, b->X, ix, b->bnd[0], b->bnd[1]) || trimed(j, b->Y, jy, b->bnd[2], b->bnd[3]) ||
            trimed(k, b->Z, kz, b->bnd[4], b->bnd[5]))
            return -1;
        int16_t *ei = bd->ei + 12 * (size_t)m;
        float *ew = bd->ew + 12 * (size_t)m;
        for (int t = 0; t < 4; t++) {
            ei[t] = (int16_t)ix[t]; ei[4 + t] = (int16_t)jy[t]; ei[8 + t] = (int16_t)kz[t];
            ew[t] = (float)phi4((double)(t - 1) - detx);
            ew[4 + t] = (float)phi4((double)(t - 1) - dety);
            ew[8 + t] = (float)phi4((double)(t - 1) - detz);
        }
    }
    return 0;
}

/* PenaltyForce_, Solidbody.f90:981-1049 */
static double penalty_body(or_body *bd, or_block *b, double denIn, double dt, double *fet) {
    size_t n = ncell(b);
    double ih = 1.0 / b->dh;
    double invh3 = ((0.5 * dt) * ((ih * ih) * ih)) / denIn;
    double tol = 0.0;
    for (int m = 0; m < bd->M; m++) {
        const int16_t *ei = bd->ei + 12 * (size_t)m;
        const float *ew = bd->ew + 12 * (size_t)m;
        double v0 = 0.0, v1 = 0.0, v2 = 0.0;
        for (int x = 0; x < 4; x++)
            for (int y = 0; y < 4; y++)
                for (int z = 0; z < 4; z++) {
                    size_t c = cidx(b, ei[8 + z] - 1, ei[4 + y] - 1, ei[x] - 1);
                    double rx = ew[x], ry = ew[4 + y], rz = ew[8 + z];
                    v0 = v0 + ((b->u[c] * rx) * ry) * rz;
                    v1 = v1 + ((b->u[c + n] * rx) * ry) * rz;
                    v2 = v2 + ((b->u[c + 2 * n] * rx) * ry) * rz;
                }
        v0 = bd->vel[3 * m] - v0;
        v1 = bd->vel[3 * m + 1] - v1;
        v2 = bd->vel[3 * m + 2] - v2;
        double a = bd->area[m];
        double F0 = v0 * a, F1 = v1 * a, F2 = v2 * a;
        tol = ((tol + fabs(v0)) + fabs(v1)) + fabs(v2);
        bd->eforce[3 * m] += F0;
        bd->eforce[3 * m + 1] += F1;
        bd->eforce[3 * m + 2] += F2;
        fet[3 * m] = F0 * invh3; fet[3 * m + 1] = F1 * invh3; fet[3 * m + 2] = F2 * invh3;
    }
    for (int m = 0; m < bd->M; m++) {
        const int16_t *ei = bd->ei + 12 * (size_t)m;
        const float *ew = bd->ew + 12 * (size_t)m;
        for (int x = 0; x < 4; x++)
            for (int y = 0; y < 4; y++)
                for (int z = 0; z < 4; z++) {
                    size_t c = cidx(b, ei[8 + z] - 1, ei[4 + y] - 1, ei[x] - 1);
                    double rx = ew[x], ry = ew[4 + y], rz = ew[8 + z];
                    b->u[c] = b->u[c] - ((fet[3 * m] * rx) * ry) * rz;
                    b->u[c + n] = b->u[c + n] - ((fet[3 * m + 1] * rx) * ry) * rz;
                    b->u[c + 2 * n] = b->u[c + 2 * n] - ((fet[3 * m + 2] * rx) * ry) * rz;
                }
    }
    return tol;
}

/* calculate_interaction_force loop, Solidbody.f90:889-906 */
void or_ib_penalty(or_body *bd, int nb, or_block *b, double denIn, double dt, double Uref,
                   int ntol, double dtol, int *iters, double *residual) {
    int maxM = 0;
    for (int i = 0; i < nb; i++) {
        if (bd[i].M > maxM) maxM = bd[i].M;
        memset(bd[i].eforce, 0, sizeof(double) * 3 * bd[i].M);
    }
    double *fet = (double *)malloc(sizeof(double) * 3 * (maxM > 0 ? maxM : 1));
    int it = 0;
    double dmax = 1e10;
    if (nb > 0) {
        while (it < ntol && dmax > dtol) {
            dmax = 0.0;
            double dsum = 0.0;
            for (int i = 0; i < nb; i++) {
                double tol = penalty_body(&bd[i], b, denIn, dt, fet);
                dmax = dmax + tol;
                dsum = dsum + (double)bd[i].M;
            }
            dmax = dmax / (dsum * Uref);
            it = it + 1;
        }
    }
    free(fet);
    if (iters) *iters = it;
    if (residual) *residual = dmax;
}

/* FluidVolumeForce_ spreading part, Solidbody.f90:936-977 */
void or_ib_spread(or_body *bd, int nb, or_block *b) {
    size_t n = ncell(b);
    double ih = 1.0 / b->dh;
    double invh3 = (ih * ih) * ih;
    for (int i = 0; i < nb; i++) {
        or_body *B = &bd[i];
        for (int m = 0; m < B->M; m++) {
            const int16_t *ei = B->ei + 12 * (size_t)m;
            const float *ew = B->ew + 12 * (size_t)m;
            double f0 = B->eforce[3 * m] * invh3, f1 = B->eforce[3 * m + 1] * invh3, f2 = B->eforce[3 * m + 2] * invh3;
            for (int x = 0; x < 4; x++)
                for (int y = 0; y < 4; y++)
                    for (int z = 0; z < 4; z++) {
                        size_t c = cidx(b, ei[8 + z] - 1, ei[4 + y] - 1, ei[x] - 1);
                        double rx = ew[x], ry = ew[4 + y], rz = ew[8 + z];
                        b->force[c] = b->force[c] + (-(((f0 * rx) * ry) * rz));
                        b->force[c + n] = b->force[c + n] + (-(((f1 * rx) * ry) * rz));
                        b->force[c + 2 * n] = b->force[c + 2 * n] + (-(((f2 * rx) * ry) * rz));
                    }
        }
    }
}

/* tree_collision_streaming_IBM_FEM for a block without sons,
 * LBMBlockComm.f90:279-305 (the structural solve is the caller's). */
int or_step(or_block *b, const or_flow *fl, or_body *bd, int nb, double Uref,
            int ntol, double dtol, double *tmp, int *iters, double *residual) {
    or_update_volume_force(b, fl);
    or_macro(b);
    or_reset_force(b);
    if (iters) *iters = 0;
    if (residual) *residual = 0.0;
    if (nb > 0) {
        for (int i = 0; i < nb; i++)
            if (or_ib_stencil(&bd[i], b)) return -2;
        or_ib_penalty(bd, nb, b, fl->denIn, b->dh, Uref, ntol, dtol, iters, residual);
        or_ib_spread(bd, nb, b);
    }
    or_add_force(b);
    or_collide(b);
    or_halfway_set(b);
    or_stream(b, tmp);
    return or_set_bc(b, fl);
}

/* ComputeFieldStat_, FluidDomain.f90:1739-1768 (sequential sums) */
void or_field_stat(const or_block *b, double Uref, double l2[3], double linf[3]) {
    size_t n = ncell(b);
    double inv = 1.0 / Uref;
    for (int k = 0; k < 3; k++) {
        double s = 0.0, m = -1.0;
        for (int x = 0; x < b->X; x++)
            for (int y = 0; y < b->Y; y++)
                for (int z = 0; z < b->Z; z++) {
                    double t = fabs(b->u[cidx(b, z, y, x) + n * k] * inv);
                    s = s + t * t;
                    if (t > m) m = t;
                }
        l2[k] = sqrt(s / (((double)b->X * (double)b->Y) * (double)b->Z));
        linf[k] = m;
    }
}

/* ---------------------------------------------------------------------------
 * Block refinement (LBMBlockComm.f90:32-96, 340-505, 546-979)
 * ------------------------------------------------------------------------- */

/* build_blocks_comunication for one father/son pair, LBMBlockComm.f90:42-92 */
void or_build_pair(const or_block *fa, const or_block *so, or_pair *p) {
    for (int j = 0; j < 6; j++) p->sds[j] = (so->bnd[j] == 0) ? ((j % 2 == 0) ? 1 : -1) : 0;
    int sxD = so->X, syD = so->Y, szD = so->Z;
    if (so->periodic[0]) sxD -= 1;
    if (so->periodic[1]) syD -= 1;
    if (so->periodic[2]) szD -= 1;
    p->s[0] = 1; p->s[2] = 1; p->s[4] = 1;
    p->s[1] = sxD; p->s[3] = syD; p->s[5] = szD;
    p->f[0] = (int)floor((so->xmin - fa->xmin) / fa->dh + 1.5);
    p->f[2] = (int)floor((so->ymin - fa->ymin) / fa->dh + 1.5);
    p->f[4] = (int)floor((so->zmin - fa->zmin) / fa->dh + 1.5);
    int ratio = (int)floor(fa->dh / so->dh + 0.5);
    sxD = (sxD - 1) / ratio; syD = (syD - 1) / ratio; szD = (szD - 1) / ratio;
    p->f[1] = p->f[0] + sxD; p->f[3] = p->f[2] + syD; p->f[5] = p->f[4] + szD;
    for (int j = 0; j < 6; j++) { p->si[j] = p->s[j] + p->sds[j] * ratio; p->fi[j] = p->f[j] + p->sds[j]; }
    p->xDimS = so->X; p->xDimF = p->f[1] - p->f[0] + 1;
    p->yDimS = so->Y; p->yDimF = p->f[3] - p->f[2] + 1;
    p->zDimS = so->Z; p->zDimF = p->f[5] - p->f[4] + 1;
}

/* father face-plane dims (a fastest) of son face k */
static void pair_face_dims(const or_pair *p, int k, int *A, int *B) {
    int ax = k / 2;
    if (ax == 0) { *A = p->zDimF; *B = p->yDimF; }
    else if (ax == 1) { *A = p->zDimF; *B = p->xDimF; }
    else { *A = p->yDimF; *B = p->xDimF; }
}
static void pair_son_dims(const or_pair *p, int k, int *A, int *B) {
    int ax = k / 2;
    if (ax == 0) { *A = p->zDimS; *B = p->yDimS; }
    else if (ax == 1) { *A = p->zDimS; *B = p->xDimS; }
    else { *A = p->yDimS; *B = p->xDimS; }
}

/* extract_interpolate_layer, LBMBlockComm.f90:340-505. Buffers are
 * (0:18, A, B) per face and time level, tau buffers (A, B). */
void or_extract_layer(const or_block *fa, const or_block *so, const or_pair *p, int time,
                      double *buf_f[6][2], double *buf_tau[6][2]) {
    size_t n = ncell(fa);
    for (int k = 0; k < 6; k++) {
        if (so->bnd[k] != 0) continue;
        int A, B, ax = k / 2;
        pair_face_dims(p, k, &A, &B);
        double *bf = buf_f[k][time - 1], *bt = buf_tau[k][time - 1];
        for (int bb = 0; bb < B; bb++)
            for (int a = 0; a < A; a++) {
                int xF, yF, zF;
                if (ax == 0) { xF = p->f[k]; yF = bb + p->f[2]; zF = a + p->f[4]; }
                else if (ax == 1) { yF = p->f[k]; xF = bb + p->f[0]; zF = a + p->f[4]; }
                else { zF = p->f[k]; xF = bb + p->f[0]; yF = a + p->f[2]; }
                size_t c = cidx(fa, zF - 1, yF - 1, xF - 1);
                for (int e = 0; e < Q; e++) bf[e + Q * ((size_t)a + (size_t)A * bb)] = fa->f[c + n * e];
                bt[(size_t)a + (size_t)A * bb] = fa->tau_all[c];
            }
        if (time == 2) {
            double *t1 = buf_f[k][0], *t2 = buf_f[k][1];
            for (size_t i = 0; i < (size_t)Q * A * B; i++) t1[i] = 0.5 * (t1[i] + t2[i]);
            double *u1 = buf_tau[k][0], *u2 = buf_tau[k][1];
            for (size_t i = 0; i < (size_t)A * B; i++) u1[i] = 0.5 * (u1[i] + u2[i]);
        }
    }
}

/* interpolate_fIn / interpolate_tau, LBMBlockComm.f90:808-956. fF(nq,bF,aF),
 * fS(nq,bS,aS), column-major, 1-based loops. */
#define FF(q, b_, a_) fF[(q) + nq * (((b_) - 1) + (size_t)bF * ((a_) - 1))]
#define FS(q, b_, a_) fS[(q) + nq * (((b_) - 1) + (size_t)bS * ((a_) - 1))]
static void interp_face(int nq, int bF, int aF, const double *fF, int bS, int aS, double *fS, int scheme) {
    int r1 = 0, r2 = 0, bSt = bS, aSt = aS;
    if (bS % 2 == 0) { bSt = bS - 1; r2 = 1; }
    if (aS % 2 == 0) { aSt = aS - 1; r1 = 1; }
    (void)aF;
    if (scheme == 2) {
        for (int b = 1; b <= bSt; b += 2) {
            int b1 = b / 2 + 1;
            for (int a = 1; a <= aSt; a += 2) {
                int a1 = a / 2 + 1;
                for (int q = 0; q < nq; q++) {
                    FS(q, b, a) = FF(q, b1, a1);
                    if (b == 1)
                        FS(q, b + 1, a) = (0.375 * FF(q, b1, a1) + 0.75 * FF(q, b1 + 1, a1)) - 0.125 * FF(q, b1 + 2, a1);
                    else if (b == bSt - 2)
                        FS(q, b + 1, a) = (0.375 * FF(q, b1 + 1, a1) + 0.75 * FF(q, b1, a1)) - 0.125 * FF(q, b1 - 1, a1);
                    else if (b != bSt)
                        FS(q, b + 1, a) = (((-(0.0625 * FF(q, b1 - 1, a1))) + 0.5625 * FF(q, b1, a1)) + 0.5625 * FF(q, b1 + 1, a1)) - 0.0625 * FF(q, b1 + 2, a1);
                }
            }
        }
        for (int b = 1; b <= bSt; b++)
            for (int a = 2; a <= aSt; a += 2)
                for (int q = 0; q < nq; q++) {
                    if (a == 2)
                        FS(q, b, a) = (0.375 * FS(q, b, a - 1) + 0.75 * FS(q, b, a + 1)) - 0.125 * FS(q, b, a + 3);
                    else if (a == aSt - 1)
                        FS(q, b, a) = (0.375 * FS(q, b, a + 1) + 0.75 * FS(q, b, a - 1)) - 0.125 * FS(q, b, a - 3);
                    else
                        FS(q, b, a) = (((-(0.0625 * FS(q, b, a - 3))) + 0.5625 * FS(q, b, a - 1)) + 0.5625 * FS(q, b, a + 1)) - 0.0625 * FS(q, b, a + 3);
                }
        if (r2)
            for (int a = 1; a <= aSt; a++)
                for (int q = 0; q < nq; q++)
                    FS(q, bSt + 1, a) = (((-(0.0625 * FS(q, bSt - 2, a))) + 0.5625 * FS(q, bSt, a)) + 0.5625 * FS(q, 1, a)) - 0.0625 * FS(q, 3, a);
        if (r1) {
            for (int b = 1; b <= bSt; b++)
                for (int q = 0; q < nq; q++)
                    FS(q, b, aSt + 1) = (((-(0.0625 * FS(q, b, aSt - 2))) + 0.5625 * FS(q, b, aSt)) + 0.5625 * FS(q, b, 1)) - 0.0625 * FS(q, b, 3);
            if (r2)
                for (int q = 0; q < nq; q++)
                    FS(q, bSt + 1, aSt + 1) = (((-(0.0625 * FS(q, bSt + 1, aSt - 2))) + 0.5625 * FS(q, bSt + 1, aSt)) + 0.5625 * FS(q, bSt + 1, 1)) - 0.0625 * FS(q, bSt + 1, 3);
        }
    } else {
        for (int b = 1; b <= bSt; b += 2) {
            int b1 = b / 2 + 1;
            for (int a = 1; a <= aSt; a += 2) {
                int a1 = a / 2 + 1;
                for (int q = 0; q < nq; q++) {
                    FS(q, b, a) = FF(q, b1, a1);
                    if (b < bSt) FS(q, b + 1, a) = (FF(q, b1, a1) + FF(q, b1 + 1, a1)) * 0.5;
                }
            }
        }
        for (int b = 1; b <= bSt; b++)
            for (int a = 2; a <= aSt; a += 2)
                for (int q = 0; q < nq; q++) FS(q, b, a) = (FS(q, b, a - 1) + FS(q, b, a + 1)) * 0.5;
        if (r2)
            for (int a = 1; a <= aSt; a++)
                for (int q = 0; q < nq; q++) FS(q, bSt + 1, a) = (FS(q, bSt, a) + FS(q, 1, a)) * 0.5;
        if (r1) {
            for (int b = 1; b <= bSt; b++)
                for (int q = 0; q < nq; q++) FS(q, b, aSt + 1) = (FS(q, b, aSt) + FS(q, b, 1)) * 0.5;
            if (r2)
                for (int q = 0; q < nq; q++) FS(q, bSt + 1, aSt + 1) = (FS(q, bSt + 1, aSt) + FS(q, bSt + 1, 1)) * 0.5;
        }
    }
}
#undef FF
#undef FS

/* fIn_GridTransform, LBMBlockComm.f90:958-979 */
void or_grid_transform(double fin[Q], double coeff, const double vf[3], double dh) {
    double den = 0.0, s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int q = 0; q < Q; q++) den += fin[q];
    for (int q = 0; q < Q; q++) s0 += fin[q] * (double)EX[q];
    for (int q = 0; q < Q; q++) s1 += fin[q] * (double)EY[q];
    for (int q = 0; q < Q; q++) s2 += fin[q] * (double)EZ[q];
    double u0 = (s0 + (0.5 * vf[0]) * dh) / den;
    double u1 = (s1 + (0.5 * vf[1]) * dh) / den;
    double u2 = (s2 + (0.5 * vf[2]) * dh) / den;
    double uSqr = (u0 * u0 + u1 * u1) + u2 * u2;
    for (int i = 0; i < Q; i++) {
        double uxyz = (u0 * (double)EX[i] + u1 * (double)EY[i]) + u2 * (double)EZ[i];
        double fEq = (WT[i] * den) * ((1.0 - 1.5 * uSqr) + uxyz * (3.0 + 4.5 * uxyz));
        fin[i] = fEq + coeff * (fin[i] - fEq);
    }
}

/* interpolation_father_to_son, LBMBlockComm.f90:655-806 */
void or_interp_f2s(or_block *so, const or_block *fa, const or_pair *p, int n_timeStep,
                   double *buf_f[6][2], double *buf_tau[6][2], int scheme) {
    size_t n = ncell(so);
    for (int k = 0; k < 6; k++) {
        if (p->sds[k] == 0) continue;
        int AF, BF, AS, BS, ax = k / 2;
        pair_face_dims(p, k, &AF, &BF);
        pair_son_dims(p, k, &AS, &BS);
        double *tf = (double *)malloc(sizeof(double) * Q * (size_t)AS * BS);
        double *tt = (double *)malloc(sizeof(double) * (size_t)AS * BS);
        int lvl = (n_timeStep == 0) ? 0 : 1;
        interp_face(Q, AF, BF, buf_f[k][lvl], AS, BS, tf, scheme);
        interp_face(1, AF, BF, buf_tau[k][lvl], AS, BS, tt, 1);
        for (int bb = 0; bb < BS; bb++)
            for (int a = 0; a < AS; a++) {
                int xS, yS, zS;
                if (ax == 0) { xS = p->s[k]; yS = bb + 1; zS = a + 1; }
                else if (ax == 1) { yS = p->s[k]; xS = bb + 1; zS = a + 1; }
                else { zS = p->s[k]; xS = bb + 1; yS = a + 1; }
                size_t c = cidx(so, zS - 1, yS - 1, xS - 1);
                size_t o = (size_t)a + (size_t)AS * bb;
                double coeff = (so->tau_all[c] / tt[o]) / 2.0;
                or_grid_transform(tf + Q * o, coeff, fa->volumeForce, fa->dh);
                for (int e = 0; e < Q; e++) so->f[c + n * e] = tf[Q * o + e];
            }
        free(tf);
        free(tt);
    }
}

/* deliver_son_to_father, LBMBlockComm.f90:546-653 */
void or_deliver_s2f(or_block *fa, const or_block *so, const or_pair *p) {
    size_t nf = ncell(fa), ns = ncell(so);
    for (int k = 0; k < 6; k++) {
        int want = (k % 2 == 0) ? 1 : -1;
        if (p->sds[k] != want) continue;
        int ax = k / 2;
        int lo[3], hi[3];
        for (int d = 0; d < 3; d++) { lo[d] = p->si[2 * d]; hi[d] = p->si[2 * d + 1]; }
        int o1 = (ax == 0) ? 1 : 0, o2 = (ax == 2) ? 1 : 2;
        for (int v1 = lo[o1]; v1 <= hi[o1]; v1 += 2)
            for (int v2 = lo[o2]; v2 <= hi[o2]; v2 += 2) {
                int S[3], F[3];
                S[ax] = p->si[k]; F[ax] = p->fi[k];
                S[o1] = v1; F[o1] = (v1 - p->si[2 * o1]) / 2 + p->fi[2 * o1];
                S[o2] = v2; F[o2] = (v2 - p->si[2 * o2]) / 2 + p->fi[2 * o2];
                size_t cs = cidx(so, S[2] - 1, S[1] - 1, S[0] - 1);
                size_t cf = cidx(fa, F[2] - 1, F[1] - 1, F[0] - 1);
                double coeff = (fa->tau_all[cf] / so->tau_all[cs]) * 2.0;
                double t[Q];
                for (int e = 0; e < Q; e++) t[e] = so->f[cs + ns * e];
                or_grid_transform(t, coeff, so->volumeForce, so->dh);
                for (int e = 0; e < Q; e++) fa->f[cf + nf * e] = t[e];
            }
    }
}

/* check_is_continue's sort of the file's blocks by dh (FluidDomain.f90:151-163):
 * the exchange sort compares the dh at the original positions i and j while
 * it permutes the index list, as the reference does */
void or_continue_order(int nold, const double *dh, int *order) {
    for (int i = 0; i < nold; i++) order[i] = i;
    for (int i = 0; i < nold - 1; i++)
        for (int j = i + 1; j < nold; j++)
            if (dh[i] > dh[j]) {
                int t = order[i];
                order[i] = order[j];
                order[j] = t;
            }
}

/* check_is_continue's trilinear re-grid, FluidDomain.f90:170-226 */
void or_continue_regrid(or_block *b, int nold, const or_block *old, const int *order) {
    size_t n = ncell(b);
    #pragma omp parallel for schedule(static)
    for (int x = 0; x < b->X; x++) {
        double xc = b->xmin + (double)x * b->dh;
        for (int y = 0; y < b->Y; y++) {
            double yc = b->ymin + (double)y * b->dh;
            for (int z = 0; z < b->Z; z++) {
                double zc = b->zmin + (double)z * b->dh;
                for (int jj = 0; jj < nold; jj++) {
                    const or_block *o = &old[order[jj]];
                    double xmx = o->xmin + (double)(o->X - 1) * o->dh;
                    double ymx = o->ymin + (double)(o->Y - 1) * o->dh;
                    double zmx = o->zmin + (double)(o->Z - 1) * o->dh;
                    if (!(zc >= o->zmin && zc <= zmx && yc >= o->ymin && yc <= ymx && xc >= o->xmin && xc <= xmx))
                        continue;
                    double c1 = (xc - o->xmin) / o->dh, c2 = (yc - o->ymin) / o->dh, c3 = (zc - o->zmin) / o->dh;
                    int i1 = (int)floor(c1), i3 = (int)floor(c2), i5 = (int)floor(c3);
                    if (i1 == o->X - 1) i1 = i1 - 1;
                    if (i3 == o->Y - 1) i3 = i3 - 1;
                    if (i5 == o->Z - 1) i5 = i5 - 1;
                    c1 = c1 - (double)i1;
                    c2 = c2 - (double)i3;
                    c3 = c3 - (double)i5;
                    size_t no = (size_t)o->X * o->Y * o->Z;
                    size_t a000 = cidx(o, i5, i3, i1), a001 = cidx(o, i5, i3, i1 + 1);
                    size_t a010 = cidx(o, i5, i3 + 1, i1), a011 = cidx(o, i5, i3 + 1, i1 + 1);
                    size_t a100 = cidx(o, i5 + 1, i3, i1), a101 = cidx(o, i5 + 1, i3, i1 + 1);
                    size_t a110 = cidx(o, i5 + 1, i3 + 1, i1), a111 = cidx(o, i5 + 1, i3 + 1, i1 + 1);
                    size_t c = cidx(b, z, y, x);
                    for (int q = 0; q < Q; q++) {
                        const double *f = o->f + no * q;
                        b->f[c + n * q] = f[a000] * (1.0 - c3) * (1.0 - c2) * (1.0 - c1) +
                                          f[a001] * (1.0 - c3) * (1.0 - c2) * c1 +
                                          f[a010] * (1.0 - c3) * c2 * (1.0 - c1) +
                                          f[a011] * (1.0 - c3) * c2 * c1 +
                                          f[a100] * c3 * (1.0 - c2) * (1.0 - c1) +
                                          f[a101] * c3 * (1.0 - c2) * c1 +
                                          f[a110] * c3 * c2 * (1.0 - c1) +
                                          f[a111] * c3 * c2 * c1;
                    }
                    break;
                }
            }
        }
    }
}
