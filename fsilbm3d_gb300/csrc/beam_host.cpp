// beam_host.cpp -- host implementation of include/fsi_beam.h: the structural
// solver of a flexible body, restated from SolidSolver.f90 (modules
// SegmentStructure and SolidSolver) and the plate parts of Solidbody.f90.
//
// FP64 throughout, in the reference's operation order (this unit is compiled
// without floating-point contraction, as gfortran builds the reference on
// x86-64): each function cites the routine it restates. Matrices are stored
// row-major with [r][c] = the reference's (r+1, c+1); node and DOF numbers are
// 0-based here and 1-based in the reference.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/fsi_beam.h"
#include "../../include/fsi_gpu.h"

namespace fsi {
int host_fail(int code, const char *msg);  // sets the message of fsi_last_error (fsi_abi.cu)
}

namespace {

constexpr int NE = 12;  // nElmtDofs
const double PI = 3.141592653589793;

int bfail(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
int bfail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return fsi::host_fail(code, buf);
}

typedef double M3[3][3];

// c = a b (3x3), sums in k order from zero as the reference's matmul
void mm3(const M3 a, const M3 b, M3 c) {
    M3 t;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s = s + a[i][k] * b[k][j];
            t[i][j] = s;
        }
    memcpy(c, t, sizeof(M3));
}

// y = a x (3x3 by 3)
void mv3(const M3 a, const double x[3], double y[3]) {
    double t[3];
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        for (int k = 0; k < 3; k++) s = s + a[i][k] * x[k];
        t[i] = s;
    }
    y[0] = t[0]; y[1] = t[1]; y[2] = t[2];
}

double dot3(const double a[3], const double b[3]) {
    double s = 0.0;
    for (int k = 0; k < 3; k++) s = s + a[k] * b[k];
    return s;
}

// Segment_get_angle_triad (SolidSolver.f90:909-952): the rotation vector
// taking triad t11 to triad t22
void angle_triad(const M3 t11, const M3 t22, double &tx, double &ty, double &tz) {
    M3 rr;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s = s + t22[i][k] * t11[j][k];
            rr[i][j] = s;
        }
    const double dtx = (rr[2][1] - rr[1][2]) / 2.0;
    const double dty = (rr[0][2] - rr[2][0]) / 2.0;
    const double dtz = (rr[1][0] - rr[0][1]) / 2.0;
    double tr = rr[0][0] + rr[1][1] + rr[2][2];
    tr = (tr - 1.0) / 2.0;
    if (tr > 1.0) tr = 1.0;
    if (tr < -1.0) tr = -1.0;
    const double sint = std::sqrt(dtx * dtx + dty * dty + dtz * dtz);
    const double theta = std::acos(tr);
    if (sint < 1.0e-10 || theta < 1.0e-10) {
        tx = dtx; ty = dty; tz = dtz;
    } else {
        const double f = theta / sint;
        tx = f * dtx; ty = f * dty; tz = f * dtz;
    }
}

// Segment_global_to_local (SolidSolver.f90:954-964)
void global_to_local(const M3 t, double tx, double ty, double tz, double &a, double &b, double &c) {
    a = t[0][0] * tx + t[1][0] * ty + t[2][0] * tz;
    b = t[0][1] * tx + t[1][1] * ty + t[2][1] * tz;
    c = t[0][2] * tx + t[1][2] * ty + t[2][2] * tz;
}

// Segment_FiniteRot (SolidSolver.f90:1066-1124): Rodrigues' rotation matrix
void finite_rot(double t1, double t2, double t3, M3 rr) {
    const double tt = std::sqrt(t1 * t1 + t2 * t2 + t3 * t3);
    const double ss = std::sin(tt), cc = std::cos(tt);
    const M3 r1 = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
    const M3 r2 = {{0.0, -t3, t2}, {t3, 0.0, -t1}, {-t2, t1, 0.0}};
    const M3 r3 = {{-(t3 * t3) - t2 * t2, t2 * t1, t3 * t1},
                   {t1 * t2, -(t3 * t3) - t1 * t1, t3 * t2},
                   {t1 * t3, t2 * t3, -(t2 * t2) - t1 * t1}};
    double c1, c2;
    if (tt < 1.0e-10) {
        c1 = 1.0;
        c2 = 0.5;
    } else {
        c1 = ss / tt;
        c2 = (1.0 - cc) / (tt * tt);
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) rr[i][j] = (r1[i][j] + r2[i][j] * c1) + r3[i][j] * c2;
}

// AoAtoTTT (SolidSolver.f90:2404-2472): body rotation from the angles of
// attack, Rx Ry Rz applied to the identity in the order z, y, x; angles
// within 1e-5 of 0 or +-pi/2 snap to exact values. The reference's pi in
// this routine is 3.141562653589793 (its ninth digit differs from pi); it
// only sets where the +-pi/2 snapping happens, and is kept.
void aoa_to_ttt(const double aoa[3], M3 T) {
    const double pi = 3.141562653589793, eps = 1.0e-5;
    double c[3], s[3];
    for (int k = 0; k < 3; k++) {
        c[k] = std::cos(aoa[k]);
        s[k] = std::sin(aoa[k]);
        if (std::fabs(aoa[k]) < eps) { c[k] = 1.0; s[k] = 0.0; }
        if (std::fabs(aoa[k] - 0.5 * pi) < eps) { c[k] = 0.0; s[k] = 1.0; }
        if (std::fabs(aoa[k] + 0.5 * pi) < eps) { c[k] = 0.0; s[k] = -1.0; }
    }
    const M3 rx = {{1.0, 0.0, 0.0}, {0.0, c[0], -s[0]}, {0.0, s[0], c[0]}};
    const M3 ry = {{c[1], 0.0, s[1]}, {0.0, 1.0, 0.0}, {-s[1], 0.0, c[1]}};
    const M3 rz = {{c[2], -s[2], 0.0}, {s[2], c[2], 0.0}, {0.0, 0.0, 1.0}};
    M3 I = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
    mm3(rz, I, T);
    mm3(ry, T, T);
    mm3(rx, T, T);
}

// Segment (SolidSolver.f90:13-57): one two-node beam element
struct Segment {
    int node0 = 0, node1 = 0, l2g[NE] = {}, itype = 0, bc[NE] = {}, Nspan = 0;
    double x00[NE] = {}, x0[NE] = {}, x1[NE] = {}, xnxt[NE] = {};
    double dx0 = 0, dy0 = 0, dz0 = 0, dx1 = 0, dy1 = 0, dz1 = 0;
    double xll0 = 0, xmm0 = 0, xnn0 = 0, xll1 = 0, xmm1 = 0, xnn1 = 0, len0 = 0, len1 = 0;
    double Lspan = 0, spanlen = 0, dirc00[3] = {}, dirc0[3] = {}, dirc1[3] = {}, dircnxt[3] = {};
    double geoFRM = 0, areaElem00 = 0, strainEnergy[2] = {};
    M3 ee = {}, n1 = {}, n2 = {};  // triad_ee, triad_n1, triad_n2
    double prop[8] = {};
    double coef[NE][NE] = {}, tan_[NE][NE] = {}, stf[NE][NE] = {}, mas[NE][NE] = {}, geo[NE][NE] = {};
    M3 rot = {};

    // Segment_Init, Segment_cptdxyz1 (SolidSolver.f90:102-129)
    void init() {
        memcpy(x1, x0, sizeof(x1));
        memcpy(xnxt, x1, sizeof(xnxt));
        memcpy(dirc1, dirc0, sizeof(dirc1));
        memcpy(dircnxt, dirc1, sizeof(dircnxt));
        dx0 = x0[6] - x0[0];
        dy0 = x0[7] - x0[1];
        dz0 = x0[8] - x0[2];
        len0 = std::sqrt(dx0 * dx0 + dy0 * dy0 + dz0 * dz0);
        xll0 = dx0 / len0;
        xmm0 = dy0 / len0;
        xnn0 = dz0 / len0;
        cptdxyz1();
    }
    void cptdxyz1() {
        dx1 = x1[6] - x1[0];
        dy1 = x1[7] - x1[1];
        dz1 = x1[8] - x1[2];
        len1 = std::sqrt(dx1 * dx1 + dy1 * dy1 + dz1 * dz1);
        xll1 = dx1 / len1;
        xmm1 = dy1 / len1;
        xnn1 = dz1 / len1;
    }

    // Segment_FormMassMatrix (SolidSolver.f90:318-363): lumped, rotary
    // inertia about the axis from Iy + Iz
    void form_mass() {
        const double area = prop[2], rho = prop[3], ziy = prop[6], ziz = prop[7], length = len0;
        memset(mas, 0, sizeof(mas));
        const double roal = ((rho * area) * length) / 2.0;
        mas[0][0] = roal; mas[1][1] = roal; mas[2][2] = roal;
        mas[3][3] = (roal * (ziy + ziz)) / area;
        mas[4][4] = (roal * ziy) / area;
        mas[5][5] = (roal * ziz) / area;
        for (int i = 0; i < 6; i++) mas[i + 6][i + 6] = mas[i][i];
    }

    // Timoshenko shear parameters of both bending planes (shear factor 5/6)
    void shear_phi(double &phiy, double &phiz) const {
        const double emod = prop[0], gmod = prop[1], area = prop[2], ziy = prop[6], ziz = prop[7], length = len0;
        const double ksy = 5.0 / 6.0, ksz = 5.0 / 6.0;
        phiy = ((12.0 * emod) * ziz) / ((((ksy * gmod) * area) * length) * length);
        phiz = ((12.0 * emod) * ziy) / ((((ksz * gmod) * area) * length) * length);
    }

    static void sym_fill(double m[NE][NE]) {
        const int pr[][2] = {{0, 6}, {1, 5}, {1, 7}, {1, 11}, {5, 7}, {5, 11}, {7, 11}, {2, 4}, {2, 8}, {2, 10},
                             {4, 8}, {4, 10}, {8, 10}, {3, 9}};
        for (auto &p : pr) m[p[1]][p[0]] = m[p[0]][p[1]];
    }

    // Segment_FormStiffMatrix (SolidSolver.f90:365-478): local elastic
    // stiffness of the 3-D Timoshenko frame
    void form_stiff() {
        const double emod = prop[0], gmod = prop[1], area = prop[2], zix = prop[5], ziy = prop[6], ziz = prop[7];
        const double length = len0;
        memset(stf, 0, sizeof(stf));
        const double inv = 1.0 / length;
        double phiy, phiz;
        shear_phi(phiy, phiz);
        const double l2 = length * length, l3 = (length * length) * length;
        const double ky1 = ((12.0 * emod) * ziz) / (l3 * (1.0 + phiy));
        const double ky2 = ((6.0 * emod) * ziz) / (l2 * (1.0 + phiy));
        const double ky3 = (((4.0 + phiy) * emod) * ziz) / (length * (1.0 + phiy));
        const double ky4 = (((2.0 - phiy) * emod) * ziz) / (length * (1.0 + phiy));
        const double kz1 = ((12.0 * emod) * ziy) / (l3 * (1.0 + phiz));
        const double kz2 = ((6.0 * emod) * ziy) / (l2 * (1.0 + phiz));
        const double kz3 = (((4.0 + phiz) * emod) * ziy) / (length * (1.0 + phiz));
        const double kz4 = (((2.0 - phiz) * emod) * ziy) / (length * (1.0 + phiz));
        stf[0][0] = (area * emod) * inv;
        stf[1][1] = ky1;
        stf[2][2] = kz1;
        stf[3][3] = (gmod * zix) * inv;
        stf[4][4] = kz3;
        stf[5][5] = ky3;
        for (int i = 0; i < 6; i++) stf[i + 6][i + 6] = stf[i][i];
        stf[0][6] = -stf[0][0];
        stf[1][5] = ky2; stf[1][7] = -ky1; stf[1][11] = ky2;
        stf[5][7] = -ky2; stf[5][11] = ky4; stf[7][11] = -ky2;
        stf[2][4] = -kz2; stf[2][8] = -kz1; stf[2][10] = -kz2;
        stf[4][8] = kz2; stf[4][10] = kz4; stf[8][10] = kz2;
        stf[3][9] = -stf[3][3];
        sym_fill(stf);
    }

    // Segment_FormGeomMatrix (SolidSolver.f90:480-600): geometric stiffness
    // of the axial force geoFRM
    void form_geom() {
        const double area = prop[2], zix = prop[5], length = len0, s = geoFRM;
        memset(geo, 0, sizeof(geo));
        double phiy, phiz;
        shear_phi(phiy, phiz);
        const double sl = s / length;
        auto terms = [&](double phi, double &g1, double &g2, double &g3, double &g4) {
            const double d = (1.0 + phi) * (1.0 + phi);
            g1 = (sl * ((6.0 / 5.0 + 2.0 * phi) + phi * phi)) / d;
            g2 = (sl * (length / 10.0)) / d;
            g3 = (sl * ((((2.0 * length) * length) / 15.0 + ((phi * length) * length) / 6.0) +
                        (((phi * phi) * length) * length) / 12.0)) / d;
            g4 = (sl * ((-((length * length) / 30.0) - ((phi * length) * length) / 6.0) -
                        (((phi * phi) * length) * length) / 12.0)) / d;
        };
        double gy1, gy2, gy3, gy4, gz1, gz2, gz3, gz4;
        terms(phiy, gy1, gy2, gy3, gy4);
        terms(phiz, gz1, gz2, gz3, gz4);
        geo[1][1] = gy1; geo[5][5] = gy3; geo[7][7] = gy1; geo[11][11] = gy3;
        geo[1][5] = gy2; geo[1][7] = -gy1; geo[1][11] = gy2;
        geo[5][7] = -gy2; geo[5][11] = gy4; geo[7][11] = -gy2;
        geo[2][2] = gz1; geo[4][4] = gz3; geo[8][8] = gz1; geo[10][10] = gz3;
        geo[2][4] = -gz2; geo[2][8] = -gz1; geo[2][10] = -gz2;
        geo[4][8] = gz2; geo[4][10] = gz4; geo[8][10] = gz2;
        const double gt = (s * zix) / (area * length);
        geo[3][3] = gt; geo[3][9] = -gt; geo[9][9] = gt;
        sym_fill(geo);
    }

    // Segment_BuildAxisDirTriad (SolidSolver.f90:624-697): ex along the axis,
    // ey the span direction made orthogonal to it, ez = ex x ey; without a
    // span direction, Doyle's default triad
    static void axis_dir_triad(double l, double m, double n, const double d[3], M3 triad) {
        double ex[3] = {l, m, n}, ey[3], ez[3], dir[3] = {d[0], d[1], d[2]};
        double dd = std::sqrt(dot3(ex, ex));
        if (dd > 1.0e-14)
            for (double &v : ex) v = v / dd;
        dd = std::sqrt(dot3(dir, dir));
        if (dd > 1.0e-14)
            for (double &v : dir) v = v / dd;
        const double proj = dot3(dir, ex);
        for (int k = 0; k < 3; k++) ey[k] = dir[k] - proj * ex[k];
        dd = std::sqrt(dot3(ey, ey));
        if (dd <= 1.0e-10) {
            if (std::fabs(ex[2]) > 0.995) {
                ey[0] = 0.0; ey[1] = 1.0; ey[2] = 0.0;
                ez[0] = -ex[2]; ez[1] = 0.0; ez[2] = 0.0;
            } else {
                dd = std::sqrt(ex[0] * ex[0] + ex[1] * ex[1]);
                ey[0] = -ex[1] / dd; ey[1] = ex[0] / dd; ey[2] = 0.0;
                ez[0] = -(ex[0] * ex[2]) / dd; ez[1] = -(ex[1] * ex[2]) / dd; ez[2] = dd;
            }
        } else {
            for (double &v : ey) v = v / dd;
            ez[0] = ex[1] * ey[2] - ex[2] * ey[1];
            ez[1] = ex[2] * ey[0] - ex[0] * ey[2];
            ez[2] = ex[0] * ey[1] - ex[1] * ey[0];
            dd = std::sqrt(dot3(ez, ez));
            if (dd > 1.0e-14)
                for (double &v : ez) v = v / dd;
        }
        for (int k = 0; k < 3; k++) {
            triad[k][0] = ex[k];
            triad[k][1] = ey[k];
            triad[k][2] = ez[k];
        }
    }

    // Segment_InitTriad_D / Segment_RigidUpdateTriad_D (SolidSolver.f90:602-622)
    void init_triad() {
        axis_dir_triad(xll0, xmm0, xnn0, dirc0, n1);
        memcpy(n2, n1, sizeof(M3));
        memcpy(ee, n1, sizeof(M3));
    }
    void rigid_update_triad() {
        axis_dir_triad(xll1, xmm1, xnn1, dirc1, n1);
        memcpy(n2, n1, sizeof(M3));
        memcpy(ee, n1, sizeof(M3));
    }

    // Segment_RotateMatrix (SolidSolver.f90:699-707): R = triad_ee^T
    void rotate_matrix() {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) rot[i][j] = ee[j][i];
    }

    // Segment_RKR (SolidSolver.f90:709-748): ek <- R^T ek R block by block
    void rkr(double ek[NE][NE]) const {
        M3 r, rt;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                r[i][j] = rot[i][j];
                rt[j][i] = rot[i][j];
            }
        double kt[NE][NE];
        for (int bi = 0; bi < 4; bi++)
            for (int bj = 0; bj < 4; bj++) {
                const int j1 = bi * 3, j2 = bj * 3;
                for (int k = 0; k < 3; k++)
                    for (int ii = 0; ii < 3; ii++) {
                        double s = 0.0;
                        for (int jj = 0; jj < 3; jj++) s = s + ek[j1 + k][j2 + jj] * r[jj][ii];
                        kt[j1 + k][j2 + ii] = s;
                    }
                for (int k = 0; k < 3; k++)
                    for (int ii = 0; ii < 3; ii++) {
                        double s = 0.0;
                        for (int jj = 0; jj < 3; jj++) s = s + rt[k][jj] * kt[j1 + jj][j2 + ii];
                        ek[j1 + k][j2 + ii] = s;
                    }
            }
    }

    // Segment_UpdateMatrix (SolidSolver.f90:131-157): coefMat = K_E + gamma
    // K_G (both rotated to the global frame) + c0 M + c1 dampM M (+ c1 dampK K_E)
    void update_matrix(const double c[8], double gamma, double dampM, double dampK) {
        form_geom();
        rotate_matrix();
        rkr(stf);
        rkr(geo);
        for (int i = 0; i < NE; i++)
            for (int j = 0; j < NE; j++) {
                tan_[i][j] = stf[i][j] + gamma * geo[i][j];
                coef[i][j] = (tan_[i][j] + c[0] * mas[i][j]) + (c[1] * dampM) * mas[i][j];
            }
        if (dampK > 0.0)
            for (int i = 0; i < NE; i++)
                for (int j = 0; j < NE; j++) coef[i][j] = coef[i][j] + (c[1] * dampK) * stf[i][j];
    }

    // Segment_MassMultiply (SolidSolver.f90:195-234)
    void mass_multiply(const double q[NE], double mq[NE]) const {
        for (int i = 0; i < NE; i++) mq[i] = 0.0;
        for (int i = 0; i < 3; i++) {
            mq[i] = mas[i][i] * q[i];
            mq[i + 6] = mas[i + 6][i + 6] * q[i + 6];
        }
        for (int b : {3, 9})
            for (int i = 0; i < 3; i++) {
                double s = 0.0;
                for (int k = 0; k < 3; k++) s = s + mas[b + i][b + k] * q[b + k];
                mq[b + i] = s;
            }
    }

    void loc_to_global(const double lx[NE], double *x) const {
        for (int i = 0; i < NE; i++) x[l2g[i]] = x[l2g[i]] + lx[i];
    }

    // Segment_UpdateLoad (SolidSolver.f90:159-193): the Newmark inertia (and
    // damping) terms of the effective load
    void update_load(const double c[8], double dampM, double dampK, const double *dspO, const double *dsp,
                     const double *vel, const double *acc, double *lodEffe) const {
        double qM[NE], qC[NE], qMC[NE], ml[NE];
        for (int i = 0; i < 6; i++)
            for (int h = 0; h < 2; h++) {
                const int n = h ? node1 : node0, o = 6 * n + i, e = i + 6 * h;
                qM[e] = (c[0] * (dspO[o] - dsp[o]) + c[2] * vel[o]) + c[3] * acc[o];
                qC[e] = (c[1] * (dspO[o] - dsp[o]) + c[4] * vel[o]) + c[5] * acc[o];
            }
        for (int i = 0; i < NE; i++) qMC[i] = qM[i] + dampM * qC[i];
        mass_multiply(qMC, ml);
        loc_to_global(ml, lodEffe);
        if (dampK > 0.0) {
            double dl[NE];
            for (int i = 0; i < NE; i++) {
                double s = 0.0;
                for (int k = 0; k < NE; k++) s = s + stf[i][k] * qC[k];
                dl[i] = dampK * s;
            }
            loc_to_global(dl, lodEffe);
        }
    }

    // Segment_BodyStress_D (SolidSolver.f90:750-839): internal nodal forces
    // from the deformation in the element frame; sets the axial force geoFRM
    void body_stress(double *lodInte) {
        const double du = dx1 - dx0, dv = dy1 - dy0, dw = dz1 - dz0;
        const double dl = (((dx0 + dx1) * du + (dy0 + dy1) * dv) + (dz0 + dz1) * dw) / (len0 + len1);
        double tx, ty, tz, tx1, ty1, tz1, tx2, ty2, tz2;
        angle_triad(ee, n1, tx, ty, tz);
        global_to_local(ee, tx, ty, tz, tx1, ty1, tz1);
        angle_triad(ee, n2, tx, ty, tz);
        global_to_local(ee, tx, ty, tz, tx2, ty2, tz2);
        const double ub[NE] = {0.0, 0.0, 0.0, tx1, ty1, tz1, dl, 0.0, 0.0, tx2, ty2, tz2};
        const double emod = prop[0], area = prop[2];
        geoFRM = ((dl * emod) * area) / len0;
        double fb[NE], f[NE];
        for (int i = 0; i < NE; i++) {
            double s = 0.0;
            for (int k = 0; k < NE; k++) s = s + stf[i][k] * ub[k];
            fb[i] = s;
        }
        for (int i = 0; i < NE; i++) f[i] = 0.0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                for (int b = 0; b < NE; b += 3) f[b + i] = f[b + i] + ee[i][j] * fb[b + j];
        loc_to_global(f, lodInte);
    }

    // Segment_UpdateTriad_D (SolidSolver.f90:966-997): nodal triads turned by
    // the nodes' rotation increments
    void update_triad(const double *dspnn) {
        M3 rr;
        finite_rot(dspnn[6 * node0 + 3], dspnn[6 * node0 + 4], dspnn[6 * node0 + 5], rr);
        mm3(rr, n1, n1);
        finite_rot(dspnn[6 * node1 + 3], dspnn[6 * node1 + 4], dspnn[6 * node1 + 5], rr);
        mm3(rr, n2, n2);
    }

    // Segment_MakeTriad_ee (SolidSolver.f90:999-1064): element triad from the
    // current axis and the mean of the two nodal triads
    void make_triad_ee() {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) ee[i][j] = 0.0;
        ee[0][0] = xll1; ee[1][0] = xmm1; ee[2][0] = xnn1;
        double tx, ty, tz;
        angle_triad(n1, n2, tx, ty, tz);
        tx = tx / 2.0; ty = ty / 2.0; tz = tz / 2.0;
        M3 rr, aa;
        finite_rot(tx, ty, tz, rr);
        mm3(rr, n1, aa);
        double r2e1 = 0.0, r3e1 = 0.0;
        for (int k = 0; k < 3; k++) {
            r2e1 = r2e1 + aa[k][1] * ee[k][0];
            r3e1 = r3e1 + aa[k][2] * ee[k][0];
        }
        for (int j = 0; j < 3; j++) {
            ee[j][1] = aa[j][1] - (r2e1 * (aa[j][0] + ee[j][0])) / 2.0;
            ee[j][2] = aa[j][2] - (r3e1 * (aa[j][0] + ee[j][0])) / 2.0;
        }
        double e1[3] = {ee[0][0], ee[1][0], ee[2][0]}, e2[3] = {ee[0][1], ee[1][1], ee[2][1]};
        const double p = dot3(e2, e1);
        for (int k = 0; k < 3; k++) e2[k] = e2[k] - p * e1[k];
        const double dd = std::sqrt(dot3(e2, e2));
        if (dd > 1.0e-14)
            for (double &v : e2) v = v / dd;
        for (int k = 0; k < 3; k++) ee[k][1] = e2[k];
        ee[0][2] = ee[1][0] * ee[2][1] - ee[2][0] * ee[1][1];
        ee[1][2] = ee[2][0] * ee[0][1] - ee[0][0] * ee[2][1];
        ee[2][2] = ee[0][0] * ee[1][1] - ee[1][0] * ee[0][1];
    }

    // Segment_MapReferencePosToCurrent / DirToCurrent (SolidSolver.f90:1126-1145)
    void map_pos(double out[NE], const M3 T, const double XYZ[3], const double AoA[3]) const {
        double a[3], b[3];
        mv3(T, x00, a);
        mv3(T, x00 + 6, b);
        for (int k = 0; k < 3; k++) {
            out[k] = a[k] + XYZ[k];
            out[3 + k] = AoA[k];
            out[6 + k] = b[k] + XYZ[k];
            out[9 + k] = AoA[k];
        }
    }
    void map_dir(double d[3], const M3 T) const { mv3(T, dirc00, d); }
};

// Invert6x6 (SolidSolver.f90:2234-2279): Gauss-Jordan with partial pivoting
int invert6(const double A[6][6], double Ainv[6][6]) {
    double aug[6][12];
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 12; j++) aug[i][j] = j < 6 ? A[i][j] : (j - 6 == i ? 1.0 : 0.0);
    for (int i = 0; i < 6; i++) {
        int p = i;
        double pivot = std::fabs(aug[i][i]);
        for (int k = i + 1; k < 6; k++)
            if (std::fabs(aug[k][i]) > pivot) {
                pivot = std::fabs(aug[k][i]);
                p = k;
            }
        if (pivot <= 1.0e-30) {
            for (int r = 0; r < 6; r++)
                for (int c = 0; c < 6; c++) Ainv[r][c] = 0.0;
            return i + 1;
        }
        if (p != i)
            for (int j = 0; j < 12; j++) {
                const double t = aug[i][j];
                aug[i][j] = aug[p][j];
                aug[p][j] = t;
            }
        pivot = aug[i][i];
        for (int j = 0; j < 12; j++) aug[i][j] = aug[i][j] / pivot;
        for (int k = 0; k < 6; k++)
            if (k != i) {
                const double f = aug[k][i];
                for (int j = 0; j < 12; j++) aug[k][j] = aug[k][j] - f * aug[i][j];
            }
    }
    for (int r = 0; r < 6; r++)
        for (int c = 0; c < 6; c++) Ainv[r][c] = aug[r][6 + c];
    return 0;
}

}  // namespace

// BeamSolver (SolidSolver.f90:1156-1217) plus the plate marker layout of a
// VirtualBody (Solidbody.f90:25-68)
struct fsi_beam {
    fsi_beam_params sp{};
    fsi_beam_body bd{};
    std::vector<Segment> el;
    int nND = 0, nEL = 0, nMT = 0, gEQ = 0;
    double FishInfo[3] = {0, 0, 0};
    std::vector<double> pos, dsp, vel, acc, mss;  // (6,nND); mss (3,nND)
    std::vector<double> lodInte, lodExte, lodEffe, lodFlow, lodRepl, lodGrav, vBC;
    double coeffs[8] = {};
    double elmax = 0, elmin = 0;
    double XYZ[3] = {}, UVW[3] = {}, AoA[3] = {}, AoAd[3] = {}, WWW1[3] = {}, WWW2[3] = {}, WWW3[3] = {};
    M3 TTT00 = {}, TTT0 = {}, TTTnxt = {};
    // plate markers: rtov(i) first marker of element i, vtor(m) element of marker m
    std::vector<int> rtov, vtor;
    int M = 0;
    bool initialised = false;

    // Beam_UpdateVelFromPosAngular (SolidSolver.f90:1478-1494): v = U + w x r
    void vel_from_angular(const double W[3], const double U[3]) {
        for (int n = 0; n < nND; n++) {
            const double r[3] = {pos[6 * n] - XYZ[0], pos[6 * n + 1] - XYZ[1], pos[6 * n + 2] - XYZ[2]};
            vel[6 * n] = (W[1] * r[2] - W[2] * r[1]) + U[0];
            vel[6 * n + 1] = (W[2] * r[0] - W[0] * r[2]) + U[1];
            vel[6 * n + 2] = (W[0] * r[1] - W[1] * r[0]) + U[2];
            vel[6 * n + 3] = W[0];
            vel[6 * n + 4] = W[1];
            vel[6 * n + 5] = W[2];
        }
    }

    // the body rotation rate of the prescribed pitching at body time t: WWW1
    // (Euler-angle rates), WWW2 (body axes), WWW3 = T WWW2 (SolidSolver.f90:1423-1428, 1850-1855)
    void rotation_rate(double t, const M3 T) {
        const double *A = bd.AoAAmpl, *P = bd.AoAPhi;
        for (int k = 0; k < 3; k++) WWW1[k] = ((((-2.0 * PI) * bd.Freq) * A[k]) * std::sin(((2.0 * PI) * bd.Freq) * t + P[k]));
        WWW2[0] = WWW1[0] * std::cos(AoA[1]) + WWW1[2];
        WWW2[1] = (WWW1[0] * std::sin(AoA[1])) * std::sin(AoA[2]) + WWW1[1] * std::cos(AoA[2]);
        WWW2[2] = (WWW1[0] * std::sin(AoA[1])) * std::cos(AoA[2]) - WWW1[1] * std::sin(AoA[2]);
        mv3(T, WWW2, WWW3);
    }

    void translation(double t) {
        for (int k = 0; k < 3; k++) {
            XYZ[k] = (bd.XYZo[k] + bd.XYZAmpl[k] * std::cos(((2.0 * PI) * bd.Freq) * t + bd.XYZPhi[k])) +
                     bd.initXYZVel[k] * t;
            AoA[k] = bd.AoAo[k] + bd.AoAAmpl[k] * std::cos(((2.0 * PI) * bd.Freq) * t + bd.AoAPhi[k]);
        }
    }
    void translation_velocity(double t) {
        for (int k = 0; k < 3; k++)
            UVW[k] = ((((-2.0 * PI) * bd.Freq) * bd.XYZAmpl[k]) * std::sin(((2.0 * PI) * bd.Freq) * t + bd.XYZPhi[k])) +
                     bd.initXYZVel[k];
    }

    // Beam_UpdateNewmarkCoeffs (SolidSolver.f90:1879-1892)
    void newmark(double dt) {
        const double g = sp.NewmarkGamma, b = sp.NewmarkBeta;
        coeffs[2] = 1.0 / (b * dt);
        coeffs[1] = g * coeffs[2];
        coeffs[0] = coeffs[2] / dt;
        coeffs[3] = 0.5 / b - 1.0;
        coeffs[4] = g / b - 1.0;
        coeffs[5] = dt * ((0.5 * g) / b - 1.0);
        coeffs[6] = dt * (1.0 - g);
        coeffs[7] = dt * g;
    }

    void matrix_multiply(const std::vector<double> &x, std::vector<double> &b) const {
        std::fill(b.begin(), b.end(), 0.0);
        for (const Segment &s : el) {
            double lx[NE], lb[NE];
            for (int i = 0; i < NE; i++) lx[i] = x[s.l2g[i]];
            for (int i = 0; i < NE; i++) {
                double t = 0.0;
                for (int k = 0; k < NE; k++) t = t + s.coef[i][k] * lx[k];
                lb[i] = t;
            }
            s.loc_to_global(lb, b.data());
        }
    }

    static double dot(const std::vector<double> &a, const std::vector<double> &b) {
        double s = 0.0;
        for (size_t i = 0; i < a.size(); i++) s = s + a[i] * b[i];
        return s;
    }

    // Beam_CG_Solve (SolidSolver.f90:1949-2020) with the node-wise 6x6 block
    // Jacobi preconditioner (:2074-2232); prescribed DOFs by lifting
    int cg_solve(std::vector<double> &x, const std::vector<double> &b, int iterNR) {
        const int n = gEQ;
        const int max_iter = 10000;
        const double err = 1.0e-6;
        std::vector<double> r(n), p(n), Ap(n), z(n), xF(n, 0.0);
        std::vector<char> fixed(n, 0);
        // Beam_BoundaryCond / Segment_BoundaryCond (SolidSolver.f90:236-258, 2022-2033)
        for (const Segment &s : el)
            for (int i = 0; i < NE; i++)
                if (s.bc[i] > 0) {
                    const int g = s.l2g[i];
                    fixed[g] = 1;
                    xF[g] = (iterNR == 1) ? vBC[g] : 0.0;
                }
        x = xF;
        matrix_multiply(x, Ap);
        for (int i = 0; i < n; i++) r[i] = b[i] - Ap[i];
        for (int i = 0; i < n; i++)
            if (fixed[i]) r[i] = 0.0;
        // block Jacobi: Beam_BlockPreconditioned, Beam_InitBlockJacobiPreconditioner
        std::vector<double> blk(36 * (size_t)nND, 0.0);
        auto B = [&](int node, int i, int j) -> double & { return blk[36 * (size_t)node + 6 * i + j]; };
        for (const Segment &s : el)
            for (int i = 0; i < 6; i++)
                for (int j = 0; j < 6; j++) {
                    B(s.node0, i, j) = B(s.node0, i, j) + s.coef[i][j];
                    B(s.node1, i, j) = B(s.node1, i, j) + s.coef[i + 6][j + 6];
                }
        for (int node = 0; node < nND; node++) {
            for (int i = 0; i < 6; i++)
                if (fixed[6 * node + i]) {
                    for (int j = 0; j < 6; j++) {
                        B(node, i, j) = 0.0;
                        B(node, j, i) = 0.0;
                    }
                    B(node, i, i) = 1.0;
                }
            double A6[6][6], inv[6][6];
            for (int i = 0; i < 6; i++)
                for (int j = 0; j < 6; j++) A6[i][j] = B(node, i, j);
            if (invert6(A6, inv) != 0) {
                // the reference warns and uses the identity block
                for (int i = 0; i < 6; i++)
                    for (int j = 0; j < 6; j++) B(node, i, j) = (i == j) ? 1.0 : 0.0;
            } else {
                for (int i = 0; i < 6; i++)
                    for (int j = 0; j < 6; j++) B(node, i, j) = inv[i][j];
            }
        }
        auto precond = [&](const std::vector<double> &rr, std::vector<double> &zz) {
            for (int node = 0; node < nND; node++)
                for (int i = 0; i < 6; i++) {
                    double s = 0.0;
                    for (int k = 0; k < 6; k++) s = s + B(node, i, k) * rr[6 * node + k];
                    zz[6 * node + i] = fixed[6 * node + i] ? 0.0 : s;
                }
        };
        precond(r, z);
        double res = std::sqrt(dot(r, r));
        if (res <= err) return FSI_OK;
        p = z;
        double rsold = dot(r, z);
        if (std::fabs(rsold) <= 1.0e-30)
            return bfail(FSI_E_NAN, "beam CG breakdown: initial (r, z) = %g, residual %g", rsold, res);
        for (int it = 1; it <= max_iter; it++) {
            matrix_multiply(p, Ap);
            for (int i = 0; i < n; i++)
                if (fixed[i]) Ap[i] = 0.0;
            const double pAp = dot(p, Ap);
            if (std::fabs(pAp) <= 1.0e-30)
                return bfail(FSI_E_NAN, "beam CG breakdown: (p, Ap) = %g at iteration %d, residual %g", pAp, it, res);
            const double alpha = rsold / pAp;
            for (int i = 0; i < n; i++) x[i] = x[i] + alpha * p[i];
            for (int i = 0; i < n; i++)
                if (fixed[i]) x[i] = xF[i];
            for (int i = 0; i < n; i++) r[i] = r[i] - alpha * Ap[i];
            for (int i = 0; i < n; i++)
                if (fixed[i]) r[i] = 0.0;
            res = std::sqrt(dot(r, r));
            if (res <= err) break;
            precond(r, z);
            const double rsnew = dot(r, z);
            if (std::fabs(rsold) <= 1.0e-30)
                return bfail(FSI_E_NAN, "beam CG breakdown: rsold = %g at iteration %d", rsold, it);
            const double beta = rsnew / rsold;
            for (int i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
            for (int i = 0; i < n; i++)
                if (fixed[i]) p[i] = 0.0;
            rsold = rsnew;
        }
        if (!std::isfinite(res)) return bfail(FSI_E_NAN, "beam CG: non-finite residual");
        return FSI_OK;
    }

    // Beam_UpdateDspANDTride (SolidSolver.f90:2304-2338)
    void update_dsp_triad(int iter, const std::vector<double> &dspn, double &dnorm) {
        const double beta0 = 1.0;
        const int maxramp = 1;
        double beta;
        if (iter <= maxramp) {
            const double zi = std::pow(2.0, iter), z0 = std::pow(2.0, maxramp);
            beta = (zi / z0) * beta0;
        } else {
            beta = 1.0 * beta0;
        }
        std::vector<double> dspnn(gEQ);
        for (int i = 0; i < gEQ; i++) dspnn[i] = beta * dspn[i];
        for (int i = 0; i < gEQ; i++) dsp[i] = dsp[i] + dspnn[i];
        for (Segment &s : el) {
            for (int k = 0; k < 6; k++) {
                s.x1[k] = s.x0[k] + dsp[6 * s.node0 + k];
                s.x1[k + 6] = s.x0[k + 6] + dsp[6 * s.node1 + k];
            }
            for (int k = 0; k < 6; k++) {
                pos[6 * s.node0 + k] = s.x1[k];
                pos[6 * s.node1 + k] = s.x1[k + 6];
            }
            s.cptdxyz1();
            s.update_triad(dspnn.data());
            s.make_triad_ee();
        }
        double mx = -HUGE_VAL;
        for (int i = 0; i < gEQ; i++) {
            const double v = (beta * dspn[i]) * (beta * dspn[i]);
            if (v > mx) mx = v;
        }
        dnorm = std::fabs(mx);
    }

    // Beam_Solver (SolidSolver.f90:1894-1914) with Beam_InitDspVelAccATTimeT,
    // Beam_UpdateMatrixANDLoad, Beam_UpdateVelAcc (:1916-1947, 2350-2359)
    int solve() {
        double dnorm = 1.0;
        std::fill(vBC.begin(), vBC.end(), 0.0);
        for (const Segment &s : el)
            for (int i = 0; i < NE; i++) vBC[s.l2g[i]] = s.xnxt[i] - s.x1[i];
        for (int i = 0; i < gEQ; i++) lodExte[i] = (lodFlow[i] + lodGrav[i]) + lodRepl[i];
        const std::vector<double> dspO = dsp, velO = vel, accO = acc;
        std::vector<double> dspn(gEQ);
        int iter = 1;
        for (; iter <= sp.ntolFEM; iter++) {
            std::fill(lodInte.begin(), lodInte.end(), 0.0);
            for (Segment &s : el) {
                s.form_stiff();
                s.body_stress(lodInte.data());
                s.update_matrix(coeffs, sp.GeoGamma, sp.dampM, sp.dampK);
            }
            for (int i = 0; i < gEQ; i++) lodEffe[i] = lodExte[i] - lodInte[i];
            for (const Segment &s : el)
                s.update_load(coeffs, sp.dampM, sp.dampK, dspO.data(), dsp.data(), vel.data(), acc.data(),
                              lodEffe.data());
            int rc = cg_solve(dspn, lodEffe, iter);
            if (rc) return rc;
            update_dsp_triad(iter, dspn, dnorm);
            if (dnorm <= sp.dtolFEM) break;
        }
        for (int i = 0; i < gEQ; i++) {
            acc[i] = (coeffs[0] * (dsp[i] - dspO[i]) - coeffs[2] * velO[i]) - coeffs[3] * accO[i];
            vel[i] = (velO[i] + coeffs[6] * accO[i]) + coeffs[7] * acc[i];
        }
        FishInfo[1] = (double)iter;
        FishInfo[2] = dnorm;
        if (!std::isfinite(dnorm)) return bfail(FSI_E_NAN, "beam Newton-Raphson: non-finite increment");
        return FSI_OK;
    }
};

extern "C" {

int fsi_beam_create(fsi_beam_t *out, const fsi_beam_params *solver, const fsi_beam_body *body, int nND, int nEL,
                    int nMT, const double *xyz, const double *material, const int *boundary, const int *elements,
                    double *Asfac, double *Lchod) {
    if (!out || !solver || !body || !xyz || !material || !boundary || !elements || nND < 2 || nEL < 1 || nMT < 1)
        return bfail(FSI_E_ARG, "fsi_beam_create: invalid argument");
    *out = nullptr;
    if (body->iBodyModel != 1 && body->iBodyModel != 2)
        return bfail(FSI_E_ARG, "no define body model %d (1 rigid, 2 elastic)", body->iBodyModel);
    if (solver->ntolFEM < 1) return bfail(FSI_E_ARG, "ntolFEM must be at least 1");
    fsi_beam *b = new (std::nothrow) fsi_beam();
    if (!b) return bfail(FSI_E_ARG, "out of host memory");
    b->sp = *solver;
    b->bd = *body;
    b->nND = nND;
    b->nEL = nEL;
    b->nMT = nMT;
    b->gEQ = 6 * nND;
    b->vBC.assign(b->gEQ, 0.0);
    b->el.assign(nEL, Segment());
    std::vector<char> built(nEL, 0);
    // Beam_ReadBuildElements: element tmpid = i, j, k, itype, imat, Nspan
    // (ids outside 1..nEL are skipped, as the reference does)
    for (int n = 0; n < nEL; n++) {
        const int *e = elements + 6 * n;
        const int tmpid = n + 1, i = e[0], j = e[1], itype = e[3], imat = e[4], Nspan = e[5];
        if (i < 1 || i > nND || j < 1 || j > nND || imat < 1 || imat > nMT || Nspan < 1) {
            delete b;
            return bfail(FSI_E_ARG, "element %d: nodes %d %d, material %d, Nspan %d out of range", tmpid, i, j, imat,
                         Nspan);
        }
        // Segment_Build (SolidSolver.f90:60-100)
        Segment &s = b->el[tmpid - 1];
        s.node0 = i - 1;
        s.node1 = j - 1;
        for (int k = 0; k < 8; k++) s.prop[k] = material[8 * (imat - 1) + k];
        for (int k = 0; k < 6; k++) {
            s.l2g[k] = 6 * s.node0 + k;
            s.l2g[k + 6] = 6 * s.node1 + k;
        }
        const double *p0 = xyz + 8 * s.node0, *p1 = xyz + 8 * s.node1;
        for (int k = 0; k < 3; k++) {
            s.x00[k] = p0[k];
            s.x00[6 + k] = p1[k];
            s.x00[3 + k] = 0.0;
            s.x00[9 + k] = 0.0;
        }
        const double ax = s.x00[6] - s.x00[0], ay = s.x00[7] - s.x00[1], az = s.x00[8] - s.x00[2];
        s.areaElem00 = std::sqrt((ax * ax + ay * ay) + az * az);
        for (int k = 0; k < 6; k++) {
            s.bc[k] = boundary[6 * s.node0 + k];
            s.bc[k + 6] = boundary[6 * s.node1 + k];
        }
        s.itype = itype;
        s.Nspan = Nspan;
        s.Lspan = 0.5 * (p0[3] + p1[3]);
        s.spanlen = 0.5 * (p0[4] + p1[4]) + s.Lspan;
        for (int k = 0; k < 3; k++) s.dirc00[k] = 0.5 * (p0[5 + k] + p1[5 + k]);
        const double dn = std::sqrt(dot3(s.dirc00, s.dirc00));
        if (dn > 1.0e-10) {
            for (double &v : s.dirc00) v = v / dn;
        } else {
            delete b;
            return bfail(FSI_E_ARG, "element %d: span directions of its nodes are opposite; no unique bisector exists",
                         tmpid);
        }
        built[n] = 1;
    }
    // Beam_cptAsfac
    double as = 0.0, mx = -HUGE_VAL, mn = HUGE_VAL;
    double c0 = HUGE_VAL, c1 = -HUGE_VAL, s0 = HUGE_VAL, s1 = -HUGE_VAL;
    for (const Segment &s : b->el) {
        as = as + s.areaElem00;
        mx = std::max(mx, s.areaElem00);
        mn = std::min(mn, s.areaElem00);
        c0 = std::min(c0, std::min(s.x00[0], s.x00[6]));
        c1 = std::max(c1, std::max(s.x00[0], s.x00[6]));
        s0 = std::min(s0, std::min(s.x00[1], s.x00[7]));
        s1 = std::max(s1, std::max(s.x00[1], s.x00[7]));
    }
    b->elmax = mx;
    b->elmin = mn;
    double lch = c1 - c0;
    if (s1 - s0 > lch) lch = s1 - s0;
    if (Asfac) *Asfac = as;
    if (Lchod) *Lchod = lch;
    // Beam_adjustBC: constrained end nodes take the body's prescribed DOFs
    for (Segment &s : b->el) {
        if (s.bc[0] == 1)
            for (int k = 0; k < 6; k++) s.bc[k] = b->bd.isMotionGiven[k];
        if (s.bc[6] == 1)
            for (int k = 0; k < 6; k++) s.bc[k + 6] = b->bd.isMotionGiven[k];
    }
    *out = b;
    return FSI_OK;
}

int fsi_beam_destroy(fsi_beam_t b) {
    delete b;
    return FSI_OK;
}

int fsi_beam_set_material(fsi_beam_t b, double Lref, double Uref, double denIn, const double uvwIn[3], double *uMax,
                          double *Lthck) {
    if (!b || !uvwIn || !uMax || !Lthck) return bfail(FSI_E_ARG, "fsi_beam_set_material: invalid argument");
    fsi_beam_body &d = b->bd;
    d.St = (Lref * d.Freq) / Uref;
    for (int k = 0; k < 3; k++) {
        d.AoAo[k] = (d.AoAo[k] / 180.0) * PI;
        d.AoAAmpl[k] = (d.AoAAmpl[k] / 180.0) * PI;
        d.AoAPhi[k] = (d.AoAPhi[k] / 180.0) * PI;
        d.XYZPhi[k] = (d.XYZPhi[k] / 180.0) * PI;
    }
    double ext[3] = {0.0, 0.0, 0.0};
    for (const Segment &s : b->el)
        for (int k = 0; k < 3; k++) ext[k] = std::max(ext[k], std::max(std::fabs(s.x00[k]), std::fabs(s.x00[6 + k])));
    const double rRot[3] = {std::max(ext[1], ext[2]), std::max(ext[0], ext[2]), std::max(ext[0], ext[1])};
    double au = 0.0, ax = 0.0, aa = 0.0;
    for (int k = 0; k < 3; k++) {
        au = std::max(au, std::fabs(uvwIn[k]));
        ax = std::max(ax, std::fabs(d.XYZAmpl[k]));
        aa = std::max(aa, std::fabs(d.AoAAmpl[k]) * rRot[k]);
    }
    *uMax = std::max(std::max(*uMax, au), std::max(((2.0 * PI) * ax) * d.Freq, ((2.0 * PI) * aa) * d.Freq));
    double nL = 0.0;
    if (b->sp.isKB == 0) {
        for (Segment &s : b->el) {
            const double len = s.spanlen;
            double *p = s.prop;
            p[0] = (d.EmR * denIn) * (Uref * Uref);
            p[1] = p[0] / (2.0 * (1.0 + d.psR));
            nL = d.tcR * Lref;
            p[2] = len * nL;
            p[3] = (((d.denR * len) * Lref) * denIn) / p[2];
            const double ratio = nL / len, r2 = ratio * ratio, r5 = (r2 * r2) * ratio;
            p[5] = ((len * ((nL * nL) * nL)) / 3.0) * ((1.0 - 0.63 * ratio) + 0.052 * r5);
            p[6] = (len * ((nL * nL) * nL)) / 12.0;
            p[7] = (nL * ((len * len) * len)) / 12.0;
        }
        const Segment &s = b->el[0];
        const double len = s.spanlen;
        d.KB = (s.prop[0] * s.prop[6]) / (((denIn * (Uref * Uref)) * ((Lref * Lref) * Lref)) * len);
        d.KS = (s.prop[0] * s.prop[2]) / (((denIn * (Uref * Uref)) * Lref) * len);
    } else if (b->sp.isKB == 1) {
        for (Segment &s : b->el) {
            const double len = s.spanlen;
            double *p = s.prop;
            nL = std::sqrt((d.KB / d.KS) * 12.0) * Lref;
            p[2] = len * nL;
            p[0] = ((((d.KS * denIn) * (Uref * Uref)) * Lref) * len) / p[2];
            p[1] = p[0] / (2.0 * (1.0 + d.psR));
            p[3] = (((d.denR * len) * Lref) * denIn) / p[2];
            const double ratio = nL / len, r2 = ratio * ratio, r5 = (r2 * r2) * ratio;
            p[5] = ((len * ((nL * nL) * nL)) / 3.0) * ((1.0 - 0.63 * ratio) + 0.052 * r5);
            p[6] = (len * ((nL * nL) * nL)) / 12.0;
            p[7] = (nL * ((len * len) * len)) / 12.0;
        }
        const Segment &s = b->el[0];
        const double len = s.spanlen;
        nL = s.prop[2] / len;
        d.EmR = s.prop[0] / (denIn * (Uref * Uref));
        d.tcR = nL / Lref;
    }
    *Lthck = nL;
    return FSI_OK;
}

int fsi_beam_initialise(fsi_beam_t b, double time, int *M) {
    if (!b) return bfail(FSI_E_ARG, "null beam");
    const M3 I = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
    memcpy(b->TTT00, I, sizeof(M3));
    b->translation(time);
    aoa_to_ttt(b->AoA, b->TTT0);
    aoa_to_ttt(b->AoA, b->TTTnxt);
    angle_triad(b->TTT0, b->TTTnxt, b->AoAd[0], b->AoAd[1], b->AoAd[2]);
    for (Segment &s : b->el) {
        s.map_pos(s.x0, b->TTT0, b->XYZ, b->AoAd);
        s.map_dir(s.dirc0, b->TTT0);
        s.init();
    }
    // Beam_InitLoad, Beam_InitPosDspVelAcc
    const int g = b->gEQ;
    for (auto *v : {&b->lodInte, &b->lodExte, &b->lodEffe, &b->lodFlow, &b->lodRepl, &b->lodGrav}) v->assign(g, 0.0);
    b->pos.assign(g, 0.0);
    for (const Segment &s : b->el)
        for (int k = 0; k < 6; k++) {
            b->pos[6 * s.node0 + k] = s.x1[k];
            b->pos[6 * s.node1 + k] = s.x1[k + 6];
        }
    b->dsp.assign(g, 0.0);
    b->vel.assign(g, 0.0);
    b->acc.assign(g, 0.0);
    b->mss.assign(3 * (size_t)b->nND, 0.0);
    if (b->bd.iBodyModel == 1) {
        b->translation_velocity(time);
        b->rotation_rate(time, b->TTT0);
        b->vel_from_angular(b->WWW3, b->UVW);
    }
    // Beam_InitTriadANDFormMass
    for (Segment &s : b->el) {
        s.init_triad();
        s.form_mass();
        s.rotate_matrix();
        s.rkr(s.mas);
    }
    // Beam_InitGrav
    double gvec[NE] = {};
    for (int k = 0; k < 3; k++) gvec[k] = gvec[6 + k] = b->sp.g[k];
    for (const Segment &s : b->el) {
        double gr[NE];
        s.mass_multiply(gvec, gr);
        s.loc_to_global(gr, b->lodGrav.data());
        for (int j = 0; j < 3; j++) {
            b->mss[3 * s.node0 + j] = b->mss[3 * s.node0 + j] + s.mas[j][j];
            b->mss[3 * s.node1 + j] = b->mss[3 * s.node1 + j] + s.mas[j + 6][j + 6];
        }
    }
    // PlateBuild_: rtov, vtor
    b->rtov.assign(b->nEL + 1, 0);
    int cnt = 0;
    for (int i = 0; i < b->nEL; i++) {
        b->rtov[i] = cnt;
        cnt += b->el[i].Nspan;
    }
    b->rtov[b->nEL] = cnt;
    b->M = cnt;
    b->vtor.assign(cnt, 0);
    for (int i = 0; i < b->nEL; i++)
        for (int j = b->rtov[i]; j < b->rtov[i + 1]; j++) b->vtor[j] = i;
    b->initialised = true;
    if (M) *M = cnt;
    return FSI_OK;
}

int fsi_beam_markers(fsi_beam_t b, double alpha, double denIn, double *xyz, double *vel, double *area) {
    if (!b || !xyz || !vel || !area) return bfail(FSI_E_ARG, "fsi_beam_markers: invalid argument");
    if (!b->initialised) return bfail(FSI_E_STATE, "fsi_beam_markers before fsi_beam_initialise");
    const double beta = -((alpha * 2.0) * denIn);
    for (int i = 0; i < b->nEL; i++) {
        const Segment &s = b->el[i];
        const int i1 = s.node0, i2 = s.node1;
        double txyz[3], tvel[3], om[3], dirc[3];
        for (int k = 0; k < 3; k++) {
            txyz[k] = 0.5 * (b->pos[6 * i1 + k] + b->pos[6 * i2 + k]);
            tvel[k] = 0.5 * (b->vel[6 * i1 + k] + b->vel[6 * i2 + k]);
            om[k] = 0.5 * (b->vel[6 * i1 + 3 + k] + b->vel[6 * i2 + 3 + k]);
        }
        const double left = s.Lspan, len = s.spanlen;
        const double dl = len / (double)s.Nspan;
        const double dh = s.len1;
        const double a = (dl * dh) * beta;
        // spanwise direction: the mean of the nodal triads' second axes
        for (int k = 0; k < 3; k++) dirc[k] = 0.5 * (s.n1[k][1] + s.n2[k][1]);
        const double dn = std::sqrt(dot3(dirc, dirc));
        if (dn > 1.0e-12) {
            for (double &v : dirc) v = v / dn;
        } else {
            for (int k = 0; k < 3; k++) dirc[k] = s.ee[k][1];
        }
        const int cnt = b->rtov[i];
        for (int sp = 1; sp <= s.Nspan; sp++) {
            const double ls = dl * (0.5 + (double)(sp - 1)) - left;
            const double r[3] = {dirc[0] * ls, dirc[1] * ls, dirc[2] * ls};
            const double w[3] = {om[1] * r[2] - om[2] * r[1], om[2] * r[0] - om[0] * r[2], om[0] * r[1] - om[1] * r[0]};
            const int m = cnt + sp - 1;
            for (int k = 0; k < 3; k++) {
                xyz[3 * m + k] = txyz[k] + r[k];
                vel[3 * m + k] = tvel[k] + w[k];
            }
            area[m] = a;
        }
    }
    return FSI_OK;
}

int fsi_beam_load(fsi_beam_t b, const double *xyz, const double *eforce) {
    if (!b || !xyz || !eforce) return bfail(FSI_E_ARG, "fsi_beam_load: invalid argument");
    if (!b->initialised) return bfail(FSI_E_STATE, "fsi_beam_load before fsi_beam_initialise");
    std::fill(b->lodFlow.begin(), b->lodFlow.end(), 0.0);
    double *L = b->lodFlow.data();
    for (int m = 0; m < b->M; m++) {
        const double *f = eforce + 3 * m;
        const Segment &s = b->el[b->vtor[m]];
        double rr[3], mo[3];
        for (int k = 0; k < 3; k++) rr[k] = xyz[3 * m + k] - 0.5 * (s.x1[k] + s.x1[6 + k]);
        mo[0] = rr[1] * f[2] - rr[2] * f[1];
        mo[1] = rr[2] * f[0] - rr[0] * f[2];
        mo[2] = rr[0] * f[1] - rr[1] * f[0];
        for (int k = 0; k < 3; k++) {
            L[s.l2g[k]] = L[s.l2g[k]] + 0.5 * f[k];
            L[s.l2g[6 + k]] = L[s.l2g[6 + k]] + 0.5 * f[k];
            L[s.l2g[3 + k]] = L[s.l2g[3 + k]] + 0.5 * mo[k];
            L[s.l2g[9 + k]] = L[s.l2g[9 + k]] + 0.5 * mo[k];
        }
    }
    return FSI_OK;
}

int fsi_beam_structure(fsi_beam_t b, double time, int isubstep, double deltat, double subdeltat, int *iters,
                       double *dnorm) {
    if (!b) return bfail(FSI_E_ARG, "null beam");
    if (!b->initialised) return bfail(FSI_E_STATE, "fsi_beam_structure before fsi_beam_initialise");
    const double t = (time - deltat) + (double)isubstep * subdeltat;
    b->translation(t);
    aoa_to_ttt(b->AoA, b->TTTnxt);
    angle_triad(b->TTT0, b->TTTnxt, b->AoAd[0], b->AoAd[1], b->AoAd[2]);
    int rc = FSI_OK;
    if (b->bd.iBodyModel == 1) {
        for (Segment &s : b->el) {
            s.map_pos(s.xnxt, b->TTTnxt, b->XYZ, b->AoAd);
            s.map_dir(s.dircnxt, b->TTTnxt);
            memcpy(s.x1, s.xnxt, sizeof(s.x1));
            memcpy(s.dirc1, s.dircnxt, sizeof(s.dirc1));
            for (int k = 0; k < 6; k++) {
                b->pos[6 * s.node0 + k] = s.x1[k];
                b->pos[6 * s.node1 + k] = s.x1[k + 6];
            }
            s.cptdxyz1();
            s.rigid_update_triad();
        }
        b->translation_velocity(t);
        b->rotation_rate(t, b->TTTnxt);
        b->vel_from_angular(b->WWW3, b->UVW);
        b->FishInfo[1] = 0.0;
        b->FishInfo[2] = 0.0;
    } else {
        for (Segment &s : b->el) s.map_pos(s.xnxt, b->TTTnxt, b->XYZ, b->AoAd);
        b->newmark(subdeltat);
        rc = b->solve();
    }
    if (iters) *iters = (int)b->FishInfo[1];
    if (dnorm) *dnorm = b->FishInfo[2];
    return rc;
}

int fsi_beam_state(fsi_beam_t b, double *pos, double *dsp, double *vel, double *acc, double *lodFlow) {
    if (!b) return bfail(FSI_E_ARG, "null beam");
    if (!b->initialised) return bfail(FSI_E_STATE, "fsi_beam_state before fsi_beam_initialise");
    const size_t n = sizeof(double) * (size_t)b->gEQ;
    if (pos) memcpy(pos, b->pos.data(), n);
    if (dsp) memcpy(dsp, b->dsp.data(), n);
    if (vel) memcpy(vel, b->vel.data(), n);
    if (acc) memcpy(acc, b->acc.data(), n);
    if (lodFlow) memcpy(lodFlow, b->lodFlow.data(), n);
    return FSI_OK;
}

int fsi_beam_info(fsi_beam_t b, int *nND, int *nEL, double XYZ[3]) {
    if (!b) return bfail(FSI_E_ARG, "null beam");
    if (nND) *nND = b->nND;
    if (nEL) *nEL = b->nEL;
    if (XYZ)
        for (int k = 0; k < 3; k++) XYZ[k] = b->XYZ[k];
    return FSI_OK;
}

}  // extern "C"
