/* plate_loop.c -- a C host time loop over one block with a rigid heaving
 * plate, making the calls a compiled host (the reference's Fortran main loop,
 * LBMBlockComm.f90:279-305) makes through include/fsi_gpu.h: per step the
 * plate's markers (prescribed heave, PlateUpdatePosVelArea_ for a flat plate:
 * element mid-points plus span stations, Solidbody.f90:604-646), one
 * fsi_block_ib_step (or fsi_block_ib_step_async, the next markers, then
 * fsi_block_ib_wait), and the drag and lift sums of the returned force.
 * bench.py builds and runs it to time the 160x96x96 plate case without an
 * interpreter in the loop.
 *
 * usage: plate_loop X Y Z dh nu U ntol dtol steps warmup async n_chord n_span
 *                   chord span le_x le_y le_z heave_amp freq
 * prints one line: ms_per_step mlups cd_last cl_last
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "fsi_gpu.h"

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

typedef struct {
    int nc, ns, M;
    double chord, span, le[3], amp, freq;
} plate_t;

/* rigid heave XYZ = le + (0, amp cos(2 pi f t), 0); markers at the element
 * mid-points of the chord-wise beam plus span stations along z; area =
 * dl * element length * (-2 alpha denIn) with alpha = denIn = 1 */
static void plate_markers(const plate_t *p, double t, double *xyz, double *vel, double *area) {
    const double pi = 3.141592653589793;
    const double arg = 2.0 * pi * p->freq * t;
    const double dy = p->amp * cos(arg), vy = -2.0 * pi * p->freq * p->amp * sin(arg);
    const double dl = p->span / p->ns, ls0 = 0.5 * p->span;
    int i, s, m = 0;
    for (i = 0; i < p->nc; i++) {
        const double x0 = p->le[0] + p->chord * i / p->nc, x1 = p->le[0] + p->chord * (i + 1) / p->nc;
        const double xm = 0.5 * (x0 + x1), len = x1 - x0;
        for (s = 0; s < p->ns; s++, m++) {
            xyz[3 * m] = xm;
            xyz[3 * m + 1] = p->le[1] + dy;
            xyz[3 * m + 2] = p->le[2] + (dl * (0.5 + s) - ls0);
            vel[3 * m] = 0.0;
            vel[3 * m + 1] = vy;
            vel[3 * m + 2] = 0.0;
            area[m] = dl * len * -2.0;
        }
    }
}

static int fail(const char *what, int rc) {
    char msg[256];
    fsi_last_error(msg, (int)sizeof msg);
    fprintf(stderr, "%s: %d %s\n", what, rc, msg);
    return 1;
}

int main(int argc, char **argv) {
    fsi_block_desc d;
    fsi_block_t h = NULL;
    plate_t p;
    double *xyz[2], *vel[2], *area[2], *ef;
    double vf[3] = {0.0, 0.0, 0.0}, U, dh, t = 0.0, res = 0.0, cd = 0.0, cl = 0.0, t0, t1;
    int X, Y, Z, ntol, steps, warmup, async, it = 0, k, s, rc, cur = 0;
    double dtol;
    if (argc != 21) {
        fprintf(stderr, "usage: plate_loop X Y Z dh nu U ntol dtol steps warmup async n_chord n_span chord span "
                        "le_x le_y le_z heave_amp freq\n");
        return 2;
    }
    X = atoi(argv[1]); Y = atoi(argv[2]); Z = atoi(argv[3]);
    dh = atof(argv[4]);
    U = atof(argv[6]);
    ntol = atoi(argv[7]); dtol = atof(argv[8]);
    steps = atoi(argv[9]); warmup = atoi(argv[10]); async = atoi(argv[11]);
    p.nc = atoi(argv[12]); p.ns = atoi(argv[13]);
    p.chord = atof(argv[14]); p.span = atof(argv[15]);
    for (k = 0; k < 3; k++) p.le[k] = atof(argv[16 + k]);
    p.amp = atof(argv[19]); p.freq = atof(argv[20]);
    p.M = p.nc * p.ns;

    memset(&d, 0, sizeof d);
    d.xDim = X; d.yDim = Y; d.zDim = Z;
    d.dh = dh;
    d.bndConds[0] = 101; d.bndConds[1] = 104;
    for (k = 2; k < 6; k++) d.bndConds[k] = 101;
    d.iCollidModel = 3;
    d.nu = atof(argv[5]);
    d.precision = FSI_PREC_F16;
    d.denIn = 1.0;
    d.uvwIn[0] = U;
    if ((rc = fsi_block_create(&h, &d))) return fail("create", rc);
    if ((rc = fsi_block_initialise(h, 0.0))) return fail("initialise", rc);
    if ((rc = fsi_block_set_boundary_conditions(h, 0.0))) return fail("set_boundary_conditions", rc);
    if ((rc = fsi_ib_set_bodies(h, 1, &p.M, d.bndConds))) return fail("ib_set_bodies", rc);
    for (k = 0; k < 2; k++) {
        xyz[k] = malloc(sizeof(double) * 3 * (size_t)p.M);
        vel[k] = malloc(sizeof(double) * 3 * (size_t)p.M);
        area[k] = malloc(sizeof(double) * (size_t)p.M);
        if (!xyz[k] || !vel[k] || !area[k]) return 4;
    }
    ef = malloc(sizeof(double) * 3 * (size_t)p.M);
    if (!ef) return 4;

    plate_markers(&p, t, xyz[cur], vel[cur], area[cur]);
    t0 = 0.0;
    for (s = 0; s < warmup + steps; s++) {
        if (s == warmup) {
            if ((rc = fsi_block_timer(h, 0, NULL))) return fail("timer", rc);
            t0 = now_s();
        }
        if (async) {
            rc = fsi_block_ib_step_async(h, xyz[cur], vel[cur], area[cur], vf, 1.0, dh, U, ntol, dtol, t + dh);
            if (rc) return fail("ib_step_async", rc);
            t += dh;
            cur ^= 1;
            plate_markers(&p, t, xyz[cur], vel[cur], area[cur]);  /* beside the GPU step */
            if ((rc = fsi_block_ib_wait(h, ef, &it, &res))) return fail("ib_wait", rc);
        } else {
            rc = fsi_block_ib_step(h, xyz[cur], vel[cur], area[cur], vf, 1.0, dh, U, ntol, dtol, t + dh, ef, &it,
                                   &res);
            if (rc) return fail("ib_step", rc);
            t += dh;
            plate_markers(&p, t, xyz[cur], vel[cur], area[cur]);
        }
        /* drag and lift sums over Fref = 0.5 denIn U^2 area (Solidbody.f90:278) */
        cd = 0.0;
        cl = 0.0;
        for (k = 0; k < p.M; k++) {
            cd += ef[3 * k];
            cl += ef[3 * k + 1];
        }
        cd /= 0.5 * U * U * p.chord * p.span;
        cl /= 0.5 * U * U * p.chord * p.span;
    }
    {
        float ms = 0.0f;
        if ((rc = fsi_block_timer(h, 1, &ms))) return fail("timer", rc);
    }
    t1 = now_s();
    {
        const double ms_step = (t1 - t0) * 1e3 / steps;
        printf("%.6f %.1f %.9e %.9e\n", ms_step, (double)X * Y * Z / (ms_step * 1e-3) / 1e6, cd, cl);
    }
    if ((rc = fsi_block_destroy(h))) return fail("destroy", rc);
    for (k = 0; k < 2; k++) {
        free(xyz[k]);
        free(vel[k]);
        free(area[k]);
    }
    free(ef);
    return 0;
}
