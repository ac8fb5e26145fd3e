/* A C host that drives one block with a plate through libfsi_gpu as a
 * Fortran or C program would (tests/test_c_host_gpu.py builds it with
 * -std=c99 -pedantic -Werror and compares its output with the oracle).
 *
 * It reads a case file, creates the block from a descriptor filled field by
 * field, uploads the initial fIn(z,y,x,0:18) in the reference's column-major
 * layout, then makes one fsi_block_ib_step call per time step with the
 * markers of that step (LBMBlockComm.f90:279-305: the IB stage, then the
 * fluid step), and writes every step's Lagrangian force and iteration count
 * and the final fIn.
 *
 * Case file (native byte order):
 *   int32  X, Y, Z, iCollidModel, precision, bnd[6], M, K, ntol
 *   double dh, nu, denIn, uvwIn[3], dtol, Uref
 *   double m_collid[361], m_force[361]   (used for iCollidModel 3)
 *   double fIn[19 X Y Z]
 *   K x { double blktime, vf[3], xyz[3M], vel[3M], area[M] }
 * Output file:
 *   K x { int32 iters, int32 rc, double residual, double eforce[3M] }
 *   double fIn[19 X Y Z]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fsi_gpu.h"

static int rd(FILE *f, void *p, size_t size, size_t n) { return fread(p, size, n, f) == n ? 0 : 1; }

static int fail(const char *what, int rc) {
    char msg[256];
    fsi_last_error(msg, (int)sizeof msg);
    fprintf(stderr, "%s: %d %s\n", what, rc, msg);
    return 1;
}

int main(int argc, char **argv) {
    int hdr[14];
    double par[8];
    double *mc, *mf, *fin, *xyz, *vel, *area, *ef;
    double vf[3], blktime, residual;
    fsi_block_desc d;
    fsi_block_t h = NULL;
    FILE *in, *out;
    long long N;
    int X, Y, Z, M, K, ntol, k, s, rc, iters;

    if (argc != 3) return 2;
    in = fopen(argv[1], "rb");
    out = fopen(argv[2], "wb");
    if (!in || !out) return 2;
    if (rd(in, hdr, sizeof(int), 14) || rd(in, par, sizeof(double), 8)) return 3;
    X = hdr[0]; Y = hdr[1]; Z = hdr[2];
    M = hdr[11]; K = hdr[12]; ntol = hdr[13];
    N = (long long)X * Y * Z;
    mc = malloc(sizeof(double) * 361);
    mf = malloc(sizeof(double) * 361);
    fin = malloc(sizeof(double) * 19 * (size_t)N);
    xyz = malloc(sizeof(double) * 3 * (size_t)M);
    vel = malloc(sizeof(double) * 3 * (size_t)M);
    area = malloc(sizeof(double) * (size_t)M);
    ef = malloc(sizeof(double) * 3 * (size_t)M);
    if (!mc || !mf || !fin || !xyz || !vel || !area || !ef) return 4;
    if (rd(in, mc, sizeof(double), 361) || rd(in, mf, sizeof(double), 361)) return 3;
    if (rd(in, fin, sizeof(double), 19 * (size_t)N)) return 3;

    memset(&d, 0, sizeof d);
    d.xDim = X;
    d.yDim = Y;
    d.zDim = Z;
    d.dh = par[0];
    for (k = 0; k < 6; k++) d.bndConds[k] = hdr[5 + k];
    d.iCollidModel = hdr[3];
    d.nu = par[1];
    d.m_collid = hdr[3] == 3 ? mc : NULL;
    d.m_force = hdr[3] == 3 ? mf : NULL;
    d.precision = hdr[4];
    d.denIn = par[2];
    for (k = 0; k < 3; k++) d.uvwIn[k] = par[3 + k];
    if ((rc = fsi_block_create(&h, &d))) return fail("create", rc);
    if ((rc = fsi_block_initialise(h, 0.0))) return fail("initialise", rc);
    if ((rc = fsi_block_set_boundary_conditions(h, 0.0))) return fail("set_boundary_conditions", rc);
    if ((rc = fsi_block_upload_f(h, fin))) return fail("upload_f", rc);
    if ((rc = fsi_ib_set_bodies(h, 1, &M, d.bndConds))) return fail("ib_set_bodies", rc);

    for (s = 0; s < K; s++) {
        if (rd(in, &blktime, sizeof(double), 1) || rd(in, vf, sizeof(double), 3) ||
            rd(in, xyz, sizeof(double), 3 * (size_t)M) || rd(in, vel, sizeof(double), 3 * (size_t)M) ||
            rd(in, area, sizeof(double), (size_t)M))
            return 3;
        iters = 0;
        residual = 0.0;
        rc = fsi_block_ib_step(h, xyz, vel, area, vf, d.denIn, d.dh, par[7], ntol, par[6], blktime, ef, &iters,
                               &residual);
        fwrite(&iters, sizeof(int), 1, out);
        fwrite(&rc, sizeof(int), 1, out);
        fwrite(&residual, sizeof(double), 1, out);
        fwrite(ef, sizeof(double), 3 * (size_t)M, out);
        if (rc) return fail("ib_step", rc);
    }
    if ((rc = fsi_block_download_f(h, fin))) return fail("download_f", rc);
    fwrite(fin, sizeof(double), 19 * (size_t)N, out);
    if ((rc = fsi_block_destroy(h))) return fail("destroy", rc);
    fclose(in);
    fclose(out);
    free(mc);
    free(mf);
    free(fin);
    free(xyz);
    free(vel);
    free(area);
    free(ef);
    return 0;
}
