/* hyb_host_couette.c -- a native host of the C ABI, in the call sequence the
 * patched Fortran host makes (the patch of Hybrid_Time_advance_LU_SGS and
 * output):
 *
 *   hyb_create(mesh, vgrid, params)      after init / init_flow_zero
 *   hyb_init_maxwellian(ctx, 1, 0, 0, 1)
 *   hyb_step(ctx, 1, &res)                once per outer iteration
 *   hyb_download_moments(ctx, S, CF)      output
 *   hyb_download_f(ctx, FRD)              backup_Macro_write
 *   hyb_destroy(ctx)
 *
 * The host owns its arrays in the reference's layouts: node coordinates
 * (nx, ny) column-major, S_GKUA(Nsum,-3:nx+3,-3:ny+3), CF(-1:nx+1,-1:ny+1),
 * FRD(NRD,-3:nx+3,-3:ny+3,NVI,NVJ).  Test infrastructure: it reads the case
 * from a binary file written by the test and writes what it downloaded.
 *
 * input:  int32 magic, sizeof(hyb_params), nx, ny, nvi, nvj, nsteps, bc[4];
 *         hyb_params; x[nx*ny]; y[nx*ny]; vi, wi; vj, wj; for each wall face
 *         in face order u, v, t (one value per face cell)
 * output: nsteps hyb_residual records; S; CF; FRD
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hyb_dvm.h"

#define MAGIC 0x48594231

static void *read_n(FILE *fp, size_t bytes) {
    void *p = malloc(bytes ? bytes : 1);
    if (!p || fread(p, 1, bytes, fp) != bytes) {
        fprintf(stderr, "short input\n");
        exit(2);
    }
    return p;
}

int main(int argc, char **argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
        return 2;
    }
    FILE *in = fopen(argv[1], "rb");
    if (!in) {
        perror(argv[1]);
        return 2;
    }
    int hdr[11];
    if (fread(hdr, sizeof(int), 11, in) != 11 || hdr[0] != MAGIC || hdr[1] != (int)sizeof(hyb_params)) {
        fprintf(stderr, "bad header (hyb_params is %d bytes here)\n", (int)sizeof(hyb_params));
        return 2;
    }
    const int nx = hdr[2], ny = hdr[3], nvi = hdr[4], nvj = hdr[5], nsteps = hdr[6];
    hyb_params prm;
    if (fread(&prm, sizeof prm, 1, in) != 1) return 2;
    hyb_mesh mesh;
    memset(&mesh, 0, sizeof mesh);
    mesh.nx = nx;
    mesh.ny = ny;
    double *x = read_n(in, sizeof(double) * nx * ny), *y = read_n(in, sizeof(double) * nx * ny);
    mesh.x = x;
    mesh.y = y;
    hyb_vgrid vg;
    vg.nvi = nvi;
    vg.nvj = nvj;
    double *vi = read_n(in, sizeof(double) * nvi), *wi = read_n(in, sizeof(double) * nvi);
    double *vj = read_n(in, sizeof(double) * nvj), *wj = read_n(in, sizeof(double) * nvj);
    vg.vi = vi;
    vg.wi = wi;
    vg.vj = vj;
    vg.wj = wj;
    double *walls[4][3] = {{0}};
    for (int f = 0; f < 4; f++) {
        mesh.bc[f] = hdr[7 + f];
        if (mesh.bc[f] != HYB_BC_WALL) continue;
        const int n = (f == 0 || f == 2) ? ny - 1 : nx - 1;
        for (int k = 0; k < 3; k++) walls[f][k] = read_n(in, sizeof(double) * n);
        mesh.wall_u[f] = walls[f][0];
        mesh.wall_v[f] = walls[f][1];
        mesh.wall_t[f] = walls[f][2];
    }
    fclose(in);

    hyb_ctx *ctx = NULL;
    int rc = hyb_create(&mesh, &vg, &prm, &ctx);
    if (rc != HYB_OK) {
        fprintf(stderr, "hyb_create: %d\n", rc);
        return 1;
    }
    rc = hyb_init_maxwellian(ctx, 1.0, 0.0, 0.0, 1.0);
    hyb_residual *res = calloc((size_t)nsteps, sizeof(hyb_residual));
    for (int k = 0; k < nsteps && rc == HYB_OK; k++) rc = hyb_step(ctx, 1, &res[k]);
    if (rc != HYB_OK) {
        fprintf(stderr, "step: %d (%s)\n", rc, hyb_last_error(ctx));
        hyb_destroy(ctx);
        return 1;
    }
    const size_t P = (size_t)(nx + 7) * (ny + 7);
    const size_t ncf = (size_t)(nx + 3) * (ny + 3);
    const size_t nfrd = (size_t)HYB_NRD * P * nvi * nvj;
    double *S = malloc(sizeof(double) * HYB_NSUM * P), *CF = malloc(sizeof(double) * ncf);
    double *FRD = malloc(sizeof(double) * nfrd);
    rc = hyb_download_moments(ctx, S, CF);
    if (rc == HYB_OK) rc = hyb_download_f(ctx, FRD);
    hyb_destroy(ctx);
    if (rc != HYB_OK) {
        fprintf(stderr, "download: %d\n", rc);
        return 1;
    }
    FILE *out = fopen(argv[2], "wb");
    if (!out) {
        perror(argv[2]);
        return 2;
    }
    fwrite(res, sizeof(hyb_residual), (size_t)nsteps, out);
    fwrite(S, sizeof(double), HYB_NSUM * P, out);
    fwrite(CF, sizeof(double), ncf, out);
    fwrite(FRD, sizeof(double), nfrd, out);
    fclose(out);
    printf("hyb_host_couette: %d steps, max rms residual %.6e\n", nsteps, res[nsteps - 1].max_rms);
    return 0;
}
