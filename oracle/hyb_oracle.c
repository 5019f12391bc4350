/*
 * hyb_oracle.c -- CPU FP64 restatement of the Hybrid2D kinetic hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see hyb_oracle.h).  Compiled with
 * -ffp-contract=off so that x86_64 and aarch64 builds round identically.
 *
 * Reference files restated here (paths inside the reference project):
 *   Hybrid2D/src/GKUA_Residual.f90        GKUA_Residual, RHSFDVsub, Get_Feq
 *   Hybrid2D/src/GKUA_DETFP.f90           DETFP, GaussLegendre (moments)
 *   Hybrid2D/src/GKUA_DETFP_RES.f90       DETFP_res, GaussLegendre_rs
 *   Hybrid2D/src/GKUA_boundary.f90        GKUA_Phy_boundary, wall extrapolation,
 *                                         inner (block-connection) exchanges
 *   Hybrid2D/src/GKUA_wall_functions.f90  GKUA_wall_boundary, NWGaussLegendre
 *   Hybrid2D/src/GKUA_DETFP_WALL.f90      GKUA_DET_wall, DETFPwall
 *   Hybrid2D/src/GKUA_lisansudu.f90       velocity grids
 *   Hybrid2D/src/GKUA_sudufenbu.f90       Maxwellian initial state
 *   Hybrid2D/src/sub_init.f90             metrics, ghost nodes, constants
 *   Hybrid2D/src/Hybrid_Sub.f90           outer iteration, Convert_NS
 *   Hybrid2D/src/sub_Residual.f90         get_viscous (used by Convert_NS)
 *   Hybrid2D/src/Functions.f90            FMINMD
 */
#include "hyb_oracle_impl.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static double pos_part(double a) { return (a + fabs(a)) * 0.5; }
static double neg_part(double a) { return (a - fabs(a)) * 0.5; }

/* FMINMD, Hybrid2D/src/Functions.f90:10-25 */
static double fminmd(double x, double y)
{
    if ((x > 0.0 && y > 0.0) || (x < 0.0 && y < 0.0))
        return (fabs(x) <= fabs(y)) ? x : y;
    return 0.0;
}

int orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* number of cells along a face, in face order (faces 2/4: i, faces 1/3: j) */
static int face_cells(const orc *o, int f) { return (f == 1 || f == 3) ? o->ny - 1 : o->nx - 1; }

/* ---- geometry: Creat_Mesh (sub_init.f90:178-208) and
 *      Update_coordinate_buffer_onemesh (sub_init.f90:719-823) ------------- */
static void build_geometry(orc *o, const double *x, const double *y)
{
    const int nx = o->nx, ny = o->ny;
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            o->xn[XN(o, i, j)] = x[(size_t)(i - 1) + (size_t)nx * (j - 1)];
            o->yn[XN(o, i, j)] = y[(size_t)(i - 1) + (size_t)nx * (j - 1)];
        }
    for (int j = 1; j <= ny - 1; j++)
        for (int i = 1; i <= nx - 1; i++) {
            const double *X = o->xn, *Y = o->yn;
            o->vol[MI(o, i, j)] =
                fabs((X[XN(o, i, j)] - X[XN(o, i + 1, j + 1)]) * (Y[XN(o, i + 1, j)] - Y[XN(o, i, j + 1)]) -
                     (X[XN(o, i + 1, j)] - X[XN(o, i, j + 1)]) * (Y[XN(o, i, j)] - Y[XN(o, i + 1, j + 1)])) * 0.5;
        }
    for (int j = 1; j <= ny - 1; j++)
        for (int i = 1; i <= nx; i++) {
            double dx = o->xn[XN(o, i, j + 1)] - o->xn[XN(o, i, j)];
            double dy = o->yn[XN(o, i, j + 1)] - o->yn[XN(o, i, j)];
            double s = sqrt(dx * dx + dy * dy);
            o->si[MI(o, i, j)] = s;
            o->ni1[MI(o, i, j)] = dy / s;
            o->ni2[MI(o, i, j)] = -dx / s;
        }
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx - 1; i++) {
            double dx = o->xn[XN(o, i + 1, j)] - o->xn[XN(o, i, j)];
            double dy = o->yn[XN(o, i + 1, j)] - o->yn[XN(o, i, j)];
            double s = sqrt(dx * dx + dy * dy);
            o->sj[MI(o, i, j)] = s;
            o->nj1[MI(o, i, j)] = -dy / s;
            o->nj2[MI(o, i, j)] = dx / s;
        }
    /* ghost nodes.  Inner (periodic) faces copy the partner face's nodes
     * (sub_init.f90:746-775); for a block connected to itself the partner
     * nodes are shifted by the period vector so the ghost cells keep their
     * true geometry.  Other faces extrapolate linearly (:779-796). */
    for (int f = 1; f <= 4; f++) {
        for (int l = 1; l <= LAP; l++) {
            if (f == 1 || f == 3) {
                for (int j = 1; j <= ny; j++) {
                    double *X = o->xn, *Y = o->yn;
                    double px = X[XN(o, nx, j)] - X[XN(o, 1, j)], py = Y[XN(o, nx, j)] - Y[XN(o, 1, j)];
                    if (f == 1) {
                        if (o->bc[0] == HYB_BC_PERIODIC) {
                            X[XN(o, 1 - l, j)] = X[XN(o, nx - l, j)] - px;
                            Y[XN(o, 1 - l, j)] = Y[XN(o, nx - l, j)] - py;
                        } else {
                            X[XN(o, 1 - l, j)] = 2.0 * X[XN(o, 1, j)] - X[XN(o, 1 + l, j)];
                            Y[XN(o, 1 - l, j)] = 2.0 * Y[XN(o, 1, j)] - Y[XN(o, 1 + l, j)];
                        }
                    } else {
                        if (o->bc[2] == HYB_BC_PERIODIC) {
                            X[XN(o, nx + l, j)] = X[XN(o, 1 + l, j)] + px;
                            Y[XN(o, nx + l, j)] = Y[XN(o, 1 + l, j)] + py;
                        } else {
                            X[XN(o, nx + l, j)] = 2.0 * X[XN(o, nx, j)] - X[XN(o, nx - l, j)];
                            Y[XN(o, nx + l, j)] = 2.0 * Y[XN(o, nx, j)] - Y[XN(o, nx - l, j)];
                        }
                    }
                }
            } else {
                for (int i = 1; i <= nx; i++) {
                    double *X = o->xn, *Y = o->yn;
                    double px = X[XN(o, i, ny)] - X[XN(o, i, 1)], py = Y[XN(o, i, ny)] - Y[XN(o, i, 1)];
                    if (f == 2) {
                        if (o->bc[1] == HYB_BC_PERIODIC) {
                            X[XN(o, i, 1 - l)] = X[XN(o, i, ny - l)] - px;
                            Y[XN(o, i, 1 - l)] = Y[XN(o, i, ny - l)] - py;
                        } else {
                            X[XN(o, i, 1 - l)] = 2.0 * X[XN(o, i, 1)] - X[XN(o, i, 1 + l)];
                            Y[XN(o, i, 1 - l)] = 2.0 * Y[XN(o, i, 1)] - Y[XN(o, i, 1 + l)];
                        }
                    } else {
                        if (o->bc[3] == HYB_BC_PERIODIC) {
                            X[XN(o, i, ny + l)] = X[XN(o, i, 1 + l)] + px;
                            Y[XN(o, i, ny + l)] = Y[XN(o, i, 1 + l)] + py;
                        } else {
                            X[XN(o, i, ny + l)] = 2.0 * X[XN(o, i, ny)] - X[XN(o, i, ny - l)];
                            Y[XN(o, i, ny + l)] = 2.0 * Y[XN(o, i, ny)] - Y[XN(o, i, ny - l)];
                        }
                    }
                }
            }
        }
    }
    /* corner points (sub_init.f90:801-810) */
    for (int j = 1; j <= LAP; j++)
        for (int i = 1; i <= LAP; i++) {
            int i1 = 1 - i, j1 = 1 - j, i2 = nx + i, j2 = ny + j;
            double *X = o->xn, *Y = o->yn;
            X[XN(o, i1, j1)] = X[XN(o, i1, 1)] + X[XN(o, 1, j1)] - X[XN(o, 1, 1)];
            Y[XN(o, i1, j1)] = Y[XN(o, i1, 1)] + Y[XN(o, 1, j1)] - Y[XN(o, 1, 1)];
            X[XN(o, i2, j2)] = X[XN(o, i2, ny)] + X[XN(o, nx, j2)] - X[XN(o, nx, ny)];
            Y[XN(o, i2, j2)] = Y[XN(o, i2, ny)] + Y[XN(o, nx, j2)] - Y[XN(o, nx, ny)];
            X[XN(o, i1, j2)] = X[XN(o, i1, ny)] + X[XN(o, 1, j2)] - X[XN(o, 1, ny)];
            Y[XN(o, i1, j2)] = Y[XN(o, i1, ny)] + Y[XN(o, 1, j2)] - Y[XN(o, 1, ny)];
            X[XN(o, i2, j1)] = X[XN(o, i2, 1)] + X[XN(o, nx, j1)] - X[XN(o, nx, 1)];
            Y[XN(o, i2, j1)] = Y[XN(o, i2, 1)] + Y[XN(o, nx, j1)] - Y[XN(o, nx, 1)];
        }
    /* cell centres (sub_init.f90:814-819) */
    for (int j = 1 - LAP; j <= ny + LAP - 1; j++)
        for (int i = 1 - LAP; i <= nx + LAP - 1; i++) {
            o->x1[C2(o, i, j)] = (o->xn[XN(o, i, j)] + o->xn[XN(o, i + 1, j)] + o->xn[XN(o, i, j + 1)] +
                                  o->xn[XN(o, i + 1, j + 1)]) * 0.25;
            o->y1[C2(o, i, j)] = (o->yn[XN(o, i, j)] + o->yn[XN(o, i + 1, j)] + o->yn[XN(o, i, j + 1)] +
                                  o->yn[XN(o, i + 1, j + 1)]) * 0.25;
        }
}

int orc_geometry(orc *o, double *vol, double *si, double *sj, double *ni1, double *ni2, double *nj1,
                 double *nj2, double *x1, double *y1)
{
    size_t n = (size_t)o->nx * o->ny, nc = (size_t)(o->nx + 3) * (o->ny + 3);
    if (vol) memcpy(vol, o->vol, n * sizeof(double));
    if (si) memcpy(si, o->si, n * sizeof(double));
    if (sj) memcpy(sj, o->sj, n * sizeof(double));
    if (ni1) memcpy(ni1, o->ni1, n * sizeof(double));
    if (ni2) memcpy(ni2, o->ni2, n * sizeof(double));
    if (nj1) memcpy(nj1, o->nj1, n * sizeof(double));
    if (nj2) memcpy(nj2, o->nj2, n * sizeof(double));
    if (x1) memcpy(x1, o->x1, nc * sizeof(double));
    if (y1) memcpy(y1, o->y1, nc * sizeof(double));
    return HYB_OK;
}

/* ---- lifecycle ---------------------------------------------------------- */
void orc_destroy(orc *o)
{
    if (!o) return;
    for (int f = 0; f < 4; f++) {
        free(o->wall_u[f]);
        free(o->wall_v[f]);
        free(o->wall_t[f]);
    }
    free(o->vi); free(o->vj); free(o->wi); free(o->wj);
    free(o->xn); free(o->yn);
    free(o->vol); free(o->si); free(o->sj); free(o->ni1); free(o->ni2); free(o->nj1); free(o->nj2);
    free(o->x1); free(o->y1);
    free(o->frd); free(o->frd00); free(o->S); free(o->S0); free(o->CF);
    free(o->tao_i_g); free(o->q_i_g); free(o->tao_j_g); free(o->q_j_g);
    free(o->tao_i_in); free(o->q_i_in); free(o->tao_j_in); free(o->q_j_in);
    orc_ns_free(o);
    free(o);
}

int orc_create(const hyb_mesh *m, const hyb_vgrid *vg, const hyb_params *p, orc **out)
{
    if (!m || !vg || !p || !out || !m->x || !m->y) return HYB_ERR_INVALID;
    if (m->nx < 3 || m->ny < 5 || vg->nvi < 1 || vg->nvj < 1) return HYB_ERR_INVALID;
    if (!vg->vi || !vg->vj || !vg->wi || !vg->wj) return HYB_ERR_INVALID;
    for (int f = 0; f < 4; f++) {
        if (m->bc[f] != HYB_BC_WALL && m->bc[f] != HYB_BC_PERIODIC) return HYB_ERR_UNSUPPORTED;
        if (m->bc[f] == HYB_BC_WALL && (!m->wall_u[f] || !m->wall_v[f] || !m->wall_t[f]))
            return HYB_ERR_INVALID;
    }
    if ((m->bc[0] == HYB_BC_PERIODIC) != (m->bc[2] == HYB_BC_PERIODIC)) return HYB_ERR_INVALID;
    if ((m->bc[1] == HYB_BC_PERIODIC) != (m->bc[3] == HYB_BC_PERIODIC)) return HYB_ERR_INVALID;
    orc *o = (orc *)calloc(1, sizeof(orc));
    if (!o) return HYB_ERR_NOMEM;
    o->nx = m->nx; o->ny = m->ny; o->nvi = vg->nvi; o->nvj = vg->nvj; o->nv = vg->nvi * vg->nvj;
    o->pw = m->nx + 7;
    o->P = (size_t)(m->nx + 7) * (m->ny + 7);
    o->prm = *p;
    for (int f = 0; f < 4; f++) o->bc[f] = m->bc[f];
    for (int f = 0; f < 4; f++)
        if (m->bc[f] == HYB_BC_WALL) {
            int n = face_cells(o, f + 1);
            o->wall_u[f] = (double *)malloc(n * sizeof(double));
            o->wall_v[f] = (double *)malloc(n * sizeof(double));
            o->wall_t[f] = (double *)malloc(n * sizeof(double));
            memcpy(o->wall_u[f], m->wall_u[f], n * sizeof(double));
            memcpy(o->wall_v[f], m->wall_v[f], n * sizeof(double));
            memcpy(o->wall_t[f], m->wall_t[f], n * sizeof(double));
        }
    o->vi = (double *)malloc(vg->nvi * sizeof(double)); memcpy(o->vi, vg->vi, vg->nvi * sizeof(double));
    o->wi = (double *)malloc(vg->nvi * sizeof(double)); memcpy(o->wi, vg->wi, vg->nvi * sizeof(double));
    o->vj = (double *)malloc(vg->nvj * sizeof(double)); memcpy(o->vj, vg->vj, vg->nvj * sizeof(double));
    o->wj = (double *)malloc(vg->nvj * sizeof(double)); memcpy(o->wj, vg->wj, vg->nvj * sizeof(double));
    size_t nn = (size_t)(m->nx + 4) * (m->ny + 4), nm = (size_t)m->nx * m->ny, nc = (size_t)(m->nx + 3) * (m->ny + 3);
    o->xn = (double *)calloc(nn, sizeof(double)); o->yn = (double *)calloc(nn, sizeof(double));
    o->vol = (double *)calloc(nm, sizeof(double)); o->si = (double *)calloc(nm, sizeof(double));
    o->sj = (double *)calloc(nm, sizeof(double)); o->ni1 = (double *)calloc(nm, sizeof(double));
    o->ni2 = (double *)calloc(nm, sizeof(double)); o->nj1 = (double *)calloc(nm, sizeof(double));
    o->nj2 = (double *)calloc(nm, sizeof(double));
    o->x1 = (double *)calloc(nc, sizeof(double)); o->y1 = (double *)calloc(nc, sizeof(double));
    o->frd = (double *)calloc(o->P * NRD * o->nv, sizeof(double));
    o->frd00 = (double *)calloc(o->P * NRD * o->nv, sizeof(double));
    o->S = (double *)calloc(o->P * NSUM, sizeof(double));
    o->S0 = (double *)calloc(o->P * NSUM, sizeof(double));
    o->CF = (double *)calloc(o->P, sizeof(double));
    o->tao_i_g = (double *)calloc(nc * 4, sizeof(double)); o->q_i_g = (double *)calloc(nc * 2, sizeof(double));
    o->tao_j_g = (double *)calloc(nc * 4, sizeof(double)); o->q_j_g = (double *)calloc(nc * 2, sizeof(double));
    o->tao_i_in = (double *)calloc(nc * 4, sizeof(double)); o->q_i_in = (double *)calloc(nc * 2, sizeof(double));
    o->tao_j_in = (double *)calloc(nc * 4, sizeof(double)); o->q_j_in = (double *)calloc(nc * 2, sizeof(double));
    if (!o->frd || !o->frd00 || !o->S || !o->CF || !o->x1 || !o->tao_j_in) {
        orc_destroy(o);
        return HYB_ERR_NOMEM;
    }
    build_geometry(o, m->x, m->y);
    *out = o;
    return HYB_OK;
}

double *orc_frd(orc *o) { return o->frd; }
double *orc_frd00(orc *o) { return o->frd00; }
double *orc_s(orc *o) { return o->S; }
double *orc_cf(orc *o) { return o->CF; }
double orc_err(orc *o) { return o->err; }

/* CF from the primitive moments, DETFP VHS branch (GKUA_DETFP.f90:87-92) */
static double cf_vhs(const orc *o, double s1, double s4)
{
    if (o->prm.x1s <= (double)1.e-8f) return o->prm.cfc * s1;
    return o->prm.cfc * s1 * pow(s4, o->prm.x1s);
}

/* ---- inner-boundary exchanges for periodic faces ------------------------
 * GKUA_inner_mesco_boundary (GKUA_boundary.f90:400-512) copies LAP layers of
 * FRD from the connected face into the ghost cells, for the face's cells
 * only; for a block whose face 1 is connected to its own face 3 this is the
 * periodic copy f(1-l,j) = f(nx-l,j), f(nx-1+l,j) = f(l,j). */
int orc_exchange_f(orc *o)
{
    const int nx = o->nx, ny = o->ny;
#pragma omp parallel for schedule(static)
    for (int v = 0; v < o->nv; v++) {
        if (o->bc[0] == HYB_BC_PERIODIC)
            for (int j = 1; j <= ny - 1; j++)
                for (int l = 1; l <= LAP; l++)
                    for (int r = 0; r < NRD; r++) {
                        FRD(o, r, 1 - l, j, v) = FRD(o, r, nx - l, j, v);
                        FRD(o, r, nx - 1 + l, j, v) = FRD(o, r, l, j, v);
                    }
        if (o->bc[1] == HYB_BC_PERIODIC)
            for (int i = 1; i <= nx - 1; i++)
                for (int l = 1; l <= LAP; l++)
                    for (int r = 0; r < NRD; r++) {
                        FRD(o, r, i, 1 - l, v) = FRD(o, r, i, ny - l, v);
                        FRD(o, r, i, ny - 1 + l, v) = FRD(o, r, i, l, v);
                    }
    }
    return HYB_OK;
}

/* GKUA_inner_macro_boundary (GKUA_boundary.f90:514-633): S(1:10), LAP layers */
static void exchange_s(orc *o)
{
    const int nx = o->nx, ny = o->ny;
    if (o->bc[0] == HYB_BC_PERIODIC)
        for (int j = 1; j <= ny - 1; j++)
            for (int l = 1; l <= LAP; l++)
                for (int k = 1; k <= 10; k++) {
                    SG(o, k, 1 - l, j) = SG(o, k, nx - l, j);
                    SG(o, k, nx - 1 + l, j) = SG(o, k, l, j);
                }
    if (o->bc[1] == HYB_BC_PERIODIC)
        for (int i = 1; i <= nx - 1; i++)
            for (int l = 1; l <= LAP; l++)
                for (int k = 1; k <= 10; k++) {
                    SG(o, k, i, 1 - l) = SG(o, k, i, ny - l);
                    SG(o, k, i, ny - 1 + l) = SG(o, k, i, l);
                }
}

/* ---- diffuse wall -------------------------------------------------------
 * GKUA_boundary_wall (GKUA_boundary.f90:49-100): limited linear
 * extrapolation of f into the wall slot (-3 / n+3), then
 * GKUA_wall_boundary + NWGaussLegendre (GKUA_wall_functions.f90:1-199):
 * n_w = -sum_{c.n<0} w c.n f / sum_{c.n>=0} w c.n M_w, and the reflected
 * (c.n >= 0) nodes of the slot become n_w M(u_w, v_w, T_w).  The face loop
 * skips the last node (icheck, :71-75), i.e. it runs over the face cells. */
static void wall_face(orc *o, int f)
{
    const int nx = o->nx, ny = o->ny;
    const int nfc = face_cells(o, f);
    for (int k = 0; k < nfc; k++) {
        int px, py, px1, py1, gx, gy;
        double swnx, swny, step;
        if (f == 1) { px = 1; py = k + 1; px1 = 2; py1 = k + 1; gx = -3; gy = k + 1;
                      swnx = o->ni1[MI(o, 1, k + 1)]; swny = o->ni2[MI(o, 1, k + 1)]; step = 1.0; }
        else if (f == 2) { px = k + 1; py = 1; px1 = k + 1; py1 = 2; gx = k + 1; gy = -3;
                      swnx = o->nj1[MI(o, k + 1, 1)]; swny = o->nj2[MI(o, k + 1, 1)]; step = 1.0; }
        else if (f == 3) { px = nx - 1; py = k + 1; px1 = nx - 2; py1 = k + 1; gx = nx + 3; gy = k + 1;
                      swnx = o->ni1[MI(o, nx, k + 1)]; swny = o->ni2[MI(o, nx, k + 1)]; step = -1.0; }
        else { px = k + 1; py = ny - 1; px1 = k + 1; py1 = ny - 2; gx = k + 1; gy = ny + 3;
                      swnx = o->nj1[MI(o, k + 1, ny)]; swny = o->nj2[MI(o, k + 1, ny)]; step = -1.0; }
        /* extrapolation, GKUA_boundary.f90:86-95 */
        for (int v = 0; v < o->nv; v++)
            for (int r = 0; r < NRD; r++) {
                double fp = FRD(o, r, px, py, v);
                double t = (-FRD(o, r, px1, py1, v) + 3.0 * fp) * 0.5;
                if (t <= 0.0) t = fp;
                if (t >= 1.5 * fp) t = 1.5 * fp;
                FRD(o, r, gx, gy, v) = t;
            }
        const double uw = o->wall_u[f - 1][k], vw = o->wall_v[f - 1][k], tw = o->wall_t[f - 1][k];
        /* NWGaussLegendre, GKUA_wall_functions.f90:148-168 */
        double sumnw = 0.0, sumnw1 = 0.0;
        for (int jv = 0; jv < o->nvj; jv++) {
            double vs1 = o->wj[jv];
            for (int iv = 0; iv < o->nvi; iv++) {
                int v = iv + o->nvi * jv;
                double s = o->wi[iv] * vs1;
                double vnw = ((o->vi[iv] - uw) * swnx + (o->vj[jv] - vw) * swny) * step;
                double vnn = (vnw - fabs(vnw)) / 2.0;
                sumnw += s * (vnn * FRD(o, 0, gx, gy, v));
                double fb = (vnw + fabs(vnw)) / 2.0 *
                            exp(-((o->vi[iv] - uw) * (o->vi[iv] - uw) + (o->vj[jv] - vw) * (o->vj[jv] - vw)) / tw) /
                            (PI * tw);
                sumnw1 += s * fb;
            }
        }
        double nw = -sumnw / sumnw1; /* :193 */
        /* reflected nodes, GKUA_wall_functions.f90:44-61.  The clamp of a
         * negative n_w at :54 cannot trigger: the slot values are >= the
         * 1e-30 floor, so sumnw <= 0 and n_w >= 0. */
        for (int jv = 0; jv < o->nvj; jv++)
            for (int iv = 0; iv < o->nvi; iv++) {
                int v = iv + o->nvi * jv;
                double vnw = ((o->vi[iv] - uw) * swnx + (o->vj[jv] - vw) * swny) * step;
                if (vnw >= 0.0) {
                    double cvuv = (o->vi[iv] - uw) * (o->vi[iv] - uw) + (o->vj[jv] - vw) * (o->vj[jv] - vw);
                    double g = nw * exp(-cvuv / tw) / (PI * tw);
                    FRD(o, 0, gx, gy, v) = g;
                    FRD(o, 1, gx, gy, v) = (tw * g / 2.0);
                }
            }
    }
}

/* GKUA_Phy_boundary (GKUA_boundary.f90:2-46) */
int orc_phy_boundary(orc *o)
{
    for (int f = 1; f <= 4; f++)
        if (o->bc[f - 1] == HYB_BC_WALL) wall_face(o, f);
    return HYB_OK;
}

/* ---- Get_Feq (GKUA_Residual.f90:420-469) for one velocity, from the
 * moments s6 = (rho, u, v, T, qx, qy) ------------------------------------- */
void orc_feq(const orc *o, const double *s6, int iv, int jv, double *g, double *h)
{
    double s1 = s6[0], s2 = s6[1], s3 = s6[2], s4 = s6[3];
    double vjv = o->vj[jv] - s3;
    double viu = o->vi[iv] - s2;
    double crt = s1 / (PI * s4);
    double cpt = o->prm.cpr / (s1 * s4 * s4);
    double viuq = viu * s6[4];
    double vq = viuq + vjv * s6[5];
    double vij2 = (viu * viu + vjv * vjv) / s4;
    double fvxdv = cpt * vq;
    double gdv = crt * exp(-vij2);
    *g = gdv * (1.0 + fvxdv * (2. * vij2 - 4.));
    *h = (s4 * gdv / 2.) * (1.0 + fvxdv * (2. * vij2 - 2.));
}

static void feq_cell(const orc *o, int i, int j, int iv, int jv, double *g, double *h)
{
    const double s6[6] = {SG(o, 1, i, j), SG(o, 2, i, j), SG(o, 3, i, j), SG(o, 4, i, j), SG(o, 8, i, j),
                          SG(o, 9, i, j)};
    orc_feq(o, s6, iv, jv, g, h);
}

/* ---- RHSFDVsub (GKUA_Residual.f90:117-418) for one velocity ---------------
 * flux arrays are on (1..nx+1, 1..ny) with pitch nx+2; atsvx / atsvy keep the
 * face speeds for the sweeps (B%ATSVX / B%ATSVY). */
static void rhs_velocity(const orc *o, int iv, int jv, double *rhs, double *atsvx, double *atsvy, double *flux,
                         double *dfrd)
{
    const int nx = o->nx, ny = o->ny, v = iv + o->nvi * jv;
    const int sch = o->prm.scheme;
    const int fp = nx + 2;
    const double vx = o->vi[iv], vy = o->vj[jv];
#define FL(r, i, j) flux[((size_t)(i) + (size_t)fp * (j)) * NRD + (r)]
#define DF(r, k) dfrd[((k) + 3) * NRD + (r)]
#define AX(i, j) atsvx[(size_t)(i) + (size_t)fp * (j)]
#define AY(i, j) atsvy[(size_t)(i) + (size_t)fp * (j)]
#define F(r, i, j) FRD(o, r, i, j, v)
    /* i-direction, :145-187 */
    for (int j = 1; j <= ny - 1; j++) {
        for (int i = 0; i <= nx + 1; i++)
            for (int r = 0; r < NRD; r++) DF(r, i) = F(r, i, j) - F(r, i - 1, j);
        for (int i = 1; i <= nx; i++) {
            AX(i, j) = (vx * o->ni1[MI(o, i, j)] + vy * o->ni2[MI(o, i, j)]) * o->si[MI(o, i, j)];
            double asp = (AX(i, j) + fabs(AX(i, j))) * 0.5, asn = (AX(i, j) - fabs(AX(i, j))) * 0.5;
            for (int r = 0; r < NRD; r++) {
                if (sch == HYB_SCHEME_UP1) {
                    FL(r, i, j) = asp * F(r, i - 1, j) + asn * F(r, i, j);
                } else if (sch == HYB_SCHEME_NND) {
                    double ulg = F(r, i - 1, j) + 0.5 * fminmd(DF(r, i), DF(r, i - 1));
                    double urg = F(r, i, j) - 0.5 * fminmd(DF(r, i), DF(r, i + 1));
                    FL(r, i, j) = asp * ulg + asn * urg;
                } else {
                    double is1 = DF(r, i - 1) * DF(r, i - 1), is2 = DF(r, i) * DF(r, i), is3 = DF(r, i + 1) * DF(r, i + 1);
                    double a1 = CWENO1 / ((is1 + EPSWENO) * (is1 + EPSWENO)), a2 = CWENO2 / ((is2 + EPSWENO) * (is2 + EPSWENO));
                    double a = a1 + a2, o1 = a1 / a, o2 = a2 / a;
                    double ulh = o1 * (-0.5 * F(r, i - 2, j) + 1.5 * F(r, i - 1, j)) + o2 * (0.5 * F(r, i - 1, j) + 0.5 * F(r, i, j));
                    a1 = CWENO2 / ((is2 + EPSWENO) * (is2 + EPSWENO)); a2 = CWENO1 / ((is3 + EPSWENO) * (is3 + EPSWENO));
                    a = a1 + a2; o1 = a1 / a; o2 = a2 / a;
                    double urh = o1 * (0.5 * F(r, i - 1, j) + 0.5 * F(r, i, j)) + o2 * (1.5 * F(r, i, j) - 0.5 * F(r, i + 1, j));
                    FL(r, i, j) = asp * ulh + asn * urh;
                }
            }
        }
    }
    /* wall face overrides on faces 1 / 3, :189-266 */
    for (int f = 1; f <= 3; f += 2) {
        if (o->bc[f - 1] != HYB_BC_WALL) continue;
        for (int j = 1; j <= ny - 1; j++) {
            int ii = (f == 1) ? 2 : nx - 1;
            double asp = (AX(ii, j) + fabs(AX(ii, j))) * 0.5, asn = (AX(ii, j) - fabs(AX(ii, j))) * 0.5;
            for (int r = 0; r < NRD; r++) {
                if (f == 1) {
                    double f1 = F(r, 1, j), f2 = F(r, 2, j), f3 = F(r, 3, j);
                    if (sch == HYB_SCHEME_UP1) FL(r, 2, j) = asp * f1 + asn * f2;
                    else if (sch == HYB_SCHEME_WENO3) {
                        double is2 = (f2 - f1) * (f2 - f1), is3 = (f3 - f2) * (f3 - f2);
                        double ulh = 0.5 * (f1 + f2);
                        double a1 = CWENO2 / ((is2 + EPSWENO) * (is2 + EPSWENO)), a2 = CWENO1 / ((is3 + EPSWENO) * (is3 + EPSWENO));
                        double a = a1 + a2, o1 = a1 / a, o2 = a2 / a;
                        double urh = o1 * (0.5 * f1 + 0.5 * f2) + o2 * (1.5 * f2 - 0.5 * f3);
                        FL(r, 2, j) = asp * ulh + asn * urh;
                    } else {
                        double ulg = f1 + 0.5 * (f2 - f1);
                        double urg = f2 - 0.5 * fminmd(f2 - f1, f3 - f2);
                        FL(r, 2, j) = asp * ulg + asn * urg;
                    }
                    FL(r, 1, j) = AX(1, j) * F(r, -3, j);
                } else {
                    double f1 = F(r, nx - 1, j), f2 = F(r, nx - 2, j), f3 = F(r, nx - 3, j);
                    if (sch == HYB_SCHEME_UP1) FL(r, nx - 1, j) = asp * f2 + asn * f1;
                    else if (sch == HYB_SCHEME_WENO3) {
                        double is1 = (f2 - f3) * (f2 - f3), is2 = (f1 - f2) * (f1 - f2);
                        double a1 = CWENO1 / ((is1 + EPSWENO) * (is1 + EPSWENO)), a2 = CWENO2 / ((is2 + EPSWENO) * (is2 + EPSWENO));
                        double a = a1 + a2, o1 = a1 / a, o2 = a2 / a;
                        double ulh = o1 * (-0.5 * f3 + 1.5 * f2) + o2 * (0.5 * f2 + 0.5 * f1);
                        double urh = 0.5 * f2 + 0.5 * f1;
                        FL(r, nx - 1, j) = asp * ulh + asn * urh;
                    } else {
                        double ulg = f2 + 0.5 * fminmd(f1 - f2, f2 - f3);
                        double urg = f1 - 0.5 * (f1 - f2);
                        FL(r, nx - 1, j) = asp * ulg + asn * urg;
                    }
                    FL(r, nx, j) = AX(nx, j) * F(r, nx + 3, j);
                }
            }
        }
    }
    /* RHS = flux difference in i, :270-276 */
    for (int j = 1; j <= ny - 1; j++)
        for (int i = 1; i <= nx - 1; i++)
            for (int r = 0; r < NRD; r++)
                rhs[IX(o, i, j) * NRD + r] = FL(r, i + 1, j) - FL(r, i, j);
    /* j-direction, :278-320 */
    for (int i = 1; i <= nx - 1; i++) {
        for (int j = 0; j <= ny + 1; j++)
            for (int r = 0; r < NRD; r++) DF(r, j) = F(r, i, j) - F(r, i, j - 1);
        for (int j = 1; j <= ny; j++) {
            AY(i, j) = (vx * o->nj1[MI(o, i, j)] + vy * o->nj2[MI(o, i, j)]) * o->sj[MI(o, i, j)];
            double asp = (AY(i, j) + fabs(AY(i, j))) * 0.5, asn = (AY(i, j) - fabs(AY(i, j))) * 0.5;
            for (int r = 0; r < NRD; r++) {
                if (sch == HYB_SCHEME_UP1) {
                    FL(r, i, j) = asp * F(r, i, j - 1) + asn * F(r, i, j);
                } else if (sch == HYB_SCHEME_NND) {
                    double ulg = F(r, i, j - 1) + 0.5 * fminmd(DF(r, j), DF(r, j - 1));
                    double urg = F(r, i, j) - 0.5 * fminmd(DF(r, j), DF(r, j + 1));
                    FL(r, i, j) = asp * ulg + asn * urg;
                } else {
                    double is1 = DF(r, j - 1) * DF(r, j - 1), is2 = DF(r, j) * DF(r, j), is3 = DF(r, j + 1) * DF(r, j + 1);
                    double a1 = CWENO1 / ((is1 + EPSWENO) * (is1 + EPSWENO)), a2 = CWENO2 / ((is2 + EPSWENO) * (is2 + EPSWENO));
                    double a = a1 + a2, o1 = a1 / a, o2 = a2 / a;
                    double ulh = o1 * (-0.5 * F(r, i, j - 2) + 1.5 * F(r, i, j - 1)) + o2 * (0.5 * F(r, i, j - 1) + 0.5 * F(r, i, j));
                    a1 = CWENO2 / ((is2 + EPSWENO) * (is2 + EPSWENO)); a2 = CWENO1 / ((is3 + EPSWENO) * (is3 + EPSWENO));
                    a = a1 + a2; o1 = a1 / a; o2 = a2 / a;
                    double urh = o1 * (0.5 * F(r, i, j - 1) + 0.5 * F(r, i, j)) + o2 * (1.5 * F(r, i, j) - 0.5 * F(r, i, j + 1));
                    FL(r, i, j) = asp * ulh + asn * urh;
                }
            }
        }
    }
    /* wall face overrides on faces 2 / 4, :321-396 */
    for (int f = 2; f <= 4; f += 2) {
        if (o->bc[f - 1] != HYB_BC_WALL) continue;
        for (int i = 1; i <= nx - 1; i++) {
            int jj = (f == 2) ? 2 : ny - 1;
            double asp = (AY(i, jj) + fabs(AY(i, jj))) * 0.5, asn = (AY(i, jj) - fabs(AY(i, jj))) * 0.5;
            for (int r = 0; r < NRD; r++) {
                if (f == 2) {
                    double f1 = F(r, i, 1), f2 = F(r, i, 2), f3 = F(r, i, 3);
                    if (sch == HYB_SCHEME_UP1) FL(r, i, 2) = asp * f1 + asn * f2;
                    else if (sch == HYB_SCHEME_WENO3) {
                        double is2 = (f2 - f1) * (f2 - f1), is3 = (f3 - f2) * (f3 - f2);
                        double ulh = 0.5 * f1 + 0.5 * f2;
                        double a1 = CWENO2 / ((is2 + EPSWENO) * (is2 + EPSWENO)), a2 = CWENO1 / ((is3 + EPSWENO) * (is3 + EPSWENO));
                        double a = a1 + a2, o1 = a1 / a, o2 = a2 / a;
                        double urh = o1 * (0.5 * f1 + 0.5 * f2) + o2 * (1.5 * f2 - 0.5 * f3);
                        FL(r, i, 2) = asp * ulh + asn * urh;
                    } else {
                        double ulg = f1 + 0.5 * (f2 - f1);
                        double urg = f2 - 0.5 * fminmd(f2 - f1, f3 - f2);
                        FL(r, i, 2) = asp * ulg + asn * urg;
                    }
                    FL(r, i, 1) = AY(i, 1) * F(r, i, -3);
                } else {
                    double f1 = F(r, i, ny - 1), f2 = F(r, i, ny - 2), f3 = F(r, i, ny - 3);
                    if (sch == HYB_SCHEME_UP1) FL(r, i, ny - 1) = asp * f2 + asn * f1;
                    else if (sch == HYB_SCHEME_WENO3) {
                        double is1 = (f2 - f3) * (f2 - f3), is2 = (f1 - f2) * (f1 - f2);
                        double a1 = CWENO1 / ((is1 + EPSWENO) * (is1 + EPSWENO)), a2 = CWENO2 / ((is2 + EPSWENO) * (is2 + EPSWENO));
                        double a = a1 + a2, o1 = a1 / a, o2 = a2 / a;
                        double ulh = o1 * (-0.5 * f3 + 1.5 * f2) + o2 * (0.5 * f2 + 0.5 * f1);
                        double urh = 0.5 * f2 + 0.5 * f1;
                        FL(r, i, ny - 1) = asp * ulh + asn * urh;
                    } else {
                        double ulg = f2 + 0.5 * fminmd(f1 - f2, f2 - f3);
                        double urg = f1 - 0.5 * (f1 - f2);
                        FL(r, i, ny - 1) = asp * ulg + asn * urg;
                    }
                    FL(r, i, ny) = AY(i, ny) * F(r, i, ny + 3);
                }
            }
        }
    }
    /* RHS += flux difference in j, then -RHS/vol + CF (feq - f), :398-414 */
    for (int i = 1; i <= nx - 1; i++)
        for (int j = 1; j <= ny - 1; j++)
            for (int r = 0; r < NRD; r++)
                rhs[IX(o, i, j) * NRD + r] = rhs[IX(o, i, j) * NRD + r] + FL(r, i, j + 1) - FL(r, i, j);
    for (int j = 1; j <= ny - 1; j++)
        for (int i = 1; i <= nx - 1; i++) {
            double g, h;
            feq_cell(o, i, j, iv, jv, &g, &h);
            double vol = o->vol[MI(o, i, j)], cf = CFA(o, i, j);
            rhs[IX(o, i, j) * NRD + 0] = -rhs[IX(o, i, j) * NRD + 0] / vol + cf * (g - F(0, i, j));
            rhs[IX(o, i, j) * NRD + 1] = -rhs[IX(o, i, j) * NRD + 1] / vol + cf * (h - F(1, i, j));
        }
#undef FL
#undef DF
#undef AX
#undef AY
#undef F
}

/* ---- moments 1-4 of the kinetic RHS of the current f with its own
 * equilibrium (RHSFDVsub with the moments of DETFP_res), per cell on the C2
 * extents: rk[m*nc2 + C2(i,j)], m = rho, rho u, rho v, energy; the per-volume
 * rate in kinetic time.  The synthetic solve is driven by it. ------------- */
int orc_kinetic_residual_moments(orc *o, double *rk)
{
    const int nx = o->nx, ny = o->ny, fp = nx + 2;
    const size_t nc2 = (size_t)(nx + 3) * (ny + 3);
    const size_t ncell = (size_t)(nx - 1) * (ny - 1);
    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    double *part = (double *)calloc((size_t)nth * 4 * ncell, sizeof(double));
    if (!part) return HYB_ERR_NOMEM;
#pragma omp parallel num_threads(nth)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *acc = part + (size_t)tid * 4 * ncell;
        double *rhs = (double *)calloc(o->P * NRD, sizeof(double));
        double *ax = (double *)calloc((size_t)fp * (ny + 2), sizeof(double));
        double *ay = (double *)calloc((size_t)fp * (ny + 2), sizeof(double));
        double *flux = (double *)calloc((size_t)fp * (ny + 2) * NRD, sizeof(double));
        int mx = (nx > ny ? nx : ny) + 8;
        double *dfrd = (double *)calloc((size_t)mx * NRD, sizeof(double));
#pragma omp for schedule(static)
        for (int v = 0; v < o->nv; v++) {
            int iv = v % o->nvi, jv = v / o->nvi;
            rhs_velocity(o, iv, jv, rhs, ax, ay, flux, dfrd);
            double vx = o->vi[iv], vy = o->vj[jv], w = o->wi[iv] * o->wj[jv];
            for (int j = 1; j <= ny - 1; j++)
                for (int i = 1; i <= nx - 1; i++) {
                    size_t k = (size_t)(i - 1) + (size_t)(nx - 1) * (j - 1);
                    double g = rhs[IX(o, i, j) * NRD + 0], h = rhs[IX(o, i, j) * NRD + 1];
                    acc[k] += w * g;
                    acc[ncell + k] += w * vx * g;
                    acc[2 * ncell + k] += w * vy * g;
                    acc[3 * ncell + k] += w * (h + (vx * vx + vy * vy) * g);
                }
        }
        free(rhs); free(ax); free(ay); free(flux); free(dfrd);
    }
    memset(rk, 0, 4 * nc2 * sizeof(double));
    for (int j = 1; j <= ny - 1; j++)
        for (int i = 1; i <= nx - 1; i++) {
            size_t k = (size_t)(i - 1) + (size_t)(nx - 1) * (j - 1);
            for (int m = 0; m < 4; m++) {
                double x = 0.0;
                for (int t = 0; t < nth; t++) x += part[((size_t)t * 4 + m) * ncell + k];
                rk[(size_t)m * nc2 + C2(o, i, j)] = x;
            }
        }
    free(part);
    return HYB_OK;
}

/* ---- GKUA_Residual (GKUA_Residual.f90:4-114) ---------------------------- */
int orc_kinetic_step(orc *o)
{
    const int nx = o->nx, ny = o->ny, fp = nx + 2;
    const double dt = o->prm.dt;
    /* mass_pin: the updated f is multiplied by m0 / M(f) of the state this
     * step starts from (its moments are the current S) */
    const double msc = o->prm.mass_pin ? o->m0 / orc_total_mass(o) : 1.0;
#pragma omp parallel
    {
        double *rhs = (double *)calloc(o->P * NRD, sizeof(double));
        double *dufrd = (double *)calloc(o->P * NRD, sizeof(double));
        double *ax = (double *)calloc((size_t)fp * (ny + 2), sizeof(double));
        double *ay = (double *)calloc((size_t)fp * (ny + 2), sizeof(double));
        double *flux = (double *)calloc((size_t)fp * (ny + 2) * NRD, sizeof(double));
        int mx = (nx > ny ? nx : ny) + 8;
        double *dfrd = (double *)calloc((size_t)mx * NRD, sizeof(double));
#pragma omp for schedule(dynamic, 4)
        for (int v = 0; v < o->nv; v++) {
            int iv = v % o->nvi, jv = v / o->nvi;
            rhs_velocity(o, iv, jv, rhs, ax, ay, flux, dfrd);
#define AX(i, j) ax[(size_t)(i) + (size_t)fp * (j)]
#define AY(i, j) ay[(size_t)(i) + (size_t)fp * (j)]
            if (o->prm.sweep_order == HYB_SWEEP_UPWIND) {
                /* one Gauss-Seidel sweep in this velocity's upwind order with
                 * the reference's alpha (:39-57): i runs downwards where the
                 * i-face speeds are negative, j where the j-face speeds are;
                 * cells not yet visited (and every ghost) carry 0, so on a
                 * Cartesian mesh every incoming neighbour is already solved.
                 * The update is applied directly (no backward step). */
                double sx = 0.0, sy = 0.0;
                for (int j = 1; j <= ny - 1; j++) sx += AX(1, j) + AX(nx, j);
                for (int i = 1; i <= nx - 1; i++) sy += AY(i, 1) + AY(i, ny);
                const int di = sx < 0.0 ? -1 : 1, dj = sy < 0.0 ? -1 : 1;
                for (int j = -3; j <= ny + 3; j++)
                    for (int i = -3; i <= nx + 3; i++)
                        for (int r = 0; r < NRD; r++) FRD00(o, r, i, j, v) = 0.0;
                for (int jj = 1; jj <= ny - 1; jj++) {
                    const int j = dj > 0 ? jj : ny - jj;
                    for (int ii = 1; ii <= nx - 1; ii++) {
                        const int i = di > 0 ? ii : nx - ii;
                        double axp = pos_part(AX(i + 1, j)), ayp = pos_part(AY(i, j + 1));
                        double axn = neg_part(AX(i, j)), ayn = neg_part(AY(i, j));
                        double vol = o->vol[MI(o, i, j)];
                        double alfa = vol / dt + (axp - axn + ayp - ayn) + vol * CFA(o, i, j);
                        double axp1 = pos_part(AX(i, j)), ayp1 = pos_part(AY(i, j));
                        double axn1 = neg_part(AX(i + 1, j)), ayn1 = neg_part(AY(i, j + 1));
                        for (int r = 0; r < NRD; r++) {
                            double in = axp1 * FRD00(o, r, i - 1, j, v) + ayp1 * FRD00(o, r, i, j - 1, v) -
                                        axn1 * FRD00(o, r, i + 1, j, v) - ayn1 * FRD00(o, r, i, j + 1, v);
                            FRD00(o, r, i, j, v) = (vol * rhs[IX(o, i, j) * NRD + r] + in) / alfa;
                        }
                    }
                }
                for (int j = 1; j <= ny - 1; j++)
                    for (int i = 1; i <= nx - 1; i++)
                        for (int r = 0; r < NRD; r++) {
                            double fn = FRD(o, r, i, j, v) + FRD00(o, r, i, j, v);
                            FRD(o, r, i, j, v) = o->prm.mass_pin ? msc * fn : fn;
                            FRD00(o, r, i, j, v) = rhs[IX(o, i, j) * NRD + r];
                        }
                for (int j = -1; j <= ny + 1; j++)
                    for (int i = -1; i <= nx + 1; i++)
                        for (int r = 0; r < NRD; r++)
                            if (FRD(o, r, i, j, v) < F_FLOOR) FRD(o, r, i, j, v) = F_FLOOR;
                continue;
            }
            /* forward sweep over anti-diagonals, :34-62.  FRD00 of ghost
             * cells is never written and stays 0, so the sweep is explicit
             * across every block face. */
            for (int plane = 2; plane <= nx - 1 + ny - 1; plane++)
                for (int j = 1; j <= ny - 1; j++) {
                    int i = plane - j;
                    if (i < 1 || i > nx - 1) continue;
                    double axp = (AX(i + 1, j) + fabs(AX(i + 1, j))) * 0.5;
                    double ayp = (AY(i, j + 1) + fabs(AY(i, j + 1))) * 0.5;
                    double axn = (AX(i, j) - fabs(AX(i, j))) * 0.5;
                    double ayn = (AY(i, j) - fabs(AY(i, j))) * 0.5;
                    double vol = o->vol[MI(o, i, j)];
                    double alfa = vol / dt + (axp - axn + ayp - ayn) + vol * CFA(o, i, j);
                    double axp1 = (AX(i, j) + fabs(AX(i, j))) * 0.5;
                    double ayp1 = (AY(i, j) + fabs(AY(i, j))) * 0.5;
                    for (int r = 0; r < NRD; r++) {
                        double dfi = axp1 * FRD00(o, r, i - 1, j, v);
                        double dfj = ayp1 * FRD00(o, r, i, j - 1, v);
                        FRD00(o, r, i, j, v) = (vol * rhs[IX(o, i, j) * NRD + r] + dfi + dfj) / alfa;
                    }
                }
            /* backward step, :64-90: reads the forward values of the
             * downstream neighbours (FRD00), not DUFRD */
            for (int plane = nx - 1 + ny - 1; plane >= 2; plane--)
                for (int j = ny - 1; j >= 1; j--) {
                    int i = plane - j;
                    if (i < 1 || i > nx - 1) continue;
                    double axp = (AX(i + 1, j) + fabs(AX(i + 1, j))) * 0.5;
                    double ayp = (AY(i, j + 1) + fabs(AY(i, j + 1))) * 0.5;
                    double axn = (AX(i, j) - fabs(AX(i, j))) * 0.5;
                    double ayn = (AY(i, j) - fabs(AY(i, j))) * 0.5;
                    double vol = o->vol[MI(o, i, j)];
                    double alfa = vol / dt + (axp - axn + ayp - ayn) + vol * CFA(o, i, j);
                    double axn1 = (AX(i + 1, j) - fabs(AX(i + 1, j))) * 0.5;
                    double ayn1 = (AY(i, j + 1) - fabs(AY(i, j + 1))) * 0.5;
                    for (int r = 0; r < NRD; r++) {
                        double dfi = -axn1 * FRD00(o, r, i + 1, j, v);
                        double dfj = -ayn1 * FRD00(o, r, i, j + 1, v);
                        dufrd[IX(o, i, j) * NRD + r] = FRD00(o, r, i, j, v) + (dfi + dfj) / alfa;
                    }
                }
#undef AX
#undef AY
            /* update and store the RHS, :91-100 */
            for (int j = 1; j <= ny - 1; j++)
                for (int i = 1; i <= nx - 1; i++)
                    for (int r = 0; r < NRD; r++) {
                        double fn = FRD(o, r, i, j, v) + dufrd[IX(o, i, j) * NRD + r];
                        FRD(o, r, i, j, v) = o->prm.mass_pin ? msc * fn : fn;
                        FRD00(o, r, i, j, v) = rhs[IX(o, i, j) * NRD + r];
                    }
            /* floor, :101-109 (ghost layers -1..n+1 included) */
            for (int j = -1; j <= ny + 1; j++)
                for (int i = -1; i <= nx + 1; i++)
                    for (int r = 0; r < NRD; r++)
                        if (FRD(o, r, i, j, v) < F_FLOOR) FRD(o, r, i, j, v) = F_FLOOR;
        }
        free(rhs); free(dufrd); free(ax); free(ay); free(flux); free(dfrd);
    }
    return HYB_OK;
}

/* ---- DETFPwall (GKUA_DETFP_WALL.f90:34-95): S ghost by linear wall
 *      extrapolation, components 1..10, over the face cells -------------- */
static void detfp_wall(orc *o)
{
    const int nx = o->nx, ny = o->ny;
    for (int f = 1; f <= 4; f++) {
        if (o->bc[f - 1] != HYB_BC_WALL) continue;
        int nfc = face_cells(o, f);
        for (int k = 1; k <= nfc; k++) {
            int g1, g2, a1, a2, b1, b2;
            if (f == 1) { g1 = 0; g2 = k; a1 = 1; a2 = k; b1 = 2; b2 = k; }
            else if (f == 2) { g1 = k; g2 = 0; a1 = k; a2 = 1; b1 = k; b2 = 2; }
            else if (f == 3) { g1 = nx; g2 = k; a1 = nx - 1; a2 = k; b1 = nx - 2; b2 = k; }
            else { g1 = k; g2 = ny; a1 = k; a2 = ny - 1; b1 = k; b2 = ny - 2; }
            for (int c = 1; c <= 10; c++) {
                double sw = (-SG(o, c, b1, b2) + 3.0 * SG(o, c, a1, a2)) * 0.5;
                SG(o, c, g1, g2) = 2.0 * sw - SG(o, c, a1, a2);
            }
        }
    }
}

/* ---- DETFP (GKUA_DETFP.f90:4-151) with the GaussLegendre moment sum
 *      (:288-363) written for any full weights w_i w_j.  Moments are formed
 *      on i=0..nx, j=0..ny like the reference; the ring of ghost cells is
 *      afterwards overwritten by DETFPwall, the periodic exchange and the
 *      corner rule of Convert_NS. ----------------------------------------- */
int orc_detfp(orc *o)
{
    const int nx = o->nx, ny = o->ny;
    double errsum = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : errsum)
    for (int j = 0; j <= ny; j++)
        for (int i = 0; i <= nx; i++) {
            double s[10] = {0};
            for (int jv = 0; jv < o->nvj; jv++) {
                double vy = o->vj[jv];
                for (int iv = 0; iv < o->nvi; iv++) {
                    double vx = o->vi[iv];
                    int v = iv + o->nvi * jv;
                    double w = o->wi[iv] * o->wj[jv];
                    double g = FRD(o, 0, i, j, v), h = FRD(o, 1, i, j, v);
                    double vxg = vx * g, vyg = vy * g, vx2g = vx * vxg, vy2g = vy * vyg;
                    double b4 = h + vx2g + vy2g;
                    s[0] += w * g;
                    s[1] += w * vxg;
                    s[2] += w * vyg;
                    s[3] += w * b4;
                    s[4] += w * vx2g;
                    s[5] += w * vy2g;
                    s[6] += w * (vx * vy * g);
                    s[7] += w * (vx * b4);
                    s[8] += w * (vy * b4);
                    s[9] += w * h;
                }
            }
            /* primitive conversion, :59-84 */
            double S1 = s[0], S4 = s[3], S5 = s[4], S6 = s[5], S7 = s[6];
            double ron = S1;
            if (ron <= 0.) ron = o->prm.r00;
            double u = s[1] / ron, vv = s[2] / ron;
            double us1 = u * u, vs1 = vv * vv, suv = us1 + vs1;
            double t = (S4 - ron * suv) / (1.5 * ron);
            if (t <= 0.) t = o->prm.t00;
            double *S = &SG(o, 1, i, j);
            S[0] = S1;
            S[1] = u;
            S[2] = vv;
            S[3] = t;
            S[4] = (S5 - ron * us1) * 2.;
            S[5] = (S6 - ron * vs1) * 2.;
            S[6] = (S7 - ron * u * vv) * 2.;
            S[7] = s[7] - 2. * u * S5 - 2. * vv * S7 + ron * u * (suv - 1.5 * t);
            S[8] = s[8] - 2. * vv * S6 - 2. * u * S7 + ron * vv * (suv - 1.5 * t);
            S[9] = s[9] * 2.;
            S[10] = 0.0;
            double cf0 = CFA(o, i, j);
            double cf = cf_vhs(o, S1, t);
            CFA(o, i, j) = cf;
            /* the CF-change diagnostic, :109-118 */
            double epr = (cf0 > (double)1.e-12f) ? ((cf - cf0) / cf0) * ((cf - cf0) / cf0) : (cf - cf0) * (cf - cf0);
            errsum += epr;
        }
    o->err = sqrt(errsum) / (1.0 * (nx + 3) * (ny + 3));
    detfp_wall(o);   /* GKUA_DET_wall, :147 */
    exchange_s(o);   /* inner macro exchange for periodic faces */
    return HYB_OK;
}

/* ---- higher-order moments of IntegralGaussHermite (GKUA_DETFP.f90:174-229)
 * HOT_GKUA(1:6), HOQ_GKUA(1:3) of the current FRD, summed with the grid's
 * full weights (the reference's GH weights are w exp(v^2), which is what a
 * Gauss-Hermite grid passes in).  Interior cells 1..nx-1 x 1..ny-1; hot is
 * (6,-3:nx+3,-3:ny+3) and hoq (4,...), column-major, zero elsewhere. */
int orc_hoq(orc *o, double *hot, double *hoq)
{
    const int nx = o->nx, ny = o->ny, pw = nx + 7;
    const size_t P = (size_t)(nx + 7) * (ny + 7);
    memset(hot, 0, 6 * P * sizeof(double));
    memset(hoq, 0, 4 * P * sizeof(double));
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny - 1; j++)
        for (int i = 1; i <= nx - 1; i++) {
            double t[6] = {0}, q[3] = {0};
            for (int jv = 0; jv < o->nvj; jv++) {
                double vy = o->vj[jv];
                for (int iv = 0; iv < o->nvi; iv++) {
                    double vx = o->vi[iv];
                    int v = iv + o->nvi * jv;
                    double w = o->wi[iv] * o->wj[jv];
                    double wg = w * FRD(o, 0, i, j, v), wh = w * FRD(o, 1, i, j, v);
                    double e = wg * (vx * vx + vy * vy) + wh;
                    t[0] += wg * vx * vx * vx;
                    t[1] += wg * vx * vx * vy;
                    t[2] += wg * vx * vy * vy;
                    t[3] += wg * vy * vy * vy;
                    t[4] += wh * vx;
                    t[5] += wh * vy;
                    q[0] += e * vx * vx;
                    q[1] += e * vx * vy;
                    q[2] += e * vy * vy;
                }
            }
            size_t ix = (size_t)(i + 3) + (size_t)pw * (j + 3);
            for (int k = 0; k < 6; k++) hot[ix * 6 + k] = t[k];
            for (int k = 0; k < 3; k++) hoq[ix * 4 + k] = q[k];
        }
    return HYB_OK;
}

/* ---- DETFP_res + GaussLegendre_rs (GKUA_DETFP_RES.f90:4-136) ------------ */
int orc_detfp_res(orc *o, hyb_residual *r)
{
    const int nx = o->nx, ny = o->ny;
    double rmax[4] = {0}, rrms[4] = {0};
    for (int j = 1; j <= ny - 1; j++)
        for (int i = 1; i <= nx - 1; i++) {
            double s[4] = {0};
            for (int jv = 0; jv < o->nvj; jv++) {
                double vy = o->vj[jv];
                for (int iv = 0; iv < o->nvi; iv++) {
                    double vx = o->vi[iv];
                    int v = iv + o->nvi * jv;
                    double w = o->wi[iv] * o->wj[jv];
                    double g = FRD00(o, 0, i, j, v), h = FRD00(o, 1, i, j, v);
                    double vxg = vx * g, vyg = vy * g;
                    s[0] += w * g;
                    s[1] += w * vxg;
                    s[2] += w * vyg;
                    s[3] += w * (h + vx * vxg + vy * vyg);
                }
            }
            for (int k = 0; k < 4; k++) {
                if (fabs(s[k]) > rmax[k]) rmax[k] = fabs(s[k]);
                rrms[k] += s[k] * s[k];
            }
        }
    double ncell = 1.0 * (nx - 1) * (ny - 1);
    if (r) {
        r->max_rms = 0.0;
        for (int k = 0; k < 4; k++) {
            r->res_max[k] = rmax[k];
            r->res_rms[k] = sqrt(rrms[k] / ncell);
            if (r->res_rms[k] > r->max_rms || isnan(r->res_rms[k])) r->max_rms = r->res_rms[k];
        }
    }
    return HYB_OK;
}

/* ---- GKUA_sudufenbu (GKUA_sudufenbu.f90:22-53): Maxwellian f on cells
 *      -1..n+1, boundary conditions, moments ------------------------------- */
int orc_init_maxwellian(orc *o, double rho, double u, double v, double t)
{
    const int nx = o->nx, ny = o->ny;
    for (int j = -3; j <= ny + 3; j++)
        for (int i = -3; i <= nx + 3; i++) {
            SG(o, 1, i, j) = rho; SG(o, 2, i, j) = u; SG(o, 3, i, j) = v; SG(o, 4, i, j) = t;
            CFA(o, i, j) = cf_vhs(o, rho, t);   /* init_flow_zero, sub_init.f90:429-434 */
        }
#pragma omp parallel for schedule(static)
    for (int vv = 0; vv < o->nv; vv++) {
        int iv = vv % o->nvi, jv = vv / o->nvi;
        for (int j = -1; j <= ny + 1; j++)
            for (int i = -1; i <= nx + 1; i++) {
                double crt = SG(o, 1, i, j) / (PI * SG(o, 4, i, j));
                double vjv = o->vj[jv] - SG(o, 3, i, j);
                double viu = o->vi[iv] - SG(o, 2, i, j);
                double vij2 = (viu * viu + vjv * vjv) / SG(o, 4, i, j);
                double g = crt * exp(-vij2);
                FRD(o, 0, i, j, vv) = g;
                FRD(o, 1, i, j, vv) = SG(o, 4, i, j) * g / 2.;
            }
    }
    memset(o->frd00, 0, o->P * NRD * o->nv * sizeof(double));
    orc_exchange_f(o);
    orc_phy_boundary(o);
    orc_detfp(o);
    o->m0 = orc_total_mass(o);
    return HYB_OK;
}

int orc_upload_f(orc *o, const double *frd)
{
    memcpy(o->frd, frd, o->P * NRD * o->nv * sizeof(double));
    orc_exchange_f(o);
    orc_detfp(o);
    o->m0 = orc_total_mass(o);
    return HYB_OK;
}

/* total mass sum(vol rho) over the interior cells, j outer / i inner (the
 * order of the GPU's single-CTA fold is not this one; the sums agree to
 * rounding) */
double orc_total_mass(const orc *o)
{
    double m = 0.0;
    for (int j = 1; j <= o->ny - 1; j++)
        for (int i = 1; i <= o->nx - 1; i++) m += o->vol[MI(o, i, j)] * SG(o, 1, i, j);
    return m;
}

/* ---- Convert_NS (Hybrid_Sub.f90:191-461) --------------------------------
 * NS conservative variables from the kinetic moments, Navier-Stokes-Fourier
 * stress and heat flux on every face, and the higher-order terms (kinetic
 * minus NSF).  Periodic faces use the connected cells on both sides (the
 * block-connection view); the reference's single-block formulas (one-sided
 * face values, linear U extrapolation, corner S extrapolation) are kept for
 * wall faces. */
/* NS conservative variables from the moments on 0..nx x 0..ny and their
 * ghost cells (Hybrid_Sub.f90:225-239), U on the C2 extents, 4 per cell. */
void orc_build_u(orc *o, double *U)
{
    const int nx = o->nx, ny = o->ny;
    const double gam = o->prm.gamma, ma = o->prm.ma;
    const double cv = 1.0 / (gam * (gam - 1.0) * ma * ma);
    const int perx = (o->bc[0] == HYB_BC_PERIODIC), pery = (o->bc[1] == HYB_BC_PERIODIC);
#define UU(m, i, j) U[C2(o, i, j) * 4 + (m)]
    /* U outside 0..n keeps the reference's initial state (sub_init.f90:416-419) */
    for (int j = -1; j <= ny + 1; j++)
        for (int i = -1; i <= nx + 1; i++) {
            UU(0, i, j) = 1.0; UU(1, i, j) = 0.0; UU(2, i, j) = 0.0; UU(3, i, j) = cv;
        }
    for (int i = 0; i <= nx; i++)
        for (int j = 0; j <= ny; j++) {
            UU(0, i, j) = SG(o, 1, i, j);
            double tu = SG(o, 2, i, j) / ma * sqrt(2.0 / gam);
            UU(1, i, j) = UU(0, i, j) * tu;
            double tv = SG(o, 3, i, j) / ma * sqrt(2.0 / gam);
            UU(2, i, j) = UU(0, i, j) * tv;
            double tt = SG(o, 4, i, j);
            UU(3, i, j) = UU(0, i, j) * cv * tt + 0.5 * UU(0, i, j) * (tu * tu + tv * tv);
        }
    /* ghost U, :236-239 */
    for (int j = -1; j <= ny + 1; j++)
        for (int m = 0; m < 4; m++) {
            if (perx) {
                UU(m, 0, j) = UU(m, nx - 1, j); UU(m, -1, j) = UU(m, nx - 2, j);
                UU(m, nx, j) = UU(m, 1, j);     UU(m, nx + 1, j) = UU(m, 2, j);
            } else {
                UU(m, 0, j) = 2.0 * UU(m, 1, j) - UU(m, 2, j);
                UU(m, nx, j) = 2.0 * UU(m, nx - 1, j) - UU(m, nx - 2, j);
            }
        }
    for (int i = -1; i <= nx + 1; i++)
        for (int m = 0; m < 4; m++) {
            if (pery) {
                UU(m, i, 0) = UU(m, i, ny - 1); UU(m, i, -1) = UU(m, i, ny - 2);
                UU(m, i, ny) = UU(m, i, 1);     UU(m, i, ny + 1) = UU(m, i, 2);
            } else {
                UU(m, i, 0) = 2.0 * UU(m, i, 1) - UU(m, i, 2);
                UU(m, i, ny) = 2.0 * UU(m, i, ny - 1) - UU(m, i, ny - 2);
            }
        }
#undef UU
}

int orc_convert_ns(orc *o)
{
    const int nx = o->nx, ny = o->ny;
    const double gam = o->prm.gamma, ma = o->prm.ma, pr = o->prm.pr;
    const double cv = 1.0 / (gam * (gam - 1.0) * ma * ma), cp = cv * gam;
    const int perx = (o->bc[0] == HYB_BC_PERIODIC), pery = (o->bc[1] == HYB_BC_PERIODIC);
    const size_t nc = (size_t)(nx + 3) * (ny + 3);
    /* corners, :221-224 (periodic faces copy the partner's ghost row) */
    for (int k = 1; k <= NSUM; k++) {
        if (perx) {
            SG(o, k, 0, 0) = SG(o, k, nx - 1, 0);   SG(o, k, nx, 0) = SG(o, k, 1, 0);
            SG(o, k, 0, ny) = SG(o, k, nx - 1, ny); SG(o, k, nx, ny) = SG(o, k, 1, ny);
        } else if (pery) {
            SG(o, k, 0, 0) = SG(o, k, 0, ny - 1);   SG(o, k, 0, ny) = SG(o, k, 0, 1);
            SG(o, k, nx, 0) = SG(o, k, nx, ny - 1); SG(o, k, nx, ny) = SG(o, k, nx, 1);
        } else {
            SG(o, k, 0, 0) = SG(o, k, 1, 0) + SG(o, k, 0, 1) - SG(o, k, 1, 1);
            SG(o, k, nx, 0) = SG(o, k, nx, 1) + SG(o, k, nx - 1, 0) - SG(o, k, nx - 1, 1);
            SG(o, k, 0, ny) = SG(o, k, 1, ny) + SG(o, k, 0, ny - 1) - SG(o, k, 1, ny - 1);
            SG(o, k, nx, ny) = SG(o, k, nx - 1, ny) + SG(o, k, nx, ny - 1) - SG(o, k, nx - 1, ny - 1);
        }
    }
    double *U = (double *)calloc(nc * 4, sizeof(double));
    double *d = (double *)calloc(nc, sizeof(double)), *uu = (double *)calloc(nc, sizeof(double));
    double *vv = (double *)calloc(nc, sizeof(double)), *T = (double *)calloc(nc, sizeof(double));
    double *amu = (double *)calloc(nc, sizeof(double));
    if (!U || !d || !uu || !vv || !T || !amu) { free(U); free(d); free(uu); free(vv); free(T); free(amu); return HYB_ERR_NOMEM; }
    orc_build_u(o, U);
#define UU(m, i, j) U[C2(o, i, j) * 4 + (m)]
    /* comput_duvtpckw (sub_NS_singlegrid.f90:121-157) and get_viscous
     * (sub_Residual.f90:553-576) */
    for (int j = -1; j <= ny + 1; j++)
        for (int i = -1; i <= nx + 1; i++) {
            size_t c = C2(o, i, j);
            d[c] = UU(0, i, j);
            uu[c] = UU(1, i, j) / d[c];
            vv[c] = UU(2, i, j) / d[c];
            T[c] = (UU(3, i, j) - 0.5 * d[c] * (uu[c] * uu[c] + vv[c] * vv[c])) / (cv * d[c]);
        }
    for (int j = 0; j <= ny; j++)
        for (int i = 0; i <= nx; i++) amu[C2(o, i, j)] = 1.0 / o->prm.re * pow(T[C2(o, i, j)], o->prm.omega_ns);
    const double g2 = gam * ma * ma, q2 = sqrt(2.0) / (pow(ma, 3) * pow(gam, 1.5));
    /* i-faces, :257-352 */
    for (int j = 1; j <= ny - 1; j++)
        for (int i = 1; i <= nx; i++) {
            int lo = (i == 1) && !perx, hi = (i == nx) && !perx;
            double amu1, amk1;
            if (lo) { amu1 = amu[C2(o, i, j)]; amk1 = cp * (amu[C2(o, i, j)] / pr); }
            else if (hi) { amu1 = amu[C2(o, i - 1, j)]; amk1 = cp * (amu[C2(o, i - 1, j)] / pr); }
            else {
                amu1 = (amu[C2(o, i - 1, j)] + amu[C2(o, i, j)]) * 0.5;
                amk1 = cp * ((amu[C2(o, i - 1, j)] + amu[C2(o, i, j)]) / pr) * 0.5;
            }
            double dix = o->x1[C2(o, i, j)] - o->x1[C2(o, i - 1, j)];
            double diy = o->y1[C2(o, i, j)] - o->y1[C2(o, i - 1, j)];
            double djx = (o->x1[C2(o, i - 1, j + 1)] + o->x1[C2(o, i, j + 1)] - o->x1[C2(o, i - 1, j - 1)] - o->x1[C2(o, i, j - 1)]) * 0.25;
            double djy = (o->y1[C2(o, i - 1, j + 1)] + o->y1[C2(o, i, j + 1)] - o->y1[C2(o, i - 1, j - 1)] - o->y1[C2(o, i, j - 1)]) * 0.25;
            double ds = 1.0 / (dix * djy - djx * diy);
            double diu = uu[C2(o, i, j)] - uu[C2(o, i - 1, j)];
            double div = vv[C2(o, i, j)] - vv[C2(o, i - 1, j)];
            double dit = T[C2(o, i, j)] - T[C2(o, i - 1, j)];
            double dju = (uu[C2(o, i - 1, j + 1)] + uu[C2(o, i, j + 1)] - uu[C2(o, i - 1, j - 1)] - uu[C2(o, i, j - 1)]) * 0.25;
            double djv = (vv[C2(o, i - 1, j + 1)] + vv[C2(o, i, j + 1)] - vv[C2(o, i - 1, j - 1)] - vv[C2(o, i, j - 1)]) * 0.25;
            double djt = (T[C2(o, i - 1, j + 1)] + T[C2(o, i, j + 1)] - T[C2(o, i - 1, j - 1)] - T[C2(o, i, j - 1)]) * 0.25;
            double ux = (diu * djy - dju * diy) * ds, vx = (div * djy - djv * diy) * ds, tx = (dit * djy - djt * diy) * ds;
            double uy = (-diu * djx + dju * dix) * ds, vy = (-div * djx + djv * dix) * ds, ty = (-dit * djx + djt * dix) * ds;
            double t11 = ((4.0 / 3.0) * ux - (2.0 / 3.0) * vy) * amu1;
            double t22 = ((4.0 / 3.0) * vy - (2.0 / 3.0) * ux) * amu1;
            double t12 = (uy + vx) * amu1;
            double t33 = amu1 * (-(2.0 / 3.0) * ux - (2.0 / 3.0) * vy);
            double qx = amk1 * tx, qy = amk1 * ty;
            size_t c = C2(o, i, j);
            o->tao_i_in[c * 4 + 0] = t11; o->tao_i_in[c * 4 + 1] = t22;
            o->tao_i_in[c * 4 + 2] = t12; o->tao_i_in[c * 4 + 3] = t33;
            o->q_i_in[c * 2 + 0] = qx; o->q_i_in[c * 2 + 1] = qy;
            double *tg = &o->tao_i_g[c * 4], *qg = &o->q_i_g[c * 2];
            if (!lo && !hi) {
                double tmp = (SG(o, 5, i, j) + SG(o, 6, i, j) + SG(o, 10, i, j) + SG(o, 5, i - 1, j) + SG(o, 6, i - 1, j) + SG(o, 10, i - 1, j)) / 6.0;
                tg[0] = -((SG(o, 5, i, j) + SG(o, 5, i - 1, j)) / 2.0 - tmp) / g2 - t11;
                tg[1] = -((SG(o, 6, i, j) + SG(o, 6, i - 1, j)) / 2.0 - tmp) / g2 - t22;
                tg[2] = -(SG(o, 7, i, j) + SG(o, 7, i - 1, j)) / 2.0 / g2 - t12;
                tg[3] = -((SG(o, 10, i, j) + SG(o, 10, i - 1, j)) / 2.0 - tmp) / g2 - t33;
                qg[0] = -(SG(o, 8, i - 1, j) + SG(o, 8, i, j)) / 2.0 * q2 - qx;
                qg[1] = -(SG(o, 9, i - 1, j) + SG(o, 9, i, j)) / 2.0 * q2 - qy;
            } else {
                int ic = lo ? i : i - 1;
                double tmp = (SG(o, 5, ic, j) + SG(o, 6, ic, j) + SG(o, 10, ic, j)) / 3.0;
                tg[0] = -(SG(o, 5, ic, j) - tmp) / g2 - t11;
                tg[1] = -(SG(o, 6, ic, j) - tmp) / g2 - t22;
                tg[2] = -SG(o, 7, ic, j) / g2 - t12;
                tg[3] = -(SG(o, 10, ic, j) - tmp) / g2 - t33;
                qg[0] = -SG(o, 8, ic, j) * q2 - qx;
                qg[1] = -SG(o, 9, ic, j) * q2 - qy;
            }
        }
    /* j-faces, :358-453 */
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx - 1; i++) {
            int lo = (j == 1) && !pery, hi = (j == ny) && !pery;
            double amu1, amk1;
            if (lo) { amu1 = amu[C2(o, i, j)]; amk1 = cp * (amu[C2(o, i, j)] / pr); }
            else if (hi) { amu1 = amu[C2(o, i, j - 1)]; amk1 = cp * (amu[C2(o, i, j - 1)] / pr); }
            else {
                amu1 = (amu[C2(o, i, j)] + amu[C2(o, i, j - 1)]) * 0.5;
                amk1 = cp * ((amu[C2(o, i, j - 1)] + amu[C2(o, i, j)]) / pr) * 0.5;
            }
            double dix = (o->x1[C2(o, i + 1, j - 1)] + o->x1[C2(o, i + 1, j)] - o->x1[C2(o, i - 1, j - 1)] - o->x1[C2(o, i - 1, j)]) * 0.25;
            double diy = (o->y1[C2(o, i + 1, j - 1)] + o->y1[C2(o, i + 1, j)] - o->y1[C2(o, i - 1, j - 1)] - o->y1[C2(o, i - 1, j)]) * 0.25;
            double djx = o->x1[C2(o, i, j)] - o->x1[C2(o, i, j - 1)];
            double djy = o->y1[C2(o, i, j)] - o->y1[C2(o, i, j - 1)];
            double ds = 1.0 / (dix * djy - djx * diy);
            double diu = (uu[C2(o, i + 1, j - 1)] + uu[C2(o, i + 1, j)] - uu[C2(o, i - 1, j - 1)] - uu[C2(o, i - 1, j)]) * 0.25;
            double div = (vv[C2(o, i + 1, j - 1)] + vv[C2(o, i + 1, j)] - vv[C2(o, i - 1, j - 1)] - vv[C2(o, i - 1, j)]) * 0.25;
            double dit = (T[C2(o, i + 1, j - 1)] + T[C2(o, i + 1, j)] - T[C2(o, i - 1, j - 1)] - T[C2(o, i - 1, j)]) * 0.25;
            double dju = uu[C2(o, i, j)] - uu[C2(o, i, j - 1)];
            double djv = vv[C2(o, i, j)] - vv[C2(o, i, j - 1)];
            double djt = T[C2(o, i, j)] - T[C2(o, i, j - 1)];
            double ux = (diu * djy - dju * diy) * ds, vx = (div * djy - djv * diy) * ds, tx = (dit * djy - djt * diy) * ds;
            double uy = (-diu * djx + dju * dix) * ds, vy = (-div * djx + djv * dix) * ds, ty = (-dit * djx + djt * dix) * ds;
            double t11 = ((4.0 / 3.0) * ux - (2.0 / 3.0) * vy) * amu1;
            double t22 = ((4.0 / 3.0) * vy - (2.0 / 3.0) * ux) * amu1;
            double t12 = (uy + vx) * amu1;
            double t33 = amu1 * (-(2.0 / 3.0) * ux - (2.0 / 3.0) * vy);
            double qx = amk1 * tx, qy = amk1 * ty;
            size_t c = C2(o, i, j);
            o->tao_j_in[c * 4 + 0] = t11; o->tao_j_in[c * 4 + 1] = t22;
            o->tao_j_in[c * 4 + 2] = t12; o->tao_j_in[c * 4 + 3] = t33;
            o->q_j_in[c * 2 + 0] = qx; o->q_j_in[c * 2 + 1] = qy;
            double *tg = &o->tao_j_g[c * 4], *qg = &o->q_j_g[c * 2];
            if (!lo && !hi) {
                double tmp = (SG(o, 5, i, j) + SG(o, 6, i, j) + SG(o, 10, i, j) + SG(o, 5, i, j - 1) + SG(o, 6, i, j - 1) + SG(o, 10, i, j - 1)) / 6.0;
                tg[0] = -((SG(o, 5, i, j) + SG(o, 5, i, j - 1)) / 2.0 - tmp) / g2 - t11;
                tg[1] = -((SG(o, 6, i, j) + SG(o, 6, i, j - 1)) / 2.0 - tmp) / g2 - t22;
                tg[2] = -(SG(o, 7, i, j) + SG(o, 7, i, j - 1)) / 2.0 / g2 - t12;
                tg[3] = -((SG(o, 10, i, j) + SG(o, 10, i, j - 1)) / 2.0 - tmp) / g2 - t33;
                qg[0] = -(SG(o, 8, i, j - 1) + SG(o, 8, i, j)) / 2.0 * q2 - qx;
                qg[1] = -(SG(o, 9, i, j - 1) + SG(o, 9, i, j)) / 2.0 * q2 - qy;
            } else {
                int jc = lo ? j : j - 1;
                double tmp = (SG(o, 5, i, jc) + SG(o, 6, i, jc) + SG(o, 10, i, jc)) / 3.0;
                tg[0] = -(SG(o, 5, i, jc) - tmp) / g2 - t11;
                tg[1] = -(SG(o, 6, i, jc) - tmp) / g2 - t22;
                tg[2] = -SG(o, 7, i, jc) / g2 - t12;
                tg[3] = -(SG(o, 10, i, jc) - tmp) / g2 - t33;
                qg[0] = -SG(o, 8, i, jc) * q2 - qx;
                qg[1] = -SG(o, 9, i, jc) * q2 - qy;
            }
        }
#undef UU
    free(U); free(d); free(uu); free(vv); free(T); free(amu);
    return HYB_OK;
}

int orc_hot(orc *o, double *tao_i, double *q_i, double *tao_j, double *q_j)
{
    size_t nc = (size_t)(o->nx + 3) * (o->ny + 3);
    if (tao_i) memcpy(tao_i, o->tao_i_g, nc * 4 * sizeof(double));
    if (q_i) memcpy(q_i, o->q_i_g, nc * 2 * sizeof(double));
    if (tao_j) memcpy(tao_j, o->tao_j_g, nc * 4 * sizeof(double));
    if (q_j) memcpy(q_j, o->q_j_g, nc * 2 * sizeof(double));
    return HYB_OK;
}

int orc_nsf_in(orc *o, double *tao_i, double *q_i, double *tao_j, double *q_j)
{
    size_t nc = (size_t)(o->nx + 3) * (o->ny + 3);
    if (tao_i) memcpy(tao_i, o->tao_i_in, nc * 4 * sizeof(double));
    if (q_i) memcpy(q_i, o->q_i_in, nc * 2 * sizeof(double));
    if (tao_j) memcpy(tao_j, o->tao_j_in, nc * 4 * sizeof(double));
    if (q_j) memcpy(q_j, o->q_j_in, nc * 2 * sizeof(double));
    return HYB_OK;
}

/* ---- Hybrid_Time_advance_LU_SGS (Hybrid_Sub.f90:4-43) as shipped (GSIS
 *      block commented) plus the periodic exchanges. -------------------- */
int orc_step(orc *o, int n_iter, hyb_residual *r)
{
    if (n_iter < 1) return HYB_ERR_INVALID;
    for (int it = 0; it < n_iter; it++) {
        memcpy(o->S0, o->S, o->P * NSUM * sizeof(double));   /* S0_GKUA := S_GKUA, :29-38 */
        orc_exchange_f(o);
        orc_phy_boundary(o);
        orc_kinetic_step(o);
        orc_detfp(o);
        orc_convert_ns(o);
        if (o->gsis.enable) {
            /* a synthetic solve that leaves the physical range corrects
             * nothing: the kinetic step of this iteration stands (the
             * reference STOPs, sub_NS_singlegrid.f90:148-151) */
            int rc = orc_gsis_solve(o);
            if (rc == HYB_ERR_TEMPERATURE || rc == HYB_ERR_NONFINITE) o->gsis_skipped++;
            else if (rc) return rc;
        }
    }
    if (r) orc_detfp_res(o, r);
    return HYB_OK;
}

/* ---- velocity grids ------------------------------------------------------ */
/* Gauss-Legendre nodes/weights on [-1,1] by Newton iteration on P_n (the
 * classical algorithm); the reference lists the same rules as 10-digit
 * REAL(4) literals, GKUA_lisansudu.f90:298-353. */
static void gauss_legendre(int n, double *x, double *w)
{
    for (int k = 0; k < n; k++) {
        double z = cos(PI * (k + 0.75) / (n + 0.5)), dp = 0.0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int l = 2; l <= n; l++) {
                double p2 = ((2.0 * l - 1.0) * z * p1 - (l - 1.0) * p0) / l;
                p0 = p1;
                p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0; }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        double p0 = 1.0, p1 = z;
        for (int l = 2; l <= n; l++) {
            double p2 = ((2.0 * l - 1.0) * z * p1 - (l - 1.0) * p0) / l;
            p0 = p1;
            p1 = p2;
        }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[k] = -z;   /* ascending */
        w[k] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

int orc_grid_gl(double dv, int n, double vdown, int kgln, int single_literals, double *v, double *w)
{
    if (kgln < 1 || kgln > 10 || n < 1) return -1;
    double a[10], h[10];
    gauss_legendre(kgln, a, h);
    if (single_literals)
        for (int k = 0; k < kgln; k++) {
            /* the table is symmetric: round the positive node, mirror it */
            double ap = fabs(a[k]);
            a[k] = (a[k] < 0 ? -1.0 : 1.0) * (double)(float)ap;
            if (ap < 1e-14) a[k] = 0.0;
            h[k] = (double)(float)h[k];
        }
    int m = 0;
    for (int iv = 0; iv < n; iv++) {
        double va = vdown + (double)iv * dv, vb = vdown + (double)(iv + 1) * dv;
        double vapb = (va + vb) / 2., vbma = (vb - va) / 2.;   /* DISVEL :206-207 */
        for (int k = 0; k < kgln; k++) {
            v[m] = vapb + vbma * a[k];
            w[m] = vbma * h[k];   /* FBAV * w, GKUA_DETFP.f90:314 */
            m++;
        }
    }
    return m;
}

int orc_grid_nc(int n, double vdown, double vup, int rule, double *v, double *w)
{
    if (n < 2) return -1;
    double dv = (vup - vdown) / (n - 1);
    for (int k = 0; k < n; k++) { v[k] = vdown + k * dv; w[k] = 0.0; }
    if (rule == 1) {
        /* reference pattern, GKUA_DETFP.f90:419-444 (1-based index kk) */
        for (int k = 0; k < n; k++) {
            int kk = k + 1;
            double c = (kk == 1 || kk == n) ? 1.0 : ((kk % 2 == 0) ? 4.0 : 2.0);
            w[k] = dv / 3.0 * c;
        }
        return n;
    }
    int intervals = n - 1;
    int simpson = (intervals % 2 == 0) ? intervals : intervals - 3;
    if (simpson < 0) {   /* n == 2: trapezoid */
        w[0] = w[1] = dv / 2.0;
        return n;
    }
    for (int p = 0; p < simpson; p += 2) {
        w[p] += dv / 3.0;
        w[p + 1] += 4.0 * dv / 3.0;
        w[p + 2] += dv / 3.0;
    }
    if (simpson != intervals) {   /* closing Simpson 3/8 panel */
        int p = simpson;
        w[p] += 3.0 * dv / 8.0;
        w[p + 1] += 9.0 * dv / 8.0;
        w[p + 2] += 9.0 * dv / 8.0;
        w[p + 3] += 3.0 * dv / 8.0;
    }
    return n;
}

double orc_cfc_vhs(double mole_mass, double gamma, double alp, double omg, double vis_ref, double tref, double ma,
                   double nd_inf, double t_inf, double lref, double *re_out)
{
    (void)alp;
    const double boltz = (double)1.38065E-23f, matom = (double)1.66053873E-27f;   /* COMMONDATA.f90:9 */
    double rcon = boltz / (matom * mole_mass);
    double vis_inf = vis_ref * pow(t_inf / tref, omg);
    double re = nd_inf * matom * mole_mass * ma * sqrt(gamma * rcon * t_inf) * lref / vis_inf;
    if (re_out) *re_out = re;
    return re / (ma * sqrt(2.0 * gamma));
}
