/*
 * hyb_oracle_impl.h -- private definitions shared by the oracle's C files.
 * TEST INFRASTRUCTURE ONLY (see hyb_oracle.h).
 */
#ifndef HYB_ORACLE_IMPL_H
#define HYB_ORACLE_IMPL_H

#include "hyb_oracle.h"

#include <stddef.h>

#define LAP 2
#define NRD 2
#define NSUM 11
#define PI 3.1415926535897932

/* REAL(4) literals of the reference, widened to double the way the Fortran
 * compiler widens them: 1.E-30 (GKUA_Residual.f90:104), 1.E-15
 * (RHSFDVsub :143), 1./3. and 2./3. (:144). */
#define F_FLOOR ((double)1.0e-30f)
#define EPSWENO ((double)1.0e-15f)
#define CWENO1 ((double)(1.0f / 3.0f))
#define CWENO2 ((double)(2.0f / 3.0f))

struct orc_ns;

struct orc {
    int nx, ny, nvi, nvj, nv;
    int pw;               /* (nx+7): pitch of -3:nx+3 arrays                  */
    size_t P;             /* (nx+7)*(ny+7)                                    */
    int bc[4];
    double *wall_u[4], *wall_v[4], *wall_t[4];
    double *vi, *vj, *wi, *wj;
    hyb_params prm;
    /* geometry */
    double *xn, *yn;      /* nodes on (1-LAP:nx+LAP, 1-LAP:ny+LAP)           */
    double *vol, *si, *sj, *ni1, *ni2, *nj1, *nj2;   /* (nx,ny)               */
    double *x1, *y1;      /* cell centres on (1-LAP:nx+LAP-1, ...)           */
    /* state */
    double *frd, *frd00, *S, *S0, *CF;
    double *tao_i_g, *q_i_g, *tao_j_g, *q_j_g;        /* HoT, C2 extents      */
    double *tao_i_in, *q_i_in, *tao_j_in, *q_j_in;    /* NSF from kinetic     */
    double err;
    double m0;            /* total mass when the state was set (mass_pin)     */
    struct orc_ns *ns;           /* GSIS synthetic solver state (hyb_oracle_ns.c) */
    hyb_gsis_params gsis;
    int gsis_last_inner;
    int gsis_skipped;     /* outer iterations whose synthetic correction was
                             skipped (NS state out of range)                */
};

/* ---- index helpers ------------------------------------------------------ */
#define IX(o, i, j) ((size_t)((i) + 3) + (size_t)(o)->pw * (size_t)((j) + 3))
#define FRD(o, ird, i, j, v) (o)->frd[((size_t)(v) * (o)->P + IX(o, i, j)) * NRD + (ird)]
#define FRD00(o, ird, i, j, v) (o)->frd00[((size_t)(v) * (o)->P + IX(o, i, j)) * NRD + (ird)]
#define SG(o, k, i, j) (o)->S[IX(o, i, j) * NSUM + (k) - 1]
#define CFA(o, i, j) (o)->CF[IX(o, i, j)]
#define MI(o, i, j) ((size_t)((i) - 1) + (size_t)(o)->nx * (size_t)((j) - 1))
#define XN(o, i, j) ((size_t)((i) + 1) + (size_t)((o)->nx + 4) * (size_t)((j) + 1))
#define C2(o, i, j) ((size_t)((i) + 1) + (size_t)((o)->nx + 3) * (size_t)((j) + 1))


void orc_ns_free(orc *o);
void orc_build_u(orc *o, double *U);
int orc_kinetic_residual_moments(orc *o, double *rk);
void orc_feq(const orc *o, const double *s6, int iv, int jv, double *g, double *h);
int orc_gsis_solve(orc *o);
double orc_total_mass(const orc *o);

#endif
