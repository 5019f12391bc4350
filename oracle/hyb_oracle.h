/*
 * hyb_oracle.h -- CPU FP64 restatement of the Hybrid2D kinetic hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA implementation is
 * checked against; it is never linked into, loaded by, or called from the
 * product library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may use it.
 *
 * Every routine restates one reference subroutine loop by loop and cites the
 * Fortran file:line it follows.  Arrays use the reference's own extents and
 * Fortran column-major order, so FRD / S_GKUA / CF can be compared with the
 * GPU path through the C ABI without any re-layout:
 *   FRD(NRD,-3:nx+3,-3:ny+3,NVIT,NVJT)      COMMONDATA.f90:49, sub_init.f90:344
 *   S_GKUA(Nsum,-3:nx+3,-3:ny+3)            sub_init.f90:351
 *   CF(1-LAP:nx+LAP-1,1-LAP:ny+LAP-1)       sub_init.f90:355 (stored here on the
 *                                            -3:n+3 extents for simplicity)
 * Parity: pinned to the reference's own output Hybrid2D/output/flow2d-GKUA.dat
 * (uniform step-0 moments of the shipped cylinder case, Gauss-Legendre grid,
 * reproduced to all printed digits) and to the reference's quadrature
 * self-check; the Couette extensions (periodic faces, moving walls, per-face
 * wall temperature, Newton-Cotes weights) are unpinned by the reference.
 */
#ifndef HYB_ORACLE_H
#define HYB_ORACLE_H

#include "../include/hyb_dvm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc orc;

/* lifecycle; same argument meaning as hyb_create */
int  orc_create(const hyb_mesh *mesh, const hyb_vgrid *vg, const hyb_params *p, orc **out);
void orc_destroy(orc *o);
int  orc_set_threads(int n);            /* OpenMP threads used by the oracle */

/* the stages, named after the reference subroutines */
int orc_init_maxwellian(orc *o, double rho, double u, double v, double t);
int orc_exchange_f(orc *o);             /* GKUA_inner_mesco_boundary (periodic) */
int orc_phy_boundary(orc *o);           /* GKUA_Phy_boundary                    */
int orc_kinetic_step(orc *o);           /* GKUA_Residual (Get_Feq, RHSFDVsub, sweeps) */
int orc_detfp(orc *o);                  /* DETFP + GKUA_DET_wall + macro exchange */
int orc_convert_ns(orc *o);             /* Convert_NS                           */
int orc_detfp_res(orc *o, hyb_residual *r);   /* DETFP_res                      */
int orc_hoq(orc *o, double *hot, double *hoq); /* HOT_GKUA / HOQ_GKUA         */
int orc_step(orc *o, int n_iter, hyb_residual *r);  /* Hybrid_Time_advance_LU_SGS */

/* state access (pointers into the oracle's own reference-layout arrays) */
double *orc_frd(orc *o);                /* FRD                                  */
double *orc_frd00(orc *o);              /* FRD00 (RHS after a kinetic step)     */
double *orc_s(orc *o);                  /* S_GKUA                               */
double *orc_cf(orc *o);                 /* CF on -3:n+3 extents                 */
int     orc_upload_f(orc *o, const double *frd);   /* copy + recompute moments  */
/* HoT arrays on (1-LAP:nx+LAP-1,1-LAP:ny+LAP-1) extents, 4 / 2 components */
int     orc_hot(orc *o, double *tao_i, double *q_i, double *tao_j, double *q_j);
/* NS-side stress at faces computed from the kinetic state (TaoNSi_in ...) */
int     orc_nsf_in(orc *o, double *tao_i, double *q_i, double *tao_j, double *q_j);
double  orc_err(orc *o);                /* DETFP's CF-change diagnostic ERR     */

/* GSIS synthetic solve (hyb_oracle_ns.c) */
int orc_gsis_configure(orc *o, const hyb_gsis_params *gp);
int orc_gsis_last_inner(orc *o);
int orc_gsis_skipped(orc *o);           /* corrections skipped since configure */
int orc_ns_state(orc *o, double *U);                  /* U[4][(nx+3)(ny+3)] */
int orc_ns_residual(orc *o, const double *U, double *res);

/* geometry derived from the nodes (Creat_Mesh, Update_coordinate_buffer) */
int orc_geometry(orc *o, double *vol, double *si, double *sj, double *ni1,
                 double *ni2, double *nj1, double *nj2, double *x1, double *y1);

/* ---- velocity grids (GKUA_lisansudu.f90) -------------------------------- */
/* Gauss-Legendre: n intervals of width dv from vdown, kgln points each.  The
 * reference's node/weight table is made of REAL(4) literals
 * (GKUA_lisansudu.f90:305-351); single_literals=1 reproduces that rounding.
 * Writes n*kgln nodes and full weights (FBAV*w).  Returns the node count. */
int orc_grid_gl(double dv, int n, double vdown, int kgln, int single_literals,
                double *v, double *w);
/* Half-range Gauss-Hermite (GKUA_lisansudu.f90:103-118, 364-436), nh in
 * {7,8,16}; 2*nh nodes; weights returned as w*exp(v^2) (GKUA_DETFP.f90:200). */
/* Uniform Newton-Cotes grid of n nodes on [vdown,vup].  rule 0: composite
 * Simpson 1/3 with a closing 3/8 panel when n is even; rule 1: the
 * reference's end/even/odd = 1/4/2 pattern (GKUA_DETFP.f90:419-444). */
int orc_grid_nc(int n, double vdown, double vup, int rule, double *v, double *w);

/* cfc of the reference from control.in quantities (sub_init.f90:13-66),
 * VHS only; Boltz and Matom are REAL(4) literals (COMMONDATA.f90:9). */
double orc_cfc_vhs(double mole_mass, double gamma, double alp, double omg,
                   double vis_ref, double tref, double ma, double nd_inf,
                   double t_inf, double lref, double *re_out);

#ifdef __cplusplus
}
#endif
#endif
