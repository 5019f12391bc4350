/*
 * hyb_dvm.h -- C ABI of the GB300 discrete-velocity Shakhov solver.
 *
 * This is the drop-in boundary for the kinetic hot path of Hybrid2D.  In the
 * reference every routine on that path is an argument-less Fortran subroutine
 * that reads and writes module globals (Global_Var, Com_ctrl in
 * Hybrid2D/src/COMMONDATA.f90:28-170).  Here the same state lives in an opaque
 * context that owns all device memory; the Fortran host keeps its mesh, input
 * and restart handling and passes plain arrays (Fortran column-major, the
 * reference's own extents) through these entry points.  A Fortran
 * ISO_C_BINDING interface module for every function is in hyb_dvm.f90.
 *
 * Conventions
 *   - every call returns an int status: HYB_OK (0) or a negative HYB_ERR_*;
 *     nothing aborts the process (the reference uses STOP / MPI_FINALIZE);
 *   - host arrays stay owned by the caller; the context owns device buffers;
 *   - one host thread per context; contexts are independent;
 *   - device waits are bounded and surface as HYB_ERR_TIMEOUT.
 *
 * Index conventions follow the reference: a block has nx*ny mesh NODES, cells
 * are i=1..nx-1, j=1..ny-1, i-faces i=1..nx, j-faces j=1..ny.  The block faces
 * are numbered like Bc%face in Hybrid2D/src/sub_init.f90:269-277:
 * 1 = i-min, 2 = j-min, 3 = i-max, 4 = j-max.
 */
#ifndef HYB_DVM_H
#define HYB_DVM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define HYB_OK                 0
#define HYB_ERR_INVALID       -1   /* bad argument / size / null pointer      */
#define HYB_ERR_NOMEM         -2   /* device or host allocation failed        */
#define HYB_ERR_CUDA          -3   /* CUDA runtime error                      */
#define HYB_ERR_NONFINITE     -4   /* NaN/Inf detected in a residual          */
#define HYB_ERR_TIMEOUT       -5   /* a bounded device wait ran out           */
#define HYB_ERR_UNSUPPORTED   -6   /* configuration outside the built scope   */
#define HYB_ERR_TEMPERATURE   -7   /* NS temperature below 0.1 (reference
                                      sub_NS_singlegrid.f90:148-151 STOPs)    */
#define HYB_ERR_NODEVICE      -8   /* no CUDA device / extension not usable   */

/* ---- boundary kinds (values follow const_var, COMMONDATA.f90:14) -------- */
#define HYB_BC_WALL        (-2)    /* diffuse wall, GKUA_boundary.f90:49-100  */
#define HYB_BC_PERIODIC      1     /* face connected to the opposite face of
                                      the same block (inner boundary with
                                      neighb = own block, GKUA_boundary.f90:
                                      400-633 exchange semantics)            */

/* ---- kinetic spatial schemes (GKUA_Scheme_*, COMMONDATA.f90:18) -------- */
#define HYB_SCHEME_UP1     0
#define HYB_SCHEME_NND     1
#define HYB_SCHEME_WENO3   3

/* ---- precision modes ---------------------------------------------------- */
#define HYB_PREC_FP64      0       /* f, fluxes, sweeps, moments in FP64      */
#define HYB_PREC_MIXED     1       /* f, fluxes, sweeps in FP32; moments,
                                      residual, synthetic solve in FP64      */

/* ---- order of the kinetic implicit step (hyb_params.sweep_order) -------- */
#define HYB_SWEEP_REFERENCE 0      /* GKUA_Residual.f90:28-112 as written: a
                                      forward sweep in increasing (i, j) and a
                                      backward step that reads the forward
                                      values of the downstream neighbours     */
#define HYB_SWEEP_UPWIND    1      /* one Gauss-Seidel sweep per velocity in
                                      its own upwind order (i and j each
                                      reversed where that velocity component
                                      is negative): the same operator alpha
                                      and the same RHS, solved exactly for the
                                      first-order upwind transport.  Per step
                                      it differs from the reference; a
                                      converged state (RHS = 0) is the same.
                                      No counterpart in the reference.        */

/* ---- moment vector length (Nsum, COMMONDATA.f90:4) ---------------------- */
#define HYB_NSUM          11
#define HYB_NRD            2       /* reduced distributions G and H          */

/* Mesh of one structured block.  Node coordinates are (nx, ny) Fortran
 * column-major, exactly B%x / B%y as read by Creat_Mesh
 * (Hybrid2D/src/sub_init.f90:178-180).  The library derives vol, si, sj,
 * ni1, ni2, nj1, nj2 (sub_init.f90:183-208) and the ghost-node / cell-centre
 * coordinates (sub_init.f90:719-823) itself. */
typedef struct hyb_mesh {
    int nx, ny;                 /* nodes; nx >= 3, ny >= 5                    */
    const double *x, *y;        /* node coordinates, nx*ny each               */
    int bc[4];                  /* HYB_BC_* for faces 1..4                    */
    /* Diffuse-wall data per wall face, one value per face cell in face order
     * (faces 2/4: i=1..nx-1, faces 1/3: j=1..ny-1).  NULL for non-wall faces.
     * The reference hard-codes wall_u=wall_v=0 (GKUA_boundary.f90:66-67) and
     * one global Twall; here every face cell carries its own values. */
    const double *wall_u[4], *wall_v[4], *wall_t[4];
} hyb_mesh;

/* Discrete velocity grid (GKUA_lisansudu.f90).  w_i / w_j are the complete
 * one-dimensional moment weights: FBAV*w for Gauss-Legendre
 * (GKUA_DETFP.f90:314), w*exp(v^2) for half-range Gauss-Hermite
 * (GKUA_DETFP.f90:200-202), the Newton-Cotes rule for uniform grids. */
typedef struct hyb_vgrid {
    int nvi, nvj;
    const double *vi, *vj;      /* nodes                                      */
    const double *wi, *wj;      /* full 1-D weights                           */
} hyb_vgrid;

/* Solver parameters (control.in / Com_ctrl equivalents). */
typedef struct hyb_params {
    double dt;          /* dt_global_GKUA (GKUA_Residual.f90:27)              */
    double cfc;         /* collision coefficient delta (sub_init.f90:65)      */
    double cpr;         /* Shakhov coefficient (1-Pr)/(5/2) (sub_init.f90:66) */
    double x1s;         /* 1 - viscosity exponent omega (sub_init.f90:14)    */
    double r00, t00;    /* positivity fall-backs of DETFP (GKUA_DETFP.f90:63,72) */
    int    scheme;      /* HYB_SCHEME_*                                       */
    int    precision;   /* HYB_PREC_*                                         */
    /* macroscopic (NS / GSIS) scaling, sub_init.f90:16-66 */
    double gamma, ma, pr, re;   /* Re = cfc * Ma * sqrt(2 gamma)             */
    double omega_ns;            /* NS viscosity exponent; the reference's
                                   get_viscous hard-codes 0.81
                                   (sub_Residual.f90:563)                    */
    int    device;              /* CUDA device ordinal                       */
    int    sweep_order;         /* HYB_SWEEP_*: order of the kinetic LU-SGS step */
    int    mass_pin;            /* 1: hold the total mass sum(vol rho) of f at
                                   its value when the state was set
                                   (hyb_init_maxwellian / hyb_upload_f): every
                                   kinetic step multiplies its updated f by
                                   m0 / M, M the total mass of the state the
                                   step starts from.  The closed channel's
                                   steady states form a family indexed by the
                                   total mass, and an iteration that does not
                                   conserve mass ends on a member that depends
                                   on its path; pinned, every variant ends on
                                   the member of mass m0.  0: the reference's
                                   update.  No counterpart in the reference.  */
    int    reserved[5];
} hyb_params;

/* Residual of the kinetic iteration: moments 1..4 of the last RHS,
 * DETFP_res (GKUA_DETFP_RES.f90:4-60). */
typedef struct hyb_residual {
    double res_max[4];
    double res_rms[4];
    double max_rms;             /* max over the four rms values               */
} hyb_residual;

/* Parameters of the GSIS synthetic macroscopic solve (the commented coupling
 * of Hybrid_Sub.f90:45-153 plus the NS solver of sub_NS_singlegrid.f90). */
typedef struct hyb_gsis_params {
    int    enable;          /* 0: plain kinetic iteration                    */
    int    max_inner;       /* cap on NS inner iterations per outer step     */
    double inner_tol;       /* reference: res_iter > 1e-6 (Hybrid_Sub.f90:99) */
    double inner_rtol;      /* also stop once max|Res(4)| <= inner_rtol times its
                               value at the first inner iteration (0: off)   */
    double cfl, dtmax, dtmin;   /* local time step (sub_NS_singlegrid.f90:160-183) */
    int    flux;            /* NS flux splitting, Flux_* (COMMONDATA.f90:12) */
    int    ns_scheme;       /* NS reconstruction: 1 NND2 (Scheme_*, :11), 0 first
                               order, 2 NND2 stencil without the limiter      */
    int    mlp_warm_after;  /* > 0: after this many outer iterations since
                               configuration, hyb_step runs the learned warm
                               start once (hyb_gsis_warm_start); if its closure
                               solve leaves the physical range the state is
                               left as it was and the iteration goes on      */
    int    ns_solver;       /* inner solver: 0 LU-SGS (du_LU_SGS_2D,
                               sub_LU_SGS.f90), 1 line-implicit ADI with the
                               LU-SGS diagonal and scalar couplings, exact
                               along each mesh line, 2 the LU-SGS matrix
                               with its 4x4 flux-Jacobian blocks solved
                               exactly along every wall-normal line, lines
                               in red-black Gauss-Seidel order (1 and 2 have
                               no counterpart in the reference)             */
    int    correct_f;       /* 1: after the moment correction also correct the
                               distribution, f += feq(S) - feq(S_k) on the band
                               (the reference corrects the moments only)     */
    int    no_mass_projection;  /* 1: keep the band's mean density change   */
    int    lusgs_planes;    /* oracle only: the reference's anti-diagonal
                               LU-SGS order instead of two colours           */
    int    mlp_warm_inner;  /* inner iterations of the warm start (0: 2000) */
    double mlp_warm_rtol;   /* ... or until max|Res(4)| drops by this factor
                               (0: 1e-3)                                     */
    int    wall_band;       /* 1: the band reaches the walls (cells 1..n-1);
                               the wall ghost cells take the reference's
                               no-slip reflection (boundary_wall,
                               sub_boundary.f90:51-118) about the kinetic
                               state at the wall face, frozen for the solve.
                               0: the reference's band 3..n-3 with the
                               kinetic state held outside it              */
    int    relax_pct;       /* the correction is applied as U_k + r (U - U_k),
                               r = relax_pct / 100 (0: r = 1, the reference)  */
    int    line_mean;       /* ns_solver 2 with a periodic axis across the
                               lines: 1 also solves, in each inner iteration
                               and before the line passes, the system of the
                               correction that is constant across the
                               periodic axis (the line system averaged over
                               the lines); n = 2..4 adds the harmonics
                               1..n-1 across that axis, each one complex
                               averaged system with the line-mean
                               coefficients; no counterpart in the
                               reference                                    */
} hyb_gsis_params;

typedef struct hyb_ctx hyb_ctx;

/* ---- lifecycle ---------------------------------------------------------- */
/* Replaces init / Alloc_GKUA_FRD (sub_init.f90:6-79, 329-386).
 * Size limits (HYB_ERR_UNSUPPORTED otherwise): the sweep's scan axis is the
 * longer cell count that is <= 1024; above 256 cells it must be even and
 * above 512 a multiple of 4; a wall-normal axis has >= 4 cells. */
int hyb_create(const hyb_mesh *mesh, const hyb_vgrid *vgrid,
               const hyb_params *params, hyb_ctx **out);
int hyb_destroy(hyb_ctx *ctx);
/* Switches a context from HYB_PREC_MIXED to HYB_PREC_FP64 on the device
 * (no counterpart in the reference): the FP32 distribution is widened in a
 * new FP64 array, the other buffers of its type are made again at FP64 size,
 * and the moments are recomputed; iterations after the call run the FP64
 * path from that state.  A mixed run can thus finish its convergence in FP64
 * without a host round trip of f.  Only MIXED -> FP64 (HYB_ERR_UNSUPPORTED
 * otherwise, and for instances of a hyb_batch); the same precision is a
 * no-op.  Allocates device memory. */
int hyb_set_precision(hyb_ctx *ctx, int precision);
/* Human-readable text of the last error on this context (never NULL). */
const char *hyb_last_error(const hyb_ctx *ctx);
/* Library version / build string. */
const char *hyb_version(void);

/* ---- state transfer ----------------------------------------------------- */
/* Uniform Maxwellian initial state and first moments: init_flow_zero +
 * GKUA_sudufenbu (sub_init.f90:390-463, GKUA_sudufenbu.f90:22-53). */
int hyb_init_maxwellian(hyb_ctx *ctx, double rho, double u, double v, double t);
/* f in the reference layout FRD(NRD,-3:nx+3,-3:ny+3,NVIT,NVJT), column-major
 * (COMMONDATA.f90:49, sub_init.f90:344).  Interior cells are transferred;
 * upload recomputes the moments (backup_Mesco_read + DETFP,
 * Backup_write_read.f90:93-108). */
int hyb_upload_f(hyb_ctx *ctx, const double *frd);
int hyb_download_f(hyb_ctx *ctx, double *frd);
/* S_GKUA(Nsum,-3:nx+3,-3:ny+3) (sub_init.f90:351) after DETFP: rho, u, v, T,
 * Pxx, Pyy, Pxy, qx, qy, Pzz, 0; CF(-1:nx+1,-1:ny+1) may be NULL. */
int hyb_download_moments(hyb_ctx *ctx, double *s_gkua, double *cf);
/* Higher-order terms of Convert_NS (Hybrid_Sub.f90:191-461):
 * TaoNSi_G(4,-1:nx+1,-1:ny+1), Qi_G(2,...), TaoNSj_G(4,...), Qj_G(2,...).
 * Any pointer may be NULL. */
int hyb_download_hot(hyb_ctx *ctx, double *tao_i, double *q_i,
                     double *tao_j, double *q_j);
/* Higher-order velocity moments of the current f (IntegralGaussHermite,
 * GKUA_DETFP.f90:174-229; written by output, IO.f90:442-445), for any
 * velocity grid: HOT_GKUA(6,-3:nx+3,-3:ny+3) = sums of w G vx^3, G vx^2 vy,
 * G vx vy^2, G vy^3, H vx, H vy; HOQ_GKUA(4,-3:nx+3,-3:ny+3) = sums of
 * w (G c^2 + H) vx^2, vx vy, vy^2 and a zero fourth component.  Interior
 * cells only (ghost cells are zero).  Either pointer may be NULL; allocates
 * a temporary device buffer. */
int hyb_download_hoq(hyb_ctx *ctx, double *hot, double *hoq);

/* ---- the iteration (Hybrid_Time_advance_LU_SGS, Hybrid_Sub.f90:4-160) --- */
/* n_iter outer iterations; each runs the boundary conditions, the kinetic
 * LU-SGS step, the moments, the wall moments and (when enabled) Convert_NS
 * and the GSIS synthetic solve.  Without GSIS, Convert_NS feeds only the NS /
 * HoT fields a caller downloads, so it runs on the call's last iteration
 * only; the state after the call is the same.  If out != NULL the residual
 * of the last iteration (DETFP_res) is written to it. */
int hyb_step(hyb_ctx *ctx, int n_iter, hyb_residual *out);
/* The same stages one at a time, named after the reference subroutines. */
int hyb_phy_boundary(hyb_ctx *ctx);          /* GKUA_Phy_boundary          */
int hyb_kinetic_step(hyb_ctx *ctx);          /* Hybrid_GKUA_Comput_Block   */
int hyb_detfp(hyb_ctx *ctx);                 /* DETFP + GKUA_DET_wall      */
int hyb_convert_ns(hyb_ctx *ctx);            /* Convert_NS                 */
int hyb_detfp_res(hyb_ctx *ctx, hyb_residual *out);   /* DETFP_res         */

/* ---- GSIS synthetic solve ---------------------------------------------- */
int hyb_gsis_configure(hyb_ctx *ctx, const hyb_gsis_params *gp);
/* Inner NS iterations used by the last outer iteration (Mesh%iter). */
int hyb_gsis_last_inner(const hyb_ctx *ctx, int *n_inner);
/* Outer iterations since hyb_gsis_configure whose synthetic correction was
 * skipped because the NS state left the physical range (temperature below
 * 0.1 or a non-finite residual): such an iteration keeps its kinetic step
 * uncorrected, where the reference STOPs (sub_NS_singlegrid.f90:148-151).
 * No counterpart in the reference. */
int hyb_gsis_skipped(const hyb_ctx *ctx, int *count);

/* Replace the diffuse-wall data of one wall face (1..4), one value per face
 * cell as in hyb_mesh.  The reference passes the wall velocity on every call
 * of GKUA_wall_boundary(nm, nn, wall_u, wall_v) (GKUA_wall_functions.f90:1)
 * and reads Twall from a global; this is that per-call input. */
int hyb_set_walls(hyb_ctx *ctx, int face, const double *wall_u,
                  const double *wall_v, const double *wall_t);

/* ---- DETFP without device allocation -----------------------------------
 * No counterpart in the reference.  For callers that cannot let this library
 * allocate device memory: a CUDA Fortran / OpenACC host that already keeps
 * FRD and S_GKUA as its own device arrays, or a process whose device memory
 * is reserved by another framework's pooling allocator.  Computes DETFP's
 * moments, primitive conversion and CF (GKUA_DETFP.f90:4-105) for the
 * interior cells i=1..nx-1, j=1..ny-1 of a device-resident FRD and writes
 * them into caller-owned device arrays; no context is needed and nothing is
 * allocated (no cudaMalloc / cudaFree, no library allocation).
 *   frd_dev     FRD(NRD,-3:nx+3,-3:ny+3,nvi,nvj), double, on the device
 *   vi/vj_dev   velocity nodes, wi/wj_dev full 1-D weights (hyb_vgrid)
 *   p           host struct; only cfc, x1s, r00, t00 are read
 *   s_gkua_dev  S_GKUA(Nsum,-3:nx+3,-3:ny+3); interior cells are written
 *   cf_dev      CF on the (1-LAP:nx+LAP-1, 1-LAP:ny+LAP-1) extents, or NULL
 *   stream      cudaStream_t to launch on (NULL: default stream)
 * Limits: at most HYB_NOALLOC_MAX_CELLS interior cells, else
 * HYB_ERR_UNSUPPORTED; every device pointer double-aligned (8 bytes), else
 * HYB_ERR_INVALID before any launch.  Intermediate sums live in one fixed
 * 16 MiB device array of the library, held by every device that loads the
 * library until the process exits; each call looks up that array's address
 * in the current context, and the first call on a device also loads the
 * library's device code there (make it before any stream capture).  Calls
 * share the array, so calls that overlap on the GPU (e.g. on two streams)
 * race. */
#define HYB_NOALLOC_MAX_CELLS 209715
int hyb_detfp_noalloc(int nx, int ny, int nvi, int nvj, const double *frd_dev,
                      const double *vi_dev, const double *vj_dev,
                      const double *wi_dev, const double *wj_dev,
                      const hyb_params *p, double *s_gkua_dev, double *cf_dev,
                      void *stream);

/* ---- failure injection for tests (no counterpart in the reference) ------ */
/* Arms one planted wait that nothing completes for the next hyb_step, with
 * every bounded device wait of that step limited to spin_cycles SM clocks
 * (> 0; the default limit is about two seconds).  site:
 *   HYB_STALL_SWEEP_ROW   the kinetic sweep never issues the bulk copy of
 *                         one row, so every CTA's wait on that row's
 *                         mbarrier runs out; the CTAs drain the copies they
 *                         issued and return before writing f;
 *   HYB_STALL_NS_BARRIER  block 0 of the synthetic solve's cooperative
 *                         inner loop (LU-SGS on meshes of up to 65,536
 *                         cells, band 3..n-3) never arrives at the grid
 *                         barrier, so every block's wait runs out.
 * The step returns HYB_ERR_TIMEOUT; the planted wait and the short limit
 * are then cleared, and the context stays usable (after a sweep stall f is
 * as it was before the step).  HYB_STALL_NONE disarms. */
#define HYB_STALL_NONE        0
#define HYB_STALL_SWEEP_ROW   1
#define HYB_STALL_NS_BARRIER  2
int hyb_test_stall(hyb_ctx *ctx, int site, long long spin_cycles);

/* ---- timing / introspection -------------------------------------------- */
/* Per-stage device timing with CUDA events on the context's stream.  While
 * enabled, hyb_step brackets every stage (wall, sweep, moments, sghost,
 * convert_ns, gsis, residual) with events and accumulates milliseconds and
 * launch counts; hyb_profile_read returns them in that order (7 entries). */
int hyb_profile_enable(hyb_ctx *ctx, int enable);
int hyb_profile_read(hyb_ctx *ctx, double *ms, long long *launches, int n);
/* Number of kernel launches issued by this context since creation. */
int hyb_launch_count(const hyb_ctx *ctx, long long *count);
/* Milliseconds of the last hyb_step measured with CUDA events on the
 * context's stream. */
int hyb_last_step_ms(const hyb_ctx *ctx, double *ms);
/* Raw CUDA stream handle (cudaStream_t) the context launches on. */
int hyb_stream(const hyb_ctx *ctx, void **stream);

/* ---- sweep launch-shape autotuner (no counterpart in the reference) ------ */
/* Times every admissible sweep shape (cells per thread, velocity groups per
 * CTA) for `reps` sweeps on the context's own distribution, restores f after
 * each candidate and keeps the fastest shape for later steps.  The chosen
 * shape is returned through cpt/vpb when they are not NULL. */
int hyb_autotune(hyb_ctx *ctx, int reps, int *cpt, int *vpb);

/* ---- batched instances (no counterpart in the reference; the reference
 * runs one case per process) ---------------------------------------------- */
/* n independent cases of any mesh / velocity-grid size on one device and one
 * precision.  One outer iteration of all instances is captured into one CUDA
 * graph; hyb_batch_step launches it once per iteration.  Instances of one
 * sweep launch shape share one launch per kernel (one graph branch per
 * shape group); batches the batched kernels do not cover (schemes other than
 * NND) get one branch per instance.  Either way each instance computes
 * exactly what a standalone context computes.  Every instance uses
 * HYB_SWEEP_REFERENCE without mass_pin (HYB_ERR_UNSUPPORTED otherwise).  res (n entries, may be NULL)
 * receives each instance's DETFP_res after the last iteration. */
typedef struct hyb_batch hyb_batch;
int hyb_batch_create(int n, const hyb_mesh *meshes, const hyb_vgrid *vgrids,
                     const hyb_params *params, hyb_batch **out);
int hyb_batch_destroy(hyb_batch *b);
const char *hyb_batch_last_error(const hyb_batch *b);
int hyb_batch_size(const hyb_batch *b, int *n);
/* The context of instance k (for state transfer and moments). */
int hyb_batch_instance(hyb_batch *b, int k, hyb_ctx **ctx);
int hyb_batch_init_maxwellian(hyb_batch *b, double rho, double u, double v, double t);
/* hyb_autotune on the first instance of each mesh and velocity-grid size,
 * whose shape the others of that size take; the captured graphs are rebuilt.
 * A shape set on one instance's context directly takes effect when the
 * graphs are next rebuilt (by this call). */
int hyb_batch_autotune(hyb_batch *b, int reps);
int hyb_batch_step(hyb_batch *b, int n_iter, hyb_residual *res);
/* Milliseconds of the last hyb_batch_step (CUDA events around the graph
 * launches) and kernel launches issued by the batch's graphs. */
int hyb_batch_last_step_ms(const hyb_batch *b, double *ms);
int hyb_batch_launch_count(const hyb_batch *b, long long *count);

/* ---- learned closure (no counterpart in the reference) ------------------ */
/* MLP 8 -> 64 -> 64 -> 64 -> 4, tanh hidden layers, 9,156 parameters; BF16
 * weights/activations on the tensor cores with FP32 accumulation, FP32 master
 * weights and Adam (beta 0.9 / 0.999, eps 1e-8).  Inputs (per face): log10
 * local Kn, rho, T, du/dn, dT/dn, NSF shear stress, NSF normal heat flux,
 * wall distance; outputs: the non-NSF shear stress t_xy, wall-normal
 * normal stress t_yy and heat-flux components q_x, q_y.  Parameter layout (FP32): W1[64][8]
 * b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[4][64] b4[4].  Inputs are
 * normalised as (x - in_mean) / in_std and outputs returned as
 * y_norm * out_std + out_mean; the loss is the mean squared error of the
 * normalised outputs.  Host arrays unless the name says _dev. */
typedef struct hyb_mlp hyb_mlp;
int hyb_mlp_create(int device, unsigned long long seed, hyb_mlp **out);
int hyb_mlp_destroy(hyb_mlp *m);
const char *hyb_mlp_last_error(const hyb_mlp *m);
int hyb_mlp_param_count(void);
int hyb_mlp_get_params(hyb_mlp *m, float *w);
/* Replaces the weights and resets the Adam state. */
int hyb_mlp_set_params(hyb_mlp *m, const float *w);
int hyb_mlp_set_norm(hyb_mlp *m, const float *in_mean, const float *in_std,
                     const float *out_mean, const float *out_std);
/* Training set x[n][8], y[n][4], kept on the device. */
int hyb_mlp_set_data(hyb_mlp *m, const float *x, const float *y, int n);
/* One epoch of Adam steps over minibatches perm[0:batch], perm[batch:2 batch],
 * ... of the training set; mean_loss = mean loss over the epoch. */
int hyb_mlp_train_epoch(hyb_mlp *m, const int *perm, int batch, float lr, float *mean_loss);
/* Gradient of the mean loss over x[n], y[n] at the current weights (no
 * update), in the parameter layout above. */
int hyb_mlp_grad(hyb_mlp *m, const float *x, const float *y, int n, float *grad, float *loss);
int hyb_mlp_predict(hyb_mlp *m, const float *x, int n, float *y);
/* Device-pointer inference on a caller stream (NULL: the network's own). */
int hyb_mlp_forward_dev(hyb_mlp *m, const float *x_dev, int n, float *y_dev, void *stream);
int hyb_mlp_last_ms(const hyb_mlp *m, double *ms);
int hyb_mlp_launch_count(const hyb_mlp *m, long long *count);

/* Use of the network by a context.  hyb_gsis_attach_mlp gives the synthetic
 * solve a network (not owned; NULL detaches).  hyb_gsis_warm_start runs the
 * learned warm start once: the NS equations closed with the network's HoT
 * (its predicted non-NSF t_xy, t_yy, q_x, q_y on the j-faces, in place of
 * the kinetic HoT, weighted by a local-Kn gate that ramps from 0 at
 * Kn/rho = 0.02 to 1 at 0.05: below that the NSF closure is the better
 * model and the network's error exceeds the HoT) are iterated from the
 * kinetic state towards a steady state on the band, then the moments and f
 * are corrected to that state as in the synthetic solve.  The kinetic GSIS
 * iteration that follows converges to the kinetic solution whatever the
 * network's error, and its residual measures that error.
 * hyb_closure_samples writes the network's inputs x[n][8] and
 * targets y[n][4] (the Convert_NS HoT t_xy, t_yy, q_x, q_y) of every j-face,
 * n = (nx-1)*ny, face (i, j) at (j-1)*(nx-1) + i-1, for the current kinetic
 * state: training data from the solver's own runs.  With x or y NULL it
 * only returns n. */
int hyb_gsis_attach_mlp(hyb_ctx *ctx, hyb_mlp *net);
int hyb_gsis_warm_start(hyb_ctx *ctx);
int hyb_closure_samples(hyb_ctx *ctx, float *x, float *y, int cap, int *n);

#ifdef __cplusplus
}
#endif
#endif /* HYB_DVM_H */
