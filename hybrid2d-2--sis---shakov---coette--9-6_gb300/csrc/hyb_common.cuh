// hyb_common.cuh -- shared device/host definitions of the GB300 kinetic solver.
//
// Device layout (one structured block, Couette-type boundaries):
//   The two mesh directions are renamed by their role in the fused LU-SGS
//   kernel: the SCAN axis "a" (contiguous in memory, the forward recurrence
//   along it is evaluated as a parallel affine scan) and the MARCH axis "b"
//   (walked sequentially by each CTA).  Which reference direction (i or j)
//   plays which role is chosen per context (scan_is_j).
//   f      : real[Nv][NRD][Nb][PA]      interior cells only, PA = Na rounded up
//                                        to a multiple of 32 (128-B rows)
//   fw_*   : real[Nv][NRD][n]           wall slot values (the reference's
//                                        ghost index -3 / n+3)
//   eqp    : real[Nb*PA/128][8][128]    Shakhov parameters, blocks of 128
//                                        cells (hyb_eqp_at)
//   S      : double[NSUM][(nx+3)(ny+3)] moments on the reference extents
//                                        (1-LAP:n+LAP-1), i fastest
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/hyb_dvm.h"

#define HYB_LAP 2
#define HYB_PI 3.1415926535897932

// REAL(4) literals of the reference widened to double
#define HYB_FLOOR_D ((double)1.0e-30f)
#define HYB_EPSWENO_D ((double)1.0e-15f)
#define HYB_CWENO1_D ((double)(1.0f / 3.0f))
#define HYB_CWENO2_D ((double)(2.0f / 3.0f))

namespace hyb {

// boundary kind of one end of an axis
enum AxisBC : int { AX_PERIODIC = 0, AX_WALL = 1 };

// geometry of the scan / march axes for the fused kernel
struct AxisGeom {
    int n;          // cells along the axis
    int bc_lo, bc_hi;  // AX_*
};

template <typename real>
struct KinArgs {
    real *f;              // [Nv][2][Nb][PA]
    real *rhs;            // optional RHS store (same layout) or nullptr
    int no_update;         // 1: compute (and store) the RHS only, f is left as is
    const real *fw_alo, *fw_ahi;   // wall slots at the scan-axis ends [Nv][2][Nb]
    const real *fw_blo, *fw_bhi;   // wall slots at the march-axis ends [Nv][2][PA]
    const real *eqp;      // hyb_eqp_at(cell, q), q: crt, u, v, invT, hT, cqx, cqy, cf
    const real *vol;      // [Nb*PA] cell volume
    // face normal * length, per face: scan faces [Nb][PA+1] (2 comps), march
    // faces [Nb+1][PA] (2 comps)
    const real *gA1, *gA2, *gB1, *gB2;
    const double *vx, *vy; // velocity nodes per v (v = iv + nvi*jv)
    int nvi, nv;
    int Na, Nb, PA;
    int bca_lo, bca_hi, bcb_lo, bcb_hi;
    int scheme;
    int scan_is_j;         // 1: scan axis = reference j
    real dt;
    int *err;              // device error word
    // mass_pin: the updated f is multiplied by *mscale (m0 / M of the state
    // the step starts from); nullptr: no scale
    const double *mscale;
    long long spin;        // limit of every bounded wait, SM clocks
    int stall_row;         // hyb_test_stall: this row's copy is never issued (0: none)
};

}  // namespace hyb

// ---- host-side context -------------------------------------------------------
struct hyb_ctx {
    int dev;
    cudaStream_t stream;
    cudaEvent_t ev0, ev1;
    int precision;
    int nx, ny, ncx, ncy, nvi, nvj, nv;
    int scan_is_j, Na, Nb, PA, cpt;         // cpt: largest scan cells per sweep thread
    int sw_cpt, sw_vpb, sw_minb;             // chosen sweep launch shape (0: default)
    int sw_generic;                          // 1: never the specialised FP32 NND sweep
    int bc[4];
    hyb_params prm;
    std::string last_error;
    long long launches;
    double last_ms;
    size_t real_size;

    // host copies of inputs
    std::vector<double> vi, vj, wi, wj;
    std::vector<double> wall_u[4], wall_v[4], wall_t[4];
    std::vector<double> xn, yn;            // nodes with ghosts (1-LAP:n+LAP)
    std::vector<double> vol, si, sj, ni1, ni2, nj1, nj2;  // (nx,ny)
    std::vector<double> x1, y1;            // (1-LAP:n+LAP-1)
    int uniform;                           // Cartesian uniform spacing

    // device buffers
    void *d_f, *d_rhs, *d_rhs_gsis, *d_fw[4], *d_eqp, *d_vol, *d_gA1, *d_gA2, *d_gB1, *d_gB2;
    double *d_vx, *d_vy, *d_w;             // per-velocity nodes and weights
    double *d_S;                           // [NSUM][(nx+3)(ny+3)]
    double *d_CF;                          // [(nx+3)(ny+3)]
    double *d_wall;                        // per wall face: u, v, t, normal
    double *d_x1, *d_y1;
    double *d_hot;                         // HoT + NSF arrays (see hyb_ns.cu)
    double *d_resid;                       // residual partials / result
    double *d_mpart;                       // moment partial sums [VS][10][Nb*PA]
    double *d_stage;                       // host-layout staging of downloads (first use)
    double *d_volc;                        // cell volumes, interior cells, i fastest (FP64)
    double *d_mass;                        // [0] total mass m0 at set-up, [1] scale m0 / M
    int *d_err;
    double *h_resid;                       // pinned
    int rhs_valid;
    // per-stage profiling (hyb_profile_enable)
    int prof_on;
    std::vector<cudaEvent_t> prof_ev;      // event pool, pairs per stage
    std::vector<int> prof_stage;           // stage of each recorded pair
    double prof_ms[8];
    long long prof_launch[8];
    double *h_wall;                        // pinned staging of wall data
    std::vector<double> wall_host;         // full wall table (u,v,t,normal)
    // GSIS
    hyb_gsis_params gsis;
    int gsis_last_inner;
    int gsis_skipped;                      // corrections skipped since hyb_gsis_configure
    long long spin_cycles;                 // limit of the device's bounded waits
    int in_batch;                          // owned by a hyb_batch (its graphs hold the buffers)
    int stall_site;                        // hyb_test_stall: planted wait of the next step (0: none)
    hyb_mlp *mlp;                          // learned closure for the warm start (not owned)
    int gsis_outer;                        // outer iterations since hyb_gsis_configure
    int warm_done;                         // the scheduled warm start has run (2: fell back)
    void *ns;                              // NS solver state (hyb_ns.cu)
};

#define HYB_CK(call)                                                              \
    do {                                                                          \
        cudaError_t _e = (call);                                                  \
        if (_e != cudaSuccess) {                                                  \
            ctx->last_error = std::string(#call) + ": " + cudaGetErrorString(_e); \
            return HYB_ERR_CUDA;                                                  \
        }                                                                         \
    } while (0)

// C2 index on the (1-LAP:n+LAP-1) extents
__host__ __device__ inline size_t hyb_c2(int nx, int i, int j) {
    return (size_t)(i + 1) + (size_t)(nx + 3) * (size_t)(j + 1);
}

// Shakhov parameter q (0..7) of sweep cell c = (b-1)*PA + (a-1).  Blocks of
// HYB_EQP_BLK consecutive cells hold their eight parameters together,
// [c/128][q][c%128]: a warp of the sweep (128 cells at 4 per thread) reads
// parameter q of its cells as one contiguous 512-byte span (FP32), and each
// thread finds its eight parameters at fixed offsets q * 128 from one
// pointer.  The array holds hyb_eqp_elems(Nb*PA) values.
#define HYB_EQP_BLK 128
__host__ __device__ inline size_t hyb_eqp_at(size_t c, int q) {
    return ((c >> 7) << 10) + ((size_t)q << 7) + (c & 127);
}
__host__ __device__ inline size_t hyb_eqp_elems(size_t ncell) {
    return (size_t)8 * ((ncell + HYB_EQP_BLK - 1) / HYB_EQP_BLK * HYB_EQP_BLK);
}

// launch helpers implemented in the .cu files
namespace hyb {
bool sweep_nnd_ok(const hyb_ctx *ctx, int cpt);
bool sweep_cpt_ok(const hyb_ctx *ctx, int cpt);
int sweep_nnd_signature(const hyb_ctx *ctx, int cpt);
int sweep_nnd_batch_f32(const KinArgs<float> *args, const int2 *work, int nwork, int PA, int vpb, int sig,
                        cudaStream_t s);
int launch_wall(hyb_ctx *ctx);
int launch_sweep(hyb_ctx *ctx, int store_rhs);
int sweep_prepare(hyb_ctx *ctx);
void sweep_shape(const hyb_ctx *ctx, int *cpt, int *vpb);
// batched launches over many contexts (hyb_batch): per-context arguments and
// work tables in device memory, one launch per launch shape
void sweep_args_f32(hyb_ctx *ctx, int store_rhs, KinArgs<float> *A);
void sweep_args_f64(hyb_ctx *ctx, int store_rhs, KinArgs<double> *A);
int sweep_batch_f32(const KinArgs<float> *args, const int2 *work, int nwork, int PA, int cpt, int vpb, bool uni,
                    int scheme, cudaStream_t s);
int sweep_batch_f64(const KinArgs<double> *args, const int2 *work, int nwork, int PA, int cpt, int vpb, bool uni,
                    int scheme, cudaStream_t s);
size_t sweep_smem_bytes(const hyb_ctx *ctx);
size_t wall_arg_bytes(int precision);
int wall_arg_fill(hyb_ctx *ctx, void *dst, size_t *smem);   // returns the wall face cells
int wall_batch_launch(int precision, const void *args, const int2 *work, int nclusters, size_t smem,
                      cudaStream_t s);
size_t mom_arg_bytes();
int mom_arg_fill(hyb_ctx *ctx, const void *f, void *dst, int *mc, int *tpv, size_t *smem, int *vs, int *lpc,
                 int *nfin);   // f: the distribution summed (nullptr: ctx->d_f)
int moments_part_batch_launch(int precision, int mc, int tpv, int nm, const void *args, const int4 *work, int nwork,
                              size_t smem, cudaStream_t s);
int residual_finish_batch_launch(int precision, const void *args, const int4 *work, double *const *parts, int nwork,
                                 cudaStream_t s);
size_t resfinal_arg_bytes();
void resfinal_arg_fill(hyb_ctx *ctx, void *dst, double **part);
int residual_final_batch_launch(const void *args, int n, double *copy, cudaStream_t s);
size_t cns_arg_bytes();
int cns_arg_fill(hyb_ctx *ctx, void *dst, int counts[7]);   // threads of the seven Convert_NS phases
int cns_batch_launch(const void *args, const int4 *work, int nwork, cudaStream_t s);
int moments_finish_batch_launch(int precision, const void *args, const int4 *work, int nwork, cudaStream_t s);
size_t sghost_arg_bytes();
int sghost_arg_fill(hyb_ctx *ctx, void *dst);   // returns the ghost threads
int sghost_batch_launch(const void *args, const int2 *work, const int *count, int nblocks, cudaStream_t s);
int gather_err_launch(int *const *errs, int *out, int n, cudaStream_t s);
int launch_moments(hyb_ctx *ctx);
int moments_slices(const hyb_ctx *ctx);
int launch_sghost(hyb_ctx *ctx);
int launch_s_host_layout(hyb_ctx *ctx, double *out);   // S as [(ny+3)(nx+3)][NSUM]
int launch_residual(hyb_ctx *ctx, hyb_residual *out);
int launch_rhs_moments(hyb_ctx *ctx, double *cellm);
int residual_blocks(const hyb_ctx *ctx);   // blocks of the residual partials
int launch_hoq(hyb_ctx *ctx, double *out);   // HOT_GKUA(1:6), HOQ_GKUA(1:3), [9][(nx+3)(ny+3)]
int launch_init_maxwellian(hyb_ctx *ctx, double rho, double u, double v, double t);
// total mass sum(vol rho) over the interior cells from S: mode 0 stores it as
// m0, mode 1 stores the mass_pin scale m0 / M
int launch_total_mass(hyb_ctx *ctx, int mode);
int launch_convert_ns(hyb_ctx *ctx);
int ns_create(hyb_ctx *ctx);
void ns_destroy(hyb_ctx *ctx);
int gsis_solve(hyb_ctx *ctx);
int gsis_warm_start(hyb_ctx *ctx);
}  // namespace hyb
