// hyb_sweep.cu -- launch-shape selection and dispatch of the fused kinetic
// sweep (kernel in hyb_sweep.cuh, instantiated per precision in
// hyb_sweep_f32.cu / hyb_sweep_f64.cu).
#include <cuda_runtime.h>

#include "hyb_common.cuh"

namespace hyb {

int sweep_launch_f32(hyb_ctx *ctx, const KinArgs<float> &A, int cpt, int vpb, bool launch);
int sweep_launch_f64(hyb_ctx *ctx, const KinArgs<double> &A, int cpt, int vpb, bool launch);
size_t sweep_group_bytes_f32(int PA, int tpv);
size_t sweep_group_bytes_f64(int PA, int tpv);

// Launch shape: cells per thread (cpt, dividing the context's layout chunk)
// and velocity groups per CTA (vpb, CTAs of at most 256 threads).  The
// autotuner sets ctx->sw_cpt / sw_vpb by timing; HYB_SWEEP_SHAPE="cpt,vpb,0"
// overrides them at context creation.
size_t sweep_nnd_group_bytes_f32(int PA, int tpv);

// the specialised FP32 NND sweep (hyb_sweep_nnd.cuh) covers this context at
// c cells per thread: FP32, uniform mesh, either order, NND, 4 cells per
// thread on the layout's 128-cell chunks
bool sweep_nnd_ok(const hyb_ctx *ctx, int c) {
    if (ctx->sw_generic || ctx->precision == HYB_PREC_FP64 || !ctx->uniform || ctx->prm.scheme != HYB_SCHEME_NND)
        return false;
    return c == 4 && ctx->cpt == 4 && ctx->Na % 4 == 0 && ctx->PA % HYB_EQP_BLK == 0;
}

// 0 when the context's sweep at c cells per thread is the generic one; else
// 8 | periodic scan axis | periodic march axis << 1 | scan axis = j << 2, the
// template signature of the specialised kernel (reference order)
int sweep_nnd_signature(const hyb_ctx *ctx, int c) {
    if (!sweep_nnd_ok(ctx, c) || ctx->prm.sweep_order != HYB_SWEEP_REFERENCE) return 0;
    const int fa_lo = ctx->scan_is_j ? 2 : 1, fb_lo = ctx->scan_is_j ? 1 : 2;
    const int pa = ctx->bc[fa_lo - 1] == HYB_BC_PERIODIC, pb = ctx->bc[fb_lo - 1] == HYB_BC_PERIODIC;
    return 8 | pa | (pb << 1) | ((ctx->scan_is_j != 0) << 2);
}

// cells per thread c admissible for the context's sweep
bool sweep_cpt_ok(const hyb_ctx *ctx, int c) {
    return (c == 1 || c == 2 || c == 4) && ctx->cpt % c == 0 && ctx->PA / c <= 256;
}

void sweep_shape(const hyb_ctx *ctx, int *cpt, int *vpb) {
    int c = ctx->sw_cpt > 0 ? ctx->sw_cpt : ctx->cpt;
    if (!sweep_cpt_ok(ctx, c)) c = ctx->cpt;
    int tpv = ctx->PA / c;
    // the specialised FP32 NND sweep runs best in CTAs of 128 threads (one
    // velocity per CTA at PA = 512: 1.67 against 1.84 ms on the 128x512 x 64^2
    // Couette case); the others default to 256
    int v = ctx->sw_vpb > 0 ? ctx->sw_vpb : (sweep_nnd_ok(ctx, c) ? 128 : 256) / tpv;
    if (v < 1) v = 1;
    while (v > 1 && tpv * v > 256) v--;
    *cpt = c;
    *vpb = v;
}

size_t sweep_smem_bytes(const hyb_ctx *ctx) {
    int cpt, vpb;
    sweep_shape(ctx, &cpt, &vpb);
    int tpv = ctx->PA / cpt;
    size_t g = ctx->precision == HYB_PREC_FP64 ? sweep_group_bytes_f64(ctx->PA, tpv)
               : sweep_nnd_ok(ctx, cpt)         ? sweep_nnd_group_bytes_f32(ctx->PA, tpv)
                                                : sweep_group_bytes_f32(ctx->PA, tpv);
    return g * vpb;
}

template <typename real>
static void fill_args(hyb_ctx *ctx, int store_rhs, KinArgs<real> &A) {
    A.f = (real *)ctx->d_f;
    A.rhs = store_rhs == 2 ? (real *)ctx->d_rhs_gsis : store_rhs ? (real *)ctx->d_rhs : nullptr;
    A.no_update = store_rhs == 2;
    A.fw_alo = A.fw_ahi = A.fw_blo = A.fw_bhi = nullptr;
    for (int face = 1; face <= 4; face++) {
        if (ctx->bc[face - 1] != HYB_BC_WALL) continue;
        int on_scan = ctx->scan_is_j ? (face == 2 || face == 4) : (face == 1 || face == 3);
        int hi = (face == 3 || face == 4);
        const real *p = (const real *)ctx->d_fw[face - 1];
        if (on_scan) (hi ? A.fw_ahi : A.fw_alo) = p;
        else (hi ? A.fw_bhi : A.fw_blo) = p;
    }
    A.eqp = (const real *)ctx->d_eqp;
    A.vol = (const real *)ctx->d_vol;
    A.gA1 = (const real *)ctx->d_gA1;
    A.gA2 = (const real *)ctx->d_gA2;
    A.gB1 = (const real *)ctx->d_gB1;
    A.gB2 = (const real *)ctx->d_gB2;
    A.vx = ctx->d_vx;
    A.vy = ctx->d_vy;
    A.nvi = ctx->nvi;
    A.nv = ctx->nv;
    A.Na = ctx->Na;
    A.Nb = ctx->Nb;
    A.PA = ctx->PA;
    int fa_lo = ctx->scan_is_j ? 2 : 1, fa_hi = ctx->scan_is_j ? 4 : 3;
    int fb_lo = ctx->scan_is_j ? 1 : 2, fb_hi = ctx->scan_is_j ? 3 : 4;
    A.bca_lo = ctx->bc[fa_lo - 1] == HYB_BC_WALL ? AX_WALL : AX_PERIODIC;
    A.bca_hi = ctx->bc[fa_hi - 1] == HYB_BC_WALL ? AX_WALL : AX_PERIODIC;
    A.bcb_lo = ctx->bc[fb_lo - 1] == HYB_BC_WALL ? AX_WALL : AX_PERIODIC;
    A.bcb_hi = ctx->bc[fb_hi - 1] == HYB_BC_WALL ? AX_WALL : AX_PERIODIC;
    A.scheme = ctx->prm.scheme;
    A.scan_is_j = ctx->scan_is_j;
    A.dt = (real)ctx->prm.dt;
    A.err = ctx->d_err;
    A.mscale = (ctx->prm.mass_pin && store_rhs != 2) ? ctx->d_mass + 1 : nullptr;
    A.spin = ctx->spin_cycles;
    A.stall_row = (ctx->stall_site == HYB_STALL_SWEEP_ROW && store_rhs != 2) ? (ctx->Nb < 3 ? ctx->Nb : 3) : 0;
}

static int sweep_dispatch(hyb_ctx *ctx, int store_rhs, bool launch) {
    int cpt, vpb;
    sweep_shape(ctx, &cpt, &vpb);
    if (ctx->precision == HYB_PREC_FP64) {
        KinArgs<double> A;
        fill_args<double>(ctx, store_rhs, A);
        return sweep_launch_f64(ctx, A, cpt, vpb, launch);
    }
    KinArgs<float> A;
    fill_args<float>(ctx, store_rhs, A);
    return sweep_launch_f32(ctx, A, cpt, vpb, launch);
}

void sweep_args_f32(hyb_ctx *ctx, int store_rhs, KinArgs<float> *A) { fill_args<float>(ctx, store_rhs, *A); }
void sweep_args_f64(hyb_ctx *ctx, int store_rhs, KinArgs<double> *A) { fill_args<double>(ctx, store_rhs, *A); }

// store_rhs: 0 no RHS store, 1 RHS to d_rhs with the update, 2 RHS only
// (to d_rhs_gsis, f unchanged).  With mass_pin the scale m0 / M of the
// current moments is formed first (the update multiplies by it).
int launch_sweep(hyb_ctx *ctx, int store_rhs) {
    if (ctx->prm.mass_pin && store_rhs != 2) {
        int rc = launch_total_mass(ctx, 1);
        if (rc) return rc;
    }
    return sweep_dispatch(ctx, store_rhs, true);
}

// sets the shared-memory attribute of the kernel the current shape selects
int sweep_prepare(hyb_ctx *ctx) { return sweep_dispatch(ctx, 0, false); }

}  // namespace hyb
