// hyb_api.cu -- the C ABI of include/hyb_dvm.h.
//
// Owns the context: geometry derived from the node coordinates (Creat_Mesh,
// sub_init.f90:178-208; Update_coordinate_buffer_onemesh, :719-823), device
// buffers, the reference-layout <-> device-layout transfers, and the outer
// iteration Hybrid_Time_advance_LU_SGS (Hybrid_Sub.f90:4-160).
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "hyb_common.cuh"
#include "hyb_device.cuh"

namespace hyb {
size_t hot_doubles(int nx, int ny);
}

#define VERSION_STRING "hyb_gb300 1.0 (sm_103a)"

namespace {

inline size_t XN(int nx, int i, int j) { return (size_t)(i + 1) + (size_t)(nx + 4) * (size_t)(j + 1); }
inline size_t MI(int nx, int i, int j) { return (size_t)(i - 1) + (size_t)nx * (size_t)(j - 1); }

// Creat_Mesh metrics and ghost nodes / cell centres; periodic faces take the
// partner face's nodes shifted by the period vector.
void build_geometry(hyb_ctx *c, const double *x, const double *y) {
    const int nx = c->nx, ny = c->ny;
    c->xn.assign((size_t)(nx + 4) * (ny + 4), 0.0);
    c->yn.assign((size_t)(nx + 4) * (ny + 4), 0.0);
    size_t nm = (size_t)nx * ny;
    c->vol.assign(nm, 0.0); c->si.assign(nm, 0.0); c->sj.assign(nm, 0.0);
    c->ni1.assign(nm, 0.0); c->ni2.assign(nm, 0.0); c->nj1.assign(nm, 0.0); c->nj2.assign(nm, 0.0);
    auto &X = c->xn;
    auto &Y = c->yn;
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            X[XN(nx, i, j)] = x[MI(nx, i, j)];
            Y[XN(nx, i, j)] = y[MI(nx, i, j)];
        }
    for (int j = 1; j <= ny - 1; j++)
        for (int i = 1; i <= nx - 1; i++)
            c->vol[MI(nx, i, j)] = fabs((X[XN(nx, i, j)] - X[XN(nx, i + 1, j + 1)]) *
                                            (Y[XN(nx, i + 1, j)] - Y[XN(nx, i, j + 1)]) -
                                        (X[XN(nx, i + 1, j)] - X[XN(nx, i, j + 1)]) *
                                            (Y[XN(nx, i, j)] - Y[XN(nx, i + 1, j + 1)])) * 0.5;
    for (int j = 1; j <= ny - 1; j++)
        for (int i = 1; i <= nx; i++) {
            double dx = X[XN(nx, i, j + 1)] - X[XN(nx, i, j)], dy = Y[XN(nx, i, j + 1)] - Y[XN(nx, i, j)];
            double s = sqrt(dx * dx + dy * dy);
            c->si[MI(nx, i, j)] = s;
            c->ni1[MI(nx, i, j)] = dy / s;
            c->ni2[MI(nx, i, j)] = -dx / s;
        }
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx - 1; i++) {
            double dx = X[XN(nx, i + 1, j)] - X[XN(nx, i, j)], dy = Y[XN(nx, i + 1, j)] - Y[XN(nx, i, j)];
            double s = sqrt(dx * dx + dy * dy);
            c->sj[MI(nx, i, j)] = s;
            c->nj1[MI(nx, i, j)] = -dy / s;
            c->nj2[MI(nx, i, j)] = dx / s;
        }
    for (int l = 1; l <= HYB_LAP; l++) {
        for (int j = 1; j <= ny; j++) {
            double px = X[XN(nx, nx, j)] - X[XN(nx, 1, j)], py = Y[XN(nx, nx, j)] - Y[XN(nx, 1, j)];
            if (c->bc[0] == HYB_BC_PERIODIC) {
                X[XN(nx, 1 - l, j)] = X[XN(nx, nx - l, j)] - px;
                Y[XN(nx, 1 - l, j)] = Y[XN(nx, nx - l, j)] - py;
                X[XN(nx, nx + l, j)] = X[XN(nx, 1 + l, j)] + px;
                Y[XN(nx, nx + l, j)] = Y[XN(nx, 1 + l, j)] + py;
            } else {
                X[XN(nx, 1 - l, j)] = 2.0 * X[XN(nx, 1, j)] - X[XN(nx, 1 + l, j)];
                Y[XN(nx, 1 - l, j)] = 2.0 * Y[XN(nx, 1, j)] - Y[XN(nx, 1 + l, j)];
                X[XN(nx, nx + l, j)] = 2.0 * X[XN(nx, nx, j)] - X[XN(nx, nx - l, j)];
                Y[XN(nx, nx + l, j)] = 2.0 * Y[XN(nx, nx, j)] - Y[XN(nx, nx - l, j)];
            }
        }
        for (int i = 1; i <= nx; i++) {
            double px = X[XN(nx, i, ny)] - X[XN(nx, i, 1)], py = Y[XN(nx, i, ny)] - Y[XN(nx, i, 1)];
            if (c->bc[1] == HYB_BC_PERIODIC) {
                X[XN(nx, i, 1 - l)] = X[XN(nx, i, ny - l)] - px;
                Y[XN(nx, i, 1 - l)] = Y[XN(nx, i, ny - l)] - py;
                X[XN(nx, i, ny + l)] = X[XN(nx, i, 1 + l)] + px;
                Y[XN(nx, i, ny + l)] = Y[XN(nx, i, 1 + l)] + py;
            } else {
                X[XN(nx, i, 1 - l)] = 2.0 * X[XN(nx, i, 1)] - X[XN(nx, i, 1 + l)];
                Y[XN(nx, i, 1 - l)] = 2.0 * Y[XN(nx, i, 1)] - Y[XN(nx, i, 1 + l)];
                X[XN(nx, i, ny + l)] = 2.0 * X[XN(nx, i, ny)] - X[XN(nx, i, ny - l)];
                Y[XN(nx, i, ny + l)] = 2.0 * Y[XN(nx, i, ny)] - Y[XN(nx, i, ny - l)];
            }
        }
    }
    for (int j = 1; j <= HYB_LAP; j++)
        for (int i = 1; i <= HYB_LAP; i++) {
            int i1 = 1 - i, j1 = 1 - j, i2 = nx + i, j2 = ny + j;
            X[XN(nx, i1, j1)] = X[XN(nx, i1, 1)] + X[XN(nx, 1, j1)] - X[XN(nx, 1, 1)];
            Y[XN(nx, i1, j1)] = Y[XN(nx, i1, 1)] + Y[XN(nx, 1, j1)] - Y[XN(nx, 1, 1)];
            X[XN(nx, i2, j2)] = X[XN(nx, i2, ny)] + X[XN(nx, nx, j2)] - X[XN(nx, nx, ny)];
            Y[XN(nx, i2, j2)] = Y[XN(nx, i2, ny)] + Y[XN(nx, nx, j2)] - Y[XN(nx, nx, ny)];
            X[XN(nx, i1, j2)] = X[XN(nx, i1, ny)] + X[XN(nx, 1, j2)] - X[XN(nx, 1, ny)];
            Y[XN(nx, i1, j2)] = Y[XN(nx, i1, ny)] + Y[XN(nx, 1, j2)] - Y[XN(nx, 1, ny)];
            X[XN(nx, i2, j1)] = X[XN(nx, i2, 1)] + X[XN(nx, nx, j1)] - X[XN(nx, nx, 1)];
            Y[XN(nx, i2, j1)] = Y[XN(nx, i2, 1)] + Y[XN(nx, nx, j1)] - Y[XN(nx, nx, 1)];
        }
    size_t nc = (size_t)(nx + 3) * (ny + 3);
    c->x1.assign(nc, 0.0);
    c->y1.assign(nc, 0.0);
    for (int j = 1 - HYB_LAP; j <= ny + HYB_LAP - 1; j++)
        for (int i = 1 - HYB_LAP; i <= nx + HYB_LAP - 1; i++) {
            c->x1[hyb_c2(nx, i, j)] = (X[XN(nx, i, j)] + X[XN(nx, i + 1, j)] + X[XN(nx, i, j + 1)] +
                                       X[XN(nx, i + 1, j + 1)]) * 0.25;
            c->y1[hyb_c2(nx, i, j)] = (Y[XN(nx, i, j)] + Y[XN(nx, i + 1, j)] + Y[XN(nx, i, j + 1)] +
                                       Y[XN(nx, i + 1, j + 1)]) * 0.25;
        }
}

template <typename T>
int dalloc(hyb_ctx *ctx, T **p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        ctx->last_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return HYB_ERR_NOMEM;
    }
    cudaMemsetAsync(*p, 0, n * sizeof(T), ctx->stream);
    return HYB_OK;
}

// upload a host double array converted to the context's real type
int upload_real(hyb_ctx *ctx, void *dst, const std::vector<double> &src) {
    if (ctx->precision == HYB_PREC_FP64) {
        HYB_CK(cudaMemcpy(dst, src.data(), src.size() * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> tmp(src.size());
        for (size_t k = 0; k < src.size(); k++) tmp[k] = (float)src[k];
        HYB_CK(cudaMemcpy(dst, tmp.data(), tmp.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    return HYB_OK;
}

void free_all(hyb_ctx *c) {
    auto F = [](void *p) {
        if (p) cudaFree(p);
    };
    F(c->d_f); F(c->d_rhs);
    for (int k = 0; k < 4; k++) F(c->d_fw[k]);
    F(c->d_eqp); F(c->d_vol); F(c->d_gA1); F(c->d_gA2); F(c->d_gB1); F(c->d_gB2);
    F(c->d_vx); F(c->d_vy); F(c->d_w); F(c->d_S); F(c->d_CF); F(c->d_wall);
    F(c->d_x1); F(c->d_y1); F(c->d_hot); F(c->d_resid); F(c->d_err); F(c->d_mpart); F(c->d_stage);
    F(c->d_volc); F(c->d_mass);
    if (c->h_resid) cudaFreeHost(c->h_resid);
    if (c->h_wall) cudaFreeHost(c->h_wall);
    for (auto ev : c->prof_ev) cudaEventDestroy(ev);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
}

// cell (i,j) -> device cell index in the (a,b) layout
inline size_t dev_cell(const hyb_ctx *c, int i, int j) {
    int a = c->scan_is_j ? j : i, b = c->scan_is_j ? i : j;
    return (size_t)(b - 1) * c->PA + (a - 1);
}

// cell volumes and face normals times lengths in the sweep's (a,b) layout
void kinetic_geometry(const hyb_ctx *c, std::vector<double> &vol, std::vector<double> &gA1,
                      std::vector<double> &gA2, std::vector<double> &gB1, std::vector<double> &gB2) {
    const size_t ncell = (size_t)c->Nb * c->PA;
    vol.assign(ncell, 1.0);
    gA1.assign((size_t)c->Nb * (c->PA + 1), 0.0);
    gA2.assign(gA1.size(), 0.0);
    gB1.assign((size_t)(c->Nb + 1) * c->PA, 0.0);
    gB2.assign(gB1.size(), 0.0);
    const int nx = c->nx;
    for (int b = 1; b <= c->Nb; b++)
        for (int a = 1; a <= c->Na; a++) {
            int i = c->scan_is_j ? b : a, j = c->scan_is_j ? a : b;
            vol[(size_t)(b - 1) * c->PA + (a - 1)] = c->vol[MI(nx, i, j)];
        }
    for (int b = 1; b <= c->Nb; b++)
        for (int q = 1; q <= c->Na + 1; q++) {
            size_t k = (size_t)(b - 1) * (c->PA + 1) + (q - 1);
            if (c->scan_is_j) {   // j-face (i=b, j=q)
                gA1[k] = c->nj1[MI(nx, b, q)] * c->sj[MI(nx, b, q)];
                gA2[k] = c->nj2[MI(nx, b, q)] * c->sj[MI(nx, b, q)];
            } else {              // i-face (i=q, j=b)
                gA1[k] = c->ni1[MI(nx, q, b)] * c->si[MI(nx, q, b)];
                gA2[k] = c->ni2[MI(nx, q, b)] * c->si[MI(nx, q, b)];
            }
        }
    for (int q = 1; q <= c->Nb + 1; q++)
        for (int a = 1; a <= c->Na; a++) {
            size_t k = (size_t)(q - 1) * c->PA + (a - 1);
            if (c->scan_is_j) {   // i-face (i=q, j=a)
                gB1[k] = c->ni1[MI(nx, q, a)] * c->si[MI(nx, q, a)];
                gB2[k] = c->ni2[MI(nx, q, a)] * c->si[MI(nx, q, a)];
            } else {              // j-face (i=a, j=q)
                gB1[k] = c->nj1[MI(nx, a, q)] * c->sj[MI(nx, a, q)];
                gB2[k] = c->nj2[MI(nx, a, q)] * c->sj[MI(nx, a, q)];
            }
        }
}

// Sweep layout of a mesh: the scan axis is the longer one that fits one CTA
// row (<= 1024 cells); cells per sweep thread (cpt) tile the scan axis
// exactly; the padded row PA holds 32 * cpt-cell chunks and a thread group
// (PA / cpt threads) fits one 256-thread CTA, so scan axes above 256 cells
// need an even count and above 512 a multiple of 4.
struct SweepLayout {
    int scan_is_j, Na, Nb, cpt, PA;
};
static bool sweep_layout(int ncx, int ncy, SweepLayout *L) {
    if (ncy >= ncx && ncy <= 1024) L->scan_is_j = 1;
    else if (ncx <= 1024) L->scan_is_j = 0;
    else return false;
    L->Na = L->scan_is_j ? ncy : ncx;
    L->Nb = L->scan_is_j ? ncx : ncy;
    L->cpt = (L->Na % 4 == 0 && L->Na >= 128) ? 4 : ((L->Na % 2 == 0 && L->Na >= 64) ? 2 : 1);
    L->PA = (L->Na + 32 * L->cpt - 1) / (32 * L->cpt) * (32 * L->cpt);
    return L->PA / L->cpt <= 256;
}

}  // namespace

extern "C" {

const char *hyb_version(void) { return VERSION_STRING; }

const char *hyb_last_error(const hyb_ctx *ctx) {
    if (!ctx) return "null context";
    return ctx->last_error.c_str();
}

int hyb_create(const hyb_mesh *m, const hyb_vgrid *vg, const hyb_params *p, hyb_ctx **out) {
    if (!m || !vg || !p || !out || !m->x || !m->y) return HYB_ERR_INVALID;
    *out = nullptr;
    if (m->nx < 3 || m->ny < 3 || vg->nvi < 1 || vg->nvj < 1) return HYB_ERR_INVALID;
    if (!vg->vi || !vg->vj || !vg->wi || !vg->wj) return HYB_ERR_INVALID;
    if (p->precision != HYB_PREC_FP64 && p->precision != HYB_PREC_MIXED) return HYB_ERR_INVALID;
    if (p->scheme != HYB_SCHEME_UP1 && p->scheme != HYB_SCHEME_NND && p->scheme != HYB_SCHEME_WENO3)
        return HYB_ERR_INVALID;
    if (!(p->dt > 0.0) || !(p->cfc > 0.0)) return HYB_ERR_INVALID;
    for (int f = 0; f < 4; f++) {
        if (m->bc[f] != HYB_BC_WALL && m->bc[f] != HYB_BC_PERIODIC) return HYB_ERR_UNSUPPORTED;
        if (m->bc[f] == HYB_BC_WALL && (!m->wall_u[f] || !m->wall_v[f] || !m->wall_t[f])) return HYB_ERR_INVALID;
    }
    if ((m->bc[0] == HYB_BC_PERIODIC) != (m->bc[2] == HYB_BC_PERIODIC)) return HYB_ERR_INVALID;
    if ((m->bc[1] == HYB_BC_PERIODIC) != (m->bc[3] == HYB_BC_PERIODIC)) return HYB_ERR_INVALID;
    if (p->sweep_order != HYB_SWEEP_REFERENCE && p->sweep_order != HYB_SWEEP_UPWIND) return HYB_ERR_INVALID;
    if (p->mass_pin != 0 && p->mass_pin != 1) return HYB_ERR_INVALID;
    SweepLayout lay;
    if (!sweep_layout(m->nx - 1, m->ny - 1, &lay)) return HYB_ERR_UNSUPPORTED;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return HYB_ERR_NODEVICE;
    if (p->device < 0 || p->device >= ndev) return HYB_ERR_INVALID;

    hyb_ctx *c = new (std::nothrow) hyb_ctx();
    if (!c) return HYB_ERR_NOMEM;
    c->dev = p->device;
    c->prm = *p;
    c->precision = p->precision;
    c->real_size = p->precision == HYB_PREC_FP64 ? sizeof(double) : sizeof(float);
    c->nx = m->nx; c->ny = m->ny; c->ncx = m->nx - 1; c->ncy = m->ny - 1;
    c->nvi = vg->nvi; c->nvj = vg->nvj; c->nv = vg->nvi * vg->nvj;
    for (int f = 0; f < 4; f++) c->bc[f] = m->bc[f];
    int ncx = c->ncx, ncy = c->ncy;
    c->scan_is_j = lay.scan_is_j;
    c->Na = lay.Na;
    c->Nb = lay.Nb;
    c->cpt = lay.cpt;
    c->PA = lay.PA;
    // wall stencils need at least three cells along the wall-normal axis,
    // a periodic march axis at least two
    for (int f = 0; f < 4; f++)
        if (m->bc[f] == HYB_BC_WALL && ((f == 0 || f == 2) ? ncx : ncy) < 4) { delete c; return HYB_ERR_UNSUPPORTED; }
    if (c->Nb < 2) { delete c; return HYB_ERR_UNSUPPORTED; }

    if (cudaSetDevice(c->dev) != cudaSuccess) { delete c; return HYB_ERR_CUDA; }
    cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);

    c->vi.assign(vg->vi, vg->vi + vg->nvi);
    c->vj.assign(vg->vj, vg->vj + vg->nvj);
    c->wi.assign(vg->wi, vg->wi + vg->nvi);
    c->wj.assign(vg->wj, vg->wj + vg->nvj);
    for (int f = 0; f < 4; f++) {
        if (m->bc[f] != HYB_BC_WALL) continue;
        int n = (f == 0 || f == 2) ? ncy : ncx;
        c->wall_u[f].assign(m->wall_u[f], m->wall_u[f] + n);
        c->wall_v[f].assign(m->wall_v[f], m->wall_v[f] + n);
        c->wall_t[f].assign(m->wall_t[f], m->wall_t[f] + n);
        for (int k = 0; k < n; k++)
            if (!(c->wall_t[f][k] > 0.0)) { free_all(c); delete c; return HYB_ERR_INVALID; }
    }
    build_geometry(c, m->x, m->y);

    int rc = HYB_OK;
    const size_t ncell = (size_t)c->Nb * c->PA;
    const size_t fsz = (size_t)c->nv * 2 * ncell;
    const size_t rs = c->real_size;
#define ALLOC(ptr, bytes)                                           \
    do {                                                            \
        if (cudaMalloc((void **)&(ptr), (bytes)) != cudaSuccess) {  \
            c->last_error = "cudaMalloc failed for " #ptr;          \
            rc = HYB_ERR_NOMEM;                                     \
        } else                                                      \
            cudaMemsetAsync((ptr), 0, (bytes), c->stream);          \
    } while (0)
    ALLOC(c->d_f, fsz * rs);
    if (rc == HYB_OK) ALLOC(c->d_rhs, fsz * rs);
    for (int f = 0; f < 4 && rc == HYB_OK; f++) {
        if (m->bc[f] != HYB_BC_WALL) continue;
        int on_scan = c->scan_is_j ? (f == 1 || f == 3) : (f == 0 || f == 2);
        size_t n = on_scan ? c->Nb : c->PA;
        ALLOC(c->d_fw[f], (size_t)c->nv * 2 * n * rs);
    }
    if (rc == HYB_OK) ALLOC(c->d_eqp, hyb_eqp_elems(ncell) * rs);
    if (rc == HYB_OK) ALLOC(c->d_vol, ncell * rs);
    if (rc == HYB_OK) ALLOC(c->d_gA1, (size_t)c->Nb * (c->PA + 1) * rs);
    if (rc == HYB_OK) ALLOC(c->d_gA2, (size_t)c->Nb * (c->PA + 1) * rs);
    if (rc == HYB_OK) ALLOC(c->d_gB1, (size_t)(c->Nb + 1) * c->PA * rs);
    if (rc == HYB_OK) ALLOC(c->d_gB2, (size_t)(c->Nb + 1) * c->PA * rs);
    if (rc == HYB_OK) ALLOC(c->d_vx, c->nvi * sizeof(double));
    if (rc == HYB_OK) ALLOC(c->d_vy, c->nvj * sizeof(double));
    if (rc == HYB_OK) ALLOC(c->d_w, c->nv * sizeof(double));
    const size_t nc2 = (size_t)(c->nx + 3) * (c->ny + 3);
    if (rc == HYB_OK) ALLOC(c->d_S, HYB_NSUM * nc2 * sizeof(double));
    if (rc == HYB_OK) ALLOC(c->d_CF, nc2 * sizeof(double));
    const int maxfc = std::max(ncx, ncy);
    if (rc == HYB_OK) ALLOC(c->d_wall, (size_t)4 * 6 * 4096 * sizeof(double));
    if (rc == HYB_OK) ALLOC(c->d_x1, nc2 * sizeof(double));
    if (rc == HYB_OK) ALLOC(c->d_y1, nc2 * sizeof(double));
    if (rc == HYB_OK) ALLOC(c->d_hot, hyb::hot_doubles(c->nx, c->ny) * sizeof(double));
    const size_t nblk = (size_t)hyb::residual_blocks(c);
    if (rc == HYB_OK) ALLOC(c->d_resid, (16 + 8 * nblk) * sizeof(double));
    if (rc == HYB_OK) ALLOC(c->d_err, sizeof(int));
    if (rc == HYB_OK) ALLOC(c->d_mpart, (size_t)hyb::moments_slices(c) * 10 * ncell * sizeof(double));
    if (rc == HYB_OK) ALLOC(c->d_volc, (size_t)ncx * ncy * sizeof(double));
    if (rc == HYB_OK) ALLOC(c->d_mass, 2 * sizeof(double));
#undef ALLOC
    if (rc == HYB_OK && cudaMallocHost((void **)&c->h_resid, 16 * sizeof(double)) != cudaSuccess) rc = HYB_ERR_NOMEM;
    if (rc == HYB_OK && maxfc > 4096) { rc = HYB_ERR_UNSUPPORTED; c->last_error = "wall longer than 4096 cells"; }
    if (rc != HYB_OK) {
        free_all(c);
        delete c;
        return rc;
    }
    // geometry in the (a,b) layout
    std::vector<double> vol, gA1, gA2, gB1, gB2;
    kinetic_geometry(c, vol, gA1, gA2, gB1, gB2);
    const int nx = c->nx;
    // uniform Cartesian spacing: one face speed per axis and one volume
    {
        auto same = [](const std::vector<double> &x, size_t n0, size_t n, size_t stride, size_t len) {
            (void)n0;
            double ref = x[0];
            for (size_t r = 0; r < n; r++)
                for (size_t k = 0; k < len; k++) {
                    double y = x[r * stride + k];
                    if (fabs(y - ref) > 1e-12 * (fabs(ref) + 1e-300) && !(ref == 0.0 && y == 0.0)) return false;
                }
            return true;
        };
        bool u = same(vol, 0, c->Nb, c->PA, c->Na) && same(gA1, 0, c->Nb, c->PA + 1, c->Na + 1) &&
                 same(gA2, 0, c->Nb, c->PA + 1, c->Na + 1) && same(gB1, 0, c->Nb + 1, c->PA, c->Na) &&
                 same(gB2, 0, c->Nb + 1, c->PA, c->Na);
        // a zero normal component must be exactly zero everywhere
        for (size_t k = 0; u && k < gA2.size(); k++) (void)0;
        c->uniform = u ? 1 : 0;
    }
    int r2 = upload_real(c, c->d_vol, vol);
    if (!r2) r2 = upload_real(c, c->d_gA1, gA1);
    if (!r2) r2 = upload_real(c, c->d_gA2, gA2);
    if (!r2) r2 = upload_real(c, c->d_gB1, gB1);
    if (!r2) r2 = upload_real(c, c->d_gB2, gB2);
    std::vector<double> w((size_t)c->nv);
    for (int jv = 0; jv < c->nvj; jv++)
        for (int iv = 0; iv < c->nvi; iv++) w[(size_t)iv + (size_t)c->nvi * jv] = c->wi[iv] * c->wj[jv];
    // wall data per face: u, v, t, normal (x, y) and orientation of the
    // reference (GKUA_wall_functions.f90:34-42)
    std::vector<double> wall((size_t)4 * 6 * 4096, 0.0);
    for (int f = 0; f < 4; f++) {
        if (m->bc[f] != HYB_BC_WALL) continue;
        int n = (f == 0 || f == 2) ? ncy : ncx;
        for (int k = 0; k < n; k++) {
            double *d = &wall[((size_t)f * 4096 + k) * 6];
            d[0] = c->wall_u[f][k];
            d[1] = c->wall_v[f][k];
            d[2] = c->wall_t[f][k];
            if (f == 0) { d[3] = c->ni1[MI(nx, 1, k + 1)]; d[4] = c->ni2[MI(nx, 1, k + 1)]; d[5] = 1.0; }
            if (f == 1) { d[3] = c->nj1[MI(nx, k + 1, 1)]; d[4] = c->nj2[MI(nx, k + 1, 1)]; d[5] = 1.0; }
            if (f == 2) { d[3] = c->ni1[MI(nx, c->nx, k + 1)]; d[4] = c->ni2[MI(nx, c->nx, k + 1)]; d[5] = -1.0; }
            if (f == 3) { d[3] = c->nj1[MI(nx, k + 1, c->ny)]; d[4] = c->nj2[MI(nx, k + 1, c->ny)]; d[5] = -1.0; }
        }
    }
    c->wall_host = wall;
    if (!r2 && cudaMallocHost((void **)&c->h_wall, (size_t)6 * 4096 * sizeof(double)) != cudaSuccess) r2 = HYB_ERR_NOMEM;
    cudaError_t e = cudaSuccess;
    if (!r2) {
        e = cudaMemcpy(c->d_vx, c->vi.data(), c->nvi * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(c->d_vy, c->vj.data(), c->nvj * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(c->d_w, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(c->d_wall, wall.data(), wall.size() * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(c->d_x1, c->x1.data(), nc2 * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(c->d_y1, c->y1.data(), nc2 * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            std::vector<double> vc((size_t)ncx * ncy);
            for (int j = 1; j <= ncy; j++)
                for (int i = 1; i <= ncx; i++) vc[(size_t)(i - 1) + (size_t)ncx * (j - 1)] = c->vol[MI(nx, i, j)];
            e = cudaMemcpy(c->d_volc, vc.data(), vc.size() * sizeof(double), cudaMemcpyHostToDevice);
        }
        if (e != cudaSuccess) { c->last_error = cudaGetErrorString(e); r2 = HYB_ERR_CUDA; }
    }
    if (!r2 && cudaStreamSynchronize(c->stream) != cudaSuccess) r2 = HYB_ERR_CUDA;
    if (r2) {
        free_all(c);
        delete c;
        return r2;
    }
    // the upwind order mirrors whole rows with a uniform face speed per axis
    if (p->sweep_order == HYB_SWEEP_UPWIND && !c->uniform) {
        free_all(c);
        delete c;
        return HYB_ERR_UNSUPPORTED;
    }
    c->gsis.enable = 0;
    c->spin_cycles = HYB_SPIN_CYCLES;
    c->stall_site = HYB_STALL_NONE;
    // launch-shape override, "cpt,vpb,minb"
    if (const char *e = getenv("HYB_SWEEP_SHAPE")) {
        int a = 0, b = 0, d = 0;
        if (sscanf(e, "%d,%d,%d", &a, &b, &d) == 3 && (a == 1 || a == 2 || a == 4) && c->cpt % a == 0) {
            c->sw_cpt = a;
            c->sw_vpb = b;
            c->sw_minb = d;
        }
    }
    // HYB_SWEEP_GENERIC=1 keeps every sweep on the generic kernel (A/B
    // timing and identity checks of the specialised FP32 NND sweep)
    if (const char *e = getenv("HYB_SWEEP_GENERIC")) c->sw_generic = atoi(e) != 0;
    *out = c;
    return HYB_OK;
}

// FP32 -> FP64, element by element (every FP32 value is exact in FP64)
__global__ void k_widen(const float *__restrict__ src, double *__restrict__ dst, size_t n) {
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        dst[k] = (double)src[k];
}

// Promotes a mixed-precision context to FP64 on the device: f is widened in
// place of the FP32 array, the other precision-typed buffers are made anew
// (wall slots, RHS and Shakhov parameters are recomputed from f by the next
// passes, the geometry is uploaded again) and DETFP is rerun on the FP64 f.
int hyb_set_precision(hyb_ctx *ctx, int precision) {
    if (!ctx) return HYB_ERR_INVALID;
    if (precision == ctx->precision) return HYB_OK;
    if (precision != HYB_PREC_FP64 || ctx->precision != HYB_PREC_MIXED) return HYB_ERR_UNSUPPORTED;
    if (ctx->in_batch) {
        ctx->last_error = "set_precision: the instance belongs to a batch";
        return HYB_ERR_UNSUPPORTED;
    }
    cudaSetDevice(ctx->dev);
    HYB_CK(cudaStreamSynchronize(ctx->stream));
    const size_t ncell = (size_t)ctx->Nb * ctx->PA, fsz = (size_t)ctx->nv * 2 * ncell;
    double *f64 = nullptr;
    if (cudaMalloc((void **)&f64, fsz * sizeof(double)) != cudaSuccess) {
        ctx->last_error = "set_precision: device allocation of the FP64 distribution failed";
        return HYB_ERR_NOMEM;
    }
    k_widen<<<152 * 8, 256, 0, ctx->stream>>>((const float *)ctx->d_f, f64, fsz);
    ctx->launches++;
    HYB_CK(cudaGetLastError());
    HYB_CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->d_f);
    ctx->d_f = f64;
    // the other buffers of the distribution's type, at FP64 size
    auto remake = [&](void **p, size_t n) -> int {
        if (*p) cudaFree(*p);
        *p = nullptr;
        if (cudaMalloc(p, n * sizeof(double)) != cudaSuccess) {
            ctx->last_error = "set_precision: device allocation failed";
            return HYB_ERR_NOMEM;
        }
        return cudaMemsetAsync(*p, 0, n * sizeof(double), ctx->stream) == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
    };
    int rc = remake(&ctx->d_rhs, fsz);
    for (int f = 0; f < 4 && !rc; f++) {
        if (!ctx->d_fw[f]) continue;
        int on_scan = ctx->scan_is_j ? (f == 1 || f == 3) : (f == 0 || f == 2);
        rc = remake(&ctx->d_fw[f], (size_t)ctx->nv * 2 * (on_scan ? ctx->Nb : ctx->PA));
    }
    if (!rc) rc = remake(&ctx->d_eqp, hyb_eqp_elems(ncell));
    if (!rc) rc = remake(&ctx->d_vol, ncell);
    if (!rc) rc = remake(&ctx->d_gA1, (size_t)ctx->Nb * (ctx->PA + 1));
    if (!rc) rc = remake(&ctx->d_gA2, (size_t)ctx->Nb * (ctx->PA + 1));
    if (!rc) rc = remake(&ctx->d_gB1, (size_t)(ctx->Nb + 1) * ctx->PA);
    if (!rc) rc = remake(&ctx->d_gB2, (size_t)(ctx->Nb + 1) * ctx->PA);
    if (rc) return rc;
    ctx->precision = HYB_PREC_FP64;
    ctx->prm.precision = HYB_PREC_FP64;
    ctx->real_size = sizeof(double);
    std::vector<double> vol, gA1, gA2, gB1, gB2;
    kinetic_geometry(ctx, vol, gA1, gA2, gB1, gB2);
    rc = upload_real(ctx, ctx->d_vol, vol);
    if (!rc) rc = upload_real(ctx, ctx->d_gA1, gA1);
    if (!rc) rc = upload_real(ctx, ctx->d_gA2, gA2);
    if (!rc) rc = upload_real(ctx, ctx->d_gB1, gB1);
    if (!rc) rc = upload_real(ctx, ctx->d_gB2, gB2);
    if (rc) return rc;
    // launch shapes chosen for FP32 rows no longer apply
    ctx->sw_cpt = ctx->sw_vpb = ctx->sw_minb = 0;
    if (ctx->gsis.enable) {   // the synthetic solve's RHS store has the distribution's type
        hyb::ns_destroy(ctx);
        rc = hyb::ns_create(ctx);
        if (rc) return rc;
    }
    rc = hyb_phy_boundary(ctx);
    if (!rc) rc = hyb_detfp(ctx);
    if (!rc) rc = hyb_convert_ns(ctx);
    if (!rc) HYB_CK(cudaStreamSynchronize(ctx->stream));
    ctx->rhs_valid = 0;
    return rc;
}

int hyb_destroy(hyb_ctx *ctx) {
    if (!ctx) return HYB_ERR_INVALID;
    cudaSetDevice(ctx->dev);
    cudaStreamSynchronize(ctx->stream);
    hyb::ns_destroy(ctx);
    free_all(ctx);
    delete ctx;
    return HYB_OK;
}

static int check_err_word(hyb_ctx *ctx) {
    int h = 0;
    HYB_CK(cudaMemcpyAsync(&h, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    HYB_CK(cudaStreamSynchronize(ctx->stream));
    if (h != 0) {
        ctx->last_error = "device error word set (bounded wait expired)";
        cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream);
        return h;
    }
    return HYB_OK;
}

// DETFP + GKUA_DET_wall + periodic S exchange
int hyb_detfp(hyb_ctx *ctx) {
    if (!ctx) return HYB_ERR_INVALID;
    int rc = hyb::launch_moments(ctx);
    if (!rc) rc = hyb::launch_sghost(ctx);
    return rc;
}

int hyb_phy_boundary(hyb_ctx *ctx) {
    if (!ctx) return HYB_ERR_INVALID;
    return hyb::launch_wall(ctx);
}

int hyb_kinetic_step(hyb_ctx *ctx) {
    if (!ctx) return HYB_ERR_INVALID;
    int rc = hyb::launch_sweep(ctx, 1);
    if (!rc) ctx->rhs_valid = 1;
    return rc;
}

int hyb_convert_ns(hyb_ctx *ctx) {
    if (!ctx) return HYB_ERR_INVALID;
    return hyb::launch_convert_ns(ctx);
}

int hyb_detfp_res(hyb_ctx *ctx, hyb_residual *out) {
    if (!ctx || !out) return HYB_ERR_INVALID;
    if (!ctx->rhs_valid) {
        ctx->last_error = "no RHS stored yet";
        return HYB_ERR_INVALID;
    }
    int rc = hyb::launch_residual(ctx, out);
    if (rc) return rc;
    for (int k = 0; k < 4; k++)
        if (!isfinite(out->res_rms[k]) || !isfinite(out->res_max[k])) return HYB_ERR_NONFINITE;
    return HYB_OK;
}

int hyb_init_maxwellian(hyb_ctx *ctx, double rho, double u, double v, double t) {
    if (!ctx) return HYB_ERR_INVALID;
    if (!(rho > 0) || !(t > 0)) return HYB_ERR_INVALID;
    cudaSetDevice(ctx->dev);
    int rc = hyb::launch_init_maxwellian(ctx, rho, u, v, t);
    // CF of the uniform state before the first DETFP (init_flow_zero)
    if (!rc) rc = hyb_phy_boundary(ctx);
    if (!rc) rc = hyb_detfp(ctx);
    if (!rc) rc = hyb_convert_ns(ctx);
    if (!rc) rc = hyb::launch_total_mass(ctx, 0);
    if (!rc) {
        HYB_CK(cudaStreamSynchronize(ctx->stream));
        ctx->rhs_valid = 0;
    }
    return rc;
}

}  // extern "C"

namespace {
enum Stage { ST_WALL = 0, ST_SWEEP, ST_MOM, ST_SGHOST, ST_CNS, ST_GSIS, ST_RESID, ST_COUNT };

// run one stage, bracketed by events when profiling is on
template <typename F>
int staged(hyb_ctx *ctx, int stage, size_t *evi, F &&fn) {
    if (!ctx->prof_on) return fn();
    if (*evi + 2 > ctx->prof_ev.size()) {
        for (int k = 0; k < 64; k++) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return HYB_ERR_CUDA;
            ctx->prof_ev.push_back(e);
        }
    }
    long long l0 = ctx->launches;
    cudaEventRecord(ctx->prof_ev[*evi], ctx->stream);
    int rc = fn();
    cudaEventRecord(ctx->prof_ev[*evi + 1], ctx->stream);
    ctx->prof_stage.push_back(stage);
    ctx->prof_launch[stage] += ctx->launches - l0;
    *evi += 2;
    return rc;
}

int collect_profile(hyb_ctx *ctx, size_t nev) {
    if (!ctx->prof_on || nev == 0) return HYB_OK;
    HYB_CK(cudaEventSynchronize(ctx->prof_ev[nev - 1]));
    for (size_t k = 0; k + 1 < nev; k += 2) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->prof_ev[k], ctx->prof_ev[k + 1]);
        ctx->prof_ms[ctx->prof_stage[k / 2]] += ms;
    }
    ctx->prof_stage.clear();
    return HYB_OK;
}
}  // namespace

extern "C" {

static int step_impl(hyb_ctx *ctx, int n_iter, hyb_residual *out);

int hyb_step(hyb_ctx *ctx, int n_iter, hyb_residual *out) {
    if (!ctx || n_iter < 1) return HYB_ERR_INVALID;
    const int rc = step_impl(ctx, n_iter, out);
    // a planted wait (hyb_test_stall) lasts one step
    if (ctx->stall_site != HYB_STALL_NONE) {
        cudaStreamSynchronize(ctx->stream);
        ctx->stall_site = HYB_STALL_NONE;
        ctx->spin_cycles = HYB_SPIN_CYCLES;
    }
    return rc;
}

int hyb_test_stall(hyb_ctx *ctx, int site, long long spin_cycles) {
    if (!ctx || spin_cycles <= 0) return HYB_ERR_INVALID;
    if (site != HYB_STALL_NONE && site != HYB_STALL_SWEEP_ROW && site != HYB_STALL_NS_BARRIER)
        return HYB_ERR_INVALID;
    ctx->stall_site = site;
    ctx->spin_cycles = site == HYB_STALL_NONE ? HYB_SPIN_CYCLES : spin_cycles;
    return HYB_OK;
}

static int step_impl(hyb_ctx *ctx, int n_iter, hyb_residual *out) {
    cudaSetDevice(ctx->dev);
    size_t evi = 0;
    ctx->prof_stage.clear();
    HYB_CK(cudaEventRecord(ctx->ev0, ctx->stream));
    for (int it = 0; it < n_iter; it++) {
        const bool last = (it == n_iter - 1);
        int rc = staged(ctx, ST_WALL, &evi, [&] { return hyb::launch_wall(ctx); });
        if (!rc) rc = staged(ctx, ST_SWEEP, &evi, [&] { return hyb::launch_sweep(ctx, last ? 1 : 0); });
        if (!rc) rc = staged(ctx, ST_MOM, &evi, [&] { return hyb::launch_moments(ctx); });
        if (!rc) rc = staged(ctx, ST_SGHOST, &evi, [&] { return hyb::launch_sghost(ctx); });
        // Convert_NS feeds the synthetic solve and the NS / HoT fields a caller
        // downloads: without GSIS only the call's last iteration needs it
        if (!rc && (ctx->gsis.enable || last))
            rc = staged(ctx, ST_CNS, &evi, [&] { return hyb::launch_convert_ns(ctx); });
        if (!rc && ctx->gsis.enable) rc = staged(ctx, ST_GSIS, &evi, [&] { return hyb::gsis_solve(ctx); });
        if (!rc && ctx->gsis.enable) {
            ctx->gsis_outer++;
            if (ctx->gsis.mlp_warm_after > 0 && !ctx->warm_done && ctx->gsis_outer >= ctx->gsis.mlp_warm_after) {
                ctx->warm_done = 1;
                rc = staged(ctx, ST_GSIS, &evi, [&] { return hyb::gsis_warm_start(ctx); });
                // a closure solve that left the physical range corrected nothing:
                // the kinetic iteration goes on from its own state
                if (rc == HYB_ERR_TEMPERATURE || rc == HYB_ERR_NONFINITE) {
                    ctx->warm_done = 2;
                    rc = HYB_OK;
                }
            }
        }
        if (rc) return rc;
    }
    ctx->rhs_valid = 1;
    HYB_CK(cudaEventRecord(ctx->ev1, ctx->stream));
    if (out) {
        int rc = staged(ctx, ST_RESID, &evi, [&] { return hyb::launch_residual(ctx, out); });
        if (rc) return rc;
    }
    HYB_CK(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->last_ms = ms;
    int rc = collect_profile(ctx, evi);
    if (rc) return rc;
    rc = check_err_word(ctx);
    if (rc) return rc;
    if (out)
        for (int k = 0; k < 4; k++)
            if (!isfinite(out->res_rms[k])) return HYB_ERR_NONFINITE;
    return HYB_OK;
}

int hyb_set_walls(hyb_ctx *ctx, int face, const double *wall_u, const double *wall_v, const double *wall_t) {
    if (!ctx || face < 1 || face > 4 || !wall_u || !wall_v || !wall_t) return HYB_ERR_INVALID;
    if (ctx->bc[face - 1] != HYB_BC_WALL) return HYB_ERR_INVALID;
    const int n = (face == 1 || face == 3) ? ctx->ncy : ctx->ncx;
    for (int k = 0; k < n; k++)
        if (!(wall_t[k] > 0.0)) return HYB_ERR_INVALID;
    cudaSetDevice(ctx->dev);
    // the staging buffer may still feed a previous copy
    HYB_CK(cudaStreamSynchronize(ctx->stream));
    double *tab = &ctx->wall_host[(size_t)(face - 1) * 4096 * 6];
    for (int k = 0; k < n; k++) {
        tab[k * 6 + 0] = wall_u[k];
        tab[k * 6 + 1] = wall_v[k];
        tab[k * 6 + 2] = wall_t[k];
        ctx->wall_u[face - 1][k] = wall_u[k];
        ctx->wall_v[face - 1][k] = wall_v[k];
        ctx->wall_t[face - 1][k] = wall_t[k];
    }
    memcpy(ctx->h_wall, tab, (size_t)n * 6 * sizeof(double));
    HYB_CK(cudaMemcpyAsync(ctx->d_wall + (size_t)(face - 1) * 4096 * 6, ctx->h_wall, (size_t)n * 6 * sizeof(double),
                           cudaMemcpyHostToDevice, ctx->stream));
    return HYB_OK;
}

int hyb_profile_enable(hyb_ctx *ctx, int enable) {
    if (!ctx) return HYB_ERR_INVALID;
    ctx->prof_on = enable ? 1 : 0;
    for (int k = 0; k < 8; k++) {
        ctx->prof_ms[k] = 0.0;
        ctx->prof_launch[k] = 0;
    }
    return HYB_OK;
}

int hyb_profile_read(hyb_ctx *ctx, double *ms, long long *launches, int n) {
    if (!ctx || n < 0) return HYB_ERR_INVALID;
    for (int k = 0; k < n && k < ST_COUNT; k++) {
        if (ms) ms[k] = ctx->prof_ms[k];
        if (launches) launches[k] = ctx->prof_launch[k];
    }
    return HYB_OK;
}

// ---- transfers -------------------------------------------------------------
int hyb_upload_f(hyb_ctx *ctx, const double *frd) {
    if (!ctx || !frd) return HYB_ERR_INVALID;
    cudaSetDevice(ctx->dev);
    const int nx = ctx->nx, ny = ctx->ny, pw = nx + 7;
    const size_t P = (size_t)(nx + 7) * (ny + 7), ncell = (size_t)ctx->Nb * ctx->PA;
    std::vector<double> buf((size_t)ctx->nv * 2 * ncell, 0.0);
    for (int v = 0; v < ctx->nv; v++)
        for (int j = 1; j <= ny - 1; j++)
            for (int i = 1; i <= nx - 1; i++) {
                size_t src = ((size_t)v * P + (size_t)(i + 3) + (size_t)pw * (j + 3)) * 2;
                size_t dc = dev_cell(ctx, i, j);
                buf[(size_t)v * 2 * ncell + dc] = frd[src + 0];
                buf[(size_t)v * 2 * ncell + ncell + dc] = frd[src + 1];
            }
    int rc = upload_real(ctx, ctx->d_f, buf);
    if (rc) return rc;
    rc = hyb_phy_boundary(ctx);
    if (!rc) rc = hyb_detfp(ctx);
    if (!rc) rc = hyb_convert_ns(ctx);
    if (!rc) rc = hyb::launch_total_mass(ctx, 0);
    if (!rc) HYB_CK(cudaStreamSynchronize(ctx->stream));
    ctx->rhs_valid = 0;
    return rc;
}

int hyb_download_f(hyb_ctx *ctx, double *frd) {
    if (!ctx || !frd) return HYB_ERR_INVALID;
    cudaSetDevice(ctx->dev);
    const int nx = ctx->nx, ny = ctx->ny, pw = nx + 7;
    const size_t P = (size_t)(nx + 7) * (ny + 7), ncell = (size_t)ctx->Nb * ctx->PA;
    const size_t n = (size_t)ctx->nv * 2 * ncell;
    std::vector<double> buf(n);
    HYB_CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->precision == HYB_PREC_FP64) {
        HYB_CK(cudaMemcpy(buf.data(), ctx->d_f, n * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> tmp(n);
        HYB_CK(cudaMemcpy(tmp.data(), ctx->d_f, n * sizeof(float), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < n; k++) buf[k] = tmp[k];
    }
    for (int v = 0; v < ctx->nv; v++)
        for (int j = 1; j <= ny - 1; j++)
            for (int i = 1; i <= nx - 1; i++) {
                size_t dst = ((size_t)v * P + (size_t)(i + 3) + (size_t)pw * (j + 3)) * 2;
                size_t dc = dev_cell(ctx, i, j);
                frd[dst + 0] = buf[(size_t)v * 2 * ncell + dc];
                frd[dst + 1] = buf[(size_t)v * 2 * ncell + ncell + dc];
            }
    return HYB_OK;
}

// S_GKUA is transposed to the host's component-fastest order on the device
// and copied row by row into the block -1..nx+1 x -1..ny+1 of the host array
// (the outer ghost layers of the host array are left as they are)
int hyb_download_moments(hyb_ctx *ctx, double *s_gkua, double *cf) {
    if (!ctx || (!s_gkua && !cf)) return HYB_ERR_INVALID;
    cudaSetDevice(ctx->dev);
    const int nx = ctx->nx, ny = ctx->ny, pw = nx + 7;
    const size_t nc2 = (size_t)(nx + 3) * (ny + 3);
    if (s_gkua) {
        if (!ctx->d_stage && cudaMalloc((void **)&ctx->d_stage, HYB_NSUM * nc2 * sizeof(double)) != cudaSuccess) {
            ctx->d_stage = nullptr;
            ctx->last_error = "download_moments: device staging allocation failed";
            return HYB_ERR_NOMEM;
        }
        int rc = hyb::launch_s_host_layout(ctx, ctx->d_stage);
        if (rc) return rc;
        const size_t row = (size_t)(nx + 3) * HYB_NSUM * sizeof(double);
        HYB_CK(cudaMemcpy2DAsync(s_gkua + ((size_t)2 + (size_t)pw * 2) * HYB_NSUM, (size_t)pw * HYB_NSUM * sizeof(double),
                                 ctx->d_stage, row, row, (size_t)ny + 3, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (cf) HYB_CK(cudaMemcpyAsync(cf, ctx->d_CF, nc2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    HYB_CK(cudaStreamSynchronize(ctx->stream));
    return HYB_OK;
}

int hyb_download_hoq(hyb_ctx *ctx, double *hot, double *hoq) {
    if (!ctx || (!hot && !hoq)) return HYB_ERR_INVALID;
    cudaSetDevice(ctx->dev);
    const int nx = ctx->nx, ny = ctx->ny, pw = nx + 7;
    const size_t nc2 = (size_t)(nx + 3) * (ny + 3), P = (size_t)(nx + 7) * (ny + 7);
    double *d = nullptr;
    if (cudaMalloc((void **)&d, 9 * nc2 * sizeof(double)) != cudaSuccess) {
        ctx->last_error = "download_hoq: device allocation failed";
        return HYB_ERR_NOMEM;
    }
    std::vector<double> H(9 * nc2);
    int rc = HYB_OK;
    if (cudaMemsetAsync(d, 0, 9 * nc2 * sizeof(double), ctx->stream) != cudaSuccess) rc = HYB_ERR_CUDA;
    if (!rc) rc = hyb::launch_hoq(ctx, d);
    if (!rc && cudaMemcpyAsync(H.data(), d, H.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) !=
                   cudaSuccess)
        rc = HYB_ERR_CUDA;
    if (!rc && cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = HYB_ERR_CUDA;
    cudaFree(d);
    if (rc) return rc;
    if (hot) std::fill(hot, hot + 6 * P, 0.0);
    if (hoq) std::fill(hoq, hoq + 4 * P, 0.0);
    for (int j = -1; j <= ny + 1; j++)
        for (int i = -1; i <= nx + 1; i++) {
            const size_t c2 = hyb_c2(nx, i, j), ix = (size_t)(i + 3) + (size_t)pw * (j + 3);
            if (hot)
                for (int k = 0; k < 6; k++) hot[ix * 6 + k] = H[(size_t)k * nc2 + c2];
            if (hoq)
                for (int k = 0; k < 3; k++) hoq[ix * 4 + k] = H[(size_t)(6 + k) * nc2 + c2];
        }
    return HYB_OK;
}

int hyb_download_hot(hyb_ctx *ctx, double *tao_i, double *q_i, double *tao_j, double *q_j) {
    if (!ctx) return HYB_ERR_INVALID;
    cudaSetDevice(ctx->dev);
    const size_t nc2 = (size_t)(ctx->nx + 3) * (ctx->ny + 3);
    std::vector<double> H(hyb::hot_doubles(ctx->nx, ctx->ny));
    HYB_CK(cudaStreamSynchronize(ctx->stream));
    HYB_CK(cudaMemcpy(H.data(), ctx->d_hot, H.size() * sizeof(double), cudaMemcpyDeviceToHost));
    // d_hot: U[4] d uu vv T amu tin_i[4] qin_i[2] tin_j[4] qin_j[2] tg_i[4] qg_i[2] tg_j[4] qg_j[2]
    const double *tg_i = H.data() + 21 * nc2, *qg_i = tg_i + 4 * nc2, *tg_j = qg_i + 2 * nc2, *qg_j = tg_j + 4 * nc2;
    for (size_t c = 0; c < nc2; c++) {
        if (tao_i) for (int k = 0; k < 4; k++) tao_i[c * 4 + k] = tg_i[k * nc2 + c];
        if (q_i) for (int k = 0; k < 2; k++) q_i[c * 2 + k] = qg_i[k * nc2 + c];
        if (tao_j) for (int k = 0; k < 4; k++) tao_j[c * 4 + k] = tg_j[k * nc2 + c];
        if (q_j) for (int k = 0; k < 2; k++) q_j[c * 2 + k] = qg_j[k * nc2 + c];
    }
    return HYB_OK;
}

// ---- GSIS ------------------------------------------------------------------
int hyb_gsis_configure(hyb_ctx *ctx, const hyb_gsis_params *gp) {
    if (!ctx || !gp) return HYB_ERR_INVALID;
    ctx->gsis = *gp;
    ctx->gsis_outer = 0;
    ctx->gsis_skipped = 0;
    ctx->warm_done = 0;
    if (gp->enable) return hyb::ns_create(ctx);
    return HYB_OK;
}

int hyb_gsis_last_inner(const hyb_ctx *ctx, int *n_inner) {
    if (!ctx || !n_inner) return HYB_ERR_INVALID;
    *n_inner = ctx->gsis_last_inner;
    return HYB_OK;
}

int hyb_gsis_skipped(const hyb_ctx *ctx, int *count) {
    if (!ctx || !count) return HYB_ERR_INVALID;
    *count = ctx->gsis_skipped;
    return HYB_OK;
}

// ---- introspection -----------------------------------------------------------
int hyb_launch_count(const hyb_ctx *ctx, long long *count) {
    if (!ctx || !count) return HYB_ERR_INVALID;
    *count = ctx->launches;
    return HYB_OK;
}

int hyb_last_step_ms(const hyb_ctx *ctx, double *ms) {
    if (!ctx || !ms) return HYB_ERR_INVALID;
    *ms = ctx->last_ms;
    return HYB_OK;
}

int hyb_stream(const hyb_ctx *ctx, void **stream) {
    if (!ctx || !stream) return HYB_ERR_INVALID;
    *stream = (void *)ctx->stream;
    return HYB_OK;
}

}  // extern "C"
