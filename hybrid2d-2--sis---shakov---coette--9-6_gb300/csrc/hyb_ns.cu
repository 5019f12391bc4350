// hyb_ns.cu -- FP64 macroscopic kernels around the kinetic step.
//
//   k_sghost       S ghost cells: DETFPwall (GKUA_DETFP_WALL.f90:34-95) on wall
//                  faces, the inner-block exchange (GKUA_boundary.f90:514-633)
//                  on periodic faces
//   k_cns_*        Convert_NS (Hybrid_Sub.f90:191-461): NS state from the
//                  moments, Navier-Stokes-Fourier stress / heat flux on every
//                  face and the higher-order terms TaoNS*_G, Q*_G
//
// All arrays are on the reference extents (1-LAP:n+LAP-1) with i fastest,
// SoA over components: X[c][(nx+3)(ny+3)].
#include <cuda_runtime.h>

#include <algorithm>
#include <math.h>

#include "hyb_common.cuh"

namespace hyb {

struct NsGeom {
    int nx, ny;
    int perx, pery;          // periodic faces 1/3, 2/4
    int wall[4];             // faces with diffuse walls
    size_t nc;               // (nx+3)(ny+3)
};

__device__ __forceinline__ size_t C2(const NsGeom &G, int i, int j) { return hyb_c2(G.nx, i, j); }

// ---- S ghosts: walls (DETFPwall), components 1..10 ---------------------------
__device__ __forceinline__ void sghost_wall(double *S, const NsGeom &G, int idx) {
    const int nx = G.nx, ny = G.ny;
    // faces 2/4: i = 1..nx-1; faces 1/3: j = 1..ny-1
    int nfx = nx - 1, nfy = ny - 1;
    int face, k;
    if (idx < nfx) { face = 2; k = idx + 1; }
    else if (idx < 2 * nfx) { face = 4; k = idx - nfx + 1; }
    else if (idx < 2 * nfx + nfy) { face = 1; k = idx - 2 * nfx + 1; }
    else if (idx < 2 * nfx + 2 * nfy) { face = 3; k = idx - 2 * nfx - nfy + 1; }
    else return;
    if (!G.wall[face - 1]) return;
    int g1, g2, a1, a2, b1, b2;
    if (face == 1) { g1 = 0; g2 = k; a1 = 1; a2 = k; b1 = 2; b2 = k; }
    else if (face == 2) { g1 = k; g2 = 0; a1 = k; a2 = 1; b1 = k; b2 = 2; }
    else if (face == 3) { g1 = nx; g2 = k; a1 = nx - 1; a2 = k; b1 = nx - 2; b2 = k; }
    else { g1 = k; g2 = ny; a1 = k; a2 = ny - 1; b1 = k; b2 = ny - 2; }
    for (int c = 0; c < 10; c++) {
        double *Sc = S + (size_t)c * G.nc;
        double sw = (-Sc[C2(G, b1, b2)] + 3.0 * Sc[C2(G, a1, a2)]) * 0.5;
        Sc[C2(G, g1, g2)] = 2.0 * sw - Sc[C2(G, a1, a2)];
    }
}

// ---- S ghosts: periodic faces, components 1..10, LAP layers -----------------
__device__ __forceinline__ void sghost_periodic(double *S, const NsGeom &G, int idx) {
    const int nx = G.nx, ny = G.ny;
    int n1 = G.perx ? (ny - 1) : 0, n2 = G.pery ? (nx - 1) : 0;
    if (idx < n1) {
        int j = idx + 1;
        for (int c = 0; c < 10; c++) {
            double *Sc = S + (size_t)c * G.nc;
            for (int l = 1; l <= HYB_LAP; l++) {
                Sc[C2(G, 1 - l, j)] = Sc[C2(G, nx - l, j)];
                Sc[C2(G, nx - 1 + l, j)] = Sc[C2(G, l, j)];
            }
        }
    } else if (idx < n1 + n2) {
        int i = idx - n1 + 1;
        for (int c = 0; c < 10; c++) {
            double *Sc = S + (size_t)c * G.nc;
            for (int l = 1; l <= HYB_LAP; l++) {
                Sc[C2(G, i, 1 - l)] = Sc[C2(G, i, ny - l)];
                Sc[C2(G, i, ny - 1 + l)] = Sc[C2(G, i, l)];
            }
        }
    }
}

// both ghost kinds in one launch: the wall ghosts (rows / columns 0 and n
// along the wall) and the periodic layers (interior rows / columns copied
// across) write disjoint cells and read interior cells only
__global__ void k_sghost(double *S, NsGeom G, int nwall) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < nwall) sghost_wall(S, G, idx);
    else sghost_periodic(S, G, idx - nwall);
}

// ---- Convert_NS ------------------------------------------------------------
struct CnsArgs {
    NsGeom G;
    double *S;           // [NSUM][nc]
    double *U;           // [4][nc]
    double *d, *uu, *vv, *T, *amu;   // [nc]
    const double *x1, *y1;
    double *tao_i_in, *q_i_in, *tao_j_in, *q_j_in;   // [4|2][nc]
    double *tao_i_g, *q_i_g, *tao_j_g, *q_j_g;
    double gamma, ma, pr, re, omega, cv, cp;
};

// corners of S (Hybrid_Sub.f90:221-224; periodic faces copy the partner)
__device__ __forceinline__ void cns_corners(const CnsArgs &A, int k) {
    const NsGeom &G = A.G;
    const int nx = G.nx, ny = G.ny;
    if (k >= HYB_NSUM) return;
    double *Sk = A.S + (size_t)k * G.nc;
    if (G.perx) {
        Sk[C2(G, 0, 0)] = Sk[C2(G, nx - 1, 0)];
        Sk[C2(G, nx, 0)] = Sk[C2(G, 1, 0)];
        Sk[C2(G, 0, ny)] = Sk[C2(G, nx - 1, ny)];
        Sk[C2(G, nx, ny)] = Sk[C2(G, 1, ny)];
    } else if (G.pery) {
        Sk[C2(G, 0, 0)] = Sk[C2(G, 0, ny - 1)];
        Sk[C2(G, 0, ny)] = Sk[C2(G, 0, 1)];
        Sk[C2(G, nx, 0)] = Sk[C2(G, nx, ny - 1)];
        Sk[C2(G, nx, ny)] = Sk[C2(G, nx, 1)];
    } else {
        Sk[C2(G, 0, 0)] = Sk[C2(G, 1, 0)] + Sk[C2(G, 0, 1)] - Sk[C2(G, 1, 1)];
        Sk[C2(G, nx, 0)] = Sk[C2(G, nx, 1)] + Sk[C2(G, nx - 1, 0)] - Sk[C2(G, nx - 1, 1)];
        Sk[C2(G, 0, ny)] = Sk[C2(G, 1, ny)] + Sk[C2(G, 0, ny - 1)] - Sk[C2(G, 1, ny - 1)];
        Sk[C2(G, nx, ny)] = Sk[C2(G, nx - 1, ny)] + Sk[C2(G, nx, ny - 1)] - Sk[C2(G, nx - 1, ny - 1)];
    }
}

// U from S on 0..nx x 0..ny (Hybrid_Sub.f90:225-235); cells outside keep
// the reference's initial state
__device__ __forceinline__ void cns_u(const CnsArgs &A, size_t idx) {
    const NsGeom &G = A.G;
    const int nx = G.nx, ny = G.ny;
    if (idx >= G.nc) return;
    int i = (int)(idx % (nx + 3)) - 1, j = (int)(idx / (nx + 3)) - 1;
    double *U0 = A.U, *U1 = A.U + G.nc, *U2 = A.U + 2 * G.nc, *U3 = A.U + 3 * G.nc;
    if (i < 0 || i > nx || j < 0 || j > ny) {
        U0[idx] = 1.0; U1[idx] = 0.0; U2[idx] = 0.0; U3[idx] = A.cv;
        return;
    }
    double s1 = A.S[idx], s2 = A.S[G.nc + idx], s3 = A.S[2 * G.nc + idx], s4 = A.S[3 * G.nc + idx];
    double r = s1;
    double tu = s2 / A.ma * sqrt(2.0 / A.gamma);
    double tv = s3 / A.ma * sqrt(2.0 / A.gamma);
    U0[idx] = r;
    U1[idx] = r * tu;
    U2[idx] = r * tv;
    U3[idx] = r * A.cv * s4 + 0.5 * r * (tu * tu + tv * tv);
}

// ghost U: columns then rows (Hybrid_Sub.f90:236-239), periodic faces copy
__device__ __forceinline__ void cns_ughost_col(const CnsArgs &A, int t) {
    const NsGeom &G = A.G;
    const int nx = G.nx;
    const int j = t - 1;
    if (j > G.ny + 1) return;
    for (int m = 0; m < 4; m++) {
        double *Um = A.U + (size_t)m * G.nc;
        if (G.perx) {
            Um[C2(G, 0, j)] = Um[C2(G, nx - 1, j)];
            Um[C2(G, -1, j)] = Um[C2(G, nx - 2, j)];
            Um[C2(G, nx, j)] = Um[C2(G, 1, j)];
            Um[C2(G, nx + 1, j)] = Um[C2(G, 2, j)];
        } else {
            Um[C2(G, 0, j)] = 2.0 * Um[C2(G, 1, j)] - Um[C2(G, 2, j)];
            Um[C2(G, nx, j)] = 2.0 * Um[C2(G, nx - 1, j)] - Um[C2(G, nx - 2, j)];
        }
    }
}
__device__ __forceinline__ void cns_ughost_row(const CnsArgs &A, int t) {
    const NsGeom &G = A.G;
    const int ny = G.ny;
    const int i = t - 1;
    if (i > G.nx + 1) return;
    for (int m = 0; m < 4; m++) {
        double *Um = A.U + (size_t)m * G.nc;
        if (G.pery) {
            Um[C2(G, i, 0)] = Um[C2(G, i, ny - 1)];
            Um[C2(G, i, -1)] = Um[C2(G, i, ny - 2)];
            Um[C2(G, i, ny)] = Um[C2(G, i, 1)];
            Um[C2(G, i, ny + 1)] = Um[C2(G, i, 2)];
        } else {
            Um[C2(G, i, 0)] = 2.0 * Um[C2(G, i, 1)] - Um[C2(G, i, 2)];
            Um[C2(G, i, ny)] = 2.0 * Um[C2(G, i, ny - 1)] - Um[C2(G, i, ny - 2)];
        }
    }
}

// primitive NS variables and viscosity (comput_duvtpckw, get_viscous)
__device__ __forceinline__ void cns_prim(const CnsArgs &A, size_t idx) {
    const NsGeom &G = A.G;
    if (idx >= G.nc) return;
    int i = (int)(idx % (G.nx + 3)) - 1, j = (int)(idx / (G.nx + 3)) - 1;
    double d = A.U[idx];
    double u = A.U[G.nc + idx] / d, v = A.U[2 * G.nc + idx] / d;
    double t = (A.U[3 * G.nc + idx] - 0.5 * d * (u * u + v * v)) / (A.cv * d);
    A.d[idx] = d;
    A.uu[idx] = u;
    A.vv[idx] = v;
    A.T[idx] = t;
    if (i >= 0 && i <= G.nx && j >= 0 && j <= G.ny) A.amu[idx] = 1.0 / A.re * pow(t, A.omega);
}

// face quantities: dir 0 = i-faces (i=1..nx, j=1..ny-1), 1 = j-faces
__device__ __forceinline__ void cns_face(const CnsArgs &A, int dir, int idx) {
    const NsGeom &G = A.G;
    const int nx = G.nx, ny = G.ny;
    int ni = dir == 0 ? nx : nx - 1, nj = dir == 0 ? ny - 1 : ny;
    if (idx >= ni * nj) return;
    int i = idx % ni + 1, j = idx / ni + 1;
    const double *x1 = A.x1, *y1 = A.y1, *uu = A.uu, *vv = A.vv, *T = A.T, *amu = A.amu;
    const double cp = A.cp, pr = A.pr;
    int lo, hi;
    double amu1, amk1, dix, diy, djx, djy, diu, div, dit, dju, djv, djt;
    if (dir == 0) {
        lo = (i == 1) && !G.perx;
        hi = (i == nx) && !G.perx;
        if (lo) { amu1 = amu[C2(G, i, j)]; amk1 = cp * (amu[C2(G, i, j)] / pr); }
        else if (hi) { amu1 = amu[C2(G, i - 1, j)]; amk1 = cp * (amu[C2(G, i - 1, j)] / pr); }
        else {
            amu1 = (amu[C2(G, i - 1, j)] + amu[C2(G, i, j)]) * 0.5;
            amk1 = cp * ((amu[C2(G, i - 1, j)] + amu[C2(G, i, j)]) / pr) * 0.5;
        }
        dix = x1[C2(G, i, j)] - x1[C2(G, i - 1, j)];
        diy = y1[C2(G, i, j)] - y1[C2(G, i - 1, j)];
        djx = (x1[C2(G, i - 1, j + 1)] + x1[C2(G, i, j + 1)] - x1[C2(G, i - 1, j - 1)] - x1[C2(G, i, j - 1)]) * 0.25;
        djy = (y1[C2(G, i - 1, j + 1)] + y1[C2(G, i, j + 1)] - y1[C2(G, i - 1, j - 1)] - y1[C2(G, i, j - 1)]) * 0.25;
        diu = uu[C2(G, i, j)] - uu[C2(G, i - 1, j)];
        div = vv[C2(G, i, j)] - vv[C2(G, i - 1, j)];
        dit = T[C2(G, i, j)] - T[C2(G, i - 1, j)];
        dju = (uu[C2(G, i - 1, j + 1)] + uu[C2(G, i, j + 1)] - uu[C2(G, i - 1, j - 1)] - uu[C2(G, i, j - 1)]) * 0.25;
        djv = (vv[C2(G, i - 1, j + 1)] + vv[C2(G, i, j + 1)] - vv[C2(G, i - 1, j - 1)] - vv[C2(G, i, j - 1)]) * 0.25;
        djt = (T[C2(G, i - 1, j + 1)] + T[C2(G, i, j + 1)] - T[C2(G, i - 1, j - 1)] - T[C2(G, i, j - 1)]) * 0.25;
    } else {
        lo = (j == 1) && !G.pery;
        hi = (j == ny) && !G.pery;
        if (lo) { amu1 = amu[C2(G, i, j)]; amk1 = cp * (amu[C2(G, i, j)] / pr); }
        else if (hi) { amu1 = amu[C2(G, i, j - 1)]; amk1 = cp * (amu[C2(G, i, j - 1)] / pr); }
        else {
            amu1 = (amu[C2(G, i, j)] + amu[C2(G, i, j - 1)]) * 0.5;
            amk1 = cp * ((amu[C2(G, i, j - 1)] + amu[C2(G, i, j)]) / pr) * 0.5;
        }
        dix = (x1[C2(G, i + 1, j - 1)] + x1[C2(G, i + 1, j)] - x1[C2(G, i - 1, j - 1)] - x1[C2(G, i - 1, j)]) * 0.25;
        diy = (y1[C2(G, i + 1, j - 1)] + y1[C2(G, i + 1, j)] - y1[C2(G, i - 1, j - 1)] - y1[C2(G, i - 1, j)]) * 0.25;
        djx = x1[C2(G, i, j)] - x1[C2(G, i, j - 1)];
        djy = y1[C2(G, i, j)] - y1[C2(G, i, j - 1)];
        diu = (uu[C2(G, i + 1, j - 1)] + uu[C2(G, i + 1, j)] - uu[C2(G, i - 1, j - 1)] - uu[C2(G, i - 1, j)]) * 0.25;
        div = (vv[C2(G, i + 1, j - 1)] + vv[C2(G, i + 1, j)] - vv[C2(G, i - 1, j - 1)] - vv[C2(G, i - 1, j)]) * 0.25;
        dit = (T[C2(G, i + 1, j - 1)] + T[C2(G, i + 1, j)] - T[C2(G, i - 1, j - 1)] - T[C2(G, i - 1, j)]) * 0.25;
        dju = uu[C2(G, i, j)] - uu[C2(G, i, j - 1)];
        djv = vv[C2(G, i, j)] - vv[C2(G, i, j - 1)];
        djt = T[C2(G, i, j)] - T[C2(G, i, j - 1)];
    }
    double ds = 1.0 / (dix * djy - djx * diy);
    double ux = (diu * djy - dju * diy) * ds, vx = (div * djy - djv * diy) * ds, tx = (dit * djy - djt * diy) * ds;
    double uy = (-diu * djx + dju * dix) * ds, vy = (-div * djx + djv * dix) * ds, ty = (-dit * djx + djt * dix) * ds;
    double t11 = ((4.0 / 3.0) * ux - (2.0 / 3.0) * vy) * amu1;
    double t22 = ((4.0 / 3.0) * vy - (2.0 / 3.0) * ux) * amu1;
    double t12 = (uy + vx) * amu1;
    double t33 = amu1 * (-(2.0 / 3.0) * ux - (2.0 / 3.0) * vy);
    double qx = amk1 * tx, qy = amk1 * ty;
    size_t c = C2(G, i, j);
    double *tin = dir == 0 ? A.tao_i_in : A.tao_j_in, *qin = dir == 0 ? A.q_i_in : A.q_j_in;
    double *tg = dir == 0 ? A.tao_i_g : A.tao_j_g, *qg = dir == 0 ? A.q_i_g : A.q_j_g;
    tin[0 * G.nc + c] = t11;
    tin[1 * G.nc + c] = t22;
    tin[2 * G.nc + c] = t12;
    tin[3 * G.nc + c] = t33;
    qin[0 * G.nc + c] = qx;
    qin[1 * G.nc + c] = qy;
    const double g2 = A.gamma * A.ma * A.ma;
    const double q2 = sqrt(2.0) / (pow(A.ma, 3) * pow(A.gamma, 1.5));
    const double *S5 = A.S + 4 * G.nc, *S6 = A.S + 5 * G.nc, *S7 = A.S + 6 * G.nc;
    const double *S8 = A.S + 7 * G.nc, *S9 = A.S + 8 * G.nc, *S10 = A.S + 9 * G.nc;
    size_t cm = dir == 0 ? C2(G, i - 1, j) : C2(G, i, j - 1);   // the other side
    if (!lo && !hi) {
        double tmp = (S5[c] + S6[c] + S10[c] + S5[cm] + S6[cm] + S10[cm]) / 6.0;
        tg[0 * G.nc + c] = -((S5[c] + S5[cm]) / 2.0 - tmp) / g2 - t11;
        tg[1 * G.nc + c] = -((S6[c] + S6[cm]) / 2.0 - tmp) / g2 - t22;
        tg[2 * G.nc + c] = -(S7[c] + S7[cm]) / 2.0 / g2 - t12;
        tg[3 * G.nc + c] = -((S10[c] + S10[cm]) / 2.0 - tmp) / g2 - t33;
        qg[0 * G.nc + c] = -(S8[cm] + S8[c]) / 2.0 * q2 - qx;
        qg[1 * G.nc + c] = -(S9[cm] + S9[c]) / 2.0 * q2 - qy;
    } else {
        size_t cc = lo ? c : cm;
        double tmp = (S5[cc] + S6[cc] + S10[cc]) / 3.0;
        tg[0 * G.nc + c] = -(S5[cc] - tmp) / g2 - t11;
        tg[1 * G.nc + c] = -(S6[cc] - tmp) / g2 - t22;
        tg[2 * G.nc + c] = -S7[cc] / g2 - t12;
        tg[3 * G.nc + c] = -(S10[cc] - tmp) / g2 - t33;
        qg[0 * G.nc + c] = -S8[cc] * q2 - qx;
        qg[1 * G.nc + c] = -S9[cc] * q2 - qy;
    }
}

__global__ void k_cns_corners(CnsArgs A) { cns_corners(A, threadIdx.x); }
__global__ void k_cns_u(CnsArgs A) { cns_u(A, (size_t)blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void k_cns_ughost_cols(CnsArgs A) { cns_ughost_col(A, blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void k_cns_ughost_rows(CnsArgs A) { cns_ughost_row(A, blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void k_cns_prim(CnsArgs A) { cns_prim(A, (size_t)blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void k_cns_faces(CnsArgs A, int dir) { cns_face(A, dir, blockIdx.x * blockDim.x + threadIdx.x); }

// Convert_NS of many contexts: block i runs phase work[i].y (0 corners, 1 U,
// 2 ghost columns, 3 ghost rows, 4 primitives, 5 i-faces, 6 j-faces) for
// threads 128 work[i].z .. of context work[i].x; a launch holds one phase, or
// the two face phases, which are independent
__global__ void __launch_bounds__(128) k_cns_batch(const CnsArgs *__restrict__ args, const int4 *__restrict__ work) {
    __shared__ CnsArgs As;
    const int4 w = work[blockIdx.x];
    if (threadIdx.x == 0) As = args[w.x];
    __syncthreads();
    const int t = w.z * 128 + threadIdx.x;
    switch (w.y) {
        case 0: cns_corners(As, t); break;
        case 1: cns_u(As, (size_t)t); break;
        case 2: cns_ughost_col(As, t); break;
        case 3: cns_ughost_row(As, t); break;
        case 4: cns_prim(As, (size_t)t); break;
        case 5: cns_face(As, 0, t); break;
        default: cns_face(As, 1, t); break;
    }
}

static NsGeom make_geom(const hyb_ctx *ctx) {
    NsGeom G;
    G.nx = ctx->nx;
    G.ny = ctx->ny;
    G.perx = ctx->bc[0] == HYB_BC_PERIODIC;
    G.pery = ctx->bc[1] == HYB_BC_PERIODIC;
    for (int f = 0; f < 4; f++) G.wall[f] = ctx->bc[f] == HYB_BC_WALL;
    G.nc = (size_t)(ctx->nx + 3) * (ctx->ny + 3);
    return G;
}

static int check(hyb_ctx *ctx, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ctx->last_error = std::string(what) + ": " + cudaGetErrorString(e);
        return HYB_ERR_CUDA;
    }
    return HYB_OK;
}

int launch_sghost(hyb_ctx *ctx) {
    NsGeom G = make_geom(ctx);
    const int nwall = 2 * (ctx->nx - 1) + 2 * (ctx->ny - 1);
    const int nper = (G.perx ? ctx->ny - 1 : 0) + (G.pery ? ctx->nx - 1 : 0);
    const int n = nwall + nper;
    k_sghost<<<(n + 127) / 128, 128, 0, ctx->stream>>>(ctx->d_S, G, nwall);
    ctx->launches++;
    return check(ctx, "k_sghost");
}

// ---- S in the host's component-fastest order ---------------------------------
// out[c * NSUM + k] = S[k][c] over the (nx+3)(ny+3) block, so that its rows
// are the host array's rows of S_GKUA(1:NSUM, -1:nx+1, j)
__global__ void k_s_host_layout(const double *__restrict__ S, size_t nc, double *__restrict__ out) {
    const size_t n = nc * HYB_NSUM;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const size_t c = t / HYB_NSUM;
        out[t] = S[(t - c * HYB_NSUM) * nc + c];
    }
}

int launch_s_host_layout(hyb_ctx *ctx, double *out) {
    const size_t nc = (size_t)(ctx->nx + 3) * (ctx->ny + 3);
    const size_t n = nc * HYB_NSUM;
    const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 8);
    k_s_host_layout<<<grid, 256, 0, ctx->stream>>>(ctx->d_S, nc, out);
    ctx->launches++;
    return check(ctx, "k_s_host_layout");
}

// ---- S ghosts of many contexts in one launch (hyb_batch) ----------------------
struct SghostArgs {
    double *S;
    NsGeom G;
    int nwall;
};

// work[blockIdx.x] = (context, first ghost index of the block)
__global__ void k_sghost_batch(const SghostArgs *__restrict__ args, const int2 *__restrict__ work,
                               const int *__restrict__ count) {
    const int2 w = work[blockIdx.x];
    const SghostArgs &A = args[w.x];
    const int idx = w.y + threadIdx.x;
    if (idx >= count[w.x]) return;
    if (idx < A.nwall) sghost_wall(A.S, A.G, idx);
    else sghost_periodic(A.S, A.G, idx - A.nwall);
}

size_t sghost_arg_bytes() { return sizeof(SghostArgs); }

// fills the context's record; returns its number of ghost threads
int sghost_arg_fill(hyb_ctx *ctx, void *dst) {
    SghostArgs a;
    a.S = ctx->d_S;
    a.G = make_geom(ctx);
    a.nwall = 2 * (ctx->nx - 1) + 2 * (ctx->ny - 1);
    memcpy(dst, &a, sizeof(a));
    return a.nwall + (a.G.perx ? ctx->ny - 1 : 0) + (a.G.pery ? ctx->nx - 1 : 0);
}

int sghost_batch_launch(const void *args, const int2 *work, const int *count, int nblocks, cudaStream_t s) {
    if (nblocks <= 0) return HYB_OK;
    k_sghost_batch<<<nblocks, 128, 0, s>>>((const SghostArgs *)args, work, count);
    return cudaGetLastError() == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
}

// layout of ctx->d_hot: U[4], d, uu, vv, T, amu, tao_i_in[4], q_i_in[2],
// tao_j_in[4], q_j_in[2], tao_i_g[4], q_i_g[2], tao_j_g[4], q_j_g[2]
static CnsArgs make_cns(hyb_ctx *ctx) {
    CnsArgs A;
    A.G = make_geom(ctx);
    size_t nc = A.G.nc;
    double *h = ctx->d_hot;
    A.S = ctx->d_S;
    A.U = h; h += 4 * nc;
    A.d = h; h += nc;
    A.uu = h; h += nc;
    A.vv = h; h += nc;
    A.T = h; h += nc;
    A.amu = h; h += nc;
    A.tao_i_in = h; h += 4 * nc;
    A.q_i_in = h; h += 2 * nc;
    A.tao_j_in = h; h += 4 * nc;
    A.q_j_in = h; h += 2 * nc;
    A.tao_i_g = h; h += 4 * nc;
    A.q_i_g = h; h += 2 * nc;
    A.tao_j_g = h; h += 4 * nc;
    A.q_j_g = h; h += 2 * nc;
    A.x1 = ctx->d_x1;
    A.y1 = ctx->d_y1;
    A.gamma = ctx->prm.gamma;
    A.ma = ctx->prm.ma;
    A.pr = ctx->prm.pr;
    A.re = ctx->prm.re;
    A.omega = ctx->prm.omega_ns;
    A.cv = 1.0 / (A.gamma * (A.gamma - 1.0) * A.ma * A.ma);
    A.cp = A.cv * A.gamma;
    return A;
}

size_t hot_doubles(int nx, int ny) { return (size_t)(nx + 3) * (ny + 3) * 33; }

size_t cns_arg_bytes() { return sizeof(CnsArgs); }

// the context's record and the threads of its seven phases
int cns_arg_fill(hyb_ctx *ctx, void *dst, int counts[7]) {
    CnsArgs A = make_cns(ctx);
    memcpy(dst, &A, sizeof(A));
    counts[0] = HYB_NSUM;
    counts[1] = (int)A.G.nc;
    counts[2] = ctx->ny + 3;
    counts[3] = ctx->nx + 3;
    counts[4] = (int)A.G.nc;
    counts[5] = ctx->nx * (ctx->ny - 1);
    counts[6] = (ctx->nx - 1) * ctx->ny;
    return HYB_OK;
}

int cns_batch_launch(const void *args, const int4 *work, int nwork, cudaStream_t s) {
    if (nwork <= 0) return HYB_OK;
    k_cns_batch<<<nwork, 128, 0, s>>>((const CnsArgs *)args, work);
    return cudaGetLastError() == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
}

int launch_convert_ns(hyb_ctx *ctx) {
    CnsArgs A = make_cns(ctx);
    size_t nc = A.G.nc;
    int bs = 128;
    k_cns_corners<<<1, 32, 0, ctx->stream>>>(A);
    k_cns_u<<<(unsigned)((nc + bs - 1) / bs), bs, 0, ctx->stream>>>(A);
    k_cns_ughost_cols<<<(ctx->ny + 3 + bs - 1) / bs, bs, 0, ctx->stream>>>(A);
    k_cns_ughost_rows<<<(ctx->nx + 3 + bs - 1) / bs, bs, 0, ctx->stream>>>(A);
    k_cns_prim<<<(unsigned)((nc + bs - 1) / bs), bs, 0, ctx->stream>>>(A);
    int nfi = ctx->nx * (ctx->ny - 1), nfj = (ctx->nx - 1) * ctx->ny;
    k_cns_faces<<<(nfi + bs - 1) / bs, bs, 0, ctx->stream>>>(A, 0);
    k_cns_faces<<<(nfj + bs - 1) / bs, bs, 0, ctx->stream>>>(A, 1);
    ctx->launches += 7;
    return check(ctx, "convert_ns");
}

}  // namespace hyb
