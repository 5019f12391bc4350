// hyb_noalloc.cu -- DETFP on caller-owned device memory, with no allocation.
//
// Who needs it: a host whose device memory is owned by someone else -- a
// CUDA Fortran / OpenACC host that keeps FRD and S_GKUA as its own device
// arrays, or a process whose device memory is fully reserved by another
// framework's pooling allocator -- and so cannot let this library call
// cudaMalloc.  Such a caller passes its device FRD and gets S_GKUA / CF back
// in its own device arrays.
//
// The velocity-slice partial sums live in the file-scope device array
// g_detfp_scratch (16 MiB, HYB_NOALLOC_MAX_CELLS cells at one slice).  Host
// code cannot pass the symbol itself to a kernel: every call looks up its
// address with cudaGetSymbolAddress on the current device and context (no
// allocation; the first call on a device also loads this library's device
// code there, so make it before any stream capture).  All calls share the
// array; every partial is written before it is read, so nothing needs
// clearing between calls, but calls that overlap on the GPU (different
// streams) race on it.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "hyb_common.cuh"

namespace {

constexpr size_t kScratchDoubles = (size_t)HYB_NOALLOC_MAX_CELLS * 10;
static __device__ __align__(256) double g_detfp_scratch[kScratchDoubles];

// moments of one velocity slice for one interior cell per thread (FRD layout
// FRD(NRD,-3:nx+3,-3:ny+3,NVI,NVJ), GaussLegendre sums of GKUA_DETFP.f90:315-345);
// the cells i fastest along a 1-D grid, the slice along grid z
__global__ void k_detfp_na_part(const double *__restrict__ frd, int nx, int ny, int nvi, int nvj, int vs,
                                const double *__restrict__ vi, const double *__restrict__ vj,
                                const double *__restrict__ wi, const double *__restrict__ wj,
                                double *__restrict__ part) {
    const size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= (size_t)(nx - 1) * (ny - 1)) return;
    const int i = (int)(cell % (nx - 1)) + 1, j = (int)(cell / (nx - 1)) + 1, slice = blockIdx.z;
    const int pw = nx + 7;
    const size_t P = (size_t)(nx + 7) * (ny + 7);
    const size_t ix = (size_t)(i + 3) + (size_t)pw * (j + 3);
    const int jv0 = (int)((long long)nvj * slice / vs), jv1 = (int)((long long)nvj * (slice + 1) / vs);
    double s[10];
#pragma unroll
    for (int k = 0; k < 10; k++) s[k] = 0.0;
    for (int jv = jv0; jv < jv1; jv++) {
        const double vy = vj[jv], wy = wj[jv];
        for (int iv = 0; iv < nvi; iv++) {
            const double vx = vi[iv], w = wi[iv] * wy;
            const size_t v = (size_t)iv + (size_t)nvi * jv;
            // two scalar loads: the caller's FRD needs only double alignment
            const double g = frd[(v * P + ix) * 2], h = frd[(v * P + ix) * 2 + 1];
            const double vxg = vx * g, vyg = vy * g, vx2g = vx * vxg, vy2g = vy * vyg;
            const double b4 = h + vx2g + vy2g;
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
    const size_t ncell = (size_t)(nx - 1) * (ny - 1);
    const size_t c = (size_t)(i - 1) + (size_t)(nx - 1) * (j - 1);
#pragma unroll
    for (int k = 0; k < 10; k++) part[((size_t)slice * 10 + k) * ncell + c] = s[k];
}

// slices added in fixed order, then DETFP's primitive conversion and CF
// (GKUA_DETFP.f90:59-92)
__global__ void k_detfp_na_finish(int nx, int ny, int vs, const double *__restrict__ part, double cfc,
                                  double x1s, double r00, double t00, double *__restrict__ s_gkua,
                                  double *__restrict__ cf) {
    const size_t ncell = (size_t)(nx - 1) * (ny - 1);
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int i = (int)(c % (nx - 1)) + 1, j = (int)(c / (nx - 1)) + 1;
    double s[10];
    for (int k = 0; k < 10; k++) {
        double x = 0.0;
        for (int sl = 0; sl < vs; sl++) x += part[((size_t)sl * 10 + k) * ncell + c];
        s[k] = x;
    }
    double S1 = s[0], S4 = s[3], S5 = s[4], S6 = s[5], S7 = s[6];
    double ron = S1;
    if (ron <= 0.) ron = r00;
    double u = s[1] / ron, vv = s[2] / ron;
    double us1 = u * u, vs1 = vv * vv, suv = us1 + vs1;
    double tt = (S4 - ron * suv) / (1.5 * ron);
    if (tt <= 0.) tt = t00;
    const size_t ix = (size_t)(i + 3) + (size_t)(nx + 7) * (j + 3);
    double *S = s_gkua + ix * HYB_NSUM;
    S[0] = S1;
    S[1] = u;
    S[2] = vv;
    S[3] = tt;
    S[4] = (S5 - ron * us1) * 2.;
    S[5] = (S6 - ron * vs1) * 2.;
    S[6] = (S7 - ron * u * vv) * 2.;
    S[7] = s[7] - 2. * u * S5 - 2. * vv * S7 + ron * u * (suv - 1.5 * tt);
    S[8] = s[8] - 2. * vv * S6 - 2. * u * S7 + ron * vv * (suv - 1.5 * tt);
    S[9] = s[9] * 2.;
    S[10] = 0.0;
    if (cf) cf[hyb_c2(nx, i, j)] = (x1s <= (double)1.e-8f) ? cfc * S1 : cfc * S1 * pow(tt, x1s);
}

// device address of the scratch array in the current device and context,
// looked up on every call (a cached address could belong to a context that
// was reset or to another context of the same device)
int scratch_for_current_device(double **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HYB_ERR_NODEVICE;
    double *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&p, g_detfp_scratch);
    if (e != cudaSuccess || p == nullptr) return HYB_ERR_CUDA;
    *out = p;
    return HYB_OK;
}

// every device array is read or written as doubles
inline bool double_aligned(const void *p) { return ((uintptr_t)p & (sizeof(double) - 1)) == 0; }

}  // namespace

extern "C" int hyb_detfp_noalloc(int nx, int ny, int nvi, int nvj, const double *frd_dev, const double *vi_dev,
                                 const double *vj_dev, const double *wi_dev, const double *wj_dev,
                                 const hyb_params *p, double *s_gkua_dev, double *cf_dev, void *stream) {
    if (nx < 3 || ny < 3 || nvi < 1 || nvj < 1 || !frd_dev || !vi_dev || !vj_dev || !wi_dev || !wj_dev || !p ||
        !s_gkua_dev)
        return HYB_ERR_INVALID;
    // checked before any CUDA call: a misaligned pointer would fault the
    // caller's context instead of returning
    if (!double_aligned(frd_dev) || !double_aligned(vi_dev) || !double_aligned(vj_dev) || !double_aligned(wi_dev) ||
        !double_aligned(wj_dev) || !double_aligned(s_gkua_dev) || (cf_dev && !double_aligned(cf_dev)))
        return HYB_ERR_INVALID;
    const size_t ncell = (size_t)(nx - 1) * (ny - 1);
    if (ncell > (size_t)HYB_NOALLOC_MAX_CELLS) return HYB_ERR_UNSUPPORTED;   // scratch would not hold one slice
    double *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != HYB_OK) return rc;
    // velocity slices: as many as fit the scratch, at most 32, at most nvj
    size_t fit = kScratchDoubles / (10 * ncell);
    int vs = (int)(fit < 32 ? fit : 32);
    if (vs > nvj) vs = nvj;
    if (vs < 1) vs = 1;
    cudaStream_t st = (cudaStream_t)stream;
    dim3 blk(128), grd((unsigned)((ncell + 127) / 128), 1, (unsigned)vs);
    k_detfp_na_part<<<grd, blk, 0, st>>>(frd_dev, nx, ny, nvi, nvj, vs, vi_dev, vj_dev, wi_dev, wj_dev, scratch);
    if (cudaGetLastError() != cudaSuccess) return HYB_ERR_CUDA;
    k_detfp_na_finish<<<(unsigned)((ncell + 255) / 256), 256, 0, st>>>(nx, ny, vs, scratch, p->cfc, p->x1s, p->r00,
                                                                       p->t00, s_gkua_dev, cf_dev);
    if (cudaGetLastError() != cudaSuccess) return HYB_ERR_CUDA;
    return HYB_OK;
}
