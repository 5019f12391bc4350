// hyb_kinetic.cu -- sm_103a kernels of the discrete-velocity Shakhov step.
//
//   k_wall      diffuse-wall slot values and n_w        GKUA_boundary_wall,
//               (GKUA_boundary.f90:49-100, GKUA_wall_functions.f90:1-199)
//   k_moments   velocity moments + primitive conversion + CF (DETFP,
//               GKUA_DETFP.f90:4-151, 288-363)
//   k_residual  moments 1-4 of the stored RHS, rms / max (DETFP_res,
//               GKUA_DETFP_RES.f90:4-136)
//   k_init      uniform Maxwellian (GKUA_sudufenbu.f90:22-42)
//
// The fused LU-SGS sweep kernel is in hyb_sweep.cu.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include <cooperative_groups.h>
#include <string.h>

#include "hyb_common.cuh"
#include "hyb_device.cuh"

namespace hyb {

// ---------------------------------------------------------------------------
// diffuse wall: one cluster of WALL_CL CTAs per wall face cell, all wall
// faces in one launch; each CTA takes a contiguous share of the velocities,
// the n_w flux balance adds the CTAs' partial sums in rank order through
// distributed shared memory
// ---------------------------------------------------------------------------
constexpr int WALL_CL = 8;

// the wall faces of one launch: face cells of face q are the global face
// cells first[q] .. first[q+1]-1; on_scan: wall at a scan-axis end (cells
// along b), else at a march end; hi: the high end
template <typename real> struct WallSet {
    real *fw[4];
    const double *wd[4];
    int on_scan[4], hi[4], first[5], nface;
};

template <typename real> struct WallArgs {
    const real *f;
    WallSet<real> W;
    const double *vx, *vy, *w;
    int nvi, nv, Na, Nb, PA;
};

// face cell kg (over all wall faces) of the cluster's context
template <typename real>
__device__ __forceinline__ void wall_body(const real *__restrict__ f, const WallSet<real> &W,
                                          const double *__restrict__ vx, const double *__restrict__ vy,
                                          const double *__restrict__ w, int nvi, int nv, int Na, int Nb, int PA,
                                          int kg) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    // the face of kg (constant indices: the set stays in parameter space)
    real *fw = W.fw[0];
    const double *wd = W.wd[0];
    int on_scan = W.on_scan[0], hi = W.hi[0], k0 = W.first[0];
#pragma unroll
    for (int u = 1; u < 4; u++)
        if (u < W.nface && kg >= W.first[u]) {
            fw = W.fw[u];
            wd = W.wd[u];
            on_scan = W.on_scan[u];
            hi = W.hi[u];
            k0 = W.first[u];
        }
    const int k = kg - k0;                // face cell (0-based, face order)
    const int per = (nv + WALL_CL - 1) / WALL_CL, vb = rank * per, ve = min(nv, vb + per);
    // wall data: [k][6] = u, v, t, swnx, swny, step
    const double uw = wd[k * 6 + 0], vw = wd[k * 6 + 1], tw = wd[k * 6 + 2];
    const float itw_f = (float)(1.0 / tw), ipt_f = (float)(1.0 / (HYB_PI * tw));
    const double swnx = wd[k * 6 + 3], swny = wd[k * 6 + 4], step = wd[k * 6 + 5];
    // cell offsets of the two cells next to the wall
    size_t cp, cp1, nslot;
    if (on_scan) {   // cells a = 1,2 (lo) or Na, Na-1 (hi) at row b = k+1
        int a0 = hi ? Na : 1, a1 = hi ? Na - 1 : 2;
        cp = (size_t)k * PA + (a0 - 1);
        cp1 = (size_t)k * PA + (a1 - 1);
        nslot = Nb;
    } else {
        int b0 = hi ? Nb : 1, b1 = hi ? Nb - 1 : 2;
        cp = (size_t)(b0 - 1) * PA + k;
        cp1 = (size_t)(b1 - 1) * PA + k;
        nslot = PA;
    }
    const size_t rs = (size_t)Nb * PA;
    extern __shared__ double emax[];   // exp(-c^2/Tw)/(pi Tw) of this CTA's velocities
    double s0 = 0.0, s1 = 0.0;
    for (int v = vb + threadIdx.x; v < ve; v += blockDim.x) {
        const real *fv = f + (size_t)v * 2 * rs;
        double vxx = vx[v % nvi], vyy = vy[v / nvi];
        double wt = w[v];
        double tG = 0;
        for (int r = 0; r < 2; r++) {
            real fp = fv[r * rs + cp];
            real tt = (-fv[r * rs + cp1] + real(3.0) * fp) * real(0.5);
            if (tt <= real(0)) tt = fp;
            if (tt >= real(1.5) * fp) tt = real(1.5) * fp;
            fw[((size_t)v * 2 + r) * nslot + k] = tt;
            if (r == 0) tG = (double)tt;
        }
        double vnw = ((vxx - uw) * swnx + (vyy - vw) * swny) * step;
        double vnn = (vnw - fabs(vnw)) / 2.0;
        s0 += wt * (vnn * tG);
        double em;
        if constexpr (sizeof(real) == 4) {
            // FP32 distribution: the wall Maxwellian in FP32 (it is stored in
            // FP32); its weighted sum below stays FP64
            const float dx = (float)(vxx - uw), dy = (float)(vyy - vw);
            em = (double)(expf(-(dx * dx + dy * dy) * itw_f) * ipt_f);
        } else {
            const double cv = (vxx - uw) * (vxx - uw) + (vyy - vw) * (vyy - vw);
            em = exp(-cv / tw) / (HYB_PI * tw);
        }
        emax[v - vb] = em;
        double fb = (vnw + fabs(vnw)) / 2.0 * em;
        s1 += wt * fb;
    }
    __shared__ double r0[256], r1[256];
    __shared__ double part[2], nw_sh;
    r0[threadIdx.x] = s0;
    r1[threadIdx.x] = s1;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            r0[threadIdx.x] += r0[threadIdx.x + s];
            r1[threadIdx.x] += r1[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[0] = r0[0];
        part[1] = r1[0];
    }
    cl.sync();
    if (threadIdx.x == 0) {
        double t0 = 0.0, t1 = 0.0;
        for (int q = 0; q < WALL_CL; q++) {
            const double *pq = cl.map_shared_rank(part, q);
            t0 += pq[0];
            t1 += pq[1];
        }
        nw_sh = -t0 / t1;
    }
    cl.sync();   // every CTA has read the partials before any exits
    const double nwall = nw_sh;
    for (int v = vb + threadIdx.x; v < ve; v += blockDim.x) {
        double vxx = vx[v % nvi], vyy = vy[v / nvi];
        double vnw = ((vxx - uw) * swnx + (vyy - vw) * swny) * step;
        if (vnw >= 0.0) {
            double gg = nwall * emax[v - vb];   // each thread reads its own entries
            fw[((size_t)v * 2 + 0) * nslot + k] = (real)gg;
            fw[((size_t)v * 2 + 1) * nslot + k] = (real)(tw * gg / 2.0);
        }
    }
}

template <typename real>
__global__ void __cluster_dims__(WALL_CL, 1, 1) __launch_bounds__(256)
    k_wall(const real *__restrict__ f, WallSet<real> W, const double *__restrict__ vx,
           const double *__restrict__ vy, const double *__restrict__ w, int nvi, int nv, int Na, int Nb, int PA) {
    wall_body<real>(f, W, vx, vy, w, nvi, nv, Na, Nb, PA, blockIdx.x / WALL_CL);
}

// many contexts: cluster i handles face cell work[i].y of context work[i].x
template <typename real>
__global__ void __cluster_dims__(WALL_CL, 1, 1) __launch_bounds__(256)
    k_wall_batch(const WallArgs<real> *__restrict__ args, const int2 *__restrict__ work) {
    __shared__ WallArgs<real> Wa;
    const int2 wk = work[blockIdx.x / WALL_CL];
    if (threadIdx.x == 0) Wa = args[wk.x];
    __syncthreads();
    wall_body<real>(Wa.f, Wa.W, Wa.vx, Wa.vy, Wa.w, Wa.nvi, Wa.nv, Wa.Na, Wa.Nb, Wa.PA, wk.y);
}

// ---------------------------------------------------------------------------
// moments.  k_moments_part: one CTA per (march row b, velocity slice); the
// slice's velocity rows stream through an NST-stage shared-memory ring filled
// by cp.async.bulk (full/empty mbarrier pairs), each thread accumulates MC
// cells.  Mixed mode sums blocks of 8 velocities in plain FP32 and adds the
// block sums with Kahan compensation (the block rounding is of the order of
// the FP32 inputs' own); FP64 mode accumulates in FP64.  k_moments_finish
// adds the slices in fixed order (float-float in mixed mode, converted to
// FP64 once per cell) and applies DETFP's primitive conversion.
// ---------------------------------------------------------------------------
struct MomArgs {
    const void *f;
    double *part;       // [VS][10][Nb*PA]: double (FP64), float2 Kahan pair (mixed)
    double *S;          // [NSUM][(nx+3)(ny+3)]
    double *CF;         // [(nx+3)(ny+3)]
    void *eqp;          // [8][Nb*PA] real
    const double *vx, *vy, *w;
    int nvi, nv, Na, Nb, PA, nx, ny, scan_is_j, vs, nloc_max, *err;
    double cfc, cpr, x1s, r00, t00;
    long long spin;     // limit of the bounded waits, SM clocks
};

constexpr int MOM_NST = 3;

template <typename real> struct KahanAcc;
template <> struct KahanAcc<double> {
    double s;
    __device__ void zero() { s = 0; }
    __device__ void add(double x) { s += x; }
};
template <> struct KahanAcc<float> {
    float s, c;
    __device__ void zero() { s = 0.f; c = 0.f; }
    __device__ void add(float x) {
        float y = x - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// Per-slice partial sums.  FP64 mode stores a double per (slice, moment,
// cell).  FP32 mode stores the slice's Kahan pair as a float2 (s, -c) whose
// value is x + y: the slices are then added in float-float arithmetic and
// converted to double once per cell, which keeps float-to-double conversions
// (2 lanes per clock per SM on GB300) out of the per-slice work.
template <typename real> struct SliceSum;
template <> struct SliceSum<double> {
    double a;
    __device__ void zero() { a = 0.0; }
    __device__ void add_part(const double *part, size_t i) { a += part[i]; }
    __device__ void add_sum(const SliceSum &o) { a += o.a; }
    __device__ double value() const { return a; }
};
template <> struct SliceSum<float> {
    float hi, lo;
    __device__ void zero() { hi = lo = 0.f; }
    // (hi, lo) += (x + y): two-sum of the leading parts, then renormalise
    __device__ void add2(float x, float y) {
        const float t = hi + x, bp = t - hi;
        float e = (hi - (t - bp)) + (x - bp);
        e += lo + y;
        hi = t + e;
        lo = e - (hi - t);
    }
    __device__ void add_part(const double *part, size_t i) {
        const float2 p = reinterpret_cast<const float2 *>(part)[i];
        add2(p.x, p.y);
    }
    __device__ void add_sum(const SliceSum &o) { add2(o.hi, o.lo); }
    __device__ double value() const { return (double)hi + (double)lo; }
};

// Slice sums of a block's cells (blocks of 256 threads).  The block takes
// 256 / lpc consecutive cells; thread (sub, c) adds slices sub, sub + lpc, ...
// of cell c, so the threads of a warp read consecutive cells of one slice,
// and the lpc partial sums of a cell are then folded pairwise in shared
// memory in a fixed order.  The threads with own set hold the cell's sums.
template <typename real, int NM>
__device__ __forceinline__ void slice_fold(const MomArgs &M, int lpc, int blk, SliceSum<real> (&acc)[NM],
                                           size_t &cell, bool &own) {
    __shared__ SliceSum<real> red[NM][256];
    const size_t ncell = (size_t)M.Nb * M.PA;
    const int cb = 256 / lpc, c = threadIdx.x % cb, sub = threadIdx.x / cb;
    cell = (size_t)blk * cb + c;
    const bool ok = cell < ncell && (int)(cell % M.PA) < M.Na;
#pragma unroll
    for (int q = 0; q < NM; q++) acc[q].zero();
    if (ok)
        for (int sl = sub; sl < M.vs; sl += lpc)
#pragma unroll
            for (int q = 0; q < NM; q++) acc[q].add_part(M.part, ((size_t)sl * NM + q) * ncell + cell);
    if (lpc > 1) {
#pragma unroll
        for (int q = 0; q < NM; q++) red[q][threadIdx.x] = acc[q];
        for (int off = lpc >> 1; off > 0; off >>= 1) {
            __syncthreads();
            if (sub < off)
#pragma unroll
                for (int q = 0; q < NM; q++) {
                    acc[q].add_sum(red[q][threadIdx.x + off * cb]);
                    red[q][threadIdx.x] = acc[q];
                }
        }
    }
    own = ok && sub == 0;
}
template <typename real> __device__ __forceinline__ void store_part(double *part, size_t i, KahanAcc<real> &k);
template <> __device__ __forceinline__ void store_part<double>(double *part, size_t i, KahanAcc<double> &k) {
    part[i] = k.s;
}
template <> __device__ __forceinline__ void store_part<float>(double *part, size_t i, KahanAcc<float> &k) {
    reinterpret_cast<float2 *>(part)[i] = make_float2(k.s, -k.c);
}

// velocities per stage slot: one mbarrier wait, one refill and one empty
// arrival per slot; 16 KB slots at PA = 512 in both precisions
template <typename real> struct MomVps { static constexpr int v = 4; };
template <> struct MomVps<double> { static constexpr int v = 2; };

template <typename real>
__host__ __device__ inline size_t mom_smem_bytes(int PA, int nloc_max) {
    size_t b = 256;                                                   // mbarriers
    b += ((size_t)3 * nloc_max * sizeof(real) + 127) / 128 * 128;     // vx, vy, w per velocity
    b += (size_t)MOM_NST * MomVps<real>::v * 2 * PA * sizeof(real);   // stage ring
    return b;
}

// NM = 10: the DETFP moments; NM = 4: moments 1-4 only (the residual of a
// stored RHS, DETFP_res); NM = 9: the higher-order moments HOT_GKUA(1:6),
// HOQ_GKUA(1:3) of IntegralGaussHermite (GKUA_DETFP.f90:217-229)
template <typename real, int MC, int NM>
__device__ __forceinline__ void moments_body(const MomArgs &M, int bidx, int slice) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int VPS = MomVps<real>::v;
    constexpr int FLUSH = 8 / VPS;                  // slots per block of 8 velocities
    const int PA = M.PA, t = threadIdx.x, TPV = blockDim.x;
    const int b = bidx + 1;
    const int a0 = t * MC + 1;
    const bool act = a0 <= M.Na;
    const int nvi = M.nvi, nvj = M.nv / M.nvi;
    const int jv0 = (int)((long long)nvj * slice / M.vs), jv1 = (int)((long long)nvj * (slice + 1) / M.vs);
    const int v0 = jv0 * nvi, nloc = (jv1 - jv0) * nvi;
    const int nslot = (nloc + VPS - 1) / VPS;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw);
    uint64_t *empty = full + MOM_NST;
    real *sv = reinterpret_cast<real *>(smem_raw + 256);             // [3][nloc]
    real *stage = reinterpret_cast<real *>(smem_raw + 256 + ((size_t)3 * M.nloc_max * sizeof(real) + 127) / 128 * 128);
    const size_t rs = (size_t)M.Nb * PA;
    const real *f = (const real *)M.f;
    const uint32_t row_bytes = (uint32_t)(PA * sizeof(real));
    const int nwarp = TPV >> 5, lane = t & 31;
    for (int k = t; k < nloc; k += TPV) {
        sv[k] = (real)M.vx[k % nvi];
        sv[nloc + k] = (real)M.vy[jv0 + k / nvi];
        sv[2 * nloc + k] = (real)M.w[(size_t)v0 + k];
    }
    if (t == 0) {
        for (int k = 0; k < MOM_NST; k++) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], nwarp);
        }
        fence_async_shared();
    }
    __syncthreads();
    auto issue = [&](int n) {
        const int k = n % MOM_NST;
        const int cnt = min(VPS, nloc - n * VPS);
        mbar_arrive_expect_tx(&full[k], 2 * row_bytes * cnt);
        for (int u = 0; u < cnt; u++) {
            const real *src = f + (size_t)(v0 + n * VPS + u) * 2 * rs + (size_t)(b - 1) * PA;
            real *dst = stage + ((size_t)k * VPS + u) * 2 * PA;
            bulk_g2s(dst, src, row_bytes, &full[k]);
            bulk_g2s(dst + PA, src + rs, row_bytes, &full[k]);
        }
    };
    int issued = 0;   // slots issued (thread 0)
    if (t == 0)
        for (; issued < MOM_NST - 1 && issued < nslot; issued++) issue(issued);
    // plain sums over blocks of 8 velocities, compensated sums of the blocks
    KahanAcc<real> ks[NM][MC];
    real blk[NM][MC];
#pragma unroll
    for (int q = 0; q < NM; q++)
#pragma unroll
        for (int c = 0; c < MC; c++) {
            ks[q][c].zero();
            blk[q][c] = real(0);
        }
    // A wait that runs out clears the thread's ok: it stops waiting (and
    // thread 0 stops issuing), and every thread still runs each slot's warp
    // sync and empty arrival, so no lane leaves a warp barrier early.
    bool ok = true;
    for (int n = 0; n < nslot; n++) {
        const int k = n % MOM_NST;
        // refill the slot freed by slot n-1 with slot n+NST-1
        if (t == 0 && ok && n + MOM_NST - 1 < nslot) {
            if (n >= 1 && !mbar_wait_bounded(&empty[(n - 1) % MOM_NST], (uint32_t)(((n - 1) / MOM_NST) & 1), M.spin))
                ok = false;
            else
                issue(issued++);
        }
        if (ok && !mbar_wait_bounded(&full[k], (uint32_t)((n / MOM_NST) & 1), M.spin)) ok = false;
        if (act && ok) {
            const int cnt = min(VPS, nloc - n * VPS);
            const real *gs = stage + (size_t)k * VPS * 2 * PA + (a0 - 1);
#pragma unroll
            for (int u = 0; u < VPS; u++) {
                if (u < cnt) {
                    const int lv = n * VPS + u;
                    const real vx = sv[lv], vy = sv[nloc + lv], wv = sv[2 * nloc + lv];
                    const real *g = gs + (size_t)u * 2 * PA;
                    real gg[MC], hh[MC];
#pragma unroll
                    for (int c = 0; c < MC; c++) { gg[c] = g[c]; hh[c] = g[PA + c]; }
                    const real wx = wv * vx, wy = wv * vy, wxy = wx * vy, c2 = vx * vx + vy * vy;
                    if constexpr (NM == 9) {
                        const real t1 = wx * vx, t2 = wy * vy;   // w vx^2, w vy^2
                        const real t1x = t1 * vx, t1y = t1 * vy, t2x = t2 * vx, t2y = t2 * vy;
#pragma unroll
                        for (int c = 0; c < MC; c++) {
                            const real e = gg[c] * c2 + hh[c];     // G c^2 + H
                            blk[0][c] += t1x * gg[c];
                            blk[1][c] += t1y * gg[c];
                            blk[2][c] += t2x * gg[c];
                            blk[3][c] += t2y * gg[c];
                            blk[4][c] += wx * hh[c];
                            blk[5][c] += wy * hh[c];
                            blk[6][c] += t1 * e;
                            blk[7][c] += wxy * e;
                            blk[8][c] += t2 * e;
                        }
                    } else {
#pragma unroll
                        for (int c = 0; c < MC; c++) {
                            const real wg = wv * gg[c];
                            const real b4 = hh[c] + c2 * gg[c];
                            blk[0][c] += wg;
                            blk[1][c] += wx * gg[c];
                            blk[2][c] += wy * gg[c];
                            blk[3][c] += wv * b4;
                            if constexpr (NM > 4) {
                                blk[4][c] += wx * (vx * gg[c]);
                                blk[5][c] += wy * (vy * gg[c]);
                                blk[6][c] += wxy * gg[c];
                                blk[7][c] += wx * b4;
                                blk[8][c] += wy * b4;
                                blk[9][c] += wv * hh[c];
                            }
                        }
                    }
                }
            }
            if ((n % FLUSH) == FLUSH - 1 || n == nslot - 1) {
#pragma unroll
                for (int q = 0; q < NM; q++)
#pragma unroll
                    for (int c = 0; c < MC; c++) {
                        ks[q][c].add(blk[q][c]);
                        blk[q][c] = real(0);
                    }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[k]);
    }
    if (__syncthreads_or(!ok)) {
        if (t == 0) {
            atomicExch(M.err, HYB_ERR_TIMEOUT);
            // the last NST issued slots may still be in flight: wait (bounded)
            for (int n = issued > MOM_NST ? issued - MOM_NST : 0; n < issued; n++)
                mbar_wait_bounded(&full[n % MOM_NST], (uint32_t)((n / MOM_NST) & 1), M.spin);
        }
        return;
    }
    if (!act) return;
    const size_t ncell = (size_t)M.Nb * PA;
    const size_t cell0 = (size_t)(b - 1) * PA + (a0 - 1);
#pragma unroll
    for (int q = 0; q < NM; q++)
#pragma unroll
        for (int c = 0; c < MC; c++) store_part<real>(M.part, ((size_t)slice * NM + q) * ncell + cell0 + c, ks[q][c]);
}

// ---- FP32 moment pass, two cells per thread, packed pairs -------------------
// The DETFP moments (NM = 10) or moments 1-4 of a stored RHS (NM = 4) of FP32
// distributions.  Same ring and slices as moments_body, plain FP32 sums over
// blocks of 16 velocities (8 there) added into Kahan sums; the arithmetic
// differs in form only:
// * the weight of each moment per velocity (w, w vx, w vy, vx^2 + vy^2,
//   w vx^2, w vy^2, w vx vy) is formed once per CTA and stored twice over, so
//   that a packed FP32 pair reads it from shared memory as a register pair;
// * the two cells of a thread are summed as one packed pair, one FFMA2 per
//   moment and velocity (w vx^2 G is (w vx^2) G here, w vx (vx G) there: FP32
//   rounding of the products differs, the sums are the same moments).
// The Kahan terms stay in registers: at 80 registers (three CTAs per SM) a
// few of them spill around the block flushes, which measured faster than
// keeping the compensations in shared memory (0.54 against 0.75 ms on the
// 128x512 x 64^2 Couette case); flushing every 16 velocities instead of 8
// halves that spill traffic (0.544 -> 0.518 ms).
constexpr int MOMF2_COEF = 16;   // floats per velocity in the weight table

__host__ __device__ inline size_t mom_f2_coef_bytes(int nloc_max) {
    return ((size_t)MOMF2_COEF * nloc_max * sizeof(float) + 127) / 128 * 128;
}
__host__ __device__ inline size_t mom_f2_smem_bytes(int PA, int nloc_max) {
    return 256 + mom_f2_coef_bytes(nloc_max) + (size_t)MOM_NST * MomVps<float>::v * 2 * PA * sizeof(float);
}

__device__ __forceinline__ float2 m2_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 m2_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 m2_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

template <int NM>
__device__ __forceinline__ void moments_body_f2(const MomArgs &M, int bidx, int slice) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int VPS = MomVps<float>::v;
    constexpr int FLUSH = 16 / VPS;                  // slots per block of 16 velocities
    const int PA = M.PA, t = threadIdx.x, TPV = blockDim.x;
    const int b = bidx + 1;
    const int a0 = t * 2 + 1;
    const bool act = a0 <= M.Na;
    const int nvi = M.nvi, nvj = M.nv / M.nvi;
    const int jv0 = (int)((long long)nvj * slice / M.vs), jv1 = (int)((long long)nvj * (slice + 1) / M.vs);
    const int v0 = jv0 * nvi, nloc = (jv1 - jv0) * nvi;
    const int nslot = (nloc + VPS - 1) / VPS;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw);
    uint64_t *empty = full + MOM_NST;
    float *coef = reinterpret_cast<float *>(smem_raw + 256);          // [nloc][16]
    float *stage = reinterpret_cast<float *>(smem_raw + 256 + mom_f2_coef_bytes(M.nloc_max));
    const size_t rs = (size_t)M.Nb * PA;
    const float *f = (const float *)M.f;
    const uint32_t row_bytes = (uint32_t)(PA * sizeof(float));
    const int nwarp = TPV >> 5, lane = t & 31;
    for (int k = t; k < nloc; k += TPV) {
        const float vx = (float)M.vx[k % nvi], vy = (float)M.vy[jv0 + k / nvi], wv = (float)M.w[(size_t)v0 + k];
        const float wx = wv * vx, wy = wv * vy;
        float4 *d = reinterpret_cast<float4 *>(coef + (size_t)k * MOMF2_COEF);
        const float c2 = vx * vx + vy * vy, wxx = wx * vx, wyy = wy * vy, wxy = wx * vy;
        d[0] = make_float4(wv, wv, wx, wx);
        d[1] = make_float4(wy, wy, c2, c2);
        d[2] = make_float4(wxx, wxx, wyy, wyy);
        d[3] = make_float4(wxy, wxy, 0.f, 0.f);
    }
    if (t == 0) {
        for (int k = 0; k < MOM_NST; k++) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], nwarp);
        }
        fence_async_shared();
    }
    __syncthreads();
    auto issue = [&](int n) {
        const int k = n % MOM_NST;
        const int cnt = min(VPS, nloc - n * VPS);
        mbar_arrive_expect_tx(&full[k], 2 * row_bytes * cnt);
        for (int u = 0; u < cnt; u++) {
            const float *src = f + (size_t)(v0 + n * VPS + u) * 2 * rs + (size_t)(b - 1) * PA;
            float *dst = stage + ((size_t)k * VPS + u) * 2 * PA;
            bulk_g2s(dst, src, row_bytes, &full[k]);
            bulk_g2s(dst + PA, src + rs, row_bytes, &full[k]);
        }
    };
    int issued = 0;   // slots issued (thread 0)
    if (t == 0)
        for (; issued < MOM_NST - 1 && issued < nslot; issued++) issue(issued);
    // plain sums over blocks of 16 velocities, Kahan sums of the blocks
    float2 blk[NM], ks[NM], kc[NM];
#pragma unroll
    for (int q = 0; q < NM; q++) blk[q] = ks[q] = kc[q] = make_float2(0.f, 0.f);
    bool ok = true;
    for (int n = 0; n < nslot; n++) {
        const int k = n % MOM_NST;
        if (t == 0 && ok && n + MOM_NST - 1 < nslot) {
            if (n >= 1 && !mbar_wait_bounded(&empty[(n - 1) % MOM_NST], (uint32_t)(((n - 1) / MOM_NST) & 1), M.spin))
                ok = false;
            else
                issue(issued++);
        }
        if (ok && !mbar_wait_bounded(&full[k], (uint32_t)((n / MOM_NST) & 1), M.spin)) ok = false;
        if (act && ok) {
            const int cnt = min(VPS, nloc - n * VPS);
            const float *gs = stage + (size_t)k * VPS * 2 * PA + (a0 - 1);
#pragma unroll
            for (int u = 0; u < VPS; u++) {
                if (u < cnt) {
                    const float4 *cw = reinterpret_cast<const float4 *>(coef + (size_t)(n * VPS + u) * MOMF2_COEF);
                    const float4 c0 = cw[0], c1 = cw[1];
                    const float2 wv = make_float2(c0.x, c0.y), wx = make_float2(c0.z, c0.w);
                    const float2 wy = make_float2(c1.x, c1.y), c2 = make_float2(c1.z, c1.w);
                    const float2 g = *reinterpret_cast<const float2 *>(gs + (size_t)u * 2 * PA);
                    const float2 h = *reinterpret_cast<const float2 *>(gs + (size_t)u * 2 * PA + PA);
                    const float2 b4 = m2_fma(c2, g, h);                     // H + c^2 G
                    blk[0] = m2_fma(wv, g, blk[0]);
                    blk[1] = m2_fma(wx, g, blk[1]);
                    blk[2] = m2_fma(wy, g, blk[2]);
                    blk[3] = m2_fma(wv, b4, blk[3]);
                    if constexpr (NM > 4) {
                        const float4 c2v = cw[2], c3v = cw[3];
                        blk[4] = m2_fma(make_float2(c2v.x, c2v.y), g, blk[4]);
                        blk[5] = m2_fma(make_float2(c2v.z, c2v.w), g, blk[5]);
                        blk[6] = m2_fma(make_float2(c3v.x, c3v.y), g, blk[6]);
                        blk[7] = m2_fma(wx, b4, blk[7]);
                        blk[8] = m2_fma(wy, b4, blk[8]);
                        blk[9] = m2_fma(wv, h, blk[9]);
                    }
                }
            }
            if ((n % FLUSH) == FLUSH - 1 || n == nslot - 1) {
#pragma unroll
                for (int q = 0; q < NM; q++) {
                    const float2 y = m2_sub(blk[q], kc[q]);
                    const float2 s2 = m2_add(ks[q], y);
                    kc[q] = m2_sub(m2_sub(s2, ks[q]), y);
                    ks[q] = s2;
                    blk[q] = make_float2(0.f, 0.f);
                }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[k]);
    }
    if (__syncthreads_or(!ok)) {
        if (t == 0) {
            atomicExch(M.err, HYB_ERR_TIMEOUT);
            for (int n = issued > MOM_NST ? issued - MOM_NST : 0; n < issued; n++)
                mbar_wait_bounded(&full[n % MOM_NST], (uint32_t)((n / MOM_NST) & 1), M.spin);
        }
        return;
    }
    if (!act) return;
    const size_t ncell = (size_t)M.Nb * PA;
    const size_t cell0 = (size_t)(b - 1) * PA + (a0 - 1);    // even: the two cells' pairs are one 16-byte store
#pragma unroll
    for (int q = 0; q < NM; q++)
        *reinterpret_cast<float4 *>(reinterpret_cast<float2 *>(M.part) + ((size_t)slice * NM + q) * ncell + cell0) =
            make_float4(ks[q].x, -kc[q].x, ks[q].y, -kc[q].y);
}

template <int NM>
__global__ void __launch_bounds__(256, 3) k_moments_f2(MomArgs M) {
    moments_body_f2<NM>(M, blockIdx.x, blockIdx.y);
}

// many contexts in one launch: CTA i takes march row work[i].y and velocity
// slice work[i].z of context work[i].x
template <int NM>
__global__ void __launch_bounds__(256, 3) k_moments_f2_batch(const MomArgs *__restrict__ args,
                                                            const int4 *__restrict__ work) {
    __shared__ MomArgs Ms;
    const int4 w = work[blockIdx.x];
    if (threadIdx.x == 0) Ms = args[w.x];
    __syncthreads();
    moments_body_f2<NM>(Ms, w.y, w.z);
}

// the packed FP32 pass takes FP32 rows of up to 512 cells at two cells per thread
static bool mom_f2_ok(int precision, int mc, int tpv) { return precision != HYB_PREC_FP64 && mc == 2 && tpv <= 256; }

// NARROW: CTAs of at most 256 threads, three per SM (80 registers); FP32
// rows of up to 512 cells take it, wider rows and FP64 keep 512 threads
template <typename real, int MC, int NM, bool NARROW>
__global__ void __launch_bounds__(NARROW ? 256 : 512, NARROW ? 3 : 1) k_moments_part(MomArgs M) {
    moments_body<real, MC, NM>(M, blockIdx.x, blockIdx.y);
}

// many contexts in one launch: CTA i takes march row work[i].y and velocity
// slice work[i].z of context work[i].x
template <typename real, int MC, int NM, bool NARROW>
__global__ void __launch_bounds__(NARROW ? 256 : 512, NARROW ? 3 : 1)
    k_moments_part_batch(const MomArgs *__restrict__ args, const int4 *__restrict__ work) {
    __shared__ MomArgs Ms;
    const int4 w = work[blockIdx.x];
    if (threadIdx.x == 0) Ms = args[w.x];
    __syncthreads();
    moments_body<real, MC, NM>(Ms, w.y, w.z);
}

template <typename real>
__device__ __forceinline__ void moments_finish_body(const MomArgs &M, int lpc, int blk) {
    SliceSum<real> acc[10];
    size_t cell;
    bool own;
    slice_fold<real, 10>(M, lpc, blk, acc, cell, own);
    if (!own) return;
    const int a = (int)(cell % M.PA) + 1, b = (int)(cell / M.PA) + 1;
    double s[10];
#pragma unroll
    for (int q = 0; q < 10; q++) s[q] = acc[q].value();
    // primitive conversion, GKUA_DETFP.f90:59-92
    double S1 = s[0], S4 = s[3], S5 = s[4], S6 = s[5], S7 = s[6];
    double ron = S1;
    if (ron <= 0.) ron = M.r00;
    double u = s[1] / ron, vv = s[2] / ron;
    double us1 = u * u, vs1 = vv * vv, suv = us1 + vs1;
    double tt = (S4 - ron * suv) / (1.5 * ron);
    if (tt <= 0.) tt = M.t00;
    int i, j;
    if (M.scan_is_j) { i = b; j = a; } else { i = a; j = b; }
    const size_t c2 = hyb_c2(M.nx, i, j);
    double *S = M.S;
    const size_t plane = (size_t)(M.nx + 3) * (size_t)(M.ny + 3);
    S[0 * plane + c2] = S1;
    S[1 * plane + c2] = u;
    S[2 * plane + c2] = vv;
    S[3 * plane + c2] = tt;
    S[4 * plane + c2] = (S5 - ron * us1) * 2.;
    S[5 * plane + c2] = (S6 - ron * vs1) * 2.;
    S[6 * plane + c2] = (S7 - ron * u * vv) * 2.;
    double qx = s[7] - 2. * u * S5 - 2. * vv * S7 + ron * u * (suv - 1.5 * tt);
    double qy = s[8] - 2. * vv * S6 - 2. * u * S7 + ron * vv * (suv - 1.5 * tt);
    S[7 * plane + c2] = qx;
    S[8 * plane + c2] = qy;
    S[9 * plane + c2] = s[9] * 2.;
    S[10 * plane + c2] = 0.0;
    double cf = (M.x1s <= (double)1.e-8f) ? M.cfc * S1 : M.cfc * S1 * pow(tt, M.x1s);
    M.CF[c2] = cf;
    // Shakhov parameters of the next kinetic step (Get_Feq uses S1, S4 = T)
    real *ep = (real *)M.eqp;
    double cpt = M.cpr / (S1 * tt * tt);
    ep[hyb_eqp_at(cell, 0)] = (real)(S1 / (HYB_PI * tt));
    ep[hyb_eqp_at(cell, 1)] = (real)u;
    ep[hyb_eqp_at(cell, 2)] = (real)vv;
    ep[hyb_eqp_at(cell, 3)] = (real)(1.0 / tt);
    ep[hyb_eqp_at(cell, 4)] = (real)(tt / 2.0);
    ep[hyb_eqp_at(cell, 5)] = (real)(cpt * qx);
    ep[hyb_eqp_at(cell, 6)] = (real)(cpt * qy);
    ep[hyb_eqp_at(cell, 7)] = (real)cf;
}

template <typename real>
__global__ void k_moments_finish(MomArgs M, int lpc) {
    moments_finish_body<real>(M, lpc, blockIdx.x);
}

// many contexts: block i is block work[i].y of context work[i].x, with
// work[i].z lanes per cell
template <typename real>
__global__ void __launch_bounds__(256) k_moments_finish_batch(const MomArgs *__restrict__ args,
                                                             const int4 *__restrict__ work) {
    __shared__ MomArgs Ms;
    const int4 w = work[blockIdx.x];
    if (threadIdx.x == 0) Ms = args[w.x];
    __syncthreads();
    moments_finish_body<real>(Ms, w.z, w.y);
}

// higher-order moments per cell: slice sums as in k_moments_finish, written
// to out[q][(nx+3)(ny+3)] (q = HOT 1..6, HOQ 1..3) at the interior cells
template <typename real>
__global__ void __launch_bounds__(256) k_hoq_finish(MomArgs M, int lpc, double *__restrict__ out) {
    SliceSum<real> acc[9];
    size_t cell;
    bool own;
    slice_fold<real, 9>(M, lpc, blockIdx.x, acc, cell, own);
    if (!own) return;
    const int a = (int)(cell % M.PA) + 1, b = (int)(cell / M.PA) + 1;
    const int i = M.scan_is_j ? b : a, j = M.scan_is_j ? a : b;
    const size_t c2 = hyb_c2(M.nx, i, j);
    const size_t plane = (size_t)(M.nx + 3) * (size_t)(M.ny + 3);
#pragma unroll
    for (int q = 0; q < 9; q++) out[(size_t)q * plane + c2] = acc[q].value();
}

// ---------------------------------------------------------------------------
// residual (DETFP_res): moments 1..4 of the stored RHS per cell by
// k_moments_part<., ., 4> over velocity slices, then per cell the slice sums
// (lanes per cell as in k_moments_finish), and per block the max |x| and the
// sum of x^2 of the block's cells; k_residual_final folds the blocks
// ---------------------------------------------------------------------------
__device__ __forceinline__ double nanmax(double a, double b) {
    if (a != a) return a;
    if (b != b) return b;
    return b > a ? b : a;
}

template <typename real>
__device__ __forceinline__ void residual_finish_body(const MomArgs &M, int lpc, int blk, double *__restrict__ part,
                                                     double *__restrict__ cellm) {
    const size_t ncell = (size_t)M.Nb * M.PA;
    SliceSum<real> acc[4];
    size_t cell;
    bool own;
    slice_fold<real, 4>(M, lpc, blk, acc, cell, own);
    double s[4];
#pragma unroll
    for (int q = 0; q < 4; q++) s[q] = acc[q].value();
    if (own && cellm)
#pragma unroll
        for (int q = 0; q < 4; q++) cellm[(size_t)q * ncell + cell] = s[q];
    double mx[4], sq[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const double x = own ? s[q] : 0.0;
        mx[q] = fabs(x);
        sq[q] = x * x;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // the cells' sums sit in threads 0 .. blockDim.x / lpc - 1 (slice_fold):
    // a warp above them holds zeros only, which its reduction would return
    // unchanged, so it skips the FP64 shuffles
    if (warp * 32 < (int)blockDim.x / lpc)
        for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int q = 0; q < 4; q++) {
                mx[q] = nanmax(mx[q], __shfl_xor_sync(0xffffffffu, mx[q], off));
                sq[q] += __shfl_xor_sync(0xffffffffu, sq[q], off);
            }
    __shared__ double wm[8][4], ws[8][4];
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            wm[warp][q] = mx[q];
            ws[warp][q] = sq[q];
        }
    __syncthreads();
    if (threadIdx.x < 4) {
        const int q = threadIdx.x;
        double m = 0.0, t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            m = nanmax(m, wm[w][q]);
            t += ws[w][q];
        }
        part[(size_t)blk * 8 + q] = m;
        part[(size_t)blk * 8 + 4 + q] = t;
    }
}

template <typename real>
__global__ void __launch_bounds__(256) k_residual_finish(MomArgs M, int lpc, double *__restrict__ part,
                                                         double *__restrict__ cellm) {
    residual_finish_body<real>(M, lpc, blockIdx.x, part, cellm);
}

// many contexts: block i is block work[i].y of context work[i].x (work[i].z
// lanes per cell), block partials to parts[work[i].x]
template <typename real>
__global__ void __launch_bounds__(256) k_residual_finish_batch(const MomArgs *__restrict__ args,
                                                               const int4 *__restrict__ work,
                                                               double *const *__restrict__ parts) {
    __shared__ MomArgs Ms;
    const int4 w = work[blockIdx.x];
    if (threadIdx.x == 0) Ms = args[w.x];
    __syncthreads();
    residual_finish_body<real>(Ms, w.z, w.y, parts[w.x], nullptr);
}

__device__ __forceinline__ void residual_final_body(const double *__restrict__ part, int nblk, double ncell,
                                                    double *__restrict__ out) {
    // one warp; deterministic sequential fold per lane
    __shared__ double mx[32][4], ss[32][4];
    const int lane = threadIdx.x;
    double m[4] = {0, 0, 0, 0}, s[4] = {0, 0, 0, 0};
    for (int bk = lane; bk < nblk; bk += 32)
        for (int k = 0; k < 4; k++) {
            double x = part[(size_t)bk * 8 + k];
            if (x > m[k] || x != x) m[k] = x;
            s[k] += part[(size_t)bk * 8 + 4 + k];
        }
    for (int k = 0; k < 4; k++) {
        mx[lane][k] = m[k];
        ss[lane][k] = s[k];
    }
    __syncwarp();
    if (lane == 0) {
        double mrms = 0.0;
        for (int k = 0; k < 4; k++) {
            double M = 0.0, Ssum = 0.0;
            for (int q = 0; q < 32; q++) {
                if (mx[q][k] > M || mx[q][k] != mx[q][k]) M = mx[q][k];
                Ssum += ss[q][k];
            }
            out[k] = M;
            out[4 + k] = sqrt(Ssum / ncell);
            if (out[4 + k] > mrms || out[4 + k] != out[4 + k]) mrms = out[4 + k];
        }
        out[8] = mrms;
    }
}

__global__ void k_residual_final(const double *__restrict__ part, int nblk, double ncell, double *__restrict__ out) {
    residual_final_body(part, nblk, ncell, out);
}

// many contexts: warp k folds context k's block partials into its residual
// and copies the 9 values to copy[9 k ..]
struct ResFinalArgs {
    const double *part;
    double *out;
    int nblk;
    double ncell;
};
__global__ void k_residual_final_batch(const ResFinalArgs *__restrict__ args, double *__restrict__ copy) {
    const ResFinalArgs A = args[blockIdx.x];
    residual_final_body(A.part, A.nblk, A.ncell, A.out);
    __syncwarp();
    if (threadIdx.x < 9) copy[(size_t)blockIdx.x * 9 + threadIdx.x] = A.out[threadIdx.x];
}

// ---------------------------------------------------------------------------
// uniform Maxwellian initial state, GKUA_sudufenbu.f90:25-40
// ---------------------------------------------------------------------------
template <typename real>
__global__ void k_init(real *__restrict__ f, const double *__restrict__ vx, const double *__restrict__ vy, int nvi,
                       int nv, int Na, int Nb, int PA, double rho, double u, double vv, double t) {
    const size_t rs = (size_t)Nb * PA;
    const size_t total = (size_t)nv * rs;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        size_t v = idx / rs, cell = idx % rs;
        int a = (int)(cell % PA) + 1;
        double g = 0.0, h = 0.0;
        if (a <= Na) {
            double crt = rho / (HYB_PI * t);
            double vjv = vy[v / nvi] - vv, viu = vx[v % nvi] - u;
            double vij2 = (viu * viu + vjv * vjv) / t;
            g = crt * exp(-vij2);
            h = t * g / 2.;
        }
        f[v * 2 * rs + cell] = (real)g;
        f[v * 2 * rs + rs + cell] = (real)h;
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static int check_err(hyb_ctx *ctx, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ctx->last_error = std::string(what) + ": " + cudaGetErrorString(e);
        return HYB_ERR_CUDA;
    }
    return HYB_OK;
}

// wall face index mapping: reference face (1..4) -> (on_scan, hi)
static void face_role(const hyb_ctx *ctx, int face, int *on_scan, int *hi) {
    if (ctx->scan_is_j) {
        *on_scan = (face == 2 || face == 4);
    } else {
        *on_scan = (face == 1 || face == 3);
    }
    *hi = (face == 3 || face == 4);
}

template <typename real>
static void launch_wall_real(hyb_ctx *ctx, const WallSet<real> &W, size_t smem) {
    k_wall<real><<<W.first[W.nface] * WALL_CL, 256, smem, ctx->stream>>>((const real *)ctx->d_f, W, ctx->d_vx,
                                                                          ctx->d_vy, ctx->d_w, ctx->nvi, ctx->nv,
                                                                          ctx->Na, ctx->Nb, ctx->PA);
}

// the wall faces of a context (returns the number of wall face cells)
static int wall_sets(hyb_ctx *ctx, WallSet<double> &Wd, WallSet<float> &Wf) {
    int nf = 0, first = 0;
    for (int face = 1; face <= 4; face++) {
        if (ctx->bc[face - 1] != HYB_BC_WALL) continue;
        int on_scan, hi;
        face_role(ctx, face, &on_scan, &hi);
        const int nfc = (face == 1 || face == 3) ? ctx->ncy : ctx->ncx;
        const double *wd = ctx->d_wall + (size_t)(face - 1) * 6 * 4096;
        Wd.fw[nf] = (double *)ctx->d_fw[face - 1];
        Wf.fw[nf] = (float *)ctx->d_fw[face - 1];
        Wd.wd[nf] = Wf.wd[nf] = wd;
        Wd.on_scan[nf] = Wf.on_scan[nf] = on_scan;
        Wd.hi[nf] = Wf.hi[nf] = hi;
        Wd.first[nf] = Wf.first[nf] = first;
        first += nfc;
        nf++;
    }
    Wd.first[nf] = Wf.first[nf] = first;
    Wd.nface = Wf.nface = nf;
    return first;
}

static size_t wall_smem_bytes(const hyb_ctx *ctx) {
    return (size_t)((ctx->nv + WALL_CL - 1) / WALL_CL) * sizeof(double);
}

// every wall face of the context in one launch
int launch_wall(hyb_ctx *ctx) {
    WallSet<double> Wd;
    WallSet<float> Wf;
    if (wall_sets(ctx, Wd, Wf) == 0) return HYB_OK;
    const size_t wall_smem = wall_smem_bytes(ctx);
    if (wall_smem > (size_t)200 * 1024) {
        ctx->last_error = "wall: velocity grid too large for one cluster's shared memory";
        return HYB_ERR_UNSUPPORTED;
    }
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_wall<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_wall<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    if (ctx->precision == HYB_PREC_FP64) launch_wall_real<double>(ctx, Wd, wall_smem);
    else launch_wall_real<float>(ctx, Wf, wall_smem);
    ctx->launches++;
    return check_err(ctx, "k_wall");
}

int moments_slices(const hyb_ctx *ctx) {
    // enough CTAs to fill the GPU: about 16 per SM (four waves of the four
    // CTAs an SM holds with a 3-slot ring at PA = 512), whole velocity rows each
    int nvj = ctx->nvj;
    int vs = (152 * 16 + ctx->Nb - 1) / ctx->Nb;
    if (vs > nvj) vs = nvj;
    if (vs < 1) vs = 1;
    return vs;
}

template <typename real, int MC, int NM, bool NARROW>
static void launch_mom_bounds(hyb_ctx *ctx, const MomArgs &M, dim3 grd, int tpv, size_t smem) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_moments_part<real, MC, NM, NARROW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             227 * 1024);
        attr = true;
    }
    k_moments_part<real, MC, NM, NARROW><<<grd, tpv, smem, ctx->stream>>>(M);
}

template <typename real>
static constexpr bool mom_narrow_ok() { return sizeof(real) == 4; }

template <typename real, int MC, int NM>
static void launch_mom(hyb_ctx *ctx, const MomArgs &M, dim3 grd, int tpv, size_t smem) {
    if (mom_narrow_ok<real>() && tpv <= 256) launch_mom_bounds<real, MC, NM, mom_narrow_ok<real>()>(ctx, M, grd, tpv, smem);
    else launch_mom_bounds<real, MC, NM, false>(ctx, M, grd, tpv, smem);
}

// lanes per cell of the slice sums: enough for the slices, while the grid
// keeps about 64K threads (one lane per cell on large meshes)
static int finish_lpc(size_t ncell, int vs) {
    int lpc = 1;
    while (lpc < 32 && lpc < vs && ncell * (size_t)(lpc * 2) <= 65536) lpc *= 2;
    return lpc;
}

int residual_blocks(const hyb_ctx *ctx) {
    const size_t ncell = (size_t)ctx->Nb * ctx->PA;
    return (int)((ncell * finish_lpc(ncell, moments_slices(ctx)) + 255) / 256);
}

// MomArgs of the moment pass over the velocity slices of distribution `f`
static MomArgs mom_args(hyb_ctx *ctx, const void *f, size_t *smem, int *mc) {
    MomArgs M;
    M.f = f;
    M.part = ctx->d_mpart;
    M.S = ctx->d_S;
    M.CF = ctx->d_CF;
    M.eqp = ctx->d_eqp;
    M.vx = ctx->d_vx;
    M.vy = ctx->d_vy;
    M.w = ctx->d_w;
    M.nvi = ctx->nvi;
    M.nv = ctx->nv;
    M.Na = ctx->Na;
    M.Nb = ctx->Nb;
    M.PA = ctx->PA;
    M.nx = ctx->nx;
    M.ny = ctx->ny;
    M.scan_is_j = ctx->scan_is_j;
    M.vs = moments_slices(ctx);
    M.nloc_max = (ctx->nvj + M.vs - 1) / M.vs * ctx->nvi;
    M.err = ctx->d_err;
    M.spin = ctx->spin_cycles;
    M.cfc = ctx->prm.cfc;
    M.cpr = ctx->prm.cpr;
    M.x1s = ctx->prm.x1s;
    M.r00 = ctx->prm.r00;
    M.t00 = ctx->prm.t00;
    // cells per thread: two where the chunk allows it (both precisions stay
    // below 128 registers without spills), one on FP64 rows of <= 256 cells
    // so that more threads share them; a CTA has at most 512 threads
    *mc = (ctx->cpt >= 2 && (ctx->precision != HYB_PREC_FP64 || ctx->PA > 256)) ? 2 : 1;
    *smem = ctx->precision == HYB_PREC_FP64 ? mom_smem_bytes<double>(ctx->PA, M.nloc_max)
                                            : mom_smem_bytes<float>(ctx->PA, M.nloc_max);
    return M;
}

template <int NM>
static int launch_mom_pass(hyb_ctx *ctx, const MomArgs &M, int mc, size_t smem) {
    if constexpr (NM == 10 || NM == 4) {
        // FP32 rows of up to 512 cells at two cells per thread: the packed pass
        const size_t s2 = mom_f2_smem_bytes(ctx->PA, M.nloc_max);
        if (ctx->precision != HYB_PREC_FP64 && mc == 2 && ctx->PA / 2 <= 256 && s2 <= (size_t)227 * 1024) {
            static bool attr = false;
            if (!attr) {
                cudaFuncSetAttribute(k_moments_f2<NM>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
                attr = true;
            }
            k_moments_f2<NM><<<dim3(ctx->Nb, M.vs), ctx->PA / 2, s2, ctx->stream>>>(M);
            ctx->launches++;
            return check_err(ctx, "k_moments_f2");
        }
    }
    if (smem > (size_t)227 * 1024) {
        ctx->last_error = "moments: velocity slice too large for shared memory";
        return HYB_ERR_UNSUPPORTED;
    }
    const int tpv = ctx->PA / mc;
    dim3 grd(ctx->Nb, M.vs);
    if (ctx->precision == HYB_PREC_FP64) {
        if (mc == 2) launch_mom<double, 2, NM>(ctx, M, grd, tpv, smem);
        else launch_mom<double, 1, NM>(ctx, M, grd, tpv, smem);
    } else {
        if (mc == 2) launch_mom<float, 2, NM>(ctx, M, grd, tpv, smem);
        else launch_mom<float, 1, NM>(ctx, M, grd, tpv, smem);
    }
    ctx->launches++;
    return check_err(ctx, "k_moments_part");
}

int launch_moments(hyb_ctx *ctx) {
    size_t smem;
    int mc;
    MomArgs M = mom_args(ctx, ctx->d_f, &smem, &mc);
    int rc = launch_mom_pass<10>(ctx, M, mc, smem);
    if (rc) return rc;
    const size_t ncell = (size_t)ctx->Nb * ctx->PA;
    const int lpc = finish_lpc(ncell, M.vs);
    const unsigned nb = (unsigned)((ncell * lpc + 255) / 256);
    if (ctx->precision == HYB_PREC_FP64) k_moments_finish<double><<<nb, 256, 0, ctx->stream>>>(M, lpc);
    else k_moments_finish<float><<<nb, 256, 0, ctx->stream>>>(M, lpc);
    ctx->launches++;
    return check_err(ctx, "k_moments_finish");
}

// moments 1-4 of a stored RHS: per-cell values to cellm (if given) and the
// per-block max / sum of squares to the residual partials
static int residual_part(hyb_ctx *ctx, const void *rhs, double *cellm, int *nblk_out) {
    size_t smem;
    int mc;
    MomArgs M = mom_args(ctx, rhs, &smem, &mc);
    int rc = launch_mom_pass<4>(ctx, M, mc, smem);
    if (rc) return rc;
    const size_t ncell = (size_t)ctx->Nb * ctx->PA;
    const int lpc = finish_lpc(ncell, M.vs);
    const unsigned nb = (unsigned)((ncell * lpc + 255) / 256);
    *nblk_out = (int)nb;
    if (ctx->precision == HYB_PREC_FP64)
        k_residual_finish<double><<<nb, 256, 0, ctx->stream>>>(M, lpc, ctx->d_resid + 16, cellm);
    else
        k_residual_finish<float><<<nb, 256, 0, ctx->stream>>>(M, lpc, ctx->d_resid + 16, cellm);
    ctx->launches++;
    return check_err(ctx, "k_residual_finish");
}

// per-cell moments 1-4 of the RHS-only sweep's output, [4][Nb*PA]
int launch_rhs_moments(hyb_ctx *ctx, double *cellm) {
    int nblk;
    return residual_part(ctx, ctx->d_rhs_gsis, cellm, &nblk);
}

// higher-order moments of the current f at the interior cells,
// out[9][(nx+3)(ny+3)] (zero-filled by the caller)
int launch_hoq(hyb_ctx *ctx, double *out) {
    size_t smem;
    int mc;
    MomArgs M = mom_args(ctx, ctx->d_f, &smem, &mc);
    int rc = launch_mom_pass<9>(ctx, M, mc, smem);
    if (rc) return rc;
    const size_t ncell = (size_t)ctx->Nb * ctx->PA;
    const int lpc = finish_lpc(ncell, M.vs);
    const unsigned nb = (unsigned)((ncell * lpc + 255) / 256);
    if (ctx->precision == HYB_PREC_FP64) k_hoq_finish<double><<<nb, 256, 0, ctx->stream>>>(M, lpc, out);
    else k_hoq_finish<float><<<nb, 256, 0, ctx->stream>>>(M, lpc, out);
    ctx->launches++;
    return check_err(ctx, "k_hoq_finish");
}

int launch_residual(hyb_ctx *ctx, hyb_residual *out) {
    int nblk;
    double *part = ctx->d_resid + 16;
    int rc = residual_part(ctx, ctx->d_rhs, nullptr, &nblk);
    if (rc) return rc;
    k_residual_final<<<1, 32, 0, ctx->stream>>>(part, nblk, (double)ctx->ncx * ctx->ncy, ctx->d_resid);
    ctx->launches++;
    rc = check_err(ctx, "k_residual_final");
    if (rc) return rc;
    if (out) {
        HYB_CK(cudaMemcpyAsync(ctx->h_resid, ctx->d_resid, 9 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        HYB_CK(cudaStreamSynchronize(ctx->stream));
        for (int k = 0; k < 4; k++) {
            out->res_max[k] = ctx->h_resid[k];
            out->res_rms[k] = ctx->h_resid[4 + k];
        }
        out->max_rms = ctx->h_resid[8];
    }
    return HYB_OK;
}

// ---------------------------------------------------------------------------
// total mass sum(vol rho) over the interior cells (mass_pin).  One CTA: each
// thread adds its cells k = tid, tid + 1024, ... in order, then a fixed-order
// tree fold.  mode 0 stores the sum as m0 in mass[0], mode 1 stores the
// scale m0 / M in mass[1].
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_total_mass(const double *__restrict__ S, const double *__restrict__ volc,
                                                     int nx, int ny, int mode, double *__restrict__ mass) {
    __shared__ double red[1024];
    const int ncx = nx - 1, n = (nx - 1) * (ny - 1);
    double acc = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int i = k % ncx + 1, j = k / ncx + 1;
        acc += volc[k] * S[hyb_c2(nx, i, j)];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (mode == 0) {
            mass[0] = red[0];
            mass[1] = 1.0;
        } else {
            mass[1] = mass[0] / red[0];
        }
    }
}

int launch_total_mass(hyb_ctx *ctx, int mode) {
    k_total_mass<<<1, 1024, 0, ctx->stream>>>(ctx->d_S, ctx->d_volc, ctx->nx, ctx->ny, mode, ctx->d_mass);
    ctx->launches++;
    return check_err(ctx, "k_total_mass");
}

int launch_init_maxwellian(hyb_ctx *ctx, double rho, double u, double v, double t) {
    int grid = 152 * 8;
    if (ctx->precision == HYB_PREC_FP64)
        k_init<double><<<grid, 256, 0, ctx->stream>>>((double *)ctx->d_f, ctx->d_vx, ctx->d_vy, ctx->nvi, ctx->nv,
                                                      ctx->Na, ctx->Nb, ctx->PA, rho, u, v, t);
    else
        k_init<float><<<grid, 256, 0, ctx->stream>>>((float *)ctx->d_f, ctx->d_vx, ctx->d_vy, ctx->nvi, ctx->nv,
                                                     ctx->Na, ctx->Nb, ctx->PA, rho, u, v, t);
    ctx->launches++;
    return check_err(ctx, "k_init");
}

// ---- batched launches over many contexts (hyb_batch) ------------------------
// Per-context argument records (filled on the host, copied to the device by
// the caller) and work tables; one launch per launch shape.
size_t wall_arg_bytes(int precision) {
    return precision == HYB_PREC_FP64 ? sizeof(WallArgs<double>) : sizeof(WallArgs<float>);
}

int wall_arg_fill(hyb_ctx *ctx, void *dst, size_t *smem) {
    WallSet<double> Wd;
    WallSet<float> Wf;
    const int n = wall_sets(ctx, Wd, Wf);
    *smem = wall_smem_bytes(ctx);
    if (ctx->precision == HYB_PREC_FP64) {
        WallArgs<double> a{(const double *)ctx->d_f, Wd, ctx->d_vx, ctx->d_vy, ctx->d_w,
                           ctx->nvi, ctx->nv, ctx->Na, ctx->Nb, ctx->PA};
        memcpy(dst, &a, sizeof(a));
    } else {
        WallArgs<float> a{(const float *)ctx->d_f, Wf, ctx->d_vx, ctx->d_vy, ctx->d_w,
                          ctx->nvi, ctx->nv, ctx->Na, ctx->Nb, ctx->PA};
        memcpy(dst, &a, sizeof(a));
    }
    return n;
}

int wall_batch_launch(int precision, const void *args, const int2 *work, int nclusters, size_t smem,
                      cudaStream_t s) {
    if (smem > (size_t)200 * 1024) return HYB_ERR_UNSUPPORTED;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_wall_batch<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_wall_batch<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    if (nclusters <= 0) return HYB_OK;   // attributes only (before a capture)
    if (precision == HYB_PREC_FP64)
        k_wall_batch<double><<<nclusters * WALL_CL, 256, smem, s>>>((const WallArgs<double> *)args, work);
    else
        k_wall_batch<float><<<nclusters * WALL_CL, 256, smem, s>>>((const WallArgs<float> *)args, work);
    return cudaGetLastError() == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
}

size_t mom_arg_bytes() { return sizeof(MomArgs); }

// the moment pass of a context: its arguments, cells per thread, threads
// per CTA, shared memory, velocity slices, lanes per cell and finish blocks
int mom_arg_fill(hyb_ctx *ctx, const void *f, void *dst, int *mc, int *tpv, size_t *smem, int *vs, int *lpc,
                 int *nfin) {
    MomArgs M = mom_args(ctx, f ? f : ctx->d_f, smem, mc);
    if (mom_f2_ok(ctx->precision, *mc, ctx->PA / *mc))   // the batched packed pass's shared memory
        *smem = mom_f2_smem_bytes(ctx->PA, M.nloc_max);
    if (*smem > (size_t)227 * 1024 - 1024) return HYB_ERR_UNSUPPORTED;   // the batched kernel's limit
    memcpy(dst, &M, sizeof(M));
    *tpv = ctx->PA / *mc;
    *vs = M.vs;
    const size_t ncell = (size_t)ctx->Nb * ctx->PA;
    *lpc = finish_lpc(ncell, M.vs);
    *nfin = (int)((ncell * *lpc + 255) / 256);
    return HYB_OK;
}

template <typename real, int MC, int NM, bool NARROW>
static int mom_part_batch_bounds(const MomArgs *args, const int4 *work, int nwork, int tpv, size_t smem,
                                 cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_moments_part_batch<real, MC, NM, NARROW>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024 - 1024);
        attr = true;
    }
    if (nwork <= 0) return HYB_OK;   // attributes only (before a capture)
    k_moments_part_batch<real, MC, NM, NARROW><<<nwork, tpv, smem, s>>>(args, work);
    return cudaGetLastError() == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
}

template <typename real, int MC, int NM>
static int mom_part_batch_one(const MomArgs *args, const int4 *work, int nwork, int tpv, size_t smem,
                              cudaStream_t s) {
    if (mom_narrow_ok<real>() && tpv <= 256)
        return mom_part_batch_bounds<real, MC, NM, mom_narrow_ok<real>()>(args, work, nwork, tpv, smem, s);
    return mom_part_batch_bounds<real, MC, NM, false>(args, work, nwork, tpv, smem, s);
}

template <int NM>
static int mom_part_batch_nm(int precision, int mc, int tpv, const MomArgs *a, const int4 *work, int nwork,
                             size_t smem, cudaStream_t s) {
    if (mom_f2_ok(precision, mc, tpv)) {
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(k_moments_f2_batch<NM>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024 - 1024);
            attr = true;
        }
        if (nwork <= 0) return HYB_OK;   // attributes only (before a capture)
        k_moments_f2_batch<NM><<<nwork, tpv, smem, s>>>(a, work);
        return cudaGetLastError() == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
    }
    if (precision == HYB_PREC_FP64)
        return mc == 2 ? mom_part_batch_one<double, 2, NM>(a, work, nwork, tpv, smem, s)
                       : mom_part_batch_one<double, 1, NM>(a, work, nwork, tpv, smem, s);
    return mc == 2 ? mom_part_batch_one<float, 2, NM>(a, work, nwork, tpv, smem, s)
                   : mom_part_batch_one<float, 1, NM>(a, work, nwork, tpv, smem, s);
}

// nm = 10: the DETFP moments; nm = 4: the residual moments of a stored RHS
int moments_part_batch_launch(int precision, int mc, int tpv, int nm, const void *args, const int4 *work, int nwork,
                              size_t smem, cudaStream_t s) {
    const MomArgs *a = (const MomArgs *)args;
    if (nm == 4) return mom_part_batch_nm<4>(precision, mc, tpv, a, work, nwork, smem, s);
    return mom_part_batch_nm<10>(precision, mc, tpv, a, work, nwork, smem, s);
}

int residual_finish_batch_launch(int precision, const void *args, const int4 *work, double *const *parts, int nwork,
                                 cudaStream_t s) {
    if (nwork <= 0) return HYB_OK;
    if (precision == HYB_PREC_FP64)
        k_residual_finish_batch<double><<<nwork, 256, 0, s>>>((const MomArgs *)args, work, parts);
    else
        k_residual_finish_batch<float><<<nwork, 256, 0, s>>>((const MomArgs *)args, work, parts);
    return cudaGetLastError() == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
}

size_t resfinal_arg_bytes() { return sizeof(ResFinalArgs); }

// the context's final residual fold; *part receives its block partials
void resfinal_arg_fill(hyb_ctx *ctx, void *dst, double **part) {
    const size_t ncell = (size_t)ctx->Nb * ctx->PA;
    ResFinalArgs a;
    a.part = ctx->d_resid + 16;
    a.out = ctx->d_resid;
    a.nblk = (int)((ncell * finish_lpc(ncell, moments_slices(ctx)) + 255) / 256);
    a.ncell = (double)ctx->ncx * ctx->ncy;
    memcpy(dst, &a, sizeof(a));
    *part = ctx->d_resid + 16;
}

int residual_final_batch_launch(const void *args, int n, double *copy, cudaStream_t s) {
    if (n <= 0) return HYB_OK;
    k_residual_final_batch<<<n, 32, 0, s>>>((const ResFinalArgs *)args, copy);
    return cudaGetLastError() == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
}

int moments_finish_batch_launch(int precision, const void *args, const int4 *work, int nwork, cudaStream_t s) {
    if (nwork <= 0) return HYB_OK;
    if (precision == HYB_PREC_FP64)
        k_moments_finish_batch<double><<<nwork, 256, 0, s>>>((const MomArgs *)args, work);
    else
        k_moments_finish_batch<float><<<nwork, 256, 0, s>>>((const MomArgs *)args, work);
    return cudaGetLastError() == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
}

// error words of many contexts into one array
__global__ void k_gather_err(int *const *__restrict__ errs, int *__restrict__ out, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = *errs[k];
}

int gather_err_launch(int *const *errs, int *out, int n, cudaStream_t s) {
    if (n <= 0) return HYB_OK;
    k_gather_err<<<(n + 127) / 128, 128, 0, s>>>(errs, out, n);
    return cudaGetLastError() == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
}

}  // namespace hyb
