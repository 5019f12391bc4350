// hyb_sweep.cuh -- the fused kinetic step of one outer iteration:
// Get_Feq + RHSFDVsub + LU-SGS forward sweep + backward step + update + floor
// (GKUA_Residual.f90:4-469), for every velocity node.  Instantiated for FP32
// and FP64 distributions in hyb_sweep_f32.cu / hyb_sweep_f64.cu.
//
// Work decomposition.  One thread group per velocity node walks the MARCH
// axis b row by row; a row of the SCAN axis a is split over the group's
// threads, CPT consecutive cells per thread.  Rows of f are staged into a
// shared-memory ring by cp.async.bulk copies that complete on mbarriers,
// three rows ahead of use.
//
// The forward recurrence dF(a,b) = c(a,b) + p(a) dF(a-1,b), with
// c = (vol RHS + pos(B) dF(a,b-1)) / alpha and p = pos(A) / alpha, is linear in
// dF(a-1,b): each thread composes the affine maps of its CPT cells, the group
// scans the composed maps (warp shuffles, then one shared-memory pass across
// warps) and each thread replays its cells from the incoming value.  When
// every face speed along the scan axis is non-positive, p = 0 and the scan is
// skipped.  The recurrence along b is carried in registers.  The reference's
// backward step reads only forward values of the downstream neighbours
// (GKUA_Residual.f90:64-90), so it is evaluated one row behind the forward
// sweep and neither dF nor the RHS is written to memory (the RHS only when a
// residual is requested).  The seam of a periodic face is explicit in both
// sweeps, as the reference's zero FRD00 ghosts make every block face.
//
// Upwind order (UPW, HYB_SWEEP_UPWIND, uniform meshes).  A velocity whose
// scan-face speed is negative is swept with the scan axis mirrored (logical
// cell a is physical cell Na+1-a), one whose march-face speed is negative
// with the march axis mirrored (logical row b is physical row Nb+1-b).  In
// the mirrored frame both speeds are >= 0, so the forward recurrence is the
// exact first-order upwind solve and the backward step adds nothing.  The
// face fluxes are the physical ones: each formula satisfies
// flux(-s, mirrored stencil) = -flux(s, stencil), and the negated face normal
// turns that back into the physical divergence.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "hyb_common.cuh"
#include "hyb_device.cuh"

namespace hyb {

constexpr int RING = 8;   // staged rows per velocity

template <typename real>
__host__ __device__ inline size_t sweep_group_bytes(int PA, int TPV) {
    size_t nw = (size_t)TPV / 32;
    size_t b = 128;                                    // RING+2 mbarriers
    b += (size_t)RING * 2 * PA * sizeof(real);         // staged rows
    b += (size_t)2 * 2 * PA * sizeof(real);            // rows Nb+1, Nb+2 (periodic)
    b += (size_t)2 * 2 * TPV * sizeof(real);           // first-cell dF per thread
    b += (size_t)2 * nw * 3 * sizeof(real);            // warp aggregates
    return (b + 127) / 128 * 128;
}

// CPT consecutive values from (shared or global) memory / to global memory
template <typename real, int CPT> struct Vec;
template <> struct Vec<float, 4> {
    static __device__ __forceinline__ void ld(const float *p, float *o) {
        float4 x = *reinterpret_cast<const float4 *>(p);
        o[0] = x.x; o[1] = x.y; o[2] = x.z; o[3] = x.w;
    }
    static __device__ __forceinline__ void st(float *p, const float *o) {
        *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
    }
};
template <> struct Vec<float, 2> {
    static __device__ __forceinline__ void ld(const float *p, float *o) {
        float2 x = *reinterpret_cast<const float2 *>(p);
        o[0] = x.x; o[1] = x.y;
    }
    static __device__ __forceinline__ void st(float *p, const float *o) {
        *reinterpret_cast<float2 *>(p) = make_float2(o[0], o[1]);
    }
};
template <> struct Vec<double, 4> {
    static __device__ __forceinline__ void ld(const double *p, double *o) {
        double2 x = *reinterpret_cast<const double2 *>(p), y = *reinterpret_cast<const double2 *>(p + 2);
        o[0] = x.x; o[1] = x.y; o[2] = y.x; o[3] = y.y;
    }
    static __device__ __forceinline__ void st(double *p, const double *o) {
        *reinterpret_cast<double2 *>(p) = make_double2(o[0], o[1]);
        *reinterpret_cast<double2 *>(p + 2) = make_double2(o[2], o[3]);
    }
};
template <> struct Vec<double, 2> {
    static __device__ __forceinline__ void ld(const double *p, double *o) {
        double2 x = *reinterpret_cast<const double2 *>(p);
        o[0] = x.x; o[1] = x.y;
    }
    static __device__ __forceinline__ void st(double *p, const double *o) {
        *reinterpret_cast<double2 *>(p) = make_double2(o[0], o[1]);
    }
};
template <typename real> struct Vec<real, 1> {
    static __device__ __forceinline__ void ld(const real *p, real *o) { o[0] = *p; }
    static __device__ __forceinline__ void st(real *p, const real *o) { *p = o[0]; }
};

// Flux through a face of speed s from f(q-2), f(q-1), f(q), f(q+1)
// (RHSFDVsub, GKUA_Residual.f90:155-185).  Only the upwind reconstruction is
// formed: with s > 0, asn = 0 and asp = s exactly, so asp*UL + asn*UR = s*UL.
template <int SCHEME, typename real>
__device__ __forceinline__ real flux_std(real s, real u1, real u2, real u3, real u4) {
    if constexpr (SCHEME == HYB_SCHEME_UP1) {
        return s > real(0) ? s * u2 : s * u3;
    } else if constexpr (SCHEME == HYB_SCHEME_NND) {
        // UR(u1,u2,u3,u4) = UL(u4,u3,u2,u1) because FMINMD(-x,-y) = -FMINMD(x,y)
        // exactly, so one limiter on mirrored inputs gives the upwind value
        const bool up = s > real(0);
        const real x1 = up ? u1 : u4, x2 = up ? u2 : u3, x3 = up ? u3 : u2;
        return s * (x2 + real(0.5) * fminmd(x3 - x2, x2 - x1));
    } else {
        return face_flux(HYB_SCHEME_WENO3, posp(s), negp(s), u1, u2, u3, u4);
    }
}
// face 2 next to a low-end wall (GKUA_Residual.f90:196-221)
template <int SCHEME, typename real>
__device__ __forceinline__ real flux_wlo(real s, real f1, real f2, real f3) {
    if constexpr (SCHEME == HYB_SCHEME_WENO3) return face_flux_wall_lo(SCHEME, posp(s), negp(s), f1, f2, f3);
    else if constexpr (SCHEME == HYB_SCHEME_UP1) return s > real(0) ? s * f1 : s * f2;
    else return s > real(0) ? s * (f1 + real(0.5) * (f2 - f1)) : s * (f2 - real(0.5) * fminmd(f2 - f1, f3 - f2));
}
// face n next to a high-end wall, f1=f(n-1), f2=f(n-2), f3=f(n-3)
// (GKUA_Residual.f90:233-257)
template <int SCHEME, typename real>
__device__ __forceinline__ real flux_whi(real s, real f1, real f2, real f3) {
    if constexpr (SCHEME == HYB_SCHEME_WENO3) return face_flux_wall_hi(SCHEME, posp(s), negp(s), f1, f2, f3);
    else if constexpr (SCHEME == HYB_SCHEME_UP1) return s > real(0) ? s * f2 : s * f1;
    else return s > real(0) ? s * (f2 + real(0.5) * fminmd(f1 - f2, f2 - f3)) : s * (f1 - real(0.5) * (f1 - f2));
}

// After a wait ran out at row `stop`: rows stop+3 .. stop+RING-4 (all
// within 1..Nb, so each is a real copy) were issued and never waited for;
// wait (bounded) for each before the CTA leaves.  Out of line, so that the
// row loop's register allocation does not carry this path.
static __device__ __noinline__ void sweep_drain(uint64_t *bars, int stop, int Nb, int stall_row, long long spin) {
    for (int bp = stop + 3; bp <= Nb && bp <= stop + RING - 4; bp++)
        if (stall_row <= 0 || bp != stall_row) mbar_wait_bounded(&bars[(bp + 1) % RING], (uint32_t)(((bp + 1) / RING) & 1), spin);
}

// the sweep of the CTA's velocity block vblk (velocities vblk * vpb + g)
template <typename real, int CPT, bool UNI, int SCHEME, bool UPW = false>
__device__ __forceinline__ void sweep_body(const KinArgs<real> &A, int vblk) {
    static_assert(!UPW || UNI, "the upwind order is built for uniform meshes");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int PA = A.PA, Na = A.Na, Nb = A.Nb;
    const int TPV = PA / CPT;
    const int g = threadIdx.y, t = threadIdx.x;
    const int a0 = t * CPT + 1;                  // first cell of this thread
    const int lane = t & 31, warp = t >> 5;
    const int v = vblk * blockDim.y + g;
    const bool vok = v < A.nv;
    const bool act = vok && (a0 <= Na);          // chunks are all-in or all-out
    const bool producer = (t == 0) && vok;

    unsigned char *base = smem_raw + (size_t)g * sweep_group_bytes<real>(PA, TPV);
    uint64_t *bars = reinterpret_cast<uint64_t *>(base);
    real *ring = reinterpret_cast<real *>(base + 128);
    real *wrap = ring + (size_t)RING * 2 * PA;
    real *dlf = wrap + (size_t)2 * 2 * PA;       // [2][2][TPV]
    real *agg = dlf + (size_t)2 * 2 * TPV;       // [2][nw][3]
    const int nw = TPV >> 5;

    const bool perB = (A.bcb_lo == AX_PERIODIC);
    const bool perA = (A.bca_lo == AX_PERIODIC);
    const size_t vrow0 = vok ? (size_t)v * 2 * Nb * PA : 0;
    const size_t rstride = (size_t)Nb * PA;
    const uint32_t row_bytes = (uint32_t)(PA * sizeof(real));

    // ---- velocity, face speeds and the frame of the sweep ---------------------
    const int iv = vok ? v % A.nvi : 0, jv = vok ? v / A.nvi : 0;
    const real vx = vok ? (real)A.vx[iv] : real(0), vy = vok ? (real)A.vy[jv] : real(0);
    const real dt = A.dt;
    const int PA1 = PA + 1;
    real sA_u = 0, sB_u = 0, vol_u = 1, ivol_u = 1, abase_u = 0;
    if (UNI) {
        sA_u = vx * A.gA1[0] + vy * A.gA2[0];
        sB_u = vx * A.gB1[0] + vy * A.gB2[0];
        vol_u = A.vol[0];
        ivol_u = real(1) / vol_u;
        abase_u = vol_u / dt + (posp(sA_u) - negp(sA_u) + posp(sB_u) - negp(sB_u));
    }
    // mirrored scan / march axis of this group (upwind order only)
    const bool ra = UPW && sA_u < real(0), rb = UPW && sB_u < real(0);
    if (ra) sA_u = -sA_u;
    if (rb) sB_u = -sB_u;
    // physical 0-based scan index of logical cell a; physical row of logical
    // row b (1..Nb)
    auto pa = [&](int a) -> int { return ra ? Na - a : a - 1; };
    auto prow = [&](int b) -> int { return rb ? Nb + 1 - b : b; };
    // the CPT logical cells of this thread from / to a row of physical cells
    const int pa0 = ra ? Na - a0 - CPT + 1 : a0 - 1;   // first physical index of the chunk
    auto ldc = [&](const real *row, real *o) {
        if (!ra) {
            Vec<real, CPT>::ld(row + pa0, o);
        } else {
            real t[CPT];
            Vec<real, CPT>::ld(row + pa0, t);
#pragma unroll
            for (int k = 0; k < CPT; k++) o[k] = t[CPT - 1 - k];
        }
    };
    auto stc = [&](real *row, const real *o) {
        if (!ra) {
            Vec<real, CPT>::st(row + pa0, o);
        } else {
            real t[CPT];
#pragma unroll
            for (int k = 0; k < CPT; k++) t[k] = o[CPT - 1 - k];
            Vec<real, CPT>::st(row + pa0, t);
        }
    };
    // wall slots of the logical low / high ends
    const real *fw_alo = ra ? A.fw_ahi : A.fw_alo, *fw_ahi = ra ? A.fw_alo : A.fw_ahi;
    const real *fw_blo = rb ? A.fw_bhi : A.fw_blo, *fw_bhi = rb ? A.fw_blo : A.fw_bhi;

    // physical row held by logical ring row bp (0: none)
    auto phys_row = [&](int bp) -> int {
        if (bp >= 1 && bp <= Nb) return prow(bp);
        if (perB && bp <= 0) return prow(bp + Nb);
        return 0;
    };
    auto issue_row = [&](int bp) {
        int s = (bp + 1) % RING;
        int pr = phys_row(bp);
        if (A.stall_row > 0 && bp == A.stall_row) return;   // hyb_test_stall: a wait nothing completes
        if (pr > 0 && bp <= Nb) {
            mbar_arrive_expect_tx(&bars[s], 2 * row_bytes);
            const real *src = A.f + vrow0 + (size_t)(pr - 1) * PA;
            bulk_g2s(ring + (size_t)s * 2 * PA, src, row_bytes, &bars[s]);
            bulk_g2s(ring + (size_t)s * 2 * PA + PA, src + rstride, row_bytes, &bars[s]);
        } else {
            mbar_arrive(&bars[s]);                // keeps the slot's phase count
        }
    };
    if (producer) {
        for (int s = 0; s < RING + 2; s++) mbar_init(&bars[s], 1);
        fence_async_shared();
    }
    __syncthreads();
    if (producer) {
        // rows -1 .. RING-3 fill slots 0 .. RING-2; step b refills the slot of
        // row b-3 with row b+RING-3
        for (int bp = -1; bp <= RING - 3; bp++) issue_row(bp);
        if (perB) {
            for (int w = 0; w < 2; w++) {
                mbar_arrive_expect_tx(&bars[RING + w], 2 * row_bytes);
                const real *src = A.f + vrow0 + (size_t)(prow(w + 1) - 1) * PA;
                bulk_g2s(wrap + (size_t)w * 2 * PA, src, row_bytes, &bars[RING + w]);
                bulk_g2s(wrap + (size_t)w * 2 * PA + PA, src + rstride, row_bytes, &bars[RING + w]);
            }
        }
    }
    // row data of logical row bp (component 0; component 1 is PA further)
    auto rowp = [&](int bp) -> const real * {
        if (bp > Nb) return wrap + (size_t)(bp - Nb - 1) * 2 * PA;
        return ring + (size_t)((bp + 1) & (RING - 1)) * 2 * PA;
    };
    bool timeout = false;
    auto wait_row = [&](int bp) {
        if (!vok) return;
        if (bp > Nb) {
            if (perB && !mbar_wait_bounded(&bars[RING + (bp - Nb - 1)], 0, A.spin)) timeout = true;
            return;
        }
        if (phys_row(bp) == 0) return;
        if (!mbar_wait_bounded(&bars[(bp + 1) % RING], (uint32_t)(((bp + 1) / RING) & 1), A.spin)) timeout = true;
    };
    // scan-axis halo cells of the thread (wrapped on a periodic axis; on a
    // wall axis they are only read by the standard faces, which never reach
    // outside 1..Na)
    auto wrapA = [&](int c) -> int {
        const int l = perA ? ((c - 1 + 2 * Na) % Na) : (c < 1 ? 0 : (c > Na ? Na - 1 : c - 1));
        return ra ? Na - 1 - l : l;
    };
    const int hm2 = wrapA(a0 - 2), hm1 = wrapA(a0 - 1), hp0 = wrapA(a0 + CPT), hp1 = wrapA(a0 + CPT + 1);
    // a thread away from both wall ends of the scan axis has standard faces only
    const bool edgeA = !perA && (a0 <= 2 || a0 + CPT >= Na);

    // the scan is needed only when some group of the CTA has a positive
    // scan-face speed somewhere (always assumed on non-uniform meshes)
    const bool need_scan = UNI ? (__syncthreads_or(vok && sA_u > real(0)) != 0) : true;
    auto speedA = [&](int q, int b) -> real {       // scan face q at row b
        if (UNI) return sA_u;
        size_t k = (size_t)(b - 1) * PA1 + (q - 1);
        return vx * A.gA1[k] + vy * A.gA2[k];
    };
    auto speedB = [&](int q, int a) -> real {       // march face q at cell a
        if (UNI) return sB_u;
        size_t k = (size_t)(q - 1) * PA + (a - 1);
        return vx * A.gB1[k] + vy * A.gB2[k];
    };
    // march-axis face flux at face q for cell a, component r, wall faces only
    auto fluxB_wall = [&](int q, int a, int r, real sp) -> real {
        const size_t o = (size_t)r * PA + pa(a);
        if (q == 1) return sp * fw_blo[((size_t)v * 2 + r) * PA + pa(a)];
        if (q == Nb + 1) return sp * fw_bhi[((size_t)v * 2 + r) * PA + pa(a)];
        if (q == 2) return flux_wlo<SCHEME>(sp, rowp(1)[o], rowp(2)[o], rowp(3)[o]);
        if (q == Nb) return flux_whi<SCHEME>(sp, rowp(Nb)[o], rowp(Nb - 1)[o], rowp(Nb - 2)[o]);
        return flux_std<SCHEME>(sp, rowp(q - 2)[o], rowp(q - 1)[o], rowp(q)[o], rowp(q + 1)[o]);
    };

    // ---- carried state per cell ------------------------------------------------
    real dG[CPT], dH[CPT];                 // forward values of the previous row
    real iap[CPT];                         // 1/alpha of the previous row
    real sAhp[CPT];                        // scan speed of face a+1, previous row
    real sBl[CPT];                         // march speed of face b (low face)
    real FBl_G[CPT], FBl_H[CPT];           // march flux through face b
#pragma unroll
    for (int k = 0; k < CPT; k++) {
        dG[k] = dH[k] = real(0);
        iap[k] = real(1);
        sAhp[k] = sBl[k] = FBl_G[k] = FBl_H[k] = real(0);
    }
    const real fl = Consts<real>::floor_();
    const real msc = A.mscale ? (real)*A.mscale : real(1);
    const real *ep = A.eqp;
    // CPT consecutive Shakhov parameters of the chunk (in the logical order)
    auto lde = [&](const real *p, real *o) {
        if (!ra) {
            Vec<real, CPT>::ld(p, o);
        } else {
            real t[CPT];
            Vec<real, CPT>::ld(p, t);
#pragma unroll
            for (int k = 0; k < CPT; k++) o[k] = t[CPT - 1 - k];
        }
    };

    for (int bp = -1; bp <= 2; bp++) wait_row(bp);
    // the copies of rows 1, 2 for rows Nb+1, Nb+2 read f rows that the
    // backward step overwrites from step 2 on: they complete before any write
    if (perB) {
        wait_row(Nb + 1);
        wait_row(Nb + 2);
    }
    if (act) {
#pragma unroll
        for (int k = 0; k < CPT; k++) {
            sBl[k] = speedB(1, a0 + k);
            if (perB) {
                const size_t o = pa(a0 + k);
                FBl_G[k] = flux_std<SCHEME>(sBl[k], rowp(-1)[o], rowp(0)[o], rowp(1)[o], rowp(2)[o]);
                FBl_H[k] = flux_std<SCHEME>(sBl[k], rowp(-1)[PA + o], rowp(0)[PA + o], rowp(1)[PA + o],
                                            rowp(2)[PA + o]);
            } else {
                FBl_G[k] = fluxB_wall(1, a0 + k, 0, sBl[k]);
                FBl_H[k] = fluxB_wall(1, a0 + k, 1, sBl[k]);
            }
        }
    }

    for (int b = 1; b <= Nb; b++) {
        // each thread waits on the row's mbarrier itself (that wait makes the
        // bulk copy visible); a timed-out wait is acted on at the row's one
        // block barrier below, before anything is written to f
        wait_row(b + 2);
        real pc[CPT], cG[CPT], cH[CPT], ia[CPT], sAh[CPT], sBh[CPT], FBh_G[CPT], FBh_H[CPT];
        real fo0[CPT], fo1[CPT];           // f of row b-1 (for the backward update)
        real P = real(1), CGt = real(0), CHt = real(0);
        if (act) {
            const real *rm = rowp(b - 1), *r0 = rowp(b), *rp = rowp(b + 1), *rq = rowp(b + 2);
            real f0[CPT], f1[CPT];
            ldc(r0, f0);
            ldc(r0 + PA, f1);
            // scan-axis window f(a0-2 .. a0+CPT+1)
            real w0[CPT + 4], w1[CPT + 4];
            w0[0] = r0[hm2]; w0[1] = r0[hm1]; w0[CPT + 2] = r0[hp0]; w0[CPT + 3] = r0[hp1];
            w1[0] = r0[PA + hm2]; w1[1] = r0[PA + hm1]; w1[CPT + 2] = r0[PA + hp0]; w1[CPT + 3] = r0[PA + hp1];
#pragma unroll
            for (int k = 0; k < CPT; k++) { w0[k + 2] = f0[k]; w1[k + 2] = f1[k]; }
            // scan-axis face fluxes, faces a0 .. a0+CPT
            real FA_G[CPT + 1], FA_H[CPT + 1], sAf[CPT + 1];
#pragma unroll
            for (int m = 0; m <= CPT; m++) {
                const int q = a0 + m;
                const real s = speedA(q, b);
                sAf[m] = s;
                if (!edgeA) {
                    FA_G[m] = flux_std<SCHEME>(s, w0[m], w0[m + 1], w0[m + 2], w0[m + 3]);
                    FA_H[m] = flux_std<SCHEME>(s, w1[m], w1[m + 1], w1[m + 2], w1[m + 3]);
                } else if (q == 1) {
                    FA_G[m] = s * fw_alo[((size_t)v * 2 + 0) * Nb + (prow(b) - 1)];
                    FA_H[m] = s * fw_alo[((size_t)v * 2 + 1) * Nb + (prow(b) - 1)];
                } else if (q == Na + 1) {
                    FA_G[m] = s * fw_ahi[((size_t)v * 2 + 0) * Nb + (prow(b) - 1)];
                    FA_H[m] = s * fw_ahi[((size_t)v * 2 + 1) * Nb + (prow(b) - 1)];
                } else if (q == 2) {
                    FA_G[m] = flux_wlo<SCHEME>(s, r0[pa(1)], r0[pa(2)], r0[pa(3)]);
                    FA_H[m] = flux_wlo<SCHEME>(s, r0[PA + pa(1)], r0[PA + pa(2)], r0[PA + pa(3)]);
                } else if (q == Na) {
                    FA_G[m] = flux_whi<SCHEME>(s, r0[pa(Na)], r0[pa(Na - 1)], r0[pa(Na - 2)]);
                    FA_H[m] = flux_whi<SCHEME>(s, r0[PA + pa(Na)], r0[PA + pa(Na - 1)], r0[PA + pa(Na - 2)]);
                } else {
                    FA_G[m] = flux_std<SCHEME>(s, w0[m], w0[m + 1], w0[m + 2], w0[m + 3]);
                    FA_H[m] = flux_std<SCHEME>(s, w1[m], w1[m + 1], w1[m + 2], w1[m + 3]);
                }
            }
            // rows b-1, b+1, b+2 at the thread's cells for the march faces
            real m0[CPT], m1[CPT];
            ldc(rm, m0);
            ldc(rm + PA, m1);
            const bool stdB = perB || (b + 1 >= 3 && b + 1 <= Nb - 1);
            // Shakhov parameters of the thread's cells
            const size_t prow0 = (size_t)(prow(b) - 1) * PA;    // physical row start
            const size_t cell0 = prow0 + pa0;
            real e_crt[CPT], e_u[CPT], e_v[CPT], e_it[CPT], e_ht[CPT], e_qx[CPT], e_qy[CPT], e_cf[CPT], vl[CPT];
            // the CPT cells of the chunk lie in one block of the parameter
            // layout (pa0 is a multiple of CPT, CPT divides the block)
            const real *ec = ep + hyb_eqp_at(cell0, 0);
            lde(ec + 0 * HYB_EQP_BLK, e_crt);
            lde(ec + 1 * HYB_EQP_BLK, e_u);
            lde(ec + 2 * HYB_EQP_BLK, e_v);
            lde(ec + 3 * HYB_EQP_BLK, e_it);
            lde(ec + 4 * HYB_EQP_BLK, e_ht);
            lde(ec + 5 * HYB_EQP_BLK, e_qx);
            lde(ec + 6 * HYB_EQP_BLK, e_qy);
            lde(ec + 7 * HYB_EQP_BLK, e_cf);
            if (!UNI) Vec<real, CPT>::ld(A.vol + cell0, vl);
            // the next row's Shakhov parameters towards L1 while this row
            // computes (one prefetch per 128-byte line)
            if (b < Nb && (pa0 * (int)sizeof(real)) % 128 == 0) {
                const size_t nxt = (size_t)(prow(b + 1) - 1) * PA + pa0;
#pragma unroll
                for (int q = 0; q < 8; q++)
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(ep + hyb_eqp_at(nxt, q)));
            }
            if (stdB) {
                real p0[CPT], p1[CPT], q0[CPT], q1[CPT];
                ldc(rp, p0);
                ldc(rp + PA, p1);
                ldc(rq, q0);
                ldc(rq + PA, q1);
#pragma unroll
                for (int k = 0; k < CPT; k++) {
                    sBh[k] = speedB(b + 1, a0 + k);
                    FBh_G[k] = flux_std<SCHEME>(sBh[k], m0[k], f0[k], p0[k], q0[k]);
                    FBh_H[k] = flux_std<SCHEME>(sBh[k], m1[k], f1[k], p1[k], q1[k]);
                }
            } else {
#pragma unroll
                for (int k = 0; k < CPT; k++) {
                    sBh[k] = speedB(b + 1, a0 + k);
                    FBh_G[k] = fluxB_wall(b + 1, a0 + k, 0, sBh[k]);
                    FBh_H[k] = fluxB_wall(b + 1, a0 + k, 1, sBh[k]);
                }
            }
            real rG[CPT], rH[CPT];
#pragma unroll
            for (int k = 0; k < CPT; k++) {
                fo0[k] = m0[k];
                fo1[k] = m1[k];
                real divG, divH;
                if (A.scan_is_j) {
                    divG = (FBh_G[k] - FBl_G[k]) + FA_G[k + 1] - FA_G[k];
                    divH = (FBh_H[k] - FBl_H[k]) + FA_H[k + 1] - FA_H[k];
                } else {
                    divG = (FA_G[k + 1] - FA_G[k]) + FBh_G[k] - FBl_G[k];
                    divH = (FA_H[k + 1] - FA_H[k]) + FBh_H[k] - FBl_H[k];
                }
                // Shakhov equilibrium (GKUA_Residual.f90:441-458)
                const real viu = vx - e_u[k], vjv = vy - e_v[k];
                const real vij2 = (viu * viu + vjv * vjv) * e_it[k];
                const real fvx = e_qx[k] * viu + e_qy[k] * vjv;
                const real gdv = e_crt[k] * sweep_exp<real>(-vij2);
                const real geq = gdv * (real(1) + fvx * (real(2) * vij2 - real(4)));
                const real heq = (e_ht[k] * gdv) * (real(1) + fvx * (real(2) * vij2 - real(2)));
                const real vol = UNI ? vol_u : vl[k];
                const real ivol = UNI ? ivol_u : sweep_rcp<real>(vol);
                rG[k] = -divG * ivol + e_cf[k] * (geq - f0[k]);
                rH[k] = -divH * ivol + e_cf[k] * (heq - f1[k]);
                // LU-SGS forward element (GKUA_Residual.f90:39-57)
                real alfa;
                if (UNI) alfa = abase_u + vol * e_cf[k];
                else
                    alfa = vol / dt + (posp(sAf[k + 1]) - negp(sAf[k]) + posp(sBh[k]) - negp(sBl[k])) +
                           vol * e_cf[k];
                ia[k] = sweep_rcp<real>(alfa);
                pc[k] = posp(sAf[k]) * ia[k];
                const real pb = posp(sBl[k]);
                cG[k] = (vol * rG[k] + pb * dG[k]) * ia[k];
                cH[k] = (vol * rH[k] + pb * dH[k]) * ia[k];
                sAh[k] = sAf[k + 1];
                // thread-local composition of the affine maps
                CGt = cG[k] + pc[k] * CGt;
                CHt = cH[k] + pc[k] * CHt;
                P = pc[k] * P;
            }
            if (A.rhs) {
                stc(A.rhs + vrow0 + prow0, rG);
                stc(A.rhs + vrow0 + rstride + prow0, rH);
            }
        } else {
#pragma unroll
            for (int k = 0; k < CPT; k++) {
                pc[k] = cG[k] = cH[k] = ia[k] = sAh[k] = sBh[k] = FBh_G[k] = FBh_H[k] = fo0[k] = fo1[k] = real(0);
            }
            P = real(0);
        }
        real Pe = real(1), Ge = real(0), He = real(0);
        real *aggb = agg + (size_t)(b & 1) * nw * 3;
        if (need_scan) {
            // inclusive warp scan of the composed maps (earlier lanes first)
            real Pi = P, Gi = CGt, Hi = CHt;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                real pu = __shfl_up_sync(0xffffffffu, Pi, off);
                real gu = __shfl_up_sync(0xffffffffu, Gi, off);
                real hu = __shfl_up_sync(0xffffffffu, Hi, off);
                if (lane >= off) {
                    Gi = Gi + Pi * gu;
                    Hi = Hi + Pi * hu;
                    Pi = Pi * pu;
                }
            }
            Pe = __shfl_up_sync(0xffffffffu, Pi, 1);
            Ge = __shfl_up_sync(0xffffffffu, Gi, 1);
            He = __shfl_up_sync(0xffffffffu, Hi, 1);
            if (lane == 0) { Pe = real(1); Ge = real(0); He = real(0); }
            if (lane == 31) {
                aggb[warp * 3 + 0] = Pi;
                aggb[warp * 3 + 1] = Gi;
                aggb[warp * 3 + 2] = Hi;
            }
        }
        if (__syncthreads_or(timeout)) {
            if (t == 0 && g == 0) atomicExch(A.err, HYB_ERR_TIMEOUT);
            if (producer) sweep_drain(bars, b, Nb, A.stall_row, A.spin);
            return;
        }
        // every thread is past this row's reads, so the slot of row b-3 is free
        if (producer) issue_row(b + RING - 3);
        real xG = Ge, xH = He;                              // dF just before cell a0
        if (need_scan && warp > 0) {
            real carG = real(0), carH = real(0);
            for (int w = 0; w < warp; w++) {
                const real pw = aggb[w * 3 + 0];
                carG = aggb[w * 3 + 1] + pw * carG;
                carH = aggb[w * 3 + 2] + pw * carH;
            }
            xG = Ge + Pe * carG;
            xH = He + Pe * carH;
        }
        real nG[CPT], nH[CPT];
#pragma unroll
        for (int k = 0; k < CPT; k++) {
            xG = cG[k] + pc[k] * xG;
            xH = cH[k] + pc[k] * xH;
            nG[k] = xG;
            nH[k] = xH;
        }
        real *dlb = dlf + (size_t)(b & 1) * 2 * TPV;
        dlb[t] = act ? nG[0] : real(0);
        dlb[TPV + t] = act ? nH[0] : real(0);
        // backward + update of row b-1 (GKUA_Residual.f90:64-109)
        if (b > 1 && act && !A.no_update) {
            const real *dlp = dlf + (size_t)((b - 1) & 1) * 2 * TPV;
            const bool has_next = (a0 + CPT <= Na);
            const real lastG = has_next ? dlp[t + 1] : real(0), lastH = has_next ? dlp[TPV + t + 1] : real(0);
            real uG[CPT], uH[CPT];
#pragma unroll
            for (int k = 0; k < CPT; k++) {
                const real nxG = (k + 1 < CPT) ? dG[k + 1] : lastG;
                const real nxH = (k + 1 < CPT) ? dH[k + 1] : lastH;
                const real ca = -negp(sAhp[k]);
                const real cb = -negp(sBl[k]);
                real fg = msc * (fo0[k] + (dG[k] + (ca * nxG + cb * nG[k]) * iap[k]));
                real fh = msc * (fo1[k] + (dH[k] + (ca * nxH + cb * nH[k]) * iap[k]));
                uG[k] = floor_at(fg, fl);
                uH[k] = floor_at(fh, fl);
            }
            const size_t c1 = (size_t)(prow(b - 1) - 1) * PA;
            stc(A.f + vrow0 + c1, uG);
            stc(A.f + vrow0 + rstride + c1, uH);
        }
#pragma unroll
        for (int k = 0; k < CPT; k++) {
            dG[k] = nG[k];
            dH[k] = nH[k];
            iap[k] = ia[k];
            sAhp[k] = sAh[k];
            sBl[k] = sBh[k];
            FBl_G[k] = FBh_G[k];
            FBl_H[k] = FBh_H[k];
        }
    }
    __syncthreads();
    if (act && !A.no_update) {   // backward + update of the last row (downstream values are 0)
        const real *dlp = dlf + (size_t)(Nb & 1) * 2 * TPV;
        const bool has_next = (a0 + CPT <= Na);
        const real *o0 = rowp(Nb);
        real f0[CPT], f1[CPT], uG[CPT], uH[CPT];
        ldc(o0, f0);
        ldc(o0 + PA, f1);
#pragma unroll
        for (int k = 0; k < CPT; k++) {
            const real nxG = (k + 1 < CPT) ? dG[k + 1] : (has_next ? dlp[t + 1] : real(0));
            const real nxH = (k + 1 < CPT) ? dH[k + 1] : (has_next ? dlp[TPV + t + 1] : real(0));
            const real ca = -negp(sAhp[k]);
            real fg = msc * (f0[k] + (dG[k] + (ca * nxG) * iap[k]));
            real fh = msc * (f1[k] + (dH[k] + (ca * nxH) * iap[k]));
            uG[k] = floor_at(fg, fl);
            uH[k] = floor_at(fh, fl);
        }
        const size_t c1 = (size_t)(prow(Nb) - 1) * PA;
        stc(A.f + vrow0 + c1, uG);
        stc(A.f + vrow0 + rstride + c1, uH);
    }
    // every bulk copy issued (rows 1..Nb and the wrap rows) has been waited
    // for above, so no copy is in flight when the CTA exits
}

template <typename real, int CPT, bool UNI, int SCHEME, bool UPW>
__global__ void __launch_bounds__(256, 2) k_sweep(KinArgs<real> A) {
    sweep_body<real, CPT, UNI, SCHEME, UPW>(A, blockIdx.x);
}

// many contexts of one launch shape in one launch: CTA i sweeps velocity
// block work[i].y of context work[i].x (arguments staged in shared memory)
template <typename real, int CPT, bool UNI, int SCHEME>
__global__ void __launch_bounds__(256, 2) k_sweep_batch(const KinArgs<real> *__restrict__ args,
                                                        const int2 *__restrict__ work) {
    __shared__ KinArgs<real> As;
    const int2 w = work[blockIdx.x];
    if (threadIdx.x == 0 && threadIdx.y == 0) As = args[w.x];
    __syncthreads();
    sweep_body<real, CPT, UNI, SCHEME>(As, w.y);
}

// ---- host side --------------------------------------------------------------
// launch = false only sets the kernel's shared-memory attribute (done before
// any stream capture of the launch)
template <typename real, int CPT, bool UNI, int SCHEME, bool UPW>
int sweep_launch_one(hyb_ctx *ctx, const KinArgs<real> &A, int vpb, bool launch) {
    const int tpv = ctx->PA / CPT;
    const size_t smem = sweep_group_bytes<real>(ctx->PA, tpv) * vpb;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_sweep<real, CPT, UNI, SCHEME, UPW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             227 * 1024);
        attr = true;
    }
    if (!launch) return HYB_OK;
    dim3 blk(tpv, vpb), grd((ctx->nv + vpb - 1) / vpb);
    k_sweep<real, CPT, UNI, SCHEME, UPW><<<grd, blk, smem, ctx->stream>>>(A);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ctx->last_error = std::string("k_sweep: ") + cudaGetErrorString(e);
        return HYB_ERR_CUDA;
    }
    return HYB_OK;
}

template <typename real, int CPT, bool UNI, bool UPW>
int sweep_launch_scheme(hyb_ctx *ctx, const KinArgs<real> &A, int vpb, bool launch) {
    switch (A.scheme) {
        case HYB_SCHEME_UP1: return sweep_launch_one<real, CPT, UNI, HYB_SCHEME_UP1, UPW>(ctx, A, vpb, launch);
        case HYB_SCHEME_WENO3: return sweep_launch_one<real, CPT, UNI, HYB_SCHEME_WENO3, UPW>(ctx, A, vpb, launch);
        default: return sweep_launch_one<real, CPT, UNI, HYB_SCHEME_NND, UPW>(ctx, A, vpb, launch);
    }
}

// the upwind order is instantiated for uniform meshes only (the context
// refuses it on other meshes)
template <typename real>
int sweep_launch_real(hyb_ctx *ctx, const KinArgs<real> &A, int cpt, int vpb, bool launch) {
    const bool u = ctx->uniform != 0;
    if (ctx->prm.sweep_order == HYB_SWEEP_UPWIND) {
        if (!u) return HYB_ERR_UNSUPPORTED;
        switch (cpt) {
            case 4: return sweep_launch_scheme<real, 4, true, true>(ctx, A, vpb, launch);
            case 2: return sweep_launch_scheme<real, 2, true, true>(ctx, A, vpb, launch);
            default: return sweep_launch_scheme<real, 1, true, true>(ctx, A, vpb, launch);
        }
    }
    switch (cpt) {
        case 4: return u ? sweep_launch_scheme<real, 4, true, false>(ctx, A, vpb, launch)
                         : sweep_launch_scheme<real, 4, false, false>(ctx, A, vpb, launch);
        case 2: return u ? sweep_launch_scheme<real, 2, true, false>(ctx, A, vpb, launch)
                         : sweep_launch_scheme<real, 2, false, false>(ctx, A, vpb, launch);
        default: return u ? sweep_launch_scheme<real, 1, true, false>(ctx, A, vpb, launch)
                          : sweep_launch_scheme<real, 1, false, false>(ctx, A, vpb, launch);
    }
}

template <typename real, int CPT, bool UNI, int SCHEME>
int sweep_batch_one(const KinArgs<real> *args, const int2 *work, int nwork, int PA, int vpb, cudaStream_t s) {
    const int tpv = PA / CPT;
    const size_t smem = sweep_group_bytes<real>(PA, tpv) * vpb;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_sweep_batch<real, CPT, UNI, SCHEME>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             227 * 1024 - 512);
        attr = true;
    }
    if (nwork <= 0) return HYB_OK;
    k_sweep_batch<real, CPT, UNI, SCHEME><<<nwork, dim3(tpv, vpb), smem, s>>>(args, work);
    return cudaGetLastError() == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
}

// batched sweeps exist for the NND scheme (the batched workloads' scheme);
// other schemes keep one launch per context
template <typename real>
int sweep_batch_real(const KinArgs<real> *args, const int2 *work, int nwork, int PA, int cpt, int vpb, bool uni,
                     int scheme, cudaStream_t s) {
    if (scheme != HYB_SCHEME_NND) return HYB_ERR_UNSUPPORTED;
    switch (cpt) {
        case 4: return uni ? sweep_batch_one<real, 4, true, HYB_SCHEME_NND>(args, work, nwork, PA, vpb, s)
                           : sweep_batch_one<real, 4, false, HYB_SCHEME_NND>(args, work, nwork, PA, vpb, s);
        case 2: return uni ? sweep_batch_one<real, 2, true, HYB_SCHEME_NND>(args, work, nwork, PA, vpb, s)
                           : sweep_batch_one<real, 2, false, HYB_SCHEME_NND>(args, work, nwork, PA, vpb, s);
        default: return uni ? sweep_batch_one<real, 1, true, HYB_SCHEME_NND>(args, work, nwork, PA, vpb, s)
                            : sweep_batch_one<real, 1, false, HYB_SCHEME_NND>(args, work, nwork, PA, vpb, s);
    }
}

}  // namespace hyb
