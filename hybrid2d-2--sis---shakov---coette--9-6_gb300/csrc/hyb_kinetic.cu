// hyb_kinetic.cu -- sm_103a kernels of the discrete-velocity Shakhov step.
//
//   k_wall      diffuse-wall slot values and n_w        GKUA_boundary_wall,
//               (GKUA_boundary.f90:49-100, GKUA_wall_functions.f90:1-199)
//   k_sweep     fused Get_Feq + RHSFDVsub + LU-SGS forward/backward + update
//               + floor, one velocity per thread group  (GKUA_Residual.f90)
//   k_moments   velocity moments + primitive conversion + CF (DETFP,
//               GKUA_DETFP.f90:4-151, 288-363)
//   k_residual  moments 1-4 of the stored RHS, rms / max (DETFP_res,
//               GKUA_DETFP_RES.f90:4-136)
//   k_init      uniform Maxwellian (GKUA_sudufenbu.f90:22-42)
//
// The fused sweep kernel walks the MARCH axis row by row.  Rows of f are
// staged into a shared-memory ring by cp.async.bulk copies completing on
// mbarriers (lookahead of three rows).  Within a row the forward recurrence
// dF(a) = c(a) + p(a) dF(a-1) is an affine scan across the threads; the
// recurrence along the march axis is carried in registers.  The backward
// step reads the forward values of its downstream neighbours only
// (GKUA_Residual.f90:64-90), so it runs one row behind the forward sweep and
// the forward values never leave the SM.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include "hyb_common.cuh"

namespace hyb {

// ---------------------------------------------------------------------------
// small device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ uint32_t mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void fence_async_shared() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// bounded wait: returns false when the spin limit ran out
// (about two seconds of SM clock; the normal wait is well under a microsecond)
#define HYB_SPIN_CYCLES 4000000000LL
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (clock64() - t0 < HYB_SPIN_CYCLES)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

template <typename real> __device__ __forceinline__ real posp(real a) { return (a + fabs(a)) * real(0.5); }
template <typename real> __device__ __forceinline__ real negp(real a) { return (a - fabs(a)) * real(0.5); }

// FMINMD, Functions.f90:10-25
template <typename real> __device__ __forceinline__ real fminmd(real x, real y) {
    if ((x > real(0) && y > real(0)) || (x < real(0) && y < real(0))) return (fabs(x) <= fabs(y)) ? x : y;
    return real(0);
}

template <typename real> __device__ __forceinline__ real dexp(real x);
template <> __device__ __forceinline__ float dexp<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double dexp<double>(double x) { return exp(x); }

template <typename real> struct Consts {
    static __device__ __forceinline__ real eps_weno() { return real(HYB_EPSWENO_D); }
    static __device__ __forceinline__ real c1() { return real(HYB_CWENO1_D); }
    static __device__ __forceinline__ real c2() { return real(HYB_CWENO2_D); }
    static __device__ __forceinline__ real floor_() { return real(HYB_FLOOR_D); }
};

// Standard face reconstruction from f(q-2), f(q-1), f(q), f(q+1)
// (RHSFDVsub, GKUA_Residual.f90:155-185): returns asp*UL + asn*UR.
template <typename real>
__device__ __forceinline__ real face_flux(int scheme, real asp, real asn, real u1, real u2, real u3, real u4) {
    if (scheme == HYB_SCHEME_UP1) return asp * u2 + asn * u3;
    real d0 = u3 - u2, dm = u2 - u1, dp = u4 - u3;
    if (scheme == HYB_SCHEME_NND) {
        real ul = u2 + real(0.5) * fminmd(d0, dm);
        real ur = u3 - real(0.5) * fminmd(d0, dp);
        return asp * ul + asn * ur;
    }
    const real e = Consts<real>::eps_weno(), c1 = Consts<real>::c1(), c2 = Consts<real>::c2();
    real is1 = dm * dm, is2 = d0 * d0, is3 = dp * dp;
    real a1 = c1 / ((is1 + e) * (is1 + e)), a2 = c2 / ((is2 + e) * (is2 + e));
    real a = a1 + a2, o1 = a1 / a, o2 = a2 / a;
    real ul = o1 * (real(-0.5) * u1 + real(1.5) * u2) + o2 * (real(0.5) * u2 + real(0.5) * u3);
    a1 = c2 / ((is2 + e) * (is2 + e));
    a2 = c1 / ((is3 + e) * (is3 + e));
    a = a1 + a2;
    o1 = a1 / a;
    o2 = a2 / a;
    real ur = o1 * (real(0.5) * u2 + real(0.5) * u3) + o2 * (real(1.5) * u3 - real(0.5) * u4);
    return asp * ul + asn * ur;
}

// Face 2 next to a low-end wall, f1=f(1), f2=f(2), f3=f(3)
// (GKUA_Residual.f90:196-221, 327-352)
template <typename real>
__device__ __forceinline__ real face_flux_wall_lo(int scheme, real asp, real asn, real f1, real f2, real f3) {
    if (scheme == HYB_SCHEME_UP1) return asp * f1 + asn * f2;
    if (scheme == HYB_SCHEME_WENO3) {
        const real e = Consts<real>::eps_weno(), c1 = Consts<real>::c1(), c2 = Consts<real>::c2();
        real is2 = (f2 - f1) * (f2 - f1), is3 = (f3 - f2) * (f3 - f2);
        real ul = real(0.5) * (f1 + f2);
        real a1 = c2 / ((is2 + e) * (is2 + e)), a2 = c1 / ((is3 + e) * (is3 + e));
        real a = a1 + a2, o1 = a1 / a, o2 = a2 / a;
        real ur = o1 * (real(0.5) * f1 + real(0.5) * f2) + o2 * (real(1.5) * f2 - real(0.5) * f3);
        return asp * ul + asn * ur;
    }
    real ul = f1 + real(0.5) * (f2 - f1);
    real ur = f2 - real(0.5) * fminmd(f2 - f1, f3 - f2);
    return asp * ul + asn * ur;
}

// Face n next to a high-end wall, f1=f(n-1), f2=f(n-2), f3=f(n-3) in cell
// numbering of the reference (GKUA_Residual.f90:233-257, 362-387)
template <typename real>
__device__ __forceinline__ real face_flux_wall_hi(int scheme, real asp, real asn, real f1, real f2, real f3) {
    if (scheme == HYB_SCHEME_UP1) return asp * f2 + asn * f1;
    if (scheme == HYB_SCHEME_WENO3) {
        const real e = Consts<real>::eps_weno(), c1 = Consts<real>::c1(), c2 = Consts<real>::c2();
        real is1 = (f2 - f3) * (f2 - f3), is2 = (f1 - f2) * (f1 - f2);
        real a1 = c1 / ((is1 + e) * (is1 + e)), a2 = c2 / ((is2 + e) * (is2 + e));
        real a = a1 + a2, o1 = a1 / a, o2 = a2 / a;
        real ul = o1 * (real(-0.5) * f3 + real(1.5) * f2) + o2 * (real(0.5) * f2 + real(0.5) * f1);
        real ur = real(0.5) * f2 + real(0.5) * f1;
        return asp * ul + asn * ur;
    }
    real ul = f2 + real(0.5) * fminmd(f1 - f2, f2 - f3);
    real ur = f1 - real(0.5) * (f1 - f2);
    return asp * ul + asn * ur;
}

// ---------------------------------------------------------------------------
// fused kinetic sweep
// ---------------------------------------------------------------------------
constexpr int RING = 8;   // staged rows per velocity (b-2 .. b+2 plus 3 ahead)

template <typename real>
struct SweepSmem {
    // per velocity group: bars[RING+2], ring[RING][2][PA], wrap[2][2][PA],
    // dl[2][2][PA], agg[2][nw][3]
    static __host__ __device__ size_t group_bytes(int PA) {
        size_t nw = (size_t)PA / 32;
        size_t b = 128;   // barriers (RING+2)*8 <= 80, padded
        b += (size_t)RING * 2 * PA * sizeof(real);
        b += (size_t)2 * 2 * PA * sizeof(real);
        b += (size_t)2 * 2 * PA * sizeof(real);
        b += (size_t)2 * nw * 3 * sizeof(real);
        return (b + 127) / 128 * 128;
    }
};

template <typename real>
__global__ void __launch_bounds__(1024) k_sweep(KinArgs<real> A) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int PA = A.PA, Na = A.Na, Nb = A.Nb;
    const int g = threadIdx.y;                 // velocity group in the CTA
    const int t = threadIdx.x;                 // scan position a-1
    const int a = t + 1;
    const int lane = t & 31, warp = t >> 5, nw = PA >> 5;
    const int v = blockIdx.x * blockDim.y + g;
    const bool vok = v < A.nv;
    const bool act = vok && (a <= Na);
    const bool producer = (t == 0) && vok;

    unsigned char *base = smem_raw + (size_t)g * SweepSmem<real>::group_bytes(PA);
    uint64_t *bars = reinterpret_cast<uint64_t *>(base);
    real *ring = reinterpret_cast<real *>(base + 128);
    real *wrap = ring + (size_t)RING * 2 * PA;
    real *dl = wrap + (size_t)2 * 2 * PA;
    real *agg = dl + (size_t)2 * 2 * PA;

    const bool perB = (A.bcb_lo == AX_PERIODIC);
    const bool perA = (A.bca_lo == AX_PERIODIC);
    const size_t vrow0 = vok ? (size_t)v * 2 * Nb * PA : 0;   // f offset of (v, r=0, b=1)
    const size_t rstride = (size_t)Nb * PA;                    // r=0 -> r=1
    const uint32_t row_bytes = (uint32_t)(PA * sizeof(real));

    // logical row bp (-1..Nb) -> physical 1-based row, or 0 when not loaded
    auto phys_row = [&](int bp) -> int {
        if (bp >= 1 && bp <= Nb) return bp;
        if (perB && bp <= 0) return bp + Nb;
        return 0;
    };
    auto issue_row = [&](int bp) {   // producer only; bp >= -1
        int s = (bp + 1) % RING;
        int pr = phys_row(bp);
        if (pr > 0 && bp <= Nb) {
            mbar_arrive_expect_tx(&bars[s], 2 * row_bytes);
            const real *src = A.f + vrow0 + (size_t)(pr - 1) * PA;
            bulk_g2s(ring + (size_t)s * 2 * PA, src, row_bytes, &bars[s]);
            bulk_g2s(ring + (size_t)s * 2 * PA + PA, src + rstride, row_bytes, &bars[s]);
        } else {
            mbar_arrive(&bars[s]);   // keep the slot's phase sequence
        }
    };

    if (producer) {
        for (int s = 0; s < RING + 2; s++) mbar_init(&bars[s], 1);
        fence_async_shared();
    }
    __syncthreads();
    if (producer) {
        // rows -1 .. RING-3 fill slots 0 .. RING-2; step b refills the slot of
        // row b-3 with row b+RING-3 (slot RING-1 is first filled at step 1)
        for (int bp = -1; bp <= RING - 3; bp++) issue_row(bp);
        if (perB) {   // rows Nb+1, Nb+2 are the old rows 1, 2
            for (int w = 0; w < 2; w++) {
                mbar_arrive_expect_tx(&bars[RING + w], 2 * row_bytes);
                const real *src = A.f + vrow0 + (size_t)w * PA;
                bulk_g2s(wrap + (size_t)w * 2 * PA, src, row_bytes, &bars[RING + w]);
                bulk_g2s(wrap + (size_t)w * 2 * PA + PA, src + rstride, row_bytes, &bars[RING + w]);
            }
        }
    }

    // row pointer of logical row bp for component r
    auto rowp = [&](int bp, int r) -> const real * {
        if (bp > Nb) return wrap + (size_t)(bp - Nb - 1) * 2 * PA + (size_t)r * PA;
        int s = (bp + 1) % RING;
        return ring + (size_t)s * 2 * PA + (size_t)r * PA;
    };
    // wait (all threads) for logical row bp
    bool timeout = false;
    auto wait_row = [&](int bp) {
        if (!vok) return;
        if (bp > Nb) {
            if (!perB) return;
            if (!mbar_wait_bounded(&bars[RING + (bp - Nb - 1)], 0)) timeout = true;
            return;
        }
        if (phys_row(bp) == 0) return;
        int s = (bp + 1) % RING;
        uint32_t par = (uint32_t)(((bp + 1) / RING) & 1);
        if (!mbar_wait_bounded(&bars[s], par)) timeout = true;
    };

    // velocity of this group
    const int iv = vok ? v % A.nvi : 0, jv = vok ? v / A.nvi : 0;
    const real vx = vok ? (real)A.vx[iv] : real(0), vy = vok ? (real)A.vy[jv] : real(0);
    const int scheme = A.scheme;
    const real dt = A.dt;
    const int PA1 = PA + 1;

    // face speed along the scan axis (face q at row b), along the march axis
    auto speedA = [&](int q, int b) -> real {
        size_t k = (size_t)(b - 1) * PA1 + (q - 1);
        return vx * A.gA1[k] + vy * A.gA2[k];
    };
    auto speedB = [&](int q, int a_) -> real {
        size_t k = (size_t)(q - 1) * PA + (a_ - 1);
        return vx * A.gB1[k] + vy * A.gB2[k];
    };
    // scan-axis face flux at face q (1..Na+1) in row b (pointer = row data)
    auto fluxA = [&](int q, int b, const real *row, int r, real sp) -> real {
        real asp = posp(sp), asn = negp(sp);
        if (!perA) {
            if (q == 1) {
                const real *fw = A.fw_alo + ((size_t)v * 2 + r) * Nb;
                return sp * fw[b - 1];
            }
            if (q == Na + 1) {
                const real *fw = A.fw_ahi + ((size_t)v * 2 + r) * Nb;
                return sp * fw[b - 1];
            }
            if (q == 2) return face_flux_wall_lo(scheme, asp, asn, row[0], row[1], row[2]);
            if (q == Na) return face_flux_wall_hi(scheme, asp, asn, row[Na - 1], row[Na - 2], row[Na - 3]);
            return face_flux(scheme, asp, asn, row[q - 3], row[q - 2], row[q - 1], row[q]);
        }
        auto w = [&](int c) { return row[((c - 1 + 2 * Na) % Na)]; };   // c is a 1-based cell
        return face_flux(scheme, asp, asn, w(q - 2), w(q - 1), w(q), w(q + 1));
    };
    // march-axis face flux at face q (1..Nb+1) for scan position a
    auto fluxB = [&](int q, int r, real sp) -> real {
        real asp = posp(sp), asn = negp(sp);
        const int ai = a - 1;
        if (!perB) {
            if (q == 1) return sp * A.fw_blo[((size_t)v * 2 + r) * PA + ai];
            if (q == Nb + 1) return sp * A.fw_bhi[((size_t)v * 2 + r) * PA + ai];
            if (q == 2) return face_flux_wall_lo(scheme, asp, asn, rowp(1, r)[ai], rowp(2, r)[ai], rowp(3, r)[ai]);
            if (q == Nb)
                return face_flux_wall_hi(scheme, asp, asn, rowp(Nb, r)[ai], rowp(Nb - 1, r)[ai], rowp(Nb - 2, r)[ai]);
        }
        return face_flux(scheme, asp, asn, rowp(q - 2, r)[ai], rowp(q - 1, r)[ai], rowp(q, r)[ai],
                         rowp(q + 1, r)[ai]);
    };

    // per-step carried state
    real dG_prev = 0, dH_prev = 0;       // forward values of row b-1 at this a
    real alfa_prev = 1, sAhi_prev = 0;   // alpha and scan-face speed A(a+1) of row b-1
    real sBlo = 0, FBlo_G = 0, FBlo_H = 0;
    const real *ep = A.eqp;
    const size_t ncell = (size_t)Nb * PA;

    // prologue waits: rows -1..2
    for (int bp = -1; bp <= 2; bp++) wait_row(bp);
    if (act) {
        sBlo = speedB(1, a);
        FBlo_G = fluxB(1, 0, sBlo);
        FBlo_H = fluxB(1, 1, sBlo);
    }

    for (int b = 1; b <= Nb; b++) {
        wait_row(b + 2);
        if (__syncthreads_or(timeout)) {
            if (t == 0 && g == 0) atomicExch(A.err, HYB_ERR_TIMEOUT);
            return;
        }
        const size_t cell = (size_t)(b - 1) * PA + (a - 1);
        real p = 0, cG = 0, cH = 0, alfa = 1, sAlo = 0, sAhi = 0, rhsG = 0, rhsH = 0, vol = 1;
        real sBhi = 0, FBhi_G = 0, FBhi_H = 0;
        if (act) {
            const real *r0 = rowp(b, 0), *r1 = rowp(b, 1);
            sAlo = speedA(a, b);
            sAhi = speedA(a + 1, b);
            sBhi = speedB(b + 1, a);
            real FAlo_G = fluxA(a, b, r0, 0, sAlo), FAhi_G = fluxA(a + 1, b, r0, 0, sAhi);
            real FAlo_H = fluxA(a, b, r1, 1, sAlo), FAhi_H = fluxA(a + 1, b, r1, 1, sAhi);
            FBhi_G = fluxB(b + 1, 0, sBhi);
            FBhi_H = fluxB(b + 1, 1, sBhi);
            // flux balance in the reference's order: i-difference, then j
            real divG, divH;
            if (A.scan_is_j) {
                divG = (FBhi_G - FBlo_G) + FAhi_G - FAlo_G;
                divH = (FBhi_H - FBlo_H) + FAhi_H - FAlo_H;
            } else {
                divG = (FAhi_G - FAlo_G) + FBhi_G - FBlo_G;
                divH = (FAhi_H - FAlo_H) + FBhi_H - FBlo_H;
            }
            // Shakhov equilibrium, Get_Feq (GKUA_Residual.f90:441-458)
            real crt = ep[0 * ncell + cell], uu = ep[1 * ncell + cell], vv = ep[2 * ncell + cell];
            real it_ = ep[3 * ncell + cell], ht = ep[4 * ncell + cell];
            real cqx = ep[5 * ncell + cell], cqy = ep[6 * ncell + cell], cf = ep[7 * ncell + cell];
            vol = A.vol[cell];
            real viu = vx - uu, vjv = vy - vv;
            real vij2 = (viu * viu + vjv * vjv) * it_;
            real fvx = cqx * viu + cqy * vjv;
            real gdv = crt * dexp<real>(-vij2);
            real geq = gdv * (real(1) + fvx * (real(2) * vij2 - real(4)));
            real heq = (ht * gdv) * (real(1) + fvx * (real(2) * vij2 - real(2)));
            real fG = r0[a - 1], fH = r1[a - 1];
            rhsG = -divG / vol + cf * (geq - fG);
            rhsH = -divH / vol + cf * (heq - fH);
            if (A.rhs) {
                A.rhs[vrow0 + cell] = rhsG;
                A.rhs[vrow0 + rstride + cell] = rhsH;
            }
            // LU-SGS forward element (GKUA_Residual.f90:39-57)
            alfa = vol / dt + (posp(sAhi) - negp(sAlo) + posp(sBhi) - negp(sBlo)) + vol * cf;
            real ia = real(1) / alfa;
            p = posp(sAlo) * ia;
            real pb = posp(sBlo);
            cG = (vol * rhsG + pb * dG_prev) * ia;
            cH = (vol * rhsH + pb * dH_prev) * ia;
        }
        // affine inclusive scan along the scan axis
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            real pu = __shfl_up_sync(0xffffffffu, p, off);
            real gu = __shfl_up_sync(0xffffffffu, cG, off);
            real hu = __shfl_up_sync(0xffffffffu, cH, off);
            if (lane >= off) {
                cG = cG + p * gu;
                cH = cH + p * hu;
                p = p * pu;
            }
        }
        real *aggb = agg + (size_t)(b & 1) * nw * 3;
        if (lane == 31) {
            aggb[warp * 3 + 0] = p;
            aggb[warp * 3 + 1] = cG;
            aggb[warp * 3 + 2] = cH;
        }
        __syncthreads();
        // producer refills the slot of row b-3 with row b+RING-3
        if (producer) issue_row(b + RING - 3);
        real carG = 0, carH = 0;
        for (int w = 0; w < warp; w++) {
            real pw = aggb[w * 3 + 0];
            carG = aggb[w * 3 + 1] + pw * carG;
            carH = aggb[w * 3 + 2] + pw * carH;
        }
        real dG = cG + p * carG, dH = cH + p * carH;
        real *dlb = dl + (size_t)(b & 1) * 2 * PA;
        dlb[t] = act ? dG : real(0);
        dlb[PA + t] = act ? dH : real(0);
        // backward + update of row b-1 (GKUA_Residual.f90:64-109)
        if (b > 1 && act) {
            const real *dlp = dl + (size_t)((b - 1) & 1) * 2 * PA;
            real nG = (a < Na) ? dlp[t + 1] : real(0);
            real nH = (a < Na) ? dlp[PA + t + 1] : real(0);
            real cb = -negp(sBlo);     // -neg(B(b)) with B(b) = face between rows b-1 and b
            real ca = -negp(sAhi_prev);
            real duG = dG_prev + (ca * nG + cb * dG) / alfa_prev;
            real duH = dH_prev + (ca * nH + cb * dH) / alfa_prev;
            const real *o0 = rowp(b - 1, 0), *o1 = rowp(b - 1, 1);
            real fg = o0[a - 1] + duG, fh = o1[a - 1] + duH;
            const real fl = Consts<real>::floor_();
            if (fg < fl) fg = fl;
            if (fh < fl) fh = fl;
            size_t c1 = (size_t)(b - 2) * PA + (a - 1);
            A.f[vrow0 + c1] = fg;
            A.f[vrow0 + rstride + c1] = fh;
        }
        dG_prev = dG;
        dH_prev = dH;
        alfa_prev = alfa;
        sAhi_prev = sAhi;
        sBlo = sBhi;
        FBlo_G = FBhi_G;
        FBlo_H = FBhi_H;
    }
    __syncthreads();
    if (act) {   // backward + update of the last row (downstream values are 0)
        const real *dlp = dl + (size_t)(Nb & 1) * 2 * PA;
        real nG = (a < Na) ? dlp[t + 1] : real(0);
        real nH = (a < Na) ? dlp[PA + t + 1] : real(0);
        real ca = -negp(sAhi_prev);
        real duG = dG_prev + (ca * nG) / alfa_prev;
        real duH = dH_prev + (ca * nH) / alfa_prev;
        const real *o0 = rowp(Nb, 0), *o1 = rowp(Nb, 1);
        real fg = o0[a - 1] + duG, fh = o1[a - 1] + duH;
        const real fl = Consts<real>::floor_();
        if (fg < fl) fg = fl;
        if (fh < fl) fh = fl;
        size_t c1 = (size_t)(Nb - 1) * PA + (a - 1);
        A.f[vrow0 + c1] = fg;
        A.f[vrow0 + rstride + c1] = fh;
    }
    // every bulk copy issued (rows 1..Nb and the wrap rows) has been waited
    // for above, so no copy is in flight when the CTA exits
}

// ---------------------------------------------------------------------------
// diffuse wall: one CTA per wall face cell
// ---------------------------------------------------------------------------
struct WallFace {
    // position of the face cells in the (a,b) layout
    int on_scan;      // 1: wall at a scan-axis end (cells along b), 0: march end
    int hi;           // 1: high end
    int nfc;          // face cells
};

template <typename real>
__global__ void k_wall(const real *__restrict__ f, real *__restrict__ fw, const double *__restrict__ wd,
                       const double *__restrict__ vx, const double *__restrict__ vy, const double *__restrict__ w,
                       int nvi, int nv, int Na, int Nb, int PA, int on_scan, int hi) {
    const int k = blockIdx.x;   // face cell (0-based, face order)
    // wall data: [k][6] = u, v, t, swnx, swny, step
    const double uw = wd[k * 6 + 0], vw = wd[k * 6 + 1], tw = wd[k * 6 + 2];
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
    double s0 = 0.0, s1 = 0.0;
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
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
        double fb = (vnw + fabs(vnw)) / 2.0 * exp(-((vxx - uw) * (vxx - uw) + (vyy - vw) * (vyy - vw)) / tw) /
                    (HYB_PI * tw);
        s1 += wt * fb;
    }
    __shared__ double r0[256], r1[256];
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
    const double nwall = -r0[0] / r1[0];
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
        double vxx = vx[v % nvi], vyy = vy[v / nvi];
        double vnw = ((vxx - uw) * swnx + (vyy - vw) * swny) * step;
        if (vnw >= 0.0) {
            double cv = (vxx - uw) * (vxx - uw) + (vyy - vw) * (vyy - vw);
            double gg = nwall * exp(-cv / tw) / (HYB_PI * tw);
            fw[((size_t)v * 2 + 0) * nslot + k] = (real)gg;
            fw[((size_t)v * 2 + 1) * nslot + k] = (real)(tw * gg / 2.0);
        }
    }
}

// ---------------------------------------------------------------------------
// moments: one thread per (cell, velocity slice); FP64 accumulation, or in
// mixed mode FP32 Kahan-compensated partial sums over each velocity row
// folded into FP64.
// ---------------------------------------------------------------------------
struct MomArgs {
    const void *f;
    double *S;          // [NSUM][(nx+3)(ny+3)]
    double *CF;         // [(nx+3)(ny+3)]
    void *eqp;          // [8][Nb*PA] real
    const double *vx, *vy, *w;
    int nvi, nv, Na, Nb, PA, nx, ny, scan_is_j;
    double cfc, cpr, x1s, r00, t00;
};

template <typename real> struct KahanAcc;
template <> struct KahanAcc<double> {
    double s;
    __device__ void zero() { s = 0; }
    __device__ void add(double x) { s += x; }
    __device__ double fold() { double r = s; s = 0; return r; }
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
    __device__ double fold() { double r = (double)s - (double)c; s = 0.f; c = 0.f; return r; }
};

template <typename real, int VS>
__global__ void __launch_bounds__(32 * VS) k_moments(MomArgs M) {
    const int tx = threadIdx.x, sl = threadIdx.y;
    const int a = blockIdx.x * 32 + tx + 1, b = blockIdx.y + 1;
    const bool act = a <= M.Na;
    const size_t cell = (size_t)(b - 1) * M.PA + (a - 1);
    const size_t rs = (size_t)M.Nb * M.PA;
    const real *f = (const real *)M.f;
    double acc[10];
#pragma unroll
    for (int k = 0; k < 10; k++) acc[k] = 0.0;
    // velocity slice: whole velocity rows jv = sl, sl+VS, ...
    const int nvj = M.nv / M.nvi;
    if (act) {
        for (int jv = sl; jv < nvj; jv += VS) {
            KahanAcc<real> s[10];
#pragma unroll
            for (int k = 0; k < 10; k++) s[k].zero();
            const real vy = (real)M.vy[jv];
            for (int iv = 0; iv < M.nvi; iv++) {
                int v = iv + M.nvi * jv;
                const real vx = (real)M.vx[iv];
                const real wv = (real)M.w[v];
                real gg = f[(size_t)v * 2 * rs + cell], hh = f[(size_t)v * 2 * rs + rs + cell];
                real vxg = vx * gg, vyg = vy * gg, vx2g = vx * vxg, vy2g = vy * vyg;
                real b4 = hh + vx2g + vy2g;
                s[0].add(wv * gg);
                s[1].add(wv * vxg);
                s[2].add(wv * vyg);
                s[3].add(wv * b4);
                s[4].add(wv * vx2g);
                s[5].add(wv * vy2g);
                s[6].add(wv * (vx * vy * gg));
                s[7].add(wv * (vx * b4));
                s[8].add(wv * (vy * b4));
                s[9].add(wv * hh);
            }
#pragma unroll
            for (int k = 0; k < 10; k++) acc[k] += s[k].fold();
        }
    }
    __shared__ double red[VS][10][33];
#pragma unroll
    for (int k = 0; k < 10; k++) red[sl][k][tx] = acc[k];
    __syncthreads();
    if (sl != 0 || !act) return;
    double s[10];
#pragma unroll
    for (int k = 0; k < 10; k++) {
        double x = 0.0;
        for (int q = 0; q < VS; q++) x += red[q][k][tx];
        s[k] = x;
    }
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
    const size_t ncell = (size_t)M.Nb * M.PA;
    double cpt = M.cpr / (S1 * tt * tt);
    ep[0 * ncell + cell] = (real)(S1 / (HYB_PI * tt));
    ep[1 * ncell + cell] = (real)u;
    ep[2 * ncell + cell] = (real)vv;
    ep[3 * ncell + cell] = (real)(1.0 / tt);
    ep[4 * ncell + cell] = (real)(tt / 2.0);
    ep[5 * ncell + cell] = (real)(cpt * qx);
    ep[6 * ncell + cell] = (real)(cpt * qy);
    ep[7 * ncell + cell] = (real)cf;
}

// ---------------------------------------------------------------------------
// residual: moments 1..4 of the stored RHS per cell, then rms / max
// ---------------------------------------------------------------------------
template <typename real, int VS>
__global__ void __launch_bounds__(32 * VS) k_residual(const real *__restrict__ rhs, const double *__restrict__ vx,
                                                       const double *__restrict__ vy, const double *__restrict__ w,
                                                       int nvi, int nv, int Na, int Nb, int PA,
                                                       double *__restrict__ part) {
    const int tx = threadIdx.x, sl = threadIdx.y;
    const int a = blockIdx.x * 32 + tx + 1, b = blockIdx.y + 1;
    const bool act = a <= Na;
    const size_t cell = (size_t)(b - 1) * PA + (a - 1);
    const size_t rs = (size_t)Nb * PA;
    double acc[4] = {0, 0, 0, 0};
    const int nvj = nv / nvi;
    if (act) {
        for (int jv = sl; jv < nvj; jv += VS) {
            KahanAcc<real> s[4];
#pragma unroll
            for (int k = 0; k < 4; k++) s[k].zero();
            const real vyy = (real)vy[jv];
            for (int iv = 0; iv < nvi; iv++) {
                int v = iv + nvi * jv;
                const real vxx = (real)vx[iv];
                const real wv = (real)w[v];
                real gg = rhs[(size_t)v * 2 * rs + cell], hh = rhs[(size_t)v * 2 * rs + rs + cell];
                real vxg = vxx * gg, vyg = vyy * gg;
                s[0].add(wv * gg);
                s[1].add(wv * vxg);
                s[2].add(wv * vyg);
                s[3].add(wv * (hh + vxx * vxg + vyy * vyg));
            }
#pragma unroll
            for (int k = 0; k < 4; k++) acc[k] += s[k].fold();
        }
    }
    __shared__ double red[VS][4][33];
#pragma unroll
    for (int k = 0; k < 4; k++) red[sl][k][tx] = acc[k];
    __syncthreads();
    // per-cell value, then block max and sum of squares (deterministic)
    __shared__ double cellv[4][32];
    if (sl == 0) {
        for (int k = 0; k < 4; k++) {
            double x = 0.0;
            for (int q = 0; q < VS; q++) x += red[q][k][tx];
            cellv[k][tx] = act ? x : 0.0;
        }
    }
    __syncthreads();
    if (sl == 0 && tx < 4) {
        double mx = 0.0, ss = 0.0;
        for (int q = 0; q < 32; q++) {
            double x = cellv[tx][q];
            if (fabs(x) > mx || x != x) mx = fabs(x);
            ss += x * x;
        }
        size_t blk = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
        part[blk * 8 + tx] = mx;
        part[blk * 8 + 4 + tx] = ss;
    }
}

__global__ void k_residual_final(const double *__restrict__ part, int nblk, double ncell, double *__restrict__ out) {
    // one warp per component pair; deterministic sequential fold per lane
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

int launch_wall(hyb_ctx *ctx) {
    for (int face = 1; face <= 4; face++) {
        if (ctx->bc[face - 1] != HYB_BC_WALL) continue;
        int on_scan, hi;
        face_role(ctx, face, &on_scan, &hi);
        int nfc = (face == 1 || face == 3) ? ctx->ncy : ctx->ncx;
        const double *wd = ctx->d_wall + (size_t)(face - 1) * 6 * 4096;
        if (ctx->precision == HYB_PREC_FP64)
            k_wall<double><<<nfc, 256, 0, ctx->stream>>>((const double *)ctx->d_f, (double *)ctx->d_fw[face - 1], wd,
                                                          ctx->d_vx, ctx->d_vy, ctx->d_w, ctx->nvi, ctx->nv, ctx->Na,
                                                          ctx->Nb, ctx->PA, on_scan, hi);
        else
            k_wall<float><<<nfc, 256, 0, ctx->stream>>>((const float *)ctx->d_f, (float *)ctx->d_fw[face - 1], wd,
                                                         ctx->d_vx, ctx->d_vy, ctx->d_w, ctx->nvi, ctx->nv, ctx->Na,
                                                         ctx->Nb, ctx->PA, on_scan, hi);
        ctx->launches++;
        int rc = check_err(ctx, "k_wall");
        if (rc) return rc;
    }
    return HYB_OK;
}

template <typename real>
static int launch_sweep_t(hyb_ctx *ctx, int store_rhs) {
    KinArgs<real> A;
    A.f = (real *)ctx->d_f;
    A.rhs = store_rhs ? (real *)ctx->d_rhs : nullptr;
    A.fw_alo = A.fw_ahi = A.fw_blo = A.fw_bhi = nullptr;
    for (int face = 1; face <= 4; face++) {
        if (ctx->bc[face - 1] != HYB_BC_WALL) continue;
        int on_scan, hi;
        face_role(ctx, face, &on_scan, &hi);
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
    int vpb = 256 / ctx->PA;
    if (vpb < 1) vpb = 1;
    if (vpb > 8) vpb = 8;
    size_t smem = SweepSmem<real>::group_bytes(ctx->PA) * vpb;
    static bool attr_set[2] = {false, false};
    int idx = sizeof(real) == 8 ? 1 : 0;
    if (!attr_set[idx]) {
        cudaFuncSetAttribute(k_sweep<real>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        attr_set[idx] = true;
    }
    dim3 blk(ctx->PA, vpb), grd((ctx->nv + vpb - 1) / vpb);
    k_sweep<real><<<grd, blk, smem, ctx->stream>>>(A);
    ctx->launches++;
    return check_err(ctx, "k_sweep");
}

int launch_sweep(hyb_ctx *ctx, int store_rhs) {
    if (ctx->precision == HYB_PREC_FP64) return launch_sweep_t<double>(ctx, store_rhs);
    return launch_sweep_t<float>(ctx, store_rhs);
}

int launch_moments(hyb_ctx *ctx) {
    MomArgs M;
    M.f = ctx->d_f;
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
    M.cfc = ctx->prm.cfc;
    M.cpr = ctx->prm.cpr;
    M.x1s = ctx->prm.x1s;
    M.r00 = ctx->prm.r00;
    M.t00 = ctx->prm.t00;
    constexpr int VS = 8;
    dim3 blk(32, VS), grd((ctx->Na + 31) / 32, ctx->Nb);
    if (ctx->precision == HYB_PREC_FP64) k_moments<double, VS><<<grd, blk, 0, ctx->stream>>>(M);
    else k_moments<float, VS><<<grd, blk, 0, ctx->stream>>>(M);
    ctx->launches++;
    return check_err(ctx, "k_moments");
}

int launch_residual(hyb_ctx *ctx, hyb_residual *out) {
    constexpr int VS = 8;
    dim3 blk(32, VS), grd((ctx->Na + 31) / 32, ctx->Nb);
    int nblk = grd.x * grd.y;
    double *part = ctx->d_resid + 16;
    if (ctx->precision == HYB_PREC_FP64)
        k_residual<double, VS><<<grd, blk, 0, ctx->stream>>>((const double *)ctx->d_rhs, ctx->d_vx, ctx->d_vy,
                                                              ctx->d_w, ctx->nvi, ctx->nv, ctx->Na, ctx->Nb, ctx->PA,
                                                              part);
    else
        k_residual<float, VS><<<grd, blk, 0, ctx->stream>>>((const float *)ctx->d_rhs, ctx->d_vx, ctx->d_vy,
                                                             ctx->d_w, ctx->nvi, ctx->nv, ctx->Na, ctx->Nb, ctx->PA,
                                                             part);
    ctx->launches++;
    int rc = check_err(ctx, "k_residual");
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

}  // namespace hyb
