// hyb_device.cuh -- device helpers shared by the kinetic kernels: mbarrier /
// bulk-copy wrappers (inline PTX), bounded waits, and the face
// reconstructions of RHSFDVsub (GKUA_Residual.f90:145-396).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

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

// bounded wait: returns false when `limit` SM clocks ran out (the default,
// HYB_SPIN_CYCLES, is about two seconds; the normal wait is well under a
// microsecond; hyb_test_stall shortens it for one step)
#define HYB_SPIN_CYCLES 4000000000LL
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, long long limit) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (clock64() - t0 < limit)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

template <typename real> __device__ __forceinline__ real posp(real a) { return (a + fabs(a)) * real(0.5); }
template <typename real> __device__ __forceinline__ real negp(real a) { return (a - fabs(a)) * real(0.5); }

// FMINMD, Functions.f90:10-25: the smaller-magnitude argument when both have
// the same strict sign, else 0.  Branch-free form: t = sign(x) y is > 0
// exactly when y has x's sign, and min(|x|, t) is then |x| or |y|; the
// result can differ from the reference only in the sign of a zero
template <typename real> __device__ __forceinline__ real fminmd(real x, real y) {
    const real t = copysign(real(1), x) * y;
    return copysign(fmax(real(0), fmin(fabs(x), t)), x);
}
// FP64: the same value from integer operations on the IEEE bit patterns,
// which keeps the limiter off the FP64 pipe (2 lanes per clock per SM on
// GB300).  Equal sign bits and a smaller magnitude field select x, else y;
// different sign bits give 0.  A zero argument gives a zero either way.
template <> __device__ __forceinline__ double fminmd<double>(double x, double y) {
    const long long ix = __double_as_longlong(x), iy = __double_as_longlong(y);
    const long long mask = 0x7fffffffffffffffLL;
    const double m = (ix & mask) < (iy & mask) ? x : y;
    return (ix ^ iy) >= 0 ? m : 0.0;
}

// max(v, fl) for the floor of the update, fl > 0 (GKUA_Residual.f90:104-109:
// values below fl become fl).  FP64 compares the bit patterns as signed
// 64-bit integers, which order every double below a positive fl (negative
// values and -0 included) below it, off the FP64 pipe.
template <typename real> __device__ __forceinline__ real floor_at(real v, real fl) { return v < fl ? fl : v; }
template <> __device__ __forceinline__ double floor_at<double>(double v, double fl) {
    return __double_as_longlong(v) < __double_as_longlong(fl) ? fl : v;
}

template <typename real> __device__ __forceinline__ real dexp(real x);
template <> __device__ __forceinline__ float dexp<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double dexp<double>(double x) { return exp(x); }

// the sweep's FP32 path uses the hardware approximations of exp and 1/x
// (a few ulp); the FP64 path keeps the correctly rounded forms
template <typename real> __device__ __forceinline__ real sweep_exp(real x);
template <> __device__ __forceinline__ float sweep_exp<float>(float x) { return __expf(x); }
template <> __device__ __forceinline__ double sweep_exp<double>(double x) { return exp(x); }
template <typename real> __device__ __forceinline__ real sweep_rcp(real x);
template <> __device__ __forceinline__ float sweep_rcp<float>(float x) { return __fdividef(1.0f, x); }
template <> __device__ __forceinline__ double sweep_rcp<double>(double x) { return 1.0 / x; }

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


// Flux through a face with speed s from f(q-2), f(q-1), f(q), f(q+1): only
// the upwind reconstruction is formed (asp*UL + asn*UR with asn = 0 when
// s > 0 and asp = 0 otherwise gives the same number).
template <typename real>
__device__ __forceinline__ real face_flux_s(int scheme, real s, real u1, real u2, real u3, real u4) {
    if (scheme == HYB_SCHEME_WENO3) return face_flux(scheme, posp(s), negp(s), u1, u2, u3, u4);
    if (s > real(0)) {
        if (scheme == HYB_SCHEME_UP1) return s * u2;
        return s * (u2 + real(0.5) * fminmd(u3 - u2, u2 - u1));
    }
    if (scheme == HYB_SCHEME_UP1) return s * u3;
    return s * (u3 - real(0.5) * fminmd(u3 - u2, u4 - u3));
}
template <typename real>
__device__ __forceinline__ real face_flux_wall_lo_s(int scheme, real s, real f1, real f2, real f3) {
    if (scheme == HYB_SCHEME_WENO3) return face_flux_wall_lo(scheme, posp(s), negp(s), f1, f2, f3);
    if (s > real(0)) return s * (scheme == HYB_SCHEME_UP1 ? f1 : f1 + real(0.5) * (f2 - f1));
    return s * (scheme == HYB_SCHEME_UP1 ? f2 : f2 - real(0.5) * fminmd(f2 - f1, f3 - f2));
}
template <typename real>
__device__ __forceinline__ real face_flux_wall_hi_s(int scheme, real s, real f1, real f2, real f3) {
    if (scheme == HYB_SCHEME_WENO3) return face_flux_wall_hi(scheme, posp(s), negp(s), f1, f2, f3);
    if (s > real(0)) return s * (scheme == HYB_SCHEME_UP1 ? f2 : f2 + real(0.5) * fminmd(f1 - f2, f2 - f3));
    return s * (scheme == HYB_SCHEME_UP1 ? f1 : f1 - real(0.5) * (f1 - f2));
}

}  // namespace hyb
