// hyb_sweep_nnd.cuh -- the fused kinetic step (GKUA_Residual.f90:4-469) for
// its most common form: FP32 distributions, a uniform Cartesian mesh, the
// NND scheme and 4 scan cells per thread, in the reference order or the
// upwind order (HYB_SWEEP_UPWIND; the mirrored frames of sweep_body).  The work
// decomposition, the affine scan and the backward step are those of
// sweep_body (hyb_sweep.cuh); what differs is how a row is read and how the
// face values are formed, so that a thread spends its instructions on the
// arithmetic of its cells rather than on addressing and operand selection:
//
// * Staged rows carry 16 bytes of pad on each side.  On a periodic scan axis
//   the producer copies the two wrapped halo cells of each end into the pads
//   (cp.async.bulk of the 16-byte blocks at the other end), so a thread reads
//   its window f(a0-2 .. a0+CPT+1) at fixed offsets from its own chunk: one
//   16-byte and two 8-byte shared loads per component at 4 cells.
// * The Shakhov parameters of the thread's cells are read at fixed offsets
//   from one pointer into the blocked layout (hyb_eqp_at; a warp's 128 cells
//   are one block, each parameter a contiguous 512-byte span), which moves
//   one row per step; the 8 chunks of each 32-cell group prefetch one
//   parameter's 128-byte line each of the next row into L1 (without it the
//   sweep is a fifth slower).
// * March faces: the three rows of the upwind stencil are chosen per row by
//   pointer (rows b-1, b, b+1 for a positive face speed, b+2, b+1, b for a
//   negative one), so one limiter formula serves both directions with no
//   per-value selects.  The value is the one RHSFDVsub forms
//   (GKUA_Residual.f90:155-185) with the same operations in the same order.
// * Scan faces: NND's left state of face q is f(q-1) + 0.5 mm(D(q-1), D(q-2))
//   and its right state f(q) - 0.5 mm(D(q-1), D(q)) with D(k) = f(k+1) - f(k)
//   (GKUA_Residual.f90:160-175).  Both use the limited slope of one cell,
//   sigma(k) = mm(D(k), D(k-1)), so the thread forms sigma once per window
//   cell and the upwind face value f(k) + h sigma(k), h = +-0.5 by the sign of
//   the face speed; the face takes the value of its upwind cell.  FMINMD is
//   symmetric, so these are the reference's values (the sign of a zero slope
//   aside, which cannot change a sum).  FMINMD itself is the median of its
//   arguments and 0 (four min/max operations).
// * Arithmetic on neighbouring cells runs as packed FP32 pairs.
// * Periodicity of each axis, the axis roles and the order are template
//   parameters.  In the upwind order a velocity whose scan (march) face speed
//   is negative works in the frame mirrored along that axis: logical cell k
//   of a thread's chunk is physical cell pp0 + CPT-1-k, logical row b is
//   physical row Nb+1-b, and the wall slots of the two ends swap.  Loads and
//   stores reverse the chunk; the row pointers step backwards.
#pragma once
#include "hyb_sweep.cuh"

namespace hyb {

constexpr int NND_PAD = 4;   // floats of pad before and after a staged row

// shared memory of one velocity group: the layout of sweep_body's with
// padded staged rows
__host__ __device__ inline size_t nnd_group_bytes(int PA, int TPV) {
    const size_t nw = (size_t)TPV / 32, rs = (size_t)PA + 2 * NND_PAD;
    size_t b = 128;                                    // RING+2 mbarriers
    b += (size_t)RING * 2 * rs * sizeof(float);        // staged rows
    b += (size_t)2 * 2 * rs * sizeof(float);           // rows Nb+1, Nb+2 (periodic)
    b += (size_t)2 * 2 * TPV * sizeof(float);          // first-cell dF per thread
    b += (size_t)2 * nw * 3 * sizeof(float);           // warp aggregates
    return (b + 127) / 128 * 128;
}

// Packed FP32 pairs (FADD2 / FMUL2 / FFMA2 of sm_100 and later): the same
// IEEE round-to-nearest results as the scalar operations, two lanes per
// instruction.  The sweep pairs neighbouring cells (2p, 2p+1) of a thread.
__device__ __forceinline__ float2 pk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 pk(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 pk(const float *a, int p) { return make_float2(a[2 * p], a[2 * p + 1]); }
__device__ __forceinline__ void upk(float2 x, float *a, int p) { a[2 * p] = x.x; a[2 * p + 1] = x.y; }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b as b * (-1) + a: one rounding, the value of the subtraction
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
// FMINMD (Functions.f90:10-25) as the median of x, y and 0: the
// smaller-magnitude argument when both have the same sign, else 0 -- the
// reference's value, from four FP32 min/max operations
__device__ __forceinline__ float mmed(float x, float y) { return fmaxf(fminf(x, y), fminf(fmaxf(x, y), 0.f)); }
__device__ __forceinline__ float2 mm2(float2 x, float2 y) { return make_float2(mmed(x.x, y.x), mmed(x.y, y.y)); }

template <int CPT, bool PERA, bool PERB, bool SJ, bool UPW>
__device__ __forceinline__ void sweep_nnd(const KinArgs<float> &A, int vblk) {
    static_assert(CPT == 4 || CPT == 8, "4 or 8 cells per thread");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int PA = A.PA, Na = A.Na, Nb = A.Nb;
    const int TPV = PA / CPT;
    const int RS = PA + 2 * NND_PAD;             // floats per staged component row
    const int g = threadIdx.y, t = threadIdx.x;
    const int pa0 = t * CPT;                     // first cell of the thread, 0-based
    const int lane = t & 31, warp = t >> 5, nw = TPV >> 5;
    const int v = vblk * blockDim.y + g;
    const bool vok = v < A.nv;
    const bool act = vok && pa0 < Na;            // chunks are all-in or all-out
    const bool producer = (t == 0) && vok;

    unsigned char *base = smem_raw + (size_t)g * nnd_group_bytes(PA, TPV);
    uint64_t *bars = reinterpret_cast<uint64_t *>(base);
    float *ring = reinterpret_cast<float *>(base + 128);
    float *wrap = ring + (size_t)RING * 2 * RS;
    float *dlf = wrap + (size_t)2 * 2 * RS;      // [2][2][TPV]
    float *agg = dlf + (size_t)2 * 2 * TPV;      // [2][nw][3]

    const size_t rstride = (size_t)Nb * PA;
    const size_t vrow0 = vok ? (size_t)v * 2 * rstride : 0;
    const uint32_t main_bytes = (uint32_t)(Na * sizeof(float));   // Na is a multiple of 4
    const uint32_t tx = 2u * (main_bytes + (PERA ? 32u : 0u));

    // ---- velocity and face speeds (uniform mesh) --------------------------------
    const int iv = vok ? v % A.nvi : 0, jv = vok ? v / A.nvi : 0;
    const float vx = vok ? (float)A.vx[iv] : 0.f, vy = vok ? (float)A.vy[jv] : 0.f;
    float sA = vx * A.gA1[0] + vy * A.gA2[0];
    float sB = vx * A.gB1[0] + vy * A.gB2[0];
    const float vol = A.vol[0];
    const float ivol = 1.f / vol;
    const float abase = vol / A.dt + (posp(sA) - negp(sA) + posp(sB) - negp(sB));
    // mirrored scan / march axis of this velocity (upwind order only)
    const bool ra = UPW && sA < 0.f, rb = UPW && sB < 0.f;
    if (ra) sA = -sA;
    if (rb) sB = -sB;
    // first physical cell of the thread's chunk; physical row of logical row b
    const int pp0 = !act ? 0 : ra ? Na - pa0 - CPT : pa0;
    auto prow = [&](int b) -> int { return rb ? Nb + 1 - b : b; };
    const float *fw_alo = ra ? A.fw_ahi : A.fw_alo, *fw_ahi = ra ? A.fw_alo : A.fw_ahi;
    const float *fw_blo = rb ? A.fw_bhi : A.fw_blo, *fw_bhi = rb ? A.fw_blo : A.fw_bhi;
    const bool upA = sA > 0.f, upB = sB > 0.f;
    const float hA = upA ? 0.5f : -0.5f;
    const float pA = posp(sA), pB = posp(sB);
    const float cA = -negp(sA), cB = -negp(sB);

    // ---- staged rows ---------------------------------------------------------
    auto phys_row = [&](int bp) -> int {
        if (bp >= 1 && bp <= Nb) return prow(bp);
        if (PERB && bp <= 0) return prow(bp + Nb);
        return 0;
    };
    // f row pr (1..Nb) into a staged row whose cell 0 is at dst
    auto copy_row = [&](float *dst, int pr, uint64_t *bar) {
        const float *src = A.f + vrow0 + (size_t)(pr - 1) * PA;
        mbar_arrive_expect_tx(bar, tx);
#pragma unroll
        for (int r = 0; r < 2; r++) {
            float *d = dst + r * RS;
            const float *s = src + r * rstride;
            bulk_g2s(d, s, main_bytes, bar);
            if (PERA) {
                bulk_g2s(d - NND_PAD, s + Na - NND_PAD, 16, bar);   // cells Na-4 .. Na-1 before cell 0
                bulk_g2s(d + Na, s, 16, bar);                       // cells 0 .. 3 after cell Na-1
            }
        }
    };
    auto issue_row = [&](int bp) {
        const int s = (bp + 1) & (RING - 1);
        const int pr = phys_row(bp);
        if (A.stall_row > 0 && bp == A.stall_row) return;   // hyb_test_stall: a wait nothing completes
        if (pr > 0 && bp <= Nb) copy_row(ring + (size_t)s * 2 * RS + NND_PAD, pr, &bars[s]);
        else mbar_arrive(&bars[s]);                          // keeps the slot's phase count
    };
    if (producer) {
        for (int s = 0; s < RING + 2; s++) mbar_init(&bars[s], 1);
        fence_async_shared();
    }
    __syncthreads();
    if (producer) {
        for (int bp = -1; bp <= RING - 3; bp++) issue_row(bp);
        if (PERB)
            for (int w = 0; w < 2; w++) copy_row(wrap + (size_t)w * 2 * RS + NND_PAD, prow(w + 1), &bars[RING + w]);
    }
    // cell 0 of the G row of logical row bp (H is RS further)
    auto rowp = [&](int bp) -> const float * {
        if (PERB && bp > Nb) return wrap + (size_t)(bp - Nb - 1) * 2 * RS + NND_PAD;
        return ring + (size_t)((bp + 1) & (RING - 1)) * 2 * RS + NND_PAD;
    };
    bool timeout = false;
    auto wait_row = [&](int bp) {
        if (!vok) return;
        if (bp > Nb) {
            if (PERB && !mbar_wait_bounded(&bars[RING + (bp - Nb - 1)], 0, A.spin)) timeout = true;
            return;
        }
        if (phys_row(bp) == 0) return;
        const unsigned k = (unsigned)(bp + 1);
        if (!mbar_wait_bounded(&bars[k & (RING - 1)], (k / RING) & 1u, A.spin)) timeout = true;
    };
    auto ld4 = [](const float *p, float *o) {
        const float4 x = *reinterpret_cast<const float4 *>(p);
        o[0] = x.x; o[1] = x.y; o[2] = x.z; o[3] = x.w;
    };
    auto st4 = [](float *p, const float *o) { *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]); };
    // the CPT consecutive values at p (16-byte aligned)
    auto ldc = [&](const float *p, float *o) {
#pragma unroll
        for (int h = 0; h < CPT / 4; h++) ld4(p + 4 * h, o + 4 * h);
    };
    // the thread's chunk starting at p (its first physical cell) in logical
    // order, and back
    auto ldl = [&](const float *p, float *o) {
        if (!ra) {
            ldc(p, o);
        } else {
            float q[CPT];
            ldc(p, q);
#pragma unroll
            for (int k = 0; k < CPT; k++) o[k] = q[CPT - 1 - k];
        }
    };
    auto stl = [&](float *p, const float *o) {
        if (!ra) {
#pragma unroll
            for (int h = 0; h < CPT / 4; h++) st4(p + 4 * h, o + 4 * h);
        } else {
            float q[CPT];
#pragma unroll
            for (int k = 0; k < CPT; k++) q[k] = o[CPT - 1 - k];
#pragma unroll
            for (int h = 0; h < CPT / 4; h++) st4(p + 4 * h, q + 4 * h);
        }
    };
    // march-face flux at the thread's cells from the upwind stencil rows
    // x1, x2, x3 (GKUA_Residual.f90:155-185 with the mirrored inputs of a
    // negative speed)
    auto march_flux = [&](const float *x1, const float *x2, const float *x3, float *FG, float *FH) {
#pragma unroll
        for (int r = 0; r < 2; r++) {
            float a[CPT], m[CPT], c[CPT];
            ldl(x1 + r * RS + pp0, a);
            ldl(x2 + r * RS + pp0, m);
            ldl(x3 + r * RS + pp0, c);
            float *F = r ? FH : FG;
#pragma unroll
            for (int p = 0; p < CPT / 2; p++) {
                const float2 mp = pk(m, p);
                upk(mul2(pk(sB), fma2(pk(0.5f), mm2(sub2(pk(c, p), mp), sub2(mp, pk(a, p))), mp)), F, p);
            }
        }
    };
    // march-face flux through face q next to a wall of the march axis
    // (faces 1, 2, Nb, Nb+1; GKUA_Residual.f90:196-257)
    auto march_wall = [&](int q, float *FG, float *FH) {
#pragma unroll
        for (int r = 0; r < 2; r++) {
            float *F = r ? FH : FG;
#pragma unroll
            for (int k = 0; k < CPT; k++) {
                const int pc = pp0 + (ra ? CPT - 1 - k : k);      // physical cell of logical cell k
                const int o = r * RS + pc;
                if (q == 1) F[k] = sB * fw_blo[((size_t)v * 2 + r) * PA + pc];
                else if (q == Nb + 1) F[k] = sB * fw_bhi[((size_t)v * 2 + r) * PA + pc];
                else if (q == 2) F[k] = flux_wlo<HYB_SCHEME_NND>(sB, rowp(1)[o], rowp(2)[o], rowp(3)[o]);
                else if (q == Nb) F[k] = flux_whi<HYB_SCHEME_NND>(sB, rowp(Nb)[o], rowp(Nb - 1)[o], rowp(Nb - 2)[o]);
                else F[k] = flux_std<HYB_SCHEME_NND>(sB, rowp(q - 2)[o], rowp(q - 1)[o], rowp(q)[o], rowp(q + 1)[o]);
            }
        }
    };

    // ---- carried state per cell --------------------------------------------------
    float dG[CPT], dH[CPT];            // forward values of the previous row
    float iap[CPT];                    // 1/alpha of the previous row
    float FBl_G[CPT], FBl_H[CPT];      // march flux through face b
#pragma unroll
    for (int k = 0; k < CPT; k++) {
        dG[k] = dH[k] = 0.f;
        iap[k] = 1.f;
        FBl_G[k] = FBl_H[k] = 0.f;
    }
    const float fl = Consts<float>::floor_();
    const float msc = A.mscale ? (float)*A.mscale : 1.f;
    // this thread's parameters in logical row 1: PA is a multiple of the
    // 128-cell block, so a row is PA / 128 whole blocks (8 * PA values)
    const float *epr = A.eqp + hyb_eqp_at((size_t)(prow(1) - 1) * PA + pp0, 0);
    const ptrdiff_t ep_row = rb ? -(ptrdiff_t)8 * PA : (ptrdiff_t)8 * PA;
    // the next row's parameter lines: the 8 chunks of a 32-cell group take
    // one parameter's 128-byte line each
    const ptrdiff_t ep_pf = ep_row + (ptrdiff_t)((pp0 >> 2) & 7) * HYB_EQP_BLK;
    const ptrdiff_t row_step = rb ? -(ptrdiff_t)PA : (ptrdiff_t)PA;
    float *fst = A.f + vrow0 + (size_t)(prow(1) - 1) * PA + pp0;                      // logical row 1
    float *rst = A.rhs ? A.rhs + vrow0 + (size_t)(prow(1) - 1) * PA + pp0 : nullptr;

    for (int bp = -1; bp <= 2; bp++) wait_row(bp);
    // the copies of rows 1, 2 for rows Nb+1, Nb+2 read f rows that the
    // backward step overwrites from step 2 on: they complete before any write
    if (PERB) {
        wait_row(Nb + 1);
        wait_row(Nb + 2);
    }
    if (act) {
        if (PERB) march_flux(upB ? rowp(-1) : rowp(2), upB ? rowp(0) : rowp(1), upB ? rowp(1) : rowp(0), FBl_G, FBl_H);
        else march_wall(1, FBl_G, FBl_H);
    }
    const bool need_scan = __syncthreads_or(vok && upA) != 0;

    // two rows per trip: the row parity of the double buffers is then fixed
    // in each copy of the body, and the carried state changes registers
    // without moves in between
#pragma unroll 2
    for (int b = 1; b <= Nb; b++) {
        // each thread waits on the row's mbarrier itself (that wait makes the
        // bulk copy visible); a timed-out wait is acted on at the row's one
        // block barrier below, before anything is written to f
        if (b + 2 <= Nb) wait_row(b + 2);
        float pc[CPT], cG[CPT], cH[CPT], ia[CPT], FBh_G[CPT], FBh_H[CPT];
        float fo0[CPT], fo1[CPT];          // f of row b-1 (for the backward update)
        float P = 1.f, CGt = 0.f, CHt = 0.f;
        if (act) {
            const float *rm = rowp(b - 1), *r0 = rowp(b), *rp = rowp(b + 1), *rq = rowp(b + 2);
            // window f(a0-2 .. a0+CPT+1) of both components
            float wG[CPT + 4], wH[CPT + 4];
            {
                // physical window pp0-2 .. pp0+CPT+1, reversed in a mirrored frame
                const float2 lg = *reinterpret_cast<const float2 *>(r0 + pp0 - 2);
                const float2 hg = *reinterpret_cast<const float2 *>(r0 + pp0 + CPT);
                const float2 lh = *reinterpret_cast<const float2 *>(r0 + RS + pp0 - 2);
                const float2 hh = *reinterpret_cast<const float2 *>(r0 + RS + pp0 + CPT);
                float pG[CPT + 4], pH[CPT + 4];
                pG[0] = lg.x; pG[1] = lg.y; pG[CPT + 2] = hg.x; pG[CPT + 3] = hg.y;
                pH[0] = lh.x; pH[1] = lh.y; pH[CPT + 2] = hh.x; pH[CPT + 3] = hh.y;
                ldc(r0 + pp0, pG + 2);
                ldc(r0 + RS + pp0, pH + 2);
#pragma unroll
                for (int i = 0; i < CPT + 4; i++) {
                    wG[i] = ra ? pG[CPT + 3 - i] : pG[i];
                    wH[i] = ra ? pH[CPT + 3 - i] : pH[i];
                }
            }
            // scan-face fluxes through faces a0 .. a0+CPT (window cells m+1 | m+2)
            float FA_G[CPT + 1], FA_H[CPT + 1];
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const float *w = r ? wH : wG;
                float *F = r ? FA_H : FA_G;
                float D[CPT + 3], val[CPT + 3];
#pragma unroll
                for (int k = 0; k < CPT + 3; k++) D[k] = w[k + 1] - w[k];
#pragma unroll
                for (int k = 1; k < CPT + 3; k++) val[k] = w[k] + hA * mmed(D[k], D[k - 1]);
#pragma unroll
                for (int m = 0; m <= CPT; m++) F[m] = sA * (upA ? val[m + 1] : val[m + 2]);
            }
            if (!PERA) {
                // faces 1, 2 and Na, Na+1 next to the walls of the scan axis
                // (GKUA_Residual.f90:196-257)
                if (pa0 == 0) {
                    FA_G[0] = sA * fw_alo[((size_t)v * 2 + 0) * Nb + (prow(b) - 1)];
                    FA_H[0] = sA * fw_alo[((size_t)v * 2 + 1) * Nb + (prow(b) - 1)];
                    FA_G[1] = flux_wlo<HYB_SCHEME_NND>(sA, wG[2], wG[3], wG[4]);
                    FA_H[1] = flux_wlo<HYB_SCHEME_NND>(sA, wH[2], wH[3], wH[4]);
                }
                if (pa0 + CPT == Na) {
                    FA_G[CPT - 1] = flux_whi<HYB_SCHEME_NND>(sA, wG[CPT + 1], wG[CPT], wG[CPT - 1]);
                    FA_H[CPT - 1] = flux_whi<HYB_SCHEME_NND>(sA, wH[CPT + 1], wH[CPT], wH[CPT - 1]);
                    FA_G[CPT] = sA * fw_ahi[((size_t)v * 2 + 0) * Nb + (prow(b) - 1)];
                    FA_H[CPT] = sA * fw_ahi[((size_t)v * 2 + 1) * Nb + (prow(b) - 1)];
                }
            }
            float m0[CPT], m1[CPT];
            ldl(rm + pp0, m0);
            ldl(rm + RS + pp0, m1);
            // Shakhov parameters of the thread's cells
            float e_crt[CPT], e_u[CPT], e_v[CPT], e_it[CPT], e_ht[CPT], e_qx[CPT], e_qy[CPT], e_cf[CPT];
            ldl(epr + 0 * HYB_EQP_BLK, e_crt);
            ldl(epr + 1 * HYB_EQP_BLK, e_u);
            ldl(epr + 2 * HYB_EQP_BLK, e_v);
            ldl(epr + 3 * HYB_EQP_BLK, e_it);
            ldl(epr + 4 * HYB_EQP_BLK, e_ht);
            ldl(epr + 5 * HYB_EQP_BLK, e_qx);
            ldl(epr + 6 * HYB_EQP_BLK, e_qy);
            ldl(epr + 7 * HYB_EQP_BLK, e_cf);
            if (b < Nb) asm volatile("prefetch.global.L1 [%0];" ::"l"(epr + ep_pf));
            // march faces b+1
            if (PERB || (b >= 2 && b <= Nb - 2)) march_flux(upB ? rm : rq, upB ? r0 : rp, upB ? rp : r0, FBh_G, FBh_H);
            else march_wall(b + 1, FBh_G, FBh_H);
            float rG[CPT], rH[CPT];
#pragma unroll
            for (int k = 0; k < CPT; k++) {
                fo0[k] = m0[k];
                fo1[k] = m1[k];
            }
            // cells in pairs (2p, 2p+1)
#pragma unroll
            for (int p = 0; p < CPT / 2; p++) {
                const float2 fa0G = pk(FA_G[2 * p], FA_G[2 * p + 1]), fa1G = pk(FA_G[2 * p + 1], FA_G[2 * p + 2]);
                const float2 fa0H = pk(FA_H[2 * p], FA_H[2 * p + 1]), fa1H = pk(FA_H[2 * p + 1], FA_H[2 * p + 2]);
                float2 divG, divH;
                if (SJ) {
                    divG = sub2(add2(sub2(pk(FBh_G, p), pk(FBl_G, p)), fa1G), fa0G);
                    divH = sub2(add2(sub2(pk(FBh_H, p), pk(FBl_H, p)), fa1H), fa0H);
                } else {
                    divG = sub2(add2(sub2(fa1G, fa0G), pk(FBh_G, p)), pk(FBl_G, p));
                    divH = sub2(add2(sub2(fa1H, fa0H), pk(FBh_H, p)), pk(FBl_H, p));
                }
                // Shakhov equilibrium (GKUA_Residual.f90:441-458)
                const float2 viu = sub2(pk(vx), pk(e_u, p)), vjv = sub2(pk(vy), pk(e_v, p));
                const float2 vij2 = mul2(fma2(viu, viu, mul2(vjv, vjv)), pk(e_it, p));
                const float2 fvx = fma2(pk(e_qx, p), viu, mul2(pk(e_qy, p), vjv));
                const float2 gdv = mul2(pk(e_crt, p), pk(sweep_exp<float>(-vij2.x), sweep_exp<float>(-vij2.y)));
                const float2 geq = mul2(gdv, fma2(fvx, fma2(pk(2.f), vij2, pk(-4.f)), pk(1.f)));
                const float2 heq = mul2(mul2(pk(e_ht, p), gdv), fma2(fvx, fma2(pk(2.f), vij2, pk(-2.f)), pk(1.f)));
                const float2 ecf = pk(e_cf, p);
                const float2 r2G = fma2(divG, pk(-ivol), mul2(ecf, sub2(geq, pk(wG + 2, p))));
                const float2 r2H = fma2(divH, pk(-ivol), mul2(ecf, sub2(heq, pk(wH + 2, p))));
                upk(r2G, rG, p);
                upk(r2H, rH, p);
                // LU-SGS forward element (GKUA_Residual.f90:39-57)
                const float2 alfa = fma2(pk(vol), ecf, pk(abase));
                const float2 ia2 = pk(sweep_rcp<float>(alfa.x), sweep_rcp<float>(alfa.y));
                upk(ia2, ia, p);
                upk(mul2(pk(pA), ia2), pc, p);
                upk(mul2(fma2(pk(vol), r2G, mul2(pk(pB), pk(dG, p))), ia2), cG, p);
                upk(mul2(fma2(pk(vol), r2H, mul2(pk(pB), pk(dH, p))), ia2), cH, p);
            }
            // thread-local composition of the affine maps
#pragma unroll
            for (int k = 0; k < CPT; k++) {
                CGt = cG[k] + pc[k] * CGt;
                CHt = cH[k] + pc[k] * CHt;
                P = pc[k] * P;
            }
            if (rst) {
                stl(rst, rG);
                stl(rst + rstride, rH);
            }
        } else {
#pragma unroll
            for (int k = 0; k < CPT; k++) pc[k] = cG[k] = cH[k] = ia[k] = FBh_G[k] = FBh_H[k] = fo0[k] = fo1[k] = 0.f;
            P = 0.f;
        }
        epr += ep_row;
        if (rst) rst += row_step;
        float Pe = 1.f, Ge = 0.f, He = 0.f;
        float *aggb = agg + (size_t)(b & 1) * nw * 3;
        if (need_scan) {
            // inclusive warp scan of the composed maps (earlier lanes first)
            float Pi = P, Gi = CGt, Hi = CHt;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const float pu = __shfl_up_sync(0xffffffffu, Pi, off);
                const float gu = __shfl_up_sync(0xffffffffu, Gi, off);
                const float hu = __shfl_up_sync(0xffffffffu, Hi, off);
                if (lane >= off) {
                    Gi = Gi + Pi * gu;
                    Hi = Hi + Pi * hu;
                    Pi = Pi * pu;
                }
            }
            Pe = __shfl_up_sync(0xffffffffu, Pi, 1);
            Ge = __shfl_up_sync(0xffffffffu, Gi, 1);
            He = __shfl_up_sync(0xffffffffu, Hi, 1);
            if (lane == 0) { Pe = 1.f; Ge = 0.f; He = 0.f; }
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
        float xG = Ge, xH = He;                              // dF just before cell a0
        if (need_scan && warp > 0) {
            float carG = 0.f, carH = 0.f;
            for (int w = 0; w < warp; w++) {
                const float pw = aggb[w * 3 + 0];
                carG = aggb[w * 3 + 1] + pw * carG;
                carH = aggb[w * 3 + 2] + pw * carH;
            }
            xG = Ge + Pe * carG;
            xH = He + Pe * carH;
        }
        float nG[CPT], nH[CPT];
#pragma unroll
        for (int k = 0; k < CPT; k++) {
            xG = cG[k] + pc[k] * xG;
            xH = cH[k] + pc[k] * xH;
            nG[k] = xG;
            nH[k] = xH;
        }
        float *dlb = dlf + (size_t)(b & 1) * 2 * TPV;
        dlb[t] = act ? nG[0] : 0.f;
        dlb[TPV + t] = act ? nH[0] : 0.f;
        // backward + update of row b-1 (GKUA_Residual.f90:64-109)
        if (b > 1) {
            if (act && !A.no_update) {
                const float *dlp = dlf + (size_t)((b - 1) & 1) * 2 * TPV;
                const bool has_next = (pa0 + CPT < Na);
                const float lastG = has_next ? dlp[t + 1] : 0.f, lastH = has_next ? dlp[TPV + t + 1] : 0.f;
                float uG[CPT], uH[CPT], nxG[CPT], nxH[CPT];
#pragma unroll
                for (int k = 0; k < CPT; k++) {
                    nxG[k] = k + 1 < CPT ? dG[k + 1] : lastG;
                    nxH[k] = k + 1 < CPT ? dH[k + 1] : lastH;
                }
#pragma unroll
                for (int p = 0; p < CPT / 2; p++) {
                    const float2 ip = pk(iap, p);
                    const float2 g2 = mul2(pk(msc), add2(pk(fo0, p), fma2(fma2(pk(cA), pk(nxG, p), mul2(pk(cB), pk(nG, p))),
                                                                          ip, pk(dG, p))));
                    const float2 h2 = mul2(pk(msc), add2(pk(fo1, p), fma2(fma2(pk(cA), pk(nxH, p), mul2(pk(cB), pk(nH, p))),
                                                                          ip, pk(dH, p))));
                    uG[2 * p] = g2.x < fl ? fl : g2.x;
                    uG[2 * p + 1] = g2.y < fl ? fl : g2.y;
                    uH[2 * p] = h2.x < fl ? fl : h2.x;
                    uH[2 * p + 1] = h2.y < fl ? fl : h2.y;
                }
                stl(fst, uG);
                stl(fst + rstride, uH);
            }
            fst += row_step;
        }
#pragma unroll
        for (int k = 0; k < CPT; k++) {
            dG[k] = nG[k];
            dH[k] = nH[k];
            iap[k] = ia[k];
            FBl_G[k] = FBh_G[k];
            FBl_H[k] = FBh_H[k];
        }
    }
    __syncthreads();
    if (act && !A.no_update) {   // backward + update of the last row (downstream values are 0)
        const float *dlp = dlf + (size_t)(Nb & 1) * 2 * TPV;
        const bool has_next = (pa0 + CPT < Na);
        const float *o0 = rowp(Nb);
        float f0[CPT], f1[CPT], uG[CPT], uH[CPT];
        ldl(o0 + pp0, f0);
        ldl(o0 + RS + pp0, f1);
#pragma unroll
        for (int k = 0; k < CPT; k++) {
            const float nxG = (k + 1 < CPT) ? dG[k + 1] : (has_next ? dlp[t + 1] : 0.f);
            const float nxH = (k + 1 < CPT) ? dH[k + 1] : (has_next ? dlp[TPV + t + 1] : 0.f);
            const float fg = msc * (f0[k] + (dG[k] + (cA * nxG) * iap[k]));
            const float fh = msc * (f1[k] + (dH[k] + (cA * nxH) * iap[k]));
            uG[k] = fg < fl ? fl : fg;
            uH[k] = fh < fl ? fl : fh;
        }
        stl(fst, uG);
        stl(fst + rstride, uH);
    }
    // every bulk copy issued (rows 1..Nb and the wrap rows) has been waited
    // for above, so no copy is in flight when the CTA exits
}

// 4 cells per thread, CTAs of up to 256 threads, 128 registers.  8 cells
// per thread compiles (the body is written for either) but measured slower
// on the 128x512 x 64^2 Couette case, 1.86 against 1.60 ms: twice the
// per-cell state leaves 10 warps per SM.  Only 4 is instantiated.
template <int CPT, bool PERA, bool PERB, bool SJ, bool UPW>
__global__ void __launch_bounds__(256, 2) k_sweep_nnd(KinArgs<float> A) {
    sweep_nnd<CPT, PERA, PERB, SJ, UPW>(A, blockIdx.x);
}

template <int CPT, bool PERA, bool PERB, bool SJ, bool UPW>
int sweep_nnd_launch(hyb_ctx *ctx, const KinArgs<float> &A, int vpb, bool launch) {
    const int tpv = ctx->PA / CPT;
    const size_t smem = nnd_group_bytes(ctx->PA, tpv) * vpb;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_sweep_nnd<CPT, PERA, PERB, SJ, UPW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             227 * 1024);
        attr = true;
    }
    if (!launch) return HYB_OK;
    dim3 blk(tpv, vpb), grd((ctx->nv + vpb - 1) / vpb);
    k_sweep_nnd<CPT, PERA, PERB, SJ, UPW><<<grd, blk, smem, ctx->stream>>>(A);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ctx->last_error = std::string("k_sweep_nnd: ") + cudaGetErrorString(e);
        return HYB_ERR_CUDA;
    }
    return HYB_OK;
}

template <int CPT, bool UPW>
inline int sweep_nnd_dispatch_cpt(hyb_ctx *ctx, const KinArgs<float> &A, int vpb, bool launch) {
    const bool pa = A.bca_lo == AX_PERIODIC, pb = A.bcb_lo == AX_PERIODIC, sj = A.scan_is_j != 0;
    if (pa) {
        if (pb) return sj ? sweep_nnd_launch<CPT, true, true, true, UPW>(ctx, A, vpb, launch)
                          : sweep_nnd_launch<CPT, true, true, false, UPW>(ctx, A, vpb, launch);
        return sj ? sweep_nnd_launch<CPT, true, false, true, UPW>(ctx, A, vpb, launch)
                  : sweep_nnd_launch<CPT, true, false, false, UPW>(ctx, A, vpb, launch);
    }
    if (pb) return sj ? sweep_nnd_launch<CPT, false, true, true, UPW>(ctx, A, vpb, launch)
                      : sweep_nnd_launch<CPT, false, true, false, UPW>(ctx, A, vpb, launch);
    return sj ? sweep_nnd_launch<CPT, false, false, true, UPW>(ctx, A, vpb, launch)
              : sweep_nnd_launch<CPT, false, false, false, UPW>(ctx, A, vpb, launch);
}

// many contexts of one launch shape and one kernel signature in one launch:
// CTA i sweeps velocity block work[i].y of context work[i].x (reference order;
// batches do not take the upwind order)
template <bool PERA, bool PERB, bool SJ>
__global__ void __launch_bounds__(256, 2) k_sweep_nnd_batch(const KinArgs<float> *__restrict__ args,
                                                            const int2 *__restrict__ work) {
    __shared__ KinArgs<float> As;
    const int2 w = work[blockIdx.x];
    if (threadIdx.x == 0 && threadIdx.y == 0) As = args[w.x];
    __syncthreads();
    sweep_nnd<4, PERA, PERB, SJ, false>(As, w.y);
}

template <bool PERA, bool PERB, bool SJ>
int sweep_nnd_batch_one(const KinArgs<float> *args, const int2 *work, int nwork, int PA, int vpb, cudaStream_t s) {
    const int tpv = PA / 4;
    const size_t smem = nnd_group_bytes(PA, tpv) * vpb;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_sweep_nnd_batch<PERA, PERB, SJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             227 * 1024 - 1024);
        attr = true;
    }
    if (nwork <= 0) return HYB_OK;   // attributes only (before a capture)
    k_sweep_nnd_batch<PERA, PERB, SJ><<<nwork, dim3(tpv, vpb), smem, s>>>(args, work);
    return cudaGetLastError() == cudaSuccess ? HYB_OK : HYB_ERR_CUDA;
}

// sig: sweep_nnd_signature (bit 0 periodic scan axis, bit 1 periodic march
// axis, bit 2 scan axis = j)
inline int sweep_nnd_batch(const KinArgs<float> *args, const int2 *work, int nwork, int PA, int vpb, int sig,
                           cudaStream_t s) {
    switch (sig & 7) {
        case 0: return sweep_nnd_batch_one<false, false, false>(args, work, nwork, PA, vpb, s);
        case 1: return sweep_nnd_batch_one<true, false, false>(args, work, nwork, PA, vpb, s);
        case 2: return sweep_nnd_batch_one<false, true, false>(args, work, nwork, PA, vpb, s);
        case 3: return sweep_nnd_batch_one<true, true, false>(args, work, nwork, PA, vpb, s);
        case 4: return sweep_nnd_batch_one<false, false, true>(args, work, nwork, PA, vpb, s);
        case 5: return sweep_nnd_batch_one<true, false, true>(args, work, nwork, PA, vpb, s);
        case 6: return sweep_nnd_batch_one<false, true, true>(args, work, nwork, PA, vpb, s);
        default: return sweep_nnd_batch_one<true, true, true>(args, work, nwork, PA, vpb, s);
    }
}

// the specialised sweep (sweep_nnd_ok(ctx, 4) holds), in the context's order
inline int sweep_nnd_dispatch(hyb_ctx *ctx, const KinArgs<float> &A, int vpb, bool launch) {
    return ctx->prm.sweep_order == HYB_SWEEP_UPWIND ? sweep_nnd_dispatch_cpt<4, true>(ctx, A, vpb, launch)
                                                    : sweep_nnd_dispatch_cpt<4, false>(ctx, A, vpb, launch);
}

}  // namespace hyb
