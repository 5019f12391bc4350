// hyb_batch.cu -- batched Couette instances and the sweep-shape autotuner.
//
// A batch owns one context per instance (each with its own stream and
// buffers, so instances of different mesh and velocity-grid sizes coexist).
// One outer iteration of every instance -- wall, sweep, moments, S ghosts
// (and Convert_NS on the last iteration of a step) -- is captured once into a
// CUDA graph, so one graph launch advances all instances by one iteration.
// Two graphs are kept: one for plain iterations and one whose sweeps also
// store the RHS (the last iteration of a step).
//
// Both graphs are made of batched launches: the instances are grouped by
// launch shape (scan-axis padding, layout chunk, sweep cells per thread and
// velocity groups per CTA, uniform spacing), and each group issues five
// kernels -- walls, sweeps, moment partials, moment finish, S ghosts; on the
// last iteration also the residual moments of the stored RHS and their
// per-block fold -- whose CTAs each read their instance's argument record
// from a device table and take one (instance, block) pair from a work table.
// The groups are the graph's branches.  After them the last iteration runs
// Convert_NS of every instance (six launches, one per phase) and the final
// residual folds (one warp per instance, which also gathers the residuals
// for the single host copy); a last kernel gathers the error words.  The
// kernels are the per-context kernels' bodies, so every instance computes
// bit for bit what a standalone context computes.  Batches the batched
// kernels do not cover (schemes other than NND, slices beyond the batched
// kernels' shared memory) keep one graph branch per instance.
//
// The autotuner (hyb_autotune) times every admissible sweep launch shape
// (cells per thread dividing the layout chunk, velocity groups per CTA up to
// 256 threads and 227 KB of shared memory) on the context's own data: f is
// saved to the RHS buffer, each candidate runs `reps` sweeps timed with CUDA
// events, f is restored after every candidate, and the fastest shape is kept
// in the context.  No counterpart in the reference.
#include <cuda_runtime.h>
#include <math.h>

#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "hyb_common.cuh"

struct hyb_batch {
    int dev = 0;
    std::vector<hyb_ctx *> inst;
    cudaStream_t main = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, fork = nullptr;
    std::vector<cudaEvent_t> done;
    cudaGraphExec_t g_iter = nullptr, g_last = nullptr;
    long long nodes_iter = 0, nodes_last = 0;   // kernel launches per graph launch
    long long launches = 0;
    double last_ms = 0.0;
    std::string last_error;
    // per-instance results gathered inside the graph: residual (9 doubles)
    // and error word, read back with one copy each per step
    double *d_res = nullptr, *h_res = nullptr;
    int *d_errs = nullptr, *h_errs = nullptr;
    // argument records and work tables of the batched graphs
    void *d_tab_iter = nullptr, *d_tab_last = nullptr;
};

namespace {

int ctx_err_word(hyb_ctx *ctx) {
    int h = 0;
    if (cudaMemcpy(&h, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return HYB_ERR_CUDA;
    if (h != 0) {
        ctx->last_error = "device error word set (bounded wait expired)";
        cudaMemset(ctx->d_err, 0, sizeof(int));
        return h;
    }
    return HYB_OK;
}

// one outer iteration of one instance: the body of hyb_step without GSIS.
// Convert_NS only feeds the synthetic solve and the HoT output, so plain
// iterations skip it and the last iteration of a step (store_rhs) runs it.
int iteration(hyb_ctx *ctx, int store_rhs) {
    int rc = hyb::launch_wall(ctx);
    if (!rc) rc = hyb::launch_sweep(ctx, store_rhs);
    if (!rc) rc = hyb::launch_moments(ctx);
    if (!rc) rc = hyb::launch_sghost(ctx);
    if (!rc && store_rhs) rc = hyb::launch_convert_ns(ctx);
    return rc;
}

void drop_graphs(hyb_batch *b) {
    if (b->g_iter) cudaGraphExecDestroy(b->g_iter);
    if (b->g_last) cudaGraphExecDestroy(b->g_last);
    b->g_iter = b->g_last = nullptr;
    if (b->d_tab_iter) cudaFree(b->d_tab_iter);
    if (b->d_tab_last) cudaFree(b->d_tab_last);
    b->d_tab_iter = b->d_tab_last = nullptr;
}

// ---- batched iterations -----------------------------------------------------
struct Group {
    std::vector<int> members;            // instance indices
    int PA = 0, cpt = 0, vpb = 0, uni = 0, mc = 0, tpv = 0;
    int nsig = 0;                        // sweep_nnd_signature of the members (0: generic sweep)
    size_t wall_smem = 0, mom_smem = 0;
    // offsets into the table (bytes) and launch sizes
    size_t o_wall, o_wwork, o_kin, o_kwork, o_mom, o_mwork, o_fwork, o_sg, o_swork, o_scount;
    size_t o_rmom = 0, o_parts = 0;      // last iteration: residual moments of the stored RHS
    int n_wall = 0, n_kin = 0, n_mom = 0, n_fin = 0, n_sg = 0;
};

// the launches of one captured iteration
struct Plan {
    bool last = false;                   // RHS store, Convert_NS and residual
    std::vector<Group> gs;
    size_t o_err = 0, o_cns = 0, o_rfin = 0;
    size_t o_cwork[6] = {0, 0, 0, 0, 0, 0};
    int n_cwork[6] = {0, 0, 0, 0, 0, 0};
};

// host image of the table: sections appended at 256-byte boundaries
struct Table {
    std::vector<unsigned char> bytes;
    size_t put(const void *src, size_t n) {
        size_t off = (bytes.size() + 255) & ~(size_t)255;
        bytes.resize(off + n);
        if (n) memcpy(bytes.data() + off, src, n);
        return off;
    }
};

// groups of one launch shape; false when an instance is outside what the
// batched kernels cover
bool make_groups(hyb_batch *b, std::vector<Group> &gs) {
    for (size_t k = 0; k < b->inst.size(); k++) {
        hyb_ctx *c = b->inst[k];
        if (c->prm.scheme != HYB_SCHEME_NND) return false;
        if (hyb::sweep_smem_bytes(c) > (size_t)227 * 1024 - 1024) return false;
        int cpt, vpb;
        hyb::sweep_shape(c, &cpt, &vpb);
        const int sig = c->precision == HYB_PREC_FP64 ? 0 : hyb::sweep_nnd_signature(c, cpt);
        Group *g = nullptr;
        for (Group &q : gs)
            if (q.PA == c->PA && q.cpt == cpt && q.vpb == vpb && q.uni == (c->uniform != 0) &&
                b->inst[q.members[0]]->cpt == c->cpt && q.nsig == sig)
                g = &q;
        if (!g) {
            gs.emplace_back();
            g = &gs.back();
            g->PA = c->PA;
            g->cpt = cpt;
            g->vpb = vpb;
            g->uni = c->uniform != 0;
            g->nsig = sig;
        }
        g->members.push_back((int)k);
    }
    return true;
}

// device tables of the plan; HYB_ERR_UNSUPPORTED when the batched kernels do
// not cover the batch
int build_tables(hyb_batch *b, Plan &P, void **d_tab) {
    if (!make_groups(b, P.gs)) return HYB_ERR_UNSUPPORTED;
    const int prec = b->inst[0]->precision;
    const int store_rhs = P.last ? 1 : 0;
    Table T;
    std::vector<unsigned char> rec, rrec;
    for (Group &g : P.gs) {
        const size_t n = g.members.size();
        std::vector<int2> wwork, kwork, swork;
        std::vector<int4> mwork, fwork;
        std::vector<int> scount(n);
        // walls
        rec.assign(hyb::wall_arg_bytes(prec) * n, 0);
        for (size_t li = 0; li < n; li++) {
            size_t sm = 0;
            const int nw = hyb::wall_arg_fill(b->inst[g.members[li]], rec.data() + li * hyb::wall_arg_bytes(prec), &sm);
            g.wall_smem = std::max(g.wall_smem, sm);
            for (int kg = 0; kg < nw; kg++) wwork.push_back(make_int2((int)li, kg));
        }
        g.o_wall = T.put(rec.data(), rec.size());
        g.o_wwork = T.put(wwork.data(), wwork.size() * sizeof(int2));
        g.n_wall = (int)wwork.size();
        // sweeps
        const size_t kb = prec == HYB_PREC_FP64 ? sizeof(hyb::KinArgs<double>) : sizeof(hyb::KinArgs<float>);
        rec.assign(kb * n, 0);
        for (size_t li = 0; li < n; li++) {
            hyb_ctx *c = b->inst[g.members[li]];
            if (prec == HYB_PREC_FP64)
                hyb::sweep_args_f64(c, store_rhs, (hyb::KinArgs<double> *)(rec.data() + li * kb));
            else
                hyb::sweep_args_f32(c, store_rhs, (hyb::KinArgs<float> *)(rec.data() + li * kb));
            const int nvb = (c->nv + g.vpb - 1) / g.vpb;
            for (int vb = 0; vb < nvb; vb++) kwork.push_back(make_int2((int)li, vb));
        }
        g.o_kin = T.put(rec.data(), rec.size());
        g.o_kwork = T.put(kwork.data(), kwork.size() * sizeof(int2));
        g.n_kin = (int)kwork.size();
        // moments (and, on the last iteration, the residual moments of the
        // RHS: the same slicing over the RHS buffer)
        const size_t mb = hyb::mom_arg_bytes();
        rec.assign(mb * n, 0);
        rrec.assign(P.last ? mb * n : 0, 0);
        std::vector<double *> parts(n, nullptr);
        for (size_t li = 0; li < n; li++) {
            hyb_ctx *c = b->inst[g.members[li]];
            int mc, tpv, vs, lpc, nfin;
            size_t sm;
            if (hyb::mom_arg_fill(c, nullptr, rec.data() + li * mb, &mc, &tpv, &sm, &vs, &lpc, &nfin))
                return HYB_ERR_UNSUPPORTED;
            if (P.last) {
                int mc2, tpv2, vs2, lpc2, nfin2;
                size_t sm2;
                if (hyb::mom_arg_fill(c, c->d_rhs, rrec.data() + li * mb, &mc2, &tpv2, &sm2, &vs2, &lpc2, &nfin2))
                    return HYB_ERR_UNSUPPORTED;
                std::vector<unsigned char> fin(hyb::resfinal_arg_bytes());
                hyb::resfinal_arg_fill(c, fin.data(), &parts[li]);   // where the block partials go
            }
            if (li == 0) {
                g.mc = mc;
                g.tpv = tpv;
            } else if (mc != g.mc || tpv != g.tpv) {
                return HYB_ERR_UNSUPPORTED;
            }
            g.mom_smem = std::max(g.mom_smem, sm);
            for (int row = 0; row < c->Nb; row++)
                for (int sl = 0; sl < vs; sl++) mwork.push_back(make_int4((int)li, row, sl, 0));
            for (int blk = 0; blk < nfin; blk++) fwork.push_back(make_int4((int)li, blk, lpc, 0));
        }
        g.o_mom = T.put(rec.data(), rec.size());
        g.o_mwork = T.put(mwork.data(), mwork.size() * sizeof(int4));
        g.o_fwork = T.put(fwork.data(), fwork.size() * sizeof(int4));
        g.n_mom = (int)mwork.size();
        g.n_fin = (int)fwork.size();
        if (P.last) {
            g.o_rmom = T.put(rrec.data(), rrec.size());
            g.o_parts = T.put(parts.data(), parts.size() * sizeof(double *));
        }
        // S ghosts
        const size_t sb = hyb::sghost_arg_bytes();
        rec.assign(sb * n, 0);
        for (size_t li = 0; li < n; li++) {
            scount[li] = hyb::sghost_arg_fill(b->inst[g.members[li]], rec.data() + li * sb);
            for (int o = 0; o < scount[li]; o += 128) swork.push_back(make_int2((int)li, o));
        }
        g.o_sg = T.put(rec.data(), rec.size());
        g.o_swork = T.put(swork.data(), swork.size() * sizeof(int2));
        g.o_scount = T.put(scount.data(), scount.size() * sizeof(int));
        g.n_sg = (int)swork.size();
    }
    const size_t ni = b->inst.size();
    if (P.last) {
        // Convert_NS of every instance: six launches (the face phases share one)
        const size_t cb = hyb::cns_arg_bytes();
        rec.assign(cb * ni, 0);
        std::vector<int4> cw[6];
        for (size_t k = 0; k < ni; k++) {
            int cnt[7];
            hyb::cns_arg_fill(b->inst[k], rec.data() + k * cb, cnt);
            for (int ph = 0; ph < 7; ph++)
                for (int o = 0; o * 128 < cnt[ph]; o++) cw[ph < 6 ? ph : 5].push_back(make_int4((int)k, ph, o, 0));
        }
        P.o_cns = T.put(rec.data(), rec.size());
        for (int L = 0; L < 6; L++) {
            P.o_cwork[L] = T.put(cw[L].data(), cw[L].size() * sizeof(int4));
            P.n_cwork[L] = (int)cw[L].size();
        }
        // final residual folds
        const size_t fb = hyb::resfinal_arg_bytes();
        rec.assign(fb * ni, 0);
        for (size_t k = 0; k < ni; k++) {
            double *unused;
            hyb::resfinal_arg_fill(b->inst[k], rec.data() + k * fb, &unused);
        }
        P.o_rfin = T.put(rec.data(), rec.size());
    }
    std::vector<int *> errp(ni);
    for (size_t k = 0; k < ni; k++) errp[k] = b->inst[k]->d_err;
    P.o_err = T.put(errp.data(), errp.size() * sizeof(int *));
    if (cudaMalloc(d_tab, T.bytes.size()) != cudaSuccess ||
        cudaMemcpy(*d_tab, T.bytes.data(), T.bytes.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        b->last_error = "batch: launch tables could not be allocated";
        return HYB_ERR_CUDA;
    }
    return HYB_OK;
}

// one group's launches on stream s
int group_launches(hyb_batch *b, const Plan &P, const Group &g, unsigned char *t, cudaStream_t s) {
    const int prec = b->inst[0]->precision;
    int rc = hyb::wall_batch_launch(prec, t + g.o_wall, (const int2 *)(t + g.o_wwork), g.n_wall, g.wall_smem, s);
    if (!rc) {
        const int2 *kw = (const int2 *)(t + g.o_kwork);
        rc = prec == HYB_PREC_FP64
                 ? hyb::sweep_batch_f64((const hyb::KinArgs<double> *)(t + g.o_kin), kw, g.n_kin, g.PA, g.cpt, g.vpb,
                                        g.uni, HYB_SCHEME_NND, s)
             : g.nsig ? hyb::sweep_nnd_batch_f32((const hyb::KinArgs<float> *)(t + g.o_kin), kw, g.n_kin, g.PA, g.vpb,
                                                 g.nsig, s)
                      : hyb::sweep_batch_f32((const hyb::KinArgs<float> *)(t + g.o_kin), kw, g.n_kin, g.PA, g.cpt, g.vpb,
                                             g.uni, HYB_SCHEME_NND, s);
    }
    const int4 *mw = (const int4 *)(t + g.o_mwork), *fw = (const int4 *)(t + g.o_fwork);
    if (!rc) rc = hyb::moments_part_batch_launch(prec, g.mc, g.tpv, 10, t + g.o_mom, mw, g.n_mom, g.mom_smem, s);
    if (!rc) rc = hyb::moments_finish_batch_launch(prec, t + g.o_mom, fw, g.n_fin, s);
    if (!rc)
        rc = hyb::sghost_batch_launch(t + g.o_sg, (const int2 *)(t + g.o_swork), (const int *)(t + g.o_scount), g.n_sg,
                                      s);
    if (!rc && P.last) {
        rc = hyb::moments_part_batch_launch(prec, g.mc, g.tpv, 4, t + g.o_rmom, mw, g.n_mom, g.mom_smem, s);
        if (!rc)
            rc = hyb::residual_finish_batch_launch(prec, t + g.o_rmom, fw, (double *const *)(t + g.o_parts), g.n_fin,
                                                   s);
    }
    return rc;
}

// shared-memory attributes of a group's kernels (outside any capture)
int group_prepare(hyb_batch *b, const Group &g) {
    const int prec = b->inst[0]->precision;
    int rc = hyb::wall_batch_launch(prec, nullptr, nullptr, 0, g.wall_smem, b->main);
    if (!rc)
        rc = prec == HYB_PREC_FP64
                 ? hyb::sweep_batch_f64(nullptr, nullptr, 0, g.PA, g.cpt, g.vpb, g.uni, HYB_SCHEME_NND, b->main)
             : g.nsig ? hyb::sweep_nnd_batch_f32(nullptr, nullptr, 0, g.PA, g.vpb, g.nsig, b->main)
                      : hyb::sweep_batch_f32(nullptr, nullptr, 0, g.PA, g.cpt, g.vpb, g.uni, HYB_SCHEME_NND, b->main);
    if (!rc) rc = hyb::moments_part_batch_launch(prec, g.mc, g.tpv, 10, nullptr, nullptr, 0, g.mom_smem, b->main);
    if (!rc) rc = hyb::moments_part_batch_launch(prec, g.mc, g.tpv, 4, nullptr, nullptr, 0, g.mom_smem, b->main);
    return rc;
}

// capture a batched iteration; HYB_ERR_UNSUPPORTED leaves the per-instance
// graph to the caller
int build_graph_batched(hyb_batch *b, bool last, cudaGraphExec_t *exec, long long *nodes, void **d_tab) {
    Plan P;
    P.last = last;
    int rc = build_tables(b, P, d_tab);
    for (size_t q = 0; q < P.gs.size() && !rc; q++) rc = group_prepare(b, P.gs[q]);
    if (rc) return rc;
    unsigned char *t = (unsigned char *)*d_tab;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        b->last_error = "batch: stream capture could not begin";
        return HYB_ERR_CUDA;
    }
    long long n = 0;
    cudaEventRecord(b->fork, b->main);
    for (size_t q = 0; q < P.gs.size() && !rc; q++) {
        // the group's branch runs on its first instance's stream
        const int k0 = P.gs[q].members[0];
        cudaStream_t s = b->inst[k0]->stream;
        cudaStreamWaitEvent(s, b->fork, 0);
        rc = group_launches(b, P, P.gs[q], t, s);
        if (rc) b->last_error = "batch: batched launch failed";
        cudaEventRecord(b->done[k0], s);
        cudaStreamWaitEvent(b->main, b->done[k0], 0);
        n += last ? 7 : 5;
    }
    if (last) {
        for (int L = 0; L < 6 && !rc; L++, n++)
            rc = hyb::cns_batch_launch(t + P.o_cns, (const int4 *)(t + P.o_cwork[L]), P.n_cwork[L], b->main);
        if (!rc) rc = hyb::residual_final_batch_launch(t + P.o_rfin, (int)b->inst.size(), b->d_res, b->main);
        n++;
    }
    if (!rc) rc = hyb::gather_err_launch((int *const *)(t + P.o_err), b->d_errs, (int)b->inst.size(), b->main);
    n++;
    cudaError_t e = cudaStreamEndCapture(b->main, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc == HYB_ERR_UNSUPPORTED ? HYB_ERR_CUDA : rc;
    }
    if (e != cudaSuccess || !g) {
        b->last_error = std::string("batch: capture failed: ") + cudaGetErrorString(e);
        return HYB_ERR_CUDA;
    }
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->last_error = std::string("batch: graph instantiation failed: ") + cudaGetErrorString(e);
        return HYB_ERR_CUDA;
    }
    *nodes = n;
    return HYB_OK;
}

// capture one iteration of every instance into one graph
int build_graph(hyb_batch *b, int store_rhs, cudaGraphExec_t *exec, long long *nodes) {
    for (hyb_ctx *c : b->inst) {
        int rc = hyb::sweep_prepare(c);   // kernel attributes outside the capture
        if (rc) return rc;
    }
    std::vector<long long> l0(b->inst.size());
    for (size_t k = 0; k < b->inst.size(); k++) l0[k] = b->inst[k]->launches;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        b->last_error = "batch: stream capture could not begin";
        return HYB_ERR_CUDA;
    }
    int rc = HYB_OK;
    cudaEventRecord(b->fork, b->main);
    for (size_t k = 0; k < b->inst.size() && !rc; k++) {
        hyb_ctx *c = b->inst[k];
        cudaStreamWaitEvent(c->stream, b->fork, 0);
        rc = iteration(c, store_rhs);
        if (!rc && store_rhs) {
            rc = hyb::launch_residual(c, nullptr);
            if (!rc && cudaMemcpyAsync(b->d_res + 9 * k, c->d_resid, 9 * sizeof(double), cudaMemcpyDeviceToDevice,
                                       c->stream) != cudaSuccess)
                rc = HYB_ERR_CUDA;
        }
        if (!rc && cudaMemcpyAsync(b->d_errs + k, c->d_err, sizeof(int), cudaMemcpyDeviceToDevice, c->stream) !=
                       cudaSuccess)
            rc = HYB_ERR_CUDA;
        if (rc) b->last_error = "batch instance " + std::to_string(k) + ": " + c->last_error;
        cudaEventRecord(b->done[k], c->stream);
        cudaStreamWaitEvent(b->main, b->done[k], 0);
    }
    cudaError_t e = cudaStreamEndCapture(b->main, &g);
    long long n = 0;
    for (size_t k = 0; k < b->inst.size(); k++) {
        n += b->inst[k]->launches - l0[k];
        b->inst[k]->launches = l0[k];      // captured, not executed
    }
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess || !g) {
        b->last_error = std::string("batch: capture failed: ") + cudaGetErrorString(e);
        return HYB_ERR_CUDA;
    }
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->last_error = std::string("batch: graph instantiation failed: ") + cudaGetErrorString(e);
        return HYB_ERR_CUDA;
    }
    *nodes = n;
    return HYB_OK;
}

}  // namespace

extern "C" {

int hyb_autotune(hyb_ctx *ctx, int reps, int *cpt_out, int *vpb_out) {
    if (!ctx || reps < 1) return HYB_ERR_INVALID;
    cudaSetDevice(ctx->dev);
    const size_t fbytes = (size_t)ctx->nv * 2 * ctx->Nb * ctx->PA * ctx->real_size;
    int rc = hyb::launch_wall(ctx);
    if (rc) return rc;
    HYB_CK(cudaMemcpyAsync(ctx->d_rhs, ctx->d_f, fbytes, cudaMemcpyDeviceToDevice, ctx->stream));
    const int old_c = ctx->sw_cpt, old_v = ctx->sw_vpb;
    const long long l0 = ctx->launches;
    float best = 1e30f;
    int bc = 0, bv = 0;
    const int cands_c[3] = {4, 2, 1}, cands_v[4] = {1, 2, 4, 8};
    for (int ci = 0; ci < 3; ci++) {
        const int c = cands_c[ci];
        if (!hyb::sweep_cpt_ok(ctx, c)) continue;
        for (int vi = 0; vi < 4; vi++) {
            const int v = cands_v[vi];
            if ((ctx->PA / c) * v > 256) continue;
            ctx->sw_cpt = c;
            ctx->sw_vpb = v;
            if (hyb::sweep_smem_bytes(ctx) > 227 * 1024) continue;
            rc = hyb::sweep_prepare(ctx);
            if (!rc) rc = hyb::launch_sweep(ctx, 0);   // warm-up
            if (rc) break;
            HYB_CK(cudaEventRecord(ctx->ev0, ctx->stream));
            for (int r = 0; r < reps && !rc; r++) rc = hyb::launch_sweep(ctx, 0);
            HYB_CK(cudaEventRecord(ctx->ev1, ctx->stream));
            HYB_CK(cudaEventSynchronize(ctx->ev1));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
            HYB_CK(cudaMemcpyAsync(ctx->d_f, ctx->d_rhs, fbytes, cudaMemcpyDeviceToDevice, ctx->stream));
            if (rc) break;
            if (ms < best) {
                best = ms;
                bc = c;
                bv = v;
            }
        }
        if (rc) break;
    }
    HYB_CK(cudaStreamSynchronize(ctx->stream));
    ctx->launches = l0;   // timing launches are not solver work
    ctx->rhs_valid = 0;
    if (rc || bc == 0) {
        ctx->sw_cpt = old_c;
        ctx->sw_vpb = old_v;
        if (!rc) {
            ctx->last_error = "autotune: no admissible sweep shape";
            rc = HYB_ERR_UNSUPPORTED;
        }
        return rc;
    }
    ctx->sw_cpt = bc;
    ctx->sw_vpb = bv;
    if (cpt_out) *cpt_out = bc;
    if (vpb_out) *vpb_out = bv;
    return ctx_err_word(ctx);
}

int hyb_batch_create(int n, const hyb_mesh *meshes, const hyb_vgrid *vgrids, const hyb_params *params,
                     hyb_batch **out) {
    if (n < 1 || !meshes || !vgrids || !params || !out) return HYB_ERR_INVALID;
    *out = nullptr;
    hyb_batch *b = new (std::nothrow) hyb_batch();
    if (!b) return HYB_ERR_NOMEM;
    b->dev = params[0].device;
    for (int k = 0; k < n; k++) {
        if (params[k].device != b->dev || params[k].precision != params[0].precision) {
            hyb_batch_destroy(b);
            return HYB_ERR_INVALID;
        }
        // the batched graphs carry the reference order without a mass scale
        if (params[k].sweep_order != HYB_SWEEP_REFERENCE || params[k].mass_pin) {
            hyb_batch_destroy(b);
            return HYB_ERR_UNSUPPORTED;
        }
        hyb_ctx *c = nullptr;
        int rc = hyb_create(&meshes[k], &vgrids[k], &params[k], &c);
        if (rc) {
            hyb_batch_destroy(b);
            return rc;
        }
        c->in_batch = 1;
        b->inst.push_back(c);
    }
    cudaSetDevice(b->dev);
    b->done.assign(n, nullptr);
    bool ok = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreate(&b->ev0) == cudaSuccess && cudaEventCreate(&b->ev1) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 0; k < n && ok; k++) ok = cudaEventCreateWithFlags(&b->done[k], cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaMalloc((void **)&b->d_res, (size_t)9 * n * sizeof(double)) == cudaSuccess &&
         cudaMalloc((void **)&b->d_errs, (size_t)n * sizeof(int)) == cudaSuccess &&
         cudaMallocHost((void **)&b->h_res, (size_t)9 * n * sizeof(double)) == cudaSuccess &&
         cudaMallocHost((void **)&b->h_errs, (size_t)n * sizeof(int)) == cudaSuccess;
    if (ok) ok = cudaMemset(b->d_errs, 0, (size_t)n * sizeof(int)) == cudaSuccess;
    if (!ok) {
        hyb_batch_destroy(b);
        return HYB_ERR_CUDA;
    }
    *out = b;
    return HYB_OK;
}

int hyb_batch_destroy(hyb_batch *b) {
    if (!b) return HYB_ERR_INVALID;
    cudaSetDevice(b->dev);
    if (b->main) cudaStreamSynchronize(b->main);
    drop_graphs(b);
    for (cudaEvent_t e : b->done)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->main) cudaStreamDestroy(b->main);
    if (b->d_res) cudaFree(b->d_res);
    if (b->d_errs) cudaFree(b->d_errs);
    if (b->h_res) cudaFreeHost(b->h_res);
    if (b->h_errs) cudaFreeHost(b->h_errs);
    for (hyb_ctx *c : b->inst) hyb_destroy(c);
    delete b;
    return HYB_OK;
}

const char *hyb_batch_last_error(const hyb_batch *b) { return b ? b->last_error.c_str() : "null batch"; }

int hyb_batch_size(const hyb_batch *b, int *n) {
    if (!b || !n) return HYB_ERR_INVALID;
    *n = (int)b->inst.size();
    return HYB_OK;
}

int hyb_batch_instance(hyb_batch *b, int k, hyb_ctx **ctx) {
    if (!b || !ctx || k < 0 || k >= (int)b->inst.size()) return HYB_ERR_INVALID;
    *ctx = b->inst[k];
    return HYB_OK;
}

int hyb_batch_init_maxwellian(hyb_batch *b, double rho, double u, double v, double t) {
    if (!b) return HYB_ERR_INVALID;
    for (size_t k = 0; k < b->inst.size(); k++) {
        int rc = hyb_init_maxwellian(b->inst[k], rho, u, v, t);
        if (rc) {
            b->last_error = "batch instance " + std::to_string(k) + ": " + b->inst[k]->last_error;
            return rc;
        }
    }
    return HYB_OK;
}

// instances of the same mesh and velocity-grid sizes share one tuned shape:
// the first of them is timed and the rest take its shape, so that they fall
// into one launch group
static bool same_sizes(const hyb_ctx *a, const hyb_ctx *c) {
    return a->PA == c->PA && a->Na == c->Na && a->Nb == c->Nb && a->nvi == c->nvi && a->nvj == c->nvj &&
           a->cpt == c->cpt && a->uniform == c->uniform && a->prm.scheme == c->prm.scheme;
}

int hyb_batch_autotune(hyb_batch *b, int reps) {
    if (!b || reps < 1) return HYB_ERR_INVALID;
    drop_graphs(b);   // the captured launches carry the old shapes
    for (size_t k = 0; k < b->inst.size(); k++) {
        hyb_ctx *c = b->inst[k];
        size_t j = 0;
        while (j < k && !same_sizes(b->inst[j], c)) j++;
        if (j < k) {
            c->sw_cpt = b->inst[j]->sw_cpt;
            c->sw_vpb = b->inst[j]->sw_vpb;
            continue;
        }
        int rc = hyb_autotune(c, reps, nullptr, nullptr);
        if (rc) {
            b->last_error = "batch instance " + std::to_string(k) + ": " + c->last_error;
            return rc;
        }
    }
    return HYB_OK;
}

int hyb_batch_step(hyb_batch *b, int n_iter, hyb_residual *res) {
    if (!b || n_iter < 1) return HYB_ERR_INVALID;
    cudaSetDevice(b->dev);
    int rc = HYB_OK;
    if (!b->g_iter) {
        rc = build_graph_batched(b, false, &b->g_iter, &b->nodes_iter, &b->d_tab_iter);
        if (rc == HYB_ERR_UNSUPPORTED) rc = build_graph(b, 0, &b->g_iter, &b->nodes_iter);
    }
    if (!rc && !b->g_last) {
        rc = build_graph_batched(b, true, &b->g_last, &b->nodes_last, &b->d_tab_last);
        if (rc == HYB_ERR_UNSUPPORTED) rc = build_graph(b, 1, &b->g_last, &b->nodes_last);
    }
    if (rc) return rc;
    cudaEventRecord(b->ev0, b->main);
    for (int it = 0; it < n_iter; it++) {
        const bool last = it == n_iter - 1;   // RHS, residual and Convert_NS
        cudaError_t e = cudaGraphLaunch(last ? b->g_last : b->g_iter, b->main);
        if (e != cudaSuccess) {
            b->last_error = std::string("batch: graph launch failed: ") + cudaGetErrorString(e);
            return HYB_ERR_CUDA;
        }
        b->launches += last ? b->nodes_last : b->nodes_iter;
    }
    cudaEventRecord(b->ev1, b->main);
    const size_t n = b->inst.size();
    cudaMemcpyAsync(b->h_errs, b->d_errs, n * sizeof(int), cudaMemcpyDeviceToHost, b->main);
    if (res) cudaMemcpyAsync(b->h_res, b->d_res, 9 * n * sizeof(double), cudaMemcpyDeviceToHost, b->main);
    if (cudaStreamSynchronize(b->main) != cudaSuccess) {
        b->last_error = std::string("batch: ") + cudaGetErrorString(cudaGetLastError());
        return HYB_ERR_CUDA;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    b->last_ms = ms;
    for (size_t k = 0; k < n; k++) {
        hyb_ctx *c = b->inst[k];
        if (b->h_errs[k] != 0) {
            rc = ctx_err_word(c);   // clears the instance's word
            cudaMemset(b->d_errs + k, 0, sizeof(int));
            b->last_error = "batch instance " + std::to_string(k) + ": " + c->last_error;
            return rc ? rc : HYB_ERR_TIMEOUT;
        }
        if (res) {
            c->rhs_valid = 1;
            const double *r = b->h_res + 9 * k;
            for (int q = 0; q < 4; q++) {
                res[k].res_max[q] = r[q];
                res[k].res_rms[q] = r[4 + q];
            }
            res[k].max_rms = r[8];
            for (int q = 0; q < 4; q++)
                if (!isfinite(r[q]) || !isfinite(r[4 + q])) {
                    b->last_error = "batch instance " + std::to_string(k) + ": non-finite residual";
                    return HYB_ERR_NONFINITE;
                }
        }
    }
    return HYB_OK;
}

int hyb_batch_last_step_ms(const hyb_batch *b, double *ms) {
    if (!b || !ms) return HYB_ERR_INVALID;
    *ms = b->last_ms;
    return HYB_OK;
}

int hyb_batch_launch_count(const hyb_batch *b, long long *count) {
    if (!b || !count) return HYB_ERR_INVALID;
    *count = b->launches;
    return HYB_OK;
}

}  // extern "C"
