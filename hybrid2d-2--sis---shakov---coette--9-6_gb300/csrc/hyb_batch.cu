// hyb_batch.cu -- batched Couette instances and the sweep-shape autotuner.
//
// A batch owns one context per instance (each with its own stream and
// buffers, so instances of different mesh and velocity-grid sizes coexist).
// One outer iteration of every instance -- wall, sweep, moments, S ghosts
// (and Convert_NS on the last iteration of a step) -- is captured once into a single
// CUDA graph whose per-instance chains are independent branches, so one
// graph launch advances all instances by one iteration and the GPU runs the
// small per-instance kernels side by side.  Two graphs are kept: one for
// plain iterations and one whose sweeps also store the RHS (used on the last
// iteration when residuals are requested).
//
// The autotuner (hyb_autotune) times every admissible sweep launch shape
// (cells per thread dividing the layout chunk, velocity groups per CTA up to
// 256 threads and 227 KB of shared memory) on the context's own data: f is
// saved to the RHS buffer, each candidate runs `reps` sweeps timed with CUDA
// events, f is restored after every candidate, and the fastest shape is kept
// in the context.  No counterpart in the reference.
#include <cuda_runtime.h>
#include <math.h>

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
        if (ctx->cpt % c != 0 || ctx->PA / c > 256) continue;
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
        hyb_ctx *c = nullptr;
        int rc = hyb_create(&meshes[k], &vgrids[k], &params[k], &c);
        if (rc) {
            hyb_batch_destroy(b);
            return rc;
        }
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

int hyb_batch_autotune(hyb_batch *b, int reps) {
    if (!b || reps < 1) return HYB_ERR_INVALID;
    drop_graphs(b);   // the captured launches carry the old shapes
    for (size_t k = 0; k < b->inst.size(); k++) {
        int rc = hyb_autotune(b->inst[k], reps, nullptr, nullptr);
        if (rc) {
            b->last_error = "batch instance " + std::to_string(k) + ": " + b->inst[k]->last_error;
            return rc;
        }
    }
    return HYB_OK;
}

int hyb_batch_step(hyb_batch *b, int n_iter, hyb_residual *res) {
    if (!b || n_iter < 1) return HYB_ERR_INVALID;
    cudaSetDevice(b->dev);
    int rc = HYB_OK;
    if (!b->g_iter) rc = build_graph(b, 0, &b->g_iter, &b->nodes_iter);
    if (!rc && !b->g_last) rc = build_graph(b, 1, &b->g_last, &b->nodes_last);
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
