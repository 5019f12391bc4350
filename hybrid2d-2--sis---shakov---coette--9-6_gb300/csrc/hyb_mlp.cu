// hyb_mlp.cu -- the learned closure: an 8 -> 64 -> 64 -> 64 -> 4 MLP (tanh
// hidden layers, linear output, 9,156 parameters) that predicts the non-NSF
// part of the stress and heat flux (the HoT of Convert_NS) from local
// macroscopic features.  No counterpart in the reference.
//
// Arithmetic: weights and activations in BF16, products on the tensor cores
// with mma.sync.m16n8k16 (BF16 in, FP32 accumulate), biases, activations,
// loss and the Adam update in FP32 on an FP32 master copy of the weights.
// One CTA of 8 warps owns a tile of 128 samples: the forward pass keeps the
// tile's activations in shared memory, the backward pass produces the
// tile's weight and bias gradients (reductions over the tile's samples run
// on the tensor cores as well), written as one partial per CTA.  A second
// kernel sums the partials in a fixed order (deterministic) and applies
// Adam.  The network is small enough that every launch is latency bound; the
// kernels are written for one pass over the data per launch.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <new>
#include <string>
#include <vector>

#include "hyb_common.cuh"

namespace hyb {
namespace mlp {

constexpr int IN = 8, H = 64, OUT = 4, TILE = 128, WARPS = 8, THREADS = 32 * WARPS;
constexpr int K1 = 16;   // input width padded to one MMA k-step
constexpr int N4 = 8;    // output width padded to one MMA n-tile
// FP32 parameter layout: W1[H][IN] b1[H] W2[H][H] b2[H] W3[H][H] b3[H] W4[OUT][H] b4[OUT]
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * IN, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H;
constexpr int OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H * H, OFF_W4 = OFF_B3 + H, OFF_B4 = OFF_W4 + OUT * H;
constexpr int NPARAM = OFF_B4 + OUT;   // 9156
// BF16 weight layout (padded): W1[H][K1] W2[H][H] W3[H][H] W4[N4][H]
constexpr int BW1 = 0, BW2 = BW1 + H * K1, BW3 = BW2 + H * H, BW4 = BW3 + H * H, NBW = BW4 + N4 * H;

typedef __nv_bfloat16 bf16;

struct Norm {
    float in_mu[IN], in_is[IN];     // x_norm = (x - mu) * is
    float out_mu[OUT], out_sd[OUT]; // y = y_norm * sd + mu
};

// shared-memory tile of one CTA
struct Smem {
    bf16 w[NBW];
    float b[3 * H + N4];
    bf16 x[TILE][K1];
    bf16 h1[TILE][H], h2[TILE][H], h3[TILE][H];
    float y[TILE][N4];
    bf16 dz[TILE][H];     // current layer's output gradient (BF16 MMA operand)
    bf16 dh[TILE][H];     // gradient w.r.t. the layer's input, before the tanh derivative
    float red[WARPS][H];  // per-warp partial bias gradients
    float lossw[WARPS];
};

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// D(16x8) += A(16xK) B(Kx8) on the tensor cores; A(m,k) and B(k,n) are
// fetched through functors (any shared-memory layout).  Fragment layout of
// mma.m16n8k16 (PTX ISA): lane = 4g + t; A regs (g,2t..) (g+8,2t..)
// (g,2t+8..) (g+8,2t+8..); B regs (k=2t..,n=g) (k=2t+8..,n=g); C (g,2t..)
// (g+8,2t..).
template <class FA, class FB>
__device__ __forceinline__ void mma_tile(const FA &A, const FB &B, int K, float c[4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int k0 = 0; k0 < K; k0 += 16) {
        const int ka = k0 + 2 * t;
        const uint32_t a0 = pack2(A(g, ka), A(g, ka + 1));
        const uint32_t a1 = pack2(A(g + 8, ka), A(g + 8, ka + 1));
        const uint32_t a2 = pack2(A(g, ka + 8), A(g, ka + 9));
        const uint32_t a3 = pack2(A(g + 8, ka + 8), A(g + 8, ka + 9));
        const uint32_t b0 = pack2(B(ka, g), B(ka + 1, g));
        const uint32_t b1 = pack2(B(ka + 8, g), B(ka + 9, g));
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};\n"
            : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
            : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
}

// one dense layer over the CTA's tile: out[r][n] = act(sum_k in[r][k] W[n][k]
// + b[n]); warp w owns rows 16w..16w+15
template <int KIN, int NOUT, bool TANH, class FIn, class FOut>
__device__ __forceinline__ void dense(const bf16 *W, const float *bias, const FIn &in, const FOut &out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int r0 = 16 * warp;
    auto A = [&](int m, int k) { return in(r0 + m, k); };
    for (int nt = 0; nt < NOUT / 8; nt++) {
        auto B = [&](int k, int n) { return W[(nt * 8 + n) * KIN + k]; };
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        mma_tile(A, B, KIN, c);
        const int n0 = nt * 8 + 2 * t;
        for (int q = 0; q < 4; q++) {
            const int r = r0 + g + (q >= 2 ? 8 : 0), n = n0 + (q & 1);
            float v = c[q] + bias[n];
            if (TANH) v = tanhf(v);
            out(r, n, v);
        }
    }
}

// weights and biases of all layers into shared memory
__device__ __forceinline__ void load_params(Smem &S, const bf16 *wb, const float *bias) {
    for (int e = threadIdx.x; e < NBW; e += THREADS) S.w[e] = wb[e];
    for (int e = threadIdx.x; e < 3 * H + N4; e += THREADS) S.b[e] = bias[e];
}

// forward pass of one tile; rows >= nrow get zero inputs.  Sample of tile
// row r: idx ? idx[pos0 + r] : pos0 + r.
__device__ void forward_tile(Smem &S, const float *x, const int *idx, int pos0, int nrow, const Norm &nm) {
    for (int e = threadIdx.x; e < TILE * K1; e += THREADS) {
        const int r = e / K1, k = e % K1;
        float v = 0.f;
        if (k < IN && r < nrow) {
            const long long smp = idx ? idx[pos0 + r] : (long long)pos0 + r;
            v = (x[smp * IN + k] - nm.in_mu[k]) * nm.in_is[k];
        }
        S.x[r][k] = __float2bfloat16(v);
    }
    __syncthreads();
    // every warp reads and writes only its own 16 rows from here on
    dense<K1, H, true>(S.w + BW1, S.b, [&](int r, int k) { return S.x[r][k]; },
                       [&](int r, int n, float v) { S.h1[r][n] = __float2bfloat16(v); });
    __syncwarp();
    dense<H, H, true>(S.w + BW2, S.b + H, [&](int r, int k) { return S.h1[r][k]; },
                      [&](int r, int n, float v) { S.h2[r][n] = __float2bfloat16(v); });
    __syncwarp();
    dense<H, H, true>(S.w + BW3, S.b + 2 * H, [&](int r, int k) { return S.h2[r][k]; },
                      [&](int r, int n, float v) { S.h3[r][n] = __float2bfloat16(v); });
    __syncwarp();
    dense<H, N4, false>(S.w + BW4, S.b + 3 * H, [&](int r, int k) { return S.h3[r][k]; },
                        [&](int r, int n, float v) { S.y[r][n] = v; });
    __syncthreads();
}

__global__ void __launch_bounds__(THREADS) k_mlp_forward(const bf16 *wb, const float *bias, Norm nm,
                                                          const float *x, int n, float *y) {
    extern __shared__ __align__(16) unsigned char raw[];
    Smem &S = *reinterpret_cast<Smem *>(raw);
    load_params(S, wb, bias);
    const int pos0 = blockIdx.x * TILE, nrow = min(TILE, n - pos0);
    forward_tile(S, x, nullptr, pos0, nrow, nm);
    for (int e = threadIdx.x; e < TILE * OUT; e += THREADS) {
        const int r = e / OUT, o = e % OUT;
        if (r < nrow) y[(size_t)(pos0 + r) * OUT + o] = S.y[r][o] * nm.out_sd[o] + nm.out_mu[o];
    }
}

// weight-gradient tile: G[o][i] += sum_r dZ[r][o] In[r][i] over the tile's
// 128 rows (K = 128), M tile mt (16 outputs), N tile nt (8 inputs)
template <class FD, class FI>
__device__ __forceinline__ void wgrad_tile(const FD &dz, const FI &inp, int mt, int nt, int nout, int nin,
                                           float *g) {
    const int lane = threadIdx.x & 31, gq = lane >> 2, t = lane & 3;
    auto A = [&](int m, int k) { return dz(k, mt * 16 + m); };
    auto B = [&](int k, int n) { return inp(k, nt * 8 + n); };
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    mma_tile(A, B, TILE, c);
    for (int q = 0; q < 4; q++) {
        const int o = mt * 16 + gq + (q >= 2 ? 8 : 0), i = nt * 8 + 2 * t + (q & 1);
        if (o < nout && i < nin) g[o * nin + i] = c[q];
    }
}

// input-gradient of a tanh layer for the warp's rows: dZ_prev[r][i] =
// (sum_o dZ[r][o] W[o][i]) (1 - h[r][i]^2); writes BF16 dZ_prev and the
// warp's partial bias gradient red[warp][i]
template <int KO, class FD, class FW, class FH, class FOut>
__device__ __forceinline__ void igrad_tanh(Smem &S, const FD &dz, const FW &W, const FH &h, const FOut &out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int r0 = 16 * warp;
    auto A = [&](int m, int k) { return dz(r0 + m, k); };
    for (int nt = 0; nt < H / 8; nt++) {
        auto B = [&](int k, int n) { return W(k, nt * 8 + n); };
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        mma_tile(A, B, KO, c);
        float col[2] = {0.f, 0.f};
        for (int q = 0; q < 4; q++) {
            const int r = r0 + g + (q >= 2 ? 8 : 0), i = nt * 8 + 2 * t + (q & 1);
            const float hv = __bfloat162float(h(r, i));
            const float v = c[q] * (1.f - hv * hv);
            out(r, i, __float2bfloat16(v));
            col[q & 1] += v;
        }
        for (int off = 4; off < 32; off <<= 1) {
            col[0] += __shfl_xor_sync(0xffffffffu, col[0], off);
            col[1] += __shfl_xor_sync(0xffffffffu, col[1], off);
        }
        if (g == 0) {
            S.red[warp][nt * 8 + 2 * t] = col[0];
            S.red[warp][nt * 8 + 2 * t + 1] = col[1];
        }
    }
}

__device__ __forceinline__ void bias_from_red(const Smem &S, float *g) {
    if (threadIdx.x < H) {
        float s = 0.f;
        for (int w = 0; w < WARPS; w++) s += S.red[w][threadIdx.x];
        g[threadIdx.x] = s;
    }
}

// forward + backward of one tile of a minibatch; writes the tile's gradient
// partial gpart[blockIdx.x][NPARAM] and loss partial lpart[blockIdx.x]
__global__ void __launch_bounds__(THREADS) k_mlp_train(const bf16 *wb, const float *bias, Norm nm, const float *x,
                                                        const float *ytrue, const int *idx, int nb, float inv_count,
                                                        float *gpart, float *lpart) {
    extern __shared__ __align__(16) unsigned char raw[];
    Smem &S = *reinterpret_cast<Smem *>(raw);
    load_params(S, wb, bias);
    const int pos0 = blockIdx.x * TILE, nrow = min(TILE, nb - pos0);
    forward_tile(S, x, idx, pos0, nrow, nm);
    float *G = gpart + (size_t)blockIdx.x * NPARAM;
    const int warp = threadIdx.x >> 5;
    // output gradient dY = 2 (y - t) / (nb OUT), loss partial
    float lsum = 0.f;
    for (int e = threadIdx.x; e < TILE * 16; e += THREADS) {
        const int r = e / 16, o = e % 16;
        float v = 0.f;
        if (r < nrow && o < OUT) {
            const long long smp = idx ? idx[pos0 + r] : (long long)pos0 + r;
            const float tn = (ytrue[smp * OUT + o] - nm.out_mu[o]) / nm.out_sd[o];
            const float d = S.y[r][o] - tn;
            lsum += d * d;
            v = 2.f * d * inv_count;
        }
        S.dz[r][o] = __float2bfloat16(v);
        if (o < N4) S.y[r][o] = v;   // FP32 copy for the bias gradient
    }
    for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
    if ((threadIdx.x & 31) == 0) S.lossw[warp] = lsum;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < WARPS; w++) s += S.lossw[w];
        lpart[blockIdx.x] = s;
    }
    if (threadIdx.x < OUT) {
        float s = 0.f;
        for (int r = 0; r < TILE; r++) s += S.y[r][threadIdx.x];
        G[OFF_B4 + threadIdx.x] = s;
    }
    // layer 4: dW4 (warp w: inputs 8w..8w+7), dZ3 = (dY W4) (1 - h3^2)
    wgrad_tile([&](int r, int o) { return S.dz[r][o]; }, [&](int r, int i) { return S.h3[r][i]; }, 0, warp, OUT, H,
               G + OFF_W4);
    igrad_tanh<16>(S, [&](int r, int o) { return S.dz[r][o]; },
                   [&](int o, int i) { return o < N4 ? S.w[BW4 + o * H + i] : __float2bfloat16(0.f); },
                   [&](int r, int i) { return S.h3[r][i]; }, [&](int r, int i, bf16 v) { S.dh[r][i] = v; });
    __syncthreads();
    bias_from_red(S, G + OFF_B3);
    __syncthreads();
    // layer 3: dW3 from dZ3 (S.dh) and h2; dZ2 into S.dz
    for (int tile = warp; tile < 32; tile += WARPS)
        wgrad_tile([&](int r, int o) { return S.dh[r][o]; }, [&](int r, int i) { return S.h2[r][i]; }, tile / 8,
                   tile % 8, H, H, G + OFF_W3);
    igrad_tanh<H>(S, [&](int r, int o) { return S.dh[r][o]; }, [&](int o, int i) { return S.w[BW3 + o * H + i]; },
                  [&](int r, int i) { return S.h2[r][i]; }, [&](int r, int i, bf16 v) { S.dz[r][i] = v; });
    __syncthreads();
    bias_from_red(S, G + OFF_B2);
    __syncthreads();
    // layer 2: dW2 from dZ2 (S.dz) and h1; dZ1 into S.dh
    for (int tile = warp; tile < 32; tile += WARPS)
        wgrad_tile([&](int r, int o) { return S.dz[r][o]; }, [&](int r, int i) { return S.h1[r][i]; }, tile / 8,
                   tile % 8, H, H, G + OFF_W2);
    igrad_tanh<H>(S, [&](int r, int o) { return S.dz[r][o]; }, [&](int o, int i) { return S.w[BW2 + o * H + i]; },
                  [&](int r, int i) { return S.h1[r][i]; }, [&](int r, int i, bf16 v) { S.dh[r][i] = v; });
    __syncthreads();
    bias_from_red(S, G + OFF_B1);
    // layer 1: dW1 from dZ1 (S.dh) and the inputs
    if (warp < 4)
        wgrad_tile([&](int r, int o) { return S.dh[r][o]; }, [&](int r, int i) { return S.x[r][i]; }, warp, 0, H, IN,
                   G + OFF_W1);
}

// fixed-order sum of the tile partials, optional gradient output, Adam on
// the FP32 master weights, BF16 / bias copies for the next forward pass
__global__ void k_mlp_adam(float *w, float *m1, float *m2, bf16 *wb, float *bias, const float *gpart, int nparts,
                           float lr, float c1, float c2, float *grad_out, const float *lpart, float *loss_out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0 && loss_out) {
        float s = 0.f;
        for (int c = 0; c < nparts; c++) s += lpart[c];
        *loss_out = s;
    }
    if (p >= NPARAM) return;
    float g = 0.f;
    for (int c = 0; c < nparts; c++) g += gpart[(size_t)c * NPARAM + p];
    if (grad_out) grad_out[p] = g;
    float wv = w[p];
    if (lr > 0.f) {
        const float a = 0.9f * m1[p] + 0.1f * g, b = 0.999f * m2[p] + 0.001f * g * g;
        m1[p] = a;
        m2[p] = b;
        wv -= lr * (a / c1) / (sqrtf(b / c2) + 1e-8f);
        w[p] = wv;
    }
    if (p < OFF_B1) wb[BW1 + (p / IN) * K1 + p % IN] = __float2bfloat16(wv);
    else if (p < OFF_W2) bias[p - OFF_B1] = wv;
    else if (p < OFF_B2) wb[BW2 + (p - OFF_W2)] = __float2bfloat16(wv);
    else if (p < OFF_W3) bias[H + p - OFF_B2] = wv;
    else if (p < OFF_B3) wb[BW3 + (p - OFF_W3)] = __float2bfloat16(wv);
    else if (p < OFF_W4) bias[2 * H + p - OFF_B3] = wv;
    else if (p < OFF_B4) wb[BW4 + (p - OFF_W4)] = __float2bfloat16(wv);
    else bias[3 * H + p - OFF_B4] = wv;
}

}  // namespace mlp
}  // namespace hyb

// ---- host side ----------------------------------------------------------------
struct hyb_mlp {
    int dev = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float *w = nullptr, *m1 = nullptr, *m2 = nullptr, *bias = nullptr, *grad = nullptr;
    hyb::mlp::bf16 *wb = nullptr;
    float *x = nullptr, *y = nullptr;   // resident training set
    int n = 0;
    int *idx = nullptr;
    int idx_cap = 0;
    float *gpart = nullptr, *lpart = nullptr, *loss = nullptr;
    int part_cap = 0, loss_cap = 0;
    float *tx = nullptr, *ty = nullptr;   // staging of predict / grad inputs
    size_t t_cap = 0;
    long long adam_t = 0;
    hyb::mlp::Norm nm;
    double last_ms = 0.0;
    long long launches = 0;
    std::string last_error;
};

namespace {
using namespace hyb::mlp;

#define MCK(call)                                                                   \
    do {                                                                            \
        cudaError_t _e = (call);                                                    \
        if (_e != cudaSuccess) {                                                    \
            m->last_error = std::string(#call) + ": " + cudaGetErrorString(_e);     \
            return HYB_ERR_CUDA;                                                    \
        }                                                                           \
    } while (0)

uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int grow_parts(hyb_mlp *m, int tiles) {
    if (tiles <= m->part_cap) return HYB_OK;
    if (m->gpart) cudaFree(m->gpart);
    if (m->lpart) cudaFree(m->lpart);
    m->gpart = m->lpart = nullptr;
    MCK(cudaMalloc((void **)&m->gpart, (size_t)tiles * NPARAM * sizeof(float)));
    MCK(cudaMalloc((void **)&m->lpart, (size_t)tiles * sizeof(float)));
    m->part_cap = tiles;
    return HYB_OK;
}

int grow_staging(hyb_mlp *m, size_t n) {
    if (n <= m->t_cap) return HYB_OK;
    if (m->tx) cudaFree(m->tx);
    if (m->ty) cudaFree(m->ty);
    m->tx = m->ty = nullptr;
    MCK(cudaMalloc((void **)&m->tx, n * IN * sizeof(float)));
    MCK(cudaMalloc((void **)&m->ty, n * OUT * sizeof(float)));
    m->t_cap = n;
    return HYB_OK;
}

int sync_copies(hyb_mlp *m) {
    // bf16 / bias copies of the master weights (an Adam launch with lr = 0)
    k_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, m->stream>>>(m->w, m->m1, m->m2, m->wb, m->bias, m->gpart, 0, 0.f, 1.f,
                                                             1.f, nullptr, nullptr, nullptr);
    m->launches++;
    MCK(cudaGetLastError());
    return HYB_OK;
}

int set_attr(hyb_mlp *m) {
    static bool done = false;
    if (done) return HYB_OK;
    MCK(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Smem)));
    MCK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Smem)));
    done = true;
    return HYB_OK;
}

// forward + backward over positions [0, nb) of idx (or of the staged rows
// when idx is null), then the reduction / Adam launch
int train_launch(hyb_mlp *m, const float *x, const float *y, const int *idx, int nb, float lr, float *loss_slot,
                 float *grad_out) {
    const int tiles = (nb + TILE - 1) / TILE;
    int rc = grow_parts(m, tiles);
    if (rc) return rc;
    k_mlp_train<<<tiles, THREADS, sizeof(Smem), m->stream>>>(m->wb, m->bias, m->nm, x, y, idx, nb,
                                                             1.f / ((float)nb * OUT), m->gpart, m->lpart);
    float c1 = 1.f, c2 = 1.f;
    if (lr > 0.f) {
        m->adam_t++;
        c1 = 1.f - powf(0.9f, (float)m->adam_t);
        c2 = 1.f - powf(0.999f, (float)m->adam_t);
    }
    k_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, m->stream>>>(m->w, m->m1, m->m2, m->wb, m->bias, m->gpart, tiles, lr,
                                                             c1, c2, grad_out, m->lpart, loss_slot);
    m->launches += 2;
    MCK(cudaGetLastError());
    return HYB_OK;
}

}  // namespace

extern "C" {

int hyb_mlp_param_count(void) { return NPARAM; }

const char *hyb_mlp_last_error(const hyb_mlp *m) { return m ? m->last_error.c_str() : "null network"; }

int hyb_mlp_destroy(hyb_mlp *m) {
    if (!m) return HYB_ERR_INVALID;
    cudaSetDevice(m->dev);
    if (m->stream) cudaStreamSynchronize(m->stream);
    void *bufs[] = {m->w, m->m1, m->m2, m->bias, m->grad, m->wb, m->x, m->y, m->idx,
                    m->gpart, m->lpart, m->loss, m->tx, m->ty};
    for (void *p : bufs)
        if (p) cudaFree(p);
    if (m->ev0) cudaEventDestroy(m->ev0);
    if (m->ev1) cudaEventDestroy(m->ev1);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return HYB_OK;
}

int hyb_mlp_set_params(hyb_mlp *m, const float *w) {
    if (!m || !w) return HYB_ERR_INVALID;
    cudaSetDevice(m->dev);
    MCK(cudaMemcpyAsync(m->w, w, NPARAM * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCK(cudaMemsetAsync(m->m1, 0, NPARAM * sizeof(float), m->stream));
    MCK(cudaMemsetAsync(m->m2, 0, NPARAM * sizeof(float), m->stream));
    m->adam_t = 0;
    int rc = sync_copies(m);
    if (!rc) MCK(cudaStreamSynchronize(m->stream));
    return rc;
}

int hyb_mlp_create(int device, unsigned long long seed, hyb_mlp **out) {
    if (!out) return HYB_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return HYB_ERR_NODEVICE;
    if (device < 0 || device >= ndev) return HYB_ERR_INVALID;
    hyb_mlp *m = new (std::nothrow) hyb_mlp();
    if (!m) return HYB_ERR_NOMEM;
    m->dev = device;
    cudaSetDevice(device);
    bool ok = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreate(&m->ev0) == cudaSuccess && cudaEventCreate(&m->ev1) == cudaSuccess;
    float **fb[] = {&m->w, &m->m1, &m->m2, &m->grad};
    for (float **p : fb) ok = ok && cudaMalloc((void **)p, NPARAM * sizeof(float)) == cudaSuccess;
    ok = ok && cudaMalloc((void **)&m->bias, (3 * H + N4) * sizeof(float)) == cudaSuccess &&
         cudaMalloc((void **)&m->wb, NBW * sizeof(bf16)) == cudaSuccess &&
         cudaMemset(m->wb, 0, NBW * sizeof(bf16)) == cudaSuccess &&
         cudaMemset(m->bias, 0, (3 * H + N4) * sizeof(float)) == cudaSuccess;
    if (!ok || set_attr(m) != HYB_OK) {
        hyb_mlp_destroy(m);
        return HYB_ERR_CUDA;
    }
    for (int k = 0; k < IN; k++) { m->nm.in_mu[k] = 0.f; m->nm.in_is[k] = 1.f; }
    for (int k = 0; k < OUT; k++) { m->nm.out_mu[k] = 0.f; m->nm.out_sd[k] = 1.f; }
    // Glorot-uniform weights, zero biases
    std::vector<float> w(NPARAM, 0.f);
    uint64_t s = seed;
    auto fill = [&](int off, int fo, int fi) {
        const double a = sqrt(6.0 / (fi + fo));
        for (int e = 0; e < fo * fi; e++) w[off + e] = (float)((2.0 * ((splitmix(s) >> 11) * 0x1.0p-53) - 1.0) * a);
    };
    fill(OFF_W1, H, IN);
    fill(OFF_W2, H, H);
    fill(OFF_W3, H, H);
    fill(OFF_W4, OUT, H);
    int rc = hyb_mlp_set_params(m, w.data());
    if (rc) {
        hyb_mlp_destroy(m);
        return rc;
    }
    *out = m;
    return HYB_OK;
}

int hyb_mlp_get_params(hyb_mlp *m, float *w) {
    if (!m || !w) return HYB_ERR_INVALID;
    cudaSetDevice(m->dev);
    MCK(cudaMemcpyAsync(w, m->w, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return HYB_OK;
}

int hyb_mlp_set_norm(hyb_mlp *m, const float *in_mean, const float *in_std, const float *out_mean,
                     const float *out_std) {
    if (!m || !in_mean || !in_std || !out_mean || !out_std) return HYB_ERR_INVALID;
    for (int k = 0; k < IN; k++)
        if (!(in_std[k] > 0.f)) return HYB_ERR_INVALID;
    for (int k = 0; k < OUT; k++)
        if (!(out_std[k] > 0.f)) return HYB_ERR_INVALID;
    for (int k = 0; k < IN; k++) {
        m->nm.in_mu[k] = in_mean[k];
        m->nm.in_is[k] = 1.f / in_std[k];
    }
    for (int k = 0; k < OUT; k++) {
        m->nm.out_mu[k] = out_mean[k];
        m->nm.out_sd[k] = out_std[k];
    }
    return HYB_OK;
}

int hyb_mlp_set_data(hyb_mlp *m, const float *x, const float *y, int n) {
    if (!m || !x || !y || n < 1) return HYB_ERR_INVALID;
    cudaSetDevice(m->dev);
    if (m->x) cudaFree(m->x);
    if (m->y) cudaFree(m->y);
    m->x = m->y = nullptr;
    m->n = 0;
    MCK(cudaMalloc((void **)&m->x, (size_t)n * IN * sizeof(float)));
    MCK(cudaMalloc((void **)&m->y, (size_t)n * OUT * sizeof(float)));
    MCK(cudaMemcpy(m->x, x, (size_t)n * IN * sizeof(float), cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(m->y, y, (size_t)n * OUT * sizeof(float), cudaMemcpyHostToDevice));
    m->n = n;
    return HYB_OK;
}

int hyb_mlp_train_epoch(hyb_mlp *m, const int *perm, int batch, float lr, float *mean_loss) {
    if (!m || !perm || batch < 1 || !(lr > 0.f) || m->n < 1) return HYB_ERR_INVALID;
    for (int k = 0; k < m->n; k++)
        if (perm[k] < 0 || perm[k] >= m->n) return HYB_ERR_INVALID;
    cudaSetDevice(m->dev);
    const int steps = (m->n + batch - 1) / batch;
    if (m->idx_cap < m->n) {
        if (m->idx) cudaFree(m->idx);
        m->idx = nullptr;
        MCK(cudaMalloc((void **)&m->idx, (size_t)m->n * sizeof(int)));
        m->idx_cap = m->n;
    }
    if (m->loss_cap < steps) {
        if (m->loss) cudaFree(m->loss);
        m->loss = nullptr;
        MCK(cudaMalloc((void **)&m->loss, (size_t)steps * sizeof(float)));
        m->loss_cap = steps;
    }
    MCK(cudaMemcpyAsync(m->idx, perm, (size_t)m->n * sizeof(int), cudaMemcpyHostToDevice, m->stream));
    MCK(cudaEventRecord(m->ev0, m->stream));
    for (int st = 0; st < steps; st++) {
        const int nb = (st + 1) * batch <= m->n ? batch : m->n - st * batch;
        int rc = train_launch(m, m->x, m->y, m->idx + (size_t)st * batch, nb, lr, m->loss + st, nullptr);
        if (rc) return rc;
    }
    MCK(cudaEventRecord(m->ev1, m->stream));
    std::vector<float> l(steps);
    MCK(cudaMemcpyAsync(l.data(), m->loss, steps * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, m->ev0, m->ev1);
    m->last_ms = ms;
    double s = 0.0;
    for (int st = 0; st < steps; st++) s += l[st];
    if (mean_loss) *mean_loss = (float)(s / ((double)m->n * OUT));
    return std::isfinite(s) ? HYB_OK : HYB_ERR_NONFINITE;
}

int hyb_mlp_grad(hyb_mlp *m, const float *x, const float *y, int n, float *grad, float *loss) {
    if (!m || !x || !y || !grad || n < 1) return HYB_ERR_INVALID;
    cudaSetDevice(m->dev);
    int rc = grow_staging(m, (size_t)n);
    if (rc) return rc;
    MCK(cudaMemcpyAsync(m->tx, x, (size_t)n * IN * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCK(cudaMemcpyAsync(m->ty, y, (size_t)n * OUT * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    if (m->loss_cap < 1) {
        MCK(cudaMalloc((void **)&m->loss, sizeof(float)));
        m->loss_cap = 1;
    }
    rc = train_launch(m, m->tx, m->ty, nullptr, n, 0.f, m->loss, m->grad);
    if (rc) return rc;
    float l = 0.f;
    MCK(cudaMemcpyAsync(grad, m->grad, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    if (loss) *loss = l / ((float)n * OUT);
    return HYB_OK;
}

int hyb_mlp_forward_dev(hyb_mlp *m, const float *x_dev, int n, float *y_dev, void *stream) {
    if (!m || !x_dev || !y_dev || n < 1) return HYB_ERR_INVALID;
    cudaStream_t s = stream ? (cudaStream_t)stream : m->stream;
    k_mlp_forward<<<(n + TILE - 1) / TILE, THREADS, sizeof(Smem), s>>>(m->wb, m->bias, m->nm, x_dev, n, y_dev);
    m->launches++;
    MCK(cudaGetLastError());
    return HYB_OK;
}

int hyb_mlp_predict(hyb_mlp *m, const float *x, int n, float *y) {
    if (!m || !x || !y || n < 1) return HYB_ERR_INVALID;
    cudaSetDevice(m->dev);
    int rc = grow_staging(m, (size_t)n);
    if (rc) return rc;
    MCK(cudaMemcpyAsync(m->tx, x, (size_t)n * IN * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCK(cudaEventRecord(m->ev0, m->stream));
    rc = hyb_mlp_forward_dev(m, m->tx, n, m->ty, nullptr);
    if (rc) return rc;
    MCK(cudaEventRecord(m->ev1, m->stream));
    MCK(cudaMemcpyAsync(y, m->ty, (size_t)n * OUT * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, m->ev0, m->ev1);
    m->last_ms = ms;
    return HYB_OK;
}

int hyb_mlp_last_ms(const hyb_mlp *m, double *ms) {
    if (!m || !ms) return HYB_ERR_INVALID;
    *ms = m->last_ms;
    return HYB_OK;
}

int hyb_mlp_launch_count(const hyb_mlp *m, long long *count) {
    if (!m || !count) return HYB_ERR_INVALID;
    *count = m->launches;
    return HYB_OK;
}

}  // extern "C"
