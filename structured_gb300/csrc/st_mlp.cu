// Learned SA correction (4-64-64-1 MLP): initialisation, training (Adam on
// BF16 tensor-core forward/backward passes with FP32 accumulation), feature
// export and beta export.  The inference used inside the residual is in
// st_mlp.cuh / k_cell.  There is no counterpart in the reference.
#include <cmath>
#include <cstring>
#include <vector>

#include "st_context.h"
#include "st_mlp.cuh"

using namespace st;
using stx::fail;
using stx::grid_for;

namespace {

constexpr int TRAIN_WARPS = 2;  // warps per training CTA (static shared memory)
// per-warp partial sums: dW1 [64][16] | dW2 [64][64] | db1 | db2 | dw3 | db3 | loss
constexpr int PT_W1 = 0, PT_W2 = PT_W1 + MLP_H * MLP_K1, PT_B1 = PT_W2 + MLP_H * MLP_H, PT_B2 = PT_B1 + MLP_H,
              PT_W3 = PT_B2 + MLP_H, PT_B3 = PT_W3 + MLP_H, PT_LOSS = PT_B3 + 1, PT_N = PT_LOSS + 1;

__host__ __device__ inline unsigned long long splitmix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// BF16 / FP32 inference blocks from the FP32 master parameters (one thread per
// master parameter; padded W1 columns stay zero from the initial memset)
__global__ void k_mlp_refresh(const float* __restrict__ m, __nv_bfloat16* __restrict__ wb, float* __restrict__ wf) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= MP_N) return;
    const float v = m[p];
    if (p < MP_B1) {
        const int o = (p - MP_W1) / MLP_IN, i = (p - MP_W1) % MLP_IN;
        wb[MLP_W1 + o * MLP_K1 + i] = __float2bfloat16_rn(v);
    } else if (p < MP_W2) {
        wf[MLP_B1 + p - MP_B1] = v;
    } else if (p < MP_B2) {
        const int o = (p - MP_W2) / MLP_H, i = (p - MP_W2) % MLP_H;
        wb[MLP_W2 + o * MLP_H + i] = __float2bfloat16_rn(v);
        wb[MLP_W2T + i * MLP_H + o] = __float2bfloat16_rn(v);
    } else if (p < MP_W3) {
        wf[MLP_B2 + p - MP_B2] = v;
    } else if (p < MP_B3) {
        wb[MLP_W3 + p - MP_W3] = __float2bfloat16_rn(v);
    } else {
        wf[MLP_B3] = v;
    }
}

// One training step's forward and backward passes, 32 samples per warp,
// samples drawn with replacement by a counter hash of (seed, step, slot).
// Loss (1/B) sum (beta - target)^2.  Writes the warp's partial gradients.
__global__ void __launch_bounds__(TRAIN_WARPS * 32)
    k_mlp_train(const float* __restrict__ feat, const float* __restrict__ target, long n, int batch,
                unsigned long long seed, int step, const __nv_bfloat16* __restrict__ wb, const float* __restrict__ wf,
                float* __restrict__ part) {
    __shared__ __nv_bfloat16 s_x[TRAIN_WARPS][MLP_SX], s_h1[TRAIN_WARPS][MLP_SH], s_h2[TRAIN_WARPS][MLP_SH];
    __shared__ __nv_bfloat16 s_d2[TRAIN_WARPS][MLP_SH], s_d1[TRAIN_WARPS][MLP_SH];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long warp_id = (long)blockIdx.x * TRAIN_WARPS + w;
    const long slot = warp_id * 32 + lane;
    const long s = (long)(splitmix64(seed ^ splitmix64((unsigned long long)step * (unsigned long long)batch + slot)) %
                          (unsigned long long)n);
    float x[MLP_IN];
#pragma unroll
    for (int k = 0; k < MLP_IN; k++) x[k] = feat[s * MLP_IN + k];
    mlp_normalise(wf, x);
    const float tg = target[s];
    __nv_bfloat16 *sx = s_x[w], *h1 = s_h1[w], *h2 = s_h2[w], *d2 = s_d2[w], *d1 = s_d1[w];
#pragma unroll
    for (int k = 0; k < MLP_K1; k++) sx[lane * MLP_K1 + k] = __float2bfloat16_rn(k < MLP_IN ? x[k] : 0.f);
    __syncwarp();
    mlp_layer_tanh<MLP_K1>(sx, wb + MLP_W1, MLP_K1, wf + MLP_B1, h1);
    mlp_layer_tanh<MLP_H>(h1, wb + MLP_W2, MLP_H, wf + MLP_B2, h2);
    float z = wf[MLP_B3];
    for (int k = 0; k < MLP_H; k++) z = fmaf(__bfloat162float(h2[lane * MLP_H + k]), __bfloat162float(wb[MLP_W3 + k]), z);
    const float y = softplus_f(z);
    const float err = y - tg;
    const float dy = (2.f / batch) * err / (1.f + expf(-z));
    // dZ2 = dy w3 (1 - h2^2), row of this lane
    for (int k = 0; k < MLP_H; k++) {
        const float hv = __bfloat162float(h2[lane * MLP_H + k]);
        d2[lane * MLP_H + k] = __float2bfloat16_rn(dy * __bfloat162float(wb[MLP_W3 + k]) * (1.f - hv * hv));
    }
    __syncwarp();
    float* pw = part + warp_id * PT_N;
    // small partials: column sums over the warp's 32 rows (lane owns columns lane, lane + 32)
    float dyr[32];
#pragma unroll
    for (int r = 0; r < 32; r++) dyr[r] = __shfl_sync(0xffffffffu, dy, r);
#pragma unroll
    for (int half = 0; half < 2; half++) {
        const int col = lane + 32 * half;
        float gw3 = 0.f, gb2 = 0.f;
#pragma unroll
        for (int r = 0; r < 32; r++) {
            gw3 = fmaf(dyr[r], __bfloat162float(h2[r * MLP_H + col]), gw3);
            gb2 += __bfloat162float(d2[r * MLP_H + col]);
        }
        pw[PT_W3 + col] = gw3;
        pw[PT_B2 + col] = gb2;
    }
    float sdy = dy, sl = err * err / batch;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sdy += __shfl_xor_sync(0xffffffffu, sdy, o);
        sl += __shfl_xor_sync(0xffffffffu, sl, o);
    }
    if (lane == 0) { pw[PT_B3] = sdy; pw[PT_LOSS] = sl; }
    // dH1 = dZ2 W2 (B(k, n) = W2[k][n]); dZ1 = dH1 (1 - h1^2)
    {
        float acc[2][8][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < 8; nt++)
#pragma unroll
                for (int e = 0; e < 4; e++) acc[mt][nt][e] = 0.f;
#pragma unroll
        for (int kt = 0; kt < MLP_H / 16; kt++) {
            unsigned a[2][4];
            frag_a(a[0], d2, 0, 16 * kt, MLP_H, 1);
            frag_a(a[1], d2, 16, 16 * kt, MLP_H, 1);
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                unsigned bb[2];
                frag_b(bb, wb + MLP_W2, 16 * kt, 8 * nt, MLP_H, 1);
                mma_bf16(acc[0][nt], a[0], bb);
                mma_bf16(acc[1][nt], a[1], bb);
            }
        }
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < 8; nt++)
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int r = 16 * mt + frag_c_row(e), cc = 8 * nt + frag_c_col(e);
                    const float hv = __bfloat162float(h1[r * MLP_H + cc]);
                    d1[r * MLP_H + cc] = __float2bfloat16_rn(acc[mt][nt][e] * (1.f - hv * hv));
                }
    }
    __syncwarp();
#pragma unroll
    for (int half = 0; half < 2; half++) {
        const int col = lane + 32 * half;
        float gb1 = 0.f;
#pragma unroll
        for (int r = 0; r < 32; r++) gb1 += __bfloat162float(d1[r * MLP_H + col]);
        pw[PT_B1 + col] = gb1;
    }
    // dW2 = dZ2^T H1: A(m, k) = d2[k][m], B(k, n) = h1[k][n]; K = the warp's 32 samples
#pragma unroll
    for (int mt = 0; mt < 4; mt++) {
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[nt][e] = 0.f;
#pragma unroll
        for (int kt = 0; kt < 2; kt++) {
            unsigned a[4];
            frag_a(a, d2, 16 * mt, 16 * kt, 1, MLP_H);
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                unsigned bb[2];
                frag_b(bb, h1, 16 * kt, 8 * nt, MLP_H, 1);
                mma_bf16(acc[nt], a, bb);
            }
        }
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++)
                pw[PT_W2 + (16 * mt + frag_c_row(e)) * MLP_H + 8 * nt + frag_c_col(e)] = acc[nt][e];
    }
    // dW1 = dZ1^T X: A(m, k) = d1[k][m], B(k, n) = sx[k][n]
#pragma unroll
    for (int mt = 0; mt < 4; mt++) {
        float acc[2][4];
#pragma unroll
        for (int nt = 0; nt < 2; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[nt][e] = 0.f;
#pragma unroll
        for (int kt = 0; kt < 2; kt++) {
            unsigned a[4];
            frag_a(a, d1, 16 * mt, 16 * kt, 1, MLP_H);
#pragma unroll
            for (int nt = 0; nt < 2; nt++) {
                unsigned bb[2];
                frag_b(bb, sx, 16 * kt, 8 * nt, MLP_K1, 1);
                mma_bf16(acc[nt], a, bb);
            }
        }
#pragma unroll
        for (int nt = 0; nt < 2; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++)
                pw[PT_W1 + (16 * mt + frag_c_row(e)) * MLP_K1 + 8 * nt + frag_c_col(e)] = acc[nt][e];
    }
}

// Fixed-order reduction of the warps' partial gradients and the Adam update
// of the FP32 master parameters (beta1 0.9, beta2 0.999, eps 1e-8), then the
// BF16 / FP32 inference blocks.  One thread per master parameter; thread MP_N
// sums the loss.
__global__ void k_mlp_adam(const float* __restrict__ part, int nwarps, float lr, int t, float* __restrict__ m,
                           float* __restrict__ am, float* __restrict__ av, __nv_bfloat16* __restrict__ wb,
                           float* __restrict__ wf, float* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > MP_N) return;
    int off;
    if (p == MP_N) off = PT_LOSS;
    else if (p < MP_B1) off = PT_W1 + ((p - MP_W1) / MLP_IN) * MLP_K1 + (p - MP_W1) % MLP_IN;
    else if (p < MP_W2) off = PT_B1 + p - MP_B1;
    else if (p < MP_B2) off = PT_W2 + p - MP_W2;
    else if (p < MP_W3) off = PT_B2 + p - MP_B2;
    else if (p < MP_B3) off = PT_W3 + p - MP_W3;
    else off = PT_B3;
    float g = 0.f;
    for (int w = 0; w < nwarps; w++) g += part[(size_t)w * PT_N + off];
    if (p == MP_N) { *loss = g; return; }
    const float b1 = 0.9f, b2 = 0.999f;
    const float mm = b1 * am[p] + (1.f - b1) * g;
    const float vv = b2 * av[p] + (1.f - b2) * g * g;
    am[p] = mm;
    av[p] = vv;
    const float mh = mm / (1.f - powf(b1, (float)t)), vh = vv / (1.f - powf(b2, (float)t));
    const float v = m[p] - lr * mh / (sqrtf(vh) + 1e-8f);
    m[p] = v;
    if (p < MP_B1) {
        wb[MLP_W1 + ((p - MP_W1) / MLP_IN) * MLP_K1 + (p - MP_W1) % MLP_IN] = __float2bfloat16_rn(v);
    } else if (p < MP_W2) {
        wf[MLP_B1 + p - MP_B1] = v;
    } else if (p < MP_B2) {
        const int o = (p - MP_W2) / MLP_H, i = (p - MP_W2) % MLP_H;
        wb[MLP_W2 + o * MLP_H + i] = __float2bfloat16_rn(v);
        wb[MLP_W2T + i * MLP_H + o] = __float2bfloat16_rn(v);
    } else if (p < MP_W3) {
        wf[MLP_B2 + p - MP_B2] = v;
    } else if (p < MP_B3) {
        wb[MLP_W3 + p - MP_W3] = __float2bfloat16_rn(v);
    } else {
        wf[MLP_B3] = v;
    }
}

// Fixed-order reduction of the warps' partial gradients into the master
// parameter layout (the same sums k_mlp_adam forms), without an update;
// thread MP_N writes the batch loss.
__global__ void k_mlp_grad_reduce(const float* __restrict__ part, int nwarps, float* __restrict__ grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > MP_N) return;
    int off;
    if (p == MP_N) off = PT_LOSS;
    else if (p < MP_B1) off = PT_W1 + ((p - MP_W1) / MLP_IN) * MLP_K1 + (p - MP_W1) % MLP_IN;
    else if (p < MP_W2) off = PT_B1 + p - MP_B1;
    else if (p < MP_B2) off = PT_W2 + p - MP_W2;
    else if (p < MP_W3) off = PT_B2 + p - MP_B2;
    else if (p < MP_B3) off = PT_W3 + p - MP_W3;
    else off = PT_B3;
    float g = 0.f;
    for (int w = 0; w < nwarps; w++) g += part[(size_t)w * PT_N + off];
    grad[p] = g;
}

// raw features of every cell (after a residual evaluation filled P and Gj)
__global__ void k_sa_features(DevCase c, const double* __restrict__ P, const double* __restrict__ Gj,
                              float* __restrict__ out) {
    const size_t n = (size_t)c.nic * c.njc;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        float f[MLP_IN];
        sa_features(c, P, Gj, (int)(idx / c.njc), (int)(idx % c.njc), f);
#pragma unroll
        for (int k = 0; k < MLP_IN; k++) out[idx * MLP_IN + k] = f[k];
    }
}

// beta of every cell from the network (whole-warp tiles)
__global__ void __launch_bounds__(256) k_mlp_beta(DevCase c, const double* __restrict__ P, const double* __restrict__ Gj,
                                                  double* __restrict__ beta) {
    __shared__ __nv_bfloat16 s_x[8 * MLP_SX], s_h[8 * MLP_SH];
    const size_t n = (size_t)c.nic * c.njc;
    const int w = threadIdx.x >> 5;
    for (size_t base = (size_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n;
         base += (size_t)gridDim.x * blockDim.x) {
        const size_t idx = base + (threadIdx.x & 31);
        float f[MLP_IN] = {0.f, 0.f, 0.f, 0.f};
        if (idx < n) {
            sa_features(c, P, Gj, (int)(idx / c.njc), (int)(idx % c.njc), f);
            mlp_normalise(c.mlp_wf, f);
        }
        const float b = mlp_warp_beta((const __nv_bfloat16*)c.mlp_wb, c.mlp_wf, f, s_x + w * MLP_SX, s_h + w * MLP_SH);
        if (idx < n) beta[idx] = (double)b;
    }
}

int ensure_mlp(st_ctx* x) {
    if (x->mlp_wb) return ST_OK;
    if (cudaMalloc(&x->mlp_wb, MLP_NBF * sizeof(__nv_bfloat16)) != cudaSuccess ||
        cudaMalloc((void**)&x->mlp_wf, MLP_NF * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void**)&x->mlp_master, 3 * MP_N * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void**)&x->mlp_loss, sizeof(float)) != cudaSuccess)
        return fail(ST_ERR_CUDA, "cudaMalloc (MLP parameters)");
    ST_CUDA(cudaMemsetAsync(x->mlp_wb, 0, MLP_NBF * sizeof(__nv_bfloat16), x->stream));
    std::vector<float> wf(MLP_NF, 0.f);
    for (int k = 0; k < MLP_IN; k++) wf[MLP_ISTD + k] = 1.f;
    ST_CUDA(cudaMemcpyAsync(x->mlp_wf, wf.data(), MLP_NF * sizeof(float), cudaMemcpyHostToDevice, x->stream));
    ST_CUDA(cudaMemsetAsync(x->mlp_master, 0, 3 * MP_N * sizeof(float), x->stream));
    return ST_OK;
}

int upload_master(st_ctx* x, const std::vector<float>& m) {
    ST_CUDA(cudaMemcpyAsync(x->mlp_master, m.data(), MP_N * sizeof(float), cudaMemcpyHostToDevice, x->stream));
    k_mlp_refresh<<<(MP_N + 255) / 256, 256, 0, x->stream>>>(x->mlp_master, (__nv_bfloat16*)x->mlp_wb, x->mlp_wf);
    ST_LAUNCH_CHECK("MLP refresh");
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

}  // namespace

extern "C" {

int st_mlp_param_count(void) { return MP_N; }

int st_mlp_init(st_ctx* x, unsigned long long seed) {
    if (!x) return fail(ST_ERR_ARG, "st_mlp_init: null context");
    int rc = ensure_mlp(x);
    if (rc) return rc;
    // Xavier (Glorot) uniform: U(-a, a), a = sqrt(6 / (fan_in + fan_out)); biases 0
    std::vector<float> m(MP_N, 0.f);
    unsigned long long st = seed;
    auto uni = [&]() { st = splitmix64(st); return (double)(st >> 11) * (1.0 / 9007199254740992.0); };
    const double a1 = std::sqrt(6.0 / (MLP_IN + MLP_H)), a2 = std::sqrt(6.0 / (2 * MLP_H)), a3 = std::sqrt(6.0 / (MLP_H + 1));
    for (int p = 0; p < MLP_H * MLP_IN; p++) m[MP_W1 + p] = (float)((2.0 * uni() - 1.0) * a1);
    for (int p = 0; p < MLP_H * MLP_H; p++) m[MP_W2 + p] = (float)((2.0 * uni() - 1.0) * a2);
    for (int p = 0; p < MLP_H; p++) m[MP_W3 + p] = (float)((2.0 * uni() - 1.0) * a3);
    ST_CUDA(cudaMemsetAsync(x->mlp_master + MP_N, 0, 2 * MP_N * sizeof(float), x->stream));  // Adam moments
    x->mlp_t = 0;
    return upload_master(x, m);
}

int st_mlp_set_params(st_ctx* x, const float* params) {
    if (!x || !params) return fail(ST_ERR_ARG, "st_mlp_set_params: null argument");
    int rc = ensure_mlp(x);
    if (rc) return rc;
    return upload_master(x, std::vector<float>(params, params + MP_N));
}

int st_mlp_get_params(st_ctx* x, float* params) {
    if (!x || !params) return fail(ST_ERR_ARG, "st_mlp_get_params: null argument");
    if (!x->mlp_wb) return fail(ST_ERR_ARG, "st_mlp_get_params: no network");
    ST_CUDA(cudaMemcpyAsync(params, x->mlp_master, MP_N * sizeof(float), cudaMemcpyDeviceToHost, x->stream));
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

int st_mlp_set_normalization(st_ctx* x, const float* mean, const float* stdev) {
    if (!x || !mean || !stdev) return fail(ST_ERR_ARG, "st_mlp_set_normalization: null argument");
    int rc = ensure_mlp(x);
    if (rc) return rc;
    float v[2 * MLP_IN];
    for (int k = 0; k < MLP_IN; k++) {
        if (!(stdev[k] > 0.f)) return fail(ST_ERR_ARG, "st_mlp_set_normalization: non-positive scale");
        v[k] = mean[k];
        v[MLP_IN + k] = 1.f / stdev[k];
    }
    ST_CUDA(cudaMemcpyAsync(x->mlp_wf + MLP_MEAN, v, sizeof(v), cudaMemcpyHostToDevice, x->stream));
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

int st_mlp_enable(st_ctx* x, int on) {
    if (!x) return fail(ST_ERR_ARG, "st_mlp_enable: null context");
    if (on && !x->mlp_wb) return fail(ST_ERR_ARG, "st_mlp_enable: no network");
    if (on && (x->nq != 5 || !x->dc.viscous))  // features read the viscous face gradients
        return fail(ST_ERR_UNSUPPORTED, "st_mlp_enable: needs the viscous SA model");
    x->dc.mlp_wb = on ? x->mlp_wb : nullptr;
    x->dc.mlp_wf = on ? x->mlp_wf : nullptr;
    return ST_OK;
}

int st_mlp_train(st_ctx* x, const float* feat_dev, const float* target_dev, long n, int steps, int batch, float lr,
                 unsigned long long seed, float* loss_host) {
    if (!x || !feat_dev || !target_dev) return fail(ST_ERR_ARG, "st_mlp_train: null argument");
    if (!x->mlp_wb) return fail(ST_ERR_ARG, "st_mlp_train: no network (st_mlp_init first)");
    if (n < 1 || steps < 0 || batch < 32 || batch % (32 * TRAIN_WARPS) != 0)
        return fail(ST_ERR_ARG, "st_mlp_train: n >= 1 and batch a multiple of 64");
    const int nwarps = batch / 32;
    const size_t need = (size_t)nwarps * PT_N;
    if (x->mlp_part_n < need) {
        if (x->mlp_part) cudaFree(x->mlp_part);
        x->mlp_part = nullptr;
        x->mlp_part_n = 0;
        if (cudaMalloc((void**)&x->mlp_part, need * sizeof(float)) != cudaSuccess)
            return fail(ST_ERR_CUDA, "cudaMalloc (MLP gradient partials)");
        x->mlp_part_n = need;
    }
    cudaStream_t s = x->stream;
    float* am = x->mlp_master + MP_N;
    float* av = x->mlp_master + 2 * MP_N;
    for (int it = 0; it < steps; it++) {
        k_mlp_train<<<nwarps / TRAIN_WARPS, TRAIN_WARPS * 32, 0, s>>>(feat_dev, target_dev, n, batch, seed, x->mlp_t,
                                                                      (const __nv_bfloat16*)x->mlp_wb, x->mlp_wf,
                                                                      x->mlp_part);
        x->mlp_t++;
        k_mlp_adam<<<(MP_N + 1 + 255) / 256, 256, 0, s>>>(x->mlp_part, nwarps, lr, x->mlp_t, x->mlp_master, am, av,
                                                         (__nv_bfloat16*)x->mlp_wb, x->mlp_wf, x->mlp_loss);
        if (loss_host) ST_CUDA(cudaMemcpyAsync(loss_host + it, x->mlp_loss, sizeof(float), cudaMemcpyDeviceToHost, s));
    }
    ST_LAUNCH_CHECK("MLP training");
    ST_CUDA(cudaStreamSynchronize(s));
    return ST_OK;
}

int st_mlp_grad(st_ctx* x, const float* feat_dev, const float* target_dev, long n, int batch,
                unsigned long long seed, int step, float* grad_host, float* loss_host) {
    if (!x || !feat_dev || !target_dev || !grad_host) return fail(ST_ERR_ARG, "st_mlp_grad: null argument");
    if (!x->mlp_wb) return fail(ST_ERR_ARG, "st_mlp_grad: no network (st_mlp_init first)");
    if (n < 1 || step < 0 || batch < 32 || batch % (32 * TRAIN_WARPS) != 0)
        return fail(ST_ERR_ARG, "st_mlp_grad: n >= 1, step >= 0 and batch a multiple of 64");
    const int nwarps = batch / 32;
    const size_t need = (size_t)nwarps * PT_N + MP_N + 1;  // partials, then the reduced gradient and loss
    if (x->mlp_part_n < need) {
        if (x->mlp_part) cudaFree(x->mlp_part);
        x->mlp_part = nullptr;
        x->mlp_part_n = 0;
        if (cudaMalloc((void**)&x->mlp_part, need * sizeof(float)) != cudaSuccess)
            return fail(ST_ERR_CUDA, "cudaMalloc (MLP gradient partials)");
        x->mlp_part_n = need;
    }
    cudaStream_t s = x->stream;
    float* g = x->mlp_part + (size_t)nwarps * PT_N;
    k_mlp_train<<<nwarps / TRAIN_WARPS, TRAIN_WARPS * 32, 0, s>>>(feat_dev, target_dev, n, batch, seed, step,
                                                                  (const __nv_bfloat16*)x->mlp_wb, x->mlp_wf,
                                                                  x->mlp_part);
    k_mlp_grad_reduce<<<(MP_N + 1 + 255) / 256, 256, 0, s>>>(x->mlp_part, nwarps, g);
    ST_LAUNCH_CHECK("MLP gradient");
    ST_CUDA(cudaMemcpyAsync(grad_host, g, MP_N * sizeof(float), cudaMemcpyDeviceToHost, s));
    if (loss_host) ST_CUDA(cudaMemcpyAsync(loss_host, g + MP_N, sizeof(float), cudaMemcpyDeviceToHost, s));
    ST_CUDA(cudaStreamSynchronize(s));
    return ST_OK;
}

int st_sa_features(st_ctx* x, float* feat_dev) {
    if (!x || !feat_dev) return fail(ST_ERR_ARG, "st_sa_features: null argument");
    if (x->nq != 5 || !x->dc.viscous) return fail(ST_ERR_UNSUPPORTED, "st_sa_features: needs the viscous SA model");
    int rc = stx::run_residual_faces(x, x->q, x->beta, x->rhs, x->c.order);
    if (rc) return rc;
    k_sa_features<<<grid_for(x->ncell), 256, 0, x->stream>>>(x->dc, x->P, x->Gj, feat_dev);
    ST_LAUNCH_CHECK("features");
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

int st_mlp_beta(st_ctx* x, double* beta_dev) {
    if (!x || !beta_dev) return fail(ST_ERR_ARG, "st_mlp_beta: null argument");
    if (!x->mlp_wb) return fail(ST_ERR_ARG, "st_mlp_beta: no network");
    if (x->nq != 5 || !x->dc.viscous) return fail(ST_ERR_UNSUPPORTED, "st_mlp_beta: needs the viscous SA model");
    int rc = stx::run_residual_faces(x, x->q, x->beta, x->rhs, x->c.order);
    if (rc) return rc;
    DevCase dc = x->dc;
    dc.mlp_wb = x->mlp_wb;
    dc.mlp_wf = x->mlp_wf;
    k_mlp_beta<<<grid_for(x->ncell), 256, 0, x->stream>>>(dc, x->P, x->Gj, beta_dev);
    ST_LAUNCH_CHECK("MLP beta");
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

}  // extern "C"
