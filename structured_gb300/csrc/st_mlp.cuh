// Learned SA correction: features of a cell and the 4-64-64-1 MLP that maps
// them to the production multiplier beta, evaluated 32 cells per warp with
// BF16 tensor-core MMAs (mma.sync m16n8k16, FP32 accumulation).  There is no
// counterpart in the reference.
//
// Network: h1 = tanh(W1 x + b1), h2 = tanh(W2 h1 + b2), beta = softplus(w3.h2 + b3),
// x = (f - mean) / std of the four features
//   f0 = P / (P + D)           SA production over production + destruction (beta = 1)
//   f1 = chi = rho nu~ / mu
//   f2 = log10(max(d u_tau rho / mu, 1e-2)),  u_tau from the wall shear of the cell's column
//   f3 = min(|S| / |Omega|, 10) from the cell's Green-Gauss velocity gradient
// Weights are BF16 (W1 [64][16] with inputs padded to 16, W2 [64][64], its
// transpose for the backward pass, w3 [64]); biases and normalisation FP32.
#pragma once
#include <cuda_bf16.h>

#include "st_common.cuh"

namespace st {

constexpr int MLP_IN = 4, MLP_K1 = 16, MLP_H = 64;
// BF16 block: W1 | W2 | W2^T | w3 ; FP32 block: b1 | b2 | b3 | mean | inv_std
constexpr int MLP_W1 = 0, MLP_W2 = MLP_W1 + MLP_H * MLP_K1, MLP_W2T = MLP_W2 + MLP_H * MLP_H,
              MLP_W3 = MLP_W2T + MLP_H * MLP_H, MLP_NBF = MLP_W3 + MLP_H;
constexpr int MLP_B1 = 0, MLP_B2 = MLP_H, MLP_B3 = 2 * MLP_H, MLP_MEAN = MLP_B3 + 1, MLP_ISTD = MLP_MEAN + MLP_IN,
              MLP_NF = MLP_ISTD + MLP_IN;
// FP32 master parameters (training): W1 [64][4] | b1 | W2 [64][64] | b2 | w3 | b3
constexpr int MP_W1 = 0, MP_B1 = MP_W1 + MLP_H * MLP_IN, MP_W2 = MP_B1 + MLP_H, MP_B2 = MP_W2 + MLP_H * MLP_H,
              MP_W3 = MP_B2 + MLP_H, MP_B3 = MP_W3 + MLP_H, MP_N = MP_B3 + 1;

// shared-memory staging per warp: 32 x 16 inputs and 32 x 64 activations (BF16)
constexpr int MLP_SX = 32 * MLP_K1, MLP_SH = 32 * MLP_H;

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
    __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<unsigned*>(&p);
}
__device__ __forceinline__ unsigned pair_at(const __nv_bfloat16* base, int r, int c, int ldr, int ldc) {
    __nv_bfloat162 p;
    p.x = base[r * ldr + c * ldc];
    p.y = base[r * ldr + (c + 1) * ldc];
    return *reinterpret_cast<unsigned*>(&p);
}
// A fragment of the 16x16 tile at (m0, k0) of A(m, k) = base[m * ldm + k * ldk]
__device__ __forceinline__ void frag_a(unsigned a[4], const __nv_bfloat16* base, int m0, int k0, int ldm, int ldk) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    a[0] = pair_at(base, m0 + g, k0 + 2 * t, ldm, ldk);
    a[1] = pair_at(base, m0 + g + 8, k0 + 2 * t, ldm, ldk);
    a[2] = pair_at(base, m0 + g, k0 + 2 * t + 8, ldm, ldk);
    a[3] = pair_at(base, m0 + g + 8, k0 + 2 * t + 8, ldm, ldk);
}
// B fragment of the 16x8 tile at (k0, n0) of B(k, n) = base[k * ldk + n * ldn]
__device__ __forceinline__ void frag_b(unsigned b[2], const __nv_bfloat16* base, int k0, int n0, int ldk, int ldn) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    __nv_bfloat162 p, q;
    p.x = base[(k0 + 2 * t) * ldk + (n0 + g) * ldn];
    p.y = base[(k0 + 2 * t + 1) * ldk + (n0 + g) * ldn];
    q.x = base[(k0 + 2 * t + 8) * ldk + (n0 + g) * ldn];
    q.y = base[(k0 + 2 * t + 9) * ldk + (n0 + g) * ldn];
    b[0] = *reinterpret_cast<unsigned*>(&p);
    b[1] = *reinterpret_cast<unsigned*>(&q);
}
__device__ __forceinline__ void mma_bf16(float c[4], const unsigned a[4], const unsigned b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
// C fragment element e (0..3) of a 16x8 tile: row and column within the tile
__device__ __forceinline__ int frag_c_row(int e) { return ((threadIdx.x & 31) >> 2) + (e >= 2 ? 8 : 0); }
__device__ __forceinline__ int frag_c_col(int e) { return 2 * (threadIdx.x & 3) + (e & 1); }

__device__ __forceinline__ float softplus_f(float z) { return z > 20.f ? z : log1pf(expf(z)); }

// One dense layer on a warp's 32 rows: out(32 x 64) = act(in(32 x K) W^T + b),
// in from shared memory (row-major, ld K), W (BF16) as [64][ldw] rows.  The
// tanh activations are written to `out` (BF16, row-major 32 x 64).
template <int K>
__device__ __forceinline__ void mlp_layer_tanh(const __nv_bfloat16* in, const __nv_bfloat16* W, int ldw,
                                               const float* b, __nv_bfloat16* out, float* keep = nullptr) {
    float acc[2][8][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[mt][nt][e] = b[8 * nt + frag_c_col(e)];
#pragma unroll
    for (int kt = 0; kt < K / 16; kt++) {
        unsigned a[2][4];
        frag_a(a[0], in, 0, 16 * kt, K, 1);
        frag_a(a[1], in, 16, 16 * kt, K, 1);
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            unsigned bb[2];
            frag_b(bb, W, 16 * kt, 8 * nt, 1, ldw);  // B(k, n) = W[n][k]
            mma_bf16(acc[0][nt], a[0], bb);
            mma_bf16(acc[1][nt], a[1], bb);
        }
    }
    __syncwarp();  // every lane has read `in` (out may alias it)
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int r = 16 * mt + frag_c_row(e), cc = 8 * nt + frag_c_col(e);
                const float h = tanhf(acc[mt][nt][e]);
                out[r * MLP_H + cc] = __float2bfloat16_rn(h);
                if (keep) keep[r * MLP_H + cc] = h;
            }
    __syncwarp();
}

// beta of the warp's 32 cells; x holds this lane's normalised features.
// sx, sh: this warp's staging buffers.  All 32 lanes must call it.
__device__ __forceinline__ float mlp_warp_beta(const __nv_bfloat16* wb, const float* wf, const float x[MLP_IN],
                                               __nv_bfloat16* sx, __nv_bfloat16* sh) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < MLP_K1; k++) sx[lane * MLP_K1 + k] = __float2bfloat16_rn(k < MLP_IN ? x[k] : 0.f);
    __syncwarp();
    mlp_layer_tanh<MLP_K1>(sx, wb + MLP_W1, MLP_K1, wf + MLP_B1, sh);
    mlp_layer_tanh<MLP_H>(sh, wb + MLP_W2, MLP_H, wf + MLP_B2, sh);
    float z = wf[MLP_B3];
#pragma unroll 8
    for (int k = 0; k < MLP_H; k++) z = fmaf(__bfloat162float(sh[lane * MLP_H + k]), __bfloat162float(wb[MLP_W3 + k]), z);
    __syncwarp();
    return softplus_f(z);
}

// ---------------------------------------------------------------------------
// features of cell (i, j) from the ghost-padded primitives P (after the BCs)
// and the j-face gradient records Gj (the residual's face pass: dudy, dvdx at
// the wall face of the column).  SA terms as in sa_source with beta = 1.
// ---------------------------------------------------------------------------
__device__ inline void sa_pd(double rho, double nut, double mu, double d, double omega, double* P, double* D) {
    if (nut <= 0.0) { *P = 0.0; *D = 0.0; return; }
    const double k2d2 = SA_KAPPA * SA_KAPPA * d * d;
    const double chi = rho * nut / mu, chi3 = chi * chi * chi;
    const double fv1 = chi3 / (chi3 + SA_CV1_3);
    const double fv2 = 1.0 - chi / (1.0 + chi * fv1);
    const double sbar = nut * fv2 / k2d2;
    double stilde;
    if (sbar >= -SA_CV2 * omega) stilde = omega + sbar;
    else stilde = omega + omega * (SA_CV2 * SA_CV2 * omega + SA_CV3 * sbar) / ((SA_CV3 - 2.0 * SA_CV2) * omega - sbar);
    double r = 10.0;
    if (stilde > 0.0) r = fmin(nut / (stilde * k2d2), 10.0);
    const double r2 = r * r;
    const double gg = r + SA_CW2 * (r2 * r2 * r2 - r);
    const double g2 = gg * gg;
    const double fw = gg * ::cbrt(::sqrt((1.0 + SA_CW3_6) / (g2 * g2 * g2 + SA_CW3_6)));
    *P = SA_CB1 * stilde * nut;
    *D = SA_CW1 * fw * nut * nut / (d * d);
}

// (values only for dual-number records: beta is lagged in Jacobian products)
template <class T>
__device__ inline void sa_features(const DevCase& c, const T* P, const T* Gj, int i, int j, float f[MLP_IN]) {
    const T* pc = P + pidx(c, i + 1, j + 1);
    const T* pw = P + pidx(c, i, j + 1);
    const T* pe = P + pidx(c, i + 2, j + 1);
    const T* ps = P + pidx(c, i + 1, j);
    const T* pn = P + pidx(c, i + 1, j + 2);
    // Green-Gauss cell gradient of u, v with face averages (normals of the metric arrays)
    const double* nW = c.nchi + ((size_t)i * c.njc + j) * 2;
    const double* nE = c.nchi + ((size_t)(i + 1) * c.njc + j) * 2;
    const double* nS = c.neta + ((size_t)i * c.nj + j) * 2;
    const double* nN = c.neta + ((size_t)i * c.nj + j + 1) * 2;
    const double iv = c.ivol[(size_t)i * c.njc + j];
    double g[2][2];
#pragma unroll
    for (int m = 0; m < 2; m++) {
        const int s = m == 0 ? P_U : P_V;
        const double fe = 0.5 * (val(pc[s]) + val(pe[s])), fw = 0.5 * (val(pc[s]) + val(pw[s]));
        const double fn = 0.5 * (val(pc[s]) + val(pn[s])), fs = 0.5 * (val(pc[s]) + val(ps[s]));
        g[m][0] = iv * (fe * nE[0] - fw * nW[0] + fn * nN[0] - fs * nS[0]);
        g[m][1] = iv * (fe * nE[1] - fw * nW[1] + fn * nN[1] - fs * nS[1]);
    }
    const double sxy = 0.5 * (g[0][1] + g[1][0]);
    const double smag = ::sqrt(2.0 * (g[0][0] * g[0][0] + g[1][1] * g[1][1] + 2.0 * sxy * sxy));
    const double wmag = ::fabs(g[1][0] - g[0][1]);
    const double rho = val(pc[P_RHO]), nut = val(pc[P_NUT]), mu = val(pc[P_MU]);
    const double d = c.wd[(size_t)i * c.njc + j];
    double Pp, Dd;
    sa_pd(rho, nut, mu, d, wmag, &Pp, &Dd);
    const T* gw = Gj + ((size_t)i * c.nj) * 4;  // wall face (i, 0)
    const double rho_w = val(P[pidx(c, i + 1, 1) + P_RHO]);
    const double utau = ::sqrt(c.mu_inf * ::fabs(val(gw[0]) - val(gw[1])) / rho_w);
    f[0] = (float)(Pp + Dd > 0.0 ? Pp / (Pp + Dd) : 0.0);
    f[1] = (float)(rho * nut / mu);
    f[2] = (float)::log10(fmax(d * utau * rho / mu, 1e-2));
    f[3] = (float)fmin(smag / (wmag + 1e-300), 10.0);
}

__device__ __forceinline__ void mlp_normalise(const float* wf, float f[MLP_IN]) {
#pragma unroll
    for (int k = 0; k < MLP_IN; k++) f[k] = (f[k] - wf[MLP_MEAN + k]) * wf[MLP_ISTD + k];
}

}  // namespace st
