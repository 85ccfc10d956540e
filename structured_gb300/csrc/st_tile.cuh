// Tiled residual sweeps: the residual of EulerEquation::calc_residual
// (src/model/eulerequation.cpp:202-232) after the primitive and boundary
// passes, as one i-sweep and one j-sweep over tiles of cells.  Each CTA stages
// its tile of ghost-padded primitive records, with a two-cell halo along the
// sweep direction and one cell across it, in shared memory by one TMA tensor
// copy (cp.async.bulk.tensor, completion on an mbarrier), then computes the
// MUSCL slopes of the tile (and the halo cells the edge faces need), the face
// fluxes of the sweep direction, and the cells' flux differences, without
// global round trips of slopes or fluxes.
//
//   i-sweep: rhs = F_i(west) - F_i(east); SA face gradient parts of the
//            i-faces to Gi (the j-sweep's SA source reads them)
//   j-sweep: rhs = (F_j(south) - F_j(north)) + rhs, SA source, body force,
//            division by the volume (k_cell's arithmetic, same order)
//
// Face fluxes use face_flux (st_kernels.cuh), the per-face passes' code, so
// the two paths agree to round-off.  Only the FP64 value path without the
// fused network beta runs here; JVPs, the network-beta residual and callers
// that need the face arrays use the per-face passes.
#pragma once
#include <cuda.h>

#include "st_kernels.cuh"

namespace st {

constexpr int SW_THREADS = 256;
// tile extents (cells): i-sweep TI_I x TJ_I, j-sweep TI_J x TJ_J.  With 62 x 4
// every phase has at most 256 items (slopes 64 x 4, faces 63 x 4, cells 62 x 4),
// one per thread: no phase ends in a partly filled round while the FP64 pipe
// waits at the barrier, and the halo recompute is 3 % (slopes), 1.6 % (faces).
constexpr int TI_I = 62, TJ_I = 4, TI_J = 4, TJ_J = 62;
// staged boxes of primitive records: i-sweep rows i0-1 .. i0+TI_I+2 (padded),
// columns j0 .. j0+TJ_I+1; j-sweep rows i0 .. i0+TI_J+1, columns j0-1 .. j0+TJ_J+2
constexpr int BI_I = TI_I + 4, BJ_I = TJ_I + 2, BI_J = TI_J + 2, BJ_J = TJ_J + 4;
constexpr unsigned BOX_BYTES_I = BI_I * BJ_I * NP * 8, BOX_BYTES_J = BI_J * BJ_J * NP * 8;
// shared memory (doubles): box | slopes [cells][SL 5 | SR 5] | fluxes [faces][NQ] (| j: gradient parts [faces][4])
constexpr int SM_LIM_I = BI_I * BJ_I * NP, SM_F_I = SM_LIM_I + (TI_I + 2) * TJ_I * 10,
              SM_END_I = SM_F_I + (TI_I + 1) * TJ_I * 5;
constexpr int SM_LIM_J = BI_J * BJ_J * NP, SM_F_J = SM_LIM_J + TI_J * (TJ_J + 2) * 10,
              SM_G_J = SM_F_J + TI_J * (TJ_J + 1) * 5, SM_END_J = SM_G_J + TI_J * (TJ_J + 1) * 4;
// the mbarrier follows the arrays (8-byte aligned: the ends are whole doubles)
constexpr size_t SWEEP_SMEM_I = SM_END_I * 8 + 16, SWEEP_SMEM_J = SM_END_J * 8 + 16;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// Stage one box of primitive records: thread 0 initialises the mbarrier and
// issues the tensor copy; every thread waits on the barrier's phase 0 with a
// bounded number of polls.  Returns false if the copy did not complete within
// the bound, or (before any copy is issued) if the destination is not
// 128-byte aligned; the caller then marks its outputs non-finite and returns.
__device__ inline bool stage_box(const CUtensorMap* map, double* box, unsigned bytes, int c1, int c2,
                                 unsigned long long* mbar) {
    if (smem_u32(box) & 127u) return false;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
                     : "memory");
        // coordinates innermost first: record slot (always 0: 16-byte aligned), padded j, padded i
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
            ::"r"(smem_u32(box)), "l"(map), "r"(0), "r"(c1), "r"(c2), "r"(smem_u32(mbar))
            : "memory");
    }
    for (int it = 0; it < SPIN_LIMIT; it++) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(mbar))
            : "memory");
        if (done) return true;
    }
    return false;
}

// MUSCL slopes of one cell along one direction from its two neighbours
// (k_limiter's formulas): sl = phi (THM d- + THP d+), sr = phi (THP d- + THM d+)
template <int NQ>
__device__ __forceinline__ void muscl_slopes(const double* pm, const double* pc, const double* pp, double eps,
                                             double* out) {
    const int slot[5] = {P_RHO, P_U, P_V, P_P, P_NUT};
#pragma unroll
    for (int k = 0; k < NQ; k++) {
        const int m = slot[k];
        const double fa = pc[m] - pm[m], fb = pp[m] - pc[m];
        const double a1 = 3.0 * fb * fa;
        const double inv = frcp(2.0 * (fb - fa) * (fb - fa) + a1 + eps);
        const double ph = 0.25 * (a1 + eps) * inv;
        const double tl = THM * fa + THP * fb, tr = THP * fa + THM * fb;
        out[k] = ph * tl;
        out[5 + k] = ph * tr;
    }
}

// i-sweep.  Grid: (ceil(nic / TI_I), ceil(njc / TJ_I)).  Box record (a, b) is
// the padded primitive record (i0 - 1 + a, j0 + b).
template <int NQ, int ORDER>
__global__ void __launch_bounds__(SW_THREADS, 2)
    k_sweep_i(DevCase c, const __grid_constant__ CUtensorMap map, double* __restrict__ rhs, double* __restrict__ Gi) {
    extern __shared__ __align__(1024) double sm[];
    unsigned long long* mbar = reinterpret_cast<unsigned long long*>(sm + SM_END_I);
    const int nic = c.nic, njc = c.njc;
    const int i0 = blockIdx.x * TI_I, j0 = blockIdx.y * TJ_I;
    double* box = sm;
    double* limS = sm + SM_LIM_I;
    double* Fs = sm + SM_F_I;
    auto rec = [&](int a, int b) -> const double* { return box + (a * BJ_I + b) * NP; };
    if (!stage_box(&map, box, BOX_BYTES_I, j0, i0 - 1, mbar)) {
        for (int t = threadIdx.x; t < TI_I * TJ_I; t += SW_THREADS) {
            const int i = i0 + t / TJ_I, j = j0 + t % TJ_I;
            if (i < nic && j < njc)
                for (int k = 0; k < NQ; k++) rhs[((size_t)i * njc + j) * NQ + k] = __longlong_as_double(0x7ff8000000000000LL);
        }
        if (threadIdx.x == 0) atomicExch(c.err, 2);
        return;
    }
    // slopes of cells i0-1 .. i0+TI_I (those inside the grid)
    if (ORDER == 2) {
        for (int t = threadIdx.x; t < (TI_I + 2) * TJ_I; t += SW_THREADS) {
            const int r = t / TJ_I, b = t % TJ_I;
            const int i = i0 - 1 + r, j = j0 + b;
            if (i < 0 || i >= nic || j >= njc) continue;
            muscl_slopes<NQ>(rec(r, b + 1), rec(r + 1, b + 1), rec(r + 2, b + 1), c.eps_chi, limS + t * 10);
        }
        __syncthreads();
    }
    // i-faces f = i0 .. i0+TI_I: L = padded (f, j+1), R = (f+1, j+1), side pairs rows j+2 and j
    for (int t = threadIdx.x; t < (TI_I + 1) * TJ_I; t += SW_THREADS) {
        const int r = t / TJ_I, b = t % TJ_I;
        const int f = i0 + r, j = j0 + b;
        if (f > nic || j >= njc) continue;
        const double* sL = (ORDER == 2 && f >= 1) ? limS + (r * TJ_I + b) * 10 : nullptr;
        const double* sR = (ORDER == 2 && f <= nic - 1) ? limS + ((r + 1) * TJ_I + b) * 10 + 5 : nullptr;
        double fl[NQ], g[4];
        const size_t face = (size_t)f * njc + j;
        face_flux<double, NQ>(c, c.geo_i + face * NGEO, rec(r + 1, b + 1), rec(r + 2, b + 1), rec(r + 1, b + 2),
                              rec(r + 2, b + 2), rec(r + 1, b), rec(r + 2, b), sL, sR, fl, g);
#pragma unroll
        for (int k = 0; k < NQ; k++) Fs[t * NQ + k] = fl[k];
        if (NQ == 5 && c.viscous && (r < TI_I || f == nic)) {
            double* go = Gi + face * 4;
#pragma unroll
            for (int k = 0; k < 4; k++) go[k] = g[k];
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < TI_I * TJ_I; t += SW_THREADS) {
        const int r = t / TJ_I, b = t % TJ_I;
        const int i = i0 + r, j = j0 + b;
        if (i >= nic || j >= njc) continue;
        const double* fw = Fs + t * NQ;
        const double* fe = Fs + (t + TJ_I) * NQ;
        double* o = rhs + ((size_t)i * njc + j) * NQ;
#pragma unroll
        for (int k = 0; k < NQ; k++) o[k] = fw[k] - fe[k];
    }
}

// j-sweep.  Grid: (ceil(njc / TJ_J), ceil(nic / TI_J)).  Box record (a, b) is
// the padded primitive record (i0 + a, j0 - 1 + b).
template <int NQ, int ORDER>
__global__ void __launch_bounds__(SW_THREADS, 2)
    k_sweep_j(DevCase c, const __grid_constant__ CUtensorMap map, const double* __restrict__ Gi,
              const double* __restrict__ beta, double* __restrict__ rhs) {
    extern __shared__ __align__(1024) double sm[];
    unsigned long long* mbar = reinterpret_cast<unsigned long long*>(sm + SM_END_J);
    const int nic = c.nic, njc = c.njc;
    const int j0 = blockIdx.x * TJ_J, i0 = blockIdx.y * TI_J;
    constexpr int NS = TJ_J + 2, NF = TJ_J + 1;
    double* box = sm;
    double* limS = sm + SM_LIM_J;
    double* Fs = sm + SM_F_J;
    double* Gs = sm + SM_G_J;
    auto rec = [&](int a, int b) -> const double* { return box + (a * BJ_J + b) * NP; };
    if (!stage_box(&map, box, BOX_BYTES_J, j0 - 1, i0, mbar)) {
        for (int t = threadIdx.x; t < TI_J * TJ_J; t += SW_THREADS) {
            const int i = i0 + t / TJ_J, j = j0 + t % TJ_J;
            if (i < nic && j < njc)
                for (int k = 0; k < NQ; k++) rhs[((size_t)i * njc + j) * NQ + k] = __longlong_as_double(0x7ff8000000000000LL);
        }
        if (threadIdx.x == 0) atomicExch(c.err, 2);
        return;
    }
    // slopes of cells j0-1 .. j0+TJ_J in rows i0 .. i0+TI_J-1
    if (ORDER == 2) {
        for (int t = threadIdx.x; t < TI_J * NS; t += SW_THREADS) {
            const int r = t / NS, s = t % NS;
            const int i = i0 + r, j = j0 - 1 + s;
            if (i >= nic || j < 0 || j >= njc) continue;
            muscl_slopes<NQ>(rec(r + 1, s), rec(r + 1, s + 1), rec(r + 1, s + 2), c.eps_eta, limS + t * 10);
        }
        __syncthreads();
    }
    // j-faces g = j0 .. j0+TJ_J: L = padded (i+1, g), R = (i+1, g+1), side pairs columns i+2 and i
    for (int t = threadIdx.x; t < TI_J * NF; t += SW_THREADS) {
        const int r = t / NF, s = t % NF;
        const int i = i0 + r, g = j0 + s;
        if (i >= nic || g > njc) continue;
        const double* sL = (ORDER == 2 && g >= 1) ? limS + (r * NS + s) * 10 : nullptr;
        const double* sR = (ORDER == 2 && g <= njc - 1) ? limS + (r * NS + s + 1) * 10 + 5 : nullptr;
        double fl[NQ], gg[4];
        face_flux<double, NQ>(c, c.geo_j + ((size_t)i * c.nj + g) * NGEO, rec(r + 1, s + 1), rec(r + 1, s + 2),
                              rec(r + 2, s + 1), rec(r + 2, s + 2), rec(r, s + 1), rec(r, s + 2), sL, sR, fl, gg);
#pragma unroll
        for (int k = 0; k < NQ; k++) Fs[t * NQ + k] = fl[k];
        if (NQ == 5 && c.viscous)
#pragma unroll
            for (int k = 0; k < 4; k++) Gs[t * 4 + k] = gg[k];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < TI_J * TJ_J; t += SW_THREADS) {
        const int r = t / TJ_J, b = t % TJ_J;
        const int i = i0 + r, j = j0 + b;
        if (i >= nic || j >= njc) continue;
        const size_t idx = (size_t)i * njc + j;
        const double* fs = Fs + (r * NF + b) * NQ;
        const double* fn = fs + NQ;
        double* o = rhs + idx * NQ;
        double rr[NQ];
#pragma unroll
        for (int k = 0; k < NQ; k++) rr[k] = (fs[k] - fn[k]) + o[k];
        const double vol = c.vol[idx];
        if (NQ == 5 && c.viscous) {
            const double* gw = Gi + idx * 4;
            const double* ge = Gi + ((size_t)(i + 1) * njc + j) * 4;
            const double* gs = Gs + (r * NF + b) * 4;
            const double* gn = gs + 4;
            const double uy = 0.25 * (gw[0] + ge[0] + gs[0] + gn[0]);
            const double vx = 0.25 * (gw[1] + ge[1] + gs[1] + gn[1]);
            const double nx = 0.25 * (gw[2] + ge[2] + gs[2] + gn[2]);
            const double ny = 0.25 * (gw[3] + ge[3] + gs[3] + gn[3]);
            const double omega = ::fabs(vx - uy);
            const double* pc = rec(r + 1, b + 2);
            const double bta = beta ? beta[idx] : 1.0;
            const double src = sa_source(pc[P_RHO], pc[P_NUT], pc[P_MU], c.wd[idx], omega, nx * nx + ny * ny, bta);
            rr[NQ - 1] = rr[NQ - 1] + src * vol;
        }
        rr[1] = rr[1] + (-c.dpdx * vol);
        rr[2] = rr[2] + (-c.dpdy * vol);
        const double iv = c.ivol[idx];
#pragma unroll
        for (int k = 0; k < NQ; k++) o[k] = rr[k] * iv;
    }
}

}  // namespace st
