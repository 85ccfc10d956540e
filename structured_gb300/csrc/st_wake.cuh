// Wake cut of the implicit solver's Jacobian: the column mask, the partner
// block pass and the partner products (st_solver.cu launches them).
//
// Self-contained apart from the C header's boundary types, so that the same
// source also compiles as plain C++ on a host (the qualifiers and the thread
// indices then come from the includer) for CPU checks of its index arithmetic.
#pragma once
#include <cstddef>

#include "../../include/structured_gb300.h"

namespace st {

// ---------------------------------------------------------------------------
// Wake cut (bc.cpp:224-263).  The bottom ghost below column a is a copy of
// cell (nic-1-a, 0); that ghost enters the residual rows (a-1, 0), (a, 0),
// (a+1, 0) and (a, 1), so each of those rows has one block outside the
// 13-point stencil.  Partner slot t of column i holds
//   W[i][t] = dR(i, wslot_j(t)) / dq(nic-1-(i-wslot_d(t)), 0).
// The regular blocks come from a colouring pass whose JVPs hold the wake
// ghosts' tangents at zero; the partners from a second pass that seeds the
// row-0 source cells of one half of the grid, columns congruent to k mod 3
// (their ghost windows, three columns wide, never share a row), and reads the
// rows next to their mirror ghosts on the other half, where the seeds have no
// local effect (the halves are at least WAKE_MIN_GAP columns apart).
// ---------------------------------------------------------------------------
constexpr int NWS = 4, WAKE_MIN_GAP = 6;
__host__ __device__ inline int wslot_j(int t) { return t == 3 ? 1 : 0; }
__host__ __device__ inline int wslot_d(int t) { return t == 3 ? 0 : t - 1; }
__host__ __device__ inline int wake_side(int i, int nic) { return 2 * i > nic - 1 ? 1 : 0; }

// Columns whose bottom ghost is a wake copy, for the boundary list in order:
// each bottom wake range, padded start..end, marks columns start-1..end-1 and
// their mirrors nic-end..nic-start.  Returns 0, or ST_ERR_UNSUPPORTED with
// *why set for the lists this layout cannot hold (periodic boundaries, a cut
// off the bottom face or on a corner ghost, halves closer than WAKE_MIN_GAP
// columns, a single row of cells).  *any = 1 if a cut was found.
inline int wake_columns(int nic, int njc, const st_bc* bcs, int nbc, int* mask, int* any, const char** why) {
    *any = 0;
    for (int i = 0; i < nic; i++) mask[i] = 0;
    for (int n = 0; n < nbc; n++) {
        const st_bc& b = bcs[n];
        if (b.type == ST_BC_PERIODIC) { *why = "periodic boundaries couple distant cells"; return ST_ERR_UNSUPPORTED; }
        if (b.type != ST_BC_WAKE) continue;
        if (b.face != ST_FACE_BOTTOM) { *why = "wake cut off the bottom face"; return ST_ERR_UNSUPPORTED; }
        const int end = b.end >= 0 ? b.end : nic + 2 + b.end;
        if (b.start > end) continue;
        if (b.start < 1 || end > nic) { *why = "wake range on a corner ghost"; return ST_ERR_UNSUPPORTED; }
        for (int ip = b.start; ip <= end; ip++) {
            mask[ip - 1] = 1;
            mask[nic - ip] = 1;
        }
        *any = 1;
    }
    if (!*any) return 0;
    int max_left = -1, min_right = nic;
    for (int i = 0; i < nic; i++)
        if (mask[i]) {
            if (wake_side(i, nic)) { if (i < min_right) min_right = i; }
            else if (i > max_left) max_left = i;
        }
    if (njc < 2 || max_left < 0 || min_right >= nic || min_right - max_left < WAKE_MIN_GAP) {
        *why = "the wake cut's halves are too close";
        return ST_ERR_UNSUPPORTED;
    }
    return 0;
}

template <int NQ>
__global__ void k_wake_seed(int nic, int njc, const int* __restrict__ wmask, int side, int k, int comp,
                            double* __restrict__ v) {
    const size_t n = (size_t)nic * njc;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / njc), j = (int)(idx % njc);
        const bool on = j == 0 && wmask[i] && wake_side(i, nic) == side && i % 3 == k;
#pragma unroll
        for (int kk = 0; kk < NQ; kk++) v[idx * NQ + kk] = (on && kk == comp) ? 1.0 : 0.0;
    }
}

template <int NQ>
__global__ void k_wake_extract(int nic, int njc, const int* __restrict__ wmask, int side, int k, int comp,
                               const double* __restrict__ jv, double* __restrict__ W) {
    const int n = nic * NWS;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int i = t / NWS, slot = t % NWS;
        const int a = i - wslot_d(slot);
        if (a < 0 || a >= nic || !wmask[a]) continue;
        const int src = nic - 1 - a;
        if (wake_side(src, nic) != side || src % 3 != k) continue;
        const size_t row = (size_t)i * njc + wslot_j(slot);
        double* b = W + (size_t)t * NQ * NQ;
#pragma unroll
        for (int kk = 0; kk < NQ; kk++) b[kk * NQ + comp] = jv[row * NQ + kk];
    }
}

// acc += b x (TRANS: b^T x) for one nq x nq block
template <int NQ, bool TRANS>
__device__ inline void block_mv(const double* __restrict__ b, const double* __restrict__ x, double* acc) {
#pragma unroll
    for (int kk = 0; kk < NQ; kk++)
#pragma unroll
        for (int l = 0; l < NQ; l++) acc[kk] += (TRANS ? b[l * NQ + kk] : b[kk * NQ + l]) * x[l];
}

// y += sj * W x (or W^T x): one thread per column, after k_spmv on the same stream
template <int NQ, bool TRANS>
__global__ void k_wake_apply(int nic, int njc, const double* __restrict__ W, const double* __restrict__ x,
                             double* __restrict__ y, double sj) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nic; i += gridDim.x * blockDim.x) {
        double* y0 = y + (size_t)i * njc * NQ;  // cell (i, 0); cell (i, 1) follows
        if (!TRANS) {
            double a0[NQ], a1[NQ];
#pragma unroll
            for (int kk = 0; kk < NQ; kk++) { a0[kk] = 0.0; a1[kk] = 0.0; }
#pragma unroll
            for (int slot = 0; slot < NWS; slot++) {
                const int a = i - wslot_d(slot);
                if (a < 0 || a >= nic) continue;
                const double* b = W + ((size_t)i * NWS + slot) * NQ * NQ;
                const double* xc = x + (size_t)(nic - 1 - a) * njc * NQ;  // cell (nic-1-a, 0)
                if (wslot_j(slot)) block_mv<NQ, false>(b, xc, a1);
                else block_mv<NQ, false>(b, xc, a0);
            }
#pragma unroll
            for (int kk = 0; kk < NQ; kk++) { y0[kk] += sj * a0[kk]; y0[NQ + kk] += sj * a1[kk]; }
        } else {
            // cell (i, 0) is the source of the ghost below column a = nic-1-i
            const int a = nic - 1 - i;
            double acc[NQ];
#pragma unroll
            for (int kk = 0; kk < NQ; kk++) acc[kk] = 0.0;
#pragma unroll
            for (int slot = 0; slot < NWS; slot++) {
                const int r = a + wslot_d(slot);
                if (r < 0 || r >= nic) continue;
                block_mv<NQ, true>(W + ((size_t)r * NWS + slot) * NQ * NQ,
                                   x + ((size_t)r * njc + wslot_j(slot)) * NQ, acc);
            }
#pragma unroll
            for (int kk = 0; kk < NQ; kk++) y0[kk] += sj * acc[kk];
        }
    }
}

}  // namespace st
