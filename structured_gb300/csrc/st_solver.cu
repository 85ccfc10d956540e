// Implicit pseudo-time Newton solve and the adjoint linear solve on the GPU.
//
// Replaces the reference's implicit step (Solver::step, src/solver/solver.cpp:
// 69-101 and 153-183): the ADOL-C tape + sparse_jac Jacobian becomes a block
// Jacobian (13-point stencil, nq x nq blocks) assembled from exact
// forward-mode JVPs over a 5x5 cell colouring, and the library LU solves
// (ls_eigen.cpp / ls_arma.cpp / ls_petsc.cpp) become restarted GMRES with a
// block ILU(0) preconditioner of the first-order Jacobian in natural cell
// order, level-scheduled in one cooperative kernel.  The pseudo-time driver keeps the reference's
// CFL / under-relaxation ramps (solver.cpp:198-236) and adds the tolerance exit
// the reference has disabled (solver.cpp:145) plus a divergence guard.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "st_adjoint.cuh"
#include "st_context.h"
#include "st_partner.cuh"

using namespace st;
using stx::fail;
using stx::grid_for;

namespace {

constexpr int NOFF = 13;
constexpr int STRIP_MAX = 1024;  // largest wake strip (unknowns) given a dense inverse
// stencil offsets (di, dj) of the block Jacobian row; 0 is the diagonal block
__constant__ int c_di[NOFF] = {0, -1, 1, 0, 0, -2, 2, 0, 0, -1, -1, 1, 1};
__constant__ int c_dj[NOFF] = {0, 0, 0, -1, 1, 0, 0, -2, 2, -1, 1, -1, 1};
constexpr int O_JM = 3, O_JP = 4;  // (0,-1), (0,+1)

__device__ inline int off_index(int di, int dj) {
#pragma unroll
    for (int o = 0; o < NOFF; o++)
        if (c_di[o] == di && c_dj[o] == dj) return o;
    return -1;
}

// seed vector of one colour class (cells with i mod cs, j mod cs = ci, cj)
// and one component
template <int NQ>
__global__ void k_seed(int nic, int njc, int cs, int ci, int cj, int comp, double* v) {
    const size_t n = (size_t)nic * njc;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / njc), j = (int)(idx % njc);
        const bool on = (i % cs == ci) && (j % cs == cj);
#pragma unroll
        for (int k = 0; k < NQ; k++) v[idx * NQ + k] = (on && k == comp) ? 1.0 : 0.0;
    }
}

// Row r's JVP with the colour seed is column `comp` of the block J(r, c) for
// the single seeded cell c in r's stencil (colours cs apart never share a row:
// cs = 5 covers the 13-point second-order stencil, cs = 3 the 9-point
// first-order one).
template <int NQ>
__global__ void k_extract(int nic, int njc, int cs, int ci, int cj, int comp, const double* __restrict__ jv,
                          double* __restrict__ jac) {
    const size_t n = (size_t)nic * njc;
    const int half = cs / 2;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / njc), j = (int)(idx % njc);
        int mi = ((ci - i) % cs + cs) % cs, mj = ((cj - j) % cs + cs) % cs;
        const int di = mi > half ? mi - cs : mi, dj = mj > half ? mj - cs : mj;
        const int o = off_index(di, dj);
        if (o < 0) continue;
        const int ic = i + di, jc = j + dj;
        if (ic < 0 || ic >= nic || jc < 0 || jc >= njc) continue;
        double* b = jac + ((idx * NOFF + o) * NQ) * NQ;
#pragma unroll
        for (int k = 0; k < NQ; k++) b[k * NQ + comp] = jv[idx * NQ + k];
    }
}

// y = sd * D x + sj * J x   (or with J^T when TRANS), D = diag(1/dt)
template <int NQ, bool TRANS>
__global__ void __launch_bounds__(256) k_spmv(int nic, int njc, const double* __restrict__ jac,
                                              const double* __restrict__ x, double* __restrict__ y,
                                              const double* __restrict__ dt, double sd, double sj) {
    const size_t n = (size_t)nic * njc;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / njc), j = (int)(idx % njc);
        double acc[NQ];
#pragma unroll
        for (int k = 0; k < NQ; k++) acc[k] = 0.0;
        for (int o = 0; o < NOFF; o++) {
            if (!TRANS) {
                const int ic = i + c_di[o], jc = j + c_dj[o];
                if (ic < 0 || ic >= nic || jc < 0 || jc >= njc) continue;
                const double* b = jac + ((idx * NOFF + o) * NQ) * NQ;
                const double* xc = x + ((size_t)ic * njc + jc) * NQ;
#pragma unroll
                for (int k = 0; k < NQ; k++)
#pragma unroll
                    for (int l = 0; l < NQ; l++) acc[k] += b[k * NQ + l] * xc[l];
            } else {
                const int ir = i - c_di[o], jr = j - c_dj[o];
                if (ir < 0 || ir >= nic || jr < 0 || jr >= njc) continue;
                const size_t r = (size_t)ir * njc + jr;
                const double* b = jac + ((r * NOFF + o) * NQ) * NQ;
                const double* xr = x + r * NQ;
#pragma unroll
                for (int k = 0; k < NQ; k++)
#pragma unroll
                    for (int l = 0; l < NQ; l++) acc[k] += b[l * NQ + k] * xr[l];
            }
        }
#pragma unroll
        for (int k = 0; k < NQ; k++) {
            double v = sj * acc[k];
            if (dt) v += sd * x[idx * NQ + k] / dt[idx * NQ + k];
            y[idx * NQ + k] = v;
        }
    }
}

// NQ x NQ helpers (row-major, registers)
template <int NQ>
__device__ inline void load_block(const double* __restrict__ jac, size_t cell, int o, bool tr, double s, double* m) {
    const double* b = jac + ((cell * NOFF + o) * NQ) * NQ;
#pragma unroll
    for (int k = 0; k < NQ; k++)
#pragma unroll
        for (int l = 0; l < NQ; l++) m[k * NQ + l] = s * (tr ? b[l * NQ + k] : b[k * NQ + l]);
}

// inverse by Gauss-Jordan elimination with partial pivoting; returns false if singular
template <int NQ>
__device__ inline bool invert(const double* a_in, double* inv) {
    double a[NQ * NQ];
#pragma unroll
    for (int t = 0; t < NQ * NQ; t++) { a[t] = a_in[t]; inv[t] = 0.0; }
#pragma unroll
    for (int k = 0; k < NQ; k++) inv[k * NQ + k] = 1.0;
    for (int c = 0; c < NQ; c++) {
        int p = c;
        double best = fabs(a[c * NQ + c]);
        for (int r = c + 1; r < NQ; r++)
            if (fabs(a[r * NQ + c]) > best) { best = fabs(a[r * NQ + c]); p = r; }
        if (!(best > 0.0)) return false;
        if (p != c)
            for (int t = 0; t < NQ; t++) {
                double u = a[c * NQ + t]; a[c * NQ + t] = a[p * NQ + t]; a[p * NQ + t] = u;
                u = inv[c * NQ + t]; inv[c * NQ + t] = inv[p * NQ + t]; inv[p * NQ + t] = u;
            }
        const double d = 1.0 / a[c * NQ + c];
        for (int t = 0; t < NQ; t++) { a[c * NQ + t] *= d; inv[c * NQ + t] *= d; }
        for (int r = 0; r < NQ; r++) {
            if (r == c) continue;
            const double f = a[r * NQ + c];
            if (f == 0.0) continue;
            for (int t = 0; t < NQ; t++) { a[r * NQ + t] -= f * a[c * NQ + t]; inv[r * NQ + t] -= f * inv[c * NQ + t]; }
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// Block ILU(0) preconditioner, natural (i-major) cell order, on the
// first-order Jacobian's 9-point stencil: M = psd D + sj J1 = L U with L unit
// lower.  Row (i,j) depends on rows (i-1,j-1), (i-1,j), (i-1,j+1), (i,j-1),
// so the rows of level 2i+j are independent.  Natural order keeps the
// downstream ordering of the convective coupling; multicolour orderings of
// the same factorisation needed 10x more Krylov iterations on the CPU.
//
// Layout and execution, built around GB300's FP64 rate (1/64 of FP32):
//  * factors and their arithmetic are FP32 ([cell][9][nq][nq]: D^-1, four L
//    blocks, four U blocks).  The preconditioner only approximates J; the
//    Jacobian, residual and Krylov vectors stay FP64, and flexible GMRES keeps
//    the preconditioned basis, so FP32 rounding in M^-1 does not limit the
//    attainable FP64 residual;
//  * one thread-block cluster of ILU_CL CTAs walks the levels, separated by
//    the hardware cluster barrier (all CTAs of a cluster are co-scheduled, so
//    no software spin is involved);
//  * a row is handled by 8 lanes, lane k owning block row k (k < nq): block
//    products are row-parallel and the pivoting 5x5 inversion exchanges rows
//    by warp shuffles.  Values written at earlier levels are read with
//    ld.global.cg (L2, coherent across the cluster's SMs).
// ---------------------------------------------------------------------------
constexpr int ILU_CL = 8;        // CTAs per cluster (portable maximum)
constexpr int ILU_THREADS = 512;
constexpr int ILU_NB = 9;        // blocks per row: 0 D^-1, 1..4 L, 5..8 U
// lower neighbours in elimination (column) order: (-1,-1) (-1,0) (-1,1) (0,-1);
// upper neighbours: (0,1) (1,-1) (1,0) (1,1)
__host__ __device__ constexpr int ldi(int a) { return a == 3 ? 0 : -1; }
__host__ __device__ constexpr int ldj(int a) { return a == 0 ? -1 : a == 1 ? 0 : a == 2 ? 1 : -1; }
__host__ __device__ constexpr int udi(int b) { return b == 0 ? 0 : 1; }
__host__ __device__ constexpr int udj(int b) { return b == 0 ? 1 : b == 1 ? -1 : b == 2 ? 0 : 1; }

__device__ inline int n_levels(int nic, int njc) { return 2 * (nic - 1) + (njc - 1) + 1; }
__device__ inline void level_range(int L, int nic, int njc, int& i_lo, int& cnt) {
    const int t = L - (njc - 1);
    i_lo = t > 0 ? (t + 1) / 2 : 0;
    const int i_hi = min(nic - 1, L / 2);
    cnt = i_hi - i_lo + 1;
}

__device__ __forceinline__ void cluster_barrier() {
    // non-.aligned form: threads reach it after per-row loops of differing trip counts
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;\n" ::: "memory");
}

// 3x3 pattern slot of offset (di, dj), |di|,|dj| <= 1
__host__ __device__ constexpr int pslot(int di, int dj) { return (di + 1) * 3 + (dj + 1); }
// 13-point Jacobian offset index of a 3x3 pattern slot
__host__ __device__ constexpr int slot_to_off(int s) {
    return s == 4 ? 0 : s == 1 ? 1 : s == 7 ? 2 : s == 3 ? 3 : s == 5 ? 4 : s == 0 ? 9 : s == 2 ? 10 : s == 6 ? 11 : 12;
}
// index of an upper offset in c_udi/c_udj (-1 if none)
__host__ __device__ constexpr int up_index(int di, int dj) {
    return (di == 0 && dj == 1) ? 0 : (di == 1 && dj == -1) ? 1 : (di == 1 && dj == 0) ? 2 : (di == 1 && dj == 1) ? 3 : -1;
}
__host__ __device__ constexpr int lo_index(int di, int dj) {
    return (di == -1 && dj == -1) ? 0 : (di == -1 && dj == 0) ? 1 : (di == -1 && dj == 1) ? 2 : (di == 0 && dj == -1) ? 3 : -1;
}

template <int NQ>
__global__ void __cluster_dims__(ILU_CL, 1, 1) __launch_bounds__(ILU_THREADS)
    k_ilu_factor(int nic, int njc, const double* __restrict__ jac1, const double* __restrict__ dt, double psd,
                 double sj, float* __restrict__ ilu, int* __restrict__ err) {
    constexpr int BS = NQ * NQ;
    const int nlev = n_levels(nic, njc);
    const int lane = threadIdx.x & 7;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    const int ngroups = (gridDim.x * blockDim.x) >> 3;
    const unsigned gmask = 0xFFu << (threadIdx.x & 24);
    const int k = lane < NQ ? lane : 0;  // idle lanes shadow row 0 and store nothing
    for (int L = 0; L < nlev; L++) {
        int i_lo, cnt;
        level_range(L, nic, njc, i_lo, cnt);
        for (int t = gid; t < cnt; t += ngroups) {
            const int i = i_lo + t, j = L - 2 * i;
            const size_t cell = (size_t)i * njc + j;
            float A[9][NQ];  // row k of the nine pattern blocks
#pragma unroll
            for (int s = 0; s < 9; s++) {
                const int di = s / 3 - 1, dj = s % 3 - 1;
                const bool in = i + di >= 0 && i + di < nic && j + dj >= 0 && j + dj < njc;
                const double* b = jac1 + (cell * NOFF + slot_to_off(s)) * BS + k * NQ;
#pragma unroll
                for (int l = 0; l < NQ; l++) A[s][l] = in ? (float)(sj * b[l]) : 0.f;
            }
            if (dt) {
                const float dd = (float)(psd / dt[cell * NQ + k]);
#pragma unroll
                for (int l = 0; l < NQ; l++)
                    if (l == k) A[4][l] += dd;
            }
            float* row = ilu + cell * ILU_NB * BS;
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int ni = i + ldi(a), nj = j + ldj(a);
                if (ni < 0 || ni >= nic || nj < 0 || nj >= njc) continue;
                const float* nrow = ilu + ((size_t)ni * njc + nj) * ILU_NB * BS;
                const int sl = pslot(ldi(a), ldj(a));
                // Lc = A_lo D_n^-1 (row k)
                float Lc[NQ];
#pragma unroll
                for (int l = 0; l < NQ; l++) Lc[l] = 0.f;
#pragma unroll
                for (int t2 = 0; t2 < NQ; t2++) {
#pragma unroll
                    for (int l = 0; l < NQ; l++) Lc[l] = fmaf(A[sl][t2], __ldcg(nrow + t2 * NQ + l), Lc[l]);
                }
                if (lane < NQ)
#pragma unroll
                    for (int l = 0; l < NQ; l++) row[(1 + a) * BS + k * NQ + l] = Lc[l];
                // A_target -= Lc U_n for the n's upper blocks that land in this row's pattern
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    constexpr int dummy = 0; (void)dummy;
                    const int di = ldi(a) + udi(b), dj = ldj(a) + udj(b);
                    if (di < -1 || di > 1 || dj < -1 || dj > 1) continue;
                    if (i + di < 0 || i + di >= nic || j + dj < 0 || j + dj >= njc) continue;
                    const int st = pslot(di, dj);
                    const float* U = nrow + (5 + b) * BS;
#pragma unroll
                    for (int t2 = 0; t2 < NQ; t2++) {
#pragma unroll
                        for (int l = 0; l < NQ; l++) A[st][l] = fmaf(-Lc[t2], __ldcg(U + t2 * NQ + l), A[st][l]);
                    }
                }
            }
            // D^-1 by Gauss-Jordan with partial pivoting across the group's lanes
            float a[NQ], inv[NQ];
#pragma unroll
            for (int l = 0; l < NQ; l++) { a[l] = A[4][l]; inv[l] = (l == k) ? 1.f : 0.f; }
            bool singular = false;
#pragma unroll
            for (int c = 0; c < NQ; c++) {
                float best = (lane >= c && lane < NQ) ? fabsf(a[c]) : -1.f;
                int p = lane;
#pragma unroll
                for (int o = 4; o > 0; o >>= 1) {
                    const float ob = __shfl_xor_sync(gmask, best, o, 8);
                    const int op = __shfl_xor_sync(gmask, p, o, 8);
                    if (ob > best || (ob == best && op < p)) { best = ob; p = op; }
                }
                if (!(best > 0.f)) singular = true;
                const int src = lane == c ? p : (lane == p ? c : lane);
#pragma unroll
                for (int l = 0; l < NQ; l++) {
                    a[l] = __shfl_sync(gmask, a[l], src, 8);
                    inv[l] = __shfl_sync(gmask, inv[l], src, 8);
                }
                if (lane == c) {
                    const float d = singular ? 0.f : 1.f / a[c];
#pragma unroll
                    for (int l = 0; l < NQ; l++) { a[l] *= d; inv[l] *= d; }
                }
                float pa[NQ], pi[NQ];
#pragma unroll
                for (int l = 0; l < NQ; l++) {
                    pa[l] = __shfl_sync(gmask, a[l], c, 8);
                    pi[l] = __shfl_sync(gmask, inv[l], c, 8);
                }
                if (lane != c) {
                    const float f = a[c];
#pragma unroll
                    for (int l = 0; l < NQ; l++) { a[l] = fmaf(-f, pa[l], a[l]); inv[l] = fmaf(-f, pi[l], inv[l]); }
                }
            }
            if (singular && lane == 0) atomicExch(err, 1);
            if (lane < NQ) {
#pragma unroll
                for (int l = 0; l < NQ; l++) row[k * NQ + l] = inv[l];
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    const int s = pslot(udi(b), udj(b));
#pragma unroll
                    for (int l = 0; l < NQ; l++) row[(5 + b) * BS + k * NQ + l] = A[s][l];
                }
            }
        }
        cluster_barrier();
    }
}

// z = M^{-1} r (TRANS: M^{-T} r), both triangular sweeps in one cluster kernel;
// FP32 arithmetic, FP64 vectors.
template <int NQ, bool TRANS>
__global__ void __cluster_dims__(ILU_CL, 1, 1) __launch_bounds__(ILU_THREADS)
    k_ilu_solve(int nic, int njc, const float* __restrict__ ilu, const double* __restrict__ r, double* __restrict__ z) {
    constexpr int BS = NQ * NQ;
    const int nlev = n_levels(nic, njc);
    const int lane = threadIdx.x & 7;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    const int ngroups = (gridDim.x * blockDim.x) >> 3;
    const unsigned gmask = 0xFFu << (threadIdx.x & 24);
    const int k = lane < NQ ? lane : 0;
    // sweep 1 (increasing levels): L y = r, or U^T w = r
    for (int L = 0; L < nlev; L++) {
        int i_lo, cnt;
        level_range(L, nic, njc, i_lo, cnt);
        for (int t = gid; t < cnt; t += ngroups) {
            const int i = i_lo + t, j = L - 2 * i;
            const size_t cell = (size_t)i * njc + j;
            float v = (float)r[cell * NQ + k];
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int ni = i + ldi(a), nj = j + ldj(a);
                if (ni < 0 || ni >= nic || nj < 0 || nj >= njc) continue;
                const size_t nc = (size_t)ni * njc + nj;
                const float* B;
                if (!TRANS) B = ilu + (cell * ILU_NB + 1 + a) * BS + k * NQ;  // L_(cell,n) row k
                else B = ilu + (nc * ILU_NB + 5 + up_index(-ldi(a), -ldj(a))) * BS + k;  // U_(n,cell) column k
#pragma unroll
                for (int l = 0; l < NQ; l++) v = fmaf(-B[TRANS ? l * NQ : l], (float)__ldcg(z + nc * NQ + l), v);
            }
            if (TRANS) {  // w = D^-T v
                const float* Di = ilu + cell * ILU_NB * BS + k;
                float w = 0.f;
#pragma unroll
                for (int l = 0; l < NQ; l++) w = fmaf(Di[l * NQ], __shfl_sync(gmask, v, l, 8), w);
                v = w;
            }
            if (lane < NQ) z[cell * NQ + k] = (double)v;
        }
        cluster_barrier();
    }
    // sweep 2 (decreasing levels): U x = y, or L^T v = w
    for (int L = nlev - 1; L >= 0; L--) {
        int i_lo, cnt;
        level_range(L, nic, njc, i_lo, cnt);
        for (int t = gid; t < cnt; t += ngroups) {
            const int i = i_lo + t, j = L - 2 * i;
            const size_t cell = (size_t)i * njc + j;
            float v = (float)__ldcg(z + cell * NQ + k);
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const int mi = i + udi(b), mj = j + udj(b);
                if (mi < 0 || mi >= nic || mj < 0 || mj >= njc) continue;
                const size_t mc = (size_t)mi * njc + mj;
                const float* B;
                if (!TRANS) B = ilu + (cell * ILU_NB + 5 + b) * BS + k * NQ;  // U_(cell,m) row k
                else B = ilu + (mc * ILU_NB + 1 + lo_index(-udi(b), -udj(b))) * BS + k;  // L_(m,cell) column k
#pragma unroll
                for (int l = 0; l < NQ; l++) v = fmaf(-B[TRANS ? l * NQ : l], (float)__ldcg(z + mc * NQ + l), v);
            }
            if (!TRANS) {  // x = D^-1 v
                const float* Di = ilu + cell * ILU_NB * BS + k * NQ;
                float w = 0.f;
#pragma unroll
                for (int l = 0; l < NQ; l++) w = fmaf(Di[l], __shfl_sync(gmask, v, l, 8), w);
                v = w;
            }
            if (lane < NQ) z[cell * NQ + k] = (double)v;
        }
        cluster_barrier();
    }
}

// Line-owned variant of k_ilu_solve for nic <= ILU_CL * ILU_LINE_GROUPS: the
// 8-lane group g of CTA r owns i-line i = r + ILU_CL g for the whole solve.  A
// row needs, besides its own line's previous value, the three nearest values
// of the neighbouring line, finished at the last three levels; each line
// keeps its last four values in a shared-memory ring that the neighbouring
// line's CTA reads through distributed shared memory.  A row's factor data
// lies in its line's contiguous records, so the next level's rows are
// prefetched while the cluster barrier is pending: the barrier is split into
// a cluster-scope release fence (ring writes), the prefetch and the deferred
// global store, a relaxed arrive and an acquiring wait.
constexpr int ILU_LINE_GROUPS = 128;  // 1024 threads per CTA

__device__ __forceinline__ void cluster_fence() { asm volatile("fence.acq_rel.cluster;" ::: "memory"); }
__device__ __forceinline__ void cluster_arrive_relaxed() { asm volatile("barrier.cluster.arrive.relaxed;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire;" ::: "memory"); }
__device__ __forceinline__ const float* peer_smem(const float* p, unsigned rank) {
    unsigned long long out;
    asm volatile("mapa.u64 %0, %1, %2;" : "=l"(out) : "l"(p), "r"(rank));
    return reinterpret_cast<const float*>(out);
}

template <int NQ, bool TRANS>
__global__ void __cluster_dims__(ILU_CL, 1, 1) __launch_bounds__(ILU_LINE_GROUPS * 8)
    k_ilu_solve_lines(int nic, int njc, const float* __restrict__ ilu, const double* __restrict__ r,
                      double* __restrict__ z) {
    constexpr int BS = NQ * NQ;
    __shared__ float ring[ILU_LINE_GROUPS * 32];  // per owned line: 4 slots x 8 floats
    const int lane = threadIdx.x & 7, g = threadIdx.x >> 3;
    const int i = blockIdx.x + ILU_CL * g;
    const bool own = i < nic;
    const int k = lane < NQ ? lane : 0;
    const unsigned gmask = 0xFFu << (threadIdx.x & 24);
    float* my_ring = ring + g * 32;
    const float* prev_ring = (own && i >= 1) ? peer_smem(ring + ((i - 1) / ILU_CL) * 32, (i - 1) % ILU_CL) : nullptr;
    const float* next_ring = (own && i + 1 < nic) ? peer_smem(ring + ((i + 1) / ILU_CL) * 32, (i + 1) % ILU_CL) : nullptr;
    const int nlev = n_levels(nic, njc);
    float blk[4][NQ], dia[NQ];  // prefetched block rows (or columns) and D^-1 row (column)
    double rk = 0.0;            // prefetched right-hand side component
    // load the factor data row (i, j) needs in sweep s (1: forward, 2: backward)
    auto fetch = [&](int s, int j) {
        const size_t cell = (size_t)i * njc + j;
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const int di = s == 1 ? ldi(a) : udi(a), dj = s == 1 ? ldj(a) : udj(a);
            const bool in = i + di >= 0 && i + di < nic && j + dj >= 0 && j + dj < njc;
            const size_t nb = in ? (size_t)(i + di) * njc + (j + dj) : cell;  // neighbour record (own if outside)
            const float* B;
            if (s == 1) B = !TRANS ? ilu + (cell * ILU_NB + 1 + a) * BS + k * NQ
                                   : ilu + (nb * ILU_NB + 5 + up_index(-di, -dj)) * BS + k;
            else B = !TRANS ? ilu + (cell * ILU_NB + 5 + a) * BS + k * NQ
                            : ilu + (nb * ILU_NB + 1 + lo_index(-di, -dj)) * BS + k;
#pragma unroll
            for (int l = 0; l < NQ; l++) blk[a][l] = in ? __ldg(B + (TRANS ? l * NQ : l)) : 0.f;
        }
        const float* Di = ilu + cell * ILU_NB * BS + (TRANS ? k : k * NQ);
#pragma unroll
        for (int l = 0; l < NQ; l++) dia[l] = __ldg(Di + (TRANS ? l * NQ : l));
        rk = s == 1 ? __ldg(r + cell * NQ + k) : z[cell * NQ + k];
    };
    for (int s = 1; s <= 2; s++) {
        if (own) {
            const int j0 = s == 1 ? 0 : njc - 1;
            const int L0 = 2 * i + j0;
            if ((s == 1 && L0 == 0) || (s == 2 && L0 == nlev - 1)) fetch(s, j0);
        }
        for (int step = 0; step < nlev; step++) {
            const int L = s == 1 ? step : nlev - 1 - step;
            const int j = L - 2 * i;
            bool done = false;
            float v = 0.f;
            size_t cell = 0;
            if (own && j >= 0 && j < njc) {
                cell = (size_t)i * njc + j;
                v = (float)rk;
#pragma unroll
                for (int a = 0; a < 4; a++) {
                    const int di = s == 1 ? ldi(a) : udi(a), dj = s == 1 ? ldj(a) : udj(a);
                    const int jn = j + dj;
                    if (i + di < 0 || i + di >= nic || jn < 0 || jn >= njc) continue;
                    const float* y = (di == 0 ? my_ring : (s == 1 ? prev_ring : next_ring)) + (jn & 3) * 8;
#pragma unroll
                    for (int l = 0; l < NQ; l++) v = fmaf(-blk[a][l], y[l], v);
                }
                if ((s == 1) == TRANS) {  // apply D^-1 (forward sweep of M^-T, backward sweep of M^-1)
                    float w = 0.f;
#pragma unroll
                    for (int l = 0; l < NQ; l++) w = fmaf(dia[l], __shfl_sync(gmask, v, l, 8), w);
                    v = w;
                }
                if (lane < NQ) my_ring[(j & 3) * 8 + k] = v;
                done = true;
            }
            cluster_fence();
            if (done && lane < NQ) z[cell * NQ + k] = (double)v;
            // prefetch the next level's row of this line
            const int jn = s == 1 ? j + 1 : j - 1;
            if (own && jn >= 0 && jn < njc) fetch(s, jn);
            cluster_arrive_relaxed();
            cluster_wait();
        }
    }
}

// ---------------------------------------------------------------------------
// Krylov vector kernels: deterministic multi-dot (fixed grid, fixed tree)
// ---------------------------------------------------------------------------
constexpr int DOT_BLOCKS = 128;
constexpr int NORM_PART_BLOCKS = 128;
__global__ void __launch_bounds__(256) k_mdot_part(const double* __restrict__ V, size_t n, const double* __restrict__ w,
                                                   double* __restrict__ part) {
    const int vi = blockIdx.y;
    const double* v = V + (size_t)vi * n;
    double acc = 0.0;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        acc = fma(v[t], w[t], acc);
    __shared__ double sm[8];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < 8; k++) s += sm[k];
        part[vi * DOT_BLOCKS + blockIdx.x] = s;
    }
}
__global__ void k_mdot_final(const double* __restrict__ part, int nvec, double* __restrict__ h) {
    const int vi = blockIdx.x * blockDim.x + threadIdx.x;
    if (vi >= nvec) return;
    double s = 0.0;
    for (int b = 0; b < DOT_BLOCKS; b++) s += part[vi * DOT_BLOCKS + b];
    h[vi] = s;
}
// w -= sum_i h[i] V_i
__global__ void k_maxpy(const double* __restrict__ V, int nvec, size_t n, const double* __restrict__ h,
                        double* __restrict__ w) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        double s = w[t];
        for (int i = 0; i < nvec; i++) s -= h[i] * V[(size_t)i * n + t];
        w[t] = s;
    }
}
// y = sum_i c[i] V_i
__global__ void k_combine(const double* __restrict__ V, int nvec, size_t n, const double* __restrict__ c,
                          double* __restrict__ y) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < nvec; i++) s += c[i] * V[(size_t)i * n + t];
        y[t] = s;
    }
}
// explicit stage, the arithmetic of update_forward_euler / update_rk4
// (src/solver/solver.cpp:12-26): out = q + rhs * dt / denom
__global__ void k_stage(size_t n, const double* q, const double* __restrict__ rhs,
                        const double* __restrict__ dt, double denom, double* out) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        out[t] = q[t] + rhs[t] * dt[t] / denom;
}
__global__ void k_axpby(size_t n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        y[t] = a * x[t] + b * y[t];
}
__global__ void k_scale_to(size_t n, const double* __restrict__ x, double a, double* __restrict__ y) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        y[t] = a * x[t];
}

// Objective gradient seed: P-bar of the wall rows from sum_i w_i Cf_i, with
// Cf_i = mu_inf (u_y - v_x)/q_inf at the j=0 face i (gathered per cell).
__global__ void k_cf_adj(DevCase c, const double* __restrict__ w, double scale, double* __restrict__ Pbar) {
    const int n = 2 * (c.nic + 2);
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int ip = t >> 1, jp = t & 1;
    double ub = 0.0, vb = 0.0;
    // roles: jp = 0 -> L of face ip-1, Pa of face ip-2, Ma of face ip
    //        jp = 1 -> R of face ip-1, Pb of face ip-2, Mb of face ip
    const int faces[3] = {ip - 1, ip - 2, ip};
    for (int r = 0; r < 3; r++) {
        const int i = faces[r];
        if (i < 0 || i >= c.nic) continue;
        const double* gm = c.geo_j + ((size_t)i * c.nj) * NGEO;
        double wx, wy;
        if (r == 0) { wx = jp == 0 ? gm[G_WLX] : gm[G_WRX]; wy = jp == 0 ? gm[G_WLY] : gm[G_WRY]; }
        else if (r == 1) { wx = gm[G_WPX]; wy = gm[G_WPY]; }
        else { wx = gm[G_WMX]; wy = gm[G_WMY]; }
        const double s = w[i] * scale;
        ub += s * wy;
        vb -= s * wx;
    }
    double* o = Pbar + pidx(c, ip, jp);
    o[P_U] += ub;
    o[P_V] += vb;
}

// per-block max of |dq_0 / q_0| (density change), deterministic
__global__ void k_max_rel_drho(size_t ncell, int nq, const double* __restrict__ q, const double* __restrict__ dq,
                               double* __restrict__ part) {
    double m = 0.0;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(dq[c * nq] / q[c * nq]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    __shared__ double sm[8];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int k = 0; k < 8; k++) r = fmax(r, sm[k]);
        part[blockIdx.x] = r;
    }
}
// SA: rho nu_tilde keeps at least `frac` of its previous value
__global__ void k_nut_floor(size_t ncell, double* __restrict__ q, const double* __restrict__ qold, double frac) {
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
        const double o = qold[c * 5 + 4];
        const double lo = o > 0.0 ? frac * o : o;
        if (q[c * 5 + 4] < lo) q[c * 5 + 4] = lo;
    }
}

template <class T>
int alloc_s(T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return stx::cuda_fail(e, "cudaMalloc (solver buffers)");
    return ST_OK;
}

int ensure_solver(st_ctx* x, int m) {
    const size_t n = x->ncell * x->nq;
    int rc = ST_OK;
    if (!x->jac) {
        rc = alloc_s(&x->jac, x->ncell * NOFF * x->nq * x->nq);
        if (rc == ST_OK) rc = alloc_s(&x->jac1, x->ncell * NOFF * x->nq * x->nq);
        if (rc == ST_OK) rc = alloc_s(&x->lfac, x->ncell * ILU_NB * x->nq * x->nq);
        if (rc == ST_OK) rc = alloc_s(&x->kz, n);
        if (rc == ST_OK) rc = alloc_s(&x->kw, n);
        if (rc == ST_OK) rc = alloc_s(&x->kr, n);
        if (rc == ST_OK) rc = alloc_s(&x->dq, n);
        if (rc == ST_OK) rc = alloc_s(&x->qsave, n);
        if (rc) return rc;
    }
    if (x->kv_m < m) {
        if (x->kv) cudaFree(x->kv);
        if (x->kzb) cudaFree(x->kzb);
        if (x->kh) cudaFree(x->kh);
        if (x->kpart) cudaFree(x->kpart);
        x->kv = nullptr; x->kzb = nullptr; x->kh = nullptr; x->kpart = nullptr;
        rc = alloc_s(&x->kv, (size_t)(m + 1) * n);
        if (rc == ST_OK) rc = alloc_s(&x->kzb, (size_t)m * n);
        if (rc == ST_OK) rc = alloc_s(&x->kh, (size_t)(m + 2));
        if (rc == ST_OK) rc = alloc_s(&x->kpart, (size_t)(m + 2) * DOT_BLOCKS);
        if (rc) return rc;
        x->kv_m = m;
    }
    return ST_OK;
}

// Boundary list check for the implicit path and the ghost masks of its
// non-local copies (once per context).
int partner_setup(st_ctx* x) {
    if (x->partners_checked) return ST_OK;
    const int nic = x->c.ni - 1, njc = x->c.nj - 1;
    std::vector<int> m[NFAM] = {std::vector<int>(nic), std::vector<int>(njc), std::vector<int>(njc)};
    int on[NFAM];
    const char* why = "";
    if (partner_masks(nic, njc, x->bcs.data(), (int)x->bcs.size(), m[0].data(), m[1].data(), m[2].data(), on, &why))
        return fail(ST_ERR_UNSUPPORTED, std::string("implicit solve: ") + why);
    for (int f = 0; f < NFAM; f++) {
        x->pmask[f] = m[f];
        x->pfam_on[f] = on[f] != 0;
        if (!on[f]) continue;
        const size_t len = (size_t)fam_len(f, nic, njc);
        int rc = x->pmask_d[f] ? ST_OK : alloc_s(&x->pmask_d[f], len);
        if (rc == ST_OK && !x->wpart[f]) rc = alloc_s(&x->wpart[f], len * NWS * x->nq * x->nq);
        if (rc) return rc;
        ST_CUDA(cudaMemcpyAsync(x->pmask_d[f], m[f].data(), len * sizeof(int), cudaMemcpyHostToDevice, x->stream));
        x->has_partners = true;
        for (int pp = 0; pp < (int)len; pp++)
            for (int t = 0; t < NWS; t++) {
                const int b = pp - wslot_d(t);
                if (b >= 0 && b < (int)len && m[f][b] && fold_offset(f, pp, t, nic, njc) >= 0) x->pfold = true;
            }
    }
    // the wake strip level (not where a fold already puts wake partners into
    // the ILU, and only while its dense block stays small)
    if (on[FAM_WAKE] && !x->pfold) {
        std::vector<int> cells(2 * (size_t)nic);
        const int ns = strip_cells(nic, njc, m[FAM_WAKE].data(), cells.data());
        if (ns > 0 && ns * x->nq <= STRIP_MAX) {
            cells.resize(ns);
            x->strip_cells = cells;
            x->strip_ns = ns;
            const size_t n = (size_t)ns * x->nq;
            int rc = x->strip_cells_d ? ST_OK : alloc_s(&x->strip_cells_d, (size_t)ns);
            if (rc == ST_OK && !x->strip_jac_d) rc = alloc_s(&x->strip_jac_d, (size_t)ns * NOFF * x->nq * x->nq);
            if (rc == ST_OK && !x->strip_dt_d) rc = alloc_s(&x->strip_dt_d, n);
            if (rc == ST_OK && !x->strip_inv_d) rc = alloc_s(&x->strip_inv_d, n * n);
            if (rc == ST_OK && !x->strip_res_d) rc = alloc_s(&x->strip_res_d, n);
            if (rc) return rc;
            ST_CUDA(cudaMemcpyAsync(x->strip_cells_d, cells.data(), ns * sizeof(int), cudaMemcpyHostToDevice, x->stream));
        }
    }
    for (int f = 0; f < NFAM && (x->pfold || x->strip_ns > 0); f++) {
        if (!on[f] || x->wpart1[f]) continue;
        int rc = alloc_s(&x->wpart1[f], (size_t)fam_len(f, nic, njc) * NWS * x->nq * x->nq);
        if (rc) return rc;
    }
    ST_CUDA(cudaStreamSynchronize(x->stream));
    x->partners_checked = true;
    return ST_OK;
}

// Partner blocks of the order-`order` residual into out[f]: per family,
// residue k and component, a full and a frozen JVP of the same seed (x->kz ->
// x->kw, x->kr; both free during assembly).
int assemble_partners(st_ctx* x, int order, double* const* out) {
    const int nq = x->nq, nic = x->c.ni - 1, njc = x->c.nj - 1;
    cudaStream_t s = x->stream;
    for (int f = 0; f < NFAM; f++) {
        if (!x->pfam_on[f]) continue;
        const int len = fam_len(f, nic, njc);
        const unsigned gl = grid_for((size_t)len), gw = grid_for((size_t)len * NWS);
        ST_CUDA(cudaMemsetAsync(out[f], 0, (size_t)len * NWS * nq * nq * 8, s));
        for (int k = 0; k < 3; k++) {
            bool seeded = false;
            for (int b = k; b < len; b += 3) seeded |= x->pmask[f][b] != 0;
            if (!seeded) continue;
            for (int comp = 0; comp < nq; comp++) {
                ST_CUDA(cudaMemsetAsync(x->kz, 0, x->ncell * nq * 8, s));
                if (nq == 5) k_partner_seed<5><<<gl, 256, 0, s>>>(f, nic, njc, x->pmask_d[f], k, comp, x->kz);
                else k_partner_seed<4><<<gl, 256, 0, s>>>(f, nic, njc, x->pmask_d[f], k, comp, x->kz);
                int rc = stx::run_jvp(x, x->kz, nullptr, x->kw, order, 0);
                if (rc == ST_OK) rc = stx::run_jvp(x, x->kz, nullptr, x->kr, order, 1);
                if (rc) return rc;
                if (nq == 5)
                    k_partner_extract<5><<<gw, 256, 0, s>>>(f, nic, njc, x->pmask_d[f], k, comp, x->kw, x->kr, out[f]);
                else
                    k_partner_extract<4><<<gw, 256, 0, s>>>(f, nic, njc, x->pmask_d[f], k, comp, x->kw, x->kr, out[f]);
            }
        }
    }
    ST_LAUNCH_CHECK("partner assembly");
    return ST_OK;
}

// jac[row][o] += W for the partner blocks inside the ILU(0) pattern
int fold_partners(st_ctx* x, double* const* W, double* jac) {
    const int nic = x->c.ni - 1, njc = x->c.nj - 1;
    for (int f = 0; f < NFAM; f++) {
        if (!x->pfam_on[f]) continue;
        const unsigned gl = grid_for((size_t)fam_len(f, nic, njc));
        if (x->nq == 5) k_partner_fold<5><<<gl, 256, 0, x->stream>>>(f, nic, njc, W[f], jac);
        else k_partner_fold<4><<<gl, 256, 0, x->stream>>>(f, nic, njc, W[f], jac);
    }
    ST_LAUNCH_CHECK("partner fold");
    return ST_OK;
}

// Block Jacobian of the order-`order` residual at the context state into
// `out` (x->jac or x->jac1).  A first-order Jacobian has the 9-point stencil,
// so 9 colours suffice; second order needs 25.
int assemble_into(st_ctx* x, int order, double* out) {
    const int nq = x->nq, nic = x->c.ni - 1, njc = x->c.nj - 1;
    cudaStream_t s = x->stream;
    ST_CUDA(cudaMemsetAsync(out, 0, x->ncell * NOFF * nq * nq * 8, s));
    const unsigned g = grid_for(x->ncell);
    const int cs = order == 1 ? 3 : 5;
    for (int ci = 0; ci < cs; ci++)
        for (int cj = 0; cj < cs; cj++)
            for (int comp = 0; comp < nq; comp++) {
                if (nq == 5) k_seed<5><<<g, 256, 0, s>>>(nic, njc, cs, ci, cj, comp, x->kz);
                else k_seed<4><<<g, 256, 0, s>>>(nic, njc, cs, ci, cj, comp, x->kz);
                int rc = stx::run_jvp(x, x->kz, nullptr, x->kw, order, x->has_partners ? 1 : 0);
                if (rc) return rc;
                if (nq == 5) k_extract<5><<<g, 256, 0, s>>>(nic, njc, cs, ci, cj, comp, x->kw, out);
                else k_extract<4><<<g, 256, 0, s>>>(nic, njc, cs, ci, cj, comp, x->kw, out);
            }
    ST_LAUNCH_CHECK("jacobian assembly");
    return ST_OK;
}

// The operator's Jacobian: regular blocks and the non-local copies' partners.
int assemble(st_ctx* x, int order) {
    int rc = partner_setup(x);
    if (rc == ST_OK) rc = ensure_solver(x, 1);
    if (rc == ST_OK) rc = assemble_into(x, order, x->jac);
    if (rc == ST_OK && x->has_partners) rc = assemble_partners(x, order, x->wpart);
    return rc;
}

// Operator Jacobian (order `order`) and, for the preconditioner, the
// first-order Jacobian (reusing the operator when it is first order).  The
// preconditioner's ILU(0) pattern is the 3x3 neighbourhood: partner blocks
// whose source lies in it (periodic boundaries two cells across) are folded
// into the preconditioner's copy of the blocks, the others left out.
int assemble_pair(st_ctx* x, int order) {
    int rc = assemble(x, order);
    if (rc) return rc;
    x->strip_W1 = nullptr;
    if (order == 1) {
        if (x->strip_ns > 0) x->strip_W1 = x->wpart[FAM_WAKE];
        if (!x->pfold) {
            x->jac1_is_jac = true;
            return ST_OK;
        }
        // the operator's blocks plus its own (first-order) partners
        x->jac1_is_jac = false;
        ST_CUDA(cudaMemcpyAsync(x->jac1, x->jac, x->ncell * NOFF * x->nq * x->nq * 8, cudaMemcpyDeviceToDevice,
                                x->stream));
        return fold_partners(x, x->wpart, x->jac1);
    }
    x->jac1_is_jac = false;
    rc = assemble_into(x, 1, x->jac1);
    if (rc || !(x->pfold || x->strip_ns > 0)) return rc;
    rc = assemble_partners(x, 1, x->wpart1);
    if (rc) return rc;
    if (x->strip_ns > 0) x->strip_W1 = x->wpart1[FAM_WAKE];
    return x->pfold ? fold_partners(x, x->wpart1, x->jac1) : ST_OK;
}

struct LinOp {
    bool trans;
    double sd, sj;         // operator: sd D + sj J (transposed if trans)
    const double* dt;      // D = diag(1/dt) (null: no D term)
    double psd;            // preconditioner: psd D + sj J on each j-line
    const double* pdt;
};

int apply_A(st_ctx* x, const LinOp& op, const double* in, double* out) {
    const int nic = x->c.ni - 1, njc = x->c.nj - 1;
    const unsigned g = grid_for(x->ncell);
    if (x->nq == 5) {
        if (op.trans) k_spmv<5, true><<<g, 256, 0, x->stream>>>(nic, njc, x->jac, in, out, op.dt, op.sd, op.sj);
        else k_spmv<5, false><<<g, 256, 0, x->stream>>>(nic, njc, x->jac, in, out, op.dt, op.sd, op.sj);
    } else {
        if (op.trans) k_spmv<4, true><<<g, 256, 0, x->stream>>>(nic, njc, x->jac, in, out, op.dt, op.sd, op.sj);
        else k_spmv<4, false><<<g, 256, 0, x->stream>>>(nic, njc, x->jac, in, out, op.dt, op.sd, op.sj);
    }
    for (int f = 0; f < NFAM; f++) {
        if (!x->pfam_on[f]) continue;
        const unsigned gl = grid_for((size_t)fam_len(f, nic, njc));
        const double* W = x->wpart[f];
        if (x->nq == 5) {
            if (op.trans) k_partner_apply<5, true><<<gl, 256, 0, x->stream>>>(f, nic, njc, W, in, out, op.sj);
            else k_partner_apply<5, false><<<gl, 256, 0, x->stream>>>(f, nic, njc, W, in, out, op.sj);
        } else {
            if (op.trans) k_partner_apply<4, true><<<gl, 256, 0, x->stream>>>(f, nic, njc, W, in, out, op.sj);
            else k_partner_apply<4, false><<<gl, 256, 0, x->stream>>>(f, nic, njc, W, in, out, op.sj);
        }
    }
    ST_LAUNCH_CHECK("spmv");
    return ST_OK;
}

int check_err(st_ctx* x, const char* what) {
    int err = 0;
    ST_CUDA(cudaMemcpyAsync(&err, x->err_d, sizeof(int), cudaMemcpyDeviceToHost, x->stream));
    ST_CUDA(cudaStreamSynchronize(x->stream));
    if (err) return fail(ST_ERR_NONFINITE, std::string(what) + ": singular diagonal block");
    return ST_OK;
}

// one cluster of ILU_CL CTAs walks the levels
// The wake strip level for a forward solve: gather the strip's blocks, build
// and invert its dense block on the host, upload the inverse.  A singular or
// non-finite block leaves the plain ILU(0).
int strip_factor(st_ctx* x, const LinOp& op, const double* j1) {
    const auto t0 = std::chrono::steady_clock::now();
    const int nic = x->c.ni - 1, njc = x->c.nj - 1, nq = x->nq, ns = x->strip_ns, n = ns * nq;
    cudaStream_t s = x->stream;
    const size_t nb = (size_t)ns * NOFF * nq * nq;
    if (nq == 5) k_strip_gather<5><<<grid_for(nb), 256, 0, s>>>(ns, x->strip_cells_d, j1, op.pdt, x->strip_jac_d, x->strip_dt_d);
    else k_strip_gather<4><<<grid_for(nb), 256, 0, s>>>(ns, x->strip_cells_d, j1, op.pdt, x->strip_jac_d, x->strip_dt_d);
    ST_LAUNCH_CHECK("strip gather");
    std::vector<double> jac_s(nb), dt_s((size_t)n), w1((size_t)nic * NWS * nq * nq);
    ST_CUDA(cudaMemcpyAsync(jac_s.data(), x->strip_jac_d, nb * 8, cudaMemcpyDeviceToHost, s));
    if (op.pdt) ST_CUDA(cudaMemcpyAsync(dt_s.data(), x->strip_dt_d, (size_t)n * 8, cudaMemcpyDeviceToHost, s));
    ST_CUDA(cudaMemcpyAsync(w1.data(), x->strip_W1, w1.size() * 8, cudaMemcpyDeviceToHost, s));
    ST_CUDA(cudaStreamSynchronize(s));
    std::vector<double> A((size_t)n * n), inv((size_t)n * n);
    strip_matrix(nic, njc, nq, ns, x->strip_cells.data(), jac_s.data(), op.pdt ? dt_s.data() : nullptr, w1.data(),
                 op.psd, op.sj, A.data());
    if (!dense_invert(n, A.data(), inv.data())) return ST_OK;
    for (double v : inv)
        if (!std::isfinite(v)) return ST_OK;
    ST_CUDA(cudaMemcpyAsync(x->strip_inv_d, inv.data(), inv.size() * 8, cudaMemcpyHostToDevice, s));
    ST_CUDA(cudaStreamSynchronize(s));
    x->strip_ready = true;
    x->strip_factored++;
    x->strip_host_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return ST_OK;
}

int factor_M(st_ctx* x, const LinOp& op) {
    const int nic = x->c.ni - 1, njc = x->c.nj - 1;
    x->strip_ready = false;
    ST_CUDA(cudaMemsetAsync(x->err_d, 0, sizeof(int), x->stream));
    const double* j1 = x->jac1_is_jac ? x->jac : x->jac1;
    if (x->nq == 5)
        k_ilu_factor<5><<<ILU_CL, ILU_THREADS, 0, x->stream>>>(nic, njc, j1, op.pdt, op.psd, op.sj, x->lfac, x->err_d);
    else
        k_ilu_factor<4><<<ILU_CL, ILU_THREADS, 0, x->stream>>>(nic, njc, j1, op.pdt, op.psd, op.sj, x->lfac, x->err_d);
    ST_LAUNCH_CHECK("ILU factorisation");
    int rc = check_err(x, "ILU factorisation");
    if (rc == ST_OK && !op.trans && x->strip_ns > 0 && x->strip_W1) rc = strip_factor(x, op, j1);
    return rc;
}

int apply_M(st_ctx* x, const LinOp& op, const double* in, double* out) {
    const int nic = x->c.ni - 1, njc = x->c.nj - 1;
    cudaStream_t s = x->stream;
    if (nic <= ILU_CL * ILU_LINE_GROUPS) {
        const int th = ILU_LINE_GROUPS * 8;
        if (x->nq == 5) {
            if (op.trans) k_ilu_solve_lines<5, true><<<ILU_CL, th, 0, s>>>(nic, njc, x->lfac, in, out);
            else k_ilu_solve_lines<5, false><<<ILU_CL, th, 0, s>>>(nic, njc, x->lfac, in, out);
        } else {
            if (op.trans) k_ilu_solve_lines<4, true><<<ILU_CL, th, 0, s>>>(nic, njc, x->lfac, in, out);
            else k_ilu_solve_lines<4, false><<<ILU_CL, th, 0, s>>>(nic, njc, x->lfac, in, out);
        }
    } else if (x->nq == 5) {
        if (op.trans) k_ilu_solve<5, true><<<ILU_CL, ILU_THREADS, 0, s>>>(nic, njc, x->lfac, in, out);
        else k_ilu_solve<5, false><<<ILU_CL, ILU_THREADS, 0, s>>>(nic, njc, x->lfac, in, out);
    } else {
        if (op.trans) k_ilu_solve<4, true><<<ILU_CL, ILU_THREADS, 0, s>>>(nic, njc, x->lfac, in, out);
        else k_ilu_solve<4, false><<<ILU_CL, ILU_THREADS, 0, s>>>(nic, njc, x->lfac, in, out);
    }
    ST_LAUNCH_CHECK("ILU solve");
    if (!op.trans && x->strip_ready) {
        const double* j1 = x->jac1_is_jac ? x->jac : x->jac1;
        const int ns = x->strip_ns;
        if (x->nq == 5) {
            k_strip_residual<5><<<grid_for((size_t)ns), 256, 0, s>>>(nic, njc, ns, x->strip_cells_d, j1, x->strip_W1,
                                                                    op.pdt, op.psd, op.sj, in, out, x->strip_res_d);
            k_strip_update<5><<<grid_for((size_t)ns * 5), 256, 0, s>>>(ns, x->strip_cells_d, x->strip_inv_d,
                                                                      x->strip_res_d, out);
        } else {
            k_strip_residual<4><<<grid_for((size_t)ns), 256, 0, s>>>(nic, njc, ns, x->strip_cells_d, j1, x->strip_W1,
                                                                    op.pdt, op.psd, op.sj, in, out, x->strip_res_d);
            k_strip_update<4><<<grid_for((size_t)ns * 4), 256, 0, s>>>(ns, x->strip_cells_d, x->strip_inv_d,
                                                                      x->strip_res_d, out);
        }
        ST_LAUNCH_CHECK("wake strip correction");
    }
    return ST_OK;
}

// dots of V_0..V_{nvec-1} with w into host h (one synchronisation)
int mdot(st_ctx* x, const double* V, int nvec, size_t n, const double* w, double* h_host) {
    k_mdot_part<<<dim3(DOT_BLOCKS, nvec), 256, 0, x->stream>>>(V, n, w, x->kpart);
    k_mdot_final<<<(nvec + 63) / 64, 64, 0, x->stream>>>(x->kpart, nvec, x->kh);
    ST_LAUNCH_CHECK("mdot");
    ST_CUDA(cudaMemcpyAsync(h_host, x->kh, nvec * 8, cudaMemcpyDeviceToHost, x->stream));
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

// Flexible restarted GMRES (classical Gram-Schmidt, repeated once) for
// op * xsol = b; xsol holds the initial guess.  The preconditioned vectors
// Z_k = M^{-1} V_k are kept and the update is x += Z y, so the Arnoldi
// relation A Z = V H holds in FP64 whatever the preconditioner's rounding.
int gmres(st_ctx* x, const LinOp& op, const double* b, double* xsol, int m, int maxit, double rtol,
          st_solve_stats* st) {
    int rc = ensure_solver(x, m);
    if (rc) return rc;
    const size_t n = x->ncell * x->nq;
    const unsigned g = grid_for(n);
    cudaStream_t s = x->stream;
    double* V = x->kv;
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), gv(m + 1), h(m + 2), h2(m + 2), y(m);
    double beta0 = -1.0, res = 0.0;
    int it = 0;
    bool conv = false;
    while (it < maxit) {
        // r = b - A x
        rc = apply_A(x, op, xsol, x->kr);
        if (rc) return rc;
        k_axpby<<<g, 256, 0, s>>>(n, 1.0, b, -1.0, x->kr);
        double beta;
        rc = mdot(x, x->kr, 1, n, x->kr, &beta);
        if (rc) return rc;
        beta = std::sqrt(beta);
        if (!std::isfinite(beta)) return fail(ST_ERR_NONFINITE, "gmres: non-finite residual");
        if (beta0 < 0) beta0 = beta;
        res = beta;
        if (beta <= rtol * beta0 || beta == 0.0) { conv = true; break; }
        k_scale_to<<<g, 256, 0, s>>>(n, x->kr, 1.0 / beta, V);
        std::fill(gv.begin(), gv.end(), 0.0);
        gv[0] = beta;
        int k = 0;
        for (; k < m && it < maxit; k++, it++) {
            double* Zk = x->kzb + (size_t)k * n;
            rc = apply_M(x, op, V + (size_t)k * n, Zk);
            if (rc) return rc;
            rc = apply_A(x, op, Zk, x->kw);
            if (rc) return rc;
            for (int pass = 0; pass < 2; pass++) {
                rc = mdot(x, V, k + 1, n, x->kw, pass == 0 ? h.data() : h2.data());
                if (rc) return rc;
                ST_CUDA(cudaMemcpyAsync(x->kh, pass == 0 ? h.data() : h2.data(), (k + 1) * 8, cudaMemcpyHostToDevice, s));
                k_maxpy<<<g, 256, 0, s>>>(V, k + 1, n, x->kh, x->kw);
                if (pass == 1)
                    for (int i = 0; i <= k; i++) h[i] += h2[i];
            }
            double hn;
            rc = mdot(x, x->kw, 1, n, x->kw, &hn);
            if (rc) return rc;
            hn = std::sqrt(hn);
            for (int i = 0; i <= k; i++) H[(size_t)i * m + k] = h[i];
            H[(size_t)(k + 1) * m + k] = hn;
            for (int i = 0; i < k; i++) {
                const double a = H[(size_t)i * m + k], c2 = H[(size_t)(i + 1) * m + k];
                H[(size_t)i * m + k] = cs[i] * a + sn[i] * c2;
                H[(size_t)(i + 1) * m + k] = -sn[i] * a + cs[i] * c2;
            }
            const double a = H[(size_t)k * m + k], c2 = H[(size_t)(k + 1) * m + k];
            const double r = std::sqrt(a * a + c2 * c2);
            cs[k] = r > 0 ? a / r : 1.0;
            sn[k] = r > 0 ? c2 / r : 0.0;
            H[(size_t)k * m + k] = r;
            H[(size_t)(k + 1) * m + k] = 0.0;
            gv[k + 1] = -sn[k] * gv[k];
            gv[k] = cs[k] * gv[k];
            res = std::fabs(gv[k + 1]);
            if (!std::isfinite(res)) return fail(ST_ERR_NONFINITE, "gmres: breakdown");
            if (hn > 0.0) k_scale_to<<<g, 256, 0, s>>>(n, x->kw, 1.0 / hn, V + (size_t)(k + 1) * n);
            if (res <= rtol * beta0 || hn == 0.0) { k++; it++; conv = true; break; }
        }
        // y = H^{-1} g, x += Z y
        for (int i = k - 1; i >= 0; i--) {
            double sum = gv[i];
            for (int l = i + 1; l < k; l++) sum -= H[(size_t)i * m + l] * y[l];
            y[i] = sum / H[(size_t)i * m + i];
        }
        ST_CUDA(cudaMemcpyAsync(x->kh, y.data(), k * 8, cudaMemcpyHostToDevice, s));
        k_combine<<<g, 256, 0, s>>>(x->kzb, k, n, x->kh, x->kw);
        k_axpby<<<g, 256, 0, s>>>(n, 1.0, x->kw, 1.0, xsol);
        ST_LAUNCH_CHECK("gmres update");
        if (conv) break;
    }
    ST_CUDA(cudaStreamSynchronize(s));
    if (st) {
        st->iterations = it;
        st->converged = conv ? 1 : 0;
        st->residual0 = beta0;
        st->residual = res;
    }
    return ST_OK;
}

}  // namespace

extern "C" {

int st_jacobian_assemble(st_ctx* x, int lhs) {
    if (!x) return fail(ST_ERR_ARG, "st_jacobian_assemble: null context");
    if (int rc0 = partner_setup(x)) return rc0;
    int rc = assemble_pair(x, lhs ? x->c.lhs_order : x->c.order);
    if (rc) return rc;
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

int st_jacobian_blocks(st_ctx* x, double* blocks_host) {
    if (!x || !blocks_host) return fail(ST_ERR_ARG, "st_jacobian_blocks: null argument");
    if (!x->jac) return fail(ST_ERR_ARG, "st_jacobian_blocks: no Jacobian assembled");
    return stx::copy_sync(x, blocks_host, x->jac, x->ncell * NOFF * x->nq * x->nq * 8, cudaMemcpyDeviceToHost);
}

int st_jacobian_apply_device(st_ctx* x, const double* v_dev, double* out_dev, int transpose) {
    if (!x || !v_dev || !out_dev) return fail(ST_ERR_ARG, "st_jacobian_apply_device: null argument");
    if (!x->jac) return fail(ST_ERR_ARG, "st_jacobian_apply_device: no Jacobian assembled");
    LinOp op{transpose != 0, 0.0, 1.0, nullptr, 0.0, nullptr};
    int rc = apply_A(x, op, v_dev, out_dev);
    if (rc) return rc;
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

int st_linear_solve_device(st_ctx* x, double cfl, const double* b_dev, double* x_dev, int transpose, int krylov_m,
                           int maxit, double rtol, st_solve_stats* stats) {
    if (!x || !b_dev || !x_dev) return fail(ST_ERR_ARG, "st_linear_solve_device: null argument");
    if (!x->jac) return fail(ST_ERR_ARG, "st_linear_solve_device: no Jacobian assembled");
    if (krylov_m < 1 || krylov_m > 500 || maxit < 1) return fail(ST_ERR_ARG, "st_linear_solve_device: krylov sizes");
    int rc = stx::run_dt(x, cfl);
    if (rc) return rc;
    // (I/dt - J) x = b, or its transpose
    LinOp op{transpose != 0, 1.0, -1.0, x->dt, 1.0, x->dt};
    rc = factor_M(x, op);
    if (rc) return rc;
    return gmres(x, op, b_dev, x_dev, krylov_m, maxit, rtol, stats);
}

int st_solve(st_ctx* x, const st_solve_params* p, st_solve_stats* stats, double* history, int history_len,
             int* steps_done) {
    if (!x || !p) return fail(ST_ERR_ARG, "st_solve: null argument");
    if (p->max_steps < 0 || p->krylov_m < 1 || p->krylov_m > 500) return fail(ST_ERR_ARG, "st_solve: bad parameters");
    if (int rc0 = partner_setup(x)) return rc0;
    int rc = ensure_solver(x, p->krylov_m);
    if (rc) return rc;
    const int nq = x->nq;
    const size_t n = x->ncell * nq;
    const unsigned g = grid_for(n);
    cudaStream_t s = x->stream;
    double cfl = p->cfl, omega = p->under_relaxation;
    std::vector<double> nrm(nq);
    auto residual_norm = [&](double* out) -> int {
        int r = stx::run_residual(x, x->q, x->beta, x->rhs, x->c.order);
        if (r) return r;
        x->have_residual = true;
        r = stx::run_norms(x, x->rhs, nrm.data());
        if (r && r != ST_ERR_NONFINITE) return r;
        double m = 0.0;
        for (int k = 0; k < nq; k++) m = std::max(m, nrm[k]);
        *out = (r == ST_ERR_NONFINITE) ? NAN : m;
        return ST_OK;
    };
    double rn;
    rc = residual_norm(&rn);
    if (rc) return rc;
    if (!std::isfinite(rn)) return fail(ST_ERR_NONFINITE, "st_solve: non-finite initial residual");
    const double r0 = rn;
    int hist = 0, fails = 0, step = 0, accepted = 0;
    bool converged = false;
    st_solve_stats ls{};
    auto record = [&]() {
        if (history && hist + nq + 3 <= history_len) {
            history[hist++] = accepted;
            history[hist++] = cfl;
            history[hist++] = ls.iterations;
            for (int k = 0; k < nq; k++) history[hist++] = nrm[k];
        }
    };
    record();
    std::vector<double> part(NORM_PART_BLOCKS);
    for (step = 0; step < p->max_steps + p->max_failures; step++) {
        if (accepted >= p->min_steps && (rn <= p->tolerance || rn <= p->rel_tolerance * r0)) { converged = true; break; }
        if (accepted >= p->max_steps) break;
        rc = stx::run_dt(x, cfl);
        if (rc) return rc;
        rc = assemble_pair(x, x->c.lhs_order);
        if (rc) return rc;
        LinOp op{false, 1.0, -1.0, x->dt, 1.0, x->dt};
        rc = factor_M(x, op);
        if (rc) return rc;
        ST_CUDA(cudaMemsetAsync(x->dq, 0, n * 8, s));
        rc = gmres(x, op, x->rhs, x->dq, p->krylov_m, p->krylov_maxit, p->krylov_rtol, &ls);
        if (rc) return rc;
        double om = omega;
        if (p->max_rel_drho > 0.0) {
            k_max_rel_drho<<<NORM_PART_BLOCKS, 256, 0, s>>>(x->ncell, nq, x->q, x->dq, x->kpart);
            ST_CUDA(cudaMemcpyAsync(part.data(), x->kpart, NORM_PART_BLOCKS * 8, cudaMemcpyDeviceToHost, s));
            ST_CUDA(cudaStreamSynchronize(s));
            double mx = 0.0;
            for (double v : part) mx = std::max(mx, v);
            if (mx * om > p->max_rel_drho) om = p->max_rel_drho / mx;
        }
        ST_CUDA(cudaMemcpyAsync(x->qsave, x->q, n * 8, cudaMemcpyDeviceToDevice, s));
        k_axpby<<<g, 256, 0, s>>>(n, om, x->dq, 1.0, x->q);
        if (nq == 5 && p->nut_floor > 0.0) k_nut_floor<<<grid_for(x->ncell), 256, 0, s>>>(x->ncell, x->q, x->qsave, p->nut_floor);
        ST_LAUNCH_CHECK("update");
        double rt;
        rc = residual_norm(&rt);
        if (rc) return rc;
        // growth near round-off (below 1e-9 of the initial residual) or below
        // the absolute tolerance is noise, not divergence
        if (!std::isfinite(rt) || (rt > p->reject_factor * rn && rt > std::max(1e-9 * r0, p->tolerance))) {
            // undo the step, smaller CFL
            if (++fails > p->max_failures) return fail(ST_ERR_NONFINITE, "st_solve: diverged");
            ST_CUDA(cudaMemcpyAsync(x->q, x->qsave, n * 8, cudaMemcpyDeviceToDevice, s));
            cfl = std::max(p->cfl_min, cfl * 0.1);
            rc = residual_norm(&rn);
            if (rc) return rc;
            continue;
        }
        rn = rt;
        accepted++;
        record();
        if (p->cfl_growth > 0.0) {
            if (om >= omega) cfl = std::min(p->cfl_max, cfl * p->cfl_growth);
        } else if (p->cfl_ramp && accepted > p->cfl_ramp_iteration) {
            // ramp of Solver::solve (src/solver/solver.cpp:212-220)
            cfl = std::min(std::pow(cfl, p->cfl_ramp_exponent), p->cfl_max);
        }
        if (p->ser_exponent > 0.0) cfl = std::min(p->cfl_max, std::max(cfl, p->cfl * std::pow(r0 / std::max(rn, 1e-300), p->ser_exponent)));
        if (p->under_relaxation_ramp && accepted > p->under_relaxation_ramp_iteration)
            omega = std::min(std::pow(omega, p->under_relaxation_ramp_exponent), 10.0);  // solver.cpp:222-230
    }
    ST_CUDA(cudaStreamSynchronize(s));
    if (stats) *stats = ls;
    if (steps_done) *steps_done = accepted;
    if (!converged) return fail(ST_ERR_NOCONV, "st_solve: tolerance not reached");
    return ST_OK;
}

int st_explicit_solve(st_ctx* x, int scheme, double cfl, int steps, double tolerance, int check_every,
                      double* history, int history_len, int* steps_done) {
    if (!x) return fail(ST_ERR_ARG, "st_explicit_solve: null context");
    if ((scheme != 0 && scheme != 1) || !(cfl > 0.0) || steps < 0 || check_every < 1)
        return fail(ST_ERR_ARG, "st_explicit_solve: scheme 0 (forward_euler) or 1 (rk4_jameson), cfl > 0, check_every >= 1");
    const int nq = x->nq;
    const size_t n = x->ncell * nq;
    const unsigned g = grid_for(n);
    cudaStream_t s = x->stream;
    if (scheme == 1 && !x->qtmp) {
        if (cudaMalloc((void**)&x->qtmp, n * 8) != cudaSuccess) return fail(ST_ERR_CUDA, "cudaMalloc (RK stage state)");
    }
    std::vector<double> nrm(nq);
    int hist = 0, done = 0;
    bool converged = false;
    for (done = 0; done < steps;) {
        int rc = stx::run_dt(x, cfl);  // EulerEquation::calc_dt at the step's start (solver.cpp:66)
        if (rc) return rc;
        if (scheme == 0) {
            rc = stx::run_residual(x, x->q, x->beta, x->rhs, x->c.order);
            if (rc) return rc;
            k_stage<<<g, 256, 0, s>>>(n, x->q, x->rhs, x->dt, 1.0, x->q);
        } else {
            ST_CUDA(cudaMemcpyAsync(x->qtmp, x->q, n * 8, cudaMemcpyDeviceToDevice, s));
            for (int st = 0; st < 4; st++) {
                rc = stx::run_residual(x, x->qtmp, x->beta, x->rhs, x->c.order);
                if (rc) return rc;
                k_stage<<<g, 256, 0, s>>>(n, x->q, x->rhs, x->dt, 4.0 - st, x->qtmp);
            }
            ST_CUDA(cudaMemcpyAsync(x->q, x->qtmp, n * 8, cudaMemcpyDeviceToDevice, s));
        }
        ST_LAUNCH_CHECK("explicit step");
        x->have_residual = false;
        done++;
        if (done % check_every == 0 || done == steps) {
            rc = stx::run_norms(x, x->rhs, nrm.data());
            if (rc) return rc;
            if (history && hist + nq + 1 <= history_len) {
                history[hist++] = done;
                for (int k = 0; k < nq; k++) history[hist++] = nrm[k];
            }
            double m = 0.0;
            for (int k = 0; k < nq; k++) m = std::max(m, nrm[k]);
            if (tolerance > 0.0 && m <= tolerance) { converged = true; break; }
        }
    }
    ST_CUDA(cudaStreamSynchronize(s));
    if (steps_done) *steps_done = done;
    if (tolerance > 0.0 && !converged) return fail(ST_ERR_NOCONV, "st_explicit_solve: tolerance not reached");
    return ST_OK;
}

int st_cf_gradient_device(st_ctx* x, const double* w_host, double* grad_dev) {
    if (!x || !w_host || !grad_dev) return fail(ST_ERR_ARG, "st_cf_gradient_device: null argument");
    int rc = stx::ensure_adjoint_buffers(x);
    if (rc) return rc;
    rc = ensure_solver(x, 1);
    if (rc) return rc;
    cudaStream_t s = x->stream;
    const int nic = x->c.ni - 1;
    ST_CUDA(cudaMemcpyAsync(x->cf, w_host, nic * 8, cudaMemcpyHostToDevice, s));
    const double qinf = 0.5 * x->c.rho_inf * (x->c.u_inf * x->c.u_inf + x->c.v_inf * x->c.v_inf);
    const DevCase& dc = x->dc;
    ST_CUDA(cudaMemsetAsync(x->Pbar, 0, x->npad * NP * 8, s));
    if (x->nq == 5) {
        k_prim<double, 5><<<grid_for(x->ncell), 256, 0, s>>>(dc, x->q, x->P);
        k_bc_taped<5><<<1, 1024, 0, s>>>(dc, x->P, x->tape);
        k_cf_adj<<<(2 * (nic + 2) + 255) / 256, 256, 0, s>>>(dc, x->cf, x->c.mu_inf / qinf, x->Pbar);
        k_bc_adj<5><<<1, 1024, 0, s>>>(dc, x->P, x->tape, x->Pbar);
        k_prim_adj<5><<<grid_for(x->ncell), 256, 0, s>>>(dc, x->q, x->P, x->Pbar, grad_dev, 0, x->ncell);
    } else {
        k_prim<double, 4><<<grid_for(x->ncell), 256, 0, s>>>(dc, x->q, x->P);
        k_bc_taped<4><<<1, 1024, 0, s>>>(dc, x->P, x->tape);
        k_cf_adj<<<(2 * (nic + 2) + 255) / 256, 256, 0, s>>>(dc, x->cf, x->c.mu_inf / qinf, x->Pbar);
        k_bc_adj<4><<<1, 1024, 0, s>>>(dc, x->P, x->tape, x->Pbar);
        k_prim_adj<4><<<grid_for(x->ncell), 256, 0, s>>>(dc, x->q, x->P, x->Pbar, grad_dev, 0, x->ncell);
    }
    ST_LAUNCH_CHECK("cf gradient");
    ST_CUDA(cudaStreamSynchronize(s));
    return ST_OK;
}

int st_adjoint_solve_device(st_ctx* x, const double* b_dev, double* psi_dev, double cfl_prec, int krylov_m, int maxit,
                            double rtol, st_solve_stats* stats) {
    if (!x || !b_dev || !psi_dev) return fail(ST_ERR_ARG, "st_adjoint_solve_device: null argument");
    if (krylov_m < 1 || krylov_m > 500 || maxit < 1) return fail(ST_ERR_ARG, "st_adjoint_solve_device: krylov sizes");
    if (int rc0 = partner_setup(x)) return rc0;
    // exact Jacobian of the residual actually solved (order, not lhs_order)
    int rc = assemble_pair(x, x->c.order);
    if (rc) return rc;
    rc = stx::run_dt(x, cfl_prec);
    if (rc) return rc;
    // operator (dR/dQ)^T exactly; the line preconditioner adds a pseudo-time
    // diagonal I/dt(cfl_prec) for robustness
    LinOp op{true, 0.0, 1.0, nullptr, -1.0, x->dt};
    rc = factor_M(x, op);
    if (rc) return rc;
    return gmres(x, op, b_dev, psi_dev, krylov_m, maxit, rtol, stats);
}

int st_tangent_solve_device(st_ctx* x, const double* b_dev, double* dq_dev, double cfl_prec, int krylov_m, int maxit,
                            double rtol, st_solve_stats* stats) {
    if (!x || !b_dev || !dq_dev) return fail(ST_ERR_ARG, "st_tangent_solve_device: null argument");
    if (krylov_m < 1 || krylov_m > 500 || maxit < 1) return fail(ST_ERR_ARG, "st_tangent_solve_device: krylov sizes");
    if (int rc0 = partner_setup(x)) return rc0;
    int rc = assemble_pair(x, x->c.order);
    if (rc) return rc;
    rc = stx::run_dt(x, cfl_prec);
    if (rc) return rc;
    LinOp op{false, 0.0, 1.0, nullptr, -1.0, x->dt};
    rc = factor_M(x, op);
    if (rc) return rc;
    return gmres(x, op, b_dev, dq_dev, krylov_m, maxit, rtol, stats);
}

int st_precond_info(st_ctx* x, int* strip_unknowns, int* strip_active, int* strip_factorisations,
                    double* strip_host_ms) {
    if (!x) return fail(ST_ERR_ARG, "st_precond_info: null context");
    if (strip_unknowns) *strip_unknowns = x->strip_ns * x->nq;
    if (strip_active) *strip_active = x->strip_ready ? 1 : 0;
    if (strip_factorisations) *strip_factorisations = x->strip_factored;
    if (strip_host_ms) *strip_host_ms = x->strip_host_ms;
    return ST_OK;
}

}  // extern "C"
