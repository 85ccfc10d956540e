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
#include <cmath>
#include <cstring>
#include <vector>

#include "st_adjoint.cuh"
#include "st_context.h"

using namespace st;
using stx::fail;
using stx::grid_for;

namespace {

constexpr int NOFF = 13;
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
// so level 2i+j rows are independent; one cooperative kernel walks the levels
// with a grid barrier between them.  Natural order keeps the downstream
// ordering of the convective coupling; multicolour orderings of the same
// factorisation were tried on the CPU and needed 10x more Krylov iterations.
// ---------------------------------------------------------------------------
__device__ inline int n_levels(int nic, int njc) { return 2 * (nic - 1) + (njc - 1) + 1; }
__device__ inline void level_range(int L, int nic, int njc, int& i_lo, int& cnt) {
    const int t = L - (njc - 1);
    i_lo = t > 0 ? (t + 1) / 2 : 0;
    const int i_hi = min(nic - 1, L / 2);
    cnt = i_hi - i_lo + 1;
}

// Grid barrier for a cooperative launch (all blocks co-resident).  The spin is
// bounded: on time-out it raises *err, and every block returns false from
// then on, so the kernel always ends.
__device__ bool grid_barrier(unsigned* count, volatile unsigned* gen, int* err) {
    __syncthreads();
    __shared__ int ok;
    if (threadIdx.x == 0) {
        ok = 1;
        const unsigned g = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(count, 1u) + 1u;
        if (arrived == gridDim.x) {
            atomicExch(count, 0u);
            __threadfence();
            atomicAdd((unsigned*)gen, 1u);
        } else {
            long spins = 0;
            while (*gen == g) {
                if (*(volatile int*)err) { ok = 0; break; }
                if (++spins > (1L << 24)) { atomicExch(err, 2); ok = 0; break; }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (*(volatile int*)err) ok = 0;
    }
    __syncthreads();
    return ok != 0;
}

// lower neighbours of a row in elimination order, and upper neighbours
__constant__ int c_lo[4] = {9, 1, 10, 3};   // (-1,-1), (-1,0), (-1,1), (0,-1)
__constant__ int c_up[4] = {4, 11, 2, 12};  // (0,1), (1,-1), (1,0), (1,1)

template <int NQ>
__device__ inline void mat_mul(const double* a, const double* b, double* c) {
#pragma unroll
    for (int k = 0; k < NQ; k++)
#pragma unroll
        for (int l = 0; l < NQ; l++) {
            double s = 0.0;
#pragma unroll
            for (int t = 0; t < NQ; t++) s += a[k * NQ + t] * b[t * NQ + l];
            c[k * NQ + l] = s;
        }
}

template <int NQ>
__global__ void __launch_bounds__(256) k_ilu_factor(int nic, int njc, const double* __restrict__ jac1,
                                                    const double* __restrict__ dt, double psd, double sj,
                                                    double* __restrict__ ilu, unsigned* bar, int* err) {
    const int nlev = n_levels(nic, njc);
    const int gt = threadIdx.x * gridDim.x + blockIdx.x;
    const int nthreads = gridDim.x * blockDim.x;
    for (int L = 0; L < nlev; L++) {
        int i_lo, cnt;
        level_range(L, nic, njc, i_lo, cnt);
        for (int t = gt; t < cnt; t += nthreads) {
            const int i = i_lo + t, j = L - 2 * i;
            const size_t cell = (size_t)i * njc + j;
            double A[9][NQ * NQ];
            const int offs[9] = {0, 1, 2, 3, 4, 9, 10, 11, 12};
            for (int s = 0; s < 9; s++) {
                const int o = offs[s];
                const int ic = i + c_di[o], jc = j + c_dj[o];
                const bool in = ic >= 0 && ic < nic && jc >= 0 && jc < njc;
                for (int e = 0; e < NQ * NQ; e++) A[s][e] = in ? sj * jac1[(cell * NOFF + o) * NQ * NQ + e] : 0.0;
            }
            if (dt)
                for (int k = 0; k < NQ; k++) A[0][k * NQ + k] += psd / dt[cell * NQ + k];
            auto slot = [&](int o) { return o <= 4 ? o : o - 4; };  // 13-offset index -> A[] slot
            for (int a = 0; a < 4; a++) {
                const int lo = c_lo[a];
                const int ni = i + c_di[lo], nj = j + c_dj[lo];
                if (ni < 0 || ni >= nic || nj < 0 || nj >= njc) continue;
                const size_t ncell = (size_t)ni * njc + nj;
                double Lc[NQ * NQ];
                mat_mul<NQ>(A[slot(lo)], ilu + (ncell * NOFF + 0) * NQ * NQ, Lc);
                for (int e = 0; e < NQ * NQ; e++) ilu[(cell * NOFF + lo) * NQ * NQ + e] = Lc[e];
                for (int b = 0; b < 4; b++) {
                    const int uo = c_up[b];
                    const int di = c_di[lo] + c_di[uo], dj = c_dj[lo] + c_dj[uo];
                    if (di < -1 || di > 1 || dj < -1 || dj > 1) continue;
                    const int mi = i + di, mj = j + dj;
                    if (mi < 0 || mi >= nic || mj < 0 || mj >= njc) continue;
                    const int ro = off_index(di, dj);
                    double P[NQ * NQ];
                    mat_mul<NQ>(Lc, ilu + (ncell * NOFF + uo) * NQ * NQ, P);
                    for (int e = 0; e < NQ * NQ; e++) A[slot(ro)][e] -= P[e];
                }
            }
            double Di[NQ * NQ];
            if (!invert<NQ>(A[0], Di)) {
                atomicExch(err, 1);
                for (int e = 0; e < NQ * NQ; e++) Di[e] = 0.0;
            }
            for (int e = 0; e < NQ * NQ; e++) ilu[(cell * NOFF + 0) * NQ * NQ + e] = Di[e];
            for (int b = 0; b < 4; b++) {
                const int uo = c_up[b];
                for (int e = 0; e < NQ * NQ; e++) ilu[(cell * NOFF + uo) * NQ * NQ + e] = A[slot(uo)][e];
            }
        }
        if (!grid_barrier(bar, bar + 1, err)) return;
    }
}

// z = M^{-1} r (TRANS: M^{-T} r), both triangular sweeps in one cooperative kernel.
template <int NQ, bool TRANS>
__global__ void __launch_bounds__(256) k_ilu_solve(int nic, int njc, const double* __restrict__ ilu,
                                                   const double* __restrict__ r, double* __restrict__ z,
                                                   unsigned* bar, int* err) {
    const int nlev = n_levels(nic, njc);
    const int gt = threadIdx.x * gridDim.x + blockIdx.x;
    const int nthreads = gridDim.x * blockDim.x;
    // sweep 1 (increasing levels): L y = r, or U^T w = r
    for (int L = 0; L < nlev; L++) {
        int i_lo, cnt;
        level_range(L, nic, njc, i_lo, cnt);
        for (int t = gt; t < cnt; t += nthreads) {
            const int i = i_lo + t, j = L - 2 * i;
            const size_t cell = (size_t)i * njc + j;
            double v[NQ];
            for (int k = 0; k < NQ; k++) v[k] = r[cell * NQ + k];
            for (int a = 0; a < 4; a++) {
                const int lo = c_lo[a];
                const int ni = i + c_di[lo], nj = j + c_dj[lo];
                if (ni < 0 || ni >= nic || nj < 0 || nj >= njc) continue;
                const size_t nc = (size_t)ni * njc + nj;
                const double* y = z + nc * NQ;
                if (!TRANS) {
                    const double* B = ilu + (cell * NOFF + lo) * NQ * NQ;  // L_(cell, n)
                    for (int k = 0; k < NQ; k++)
                        for (int l = 0; l < NQ; l++) v[k] -= B[k * NQ + l] * y[l];
                } else {
                    // U^T: (U^T)_(cell, n) = U_(n, cell)^T, stored in row n at offset cell - n
                    const int uo = off_index(-c_di[lo], -c_dj[lo]);
                    const double* B = ilu + (nc * NOFF + uo) * NQ * NQ;
                    for (int k = 0; k < NQ; k++)
                        for (int l = 0; l < NQ; l++) v[k] -= B[l * NQ + k] * y[l];
                }
            }
            if (TRANS) {
                const double* Di = ilu + (cell * NOFF + 0) * NQ * NQ;  // D'^{-T}
                double w[NQ];
                for (int k = 0; k < NQ; k++) {
                    double s = 0.0;
                    for (int l = 0; l < NQ; l++) s += Di[l * NQ + k] * v[l];
                    w[k] = s;
                }
                for (int k = 0; k < NQ; k++) v[k] = w[k];
            }
            for (int k = 0; k < NQ; k++) z[cell * NQ + k] = v[k];
        }
        if (!grid_barrier(bar, bar + 1, err)) return;
    }
    // sweep 2 (decreasing levels): U x = y, or L^T v = w
    for (int L = nlev - 1; L >= 0; L--) {
        int i_lo, cnt;
        level_range(L, nic, njc, i_lo, cnt);
        for (int t = gt; t < cnt; t += nthreads) {
            const int i = i_lo + t, j = L - 2 * i;
            const size_t cell = (size_t)i * njc + j;
            double v[NQ];
            for (int k = 0; k < NQ; k++) v[k] = z[cell * NQ + k];
            for (int b = 0; b < 4; b++) {
                const int uo = c_up[b];
                const int mi = i + c_di[uo], mj = j + c_dj[uo];
                if (mi < 0 || mi >= nic || mj < 0 || mj >= njc) continue;
                const size_t mc = (size_t)mi * njc + mj;
                const double* x = z + mc * NQ;
                if (!TRANS) {
                    const double* B = ilu + (cell * NOFF + uo) * NQ * NQ;  // U_(cell, m)
                    for (int k = 0; k < NQ; k++)
                        for (int l = 0; l < NQ; l++) v[k] -= B[k * NQ + l] * x[l];
                } else {
                    // L^T: (L^T)_(cell, m) = L_(m, cell)^T, stored in row m at offset cell - m
                    const int lo = off_index(-c_di[uo], -c_dj[uo]);
                    const double* B = ilu + (mc * NOFF + lo) * NQ * NQ;
                    for (int k = 0; k < NQ; k++)
                        for (int l = 0; l < NQ; l++) v[k] -= B[l * NQ + k] * x[l];
                }
            }
            if (!TRANS) {
                const double* Di = ilu + (cell * NOFF + 0) * NQ * NQ;
                double w[NQ];
                for (int k = 0; k < NQ; k++) {
                    double s = 0.0;
                    for (int l = 0; l < NQ; l++) s += Di[k * NQ + l] * v[l];
                    w[k] = s;
                }
                for (int k = 0; k < NQ; k++) v[k] = w[k];
            }
            for (int k = 0; k < NQ; k++) z[cell * NQ + k] = v[k];
        }
        if (!grid_barrier(bar, bar + 1, err)) return;
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
        if (rc == ST_OK) rc = alloc_s(&x->lfac, x->ncell * NOFF * x->nq * x->nq);
        if (rc == ST_OK) rc = alloc_s(&x->bar_d, 4);
        if (rc == ST_OK) rc = alloc_s(&x->kz, n);
        if (rc == ST_OK) rc = alloc_s(&x->kw, n);
        if (rc == ST_OK) rc = alloc_s(&x->kr, n);
        if (rc == ST_OK) rc = alloc_s(&x->dq, n);
        if (rc == ST_OK) rc = alloc_s(&x->qsave, n);
        if (rc) return rc;
    }
    if (x->kv_m < m) {
        if (x->kv) cudaFree(x->kv);
        if (x->kh) cudaFree(x->kh);
        if (x->kpart) cudaFree(x->kpart);
        x->kv = nullptr; x->kh = nullptr; x->kpart = nullptr;
        rc = alloc_s(&x->kv, (size_t)(m + 1) * n);
        if (rc == ST_OK) rc = alloc_s(&x->kh, (size_t)(m + 2));
        if (rc == ST_OK) rc = alloc_s(&x->kpart, (size_t)(m + 2) * DOT_BLOCKS);
        if (rc) return rc;
        x->kv_m = m;
    }
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
                int rc = stx::run_jvp(x, x->kz, nullptr, x->kw, order);
                if (rc) return rc;
                if (nq == 5) k_extract<5><<<g, 256, 0, s>>>(nic, njc, cs, ci, cj, comp, x->kw, out);
                else k_extract<4><<<g, 256, 0, s>>>(nic, njc, cs, ci, cj, comp, x->kw, out);
            }
    ST_LAUNCH_CHECK("jacobian assembly");
    return ST_OK;
}

int assemble(st_ctx* x, int order) {
    int rc = ensure_solver(x, 1);
    if (rc) return rc;
    return assemble_into(x, order, x->jac);
}

// Operator Jacobian (order `order`) and, for the preconditioner, the
// first-order Jacobian (reusing the operator when it is first order).
int assemble_pair(st_ctx* x, int order) {
    int rc = assemble(x, order);
    if (rc) return rc;
    if (order == 1) {
        x->jac1_is_jac = true;
        return ST_OK;
    }
    x->jac1_is_jac = false;
    return assemble_into(x, 1, x->jac1);
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
    ST_LAUNCH_CHECK("spmv");
    return ST_OK;
}

// cooperative launch of an ILU kernel over one block per SM
int coop_launch(st_ctx* x, void* fn, void** args) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, x->device);
    ST_CUDA(cudaMemsetAsync(x->bar_d, 0, 2 * sizeof(unsigned), x->stream));
    ST_CUDA(cudaLaunchCooperativeKernel(fn, dim3(sms), dim3(256), args, 0, x->stream));
    return ST_OK;
}

int check_err(st_ctx* x, const char* what) {
    int err = 0;
    ST_CUDA(cudaMemcpyAsync(&err, x->err_d, sizeof(int), cudaMemcpyDeviceToHost, x->stream));
    ST_CUDA(cudaStreamSynchronize(x->stream));
    if (err == 2) return fail(ST_ERR_TIMEOUT, std::string(what) + ": grid barrier timed out");
    if (err) return fail(ST_ERR_NONFINITE, std::string(what) + ": singular diagonal block");
    return ST_OK;
}

int factor_M(st_ctx* x, const LinOp& op) {
    int nic = x->c.ni - 1, njc = x->c.nj - 1;
    ST_CUDA(cudaMemsetAsync(x->err_d, 0, sizeof(int), x->stream));
    const double* j1 = x->jac1_is_jac ? x->jac : x->jac1;
    const double* pdt = op.pdt;
    double psd = op.psd, sj = op.sj;
    double* ilu = x->lfac;
    unsigned* bar = x->bar_d;
    int* err = x->err_d;
    void* args[] = {&nic, &njc, (void*)&j1, (void*)&pdt, &psd, &sj, &ilu, &bar, &err};
    int rc = coop_launch(x, x->nq == 5 ? (void*)k_ilu_factor<5> : (void*)k_ilu_factor<4>, args);
    if (rc) return rc;
    return check_err(x, "ILU factorisation");
}

int apply_M(st_ctx* x, const LinOp& op, const double* in, double* out) {
    int nic = x->c.ni - 1, njc = x->c.nj - 1;
    const double* ilu = x->lfac;
    unsigned* bar = x->bar_d;
    int* err = x->err_d;
    void* args[] = {&nic, &njc, (void*)&ilu, (void*)&in, &out, &bar, &err};
    void* fn;
    if (x->nq == 5) fn = op.trans ? (void*)k_ilu_solve<5, true> : (void*)k_ilu_solve<5, false>;
    else fn = op.trans ? (void*)k_ilu_solve<4, true> : (void*)k_ilu_solve<4, false>;
    return coop_launch(x, fn, args);
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

// Right-preconditioned restarted GMRES (classical Gram-Schmidt, repeated
// once) for op * xsol = b; xsol holds the initial guess.
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
            rc = apply_M(x, op, V + (size_t)k * n, x->kz);
            if (rc) return rc;
            rc = apply_A(x, op, x->kz, x->kw);
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
        // y = H^{-1} g, x += M^{-1} V y
        for (int i = k - 1; i >= 0; i--) {
            double sum = gv[i];
            for (int l = i + 1; l < k; l++) sum -= H[(size_t)i * m + l] * y[l];
            y[i] = sum / H[(size_t)i * m + i];
        }
        ST_CUDA(cudaMemcpyAsync(x->kh, y.data(), k * 8, cudaMemcpyHostToDevice, s));
        k_combine<<<g, 256, 0, s>>>(V, k, n, x->kh, x->kw);
        rc = apply_M(x, op, x->kw, x->kz);
        if (rc) return rc;
        k_axpby<<<g, 256, 0, s>>>(n, 1.0, x->kz, 1.0, xsol);
        ST_LAUNCH_CHECK("gmres update");
        if (conv) break;
    }
    ST_CUDA(cudaStreamSynchronize(s));
    rc = check_err(x, "ILU solve");
    if (rc) return rc;
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
    for (const auto& b : x->bcs)
        if (b.type == ST_BC_PERIODIC || b.type == ST_BC_WAKE)
            return fail(ST_ERR_UNSUPPORTED, "st_jacobian_assemble: periodic/wake boundaries couple distant cells");
    int rc = assemble_pair(x, lhs ? x->c.lhs_order : x->c.order);
    if (rc) return rc;
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

int st_jacobian_blocks(st_ctx* x, double* blocks_host) {
    if (!x || !blocks_host) return fail(ST_ERR_ARG, "st_jacobian_blocks: null argument");
    if (!x->jac) return fail(ST_ERR_ARG, "st_jacobian_blocks: no Jacobian assembled");
    ST_CUDA(cudaMemcpyAsync(blocks_host, x->jac, x->ncell * NOFF * x->nq * x->nq * 8, cudaMemcpyDeviceToHost, x->stream));
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
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
    for (const auto& b : x->bcs)
        if (b.type == ST_BC_PERIODIC || b.type == ST_BC_WAKE)
            return fail(ST_ERR_UNSUPPORTED, "st_solve: periodic/wake boundaries couple distant cells");
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
        // near round-off (below 1e-9 of the initial residual) growth is noise, not divergence
        if (!std::isfinite(rt) || (rt > p->reject_factor * rn && rt > 1e-9 * r0)) {
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
        k_prim_adj<5><<<grid_for(x->ncell), 256, 0, s>>>(dc, x->q, x->P, x->Pbar, grad_dev);
    } else {
        k_prim<double, 4><<<grid_for(x->ncell), 256, 0, s>>>(dc, x->q, x->P);
        k_bc_taped<4><<<1, 1024, 0, s>>>(dc, x->P, x->tape);
        k_cf_adj<<<(2 * (nic + 2) + 255) / 256, 256, 0, s>>>(dc, x->cf, x->c.mu_inf / qinf, x->Pbar);
        k_bc_adj<4><<<1, 1024, 0, s>>>(dc, x->P, x->tape, x->Pbar);
        k_prim_adj<4><<<grid_for(x->ncell), 256, 0, s>>>(dc, x->q, x->P, x->Pbar, grad_dev);
    }
    ST_LAUNCH_CHECK("cf gradient");
    ST_CUDA(cudaStreamSynchronize(s));
    return ST_OK;
}

int st_adjoint_solve_device(st_ctx* x, const double* b_dev, double* psi_dev, double cfl_prec, int krylov_m, int maxit,
                            double rtol, st_solve_stats* stats) {
    if (!x || !b_dev || !psi_dev) return fail(ST_ERR_ARG, "st_adjoint_solve_device: null argument");
    if (krylov_m < 1 || krylov_m > 500 || maxit < 1) return fail(ST_ERR_ARG, "st_adjoint_solve_device: krylov sizes");
    for (const auto& b : x->bcs)
        if (b.type == ST_BC_PERIODIC || b.type == ST_BC_WAKE)
            return fail(ST_ERR_UNSUPPORTED, "st_adjoint_solve_device: periodic/wake boundaries couple distant cells");
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
    for (const auto& b : x->bcs)
        if (b.type == ST_BC_PERIODIC || b.type == ST_BC_WAKE)
            return fail(ST_ERR_UNSUPPORTED, "st_tangent_solve_device: periodic/wake boundaries couple distant cells");
    int rc = assemble_pair(x, x->c.order);
    if (rc) return rc;
    rc = stx::run_dt(x, cfl_prec);
    if (rc) return rc;
    LinOp op{false, 0.0, 1.0, nullptr, -1.0, x->dt};
    rc = factor_M(x, op);
    if (rc) return rc;
    return gmres(x, op, b_dev, dq_dev, krylov_m, maxit, rtol, stats);
}

}  // extern "C"
