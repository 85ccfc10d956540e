// Partner blocks of the implicit solver's Jacobian: the coupling that the
// non-local boundary copies add to the 13-point stencil (st_solver.cu
// launches these kernels).
//
// Self-contained apart from the C header's boundary types, so that the same
// source also compiles as plain C++ on a host (the qualifiers and the thread
// indices then come from the includer) for CPU checks of its index arithmetic.
#pragma once
#include <cstddef>

#include "../../include/structured_gb300.h"

namespace st {

// ---------------------------------------------------------------------------
// Three families of ghosts are copies of cells elsewhere in the grid:
//   FAM_WAKE   wake cut (bc.cpp:224-263): the bottom ghost below column b is a
//              copy of cell (nic-1-b, 0);
//   FAM_LEFT   periodic in i (bc.cpp:329-365): the ghost left of row b is a
//              copy of cell (nic-1, b);
//   FAM_RIGHT  the ghost right of row b is a copy of cell (0, b).
// Ghost b of a family enters four residual rows: at distance 0 from its
// boundary the rows at line positions b-1, b, b+1, at distance 1 the row at b
// (wake: rows (b-1,0), (b,0), (b+1,0), (b,1); left: (0,b-1), (0,b), (0,b+1),
// (1,b)).  A corner ghost that copies a wall ghost of the far column reaches
// only rows already in these windows.  Partner slot t of line position p holds
//   W_f[p][t] = d R(row f(p, t)) / d q(source of ghost p - wslot_d(t)),
// the part of that block carried by the copy.  The regular 13-point blocks
// come from a colouring pass whose JVPs hold every copy's tangent at zero; a
// partner pass seeds the sources of the ghosts b = k mod 3 of one family (their
// windows, three positions wide, share no row) and reads the difference of a
// full and a frozen JVP, which is exactly the part carried by the copies.
// ---------------------------------------------------------------------------
constexpr int NWS = 4;
enum { FAM_WAKE = 0, FAM_LEFT = 1, FAM_RIGHT = 2, NFAM = 3 };

__host__ __device__ inline int wslot_j(int t) { return t == 3 ? 1 : 0; }     // distance from the boundary
__host__ __device__ inline int wslot_d(int t) { return t == 3 ? 0 : t - 1; }  // row position - ghost position
__host__ __device__ inline int fam_len(int f, int nic, int njc) { return f == FAM_WAKE ? nic : njc; }

// cell index i * njc + j of the row of slot t at line position p
__host__ __device__ inline size_t fam_row(int f, int p, int t, int nic, int njc) {
    const int l = wslot_j(t);
    const int i = f == FAM_WAKE ? p : (f == FAM_LEFT ? l : nic - 1 - l);
    const int j = f == FAM_WAKE ? l : p;
    return (size_t)i * njc + j;
}

// cell index of the cell that ghost b of family f copies
__host__ __device__ inline size_t fam_src(int f, int b, int nic, int njc) {
    if (f == FAM_WAKE) return (size_t)(nic - 1 - b) * njc;
    if (f == FAM_LEFT) return (size_t)(nic - 1) * njc + b;
    return (size_t)b;
}

// Ghost masks of the boundary list, in order: mask[f][b] = 1 if ghost b of
// family f is a copy (mask[FAM_WAKE] has nic entries, the others njc);
// on[f] = 1 if the family occurs.  Returns 0, or ST_ERR_UNSUPPORTED with *why
// set for lists this layout cannot hold: a wake cut off the bottom face or on
// a corner ghost, periodic boundaries on the bottom/top faces or not covering
// every row, a wake cut together with periodic boundaries, fewer than two
// cells across the grid.
inline int partner_masks(int nic, int njc, const st_bc* bcs, int nbc, int* mask_wake, int* mask_left,
                         int* mask_right, int* on, const char** why) {
    for (int f = 0; f < NFAM; f++) on[f] = 0;
    for (int i = 0; i < nic; i++) mask_wake[i] = 0;
    for (int j = 0; j < njc; j++) mask_left[j] = mask_right[j] = 0;
    for (int n = 0; n < nbc; n++) {
        const st_bc& b = bcs[n];
        if (b.type != ST_BC_WAKE && b.type != ST_BC_PERIODIC) continue;
        const bool bt = b.face == ST_FACE_BOTTOM || b.face == ST_FACE_TOP;
        const int end = b.end >= 0 ? b.end : (bt ? nic : njc) + 2 + b.end;
        if (b.start > end) continue;
        if (b.type == ST_BC_WAKE) {
            if (b.face != ST_FACE_BOTTOM) { *why = "wake cut off the bottom face"; return ST_ERR_UNSUPPORTED; }
            if (b.start < 1 || end > nic) { *why = "wake range on a corner ghost"; return ST_ERR_UNSUPPORTED; }
            for (int ip = b.start; ip <= end; ip++) {
                mask_wake[ip - 1] = 1;
                mask_wake[nic - ip] = 1;
            }
            on[FAM_WAKE] = 1;
        } else {
            if (bt) { *why = "periodic boundaries on the bottom/top faces"; return ST_ERR_UNSUPPORTED; }
            if (b.start > 1 || end < njc) { *why = "periodic range not covering every row"; return ST_ERR_UNSUPPORTED; }
            for (int j = 0; j < njc; j++) mask_left[j] = mask_right[j] = 1;
            on[FAM_LEFT] = on[FAM_RIGHT] = 1;
        }
    }
    if (on[FAM_WAKE] && on[FAM_LEFT]) { *why = "a wake cut together with periodic boundaries"; return ST_ERR_UNSUPPORTED; }
    if ((on[FAM_WAKE] || on[FAM_LEFT]) && (nic < 2 || njc < 2)) { *why = "fewer than two cells across"; return ST_ERR_UNSUPPORTED; }
    return 0;
}

// v = 0 except unit `comp` at the sources of the family's ghosts b = k mod 3
// (v zeroed beforehand); one thread per ghost
template <int NQ>
__global__ void k_partner_seed(int f, int nic, int njc, const int* __restrict__ mask, int k, int comp,
                               double* __restrict__ v) {
    const int n = fam_len(f, nic, njc);
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x)
        if (mask[b] && b % 3 == k) v[fam_src(f, b, nic, njc) * NQ + comp] = 1.0;
}

// W column `comp` of the slots whose ghost was seeded: full - frozen JVP
template <int NQ>
__global__ void k_partner_extract(int f, int nic, int njc, const int* __restrict__ mask, int k, int comp,
                                  const double* __restrict__ jv_full, const double* __restrict__ jv_frozen,
                                  double* __restrict__ W) {
    const int len = fam_len(f, nic, njc), n = len * NWS;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int p = t / NWS, slot = t % NWS;
        const int b = p - wslot_d(slot);
        if (b < 0 || b >= len || !mask[b] || b % 3 != k) continue;
        const size_t row = fam_row(f, p, slot, nic, njc);
        double* w = W + (size_t)t * NQ * NQ;
#pragma unroll
        for (int kk = 0; kk < NQ; kk++) w[kk * NQ + comp] = jv_full[row * NQ + kk] - jv_frozen[row * NQ + kk];
    }
}

// Index of offset (di, dj) in the 13-point block row of the Jacobian
// ((0,0), (-1,0), (1,0), (0,-1), (0,1), (-2,0), (2,0), (0,-2), (0,2),
// (-1,-1), (-1,1), (1,-1), (1,1)); -1 outside it.
__host__ __device__ inline int off13(int di, int dj) {
    if (di == 0) return dj == 0 ? 0 : dj == -1 ? 3 : dj == 1 ? 4 : dj == -2 ? 7 : dj == 2 ? 8 : -1;
    if (dj == 0) return di == -1 ? 1 : di == 1 ? 2 : di == -2 ? 5 : di == 2 ? 6 : -1;
    if (di == -1) return dj == -1 ? 9 : dj == 1 ? 10 : -1;
    if (di == 1) return dj == -1 ? 11 : dj == 1 ? 12 : -1;
    return -1;
}

// Block-row offset of the partner of slot t at line position p when its
// source lies in the row's 3x3 neighbourhood (the ILU(0) pattern), else -1.
// Periodic boundaries two cells across put every partner there.
__host__ __device__ inline int fold_offset(int f, int p, int t, int nic, int njc) {
    const int b = p - wslot_d(t);
    const size_t row = fam_row(f, p, t, nic, njc), src = fam_src(f, b, nic, njc);
    const int di = (int)(src / njc) - (int)(row / njc), dj = (int)(src % njc) - (int)(row % njc);
    return (di >= -1 && di <= 1 && dj >= -1 && dj <= 1) ? off13(di, dj) : -1;
}

// jac[row][o] += W[p][t] for the partners inside the ILU(0) pattern, so that
// the preconditioner sees them; one thread per line position (its rows are
// distinct from every other position's).  jac: [ncell][13][NQ][NQ].
template <int NQ>
__global__ void k_partner_fold(int f, int nic, int njc, const double* __restrict__ W, double* __restrict__ jac) {
    const int len = fam_len(f, nic, njc);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < len; p += gridDim.x * blockDim.x) {
        for (int slot = 0; slot < NWS; slot++) {
            const int b = p - wslot_d(slot);
            if (b < 0 || b >= len) continue;
            const int o = fold_offset(f, p, slot, nic, njc);
            if (o < 0) continue;
            double* dst = jac + (fam_row(f, p, slot, nic, njc) * 13 + o) * NQ * NQ;
            const double* w = W + ((size_t)p * NWS + slot) * NQ * NQ;
#pragma unroll
            for (int e = 0; e < NQ * NQ; e++) dst[e] += w[e];
        }
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

// y += sj * W x (or W^T x) for one family, after k_spmv on the same stream.
// Forward: one thread per line position writes its two rows; transposed: one
// thread per ghost gathers into the ghost's source cell (sources are
// distinct), so neither needs atomics.
template <int NQ, bool TRANS>
__global__ void k_partner_apply(int f, int nic, int njc, const double* __restrict__ W,
                                const double* __restrict__ x, double* __restrict__ y, double sj) {
    const int len = fam_len(f, nic, njc);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < len; p += gridDim.x * blockDim.x) {
        if (!TRANS) {
            double a0[NQ], a1[NQ];
#pragma unroll
            for (int kk = 0; kk < NQ; kk++) { a0[kk] = 0.0; a1[kk] = 0.0; }
#pragma unroll
            for (int slot = 0; slot < NWS; slot++) {
                const int b = p - wslot_d(slot);
                if (b < 0 || b >= len) continue;
                const double* w = W + ((size_t)p * NWS + slot) * NQ * NQ;
                const double* xs = x + fam_src(f, b, nic, njc) * NQ;
                if (wslot_j(slot)) block_mv<NQ, false>(w, xs, a1);
                else block_mv<NQ, false>(w, xs, a0);
            }
            double* y0 = y + fam_row(f, p, 0, nic, njc) * NQ;
            double* y1 = y + fam_row(f, p, 3, nic, njc) * NQ;
#pragma unroll
            for (int kk = 0; kk < NQ; kk++) { y0[kk] += sj * a0[kk]; y1[kk] += sj * a1[kk]; }
        } else {
            const int b = p;  // this thread's ghost
            double acc[NQ];
#pragma unroll
            for (int kk = 0; kk < NQ; kk++) acc[kk] = 0.0;
#pragma unroll
            for (int slot = 0; slot < NWS; slot++) {
                const int r = b + wslot_d(slot);
                if (r < 0 || r >= len) continue;
                block_mv<NQ, true>(W + ((size_t)r * NWS + slot) * NQ * NQ, x + fam_row(f, r, slot, nic, njc) * NQ,
                                   acc);
            }
            double* ys = y + fam_src(f, b, nic, njc) * NQ;
#pragma unroll
            for (int kk = 0; kk < NQ; kk++) ys[kk] += sj * acc[kk];
        }
    }
}

// ---------------------------------------------------------------------------
// Wake strip: a second preconditioner level for the wake cut, whose partner
// blocks lie outside the ILU(0) pattern.  The strip is rows 0 and 1 of every
// column within one of a wake ghost column (it holds each wake partner's row
// and source).  After the ILU sweep z = M^-1 v, the correction
//   z_S += A_SS^-1 (v - P z)_S,   P = psd D + sj (J1 + W1),
// with A_SS the strip's block of P (dense, inverted on the host once per
// factorisation), solves the strip's coupling exactly.
// ---------------------------------------------------------------------------
__host__ __device__ inline int off_di(int o) {
    return o == 1 || o == 9 || o == 10 ? -1 : o == 2 || o == 11 || o == 12 ? 1 : o == 5 ? -2 : o == 6 ? 2 : 0;
}
__host__ __device__ inline int off_dj(int o) {
    return o == 3 || o == 9 || o == 11 ? -1 : o == 4 || o == 10 || o == 12 ? 1 : o == 7 ? -2 : o == 8 ? 2 : 0;
}

// strip cells in increasing cell order into cells[] (room for 2 nic); returns the count
inline int strip_cells(int nic, int njc, const int* mask_wake, int* cells) {
    int n = 0;
    for (int i = 0; i < nic; i++) {
        const bool on = mask_wake[i] || (i > 0 && mask_wake[i - 1]) || (i + 1 < nic && mask_wake[i + 1]);
        if (!on) continue;
        for (int j = 0; j < 2 && j < njc; j++) cells[n++] = i * njc + j;
    }
    return n;
}

// index of cell c in the sorted strip, -1 if absent
__host__ __device__ inline int strip_find(int ns, const int* cells, long c) {
    int lo = 0, hi = ns - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) / 2;
        if (cells[mid] == c) return mid;
        if (cells[mid] < c) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// Dense strip block A (n = ns nq, row-major) of psd D + sj (J1 + W1): jac_s the
// strip cells' 13 regular blocks [ns][13][nq][nq], dt_s their time steps
// [ns][nq] (NULL: no D term), W1 the first-order wake partners [nic][4][nq][nq].
inline void strip_matrix(int nic, int njc, int nq, int ns, const int* cells, const double* jac_s, const double* dt_s,
                         const double* W1, double psd, double sj, double* A) {
    const int n = ns * nq;
    for (long e = 0; e < (long)n * n; e++) A[e] = 0.0;
    auto add = [&](int a, int b, const double* blk, double f) {
        for (int k = 0; k < nq; k++)
            for (int l = 0; l < nq; l++) A[(long)(a * nq + k) * n + b * nq + l] += f * blk[k * nq + l];
    };
    for (int a = 0; a < ns; a++) {
        const int ri = cells[a] / njc, rj = cells[a] % njc;
        if (dt_s)
            for (int k = 0; k < nq; k++) A[(long)(a * nq + k) * n + a * nq + k] += psd / dt_s[a * nq + k];
        for (int o = 0; o < 13; o++) {
            const int ci = ri + off_di(o), cj = rj + off_dj(o);
            if (ci < 0 || ci >= nic || cj < 0 || cj >= njc) continue;
            const int b = strip_find(ns, cells, (long)ci * njc + cj);
            if (b >= 0) add(a, b, jac_s + ((size_t)a * 13 + o) * nq * nq, sj);
        }
        for (int t = 0; t < NWS; t++) {
            if (wslot_j(t) != rj) continue;
            const int g = ri - wslot_d(t);
            if (g < 0 || g >= nic) continue;
            const int b = strip_find(ns, cells, (long)fam_src(FAM_WAKE, g, nic, njc));
            if (b >= 0) add(a, b, W1 + ((size_t)ri * NWS + t) * nq * nq, sj);
        }
    }
}

// inv = A^-1 by Gauss-Jordan elimination with partial pivoting (A is
// overwritten); returns 0 if a pivot vanishes
inline int dense_invert(int n, double* A, double* inv) {
    for (long e = 0; e < (long)n * n; e++) inv[e] = 0.0;
    for (int i = 0; i < n; i++) inv[(long)i * n + i] = 1.0;
    for (int c = 0; c < n; c++) {
        int p = c;
        double best = A[(long)c * n + c] < 0 ? -A[(long)c * n + c] : A[(long)c * n + c];
        for (int r = c + 1; r < n; r++) {
            const double v = A[(long)r * n + c] < 0 ? -A[(long)r * n + c] : A[(long)r * n + c];
            if (v > best) { best = v; p = r; }
        }
        if (!(best > 0.0)) return 0;
        if (p != c)
            for (int l = 0; l < n; l++) {
                double t = A[(long)c * n + l]; A[(long)c * n + l] = A[(long)p * n + l]; A[(long)p * n + l] = t;
                t = inv[(long)c * n + l]; inv[(long)c * n + l] = inv[(long)p * n + l]; inv[(long)p * n + l] = t;
            }
        const double d = 1.0 / A[(long)c * n + c];
        for (int l = 0; l < n; l++) { A[(long)c * n + l] *= d; inv[(long)c * n + l] *= d; }
        // columns < c of A are already zero outside their pivot rows; the rows
        // are independent here, so the host's cores share them
#pragma omp parallel for schedule(static)
        for (int r = 0; r < n; r++) {
            if (r == c) continue;
            const double f = A[(long)r * n + c];
            if (f == 0.0) continue;
            for (int l = c; l < n; l++) A[(long)r * n + l] -= f * A[(long)c * n + l];
            for (int l = 0; l < n; l++) inv[(long)r * n + l] -= f * inv[(long)c * n + l];
        }
    }
    return 1;
}

// the strip cells' regular blocks and time steps, compacted for the host
template <int NQ>
__global__ void k_strip_gather(int ns, const int* __restrict__ cells, const double* __restrict__ jac,
                               const double* __restrict__ dt, double* __restrict__ jac_s, double* __restrict__ dt_s) {
    const size_t per = 13 * NQ * NQ, n = (size_t)ns * per;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const size_t a = e / per, w = e % per;
        jac_s[e] = jac[(size_t)cells[a] * per + w];
        if (dt && w < NQ) dt_s[a * NQ + w] = dt[(size_t)cells[a] * NQ + w];
    }
}

// res = (v - P z) on the strip, one thread per strip cell
template <int NQ>
__global__ void k_strip_residual(int nic, int njc, int ns, const int* __restrict__ cells,
                                 const double* __restrict__ jac, const double* __restrict__ W1,
                                 const double* __restrict__ dt, double psd, double sj, const double* __restrict__ v,
                                 const double* __restrict__ z, double* __restrict__ res) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < ns; a += gridDim.x * blockDim.x) {
        const size_t r = (size_t)cells[a];
        const int ri = (int)(r / njc), rj = (int)(r % njc);
        double acc[NQ];
#pragma unroll
        for (int k = 0; k < NQ; k++) acc[k] = 0.0;
        for (int o = 0; o < 13; o++) {
            const int ci = ri + off_di(o), cj = rj + off_dj(o);
            if (ci < 0 || ci >= nic || cj < 0 || cj >= njc) continue;
            block_mv<NQ, false>(jac + (r * 13 + o) * NQ * NQ, z + ((size_t)ci * njc + cj) * NQ, acc);
        }
        for (int t = 0; t < NWS; t++) {
            if (wslot_j(t) != rj) continue;
            const int g = ri - wslot_d(t);
            if (g < 0 || g >= nic) continue;
            block_mv<NQ, false>(W1 + ((size_t)ri * NWS + t) * NQ * NQ, z + fam_src(FAM_WAKE, g, nic, njc) * NQ, acc);
        }
#pragma unroll
        for (int k = 0; k < NQ; k++) {
            double pz = sj * acc[k];
            if (dt) pz += psd * z[r * NQ + k] / dt[r * NQ + k];
            res[(size_t)a * NQ + k] = v[r * NQ + k] - pz;
        }
    }
}

// z_S += Ainv res, one thread per strip unknown (rows of Ainv are distinct)
template <int NQ>
__global__ void k_strip_update(int ns, const int* __restrict__ cells, const double* __restrict__ Ainv,
                               const double* __restrict__ res, double* __restrict__ z) {
    const int n = ns * NQ;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
        double s = 0.0;
        const double* row = Ainv + (size_t)m * n;
        for (int l = 0; l < n; l++) s += row[l] * res[l];
        z[(size_t)cells[m / NQ] * NQ + m % NQ] += s;
    }
}

}  // namespace st
