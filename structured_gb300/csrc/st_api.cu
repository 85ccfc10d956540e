// C ABI: context lifecycle, state transfer, residual, time step, norms, skin
// friction, forward-mode JVP and diagnostics.  See include/structured_gb300.h
// for the reference member each entry point replaces.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "st_context.h"
#include "st_kernels.cuh"
#include "st_tile.cuh"

using namespace st;

namespace {
thread_local std::string g_last_error;
}

namespace stx {
int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char* where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return ST_ERR_CUDA;
}
}  // namespace stx

using stx::fail;
using stx::grid_for;

namespace {

// ---------------------------------------------------------------------------
// host-side mesh setup
// ---------------------------------------------------------------------------
// Mesh::calc_metrics (src/utils/mesh.cpp:172-205), same operation order.
void host_metrics(st_ctx* x) {
    const int ni = x->c.ni, nj = x->c.nj, nic = ni - 1, njc = nj - 1;
    auto X = [&](int i, int j) { return x->xv[(size_t)i * nj + j]; };
    auto Y = [&](int i, int j) { return x->yv[(size_t)i * nj + j]; };
    x->nchi.assign((size_t)ni * njc * 2, 0.0);
    x->neta.assign((size_t)nic * nj * 2, 0.0);
    x->vol.assign((size_t)nic * njc, 0.0);
    x->ds_min.assign((size_t)nic * njc, 0.0);
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < nj; j++) {
            double rx = X(i + 1, j) - X(i, j), ry = Y(i + 1, j) - Y(i, j);
            x->neta[((size_t)i * nj + j) * 2 + 0] = -ry;
            x->neta[((size_t)i * nj + j) * 2 + 1] = rx;
        }
    for (int i = 0; i < ni; i++)
        for (int j = 0; j < njc; j++) {
            double rx = X(i, j + 1) - X(i, j), ry = Y(i, j + 1) - Y(i, j);
            x->nchi[((size_t)i * njc + j) * 2 + 0] = ry;
            x->nchi[((size_t)i * njc + j) * 2 + 1] = -rx;
        }
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < njc; j++) {
            // reta = (x(i+1,j)-x(i,j), ...), rchi = (x(i,j+1)-x(i,j), ...)
            double re0 = X(i + 1, j) - X(i, j), re1 = Y(i + 1, j) - Y(i, j);
            double rc0 = X(i, j + 1) - X(i, j), rc1 = Y(i, j + 1) - Y(i, j);
            double re0t = X(i + 1, j + 1) - X(i, j + 1), re1t = Y(i + 1, j + 1) - Y(i, j + 1);
            double rc0r = X(i + 1, j + 1) - X(i + 1, j), rc1r = Y(i + 1, j + 1) - Y(i + 1, j);
            size_t cidx = (size_t)i * njc + j;
            x->vol[cidx] = 0.5 * (re0 * rc1 - rc0 * re1 + re0t * rc1r - rc0r * re1t);
            double ne0 = x->neta[((size_t)i * nj + j) * 2], ne1 = x->neta[((size_t)i * nj + j) * 2 + 1];
            double nc0 = x->nchi[((size_t)i * njc + j) * 2], nc1 = x->nchi[((size_t)i * njc + j) * 2 + 1];
            double dse = std::sqrt(ne0 * ne0 + ne1 * ne1);
            double dsc = std::sqrt(nc0 * nc0 + nc1 * nc1);
            x->ds_min[cidx] = std::min(dse, dsc);
        }
}

// Per-face geometry records: normal, unit normal and half length (flux.cpp:
// 95-99, 127) and the Green-Gauss weights of the face gradient
// (mesh.cpp:36-131, including its boundary-face special cases), folded so
// grad = wL qL + wR qR + wP (qP1+qP2) + wM (qM1+qM2).
void host_geometry(st_ctx* x, std::vector<double>& gi, std::vector<double>& gj) {
    const int ni = x->c.ni, nj = x->c.nj, nic = ni - 1, njc = nj - 1;
    auto NC = [&](int i, int j, int k) { return x->nchi[((size_t)i * njc + j) * 2 + k]; };
    auto NE = [&](int i, int j, int k) { return x->neta[((size_t)i * nj + j) * 2 + k]; };
    auto V = [&](int i, int j) { return x->vol[(size_t)i * njc + j]; };
    gi.assign((size_t)ni * njc * NGEO, 0.0);
    gj.assign((size_t)nic * nj * NGEO, 0.0);
    auto unit = [](double* g, double nx, double ny) {
        g[G_NX] = nx; g[G_NY] = ny;
        double dr = std::sqrt(nx * nx + ny * ny);
        g[G_R1] = nx / dr; g[G_R2] = ny / dr; g[G_AJ] = 0.5 * dr;
    };
    for (int i = 0; i < ni; i++)
        for (int j = 0; j < njc; j++) {
            double nt[2], nb[2], nl[2], nr[2], vol;
            if (i == 0) {
                vol = V(i, j);
                for (int k = 0; k < 2; k++) { nt[k] = NE(i, j + 1, k); nb[k] = NE(i, j, k); nr[k] = 0.5 * (NC(i, j, k) + NC(i + 1, j, k)); nl[k] = NC(i, j, k); }
            } else if (i == ni - 1) {
                vol = V(i - 1, j);
                for (int k = 0; k < 2; k++) { nt[k] = NE(i - 1, j + 1, k); nb[k] = NE(i - 1, j, k); nr[k] = NC(i, j, k); nl[k] = 0.5 * (NC(i, j, k) + NC(i - 1, j, k)); }
            } else {
                vol = 0.5 * (V(i, j) + V(i - 1, j));
                for (int k = 0; k < 2; k++) {
                    nt[k] = 0.5 * (NE(i, j + 1, k) + NE(i - 1, j + 1, k)); nb[k] = 0.5 * (NE(i, j, k) + NE(i - 1, j, k));
                    nr[k] = 0.5 * (NC(i, j, k) + NC(i + 1, j, k)); nl[k] = 0.5 * (NC(i, j, k) + NC(i - 1, j, k));
                }
            }
            double* g = &gi[((size_t)i * njc + j) * NGEO];
            unit(g, NC(i, j, 0), NC(i, j, 1));
            for (int k = 0; k < 2; k++) {
                g[G_WLX + k] = (0.25 * nt[k] - 0.25 * nb[k] - nl[k]) / vol;
                g[G_WRX + k] = (0.25 * nt[k] - 0.25 * nb[k] + nr[k]) / vol;
                g[G_WPX + k] = 0.25 * nt[k] / vol;
                g[G_WMX + k] = -0.25 * nb[k] / vol;
            }
        }
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < nj; j++) {
            double nt[2], nb[2], nl[2], nr[2], vol;
            if (j == 0) {
                vol = V(i, j);
                for (int k = 0; k < 2; k++) { nt[k] = 0.5 * (NE(i, j, k) + NE(i, j + 1, k)); nb[k] = NE(i, j, k); nl[k] = NC(i, j, k); nr[k] = NC(i + 1, j, k); }
            } else if (j == nj - 1) {
                for (int k = 0; k < 2; k++) { nt[k] = NE(i, j, k); nb[k] = 0.5 * (NE(i, j, k) + NE(i, j - 1, k)); nl[k] = NC(i, j - 1, k); nr[k] = NC(i + 1, j - 1, k); }
                vol = V(i, j - 1);
            } else {
                for (int k = 0; k < 2; k++) {
                    nt[k] = 0.5 * (NE(i, j, k) + NE(i, j + 1, k)); nb[k] = 0.5 * (NE(i, j, k) + NE(i, j - 1, k));
                    nl[k] = 0.5 * (NC(i, j, k) + NC(i, j - 1, k)); nr[k] = 0.5 * (NC(i + 1, j, k) + NC(i + 1, j - 1, k));
                }
                vol = 0.5 * (V(i, j) + V(i, j - 1));
            }
            double* g = &gj[((size_t)i * nj + j) * NGEO];
            unit(g, NE(i, j, 0), NE(i, j, 1));
            for (int k = 0; k < 2; k++) {
                g[G_WRX + k] = (nt[k] + 0.25 * nr[k] - 0.25 * nl[k]) / vol;   // top cell (R)
                g[G_WLX + k] = (-nb[k] + 0.25 * nr[k] - 0.25 * nl[k]) / vol;  // bottom cell (L)
                g[G_WPX + k] = 0.25 * nr[k] / vol;
                g[G_WMX + k] = -0.25 * nl[k] / vol;
            }
        }
}

// Wall distance: nearest point on any bottom no-slip wall segment, brute force
// over segments staged in shared memory.
// Distance from each cell centre to the nearest no-slip wall segment (exact
// minimum over every segment).  Segments come in chunks of WD_CHUNK in wall
// order with the chunk's bounding box; a chunk is scanned only if the squared
// distance from the point to its box (a lower bound for every segment in it,
// with a relative margin for rounding) does not exceed the best so far, so the
// minimum is the brute-force one while most chunks are skipped.  The first
// chunk scanned is the one holding the cell's own column when that column is
// on the wall (a tight starting bound for body-fitted grids).
constexpr int WD_CHUNK = 32;
__device__ inline double seg_dist2(double px, double py, double x0, double y0, double x1, double y1) {
    const double ax = x1 - x0, ay = y1 - y0;
    const double wx = px - x0, wy = py - y0;
    const double l2 = ax * ax + ay * ay;
    double t = l2 > 0.0 ? (wx * ax + wy * ay) / l2 : 0.0;
    t = fmin(1.0, fmax(0.0, t));
    const double dx = wx - t * ax, dy = wy - t * ay;
    return dx * dx + dy * dy;
}
__global__ void k_wall_distance(int nic, int njc, int nj, const double* __restrict__ xv, const double* __restrict__ yv,
                                const int* __restrict__ seg, int nseg, const double* __restrict__ cbox,
                                const int* __restrict__ col_chunk, double* __restrict__ wd) {
    const size_t n = (size_t)nic * njc;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / njc), j = (int)(idx % njc);
        const double px = 0.25 * (xv[(size_t)i * nj + j] + xv[(size_t)(i + 1) * nj + j] + xv[(size_t)i * nj + j + 1] +
                                  xv[(size_t)(i + 1) * nj + j + 1]);
        const double py = 0.25 * (yv[(size_t)i * nj + j] + yv[(size_t)(i + 1) * nj + j] + yv[(size_t)i * nj + j + 1] +
                                  yv[(size_t)(i + 1) * nj + j + 1]);
        double best = 1e300;
        const int nch = (nseg + WD_CHUNK - 1) / WD_CHUNK;
        auto scan = [&](int ch) {
            const int k1 = min(nseg, (ch + 1) * WD_CHUNK);
            for (int k = ch * WD_CHUNK; k < k1; k++) {
                const int s = seg[k];
                best = fmin(best, seg_dist2(px, py, xv[(size_t)s * nj], yv[(size_t)s * nj], xv[(size_t)(s + 1) * nj],
                                            yv[(size_t)(s + 1) * nj]));
            }
        };
        const int first = col_chunk[i];
        if (first >= 0) scan(first);
        for (int ch = 0; ch < nch; ch++) {
            if (ch == first) continue;
            const double* b = cbox + ch * 4;  // xmin, ymin, xmax, ymax
            const double dx = fmax(0.0, fmax(b[0] - px, px - b[2]));
            const double dy = fmax(0.0, fmax(b[1] - py, py - b[3]));
            const double lb = dx * dx + dy * dy;
            if (lb * (1.0 - 1e-12) > best) continue;
            scan(ch);
        }
        wd[idx] = nseg ? ::sqrt(best) : 1e30;
    }
}

// ---------------------------------------------------------------------------
// small kernels: time step, norms, skin friction, fill
// ---------------------------------------------------------------------------
// calc_dt, src/model/eulerequation.cpp:237-259 (every slot set, SA included)
template <int NQ>
__global__ void k_dt(DevCase c, const double* __restrict__ q, const double* __restrict__ dsmin, double cfl,
                     double* __restrict__ dt) {
    const size_t n = (size_t)c.nic * c.njc;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const double* Q = q + idx * NQ;
        double rho = Q[0], u = Q[1] / rho, v = Q[2] / rho, rhoE = Q[3];
        double p = (rhoE - 0.5 * rho * (u * u + v * v)) * GM1;
        double lambda = ::sqrt(GAMMA * p / rho) + ::fabs(u) + ::fabs(v);
        double len = dsmin[idx];
        double d = cfl / (lambda / len + 2.0 * c.mu_inf / len / len);
        for (int k = 0; k < NQ; k++) dt[idx * NQ + k] = d;
    }
}

constexpr int NORM_BLOCKS = 304;
// Sum of squares per component, fixed grid and fixed tree: deterministic.
template <int NQ>
__global__ void __launch_bounds__(256) k_norm_partial(const double* __restrict__ r, size_t ncell, double* part) {
    double acc[NQ];
    for (int k = 0; k < NQ; k++) acc[k] = 0.0;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < ncell; idx += (size_t)gridDim.x * blockDim.x)
        for (int k = 0; k < NQ; k++) { double x = r[idx * NQ + k]; acc[k] = fma(x, x, acc[k]); }
    __shared__ double sm[8][NQ];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int k = 0; k < NQ; k++) {
        double x = acc[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sm[wid][k] = x;
    }
    __syncthreads();
    if (threadIdx.x < NQ) {
        double s = 0.0;
        for (int w = 0; w < 8; w++) s += sm[w][threadIdx.x];
        part[blockIdx.x * NQ + threadIdx.x] = s;
    }
}
template <int NQ>
__global__ void k_norm_final(const double* part, int nblocks, double* out) {
    if (threadIdx.x < NQ) {
        double s = 0.0;
        for (int b = 0; b < nblocks; b++) s += part[b * NQ + threadIdx.x];
        out[threadIdx.x] = ::sqrt(s);
    }
}

// Wall Cf from the j=0 face gradient (IOManager::write_surface,
// src/utils/io.cpp:217-226): Cf = mu_inf (du/dy - dv/dx) / q_inf.
__global__ void k_skin_friction(DevCase c, const double* __restrict__ P, double qinf, double* cf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nic) return;
    const FaceIdx fi = face_idx<1>(c, i, 0);
    const double* gm = c.geo_j + fi.face * NGEO;
    const double* pL = P + fi.L; const double* pR = P + fi.R;
    const double* a = P + fi.Pa; const double* b = P + fi.Pb;
    const double* m = P + fi.Ma; const double* n = P + fi.Mb;
    double uy = gm[G_WLY] * pL[P_U] + gm[G_WRY] * pR[P_U] + gm[G_WPY] * (a[P_U] + b[P_U]) + gm[G_WMY] * (m[P_U] + n[P_U]);
    double vx = gm[G_WLX] * pL[P_V] + gm[G_WRX] * pR[P_V] + gm[G_WPX] * (a[P_V] + b[P_V]) + gm[G_WMX] * (m[P_V] + n[P_V]);
    cf[i] = c.mu_inf * (uy - vx) / qinf;
}

// J = sum_i w_i Cf_i over the wall faces, one CTA: strided partial sums,
// warp-shuffle tree, then the eight warp sums in a fixed order
// (deterministic).  out[0] = J.
__global__ void __launch_bounds__(256) k_drag(const double* __restrict__ cf, const double* __restrict__ w, int n,
                                              double* __restrict__ out) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc = fma(cf[i], w[i], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double sm[8];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < 8; k++) s += sm[k];
        out[0] = s;
    }
}

// velocity gradients (u_x, u_y, v_x, v_y) at the j = 0 faces, the row of
// grad_u_eta / grad_v_eta that IOManager::write_surface reads
// (src/utils/io.cpp:217-236), with the face-gradient weights of k_skin_friction
__global__ void k_wall_gradients(DevCase c, const double* __restrict__ P, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nic) return;
    const FaceIdx fi = face_idx<1>(c, i, 0);
    const double* gm = c.geo_j + fi.face * NGEO;
    const double* pL = P + fi.L; const double* pR = P + fi.R;
    const double* a = P + fi.Pa; const double* b = P + fi.Pb;
    const double* m = P + fi.Ma; const double* n = P + fi.Mb;
    double* o = out + (size_t)i * 4;
#pragma unroll
    for (int s = 0; s < 2; s++) {
        const int f = s == 0 ? P_U : P_V;
        o[2 * s + 0] = gm[G_WLX] * pL[f] + gm[G_WRX] * pR[f] + gm[G_WPX] * (a[f] + b[f]) + gm[G_WMX] * (m[f] + n[f]);
        o[2 * s + 1] = gm[G_WLY] * pL[f] + gm[G_WRY] * pR[f] + gm[G_WPY] * (a[f] + b[f]) + gm[G_WMY] * (m[f] + n[f]);
    }
}

__global__ void k_fill(double* a, size_t n, double v) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) a[i] = v;
}
__global__ void k_to_dual(const double* x, const double* dx, st::dual* y, size_t n, double fill) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        y[i] = st::dual(x ? x[i] : fill, dx ? dx[i] : 0.0);
}
__global__ void k_tangent(const st::dual* y, double* d, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) d[i] = y[i].d;
}

// FP64 FMA throughput probe: independent chains, result kept live.
__global__ void k_dfma_probe(double* out, int iters, double a, double b) {
    double x[8];
    for (int k = 0; k < 8; k++) x[k] = threadIdx.x * 1e-3 + k;
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
    double s = 0;
    for (int k = 0; k < 8; k++) s += x[k];
    if (s == 12345.678) out[0] = s;
}

// Newton-Raphson reciprocal and square roots of st_common.cuh on a device
// array: out[i][0..4] = nr_rcp, nr_rsqrt, nr_sqrt, nr_sqrt_inv (root, inverse)
__global__ void k_nr_probe(const double* __restrict__ x, size_t n, double* __restrict__ out) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double v = x[i];
        double inv;
        const double s = nr_sqrt_inv(v, &inv);
        out[i * 5 + 0] = nr_rcp(v);
        out[i * 5 + 1] = nr_rsqrt(v);
        out[i * 5 + 2] = nr_sqrt(v);
        out[i * 5 + 3] = s;
        out[i * 5 + 4] = inv;
    }
}

template <class T>
int alloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return stx::cuda_fail(e, "cudaMalloc");
    return ST_OK;
}

// ---------------------------------------------------------------------------
// forward pipelines
// ---------------------------------------------------------------------------
template <class T, int NQ>
int launch_forward(st_ctx* x, const DevCase& dc, const T* q, const T* beta, T* P, T* lim, T* Fi, T* Fj,
                   T* Gi, T* Gj, T* rhs, int order) {
    cudaStream_t s = x->stream;
    const unsigned gc = grid_for(x->ncell);
    k_prim<T, NQ><<<gc, 256, 0, s>>>(dc, q, P);
    stx::mark(x, "k_prim");
    launch_bcs<T, NQ>(dc, x->bcs.data(), (int)x->bcs.size(), P, s);
    stx::mark(x, "k_bc");
    if (order == 2) {
        k_limiter<T, NQ, false><<<gc, 256, 0, s>>>(dc, P, lim);
        stx::mark(x, "k_limiter");
        k_face<T, NQ, 0, 2><<<grid_for(x->nfi), 256, 0, s>>>(dc, P, lim, Fi, Gi);
        stx::mark(x, "k_face_i");
        k_face<T, NQ, 1, 2><<<grid_for(x->nfj), 256, 0, s>>>(dc, P, lim, Fj, Gj);
        stx::mark(x, "k_face_j");
    } else {
        k_face<T, NQ, 0, 1><<<grid_for(x->nfi), 256, 0, s>>>(dc, P, lim, Fi, Gi);
        stx::mark(x, "k_face_i");
        k_face<T, NQ, 1, 1><<<grid_for(x->nfj), 256, 0, s>>>(dc, P, lim, Fj, Gj);
        stx::mark(x, "k_face_j");
    }
    // the host-buffer residual copies the state's residual out band by band
    double* dst = nullptr;
    if constexpr (std::is_same_v<T, double>) dst = rhs == x->rhs ? x->hio.rhs : nullptr;
    auto cell = [&](size_t f, size_t l) {
        const unsigned g = grid_for(l - f);
        if constexpr (NQ == 5) {
            if (dc.mlp_wb) k_cell<T, NQ, true><<<g, 256, 0, s>>>(dc, P, Fi, Fj, Gi, Gj, beta, rhs, f, l);
            else k_cell<T, NQ><<<g, 256, 0, s>>>(dc, P, Fi, Fj, Gi, Gj, beta, rhs, f, l);
        } else {
            k_cell<T, NQ><<<g, 256, 0, s>>>(dc, P, Fi, Fj, Gi, Gj, beta, rhs, f, l);
        }
    };
    if constexpr (std::is_same_v<T, double>) {
        const int rc = stx::run_banded(x, dst, rhs, NQ, cell);
        if (rc) return rc;
    } else {
        cell(0, x->ncell);
    }
    stx::mark(x, "k_cell");
    ST_LAUNCH_CHECK("residual launch");
    return ST_OK;
}

// Residual by the tiled sweeps: primitives and boundary ghosts as in the
// per-face pipeline, then one TMA-staged i-sweep and one j-sweep.
template <int NQ>
int launch_tiled(st_ctx* x, const double* q, const double* beta, double* rhs, int order) {
    cudaStream_t s = x->stream;
    const DevCase& dc = x->dc;
    const int nic = x->c.ni - 1, njc = x->c.nj - 1;
    k_prim<double, NQ><<<grid_for(x->ncell), 256, 0, s>>>(dc, q, x->P);
    stx::mark(x, "k_prim");
    launch_bcs<double, NQ>(dc, x->bcs.data(), (int)x->bcs.size(), x->P, s);
    stx::mark(x, "k_bc");
    const dim3 gi((nic + TI_I - 1) / TI_I, (njc + TJ_I - 1) / TJ_I);
    const dim3 gj((njc + TJ_J - 1) / TJ_J, (nic + TI_J - 1) / TI_J);
    if (order == 2) {
        k_sweep_i<NQ, 2><<<gi, SW_THREADS, SWEEP_SMEM_I, s>>>(dc, x->tmap_i, rhs, x->Gi);
        stx::mark(x, "k_sweep_i");
        k_sweep_j<NQ, 2><<<gj, SW_THREADS, SWEEP_SMEM_J, s>>>(dc, x->tmap_j, x->Gi, beta, rhs);
    } else {
        k_sweep_i<NQ, 1><<<gi, SW_THREADS, SWEEP_SMEM_I, s>>>(dc, x->tmap_i, rhs, x->Gi);
        stx::mark(x, "k_sweep_i");
        k_sweep_j<NQ, 1><<<gj, SW_THREADS, SWEEP_SMEM_J, s>>>(dc, x->tmap_j, x->Gi, beta, rhs);
    }
    stx::mark(x, "k_sweep_j");
    if (x->hio.rhs && rhs == x->rhs) {
        const int rc = stx::copy_out(x, x->xev[3], x->hio.rhs, rhs, x->ncell * NQ * 8);
        if (rc) return rc;
    }
    ST_LAUNCH_CHECK("tiled residual launch");
    return ST_OK;
}

// TMA descriptors of P = [nic+2][njc+2][8] doubles (innermost first: record
// slot, padded j, padded i) for the two sweep boxes, and the sweeps' dynamic
// shared memory limits.  Leaves tile_ok false (the per-face passes then run)
// if the driver entry point or an encoding is unavailable.
int setup_tiles(st_ctx* x) {
    x->tile_ok = false;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return ST_OK;
    }
    auto encode = reinterpret_cast<CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                                CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                                CUtensorMapFloatOOBfill)>(fn);
    const int nic = x->c.ni - 1, njc = x->c.nj - 1;
    const cuuint64_t dims[3] = {(cuuint64_t)NP, (cuuint64_t)(njc + 2), (cuuint64_t)(nic + 2)};
    const cuuint64_t strides[2] = {(cuuint64_t)NP * 8, (cuuint64_t)(njc + 2) * NP * 8};
    const cuuint32_t estr[3] = {1, 1, 1};
    const cuuint32_t box_i[3] = {(cuuint32_t)NP, (cuuint32_t)BJ_I, (cuuint32_t)BI_I};
    const cuuint32_t box_j[3] = {(cuuint32_t)NP, (cuuint32_t)BJ_J, (cuuint32_t)BI_J};
    if (reinterpret_cast<uintptr_t>(x->P) % 16) return ST_OK;
    for (int w = 0; w < 2; w++) {
        CUresult r = encode(w == 0 ? &x->tmap_i : &x->tmap_j, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, x->P, dims, strides,
                            w == 0 ? box_i : box_j, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return ST_OK;
    }
    ST_CUDA(cudaFuncSetAttribute(k_sweep_i<5, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SWEEP_SMEM_I));
    ST_CUDA(cudaFuncSetAttribute(k_sweep_i<5, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SWEEP_SMEM_I));
    ST_CUDA(cudaFuncSetAttribute(k_sweep_i<4, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SWEEP_SMEM_I));
    ST_CUDA(cudaFuncSetAttribute(k_sweep_i<4, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SWEEP_SMEM_I));
    ST_CUDA(cudaFuncSetAttribute(k_sweep_j<5, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SWEEP_SMEM_J));
    ST_CUDA(cudaFuncSetAttribute(k_sweep_j<5, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SWEEP_SMEM_J));
    ST_CUDA(cudaFuncSetAttribute(k_sweep_j<4, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SWEEP_SMEM_J));
    ST_CUDA(cudaFuncSetAttribute(k_sweep_j<4, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SWEEP_SMEM_J));
    x->tile_ok = true;
    return ST_OK;
}

int order_of(st_ctx* x, int lhs) { return lhs ? x->c.lhs_order : x->c.order; }

}  // namespace

namespace stx {
int run_jvp(st_ctx* x, const double* v_dev, const double* vb_dev, double* jv_dev, int order, int freeze_nonlocal) {
    const int nq = x->nq;
    if (!x->qd) {
        int rc = ST_OK;
        if (rc == ST_OK) rc = alloc(&x->qd, x->ncell * nq);
        if (rc == ST_OK) rc = alloc(&x->Pd, x->npad * NP);
        if (rc == ST_OK) rc = alloc(&x->limd, x->ncell * 4 * 5);
        if (rc == ST_OK) rc = alloc(&x->Fdi, x->nfi * nq);
        if (rc == ST_OK) rc = alloc(&x->Fdj, x->nfj * nq);
        if (rc == ST_OK) rc = alloc(&x->Gdi, x->nfi * 4);
        if (rc == ST_OK) rc = alloc(&x->Gdj, x->nfj * 4);
        if (rc == ST_OK) rc = alloc(&x->rhsd, x->ncell * nq);
        if (rc == ST_OK) rc = alloc(&x->betad, x->ncell);
        if (rc) return rc;
        ST_CUDA(cudaMemsetAsync(x->Pd, 0, x->npad * NP * sizeof(st::dual), x->stream));
        ST_CUDA(cudaMemsetAsync(x->Gdi, 0, x->nfi * 4 * sizeof(st::dual), x->stream));
        ST_CUDA(cudaMemsetAsync(x->Gdj, 0, x->nfj * 4 * sizeof(st::dual), x->stream));
    }
    cudaStream_t s = x->stream;
    k_to_dual<<<grid_for(x->ncell * nq), 256, 0, s>>>(x->q, v_dev, x->qd, x->ncell * nq, 0.0);
    k_to_dual<<<grid_for(x->ncell), 256, 0, s>>>(x->beta, vb_dev, x->betad, x->ncell, 1.0);
    st::DevCase dc = x->dc;
    dc.nonlocal_frozen = freeze_nonlocal;
    int rc;
    if (nq == 5)
        rc = launch_forward<st::dual, 5>(x, dc, x->qd, x->betad, x->Pd, x->limd, x->Fdi, x->Fdj,
                                          x->Gdi, x->Gdj, x->rhsd, order);
    else
        rc = launch_forward<st::dual, 4>(x, dc, x->qd, x->betad, x->Pd, x->limd, x->Fdi, x->Fdj,
                                          x->Gdi, x->Gdj, x->rhsd, order);
    if (rc) return rc;
    k_tangent<<<grid_for(x->ncell * nq), 256, 0, s>>>(x->rhsd, jv_dev, x->ncell * nq);
    ST_LAUNCH_CHECK("jvp");
    return ST_OK;
}

int run_dt(st_ctx* x, double cfl) {
    if (x->nq == 5) k_dt<5><<<grid_for(x->ncell), 256, 0, x->stream>>>(x->dc, x->q, x->dsmin_d, cfl, x->dt);
    else k_dt<4><<<grid_for(x->ncell), 256, 0, x->stream>>>(x->dc, x->q, x->dsmin_d, cfl, x->dt);
    ST_LAUNCH_CHECK("k_dt");
    return ST_OK;
}

int run_norms(st_ctx* x, const double* rhs, double* out) {
    if (x->nq == 5) {
        k_norm_partial<5><<<NORM_BLOCKS, 256, 0, x->stream>>>(rhs, x->ncell, x->norm_part);
        k_norm_final<5><<<1, 32, 0, x->stream>>>(x->norm_part, NORM_BLOCKS, x->norm_out);
    } else {
        k_norm_partial<4><<<NORM_BLOCKS, 256, 0, x->stream>>>(rhs, x->ncell, x->norm_part);
        k_norm_final<4><<<1, 32, 0, x->stream>>>(x->norm_part, NORM_BLOCKS, x->norm_out);
    }
    ST_LAUNCH_CHECK("norms");
    ST_CUDA(cudaMemcpyAsync(out, x->norm_out, x->nq * 8, cudaMemcpyDeviceToHost, x->stream));
    ST_CUDA(cudaStreamSynchronize(x->stream));
    for (int k = 0; k < x->nq; k++)
        if (!std::isfinite(out[k])) return fail(ST_ERR_NONFINITE, "non-finite residual norm");
    return ST_OK;
}

int run_residual(st_ctx* x, const double* q, const double* beta, double* rhs, int order) {
    if (x->tile_ok && x->res_path == 1 && !x->dc.mlp_wb)
        return x->nq == 5 ? launch_tiled<5>(x, q, beta, rhs, order) : launch_tiled<4>(x, q, beta, rhs, order);
    return run_residual_faces(x, q, beta, rhs, order);
}

int run_residual_faces(st_ctx* x, const double* q, const double* beta, double* rhs, int order) {
    if (x->nq == 5)
        return launch_forward<double, 5>(x, x->dc, q, beta, x->P, x->lim, x->Fi, x->Fj, x->Gi, x->Gj, rhs, order);
    return launch_forward<double, 4>(x, x->dc, q, beta, x->P, x->lim, x->Fi, x->Fj, x->Gi, x->Gj, rhs, order);
}
}  // namespace stx

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* st_last_error(void) { return g_last_error.c_str(); }
int st_version(void) { return 1; }

int st_create(const st_case* c, const double* xv, const double* yv, int device, st_ctx** out) {
    if (!c || !xv || !yv || !out) return fail(ST_ERR_ARG, "st_create: null argument");
    if (c->ni < 3 || c->nj < 3) return fail(ST_ERR_ARG, "st_create: grid must have ni, nj >= 3");
    if (c->order != 1 && c->order != 2) return fail(ST_ERR_ARG, "st_create: order must be 1 or 2");
    if (c->lhs_order != 1 && c->lhs_order != 2) return fail(ST_ERR_ARG, "st_create: lhs_order must be 1 or 2");
    if (c->nbc < 0 || (c->nbc > 0 && !c->bcs)) return fail(ST_ERR_ARG, "st_create: bad boundary list");
    if (c->turbulence != ST_TURB_NONE && c->turbulence != ST_TURB_SA) return fail(ST_ERR_ARG, "st_create: turbulence");
    if (c->viscosity_law != ST_VISC_POWER && c->viscosity_law != ST_VISC_SUTHERLAND) return fail(ST_ERR_ARG, "st_create: viscosity_law");
    if (c->flux != ST_FLUX_ROE && c->flux != ST_FLUX_AUSM) return fail(ST_ERR_ARG, "st_create: flux");
    for (int b = 0; b < c->nbc; b++) {
        const st_bc& bc = c->bcs[b];
        if (bc.type < 0 || bc.type > ST_BC_WAKE || bc.face < 0 || bc.face > 3)
            return fail(ST_ERR_ARG, "st_create: bad boundary type/face");
        const int lim = (bc.face == ST_FACE_BOTTOM || bc.face == ST_FACE_TOP) ? c->ni + 1 : c->nj + 1;
        const int end = bc.end >= 0 ? bc.end : lim + bc.end;
        if (bc.start < 0 || end >= lim || bc.start > end + 1)
            return fail(ST_ERR_ARG, "st_create: boundary range outside the ghost layer");
        if (bc.type == ST_BC_SLIPWALL && (bc.start < 1 || end > c->ni - 1))
            return fail(ST_ERR_ARG, "st_create: slipwall range must lie in [1, nic] (it reads the face normal of cell index-1)");
        if (bc.type == ST_BC_WAKE && end > c->ni - 1)
            return fail(ST_ERR_ARG, "st_create: wake range");
    }
    st_ctx* x = new st_ctx();
    x->c = *c;
    x->bcs.assign(c->bcs, c->bcs + c->nbc);
    x->c.bcs = nullptr;
    if (device >= 0) {
        cudaError_t e = cudaSetDevice(device);
        if (e != cudaSuccess) { delete x; return stx::cuda_fail(e, "cudaSetDevice"); }
    }
    cudaGetDevice(&x->device);
    const int ni = c->ni, nj = c->nj, nic = ni - 1, njc = nj - 1;
    x->nq = (c->turbulence == ST_TURB_SA) ? 5 : 4;
    x->ncell = (size_t)nic * njc;
    x->npad = (size_t)(nic + 2) * (njc + 2);
    x->nfi = (size_t)ni * njc;
    x->nfj = (size_t)nic * nj;
    x->xv.assign(xv, xv + (size_t)ni * nj);
    x->yv.assign(yv, yv + (size_t)ni * nj);
    host_metrics(x);
    std::vector<double> gi, gj;
    host_geometry(x, gi, gj);
    std::vector<double> ivol(x->ncell);
    for (size_t n = 0; n < x->ncell; n++) {
        if (!(x->vol[n] > 0.0)) { delete x; return fail(ST_ERR_ARG, "st_create: non-positive cell volume (grid orientation)"); }
        ivol[n] = 1.0 / x->vol[n];
    }
    // wall dx per bottom face (objective integral)
    x->wall_dx.assign(nic, 0.0);
    for (int i = std::max(c->plate_vertex, 0); i < nic; i++) {
        double x0 = x->xv[(size_t)i * nj], x1 = x->xv[(size_t)(i + 1) * nj];
        if (0.5 * (x0 + x1) <= c->plate_x_end && c->plate_vertex >= 0) x->wall_dx[i] = x1 - x0;
    }
    const int nq = x->nq;
    int rc = ST_OK;
#define AL(p, n) if (rc == ST_OK) rc = alloc(&(p), (n))
    AL(x->q, x->ncell * nq); AL(x->rhs, x->ncell * nq); AL(x->beta, x->ncell); AL(x->P, x->npad * NP);
    AL(x->lim, x->ncell * 12 * 5); AL(x->Fi, x->nfi * nq); AL(x->Fj, x->nfj * nq);
    AL(x->Gi, x->nfi * 4); AL(x->Gj, x->nfj * 4); AL(x->vol_d, x->ncell); AL(x->ivol_d, x->ncell);
    AL(x->geo_i, x->nfi * NGEO); AL(x->geo_j, x->nfj * NGEO); AL(x->wd, x->ncell);
    AL(x->nchi_d, x->nchi.size()); AL(x->neta_d, x->neta.size()); AL(x->dsmin_d, x->ncell); AL(x->dt, x->ncell * nq);
    AL(x->norm_part, NORM_BLOCKS * 8); AL(x->norm_out, 8); AL(x->cf, nic); AL(x->wall_dx_d, nic);
    AL(x->bcs_d, std::max(1, c->nbc)); AL(x->err_d, 1);
#undef AL
    if (rc != ST_OK) { st_destroy(x); return rc; }
    cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking);
    for (auto& e : x->ev) cudaEventCreate(&e);
    cudaStreamCreateWithFlags(&x->xfer, cudaStreamNonBlocking);
    for (auto& e : x->xev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    for (auto& e : x->band_ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    std::vector<DevBC> dbc(std::max(1, c->nbc));
    for (int b = 0; b < c->nbc; b++)
        dbc[b] = DevBC{c->bcs[b].type, c->bcs[b].face, c->bcs[b].start, c->bcs[b].end, c->bcs[b].u, c->bcs[b].v, c->bcs[b].T};
    cudaMemcpy(x->bcs_d, dbc.data(), dbc.size() * sizeof(DevBC), cudaMemcpyHostToDevice);
    cudaMemcpy(x->vol_d, x->vol.data(), x->ncell * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(x->ivol_d, ivol.data(), x->ncell * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(x->geo_i, gi.data(), gi.size() * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(x->geo_j, gj.data(), gj.size() * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(x->nchi_d, x->nchi.data(), x->nchi.size() * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(x->neta_d, x->neta.data(), x->neta.size() * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(x->dsmin_d, x->ds_min.data(), x->ncell * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(x->wall_dx_d, x->wall_dx.data(), nic * 8, cudaMemcpyHostToDevice);
    cudaMemset(x->P, 0, x->npad * NP * 8);
    cudaMemset(x->Gi, 0, x->nfi * 4 * 8);
    cudaMemset(x->Gj, 0, x->nfj * 4 * 8);
    cudaMemset(x->err_d, 0, sizeof(int));
    k_fill<<<grid_for(x->ncell), 256, 0, x->stream>>>(x->beta, x->ncell, 1.0);
    if (int rt = setup_tiles(x)) { st_destroy(x); return rt; }

    // wall distance (no-slip bottom segments, last writer wins per column)
    {
        std::vector<int> wall(nic, 0);
        for (const auto& b : x->bcs) {
            if (b.face != ST_FACE_BOTTOM) continue;
            int end = b.end >= 0 ? b.end : nic + 2 + b.end;
            bool isw = (b.type == ST_BC_WALL || b.type == ST_BC_ISOTHERMALWALL);
            for (int g = b.start; g <= end; g++)
                if (g >= 1 && g <= nic) wall[g - 1] = isw ? 1 : 0;
        }
        std::vector<int> seg;
        for (int i = 0; i < nic; i++) if (wall[i]) seg.push_back(i);
        // chunk bounding boxes (wall order) and each column's own chunk
        const int nch = (int)((seg.size() + WD_CHUNK - 1) / WD_CHUNK);
        std::vector<double> cbox((size_t)std::max(1, nch) * 4);
        std::vector<int> col_chunk(nic, -1);
        for (int ch = 0; ch < nch; ch++) {
            double b[4] = {1e300, 1e300, -1e300, -1e300};
            for (size_t k = (size_t)ch * WD_CHUNK; k < std::min(seg.size(), (size_t)(ch + 1) * WD_CHUNK); k++) {
                col_chunk[seg[k]] = ch;
                for (int e = 0; e < 2; e++) {
                    const double px = x->xv[(size_t)(seg[k] + e) * nj], py = x->yv[(size_t)(seg[k] + e) * nj];
                    b[0] = std::min(b[0], px); b[1] = std::min(b[1], py);
                    b[2] = std::max(b[2], px); b[3] = std::max(b[3], py);
                }
            }
            for (int e = 0; e < 4; e++) cbox[(size_t)ch * 4 + e] = b[e];
        }
        double *xv_d = nullptr, *yv_d = nullptr, *cbox_d = nullptr; int *seg_d = nullptr, *col_d = nullptr;
        rc = alloc(&xv_d, x->xv.size());
        if (rc == ST_OK) rc = alloc(&yv_d, x->yv.size());
        if (rc == ST_OK) rc = alloc(&seg_d, std::max<size_t>(1, seg.size()));
        if (rc == ST_OK) rc = alloc(&cbox_d, cbox.size());
        if (rc == ST_OK) rc = alloc(&col_d, (size_t)nic);
        if (rc != ST_OK) { st_destroy(x); return rc; }
        cudaMemcpy(xv_d, x->xv.data(), x->xv.size() * 8, cudaMemcpyHostToDevice);
        cudaMemcpy(yv_d, x->yv.data(), x->yv.size() * 8, cudaMemcpyHostToDevice);
        if (!seg.empty()) cudaMemcpy(seg_d, seg.data(), seg.size() * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(cbox_d, cbox.data(), cbox.size() * 8, cudaMemcpyHostToDevice);
        cudaMemcpy(col_d, col_chunk.data(), (size_t)nic * sizeof(int), cudaMemcpyHostToDevice);
        k_wall_distance<<<grid_for(x->ncell), 256, 0, x->stream>>>(nic, njc, nj, xv_d, yv_d, seg_d, (int)seg.size(),
                                                                   cbox_d, col_d, x->wd);
        cudaStreamSynchronize(x->stream);
        cudaFree(xv_d); cudaFree(yv_d); cudaFree(seg_d); cudaFree(cbox_d); cudaFree(col_d);
    }

    DevCase& dc = x->dc;
    dc.ni = ni; dc.nj = nj; dc.nic = nic; dc.njc = njc; dc.nq = nq;
    dc.viscous = c->mu_inf > 1e-15;  // src/utils/config.cpp:41
    dc.sa = (c->turbulence == ST_TURB_SA);
    dc.law = c->viscosity_law;
    dc.flux = c->flux;
    dc.nbc = c->nbc;
    dc.R = c->p_inf / c->rho_inf / c->T_inf;  // src/model/fluid.cpp:12
    dc.cp = GAMMA * dc.R / (GAMMA - 1.0);
    dc.pr = c->pr_inf;
    dc.cp_pr = dc.cp / dc.pr;
    dc.cp_prt = dc.cp / PR_TURB;
    dc.iR = 1.0 / dc.R;
    dc.rho_inf = c->rho_inf; dc.u_inf = c->u_inf; dc.v_inf = c->v_inf; dc.p_inf = c->p_inf;
    dc.T_inf = c->T_inf; dc.mu_inf = c->mu_inf; dc.nut_inf = c->nu_tilde_inf;
    dc.iT_inf = 1.0 / dc.T_inf;
    dc.suth_S = 110.4 / 288.15 * c->T_inf;
    dc.eps_chi = std::pow(10.0 / nic, 3);  // src/model/reconstruction.cpp:59-60
    dc.eps_eta = std::pow(10.0 / njc, 3);
    dc.dpdx = c->dpdx; dc.dpdy = c->dpdy;
    dc.vol = x->vol_d; dc.ivol = x->ivol_d; dc.geo_i = x->geo_i; dc.geo_j = x->geo_j; dc.wd = x->wd;
    dc.nchi = x->nchi_d; dc.neta = x->neta_d; dc.bcs = x->bcs_d; dc.err = x->err_d;
    dc.mlp_wb = nullptr; dc.mlp_wf = nullptr; dc.nonlocal_frozen = 0;
    cudaError_t e = cudaStreamSynchronize(x->stream);
    if (e != cudaSuccess) { st_destroy(x); return stx::cuda_fail(e, "st_create"); }
    *out = x;
    return ST_OK;
}

int st_destroy(st_ctx* x) {
    if (!x) return ST_OK;
    if (x->stream) cudaStreamSynchronize(x->stream);
    if (x->xfer) cudaStreamSynchronize(x->xfer);
    double* bufs[] = {x->q, x->rhs, x->beta, x->P, x->lim, x->Fi, x->Fj, x->Gi, x->Gj, x->vol_d, x->ivol_d,
                      x->geo_i, x->geo_j, x->wd, x->nchi_d, x->neta_d, x->dsmin_d, x->dt, x->norm_part, x->norm_out,
                      x->cf, x->wall_dx_d, x->Pbar, x->srec, x->arec_i, x->arec_j, x->psi_tmp,
                      x->outq_tmp, x->outb_tmp, x->tape, x->jac, x->jac1, x->kv, x->kzb, x->kz, x->kw, x->kr, x->kh, x->kpart, x->dq, x->qsave,
                      x->qtmp, x->wpart[0], x->wpart[1], x->wpart[2], x->wpart1[0], x->wpart1[1], x->wpart1[2],
                      x->wallg, x->strip_jac_d, x->strip_dt_d, x->strip_inv_d, x->strip_res_d, x->ring_dev};
    for (double* b : bufs) if (b) cudaFree(b);
    if (x->ring_host) cudaFreeHost(x->ring_host);
    for (int* m : x->pmask_d) if (m) cudaFree(m);
    if (x->strip_cells_d) cudaFree(x->strip_cells_d);
    st::dual* dbufs[] = {x->qd, x->Pd, x->limd, x->Fdi, x->Fdj, x->Gdi, x->Gdj, x->rhsd, x->betad};
    for (st::dual* b : dbufs) if (b) cudaFree(b);
    if (x->bcs_d) cudaFree(x->bcs_d);
    if (x->err_d) cudaFree(x->err_d);
    if (x->lfac) cudaFree(x->lfac);
    if (x->mlp_wb) cudaFree(x->mlp_wb);
    float* fbufs[] = {x->mlp_wf, x->mlp_master, x->mlp_loss, x->mlp_part};
    for (float* b : fbufs) if (b) cudaFree(b);
    for (auto& e : x->ev) if (e) cudaEventDestroy(e);
    for (auto& e : x->xev) if (e) cudaEventDestroy(e);
    for (auto& e : x->band_ev) if (e) cudaEventDestroy(e);
    if (x->stream) cudaStreamDestroy(x->stream);
    if (x->xfer) cudaStreamDestroy(x->xfer);
    delete x;
    return ST_OK;
}

int st_dims(const st_ctx* x, int* nic, int* njc, int* nq) {
    if (!x) return fail(ST_ERR_ARG, "st_dims: null context");
    if (nic) *nic = x->c.ni - 1;
    if (njc) *njc = x->c.nj - 1;
    if (nq) *nq = x->nq;
    return ST_OK;
}

int st_set_state(st_ctx* x, const double* q) {
    if (!x || !q) return fail(ST_ERR_ARG, "st_set_state: null argument");
    return stx::copy_sync(x, x->q, q, x->ncell * x->nq * 8, cudaMemcpyHostToDevice);
}

int st_get_state(st_ctx* x, double* q) {
    if (!x || !q) return fail(ST_ERR_ARG, "st_get_state: null argument");
    return stx::copy_sync(x, q, x->q, x->ncell * x->nq * 8, cudaMemcpyDeviceToHost);
}

int st_set_beta(st_ctx* x, const double* b) {
    if (!x || !b) return fail(ST_ERR_ARG, "st_set_beta: null argument");
    return stx::copy_sync(x, x->beta, b, x->ncell * 8, cudaMemcpyHostToDevice);
}

int st_get_wall_distance(st_ctx* x, double* d) {
    if (!x || !d) return fail(ST_ERR_ARG, "st_get_wall_distance: null argument");
    return stx::copy_sync(x, d, x->wd, x->ncell * 8, cudaMemcpyDeviceToHost);
}

int st_residual_device(st_ctx* x, const double* q_dev, const double* beta_dev, double* rhs_dev, int lhs) {
    if (!x || !q_dev || !rhs_dev) return fail(ST_ERR_ARG, "st_residual_device: null argument");
    cudaEventRecord(x->ev[0], x->stream);
    int rc = stx::run_residual(x, q_dev, beta_dev, rhs_dev, order_of(x, lhs));
    if (rc) return rc;
    cudaEventRecord(x->ev[1], x->stream);
    x->res_pending = true;
    return ST_OK;
}

// The residual goes out on the copy stream: band by band behind the per-stage
// cell pass, or whole after the tiled sweeps.
int st_residual(st_ctx* x, int lhs, double* rhs_host) {
    if (!x) return fail(ST_ERR_ARG, "st_residual: null context");
    x->hio.rhs = rhs_host;
    const int rc = st_residual_device(x, x->q, x->beta, x->rhs, lhs);
    x->hio = {};
    const cudaError_t e1 = cudaStreamSynchronize(x->xfer);
    const cudaError_t e2 = cudaStreamSynchronize(x->stream);
    if (rc) return rc;
    if (e1 != cudaSuccess) return stx::cuda_fail(e1, "cudaStreamSynchronize (copy stream)");
    if (e2 != cudaSuccess) return stx::cuda_fail(e2, "cudaStreamSynchronize");
    x->have_residual = true;
    return ST_OK;
}

int st_dt(st_ctx* x, double cfl, double* dt_host) {
    if (!x) return fail(ST_ERR_ARG, "st_dt: null context");
    if (x->nq == 5) k_dt<5><<<grid_for(x->ncell), 256, 0, x->stream>>>(x->dc, x->q, x->dsmin_d, cfl, x->dt);
    else k_dt<4><<<grid_for(x->ncell), 256, 0, x->stream>>>(x->dc, x->q, x->dsmin_d, cfl, x->dt);
    ST_LAUNCH_CHECK("k_dt");
    if (dt_host) return stx::copy_sync(x, dt_host, x->dt, x->ncell * x->nq * 8, cudaMemcpyDeviceToHost);
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

int st_norms(st_ctx* x, double* out) {
    if (!x || !out) return fail(ST_ERR_ARG, "st_norms: null argument");
    if (!x->have_residual) return fail(ST_ERR_ARG, "st_norms: no residual evaluated yet");
    if (x->nq == 5) {
        k_norm_partial<5><<<NORM_BLOCKS, 256, 0, x->stream>>>(x->rhs, x->ncell, x->norm_part);
        k_norm_final<5><<<1, 32, 0, x->stream>>>(x->norm_part, NORM_BLOCKS, x->norm_out);
    } else {
        k_norm_partial<4><<<NORM_BLOCKS, 256, 0, x->stream>>>(x->rhs, x->ncell, x->norm_part);
        k_norm_final<4><<<1, 32, 0, x->stream>>>(x->norm_part, NORM_BLOCKS, x->norm_out);
    }
    ST_LAUNCH_CHECK("norms");
    ST_CUDA(cudaMemcpyAsync(out, x->norm_out, x->nq * 8, cudaMemcpyDeviceToHost, x->stream));
    ST_CUDA(cudaStreamSynchronize(x->stream));
    for (int k = 0; k < x->nq; k++)
        if (!std::isfinite(out[k])) return fail(ST_ERR_NONFINITE, "st_norms: non-finite residual norm");
    return ST_OK;
}

// wall Cf of the current state into x->cf and J into x->norm_out[7] (async)
static int skin_friction_device(st_ctx* x) {
    const DevCase& dc = x->dc;
    if (x->nq == 5) {
        k_prim<double, 5><<<grid_for(x->ncell), 256, 0, x->stream>>>(dc, x->q, x->P);
        k_bc<double, 5><<<1, 1024, 0, x->stream>>>(dc, x->P);
    } else {
        k_prim<double, 4><<<grid_for(x->ncell), 256, 0, x->stream>>>(dc, x->q, x->P);
        k_bc<double, 4><<<1, 1024, 0, x->stream>>>(dc, x->P);
    }
    const double qinf = 0.5 * x->c.rho_inf * (x->c.u_inf * x->c.u_inf + x->c.v_inf * x->c.v_inf);
    k_skin_friction<<<grid_for(x->c.ni - 1), 256, 0, x->stream>>>(dc, x->P, qinf, x->cf);
    k_drag<<<1, 256, 0, x->stream>>>(x->cf, x->wall_dx_d, x->c.ni - 1, x->norm_out + 7);
    ST_LAUNCH_CHECK("skin friction");
    return ST_OK;
}

int st_skin_friction(st_ctx* x, double* cf_host, double* J) {
    if (!x) return fail(ST_ERR_ARG, "st_skin_friction: null context");
    int rc = skin_friction_device(x);
    if (rc) return rc;
    if (cf_host) ST_CUDA(cudaMemcpyAsync(cf_host, x->cf, (size_t)(x->c.ni - 1) * 8, cudaMemcpyDeviceToHost, x->stream));
    double s = 0.0;
    ST_CUDA(cudaMemcpyAsync(&s, x->norm_out + 7, 8, cudaMemcpyDeviceToHost, x->stream));
    ST_CUDA(cudaStreamSynchronize(x->stream));
    if (J) *J = s;
    return ST_OK;
}

int st_skin_friction_device(st_ctx* x, double* cf_dev, double* J_dev) {
    if (!x) return fail(ST_ERR_ARG, "st_skin_friction_device: null context");
    int rc = skin_friction_device(x);
    if (rc) return rc;
    if (cf_dev) ST_CUDA(cudaMemcpyAsync(cf_dev, x->cf, (size_t)(x->c.ni - 1) * 8, cudaMemcpyDeviceToDevice, x->stream));
    if (J_dev) ST_CUDA(cudaMemcpyAsync(J_dev, x->norm_out + 7, 8, cudaMemcpyDeviceToDevice, x->stream));
    return ST_OK;
}

int st_wall_gradients(st_ctx* x, double* out_host) {
    if (!x || !out_host) return fail(ST_ERR_ARG, "st_wall_gradients: null argument");
    const DevCase& dc = x->dc;
    if (x->nq == 5) {
        k_prim<double, 5><<<grid_for(x->ncell), 256, 0, x->stream>>>(dc, x->q, x->P);
        k_bc<double, 5><<<1, 1024, 0, x->stream>>>(dc, x->P);
    } else {
        k_prim<double, 4><<<grid_for(x->ncell), 256, 0, x->stream>>>(dc, x->q, x->P);
        k_bc<double, 4><<<1, 1024, 0, x->stream>>>(dc, x->P);
    }
    const int nic = x->c.ni - 1;
    if (!x->wallg) {
        int rc = alloc(&x->wallg, (size_t)nic * 4);
        if (rc) return rc;
    }
    k_wall_gradients<<<grid_for(nic), 256, 0, x->stream>>>(dc, x->P, x->wallg);
    ST_LAUNCH_CHECK("wall gradients");
    ST_CUDA(cudaMemcpyAsync(out_host, x->wallg, (size_t)nic * 4 * 8, cudaMemcpyDeviceToHost, x->stream));
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

int st_jvp_device(st_ctx* x, const double* v_dev, const double* vb_dev, double* jv_dev, int lhs) {
    if (!x || !v_dev || !jv_dev) return fail(ST_ERR_ARG, "st_jvp_device: null argument");
    int rc = stx::run_jvp(x, v_dev, vb_dev, jv_dev, order_of(x, lhs));
    if (rc) return rc;
    ST_CUDA(cudaStreamSynchronize(x->stream));
    return ST_OK;
}

int st_probe_fp64(st_ctx* x, double* tflops) {
    if (!x || !tflops) return fail(ST_ERR_ARG, "st_probe_fp64: null argument");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, x->device);
    const int blocks = sms * 2, threads = 256, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_dfma_probe<<<blocks, threads, 0, x->stream>>>(x->norm_out, 16, 0.999, 1e-3);
    cudaEventRecord(e0, x->stream);
    k_dfma_probe<<<blocks, threads, 0, x->stream>>>(x->norm_out, iters, 0.999, 1e-3);
    cudaEventRecord(e1, x->stream);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) return stx::cuda_fail(err, "st_probe_fp64");
    *tflops = 2.0 * blocks * threads * (double)iters * 8 / (ms * 1e-3) / 1e12;
    return ST_OK;
}

int st_probe_nr_math(const double* x_dev, long long n, double* out_dev) {
    if (!x_dev || !out_dev || n < 1) return fail(ST_ERR_ARG, "st_probe_nr_math: bad argument");
    k_nr_probe<<<grid_for((size_t)n), 256>>>(x_dev, (size_t)n, out_dev);
    ST_LAUNCH_CHECK("st_probe_nr_math");
    ST_CUDA(cudaDeviceSynchronize());
    return ST_OK;
}

// Runs one pipeline (which = 0 residual, 1 adjoint VJP with psi = the
// context's last residual) with a CUDA event after every launch and returns
// the per-launch device times and names.
int st_profile_pipeline(st_ctx* x, int which, int lhs, double* ms, int max_n, char* names, int names_len,
                        int* n) {
    if (!x || !ms || !n) return fail(ST_ERR_ARG, "st_profile_pipeline: null argument");
    if (!x->prof_ev[0])
        for (auto& e : x->prof_ev) cudaEventCreate(&e);
    x->prof_on = true;
    x->prof_n = 0;
    cudaEventRecord(x->prof_ev[0], x->stream);
    int rc;
    if (which == 0) rc = stx::run_residual(x, x->q, x->beta, x->rhs, order_of(x, lhs));
    else if (which == 1) rc = st_vjp_device(x, x->rhs, nullptr, nullptr, lhs);
    else rc = st_residual_vjp_device(x, x->rhs, x->rhs, nullptr, nullptr, lhs);
    x->prof_on = false;
    if (rc) return rc;
    ST_CUDA(cudaEventSynchronize(x->prof_ev[x->prof_n]));
    const int cnt = std::min(x->prof_n, max_n);
    std::string all;
    for (int k = 0; k < cnt; k++) {
        float t = 0.f;
        cudaEventElapsedTime(&t, x->prof_ev[k], x->prof_ev[k + 1]);
        ms[k] = t;
        if (k) all += ",";
        all += x->prof_name[k + 1];
    }
    if (names && names_len > 0) {
        std::strncpy(names, all.c_str(), names_len - 1);
        names[names_len - 1] = 0;
    }
    *n = cnt;
    return ST_OK;
}

int st_set_residual_path(st_ctx* x, int path, int* active) {
    if (!x || (path != 0 && path != 1)) return fail(ST_ERR_ARG, "st_set_residual_path: path must be 0 or 1");
    if (path == 1 && !x->tile_ok) return fail(ST_ERR_UNSUPPORTED, "st_set_residual_path: tiled sweeps unavailable");
    x->res_path = path;
    if (active) *active = (x->tile_ok && x->res_path == 1) ? 1 : 0;
    return ST_OK;
}

int st_last_kernel_ms(st_ctx* x, double* res_ms, double* vjp_ms) {
    if (!x) return fail(ST_ERR_ARG, "st_last_kernel_ms: null context");
    if (x->res_pending) {
        ST_CUDA(cudaEventSynchronize(x->ev[1]));
        cudaEventElapsedTime(&x->last_res_ms, x->ev[0], x->ev[1]);
        x->res_pending = false;
    }
    if (x->vjp_pending) {
        ST_CUDA(cudaEventSynchronize(x->ev[3]));
        cudaEventElapsedTime(&x->last_vjp_ms, x->ev[2], x->ev[3]);
        x->vjp_pending = false;
    }
    if (res_ms) *res_ms = x->last_res_ms;
    if (vjp_ms) *vjp_ms = x->last_vjp_ms;
    return ST_OK;
}

int st_device_state(st_ctx* x, double** q_dev, double** rhs_dev, void** stream) {
    if (!x) return fail(ST_ERR_ARG, "st_device_state: null context");
    if (q_dev) *q_dev = x->q;
    if (rhs_dev) *rhs_dev = x->rhs;
    if (stream) *stream = (void*)x->stream;
    return ST_OK;
}

}  // extern "C"
