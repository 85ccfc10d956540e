// Forward residual kernels, templated on the scalar (double for values,
// st::dual for exact JVPs).  Each restates a stage of the reference's
// EulerEquation::calc_residual (src/model/eulerequation.cpp:202-232) as one
// data-parallel pass; face work is done once per face (the reference also
// evaluates each face once, but through >40 full-grid temporaries).
#pragma once
#include "st_common.cuh"
#include "st_mlp.cuh"

namespace st {

// ----------------------------------------------------------------------------
// K1  conserved -> primitives, FluidModel::primvars (src/model/fluid.cpp:50-67)
//     plus mu(T) (fluid.cpp:38-40) and SA mu_t.  One thread per cell.
// ----------------------------------------------------------------------------
template <class T, int NQ>
__global__ void __launch_bounds__(256) k_prim(DevCase c, const T* __restrict__ q, T* __restrict__ P) {
    const size_t n = (size_t)c.nic * c.njc;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / c.njc), j = (int)(idx % c.njc);
        const T* Q = q + idx * NQ;
        T rho = Q[0];
        T ri = frcp(rho);
        T u = Q[1] * ri, v = Q[2] * ri;
        T p = (Q[3] - 0.5 * rho * (u * u + v * v)) * GM1;
        T temp = p * ri * c.iR;
        T nut = (NQ == 5) ? Q[NQ - 1] * ri : T(0.0);
        T mu = c.viscous ? laminar_mu(c, temp) : T(0.0);
        T mut = (NQ == 5 && c.viscous) ? sa_mut(rho, nut, mu) : T(0.0);
        T* o = P + pidx(c, i + 1, j + 1);
        o[P_RHO] = rho; o[P_U] = u; o[P_V] = v; o[P_P] = p;
        o[P_T] = temp; o[P_NUT] = nut; o[P_MU] = mu; o[P_MUT] = mut;
    }
}

// ----------------------------------------------------------------------------
// K2  ghost layer from the boundary list in list order
//     (BoundaryContainer::apply, src/model/bc.cpp:430-433; each BC type
//     restates its apply() in bc.cpp:26-427).  One CTA: BCs are sequential
//     because later ones read ghosts written by earlier ones (corners).
// ----------------------------------------------------------------------------
template <class T>
__device__ inline void bc_copy(T* g, const T* s) {
    g[P_RHO] = s[P_RHO]; g[P_U] = s[P_U]; g[P_V] = s[P_V]; g[P_P] = s[P_P];
    g[P_T] = s[P_T]; g[P_NUT] = s[P_NUT];
}

// Non-local copy (periodic, wake).  With c.nonlocal_frozen (the implicit
// solver's colouring JVPs) a dual ghost keeps the source's value and a zero
// tangent: the copies' distant coupling is assembled separately.
template <class T>
__device__ inline void bc_copy_nl(const DevCase& c, T* g, const T* s) {
    if (c.nonlocal_frozen) {
        g[P_RHO] = T(val(s[P_RHO])); g[P_U] = T(val(s[P_U])); g[P_V] = T(val(s[P_V])); g[P_P] = T(val(s[P_P]));
        g[P_T] = T(val(s[P_T])); g[P_NUT] = T(val(s[P_NUT]));
    } else {
        bc_copy(g, s);
    }
}

// Boundary condition b of the list, applied by threads tid = 0 .. nth-1 of a
// launch (or of a block).  The wake cut writes its two ghost halves in two
// parts (part 0, then part 1 after every thread finished part 0); every other
// type is done in part 0 and ignores part 1.
template <class T, int NQ>
__device__ void bc_apply_one(const DevCase& c, T* __restrict__ P, int b, int part, int tid, int nth) {
    const int nic = c.nic, njc = c.njc;
    const double iR = c.iR;
    {
        const DevBC bc = c.bcs[b];
        const bool bt = (bc.face == 0 || bc.face == 2);
        const int end = bc.end >= 0 ? bc.end : (bt ? nic : njc) + 2 + bc.end;
        const int start = bc.start;
        if (part == 1 && bc.type != 6) return;
        if (bc.type == 0) {  // freestream, bc.cpp:26-60
            for (int s = start + tid; s <= end; s += nth) {
                int ip = bt ? s : (bc.face == 3 ? 0 : nic + 1);
                int jp = bt ? (bc.face == 0 ? 0 : njc + 1) : s;
                T* g = P + pidx(c, ip, jp);
                g[P_RHO] = c.rho_inf; g[P_U] = c.u_inf; g[P_V] = c.v_inf; g[P_P] = c.p_inf;
                g[P_T] = T(c.p_inf) * rcp(T(c.rho_inf)) * iR;
                g[P_NUT] = c.nut_inf;
            }
        } else if (bc.type == 1) {  // slip wall, bc.cpp:78-128
            if (bt) {
                for (int ip = start + tid; ip <= end; ip += nth) {
                    const bool bot = (bc.face == 0);
                    const int jg = bot ? 0 : njc + 1, j1 = bot ? 1 : njc, j2 = bot ? 2 : njc - 1;
                    const double* nn = c.neta + ((size_t)(ip - 1) * c.nj + (bot ? 0 : njc)) * 2;
                    const double nx = nn[0], ny = nn[1];
                    const double ds = nx * nx + ny * ny;
                    T* g = P + pidx(c, ip, jg);
                    const T* a = P + pidx(c, ip, j1);
                    const T* d = P + pidx(c, ip, j2);
                    g[P_P] = 1.5 * a[P_P] - 0.5 * d[P_P];
                    g[P_RHO] = 1.5 * a[P_RHO] - 0.5 * d[P_RHO];
                    T un = a[P_U] * nx + a[P_V] * ny;
                    g[P_U] = a[P_U] - 2.0 * un * nx / ds;
                    g[P_V] = a[P_V] - 2.0 * un * ny / ds;
                    g[P_T] = g[P_P] * rcp(g[P_RHO]) * iR;
                    g[P_NUT] = 1.5 * a[P_NUT] - 0.5 * d[P_NUT];
                }
            }
        } else if (bc.type == 2 || bc.type == 5) {  // adiabatic wall bc.cpp:150-204, isothermal :388-427
            for (int s = start + tid; s <= end; s += nth) {
                T *g; const T *a, *d;
                if (bt) {
                    const bool bot = (bc.face == 0);
                    g = P + pidx(c, s, bot ? 0 : njc + 1);
                    a = P + pidx(c, s, bot ? 1 : njc);
                    d = P + pidx(c, s, bot ? 2 : njc - 1);
                } else {
                    if (bc.type == 5) break;  // isothermal: bottom/top only
                    const bool left = (bc.face == 3);
                    g = P + pidx(c, left ? 0 : nic + 1, s);
                    a = P + pidx(c, left ? 1 : nic, s);
                    d = P + pidx(c, left ? 2 : nic - 1, s);
                }
                g[P_U] = 2.0 * bc.u - (1.5 * a[P_U] - 0.5 * d[P_U]);
                g[P_V] = 2.0 * bc.v - (1.5 * a[P_V] - 0.5 * d[P_V]);
                if (bc.type == 2) {
                    g[P_T] = 1.5 * a[P_T] - 0.5 * d[P_T];
                    g[P_RHO] = 1.5 * a[P_RHO] - 0.5 * d[P_RHO];
                    g[P_P] = g[P_RHO] * c.R * g[P_T];
                } else {
                    g[P_P] = 1.5 * a[P_P] - 0.5 * d[P_P];
                    g[P_T] = bc.T;
                    g[P_RHO] = g[P_P] * rcp(g[P_T]) * iR;
                }
                g[P_NUT] = -(1.5 * a[P_NUT] - 0.5 * d[P_NUT]);
            }
        } else if (bc.type == 3) {  // outflow, bc.cpp:284-311 (right face)
            if (!bt && bc.face == 1) {
                for (int jp = start + tid; jp <= end; jp += nth) {
                    T* g = P + pidx(c, nic + 1, jp);
                    const T* a = P + pidx(c, nic, jp);
                    g[P_RHO] = a[P_RHO]; g[P_U] = a[P_U]; g[P_V] = a[P_V]; g[P_P] = c.p_inf;
                    g[P_T] = g[P_P] * rcp(g[P_RHO]) * iR;
                    g[P_NUT] = a[P_NUT];
                }
            }
        } else if (bc.type == 4) {  // periodic, bc.cpp:329-365
            for (int s = start + tid; s <= end; s += nth) {
                if (bt) {
                    bc_copy_nl(c, P + pidx(c, s, 0), P + pidx(c, s, njc));
                    bc_copy_nl(c, P + pidx(c, s, njc + 1), P + pidx(c, s, 1));
                } else {
                    bc_copy_nl(c, P + pidx(c, 0, s), P + pidx(c, nic, s));
                    bc_copy_nl(c, P + pidx(c, nic + 1, s), P + pidx(c, 1, s));
                }
            }
        } else if (bc.type == 6) {  // wake, bc.cpp:224-263
            if (bt) {
                const int jg = (bc.face == 0) ? 0 : njc + 1;
                if (part == 0)
                    for (int ip = start + tid; ip <= end; ip += nth)
                        bc_copy_nl(c, P + pidx(c, ip, jg), P + pidx(c, nic + 1 - ip, 1));
                else
                    for (int ip = start + tid; ip <= end; ip += nth)
                        bc_copy_nl(c, P + pidx(c, nic + 1 - ip, jg), P + pidx(c, ip, 1));
            }
        }
    }
}

// All threads of the block apply c.bcs[0..nbc) in order.
template <class T, int NQ>
__device__ void bc_apply_block(const DevCase& c, T* __restrict__ P) {
    for (int b = 0; b < c.nbc; b++) {
        for (int part = 0; part < 2; part++) {
            bc_apply_one<T, NQ>(c, P, b, part, threadIdx.x, blockDim.x);
            __syncthreads();
        }
    }
}

// mu, mu_t of every ghost cell (eulerequation.cpp:183-188 covers the whole
// padded array)
template <class T, int NQ>
__device__ void bc_ghost_mu(const DevCase& c, T* __restrict__ P, int tid, int nth) {
    const int nic = c.nic, njc = c.njc;
    {
        const int nring = 2 * (nic + 2) + 2 * njc;
        for (int r = tid; r < nring; r += nth) {
            int ip, jp;
            if (r < nic + 2) { ip = r; jp = 0; }
            else if (r < 2 * (nic + 2)) { ip = r - (nic + 2); jp = njc + 1; }
            else if (r < 2 * (nic + 2) + njc) { ip = 0; jp = r - 2 * (nic + 2) + 1; }
            else { ip = nic + 1; jp = r - 2 * (nic + 2) - njc + 1; }
            T* g = P + pidx(c, ip, jp);
            T mu = laminar_mu(c, g[P_T]);
            g[P_MU] = mu;
            g[P_MUT] = (NQ == 5 && val(mu) != 0.0) ? sa_mut(g[P_RHO], g[P_NUT], mu) : T(0.0);
        }
    }
}

template <class T, int NQ>
__global__ void __launch_bounds__(1024) k_bc(DevCase c, T* __restrict__ P) {
    bc_apply_block<T, NQ>(c, P);
    if (c.viscous) bc_ghost_mu<T, NQ>(c, P, threadIdx.x, blockDim.x);
}

// The same boundary pass as a sequence of grid-wide launches: one per
// boundary condition (two for a wake cut), in list order, then the ghost
// viscosities (bc_launches in the host code issues them).
template <class T, int NQ>
__global__ void __launch_bounds__(256) k_bc_one(DevCase c, T* __restrict__ P, int b, int part) {
    bc_apply_one<T, NQ>(c, P, b, part, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}
template <class T, int NQ>
__global__ void __launch_bounds__(256) k_bc_mu(DevCase c, T* __restrict__ P) {
    bc_ghost_mu<T, NQ>(c, P, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// Host side: the boundary pass as grid-wide launches on stream s (bcs: the
// host copy of the list, for the wake cut's second part).
template <class T, int NQ>
inline void launch_bcs(const DevCase& dc, const st_bc* bcs, int nbc, T* P, cudaStream_t s) {
    const unsigned g = (unsigned)((max(dc.nic, dc.njc) + 2 + 255) / 256);
    for (int b = 0; b < nbc; b++) {
        k_bc_one<T, NQ><<<g, 256, 0, s>>>(dc, P, b, 0);
        if (bcs[b].type == ST_BC_WAKE) k_bc_one<T, NQ><<<g, 256, 0, s>>>(dc, P, b, 1);
    }
    if (dc.viscous) k_bc_mu<T, NQ><<<(unsigned)((2 * (dc.nic + 2) + 2 * dc.njc + 255) / 256), 256, 0, s>>>(dc, P);
}

// ----------------------------------------------------------------------------
// K3  MUSCL slopes per cell and direction, ReconstructionSecondOrder
//     (src/model/reconstruction.cpp:85-113): with d- = P(c)-P(c-1),
//     d+ = P(c+1)-P(c) and the limiter
//         phi = 0.25 (3 d+ d- + eps) / (2 (d+ - d-)^2 + 3 d+ d- + eps),
//     the cell's high face sees P + sL, its low face P - sR, where
//         sL = phi (THM d- + THP d+),  sR = phi (THP d- + THM d+).
//     With ADJ the kernel also stores dsL/dd-, dsL/dd+, dsR/dd-, dsR/dd+ for
//     the adjoint, from the same reciprocal.
// lim layout: group-major [group][cell][5]; groups 0..3 = (sL,sR) of i then j,
// groups 4..11 = (dsL/dd-, dsL/dd+, dsR/dd-, dsR/dd+) of i then j.
// ----------------------------------------------------------------------------
enum { LIM_SL = 0, LIM_SR = 1, LIM_AM = 2, LIM_AP = 3, LIM_BM = 4, LIM_BP = 5 };
__host__ __device__ inline size_t lim_off(const DevCase& c, int dir, int g, size_t cell) {
    const int grp = g < 2 ? dir * 2 + g : 4 + dir * 4 + (g - 2);
    return ((size_t)grp * ((size_t)c.nic * c.njc) + cell) * 5;
}

template <class T, int NQ, bool ADJ>
__global__ void __launch_bounds__(256) k_limiter(DevCase c, const T* __restrict__ P, T* __restrict__ lim) {
    const size_t n = (size_t)c.nic * c.njc;
    const int slot[5] = {P_RHO, P_U, P_V, P_P, P_NUT};
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / c.njc), j = (int)(idx % c.njc);
        const T* pc = P + pidx(c, i + 1, j + 1);
#pragma unroll
        for (int dir = 0; dir < 2; dir++) {
            const T* pm = dir == 0 ? P + pidx(c, i, j + 1) : P + pidx(c, i + 1, j);
            const T* pp = dir == 0 ? P + pidx(c, i + 2, j + 1) : P + pidx(c, i + 1, j + 2);
            const double eps = dir == 0 ? c.eps_chi : c.eps_eta;
#pragma unroll
            for (int k = 0; k < NQ; k++) {
                const int m = slot[k];
                const T fa = pc[m] - pm[m], fb = pp[m] - pc[m];
                const T a1 = 3.0 * fb * fa;
                const T inv = frcp(2.0 * (fb - fa) * (fb - fa) + a1 + eps);
                const T ph = 0.25 * (a1 + eps) * inv;
                const T tl = THM * fa + THP * fb, tr = THP * fa + THM * fb;
                lim[lim_off(c, dir, LIM_SL, idx) + k] = ph * tl;
                lim[lim_off(c, dir, LIM_SR, idx) + k] = ph * tr;
                if (ADJ) {
                    // d phi / d d-, d+: 3 d+ - 4 (d+ - d-) = 4 d- - d+, 3 d- + 4 (d+ - d-) = 4 d+ - d-
                    const T dfa = (0.75 * fb - ph * (4.0 * fa - fb)) * inv;
                    const T dfb = (0.75 * fa - ph * (4.0 * fb - fa)) * inv;
                    lim[lim_off(c, dir, LIM_AM, idx) + k] = ph * THM + tl * dfa;
                    lim[lim_off(c, dir, LIM_AP, idx) + k] = ph * THP + tl * dfb;
                    lim[lim_off(c, dir, LIM_BM, idx) + k] = ph * THP + tr * dfa;
                    lim[lim_off(c, dir, LIM_BP, idx) + k] = ph * THM + tr * dfb;
                }
            }
        }
    }
}

// ----------------------------------------------------------------------------
// AUSM flux, ConvectiveFluxAUSM::evaluate (src/model/flux.cpp:148-224): split
// Mach numbers and pressures (van Leer polynomials for |M| <= 1), upwinded by
// the sign of the interface Mach number; nx, ny the face normal scaled by its
// length ds.
// ----------------------------------------------------------------------------
template <class T>
__device__ inline T ausm_mach(T M, double s) {  // s = +1: M+, s = -1: M-
    if (val(tfabs(M)) <= 1.0) return (0.25 * s) * (M + s) * (M + s);
    return 0.5 * (M + s * tfabs(M));
}
template <class T>
__device__ inline T ausm_pres(T M, T p, double s) {
    if (val(tfabs(M)) <= 1.0) return 0.25 * p * (M + s) * (M + s) * (2.0 - s * M);
    return 0.5 * p * (M + s * tfabs(M)) * rcp(M);
}
template <class T>
__device__ inline void ausm_flux(T rlft, T ulft, T vlft, T plft, T rrht, T urht, T vrht, T prht, double nx, double ny,
                                 double ds, T* f) {
    const double ids = 1.0 / ds;
    const T alft = tsqrt(GAMMA * plft * rcp(rlft));
    const T arht = tsqrt(GAMMA * prht * rcp(rrht));
    const T mlft = (ulft * nx + vlft * ny) * ids * rcp(alft);
    const T mrht = (urht * nx + vrht * ny) * ids * rcp(arht);
    const T mhalf = ausm_mach(mlft, 1.0) + ausm_mach(mrht, -1.0);
    const T phalf = ausm_pres(mlft, plft, 1.0) + ausm_pres(mrht, prht, -1.0);
    const bool left = val(mhalf) >= 0.0;
    const T r = left ? rlft : rrht, a = left ? alft : arht, u = left ? ulft : urht, v = left ? vlft : vrht;
    const T p = left ? plft : prht;
    const T h = (p * OGM1 + r * (0.5 * (u * u + v * v)) + p) * rcp(r);
    const T m = r * a * mhalf * ds;
    f[0] = m;
    f[1] = m * u + phalf * nx;
    f[2] = m * v + phalf * ny;
    f[3] = m * h;
}

// ----------------------------------------------------------------------------
// Roe flux, ConvectiveFluxRoe::evaluate (src/model/flux.cpp:51-146), with the
// face's unit normal and half length precomputed.
// ----------------------------------------------------------------------------
template <class T>
__device__ inline void roe_flux(T rlft, T ulft, T vlft, T plft, T rrht, T urht, T vrht, T prht,
                                double r1, double r2, double aj, T* f) {
    const T rlfti = rcp(rlft);
    const T rulft = rlft * ulft;
    const T rvlft = rlft * vlft;
    const T uvl = 0.5 * (ulft * ulft + vlft * vlft);
    const T elft = plft * OGM1 + rlft * uvl;
    const T hlft = (elft + plft) * rlfti;
    const T rrhti = rcp(rrht);
    const T rurht = rrht * urht;
    const T rvrht = rrht * vrht;
    const T uvr = 0.5 * (urht * urht + vrht * vrht);
    const T erht = prht * OGM1 + rrht * uvr;
    const T hrht = (erht + prht) * rrhti;
    const T rat = tsqrt(rrht * rlfti);
    const T rati = rcp(rat + 1.0);
    const T rav = rat * rlft;
    const T uav = (rat * urht + ulft) * rati;
    const T vav = (rat * vrht + vlft) * rati;
    const T hav = (rat * hrht + hlft) * rati;
    const T uv = 0.5 * (uav * uav + vav * vav);
    T icav;
    const T cav = tsqrt_inv(GM1 * (hav - uv), &icav);
    const T aq1 = rrht - rlft, aq2 = urht - ulft, aq3 = vrht - vlft, aq4 = prht - plft;
    const T uu = r1 * uav + r2 * vav;
    const T c2 = cav * cav;
    const T c2i = icav * icav;
    const T auu = tfabs(uu);
    const T aupc = tfabs(uu + cav);
    const T aumc = tfabs(uu - cav);
    const T uulft = r1 * ulft + r2 * vlft;
    const T uurht = r1 * urht + r2 * vrht;
    const T rcav = rav * cav;
    const T aquu = uurht - uulft;
    const T c2ih = 0.5 * c2i;
    const T ruuav = auu * rav;
    const T b1 = auu * (aq1 - c2i * aq4);
    const T b2 = c2ih * aupc * (aq4 + rcav * aquu);
    const T b3 = c2ih * aumc * (aq4 - rcav * aquu);
    const T b4 = b1 + b2 + b3;
    const T b5 = cav * (b2 - b3);
    const T b6 = ruuav * (aq2 - r1 * aquu);
    const T b7 = ruuav * (aq3 - r2 * aquu);
    const T d1 = b4;
    const T d2 = uav * b4 + r1 * b5 + b6;
    const T d3 = vav * b4 + r2 * b5 + b7;
    const T d4 = hav * b4 + uu * b5 + uav * b6 + vav * b7 - c2 * b1 * OGM1;
    const T plar = plft + prht;
    const T eplft = elft + plft;
    const T eprht = erht + prht;
    f[0] = aj * (rlft * uulft + rrht * uurht - d1);
    f[1] = aj * (rulft * uulft + rurht * uurht + r1 * plar - d2);
    f[2] = aj * (rvlft * uulft + rvrht * uurht + r2 * plar - d3);
    f[3] = aj * (eplft * uulft + eprht * uurht - d4);
}

// Face addressing shared by the i-face (DIR 0) and j-face (DIR 1) passes.
// A face has a low cell L and a high cell R along DIR, their outer
// neighbours LL and RR (MUSCL), and two side pairs (+, -) that close the
// Green-Gauss dual cell of src/utils/mesh.cpp:36-131.
struct FaceIdx {
    size_t L, R, LL, RR, Pa, Pb, Ma, Mb;  // primitive record offsets
    bool limL, limR;                       // L / R are physical cells
    size_t phL, phR;                       // physical cell index of L / R (if lim)
    size_t face;                           // face index in F/G/geo arrays
};

template <int DIR>
__device__ inline FaceIdx face_idx(const DevCase& c, int a, int b) {
    FaceIdx fi;
    if (DIR == 0) {  // i-face f=a in [0,ni), row j=b in [0,njc)
        const int f = a, j = b;
        fi.L = pidx(c, f, j + 1); fi.R = pidx(c, f + 1, j + 1);
        fi.limL = f >= 1; fi.limR = f <= c.nic - 1;
        fi.LL = fi.limL ? pidx(c, f - 1, j + 1) : fi.L;
        fi.RR = fi.limR ? pidx(c, f + 2, j + 1) : fi.R;
        fi.Pa = pidx(c, f, j + 2); fi.Pb = pidx(c, f + 1, j + 2);
        fi.Ma = pidx(c, f, j); fi.Mb = pidx(c, f + 1, j);
        fi.phL = (size_t)(f - 1) * c.njc + j; fi.phR = (size_t)f * c.njc + j;
        fi.face = (size_t)f * c.njc + j;
    } else {  // j-face g=b in [0,nj), column i=a in [0,nic)
        const int i = a, g = b;
        fi.L = pidx(c, i + 1, g); fi.R = pidx(c, i + 1, g + 1);
        fi.limL = g >= 1; fi.limR = g <= c.njc - 1;
        fi.LL = fi.limL ? pidx(c, i + 1, g - 1) : fi.L;
        fi.RR = fi.limR ? pidx(c, i + 1, g + 2) : fi.R;
        fi.Pa = pidx(c, i + 2, g); fi.Pb = pidx(c, i + 2, g + 1);
        fi.Ma = pidx(c, i, g); fi.Mb = pidx(c, i, g + 1);
        fi.phL = (size_t)i * c.njc + (g - 1); fi.phR = (size_t)i * c.njc + g;
        fi.face = (size_t)i * c.nj + g;
    }
    return fi;
}

// ----------------------------------------------------------------------------
// K4/K5  face flux pass: MUSCL face states, Roe flux, and the viscous flux
//     (DiffusiveFluxGreenGauss::evaluate, src/model/flux.cpp:12-48) from the
//     face gradients (mesh.cpp:36-131) and face averages (mesh.cpp:10-32).
//     Writes the net flux F = F_conv - F_visc and, with SA, the gradient parts
//     the cell source needs.
// ----------------------------------------------------------------------------
// The net flux of one face from its six primitive records (L, R and the side
// pairs P, M that close the Green-Gauss dual cell) and the MUSCL slopes of L
// (its high-face slope sL) and R (its low-face slope sR), each null on a
// first-order side.  f[NQ]: F_conv - F_visc; with SA and viscosity g[4]
// receives the gradient parts (u_y, v_x, nut_x, nut_y) of the cell source.
// Shared by the per-face passes and the tiled sweeps (same arithmetic).
template <class T, int NQ>
__device__ __forceinline__ void face_flux(const DevCase& c, const double* __restrict__ gm, const T* pL, const T* pR,
                                          const T* pPa, const T* pPb, const T* pMa, const T* pMb, const T* sL,
                                          const T* sR, T* f, T* g) {
    const int slot[5] = {P_RHO, P_U, P_V, P_P, P_NUT};
    T qL[5], qR[5];
#pragma unroll
    for (int k = 0; k < NQ; k++) {
        const int m = slot[k];
        qL[k] = pL[m];
        qR[k] = pR[m];
        if (sL) qL[k] = qL[k] + sL[k];
        if (sR) qR[k] = qR[k] - sR[k];
    }
    if (c.flux == ST_FLUX_AUSM)
        ausm_flux(qL[0], qL[1], qL[2], qL[3], qR[0], qR[1], qR[2], qR[3], gm[G_NX], gm[G_NY], 2.0 * gm[G_AJ], f);
    else
        roe_flux(qL[0], qL[1], qL[2], qL[3], qR[0], qR[1], qR[2], qR[3], gm[G_R1], gm[G_R2], gm[G_AJ], f);
    if (NQ == 5) f[4] = f[0] * (val(f[0]) >= 0.0 ? qL[4] : qR[4]);
    if (c.viscous) {
        const double wLx = gm[G_WLX], wLy = gm[G_WLY], wRx = gm[G_WRX], wRy = gm[G_WRY];
        const double wPx = gm[G_WPX], wPy = gm[G_WPY], wMx = gm[G_WMX], wMy = gm[G_WMY];
        // gradient and face average of one slot
#define ST_GRAD(m, gx, gy, avg)                                                              \
        {                                                                                    \
            const T sP = pPa[m] + pPb[m], sM = pMa[m] + pMb[m];                              \
            gx = wLx * pL[m] + wRx * pR[m] + wPx * sP + wMx * sM;                            \
            gy = wLy * pL[m] + wRy * pR[m] + wPy * sP + wMy * sM;                            \
            avg = 0.375 * (pL[m] + pR[m]) + 0.0625 * (sP + sM);                              \
        }
        T dudx, dudy, ubar, dvdx, dvdy, vbar, dTdx, dTdy, Tbar;
        ST_GRAD(P_U, dudx, dudy, ubar)
        ST_GRAD(P_V, dvdx, dvdy, vbar)
        ST_GRAD(P_T, dTdx, dTdy, Tbar)
        (void)Tbar;
        const T mub = 0.375 * (pL[P_MU] + pR[P_MU]) + 0.0625 * (pPa[P_MU] + pPb[P_MU] + pMa[P_MU] + pMb[P_MU]);
        T mu = mub, k;
        if (NQ == 5) {
            const T mutb = 0.375 * (pL[P_MUT] + pR[P_MUT]) + 0.0625 * (pPa[P_MUT] + pPb[P_MUT] + pMa[P_MUT] + pMb[P_MUT]);
            mu = mub + mutb;
            k = mub * c.cp_pr + mutb * c.cp_prt;
        } else {
            k = mub * c.cp_pr;
        }
        const double nx = gm[G_NX], ny = gm[G_NY];
        const T tau_xy = mu * (dudy + dvdx);
        const T tau_xx = mu * (2.0 * dudx - 2.0 / 3.0 * (dudx + dvdy));
        const T tau_yy = mu * (2.0 * dvdy - 2.0 / 3.0 * (dudx + dvdy));
        const T q_x = -k * dTdx;
        const T q_y = -k * dTdy;
        f[1] = f[1] - (tau_xx * nx + tau_xy * ny);
        f[2] = f[2] - (tau_xy * nx + tau_yy * ny);
        f[3] = f[3] - ((ubar * tau_xx + vbar * tau_xy - q_x) * nx + (ubar * tau_xy + vbar * tau_yy - q_y) * ny);
        if (NQ == 5) {
            T dndx, dndy, nbar;
            ST_GRAD(P_NUT, dndx, dndy, nbar)
            (void)nbar;
#define ST_SD(p) sa_diff(p[P_RHO], p[P_NUT], p[P_MU])
            const T rnb = 0.375 * (ST_SD(pL) + ST_SD(pR)) + 0.0625 * (ST_SD(pPa) + ST_SD(pPb) + ST_SD(pMa) + ST_SD(pMb));
#undef ST_SD
            f[4] = f[4] - (1.0 / SA_SIGMA) * (mub + rnb) * (dndx * nx + dndy * ny);
            g[0] = dudy; g[1] = dvdx; g[2] = dndx; g[3] = dndy;
        }
#undef ST_GRAD
    }
}

template <class T, int NQ, int DIR, int ORDER>
__global__ void __launch_bounds__(256) k_face(DevCase c, const T* __restrict__ P, const T* __restrict__ lim,
                                              T* __restrict__ F, T* __restrict__ G) {
    const int na = DIR == 0 ? c.ni : c.nic;
    const int nb = DIR == 0 ? c.njc : c.nj;
    const size_t n = (size_t)na * nb;
    const double* geo = DIR == 0 ? c.geo_i : c.geo_j;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(idx / nb), b = (int)(idx % nb);
        const FaceIdx fi = face_idx<DIR>(c, a, b);
        const T* sL = (ORDER == 2 && fi.limL) ? lim + lim_off(c, DIR, LIM_SL, fi.phL) : nullptr;
        const T* sR = (ORDER == 2 && fi.limR) ? lim + lim_off(c, DIR, LIM_SR, fi.phR) : nullptr;
        T f[NQ], g[4];
        face_flux<T, NQ>(c, geo + fi.face * NGEO, P + fi.L, P + fi.R, P + fi.Pa, P + fi.Pb, P + fi.Ma, P + fi.Mb, sL,
                         sR, f, g);
        if (NQ == 5 && c.viscous) {
            T* go = G + fi.face * 4;
#pragma unroll
            for (int t = 0; t < 4; t++) go[t] = g[t];
        }
        T* o = F + fi.face * NQ;
#pragma unroll
        for (int k = 0; k < NQ; k++) o[k] = f[k];
    }
}

// SA source per unit volume: rho (beta P - D) + (cb2/sigma) rho |grad nut|^2,
// P = cb1 S~ nut, D = cw1 fw (nut/d)^2 (Spalart & Allmaras 1992, SA-noft2);
// for nut < 0 (SA-neg) P = cb1 (1 - ct3) Omega nut, D = -cw1 (nut/d)^2.
// fw = g ((1 + cw3^6) / (g^6 + cw3^6))^(1/6) is evaluated as
// g (1 + cw3^6)^(1/6) (g^6 + cw3^6)^(-1/6), with one reciprocal per
// quotient and the inverse sixth root by Newton's iteration.
template <class T>
__device__ inline T sa_source(T rho, T nut, T mu, double d, T omega, T gnut2, T beta) {
    const double id2 = nr_rcp(d * d);
    if (val(nut) < 0.0)
        return rho * (beta * (SA_CB1 * (1.0 - SA_CT3)) * omega * nut + SA_CW1 * (nut * nut) * id2)
             + (SA_CB2 / SA_SIGMA) * rho * gnut2;
    const double ik2d2 = id2 * (1.0 / (SA_KAPPA * SA_KAPPA));
    const T chi = rho * nut * frcp(mu);
    const T chi3 = chi * chi * chi;
    const T fv1 = chi3 * frcp(chi3 + SA_CV1_3);
    const T fv2 = 1.0 - chi * frcp(1.0 + chi * fv1);
    const T sbar = nut * fv2 * ik2d2;
    T stilde;
    if (val(sbar) >= -SA_CV2 * val(omega)) stilde = omega + sbar;
    else stilde = omega + omega * (SA_CV2 * SA_CV2 * omega + SA_CV3 * sbar) * frcp((SA_CV3 - 2.0 * SA_CV2) * omega - sbar);
    T r;
    if (val(stilde) > 0.0) r = tmin(nut * frcp(stilde) * ik2d2, 10.0);
    else r = T(10.0);
    const T r2 = r * r;
    const T gg = r + SA_CW2 * (r2 * r2 * r2 - r);
    const T g2 = gg * gg;
    const T fw = gg * (SA_C6 * inv_root6(g2 * g2 * g2 + SA_CW3_6));
    const T prod = beta * SA_CB1 * stilde * nut;
    const T dest = SA_CW1 * fw * (nut * nut) * id2;
    return rho * (prod - dest) + (SA_CB2 / SA_SIGMA) * rho * gnut2;
}

// ----------------------------------------------------------------------------
// K6  cell assembly: flux differences (eulerequation.cpp:136-154, :5-20),
//     SA source, body force (:22-29), division by volume (:223-230).
// ----------------------------------------------------------------------------
// MLP: beta of each cell from the learned correction (st_mlp.cuh), evaluated
// in-kernel 32 cells per warp; the loop then runs over whole-warp tiles so
// that every lane reaches the warp-wide MMAs.
// The pass covers the cells [first, n) (a band of the grid when the host
// call copies the residual out band by band).
template <class T, int NQ, bool MLP = false>
__global__ void __launch_bounds__(256) k_cell(DevCase c, const T* __restrict__ P, const T* __restrict__ Fi,
                                              const T* __restrict__ Fj, const T* __restrict__ Gi,
                                              const T* __restrict__ Gj, const T* __restrict__ beta,
                                              T* __restrict__ rhs, size_t first, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t base = first + (size_t)blockIdx.x * blockDim.x + (MLP ? (threadIdx.x & ~31u) : threadIdx.x);
         base < n; base += stride) {
        const size_t idx = MLP ? base + (threadIdx.x & 31) : base;
        float mlp_beta = 1.f;
        if constexpr (MLP) {
            __shared__ __nv_bfloat16 s_x[8 * MLP_SX], s_h[8 * MLP_SH];
            const int w = threadIdx.x >> 5;
            float f[MLP_IN] = {0.f, 0.f, 0.f, 0.f};
            if (idx < n) {
                sa_features(c, P, Gj, (int)(idx / c.njc), (int)(idx % c.njc), f);
                mlp_normalise(c.mlp_wf, f);
            }
            mlp_beta = mlp_warp_beta((const __nv_bfloat16*)c.mlp_wb, c.mlp_wf, f, s_x + w * MLP_SX, s_h + w * MLP_SH);
            if (idx >= n) continue;
        }
        const int i = (int)(idx / c.njc), j = (int)(idx % c.njc);
        const T* fs = Fj + ((size_t)i * c.nj + j) * NQ;
        const T* fn = fs + NQ;
        const T* fw = Fi + ((size_t)i * c.njc + j) * NQ;
        const T* fe = Fi + ((size_t)(i + 1) * c.njc + j) * NQ;
        T r[NQ];
#pragma unroll
        for (int k = 0; k < NQ; k++) r[k] = (fs[k] - fn[k]) + (fw[k] - fe[k]);
        const double vol = c.vol[idx];
        if (NQ == 5 && c.viscous) {
            const T* gw = Gi + ((size_t)i * c.njc + j) * 4;
            const T* ge = Gi + ((size_t)(i + 1) * c.njc + j) * 4;
            const T* gs = Gj + ((size_t)i * c.nj + j) * 4;
            const T* gn = Gj + ((size_t)i * c.nj + j + 1) * 4;
            const T uy = 0.25 * (gw[0] + ge[0] + gs[0] + gn[0]);
            const T vx = 0.25 * (gw[1] + ge[1] + gs[1] + gn[1]);
            const T nx = 0.25 * (gw[2] + ge[2] + gs[2] + gn[2]);
            const T ny = 0.25 * (gw[3] + ge[3] + gs[3] + gn[3]);
            const T omega = tfabs(vx - uy);
            const T* pc = P + pidx(c, i + 1, j + 1);
            const T bta = MLP ? T((double)mlp_beta) : (beta ? beta[idx] : T(1.0));
            const T s = sa_source(pc[P_RHO], pc[P_NUT], pc[P_MU], c.wd[idx], omega, nx * nx + ny * ny, bta);
            r[NQ - 1] = r[NQ - 1] + s * vol;
        }
        r[1] = r[1] + (-c.dpdx * vol);
        r[2] = r[2] + (-c.dpdy * vol);
        const double iv = c.ivol[idx];
        T* o = rhs + idx * NQ;
#pragma unroll
        for (int k = 0; k < NQ; k++) o[k] = r[k] * iv;
    }
}

}  // namespace st
