// Shared device definitions for the structured-grid residual / adjoint path.
//
// Data layout in HBM (one context):
//   q     [nic][njc][nq]        conserved state, the reference's Solution::q
//                               (src/solver/solution.cpp:28), FP64
//   P     [nic+2][njc+2][8]     ghost-padded primitives per cell, 64 B records
//                               {rho,u,v,p,T,nu_tilde,mu,mu_t}; the reference
//                               keeps the first five as separate padded arrays
//                               (src/model/eulerequation.cpp:41-47)
//   phi_i, phi_j [nic][njc][NQ] MUSCL limiter factor per cell and primitive
//                               (src/model/reconstruction.cpp:85-113)
//   geo_i [ni][njc][16], geo_j [nic][nj][16]
//                               per-face geometry: normal (n_x,n_y), unit normal,
//                               half length, and the Green-Gauss weights of the
//                               face gradient of src/utils/mesh.cpp:36-131
//   F_i [ni][njc][NQ], F_j [nic][nj][NQ]  net face fluxes (convective - viscous)
//   G_i, G_j [..][4]            SA only: face gradient parts (u_y, v_x, nt_x, nt_y)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/structured_gb300.h"

namespace st {

constexpr double GAMMA = 1.4;
constexpr double GM1 = GAMMA - 1.0;
constexpr double OGM1 = 1.0 / GM1;
constexpr double THM = 2.0 / 3.0, THP = 4.0 / 3.0;   // reconstruction.h:55-56

// Spalart-Allmaras (SA-noft2, negative-S~ safeguard of Allmaras et al. 2012)
constexpr double SA_CB1 = 0.1355, SA_CB2 = 0.622, SA_SIGMA = 2.0 / 3.0, SA_KAPPA = 0.41;
constexpr double SA_CW2 = 0.3, SA_CW3 = 2.0, SA_CV1 = 7.1, SA_CV2 = 0.7, SA_CV3 = 0.9;
constexpr double SA_CW1 = SA_CB1 / (SA_KAPPA * SA_KAPPA) + (1.0 + SA_CB2) / SA_SIGMA;
constexpr double SA_CV1_3 = SA_CV1 * SA_CV1 * SA_CV1;
constexpr double SA_CW3_6 = SA_CW3 * SA_CW3 * SA_CW3 * SA_CW3 * SA_CW3 * SA_CW3;
constexpr double SA_C6 = 2.005174745150421541;  // (1 + c_w3^6)^(1/6) = 65^(1/6)
// negative-nu_tilde branch (SA-neg: Allmaras, Johnson & Spalart, ICCFD7-1902, 2012)
constexpr double SA_CT3 = 1.2, SA_CN1 = 16.0;
constexpr double PR_TURB = 0.9;

// primitive record slots
enum { P_RHO = 0, P_U, P_V, P_P, P_T, P_NUT, P_MU, P_MUT, NP = 8 };
// geometry record slots
enum { G_NX = 0, G_NY, G_R1, G_R2, G_AJ, G_WLX, G_WLY, G_WRX, G_WRY, G_WPX, G_WPY, G_WMX, G_WMY, NGEO = 16 };

struct DevBC {
    int type, face, start, end;
    double u, v, T;
};

// Everything a kernel needs about the case, passed by value.
struct DevCase {
    int ni, nj, nic, njc, nq;
    int viscous, sa, law, nbc;
    int flux;              // ST_FLUX_ROE / ST_FLUX_AUSM
    double R, cp, pr, rho_inf, u_inf, v_inf, p_inf, T_inf, mu_inf, nut_inf;
    double cp_pr, cp_prt;  // c_p / Pr and c_p / Pr_t (heat conductivity per unit viscosity)
    double iR, iT_inf;     // 1 / R, 1 / T_inf
    double suth_S, eps_chi, eps_eta, dpdx, dpdy;
    const double* vol;     // [nic][njc]
    const double* ivol;    // [nic][njc] 1/vol
    const double* geo_i;   // [ni][njc][NGEO]
    const double* geo_j;   // [nic][nj][NGEO]
    const double* wd;      // [nic][njc] wall distance
    const double* nchi;    // [ni][njc][2] (raw normals, for BCs)
    const double* neta;    // [nic][nj][2]
    const DevBC* bcs;      // [nbc]
    int* err;              // device error flag
    const void* mlp_wb;    // learned beta: BF16 weight block (null: beta from the beta array)
    const float* mlp_wf;   // its FP32 biases and feature normalisation
    int nonlocal_frozen;   // periodic and wake ghosts take their source's value with a zero tangent
};

__host__ __device__ inline size_t pidx(const DevCase& c, int ip, int jp) {
    return ((size_t)ip * (c.njc + 2) + jp) * NP;
}

// ---------------------------------------------------------------------------
// Reciprocal and square roots by Newton-Raphson refinement of the hardware
// approximations (PTX rcp.approx.ftz.f64 / rsqrt.approx.ftz.f64).  The FP64
// pipe issues about two instructions per clock per SM on this part, and the
// IEEE-rounded divide and square root take about ten of them each; a Newton
// step squares the relative error, so two steps from the hardware seed reach
// FP64 round-off (within a few ulp of the correctly rounded result; the GPU
// tests bound the error against 1.0 / x and sqrt(x)).  Inputs: positive,
// finite, normal numbers (densities, pressures, viscosities, sound speeds).
//   nr_rcp:   r <- r + r (1 - x r), twice                      (4 DFMA)
//   nr_rsqrt: y <- y + y (1/2 - (x/2) y^2), twice               (7)
//   nr_sqrt:  one rsqrt step, s = x y, then s + (y/2)(x - s^2)  (8)
//   nr_sqrt_inv: sqrt(x) and 1/sqrt(x) (two rsqrt steps, then the correction)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double nr_rcp(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}
__device__ __forceinline__ double rsqrt_seed(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    return y;
}
__device__ __forceinline__ double nr_rsqrt(double x) {
    double y = rsqrt_seed(x);
    const double mh = -0.5 * x;
    y = fma(y, fma(mh * y, y, 0.5), y);
    return fma(y, fma(mh * y, y, 0.5), y);
}
__device__ __forceinline__ double nr_sqrt(double x) {
    double y = rsqrt_seed(x);
    y = fma(y, fma(-0.5 * x * y, y, 0.5), y);
    const double s = x * y;
    return fma(0.5 * y, fma(-s, s, x), s);
}
__device__ __forceinline__ double nr_sqrt_inv(double x, double* inv) {
    const double y = nr_rsqrt(x);
    const double s = x * y;
    *inv = y;
    return fma(0.5 * y, fma(-s, s, x), s);
}

// w^(-1/6) for positive w below FP32 overflow (3e38) by Newton's iteration on q^-6 - w = 0,
// q <- q + (q/6)(1 - w q^6), twice from an FP32 seed w^(-1/6) by the fast
// single-precision power (about 18 correct bits; each step roughly squares
// the error, times 3.5).
__device__ __forceinline__ double nr_inv_root6(double w) {
    double q = (double)__powf((float)w, -1.0f / 6.0f);
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const double q2 = q * q;
        const double q6 = q2 * q2 * q2;
        q = fma(q * (1.0 / 6.0), fma(-w, q6, 1.0), q);
    }
    return q;
}

// ---------------------------------------------------------------------------
// forward-mode dual number (value, tangent) for exact JVPs on the device
// ---------------------------------------------------------------------------
struct dual {
    double v, d;
    __host__ __device__ dual() {}
    __host__ __device__ dual(double x) : v(x), d(0.0) {}
    __host__ __device__ dual(double x, double dx) : v(x), d(dx) {}
};
__device__ inline dual operator+(dual a, dual b) { return dual(a.v + b.v, a.d + b.d); }
__device__ inline dual operator-(dual a, dual b) { return dual(a.v - b.v, a.d - b.d); }
__device__ inline dual operator-(dual a) { return dual(-a.v, -a.d); }
__device__ inline dual operator*(dual a, dual b) { return dual(a.v * b.v, fma(a.d, b.v, a.v * b.d)); }
__device__ inline dual operator/(dual a, dual b) {
    double r = nr_rcp(b.v), q = a.v * r;
    return dual(q, (a.d - q * b.d) * r);
}
__device__ inline dual operator+(dual a, double b) { return dual(a.v + b, a.d); }
__device__ inline dual operator+(double b, dual a) { return dual(a.v + b, a.d); }
__device__ inline dual operator-(dual a, double b) { return dual(a.v - b, a.d); }
__device__ inline dual operator-(double b, dual a) { return dual(b - a.v, -a.d); }
__device__ inline dual operator*(dual a, double b) { return dual(a.v * b, a.d * b); }
__device__ inline dual operator*(double b, dual a) { return dual(a.v * b, a.d * b); }
__device__ inline dual operator/(dual a, double b) { double r = nr_rcp(b); return dual(a.v * r, a.d * r); }
__device__ inline bool operator>=(dual a, double b) { return a.v >= b; }
__device__ inline bool operator>(dual a, double b) { return a.v > b; }
__device__ inline bool operator<(dual a, double b) { return a.v < b; }

__device__ inline double val(double x) { return x; }
__device__ inline double val(dual x) { return x.v; }

// rcp / tsqrt: IEEE-rounded reciprocal and square root.  frcp: the
// Newton-Raphson reciprocal above.  Measured per kernel on this part (one
// fused residual + adjoint step at 4097x2049): frcp is the faster one in the
// cell-wise passes (primitives, limiter, SA source), the IEEE forms in the
// register-capped face passes.
__device__ inline double rcp(double x) { return 1.0 / x; }
__device__ inline double tsqrt(double x) { return ::sqrt(x); }
__device__ inline double tfabs(double x) { return ::fabs(x); }
__device__ inline dual rcp(dual x) { double r = 1.0 / x.v; return dual(r, -x.d * r * r); }
__device__ inline dual tsqrt(dual x) { double s = ::sqrt(x.v); return dual(s, x.d * 0.5 / s); }
__device__ inline double frcp(double x) { return nr_rcp(x); }
__device__ inline dual frcp(dual x) { double r = nr_rcp(x.v); return dual(r, -x.d * r * r); }
// sqrt(x) with 1/sqrt(x) in *inv
__device__ inline double tsqrt_inv(double x, double* inv) { return nr_sqrt_inv(x, inv); }
__device__ inline dual tsqrt_inv(dual x, dual* inv) {
    double y;
    const double s = nr_sqrt_inv(x.v, &y);
    *inv = dual(y, -0.5 * x.d * y * y * y);
    return dual(s, x.d * 0.5 * y);
}
__device__ inline dual tfabs(dual x) { return x.v < 0.0 ? -x : x; }
__device__ inline double cbrt_(double x) { return ::cbrt(x); }
__device__ inline dual cbrt_(dual x) { double c = ::cbrt(x.v); return dual(c, x.d * c / (3.0 * x.v)); }
// x^(-1/6) for x > 0 (nr_inv_root6)
__device__ inline double inv_root6(double x) { return nr_inv_root6(x); }
__device__ inline dual inv_root6(dual x) {
    const double q = nr_inv_root6(x.v), q2 = q * q;
    return dual(q, x.d * (-1.0 / 6.0) * (q2 * q2 * q2 * q));  // d/dx x^(-1/6) = -(1/6) x^(-7/6)
}

template <class T> __device__ inline T tmin(T a, double b) { return val(a) < b ? a : T(b); }

// Laminar viscosity: power law of the reference (src/model/fluid.cpp:38-40,
// (T/T_ref)^(2/3) evaluated as cbrt(x)^2) or Sutherland.
template <class T>
__device__ inline T laminar_mu(const DevCase& c, T temp) {
    if (c.law == 1) {
        T tr = temp * c.iT_inf;
        return c.mu_inf * tr * tsqrt(tr) * ((c.T_inf + c.suth_S) * frcp(temp + c.suth_S));
    }
    T cb = cbrt_(temp * c.iT_inf);
    return c.mu_inf * (cb * cb);
}

// SA eddy viscosity mu_t = rho nu_tilde f_v1(chi), chi = rho nu_tilde / mu;
// zero for nu_tilde < 0 (SA-neg)
template <class T>
__device__ inline T sa_mut(T rho, T nut, T mu) {
    if (val(nut) < 0.0) return T(0.0);
    T chi = rho * nut * frcp(mu);
    T chi3 = chi * chi * chi;
    return rho * nut * (chi3 * frcp(chi3 + SA_CV1_3));
}

// The nu_tilde part of the SA diffusion coefficient, rho nu_tilde f_n(chi):
// f_n = 1 for nu_tilde >= 0, (c_n1 + chi^3) / (c_n1 - chi^3) below (SA-neg),
// which keeps mu + rho nu_tilde f_n > 0.
template <class T>
__device__ inline T sa_diff(T rho, T nut, T mu) {
    const T m = rho * nut;
    if (val(nut) >= 0.0) return m;
    const T chi = m * rcp(mu);
    const T chi3 = chi * chi * chi;
    return m * ((SA_CN1 + chi3) * rcp(SA_CN1 - chi3));
}
// its partial derivatives with respect to rho, nu_tilde and mu
__device__ inline void sa_diff_d(double rho, double nut, double mu, double* d_rho, double* d_nut, double* d_mu) {
    if (nut >= 0.0) { *d_rho = nut; *d_nut = rho; *d_mu = 0.0; return; }
    const double m = rho * nut, chi = m / mu, chi3 = chi * chi * chi, den = SA_CN1 - chi3;
    const double fn = (SA_CN1 + chi3) / den;
    const double fnp = 6.0 * SA_CN1 * chi * chi / (den * den);  // d f_n / d chi
    const double dm = fn + chi * fnp;
    *d_rho = dm * nut;
    *d_nut = dm * rho;
    *d_mu = -chi * chi * fnp;
}

// bounded mbarrier / flag spin helper limit
constexpr int SPIN_LIMIT = 1 << 22;

}  // namespace st
