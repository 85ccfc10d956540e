// Test infrastructure (oracle): FP64 CPU restatement of the reference
// residual path, extended with the parts the reference does not have
// (Spalart-Allmaras transport of rho*nu_tilde with a production multiplier
// beta, Sutherland viscosity, wall skin-friction objective, exact JVPs and
// Jacobian-transpose products).  It is the checker for the CUDA library,
// never the product: only tests/, the smoke check and bench.py's CPU
// baseline load libport.so.
//
// The laminar part restates, step by step and in the reference's operation
// order, src/model/eulerequation.cpp:202-232 (calc_residual) with
//   primvars        src/model/fluid.cpp:50-67
//   boundary conds  src/model/bc.cpp:26-433
//   MUSCL + limiter src/model/reconstruction.cpp:16-154
//   Roe flux        src/model/flux.cpp:51-146
//   face gradients  src/utils/mesh.cpp:10-131
//   viscous flux    src/model/flux.cpp:12-48
//   metrics         src/utils/mesh.cpp:172-205
//   calc_dt         src/model/eulerequation.cpp:237-259
// and is pinned against the compiled reference by tests/test_oracle.py.
//
// The residual is templated on the scalar: double for values, Dual for
// forward-mode derivatives.
#include "../../include/structured_gb300.h"
#include "dual.h"

#include <algorithm>
#include <cmath>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <cstring>
#include <vector>

namespace {

constexpr double GAMMA = 1.4;

// Spalart-Allmaras constants (Spalart & Allmaras 1992; SA-noft2 with the
// negative-S~ safeguard of Allmaras, Johnson & Spalart, ICCFD7 2012).
constexpr double SA_CB1 = 0.1355, SA_CB2 = 0.622, SA_SIGMA = 2.0 / 3.0, SA_KAPPA = 0.41;
constexpr double SA_CW2 = 0.3, SA_CW3 = 2.0, SA_CV1 = 7.1, SA_CV2 = 0.7, SA_CV3 = 0.9;
constexpr double SA_CW1 = SA_CB1 / (SA_KAPPA * SA_KAPPA) + (1.0 + SA_CB2) / SA_SIGMA;
// negative-nu_tilde branch (SA-neg: Allmaras, Johnson & Spalart, ICCFD7-1902, 2012)
constexpr double SA_CT3 = 1.2, SA_CN1 = 16.0;
constexpr double PR_TURB = 0.9;

struct PCase {
    st_case c;
    std::vector<st_bc> bcs;
    int ni, nj, nic, njc, nq;
    bool viscous, sa;
    bool freeze_nonlocal = false;  // periodic and wake ghosts copy values only (tangent 0)
    double R, cp;
    double eps_chi, eps_eta;
    std::vector<double> xv, yv, nchi, neta, vol, ds_chi, ds_eta, xc, yc, wd;
    double& NCHI(int i, int j, int k) { return nchi[((size_t)i * njc + j) * 2 + k]; }
    double& NETA(int i, int j, int k) { return neta[((size_t)i * nj + j) * 2 + k]; }
    double NCHI(int i, int j, int k) const { return nchi[((size_t)i * njc + j) * 2 + k]; }
    double NETA(int i, int j, int k) const { return neta[((size_t)i * nj + j) * 2 + k]; }
    double VOL(int i, int j) const { return vol[(size_t)i * njc + j]; }
};

// Mesh::calc_metrics, src/utils/mesh.cpp:172-205
void compute_metrics(PCase& pc) {
    const int ni = pc.ni, nj = pc.nj, nic = pc.nic, njc = pc.njc;
    auto X = [&](int i, int j) { return pc.xv[(size_t)i * nj + j]; };
    auto Y = [&](int i, int j) { return pc.yv[(size_t)i * nj + j]; };
    pc.nchi.assign((size_t)ni * njc * 2, 0.0);
    pc.neta.assign((size_t)nic * nj * 2, 0.0);
    pc.vol.assign((size_t)nic * njc, 0.0);
    pc.ds_chi.assign((size_t)nic * njc, 0.0);
    pc.ds_eta.assign((size_t)nic * njc, 0.0);
    pc.xc.assign((size_t)nic * njc, 0.0);
    pc.yc.assign((size_t)nic * njc, 0.0);
    std::vector<double> reta((size_t)nic * nj * 2), rchi((size_t)ni * njc * 2);
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < nj; j++) {
            double rx = X(i + 1, j) - X(i, j), ry = Y(i + 1, j) - Y(i, j);
            reta[((size_t)i * nj + j) * 2 + 0] = rx;
            reta[((size_t)i * nj + j) * 2 + 1] = ry;
            pc.NETA(i, j, 0) = -ry;
            pc.NETA(i, j, 1) = rx;
        }
    for (int i = 0; i < ni; i++)
        for (int j = 0; j < njc; j++) {
            double rx = X(i, j + 1) - X(i, j), ry = Y(i, j + 1) - Y(i, j);
            rchi[((size_t)i * njc + j) * 2 + 0] = rx;
            rchi[((size_t)i * njc + j) * 2 + 1] = ry;
            pc.NCHI(i, j, 0) = ry;
            pc.NCHI(i, j, 1) = -rx;
        }
    auto RE = [&](int i, int j, int k) { return reta[((size_t)i * nj + j) * 2 + k]; };
    auto RC = [&](int i, int j, int k) { return rchi[((size_t)i * njc + j) * 2 + k]; };
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < njc; j++) {
            size_t c = (size_t)i * njc + j;
            pc.vol[c] = 0.5 * (RE(i, j, 0) * RC(i, j, 1) - RC(i, j, 0) * RE(i, j, 1)
                               + RE(i, j + 1, 0) * RC(i + 1, j, 1) - RC(i + 1, j, 0) * RE(i, j + 1, 1));
            pc.xc[c] = 0.25 * (X(i, j) + X(i + 1, j) + X(i, j + 1) + X(i + 1, j + 1));
            pc.yc[c] = 0.25 * (Y(i, j) + Y(i + 1, j) + Y(i, j + 1) + Y(i + 1, j + 1));
            pc.ds_eta[c] = std::sqrt(std::pow(pc.NETA(i, j, 0), 2) + std::pow(pc.NETA(i, j, 1), 2));
            pc.ds_chi[c] = std::sqrt(std::pow(pc.NCHI(i, j, 0), 2) + std::pow(pc.NCHI(i, j, 1), 2));
        }
}

// Distance from each cell centre to the nearest no-slip wall segment
// (bottom-face wall/isothermalwall BCs), brute force over segments.
void compute_wall_distance(PCase& pc) {
    const int nic = pc.nic, njc = pc.njc, nj = pc.nj;
    std::vector<int> wall(nic, 0);
    for (const auto& b : pc.bcs) {
        if (b.face != ST_FACE_BOTTOM) continue;
        if (b.type != ST_BC_WALL && b.type != ST_BC_ISOTHERMALWALL) continue;
        int end = b.end >= 0 ? b.end : nic + 2 + b.end;
        for (int g = b.start; g <= end; g++)
            if (g >= 1 && g <= nic) wall[g - 1] = 1;
    }
    // a ghost-padded column later overwritten by a non-wall bottom BC is not a wall
    for (const auto& b : pc.bcs) {
        if (b.face != ST_FACE_BOTTOM) continue;
        int end = b.end >= 0 ? b.end : nic + 2 + b.end;
        bool is_wall = (b.type == ST_BC_WALL || b.type == ST_BC_ISOTHERMALWALL);
        for (int g = b.start; g <= end; g++)
            if (g >= 1 && g <= nic) wall[g - 1] = is_wall ? 1 : 0;
    }
    std::vector<double> sx0, sy0, sx1, sy1;
    for (int i = 0; i < nic; i++)
        if (wall[i]) {
            sx0.push_back(pc.xv[(size_t)i * nj]);
            sy0.push_back(pc.yv[(size_t)i * nj]);
            sx1.push_back(pc.xv[(size_t)(i + 1) * nj]);
            sy1.push_back(pc.yv[(size_t)(i + 1) * nj]);
        }
    pc.wd.assign((size_t)nic * njc, 1e30);
    const size_t ns = sx0.size();
#pragma omp parallel for schedule(static)
    for (long c = 0; c < (long)nic * njc; c++) {
        double px = pc.xc[c], py = pc.yc[c], best = 1e300;
        for (size_t s = 0; s < ns; s++) {
            double ax = sx1[s] - sx0[s], ay = sy1[s] - sy0[s];
            double wx = px - sx0[s], wy = py - sy0[s];
            double l2 = ax * ax + ay * ay;
            double t = l2 > 0.0 ? (wx * ax + wy * ay) / l2 : 0.0;
            t = std::min(1.0, std::max(0.0, t));
            double dx = wx - t * ax, dy = wy - t * ay;
            best = std::min(best, dx * dx + dy * dy);
        }
        pc.wd[c] = ns ? std::sqrt(best) : 1e30;
    }
}

template <class T>
struct Work {
    int nic, njc, ni, nj, np;  // np = (nic+2)*(njc+2)
    // ghost-padded primitives [nic+2][njc+2]
    std::vector<T> rho, u, v, p, T_, nut, mu, k, mud;
    // face states: chi [ni][njc], eta [nic][nj]
    std::vector<T> lchi[5], rchi[5], leta[5], reta[5];
    std::vector<T> fchi, feta;  // [..][nq]
    std::vector<T> gchi[4], geta[4];  // gradients of u, v, T, nut: [..][2]
    std::vector<T> ubc, vbc, Tbc, mubc, kbc, mudbc;  // chi face averages
    std::vector<T> ube, vbe, Tbe, mube, kbe, mudbe;  // eta face averages
    void init(const PCase& pc) {
        nic = pc.nic; njc = pc.njc; ni = pc.ni; nj = pc.nj;
        np = (nic + 2) * (njc + 2);
        for (auto* a : {&rho, &u, &v, &p, &T_, &nut, &mu, &k, &mud}) a->assign(np, T(0.0));
        for (int m = 0; m < 5; m++) {
            lchi[m].assign((size_t)ni * njc, T(0.0)); rchi[m].assign((size_t)ni * njc, T(0.0));
            leta[m].assign((size_t)nic * nj, T(0.0)); reta[m].assign((size_t)nic * nj, T(0.0));
        }
        fchi.assign((size_t)ni * njc * pc.nq, T(0.0));
        feta.assign((size_t)nic * nj * pc.nq, T(0.0));
        for (int m = 0; m < 4; m++) {
            gchi[m].assign((size_t)ni * njc * 2, T(0.0));
            geta[m].assign((size_t)nic * nj * 2, T(0.0));
        }
        for (auto* a : {&ubc, &vbc, &Tbc, &mubc, &kbc, &mudbc}) a->assign((size_t)ni * njc, T(0.0));
        for (auto* a : {&ube, &vbe, &Tbe, &mube, &kbe, &mudbe}) a->assign((size_t)nic * nj, T(0.0));
    }
    int P(int i, int j) const { return i * (njc + 2) + j; }
};

template <class T>
T laminar_mu(const PCase& pc, const T& temp) {
    if (pc.c.viscosity_law == ST_VISC_SUTHERLAND) {
        // Sutherland's law with S = 110.4 K at T_ref = 288.15 K, in units of T_inf.
        const double S = 110.4 / 288.15 * pc.c.T_inf;
        T tr = temp / pc.c.T_inf;
        return pc.c.mu_inf * tr * sqrt(tr) * ((pc.c.T_inf + S) / (temp + S));
    }
    // FluidModel::get_laminar_viscosity, src/model/fluid.cpp:38-40
    return pc.c.mu_inf * pow(temp / pc.c.T_inf, 2.0 / 3.0);
}

// Ghost cells from the boundary list, in list order (BoundaryContainer::apply,
// src/model/bc.cpp:430-433).  nut is SA's nu_tilde; its ghost rule per type is
// this project's addition (wall: antisymmetric about 0, slip wall:
// extrapolated like p and rho, freestream: nu_tilde_inf, others: copied).
// Ghost g takes cell s's primitives (periodic and wake copies).  With
// pc.freeze_nonlocal the copy carries the value only, so a JVP sees the
// residual's local dependencies alone.
template <class T>
void copy_ghost(const PCase& pc, Work<T>& w, int g, int s) {
    if (pc.freeze_nonlocal) {
        w.rho[g] = T(value(w.rho[s])); w.u[g] = T(value(w.u[s])); w.v[g] = T(value(w.v[s]));
        w.p[g] = T(value(w.p[s])); w.T_[g] = T(value(w.T_[s])); w.nut[g] = T(value(w.nut[s]));
    } else {
        w.rho[g] = w.rho[s]; w.u[g] = w.u[s]; w.v[g] = w.v[s]; w.p[g] = w.p[s]; w.T_[g] = w.T_[s]; w.nut[g] = w.nut[s];
    }
}

template <class T>
void apply_bcs(const PCase& pc, Work<T>& w) {
    const int nic = pc.nic, njc = pc.njc;
    const double R = pc.R;
    for (const auto& b : pc.bcs) {
        int bottom_top = (b.face == ST_FACE_BOTTOM || b.face == ST_FACE_TOP);
        int end = b.end;
        if (end < 0) end = (bottom_top ? nic : njc) + 2 + end;
        int start = b.start;
        switch (b.type) {
        case ST_BC_FREESTREAM: {  // bc.cpp:26-60
            for (int s = start; s <= end; s++) {
                int i, j;
                if (bottom_top) { i = s; j = (b.face == ST_FACE_BOTTOM) ? 0 : njc + 1; }
                else { j = s; i = (b.face == ST_FACE_LEFT) ? 0 : nic + 1; }
                int g = w.P(i, j);
                w.rho[g] = pc.c.rho_inf; w.u[g] = pc.c.u_inf; w.v[g] = pc.c.v_inf; w.p[g] = pc.c.p_inf;
                w.T_[g] = w.p[g] / w.rho[g] / R;
                w.nut[g] = pc.c.nu_tilde_inf;
            }
        } break;
        case ST_BC_SLIPWALL: {  // bc.cpp:78-128 (bottom/top only)
            if (!bottom_top) break;
            for (int i = start; i <= end; i++) {
                int j0, j1, j2; double nx, ny;
                if (b.face == ST_FACE_BOTTOM) { j0 = 0; j1 = 1; j2 = 2; nx = pc.NETA(i - 1, 0, 0); ny = pc.NETA(i - 1, 0, 1); }
                else { j0 = njc + 1; j1 = njc; j2 = njc - 1; nx = pc.NETA(i - 1, njc, 0); ny = pc.NETA(i - 1, njc, 1); }
                int g = w.P(i, j0), a = w.P(i, j1), c = w.P(i, j2);
                double ds = nx * nx + ny * ny;
                w.p[g] = 1.5 * w.p[a] - 0.5 * w.p[c];
                w.rho[g] = 1.5 * w.rho[a] - 0.5 * w.rho[c];
                T un = w.u[a] * nx + w.v[a] * ny;
                w.u[g] = w.u[a] - 2.0 * un * nx / ds;
                w.v[g] = w.v[a] - 2.0 * un * ny / ds;
                w.T_[g] = w.p[g] / w.rho[g] / R;
                w.nut[g] = 1.5 * w.nut[a] - 0.5 * w.nut[c];
            }
        } break;
        case ST_BC_WALL: {  // bc.cpp:150-204
            for (int s = start; s <= end; s++) {
                int g, a, c;
                if (bottom_top) {
                    int i = s;
                    if (b.face == ST_FACE_BOTTOM) { g = w.P(i, 0); a = w.P(i, 1); c = w.P(i, 2); }
                    else { g = w.P(i, njc + 1); a = w.P(i, njc); c = w.P(i, njc - 1); }
                } else {
                    int j = s;
                    if (b.face == ST_FACE_LEFT) { g = w.P(0, j); a = w.P(1, j); c = w.P(2, j); }
                    else { g = w.P(nic + 1, j); a = w.P(nic, j); c = w.P(nic - 1, j); }
                }
                w.T_[g] = 1.5 * w.T_[a] - 0.5 * w.T_[c];
                w.rho[g] = 1.5 * w.rho[a] - 0.5 * w.rho[c];
                w.u[g] = 2.0 * b.u - (1.5 * w.u[a] - 0.5 * w.u[c]);
                w.v[g] = 2.0 * b.v - (1.5 * w.v[a] - 0.5 * w.v[c]);
                w.p[g] = w.rho[g] * R * w.T_[g];
                w.nut[g] = -(1.5 * w.nut[a] - 0.5 * w.nut[c]);
            }
        } break;
        case ST_BC_ISOTHERMALWALL: {  // bc.cpp:388-427 (bottom/top only)
            if (!bottom_top) break;
            for (int i = start; i <= end; i++) {
                int g, a, c;
                if (b.face == ST_FACE_BOTTOM) { g = w.P(i, 0); a = w.P(i, 1); c = w.P(i, 2); }
                else { g = w.P(i, njc + 1); a = w.P(i, njc); c = w.P(i, njc - 1); }
                w.p[g] = 1.5 * w.p[a] - 0.5 * w.p[c];
                w.u[g] = 2.0 * b.u - (1.5 * w.u[a] - 0.5 * w.u[c]);
                w.v[g] = 2.0 * b.v - (1.5 * w.v[a] - 0.5 * w.v[c]);
                w.T_[g] = b.T;
                w.rho[g] = w.p[g] / w.T_[g] / R;
                w.nut[g] = -(1.5 * w.nut[a] - 0.5 * w.nut[c]);
            }
        } break;
        case ST_BC_OUTFLOW: {  // bc.cpp:284-311 (left/right only)
            if (bottom_top) break;
            int ie = (b.face == ST_FACE_LEFT) ? 0 : nic + 1;
            // the reference reads rho[iend-1]; for the left face that is
            // index -1, so only the right face is meaningful
            if (ie == 0) break;
            for (int j = start; j <= end; j++) {
                int g = w.P(ie, j), a = w.P(ie - 1, j);
                w.rho[g] = w.rho[a]; w.u[g] = w.u[a]; w.v[g] = w.v[a]; w.p[g] = pc.c.p_inf;
                w.T_[g] = w.p[g] / w.rho[g] / R;
                w.nut[g] = w.nut[a];
            }
        } break;
        case ST_BC_PERIODIC: {  // bc.cpp:329-365
            if (bottom_top) {
                for (int i = start; i <= end; i++) {
                    copy_ghost(pc, w, w.P(i, 0), w.P(i, njc));
                    copy_ghost(pc, w, w.P(i, njc + 1), w.P(i, 1));
                }
            } else {
                for (int j = start; j <= end; j++) {
                    copy_ghost(pc, w, w.P(0, j), w.P(nic, j));
                    copy_ghost(pc, w, w.P(nic + 1, j), w.P(1, j));
                }
            }
        } break;
        case ST_BC_WAKE: {  // bc.cpp:224-263 (bottom/top only)
            if (!bottom_top) break;
            int je = (b.face == ST_FACE_BOTTOM) ? 0 : njc + 1;
            for (int i = start; i <= end; i++) copy_ghost(pc, w, w.P(i, je), w.P(nic + 1 - i, 1));
            for (int i = start; i <= end; i++) copy_ghost(pc, w, w.P(nic + 1 - i, je), w.P(i, 1));
        } break;
        default: break;
        }
    }
}

// ReconstructionSecondOrder::evaluate_chi / evaluate_eta,
// src/model/reconstruction.cpp:78-154 (first order: :16-48)
template <class T>
void reconstruct(const PCase& pc, const Work<T>& w, const std::vector<T>& q,
                 std::vector<T>& lchi, std::vector<T>& rchi, std::vector<T>& leta, std::vector<T>& reta,
                 int order) {
    const int ni = pc.ni, nj = pc.nj, nic = pc.nic, njc = pc.njc;
    const double thm = 2.0 / 3.0, thp = 4.0 / 3.0;
    auto Q = [&](int i, int j) -> const T& { return q[(size_t)i * (njc + 2) + j]; };
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ni; i++)
        for (int j = 0; j < njc; j++) {
            lchi[(size_t)i * njc + j] = Q(i, j + 1);
            rchi[(size_t)i * njc + j] = Q(i + 1, j + 1);
        }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < nj; j++) {
            leta[(size_t)i * nj + j] = Q(i + 1, j);
            reta[(size_t)i * nj + j] = Q(i + 1, j + 1);
        }
    if (order != 2) return;
    {
        const double eps = pc.eps_chi;
        std::vector<T> f2((size_t)ni * njc);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < ni; i++)
            for (int j = 0; j < njc; j++) f2[(size_t)i * njc + j] = Q(i + 1, j + 1) - Q(i, j + 1);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nic; i++)
            for (int j = 0; j < njc; j++) {
                const T& fa = f2[(size_t)i * njc + j];
                const T& fb = f2[(size_t)(i + 1) * njc + j];
                T a1 = 3.0 * fb * fa;
                T a2 = 2.0 * (fb - fa) * (fb - fa) + a1;
                T f3qt = 0.25 * (a1 + eps) / (a2 + eps);
                lchi[(size_t)(i + 1) * njc + j] = lchi[(size_t)(i + 1) * njc + j] + f3qt * (thm * fa + thp * fb);
                rchi[(size_t)i * njc + j] = rchi[(size_t)i * njc + j] - f3qt * (thp * fa + thm * fb);
            }
    }
    {
        const double eps = pc.eps_eta;
        std::vector<T> f2((size_t)nic * nj);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nic; i++)
            for (int j = 0; j < nj; j++) f2[(size_t)i * nj + j] = Q(i + 1, j + 1) - Q(i + 1, j);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nic; i++)
            for (int j = 0; j < njc; j++) {
                const T& fa = f2[(size_t)i * nj + j];
                const T& fb = f2[(size_t)i * nj + j + 1];
                T a1 = 3.0 * fb * fa;
                T a2 = 2.0 * (fb - fa) * (fb - fa) + a1;
                T f3qt = 0.25 * (a1 + eps) / (a2 + eps);
                leta[(size_t)i * nj + j + 1] = leta[(size_t)i * nj + j + 1] + f3qt * (thm * fa + thp * fb);
                reta[(size_t)i * nj + j] = reta[(size_t)i * nj + j] - f3qt * (thp * fa + thm * fb);
            }
    }
}

// Mesh::calc_face, src/utils/mesh.cpp:10-32
template <class T>
void calc_face(const PCase& pc, const std::vector<T>& q, std::vector<T>& qc, std::vector<T>& qe) {
    const int ni = pc.ni, nj = pc.nj, nic = pc.nic, njc = pc.njc;
    auto Q = [&](int i, int j) -> const T& { return q[(size_t)i * (njc + 2) + j]; };
    for (int i = 0; i < ni; i++)
        for (int j = 0; j < njc; j++) {
            const int b = 1;
            T ql = Q(i + b - 1, j + b), qr = Q(i + b, j + b);
            T qt = 0.25 * (ql + qr + Q(i + b - 1, j + b + 1) + Q(i + b, j + b + 1));
            T qb = 0.25 * (ql + qr + Q(i + b - 1, j + b - 1) + Q(i + b, j + b - 1));
            qc[(size_t)i * njc + j] = 0.25 * (ql + qr + qt + qb);
        }
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < nj; j++) {
            const int b = 1;
            T qt = Q(i + b, j + b), qb = Q(i + b, j + b - 1);
            T ql = 0.25 * (qt + qb + Q(i + b - 1, j + b) + Q(i + b - 1, j + b - 1));
            T qr = 0.25 * (qt + qb + Q(i + b + 1, j + b) + Q(i + b + 1, j + b - 1));
            qe[(size_t)i * nj + j] = 0.25 * (ql + qr + qt + qb);
        }
}

// Mesh::calc_gradient (face Green-Gauss), src/utils/mesh.cpp:36-131
template <class T>
void calc_gradient(const PCase& pc, const std::vector<T>& q, std::vector<T>& gc, std::vector<T>& ge) {
    const int ni = pc.ni, nj = pc.nj, nic = pc.nic, njc = pc.njc;
    auto Q = [&](int i, int j) -> const T& { return q[(size_t)i * (njc + 2) + j]; };
    double nt[2], nb[2], nl[2], nr[2], vol;
    for (int i = 0; i < ni; i++)
        for (int j = 0; j < njc; j++) {
            const int b = 1;
            T ql = Q(i + b - 1, j + b), qr = Q(i + b, j + b);
            T qt = 0.25 * (ql + qr + Q(i + b - 1, j + b + 1) + Q(i + b, j + b + 1));
            T qb = 0.25 * (ql + qr + Q(i + b - 1, j + b - 1) + Q(i + b, j + b - 1));
            if (i == 0) {
                vol = pc.VOL(i, j);
                for (int k = 0; k < 2; k++) {
                    nt[k] = pc.NETA(i, j + 1, k); nb[k] = pc.NETA(i, j, k);
                    nr[k] = 0.5 * (pc.NCHI(i, j, k) + pc.NCHI(i + 1, j, k)); nl[k] = pc.NCHI(i, j, k);
                }
            } else if (i == ni - 1) {
                vol = pc.VOL(i - 1, j);
                for (int k = 0; k < 2; k++) {
                    nt[k] = pc.NETA(i - 1, j + 1, k); nb[k] = pc.NETA(i - 1, j, k);
                    nr[k] = pc.NCHI(i, j, k); nl[k] = 0.5 * (pc.NCHI(i, j, k) + pc.NCHI(i - 1, j, k));
                }
            } else {
                vol = 0.5 * (pc.VOL(i, j) + pc.VOL(i - 1, j));
                for (int k = 0; k < 2; k++) {
                    nt[k] = 0.5 * (pc.NETA(i, j + 1, k) + pc.NETA(i - 1, j + 1, k));
                    nb[k] = 0.5 * (pc.NETA(i, j, k) + pc.NETA(i - 1, j, k));
                    nr[k] = 0.5 * (pc.NCHI(i, j, k) + pc.NCHI(i + 1, j, k));
                    nl[k] = 0.5 * (pc.NCHI(i, j, k) + pc.NCHI(i - 1, j, k));
                }
            }
            for (int k = 0; k < 2; k++)
                gc[((size_t)i * njc + j) * 2 + k] = (nt[k] * qt - nb[k] * qb + nr[k] * qr - nl[k] * ql) / vol;
        }
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < nj; j++) {
            const int b = 1;
            T qt = Q(i + b, j + b), qb = Q(i + b, j + b - 1);
            T ql = 0.25 * (qt + qb + Q(i + b - 1, j + b) + Q(i + b - 1, j + b - 1));
            T qr = 0.25 * (qt + qb + Q(i + b + 1, j + b) + Q(i + b + 1, j + b - 1));
            if (j == 0) {
                vol = pc.VOL(i, j);
                for (int k = 0; k < 2; k++) {
                    nt[k] = 0.5 * (pc.NETA(i, j, k) + pc.NETA(i, j + 1, k)); nb[k] = pc.NETA(i, j, k);
                    nl[k] = pc.NCHI(i, j, k); nr[k] = pc.NCHI(i + 1, j, k);
                }
            } else if (j == nj - 1) {
                for (int k = 0; k < 2; k++) {
                    nt[k] = pc.NETA(i, j, k); nb[k] = 0.5 * (pc.NETA(i, j, k) + pc.NETA(i, j - 1, k));
                    nl[k] = pc.NCHI(i, j - 1, k); nr[k] = pc.NCHI(i + 1, j - 1, k);
                }
                vol = pc.VOL(i, j - 1);
            } else {
                for (int k = 0; k < 2; k++) {
                    nt[k] = 0.5 * (pc.NETA(i, j, k) + pc.NETA(i, j + 1, k));
                    nb[k] = 0.5 * (pc.NETA(i, j, k) + pc.NETA(i, j - 1, k));
                    nl[k] = 0.5 * (pc.NCHI(i, j, k) + pc.NCHI(i, j - 1, k));
                    nr[k] = 0.5 * (pc.NCHI(i + 1, j, k) + pc.NCHI(i + 1, j - 1, k));
                }
                vol = 0.5 * (pc.VOL(i, j) + pc.VOL(i, j - 1));
            }
            for (int k = 0; k < 2; k++)
                ge[((size_t)i * nj + j) * 2 + k] = (nt[k] * qt - nb[k] * qb + nr[k] * qr - nl[k] * ql) / vol;
        }
}

// ConvectiveFluxRoe::evaluate, src/model/flux.cpp:51-146; with SA the
// nu_tilde flux is the Roe mass flux times the upwind reconstructed nu_tilde.
template <class T>
void roe_flux(const PCase& pc, const double* normal, int nfaces,
              const std::vector<T>* L, const std::vector<T>* Rr, std::vector<T>& f) {
    constexpr double gm1 = GAMMA - 1.0;
    constexpr double ogm1 = 1.0 / gm1;
    const int nq = pc.nq;
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < nfaces; idx++) {
        const double nx = normal[idx * 2 + 0], ny = normal[idx * 2 + 1];
        const T rlft = L[0][idx], ulft = L[1][idx], vlft = L[2][idx], plft = L[3][idx];
        const T rrht = Rr[0][idx], urht = Rr[1][idx], vrht = Rr[2][idx], prht = Rr[3][idx];
        const T rlfti = 1.0 / rlft;
        const T rulft = rlft * ulft;
        const T rvlft = rlft * vlft;
        const T uvl = 0.5 * (ulft * ulft + vlft * vlft);
        const T elft = plft * ogm1 + rlft * uvl;
        const T hlft = (elft + plft) * rlfti;
        const T rrhti = 1.0 / rrht;
        const T rurht = rrht * urht;
        const T rvrht = rrht * vrht;
        const T uvr = 0.5 * (urht * urht + vrht * vrht);
        const T erht = prht * ogm1 + rrht * uvr;
        const T hrht = (erht + prht) * rrhti;
        const T rat = sqrt(rrht * rlfti);
        const T rati = 1.0 / (rat + 1.0);
        const T rav = rat * rlft;
        const T uav = (rat * urht + ulft) * rati;
        const T vav = (rat * vrht + vlft) * rati;
        const T hav = (rat * hrht + hlft) * rati;
        const T uv = 0.5 * (uav * uav + vav * vav);
        const T cav = sqrt(gm1 * (hav - uv));
        T aq1 = rrht - rlft, aq2 = urht - ulft, aq3 = vrht - vlft, aq4 = prht - plft;
        const double dr = std::sqrt(nx * nx + ny * ny);
        const double r1 = nx / dr, r2 = ny / dr;
        const T uu = r1 * uav + r2 * vav;
        const T c2 = cav * cav;
        const T c2i = 1.0 / c2;
        const T auu = fabs(uu);
        const T aupc = fabs(uu + cav);
        const T aumc = fabs(uu - cav);
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
        aq1 = b4;
        aq2 = uav * b4 + r1 * b5 + b6;
        aq3 = vav * b4 + r2 * b5 + b7;
        aq4 = hav * b4 + uu * b5 + uav * b6 + vav * b7 - c2 * b1 * ogm1;
        const double aj = 0.5 * dr;
        const T plar = plft + prht;
        const T eplft = elft + plft;
        const T eprht = erht + prht;
        T* o = &f[(size_t)idx * nq];
        o[0] = aj * (rlft * uulft + rrht * uurht - aq1);
        o[1] = aj * (rulft * uulft + rurht * uurht + r1 * plar - aq2);
        o[2] = aj * (rvlft * uulft + rvrht * uurht + r2 * plar - aq3);
        o[3] = aj * (eplft * uulft + eprht * uurht - aq4);
        if (nq == 5) o[4] = o[0] * (o[0] >= 0.0 ? L[4][idx] : Rr[4][idx]);
    }
}

// ConvectiveFluxAUSM::evaluate, src/model/flux.cpp:148-224, in its operation
// order (split Mach numbers / pressures of flux.cpp:148-155).
template <class T> T ausm_mach_p(const T& M) { return fabs(M) <= 1.0 ? 0.25 * (M + 1.0) * (M + 1.0) : 0.5 * (M + fabs(M)); }
template <class T> T ausm_mach_m(const T& M) { return fabs(M) <= 1.0 ? -0.25 * (M - 1.0) * (M - 1.0) : 0.5 * (M - fabs(M)); }
template <class T> T ausm_pres_p(const T& M, const T& p) {
    return fabs(M) <= 1.0 ? 0.25 * p * (M + 1.0) * (M + 1.0) * (2.0 - M) : 0.5 * p * (M + fabs(M)) / M;
}
template <class T> T ausm_pres_m(const T& M, const T& p) {
    return fabs(M) <= 1.0 ? 0.25 * p * (M - 1.0) * (M - 1.0) * (2.0 + M) : 0.5 * p * (M - fabs(M)) / M;
}

template <class T>
void ausm_flux(const PCase& pc, const double* normal, int nfaces,
               const std::vector<T>* L, const std::vector<T>* Rr, std::vector<T>& f) {
    constexpr double gm1 = GAMMA - 1.0;
    constexpr double ogm1 = 1.0 / gm1;
    const int nq = pc.nq;
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < nfaces; idx++) {
        const double nx = normal[idx * 2 + 0], ny = normal[idx * 2 + 1];
        const T rlft = L[0][idx], ulft = L[1][idx], vlft = L[2][idx], plft = L[3][idx];
        const T rrht = Rr[0][idx], urht = Rr[1][idx], vrht = Rr[2][idx], prht = Rr[3][idx];
        const double ds = std::sqrt(nx * nx + ny * ny);
        const T ulft_normal = (ulft * nx + vlft * ny) / ds;
        const T urht_normal = (urht * nx + vrht * ny) / ds;
        const T alft = sqrt(GAMMA * plft / rlft);
        const T arht = sqrt(GAMMA * prht / rrht);
        const T machlft = ulft_normal / alft;
        const T machrht = urht_normal / arht;
        const T rlfti = 1.0 / rlft;
        const T uvl = 0.5 * (ulft * ulft + vlft * vlft);
        const T elft = plft * ogm1 + rlft * uvl;
        const T hlft = (elft + plft) * rlfti;
        const T rrhti = 1.0 / rrht;
        const T uvr = 0.5 * (urht * urht + vrht * vrht);
        const T erht = prht * ogm1 + rrht * uvr;
        const T hrht = (erht + prht) * rrhti;
        const T mach_half = ausm_mach_p(machlft) + ausm_mach_m(machrht);
        const T p_half = ausm_pres_p(machlft, plft) + ausm_pres_m(machrht, prht);
        T* o = &f[(size_t)idx * nq];
        if (mach_half >= 0.0) {
            o[0] = rlft * alft * mach_half * ds;
            o[1] = rlft * alft * ulft * mach_half * ds + p_half * nx;
            o[2] = rlft * alft * vlft * mach_half * ds + p_half * ny;
            o[3] = rlft * alft * hlft * mach_half * ds;
        } else {
            o[0] = rrht * arht * mach_half * ds;
            o[1] = rrht * arht * urht * mach_half * ds + p_half * nx;
            o[2] = rrht * arht * vrht * mach_half * ds + p_half * ny;
            o[3] = rrht * arht * hrht * mach_half * ds;
        }
        if (nq == 5) o[4] = o[0] * (o[0] >= 0.0 ? L[4][idx] : Rr[4][idx]);
    }
}

// DiffusiveFluxGreenGauss::evaluate, src/model/flux.cpp:12-48 (+ SA diffusion
// (1/sigma)(mu + rho nu_tilde) grad(nu_tilde) . n in slot 4).
template <class T>
void viscous_flux(const PCase& pc, const double* normal, int nfaces, const std::vector<T>* g,
                  const std::vector<T>& ub, const std::vector<T>& vb, const std::vector<T>& mub,
                  const std::vector<T>& kb, const std::vector<T>& mudb, std::vector<T>& f) {
    const int nq = pc.nq;
    for (int idx = 0; idx < nfaces; idx++) {
        const double nx = normal[idx * 2 + 0], ny = normal[idx * 2 + 1];
        const T dudx = g[0][idx * 2], dudy = g[0][idx * 2 + 1];
        const T dvdx = g[1][idx * 2], dvdy = g[1][idx * 2 + 1];
        const T dTdx = g[2][idx * 2], dTdy = g[2][idx * 2 + 1];
        const T ubar = ub[idx], vbar = vb[idx], mu = mub[idx], k = kb[idx];
        const T tau_xy = mu * (dudy + dvdx);
        const T tau_xx = mu * (2.0 * dudx - 2.0 / 3.0 * (dudx + dvdy));
        const T tau_yy = mu * (2.0 * dvdy - 2.0 / 3.0 * (dudx + dvdy));
        const T q_x = -k * dTdx;
        const T q_y = -k * dTdy;
        T* o = &f[(size_t)idx * nq];
        o[0] = 0.0;
        o[1] = tau_xx * nx + tau_xy * ny;
        o[2] = tau_xy * nx + tau_yy * ny;
        o[3] = (ubar * tau_xx + vbar * tau_xy - q_x) * nx + (ubar * tau_xy + vbar * tau_yy - q_y) * ny;
        if (nq == 5) o[4] = (1.0 / SA_SIGMA) * mudb[idx] * (g[3][idx * 2] * nx + g[3][idx * 2 + 1] * ny);
    }
}

// SA source for one cell (per unit volume): rho*(beta*P - D) + cb2/sigma*rho*|grad nut|^2.
template <class T>
T sa_source(const T& rho, const T& nut, const T& mu, double d, const T& omega, const T& gnut2, const T& beta) {
    if (nut < 0.0)  // SA-neg: P = cb1 (1 - ct3) Omega nut, D = -cw1 (nut / d)^2
        return rho * (beta * SA_CB1 * (1.0 - SA_CT3) * omega * nut + SA_CW1 * (nut * nut) / (d * d))
             + (SA_CB2 / SA_SIGMA) * rho * gnut2;
    const double k2d2 = SA_KAPPA * SA_KAPPA * d * d;
    const T nu = mu / rho;
    const T chi = nut / nu;
    const T chi3 = chi * chi * chi;
    const T fv1 = chi3 / (chi3 + SA_CV1 * SA_CV1 * SA_CV1);
    const T fv2 = 1.0 - chi / (1.0 + chi * fv1);
    const T sbar = nut * fv2 / k2d2;
    T stilde;
    if (sbar >= -SA_CV2 * omega) stilde = omega + sbar;
    else stilde = omega + omega * (SA_CV2 * SA_CV2 * omega + SA_CV3 * sbar) / ((SA_CV3 - 2.0 * SA_CV2) * omega - sbar);
    T r;
    if (stilde > 0.0) {
        r = nut / (stilde * k2d2);
        if (r > 10.0) r = T(10.0);
    } else {
        r = T(10.0);
    }
    const T r5 = r * r * r * r * r;
    const T gg = r + SA_CW2 * (r5 * r - r);
    const T g6 = gg * gg * gg * gg * gg * gg;
    const double cw36 = std::pow(SA_CW3, 6);
    const T fw = gg * pow((1.0 + cw36) / (g6 + cw36), 1.0 / 6.0);
    const T prod = beta * SA_CB1 * stilde * nut;
    const T dest = SA_CW1 * fw * (nut * nut) / (d * d);
    return rho * (prod - dest) + (SA_CB2 / SA_SIGMA) * rho * gnut2;
}

inline void add_abs(double* scale, size_t i, const double& x) { if (scale) scale[i] += std::fabs(x); }
inline void add_abs(double*, size_t, const Dual&) {}

// scale (double evaluation only, may be null): per cell and component, the sum
// of |face flux| over the cell's four faces (convective and viscous parts
// separately) divided by the volume -- the magnitude the residual is a small
// difference of, used to state per-cell relative parity errors.
template <class T>
void residual(const PCase& pc, const T* q, const T* beta, T* rhs, int order, Work<T>& w,
              T* cf_wall = nullptr, double* scale = nullptr) {
    const int nic = pc.nic, njc = pc.njc, ni = pc.ni, nj = pc.nj, nq = pc.nq;
    const double R = pc.R;
    // primvars, src/model/fluid.cpp:50-67 (shift 1,1 into the ghost-padded arrays).
    // OpenMP pragmas sit on the loops the reference parallelises
    // (fluid.cpp:53, reconstruction.cpp:30-107, flux.cpp:60, eulerequation.cpp:145,227)
    // and on this project's cell-local SA loops.
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < njc; j++) {
            const T* Q = &q[((size_t)i * njc + j) * nq];
            int g = w.P(i + 1, j + 1);
            T r = Q[0];
            T uu = Q[1] / r;
            T vv = Q[2] / r;
            w.rho[g] = r; w.u[g] = uu; w.v[g] = vv;
            w.p[g] = (Q[3] - 0.5 * r * (uu * uu + vv * vv)) * (GAMMA - 1.0);
            w.T_[g] = w.p[g] / w.rho[g] / R;
            if (nq == 5) w.nut[g] = Q[4] / r;
        }
    apply_bcs(pc, w);
    reconstruct(pc, w, w.rho, w.lchi[0], w.rchi[0], w.leta[0], w.reta[0], order);
    reconstruct(pc, w, w.u, w.lchi[1], w.rchi[1], w.leta[1], w.reta[1], order);
    reconstruct(pc, w, w.v, w.lchi[2], w.rchi[2], w.leta[2], w.reta[2], order);
    reconstruct(pc, w, w.p, w.lchi[3], w.rchi[3], w.leta[3], w.reta[3], order);
    if (nq == 5) reconstruct(pc, w, w.nut, w.lchi[4], w.rchi[4], w.leta[4], w.reta[4], order);

    for (size_t n = 0; n < (size_t)nic * njc * nq; n++) rhs[n] = 0.0;
    if (scale) for (size_t n = 0; n < (size_t)nic * njc * nq; n++) scale[n] = 0.0;
    if (pc.c.flux == ST_FLUX_AUSM) {  // EulerEquation's flux choice, eulerequation.cpp:121-128
        ausm_flux(pc, pc.nchi.data(), ni * njc, w.lchi, w.rchi, w.fchi);
        ausm_flux(pc, pc.neta.data(), nic * nj, w.leta, w.reta, w.feta);
    } else {
        roe_flux(pc, pc.nchi.data(), ni * njc, w.lchi, w.rchi, w.fchi);
        roe_flux(pc, pc.neta.data(), nic * nj, w.leta, w.reta, w.feta);
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < njc; j++)
            for (int k = 0; k < nq; k++) {
                T& r = rhs[((size_t)i * njc + j) * nq + k];
                r -= (w.feta[((size_t)i * nj + j + 1) * nq + k] - w.feta[((size_t)i * nj + j) * nq + k]);
                r -= (w.fchi[((size_t)(i + 1) * njc + j) * nq + k] - w.fchi[((size_t)i * njc + j) * nq + k]);
            }
    auto accumulate_scale = [&]() {
        for (int i = 0; i < nic; i++)
            for (int j = 0; j < njc; j++)
                for (int k = 0; k < nq; k++) {
                    size_t r = ((size_t)i * njc + j) * nq + k;
                    add_abs(scale, r, w.feta[((size_t)i * nj + j + 1) * nq + k]);
                    add_abs(scale, r, w.feta[((size_t)i * nj + j) * nq + k]);
                    add_abs(scale, r, w.fchi[((size_t)(i + 1) * njc + j) * nq + k]);
                    add_abs(scale, r, w.fchi[((size_t)i * njc + j) * nq + k]);
                }
    };
    if (scale) accumulate_scale();
    if (pc.viscous) {
        for (int g = 0; g < w.np; g++) {
            T mu = laminar_mu(pc, w.T_[g]);
            if (nq == 5) {
                T nu = mu / w.rho[g];
                T chi = w.nut[g] / nu;
                T chi3 = chi * chi * chi;
                T fv1 = chi3 / (chi3 + SA_CV1 * SA_CV1 * SA_CV1);
                // SA-neg below nu_tilde = 0: mu_t = 0, diffusion rho nu_tilde f_n(chi)
                const bool neg = w.nut[g] < 0.0;
                T mut = neg ? T(0.0) : w.rho[g] * w.nut[g] * fv1;
                T fn = neg ? (SA_CN1 + chi3) / (SA_CN1 - chi3) : T(1.0);
                w.mu[g] = mu + mut;
                w.k[g] = pc.cp * (mu / pc.c.pr_inf + mut / PR_TURB);
                w.mud[g] = mu + w.rho[g] * w.nut[g] * fn;
            } else {
                w.mu[g] = mu;
                w.k[g] = mu * pc.cp / pc.c.pr_inf;  // get_thermal_conductivity, fluid.cpp:44-46
            }
        }
        calc_gradient(pc, w.u, w.gchi[0], w.geta[0]);
        calc_gradient(pc, w.v, w.gchi[1], w.geta[1]);
        calc_gradient(pc, w.T_, w.gchi[2], w.geta[2]);
        if (nq == 5) calc_gradient(pc, w.nut, w.gchi[3], w.geta[3]);
        calc_face(pc, w.u, w.ubc, w.ube);
        calc_face(pc, w.v, w.vbc, w.vbe);
        calc_face(pc, w.T_, w.Tbc, w.Tbe);
        calc_face(pc, w.mu, w.mubc, w.mube);
        calc_face(pc, w.k, w.kbc, w.kbe);
        if (nq == 5) calc_face(pc, w.mud, w.mudbc, w.mudbe);
        viscous_flux(pc, pc.nchi.data(), ni * njc, w.gchi, w.ubc, w.vbc, w.mubc, w.kbc, w.mudbc, w.fchi);
        viscous_flux(pc, pc.neta.data(), nic * nj, w.geta, w.ube, w.vbe, w.mube, w.kbe, w.mudbe, w.feta);
        if (scale) accumulate_scale();
        for (int i = 0; i < nic; i++)
            for (int j = 0; j < njc; j++)
                for (int k = 1; k < nq; k++) {
                    T& r = rhs[((size_t)i * njc + j) * nq + k];
                    r += (w.feta[((size_t)i * nj + j + 1) * nq + k] - w.feta[((size_t)i * nj + j) * nq + k]);
                    r += (w.fchi[((size_t)(i + 1) * njc + j) * nq + k] - w.fchi[((size_t)i * njc + j) * nq + k]);
                }
        if (nq == 5) {
#pragma omp parallel for schedule(static)
            for (int i = 0; i < nic; i++)
                for (int j = 0; j < njc; j++) {
                    auto cg = [&](int m, int k) {
                        return 0.25 * (w.gchi[m][((size_t)i * njc + j) * 2 + k] + w.gchi[m][((size_t)(i + 1) * njc + j) * 2 + k]
                                       + w.geta[m][((size_t)i * nj + j) * 2 + k] + w.geta[m][((size_t)i * nj + j + 1) * 2 + k]);
                    };
                    T omega = fabs(cg(1, 0) - cg(0, 1));
                    T gx = cg(3, 0), gy = cg(3, 1);
                    T gn2 = gx * gx + gy * gy;
                    int g = w.P(i + 1, j + 1);
                    T mu = laminar_mu(pc, w.T_[g]);
                    T b = beta ? beta[(size_t)i * njc + j] : T(1.0);
                    T s = sa_source(w.rho[g], w.nut[g], mu, pc.wd[(size_t)i * njc + j], omega, gn2, b);
                    rhs[((size_t)i * njc + j) * nq + 4] += s * pc.VOL(i, j);
                }
        }
    }
    // calc_source_residual, eulerequation.cpp:22-29
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < njc; j++) {
            rhs[((size_t)i * njc + j) * nq + 1] += -pc.c.dpdx * pc.VOL(i, j);
            rhs[((size_t)i * njc + j) * nq + 2] += -pc.c.dpdy * pc.VOL(i, j);
        }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nic; i++)
        for (int j = 0; j < njc; j++)
            for (int k = 0; k < nq; k++) rhs[((size_t)i * njc + j) * nq + k] /= pc.VOL(i, j);
    if (scale)
        for (int i = 0; i < nic; i++)
            for (int j = 0; j < njc; j++)
                for (int k = 0; k < nq; k++) scale[((size_t)i * njc + j) * nq + k] /= pc.VOL(i, j);

    if (cf_wall) {
        // IOManager::write_surface, src/utils/io.cpp:217-226: the j=0 face
        // gradients of u and v with mu_inf.
        const double qinf = 0.5 * pc.c.rho_inf * (pc.c.u_inf * pc.c.u_inf + pc.c.v_inf * pc.c.v_inf);
        if (!pc.viscous) {
            calc_gradient(pc, w.u, w.gchi[0], w.geta[0]);
            calc_gradient(pc, w.v, w.gchi[1], w.geta[1]);
        }
        for (int i = 0; i < nic; i++)
            cf_wall[i] = pc.c.mu_inf * (w.geta[0][((size_t)i * nj + 0) * 2 + 1] - w.geta[1][((size_t)i * nj + 0) * 2 + 0]) / qinf;
    }
}

struct Handle {
    PCase pc;
    Work<double> wd;
    Work<Dual> wjvp;                 // reused by port_jvp
    std::vector<Dual> qd, bd, rd;
    bool jvp_ready = false;
};

}  // namespace

extern "C" {

void* port_create(const st_case* c, const double* xv, const double* yv) {
    auto* h = new Handle();
    PCase& pc = h->pc;
    pc.c = *c;
    pc.bcs.assign(c->bcs, c->bcs + c->nbc);
    pc.c.bcs = nullptr;
    pc.ni = c->ni; pc.nj = c->nj; pc.nic = c->ni - 1; pc.njc = c->nj - 1;
    pc.sa = (c->turbulence == ST_TURB_SA);
    pc.nq = pc.sa ? 5 : 4;
    pc.viscous = c->mu_inf > 1e-15;  // config.cpp:41
    pc.R = c->p_inf / c->rho_inf / c->T_inf;  // fluid.cpp:12
    pc.cp = GAMMA * pc.R / (GAMMA - 1.0);
    pc.eps_chi = std::pow(10.0 / pc.nic, 3);  // reconstruction.cpp:59-60
    pc.eps_eta = std::pow(10.0 / pc.njc, 3);
    pc.xv.assign(xv, xv + (size_t)c->ni * c->nj);
    pc.yv.assign(yv, yv + (size_t)c->ni * c->nj);
    compute_metrics(pc);
    compute_wall_distance(pc);
    h->wd.init(pc);
    return h;
}

void port_destroy(void* h) { delete static_cast<Handle*>(h); }

// JVPs with the periodic and wake ghosts' tangents held at zero (the local
// part of the Jacobian, as the implicit solver's colouring pass assembles it)
int port_set_freeze_nonlocal(void* hp, int on) {
    static_cast<Handle*>(hp)->pc.freeze_nonlocal = on != 0;
    return 0;
}

int port_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

int port_metrics(void* hp, double* nchi, double* neta, double* vol, double* wd) {
    auto* h = static_cast<Handle*>(hp);
    if (nchi) std::memcpy(nchi, h->pc.nchi.data(), h->pc.nchi.size() * 8);
    if (neta) std::memcpy(neta, h->pc.neta.data(), h->pc.neta.size() * 8);
    if (vol) std::memcpy(vol, h->pc.vol.data(), h->pc.vol.size() * 8);
    if (wd) std::memcpy(wd, h->pc.wd.data(), h->pc.wd.size() * 8);
    return 0;
}

int port_residual(void* hp, const double* q, const double* beta, double* rhs, int order) {
    auto* h = static_cast<Handle*>(hp);
    residual<double>(h->pc, q, beta, rhs, order, h->wd);
    return 0;
}

int port_flux_scale(void* hp, const double* q, const double* beta, double* scale, int order) {
    auto* h = static_cast<Handle*>(hp);
    std::vector<double> rhs((size_t)h->pc.nic * h->pc.njc * h->pc.nq);
    residual<double>(h->pc, q, beta, rhs.data(), order, h->wd, nullptr, scale);
    return 0;
}

// Cf at the nic bottom faces and J = sum Cf dx over plate faces.
int port_skin_friction(void* hp, const double* q, double* cf, double* J) {
    auto* h = static_cast<Handle*>(hp);
    const PCase& pc = h->pc;
    std::vector<double> rhs((size_t)pc.nic * pc.njc * pc.nq);
    residual<double>(pc, q, nullptr, rhs.data(), pc.c.order, h->wd, cf);
    double s = 0.0;
    for (int i = std::max(pc.c.plate_vertex, 0); i < pc.nic; i++) {
        double x0 = pc.xv[(size_t)i * pc.nj], x1 = pc.xv[(size_t)(i + 1) * pc.nj];
        if (0.5 * (x0 + x1) <= pc.c.plate_x_end) s += cf[i] * (x1 - x0);
    }
    *J = s;
    return 0;
}

// calc_dt, src/model/eulerequation.cpp:237-259 (all nq slots set)
int port_dt(void* hp, const double* q, double cfl, double* dt) {
    auto* h = static_cast<Handle*>(hp);
    const PCase& pc = h->pc;
    const int nq = pc.nq;
    for (int i = 0; i < pc.nic; i++)
        for (int j = 0; j < pc.njc; j++) {
            const double* Q = &q[((size_t)i * pc.njc + j) * nq];
            double rho = Q[0], u = Q[1] / rho, v = Q[2] / rho, rhoE = Q[3];
            double p = (rhoE - 0.5 * rho * (u * u + v * v)) * (GAMMA - 1.0);
            double lambda = std::sqrt(GAMMA * p / rho) + std::fabs(u) + std::fabs(v);
            size_t c = (size_t)i * pc.njc + j;
            double len_min = std::min(pc.ds_eta[c], pc.ds_chi[c]);
            double mu = pc.c.mu_inf;
            for (int k = 0; k < nq; k++) dt[c * nq + k] = cfl / (lambda / len_min + 2.0 * mu / len_min / len_min);
        }
    return 0;
}

// Exact JVP: jv = dR/dQ . v + dR/dbeta . vb (vb may be NULL).
int port_jvp(void* hp, const double* q, const double* beta, const double* v, const double* vb,
             double* jv, int order) {
    auto* h = static_cast<Handle*>(hp);
    const PCase& pc = h->pc;
    const size_t n = (size_t)pc.nic * pc.njc * pc.nq, nc = (size_t)pc.nic * pc.njc;
    if (!h->jvp_ready) {
        h->qd.resize(n); h->bd.resize(nc); h->rd.resize(n);
        h->wjvp.init(pc);
        h->jvp_ready = true;
    }
    std::vector<Dual>& qd = h->qd;
    std::vector<Dual>& bd = h->bd;
    std::vector<Dual>& rd = h->rd;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; i++) qd[i] = Dual(q[i], v[i]);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)nc; i++) bd[i] = Dual(beta ? beta[i] : 1.0, vb ? vb[i] : 0.0);
    residual<Dual>(pc, qd.data(), bd.data(), rd.data(), order, h->wjvp);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; i++) jv[i] = rd[i].d;
    return 0;
}

// Exact transposed products out_q = (dR/dQ)^T psi, out_b = (dR/dbeta)^T psi,
// assembled from coloured JVPs: cells coloured by (i mod 5, j mod 5) never
// share a residual row (13-point stencil), so each JVP recovers whole columns.
int port_vjp(void* hp, const double* q, const double* beta, const double* psi,
             double* out_q, double* out_b, int order) {
    auto* h = static_cast<Handle*>(hp);
    const PCase& pc = h->pc;
    const int nic = pc.nic, njc = pc.njc, nq = pc.nq;
    const size_t n = (size_t)nic * njc * nq, nc = (size_t)nic * njc;
    const int nseeds = 25 * (nq + 1);
    if (out_q) std::memset(out_q, 0, n * 8);
    if (out_b) std::memset(out_b, 0, nc * 8);
    // Wake and periodic boundaries couple cells far apart (bc.cpp:224-263,
    // 329-364): a 5x5 colouring would alias their rows, so each cell is seeded
    // alone and psi is dotted with every row (exact, dense; small grids).
    bool nonlocal = false;
    for (const auto& b : pc.bcs) nonlocal |= (b.type == ST_BC_WAKE || b.type == ST_BC_PERIODIC);
    if (nonlocal) {
#pragma omp parallel
        {
            std::vector<Dual> qd(n), bd(nc), rd(n);
            Work<Dual> w;
            w.init(pc);
#pragma omp for schedule(dynamic, 8)
            for (long s = 0; s < (long)(nc * (nq + 1)); s++) {
                const size_t cell = (size_t)s / (nq + 1);
                const int comp = (int)(s % (nq + 1));
                if (comp == nq && (!out_b || !pc.sa)) continue;
                for (size_t i = 0; i < n; i++) qd[i] = Dual(q[i], 0.0);
                for (size_t i = 0; i < nc; i++) bd[i] = Dual(beta ? beta[i] : 1.0, 0.0);
                if (comp < nq) qd[cell * nq + comp].d = 1.0;
                else bd[cell].d = 1.0;
                residual<Dual>(pc, qd.data(), bd.data(), rd.data(), order, w);
                double acc = 0.0;
                for (size_t r = 0; r < n; r++) acc += psi[r] * rd[r].d;
                if (comp < nq) { if (out_q) out_q[cell * nq + comp] = acc; }
                else out_b[cell] = acc;
            }
        }
        return 0;
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int s = 0; s < nseeds; s++) {
        int colour = s / (nq + 1), comp = s % (nq + 1);
        int ci = colour / 5, cj = colour % 5;
        if (comp == nq && (!out_b || !pc.sa)) continue;
        std::vector<Dual> qd(n), bd(nc), rd(n);
        for (size_t i = 0; i < n; i++) qd[i] = Dual(q[i], 0.0);
        for (size_t i = 0; i < nc; i++) bd[i] = Dual(beta ? beta[i] : 1.0, 0.0);
        for (int i = ci; i < nic; i += 5)
            for (int j = cj; j < njc; j += 5) {
                if (comp < nq) qd[((size_t)i * njc + j) * nq + comp].d = 1.0;
                else bd[(size_t)i * njc + j].d = 1.0;
            }
        Work<Dual> w;
        w.init(pc);
        residual<Dual>(pc, qd.data(), bd.data(), rd.data(), order, w);
        // column (cell c, comp) collects psi . dR/dx_c over rows near c
        for (int i = ci; i < nic; i += 5)
            for (int j = cj; j < njc; j += 5) {
                double acc = 0.0;
                for (int di = -2; di <= 2; di++)
                    for (int dj = -2; dj <= 2; dj++) {
                        int ii = i + di, jj = j + dj;
                        if (ii < 0 || jj < 0 || ii >= nic || jj >= njc) continue;
                        for (int k = 0; k < nq; k++) {
                            size_t r = ((size_t)ii * njc + jj) * nq + k;
                            acc += psi[r] * rd[r].d;
                        }
                    }
                if (comp < nq) { if (out_q) out_q[((size_t)i * njc + j) * nq + comp] = acc; }
                else out_b[(size_t)i * njc + j] = acc;
            }
    }
    return 0;
}

// dJ/dQ (J from port_skin_friction) by coloured JVPs of the wall rows.
int port_objective_grad(void* hp, const double* q, double* dJdq) {
    auto* h = static_cast<Handle*>(hp);
    const PCase& pc = h->pc;
    const int nic = pc.nic, njc = pc.njc, nq = pc.nq;
    const size_t n = (size_t)nic * njc * nq, nc = (size_t)nic * njc;
    std::memset(dJdq, 0, n * 8);
    std::vector<double> dx(nic, 0.0);
    for (int i = std::max(pc.c.plate_vertex, 0); i < nic; i++) {
        double x0 = pc.xv[(size_t)i * pc.nj], x1 = pc.xv[(size_t)(i + 1) * pc.nj];
        if (0.5 * (x0 + x1) <= pc.c.plate_x_end) dx[i] = x1 - x0;
    }
    // a wake ghost reaches a distant column (see port_vjp): seed the first
    // three rows cell by cell and sum over every face
    bool nonlocal = false;
    for (const auto& b : pc.bcs) nonlocal |= (b.type == ST_BC_WAKE || b.type == ST_BC_PERIODIC);
    if (nonlocal) {
        const int rows = std::min(3, njc);
#pragma omp parallel
        {
            std::vector<Dual> qd(n), bd(nc), rd(n), cf(nic);
            Work<Dual> w;
            w.init(pc);
#pragma omp for schedule(dynamic, 4)
            for (long s = 0; s < (long)nic * rows * nq; s++) {
                const int comp = (int)(s % nq), j = (int)((s / nq) % rows), i = (int)(s / nq / rows);
                for (size_t t = 0; t < n; t++) qd[t] = Dual(q[t], 0.0);
                for (size_t t = 0; t < nc; t++) bd[t] = Dual(1.0, 0.0);
                qd[((size_t)i * njc + j) * nq + comp].d = 1.0;
                residual<Dual>(pc, qd.data(), bd.data(), rd.data(), pc.c.order, w, cf.data());
                double acc = 0.0;
                for (int ii = 0; ii < nic; ii++) acc += dx[ii] * cf[ii].d;
                dJdq[((size_t)i * njc + j) * nq + comp] = acc;
            }
        }
        return 0;
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int s = 0; s < 25 * nq; s++) {
        int colour = s / nq, comp = s % nq, ci = colour / 5, cj = colour % 5;
        if (cj > 2) continue;  // wall Cf depends on rows 0..1 (and 2 via ghosts)
        std::vector<Dual> qd(n), bd(nc), rd(n), cf(nic);
        for (size_t i = 0; i < n; i++) qd[i] = Dual(q[i], 0.0);
        for (size_t i = 0; i < nc; i++) bd[i] = Dual(1.0, 0.0);
        for (int i = ci; i < nic; i += 5)
            if (cj < njc) qd[((size_t)i * njc + cj) * nq + comp].d = 1.0;
        Work<Dual> w;
        w.init(pc);
        residual<Dual>(pc, qd.data(), bd.data(), rd.data(), pc.c.order, w, cf.data());
        for (int i = ci; i < nic; i += 5) {
            if (cj >= njc) continue;
            double acc = 0.0;
            for (int di = -2; di <= 2; di++) {
                int ii = i + di;
                if (ii < 0 || ii >= nic) continue;
                acc += dx[ii] * cf[ii].d;
            }
            dJdq[((size_t)i * njc + cj) * nq + comp] = acc;
        }
    }
    return 0;
}

}  // extern "C"
