// Hand-written reverse mode of the residual pipeline (discrete adjoint).
//
// psi^T R(Q, beta) is differentiated pass by pass, in reverse order, without a
// tape: each face recomputes its forward flux from the primitives and then
// runs the adjoint of that computation.  There are no atomics: a face writes
// its own adjoint record, and each cell gathers from the fixed set of faces
// whose stencil contains it (face colouring collapsed to one colour per face
// family, scatter turned into gather), so results are deterministic.
//
// The reference tapes the same residual with ADOL-C (src/solver/solver.cpp:
// 72-90) and only ever forms dR/dQ by sparse_jac (:156); it has no adjoint.
#pragma once
#include "st_kernels.cuh"

namespace st {

// face adjoint record layout (ARW doubles per face)
enum {
    A_QL = 0,          // [5] adjoint of the left reconstructed state (rho,u,v,p,nut)
    A_QR = 5,          // [5] right state
    A_DUDX = 10, A_DUDY, A_DVDX, A_DVDY, A_DTDX, A_DTDY,
    A_UB, A_VB, A_MUB, A_MUTB, A_DNDX, A_DNDY, A_RNB,
    ARW = 24
};
// per-cell source adjoint record: gbar (4), rho, nut, mu
enum { S_GU = 0, S_GV, S_GNX, S_GNY, S_RHO, S_NUT, S_MU, SRW = 8 };

__device__ inline double sgn(double x) { return x < 0.0 ? -1.0 : 1.0; }

// Reverse of roe_flux: given fb[0..3] (adjoint of f), accumulate the adjoints
// of the eight face states.
__device__ inline void roe_flux_adj(double rlft, double ulft, double vlft, double plft, double rrht, double urht,
                                    double vrht, double prht, double r1, double r2, double aj, const double* fb,
                                    double* bl, double* br) {
    // ---- forward recompute -------------------------------------------------
    const double rlfti = 1.0 / rlft;
    const double rulft = rlft * ulft, rvlft = rlft * vlft;
    const double uvl = 0.5 * (ulft * ulft + vlft * vlft);
    const double elft = plft * OGM1 + rlft * uvl;
    const double hlft = (elft + plft) * rlfti;
    const double rrhti = 1.0 / rrht;
    const double rurht = rrht * urht, rvrht = rrht * vrht;
    const double uvr = 0.5 * (urht * urht + vrht * vrht);
    const double erht = prht * OGM1 + rrht * uvr;
    const double hrht = (erht + prht) * rrhti;
    const double rat = ::sqrt(rrht * rlfti);
    const double rati = 1.0 / (rat + 1.0);
    const double rav = rat * rlft;
    const double uav = (rat * urht + ulft) * rati;
    const double vav = (rat * vrht + vlft) * rati;
    const double hav = (rat * hrht + hlft) * rati;
    const double uv = 0.5 * (uav * uav + vav * vav);
    const double cav = ::sqrt(GM1 * (hav - uv));
    const double aq1 = rrht - rlft, aq2 = urht - ulft, aq3 = vrht - vlft, aq4 = prht - plft;
    const double uu = r1 * uav + r2 * vav;
    const double c2 = cav * cav;
    const double c2i = 1.0 / c2;
    const double auu = ::fabs(uu), aupc = ::fabs(uu + cav), aumc = ::fabs(uu - cav);
    const double uulft = r1 * ulft + r2 * vlft, uurht = r1 * urht + r2 * vrht;
    const double rcav = rav * cav;
    const double aquu = uurht - uulft;
    const double c2ih = 0.5 * c2i;
    const double ruuav = auu * rav;
    const double t2 = aq4 + rcav * aquu, t3 = aq4 - rcav * aquu;
    const double b1 = auu * (aq1 - c2i * aq4);
    const double b2 = c2ih * aupc * t2;
    const double b3 = c2ih * aumc * t3;
    const double b4 = b1 + b2 + b3;
    const double b5 = cav * (b2 - b3);
    const double b6 = ruuav * (aq2 - r1 * aquu);
    const double b7 = ruuav * (aq3 - r2 * aquu);
    const double eplft = elft + plft, eprht = erht + prht;
    // ---- reverse -------------------------------------------------------------
    const double g0 = aj * fb[0], g1 = aj * fb[1], g2 = aj * fb[2], g3 = aj * fb[3];
    double rlft_ = 0, ulft_ = 0, vlft_ = 0, plft_ = 0, rrht_ = 0, urht_ = 0, vrht_ = 0, prht_ = 0;
    double uulft_ = 0, uurht_ = 0, rulft_ = 0, rurht_ = 0, rvlft_ = 0, rvrht_ = 0, eplft_ = 0, eprht_ = 0;
    double plar_ = 0;
    rlft_ += g0 * uulft; uulft_ += g0 * rlft; rrht_ += g0 * uurht; uurht_ += g0 * rrht;
    const double d1_ = -g0;
    rulft_ += g1 * uulft; uulft_ += g1 * rulft; rurht_ += g1 * uurht; uurht_ += g1 * rurht; plar_ += g1 * r1;
    const double d2_ = -g1;
    rvlft_ += g2 * uulft; uulft_ += g2 * rvlft; rvrht_ += g2 * uurht; uurht_ += g2 * rvrht; plar_ += g2 * r2;
    const double d3_ = -g2;
    eplft_ += g3 * uulft; uulft_ += g3 * eplft; eprht_ += g3 * uurht; uurht_ += g3 * eprht;
    const double d4_ = -g3;
    double elft_ = eplft_, erht_ = eprht_;
    plft_ += eplft_ + plar_;
    prht_ += eprht_ + plar_;
    // d4 = hav b4 + uu b5 + uav b6 + vav b7 - c2 b1 OGM1
    double hav_ = d4_ * b4, b4_ = d4_ * hav, uu_ = d4_ * b5, b5_ = d4_ * uu, uav_ = d4_ * b6, b6_ = d4_ * uav;
    double vav_ = d4_ * b7, b7_ = d4_ * vav, c2_ = -d4_ * b1 * OGM1, b1_ = -d4_ * c2 * OGM1;
    // d3 = vav b4 + r2 b5 + b7
    vav_ += d3_ * b4; b4_ += d3_ * vav; b5_ += d3_ * r2; b7_ += d3_;
    // d2 = uav b4 + r1 b5 + b6
    uav_ += d2_ * b4; b4_ += d2_ * uav; b5_ += d2_ * r1; b6_ += d2_;
    b4_ += d1_;
    double ruuav_ = b7_ * (aq3 - r2 * aquu) + b6_ * (aq2 - r1 * aquu);
    double aq3_ = b7_ * ruuav, aq2_ = b6_ * ruuav;
    double aquu_ = -b7_ * ruuav * r2 - b6_ * ruuav * r1;
    double cav_ = b5_ * (b2 - b3);
    double b2_ = b5_ * cav, b3_ = -b5_ * cav;
    b1_ += b4_; b2_ += b4_; b3_ += b4_;
    double c2ih_ = b3_ * aumc * t3 + b2_ * aupc * t2;
    double aumc_ = b3_ * c2ih * t3, aupc_ = b2_ * c2ih * t2;
    double aq4_ = b3_ * c2ih * aumc + b2_ * c2ih * aupc;
    double rcav_ = -b3_ * c2ih * aumc * aquu + b2_ * c2ih * aupc * aquu;
    aquu_ += -b3_ * c2ih * aumc * rcav + b2_ * c2ih * aupc * rcav;
    double auu_ = b1_ * (aq1 - c2i * aq4);
    double aq1_ = b1_ * auu;
    double c2i_ = -b1_ * auu * aq4;
    aq4_ += -b1_ * auu * c2i;
    auu_ += ruuav_ * rav;
    double rav_ = ruuav_ * auu;
    c2i_ += 0.5 * c2ih_;
    uurht_ += aquu_; uulft_ -= aquu_;
    rav_ += rcav_ * cav; cav_ += rcav_ * rav;
    urht_ += uurht_ * r1; vrht_ += uurht_ * r2; ulft_ += uulft_ * r1; vlft_ += uulft_ * r2;
    const double sm = sgn(uu - cav), sp = sgn(uu + cav), s0 = sgn(uu);
    uu_ += aumc_ * sm; cav_ -= aumc_ * sm;
    uu_ += aupc_ * sp; cav_ += aupc_ * sp;
    uu_ += auu_ * s0;
    c2_ += -c2i_ * c2i * c2i;
    cav_ += 2.0 * cav * c2_;
    uav_ += uu_ * r1; vav_ += uu_ * r2;
    rrht_ += aq1_; rlft_ -= aq1_; urht_ += aq2_; ulft_ -= aq2_; vrht_ += aq3_; vlft_ -= aq3_; prht_ += aq4_; plft_ -= aq4_;
    {
        const double tmp = cav_ * GM1 * 0.5 / cav;
        hav_ += tmp;
        const double uv_ = -tmp;
        uav_ += uv_ * uav; vav_ += uv_ * vav;
    }
    double rat_ = 0, rati_ = 0, hrht_ = 0, hlft_ = 0;
    rat_ += hav_ * hrht * rati; hrht_ += hav_ * rat * rati; hlft_ += hav_ * rati; rati_ += hav_ * (rat * hrht + hlft);
    rat_ += vav_ * vrht * rati; vrht_ += vav_ * rat * rati; vlft_ += vav_ * rati; rati_ += vav_ * (rat * vrht + vlft);
    rat_ += uav_ * urht * rati; urht_ += uav_ * rat * rati; ulft_ += uav_ * rati; rati_ += uav_ * (rat * urht + ulft);
    rat_ += rav_ * rlft; rlft_ += rav_ * rat;
    rat_ += -rati_ * rati * rati;
    double rlfti_ = 0, rrhti_ = 0;
    {
        const double tmp = rat_ * 0.5 / rat;
        rrht_ += tmp * rlfti; rlfti_ += tmp * rrht;
    }
    erht_ += hrht_ * rrhti; prht_ += hrht_ * rrhti; rrhti_ += hrht_ * (erht + prht);
    prht_ += erht_ * OGM1; rrht_ += erht_ * uvr;
    {
        const double uvr_ = erht_ * rrht;
        urht_ += uvr_ * urht; vrht_ += uvr_ * vrht;
    }
    rrht_ += rvrht_ * vrht + rurht_ * urht; vrht_ += rvrht_ * rrht; urht_ += rurht_ * rrht;
    rrht_ += -rrhti_ * rrhti * rrhti;
    elft_ += hlft_ * rlfti; plft_ += hlft_ * rlfti; rlfti_ += hlft_ * (elft + plft);
    plft_ += elft_ * OGM1; rlft_ += elft_ * uvl;
    {
        const double uvl_ = elft_ * rlft;
        ulft_ += uvl_ * ulft; vlft_ += uvl_ * vlft;
    }
    rlft_ += rvlft_ * vlft + rulft_ * ulft; vlft_ += rvlft_ * rlft; ulft_ += rulft_ * rlft;
    rlft_ += -rlfti_ * rlfti * rlfti;
    bl[0] += rlft_; bl[1] += ulft_; bl[2] += vlft_; bl[3] += plft_;
    br[0] += rrht_; br[1] += urht_; br[2] += vrht_; br[3] += prht_;
}

// Reverse of sa_source (same forward formulas); outputs adjoints of rho, nut,
// mu, omega, |grad nut|^2 and beta for source adjoint sb.
__device__ inline void sa_source_adj(double rho, double nut, double mu, double d, double omega, double gnut2,
                                     double beta, double sb, double* rho_, double* nut_, double* mu_,
                                     double* omega_, double* gnut2_, double* beta_) {
    const double k2d2 = SA_KAPPA * SA_KAPPA * d * d;
    const double chi = rho * nut / mu;
    const double chi3 = chi * chi * chi;
    const double den = chi3 + SA_CV1_3;
    const double fv1 = chi3 / den;
    const double E = 1.0 + chi * fv1;
    const double fv2 = 1.0 - chi / E;
    const double sbar = nut * fv2 * (1.0 / k2d2);
    const bool br1 = sbar >= -SA_CV2 * omega;
    double stilde, N = 0, D = 1;
    if (br1) {
        stilde = omega + sbar;
    } else {
        N = SA_CV2 * SA_CV2 * omega + SA_CV3 * sbar;
        D = (SA_CV3 - 2.0 * SA_CV2) * omega - sbar;
        stilde = omega + omega * N / D;
    }
    double r;
    bool rfree = false;
    if (stilde > 0.0) {
        r = nut / (stilde * k2d2);
        if (r < 10.0) rfree = true; else r = 10.0;
    } else {
        r = 10.0;
    }
    const double r2 = r * r;
    const double gg = r + SA_CW2 * (r2 * r2 * r2 - r);
    const double g2 = gg * gg;
    const double g6 = g2 * g2 * g2;
    const double z = (1.0 + SA_CW3_6) / (g6 + SA_CW3_6);
    const double h = ::cbrt(::sqrt(z));
    const double fw = gg * h;
    const double prod = beta * SA_CB1 * stilde * nut;
    const double dest = SA_CW1 * fw * (nut * nut) / (d * d);
    // reverse
    double rhob = sb * (prod - dest + (SA_CB2 / SA_SIGMA) * gnut2);
    const double prod_ = sb * rho, dest_ = -sb * rho;
    *gnut2_ = sb * rho * (SA_CB2 / SA_SIGMA);
    double fw_ = dest_ * SA_CW1 * nut * nut / (d * d);
    double nutb = dest_ * SA_CW1 * fw * 2.0 * nut / (d * d);
    *beta_ = prod_ * SA_CB1 * stilde * nut;
    double stilde_ = prod_ * beta * SA_CB1 * nut;
    nutb += prod_ * beta * SA_CB1 * stilde;
    double gg_ = fw_ * h;
    const double h_ = fw_ * gg;
    const double z_ = h_ * h / (6.0 * z);
    const double g6_ = -z_ * z / (g6 + SA_CW3_6);
    const double g2_ = g6_ * 3.0 * g2 * g2;
    gg_ += g2_ * 2.0 * gg;
    const double r_ = gg_ * (1.0 + SA_CW2 * (6.0 * r2 * r2 * r - 1.0));
    if (rfree) {
        nutb += r_ / (stilde * k2d2);
        stilde_ += -r_ * r / stilde;
    }
    double omegab = 0.0, sbar_ = 0.0;
    if (br1) {
        omegab += stilde_;
        sbar_ += stilde_;
    } else {
        omegab += stilde_ * (1.0 + N / D);
        const double N_ = stilde_ * omega / D;
        const double D_ = -stilde_ * omega * N / (D * D);
        omegab += N_ * SA_CV2 * SA_CV2 + D_ * (SA_CV3 - 2.0 * SA_CV2);
        sbar_ += N_ * SA_CV3 - D_;
    }
    nutb += sbar_ * fv2 / k2d2;
    const double fv2_ = sbar_ * nut / k2d2;
    double chi_ = -fv2_ / E + fv2_ * chi * fv1 / (E * E);
    const double fv1_ = fv2_ * chi * chi / (E * E);
    const double chi3_ = fv1_ * SA_CV1_3 / (den * den);
    chi_ += chi3_ * 3.0 * chi * chi;
    rhob += chi_ * nut / mu;
    nutb += chi_ * rho / mu;
    *mu_ = -chi_ * chi / mu;
    *rho_ = rhob;
    *nut_ = nutb;
    *omega_ = omegab;
}

// SA only: face gradient parts (u_y, v_x, nut_x, nut_y) the cell source needs.
template <int DIR>
__global__ void __launch_bounds__(256) k_face_grad(DevCase c, const double* __restrict__ P, double* __restrict__ G) {
    const int na = DIR == 0 ? c.ni : c.nic;
    const int nb = DIR == 0 ? c.njc : c.nj;
    const size_t n = (size_t)na * nb;
    const double* geo = DIR == 0 ? c.geo_i : c.geo_j;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const FaceIdx fi = face_idx<DIR>(c, (int)(idx / nb), (int)(idx % nb));
        const double* gm = geo + fi.face * NGEO;
        const double* L = P + fi.L; const double* R = P + fi.R;
        const double* a = P + fi.Pa; const double* b = P + fi.Pb;
        const double* m = P + fi.Ma; const double* q = P + fi.Mb;
        double* g = G + fi.face * 4;
        g[0] = gm[G_WLY] * L[P_U] + gm[G_WRY] * R[P_U] + gm[G_WPY] * (a[P_U] + b[P_U]) + gm[G_WMY] * (m[P_U] + q[P_U]);
        g[1] = gm[G_WLX] * L[P_V] + gm[G_WRX] * R[P_V] + gm[G_WPX] * (a[P_V] + b[P_V]) + gm[G_WMX] * (m[P_V] + q[P_V]);
        g[2] = gm[G_WLX] * L[P_NUT] + gm[G_WRX] * R[P_NUT] + gm[G_WPX] * (a[P_NUT] + b[P_NUT]) + gm[G_WMX] * (m[P_NUT] + q[P_NUT]);
        g[3] = gm[G_WLY] * L[P_NUT] + gm[G_WRY] * R[P_NUT] + gm[G_WPY] * (a[P_NUT] + b[P_NUT]) + gm[G_WMY] * (m[P_NUT] + q[P_NUT]);
    }
}

// R1: adjoint weights w = psi / V per cell, and the SA source adjoint.
template <int NQ>
__global__ void __launch_bounds__(256) k_cell_adj(DevCase c, const double* __restrict__ P, const double* __restrict__ Gi,
                                                  const double* __restrict__ Gj, const double* __restrict__ beta,
                                                  const double* __restrict__ psi, double* __restrict__ w,
                                                  double* __restrict__ srec, double* __restrict__ outb) {
    const size_t n = (size_t)c.nic * c.njc;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / c.njc), j = (int)(idx % c.njc);
        const double iv = c.ivol[idx];
#pragma unroll
        for (int k = 0; k < NQ; k++) w[idx * NQ + k] = psi[idx * NQ + k] * iv;
        if (NQ == 5) {
            double* s = srec + idx * SRW;
            double bb = 0.0;
            if (c.viscous) {
                const double* gw = Gi + ((size_t)i * c.njc + j) * 4;
                const double* ge = Gi + ((size_t)(i + 1) * c.njc + j) * 4;
                const double* gs = Gj + ((size_t)i * c.nj + j) * 4;
                const double* gn = Gj + ((size_t)i * c.nj + j + 1) * 4;
                const double uy = 0.25 * (gw[0] + ge[0] + gs[0] + gn[0]);
                const double vx = 0.25 * (gw[1] + ge[1] + gs[1] + gn[1]);
                const double nx = 0.25 * (gw[2] + ge[2] + gs[2] + gn[2]);
                const double ny = 0.25 * (gw[3] + ge[3] + gs[3] + gn[3]);
                const double om = ::fabs(vx - uy);
                const double* pc = P + pidx(c, i + 1, j + 1);
                const double bt = beta ? beta[idx] : 1.0;
                // rhs_4 = (... + S V) / V, so dJ/dS = psi_4 (V/V)
                const double sb = psi[idx * NQ + 4] * (c.vol[idx] * iv);
                double rho_, nut_, mu_, om_, g2_, b_;
                sa_source_adj(pc[P_RHO], pc[P_NUT], pc[P_MU], c.wd[idx], om, nx * nx + ny * ny, bt, sb, &rho_, &nut_,
                              &mu_, &om_, &g2_, &b_);
                const double sg = sgn(vx - uy);
                s[S_GU] = 0.25 * (-om_ * sg);
                s[S_GV] = 0.25 * (om_ * sg);
                s[S_GNX] = 0.25 * (2.0 * nx * g2_);
                s[S_GNY] = 0.25 * (2.0 * ny * g2_);
                s[S_RHO] = rho_; s[S_NUT] = nut_; s[S_MU] = mu_;
                bb = b_;
            } else {
                for (int k = 0; k < SRW; k++) s[k] = 0.0;
            }
            if (outb) outb[idx] = bb;
        }
    }
}

// R2: per face, recompute the flux and run its adjoint.  Seed: the flux
// adjoint w(R) - w(L) (ghost sides 0) and, with SA, the gradient-part
// adjoints of the two adjacent cells' sources.
template <int NQ, int DIR, int ORDER>
__global__ void __launch_bounds__(256) k_face_adj(DevCase c, const double* __restrict__ P, const double* __restrict__ phi,
                                                  const double* __restrict__ w, const double* __restrict__ srec,
                                                  double* __restrict__ arec) {
    const int na = DIR == 0 ? c.ni : c.nic;
    const int nb = DIR == 0 ? c.njc : c.nj;
    const size_t n = (size_t)na * nb;
    const double* geo = DIR == 0 ? c.geo_i : c.geo_j;
    const int slot[5] = {P_RHO, P_U, P_V, P_P, P_NUT};
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(idx / nb), b = (int)(idx % nb);
        const FaceIdx fi = face_idx<DIR>(c, a, b);
        const double* gm = geo + fi.face * NGEO;
        const double* pL = P + fi.L;
        const double* pR = P + fi.R;
        double* o = arec + fi.face * ARW;
        // flux seed
        double fb[5];
#pragma unroll
        for (int k = 0; k < NQ; k++) {
            const double wr = fi.limR ? w[fi.phR * NQ + k] : 0.0;
            const double wl = fi.limL ? w[fi.phL * NQ + k] : 0.0;
            fb[k] = wr - wl;
        }
        // face states
        double qL[5], qR[5];
#pragma unroll
        for (int k = 0; k < NQ; k++) {
            const int m = slot[k];
            qL[k] = pL[m];
            qR[k] = pR[m];
            if (ORDER == 2) {
                const double dC = pR[m] - pL[m];
                if (fi.limL) qL[k] += phi[fi.phL * NQ + k] * (THM * (pL[m] - P[fi.LL + m]) + THP * dC);
                if (fi.limR) qR[k] -= phi[fi.phR * NQ + k] * (THP * dC + THM * (P[fi.RR + m] - pR[m]));
            }
        }
        double bl[5] = {0, 0, 0, 0, 0}, br[5] = {0, 0, 0, 0, 0};
        double fc0b = fb[0];
        if (NQ == 5) {
            // f4 = f0 * nut_upwind
            double f[4];
            roe_flux<double>(qL[0], qL[1], qL[2], qL[3], qR[0], qR[1], qR[2], qR[3], gm[G_R1], gm[G_R2], gm[G_AJ], f);
            const bool up = f[0] >= 0.0;
            const double nup = up ? qL[4] : qR[4];
            fc0b += fb[4] * nup;
            if (up) bl[4] += fb[4] * f[0]; else br[4] += fb[4] * f[0];
        }
        {
            const double fcb[4] = {fc0b, fb[1], fb[2], fb[3]};
            roe_flux_adj(qL[0], qL[1], qL[2], qL[3], qR[0], qR[1], qR[2], qR[3], gm[G_R1], gm[G_R2], gm[G_AJ], fcb, bl, br);
        }
#pragma unroll
        for (int k = 0; k < 5; k++) { o[A_QL + k] = bl[k]; o[A_QR + k] = br[k]; }
        if (c.viscous) {
            const double* pPa = P + fi.Pa; const double* pPb = P + fi.Pb;
            const double* pMa = P + fi.Ma; const double* pMb = P + fi.Mb;
            const double wLx = gm[G_WLX], wLy = gm[G_WLY], wRx = gm[G_WRX], wRy = gm[G_WRY];
            const double wPx = gm[G_WPX], wPy = gm[G_WPY], wMx = gm[G_WMX], wMy = gm[G_WMY];
#define ST_GRAD_D(m, gx, gy, avg)                                                    \
            {                                                                        \
                const double sP = pPa[m] + pPb[m], sM = pMa[m] + pMb[m];             \
                gx = wLx * pL[m] + wRx * pR[m] + wPx * sP + wMx * sM;                \
                gy = wLy * pL[m] + wRy * pR[m] + wPy * sP + wMy * sM;                \
                avg = 0.375 * (pL[m] + pR[m]) + 0.0625 * (sP + sM);                  \
            }
            double dudx, dudy, ub, dvdx, dvdy, vb, dTdx, dTdy, Tb;
            ST_GRAD_D(P_U, dudx, dudy, ub)
            ST_GRAD_D(P_V, dvdx, dvdy, vb)
            ST_GRAD_D(P_T, dTdx, dTdy, Tb)
            (void)Tb;
            const double mub = 0.375 * (pL[P_MU] + pR[P_MU]) + 0.0625 * (pPa[P_MU] + pPb[P_MU] + pMa[P_MU] + pMb[P_MU]);
            double mutb = 0.0, mu = mub, k;
            if (NQ == 5) {
                mutb = 0.375 * (pL[P_MUT] + pR[P_MUT]) + 0.0625 * (pPa[P_MUT] + pPb[P_MUT] + pMa[P_MUT] + pMb[P_MUT]);
                mu = mub + mutb;
                k = c.cp * (mub * (1.0 / c.pr) + mutb * (1.0 / PR_TURB));
            } else {
                k = mub * (c.cp / c.pr);
            }
            const double nx = gm[G_NX], ny = gm[G_NY];
            const double div = dudx + dvdy;
            const double txy = mu * (dudy + dvdx);
            const double txx = mu * (2.0 * dudx - 2.0 / 3.0 * div);
            const double tyy = mu * (2.0 * dvdy - 2.0 / 3.0 * div);
            // F_net = F_conv - F_visc
            const double v1 = -fb[1], v2 = -fb[2], v3 = -fb[3];
            const double A_ = v3 * nx, B_ = v3 * ny;
            const double ub_ = A_ * txx + B_ * txy;
            const double vb_ = A_ * txy + B_ * tyy;
            double txx_ = A_ * ub + v1 * nx;
            double txy_ = A_ * vb + B_ * ub + v2 * nx + v1 * ny;
            double tyy_ = B_ * vb + v2 * ny;
            const double qx_ = -A_, qy_ = -B_;
            const double k_ = -qx_ * dTdx - qy_ * dTdy;
            const double dTdx_ = -qx_ * k, dTdy_ = -qy_ * k;
            double mu_ = tyy_ * (2.0 * dvdy - 2.0 / 3.0 * div) + txx_ * (2.0 * dudx - 2.0 / 3.0 * div) + txy_ * (dudy + dvdx);
            double dvdy_ = tyy_ * mu * 2.0, dudx_ = txx_ * mu * 2.0;
            const double div_ = -(tyy_ + txx_) * mu * (2.0 / 3.0);
            double dudy_ = txy_ * mu, dvdx_ = txy_ * mu;
            dudx_ += div_; dvdy_ += div_;
            double mub_ = mu_, mutb_ = 0.0;
            if (NQ == 5) { mutb_ = mu_; mub_ += k_ * c.cp / c.pr; mutb_ += k_ * c.cp / PR_TURB; }
            else mub_ += k_ * (c.cp / c.pr);
            o[A_DTDX] = dTdx_; o[A_DTDY] = dTdy_;
            o[A_UB] = ub_; o[A_VB] = vb_;
            if (NQ == 5) {
                double dndx, dndy, nb_;
                ST_GRAD_D(P_NUT, dndx, dndy, nb_)
                (void)nb_;
                const double rnb = 0.375 * (pL[P_RHO] * pL[P_NUT] + pR[P_RHO] * pR[P_NUT])
                                 + 0.0625 * (pPa[P_RHO] * pPa[P_NUT] + pPb[P_RHO] * pPb[P_NUT]
                                             + pMa[P_RHO] * pMa[P_NUT] + pMb[P_RHO] * pMb[P_NUT]);
                const double v4 = -fb[4];
                const double cs = 1.0 / SA_SIGMA;
                const double gdn = dndx * nx + dndy * ny;
                mub_ += v4 * cs * gdn;
                const double rnb_ = v4 * cs * gdn;
                double dndx_ = v4 * cs * (mub + rnb) * nx, dndy_ = v4 * cs * (mub + rnb) * ny;
                // cell-source seeds on this face's gradient parts
                const double* sl = fi.limL ? srec + fi.phL * SRW : nullptr;
                const double* sr = fi.limR ? srec + fi.phR * SRW : nullptr;
                double gs[4] = {0, 0, 0, 0};
                if (sl) for (int t = 0; t < 4; t++) gs[t] += sl[t];
                if (sr) for (int t = 0; t < 4; t++) gs[t] += sr[t];
                dudy_ += gs[0]; dvdx_ += gs[1]; dndx_ += gs[2]; dndy_ += gs[3];
                o[A_DNDX] = dndx_; o[A_DNDY] = dndy_; o[A_RNB] = rnb_;
            } else {
                o[A_DNDX] = 0.0; o[A_DNDY] = 0.0; o[A_RNB] = 0.0;
            }
            o[A_DUDX] = dudx_; o[A_DUDY] = dudy_; o[A_DVDX] = dvdx_; o[A_DVDY] = dvdy_;
            o[A_MUB] = mub_; o[A_MUTB] = mutb_;
#undef ST_GRAD_D
        } else {
            for (int t = A_DUDX; t <= A_RNB; t++) o[t] = 0.0;
        }
    }
}

// R3: limiter adjoint per physical cell and direction.  For cell c the
// limited states are qL(c's high face) = P + phi (THM d- + THP d+) and
// qR(c's low face) = P - phi (THP d- + THM d+) with d- = P(c)-P(c-1),
// d+ = P(c+1)-P(c).  Writes (dbar-, dbar+) per component.
template <int NQ>
__global__ void __launch_bounds__(256) k_limiter_adj(DevCase c, const double* __restrict__ P,
                                                     const double* __restrict__ phi_i, const double* __restrict__ phi_j,
                                                     const double* __restrict__ ai, const double* __restrict__ aj,
                                                     double* __restrict__ lrec) {
    const size_t n = (size_t)c.nic * c.njc;
    const int slot[5] = {P_RHO, P_U, P_V, P_P, P_NUT};
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / c.njc), j = (int)(idx % c.njc);
        const double* pc = P + pidx(c, i + 1, j + 1);
#pragma unroll
        for (int dir = 0; dir < 2; dir++) {
            const double* pm = dir == 0 ? P + pidx(c, i, j + 1) : P + pidx(c, i + 1, j);
            const double* pp = dir == 0 ? P + pidx(c, i + 2, j + 1) : P + pidx(c, i + 1, j + 2);
            const double* phi = dir == 0 ? phi_i : phi_j;
            const double eps = dir == 0 ? c.eps_chi : c.eps_eta;
            // adjoint records of the high face (c is its L) and low face (c is its R)
            const double* hi = dir == 0 ? ai + ((size_t)(i + 1) * c.njc + j) * ARW : aj + ((size_t)i * c.nj + j + 1) * ARW;
            const double* lo = dir == 0 ? ai + ((size_t)i * c.njc + j) * ARW : aj + ((size_t)i * c.nj + j) * ARW;
            double* out = lrec + (idx * 2 + dir) * 2 * NQ;
#pragma unroll
            for (int k = 0; k < NQ; k++) {
                const int m = slot[k];
                const double fa = pc[m] - pm[m], fb = pp[m] - pc[m];
                const double ph = phi[idx * NQ + k];
                const double A = hi[A_QL + k], B = lo[A_QR + k];
                const double phb = A * (THM * fa + THP * fb) - B * (THP * fa + THM * fb);
                const double a2e = 2.0 * (fb - fa) * (fb - fa) + 3.0 * fb * fa + eps;
                const double dphi_dfa = (0.75 * fb - ph * (-4.0 * (fb - fa) + 3.0 * fb)) / a2e;
                const double dphi_dfb = (0.75 * fa - ph * (4.0 * (fb - fa) + 3.0 * fa)) / a2e;
                out[k] = A * ph * THM - B * ph * THP + phb * dphi_dfa;        // dbar-
                out[NQ + k] = A * ph * THP - B * ph * THM + phb * dphi_dfb;   // dbar+
            }
        }
    }
}

// R4: gather the adjoint of every ghost-padded primitive record from the
// faces whose stencils contain it.
template <int NQ, int ORDER>
__global__ void __launch_bounds__(256) k_gather(DevCase c, const double* __restrict__ P, const double* __restrict__ ai,
                                                const double* __restrict__ aj, const double* __restrict__ lrec,
                                                const double* __restrict__ srec, double* __restrict__ Pbar) {
    const size_t n = (size_t)(c.nic + 2) * (c.njc + 2);
    const int slot[5] = {P_RHO, P_U, P_V, P_P, P_NUT};
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int ip = (int)(idx / (c.njc + 2)), jp = (int)(idx % (c.njc + 2));
        double acc[NP];
#pragma unroll
        for (int s = 0; s < NP; s++) acc[s] = 0.0;
        const bool phys = ip >= 1 && ip <= c.nic && jp >= 1 && jp <= c.njc;
        const double* self = P + idx * NP;
        // ---- i-faces (f, j): L=(f, j+1) R=(f+1, j+1) P=(f|f+1, j+2) M=(f|f+1, j)
        {
            auto visc = [&](int f, int j, int role) {
                if (f < 0 || f > c.nic || j < 0 || j >= c.njc) return;
                const size_t fid = (size_t)f * c.njc + j;
                const double* r = ai + fid * ARW;
                const double* gm = c.geo_i + fid * NGEO;
                double wx, wy, co;
                if (role == 0) { wx = gm[G_WLX]; wy = gm[G_WLY]; co = 0.375; }
                else if (role == 1) { wx = gm[G_WRX]; wy = gm[G_WRY]; co = 0.375; }
                else if (role == 2) { wx = gm[G_WPX]; wy = gm[G_WPY]; co = 0.0625; }
                else { wx = gm[G_WMX]; wy = gm[G_WMY]; co = 0.0625; }
                acc[P_U] += r[A_DUDX] * wx + r[A_DUDY] * wy + r[A_UB] * co;
                acc[P_V] += r[A_DVDX] * wx + r[A_DVDY] * wy + r[A_VB] * co;
                acc[P_T] += r[A_DTDX] * wx + r[A_DTDY] * wy;
                acc[P_MU] += r[A_MUB] * co;
                if (NQ == 5) {
                    acc[P_MUT] += r[A_MUTB] * co;
                    acc[P_NUT] += r[A_DNDX] * wx + r[A_DNDY] * wy + r[A_RNB] * co * self[P_RHO];
                    acc[P_RHO] += r[A_RNB] * co * self[P_NUT];
                }
            };
            if (jp >= 1 && jp <= c.njc) {
                const int j = jp - 1;
                if (ip <= c.nic) {  // L of face ip
                    const double* r = ai + ((size_t)ip * c.njc + j) * ARW;
                    for (int k = 0; k < NQ; k++) acc[slot[k]] += r[A_QL + k];
                }
                if (ip >= 1) {  // R of face ip-1
                    const double* r = ai + ((size_t)(ip - 1) * c.njc + j) * ARW;
                    for (int k = 0; k < NQ; k++) acc[slot[k]] += r[A_QR + k];
                }
                if (ORDER == 2) {
                    if (phys) {
                        const double* l = lrec + (((size_t)(ip - 1) * c.njc + j) * 2 + 0) * 2 * NQ;
                        for (int k = 0; k < NQ; k++) acc[slot[k]] += l[k] - l[NQ + k];
                    }
                    if (ip - 1 >= 1 && ip - 1 <= c.nic) {  // left neighbour is physical: +dbar+
                        const double* l = lrec + (((size_t)(ip - 2) * c.njc + j) * 2 + 0) * 2 * NQ;
                        for (int k = 0; k < NQ; k++) acc[slot[k]] += l[NQ + k];
                    }
                    if (ip + 1 >= 1 && ip + 1 <= c.nic) {  // right neighbour is physical: -dbar-
                        const double* l = lrec + (((size_t)ip * c.njc + j) * 2 + 0) * 2 * NQ;
                        for (int k = 0; k < NQ; k++) acc[slot[k]] -= l[k];
                    }
                }
            }
            if (c.viscous) {
                visc(ip, jp - 1, 0);       // L
                visc(ip - 1, jp - 1, 1);   // R
                visc(ip, jp - 2, 2);       // P, low
                visc(ip - 1, jp - 2, 2);   // P, high
                visc(ip, jp, 3);           // M, low
                visc(ip - 1, jp, 3);       // M, high
            }
        }
        // ---- j-faces (i, g): L=(i+1, g) R=(i+1, g+1) P=(i+2, g|g+1) M=(i, g|g+1)
        {
            auto visc = [&](int i, int g, int role) {
                if (i < 0 || i >= c.nic || g < 0 || g > c.njc) return;
                const size_t fid = (size_t)i * c.nj + g;
                const double* r = aj + fid * ARW;
                const double* gm = c.geo_j + fid * NGEO;
                double wx, wy, co;
                if (role == 0) { wx = gm[G_WLX]; wy = gm[G_WLY]; co = 0.375; }
                else if (role == 1) { wx = gm[G_WRX]; wy = gm[G_WRY]; co = 0.375; }
                else if (role == 2) { wx = gm[G_WPX]; wy = gm[G_WPY]; co = 0.0625; }
                else { wx = gm[G_WMX]; wy = gm[G_WMY]; co = 0.0625; }
                acc[P_U] += r[A_DUDX] * wx + r[A_DUDY] * wy + r[A_UB] * co;
                acc[P_V] += r[A_DVDX] * wx + r[A_DVDY] * wy + r[A_VB] * co;
                acc[P_T] += r[A_DTDX] * wx + r[A_DTDY] * wy;
                acc[P_MU] += r[A_MUB] * co;
                if (NQ == 5) {
                    acc[P_MUT] += r[A_MUTB] * co;
                    acc[P_NUT] += r[A_DNDX] * wx + r[A_DNDY] * wy + r[A_RNB] * co * self[P_RHO];
                    acc[P_RHO] += r[A_RNB] * co * self[P_NUT];
                }
            };
            if (ip >= 1 && ip <= c.nic) {
                const int i = ip - 1;
                if (jp <= c.njc) {  // L of face jp
                    const double* r = aj + ((size_t)i * c.nj + jp) * ARW;
                    for (int k = 0; k < NQ; k++) acc[slot[k]] += r[A_QL + k];
                }
                if (jp >= 1) {  // R of face jp-1
                    const double* r = aj + ((size_t)i * c.nj + jp - 1) * ARW;
                    for (int k = 0; k < NQ; k++) acc[slot[k]] += r[A_QR + k];
                }
                if (ORDER == 2) {
                    if (phys) {
                        const double* l = lrec + (((size_t)i * c.njc + jp - 1) * 2 + 1) * 2 * NQ;
                        for (int k = 0; k < NQ; k++) acc[slot[k]] += l[k] - l[NQ + k];
                    }
                    if (jp - 1 >= 1 && jp - 1 <= c.njc) {
                        const double* l = lrec + (((size_t)i * c.njc + jp - 2) * 2 + 1) * 2 * NQ;
                        for (int k = 0; k < NQ; k++) acc[slot[k]] += l[NQ + k];
                    }
                    if (jp + 1 >= 1 && jp + 1 <= c.njc) {
                        const double* l = lrec + (((size_t)i * c.njc + jp) * 2 + 1) * 2 * NQ;
                        for (int k = 0; k < NQ; k++) acc[slot[k]] -= l[k];
                    }
                }
            }
            if (c.viscous) {
                visc(ip - 1, jp, 0);       // L
                visc(ip - 1, jp - 1, 1);   // R
                visc(ip - 2, jp, 2);       // P, low
                visc(ip - 2, jp - 1, 2);   // P, high
                visc(ip, jp, 3);           // M, low
                visc(ip, jp - 1, 3);       // M, high
            }
        }
        if (NQ == 5 && phys && c.viscous) {
            const double* s = srec + ((size_t)(ip - 1) * c.njc + (jp - 1)) * SRW;
            acc[P_RHO] += s[S_RHO]; acc[P_NUT] += s[S_NUT]; acc[P_MU] += s[S_MU];
        }
        double* o = Pbar + idx * NP;
#pragma unroll
        for (int s = 0; s < NP; s++) o[s] = acc[s];
    }
}

// ring index of a ghost-padded cell on the ghost layer
__device__ inline int ring_index(const DevCase& c, int ip, int jp) {
    if (jp == 0) return ip;
    if (jp == c.njc + 1) return c.nic + 2 + ip;
    if (ip == 0) return 2 * (c.nic + 2) + jp - 1;
    return 2 * (c.nic + 2) + c.njc + jp - 1;  // ip == nic+1
}
__device__ inline bool on_ring(const DevCase& c, int ip, int jp) {
    return ip == 0 || jp == 0 || ip == c.nic + 1 || jp == c.njc + 1;
}
__device__ inline int ring_size(const DevCase& c) { return 2 * (c.nic + 2) + 2 * c.njc; }
constexpr int RW = 6;  // taped slots rho,u,v,p,T,nut

// Forward boundary pass that also records the ghost layer before each BC
// (tape [nbc][ring][RW]); identical results to k_bc.
template <int NQ>
__global__ void __launch_bounds__(1024) k_bc_taped(DevCase c, double* __restrict__ P, double* __restrict__ tape) {
    const int nr = ring_size(c);
    for (int b = 0; b < c.nbc; b++) {
        for (int r = threadIdx.x; r < nr; r += blockDim.x) {
            int ip, jp;
            if (r < c.nic + 2) { ip = r; jp = 0; }
            else if (r < 2 * (c.nic + 2)) { ip = r - (c.nic + 2); jp = c.njc + 1; }
            else if (r < 2 * (c.nic + 2) + c.njc) { ip = 0; jp = r - 2 * (c.nic + 2) + 1; }
            else { ip = c.nic + 1; jp = r - 2 * (c.nic + 2) - c.njc + 1; }
            const double* g = P + pidx(c, ip, jp);
            double* t = tape + ((size_t)b * nr + r) * RW;
            for (int s = 0; s < RW; s++) t[s] = g[s];
        }
        __syncthreads();
        DevCase one = c;
        one.bcs = c.bcs + b;
        one.nbc = 1;
        one.viscous = 0;
        bc_apply_block<double, NQ>(one, P);
        __syncthreads();
    }
    if (c.viscous) bc_ghost_mu<double, NQ>(c, P);
}

// R5: reverse of the boundary pass.  First the ghost mu, mu_t, then each BC in
// reverse order: the ghost adjoint flows to the BC's inputs (read from the
// tape where they are ghosts themselves) and is cleared.
template <int NQ>
__global__ void __launch_bounds__(1024) k_bc_adj(DevCase c, const double* __restrict__ P, const double* __restrict__ tape,
                                                 double* __restrict__ Pbar) {
    const int nic = c.nic, njc = c.njc;
    const int nr = ring_size(c);
    const double iR = 1.0 / c.R;
    if (c.viscous) {
        for (int r = threadIdx.x; r < nr; r += blockDim.x) {
            int ip, jp;
            if (r < nic + 2) { ip = r; jp = 0; }
            else if (r < 2 * (nic + 2)) { ip = r - (nic + 2); jp = njc + 1; }
            else if (r < 2 * (nic + 2) + njc) { ip = 0; jp = r - 2 * (nic + 2) + 1; }
            else { ip = nic + 1; jp = r - 2 * (nic + 2) - njc + 1; }
            const double* g = P + pidx(c, ip, jp);
            double* gb = Pbar + pidx(c, ip, jp);
            double mub = gb[P_MU];
            const double T = g[P_T], mu = g[P_MU];
            if (NQ == 5 && mu != 0.0) {
                const double s = g[P_RHO] * g[P_NUT];
                const double chi = s / mu, chi3 = chi * chi * chi, den = chi3 + SA_CV1_3;
                const double f = chi3 / den, fp = 3.0 * chi * chi * SA_CV1_3 / (den * den);
                const double ds = f + chi * fp;
                gb[P_RHO] += gb[P_MUT] * ds * g[P_NUT];
                gb[P_NUT] += gb[P_MUT] * ds * g[P_RHO];
                mub += gb[P_MUT] * (-chi * chi * fp);
            }
            if (T != 0.0) {
                double dmu;
                if (c.law == 1) dmu = mu * (1.5 / T - 1.0 / (T + c.suth_S));
                else dmu = (2.0 / 3.0) * mu / T;
                gb[P_T] += mub * dmu;
            }
            gb[P_MU] = 0.0;
            gb[P_MUT] = 0.0;
        }
        __syncthreads();
    }
    // input value: ghost inputs from the tape before BC b, interior from P
    auto in = [&](int b, int ip, int jp, int s) -> double {
        if (on_ring(c, ip, jp)) return tape[((size_t)b * nr + ring_index(c, ip, jp)) * RW + s];
        return P[pidx(c, ip, jp) + s];
    };
    for (int b = c.nbc - 1; b >= 0; b--) {
        const DevBC bc = c.bcs[b];
        const bool bt = (bc.face == 0 || bc.face == 2);
        const int end = bc.end >= 0 ? bc.end : (bt ? nic : njc) + 2 + bc.end;
        const int start = bc.start;
        if (bc.type == 0) {
            for (int s = start + threadIdx.x; s <= end; s += blockDim.x) {
                int ip = bt ? s : (bc.face == 3 ? 0 : nic + 1);
                int jp = bt ? (bc.face == 0 ? 0 : njc + 1) : s;
                double* gb = Pbar + pidx(c, ip, jp);
                for (int t = 0; t < RW; t++) gb[t] = 0.0;
            }
        } else if (bc.type == 1 && bt) {
            for (int ip = start + threadIdx.x; ip <= end; ip += blockDim.x) {
                const bool bot = (bc.face == 0);
                const int jg = bot ? 0 : njc + 1, j1 = bot ? 1 : njc, j2 = bot ? 2 : njc - 1;
                const double* nn = c.neta + ((size_t)(ip - 1) * c.nj + (bot ? 0 : njc)) * 2;
                const double nx = nn[0], ny = nn[1], ds = nx * nx + ny * ny;
                double* gb = Pbar + pidx(c, ip, jg);
                double* ab = Pbar + pidx(c, ip, j1);
                double* db = Pbar + pidx(c, ip, j2);
                const double pg = 1.5 * in(b, ip, j1, P_P) - 0.5 * in(b, ip, j2, P_P);
                const double rg = 1.5 * in(b, ip, j1, P_RHO) - 0.5 * in(b, ip, j2, P_RHO);
                double pgb = gb[P_P] + gb[P_T] * iR / rg;
                double rgb = gb[P_RHO] - gb[P_T] * pg * iR / (rg * rg);
                const double un_ = -2.0 * gb[P_U] * nx / ds - 2.0 * gb[P_V] * ny / ds;
                ab[P_U] += gb[P_U] + un_ * nx;
                ab[P_V] += gb[P_V] + un_ * ny;
                ab[P_P] += 1.5 * pgb; db[P_P] -= 0.5 * pgb;
                ab[P_RHO] += 1.5 * rgb; db[P_RHO] -= 0.5 * rgb;
                ab[P_NUT] += 1.5 * gb[P_NUT]; db[P_NUT] -= 0.5 * gb[P_NUT];
                for (int t = 0; t < RW; t++) gb[t] = 0.0;
            }
        } else if (bc.type == 2 || bc.type == 5) {
            for (int s = start + threadIdx.x; s <= end; s += blockDim.x) {
                int gi, gj, ai_, aj_, di, dj;
                if (bt) {
                    const bool bot = (bc.face == 0);
                    gi = ai_ = di = s;
                    gj = bot ? 0 : njc + 1; aj_ = bot ? 1 : njc; dj = bot ? 2 : njc - 1;
                } else {
                    if (bc.type == 5) break;
                    const bool left = (bc.face == 3);
                    gj = aj_ = dj = s;
                    gi = left ? 0 : nic + 1; ai_ = left ? 1 : nic; di = left ? 2 : nic - 1;
                }
                double* gb = Pbar + pidx(c, gi, gj);
                double* ab = Pbar + pidx(c, ai_, aj_);
                double* db = Pbar + pidx(c, di, dj);
                ab[P_U] -= 1.5 * gb[P_U]; db[P_U] += 0.5 * gb[P_U];
                ab[P_V] -= 1.5 * gb[P_V]; db[P_V] += 0.5 * gb[P_V];
                ab[P_NUT] -= 1.5 * gb[P_NUT]; db[P_NUT] += 0.5 * gb[P_NUT];
                if (bc.type == 2) {
                    const double Tg = 1.5 * in(b, ai_, aj_, P_T) - 0.5 * in(b, di, dj, P_T);
                    const double rg = 1.5 * in(b, ai_, aj_, P_RHO) - 0.5 * in(b, di, dj, P_RHO);
                    const double rgb = gb[P_RHO] + gb[P_P] * c.R * Tg;
                    const double Tgb = gb[P_T] + gb[P_P] * c.R * rg;
                    ab[P_T] += 1.5 * Tgb; db[P_T] -= 0.5 * Tgb;
                    ab[P_RHO] += 1.5 * rgb; db[P_RHO] -= 0.5 * rgb;
                } else {
                    const double pgb = gb[P_P] + gb[P_RHO] * iR / bc.T;
                    ab[P_P] += 1.5 * pgb; db[P_P] -= 0.5 * pgb;
                }
                for (int t = 0; t < RW; t++) gb[t] = 0.0;
            }
        } else if (bc.type == 3 && !bt && bc.face == 1) {
            for (int jp = start + threadIdx.x; jp <= end; jp += blockDim.x) {
                double* gb = Pbar + pidx(c, nic + 1, jp);
                double* ab = Pbar + pidx(c, nic, jp);
                const double rg = in(b, nic, jp, P_RHO);
                ab[P_RHO] += gb[P_RHO] - gb[P_T] * c.p_inf * iR / (rg * rg);
                ab[P_U] += gb[P_U]; ab[P_V] += gb[P_V]; ab[P_NUT] += gb[P_NUT];
                for (int t = 0; t < RW; t++) gb[t] = 0.0;
            }
        } else if (bc.type == 4) {
            for (int s = start + threadIdx.x; s <= end; s += blockDim.x) {
                int g0i, g0j, s0i, s0j, g1i, g1j, s1i, s1j;
                if (bt) { g0i = s; g0j = 0; s0i = s; s0j = njc; g1i = s; g1j = njc + 1; s1i = s; s1j = 1; }
                else { g0i = 0; g0j = s; s0i = nic; s0j = s; g1i = nic + 1; g1j = s; s1i = 1; s1j = s; }
                double* g1b = Pbar + pidx(c, g1i, g1j);
                double* s1b = Pbar + pidx(c, s1i, s1j);
                for (int t = 0; t < RW; t++) { s1b[t] += g1b[t]; g1b[t] = 0.0; }
                double* g0b = Pbar + pidx(c, g0i, g0j);
                double* s0b = Pbar + pidx(c, s0i, s0j);
                for (int t = 0; t < RW; t++) { s0b[t] += g0b[t]; g0b[t] = 0.0; }
            }
        } else if (bc.type == 6 && bt) {
            const int jg = (bc.face == 0) ? 0 : njc + 1;
            for (int ip = start + threadIdx.x; ip <= end; ip += blockDim.x) {
                double* gb = Pbar + pidx(c, nic + 1 - ip, jg);
                double* sb = Pbar + pidx(c, ip, 1);
                for (int t = 0; t < RW; t++) { sb[t] += gb[t]; gb[t] = 0.0; }
            }
            __syncthreads();
            for (int ip = start + threadIdx.x; ip <= end; ip += blockDim.x) {
                double* gb = Pbar + pidx(c, ip, jg);
                double* sb = Pbar + pidx(c, nic + 1 - ip, 1);
                for (int t = 0; t < RW; t++) { sb[t] += gb[t]; gb[t] = 0.0; }
            }
        }
        __syncthreads();
    }
}

// R6: primitives -> conserved adjoint per physical cell (reverse of k_prim).
template <int NQ>
__global__ void __launch_bounds__(256) k_prim_adj(DevCase c, const double* __restrict__ q, const double* __restrict__ P,
                                                  const double* __restrict__ Pbar, double* __restrict__ out) {
    const size_t n = (size_t)c.nic * c.njc;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / c.njc), j = (int)(idx % c.njc);
        const double* Q = q + idx * NQ;
        const double* p = P + pidx(c, i + 1, j + 1);
        const double* b = Pbar + pidx(c, i + 1, j + 1);
        const double rho = Q[0], ri = 1.0 / rho, u = p[P_U], v = p[P_V];
        double rhob = b[P_RHO], ub = b[P_U], vb = b[P_V], pb = b[P_P], Tb = b[P_T], nutb = b[P_NUT], mub = b[P_MU];
        if (c.viscous) {
            const double mu = p[P_MU];
            if (NQ == 5) {
                const double s = rho * p[P_NUT];
                const double chi = s / mu, chi3 = chi * chi * chi, den = chi3 + SA_CV1_3;
                const double f = chi3 / den, fp = 3.0 * chi * chi * SA_CV1_3 / (den * den);
                const double ds = f + chi * fp;
                rhob += b[P_MUT] * ds * p[P_NUT];
                nutb += b[P_MUT] * ds * rho;
                mub += b[P_MUT] * (-chi * chi * fp);
            }
            const double T = p[P_T];
            const double dmu = c.law == 1 ? mu * (1.5 / T - 1.0 / (T + c.suth_S)) : (2.0 / 3.0) * mu / T;
            Tb += mub * dmu;
        }
        const double iR = 1.0 / c.R;
        pb += Tb * ri * iR;
        double rib = Tb * p[P_P] * iR;
        double Qb[5] = {0, 0, 0, 0, 0};
        if (NQ == 5) { Qb[4] = nutb * ri; rib += nutb * Q[4]; }
        Qb[3] = pb * GM1;
        rhob += -0.5 * (u * u + v * v) * GM1 * pb;
        ub += -rho * GM1 * u * pb;
        vb += -rho * GM1 * v * pb;
        Qb[2] = vb * ri; rib += vb * Q[2];
        Qb[1] = ub * ri; rib += ub * Q[1];
        rhob += -rib * ri * ri;
        Qb[0] = rhob;
#pragma unroll
        for (int k = 0; k < NQ; k++) out[idx * NQ + k] = Qb[k];
    }
}

}  // namespace st
