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

// Face adjoint record (ARW doubles per face).  The low cell L and high cell R
// of the face each get three parts per reconstructed primitive k (rho,u,v,p,
// nut): the adjoint of its reconstructed state (direct term) and the
// adjoint's contribution to the cell's d- and d+ through its slope
// (k_limiter<ADJ> stores the slope derivatives).  Then the adjoints of the
// face gradients and face averages of the viscous flux.
enum {
    A_AL = 0, A_DML = 5, A_DPL = 10,    // L: direct, d-, d+
    A_BR = 15, A_DMR = 20, A_DPR = 25,  // R: direct, d-, d+
    A_DUDX = 30, A_DUDY, A_DVDX, A_DVDY, A_DTDX, A_DTDY,
    A_UB, A_VB, A_MUB, A_MUTB, A_DNDX, A_DNDY, A_RNB,
    ARW = 44
};
// per-cell SA source record: gradient-part adjoints (4), rho, nut, mu
// adjoints, and the source value itself
enum { S_GU = 0, S_GV, S_GNX, S_GNY, S_RHO, S_NUT, S_MU, S_VAL, SRW = 8 };

__device__ inline double sgn(double x) { return x < 0.0 ? -1.0 : 1.0; }

// Roe flux forward with every intermediate kept for the reverse sweep
// (same arithmetic as roe_flux, src/model/flux.cpp:51-146).
struct RoeTape {
    double rlft, ulft, vlft, plft, rrht, urht, vrht, prht, r1, r2, aj;
    double rlfti, rulft, rvlft, uvl, elft, hlft, rrhti, rurht, rvrht, uvr, erht, hrht;
    double rat, irat, rati, rav, uav, vav, hav, uv, cav, icav, aq1, aq2, aq3, aq4, uu, c2, c2i, auu, aupc, aumc;
    double uulft, uurht, rcav, aquu, c2ih, ruuav, t2, t3, b1, b2, b3, b4, b5, b6, b7, eplft, eprht;
    double f[4];
};

__device__ inline void roe_fwd(RoeTape& t) {
    t.rlfti = nr_rcp(t.rlft);
    t.rulft = t.rlft * t.ulft; t.rvlft = t.rlft * t.vlft;
    t.uvl = 0.5 * (t.ulft * t.ulft + t.vlft * t.vlft);
    t.elft = t.plft * OGM1 + t.rlft * t.uvl;
    t.hlft = (t.elft + t.plft) * t.rlfti;
    t.rrhti = nr_rcp(t.rrht);
    t.rurht = t.rrht * t.urht; t.rvrht = t.rrht * t.vrht;
    t.uvr = 0.5 * (t.urht * t.urht + t.vrht * t.vrht);
    t.erht = t.prht * OGM1 + t.rrht * t.uvr;
    t.hrht = (t.erht + t.prht) * t.rrhti;
    t.rat = nr_sqrt_inv(t.rrht * t.rlfti, &t.irat);
    t.rati = nr_rcp(t.rat + 1.0);
    t.rav = t.rat * t.rlft;
    t.uav = (t.rat * t.urht + t.ulft) * t.rati;
    t.vav = (t.rat * t.vrht + t.vlft) * t.rati;
    t.hav = (t.rat * t.hrht + t.hlft) * t.rati;
    t.uv = 0.5 * (t.uav * t.uav + t.vav * t.vav);
    t.cav = nr_sqrt_inv(GM1 * (t.hav - t.uv), &t.icav);
    t.aq1 = t.rrht - t.rlft; t.aq2 = t.urht - t.ulft; t.aq3 = t.vrht - t.vlft; t.aq4 = t.prht - t.plft;
    t.uu = t.r1 * t.uav + t.r2 * t.vav;
    t.c2 = t.cav * t.cav;
    t.c2i = t.icav * t.icav;
    t.auu = ::fabs(t.uu); t.aupc = ::fabs(t.uu + t.cav); t.aumc = ::fabs(t.uu - t.cav);
    t.uulft = t.r1 * t.ulft + t.r2 * t.vlft; t.uurht = t.r1 * t.urht + t.r2 * t.vrht;
    t.rcav = t.rav * t.cav;
    t.aquu = t.uurht - t.uulft;
    t.c2ih = 0.5 * t.c2i;
    t.ruuav = t.auu * t.rav;
    t.t2 = t.aq4 + t.rcav * t.aquu; t.t3 = t.aq4 - t.rcav * t.aquu;
    t.b1 = t.auu * (t.aq1 - t.c2i * t.aq4);
    t.b2 = t.c2ih * t.aupc * t.t2;
    t.b3 = t.c2ih * t.aumc * t.t3;
    t.b4 = t.b1 + t.b2 + t.b3;
    t.b5 = t.cav * (t.b2 - t.b3);
    t.b6 = t.ruuav * (t.aq2 - t.r1 * t.aquu);
    t.b7 = t.ruuav * (t.aq3 - t.r2 * t.aquu);
    t.eplft = t.elft + t.plft; t.eprht = t.erht + t.prht;
    const double d2 = t.uav * t.b4 + t.r1 * t.b5 + t.b6;
    const double d3 = t.vav * t.b4 + t.r2 * t.b5 + t.b7;
    const double d4 = t.hav * t.b4 + t.uu * t.b5 + t.uav * t.b6 + t.vav * t.b7 - t.c2 * t.b1 * OGM1;
    const double plar = t.plft + t.prht;
    t.f[0] = t.aj * (t.rlft * t.uulft + t.rrht * t.uurht - t.b4);
    t.f[1] = t.aj * (t.rulft * t.uulft + t.rurht * t.uurht + t.r1 * plar - d2);
    t.f[2] = t.aj * (t.rvlft * t.uulft + t.rvrht * t.uurht + t.r2 * plar - d3);
    t.f[3] = t.aj * (t.eplft * t.uulft + t.eprht * t.uurht - d4);
}

// Reverse sweep: fb[0..3] = adjoint of f; accumulates the adjoints of the
// eight face states into bl[0..3], br[0..3].
__device__ inline void roe_rev(const RoeTape& t, const double* fb, double* bl, double* br) {
    const double rlft = t.rlft, ulft = t.ulft, vlft = t.vlft, rrht = t.rrht, urht = t.urht, vrht = t.vrht;
    const double r1 = t.r1, r2 = t.r2;
    const double g0 = t.aj * fb[0], g1 = t.aj * fb[1], g2 = t.aj * fb[2], g3 = t.aj * fb[3];
    double rlft_ = 0, ulft_ = 0, vlft_ = 0, plft_ = 0, rrht_ = 0, urht_ = 0, vrht_ = 0, prht_ = 0;
    double uulft_ = 0, uurht_ = 0, rulft_ = 0, rurht_ = 0, rvlft_ = 0, rvrht_ = 0, eplft_ = 0, eprht_ = 0;
    double plar_ = 0;
    rlft_ += g0 * t.uulft; uulft_ += g0 * rlft; rrht_ += g0 * t.uurht; uurht_ += g0 * rrht;
    const double d1_ = -g0;
    rulft_ += g1 * t.uulft; uulft_ += g1 * t.rulft; rurht_ += g1 * t.uurht; uurht_ += g1 * t.rurht; plar_ += g1 * r1;
    const double d2_ = -g1;
    rvlft_ += g2 * t.uulft; uulft_ += g2 * t.rvlft; rvrht_ += g2 * t.uurht; uurht_ += g2 * t.rvrht; plar_ += g2 * r2;
    const double d3_ = -g2;
    eplft_ += g3 * t.uulft; uulft_ += g3 * t.eplft; eprht_ += g3 * t.uurht; uurht_ += g3 * t.eprht;
    const double d4_ = -g3;
    double elft_ = eplft_, erht_ = eprht_;
    plft_ += eplft_ + plar_;
    prht_ += eprht_ + plar_;
    double hav_ = d4_ * t.b4, b4_ = d4_ * t.hav, uu_ = d4_ * t.b5, b5_ = d4_ * t.uu, uav_ = d4_ * t.b6, b6_ = d4_ * t.uav;
    double vav_ = d4_ * t.b7, b7_ = d4_ * t.vav, c2_ = -d4_ * t.b1 * OGM1, b1_ = -d4_ * t.c2 * OGM1;
    vav_ += d3_ * t.b4; b4_ += d3_ * t.vav; b5_ += d3_ * r2; b7_ += d3_;
    uav_ += d2_ * t.b4; b4_ += d2_ * t.uav; b5_ += d2_ * r1; b6_ += d2_;
    b4_ += d1_;
    double ruuav_ = b7_ * (t.aq3 - r2 * t.aquu) + b6_ * (t.aq2 - r1 * t.aquu);
    double aq3_ = b7_ * t.ruuav, aq2_ = b6_ * t.ruuav;
    double aquu_ = -b7_ * t.ruuav * r2 - b6_ * t.ruuav * r1;
    double cav_ = b5_ * (t.b2 - t.b3);
    double b2_ = b5_ * t.cav, b3_ = -b5_ * t.cav;
    b1_ += b4_; b2_ += b4_; b3_ += b4_;
    double c2ih_ = b3_ * t.aumc * t.t3 + b2_ * t.aupc * t.t2;
    double aumc_ = b3_ * t.c2ih * t.t3, aupc_ = b2_ * t.c2ih * t.t2;
    double aq4_ = b3_ * t.c2ih * t.aumc + b2_ * t.c2ih * t.aupc;
    double rcav_ = (b2_ * t.aupc - b3_ * t.aumc) * t.c2ih * t.aquu;
    aquu_ += (b2_ * t.aupc - b3_ * t.aumc) * t.c2ih * t.rcav;
    double auu_ = b1_ * (t.aq1 - t.c2i * t.aq4);
    double aq1_ = b1_ * t.auu;
    double c2i_ = -b1_ * t.auu * t.aq4;
    aq4_ += -b1_ * t.auu * t.c2i;
    auu_ += ruuav_ * t.rav;
    double rav_ = ruuav_ * t.auu;
    c2i_ += 0.5 * c2ih_;
    uurht_ += aquu_; uulft_ -= aquu_;
    rav_ += rcav_ * t.cav; cav_ += rcav_ * t.rav;
    urht_ += uurht_ * r1; vrht_ += uurht_ * r2; ulft_ += uulft_ * r1; vlft_ += uulft_ * r2;
    const double sm = sgn(t.uu - t.cav), sp = sgn(t.uu + t.cav), s0 = sgn(t.uu);
    uu_ += aumc_ * sm; cav_ -= aumc_ * sm;
    uu_ += aupc_ * sp; cav_ += aupc_ * sp;
    uu_ += auu_ * s0;
    c2_ += -c2i_ * t.c2i * t.c2i;
    cav_ += 2.0 * t.cav * c2_;
    uav_ += uu_ * r1; vav_ += uu_ * r2;
    rrht_ += aq1_; rlft_ -= aq1_; urht_ += aq2_; ulft_ -= aq2_; vrht_ += aq3_; vlft_ -= aq3_; prht_ += aq4_; plft_ -= aq4_;
    {
        const double tmp = cav_ * GM1 * 0.5 * t.icav;
        hav_ += tmp;
        uav_ -= tmp * t.uav; vav_ -= tmp * t.vav;
    }
    // x_av = (rat x_rht + x_lft) rati with rati = 1 / (rat + 1): d x_av / d rat = rati (x_rht - x_av)
    const double w = t.rat * t.rati;
    double hrht_ = hav_ * w, hlft_ = hav_ * t.rati;
    vrht_ += vav_ * w; vlft_ += vav_ * t.rati;
    urht_ += uav_ * w; ulft_ += uav_ * t.rati;
    const double rat_ = t.rati * (hav_ * (t.hrht - t.hav) + vav_ * (vrht - t.vav) + uav_ * (urht - t.uav)) + rav_ * rlft;
    rlft_ += rav_ * t.rat;
    double rlfti_ = 0, rrhti_ = 0;
    {
        const double tmp = rat_ * 0.5 * t.irat;
        rrht_ += tmp * t.rlfti; rlfti_ += tmp * rrht;
    }
    erht_ += hrht_ * t.rrhti; prht_ += hrht_ * t.rrhti; rrhti_ += hrht_ * (t.erht + t.prht);
    prht_ += erht_ * OGM1; rrht_ += erht_ * t.uvr;
    {
        const double uvr_ = erht_ * rrht;
        urht_ += uvr_ * urht; vrht_ += uvr_ * vrht;
    }
    rrht_ += rvrht_ * vrht + rurht_ * urht; vrht_ += rvrht_ * rrht; urht_ += rurht_ * rrht;
    rrht_ += -rrhti_ * t.rrhti * t.rrhti;
    elft_ += hlft_ * t.rlfti; plft_ += hlft_ * t.rlfti; rlfti_ += hlft_ * (t.elft + t.plft);
    plft_ += elft_ * OGM1; rlft_ += elft_ * t.uvl;
    {
        const double uvl_ = elft_ * rlft;
        ulft_ += uvl_ * ulft; vlft_ += uvl_ * vlft;
    }
    rlft_ += rvlft_ * vlft + rulft_ * ulft; vlft_ += rvlft_ * rlft; ulft_ += rulft_ * rlft;
    rlft_ += -rlfti_ * t.rlfti * t.rlfti;
    bl[0] += rlft_; bl[1] += ulft_; bl[2] += vlft_; bl[3] += plft_;
    br[0] += rrht_; br[1] += urht_; br[2] += vrht_; br[3] += prht_;
}

// AUSM flux forward with the intermediates the reverse sweep needs (same
// arithmetic as ausm_flux, src/model/flux.cpp:148-224): nx, ny the face normal
// scaled by its length ds.
struct AusmTape {
    double rl, ul, vl, pl, rr, ur, vr, pr, nx, ny, ds;
    double ids, al, ar, ial, iar, ml, mr, mhalf, phalf, ri, uv, h, m;
    bool left;
    double f[4];
};

__device__ inline double ausm_mach_d(double M, double s) {  // d ausm_mach / dM
    return ::fabs(M) <= 1.0 ? 0.5 * s * (M + s) : 0.5 * (1.0 + s * sgn(M));
}

__device__ inline void ausm_fwd(AusmTape& t) {
    t.ids = 1.0 / t.ds;
    t.al = ::sqrt(GAMMA * t.pl * (1.0 / t.rl));
    t.ar = ::sqrt(GAMMA * t.pr * (1.0 / t.rr));
    t.ial = 1.0 / t.al;
    t.iar = 1.0 / t.ar;
    t.ml = (t.ul * t.nx + t.vl * t.ny) * t.ids * t.ial;
    t.mr = (t.ur * t.nx + t.vr * t.ny) * t.ids * t.iar;
    t.mhalf = ausm_mach(t.ml, 1.0) + ausm_mach(t.mr, -1.0);
    t.phalf = ausm_pres(t.ml, t.pl, 1.0) + ausm_pres(t.mr, t.pr, -1.0);
    t.left = t.mhalf >= 0.0;
    const double r = t.left ? t.rl : t.rr, a = t.left ? t.al : t.ar, u = t.left ? t.ul : t.ur;
    const double v = t.left ? t.vl : t.vr, p = t.left ? t.pl : t.pr;
    t.ri = 1.0 / r;
    t.uv = 0.5 * (u * u + v * v);
    t.h = (p * OGM1 + r * t.uv + p) * t.ri;
    t.m = r * a * t.mhalf * t.ds;
    t.f[0] = t.m;
    t.f[1] = t.m * u + t.phalf * t.nx;
    t.f[2] = t.m * v + t.phalf * t.ny;
    t.f[3] = t.m * t.h;
}

// d ausm_pres / dp and / dM on one side (s = +1 left, -1 right); above |M| = 1
// the pressure split is p (1 + s sgn M) / 2, independent of M
__device__ inline void ausm_pres_d(double M, double p, double s, double* dp, double* dM) {
    if (::fabs(M) <= 1.0) {
        const double a = M + s, b = 2.0 - s * M;
        *dp = 0.25 * a * a * b;
        *dM = 0.25 * p * (2.0 * a * b - s * a * a);
    } else {
        *dp = 0.5 * (M + s * ::fabs(M)) / M;
        *dM = 0.0;
    }
}

// Reverse sweep of ausm_fwd: fb[0..3] = adjoint of f; accumulates the adjoints
// of the eight face states into bl[0..3], br[0..3].
__device__ inline void ausm_rev(const AusmTape& t, const double* fb, double* bl, double* br) {
    const double u = t.left ? t.ul : t.ur, v = t.left ? t.vl : t.vr, p = t.left ? t.pl : t.pr;
    const double r = t.left ? t.rl : t.rr, a = t.left ? t.al : t.ar;
    double m_ = fb[0] + fb[1] * u + fb[2] * v + fb[3] * t.h;
    double u_ = fb[1] * t.m, v_ = fb[2] * t.m;
    const double h_ = fb[3] * t.m;
    const double phalf_ = fb[1] * t.nx + fb[2] * t.ny;
    // h = (p / (gamma - 1) + r uv + p) / r
    const double nh_ = h_ * t.ri;
    double r_ = nh_ * t.uv - h_ * t.h * t.ri;
    double p_ = nh_ * (OGM1 + 1.0);
    const double uv_ = nh_ * r;
    u_ += uv_ * u;
    v_ += uv_ * v;
    // m = r a mhalf ds
    r_ += m_ * a * t.mhalf * t.ds;
    double a_ = m_ * r * t.mhalf * t.ds;
    const double mhalf_ = m_ * r * a * t.ds;
    double ml_ = mhalf_ * ausm_mach_d(t.ml, 1.0), mr_ = mhalf_ * ausm_mach_d(t.mr, -1.0);
    double dpl, dml, dpr, dmr;
    ausm_pres_d(t.ml, t.pl, 1.0, &dpl, &dml);
    ausm_pres_d(t.mr, t.pr, -1.0, &dpr, &dmr);
    ml_ += phalf_ * dml;
    mr_ += phalf_ * dmr;
    double al_ = 0.0, ar_ = 0.0;
    if (t.left) { bl[0] += r_; bl[1] += u_; bl[2] += v_; bl[3] += p_; al_ += a_; }
    else { br[0] += r_; br[1] += u_; br[2] += v_; br[3] += p_; ar_ += a_; }
    bl[3] += phalf_ * dpl;
    br[3] += phalf_ * dpr;
    // ml = (ul nx + vl ny) / (ds al)
    const double cl = ml_ * t.ids * t.ial, cr = mr_ * t.ids * t.iar;
    bl[1] += cl * t.nx; bl[2] += cl * t.ny; al_ -= ml_ * t.ml * t.ial;
    br[1] += cr * t.nx; br[2] += cr * t.ny; ar_ -= mr_ * t.mr * t.iar;
    // a = sqrt(gamma p / r): da/dp = a / (2p), da/dr = -a / (2r)
    bl[3] += al_ * t.al * 0.5 / t.pl; bl[0] -= al_ * t.al * 0.5 / t.rl;
    br[3] += ar_ * t.ar * 0.5 / t.pr; br[0] -= ar_ * t.ar * 0.5 / t.rr;
}

// Reverse of sa_source (same forward formulas); outputs adjoints of rho, nut,
// mu, omega, |grad nut|^2 and beta for source adjoint sb.  Each quotient's
// reciprocal is formed once (Newton-Raphson, st_common.cuh) and shared by the
// forward and reverse sweeps; fw's sixth root is (g^6 + cw3^6)^(-1/6) = q, so
// d fw / d g^6 needs q^6 = 1 / (g^6 + cw3^6) and no further division.
__device__ inline double sa_source_adj(double rho, double nut, double mu, double d, double omega, double gnut2,
                                       double beta, double sb, double* rho_, double* nut_, double* mu_,
                                       double* omega_, double* gnut2_, double* beta_) {
    const double id2 = nr_rcp(d * d);
    if (nut < 0.0) {  // SA-neg branch of sa_source
        const double cp = SA_CB1 * (1.0 - SA_CT3);
        const double src = beta * cp * omega * nut + SA_CW1 * nut * nut * id2;
        *rho_ = sb * (src + (SA_CB2 / SA_SIGMA) * gnut2);
        *nut_ = sb * rho * (beta * cp * omega + 2.0 * SA_CW1 * nut * id2);
        *mu_ = 0.0;
        *omega_ = sb * rho * beta * cp * nut;
        *gnut2_ = sb * rho * (SA_CB2 / SA_SIGMA);
        *beta_ = sb * rho * cp * omega * nut;
        return rho * src + (SA_CB2 / SA_SIGMA) * rho * gnut2;
    }
    const double ik2d2 = id2 * (1.0 / (SA_KAPPA * SA_KAPPA));
    const double imu = nr_rcp(mu);
    const double chi = rho * nut * imu;
    const double chi3 = chi * chi * chi;
    const double iden = nr_rcp(chi3 + SA_CV1_3);
    const double fv1 = chi3 * iden;
    const double iE = nr_rcp(1.0 + chi * fv1);
    const double fv2 = 1.0 - chi * iE;
    const double sbar = nut * fv2 * ik2d2;
    const bool br1 = sbar >= -SA_CV2 * omega;
    double stilde, N = 0.0, iD = 1.0;
    if (br1) {
        stilde = omega + sbar;
    } else {
        N = SA_CV2 * SA_CV2 * omega + SA_CV3 * sbar;
        iD = nr_rcp((SA_CV3 - 2.0 * SA_CV2) * omega - sbar);
        stilde = omega + omega * N * iD;
    }
    double r, ist = 0.0;
    bool rfree = false;
    if (stilde > 0.0) {
        ist = nr_rcp(stilde);
        r = nut * ist * ik2d2;
        if (r < 10.0) rfree = true; else r = 10.0;
    } else {
        r = 10.0;
    }
    const double r2 = r * r;
    const double gg = r + SA_CW2 * (r2 * r2 * r2 - r);
    const double g2 = gg * gg;
    const double q = nr_inv_root6(g2 * g2 * g2 + SA_CW3_6);
    const double h = SA_C6 * q;
    const double fw = gg * h;
    const double prod = beta * SA_CB1 * stilde * nut;
    const double dest = SA_CW1 * fw * (nut * nut) * id2;
    // reverse
    double rhob = sb * (prod - dest + (SA_CB2 / SA_SIGMA) * gnut2);
    const double prod_ = sb * rho, dest_ = -sb * rho;
    *gnut2_ = sb * rho * (SA_CB2 / SA_SIGMA);
    double fw_ = dest_ * SA_CW1 * nut * nut * id2;
    double nutb = dest_ * SA_CW1 * fw * 2.0 * nut * id2;
    *beta_ = prod_ * SA_CB1 * stilde * nut;
    double stilde_ = prod_ * beta * SA_CB1 * nut;
    nutb += prod_ * beta * SA_CB1 * stilde;
    double gg_ = fw_ * h;
    const double h_ = fw_ * gg;
    // h = C6 w^(-1/6), w = g^6 + cw3^6: dh/dw = -(1/6) h / w = -(1/6) h q^6
    const double q2 = q * q;
    const double g6_ = h_ * h * (q2 * q2 * q2) * (-1.0 / 6.0);
    const double g2_ = g6_ * 3.0 * g2 * g2;
    gg_ += g2_ * 2.0 * gg;
    const double r_ = gg_ * (1.0 + SA_CW2 * (6.0 * r2 * r2 * r - 1.0));
    if (rfree) {
        nutb += r_ * ist * ik2d2;
        stilde_ += -r_ * r * ist;
    }
    double omegab = 0.0, sbar_ = 0.0;
    if (br1) {
        omegab += stilde_;
        sbar_ += stilde_;
    } else {
        omegab += stilde_ * (1.0 + N * iD);
        const double N_ = stilde_ * omega * iD;
        const double D_ = -stilde_ * omega * N * (iD * iD);
        omegab += N_ * SA_CV2 * SA_CV2 + D_ * (SA_CV3 - 2.0 * SA_CV2);
        sbar_ += N_ * SA_CV3 - D_;
    }
    nutb += sbar_ * fv2 * ik2d2;
    const double fv2_ = sbar_ * nut * ik2d2;
    const double iE2 = iE * iE;
    double chi_ = -fv2_ * iE + fv2_ * chi * fv1 * iE2;
    const double fv1_ = fv2_ * chi * chi * iE2;
    const double chi3_ = fv1_ * SA_CV1_3 * (iden * iden);
    chi_ += chi3_ * 3.0 * chi * chi;
    rhob += chi_ * nut * imu;
    nutb += chi_ * rho * imu;
    *mu_ = -chi_ * chi * imu;
    *rho_ = rhob;
    *nut_ = nutb;
    *omega_ = omegab;
    return rho * (prod - dest) + (SA_CB2 / SA_SIGMA) * rho * gnut2;
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

// R1 (SA): the cell source, forward and reverse.  rhs_4 = (... + S V) / V,
// so the source adjoint is psi_4 (V/V).  Writes the source value, the
// adjoints of the cell's own rho, nut, mu, and of the four face gradient parts
// it averages (the same for all four faces), and (dR/dbeta)^T psi.
static __global__ void __launch_bounds__(256) k_cell_src(DevCase c, const double* __restrict__ P, const double* __restrict__ Gi,
                                                  const double* __restrict__ Gj, const double* __restrict__ beta,
                                                  const double* __restrict__ psi, double* __restrict__ srec,
                                                  double* __restrict__ outb) {
    const size_t n = (size_t)c.nic * c.njc;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / c.njc), j = (int)(idx % c.njc);
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
        const double sb = psi ? psi[idx * 5 + 4] * (c.vol[idx] * c.ivol[idx]) : 0.0;
        double rho_, nut_, mu_, om_, g2_, b_;
        const double S = sa_source_adj(pc[P_RHO], pc[P_NUT], pc[P_MU], c.wd[idx], om, nx * nx + ny * ny, bt, sb, &rho_,
                                       &nut_, &mu_, &om_, &g2_, &b_);
        const double sg = sgn(vx - uy);
        double* s = srec + idx * SRW;
        s[S_GU] = 0.25 * (-om_ * sg);
        s[S_GV] = 0.25 * (om_ * sg);
        s[S_GNX] = 0.25 * (2.0 * nx * g2_);
        s[S_GNY] = 0.25 * (2.0 * ny * g2_);
        s[S_RHO] = rho_; s[S_NUT] = nut_; s[S_MU] = mu_; s[S_VAL] = S;
        if (outb) outb[idx] = b_;
    }
}

// R2: one pass per face family that computes the face flux (for the
// residual, when F != nullptr) and runs its reverse sweep in place, seeded by
// the flux adjoint w(R) - w(L), w = psi / V (0 on ghost sides), and, with SA,
// by the gradient-part adjoints of the two adjacent cells' sources.  FLUX:
// ST_FLUX_ROE or ST_FLUX_AUSM (a separate instantiation each, so the Roe pass
// carries none of the AUSM code).
template <int NQ, int DIR, int ORDER, int FLUX = ST_FLUX_ROE>
__global__ void __launch_bounds__(256, 2) k_face_fused(DevCase c, const double* __restrict__ P,
                                                    const double* __restrict__ lim, const double* __restrict__ psi,
                                                    const double* __restrict__ srec, double* __restrict__ F,
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
        double fb[5];
        {
            const double ivr = fi.limR ? c.ivol[fi.phR] : 0.0, ivl = fi.limL ? c.ivol[fi.phL] : 0.0;
#pragma unroll
            for (int k = 0; k < NQ; k++) {
                const double wr = fi.limR ? psi[fi.phR * NQ + k] * ivr : 0.0;
                const double wl = fi.limL ? psi[fi.phL * NQ + k] * ivl : 0.0;
                fb[k] = wr - wl;
            }
        }
        double qL[5], qR[5];
#pragma unroll
        for (int k = 0; k < NQ; k++) {
            qL[k] = pL[slot[k]];
            qR[k] = pR[slot[k]];
            if (ORDER == 2) {
                if (fi.limL) qL[k] += lim[lim_off(c, DIR, LIM_SL, fi.phL) + k];
                if (fi.limR) qR[k] -= lim[lim_off(c, DIR, LIM_SR, fi.phR) + k];
            }
        }
        double f[5], bl[5] = {0, 0, 0, 0, 0}, br[5] = {0, 0, 0, 0, 0};
        double fcb[4] = {fb[0], fb[1], fb[2], fb[3]};
        // SA convection: the mass flux upwinds nu_tilde
        auto sa_upwind = [&]() {
            if (NQ == 5) {
                const bool up = f[0] >= 0.0;
                const double nup = up ? qL[4] : qR[4];
                f[4] = f[0] * nup;
                fcb[0] += fb[4] * nup;
                if (up) bl[4] += fb[4] * f[0]; else br[4] += fb[4] * f[0];
            } else {
                f[4] = 0.0;
            }
        };
        if constexpr (FLUX == ST_FLUX_AUSM) {
            AusmTape at;
            at.rl = qL[0]; at.ul = qL[1]; at.vl = qL[2]; at.pl = qL[3];
            at.rr = qR[0]; at.ur = qR[1]; at.vr = qR[2]; at.pr = qR[3];
            at.nx = gm[G_NX]; at.ny = gm[G_NY]; at.ds = 2.0 * gm[G_AJ];
            ausm_fwd(at);
            for (int k = 0; k < 4; k++) f[k] = at.f[k];
            sa_upwind();
            ausm_rev(at, fcb, bl, br);
        } else {
            RoeTape rt;
            rt.rlft = qL[0]; rt.ulft = qL[1]; rt.vlft = qL[2]; rt.plft = qL[3];
            rt.rrht = qR[0]; rt.urht = qR[1]; rt.vrht = qR[2]; rt.prht = qR[3];
            rt.r1 = gm[G_R1]; rt.r2 = gm[G_R2]; rt.aj = gm[G_AJ];
            roe_fwd(rt);
            for (int k = 0; k < 4; k++) f[k] = rt.f[k];
            sa_upwind();
            roe_rev(rt, fcb, bl, br);
        }
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
                k = mub * c.cp_pr + mutb * c.cp_prt;
            } else {
                k = mub * c.cp_pr;
            }
            const double nx = gm[G_NX], ny = gm[G_NY];
            const double div = dudx + dvdy;
            const double txy = mu * (dudy + dvdx);
            const double txx = mu * (2.0 * dudx - 2.0 / 3.0 * div);
            const double tyy = mu * (2.0 * dvdy - 2.0 / 3.0 * div);
            // forward viscous flux (for the residual)
            f[1] -= txx * nx + txy * ny;
            f[2] -= txy * nx + tyy * ny;
            f[3] -= (ub * txx + vb * txy + k * dTdx) * nx + (ub * txy + vb * tyy + k * dTdy) * ny;
            // reverse; F_net = F_conv - F_visc
            const double v1 = -fb[1], v2 = -fb[2], v3 = -fb[3];
            const double A_ = v3 * nx, B_ = v3 * ny;
            const double ub_ = A_ * txx + B_ * txy;
            const double vb_ = A_ * txy + B_ * tyy;
            const double txx_ = A_ * ub + v1 * nx;
            const double txy_ = A_ * vb + B_ * ub + v2 * nx + v1 * ny;
            const double tyy_ = B_ * vb + v2 * ny;
            const double k_ = A_ * dTdx + B_ * dTdy;
            const double dTdx_ = A_ * k, dTdy_ = B_ * k;
            const double mu_ = tyy_ * (2.0 * dvdy - 2.0 / 3.0 * div) + txx_ * (2.0 * dudx - 2.0 / 3.0 * div)
                             + txy_ * (dudy + dvdx);
            double dvdy_ = tyy_ * mu * 2.0, dudx_ = txx_ * mu * 2.0;
            const double div_ = -(tyy_ + txx_) * mu * (2.0 / 3.0);
            double dudy_ = txy_ * mu, dvdx_ = txy_ * mu;
            dudx_ += div_; dvdy_ += div_;
            double mub_ = mu_, mutb_ = 0.0;
            if (NQ == 5) { mutb_ = mu_ + k_ * c.cp_prt; mub_ += k_ * c.cp_pr; }
            else mub_ += k_ * c.cp_pr;
            o[A_DTDX] = dTdx_; o[A_DTDY] = dTdy_;
            o[A_UB] = ub_; o[A_VB] = vb_;
            if (NQ == 5) {
                double dndx, dndy, nb_;
                ST_GRAD_D(P_NUT, dndx, dndy, nb_)
                (void)nb_;
#define ST_SD(p) sa_diff(p[P_RHO], p[P_NUT], p[P_MU])
                const double rnb = 0.375 * (ST_SD(pL) + ST_SD(pR)) + 0.0625 * (ST_SD(pPa) + ST_SD(pPb) + ST_SD(pMa) + ST_SD(pMb));
#undef ST_SD
                const double cs = 1.0 / SA_SIGMA;
                const double gdn = dndx * nx + dndy * ny;
                f[4] -= cs * (mub + rnb) * gdn;
                const double v4 = -fb[4];
                mub_ += v4 * cs * gdn;
                const double rnb_ = v4 * cs * gdn;
                double dndx_ = v4 * cs * (mub + rnb) * nx, dndy_ = v4 * cs * (mub + rnb) * ny;
                double gs[4] = {0, 0, 0, 0};
                if (fi.limL) { const double* sl = srec + fi.phL * SRW; for (int t = 0; t < 4; t++) gs[t] += sl[t]; }
                if (fi.limR) { const double* sr = srec + fi.phR * SRW; for (int t = 0; t < 4; t++) gs[t] += sr[t]; }
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
        // reconstruction reverse: direct terms and the slopes' d-, d+ parts
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const bool kk = k < NQ;
            const double A = kk ? bl[k] : 0.0, B = kk ? br[k] : 0.0;
            o[A_AL + k] = A;
            o[A_BR + k] = B;
            double dml = 0.0, dpl = 0.0, dmr = 0.0, dpr = 0.0;
            if (ORDER == 2 && kk) {
                if (fi.limL) {
                    dml = A * lim[lim_off(c, DIR, LIM_AM, fi.phL) + k];
                    dpl = A * lim[lim_off(c, DIR, LIM_AP, fi.phL) + k];
                }
                if (fi.limR) {
                    dmr = -B * lim[lim_off(c, DIR, LIM_BM, fi.phR) + k];
                    dpr = -B * lim[lim_off(c, DIR, LIM_BP, fi.phR) + k];
                }
            }
            o[A_DML + k] = dml; o[A_DPL + k] = dpl; o[A_DMR + k] = dmr; o[A_DPR + k] = dpr;
        }
        if (F) {
            double* fo = F + fi.face * NQ;
#pragma unroll
            for (int k = 0; k < NQ; k++) fo[k] = f[k];
        }
    }
}

// Residual assembly from precomputed face fluxes and (SA) source values.
template <int NQ>
__global__ void __launch_bounds__(256) k_cell_res(DevCase c, const double* __restrict__ Fi, const double* __restrict__ Fj,
                                                  const double* __restrict__ srec, double* __restrict__ rhs) {
    const size_t n = (size_t)c.nic * c.njc;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / c.njc), j = (int)(idx % c.njc);
        const double* fs = Fj + ((size_t)i * c.nj + j) * NQ;
        const double* fn = fs + NQ;
        const double* fw = Fi + ((size_t)i * c.njc + j) * NQ;
        const double* fe = Fi + ((size_t)(i + 1) * c.njc + j) * NQ;
        double r[NQ];
#pragma unroll
        for (int k = 0; k < NQ; k++) r[k] = (fs[k] - fn[k]) + (fw[k] - fe[k]);
        const double vol = c.vol[idx];
        if (NQ == 5 && c.viscous) r[NQ - 1] += srec[idx * SRW + S_VAL] * vol;
        r[1] += -c.dpdx * vol;
        r[2] += -c.dpdy * vol;
        const double iv = c.ivol[idx];
#pragma unroll
        for (int k = 0; k < NQ; k++) rhs[idx * NQ + k] = r[k] * iv;
    }
}

// R3: gather the adjoint of every ghost-padded primitive record from the
// faces whose stencils contain it: the two faces it is a side of (direct and
// slope parts), the faces of its two neighbours along each direction (their
// slopes depend on this cell), and the six viscous stencils per direction.
template <int NQ, int ORDER>
__global__ void __launch_bounds__(256) k_gather(DevCase c, const double* __restrict__ P, const double* __restrict__ ai,
                                                const double* __restrict__ aj, const double* __restrict__ srec,
                                                double* __restrict__ Pbar, size_t first, size_t n) {
    const int slot[5] = {P_RHO, P_U, P_V, P_P, P_NUT};
    for (size_t idx = first + (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int ip = (int)(idx / (c.njc + 2)), jp = (int)(idx % (c.njc + 2));
        double acc[NP];
#pragma unroll
        for (int s = 0; s < NP; s++) acc[s] = 0.0;
        const double* self = P + idx * NP;
        double sd_r = 0.0, sd_n = 0.0, sd_m = 0.0;  // d (rho nut f_n) / d (rho, nut, mu) of this record
        if (NQ == 5 && c.viscous) sa_diff_d(self[P_RHO], self[P_NUT], self[P_MU], &sd_r, &sd_n, &sd_m);
        double rnb_acc = 0.0;  // sum over the viscous stencils of the face-average adjoint of rho nut f_n
        auto visc = [&](const double* r, const double* gm, int role) {
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
                acc[P_NUT] += r[A_DNDX] * wx + r[A_DNDY] * wy;
                rnb_acc += r[A_RNB] * co;  // times this record's d(rho nut f_n) at the end
            }
        };
        // ---- i-faces (f, j): L=(f, j+1) R=(f+1, j+1) P=(f|f+1, j+2) M=(f|f+1, j)
        {
            auto rec = [&](int f, int j) -> const double* {
                return (f < 0 || f > c.nic || j < 0 || j >= c.njc) ? nullptr : ai + ((size_t)f * c.njc + j) * ARW;
            };
            if (jp >= 1 && jp <= c.njc) {
                const int j = jp - 1;
                const double* f0 = rec(ip, j);       // this cell is its L
                const double* f1 = rec(ip - 1, j);   // this cell is its R
                for (int k = 0; k < NQ; k++) {
                    double s = 0.0;
                    if (f0) s += f0[A_AL + k];
                    if (f1) s += f1[A_BR + k];
                    if (ORDER == 2) {
                        const double* fm2 = rec(ip - 2, j);
                        const double* fp1 = rec(ip + 1, j);
                        if (f0) s += f0[A_DML + k] - f0[A_DPL + k] - f0[A_DMR + k];
                        if (f1) s += f1[A_DMR + k] - f1[A_DPR + k] + f1[A_DPL + k];
                        if (fm2) s += fm2[A_DPR + k];
                        if (fp1) s -= fp1[A_DML + k];
                    }
                    acc[slot[k]] += s;
                }
            }
            if (c.viscous) {
                const int fs[6] = {ip, ip - 1, ip, ip - 1, ip, ip - 1};
                const int js[6] = {jp - 1, jp - 1, jp - 2, jp - 2, jp, jp};
                const int roles[6] = {0, 1, 2, 2, 3, 3};
#pragma unroll
                for (int t = 0; t < 6; t++) {
                    const double* r = rec(fs[t], js[t]);
                    if (r) visc(r, c.geo_i + ((size_t)fs[t] * c.njc + js[t]) * NGEO, roles[t]);
                }
            }
        }
        // ---- j-faces (i, g): L=(i+1, g) R=(i+1, g+1) P=(i+2, g|g+1) M=(i, g|g+1)
        {
            auto rec = [&](int i, int g) -> const double* {
                return (i < 0 || i >= c.nic || g < 0 || g > c.njc) ? nullptr : aj + ((size_t)i * c.nj + g) * ARW;
            };
            if (ip >= 1 && ip <= c.nic) {
                const int i = ip - 1;
                const double* f0 = rec(i, jp);
                const double* f1 = rec(i, jp - 1);
                for (int k = 0; k < NQ; k++) {
                    double s = 0.0;
                    if (f0) s += f0[A_AL + k];
                    if (f1) s += f1[A_BR + k];
                    if (ORDER == 2) {
                        const double* fm2 = rec(i, jp - 2);
                        const double* fp1 = rec(i, jp + 1);
                        if (f0) s += f0[A_DML + k] - f0[A_DPL + k] - f0[A_DMR + k];
                        if (f1) s += f1[A_DMR + k] - f1[A_DPR + k] + f1[A_DPL + k];
                        if (fm2) s += fm2[A_DPR + k];
                        if (fp1) s -= fp1[A_DML + k];
                    }
                    acc[slot[k]] += s;
                }
            }
            if (c.viscous) {
                const int is[6] = {ip - 1, ip - 1, ip - 2, ip - 2, ip, ip};
                const int gs[6] = {jp, jp - 1, jp, jp - 1, jp, jp - 1};
                const int roles[6] = {0, 1, 2, 2, 3, 3};
#pragma unroll
                for (int t = 0; t < 6; t++) {
                    const double* r = rec(is[t], gs[t]);
                    if (r) visc(r, c.geo_j + ((size_t)is[t] * c.nj + gs[t]) * NGEO, roles[t]);
                }
            }
        }
        if (NQ == 5 && c.viscous) {
            acc[P_NUT] += rnb_acc * sd_n;
            acc[P_RHO] += rnb_acc * sd_r;
            acc[P_MU] += rnb_acc * sd_m;
        }
        const bool phys = ip >= 1 && ip <= c.nic && jp >= 1 && jp <= c.njc;
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
    if (c.viscous) bc_ghost_mu<double, NQ>(c, P, threadIdx.x, blockDim.x);
}

// R5: reverse of the boundary pass.  First the ghost mu, mu_t (bc_adj_mu),
// then each BC in reverse order (bc_adj_one): the ghost adjoint flows to the
// BC's inputs (read from the tape where they are ghosts themselves) and is
// cleared.  A wake cut is reversed in two parts, its second ghost half first.
// Threads tid = 0 .. nth-1 of a block or of a launch.
template <int NQ>
__device__ void bc_adj_mu(const DevCase& c, const double* __restrict__ P, double* __restrict__ Pbar, int tid, int nth) {
    const int nic = c.nic, njc = c.njc;
    const int nr = ring_size(c);
    {
        for (int r = tid; r < nr; r += nth) {
            int ip, jp;
            if (r < nic + 2) { ip = r; jp = 0; }
            else if (r < 2 * (nic + 2)) { ip = r - (nic + 2); jp = njc + 1; }
            else if (r < 2 * (nic + 2) + njc) { ip = 0; jp = r - 2 * (nic + 2) + 1; }
            else { ip = nic + 1; jp = r - 2 * (nic + 2) - njc + 1; }
            const double* g = P + pidx(c, ip, jp);
            double* gb = Pbar + pidx(c, ip, jp);
            double mub = gb[P_MU];
            const double T = g[P_T], mu = g[P_MU];
            if (NQ == 5 && mu != 0.0 && g[P_NUT] >= 0.0) {  // mu_t = 0 for nut < 0
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
    }
}

template <int NQ>
__device__ void bc_adj_one(const DevCase& c, const double* __restrict__ P, const double* __restrict__ tape,
                           double* __restrict__ Pbar, int b, int part, int tid, int nth) {
    const int nic = c.nic, njc = c.njc;
    const int nr = ring_size(c);
    const double iR = c.iR;
    // input value: ghost inputs from the tape before BC b, interior from P
    auto in = [&](int b, int ip, int jp, int s) -> double {
        if (on_ring(c, ip, jp)) return tape[((size_t)b * nr + ring_index(c, ip, jp)) * RW + s];
        return P[pidx(c, ip, jp) + s];
    };
    {
        const DevBC bc = c.bcs[b];
        const bool bt = (bc.face == 0 || bc.face == 2);
        const int end = bc.end >= 0 ? bc.end : (bt ? nic : njc) + 2 + bc.end;
        const int start = bc.start;
        if (part == 1 && bc.type != 6) return;
        if (bc.type == 0) {
            for (int s = start + tid; s <= end; s += nth) {
                int ip = bt ? s : (bc.face == 3 ? 0 : nic + 1);
                int jp = bt ? (bc.face == 0 ? 0 : njc + 1) : s;
                double* gb = Pbar + pidx(c, ip, jp);
                for (int t = 0; t < RW; t++) gb[t] = 0.0;
            }
        } else if (bc.type == 1 && bt) {
            for (int ip = start + tid; ip <= end; ip += nth) {
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
            for (int s = start + tid; s <= end; s += nth) {
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
            for (int jp = start + tid; jp <= end; jp += nth) {
                double* gb = Pbar + pidx(c, nic + 1, jp);
                double* ab = Pbar + pidx(c, nic, jp);
                const double rg = in(b, nic, jp, P_RHO);
                ab[P_RHO] += gb[P_RHO] - gb[P_T] * c.p_inf * iR / (rg * rg);
                ab[P_U] += gb[P_U]; ab[P_V] += gb[P_V]; ab[P_NUT] += gb[P_NUT];
                for (int t = 0; t < RW; t++) gb[t] = 0.0;
            }
        } else if (bc.type == 4) {
            for (int s = start + tid; s <= end; s += nth) {
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
            if (part == 0)
                for (int ip = start + tid; ip <= end; ip += nth) {
                    double* gb = Pbar + pidx(c, nic + 1 - ip, jg);
                    double* sb = Pbar + pidx(c, ip, 1);
                    for (int t = 0; t < RW; t++) { sb[t] += gb[t]; gb[t] = 0.0; }
                }
            else
                for (int ip = start + tid; ip <= end; ip += nth) {
                    double* gb = Pbar + pidx(c, ip, jg);
                    double* sb = Pbar + pidx(c, nic + 1 - ip, 1);
                    for (int t = 0; t < RW; t++) { sb[t] += gb[t]; gb[t] = 0.0; }
                }
        }
    }
}

template <int NQ>
__global__ void __launch_bounds__(1024) k_bc_adj(DevCase c, const double* __restrict__ P, const double* __restrict__ tape,
                                                 double* __restrict__ Pbar) {
    if (c.viscous) {
        bc_adj_mu<NQ>(c, P, Pbar, threadIdx.x, blockDim.x);
        __syncthreads();
    }
    for (int b = c.nbc - 1; b >= 0; b--)
        for (int part = 0; part < 2; part++) {
            bc_adj_one<NQ>(c, P, tape, Pbar, b, part, threadIdx.x, blockDim.x);
            __syncthreads();
        }
}

// Grid-wide launches of the same passes (one per BC and part, issued in order
// by the host), and of the taped forward pass: the ring is recorded before
// BC b by k_tape_ring, then BC b is applied by k_bc_one.
template <int NQ>
__global__ void __launch_bounds__(256) k_bc_adj_mu(DevCase c, const double* __restrict__ P, double* __restrict__ Pbar) {
    bc_adj_mu<NQ>(c, P, Pbar, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}
template <int NQ>
__global__ void __launch_bounds__(256) k_bc_adj_one(DevCase c, const double* __restrict__ P,
                                                     const double* __restrict__ tape, double* __restrict__ Pbar, int b,
                                                     int part) {
    bc_adj_one<NQ>(c, P, tape, Pbar, b, part, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}
static __global__ void __launch_bounds__(256) k_tape_ring(DevCase c, const double* __restrict__ P, double* __restrict__ tape,
                                                   int b) {
    const int nr = ring_size(c);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nr; r += gridDim.x * blockDim.x) {
        int ip, jp;
        if (r < c.nic + 2) { ip = r; jp = 0; }
        else if (r < 2 * (c.nic + 2)) { ip = r - (c.nic + 2); jp = c.njc + 1; }
        else if (r < 2 * (c.nic + 2) + c.njc) { ip = 0; jp = r - 2 * (c.nic + 2) + 1; }
        else { ip = c.nic + 1; jp = r - 2 * (c.nic + 2) - c.njc + 1; }
        const double* g = P + pidx(c, ip, jp);
        double* t = tape + ((size_t)b * nr + r) * RW;
        for (int k = 0; k < RW; k++) t[k] = g[k];
    }
}

// R6: primitives -> conserved adjoint per physical cell (reverse of k_prim).
template <int NQ>
__device__ inline void prim_adj_cell(const DevCase& c, const double* __restrict__ q, const double* __restrict__ P,
                                     const double* __restrict__ Pbar, double* __restrict__ Qb_out, size_t idx) {
    const int i = (int)(idx / c.njc), j = (int)(idx % c.njc);
    const double* Q = q + idx * NQ;
    const double* p = P + pidx(c, i + 1, j + 1);
    const double* b = Pbar + pidx(c, i + 1, j + 1);
    const double rho = Q[0], ri = nr_rcp(rho), u = p[P_U], v = p[P_V];
    double rhob = b[P_RHO], ub = b[P_U], vb = b[P_V], pb = b[P_P], Tb = b[P_T], nutb = b[P_NUT], mub = b[P_MU];
    if (c.viscous) {
        const double mu = p[P_MU];
        if (NQ == 5 && p[P_NUT] >= 0.0) {  // mu_t = 0 for nut < 0
            const double s = rho * p[P_NUT];
            const double chi = s * nr_rcp(mu), chi3 = chi * chi * chi, iden = nr_rcp(chi3 + SA_CV1_3);
            const double f = chi3 * iden, fp = 3.0 * chi * chi * SA_CV1_3 * (iden * iden);
            const double ds = f + chi * fp;
            rhob += b[P_MUT] * ds * p[P_NUT];
            nutb += b[P_MUT] * ds * rho;
            mub += b[P_MUT] * (-chi * chi * fp);
        }
        const double iT = nr_rcp(p[P_T]);
        const double dmu = c.law == 1 ? mu * (1.5 * iT - nr_rcp(p[P_T] + c.suth_S)) : (2.0 / 3.0) * mu * iT;
        Tb += mub * dmu;
    }
    const double iR = c.iR;
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
    for (int k = 0; k < NQ; k++) Qb_out[k] = Qb[k];
}

// Boundary ring of the physical cells: the two outermost rows and columns,
// whose primitive adjoints the boundary reverse still changes after the
// gather.  Ring index r: rows 0, 1 (r < 2 njc), rows nic-2, nic-1 (< 4 njc),
// then columns 0, 1, njc-2, njc-1 of rows 2 .. nic-3.  Needs nic, njc >= 4.
__host__ __device__ inline size_t ring_cells(int nic, int njc) { return 4 * (size_t)njc + 4 * (size_t)(nic - 4); }
__host__ __device__ inline size_t ring_cell(int nic, int njc, size_t r) {
    if (r < 2 * (size_t)njc) return r;
    if (r < 4 * (size_t)njc) return (size_t)(nic - 2) * njc + (r - 2 * (size_t)njc);
    const size_t rr = r - 4 * (size_t)njc;
    const int i = 2 + (int)(rr / 4), k = (int)(rr % 4);
    const int j = k < 2 ? k : njc - 4 + k;
    return (size_t)i * njc + j;
}
__host__ __device__ inline bool in_ring(int nic, int njc, size_t idx) {
    const int i = (int)(idx / njc), j = (int)(idx % njc);
    return i < 2 || i >= nic - 2 || j < 2 || j >= njc - 2;
}

// The pass over the cells [first, n); skip_ring leaves the boundary ring out
// (the host-buffer call runs it after the boundary reverse).
template <int NQ>
__global__ void __launch_bounds__(256) k_prim_adj(DevCase c, const double* __restrict__ q, const double* __restrict__ P,
                                                  const double* __restrict__ Pbar, double* __restrict__ out,
                                                  size_t first, size_t n, bool skip_ring = false) {
    for (size_t idx = first + (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        if (skip_ring && in_ring(c.nic, c.njc, idx)) continue;
        prim_adj_cell<NQ>(c, q, P, Pbar, out + idx * NQ, idx);
    }
}

// The boundary ring's pass: writes out and, packed by ring index, pack.
template <int NQ>
__global__ void __launch_bounds__(256) k_prim_adj_ring(DevCase c, const double* __restrict__ q,
                                                       const double* __restrict__ P, const double* __restrict__ Pbar,
                                                       double* __restrict__ out, double* __restrict__ pack) {
    const size_t nr = ring_cells(c.nic, c.njc);
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < nr; r += (size_t)gridDim.x * blockDim.x) {
        const size_t idx = ring_cell(c.nic, c.njc, r);
        double v[NQ];
        prim_adj_cell<NQ>(c, q, P, Pbar, v, idx);
#pragma unroll
        for (int k = 0; k < NQ; k++) {
            out[idx * NQ + k] = v[k];
            pack[r * NQ + k] = v[k];
        }
    }
}

}  // namespace st
