// Reverse-mode arithmetic of the volume-element SPH chain
//   xmass -> kx/gradh -> EOS -> IAD + divv/curlv/dV -> AV switches -> momentum-energy<avClean>
// one pair or one particle at a time, in FP64.  Pure functions of plain values (no table, list or
// memory access), shared by the device kernels and by host-side checks.
//
// Conventions: pair (i, j) of i's list, r = x_i - x_j with the legacy periodic fold at 2 h_i,
// d = |r|, v = v_i - v_j, v1 = d / h_i, v2 = d / h_j.  w(v) and dw are the table interpolant and
// its slope on the interval holding v (so forward and reverse describe one piecewise function).
// "b" suffixes are adjoints dL/d(quantity).  C and g (the symmetric velocity gradient of the
// avClean correction) are 6 stored components {11 12 13 22 23 33}; their adjoints are with respect
// to those components.
//
// Forward formulas (reference j-loops):
//   xm_i    = m_i h_i^3 / (K (m_i + sum_j m_j w(v1)))                       hydro_ve/xmass_kern.hpp:50-79
//   kx_i    = K h^-3 (xm_i + sum_j xm_j w),  gradh_i = 1 + h_i whomega_i / (3 rho_i)
//   whomega = K h^-4 [S_om m_i/xm_i + (kx h^4/K - xm_i h) S_r0],  dterh = -(3 w + v1 wd(v1))
//             S_om = -3 xm_i + sum_j xm_j dterh,  S_r0 = -3 m_i + sum_j m_j dterh
//                                                                          hydro_ve/ve_def_gradh_kern.hpp:43-90
//   rho = kx m / xm, p = (gamma-1) rho u, c = sqrt(gamma (gamma-1) u), prho = p / (kx m^2 gradh)
//                                                                          hydro_ve/eos.hpp:52-94
//   C_i = tau_i^-1 h^3 / K, tau_i = sum_j (xm_j/kx_j) w r r^T                hydro_ve/iad_kern.hpp:43-109
//   dV_i = -K h^-3 / kx_i  P_i C_i, P_i = sum_j xm_j w (v_j - v_i) r^T: divv = tr dV,
//   g = {dV11, dV12+dV21, dV13+dV31, dV22, dV23+dV32, dV33}             hydro_ve/divv_curlv_kern.hpp:43-123
//   alpha_i from divv_i, |G_i|, G_i = sum_j (xm_j/kx_j)(divv_i - divv_j)(-K h^-3 w C_i r) and the
//   signal velocity max                                                   hydro_ve/av_switches_kern.hpp:43-137
//   a_i, du_i with the Atwood-weighted volume terms and the AV            hydro_ve/momentum_energy_kern.hpp:43-222
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define VEAD_HD __host__ __device__ __forceinline__
#else
#define VEAD_HD inline
#endif

namespace sphgb {
namespace vead {

constexpr double kAtmin = 0.1, kAtmax = 0.2, kRamp = 1.0 / (kAtmax - kAtmin);

VEAD_HD void symv(const double C[6], const double r[3], double o[3])
{
    o[0] = C[0] * r[0] + C[1] * r[1] + C[2] * r[2];
    o[1] = C[1] * r[0] + C[3] * r[1] + C[4] * r[2];
    o[2] = C[2] * r[0] + C[4] * r[1] + C[5] * r[2];
}

// Cb += s * d(a . C r) / dC, with s folded into a first (3 products and 9 FMAs)
VEAD_HD void symvAdj(const double a[3], const double r[3], double s, double Cb[6])
{
    const double sa0 = s * a[0], sa1 = s * a[1], sa2 = s * a[2];
    Cb[0] = fma(sa0, r[0], Cb[0]);
    Cb[1] = fma(sa0, r[1], fma(sa1, r[0], Cb[1]));
    Cb[2] = fma(sa0, r[2], fma(sa2, r[0], Cb[2]));
    Cb[3] = fma(sa1, r[1], Cb[3]);
    Cb[4] = fma(sa1, r[2], fma(sa2, r[1], Cb[4]));
    Cb[5] = fma(sa2, r[2], Cb[5]);
}

// r^T g r with the stored components (avRvCorrection's quadratic form, momentum_energy_kern.hpp:43-50)
VEAD_HD double quad(const double g[6], const double r[3])
{
    return g[0] * r[0] * r[0] + g[1] * r[0] * r[1] + g[2] * r[0] * r[2] + g[3] * r[1] * r[1] + g[4] * r[1] * r[2] +
           g[5] * r[2] * r[2];
}

VEAD_HD void quadAdjR(const double g[6], const double r[3], double s, double rb[3])
{
    rb[0] += s * (2.0 * g[0] * r[0] + g[1] * r[1] + g[2] * r[2]);
    rb[1] += s * (g[1] * r[0] + 2.0 * g[3] * r[1] + g[4] * r[2]);
    rb[2] += s * (g[2] * r[0] + g[4] * r[1] + 2.0 * g[5] * r[2]);
}

VEAD_HD void quadAdjG(const double r[3], double s, double gb[6])
{
    gb[0] += s * r[0] * r[0];
    gb[1] += s * r[0] * r[1];
    gb[2] += s * r[0] * r[2];
    gb[3] += s * r[1] * r[1];
    gb[4] += s * r[1] * r[2];
    gb[5] += s * r[2] * r[2];
}

// ------------------------------------------------------------------ momentum-energy
struct MeSide {
    double hInv, c, alpha, m, rho, rhoInv, xm, xmInv, lnxm, prho;
    double C[6], g[6];
};

struct MeFwd {
    double v1, v2, hi3, hj3, Wi, Wj, CIr[3], CJr[3], Ai[3], Aj[3];
    double rv, wij, asum, csum, visc;
    bool approaching;
    double d1, d2, d3, e, A, praw, pc, phi;
    bool etaIsV2, etaBelow, clampActive;
    int branch;
    double srInv, At, s, am, bm;
    double av, bv, avv[3];
};

VEAD_HD void meFwd(const double r[3], double d, double rinv, const double v[3], const MeSide& I, const MeSide& J,
                   double wi, double wj, bool avClean, double etaCrit, MeFwd& f)
{
    f.v1 = d * I.hInv;
    f.v2 = d * J.hInv;
    f.hi3 = I.hInv * I.hInv * I.hInv;
    f.hj3 = J.hInv * J.hInv * J.hInv;
    f.Wi = f.hi3 * wi;
    f.Wj = f.hj3 * wj;
    symv(I.C, r, f.CIr);
    symv(J.C, r, f.CJr);
    for (int k = 0; k < 3; ++k) {
        f.Ai[k] = -f.Wi * f.CIr[k];
        f.Aj[k] = -f.Wj * f.CJr[k];
    }
    double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    f.d1 = f.d2 = f.e = f.A = f.praw = f.pc = f.phi = 0.0;
    f.d3 = 1.0;
    f.etaIsV2 = f.etaBelow = f.clampActive = false;
    if (avClean) {
        f.d1 = quad(I.g, r);
        f.d2 = quad(J.g, r);
        f.etaIsV2 = f.v2 < f.v1;  // std::min(v1, v2) keeps v1 on a tie
        const double eta = f.etaIsV2 ? f.v2 : f.v1;
        f.etaBelow = eta < etaCrit;
        f.e = 5.0 * (eta - etaCrit);
        if (f.etaBelow) f.d3 = exp(-f.e * f.e);
        f.A = f.d2 != 0.0 ? f.d1 / f.d2 : 0.0;
        const double Ap1 = 1.0 + f.A;
        f.praw = 4.0 * f.A / (Ap1 * Ap1);
        f.clampActive = f.praw >= 0.0 && f.praw <= 1.0;
        f.pc = fmax(0.0, fmin(1.0, f.praw));
        f.phi = 0.5 * f.d3 * f.pc;
        rv -= f.phi * (f.d1 + f.d2);
    }
    f.rv = rv;
    f.wij = rv * rinv;
    f.approaching = f.wij < 0.0;
    f.asum = I.alpha + J.alpha;
    f.csum = I.c + J.c;
    f.visc = f.approaching ? -(0.25 * f.asum * f.csum - 2.0 * f.wij) * f.wij : 0.0;
    // Atwood number |rho_i - rho_j| / (rho_i + rho_j) against Atmin / Atmax without dividing
    const double dr = fabs(I.rho - J.rho), sr = I.rho + J.rho;
    f.s = f.At = f.srInv = 0.0;
    if (dr < kAtmin * sr) {
        f.branch = 0;
        f.am = I.xm * I.xm;
        f.bm = J.xm * J.xm;
    } else if (kAtmax * sr < dr) {
        f.branch = 2;
        f.am = I.xm * J.xm;
        f.bm = f.am;
    } else {
        f.branch = 1;
        f.srInv = 1.0 / sr;
        f.At = dr * f.srInv;
        f.s = kRamp * (f.At - kAtmin);
        const double q = exp(f.s * (J.lnxm - I.lnxm));
        f.am = I.xm * I.xm * q;
        f.bm = J.xm * J.xm / q;
    }
    f.av = J.m * I.rhoInv * f.visc;
    f.bv = J.m * J.rhoInv * f.visc;
    for (int k = 0; k < 3; ++k) f.avv[k] = 0.5 * (f.av * f.Ai[k] + f.bv * f.Aj[k]);
}

// the pair's contributions to i's energy sums: en (pressure part) and avE (AV part, before max(0, .))
VEAD_HD void meSums(const double v[3], const MeSide& J, const MeFwd& f, double& en, double& avE)
{
    en += J.m * f.am * (v[0] * f.Ai[0] + v[1] * f.Ai[1] + v[2] * f.Ai[2]);
    avE += f.avv[0] * v[0] + f.avv[1] * v[1] + f.avv[2] * v[2];
}

struct MeGrad {
    double r[3], v[3], c, alpha;                 // r: x_i += , x_j -= ; v: v_i += , v_j -= ; c, alpha: both ends
    double hI, prhoI, rhoI, xmI, CI[6], gI[6];   // i's fields
    double hJ, prhoJ, rhoJ, xmJ, CJ[6], gJ[6];   // j's fields
};

// adjoints of the pair's shared intermediates, set by the seed-dependent head
struct MeBar {
    double Aib[3], Ajb[3], amb, bmb, viscb;
};

// from the intermediates' adjoints to the pair's inputs (common to one term and to a mutual pair)
template<bool AvClean>
VEAD_HD void meTail(const double r[3], double rinv, const double v[3], const MeSide& I, const MeSide& J, double wi,
                    double dwi, double wj, double dwj, const MeFwd& f, const MeBar& b, MeGrad& o)
{
    // Atwood weights
    if (f.branch == 0) {
        o.xmI += 2.0 * b.amb * I.xm;
        o.xmJ += 2.0 * b.bmb * J.xm;
    } else if (f.branch == 2) {
        o.xmI += (b.amb + b.bmb) * J.xm;
        o.xmJ += (b.amb + b.bmb) * I.xm;
    } else {
        const double pa = b.amb * f.am, pb = b.bmb * f.bm;
        o.xmI += ((2.0 - f.s) * pa + f.s * pb) * I.xmInv;
        o.xmJ += (f.s * pa + (2.0 - f.s) * pb) * J.xmInv;
        const double Atb = (pa - pb) * (J.lnxm - I.lnxm) * kRamp;
        const double sgn = I.rho > J.rho ? 1.0 : (I.rho < J.rho ? -1.0 : 0.0);
        o.rhoI += Atb * (sgn - f.At) * f.srInv;
        o.rhoJ += Atb * (-sgn - f.At) * f.srInv;
    }
    // viscosity
    double wijb = 0.0;
    if (f.approaching) {
        wijb = b.viscb * (-0.25 * f.asum * f.csum + 4.0 * f.wij);
        o.c = b.viscb * (-0.25 * f.asum * f.wij);
        o.alpha = b.viscb * (-0.25 * f.csum * f.wij);
    }
    const double rvb = wijb * rinv;
    double db = -wijb * f.wij * rinv;
    double v1b = 0.0, v2b = 0.0;
    if (AvClean) {
        const double phib = -rvb * (f.d1 + f.d2);
        double d1b = -rvb * f.phi, d2b = -rvb * f.phi;
        const double pcb = phib * 0.5 * f.d3;
        const double d3b = phib * 0.5 * f.pc;
        if (f.clampActive && f.d2 != 0.0) {
            const double Ap1 = 1.0 + f.A;
            const double Ab = pcb * 4.0 * (1.0 - f.A) / (Ap1 * Ap1 * Ap1);
            d1b += Ab / f.d2;
            d2b -= Ab * f.A / f.d2;
        }
        if (f.etaBelow) {
            const double etab = d3b * f.d3 * (-2.0 * f.e) * 5.0;
            if (f.etaIsV2) v2b += etab;
            else v1b += etab;
        }
        quadAdjR(I.g, r, d1b, o.r);
        quadAdjR(J.g, r, d2b, o.r);
        quadAdjG(r, d1b, o.gI);
        quadAdjG(r, d2b, o.gJ);
    }
    for (int k = 0; k < 3; ++k) {
        o.r[k] += rvb * v[k];
        o.v[k] += rvb * r[k];
    }
    // A_i = -W_i C_i r, A_j = -W_j C_j r
    const double Wib = -(b.Aib[0] * f.CIr[0] + b.Aib[1] * f.CIr[1] + b.Aib[2] * f.CIr[2]);
    const double Wjb = -(b.Ajb[0] * f.CJr[0] + b.Ajb[1] * f.CJr[1] + b.Ajb[2] * f.CJr[2]);
    symvAdj(b.Aib, r, -f.Wi, o.CI);
    symvAdj(b.Ajb, r, -f.Wj, o.CJ);
    double CAi[3], CAj[3];
    symv(I.C, b.Aib, CAi);
    symv(J.C, b.Ajb, CAj);
    for (int k = 0; k < 3; ++k) o.r[k] += -f.Wi * CAi[k] - f.Wj * CAj[k];
    // W_i = h_i^-3 w(d / h_i): dW_i/dh_i = -h_i^-4 (3 w + v1 dw), dW_i/dd = h_i^-4 dw
    const double bi4 = Wib * (f.hi3 * I.hInv), bj4 = Wjb * (f.hj3 * J.hInv);
    o.hI = -bi4 * fma(f.v1, dwi, 3.0 * wi);
    o.hJ = -bj4 * fma(f.v2, dwj, 3.0 * wj);
    db = fma(bi4, dwi, fma(bj4, dwj, db));
    if constexpr (AvClean) {
        o.hI -= v1b * f.v1 * I.hInv;
        o.hJ -= v2b * f.v2 * J.hInv;
        db += v1b * I.hInv + v2b * J.hInv;
    }
    const double dr = db * rinv;  // d|r|/dr = r / |r|
    for (int k = 0; k < 3; ++k) o.r[k] = fma(dr, r[k], o.r[k]);
}

VEAD_HD void meGradZero(MeGrad& o)
{
    for (int k = 0; k < 3; ++k) o.r[k] = o.v[k] = 0.0;
    for (int q = 0; q < 6; ++q) o.CI[q] = o.CJ[q] = o.gI[q] = o.gJ[q] = 0.0;
    o.c = o.alpha = o.xmI = o.xmJ = 0.0;
}

// i's term of one pair.  Seeds of i: mb = dL/d(sum of momentum terms) = -K abar_i, enb = K prho_i
// dubar_i, avEb = K/2 dubar_i where the sum avE_i >= 0 (0 otherwise).  WithDu = false: enb = avEb
// = 0 (no du seed) and the energy terms drop out; AvClean selects momentumAndEnergy<avClean>.
template<bool AvClean, bool WithDu>
VEAD_HD void meAdj(const double r[3], double d, double rinv, const double v[3], const MeSide& I, const MeSide& J,
                   double wi, double dwi, double wj, double dwj, double etaCrit, const double mb[3], double enb,
                   double avEb, MeGrad& o)
{
    MeFwd f;
    meFwd(r, d, rinv, v, I, J, wi, wj, AvClean, etaCrit, f);
    meGradZero(o);
    const double mj = J.m;
    MeBar b;
    double avvb[3], mbAi = 0.0, mbAj = 0.0, vAi = 0.0;
    for (int k = 0; k < 3; ++k) {
        avvb[k] = WithDu ? mb[k] + avEb * v[k] : mb[k];
        mbAi += mb[k] * f.Ai[k];
        mbAj += mb[k] * f.Aj[k];
        if (WithDu) vAi += v[k] * f.Ai[k];
    }
    for (int k = 0; k < 3; ++k) {
        if (WithDu) o.v[k] = avEb * f.avv[k] + enb * mj * f.am * f.Ai[k];
        b.Aib[k] = mb[k] * mj * I.prho * f.am + 0.5 * f.av * avvb[k];
        if (WithDu) b.Aib[k] += enb * mj * f.am * v[k];
        b.Ajb[k] = mb[k] * mj * J.prho * f.bm + 0.5 * f.bv * avvb[k];
    }
    b.amb = WithDu ? mbAi * mj * I.prho + enb * mj * vAi : mbAi * mj * I.prho;
    b.bmb = mbAj * mj * J.prho;
    o.prhoI = mbAi * mj * f.am;
    o.prhoJ = mbAj * mj * f.bm;
    const double avb = 0.5 * (avvb[0] * f.Ai[0] + avvb[1] * f.Ai[1] + avvb[2] * f.Ai[2]);
    const double bvb = 0.5 * (avvb[0] * f.Aj[0] + avvb[1] * f.Aj[1] + avvb[2] * f.Aj[2]);
    b.viscb = (avb * I.rhoInv + bvb * J.rhoInv) * mj;
    o.rhoI = -avb * f.av * I.rhoInv;
    o.rhoJ = -bvb * f.bv * J.rhoInv;
    meTail<AvClean>(r, rinv, v, I, J, wi, dwi, wj, dwj, f, b, o);
}

// both terms of a mutual pair (i's term of j and j's term of i, same image, no avClean correction)
// from one evaluation.  With r_ji = -r, v_ji = -v the two terms share every intermediate and
// their seeds enter only through s = m_j mb_i - m_i mb_j, sigma = m_j avEb_i + m_i avEb_j and the
// energy seeds.
template<bool WithDu>
VEAD_HD void meAdjMutual(const double r[3], double d, double rinv, const double v[3], const MeSide& I,
                         const MeSide& J, double wi, double dwi, double wj, double dwj, const double mbI[3],
                         double enbI, double avEbI, const double mbJ[3], double enbJ, double avEbJ, MeGrad& o)
{
    MeFwd f;
    meFwd(r, d, rinv, v, I, J, wi, wj, false, 0.0, f);
    meGradZero(o);
    if constexpr (!WithDu) {
        // no du seed: u_i = prho_i s, u_j = prho_j s and t = s, so every projection follows from
        // s . A_i and s . A_j, and Abar_i = (am prho_i + hv_i) s, Abar_j = (bm prho_j + hv_j) s
        double s3[3];
        for (int k = 0; k < 3; ++k) s3[k] = J.m * mbI[k] - I.m * mbJ[k];
        const double sAi = s3[0] * f.Ai[0] + s3[1] * f.Ai[1] + s3[2] * f.Ai[2];
        const double sAj = s3[0] * f.Aj[0] + s3[1] * f.Aj[1] + s3[2] * f.Aj[2];
        const double hvi = 0.5 * f.visc * I.rhoInv, hvj = 0.5 * f.visc * J.rhoInv;
        const double ci = fma(f.am, I.prho, hvi), cj = fma(f.bm, J.prho, hvj);
        MeBar b;
        for (int k = 0; k < 3; ++k) {
            b.Aib[k] = ci * s3[k];
            b.Ajb[k] = cj * s3[k];
        }
        b.amb = I.prho * sAi;
        b.bmb = J.prho * sAj;
        b.viscb = 0.5 * (sAi * I.rhoInv + sAj * J.rhoInv);
        o.prhoI = f.am * sAi;
        o.prhoJ = f.bm * sAj;
        o.rhoI = -hvi * sAi * I.rhoInv;
        o.rhoJ = -hvj * sAj * J.rhoInv;
        meTail<false>(r, rinv, v, I, J, wi, dwi, wj, dwj, f, b, o);
        return;
    }
    double sv[3], ui[3], uj[3], t[3];
    const double sigma = WithDu ? J.m * avEbI + I.m * avEbJ : 0.0;
    for (int k = 0; k < 3; ++k) {
        sv[k] = J.m * mbI[k] - I.m * mbJ[k];
        ui[k] = I.prho * sv[k];
        uj[k] = J.prho * sv[k];
        t[k] = sv[k];
        if (WithDu) {
            ui[k] += enbI * J.m * v[k];
            uj[k] += enbJ * I.m * v[k];
            t[k] += sigma * v[k];
        }
    }
    double sAi = 0.0, sAj = 0.0, tAi = 0.0, tAj = 0.0, uAi = 0.0, uAj = 0.0;
    for (int k = 0; k < 3; ++k) {
        sAi += sv[k] * f.Ai[k];
        sAj += sv[k] * f.Aj[k];
        tAi += t[k] * f.Ai[k];
        tAj += t[k] * f.Aj[k];
        uAi += ui[k] * f.Ai[k];
        uAj += uj[k] * f.Aj[k];
    }
    const double hvi = 0.5 * f.visc * I.rhoInv, hvj = 0.5 * f.visc * J.rhoInv;
    MeBar b;
    for (int k = 0; k < 3; ++k) {
        b.Aib[k] = f.am * ui[k] + hvi * t[k];
        b.Ajb[k] = f.bm * uj[k] + hvj * t[k];
        if (WithDu)
            o.v[k] = enbI * J.m * f.am * f.Ai[k] + enbJ * I.m * f.bm * f.Aj[k] +
                     sigma * (hvi * f.Ai[k] + hvj * f.Aj[k]);
    }
    b.amb = uAi;
    b.bmb = uAj;
    b.viscb = 0.5 * (tAi * I.rhoInv + tAj * J.rhoInv);
    o.prhoI = f.am * sAi;
    o.prhoJ = f.bm * sAj;
    o.rhoI = -hvi * tAi * I.rhoInv;
    o.rhoJ = -hvj * tAj * J.rhoInv;
    meTail<false>(r, rinv, v, I, J, wi, dwi, wj, dwj, f, b, o);
}

// ------------------------------------------------------------------ AV switches
struct AvPrm {
    double K, dt, alphamin, alphamax, decay;
};

// per-particle part of the reverse AV switch.  In: alphab (dL/dalpha_i after the switch), the
// alpha before it, h, c, divv, G (3), the signal velocity vsig.  Out: Gb (seed of the pair terms of
// G), vsigb (seed of the pair that set vsig), and the particle's own partials.
VEAD_HD void avSeed(const AvPrm& P, double alphab, double alpha0, double h, double c, double divv, const double G[3],
                    double vsig, double Gb[3], double& vsigb, double& hb, double& divvb, double& cb)
{
    Gb[0] = Gb[1] = Gb[2] = 0.0;
    vsigb = hb = divvb = cb = 0.0;
    const double gdv = sqrt(G[0] * G[0] + G[1] * G[1] + G[2] * G[2]);
    double aloc = 0.0, ac = 0.0, E = 0.0, D = 1.0;
    if (divv < 0.0) {
        ac = h * h * gdv;
        E = h * fabs(divv) + 0.05 * c;
        D = ac + E;
        aloc = P.alphamax * ac / D;
    }
    double alocb = 0.0;
    if (aloc >= alpha0) alocb = alphab;
    else {
        const double X = aloc >= P.alphamin ? aloc : P.alphamin;
        // alpha = alpha0 + (X - alpha0) dt decay vsig / h
        const double k = P.dt * P.decay / h;
        if (aloc >= P.alphamin) alocb = alphab * k * vsig;
        vsigb = alphab * (X - alpha0) * k;
        hb -= alphab * (X - alpha0) * k * vsig / h;
    }
    if (divv < 0.0) {
        const double acb = alocb * P.alphamax * E / (D * D);
        const double Eb = -alocb * P.alphamax * ac / (D * D);
        hb += Eb * fabs(divv) + acb * 2.0 * h * gdv;
        divvb -= Eb * h;
        cb += 0.05 * Eb;
        const double gdvb = acb * h * h;
        if (gdv > 0.0)
            for (int k = 0; k < 3; ++k) Gb[k] = gdvb * G[k] / gdv;
    }
}

struct AvGrad {
    double r[3], v[3], cI, cJ;
    double hI, divvI, R[3];   // R: this pair's part of sum_j fac_j W_j r_j (i's C partials, see avCbar)
    double divvJ, xmJ, kxJ;
};

// pair term of G_i = sum_j fac_j t_j, fac_j = vol_j (divv_i - divv_j), t_j = -W_j C_i r_j,
// W_j = K h_i^-3 w(d_j / h_i), given Gb (dL/dG_i) through CGb = C_i Gb (C symmetric): the pair
// needs only r . CGb; i's C partials are -sym(Gb R^T) with R = sum_j fac_j W_j r_j (avCbar).  For
// the pair that set vsig_i, the signal velocity c_i + c_j - 3 rv / d as well.
VEAD_HD void avAdj(const double r[3], double d, double rinv, const double v[3], double hiInv, double wi, double dwi,
                   double K, double volj, double kxInvj, double divvi, double divvj, const double CGb[3],
                   double vsigb, bool isVsigPair, AvGrad& o)
{
    const double hi3 = hiInv * hiInv * hiInv;
    const double Wk = K * hi3 * wi;
    const double ddiv = divvi - divvj;
    const double fac = volj * ddiv;
    const double rc = r[0] * CGb[0] + r[1] * CGb[1] + r[2] * CGb[2];
    const double facb = -Wk * rc;
    const double Wkb = -fac * rc;
    const double volb = facb * ddiv;
    o.divvI = facb * volj;
    o.divvJ = -facb * volj;
    o.xmJ = volb * kxInvj;
    o.kxJ = -volb * volj * kxInvj;
    // W = K h^-3 w(d / h): dW/dh = -K h^-4 (3 w + v1 dw), dW/dd = K h^-4 dw
    const double v1 = d * hiInv;
    const double b4 = Wkb * K * (hi3 * hiInv);
    o.hI = -b4 * fma(v1, dwi, 3.0 * wi);
    double db = b4 * dwi;
    const double fw = fac * Wk;
    for (int k = 0; k < 3; ++k) {
        o.r[k] = -fw * CGb[k];
        o.R[k] = fw * r[k];
        o.v[k] = 0.0;
    }
    o.cI = o.cJ = 0.0;
    if (isVsigPair) {
        const double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
        o.cI = vsigb;
        o.cJ = vsigb;
        const double rvb = -3.0 * vsigb * rinv;
        db += 3.0 * vsigb * rv * rinv * rinv;
        for (int k = 0; k < 3; ++k) {
            o.r[k] += rvb * v[k];
            o.v[k] += rvb * r[k];
        }
    }
    const double dr = db * rinv;  // d|r|/dr = r / |r|
    for (int k = 0; k < 3; ++k) o.r[k] = fma(dr, r[k], o.r[k]);
}

// i's C partials from the AV pair sum: Cb += -sym(Gb R^T), R = sum_j fac_j W_j r_j
VEAD_HD void avCbar(const double Gb[3], const double R[3], double Cb[6]) { symvAdj(Gb, R, -1.0, Cb); }

// ------------------------------------------------------------------ IAD + divv
// per-particle part: from Cb (6), divvb and gb (6, the avClean velocity gradient) of particle i and
// P_i (9, row-major P[a][q]), the seeds of the pair terms: tauB (6, symmetric tau adjoint) and
// PB (9); adds the particle's own partials to hb, kxb.
VEAD_HD void iadDivvSeed(double K, double h, double kx, const double C[6], const double Cb_in[6], double divvb,
                         const double gb[6], const double P[9], double tauB[6], double PB[9], double& hb, double& kxb)
{
    const double hInv = 1.0 / h;
    const double nk = K * hInv * hInv * hInv / kx;
    const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    double Cf[3][3], dV[3][3], Db[3][3];
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 3; ++q) Cf[a][q] = C[idx[a][q]];
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 3; ++q) dV[a][q] = -(P[3 * a] * Cf[0][q] + P[3 * a + 1] * Cf[1][q] + P[3 * a + 2] * Cf[2][q]);
    // divv = nk tr dV, g = nk {dV00, dV01 + dV10, dV02 + dV20, dV11, dV12 + dV21, dV22}
    Db[0][0] = divvb + gb[0];
    Db[1][1] = divvb + gb[3];
    Db[2][2] = divvb + gb[5];
    Db[0][1] = Db[1][0] = gb[1];
    Db[0][2] = Db[2][0] = gb[2];
    Db[1][2] = Db[2][1] = gb[4];
    double nkb = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 3; ++q) {
            nkb += Db[a][q] * dV[a][q];
            Db[a][q] *= nk;
        }
    hb += nkb * (-3.0 * nk * hInv);
    kxb += -nkb * nk / kx;
    // dV = -P C: PB = -Db C, full-matrix Cbar = -P^T Db
    double Fc[3][3];
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 3; ++q) {
            PB[3 * a + q] = -(Db[a][0] * Cf[0][q] + Db[a][1] * Cf[1][q] + Db[a][2] * Cf[2][q]);
            Fc[a][q] = -(P[a] * Db[0][q] + P[3 + a] * Db[1][q] + P[6 + a] * Db[2][q]);
        }
    double Cb[6];
    for (int q = 0; q < 6; ++q) Cb[q] = Cb_in[q];
    Cb[0] += Fc[0][0];
    Cb[1] += Fc[0][1] + Fc[1][0];
    Cb[2] += Fc[0][2] + Fc[2][0];
    Cb[3] += Fc[1][1];
    Cb[4] += Fc[1][2] + Fc[2][1];
    Cb[5] += Fc[2][2];
    // C = s tau^-1, s = h^3 / K: tauB = -s M G M with M = C / s, G the symmetric gradient; hb from s
    const double s = h * h * h / K;
    double M[3][3], G[3][3];
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 3; ++q) {
            M[a][q] = Cf[a][q] / s;
            const double cb = Cb[idx[a][q]];
            G[a][q] = a == q ? cb : 0.5 * cb;
        }
    double MG[3][3], T[3][3], sb = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 3; ++q) MG[a][q] = M[a][0] * G[0][q] + M[a][1] * G[1][q] + M[a][2] * G[2][q];
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 3; ++q) {
            T[a][q] = -s * (MG[a][0] * M[0][q] + MG[a][1] * M[1][q] + MG[a][2] * M[2][q]);
            sb += G[a][q] * M[a][q];
        }
    hb += sb * 3.0 * h * h / K;
    tauB[0] = T[0][0];
    tauB[1] = 0.5 * (T[0][1] + T[1][0]);
    tauB[2] = 0.5 * (T[0][2] + T[2][0]);
    tauB[3] = T[1][1];
    tauB[4] = 0.5 * (T[1][2] + T[2][1]);
    tauB[5] = T[2][2];
}

struct IadGrad {
    double r[3], v[3];  // r: x_i += , x_j -= ; v (= d/dv_ij): v_i += , v_j -=
    double hI, xmJ, kxJ;
};

// pair terms of tau_i (vol_j w r r^T) and P_i (xm_j w (v_j - v_i) r^T)
VEAD_HD void iadDivvAdj(const double r[3], double d, double rinv, const double v[3], double hiInv, double wi,
                        double dwi, double volj, double kxInvj, double xmj, const double tauB[6], const double PB[9],
                        IadGrad& o)
{
    double Tr[3];
    symv(tauB, r, Tr);
    const double Q = r[0] * Tr[0] + r[1] * Tr[1] + r[2] * Tr[2];
    // P term with vji = -v
    double PBr[3];
    for (int a = 0; a < 3; ++a) PBr[a] = PB[3 * a] * r[0] + PB[3 * a + 1] * r[1] + PB[3 * a + 2] * r[2];
    const double vPr = -(v[0] * PBr[0] + v[1] * PBr[1] + v[2] * PBr[2]);
    const double wb = volj * Q + xmj * vPr;
    const double volb = wi * Q;
    o.xmJ = volb * kxInvj + wi * vPr;
    o.kxJ = -volb * volj * kxInvj;
    for (int a = 0; a < 3; ++a) o.v[a] = -xmj * wi * PBr[a];
    for (int q = 0; q < 3; ++q) {
        const double PtV = -(v[0] * PB[q] + v[1] * PB[3 + q] + v[2] * PB[6 + q]);
        o.r[q] = volj * wi * 2.0 * Tr[q] + xmj * wi * PtV;
    }
    const double v1 = d * hiInv;
    const double v1b = wb * dwi;
    o.hI = -v1b * v1 * hiInv;
    const double db = v1b * hiInv;
    const double dr = db * rinv;  // d|r|/dr = r / |r|
    for (int k = 0; k < 3; ++k) o.r[k] = fma(dr, r[k], o.r[k]);
}

// ------------------------------------------------------------------ EOS
// rho = kx m / xm, p = (gamma-1) rho u, c = sqrt(gamma (gamma-1) u), prho = p / (kx m^2 gradh)
VEAD_HD void eosAdj(double gamma, double u, double m, double kx, double xm, double gradh, double c, double prhob,
                    double cb, double rhob, double& kxb, double& xmb, double& gradhb, double& ub)
{
    const double g1 = gamma - 1.0;
    const double rho = kx * m / xm;
    const double den = kx * m * m * gradh;
    const double prho = g1 * rho * u / den;
    const double pb = prhob / den;
    kxb -= prhob * prho / kx;
    gradhb -= prhob * prho / gradh;
    const double rhoTot = rhob + pb * g1 * u;
    ub += pb * g1 * rho + (c > 0.0 ? cb * gamma * g1 / (2.0 * c) : 0.0);
    kxb += rhoTot * m / xm;
    xmb -= rhoTot * rho / xm;
}

// ------------------------------------------------------------------ kx / gradh
// per-particle part: from kxb, gradhb (complete) and the sums whomega0 = K h^-4 S_om and
// wrho0 = K h^-4 S_r0, the seeds Skxb, Somb, Sr0b of the pair sums and the own partials
VEAD_HD void gradhSeed(double K, double h, double m, double xm, double kx, double whomega0, double wrho0, double kxb_in,
                       double gradhb, double& Skxb, double& Somb, double& Sr0b, double& hb, double& xmb)
{
    const double hInv = 1.0 / h, h3 = hInv * hInv * hInv;
    const double whomega = whomega0 * m / xm + (kx - K * xm * h3) * wrho0;
    const double rho = kx * m / xm;
    // gradh = 1 + h whomega / (3 rho)
    hb += gradhb * whomega / (3.0 * rho);
    const double whomegab = gradhb * h / (3.0 * rho);
    const double rhob = -gradhb * h * whomega / (3.0 * rho * rho);
    double kxb = kxb_in + rhob * m / xm;
    xmb -= rhob * rho / xm;
    const double whomega0b = whomegab * m / xm;
    xmb -= whomegab * whomega0 * m / (xm * xm);
    kxb += whomegab * wrho0;
    xmb -= whomegab * wrho0 * K * h3;
    hb += whomegab * wrho0 * K * xm * 3.0 * h3 * hInv;
    const double wrho0b = whomegab * (kx - K * xm * h3);
    // kx = K h^-3 S_kx, whomega0 = K h^-4 S_om, wrho0 = K h^-4 S_r0
    Skxb = kxb * K * h3;
    hb -= 3.0 * kxb * kx * hInv;
    Somb = whomega0b * K * h3 * hInv;
    hb -= 4.0 * whomega0b * whomega0 * hInv;
    Sr0b = wrho0b * K * h3 * hInv;
    hb -= 4.0 * wrho0b * wrho0 * hInv;
    // self terms S_kx = xm_i + ..., S_om = -3 xm_i + ...
    xmb += Skxb - 3.0 * Somb;
}

struct GradhGrad {
    double r[3], hI, xmJ;
};

// pair terms w xm_j (S_kx), dterh xm_j (S_om), dterh m_j (S_r0), dterh = -(3 w + v1 wd(v1))
VEAD_HD void gradhAdj(const double r[3], double d, double rinv, double hiInv, double wi, double dwi, double wdi,
                      double dwdi, double xmj, double mj, double Skxb, double Somb, double Sr0b, GradhGrad& o)
{
    const double v1 = d * hiInv;
    const double dterh = -(3.0 * wi + v1 * wdi);
    o.xmJ = Skxb * wi + Somb * dterh;
    const double dterhb = Somb * xmj + Sr0b * mj;
    const double wb = Skxb * xmj - 3.0 * dterhb;
    const double wdb = -dterhb * v1;
    const double v1b = -dterhb * wdi + wb * dwi + wdb * dwdi;
    o.hI = -v1b * v1 * hiInv;
    const double db = v1b * hiInv;
    const double dr = db * rinv;
    for (int k = 0; k < 3; ++k) o.r[k] = dr * r[k];
}

// ------------------------------------------------------------------ xmass
// xm = m h^3 / (K R0), R0 = m + sum_j m_j w: own partial of h and the seed R0b of the pair sum
VEAD_HD void xmassSeed(double K, double h, double m, double xm, double xmb, double& R0b, double& hb)
{
    hb += xmb * 3.0 * xm / h;
    const double R0 = m * h * h * h / (K * xm);
    R0b = -xmb * xm / R0;
}

VEAD_HD void xmassAdj(const double r[3], double d, double rinv, double hiInv, double dwi, double mj, double R0b,
                      double rb[3], double& hIb)
{
    const double v1 = d * hiInv;
    const double v1b = R0b * mj * dwi;
    hIb = -v1b * v1 * hiInv;
    const double db = v1b * hiInv;
    const double dr = db * rinv;
    for (int k = 0; k < 3; ++k) rb[k] = dr * r[k];
}

}  // namespace vead
}  // namespace sphgb
