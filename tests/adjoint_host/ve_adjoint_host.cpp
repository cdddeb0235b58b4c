// Host driver of the VE adjoint arithmetic (sphexa_gb300/csrc/adjoint_ve.cuh): the pass sequence of
// the device adjoint (adjoint_ve.cu) as plain sequential loops over a CSR neighbour list, so that
// the pair and particle functions the kernels call can be checked against torch autograd on the
// CPU.  Test infrastructure; built by tests/test_adjoint_host.py with g++.
//
// mutualMode = 1 evaluates a pair whose ends list each other once, through meAdjMutual (the form
// the device uses with owned lists); 0 evaluates every list entry through meAdj.
#include <cmath>
#include <cstdint>
#include <vector>

#include "adjoint_ve.cuh"
using namespace sphgb::vead;

struct In {
    int64_t n;
    const double *x, *y, *z, *vx, *vy, *vz, *h, *u, *m, *alpha0, *alpha, *xm, *kx, *gradh, *prho, *c, *divv;
    const double* C[6];
    const double* dV[6];
    const int64_t *off, *idx;
    const double *wh, *whd;
    int64_t ntab;
    double K, gamma, L[3];
    int pbc[3];
    double dt, amin, amax, decay;
    int avClean;
    const double *sRho, *sAx, *sAy, *sAz, *sDu;
    double *gx, *gy, *gz, *gvx, *gvy, *gvz, *gh, *gu;
};

static double look(const In& a, const double* t, double v, double& slope)
{
    double invDx = (a.ntab - 1) / 2.0;
    int64_t k = int64_t(v * invDx);
    if (k >= a.ntab - 1) { slope = 0; return 0; }
    slope = (t[k + 1] - t[k]) * invDx;
    return t[k] + (t[k + 1] - t[k]) * (v * invDx - k);
}

static void pairR(const In& a, int64_t i, int64_t j, double r[3], double& d, double& rinv)
{
    double dd[3] = {a.x[i] - a.x[j], a.y[i] - a.y[j], a.z[i] - a.z[j]};
    double th = 2.0 * a.h[i];
    for (int k = 0; k < 3; ++k) {
        r[k] = dd[k];
        if (a.pbc[k]) {
            if (r[k] > th) r[k] -= a.L[k];
            else if (r[k] < -th) r[k] += a.L[k];
        }
    }
    d = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    rinv = 1.0 / d;
}

extern "C" int ve_adj_host(const In* ap, int mutualMode)
{
    const In& a = *ap;
    int64_t n = a.n;
    std::vector<double> hInv(n), rho(n), vol(n), lnxm(n);
    for (int64_t i = 0; i < n; ++i) {
        hInv[i] = 1.0 / a.h[i];
        rho[i] = a.kx[i] * a.m[i] / a.xm[i];
        vol[i] = a.xm[i] / a.kx[i];
        lnxm[i] = std::log(a.xm[i]);
    }
    auto side = [&](int64_t i) {
        MeSide s;
        s.hInv = hInv[i]; s.c = a.c[i]; s.alpha = a.alpha[i]; s.m = a.m[i]; s.rho = rho[i]; s.xm = a.xm[i];
        s.rhoInv = 1.0 / rho[i]; s.xmInv = 1.0 / a.xm[i];
        s.lnxm = lnxm[i]; s.prho = a.prho[i];
        for (int q = 0; q < 6; ++q) { s.C[q] = a.C[q][i]; s.g[q] = a.avClean ? a.dV[q][i] : 0.0; }
        return s;
    };
    std::vector<double> en(n), avE(n), G(3 * n), vsig(n), P(9 * n), wom(n), wr0(n);
    std::vector<int64_t> arg(n);
    for (int64_t i = 0; i < n; ++i) {
        MeSide I = side(i);
        int64_t cnt = a.off[i + 1] - a.off[i];
        double etaCrit = std::cbrt(32.0 * M_PI / 3.0 / double(cnt + 1));
        double e = 0, ae = 0, g[3] = {0, 0, 0}, vs = 1e-40 * a.c[i], Pi[9] = {0}, so = -3 * a.xm[i], sr = -3 * a.m[i];
        int64_t ag = -1;
        double Cr_[6];
        for (int q = 0; q < 6; ++q) Cr_[q] = a.C[q][i];
        for (int64_t q = a.off[i]; q < a.off[i + 1]; ++q) {
            int64_t j = a.idx[q];
            double r[3], d, rinv;
            pairR(a, i, j, r, d, rinv);
            double v[3] = {a.vx[i] - a.vx[j], a.vy[i] - a.vy[j], a.vz[i] - a.vz[j]};
            MeSide J = side(j);
            double dwi, dwj, dwd;
            double wi = look(a, a.wh, d * hInv[i], dwi), wj = look(a, a.wh, d * hInv[j], dwj);
            MeFwd f;
            meFwd(r, d, rinv, v, I, J, wi, wj, a.avClean, etaCrit, f);
            meSums(v, J, f, e, ae);
            double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
            double vsp = rv < 0 ? a.c[i] + a.c[j] - 3.0 * rv / d : 0.0;
            if (vsp > vs) { vs = vsp; ag = j; }
            double CIr[3];
            symv(Cr_, r, CIr);
            double Wk = a.K * hInv[i] * hInv[i] * hInv[i] * wi;
            double fac = vol[j] * (a.divv[i] - a.divv[j]);
            for (int k = 0; k < 3; ++k) g[k] += fac * (-Wk * CIr[k]);
            for (int aa = 0; aa < 3; ++aa)
                for (int k = 0; k < 3; ++k) Pi[3 * aa + k] += a.xm[j] * wi * (-v[aa]) * r[k];
            double wd = look(a, a.whd, d * hInv[i], dwd);
            double dterh = -(3 * wi + d * hInv[i] * wd);
            so += a.xm[j] * dterh;
            sr += a.m[j] * dterh;
        }
        en[i] = e; avE[i] = ae; vsig[i] = vs; arg[i] = ag;
        for (int k = 0; k < 3; ++k) G[3 * i + k] = g[k];
        for (int k = 0; k < 9; ++k) P[9 * i + k] = Pi[k];
        double h4 = a.K * std::pow(hInv[i], 4);
        wom[i] = h4 * so; wr0[i] = h4 * sr;
    }
    // accumulators
    std::vector<double> prhoB(n), cB(n), alphaB(n), rhoB(n), xmB(n), kxB(n), CB(6 * n), gB(6 * n), divvB(n), gradhB(n);
    double *bx = a.gx, *by = a.gy, *bz = a.gz, *bvx = a.gvx, *bvy = a.gvy, *bvz = a.gvz, *bh = a.gh, *bu = a.gu;
    for (int64_t i = 0; i < n; ++i) { bx[i] = by[i] = bz[i] = bvx[i] = bvy[i] = bvz[i] = bh[i] = bu[i] = 0; }
    // ME
    for (int64_t i = 0; i < n; ++i) {
        double mb[3] = {-a.K * a.sAx[i], -a.K * a.sAy[i], -a.K * a.sAz[i]};
        double enb = a.K * a.prho[i] * a.sDu[i];
        double avEb = avE[i] >= 0 ? 0.5 * a.K * a.sDu[i] : 0.0;
        prhoB[i] += a.K * en[i] * a.sDu[i];
        rhoB[i] += a.sRho[i];
        MeSide I = side(i);
        int64_t cnt = a.off[i + 1] - a.off[i];
        double etaCrit = std::cbrt(32.0 * M_PI / 3.0 / double(cnt + 1));
        for (int64_t q = a.off[i]; q < a.off[i + 1]; ++q) {
            int64_t j = a.idx[q];
            double r[3], d, rinv;
            pairR(a, i, j, r, d, rinv);
            double v[3] = {a.vx[i] - a.vx[j], a.vy[i] - a.vy[j], a.vz[i] - a.vz[j]};
            MeSide J = side(j);
            double dwi, dwj;
            double wi = look(a, a.wh, d * hInv[i], dwi), wj = look(a, a.wh, d * hInv[j], dwj);
            MeGrad o;
            bool mutual = false;
            if (mutualMode && !a.avClean)
                for (int64_t q2 = a.off[j]; q2 < a.off[j + 1]; ++q2) mutual |= a.idx[q2] == i;
            if (mutual && i > j) continue;  // evaluated by j
            if (mutual) {
                double mbJ[3] = {-a.K * a.sAx[j], -a.K * a.sAy[j], -a.K * a.sAz[j]};
                double enbJ = a.K * a.prho[j] * a.sDu[j];
                double avEbJ = avE[j] >= 0 ? 0.5 * a.K * a.sDu[j] : 0.0;
                meAdjMutual<true>(r, d, rinv, v, I, J, wi, dwi, wj, dwj, mb, enb, avEb, mbJ, enbJ, avEbJ, o);
            }
            else if (a.avClean) meAdj<true, true>(r, d, rinv, v, I, J, wi, dwi, wj, dwj, etaCrit, mb, enb, avEb, o);
            else meAdj<false, true>(r, d, rinv, v, I, J, wi, dwi, wj, dwj, etaCrit, mb, enb, avEb, o);
            bx[i] += o.r[0]; by[i] += o.r[1]; bz[i] += o.r[2];
            bx[j] -= o.r[0]; by[j] -= o.r[1]; bz[j] -= o.r[2];
            bvx[i] += o.v[0]; bvy[i] += o.v[1]; bvz[i] += o.v[2];
            bvx[j] -= o.v[0]; bvy[j] -= o.v[1]; bvz[j] -= o.v[2];
            bh[i] += o.hI; bh[j] += o.hJ;
            cB[i] += o.c; cB[j] += o.c; alphaB[i] += o.alpha; alphaB[j] += o.alpha;
            prhoB[i] += o.prhoI; prhoB[j] += o.prhoJ; rhoB[i] += o.rhoI; rhoB[j] += o.rhoJ;
            xmB[i] += o.xmI; xmB[j] += o.xmJ;
            for (int t = 0; t < 6; ++t) { CB[6 * i + t] += o.CI[t]; CB[6 * j + t] += o.CJ[t]; gB[6 * i + t] += o.gI[t]; gB[6 * j + t] += o.gJ[t]; }
        }
    }
    // AV
    AvPrm avp{a.K, a.dt, a.amin, a.amax, a.decay};
    std::vector<double> GB(3 * n), vsigB(n);
    for (int64_t i = 0; i < n; ++i) {
        double hb, db, cb;
        avSeed(avp, alphaB[i], a.alpha0[i], a.h[i], a.c[i], a.divv[i], &G[3 * i], vsig[i], &GB[3 * i], vsigB[i], hb, db, cb);
        bh[i] += hb; divvB[i] += db; cB[i] += cb;
        if (arg[i] < 0) cB[i] += 1e-40 * vsigB[i];
    }
    for (int64_t i = 0; i < n; ++i) {
        double Ci[6];
        for (int q = 0; q < 6; ++q) Ci[q] = a.C[q][i];
        double CGb[3], R[3] = {0, 0, 0};
        symv(Ci, &GB[3 * i], CGb);
        for (int64_t q = a.off[i]; q < a.off[i + 1]; ++q) {
            int64_t j = a.idx[q];
            double r[3], d, rinv;
            pairR(a, i, j, r, d, rinv);
            double v[3] = {a.vx[i] - a.vx[j], a.vy[i] - a.vy[j], a.vz[i] - a.vz[j]};
            double dwi;
            double wi = look(a, a.wh, d * hInv[i], dwi);
            AvGrad o;
            avAdj(r, d, rinv, v, hInv[i], wi, dwi, a.K, vol[j], 1.0 / a.kx[j], a.divv[i], a.divv[j], CGb,
                  vsigB[i], j == arg[i], o);
            for (int t = 0; t < 3; ++t) R[t] += o.R[t];
            bx[i] += o.r[0]; by[i] += o.r[1]; bz[i] += o.r[2];
            bx[j] -= o.r[0]; by[j] -= o.r[1]; bz[j] -= o.r[2];
            bvx[i] += o.v[0]; bvy[i] += o.v[1]; bvz[i] += o.v[2];
            bvx[j] -= o.v[0]; bvy[j] -= o.v[1]; bvz[j] -= o.v[2];
            cB[i] += o.cI; cB[j] += o.cJ; bh[i] += o.hI; divvB[i] += o.divvI; divvB[j] += o.divvJ;
            xmB[j] += o.xmJ; kxB[j] += o.kxJ;
        }
        avCbar(&GB[3 * i], R, &CB[6 * i]);
    }
    // IAD + divv
    std::vector<double> TB(6 * n), PBv(9 * n);
    for (int64_t i = 0; i < n; ++i) {
        double Ci[6];
        for (int q = 0; q < 6; ++q) Ci[q] = a.C[q][i];
        double hb = 0, kb = 0;
        iadDivvSeed(a.K, a.h[i], a.kx[i], Ci, &CB[6 * i], divvB[i], &gB[6 * i], &P[9 * i], &TB[6 * i], &PBv[9 * i], hb, kb);
        bh[i] += hb; kxB[i] += kb;
    }
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t q = a.off[i]; q < a.off[i + 1]; ++q) {
            int64_t j = a.idx[q];
            double r[3], d, rinv;
            pairR(a, i, j, r, d, rinv);
            double v[3] = {a.vx[i] - a.vx[j], a.vy[i] - a.vy[j], a.vz[i] - a.vz[j]};
            double dwi;
            double wi = look(a, a.wh, d * hInv[i], dwi);
            IadGrad o;
            iadDivvAdj(r, d, rinv, v, hInv[i], wi, dwi, vol[j], 1.0 / a.kx[j], a.xm[j], &TB[6 * i], &PBv[9 * i], o);
            bx[i] += o.r[0]; by[i] += o.r[1]; bz[i] += o.r[2];
            bx[j] -= o.r[0]; by[j] -= o.r[1]; bz[j] -= o.r[2];
            bvx[i] += o.v[0]; bvy[i] += o.v[1]; bvz[i] += o.v[2];
            bvx[j] -= o.v[0]; bvy[j] -= o.v[1]; bvz[j] -= o.v[2];
            bh[i] += o.hI; xmB[j] += o.xmJ; kxB[j] += o.kxJ;
        }
    }
    // EOS
    for (int64_t i = 0; i < n; ++i)
        eosAdj(a.gamma, a.u[i], a.m[i], a.kx[i], a.xm[i], a.gradh[i], a.c[i], prhoB[i], cB[i], rhoB[i], kxB[i], xmB[i],
               gradhB[i], bu[i]);
    // gradh
    std::vector<double> Sk(n), So(n), Sr(n);
    for (int64_t i = 0; i < n; ++i) {
        double hb = 0, xb = 0;
        gradhSeed(a.K, a.h[i], a.m[i], a.xm[i], a.kx[i], wom[i], wr0[i], kxB[i], gradhB[i], Sk[i], So[i], Sr[i], hb, xb);
        bh[i] += hb; xmB[i] += xb;
    }
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t q = a.off[i]; q < a.off[i + 1]; ++q) {
            int64_t j = a.idx[q];
            double r[3], d, rinv;
            pairR(a, i, j, r, d, rinv);
            double dwi, dwd;
            double wi = look(a, a.wh, d * hInv[i], dwi), wd = look(a, a.whd, d * hInv[i], dwd);
            GradhGrad o;
            gradhAdj(r, d, rinv, hInv[i], wi, dwi, wd, dwd, a.xm[j], a.m[j], Sk[i], So[i], Sr[i], o);
            bx[i] += o.r[0]; by[i] += o.r[1]; bz[i] += o.r[2];
            bx[j] -= o.r[0]; by[j] -= o.r[1]; bz[j] -= o.r[2];
            bh[i] += o.hI; xmB[j] += o.xmJ;
        }
    }
    // xmass
    std::vector<double> R0b(n);
    for (int64_t i = 0; i < n; ++i) {
        double hb = 0;
        xmassSeed(a.K, a.h[i], a.m[i], a.xm[i], xmB[i], R0b[i], hb);
        bh[i] += hb;
    }
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t q = a.off[i]; q < a.off[i + 1]; ++q) {
            int64_t j = a.idx[q];
            double r[3], d, rinv;
            pairR(a, i, j, r, d, rinv);
            double dwi;
            look(a, a.wh, d * hInv[i], dwi);
            double rb[3], hIb;
            xmassAdj(r, d, rinv, hInv[i], dwi, a.m[j], R0b[i], rb, hIb);
            bx[i] += rb[0]; by[i] += rb[1]; bz[i] += rb[2];
            bx[j] -= rb[0]; by[j] -= rb[1]; bz[j] -= rb[2];
            bh[i] += hIb;
        }
    }
    return 0;
}
