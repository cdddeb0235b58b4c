// Host driver of the std adjoint arithmetic (sphexa_gb300/csrc/adjoint_std.cuh): the device pass
// sequence of the std adjoint (adjoint.cu) as sequential loops over a CSR neighbour list, to check
// the functions the kernels call against torch autograd on the CPU.  Test infrastructure; built by
// tests/test_adjoint_host.py with g++.  mutualMode = 1 evaluates a pair whose ends list each other
// once through the combined momentum-energy function (the form the device uses with owned lists).
#include <cmath>
#include <cstdint>
#include <vector>

#include "adjoint_std.cuh"
using namespace sphgb::stdad;
struct In {
    int64_t n;
    const double *x, *y, *z, *vx, *vy, *vz, *h, *u, *m, *rho, *p, *c;
    const double* C[6];
    const int64_t *off, *idx;
    const double* wh;
    int64_t ntab;
    double K, gamma, L[3];
    int pbc[3];
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
        if (a.pbc[k]) { if (r[k] > th) r[k] -= a.L[k]; else if (r[k] < -th) r[k] += a.L[k]; }
    }
    d = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    rinv = 1.0 / d;
}
extern "C" int std_adj_host(const In* ap, int mutualMode)
{
    const In& a = *ap;
    int64_t n = a.n;
    auto side = [&](int64_t i) {
        MeSide<> s;
        s.hInv = 1.0 / a.h[i]; s.c = a.c[i]; s.m = a.m[i]; s.rhoInv = 1.0 / a.rho[i];
        s.poR = a.p[i] / a.rho[i]; s.poR2 = a.p[i] / (a.rho[i] * a.rho[i]);
        for (int q = 0; q < 6; ++q) s.C[q] = a.C[q][i];
        return s;
    };
    double *bx = a.gx, *by = a.gy, *bz = a.gz, *bvx = a.gvx, *bvy = a.gvy, *bvz = a.gvz, *bh = a.gh, *bu = a.gu;
    for (int64_t i = 0; i < n; ++i) bx[i] = by[i] = bz[i] = bvx[i] = bvy[i] = bvz[i] = bh[i] = bu[i] = 0;
    std::vector<double> rhoB(n), pB(n), cB(n), CB(6 * n);
    auto seeds = [&](int64_t i, double gA[3], double& gE) {
        gA[0] = a.K * a.sAx[i]; gA[1] = a.K * a.sAy[i]; gA[2] = a.K * a.sAz[i]; gE = -0.5 * a.K * a.sDu[i];
    };
    for (int64_t i = 0; i < n; ++i) {
        rhoB[i] += a.sRho[i];
        MeSide<> I = side(i);
        double gAi[3], gEi;
        seeds(i, gAi, gEi);
        for (int64_t q = a.off[i]; q < a.off[i + 1]; ++q) {
            int64_t j = a.idx[q];
            bool mutual = false;
            if (mutualMode)
                for (int64_t q2 = a.off[j]; q2 < a.off[j + 1]; ++q2) mutual |= a.idx[q2] == i;
            if (mutual && i > j) continue;
            double gAj[3] = {0, 0, 0}, gEj = 0;
            if (mutual) seeds(j, gAj, gEj);
            double r[3], d, rinv;
            pairR(a, i, j, r, d, rinv);
            double v[3] = {a.vx[i] - a.vx[j], a.vy[i] - a.vy[j], a.vz[i] - a.vz[j]};
            MeSide<> J = side(j);
            double dwi, dwj;
            double wi = look(a, a.wh, d * I.hInv, dwi), wj = look(a, a.wh, d * J.hInv, dwj);
            MeGrad<> o;
            meStdAdjPair(r, d, rinv, v, I, J, wi, dwi, wj, dwj, gAi, gEi, gAj, gEj, o);
            bx[i] += o.r[0]; by[i] += o.r[1]; bz[i] += o.r[2];
            bx[j] -= o.r[0]; by[j] -= o.r[1]; bz[j] -= o.r[2];
            bvx[i] += o.v[0]; bvy[i] += o.v[1]; bvz[i] += o.v[2];
            bvx[j] -= o.v[0]; bvy[j] -= o.v[1]; bvz[j] -= o.v[2];
            bh[i] += o.hI; bh[j] += o.hJ; rhoB[i] += o.rhoI; rhoB[j] += o.rhoJ; pB[i] += o.pI; pB[j] += o.pJ;
            cB[i] += o.c; cB[j] += o.c;
            for (int t = 0; t < 6; ++t) { CB[6 * i + t] += o.CI[t]; CB[6 * j + t] += o.CJ[t]; }
        }
    }
    std::vector<double> TB(6 * n);
    for (int64_t i = 0; i < n; ++i) {
        double C[6];
        for (int q = 0; q < 6; ++q) C[q] = a.C[q][i];
        iadSeed(a.K, a.h[i], C, &CB[6 * i], &TB[6 * i], bh[i]);
    }
    for (int64_t i = 0; i < n; ++i)
        for (int64_t q = a.off[i]; q < a.off[i + 1]; ++q) {
            int64_t j = a.idx[q];
            double r[3], d, rinv, dwi;
            pairR(a, i, j, r, d, rinv);
            double wi = look(a, a.wh, d / a.h[i], dwi);
            double rb[3], hIb, rhoJb;
            iadAdjTerm(r, d, rinv, 1.0 / a.h[i], wi, dwi, a.m[j] / a.rho[j], 1.0 / a.rho[j], &TB[6 * i], rb, hIb, rhoJb);
            bx[i] += rb[0]; by[i] += rb[1]; bz[i] += rb[2];
            bx[j] -= rb[0]; by[j] -= rb[1]; bz[j] -= rb[2];
            bh[i] += hIb; rhoB[j] += rhoJb;
        }
    for (int64_t i = 0; i < n; ++i) {
        double g1 = a.gamma - 1.0;
        rhoB[i] += pB[i] * g1 * a.u[i];
        bu[i] = pB[i] * g1 * a.rho[i] + (a.c[i] > 0 ? cB[i] * a.gamma * g1 / (2.0 * a.c[i]) : 0.0);
    }
    for (int64_t i = 0; i < n; ++i) {
        bh[i] += rhoB[i] * (-3.0 * a.rho[i] / a.h[i]);
        for (int64_t q = a.off[i]; q < a.off[i + 1]; ++q) {
            int64_t j = a.idx[q];
            double r[3], d, rinv, dwi;
            pairR(a, i, j, r, d, rinv);
            look(a, a.wh, d / a.h[i], dwi);
            double rb[3], hIb;
            densityAdjTerm(r, d, rinv, 1.0 / a.h[i], dwi, a.m[j], a.K, rhoB[i], rb, hIb);
            bx[i] += rb[0]; by[i] += rb[1]; bz[i] += rb[2];
            bx[j] -= rb[0]; by[j] -= rb[1]; bz[j] -= rb[2];
            bh[i] += hIb;
        }
    }
    return 0;
}
