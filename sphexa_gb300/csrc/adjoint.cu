// Adjoint (reverse mode) of the standard SPH chain  density -> EOS -> IAD -> momentum-energy
// over the frozen neighbour lists of the last search, FP64 and mixed (FP32 pair arithmetic).
//
// Forward functions differentiated (reference j-loops):
//   rho_i = K h_i^-3 (m_i + sum_j m_j w(r_ij / h_i))                 hydro_std/density.hpp:41-60
//   p_i = (gamma-1) rho_i u_i,  c_i = sqrt(gamma (gamma-1) u_i)      hydro_std/eos.hpp:54-80
//   C_i = tau_i^-1 h_i^3 / K,  tau_i = sum_j (m_j/rho_j) w r r^T       hydro_std/iad_kern.hpp:12-77
//   a_i = K sum_j (alpha A_i + beta A_j),  du_i = -K/2 sum_j v_ij.(alpha' A_i + beta' A_j)
//                                                                    hydro_std/momentum_energy_kern.hpp:12-134
// w is the table interpolant (sph/include/sph/table_lookup.hpp:10-26) and its derivative is the
// slope of the interval, so forward and adjoint describe the same piecewise function.  The
// Courant time step is not differentiated.
//
// Three walks of the pairs, no per-pair value stored:
//   deterministic (FP64): every pair (i owns the list, j is the neighbour) is evaluated twice, once
//     by thread i over its list for the partials of i's quantities and once by thread j over the
//     transposed list for the partials of j's quantities; each thread writes only its own particle,
//     so the sums are bit-reproducible;
//   once (FP64, and the mixed momentum-energy term): one evaluation per owned entry of the owned
//     lists, a mutual pair giving both directed terms, the neighbour's partials by atomics;
//   scatter (the mixed IAD and density terms, FP64 with a deterministic context): every list entry
//     evaluated by its owner, the neighbour's partials by atomics.
#include "adjoint_std.cuh"
#include "pairs.cuh"

namespace sphgb {

namespace {

constexpr int kAdjBlock = 128;

// kernel function value and derivative dw/dv at v, on the interval the forward passes select (from
// the bits of v / dx): the slope of the linear interpolant, or the derivative of the cubic piece in
// the smooth form
template<bool Smooth>
__device__ __forceinline__ double lookupSlope(const KTab<Smooth>& tab, double v, double& slope)
{
    return lookupVSlope(tab, v, slope);
}

// the table a kernel reads, with the kernel form of its instantiation (FP64) or as it is (FP32)
template<bool Smooth>
__device__ __forceinline__ KTab<Smooth> kernelTab(const double2* t)
{
    return {t};
}
template<bool Smooth>
__device__ __forceinline__ const float2* kernelTab(const float2* t)
{
    return t;
}

struct AdjArgs {
    // forward state
    const double *x, *y, *z, *vx, *vy, *vz, *h, *m, *u, *rho, *p, *c;
    const double *c11, *c12, *c13, *c22, *c23, *c33;
    const double2* wh;  // W in the context's form (the kernels' Smooth argument tells which)
    double K, gamma;
    DevBox box;
    // lists: own (transposed layout) and incoming (CSR by neighbour)
    ListView lv;
    const uint32_t* tOff;
    const uint32_t* tIdx;
    int64_t n;
    // seeds
    const double *sRho, *sAx, *sAy, *sAz, *sDu;
    // per-particle adjoint state
    double *bx, *by, *bz, *bvx, *bvy, *bvz, *bh, *bu;  // outputs
    double *bRho, *bP, *bC, *bCij;                      // bCij: 6 x n
    double* tauBar;                                     // 6 x n
    // per-particle quotients formed once: 1/h, m/rho, p/rho, 1/rho, p/rho^2
    const double *hInv, *mOverRho, *pOverRho, *rhoInv, *pOverRho2;
};

struct Side {
    double x, y, z, vx, vy, vz, h, hInv, m, moR, poR, rInv, poR2, c, C[6];
};

__device__ __forceinline__ Side loadSide(const AdjArgs& a, int64_t i)
{
    Side s;
    s.x = a.x[i];
    s.y = a.y[i];
    s.z = a.z[i];
    s.vx = a.vx[i];
    s.vy = a.vy[i];
    s.vz = a.vz[i];
    s.h = a.h[i];
    s.hInv = a.hInv[i];
    s.m = a.m[i];
    s.moR = a.mOverRho[i];
    s.poR = a.pOverRho[i];
    s.rInv = a.rhoInv[i];
    s.poR2 = a.pOverRho2[i];
    s.c = a.c[i];
    s.C[0] = a.c11[i];
    s.C[1] = a.c12[i];
    s.C[2] = a.c13[i];
    s.C[3] = a.c22[i];
    s.C[4] = a.c23[i];
    s.C[5] = a.c33[i];
    return s;
}

// the fields the IAD and density reverse passes read of a particle
__device__ __forceinline__ Side loadPos(const AdjArgs& a, int64_t i)
{
    Side s;
    s.x = a.x[i];
    s.y = a.y[i];
    s.z = a.z[i];
    s.h = a.h[i];
    s.hInv = a.hInv[i];
    s.m = a.m[i];
    s.moR = a.mOverRho[i];
    s.rInv = a.rhoInv[i];
    return s;
}

// r = x_i - x_j with the legacy periodic fold at 2 h_i (box.hpp:216-238)
__device__ __forceinline__ void pairR(const DevBox& b, const Side& I, const Side& J, double r[3])
{
    const long long twoHBits = __double_as_longlong(2.0 * I.h);
    const double d[3] = {I.x - J.x, I.y - J.y, I.z - J.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = b.pbc[k] ? CoordFp64::wrapLegacy(d[k], twoHBits, b.L[k]) : d[k];
}

__device__ __forceinline__ void symv(const double C[6], const double r[3], double out[3])
{
    out[0] = C[0] * r[0] + C[1] * r[1] + C[2] * r[2];
    out[1] = C[1] * r[0] + C[3] * r[1] + C[4] * r[2];
    out[2] = C[2] * r[0] + C[4] * r[1] + C[5] * r[2];
}

// gradient of the stored components of a symmetric C from A = C r and Abar
__device__ __forceinline__ void symvAdj(const double Ab[3], const double r[3], double Cb[6])
{
    Cb[0] += Ab[0] * r[0];
    Cb[1] += Ab[0] * r[1] + Ab[1] * r[0];
    Cb[2] += Ab[0] * r[2] + Ab[2] * r[0];
    Cb[3] += Ab[1] * r[1];
    Cb[4] += Ab[1] * r[2] + Ab[2] * r[1];
    Cb[5] += Ab[2] * r[2];
}

// partials of one momentum-energy pair term of i (list owner) with neighbour j, given the seeds
// gA = K abar_i and gE = -K/2 dubar_i.  Output for the side selected by ForI.
struct PairGrad {
    double r[3], v[3], c;                 // dS/dr (r = x_i - x_j), dS/dv_ij, dS/dc_i = dS/dc_j
    double hI, rhoI, pI, CI[6];           // partials of i's fields (WantI)
    double hJ, rhoJ, pJ, CJ[6];           // partials of j's fields (WantJ)
};

template<bool WantI, bool WantJ, bool Smooth>
__device__ __forceinline__ void mePairAdj(const DevBox& b, const KTab<Smooth>& tab, const Side& I, const Side& J,
                                          const double gA[3], double gE, PairGrad& g)
{
    double r[3];
    pairR(b, I, J, r);
    const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    const double rinv = rsqrt(r2), d = r2 * rinv;
    const double v[3] = {I.vx - J.vx, I.vy - J.vy, I.vz - J.vz};
    const double v1 = d * I.hInv, v2 = d * J.hInv;
    double dwi, dwj;
    const double wi = lookupSlope(tab, v1, dwi), wj = lookupSlope(tab, v2, dwj);
    const double hi3 = I.hInv * I.hInv * I.hInv, hj3 = J.hInv * J.hInv * J.hInv;
    const double Wi = hi3 * wi, Wj = hj3 * wj;
    double Ai[3], Aj[3];
    symv(I.C, r, Ai);
    symv(J.C, r, Aj);
    const double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    const double W = rv * rinv;
    const double cs = I.c + J.c;
    const bool approaching = negative(W);
    const double visc = approaching ? 0.5 * (-(0.5 * cs - 2.0 * W) * W) : 0.0;
    const double qi = J.m * I.poR2, si = I.moR, tj = J.moR, uj = J.poR;
    const double alpha = Wi * (qi + visc * si), beta = tj * Wj * (uj + visc);
    const double alphaP = Wi * (2.0 * qi + visc * si), betaP = visc * tj * Wj;

    const double vAi = v[0] * Ai[0] + v[1] * Ai[1] + v[2] * Ai[2];
    const double vAj = v[0] * Aj[0] + v[1] * Aj[1] + v[2] * Aj[2];
    const double bAlpha = gA[0] * Ai[0] + gA[1] * Ai[1] + gA[2] * Ai[2];
    const double bBeta = gA[0] * Aj[0] + gA[1] * Aj[1] + gA[2] * Aj[2];
    const double bAlphaP = gE * vAi, bBetaP = gE * vAj;

    double Abi[3], Abj[3], vb[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        Abi[k] = gA[k] * alpha + gE * alphaP * v[k];
        Abj[k] = gA[k] * beta + gE * betaP * v[k];
        vb[k] = gE * (alphaP * Ai[k] + betaP * Aj[k]);
    }
    const double bWi = bAlpha * (qi + visc * si) + bAlphaP * (2.0 * qi + visc * si);
    const double bqi = (bAlpha + 2.0 * bAlphaP) * Wi;
    const double bsi = (bAlpha + bAlphaP) * Wi * visc;
    const double bVisc = (bAlpha + bAlphaP) * Wi * si + (bBeta + bBetaP) * tj * Wj;
    const double btj = bBeta * Wj * (uj + visc) + bBetaP * visc * Wj;
    const double bWj = bBeta * tj * (uj + visc) + bBetaP * visc * tj;
    const double buj = bBeta * tj * Wj;

    double bW = 0.0, bcs = 0.0;
    if (approaching) {
        bW = bVisc * 0.5 * (-0.5 * cs + 4.0 * W);
        bcs = bVisc * 0.5 * (-0.5 * W);
    }
    double rb[3];
    const double bd = bWi * hi3 * dwi * I.hInv + bWj * hj3 * dwj * J.hInv;
    double CAi[3], CAj[3];
    symv(I.C, Abi, CAi);
    symv(J.C, Abj, CAj);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        rb[k] = bW * rinv * (v[k] - W * r[k] * rinv) + CAi[k] + CAj[k] + bd * r[k] * rinv;
        vb[k] += bW * r[k] * rinv;
    }
    for (int k = 0; k < 3; ++k) {
        g.r[k] = rb[k];
        g.v[k] = vb[k];
    }
    g.c = bcs;
    if constexpr (WantI) {
        for (int q = 0; q < 6; ++q) g.CI[q] = 0.0;
        g.hI = bWi * (-I.hInv * hi3 * (3.0 * wi + v1 * dwi));
        g.pI = bqi * J.m * I.rInv * I.rInv;
        g.rhoI = (bqi * (-2.0 * qi) + bsi * (-si)) * I.rInv;
        symvAdj(Abi, r, g.CI);
    }
    if constexpr (WantJ) {
        for (int q = 0; q < 6; ++q) g.CJ[q] = 0.0;
        g.hJ = bWj * (-J.hInv * hj3 * (3.0 * wj + v2 * dwj));
        g.pJ = buj * J.rInv;
        g.rhoJ = (btj * (-tj) + buj * (-uj)) * J.rInv;
        symvAdj(Abj, r, g.CJ);
    }
}

// seeds of the pair terms of list owner i: gA = K abar_i, gE = -K/2 dubar_i
__device__ __forceinline__ bool seedsOf(const AdjArgs& a, int64_t i, double gA[3], double& gE)
{
    gA[0] = a.sAx ? a.K * a.sAx[i] : 0.0;
    gA[1] = a.sAy ? a.K * a.sAy[i] : 0.0;
    gA[2] = a.sAz ? a.K * a.sAz[i] : 0.0;
    gE = a.sDu ? -0.5 * a.K * a.sDu[i] : 0.0;
    return gA[0] != 0.0 || gA[1] != 0.0 || gA[2] != 0.0 || gE != 0.0;
}

template<bool Smooth>
__global__ void __launch_bounds__(kAdjBlock) meAdjKernel(AdjArgs a)
{
    const auto tab = kernelTab<Smooth>(a.wh);
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    const Side S = loadSide(a, k);
    double bx[3] = {0, 0, 0}, bv[3] = {0, 0, 0}, bh = 0, brho = 0, bp = 0, bc = 0, bC[6] = {0, 0, 0, 0, 0, 0};
    // k as list owner
    {
        double gA[3], gE;
        if (seedsOf(a, k, gA, gE)) {
            const unsigned nc = a.lv.capped(k);
            for (unsigned q = 0; q < nc; ++q) {
                const Side J = loadSide(a, a.lv.at(k, q));
                PairGrad g;
                mePairAdj<true, false>(a.box, tab, S, J, gA, gE, g);
                for (int t = 0; t < 3; ++t) {
                    bx[t] += g.r[t];
                    bv[t] += g.v[t];
                }
                bh += g.hI;
                brho += g.rhoI;
                bp += g.pI;
                bc += g.c;
                for (int t = 0; t < 6; ++t) bC[t] += g.CI[t];
            }
        }
    }
    // k as neighbour of i
    for (uint32_t e = a.tOff[k]; e < a.tOff[k + 1]; ++e) {
        const int64_t i = a.tIdx[e];
        double gA[3], gE;
        if (!seedsOf(a, i, gA, gE)) continue;
        const Side I = loadSide(a, i);
        PairGrad g;
        mePairAdj<false, true>(a.box, tab, I, S, gA, gE, g);
        for (int t = 0; t < 3; ++t) {
            bx[t] -= g.r[t];
            bv[t] -= g.v[t];
        }
        bh += g.hJ;
        brho += g.rhoJ;
        bp += g.pJ;
        bc += g.c;
        for (int t = 0; t < 6; ++t) bC[t] += g.CJ[t];
    }
    a.bx[k] = bx[0];
    a.by[k] = bx[1];
    a.bz[k] = bx[2];
    a.bvx[k] = bv[0];
    a.bvy[k] = bv[1];
    a.bvz[k] = bv[2];
    a.bh[k] = bh;
    a.bRho[k] = brho + (a.sRho ? a.sRho[k] : 0.0);
    a.bP[k] = bp;
    a.bC[k] = bc;
    for (int t = 0; t < 6; ++t) a.bCij[t * a.n + k] = bC[t];
}

// tau_bar = -s M G M with M = C / s, s = h^3 / K, G the symmetric gradient of C;
// s_bar = G : M  -> h_bar += s_bar 3 h^2 / K
__global__ void iadPrepKernel(AdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    const double h = a.h[k], s = h * h * h / a.K;
    const double C[6] = {a.c11[k], a.c12[k], a.c13[k], a.c22[k], a.c23[k], a.c33[k]};
    double Mf[3][3], G[3][3];
    const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) {
            int t = idx[r][q];
            Mf[r][q] = C[t] / s;
            double cb = a.bCij[t * a.n + k];
            G[r][q] = (r == q) ? cb : 0.5 * cb;
        }
    double MG[3][3], T[3][3];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) {
            MG[r][q] = Mf[r][0] * G[0][q] + Mf[r][1] * G[1][q] + Mf[r][2] * G[2][q];
        }
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) T[r][q] = -s * (MG[r][0] * Mf[0][q] + MG[r][1] * Mf[1][q] + MG[r][2] * Mf[2][q]);
    double sb = 0.0;
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) sb += G[r][q] * Mf[r][q];
    a.bh[k] += sb * 3.0 * h * h / a.K;
    a.tauBar[0 * a.n + k] = T[0][0];
    a.tauBar[1 * a.n + k] = 0.5 * (T[0][1] + T[1][0]);
    a.tauBar[2 * a.n + k] = 0.5 * (T[0][2] + T[2][0]);
    a.tauBar[3 * a.n + k] = T[1][1];
    a.tauBar[4 * a.n + k] = 0.5 * (T[1][2] + T[2][1]);
    a.tauBar[5 * a.n + k] = T[2][2];
}

__device__ __forceinline__ double quadTau(const AdjArgs& a, int64_t i, const double r[3], double Tr[3])
{
    const double t11 = a.tauBar[i], t12 = a.tauBar[a.n + i], t13 = a.tauBar[2 * a.n + i];
    const double t22 = a.tauBar[3 * a.n + i], t23 = a.tauBar[4 * a.n + i], t33 = a.tauBar[5 * a.n + i];
    Tr[0] = t11 * r[0] + t12 * r[1] + t13 * r[2];
    Tr[1] = t12 * r[0] + t22 * r[1] + t23 * r[2];
    Tr[2] = t13 * r[0] + t23 * r[1] + t33 * r[2];
    return r[0] * Tr[0] + r[1] * Tr[1] + r[2] * Tr[2];
}

// tau_i += V_j w(d/h_i) r r^T, V_j = m_j / rho_j
template<bool Smooth>
__global__ void __launch_bounds__(kAdjBlock) iadAdjKernel(AdjArgs a)
{
    const auto tab = kernelTab<Smooth>(a.wh);
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    const Side S = loadPos(a, k);
    double bx[3] = {0, 0, 0}, bh = 0, brho = 0;
    {
        const unsigned nc = a.lv.capped(k);
        for (unsigned q = 0; q < nc; ++q) {
            const int64_t j = a.lv.at(k, q);
            const Side J = loadPos(a, j);
            double r[3], Tr[3];
            pairR(a.box, S, J, r);
            const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            const double rinv = rsqrt(r2), d = r2 * rinv;
            double dw;
            const double w = lookupSlope(tab, d * S.hInv, dw);
            const double Q = quadTau(a, k, r, Tr);
            const double V = J.moR;
            for (int t = 0; t < 3; ++t) bx[t] += V * (2.0 * w * Tr[t] + Q * dw * S.hInv * r[t] * rinv);
            bh += -V * Q * dw * d * S.hInv * S.hInv;
        }
    }
    for (uint32_t e = a.tOff[k]; e < a.tOff[k + 1]; ++e) {
        const int64_t i = a.tIdx[e];
        const Side I = loadPos(a, i);
        double r[3], Tr[3];
        pairR(a.box, I, S, r);
        const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        const double rinv = rsqrt(r2), d = r2 * rinv;
        double dw;
        const double w = lookupSlope(tab, d * I.hInv, dw);
        const double Q = quadTau(a, i, r, Tr);
        const double V = S.moR;
        for (int t = 0; t < 3; ++t) bx[t] -= V * (2.0 * w * Tr[t] + Q * dw * I.hInv * r[t] * rinv);
        brho += -(V * S.rInv) * w * Q;
    }
    a.bx[k] += bx[0];
    a.by[k] += bx[1];
    a.bz[k] += bx[2];
    a.bh[k] += bh;
    a.bRho[k] += brho;
}

// p = (gamma-1) rho u, c = sqrt(gamma (gamma-1) u)
__global__ void eosAdjKernel(AdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    const double g1 = a.gamma - 1.0;
    const double u = a.u[k], rho = a.rho[k], c = a.c[k];
    a.bRho[k] += a.bP[k] * g1 * u;
    a.bu[k] = a.bP[k] * g1 * rho + (c > 0.0 ? a.bC[k] * a.gamma * g1 / (2.0 * c) : 0.0);
}

// rho_i = K h_i^-3 (m_i + sum_j m_j w(d/h_i))
template<bool Smooth>
__global__ void __launch_bounds__(kAdjBlock) densityAdjKernel(AdjArgs a)
{
    const auto tab = kernelTab<Smooth>(a.wh);
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    const Side S = loadPos(a, k);
    double bx[3] = {0, 0, 0};
    const double brk = a.bRho[k];
    const double hi3 = S.hInv * S.hInv * S.hInv;
    double bh = brk * (-3.0 * a.rho[k] * S.hInv);
    {
        const unsigned nc = a.lv.capped(k);
        double sdw = 0.0;
        for (unsigned q = 0; q < nc; ++q) {
            const int64_t j = a.lv.at(k, q);
            double r[3];
            const Side J = loadPos(a, j);
            pairR(a.box, S, J, r);
            const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            const double rinv = rsqrt(r2), d = r2 * rinv;
            double dw;
            lookupSlope(tab, d * S.hInv, dw);
            const double f = brk * a.K * hi3 * J.m * dw * S.hInv * rinv;
            for (int t = 0; t < 3; ++t) bx[t] += f * r[t];
            sdw += J.m * dw * d;
        }
        bh += brk * a.K * hi3 * sdw * (-S.hInv * S.hInv);
    }
    for (uint32_t e = a.tOff[k]; e < a.tOff[k + 1]; ++e) {
        const int64_t i = a.tIdx[e];
        const Side I = loadPos(a, i);
        double r[3];
        pairR(a.box, I, S, r);
        const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        const double rinv = rsqrt(r2), d = r2 * rinv;
        double dw;
        lookupSlope(tab, d * I.hInv, dw);
        const double hI3 = I.hInv * I.hInv * I.hInv;
        const double f = a.bRho[i] * a.K * hI3 * S.m * dw * I.hInv * rinv;
        (void)d;
        for (int t = 0; t < 3; ++t) bx[t] -= f * r[t];
    }
    a.bx[k] += bx[0];
    a.by[k] += bx[1];
    a.bz[k] += bx[2];
    a.bh[k] += bh;
}

// ---- scatter form over the full lists, in the pair arithmetic of either precision ----
// Every list entry is evaluated by its owner; the neighbour's partials go by FP64 atomics.  T is
// the arithmetic of the pairs: double (FP64 form, with the context in deterministic mode) or float
// (mixed form: FP64 coordinate differences rounded once, FP32 pair arithmetic, the table interval
// of the mixed forward); every accumulation is FP64.
template<class T>
struct TabOf {
    using type = const double2*;
};
template<>
struct TabOf<float> {
    using type = const float2*;
};

template<bool Smooth>
__device__ __forceinline__ double lookupSlopeT(const KTab<Smooth>& tab, double v, double& slope)
{
    return lookupSlope(tab, v, slope);
}

// FP32 interval of the 20000-entry linear table that the FP64 passes interpolate: k = int(v / dx),
// value and slope of that interval (the mixed forward's cubic pieces agree with it to ~1e-8)
__device__ __forceinline__ float lookupSlopeT(const float2* __restrict__ tab, float v, float& slope)
{
    constexpr int nInt = kTableSize - 1;
    const float x = v * float(kTabInvDx);
    const int k = int(x);
    if (k >= nInt) {
        slope = 0.f;
        return 0.f;
    }
    const float2 t = __ldg(tab + k);
    slope = t.y * float(kTabInvDx);
    return fmaf(t.y, x - float(k), t.x);
}

template<class T>
struct StdScatterArgs {
    const double *x, *y, *z, *u;
    const T *vx, *vy, *vz, *h, *m, *rho, *p, *c;
    const T* C[6];
    typename TabOf<T>::type wh;  // FP64: W in the context's form; FP32: the linear table
    double K, gamma;
    DevBox box;
    ListView lv;
    int64_t n;
    const T *sRho, *sAx, *sAy, *sAz;
    const double* sDu;
    // adjoints, accumulated in the pair type: the FP64 form writes the caller's gradients and FP64
    // state, the mixed form FP32 arrays (converted to the FP64 gradients at the end)
    T *bx, *by, *bz, *bvx, *bvy, *bvz, *bh, *bu;
    T *bRho, *bP, *bC, *bCij, *tauBar;
    T *hInv, *moR, *poR, *rhoInv, *poR2;  // per-particle quotients in the pair type
    CoordMixed cm;                         // mixed form: the grid-form coordinates of the forward passes
};

template<class T>
__global__ void stdQuotKernel(StdScatterArgs<T> a)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.n) return;
    const double rho = double(a.rho[i]), p = double(a.p[i]);
    a.hInv[i] = T(1.0 / double(a.h[i]));
    a.moR[i] = T(double(a.m[i]) / rho);
    a.poR[i] = T(p / rho);
    a.rhoInv[i] = T(1.0 / rho);
    a.poR2[i] = T(p / (rho * rho));
}

template<class T>
__device__ __forceinline__ stdad::MeSide<T> stdSideT(const StdScatterArgs<T>& a, int64_t i)
{
    stdad::MeSide<T> s;
    s.hInv = a.hInv[i];
    s.c = a.c[i];
    s.m = a.m[i];
    s.rhoInv = a.rhoInv[i];
    s.poR = a.poR[i];
    s.poR2 = a.poR2[i];
#pragma unroll
    for (int q = 0; q < 6; ++q) s.C[q] = a.C[q][i];
    return s;
}

// r = x_i - x_j as the forward passes of that form take it: FP64 differences with the legacy fold
// at 2 h_i, or (mixed) the FP32 grid form (integer cell difference times the cell edge plus the
// in-cell offsets, the minimum image across periodic faces)
template<class T>
__device__ __forceinline__ void geomT(const StdScatterArgs<T>& a, int64_t i, int64_t j, T r[3], T& d, T& rinv)
{
    if constexpr (std::is_same_v<T, double>) {
        const long long twoHBits = __double_as_longlong(2.0 * a.h[i]);
        const double dd[3] = {a.x[i] - a.x[j], a.y[i] - a.y[j], a.z[i] - a.z[j]};
#pragma unroll
        for (int k = 0; k < 3; ++k) r[k] = a.box.pbc[k] ? CoordFp64::wrapLegacy(dd[k], twoHBits, a.box.L[k]) : dd[k];
        const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        rinv = rsqrt(r2);
        d = r2 * rinv;
    } else {
        float hjInv;
        a.cm.diff(a.cm.target(i), j, r[0], r[1], r[2], hjInv);
        const float r2 = fmaf(r[0], r[0], fmaf(r[1], r[1], r[2] * r[2]));
        rinv = rsqrtf(r2);
        d = r2 * rinv;
    }
}

template<class T, bool Smooth>
__global__ void __launch_bounds__(kAdjBlock) meAdjScatterT(StdScatterArgs<T> a)
{
    const auto tab = kernelTab<Smooth>(a.wh);
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    const T gA[3] = {a.sAx ? T(a.K * double(a.sAx[k])) : T(0), a.sAy ? T(a.K * double(a.sAy[k])) : T(0),
                     a.sAz ? T(a.K * double(a.sAz[k])) : T(0)};
    const T gE = a.sDu ? T(-0.5 * a.K * a.sDu[k]) : T(0);
    T bx[3] = {0, 0, 0}, bv[3] = {0, 0, 0}, bh = 0, brho = 0, bp = 0, bc = 0, bC[6] = {0, 0, 0, 0, 0, 0};
    if (gA[0] != T(0) || gA[1] != T(0) || gA[2] != T(0) || gE != T(0)) {
        const stdad::MeSide<T> S = stdSideT(a, k);
        const T zero[3] = {T(0), T(0), T(0)};
        const unsigned nc = a.lv.capped(k);
        for (unsigned q = 0; q < nc; ++q) {
            const int64_t j = a.lv.at(k, q);
            const stdad::MeSide<T> J = stdSideT(a, j);
            T r[3], d, rinv;
            geomT(a, k, j, r, d, rinv);
            const T v[3] = {a.vx[k] - a.vx[j], a.vy[k] - a.vy[j], a.vz[k] - a.vz[j]};
            T dwi, dwj;
            const T wi = lookupSlopeT(tab, d * S.hInv, dwi), wj = lookupSlopeT(tab, d * J.hInv, dwj);
            stdad::MeGrad<T> o;
            stdad::meStdAdjPair<T>(r, d, rinv, v, S, J, wi, dwi, wj, dwj, gA, gE, zero, T(0), o);
            for (int t = 0; t < 3; ++t) {
                bx[t] += o.r[t];
                bv[t] += o.v[t];
            }
            bh += o.hI;
            brho += o.rhoI;
            bp += o.pI;
            bc += o.c;
            for (int t = 0; t < 6; ++t) bC[t] += o.CI[t];
            atomicAdd(a.bx + j, -o.r[0]);
            atomicAdd(a.by + j, -o.r[1]);
            atomicAdd(a.bz + j, -o.r[2]);
            atomicAdd(a.bvx + j, -o.v[0]);
            atomicAdd(a.bvy + j, -o.v[1]);
            atomicAdd(a.bvz + j, -o.v[2]);
            atomicAdd(a.bh + j, o.hJ);
            atomicAdd(a.bRho + j, o.rhoJ);
            atomicAdd(a.bP + j, o.pJ);
            atomicAdd(a.bC + j, o.c);
            for (int t = 0; t < 6; ++t) atomicAdd(a.bCij + t * a.n + j, o.CJ[t]);
        }
    }
    atomicAdd(a.bx + k, bx[0]);
    atomicAdd(a.by + k, bx[1]);
    atomicAdd(a.bz + k, bx[2]);
    atomicAdd(a.bvx + k, bv[0]);
    atomicAdd(a.bvy + k, bv[1]);
    atomicAdd(a.bvz + k, bv[2]);
    atomicAdd(a.bh + k, bh);
    atomicAdd(a.bRho + k, brho + (a.sRho ? a.sRho[k] : T(0)));
    atomicAdd(a.bP + k, bp);
    atomicAdd(a.bC + k, bc);
    for (int t = 0; t < 6; ++t) atomicAdd(a.bCij + t * a.n + k, bC[t]);
}

template<class T>
__global__ void iadPrepT(StdScatterArgs<T> a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double C[6], Cb[6], tauB[6], hb = 0.0;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        C[q] = double(a.C[q][k]);
        Cb[q] = double(a.bCij[q * a.n + k]);
    }
    stdad::iadSeed(a.K, double(a.h[k]), C, Cb, tauB, hb);
    a.bh[k] += T(hb);
#pragma unroll
    for (int q = 0; q < 6; ++q) a.tauBar[q * a.n + k] = T(tauB[q]);
}

template<class T, bool Smooth>
__global__ void __launch_bounds__(kAdjBlock) iadAdjScatterT(StdScatterArgs<T> a)
{
    const auto tab = kernelTab<Smooth>(a.wh);
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    T tauB[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) tauB[q] = a.tauBar[q * a.n + k];
    const T hInv = a.hInv[k];
    T bx[3] = {0, 0, 0}, bh = 0;
    const unsigned nc = a.lv.capped(k);
    for (unsigned q = 0; q < nc; ++q) {
        const int64_t j = a.lv.at(k, q);
        T r[3], d, rinv, dw;
        geomT(a, k, j, r, d, rinv);
        const T w = lookupSlopeT(tab, d * hInv, dw);
        T rb[3], hIb, rhoJb;
        stdad::iadAdjTerm<T>(r, d, rinv, hInv, w, dw, a.moR[j], a.rhoInv[j], tauB, rb, hIb, rhoJb);
        for (int t = 0; t < 3; ++t) bx[t] += rb[t];
        bh += hIb;
        atomicAdd(a.bx + j, -rb[0]);
        atomicAdd(a.by + j, -rb[1]);
        atomicAdd(a.bz + j, -rb[2]);
        atomicAdd(a.bRho + j, rhoJb);
    }
    atomicAdd(a.bx + k, bx[0]);
    atomicAdd(a.by + k, bx[1]);
    atomicAdd(a.bz + k, bx[2]);
    atomicAdd(a.bh + k, bh);
}

// p = (gamma-1) rho u, c = sqrt(gamma (gamma-1) u)
template<class T>
__global__ void eosAdjT(StdScatterArgs<T> a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    const double g1 = a.gamma - 1.0;
    const double u = a.u[k], rho = double(a.rho[k]), c = double(a.c[k]), bp = double(a.bP[k]);
    a.bRho[k] += T(bp * g1 * u);
    a.bu[k] = T(bp * g1 * rho + (c > 0.0 ? double(a.bC[k]) * a.gamma * g1 / (2.0 * c) : 0.0));
}

// the mixed form's FP32 gradients to the caller's FP64 arrays
__global__ void gradsToDouble(int64_t n, const float* __restrict__ src, double* x, double* y, double* z, double* vx,
                              double* vy, double* vz, double* h, double* u)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    double* dst[8] = {x, y, z, vx, vy, vz, h, u};
#pragma unroll
    for (int k = 0; k < 8; ++k) dst[k][i] = double(src[k * n + i]);
}

template<class T, bool Smooth>
__global__ void __launch_bounds__(kAdjBlock) densityAdjScatterT(StdScatterArgs<T> a)
{
    const auto tab = kernelTab<Smooth>(a.wh);
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    const T rhob = a.bRho[k];
    const T hInv = a.hInv[k];
    T bx[3] = {0, 0, 0}, bh = rhob * (T(-3) * a.rho[k] * hInv);
    const unsigned nc = a.lv.capped(k);
    for (unsigned q = 0; q < nc; ++q) {
        const int64_t j = a.lv.at(k, q);
        T r[3], d, rinv, dw;
        geomT(a, k, j, r, d, rinv);
        lookupSlopeT(tab, d * hInv, dw);
        T rb[3], hIb;
        stdad::densityAdjTerm<T>(r, d, rinv, hInv, dw, a.m[j], T(a.K), rhob, rb, hIb);
        for (int t = 0; t < 3; ++t) bx[t] += rb[t];
        bh += hIb;
        atomicAdd(a.bx + j, -rb[0]);
        atomicAdd(a.by + j, -rb[1]);
        atomicAdd(a.bz + j, -rb[2]);
    }
    atomicAdd(a.bx + k, bx[0]);
    atomicAdd(a.by + k, bx[1]);
    atomicAdd(a.bz + k, bx[2]);
    atomicAdd(a.bh + k, bh);
}

// seeds of particle k in the pair type: K times the acceleration seeds and -K/2 times the du seed;
// false when they are all zero
template<class T>
__device__ __forceinline__ bool seedsOfT(const StdScatterArgs<T>& a, int64_t k, T gA[3], T& gE)
{
    gA[0] = a.sAx ? T(a.K * double(a.sAx[k])) : T(0);
    gA[1] = a.sAy ? T(a.K * double(a.sAy[k])) : T(0);
    gA[2] = a.sAz ? T(a.K * double(a.sAz[k])) : T(0);
    gE = a.sDu ? T(-0.5 * a.K * a.sDu[k]) : T(0);
    return gA[0] != T(0) || gA[1] != T(0) || gA[2] != T(0) || gE != T(0);
}

// the momentum-energy adjoint of the mixed form over owned lists: one evaluation per owned entry,
// a mutual pair's entry giving both directed terms (the neighbour's through its own seeds), as the
// FP64 meAdjOnceKernel; the grid-form geometry is antisymmetric (r_ji = -r_ij exactly), so the one
// evaluation equals the two of the scatter form.  Half the pair evaluations and atomics of
// meAdjScatterT.
template<class T, bool Smooth>
__global__ void __launch_bounds__(kAdjBlock) meAdjOnceT(StdScatterArgs<T> a, OwnedView ov)
{
    const auto tab = kernelTab<Smooth>(a.wh);
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    T gA[3], gE;
    const bool anyK = seedsOfT(a, k, gA, gE);
    T bx[3] = {0, 0, 0}, bv[3] = {0, 0, 0}, bh = 0, brho = 0, bp = 0, bc = 0, bC[6] = {0, 0, 0, 0, 0, 0};
    const stdad::MeSide<T> S = stdSideT(a, k);
    const T zero[3] = {T(0), T(0), T(0)};
    const unsigned cnt = ov.size(k);
    for (unsigned q = 0; q < cnt; ++q) {
        bool mutual;
        const uint32_t j = ov.at(k, q, mutual);
        T gAj[3] = {T(0), T(0), T(0)}, gEj = T(0);
        const bool anyJ = mutual && seedsOfT(a, j, gAj, gEj);
        if (!anyK && !anyJ) continue;
        const stdad::MeSide<T> J = stdSideT(a, j);
        T r[3], d, rinv;
        geomT(a, k, j, r, d, rinv);
        const T v[3] = {a.vx[k] - a.vx[j], a.vy[k] - a.vy[j], a.vz[k] - a.vz[j]};
        T dwi, dwj;
        const T wi = lookupSlopeT(tab, d * S.hInv, dwi), wj = lookupSlopeT(tab, d * J.hInv, dwj);
        stdad::MeGrad<T> o;
        stdad::meStdAdjPair<T>(r, d, rinv, v, S, J, wi, dwi, wj, dwj, anyK ? gA : zero, anyK ? gE : T(0), gAj, gEj, o);
        for (int t = 0; t < 3; ++t) {
            bx[t] += o.r[t];
            bv[t] += o.v[t];
        }
        bh += o.hI;
        brho += o.rhoI;
        bp += o.pI;
        bc += o.c;
        for (int t = 0; t < 6; ++t) bC[t] += o.CI[t];
        atomicAdd(a.bx + j, -o.r[0]);
        atomicAdd(a.by + j, -o.r[1]);
        atomicAdd(a.bz + j, -o.r[2]);
        atomicAdd(a.bvx + j, -o.v[0]);
        atomicAdd(a.bvy + j, -o.v[1]);
        atomicAdd(a.bvz + j, -o.v[2]);
        atomicAdd(a.bh + j, o.hJ);
        atomicAdd(a.bRho + j, o.rhoJ);
        atomicAdd(a.bP + j, o.pJ);
        atomicAdd(a.bC + j, o.c);
        for (int t = 0; t < 6; ++t) atomicAdd(a.bCij + t * a.n + j, o.CJ[t]);
    }
    atomicAdd(a.bx + k, bx[0]);
    atomicAdd(a.by + k, bx[1]);
    atomicAdd(a.bz + k, bx[2]);
    atomicAdd(a.bvx + k, bv[0]);
    atomicAdd(a.bvy + k, bv[1]);
    atomicAdd(a.bvz + k, bv[2]);
    atomicAdd(a.bh + k, bh);
    atomicAdd(a.bRho + k, brho + (a.sRho ? a.sRho[k] : T(0)));
    atomicAdd(a.bP + k, bp);
    atomicAdd(a.bC + k, bc);
    for (int t = 0; t < 6; ++t) atomicAdd(a.bCij + t * a.n + k, bC[t]);
}

// ---- one evaluation per owned entry of the owned lists (mutual pairs give both directed terms) ----
__device__ __forceinline__ stdad::MeSide<> stdSide(const AdjArgs& a, int64_t i)
{
    stdad::MeSide<> s;
    s.hInv = a.hInv[i];
    s.c = a.c[i];
    s.m = a.m[i];
    s.rhoInv = a.rhoInv[i];
    s.poR = a.pOverRho[i];
    s.poR2 = a.pOverRho2[i];
    s.C[0] = a.c11[i];
    s.C[1] = a.c12[i];
    s.C[2] = a.c13[i];
    s.C[3] = a.c22[i];
    s.C[4] = a.c23[i];
    s.C[5] = a.c33[i];
    return s;
}

// r = x_i - x_j with the legacy periodic fold at 2 h_i, d = |r|
__device__ __forceinline__ void pairGeom(const AdjArgs& a, int64_t i, int64_t j, double r[3], double& d, double& rinv)
{
    const long long twoHBits = __double_as_longlong(2.0 * a.h[i]);
    const double dd[3] = {a.x[i] - a.x[j], a.y[i] - a.y[j], a.z[i] - a.z[j]};
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = a.box.pbc[k] ? CoordFp64::wrapLegacy(dd[k], twoHBits, a.box.L[k]) : dd[k];
    const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    rinv = rsqrt(r2);
    d = r2 * rinv;
}

template<bool Smooth>
__global__ void __launch_bounds__(kAdjBlock) meAdjOnceKernel(AdjArgs a, OwnedView ov)
{
    const auto tab = kernelTab<Smooth>(a.wh);
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double gA[3], gE;
    const bool anyK = seedsOf(a, k, gA, gE);
    double bx[3] = {0, 0, 0}, bv[3] = {0, 0, 0}, bh = 0, brho = 0, bp = 0, bc = 0, bC[6] = {0, 0, 0, 0, 0, 0};
    const stdad::MeSide<> S = stdSide(a, k);
    const unsigned cnt = ov.size(k);
    for (unsigned q = 0; q < cnt; ++q) {
        bool mutual;
        const uint32_t j = ov.at(k, q, mutual);
        double gAj[3] = {0.0, 0.0, 0.0}, gEj = 0.0;
        const bool anyJ = mutual && seedsOf(a, j, gAj, gEj);
        if (!anyK && !anyJ) continue;
        const stdad::MeSide<> J = stdSide(a, j);
        double r[3], d, rinv;
        pairGeom(a, k, j, r, d, rinv);
        const double v[3] = {a.vx[k] - a.vx[j], a.vy[k] - a.vy[j], a.vz[k] - a.vz[j]};
        double dwi, dwj;
        const double wi = lookupSlope(tab, d * S.hInv, dwi), wj = lookupSlope(tab, d * J.hInv, dwj);
        const double zero[3] = {0.0, 0.0, 0.0};
        stdad::MeGrad<> o;
        stdad::meStdAdjPair(r, d, rinv, v, S, J, wi, dwi, wj, dwj, anyK ? gA : zero, anyK ? gE : 0.0, gAj, gEj, o);
        for (int t = 0; t < 3; ++t) {
            bx[t] += o.r[t];
            bv[t] += o.v[t];
        }
        bh += o.hI;
        brho += o.rhoI;
        bp += o.pI;
        bc += o.c;
        for (int t = 0; t < 6; ++t) bC[t] += o.CI[t];
        atomicAdd(a.bx + j, -o.r[0]);
        atomicAdd(a.by + j, -o.r[1]);
        atomicAdd(a.bz + j, -o.r[2]);
        atomicAdd(a.bvx + j, -o.v[0]);
        atomicAdd(a.bvy + j, -o.v[1]);
        atomicAdd(a.bvz + j, -o.v[2]);
        atomicAdd(a.bh + j, o.hJ);
        atomicAdd(a.bRho + j, o.rhoJ);
        atomicAdd(a.bP + j, o.pJ);
        atomicAdd(a.bC + j, o.c);
        for (int t = 0; t < 6; ++t) atomicAdd(a.bCij + t * a.n + j, o.CJ[t]);
    }
    atomicAdd(a.bx + k, bx[0]);
    atomicAdd(a.by + k, bx[1]);
    atomicAdd(a.bz + k, bx[2]);
    atomicAdd(a.bvx + k, bv[0]);
    atomicAdd(a.bvy + k, bv[1]);
    atomicAdd(a.bvz + k, bv[2]);
    atomicAdd(a.bh + k, bh);
    atomicAdd(a.bRho + k, brho + (a.sRho ? a.sRho[k] : 0.0));
    atomicAdd(a.bP + k, bp);
    atomicAdd(a.bC + k, bc);
    for (int t = 0; t < 6; ++t) atomicAdd(a.bCij + t * a.n + k, bC[t]);
}

__device__ __forceinline__ void tauOf(const AdjArgs& a, int64_t i, double t[6])
{
#pragma unroll
    for (int q = 0; q < 6; ++q) t[q] = a.tauBar[q * a.n + i];
}

template<bool Smooth>
__global__ void __launch_bounds__(kAdjBlock) iadAdjOnceKernel(AdjArgs a, OwnedView ov)
{
    const auto tab = kernelTab<Smooth>(a.wh);
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double bx[3] = {0, 0, 0}, bh = 0, brho = 0, tauK[6];
    tauOf(a, k, tauK);
    const double hInvK = a.hInv[k], volK = a.mOverRho[k], rhoInvK = a.rhoInv[k];
    const unsigned cnt = ov.size(k);
    for (unsigned q = 0; q < cnt; ++q) {
        bool mutual;
        const uint32_t j = ov.at(k, q, mutual);
        double r[3], d, rinv, dw;
        pairGeom(a, k, j, r, d, rinv);
        double w = lookupSlope(tab, d * hInvK, dw);
        double rb[3], hIb, rhoJb;
        stdad::iadAdjTerm(r, d, rinv, hInvK, w, dw, a.mOverRho[j], a.rhoInv[j], tauK, rb, hIb, rhoJb);
        bh += hIb;
        if (mutual) {  // j's term of the same pair: r -> -r, roles swapped
            double tauJ[6];
            tauOf(a, j, tauJ);
            const double hInvJ = a.hInv[j];
            const double rm[3] = {-r[0], -r[1], -r[2]};
            w = lookupSlope(tab, d * hInvJ, dw);
            double pb[3], hJb, rhoKb;
            stdad::iadAdjTerm(rm, d, rinv, hInvJ, w, dw, volK, rhoInvK, tauJ, pb, hJb, rhoKb);
            for (int t = 0; t < 3; ++t) rb[t] -= pb[t];
            brho += rhoKb;
            atomicAdd(a.bh + j, hJb);
        }
        for (int t = 0; t < 3; ++t) bx[t] += rb[t];
        atomicAdd(a.bx + j, -rb[0]);
        atomicAdd(a.by + j, -rb[1]);
        atomicAdd(a.bz + j, -rb[2]);
        atomicAdd(a.bRho + j, rhoJb);
    }
    atomicAdd(a.bx + k, bx[0]);
    atomicAdd(a.by + k, bx[1]);
    atomicAdd(a.bz + k, bx[2]);
    atomicAdd(a.bh + k, bh);
    atomicAdd(a.bRho + k, brho);
}

template<bool Smooth>
__global__ void __launch_bounds__(kAdjBlock) densityAdjOnceKernel(AdjArgs a, OwnedView ov)
{
    const auto tab = kernelTab<Smooth>(a.wh);
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    const double rhobK = a.bRho[k], hInvK = a.hInv[k], mK = a.m[k];
    double bx[3] = {0, 0, 0}, bh = rhobK * (-3.0 * a.rho[k] * hInvK);
    const unsigned cnt = ov.size(k);
    for (unsigned q = 0; q < cnt; ++q) {
        bool mutual;
        const uint32_t j = ov.at(k, q, mutual);
        double r[3], d, rinv, dw;
        pairGeom(a, k, j, r, d, rinv);
        lookupSlope(tab, d * hInvK, dw);
        double rb[3], hIb;
        stdad::densityAdjTerm(r, d, rinv, hInvK, dw, a.m[j], a.K, rhobK, rb, hIb);
        bh += hIb;
        if (mutual) {
            const double hInvJ = a.hInv[j];
            const double rm[3] = {-r[0], -r[1], -r[2]};
            lookupSlope(tab, d * hInvJ, dw);
            double pb[3], hJb;
            stdad::densityAdjTerm(rm, d, rinv, hInvJ, dw, mK, a.K, a.bRho[j], pb, hJb);
            for (int t = 0; t < 3; ++t) rb[t] -= pb[t];
            atomicAdd(a.bh + j, hJb);
        }
        for (int t = 0; t < 3; ++t) bx[t] += rb[t];
        atomicAdd(a.bx + j, -rb[0]);
        atomicAdd(a.by + j, -rb[1]);
        atomicAdd(a.bz + j, -rb[2]);
    }
    atomicAdd(a.bx + k, bx[0]);
    atomicAdd(a.by + k, bx[1]);
    atomicAdd(a.bz + k, bx[2]);
    atomicAdd(a.bh + k, bh);
}

__global__ void adjQuotientsKernel(AdjArgs a, double* q)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    const double rho = a.rho[k], rInv = 1.0 / rho;
    q[k] = 1.0 / a.h[k];
    q[a.n + k] = a.m[k] / rho;
    q[2 * a.n + k] = a.p[k] / rho;
    q[3 * a.n + k] = rInv;
    q[4 * a.n + k] = a.p[k] / (rho * rho);
}

// ---- transposed lists: (j << 32 | i) keys sorted, CSR offsets by j ----
__global__ void pairKeysKernel(ListView lv, const uint32_t* __restrict__ off, u64* __restrict__ keys)
{
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last - lv.first) return;
    unsigned nc = lv.capped(i);
    uint64_t base = off[i];
    for (unsigned q = 0; q < nc; ++q) keys[base + q] = (u64(lv.at(i, q)) << 32) | u64(i);
}

__global__ void cappedCountKernel(ListView lv, uint32_t* __restrict__ cnt)
{
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < lv.last - lv.first) cnt[i] = lv.capped(i);
    else if (i == lv.last - lv.first) cnt[i] = 0;
}

__global__ void csrFromKeysKernel(const u64* __restrict__ keys, int64_t pairs, int64_t n, uint32_t* __restrict__ tOff,
                                  uint32_t* __restrict__ tIdx)
{
    int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (e < pairs) {
        u64 kk = keys[e];
        tIdx[e] = uint32_t(kk & 0xffffffffu);
        uint32_t j = uint32_t(kk >> 32);
        uint32_t jPrev = e == 0 ? 0xffffffffu : uint32_t(keys[e - 1] >> 32);
        if (j != jPrev) {
            // first entry of column j: also fill empty columns between jPrev and j
            uint32_t from = (e == 0) ? 0u : jPrev + 1;
            for (uint32_t q = from; q <= j; ++q) tOff[q] = uint32_t(e);
        }
        if (e == pairs - 1)
            for (int64_t q = int64_t(j) + 1; q <= n; ++q) tOff[q] = uint32_t(pairs);
    }
    if (pairs == 0 && e <= n) tOff[e] = 0;
}

}  // namespace

int buildTranspose(sphgb_ctx* c)
{
    if (c->transEpoch == c->nbrEpoch) return SPHGB_OK;
    ListView lv = listView(c);
    const int64_t nWork = lv.last - lv.first;
    // list entries are counted and sorted with 32-bit offsets
    if (nWork * int64_t(c->nbrNgmax) >= (int64_t(1) << 32)) return SPHGB_ERR_TOO_LARGE;
    SPHGB_TRY(c->splitCount.ensure(sizeof(uint32_t) * (nWork + 1)));
    SPHGB_TRY(c->splitOffset.ensure(sizeof(uint32_t) * (nWork + 1)));
    cappedCountKernel<<<gridFor(nWork + 1, 256), 256, 0, c->stream>>>(lv, c->splitCount.as<uint32_t>());
    SPHGB_TRY(launched(c, "cappedCountKernel"));
    SPHGB_TRY(exclusiveScan(c, c->splitCount.as<uint32_t>(), c->splitOffset.as<uint32_t>(), nWork + 1));
    uint32_t pairs32 = 0;
    SPHGB_CUDA(cudaMemcpyAsync(&pairs32, c->splitOffset.as<uint32_t>() + nWork, sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, c->stream));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    const int64_t pairs = pairs32;
    SPHGB_TRY(c->adjKeys.ensure(sizeof(u64) * (pairs + 1)));
    SPHGB_TRY(c->adjKeysAlt.ensure(sizeof(u64) * (pairs + 1)));
    SPHGB_TRY(c->tOff.ensure(sizeof(uint32_t) * (nWork + 1)));
    SPHGB_TRY(c->tIdx.ensure(sizeof(uint32_t) * (pairs + 1)));
    pairKeysKernel<<<gridFor(nWork, 256), 256, 0, c->stream>>>(lv, c->splitOffset.as<uint32_t>(),
                                                              c->adjKeysAlt.as<u64>());
    SPHGB_TRY(launched(c, "pairKeysKernel"));
    if (pairs > 0)  // keys (j << 32 | i) with j < 2^31: 63 bits
        SPHGB_TRY(radixSort(c, c->adjKeysAlt.as<u64>(), c->adjKeys.as<u64>(), nullptr, nullptr, pairs, 63));
    int64_t work = pairs > 0 ? pairs : nWork + 1;
    csrFromKeysKernel<<<gridFor(work, 256), 256, 0, c->stream>>>(c->adjKeys.as<u64>(), pairs, nWork,
                                                                c->tOff.as<uint32_t>(), c->tIdx.as<uint32_t>());
    SPHGB_TRY(launched(c, "csrFromKeysKernel"));
    SPHGB_TRY(sortStatusAsync(c));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    SPHGB_TRY(sortStatusAfterSync(c));
    c->transEpoch = c->nbrEpoch;
    c->transPairs = pairs;
    return SPHGB_OK;
}

// the scatter form in the pair arithmetic T (FP64 form in deterministic context mode, or mixed form)
template<class T>
static int adjointStdScatter(sphgb_ctx* c, sphgb_particles* p, const sphgb_seeds* s, sphgb_grads* g)
{
    const int64_t n = p->n;
    constexpr bool fp32 = std::is_same_v<T, float>;
    // state in T: rho, p, c adjoints, C adjoint (6), tau adjoint (6), quotients (5), and for the
    // mixed form the 8 gradients before their conversion to FP64
    SPHGB_TRY(c->adjState.ensure(sizeof(T) * (fp32 ? 28 : 20) * n));
    T* st = c->adjState.as<T>();
    StdScatterArgs<T> a{};
    auto f = [](const void* q) { return static_cast<const T*>(q); };
    a.x = p->x;
    a.y = p->y;
    a.z = p->z;
    a.u = p->u;
    a.vx = f(p->vx);
    a.vy = f(p->vy);
    a.vz = f(p->vz);
    a.h = f(p->h);
    a.m = f(p->m);
    a.rho = f(p->rho);
    a.p = f(p->p);
    a.c = f(p->c);
    const void* Cs[6] = {p->c11, p->c12, p->c13, p->c22, p->c23, p->c33};
    for (int q = 0; q < 6; ++q) a.C[q] = f(Cs[q]);
    if constexpr (std::is_same_v<T, double>) a.wh = tabW64(c);
    else a.wh = c->whx32.as<float2>();
    a.K = c->K;
    a.gamma = c->prm.gamma;
    a.box = c->box;
    a.lv = listView(c);
    a.n = n;
    if constexpr (fp32) a.cm = coordMixed(c);
    if (s) {
        a.sRho = f(s->rho);
        a.sAx = f(s->ax);
        a.sAy = f(s->ay);
        a.sAz = f(s->az);
        a.sDu = s->du;
    }
    a.bRho = st;
    a.bP = st + n;
    a.bC = st + 2 * n;
    a.bCij = st + 3 * n;
    a.tauBar = st + 9 * n;
    T* quot = st + 15 * n;
    a.hInv = quot;
    a.moR = quot + n;
    a.poR = quot + 2 * n;
    a.rhoInv = quot + 3 * n;
    a.poR2 = quot + 4 * n;
    if constexpr (fp32) {
        T* gr = st + 20 * n;
        a.bx = gr;
        a.by = gr + n;
        a.bz = gr + 2 * n;
        a.bvx = gr + 3 * n;
        a.bvy = gr + 4 * n;
        a.bvz = gr + 5 * n;
        a.bh = gr + 6 * n;
        a.bu = gr + 7 * n;
        SPHGB_CUDA(cudaMemsetAsync(gr, 0, sizeof(T) * 8 * n, c->stream));
    } else {
        a.bx = g->x;
        a.by = g->y;
        a.bz = g->z;
        a.bvx = g->vx;
        a.bvy = g->vy;
        a.bvz = g->vz;
        a.bh = g->h;
        a.bu = g->u;
        for (double* q : {g->x, g->y, g->z, g->vx, g->vy, g->vz, g->h})
            SPHGB_CUDA(cudaMemsetAsync(q, 0, sizeof(double) * n, c->stream));
    }
    SPHGB_CUDA(cudaMemsetAsync(st, 0, sizeof(T) * 9 * n, c->stream));
    if (fp32 && !c->deterministic && (c->ownedEpoch != c->nbrEpoch || !c->ownedFromLists))
        SPHGB_TRY(buildOwnedFromLists(c));
    const unsigned blocks = gridFor(n, kAdjBlock), eb = gridFor(n, 256);
    SPHGB_TRY(withKernelForm(c, [&](auto smooth) {
        constexpr bool S = !fp32 && decltype(smooth)::value;  // the FP32 form has one (linear) table
        stdQuotKernel<T><<<eb, 256, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "stdQuotKernel"));
        if (fp32 && !c->deterministic) {  // owned lists of the frozen lists: one evaluation per mutual pair
            meAdjOnceT<T, S><<<blocks, kAdjBlock, 0, c->stream>>>(a, ownedView(c));
            SPHGB_TRY(launched(c, "meAdjOnceT"));
        } else {
            meAdjScatterT<T, S><<<blocks, kAdjBlock, 0, c->stream>>>(a);
            SPHGB_TRY(launched(c, "meAdjScatterT"));
        }
        iadPrepT<T><<<eb, 256, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "iadPrepT"));
        iadAdjScatterT<T, S><<<blocks, kAdjBlock, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "iadAdjScatterT"));
        eosAdjT<T><<<eb, 256, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "eosAdjT"));
        densityAdjScatterT<T, S><<<blocks, kAdjBlock, 0, c->stream>>>(a);
        return launched(c, "densityAdjScatterT");
    }));
    if constexpr (fp32) {
        gradsToDouble<<<eb, 256, 0, c->stream>>>(n, st + 20 * n, g->x, g->y, g->z, g->vx, g->vy, g->vz, g->h, g->u);
        SPHGB_TRY(launched(c, "gradsToDouble"));
    }
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    return SPHGB_OK;
}

int adjointStd(sphgb_ctx* c, sphgb_particles* p, const sphgb_seeds* s, sphgb_grads* g, int deterministic)
{
    if (!c->haveNbr) return SPHGB_ERR_STATE;
    if (p->precision != SPHGB_FP64 && p->precision != SPHGB_MIXED) return SPHGB_ERR_ARG;
    if (c->nbrFirst != 0 || c->nbrLast != p->n) return SPHGB_ERR_ARG;
    if (!p->x || !p->y || !p->z || !p->vx || !p->vy || !p->vz || !p->h || !p->m || !p->u || !p->rho || !p->p ||
        !p->c || !p->c11 || !p->c12 || !p->c13 || !p->c22 || !p->c23 || !p->c33)
        return SPHGB_ERR_ARG;
    if (!g || !g->x || !g->y || !g->z || !g->vx || !g->vy || !g->vz || !g->h || !g->u) return SPHGB_ERR_ARG;
    if (p->precision == SPHGB_MIXED) {  // FP32 pair arithmetic, FP64 sums; scatter form only
        if (deterministic) return SPHGB_ERR_ARG;
        return adjointStdScatter<float>(c, p, s, g);
    }
    // one evaluation per mutual pair: owned lists of the current lists, order-free sums allowed
    const bool once = !deterministic && !c->deterministic && c->ownedEpoch == c->nbrEpoch && !c->ownedFromLists;
    if (!deterministic && !once) return adjointStdScatter<double>(c, p, s, g);
    const int64_t n = p->n;
    if (deterministic) SPHGB_TRY(buildTranspose(c));
    SPHGB_TRY(c->adjState.ensure(sizeof(double) * 20 * n));
    double* st = c->adjState.as<double>();

    AdjArgs a{};
    a.x = p->x;
    a.y = p->y;
    a.z = p->z;
    a.vx = static_cast<const double*>(p->vx);
    a.vy = static_cast<const double*>(p->vy);
    a.vz = static_cast<const double*>(p->vz);
    a.h = static_cast<const double*>(p->h);
    a.m = static_cast<const double*>(p->m);
    a.u = p->u;
    a.rho = static_cast<const double*>(p->rho);
    a.p = static_cast<const double*>(p->p);
    a.c = static_cast<const double*>(p->c);
    a.c11 = static_cast<const double*>(p->c11);
    a.c12 = static_cast<const double*>(p->c12);
    a.c13 = static_cast<const double*>(p->c13);
    a.c22 = static_cast<const double*>(p->c22);
    a.c23 = static_cast<const double*>(p->c23);
    a.c33 = static_cast<const double*>(p->c33);
    a.wh = tabW64(c);
    a.K = c->K;
    a.gamma = c->prm.gamma;
    a.box = c->box;
    a.lv = listView(c);
    a.tOff = c->tOff.as<uint32_t>();
    a.tIdx = c->tIdx.as<uint32_t>();
    a.n = n;
    if (s) {
        a.sRho = static_cast<const double*>(s->rho);
        a.sAx = static_cast<const double*>(s->ax);
        a.sAy = static_cast<const double*>(s->ay);
        a.sAz = static_cast<const double*>(s->az);
        a.sDu = s->du;
    }
    a.bx = g->x;
    a.by = g->y;
    a.bz = g->z;
    a.bvx = g->vx;
    a.bvy = g->vy;
    a.bvz = g->vz;
    a.bh = g->h;
    a.bu = g->u;
    a.bRho = st;
    a.bP = st + n;
    a.bC = st + 2 * n;
    a.bCij = st + 3 * n;
    a.tauBar = st + 9 * n;
    double* quot = st + 15 * n;
    a.hInv = quot;
    a.mOverRho = quot + n;
    a.pOverRho = quot + 2 * n;
    a.rhoInv = quot + 3 * n;
    a.pOverRho2 = quot + 4 * n;

    const unsigned blocks = gridFor(n, kAdjBlock);
    adjQuotientsKernel<<<gridFor(n, 256), 256, 0, c->stream>>>(a, quot);
    SPHGB_TRY(launched(c, "adjQuotientsKernel"));
    if (!deterministic) {
        // accumulators start at zero; every contribution arrives by atomic add
        for (double* q : {g->x, g->y, g->z, g->vx, g->vy, g->vz, g->h})
            SPHGB_CUDA(cudaMemsetAsync(q, 0, sizeof(double) * n, c->stream));
        SPHGB_CUDA(cudaMemsetAsync(st, 0, sizeof(double) * 9 * n, c->stream));
    }
    SPHGB_TRY(withKernelForm(c, [&](auto smooth) {
        constexpr bool S = decltype(smooth)::value;
        if (deterministic) meAdjKernel<S><<<blocks, kAdjBlock, 0, c->stream>>>(a);
        else meAdjOnceKernel<S><<<blocks, kAdjBlock, 0, c->stream>>>(a, ownedView(c));
        SPHGB_TRY(launched(c, "meAdjKernel"));
        iadPrepKernel<<<gridFor(n, 256), 256, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "iadPrepKernel"));
        if (deterministic) iadAdjKernel<S><<<blocks, kAdjBlock, 0, c->stream>>>(a);
        else iadAdjOnceKernel<S><<<blocks, kAdjBlock, 0, c->stream>>>(a, ownedView(c));
        SPHGB_TRY(launched(c, "iadAdjKernel"));
        eosAdjKernel<<<gridFor(n, 256), 256, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "eosAdjKernel"));
        if (deterministic) densityAdjKernel<S><<<blocks, kAdjBlock, 0, c->stream>>>(a);
        else densityAdjOnceKernel<S><<<blocks, kAdjBlock, 0, c->stream>>>(a, ownedView(c));
        return launched(c, "densityAdjKernel");
    }));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    return SPHGB_OK;
}

}  // namespace sphgb
