// Reverse-mode arithmetic of the standard SPH chain density -> EOS -> IAD -> momentum-energy, one
// pair or one particle at a time: pure functions shared by the device kernels (adjoint.cu) and
// host-side checks.  The pair functions take the arithmetic type T: double for the FP64 form, float
// for the mixed form (the caller accumulates their results in FP64).  Conventions as in
// adjoint_ve.cuh: pair (i, j) of i's list, r = x_i - x_j (legacy fold at 2 h_i), d = |r|,
// v = v_i - v_j, w / dw the table interpolant and its slope.
//
// Forward formulas (reference j-loops):
//   rho_i = K h_i^-3 (m_i + sum_j m_j w(d / h_i))                       hydro_std/density.hpp:41-60
//   p = (gamma-1) rho u, c = sqrt(gamma (gamma-1) u)                   hydro_std/eos.hpp:54-80
//   C_i = tau_i^-1 h_i^3 / K, tau_i = sum_j (m_j/rho_j) w r r^T         hydro_std/iad_kern.hpp:12-77
//   a_i = K sum_j (alpha A_i + beta A_j), du_i = -K/2 sum_j v.(alpha' A_i + beta' A_j), A = C r
//   alpha = W_i (q_i + visc s_i), beta = t_j W_j (u_j + visc), alpha' = W_i (2 q_i + visc s_i),
//   beta' = visc t_j W_j, q_i = m_j p_i / rho_i^2, s_i = m_i / rho_i, t_j = m_j / rho_j,
//   u_j = p_j / rho_j                                                 hydro_std/momentum_energy_kern.hpp:12-134
#pragma once

#include "adjoint_ve.cuh"

namespace sphgb {
namespace stdad {

template<class T>
VEAD_HD void symv(const T C[6], const T r[3], T o[3])
{
    o[0] = C[0] * r[0] + C[1] * r[1] + C[2] * r[2];
    o[1] = C[1] * r[0] + C[3] * r[1] + C[4] * r[2];
    o[2] = C[2] * r[0] + C[4] * r[1] + C[5] * r[2];
}

// Cb += s * d(a . C r) / dC
template<class T>
VEAD_HD void symvAdj(const T a[3], const T r[3], T s, T Cb[6])
{
    Cb[0] += s * (a[0] * r[0]);
    Cb[1] += s * (a[0] * r[1] + a[1] * r[0]);
    Cb[2] += s * (a[0] * r[2] + a[2] * r[0]);
    Cb[3] += s * (a[1] * r[1]);
    Cb[4] += s * (a[1] * r[2] + a[2] * r[1]);
    Cb[5] += s * (a[2] * r[2]);
}

// d(h^-3 w(d/h))/dh with v = d/h
template<class T>
VEAD_HD T dWdh(T hInv, T w, T dw, T v)
{
    return -hInv * hInv * hInv * hInv * (T(3) * w + v * dw);
}

template<class T = double>
struct MeSide {
    T hInv, c, m, rhoInv, poR, poR2;  // poR = p / rho, poR2 = p / rho^2
    T C[6];
};

template<class T = double>
struct MeGrad {
    T r[3], v[3], c;         // r: x_i += , x_j -= ; v: v_i += , v_j -= ; c: both ends
    T hI, rhoI, pI, CI[6];   // i's fields
    T hJ, rhoJ, pJ, CJ[6];   // j's fields
};

// Both momentum-energy terms of one pair: i's term with seeds gAi = K abar_i, gEi = -K/2 dubar_i,
// and j's term of the same pair (r -> -r, v -> -v, roles swapped) with gAj, gEj.  With r_ji = -r
// every intermediate is shared: the pair's part of L is Ui . A_i + Uj . A_j with the seed vectors
//   Ui = alpha gAi - beta2 gAj + (gEi alpha' + gEj beta2') v,  Uj = beta gAi - alpha2 gAj + (gEi beta' + gEj alpha2') v
// (alpha2 = W_j (q_j + visc t_j), beta2 = s_i W_i (u_i + visc), alpha2' = W_j (2 q_j + visc t_j),
//  beta2' = visc s_i W_i are j's coefficients).  Zero j seeds give i's term alone.
template<class T>
VEAD_HD void meStdAdjPair(const T r[3], T d, T rinv, const T v[3], const MeSide<T>& I, const MeSide<T>& J, T wi, T dwi,
                          T wj, T dwj, const T gAi[3], T gEi, const T gAj[3], T gEj, MeGrad<T>& o)
{
    const T v1 = d * I.hInv, v2 = d * J.hInv;
    const T hi3 = I.hInv * I.hInv * I.hInv, hj3 = J.hInv * J.hInv * J.hInv;
    const T Wi = hi3 * wi, Wj = hj3 * wj;
    T Ai[3], Aj[3];
    symv<T>(I.C, r, Ai);
    symv<T>(J.C, r, Aj);
    const T rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    const T W = rv * rinv;
    const T cs = I.c + J.c;
    const bool approaching = W < T(0);
    const T visc = approaching ? T(0.5) * (-(T(0.5) * cs - T(2) * W) * W) : T(0);
    const T qi = J.m * I.poR2, si = I.m * I.rhoInv, tj = J.m * J.rhoInv, uj = J.poR;
    const T qj = I.m * J.poR2, ui = I.poR;
    const T alpha = Wi * (qi + visc * si), beta = tj * Wj * (uj + visc);
    const T alphaP = Wi * (T(2) * qi + visc * si), betaP = visc * tj * Wj;
    const T alpha2 = Wj * (qj + visc * tj), beta2 = si * Wi * (ui + visc);
    const T alphaP2 = Wj * (T(2) * qj + visc * tj), betaP2 = visc * si * Wi;

    T Ui[3], Uj[3];
    T aI = 0, bI = 0, aJ = 0, bJ = 0, vAi = 0, vAj = 0;
    for (int k = 0; k < 3; ++k) {
        Ui[k] = alpha * gAi[k] - beta2 * gAj[k] + (gEi * alphaP + gEj * betaP2) * v[k];
        Uj[k] = beta * gAi[k] - alpha2 * gAj[k] + (gEi * betaP + gEj * alphaP2) * v[k];
        aI += gAi[k] * Ai[k];
        bI += gAi[k] * Aj[k];
        aJ += gAj[k] * Aj[k];
        bJ += gAj[k] * Ai[k];
        vAi += v[k] * Ai[k];
        vAj += v[k] * Aj[k];
    }
    // adjoints of the scalar coefficients
    const T bAlpha = aI, bBeta = bI, bAlpha2 = -aJ, bBeta2 = -bJ;
    const T bAlphaP = gEi * vAi, bBetaP = gEi * vAj, bAlphaP2 = gEj * vAj, bBetaP2 = gEj * vAi;
    const T bWi = bAlpha * (qi + visc * si) + bAlphaP * (T(2) * qi + visc * si) + bBeta2 * si * (ui + visc) +
                  bBetaP2 * visc * si;
    const T bWj = bBeta * tj * (uj + visc) + bBetaP * visc * tj + bAlpha2 * (qj + visc * tj) +
                  bAlphaP2 * (T(2) * qj + visc * tj);
    const T bqi = (bAlpha + T(2) * bAlphaP) * Wi, bqj = (bAlpha2 + T(2) * bAlphaP2) * Wj;
    const T bsi = (bAlpha + bAlphaP) * Wi * visc + bBeta2 * Wi * (ui + visc) + bBetaP2 * visc * Wi;
    const T btj = bBeta * Wj * (uj + visc) + bBetaP * visc * Wj + (bAlpha2 + bAlphaP2) * Wj * visc;
    const T buj = bBeta * tj * Wj, bui = bBeta2 * si * Wi;
    const T bVisc = (bAlpha + bAlphaP) * Wi * si + (bBeta + bBetaP) * tj * Wj + (bAlpha2 + bAlphaP2) * Wj * tj +
                    (bBeta2 + bBetaP2) * si * Wi;

    // particle fields
    o.pI = bqi * J.m * I.rhoInv * I.rhoInv + bui * I.rhoInv;
    o.rhoI = (bqi * (T(-2) * qi) + bsi * (-si) + bui * (-ui)) * I.rhoInv;
    o.pJ = buj * J.rhoInv + bqj * I.m * J.rhoInv * J.rhoInv;
    o.rhoJ = (btj * (-tj) + buj * (-uj) + bqj * (T(-2) * qj)) * J.rhoInv;
    // viscosity
    T bW = 0;
    o.c = 0;
    if (approaching) {
        bW = bVisc * (T(-0.25) * cs + T(2) * W);
        o.c = bVisc * (T(-0.25) * W);
    }
    const T brv = bW * rinv;
    T db = -bW * W * rinv;
    for (int k = 0; k < 3; ++k) {
        o.r[k] = brv * v[k];
        o.v[k] = brv * r[k] + gEi * (alphaP * Ai[k] + betaP * Aj[k]) + gEj * (alphaP2 * Aj[k] + betaP2 * Ai[k]);
    }
    // A = C r
    for (int q = 0; q < 6; ++q) o.CI[q] = o.CJ[q] = 0;
    symvAdj<T>(Ui, r, T(1), o.CI);
    symvAdj<T>(Uj, r, T(1), o.CJ);
    T CUi[3], CUj[3];
    symv<T>(I.C, Ui, CUi);
    symv<T>(J.C, Uj, CUj);
    // W = h^-3 w(d / h)
    o.hI = bWi * dWdh<T>(I.hInv, wi, dwi, v1);
    o.hJ = bWj * dWdh<T>(J.hInv, wj, dwj, v2);
    db += bWi * hi3 * dwi * I.hInv + bWj * hj3 * dwj * J.hInv;
    for (int k = 0; k < 3; ++k) o.r[k] += CUi[k] + CUj[k] + db * r[k] * rinv;
}

// per particle: C = s tau^-1, s = h^3 / K: the symmetric tau adjoint tauB = -s M G M (M = C / s, G
// the symmetric gradient of C from Cb) and h's partial from s
VEAD_HD void iadSeed(double K, double h, const double C[6], const double Cb[6], double tauB[6], double& hb)
{
    const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    const double s = h * h * h / K;
    double M[3][3], G[3][3];
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 3; ++q) {
            M[a][q] = C[idx[a][q]] / s;
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

// i's IAD term V_j w(d / h_i) r r^T (V_j = m_j / rho_j) with i's tau adjoint: partials of r, h_i, rho_j
template<class T>
VEAD_HD void iadAdjTerm(const T r[3], T d, T rinv, T hiInv, T wi, T dwi, T Vj, T rhoInvJ, const T tauB[6], T rb[3],
                        T& hIb, T& rhoJb)
{
    T Tr[3];
    symv<T>(tauB, r, Tr);
    const T Q = r[0] * Tr[0] + r[1] * Tr[1] + r[2] * Tr[2];
    for (int k = 0; k < 3; ++k) rb[k] = Vj * (T(2) * wi * Tr[k] + Q * dwi * hiInv * r[k] * rinv);
    hIb = -Vj * Q * dwi * d * hiInv * hiInv;
    rhoJb = -(Vj * rhoInvJ) * wi * Q;
}

// i's density term K h_i^-3 m_j w(d / h_i) with rhob_i: partials of r and h_i (the pair part; the
// factor h_i^-3 enters per particle)
template<class T>
VEAD_HD void densityAdjTerm(const T r[3], T d, T rinv, T hiInv, T dwi, T mj, T K, T rhob, T rb[3], T& hIb)
{
    const T hi3 = hiInv * hiInv * hiInv;
    const T f = rhob * K * hi3 * mj * dwi * hiInv * rinv;
    for (int k = 0; k < 3; ++k) rb[k] = f * r[k];
    hIb = -rhob * K * hi3 * mj * dwi * d * hiInv * hiInv;
}

}  // namespace stdad
}  // namespace sphgb
