// Adjoint (reverse mode) of the volume-element SPH chain over the frozen neighbour lists of the
// last search, in FP64:
//   xmass -> kx/gradh -> EOS -> IAD + divv/curlv (+dV) -> AV switches -> momentum-energy<avClean>
// The arithmetic of one pair or one particle lives in adjoint_ve.cuh; this file holds the passes.
//
// Pass order (reverse of the forward):
//   quotients            1/h, rho = kx m/xm, xm/kx, ln xm
//   forward sums         en_i, avE_i (momentum-energy), G_i, vsig_i (AV), P_i (divv), S_om, S_r0 (gradh)
//   momentum-energy      pair partials -> x, v, h, prho, c, alpha, rho, xm, C, dV
//   AV switch            per particle (alpha -> G, vsig seeds), then pair partials
//   IAD + divv           per particle (C, divv, dV -> tau, P seeds), then pair partials
//   EOS                  per particle -> kx, xm, gradh, u
//   kx / gradh           per particle (-> sum seeds), then pair partials
//   xmass                per particle, then pair partials
// Every pair pass runs in one of two forms: scatter (each pair evaluated once by its list owner,
// the neighbour's partials added with FP64 atomics) or two-sided (each particle evaluates its own
// list for its partials and walks its incoming list, a CSR built once per list set, for the
// neighbour-side partials; each thread writes only its particle: bit-reproducible).
#include "adjoint_ve.cuh"
#include "pairs.cuh"

namespace sphgb {

namespace {

using namespace vead;

constexpr int kVeAdjBlock = 128;

struct VeAdjArgs {
    // forward state
    const double *x, *y, *z, *vx, *vy, *vz, *h, *m, *u, *alpha0, *alpha, *xm, *kx, *gradh, *prho, *c, *divv;
    const double* C[6];
    const double* dV[6];
    const double2 *wh, *whd;  // interleaved {t[k], t[k+1] - t[k]}
    double K, gamma;
    AvPrm av;
    DevBox box;
    int avClean;
    ListView lv;
    const uint32_t* tOff;
    const uint32_t* tIdx;
    int64_t n;
    // seeds
    const double *sRho, *sAx, *sAy, *sAz, *sDu;
    // outputs
    double *bx, *by, *bz, *bvx, *bvy, *bvz, *bh, *bu;
    // per-particle quotients
    double *hInv, *rho, *vol, *lnxm;
    // forward sums
    double *en, *avE, *G, *vsig, *P, *wom, *wr0;
    uint32_t* vsigArg;
    // adjoints of the intermediate fields
    double *prhoB, *cB, *alphaB, *rhoB, *xmB, *kxB, *CB, *gB, *divvB, *gradhB;
    // seeds of the pair terms
    double *GB, *vsigB, *tauB, *PB, *Skx, *Som, *Sr0, *R0b;
};

constexpr uint32_t kNoPair = 0xffffffffu;

// interpolant value and slope (dw/dv) on the interval holding v (as the forward passes select it)
__device__ __forceinline__ double lookupVS(const double2* __restrict__ tab, double v, double& slope)
{
    const TabSlot s = tabSlot(v * kTabInvDx);
    if (s.k < 0) {
        slope = 0.0;
        return 0.0;
    }
    const double2 t = __ldg(tab + s.k);
    slope = t.y * kTabInvDx;
    return fma(t.y, s.frac, t.x);
}

// r = x_i - x_j with the legacy periodic fold at 2 h_i (box.hpp:216-238), d = |r|
__device__ __forceinline__ void geom(const VeAdjArgs& a, int64_t i, int64_t j, double r[3], double& d, double& rinv)
{
    const long long twoHBits = __double_as_longlong(2.0 * a.h[i]);
    const double dd[3] = {a.x[i] - a.x[j], a.y[i] - a.y[j], a.z[i] - a.z[j]};
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = a.box.pbc[k] ? CoordFp64::wrapLegacy(dd[k], twoHBits, a.box.L[k]) : dd[k];
    const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    rinv = rsqrt(r2);
    d = r2 * rinv;
}

__device__ __forceinline__ void vdiff(const VeAdjArgs& a, int64_t i, int64_t j, double v[3])
{
    v[0] = a.vx[i] - a.vx[j];
    v[1] = a.vy[i] - a.vy[j];
    v[2] = a.vz[i] - a.vz[j];
}

__device__ __forceinline__ MeSide meSide(const VeAdjArgs& a, int64_t i)
{
    MeSide s;
    s.hInv = a.hInv[i];
    s.c = a.c[i];
    s.alpha = a.alpha[i];
    s.m = a.m[i];
    s.rho = a.rho[i];
    s.xm = a.xm[i];
    s.lnxm = a.lnxm[i];
    s.prho = a.prho[i];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        s.C[q] = a.C[q][i];
        s.g[q] = a.avClean ? a.dV[q][i] : 0.0;
    }
    return s;
}

__device__ __forceinline__ void loadC(const VeAdjArgs& a, int64_t i, double C[6])
{
#pragma unroll
    for (int q = 0; q < 6; ++q) C[q] = a.C[q][i];
}

__device__ __forceinline__ double etaCritOf(unsigned cnt) { return cbrt(32.0 * M_PI / 3.0 / double(cnt + 1)); }

// add v to p[i]: atomically where other threads add to the same particle (scatter form)
__device__ __forceinline__ void put(double* p, int64_t i, double v, bool atomic)
{
    if (atomic) atomicAdd(p + i, v);
    else p[i] += v;
}

__global__ void veQuotKernel(VeAdjArgs a)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.n) return;
    const double xm = a.xm[i], kx = a.kx[i];
    a.hInv[i] = 1.0 / a.h[i];
    a.rho[i] = kx * a.m[i] / xm;
    a.vol[i] = xm / kx;
    a.lnxm[i] = log(xm);
}

// forward sums of the momentum-energy pass: en_i, avE_i (before max(0, .))
__global__ void __launch_bounds__(kVeAdjBlock) vePreMeKernel(VeAdjArgs a)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.n) return;
    const MeSide I = meSide(a, i);
    const unsigned nc = a.lv.capped(i);
    const double etaCrit = etaCritOf(nc);
    double en = 0.0, avE = 0.0;
    for (unsigned q = 0; q < nc; ++q) {
        const int64_t j = a.lv.at(i, q);
        double r[3], d, rinv, v[3];
        geom(a, i, j, r, d, rinv);
        vdiff(a, i, j, v);
        const MeSide J = meSide(a, j);
        double s;
        const double wi = lookupVS(a.wh, d * I.hInv, s), wj = lookupVS(a.wh, d * J.hInv, s);
        MeFwd f;
        meFwd(r, d, rinv, v, I, J, wi, wj, a.avClean != 0, etaCrit, f);
        meSums(v, J, f, en, avE);
    }
    a.en[i] = en;
    a.avE[i] = avE;
}

// forward sums of the AV switch (G_i, vsig_i and the pair that set it), of divv (P_i) and of
// gradh (whomega0 = K h^-4 S_om, wrho0 = K h^-4 S_r0)
__global__ void __launch_bounds__(kVeAdjBlock) vePreKernel(VeAdjArgs a)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.n) return;
    double Ci[6];
    loadC(a, i, Ci);
    const double hInv = a.hInv[i], ci = a.c[i], divvi = a.divv[i];
    const double Wk0 = a.K * hInv * hInv * hInv;
    double G[3] = {0.0, 0.0, 0.0}, P[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double vsig = 1e-40 * ci, so = -3.0 * a.xm[i], sr = -3.0 * a.m[i];
    uint32_t arg = kNoPair;
    const unsigned nc = a.lv.capped(i);
    for (unsigned q = 0; q < nc; ++q) {
        const uint32_t j = a.lv.at(i, q);
        double r[3], d, rinv, v[3];
        geom(a, i, j, r, d, rinv);
        vdiff(a, i, j, v);
        const double v1 = d * hInv;
        double dw, dwd;
        const double w = lookupVS(a.wh, v1, dw);
        const double wd = lookupVS(a.whd, v1, dwd);
        const double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
        if (rv < 0.0) {
            const double vs = ci + a.c[j] - 3.0 * rv * rinv;
            if (vs > vsig) {
                vsig = vs;
                arg = j;
            }
        }
        double CIr[3];
        symv(Ci, r, CIr);
        const double fac = -a.vol[j] * (divvi - a.divv[j]) * Wk0 * w;
        const double xw = a.xm[j] * w;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            G[k] += fac * CIr[k];
#pragma unroll
            for (int t = 0; t < 3; ++t) P[3 * k + t] -= xw * v[k] * r[t];
        }
        const double dterh = -(3.0 * w + v1 * wd);
        so += a.xm[j] * dterh;
        sr += a.m[j] * dterh;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) a.G[k * a.n + i] = G[k];
#pragma unroll
    for (int k = 0; k < 9; ++k) a.P[k * a.n + i] = P[k];
    a.vsig[i] = vsig;
    a.vsigArg[i] = arg;
    const double h4 = a.K * hInv * hInv * hInv * hInv;
    a.wom[i] = h4 * so;
    a.wr0[i] = h4 * sr;
}

// ---------------------------------------------------------------- momentum-energy
struct MeSeed {
    double mb[3], enb, avEb;
    bool any;
};

__device__ __forceinline__ MeSeed meSeed(const VeAdjArgs& a, int64_t i)
{
    MeSeed s;
    s.mb[0] = a.sAx ? -a.K * a.sAx[i] : 0.0;
    s.mb[1] = a.sAy ? -a.K * a.sAy[i] : 0.0;
    s.mb[2] = a.sAz ? -a.K * a.sAz[i] : 0.0;
    const double du = a.sDu ? a.sDu[i] : 0.0;
    s.enb = a.K * a.prho[i] * du;
    s.avEb = a.avE[i] >= 0.0 ? 0.5 * a.K * du : 0.0;
    s.any = s.mb[0] != 0.0 || s.mb[1] != 0.0 || s.mb[2] != 0.0 || du != 0.0;
    return s;
}

struct MeAcc {
    double x[3], v[3], h, prho, c, alpha, rho, xm, C[6], g[6];
};

__device__ __forceinline__ void meAddI(MeAcc& s, const MeGrad& o)
{
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        s.x[k] += o.r[k];
        s.v[k] += o.v[k];
    }
    s.h += o.hI;
    s.prho += o.prhoI;
    s.c += o.c;
    s.alpha += o.alpha;
    s.rho += o.rhoI;
    s.xm += o.xmI;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        s.C[q] += o.CI[q];
        s.g[q] += o.gI[q];
    }
}

__device__ __forceinline__ void meAddJ(MeAcc& s, const MeGrad& o)
{
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        s.x[k] -= o.r[k];
        s.v[k] -= o.v[k];
    }
    s.h += o.hJ;
    s.prho += o.prhoJ;
    s.c += o.c;
    s.alpha += o.alpha;
    s.rho += o.rhoJ;
    s.xm += o.xmJ;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        s.C[q] += o.CJ[q];
        s.g[q] += o.gJ[q];
    }
}

__device__ __forceinline__ void meFlush(const VeAdjArgs& a, int64_t k, const MeAcc& s, bool atomic)
{
    put(a.bx, k, s.x[0], atomic);
    put(a.by, k, s.x[1], atomic);
    put(a.bz, k, s.x[2], atomic);
    put(a.bvx, k, s.v[0], atomic);
    put(a.bvy, k, s.v[1], atomic);
    put(a.bvz, k, s.v[2], atomic);
    put(a.bh, k, s.h, atomic);
    put(a.prhoB, k, s.prho, atomic);
    put(a.cB, k, s.c, atomic);
    put(a.alphaB, k, s.alpha, atomic);
    put(a.rhoB, k, s.rho, atomic);
    put(a.xmB, k, s.xm, atomic);
#pragma unroll
    for (int q = 0; q < 6; ++q) put(a.CB + q * a.n, k, s.C[q], atomic);
    if (a.avClean)
#pragma unroll
        for (int q = 0; q < 6; ++q) put(a.gB + q * a.n, k, s.g[q], atomic);
}

__device__ __forceinline__ void mePair(const VeAdjArgs& a, int64_t i, int64_t j, const MeSide& I, const MeSide& J,
                                       double etaCrit, const MeSeed& sd, MeGrad& o)
{
    double r[3], d, rinv, v[3];
    geom(a, i, j, r, d, rinv);
    vdiff(a, i, j, v);
    double dwi, dwj;
    const double wi = lookupVS(a.wh, d * I.hInv, dwi), wj = lookupVS(a.wh, d * J.hInv, dwj);
    meAdj(r, d, rinv, v, I, J, wi, dwi, wj, dwj, a.avClean != 0, etaCrit, sd.mb, sd.enb, sd.avEb, o);
}

template<bool TwoSided>
__global__ void __launch_bounds__(kVeAdjBlock) meVeAdjKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    MeAcc s{};
    const MeSide S = meSide(a, k);
    const MeSeed sd = meSeed(a, k);
    // own terms outside the pairs: du = K (prho en + avE / 2) and the rho seed
    s.prho = a.sDu ? a.K * a.en[k] * a.sDu[k] : 0.0;
    s.rho = a.sRho ? a.sRho[k] : 0.0;
    if (sd.any) {
        const unsigned nc = a.lv.capped(k);
        const double etaCrit = etaCritOf(nc);
        for (unsigned q = 0; q < nc; ++q) {
            const int64_t j = a.lv.at(k, q);
            const MeSide J = meSide(a, j);
            MeGrad o;
            mePair(a, k, j, S, J, etaCrit, sd, o);
            meAddI(s, o);
            if (!TwoSided) {
                atomicAdd(a.bx + j, -o.r[0]);
                atomicAdd(a.by + j, -o.r[1]);
                atomicAdd(a.bz + j, -o.r[2]);
                atomicAdd(a.bvx + j, -o.v[0]);
                atomicAdd(a.bvy + j, -o.v[1]);
                atomicAdd(a.bvz + j, -o.v[2]);
                atomicAdd(a.bh + j, o.hJ);
                atomicAdd(a.prhoB + j, o.prhoJ);
                atomicAdd(a.cB + j, o.c);
                atomicAdd(a.alphaB + j, o.alpha);
                atomicAdd(a.rhoB + j, o.rhoJ);
                atomicAdd(a.xmB + j, o.xmJ);
#pragma unroll
                for (int t = 0; t < 6; ++t) atomicAdd(a.CB + t * a.n + j, o.CJ[t]);
                if (a.avClean)
#pragma unroll
                    for (int t = 0; t < 6; ++t) atomicAdd(a.gB + t * a.n + j, o.gJ[t]);
            }
        }
    }
    if (TwoSided) {
        for (uint32_t e = a.tOff[k]; e < a.tOff[k + 1]; ++e) {
            const int64_t i = a.tIdx[e];
            const MeSeed si = meSeed(a, i);
            if (!si.any) continue;
            const MeSide I = meSide(a, i);
            MeGrad o;
            mePair(a, i, k, I, S, etaCritOf(a.lv.capped(i)), si, o);
            meAddJ(s, o);
        }
    }
    meFlush(a, k, s, !TwoSided);
}

// ---------------------------------------------------------------- AV switch
__global__ void veAvSeedKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    const double G[3] = {a.G[k], a.G[a.n + k], a.G[2 * a.n + k]};
    double Gb[3], vsigb, hb, divvb, cb;
    avSeed(a.av, a.alphaB[k], a.alpha0[k], a.h[k], a.c[k], a.divv[k], G, a.vsig[k], Gb, vsigb, hb, divvb, cb);
    if (a.vsigArg[k] == kNoPair) cb += 1e-40 * vsigb;  // vsig = 1e-40 c_i when no pair approaches
#pragma unroll
    for (int t = 0; t < 3; ++t) a.GB[t * a.n + k] = Gb[t];
    a.vsigB[k] = vsigb;
    a.bh[k] += hb;
    a.divvB[k] += divvb;
    a.cB[k] += cb;
}

struct AvSeedV {
    double Gb[3], vsigb;
    uint32_t arg;
    bool any;
};

__device__ __forceinline__ AvSeedV avSeedOf(const VeAdjArgs& a, int64_t i)
{
    AvSeedV s;
    s.Gb[0] = a.GB[i];
    s.Gb[1] = a.GB[a.n + i];
    s.Gb[2] = a.GB[2 * a.n + i];
    s.vsigb = a.vsigB[i];
    s.arg = a.vsigArg[i];
    s.any = s.Gb[0] != 0.0 || s.Gb[1] != 0.0 || s.Gb[2] != 0.0 || s.vsigb != 0.0;
    return s;
}

__device__ __forceinline__ void avPair(const VeAdjArgs& a, int64_t i, int64_t j, const double Ci[6],
                                       const AvSeedV& sd, AvGrad& o)
{
    double r[3], d, rinv, v[3];
    geom(a, i, j, r, d, rinv);
    vdiff(a, i, j, v);
    const double hInv = a.hInv[i];
    double dw;
    const double w = lookupVS(a.wh, d * hInv, dw);
    avAdj(r, d, rinv, v, hInv, w, dw, Ci, a.K, a.vol[j], a.kx[j], a.xm[j], a.divv[i], a.divv[j], sd.Gb, sd.vsigb,
          uint32_t(j) == sd.arg, o);
}

template<bool TwoSided>
__global__ void __launch_bounds__(kVeAdjBlock) veAvAdjKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double x[3] = {0, 0, 0}, v[3] = {0, 0, 0}, c = 0, h = 0, C[6] = {0, 0, 0, 0, 0, 0}, divv = 0, xm = 0, kx = 0;
    const AvSeedV sd = avSeedOf(a, k);
    if (sd.any) {
        double Ck[6];
        loadC(a, k, Ck);
        const unsigned nc = a.lv.capped(k);
        for (unsigned q = 0; q < nc; ++q) {
            const int64_t j = a.lv.at(k, q);
            AvGrad o;
            avPair(a, k, j, Ck, sd, o);
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                x[t] += o.r[t];
                v[t] += o.v[t];
            }
            c += o.cI;
            h += o.hI;
            divv += o.divvI;
#pragma unroll
            for (int t = 0; t < 6; ++t) C[t] += o.CI[t];
            if (!TwoSided) {
                atomicAdd(a.bx + j, -o.r[0]);
                atomicAdd(a.by + j, -o.r[1]);
                atomicAdd(a.bz + j, -o.r[2]);
                if (uint32_t(j) == sd.arg) {
                    atomicAdd(a.bvx + j, -o.v[0]);
                    atomicAdd(a.bvy + j, -o.v[1]);
                    atomicAdd(a.bvz + j, -o.v[2]);
                    atomicAdd(a.cB + j, o.cJ);
                }
                atomicAdd(a.divvB + j, o.divvJ);
                atomicAdd(a.xmB + j, o.xmJ);
                atomicAdd(a.kxB + j, o.kxJ);
            }
        }
    }
    if (TwoSided) {
        for (uint32_t e = a.tOff[k]; e < a.tOff[k + 1]; ++e) {
            const int64_t i = a.tIdx[e];
            const AvSeedV si = avSeedOf(a, i);
            if (!si.any) continue;
            double Ci[6];
            loadC(a, i, Ci);
            AvGrad o;
            avPair(a, i, k, Ci, si, o);
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                x[t] -= o.r[t];
                v[t] -= o.v[t];
            }
            c += o.cJ;
            divv += o.divvJ;
            xm += o.xmJ;
            kx += o.kxJ;
        }
    }
    const bool at = !TwoSided;
    put(a.bx, k, x[0], at);
    put(a.by, k, x[1], at);
    put(a.bz, k, x[2], at);
    put(a.bvx, k, v[0], at);
    put(a.bvy, k, v[1], at);
    put(a.bvz, k, v[2], at);
    put(a.cB, k, c, at);
    put(a.bh, k, h, at);
    put(a.divvB, k, divv, at);
    put(a.xmB, k, xm, at);
    put(a.kxB, k, kx, at);
#pragma unroll
    for (int t = 0; t < 6; ++t) put(a.CB + t * a.n, k, C[t], at);
}

// ---------------------------------------------------------------- IAD + divv
__global__ void veIadSeedKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double C[6], Cb[6], gb[6], P[9], tauB[6], PB[9];
    loadC(a, k, C);
#pragma unroll
    for (int t = 0; t < 6; ++t) {
        Cb[t] = a.CB[t * a.n + k];
        gb[t] = a.avClean ? a.gB[t * a.n + k] : 0.0;
    }
#pragma unroll
    for (int t = 0; t < 9; ++t) P[t] = a.P[t * a.n + k];
    double hb = 0.0, kxb = 0.0;
    iadDivvSeed(a.K, a.h[k], a.kx[k], C, Cb, a.divvB[k], gb, P, tauB, PB, hb, kxb);
#pragma unroll
    for (int t = 0; t < 6; ++t) a.tauB[t * a.n + k] = tauB[t];
#pragma unroll
    for (int t = 0; t < 9; ++t) a.PB[t * a.n + k] = PB[t];
    a.bh[k] += hb;
    a.kxB[k] += kxb;
}

__device__ __forceinline__ void iadPair(const VeAdjArgs& a, int64_t i, int64_t j, const double tauB[6],
                                        const double PB[9], IadGrad& o)
{
    double r[3], d, rinv, v[3];
    geom(a, i, j, r, d, rinv);
    vdiff(a, i, j, v);
    const double hInv = a.hInv[i];
    double dw;
    const double w = lookupVS(a.wh, d * hInv, dw);
    iadDivvAdj(r, d, rinv, v, hInv, w, dw, a.vol[j], a.kx[j], a.xm[j], tauB, PB, o);
}

__device__ __forceinline__ void iadSeedOf(const VeAdjArgs& a, int64_t i, double tauB[6], double PB[9])
{
#pragma unroll
    for (int t = 0; t < 6; ++t) tauB[t] = a.tauB[t * a.n + i];
#pragma unroll
    for (int t = 0; t < 9; ++t) PB[t] = a.PB[t * a.n + i];
}

template<bool TwoSided>
__global__ void __launch_bounds__(kVeAdjBlock) veIadAdjKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double x[3] = {0, 0, 0}, v[3] = {0, 0, 0}, h = 0, xm = 0, kx = 0;
    {
        double tauB[6], PB[9];
        iadSeedOf(a, k, tauB, PB);
        const unsigned nc = a.lv.capped(k);
        for (unsigned q = 0; q < nc; ++q) {
            const int64_t j = a.lv.at(k, q);
            IadGrad o;
            iadPair(a, k, j, tauB, PB, o);
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                x[t] += o.r[t];
                v[t] += o.v[t];
            }
            h += o.hI;
            if (!TwoSided) {
                atomicAdd(a.bx + j, -o.r[0]);
                atomicAdd(a.by + j, -o.r[1]);
                atomicAdd(a.bz + j, -o.r[2]);
                atomicAdd(a.bvx + j, -o.v[0]);
                atomicAdd(a.bvy + j, -o.v[1]);
                atomicAdd(a.bvz + j, -o.v[2]);
                atomicAdd(a.xmB + j, o.xmJ);
                atomicAdd(a.kxB + j, o.kxJ);
            }
        }
    }
    if (TwoSided) {
        for (uint32_t e = a.tOff[k]; e < a.tOff[k + 1]; ++e) {
            const int64_t i = a.tIdx[e];
            double tauB[6], PB[9];
            iadSeedOf(a, i, tauB, PB);
            IadGrad o;
            iadPair(a, i, k, tauB, PB, o);
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                x[t] -= o.r[t];
                v[t] -= o.v[t];
            }
            xm += o.xmJ;
            kx += o.kxJ;
        }
    }
    const bool at = !TwoSided;
    put(a.bx, k, x[0], at);
    put(a.by, k, x[1], at);
    put(a.bz, k, x[2], at);
    put(a.bvx, k, v[0], at);
    put(a.bvy, k, v[1], at);
    put(a.bvz, k, v[2], at);
    put(a.bh, k, h, at);
    put(a.xmB, k, xm, at);
    put(a.kxB, k, kx, at);
}

// ---------------------------------------------------------------- EOS, gradh, xmass
__global__ void veEosAdjKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double kxb = a.kxB[k], xmb = a.xmB[k], gradhb = 0.0, ub = 0.0;
    eosAdj(a.gamma, a.u[k], a.m[k], a.kx[k], a.xm[k], a.gradh[k], a.c[k], a.prhoB[k], a.cB[k], a.rhoB[k], kxb, xmb,
           gradhb, ub);
    a.kxB[k] = kxb;
    a.xmB[k] = xmb;
    a.gradhB[k] = gradhb;
    a.bu[k] = ub;
}

__global__ void veGradhSeedKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double skx, som, sr0, hb = 0.0, xmb = 0.0;
    gradhSeed(a.K, a.h[k], a.m[k], a.xm[k], a.kx[k], a.wom[k], a.wr0[k], a.kxB[k], a.gradhB[k], skx, som, sr0, hb, xmb);
    a.Skx[k] = skx;
    a.Som[k] = som;
    a.Sr0[k] = sr0;
    a.bh[k] += hb;
    a.xmB[k] += xmb;
}

__device__ __forceinline__ void gradhPair(const VeAdjArgs& a, int64_t i, int64_t j, GradhGrad& o)
{
    double r[3], d, rinv;
    geom(a, i, j, r, d, rinv);
    const double hInv = a.hInv[i];
    double dw, dwd;
    const double w = lookupVS(a.wh, d * hInv, dw);
    const double wd = lookupVS(a.whd, d * hInv, dwd);
    gradhAdj(r, d, rinv, hInv, w, dw, wd, dwd, a.xm[j], a.m[j], a.Skx[i], a.Som[i], a.Sr0[i], o);
}

template<bool TwoSided>
__global__ void __launch_bounds__(kVeAdjBlock) veGradhAdjKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double x[3] = {0, 0, 0}, h = 0, xm = 0;
    const unsigned nc = a.lv.capped(k);
    for (unsigned q = 0; q < nc; ++q) {
        const int64_t j = a.lv.at(k, q);
        GradhGrad o;
        gradhPair(a, k, j, o);
#pragma unroll
        for (int t = 0; t < 3; ++t) x[t] += o.r[t];
        h += o.hI;
        if (!TwoSided) {
            atomicAdd(a.bx + j, -o.r[0]);
            atomicAdd(a.by + j, -o.r[1]);
            atomicAdd(a.bz + j, -o.r[2]);
            atomicAdd(a.xmB + j, o.xmJ);
        }
    }
    if (TwoSided) {
        for (uint32_t e = a.tOff[k]; e < a.tOff[k + 1]; ++e) {
            const int64_t i = a.tIdx[e];
            GradhGrad o;
            gradhPair(a, i, k, o);
#pragma unroll
            for (int t = 0; t < 3; ++t) x[t] -= o.r[t];
            xm += o.xmJ;
        }
    }
    const bool at = !TwoSided;
    put(a.bx, k, x[0], at);
    put(a.by, k, x[1], at);
    put(a.bz, k, x[2], at);
    put(a.bh, k, h, at);
    put(a.xmB, k, xm, at);
}

__global__ void veXmassSeedKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double r0b, hb = 0.0;
    xmassSeed(a.K, a.h[k], a.m[k], a.xm[k], a.xmB[k], r0b, hb);
    a.R0b[k] = r0b;
    a.bh[k] += hb;
}

__device__ __forceinline__ void xmassPair(const VeAdjArgs& a, int64_t i, int64_t j, double rb[3], double& hIb)
{
    double r[3], d, rinv;
    geom(a, i, j, r, d, rinv);
    const double hInv = a.hInv[i];
    double dw;
    lookupVS(a.wh, d * hInv, dw);
    xmassAdj(r, d, rinv, hInv, dw, a.m[j], a.R0b[i], rb, hIb);
}

template<bool TwoSided>
__global__ void __launch_bounds__(kVeAdjBlock) veXmassAdjKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double x[3] = {0, 0, 0}, h = 0;
    const unsigned nc = a.lv.capped(k);
    for (unsigned q = 0; q < nc; ++q) {
        const int64_t j = a.lv.at(k, q);
        double rb[3], hIb;
        xmassPair(a, k, j, rb, hIb);
#pragma unroll
        for (int t = 0; t < 3; ++t) x[t] += rb[t];
        h += hIb;
        if (!TwoSided) {
            atomicAdd(a.bx + j, -rb[0]);
            atomicAdd(a.by + j, -rb[1]);
            atomicAdd(a.bz + j, -rb[2]);
        }
    }
    if (TwoSided) {
        for (uint32_t e = a.tOff[k]; e < a.tOff[k + 1]; ++e) {
            const int64_t i = a.tIdx[e];
            double rb[3], hIb;
            xmassPair(a, i, k, rb, hIb);
#pragma unroll
            for (int t = 0; t < 3; ++t) x[t] -= rb[t];
        }
    }
    const bool at = !TwoSided;
    put(a.bx, k, x[0], at);
    put(a.by, k, x[1], at);
    put(a.bz, k, x[2], at);
    put(a.bh, k, h, at);
}

}  // namespace

// number of n-sized double sections of the VE adjoint state
constexpr int kVeAdjSections = 65;

int adjointVe(sphgb_ctx* c, sphgb_particles* p, const double* alphaPrev, int avClean, const sphgb_seeds* s,
              sphgb_grads* g, int deterministic)
{
    if (!c->haveNbr) return SPHGB_ERR_STATE;
    if (p->precision != SPHGB_FP64) return SPHGB_ERR_ARG;
    if (c->nbrFirst != 0 || c->nbrLast != p->n) return SPHGB_ERR_ARG;
    if (!alphaPrev || !p->x || !p->y || !p->z || !p->vx || !p->vy || !p->vz || !p->h || !p->m || !p->u || !p->alpha ||
        !p->xm || !p->kx || !p->gradh || !p->prho || !p->c || !p->divv || !p->c11 || !p->c12 || !p->c13 || !p->c22 ||
        !p->c23 || !p->c33)
        return SPHGB_ERR_ARG;
    if (avClean && (!p->dV11 || !p->dV12 || !p->dV13 || !p->dV22 || !p->dV23 || !p->dV33)) return SPHGB_ERR_ARG;
    if (!g || !g->x || !g->y || !g->z || !g->vx || !g->vy || !g->vz || !g->h || !g->u) return SPHGB_ERR_ARG;
    const int64_t n = p->n;
    if (deterministic) SPHGB_TRY(buildTranspose(c));
    SPHGB_TRY(c->adjState.ensure(sizeof(double) * kVeAdjSections * n));
    double* st = c->adjState.as<double>();

    VeAdjArgs a{};
    auto d = [](const void* q) { return static_cast<const double*>(q); };
    a.x = p->x;
    a.y = p->y;
    a.z = p->z;
    a.vx = d(p->vx);
    a.vy = d(p->vy);
    a.vz = d(p->vz);
    a.h = d(p->h);
    a.m = d(p->m);
    a.u = p->u;
    a.alpha0 = alphaPrev;
    a.alpha = d(p->alpha);
    a.xm = d(p->xm);
    a.kx = d(p->kx);
    a.gradh = d(p->gradh);
    a.prho = d(p->prho);
    a.c = d(p->c);
    a.divv = d(p->divv);
    const void* Cs[6] = {p->c11, p->c12, p->c13, p->c22, p->c23, p->c33};
    const void* dVs[6] = {p->dV11, p->dV12, p->dV13, p->dV22, p->dV23, p->dV33};
    for (int q = 0; q < 6; ++q) {
        a.C[q] = d(Cs[q]);
        a.dV[q] = avClean ? d(dVs[q]) : nullptr;
    }
    a.wh = c->whx64.as<double2>();
    a.whd = c->whdx64.as<double2>();
    a.K = c->K;
    a.gamma = c->prm.gamma;
    a.av = AvPrm{c->K, c->prm.minDt, c->prm.alphamin, c->prm.alphamax, c->prm.decay_constant};
    a.box = c->box;
    a.avClean = avClean ? 1 : 0;
    a.lv = listView(c);
    a.tOff = c->tOff.as<uint32_t>();
    a.tIdx = c->tIdx.as<uint32_t>();
    a.n = n;
    if (s) {
        a.sRho = d(s->rho);
        a.sAx = d(s->ax);
        a.sAy = d(s->ay);
        a.sAz = d(s->az);
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
    double* q = st;
    auto take = [&](int sections) {
        double* r = q;
        q += int64_t(sections) * n;
        return r;
    };
    // accumulators first: one memset clears them
    a.prhoB = take(1);
    a.cB = take(1);
    a.alphaB = take(1);
    a.rhoB = take(1);
    a.xmB = take(1);
    a.kxB = take(1);
    a.CB = take(6);
    a.gB = take(6);
    a.divvB = take(1);
    a.gradhB = take(1);
    const int64_t accSections = 20;
    a.hInv = take(1);
    a.rho = take(1);
    a.vol = take(1);
    a.lnxm = take(1);
    a.en = take(1);
    a.avE = take(1);
    a.G = take(3);
    a.vsig = take(1);
    a.P = take(9);
    a.wom = take(1);
    a.wr0 = take(1);
    a.vsigArg = reinterpret_cast<uint32_t*>(take(1));
    a.GB = take(3);
    a.vsigB = take(1);
    a.tauB = take(6);
    a.PB = take(9);
    a.Skx = take(1);
    a.Som = take(1);
    a.Sr0 = take(1);
    a.R0b = take(1);
    if (q - st > int64_t(kVeAdjSections) * n) return SPHGB_ERR_TOO_LARGE;  // layout and size disagree

    for (double* z : {g->x, g->y, g->z, g->vx, g->vy, g->vz, g->h, g->u})
        SPHGB_CUDA(cudaMemsetAsync(z, 0, sizeof(double) * n, c->stream));
    SPHGB_CUDA(cudaMemsetAsync(st, 0, sizeof(double) * accSections * n, c->stream));

    const unsigned pb = gridFor(n, kVeAdjBlock), eb = gridFor(n, 256);
    const bool two = deterministic != 0;
    veQuotKernel<<<eb, 256, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "veQuotKernel"));
    vePreMeKernel<<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "vePreMeKernel"));
    vePreKernel<<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "vePreKernel"));
    if (two) meVeAdjKernel<true><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    else meVeAdjKernel<false><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "meVeAdjKernel"));
    veAvSeedKernel<<<eb, 256, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "veAvSeedKernel"));
    if (two) veAvAdjKernel<true><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    else veAvAdjKernel<false><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "veAvAdjKernel"));
    veIadSeedKernel<<<eb, 256, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "veIadSeedKernel"));
    if (two) veIadAdjKernel<true><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    else veIadAdjKernel<false><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "veIadAdjKernel"));
    veEosAdjKernel<<<eb, 256, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "veEosAdjKernel"));
    veGradhSeedKernel<<<eb, 256, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "veGradhSeedKernel"));
    if (two) veGradhAdjKernel<true><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    else veGradhAdjKernel<false><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "veGradhAdjKernel"));
    veXmassSeedKernel<<<eb, 256, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "veXmassSeedKernel"));
    if (two) veXmassAdjKernel<true><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    else veXmassAdjKernel<false><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "veXmassAdjKernel"));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    return SPHGB_OK;
}

}  // namespace sphgb
