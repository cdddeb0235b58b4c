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
    const double2 *wh, *whd;  // W and dW/dv in the context's form (the kernels' Smooth argument tells which)
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
    double *hInv, *rho, *rhoInv, *vol, *kxInv, *xmInv, *lnxm;
    // forward sums
    double *en, *avE, *G, *vsig, *P, *wom, *wr0;
    uint32_t* vsigArg;
    // FP32 copies {x y z c} and {vx vy vz 0} for the signal-velocity filter, and the bound on the
    // FP32 error of a position difference per component
    float4 *xc32, *v32;
    float ePos;
    // adjoints of the intermediate fields
    double *prhoB, *cB, *alphaB, *rhoB, *xmB, *kxB, *CB, *gB, *divvB, *gradhB;
    double* Rav;  // 3 x n: R_i = sum_j fac_j W_j r_j of the AV pair terms (i's C partials, avCbar)
    // seeds of the pair terms
    double *GB, *CGB, *vsigB, *tauB, *PB, *Skx, *Som, *Sr0, *R0b;
};

constexpr uint32_t kNoPair = 0xffffffffu;

// interpolant value and slope (dw/dv) on the interval holding v (as the forward passes select it)
template<bool Smooth>
__device__ __forceinline__ double lookupVS(const KTab<Smooth>& tab, double v, double& slope)
{
    return lookupVSlope(tab, v, slope);
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
    s.rhoInv = a.rhoInv[i];
    s.xm = a.xm[i];
    s.xmInv = a.xmInv[i];
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
    const double rho = kx * a.m[i] / xm;
    a.hInv[i] = 1.0 / a.h[i];
    a.rho[i] = rho;
    a.rhoInv[i] = 1.0 / rho;
    a.vol[i] = xm / kx;
    a.kxInv[i] = 1.0 / kx;
    a.xmInv[i] = 1.0 / xm;
    a.lnxm[i] = log(xm);
    a.xc32[i] = make_float4(float(a.x[i]), float(a.y[i]), float(a.z[i]), float(a.c[i]));
    a.v32[i] = make_float4(float(a.vx[i]), float(a.vy[i]), float(a.vz[i]), 0.f);
}

// forward sums of the momentum-energy pass: en_i, avE_i (before max(0, .))
template<bool Smooth>
__global__ void __launch_bounds__(kVeAdjBlock) vePreMeKernel(VeAdjArgs a)
{
    const KTab<Smooth> tw{a.wh};
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
        const double wi = lookupVS(tw, d * I.hInv, s), wj = lookupVS(tw, d * J.hInv, s);
        MeFwd f;
        meFwd(r, d, rinv, v, I, J, wi, wj, a.avClean != 0, etaCrit, f);
        meSums(v, J, f, en, avE);
    }
    a.en[i] = en;
    a.avE[i] = avE;
}

// the signal velocity of the AV switch (av_switches_kern.hpp:66-86): the first of i's approaching
// pairs, in list order, with the largest c_i + c_j - 3 (r.v)/|r| sets vsig_i (1e-40 c_i when none)
__device__ __forceinline__ void vsigStep(const VeAdjArgs& a, int64_t j, const double r[3], double rinv,
                                         const double v[3], double ci, double& vsig, uint32_t& arg)
{
    const double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    if (rv < 0.0) {
        const double vs = ci + a.c[j] - 3.0 * rv * rinv;
        if (vs > vsig) {
            vsig = vs;
            arg = uint32_t(j);
        }
    }
}

// vsig_i and its pair alone, when the forward passes kept the other sums of vePreKernel.  One FP32
// walk over i's list keeps a lower bound L on vsig_i from the pairs that surely approach; a pair
// is evaluated in FP64 (vsigStep, in list order) only when its FP32 signal velocity plus the error
// bound reaches the current L, which every pair able to set vsig_i does, so vsig_i and its pair
// come out as in vePreKernel.  Particles whose 2h exceeds a quarter of a periodic box edge (where
// the threshold-2h image rule of the FP64 geometry need not be the minimum image) walk in FP64.
__global__ void __launch_bounds__(kVeAdjBlock) veArgKernel(VeAdjArgs a)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.n) return;
    const double ci = a.c[i];
    double vsig = 1e-40 * ci;
    uint32_t arg = kNoPair;
    const unsigned nc = a.lv.capped(i);
    auto exact = [&](uint32_t j) {
        double r[3], d, rinv, v[3];
        geom(a, i, j, r, d, rinv);
        vdiff(a, i, j, v);
        vsigStep(a, j, r, rinv, v, ci, vsig, arg);
    };
    const double twoH = 2.0 * a.h[i];
    bool fp64Walk = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) fp64Walk |= a.box.pbc[k] && twoH > 0.25 * a.box.L[k];
    if (fp64Walk) {
        for (unsigned q = 0; q < nc; ++q) exact(a.lv.at(i, q));
    } else {
        const float4 Xi = a.xc32[i], Vi = a.v32[i];
        const float viMax = fmaxf(fabsf(Vi.x), fmaxf(fabsf(Vi.y), fabsf(Vi.z)));
        const float dr = 2.f * a.ePos;  // >= |r_f - r| (three components)
        float L = 0.f;                  // vsig_i > 0
        for (unsigned q = 0; q < nc; ++q) {
            const uint32_t j = a.lv.at(i, q);
            const float4 Xj = a.xc32[j], Vj = a.v32[j];
            float r[3] = {Xi.x - Xj.x, Xi.y - Xj.y, Xi.z - Xj.z};
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if (a.box.pbc[k]) {  // minimum image: |r| <= 2h < L/4 for every listed pair
                    if (r[k] > 0.5f * a.box.Lf[k]) r[k] -= a.box.Lf[k];
                    else if (r[k] < -0.5f * a.box.Lf[k]) r[k] += a.box.Lf[k];
                }
            const float v[3] = {Vi.x - Vj.x, Vi.y - Vj.y, Vi.z - Vj.z};
            const float d = sqrtf(fmaf(r[0], r[0], fmaf(r[1], r[1], r[2] * r[2])));
            const float rv = fmaf(r[0], v[0], fmaf(r[1], v[1], r[2] * v[2]));
            // bounds: |v_f - v| <= dv, |r.v error| <= erv, |signal velocity error| <= ev
            const float vn = 1.8f * (viMax + fmaxf(fabsf(Vj.x), fmaxf(fabsf(Vj.y), fabsf(Vj.z))));
            const float dv = 1e-6f * vn;
            const float erv = dr * vn + d * (dv + 1e-6f * vn);
            const float vs = Xi.w + Xj.w - 3.f * rv / d;
            const float ev = 3.f * (4.f * dr * vn / d + 2.f * dv + 1e-6f * vn) +
                             1e-6f * (Xi.w + Xj.w + 3.f * fabsf(rv) / d);
            if (!(rv >= erv) && !(vs + ev < L)) exact(j);  // may approach and may reach L (NaN: evaluate)
            if (rv < -erv) L = fmaxf(L, vs - ev);          // surely approaches
        }
    }
    a.vsig[i] = vsig;
    a.vsigArg[i] = arg;
}

// forward sums of the AV switch (G_i, vsig_i and the pair that set it), of divv (P_i) and of
// gradh (whomega0 = K h^-4 S_om, wrho0 = K h^-4 S_r0)
template<bool Smooth>
__global__ void __launch_bounds__(kVeAdjBlock) vePreKernel(VeAdjArgs a)
{
    const KTab<Smooth> tw{a.wh};
    const KTab<Smooth> tdw{a.whd};
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.n) return;
    double Ci[6];
    loadC(a, i, Ci);
    const double hInv = a.hInv[i], ci = a.c[i], divvi = a.divv[i];
    const double Wk0 = a.K * hInv * hInv * hInv;
    double S[3] = {0.0, 0.0, 0.0}, P[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
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
        const double w = lookupVS(tw, v1, dw);
        const double wd = lookupVS(tdw, v1, dwd);
        vsigStep(a, j, r, rinv, v, ci, vsig, arg);
        const double fac = a.vol[j] * (divvi - a.divv[j]) * w;
        const double xw = a.xm[j] * w;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            S[k] += fac * r[k];
#pragma unroll
            for (int t = 0; t < 3; ++t) P[3 * k + t] -= xw * v[k] * r[t];
        }
        const double dterh = -(3.0 * w + v1 * wd);
        so += a.xm[j] * dterh;
        sr += a.m[j] * dterh;
    }
    // G = -K h^-3 C_i S, S = sum_j vol_j (divv_i - divv_j) w r
    double G[3];
    symv(Ci, S, G);
#pragma unroll
    for (int k = 0; k < 3; ++k) a.G[k * a.n + i] = -Wk0 * G[k];
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

template<bool WithDu>
__device__ __forceinline__ MeSeed meSeed(const VeAdjArgs& a, int64_t i)
{
    MeSeed s;
    s.mb[0] = a.sAx ? -a.K * a.sAx[i] : 0.0;
    s.mb[1] = a.sAy ? -a.K * a.sAy[i] : 0.0;
    s.mb[2] = a.sAz ? -a.K * a.sAz[i] : 0.0;
    s.any = s.mb[0] != 0.0 || s.mb[1] != 0.0 || s.mb[2] != 0.0;
    s.enb = s.avEb = 0.0;
    if (WithDu) {
        const double du = a.sDu[i];
        s.enb = a.K * a.prho[i] * du;
        s.avEb = a.avE[i] >= 0.0 ? 0.5 * a.K * du : 0.0;
        s.any = s.any || du != 0.0;
    }
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

template<bool AvClean>
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
    if (AvClean)
#pragma unroll
        for (int q = 0; q < 6; ++q) put(a.gB + q * a.n, k, s.g[q], atomic);
}

template<bool AvClean, bool WithDu, bool Smooth>
__device__ __forceinline__ void mePair(const VeAdjArgs& a, int64_t i, int64_t j, const MeSide& I, const MeSide& J,
                                       double etaCrit, const MeSeed& sd, MeGrad& o)
{
    const KTab<Smooth> tw{a.wh};
    double r[3], d, rinv, v[3];
    geom(a, i, j, r, d, rinv);
    vdiff(a, i, j, v);
    double dwi, dwj;
    const double wi = lookupVS(tw, d * I.hInv, dwi), wj = lookupVS(tw, d * J.hInv, dwj);
    meAdj<AvClean, WithDu>(r, d, rinv, v, I, J, wi, dwi, wj, dwj, etaCrit, sd.mb, sd.enb, sd.avEb, o);
}

// WithDu: a du seed is given (the energy sums en, avE of the forward are then needed)
template<bool TwoSided, bool AvClean, bool WithDu, bool Smooth>
__global__ void __launch_bounds__(kVeAdjBlock) meVeAdjKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    MeAcc s{};
    const MeSide S = meSide(a, k);
    const MeSeed sd = meSeed<WithDu>(a, k);
    // own terms outside the pairs: du = K (prho en + avE / 2) and the rho seed
    s.prho = WithDu ? a.K * a.en[k] * a.sDu[k] : 0.0;
    s.rho = a.sRho ? a.sRho[k] : 0.0;
    if (sd.any) {
        const unsigned nc = a.lv.capped(k);
        const double etaCrit = etaCritOf(nc);
        for (unsigned q = 0; q < nc; ++q) {
            const int64_t j = a.lv.at(k, q);
            const MeSide J = meSide(a, j);
            MeGrad o;
            mePair<AvClean, WithDu, Smooth>(a, k, j, S, J, etaCrit, sd, o);
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
                if (AvClean)
#pragma unroll
                    for (int t = 0; t < 6; ++t) atomicAdd(a.gB + t * a.n + j, o.gJ[t]);
            }
        }
    }
    if (TwoSided) {
        for (uint32_t e = a.tOff[k]; e < a.tOff[k + 1]; ++e) {
            const int64_t i = a.tIdx[e];
            const MeSeed si = meSeed<WithDu>(a, i);
            if (!si.any) continue;
            const MeSide I = meSide(a, i);
            MeGrad o;
            mePair<AvClean, WithDu, Smooth>(a, i, k, I, S, etaCritOf(a.lv.capped(i)), si, o);
            meAddJ(s, o);
        }
    }
    meFlush<AvClean>(a, k, s, !TwoSided);
}

// one evaluation per owned entry of the owned lists built with the neighbour lists: a mutual pair
// gives both particles' terms (meAdjMutual), a one-sided entry its owner's (the same function with
// the neighbour's seeds zero); the neighbour's partials are added with FP64 atomics.  No avClean.
template<bool WithDu, bool Smooth>
__global__ void __launch_bounds__(kVeAdjBlock) meVeAdjOnceKernel(VeAdjArgs a, OwnedView ov)
{
    const KTab<Smooth> tw{a.wh};
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    MeAcc s{};
    const MeSide S = meSide(a, k);
    const MeSeed sd = meSeed<WithDu>(a, k);
    s.prho = WithDu ? a.K * a.en[k] * a.sDu[k] : 0.0;
    s.rho = a.sRho ? a.sRho[k] : 0.0;
    const unsigned cnt = ov.size(k);
    for (unsigned q = 0; q < cnt; ++q) {
        bool mutual;
        const uint32_t j = ov.at(k, q, mutual);
        MeSeed sj{};
        if (mutual) sj = meSeed<WithDu>(a, j);
        if (!sd.any && !sj.any) continue;
        const MeSide J = meSide(a, j);
        double r[3], d, rinv, v[3];
        geom(a, k, j, r, d, rinv);
        vdiff(a, k, j, v);
        double dwi, dwj;
        const double wi = lookupVS(tw, d * S.hInv, dwi), wj = lookupVS(tw, d * J.hInv, dwj);
        MeGrad o;
        meAdjMutual<WithDu>(r, d, rinv, v, S, J, wi, dwi, wj, dwj, sd.mb, sd.enb, sd.avEb, sj.mb, sj.enb, sj.avEb, o);
        meAddI(s, o);
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
    }
    meFlush<false>(a, k, s, true);
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
    double C[6], CGb[3];
    loadC(a, k, C);
    symv(C, Gb, CGb);
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        a.GB[t * a.n + k] = Gb[t];
        a.CGB[t * a.n + k] = CGb[t];
    }
    a.vsigB[k] = vsigb;
    a.bh[k] += hb;
    a.divvB[k] += divvb;
    a.cB[k] += cb;
}

struct AvSeedV {
    double Gb[3], CGb[3], vsigb;
    uint32_t arg;
    bool any, gAny;  // gAny: a G seed; without one only the pair that set vsig has partials
};

__device__ __forceinline__ AvSeedV avSeedOf(const VeAdjArgs& a, int64_t i)
{
    AvSeedV s;
    s.Gb[0] = a.GB[i];
    s.Gb[1] = a.GB[a.n + i];
    s.Gb[2] = a.GB[2 * a.n + i];
#pragma unroll
    for (int t = 0; t < 3; ++t) s.CGb[t] = a.CGB[t * a.n + i];
    s.vsigb = a.vsigB[i];
    s.arg = a.vsigArg[i];
    s.gAny = s.Gb[0] != 0.0 || s.Gb[1] != 0.0 || s.Gb[2] != 0.0;
    s.any = s.gAny || s.vsigb != 0.0;
    return s;
}

template<bool Smooth>
__device__ __forceinline__ void avPair(const VeAdjArgs& a, int64_t i, int64_t j, const AvSeedV& sd, AvGrad& o)
{
    const KTab<Smooth> tw{a.wh};
    double r[3], d, rinv, v[3];
    geom(a, i, j, r, d, rinv);
    vdiff(a, i, j, v);
    const double hInv = a.hInv[i];
    double dw;
    const double w = lookupVS(tw, d * hInv, dw);
    avAdj(r, d, rinv, v, hInv, w, dw, a.K, a.vol[j], a.kxInv[j], a.divv[i], a.divv[j], sd.CGb, sd.vsigb,
          uint32_t(j) == sd.arg, o);
}

template<bool TwoSided, bool Smooth>
__global__ void __launch_bounds__(kVeAdjBlock) veAvAdjKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double x[3] = {0, 0, 0}, v[3] = {0, 0, 0}, c = 0, h = 0, divv = 0, xm = 0, kx = 0;
    const AvSeedV sd = avSeedOf(a, k);
    if (sd.any) {
        double R[3] = {0.0, 0.0, 0.0};
        const unsigned nc = a.lv.capped(k);
        for (unsigned q = 0; q < nc; ++q) {
            const int64_t j = a.lv.at(k, q);
            if (!sd.gAny && uint32_t(j) != sd.arg) continue;
            AvGrad o;
            avPair<Smooth>(a, k, j, sd, o);
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                x[t] += o.r[t];
                v[t] += o.v[t];
                R[t] += o.R[t];
            }
            c += o.cI;
            h += o.hI;
            divv += o.divvI;
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
#pragma unroll
        for (int t = 0; t < 3; ++t) put(a.Rav + t * a.n, k, R[t], !TwoSided);
    }
    if (TwoSided) {
        for (uint32_t e = a.tOff[k]; e < a.tOff[k + 1]; ++e) {
            const int64_t i = a.tIdx[e];
            const AvSeedV si = avSeedOf(a, i);
            if (!si.any || (!si.gAny && uint32_t(k) != si.arg)) continue;
            AvGrad o;
            avPair<Smooth>(a, i, k, si, o);
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
}

// scatter form over the owned lists: a mutual pair gives both directed terms from one geometry
template<bool Smooth>
__global__ void __launch_bounds__(kVeAdjBlock) veAvAdjOnceKernel(VeAdjArgs a, OwnedView ov)
{
    const KTab<Smooth> tw{a.wh};
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double x[3] = {0, 0, 0}, v[3] = {0, 0, 0}, R[3] = {0, 0, 0}, c = 0, h = 0, divv = 0, xm = 0, kx = 0;
    const AvSeedV sk = avSeedOf(a, k);
    const double hInvK = a.hInv[k], divvK = a.divv[k], volK = a.vol[k], kxInvK = a.kxInv[k];
    const unsigned cnt = ov.size(k);
    for (unsigned q = 0; q < cnt; ++q) {
        bool mutual;
        const uint32_t j = ov.at(k, q, mutual);
        const bool wantK = sk.any && (sk.gAny || j == sk.arg);
        AvSeedV sj{};
        bool wantJ = false;
        if (mutual) {
            sj = avSeedOf(a, j);
            wantJ = sj.any && (sj.gAny || uint32_t(k) == sj.arg);
        }
        if (!wantK && !wantJ) continue;
        double r[3], d, rinv, vv[3];
        geom(a, k, j, r, d, rinv);
        vdiff(a, k, j, vv);
        double rj[3] = {0, 0, 0}, vj[3] = {0, 0, 0}, cj = 0, hj = 0, divvj = 0, xmj = 0, kxj = 0;
        const double divvJ = a.divv[j];
        if (wantK) {
            double dw;
            const double w = lookupVS(tw, d * hInvK, dw);
            AvGrad o;
            avAdj(r, d, rinv, vv, hInvK, w, dw, a.K, a.vol[j], a.kxInv[j], divvK, divvJ, sk.CGb, sk.vsigb,
                  j == sk.arg, o);
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                x[t] += o.r[t];
                v[t] += o.v[t];
                R[t] += o.R[t];
                rj[t] -= o.r[t];
                vj[t] -= o.v[t];
            }
            c += o.cI;
            h += o.hI;
            divv += o.divvI;
            cj += o.cJ;
            divvj += o.divvJ;
            xmj += o.xmJ;
            kxj += o.kxJ;
        }
        if (wantJ) {
            const double hInvJ = a.hInv[j];
            double dw;
            const double w = lookupVS(tw, d * hInvJ, dw);
            const double rm[3] = {-r[0], -r[1], -r[2]}, vm[3] = {-vv[0], -vv[1], -vv[2]};
            AvGrad p;
            avAdj(rm, d, rinv, vm, hInvJ, w, dw, a.K, volK, kxInvK, divvJ, divvK, sj.CGb, sj.vsigb,
                  uint32_t(k) == sj.arg, p);
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                rj[t] += p.r[t];
                vj[t] += p.v[t];
                x[t] -= p.r[t];
                v[t] -= p.v[t];
                atomicAdd(a.Rav + t * a.n + j, p.R[t]);
            }
            cj += p.cI;
            c += p.cJ;
            hj = p.hI;
            divvj += p.divvI;
            divv += p.divvJ;
            xm += p.xmJ;
            kx += p.kxJ;
            atomicAdd(a.bh + j, hj);
        }
        atomicAdd(a.bx + j, rj[0]);
        atomicAdd(a.by + j, rj[1]);
        atomicAdd(a.bz + j, rj[2]);
        if (vj[0] != 0.0 || vj[1] != 0.0 || vj[2] != 0.0) {
            atomicAdd(a.bvx + j, vj[0]);
            atomicAdd(a.bvy + j, vj[1]);
            atomicAdd(a.bvz + j, vj[2]);
            atomicAdd(a.cB + j, cj);
        }
        atomicAdd(a.divvB + j, divvj);
        atomicAdd(a.xmB + j, xmj);
        atomicAdd(a.kxB + j, kxj);
    }
    atomicAdd(a.bx + k, x[0]);
    atomicAdd(a.by + k, x[1]);
    atomicAdd(a.bz + k, x[2]);
    atomicAdd(a.bvx + k, v[0]);
    atomicAdd(a.bvy + k, v[1]);
    atomicAdd(a.bvz + k, v[2]);
    atomicAdd(a.cB + k, c);
    atomicAdd(a.bh + k, h);
    atomicAdd(a.divvB + k, divv);
    atomicAdd(a.xmB + k, xm);
    atomicAdd(a.kxB + k, kx);
#pragma unroll
    for (int t = 0; t < 3; ++t) atomicAdd(a.Rav + t * a.n + k, R[t]);
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
    {  // C partials of the AV pair terms
        const double Gb[3] = {a.GB[k], a.GB[a.n + k], a.GB[2 * a.n + k]};
        const double R[3] = {a.Rav[k], a.Rav[a.n + k], a.Rav[2 * a.n + k]};
        avCbar(Gb, R, Cb);
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

template<bool Smooth>
__device__ __forceinline__ void iadPair(const VeAdjArgs& a, int64_t i, int64_t j, const double tauB[6],
                                        const double PB[9], IadGrad& o)
{
    const KTab<Smooth> tw{a.wh};
    double r[3], d, rinv, v[3];
    geom(a, i, j, r, d, rinv);
    vdiff(a, i, j, v);
    const double hInv = a.hInv[i];
    double dw;
    const double w = lookupVS(tw, d * hInv, dw);
    iadDivvAdj(r, d, rinv, v, hInv, w, dw, a.vol[j], a.kxInv[j], a.xm[j], tauB, PB, o);
}

__device__ __forceinline__ void iadSeedOf(const VeAdjArgs& a, int64_t i, double tauB[6], double PB[9])
{
#pragma unroll
    for (int t = 0; t < 6; ++t) tauB[t] = a.tauB[t * a.n + i];
#pragma unroll
    for (int t = 0; t < 9; ++t) PB[t] = a.PB[t * a.n + i];
}

template<bool TwoSided, bool Smooth>
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
            iadPair<Smooth>(a, k, j, tauB, PB, o);
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
            iadPair<Smooth>(a, i, k, tauB, PB, o);
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

// scatter form over the owned lists: a mutual pair gives both directed terms from one geometry
// (the neighbour's term with r -> -r, v -> -v and the roles swapped), a one-sided entry its owner's
template<bool Smooth>
__global__ void __launch_bounds__(kVeAdjBlock) veIadAdjOnceKernel(VeAdjArgs a, OwnedView ov)
{
    const KTab<Smooth> tw{a.wh};
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double x[3] = {0, 0, 0}, v[3] = {0, 0, 0}, h = 0, xm = 0, kx = 0;
    double tauK[6], PK[9];
    iadSeedOf(a, k, tauK, PK);
    const double hInvK = a.hInv[k];
    const unsigned cnt = ov.size(k);
    for (unsigned q = 0; q < cnt; ++q) {
        bool mutual;
        const uint32_t j = ov.at(k, q, mutual);
        double r[3], d, rinv, vv[3];
        geom(a, k, j, r, d, rinv);
        vdiff(a, k, j, vv);
        double dw;
        double w = lookupVS(tw, d * hInvK, dw);
        IadGrad o;
        iadDivvAdj(r, d, rinv, vv, hInvK, w, dw, a.vol[j], a.kxInv[j], a.xm[j], tauK, PK, o);
        double rj[3], vj[3], hj = 0.0;
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            x[t] += o.r[t];
            v[t] += o.v[t];
            rj[t] = -o.r[t];
            vj[t] = -o.v[t];
        }
        h += o.hI;
        if (mutual) {
            double tauJ[6], PJ[9];
            iadSeedOf(a, j, tauJ, PJ);
            const double hInvJ = a.hInv[j];
            const double rm[3] = {-r[0], -r[1], -r[2]}, vm[3] = {-vv[0], -vv[1], -vv[2]};
            w = lookupVS(tw, d * hInvJ, dw);
            IadGrad p;
            iadDivvAdj(rm, d, rinv, vm, hInvJ, w, dw, a.vol[k], a.kxInv[k], a.xm[k], tauJ, PJ, p);
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                rj[t] += p.r[t];
                vj[t] += p.v[t];
                x[t] -= p.r[t];
                v[t] -= p.v[t];
            }
            hj = p.hI;
            xm += p.xmJ;
            kx += p.kxJ;
            atomicAdd(a.bh + j, hj);
        }
        atomicAdd(a.bx + j, rj[0]);
        atomicAdd(a.by + j, rj[1]);
        atomicAdd(a.bz + j, rj[2]);
        atomicAdd(a.bvx + j, vj[0]);
        atomicAdd(a.bvy + j, vj[1]);
        atomicAdd(a.bvz + j, vj[2]);
        atomicAdd(a.xmB + j, o.xmJ);
        atomicAdd(a.kxB + j, o.kxJ);
    }
    atomicAdd(a.bx + k, x[0]);
    atomicAdd(a.by + k, x[1]);
    atomicAdd(a.bz + k, x[2]);
    atomicAdd(a.bvx + k, v[0]);
    atomicAdd(a.bvy + k, v[1]);
    atomicAdd(a.bvz + k, v[2]);
    atomicAdd(a.bh + k, h);
    atomicAdd(a.xmB + k, xm);
    atomicAdd(a.kxB + k, kx);
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

template<bool Smooth>
__device__ __forceinline__ void gradhPair(const VeAdjArgs& a, int64_t i, int64_t j, GradhGrad& o)
{
    const KTab<Smooth> tw{a.wh};
    const KTab<Smooth> tdw{a.whd};
    double r[3], d, rinv;
    geom(a, i, j, r, d, rinv);
    const double hInv = a.hInv[i];
    double dw, dwd;
    const double w = lookupVS(tw, d * hInv, dw);
    const double wd = lookupVS(tdw, d * hInv, dwd);
    gradhAdj(r, d, rinv, hInv, w, dw, wd, dwd, a.xm[j], a.m[j], a.Skx[i], a.Som[i], a.Sr0[i], o);
}

template<bool TwoSided, bool Smooth>
__global__ void __launch_bounds__(kVeAdjBlock) veGradhAdjKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double x[3] = {0, 0, 0}, h = 0, xm = 0;
    const unsigned nc = a.lv.capped(k);
    for (unsigned q = 0; q < nc; ++q) {
        const int64_t j = a.lv.at(k, q);
        GradhGrad o;
        gradhPair<Smooth>(a, k, j, o);
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
            gradhPair<Smooth>(a, i, k, o);
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

template<bool Smooth>
__global__ void __launch_bounds__(kVeAdjBlock) veGradhAdjOnceKernel(VeAdjArgs a, OwnedView ov)
{
    const KTab<Smooth> tw{a.wh};
    const KTab<Smooth> tdw{a.whd};
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double x[3] = {0, 0, 0}, h = 0, xm = 0;
    const double hInvK = a.hInv[k], skx = a.Skx[k], som = a.Som[k], sr0 = a.Sr0[k];
    const double xmK = a.xm[k], mK = a.m[k];
    const unsigned cnt = ov.size(k);
    for (unsigned q = 0; q < cnt; ++q) {
        bool mutual;
        const uint32_t j = ov.at(k, q, mutual);
        double r[3], d, rinv;
        geom(a, k, j, r, d, rinv);
        double dw, dwd;
        double w = lookupVS(tw, d * hInvK, dw), wd = lookupVS(tdw, d * hInvK, dwd);
        GradhGrad o;
        gradhAdj(r, d, rinv, hInvK, w, dw, wd, dwd, a.xm[j], a.m[j], skx, som, sr0, o);
        double rj[3];
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            x[t] += o.r[t];
            rj[t] = -o.r[t];
        }
        h += o.hI;
        if (mutual) {
            const double hInvJ = a.hInv[j];
            const double rm[3] = {-r[0], -r[1], -r[2]};
            w = lookupVS(tw, d * hInvJ, dw);
            wd = lookupVS(tdw, d * hInvJ, dwd);
            GradhGrad p;
            gradhAdj(rm, d, rinv, hInvJ, w, dw, wd, dwd, xmK, mK, a.Skx[j], a.Som[j], a.Sr0[j], p);
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                rj[t] += p.r[t];
                x[t] -= p.r[t];
            }
            xm += p.xmJ;
            atomicAdd(a.bh + j, p.hI);
        }
        atomicAdd(a.bx + j, rj[0]);
        atomicAdd(a.by + j, rj[1]);
        atomicAdd(a.bz + j, rj[2]);
        atomicAdd(a.xmB + j, o.xmJ);
    }
    atomicAdd(a.bx + k, x[0]);
    atomicAdd(a.by + k, x[1]);
    atomicAdd(a.bz + k, x[2]);
    atomicAdd(a.bh + k, h);
    atomicAdd(a.xmB + k, xm);
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

template<bool Smooth>
__device__ __forceinline__ void xmassPair(const VeAdjArgs& a, int64_t i, int64_t j, double rb[3], double& hIb)
{
    const KTab<Smooth> tw{a.wh};
    double r[3], d, rinv;
    geom(a, i, j, r, d, rinv);
    const double hInv = a.hInv[i];
    double dw;
    lookupVS(tw, d * hInv, dw);
    xmassAdj(r, d, rinv, hInv, dw, a.m[j], a.R0b[i], rb, hIb);
}

template<bool TwoSided, bool Smooth>
__global__ void __launch_bounds__(kVeAdjBlock) veXmassAdjKernel(VeAdjArgs a)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double x[3] = {0, 0, 0}, h = 0;
    const unsigned nc = a.lv.capped(k);
    for (unsigned q = 0; q < nc; ++q) {
        const int64_t j = a.lv.at(k, q);
        double rb[3], hIb;
        xmassPair<Smooth>(a, k, j, rb, hIb);
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
            xmassPair<Smooth>(a, i, k, rb, hIb);
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

template<bool Smooth>
__global__ void __launch_bounds__(kVeAdjBlock) veXmassAdjOnceKernel(VeAdjArgs a, OwnedView ov)
{
    const KTab<Smooth> tw{a.wh};
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= a.n) return;
    double x[3] = {0, 0, 0}, h = 0;
    const double hInvK = a.hInv[k], r0b = a.R0b[k], mK = a.m[k];
    const unsigned cnt = ov.size(k);
    for (unsigned q = 0; q < cnt; ++q) {
        bool mutual;
        const uint32_t j = ov.at(k, q, mutual);
        double r[3], d, rinv;
        geom(a, k, j, r, d, rinv);
        double dw;
        lookupVS(tw, d * hInvK, dw);
        double rb[3], hIb;
        xmassAdj(r, d, rinv, hInvK, dw, a.m[j], r0b, rb, hIb);
        h += hIb;
        if (mutual) {
            const double hInvJ = a.hInv[j];
            const double rm[3] = {-r[0], -r[1], -r[2]};
            lookupVS(tw, d * hInvJ, dw);
            double pb[3], hJb;
            xmassAdj(rm, d, rinv, hInvJ, dw, mK, a.R0b[j], pb, hJb);
#pragma unroll
            for (int t = 0; t < 3; ++t) rb[t] -= pb[t];
            atomicAdd(a.bh + j, hJb);
        }
#pragma unroll
        for (int t = 0; t < 3; ++t) x[t] += rb[t];
        atomicAdd(a.bx + j, -rb[0]);
        atomicAdd(a.by + j, -rb[1]);
        atomicAdd(a.bz + j, -rb[2]);
    }
    atomicAdd(a.bx + k, x[0]);
    atomicAdd(a.by + k, x[1]);
    atomicAdd(a.bz + k, x[2]);
    atomicAdd(a.bh + k, h);
}

}  // namespace

// number of n-sized double sections of the VE adjoint state
constexpr int kVeAdjSections = 78;

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
    a.wh = tabW64(c);
    a.whd = tabDW64(c);
    a.K = c->K;
    a.gamma = c->prm.gamma;
    a.av = AvPrm{c->K, c->prm.minDt, c->prm.alphamin, c->prm.alphamax, c->prm.decay_constant};
    a.box = c->box;
    {  // FP32 error of a position difference: a few ulp of the largest coordinate plus a box edge
        double xmax = 0.0, lmax = 0.0;
        for (int k = 0; k < 3; ++k) {
            xmax = fmax(xmax, fmax(fabs(c->box.lo[k]), fabs(c->box.hi[k])));
            lmax = fmax(lmax, c->box.L[k]);
        }
        a.ePos = float(4.0 * 0x1p-24 * (xmax + lmax) * 1.001);
    }
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
    a.Rav = take(3);
    const int64_t accSections = 23;
    a.hInv = take(1);
    a.rho = take(1);
    a.rhoInv = take(1);
    a.vol = take(1);
    a.kxInv = take(1);
    a.xmInv = take(1);
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
    a.CGB = take(3);
    a.vsigB = take(1);
    a.tauB = take(6);
    a.PB = take(9);
    a.Skx = take(1);
    a.Som = take(1);
    a.Sr0 = take(1);
    a.R0b = take(1);
    a.xc32 = reinterpret_cast<float4*>(take(2));
    a.v32 = reinterpret_cast<float4*>(take(2));
    if ((reinterpret_cast<uintptr_t>(a.xc32) | reinterpret_cast<uintptr_t>(a.v32)) & 15) return SPHGB_ERR_STATE;
    if (q - st > int64_t(kVeAdjSections) * n) return SPHGB_ERR_TOO_LARGE;  // layout and size disagree

    for (double* z : {g->x, g->y, g->z, g->vx, g->vy, g->vz, g->h, g->u})
        SPHGB_CUDA(cudaMemsetAsync(z, 0, sizeof(double) * n, c->stream));
    SPHGB_CUDA(cudaMemsetAsync(st, 0, sizeof(double) * accSections * n, c->stream));

    const unsigned pb = gridFor(n, kVeAdjBlock), eb = gridFor(n, 256);
    const bool two = deterministic != 0;
    veQuotKernel<<<eb, 256, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "veQuotKernel"));
    const bool withDu = a.sDu != nullptr;
    // forward sums kept by the forward passes on these lists (sphgb_set_adjoint_tape) are read from
    // the tape instead of being summed again; vsig_i and its pair are always found here
    constexpr unsigned kTapeNeeded = kTapeGradh | kTapeIad | kTapeAv;
    const bool taped = c->tapeEpoch == c->nbrEpoch && c->tapeN == n && (c->tapeMask & kTapeNeeded) == kTapeNeeded;
    const bool tapedMe = taped && (c->tapeMask & kTapeMe) != 0;
    if (taped) {
        double* tp = c->veTape.as<double>();
        a.G = tp + int64_t(kTapeG) * n;
        a.P = tp + int64_t(kTapeP) * n;
        a.wom = tp + int64_t(kTapeWom) * n;
        a.wr0 = tp + int64_t(kTapeWr0) * n;
        if (tapedMe) {
            a.en = tp + int64_t(kTapeEn) * n;
            a.avE = tp + int64_t(kTapeAvE) * n;
        }
    }
    return withKernelForm(c, [&](auto smooth) -> int {
        constexpr bool S = decltype(smooth)::value;
        if (withDu && !tapedMe) {  // en and avE enter only through the du seed
            vePreMeKernel<S><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
            SPHGB_TRY(launched(c, "vePreMeKernel"));
        }
        if (taped) {
            veArgKernel<<<pb, kVeAdjBlock, 0, c->stream>>>(a);
            SPHGB_TRY(launched(c, "veArgKernel"));
        } else {
            vePreKernel<S><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
            SPHGB_TRY(launched(c, "vePreKernel"));
        }
        {
            using K = void (*)(VeAdjArgs);
            // [two-sided][avClean][du seed]
            const K me[2][2][2] = {{{meVeAdjKernel<false, false, false, S>, meVeAdjKernel<false, false, true, S>},
                                    {meVeAdjKernel<false, true, false, S>, meVeAdjKernel<false, true, true, S>}},
                                   {{meVeAdjKernel<true, false, false, S>, meVeAdjKernel<true, false, true, S>},
                                    {meVeAdjKernel<true, true, false, S>, meVeAdjKernel<true, true, true, S>}}};
            // one evaluation per mutual pair: owned lists of the current lists, order-free sums allowed
            if (!two && !c->deterministic && !a.avClean && c->ownedEpoch == c->nbrEpoch && !c->ownedFromLists) {
                if (withDu) meVeAdjOnceKernel<true, S><<<pb, kVeAdjBlock, 0, c->stream>>>(a, ownedView(c));
                else meVeAdjOnceKernel<false, S><<<pb, kVeAdjBlock, 0, c->stream>>>(a, ownedView(c));
            } else
                me[two][a.avClean][withDu]<<<pb, kVeAdjBlock, 0, c->stream>>>(a);
            SPHGB_TRY(launched(c, "meVeAdjKernel"));
        }
        veAvSeedKernel<<<eb, 256, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "veAvSeedKernel"));
        const bool once = !two && !c->deterministic && c->ownedEpoch == c->nbrEpoch && !c->ownedFromLists;
        if (two) veAvAdjKernel<true, S><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
        else if (once) veAvAdjOnceKernel<S><<<pb, kVeAdjBlock, 0, c->stream>>>(a, ownedView(c));
        else veAvAdjKernel<false, S><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "veAvAdjKernel"));
        veIadSeedKernel<<<eb, 256, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "veIadSeedKernel"));
        if (two) veIadAdjKernel<true, S><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
        else if (once) veIadAdjOnceKernel<S><<<pb, kVeAdjBlock, 0, c->stream>>>(a, ownedView(c));
        else veIadAdjKernel<false, S><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "veIadAdjKernel"));
        veEosAdjKernel<<<eb, 256, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "veEosAdjKernel"));
        veGradhSeedKernel<<<eb, 256, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "veGradhSeedKernel"));
        if (two) veGradhAdjKernel<true, S><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
        else if (once) veGradhAdjOnceKernel<S><<<pb, kVeAdjBlock, 0, c->stream>>>(a, ownedView(c));
        else veGradhAdjKernel<false, S><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "veGradhAdjKernel"));
        veXmassSeedKernel<<<eb, 256, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "veXmassSeedKernel"));
        if (two) veXmassAdjKernel<true, S><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
        else if (once) veXmassAdjOnceKernel<S><<<pb, kVeAdjBlock, 0, c->stream>>>(a, ownedView(c));
        else veXmassAdjKernel<false, S><<<pb, kVeAdjBlock, 0, c->stream>>>(a);
        SPHGB_TRY(launched(c, "veXmassAdjKernel"));
        SPHGB_CUDA(cudaStreamSynchronize(c->stream));
        return SPHGB_OK;
    });
}

}  // namespace sphgb
