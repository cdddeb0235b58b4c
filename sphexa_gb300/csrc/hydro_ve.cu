// Volume-element SPH pair passes with the artificial-viscosity switch.
//
// Reference j-loops restated:
//   gradh     -> veDefGradhJLoop (sph/include/sph/hydro_ve/ve_def_gradh_kern.hpp:43-90)
//   EOS       -> computeIdealGasEOS_Impl (hydro_ve/eos.hpp:52-94)
//   IAD+divv  -> IADJLoop then divV_curlVJLoop over the same list in one kernel
//                (hydro_ve/iad_kern.hpp:43-109, divv_curlv_kern.hpp:43-123)
//   AV switch -> AVswitchesJLoop (hydro_ve/av_switches_kern.hpp:43-137)
//   ME        -> momentumAndEnergyJLoop<avClean> + avRvCorrection (hydro_ve/momentum_energy_kern.hpp)
//
// The passes are FP64-pipe bound in the FP64 form, so the pair loops spend as few FP64
// instructions as the result allows: quotients of per-particle fields (rho_j, m_j/rho_j,
// xm_j/kx_j, m_j*prho_j) are formed once per particle; 1/|r| comes from rsqrt and serves both
// |r| and rv/|r|; the Atwood-number branches are decided by comparison, and the ramp's four
// pow() calls become one exp() of the precomputed ln xm difference; the periodic wrap tests run
// only for targets whose 2h box touches a periodic face; inside a sweep the pair-once passes read
// r, v_j - v_i, |r|, 1/|r| and both kernel values from the cache the xmass pass fills (PairGeo).
// Results agree with the reference to rounding (<= 1e-12 relative).  The mixed form runs the same
// loops in FP32 on grid-local offsets with Kahan sums.
#include "pairs.cuh"

namespace sphgb {

namespace {

// ---------------------------------------------------------------- per-particle quotients
// aux = {rho, m/rho, xm/kx, m*prho, ln xm, 1/rho} x n; a pass asks only for the parts it reads
enum AuxPart : int { kAuxVol = 1, kAuxMe = 2 };

template<class T, int Parts>
__global__ void veAuxKernel(int64_t n, const void* m, const void* kx, const void* xm, const void* prho, T* aux)
{
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    T mi = ld<T>(m, i), kxi = ld<T>(kx, i), xmi = ld<T>(xm, i);
    if constexpr ((Parts & kAuxVol) != 0) aux[2 * n + i] = xmi / kxi;
    if constexpr ((Parts & kAuxMe) != 0) {
        T rho = kxi * mi / xmi;
        aux[i] = rho;
        aux[n + i] = mi / rho;
        aux[3 * n + i] = mi * ld<T>(prho, i);
        if constexpr (std::is_same_v<T, double>) aux[4 * n + i] = log(xmi);
        else aux[4 * n + i] = log2f(xmi);
        aux[5 * n + i] = T(1) / rho;
    }
}

// all aux parts of particle i from its own m, kx, xm, prho (the sweep forms them once, fused)
template<class T>
__device__ __forceinline__ void veAuxAll(int64_t n, int64_t i, T mi, T kxi, T xmi, T prhoi, T* aux)
{
    const T rho = kxi * mi / xmi;
    aux[i] = rho;
    aux[n + i] = mi / rho;
    aux[2 * n + i] = xmi / kxi;
    aux[3 * n + i] = mi * prhoi;
    if constexpr (std::is_same_v<T, double>) aux[4 * n + i] = log(xmi);
    else aux[4 * n + i] = log2f(xmi);
    aux[5 * n + i] = T(1) / rho;
}

template<class P, int Parts>
int launchVeAux(sphgb_ctx* c, const sphgb_particles* p)
{
    using T = typename P::T;
    const int64_t n = p->n;
    SPHGB_TRY(c->aux.ensure(sizeof(T) * 6 * n));
    veAuxKernel<T, Parts><<<gridFor(n, 256), 256, 0, c->stream>>>(n, p->m, p->kx, p->xm, p->prho, c->aux.as<T>());
    return launched(c, "veAuxKernel");
}

template<int Parts>
int launchVeAux(sphgb_ctx* c, const sphgb_particles* p)
{
    if (c->inSweep && c->auxReady) return SPHGB_OK;  // formed by the fused EOS of this sweep
    return p->precision == SPHGB_MIXED ? launchVeAux<MixedTag, Parts>(c, p) : launchVeAux<Fp64Tag, Parts>(c, p);
}

// ---------------------------------------------------------------- gradh (kx, gradh)
// neighbour-side fields of the mixed gradh pass: grid position, xm and m in one 32-byte block per
// particle (one 256-bit load)
__global__ void packGradhKernel(int64_t n, const void* xm, const void* m, const u64* __restrict__ cell,
                                const float4* __restrict__ loc, float4* __restrict__ rec)
{
    const int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (j >= n) return;
    packGridBlock(rec + 2 * j, cell[j], loc[j], ld<float>(xm, j), ld<float>(m, j), 0.f);
}

template<class P, bool Smooth = false>
__global__ void __launch_bounds__(kPairBlock) gradhKernel(ListView lv, CoordFp64 cf, CoordMixed cm, const void* h,
                                                          const void* m, const void* xm, const void* wh,
                                                          const void* whd, const double2* w64, const double2* dw64,
                                                          double K,
                                                          void* kxOut, void* gradhOut,
                                                          double* tapeWom = nullptr, double* tapeWr0 = nullptr,
                                                          const Rec8* rec = nullptr)
{
    const int64_t i = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last) return;
    const int64_t ii = i - lv.first;
    const unsigned nc = lv.capped(ii);
    if constexpr (std::is_same_v<P, Fp64Tag>) {
        const KTab<Smooth> tw{w64}, tdw{dw64};
        auto t = cf.target(i);
        double hi = ld<double>(h, i), mi = ld<double>(m, i), xmi = ld<double>(xm, i);
        double hInv = 1.0 / hi, h3Inv = hInv * hInv * hInv, twoH = 2.0 * hi, hInvDx = hInv * kTabInvDx;
        const bool wrap = cf.needsWrap(t, twoH);
        double kxi = xmi, whomega = -3.0 * xmi, wrho0 = -3.0 * mi;
        for (unsigned k = 0; k < nc; ++k) {
            uint32_t j = lv.at(ii, k);
            double rx, ry, rz;
            cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
            double r2 = dist2(rx, ry, rz);
            double dist = r2 * invDist(r2);
            double v = dist * hInv;
            const TabSlot sl = tabSlot(dist * hInvDx);
            double w = lookupX(tw, sl), dw = lookupX(tdw, sl);
            double dterh = -(3.0 * w + v * dw);
            double xmj = ld<double>(xm, j);
            kxi += w * xmj;
            whomega += dterh * xmj;
            wrho0 += dterh * ld<double>(m, j);
        }
        kxi *= K * h3Inv;
        whomega *= K * h3Inv * hInv;
        wrho0 *= K * h3Inv * hInv;
        if (tapeWom) {
            tapeWom[i] = whomega;
            tapeWr0[i] = wrho0;
        }
        whomega = whomega * mi / xmi + (kxi - K * xmi * h3Inv) * wrho0;
        double rhoi = kxi * mi / xmi;
        double dhdrho = -hi / (rhoi * 3.0);
        st<double>(kxOut, i, kxi);
        st<double>(gradhOut, i, 1.0 - dhdrho * whomega);
    } else {
        auto t = cm.target(i);
        float mi = ld<float>(m, i), xmi = ld<float>(xm, i);
        KSum kx, whom, wr0;
        kx.add(xmi);
        whom.add(-3.f * xmi);
        wr0.add(-3.f * mi);
        // the list is read a granule (four entries) per load, the next granule one ahead, and the
        // next neighbour's block is loaded while the current pair is evaluated
        uint4 G = nc > 0 ? lv.granule(ii, 0) : make_uint4(uint32_t(i), 0u, 0u, 0u);
        uint4 Gn = nc > 4 ? lv.granule(ii, 1) : G;
        Rec8 Bn = ldRec8(rec + G.x);
        for (unsigned k = 0; k < nc; ++k) {
            const Rec8 B = Bn;  // cell xl yl zl xm m
            if (k + 1 < nc) {
                const unsigned s = (k + 1) & 3u;
                if (s == 0) {
                    G = Gn;
                    if (k + 5 < nc) Gn = lv.granule(ii, (k + 5) >> 2);
                }
                Bn = ldRec8(rec + pick(G, s));
            }
            float rx, ry, rz;
            cm.diffBlock(t, B, rx, ry, rz);
            float dist = sqrtf(fmaf(rx, rx, fmaf(ry, ry, rz * rz)));
            float v = dist * t.hInv;
            float w, dw;
            lookupH32Pair(static_cast<const float4*>(wh), static_cast<const float4*>(whd), v, w, dw);
            float dterh = -(3.f * w + v * dw);
            kx.add(w * B.v[5]);
            whom.add(dterh * B.v[5]);
            wr0.add(dterh * B.v[6]);
        }
        double hi = double(ld<float>(h, i)), hInv = 1.0 / hi, h3Inv = hInv * hInv * hInv;
        double kxi = kx.value64() * (K * h3Inv);
        double wo = whom.value64() * (K * h3Inv * hInv);
        double wr = wr0.value64() * (K * h3Inv * hInv);
        wo = wo * double(mi) / double(xmi) + (kxi - K * double(xmi) * h3Inv) * wr;
        double rhoi = kxi * double(mi) / double(xmi);
        double dhdrho = -hi / (rhoi * 3.0);
        st<float>(kxOut, i, float(kxi));
        st<float>(gradhOut, i, float(1.0 - dhdrho * wo));
    }
}

// ---------------------------------------------------------------- EOS (ideal gas, VE)
// computeIdealGasEOS_Impl (hydro_ve/eos.hpp:52-94) for particle i; returns prho in the field type
template<class T>
__device__ __forceinline__ T eosVe(int64_t i, double ui, T mi, T kxi, T xmi, T gradhi, double gamma, void* prho,
                                   void* c, void* rho, void* p)
{
    T rhoi = kxi * mi / xmi;
    double tmp = ui * (gamma - 1.0);
    double pi = double(rhoi) * tmp;
    const T prhoi = T(pi / double(kxi * mi * mi * gradhi));
    st<T>(prho, i, prhoi);
    st<T>(c, i, T(sqrt(gamma * tmp)));
    if (rho) st<T>(rho, i, rhoi);
    if (p) st<T>(p, i, T(pi));
    return prhoi;
}

template<class P>
__global__ void eosVeKernel(int64_t first, int64_t last, const double* u, const void* m, const void* kx,
                            const void* xm, const void* gradh, double gamma, void* prho, void* c, void* rho, void* p)
{
    using T = typename P::T;
    int64_t i = first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= last) return;
    eosVe<T>(i, u[i], ld<T>(m, i), ld<T>(kx, i), ld<T>(xm, i), ld<T>(gradh, i), gamma, prho, c, rho, p);
}

// EOS fused with the per-particle quotients of the later passes (one read of m, kx, xm, gradh)
template<class P>
__global__ void eosAuxVeKernel(int64_t n, const double* u, const void* m, const void* kx, const void* xm,
                               const void* gradh, double gamma, void* prho, void* c, void* rho, void* p,
                               typename P::T* aux)
{
    using T = typename P::T;
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const T mi = ld<T>(m, i), kxi = ld<T>(kx, i), xmi = ld<T>(xm, i);
    const T prhoi = eosVe<T>(i, u[i], mi, kxi, xmi, ld<T>(gradh, i), gamma, prho, c, rho, p);
    veAuxAll<T>(n, i, mi, kxi, xmi, prhoi, aux);
}

// ---------------------------------------------------------------- IAD + divv/curlv
struct IadDivvArgs {
    const void *h, *vx, *vy, *vz, *xm, *kx, *wh;
    const double2* w64;  // FP64: W in the context's form (wh: the mixed pieces)
    const void* vol;    // aux: xm/kx per particle
    float* divvBound;   // mixed: error bound of divv per particle (refinement flag), may be null
    double K;
    void *c11, *c12, *c13, *c22, *c23, *c33, *divv, *curlv;
    void *dV11, *dV12, *dV13, *dV22, *dV23, *dV33;
    double* tapeP;  // FP64: P_i = sum xm_j W (v_j - v_i) r^T for the VE adjoint (9 x tapeN), or null
    int64_t tapeN;
    const Rec8* rec;    // mixed: neighbour blocks {cell xl yl zl vx vy vz} (packIadKernel)
    const float2* rec2; // mixed: {vol xm}
};

// neighbour-side fields of the mixed IAD + divv/curlv pass: the grid position and velocity in one
// 32-byte block (one 256-bit load) and {vol xm} in 8 bytes
__global__ void packIadKernel(int64_t n, const void* vx, const void* vy, const void* vz, const void* vol,
                              const void* xm, const u64* __restrict__ cell, const float4* __restrict__ loc,
                              float4* __restrict__ rec, float2* __restrict__ rec2)
{
    const int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (j >= n) return;
    packGridBlock(rec + 2 * j, cell[j], loc[j], ld<float>(vx, j), ld<float>(vy, j), ld<float>(vz, j));
    rec2[j] = make_float2(ld<float>(vol, j), ld<float>(xm, j));
}

// FP64 epilogue of IAD + divv/curlv for particle i from its sums tau = sum vol_j W r r^T and
// M = sum xm_j W (v_j - v_i) r^T: c_i = tau^-1 (iad_kern.hpp), dV = -M c_i and its trace, curl and
// symmetric part (divv_curlv_kern.hpp), and the adjoint tape's copy of M
__device__ __forceinline__ void iadEpilogue64(const IadDivvArgs& a, int64_t i, double hi, const double tau[6],
                                              const double M[9])
{
    using T = double;
    const T hiInv = 1.0 / hi;
    if (a.tapeP) {
#pragma unroll
        for (int q = 0; q < 9; ++q) a.tapeP[q * a.tapeN + i] = M[q];
    }
    T cc[6];
    iadInvert<T>(tau[0], tau[1], tau[2], tau[3], tau[4], tau[5], hi, a.K, cc);
    st<T>(a.c11, i, cc[0]);
    st<T>(a.c12, i, cc[1]);
    st<T>(a.c13, i, cc[2]);
    st<T>(a.c22, i, cc[3]);
    st<T>(a.c23, i, cc[4]);
    st<T>(a.c33, i, cc[5]);
    // dV[a][b] = -sum_c c_bc M[a][c]
    const T C[3][3] = {{cc[0], cc[1], cc[2]}, {cc[1], cc[3], cc[4]}, {cc[2], cc[4], cc[5]}};
    T dVx[3], dVy[3], dVz[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        dVx[b] = -(C[b][0] * M[0] + C[b][1] * M[1] + C[b][2] * M[2]);
        dVy[b] = -(C[b][0] * M[3] + C[b][1] * M[4] + C[b][2] * M[5]);
        dVz[b] = -(C[b][0] * M[6] + C[b][1] * M[7] + C[b][2] * M[8]);
    }
    T nk = a.K * (hiInv * hiInv * hiInv) / ld<T>(a.kx, i);
    st<T>(a.divv, i, nk * (dVx[0] + dVy[1] + dVz[2]));
    if (a.curlv) {
        T cv0 = dVz[1] - dVy[2], cv1 = dVx[2] - dVz[0], cv2 = dVy[0] - dVx[1];
        st<T>(a.curlv, i, nk * sqrt(cv0 * cv0 + (cv1 * cv1 + cv2 * cv2)));
    }
    if (a.dV11) {
        st<T>(a.dV11, i, nk * dVx[0]);
        st<T>(a.dV12, i, nk * (dVx[1] + dVy[0]));
        st<T>(a.dV13, i, nk * (dVx[2] + dVz[0]));
        st<T>(a.dV22, i, nk * dVy[1]);
        st<T>(a.dV23, i, nk * (dVy[2] + dVz[1]));
        st<T>(a.dV33, i, nk * dVz[2]);
    }
}

template<class P, bool Smooth = false>
__global__ void __launch_bounds__(kPairBlock, std::is_same_v<P, MixedTag> ? 7 : 1)
iadDivvKernel(ListView lv, CoordFp64 cf, CoordMixed cm, IadDivvArgs a)
{
    const int64_t i = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last) return;
    const int64_t ii = i - lv.first;
    const unsigned nc = lv.capped(ii);
    if constexpr (std::is_same_v<P, Fp64Tag>) {
        using T = double;
        const KTab<Smooth> tab{a.w64};
        auto t = cf.target(i);
        T hi = ld<T>(a.h, i), hiInv = 1.0 / hi, twoH = 2.0 * hi;
        const T hInvDx = hiInv * kTabInvDx;
        const bool wrap = cf.needsWrap(t, twoH);
        const T vxi = ld<T>(a.vx, i), vyi = ld<T>(a.vy, i), vzi = ld<T>(a.vz, i);
        // one walk over the list: tau = sum vol_j W r r^T and M = sum xm_j W (v_j - v_i) r^T;
        // the reference's second loop sums xm_j (v_j - v_i) (-(c_i r) W)^T, which is -M c_i^T
        // (c_i symmetric), so c_i is applied once after the walk instead of per pair
        T t11 = 0, t12 = 0, t13 = 0, t22 = 0, t23 = 0, t33 = 0;
        T M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (unsigned k = 0; k < nc; ++k) {
            uint32_t j = lv.at(ii, k);
            T rx, ry, rz;
            cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
            T r2 = dist2(rx, ry, rz);
            T w = lookupX(tab, r2 * invDist(r2) * hInvDx);
            T vw = ld<T>(a.vol, j) * w;
            T rxv = rx * vw, ryv = ry * vw, rzv = rz * vw;
            t11 += rx * rxv;
            t12 += ry * rxv;
            t13 += rz * rxv;
            t22 += ry * ryv;
            t23 += rz * ryv;
            t33 += rz * rzv;
            T xw = ld<T>(a.xm, j) * w;
            T sx = (ld<T>(a.vx, j) - vxi) * xw, sy = (ld<T>(a.vy, j) - vyi) * xw, sz = (ld<T>(a.vz, j) - vzi) * xw;
            M[0] += sx * rx;
            M[1] += sx * ry;
            M[2] += sx * rz;
            M[3] += sy * rx;
            M[4] += sy * ry;
            M[5] += sy * rz;
            M[6] += sz * rx;
            M[7] += sz * ry;
            M[8] += sz * rz;
        }
        const double tau[6] = {t11, t12, t13, t22, t23, t33};
        iadEpilogue64(a, i, hi, tau, M);
    } else {
        using T = float;
        auto t = cm.target(i);
        const T vxi = ld<T>(a.vx, i), vyi = ld<T>(a.vy, i), vzi = ld<T>(a.vz, i);
        // one walk, as in the FP64 form: tau and M = sum xm_j W (v_j - v_i) r^T, c_i applied after
        KSum t11, t12, t13, t22, t23, t33;
        KSum M[9];
        // A[a][c] = sum over pairs of |s_a| |r_c| >= sum |term| of M entry (a, c), s = xm_j W (v_j - v_i)
        float A[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (unsigned k = 0; k < nc; ++k) {
            uint32_t j = lv.at(ii, k);
            const Rec8 B = ldRec8(a.rec + j);  // cell xl yl zl vx vy vz
            const float2 Q = __ldg(a.rec2 + j);  // vol xm
            T rx, ry, rz;
            cm.diffBlock(t, B, rx, ry, rz);
            T dist = sqrtf(fmaf(rx, rx, fmaf(ry, ry, rz * rz)));
            T w = lookupH32(static_cast<const float4*>(a.wh), dist * t.hInv);
            T vw = Q.x * w;
            T rxv = rx * vw, ryv = ry * vw, rzv = rz * vw;
            t11.add(rx * rxv);
            t12.add(ry * rxv);
            t13.add(rz * rxv);
            t22.add(ry * ryv);
            t23.add(rz * ryv);
            t33.add(rz * rzv);
            T xw = Q.y * w;
            const T dvx = B.v[5] - vxi, dvy = B.v[6] - vyi, dvz = B.v[7] - vzi;
            T sx = dvx * xw, sy = dvy * xw, sz = dvz * xw;
            {
                const float as[3] = {fabsf(sx), fabsf(sy), fabsf(sz)}, ar[3] = {fabsf(rx), fabsf(ry), fabsf(rz)};
#pragma unroll
                for (int q = 0; q < 9; ++q) A[q] = fmaf(as[q / 3], ar[q % 3], A[q]);
            }
            M[0].add(sx * rx);
            M[1].add(sx * ry);
            M[2].add(sx * rz);
            M[3].add(sy * rx);
            M[4].add(sy * ry);
            M[5].add(sy * rz);
            M[6].add(sz * rx);
            M[7].add(sz * ry);
            M[8].add(sz * rz);
        }
        double hi = double(ld<T>(a.h, i));
        T cc[6];
        iadInvert<T>(t11.value(), t12.value(), t13.value(), t22.value(), t23.value(), t33.value(), hi, a.K, cc);
        st<T>(a.c11, i, cc[0]);
        st<T>(a.c12, i, cc[1]);
        st<T>(a.c13, i, cc[2]);
        st<T>(a.c22, i, cc[3]);
        st<T>(a.c23, i, cc[4]);
        st<T>(a.c33, i, cc[5]);
        // FP32 epilogue: the compensated sums collapse to FP32 (rounding 2^-24 of each entry), the
        // gradient sums and the normalisation run in FP32
        float m32[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) m32[q] = M[q].value();
        const float C[3][3] = {{cc[0], cc[1], cc[2]}, {cc[1], cc[3], cc[4]}, {cc[2], cc[4], cc[5]}};
        float gx[3], gy[3], gz[3];
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            gx[b] = -fmaf(C[b][0], m32[0], fmaf(C[b][1], m32[1], C[b][2] * m32[2]));
            gy[b] = -fmaf(C[b][0], m32[3], fmaf(C[b][1], m32[4], C[b][2] * m32[5]));
            gz[b] = -fmaf(C[b][0], m32[6], fmaf(C[b][1], m32[7], C[b][2] * m32[8]));
        }
        const float hInvF = t.hInv;
        const float nk = float(a.K) * (hInvF * hInvF * hInvF) / ld<T>(a.kx, i);
        st<T>(a.divv, i, nk * (gx[0] + gy[1] + gz[2]));
        if (a.divvBound) {
            // divv = -nk sum_ac C_ac M_ac with S = nk sum_ac |C_ac| A_ac >= the sum of |C_ac term| over
            // every entry and pair.  Its FP32 error is at most (eps_terms + eps_c + eps_xm + eps_kx) S
            // with the measured input errors (1e-7, 7e-7, 4e-7, 2e-7 relative), about 1.4e-6 S, plus
            // the epilogue's own rounding (a few 2^-24 S); the flag bound is 4e-6 S
            float sCA = 0.f;
#pragma unroll
            for (int q = 0; q < 9; ++q) sCA = fmaf(fabsf(C[q / 3][q % 3]), A[q], sCA);
            a.divvBound[i] = 4e-6f * fabsf(nk) * sCA;
        }
        if (a.curlv) {
            const float cv0 = gz[1] - gy[2], cv1 = gx[2] - gz[0], cv2 = gy[0] - gx[1];
            st<T>(a.curlv, i, nk * sqrtf(fmaf(cv0, cv0, fmaf(cv1, cv1, cv2 * cv2))));
        }
        if (a.dV11) {
            st<T>(a.dV11, i, nk * gx[0]);
            st<T>(a.dV12, i, nk * (gx[1] + gy[0]));
            st<T>(a.dV13, i, nk * (gx[2] + gz[0]));
            st<T>(a.dV22, i, nk * gy[1]);
            st<T>(a.dV23, i, nk * (gy[2] + gz[1]));
            st<T>(a.dV33, i, nk * gz[2]);
        }
    }
}

// ---------------------------------------------------------------- AV switches
struct AvArgs {
    const void *h, *vx, *vy, *vz, *c, *c11, *c12, *c13, *c22, *c23, *c33, *divv, *wh;
    const void* vol;  // aux: xm/kx
    double K, dt, alphamin, alphamax, decay;
    void* alpha;
    double* tapeG;  // FP64: G_i (3 x tapeN) for the VE adjoint, or null
    int64_t tapeN;
    const Rec8* rec;     // mixed: neighbour blocks {cell xl yl zl vx vy vz} and {c vol divv} (packAvKernel)
    const float4* rec2;
    const double2* w64;  // FP64: W in the context's form (wh: the mixed pieces)
};

// neighbour-side fields of the mixed AV-switch pass: the grid position and velocity in one 32-byte
// block (one 256-bit load) and {c vol divv} in 16 bytes
__global__ void packAvKernel(int64_t n, AvArgs a, const u64* __restrict__ cell, const float4* __restrict__ loc,
                             float4* __restrict__ rec, float4* __restrict__ rec2)
{
    const int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (j >= n) return;
    packGridBlock(rec + 2 * j, cell[j], loc[j], ld<float>(a.vx, j), ld<float>(a.vy, j), ld<float>(a.vz, j));
    rec2[j] = make_float4(ld<float>(a.c, j), ld<float>(a.vol, j), ld<float>(a.divv, j), 0.f);
}

// alpha update in the arithmetic of the field type (av_switches_kern.hpp:114-134)
template<class T>
__device__ __forceinline__ T avAlpha(const AvArgs& a, T alpha_i, T hi, T ci, T divvi, T vsig_i, T gx, T gy, T gz)
{
    T gdv = sqrt(gx * gx + gy * gy + gz * gz);
    T aloc = 0.0;
    if (divvi < T(0)) {
        T ac = hi * hi * gdv;
        aloc = T(a.alphamax) * ac / (ac + hi * fabs(divvi) + T(0.05) * ci);
    }
    if (aloc >= alpha_i) return aloc;
    T decay = hi / (T(a.decay) * vsig_i);
    T adot = (aloc >= T(a.alphamin)) ? (aloc - alpha_i) / decay : (T(a.alphamin) - alpha_i) / decay;
    return alpha_i + adot * T(a.dt);
}

template<class P, bool Smooth = false>
__global__ void __launch_bounds__(kPairBlock) avKernel(ListView lv, CoordFp64 cf, CoordMixed cm, AvArgs a)
{
    using T = typename P::T;
    const int64_t i = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last) return;
    const int64_t ii = i - lv.first;
    const unsigned nc = lv.capped(ii);
    T hi = ld<T>(a.h, i), ci = ld<T>(a.c, i);
    T vxi = ld<T>(a.vx, i), vyi = ld<T>(a.vy, i), vzi = ld<T>(a.vz, i);
    T c11 = ld<T>(a.c11, i), c12 = ld<T>(a.c12, i), c13 = ld<T>(a.c13, i);
    T c22 = ld<T>(a.c22, i), c23 = ld<T>(a.c23, i), c33 = ld<T>(a.c33, i);
    T vsig_i = T(1.e-40) * ci;
    T divvi = ld<T>(a.divv, i);
    T gx, gy, gz;
    if constexpr (std::is_same_v<P, Fp64Tag>) {
        auto t = cf.target(i);
        const KTab<Smooth> tabX{a.w64};
        T hiInv = 1.0 / hi, hiInv3 = hiInv * hiInv * hiInv, twoH = 2.0 * hi, hInvDx = hiInv * kTabInvDx;
        const bool wrap = cf.needsWrap(t, twoH);
        const T kh3 = a.K * hiInv3;
        // the reference sums fac_j (-(c_i r) W) per pair; with S = sum fac_j W r that is -c_i S,
        // so c_i is applied once after the walk
        T Sx = 0, Sy = 0, Sz = 0;
        long long vsigBits = __double_as_longlong(vsig_i);  // > 0
        for (unsigned k = 0; k < nc; ++k) {
            uint32_t j = lv.at(ii, k);
            T rx, ry, rz;
            cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
            T r2 = dist2(rx, ry, rz);
            T rinv = invDist(r2);
            T dist = r2 * rinv;
            T vxij = vxi - ld<T>(a.vx, j), vyij = vyi - ld<T>(a.vy, j), vzij = vzi - ld<T>(a.vz, j);
            T rv = fma(rz, vzij, fma(ry, vyij, rx * vxij));  // one order in every FP64 form
            if (negative(rv)) vsigBits = maxBitsNonNeg(vsigBits, fma(-3.0 * rv, rinv, ci + ld<T>(a.c, j)));
            T fw = ld<T>(a.vol, j) * (divvi - ld<T>(a.divv, j)) * lookupX(tabX, dist * hInvDx);
            Sx += fw * rx;
            Sy += fw * ry;
            Sz += fw * rz;
        }
        vsig_i = __longlong_as_double(vsigBits);
        gx = -kh3 * (c11 * Sx + c12 * Sy + c13 * Sz);
        gy = -kh3 * (c12 * Sx + c22 * Sy + c23 * Sz);
        gz = -kh3 * (c13 * Sx + c23 * Sy + c33 * Sz);
    } else {
        auto t = cm.target(i);
        const float kh3 = float(a.K) * t.hInv * t.hInv * t.hInv;
        KSum sx, sy, sz;
        // the list is read a granule (four entries) per load, the next granule one ahead, and the
        // next neighbour's fields are loaded while the current pair is evaluated
        uint4 G = nc > 0 ? lv.granule(ii, 0) : make_uint4(uint32_t(i), 0u, 0u, 0u);
        uint4 Gn = nc > 4 ? lv.granule(ii, 1) : G;
        Rec8 Bn = ldRec8(a.rec + G.x);
        float4 Qn = __ldg(a.rec2 + G.x);
        for (unsigned k = 0; k < nc; ++k) {
            const Rec8 B = Bn;     // cell xl yl zl vx vy vz
            const float4 Q = Qn;  // c vol divv
            if (k + 1 < nc) {
                const unsigned s = (k + 1) & 3u;
                if (s == 0) {
                    G = Gn;
                    if (k + 5 < nc) Gn = lv.granule(ii, (k + 5) >> 2);
                }
                const uint32_t jn = pick(G, s);
                Bn = ldRec8(a.rec + jn);
                Qn = __ldg(a.rec2 + jn);
            }
            T rx, ry, rz;
            cm.diffBlock(t, B, rx, ry, rz);
            T r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
            T rinv = rsqrtf(r2);
            T dist = r2 * rinv;
            T vxij = vxi - B.v[5], vyij = vyi - B.v[6], vzij = vzi - B.v[7];
            T rv = rx * vxij + ry * vyij + rz * vzij;
            if (rv < 0.f) vsig_i = fmaxf(vsig_i, ci + Q.x - 3.f * rv * rinv);
            T fw = Q.y * (divvi - Q.z) * lookupH32(static_cast<const float4*>(a.wh), dist * t.hInv);
            sx.add(fw * rx);
            sy.add(fw * ry);
            sz.add(fw * rz);
        }
        const double Sx = sx.value64(), Sy = sy.value64(), Sz = sz.value64();
        gx = T(-double(kh3) * (double(c11) * Sx + double(c12) * Sy + double(c13) * Sz));
        gy = T(-double(kh3) * (double(c12) * Sx + double(c22) * Sy + double(c23) * Sz));
        gz = T(-double(kh3) * (double(c13) * Sx + double(c23) * Sy + double(c33) * Sz));
    }
    if constexpr (std::is_same_v<P, Fp64Tag>) {
        if (a.tapeG) {
            a.tapeG[i] = gx;
            a.tapeG[a.tapeN + i] = gy;
            a.tapeG[2 * a.tapeN + i] = gz;
        }
    }
    st<T>(a.alpha, i, avAlpha<T>(a, ld<T>(a.alpha, i), hi, ci, divvi, vsig_i, gx, gy, gz));
}

// ---------------------------------------------------------------- momentum and energy (VE)
struct MeVeArgs {
    const void *vx, *vy, *vz, *h, *m, *prho, *c, *kx, *xm, *alpha;
    const void *c11, *c12, *c13, *c22, *c23, *c33;
    const void *dV11, *dV12, *dV13, *dV22, *dV23, *dV33;
    const void* wh;        // mixed: cubic pieces of W
    const double2* w64;    // FP64: W in the context's form
    const double* hInv64;  // [0,n) 1/h, [n,2n) 1/h^3, [2n,3n) 1/(h dx)
    const void* aux;       // rho, m/rho, xm/kx, m*prho, ln xm, 1/rho (6 x n)
    int64_t n;
    double K;
    float Kcour;
    void *ax, *ay, *az;
    double* du;
    float* groupDt;
    unsigned long long* minDt;
    // pair-once form: owned pair lists (j | mutual << 31) with their counts, and the accumulators
    // (mx my mz en avE, maxv bits) x n
    const uint32_t* owned;
    const uint32_t* ownedCount;
    double* acc;
    // mixed form: the neighbour side of a pair in three 32-byte blocks per particle (meVePackKernel):
    // {cell (2 words) xl yl zl 1/h vx vy} {vz c c11 c12 c13 c22 c23 c33} {m xm alpha rho m/rho m*prho}
    const Rec8* pack;
    // FP64: the energy sums (en, avE before max(0, .)) for the VE adjoint, or null
    double *tapeEn, *tapeAvE;
};

template<class T>
__device__ __forceinline__ T quadForm(T rx, T ry, T rz, const T g[6])
{
    T s0 = g[0] * rx + g[1] * ry + g[2] * rz;
    T s1 = g[3] * ry + g[4] * rz;
    T s2 = g[5] * rz;
    return rx * s0 + (ry * s1 + rz * s2);  // dot is a right fold (util/array.hpp:237-240)
}

// avRvCorrection (hydro_ve/momentum_energy_kern.hpp:43-63)
template<class T>
__device__ __forceinline__ T avRv(T rx, T ry, T rz, T eta, T etaCrit, const T gi[6], const T gj[6])
{
    T d1 = quadForm(rx, ry, rz, gi), d2 = quadForm(rx, ry, rz, gj), d3 = T(1);
    if (eta < etaCrit) {
        T e = T(5) * (eta - etaCrit);
        d3 = exp(-e * e);
    }
    T A = (d2 != T(0)) ? d1 / d2 : T(0);
    T Ap1 = T(1) + A;
    T phi = T(0.5) * d3 * fmax(T(0), fmin(T(1), T(4) * A / (Ap1 * Ap1)));
    return -phi * (d1 + d2);
}

// neighbour-side fields of the mixed momentum-energy pass as three 32-byte blocks per particle,
// the grid position (cell, in-cell offset, 1/h) included, each block read by one 256-bit load
__global__ void meVePackKernel(int64_t n, MeVeArgs a, const u64* __restrict__ cell, const float4* __restrict__ loc,
                               float4* __restrict__ pack)
{
    const int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (j >= n) return;
    const float m = ld<float>(a.m, j), xm = ld<float>(a.xm, j), kx = ld<float>(a.kx, j);
    const float rho = kx * m / xm;
    const u64 cj = cell[j];
    const float4 l = loc[j];
    float4* q = pack + 6 * j;
    q[0] = make_float4(__uint_as_float(unsigned(cj)), __uint_as_float(unsigned(cj >> 32)), l.x, l.y);
    q[1] = make_float4(l.z, l.w, ld<float>(a.vx, j), ld<float>(a.vy, j));
    q[2] = make_float4(ld<float>(a.vz, j), ld<float>(a.c, j), ld<float>(a.c11, j), ld<float>(a.c12, j));
    q[3] = make_float4(ld<float>(a.c13, j), ld<float>(a.c22, j), ld<float>(a.c23, j), ld<float>(a.c33, j));
    q[4] = make_float4(m, xm, ld<float>(a.alpha, j), rho);
    q[5] = make_float4(m / rho, m * ld<float>(a.prho, j), 0.f, 0.f);
}

template<class P, bool AvClean, bool Smooth = false>
__global__ void __launch_bounds__(kPairBlock) meVeKernel(ListView lv, CoordFp64 cf, CoordMixed cm, MeVeArgs a)
{
    using T = typename P::T;
    const int64_t i0 = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const bool valid = i0 < lv.last;
    const int64_t i = valid ? i0 : lv.first;
    const int64_t ii = i - lv.first;
    const unsigned nc = valid ? lv.capped(ii) : 0u;
    const T* aux = static_cast<const T*>(a.aux);
    const T *auxRho = aux, *auxMoR = aux + a.n, *auxMprho = aux + 3 * a.n, *auxLnXm = aux + 4 * a.n;
    constexpr T Atmin = T(0.1), Atmax = T(0.2), ramp = T(1) / (Atmax - Atmin);

    T hi = ld<T>(a.h, i), mi = ld<T>(a.m, i), ci = ld<T>(a.c, i), ai = ld<T>(a.alpha, i);
    T xmi = ld<T>(a.xm, i), prhoi = ld<T>(a.prho, i);
    T rhoi = auxRho[i], lnxmi = auxLnXm[i];
    T vxi = ld<T>(a.vx, i), vyi = ld<T>(a.vy, i), vzi = ld<T>(a.vz, i);
    T c11i = ld<T>(a.c11, i), c12i = ld<T>(a.c12, i), c13i = ld<T>(a.c13, i);
    T c22i = ld<T>(a.c22, i), c23i = ld<T>(a.c23, i), c33i = ld<T>(a.c33, i);
    T gi[6] = {0, 0, 0, 0, 0, 0};
    if constexpr (AvClean) {
        gi[0] = ld<T>(a.dV11, i);
        gi[1] = ld<T>(a.dV12, i);
        gi[2] = ld<T>(a.dV13, i);
        gi[3] = ld<T>(a.dV22, i);
        gi[4] = ld<T>(a.dV23, i);
        gi[5] = ld<T>(a.dV33, i);
    }
    const T etaCrit = T(cbrt(32.0 * M_PI / 3.0 / double(nc + 1)));
    const T xmi2 = xmi * xmi;
    (void)mi;
    T maxv = 0;
    double dt = INFINITY;

    if constexpr (std::is_same_v<P, Fp64Tag>) {
        auto t = cf.target(i);
        const KTab<Smooth> tabX{a.w64};
        const double* hInv = a.hInv64;
        const double* hInv3 = a.hInv64 + a.n;
        const double* hInvDx = a.hInv64 + 2 * a.n;
        T hiInv = hInv[i], hiInv3 = hInv3[i], hiInvDx = hInvDx[i], twoH = 2.0 * hi;
        const bool wrap = cf.needsWrap(t, twoH);
        const T rhoiInv = 1.0 / rhoi;
        const T mprhoi = prhoi;
        T mx = 0, my = 0, mz = 0, en = 0, avE = 0;
        long long maxvBits = 0;
        for (unsigned k = 0; k < nc; ++k) {
            uint32_t j = lv.at(ii, k);
            T rx, ry, rz;
            cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
            T r2 = dist2(rx, ry, rz);
            T rinv = invDist(r2);
            T dist = r2 * rinv;
            T vxij = vxi - ld<T>(a.vx, j), vyij = vyi - ld<T>(a.vy, j), vzij = vzi - ld<T>(a.vz, j);
            T Wi = hiInv3 * lookupX(tabX, dist * hiInvDx);
            T Wj = __ldg(hInv3 + j) * lookupX(tabX, dist * __ldg(hInvDx + j));
            // G = c r at both ends; the reference's a_i = -G_i W_i, a_j = -G_j W_j
            T gix = c11i * rx + c12i * ry + c13i * rz;
            T giy = c12i * rx + c22i * ry + c23i * rz;
            T giz = c13i * rx + c23i * ry + c33i * rz;
            T c11j = ld<T>(a.c11, j), c12j = ld<T>(a.c12, j), c13j = ld<T>(a.c13, j);
            T c22j = ld<T>(a.c22, j), c23j = ld<T>(a.c23, j), c33j = ld<T>(a.c33, j);
            T gjx = c11j * rx + c12j * ry + c13j * rz;
            T gjy = c12j * rx + c22j * ry + c23j * rz;
            T gjz = c13j * rx + c23j * ry + c33j * rz;
            T mj = ld<T>(a.m, j), cj = ld<T>(a.c, j), xmj = ld<T>(a.xm, j);
            T rhoj = __ldg(auxRho + j);
            T rv = fma(rz, vzij, fma(ry, vyij, rx * vxij));
            if constexpr (AvClean) {
                T gj[6] = {ld<T>(a.dV11, j), ld<T>(a.dV12, j), ld<T>(a.dV13, j),
                           ld<T>(a.dV22, j), ld<T>(a.dV23, j), ld<T>(a.dV33, j)};
                rv += avRv<T>(rx, ry, rz, fmin(dist * hiInv, dist * __ldg(hInv + j)), etaCrit, gi, gj);
            }
            T wij = rv * rinv;
            T visc = artificialViscosity<T>(ai, ld<T>(a.alpha, j), ci, cj, wij);
            maxvBits = maxBitsNonNeg(maxvBits, fma(T(-2), wij, T(0.5) * (ci + cj)));
            // Atwood number |rhoi - rhoj| / (rhoi + rhoj) against Atmin / Atmax, without dividing
            // and with the comparisons on bit patterns (all operands >= 0)
            T dr = fabs(rhoi - rhoj), sr = rhoi + rhoj;
            T am, bm;
            if (lessNonNeg(dr, Atmin * sr)) {
                am = xmi2;
                bm = xmj * xmj;
            } else if (lessNonNeg(Atmax * sr, dr)) {
                am = xmi * xmj;
                bm = am;
            } else {
                // xmi^(2-s) xmj^s = xmi^2 q and xmj^(2-s) xmi^s = xmj^2 / q, q = (xmj/xmi)^s
                T s = ramp * (dr / sr - Atmin);
                T q = exp(s * (__ldg(auxLnXm + j) - lnxmi));
                am = xmi2 * q;
                bm = xmj * xmj / q;
            }
            T av = mj * rhoiInv * visc, bv = __ldg(auxMoR + j) * visc;
            T momi = mj * mprhoi * am, momj = __ldg(auxMprho + j) * bm;
            T si = vxij * gix + vyij * giy + vzij * giz;
            T sj = vxij * gjx + vyij * gjy + vzij * gjz;
            T avWi = av * Wi, bvWj = bv * Wj;
            // momentum: momi a_i + momj a_j + 0.5 (av a_i + bv a_j)
            T ki = momi * Wi + T(0.5) * avWi, kj = momj * Wj + T(0.5) * bvWj;
            mx -= ki * gix + kj * gjx;
            my -= ki * giy + kj * gjy;
            mz -= ki * giz + kj * gjz;
            // energy: mj am (v_ij . a_i) and the viscous work 0.5 (av v_ij.a_i + bv v_ij.a_j)
            en -= mj * am * Wi * si;
            avE -= T(0.5) * (avWi * si + bvWj * sj);
        }
        if (valid) {
            if (a.tapeEn) {
                a.tapeEn[i] = en;
                a.tapeAvE[i] = avE;
            }
            avE = fmax(T(0), avE);
            a.du[i] = a.K * (prhoi * en + T(0.5) * avE);
            st<T>(a.ax, i, -a.K * mx);
            st<T>(a.ay, i, -a.K * my);
            st<T>(a.az, i, -a.K * mz);
            dt = courantDt(__longlong_as_double(maxvBits), hi, ci, a.Kcour);
        }
    } else {
        // neighbour fields from three 32-byte blocks per particle (meVePackKernel), one 256-bit
        // load each; the kernel function's 8 KB of cubic pieces stay in L1 (a smaller polynomial table
        // or the 160 KB linear table measured slower)
        const float4* tabW = static_cast<const float4*>(a.wh);
        auto t = cm.target(i);
        T hiInv = t.hInv, hiInv3 = hiInv * hiInv * hiInv;
        T rhoiInv = __frcp_rn(rhoi);
        KSum mx, my, mz, en, avE;
        // the list entry two pairs ahead and the next neighbour's blocks are loaded while the
        // current pair is evaluated
        uint32_t jn = nc > 0 ? lv.at(ii, 0) : uint32_t(i);
        uint32_t jnn = nc > 1 ? lv.at(ii, 1) : uint32_t(i);
        Rec8 n0 = ldRec8(a.pack + 3 * int64_t(jn)), n1 = ldRec8(a.pack + 3 * int64_t(jn) + 1),
             n2 = ldRec8(a.pack + 3 * int64_t(jn) + 2);
        for (unsigned k = 0; k < nc; ++k) {
            const uint32_t j = jn;
            const Rec8 b0 = n0;  // cell xl yl zl 1/h vx vy
            const Rec8 b1 = n1;  // vz c c11 c12 c13 c22 c23 c33
            const Rec8 b2 = n2;  // m xm alpha rho m/rho m*prho
            if (k + 1 < nc) {
                jn = jnn;
                if (k + 2 < nc) jnn = lv.at(ii, k + 2);
                n0 = ldRec8(a.pack + 3 * int64_t(jn));
                n1 = ldRec8(a.pack + 3 * int64_t(jn) + 1);
                n2 = ldRec8(a.pack + 3 * int64_t(jn) + 2);
            }
            const u64 cj = u64(__float_as_uint(b0.v[0])) | (u64(__float_as_uint(b0.v[1])) << 32);
            const int ddx = CoordMixed::wrap(t.ix - int(cj & kGridMask), cm.pbc[0]);
            const int ddy = CoordMixed::wrap(t.iy - int((cj >> kGridBits) & kGridMask), cm.pbc[1]);
            const int ddz = CoordMixed::wrap(t.iz - int(cj >> (2 * kGridBits)), cm.pbc[2]);
            const T rx = fmaf(float(ddx), cm.u[0], t.xl - b0.v[2]);
            const T ry = fmaf(float(ddy), cm.u[1], t.yl - b0.v[3]);
            const T rz = fmaf(float(ddz), cm.u[2], t.zl - b0.v[4]);
            const T hjInv = b0.v[5];
            T r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
            T rinv = rsqrtf(r2);
            T dist = r2 * rinv;
            T vxij = vxi - b0.v[6], vyij = vyi - b0.v[7], vzij = vzi - b1.v[0];
            T v1 = dist * hiInv, v2 = dist * hjInv;
            T Wi = hiInv3 * lookupH32(tabW, v1);
            T Wj = (hjInv * hjInv * hjInv) * lookupH32(tabW, v2);
            T gix = c11i * rx + c12i * ry + c13i * rz;
            T giy = c12i * rx + c22i * ry + c23i * rz;
            T giz = c13i * rx + c23i * ry + c33i * rz;
            T gjx = b1.v[2] * rx + b1.v[3] * ry + b1.v[4] * rz;
            T gjy = b1.v[3] * rx + b1.v[5] * ry + b1.v[6] * rz;
            T gjz = b1.v[4] * rx + b1.v[6] * ry + b1.v[7] * rz;
            T mj = b2.v[0], csj = b1.v[1], xmj = b2.v[1];
            T rhoj = b2.v[3];
            T rv = rx * vxij + ry * vyij + rz * vzij;
            if constexpr (AvClean) {
                T gj[6] = {ld<T>(a.dV11, j), ld<T>(a.dV12, j), ld<T>(a.dV13, j),
                           ld<T>(a.dV22, j), ld<T>(a.dV23, j), ld<T>(a.dV33, j)};
                rv += avRv<T>(rx, ry, rz, fminf(v1, v2), etaCrit, gi, gj);
            }
            T wij = rv * rinv;
            T visc = artificialViscosity<T>(ai, b2.v[2], ci, csj, wij);
            T vsig = T(0.5) * (ci + csj) - T(2) * wij;
            maxv = (vsig > maxv) ? vsig : maxv;
            T dr = fabsf(rhoi - rhoj), sr = rhoi + rhoj;
            T am, bm;
            if (dr < Atmin * sr) {
                am = xmi2;
                bm = xmj * xmj;
            } else if (dr > Atmax * sr) {
                am = xmi * xmj;
                bm = am;
            } else {
                T s = ramp * (__fdividef(dr, sr) - Atmin);
                T q = exp2f(s * (log2f(xmj) - lnxmi));
                am = xmi2 * q;
                bm = xmj * xmj * __frcp_rn(q);
            }
            T av = mj * rhoiInv * visc, bv = b2.v[4] * visc;
            T momi = mj * prhoi * am, momj = b2.v[5] * bm;
            T si = vxij * gix + vyij * giy + vzij * giz;
            T sj = vxij * gjx + vyij * gjy + vzij * gjz;
            T avWi = av * Wi, bvWj = bv * Wj;
            // a_i = -G_i W_i, a_j = -G_j W_j: momentum momi a_i + momj a_j + 0.5 (av a_i + bv a_j),
            // energy mj am (v_ij . a_i), viscous work 0.5 (av v_ij . a_i + bv v_ij . a_j)
            T ki = momi * Wi + T(0.5) * avWi, kj = momj * Wj + T(0.5) * bvWj;
            mx.add(-(ki * gix + kj * gjx));
            my.add(-(ki * giy + kj * gjy));
            mz.add(-(ki * giz + kj * gjz));
            en.add(-(mj * am * Wi * si));
            avE.add(T(-0.5) * (avWi * si + bvWj * sj));
        }
        if (valid) {
            double ave = fmax(0.0, avE.value64());
            a.du[i] = a.K * (double(prhoi) * en.value64() + 0.5 * ave);
            st<T>(a.ax, i, T(-a.K * mx.value64()));
            st<T>(a.ay, i, T(-a.K * my.value64()));
            st<T>(a.az, i, T(-a.K * mz.value64()));
            dt = courantDt(double(maxv), double(hi), double(ci), a.Kcour);
        }
    }
    if (a.groupDt) {
        double g = dt;
        for (int o = 16; o > 0; o >>= 1) g = fmin(g, __shfl_xor_sync(0xffffffffu, g, o));
        if ((threadIdx.x & 31) == 0 && i0 < lv.last) a.groupDt[(i0 - lv.first) / 32] = float(g);
    }
    if (a.minDt) blockMinDt(dt, a.minDt);
}

// FP64 gradh with one evaluation per mutual pair over the owned lists.  i adds w_i xm_j,
// dterh_i xm_j and dterh_i m_j (veDefGradhJLoop, ve_def_gradh_kern.hpp:64-78); a mutual pair also
// gives j its terms at v_j = d / h_j with xm_i and m_i, by FP64 atomics.  The self terms and the
// epilogue (ve_def_gradh_kern.hpp:60-62, 80-88) run in gradhOnceFinish.
template<bool Smooth>
__global__ void __launch_bounds__(kPairBlock) gradhOnceKernel(ListView lv, OwnedView ov, CoordFp64 cf,
                                                               const double* h, const double* m, const double* xm,
                                                               KTab<Smooth> tw, KTab<Smooth> tdw,
                                                               const double* hInv64, int64_t n, double* acc,
                                                               PairGeo geo)
{
    const int64_t i = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last) return;
    const int64_t ii = i - lv.first;
    const unsigned no = ov.size(ii);
    const double* hInv = hInv64;
    const double* hInvDx = hInv64 + 2 * n;
    auto t = cf.target(i);
    const double hi = h[i], mi = m[i], xmi = xm[i], twoH = 2.0 * hi, hiInv = hInv[i], hiInvDx = hInvDx[i];
    const bool wrap = cf.needsWrap(t, twoH);
    const int64_t gb = geo.base(ii);
    double kx = 0.0, whom = 0.0, wr0 = 0.0;
    for (unsigned k = 0; k < no; ++k) {
        bool mutual;
        const uint32_t j = ov.at(ii, k, mutual);
        double dist;
        double2 wv = make_double2(0.0, 0.0);
        if (geo.g) {
            const int64_t e = gb + 32 * int64_t(k);
            dist = __ldg(geo.g + e).x;
            wv = __ldg(geo.w + e);
        } else {
            double rx, ry, rz;
            cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
            const double r2 = dist2(rx, ry, rz);
            dist = r2 * invDist(r2);
        }
        {
            const double v = dist * hiInv;
            const TabSlot sl = tabSlot(dist * hiInvDx);
            const double w = geo.g ? wv.x : lookupX(tw, sl), dw = lookupX(tdw, sl);
            const double dterh = -(3.0 * w + v * dw);
            const double xmj = __ldg(xm + j);
            kx += w * xmj;
            whom += dterh * xmj;
            wr0 += dterh * __ldg(m + j);
        }
        if (mutual) {
            const double v = dist * __ldg(hInv + j);
            const TabSlot sl = tabSlot(dist * __ldg(hInvDx + j));
            const double w = geo.g ? wv.y : lookupX(tw, sl), dw = lookupX(tdw, sl);
            const double dterh = -(3.0 * w + v * dw);
            atomicAdd(acc + j, w * xmi);
            atomicAdd(acc + n + j, dterh * xmi);
            atomicAdd(acc + 2 * n + j, dterh * mi);
        }
    }
    atomicAdd(acc + i, kx);
    atomicAdd(acc + n + i, whom);
    atomicAdd(acc + 2 * n + i, wr0);
}

__global__ void gradhOnceFinish(int64_t first, int64_t last, int64_t n, const double* h, const double* m,
                                const double* xm, double K, const double* acc, double* kxOut, double* gradhOut,
                                double* tapeWom, double* tapeWr0)
{
    const int64_t i = first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= last) return;
    const double hi = h[i], mi = m[i], xmi = xm[i];
    const double hInv = 1.0 / hi, h3Inv = hInv * hInv * hInv;
    double kxi = xmi + acc[i], whomega = -3.0 * xmi + acc[n + i], wrho0 = -3.0 * mi + acc[2 * n + i];
    kxi *= K * h3Inv;
    whomega *= K * h3Inv * hInv;
    wrho0 *= K * h3Inv * hInv;
    if (tapeWom) {
        tapeWom[i] = whomega;
        tapeWr0[i] = wrho0;
    }
    whomega = whomega * mi / xmi + (kxi - K * xmi * h3Inv) * wrho0;
    const double rhoi = kxi * mi / xmi;
    const double dhdrho = -hi / (rhoi * 3.0);
    kxOut[i] = kxi;
    gradhOut[i] = 1.0 - dhdrho * whomega;
}

// the same epilogue fused with the EOS and the quotients of the later passes (inside a sweep)
__global__ void gradhEosFinish(int64_t n, const double* h, const double* m, const double* xm, double K,
                               const double* acc, double* kxOut, double* gradhOut, const double* u, double gamma,
                               void* prho, void* c, void* rho, void* p, double* aux, double* tapeWom,
                               double* tapeWr0)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const double hi = h[i], mi = m[i], xmi = xm[i];
    const double hInv = 1.0 / hi, h3Inv = hInv * hInv * hInv;
    double kxi = xmi + acc[i], whomega = -3.0 * xmi + acc[n + i], wrho0 = -3.0 * mi + acc[2 * n + i];
    kxi *= K * h3Inv;
    whomega *= K * h3Inv * hInv;
    wrho0 *= K * h3Inv * hInv;
    if (tapeWom) {
        tapeWom[i] = whomega;
        tapeWr0[i] = wrho0;
    }
    whomega = whomega * mi / xmi + (kxi - K * xmi * h3Inv) * wrho0;
    const double rhoi = kxi * mi / xmi;
    const double dhdrho = -hi / (rhoi * 3.0);
    const double gradhi = 1.0 - dhdrho * whomega;
    kxOut[i] = kxi;
    gradhOut[i] = gradhi;
    const double prhoi = eosVe<double>(i, u[i], mi, kxi, xmi, gradhi, gamma, prho, c, rho, p);
    veAuxAll<double>(n, i, mi, kxi, xmi, prhoi, aux);
}

// FP64 IAD + divv/curlv with one evaluation per mutual pair over the owned lists.  i adds
// vol_j W_i r r^T and xm_j W_i (v_j - v_i) r^T (r = x_i - x_j); a mutual pair also gives j
// vol_i W_j r r^T and xm_i W_j (v_j - v_i) r^T (r and the velocity difference both change sign) by
// FP64 atomics.  The inversion and divv/curlv follow per particle in iadOnceFinish.
template<bool Smooth>
__global__ void __launch_bounds__(kPairBlock) iadOnceKernel(ListView lv, OwnedView ov, CoordFp64 cf, IadDivvArgs a,
                                                             const double* hInv64, int64_t n, double* acc, PairGeo geo)
{
    const int64_t i = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last) return;
    const int64_t ii = i - lv.first;
    const unsigned no = ov.size(ii);
    const KTab<Smooth> tab{a.w64};
    const double* hInvDx = hInv64 + 2 * n;
    const double *vx = static_cast<const double*>(a.vx), *vy = static_cast<const double*>(a.vy),
                 *vz = static_cast<const double*>(a.vz), *xm = static_cast<const double*>(a.xm),
                 *vol = static_cast<const double*>(a.vol);
    auto t = cf.target(i);
    const double hi = ld<double>(a.h, i), twoH = 2.0 * hi, hiInvDx = hInvDx[i];
    const bool wrap = cf.needsWrap(t, twoH);
    const double vxi = vx[i], vyi = vy[i], vzi = vz[i], voli = vol[i], xmi = xm[i];
    const int64_t gb = geo.base(ii);
    double tau[6] = {0, 0, 0, 0, 0, 0}, M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (unsigned k = 0; k < no; ++k) {
        bool mutual;
        const uint32_t j = ov.at(ii, k, mutual);
        double rx, ry, rz, dvx, dvy, dvz, dist;
        double2 wv = make_double2(0.0, 0.0);
        if (geo.x) {
            const int64_t e = gb + 32 * int64_t(k);
            const double2 a0 = __ldg(geo.x + e), a1 = __ldg(geo.x + geo.plane + e),
                          a2 = __ldg(geo.x + 2 * geo.plane + e);
            rx = a0.x, ry = a0.y, rz = a1.x, dvx = a1.y, dvy = a2.x, dvz = a2.y;
            dist = __ldg(geo.g + e).x;
            wv = __ldg(geo.w + e);
        } else {
            cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
            if (geo.g) {
                const int64_t e = gb + 32 * int64_t(k);
                dist = __ldg(geo.g + e).x;
                wv = __ldg(geo.w + e);
            } else {
                const double r2 = dist2(rx, ry, rz);
                dist = r2 * invDist(r2);
            }
            dvx = vx[j] - vxi, dvy = vy[j] - vyi, dvz = vz[j] - vzi;
        }
        {
            const double w = geo.g ? wv.x : lookupX(tab, dist * hiInvDx);
            const double vw = vol[j] * w, xw = xm[j] * w;
            const double rxv = rx * vw, ryv = ry * vw, rzv = rz * vw;
            tau[0] += rx * rxv;
            tau[1] += ry * rxv;
            tau[2] += rz * rxv;
            tau[3] += ry * ryv;
            tau[4] += rz * ryv;
            tau[5] += rz * rzv;
            const double sx = dvx * xw, sy = dvy * xw, sz = dvz * xw;
            M[0] += sx * rx;
            M[1] += sx * ry;
            M[2] += sx * rz;
            M[3] += sy * rx;
            M[4] += sy * ry;
            M[5] += sy * rz;
            M[6] += sz * rx;
            M[7] += sz * ry;
            M[8] += sz * rz;
        }
        if (mutual) {
            const double w = geo.g ? wv.y : lookupX(tab, dist * __ldg(hInvDx + j));
            const double vw = voli * w, xw = xmi * w;
            const double rxv = rx * vw, ryv = ry * vw, rzv = rz * vw;
            atomicAdd(acc + j, rx * rxv);
            atomicAdd(acc + n + j, ry * rxv);
            atomicAdd(acc + 2 * n + j, rz * rxv);
            atomicAdd(acc + 3 * n + j, ry * ryv);
            atomicAdd(acc + 4 * n + j, rz * ryv);
            atomicAdd(acc + 5 * n + j, rz * rzv);
            const double sx = dvx * xw, sy = dvy * xw, sz = dvz * xw;
            atomicAdd(acc + 6 * n + j, sx * rx);
            atomicAdd(acc + 7 * n + j, sx * ry);
            atomicAdd(acc + 8 * n + j, sx * rz);
            atomicAdd(acc + 9 * n + j, sy * rx);
            atomicAdd(acc + 10 * n + j, sy * ry);
            atomicAdd(acc + 11 * n + j, sy * rz);
            atomicAdd(acc + 12 * n + j, sz * rx);
            atomicAdd(acc + 13 * n + j, sz * ry);
            atomicAdd(acc + 14 * n + j, sz * rz);
        }
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) atomicAdd(acc + q * n + i, tau[q]);
#pragma unroll
    for (int q = 0; q < 9; ++q) atomicAdd(acc + (6 + q) * n + i, M[q]);
}

__global__ void iadOnceFinish(int64_t first, int64_t last, int64_t n, IadDivvArgs a, const double* acc)
{
    const int64_t i = first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= last) return;
    double tau[6], M[9];
#pragma unroll
    for (int q = 0; q < 6; ++q) tau[q] = acc[q * n + i];
#pragma unroll
    for (int q = 0; q < 9; ++q) M[q] = acc[(6 + q) * n + i];
    iadEpilogue64(a, i, ld<double>(a.h, i), tau, M);
}

// FP64 AV switches with one evaluation per mutual pair over the owned lists.  i's sum is
// S_i = sum vol_j (divv_i - divv_j) W_i r (r = x_i - x_j; c_i is applied after the walk), j's term of
// the same pair is vol_i (divv_i - divv_j) W_j r (r and the divv difference both change sign);
// the signal-velocity candidate c_i + c_j - 3 (r.v) / |r| of approaching pairs is symmetric.
template<bool Smooth>
__global__ void __launch_bounds__(kPairBlock) avOnceKernel(ListView lv, OwnedView ov, CoordFp64 cf, AvArgs a,
                                                            const double* hInv64, int64_t n, double* acc, PairGeo geo)
{
    const int64_t i = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last) return;
    const int64_t ii = i - lv.first;
    const unsigned no = ov.size(ii);
    const KTab<Smooth> tabX{a.w64};
    const double* hInvDx = hInv64 + 2 * n;
    const double *vx = static_cast<const double*>(a.vx), *vy = static_cast<const double*>(a.vy),
                 *vz = static_cast<const double*>(a.vz), *c = static_cast<const double*>(a.c),
                 *divv = static_cast<const double*>(a.divv), *vol = static_cast<const double*>(a.vol);
    auto t = cf.target(i);
    const double hi = ld<double>(a.h, i), ci = c[i], divvi = divv[i], voli = vol[i];
    const double vxi = vx[i], vyi = vy[i], vzi = vz[i], twoH = 2.0 * hi, hiInvDx = hInvDx[i];
    const bool wrap = cf.needsWrap(t, twoH);
    const int64_t gb = geo.base(ii);
    double Sx = 0, Sy = 0, Sz = 0;
    long long vsigBits = 0;
    long long* accV = reinterpret_cast<long long*>(acc + 3 * n);
    for (unsigned k = 0; k < no; ++k) {
        bool mutual;
        const uint32_t j = ov.at(ii, k, mutual);
        double rx, ry, rz, rinv, dist, rv;
        double2 wv = make_double2(0.0, 0.0);
        if (geo.g) {
            const int64_t e = gb + 32 * int64_t(k);
            const double2 gd = __ldg(geo.g + e);
            dist = gd.x;
            rinv = gd.y;
            wv = __ldg(geo.w + e);
            if (geo.x) {  // v_i - v_j = -dv exactly
                const double2 a0 = __ldg(geo.x + e), a1 = __ldg(geo.x + geo.plane + e),
                              a2 = __ldg(geo.x + 2 * geo.plane + e);
                rx = a0.x, ry = a0.y, rz = a1.x;
                rv = fma(rz, -a2.y, fma(ry, -a2.x, rx * -a1.y));
            } else {
                cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
                rv = fma(rz, vzi - vz[j], fma(ry, vyi - vy[j], rx * (vxi - vx[j])));
            }
        } else {
            cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
            const double r2 = dist2(rx, ry, rz);
            rinv = invDist(r2);
            dist = r2 * rinv;
            rv = fma(rz, vzi - vz[j], fma(ry, vyi - vy[j], rx * (vxi - vx[j])));
        }
        const bool approaching = negative(rv);
        double vs = 0.0;
        if (approaching) {
            vs = fma(-3.0 * rv, rinv, ci + c[j]);
            vsigBits = maxBitsNonNeg(vsigBits, vs);
        }
        const double dd = divvi - divv[j];
        const double fw = vol[j] * dd * (geo.g ? wv.x : lookupX(tabX, dist * hiInvDx));
        Sx += fw * rx;
        Sy += fw * ry;
        Sz += fw * rz;
        if (mutual) {
            const double fwj = voli * dd * (geo.g ? wv.y : lookupX(tabX, dist * __ldg(hInvDx + j)));
            atomicAdd(acc + j, fwj * rx);
            atomicAdd(acc + n + j, fwj * ry);
            atomicAdd(acc + 2 * n + j, fwj * rz);
            if (approaching) atomicMax(accV + j, __double_as_longlong(vs));
        }
    }
    atomicAdd(acc + i, Sx);
    atomicAdd(acc + n + i, Sy);
    atomicAdd(acc + 2 * n + i, Sz);
    atomicMax(accV + i, vsigBits);
}

__global__ void avOnceFinish(int64_t first, int64_t last, int64_t n, AvArgs a, const double* acc)
{
    const int64_t i = first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= last) return;
    const double hi = ld<double>(a.h, i), ci = ld<double>(a.c, i), divvi = ld<double>(a.divv, i);
    const double hiInv = 1.0 / hi, kh3 = a.K * hiInv * hiInv * hiInv;
    const double c11 = ld<double>(a.c11, i), c12 = ld<double>(a.c12, i), c13 = ld<double>(a.c13, i);
    const double c22 = ld<double>(a.c22, i), c23 = ld<double>(a.c23, i), c33 = ld<double>(a.c33, i);
    const double Sx = acc[i], Sy = acc[n + i], Sz = acc[2 * n + i];
    const double gx = -kh3 * (c11 * Sx + c12 * Sy + c13 * Sz);
    const double gy = -kh3 * (c12 * Sx + c22 * Sy + c23 * Sz);
    const double gz = -kh3 * (c13 * Sx + c23 * Sy + c33 * Sz);
    if (a.tapeG) {
        a.tapeG[i] = gx;
        a.tapeG[a.tapeN + i] = gy;
        a.tapeG[2 * a.tapeN + i] = gz;
    }
    // vsig_i starts at 1e-40 c_i (av_switches_kern.hpp:66); both candidates are >= 0
    const long long vb = max(__double_as_longlong(1.e-40 * ci), reinterpret_cast<const long long*>(acc + 3 * n)[i]);
    st<double>(a.alpha, i,
               avAlpha<double>(a, ld<double>(a.alpha, i), hi, ci, divvi, __longlong_as_double(vb), gx, gy, gz));
}

// FP64 VE momentum-energy with one evaluation per mutual pair, for lists that cover every particle.
// i walks its owned list: every pair of its list that j does not list back, and half of the
// mutual pairs (the other half is in the owned lists of the other ends).  The two ends' terms follow from one
// another (momentum_energy_kern.hpp:125-210): r and v_ij change sign, so G = c r changes sign at
// both ends and v_ij . G does not; W_i and W_j, the Atwood weights (a_mom, b_mom), m_j and m_i, and
// 1/rho_i and 1/rho_j trade places; the viscosity and the signal velocity are symmetric.  i's terms
// stay in registers; j's go to its accumulators with FP64 atomics (the signal-velocity maximum as an
// integer maximum of non-negative bit patterns).
template<bool Smooth>
__global__ void __launch_bounds__(kPairBlock) meVeOnceKernel(ListView lv, CoordFp64 cf, MeVeArgs a, PairGeo geo)
{
    using T = double;
    const int64_t i = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last) return;
    const int64_t ii = i - lv.first;
    const unsigned nOwned = __ldg(a.ownedCount + ii);
    const KTab<Smooth> tabX{a.w64};
    const T* aux = static_cast<const T*>(a.aux);
    const T *auxRho = aux, *auxLnXm = aux + 4 * a.n, *auxRhoInv = aux + 5 * a.n;
    const double* hInv3 = a.hInv64 + a.n;
    const double* hInvDx = a.hInv64 + 2 * a.n;
    const T *vxA = static_cast<const T*>(a.vx), *vyA = static_cast<const T*>(a.vy),
            *vzA = static_cast<const T*>(a.vz), *prhoA = static_cast<const T*>(a.prho);
    constexpr T Atmin = 0.1, Atmax = 0.2, ramp = 1.0 / (Atmax - Atmin);

    const T hi = ld<T>(a.h, i), mi = ld<T>(a.m, i), ci = ld<T>(a.c, i), ai = ld<T>(a.alpha, i);
    const T xmi = ld<T>(a.xm, i), prhoi = prhoA[i];
    const T rhoi = auxRho[i], lnxmi = auxLnXm[i], rhoiInv = auxRhoInv[i];
    const T vxi = vxA[i], vyi = vyA[i], vzi = vzA[i];
    const T c11i = ld<T>(a.c11, i), c12i = ld<T>(a.c12, i), c13i = ld<T>(a.c13, i);
    const T c22i = ld<T>(a.c22, i), c23i = ld<T>(a.c23, i), c33i = ld<T>(a.c33, i);
    const T xmi2 = xmi * xmi;
    auto t = cf.target(i);
    const T hiInv3 = hInv3[i], hiInvDx = hInvDx[i], twoH = 2.0 * hi;
    const bool wrap = cf.needsWrap(t, twoH);
    const int64_t gb = geo.base(ii);
    T mx = 0, my = 0, mz = 0, en = 0, avE = 0;
    long long maxvBits = 0;
    double *accX = a.acc, *accY = a.acc + a.n, *accZ = a.acc + 2 * a.n, *accE = a.acc + 3 * a.n,
           *accV = a.acc + 4 * a.n;
    long long* accS = reinterpret_cast<long long*>(a.acc + 5 * a.n);
    for (unsigned k = 0; k < nOwned; ++k) {
        const uint32_t e = __ldg(a.owned + listSlot(ii, k, lv.stride));
        const uint32_t j = e & 0x7fffffffu;
        const bool mutual = (e >> 31) != 0;
        T rx, ry, rz, rinv, Wi, Wj, vxij, vyij, vzij;
        if (geo.g) {
            const int64_t e = gb + 32 * int64_t(k);
            const double2 gd = __ldg(geo.g + e), wv = __ldg(geo.w + e);
            rinv = gd.y;
            Wi = hiInv3 * wv.x;
            Wj = __ldg(hInv3 + j) * wv.y;
            if (geo.x) {  // v_ij = v_i - v_j = -dv exactly
                const double2 a0 = __ldg(geo.x + e), a1 = __ldg(geo.x + geo.plane + e),
                              a2 = __ldg(geo.x + 2 * geo.plane + e);
                rx = a0.x, ry = a0.y, rz = a1.x;
                vxij = -a1.y, vyij = -a2.x, vzij = -a2.y;
            } else {
                cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
                vxij = vxi - vxA[j], vyij = vyi - vyA[j], vzij = vzi - vzA[j];
            }
        } else {
            cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
            const T r2 = dist2(rx, ry, rz);
            rinv = invDist(r2);
            const T dist = r2 * rinv;
            Wi = hiInv3 * lookupX(tabX, dist * hiInvDx);
            Wj = __ldg(hInv3 + j) * lookupX(tabX, dist * __ldg(hInvDx + j));
            vxij = vxi - vxA[j], vyij = vyi - vyA[j], vzij = vzi - vzA[j];
        }
        T gix = c11i * rx + c12i * ry + c13i * rz;
        T giy = c12i * rx + c22i * ry + c23i * rz;
        T giz = c13i * rx + c23i * ry + c33i * rz;
        T c11j = ld<T>(a.c11, j), c12j = ld<T>(a.c12, j), c13j = ld<T>(a.c13, j);
        T c22j = ld<T>(a.c22, j), c23j = ld<T>(a.c23, j), c33j = ld<T>(a.c33, j);
        T gjx = c11j * rx + c12j * ry + c13j * rz;
        T gjy = c12j * rx + c22j * ry + c23j * rz;
        T gjz = c13j * rx + c23j * ry + c33j * rz;
        T mj = ld<T>(a.m, j), cj = ld<T>(a.c, j), xmj = ld<T>(a.xm, j);
        T rhoj = __ldg(auxRho + j);
        T rv = fma(rz, vzij, fma(ry, vyij, rx * vxij));
        T wij = rv * rinv;
        T visc = artificialViscosity<T>(ai, ld<T>(a.alpha, j), ci, cj, wij);
        const T vsig = fma(T(-2), wij, T(0.5) * (ci + cj));
        maxvBits = maxBitsNonNeg(maxvBits, vsig);
        T dr = fabs(rhoi - rhoj), sr = rhoi + rhoj;
        T am, bm;
        if (lessNonNeg(dr, Atmin * sr)) {
            am = xmi2;
            bm = xmj * xmj;
        } else if (lessNonNeg(Atmax * sr, dr)) {
            am = xmi * xmj;
            bm = am;
        } else {
            T s = ramp * (dr / sr - Atmin);
            T q = exp(s * (__ldg(auxLnXm + j) - lnxmi));
            am = xmi2 * q;
            bm = xmj * xmj / q;
        }
        T si = vxij * gix + vyij * giy + vzij * giz;
        T sj = vxij * gjx + vyij * gjy + vzij * gjz;
        // the reference's terms, factored: with hv = visc / 2, t_i = hv / rho_i and t_j = hv / rho_j,
        // P_i = W_i (prho_i am + t_i) and P_j = W_j (prho_j bm + t_j), i's momentum term momi a_i +
        // momj a_j + (av a_i + bv a_j) / 2 is m_j V with V = P_i G_i + P_j G_j and its viscous work
        // m_j Q with Q = t_i W_i s_i + t_j W_j s_j; j's terms of the same pair are m_i V and m_i Q
        // (i and j trade places, G and v_ij change sign); the energy terms m_j am W_i s_i and
        // m_i bm W_j s_j stay apart
        const T hv = T(0.5) * visc;
        const T wsi = Wi * si, wsj = Wj * sj;
        const T ti = rhoiInv * hv, tj = __ldg(auxRhoInv + j) * hv;
        const T Pi = Wi * fma(prhoi, am, ti), Pj = Wj * fma(prhoA[j], bm, tj);
        const T Vx = fma(Pi, gix, Pj * gjx), Vy = fma(Pi, giy, Pj * gjy), Vz = fma(Pi, giz, Pj * gjz);
        const T Q = fma(ti, wsi, tj * wsj);
        mx = fma(-mj, Vx, mx);
        my = fma(-mj, Vy, my);
        mz = fma(-mj, Vz, mz);
        en = fma(-(mj * am), wsi, en);
        avE = fma(-mj, Q, avE);
        if (mutual) {
            atomicAdd(accX + j, mi * Vx);
            atomicAdd(accY + j, mi * Vy);
            atomicAdd(accZ + j, mi * Vz);
            atomicAdd(accE + j, -(mi * bm) * wsj);
            atomicAdd(accV + j, -mi * Q);
            atomicMax(accS + j, __double_as_longlong(vsig));
        }
    }
    atomicAdd(accX + i, mx);
    atomicAdd(accY + i, my);
    atomicAdd(accZ + i, mz);
    atomicAdd(accE + i, en);
    atomicAdd(accV + i, avE);
    atomicMax(accS + i, maxvBits);
}

__global__ void __launch_bounds__(kPairBlock) meVeOnceFinish(ListView lv, MeVeArgs a)
{
    const int64_t i0 = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const bool valid = i0 < lv.last;
    double dt = INFINITY;
    if (valid) {
        const int64_t i = i0;
        const double prhoi = ld<double>(a.prho, i);
        if (a.tapeEn) {
            a.tapeEn[i] = a.acc[3 * a.n + i];
            a.tapeAvE[i] = a.acc[4 * a.n + i];
        }
        const double avE = fmax(0.0, a.acc[4 * a.n + i]);
        a.du[i] = a.K * (prhoi * a.acc[3 * a.n + i] + 0.5 * avE);
        st<double>(a.ax, i, -a.K * a.acc[i]);
        st<double>(a.ay, i, -a.K * a.acc[a.n + i]);
        st<double>(a.az, i, -a.K * a.acc[2 * a.n + i]);
        const long long mb = reinterpret_cast<const long long*>(a.acc + 5 * a.n)[i];
        dt = courantDt(__longlong_as_double(mb), ld<double>(a.h, i), ld<double>(a.c, i), a.Kcour);
    }
    if (a.groupDt) {
        double g = dt;
        for (int o = 16; o > 0; o >>= 1) g = fmin(g, __shfl_xor_sync(0xffffffffu, g, o));
        if ((threadIdx.x & 31) == 0 && i0 < lv.last) a.groupDt[(i0 - lv.first) / 32] = float(g);
    }
    if (a.minDt) blockMinDt(dt, a.minDt);
}

}  // namespace

int passGradh(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    if (!p->h || !p->m || !p->xm || !p->kx || !p->gradh) return SPHGB_ERR_ARG;
    SPHGB_TRY(checkPass(c, p, first, last));
    ListView lv = listView(c);
    lv.first = first;
    lv.last = last;
    unsigned blocks = gridFor(last - first, kPairBlock);
    double* tape;
    SPHGB_TRY(tapeFor(c, p, first, last, kTapeGradh, &tape));
    double* tWom = tape ? tape + int64_t(kTapeWom) * p->n : nullptr;
    double* tWr0 = tape ? tape + int64_t(kTapeWr0) * p->n : nullptr;
    if (pairOnce(c, p, first, last)) {
        const int64_t n = p->n;
        SPHGB_TRY(c->pairAcc.ensure(sizeof(double) * 3 * size_t(n)));
        SPHGB_CUDA(cudaMemsetAsync(c->pairAcc.p, 0, sizeof(double) * 3 * size_t(n), c->stream));
        SPHGB_TRY(withKernelForm(c, [&](auto smooth) {
            constexpr bool S = decltype(smooth)::value;
            gradhOnceKernel<S><<<blocks, kPairBlock, 0, c->stream>>>(
                lv, ownedView(c), coordFp64(c, p), static_cast<const double*>(p->h), static_cast<const double*>(p->m),
                static_cast<const double*>(p->xm), KTab<S>{tabW64(c)}, KTab<S>{tabDW64(c)}, c->hInv64.as<double>(),
                n, c->pairAcc.as<double>(), pairGeoRead(c));
            return launched(c, "gradhOnceKernel");
        }));
        if (c->inSweep && p->u && p->prho && p->c) {  // EOS and quotients fused into the epilogue
            SPHGB_TRY(c->aux.ensure(sizeof(double) * 6 * n));
            gradhEosFinish<<<gridFor(n, 256), 256, 0, c->stream>>>(
                n, static_cast<const double*>(p->h), static_cast<const double*>(p->m), static_cast<const double*>(p->xm),
                c->K, c->pairAcc.as<double>(), static_cast<double*>(p->kx), static_cast<double*>(p->gradh), p->u,
                c->prm.gamma, p->prho, p->c, p->rho, p->p, c->aux.as<double>(), tWom, tWr0);
            c->eosFused = c->auxReady = true;
            return launched(c, "gradhEosFinish");
        }
        gradhOnceFinish<<<gridFor(last - first, 256), 256, 0, c->stream>>>(
            first, last, n, static_cast<const double*>(p->h), static_cast<const double*>(p->m),
            static_cast<const double*>(p->xm), c->K, c->pairAcc.as<double>(), static_cast<double*>(p->kx),
            static_cast<double*>(p->gradh), tWom, tWr0);
        return launched(c, "gradhOnceFinish");
    }
    if (p->precision == SPHGB_MIXED) {
        SPHGB_TRY(c->pack.ensure(sizeof(Rec8) * 3 * size_t(p->n)));  // the ME blocks' space, free here
        const Rec8* rec = c->pack.as<Rec8>();
        packGradhKernel<<<gridFor(p->n, 256), 256, 0, c->stream>>>(p->n, p->xm, p->m, c->gridKey.as<u64>(),
                                                                    c->gridLoc.as<float4>(), c->pack.as<float4>());
        SPHGB_TRY(launched(c, "packGradhKernel"));
        gradhKernel<MixedTag><<<blocks, kPairBlock, 0, c->stream>>>(lv, coordFp64(c, p), coordMixed(c), p->h, p->m,
                                                                    p->xm, c->whH32.p, c->whdH32.p, nullptr,
                                                                    nullptr, c->K, p->kx, p->gradh, nullptr, nullptr,
                                                                    rec);
        SPHGB_TRY(launched(c, "gradhKernel"));
        if (first == 0 && last == p->n) return refineMixedGradh(c, p);
        c->stats_refinedGradh = 0;
        return SPHGB_OK;
    }
    return withKernelForm(c, [&](auto smooth) {
        gradhKernel<Fp64Tag, decltype(smooth)::value><<<blocks, kPairBlock, 0, c->stream>>>(
            lv, coordFp64(c, p), coordMixed(c), p->h, p->m, p->xm, c->whx64.p, c->whdx64.p, tabW64(c), tabDW64(c),
            c->K, p->kx, p->gradh, tWom, tWr0);
        return launched(c, "gradhKernel");
    });
}

int passEosVe(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    if (!p->u || !p->m || !p->kx || !p->xm || !p->gradh || !p->prho || !p->c || first < 0 || last > p->n ||
        first >= last)
        return SPHGB_ERR_ARG;
    if (c->inSweep && c->eosFused) return SPHGB_OK;  // done in the gradh epilogue of this sweep
    unsigned blocks = gridFor(last - first, 256);
    if (c->inSweep && first == 0 && last == p->n) {  // EOS and the quotients of the later passes together
        const int64_t n = p->n;
        if (p->precision == SPHGB_MIXED) {
            SPHGB_TRY(c->aux.ensure(sizeof(float) * 6 * n));
            eosAuxVeKernel<MixedTag><<<blocks, 256, 0, c->stream>>>(n, p->u, p->m, p->kx, p->xm, p->gradh, c->prm.gamma,
                                                                   p->prho, p->c, p->rho, p->p, c->aux.as<float>());
        } else {
            SPHGB_TRY(c->aux.ensure(sizeof(double) * 6 * n));
            eosAuxVeKernel<Fp64Tag><<<blocks, 256, 0, c->stream>>>(n, p->u, p->m, p->kx, p->xm, p->gradh, c->prm.gamma,
                                                                  p->prho, p->c, p->rho, p->p, c->aux.as<double>());
        }
        c->auxReady = true;
        return launched(c, "eosAuxVeKernel");
    }
    if (p->precision == SPHGB_MIXED)
        eosVeKernel<MixedTag><<<blocks, 256, 0, c->stream>>>(first, last, p->u, p->m, p->kx, p->xm, p->gradh,
                                                            c->prm.gamma, p->prho, p->c, p->rho, p->p);
    else
        eosVeKernel<Fp64Tag><<<blocks, 256, 0, c->stream>>>(first, last, p->u, p->m, p->kx, p->xm, p->gradh,
                                                           c->prm.gamma, p->prho, p->c, p->rho, p->p);
    return launched(c, "eosVeKernel");
}

int passIadDivvCurlv(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    if (!p->h || !p->vx || !p->vy || !p->vz || !p->xm || !p->kx || !p->c11 || !p->c12 || !p->c13 || !p->c22 ||
        !p->c23 || !p->c33 || !p->divv || !p->m)
        return SPHGB_ERR_ARG;
    const bool gradV = p->dV11 && p->dV12 && p->dV13 && p->dV22 && p->dV23 && p->dV33;
    SPHGB_TRY(checkPass(c, p, first, last));
    const bool mixed = p->precision == SPHGB_MIXED;
    SPHGB_TRY(launchVeAux<kAuxVol>(c, p));
    ListView lv = listView(c);
    lv.first = first;
    lv.last = last;
    const size_t es = mixed ? 4 : 8;
    IadDivvArgs a{};
    a.h = p->h;
    a.vx = p->vx;
    a.vy = p->vy;
    a.vz = p->vz;
    a.xm = p->xm;
    a.kx = p->kx;
    a.vol = c->aux.as<char>() + 2 * es * p->n;
    a.K = c->K;
    a.c11 = p->c11;
    a.c12 = p->c12;
    a.c13 = p->c13;
    a.c22 = p->c22;
    a.c23 = p->c23;
    a.c33 = p->c33;
    a.divv = p->divv;
    a.curlv = p->curlv;
    if (gradV) {
        a.dV11 = p->dV11;
        a.dV12 = p->dV12;
        a.dV13 = p->dV13;
        a.dV22 = p->dV22;
        a.dV23 = p->dV23;
        a.dV33 = p->dV33;
    }
    unsigned blocks = gridFor(last - first, kPairBlock);
    if (mixed) {
        a.wh = c->whH32.p;
        const bool refine = c->refineMixed && first == 0 && last == p->n && c->nbrFirst == 0 && c->nbrLast == p->n;
        if (refine) {
            SPHGB_TRY(c->divvBound.ensure(sizeof(float) * size_t(p->n)));
            a.divvBound = c->divvBound.as<float>();
        }
        SPHGB_TRY(c->pack.ensure(sizeof(Rec8) * 3 * size_t(p->n)));  // the ME blocks' space, free here
        a.rec = c->pack.as<Rec8>();
        a.rec2 = reinterpret_cast<const float2*>(c->pack.as<Rec8>() + p->n);
        packIadKernel<<<gridFor(p->n, 256), 256, 0, c->stream>>>(
            p->n, p->vx, p->vy, p->vz, a.vol, p->xm, c->gridKey.as<u64>(), c->gridLoc.as<float4>(),
            c->pack.as<float4>(), reinterpret_cast<float2*>(c->pack.as<Rec8>() + p->n));
        SPHGB_TRY(launched(c, "packIadKernel"));
        iadDivvKernel<MixedTag><<<blocks, kPairBlock, 0, c->stream>>>(lv, coordFp64(c, p), coordMixed(c), a);
        SPHGB_TRY(launched(c, "iadDivvKernel"));
        return refineMixedDivv(c, p, refine ? a.divvBound : nullptr);
    } else {
        a.wh = c->whx64.p;
        a.w64 = tabW64(c);
        SPHGB_TRY(tapeFor(c, p, first, last, kTapeIad, &a.tapeP));
        if (a.tapeP) a.tapeP += int64_t(kTapeP) * p->n;
        a.tapeN = p->n;
        if (pairOnce(c, p, first, last)) {
            const int64_t n = p->n;
            SPHGB_TRY(c->pairAcc.ensure(sizeof(double) * 15 * size_t(n)));
            SPHGB_CUDA(cudaMemsetAsync(c->pairAcc.p, 0, sizeof(double) * 15 * size_t(n), c->stream));
            SPHGB_TRY(withKernelForm(c, [&](auto smooth) {
                iadOnceKernel<decltype(smooth)::value><<<blocks, kPairBlock, 0, c->stream>>>(
                    lv, ownedView(c), coordFp64(c, p), a, c->hInv64.as<double>(), n, c->pairAcc.as<double>(),
                    pairGeoRead(c));
                return launched(c, "iadOnceKernel");
            }));
            iadOnceFinish<<<gridFor(last - first, 256), 256, 0, c->stream>>>(first, last, n, a, c->pairAcc.as<double>());
            return launched(c, "iadOnceFinish");
        }
        return withKernelForm(c, [&](auto smooth) {
            iadDivvKernel<Fp64Tag, decltype(smooth)::value><<<blocks, kPairBlock, 0, c->stream>>>(
                lv, coordFp64(c, p), coordMixed(c), a);
            return launched(c, "iadDivvKernel");
        });
    }
    return launched(c, "iadDivvKernel");
}

int passAVswitches(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    if (!p->h || !p->vx || !p->c || !p->c11 || !p->kx || !p->xm || !p->divv || !p->alpha || !p->m)
        return SPHGB_ERR_ARG;
    SPHGB_TRY(checkPass(c, p, first, last));
    const bool mixed = p->precision == SPHGB_MIXED;
    SPHGB_TRY(launchVeAux<kAuxVol>(c, p));
    ListView lv = listView(c);
    lv.first = first;
    lv.last = last;
    const size_t es = mixed ? 4 : 8;
    AvArgs a{p->h,   p->vx,  p->vy,  p->vz,   p->c,    p->c11, p->c12,
             p->c13, p->c22, p->c23, p->c33,  p->divv, nullptr, c->aux.as<char>() + 2 * es * p->n,
             c->K,   c->prm.minDt, c->prm.alphamin, c->prm.alphamax, c->prm.decay_constant, p->alpha};
    unsigned blocks = gridFor(last - first, kPairBlock);
    if (!mixed) {
        SPHGB_TRY(tapeFor(c, p, first, last, kTapeAv, &a.tapeG));
        if (a.tapeG) a.tapeG += int64_t(kTapeG) * p->n;
        a.tapeN = p->n;
    }
    if (mixed) {
        a.wh = c->whH32.p;
        SPHGB_TRY(c->pack.ensure(sizeof(Rec8) * 3 * size_t(p->n)));  // the ME blocks' space, free here
        a.rec = c->pack.as<Rec8>();
        a.rec2 = reinterpret_cast<const float4*>(c->pack.as<Rec8>() + p->n);
        packAvKernel<<<gridFor(p->n, 256), 256, 0, c->stream>>>(
            p->n, a, c->gridKey.as<u64>(), c->gridLoc.as<float4>(), c->pack.as<float4>(),
            reinterpret_cast<float4*>(c->pack.as<Rec8>() + p->n));
        SPHGB_TRY(launched(c, "packAvKernel"));
        avKernel<MixedTag><<<blocks, kPairBlock, 0, c->stream>>>(lv, coordFp64(c, p), coordMixed(c), a);
    } else if (pairOnce(c, p, first, last)) {
        const int64_t n = p->n;
        a.wh = c->whx64.p;
        a.w64 = tabW64(c);
        SPHGB_TRY(c->pairAcc.ensure(sizeof(double) * 4 * size_t(n)));
        SPHGB_CUDA(cudaMemsetAsync(c->pairAcc.p, 0, sizeof(double) * 4 * size_t(n), c->stream));
        SPHGB_TRY(withKernelForm(c, [&](auto smooth) {
            avOnceKernel<decltype(smooth)::value><<<blocks, kPairBlock, 0, c->stream>>>(
                lv, ownedView(c), coordFp64(c, p), a, c->hInv64.as<double>(), n, c->pairAcc.as<double>(),
                pairGeoRead(c));
            return launched(c, "avOnceKernel");
        }));
        avOnceFinish<<<gridFor(last - first, 256), 256, 0, c->stream>>>(first, last, n, a, c->pairAcc.as<double>());
        return launched(c, "avOnceFinish");
    } else {
        a.wh = c->whx64.p;
        a.w64 = tabW64(c);
        return withKernelForm(c, [&](auto smooth) {
            avKernel<Fp64Tag, decltype(smooth)::value><<<blocks, kPairBlock, 0, c->stream>>>(lv, coordFp64(c, p),
                                                                                              coordMixed(c), a);
            return launched(c, "avKernel");
        });
    }
    return launched(c, "avKernel");
}

int passMomentumEnergyVe(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last, int avClean, float* groupDt,
                         double* minDt)
{
    if (!p->vx || !p->vy || !p->vz || !p->prho || !p->c || !p->kx || !p->xm || !p->alpha || !p->ax || !p->ay ||
        !p->az || !p->du || !p->c11 || !p->m)
        return SPHGB_ERR_ARG;
    if (avClean && !(p->dV11 && p->dV12 && p->dV13 && p->dV22 && p->dV23 && p->dV33)) return SPHGB_ERR_ARG;
    SPHGB_TRY(checkPass(c, p, first, last));
    const bool mixed = p->precision == SPHGB_MIXED;
    SPHGB_TRY(launchVeAux<kAuxMe>(c, p));
    ListView lv = listView(c);
    lv.first = first;
    lv.last = last;
    MeVeArgs a{};
    a.vx = p->vx;
    a.vy = p->vy;
    a.vz = p->vz;
    a.h = p->h;
    a.m = p->m;
    a.prho = p->prho;
    a.c = p->c;
    a.kx = p->kx;
    a.xm = p->xm;
    a.alpha = p->alpha;
    a.c11 = p->c11;
    a.c12 = p->c12;
    a.c13 = p->c13;
    a.c22 = p->c22;
    a.c23 = p->c23;
    a.c33 = p->c33;
    a.dV11 = p->dV11;
    a.dV12 = p->dV12;
    a.dV13 = p->dV13;
    a.dV22 = p->dV22;
    a.dV23 = p->dV23;
    a.dV33 = p->dV33;
    a.hInv64 = c->hInv64.as<double>();
    a.aux = c->aux.p;
    a.n = p->n;
    a.K = c->K;
    a.Kcour = float(c->prm.Kcour);
    a.ax = p->ax;
    a.ay = p->ay;
    a.az = p->az;
    a.du = p->du;
    a.groupDt = groupDt;
    SPHGB_TRY(beginDtReduction(c, &a.minDt));
    unsigned blocks = gridFor(last - first, kPairBlock);
    auto cf = coordFp64(c, p);
    auto cm = coordMixed(c);
    if (mixed) {
        a.wh = c->whH32.p;
        SPHGB_TRY(c->pack.ensure(sizeof(Rec8) * 3 * size_t(p->n)));
        meVePackKernel<<<gridFor(p->n, 256), 256, 0, c->stream>>>(p->n, a, c->gridKey.as<u64>(),
                                                                 c->gridLoc.as<float4>(), c->pack.as<float4>());
        SPHGB_TRY(launched(c, "meVePackKernel"));
        a.pack = c->pack.as<Rec8>();
        if (avClean) meVeKernel<MixedTag, true><<<blocks, kPairBlock, 0, c->stream>>>(lv, cf, cm, a);
        else meVeKernel<MixedTag, false><<<blocks, kPairBlock, 0, c->stream>>>(lv, cf, cm, a);
    } else {
        a.wh = c->whx64.p;
        a.w64 = tabW64(c);
        double* tape;
        SPHGB_TRY(tapeFor(c, p, first, last, kTapeMe, &tape));
        if (tape) {
            a.tapeEn = tape + int64_t(kTapeEn) * p->n;
            a.tapeAvE = tape + int64_t(kTapeAvE) * p->n;
        }
        // one evaluation per mutual pair when the lists cover all particles and the order may vary
        const bool once = !avClean && pairOnce(c, p, first, last);
        if (once) {
            SPHGB_TRY(c->pairAcc.ensure(sizeof(double) * 6 * size_t(p->n)));
            SPHGB_CUDA(cudaMemsetAsync(c->pairAcc.p, 0, sizeof(double) * 6 * size_t(p->n), c->stream));
            a.owned = c->owned.as<uint32_t>();
            a.ownedCount = c->ownedCount.as<uint32_t>();
            a.acc = c->pairAcc.as<double>();
            SPHGB_TRY(withKernelForm(c, [&](auto smooth) {
                meVeOnceKernel<decltype(smooth)::value><<<blocks, kPairBlock, 0, c->stream>>>(lv, cf, a,
                                                                                              pairGeoRead(c));
                return launched(c, "meVeOnceKernel");
            }));
            meVeOnceFinish<<<blocks, kPairBlock, 0, c->stream>>>(lv, a);
            SPHGB_TRY(launched(c, "meVeOnceFinish"));
            return endDtReduction(c, a.minDt, minDt);
        }
        SPHGB_TRY(withKernelForm(c, [&](auto smooth) {
            constexpr bool S = decltype(smooth)::value;
            if (avClean) meVeKernel<Fp64Tag, true, S><<<blocks, kPairBlock, 0, c->stream>>>(lv, cf, cm, a);
            else meVeKernel<Fp64Tag, false, S><<<blocks, kPairBlock, 0, c->stream>>>(lv, cf, cm, a);
            return launched(c, "meVeKernel");
        }));
        return endDtReduction(c, a.minDt, minDt);
    }
    SPHGB_TRY(launched(c, "meVeKernel"));
    return endDtReduction(c, a.minDt, minDt);
}

}  // namespace sphgb
