// Standard-SPH pair passes: density, ideal-gas EOS, IAD, momentum and energy.
//
// Reference j-loops restated:
//   density  -> xmassJLoop with rho<->xm swapped, then rho = m / xm
//               (sph/include/sph/hydro_std/density.hpp:41-60, hydro_ve/xmass_kern.hpp:50-79)
//   EOS      -> idealGasEOS_u (hydro_std/eos.hpp:54-80, sph/eos.hpp:34-44)
//   IAD      -> IADJLoopSTD (hydro_std/iad_kern.hpp:12-77)
//   ME       -> momentumAndEnergyJLoop + tsKCourant (hydro_std/momentum_energy_kern.hpp:12-134,
//               momentum_energy.hpp:41-101)
// FP64 form: per-particle quotients (m/rho, p/rho, p/rho^2, 1/h, 1/h^3) are formed once per
// particle, 1/|r| comes from rsqrt, periodic wrap tests run only where they can fire; results
// agree with the reference to rounding.  Mixed form: FP32 pair arithmetic on grid-local
// offsets, Kahan sums, per-particle epilogues (normalisation, 3x3 inverse factor) in FP64.
#include "pairs.cuh"

namespace sphgb {

namespace {

// ---------------------------------------------------------------- density / xmass
// neighbour-side fields of the mixed density / xmass pass: grid position and m in one 32-byte block
// per particle (one 256-bit load)
__global__ void packXmassKernel(int64_t n, const void* m, const u64* __restrict__ cell, const float4* __restrict__ loc,
                                float4* __restrict__ rec)
{
    const int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (j >= n) return;
    packGridBlock(rec + 2 * j, cell[j], loc[j], ld<float>(m, j), 0.f, 0.f);
}

template<class P, bool StoreRho, bool Smooth = false>
__global__ void __launch_bounds__(kPairBlock) xmassKernel(ListView lv, CoordFp64 cf, CoordMixed cm, const void* h,
                                                          const void* m, const void* wh, const double2* w64,
                                                          double K, void* out, const Rec8* rec = nullptr)
{
    const int64_t i = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last) return;
    const int64_t ii = i - lv.first;
    const unsigned nc = lv.capped(ii);
    if constexpr (std::is_same_v<P, Fp64Tag>) {
        const KTab<Smooth> tab{w64};
        auto t = cf.target(i);
        double hi = ld<double>(h, i), mi = ld<double>(m, i);
        double hInv = 1.0 / hi, h3Inv = hInv * hInv * hInv, twoH = 2.0 * hi, hInvDx = hInv * kTabInvDx;
        const bool wrap = cf.needsWrap(t, twoH);
        double rho0 = mi;
        for (unsigned k = 0; k < nc; ++k) {
            uint32_t j = lv.at(ii, k);
            double rx, ry, rz;
            cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
            double r2 = dist2(rx, ry, rz);
            rho0 += lookupX(tab, r2 * invDist(r2) * hInvDx) * ld<double>(m, j);
        }
        double xm = mi / (rho0 * K * h3Inv);
        st<double>(out, i, StoreRho ? mi / xm : xm);
    } else {
        auto t = cm.target(i);
        float mi = ld<float>(m, i);
        KSum rho0;
        rho0.add(mi);
        // the list is read a granule (four entries) per load, the next granule one ahead, and the
        // next neighbour's block is loaded while the current pair is evaluated
        uint4 G = nc > 0 ? lv.granule(ii, 0) : make_uint4(uint32_t(i), 0u, 0u, 0u);
        uint4 Gn = nc > 4 ? lv.granule(ii, 1) : G;
        Rec8 Bn = ldRec8(rec + G.x);
        for (unsigned k = 0; k < nc; ++k) {
            const Rec8 B = Bn;  // cell xl yl zl m
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
            rho0.add(lookupH32(static_cast<const float4*>(wh), dist * t.hInv) * B.v[5]);
        }
        double hi = double(ld<float>(h, i));
        double rho = rho0.value64() * K / (hi * hi * hi);
        st<float>(out, i, StoreRho ? float(rho) : float(double(mi) / rho));
    }
}

// FP64 xmass / density with one evaluation per mutual pair over the owned lists: i adds
// W(d / h_i) m_j, and for a mutual pair j receives W(d / h_j) m_i by an FP64 atomic.  Inside a
// sweep it also fills the pair-geometry cache (geo) the later pair-once passes read.
template<bool Smooth>
__global__ void __launch_bounds__(kPairBlock) xmassOnceKernel(ListView lv, OwnedView ov, CoordFp64 cf,
                                                               const double* h, const double* m, KTab<Smooth> tab,
                                                               const double* hInvDx, double* acc, PairGeo geo,
                                                               const double* vx, const double* vy, const double* vz)
{
    const int64_t i = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last) return;
    const int64_t ii = i - lv.first;
    const unsigned no = ov.size(ii);
    auto t = cf.target(i);
    const double hi = h[i], mi = m[i], twoH = 2.0 * hi, hiInvDx = hInvDx[i];
    const bool wrap = cf.needsWrap(t, twoH);
    const int64_t gb = geo.base(ii);
    const double vxi = geo.x ? vx[i] : 0.0, vyi = geo.x ? vy[i] : 0.0, vzi = geo.x ? vz[i] : 0.0;
    double rho0 = 0.0;
    for (unsigned k = 0; k < no; ++k) {
        bool mutual;
        const uint32_t j = ov.at(ii, k, mutual);
        double rx, ry, rz;
        cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
        const double r2 = dist2(rx, ry, rz);
        const double rinv = invDist(r2);
        const double dist = r2 * rinv;
        const double wi = lookupX(tab, dist * hiInvDx);
        rho0 += wi * __ldg(m + j);
        if (geo.g) {  // the sweep's later pair-once passes load the geometry and both kernel values
            const double wj = lookupX(tab, dist * __ldg(hInvDx + j));
            const int64_t e = gb + 32 * int64_t(k);
            geo.g[e] = make_double2(dist, rinv);
            geo.w[e] = make_double2(wi, wj);
            if (geo.x) {
                const double dvx = __ldg(vx + j) - vxi, dvy = __ldg(vy + j) - vyi, dvz = __ldg(vz + j) - vzi;
                geo.x[e] = make_double2(rx, ry);
                geo.x[geo.plane + e] = make_double2(rz, dvx);
                geo.x[2 * geo.plane + e] = make_double2(dvy, dvz);
            }
            if (mutual) atomicAdd(acc + j, wj * mi);
        } else if (mutual) {
            atomicAdd(acc + j, lookupX(tab, dist * __ldg(hInvDx + j)) * mi);
        }
    }
    atomicAdd(acc + i, rho0);
}

template<bool StoreRho>
__global__ void xmassOnceFinish(int64_t first, int64_t last, const double* h, const double* m, double K,
                                const double* acc, double* out)
{
    const int64_t i = first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= last) return;
    const double hi = h[i], mi = m[i];
    const double hInv = 1.0 / hi, h3Inv = hInv * hInv * hInv;
    const double xm = mi / ((mi + acc[i]) * K * h3Inv);
    out[i] = StoreRho ? mi / xm : xm;
}

// ---------------------------------------------------------------- EOS
template<class P>
__global__ void eosStdKernel(int64_t first, int64_t last, const double* u, const void* rho, double gamma, void* p,
                             void* c)
{
    using T = typename P::T;
    int64_t i = first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= last) return;
    double tmp = u[i] * (gamma - 1.0);
    double pi = double(ld<T>(rho, i)) * tmp;
    st<T>(p, i, T(pi));
    st<T>(c, i, T(sqrt(gamma * tmp)));
}

// ---------------------------------------------------------------- per-particle quotients
// aux[0,n) m/rho, [n,2n) p/rho, [2n,3n) p/rho^2
template<class T>
__global__ void stdAuxKernel(int64_t n, const void* m, const void* rho, const void* p, T* aux)
{
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    T ri = ld<T>(rho, i);
    aux[i] = ld<T>(m, i) / ri;
    if (p) {
        T pi = ld<T>(p, i);
        aux[n + i] = pi / (ri * T(1));
        aux[2 * n + i] = pi / (T(1) * ri * ri);
    }
}

template<class P>
int launchStdAux(sphgb_ctx* c, const sphgb_particles* p, bool withPressure)
{
    using T = typename P::T;
    const int64_t n = p->n;
    SPHGB_TRY(c->aux.ensure(sizeof(T) * 3 * n));
    stdAuxKernel<T><<<gridFor(n, 256), 256, 0, c->stream>>>(n, p->m, p->rho, withPressure ? p->p : nullptr,
                                                            c->aux.as<T>());
    return launched(c, "stdAuxKernel");
}

// ---------------------------------------------------------------- IAD
struct IadOut {
    void *c11, *c12, *c13, *c22, *c23, *c33;
};

// vol[j] = m[j] / rho[j], formed once per particle (the reference divides per pair)
template<class P, bool Smooth = false>
__global__ void __launch_bounds__(kPairBlock) iadKernel(ListView lv, CoordFp64 cf, CoordMixed cm, const void* h,
                                                        const void* vol, const void* wh, const double2* w64,
                                                        double K, IadOut o)
{
    const int64_t i = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last) return;
    const int64_t ii = i - lv.first;
    const unsigned nc = lv.capped(ii);
    if constexpr (std::is_same_v<P, Fp64Tag>) {
        const KTab<Smooth> tab{w64};
        auto t = cf.target(i);
        double hi = ld<double>(h, i), hiInv = 1.0 / hi, twoH = 2.0 * hi, hInvDx = hiInv * kTabInvDx;
        const bool wrap = cf.needsWrap(t, twoH);
        double t11 = 0, t12 = 0, t13 = 0, t22 = 0, t23 = 0, t33 = 0;
        for (unsigned k = 0; k < nc; ++k) {
            uint32_t j = lv.at(ii, k);
            double rx, ry, rz;
            cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
            double r2 = dist2(rx, ry, rz);
            double w = lookupX(tab, r2 * invDist(r2) * hInvDx);
            double vw = ld<double>(vol, j) * w;
            t11 += rx * rx * vw;
            t12 += rx * ry * vw;
            t13 += rx * rz * vw;
            t22 += ry * ry * vw;
            t23 += ry * rz * vw;
            t33 += rz * rz * vw;
        }
        double cc[6];
        iadInvert<double>(t11, t12, t13, t22, t23, t33, hi, K, cc);
        st<double>(o.c11, i, cc[0]);
        st<double>(o.c12, i, cc[1]);
        st<double>(o.c13, i, cc[2]);
        st<double>(o.c22, i, cc[3]);
        st<double>(o.c23, i, cc[4]);
        st<double>(o.c33, i, cc[5]);
    } else {
        const float4* tab = static_cast<const float4*>(wh);
        auto t = cm.target(i);
        KSum t11, t12, t13, t22, t23, t33;
        for (unsigned k = 0; k < nc; ++k) {
            uint32_t j = lv.at(ii, k);
            float rx, ry, rz, hjInv;
            cm.diff(t, j, rx, ry, rz, hjInv);
            float dist = sqrtf(fmaf(rx, rx, fmaf(ry, ry, rz * rz)));
            float w = lookupH32(tab, dist * t.hInv);
            float vw = ld<float>(vol, j) * w;
            t11.add(rx * rx * vw);
            t12.add(rx * ry * vw);
            t13.add(rx * rz * vw);
            t22.add(ry * ry * vw);
            t23.add(ry * rz * vw);
            t33.add(rz * rz * vw);
        }
        float cc[6];
        iadInvert<float>(t11.value(), t12.value(), t13.value(), t22.value(), t23.value(), t33.value(),
                         double(ld<float>(h, i)), K, cc);
        st<float>(o.c11, i, cc[0]);
        st<float>(o.c12, i, cc[1]);
        st<float>(o.c13, i, cc[2]);
        st<float>(o.c22, i, cc[3]);
        st<float>(o.c23, i, cc[4]);
        st<float>(o.c33, i, cc[5]);
    }
}

// ---------------------------------------------------------------- momentum and energy (std)
struct MeStdArgs {
    const void *vx, *vy, *vz, *h, *m, *rho, *p, *c;
    const void *c11, *c12, *c13, *c22, *c23, *c33;
    const void* wh;        // mixed: cubic pieces of W
    const double2* w64;    // FP64: W in the context's form
    const double* hInv64;  // [0,n) 1/h, [n,2n) 1/h^3, [2n,3n) 1/(h dx)
    const void* aux;       // m/rho, p/rho, p/rho^2
    int64_t n;
    double K;
    float Kcour;
    void *ax, *ay, *az;
    double* du;
    unsigned long long* minDt;
};

template<class P, bool Smooth = false>
__global__ void __launch_bounds__(kPairBlock) meStdKernel(ListView lv, CoordFp64 cf, CoordMixed cm, MeStdArgs a)
{
    using T = typename P::T;
    const int64_t i0 = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const bool valid = i0 < lv.last;
    const int64_t i = valid ? i0 : lv.first;
    const int64_t ii = i - lv.first;
    const unsigned nc = valid ? lv.capped(ii) : 0u;
    const T* aux = static_cast<const T*>(a.aux);
    const T *auxMoR = aux, *auxPoR = aux + a.n, *auxPoR2 = aux + 2 * a.n;
    double dt = INFINITY;

    T hi = ld<T>(a.h, i), ci = ld<T>(a.c, i);
    T vxi = ld<T>(a.vx, i), vyi = ld<T>(a.vy, i), vzi = ld<T>(a.vz, i);
    T mi_roi = auxMoR[i], proi2 = auxPoR2[i];
    T c11i = ld<T>(a.c11, i), c12i = ld<T>(a.c12, i), c13i = ld<T>(a.c13, i);
    T c22i = ld<T>(a.c22, i), c23i = ld<T>(a.c23, i), c33i = ld<T>(a.c33, i);
    T maxv = 0;

    if constexpr (std::is_same_v<P, Fp64Tag>) {
        auto t = cf.target(i);
        const KTab<Smooth> tabX{a.w64};
        const double* hInv3 = a.hInv64 + a.n;
        const double* hInvDx = a.hInv64 + 2 * a.n;
        T hiInv3 = hInv3[i], hiInvDx = hInvDx[i], twoH = 2.0 * hi;
        const bool wrap = cf.needsWrap(t, twoH);
        T mx = 0, my = 0, mz = 0, en = 0;
        long long maxvBits = 0;
        for (unsigned k = 0; k < nc; ++k) {
            uint32_t j = lv.at(ii, k);
            T rx, ry, rz;
            cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
            T r2 = dist2(rx, ry, rz);
            T rinv = invDist(r2);
            T dist = r2 * rinv;
            T vxij = vxi - ld<T>(a.vx, j), vyij = vyi - ld<T>(a.vy, j), vzij = vzi - ld<T>(a.vz, j);
            T rv = rx * vxij + ry * vyij + rz * vzij;
            T Wi = hiInv3 * lookupX(tabX, dist * hiInvDx);
            T Wj = __ldg(hInv3 + j) * lookupX(tabX, dist * __ldg(hInvDx + j));
            T a1i = c11i * rx + c12i * ry + c13i * rz;
            T a2i = c12i * rx + c22i * ry + c23i * rz;
            T a3i = c13i * rx + c23i * ry + c33i * rz;
            T c11j = ld<T>(a.c11, j), c12j = ld<T>(a.c12, j), c13j = ld<T>(a.c13, j);
            T c22j = ld<T>(a.c22, j), c23j = ld<T>(a.c23, j), c33j = ld<T>(a.c33, j);
            T a1j = c11j * rx + c12j * ry + c13j * rz;
            T a2j = c12j * rx + c22j * ry + c23j * rz;
            T a3j = c13j * rx + c23j * ry + c33j * rz;
            T cj = ld<T>(a.c, j);
            T wij = rv * rinv;
            T visc = T(0.5) * artificialViscosity<T>(1.0, 1.0, ci, cj, wij);
            maxvBits = maxBitsNonNeg(maxvBits, ci + cj - T(3) * wij);
            T mj = ld<T>(a.m, j);
            T mjrojWj = __ldg(auxMoR + j) * Wj;
            T mjproi = mj * proi2;
            {
                T aa = Wi * (mjproi + visc * mi_roi);
                T bb = mjrojWj * (__ldg(auxPoR + j) + visc);
                mx += aa * a1i + bb * a1j;
                my += aa * a2i + bb * a2j;
                mz += aa * a3i + bb * a3j;
            }
            {
                T aa = Wi * (T(2) * mjproi + visc * mi_roi);
                T bb = visc * mjrojWj;
                en += vxij * (aa * a1i + bb * a1j) + vyij * (aa * a2i + bb * a2j) + vzij * (aa * a3i + bb * a3j);
            }
        }
        if (valid) {
            a.du[i] = -a.K * 0.5 * en;
            st<T>(a.ax, i, a.K * mx);
            st<T>(a.ay, i, a.K * my);
            st<T>(a.az, i, a.K * mz);
            dt = courantDt(__longlong_as_double(maxvBits), hi, ci, a.Kcour);
        }
    } else {
        auto t = cm.target(i);
        const float4* tab2 = reinterpret_cast<const float4*>(a.wh);
        T hiInv = t.hInv, hiInv3 = hiInv * hiInv * hiInv;
        KSum mx, my, mz, en;
        for (unsigned k = 0; k < nc; ++k) {
            uint32_t j = lv.at(ii, k);
            T rx, ry, rz, hjInv;
            cm.diff(t, j, rx, ry, rz, hjInv);
            T r2 = fmaf(rx, rx, fmaf(ry, ry, rz * rz));
            T rinv = rsqrtf(r2);
            T dist = r2 * rinv;
            T vxij = vxi - ld<T>(a.vx, j), vyij = vyi - ld<T>(a.vy, j), vzij = vzi - ld<T>(a.vz, j);
            T v1 = dist * hiInv, v2 = dist * hjInv;
            T rv = rx * vxij + ry * vyij + rz * vzij;
            T Wi = hiInv3 * lookupH32(tab2, v1);
            T Wj = (hjInv * hjInv * hjInv) * lookupH32(tab2, v2);
            T a1i = c11i * rx + c12i * ry + c13i * rz;
            T a2i = c12i * rx + c22i * ry + c23i * rz;
            T a3i = c13i * rx + c23i * ry + c33i * rz;
            T c11j = ld<T>(a.c11, j), c12j = ld<T>(a.c12, j), c13j = ld<T>(a.c13, j);
            T c22j = ld<T>(a.c22, j), c23j = ld<T>(a.c23, j), c33j = ld<T>(a.c33, j);
            T a1j = c11j * rx + c12j * ry + c13j * rz;
            T a2j = c12j * rx + c22j * ry + c23j * rz;
            T a3j = c13j * rx + c23j * ry + c33j * rz;
            T cj = ld<T>(a.c, j);
            T wij = rv * rinv;
            T visc = T(0.5) * artificialViscosity<T>(1.f, 1.f, ci, cj, wij);
            T vsig = ci + cj - T(3) * wij;
            maxv = (vsig > maxv) ? vsig : maxv;
            T mj = ld<T>(a.m, j);
            T mjrojWj = __ldg(auxMoR + j) * Wj;
            T mjproi = mj * proi2;
            T aa = Wi * (mjproi + visc * mi_roi);
            T bb = mjrojWj * (__ldg(auxPoR + j) + visc);
            mx.add(aa * a1i + bb * a1j);
            my.add(aa * a2i + bb * a2j);
            mz.add(aa * a3i + bb * a3j);
            T ae = Wi * (T(2) * mjproi + visc * mi_roi);
            T be = visc * mjrojWj;
            en.add(vxij * (ae * a1i + be * a1j) + vyij * (ae * a2i + be * a2j) + vzij * (ae * a3i + be * a3j));
        }
        if (valid) {
            a.du[i] = -a.K * 0.5 * en.value64();
            st<T>(a.ax, i, float(a.K * mx.value64()));
            st<T>(a.ay, i, float(a.K * my.value64()));
            st<T>(a.az, i, float(a.K * mz.value64()));
            dt = courantDt(double(maxv), double(hi), double(ci), a.Kcour);
        }
    }
    if (a.minDt) blockMinDt(dt, a.minDt);
}

template<class P>
int launchXmass(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last, void* out, bool storeRho)
{
    SPHGB_TRY(checkPass(c, p, first, last));
    ListView lv = listView(c);
    lv.first = first;
    lv.last = last;
    CoordFp64 cf = coordFp64(c, p);
    CoordMixed cm = coordMixed(c);
    const void* wh = std::is_same_v<P, Fp64Tag> ? c->whx64.p : c->whH32.p;
    unsigned blocks = gridFor(last - first, kPairBlock);
    // pair-once for the VE xmass; the std density keeps the order-fixed walk
    if (std::is_same_v<P, Fp64Tag> && !storeRho && pairOnce(c, p, first, last)) {
        const int64_t n = p->n;
        SPHGB_TRY(c->pairAcc.ensure(sizeof(double) * size_t(n)));
        SPHGB_CUDA(cudaMemsetAsync(c->pairAcc.p, 0, sizeof(double) * size_t(n), c->stream));
        PairGeo geo;
        SPHGB_TRY(pairGeoStore(c, &geo));
        SPHGB_TRY(withKernelForm(c, [&](auto smooth) {
            constexpr bool S = decltype(smooth)::value;
            xmassOnceKernel<S><<<blocks, kPairBlock, 0, c->stream>>>(
                lv, ownedView(c), cf, static_cast<const double*>(p->h), static_cast<const double*>(p->m),
                KTab<S>{tabW64(c)}, c->hInv64.as<double>() + 2 * n, c->pairAcc.as<double>(), geo,
                static_cast<const double*>(p->vx), static_cast<const double*>(p->vy),
                static_cast<const double*>(p->vz));
            return launched(c, "xmassOnceKernel");
        }));
        const unsigned eb = gridFor(last - first, 256);
        if (storeRho)
            xmassOnceFinish<true><<<eb, 256, 0, c->stream>>>(first, last, static_cast<const double*>(p->h),
                                                              static_cast<const double*>(p->m), c->K,
                                                              c->pairAcc.as<double>(), static_cast<double*>(out));
        else
            xmassOnceFinish<false><<<eb, 256, 0, c->stream>>>(first, last, static_cast<const double*>(p->h),
                                                               static_cast<const double*>(p->m), c->K,
                                                               c->pairAcc.as<double>(), static_cast<double*>(out));
        return launched(c, "xmassOnceFinish");
    }
    const Rec8* rec = nullptr;
    if constexpr (std::is_same_v<P, MixedTag>) {
        SPHGB_TRY(c->pack.ensure(sizeof(Rec8) * 3 * size_t(p->n)));  // the ME blocks' space, free here
        packXmassKernel<<<gridFor(p->n, 256), 256, 0, c->stream>>>(p->n, p->m, c->gridKey.as<u64>(),
                                                                    c->gridLoc.as<float4>(), c->pack.as<float4>());
        SPHGB_TRY(launched(c, "packXmassKernel"));
        rec = c->pack.as<Rec8>();
    }
    return withKernelForm(c, [&](auto smooth) {
        constexpr bool S = std::is_same_v<P, Fp64Tag> && decltype(smooth)::value;
        if (storeRho)
            xmassKernel<P, true, S><<<blocks, kPairBlock, 0, c->stream>>>(lv, cf, cm, p->h, p->m, wh, tabW64(c),
                                                                           c->K, out, rec);
        else
            xmassKernel<P, false, S><<<blocks, kPairBlock, 0, c->stream>>>(lv, cf, cm, p->h, p->m, wh, tabW64(c),
                                                                            c->K, out, rec);
        return launched(c, "xmassKernel");
    });
}

template<class P>
int launchIad(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    SPHGB_TRY(launchStdAux<P>(c, p, false));
    ListView lv = listView(c);
    lv.first = first;
    lv.last = last;
    const void* wh = std::is_same_v<P, Fp64Tag> ? c->whx64.p : c->whH32.p;
    return withKernelForm(c, [&](auto smooth) {
        constexpr bool S = std::is_same_v<P, Fp64Tag> && decltype(smooth)::value;
        iadKernel<P, S><<<gridFor(last - first, kPairBlock), kPairBlock, 0, c->stream>>>(
            lv, coordFp64(c, p), coordMixed(c), p->h, c->aux.p, wh, tabW64(c), c->K,
            IadOut{p->c11, p->c12, p->c13, p->c22, p->c23, p->c33});
        return launched(c, "iadKernel");
    });
}

template<class P>
int launchMeStd(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last, double* minDt)
{
    SPHGB_TRY(launchStdAux<P>(c, p, true));
    ListView lv = listView(c);
    lv.first = first;
    lv.last = last;
    MeStdArgs a{};
    a.vx = p->vx;
    a.vy = p->vy;
    a.vz = p->vz;
    a.h = p->h;
    a.m = p->m;
    a.rho = p->rho;
    a.p = p->p;
    a.c = p->c;
    a.c11 = p->c11;
    a.c12 = p->c12;
    a.c13 = p->c13;
    a.c22 = p->c22;
    a.c23 = p->c23;
    a.c33 = p->c33;
    a.wh = std::is_same_v<P, Fp64Tag> ? c->whx64.p : c->whH32.p;
    a.w64 = tabW64(c);
    a.hInv64 = c->hInv64.as<double>();
    a.aux = c->aux.p;
    a.n = p->n;
    a.K = c->K;
    a.Kcour = float(c->prm.Kcour);
    a.ax = p->ax;
    a.ay = p->ay;
    a.az = p->az;
    a.du = p->du;
    SPHGB_TRY(beginDtReduction(c, &a.minDt));
    SPHGB_TRY(withKernelForm(c, [&](auto smooth) {
        constexpr bool S = std::is_same_v<P, Fp64Tag> && decltype(smooth)::value;
        meStdKernel<P, S><<<gridFor(last - first, kPairBlock), kPairBlock, 0, c->stream>>>(lv, coordFp64(c, p),
                                                                                            coordMixed(c), a);
        return launched(c, "meStdKernel");
    }));
    return endDtReduction(c, a.minDt, minDt);
}

}  // namespace

int passDensity(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    if (!p->rho || !p->m || !p->h) return SPHGB_ERR_ARG;
    if (p->precision == SPHGB_MIXED) return launchXmass<MixedTag>(c, p, first, last, p->rho, true);
    return launchXmass<Fp64Tag>(c, p, first, last, p->rho, true);
}

int passXMass(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    if (!p->xm || !p->m || !p->h) return SPHGB_ERR_ARG;
    if (p->precision == SPHGB_MIXED) return launchXmass<MixedTag>(c, p, first, last, p->xm, false);
    return launchXmass<Fp64Tag>(c, p, first, last, p->xm, false);
}

int passEosStd(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    if (!p->u || !p->rho || !p->p || !p->c || first < 0 || last > p->n || first >= last) return SPHGB_ERR_ARG;
    unsigned blocks = gridFor(last - first, 256);
    if (p->precision == SPHGB_MIXED)
        eosStdKernel<MixedTag><<<blocks, 256, 0, c->stream>>>(first, last, p->u, p->rho, c->prm.gamma, p->p, p->c);
    else
        eosStdKernel<Fp64Tag><<<blocks, 256, 0, c->stream>>>(first, last, p->u, p->rho, c->prm.gamma, p->p, p->c);
    return launched(c, "eosStdKernel");
}

int passIadStd(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    if (!p->m || !p->rho || !p->c11 || !p->c12 || !p->c13 || !p->c22 || !p->c23 || !p->c33) return SPHGB_ERR_ARG;
    SPHGB_TRY(checkPass(c, p, first, last));
    if (p->precision == SPHGB_MIXED) return launchIad<MixedTag>(c, p, first, last);
    return launchIad<Fp64Tag>(c, p, first, last);
}

int passMomentumEnergyStd(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last, double* minDt)
{
    if (!p->vx || !p->vy || !p->vz || !p->rho || !p->p || !p->c || !p->ax || !p->ay || !p->az || !p->du ||
        !p->c11 || !p->m)
        return SPHGB_ERR_ARG;
    SPHGB_TRY(checkPass(c, p, first, last));
    if (p->precision == SPHGB_MIXED) return launchMeStd<MixedTag>(c, p, first, last, minDt);
    return launchMeStd<Fp64Tag>(c, p, first, last, minDt);
}

}  // namespace sphgb
