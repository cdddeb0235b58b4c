// FP64 refinement of ill-conditioned particles in the mixed form.
//
// Two outputs of the VE chain can be ill-conditioned in their inputs, so that the mixed form's
// input errors (a few 1e-7 relative in xm, kx, c_ij) move them far more than 1e-7:
//   gradh_i = 1 - dhdrho * whomega (ve_def_gradh_kern.hpp:80-88) near 0, as at the open surface
//     of a clustered set: prho_i ~ 1 / gradh_i inherits the relative error times 1 / gradh_i;
//   the sign of divv_i, which switches the AV source term on and off (av_switches_kern.hpp:114-120),
//     when |divv_i| is below the mixed error: alpha_i then jumps between branches.
// The passes flag such particles (|gradh| < 0.1; |divv| below an error bound the mixed IAD+divv
// kernel accumulates) and this file recomputes their dependency cone in FP64 from the exact inputs
// (x y z in FP64; h m v u are FP32 fields, converted exactly):
//   gradh: xm on the flagged particles and their neighbours, then kx and gradh on the flagged ones;
//   divv:  xm two neighbour shells out, kx on the flagged particles and their neighbours, then the
//          IAD matrix and divv of the flagged ones.
// The refined values are written back (rounded to FP32) before the next pass reads them.  Work is
// proportional to the flagged cones; nothing runs when no particle is flagged.
#include "pairs.cuh"

namespace sphgb {

namespace {

constexpr int kRefBlock = 128;

struct RefArgs {
    ListView lv;
    CoordFp64 cf;
    const float *h, *m, *xm, *vx, *vy, *vz;
    const double2 *tw, *tdw;  // FP64 kernel tables, interleaved
    double K;
    int64_t n;
    uint8_t *flag, *shell1, *shell2;  // target set, its first and second neighbour shells
    double *xm64, *kx64, *gradh64;
};

__device__ __forceinline__ double pairDist(const RefArgs& a, const CoordFp64::Target& t, uint32_t j, double twoH,
                                           bool wrap)
{
    double rx, ry, rz;
    a.cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
    const double r2 = rx * rx + ry * ry + rz * rz;
    return r2 * invDist(r2);
}

// mark the particles in `src` and their neighbours in `dst` (every writer stores 1)
__global__ void dilateKernel(ListView lv, const uint8_t* __restrict__ src, uint8_t* __restrict__ dst)
{
    const int64_t i = lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= lv.last || !src[i]) return;
    dst[i] = 1;
    const int64_t ii = i - lv.first;
    const unsigned nc = lv.capped(ii);
    for (unsigned k = 0; k < nc; ++k) dst[lv.at(ii, k)] = 1;
}

// xmassJLoop in FP64 (hydro_ve/xmass_kern.hpp:50-79) for the marked particles
__global__ void __launch_bounds__(kRefBlock) refXmassKernel(RefArgs a, const uint8_t* __restrict__ mark)
{
    const int64_t i = a.lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.lv.last || !mark[i]) return;
    const int64_t ii = i - a.lv.first;
    const unsigned nc = a.lv.capped(ii);
    auto t = a.cf.target(i);
    const double hi = a.h[i], mi = a.m[i], hInv = 1.0 / hi, twoH = 2.0 * hi;
    const bool wrap = a.cf.needsWrap(t, twoH);
    double rho0 = mi;
    for (unsigned k = 0; k < nc; ++k) {
        const uint32_t j = a.lv.at(ii, k);
        rho0 += lookupX(a.tw, pairDist(a, t, j, twoH, wrap) * hInv * kTabInvDx) * double(a.m[j]);
    }
    a.xm64[i] = mi / (rho0 * a.K * (hInv * hInv * hInv));
}

// veDefGradhJLoop in FP64 (hydro_ve/ve_def_gradh_kern.hpp:43-90) on the FP64 xm of the neighbours
__global__ void __launch_bounds__(kRefBlock) refGradhKernel(RefArgs a, const uint8_t* __restrict__ mark)
{
    const int64_t i = a.lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.lv.last || !mark[i]) return;
    const int64_t ii = i - a.lv.first;
    const unsigned nc = a.lv.capped(ii);
    auto t = a.cf.target(i);
    const double hi = a.h[i], mi = a.m[i], xmi = a.xm64[i];
    const double hInv = 1.0 / hi, h3Inv = hInv * hInv * hInv, twoH = 2.0 * hi;
    const bool wrap = a.cf.needsWrap(t, twoH);
    double kxi = xmi, whomega = -3.0 * xmi, wrho0 = -3.0 * mi;
    for (unsigned k = 0; k < nc; ++k) {
        const uint32_t j = a.lv.at(ii, k);
        const double v = pairDist(a, t, j, twoH, wrap) * hInv;
        const TabSlot sl = tabSlot(v * kTabInvDx);
        const double w = lookupX(a.tw, sl), dw = lookupX(a.tdw, sl);
        const double dterh = -(3.0 * w + v * dw);
        const double xmj = a.xm64[j];
        kxi += w * xmj;
        whomega += dterh * xmj;
        wrho0 += dterh * double(a.m[j]);
    }
    kxi *= a.K * h3Inv;
    whomega *= a.K * h3Inv * hInv;
    wrho0 *= a.K * h3Inv * hInv;
    whomega = whomega * mi / xmi + (kxi - a.K * xmi * h3Inv) * wrho0;
    const double rhoi = kxi * mi / xmi;
    const double dhdrho = -hi / (rhoi * 3.0);
    a.kx64[i] = kxi;
    a.gradh64[i] = 1.0 - dhdrho * whomega;
}

__global__ void writeGradhKernel(RefArgs a, float* __restrict__ kx, float* __restrict__ gradh)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.n || !a.flag[i]) return;
    kx[i] = float(a.kx64[i]);
    gradh[i] = float(a.gradh64[i]);
}

// IADJLoop + divV_curlVJLoop in FP64 (hydro_ve/iad_kern.hpp:43-109, divv_curlv_kern.hpp:43-123):
// divv of the flagged particles from FP64 xm and kx of their neighbours
__global__ void __launch_bounds__(kRefBlock) refDivvKernel(RefArgs a, float* __restrict__ divv)
{
    const int64_t i = a.lv.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.lv.last || !a.flag[i]) return;
    const int64_t ii = i - a.lv.first;
    const unsigned nc = a.lv.capped(ii);
    auto t = a.cf.target(i);
    const double hi = a.h[i], hInv = 1.0 / hi, twoH = 2.0 * hi;
    const bool wrap = a.cf.needsWrap(t, twoH);
    const double vxi = a.vx[i], vyi = a.vy[i], vzi = a.vz[i];
    double t11 = 0, t12 = 0, t13 = 0, t22 = 0, t23 = 0, t33 = 0;
    double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (unsigned k = 0; k < nc; ++k) {
        const uint32_t j = a.lv.at(ii, k);
        double rx, ry, rz;
        a.cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
        const double r2 = rx * rx + ry * ry + rz * rz;
        const double w = lookupX(a.tw, r2 * invDist(r2) * hInv * kTabInvDx);
        const double vw = a.xm64[j] / a.kx64[j] * w;
        t11 += rx * rx * vw;
        t12 += rx * ry * vw;
        t13 += rx * rz * vw;
        t22 += ry * ry * vw;
        t23 += ry * rz * vw;
        t33 += rz * rz * vw;
        const double xw = a.xm64[j] * w;
        const double sx = (double(a.vx[j]) - vxi) * xw, sy = (double(a.vy[j]) - vyi) * xw,
                     sz = (double(a.vz[j]) - vzi) * xw;
        M[0] += sx * rx;
        M[4] += sy * ry;
        M[8] += sz * rz;
        M[1] += sx * ry;
        M[2] += sx * rz;
        M[3] += sy * rx;
        M[5] += sy * rz;
        M[6] += sz * rx;
        M[7] += sz * ry;
    }
    double cc[6];
    iadInvert<double>(t11, t12, t13, t22, t23, t33, hi, a.K, cc);
    // divv = trace(-M c^T) K / (h^3 kx)
    const double tr = cc[0] * M[0] + cc[1] * (M[1] + M[3]) + cc[2] * (M[2] + M[6]) + cc[3] * M[4] +
                      cc[4] * (M[5] + M[7]) + cc[5] * M[8];
    const double nk = a.K * (hInv * hInv * hInv) / a.kx64[i];
    divv[i] = float(-nk * tr);
}

__global__ void flagGradhKernel(int64_t n, const float* __restrict__ gradh, uint8_t* __restrict__ flag,
                                unsigned long long* __restrict__ count)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    bool f = false;
    if (i < n) {
        f = fabsf(gradh[i]) < 0.1f;
        flag[i] = f;
    }
    const unsigned b = __ballot_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(count, (unsigned long long)__popc(b));
}

__global__ void flagDivvKernel(int64_t n, const float* __restrict__ divv, const float* __restrict__ bound,
                               uint8_t* __restrict__ flag, unsigned long long* __restrict__ count)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    bool f = false;
    if (i < n) {
        f = fabsf(divv[i]) < bound[i];  // bound 0 (no velocity differences): the sign is exact
        flag[i] = f;
    }
    const unsigned b = __ballot_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(count, (unsigned long long)__popc(b));
}

int setup(sphgb_ctx* c, const sphgb_particles* p, RefArgs& a)
{
    const int64_t n = p->n;
    SPHGB_TRY(c->refMask.ensure(3 * size_t(n)));
    SPHGB_TRY(c->refFp64.ensure(sizeof(double) * 3 * size_t(n)));
    SPHGB_TRY(c->counters.ensure(sizeof(unsigned long long) * 8));
    a.lv = listView(c);
    a.cf = coordFp64(c, p);
    a.h = static_cast<const float*>(p->h);
    a.m = static_cast<const float*>(p->m);
    a.xm = static_cast<const float*>(p->xm);
    a.vx = static_cast<const float*>(p->vx);
    a.vy = static_cast<const float*>(p->vy);
    a.vz = static_cast<const float*>(p->vz);
    a.tw = c->whx64.as<double2>();
    a.tdw = c->whdx64.as<double2>();
    a.K = c->K;
    a.n = n;
    a.flag = c->refMask.as<uint8_t>();
    a.shell1 = a.flag + n;
    a.shell2 = a.flag + 2 * n;
    a.xm64 = c->refFp64.as<double>();
    a.kx64 = a.xm64 + n;
    a.gradh64 = a.xm64 + 2 * n;
    return SPHGB_OK;
}

// number of flagged particles, read back (the cone work is skipped when it is 0)
int flaggedCount(sphgb_ctx* c, unsigned long long* dev, int64_t* out)
{
    unsigned long long h = 0;
    SPHGB_CUDA(cudaMemcpyAsync(&h, dev, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    *out = int64_t(h);
    return SPHGB_OK;
}

}  // namespace

int refineMixedGradh(sphgb_ctx* c, sphgb_particles* p)
{
    c->stats_refinedGradh = 0;
    if (!c->refineMixed || p->precision != SPHGB_MIXED || c->nbrFirst != 0 || c->nbrLast != p->n) return SPHGB_OK;
    RefArgs a;
    SPHGB_TRY(setup(c, p, a));
    const int64_t n = p->n;
    unsigned long long* cnt = c->counters.as<unsigned long long>() + 7;
    SPHGB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), c->stream));
    flagGradhKernel<<<gridFor(n, 256), 256, 0, c->stream>>>(n, static_cast<const float*>(p->gradh), a.flag, cnt);
    SPHGB_TRY(launched(c, "flagGradhKernel"));
    int64_t flagged = 0;
    SPHGB_TRY(flaggedCount(c, cnt, &flagged));
    c->stats_refinedGradh = flagged;
    if (flagged == 0) return SPHGB_OK;
    SPHGB_CUDA(cudaMemsetAsync(a.shell1, 0, size_t(n), c->stream));
    const unsigned blocks = gridFor(n, kRefBlock);
    dilateKernel<<<blocks, kRefBlock, 0, c->stream>>>(a.lv, a.flag, a.shell1);
    SPHGB_TRY(launched(c, "dilateKernel"));
    refXmassKernel<<<blocks, kRefBlock, 0, c->stream>>>(a, a.shell1);
    SPHGB_TRY(launched(c, "refXmassKernel"));
    refGradhKernel<<<blocks, kRefBlock, 0, c->stream>>>(a, a.flag);
    SPHGB_TRY(launched(c, "refGradhKernel"));
    writeGradhKernel<<<gridFor(n, 256), 256, 0, c->stream>>>(a, static_cast<float*>(p->kx),
                                                             static_cast<float*>(p->gradh));
    return launched(c, "writeGradhKernel");
}

int refineMixedDivv(sphgb_ctx* c, sphgb_particles* p, const float* bound)
{
    c->stats_refinedDivv = 0;
    if (!c->refineMixed || p->precision != SPHGB_MIXED || !bound || c->nbrFirst != 0 || c->nbrLast != p->n)
        return SPHGB_OK;
    RefArgs a;
    SPHGB_TRY(setup(c, p, a));
    const int64_t n = p->n;
    unsigned long long* cnt = c->counters.as<unsigned long long>() + 7;
    SPHGB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), c->stream));
    flagDivvKernel<<<gridFor(n, 256), 256, 0, c->stream>>>(n, static_cast<const float*>(p->divv), bound, a.flag, cnt);
    SPHGB_TRY(launched(c, "flagDivvKernel"));
    int64_t flagged = 0;
    SPHGB_TRY(flaggedCount(c, cnt, &flagged));
    c->stats_refinedDivv = flagged;
    if (flagged == 0) return SPHGB_OK;
    SPHGB_CUDA(cudaMemsetAsync(a.shell1, 0, 2 * size_t(n), c->stream));
    const unsigned blocks = gridFor(n, kRefBlock);
    dilateKernel<<<blocks, kRefBlock, 0, c->stream>>>(a.lv, a.flag, a.shell1);  // kx needed here
    SPHGB_TRY(launched(c, "dilateKernel"));
    dilateKernel<<<blocks, kRefBlock, 0, c->stream>>>(a.lv, a.shell1, a.shell2);  // xm needed here
    SPHGB_TRY(launched(c, "dilateKernel"));
    refXmassKernel<<<blocks, kRefBlock, 0, c->stream>>>(a, a.shell2);
    SPHGB_TRY(launched(c, "refXmassKernel"));
    refGradhKernel<<<blocks, kRefBlock, 0, c->stream>>>(a, a.shell1);
    SPHGB_TRY(launched(c, "refGradhKernel"));
    refDivvKernel<<<blocks, kRefBlock, 0, c->stream>>>(a, static_cast<float*>(p->divv));
    return launched(c, "refDivvKernel");
}

}  // namespace sphgb
