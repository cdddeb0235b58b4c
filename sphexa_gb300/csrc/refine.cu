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
// The refined values are written back (rounded to FP32) before the next pass reads them.
// The cones are compacted: the flag kernel lists the flagged particles and marks them in a bitmap;
// each dilation walks the lists of the previous shell's particles and appends every neighbour not
// yet marked (atomicOr on the bitmap decides who appends it), so the one index list holds the
// flagged particles, then the first shell, then the second.  The FP64 kernels run one thread per
// listed particle: work is proportional to the cones, in full warps, and nothing runs when no
// particle is flagged.
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
    uint32_t* bits;  // one bit per particle: listed already
    uint32_t* list;  // flagged particles, then the first shell, then the second
    double *xm64, *kx64, *gradh64, *vol64;
};

__device__ __forceinline__ double pairDist(const RefArgs& a, const CoordFp64::Target& t, uint32_t j, double twoH,
                                           bool wrap)
{
    double rx, ry, rz;
    a.cf.diffFast(t, j, twoH, wrap, rx, ry, rz);
    const double r2 = dist2(rx, ry, rz);
    return r2 * invDist(r2);
}

// flag test per particle: one warp covers the 32 particles of one bitmap word, which it writes
// whole; flagged particles are appended to the list (one atomic per warp)
template<class F>
__device__ __forceinline__ void flagAndList(int64_t n, F&& test, uint32_t* __restrict__ bits,
                                            uint32_t* __restrict__ list, unsigned long long* __restrict__ count)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const bool f = i < n && test(i);
    const unsigned b = __ballot_sync(0xffffffffu, f);
    const int lane = threadIdx.x & 31;
    if (lane == 0 && (i >> 5) < (n + 31) / 32) bits[i >> 5] = b;
    unsigned long long base = 0;
    if (lane == 0 && b) base = atomicAdd(count, (unsigned long long)__popc(b));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (f) list[base + __popc(b & ((1u << lane) - 1u))] = uint32_t(i);
}

__global__ void flagGradhKernel(int64_t n, const float* __restrict__ gradh, uint32_t* __restrict__ bits,
                                uint32_t* __restrict__ list, unsigned long long* __restrict__ count)
{
    flagAndList(n, [&](int64_t i) { return fabsf(gradh[i]) < 0.1f; }, bits, list, count);
}

__global__ void flagDivvKernel(int64_t n, const float* __restrict__ divv, const float* __restrict__ bound,
                               uint32_t* __restrict__ bits, uint32_t* __restrict__ list,
                               unsigned long long* __restrict__ count)
{
    // bound 0 (no velocity differences): the sign is exact
    flagAndList(n, [&](int64_t i) { return fabsf(divv[i]) < bound[i]; }, bits, list, count);
}

// appends the not yet listed neighbours of list[from, to) at list[*count ...]; the warp's lanes walk
// their lists in step so that each step's new entries take one atomic
__global__ void __launch_bounds__(kRefBlock) dilateKernel(ListView lv, uint32_t* __restrict__ bits,
                                                          uint32_t* __restrict__ list, int64_t from, int64_t to,
                                                          unsigned long long* __restrict__ count)
{
    const int64_t t = from + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const bool valid = t < to;
    const int64_t ii = valid ? int64_t(list[t]) - lv.first : 0;
    const unsigned nc = valid ? lv.capped(ii) : 0u;
    const int lane = threadIdx.x & 31;
    for (unsigned k = 0; __any_sync(0xffffffffu, k < nc); ++k) {
        bool fresh = false;
        uint32_t j = 0;
        if (k < nc) {
            j = lv.at(ii, k);
            const uint32_t bit = 1u << (j & 31u);
            fresh = (atomicOr(bits + (j >> 5), bit) & bit) == 0u;
        }
        const unsigned b = __ballot_sync(0xffffffffu, fresh);
        if (b == 0u) continue;
        unsigned long long base = 0;
        if (lane == __ffs(b) - 1) base = atomicAdd(count, (unsigned long long)__popc(b));
        base = __shfl_sync(0xffffffffu, base, __ffs(b) - 1);
        if (fresh) list[base + __popc(b & ((1u << lane) - 1u))] = j;
    }
}

// xmassJLoop in FP64 (hydro_ve/xmass_kern.hpp:50-79) for the listed particles list[0, cnt)
__global__ void __launch_bounds__(kRefBlock) refXmassKernel(RefArgs a, int64_t cnt)
{
    const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t >= cnt) return;
    const int64_t i = a.list[t];
    const int64_t ii = i - a.lv.first;
    const unsigned nc = a.lv.capped(ii);
    auto tg = a.cf.target(i);
    const double hi = a.h[i], mi = a.m[i], hInv = 1.0 / hi, twoH = 2.0 * hi;
    const bool wrap = a.cf.needsWrap(tg, twoH);
    double rho0 = mi;
    for (unsigned k = 0; k < nc; ++k) {
        const uint32_t j = a.lv.at(ii, k);
        rho0 += lookupX(a.tw, pairDist(a, tg, j, twoH, wrap) * hInv * kTabInvDx) * double(a.m[j]);
    }
    a.xm64[i] = mi / (rho0 * a.K * (hInv * hInv * hInv));
}

// veDefGradhJLoop in FP64 (hydro_ve/ve_def_gradh_kern.hpp:43-90) on the FP64 xm of the neighbours,
// for list[0, cnt); also the particle's volume xm / kx for the IAD of the divv refinement
__global__ void __launch_bounds__(kRefBlock) refGradhKernel(RefArgs a, int64_t cnt)
{
    const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t >= cnt) return;
    const int64_t i = a.list[t];
    const int64_t ii = i - a.lv.first;
    const unsigned nc = a.lv.capped(ii);
    auto tg = a.cf.target(i);
    const double hi = a.h[i], mi = a.m[i], xmi = a.xm64[i];
    const double hInv = 1.0 / hi, h3Inv = hInv * hInv * hInv, twoH = 2.0 * hi;
    const bool wrap = a.cf.needsWrap(tg, twoH);
    double kxi = xmi, whomega = -3.0 * xmi, wrho0 = -3.0 * mi;
    for (unsigned k = 0; k < nc; ++k) {
        const uint32_t j = a.lv.at(ii, k);
        const double v = pairDist(a, tg, j, twoH, wrap) * hInv;
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
    a.vol64[i] = xmi / kxi;
}

__global__ void writeGradhKernel(RefArgs a, int64_t cnt, float* __restrict__ kx, float* __restrict__ gradh)
{
    const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t >= cnt) return;
    const int64_t i = a.list[t];
    kx[i] = float(a.kx64[i]);
    gradh[i] = float(a.gradh64[i]);
}

// IADJLoop + divV_curlVJLoop in FP64 (hydro_ve/iad_kern.hpp:43-109, divv_curlv_kern.hpp:43-123):
// divv of the flagged particles list[0, cnt) from FP64 xm, kx and volumes of their neighbours
__global__ void __launch_bounds__(kRefBlock) refDivvKernel(RefArgs a, int64_t cnt, float* __restrict__ divv)
{
    const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t >= cnt) return;
    const int64_t i = a.list[t];
    const int64_t ii = i - a.lv.first;
    const unsigned nc = a.lv.capped(ii);
    auto tg = a.cf.target(i);
    const double hi = a.h[i], hInv = 1.0 / hi, twoH = 2.0 * hi;
    const bool wrap = a.cf.needsWrap(tg, twoH);
    const double vxi = a.vx[i], vyi = a.vy[i], vzi = a.vz[i];
    double t11 = 0, t12 = 0, t13 = 0, t22 = 0, t23 = 0, t33 = 0;
    double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (unsigned k = 0; k < nc; ++k) {
        const uint32_t j = a.lv.at(ii, k);
        double rx, ry, rz;
        a.cf.diffFast(tg, j, twoH, wrap, rx, ry, rz);
        const double r2 = dist2(rx, ry, rz);
        const double w = lookupX(a.tw, r2 * invDist(r2) * hInv * kTabInvDx);
        const double vw = a.vol64[j] * w;
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

int setup(sphgb_ctx* c, const sphgb_particles* p, RefArgs& a)
{
    const int64_t n = p->n;
    const size_t words = size_t((n + 31) / 32);
    SPHGB_TRY(c->refMask.ensure(sizeof(uint32_t) * (words + size_t(n))));
    SPHGB_TRY(c->refFp64.ensure(sizeof(double) * 4 * size_t(n)));
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
    a.bits = c->refMask.as<uint32_t>();
    a.list = a.bits + words;
    a.xm64 = c->refFp64.as<double>();
    a.kx64 = a.xm64 + n;
    a.gradh64 = a.xm64 + 2 * n;
    a.vol64 = a.xm64 + 3 * n;
    return SPHGB_OK;
}

// the list length so far, read back (the cone work is skipped when nothing is flagged)
int listLength(sphgb_ctx* c, unsigned long long* dev, int64_t* out)
{
    unsigned long long h = 0;
    SPHGB_CUDA(cudaMemcpyAsync(&h, dev, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    *out = int64_t(h);
    return SPHGB_OK;
}

// appends the neighbours of list[from, to) not listed yet; returns the new length
int dilate(sphgb_ctx* c, const RefArgs& a, int64_t from, int64_t to, unsigned long long* cnt, int64_t* len)
{
    if (to > from) {
        dilateKernel<<<gridFor(to - from, kRefBlock), kRefBlock, 0, c->stream>>>(a.lv, a.bits, a.list, from, to, cnt);
        SPHGB_TRY(launched(c, "dilateKernel"));
    }
    return listLength(c, cnt, len);
}

unsigned blocksFor(int64_t n) { return gridFor(n, kRefBlock); }

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
    flagGradhKernel<<<gridFor(n, 256), 256, 0, c->stream>>>(n, static_cast<const float*>(p->gradh), a.bits, a.list,
                                                          cnt);
    SPHGB_TRY(launched(c, "flagGradhKernel"));
    int64_t flagged = 0, shell1 = 0;
    SPHGB_TRY(listLength(c, cnt, &flagged));
    c->stats_refinedGradh = flagged;
    if (flagged == 0) return SPHGB_OK;
    SPHGB_TRY(dilate(c, a, 0, flagged, cnt, &shell1));  // xm needed on list[0, shell1)
    refXmassKernel<<<blocksFor(shell1), kRefBlock, 0, c->stream>>>(a, shell1);
    SPHGB_TRY(launched(c, "refXmassKernel"));
    refGradhKernel<<<blocksFor(flagged), kRefBlock, 0, c->stream>>>(a, flagged);
    SPHGB_TRY(launched(c, "refGradhKernel"));
    writeGradhKernel<<<blocksFor(flagged), kRefBlock, 0, c->stream>>>(a, flagged, static_cast<float*>(p->kx),
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
    flagDivvKernel<<<gridFor(n, 256), 256, 0, c->stream>>>(n, static_cast<const float*>(p->divv), bound, a.bits,
                                                         a.list, cnt);
    SPHGB_TRY(launched(c, "flagDivvKernel"));
    int64_t flagged = 0, shell1 = 0, shell2 = 0;
    SPHGB_TRY(listLength(c, cnt, &flagged));
    c->stats_refinedDivv = flagged;
    if (flagged == 0) return SPHGB_OK;
    SPHGB_TRY(dilate(c, a, 0, flagged, cnt, &shell1));       // kx needed on list[0, shell1)
    SPHGB_TRY(dilate(c, a, flagged, shell1, cnt, &shell2));  // xm needed on list[0, shell2)
    refXmassKernel<<<blocksFor(shell2), kRefBlock, 0, c->stream>>>(a, shell2);
    SPHGB_TRY(launched(c, "refXmassKernel"));
    refGradhKernel<<<blocksFor(shell1), kRefBlock, 0, c->stream>>>(a, shell1);
    SPHGB_TRY(launched(c, "refGradhKernel"));
    refDivvKernel<<<blocksFor(flagged), kRefBlock, 0, c->stream>>>(a, flagged, static_cast<float*>(p->divv));
    return launched(c, "refDivvKernel");
}

}  // namespace sphgb
