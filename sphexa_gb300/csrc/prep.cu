// Per-sweep preparation shared by the pair passes: kernel tables and normalisation K, the
// mixed form's grid-local coordinates, FP64 reciprocals, and the Courant-dt reduction word.
#include <cmath>
#include <vector>
#include <algorithm>
#include <numeric>

#include "kernel_tables.hpp"
#include "pairs.cuh"

namespace sphgb {

namespace {

using tables::kernelNormalisation;
using tables::sincStd;
using tables::sincStdDeriv;

__global__ void mixedCoordsKernel(const double* __restrict__ x, const double* __restrict__ y,
                                  const double* __restrict__ z, const void* __restrict__ h, int hIsFloat, int64_t n,
                                  DevBox box, u64* __restrict__ cell, float4* __restrict__ loc)
{
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const double c[3] = {x[i], y[i], z[i]};
    unsigned ic[3];
    float l[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        // cell = floor((x - lo) / u) by a multiply: a cell off by one near a boundary only gives an
        // offset just outside [0, u), which the FP32 offset still holds to 2^-24 of u
        double u = box.L[k] / double(1 << kGridBits);
        double g = floor((c[k] - box.lo[k]) * (double(1 << kGridBits) * box.iL[k]));
        g = fmin(fmax(g, 0.0), double(kGridMask));
        ic[k] = unsigned(g);
        l[k] = float(c[k] - (box.lo[k] + g * u));
    }
    double hi = hIsFloat ? double(static_cast<const float*>(h)[i]) : static_cast<const double*>(h)[i];
    cell[i] = u64(ic[0]) | (u64(ic[1]) << kGridBits) | (u64(ic[2]) << (2 * kGridBits));
    loc[i] = make_float4(l[0], l[1], l[2], float(1.0 / hi));
}

// 1/h into the w of the grid-form offsets, whose cells and offsets the neighbour search of this sweep
// formed from the same positions.  For FP32 h, 1.0f / h (correctly rounded) equals float(1.0 / h) in
// FP64: rounding to 53 bits first is innocuous for a quotient of 24-bit operands (53 >= 2 * 24 + 2).
__global__ void gridHInvKernel(const void* __restrict__ h, int hIsFloat, int64_t n, float4* __restrict__ loc)
{
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    float4 l = loc[i];
    l.w = hIsFloat ? 1.0f / static_cast<const float*>(h)[i] : float(1.0 / static_cast<const double*>(h)[i]);
    loc[i] = l;
}

// per particle 1/h, 1/h^3 and (1/h) / dx: the last turns a pair distance into table-interval units
// with one multiply
__global__ void recipKernel(const double* __restrict__ h, int64_t n, double* __restrict__ out)
{
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    double hi = 1.0 / h[i];
    out[i] = hi;
    out[n + i] = hi * hi * hi;
    out[2 * n + i] = hi * kTabInvDx;
}

__global__ void initDtWord(unsigned long long* p) { *p = 0x7ff0000000000000ull; /* +inf */ }

}  // namespace

int buildTables(sphgb_ctx* c)
{
    const double n = c->prm.sincIndex;
    std::vector<double> wh(kTableSize), whd(kTableSize);
    std::vector<float> wf(kTableSize);
    // tabulateFunction on [0, 2] (sph/include/sph/sph_kernel_tables.hpp:81-95)
    const double dx = (2.0 - 0.0) / (kTableSize - 1);
    for (int i = 0; i < kTableSize; ++i) {
        double v = 0.0 + i * dx;
        wh[i] = std::pow(sincStd(v), n);
        whd[i] = n * std::pow(sincStd(v), n - 1) * sincStdDeriv(v);
        wf[i] = float(wh[i]);
    }
    c->K = kernelNormalisation(n);
    // lookups read {t[k], t[k+1] - t[k]} in one load; the difference is the one the reference
    // interpolant forms (sph/include/sph/table_lookup.hpp:23)
    std::vector<double> wx(2 * kTableSize), wdx(2 * kTableSize);
    for (int i = 0; i < kTableSize; ++i) {
        const bool last = i + 1 == kTableSize;
        wx[2 * i] = wh[i];
        wx[2 * i + 1] = last ? 0.0 : wh[i + 1] - wh[i];
        wdx[2 * i] = whd[i];
        wdx[2 * i + 1] = last ? 0.0 : whd[i + 1] - whd[i];
    }
    // FP32 copy of the linear table for the mixed adjoint, which differentiates the interpolant of
    // the FP64 passes
    std::vector<float> wx32(2 * kTableSize);
    for (int i = 0; i < kTableSize; ++i) {
        const bool last = i + 1 == kTableSize;
        wx32[2 * i] = wf[i];
        wx32[2 * i + 1] = last ? 0.f : wf[i + 1] - wf[i];
    }
    SPHGB_TRY(c->whx32.ensure(sizeof(float) * 2 * kTableSize));
    SPHGB_CUDA(cudaMemcpy(c->whx32.p, wx32.data(), sizeof(float) * 2 * kTableSize, cudaMemcpyHostToDevice));
    {  // the mixed passes' cubic pieces of W and dW/dv
        std::vector<float> hw, hd;
        tables::hermitePieces(n, kHermIntervals, hw, hd);
        SPHGB_TRY(c->whH32.ensure(sizeof(float) * hw.size()));
        SPHGB_TRY(c->whdH32.ensure(sizeof(float) * hd.size()));
        SPHGB_CUDA(cudaMemcpy(c->whH32.p, hw.data(), sizeof(float) * hw.size(), cudaMemcpyHostToDevice));
        SPHGB_CUDA(cudaMemcpy(c->whdH32.p, hd.data(), sizeof(float) * hd.size(), cudaMemcpyHostToDevice));
    }
    {  // smooth form of the FP64 kernel function: cubic pieces on the linear table's intervals
        std::vector<double> sw, sd;
        tables::hermitePieces(n, kTableSize - 1, sw, sd);
        SPHGB_TRY(c->whS64.ensure(sizeof(double) * sw.size()));
        SPHGB_TRY(c->whdS64.ensure(sizeof(double) * sd.size()));
        SPHGB_CUDA(cudaMemcpy(c->whS64.p, sw.data(), sizeof(double) * sw.size(), cudaMemcpyHostToDevice));
        SPHGB_CUDA(cudaMemcpy(c->whdS64.p, sd.data(), sizeof(double) * sd.size(), cudaMemcpyHostToDevice));
    }
    SPHGB_TRY(c->whx64.ensure(sizeof(double) * 2 * kTableSize));
    SPHGB_TRY(c->whdx64.ensure(sizeof(double) * 2 * kTableSize));
    SPHGB_CUDA(cudaMemcpy(c->whx64.p, wx.data(), sizeof(double) * 2 * kTableSize, cudaMemcpyHostToDevice));
    SPHGB_CUDA(cudaMemcpy(c->whdx64.p, wdx.data(), sizeof(double) * 2 * kTableSize, cudaMemcpyHostToDevice));
    c->tablesReady = true;
    return SPHGB_OK;
}

int prepareMixed(sphgb_ctx* c, sphgb_particles* p, int64_t, int64_t)
{
    const int64_t n = p->n;
    if (c->inSweep && c->xBuilt == p->x && c->gridKey.bytes >= sizeof(u64) * n && c->gridLoc.bytes >= sizeof(float4) * n) {
        // the search of this sweep formed the grid form from these positions; only 1/h is missing
        gridHInvKernel<<<gridFor(n, 256), 256, 0, c->stream>>>(p->h, p->precision == SPHGB_MIXED, n,
                                                              c->gridLoc.as<float4>());
        return launched(c, "gridHInvKernel");
    }
    SPHGB_TRY(c->gridKey.ensure(sizeof(u64) * n));
    SPHGB_TRY(c->gridLoc.ensure(sizeof(float4) * n));
    mixedCoordsKernel<<<gridFor(n, 256), 256, 0, c->stream>>>(p->x, p->y, p->z, p->h, p->precision == SPHGB_MIXED, n,
                                                             c->box, c->gridKey.as<u64>(), c->gridLoc.as<float4>());
    return launched(c, "mixedCoordsKernel");
}

int prepareFp64(sphgb_ctx* c, sphgb_particles* p)
{
    const int64_t n = p->n;
    SPHGB_TRY(c->hInv64.ensure(sizeof(double) * 3 * n));
    recipKernel<<<gridFor(n, 256), 256, 0, c->stream>>>(static_cast<const double*>(p->h), n, c->hInv64.as<double>());
    return launched(c, "recipKernel");
}

// preconditions of every pair pass; rebuilds the per-particle precomputes from the current x y z
// h on every call (one elementwise kernel): a caller may change positions or smoothing lengths
// between passes while the neighbour lists stay frozen, as gradient checks do
int checkPass(sphgb_ctx* c, const sphgb_particles* p, int64_t first, int64_t last)
{
    if (!c->haveNbr || !c->tablesReady) return SPHGB_ERR_STATE;
    if (!p || !p->x || !p->y || !p->z || !p->h) return SPHGB_ERR_ARG;
    if (first < c->nbrFirst || last > c->nbrLast || first >= last || p->n < last) return SPHGB_ERR_ARG;
    if (p->precision != SPHGB_FP64 && p->precision != SPHGB_MIXED) return SPHGB_ERR_ARG;
    sphgb_particles* q = const_cast<sphgb_particles*>(p);
    // inside one sweep positions and h stay put after the neighbour search: prepare once
    if (c->sweepPrepared) return SPHGB_OK;
    const int s = p->precision == SPHGB_MIXED ? prepareMixed(c, q, first, last) : prepareFp64(c, q);
    if (s == SPHGB_OK && c->inSweep) c->sweepPrepared = true;
    return s;
}

int beginDtReduction(sphgb_ctx* c, unsigned long long** dst)
{
    SPHGB_TRY(c->reduceScratch.ensure(sizeof(unsigned long long) * 4));
    *dst = c->reduceScratch.as<unsigned long long>();
    initDtWord<<<1, 1, 0, c->stream>>>(*dst);
    return launched(c, "initDtWord");
}

int endDtReduction(sphgb_ctx* c, unsigned long long* dst, double* out)
{
    if (!out) return SPHGB_OK;
    unsigned long long bits = 0;
    SPHGB_CUDA(cudaMemcpyAsync(&bits, dst, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    double v;
    std::memcpy(&v, &bits, sizeof(v));
    *out = v;
    return SPHGB_OK;
}

}  // namespace sphgb
