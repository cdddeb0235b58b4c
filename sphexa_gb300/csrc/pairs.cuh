// Pair-loop building blocks shared by the std and VE passes.
//
// One thread per target particle i walks its own neighbour list; a warp holds 32 SFC-consecutive
// targets, so entry k of the warp's 32 lists is one coalesced read (512 contiguous bytes shared by
// four consecutive k) and the neighbours of a warp overlap heavily in L1.
//
// Two arithmetic forms:
//   Fp64  : every operation in double, in the reference's order (the plain drop-in);
//   Mixed : FP32 pair arithmetic.  A coordinate difference is formed from the 21-bit grid cells
//           of both particles (exact integer difference, periodic wrap in integers) plus the
//           difference of their FP32 offsets inside the cell: rx = di * u + (xl_i - xl_j), one
//           rounding.  Sums that the error budget needs are Kahan-compensated.
#pragma once

#include <type_traits>

#include "context.cuh"

namespace sphgb {

struct Fp64Tag {
    using T = double;
};
struct MixedTag {
    using T = float;
};

constexpr int kPairBlock = 128;

// ---- neighbour list layout ----
// Lists are stored in granules of kListGran entries, transposed per granule: entries 4g .. 4g+3 of
// the list of target ii = i - first occupy the 16 contiguous bytes of granule (g * stride + ii).
// The search writes a granule with one 16-byte store instead of four scattered 4-byte stores, and a
// warp of 32 consecutive targets reads entry k of its lists from 512 contiguous bytes that also hold
// entries k+1 .. of the same granule row.  The owned lists of the pair-once passes use the same layout.
constexpr unsigned kListGran = 4;

__host__ __device__ __forceinline__ int64_t listSlot(int64_t ii, unsigned k, int64_t stride)
{
    return (int64_t(k / kListGran) * stride + ii) * kListGran + (k % kListGran);
}

// entries per target that the buffers reserve for a capacity of ngmax (whole granules)
inline size_t listCapacity(uint32_t ngmax) { return (size_t(ngmax) + kListGran - 1) / kListGran * kListGran; }

// writes one target's list in order: entries collect in registers, every fourth one stores the
// granule; finish() stores the last, partial granule.  Granules at or beyond the capacity are not
// written (entries past ngmax of a capped list are dropped, as the reference drops them).
struct GranuleWriter {
    uint4* out;  // granule 0 of this target; granule g at out[g * stride]
    int64_t stride;
    unsigned capG;
    uint32_t b0 = 0, b1 = 0, b2 = 0;
    __device__ __forceinline__ GranuleWriter(uint32_t* base, int64_t ii, int64_t stride_, uint32_t ngmax)
        : out(reinterpret_cast<uint4*>(base) + ii), stride(stride_), capG((ngmax + kListGran - 1) / kListGran)
    {
    }
    __device__ __forceinline__ void put(unsigned cnt, uint32_t j)
    {
        const unsigned s = cnt % kListGran, g = cnt / kListGran;
        b0 = s == 0 ? j : b0;
        b1 = s == 1 ? j : b1;
        b2 = s == 2 ? j : b2;
        if (s == kListGran - 1 && g < capG) out[int64_t(g) * stride] = make_uint4(b0, b1, b2, j);
    }
    __device__ __forceinline__ void finish(unsigned cnt)
    {
        const unsigned g = cnt / kListGran;
        if (cnt % kListGran != 0 && g < capG) out[int64_t(g) * stride] = make_uint4(b0, b1, b2, 0u);
    }
};

struct ListView {
    const uint32_t* nbr;
    const uint32_t* count;
    int64_t stride, first, last;
    uint32_t ngmax;
    __device__ __forceinline__ unsigned capped(int64_t ii) const { return min(count[ii], ngmax); }
    __device__ __forceinline__ uint32_t at(int64_t ii, unsigned k) const { return __ldg(nbr + listSlot(ii, k, stride)); }
    // granule g of target ii: entries 4g .. 4g+3
    __device__ __forceinline__ uint4 granule(int64_t ii, unsigned g) const
    {
        return __ldg(reinterpret_cast<const uint4*>(nbr) + (int64_t(g) * stride + ii));
    }
};
// entry s of a granule
__device__ __forceinline__ uint32_t pick(uint4 g, unsigned s) { return s == 0 ? g.x : s == 1 ? g.y : s == 2 ? g.z : g.w; }

inline ListView listView(const sphgb_ctx* c)
{
    return ListView{c->nbr.as<uint32_t>(), c->ncount.as<uint32_t>(), c->nbrStride, c->nbrFirst, c->nbrLast,
                    c->nbrNgmax};
}

// ---- owned lists: the pairs particle i evaluates in the pair-once FP64 passes ----
// entry k < count[i - first] of i's owned list (granule layout) = j | mutual << 31: every pair of i's list
// that j does not list back, and half of the mutual pairs (the other half sits in the owned lists
// of the other ends).  A mutual pair's evaluation also produces j's terms, added with FP64 atomics.
struct OwnedView {
    const uint32_t* owned;
    const uint32_t* count;
    int64_t stride;
    __device__ __forceinline__ unsigned size(int64_t ii) const { return __ldg(count + ii); }
    __device__ __forceinline__ uint32_t at(int64_t ii, unsigned k, bool& mutual) const
    {
        const uint32_t e = __ldg(owned + listSlot(ii, k, stride));
        mutual = (e >> 31) != 0;
        return e & 0x7fffffffu;
    }
};

inline OwnedView ownedView(const sphgb_ctx* c)
{
    return OwnedView{c->owned.as<uint32_t>(), c->ownedCount.as<uint32_t>(), c->nbrStride};
}

// a pass over [first, last) may evaluate pairs once: FP64 fields, order-free summation allowed,
// owned lists of the current neighbour lists, and lists covering every particle
inline bool pairOnce(const sphgb_ctx* c, const sphgb_particles* p, int64_t first, int64_t last)
{
    return !c->deterministic && p->precision == SPHGB_FP64 && c->ownedEpoch == c->nbrEpoch && !c->ownedFromLists &&
           first == 0 &&
           last == p->n && c->nbrFirst == 0 && c->nbrLast == p->n;
}

// ---- pair geometry shared by the pair-once passes of one sweep ----
// Inside one sweep positions, velocities and h stay put, so an owned entry's |r| and 1/|r| (the FP64
// difference, its square and the reciprocal square root: about a dozen FP64-pipe instructions), the
// kernel function at both ends, w(|r| / h_i) and w(|r| / h_j), and, where the memory is there, the
// difference vector r = x_i - x_j and the velocity difference dv = v_j - v_i are formed once by the
// xmass pass and loaded by gradh, IAD, AV and momentum-energy.  Layout: the 32 targets of a warp own
// rows rowOff[w] .. rowOff[w] + (their longest owned list) - 1, a row holding entry k of all 32 side
// by side, so a warp reads 512 contiguous bytes per entry and array.
struct PairGeo {
    const uint32_t* rowOff;  // first row of each warp of 32 targets
    double2* g;              // {|r|, 1/|r|}; null: the pass forms the geometry itself
    double2* w;              // {w(|r| / h_i), w(|r| / h_j)}
    double2* x;              // {rx, ry}, {rz, dvx}, {dvy, dvz} at x, x + plane, x + 2 plane; or null
    int64_t plane;           // entries per array
    // entry k of target ii is at base(ii) + 32 k
    __device__ __forceinline__ int64_t base(int64_t ii) const
    {
        return g ? int64_t(__ldg(rowOff + (ii >> 5))) * 32 + (ii & 31) : 0;
    }
};

// the space for the xmass pass of this sweep to fill (rows from the owned counts; null outside a
// sweep or when it cannot be had within half of the free device memory)
int pairGeoStore(sphgb_ctx* c, PairGeo* out);

// what this sweep's xmass pass stored, or null
inline PairGeo pairGeoRead(const sphgb_ctx* c)
{
    if (!c->inSweep || !c->geoValid) return PairGeo{nullptr, nullptr, nullptr, nullptr, 0};
    double2* g = c->pairGeo.as<double2>();
    const int64_t nWarps = (c->nbrLast - c->nbrFirst + 31) / 32, plane = 32 * int64_t(c->geoRowCount);
    return PairGeo{c->geoRows.as<uint32_t>() + nWarps, g, g + plane, c->geoArrays == 5 ? g + 2 * plane : nullptr, plane};
}

// ---- forward tape of the VE adjoint: sections of n doubles in c->veTape ----
constexpr int kTapeG = 0;      // G_i = -K h_i^-3 C_i S_i of the AV switch (3 sections)
constexpr int kTapeP = 3;      // P_i = sum xm_j W_ij (v_j - v_i) r_ij^T of divv/curlv, row-major (9)
constexpr int kTapeWom = 12;   // K h_i^-4 (-3 xm_i + sum xm_j dterh_ij) of gradh
constexpr int kTapeWr0 = 13;   // K h_i^-4 (-3 m_i + sum m_j dterh_ij)
constexpr int kTapeEn = 14;    // energy sum of the momentum-energy pass
constexpr int kTapeAvE = 15;   // viscous energy sum before max(0, .)
constexpr int kTapeSections = 16;
enum : unsigned { kTapeGradh = 1, kTapeIad = 2, kTapeAv = 4, kTapeMe = 8 };

// the tape of an FP64 VE pass over all particles (null when the tape is off or the pass covers
// part of the particles); marks the pass's part as written on the current lists
inline int tapeFor(sphgb_ctx* c, const sphgb_particles* p, int64_t first, int64_t last, unsigned part,
                   double** out)
{
    *out = nullptr;
    if (!c->tapeOn || p->precision != SPHGB_FP64 || first != 0 || last != p->n) return SPHGB_OK;
    const int64_t n = p->n;
    if (c->tapeEpoch != c->nbrEpoch || c->tapeN != n) {
        c->tapeMask = 0;
        c->tapeEpoch = c->nbrEpoch;
        c->tapeN = n;
    }
    SPHGB_TRY(c->veTape.ensure(sizeof(double) * kTapeSections * size_t(n)));
    c->tapeMask |= part;
    *out = c->veTape.as<double>();
    return SPHGB_OK;
}

// ---- FP64 coordinates: reference distancePBC / legacy applyPBC (box.hpp:216-254) ----
struct CoordFp64 {
    const double *x, *y, *z;
    double L[3], lo[3], hi[3];
    int pbc[3];
    struct Target {
        double x, y, z;
    };
    __device__ __forceinline__ Target target(int64_t i) const { return {x[i], y[i], z[i]}; }
    // true when the 2h box of the target crosses a periodic face; otherwise no neighbour can be a
    // periodic image (|rx| < 2h < L/2) and the wrap tests of applyPBC never fire
    __device__ __forceinline__ bool needsWrap(const Target& t, double twoH) const
    {
        return (pbc[0] && (t.x - twoH < lo[0] || t.x + twoH > hi[0])) ||
               (pbc[1] && (t.y - twoH < lo[1] || t.y + twoH > hi[1])) ||
               (pbc[2] && (t.z - twoH < lo[2] || t.z + twoH > hi[2]));
    }
    // legacy applyPBC with threshold 2h_i; the comparisons |r| > 2h run on the bit patterns
    // (integer pipe): for twoH > 0, r > twoH <=> bits(r) > bits(twoH) and r < -twoH <=>
    // bits(-r) > bits(twoH), negative values having negative signed patterns
    __device__ __forceinline__ static double wrapLegacy(double r, long long twoHBits, double L)
    {
        const long long b = __double_as_longlong(r);
        if (b > twoHBits) return r - L;
        if ((b ^ (1LL << 63)) > twoHBits) return r + L;
        return r;
    }
    __device__ __forceinline__ void diff(const Target& t, int64_t j, double twoH, double& rx, double& ry,
                                         double& rz) const
    {
        rx = t.x - x[j];
        ry = t.y - y[j];
        rz = t.z - z[j];
        const long long hb = __double_as_longlong(twoH);
        if (pbc[0]) rx = wrapLegacy(rx, hb, L[0]);
        if (pbc[1]) ry = wrapLegacy(ry, hb, L[1]);
        if (pbc[2]) rz = wrapLegacy(rz, hb, L[2]);
    }
    // legacy applyPBC only where it can change the result
    __device__ __forceinline__ void diffFast(const Target& t, int64_t j, double twoH, bool wrap, double& rx,
                                             double& ry, double& rz) const
    {
        if (wrap) diff(t, j, twoH, rx, ry, rz);
        else {
            rx = t.x - x[j];
            ry = t.y - y[j];
            rz = t.z - z[j];
        }
    }
};

inline CoordFp64 coordFp64(const sphgb_ctx* c, const sphgb_particles* p)
{
    CoordFp64 r;
    r.x = p->x;
    r.y = p->y;
    r.z = p->z;
    for (int k = 0; k < 3; ++k) {
        r.L[k] = c->box.L[k];
        r.lo[k] = c->box.lo[k];
        r.hi[k] = c->box.hi[k];
        r.pbc[k] = c->box.pbc[k];
    }
    return r;
}

// 1/sqrt(r2) and sqrt(r2) in FP64 through the reciprocal square root: one special-function
// seed plus FMA refinement instead of an IEEE sqrt and an IEEE divide
__device__ __forceinline__ double invDist(double r2) { return rsqrt(r2); }

// |r|^2 in one fixed order of FMAs: every FP64 pass, the order-fixed and the pair-once forms and the
// per-sweep geometry cache form the same bits for a pair, so their Courant time steps agree exactly
template<class T>
__device__ __forceinline__ T dist2(T x, T y, T z)
{
    return fma(z, z, fma(y, y, x * x));
}

// ---- FP64 pair-loop arithmetic kept off the FP64 pipe ----
// On GB300 the SM's FP64 pipe retires 2 lanes per cycle: one warp-wide FP64 instruction holds it
// for 16 cycles, in which the integer and FP32 pipes issue dozens of instructions.  The FP64
// passes therefore do comparisons, table indexing and interval offsets on bit patterns.

// x < 0 (false for -0.0, as the FP64 comparison) from the bit pattern
__device__ __forceinline__ bool negative(double x)
{
    const long long b = __double_as_longlong(x);
    return b < 0 && (b << 1) != 0;
}

// max(a, b) for b >= 0 (or +-0): bit patterns of non-negative doubles order like their values and
// negative values have negative signed patterns
__device__ __forceinline__ long long maxBitsNonNeg(long long bBits, double a)
{
    return max(bBits, __double_as_longlong(a));
}

// a < b for a, b >= 0
__device__ __forceinline__ bool lessNonNeg(double a, double b)
{
    return __double_as_longlong(a) < __double_as_longlong(b);
}

// 1 / table spacing, formed as the reference forms it (sph/include/sph/table_lookup.hpp:17-19)
constexpr double kTabInvDx = 1.0 / (2.0 / double(kTableSize - 1));

// Interval of the kernel table for x = v / dx >= 0: k = floor(x) and x - k, taken from the bits
// of x with integer operations (k < 0 marks x beyond the last interval, where the table reads 0).
struct TabSlot {
    int k;
    double frac;
};

__device__ __forceinline__ TabSlot tabSlot(double x)
{
    constexpr int nInt = kTableSize - 1;
    const long long b = __double_as_longlong(x);
    const int e = int(b >> 52) - 1023;
    if (e < 0) return {0, x};    // x < 1
    if (e > 14) return {-1, 0.0};  // x >= 2^15 > nInt
    const long long m = (b & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
    const int sh = 52 - e;
    const int k = int(m >> sh);
    if (k >= nInt) return {-1, 0.0};
    const long long fm = m & ((1LL << sh) - 1);  // (x - k) * 2^sh, exact
    double frac = 0.0;
    if (fm != 0) {
        const int lz = __clzll(fm) - 11;  // moves the leading bit of fm to bit 52
        frac = __longlong_as_double((static_cast<long long>(1075 - sh - lz) << 52) |
                                    ((fm << lz) & 0xFFFFFFFFFFFFFLL));
    }
    return {k, frac};
}

// tabX[k] = {t[k], t[k+1] - t[k]}: W = t[k] + (t[k+1] - t[k]) (x - k), the reference's linear
// interpolant (table_lookup.hpp:14-25) up to the rounding of its last two operations
__device__ __forceinline__ double lookupX(const double2* __restrict__ tabX, const TabSlot& s)
{
    if (s.k < 0) return 0.0;
    const double2 t = __ldg(tabX + s.k);
    return fma(t.y, s.frac, t.x);
}

__device__ __forceinline__ double lookupX(const double2* __restrict__ tabX, double x)
{
    return lookupX(tabX, tabSlot(x));
}

// ---- the FP64 passes' kernel function, W or dW/dv, in one of two forms ----
// table (default): the reference's linear interpolant, t[k] = {t[k], t[k+1] - t[k]};
// smooth (sphgb_set_kernel_form): a cubic Hermite piece on each of the same 19999 intervals, through
//   the closed-form values and derivatives at both nodes, t[2k] = {c0, c1}, t[2k+1] = {c2, c3} of
//   c0 + f (c1 + f (c2 + f c3)), f = x - k.  The function is then continuously differentiable, so
//   central differences of the forward passes agree with the adjoint (which differentiates the same
//   pieces); it differs from the table form by the table's interpolation error (within 2e-8 of the
//   function's maximum).
// The form is a template argument of the kernels (withKernelForm picks the instantiation at launch):
// a run-time test inside the lookup cost the FP64-bound passes 5-35 % of their time.
template<bool Smooth>
struct KTab {
    const double2* t;
};

template<bool Smooth>
__device__ __forceinline__ double lookupX(const KTab<Smooth>& tb, const TabSlot& s)
{
    if (s.k < 0) return 0.0;
    if constexpr (Smooth) {
        const double2 a = __ldg(tb.t + 2 * s.k), b = __ldg(tb.t + 2 * s.k + 1);
        return fma(fma(fma(b.y, s.frac, b.x), s.frac, a.y), s.frac, a.x);
    } else {
        const double2 t = __ldg(tb.t + s.k);
        return fma(t.y, s.frac, t.x);
    }
}

template<bool Smooth>
__device__ __forceinline__ double lookupX(const KTab<Smooth>& tb, double x)
{
    return lookupX(tb, tabSlot(x));
}

// value at v and its derivative d/dv (the slope of the interval in the table form)
template<bool Smooth>
__device__ __forceinline__ double lookupVSlope(const KTab<Smooth>& tb, double v, double& slope)
{
    const TabSlot s = tabSlot(v * kTabInvDx);
    if (s.k < 0) {
        slope = 0.0;
        return 0.0;
    }
    if constexpr (Smooth) {
        const double2 a = __ldg(tb.t + 2 * s.k), b = __ldg(tb.t + 2 * s.k + 1);
        const double f = s.frac;
        slope = fma(fma(3.0 * b.y, f, 2.0 * b.x), f, a.y) * kTabInvDx;
        return fma(fma(fma(b.y, f, b.x), f, a.y), f, a.x);
    } else {
        const double2 t = __ldg(tb.t + s.k);
        slope = t.y * kTabInvDx;
        return fma(t.y, s.frac, t.x);
    }
}

// the context's FP64 tables of W and dW/dv in its kernel form
inline const double2* tabW64(const sphgb_ctx* c)
{
    return c->smoothKernel ? c->whS64.as<double2>() : c->whx64.as<double2>();
}
inline const double2* tabDW64(const sphgb_ctx* c)
{
    return c->smoothKernel ? c->whdS64.as<double2>() : c->whdx64.as<double2>();
}

// calls launch(std::integral_constant<bool, smooth>) for the context's kernel form
template<class F>
inline int withKernelForm(const sphgb_ctx* c, F&& launch)
{
    if (c->smoothKernel) return launch(std::true_type{});
    return launch(std::false_type{});
}

// ---- the mixed passes' kernel function: a cubic Hermite piece per interval of [0, 2] ----
// The pieces interpolate W and dW/dv at kHermIntervals + 1 nodes with their derivatives (error
// ~1e-11, below FP32 rounding), so the FP32 result is the kernel function itself, within 1e-8 of
// the reference's linear interpolant on its 20000-entry table; the 8 KB tables stay in L1.
constexpr int kHermIntervals = 512;

__device__ __forceinline__ float hermEval(float4 c, float t) { return fmaf(fmaf(fmaf(c.w, t, c.z), t, c.y), t, c.x); }

__device__ __forceinline__ float lookupH32(const float4* __restrict__ tab, float v)
{
    const float x = v * (0.5f * kHermIntervals);
    const int k = int(x);
    if (k >= kHermIntervals) return 0.f;  // v >= 2
    return hermEval(__ldg(tab + k), x - float(k));
}

// ---- 32-byte neighbour records, one 256-bit load each ----
// A warp's gather of 16-byte records touches about one L1 sector per lane and record; packing a
// neighbour's fields into 32-byte blocks halves the sector accesses per pair.
struct alignas(32) Rec8 {
    float v[8];
};

__device__ __forceinline__ Rec8 ldRec8(const Rec8* p)
{
    Rec8 r;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r.v[0]), "=f"(r.v[1]), "=f"(r.v[2]), "=f"(r.v[3]), "=f"(r.v[4]), "=f"(r.v[5]), "=f"(r.v[6]),
          "=f"(r.v[7])
        : "l"(p));
    return r;
}

// A neighbour block that starts with the grid position: v[0], v[1] the packed 21-bit cells (low,
// high word), v[2..4] the FP32 offset inside the cell; v[5..7] belong to the pass.
__device__ __forceinline__ void packGridBlock(float4* q, u64 cell, float4 loc, float f5, float f6, float f7)
{
    q[0] = make_float4(__uint_as_float(unsigned(cell)), __uint_as_float(unsigned(cell >> 32)), loc.x, loc.y);
    q[1] = make_float4(loc.z, f5, f6, f7);
}

// W and dW/dv at the same v
__device__ __forceinline__ void lookupH32Pair(const float4* __restrict__ tw, const float4* __restrict__ tdw, float v,
                                              float& w, float& dw)
{
    const float x = v * (0.5f * kHermIntervals);
    const int k = int(x);
    if (k >= kHermIntervals) {
        w = dw = 0.f;
        return;
    }
    const float t = x - float(k);
    w = hermEval(__ldg(tw + k), t);
    dw = hermEval(__ldg(tdw + k), t);
}


// ---- Mixed coordinates: 21-bit grid cell per axis packed in 64 bits + FP32 in-cell offset ----
constexpr int kGridBits = 21;
constexpr int kGridMask = (1 << kGridBits) - 1;

struct CoordMixed {
    const u64* cell;     // ix | iy << 21 | iz << 42
    const float4* loc;   // {xl, yl, zl, 1/h}
    float u[3];          // cell edge per axis (box length / 2^21)
    int pbc[3];
    int sh[3];           // 32 - 21 on periodic axes, 0 on open ones (wrapShift)
    struct Target {
        int ix, iy, iz;
        float xl, yl, zl, hInv;
    };
    __device__ __forceinline__ Target target(int64_t i) const
    {
        u64 k = cell[i];
        float4 l = loc[i];
        return {int(k & kGridMask), int((k >> kGridBits) & kGridMask), int(k >> (2 * kGridBits)), l.x, l.y, l.z, l.w};
    }
    __device__ __forceinline__ static int wrap(int d, int on)
    {
        constexpr int R = 1 << kGridBits;
        if (on) {
            d = d > R / 2 ? d - R : d;
            d = d < -R / 2 ? d + R : d;
        }
        return d;
    }
    // returns 1/h_j through hjInv
    __device__ __forceinline__ void diff(const Target& t, int64_t j, float& rx, float& ry, float& rz,
                                         float& hjInv) const
    {
        u64 k = __ldg(cell + j);
        float4 l = __ldg(loc + j);
        int dx = wrap(t.ix - int(k & kGridMask), pbc[0]);
        int dy = wrap(t.iy - int((k >> kGridBits) & kGridMask), pbc[1]);
        int dz = wrap(t.iz - int(k >> (2 * kGridBits)), pbc[2]);
        rx = fmaf(float(dx), u[0], t.xl - l.x);
        ry = fmaf(float(dy), u[1], t.yl - l.y);
        rz = fmaf(float(dz), u[2], t.zl - l.z);
        hjInv = l.w;
    }
    // minimum image of a cell difference d in (-2^21, 2^21) by sign extension from bit 20 (s =
    // 11): d itself when |d| < 2^20, d -/+ 2^21 beyond; s = 0 leaves d unchanged.  The same
    // image as wrap() except at exactly half the box, where both images are equally near.
    __device__ __forceinline__ static int wrapShift(int d, int s) { return int(unsigned(d) << s) >> s; }
    // the same difference from a neighbour block written by packGridBlock
    __device__ __forceinline__ void diffBlock(const Target& t, const Rec8& b, float& rx, float& ry, float& rz) const
    {
        const u64 k = u64(__float_as_uint(b.v[0])) | (u64(__float_as_uint(b.v[1])) << 32);
        int dx = wrapShift(t.ix - int(k & kGridMask), sh[0]);
        int dy = wrapShift(t.iy - int((k >> kGridBits) & kGridMask), sh[1]);
        int dz = wrapShift(t.iz - int(k >> (2 * kGridBits)), sh[2]);
        rx = fmaf(float(dx), u[0], t.xl - b.v[2]);
        ry = fmaf(float(dy), u[1], t.yl - b.v[3]);
        rz = fmaf(float(dz), u[2], t.zl - b.v[4]);
    }
};

inline CoordMixed coordMixed(const sphgb_ctx* c)
{
    CoordMixed r;
    r.cell = c->gridKey.as<u64>();
    r.loc = c->gridLoc.as<float4>();
    for (int k = 0; k < 3; ++k) {
        r.u[k] = float(c->box.L[k] / double(1 << kGridBits));
        r.pbc[k] = c->box.pbc[k];
        r.sh[k] = c->box.pbc[k] ? 32 - kGridBits : 0;
    }
    return r;
}

// ---- Kahan-compensated FP32 accumulator ----
struct KSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v)
    {
        float y = v - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s - c; }
    __device__ __forceinline__ double value64() const { return double(s) - double(c); }
};

// ---- helpers ----
template<class T>
__device__ __forceinline__ T ld(const void* p, int64_t i)
{
    return __ldg(static_cast<const T*>(p) + i);
}

template<class T>
__device__ __forceinline__ void st(void* p, int64_t i, T v)
{
    static_cast<T*>(p)[i] = v;
}

// reference artificial_viscosity (sph/include/sph/kernels.hpp:70-84)
template<class T>
__device__ __forceinline__ T artificialViscosity(T ai, T aj, T ci, T cj, T w)
{
    T v = T(0);
    bool approaching;
    if constexpr (std::is_same_v<T, double>) approaching = negative(w);
    else approaching = w < T(0);
    if (approaching) {
        T sig = (ai + aj) / T(4.0) * (ci + cj) - T(2.0) * w;
        v = -sig * w;
    }
    return v;
}

// reference tsKCourant (kernels.hpp:10-16); Kcour travels as float
__device__ __forceinline__ double courantDt(double vsig, double h, double c, float kc)
{
    double v = vsig > 0.0 ? vsig : c;
    return double(kc) * h / v;
}

// block-wide min of positive doubles into one device word (bit patterns of positive doubles are
// ordered like their values)
__device__ __forceinline__ void blockMinDt(double v, unsigned long long* out)
{
    __shared__ unsigned long long s[kPairBlock / kWarp];
    unsigned long long b = __double_as_longlong(v);
    for (int o = 16; o > 0; o >>= 1) b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
    if ((threadIdx.x & 31) == 0) s[threadIdx.x / 32] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = s[0];
        for (int q = 1; q < kPairBlock / kWarp; ++q) m = min(m, s[q]);
        atomicMin(out, m);
    }
}

// normalise tau by 2^-(mean exponent), invert, scale by h^3 / K (hydro_std/iad_kern.hpp:52-76)
template<class T>
__device__ __forceinline__ void iadInvert(T t11, T t12, T t13, T t22, T t23, T t33, double hi, double K, T* cOut)
{
    auto ex = [](T v) { return v == T(0) ? 0 : ilogb(v); };
    int es = ex(t11) + ex(t12) + ex(t13) + ex(t22) + ex(t23) + ex(t33);
    T nrm = ldexp(T(1), -es / 6);
    t11 *= nrm;
    t12 *= nrm;
    t13 *= nrm;
    t22 *= nrm;
    t23 *= nrm;
    t33 *= nrm;
    T det = t11 * t22 * t33 + T(2) * t12 * t23 * t13 - t11 * t23 * t23 - t22 * t13 * t13 - t33 * t12 * t12;
    // factor = normalization * h^3 / (det * K); the reference forms it with K in FP64
    double fac = double(nrm) * (hi * hi * hi) / (double(det) * K);
    T f = T(fac);
    cOut[0] = (t22 * t33 - t23 * t23) * f;
    cOut[1] = (t13 * t23 - t33 * t12) * f;
    cOut[2] = (t12 * t23 - t22 * t13) * f;
    cOut[3] = (t11 * t33 - t13 * t13) * f;
    cOut[4] = (t13 * t12 - t11 * t23) * f;
    cOut[5] = (t11 * t22 - t12 * t12) * f;
}

// per-pass launch helpers implemented in prep.cu
int beginDtReduction(sphgb_ctx* c, unsigned long long** dst);
int endDtReduction(sphgb_ctx* c, unsigned long long* dst, double* out);
int checkPass(sphgb_ctx* c, const sphgb_particles* p, int64_t first, int64_t last);

}  // namespace sphgb
