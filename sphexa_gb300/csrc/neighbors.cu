// Neighbour lists per warp-group of 32 SFC-consecutive target particles.
//
// Replaces cstone::findNeighbors / sph::findNeighborsSph (domain/include/cstone/findneighbors.hpp:
// 77-170, sph/include/sph/find_neighbors.hpp:10-56) and the reference GPU's per-pass warp
// traversal (domain/include/cstone/traversal/find_neighbors.cuh:182-489).  The set of neighbours
// of i is exactly the reference CPU set {j != i : d2(i,j) < 4 h_i^2}, with d2 rounded as in
// distanceSq (minimum image by rint when the 2h box of i leaves a periodic box).
//
// Per warp: one depth-first walk of the octree in SFC order against the group's search box, so
// candidate ranges arrive in ascending particle order and every list comes out sorted.  Leaves,
// internal nodes whose box lies inside the search box and internal nodes of few particles each
// give one contiguous particle range (per-node ranges precomputed with the tree); contiguous
// ranges are merged and staged 32 candidates at a time in shared memory.
// Positions are read in the grid form of the mixed passes: a 21-bit cell per axis plus an FP32
// offset inside the cell.  Offsets from the group origin are (cell difference, wrapped exactly
// in integers) x cell edge + (offset difference), so neither staging nor the distance filter
// runs an FP64 instruction.  Only pairs whose FP32 distance lies within a rounding margin of the
// radius are re-tested in FP64 from the original coordinates.  Lists are stored in granules of four
// entries transposed per granule (listSlot), written one 16-byte granule at a time, so that the pair
// passes read them coalesced.
#include <algorithm>


#include "pairs.cuh"

namespace sphgb {

namespace {

constexpr int kNbrBlock = 128;
constexpr int kWarpsPerBlock = kNbrBlock / kWarp;
constexpr int kStack = 192;  // 8 children x (21 levels + 3)
// internal nodes of at most this many particles are taken whole (about eight leaves of 13-16:
// the octree's last level when a cell of 64 + particles splits into small leaves)
constexpr uint32_t kCoarseNode = 128;

struct NbrArgs {
    const double *x, *y, *z;
    const void* h;
    int hIsFloat;
    const u64* cell;      // packed grid cell per particle
    const float4* loc;    // FP32 offset inside the cell (w unused here)
    float u[3];           // cell edge per axis
    int64_t first, last;
    const uint32_t* active;  // optional: only targets with active[i - first] != 0 are searched
    const int32_t* childOffsets;
    const int32_t* internalToLeaf;
    const uint32_t* layout;
    const float4* nodeBox;
    const uint2* nodeRange;  // particles [start, end) per node
    int64_t numNodes;
    DevBox box;
    uint32_t ngmax;
    int64_t stride;
    uint32_t* nbr;
    uint32_t* count;           // [last-first] neighbours excluding self (uncapped)
    int* flags;
    unsigned long long* stats; // [0] candidates [1] fp64 rechecks
};

__device__ __forceinline__ double loadH(const void* h, int isFloat, int64_t i)
{
    return isFloat ? double(static_cast<const float*>(h)[i]) : static_cast<const double*>(h)[i];
}

__device__ __forceinline__ double foldRint(double d, const DevBox& b, int k)
{
    // minimum image of the reference's distanceSq<true> / applyPbc: d - L * rint(d / L)
    return __dsub_rn(d, __dmul_rn(b.L[k], rint(__dmul_rn(d, b.iL[k]))));
}

__device__ __forceinline__ void unpackCell(u64 c, int ic[3])
{
    ic[0] = int(c & kGridMask);
    ic[1] = int((c >> kGridBits) & kGridMask);
    ic[2] = int(c >> (2 * kGridBits));
}

// offset of a particle (cell cj, offset lj) from the origin (cell co, offset lo), FP32
__device__ __forceinline__ void gridOffset(const NbrArgs& a, const int cj[3], float4 lj, const int co[3], float4 lo,
                                           float r[3])
{
    const float lv[3] = {lj.x - lo.x, lj.y - lo.y, lj.z - lo.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = fmaf(float(CoordMixed::wrap(cj[k] - co[k], a.box.pbc[k])), a.u[k], lv[k]);
}

struct WarpSmem {
    int32_t stack[kStack];
    // queue of staged candidates that lie in the group's search box: negated offsets from the
    // group origin, one array per axis so that one 16-byte broadcast load gives four candidates'
    // coordinate for the packed FP32x2 arithmetic, and their particle indices (ascending)
    alignas(16) float nx[2 * kWarp];
    alignas(16) float ny[2 * kWarp];
    alignas(16) float nz[2 * kWarp];
    alignas(16) uint32_t idx[2 * kWarp];
    // the second cull: box of the target positions (lo x y z, squared radius, hi x y z)
    alignas(16) float cull[8];
};

__global__ void __launch_bounds__(kNbrBlock, 6) nbrGroupKernel(NbrArgs a)
{
    __shared__ WarpSmem smem[kWarpsPerBlock];
    const int lane = threadIdx.x & (kWarp - 1);
    WarpSmem& sm = smem[threadIdx.x / kWarp];
    const int64_t g0 = a.first + (int64_t(blockIdx.x) * kWarpsPerBlock + threadIdx.x / kWarp) * kWarp;
    if (g0 >= a.last) return;
    const int64_t i = g0 + lane;
    bool valid = i < a.last && (a.active == nullptr || a.active[i - a.first] != 0);
    const unsigned validMask = __ballot_sync(0xffffffffu, valid);
    if (validMask == 0) return;
    const int leader = __ffs(validMask) - 1;
    const DevBox& b = a.box;

    // targets: grid form for the filter, exact FP64 radius and periodic decision
    const int64_t iv = valid ? i : g0 + leader;
    const u64 cellI = a.cell[iv];
    const float4 locI = a.loc[iv];
    const double hi = valid ? loadH(a.h, a.hIsFloat, i) : 0.0;
    const double r2 = __dmul_rn(__dmul_rn(4.0, hi), hi);  // reference radiusSq = 4 h h
    const double twoH = __dmul_rn(2.0, hi);
    bool usePbc = false;
    if (valid && (b.pbc[0] | b.pbc[1] | b.pbc[2])) {
        const double xi = a.x[i], yi = a.y[i], zi = a.z[i];
        const bool inside = __dsub_rn(xi, twoH) >= b.lo[0] && __dsub_rn(yi, twoH) >= b.lo[1] &&
                            __dsub_rn(zi, twoH) >= b.lo[2] && __dadd_rn(xi, twoH) <= b.hi[0] &&
                            __dadd_rn(yi, twoH) <= b.hi[1] && __dadd_rn(zi, twoH) <= b.hi[2];
        usePbc = !inside;
    }

    // group origin = the leader's cell and offset
    int co[3], ci[3];
    unpackCell(__shfl_sync(0xffffffffu, cellI, leader), co);
    unpackCell(cellI, ci);
    float4 lo;
    lo.x = __shfl_sync(0xffffffffu, locI.x, leader);
    lo.y = __shfl_sync(0xffffffffu, locI.y, leader);
    lo.z = __shfl_sync(0xffffffffu, locI.z, leader);
    lo.w = 0.f;
    float reli[3];
    gridOffset(a, ci, locI, co, lo, reli);
    const float dxi = reli[0], dyi = reli[1], dzi = reli[2];
    const float rf = valid ? __double2float_ru(twoH) : 0.f;

    // group search box relative to the origin
    float gmin[3] = {valid ? dxi - rf : INFINITY, valid ? dyi - rf : INFINITY, valid ? dzi - rf : INFINITY};
    float gmax[3] = {valid ? dxi + rf : -INFINITY, valid ? dyi + rf : -INFINITY, valid ? dzi + rf : -INFINITY};
#pragma unroll
    for (int k = 0; k < 3; ++k)
        for (int o = 16; o > 0; o >>= 1) {
            gmin[k] = fminf(gmin[k], __shfl_xor_sync(0xffffffffu, gmin[k], o));
            gmax[k] = fmaxf(gmax[k], __shfl_xor_sync(0xffffffffu, gmax[k], o));
        }
    // absolute position of the origin from its cell (FP32 suffices for pruning, see the pad)
    bool exactOnly = false;
    float gc[3], gs[3], Rg = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (b.pbc[k] && (gmax[k] - gmin[k]) > 0.25f * b.Lf[k]) exactOnly = true;
        const float lok = (k == 0) ? lo.x : (k == 1 ? lo.y : lo.z);
        float cAbs = float(b.lo[k]) + fmaf(float(co[k]), a.u[k], lok) + 0.5f * (gmin[k] + gmax[k]);
        if (b.pbc[k]) {
            if (cAbs >= float(b.hi[k])) cAbs -= b.Lf[k];
            else if (cAbs < float(b.lo[k])) cAbs += b.Lf[k];
        }
        gc[k] = cAbs;
        const float pad = float((fabs(b.lo[k]) + fabs(b.hi[k])) * 0x1p-19);
        gs[k] = 0.5f * (gmax[k] - gmin[k]) + pad;
        Rg = fmaxf(Rg, fmaxf(fabsf(gmin[k]), fabsf(gmax[k])));
    }
    // FP32 decision margin on d2: covers the rounding of cell edge, offsets and the squared sum;
    // pairs inside the margin get the exact FP64 test (every pair when exactOnly)
    const float r2f = float(r2);
    const float margin = 64.f * 0x1p-24f * (Rg + rf) * (Rg + rf);
    const float inBelow = r2f - margin;   // d2f < inBelow: neighbour
    const float outAbove = r2f + margin;  // d2f > outAbove: not a neighbour

    unsigned cnt = 0;
    unsigned long long tested = 0, rechecked = 0;
    const int64_t ii = i - a.first;
    const uint32_t iu = uint32_t(i);
    GranuleWriter out(a.nbr, ii, a.stride, a.ngmax);

    // the reference's distanceSq decision in FP64 (findneighbors.hpp:33-60)
    auto exactIn = [&](uint32_t j) {
        ++rechecked;
        double dx = __dsub_rn(a.x[j], a.x[i]), dy = __dsub_rn(a.y[j], a.y[i]), dz = __dsub_rn(a.z[j], a.z[i]);
        if (usePbc) {
            if (b.pbc[0]) dx = foldRint(dx, b, 0);
            if (b.pbc[1]) dy = foldRint(dy, b, 1);
            if (b.pbc[2]) dz = foldRint(dz, b, 2);
        }
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
        return d2 < r2;
    };
    auto take = [&](uint32_t j) {
        if (j != iu) {
            out.put(cnt, j);
            ++cnt;
        }
    };

    // one chunk of m <= 32 contiguous candidates [ja, ja + m), staged by the warp.  Every target
    // tests all 32 slots with a fixed trip count; slots >= m hold a far-away sentinel whose FP32
    // distance is +inf.  Groups that need the exact test for every pair loop over the m slots.
    // Candidates are staged 32 at a time (one per lane, coalesced loads of cell and offset); those
    // outside the group's search box by more than the FP32 rounding of the offsets (cullPad) are
    // dropped and the rest appended, in ascending index order, to the warp's queue by ballot
    // compaction.  A dropped candidate is farther than 2h from every target along one axis, so the
    // reference's FP64 test rejects it too.  Each full queue block of 32 is tested by every target
    // with a fixed trip count; the last, partial block has far-away sentinels in its empty slots.
    // Groups that need the exact test for every pair keep every candidate and test the filled slots.
    const float cullPad = 32.f * 0x1p-24f * (Rg + fmaxf(a.u[0], fmaxf(a.u[1], a.u[2])));
    const float bxl = gmin[0] - cullPad, bxh = gmax[0] + cullPad;
    const float byl = gmin[1] - cullPad, byh = gmax[1] + cullPad;
    const float bzl = gmin[2] - cullPad, bzh = gmax[2] + cullPad;
    // second cull: the box of the target positions grown by the largest radius with rounded
    // edges and corners (a candidate farther than max 2h from that box is farther than 2h_i from
    // every target i); the pad covers the offsets' FP32 rounding, the factor the squared sum's
    float tmn[3] = {valid ? dxi : INFINITY, valid ? dyi : INFINITY, valid ? dzi : INFINITY};
    float tmx[3] = {valid ? dxi : -INFINITY, valid ? dyi : -INFINITY, valid ? dzi : -INFINITY};
    float rfm = rf;
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            tmn[k] = fminf(tmn[k], __shfl_xor_sync(0xffffffffu, tmn[k], o));
            tmx[k] = fmaxf(tmx[k], __shfl_xor_sync(0xffffffffu, tmx[k], o));
        }
        rfm = fmaxf(rfm, __shfl_xor_sync(0xffffffffu, rfm, o));
    }
    const float cullR = rfm + cullPad;
    if (lane == 0) {
        sm.cull[0] = tmn[0];
        sm.cull[1] = tmn[1];
        sm.cull[2] = tmn[2];
        sm.cull[3] = cullR * cullR * (1.f + 0x1p-18f);
        sm.cull[4] = tmx[0];
        sm.cull[5] = tmx[1];
        sm.cull[6] = tmx[2];
        sm.cull[7] = 0.f;
    }
    __syncwarp();
    int qn = 0;  // candidates in the queue
    auto testBlock = [&](int filled) {
        if (valid) tested += unsigned(filled);
        if (exactOnly) {
            if (valid)
                for (int t = 0; t < filled; ++t) {
                    const uint32_t j = sm.idx[t];
                    if (exactIn(j)) take(j);
                }
        } else {
            // four slots per step on packed FP32x2 operations: e = d_i + (-r_j) rounds as
            // d_i - r_j, and d2 = fma(ex, ex, fma(ey, ey, ez * ez)) per slot as in scalar form.
            // The block's decisions go into two 32-bit masks (d2 below the margin: neighbour; d2
            // within it: exact FP64 test), then each lane appends its neighbours slot by slot in
            // ascending order, one loop trip per neighbour instead of a predicated append per slot.
            const float2 dx2 = make_float2(dxi, dxi), dy2 = make_float2(dyi, dyi), dz2 = make_float2(dzi, dzi);
            uint32_t hit = 0, nearm = 0;
#pragma unroll
            for (int t = 0; t < kWarp; t += 4) {
                const float4 X = *reinterpret_cast<const float4*>(&sm.nx[t]);
                const float4 Y = *reinterpret_cast<const float4*>(&sm.ny[t]);
                const float4 Z = *reinterpret_cast<const float4*>(&sm.nz[t]);
                const float2 ex0 = __fadd2_rn(dx2, make_float2(X.x, X.y));
                const float2 ex1 = __fadd2_rn(dx2, make_float2(X.z, X.w));
                const float2 ey0 = __fadd2_rn(dy2, make_float2(Y.x, Y.y));
                const float2 ey1 = __fadd2_rn(dy2, make_float2(Y.z, Y.w));
                const float2 ez0 = __fadd2_rn(dz2, make_float2(Z.x, Z.y));
                const float2 ez1 = __fadd2_rn(dz2, make_float2(Z.z, Z.w));
                const float2 q0 = __ffma2_rn(ex0, ex0, __ffma2_rn(ey0, ey0, __fmul2_rn(ez0, ez0)));
                const float2 q1 = __ffma2_rn(ex1, ex1, __ffma2_rn(ey1, ey1, __fmul2_rn(ez1, ez1)));
                const float d2[4] = {q0.x, q0.y, q1.x, q1.y};
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    hit |= (d2[s] < inBelow ? 1u : 0u) << (t + s);
                    nearm |= (d2[s] <= outAbove ? 1u : 0u) << (t + s);
                }
            }
            if (valid) {
                // a pair within the FP32 margin of the radius (rare): the exact test
                for (uint32_t band = nearm & ~hit; band != 0; band &= band - 1u) {
                    const int s = __ffs(band) - 1;
                    if (exactIn(sm.idx[s])) hit |= 1u << s;
                }
                for (; hit != 0; hit &= hit - 1u) take(sm.idx[__ffs(hit) - 1]);
            }
        }
        __syncwarp();
    };
    auto flush = [&](int64_t ja, int m) {
        float rj[3];
        bool keep = false;
        if (lane < m) {
            const int64_t j = ja + lane;
            int cj[3];
            unpackCell(a.cell[j], cj);
            gridOffset(a, cj, a.loc[j], co, lo, rj);
            const float4 cl = *reinterpret_cast<const float4*>(&sm.cull[0]);
            const float4 ch = *reinterpret_cast<const float4*>(&sm.cull[4]);
            const float ex = fmaxf(fmaxf(cl.x - rj[0], rj[0] - ch.x), 0.f);
            const float ey = fmaxf(fmaxf(cl.y - rj[1], rj[1] - ch.y), 0.f);
            const float ez = fmaxf(fmaxf(cl.z - rj[2], rj[2] - ch.z), 0.f);
            keep = exactOnly || (rj[0] >= bxl && rj[0] <= bxh && rj[1] >= byl && rj[1] <= byh && rj[2] >= bzl &&
                                 rj[2] <= bzh && fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= cl.w);
        }
        const unsigned km = __ballot_sync(0xffffffffu, keep);
        if (keep) {
            const int q = qn + __popc(km & ((1u << lane) - 1u));
            sm.nx[q] = -rj[0];
            sm.ny[q] = -rj[1];
            sm.nz[q] = -rj[2];
            sm.idx[q] = uint32_t(ja + lane);
        }
        qn += __popc(km);
        __syncwarp();
        if (qn >= kWarp) {
            testBlock(kWarp);
            qn -= kWarp;
            if (lane < qn) {  // move the queue's tail [32, 32 + qn) to the front
                sm.nx[lane] = sm.nx[kWarp + lane];
                sm.ny[lane] = sm.ny[kWarp + lane];
                sm.nz[lane] = sm.nz[kWarp + lane];
                sm.idx[lane] = sm.idx[kWarp + lane];
            }
            __syncwarp();
        }
    };
    // the partial last block: sentinels (FP32 distance +inf) in the empty slots
    auto drain = [&]() {
        if (qn == 0) return;
        if (lane >= qn) {
            sm.nx[lane] = -1e30f;
            sm.ny[lane] = -1e30f;
            sm.nz[lane] = -1e30f;
        }
        __syncwarp();
        testBlock(qn);
        qn = 0;
    };

    int64_t pa = 0, pb = 0;  // pending contiguous candidate range
    auto addRange = [&](int64_t la, int64_t lb) {
        if (la == lb) return;
        if (la != pb) {
            while (pb > pa) {
                const int m = int(pb - pa < kWarp ? pb - pa : int64_t(kWarp));
                flush(pa, m);
                pa += m;
            }
            pa = la;
        }
        pb = lb;
        while (pb - pa >= kWarp) {
            flush(pa, kWarp);
            pa += kWarp;
        }
    };

    // depth-first walk in SFC order: children pushed in reverse so child 0 is popped first
    if (lane == 0) sm.stack[0] = 0;
    int sp = 1;
    __syncwarp();
    bool overflow = false;
    while (sp > 0) {
        // stack entries: node index, sign bit set when the node's box lies inside the search box
        const int32_t e = sm.stack[--sp];
        const int32_t node = e & 0x7fffffff;
        // a leaf, an internal node inside the search box (all its children would be walked) or one
        // of at most kCoarseNode particles: one contiguous range of particles instead of a walk over
        // its leaves.  Extra candidates only cost staging: the culls and the pair test decide.
        const int32_t co8 = a.childOffsets[node];
        const uint2 nr = a.nodeRange[node];
        if (co8 == 0 || e < 0 || nr.y - nr.x <= kCoarseNode) {
            addRange(nr.x, nr.y);
            continue;
        }
        bool ov = false, inside = false;
        const int32_t child = co8 + (lane & 7);
        if (lane < 8) {
            const float4 c4 = a.nodeBox[2 * child], s4 = a.nodeBox[2 * child + 1];
            const float cc[3] = {c4.x, c4.y, c4.z}, ss[3] = {s4.x, s4.y, s4.z};
            ov = true;
            inside = true;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float dd = fabsf(cc[k] - gc[k]);
                if (b.pbc[k]) dd = fminf(dd, b.Lf[k] - dd);
                ov = ov && (dd <= ss[k] + gs[k]);
                inside = inside && (dd + ss[k] <= gs[k]);
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, ov);
        const int k = __popc(m);
        if (sp + k > kStack) {
            overflow = true;
            break;
        }
        __syncwarp();
        if (ov) sm.stack[sp + __popc(m >> (lane + 1))] = inside ? int32_t(uint32_t(child) | 0x80000000u) : child;
        sp += k;
        __syncwarp();
    }
    if (overflow) {
        if (lane == 0) atomicOr(a.flags, kFlagStackOverflow);
        return;
    }
    while (pb > pa) {
        const int m = int(pb - pa < kWarp ? pb - pa : int64_t(kWarp));
        flush(pa, m);
        pa += m;
    }
    drain();

    if (valid) {
        out.finish(cnt);
        a.count[ii] = cnt;
    }
    // warp-aggregated statistics
    for (int o = 16; o > 0; o >>= 1) {
        tested += __shfl_xor_sync(0xffffffffu, tested, o);
        rechecked += __shfl_xor_sync(0xffffffffu, rechecked, o);
    }
    if (lane == 0 && a.stats) {
        atomicAdd(&a.stats[0], tested);
        atomicAdd(&a.stats[1], rechecked);
    }
}

// h / nc iteration step (sph/include/sph/find_neighbors.hpp:26-37, updateH kernels.hpp:26-32):
// marks targets that leave [ng0/4, ngmax+1] and updates their h; counts active and failed.
template<class Th>
__global__ void hIterKernel(const uint32_t* __restrict__ count, Th* __restrict__ h, uint32_t* __restrict__ active,
                            uint8_t* __restrict__ iters, int64_t first, int64_t nWork, unsigned ng0, unsigned ngmax,
                            unsigned long long* __restrict__ counters)
{
    int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= nWork) return;
    unsigned nc = count[k] + 1;
    unsigned ngmin = ng0 / 4;
    bool bad = (ngmin > nc) || (nc - 1 > ngmax);
    bool go = bad && iters[k] < 10 && (active[k] != 0);
    if (go) {
        Th hv = h[first + k];
        const Th c0 = Th(1023.0);
        const Th ex = Th(1.0) / Th(10.0);
        h[first + k] = hv * Th(0.5) * pow(Th(1) + c0 * ng0 / Th(nc), ex);
        iters[k]++;
        atomicAdd(&counters[2], 1ull);
    }
    active[k] = go ? 1u : 0u;
}

constexpr int kNcOutBlock = 256;

__global__ void __launch_bounds__(kNcOutBlock) ncOutKernel(const uint32_t* __restrict__ count, const uint8_t* __restrict__ iters, int64_t nWork,
                            uint32_t ngmax, uint32_t* __restrict__ nc, int addSelf,
                            unsigned long long* __restrict__ counters)
{
    int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    unsigned long long capped = 0, sum = 0, fails = 0;
    unsigned mx = 0;
    if (k < nWork) {
        uint32_t cnt = count[k];
        if (nc) nc[k] = cnt + (addSelf ? 1u : 0u);
        capped = cnt > ngmax;
        sum = min(cnt, ngmax);
        mx = cnt + 1;
        fails = (iters && iters[k] >= 10) ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        capped += __shfl_xor_sync(0xffffffffu, capped, o);
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        fails += __shfl_xor_sync(0xffffffffu, fails, o);
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    // one atomic per block and counter: same-address atomics from every warp serialise in L2
    __shared__ unsigned long long sS[kNcOutBlock / kWarp], sC[kNcOutBlock / kWarp], sF[kNcOutBlock / kWarp];
    __shared__ unsigned sM[kNcOutBlock / kWarp];
    const int w = threadIdx.x / kWarp;
    if ((threadIdx.x & 31) == 0) {
        sS[w] = sum;
        sC[w] = capped;
        sF[w] = fails;
        sM[w] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < kNcOutBlock / kWarp; ++q) {
            sum += sS[q];
            capped += sC[q];
            fails += sF[q];
            mx = max(mx, sM[q]);
        }
        atomicAdd(&counters[3], sum);
        atomicAdd(&counters[4], capped);
        atomicMax(&counters[5], (unsigned long long)mx);
        atomicAdd(&counters[6], fails);
    }
}

__global__ void exportKernel(const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ count, int64_t nWork,
                             int64_t stride, uint32_t ngmax, uint32_t* __restrict__ out)
{
    int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= nWork) return;
    uint32_t c = min(count[k], ngmax);
    for (uint32_t q = 0; q < c; ++q) out[k * ngmax + q] = nbr[listSlot(k, q, stride)];
}

// ---- owned pair lists for the pair-once momentum-energy pass ----
// Pair (i, j) is mutual when the k-th neighbour j of i also lists i: j has a list (inside the
// searched range), i lies within j's capped list (the ngmax smallest indices), and |x_i - x_j|^2 <
// 4 h_j^2 in the reference's distanceSq semantics for target j (rint minimum image when the 2h box of
// j leaves the periodic box).  Decided in FP32 on the grid form with a relative margin of 2^-17 (the
// grid-form d2 and the FP32 radius are within a few 2^-24 relative of the exact values); pairs inside
// the margin or crossing a periodic face take the exact FP64 test.
// i owns every non-mutual entry and half of its mutual ones: the mutual pair {i, j} belongs to the
// smaller index when i + j is odd and to the larger when it is even, so each particle owns about
// half of its mutual pairs wherever it sits in the SFC order.  The owned entries are written
// compacted in the granule layout of the lists, entry = j | mutual << 31, with their count per particle.
struct MutualArgs {
    const double *x, *y, *z;
    const void* h;
    int hIsFloat;
    const u64* cell;
    const float4* loc;
    float u[3];
    DevBox box;
    int64_t first, last, stride;
    uint32_t ngmax;
    const uint32_t* nbr;
    const uint32_t* count;
    // (2 h_j)^2 in FP32 per particle, negative when the 2h box of j leaves the periodic box (j's
    // search takes the minimum image): no FP64 work per pair outside the rounding margin
    const float* r2f;
    // (L/4)^2 of the smallest periodic box length (INFINITY without periodic axes): pairs whose
    // larger 2h exceeds L/4 are not evaluated once, because the legacy wrap of the pair loops
    // (threshold 2h of the list owner, box.hpp:216-238) may then pick different images at the two ends
    float wrapSafe2;
    uint32_t* owned;
    uint32_t* ownedCount;
};

__global__ void radius2Kernel(const double* __restrict__ x, const double* __restrict__ y,
                              const double* __restrict__ z, const void* h, int hIsFloat, int64_t n, DevBox b,
                              float* __restrict__ r2f)
{
    const int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (j >= n) return;
    const double hj = loadH(h, hIsFloat, j);
    const float tf = 2.f * float(hj);
    bool usePbc = false;
    if (b.pbc[0] | b.pbc[1] | b.pbc[2]) {  // the search's decision for target j (nbrGroupKernel)
        const double twoH = __dmul_rn(2.0, hj);
        const bool inside = __dsub_rn(x[j], twoH) >= b.lo[0] && __dsub_rn(y[j], twoH) >= b.lo[1] &&
                            __dsub_rn(z[j], twoH) >= b.lo[2] && __dadd_rn(x[j], twoH) <= b.hi[0] &&
                            __dadd_rn(y[j], twoH) <= b.hi[1] && __dadd_rn(z[j], twoH) <= b.hi[2];
        usePbc = !inside;
    }
    r2f[j] = usePbc ? -(tf * tf) : tf * tf;
}

__device__ bool mutualExact(const MutualArgs& a, int64_t i, int64_t j, double hj)
{
    const DevBox& b = a.box;
    const double r2 = __dmul_rn(__dmul_rn(4.0, hj), hj);
    const double twoH = __dmul_rn(2.0, hj);
    const double xj = a.x[j], yj = a.y[j], zj = a.z[j];
    bool usePbc = false;
    if (b.pbc[0] | b.pbc[1] | b.pbc[2]) {
        const bool inside = __dsub_rn(xj, twoH) >= b.lo[0] && __dsub_rn(yj, twoH) >= b.lo[1] &&
                            __dsub_rn(zj, twoH) >= b.lo[2] && __dadd_rn(xj, twoH) <= b.hi[0] &&
                            __dadd_rn(yj, twoH) <= b.hi[1] && __dadd_rn(zj, twoH) <= b.hi[2];
        usePbc = !inside;
    }
    double dx = __dsub_rn(a.x[i], xj), dy = __dsub_rn(a.y[i], yj), dz = __dsub_rn(a.z[i], zj);
    if (usePbc) {
        if (b.pbc[0]) dx = foldRint(dx, b, 0);
        if (b.pbc[1]) dy = foldRint(dy, b, 1);
        if (b.pbc[2]) dz = foldRint(dz, b, 2);
    }
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return d2 < r2;
}

__device__ bool mutualPair(const MutualArgs& a, int64_t i, int ci[3], float4 li, int64_t j)
{
    if (j < a.first || j >= a.last) return false;
    const int64_t jj = j - a.first;
    if (__ldg(a.count + jj) > a.ngmax && i > int64_t(__ldg(a.nbr + listSlot(jj, a.ngmax - 1, a.stride))))
        return false;
    int cj[3];
    unpackCell(__ldg(a.cell + j), cj);
    const float4 lj = __ldg(a.loc + j);
    const float lv[3] = {li.x - lj.x, li.y - lj.y, li.z - lj.z};
    constexpr int R = 1 << kGridBits;
    bool wrapped = false;
    float r[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int d = ci[k] - cj[k];
        if (a.box.pbc[k]) {
            if (d > R / 2) {
                d -= R;
                wrapped = true;
            } else if (d < -R / 2) {
                d += R;
                wrapped = true;
            }
        }
        r[k] = fmaf(float(d), a.u[k], lv[k]);
    }
    const float R2s = __ldg(a.r2f + j);
    // across a periodic face only a target that takes the minimum image can list i
    if (wrapped && !(R2s < 0.f)) return false;
    if (fmaxf(fabsf(R2s), fabsf(__ldg(a.r2f + i))) > a.wrapSafe2) return false;
    const float d2 = fmaf(r[0], r[0], fmaf(r[1], r[1], r[2] * r[2]));
    const float R2 = fabsf(R2s), eps = 0x1p-17f * R2;
    if (d2 < R2 - eps) return true;
    if (d2 > R2 + eps) return false;
    return mutualExact(a, i, j, loadH(a.h, a.hIsFloat, j));
}

__global__ void __launch_bounds__(128) ownedListKernel(MutualArgs a)
{
    const int64_t i = a.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.last) return;
    const int64_t ii = i - a.first;
    const unsigned nc = min(__ldg(a.count + ii), a.ngmax);
    int ci[3];
    unpackCell(__ldg(a.cell + i), ci);
    const float4 li = __ldg(a.loc + i);
    unsigned cnt = 0;
    GranuleWriter out(a.owned, ii, a.stride, a.ngmax);
    for (unsigned k = 0; k < nc; ++k) {
        const uint32_t j = __ldg(a.nbr + listSlot(ii, k, a.stride));
        const bool m = mutualPair(a, i, ci, li, j);
        const bool own = !m || ((((i ^ int64_t(j)) & 1) != 0) == (i < int64_t(j)));
        if (own) out.put(cnt++, j | (m ? 0x80000000u : 0u));
    }
    out.finish(cnt);
    a.ownedCount[ii] = cnt;
}

// owned lists from list membership alone: (i, j) is mutual when i is in j's (capped, ascending)
// list, found by binary search, so the decision holds whatever the positions are now (frozen lists
// after moved particles).  Ownership of a mutual pair as in ownedListKernel (index parity).
__global__ void __launch_bounds__(128) ownedByListKernel(const uint32_t* __restrict__ nbr,
                                                         const uint32_t* __restrict__ count, int64_t first, int64_t last,
                                                         int64_t stride, uint32_t ngmax, uint32_t* __restrict__ owned,
                                                         uint32_t* __restrict__ ownedCount)
{
    const int64_t i = first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= last) return;
    const int64_t ii = i - first;
    const unsigned nc = min(__ldg(count + ii), ngmax);
    unsigned cnt = 0;
    GranuleWriter out(owned, ii, stride, ngmax);
    for (unsigned k = 0; k < nc; ++k) {
        const uint32_t j = __ldg(nbr + listSlot(ii, k, stride));
        bool m = false;
        if (int64_t(j) >= first && int64_t(j) < last) {
            const int64_t jj = int64_t(j) - first;
            unsigned lo = 0, hi = min(__ldg(count + jj), ngmax);  // search [lo, hi) of j's sorted list
            while (lo < hi) {
                const unsigned mid = (lo + hi) >> 1;
                const uint32_t e = __ldg(nbr + listSlot(jj, mid, stride));
                if (int64_t(e) < i) lo = mid + 1;
                else hi = mid;
            }
            m = lo < min(__ldg(count + jj), ngmax) && int64_t(__ldg(nbr + listSlot(jj, lo, stride))) == i;
        }
        const bool own = !m || ((((i ^ int64_t(j)) & 1) != 0) == (i < int64_t(j)));
        if (own) out.put(cnt++, j | (m ? 0x80000000u : 0u));
    }
    out.finish(cnt);
    ownedCount[ii] = cnt;
}

// longest owned list of each warp of 32 targets
__global__ void warpMaxKernel(const uint32_t* __restrict__ count, int64_t n, uint32_t* __restrict__ wmax)
{
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const uint32_t m = __reduce_max_sync(0xffffffffu, i < n ? __ldg(count + i) : 0u);
    if ((threadIdx.x & 31) == 0 && i < n) wmax[i >> 5] = m;
}

__global__ void fillOnes(uint32_t* p, int64_t n)
{
    int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k < n) p[k] = 1u;
}

// grid form of all particles' positions (cells + FP32 offsets), shared with the mixed passes
__global__ void gridFormKernel(const double* __restrict__ x, const double* __restrict__ y,
                               const double* __restrict__ z, int64_t n, DevBox box, u64* __restrict__ cell,
                               float4* __restrict__ loc)
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
    cell[i] = u64(ic[0]) | (u64(ic[1]) << kGridBits) | (u64(ic[2]) << (2 * kGridBits));
    loc[i] = make_float4(l[0], l[1], l[2], 0.f);
}

int runSearch(sphgb_ctx* c, const double* x, const double* y, const double* z, const void* h, int hIsFloat,
              int64_t first, int64_t last, uint32_t ngmax, const uint32_t* active)
{
    NbrArgs a;
    a.x = x;
    a.y = y;
    a.z = z;
    a.h = h;
    a.hIsFloat = hIsFloat;
    a.cell = c->gridKey.as<u64>();
    a.loc = c->gridLoc.as<float4>();
    for (int k = 0; k < 3; ++k) a.u[k] = float(c->box.L[k] / double(1 << kGridBits));
    a.first = first;
    a.last = last;
    a.active = active;
    a.childOffsets = c->childOffsets.as<int32_t>();
    a.internalToLeaf = c->internalToLeaf.as<int32_t>();
    a.layout = c->layout.as<uint32_t>();
    a.nodeBox = c->nodeBoxF.as<float4>();
    a.nodeRange = c->nodeRange.as<uint2>();
    a.numNodes = c->numNodes;
    a.box = c->box;
    a.ngmax = ngmax;
    a.stride = c->nbrStride;
    a.nbr = c->nbr.as<uint32_t>();
    a.count = c->ncount.as<uint32_t>();
    a.flags = c->dFlags;
    a.stats = c->counters.as<unsigned long long>();
    int64_t groups = (last - first + kWarp - 1) / kWarp;
    unsigned blocks = unsigned((groups + kWarpsPerBlock - 1) / kWarpsPerBlock);
    nbrGroupKernel<<<blocks, kNbrBlock, 0, c->stream>>>(a);
    return launched(c, "nbrGroupKernel");
}

int buildOwned(sphgb_ctx* c, const double* x, const double* y, const double* z, const void* h, int hIsFloat)
{
    const int64_t nWork = c->nbrLast - c->nbrFirst;
    SPHGB_TRY(c->owned.ensure(sizeof(uint32_t) * listCapacity(c->nbrNgmax) * size_t(c->nbrStride)));
    SPHGB_TRY(c->ownedCount.ensure(sizeof(uint32_t) * size_t(c->nbrStride)));
    SPHGB_TRY(c->ownedR2.ensure(sizeof(float) * size_t(c->n)));
    radius2Kernel<<<gridFor(c->n, 256), 256, 0, c->stream>>>(x, y, z, h, hIsFloat, c->n, c->box,
                                                            c->ownedR2.as<float>());
    SPHGB_TRY(launched(c, "radius2Kernel"));
    MutualArgs a;
    a.x = x;
    a.y = y;
    a.z = z;
    a.h = h;
    a.hIsFloat = hIsFloat;
    a.cell = c->gridKey.as<u64>();
    a.loc = c->gridLoc.as<float4>();
    for (int k = 0; k < 3; ++k) a.u[k] = float(c->box.L[k] / double(1 << kGridBits));
    a.box = c->box;
    a.first = c->nbrFirst;
    a.last = c->nbrLast;
    a.stride = c->nbrStride;
    a.ngmax = c->nbrNgmax;
    a.nbr = c->nbr.as<uint32_t>();
    a.count = c->ncount.as<uint32_t>();
    a.r2f = c->ownedR2.as<float>();
    a.wrapSafe2 = INFINITY;
    for (int k = 0; k < 3; ++k)
        if (c->box.pbc[k]) a.wrapSafe2 = std::min(a.wrapSafe2, float(0.0625 * c->box.L[k] * c->box.L[k]));
    a.owned = c->owned.as<uint32_t>();
    a.ownedCount = c->ownedCount.as<uint32_t>();
    ownedListKernel<<<gridFor(nWork, 128), 128, 0, c->stream>>>(a);
    SPHGB_TRY(launched(c, "ownedListKernel"));
    c->ownedEpoch = c->nbrEpoch;
    c->ownedFromLists = false;
    return SPHGB_OK;
}

int prepareLists(sphgb_ctx* c, const double* x, const double* y, const double* z, int64_t first, int64_t last,
                 uint32_t ngmax)
{
    if (!c->haveTree) return SPHGB_ERR_STATE;
    if (first < 0 || last > c->n || first >= last) return SPHGB_ERR_ARG;
    const int64_t nWork = last - first;
    c->nbrStride = (nWork + 31) / 32 * 32;
    // lists larger than the buffers hold: the pair-geometry cache of an earlier sweep gives its
    // memory back first (the next FP64 sweep sizes it again within half of the free memory)
    if (c->nbr.bytes < sizeof(uint32_t) * listCapacity(ngmax) * c->nbrStride) c->pairGeo.release();
    SPHGB_TRY(c->nbr.ensure(sizeof(uint32_t) * listCapacity(ngmax) * c->nbrStride));
    SPHGB_TRY(c->ncount.ensure(sizeof(uint32_t) * c->nbrStride));
    SPHGB_TRY(c->active.ensure(sizeof(uint32_t) * c->nbrStride + c->nbrStride));
    SPHGB_TRY(c->counters.ensure(sizeof(unsigned long long) * 8));
    SPHGB_CUDA(cudaMemsetAsync(c->counters.p, 0, sizeof(unsigned long long) * 8, c->stream));
    SPHGB_CUDA(cudaMemsetAsync(c->dFlags, 0, sizeof(int), c->stream));
    // grid form of every particle (neighbours may be anywhere in [0, n))
    SPHGB_TRY(c->gridKey.ensure(sizeof(u64) * c->n));
    SPHGB_TRY(c->gridLoc.ensure(sizeof(float4) * c->n));
    gridFormKernel<<<gridFor(c->n, 256), 256, 0, c->stream>>>(x, y, z, c->n, c->box, c->gridKey.as<u64>(),
                                                             c->gridLoc.as<float4>());
    SPHGB_TRY(launched(c, "gridFormKernel"));
    c->nbrFirst = first;
    c->nbrLast = last;
    c->nbrNgmax = ngmax;
    return SPHGB_OK;
}

int finishStats(sphgb_ctx* c, int64_t hIters)
{
    unsigned long long h[8];
    int flags = 0;
    SPHGB_CUDA(cudaMemcpyAsync(h, c->counters.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    SPHGB_CUDA(cudaMemcpyAsync(&flags, c->dFlags, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    c->stats.candidates = int64_t(h[0]);
    c->stats.fp64_rechecks = int64_t(h[1]);
    c->stats.nc_sum = int64_t(h[3]);
    c->stats.capped = int64_t(h[4]);
    c->stats.nc_max = uint32_t(h[5]);
    c->stats.h_fails = int64_t(h[6]);
    c->stats.h_iterations = hIters;
    if (flags & kFlagStackOverflow) return SPHGB_ERR_TRAVERSAL;
    return SPHGB_OK;
}

}  // namespace

int pairGeoStore(sphgb_ctx* c, PairGeo* out)
{
    *out = PairGeo{nullptr, nullptr, nullptr, nullptr, 0};
    c->geoValid = false;
    if (!c->inSweep || c->ownedEpoch != c->nbrEpoch || c->ownedFromLists) return SPHGB_OK;
    const int64_t nWork = c->nbrLast - c->nbrFirst, nWarps = (nWork + 31) / 32;
    if (nWork <= 0) return SPHGB_OK;
    SPHGB_TRY(c->geoRows.ensure(sizeof(uint32_t) * 2 * size_t(nWarps)));
    uint32_t* wmax = c->geoRows.as<uint32_t>();
    uint32_t* rowOff = wmax + nWarps;
    warpMaxKernel<<<gridFor(nWarps * 32, 256), 256, 0, c->stream>>>(c->ownedCount.as<uint32_t>(), nWork, wmax);
    SPHGB_TRY(launched(c, "warpMaxKernel"));
    SPHGB_TRY(exclusiveScan(c, wmax, rowOff, nWarps));
    uint32_t lastOff = 0, lastMax = 0;
    SPHGB_CUDA(cudaMemcpyAsync(&lastOff, rowOff + nWarps - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    SPHGB_CUDA(cudaMemcpyAsync(&lastMax, wmax + nWarps - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    const size_t rows = size_t(lastOff) + lastMax;
    // five arrays (|r| and 1/|r|, the two kernel values, r and dv) or the first two, whichever fits
    // in the buffer already held or in half of the free device memory
    int arrays = 0;
    for (int a : {5, 2}) {
        const size_t need = size_t(a) * 32 * sizeof(double2) * rows;
        if (c->pairGeo.bytes >= need) {
            arrays = a;
            break;
        }
        size_t freeB = 0, totalB = 0;
        if (cudaMemGetInfo(&freeB, &totalB) != cudaSuccess || need > (freeB + c->pairGeo.bytes) / 2) continue;
        if (c->pairGeo.ensure(need) != SPHGB_OK) {
            (void)cudaGetLastError();
            continue;
        }
        arrays = a;
        break;
    }
    if (arrays == 0) return SPHGB_OK;
    c->geoRowCount = rows;
    c->geoArrays = arrays;
    c->geoValid = true;
    *out = pairGeoRead(c);
    return SPHGB_OK;
}

int buildOwnedFromLists(sphgb_ctx* c)
{
    const int64_t nWork = c->nbrLast - c->nbrFirst;
    SPHGB_TRY(c->owned.ensure(sizeof(uint32_t) * listCapacity(c->nbrNgmax) * size_t(c->nbrStride)));
    SPHGB_TRY(c->ownedCount.ensure(sizeof(uint32_t) * size_t(c->nbrStride)));
    ownedByListKernel<<<gridFor(nWork, 128), 128, 0, c->stream>>>(c->nbr.as<uint32_t>(), c->ncount.as<uint32_t>(),
                                                                 c->nbrFirst, c->nbrLast, c->nbrStride, c->nbrNgmax,
                                                                 c->owned.as<uint32_t>(), c->ownedCount.as<uint32_t>());
    SPHGB_TRY(launched(c, "ownedByListKernel"));
    c->ownedEpoch = c->nbrEpoch;
    c->ownedFromLists = true;
    return SPHGB_OK;
}

int findNeighborsSph(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    if (!p->x || !p->y || !p->z || !p->h) return SPHGB_ERR_ARG;
    const uint32_t ngmax = c->prm.ngmax;
    if (c->prm.ng0 > ngmax) return SPHGB_ERR_ARG;  // reference: "ng0 should be smaller than ngmax"
    if (!c->haveTree) return SPHGB_ERR_STATE;
    if (!c->inputsChecked)
        SPHGB_TRY(validateParticles(c, p->x, p->y, p->z, p->h, p->precision == SPHGB_MIXED, c->n));
    SPHGB_TRY(prepareLists(c, p->x, p->y, p->z, first, last, ngmax));
    const int64_t nWork = last - first;
    const int hf = p->precision == SPHGB_MIXED;
    uint32_t* active = c->active.as<uint32_t>();
    uint8_t* iters = reinterpret_cast<uint8_t*>(active + c->nbrStride);
    SPHGB_CUDA(cudaMemsetAsync(iters, 0, c->nbrStride, c->stream));
    SPHGB_TRY(runSearch(c, p->x, p->y, p->z, p->h, hf, first, last, ngmax, nullptr));

    unsigned long long* ctr = c->counters.as<unsigned long long>();
    fillOnes<<<gridFor(nWork, 256), 256, 0, c->stream>>>(active, nWork);
    SPHGB_TRY(launched(c, "fillOnes"));
    int64_t rounds = 0;
    for (int it = 0; it < 10; ++it) {
        SPHGB_CUDA(cudaMemsetAsync(ctr + 2, 0, sizeof(unsigned long long), c->stream));
        if (hf)
            hIterKernel<float><<<gridFor(nWork, 256), 256, 0, c->stream>>>(
                c->ncount.as<uint32_t>(), static_cast<float*>(p->h), active, iters, first, nWork, c->prm.ng0, ngmax,
                ctr);
        else
            hIterKernel<double><<<gridFor(nWork, 256), 256, 0, c->stream>>>(
                c->ncount.as<uint32_t>(), static_cast<double*>(p->h), active, iters, first, nWork, c->prm.ng0, ngmax,
                ctr);
        SPHGB_TRY(launched(c, "hIterKernel"));
        unsigned long long nact = 0;
        SPHGB_CUDA(cudaMemcpyAsync(&nact, ctr + 2, sizeof(nact), cudaMemcpyDeviceToHost, c->stream));
        SPHGB_CUDA(cudaStreamSynchronize(c->stream));
        if (nact == 0) break;
        ++rounds;
        SPHGB_TRY(runSearch(c, p->x, p->y, p->z, p->h, hf, first, last, ngmax, active));
    }
    ncOutKernel<<<gridFor(nWork, kNcOutBlock), kNcOutBlock, 0, c->stream>>>(c->ncount.as<uint32_t>(), iters, nWork, ngmax,
                                                             p->nc ? p->nc + first : nullptr, 1, ctr);
    SPHGB_TRY(launched(c, "ncOutKernel"));
    SPHGB_TRY(finishStats(c, rounds));
    c->nbrEpoch++;
    c->haveNbr = true;
    c->precisionBuilt = p->precision;
    c->xBuilt = p->x;
    // the pair-once FP64 momentum-energy pass reads the owned lists; the mixed passes do not
    if (p->precision == SPHGB_FP64) SPHGB_TRY(buildOwned(c, p->x, p->y, p->z, p->h, hf));
    return c->stats.h_fails > 0 ? SPHGB_ERR_NOCONV : SPHGB_OK;
}

int findNeighborsFixed(sphgb_ctx* c, const double* x, const double* y, const double* z, const void* h, int32_t hPrec,
                       int64_t first, int64_t last, uint32_t ngmax, uint32_t* nbrOut, uint32_t* ncOut)
{
    if (!x || !y || !z || !h || ngmax == 0) return SPHGB_ERR_ARG;
    if (!c->haveTree) return SPHGB_ERR_STATE;
    SPHGB_TRY(validateParticles(c, x, y, z, h, hPrec == SPHGB_MIXED, c->n));
    SPHGB_TRY(prepareLists(c, x, y, z, first, last, ngmax));
    const int64_t nWork = last - first;
    SPHGB_TRY(runSearch(c, x, y, z, h, hPrec == SPHGB_MIXED, first, last, ngmax, nullptr));
    ncOutKernel<<<gridFor(nWork, kNcOutBlock), kNcOutBlock, 0, c->stream>>>(c->ncount.as<uint32_t>(), nullptr, nWork, ngmax, ncOut, 0,
                                                             c->counters.as<unsigned long long>());
    SPHGB_TRY(launched(c, "ncOutKernel"));
    if (nbrOut) {
        exportKernel<<<gridFor(nWork, 256), 256, 0, c->stream>>>(c->nbr.as<uint32_t>(), c->ncount.as<uint32_t>(),
                                                                  nWork, c->nbrStride, ngmax, nbrOut);
        SPHGB_TRY(launched(c, "exportKernel"));
    }
    SPHGB_TRY(finishStats(c, 0));
    c->nbrEpoch++;
    c->haveNbr = true;
    c->precisionBuilt = hPrec;
    c->xBuilt = x;
    if (hPrec == SPHGB_FP64) SPHGB_TRY(buildOwned(c, x, y, z, h, 0));
    return SPHGB_OK;
}

int exportNeighbors(sphgb_ctx* c, uint32_t* out)
{
    if (!c->haveNbr) return SPHGB_ERR_STATE;
    if (!out) return SPHGB_ERR_ARG;
    const int64_t nWork = c->nbrLast - c->nbrFirst;
    exportKernel<<<gridFor(nWork, 256), 256, 0, c->stream>>>(c->nbr.as<uint32_t>(), c->ncount.as<uint32_t>(), nWork,
                                                              c->nbrStride, c->nbrNgmax, out);
    SPHGB_TRY(launched(c, "exportKernel"));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    return SPHGB_OK;
}

}  // namespace sphgb
