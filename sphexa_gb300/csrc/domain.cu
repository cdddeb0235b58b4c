// Domain sync at one rank: box fit, Hilbert keys, stable key sort, field permutation, and the
// cornerstone leaf array + internal octree built directly from the sorted keys.
//
// Reference behaviour replaced: GlobalAssignmentGpu::assign + focus-tree convergence
// (domain/include/cstone/domain/assignment_gpu.cuh:78-119, focus/octree_focus.hpp:136-197),
// which at one rank converges to computeOctree(keys, bucket) (tree/csarray.hpp:429-440) and
// buildOctreeGpu (tree/octree_gpu.cu:136-157).  Here the converged tree is produced in one
// pass: particle s is the first particle of every node whose key range also holds key[s+bucket];
// such a node holds more than `bucket` particles and is split.  The children c >= 1 of all split
// nodes, plus key 0, are exactly the leaf start keys.
#include <algorithm>


#include <cmath>

#include "context.cuh"

namespace sphgb {

namespace {

constexpr int kBlock = 256;

// ---- box: min/max of the coordinates of open dimensions (sfc/box_mpi.hpp:68-103) ----
__global__ void minmaxPartials(const double* __restrict__ x, const double* __restrict__ y,
                               const double* __restrict__ z, int64_t n, double* __restrict__ part)
{
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double v[3] = {x[i], y[i], z[i]};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            mn[k] = fmin(mn[k], v[k]);
            mx[k] = fmax(mx[k], v[k]);
        }
    }
    __shared__ double s[6][kBlock / kWarp];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[k] = fmin(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmax(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    }
    int w = threadIdx.x / kWarp, l = threadIdx.x % kWarp;
    if (l == 0)
        for (int k = 0; k < 3; ++k) {
            s[2 * k][w] = mn[k];
            s[2 * k + 1][w] = mx[k];
        }
    __syncthreads();
    if (threadIdx.x < 6) {
        double r = s[threadIdx.x][0];
        for (int q = 1; q < kBlock / kWarp; ++q)
            r = (threadIdx.x & 1) ? fmax(r, s[threadIdx.x][q]) : fmin(r, s[threadIdx.x][q]);
        part[blockIdx.x * 6 + threadIdx.x] = r;
    }
}

__global__ void minmaxFinal(const double* __restrict__ part, int nb, double* __restrict__ out)
{
    int k = threadIdx.x;
    if (k >= 6) return;
    double r = part[k];
    for (int b = 1; b < nb; ++b) r = (k & 1) ? fmax(r, part[b * 6 + k]) : fmin(r, part[b * 6 + k]);
    out[k] = r;
}

// ---- keys ----
__global__ void keysKernel(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                           int64_t n, DevBox box, u64* __restrict__ keys, uint32_t* __restrict__ idx)
{
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    keys[i] = sfcKey(x[i], y[i], z[i], box);
    idx[i] = uint32_t(i);
}

// ---- gather of up to kMaxGather fields in one launch ----
constexpr int kMaxGather = 16;
struct GatherSet {
    const void* src[kMaxGather];
    void* dst[kMaxGather];
    int esz[kMaxGather];
    int count;
};

__global__ void gatherKernel(GatherSet g, const uint32_t* __restrict__ order, int64_t n)
{
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    uint32_t s = order[i];
    for (int f = 0; f < g.count; ++f) {
        if (g.esz[f] == 8) static_cast<double*>(g.dst[f])[i] = static_cast<const double*>(g.src[f])[s];
        else static_cast<float*>(g.dst[f])[i] = static_cast<const float*>(g.src[f])[s];
    }
}

// ---- tree ----
__global__ void splitCountKernel(const u64* __restrict__ keys, int64_t n, int bucket, uint32_t* __restrict__ cnt)
{
    int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (s > n) return;
    uint32_t c = 0;
    if (s + bucket < n) {
        int deep = min(commonPrefixBits(keys[s], keys[s + bucket]) / 3, kMaxLevel - 1);
        int first = (s == 0) ? 0 : commonPrefixBits(keys[s - 1], keys[s]) / 3 + 1;
        c = deep >= first ? uint32_t(deep - first + 1) : 0u;
    }
    cnt[s] = c;  // cnt[n] = 0 closes the exclusive scan
}

__global__ void splitEmitKernel(const u64* __restrict__ keys, int64_t n, int bucket, const uint32_t* __restrict__ off,
                                int64_t numSplit, u64* __restrict__ leafKeys, u64* __restrict__ internalCodes)
{
    int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (s == 0) leafKeys[7 * numSplit] = 0;
    if (s >= n || s + bucket >= n) return;
    uint32_t o = off[s], c = off[s + 1] - o;
    if (c == 0) return;
    int first = (s == 0) ? 0 : commonPrefixBits(keys[s - 1], keys[s]) / 3 + 1;
    for (uint32_t k = 0; k < c; ++k) {
        int l = first + int(k);
        u64 start = keys[s] & ~(nodeRange(l) - 1);
        internalCodes[o + k] = placeholder(start, l);
        u64 step = nodeRange(l + 1);
#pragma unroll
        for (int ch = 1; ch < 8; ++ch) leafKeys[7 * (int64_t(o) + k) + ch - 1] = start + u64(ch) * step;
    }
}

// ---- one rebalance of the previous sync's tree (the single-rank focus tree across syncs) ----
__device__ __forceinline__ int leafLevel(u64 span) { return kMaxLevel - (63 - __clzll((long long)span)) / 3; }

__device__ __forceinline__ int64_t lowerBoundLeaves(const u64* __restrict__ a, int64_t n, u64 v);

// particles of the node [start, start + nodeRange(level)) in the previous tree: node boundaries are
// leaf boundaries of that tree, so two positions in its leaf array and its layout give the count
__device__ __forceinline__ uint32_t prevNodeCount(const u64* __restrict__ leaves, int64_t numLeaves,
                                                  const uint32_t* __restrict__ layout, u64 start, int level)
{
    const int64_t a = lowerBoundLeaves(leaves, numLeaves + 1, start);
    const int64_t b = lowerBoundLeaves(leaves, numLeaves + 1, start + nodeRange(level));
    return layout[b] - layout[a];
}

// per leaf of the previous tree: 8 = split, 1 = keep, 0 = merged away (CombinedUpdate::updateFocus,
// domain/include/cstone/focus/octree_focus.hpp:65-113, decisions of focus/rebalance.hpp:32-66 and
// protectAncestors :152-165, at one rank where the focus is the whole key range).  A leaf whose
// parent holds more than bucket particles splits when it holds more than bucket itself, else stays;
// otherwise the subtree under its highest ancestor holding at most bucket particles collapses into
// that ancestor, whose left-most leaf keeps the start key.
__global__ void rebalanceOpsKernel(const u64* __restrict__ leaves, const uint32_t* __restrict__ layout,
                                   int64_t numLeaves, uint32_t bucket, uint32_t* __restrict__ ops)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k > numLeaves) return;
    if (k == numLeaves) {
        ops[k] = 0;  // closes the exclusive scan
        return;
    }
    const u64 s = leaves[k];
    const int level = leafLevel(leaves[k + 1] - s);
    const uint32_t own = layout[k + 1] - layout[k];
    uint32_t op;
    if (level == 0) op = own > bucket ? 8u : 1u;
    else {
        const u64 ps = s & ~(nodeRange(level - 1) - 1);
        if (prevNodeCount(leaves, numLeaves, layout, ps, level - 1) > bucket)
            op = (own > bucket && level < kMaxLevel) ? 8u : 1u;
        else {
            u64 as = ps;
            int al = level - 1;
            while (al > 0) {
                const u64 pp = as & ~(nodeRange(al - 1) - 1);
                if (prevNodeCount(leaves, numLeaves, layout, pp, al - 1) > bucket) break;
                as = pp;
                --al;
            }
            op = s == as ? 1u : 0u;
        }
    }
    ops[k] = op;
}

__global__ void rebalanceEmitKernel(const u64* __restrict__ leaves, int64_t numLeaves, const uint32_t* __restrict__ ops,
                                    const uint32_t* __restrict__ off, u64* __restrict__ out)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= numLeaves) return;
    const uint32_t op = ops[k];
    if (op == 0) return;
    const u64 s = leaves[k];
    const uint32_t o = off[k];
    if (op == 1) out[o] = s;
    else {
        const u64 step = nodeRange(leafLevel(leaves[k + 1] - s) + 1);
#pragma unroll
        for (int c = 0; c < 8; ++c) out[o + c] = s + u64(c) * step;
    }
}

// internal nodes of a cornerstone leaf array: leaf k (start s, level l) is the left-most leaf of the
// nodes that start at s on the levels d..l-1, d the level of the last non-zero octal digit of s
__device__ __forceinline__ int alignLevel(u64 s) { return s == 0 ? 0 : kMaxLevel - (__ffsll((long long)s) - 1) / 3; }

__global__ void internalCountKernel(const u64* __restrict__ leaves, int64_t numLeaves, uint32_t* __restrict__ cnt)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k > numLeaves) return;
    if (k == numLeaves) {
        cnt[k] = 0;
        return;
    }
    const int l = leafLevel(leaves[k + 1] - leaves[k]), d = alignLevel(leaves[k]);
    cnt[k] = l > d ? uint32_t(l - d) : 0u;
}

__global__ void internalEmitKernel(const u64* __restrict__ leaves, int64_t numLeaves, const uint32_t* __restrict__ off,
                                   u64* __restrict__ codes)
{
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= numLeaves) return;
    const u64 s = leaves[k];
    const int l = leafLevel(leaves[k + 1] - s), d = alignLevel(s);
    uint32_t o = off[k];
    for (int q = d; q < l; ++q) codes[o++] = placeholder(s, q);
}

__global__ void levelRangeKernel(const u64* __restrict__ codes, int64_t numInternal, int32_t* __restrict__ out)
{
    // out[0..22]: first internal node of each level (level-major order); out[23..45]: levelRange
    __shared__ int32_t intStart[kMaxLevel + 2];
    int l = threadIdx.x;
    if (l <= kMaxLevel + 1) {
        int32_t v = int32_t(numInternal);
        if (l <= kMaxLevel) {
            u64 target = u64(1) << (3 * l);
            int64_t lo = 0, hi = numInternal;
            while (lo < hi) {
                int64_t mid = (lo + hi) / 2;
                if (codes[mid] < target) lo = mid + 1;
                else hi = mid;
            }
            v = int32_t(lo);
        }
        intStart[l] = v;
        out[l] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int32_t* lr = out + (kMaxLevel + 2);
        lr[0] = 0;
        lr[1] = 1;
        for (int lev = 1; lev <= kMaxLevel; ++lev) lr[lev + 1] = lr[lev] + 8 * (intStart[lev] - intStart[lev - 1]);
    }
}

__device__ __forceinline__ int64_t lowerBoundKeys(const u64* __restrict__ a, int64_t n, u64 v)
{
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int64_t lowerBoundLeaves(const u64* __restrict__ a, int64_t n, u64 v)
{
    return lowerBoundKeys(a, n, v);
}

__global__ void octreeNodesKernel(const u64* __restrict__ internalCodes, const int32_t* __restrict__ ranges,
                                  const u64* __restrict__ leaves, int64_t numLeaves, int64_t numInternal,
                                  int64_t numNodes, DevBox box, u64* __restrict__ prefixes,
                                  int32_t* __restrict__ childOffsets, int32_t* __restrict__ internalToLeaf,
                                  double* __restrict__ center, double* __restrict__ size, float4* __restrict__ boxF)
{
    int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= numNodes) return;
    const int32_t* intStart = ranges;
    const int32_t* levelRange = ranges + (kMaxLevel + 2);
    int l = 0;
    while (l < kMaxLevel && levelRange[l + 1] <= idx) ++l;
    u64 code;
    if (l == 0) code = 1;
    else {
        int64_t q = idx - levelRange[l];
        code = (internalCodes[intStart[l - 1] + (q >> 3)] << 3) | u64(q & 7);
    }
    prefixes[idx] = code;
    u64 start = placeholderKey(code);

    int32_t child = 0;
    int64_t r = -1;
    if (l < kMaxLevel) {
        int64_t b = intStart[l], e = intStart[l + 1];
        int64_t p = b + lowerBoundKeys(internalCodes + b, e - b, code);
        if (p < e && internalCodes[p] == code) r = p - b;
    }
    if (r >= 0) {
        child = int32_t(levelRange[l + 1] + 8 * r);
        // reference label: unsorted-layout slot (binaryKeyWeight, tree/octree.hpp:54-89) - numInternal
        int64_t tid = lowerBoundKeys(leaves, numLeaves + 1, start + 4 * nodeRange(l + 1)) - 1;
        u64 lk = leaves[tid];
        int64_t w = 0;
        for (int q = 1; q <= l + 1; ++q) {
            int dig = int((lk >> (3 * (kMaxLevel - q))) & 7u);
            w += dig >= 4 ? 7 - dig : -dig;
        }
        internalToLeaf[idx] = int32_t((tid + w) / 7 - numInternal);
    } else {
        internalToLeaf[idx] = int32_t(lowerBoundKeys(leaves, numLeaves + 1, start));
    }
    childOffsets[idx] = child;

    // geometric center and half size: nodeFpCenters + centerAndSize
    // (focus/source_center.hpp:129-141, sfc/box.hpp:317-334), rounded step by step
    unsigned ic[3];
    hilbertDecode(start, ic);
    unsigned edge = (1u << kMaxLevel) >> l;
    const double uL = 1.0 / double(1u << kMaxLevel);
    float cf[3], sf[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int lo = int(ic[k] & ~(edge - 1)), hi = lo + int(edge);
        double half = __dmul_rn(__dmul_rn(0.5, uL), box.L[k]);
        double c = __dadd_rn(box.lo[k], __dmul_rn(double(hi + lo), half));
        double s = __dmul_rn(double(hi - lo), half);
        center[3 * idx + k] = c;
        size[3 * idx + k] = s;
        // float copy for pruning, widened to cover the rounding of both numbers
        double pad = (fabs(box.lo[k]) + fabs(box.hi[k])) * 0x1p-22;
        cf[k] = __double2float_rn(c);
        sf[k] = __double2float_ru(s + pad);
    }
    boxF[2 * idx] = make_float4(cf[0], cf[1], cf[2], 0.f);
    boxF[2 * idx + 1] = make_float4(sf[0], sf[1], sf[2], 0.f);
}

// particles [start, end) of every node: from the first leaf (child-0 chain) to the last (child-7
// chain) under it; a node's particles are contiguous in SFC order
__global__ void nodeRangeKernel(int64_t numNodes, const int32_t* __restrict__ childOffsets,
                                const int32_t* __restrict__ internalToLeaf, const uint32_t* __restrict__ layout,
                                uint2* __restrict__ range)
{
    const int64_t n = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (n >= numNodes) return;
    int32_t a = int32_t(n), b = int32_t(n), co;
    for (int d = 0; d <= kMaxLevel && (co = childOffsets[a]) != 0; ++d) a = co;
    for (int d = 0; d <= kMaxLevel && (co = childOffsets[b]) != 0; ++d) b = co + 7;
    range[n] = make_uint2(layout[internalToLeaf[a]], layout[internalToLeaf[b] + 1]);
}

__global__ void layoutKernel(const u64* __restrict__ keys, int64_t n, const u64* __restrict__ leaves,
                             int64_t numLeaves, uint32_t* __restrict__ layout)
{
    int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t > numLeaves) return;
    layout[t] = uint32_t(lowerBoundKeys(keys, n, leaves[t]));
}

__global__ void setKey(u64* p, u64 v) { *p = v; }

template<class T>
__global__ void permuteKernel(const T* __restrict__ src, T* __restrict__ dst, const uint32_t* __restrict__ order,
                              int64_t n)
{
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < n) dst[i] = src[order[i]];
}

}  // namespace

int applyOrder(sphgb_ctx* c, void* field, int esz)
{
    if (!c->haveSync) return SPHGB_ERR_STATE;
    if (!field || (esz != 1 && esz != 2 && esz != 4 && esz != 8)) return SPHGB_ERR_ARG;
    const int64_t n = c->n;
    SPHGB_TRY(c->gatherScratch.ensure(size_t(esz) * n));
    const uint32_t* ord = c->order.as<uint32_t>();
    unsigned blocks = gridFor(n, kBlock);
    switch (esz) {
    case 1: permuteKernel<uint8_t><<<blocks, kBlock, 0, c->stream>>>((const uint8_t*)field, c->gatherScratch.as<uint8_t>(), ord, n); break;
    case 2: permuteKernel<uint16_t><<<blocks, kBlock, 0, c->stream>>>((const uint16_t*)field, c->gatherScratch.as<uint16_t>(), ord, n); break;
    case 4: permuteKernel<uint32_t><<<blocks, kBlock, 0, c->stream>>>((const uint32_t*)field, c->gatherScratch.as<uint32_t>(), ord, n); break;
    default: permuteKernel<u64><<<blocks, kBlock, 0, c->stream>>>((const u64*)field, c->gatherScratch.as<u64>(), ord, n); break;
    }
    SPHGB_TRY(launched(c, "permuteKernel"));
    SPHGB_CUDA(cudaMemcpyAsync(field, c->gatherScratch.p, size_t(esz) * n, cudaMemcpyDeviceToDevice, c->stream));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    return SPHGB_OK;
}

int domainSync(sphgb_ctx* c, sphgb_particles* p, sphgb_box* box)
{
    const int64_t n = p->n;
    if (n <= 0 || n >= (int64_t(1) << 31) || !p->x || !p->y || !p->z) return SPHGB_ERR_ARG;
    cudaStream_t st = c->stream;
    for (int k = 0; k < 6; ++k)
        if (!std::isfinite(box->lim[k])) return SPHGB_ERR_INPUT;
    // no key, sort or tree kernel sees a non-finite coordinate or smoothing length
    SPHGB_TRY(validateParticles(c, p->x, p->y, p->z, p->h, p->precision == SPHGB_MIXED, n));
    c->n = n;

    // box: periodic dims keep their limits, open dims take the particle extrema
    sphgb_box b = *box;
    if (b.bc[0] != SPHGB_BC_PERIODIC || b.bc[1] != SPHGB_BC_PERIODIC || b.bc[2] != SPHGB_BC_PERIODIC) {
        int nb = 4 * 152;
        SPHGB_TRY(c->minmax.ensure(sizeof(double) * (6 * nb + 6)));
        double* part = c->minmax.as<double>();
        minmaxPartials<<<nb, kBlock, 0, st>>>(p->x, p->y, p->z, n, part);
        SPHGB_TRY(launched(c, "minmaxPartials"));
        minmaxFinal<<<1, 32, 0, st>>>(part, nb, part + 6 * nb);
        SPHGB_TRY(launched(c, "minmaxFinal"));
        double ext[6];
        SPHGB_CUDA(cudaMemcpyAsync(ext, part + 6 * nb, sizeof(ext), cudaMemcpyDeviceToHost, st));
        SPHGB_CUDA(cudaStreamSynchronize(st));
        for (int k = 0; k < 3; ++k)
            if (b.bc[k] != SPHGB_BC_PERIODIC) {
                b.lim[2 * k] = ext[2 * k];
                b.lim[2 * k + 1] = ext[2 * k + 1];
            }
    }
    // across the steps of one simulation the box may grow freely but shrinks by at most 5 % of its
    // previous length per side and sync (limitBoxShrinking, domain/include/cstone/sfc/box.hpp:397-414,
    // applied from the second sync on, domain/assignment.hpp:80-82)
    if (c->domainMode == 1 && !c->domainFirst) {
        const sphgb_box& q = c->prevBox;
        for (int k = 0; k < 3; ++k) {
            const double lo = q.lim[2 * k], hi = q.lim[2 * k + 1], len = hi - lo;
            b.lim[2 * k] = std::min(b.lim[2 * k], lo + 0.05 * len);
            b.lim[2 * k + 1] = std::max(b.lim[2 * k + 1], hi - 0.05 * len);
        }
    }
    for (int k = 0; k < 3; ++k)
        if (!(b.lim[2 * k + 1] > b.lim[2 * k])) return SPHGB_ERR_ARG;
    // across the syncs of one simulation the tree is updated once per sync from the previous tree
    // and its counts (the reference's focus tree, converged only at the first sync)
    const bool rebalance = c->domainMode == 1 && !c->domainFirst && c->haveTree;
    c->prevBox = b;
    c->domainFirst = false;
    *box = b;
    c->hbox = b;
    c->box = makeDevBox(b);
    c->haveBox = true;

    // keys + stable radix sort (63 key bits) of (key, index) pairs
    SPHGB_TRY(c->keys.ensure(sizeof(u64) * n));
    SPHGB_TRY(c->keysAlt.ensure(sizeof(u64) * n));
    SPHGB_TRY(c->order.ensure(sizeof(uint32_t) * n));
    SPHGB_TRY(c->orderAlt.ensure(sizeof(uint32_t) * n));
    keysKernel<<<gridFor(n, kBlock), kBlock, 0, st>>>(p->x, p->y, p->z, n, c->box, c->keysAlt.as<u64>(),
                                                       c->orderAlt.as<uint32_t>());
    SPHGB_TRY(launched(c, "keysKernel"));
    SPHGB_TRY(radixSort(c, c->keysAlt.as<u64>(), c->keys.as<u64>(), c->orderAlt.as<uint32_t>(),
                        c->order.as<uint32_t>(), n, 63));

    // permute the conserved fields in place (the reference's particleProperties of sync)
    const size_t hs = p->precision == SPHGB_MIXED ? 4 : 8;
    GatherSet g{};
    size_t bytes = 0;
    auto add = [&](void* f, int esz) {
        if (!f) return;
        g.src[g.count] = f;
        g.esz[g.count] = esz;
        g.count++;
        bytes += size_t(esz) * n;
    };
    add(p->x, 8);
    add(p->y, 8);
    add(p->z, 8);
    add(p->u, 8);
    add(p->h, int(hs));
    add(p->m, int(hs));
    add(p->vx, int(hs));
    add(p->vy, int(hs));
    add(p->vz, int(hs));
    add(p->alpha, int(hs));
    SPHGB_TRY(c->gatherScratch.ensure(bytes));
    char* scratch = c->gatherScratch.as<char>();
    size_t offs = 0;
    for (int f = 0; f < g.count; ++f) {
        g.dst[f] = scratch + offs;
        offs += size_t(g.esz[f]) * n;
    }
    gatherKernel<<<gridFor(n, kBlock), kBlock, 0, st>>>(g, c->order.as<uint32_t>(), n);
    SPHGB_TRY(launched(c, "gatherKernel"));
    for (int f = 0; f < g.count; ++f)
        SPHGB_CUDA(cudaMemcpyAsync(const_cast<void*>(g.src[f]), g.dst[f], size_t(g.esz[f]) * n,
                                   cudaMemcpyDeviceToDevice, st));
    if (p->keys) SPHGB_CUDA(cudaMemcpyAsync(p->keys, c->keys.p, sizeof(u64) * n, cudaMemcpyDeviceToDevice, st));
    c->haveSync = true;
    c->haveNbr = false;
    return buildTree(c, rebalance);
}

// exclusive sum of cnt[0..count) into off[0..count), returns off[count - 1] + cnt[count - 1]
static int scanCounts(sphgb_ctx* c, uint32_t* cnt, uint32_t* off, int64_t count, int64_t* total)
{
    SPHGB_TRY(exclusiveScan(c, cnt, off, count));
    uint32_t t = 0;
    SPHGB_CUDA(cudaMemcpyAsync(&t, off + count - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    *total = t;  // cnt[count - 1] is 0 by construction
    return SPHGB_OK;
}

// rebalance = false: the converged cornerstone tree of the sorted keys (leaves split until no leaf
// holds more than bucket particles).  rebalance = true: one update of the previous sync's tree with
// the previous sync's counts, as the reference's focus tree evolves between syncs.
int buildTree(sphgb_ctx* c, bool rebalance)
{
    const int64_t n = c->n;
    cudaStream_t st = c->stream;
    const int bucket = int(c->prm.bucket);
    const u64* keys = c->keys.as<u64>();
    int64_t S = 0, L = 0;

    if (!rebalance) {
        SPHGB_TRY(c->splitCount.ensure(sizeof(uint32_t) * (n + 1)));
        SPHGB_TRY(c->splitOffset.ensure(sizeof(uint32_t) * (n + 1)));
        splitCountKernel<<<gridFor(n + 1, kBlock), kBlock, 0, st>>>(keys, n, bucket, c->splitCount.as<uint32_t>());
        SPHGB_TRY(launched(c, "splitCountKernel"));
        SPHGB_TRY(scanCounts(c, c->splitCount.as<uint32_t>(), c->splitOffset.as<uint32_t>(), n + 1, &S));
        L = 7 * S + 1;
        SPHGB_TRY(c->leafKeysTmp.ensure(sizeof(u64) * (L + 1)));
        SPHGB_TRY(c->leaves.ensure(sizeof(u64) * (L + 1)));
        SPHGB_TRY(c->internalTmp.ensure(sizeof(u64) * (S + 1)));
        SPHGB_TRY(c->internalCodes.ensure(sizeof(u64) * (S + 1)));
        splitEmitKernel<<<gridFor(n, kBlock), kBlock, 0, st>>>(keys, n, bucket, c->splitOffset.as<uint32_t>(), S,
                                                               c->leafKeysTmp.as<u64>(), c->internalTmp.as<u64>());
        SPHGB_TRY(launched(c, "splitEmitKernel"));
        if (L > 1) {
            SPHGB_TRY(radixSort(c, c->leafKeysTmp.as<u64>(), c->leaves.as<u64>(), nullptr, nullptr, L, 63));
        } else {
            SPHGB_CUDA(cudaMemsetAsync(c->leaves.p, 0, sizeof(u64), st));
        }
    } else {
        // the previous tree: c->leaves (numLeaves + 1 keys) and its layout of the previous keys
        const int64_t Lp = c->numLeaves;
        SPHGB_TRY(c->splitCount.ensure(sizeof(uint32_t) * (Lp + 1)));
        SPHGB_TRY(c->splitOffset.ensure(sizeof(uint32_t) * (Lp + 1)));
        rebalanceOpsKernel<<<gridFor(Lp + 1, kBlock), kBlock, 0, st>>>(c->leaves.as<u64>(), c->layout.as<uint32_t>(), Lp,
                                                                      uint32_t(bucket), c->splitCount.as<uint32_t>());
        SPHGB_TRY(launched(c, "rebalanceOpsKernel"));
        SPHGB_TRY(scanCounts(c, c->splitCount.as<uint32_t>(), c->splitOffset.as<uint32_t>(), Lp + 1, &L));
        SPHGB_TRY(c->leafKeysTmp.ensure(sizeof(u64) * (L + 1)));
        rebalanceEmitKernel<<<gridFor(Lp, kBlock), kBlock, 0, st>>>(c->leaves.as<u64>(), Lp, c->splitCount.as<uint32_t>(),
                                                                   c->splitOffset.as<uint32_t>(), c->leafKeysTmp.as<u64>());
        SPHGB_TRY(launched(c, "rebalanceEmitKernel"));
        setKey<<<1, 1, 0, st>>>(c->leafKeysTmp.as<u64>() + L, kKeyEnd);
        SPHGB_TRY(launched(c, "setKey"));
        // internal nodes of the new leaves
        SPHGB_TRY(c->splitCount.ensure(sizeof(uint32_t) * (L + 1)));
        SPHGB_TRY(c->splitOffset.ensure(sizeof(uint32_t) * (L + 1)));
        internalCountKernel<<<gridFor(L + 1, kBlock), kBlock, 0, st>>>(c->leafKeysTmp.as<u64>(), L,
                                                                      c->splitCount.as<uint32_t>());
        SPHGB_TRY(launched(c, "internalCountKernel"));
        SPHGB_TRY(scanCounts(c, c->splitCount.as<uint32_t>(), c->splitOffset.as<uint32_t>(), L + 1, &S));
        if (7 * S + 1 != L) return SPHGB_ERR_STATE;  // not a cornerstone leaf array
        SPHGB_TRY(c->internalTmp.ensure(sizeof(u64) * (S + 1)));
        SPHGB_TRY(c->internalCodes.ensure(sizeof(u64) * (S + 1)));
        internalEmitKernel<<<gridFor(L, kBlock), kBlock, 0, st>>>(c->leafKeysTmp.as<u64>(), L,
                                                                 c->splitOffset.as<uint32_t>(), c->internalTmp.as<u64>());
        SPHGB_TRY(launched(c, "internalEmitKernel"));
        SPHGB_TRY(c->leaves.ensure(sizeof(u64) * (L + 1)));
        SPHGB_CUDA(cudaMemcpyAsync(c->leaves.p, c->leafKeysTmp.p, sizeof(u64) * L, cudaMemcpyDeviceToDevice, st));
    }
    c->numInternal = S;
    c->numLeaves = L;
    c->numNodes = L + S;
    if (S > 0) SPHGB_TRY(radixSort(c, c->internalTmp.as<u64>(), c->internalCodes.as<u64>(), nullptr, nullptr, S, 62));
    setKey<<<1, 1, 0, st>>>(c->leaves.as<u64>() + L, kKeyEnd);
    SPHGB_TRY(launched(c, "setKey"));

    SPHGB_TRY(c->levelRangeDev.ensure(sizeof(int32_t) * 2 * (kMaxLevel + 2)));
    levelRangeKernel<<<1, 32, 0, st>>>(c->internalCodes.as<u64>(), S, c->levelRangeDev.as<int32_t>());
    SPHGB_TRY(launched(c, "levelRangeKernel"));

    const int64_t NN = c->numNodes;
    SPHGB_TRY(c->prefixes.ensure(sizeof(u64) * NN));
    SPHGB_TRY(c->childOffsets.ensure(sizeof(int32_t) * (NN + 1)));
    SPHGB_TRY(c->internalToLeaf.ensure(sizeof(int32_t) * NN));
    SPHGB_TRY(c->nodeCenter.ensure(sizeof(double) * 3 * NN));
    SPHGB_TRY(c->nodeSize.ensure(sizeof(double) * 3 * NN));
    SPHGB_TRY(c->nodeBoxF.ensure(sizeof(float4) * 2 * NN));
    octreeNodesKernel<<<gridFor(NN, kBlock), kBlock, 0, st>>>(
        c->internalCodes.as<u64>(), c->levelRangeDev.as<int32_t>(), c->leaves.as<u64>(), L, S, NN, c->box,
        c->prefixes.as<u64>(), c->childOffsets.as<int32_t>(), c->internalToLeaf.as<int32_t>(),
        c->nodeCenter.as<double>(), c->nodeSize.as<double>(), c->nodeBoxF.as<float4>());
    SPHGB_TRY(launched(c, "octreeNodesKernel"));

    SPHGB_TRY(c->layout.ensure(sizeof(uint32_t) * (L + 1)));
    layoutKernel<<<gridFor(L + 1, kBlock), kBlock, 0, st>>>(keys, n, c->leaves.as<u64>(), L,
                                                            c->layout.as<uint32_t>());
    SPHGB_TRY(launched(c, "layoutKernel"));
    SPHGB_TRY(c->nodeRange.ensure(sizeof(uint2) * NN));
    nodeRangeKernel<<<gridFor(NN, kBlock), kBlock, 0, st>>>(NN, c->childOffsets.as<int32_t>(),
                                                            c->internalToLeaf.as<int32_t>(), c->layout.as<uint32_t>(),
                                                            c->nodeRange.as<uint2>());
    SPHGB_TRY(launched(c, "nodeRangeKernel"));
    SPHGB_CUDA(cudaMemcpyAsync(c->levelRange, c->levelRangeDev.as<int32_t>() + (kMaxLevel + 2),
                               sizeof(int32_t) * (kMaxLevel + 2), cudaMemcpyDeviceToHost, st));
    SPHGB_TRY(sortStatusAsync(c));  // the key and tree sorts of this sync
    SPHGB_CUDA(cudaStreamSynchronize(st));
    SPHGB_TRY(sortStatusAfterSync(c));
    c->stats.num_leaves = L;
    c->stats.num_nodes = NN;
    c->stats.num_internal = S;
    for (int k = 0; k < kMaxLevel + 2; ++k) c->stats.level_range[k] = c->levelRange[k];
    c->haveTree = true;
    return SPHGB_OK;
}

}  // namespace sphgb
