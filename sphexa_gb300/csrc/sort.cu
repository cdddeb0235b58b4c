// Stable LSD radix sort of 64-bit keys (with optional 32-bit values) and exclusive prefix sum of
// 32-bit counts: the sort of (SFC key, index) pairs behind the reference's sort_by_key
// (domain/include/cstone/primitives/gather.hpp:43-74, primitives_gpu.cu:323-340), the tree's key
// sorts and the count scans.
//
// Sort: 8-bit digits, one pass per digit.  A pass is three launches over tiles of 4096 keys:
//   histogram   per-tile digit counts, stored digit-major: counts[digit * tiles + tile]
//   scan        exclusive prefix of that matrix: each (digit, tile) gets its first output slot
//   scatter     each tile ranks its keys per digit in index order (warp match for the lanes of one
//               round, per-warp prefix in shared memory, a running base across the tile's rounds)
//               into shared memory, grouped by digit, then writes each digit's run to its slots:
//               equal digits keep their input order, so every pass, and the sort, is stable.
// Scan: per-tile sums, one block scanning the sums, per-tile scan with its base.
#include "context.cuh"

namespace sphgb {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;
constexpr int kWarps = kThreads / 32;
constexpr int kRadix = 256;
constexpr size_t kStageKeys = sizeof(u64) * kTile, kStagePairs = (sizeof(u64) + sizeof(uint32_t)) * kTile;

__global__ void __launch_bounds__(kThreads) radixHistKernel(const u64* __restrict__ keys, int64_t n, int shift,
                                                            int64_t tiles, uint32_t* __restrict__ counts)
{
    __shared__ uint32_t h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = int64_t(blockIdx.x) * kTile;
#pragma unroll 4
    for (int r = 0; r < kItems; ++r) {
        const int64_t i = base + int64_t(r) * kThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[unsigned(keys[i] >> shift) & (kRadix - 1)], 1u);
    }
    __syncthreads();
    counts[int64_t(threadIdx.x) * tiles + blockIdx.x] = h[threadIdx.x];
}

__device__ __forceinline__ uint32_t blockExclusiveScan(uint32_t v, uint32_t* sh, uint32_t& blockTotal);

// ranks the tile's keys per digit in index order into shared memory (tile-local digit runs), then
// writes the runs out: consecutive slots of one digit go to consecutive global slots (coalesced)
template<bool WithVals>
__global__ void __launch_bounds__(kThreads) radixScatterKernel(const u64* __restrict__ keysIn,
                                                               const uint32_t* __restrict__ valsIn,
                                                               u64* __restrict__ keysOut, uint32_t* __restrict__ valsOut,
                                                               int64_t n, int shift, int64_t tiles,
                                                               const uint32_t* __restrict__ counts,
                                                               const uint32_t* __restrict__ offsets)
{
    extern __shared__ u64 staged[];  // kTile keys, then kTile values
    uint32_t* stagedVals = reinterpret_cast<uint32_t*>(staged + kTile);
    __shared__ uint32_t base[kRadix], localStart[kRadix], globalStart[kRadix];
    __shared__ uint32_t warpCnt[kWarps][kRadix];
    __shared__ uint32_t sh[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t cell = int64_t(tid) * tiles + blockIdx.x;
    uint32_t tileTotal;
    const uint32_t ls = blockExclusiveScan(counts[cell], sh, tileTotal);
    localStart[tid] = ls;
    base[tid] = ls;
    globalStart[tid] = offsets[cell];
    const int64_t tileStart = int64_t(blockIdx.x) * kTile;
    for (int r = 0; r < kItems; ++r) {
#pragma unroll
        for (int w = 0; w < kWarps; ++w) warpCnt[w][tid] = 0;
        __syncthreads();
        const int64_t i = tileStart + int64_t(r) * kThreads + tid;
        const bool valid = i < n;
        const u64 key = valid ? keysIn[i] : 0;
        const uint32_t val = (WithVals && valid) ? valsIn[i] : 0u;
        const unsigned digit = valid ? (unsigned(key >> shift) & (kRadix - 1)) : unsigned(kRadix);
        const unsigned peers = __match_any_sync(0xffffffffu, digit);
        const unsigned rankInWarp = __popc(peers & ((1u << lane) - 1u));
        if (valid && rankInWarp == 0) warpCnt[warp][digit] = __popc(peers);
        __syncthreads();
        uint32_t total = 0;  // keys of digit tid in this pass; warpCnt becomes the prefix over warps
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t t = warpCnt[w][tid];
            warpCnt[w][tid] = total;
            total += t;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = base[digit] + warpCnt[warp][digit] + rankInWarp;
            staged[pos] = key;
            if (WithVals) stagedVals[pos] = val;
        }
        __syncthreads();
        base[tid] += total;
    }
    __syncthreads();
    for (uint32_t t = tid; t < tileTotal; t += kThreads) {
        const u64 key = staged[t];
        const unsigned d = unsigned(key >> shift) & (kRadix - 1);
        const uint32_t pos = globalStart[d] + (t - localStart[d]);
        keysOut[pos] = key;
        if (WithVals) valsOut[pos] = stagedVals[t];
    }
}

// ---- exclusive scan ----
__device__ __forceinline__ uint32_t blockExclusiveScan(uint32_t v, uint32_t* sh, uint32_t& blockTotal)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < warps ? sh[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < warps) sh[lane] = s;  // inclusive prefix of warp totals
    }
    __syncthreads();
    blockTotal = sh[warps - 1];
    const uint32_t warpBase = warp > 0 ? sh[warp - 1] : 0u;
    __syncthreads();  // sh is reused by the caller's next scan
    return warpBase + x - v;
}

__global__ void __launch_bounds__(kThreads) scanReduceKernel(const uint32_t* __restrict__ in, int64_t n,
                                                             uint32_t* __restrict__ partial)
{
    __shared__ uint32_t sh[32];
    const int64_t start = int64_t(blockIdx.x) * kTile + int64_t(threadIdx.x) * kItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k)
        if (start + k < n) s += in[start + k];
    uint32_t total;
    blockExclusiveScan(s, sh, total);
    if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

// one block: exclusive scan of the tile sums in place, in chunks of blockDim with a carry
__global__ void scanPartialsKernel(uint32_t* __restrict__ partial, int64_t tiles)
{
    __shared__ uint32_t sh[32];
    uint32_t carry = 0;
    for (int64_t c0 = 0; c0 < tiles; c0 += blockDim.x) {
        const int64_t i = c0 + threadIdx.x;
        const uint32_t v = i < tiles ? partial[i] : 0u;
        uint32_t total;
        const uint32_t ex = blockExclusiveScan(v, sh, total);
        if (i < tiles) partial[i] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(kThreads) scanDownKernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                           int64_t n, const uint32_t* __restrict__ partial)
{
    __shared__ uint32_t sh[32];
    const int64_t start = int64_t(blockIdx.x) * kTile + int64_t(threadIdx.x) * kItems;
    uint32_t v[kItems], s = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        v[k] = start + k < n ? in[start + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = partial[blockIdx.x] + blockExclusiveScan(s, sh, total);
#pragma unroll
    for (int k = 0; k < kItems; ++k)
        if (start + k < n) {
            out[start + k] = run;
            run += v[k];
        }
}

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

int exclusiveScan(sphgb_ctx* c, const uint32_t* in, uint32_t* out, int64_t n, uint32_t* scratch)
{
    if (n <= 0) return SPHGB_OK;
    if (n >= (int64_t(1) << 32)) return SPHGB_ERR_TOO_LARGE;
    const int64_t tiles = (n + kTile - 1) / kTile;
    scanReduceKernel<<<unsigned(tiles), kThreads, 0, c->stream>>>(in, n, scratch);
    SPHGB_TRY(launched(c, "scanReduceKernel"));
    scanPartialsKernel<<<1, 1024, 0, c->stream>>>(scratch, tiles);
    SPHGB_TRY(launched(c, "scanPartialsKernel"));
    scanDownKernel<<<unsigned(tiles), kThreads, 0, c->stream>>>(in, out, n, scratch);
    return launched(c, "scanDownKernel");
}

size_t scanScratchBytes(int64_t n) { return sizeof(uint32_t) * size_t((n + kTile - 1) / kTile + 1); }

int exclusiveScan(sphgb_ctx* c, const uint32_t* in, uint32_t* out, int64_t n)
{
    SPHGB_TRY(c->scanTemp.ensure(scanScratchBytes(n)));
    return exclusiveScan(c, in, out, n, c->scanTemp.as<uint32_t>());
}

int radixSort(sphgb_ctx* c, const u64* keysIn, u64* keysOut, const uint32_t* valsIn, uint32_t* valsOut, int64_t n,
              int endBit)
{
    if (n <= 0) return SPHGB_OK;
    if (endBit < 1 || endBit > 64 || (valsIn == nullptr) != (valsOut == nullptr)) return SPHGB_ERR_ARG;
    if (n >= (int64_t(1) << 32)) return SPHGB_ERR_TOO_LARGE;  // output slots are 32-bit
    cudaStream_t st = c->stream;
    if (n == 1) {
        SPHGB_CUDA(cudaMemcpyAsync(keysOut, keysIn, sizeof(u64), cudaMemcpyDeviceToDevice, st));
        if (valsIn) SPHGB_CUDA(cudaMemcpyAsync(valsOut, valsIn, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
        return SPHGB_OK;
    }
    const bool withVals = valsIn != nullptr;
    const int64_t tiles = (n + kTile - 1) / kTile;
    const int64_t cells = int64_t(kRadix) * tiles;
    // scratch: ping-pong keys (and values), digit counts, their offsets, scan partials
    const size_t bKeys = align256(sizeof(u64) * n), bVals = withVals ? align256(sizeof(uint32_t) * n) : 0;
    const size_t bCells = align256(sizeof(uint32_t) * cells);
    const size_t bScan = align256(scanScratchBytes(cells));
    SPHGB_TRY(c->sortTemp.ensure(bKeys + bVals + 2 * bCells + bScan));
    char* base = c->sortTemp.as<char>();
    u64* keysTmp = reinterpret_cast<u64*>(base);
    uint32_t* valsTmp = withVals ? reinterpret_cast<uint32_t*>(base + bKeys) : nullptr;
    uint32_t* counts = reinterpret_cast<uint32_t*>(base + bKeys + bVals);
    uint32_t* offsets = reinterpret_cast<uint32_t*>(base + bKeys + bVals + bCells);
    uint32_t* scan = reinterpret_cast<uint32_t*>(base + bKeys + bVals + 2 * bCells);

    if (!c->sortSmemSet) {  // the staged tile of (key, value) pairs exceeds the default 48 KB
        SPHGB_CUDA(cudaFuncSetAttribute(radixScatterKernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        int(kStagePairs)));
        SPHGB_CUDA(cudaFuncSetAttribute(radixScatterKernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        int(kStageKeys)));
        c->sortSmemSet = true;
    }
    const int passes = (endBit + 7) / 8;
    const u64* kSrc = keysIn;
    const uint32_t* vSrc = valsIn;
    for (int pass = 0; pass < passes; ++pass) {
        // the last pass writes the output buffers
        const bool toOut = ((passes - 1 - pass) & 1) == 0;
        u64* kDst = toOut ? keysOut : keysTmp;
        uint32_t* vDst = toOut ? valsOut : valsTmp;
        const int shift = 8 * pass;
        radixHistKernel<<<unsigned(tiles), kThreads, 0, st>>>(kSrc, n, shift, tiles, counts);
        SPHGB_TRY(launched(c, "radixHistKernel"));
        SPHGB_TRY(exclusiveScan(c, counts, offsets, cells, scan));
        if (withVals)
            radixScatterKernel<true><<<unsigned(tiles), kThreads, kStagePairs, st>>>(kSrc, vSrc, kDst, vDst, n, shift,
                                                                                    tiles, counts, offsets);
        else
            radixScatterKernel<false><<<unsigned(tiles), kThreads, kStageKeys, st>>>(kSrc, nullptr, kDst, nullptr, n,
                                                                                    shift, tiles, counts, offsets);
        SPHGB_TRY(launched(c, "radixScatterKernel"));
        kSrc = kDst;
        vSrc = vDst;
    }
    return SPHGB_OK;
}

}  // namespace sphgb
