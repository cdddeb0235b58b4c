// Stable LSD radix sort of 64-bit keys (with optional 32-bit values) and exclusive prefix sum of
// 32-bit counts: the sort of (SFC key, index) pairs behind the reference's sort_by_key
// (domain/include/cstone/primitives/gather.hpp:43-74, primitives_gpu.cu:323-340), the tree's key
// sorts, the adjoint's pair sort and the count scans.
//
// Sort: 8-bit digits, one scatter launch per digit with decoupled look-back between tiles:
//   allDigitsHist   one read of the keys: the digit histograms of every pass at once
//   digitPlan       one block: per pass the exclusive prefix over the 256 digits, which passes
//                   have more than one populated digit (the others are skipped), each pass's
//                   source and destination buffer, a fresh epoch per pass and its tile tickets
//   onesweep        per pass, tiles of 4096 keys in ticket order.  Each warp ranks its 512
//                   consecutive keys per digit (warp match, warp-private counters); the block
//                   turns the per-warp counts into per-digit tile counts, publishes them, and
//                   looks back over the preceding tiles' published counts for its global slot of
//                   each digit (a tile publishes its inclusive prefix once it has it, so a
//                   look-back stops at the first tile that has).  The tile is staged in shared
//                   memory grouped by digit and written out in runs: equal digits keep their input
//                   order, so every pass, and the sort, is stable.
// A tile waits only on tiles that drew earlier tickets, which are already resident, so the
// look-back always ends; its spin is bounded all the same and a give-up raises the context's
// sort flag (read by sortStatus) instead of hanging.
// Scan: per-tile sums, one block scanning the sums, per-tile scan with its base.
#include "context.cuh"

namespace sphgb {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;
constexpr int kWarps = kThreads / 32;
constexpr int kWarpKeys = 32 * kItems;
constexpr int kRadix = 256;
constexpr int kMaxPasses = 8;
constexpr size_t kStageKeys = sizeof(u64) * kTile, kStagePairs = (sizeof(u64) + sizeof(uint32_t)) * kTile;

// sortState words: [0] give-up flag, [1] epoch counter, then per pass: epoch, ticket, source
// buffer (0 input, 1 temporary, 2 output), destination buffer (1 or 2, or 3: pass skipped)
constexpr int kFlag = 0, kCounter = 1, kEpoch = 2, kTicket = kEpoch + kMaxPasses, kSrc = kTicket + kMaxPasses,
              kDst = kSrc + kMaxPasses, kStateWords = kDst + kMaxPasses;
constexpr uint32_t kSkip = 3;
// look-back words: epoch << 34 | kind << 32 | count, kind 1 = this tile's count, 2 = inclusive prefix
constexpr uint32_t kEpochMod = (1u << 30) - 1;
constexpr u64 kTileCount = 1, kInclusive = 2;
constexpr uint32_t kSpinLimit = 1u << 20;
constexpr int kWindow = 16;  // look-back words read per round trip

__device__ __forceinline__ u64 loadRelaxed(const u64* p)
{
    u64 v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void storeRelaxed(u64* p, u64 v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint32_t loadRelaxed32(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// digit histograms of passes [0, passes) over all keys; a warp whose 32 keys share a digit adds
// them with one atomic (sorted or nearly sorted input would otherwise serialise on one counter)
__global__ void __launch_bounds__(kThreads) allDigitsHist(const u64* __restrict__ keys, int64_t n, int passes,
                                                          uint32_t* __restrict__ hist)
{
    __shared__ uint32_t h[kMaxPasses][kRadix];
    for (int p = 0; p < kMaxPasses; ++p) h[p][threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t stride = int64_t(gridDim.x) * kThreads;
    for (int64_t w0 = int64_t(blockIdx.x) * kThreads + (threadIdx.x & ~31); w0 < n; w0 += stride) {
        const int64_t i = w0 + lane;
        const bool valid = i < n;
        const u64 key = valid ? keys[i] : 0;
        const unsigned vm = __ballot_sync(0xffffffffu, valid);
#pragma unroll
        for (int p = 0; p < kMaxPasses; ++p) {
            if (p >= passes) break;
            const unsigned d = unsigned(key >> (8 * p)) & (kRadix - 1);
            const unsigned d0 = __shfl_sync(0xffffffffu, d, 0);
            if (__all_sync(0xffffffffu, !valid || d == d0)) {
                if (lane == 0) atomicAdd(&h[p][d0], unsigned(__popc(vm)));
            } else if (valid) {
                atomicAdd(&h[p][d], 1u);
            }
        }
    }
    __syncthreads();
    for (int p = 0; p < passes; ++p)
        if (h[p][threadIdx.x]) atomicAdd(hist + p * kRadix + threadIdx.x, h[p][threadIdx.x]);
}

__device__ __forceinline__ uint32_t blockExclusiveScan(uint32_t v, uint32_t* sh, uint32_t& blockTotal);

// one block of kRadix threads: digit starts per pass, the pass plan, epochs and tickets
__global__ void __launch_bounds__(kRadix) digitPlan(uint32_t* __restrict__ hist, int passes, int64_t n,
                                                    uint32_t* __restrict__ state)
{
    __shared__ uint32_t sh[32];
    __shared__ int active[kMaxPasses];
    for (int p = 0; p < passes; ++p) {
        const uint32_t v = hist[p * kRadix + threadIdx.x];
        uint32_t total;
        const uint32_t ex = blockExclusiveScan(v, sh, total);
        // a pass whose keys all share one digit moves nothing
        const int trivial = __syncthreads_or(uint64_t(v) == uint64_t(n));
        hist[p * kRadix + threadIdx.x] = ex;
        if (threadIdx.x == 0) active[p] = !trivial;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int count = 0;
        for (int p = 0; p < passes; ++p) count += active[p];
        if (count == 0) {  // every key equal: one pass still copies input to output
            active[0] = 1;
            count = 1;
        }
        const uint32_t e0 = state[kCounter];
        state[kCounter] = (e0 + uint32_t(passes)) % kEpochMod;
        // the k-th of `count` active passes reads the previous active pass's output and writes the
        // output buffer when count-1-k is even, so the last one always does
        uint32_t src = 0;
        int k = 0;
        for (int p = 0; p < kMaxPasses; ++p) {
            state[kEpoch + p] = 1u + (e0 + uint32_t(p)) % kEpochMod;
            state[kTicket + p] = 0;
            if (p < passes && active[p]) {
                const uint32_t dst = ((count - 1 - k) & 1) == 0 ? 2u : 1u;
                state[kSrc + p] = src;
                state[kDst + p] = dst;
                src = dst;
                ++k;
            } else {
                state[kSrc + p] = 0;
                state[kDst + p] = kSkip;
            }
        }
    }
}

template<bool WithVals>
__global__ void __launch_bounds__(kThreads, 3) onesweep(const u64* keysIn, const uint32_t* valsIn, u64* keysTmp,
                                                     uint32_t* valsTmp, u64* keysOut, uint32_t* valsOut,
                                                     int64_t n, int pass, const uint32_t* __restrict__ digitStart,
                                                     u64* __restrict__ look, uint32_t* __restrict__ state)
{
    extern __shared__ u64 staged[];  // kTile keys, then kTile values
    uint32_t* stagedVals = reinterpret_cast<uint32_t*>(staged + kTile);
    __shared__ uint32_t warpCnt[kWarps][kRadix];
    __shared__ uint32_t localStart[kRadix], globalStart[kRadix];
    __shared__ uint32_t sh[32];
    __shared__ uint32_t tileSh;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t dstSel = state[kDst + pass];
    if (dstSel == kSkip) return;  // uniform across the grid
    const uint32_t srcSel = state[kSrc + pass];
    const u64* kSrc = srcSel == 0 ? keysIn : srcSel == 1 ? keysTmp : keysOut;
    const uint32_t* vSrc = srcSel == 0 ? valsIn : srcSel == 1 ? valsTmp : valsOut;
    u64* kDst = dstSel == 1 ? keysTmp : keysOut;
    uint32_t* vDst = dstSel == 1 ? valsTmp : valsOut;
    const int shift = 8 * pass;
    const uint32_t epoch = state[kEpoch + pass];

    if (tid == 0) tileSh = atomicAdd(state + kTicket + pass, 1u);
#pragma unroll
    for (int w = 0; w < kWarps; ++w) warpCnt[w][tid] = 0;
    __syncthreads();
    const uint32_t tile = tileSh;

    // rank each warp's 512 consecutive keys per digit in index order
    const int64_t wBase = int64_t(tile) * kTile + int64_t(warp) * kWarpKeys;
    u64 key[kItems];
    uint32_t val[kItems], rank[kItems];
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const int64_t i = wBase + r * 32 + lane;
        const bool valid = i < n;
        key[r] = valid ? kSrc[i] : 0;
        if (WithVals) val[r] = valid ? vSrc[i] : 0u;
        const unsigned d = valid ? (unsigned(key[r] >> shift) & (kRadix - 1)) : unsigned(kRadix);
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = 0;
        if (valid) before = warpCnt[warp][d];
        __syncwarp();
        if (valid && (peers & lt) == 0) warpCnt[warp][d] = before + __popc(peers);
        __syncwarp();
        rank[r] = valid ? (d | ((before + __popc(peers & lt)) << 8)) : 0xffffffffu;
    }
    __syncthreads();

    // thread tid owns digit tid: prefix over warps, tile count, tile-local start
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        const uint32_t t = warpCnt[w][tid];
        warpCnt[w][tid] = cnt;
        cnt += t;
    }
    uint32_t tileTotal;
    localStart[tid] = blockExclusiveScan(cnt, sh, tileTotal);

    // publish this tile's count (its inclusive prefix right away for the first tile)
    const u64 tag = u64(epoch) << 34;
    u64* mine = look + int64_t(tile) * kRadix + tid;
    storeRelaxed(mine, tag | ((tile == 0 ? kInclusive : kTileCount) << 32) | cnt);
    __syncthreads();

    // stage the tile grouped by digit (the keys' registers are free for the look-back)
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        if (rank[r] == 0xffffffffu) continue;
        const unsigned d = rank[r] & (kRadix - 1);
        const uint32_t pos = localStart[d] + warpCnt[warp][d] + (rank[r] >> 8);
        staged[pos] = key[r];
        if (WithVals) stagedVals[pos] = val[r];
    }

    // look back over the preceding tiles' words of digit tid, kWindow tiles per round trip: add
    // tile counts until a tile's inclusive prefix; a tile that has not published yet is polled
    // again (bounded), the ones after it already summed are not read twice
    uint32_t excl = 0;
    if (tile > 0) {
        int64_t p = int64_t(tile) - 1;
        uint32_t spins = 0;
        bool gaveUp = false;
        while (true) {
            u64 w[kWindow];
#pragma unroll
            for (int q = 0; q < kWindow; ++q)
                w[q] = p - q >= 0 ? loadRelaxed(look + (p - q) * kRadix + tid) : (tag | (kInclusive << 32));
            int used = 0;
            bool done = false;
#pragma unroll
            for (int q = 0; q < kWindow; ++q) {
                if (done || used < q || uint32_t(w[q] >> 34) != epoch) continue;
                excl += uint32_t(w[q]);
                used = q + 1;
                done = ((w[q] >> 32) & 3u) == kInclusive;
            }
            if (done) break;
            p -= used;
            if (used == 0) {  // the nearest unread tile has not published yet
                if (++spins >= kSpinLimit || ((spins & 1023u) == 0 && loadRelaxed32(state + kFlag) != 0u)) {
                    gaveUp = true;
                    break;
                }
                __nanosleep(64);
            }
        }
        if (gaveUp) atomicOr(state + kFlag, 1u);  // gave up: flag the sort, stop waiting
        storeRelaxed(mine, tag | (kInclusive << 32) | (excl + cnt));
    }
    globalStart[tid] = digitStart[pass * kRadix + tid] + excl;
    __syncthreads();

    // write each digit's run to its global slots
    for (uint32_t t = tid; t < tileTotal; t += kThreads) {
        const u64 k = staged[t];
        const unsigned d = unsigned(k >> shift) & (kRadix - 1);
        const uint32_t pos = globalStart[d] + (t - localStart[d]);
        kDst[pos] = k;
        if (WithVals) vDst[pos] = stagedVals[t];
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

// grows a buffer whose contents must start at zero (look-back words, sort state)
static int ensureZeroed(sphgb_ctx* c, DBuf& b, size_t need)
{
    const bool grows = b.p == nullptr || need > b.bytes;
    SPHGB_TRY(b.ensure(need));
    if (grows) SPHGB_CUDA(cudaMemsetAsync(b.p, 0, b.bytes, c->stream));
    return SPHGB_OK;
}

int radixSort(sphgb_ctx* c, const u64* keysIn, u64* keysOut, const uint32_t* valsIn, uint32_t* valsOut, int64_t n,
              int endBit)
{
    if (n <= 0) return SPHGB_OK;
    if (endBit < 1 || endBit > 64 || (valsIn == nullptr) != (valsOut == nullptr)) return SPHGB_ERR_ARG;
    if (n >= (int64_t(1) << 32)) return SPHGB_ERR_TOO_LARGE;  // slots and counts are 32-bit
    cudaStream_t st = c->stream;
    if (n == 1) {
        SPHGB_CUDA(cudaMemcpyAsync(keysOut, keysIn, sizeof(u64), cudaMemcpyDeviceToDevice, st));
        if (valsIn) SPHGB_CUDA(cudaMemcpyAsync(valsOut, valsIn, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
        return SPHGB_OK;
    }
    const bool withVals = valsIn != nullptr;
    const int passes = (endBit + 7) / 8;
    const int64_t tiles = (n + kTile - 1) / kTile;
    // scratch: ping-pong keys (and values), digit histograms; look-back words; sort state
    const size_t bKeys = align256(sizeof(u64) * n), bVals = withVals ? align256(sizeof(uint32_t) * n) : 0;
    SPHGB_TRY(c->sortTemp.ensure(bKeys + bVals + sizeof(uint32_t) * kMaxPasses * kRadix));
    char* base = c->sortTemp.as<char>();
    u64* keysTmp = reinterpret_cast<u64*>(base);
    uint32_t* valsTmp = withVals ? reinterpret_cast<uint32_t*>(base + bKeys) : nullptr;
    uint32_t* hist = reinterpret_cast<uint32_t*>(base + bKeys + bVals);
    SPHGB_TRY(ensureZeroed(c, c->sortLook, sizeof(u64) * kRadix * size_t(tiles)));
    SPHGB_TRY(ensureZeroed(c, c->sortState, sizeof(uint32_t) * kStateWords));
    uint32_t* state = c->sortState.as<uint32_t>();

    if (!c->sortSmemSet) {  // the staged tile of (key, value) pairs exceeds the default 48 KB
        SPHGB_CUDA(cudaFuncSetAttribute(onesweep<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        int(kStagePairs)));
        SPHGB_CUDA(cudaFuncSetAttribute(onesweep<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        int(kStageKeys)));
        c->sortSmemSet = true;
    }
    SPHGB_CUDA(cudaMemsetAsync(hist, 0, sizeof(uint32_t) * kMaxPasses * kRadix, st));
    const unsigned histBlocks = unsigned(tiles < 8 * 152 ? tiles : 8 * 152);
    allDigitsHist<<<histBlocks, kThreads, 0, st>>>(keysIn, n, passes, hist);
    SPHGB_TRY(launched(c, "allDigitsHist"));
    digitPlan<<<1, kRadix, 0, st>>>(hist, passes, n, state);
    SPHGB_TRY(launched(c, "digitPlan"));
    for (int pass = 0; pass < passes; ++pass) {
        if (withVals)
            onesweep<true><<<unsigned(tiles), kThreads, kStagePairs, st>>>(keysIn, valsIn, keysTmp, valsTmp, keysOut,
                                                                           valsOut, n, pass, hist, c->sortLook.as<u64>(),
                                                                           state);
        else
            onesweep<false><<<unsigned(tiles), kThreads, kStageKeys, st>>>(keysIn, nullptr, keysTmp, nullptr, keysOut,
                                                                           nullptr, n, pass, hist,
                                                                           c->sortLook.as<u64>(), state);
        SPHGB_TRY(launched(c, "onesweep"));
    }
    return SPHGB_OK;
}

int sortStatusAsync(sphgb_ctx* c)
{
    if (!c->sortState.p) return SPHGB_OK;
    SPHGB_CUDA(cudaMemcpyAsync(&c->sortFlagHost, c->sortState.as<uint32_t>() + kFlag, sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, c->stream));
    c->sortFlagPending = true;
    return SPHGB_OK;
}

int sortStatusAfterSync(sphgb_ctx* c)
{
    if (!c->sortFlagPending) return SPHGB_OK;
    c->sortFlagPending = false;
    if (c->sortFlagHost == 0) return SPHGB_OK;
    c->sortFlagHost = 0;
    SPHGB_CUDA(cudaMemsetAsync(c->sortState.as<uint32_t>() + kFlag, 0, sizeof(uint32_t), c->stream));
    return SPHGB_ERR_TIMEOUT;
}

}  // namespace sphgb
