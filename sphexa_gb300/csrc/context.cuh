// Internal state of an sphgb context and the helpers every translation unit uses.
#pragma once

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

namespace sphgb {

// last CUDA error text, readable through sphgb_last_cuda_error()
void setCudaError(cudaError_t e, const char* what);

#define SPHGB_CUDA(call)                                   \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) {                           \
            ::sphgb::setCudaError(e_, #call);              \
            return SPHGB_ERR_CUDA;                         \
        }                                                  \
    } while (0)

#define SPHGB_TRY(call)                      \
    do {                                     \
        int s_ = (call);                     \
        if (s_ != SPHGB_OK) return s_;       \
    } while (0)

// growable device buffer
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    int ensure(size_t need)
    {
        if (need <= bytes && p) return SPHGB_OK;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        size_t alloc = need < 256 ? 256 : need;
        cudaError_t e = cudaMalloc(&p, alloc);
        if (e != cudaSuccess) {
            setCudaError(e, "cudaMalloc");
            p = nullptr;
            return SPHGB_ERR_ALLOC;
        }
        bytes = alloc;
        return SPHGB_OK;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template<class T>
    T* as() const
    {
        return static_cast<T*>(p);
    }
};

enum Stage { kStageSync = 0, kStageNbr = 1, kStagePass0 = 2, kNumStages = 8 };

}  // namespace sphgb

struct sphgb_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    sphgb_params prm{};
    double K = 0.0;
    bool tablesReady = false;

    sphgb::DevBox box{};
    sphgb_box hbox{};
    bool haveBox = false;
    int64_t n = 0;

    // domain sync
    sphgb::DBuf keys, keysAlt, order, orderAlt, sortTemp, gatherScratch, minmax;
    bool haveSync = false;

    // cornerstone tree and octree
    int64_t numLeaves = 0, numInternal = 0, numNodes = 0;
    int32_t levelRange[sphgb::kMaxLevel + 2] = {};
    sphgb::DBuf splitCount, splitOffset, leafKeysTmp, internalTmp, internalCodes;
    sphgb::DBuf leaves, layout, prefixes, childOffsets, internalToLeaf;
    sphgb::DBuf nodeCenter, nodeSize;   // double3-packed, 3 doubles per node (reference nodeFpCenters)
    sphgb::DBuf nodeBoxF;               // float4 {cx, cy, cz, pad} + float4 {sx, sy, sz, -}: traversal
    sphgb::DBuf nodeRange;              // uint2 per node: its particles [start, end) in SFC order
    sphgb::DBuf levelRangeDev;
    bool haveTree = false;

    // neighbour lists in granules of four entries, transposed per granule (listSlot in pairs.cuh)
    int64_t nbrFirst = 0, nbrLast = 0, nbrStride = 0;
    uint32_t nbrNgmax = 0;
    sphgb::DBuf nbr, ncount, active, counters;
    bool haveNbr = false;
    // owned pair lists of the pair-once passes, in the granule layout of the lists (listSlot): entry
    // j | mutual << 31 for the pairs i evaluates, ownedCount per particle; valid for epoch ownedEpoch
    sphgb::DBuf owned, ownedCount, ownedR2;
    int64_t ownedEpoch = -1;
    bool ownedFromLists = false;  // owned lists decided from list membership (mixed adjoint); the FP64 passes skip them
    // summation mode of the FP64 passes (order-fixed, or one evaluation per mutual pair) and the
    // per-particle accumulators of the pair-once passes (up to 6 x n doubles)
    bool deterministic = false;
    sphgb::DBuf pairAcc;
    // within one sweep: |r|, 1/|r| and the kernel function at both ends of every owned entry, stored
    // by the pair-once xmass pass and read by the later pair-once passes of the same sweep (PairGeo in
    // pairs.cuh); geoRows: per warp of 32 targets its longest owned list, then its first row
    sphgb::DBuf pairGeo, geoRows;
    size_t geoRowCount = 0;
    int geoArrays = 0;  // 5: with the difference and velocity-difference vectors, 2: without
    bool geoValid = false;
    // inside sphgb_sweep_passes the per-particle precomputes are built by the first pass only
    bool inSweep = false, sweepPrepared = false;
    // within one sweep: the EOS ran in the gradh epilogue / the per-particle quotients are formed
    bool eosFused = false, auxReady = false;
    // packed neighbour-side records of the mixed pair passes (float4 x 4 per particle)
    sphgb::DBuf pack;
    // forward tape of the VE adjoint: with tapeOn the FP64 VE passes over all particles keep the
    // per-particle sums the adjoint needs (kTape* sections x n doubles); tapeMask tells which passes
    // wrote theirs on the lists of epoch tapeEpoch for tapeN particles
    bool tapeOn = false;
    sphgb::DBuf veTape;
    int64_t tapeEpoch = -1, tapeN = 0;
    unsigned tapeMask = 0;
    // mixed form: FP64 refinement of ill-conditioned particles (masks, FP64 xm/kx/gradh scratch,
    // divv error bound per particle) and the counts of the last passes
    bool refineMixed = true;
    sphgb::DBuf refMask, refFp64, divvBound;
    int64_t stats_refinedGradh = 0, stats_refinedDivv = 0;
    // block partials of the integration-step reductions
    sphgb::DBuf intScratch;
    // domain mode: 0 every sync stands alone; 1 the syncs are the steps of one simulation (the box
    // of a later sync is limited in how far it shrinks against the previous one)
    int domainMode = 0;
    bool domainFirst = true;
    sphgb_box prevBox{};
    int precisionBuilt = -1;
    const double* xBuilt = nullptr;

    // kernel tables W and dW/dv, FP64 and FP32, interleaved {t[k], t[k+1] - t[k]}
    sphgb::DBuf whx64, whdx64;
    // smooth form of the FP64 kernel function (sphgb_set_kernel_form): cubic Hermite pieces of W and
    // dW/dv on the table's intervals, {c0 c1} {c2 c3} per interval; used when smoothKernel is set
    sphgb::DBuf whS64, whdS64;
    bool smoothKernel = false;
    sphgb::DBuf whx32;  // FP32 linear table (the mixed adjoint)
    sphgb::DBuf whH32, whdH32;  // mixed passes: cubic pieces of W and dW/dv (kHermIntervals float4)

    // mixed precision grid-local coordinates: packed cell (21 bits per axis) + float4 {dx,dy,dz,1/h}
    sphgb::DBuf gridKey, gridLoc;
    // per-particle reciprocals reused by the FP64 passes: [0,n) 1/h, [n,2n) 1/h^3 (same IEEE
    // results as the in-loop divisions of the reference)
    sphgb::DBuf hInv64;
    // per-particle quotients of pass inputs, rebuilt at the start of every pass that reads them
    // (VE: rho, m/rho, xm/kx, m*prho, ln xm; std: m/rho, p/rho, p/rho^2)
    sphgb::DBuf aux;
    // adjoint: incoming lists as CSR (tOff, tIdx) built from sorted (j<<32|i) keys, and the
    // per-particle adjoint state of the intermediate fields
    sphgb::DBuf adjKeys, adjKeysAlt, tOff, tIdx, adjState;
    sphgb::DBuf scanTemp;  // tile sums of exclusiveScan
    bool sortSmemSet = false;
    // radix sort: look-back words (256 per tile) and state (give-up flag, epochs, tickets, plan);
    // the flag is read back by sortStatusAsync / sortStatusAfterSync around a stream sync
    sphgb::DBuf sortLook, sortState;
    uint32_t sortFlagHost = 0;
    bool sortFlagPending = false;
    int64_t transEpoch = -1, transPairs = 0;
    // validity of the precomputes: the lists' epoch and the field pointers they were made from
    int64_t nbrEpoch = 0, prepEpoch = -1, prepEpoch64 = -1;
    const void* prepMixedFor = nullptr;
    const void* prepMixedH = nullptr;
    const void* prepFp64H = nullptr;
    sphgb::DBuf reduceScratch;

    // device status word and small counters
    int* dFlags = nullptr;
    // input validation word (validate.cu); inputsChecked: the fields were validated within the
    // current sphgb_sweep call and cannot have changed since
    sphgb::DBuf checkWord;
    bool inputsChecked = false;

    // statistics and timing
    sphgb_stats stats{};
    cudaEvent_t ev[2 * sphgb::kNumStages] = {};
    float stageMs[sphgb::kNumStages] = {};
    int64_t launches = 0;
};

namespace sphgb {

// per-translation-unit entry points used by capi.cu
int domainSync(sphgb_ctx* c, sphgb_particles* p, sphgb_box* box);
int applyOrder(sphgb_ctx* c, void* field, int esz);
int buildTree(sphgb_ctx* c, bool rebalance);
int buildTables(sphgb_ctx* c);
int findNeighborsSph(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last);
// SPHGB_ERR_INPUT when a coordinate of [0, n) is not finite or h (if non-null) is not finite or <= 0
int validateParticles(sphgb_ctx* c, const double* x, const double* y, const double* z, const void* h, int hIsFloat,
                      int64_t n);
int findNeighborsFixed(sphgb_ctx* c, const double* x, const double* y, const double* z, const void* h,
                       int32_t hPrec, int64_t first, int64_t last, uint32_t ngmax, uint32_t* nbrOut, uint32_t* ncOut);
int exportNeighbors(sphgb_ctx* c, uint32_t* out);
int prepareMixed(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last);
int prepareFp64(sphgb_ctx* c, sphgb_particles* p);

int passDensity(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last);
int passEosStd(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last);
int passIadStd(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last);
int passMomentumEnergyStd(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last, double* minDt);
int passXMass(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last);
int passGradh(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last);
int passEosVe(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last);
int passIadDivvCurlv(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last);
int passAVswitches(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last);
int passMomentumEnergyVe(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last, int avClean, float* groupDt,
                         double* minDt);

int buildTranspose(sphgb_ctx* c);
// owned lists of the current lists from list membership (mixed adjoint)
int buildOwnedFromLists(sphgb_ctx* c);
// stable LSD radix sort of 64-bit keys (bits [0, endBit)) with optional 32-bit values, out of place
int radixSort(sphgb_ctx* c, const u64* keysIn, u64* keysOut, const uint32_t* valsIn, uint32_t* valsOut, int64_t n,
              int endBit);
// the radix sort's give-up flag: queue its copy to the host before a stream sync, test it after
// (SPHGB_ERR_TIMEOUT when a look-back wait gave up; the flag is then cleared)
int sortStatusAsync(sphgb_ctx* c);
int sortStatusAfterSync(sphgb_ctx* c);
// exclusive prefix sum of n 32-bit counts (out may not alias in)
int exclusiveScan(sphgb_ctx* c, const uint32_t* in, uint32_t* out, int64_t n);
int adjointStd(sphgb_ctx* c, sphgb_particles* p, const sphgb_seeds* s, sphgb_grads* g, int deterministic);
int adjointVe(sphgb_ctx* c, sphgb_particles* p, const double* alphaPrev, int avClean, const sphgb_seeds* s,
              sphgb_grads* g, int deterministic);
int refineMixedGradh(sphgb_ctx* c, sphgb_particles* p);
int refineMixedDivv(sphgb_ctx* c, sphgb_particles* p, const float* bound);

// min-reduction of per-block Courant dt partials into one double on the host
int reduceMinDt(sphgb_ctx* c, const double* partials, int count, double* out);

inline unsigned gridFor(int64_t work, int block) { return unsigned((work + block - 1) / block); }

// launch bookkeeping: count one kernel launch and check the launch error
inline int launched(sphgb_ctx* c, const char* what)
{
    c->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        setCudaError(e, what);
        return SPHGB_ERR_CUDA;
    }
    return SPHGB_OK;
}

}  // namespace sphgb
