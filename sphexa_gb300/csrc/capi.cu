// C ABI of the sphgb sweep (include/sphgb.h).  Every entry point validates its arguments,
// selects the context's device, runs on the context's stream and returns an sphgb_status;
// no C++ exception crosses the boundary.
#include <cstdio>
#include <mutex>
#include <new>

#include "pairs.cuh"

namespace sphgb {

namespace {
thread_local char gCudaError[256] = "";
}

void setCudaError(cudaError_t e, const char* what)
{
    std::snprintf(gCudaError, sizeof(gCudaError), "%s: %s (%d)", what, cudaGetErrorString(e), int(e));
}

namespace {

int useDevice(sphgb_ctx* c)
{
    if (!c) return SPHGB_ERR_ARG;
    SPHGB_CUDA(cudaSetDevice(c->device));
    return SPHGB_OK;
}

// CUDA-event bracket of one stage on the context stream
struct StageTimer {
    sphgb_ctx* c;
    int stage;
    StageTimer(sphgb_ctx* ctx, int s) : c(ctx), stage(s) { cudaEventRecord(c->ev[2 * s], c->stream); }
    void stop()
    {
        cudaEventRecord(c->ev[2 * stage + 1], c->stream);
    }
};

void collectTimings(sphgb_ctx* c, int upto)
{
    for (int s = 0; s < upto; ++s) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c->ev[2 * s], c->ev[2 * s + 1]) == cudaSuccess) c->stageMs[s] = ms;
    }
}

// boundaries of the 32-particle target groups of [first, last): splits[g] = first + 32 g, splits[G] = last
__global__ void targetGroupsKernel(int64_t first, int64_t last, int64_t groups, uint32_t* __restrict__ splits)
{
    const int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (g > groups) return;
    splits[g] = uint32_t(g == groups ? last : first + int64_t(kWarp) * g);
}

int checkRange(const sphgb_particles* p, int64_t first, int64_t last)
{
    if (!p || first < 0 || last > p->n || first >= last) return SPHGB_ERR_ARG;
    return SPHGB_OK;
}

}  // namespace

// for the entry points in other translation units
int useDeviceOf(sphgb_ctx* c) { return useDevice(c); }
}  // namespace sphgb

using namespace sphgb;

extern "C" {

const char* sphgb_status_string(int s)
{
    switch (s) {
    case SPHGB_OK: return "ok";
    case SPHGB_ERR_ARG: return "invalid argument";
    case SPHGB_ERR_CUDA: return "CUDA runtime error";
    case SPHGB_ERR_ALLOC: return "device allocation failed";
    case SPHGB_ERR_STATE: return "call out of order";
    case SPHGB_ERR_TRAVERSAL: return "octree traversal stack overflow";
    case SPHGB_ERR_NOCONV: return "h / neighbour-count iteration did not converge for some particles";
    case SPHGB_ERR_NOTFOUND: return "no usable CUDA device";
    case SPHGB_ERR_TOO_LARGE: return "request exceeds a fixed capacity";
    case SPHGB_ERR_INPUT: return "non-finite coordinate, smoothing length or box limit, or h <= 0";
    case SPHGB_ERR_TIMEOUT: return "a bounded device wait gave up (radix sort look-back)";
    default: return "unknown status";
    }
}

const char* sphgb_last_cuda_error(void) { return sphgb::gCudaError; }

int sphgb_version(void) { return 100; }

int sphgb_default_params(sphgb_params* p)
{
    if (!p) return SPHGB_ERR_ARG;
    p->ng0 = 100;
    p->ngmax = 150;
    p->bucket = 64;
    p->gamma = 5.0 / 3.0;
    p->Kcour = 0.2;
    p->sincIndex = 6.0;
    p->alphamin = 0.05;
    p->alphamax = 1.0;
    p->decay_constant = 0.2;
    p->minDt = 1e-6;
    return SPHGB_OK;
}

int sphgb_create(sphgb_ctx** out, int device)
{
    if (!out) return SPHGB_ERR_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return SPHGB_ERR_NOTFOUND;
    if (device < 0 || device >= count) return SPHGB_ERR_ARG;
    SPHGB_CUDA(cudaSetDevice(device));
    sphgb_ctx* c = new (std::nothrow) sphgb_ctx();
    if (!c) return SPHGB_ERR_ALLOC;
    c->device = device;
    sphgb_default_params(&c->prm);
    cudaError_t e = cudaMalloc(&c->dFlags, sizeof(int));
    if (e != cudaSuccess) {
        setCudaError(e, "cudaMalloc");
        delete c;
        return SPHGB_ERR_ALLOC;
    }
    cudaMemset(c->dFlags, 0, sizeof(int));
    for (auto& ev : c->ev) cudaEventCreate(&ev);
    int s = buildTables(c);
    if (s != SPHGB_OK) {
        sphgb_destroy(c);
        return s;
    }
    *out = c;
    return SPHGB_OK;
}

int sphgb_destroy(sphgb_ctx* c)
{
    if (!c) return SPHGB_ERR_ARG;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    DBuf* bufs[] = {&c->keys,     &c->keysAlt,      &c->order,         &c->orderAlt,      &c->sortTemp,
                    &c->gatherScratch, &c->minmax,  &c->splitCount,    &c->splitOffset,   &c->leafKeysTmp,
                    &c->internalTmp,   &c->internalCodes, &c->leaves,  &c->layout,        &c->prefixes,
                    &c->childOffsets,  &c->internalToLeaf, &c->nodeCenter, &c->nodeSize,  &c->nodeBoxF,     &c->nodeRange,
                    &c->levelRangeDev, &c->nbr,     &c->ncount,        &c->active,        &c->counters,
                    &c->gridKey,
                    &c->gridLoc,  &c->hInv64,       &c->reduceScratch, &c->aux,         &c->adjKeys,
                    &c->adjKeysAlt, &c->tOff,       &c->tIdx,          &c->adjState,      &c->whx64,
                    &c->whdx64,     &c->owned,      &c->ownedCount, &c->ownedR2,    &c->pairAcc,    &c->pairGeo,    &c->geoRows,    &c->pack,       &c->whx32,     &c->whH32, &c->whdH32,    &c->refMask,
                    &c->refFp64,    &c->divvBound,  &c->intScratch, &c->scanTemp, &c->veTape,
                    &c->checkWord,  &c->whS64,      &c->whdS64,     &c->sortLook,   &c->sortState};
    for (DBuf* b : bufs) b->release();
    if (c->dFlags) cudaFree(c->dFlags);
    for (auto& ev : c->ev)
        if (ev) cudaEventDestroy(ev);
    delete c;
    return SPHGB_OK;
}

int sphgb_set_stream(sphgb_ctx* c, void* stream)
{
    SPHGB_TRY(useDevice(c));
    c->stream = static_cast<cudaStream_t>(stream);
    return SPHGB_OK;
}

int sphgb_set_params(sphgb_ctx* c, const sphgb_params* p)
{
    SPHGB_TRY(useDevice(c));
    if (!p || p->ngmax == 0 || p->bucket == 0 || p->ng0 == 0 || !(p->sincIndex > 0)) return SPHGB_ERR_ARG;
    bool tables = p->sincIndex != c->prm.sincIndex || !c->tablesReady;
    c->prm = *p;
    if (tables) SPHGB_TRY(buildTables(c));
    return SPHGB_OK;
}

int sphgb_set_deterministic(sphgb_ctx* c, int32_t on)
{
    if (!c || (on != 0 && on != 1)) return SPHGB_ERR_ARG;
    c->deterministic = on != 0;
    return SPHGB_OK;
}

int sphgb_set_adjoint_tape(sphgb_ctx* c, int32_t on)
{
    if (!c || (on != 0 && on != 1)) return SPHGB_ERR_ARG;
    c->tapeOn = on != 0;
    if (!c->tapeOn) {
        c->tapeMask = 0;
        c->veTape.release();
    }
    return SPHGB_OK;
}

int sphgb_set_domain_mode(sphgb_ctx* c, int32_t mode)
{
    if (!c || (mode != 0 && mode != 1)) return SPHGB_ERR_ARG;
    c->domainMode = mode;
    c->domainFirst = true;
    return SPHGB_OK;
}

int sphgb_set_kernel_form(sphgb_ctx* c, int32_t form)
{
    if (!c || (form != SPHGB_KERNEL_TABLE && form != SPHGB_KERNEL_SMOOTH)) return SPHGB_ERR_ARG;
    c->smoothKernel = form == SPHGB_KERNEL_SMOOTH;
    return SPHGB_OK;
}

int sphgb_set_mixed_refinement(sphgb_ctx* c, int32_t on)
{
    if (!c || (on != 0 && on != 1)) return SPHGB_ERR_ARG;
    c->refineMixed = on != 0;
    return SPHGB_OK;
}

int sphgb_get_kernel_K(sphgb_ctx* c, double* K)
{
    if (!c || !K) return SPHGB_ERR_ARG;
    *K = c->K;
    return SPHGB_OK;
}

int sphgb_domain_sync(sphgb_ctx* c, sphgb_particles* p, sphgb_box* box)
{
    SPHGB_TRY(useDevice(c));
    if (!p || !box) return SPHGB_ERR_ARG;
    if (p->precision != SPHGB_FP64 && p->precision != SPHGB_MIXED) return SPHGB_ERR_ARG;
    StageTimer t(c, kStageSync);
    int s = domainSync(c, p, box);
    t.stop();
    if (s == SPHGB_OK) {
        SPHGB_CUDA(cudaStreamSynchronize(c->stream));
        collectTimings(c, 1);
    }
    return s;
}

int sphgb_get_tree(sphgb_ctx* c, const uint64_t** leaves, const uint32_t** layout, const uint64_t** prefixes,
                   const int32_t** childOffsets, const int32_t** internalToLeaf, sphgb_stats* stats)
{
    if (!c) return SPHGB_ERR_ARG;
    if (!c->haveTree) return SPHGB_ERR_STATE;
    if (leaves) *leaves = reinterpret_cast<const uint64_t*>(c->leaves.p);
    if (layout) *layout = c->layout.as<uint32_t>();
    if (prefixes) *prefixes = reinterpret_cast<const uint64_t*>(c->prefixes.p);
    if (childOffsets) *childOffsets = c->childOffsets.as<int32_t>();
    if (internalToLeaf) *internalToLeaf = c->internalToLeaf.as<int32_t>();
    if (stats) *stats = c->stats;
    return SPHGB_OK;
}

int sphgb_get_octree_view(sphgb_ctx* c, sphgb_octree_view* v)
{
    if (!c || !v) return SPHGB_ERR_ARG;
    if (!c->haveTree) return SPHGB_ERR_STATE;
    v->num_leaf_nodes = c->numLeaves;
    v->num_nodes = c->numNodes;
    v->num_internal = c->numInternal;
    v->prefixes = reinterpret_cast<const uint64_t*>(c->prefixes.p);
    v->child_offsets = c->childOffsets.as<int32_t>();
    v->internal_to_leaf = c->internalToLeaf.as<int32_t>();
    // levelRangeDev holds the internal nodes' level starts, then the level ranges of all nodes
    v->level_range = c->levelRangeDev.as<int32_t>() + (kMaxLevel + 2);
    v->leaves = reinterpret_cast<const uint64_t*>(c->leaves.p);
    v->layout = c->layout.as<uint32_t>();
    v->centers = c->nodeCenter.as<double>();
    v->sizes = c->nodeSize.as<double>();
    int depth = 0;
    for (int l = 0; l <= kMaxLevel; ++l)
        if (c->levelRange[l + 1] > c->levelRange[l]) depth = l;
    v->max_depth = depth;
    return SPHGB_OK;
}

int sphgb_get_params(sphgb_ctx* c, sphgb_params* p)
{
    if (!c || !p) return SPHGB_ERR_ARG;
    *p = c->prm;
    return SPHGB_OK;
}

int sphgb_target_groups(sphgb_ctx* c, int64_t first, int64_t last, uint32_t* splits, int64_t capacity,
                        int64_t* numGroups)
{
    SPHGB_TRY(useDevice(c));
    if (!numGroups || first < 0 || last < first || last > int64_t(UINT32_MAX)) return SPHGB_ERR_ARG;
    const int64_t groups = (last - first + kWarp - 1) / kWarp;
    *numGroups = groups;
    if (!splits) return SPHGB_OK;
    if (capacity < groups + 1) return SPHGB_ERR_ARG;
    targetGroupsKernel<<<gridFor(groups + 1, 256), 256, 0, c->stream>>>(first, last, groups, splits);
    SPHGB_TRY(launched(c, "targetGroupsKernel"));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    return SPHGB_OK;
}

int sphgb_get_order(sphgb_ctx* c, const uint32_t** order)
{
    if (!c || !order) return SPHGB_ERR_ARG;
    if (!c->haveSync) return SPHGB_ERR_STATE;
    *order = c->order.as<uint32_t>();
    return SPHGB_OK;
}

int sphgb_apply_order(sphgb_ctx* c, void* field, int32_t elemBytes)
{
    SPHGB_TRY(useDevice(c));
    return applyOrder(c, field, elemBytes);
}

int sphgb_sort_by_key(sphgb_ctx* c, const uint64_t* keysIn, uint64_t* keysOut, const uint32_t* valsIn,
                      uint32_t* valsOut, int64_t n, int32_t endBit)
{
    SPHGB_TRY(useDevice(c));
    if (n < 0 || (n > 0 && (!keysIn || !keysOut))) return SPHGB_ERR_ARG;
    if (n > 0 && (keysIn == keysOut || (valsIn && valsIn == valsOut))) return SPHGB_ERR_ARG;
    SPHGB_TRY(radixSort(c, reinterpret_cast<const u64*>(keysIn), reinterpret_cast<u64*>(keysOut), valsIn, valsOut, n,
                        endBit));
    SPHGB_TRY(sortStatusAsync(c));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    return sortStatusAfterSync(c);
}

int sphgb_find_neighbors(sphgb_ctx* c, const double* x, const double* y, const double* z, const void* h,
                         int32_t hPrec, int64_t first, int64_t last, uint32_t ngmax, uint32_t* neighbors, uint32_t* nc)
{
    SPHGB_TRY(useDevice(c));
    if (!c->haveTree) return SPHGB_ERR_STATE;
    if (first < 0 || last > c->n || first >= last) return SPHGB_ERR_ARG;
    StageTimer t(c, kStageNbr);
    int s = findNeighborsFixed(c, x, y, z, h, hPrec, first, last, ngmax, neighbors, nc);
    t.stop();
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    return s;
}

int sphgb_find_neighbors_sph(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    SPHGB_TRY(useDevice(c));
    if (!c->haveTree) return SPHGB_ERR_STATE;
    SPHGB_TRY(checkRange(p, first, last));
    if (last > c->n) return SPHGB_ERR_ARG;
    StageTimer t(c, kStageNbr);
    int s = findNeighborsSph(c, p, first, last);
    t.stop();
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    collectTimings(c, 2);
    return s;
}

int sphgb_export_neighbors(sphgb_ctx* c, uint32_t* out)
{
    SPHGB_TRY(useDevice(c));
    return exportNeighbors(c, out);
}

#define SPHGB_PASS(name, call)                                  \
    int name                                                    \
    {                                                           \
        SPHGB_TRY(useDevice(c));                                \
        SPHGB_TRY(checkRange(p, first, last));                  \
        int s_ = (call);                                        \
        if (s_ != SPHGB_OK) return s_;                          \
        SPHGB_CUDA(cudaStreamSynchronize(c->stream));           \
        return SPHGB_OK;                                        \
    }

SPHGB_PASS(sphgb_compute_density(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last),
           passDensity(c, p, first, last))
SPHGB_PASS(sphgb_compute_eos_std(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last),
           passEosStd(c, p, first, last))
SPHGB_PASS(sphgb_compute_iad(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last),
           passIadStd(c, p, first, last))
SPHGB_PASS(sphgb_compute_momentum_energy_std(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last,
                                             double* minDtCourant),
           passMomentumEnergyStd(c, p, first, last, minDtCourant))
SPHGB_PASS(sphgb_compute_xmass(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last),
           passXMass(c, p, first, last))
SPHGB_PASS(sphgb_compute_ve_def_gradh(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last),
           passGradh(c, p, first, last))
SPHGB_PASS(sphgb_compute_eos(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last),
           passEosVe(c, p, first, last))
SPHGB_PASS(sphgb_compute_iad_divv_curlv(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last),
           passIadDivvCurlv(c, p, first, last))
SPHGB_PASS(sphgb_compute_av_switches(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last),
           passAVswitches(c, p, first, last))
SPHGB_PASS(sphgb_compute_momentum_energy(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last,
                                         int32_t avClean, float* groupDt, double* minDtCourant),
           passMomentumEnergyVe(c, p, first, last, avClean, groupDt, minDtCourant))

int sphgb_sweep_passes(sphgb_ctx* c, sphgb_particles* p, int32_t variant, int32_t avClean, double* minDtCourant)
{
    SPHGB_TRY(useDevice(c));
    if (!p || !c->haveTree) return SPHGB_ERR_STATE;
    const int64_t first = 0, last = p->n;
    int s;
    {
        StageTimer t(c, kStageNbr);
        s = findNeighborsSph(c, p, first, last);
        t.stop();
        if (s != SPHGB_OK && s != SPHGB_ERR_NOCONV) return s;
    }
    int st = s;
    struct SweepScope {  // precomputes once per sweep, released on every exit path
        sphgb_ctx* c;
        explicit SweepScope(sphgb_ctx* cc) : c(cc) { reset(true); }
        ~SweepScope() { reset(false); }
        void reset(bool in) { c->inSweep = in, c->sweepPrepared = c->eosFused = c->auxReady = c->geoValid = false; }
    } scope(c);
    auto stage = [&](int k, auto&& fn) {
        StageTimer t(c, kStagePass0 + k);
        int r = fn();
        t.stop();
        return r;
    };
    if (variant == SPHGB_STD) {
        SPHGB_TRY(stage(0, [&] { return passDensity(c, p, first, last); }));
        SPHGB_TRY(stage(1, [&] { return passEosStd(c, p, first, last); }));
        SPHGB_TRY(stage(2, [&] { return passIadStd(c, p, first, last); }));
        SPHGB_TRY(stage(3, [&] { return passMomentumEnergyStd(c, p, first, last, minDtCourant); }));
    } else if (variant == SPHGB_VE) {
        SPHGB_TRY(stage(0, [&] { return passXMass(c, p, first, last); }));
        SPHGB_TRY(stage(1, [&] { return passGradh(c, p, first, last); }));
        SPHGB_TRY(stage(2, [&] { return passEosVe(c, p, first, last); }));
        SPHGB_TRY(stage(3, [&] { return passIadDivvCurlv(c, p, first, last); }));
        SPHGB_TRY(stage(4, [&] { return passAVswitches(c, p, first, last); }));
        SPHGB_TRY(stage(5, [&] { return passMomentumEnergyVe(c, p, first, last, avClean, nullptr, minDtCourant); }));
    } else {
        return SPHGB_ERR_ARG;
    }
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    collectTimings(c, variant == SPHGB_STD ? kStagePass0 + 4 : kStagePass0 + 6);
    return st;
}

int sphgb_sweep(sphgb_ctx* c, sphgb_particles* p, sphgb_box* box, int32_t variant, int32_t avClean,
                double* minDtCourant)
{
    SPHGB_TRY(useDevice(c));
    if (!p || !box) return SPHGB_ERR_ARG;
    if (variant != SPHGB_STD && variant != SPHGB_VE) return SPHGB_ERR_ARG;
    {
        StageTimer t(c, kStageSync);
        int s = domainSync(c, p, box);
        t.stop();
        if (s != SPHGB_OK) return s;
    }
    // the sync validated the fields and nothing can change them before the search of this call
    c->inputsChecked = true;
    const int s = sphgb_sweep_passes(c, p, variant, avClean, minDtCourant);
    c->inputsChecked = false;
    return s;
}

int sphgb_adjoint_std(sphgb_ctx* c, sphgb_particles* p, const sphgb_seeds* seeds, sphgb_grads* grads,
                      int32_t deterministic)
{
    SPHGB_TRY(useDevice(c));
    if (!p || !grads) return SPHGB_ERR_ARG;
    return adjointStd(c, p, seeds, grads, deterministic);
}

int sphgb_adjoint_ve(sphgb_ctx* c, sphgb_particles* p, const double* alpha_prev, int32_t av_clean,
                     const sphgb_seeds* seeds, sphgb_grads* grads, int32_t deterministic)
{
    SPHGB_TRY(useDevice(c));
    if (!p || !grads) return SPHGB_ERR_ARG;
    return adjointVe(c, p, alpha_prev, av_clean, seeds, grads, deterministic);
}

int sphgb_get_stats(sphgb_ctx* c, sphgb_stats* s)
{
    if (!c || !s) return SPHGB_ERR_ARG;
    *s = c->stats;
    s->refined_gradh = c->stats_refinedGradh;
    s->refined_divv = c->stats_refinedDivv;
    return SPHGB_OK;
}

int sphgb_get_timings(sphgb_ctx* c, float* ms, int32_t count)
{
    if (!c || !ms || count < 0) return SPHGB_ERR_ARG;
    for (int k = 0; k < count && k < kNumStages; ++k) ms[k] = c->stageMs[k];
    return SPHGB_OK;
}

int sphgb_kernel_launches(sphgb_ctx* c, int64_t* n)
{
    if (!c || !n) return SPHGB_ERR_ARG;
    *n = c->launches;
    return SPHGB_OK;
}

}  // extern "C"
