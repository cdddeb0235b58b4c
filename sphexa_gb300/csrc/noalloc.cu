// Box fit + Hilbert keys without any device allocation.
//
// Some callers cannot let a library call cudaMalloc: codes whose device memory is owned by their
// own pool allocator (the whole HBM reserved up front and handed out by the application), codes
// that must not hit the implicit device-wide synchronisation of cudaMalloc/cudaFree inside a
// latency-bound time-step loop, and embeddings where allocation is forbidden while work is being
// enqueued.  For them this file offers one entry point that needs only the caller's inputs and
// outputs: its reduction scratch is a fixed file-scope device array.
//
// The scratch holds one (min, max) partial per axis for every block of the extrema reduction,
// plus the six reduced extrema.  A block covers kItemsPerBlock particles, so the array bounds
// the particle count at kMaxBlocks * kItemsPerBlock.
#include <mutex>

#include "context.cuh"

namespace sphgb {
namespace {

constexpr int kThreads = 256;
constexpr int kItemsPerThread = 16;
constexpr int64_t kItemsPerBlock = int64_t(kThreads) * kItemsPerThread;   // 4096 particles
constexpr int kMaxBlocks = 65536;                                           // -> 268,435,456 particles
constexpr int64_t kMaxParticles = kItemsPerBlock * kMaxBlocks;
constexpr int kMaxDevices = 64;

// 6 partials per block + 6 reduced extrema: 3 MiB, held by every GPU that loads the library
static __device__ __align__(256) double gKeysScratch[6 * kMaxBlocks + 6];

// device address of gKeysScratch per device; the host symbol is only a stand-in for it
double* gScratchAddr[kMaxDevices] = {};
std::mutex gScratchMutex;

int scratchFor(int device, double** out)
{
    std::lock_guard<std::mutex> lock(gScratchMutex);
    if (!gScratchAddr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, gKeysScratch);
        if (e != cudaSuccess) {
            setCudaError(e, "cudaGetSymbolAddress");
            return SPHGB_ERR_CUDA;
        }
        gScratchAddr[device] = static_cast<double*>(p);
    }
    *out = gScratchAddr[device];
    return SPHGB_OK;
}

__global__ void __launch_bounds__(kThreads) extremaPartials(const double* __restrict__ x,
                                                            const double* __restrict__ y,
                                                            const double* __restrict__ z, int64_t n,
                                                            double* __restrict__ part)
{
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    const int64_t base = int64_t(blockIdx.x) * kItemsPerBlock;
    for (int q = 0; q < kItemsPerThread; ++q) {
        int64_t i = base + int64_t(q) * kThreads + threadIdx.x;
        if (i < n) {
            double v[3] = {x[i], y[i], z[i]};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                mn[k] = fmin(mn[k], v[k]);
                mx[k] = fmax(mx[k], v[k]);
            }
        }
    }
    __shared__ double s[6][kThreads / kWarp];
#pragma unroll
    for (int k = 0; k < 3; ++k)
        for (int o = 16; o > 0; o >>= 1) {
            mn[k] = fmin(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmax(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    const int w = threadIdx.x / kWarp, l = threadIdx.x % kWarp;
    if (l == 0)
        for (int k = 0; k < 3; ++k) {
            s[2 * k][w] = mn[k];
            s[2 * k + 1][w] = mx[k];
        }
    __syncthreads();
    if (threadIdx.x < 6) {
        double r = s[threadIdx.x][0];
        for (int q = 1; q < kThreads / kWarp; ++q)
            r = (threadIdx.x & 1) ? fmax(r, s[threadIdx.x][q]) : fmin(r, s[threadIdx.x][q]);
        part[6 * int64_t(blockIdx.x) + threadIdx.x] = r;  // every slot below 6 * gridDim.x is written
    }
}

__global__ void __launch_bounds__(kThreads) extremaFinal(const double* __restrict__ part, int blocks,
                                                         double* __restrict__ out)
{
    // thread t reduces slot t % 6 over a strided subset of blocks; warp 0 combines
    __shared__ double s[kThreads];
    const int slot = threadIdx.x % 6;
    const int lane = threadIdx.x / 6;           // 0..41
    const int lanes = kThreads / 6;             // 42 strides per slot
    double r = (slot & 1) ? -INFINITY : INFINITY;
    if (threadIdx.x < 6 * lanes)
        for (int b = lane; b < blocks; b += lanes)
            r = (slot & 1) ? fmax(r, part[6 * int64_t(b) + slot]) : fmin(r, part[6 * int64_t(b) + slot]);
    s[threadIdx.x] = r;
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = s[threadIdx.x];
        for (int q = 1; q < lanes; ++q) {
            double u = s[threadIdx.x + 6 * q];
            v = (threadIdx.x & 1) ? fmax(v, u) : fmin(v, u);
        }
        out[threadIdx.x] = v;
    }
}

__global__ void __launch_bounds__(kThreads) keysOnly(const double* __restrict__ x, const double* __restrict__ y,
                                                     const double* __restrict__ z, int64_t n, DevBox box,
                                                     unsigned long long* __restrict__ keys)
{
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < n) keys[i] = sfcKey(x[i], y[i], z[i], box);
}

}  // namespace
}  // namespace sphgb

using namespace sphgb;

extern "C" int sphgb_sfc_keys_noalloc(const double* x, const double* y, const double* z, int64_t n, sphgb_box* box,
                                      uint64_t* keys, void* stream)
{
    if (!x || !y || !z || !box || !keys || n <= 0) return SPHGB_ERR_ARG;
    if (n > kMaxParticles) return SPHGB_ERR_TOO_LARGE;
    int device = 0;
    SPHGB_CUDA(cudaGetDevice(&device));
    if (device < 0 || device >= kMaxDevices) return SPHGB_ERR_ARG;
    double* scratch = nullptr;
    SPHGB_TRY(scratchFor(device, &scratch));
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    sphgb_box b = *box;
    const bool open = b.bc[0] != SPHGB_BC_PERIODIC || b.bc[1] != SPHGB_BC_PERIODIC || b.bc[2] != SPHGB_BC_PERIODIC;
    if (open) {
        const int blocks = int((n + kItemsPerBlock - 1) / kItemsPerBlock);
        extremaPartials<<<blocks, kThreads, 0, st>>>(x, y, z, n, scratch);
        SPHGB_CUDA(cudaGetLastError());
        extremaFinal<<<1, kThreads, 0, st>>>(scratch, blocks, scratch + 6 * kMaxBlocks);
        SPHGB_CUDA(cudaGetLastError());
        double ext[6];
        SPHGB_CUDA(cudaMemcpyAsync(ext, scratch + 6 * kMaxBlocks, sizeof(ext), cudaMemcpyDeviceToHost, st));
        SPHGB_CUDA(cudaStreamSynchronize(st));
        for (int k = 0; k < 3; ++k)
            if (b.bc[k] != SPHGB_BC_PERIODIC) {
                b.lim[2 * k] = ext[2 * k];
                b.lim[2 * k + 1] = ext[2 * k + 1];
            }
    }
    for (int k = 0; k < 3; ++k)
        if (!(b.lim[2 * k + 1] > b.lim[2 * k])) return SPHGB_ERR_ARG;
    keysOnly<<<unsigned((n + kThreads - 1) / kThreads), kThreads, 0, st>>>(
        x, y, z, n, makeDevBox(b), reinterpret_cast<unsigned long long*>(keys));
    SPHGB_CUDA(cudaGetLastError());
    SPHGB_CUDA(cudaStreamSynchronize(st));
    *box = b;
    return SPHGB_OK;
}
