// FMA-throughput probe: the FP64 and FP32 pipe peaks that the pair passes are measured against.
// The device-wide figure is taken in the same process as the measurement it normalises, with
// 8 independent FMA chains per thread so that issue, not latency, is the limit.
#include "context.cuh"

namespace sphgb {
namespace {

constexpr int kChains = 8;
constexpr int kIters = 2048;

template<class T>
__global__ void __launch_bounds__(256) fmaProbe(T* out, T seed)
{
    T a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = seed + T(threadIdx.x + k);
    const T m = T(0.999999), c = T(1e-7);
    for (int it = 0; it < kIters; ++it) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], m, c);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == T(-1)) out[0] = s;  // never true; keeps the chains alive
}

}  // namespace
}  // namespace sphgb

using namespace sphgb;

extern "C" int sphgb_measure_fma_peak(sphgb_ctx* c, int32_t fp64, double* flops_per_s)
{
    if (!c || !flops_per_s) return SPHGB_ERR_ARG;
    SPHGB_CUDA(cudaSetDevice(c->device));
    int sms = 0;
    SPHGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    SPHGB_TRY(c->reduceScratch.ensure(64));
    const int blocks = sms * 8, threads = 256;
    cudaEvent_t a, b;
    SPHGB_CUDA(cudaEventCreate(&a));
    SPHGB_CUDA(cudaEventCreate(&b));
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        SPHGB_CUDA(cudaEventRecord(a, c->stream));
        if (fp64) fmaProbe<double><<<blocks, threads, 0, c->stream>>>(c->reduceScratch.as<double>(), 1.0);
        else fmaProbe<float><<<blocks, threads, 0, c->stream>>>(c->reduceScratch.as<float>(), 1.f);
        SPHGB_TRY(launched(c, "fmaProbe"));
        SPHGB_CUDA(cudaEventRecord(b, c->stream));
        SPHGB_CUDA(cudaEventSynchronize(b));
        float ms = 0;
        SPHGB_CUDA(cudaEventElapsedTime(&ms, a, b));
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    double fmas = double(blocks) * threads * kChains * kIters;
    *flops_per_s = 2.0 * fmas / (double(best) * 1e-3);
    return SPHGB_OK;
}
