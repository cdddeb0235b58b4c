// Input validation before the domain sync and the neighbour searches.
//
// A non-finite coordinate or smoothing length, or h <= 0, would otherwise flow into the key
// generation (sfc3D floors NaN to an arbitrary cell), the tree and the searches (a NaN radius
// matches nothing, an infinite one everything) without any error.  One pass over the fields sets a
// device word when any particle is bad; the host reads it back and returns SPHGB_ERR_INPUT before
// the first kernel that would use the data.  The reference has no such check (its neighbour search
// assumes finite inputs, domain/include/cstone/findneighbors.hpp:77-170); the cost is one read of
// x, y, z and h (about 40 us for 8M particles).
#include "context.cuh"

namespace sphgb {

namespace {

constexpr int kValBlock = 256;

__device__ __forceinline__ bool finite64(double v)
{
    return (__double_as_longlong(v) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
}

// bit 0: a non-finite coordinate; bit 1: h non-finite or h <= 0
__global__ void __launch_bounds__(kValBlock) validateKernel(const double* __restrict__ x, const double* __restrict__ y,
                                                            const double* __restrict__ z, const void* __restrict__ h,
                                                            int hIsFloat, int64_t n, int* __restrict__ word)
{
    int bad = 0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += stride) {
        if (!finite64(x[i]) || !finite64(y[i]) || !finite64(z[i])) bad |= 1;
        if (h) {
            const double hi = hIsFloat ? double(static_cast<const float*>(h)[i]) : static_cast<const double*>(h)[i];
            if (!(hi > 0.0) || !finite64(hi)) bad |= 2;  // !(hi > 0) also holds for NaN
        }
    }
    const int any = __syncthreads_or(bad);
    if (any) {
        if ((bad & 1) != 0) atomicOr(word, 1);
        if ((bad & 2) != 0) atomicOr(word, 2);
    }
}

}  // namespace

int validateParticles(sphgb_ctx* c, const double* x, const double* y, const double* z, const void* h, int hIsFloat,
                      int64_t n)
{
    if (n <= 0) return SPHGB_OK;
    SPHGB_TRY(c->checkWord.ensure(sizeof(int)));
    int* word = c->checkWord.as<int>();
    SPHGB_CUDA(cudaMemsetAsync(word, 0, sizeof(int), c->stream));
    const int64_t need = (n + kValBlock - 1) / kValBlock;
    const unsigned blocks = unsigned(need < 152 * 8 ? need : 152 * 8);
    validateKernel<<<blocks, kValBlock, 0, c->stream>>>(x, y, z, h, hIsFloat, n, word);
    SPHGB_TRY(launched(c, "validateKernel"));
    int flags = 0;
    SPHGB_CUDA(cudaMemcpyAsync(&flags, word, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    return flags != 0 ? SPHGB_ERR_INPUT : SPHGB_OK;
}

}  // namespace sphgb
