// Time integration and global reductions of one step, all particles on one time step (no rungs).
//
//   positions + energy: sph::computePositions (sph/include/sph/positions.hpp:54-88, 180-200;
//                       GPU computePositionsKernel, positions_gpu.cu:118-165)
//   smoothing length:   sph::updateSmoothingLength (update_h.hpp:26-45, updateH kernels.hpp:26-32)
//   time step:          sph::rhoTimestep, accelerationTimestep, computeTimestep (ts_global.hpp:36-113)
//   conserved sums:     sphexa::localConservedQuantities (main/src/observables/conserved_quantities.hpp:49-113)
//
// The update kernels are elementwise and HBM-bound.  They evaluate the reference's expressions in
// its order with round-to-nearest intrinsics (no contraction into FMAs), so positions, velocities,
// x_m1 and u match the reference CPU functions bit for bit.  Reductions go through block partials
// in a fixed order and one final block: the result does not depend on scheduling.
#include <cmath>

#include "pairs.cuh"

namespace sphgb {

int useDeviceOf(sphgb_ctx* c);

namespace {

constexpr int kIntBlock = 256;

struct PosArgs {
    double *x, *y, *z, *u;
    const double* du;
    void *vx, *vy, *vz, *xm1, *ym1, *zm1, *dum1;
    const void *ax, *ay, *az, *h;
    double dt, dtm1;
    double idtm1, halfDtm1, adt;  // 1/dt_m1, 0.5 dt_m1, |dt|: the same values for every particle
    DevBox box;
    int fixed[3];
    int64_t first, last;
};

// reference fbcCheck (positions.hpp:46-51)
template<class T>
__device__ __forceinline__ bool nearFixed(double coord, T h, double top, double bottom, int fbc)
{
    const double twoH = double(T(2) * h);
    return fbc && (fabs(__dsub_rn(top, coord)) < twoH || fabs(__dsub_rn(bottom, coord)) < twoH);
}

// reference energyUpdate (positions.hpp:54-61): u + du dt + 0.5 (du - du_m1) / dt_m1 |dt| dt
__device__ __forceinline__ double energyUpdate(double uOld, double dt, double dtm1, double du, double dum1)
{
    double t = __ddiv_rn(__dmul_rn(0.5, __dsub_rn(du, dum1)), dtm1);
    t = __dmul_rn(__dmul_rn(t, fabs(dt)), dt);
    double uNew = __dadd_rn(__dadd_rn(uOld, __dmul_rn(du, dt)), t);
    if (uNew < 0.0) uNew = __dmul_rn(uOld, exp(__ddiv_rn(__dmul_rn(uNew, dt), uOld)));
    return uNew;
}

// reference positionUpdate (positions.hpp:74-85) for one component, and putInBox (box.hpp:193-214)
template<class T>
__global__ void __launch_bounds__(kIntBlock) positionsKernel(PosArgs a)
{
    const int64_t i = a.first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= a.last) return;
    T* vx = static_cast<T*>(a.vx);
    T* vy = static_cast<T*>(a.vy);
    T* vz = static_cast<T*>(a.vz);
    T* xm1 = static_cast<T*>(a.xm1);
    T* ym1 = static_cast<T*>(a.ym1);
    T* zm1 = static_cast<T*>(a.zm1);
    if ((a.fixed[0] | a.fixed[1] | a.fixed[2]) && vx[i] == T(0) && vy[i] == T(0) && vz[i] == T(0)) {
        const T hi = static_cast<const T*>(a.h)[i];
        if (nearFixed(a.x[i], hi, a.box.hi[0], a.box.lo[0], a.fixed[0]) ||
            nearFixed(a.y[i], hi, a.box.hi[1], a.box.lo[1], a.fixed[1]) ||
            nearFixed(a.z[i], hi, a.box.hi[2], a.box.lo[2], a.fixed[2]))
            return;  // the GPU kernel leaves these particles (and their energy) untouched
    }
    const double A[3] = {double(static_cast<const T*>(a.ax)[i]), double(static_cast<const T*>(a.ay)[i]),
                         double(static_cast<const T*>(a.az)[i])};
    double* X[3] = {a.x + i, a.y + i, a.z + i};
    T* dX[3] = {xm1 + i, ym1 + i, zm1 + i};
    T* V[3] = {vx + i, vy + i, vz + i};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double vHalf = __dmul_rn(double(*dX[k]), a.idtm1);
        const double vn = __dadd_rn(vHalf, __dmul_rn(a.halfDtm1, A[k]));
        const double vnp1 = __dadd_rn(vn, __dmul_rn(A[k], a.dt));
        const double dxn = __dmul_rn(__dadd_rn(vn, __dmul_rn(__dmul_rn(0.5, A[k]), a.adt)), a.dt);
        double xn = __dadd_rn(*X[k], dxn);
        if (a.box.pbc[k]) {
            if (xn > a.box.hi[k]) xn = __dsub_rn(xn, a.box.L[k]);
            else if (xn < a.box.lo[k]) xn = __dadd_rn(xn, a.box.L[k]);
        }
        *X[k] = xn;
        *dX[k] = T(dxn);
        *V[k] = T(vnp1);
    }
    if (a.u) {
        T* dum1 = static_cast<T*>(a.dum1);
        a.u[i] = energyUpdate(a.u[i], a.dt, a.dtm1, a.du[i], double(dum1[i]));
        dum1[i] = T(a.du[i]);
    }
}

// reference updateH (kernels.hpp:26-32) in the arithmetic of h's type
template<class T>
__global__ void updateHKernel(int64_t first, int64_t last, unsigned ng0, const uint32_t* __restrict__ nc,
                              T* __restrict__ h)
{
    const int64_t i = first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= last) return;
    constexpr T c0 = 1023.0;
    constexpr T ex = 1.0 / 10.0;
    h[i] = h[i] * T(0.5) * pow(T(1) + c0 * T(ng0) / T(nc[i]), ex);
}

// ---- deterministic reductions: per-block partials in a fixed tree order, then one block ----
template<int N>
struct Sums {
    double v[N];
};

template<int N, class Op>
__device__ __forceinline__ void blockReduce(Sums<N>& s, Op op)
{
    __shared__ double sh[N][kIntBlock / kWarp];
    const int lane = threadIdx.x & (kWarp - 1), w = threadIdx.x / kWarp;
#pragma unroll
    for (int q = 0; q < N; ++q) {
        for (int o = 16; o > 0; o >>= 1) s.v[q] = op(s.v[q], __shfl_xor_sync(0xffffffffu, s.v[q], o));
        if (lane == 0) sh[q][w] = s.v[q];
    }
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < N; ++q) {
            double r = sh[q][0];
            for (int k = 1; k < kIntBlock / kWarp; ++k) r = op(r, sh[q][k]);
            s.v[q] = r;
        }
}

struct AddOp {
    __device__ double operator()(double a, double b) const { return a + b; }
};
struct MaxOp {
    __device__ double operator()(double a, double b) const { return fmax(a, b); }
};

// conserved quantities per particle: m |v|^2, m u, m v, m (x cross v)
template<class T>
__global__ void __launch_bounds__(kIntBlock) conservedKernel(int64_t first, int64_t last, const double* x,
                                                             const double* y, const double* z, const void* vx,
                                                             const void* vy, const void* vz, const void* m,
                                                             const double* u, double* partials)
{
    Sums<8> s{};
    for (int64_t i = first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < last;
         i += int64_t(gridDim.x) * blockDim.x) {
        const double X[3] = {x[i], y[i], z[i]};
        const double V[3] = {double(static_cast<const T*>(vx)[i]), double(static_cast<const T*>(vy)[i]),
                             double(static_cast<const T*>(vz)[i])};
        const double mi = double(static_cast<const T*>(m)[i]);
        s.v[0] += mi * (V[0] * V[0] + (V[1] * V[1] + V[2] * V[2]));  // norm2, a right fold (util/array.hpp)
        s.v[1] += u ? u[i] * mi : 0.0;
        s.v[2] += mi * V[0];
        s.v[3] += mi * V[1];
        s.v[4] += mi * V[2];
        s.v[5] += mi * (X[1] * V[2] - X[2] * V[1]);
        s.v[6] += mi * (X[2] * V[0] - X[0] * V[2]);
        s.v[7] += mi * (X[0] * V[1] - X[1] * V[0]);
    }
    blockReduce(s, AddOp{});
    if (threadIdx.x == 0)
        for (int q = 0; q < 8; ++q) partials[q * gridDim.x + blockIdx.x] = s.v[q];
}

// max over particles of field f (divv) or of |a|^2
template<class T, bool Norm2>
__global__ void __launch_bounds__(kIntBlock) maxKernel(int64_t first, int64_t last, const void* f0, const void* f1,
                                                       const void* f2, double* partials)
{
    Sums<1> s{{-INFINITY}};
    for (int64_t i = first + blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < last;
         i += int64_t(gridDim.x) * blockDim.x) {
        double v;
        if constexpr (Norm2) {
            const double a0 = static_cast<const T*>(f0)[i], a1 = static_cast<const T*>(f1)[i],
                         a2 = static_cast<const T*>(f2)[i];
            v = a0 * a0 + (a1 * a1 + a2 * a2);
        } else
            v = double(static_cast<const T*>(f0)[i]);
        s.v[0] = fmax(s.v[0], v);
    }
    blockReduce(s, MaxOp{});
    if (threadIdx.x == 0) partials[blockIdx.x] = s.v[0];
}

template<int N, bool Max>
__global__ void __launch_bounds__(kIntBlock) finalKernel(const double* partials, int blocks, double* out)
{
    Sums<N> s;
    for (int q = 0; q < N; ++q) s.v[q] = Max ? -INFINITY : 0.0;
    for (int b = threadIdx.x; b < blocks; b += blockDim.x)
        for (int q = 0; q < N; ++q)
            s.v[q] = Max ? fmax(s.v[q], partials[q * blocks + b]) : s.v[q] + partials[q * blocks + b];
    if constexpr (Max) blockReduce(s, MaxOp{});
    else blockReduce(s, AddOp{});
    if (threadIdx.x == 0)
        for (int q = 0; q < N; ++q) out[q] = s.v[q];
}

constexpr int kReduceBlocks = 2 * 152;  // two blocks per SM, grid-stride

bool validRange(const sphgb_particles* p, int64_t first, int64_t last)
{
    return p && first >= 0 && last <= p->n && first <= last;
}

template<int N, bool Max>
int finish(sphgb_ctx* c, double* partials, double* host)
{
    double* out = partials + N * kReduceBlocks;
    finalKernel<N, Max><<<1, kIntBlock, 0, c->stream>>>(partials, kReduceBlocks, out);
    SPHGB_TRY(launched(c, "finalKernel"));
    SPHGB_CUDA(cudaMemcpyAsync(host, out, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
    SPHGB_CUDA(cudaStreamSynchronize(c->stream));
    return SPHGB_OK;
}

int maxReduce(sphgb_ctx* c, const sphgb_particles* p, int64_t first, int64_t last, bool norm2, double* result)
{
    SPHGB_TRY(c->intScratch.ensure(sizeof(double) * (kReduceBlocks + 1)));
    double* part = c->intScratch.as<double>();
    const bool mixed = p->precision == SPHGB_MIXED;
    if (norm2) {
        if (mixed) maxKernel<float, true><<<kReduceBlocks, kIntBlock, 0, c->stream>>>(first, last, p->ax, p->ay, p->az, part);
        else maxKernel<double, true><<<kReduceBlocks, kIntBlock, 0, c->stream>>>(first, last, p->ax, p->ay, p->az, part);
    } else {
        if (mixed) maxKernel<float, false><<<kReduceBlocks, kIntBlock, 0, c->stream>>>(first, last, p->divv, nullptr, nullptr, part);
        else maxKernel<double, false><<<kReduceBlocks, kIntBlock, 0, c->stream>>>(first, last, p->divv, nullptr, nullptr, part);
    }
    SPHGB_TRY(launched(c, "maxKernel"));
    return finish<1, true>(c, part, result);
}

}  // namespace

int accelerationTimestep(sphgb_ctx* c, const sphgb_particles* p, int64_t first, int64_t last, double etaAcc,
                         double eps, double* dt)
{
    if (!validRange(p, first, last) || !p->ax || !p->ay || !p->az || !dt) return SPHGB_ERR_ARG;
    double maxAccSq = 0.0;
    if (last > first) SPHGB_TRY(maxReduce(c, p, first, last, true, &maxAccSq));
    maxAccSq = std::fmax(maxAccSq, 0.0);
    *dt = etaAcc * std::sqrt(eps / std::sqrt(maxAccSq));
    return SPHGB_OK;
}

}  // namespace sphgb

using namespace sphgb;

extern "C" {

int sphgb_compute_positions(sphgb_ctx* c, sphgb_particles* p, const sphgb_box* box, void* x_m1, void* y_m1,
                            void* z_m1, void* du_m1, const sphgb_timestep* ts, int64_t first, int64_t last)
{
    SPHGB_TRY(useDeviceOf(c));
    if (!validRange(p, first, last) || !box || !ts || !p->x || !p->y || !p->z || !p->vx || !p->vy || !p->vz ||
        !p->ax || !p->ay || !p->az || !p->h || !x_m1 || !y_m1 || !z_m1)
        return SPHGB_ERR_ARG;
    if (p->u && (!p->du || !du_m1)) return SPHGB_ERR_ARG;
    if (!(ts->minDt_m1 != 0.0)) return SPHGB_ERR_ARG;
    for (int k = 0; k < 3; ++k)
        if (box->bc[k] > SPHGB_BC_FIXED) return SPHGB_ERR_ARG;
    if (last == first) return SPHGB_OK;
    PosArgs a;
    a.x = p->x;
    a.y = p->y;
    a.z = p->z;
    a.u = p->u;
    a.du = p->du;
    a.vx = p->vx;
    a.vy = p->vy;
    a.vz = p->vz;
    a.xm1 = x_m1;
    a.ym1 = y_m1;
    a.zm1 = z_m1;
    a.dum1 = du_m1;
    a.ax = p->ax;
    a.ay = p->ay;
    a.az = p->az;
    a.h = p->h;
    a.dt = ts->minDt;
    a.dtm1 = ts->minDt_m1;
    a.idtm1 = 1.0 / a.dtm1;  // the host's IEEE division: the value the reference forms per particle
    a.halfDtm1 = 0.5 * a.dtm1;
    a.adt = std::fabs(a.dt);
    a.box = makeDevBox(*box);
    for (int k = 0; k < 3; ++k) a.fixed[k] = box->bc[k] == SPHGB_BC_FIXED;
    a.first = first;
    a.last = last;
    const unsigned blocks = gridFor(last - first, kIntBlock);
    if (p->precision == SPHGB_MIXED) positionsKernel<float><<<blocks, kIntBlock, 0, c->stream>>>(a);
    else positionsKernel<double><<<blocks, kIntBlock, 0, c->stream>>>(a);
    return launched(c, "positionsKernel");
}

int sphgb_update_smoothing_length(sphgb_ctx* c, sphgb_particles* p, int64_t first, int64_t last)
{
    SPHGB_TRY(useDeviceOf(c));
    if (!validRange(p, first, last) || !p->h || !p->nc) return SPHGB_ERR_ARG;
    if (last == first) return SPHGB_OK;
    const unsigned blocks = gridFor(last - first, kIntBlock);
    if (p->precision == SPHGB_MIXED)
        updateHKernel<float><<<blocks, kIntBlock, 0, c->stream>>>(first, last, c->prm.ng0, p->nc,
                                                                  static_cast<float*>(p->h));
    else
        updateHKernel<double><<<blocks, kIntBlock, 0, c->stream>>>(first, last, c->prm.ng0, p->nc,
                                                                   static_cast<double*>(p->h));
    return launched(c, "updateHKernel");
}

int sphgb_rho_timestep(sphgb_ctx* c, const sphgb_particles* p, int64_t first, int64_t last, double Krho, double* dt)
{
    SPHGB_TRY(useDeviceOf(c));
    if (!validRange(p, first, last) || !p->divv || !dt) return SPHGB_ERR_ARG;
    double maxDivv = -INFINITY;
    if (last > first) SPHGB_TRY(maxReduce(c, p, first, last, false, &maxDivv));
    *dt = Krho / std::fabs(maxDivv);
    return SPHGB_OK;
}

int sphgb_acceleration_timestep(sphgb_ctx* c, const sphgb_particles* p, int64_t first, int64_t last, double etaAcc,
                                double eps, double* dt)
{
    SPHGB_TRY(useDeviceOf(c));
    return accelerationTimestep(c, p, first, last, etaAcc, eps, dt);
}

int sphgb_compute_timestep(sphgb_ctx* c, const sphgb_particles* p, int64_t first, int64_t last, sphgb_timestep* ts)
{
    SPHGB_TRY(useDeviceOf(c));
    if (!ts) return SPHGB_ERR_ARG;
    double minDtAcc = INFINITY;
    if (ts->g != 0.0) SPHGB_TRY(accelerationTimestep(c, p, first, last, ts->etaAcc, ts->eps, &minDtAcc));
    const double cand[4] = {minDtAcc, ts->minDtCourant, ts->minDtRho, ts->maxDtIncrease * ts->minDt};
    double m = cand[0];
    for (int k = 1; k < 4; ++k) m = std::min(m, cand[k]);
    ts->ttot += m;
    ts->minDt_m1 = ts->minDt;
    ts->minDt = m;
    return SPHGB_OK;
}

int sphgb_conserved_quantities(sphgb_ctx* c, const sphgb_particles* p, int64_t first, int64_t last, double out[8])
{
    SPHGB_TRY(useDeviceOf(c));
    if (!validRange(p, first, last) || !out || !p->x || !p->y || !p->z || !p->vx || !p->vy || !p->vz || !p->m)
        return SPHGB_ERR_ARG;
    SPHGB_TRY(c->intScratch.ensure(sizeof(double) * 9 * kReduceBlocks));
    double* part = c->intScratch.as<double>();
    if (p->precision == SPHGB_MIXED)
        conservedKernel<float><<<kReduceBlocks, kIntBlock, 0, c->stream>>>(first, last, p->x, p->y, p->z, p->vx, p->vy,
                                                                           p->vz, p->m, p->u, part);
    else
        conservedKernel<double><<<kReduceBlocks, kIntBlock, 0, c->stream>>>(first, last, p->x, p->y, p->z, p->vx,
                                                                            p->vy, p->vz, p->m, p->u, part);
    SPHGB_TRY(launched(c, "conservedKernel"));
    double s[8];
    SPHGB_TRY((finish<8, false>(c, part, s)));
    out[0] = 0.5 * s[0];
    for (int q = 1; q < 8; ++q) out[q] = s[q];
    return SPHGB_OK;
}

}  // extern "C"
