/* sphgb/dropin.hpp: the reference's hot-path call signatures, implemented over the sphgb C ABI.
 *
 * Header-only C++20.  It depends on no reference header: Dataset, Box and GroupView are template
 * parameters used through the member names of the reference types
 *   Dataset   sphexa::ParticlesData<GpuTag> (sph/include/sph/particles_data.hpp:63-391), its
 *             DeviceParticlesData in d.devData (particles_data_gpu.cuh:49-210) and scalars ng0,
 *             ngmax, gamma, Kcour, sincIndex, alphamin, alphamax, decay_constant, minDt,
 *             minDtCourant, HydroType, RealType;
 *   Box       cstone::Box<T> (domain/include/cstone/sfc/box.hpp:94-174);
 *   GroupView cstone::GroupView {firstBody, lastBody, ...} (traversal/groups.hpp:28-34).
 * Every function throws std::runtime_error with the C ABI's status text on failure, as the
 * reference throws on its own error conditions (sph/include/sph/hydro_ve/xmass_gpu.cu:127-128).
 *
 * The neighbour lists and the tree live in one sphgb context per host thread and device: the
 * SingleRankDomain below builds the tree, findNeighborsSfc builds the lists, and the compute*
 * calls read both.  The adapter converts types only; all work runs in libsphgb.so.
 */
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>

#include "../sphgb.h"

namespace sphgb {
namespace dropin {

inline void check(int status, const char* where)
{
    if (status == SPHGB_OK) return;
    std::string msg = std::string(where) + ": " + sphgb_status_string(status);
    if (status == SPHGB_ERR_CUDA) msg += std::string(" (") + sphgb_last_cuda_error() + ")";
    throw std::runtime_error(msg);
}

//! one context per host thread and device, created on first use
inline sphgb_ctx* context(int device = 0)
{
    struct Holder {
        sphgb_ctx* c[64] = {};
        ~Holder()
        {
            for (auto* p : c)
                if (p) sphgb_destroy(p);
        }
    };
    static thread_local Holder h;
    if (device < 0 || device >= 64) throw std::runtime_error("sphgb: device index out of range");
    if (!h.c[device]) check(sphgb_create(&h.c[device], device), "sphgb_create");
    return h.c[device];
}

template<class V>
void* ptr(V& v)
{
    if (v.size() == 0) return nullptr;
    return static_cast<void*>(rawPtr(v));  // cstone::rawPtr(DeviceVector&), found by ADL
}

template<class Dataset>
constexpr int32_t precisionOf()
{
    return sizeof(typename Dataset::HydroType) == sizeof(double) ? SPHGB_FP64 : SPHGB_MIXED;
}

template<class Dataset>
sphgb_particles particles(Dataset& d)
{
    auto& dv = d.devData;
    sphgb_particles p{};
    p.n = int64_t(dv.x.size());
    p.precision = precisionOf<Dataset>();
    p.keys = static_cast<uint64_t*>(ptr(dv.keys));
    p.x = static_cast<double*>(ptr(dv.x));
    p.y = static_cast<double*>(ptr(dv.y));
    p.z = static_cast<double*>(ptr(dv.z));
    p.u = static_cast<double*>(ptr(dv.u));
    p.du = static_cast<double*>(ptr(dv.du));
    p.h = ptr(dv.h);
    p.m = ptr(dv.m);
    p.vx = ptr(dv.vx);
    p.vy = ptr(dv.vy);
    p.vz = ptr(dv.vz);
    p.alpha = ptr(dv.alpha);
    p.rho = ptr(dv.rho);
    p.p = ptr(dv.p);
    p.c = ptr(dv.c);
    p.xm = ptr(dv.xm);
    p.kx = ptr(dv.kx);
    p.gradh = ptr(dv.gradh);
    p.prho = ptr(dv.prho);
    p.divv = ptr(dv.divv);
    p.curlv = ptr(dv.curlv);
    p.c11 = ptr(dv.c11);
    p.c12 = ptr(dv.c12);
    p.c13 = ptr(dv.c13);
    p.c22 = ptr(dv.c22);
    p.c23 = ptr(dv.c23);
    p.c33 = ptr(dv.c33);
    p.ax = ptr(dv.ax);
    p.ay = ptr(dv.ay);
    p.az = ptr(dv.az);
    p.dV11 = ptr(dv.dV11);
    p.dV12 = ptr(dv.dV12);
    p.dV13 = ptr(dv.dV13);
    p.dV22 = ptr(dv.dV22);
    p.dV23 = ptr(dv.dV23);
    p.dV33 = ptr(dv.dV33);
    p.nc = static_cast<uint32_t*>(ptr(dv.nc));
    return p;
}

//! the physics constants of the dataset, pushed before every call
template<class Dataset>
sphgb_ctx* bind(Dataset& d, int device = 0)
{
    sphgb_ctx* c = context(device);
    sphgb_params prm{};
    check(sphgb_default_params(&prm), "sphgb_default_params");
    prm.ng0 = d.ng0;
    prm.ngmax = d.ngmax;
    prm.gamma = double(d.gamma);
    prm.Kcour = double(d.Kcour);
    prm.sincIndex = double(d.sincIndex);
    prm.alphamin = double(d.alphamin);
    prm.alphamax = double(d.alphamax);
    prm.decay_constant = double(d.decay_constant);
    prm.minDt = double(d.minDt);
    check(sphgb_set_params(c, &prm), "sphgb_set_params");
    return c;
}

template<class Box>
sphgb_box toBox(const Box& box)
{
    sphgb_box b{};
    b.lim[0] = double(box.xmin());
    b.lim[1] = double(box.xmax());
    b.lim[2] = double(box.ymin());
    b.lim[3] = double(box.ymax());
    b.lim[4] = double(box.zmin());
    b.lim[5] = double(box.zmax());
    // cstone::BoundaryType and sphgb_boundary share their numbering (open 0, periodic 1, fixed 2)
    auto bt = [](auto t) { return uint8_t(t) <= SPHGB_BC_FIXED ? uint8_t(t) : uint8_t(SPHGB_BC_OPEN); };
    b.bc[0] = bt(box.boundaryX());
    b.bc[1] = bt(box.boundaryY());
    b.bc[2] = bt(box.boundaryZ());
    return b;
}

/*! cstone::Domain at one rank (domain/include/cstone/domain/domain.hpp:181-234, 416-428):
 *  sync() fits the box, sorts by Hilbert key, permutes x y z h and every property field, and
 *  builds the cornerstone tree with the bucket size; exchangeHalos is a no-op at one rank. */
template<class KeyType, class T, class Box>
class SingleRankDomain
{
public:
    // the tree the reference's octreeProperties() exposes is its focus tree, refined to
    // bucketSizeFocus (domain/domain.hpp:416-428); the coarser global tree (bucketSize) only assigns
    // ranks, which has no counterpart at one rank
    SingleRankDomain(int /*rank*/, int /*numRanks*/, unsigned /*bucketSize*/, unsigned bucketSizeFocus,
                     float /*theta*/, const Box& box, int device = 0)
        : box_(box)
        , bucket_(bucketSizeFocus)
        , device_(device)
    {
    }

    template<class Dataset, class... Props>
    void sync(Dataset& d, Props&... extraProperties)
    {
        sphgb_ctx* c = bind(d, device_);
        if (!started_) {  // this domain's syncs are the steps of one simulation (box shrink limit)
            check(sphgb_set_domain_mode(c, 1), "sphgb_set_domain_mode");
            started_ = true;
        }
        sphgb_params prm{};
        sphgb_default_params(&prm);
        prm.ng0 = d.ng0;
        prm.ngmax = d.ngmax;
        prm.bucket = bucket_;
        prm.gamma = double(d.gamma);
        prm.Kcour = double(d.Kcour);
        prm.sincIndex = double(d.sincIndex);
        prm.alphamin = double(d.alphamin);
        prm.alphamax = double(d.alphamax);
        prm.decay_constant = double(d.decay_constant);
        prm.minDt = double(d.minDt);
        check(sphgb_set_params(c, &prm), "sphgb_set_params");
        sphgb_particles p = particles(d);
        // dependent fields are recomputed by the passes; only conserved ones move with the sort
        sphgb_particles q{};
        q.n = p.n;
        q.precision = p.precision;
        q.keys = p.keys;
        q.x = p.x;
        q.y = p.y;
        q.z = p.z;
        q.u = p.u;
        q.h = p.h;
        q.m = p.m;
        q.vx = p.vx;
        q.vy = p.vy;
        q.vz = p.vz;
        q.alpha = p.alpha;
        sphgb_box b = toBox(box_);
        check(sphgb_domain_sync(c, &q, &b), "Domain::sync");
        (applyOrder(c, extraProperties), ...);
        box_ = Box(b.lim[0], b.lim[1], b.lim[2], b.lim[3], b.lim[4], b.lim[5], box_.boundaryX(), box_.boundaryY(),
                   box_.boundaryZ());
    }

    const Box& box() const { return box_; }
    std::size_t startIndex() const { return 0; }
    template<class Dataset>
    std::size_t endIndex(Dataset& d) const
    {
        return d.devData.x.size();
    }
    template<class... Fields>
    void exchangeHalos(Fields&&...) const
    {
    }

private:
    template<class V>
    static void applyOrder(sphgb_ctx* c, V& v)
    {
        if (v.size() == 0) return;
        check(sphgb_apply_order(c, ptr(v), int32_t(sizeof(*rawPtr(v)))), "sphgb_apply_order");
    }

    Box box_;
    unsigned bucket_;
    int device_;
    bool started_ = false;
};

/*! cstone::findNeighbors (domain/include/cstone/findneighbors.hpp:149-170) on the tree of the last
 *  SingleRankDomain::sync; the tree view argument is accepted for signature parity.  Writes
 *  neighbors[(i-first)*ngmax + k] and nc[i-first] (excluding self), device pointers. */
template<class T, class Th, class Box, class TreeView>
void findNeighbors(const T* x, const T* y, const T* z, const Th* h, std::size_t firstId, std::size_t lastId,
                   const Box& /*box*/, const TreeView& /*treeView*/, unsigned ngmax, uint32_t* neighbors,
                   unsigned* neighborsCount, int device = 0)
{
    static_assert(std::is_same_v<T, double>, "coordinates are FP64 (SphTypes::CoordinateType)");
    const int32_t hp = sizeof(Th) == sizeof(double) ? SPHGB_FP64 : SPHGB_MIXED;
    check(sphgb_find_neighbors(context(device), x, y, z, h, hp, int64_t(firstId), int64_t(lastId), ngmax, neighbors,
                               neighborsCount),
          "cstone::findNeighbors");
}

/*! sph::findNeighborsSfc (sph/include/sph/find_neighbors.hpp:47-56): neighbour lists with the
 *  coupled h iteration; prints the non-converged count like the reference. */
template<class Dataset, class Box>
void findNeighborsSfc(std::size_t startIndex, std::size_t endIndex, Dataset& d, const Box& /*box*/)
{
    if (d.ng0 > d.ngmax) throw std::runtime_error("ng0 should be smaller than ngmax\n");
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    int s = sphgb_find_neighbors_sph(c, &p, int64_t(startIndex), int64_t(endIndex));
    if (s == SPHGB_ERR_NOCONV) {
        sphgb_stats st{};
        sphgb_get_stats(c, &st);
        std::fprintf(stderr, "Coupled h-neighbor count updated failed to converge for %lld particles\n",
                     (long long)st.h_fails);
        return;
    }
    check(s, "findNeighborsSfc");
}

//! sph::computeGroups: groups are the 32 SFC-consecutive targets of each warp; nothing to build
template<class Dataset, class Box, class GroupData>
void computeGroups(std::size_t startIndex, std::size_t endIndex, Dataset&, const Box&, GroupData& groups)
{
    groups.firstBody = decltype(groups.firstBody)(startIndex);
    groups.lastBody = decltype(groups.lastBody)(endIndex);
}

#define SPHGB_DROPIN_PASS(NAME, CALL)                                                    \
    template<class GroupView, class Dataset, class Box>                                  \
    void NAME(const GroupView& grp, Dataset& d, const Box& /*box*/)                      \
    {                                                                                    \
        sphgb_ctx* c = bind(d);                                                          \
        sphgb_particles p = particles(d);                                                \
        check(CALL(c, &p, int64_t(grp.firstBody), int64_t(grp.lastBody)), #NAME);       \
    }

//! sph::computeDensity (sph/include/sph/hydro_std/density.hpp:55-60)
SPHGB_DROPIN_PASS(computeDensity, sphgb_compute_density)
//! sph::computeIAD (hydro_std/iad.hpp:74-79)
SPHGB_DROPIN_PASS(computeIAD, sphgb_compute_iad)
//! sph::computeXMass (hydro_ve/xmass.hpp:69-74)
SPHGB_DROPIN_PASS(computeXMass, sphgb_compute_xmass)
//! sph::computeVeDefGradh (hydro_ve/ve_def_gradh.hpp:80-85)
SPHGB_DROPIN_PASS(computeVeDefGradh, sphgb_compute_ve_def_gradh)
//! sph::computeIadDivvCurlv (hydro_ve/iad_divv_curlv.hpp:93-98)
SPHGB_DROPIN_PASS(computeIadDivvCurlv, sphgb_compute_iad_divv_curlv)
//! sph::computeAVswitches (hydro_ve/av_switches.hpp:81-86)
SPHGB_DROPIN_PASS(computeAVswitches, sphgb_compute_av_switches)
#undef SPHGB_DROPIN_PASS

//! sph::computeMomentumEnergySTD (hydro_std/momentum_energy.hpp:96-101); sets d.minDtCourant
template<class GroupView, class Dataset, class Box>
void computeMomentumEnergySTD(const GroupView& grp, Dataset& d, const Box& /*box*/)
{
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    double dt = 0;
    check(sphgb_compute_momentum_energy_std(c, &p, int64_t(grp.firstBody), int64_t(grp.lastBody), &dt),
          "computeMomentumEnergySTD");
    d.minDtCourant = dt;
}

//! sph::computeMomentumEnergy<avClean> (hydro_ve/momentum_energy.hpp:107-115); groupDt per 32-particle group
template<bool avClean, class GroupView, class Dataset, class Box>
void computeMomentumEnergy(const GroupView& grp, float* groupDt, Dataset& d, const Box& /*box*/)
{
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    double dt = 0;
    check(sphgb_compute_momentum_energy(c, &p, int64_t(grp.firstBody), int64_t(grp.lastBody), avClean ? 1 : 0,
                                        groupDt, &dt),
          "computeMomentumEnergy");
    d.minDtCourant = dt;
}

//! sph::computeEOS, ideal gas (hydro_ve/eos.hpp:191-197)
template<class Dataset>
void computeEOS(std::size_t startIndex, std::size_t endIndex, Dataset& d)
{
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    check(sphgb_compute_eos(c, &p, int64_t(startIndex), int64_t(endIndex)), "computeEOS");
}

//! sph::computeEOS_HydroStd, ideal gas (hydro_std/eos.hpp:147-152)
template<class Dataset>
void computeEOS_HydroStd(std::size_t startIndex, std::size_t endIndex, Dataset& d)
{
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    check(sphgb_compute_eos_std(c, &p, int64_t(startIndex), int64_t(endIndex)), "computeEOS_HydroStd");
}

// ---- time integration and reductions ----

template<class Dataset>
sphgb_timestep timestepOf(const Dataset& d)
{
    sphgb_timestep ts{};
    ts.minDt = double(d.minDt);
    ts.minDt_m1 = double(d.minDt_m1);
    ts.ttot = double(d.ttot);
    ts.minDtCourant = double(d.minDtCourant);
    ts.minDtRho = double(d.minDtRho);
    ts.maxDtIncrease = double(Dataset::maxDtIncrease);
    ts.g = double(d.g);
    ts.etaAcc = double(d.etaAcc);
    ts.eps = double(d.eps);
    return ts;
}

//! sph::computePositions (positions.hpp:180-200), every particle on the step d.minDt (no rungs)
template<class GroupView, class Dataset, class Box>
void computePositions(const GroupView& grp, Dataset& d, const Box& box)
{
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    auto& dv = d.devData;
    const sphgb_box b = toBox(box);
    const sphgb_timestep ts = timestepOf(d);
    check(sphgb_compute_positions(c, &p, &b, ptr(dv.x_m1), ptr(dv.y_m1), ptr(dv.z_m1), ptr(dv.du_m1), &ts,
                                  int64_t(grp.firstBody), int64_t(grp.lastBody)),
          "computePositions");
}

//! sph::updateSmoothingLength (update_h.hpp:26-45)
template<class GroupView, class Dataset>
void updateSmoothingLength(const GroupView& grp, Dataset& d)
{
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    check(sphgb_update_smoothing_length(c, &p, int64_t(grp.firstBody), int64_t(grp.lastBody)),
          "updateSmoothingLength");
}

//! sph::rhoTimestep (ts_global.hpp:72-95)
template<class Dataset>
double rhoTimestep(std::size_t first, std::size_t last, Dataset& d)
{
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    double dt = 0;
    check(sphgb_rho_timestep(c, &p, int64_t(first), int64_t(last), double(d.Krho), &dt), "rhoTimestep");
    return dt;
}

//! sph::computeTimestep at one rank (ts_global.hpp:97-113): updates d.ttot, d.minDt_m1, d.minDt
template<class Dataset>
void computeTimestep(std::size_t first, std::size_t last, Dataset& d)
{
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    sphgb_timestep ts = timestepOf(d);
    check(sphgb_compute_timestep(c, &p, int64_t(first), int64_t(last), &ts), "computeTimestep");
    d.ttot = ts.ttot;
    d.minDt_m1 = ts.minDt_m1;
    d.minDt = ts.minDt;
}

//! sphexa::localConservedQuantities (conserved_quantities.hpp:49-113): {eKin, eInt, linmom, angmom}
template<class Dataset>
std::tuple<double, double, std::array<double, 3>, std::array<double, 3>>
localConservedQuantities(std::size_t first, std::size_t last, Dataset& d)
{
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    double o[8];
    check(sphgb_conserved_quantities(c, &p, int64_t(first), int64_t(last), o), "localConservedQuantities");
    return {o[0], o[1], {o[2], o[3], o[4]}, {o[5], o[6], o[7]}};
}

/*! Gradients of one forward pass sequence (no reference counterpart).  Seeds and results are device
 *  arrays of n doubles in SFC order (a null seed counts as zero); the lists are those of the last
 *  neighbour search, the state that of the last forward passes (FP64 fields). */
struct Seeds {
    const double *rho = nullptr, *ax = nullptr, *ay = nullptr, *az = nullptr, *du = nullptr;
};
struct Grads {
    double *x, *y, *z, *vx, *vy, *vz, *h, *u;
};

//! adjoint of the std chain computeDensity -> computeEOS_HydroStd -> computeIAD -> computeMomentumEnergySTD
template<class Dataset>
void adjointStd(Dataset& d, const Seeds& s, const Grads& g, bool deterministic = false)
{
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    sphgb_seeds sd{s.rho, s.ax, s.ay, s.az, s.du};
    sphgb_grads gr{g.x, g.y, g.z, g.vx, g.vy, g.vz, g.h, g.u};
    check(sphgb_adjoint_std(c, &p, &sd, &gr, deterministic ? 1 : 0), "adjointStd");
}

/*! adjoint of the VE chain computeXMass -> computeVeDefGradh -> computeEOS -> computeIadDivvCurlv ->
 *  computeAVswitches -> computeMomentumEnergy<avClean>; alphaPrev: a device copy of alpha taken
 *  before computeAVswitches (which updates alpha in place) */
template<bool avClean, class Dataset>
void adjointVe(Dataset& d, const double* alphaPrev, const Seeds& s, const Grads& g, bool deterministic = false)
{
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    sphgb_seeds sd{s.rho, s.ax, s.ay, s.az, s.du};
    sphgb_grads gr{g.x, g.y, g.z, g.vx, g.vy, g.vz, g.h, g.u};
    check(sphgb_adjoint_ve(c, &p, alphaPrev, avClean ? 1 : 0, &sd, &gr, deterministic ? 1 : 0), "adjointVe");
}

}  // namespace dropin
}  // namespace sphgb
