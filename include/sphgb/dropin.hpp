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
    // momentumAndEnergyJLoop takes the energy coefficient from tdpdTrho when that field is active
    // (hydro_ve/momentum_energy_kern.hpp:213-214); this library always uses prho, so an active
    // tdpdTrho (a non-ideal equation of state) is refused instead of giving a different du
    if (dv.tdpdTrho.size() != 0)
        throw std::runtime_error("sphgb: the tdpdTrho field is active; only the ideal-gas energy coefficient "
                                 "prho is supported");
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

//! the tree summary the propagators print (ipropagator.hpp:108,124-125): leaf count and depth
struct TreeSummary {
    struct View {
        int64_t numLeafNodes;
    };
    int64_t leaves = 0;
    int maxDepth = 0;
    int64_t numLeafNodes() const { return leaves; }
    View octreeViewAcc() const { return {leaves}; }
    int depth() const { return maxDepth; }
};

/*! Domain::octreeProperties at one rank: converts to the caller's cstone::OctreeNsView<T, KeyType>
 *  (tree/octree.hpp:279-300) member by member; every pointer is device memory of the context, valid
 *  until the next sync.  searchExtFactor keeps its default 1 (the tree is converged at every sync
 *  of domain mode 1 that rebuilds it, and the search does not read it). */
struct OctreeNsViewProxy {
    sphgb_octree_view v;
    template<class View>
    operator View() const
    {
        View o{};
        static_assert(sizeof(*o.prefixes) == sizeof(uint64_t), "the tree is built on 64-bit SFC keys");
        static_assert(sizeof(*o.centers) == 3 * sizeof(double), "node centers are FP64 Vec3");
        o.numLeafNodes = decltype(o.numLeafNodes)(v.num_leaf_nodes);
        o.prefixes = reinterpret_cast<decltype(o.prefixes)>(v.prefixes);
        o.childOffsets = reinterpret_cast<decltype(o.childOffsets)>(v.child_offsets);
        o.internalToLeaf = reinterpret_cast<decltype(o.internalToLeaf)>(v.internal_to_leaf);
        o.levelRange = reinterpret_cast<decltype(o.levelRange)>(v.level_range);
        o.leaves = reinterpret_cast<decltype(o.leaves)>(v.leaves);
        o.layout = reinterpret_cast<decltype(o.layout)>(v.layout);
        o.centers = reinterpret_cast<decltype(o.centers)>(v.centers);
        o.sizes = reinterpret_cast<decltype(o.sizes)>(v.sizes);
        return o;
    }
};

/*! cstone::Domain at one rank (domain/include/cstone/domain/domain.hpp:181-234, 372-428) with the
 *  surface HydroVeProp / HydroProp use (main/src/propagator/ve_hydro.hpp:119-217,
 *  std_hydro.hpp:110-170, ipropagator.hpp:104-130):
 *   sync(keys, x, y, z, h, tuple<properties...>, tuple<scratch...>) fits the box, sorts by Hilbert
 *     key, permutes x y z h and every property, writes the sorted keys and builds the cornerstone
 *     tree with bucketSizeFocus; the syncs of one domain are the steps of one simulation (box shrink
 *     limit and focus-tree update, domain mode 1).  Scratch buffers are not needed (the context
 *     owns its scratch) and keep their contents.
 *   startIndex() = 0, endIndex() = nParticles() = nParticlesWithHalos() = particles of the last sync;
 *   octreeProperties(), box(), globalTree(), focusTree(); exchangeHalos is a no-op (no halos). */
template<class KeyType, class T, class Box>
class SingleRankDomain
{
public:
    // the tree the reference's octreeProperties() exposes is its focus tree, refined to
    // bucketSizeFocus (domain/domain.hpp:416-428); the coarser global tree (bucketSize) only assigns
    // ranks, which has no counterpart at one rank, so globalTree() reports the focus tree too
    SingleRankDomain(int /*rank*/, int /*numRanks*/, unsigned /*bucketSize*/, unsigned bucketSizeFocus,
                     float /*theta*/, const Box& box, int device = 0)
        : box_(box)
        , bucket_(bucketSizeFocus)
        , device_(device)
    {
        static_assert(sizeof(KeyType) == sizeof(uint64_t), "the tree is built on 64-bit SFC keys");
    }

    //! Domain::sync (domain.hpp:181-234) at one rank
    template<class KeyVec, class VectorX, class VectorH, class... Props, class... Scratch>
    void sync(KeyVec& keys, VectorX& x, VectorX& y, VectorX& z, VectorH& h, std::tuple<Props&...> properties,
              std::tuple<Scratch&...> /*scratchBuffers*/)
    {
        static_assert(sizeof(*rawPtr(x)) == sizeof(double), "coordinates are FP64 (SphTypes::CoordinateType)");
        sphgb_ctx* c = context(device_);
        begin(c);
        const std::size_t n = x.size();
        if (y.size() != n || z.size() != n || h.size() != n) throw std::runtime_error("Domain::sync: field sizes differ");
        if (keys.size() < n) keys.resize(n);
        sphgb_particles q{};
        q.n = int64_t(n);
        q.precision = sizeof(*rawPtr(h)) == sizeof(double) ? SPHGB_FP64 : SPHGB_MIXED;
        q.keys = reinterpret_cast<uint64_t*>(ptr(keys));
        q.x = static_cast<double*>(ptr(x));
        q.y = static_cast<double*>(ptr(y));
        q.z = static_cast<double*>(ptr(z));
        q.h = ptr(h);
        sphgb_box b = toBox(box_);
        check(sphgb_domain_sync(c, &q, &b), "Domain::sync");
        std::apply([&](auto&... v) { (applyOrder(c, v, n), ...); }, properties);
        finish(c, b, n);
    }

    /*! the same sync over the conserved fields of a dataset (x y z h m u vx vy vz alpha and keys of
     *  its devData) plus any further device vectors to permute alike */
    template<class Dataset, class... Props>
    void syncDataset(Dataset& d, Props&... extraProperties)
    {
        auto& dv = d.devData;
        sync(dv.keys, dv.x, dv.y, dv.z, dv.h, std::tie(dv.m, dv.u, dv.vx, dv.vy, dv.vz, dv.alpha, extraProperties...),
             std::tuple<>{});
    }

    const Box& box() const { return box_; }
    uint32_t startIndex() const { return 0; }
    uint32_t endIndex() const { return uint32_t(n_); }
    uint32_t nParticles() const { return uint32_t(n_); }
    uint32_t nParticlesWithHalos() const { return uint32_t(n_); }
    const TreeSummary& globalTree() const { return tree_; }
    const TreeSummary& focusTree() const { return tree_; }

    OctreeNsViewProxy octreeProperties() const
    {
        OctreeNsViewProxy p{};
        check(sphgb_get_octree_view(context(device_), &p.v), "Domain::octreeProperties");
        return p;
    }

    template<class... Fields>
    void exchangeHalos(Fields&&...) const
    {
    }

private:
    void begin(sphgb_ctx* c)
    {
        if (!started_) {  // this domain's syncs are the steps of one simulation (box shrink limit)
            check(sphgb_set_domain_mode(c, 1), "sphgb_set_domain_mode");
            started_ = true;
        }
        sphgb_params prm{};
        check(sphgb_get_params(c, &prm), "sphgb_get_params");
        if (prm.bucket != bucket_) {
            prm.bucket = bucket_;
            check(sphgb_set_params(c, &prm), "sphgb_set_params");
        }
    }

    void finish(sphgb_ctx* c, const sphgb_box& b, std::size_t n)
    {
        box_ = Box(b.lim[0], b.lim[1], b.lim[2], b.lim[3], b.lim[4], b.lim[5], box_.boundaryX(), box_.boundaryY(),
                   box_.boundaryZ());
        n_ = n;
        sphgb_octree_view v{};
        check(sphgb_get_octree_view(c, &v), "Domain::octreeProperties");
        tree_.leaves = v.num_leaf_nodes;
        tree_.maxDepth = v.max_depth;
    }

    template<class V>
    static void applyOrder(sphgb_ctx* c, V& v, std::size_t n)
    {
        if (v.size() == 0) return;  // an inactive field
        if (v.size() != n) throw std::runtime_error("Domain::sync: a property's size differs from x");
        check(sphgb_apply_order(c, ptr(v), int32_t(sizeof(*rawPtr(v)))), "sphgb_apply_order");
    }

    Box box_;
    unsigned bucket_;
    int device_;
    bool started_ = false;
    std::size_t n_ = 0;
    TreeSummary tree_;
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

/*! sph::computeGroups on the GPU (sph/include/sph/groups.hpp:41-56): the target groups of the pair
 *  passes are the runs of 32 SFC-consecutive particles of [startIndex, endIndex) (one warp each);
 *  groups.data (a device vector) receives their numGroups + 1 boundaries and the view members point
 *  into it as in computeSpatialGroups, so groupDt and the rung logic of the propagators
 *  (ve_hydro_bdt.hpp) see numGroups groups */
template<class Dataset, class Box, class GroupData>
void computeGroups(std::size_t startIndex, std::size_t endIndex, Dataset& d, const Box&, GroupData& groups)
{
    sphgb_ctx* c = bind(d);
    int64_t ng = 0;
    check(sphgb_target_groups(c, int64_t(startIndex), int64_t(endIndex), nullptr, 0, &ng), "computeGroups");
    groups.data.resize(std::size_t(ng + 1));
    static_assert(sizeof(*rawPtr(groups.data)) == sizeof(uint32_t), "cstone::LocalIndex is 32-bit");
    check(sphgb_target_groups(c, int64_t(startIndex), int64_t(endIndex), reinterpret_cast<uint32_t*>(rawPtr(groups.data)),
                              ng + 1, &ng),
          "computeGroups");
    groups.firstBody = decltype(groups.firstBody)(startIndex);
    groups.lastBody = decltype(groups.lastBody)(endIndex);
    groups.numGroups = decltype(groups.numGroups)(ng);
    groups.groupStart = rawPtr(groups.data);
    groups.groupEnd = rawPtr(groups.data) + 1;
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

/*! sph::computePositions with the reference's argument list (positions.hpp:177-200): every particle
 *  on the step dt_forward after dt_m1[0] (the propagator passes d.minDt and {float(d.minDt_m1)}; a
 *  braced list becomes the reference's Timestep::maxNumRungs = 4 entries, sph/timestep.h:19);
 *  per-particle rungs are refused */
template<class GroupView, class Dataset, class Box, class DtM1 = std::array<float, 4>>
void computePositions(const GroupView& grp, Dataset& d, const Box& box, float dt_forward, const DtM1& dt_m1,
                      const uint8_t* rung = nullptr)
{
    if (rung) throw std::runtime_error("computePositions: per-particle time-step rungs are not supported");
    sphgb_ctx* c = bind(d);
    sphgb_particles p = particles(d);
    auto& dv = d.devData;
    const sphgb_box b = toBox(box);
    sphgb_timestep ts = timestepOf(d);
    ts.minDt = double(dt_forward);
    ts.minDt_m1 = double(dt_m1[0]);
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
