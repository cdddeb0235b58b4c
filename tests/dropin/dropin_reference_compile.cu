// Compile-only check of include/sphgb/dropin.hpp against the reference's own types: every adapter
// entry point the propagators call (main/src/propagator/ve_hydro.hpp:100-217, std_hydro.hpp:100-170)
// is instantiated over sphexa::ParticlesData<cstone::GpuTag>, cstone::GroupData<cstone::GpuTag>,
// cstone::Box<double> and cstone::OctreeNsView, as a maintainer's binding translation unit would.
// Built by tests/test_dropin.py with nvcc -c where the reference headers are present; never linked
// or run (the reference's DeviceVector implementation lives in its own compiled sources).
#include "cstone/sfc/box.hpp"
#include "cstone/traversal/groups.hpp"
#include "cstone/tree/octree.hpp"
#include "sph/particles_data.hpp"

#include "sphgb/dropin.hpp"

namespace dr = sphgb::dropin;

using Data   = sphexa::ParticlesData<cstone::GpuTag>;
using BoxT   = cstone::Box<double>;
using Groups = cstone::GroupData<cstone::GpuTag>;
using Domain = dr::SingleRankDomain<Data::KeyType, double, BoxT>;

void veStep(Domain& domain, Data& d, Groups& groups_)
{
    auto& dv = d.devData;
    domain.sync(dv.keys, dv.x, dv.y, dv.z, dv.h, std::tie(dv.m, dv.u, dv.vx, dv.vy, dv.vz, dv.alpha, dv.du_m1),
                std::tie(dv.rho, dv.p));
    d.treeView = domain.octreeProperties();
    std::size_t first = domain.startIndex(), last = domain.endIndex();
    (void)domain.nParticles();
    (void)domain.nParticlesWithHalos();
    (void)domain.globalTree().numLeafNodes();
    (void)domain.focusTree().octreeViewAcc().numLeafNodes;
    (void)domain.focusTree().depth();
    dr::findNeighborsSfc(first, last, d, domain.box());
    dr::computeGroups(first, last, d, domain.box(), groups_);
    dr::computeXMass(groups_.view(), d, domain.box());
    domain.exchangeHalos(std::tie(dv.xm), dv.ax, dv.keys);
    dr::computeVeDefGradh(groups_.view(), d, domain.box());
    dr::computeEOS(first, last, d);
    dr::computeIadDivvCurlv(groups_.view(), d, domain.box());
    d.minDtRho = dr::rhoTimestep(first, last, d);
    dr::computeAVswitches(groups_.view(), d, domain.box());
    dr::computeMomentumEnergy<true>(groups_.view(), nullptr, d, domain.box());
    dr::computeMomentumEnergy<false>(groups_.view(), nullptr, d, domain.box());
    dr::computeTimestep(first, last, d);
    dr::computePositions(groups_.view(), d, domain.box(), d.minDt, {float(d.minDt_m1)});
    dr::updateSmoothingLength(groups_.view(), d);
    auto [eKin, eInt, linmom, angmom] = dr::localConservedQuantities(first, last, d);
    (void)eKin;
}

void stdStep(Domain& domain, Data& d, Groups& groups_)
{
    std::size_t first = domain.startIndex(), last = domain.endIndex();
    dr::findNeighborsSfc(first, last, d, domain.box());
    dr::computeGroups(first, last, d, domain.box(), groups_);
    dr::computeDensity(groups_.view(), d, domain.box());
    dr::computeEOS_HydroStd(first, last, d);
    dr::computeIAD(groups_.view(), d, domain.box());
    dr::computeMomentumEnergySTD(groups_.view(), d, domain.box());
}

void adjoint(Data& d, const double* alphaPrev, const dr::Seeds& s, const dr::Grads& g)
{
    dr::adjointStd(d, s, g);
    dr::adjointVe<false>(d, alphaPrev, s, g);
}

Domain makeDomain(const BoxT& box) { return Domain(0, 1, 8192, 64, 0.5f, box); }
