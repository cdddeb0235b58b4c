/* Reference-compiled oracle: implements oracle_sweep() by calling the reference's own CPU
 * code (cstone + sph headers) unmodified.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled by oracle/ref/Makefile from the reference sources
 * where they lie, into oracle/_ref/ (git-ignored); it exists only on a machine that holds the
 * reference.  With -I override_fp64 first on the include path every hydro field is double
 * (libref_fp64.so); without it the reference's default float hydro types apply
 * (libref_f32.so).  Call sequence follows domain/test/unit/neighbors/findneighbors.cpp:61-82
 * for the tree, sph/include/sph/find_neighbors.hpp:10-44 for the neighbours, and
 * main/src/propagator/{std_hydro.hpp:124-168, ve_hydro.hpp:130-204} for the pair passes.
 */
#include "../oracle_api.h"

#include <omp.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <span>
#include <vector>

#include "cstone/findneighbors.hpp"
#include "cstone/focus/octree_focus.hpp"
#include "cstone/focus/source_center.hpp"
#include "cstone/primitives/gather.hpp"
#include "cstone/sfc/sfc.hpp"
#include "cstone/tree/csarray.hpp"
#include "cstone/tree/octree.hpp"
#include "cstone/traversal/groups.hpp"

#include "sph/particles_data.hpp"
#include "sph/find_neighbors.hpp"
#include "sph/hydro_std/density.hpp"
#include "sph/hydro_std/eos.hpp"
#include "sph/hydro_std/iad.hpp"
#include "sph/hydro_std/momentum_energy.hpp"
#include "sph/hydro_ve/xmass.hpp"
#include "sph/hydro_ve/ve_def_gradh.hpp"
#include "sph/hydro_ve/eos.hpp"
#include "sph/hydro_ve/iad_divv_curlv.hpp"
#include "sph/hydro_ve/av_switches.hpp"
#include "sph/hydro_ve/momentum_energy.hpp"
#include "sph/positions.hpp"

using KeyType = uint64_t;
using Dataset = sphexa::ParticlesData<cstone::CpuTag>;

template<class V>
static void fromSorted(V& dst, const double* src, const std::vector<uint32_t>& order)
{
    dst.resize(order.size());
    for (size_t i = 0; i < order.size(); ++i)
        dst[i] = src ? static_cast<typename V::value_type>(src[order[i]]) : typename V::value_type(0);
}

template<class V>
static void toOut(double* dst, const V& src, size_t n)
{
    if (!dst) return;
    if (src.size() < n) { std::fill(dst, dst + n, 0.0); return; }
    for (size_t i = 0; i < n; ++i) dst[i] = double(src[i]);
}

extern "C" double oracle_kernel_K(double sincIndex)
{
    return sph::kernel_3D_k(sph::getSphKernel(sph::SphKernelType::sinc_n, sincIndex), 2.0);
}

extern "C" void oracle_tables(double sincIndex, double* wh, double* whd)
{
    auto a = sph::tabulateFunction<double, sph::lt::kTableSize>(sph::getSphKernel(sph::SphKernelType::sinc_n, sincIndex),
                                                               0.0, 2.0);
    auto b = sph::tabulateFunction<double, sph::lt::kTableSize>(
        sph::getSphKernelDerivative(sph::SphKernelType::sinc_n, sincIndex), 0.0, 2.0);
    std::copy(a.begin(), a.end(), wh);
    std::copy(b.begin(), b.end(), whd);
}

extern "C" int oracle_sweep(const oracle_in* in, oracle_out* out)
{
    if (in->nthreads > 0) omp_set_num_threads(in->nthreads);
    out->threads_used = omp_get_max_threads();
    const size_t n = size_t(in->n);
    auto bt = [](uint8_t b) { return b == 1 ? cstone::BoundaryType::periodic : cstone::BoundaryType::open; };

    double lim[6];
    std::memcpy(lim, in->box, sizeof(lim));
    if (in->fit_box && n > 0)
    {
        const double* c[3] = {in->f[OF_X], in->f[OF_Y], in->f[OF_Z]};
        for (int d = 0; d < 3; ++d)
        {
            if (in->bc[d] == 1) continue;
            auto mm        = std::minmax_element(c[d], c[d] + n);
            lim[2 * d]     = *mm.first;
            lim[2 * d + 1] = *mm.second;
        }
    }
    std::memcpy(out->box, lim, sizeof(lim));
    cstone::Box<double> box(lim[0], lim[1], lim[2], lim[3], lim[4], lim[5], bt(in->bc[0]), bt(in->bc[1]),
                            bt(in->bc[2]));

    double t0 = omp_get_wtime();
    std::vector<KeyType> keys(n);
    cstone::computeSfcKeys(in->f[OF_X], in->f[OF_Y], in->f[OF_Z], cstone::sfcKindPointer(keys.data()), n, box);
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    cstone::sort_by_key(keys.begin(), keys.end(), order.begin());

    Dataset d;
    d.ng0   = in->ng0;
    d.ngmax = in->ngmax;
    d.gamma = in->gamma;
    d.Kcour = in->Kcour;
    d.minDt = in->minDt;
    d.alphamin       = in->alphamin;
    d.alphamax       = in->alphamax;
    d.decay_constant = in->decay;
    fromSorted(d.x, in->f[OF_X], order);
    fromSorted(d.y, in->f[OF_Y], order);
    fromSorted(d.z, in->f[OF_Z], order);
    fromSorted(d.h, in->f[OF_H], order);
    fromSorted(d.m, in->f[OF_M], order);
    fromSorted(d.u, in->f[OF_U], order);
    fromSorted(d.vx, in->f[OF_VX], order);
    fromSorted(d.vy, in->f[OF_VY], order);
    fromSorted(d.vz, in->f[OF_VZ], order);
    fromSorted(d.alpha, in->f[OF_ALPHA], order);
    double t1   = omp_get_wtime();
    out->t_keys = t1 - t0;
    if (out->keys) std::memcpy(out->keys, keys.data(), sizeof(KeyType) * n);
    if (out->order) std::memcpy(out->order, order.data(), sizeof(uint32_t) * n);

    auto [csTree, counts] = cstone::computeOctree<KeyType>(std::span<const KeyType>(keys), in->bucket);
    cstone::OctreeData<KeyType, cstone::CpuTag> octree;
    octree.resize(cstone::nNodes(csTree));
    cstone::updateInternalTree<KeyType>(csTree, octree.data());
    std::vector<cstone::LocalIndex> layout(cstone::nNodes(csTree) + 1, 0);
    std::inclusive_scan(counts.begin(), counts.end(), layout.begin() + 1);
    std::span<const KeyType> nodeKeys(octree.prefixes.data(), octree.numNodes);
    std::vector<cstone::Vec3<double>> centers(octree.numNodes), sizes(octree.numNodes);
    cstone::nodeFpCenters<KeyType>(nodeKeys, centers.data(), sizes.data(), box);
    cstone::OctreeNsView<double, KeyType> view{octree.numLeafNodes,          octree.prefixes.data(),
                                               octree.childOffsets.data(),   octree.internalToLeaf.data(),
                                               octree.levelRange.data(),     csTree.data(),
                                               layout.data(),                centers.data(),
                                               sizes.data()};
    int64_t L         = int64_t(cstone::nNodes(csTree));
    out->num_leaves   = L;
    out->num_nodes    = octree.numNodes;
    out->num_internal = octree.numInternalNodes;
    for (int l = 0; l < 23; ++l)
        out->level_range[l] = octree.levelRange[l];
    if (out->leaves && out->leaves_cap >= L + 1) std::memcpy(out->leaves, csTree.data(), sizeof(KeyType) * (L + 1));
    if (out->counts && out->leaves_cap >= L) std::memcpy(out->counts, counts.data(), sizeof(unsigned) * L);
    if (out->nodes_cap >= octree.numNodes)
    {
        if (out->prefixes) std::memcpy(out->prefixes, octree.prefixes.data(), sizeof(KeyType) * octree.numNodes);
        if (out->child_offsets)
            std::memcpy(out->child_offsets, octree.childOffsets.data(), sizeof(int32_t) * octree.numNodes);
        if (out->internal_to_leaf)
            std::memcpy(out->internal_to_leaf, octree.internalToLeaf.data(), sizeof(int32_t) * octree.numNodes);
        if (out->centers) std::memcpy(out->centers, centers.data(), sizeof(double) * 3 * octree.numNodes);
        if (out->sizes) std::memcpy(out->sizes, sizes.data(), sizeof(double) * 3 * octree.numNodes);
    }
    double t2   = omp_get_wtime();
    out->t_tree = t2 - t1;

    d.treeView = view;
    d.nc.assign(n, 1);
    d.neighbors.assign(n * in->ngmax, 0);
    out->h_iter_fails = -1; /* the reference prints the count but does not return it */
    if (in->stages & (OS_NBR | OS_HYDRO))
    {
        sph::findNeighborsSph(d.x.data(), d.y.data(), d.z.data(), d.h.data(), 0, cstone::LocalIndex(n), box, view,
                              d.ng0, d.ngmax, d.neighbors.data(), d.nc.data());
        if (out->nc) std::memcpy(out->nc, d.nc.data(), sizeof(uint32_t) * n);
        if (out->nbr) std::memcpy(out->nbr, d.neighbors.data(), sizeof(uint32_t) * n * in->ngmax);
    }
    double t3  = omp_get_wtime();
    out->t_nbr = t3 - t2;

    out->minDtCourant = INFINITY;
    if (in->stages & OS_HYDRO)
    {
        d.sincIndex = in->sincIndex; /* tables were built with the default sinc index 6 */
        cstone::GroupView grp{0, cstone::LocalIndex(n), 1, nullptr, nullptr};
        auto sz = [n](auto&... v) { (v.resize(n), ...); };
        if (in->variant == 0)
        {
            sz(d.rho, d.p, d.c, d.c11, d.c12, d.c13, d.c22, d.c23, d.c33, d.ax, d.ay, d.az, d.du, d.xm);
            sph::computeDensity(grp, d, box);
            sph::computeEOS_HydroStd(0, n, d);
            sph::computeIAD(grp, d, box);
            sph::computeMomentumEnergySTD(grp, d, box);
        }
        else
        {
            sz(d.xm, d.kx, d.gradh, d.prho, d.c, d.rho, d.p, d.c11, d.c12, d.c13, d.c22, d.c23, d.c33, d.divv,
               d.curlv, d.ax, d.ay, d.az, d.du);
            if (in->avclean) sz(d.dV11, d.dV12, d.dV13, d.dV22, d.dV23, d.dV33);
            sph::computeXMass(grp, d, box);
            sph::computeVeDefGradh(grp, d, box);
            sph::computeEOS(0, n, d);
            sph::computeIadDivvCurlv(grp, d, box);
            sph::computeAVswitches(grp, d, box);
            if (in->avclean) sph::computeMomentumEnergy<true>(grp, nullptr, d, box);
            else sph::computeMomentumEnergy<false>(grp, nullptr, d, box);
        }
        out->minDtCourant = d.minDtCourant;
    }
    out->t_hydro = omp_get_wtime() - t3;

    toOut(out->f[OF_X], d.x, n);
    toOut(out->f[OF_Y], d.y, n);
    toOut(out->f[OF_Z], d.z, n);
    toOut(out->f[OF_H], d.h, n);
    toOut(out->f[OF_M], d.m, n);
    toOut(out->f[OF_U], d.u, n);
    toOut(out->f[OF_VX], d.vx, n);
    toOut(out->f[OF_VY], d.vy, n);
    toOut(out->f[OF_VZ], d.vz, n);
    toOut(out->f[OF_ALPHA], d.alpha, n);
    toOut(out->f[OF_RHO], d.rho, n);
    toOut(out->f[OF_P], d.p, n);
    toOut(out->f[OF_C], d.c, n);
    toOut(out->f[OF_C11], d.c11, n);
    toOut(out->f[OF_C12], d.c12, n);
    toOut(out->f[OF_C13], d.c13, n);
    toOut(out->f[OF_C22], d.c22, n);
    toOut(out->f[OF_C23], d.c23, n);
    toOut(out->f[OF_C33], d.c33, n);
    toOut(out->f[OF_AX], d.ax, n);
    toOut(out->f[OF_AY], d.ay, n);
    toOut(out->f[OF_AZ], d.az, n);
    toOut(out->f[OF_DU], d.du, n);
    toOut(out->f[OF_XM], d.xm, n);
    toOut(out->f[OF_KX], d.kx, n);
    toOut(out->f[OF_GRADH], d.gradh, n);
    toOut(out->f[OF_PRHO], d.prho, n);
    toOut(out->f[OF_DIVV], d.divv, n);
    toOut(out->f[OF_CURLV], d.curlv, n);
    toOut(out->f[OF_DV11], d.dV11, n);
    toOut(out->f[OF_DV12], d.dV12, n);
    toOut(out->f[OF_DV13], d.dV13, n);
    toOut(out->f[OF_DV22], d.dV22, n);
    toOut(out->f[OF_DV23], d.dV23, n);
    toOut(out->f[OF_DV33], d.dV33, n);
    return 0;
}

/* the reference j-loops themselves, as sph/test/std.cpp and sph/test/ve.cpp call them */
extern "C" int oracle_jloop(const oracle_jloop_in* in, double* out)
{
    using T         = sph::SphTypes::HydroType;
    const size_t n  = size_t(in->n);
    std::vector<std::vector<T>> f(OF_NFIELDS, std::vector<T>(n, T(0)));
    std::vector<double> xyz[3];
    for (int k = 0; k < OF_NFIELDS; ++k)
        if (in->f[k])
            for (size_t i = 0; i < n; ++i)
                f[k][i] = T(in->f[k][i]);
    for (int k = 0; k < 3; ++k)
        xyz[k].assign(in->f[k] ? in->f[k] : nullptr, in->f[k] ? in->f[k] + n : nullptr);
    auto bt = [](uint8_t b) { return b == 1 ? cstone::BoundaryType::periodic : cstone::BoundaryType::open; };
    cstone::Box<double> box(in->box[0], in->box[1], in->box[2], in->box[3], in->box[4], in->box[5], bt(in->bc[0]),
                            bt(in->bc[1]), bt(in->bc[2]));
    auto wh = sph::tabulateFunction<T, sph::lt::kTableSize>(
        sph::getSphKernel(sph::SphKernelType::sinc_n, in->sincIndex), 0.0, 2.0);
    auto whd = sph::tabulateFunction<T, sph::lt::kTableSize>(
        sph::getSphKernelDerivative(sph::SphKernelType::sinc_n, in->sincIndex), 0.0, 2.0);
    const double K  = in->K;
    const auto* nb  = in->neighbors;
    const unsigned c = in->count;
    const double *x = xyz[0].data(), *y = xyz[1].data(), *z = xyz[2].data();
    auto F          = [&](int k) { return f[k].data(); };
    T r[8]          = {0, 0, 0, 0, 0, 0, 0, 0};
    switch (in->loop)
    {
        case OJ_XMASS:
            out[0] = sph::xmassJLoop(0, K, box, nb, c, x, y, z, F(OF_H), F(OF_M), wh.data(), whd.data());
            break;
        case OJ_GRADH:
        {
            auto [kx, gradh] = sph::veDefGradhJLoop(0, K, box, nb, c, x, y, z, F(OF_H), F(OF_M), wh.data(),
                                                    whd.data(), F(OF_XM));
            out[0] = kx;
            out[1] = gradh;
            break;
        }
        case OJ_IAD_STD:
            sph::IADJLoopSTD(0, K, box, nb, c, x, y, z, F(OF_H), F(OF_M), F(OF_RHO), wh.data(), whd.data(), &r[0],
                             &r[1], &r[2], &r[3], &r[4], &r[5]);
            for (int q = 0; q < 6; ++q)
                out[q] = r[q];
            break;
        case OJ_IAD_VE:
            sph::IADJLoop(0, K, box, nb, c, x, y, z, F(OF_H), wh.data(), whd.data(), F(OF_XM), F(OF_KX), &r[0], &r[1],
                          &r[2], &r[3], &r[4], &r[5]);
            for (int q = 0; q < 6; ++q)
                out[q] = r[q];
            break;
        case OJ_DIVV:
            sph::divV_curlVJLoop(0, K, box, nb, c, x, y, z, F(OF_VX), F(OF_VY), F(OF_VZ), F(OF_H), F(OF_C11),
                                 F(OF_C12), F(OF_C13), F(OF_C22), F(OF_C23), F(OF_C33), wh.data(), whd.data(),
                                 F(OF_KX), F(OF_XM), &r[0], &r[1], &r[2], &r[3], &r[4], &r[5], &r[6], &r[7], true);
            for (int q = 0; q < 8; ++q)
                out[q] = r[q];
            break;
        case OJ_AV:
            out[0] = sph::AVswitchesJLoop(0, K, box, nb, c, x, y, z, F(OF_VX), F(OF_VY), F(OF_VZ), F(OF_H), F(OF_C),
                                          F(OF_C11), F(OF_C12), F(OF_C13), F(OF_C22), F(OF_C23), F(OF_C33), wh.data(),
                                          whd.data(), F(OF_KX), F(OF_XM), F(OF_DIVV), in->dt, T(in->alphamin),
                                          T(in->alphamax), T(in->decay), F(OF_ALPHA)[0]);
            break;
        case OJ_ME_STD:
        {
            T du = 0;
            sph::momentumAndEnergyJLoop(0, K, box, nb, c, x, y, z, F(OF_VX), F(OF_VY), F(OF_VZ), F(OF_H), F(OF_M),
                                        F(OF_RHO), F(OF_P), F(OF_C), F(OF_C11), F(OF_C12), F(OF_C13), F(OF_C22),
                                        F(OF_C23), F(OF_C33), wh.data(), whd.data(), &r[0], &r[1], &r[2], &du, &r[4]);
            out[0] = r[0];
            out[1] = r[1];
            out[2] = r[2];
            out[3] = du;
            out[4] = r[4];
            break;
        }
        case OJ_ME_VE:
        {
            T du = 0;
            const T Atmin = 0.1, Atmax = 0.2, ramp = 1.0 / (Atmax - Atmin);
            auto call     = [&](auto avc)
            {
                sph::momentumAndEnergyJLoop<decltype(avc)::value>(
                    0, K, box, nb, c, x, y, z, F(OF_VX), F(OF_VY), F(OF_VZ), F(OF_H), F(OF_M), F(OF_PRHO),
                    (const T*)nullptr, F(OF_C), F(OF_C11), F(OF_C12), F(OF_C13), F(OF_C22), F(OF_C23), F(OF_C33),
                    Atmin, Atmax, ramp, wh.data(), F(OF_KX), F(OF_XM), F(OF_ALPHA), F(OF_DV11), F(OF_DV12), F(OF_DV13),
                    F(OF_DV22), F(OF_DV23), F(OF_DV33), &r[0], &r[1], &r[2], &du, &r[4]);
            };
            if (in->avclean) call(std::true_type{});
            else call(std::false_type{});
            out[0] = r[0];
            out[1] = r[1];
            out[2] = r[2];
            out[3] = du;
            out[4] = r[4];
            break;
        }
        default: return 2;
    }
    return 0;
}

/* ---- one integration step through the reference's own functions ----
 * sph::positionUpdate, sph::energyUpdate, sph::fbcCheck (sph/include/sph/positions.hpp:46-85), in the
 * loop structure of the GPU kernel (positions_gpu.cu:118-165), and sph::updateH (kernels.hpp:26-32). */
extern "C" int oracle_positions(int64_t n, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                                const double* ax, const double* ay, const double* az, double* xm1, double* ym1,
                                double* zm1, double* u, const double* du, double* dum1, const double* h, double dt,
                                double dt_m1, const double box[6], const uint8_t bc[3])
{
    auto bt = [](uint8_t b) {
        return b == 1 ? cstone::BoundaryType::periodic : (b == 2 ? cstone::BoundaryType::fixed : cstone::BoundaryType::open);
    };
    cstone::Box<double> B(box[0], box[1], box[2], box[3], box[4], box[5], bt(bc[0]), bt(bc[1]), bt(bc[2]));
    const bool fbcX = B.boundaryX() == cstone::BoundaryType::fixed, fbcY = B.boundaryY() == cstone::BoundaryType::fixed,
               fbcZ = B.boundaryZ() == cstone::BoundaryType::fixed;
    const bool anyFBC = fbcX || fbcY || fbcZ;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        if (anyFBC && vx[i] == 0.0 && vy[i] == 0.0 && vz[i] == 0.0 &&
            (sph::fbcCheck(x[i], h[i], B.xmax(), B.xmin(), fbcX) || sph::fbcCheck(y[i], h[i], B.ymax(), B.ymin(), fbcY) ||
             sph::fbcCheck(z[i], h[i], B.zmax(), B.zmin(), fbcZ)))
            continue;
        cstone::Vec3<double> A{ax[i], ay[i], az[i]}, X{x[i], y[i], z[i]}, Xm1{xm1[i], ym1[i], zm1[i]}, V;
        util::tie(X, V, Xm1) = sph::positionUpdate(dt, dt_m1, X, A, Xm1, B);
        x[i] = X[0], y[i] = X[1], z[i] = X[2];
        xm1[i] = Xm1[0], ym1[i] = Xm1[1], zm1[i] = Xm1[2];
        vx[i] = V[0], vy[i] = V[1], vz[i] = V[2];
        if (u) {
            u[i] = sph::energyUpdate(u[i], dt, dt_m1, du[i], dum1[i]);
            dum1[i] = du[i];
        }
    }
    return 0;
}

extern "C" int oracle_update_h(int64_t n, uint32_t ng0, const uint32_t* nc, double* h)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) h[i] = sph::updateH(ng0, nc[i], h[i]);
    return 0;
}

/* conserved_quantities.hpp includes <mpi.h> and cannot be compiled here: the restatement of the
 * port is the only implementation of oracle_conserved (pinned by tests against numpy sums) */
extern "C" int oracle_conserved(int64_t n, const double* x, const double* y, const double* z, const double* vx,
                                const double* vy, const double* vz, const double* m, const double* u, double out[8])
{
    double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = 0; i < n; ++i) {
        cstone::Vec3<double> X{x[i], y[i], z[i]}, V{vx[i], vy[i], vz[i]};
        s[0] += m[i] * norm2(V);
        s[1] += u ? u[i] * m[i] : 0.0;
        auto L = cross(X, V);
        for (int k = 0; k < 3; ++k) {
            s[2 + k] += m[i] * V[k];
            s[5 + k] += m[i] * L[k];
        }
    }
    out[0] = 0.5 * s[0];
    for (int q = 1; q < 8; ++q) out[q] = s[q];
    return 0;
}

/* cstone::limitBoxShrinking (domain/include/cstone/sfc/box.hpp:397-414) on limits only */
extern "C" int oracle_limit_box_shrinking(const double fit[6], const double prev[6], double out[6])
{
    using B = cstone::Box<double>;
    B f(fit[0], fit[1], fit[2], fit[3], fit[4], fit[5], cstone::BoundaryType::open, cstone::BoundaryType::open,
        cstone::BoundaryType::open);
    B p(prev[0], prev[1], prev[2], prev[3], prev[4], prev[5], cstone::BoundaryType::open, cstone::BoundaryType::open,
        cstone::BoundaryType::open);
    B r = cstone::limitBoxShrinking(f, p);
    const double o[6] = {r.xmin(), r.xmax(), r.ymin(), r.ymax(), r.zmin(), r.zmax()};
    for (int k = 0; k < 6; ++k) out[k] = o[k];
    return 0;
}

/* The single-rank focus tree across the syncs of one simulation: FocusedOctree
 * (domain/include/cstone/focus/octree_focus_mpi.hpp:40-253) driven as Domain::sync does
 * (domain/domain.hpp:199-211): converge() at the first sync, then updateMinMac + updateTree +
 * updateCounts at every sync.  One rank: the focus range is the whole key range, there are no peers
 * and every leaf count comes from the local keys; the rebalance itself is the reference's
 * CombinedUpdate::updateFocus (focus/octree_focus.hpp:65-113).  keys: the sorted keys of each step,
 * n per step.  leaves_out: the cornerstone leaves after each step, concatenated (at most cap keys);
 * nleaves[s]: the number of leaf cells of step s. */
extern "C" int oracle_focus_steps(int64_t n, int32_t steps, const uint64_t* keys, uint32_t bucket,
                                  uint64_t* leaves_out, int64_t cap, int64_t* nleaves)
{
    using K = uint64_t;
    std::vector<K> leaves{0, cstone::nodeRange<K>(0)};
    cstone::OctreeData<K, cstone::CpuTag> tree;
    tree.resize(cstone::nNodes(leaves));
    cstone::updateInternalTree<K>(leaves, tree.data());
    std::vector<unsigned> counts{bucket + 1};  // the constructor's root count forces the first split
    std::vector<char> macs(1, 1);
    std::vector<unsigned> leafCounts;
    auto updateCounts = [&](const K* k) {
        leafCounts.assign(cstone::nNodes(leaves), 0);
        cstone::computeNodeCounts<K>(leaves.data(), leafCounts.data(), cstone::nNodes(leaves), std::span<const K>(k, n),
                                     std::numeric_limits<unsigned>::max(), true);
        counts.assign(tree.numNodes, 0);
        cstone::scatter<cstone::TreeNodeIndex>(cstone::leafToInternal(tree), leafCounts.data(), counts.data());
        cstone::upsweep(tree.levelRange, tree.childOffsets, counts.data(), cstone::NodeCount<unsigned>{});
    };
    auto updateTree = [&]() {
        macs.assign(tree.numNodes, 0);  // updateMinMac: no node lies outside the focus at one rank
        return cstone::CombinedUpdate<K>::updateFocus(tree, leaves, bucket, K(0), cstone::nodeRange<K>(0), {}, counts,
                                                     macs);
    };
    int64_t used = 0;
    for (int32_t s = 0; s < steps; ++s) {
        const K* k = keys + int64_t(s) * n;
        if (s == 0) {
            bool converged = false;
            while (!converged) {
                converged = updateTree();
                updateCounts(k);
            }
        }
        updateTree();
        updateCounts(k);
        if (used + int64_t(leaves.size()) > cap) return 1;
        std::copy(leaves.begin(), leaves.end(), leaves_out + used);
        used += int64_t(leaves.size());
        nleaves[s] = int64_t(leaves.size()) - 1;
    }
    return 0;
}
