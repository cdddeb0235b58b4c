// A VE and a std sweep written the way the reference's propagators call them
// (main/src/propagator/ve_hydro.hpp:130-204, std_hydro.hpp:124-168), through the drop-in adapter.
// Reads binary particle fields (x y z h m u vx vy vz alpha as FP64) from argv[1], writes the
// outputs in SFC order to argv[2].  Precision: "fp64" or "mixed" in argv[3], variant "ve"/"std" in argv[4];
// argv[3] = "adjoint": the VE adjoint check of runAdjoint instead.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mock_reference.hpp"
#include "sphgb/dropin.hpp"

using namespace mockref;
namespace dr = sphgb::dropin;

template<class V, class T>
void upload(V& dv, const std::vector<T>& host)
{
    dv.resize(host.size());
    cudaMemcpy(rawPtr(dv), host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice);
}

template<class V>
void download(V& dv, std::FILE* f)
{
    using T = std::remove_pointer_t<decltype(rawPtr(dv))>;
    std::vector<T> h(dv.size());
    cudaMemcpy(h.data(), rawPtr(dv), h.size() * sizeof(T), cudaMemcpyDeviceToHost);
    std::vector<double> o(h.begin(), h.end());
    std::fwrite(o.data(), sizeof(double), o.size(), f);
}

template<class Th>
int run(const char* in, const char* out, bool ve, double lim[6], int bc[3])
{
    std::FILE* f = std::fopen(in, "rb");
    if (!f) return 2;
    long long n = 0;
    if (std::fread(&n, sizeof(n), 1, f) != 1) return 2;
    std::vector<double> a(10 * n);
    if (std::fread(a.data(), sizeof(double), a.size(), f) != a.size()) return 2;
    std::fclose(f);
    auto col = [&](int k) { return std::vector<double>(a.begin() + k * n, a.begin() + (k + 1) * n); };
    auto colT = [&](int k) { auto c = col(k); return std::vector<Th>(c.begin(), c.end()); };

    ParticlesData<Th, Th> d;
    auto& dv = d.devData;
    upload(dv.x, col(0));
    upload(dv.y, col(1));
    upload(dv.z, col(2));
    upload(dv.h, colT(3));
    upload(dv.m, colT(4));
    upload(dv.u, col(5));
    upload(dv.vx, colT(6));
    upload(dv.vy, colT(7));
    upload(dv.vz, colT(8));
    upload(dv.alpha, colT(9));
    for (auto* v : {&dv.rho, &dv.p, &dv.c, &dv.xm, &dv.kx, &dv.gradh, &dv.prho, &dv.divv, &dv.curlv, &dv.c11, &dv.c12,
                    &dv.c13, &dv.c22, &dv.c23, &dv.c33, &dv.ax, &dv.ay, &dv.az})
        v->resize(n);
    dv.du.resize(n);
    dv.keys.resize(n);
    dv.nc.resize(n);

    auto bt = [](int b) { return b == 1 ? BoundaryType::periodic : BoundaryType::open; };
    Box<double> box(lim[0], lim[1], lim[2], lim[3], lim[4], lim[5], bt(bc[0]), bt(bc[1]), bt(bc[2]));
    dr::SingleRankDomain<uint64_t, double, Box<double>> domain(0, 1, 64, 64, 0.5f, box);
    domain.syncDataset(d);
    GroupView grp{0, uint32_t(n), 1, nullptr, nullptr};
    dr::findNeighborsSfc(0, n, d, domain.box());
    if (ve) {
        dr::computeXMass(grp, d, domain.box());
        dr::computeVeDefGradh(grp, d, domain.box());
        dr::computeEOS(0, n, d);
        dr::computeIadDivvCurlv(grp, d, domain.box());
        dr::computeAVswitches(grp, d, domain.box());
        dr::computeMomentumEnergy<false>(grp, nullptr, d, domain.box());
    } else {
        dr::computeDensity(grp, d, domain.box());
        dr::computeEOS_HydroStd(0, n, d);
        dr::computeIAD(grp, d, domain.box());
        dr::computeMomentumEnergySTD(grp, d, domain.box());
    }
    std::FILE* o = std::fopen(out, "wb");
    for (auto* v : {&dv.rho, &dv.c11, &dv.c12, &dv.ax, &dv.ay, &dv.az, &dv.xm, &dv.kx, &dv.divv, &dv.alpha})
        download(*v, o);
    download(dv.du, o);
    std::fwrite(&d.minDtCourant, sizeof(double), 1, o);

    // the rest of the propagator's step (ve_hydro.hpp:190-204): time step, positions, h, observables
    for (auto* v : {&dv.x_m1, &dv.y_m1, &dv.z_m1, &dv.du_m1}) v->resize(n);
    dr::computeTimestep(0, n, d);
    dr::computePositions(grp, d, domain.box());
    dr::updateSmoothingLength(grp, d);
    auto [eKin, eInt, linmom, angmom] = dr::localConservedQuantities(0, n, d);
    download(dv.x, o);
    download(dv.vx, o);
    download(dv.u, o);
    download(dv.h, o);
    const double tail[10] = {d.minDt, d.ttot, eKin, eInt, linmom[0], linmom[1], linmom[2],
                             angmom[0], angmom[1], angmom[2]};
    std::fwrite(tail, sizeof(double), 10, o);
    std::fclose(o);
    return 0;
}

// The VE adjoint through the adapter: L = sum |a|^2 after the VE passes; writes the derivative of L
// along a fixed +-1 direction in u from adjointVe and from a central difference of the passes on
// the frozen lists (u moves no pair distance).
int runAdjoint(const char* in, const char* out, double lim[6], int bc[3])
{
    using Th = double;
    std::FILE* f = std::fopen(in, "rb");
    if (!f) return 2;
    long long n = 0;
    if (std::fread(&n, sizeof(n), 1, f) != 1) return 2;
    std::vector<double> a(10 * n);
    if (std::fread(a.data(), sizeof(double), a.size(), f) != a.size()) return 2;
    std::fclose(f);
    auto col = [&](int k) { return std::vector<double>(a.begin() + k * n, a.begin() + (k + 1) * n); };
    ParticlesData<Th, Th> d;
    auto& dv = d.devData;
    DeviceVector<double>* inputs[] = {&dv.x, &dv.y, &dv.z, &dv.h, &dv.m, &dv.u, &dv.vx, &dv.vy, &dv.vz, &dv.alpha};
    for (int k = 0; k < 10; ++k) upload(*inputs[k], col(k));
    for (auto* v : {&dv.rho, &dv.p, &dv.c, &dv.xm, &dv.kx, &dv.gradh, &dv.prho, &dv.divv, &dv.curlv, &dv.c11, &dv.c12,
                    &dv.c13, &dv.c22, &dv.c23, &dv.c33, &dv.ax, &dv.ay, &dv.az, &dv.du})
        v->resize(n);
    dv.keys.resize(n);
    dv.nc.resize(n);
    auto bt = [](int b) { return b == 1 ? BoundaryType::periodic : BoundaryType::open; };
    Box<double> box(lim[0], lim[1], lim[2], lim[3], lim[4], lim[5], bt(bc[0]), bt(bc[1]), bt(bc[2]));
    dr::SingleRankDomain<uint64_t, double, Box<double>> domain(0, 1, 64, 64, 0.5f, box);
    domain.syncDataset(d);
    GroupView grp{0, uint32_t(n), 1, nullptr, nullptr};
    dr::findNeighborsSfc(0, n, d, domain.box());
    DeviceVector<double> alphaPrev(n);
    cudaMemcpy(rawPtr(alphaPrev), rawPtr(dv.alpha), n * sizeof(double), cudaMemcpyDeviceToDevice);
    auto host = [&](DeviceVector<double>& v) {
        std::vector<double> h(n);
        cudaMemcpy(h.data(), rawPtr(v), n * sizeof(double), cudaMemcpyDeviceToHost);
        return h;
    };
    auto forward = [&]() {  // the VE passes on the frozen lists, from the same alpha; returns L
        cudaMemcpy(rawPtr(dv.alpha), rawPtr(alphaPrev), n * sizeof(double), cudaMemcpyDeviceToDevice);
        dr::computeXMass(grp, d, domain.box());
        dr::computeVeDefGradh(grp, d, domain.box());
        dr::computeEOS(0, n, d);
        dr::computeIadDivvCurlv(grp, d, domain.box());
        dr::computeAVswitches(grp, d, domain.box());
        dr::computeMomentumEnergy<false>(grp, nullptr, d, domain.box());
        auto ax = host(dv.ax), ay = host(dv.ay), az = host(dv.az);
        double L = 0;
        for (long long i = 0; i < n; ++i) L += ax[i] * ax[i] + ay[i] * ay[i] + az[i] * az[i];
        return L;
    };
    forward();
    std::vector<double> s[3] = {host(dv.ax), host(dv.ay), host(dv.az)};
    DeviceVector<double> seed[3], grad[8];
    for (int k = 0; k < 3; ++k) {
        for (auto& v : s[k]) v *= 2.0;
        upload(seed[k], s[k]);
    }
    for (auto& g : grad) g.resize(n);
    dr::Seeds sd;
    sd.ax = rawPtr(seed[0]);
    sd.ay = rawPtr(seed[1]);
    sd.az = rawPtr(seed[2]);
    dr::Grads gr{rawPtr(grad[0]), rawPtr(grad[1]), rawPtr(grad[2]), rawPtr(grad[3]),
                 rawPtr(grad[4]), rawPtr(grad[5]), rawPtr(grad[6]), rawPtr(grad[7])};
    dr::adjointVe<false>(d, rawPtr(alphaPrev), sd, gr);
    auto gu = host(grad[7]);
    auto u0 = host(dv.u);
    std::vector<double> dir(n), up(n);
    unsigned long long st = 12345;
    double ad = 0;
    for (long long i = 0; i < n; ++i) {
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        dir[i] = (st >> 63) ? 1.0 : -1.0;
        ad += gu[i] * dir[i];
    }
    const double eps = 1e-6;
    for (long long i = 0; i < n; ++i) up[i] = u0[i] + eps * dir[i];
    upload(dv.u, up);
    const double lp = forward();
    for (long long i = 0; i < n; ++i) up[i] = u0[i] - eps * dir[i];
    upload(dv.u, up);
    const double lm = forward();
    const double res[2] = {ad, (lp - lm) / (2 * eps)};
    std::FILE* o = std::fopen(out, "wb");
    std::fwrite(res, sizeof(double), 2, o);
    std::fclose(o);
    return 0;
}

// One step of HydroVeProp as the reference propagator writes it (main/src/propagator/ve_hydro.hpp:
// 100-217): Domain::sync of keys x y z h with the conserved fields as properties and the dependent
// ones as scratch, d.treeView = domain.octreeProperties(), findNeighborsSfc, computeGroups into a
// GroupData, the VE passes on groups_.view() with the (no-op) halo exchanges between them,
// rhoTimestep, then computeTimestep, computePositions with the reference's argument list and
// updateSmoothingLength.  Writes the forces, the groups, the tree view (leaf count, depth, node
// centers and sizes) and the integrated fields.
int runPropagator(const char* in, const char* out, double lim[6], int bc[3])
{
    using Th = double;
    std::FILE* f = std::fopen(in, "rb");
    if (!f) return 2;
    long long n = 0;
    if (std::fread(&n, sizeof(n), 1, f) != 1) return 2;
    std::vector<double> a(10 * n);
    if (std::fread(a.data(), sizeof(double), a.size(), f) != a.size()) return 2;
    std::fclose(f);
    auto col = [&](int k) { return std::vector<double>(a.begin() + k * n, a.begin() + (k + 1) * n); };
    ParticlesData<Th, Th> d;
    auto& dv = d.devData;
    DeviceVector<double>* inputs[] = {&dv.x, &dv.y, &dv.z, &dv.h, &dv.m, &dv.u, &dv.vx, &dv.vy, &dv.vz, &dv.alpha};
    for (int k = 0; k < 10; ++k) upload(*inputs[k], col(k));
    for (auto* v : {&dv.rho, &dv.p, &dv.c, &dv.xm, &dv.kx, &dv.gradh, &dv.prho, &dv.divv, &dv.curlv, &dv.c11, &dv.c12,
                    &dv.c13, &dv.c22, &dv.c23, &dv.c33, &dv.ax, &dv.ay, &dv.az, &dv.du, &dv.x_m1, &dv.y_m1,
                    &dv.z_m1, &dv.du_m1})
        v->resize(n);
    dv.nc.resize(n);  // keys are sized by the sync
    auto bt = [](int b) { return b == 1 ? BoundaryType::periodic : BoundaryType::open; };
    Box<double> box(lim[0], lim[1], lim[2], lim[3], lim[4], lim[5], bt(bc[0]), bt(bc[1]), bt(bc[2]));
    dr::SingleRankDomain<uint64_t, double, Box<double>> domain(0, 1, 64, 64, 0.5f, box);
    GroupData groups_;

    // sync(domain, simData) (ve_hydro.hpp:100-117)
    domain.sync(dv.keys, dv.x, dv.y, dv.z, dv.h,
                std::tie(dv.m, dv.u, dv.vx, dv.vy, dv.vz, dv.x_m1, dv.y_m1, dv.z_m1, dv.du_m1, dv.alpha),
                std::tie(dv.rho, dv.p, dv.c, dv.kx));
    d.treeView = domain.octreeProperties();
    // computeForces (ve_hydro.hpp:119-190)
    if (domain.nParticlesWithHalos() != uint32_t(n) || domain.nParticles() != uint32_t(n)) return 4;
    std::size_t first = domain.startIndex();
    std::size_t last = domain.endIndex();
    dr::findNeighborsSfc(first, last, d, domain.box());
    dr::computeGroups(first, last, d, domain.box(), groups_);
    dr::computeXMass(groups_.view(), d, domain.box());
    domain.exchangeHalos(std::tie(dv.xm), dv.ax, dv.keys);
    dr::computeVeDefGradh(groups_.view(), d, domain.box());
    dr::computeEOS(first, last, d);
    domain.exchangeHalos(std::tie(dv.vx, dv.vy, dv.vz, dv.prho, dv.c, dv.kx), dv.ax, dv.keys);
    dr::computeIadDivvCurlv(groups_.view(), d, domain.box());
    d.minDtRho = dr::rhoTimestep(first, last, d);
    domain.exchangeHalos(std::tie(dv.c11, dv.c12, dv.c13, dv.c22, dv.c23, dv.c33, dv.divv), dv.ax, dv.keys);
    dr::computeAVswitches(groups_.view(), d, domain.box());
    domain.exchangeHalos(std::tie(dv.alpha), dv.ax, dv.keys);
    std::vector<float> groupDt(groups_.numGroups);
    DeviceVector<float> groupDtDev(groups_.numGroups);
    dr::computeMomentumEnergy<false>(groups_.view(), rawPtr(groupDtDev), d, domain.box());

    std::FILE* o = std::fopen(out, "wb");
    for (auto* v : {&dv.xm, &dv.kx, &dv.c11, &dv.divv, &dv.alpha, &dv.ax, &dv.ay, &dv.az, &dv.du}) download(*v, o);
    std::vector<uint32_t> gs(groups_.numGroups + 1);
    cudaMemcpy(gs.data(), groups_.groupStart, gs.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaMemcpy(groupDt.data(), rawPtr(groupDtDev), groupDt.size() * sizeof(float), cudaMemcpyDeviceToHost);
    const auto& tv = d.treeView;
    const long long nn = (long long)(domain.focusTree().octreeViewAcc().numLeafNodes);
    if (domain.globalTree().numLeafNodes() != nn) return 5;
    int lr[23];
    cudaMemcpy(lr, tv.levelRange, sizeof(lr), cudaMemcpyDeviceToHost);
    const long long numNodes = lr[22] > 0 ? lr[22] : 0;  // levelRange[maxTreeLevel + 1] = node count
    std::vector<double> cen(3 * numNodes), siz(3 * numNodes);
    cudaMemcpy(cen.data(), tv.centers, cen.size() * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(siz.data(), tv.sizes, siz.size() * sizeof(double), cudaMemcpyDeviceToHost);
    const double head[6] = {double(groups_.numGroups), double(groups_.firstBody), double(groups_.lastBody),
                            double(tv.numLeafNodes), double(nn), double(domain.focusTree().depth())};
    std::fwrite(head, sizeof(double), 6, o);
    std::vector<double> gsd(gs.begin(), gs.end()), gdt(groupDt.begin(), groupDt.end());
    std::fwrite(gsd.data(), sizeof(double), gsd.size(), o);
    std::fwrite(gdt.data(), sizeof(double), gdt.size(), o);
    const double nnd = double(numNodes);
    std::fwrite(&nnd, sizeof(double), 1, o);
    std::fwrite(cen.data(), sizeof(double), cen.size(), o);
    std::fwrite(siz.data(), sizeof(double), siz.size(), o);

    // integrate (ve_hydro.hpp:192-204)
    dr::computeTimestep(first, last, d);
    dr::computePositions(groups_.view(), d, domain.box(), d.minDt, {float(d.minDt_m1)});
    dr::updateSmoothingLength(groups_.view(), d);
    download(dv.x, o);
    download(dv.u, o);
    download(dv.h, o);
    const double tail[2] = {d.minDt, d.minDtRho};
    std::fwrite(tail, sizeof(double), 2, o);
    std::fclose(o);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc < 5) return 1;
    double lim[6];
    int bc[3];
    for (int k = 0; k < 6; ++k) lim[k] = std::atof(argv[5 + k]);
    for (int k = 0; k < 3; ++k) bc[k] = std::atoi(argv[11 + k]);
    bool ve = std::string(argv[4]) == "ve";
    try {
        if (std::string(argv[3]) == "adjoint") return runAdjoint(argv[1], argv[2], lim, bc);
        if (std::string(argv[3]) == "propagator") return runPropagator(argv[1], argv[2], lim, bc);
        if (std::string(argv[3]) == "mixed") return run<float>(argv[1], argv[2], ve, lim, bc);
        return run<double>(argv[1], argv[2], ve, lim, bc);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 3;
    }
}
