// Minimal stand-ins with the member names of the reference types the drop-in adapter reads
// (cstone::DeviceVector, cstone::Box, cstone::GroupView, cstone::GroupData, cstone::OctreeNsView,
// sphexa::ParticlesData<GpuTag>), so that
// include/sphgb/dropin.hpp can be compiled and linked without the reference sources.
#pragma once

#include <cmath>

#include <cuda_runtime.h>

#include <cstdint>
#include <cstddef>

namespace mockref
{
template<class T>
class DeviceVector
{
public:
    DeviceVector() = default;
    explicit DeviceVector(std::size_t n) { resize(n); }
    ~DeviceVector()
    {
        if (p_) cudaFree(p_);
    }
    DeviceVector(const DeviceVector&) = delete;
    DeviceVector& operator=(const DeviceVector&) = delete;
    void resize(std::size_t n)
    {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        n_ = n;
        if (n) {
            cudaMalloc(&p_, n * sizeof(T));
            cudaMemset(p_, 0, n * sizeof(T));  // value-initialised, as thrust::device_vector::resize
        }
    }
    std::size_t size() const { return n_; }
    T* data() { return p_; }

private:
    T* p_ = nullptr;
    std::size_t n_ = 0;
};

template<class T>
T* rawPtr(DeviceVector<T>& v)
{
    return v.data();
}

enum class BoundaryType : char { open = 0, periodic = 1, fixed = 2 };

template<class T>
class Box
{
public:
    Box(T xmin, T xmax, T ymin, T ymax, T zmin, T zmax, BoundaryType bx = BoundaryType::open,
        BoundaryType by = BoundaryType::open, BoundaryType bz = BoundaryType::open)
        : l_{xmin, xmax, ymin, ymax, zmin, zmax}
        , b_{bx, by, bz}
    {
    }
    T xmin() const { return l_[0]; }
    T xmax() const { return l_[1]; }
    T ymin() const { return l_[2]; }
    T ymax() const { return l_[3]; }
    T zmin() const { return l_[4]; }
    T zmax() const { return l_[5]; }
    BoundaryType boundaryX() const { return b_[0]; }
    BoundaryType boundaryY() const { return b_[1]; }
    BoundaryType boundaryZ() const { return b_[2]; }

private:
    T l_[6];
    BoundaryType b_[3];
};

struct GroupView
{
    uint32_t firstBody, lastBody, numGroups;
    const uint32_t* groupStart;
    const uint32_t* groupEnd;
};

// cstone::GroupData<GpuTag> (traversal/groups.hpp:37-52): uninitialised scalars until filled
struct GroupData
{
    GroupView view() const { return {firstBody, lastBody, numGroups, groupStart, groupEnd}; }
    DeviceVector<uint32_t> data;
    uint32_t firstBody, lastBody;
    uint32_t numGroups;
    uint32_t* groupStart;
    uint32_t* groupEnd;
};

template<class T>
struct Vec3
{
    T v[3];
};

// cstone::OctreeNsView (tree/octree.hpp:279-300)
template<class T, class KeyType>
struct OctreeNsView
{
    int numLeafNodes;
    const KeyType* prefixes;
    const int* childOffsets;
    const int* internalToLeaf;
    const int* levelRange;
    const KeyType* leaves;
    const uint32_t* layout;
    const Vec3<T>* centers;
    const Vec3<T>* sizes;
    float searchExtFactor{1.0};
};

template<class Th, class Tm>
struct DeviceParticlesData
{
    DeviceVector<double> x, y, z, u, du;
    DeviceVector<Th> h, vx, vy, vz, alpha, rho, p, c, xm, kx, gradh, prho, divv, curlv, c11, c12, c13, c22, c23, c33,
        ax, ay, az, dV11, dV12, dV13, dV22, dV23, dV33;
    DeviceVector<Tm> m;
    DeviceVector<Th> x_m1, y_m1, z_m1, du_m1, tdpdTrho;
    DeviceVector<uint64_t> keys;
    DeviceVector<unsigned> nc;
};

template<class Th, class Tm>
struct ParticlesData
{
    using HydroType = Th;
    using RealType  = double;
    unsigned ng0{100}, ngmax{150};
    double gamma{5.0 / 3.0}, Kcour{0.2}, sincIndex{6.0}, minDt{1e-6}, minDtCourant{0};
    double minDt_m1{1e-6}, ttot{0}, minDtRho{INFINITY}, Krho{0.06}, g{0}, etaAcc{0.2}, eps{0.005};
    constexpr static double maxDtIncrease = 1.1;
    Th alphamin{0.05f}, alphamax{1.0f}, decay_constant{0.2f};
    DeviceParticlesData<Th, Tm> devData;
    OctreeNsView<double, uint64_t> treeView;
};
} // namespace mockref
