/* CPU oracle: my own C++/OpenMP restatement of the reference's single-rank SPH hydro sweep.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py; never by the product path in sphexa_gb300/.
 *
 * It restates the algorithms of the reference files cited at each function, with FP64 hydro
 * types (the reference with HydroType = XM1Type = Tmass = double).  Build with
 * -ffp-contract=off: the keys and the neighbour distance tests must round exactly like the
 * reference's parity build.  The cornerstone tree is built here by a direct rule (a node is
 * split iff it holds more than `bucket` particles) instead of the reference's iterative
 * rebalance; both give the unique converged tree, which the reference-compiled oracle checks.
 */
#include "oracle_api.h"

#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

namespace orc {

using u64 = uint64_t;
constexpr int kMaxLevel = 21;
constexpr int kTable = 20000;
constexpr u64 kKeyEnd = u64(1) << 63;

struct Box {
    double lo[3], hi[3], L[3], iL[3];
    bool pbc[3];
};

static Box makeBox(const double lim[6], const uint8_t bc[3])
{
    Box b;
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = lim[2 * d];
        b.hi[d] = lim[2 * d + 1];
        b.L[d] = b.hi[d] - b.lo[d];
        b.iL[d] = 1.0 / (b.hi[d] - b.lo[d]); /* Box ctor, domain/include/cstone/sfc/box.hpp:115-118 */
        b.pbc[d] = bc[d] == 1;
    }
    return b;
}

/* ---- Hilbert curve --------------------------------------------------------------------
 * Same curve as iHilbert (domain/include/cstone/sfc/hilbert.hpp:42-93), written as a walk
 * that carries the current sub-cube orientation (an axis permutation plus a per-axis
 * reflection) instead of rewriting the coordinates in place.                              */
static const unsigned kOctToDigit[8] = {0, 1, 3, 2, 7, 6, 4, 5};
static const unsigned kDigitToOct[8] = {0, 1, 3, 2, 6, 7, 5, 4};

struct Orient {
    unsigned perm[3];
    unsigned flip[3];
};

static inline void advance(Orient& o, unsigned bx, unsigned by, unsigned bz)
{
    /* reflections of the three view axes for the next finer level */
    o.flip[0] ^= bx & ((!by) | bz);
    o.flip[1] ^= (bx & (by | bz)) | (by & (!bz));
    o.flip[2] ^= (bx & (!by) & (!bz)) | (by & (!bz));
    if (bz) { /* view axes rotate (x,y,z) <- (y,z,x) */
        Orient t = o;
        o.perm[0] = t.perm[1]; o.perm[1] = t.perm[2]; o.perm[2] = t.perm[0];
        o.flip[0] = t.flip[1]; o.flip[1] = t.flip[2]; o.flip[2] = t.flip[0];
    } else if (!by) { /* view axes x and z exchange */
        std::swap(o.perm[0], o.perm[2]);
        std::swap(o.flip[0], o.flip[2]);
    }
}

static u64 hilbertEncode(unsigned px, unsigned py, unsigned pz)
{
    const unsigned p[3] = {px, py, pz};
    Orient o{{0, 1, 2}, {0, 0, 0}};
    u64 key = 0;
    for (int lvl = kMaxLevel - 1; lvl >= 0; --lvl) {
        unsigned b[3];
        for (int a = 0; a < 3; ++a) b[a] = ((p[o.perm[a]] >> lvl) & 1u) ^ o.flip[a];
        key = (key << 3) | kOctToDigit[(b[0] << 2) | (b[1] << 1) | b[2]];
        advance(o, b[0], b[1], b[2]);
    }
    return key;
}

static void hilbertDecode(u64 key, unsigned out[3])
{
    out[0] = out[1] = out[2] = 0;
    Orient o{{0, 1, 2}, {0, 0, 0}};
    for (int lvl = kMaxLevel - 1; lvl >= 0; --lvl) {
        unsigned oct = kDigitToOct[(key >> (3 * lvl)) & 7u];
        unsigned b[3] = {oct >> 2, (oct >> 1) & 1u, oct & 1u};
        for (int a = 0; a < 3; ++a) out[o.perm[a]] |= (b[a] ^ o.flip[a]) << lvl;
        advance(o, b[0], b[1], b[2]);
    }
}

/* sfc3D (domain/include/cstone/sfc/sfc.hpp:141-178): floor(x*mx) - xmin*mx, truncated */
static u64 sfcKey(double x, double y, double z, const Box& b)
{
    constexpr int mcoord = (1 << kMaxLevel) - 1;
    const double cube = double(1u << kMaxLevel);
    const double c[3] = {x, y, z};
    unsigned ic[3];
    for (int d = 0; d < 3; ++d) {
        double m = cube * b.iL[d];
        int i = int(std::floor(c[d] * m) - b.lo[d] * m);
        ic[d] = unsigned(std::min(i, mcoord));
    }
    return hilbertEncode(ic[0], ic[1], ic[2]);
}

/* ---- key utilities (domain/include/cstone/sfc/common.hpp:95-228) ---------------------- */
static inline int clz64(u64 v) { return v ? __builtin_clzll(v) : 64; }
static inline int commonPrefixBits(u64 a, u64 b) { return clz64(a ^ b) - 1; }
static inline u64 nodeRange(int level) { return u64(1) << (3 * (kMaxLevel - level)); }
static inline int levelOfRange(u64 r) { return (clz64(r - 1) - 1) / 3; }
static inline u64 placeholder(u64 key, int level)
{
    return (u64(1) << (3 * level)) | (key >> (3 * (kMaxLevel - level)));
}
static inline int placeholderLevel(u64 code) { return (63 - clz64(code)) / 3; }
static inline u64 placeholderKey(u64 code)
{
    int len = 63 - clz64(code);
    return (code ^ (u64(1) << len)) << (3 * kMaxLevel - len);
}

/* ---- cornerstone leaves ----------------------------------------------------------------
 * Converged state of computeOctree (domain/include/cstone/tree/csarray.hpp:181-440): a node
 * is split iff it holds more than `bucket` particles and is above the deepest level.  Its
 * first particle s sees key[s + bucket] inside the node.  Every leaf start key is the start
 * of a child c >= 1 of some split node, or 0.                                              */
static std::vector<u64> buildLeaves(const std::vector<u64>& keys, unsigned bucket)
{
    const int64_t n = int64_t(keys.size());
    std::vector<u64> leafKeys{0};
    for (int64_t s = 0; s + int64_t(bucket) < n; ++s) {
        int deep = commonPrefixBits(keys[s], keys[s + bucket]) / 3;       /* levels 0..deep hold > bucket */
        int first = (s == 0) ? 0 : commonPrefixBits(keys[s - 1], keys[s]) / 3 + 1;
        deep = std::min(deep, kMaxLevel - 1);
        for (int l = first; l <= deep; ++l) {
            u64 start = keys[s] & ~(nodeRange(l) - 1);
            for (int c = 1; c < 8; ++c) leafKeys.push_back(start + u64(c) * nodeRange(l + 1));
        }
    }
    std::sort(leafKeys.begin(), leafKeys.end());
    leafKeys.push_back(kKeyEnd);
    return leafKeys;
}

/* ---- internal octree (domain/include/cstone/tree/octree.hpp:78-197 semantics) ----------
 * Level-major node order sorted by placeholder-bit prefix; childOffsets point at the first
 * of 8 contiguous children; internalToLeaf holds the leaf index for leaves and, for internal
 * nodes, the reference's unsorted-layout slot minus numInternal (always negative).                                       */
struct Octree {
    int64_t numLeaves = 0, numInternal = 0, numNodes = 0;
    std::vector<u64> prefixes;
    std::vector<int32_t> childOffsets, internalToLeaf;
    std::array<int32_t, kMaxLevel + 2> levelRange{};
    std::vector<double> center, size; /* 3 per node */
};

static void buildOctree(const std::vector<u64>& leaves, const Box& box, Octree& o)
{
    const int64_t L = int64_t(leaves.size()) - 1;
    o.numLeaves = L;
    o.numInternal = (L - 1) / 7;
    o.numNodes = L + o.numInternal;

    /* internal nodes = all proper ancestors of leaves */
    std::vector<std::pair<u64, int>> internal; /* (start key, level) */
    for (int64_t t = 0; t < L; ++t) {
        int lev = levelOfRange(leaves[t + 1] - leaves[t]);
        for (int a = 0; a < lev; ++a) {
            u64 start = leaves[t] & ~(nodeRange(a) - 1);
            if (start == leaves[t] || a == lev - 1) internal.emplace_back(start, a);
        }
    }
    std::sort(internal.begin(), internal.end());
    internal.erase(std::unique(internal.begin(), internal.end()), internal.end());

    struct Node { u64 code; int32_t tag; };
    std::vector<Node> nodes;
    nodes.reserve(size_t(o.numNodes));
    for (size_t r = 0; r < internal.size(); ++r) {
        /* label of an internal node: its slot in the reference's unsorted layout, taken at the leaf
         * that closes child 3 (binaryKeyWeight, domain/include/cstone/tree/octree.hpp:54-89) */
        u64 start = internal[r].first;
        int lev = internal[r].second;
        int64_t tid = int64_t(std::lower_bound(leaves.begin(), leaves.end(), start + 4 * nodeRange(lev + 1)) -
                              leaves.begin()) - 1;
        int64_t w = 0;
        for (int l = 1; l <= lev + 1; ++l) {
            int dig = int((leaves[tid] >> (3 * (kMaxLevel - l))) & 7u);
            w += dig >= 4 ? 7 - dig : -dig;
        }
        nodes.push_back({placeholder(start, lev), int32_t((tid + w) / 7 - o.numInternal)});
    }
    for (int64_t t = 0; t < L; ++t)
        nodes.push_back({placeholder(leaves[t], levelOfRange(leaves[t + 1] - leaves[t])), int32_t(t)});
    std::sort(nodes.begin(), nodes.end(), [](const Node& a, const Node& b) { return a.code < b.code; });

    o.prefixes.resize(nodes.size());
    o.internalToLeaf.resize(nodes.size());
    for (size_t i = 0; i < nodes.size(); ++i) {
        o.prefixes[i] = nodes[i].code;
        o.internalToLeaf[i] = nodes[i].tag;
    }
    for (int l = 0; l <= kMaxLevel; ++l)
        o.levelRange[l] = int32_t(std::lower_bound(o.prefixes.begin(), o.prefixes.end(), u64(1) << (3 * l)) -
                                  o.prefixes.begin());
    o.levelRange[kMaxLevel + 1] = int32_t(o.numNodes);

    o.childOffsets.assign(nodes.size(), 0);
    for (size_t i = 0; i < nodes.size(); ++i) {
        if (o.internalToLeaf[i] >= 0) continue;
        int lev = placeholderLevel(o.prefixes[i]);
        u64 child = o.prefixes[i] << 3;
        auto b = o.prefixes.begin() + o.levelRange[lev + 1], e = o.prefixes.begin() + o.levelRange[lev + 2];
        o.childOffsets[i] = int32_t(std::lower_bound(b, e, child) - o.prefixes.begin());
    }

    /* geometric centers and half sizes: nodeFpCenters + centerAndSize
     * (domain/include/cstone/focus/source_center.hpp:129-141, sfc/box.hpp:317-334) */
    o.center.resize(3 * nodes.size());
    o.size.resize(3 * nodes.size());
    const double uL = 1.0 / double(1 << kMaxLevel);
    for (size_t i = 0; i < nodes.size(); ++i) {
        int lev = placeholderLevel(o.prefixes[i]);
        unsigned ic[3];
        hilbertDecode(placeholderKey(o.prefixes[i]), ic);
        unsigned edge = (1u << kMaxLevel) >> lev;
        for (int d = 0; d < 3; ++d) {
            int lo = int(ic[d] & ~(edge - 1)), hi = lo + int(edge);
            double half = 0.5 * uL * box.L[d];
            o.center[3 * i + d] = box.lo[d] + (hi + lo) * half;
            o.size[3 * i + d] = (hi - lo) * half;
        }
    }
}

/* ---- neighbour search (domain/include/cstone/findneighbors.hpp:77-146,
 *      traversal/traversal.hpp:51-93, traversal/boxoverlap.hpp:184-223) ---------------- */
struct NsView {
    const Octree* o;
    const uint32_t* layout;
};

static inline double rintPbc(double d, const Box& b, int k)
{
    return d - double(b.pbc[k]) * b.L[k] * std::rint(d * b.iL[k]);
}

static unsigned neighborsOf(int64_t i, const double* x, const double* y, const double* z, const double* h,
                            const NsView& t, const Box& b, unsigned ngmax, uint32_t* out)
{
    const double xi = x[i], yi = y[i], zi = z[i], hi = h[i];
    const double r2 = 4.0 * hi * hi;
    const double p[3] = {xi, yi, zi};
    const bool anyPbc = b.pbc[0] || b.pbc[1] || b.pbc[2];
    bool inside = true;
    for (int d = 0; d < 3; ++d)
        inside = inside && (p[d] - 2.0 * hi >= b.lo[d]) && (p[d] + 2.0 * hi <= b.hi[d]);
    const bool usePbc = anyPbc && !inside;
    const Octree& o = *t.o;

    auto overlaps = [&](int32_t idx) {
        double dd[3];
        for (int d = 0; d < 3; ++d) {
            double dx = o.center[3 * idx + d] - p[d];
            if (usePbc) dx = rintPbc(dx, b, d);
            dx = std::fabs(dx) - o.size[3 * idx + d];
            dx += std::fabs(dx);
            dd[d] = dx * 0.5;
        }
        return dd[0] * dd[0] + (dd[1] * dd[1] + dd[2] * dd[2]) < r2; /* norm2 is a right fold */
    };
    unsigned cnt = 0;
    auto leafAction = [&](int32_t idx) {
        int32_t leaf = o.internalToLeaf[idx];
        for (uint32_t j = t.layout[leaf]; j < t.layout[leaf + 1]; ++j) {
            if (int64_t(j) == i) continue;
            double dx = x[j] - xi, dy = y[j] - yi, dz = z[j] - zi;
            if (usePbc) { dx = rintPbc(dx, b, 0); dy = rintPbc(dy, b, 1); dz = rintPbc(dz, b, 2); }
            if (dx * dx + dy * dy + dz * dz < r2) {
                if (cnt < ngmax) out[cnt] = j;
                ++cnt;
            }
        }
    };

    if (!overlaps(0)) return 0;
    if (o.childOffsets[0] == 0) { leafAction(0); return cnt; }
    int32_t stack[128];
    int sp = 1;
    stack[0] = 0;
    int32_t node = 0;
    do {
        for (int oct = 0; oct < 8; ++oct) {
            int32_t child = o.childOffsets[node] + oct;
            if (overlaps(child)) {
                if (o.childOffsets[child] == 0) leafAction(child);
                else stack[sp++] = child;
            }
        }
        node = stack[--sp];
    } while (node != 0);
    return cnt;
}

/* updateH (sph/include/sph/kernels.hpp:26-32) */
static inline double updateH(unsigned ng0, unsigned nc, double h)
{
    return h * 0.5 * std::pow(1.0 + 1023.0 * ng0 / double(nc), 1.0 / 10.0);
}

/* ---- kernel tables (sph/include/sph/sph_kernel_tables.hpp:30-157, kernels.hpp:35-61) --- */
static inline double sincStd(double v)
{
    if (v == 0.0) return 1.0;
    const double pv = M_PI_2 * v;
    return std::sin(pv) / pv;
}
static inline double sincStdDeriv(double v)
{
    if (v == 0.0) return 0.0;
    const double pv = M_PI_2 * v;
    const double s = std::sin(pv) / pv;
    return s * M_PI_2 * ((std::cos(pv) / std::sin(pv)) - 1.0 / pv);
}

static double kernelK(double n)
{
    auto f = [n](double x) { return 4.0 * M_PI * x * x * std::pow(sincStd(x), n); };
    const uint64_t intervals = 2000;
    const double a = 0.0, bnd = 2.0, hstep = (bnd - a) / double(intervals);
    std::vector<double> odd(intervals / 2), even(intervals / 2 - 1);
    for (uint64_t i = 0; i < odd.size(); ++i) odd[i] = f(a + double(2 * (i + 1) - 1) * hstep);
    for (uint64_t i = 0; i < even.size(); ++i) even[i] = f(a + double(2 * (i + 1)) * hstep);
    std::sort(odd.begin(), odd.end());
    std::sort(even.begin(), even.end());
    double s = hstep / 3.0 *
               (f(a) + f(bnd) + 4.0 * std::accumulate(odd.begin(), odd.end(), 0.0) +
                2.0 * std::accumulate(even.begin(), even.end(), 0.0));
    return 1.0 / s;
}

static void tables(double n, std::vector<double>& wh, std::vector<double>& whd)
{
    wh.resize(kTable);
    whd.resize(kTable);
    const double dx = (2.0 - 0.0) / (kTable - 1);
    for (int i = 0; i < kTable; ++i) {
        double v = 0.0 + i * dx;
        wh[i] = std::pow(sincStd(v), n);
        whd[i] = n * std::pow(sincStd(v), n - 1) * sincStdDeriv(v);
    }
}

/* lt::lookup (sph/include/sph/table_lookup.hpp:10-26) */
static inline double lookup(const double* tab, double v)
{
    constexpr int nInt = kTable - 1;
    constexpr double dx = 2.0 / nInt;
    constexpr double invDx = 1.0 / dx;
    int idx = int(v * invDx);
    double der = (idx >= nInt) ? 0.0 : (tab[idx + 1] - tab[idx]) * invDx;
    return (idx >= nInt) ? 0.0 : tab[idx] + der * (v - double(idx) * dx);
}

/* legacy applyPBC (domain/include/cstone/sfc/box.hpp:216-238) */
static inline void applyPBC(const Box& b, double r, double& xx, double& yy, double& zz)
{
    double* v[3] = {&xx, &yy, &zz};
    for (int d = 0; d < 3; ++d) {
        if (b.pbc[d] && *v[d] > r) *v[d] -= b.L[d];
        else if (b.pbc[d] && *v[d] < -r) *v[d] += b.L[d];
    }
}

/* ---- the sweep ------------------------------------------------------------------------ */
struct Data {
    int64_t n;
    std::vector<double> f[OF_NFIELDS];
    std::vector<uint32_t> nc, nbr;
    unsigned ngmax;
    double K;
    std::vector<double> wh, whd;
};

static inline unsigned capped(const Data& d, int64_t i) { return std::min(d.nc[i] - 1, d.ngmax); }

/* xmassJLoop (sph/include/sph/hydro_ve/xmass_kern.hpp:50-79) */
static double xmassJ(const Data& d, const Box& b, int64_t i)
{
    const double *x = d.f[OF_X].data(), *y = d.f[OF_Y].data(), *z = d.f[OF_Z].data();
    const double *h = d.f[OF_H].data(), *m = d.f[OF_M].data();
    const uint32_t* nb = d.nbr.data() + i * d.ngmax;
    double hi = h[i], mi = m[i];
    double hInv = 1.0 / hi, h3Inv = hInv * hInv * hInv;
    double rho0 = mi;
    for (unsigned k = 0, cnt = capped(d, i); k < cnt; ++k) {
        uint32_t j = nb[k];
        double xx = x[i] - x[j], yy = y[i] - y[j], zz = z[i] - z[j];
        applyPBC(b, 2.0 * hi, xx, yy, zz);
        double dist = std::sqrt(xx * xx + yy * yy + zz * zz);
        rho0 += lookup(d.wh.data(), dist * hInv) * m[j];
    }
    return mi / (rho0 * d.K * h3Inv);
}

/* IADJLoopSTD / IADJLoop (hydro_std/iad_kern.hpp:12-77, hydro_ve/iad_kern.hpp:43-109):
 * volj = m/rho (std) or xm/kx (ve) */
static void iadJ(Data& d, const Box& b, int64_t i, const double* vnum, const double* vden)
{
    const double *x = d.f[OF_X].data(), *y = d.f[OF_Y].data(), *z = d.f[OF_Z].data();
    const double* h = d.f[OF_H].data();
    const uint32_t* nb = d.nbr.data() + i * d.ngmax;
    double t11 = 0, t12 = 0, t13 = 0, t22 = 0, t23 = 0, t33 = 0;
    double hi = h[i], hiInv = 1.0 / hi;
    for (unsigned k = 0, cnt = capped(d, i); k < cnt; ++k) {
        uint32_t j = nb[k];
        double rx = x[i] - x[j], ry = y[i] - y[j], rz = z[i] - z[j];
        applyPBC(b, 2.0 * hi, rx, ry, rz);
        double dist = std::sqrt(rx * rx + ry * ry + rz * rz);
        double w = lookup(d.wh.data(), dist * hiInv);
        double vw = vnum[j] / vden[j] * w;
        t11 += rx * rx * vw; t12 += rx * ry * vw; t13 += rx * rz * vw;
        t22 += ry * ry * vw; t23 += ry * rz * vw; t33 += rz * rz * vw;
    }
    auto ex = [](double v) { return v == 0.0 ? 0 : std::ilogb(v); };
    int es = ex(t11) + ex(t12) + ex(t13) + ex(t22) + ex(t23) + ex(t33);
    double nrm = std::ldexp(1.0, -es / 6);
    t11 *= nrm; t12 *= nrm; t13 *= nrm; t22 *= nrm; t23 *= nrm; t33 *= nrm;
    double det = t11 * t22 * t33 + 2.0 * t12 * t23 * t13 - t11 * t23 * t23 - t22 * t13 * t13 - t33 * t12 * t12;
    double fac = nrm * (hi * hi * hi) / (det * d.K);
    d.f[OF_C11][i] = (t22 * t33 - t23 * t23) * fac;
    d.f[OF_C12][i] = (t13 * t23 - t33 * t12) * fac;
    d.f[OF_C13][i] = (t12 * t23 - t22 * t13) * fac;
    d.f[OF_C22][i] = (t11 * t33 - t13 * t13) * fac;
    d.f[OF_C23][i] = (t13 * t12 - t11 * t23) * fac;
    d.f[OF_C33][i] = (t11 * t22 - t12 * t12) * fac;
}

/* artificial_viscosity (sph/include/sph/kernels.hpp:70-84) */
static inline double artVisc(double ai, double aj, double ci, double cj, double w)
{
    double v = 0.0;
    if (w < 0.0) {
        double sig = (ai + aj) / 4.0 * (ci + cj) - 2.0 * w;
        v = -sig * w;
    }
    return v;
}

/* tsKCourant (kernels.hpp:10-16); Kcour travels as float in the reference signature */
static inline double courant(double vsig, double h, double c, float kc)
{
    double v = vsig > 0.0 ? vsig : c;
    return double(kc * h / v);
}

/* std momentumAndEnergyJLoop (hydro_std/momentum_energy_kern.hpp:12-134) */
static double meStdJ(Data& d, const Box& b, int64_t i, float kcour, double* maxvOut = nullptr)
{
    auto F = [&](int k) { return d.f[k].data(); };
    const double *x = F(OF_X), *y = F(OF_Y), *z = F(OF_Z), *vx = F(OF_VX), *vy = F(OF_VY), *vz = F(OF_VZ);
    const double *h = F(OF_H), *m = F(OF_M), *rho = F(OF_RHO), *p = F(OF_P), *c = F(OF_C);
    const double *c11 = F(OF_C11), *c12 = F(OF_C12), *c13 = F(OF_C13), *c22 = F(OF_C22), *c23 = F(OF_C23),
                 *c33 = F(OF_C33);
    const uint32_t* nb = d.nbr.data() + i * d.ngmax;
    double hi = h[i], roi = rho[i], pri = p[i], ci = c[i];
    double mi_roi = m[i] / rho[i];
    double hiInv = 1.0 / hi, hiInv3 = hiInv * hiInv * hiInv;
    double maxv = 0.0, mx = 0, my = 0, mz = 0, en = 0;
    for (unsigned k = 0, cnt = capped(d, i); k < cnt; ++k) {
        uint32_t j = nb[k];
        double rx = x[i] - x[j], ry = y[i] - y[j], rz = z[i] - z[j];
        applyPBC(b, 2.0 * hi, rx, ry, rz);
        double r2 = rx * rx + ry * ry + rz * rz;
        double dist = std::sqrt(r2);
        double vxij = vx[i] - vx[j], vyij = vy[i] - vy[j], vzij = vz[i] - vz[j];
        double hj = h[j], hjInv = 1.0 / hj;
        double v1 = dist * hiInv, v2 = dist * hjInv;
        double rv = rx * vxij + ry * vyij + rz * vzij;
        double hjInv3 = hjInv * hjInv * hjInv;
        double Wi = hiInv3 * lookup(d.wh.data(), v1);
        double Wj = hjInv3 * lookup(d.wh.data(), v2);
        double a1i = c11[i] * rx + c12[i] * ry + c13[i] * rz;
        double a2i = c12[i] * rx + c22[i] * ry + c23[i] * rz;
        double a3i = c13[i] * rx + c23[i] * ry + c33[i] * rz;
        double a1j = c11[j] * rx + c12[j] * ry + c13[j] * rz;
        double a2j = c12[j] * rx + c22[j] * ry + c23[j] * rz;
        double a3j = c13[j] * rx + c23[j] * ry + c33[j] * rz;
        double roj = rho[j], cj = c[j];
        double wij = rv / dist;
        double visc = 0.5 * artVisc(1.0, 1.0, ci, cj, wij);
        double vsig = ci + cj - 3.0 * wij;
        maxv = (vsig > maxv) ? vsig : maxv;
        double mj = m[j];
        double mjrojWj = mj / roj * Wj;
        double mjproi = mj * pri / (1.0 * roi * roi);
        {
            double a = Wi * (mjproi + visc * mi_roi);
            double bb = mjrojWj * (p[j] / (roj * 1.0) + visc);
            mx += a * a1i + bb * a1j;
            my += a * a2i + bb * a2j;
            mz += a * a3i + bb * a3j;
        }
        {
            double a = Wi * (2.0 * mjproi + visc * mi_roi);
            double bb = visc * mjrojWj;
            en += vxij * (a * a1i + bb * a1j) + vyij * (a * a2i + bb * a2j) + vzij * (a * a3i + bb * a3j);
        }
    }
    d.f[OF_DU][i] = -d.K * 0.5 * en;
    d.f[OF_AX][i] = d.K * mx;
    d.f[OF_AY][i] = d.K * my;
    d.f[OF_AZ][i] = d.K * mz;
    if (maxvOut) *maxvOut = maxv;
    return courant(maxv, h[i], c[i], kcour);
}

/* veDefGradhJLoop (hydro_ve/ve_def_gradh_kern.hpp:43-90) */
static void gradhJ(Data& d, const Box& b, int64_t i)
{
    auto F = [&](int k) { return d.f[k].data(); };
    const double *x = F(OF_X), *y = F(OF_Y), *z = F(OF_Z), *h = F(OF_H), *m = F(OF_M), *xm = F(OF_XM);
    const uint32_t* nb = d.nbr.data() + i * d.ngmax;
    double hi = h[i], mi = m[i], xmi = xm[i];
    double hInv = 1.0 / hi, h3Inv = hInv * hInv * hInv;
    double kxi = xmi, whomega = -3.0 * xmi, wrho0 = -3.0 * mi;
    for (unsigned k = 0, cnt = capped(d, i); k < cnt; ++k) {
        uint32_t j = nb[k];
        double xx = x[i] - x[j], yy = y[i] - y[j], zz = z[i] - z[j];
        applyPBC(b, 2.0 * hi, xx, yy, zz);
        double dist = std::sqrt(xx * xx + yy * yy + zz * zz);
        double v = dist * hInv;
        double w = lookup(d.wh.data(), v), dw = lookup(d.whd.data(), v);
        double dterh = -(3.0 * w + v * dw);
        kxi += w * xm[j];
        whomega += dterh * xm[j];
        wrho0 += dterh * m[j];
    }
    kxi *= d.K * h3Inv;
    whomega *= d.K * h3Inv * hInv;
    wrho0 *= d.K * h3Inv * hInv;
    whomega = whomega * mi / xmi + (kxi - d.K * xmi * h3Inv) * wrho0;
    double rhoi = kxi * mi / xmi;
    double dhdrho = -hi / (rhoi * 3.0);
    d.f[OF_KX][i] = kxi;
    d.f[OF_GRADH][i] = 1.0 - dhdrho * whomega;
}

/* divV_curlVJLoop (hydro_ve/divv_curlv_kern.hpp:43-123) */
static void divvJ(Data& d, const Box& b, int64_t i, bool gradV)
{
    auto F = [&](int k) { return d.f[k].data(); };
    const double *x = F(OF_X), *y = F(OF_Y), *z = F(OF_Z), *vx = F(OF_VX), *vy = F(OF_VY), *vz = F(OF_VZ);
    const double *h = F(OF_H), *kx = F(OF_KX), *xm = F(OF_XM);
    const uint32_t* nb = d.nbr.data() + i * d.ngmax;
    double hi = h[i], hiInv = 1.0 / hi, hiInv3 = hiInv * hiInv * hiInv;
    double dVx[3] = {0, 0, 0}, dVy[3] = {0, 0, 0}, dVz[3] = {0, 0, 0};
    double c11 = F(OF_C11)[i], c12 = F(OF_C12)[i], c13 = F(OF_C13)[i], c22 = F(OF_C22)[i], c23 = F(OF_C23)[i],
           c33 = F(OF_C33)[i];
    for (unsigned k = 0, cnt = capped(d, i); k < cnt; ++k) {
        uint32_t j = nb[k];
        double rx = x[i] - x[j], ry = y[i] - y[j], rz = z[i] - z[j];
        applyPBC(b, 2.0 * hi, rx, ry, rz);
        double dist = std::sqrt(rx * rx + ry * ry + rz * rz);
        double vxji = vx[j] - vx[i], vyji = vy[j] - vy[i], vzji = vz[j] - vz[i];
        double Wi = lookup(d.wh.data(), dist * hiInv);
        double tA[3] = {-(c11 * rx + c12 * ry + c13 * rz) * Wi, -(c12 * rx + c22 * ry + c23 * rz) * Wi,
                        -(c13 * rx + c23 * ry + c33 * rz) * Wi};
        double xmj = xm[j];
        double sx = vxji * xmj, sy = vyji * xmj, sz = vzji * xmj;
        for (int q = 0; q < 3; ++q) {
            dVx[q] += sx * tA[q];
            dVy[q] += sy * tA[q];
            dVz[q] += sz * tA[q];
        }
    }
    double nk = d.K * hiInv3 / kx[i];
    d.f[OF_DIVV][i] = nk * (dVx[0] + dVy[1] + dVz[2]);
    double cv[3] = {dVz[1] - dVy[2], dVx[2] - dVz[0], dVy[0] - dVx[1]};
    d.f[OF_CURLV][i] = nk * std::sqrt(cv[0] * cv[0] + (cv[1] * cv[1] + cv[2] * cv[2]));
    if (gradV) {
        d.f[OF_DV11][i] = nk * dVx[0];
        d.f[OF_DV12][i] = nk * (dVx[1] + dVy[0]);
        d.f[OF_DV13][i] = nk * (dVx[2] + dVz[0]);
        d.f[OF_DV22][i] = nk * dVy[1];
        d.f[OF_DV23][i] = nk * (dVy[2] + dVz[1]);
        d.f[OF_DV33][i] = nk * dVz[2];
    }
}

/* AVswitchesJLoop (hydro_ve/av_switches_kern.hpp:43-137) */
static double avJ(const Data& d, const Box& b, int64_t i, double dt, double amin, double amax, double decayc,
                  double alpha_i)
{
    auto F = [&](int k) { return d.f[k].data(); };
    const double *x = F(OF_X), *y = F(OF_Y), *z = F(OF_Z), *vx = F(OF_VX), *vy = F(OF_VY), *vz = F(OF_VZ);
    const double *h = F(OF_H), *c = F(OF_C), *kx = F(OF_KX), *xm = F(OF_XM), *divv = F(OF_DIVV);
    const uint32_t* nb = d.nbr.data() + i * d.ngmax;
    double hi = h[i], ci = c[i];
    double c11 = F(OF_C11)[i], c12 = F(OF_C12)[i], c13 = F(OF_C13)[i], c22 = F(OF_C22)[i], c23 = F(OF_C23)[i],
           c33 = F(OF_C33)[i];
    double vsig_i = 1.e-40 * ci;
    double hiInv = 1.0 / hi, hiInv3 = hiInv * hiInv * hiInv;
    double divvi = divv[i];
    double gx = 0, gy = 0, gz = 0;
    for (unsigned k = 0, cnt = capped(d, i); k < cnt; ++k) {
        uint32_t j = nb[k];
        double rx = x[i] - x[j], ry = y[i] - y[j], rz = z[i] - z[j];
        applyPBC(b, 2.0 * hi, rx, ry, rz);
        double dist = std::sqrt(rx * rx + ry * ry + rz * rz);
        double vxij = vx[i] - vx[j], vyij = vy[i] - vy[j], vzij = vz[i] - vz[j];
        double rv = rx * vxij + ry * vyij + rz * vzij;
        double vsig = 0.0;
        if (rv < 0.0) vsig = ci + c[j] - 3.0 * rv / dist;
        vsig_i = std::max(vsig_i, vsig);
        double Wi = d.K * hiInv3 * lookup(d.wh.data(), dist * hiInv);
        double t1 = -(c11 * rx + c12 * ry + c13 * rz) * Wi;
        double t2 = -(c12 * rx + c22 * ry + c23 * rz) * Wi;
        double t3 = -(c13 * rx + c23 * ry + c33 * rz) * Wi;
        double volj = xm[j] / kx[j];
        double fac = volj * (divvi - divv[j]);
        gx += fac * t1; gy += fac * t2; gz += fac * t3;
    }
    double gdv = std::sqrt(gx * gx + gy * gy + gz * gz);
    double aloc = 0.0;
    if (divvi < 0.0) {
        double ac = hi * hi * gdv;
        aloc = amax * ac / (ac + hi * std::fabs(divvi) + 0.05 * ci);
    }
    if (aloc >= alpha_i) alpha_i = aloc;
    else {
        double decay = hi / (decayc * vsig_i);
        double adot = (aloc >= amin) ? (aloc - alpha_i) / decay : (amin - alpha_i) / decay;
        alpha_i += adot * dt;
    }
    return alpha_i;
}

/* avRvCorrection (hydro_ve/momentum_energy_kern.hpp:43-63) */
static inline double quadForm(const double R[3], const double g[6])
{
    double s0 = g[0] * R[0] + g[1] * R[1] + g[2] * R[2];
    double s1 = g[3] * R[1] + g[4] * R[2];
    double s2 = g[5] * R[2];
    return R[0] * s0 + (R[1] * s1 + R[2] * s2); /* dot is a right fold */
}
static double avRv(const double R[3], double eta, double etaCrit, const double gi[6], const double gj[6])
{
    double d1 = quadForm(R, gi), d2 = quadForm(R, gj), d3 = 1.0;
    if (eta < etaCrit) {
        double e = 5.0 * (eta - etaCrit);
        d3 = std::exp(-e * e);
    }
    double A = (d2 != 0.0) ? d1 / d2 : 0.0;
    double Ap1 = 1.0 + A;
    double phi = 0.5 * d3 * std::max(0.0, std::min(1.0, 4.0 * A / (Ap1 * Ap1)));
    return -phi * (d1 + d2);
}

/* VE momentumAndEnergyJLoop<avClean> (hydro_ve/momentum_energy_kern.hpp:65-222) */
static double meVeJ(Data& d, const Box& b, int64_t i, bool avClean, float kcour, double* maxvOut = nullptr)
{
    auto F = [&](int k) { return d.f[k].data(); };
    const double *x = F(OF_X), *y = F(OF_Y), *z = F(OF_Z), *vx = F(OF_VX), *vy = F(OF_VY), *vz = F(OF_VZ);
    const double *h = F(OF_H), *m = F(OF_M), *prho = F(OF_PRHO), *c = F(OF_C), *kx = F(OF_KX), *xm = F(OF_XM),
                 *alpha = F(OF_ALPHA);
    const double *c11 = F(OF_C11), *c12 = F(OF_C12), *c13 = F(OF_C13), *c22 = F(OF_C22), *c23 = F(OF_C23),
                 *c33 = F(OF_C33);
    const double* dV[6] = {F(OF_DV11), F(OF_DV12), F(OF_DV13), F(OF_DV22), F(OF_DV23), F(OF_DV33)};
    const uint32_t* nb = d.nbr.data() + i * d.ngmax;
    const double Atmin = 0.1, Atmax = 0.2, ramp = 1.0 / (Atmax - Atmin);
    double hi = h[i], mi = m[i], ci = c[i], kxi = kx[i], ai = alpha[i], xmi = xm[i];
    double rhoi = kxi * mi / xmi, prhoi = prho[i];
    double hiInv = 1.0 / hi, hiInv3 = hiInv * hiInv * hiInv;
    double maxv = 0.0, mx = 0, my = 0, mz = 0, en = 0, avE = 0;
    double gi[6] = {0, 0, 0, 0, 0, 0};
    if (avClean)
        for (int q = 0; q < 6; ++q) gi[q] = dV[q][i];
    unsigned cnt = capped(d, i);
    double etaCrit = std::cbrt(32.0 * M_PI / 3.0 / double(cnt + 1));
    for (unsigned k = 0; k < cnt; ++k) {
        uint32_t j = nb[k];
        double rx = x[i] - x[j], ry = y[i] - y[j], rz = z[i] - z[j];
        applyPBC(b, 2.0 * hi, rx, ry, rz);
        double r2 = rx * rx + ry * ry + rz * rz;
        double dist = std::sqrt(r2);
        double vxij = vx[i] - vx[j], vyij = vy[i] - vy[j], vzij = vz[i] - vz[j];
        double hj = h[j], hjInv = 1.0 / hj;
        double v1 = dist * hiInv, v2 = dist * hjInv;
        double hjInv3 = hjInv * hjInv * hjInv;
        double Wi = hiInv3 * lookup(d.wh.data(), v1);
        double Wj = hjInv3 * lookup(d.wh.data(), v2);
        double a1i = -(c11[i] * rx + c12[i] * ry + c13[i] * rz) * Wi;
        double a2i = -(c12[i] * rx + c22[i] * ry + c23[i] * rz) * Wi;
        double a3i = -(c13[i] * rx + c23[i] * ry + c33[i] * rz) * Wi;
        double a1j = -(c11[j] * rx + c12[j] * ry + c13[j] * rz) * Wj;
        double a2j = -(c12[j] * rx + c22[j] * ry + c23[j] * rz) * Wj;
        double a3j = -(c13[j] * rx + c23[j] * ry + c33[j] * rz) * Wj;
        double mj = m[j], cj = c[j], xmj = xm[j];
        double rhoj = kx[j] * mj / xmj;
        double rv = rx * vxij + ry * vyij + rz * vzij;
        if (avClean) {
            double R[3] = {rx, ry, rz};
            double gj[6];
            for (int q = 0; q < 6; ++q) gj[q] = dV[q][j];
            rv += avRv(R, std::min(v1, v2), etaCrit, gi, gj);
        }
        double wij = rv / dist;
        double visc = artVisc(ai, alpha[j], ci, cj, wij);
        double vsig = 0.5 * (ci + cj) - 2.0 * wij;
        maxv = (vsig > maxv) ? vsig : maxv;
        double am, bm;
        double At = std::fabs(rhoi - rhoj) / (rhoi + rhoj);
        if (At < Atmin) { am = xmi * xmi; bm = xmj * xmj; }
        else if (At > Atmax) { am = xmi * xmj; bm = am; }
        else {
            double s = ramp * (At - Atmin);
            am = std::pow(xmi, 2.0 - s) * std::pow(xmj, s);
            bm = std::pow(xmj, 2.0 - s) * std::pow(xmi, s);
        }
        double av = mj / rhoi * visc, bv = mj / rhoj * visc;
        double avx = 0.5 * (av * a1i + bv * a1j);
        double avy = 0.5 * (av * a2i + bv * a2j);
        double avz = 0.5 * (av * a3i + bv * a3j);
        avE += avx * vxij + avy * vyij + avz * vzij;
        en += mj * am * (vxij * a1i + vyij * a2i + vzij * a3i);
        double momi = mj * prhoi * am, momj = mj * prho[j] * bm;
        mx += momi * a1i + momj * a1j + avx;
        my += momi * a2i + momj * a2j + avy;
        mz += momi * a3i + momj * a3j + avz;
    }
    avE = std::max(0.0, avE);
    d.f[OF_DU][i] = d.K * (prhoi * en + 0.5 * avE);
    d.f[OF_AX][i] = -d.K * mx;
    d.f[OF_AY][i] = -d.K * my;
    d.f[OF_AZ][i] = -d.K * mz;
    if (maxvOut) *maxvOut = maxv;
    return courant(maxv, h[i], c[i], kcour);
}

} // namespace orc

using namespace orc;

extern "C" double oracle_kernel_K(double sincIndex) { return kernelK(sincIndex); }

extern "C" void oracle_tables(double sincIndex, double* wh, double* whd)
{
    std::vector<double> a, b;
    tables(sincIndex, a, b);
    std::memcpy(wh, a.data(), sizeof(double) * kTable);
    std::memcpy(whd, b.data(), sizeof(double) * kTable);
}

extern "C" int oracle_sweep(const oracle_in* in, oracle_out* out)
{
    if (!in || !out || in->n < 0) return 1;
    if (in->nthreads > 0) omp_set_num_threads(in->nthreads);
    out->threads_used = omp_get_max_threads();
    const int64_t n = in->n;
    const unsigned ngmax = in->ngmax;

    /* ---- box (sfc/box_mpi.hpp:68-103): periodic dims keep their limits ---- */
    double lim[6];
    std::memcpy(lim, in->box, sizeof(lim));
    if (in->fit_box && n > 0) {
        const double* c[3] = {in->f[OF_X], in->f[OF_Y], in->f[OF_Z]};
        for (int d = 0; d < 3; ++d) {
            if (in->bc[d] == 1) continue;
            auto mm = std::minmax_element(c[d], c[d] + n);
            lim[2 * d] = *mm.first;
            lim[2 * d + 1] = *mm.second;
        }
    }
    std::memcpy(out->box, lim, sizeof(lim));
    Box box = makeBox(lim, in->bc);

    double t0 = omp_get_wtime();
    /* ---- keys + stable sort + gather (sfc.hpp:267-275, primitives/gather.hpp:43-74) ---- */
    std::vector<u64> keys(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) keys[i] = sfcKey(in->f[OF_X][i], in->f[OF_Y][i], in->f[OF_Z][i], box);
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
    std::vector<u64> skeys(n);
    for (int64_t i = 0; i < n; ++i) skeys[i] = keys[order[i]];

    Data d;
    d.n = n;
    d.ngmax = ngmax;
    const int inFields[] = {OF_X, OF_Y, OF_Z, OF_H, OF_M, OF_U, OF_VX, OF_VY, OF_VZ, OF_ALPHA};
    for (int k = 0; k < OF_NFIELDS; ++k) d.f[k].assign(n, 0.0);
    for (int k : inFields) {
        if (!in->f[k]) continue;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) d.f[k][i] = in->f[k][order[i]];
    }
    double t1 = omp_get_wtime();
    out->t_keys = t1 - t0;
    if (out->keys) std::memcpy(out->keys, skeys.data(), sizeof(u64) * n);
    if (out->order) std::memcpy(out->order, order.data(), sizeof(uint32_t) * n);

    /* ---- tree ---- */
    Octree oct;
    std::vector<uint32_t> layout;
    if (in->stages & (OS_TREE | OS_NBR | OS_HYDRO)) {
        std::vector<u64> leaves = buildLeaves(skeys, in->bucket);
        buildOctree(leaves, box, oct);
        int64_t L = int64_t(leaves.size()) - 1;
        layout.resize(L + 1);
#pragma omp parallel for schedule(static)
        for (int64_t t = 0; t <= L; ++t)
            layout[t] = uint32_t(std::lower_bound(skeys.begin(), skeys.end(), leaves[t]) - skeys.begin());
        out->num_leaves = L;
        out->num_nodes = oct.numNodes;
        out->num_internal = oct.numInternal;
        for (int l = 0; l < kMaxLevel + 2; ++l) out->level_range[l] = oct.levelRange[l];
        if (out->leaves && out->leaves_cap >= L + 1) std::memcpy(out->leaves, leaves.data(), sizeof(u64) * (L + 1));
        if (out->counts && out->leaves_cap >= L)
            for (int64_t t = 0; t < L; ++t) out->counts[t] = layout[t + 1] - layout[t];
        if (out->nodes_cap >= oct.numNodes) {
            if (out->prefixes) std::memcpy(out->prefixes, oct.prefixes.data(), sizeof(u64) * oct.numNodes);
            if (out->child_offsets)
                std::memcpy(out->child_offsets, oct.childOffsets.data(), sizeof(int32_t) * oct.numNodes);
            if (out->internal_to_leaf)
                std::memcpy(out->internal_to_leaf, oct.internalToLeaf.data(), sizeof(int32_t) * oct.numNodes);
            if (out->centers) std::memcpy(out->centers, oct.center.data(), sizeof(double) * 3 * oct.numNodes);
            if (out->sizes) std::memcpy(out->sizes, oct.size.data(), sizeof(double) * 3 * oct.numNodes);
        }
    }
    double t2 = omp_get_wtime();
    out->t_tree = t2 - t1;

    /* ---- neighbours with coupled h iteration (sph/include/sph/find_neighbors.hpp:10-44) ---- */
    d.nc.assign(n, 1);
    int64_t fails = 0;
    if (in->stages & (OS_NBR | OS_HYDRO)) {
        d.nbr.assign(size_t(n) * ngmax, 0);
        NsView view{&oct, layout.data()};
        const unsigned ngmin = in->ng0 / 4;
        double* h = d.f[OF_H].data();
        const double *x = d.f[OF_X].data(), *y = d.f[OF_Y].data(), *z = d.f[OF_Z].data();
#pragma omp parallel for reduction(+ : fails)
        for (int64_t i = 0; i < n; ++i) {
            uint32_t* nb = d.nbr.data() + size_t(i) * ngmax;
            unsigned nc = 1 + neighborsOf(i, x, y, z, h, view, box, ngmax, nb);
            int it = 0;
            while ((ngmin > nc || (nc - 1) > ngmax) && it++ < 10) {
                h[i] = updateH(in->ng0, nc, h[i]);
                nc = 1 + neighborsOf(i, x, y, z, h, view, box, ngmax, nb);
            }
            fails += (it >= 10);
            d.nc[i] = nc;
        }
        if (out->nc) std::memcpy(out->nc, d.nc.data(), sizeof(uint32_t) * n);
        if (out->nbr) std::memcpy(out->nbr, d.nbr.data(), sizeof(uint32_t) * size_t(n) * ngmax);
    }
    out->h_iter_fails = fails;
    double t3 = omp_get_wtime();
    out->t_nbr = t3 - t2;

    /* ---- hydro passes ---- */
    out->minDtCourant = INFINITY;
    if (in->stages & OS_HYDRO) {
        d.K = kernelK(in->sincIndex);
        tables(in->sincIndex, d.wh, d.whd);
        const float kc = float(in->Kcour);
        double minDt = INFINITY;
        if (in->variant == 0) {
            /* computeDensity (hydro_std/density.hpp:41-60): xmass loop into rho, then rho = m / rho */
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) d.f[OF_RHO][i] = xmassJ(d, box, i);
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) d.f[OF_RHO][i] = d.f[OF_M][i] / d.f[OF_RHO][i];
            /* computeEOS_HydroStd -> idealGasEOS_u (hydro_std/eos.hpp:54-80, sph/eos.hpp:34-44) */
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) {
                double tmp = d.f[OF_U][i] * (in->gamma - 1.0);
                d.f[OF_P][i] = d.f[OF_RHO][i] * tmp;
                d.f[OF_C][i] = std::sqrt(in->gamma * tmp);
            }
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) iadJ(d, box, i, d.f[OF_M].data(), d.f[OF_RHO].data());
#pragma omp parallel for schedule(static) reduction(min : minDt)
            for (int64_t i = 0; i < n; ++i) minDt = std::min(minDt, meStdJ(d, box, i, kc));
        } else {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) d.f[OF_XM][i] = xmassJ(d, box, i);
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) gradhJ(d, box, i);
            /* computeIdealGasEOS_Impl (hydro_ve/eos.hpp:52-94), rho and p stored */
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) {
                double kx = d.f[OF_KX][i], m = d.f[OF_M][i], xm = d.f[OF_XM][i];
                double rho = kx * m / xm;
                double tmp = d.f[OF_U][i] * (in->gamma - 1.0);
                double p = rho * tmp;
                d.f[OF_PRHO][i] = p / (kx * m * m * d.f[OF_GRADH][i]);
                d.f[OF_C][i] = std::sqrt(in->gamma * tmp);
                d.f[OF_RHO][i] = rho;
                d.f[OF_P][i] = p;
            }
            /* computeIadDivvCurlvImpl (hydro_ve/iad_divv_curlv.hpp:41-98) */
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) {
                iadJ(d, box, i, d.f[OF_XM].data(), d.f[OF_KX].data());
                divvJ(d, box, i, in->avclean != 0);
            }
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i)
                d.f[OF_ALPHA][i] = avJ(d, box, i, in->minDt, in->alphamin, in->alphamax, in->decay, d.f[OF_ALPHA][i]);
#pragma omp parallel for schedule(static) reduction(min : minDt)
            for (int64_t i = 0; i < n; ++i) minDt = std::min(minDt, meVeJ(d, box, i, in->avclean != 0, kc));
        }
        out->minDtCourant = minDt;
    }
    out->t_hydro = omp_get_wtime() - t3;

    for (int k = 0; k < OF_NFIELDS; ++k)
        if (out->f[k]) std::memcpy(out->f[k], d.f[k].data(), sizeof(double) * n);
    return 0;
}

/* One j-loop of particle 0 over an explicit list, for the reference's known-answer tests. */
extern "C" int oracle_jloop(const oracle_jloop_in* in, double* out)
{
    if (!in || !out || in->n <= 0 || !in->neighbors) return 1;
    const int64_t n = in->n;
    Data d;
    d.n = n;
    d.ngmax = in->count;
    for (int k = 0; k < OF_NFIELDS; ++k) {
        d.f[k].assign(n, 0.0);
        if (in->f[k]) std::memcpy(d.f[k].data(), in->f[k], sizeof(double) * n);
    }
    d.nc.assign(n, 1);
    d.nc[0] = in->count + 1;
    d.nbr.assign(size_t(n) * in->count, 0);
    std::memcpy(d.nbr.data(), in->neighbors, sizeof(uint32_t) * in->count);
    d.K = in->K;
    tables(in->sincIndex, d.wh, d.whd);
    Box box = makeBox(in->box, in->bc);
    double maxv = 0;
    switch (in->loop) {
    case OJ_XMASS: out[0] = xmassJ(d, box, 0); break;
    case OJ_GRADH:
        gradhJ(d, box, 0);
        out[0] = d.f[OF_KX][0];
        out[1] = d.f[OF_GRADH][0];
        break;
    case OJ_IAD_STD:
    case OJ_IAD_VE:
        if (in->loop == OJ_IAD_STD) iadJ(d, box, 0, d.f[OF_M].data(), d.f[OF_RHO].data());
        else iadJ(d, box, 0, d.f[OF_XM].data(), d.f[OF_KX].data());
        for (int q = 0; q < 6; ++q) out[q] = d.f[OF_C11 + q][0];
        break;
    case OJ_DIVV:
        divvJ(d, box, 0, true);
        out[0] = d.f[OF_DIVV][0];
        out[1] = d.f[OF_CURLV][0];
        for (int q = 0; q < 6; ++q) out[2 + q] = d.f[OF_DV11 + q][0];
        break;
    case OJ_AV:
        out[0] = avJ(d, box, 0, in->dt, in->alphamin, in->alphamax, in->decay, d.f[OF_ALPHA][0]);
        break;
    case OJ_ME_STD:
    case OJ_ME_VE:
        if (in->loop == OJ_ME_STD) meStdJ(d, box, 0, 0.2f, &maxv);
        else meVeJ(d, box, 0, in->avclean != 0, 0.2f, &maxv);
        out[0] = d.f[OF_AX][0];
        out[1] = d.f[OF_AY][0];
        out[2] = d.f[OF_AZ][0];
        out[3] = d.f[OF_DU][0];
        out[4] = maxv;
        break;
    default: return 2;
    }
    return 0;
}

/* ---- one integration step (port) ----
 * positionUpdate / energyUpdate / fbcCheck of sph/include/sph/positions.hpp:46-85 and putInBox of
 * domain/include/cstone/sfc/box.hpp:193-214, with the GPU kernel's handling of particles frozen next
 * to a fixed boundary (sph/include/sph/positions_gpu.cu:131-139: neither position nor energy moves). */
extern "C" int oracle_positions(int64_t n, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                                const double* ax, const double* ay, const double* az, double* xm1, double* ym1,
                                double* zm1, double* u, const double* du, double* dum1, const double* h, double dt,
                                double dt_m1, const double box[6], const uint8_t bc[3])
{
    const bool fixed[3] = {bc[0] == 2, bc[1] == 2, bc[2] == 2};
    const bool anyFixed = fixed[0] || fixed[1] || fixed[2];
    auto nearFixed = [&](double c, double hi, int k) {
        return fixed[k] && (std::abs(box[2 * k + 1] - c) < 2.0 * hi || std::abs(box[2 * k] - c) < 2.0 * hi);
    };
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        if (anyFixed && vx[i] == 0.0 && vy[i] == 0.0 && vz[i] == 0.0 &&
            (nearFixed(x[i], h[i], 0) || nearFixed(y[i], h[i], 1) || nearFixed(z[i], h[i], 2)))
            continue;
        double* X[3] = {x + i, y + i, z + i};
        double* dX[3] = {xm1 + i, ym1 + i, zm1 + i};
        double* V[3] = {vx + i, vy + i, vz + i};
        const double A[3] = {ax[i], ay[i], az[i]};
        const double idt = 1.0 / dt_m1, halfDtm1 = 0.5 * dt_m1;
        for (int k = 0; k < 3; ++k) {
            const double vn = *dX[k] * idt + halfDtm1 * A[k];
            const double vnp1 = vn + A[k] * dt;
            const double dxn = (vn + 0.5 * A[k] * std::abs(dt)) * dt;
            double xn = *X[k] + dxn;
            const double lo = box[2 * k], hi = box[2 * k + 1];
            if (bc[k] == 1) {
                if (xn > hi) xn -= hi - lo;
                else if (xn < lo) xn += hi - lo;
            }
            *X[k] = xn;
            *dX[k] = dxn;
            *V[k] = vnp1;
        }
        if (u) {
            double un = u[i] + du[i] * dt + 0.5 * (du[i] - dum1[i]) / dt_m1 * std::abs(dt) * dt;
            if (un < 0.0) un = u[i] * std::exp(un * dt / u[i]);
            u[i] = un;
            dum1[i] = du[i];
        }
    }
    return 0;
}

extern "C" int oracle_update_h(int64_t n, uint32_t ng0, const uint32_t* nc, double* h)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) h[i] = updateH(ng0, nc[i], h[i]);
    return 0;
}

extern "C" int oracle_conserved(int64_t n, const double* x, const double* y, const double* z, const double* vx,
                                const double* vy, const double* vz, const double* m, const double* u, double out[8])
{
    double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = 0; i < n; ++i) {
        const double X[3] = {x[i], y[i], z[i]}, V[3] = {vx[i], vy[i], vz[i]}, mi = m[i];
        s[0] += mi * (V[0] * V[0] + (V[1] * V[1] + V[2] * V[2]));
        s[1] += u ? u[i] * mi : 0.0;
        for (int k = 0; k < 3; ++k) s[2 + k] += mi * V[k];
        s[5] += mi * (X[1] * V[2] - X[2] * V[1]);
        s[6] += mi * (X[2] * V[0] - X[0] * V[2]);
        s[7] += mi * (X[0] * V[1] - X[1] * V[0]);
    }
    out[0] = 0.5 * s[0];
    for (int q = 1; q < 8; ++q) out[q] = s[q];
    return 0;
}
