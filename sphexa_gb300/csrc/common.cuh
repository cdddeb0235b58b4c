// Shared device/host definitions of the sphgb sweep: key utilities, the Hilbert walk, box
// helpers, the SPH kernel table lookup, and the internal context layout.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sphgb.h"

#define SPHGB_HD __host__ __device__ __forceinline__

namespace sphgb {

using u64 = unsigned long long;
constexpr int kMaxLevel = 21;
constexpr int kTableSize = 20000;
constexpr u64 kKeyEnd = u64(1) << 63;
constexpr int kWarp = 32;

// ---- SFC key utilities (domain/include/cstone/sfc/common.hpp:95-228 semantics) ----
SPHGB_HD int clz64(u64 v)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}
SPHGB_HD int commonPrefixBits(u64 a, u64 b) { return clz64(a ^ b) - 1; }
SPHGB_HD u64 nodeRange(int level) { return u64(1) << (3 * (kMaxLevel - level)); }
SPHGB_HD int levelOfRange(u64 r) { return (clz64(r - 1) - 1) / 3; }
SPHGB_HD u64 placeholder(u64 key, int level) { return (u64(1) << (3 * level)) | (key >> (3 * (kMaxLevel - level))); }
SPHGB_HD int placeholderLevel(u64 code) { return (63 - clz64(code)) / 3; }
SPHGB_HD u64 placeholderKey(u64 code)
{
    int len = 63 - clz64(code);
    return (code ^ (u64(1) << len)) << (3 * kMaxLevel - len);
}

// ---- Hilbert curve: the curve of iHilbert/decodeHilbert (domain/include/cstone/sfc/hilbert.hpp),
// evaluated as a top-down walk that carries the sub-cube orientation (axis permutation packed
// in `perm`, reflections in `flip`) instead of rewriting the coordinates. ----
struct Orient {
    unsigned perm;  // 3 x 2-bit axis index, view axis a -> bits [2a, 2a+1]
    unsigned flip;  // bit a: view axis a reflected
};

SPHGB_HD unsigned octToDigit(unsigned oct) { return (0x54672310u >> (4 * oct)) & 0xFu; }  // {0,1,3,2,7,6,4,5}
SPHGB_HD unsigned digitToOct(unsigned dig) { return (0x45762310u >> (4 * dig)) & 0xFu; }  // {0,1,3,2,6,7,5,4}

SPHGB_HD void orientAdvance(Orient& o, unsigned bx, unsigned by, unsigned bz)
{
    unsigned fx = bx & ((by ^ 1u) | bz);
    unsigned fy = (bx & (by | bz)) | (by & (bz ^ 1u));
    unsigned fz = (bx & (by ^ 1u) & (bz ^ 1u)) | (by & (bz ^ 1u));
    unsigned flip = o.flip ^ (fx | (fy << 1) | (fz << 2));
    unsigned p0 = o.perm & 3u, p1 = (o.perm >> 2) & 3u, p2 = (o.perm >> 4) & 3u;
    unsigned f0 = flip & 1u, f1 = (flip >> 1) & 1u, f2 = (flip >> 2) & 1u;
    if (bz) {  // view axes rotate (x,y,z) <- (y,z,x)
        o.perm = p1 | (p2 << 2) | (p0 << 4);
        o.flip = f1 | (f2 << 1) | (f0 << 2);
    } else if (!by) {  // view axes x and z exchange
        o.perm = p2 | (p1 << 2) | (p0 << 4);
        o.flip = f2 | (f1 << 1) | (f0 << 2);
    } else {
        o.flip = flip;
    }
}

SPHGB_HD u64 hilbertEncode(unsigned px, unsigned py, unsigned pz)
{
    const unsigned p[3] = {px, py, pz};
    Orient o{0u | (1u << 2) | (2u << 4), 0u};
    u64 key = 0;
#pragma unroll
    for (int lvl = kMaxLevel - 1; lvl >= 0; --lvl) {
        unsigned bx = ((p[o.perm & 3u] >> lvl) & 1u) ^ (o.flip & 1u);
        unsigned by = ((p[(o.perm >> 2) & 3u] >> lvl) & 1u) ^ ((o.flip >> 1) & 1u);
        unsigned bz = ((p[(o.perm >> 4) & 3u] >> lvl) & 1u) ^ ((o.flip >> 2) & 1u);
        key = (key << 3) | octToDigit((bx << 2) | (by << 1) | bz);
        orientAdvance(o, bx, by, bz);
    }
    return key;
}

SPHGB_HD void hilbertDecode(u64 key, unsigned out[3])
{
    out[0] = out[1] = out[2] = 0;
    Orient o{0u | (1u << 2) | (2u << 4), 0u};
    for (int lvl = kMaxLevel - 1; lvl >= 0; --lvl) {
        unsigned oct = digitToOct(unsigned(key >> (3 * lvl)) & 7u);
        unsigned bx = oct >> 2, by = (oct >> 1) & 1u, bz = oct & 1u;
        out[o.perm & 3u] |= (bx ^ (o.flip & 1u)) << lvl;
        out[(o.perm >> 2) & 3u] |= (by ^ ((o.flip >> 1) & 1u)) << lvl;
        out[(o.perm >> 4) & 3u] |= (bz ^ ((o.flip >> 2) & 1u)) << lvl;
        orientAdvance(o, bx, by, bz);
    }
}

// ---- box ----
struct DevBox {
    double lo[3], hi[3], L[3], iL[3];
    int pbc[3];
    float Lf[3];
};

inline DevBox makeDevBox(const sphgb_box& b)
{
    DevBox d;
    for (int k = 0; k < 3; ++k) {
        d.lo[k] = b.lim[2 * k];
        d.hi[k] = b.lim[2 * k + 1];
        d.L[k] = d.hi[k] - d.lo[k];
        d.iL[k] = 1.0 / (d.hi[k] - d.lo[k]);
        d.pbc[k] = b.bc[k] == SPHGB_BC_PERIODIC;
        d.Lf[k] = float(d.L[k]);
    }
    return d;
}

// sfc3D (domain/include/cstone/sfc/sfc.hpp:141-178) with every FP64 step rounded explicitly so
// that no multiply-add contraction changes a key.
__device__ __forceinline__ u64 sfcKey(double x, double y, double z, const DevBox& b)
{
    const double cube = double(1u << kMaxLevel);
    const double c[3] = {x, y, z};
    unsigned ic[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double m = __dmul_rn(cube, b.iL[k]);
        double v = __dsub_rn(floor(__dmul_rn(c[k], m)), __dmul_rn(b.lo[k], m));
        int i = int(v);
        ic[k] = unsigned(min(i, (1 << kMaxLevel) - 1));
    }
    return hilbertEncode(ic[0], ic[1], ic[2]);
}

// ---- status word bits set by kernels ----
enum DevFlag : int {
    kFlagStackOverflow = 1,
    kFlagListOverflow = 2,
};

}  // namespace sphgb
