/* Operation counts of the reference's own j-loops, instantiated on a counting scalar.
 *
 * TEST / MEASUREMENT INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile (target `flops`) from the
 * reference headers where they lie, into oracle/_ref/libref_flops.so (git-ignored).  Every
 * scalar type of the loops (coordinates Tc, hydro fields T, masses Tm) becomes `opc::F`, a double
 * that counts each +, -, *, /, sqrt, transcendental call and comparison it takes part in, so the
 * counts are those of the loop bodies as written, per particle, with the branches the data takes:
 *   xmassJLoop            sph/include/sph/hydro_ve/xmass_kern.hpp:50-79 (also the std density)
 *   veDefGradhJLoop       sph/include/sph/hydro_ve/ve_def_gradh_kern.hpp:43-90
 *   IADJLoopSTD           sph/include/sph/hydro_std/iad_kern.hpp:12-77
 *   IADJLoop              sph/include/sph/hydro_ve/iad_kern.hpp:43-109
 *   divV_curlVJLoop       sph/include/sph/hydro_ve/divv_curlv_kern.hpp:43-123
 *   AVswitchesJLoop       sph/include/sph/hydro_ve/av_switches_kern.hpp:43-137
 *   momentumAndEnergyJLoop (std)  sph/include/sph/hydro_std/momentum_energy_kern.hpp:12-134
 *   momentumAndEnergyJLoop<avClean> (ve)  sph/include/sph/hydro_ve/momentum_energy_kern.hpp:65-222
 * Counting convention: a fused multiply-add in a compiled build is one * plus one + here (2 flops);
 * sqrt, division and each transcendental call (exp, pow, cbrt) are 1 flop each and are also
 * reported on their own; comparisons (including min/max) are counted but are not flops; negation
 * and absolute value are free operand modifiers and are not counted.  Compile-time constants
 * (constexpr evaluation, e.g. the table spacing in sph/include/sph/table_lookup.hpp) are not counted.
 */
#include "../oracle_api.h"

#include <cmath>
#include <concepts>
#include <cstring>
#include <type_traits>
#include <vector>

namespace opc
{

struct Counts
{
    uint64_t add, mul, div, sqrt, transc, cmp;
};

inline Counts g_counts{};

#define OPC_TICK(field)                                                                                                \
    do                                                                                                                 \
    {                                                                                                                  \
        if (!std::is_constant_evaluated()) ++opc::g_counts.field;                                                           \
    } while (0)

template<class A>
concept Arith = std::is_arithmetic_v<A>;

struct F
{
    double v{};
    constexpr F() = default;
    template<Arith A>
    constexpr F(A a)
        : v(double(a))
    {
    }
    // only an exact int target converts implicitly (sph/include/sph/table_lookup.hpp: `int idx = v * invDx`)
    template<class I>
        requires std::same_as<I, int>
    constexpr operator I() const
    {
        return int(v);
    }
    constexpr explicit operator double() const { return v; }
    constexpr explicit operator unsigned() const { return unsigned(v); }
    constexpr explicit operator float() const { return float(v); }

    constexpr F operator-() const { return F(-v); }
    constexpr F operator+() const { return *this; }
};

constexpr double val(F a) { return a.v; }
template<Arith A>
constexpr double val(A a)
{
    return double(a);
}

#define OPC_BINARY(op, field)                                                                                          \
    constexpr F operator op(F a, F b)                                                                                  \
    {                                                                                                                  \
        OPC_TICK(field);                                                                                               \
        return F(a.v op b.v);                                                                                          \
    }                                                                                                                  \
    template<Arith A>                                                                                                  \
    constexpr F operator op(F a, A b)                                                                                  \
    {                                                                                                                  \
        OPC_TICK(field);                                                                                               \
        return F(a.v op double(b));                                                                                    \
    }                                                                                                                  \
    template<Arith A>                                                                                                  \
    constexpr F operator op(A a, F b)                                                                                  \
    {                                                                                                                  \
        OPC_TICK(field);                                                                                               \
        return F(double(a) op b.v);                                                                                    \
    }                                                                                                                  \
    constexpr F& operator op##=(F & a, F b)                                                                            \
    {                                                                                                                  \
        a = a op b;                                                                                                    \
        return a;                                                                                                      \
    }                                                                                                                  \
    template<Arith A>                                                                                                  \
    constexpr F& operator op##=(F & a, A b)                                                                            \
    {                                                                                                                  \
        a = a op b;                                                                                                    \
        return a;                                                                                                      \
    }

OPC_BINARY(+, add)
OPC_BINARY(-, add)
OPC_BINARY(*, mul)
OPC_BINARY(/, div)

#define OPC_COMPARE(op)                                                                                                \
    constexpr bool operator op(F a, F b)                                                                               \
    {                                                                                                                  \
        OPC_TICK(cmp);                                                                                                 \
        return a.v op b.v;                                                                                             \
    }                                                                                                                  \
    template<Arith A>                                                                                                  \
    constexpr bool operator op(F a, A b)                                                                               \
    {                                                                                                                  \
        OPC_TICK(cmp);                                                                                                 \
        return a.v op double(b);                                                                                       \
    }                                                                                                                  \
    template<Arith A>                                                                                                  \
    constexpr bool operator op(A a, F b)                                                                               \
    {                                                                                                                  \
        OPC_TICK(cmp);                                                                                                 \
        return double(a) op b.v;                                                                                       \
    }

OPC_COMPARE(<)
OPC_COMPARE(>)
OPC_COMPARE(<=)
OPC_COMPARE(>=)
OPC_COMPARE(==)
OPC_COMPARE(!=)

inline F pow(F a, F b)
{
    OPC_TICK(transc);
    return F(std::pow(a.v, b.v));
}
template<Arith A>
inline F pow(F a, A b)
{
    OPC_TICK(transc);
    return F(std::pow(a.v, double(b)));
}

} // namespace opc

// The loops call std::sqrt / std::exp / std::abs ... qualified; these overloads make those calls
// resolve to the counting scalar (this file is a measurement harness, never linked into the product).
namespace std
{
inline opc::F sqrt(opc::F a)
{
    OPC_TICK(sqrt);
    return opc::F(std::sqrt(a.v));
}
inline opc::F exp(opc::F a)
{
    OPC_TICK(transc);
    return opc::F(std::exp(a.v));
}
inline opc::F cbrt(opc::F a)
{
    OPC_TICK(transc);
    return opc::F(std::cbrt(a.v));
}
inline opc::F pow(opc::F a, opc::F b) { return opc::pow(a, b); }
inline opc::F abs(opc::F a) { return opc::F(std::abs(a.v)); }
// exponent extraction is an integer operation; a power-of-two scaling counts as one multiply
inline int    ilogb(opc::F a) { return std::ilogb(a.v); }
inline opc::F ldexp(opc::F a, int e)
{
    OPC_TICK(mul);
    return opc::F(std::ldexp(a.v, e));
}
inline opc::F rint(opc::F a)
{
    OPC_TICK(add);
    return opc::F(std::rint(a.v));
}
template<>
struct common_type<opc::F, opc::F>
{
    using type = opc::F;
};
} // namespace std

#include "cstone/sfc/box.hpp"
#include "sph/kernels.hpp"
#include "sph/sph_kernel_tables.hpp"
#include "sph/hydro_ve/xmass_kern.hpp"
#include "sph/hydro_ve/ve_def_gradh_kern.hpp"
#include "sph/hydro_std/iad_kern.hpp"
#include "sph/hydro_std/momentum_energy_kern.hpp"
#include "sph/hydro_ve/iad_kern.hpp"
#include "sph/hydro_ve/divv_curlv_kern.hpp"
#include "sph/hydro_ve/av_switches_kern.hpp"
#include "sph/hydro_ve/momentum_energy_kern.hpp"

extern "C" int oracle_count_jloop(const oracle_jloop_in* in, const uint32_t* nbr, const uint32_t* nc, uint32_t ngmax,
                                  uint64_t* flops, uint64_t* totals)
{
    using opc::F;
    const size_t n = size_t(in->n);
    std::vector<std::vector<F>> f(OF_NFIELDS, std::vector<F>(n, F(0)));
    for (int k = 0; k < OF_NFIELDS; ++k)
        if (in->f[k])
            for (size_t i = 0; i < n; ++i)
                f[k][i] = F(in->f[k][i]);
    auto bt = [](uint8_t b) { return b == 1 ? cstone::BoundaryType::periodic : cstone::BoundaryType::open; };
    cstone::Box<F> box(F(in->box[0]), F(in->box[1]), F(in->box[2]), F(in->box[3]), F(in->box[4]), F(in->box[5]),
                       bt(in->bc[0]), bt(in->bc[1]), bt(in->bc[2]));
    auto whD  = sph::tabulateFunction<double, sph::lt::kTableSize>(
        sph::getSphKernel(sph::SphKernelType::sinc_n, in->sincIndex), 0.0, 2.0);
    auto whdD = sph::tabulateFunction<double, sph::lt::kTableSize>(
        sph::getSphKernelDerivative(sph::SphKernelType::sinc_n, in->sincIndex), 0.0, 2.0);
    std::vector<F> wh(whD.begin(), whD.end()), whd(whdD.begin(), whdD.end());
    const F  K = F(in->K);
    auto     P = [&](int k) { return f[k].data(); };
    const F *x = P(OF_X), *y = P(OF_Y), *z = P(OF_Z);
    const F  Atmin = 0.1, Atmax = 0.2;
    const F  ramp  = F(1.0 / (0.2 - 0.1));

    opc::Counts sum{};
    for (size_t i = 0; i < n; ++i)
    {
        const uint32_t* nb = nbr + size_t(ngmax) * i;
        unsigned        c  = std::min(nc[i] - 1, ngmax);
        F               r[8];
        opc::g_counts = opc::Counts{};
        switch (in->loop)
        {
            case OJ_XMASS: r[0] = sph::xmassJLoop(i, K, box, nb, c, x, y, z, P(OF_H), P(OF_M), wh.data(), whd.data()); break;
            case OJ_GRADH:
            {
                auto [kx, gradh] =
                    sph::veDefGradhJLoop(i, K, box, nb, c, x, y, z, P(OF_H), P(OF_M), wh.data(), whd.data(), P(OF_XM));
                r[0] = kx;
                r[1] = gradh;
                break;
            }
            case OJ_IAD_STD:
                sph::IADJLoopSTD(i, K, box, nb, c, x, y, z, P(OF_H), P(OF_M), P(OF_RHO), wh.data(), whd.data(), &r[0],
                                 &r[1], &r[2], &r[3], &r[4], &r[5]);
                break;
            case OJ_IAD_VE:
                sph::IADJLoop(i, K, box, nb, c, x, y, z, P(OF_H), wh.data(), whd.data(), P(OF_XM), P(OF_KX), &r[0],
                              &r[1], &r[2], &r[3], &r[4], &r[5]);
                break;
            case OJ_DIVV:
                sph::divV_curlVJLoop(i, K, box, nb, c, x, y, z, P(OF_VX), P(OF_VY), P(OF_VZ), P(OF_H), P(OF_C11),
                                     P(OF_C12), P(OF_C13), P(OF_C22), P(OF_C23), P(OF_C33), wh.data(), whd.data(),
                                     P(OF_KX), P(OF_XM), &r[0], &r[1], &r[2], &r[3], &r[4], &r[5], &r[6], &r[7],
                                     bool(in->avclean));
                break;
            case OJ_AV:
                r[0] = sph::AVswitchesJLoop(i, K, box, nb, c, x, y, z, P(OF_VX), P(OF_VY), P(OF_VZ), P(OF_H), P(OF_C),
                                            P(OF_C11), P(OF_C12), P(OF_C13), P(OF_C22), P(OF_C23), P(OF_C33), wh.data(),
                                            whd.data(), P(OF_KX), P(OF_XM), P(OF_DIVV), F(in->dt), F(in->alphamin),
                                            F(in->alphamax), F(in->decay), P(OF_ALPHA)[i]);
                break;
            case OJ_ME_STD:
                sph::momentumAndEnergyJLoop(i, K, box, nb, c, x, y, z, P(OF_VX), P(OF_VY), P(OF_VZ), P(OF_H), P(OF_M),
                                            P(OF_RHO), P(OF_P), P(OF_C), P(OF_C11), P(OF_C12), P(OF_C13), P(OF_C22),
                                            P(OF_C23), P(OF_C33), wh.data(), whd.data(), &r[0], &r[1], &r[2], &r[3],
                                            &r[4]);
                break;
            case OJ_ME_VE:
            {
                auto call = [&](auto avc)
                {
                    sph::momentumAndEnergyJLoop<decltype(avc)::value>(
                        i, K, box, nb, c, x, y, z, P(OF_VX), P(OF_VY), P(OF_VZ), P(OF_H), P(OF_M), P(OF_PRHO),
                        (const F*)nullptr, P(OF_C), P(OF_C11), P(OF_C12), P(OF_C13), P(OF_C22), P(OF_C23), P(OF_C33),
                        Atmin, Atmax, ramp, wh.data(), P(OF_KX), P(OF_XM), P(OF_ALPHA), P(OF_DV11), P(OF_DV12),
                        P(OF_DV13), P(OF_DV22), P(OF_DV23), P(OF_DV33), &r[0], &r[1], &r[2], &r[3], &r[4]);
                };
                if (in->avclean) call(std::true_type{});
                else call(std::false_type{});
                break;
            }
            default: return 1;
        }
        const opc::Counts& g = opc::g_counts;
        flops[i]             = g.add + g.mul + g.div + g.sqrt + g.transc;
        sum.add += g.add;
        sum.mul += g.mul;
        sum.div += g.div;
        sum.sqrt += g.sqrt;
        sum.transc += g.transc;
        sum.cmp += g.cmp;
    }
    totals[0] = sum.add;
    totals[1] = sum.mul;
    totals[2] = sum.div;
    totals[3] = sum.sqrt;
    totals[4] = sum.transc;
    totals[5] = sum.cmp;
    return 0;
}
