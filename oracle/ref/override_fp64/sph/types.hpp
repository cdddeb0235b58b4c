/* Include-path override used only when compiling the reference headers into the FP64
 * oracle (oracle/_ref/libref_fp64.so).  It shadows the reference's sph/types.hpp
 * (sph/include/sph/types.hpp:39-46), which fixes HydroType = XM1Type = Tmass = float, so that
 * every hydro field of sphexa::ParticlesData becomes double.  The struct and member names
 * must match the reference's for its headers to compile against it. */
#pragma once

#include <cstdint>

namespace sph
{
struct SphTypes
{
    using KeyType        = uint64_t;
    using CoordinateType = double;
    using HydroType      = double;
    using XM1Type        = double;
    using Tmass          = double;
};
} // namespace sph
