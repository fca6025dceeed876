// cmg/core/geometry.hpp — point and index types of the C++ surface.
//
// Replaces include/cmg/core/geometry.hpp of the reference for the voxelization path.
// The members, their order and their types are the reference's (a PLC built by a
// program written against the reference passes unchanged), so Point3 is three
// contiguous doubles.
#pragma once

#include <array>
#include <cstddef>

#include "cmg/core/real.hpp"

namespace cmg {

struct Point3 {
    Real x = 0;
    Real y = 0;
    Real z = 0;

    constexpr Real& operator[](std::size_t axis) noexcept { return axis == 0 ? x : (axis == 1 ? y : z); }
    constexpr Real operator[](std::size_t axis) const noexcept {
        return axis == 0 ? x : (axis == 1 ? y : z);
    }
    friend constexpr bool operator==(const Point3&, const Point3&) = default;
};

static_assert(sizeof(Point3) == 3 * sizeof(Real), "Point3 is three packed coordinates");

using Index = int;
using Triangle = std::array<Index, 3>;
using Tetrahedron = std::array<Index, 4>;

// Whether the indices of an input start at 0 or 1 (the voxelizer reads them as given).
enum class IndexBase { Zero, One };

}  // namespace cmg
