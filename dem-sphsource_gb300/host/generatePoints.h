// Lattice point generators of the host API.
//
// Case drivers build their particle sets with these two functions by these
// names (core/generatePoints.h:5-73 in the reference).  The point ORDER is part
// of the contract: particle indices, cluster ids and clump pebble ranges of a
// driver follow it, so both generators emit x-major, then y, then z, exactly
// as the reference does.
#pragma once
#include <cmath>
#include <vector>
#include "myVec.h"

// Cell-centred cubic lattice filling the box [origin, origin + size): the
// number of points per axis is floor((extent + 1e-10) / spacing) and the
// lattice step is stretched so the points span the box evenly.  A box smaller
// than one spacing on any axis yields its centre alone.
inline std::vector<double3> getRegularPackedPoints(double3 origin, double3 size, double spacing)
{
    const int n[3] = {int((size.x + 1.e-10) / spacing), int((size.y + 1.e-10) / spacing),
                      int((size.z + 1.e-10) / spacing)};
    if (n[0] == 0 || n[1] == 0 || n[2] == 0) return {origin + 0.5 * size};
    const double3 step = make_double3(size.x / double(n[0]), size.y / double(n[1]), size.z / double(n[2]));
    std::vector<double3> out;
    out.reserve(size_t(n[0]) * n[1] * n[2]);
    for (int i = 0; i < n[0]; ++i)
        for (int j = 0; j < n[1]; ++j)
            for (int k = 0; k < n[2]; ++k)
                out.push_back(make_double3(origin.x + step.x * (double(i + 1) - 0.5),
                                           origin.y + step.y * (double(j + 1) - 0.5),
                                           origin.z + step.z * (double(k + 1) - 0.5)));
    return out;
}

// Hexagonal close packing of spheres of diameter `spacing` (layers ABAB...),
// centred in the box: rows are spacing apart in x, sqrt(3)/2 spacing in y and
// layers sqrt(6)/3 spacing in z; odd rows shift by half a spacing in x and
// odd layers by a third of a row in y and half a spacing in x.
inline std::vector<double3> getHexagonalClosePackedPoints(double3 origin, double3 size, double spacing)
{
    const double r3 = std::sqrt(3.0), r6 = std::sqrt(6.0);
    const int nx = int(size.x / spacing);
    const int ny = int(size.y / r3 / spacing * 2.0) - 1;
    const int nz = int(size.z / r6 / spacing * 3.0);
    const double ax = spacing, ay = spacing * r3 / 2.0, az = spacing * r6 / 3.0;
    // extent actually covered, to centre the packing in the box
    const double ex = double(2. * nx - 1 + 2) * ax / 2. + 0.5 * spacing;
    const double ey = double(2. * ny - 1 + 2. / 3.) * ay / 2. + (1. / r3 - 0.5) * ay + 0.5 * spacing;
    const double ez = 0.5 * (spacing - az) + (2. * nz - 1) * az / 2. + 0.5 * spacing;
    const double3 o = make_double3(origin.x + (size.x - ex) / 2., origin.y + (size.y - ey) / 2.,
                                   origin.z + (size.z - ez) / 2.);
    std::vector<double3> out;
    for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j)
            for (int k = 1; k <= nz; ++k)
                out.push_back(make_double3(o.x + double(2. * i - 1 + j % 2 + k % 2) * ax / 2.,
                                           o.y + double(2. * j - 1 + 2. * (k % 2) / 3.) * ay / 2. + (1. / r3 - 0.5) * ay,
                                           o.z + 0.5 * (spacing - az) + (2. * k - 1) * az / 2.));
    return out;
}
