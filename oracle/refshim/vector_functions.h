// Host-only constructors for the shim's vector types.  Test infrastructure.
#pragma once
#include "vector_types.h"

inline double3 make_double3(double x, double y, double z) { double3 r; r.x = x; r.y = y; r.z = z; return r; }
inline int3 make_int3(int x, int y, int z) { int3 r; r.x = x; r.y = y; r.z = z; return r; }
