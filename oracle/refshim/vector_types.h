// Host-only stand-ins for the CUDA vector types the reference's code names.
// Part of the CPU launch shim that compiles the reference's own kernels as
// host code (see oracle/build_ref.sh).  Test infrastructure only.
#pragma once

struct double3 { double x, y, z; };
struct int3 { int x, y, z; };
struct uint3 { unsigned x, y, z; };
struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
