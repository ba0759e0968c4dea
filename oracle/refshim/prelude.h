// Force-included first when oracle/build_ref.sh compiles the reference's
// sources for the CPU.  Pulls in every standard header the reference uses (so
// that the access-specifier macros below never reach a standard header), then
// opens the reference's private/protected members to the dump harness in
// oracle/ref_harness.cpp, which copies device-side arrays out for comparison.
// Test infrastructure only.
#pragma once
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <map>
#include <numeric>
#include <sstream>
#include <string>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>
#include <dirent.h>
#include <sys/stat.h>
#include "cuda_runtime.h"

// The reference calls abs() on doubles in device code, where CUDA provides the
// double overload; make the same overload visible to the host compiler.
using std::abs;

#define private public
#define protected public
