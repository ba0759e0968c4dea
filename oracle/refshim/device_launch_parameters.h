// CPU launch shim: the built-in index variables live in cuda_runtime.h.
#pragma once
#include "cuda_runtime.h"
