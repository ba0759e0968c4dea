// CPU launch shim: see shim_algorithms.h.
#pragma once
#include "shim_algorithms.h"
