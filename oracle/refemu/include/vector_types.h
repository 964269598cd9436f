// Stand-in for the CUDA toolkit header of this name: CPU execution of the
// reference kernels (test infrastructure only).
#pragma once
#include "refemu.h"
