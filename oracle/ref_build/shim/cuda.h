#pragma once
/* Host-build stand-in for <cuda.h>: the reference's kernels need no driver API. */
#include "cuda_shim.h"
