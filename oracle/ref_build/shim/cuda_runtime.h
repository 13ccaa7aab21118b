#pragma once
/* Host-build stand-in for <cuda_runtime.h>: the reference's kernels need no runtime API. */
#include "cuda_shim.h"
