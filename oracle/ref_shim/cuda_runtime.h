/* Stand-in for <cuda_runtime.h>; see cuda.h in this directory. */
#include "cuda.h"
