/* CPU emulation of CUDA for the reference build (TEST INFRASTRUCTURE ONLY):
   __syncthreads and the intrinsics live in cuda_runtime.h. */
#include "cuda_runtime.h"
