/* CPU emulation of CUDA for the reference build (TEST INFRASTRUCTURE ONLY):
   the thread-index variables live in cuda_runtime.h. */
#include "cuda_runtime.h"
