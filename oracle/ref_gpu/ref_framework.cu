// The reference framework's GPU kernels, compiled unchanged from the
// reference sources (CUDA/framework/kernel.h and the tile bodies it includes:
// kernel_128_new.h, kernel_256_new.h) into a cubin for sm_103a.
//
// TEST INFRASTRUCTURE ONLY: tests/test_ref_gpu.py loads the cubin with the
// driver API and runs the reference's own `gemm` kernel
// (CUDA/framework/kernel.h:11) beside the library's drop-in, as a GPU parity
// pin and a timing comparison.  The library never loads it.  Built by
// oracle/ref_gpu/Makefile where the reference checkout exists.
#include "kernel.h"
