// Stand-in for the CUDA samples' helper_cuda.h, which uses cudaDeviceProp fields
// that CUDA 13 removed. The reference's kernels need only these three macros.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>
#define checkCudaErrors(x) (x)
#define getLastCudaError(m) ((void)0)
#define getLastCudaErrorSync(m) ((void)0)
