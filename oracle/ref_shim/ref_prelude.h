// Included before every reference translation unit when the reference's CUDA
// kernels are compiled for sm_103a with nvcc on Linux (TEST INFRASTRUCTURE).
// It adds declarations only; no reference source is modified.
#pragma once
#include <cuda_runtime.h>

// The reference writes one MSVC integer literal, 0x00000001Ui32
// (src/dcgrid/dcgrid_utils.cuh:86). A literal operator named Ui32 gives it its
// MSVC meaning (a 32-bit unsigned value) under nvcc.
__host__ __device__ constexpr unsigned int operator""Ui32(unsigned long long v) {
  return (unsigned int)v;
}

// size_t is unsigned long on LP64 Linux, for which CUDA declares no atomicCAS /
// atomicAdd overloads (used at src/utils/cudamath.cuh:306,316 and
// src/dcgrid/dcgrid_utils.cuh:118). These forward to the 64-bit versions.
__device__ inline unsigned long atomicCAS(unsigned long *a, unsigned long c, unsigned long v) {
  return (unsigned long)atomicCAS((unsigned long long *)a, (unsigned long long)c,
                                  (unsigned long long)v);
}
__device__ inline unsigned long atomicAdd(unsigned long *a, unsigned long v) {
  return (unsigned long)atomicAdd((unsigned long long *)a, (unsigned long long)v);
}
