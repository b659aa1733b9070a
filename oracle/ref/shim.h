// shim.h -- lets the reference's CUDA device code compile as host C++.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle).  build_ref.py force-includes
// this header (g++ -include) into the reference's own kernel sources, which
// are taken unmodified from the reference checkout except that the host-side
// launch wrappers (the only lines using the <<<grid, block>>> syntax) are left
// out.  Each definition below gives the host meaning of one CUDA construct
// the reference's device code uses.
#pragma once
#include <cuda_runtime.h>  // __host__/__device__ expand to nothing under g++; dim3, uint3, int2
#include <math.h>
#include <stdint.h>

// Launch coordinates: the harness runs a kernel as nested loops and sets
// these per simulated thread.  thread_local lets OpenMP threads each run
// their own simulated CUDA threads.
extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

// __clz: number of leading zero bits of a 32-bit integer (32 for zero).
static inline int __clz(int x) { return x ? __builtin_clz((unsigned)x) : 32; }

// atomicCAS on a simulated thread run to completion one at a time: compare,
// conditionally store, return the old value.
static inline int atomicCAS(int* address, int compare, int val) {
  int old = *address;
  if (old == compare) *address = val;
  return old;
}

// CUDA's device min/max overloads.  For integers they are the usual
// comparisons.  For floating point they follow fmin/fmax (a NaN operand is
// ignored), and a float operand mixed with a double is widened to double.
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }
static inline double max(double a, double b) { return fmax(a, b); }
static inline double min(double a, double b) { return fmin(a, b); }
static inline double max(double a, float b) { return fmax(a, (double)b); }
static inline double min(double a, float b) { return fmin(a, (double)b); }
