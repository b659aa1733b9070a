// Checks that CUDA's sincos(a) equals (sin(a), cos(a)) bit for bit for every
// lens angle the pixel kernel can produce, a = 2*pi * (double)__uint2float_rn(u)
// * 2^-32 for a 32-bit draw u: the integers below 2^24 and every float from
// 2^24 to 2^32.  The reference's pixel kernel calls cos and sin
// (kernels/raytracer.cu:143-147); the library calls sincos.  Compiled with the
// library's flags by tests/test_gpu_sincos.py.
#include <cstdio>
#include <cstdint>
__global__ void k(unsigned long long n, unsigned long long* bad, unsigned long long* first) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    float f = i < (1ull << 24) ? (float)i : __int_as_float(0x4B800000 + (int)(i - (1ull << 24)));
    const double d = (double)f * 2.3283064365386963e-10;
    const double a = 2 * 3.14159265358979323846 * d;
    const double s1 = sin(a), c1 = cos(a);
    double s2, c2;
    sincos(a, &s2, &c2);
    if (__double_as_longlong(s1) != __double_as_longlong(s2) || __double_as_longlong(c1) != __double_as_longlong(c2)) {
      atomicAdd(bad, 1ull);
      atomicMin(first, i);
    }
  }
}
int main() {
  const unsigned long long n = (1ull << 24) + 0x4000000ull + 1;
  unsigned long long *bad, *first, h[2] = {0, ~0ull};
  cudaMalloc(&bad, 8); cudaMalloc(&first, 8);
  cudaMemcpy(bad, &h[0], 8, cudaMemcpyHostToDevice); cudaMemcpy(first, &h[1], 8, cudaMemcpyHostToDevice);
  k<<<152 * 8, 256>>>(n, bad, first);
  cudaError_t e = cudaDeviceSynchronize();
  cudaMemcpy(&h[0], bad, 8, cudaMemcpyDeviceToHost); cudaMemcpy(&h[1], first, 8, cudaMemcpyDeviceToHost);
  printf("sincos probe: %s, %llu angles, %llu mismatches, first %llu\n", cudaGetErrorString(e), n, h[0], h[1]);
  return e == cudaSuccess ? 0 : 1;
}
