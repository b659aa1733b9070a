// Which component of randVec3d's result each of its three draws lands in,
// as nvcc compiles the reference's form of it for the GPU and as the host
// compiler compiles it for the CPU.  The reference writes
//   Vec3d randVec3d(uint32_t* seeds) {
//     return Vec3d(randDouble(seeds), randDouble(seeds), randDouble(seeds)); }
// (kernels/mrand.cu:33-35): the three arguments of a constructor call are
// unsequenced in C++, so the compiler picks the order.  This probe has the
// same shape (a class with a three-double constructor, a draw that updates
// the stream through memory, not inlined) and prints, for the device and the
// host, the component that the first, second and third draw went to, e.g.
// "device order: 0 1 2" for left to right.  Compiled with the library's flags
// by tests/test_gpu_draw_order.py.
#include <cstdint>
#include <cstdio>

struct V3 {
  double x, y, z;
  __host__ __device__ V3(double a, double b, double c) : x(a), y(b), z(c) {}
};

__host__ __device__ __noinline__ double draw(uint32_t* state) {
  uint32_t s = *state;
  s ^= s << 13;
  s ^= s >> 17;
  s ^= s << 5;
  *state = s;
  return double(float(s) * 1.0 / 4294967296.0);
}

__host__ __device__ __noinline__ V3 draw3(uint32_t* state) { return V3(draw(state), draw(state), draw(state)); }

__global__ void k(uint32_t* state, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const V3 v = draw3(state);
    out[0] = v.x, out[1] = v.y, out[2] = v.z;
  }
}

// order[i] = the component equal to the i-th sequential draw, or -1.
static bool order_of(const double* got, uint32_t seed, int order[3]) {
  double seq[3];
  for (int i = 0; i < 3; i++) seq[i] = draw(&seed);
  int seen = 0;
  for (int i = 0; i < 3; i++) {
    order[i] = -1;
    for (int c = 0; c < 3; c++)
      if (got[c] == seq[i] && !(seen & (1 << c))) {
        order[i] = c;
        seen |= 1 << c;
        break;
      }
    if (order[i] < 0) return false;
  }
  return true;
}

int main() {
  const uint32_t seed = 0x2545F491u;  // any non-zero state; the three draws differ
  uint32_t* d_state = nullptr;
  double* d_out = nullptr;
  if (cudaMalloc(&d_state, sizeof(uint32_t)) != cudaSuccess || cudaMalloc(&d_out, 3 * sizeof(double)) != cudaSuccess)
    return 2;
  cudaMemcpy(d_state, &seed, sizeof(seed), cudaMemcpyHostToDevice);
  k<<<1, 32>>>(d_state, d_out);
  double dev[3];
  if (cudaMemcpy(dev, d_out, sizeof(dev), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
  uint32_t hs = seed;
  const V3 hv = draw3(&hs);
  const double host[3] = {hv.x, hv.y, hv.z};
  int od[3], oh[3];
  if (!order_of(dev, seed, od) || !order_of(host, seed, oh)) {
    printf("draws not found\n");
    return 4;
  }
  printf("device order: %d %d %d\n", od[0], od[1], od[2]);
  printf("host order: %d %d %d\n", oh[0], oh[1], oh[2]);
  cudaFree(d_state);
  cudaFree(d_out);
  return 0;
}
