// lens.cu -- thin-lens sample tables.
//
// Every thin-lens sample of the pixel kernel computes cos and sin of
// 2*pi*u1 and sqrt(u2) in double for two mrand draws (raytracer.cu:141-142).
// GB300's double pipe is narrow, and these two functions are most of the
// double work of ray generation.  A draw takes only kLensValues distinct
// values (crt_device.cuh), so this file tabulates both functions at every
// value once per device, by the same expressions (lens_angle, sqrt) the
// kernels otherwise evaluate inline: 16 + 8 bytes per value, 2.0 GB in all,
// a small part of GB300's HBM.  The kernels then load the two results
// (lens_origin), and every ray is the same bit for bit with or without the
// tables.  crt_set_lens_tables(0) turns them off; they are skipped when the
// device has less than 8 GB free beyond them or the stream is being
// captured (the first build allocates and synchronises).
#include <mutex>

#include "crt.h"
#include "crt_internal.h"

namespace crt {

namespace {

__global__ void __launch_bounds__(256) k_lens_tables(double2* __restrict__ cs, double* __restrict__ sq) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < kLensValues; i += gridDim.x * blockDim.x) {
    const double u = draw_value(lens_value(i));
    double ca, sa;
    lens_angle(u, ca, sa);
    cs[i] = make_double2(ca, sa);
    sq[i] = sqrt(u);
  }
}

constexpr int kMaxDevices = 64;
constexpr size_t kLensBytes = (size_t)kLensValues * (sizeof(double2) + sizeof(double));
constexpr size_t kLensHeadroom = (size_t)8 << 30;

std::mutex g_lens_mu;
bool g_lens_enabled = true;
bool g_lens_tried[kMaxDevices] = {};
LensTables g_lens[kMaxDevices];

}  // namespace

LensTables lens_tables(cudaStream_t st) {
  std::lock_guard<std::mutex> lock(g_lens_mu);
  int dev = 0;
  if (!g_lens_enabled || cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return LensTables{};
  if (g_lens_tried[dev]) return g_lens[dev];
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) return LensTables{};
  g_lens_tried[dev] = true;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || free_b < kLensBytes + kLensHeadroom) return LensTables{};
  void* p = nullptr;
  if (cudaMalloc(&p, kLensBytes) != cudaSuccess) {
    cudaGetLastError();
    return LensTables{};
  }
  double2* cs = static_cast<double2*>(p);
  double* sq = reinterpret_cast<double*>(cs + kLensValues);
  k_lens_tables<<<num_sms() * 8, 256, 0, st>>>(cs, sq);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
    cudaFree(p);
    return LensTables{};
  }
  g_lens[dev].cs = cs;
  g_lens[dev].sq = sq;
  return g_lens[dev];
}

}  // namespace crt

extern "C" crt_status crt_set_lens_tables(int32_t enable) {
  std::lock_guard<std::mutex> lock(crt::g_lens_mu);
  crt::g_lens_enabled = enable != 0;
  return CRT_OK;
}
