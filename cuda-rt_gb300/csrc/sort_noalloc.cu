// sort_noalloc.cu -- crt_sort_pairs_noalloc: the stable radix sort of
// crt_sort_pairs with its scratch in a fixed device array instead of a
// per-call allocation.
//
// Who needs it: callers that must not allocate device memory at the point
// where they sort.  cudaMalloc synchronises the whole device, so a renderer
// or simulation loop that rebuilds a BVH every frame would stall every frame
// on it; host frameworks that hand a plugin pre-allocated buffers often forbid
// the plugin from allocating on its own; and a sort on a hot path must not be
// able to fail with out-of-memory half way through a frame.
//
// The scratch is one file-scope __device__ array of kNoAllocScratchBytes
// (about 16.8 MB), enough for CRT_SORT_NOALLOC_MAX_PAIRS pairs with 32-bit
// keys.  Every GPU on which the library is loaded holds it until the process
// exits.  All calls share it: every call clears what must start at zero
// (histograms, tile counters, look-back status, error flag), and two calls
// whose work overlaps on the GPU (different streams, no ordering between
// them) race on it.
//
// Set-up: host code cannot pass the array's name to a kernel (in host code it
// names a host-side stand-in), so the first call in each CUDA context (per
// device, and again after cudaDeviceReset gives the device a new context)
// looks up its device address with cudaGetSymbolAddress while that device is
// current.  With lazy module loading that first lookup also loads this
// library's device code onto the device, which is when the array's memory is
// taken: make the first call at initialisation (it can fail there with an
// out-of-memory error) and before any stream capture.
#include <mutex>

#include "crt.h"
#include "crt_internal.h"

namespace crt {
void set_last_error(const char* msg);
}

namespace {

constexpr size_t kMaxPairs = CRT_SORT_NOALLOC_MAX_PAIRS;
constexpr size_t kMaxPasses = 4;  // 32-bit keys, 10-bit digits
constexpr size_t kMaxTiles = (kMaxPairs + crt::kSortTile - 1) / crt::kSortTile;
// the layout of crt::sort_scratch_bytes() at the maximum size, then the error flag
constexpr size_t kSortWords = 2 * kMaxPairs + kMaxPasses * crt::kRadix + kMaxPasses * kMaxTiles * crt::kRadix + 8;
constexpr size_t kErrOffset = ((kSortWords * 4 + 255) / 256) * 256;
constexpr size_t kNoAllocScratchBytes = kErrOffset + 256;

static __device__ __align__(256) unsigned char g_sort_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct ScratchAddr {
  unsigned long long ctx_id = 0;  // the CUDA context the address belongs to
  void* addr = nullptr;
};
ScratchAddr g_scratch_addr[kMaxDevices];

// cuCtxGetCurrent and cuCtxGetId through the runtime's driver entry points
// (no link-time dependence on libcuda): a context's id is unique for the
// life of the process, so an address looked up in a context that
// cudaDeviceReset has since destroyed is never reused.
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);
void* driver_fn(const char* name) {
  void* f = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return f;
}
bool current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = reinterpret_cast<CtxGetCurrentFn>(driver_fn("cuCtxGetCurrent"));
  static CtxGetIdFn get_id = reinterpret_cast<CtxGetIdFn>(driver_fn("cuCtxGetId"));
  void* ctx = nullptr;
  return get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, id) == 0;
}

// The device address of g_sort_scratch in the current context, looked up
// once per context with its device current.
cudaError_t scratch_on_current_device(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  e = cudaSetDevice(dev);  // initialises the device's primary context and makes it current
  if (e != cudaSuccess) return e;
  unsigned long long id = 0;
  if (!current_context_id(&id)) return cudaErrorInitializationError;
  std::lock_guard<std::mutex> lk(g_mu);
  ScratchAddr& c = g_scratch_addr[dev];
  if (!c.addr || c.ctx_id != id) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess) return e;
    c.addr = p;
    c.ctx_id = id;
  }
  *out = c.addr;
  return cudaSuccess;
}

crt_status fail(crt_status s, const char* msg) {
  crt::set_last_error(msg);
  return s;
}

}  // namespace

extern "C" crt_status crt_sort_pairs_noalloc(const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                                             uint32_t* vout, int32_t n, int32_t key_bits, void* stream) {
  if (n < 0 || key_bits < 1 || key_bits > 32) return fail(CRT_INVALID_ARG, "bad sizes");
  if ((size_t)n > kMaxPairs)
    return fail(CRT_INVALID_ARG, "crt_sort_pairs_noalloc: more than CRT_SORT_NOALLOC_MAX_PAIRS pairs");
  if (n == 0) return CRT_OK;
  if (const char* why = crt::sort_args_problem(kin, vin, kout, vout, n)) return fail(CRT_INVALID_ARG, why);
  void* scratch = nullptr;
  cudaError_t e = scratch_on_current_device(&scratch);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(CRT_CUDA_ERROR, "cudaGetSymbolAddress of the sort scratch failed");
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int* err = reinterpret_cast<int*>(static_cast<unsigned char*>(scratch) + kErrOffset);
  e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e == cudaSuccess) e = crt::launch_sort_pairs(kin, vin, kout, vout, n, key_bits, scratch, err, st);
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(CRT_CUDA_ERROR, cudaGetErrorString(e));
  }
  if (herr & crt::kErrTimeout) return fail(CRT_TIMEOUT, "a radix-sort look-back wait timed out");
  return CRT_OK;
}
