// Deterministic backprojection with library-owned scratch: an entry point for
// callers that cannot allocate device memory themselves.
//
// Some hosts of this library own every byte of device memory through their
// own allocator or a fixed budget and do not let a plug-in call cudaMalloc
// (which also synchronises the device), and some FFI callers reach only this
// C ABI, with no way to allocate a device workspace to pass in.  For them,
// tg_conic_full_backprojector_deterministic_noalloc() uses a fixed scratch
// array compiled into the library instead of a caller-provided workspace.
//
// The scratch is a file-scope __device__ array of kNoAllocScratchBytes
// (32 MiB): every GPU that loads the library holds it until the process
// exits.  Host code cannot use the array's name as a device address, so the
// first call on each device looks the address up with cudaGetSymbolAddress
// (with that device current) and caches it for the life of the process; that
// first call should therefore come before any stream capture, and no call may
// follow a cudaDeviceReset() of a device the entry point has already been used
// on (the reset unloads the library's device code, so the cached address would
// name freed memory).  All calls share the one array: the scratch
// is cleared at the start of every call (it keeps the previous call's
// contents until then), and calls that overlap on the GPU -- on different
// streams, or from different host threads -- race on it.
#include <mutex>

#include "tg_internal.cuh"

namespace tg {

constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;
// The workspace of a deterministic backprojection is 256 header bytes plus 8
// bytes per voxel, rounded up to 256 bytes; with a scratch size that is a
// multiple of 256 the largest cube that fits is (scratch - 256) / 8 voxels.
static_assert(kNoAllocScratchBytes % 256 == 0, "scratch size must be a multiple of 256 bytes");
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_scratch_mu;
static void *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once).
cudaError_t noalloc_scratch(void **ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = p;
  }
  *ptr = g_scratch_ptr[dev];
  return cudaSuccess;
}

size_t noalloc_scratch_bytes() { return kNoAllocScratchBytes; }

size_t noalloc_scratch_voxels() { return (kNoAllocScratchBytes - 256) / 8; }

}  // namespace tg
