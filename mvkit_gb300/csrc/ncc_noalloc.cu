// Search-pyramid level without any device allocation.
//
// Some callers cannot call cudaMalloc: code running inside a host framework
// that owns all device memory through its own pool, real-time loops where an
// allocation may block or fragment the heap for an unbounded time, or
// processes whose memory budget is fixed at start-up.  This entry point gives
// them the matcher's integer pyramid from a device image into a caller-owned
// device buffer.  The intermediate levels live in one file-scope device array
// of fixed size (kScratchFloats floats = 24 MiB), which every GPU that loads
// the library holds until the process exits.  No cudaMalloc, cudaFree or
// allocating library routine is called.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/mvkit_gb300_ncc.h"
#include "ncc_kernels.h"

namespace mvg {

void set_last_error(const char* message);

namespace {

constexpr size_t kScratchFloats = size_t(6) * 1024 * 1024;  // levels 0..L-1 of the requested level
constexpr int kMaxDevices = 64;
constexpr int kMaxRows = 65535 * 8;  // pyramid grid: 8 rows per block, 65535 blocks in y

// Shared by every call on a device; a call clears what it needs before use.
static __device__ __align__(256) float g_level_scratch[kScratchFloats];
static __device__ __align__(256) int32_t g_error_flag[64];

struct DeviceScratch {
  float* levels = nullptr;
  int32_t* flag = nullptr;
};

std::mutex g_setup_mutex;
DeviceScratch g_scratch[kMaxDevices];

// Device addresses of the scratch arrays on device `dev` (current), looked up
// once per device with that device current.  A cudaDeviceReset destroys the
// context that holds them; the process must not call this entry point on
// that device again afterwards.
int32_t scratch_of_device(int dev, DeviceScratch* out, std::string* why) {
  cudaError_t e = cudaSuccess;
  if (dev < 0 || dev >= kMaxDevices) {
    *why = "device index beyond the scratch table";
    return kUnsupported;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch[dev].levels) {
    void* levels = nullptr;
    void* flag = nullptr;
    e = cudaGetSymbolAddress(&levels, g_level_scratch);
    if (e != cudaSuccess) {
      *why = std::string("cudaGetSymbolAddress(level scratch): ") + cudaGetErrorString(e);
      return kInternal;
    }
    e = cudaGetSymbolAddress(&flag, g_error_flag);
    if (e != cudaSuccess) {
      *why = std::string("cudaGetSymbolAddress(error flag): ") + cudaGetErrorString(e);
      return kInternal;
    }
    g_scratch[dev].levels = static_cast<float*>(levels);
    g_scratch[dev].flag = static_cast<int32_t*>(flag);
  }
  *out = g_scratch[dev];
  return kOk;
}

int32_t fail(int32_t status, const std::string& message) {
  set_last_error(message.c_str());
  return status;
}

// True when `p` is device (or managed) memory of device `dev`.  A host
// pointer, pageable or pinned, would make the kernels fault or, where the GPU
// can reach host memory, read and write the wrong memory.
bool on_device(const void* p, int dev, std::string* why) {
  cudaPointerAttributes a{};
  const cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *why = std::string("cudaPointerGetAttributes: ") + cudaGetErrorString(e);
    return false;
  }
  if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) {
    *why = "not device memory";
    return false;
  }
  if (a.device != dev) {
    *why = "memory of device " + std::to_string(a.device) + ", not of the current device " + std::to_string(dev);
    return false;
  }
  return true;
}

}  // namespace
}  // namespace mvg

using namespace mvg;

extern "C" MVG_API int32_t mvg_ncc_pyramid_level_noalloc(const void* pixels, int32_t pixel_type, int64_t width,
                                                         int64_t height, int64_t row_stride, int32_t level,
                                                         float* out, int64_t out_capacity, int64_t* out_width,
                                                         int64_t* out_height, void* stream) {
  if (!pixels || !out) return fail(kInvalidArgument, "pixels and out must be device pointers, not null");
  if (pixel_type != MVG_PIXEL_BYTE && pixel_type != MVG_PIXEL_UINT2)
    return fail(kTypeMismatch, "one byte or uint2 channel required");
  const int64_t bpp = pixel_type == MVG_PIXEL_UINT2 ? 2 : 1;
  if (width <= 0 || height <= 0 || width > (1 << 30) || height > (1 << 30) || row_stride < width * bpp ||
      row_stride % bpp)
    return fail(kInvalidArgument, "invalid image geometry");
  if (reinterpret_cast<uintptr_t>(pixels) % uintptr_t(bpp))
    return fail(kInvalidArgument, "pixels must be aligned to the pixel size");
  if (reinterpret_cast<uintptr_t>(out) % alignof(float)) return fail(kInvalidArgument, "out must be 4-byte aligned");
  if (level < 0 || level > 15) return fail(kInvalidArgument, "level must be 0..15");
  // the pyramid kernels run one block per 8 rows; the grid's y extent is 65535
  if (height > int64_t(kMaxRows)) return fail(kLimitExceeded, "image taller than " + std::to_string(kMaxRows) + " rows");
  // level geometry (2x2 sums, floor, never below one pixel) and the scratch
  // the levels below the requested one need
  int64_t w = width, h = height, below = 0;
  for (int l = 0; l < level; ++l) {
    below += w * h;
    w = w / 2 > 1 ? w / 2 : 1;
    h = h / 2 > 1 ? h / 2 : 1;
  }
  if (below > int64_t(kScratchFloats))
    return fail(kLimitExceeded, "image too large for the fixed pyramid scratch: levels below the requested one need " +
                                    std::to_string(below) + " floats, the scratch holds " +
                                    std::to_string(kScratchFloats));
  if (w * h > out_capacity) return fail(kInvalidArgument, "output capacity too small for the level");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(kInternal, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  }
  std::string why;
  if (!on_device(pixels, dev, &why)) return fail(kInvalidArgument, "pixels: " + why);
  if (!on_device(out, dev, &why)) return fail(kInvalidArgument, "out: " + why);
  DeviceScratch sc;
  const int32_t st = scratch_of_device(dev, &sc, &why);
  if (st != kOk) return fail(st, why);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  e = cudaMemsetAsync(sc.flag, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return fail(kInternal, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  LevelImage prev;
  int64_t at = 0, lw = width, lh = height;
  for (int l = 0; l <= level; ++l) {
    LevelImage cur;
    cur.w = int(lw);
    cur.h = int(lh);
    cur.v = l == level ? out : sc.levels + at;
    e = l == 0 ? launch_pyramid0(pixels, pixel_type, row_stride / bpp, 0, 0, cur, sc.flag, s)
               : launch_pyramid(prev, cur, sc.flag, s);
    if (e != cudaSuccess) return fail(kInternal, std::string("pyramid launch: ") + cudaGetErrorString(e));
    at += lw * lh;
    prev = cur;
    lw = lw / 2 > 1 ? lw / 2 : 1;
    lh = lh / 2 > 1 ? lh / 2 : 1;
  }
  int32_t flag = 0;
  e = cudaMemcpyAsync(&flag, sc.flag, sizeof(flag), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(kInternal, std::string("pyramid: ") + cudaGetErrorString(e));
  if (flag) return fail(kUnsupported, "pyramid sums exceed the exact float range");
  if (out_width) *out_width = w;
  if (out_height) *out_height = h;
  set_last_error("");
  return kOk;
}
