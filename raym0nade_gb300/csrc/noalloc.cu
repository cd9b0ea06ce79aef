// rmn_compose_noalloc: Photo::shade + gammaCorrection + FXAA without any
// device allocation, for callers that cannot allocate device memory -- a
// host application whose device memory is owned by its own arena allocator
// (so cudaMalloc fails or breaks its budget), or a frame loop that must not
// stall: cudaMalloc and cudaFree can synchronise the whole device, and the
// stream-ordered allocator may grow its pool at an arbitrary call.
//
// rmn_compose needs a temporary image between the compose and FXAA kernels
// and allocates it per call. Here that image lives in a file-scope device
// array sized for RMN_NOALLOC_MAX_PIXELS pixels (24 MiB), which every GPU
// that loads the library holds until the process exits. Nothing in it needs
// to start at zero: the compose kernel writes every pixel FXAA reads.
//
// Host code must not use g_compose_scratch's name as a device address (on
// the host it names a host-side stand-in). The first call on each device
// resolves the array's device address with cudaGetSymbolAddress, with that
// device current, and caches it; make that first call before any stream
// capture. A device reset (cudaDeviceReset) invalidates that address with the
// rest of the device's state: rmn_release_cached_memory, called after the
// reset, makes the next call resolve it again. All calls share the one
// array, so calls whose work overlaps on the GPU (different streams, or
// different host threads) race on it. A call returns once its work on
// `stream` has finished (it synchronises the stream).
#include <mutex>

#include "rmn_host.h"

namespace {

__device__ __align__(256) float g_compose_scratch[3 * RMN_NOALLOC_MAX_PIXELS];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
float* g_scratch[kMaxDevices] = {};

rmn_status scratch_for_current_device(float** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return rmn::cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices)
    return rmn::fail(RMN_ERR_UNSUPPORTED, "rmn_compose_noalloc: device %d beyond the %d it tracks", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_compose_scratch);
    if (e != cudaSuccess) return rmn::cuda_fail(e, "cudaGetSymbolAddress (rmn_compose_noalloc scratch)");
    g_scratch[dev] = static_cast<float*>(p);
  }
  *out = g_scratch[dev];
  return RMN_OK;
}

}  // namespace

namespace rmn {
void noalloc_forget_addresses() {
  std::lock_guard<std::mutex> lock(g_mu);
  for (float*& p : g_scratch) p = nullptr;
}
}  // namespace rmn

extern "C" rmn_status rmn_compose_noalloc(const rmn_image* image, int32_t width, int32_t height, float exposure,
                                          int32_t options, float* rgb, void* stream) {
  using namespace rmn;
  clear_error();
  if (!image || !rgb || width <= 0 || height <= 0 || !image->gbuffer || !image->radiance_Dd || !image->radiance_Ds ||
      !image->radiance_Id || !image->radiance_Is)
    return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_compose_noalloc needs all four radiance buffers, the G-buffer and rgb");
  if ((int64_t)width * height > RMN_NOALLOC_MAX_PIXELS)
    return fail(RMN_ERR_INVALID_ARGUMENT,
                "rmn_compose_noalloc: %d x %d pixels exceed its fixed scratch of %d pixels; use rmn_compose", width,
                height, RMN_NOALLOC_MAX_PIXELS);
  for (const void* p : {(const void*)image->radiance_Dd, (const void*)image->radiance_Ds,
                        (const void*)image->radiance_Id, (const void*)image->radiance_Is, (const void*)image->gbuffer,
                        (const void*)rgb})
    if (!is_device_pointer(p))
      return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_compose_noalloc: every buffer must be device memory (no staging)");
  float* scratch = nullptr;
  rmn_status r = scratch_for_current_device(&scratch);
  if (r != RMN_OK) return r;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool fx = (options & RMN_SHADE_FXAA) != 0;
  float* target = fx ? scratch : rgb;
  cudaError_t e = launch_compose(image->radiance_Dd, image->radiance_Ds, image->radiance_Id, image->radiance_Is,
                                 image->gbuffer, width, height, exposure, options, target, st);
  if (e == cudaSuccess && fx) e = launch_fxaa(scratch, rgb, width, height, st);
  if (e != cudaSuccess) return cuda_fail(e, "rmn_compose_noalloc launch");
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "rmn_compose_noalloc");
  return RMN_OK;
}
