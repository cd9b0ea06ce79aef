// C ABI of librmn (include/rmn.h): argument checks, host/device staging and
// error reporting around the kernels.
#include <cstdarg>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <algorithm>
#include <new>
#include <vector>

#include "rmn_host.h"

namespace rmn {
namespace {
thread_local char g_error[512] = "";

// A caller array: device-resident (used in place) or host memory (staged
// through a device buffer on the call's stream).
struct Arg {
  void* dev = nullptr;
  bool owned = false;
};

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

rmn_status stage_in(const void* host_or_dev, size_t bytes, cudaStream_t st, Arg* out) {
  if (is_device_ptr(host_or_dev)) {
    out->dev = const_cast<void*>(host_or_dev);
    return RMN_OK;
  }
  cudaError_t e = rmn::staging_malloc(&out->dev, bytes ? bytes : 1, st);
  if (e != cudaSuccess) return cuda_fail(e, "staging allocation (staging)");
  out->owned = true;
  if (bytes) {
    e = cudaMemcpyAsync(out->dev, host_or_dev, bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync (host to device)");
  }
  return RMN_OK;
}

rmn_status stage_out(void* host_or_dev, size_t bytes, cudaStream_t st, Arg* out) {
  if (is_device_ptr(host_or_dev)) {
    out->dev = host_or_dev;
    return RMN_OK;
  }
  cudaError_t e = rmn::staging_malloc(&out->dev, bytes ? bytes : 1, st);
  if (e != cudaSuccess) return cuda_fail(e, "staging allocation (staging)");
  out->owned = true;
  return RMN_OK;
}

rmn_status finish_out(void* host_or_dev, size_t bytes, cudaStream_t st, const Arg& a) {
  if (!a.owned || !bytes) return RMN_OK;
  cudaError_t e = cudaMemcpyAsync(host_or_dev, a.dev, bytes, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync (device to host)");
  return RMN_OK;
}

void release(Arg& a, cudaStream_t st) {
  if (a.owned && a.dev) cudaFreeAsync(a.dev, st);
  a.dev = nullptr;
  a.owned = false;
}

// Device status word of one call.
struct Status {
  int* dev = nullptr;
  rmn_status init(cudaStream_t st) {
    cudaError_t e = rmn::staging_malloc(reinterpret_cast<void**>(&dev), sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(e, "staging allocation (status)");
    e = cudaMemsetAsync(dev, 0, sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync (status)");
    return RMN_OK;
  }
  rmn_status check(cudaStream_t st, const char* what) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, dev, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (h == kDevStackOverflow) return fail(RMN_ERR_DEVICE_LIMIT, "%s: traversal stack bound reached", what);
    if (h != kDevOk) return fail(RMN_ERR_DEVICE_LIMIT, "%s: device status %d", what, h);
    return RMN_OK;
  }
  void free(cudaStream_t st) {
    if (dev) cudaFreeAsync(dev, st);
    dev = nullptr;
  }
};
}  // namespace

bool is_device_pointer(const void* p) { return is_device_ptr(p); }

rmn_status fail(rmn_status status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_error, sizeof g_error, fmt, ap);
  va_end(ap);
  return status;
}

rmn_status cuda_fail(cudaError_t err, const char* what) {
  rmn_status s = err == cudaErrorMemoryAllocation ? RMN_ERR_OUT_OF_MEMORY : RMN_ERR_CUDA;
  return fail(s, "%s: %s (%s)", what, cudaGetErrorName(err), cudaGetErrorString(err));
}

void clear_error() { g_error[0] = 0; }

}  // namespace rmn

using namespace rmn;

namespace {

// Photo::postProcessing(options) on device buffers into `out` (device,
// 3 floats per pixel): shade, depth of field, bloom, gamma, FXAA. `plan`:
// the depth-of-field plan of this G-buffer, or null to make one.
rmn_status post_device(const float* dd, const float* ds, const float* id, const float* is, const float* gb,
                       const rmn_post_args& a, int options, float* out, cudaStream_t st,
                       const DofPlan* plan = nullptr) {
  const int W = a.width, H = a.height;
  const size_t npx = (size_t)W * H;
  const bool fx = (options & RMN_SHADE_FXAA) != 0;
  const bool dof = (options & RMN_SHADE_DEPTH_OF_FIELD) != 0, bloom = (options & RMN_SHADE_BLOOM) != 0;
  float* tmp = nullptr;
  if (fx) {
    cudaError_t e = rmn::staging_malloc(reinterpret_cast<void**>(&tmp), npx * 12, st);
    if (e != cudaSuccess) return cuda_fail(e, "staging allocation (post)");
  }
  float* target = fx ? tmp : out;
  // the gamma of compose itself only when nothing runs between shade and gamma
  const int copt = (dof || bloom) ? (options & ~RMN_SHADE_GAMMA) : options;
  cudaError_t e = launch_compose(dd, ds, id, is, gb, W, H, a.exposure, copt, target, st);
  if (e == cudaSuccess && dof)
    e = plan ? dof_apply(plan, target, st) : launch_dof(target, gb, W, H, a.focus, a.CoC, a.camera_position, st);
  if (e == cudaSuccess && bloom) e = launch_bloom(target, W, H, st);
  if (e == cudaSuccess && (dof || bloom) && (options & RMN_SHADE_GAMMA)) e = launch_gamma(target, (int)npx, st);
  if (e == cudaSuccess && fx) e = launch_fxaa(target, out, W, H, st);
  if (tmp) cudaFreeAsync(tmp, st);
  if (e != cudaSuccess) return cuda_fail(e, "post-processing launch");
  return RMN_OK;
}

// The radiance buffers and G-buffer of an rmn_image, staged in (and, for
// the in-place passes, back out).
struct ImageArgs {
  Arg b[4], gb;
  rmn_status stage(const rmn_image* img, size_t npx, cudaStream_t st, bool need_gbuffer) {
    const float* src[4] = {img->radiance_Dd, img->radiance_Ds, img->radiance_Id, img->radiance_Is};
    rmn_status r = RMN_OK;
    for (int k = 0; k < 4 && r == RMN_OK; ++k) r = stage_in(src[k], npx * 16, st, &b[k]);
    if (r == RMN_OK && need_gbuffer) r = stage_in(img->gbuffer, npx * RMN_GBUFFER_FLOATS * 4, st, &gb);
    return r;
  }
  rmn_status write_back(const rmn_image* img, size_t npx, cudaStream_t st) {
    float* dst[4] = {img->radiance_Dd, img->radiance_Ds, img->radiance_Id, img->radiance_Is};
    rmn_status r = RMN_OK;
    for (int k = 0; k < 4 && r == RMN_OK; ++k) r = finish_out(dst[k], npx * 16, st, b[k]);
    return r;
  }
  float* const* bufs() {
    for (int k = 0; k < 4; ++k) p[k] = static_cast<float*>(b[k].dev);
    return p;
  }
  void release_all(cudaStream_t st) {
    for (Arg& a : b) release(a, st);
    release(gb, st);
  }
  float* p[4] = {};
};

bool image_complete(const rmn_image* img, bool need_gbuffer) {
  return img && img->radiance_Dd && img->radiance_Ds && img->radiance_Id && img->radiance_Is &&
         (!need_gbuffer || img->gbuffer);
}

// render_multiThread's exports (src/render.cpp:641-674), in order.
struct ExportSpec {
  const char* tag;
  int options;
};
constexpr int kFull = RMN_SHADE_FULL, kFX = RMN_SHADE_FXAA, kBl = RMN_SHADE_BLOOM, kDoF = RMN_SHADE_DEPTH_OF_FIELD;
const ExportSpec kExports[RMN_EXPORTS + RMN_EXPORTS_DOF] = {
    {"DiffuseColor", RMN_SHADE_BASECOLOR},
    {"DiffuseColor_FXAA", RMN_SHADE_BASECOLOR | kFX},
    {"shapeNormal", RMN_SHADE_SHAPE_NORMAL},
    {"surfaceNormal", RMN_SHADE_SURFACE_NORMAL},
    {"Direct_Diffuse", RMN_SHADE_DIRECT | RMN_SHADE_DIFFUSE},  // after spatialClamp
    {"Direct_Specular", RMN_SHADE_DIRECT | RMN_SHADE_SPECULAR},
    {"Indirect_Diffuse", RMN_SHADE_INDIRECT | RMN_SHADE_DIFFUSE},
    {"Indirect_Specular", RMN_SHADE_INDIRECT | RMN_SHADE_SPECULAR},
    {"Raw", kFull},
    {"Raw_Bloom", kFull | kBl},
    {"Raw_FXAA", kFull | kFX},
    {"Raw_Bloom_FXAA", kFull | kBl | kFX},
    {"Direct_Diffuse_Filter", RMN_SHADE_DIRECT | RMN_SHADE_DIFFUSE},  // after filter
    {"Direct_Specular_Filter", RMN_SHADE_DIRECT | RMN_SHADE_SPECULAR},
    {"Indirect_Diffuse_Filter", RMN_SHADE_INDIRECT | RMN_SHADE_DIFFUSE},
    {"Indirect_Specular_Filter", RMN_SHADE_INDIRECT | RMN_SHADE_SPECULAR},
    {"Filter", kFull},
    {"Filter_Bloom", kFull | kBl},
    {"Filter_FXAA", kFull | kFX},
    {"Filter_Bloom_FXAA", kFull | kBl | kFX},
    {"BaseColor_DepthFieldBlur", RMN_SHADE_BASECOLOR | kDoF},  // when CoC > eps
    {"Filter_DepthFieldBlur", kFull | kDoF},
    {"Filter_DepthFieldBlur_Bloom", kFull | kDoF | kBl},
    {"Filter_DepthFieldBlur_FXAA", kFull | kDoF | kFX},
    {"Filter_DepthFieldBlur_Bloom_FXAA", kFull | kDoF | kBl | kFX},
};

rmn_status check_post(const rmn_post_args* a) {
  if (!a || a->width <= 0 || a->height <= 0 || a->height > 65535 || (int64_t)a->width * a->height > (1LL << 30))
    return fail(RMN_ERR_INVALID_ARGUMENT, "post arguments: image size out of range (height <= 65535)");
  // a finite, non-negative CoC keeps every blur radius in [0, 96]
  if (!(a->CoC >= 0.0f) || !std::isfinite(a->CoC))
    return fail(RMN_ERR_INVALID_ARGUMENT, "post arguments: CoC must be finite and >= 0");
  return RMN_OK;
}

}  // namespace

extern "C" {

const char* rmn_last_error(void) { return g_error; }

const char* rmn_version(void) { return "raym0nade-gb300 0.1 (sm_103a)"; }

rmn_status rmn_scene_create(const rmn_scene_desc* desc, rmn_scene** out) {
  clear_error();
  if (!out) return fail(RMN_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  rmn_scene* s = new (std::nothrow) rmn_scene();
  if (!s) return fail(RMN_ERR_OUT_OF_MEMORY, "host allocation failed");
  cudaGetDevice(&s->device);
  rmn_status st;
  try {
    st = build_scene(desc, s);
  } catch (const std::bad_alloc&) {
    st = fail(RMN_ERR_OUT_OF_MEMORY, "host allocation failed while building the scene");
  } catch (...) {
    st = fail(RMN_ERR_INTERNAL, "unexpected exception while building the scene");
  }
  if (st != RMN_OK) {
    free_scene(s);
    delete s;
    return st;
  }
  *out = s;
  return RMN_OK;
}

rmn_status rmn_scene_destroy(rmn_scene* scene) {
  clear_error();
  if (!scene) return RMN_OK;
  free_scene(scene);
  delete scene;
  return RMN_OK;
}

rmn_status rmn_release_cached_memory(void) {
  clear_error();
  release_cached_memory();
  noalloc_forget_addresses();
  return RMN_OK;
}

rmn_status rmn_scene_info_get(const rmn_scene* scene, rmn_scene_info* info) {
  clear_error();
  if (!scene || !info) return fail(RMN_ERR_INVALID_ARGUMENT, "scene or info is NULL");
  *info = scene->info;
  return RMN_OK;
}

rmn_status rmn_scene_texture_get(const rmn_scene* scene, int32_t texture, int32_t level, rmn_image_desc* info,
                                 uint8_t* out, size_t capacity) {
  clear_error();
  if (!scene || !info) return fail(RMN_ERR_INVALID_ARGUMENT, "scene or info is NULL");
  if (texture < 0 || texture >= (int32_t)scene->textures.size())
    return fail(RMN_ERR_INVALID_ARGUMENT, "texture %d: the scene holds %zu textures", texture, scene->textures.size());
  const DevTex& t = scene->textures[texture];
  if (level < 0 || level >= t.depth)
    return fail(RMN_ERR_INVALID_ARGUMENT, "level %d: texture %d has %d levels", level, texture, t.depth);
  info->width = t.w >> level;
  info->height = t.h >> level;
  info->channels = 4;
  info->bytes_per_channel = 1;
  if (!out) return RMN_OK;
  const size_t n = (size_t)info->width * info->height * 4;
  if (capacity < n) return fail(RMN_ERR_INVALID_ARGUMENT, "%zu bytes needed, %zu given", n, capacity);
  cudaError_t e = cudaMemcpy(out, scene->dev.texels + t.off[level], n, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy (rmn_scene_texture_get)");
  return RMN_OK;
}

static rmn_status trace_common(rmn_scene* scene, const rmn_ray* rays, int64_t n, void* out, size_t out_bytes,
                               bool shadow, void* stream) {
  clear_error();
  if (!scene || (n > 0 && (!rays || !out))) return fail(RMN_ERR_INVALID_ARGUMENT, "NULL scene, rays or output");
  if (n < 0) return fail(RMN_ERR_INVALID_ARGUMENT, "negative ray count");
  if (n == 0) return RMN_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  Arg in, o;
  Status status;
  rmn_status r = stage_in(rays, (size_t)n * sizeof(rmn_ray), st, &in);
  if (r == RMN_OK) r = stage_out(out, out_bytes, st, &o);
  if (r == RMN_OK) r = status.init(st);
  if (r == RMN_OK) {
    cudaError_t e = shadow ? launch_trace_shadow(scene->dev, static_cast<const rmn_ray*>(in.dev), n,
                                                 static_cast<uint8_t*>(o.dev), status.dev, st)
                           : launch_trace_closest(scene->dev, static_cast<const rmn_ray*>(in.dev), n,
                                                  static_cast<rmn_hit*>(o.dev), status.dev, st);
    if (e != cudaSuccess) r = cuda_fail(e, shadow ? "trace_shadow launch" : "trace_closest launch");
  }
  if (r == RMN_OK) r = finish_out(out, out_bytes, st, o);
  rmn_status r2 = status.dev ? status.check(st, shadow ? "rmn_trace_shadow" : "rmn_trace_closest") : RMN_OK;
  release(in, st);
  release(o, st);
  status.free(st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (r == RMN_OK) r = r2;
  if (r == RMN_OK && e != cudaSuccess) r = cuda_fail(e, "stream synchronize");
  return r;
}

rmn_status rmn_trace_closest(rmn_scene* scene, const rmn_ray* rays, int64_t n, rmn_hit* hits, void* stream) {
  return trace_common(scene, rays, n, hits, (size_t)n * sizeof(rmn_hit), false, stream);
}

rmn_status rmn_trace_shadow(rmn_scene* scene, const rmn_ray* rays, int64_t n, uint8_t* occluded, void* stream) {
  return trace_common(scene, rays, n, occluded, (size_t)n, true, stream);
}

rmn_status rmn_fxaa(const float* rgb_in, float* rgb_out, int32_t width, int32_t height, void* stream) {
  clear_error();
  if (!rgb_in || !rgb_out || width <= 0 || height <= 0) return fail(RMN_ERR_INVALID_ARGUMENT, "bad FXAA arguments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  size_t bytes = (size_t)width * height * 3 * sizeof(float);
  Arg in, o;
  rmn_status r = stage_in(rgb_in, bytes, st, &in);
  if (r == RMN_OK) r = stage_out(rgb_out, bytes, st, &o);
  if (r == RMN_OK) {
    cudaError_t e = launch_fxaa(static_cast<const float*>(in.dev), static_cast<float*>(o.dev), width, height, st);
    if (e != cudaSuccess) r = cuda_fail(e, "fxaa launch");
  }
  if (r == RMN_OK) r = finish_out(rgb_out, bytes, st, o);
  release(in, st);
  release(o, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (r == RMN_OK && e != cudaSuccess) r = cuda_fail(e, "stream synchronize");
  return r;
}

rmn_status rmn_post_process(const rmn_image* image, const rmn_post_args* args, int32_t options, float* rgb,
                            void* stream) {
  clear_error();
  rmn_status r = check_post(args);
  if (r != RMN_OK) return r;
  if (!rgb || !image_complete(image, true))
    return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_post_process needs all four radiance buffers, the G-buffer and rgb");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t npx = (size_t)args->width * args->height;
  ImageArgs in;
  Arg o;
  r = in.stage(image, npx, st, true);
  if (r == RMN_OK) r = stage_out(rgb, npx * 12, st, &o);
  if (r == RMN_OK) {
    float* const* b = in.bufs();
    r = post_device(b[0], b[1], b[2], b[3], static_cast<const float*>(in.gb.dev), *args, options,
                    static_cast<float*>(o.dev), st);
  }
  if (r == RMN_OK) r = finish_out(rgb, npx * 12, st, o);
  in.release_all(st);
  release(o, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (r == RMN_OK && e != cudaSuccess) r = cuda_fail(e, "stream synchronize");
  return r;
}

rmn_status rmn_spatial_clamp(const rmn_image* image, int32_t width, int32_t height, void* stream) {
  clear_error();
  if (!image_complete(image, false) || width <= 0 || height <= 0 || height > 65535)
    return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_spatial_clamp needs the four radiance buffers and a size");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t npx = (size_t)width * height;
  ImageArgs in;
  rmn_status r = in.stage(image, npx, st, false);
  if (r == RMN_OK) {
    cudaError_t e = launch_spatial_clamp(in.bufs(), width, height, st);
    if (e != cudaSuccess) r = cuda_fail(e, "spatial clamp launch");
  }
  if (r == RMN_OK) r = in.write_back(image, npx, st);
  in.release_all(st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (r == RMN_OK && e != cudaSuccess) r = cuda_fail(e, "stream synchronize");
  return r;
}

rmn_status rmn_filter(const rmn_image* image, int32_t width, int32_t height, void* stream) {
  clear_error();
  if (!image_complete(image, true) || width <= 0 || height <= 0 || height > 65535)
    return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_filter needs the four radiance buffers, the G-buffer and a size");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t npx = (size_t)width * height;
  ImageArgs in;
  rmn_status r = in.stage(image, npx, st, true);
  if (r == RMN_OK) {
    cudaError_t e = launch_filter(in.bufs(), static_cast<const float*>(in.gb.dev), width, height, st);
    if (e != cudaSuccess) r = cuda_fail(e, "filter launch");
  }
  if (r == RMN_OK) r = in.write_back(image, npx, st);
  in.release_all(st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (r == RMN_OK && e != cudaSuccess) r = cuda_fail(e, "stream synchronize");
  return r;
}

rmn_status rmn_export_set(const rmn_image* image, const rmn_post_args* args, float* rgb, int32_t* count,
                          void* stream) {
  clear_error();
  rmn_status r = check_post(args);
  if (r != RMN_OK) return r;
  if (!rgb || !count || !image_complete(image, true))
    return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_export_set needs the radiance buffers, the G-buffer, rgb and count");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t npx = (size_t)args->width * args->height;
  const int n = RMN_EXPORTS + (args->CoC > RMN_EPS ? RMN_EXPORTS_DOF : 0);
  ImageArgs in;
  Arg o;
  r = in.stage(image, npx, st, true);
  if (r == RMN_OK) r = stage_out(rgb, npx * 12 * n, st, &o);
  float* const* b = in.bufs();
  const float* gb = static_cast<const float*>(in.gb.dev);
  DofPlan* plan = nullptr;  // one depth order for the five depth-of-field exports
  for (int k = 0; k < n && r == RMN_OK; ++k) {
    cudaError_t e = cudaSuccess;
    if (k == 4) e = launch_spatial_clamp(b, args->width, args->height, st);  // photo.spatialClamp()
    if (k == 12) e = launch_filter(b, gb, args->width, args->height, st);    // photo.filter()
    if (e == cudaSuccess && !plan && (kExports[k].options & RMN_SHADE_DEPTH_OF_FIELD))
      e = dof_plan_create(gb, args->width, args->height, args->focus, args->CoC, args->camera_position, st, &plan);
    if (e != cudaSuccess) {
      r = cuda_fail(e, "export pass launch");
      break;
    }
    r = post_device(b[0], b[1], b[2], b[3], gb, *args, kExports[k].options | RMN_SHADE_GAMMA,
                    static_cast<float*>(o.dev) + 3 * npx * k, st, plan);
  }
  dof_plan_destroy(plan, st);
  if (r == RMN_OK) r = finish_out(rgb, npx * 12 * n, st, o);
  if (r == RMN_OK) r = in.write_back(image, npx, st);
  in.release_all(st);
  release(o, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (r == RMN_OK && e != cudaSuccess) r = cuda_fail(e, "stream synchronize");
  *count = r == RMN_OK ? n : 0;
  return r;
}

rmn_status rmn_reverse_gamma(const float* in, int64_t n, float* out) {
  clear_error();
  if (!in || !out || n < 0) return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_reverse_gamma needs host arrays and n >= 0");
  for (int64_t i = 0; i < 3 * n; ++i) out[i] = powf(in[i], 2.2f);
  return RMN_OK;
}

rmn_status rmn_save_png(const float* rgb, int32_t width, int32_t height, const char* path) {
  clear_error();
  if (!rgb || !path || width <= 0 || height <= 0 || (int64_t)width * height > (1LL << 30))
    return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_save_png needs an image, a size and a path");
  const size_t n = (size_t)width * height * 3;
  try {  // no C++ exception crosses the ABI
    if (is_device_ptr(rgb)) {
      std::vector<float> h(n);
      cudaError_t e = cudaMemcpy(h.data(), rgb, n * sizeof(float), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy (rmn_save_png)");
      return write_png(h.data(), width, height, path);
    }
    return write_png(rgb, width, height, path);
  } catch (const std::bad_alloc&) {
    return fail(RMN_ERR_OUT_OF_MEMORY, "out of host memory writing %s", path);
  }
}

const char* rmn_export_tag(int32_t k) {
  return (k >= 0 && k < RMN_EXPORTS + RMN_EXPORTS_DOF) ? kExports[k].tag : nullptr;
}

int32_t rmn_export_options(int32_t k) {
  return (k >= 0 && k < RMN_EXPORTS + RMN_EXPORTS_DOF) ? (kExports[k].options | RMN_SHADE_GAMMA) : -1;
}

rmn_status rmn_compose(const rmn_image* image, int32_t width, int32_t height, float exposure, int32_t options,
                       float* rgb, void* stream) {
  clear_error();
  options &= ~(RMN_SHADE_BLOOM | RMN_SHADE_DEPTH_OF_FIELD);  // rmn_post_process's passes
  if (!image || !rgb || width <= 0 || height <= 0 || !image->gbuffer || !image->radiance_Dd || !image->radiance_Ds ||
      !image->radiance_Id || !image->radiance_Is)
    return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_compose needs all four radiance buffers and the G-buffer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  size_t npx = (size_t)width * height;
  Arg dd, ds, id, is, gb, o, tmp;
  rmn_status r = stage_in(image->radiance_Dd, npx * 16, st, &dd);
  if (r == RMN_OK) r = stage_in(image->radiance_Ds, npx * 16, st, &ds);
  if (r == RMN_OK) r = stage_in(image->radiance_Id, npx * 16, st, &id);
  if (r == RMN_OK) r = stage_in(image->radiance_Is, npx * 16, st, &is);
  if (r == RMN_OK) r = stage_in(image->gbuffer, npx * RMN_GBUFFER_FLOATS * 4, st, &gb);
  if (r == RMN_OK) r = stage_out(rgb, npx * 12, st, &o);
  bool fx = (options & RMN_SHADE_FXAA) != 0;
  if (r == RMN_OK && fx) {
    cudaError_t e = rmn::staging_malloc(&tmp.dev, npx * 12, st);
    if (e != cudaSuccess) r = cuda_fail(e, "staging allocation (compose)");
    tmp.owned = true;
  }
  if (r == RMN_OK) {
    float* target = fx ? static_cast<float*>(tmp.dev) : static_cast<float*>(o.dev);
    cudaError_t e = launch_compose(static_cast<const float*>(dd.dev), static_cast<const float*>(ds.dev),
                                   static_cast<const float*>(id.dev), static_cast<const float*>(is.dev),
                                   static_cast<const float*>(gb.dev), width, height, exposure, options, target, st);
    if (e == cudaSuccess && fx) e = launch_fxaa(target, static_cast<float*>(o.dev), width, height, st);
    if (e != cudaSuccess) r = cuda_fail(e, "compose launch");
  }
  if (r == RMN_OK) r = finish_out(rgb, npx * 12, st, o);
  for (Arg* a : {&dd, &ds, &id, &is, &gb, &o, &tmp}) release(*a, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (r == RMN_OK && e != cudaSuccess) r = cuda_fail(e, "stream synchronize");
  return r;
}

}  // extern "C"

static rmn_status check_args(const rmn_render_args& a) {
  if (a.width <= 0 || a.height <= 0 || (int64_t)a.width * a.height > (1LL << 30))
    return fail(RMN_ERR_INVALID_ARGUMENT, "image size %d x %d out of range", a.width, a.height);
  if (a.spp < 0 || a.spp > (1 << 20)) return fail(RMN_ERR_INVALID_ARGUMENT, "spp %d out of range", a.spp);
  if (!(a.P_Direct >= 0.0f && a.P_Direct <= 1.0f)) return fail(RMN_ERR_INVALID_ARGUMENT, "P_Direct must lie in [0, 1]");
  if (a.max_depth < 1 || a.max_depth > 16) return fail(RMN_ERR_INVALID_ARGUMENT, "max_depth must lie in [1, 16]");
  int k = a.lanes_per_pixel;
  if (k < 0 || k > 64) return fail(RMN_ERR_INVALID_ARGUMENT, "lanes_per_pixel must lie in [0, 64]");
  if (a.slots_per_unit < 0 || a.slots_per_unit > (1 << 20))
    return fail(RMN_ERR_INVALID_ARGUMENT, "slots_per_unit must lie in [0, 2^20]");
  return RMN_OK;
}

// rmn_render / rmn_render_profile_get: a one-render batch without a graph.
static rmn_status render_one(rmn_scene* scene, const rmn_render_args* args, const rmn_image* image, void* stream,
                             RenderProfileData* prof) {
  clear_error();
  if (!scene || !args || !image) return fail(RMN_ERR_INVALID_ARGUMENT, "NULL scene, args or image");
  if (!image->radiance_Dd || !image->radiance_Ds || !image->radiance_Id || !image->radiance_Is)
    return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_render needs the four radiance buffers");
  const rmn_render_args& a = *args;
  rmn_status r = check_args(a);
  if (r != RMN_OK) return r;
  if (scene->dev.num_lights > 8) return fail(RMN_ERR_UNSUPPORTED, "more than 8 light objects");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t npx = (size_t)a.width * a.height;
  Arg dd, ds, id, is, gb, dr;
  r = stage_out(image->radiance_Dd, npx * 16, st, &dd);
  if (r == RMN_OK && image->dropped) r = stage_out(image->dropped, npx * 4, st, &dr);
  if (r == RMN_OK) r = stage_out(image->radiance_Ds, npx * 16, st, &ds);
  if (r == RMN_OK) r = stage_out(image->radiance_Id, npx * 16, st, &id);
  if (r == RMN_OK) r = stage_out(image->radiance_Is, npx * 16, st, &is);
  if (r == RMN_OK) {
    if (image->gbuffer) {
      r = stage_out(image->gbuffer, npx * RMN_GBUFFER_FLOATS * 4, st, &gb);
    } else {
      cudaError_t e = rmn::staging_malloc(&gb.dev, npx * RMN_GBUFFER_FLOATS * 4, st);
      if (e != cudaSuccess) r = cuda_fail(e, "staging allocation (G-buffer)");
      gb.owned = true;
    }
  }
  BatchState* b = nullptr;
  if (r == RMN_OK) {
    RenderItem it{scene, a, static_cast<float*>(gb.dev), static_cast<float*>(dd.dev), static_cast<float*>(ds.dev),
                  static_cast<float*>(id.dev), static_cast<float*>(is.dev), static_cast<int*>(dr.dev)};
    r = batch_create(&it, 1, false, 0, 0, 0, 0, st, &b);
  }
  if (r == RMN_OK) r = prof ? batch_profile(b, st, prof) : batch_launch(b, st);
  if (r == RMN_OK) r = finish_out(image->radiance_Dd, npx * 16, st, dd);
  if (r == RMN_OK) r = finish_out(image->radiance_Ds, npx * 16, st, ds);
  if (r == RMN_OK) r = finish_out(image->radiance_Id, npx * 16, st, id);
  if (r == RMN_OK) r = finish_out(image->radiance_Is, npx * 16, st, is);
  if (r == RMN_OK && image->gbuffer) r = finish_out(image->gbuffer, npx * RMN_GBUFFER_FLOATS * 4, st, gb);
  if (r == RMN_OK && image->dropped) r = finish_out(image->dropped, npx * 4, st, dr);
  if (r == RMN_OK && b) r = batch_status(b, st);
  for (Arg* x : {&dd, &ds, &id, &is, &gb, &dr}) release(*x, st);
  cudaError_t e = cudaStreamSynchronize(st);
  batch_destroy(b);
  if (r == RMN_OK && e != cudaSuccess) r = cuda_fail(e, "stream synchronize");
  return r;
}

extern "C" {

rmn_status rmn_adjoint(const rmn_scene* scene, const rmn_render_args* args, const rmn_image* image,
                       const float* d_image, float* d_materials, void* stream) {
  clear_error();
  if (!scene || !args || !image || !d_image || !d_materials)
    return fail(RMN_ERR_INVALID_ARGUMENT, "NULL scene, args, image, d_image or d_materials");
  if (!image->gbuffer || !image->dropped)
    return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_adjoint needs the forward's G-buffer and dropped-sample record");
  if (scene->dev.has_glass)
    return fail(RMN_ERR_UNSUPPORTED, "rmn_adjoint: transmissive and half-opaque materials are not differentiated");
  if (scene->dev.has_tex)
    return fail(RMN_ERR_UNSUPPORTED, "rmn_adjoint: textured materials are not differentiated");
  const rmn_render_args& a = *args;
  rmn_status r = check_args(a);
  if (r != RMN_OK) return r;
  if (scene->dev.num_lights > 8) return fail(RMN_ERR_UNSUPPORTED, "more than 8 light objects");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t npx = (size_t)a.width * a.height;
  const size_t nm = (size_t)scene->dev.num_mats * RMN_GRAD_PER_MATERIAL;
  Arg gb, dr, di, dm;
  r = stage_in(image->gbuffer, npx * RMN_GBUFFER_FLOATS * 4, st, &gb);
  if (r == RMN_OK) r = stage_in(image->dropped, npx * 4, st, &dr);
  if (r == RMN_OK) r = stage_in(d_image, npx * 12, st, &di);
  if (r == RMN_OK) r = stage_out(d_materials, nm * 4, st, &dm);
  if (r == RMN_OK)
    r = launch_adjoint(scene, a, static_cast<const float*>(gb.dev), static_cast<const int*>(dr.dev),
                       static_cast<const float*>(di.dev), static_cast<float*>(dm.dev), st);
  if (r == RMN_OK) r = finish_out(d_materials, nm * 4, st, dm);
  for (Arg* x : {&gb, &dr, &di, &dm}) release(*x, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (r == RMN_OK && e != cudaSuccess) r = cuda_fail(e, "stream synchronize");
  return r;
}

rmn_status rmn_render(rmn_scene* scene, const rmn_render_args* args, const rmn_image* image, void* stream) {
  return render_one(scene, args, image, stream, nullptr);
}

static void put_profile(const RenderProfileData& p, rmn_render_profile* out) {
  out->primary_ms = p.primary_ms;
  out->path_ms = p.path_ms;
  out->logic_ms = p.logic_ms;
  out->trace_ms = p.trace_ms;
  out->iterations = p.iterations;
  out->closest_rays = p.closest;
  out->shadow_rays = p.shadow;
  out->inner_visits = p.inner;
  out->leaf_visits = p.leaves;
  out->triangle_tests = p.tris;
  out->sample_slots = p.slots;
  out->pixels = p.pixels;
}

rmn_status rmn_render_profile_get(rmn_scene* scene, const rmn_render_args* args, const rmn_image* image,
                                  rmn_render_profile* out, void* stream) {
  if (!out) return fail(RMN_ERR_INVALID_ARGUMENT, "out is NULL");
  RenderProfileData p{};
  rmn_status r = render_one(scene, args, image, stream, &p);
  if (r == RMN_OK) put_profile(p, out);
  return r;
}

struct rmn_batch {
  BatchState* state = nullptr;
};

static rmn_status make_items(const rmn_batch_item* items, int32_t n, std::vector<RenderItem>& its, bool device_only);

rmn_status rmn_batch_create(const rmn_batch_item* items, int32_t n, const rmn_batch_options* options, void* stream,
                            rmn_batch** out) {
  clear_error();
  if (!items || n <= 0 || !out) return fail(RMN_ERR_INVALID_ARGUMENT, "a batch needs at least one item");
  *out = nullptr;
  rmn_batch_options opt = options ? *options : rmn_batch_options{1, 0, 0, 0, 0, 0};
  if (opt.pool_workers < 0) return fail(RMN_ERR_INVALID_ARGUMENT, "pool_workers must be >= 0");
  if (opt.ray_order != 0 && opt.ray_order != 1) return fail(RMN_ERR_INVALID_ARGUMENT, "ray_order must be 0 or 1");
  if (opt.lanes < 0 || opt.lanes > 4) return fail(RMN_ERR_INVALID_ARGUMENT, "lanes must lie in [0, 4]");
  if (opt.stack_entries != 0 && opt.stack_entries != RMN_STACK_SMALL && opt.stack_entries != RMN_STACK)
    return fail(RMN_ERR_INVALID_ARGUMENT, "stack_entries must be 0, %d or %d", RMN_STACK_SMALL, RMN_STACK);
  std::vector<RenderItem> its;
  rmn_status r = make_items(items, n, its, true);
  if (r != RMN_OK) return r;
  rmn_batch* bt = new (std::nothrow) rmn_batch();
  if (!bt) return fail(RMN_ERR_OUT_OF_MEMORY, "host allocation failed");
  r = batch_create(its.data(), n, opt.use_graph != 0, opt.pool_workers, opt.lanes, opt.stack_entries,
                   opt.ray_order, static_cast<cudaStream_t>(stream), &bt->state);
  if (r != RMN_OK) {
    delete bt;
    return r;
  }
  *out = bt;
  return RMN_OK;
}

static rmn_status make_items(const rmn_batch_item* items, int32_t n, std::vector<RenderItem>& its, bool device_only) {
  its.clear();
  its.reserve(n);
  int64_t total = 0;
  for (int i = 0; i < n; ++i) {
    const rmn_batch_item& b = items[i];
    if (!b.scene) return fail(RMN_ERR_INVALID_ARGUMENT, "batch item %d has no scene", i);
    rmn_status r = check_args(b.args);
    if (r != RMN_OK) return fail(r, "batch item %d: %s", i, rmn_last_error());
    if (b.scene->dev.num_lights > 8) return fail(RMN_ERR_UNSUPPORTED, "batch item %d: more than 8 light objects", i);
    const rmn_image& im = b.image;
    for (const void* p : {(const void*)im.radiance_Dd, (const void*)im.radiance_Ds, (const void*)im.radiance_Id,
                          (const void*)im.radiance_Is, (const void*)im.gbuffer})
      if (device_only && !is_device_ptr(p))
        return fail(RMN_ERR_INVALID_ARGUMENT, "batch item %d: batch buffers (all five) must be device memory", i);
    total += (int64_t)b.args.width * b.args.height;
    if (total > (1LL << 31) - 1) return fail(RMN_ERR_INVALID_ARGUMENT, "a batch holds at most 2^31 - 1 pixels");
    if (im.dropped && device_only && !is_device_ptr(im.dropped))
      return fail(RMN_ERR_INVALID_ARGUMENT, "batch item %d: batch buffers must be device memory", i);
    its.push_back(RenderItem{b.scene, b.args, im.gbuffer, im.radiance_Dd, im.radiance_Ds, im.radiance_Id,
                             im.radiance_Is, im.dropped});
  }
  return RMN_OK;
}

rmn_status rmn_batch_device_bytes(const rmn_batch_item* items, int32_t n, const rmn_batch_options* options,
                                  int64_t* out) {
  clear_error();
  if (!items || n <= 0 || !out) return fail(RMN_ERR_INVALID_ARGUMENT, "a batch needs at least one item and an output");
  const rmn_batch_options opt = options ? *options : rmn_batch_options{1, 0, 0, 0, 0, 0};
  if (opt.pool_workers < 0 || opt.lanes < 0 || opt.lanes > 4)
    return fail(RMN_ERR_INVALID_ARGUMENT, "pool_workers must be >= 0 and lanes lie in [0, 4]");
  std::vector<RenderItem> its;
  rmn_status r = make_items(items, n, its, false);
  if (r != RMN_OK) return r;
  *out = (int64_t)batch_device_bytes(its.data(), n, opt.pool_workers, opt.lanes, opt.ray_order);
  return RMN_OK;
}

rmn_status rmn_batch_autotune(const rmn_batch_item* items, int32_t n, float pixel_fraction, rmn_tune_result* out,
                              void* stream) {
  clear_error();
  if (!items || n <= 0 || !out) return fail(RMN_ERR_INVALID_ARGUMENT, "autotune needs at least one item and an output");
  if (!(pixel_fraction > 0.0f && pixel_fraction <= 1.0f))
    return fail(RMN_ERR_INVALID_ARGUMENT, "pixel_fraction must lie in (0, 1]");
  std::vector<RenderItem> its;
  rmn_status r = make_items(items, n, its, false);
  if (r != RMN_OK) return r;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // Candidates whose full-size batch would take more than half of the free
  // device memory are not tried.
  const std::vector<RenderItem> full = its;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    free_b = 0;
  }
  auto fits = [&](int slots, int pool, int lanes, int order) {
    std::vector<RenderItem> f = full;
    for (RenderItem& it : f) it.args.slots_per_unit = slots;
    return batch_device_bytes(f.data(), n, pool, lanes, order) <= free_b / 2;
  };
  // the batch cannot be built at all when its default unit records and the
  // smallest pool exceed what is free
  if (batch_device_bytes(full.data(), n, 4096, 1) > free_b)
    return fail(RMN_ERR_OUT_OF_MEMORY, "autotune: no configuration of this batch fits in the %zu free device bytes",
                free_b);
  // Proxy renders: the same scenes, spp, depth and field of view at a
  // fraction of the pixels, into buffers owned by the tuner. A candidate's
  // pool is scaled by the same fraction for its proxy run, so each worker
  // has as many units to work through as in the full batch: the proxy then
  // runs the full batch's number of wavefront iterations, its fill and its
  // drain, instead of a pool the size of the full batch's draining after
  // one pass over a sixteenth of the work.
  const float scale = std::sqrt(pixel_fraction);
  std::vector<void*> bufs;
  cudaError_t e = cudaSuccess;
  double pix_full = 0.0, pix_proxy = 0.0;
  for (RenderItem& it : its) {
    rmn_render_args& a = it.args;
    int w = std::max(8, (int)std::lround(a.width * scale)), h = std::max(8, (int)std::lround(a.height * scale));
    pix_full += (double)a.width * a.height;
    pix_proxy += (double)w * h;
    a.accuracy *= (float)a.width / (float)w;
    a.width = w;
    a.height = h;
    a.lanes_per_pixel = 0;
    it.dropped = nullptr;
    float** dst[5] = {&it.gbuf, &it.dd, &it.ds, &it.id, &it.is};
    size_t bytes[5] = {(size_t)w * h * RMN_GBUFFER_FLOATS * 4, (size_t)w * h * 16, (size_t)w * h * 16,
                       (size_t)w * h * 16, (size_t)w * h * 16};
    for (int k = 0; k < 5 && e == cudaSuccess; ++k) {
      void* p = nullptr;
      e = cudaMalloc(&p, bytes[k]);
      if (e == cudaSuccess) {
        bufs.push_back(p);
        *dst[k] = static_cast<float*>(p);
      }
    }
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e != cudaSuccess) r = cuda_fail(e, "autotune set-up");
  const int slots[] = {2, 4, 8, 16};
  const int pools[] = {1 << 20, 1 << 21, 1 << 22, 1 << 23};
  const int lanes[] = {2, 3, 4};
  // candidate 0: the library's own choice (the items' slots_per_unit, pool,
  // lanes, stack and ray order left at 0); then the grid at the default
  // stack; then the fastest so far with the deeper stack build, where the
  // default is the shallow one (the stack must hold every tree, so only
  // larger stacks are admissible; they cost shared memory and so persistent
  // blocks per SM); last, the fastest so far with its ray queues binned
  const int stack_def = default_stack_entries(its.data(), n);
  rmn_tune_result best{0, 0, 1e30, 0.0, 0, 0, stack_def, 0};
  std::vector<int> proxy_slots(its.size());
  for (size_t i = 0; i < its.size(); ++i) proxy_slots[i] = its[i].args.slots_per_unit;
  const int grid = 4 * 4 * 3;
  for (int ci = -1; ci <= grid + 1 && r == RMN_OK; ++ci) {
    const bool is_default = ci < 0, stack_pass = ci == grid, order_pass = ci == grid + 1;
    if (stack_pass && stack_def == RMN_STACK) continue;
    const bool refine = stack_pass || order_pass;
    const int si = ci < 0 || refine ? 0 : ci / 12, pi = ci < 0 || refine ? 0 : (ci / 3) % 4,
              li = ci < 0 || refine ? 0 : ci % 3;
    int cs = is_default ? 0 : slots[si], cp = is_default ? 0 : pools[pi], cl = is_default ? 0 : lanes[li];
    int ck = stack_def, co = 0;
    if (refine) {
      cs = best.slots_per_unit;
      cp = best.pool_workers;
      cl = best.lanes;
      ck = stack_pass ? RMN_STACK : best.stack_entries;
      co = order_pass ? 1 : 0;
      if (order_pass && !fits(cs, cp, cl, co)) continue;
    } else if (!is_default && !fits(cs, cp, cl, 0)) {
      continue;
    }
    for (size_t i = 0; i < its.size(); ++i) its[i].args.slots_per_unit = cs == 0 ? proxy_slots[i] : cs;
    const double f = pix_proxy / pix_full;
    const int proxy_pool =
        (int)std::max<double>(4096.0, std::round((cp > 0 ? cp : kDefaultPoolWorkers) * f / 128.0) * 128.0);
    BatchState* b = nullptr;
    r = batch_create(its.data(), n, true, proxy_pool, cl, ck, co, st, &b);
    if (r != RMN_OK) break;
    r = batch_launch(b, st);  // warm-up
    if (r == RMN_OK) {
      cudaEventRecord(e0, st);
      r = batch_launch(b, st);
      cudaEventRecord(e1, st);
    }
    if (r == RMN_OK) r = batch_status(b, st);
    float ms = 0.0f;
    if (r == RMN_OK && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) r = fail(RMN_ERR_CUDA, "event timing");
    batch_destroy(b);
    if (r != RMN_OK) break;
    best.candidates++;
    if (is_default) best.default_ms = ms;
    if (ms < best.best_ms) {
      best.best_ms = ms;
      best.slots_per_unit = cs;
      best.pool_workers = cp;
      best.lanes = cl;
      best.stack_entries = ck;
      best.ray_order = co;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(st);
  for (void* p : bufs) cudaFree(p);
  if (r == RMN_OK) *out = best;
  return r;
}

rmn_status rmn_batch_update(rmn_batch* batch, const rmn_render_args* args, int32_t n, void* stream) {
  clear_error();
  if (!batch || !batch->state || !args) return fail(RMN_ERR_INVALID_ARGUMENT, "NULL batch or arguments");
  for (int i = 0; i < n; ++i) {
    rmn_status r = check_args(args[i]);
    if (r != RMN_OK) return fail(r, "rmn_batch_update item %d: %s", i, rmn_last_error());
  }
  return batch_update(batch->state, args, n, static_cast<cudaStream_t>(stream));
}

int64_t rmn_batch_update_bytes(const rmn_batch* batch) {
  return (batch && batch->state) ? (int64_t)batch_job_bytes() * batch_items(batch->state) : 0;
}

rmn_status rmn_batch_render(rmn_batch* batch, void* stream) {
  clear_error();
  if (!batch || !batch->state) return fail(RMN_ERR_INVALID_ARGUMENT, "NULL batch");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rmn_status r = batch_launch(batch->state, st);
  if (r == RMN_OK) r = batch_status(batch->state, st);
  return r;
}

rmn_status rmn_batch_profile(rmn_batch* batch, rmn_render_profile* out, void* stream) {
  clear_error();
  if (!batch || !batch->state || !out) return fail(RMN_ERR_INVALID_ARGUMENT, "NULL batch or output");
  RenderProfileData p{};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rmn_status r = batch_profile(batch->state, st, &p);
  if (r == RMN_OK) r = batch_status(batch->state, st);
  if (r == RMN_OK) put_profile(p, out);
  return r;
}

rmn_status rmn_batch_destroy(rmn_batch* batch) {
  clear_error();
  if (!batch) return RMN_OK;
  batch_destroy(batch->state);
  delete batch;
  return RMN_OK;
}

}  // extern "C"
