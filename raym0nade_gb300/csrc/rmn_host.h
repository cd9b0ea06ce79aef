// Host-side internals of librmn: scene object, error reporting and the
// kernel launchers implemented in the .cu files.
#pragma once
#include <exception>
#include <string>
#include <thread>
#include <vector>

#include "../../include/rmn.h"
#include "rmn_internal.h"

struct rmn_scene {
  DevScene dev{};
  std::vector<void*> device_allocations;
  rmn_scene_info info{};
  int device = 0;
  void* sky_share = nullptr;  // the sky's device tables, shared by every scene with the same sky map
  std::vector<DevTex> textures;  // host copy of dev.texs (sizes, depths, level offsets)
};

namespace rmn {

rmn_status fail(rmn_status status, const char* fmt, ...);
bool is_device_pointer(const void* p);  // device or managed memory of the current context
rmn_status cuda_fail(cudaError_t err, const char* what);
void clear_error();

#define RMN_CHECK_CUDA(call)                                  \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ::rmn::cuda_fail(e_, #call); \
  } while (0)

rmn_status build_scene(const rmn_scene_desc* desc, rmn_scene* scene);
void free_scene(rmn_scene* scene);

// Device-side status word written by kernels that hit one of their bounds.
enum DeviceStatus { kDevOk = 0, kDevStackOverflow = 1, kDevBadIndex = 2, kDevMediaOverflow = 3 };

// Kernel launchers (trace.cu, render.cu, post.cu). All take device pointers.
cudaError_t launch_trace_closest(const DevScene& s, const rmn_ray* rays, int64_t n, rmn_hit* hits, int* status,
                                 cudaStream_t stream);
cudaError_t launch_trace_shadow(const DevScene& s, const rmn_ray* rays, int64_t n, uint8_t* occluded, int* status,
                                cudaStream_t stream);
// One render of a batch; all pointers are device memory.
struct RenderItem {
  const rmn_scene* scene;
  rmn_render_args args;
  float *gbuf, *dd, *ds, *id, *is;
  int* dropped;  // optional
};
struct RenderProfileData {
  double primary_ms, path_ms, logic_ms, trace_ms;
  long long iterations;
  unsigned long long closest, shadow, inner, leaves, tris, slots, pixels;
};
struct BatchState;

// The mip chains of ImageData::generateMipmaps (mips.cu): level 0 of every
// texture already in `texels` at tex[t].off[0]; levels 1.. are written at
// their offsets. Synchronises `stream`.
cudaError_t launch_build_mips(uint8_t* texels, const DevTex* tex, int ntex, cudaStream_t stream);

// Photo::save as an 8-bit RGB PNG (png.cpp); rgb in host memory.
rmn_status write_png(const float* rgb, int w, int h, const char* path);
// A decoded image file (image_io.cpp): uint8 samples or float32 values,
// row-major, row 0 = the image's top row.
struct DecodedImage {
  int w = 0, h = 0, channels = 0, bytes_per_channel = 1;
  std::vector<uint8_t> bytes;
};
// Decode `path` as RMN_IMAGE_PNG / _DDS / _HDR (the size only with header_only).
rmn_status decode_image_file(const char* path, int kind, bool header_only, DecodedImage& img);

// A binary FBX model as assimp's import with PreTransformVertices and
// Triangulate leaves it (fbx.cpp): per mesh (a geometry's polygons of one
// material) the world-space position, normal and uv of every polygon
// corner, the fan triangles over the corners and the material's index; per
// material its name, opacity and texture file names by RMN_TEX_* slot.
struct FbxMesh {
  std::vector<float> pos, nrm, uv;
  bool has_nrm = false, has_uv = false;
  std::vector<int32_t> tris;
  int material = -1;
};
struct FbxMaterial {
  std::string name;
  float opacity = 1.0f;
  std::string textures[4];
};
rmn_status read_fbx(const std::string& path, std::vector<FbxMesh>& meshes, std::vector<FbxMaterial>& materials);

// The whole file, read at its size (image_io.cpp); false if it cannot be
// opened or read.
bool read_whole_file(const char* path, std::vector<uint8_t>& out);
bool read_whole_file(const char* path, std::string& out);

// fn(0) .. fn(n - 1), each on its own thread (fn(0) on the caller's). Every
// thread started is joined, also when starting another fails; the first
// exception of any of them is rethrown here.
template <class F>
void run_threads(size_t n, F fn) {
  std::vector<std::exception_ptr> err(n);
  auto guarded = [&](size_t k) {
    try {
      fn(k);
    } catch (...) {
      err[k] = std::current_exception();
    }
  };
  std::vector<std::thread> pool;
  std::exception_ptr start_err;
  try {
    for (size_t k = 1; k < n; ++k) pool.emplace_back(guarded, k);
  } catch (...) {
    start_err = std::current_exception();
  }
  if (!start_err && n > 0) guarded(0);
  for (std::thread& th : pool) th.join();
  if (start_err) std::rethrow_exception(start_err);
  for (const std::exception_ptr& e : err)
    if (e) std::rethrow_exception(e);
}
// Worker threads for host-side parallel work: the hardware threads, 1..16.
inline size_t host_threads() {
  const unsigned hw = std::thread::hardware_concurrency();
  return hw < 1 ? 1 : hw > 16 ? 16 : hw;
}

// A zlib stream of n bytes (image_io.cpp): LZ77 + dynamic Huffman blocks.
std::vector<uint8_t> zlib_compress(const uint8_t* data, size_t n);
// Inflates a zlib stream of n bytes that must hold exactly `want` bytes
// (image_io.cpp); nullptr, or what is wrong with the stream.
const char* zlib_inflate(const uint8_t* p, size_t n, std::vector<uint8_t>& out, size_t want);

// CRC-32 of PNG chunks (ISO 3309 polynomial), shared by the writer and the reader.
uint32_t png_crc32(uint32_t crc, const uint8_t* p, size_t n);

// Device memory kept for reuse between batches (devmem.cpp).
cudaError_t cached_malloc(void** p, size_t bytes);
void cached_free(void* p);
void release_cached_memory();
// A stream-ordered allocation from the library's staging pool (devmem.cpp),
// freed with cudaFreeAsync.
cudaError_t staging_malloc(void** p, size_t bytes, cudaStream_t st);
// Forgets the device addresses rmn_compose_noalloc resolved (after a device
// reset they name nothing); the next call on each device resolves them anew.
void noalloc_forget_addresses();

// stack_entries: the traversal kernels' deferred-child stack, RMN_STACK_SMALL
// or RMN_STACK entries (0: the smallest that holds every item's tree).
// ray_order: 1 bins each ray queue by origin cell and direction octant
// before it is traced, 0 traces the queues in the order they were filled.
rmn_status batch_create(const RenderItem* items, int n, bool use_graph, int pool_workers, int lanes,
                        int stack_entries, int ray_order, cudaStream_t st, BatchState** out);
// The traversal stack the library picks for these items (RMN_STACK_SMALL when
// every tree is at most RMN_STACK_SMALL - 1 deep, else RMN_STACK).
int default_stack_entries(const RenderItem* items, int n);
// Workers per lane when a batch leaves the pool size open (fewer when device
// memory is short).
constexpr int kDefaultPoolWorkers = 1 << 22;
rmn_status batch_launch(BatchState* b, cudaStream_t st);
rmn_status batch_update(BatchState* b, const rmn_render_args* args, int n, cudaStream_t st);
size_t batch_job_bytes();
size_t batch_device_bytes(const RenderItem* items, int n, int pool_workers, int lanes, int ray_order = 0);
void default_slots_per_unit(const RenderItem* items, int n, int* S);
int batch_items(const BatchState* b);
rmn_status batch_status(BatchState* b, cudaStream_t st);
rmn_status batch_profile(BatchState* b, cudaStream_t st, RenderProfileData* prof);
void batch_destroy(BatchState* b);

// Adjoint of one render (adjoint.cu): device buffers only; dmat receives
// num_materials * RMN_GRAD_PER_MATERIAL floats.
rmn_status launch_adjoint(const rmn_scene* scene, const rmn_render_args& args, const float* gbuf, const int* dropped,
                          const float* dimg, float* dmat, cudaStream_t st);
cudaError_t launch_fxaa(const float* in, float* out, int w, int h, cudaStream_t stream);
// Post passes (photo.cu); bufs = Dd, Ds, Id, Is (4 floats per pixel).
cudaError_t launch_spatial_clamp(float* const bufs[4], int w, int h, cudaStream_t st);
cudaError_t launch_filter(float* const bufs[4], const float* gbuf, int w, int h, cudaStream_t st);
cudaError_t launch_bloom(float* rgb, int w, int h, cudaStream_t st);
cudaError_t launch_dof(float* rgb, const float* gbuf, int w, int h, float focus, float coc, const float cam[3],
                       cudaStream_t st);
// A depth-of-field plan serves every blur of the same G-buffer and camera.
struct DofPlan;
cudaError_t dof_plan_create(const float* gbuf, int w, int h, float focus, float coc, const float cam[3],
                            cudaStream_t st, DofPlan** out);
cudaError_t dof_apply(const DofPlan* plan, float* rgb, cudaStream_t st);
void dof_plan_destroy(DofPlan* plan, cudaStream_t st);
cudaError_t launch_gamma(float* rgb, int n, cudaStream_t st);
cudaError_t launch_compose(const float* dd, const float* ds, const float* id, const float* is, const float* gbuf,
                           int w, int h, float exposure, int options, float* rgb, cudaStream_t stream);

}  // namespace rmn
