// api.cpp — implementation of the C ABI declared in include/rtx.h.
//
// Host code here is compiled with -ffp-contract=off: the per-triangle data it
// derives (edges, flat normal, area: RenderToy Triangle::UpdateCache,
// src/object.cpp:224-243), the camera's film extents
// (Renderer::PrepareScreenSpace, src/renderer.cpp:103-124) and the Gaussian
// weights (UnitizedGaussianKernel, include/RenderToy/rtmath.h:1019-1059) are
// computed in the reference's operation order, so they equal the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <thread>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "nn.h"
#include "nn_ops.h"
#include "nn_unet.h"
#include "host_threads.h"
#include "rtx_internal.h"

using namespace rtx;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max(bytes, (size_t)256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

struct V3 {
  float x, y, z;
};
inline V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float dot(V3 a, V3 b) {
  float r = 0.0f;
  r += a.x * b.x;
  r += a.y * b.y;
  r += a.z * b.z;
  return r;
}
inline V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 normalized(V3 a) {
  float l = std::sqrt(dot(a, a));
  return V3{a.x / l, a.y / l, a.z / l};
}

}  // namespace

struct rtx_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  // options
  bool async = false;
  int64_t wave_paths = 0;
  int block = 128;
  int sort_material = 2;  // 0 off, 1 on, 2 on for scenes with refraction or 8+ materials
  int sort_rays = 2;  // 0 off, 1 on, 2 on for scenes of kSortRaysMinTris triangles or more
  bool count_visits = false;
  int leaf_size = 4;
  bool primary_cache = true;
  bool accumulate = false;
  int traversal = 2;
  int min_busy = 20;
  int stack_limit = kStackSize;
  bool compositor_fma = false;
  bool overlap = true;
  KernelTimer timer;
  // scene
  bool has_scene = false;
  DeviceScene ds{};
  DevBuf nodes, nodes4, tris, shade, geo, mats, emit;
  std::vector<int32_t> emitters;
  // device scratch
  int* d_err = nullptr;
  Counters* d_counters = nullptr;
  PtWorkspace* pt = nullptr;
  DevBuf stage[8];
  DevBuf perm;  // Perlin texture permutation (256 bytes)
  // multi-scene batch (rtx_batch_upload / rtx_render_batch)
  struct BatchScene {
    int root, root4, e_begin, n_emitters, n_tris;
    float sky[3], ground[3];
    SortKeyBounds keyb;
  };
  bool has_batch = false;
  DeviceScene bds{};
  DevBuf b_nodes, b_nodes4, b_tris, b_shade, b_geo, b_mats, b_emit, b_jobs, b_jobq;
  std::vector<BatchScene> bscenes;
  // CUDA graph of the last batch frame, keyed by its launch shape
  bool use_graph = false;
  cudaGraphExec_t graph = nullptr;
  std::vector<int64_t> graph_key;
  PtJob* h_jobs_pinned = nullptr;
  long long* h_jobq_pinned = nullptr;
  int pinned_cap = 0;
  rtx::nn::UNet* dn = nullptr;
  DevBuf weights;
  std::vector<float> host_weights;  // what `weights` holds when weights_valid
  bool weights_valid = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  rtx_stats stats{};
  bool pending_timing = false;
};

namespace {

int fail(rtx_context* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(rtx_context* c, cudaError_t e, const char* where) {
  return fail(c, e == cudaErrorMemoryAllocation ? RTX_ERR_NOMEM : RTX_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

#define RTX_CUDA(call, where)                         \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, where); \
  } while (0)

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Begin a call: select the device, clear the error word, start the timer.
// Ray sorting pays for its sort launches once a scene's tree no longer sits
// in L1: measured at 256^2 x 16 spp, depth 8, it is 2-12 % slower below
// ~1,300 triangles (the 36-triangle Cornell box: 1.12 -> 1.28 ms per
// frame), 1-2 % faster from ~5,000 and 8-9 % faster at 20,000.
constexpr int kSortRaysMinTris = 4096;
// Material-sorted shading pays where a warp's paths would otherwise run
// different lobes: measured on the 9-material room with glass, metal,
// clearcoat and subsurface (512^2 x 16 spp) 9.43 -> 6.37 ms per frame, on the
// 1.3M-triangle icosphere room (5 materials, no refraction) 105.8 -> 116.4 ms.
static bool sort_material_for(const rtx_context* c, const DeviceScene& s) {
  return c->sort_material == 2 ? ((s.lobes & kLobeTrans) != 0 || s.n_mats >= 8) : c->sort_material != 0;
}
static bool sort_rays_for(const rtx_context* c, int n_tris) {
  return c->sort_rays == 2 ? n_tris >= kSortRaysMinTris : c->sort_rays != 0;
}

// The ray sort's origin grids over a scene's bounds: the union of its 4-wide
// root's children (empty slots hold planes at 1e30 and are skipped), as the
// device-side key of the sort's histogram pass computes it.
static SortKeyBounds sort_key_bounds(const Float4Array& nodes4, int root4) {
  SortKeyBounds kb;
  if (root4 < 0 || nodes4.size() < (size_t)kNode4Vecs * (root4 + 1)) return kb;
  const float4* n = &nodes4[(size_t)kNode4Vecs * root4];
  const float big = 1e29f;
  auto lo4 = [](float4 v) { return std::min(std::min(v.x, v.y), std::min(v.z, v.w)); };
  auto hi4 = [&](float4 v) {
    auto f = [&](float x) { return x < big ? x : -big; };
    return std::max(std::max(f(v.x), f(v.y)), std::max(f(v.z), f(v.w)));
  };
  const float lo[3] = {lo4(n[0]), lo4(n[2]), lo4(n[4])}, hi[3] = {hi4(n[1]), hi4(n[3]), hi4(n[5])};
  for (int k = 0; k < 3; ++k) {
    const float ext = std::max(hi[k] - lo[k], 1e-20f);
    kb.lo[k] = lo[k];
    kb.inv4[k] = 4.0f / ext;
    kb.inv16[k] = 16.0f / ext;
  }
  kb.ok = 1;
  return kb;
}

int begin(rtx_context* c) {
  RTX_CUDA(cudaSetDevice(c->device), "cudaSetDevice");
  RTX_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream), "cudaMemsetAsync(err)");
  RTX_CUDA(cudaEventRecord(c->ev0, c->stream), "cudaEventRecord");
  c->stats.kernel_launches = 0;
  return RTX_OK;
}

// End a call: stop the timer; synchronise unless the call may stay async.
int finish(rtx_context* c, bool may_async) {
  RTX_CUDA(cudaEventRecord(c->ev1, c->stream), "cudaEventRecord");
  if (may_async && c->async) {
    c->pending_timing = true;
    return RTX_OK;
  }
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  float ms = 0.0f;
  RTX_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "cudaEventElapsedTime");
  c->stats.last_gpu_ms = ms;
  c->pending_timing = false;
  int herr = 0;
  RTX_CUDA(cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost), "read error word");
  if (herr) {
    std::string m = "kernel error:";
    if (herr & kErrStackOverflow) m += " traversal stack overflow";
    if (herr & kErrQueueOverflow) m += " queue overflow";
    if (herr & kErrBadIndex) m += " index out of range";
    if (herr & 8) m += " tensor-core barrier wait timed out";
    return fail(c, RTX_ERR_DEVICE, m);
  }
  return RTX_OK;
}

// A caller buffer of `bytes`: device pointers are used in place, host
// pointers are staged through stage[slot].
struct Arg {
  void* dev = nullptr;
  void* host = nullptr;
  size_t bytes = 0;
};

int bind_in(rtx_context* c, const void* p, size_t bytes, int slot, Arg& a) {
  a.bytes = bytes;
  if (!p || bytes == 0) return RTX_OK;
  if (is_device_ptr(p)) {
    a.dev = const_cast<void*>(p);
    return RTX_OK;
  }
  RTX_CUDA(c->stage[slot].ensure(bytes), "stage alloc");
  a.dev = c->stage[slot].p;
  RTX_CUDA(cudaMemcpyAsync(a.dev, p, bytes, cudaMemcpyHostToDevice, c->stream), "H2D");
  return RTX_OK;
}

int bind_out(rtx_context* c, void* p, size_t bytes, int slot, Arg& a) {
  a.bytes = bytes;
  if (!p || bytes == 0) return RTX_OK;
  if (is_device_ptr(p)) {
    a.dev = p;
    return RTX_OK;
  }
  RTX_CUDA(c->stage[slot].ensure(bytes), "stage alloc");
  a.dev = c->stage[slot].p;
  a.host = p;
  return RTX_OK;
}

int copy_back(rtx_context* c, const Arg& a) {
  if (a.host)
    RTX_CUDA(cudaMemcpyAsync(a.host, a.dev, a.bytes, cudaMemcpyDeviceToHost, c->stream), "D2H");
  return RTX_OK;
}

bool all_device(std::initializer_list<const Arg*> args) {
  for (const Arg* a : args)
    if (a->host) return false;
  return true;
}

int check_cam(rtx_context* c, const float* cam, int W, int H) {
  if (!cam) return fail(c, RTX_ERR_INVALID, "camera is NULL");
  if (W <= 0 || H <= 0) return fail(c, RTX_ERR_INVALID, "image size must be positive");
  if ((long long)W * H > (1LL << 30)) return fail(c, RTX_ERR_INVALID, "image too large");
  if (!c->has_scene) return fail(c, RTX_ERR_NO_SCENE, "no scene uploaded");
  return RTX_OK;
}

// UnitizedGaussianKernel<float, X> weights (rtmath.h:1019-1059)
void gaussian_weights(int size, float sigma, float* w) {
  float orig = float(size >> 1);
  float sum = 0.0f;
  for (int j = 0; j < size; ++j) {
    float x2 = std::pow(float(j) - orig, 2.0f);
    float g = std::exp(-(x2) / (2.0f * sigma * sigma));
    sum += g;
    w[j] = g;
  }
  for (int j = 0; j < size; ++j) w[j] /= sum;
}

// Filter weights to the device.  The device copy is kept while the weights
// do not change: a frame loop applies the same filters every frame.
int upload_weights(rtx_context* c, const float* w, size_t n) {
  if (c->weights_valid && c->host_weights.size() == n &&
      std::memcmp(c->host_weights.data(), w, n * sizeof(float)) == 0)
    return RTX_OK;
  c->weights_valid = false;
  c->host_weights.assign(w, w + n);
  RTX_CUDA(c->weights.ensure(n * sizeof(float)), "weights alloc");
  RTX_CUDA(cudaMemcpyAsync(c->weights.p, c->host_weights.data(), n * sizeof(float),
                           cudaMemcpyHostToDevice, c->stream),
           "weights H2D");
  c->weights_valid = true;
  return RTX_OK;
}

// The default permutation of the Perlin texture: a Fisher-Yates shuffle of
// 0..255 driven by splitmix64 from 0 (siv::PerlinNoise's own default table is
// not reproduced; rtx_scene_set_texture_table installs any table).
void default_texture_table(uint8_t* p) {
  for (int i = 0; i < 256; ++i) p[i] = (uint8_t)i;
  uint64_t x = 0;
  for (int i = 255; i > 0; --i) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    int j = (int)(z % (uint64_t)(i + 1));
    uint8_t t = p[i];
    p[i] = p[j];
    p[j] = t;
  }
}

}  // namespace

namespace rtx {
// Renderer::PrepareScreenSpace (renderer.cpp:103-124); InchToMM multiplies by
// float(25.4) (rtmath.h:1098-1103)
CamParams make_cam_params(const float* cam, int W, int H) {
  CamParams k;
  for (int i = 0; i < 12; ++i) k.m[i] = cam[i];
  float focal = cam[16], gx = cam[17], gy = cam[18];
  k.top = ((gy * 25.4f) / 2.0f) / focal;
  k.right = ((gx * 25.4f) / 2.0f) / focal;
  float gate_aspr = gx / gy;
  float film_aspr = float(W) / float(H);
  float xscale = 1.0f, yscale = 1.0f;
  if (gate_aspr >= film_aspr)
    xscale = film_aspr / gate_aspr;
  else
    yscale = gate_aspr / film_aspr;
  k.right *= xscale;
  k.top *= yscale;
  k.inv_w = 1.0f / float(W);
  k.inv_h = 1.0f / float(H);
  k.W = W;
  k.H = H;
  return k;
}
}  // namespace rtx

extern "C" {

int rtx_version(void) { return RTX_VERSION; }

int rtx_create(rtx_context** out, int device) {
  if (!out) return RTX_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return RTX_ERR_CUDA;
  }
  if (device < 0 || device >= n) return RTX_ERR_INVALID;
  rtx_context* c = new (std::nothrow) rtx_context();
  if (!c) return RTX_ERR_NOMEM;
  c->device = device;
  auto bail = [&](cudaError_t e) {
    cuda_fail(c, e, "rtx_create");
    rtx_destroy(c);
    return e == cudaErrorMemoryAllocation ? RTX_ERR_NOMEM : RTX_ERR_CUDA;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(device)) != cudaSuccess) return bail(e);
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
  c->own_stream = true;
  if ((e = cudaEventCreate(&c->ev0)) != cudaSuccess) return bail(e);
  if ((e = cudaEventCreate(&c->ev1)) != cudaSuccess) return bail(e);
  if ((e = cudaMalloc(&c->d_err, sizeof(int))) != cudaSuccess) return bail(e);
  if ((e = cudaMalloc(&c->d_counters, sizeof(Counters))) != cudaSuccess) return bail(e);
  if ((e = cudaMemset(c->d_counters, 0, sizeof(Counters))) != cudaSuccess) return bail(e);
  {
    uint8_t tbl[256];
    default_texture_table(tbl);
    if ((e = c->perm.ensure(256)) != cudaSuccess) return bail(e);
    if ((e = cudaMemcpy(c->perm.p, tbl, 256, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e);
    c->ds.perm = (const uint8_t*)c->perm.p;
  }
  c->pt = pt_workspace_create();
  *out = c;
  return RTX_OK;
}

void rtx_destroy(rtx_context* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->nodes.release();
  c->nodes4.release();
  c->tris.release();
  c->shade.release();
  c->geo.release();
  c->mats.release();
  c->emit.release();
  for (auto& s : c->stage) s.release();
  c->perm.release();
  DevBuf* bb[] = {&c->b_nodes, &c->b_nodes4, &c->b_tris, &c->b_shade, &c->b_geo, &c->b_mats, &c->b_emit,
                  &c->b_jobs, &c->b_jobq};
  for (DevBuf* b : bb) b->release();
  if (c->graph) cudaGraphExecDestroy(c->graph);
  if (c->h_jobs_pinned) cudaFreeHost(c->h_jobs_pinned);
  if (c->h_jobq_pinned) cudaFreeHost(c->h_jobq_pinned);
  delete c->dn;
  c->weights.release();
  c->weights_valid = false;
  if (c->pt) pt_workspace_destroy(c->pt);
  if (c->d_err) cudaFree(c->d_err);
  if (c->d_counters) cudaFree(c->d_counters);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* rtx_last_error(const rtx_context* c) { return c ? c->err.c_str() : "null context"; }

int rtx_set_option(rtx_context* c, int option, int64_t v) {
  if (!c) return RTX_ERR_INVALID;
  switch (option) {
    case RTX_OPT_ASYNC: c->async = v != 0; return RTX_OK;
    case RTX_OPT_GRAPH: c->use_graph = v != 0; return RTX_OK;
    case RTX_OPT_WAVE_PATHS:
      if (v < 0 || v > (1LL << 30)) return fail(c, RTX_ERR_INVALID, "wave paths out of range");
      c->wave_paths = v;
      return RTX_OK;
    case RTX_OPT_BLOCK:
      if (v != 64 && v != 128) return fail(c, RTX_ERR_INVALID, "block must be 64 or 128");
      c->block = (int)v;
      return RTX_OK;
    case RTX_OPT_SORT_MATERIAL: c->sort_material = v == 2 ? 2 : (v != 0); return RTX_OK;
    case RTX_OPT_SORT_RAYS: c->sort_rays = v == 2 ? 2 : (v != 0); return RTX_OK;
    case RTX_OPT_COUNT_VISITS: c->count_visits = v != 0; return RTX_OK;
    case RTX_OPT_LEAF_SIZE:
      if (v < 1 || v > kMaxLeaf) return fail(c, RTX_ERR_INVALID, "leaf size must be in [1, 8]");
      c->leaf_size = (int)v;
      return RTX_OK;
    case RTX_OPT_PRIMARY_CACHE: c->primary_cache = v != 0; return RTX_OK;
    case RTX_OPT_KERNEL_TIMING: c->timer.on = v != 0; return RTX_OK;
    case RTX_OPT_ACCUMULATE: c->accumulate = v != 0; return RTX_OK;
    case RTX_OPT_TRAVERSAL:
      if (v < 0 || v > 2) return fail(c, RTX_ERR_INVALID, "traversal must be 0, 1 or 2");
      c->traversal = (int)v;
      return RTX_OK;
    case RTX_OPT_MIN_BUSY:
      if (v < 0 || v > 32) return fail(c, RTX_ERR_INVALID, "min busy lanes must be in [0, 32]");
      c->min_busy = (int)v;
      return RTX_OK;
    case RTX_OPT_COMPOSITOR_FMA: c->compositor_fma = v != 0; return RTX_OK;
    case RTX_OPT_OVERLAP: c->overlap = v != 0; return RTX_OK;
    case RTX_OPT_STACK_LIMIT:
      if (v < 2 || v > kStackSize) return fail(c, RTX_ERR_INVALID, "stack limit must be in [2, 64]");
      c->stack_limit = (int)v;
      c->ds.stack_limit = c->stack_limit;
      c->bds.stack_limit = c->stack_limit;
      return RTX_OK;
  }
  return fail(c, RTX_ERR_INVALID, "unknown option");
}

int rtx_get_option(rtx_context* c, int option, int64_t* v) {
  if (!c || !v) return RTX_ERR_INVALID;
  switch (option) {
    case RTX_OPT_ASYNC: *v = c->async; return RTX_OK;
    case RTX_OPT_GRAPH: *v = c->use_graph; return RTX_OK;
    case RTX_OPT_WAVE_PATHS: *v = c->wave_paths; return RTX_OK;
    case RTX_OPT_BLOCK: *v = c->block; return RTX_OK;
    case RTX_OPT_SORT_MATERIAL: *v = c->sort_material; return RTX_OK;
    case RTX_OPT_SORT_RAYS: *v = c->sort_rays; return RTX_OK;
    case RTX_OPT_COUNT_VISITS: *v = c->count_visits; return RTX_OK;
    case RTX_OPT_LEAF_SIZE: *v = c->leaf_size; return RTX_OK;
    case RTX_OPT_PRIMARY_CACHE: *v = c->primary_cache; return RTX_OK;
    case RTX_OPT_KERNEL_TIMING: *v = c->timer.on; return RTX_OK;
    case RTX_OPT_ACCUMULATE: *v = c->accumulate; return RTX_OK;
    case RTX_OPT_TRAVERSAL: *v = c->traversal; return RTX_OK;
    case RTX_OPT_MIN_BUSY: *v = c->min_busy; return RTX_OK;
    case RTX_OPT_STACK_LIMIT: *v = c->stack_limit; return RTX_OK;
    case RTX_OPT_COMPOSITOR_FMA: *v = c->compositor_fma; return RTX_OK;
    case RTX_OPT_OVERLAP: *v = c->overlap; return RTX_OK;
  }
  return fail(c, RTX_ERR_INVALID, "unknown option");
}

void* rtx_get_stream(rtx_context* c) { return c ? (void*)c->stream : nullptr; }

int rtx_set_stream(rtx_context* c, void* stream) {
  if (!c) return RTX_ERR_INVALID;
  RTX_CUDA(cudaSetDevice(c->device), "cudaSetDevice");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  if (c->own_stream) cudaStreamDestroy(c->stream);
  c->stream = (cudaStream_t)stream;
  c->own_stream = false;
  return RTX_OK;
}

int rtx_synchronize(rtx_context* c) {
  if (!c) return RTX_ERR_INVALID;
  RTX_CUDA(cudaSetDevice(c->device), "cudaSetDevice");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  if (c->pending_timing) {
    float ms = 0.0f;
    RTX_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "cudaEventElapsedTime");
    c->stats.last_gpu_ms = ms;
    c->pending_timing = false;
  }
  int herr = 0;
  RTX_CUDA(cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost), "read error word");
  if (herr) return fail(c, RTX_ERR_DEVICE, "kernel error reported by an asynchronous call");
  return RTX_OK;
}

int rtx_get_stats(rtx_context* c, rtx_stats* out) {
  if (!c || !out) return RTX_ERR_INVALID;
  int r = rtx_synchronize(c);
  if (r) return r;
  Counters h;
  RTX_CUDA(cudaMemcpy(&h, c->d_counters, sizeof(Counters), cudaMemcpyDeviceToHost), "read counters");
  c->stats.extension_rays = h.ext_rays;
  c->stats.shadow_rays = h.shadow_rays;
  c->stats.ext_node_visits = h.ext_node_visits;
  c->stats.ext_tri_tests = h.ext_tri_tests;
  c->stats.shadow_node_visits = h.sh_node_visits;
  c->stats.shadow_tri_tests = h.sh_tri_tests;
  for (int d = 0; d < 16; ++d) c->stats.ext_rays_by_depth[d] = h.ext_rays_by_depth[d];
  // node visits count records of the tree in use: 4 x 16 B binary, 7 x 16 B 4-wide
  c->stats.node_bytes = c->traversal == 2 ? 112 : 64;  // bytes a node visit reads
  RTX_CUDA(c->timer.collect(), "kernel timing");
  c->stats.extend_ms = c->timer.ms[0];
  c->stats.shade_ms = c->timer.ms[1];
  c->stats.connect_ms = c->timer.ms[2];
  *out = c->stats;
  return RTX_OK;
}

}  // extern "C"

namespace {

// One scene prepared on the host: BVH, per-triangle shading and geometry
// records, materials and the emitter list.
struct HostScene {
  BvhBuildResult b;
  Float4Array shade, geo;  // every element written by build_host_scene
  std::vector<float> mats;
  std::vector<int32_t> emitters;
  int n_tris = 0, n_mats = 0;
  float sky[3], ground[3];
};

int check_scene(rtx_context* c, int n, const float* verts, const float* norms, const int32_t* tri_mesh,
                int n_meshes, const int32_t* mesh_mat, const uint8_t* mesh_smooth, int n_mat, const float* mats,
                const float* sky, const float* ground) {
  if (n < 0 || n_meshes < 0 || n_mat < 0) return fail(c, RTX_ERR_INVALID, "negative count");
  if (n > (1 << 27)) return fail(c, RTX_ERR_INVALID, "more than 2^27 triangles");
  if (n > 0 && (!verts || !tri_mesh)) return fail(c, RTX_ERR_INVALID, "verts / tri_mesh is NULL");
  if (n_meshes > 0 && (!mesh_mat || !mesh_smooth)) return fail(c, RTX_ERR_INVALID, "mesh arrays are NULL");
  if (n_mat > 0 && !mats) return fail(c, RTX_ERR_INVALID, "materials is NULL");
  if (!sky || !ground) return fail(c, RTX_ERR_INVALID, "sky / ground is NULL");
  for (int m = 0; m < n_meshes; ++m)
    if (mesh_mat[m] < 0 || mesh_mat[m] >= n_mat) return fail(c, RTX_ERR_INVALID, "mesh material index out of range");
  for (int m = 0; m < n_mat; ++m) {
    float k = mats[RTX_MATERIAL_FLOATS * (size_t)m + 21];
    if (!(k == 0.0f || k == 1.0f || k == 2.0f || k == 3.0f))
      return fail(c, RTX_ERR_INVALID, "material texture kind must be 0, 1, 2 or 3");
    float prm = mats[RTX_MATERIAL_FLOATS * (size_t)m + 22];
    if (k == 1.0f && !(std::fabs(prm) < 1e6f))
      return fail(c, RTX_ERR_INVALID, "checkerboard scale out of range");
  }
  bool any_smooth = false;
  for (int m = 0; m < n_meshes; ++m) any_smooth |= mesh_smooth[m] != 0;
  if (any_smooth && !norms) return fail(c, RTX_ERR_INVALID, "a smooth mesh needs vertex normals");
  for (int i = 0; i < n; ++i)
    if (tri_mesh[i] < 0 || tri_mesh[i] >= n_meshes) return fail(c, RTX_ERR_INVALID, "triangle mesh index out of range");
  return RTX_OK;
}

void build_host_scene(HostScene& h, int n, const float* verts, const float* norms, const int32_t* tri_mesh,
                      int n_meshes, const int32_t* mesh_mat, const uint8_t* mesh_smooth, int n_mat,
                      const float* mats, const float* sky, const float* ground, int leaf_size) {
  // per-triangle work in chunks on host threads (each triangle's records
  // are its own, so any split gives the same arrays)
  unsigned nt = n >= (1 << 16) ? std::max(1u, std::min(std::thread::hardware_concurrency(), 64u)) : 1u;
  size_t chunks = std::max<size_t>(1, std::min<size_t>(nt, (size_t)n >> 15));
  auto chunk_range = [&](size_t k, int& b, int& e) {
    b = (int)((int64_t)n * (int64_t)k / (int64_t)chunks);
    e = (int)((int64_t)n * (int64_t)(k + 1) / (int64_t)chunks);
  };
  // Mesh's identity object-to-world turns -0.0 into +0.0 (object.cpp:42-48)
  std::vector<float> v((size_t)n * 9);
  run_parallel(chunks, nt, [&](size_t k) {
    int b, e;
    chunk_range(k, b, e);
    for (size_t i = 9 * (size_t)b; i < 9 * (size_t)e; ++i) v[i] = verts[i] + 0.0f;
  });
  h.b = build_bvh(v.data(), n, leaf_size);
  h.shade.resize((size_t)n * 4);
  h.geo.resize((size_t)n * 3);
  run_parallel(chunks, nt, [&](size_t k) {
    int b, e;
    chunk_range(k, b, e);
    for (int i = b; i < e; ++i) {
      const float* p = &v[9 * (size_t)i];
      V3 v0{p[0], p[1], p[2]}, v1{p[3], p[4], p[5]}, v2{p[6], p[7], p[8]};
      V3 e1 = sub(v1, v0), e2 = sub(v2, v0);
      V3 cr = cross(e1, e2);
      float area = std::sqrt(dot(cr, cr)) * 0.5f;                 // Triangle::Area
      V3 nrm = normalized(cross(normalized(e1), sub(v2, v1)));  // Triangle::Normal
      int mesh = tri_mesh[i];
      uint32_t info = (uint32_t)mesh_mat[mesh] | (mesh_smooth[mesh] ? 0x80000000u : 0u);
      float infof;
      std::memcpy(&infof, &info, 4);
      const float* q = norms ? norms + 9 * (size_t)i : nullptr;
      h.shade[4 * (size_t)i] = make_float4(nrm.x, nrm.y, nrm.z, area);
      h.shade[4 * (size_t)i + 1] = make_float4(q ? q[0] : 0.f, q ? q[1] : 0.f, q ? q[2] : 0.f, infof);
      h.shade[4 * (size_t)i + 2] = make_float4(q ? q[3] : 0.f, q ? q[4] : 0.f, q ? q[5] : 0.f, 0.f);
      h.shade[4 * (size_t)i + 3] = make_float4(q ? q[6] : 0.f, q ? q[7] : 0.f, q ? q[8] : 0.f, 0.f);
      h.geo[3 * (size_t)i] = make_float4(v0.x, v0.y, v0.z, 0.f);
      h.geo[3 * (size_t)i + 1] = make_float4(e1.x, e1.y, e1.z, 0.f);
      h.geo[3 * (size_t)i + 2] = make_float4(e2.x, e2.y, e2.z, 0.f);
    }
  });
  // World::PrepareDirectLightSampling (world.cpp:24-37): the emissive meshes
  // in order, each one's triangles in id order
  std::vector<uint8_t> emissive(n_meshes);
  for (int m = 0; m < n_meshes; ++m) {
    const float* em = mats + RTX_MATERIAL_FLOATS * (size_t)mesh_mat[m] + 3;
    emissive[m] = std::fabs(em[0]) > 1e-7f || std::fabs(em[1]) > 1e-7f || std::fabs(em[2]) > 1e-7f;
  }
  std::vector<std::vector<int>> per_mesh(n_meshes);
  for (int i = 0; i < n; ++i)
    if (emissive[tri_mesh[i]]) per_mesh[tri_mesh[i]].push_back(i);
  h.emitters.clear();
  for (int m = 0; m < n_meshes; ++m) h.emitters.insert(h.emitters.end(), per_mesh[m].begin(), per_mesh[m].end());
  h.mats.assign(mats, mats + (size_t)n_mat * RTX_MATERIAL_FLOATS);
  h.n_tris = n;
  h.n_mats = n_mat;
  for (int k = 0; k < 3; ++k) {
    h.sky[k] = sky[k];
    h.ground[k] = ground[k];
  }
}

int upload_buf(rtx_context* c, DevBuf& d, const void* src, size_t bytes, const char* what) {
  RTX_CUDA(d.ensure(bytes), what);
  if (bytes) RTX_CUDA(cudaMemcpy(d.p, src, bytes, cudaMemcpyHostToDevice), what);
  return RTX_OK;
}

// leaf reference of the binary tree, rebased by `tri_base` leaf-order records
int rebase_leaf(int ref, int tri_base) {
  int r = ~ref;
  int first = r >> 3, cnt = r & 7;
  return ~(((first + tri_base) << 3) | cnt);
}

// Runs an entry point's host work and turns an exception (a host allocation
// that failed, in the scene builders) into an error code: no exception
// crosses the C ABI.
template <class F>
int host_guard(rtx_context* c, F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    return c ? fail(c, RTX_ERR_NOMEM, "host allocation failed") : RTX_ERR_NOMEM;
  } catch (const std::exception& e) {
    return c ? fail(c, RTX_ERR_INVALID, e.what()) : RTX_ERR_INVALID;
  }
}

}  // namespace

extern "C" {

static int scene_upload(rtx_context* c, int n, const float* verts, const float* norms,
                        const int32_t* tri_mesh, int n_meshes, const int32_t* mesh_mat,
                        const uint8_t* mesh_smooth, int n_mat, const float* mats, const float* sky,
                        const float* ground) {
  if (!c) return RTX_ERR_INVALID;
  int r;
  if ((r = check_scene(c, n, verts, norms, tri_mesh, n_meshes, mesh_mat, mesh_smooth, n_mat, mats, sky, ground)))
    return r;
  RTX_CUDA(cudaSetDevice(c->device), "cudaSetDevice");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  HostScene h;
  build_host_scene(h, n, verts, norms, tri_mesh, n_meshes, mesh_mat, mesh_smooth, n_mat, mats, sky, ground,
                   c->leaf_size);
  const BvhBuildResult& b = h.b;
  c->emitters = h.emitters;
  if ((r = upload_buf(c, c->nodes, b.nodes.data(), b.nodes.size() * sizeof(float4), "upload nodes"))) return r;
  if ((r = upload_buf(c, c->nodes4, b.nodes4.data(), b.nodes4.size() * sizeof(float4), "upload nodes4"))) return r;
  if ((r = upload_buf(c, c->tris, b.tris.data(), b.tris.size() * sizeof(float4), "upload tris"))) return r;
  if ((r = upload_buf(c, c->shade, h.shade.data(), h.shade.size() * sizeof(float4), "upload shade"))) return r;
  if ((r = upload_buf(c, c->geo, h.geo.data(), h.geo.size() * sizeof(float4), "upload geo"))) return r;
  if ((r = upload_buf(c, c->mats, h.mats.data(), h.mats.size() * sizeof(float), "upload mats"))) return r;
  if ((r = upload_buf(c, c->emit, c->emitters.data(), c->emitters.size() * sizeof(int32_t), "upload emitters")))
    return r;

  DeviceScene& s = c->ds;
  s.nodes = (const float4*)c->nodes.p;
  s.nodes4 = (const float4*)c->nodes4.p;
  s.root4 = b.root4;
  s.tris = (const float4*)c->tris.p;
  s.shade = (const float4*)c->shade.p;
  s.geo = (const float4*)c->geo.p;
  s.mats = (const float*)c->mats.p;
  s.emitters = (const int*)c->emit.p;
  s.perm = (const uint8_t*)c->perm.p;
  s.root = b.root;
  s.n_tris = n;
  s.n_emitters = (int)c->emitters.size();
  s.n_mats = n_mat;
  s.textured = 0;
  for (int m = 0; m < n_mat; ++m) s.textured |= mats[RTX_MATERIAL_FLOATS * (size_t)m + 21] != 0.0f;
  s.lobes = material_lobes(mats, n_mat);
  for (int k = 0; k < 3; ++k) {
    s.sky[k] = sky[k];
    s.ground[k] = ground[k];
  }
  s.stack_limit = c->stack_limit;
  s.keyb = sort_key_bounds(b.nodes4, b.root4);
  c->has_scene = true;
  c->stats.bvh_build_ms = b.ms;
  c->stats.bvh_nodes = b.n_nodes;
  c->stats.bvh_leaves = b.n_leaves;
  c->stats.bvh_depth = b.depth;
  c->stats.node_bytes = 64;
  c->stats.tri_bytes = 48;
  return RTX_OK;
}

int rtx_scene_upload(rtx_context* c, int n, const float* verts, const float* norms,
                     const int32_t* tri_mesh, int n_meshes, const int32_t* mesh_mat,
                     const uint8_t* mesh_smooth, int n_mat, const float* mats, const float* sky,
                     const float* ground) {
  return host_guard(c, [&] {
    return scene_upload(c, n, verts, norms, tri_mesh, n_meshes, mesh_mat, mesh_smooth, n_mat, mats, sky, ground);
  });
}

static int batch_upload(rtx_context* c, int n_scenes, const rtx_scene_desc* d) {
  if (!c) return RTX_ERR_INVALID;
  if (n_scenes < 1 || !d) return fail(c, RTX_ERR_INVALID, "at least one scene is needed");
  int r;
  for (int i = 0; i < n_scenes; ++i) {
    if ((r = check_scene(c, d[i].n_tris, d[i].verts, d[i].norms, d[i].tri_mesh, d[i].n_meshes, d[i].mesh_mat,
                         d[i].mesh_smooth, d[i].n_materials, d[i].materials, d[i].sky, d[i].ground)))
      return fail(c, r, "scene " + std::to_string(i) + ": " + c->err);
    if (d[i].n_emitters >= 0 && d[i].n_emitters > 0 && !d[i].emitters)
      return fail(c, RTX_ERR_INVALID, "scene " + std::to_string(i) + ": emitters is NULL");
    for (int k = 0; k < std::max(d[i].n_emitters, 0); ++k)
      if (d[i].emitters[k] < 0 || d[i].emitters[k] >= d[i].n_tris)
        return fail(c, RTX_ERR_INVALID, "scene " + std::to_string(i) + ": emitter id out of range");
  }
  long long tot = 0;
  for (int i = 0; i < n_scenes; ++i) tot += d[i].n_tris;
  if (tot > (1 << 27)) return fail(c, RTX_ERR_INVALID, "more than 2^27 triangles in the batch");
  RTX_CUDA(cudaSetDevice(c->device), "cudaSetDevice");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  // host builds, several scenes at a time
  std::vector<HostScene> hs(n_scenes);
  auto t0 = std::chrono::steady_clock::now();
  run_parallel((size_t)n_scenes, std::max(1u, std::min(std::thread::hardware_concurrency(), 16u)), [&](size_t i) {
    build_host_scene(hs[i], d[i].n_tris, d[i].verts, d[i].norms, d[i].tri_mesh, d[i].n_meshes, d[i].mesh_mat,
                     d[i].mesh_smooth, d[i].n_materials, d[i].materials, d[i].sky, d[i].ground, c->leaf_size);
  });
  // merge: node, leaf-record, triangle-id, material and emitter indices
  // rebased.  Each scene's block starts where the sizes of the scenes before
  // it end, so the scenes are copied into place on host threads.
  std::vector<size_t> o_nodes(n_scenes + 1, 0), o_nodes4(n_scenes + 1, 0), o_tris(n_scenes + 1, 0),
      o_mats(n_scenes + 1, 0), o_emit(n_scenes + 1, 0);
  std::vector<int> tri_bases(n_scenes), mat_bases(n_scenes);
  int tri_base = 0, mat_base = 0;
  for (int i = 0; i < n_scenes; ++i) {
    const HostScene& h = hs[i];
    o_nodes[i + 1] = o_nodes[i] + h.b.nodes.size();
    o_nodes4[i + 1] = o_nodes4[i] + h.b.nodes4.size();
    o_tris[i + 1] = o_tris[i] + (size_t)h.n_tris;
    o_mats[i + 1] = o_mats[i] + h.mats.size();
    o_emit[i + 1] = o_emit[i] + (d[i].n_emitters >= 0 ? (size_t)d[i].n_emitters : h.emitters.size());
    tri_bases[i] = tri_base;
    mat_bases[i] = mat_base;
    tri_base += h.n_tris;
    mat_base += h.n_mats;
  }
  Float4Array nodes(o_nodes[n_scenes]), nodes4(o_nodes4[n_scenes]), tris(3 * o_tris[n_scenes]),
      shade(4 * o_tris[n_scenes]), geo(3 * o_tris[n_scenes]);
  std::vector<float> mats(o_mats[n_scenes]);
  std::vector<int32_t> emit(o_emit[n_scenes]);
  c->bscenes.assign(n_scenes, {});
  run_parallel((size_t)n_scenes, std::max(1u, std::min(std::thread::hardware_concurrency(), 16u)), [&](size_t i) {
    const HostScene& h = hs[i];
    const int tb = tri_bases[i], mb = mat_bases[i];
    const int node_base = (int)(o_nodes[i] / 4), node4_base = (int)(o_nodes4[i] / kNode4Vecs);
    float4* nd = nodes.data() + o_nodes[i];
    for (size_t k = 0; k < h.b.nodes.size(); k += 4) {
      float4 n3 = h.b.nodes[k + 3];
      int ch[2];
      std::memcpy(ch, &n3.x, 8);
      for (int& x : ch) x = x >= 0 ? x + node_base : rebase_leaf(x, tb);
      std::memcpy(&n3.x, ch, 8);
      nd[k] = h.b.nodes[k];
      nd[k + 1] = h.b.nodes[k + 1];
      nd[k + 2] = h.b.nodes[k + 2];
      nd[k + 3] = n3;
    }
    // 4-wide nodes: six float4 of planes, child references in the seventh
    // (empty slots hold 0 behind a box that is never hit)
    float4* nd4 = nodes4.data() + o_nodes4[i];
    for (size_t k = 0; k < h.b.nodes4.size(); k += kNode4Vecs) {
      for (int r6 = 0; r6 < 6; ++r6) nd4[k + r6] = h.b.nodes4[k + r6];
      float4 m = h.b.nodes4[k + 6];
      int ch[4];
      std::memcpy(ch, &m, 16);
      for (int& x : ch) x = x >= 0 ? x + node4_base : rebase_leaf(x, tb);
      std::memcpy(&m, ch, 16);
      nd4[k + 6] = m;
    }
    float4* tr = tris.data() + 3 * o_tris[i];
    for (size_t k = 0; k < h.b.tris.size(); k += 3) {
      float4 a4 = h.b.tris[k];
      int id;
      std::memcpy(&id, &a4.w, 4);
      id += tb;
      std::memcpy(&a4.w, &id, 4);
      tr[k] = a4;
      tr[k + 1] = h.b.tris[k + 1];
      tr[k + 2] = h.b.tris[k + 2];
    }
    float4* sh = shade.data() + 4 * o_tris[i];
    for (size_t k = 0; k < h.shade.size(); ++k) {
      float4 v = h.shade[k];
      if (k % 4 == 1) {
        uint32_t info;
        std::memcpy(&info, &v.w, 4);
        info = ((info & 0x7fffffffu) + (uint32_t)mb) | (info & 0x80000000u);
        std::memcpy(&v.w, &info, 4);
      }
      sh[k] = v;
    }
    std::copy(h.geo.begin(), h.geo.end(), geo.begin() + 3 * o_tris[i]);
    std::copy(h.mats.begin(), h.mats.end(), mats.begin() + o_mats[i]);
    rtx_context::BatchScene& bs = c->bscenes[i];
    int root = h.b.root;
    bs.root = root == kEmptyRoot ? kEmptyRoot : (root >= 0 ? root + node_base : rebase_leaf(root, tb));
    int root4 = h.b.root4;
    bs.root4 = root4 == kEmptyRoot ? kEmptyRoot : (root4 >= 0 ? root4 + node4_base : rebase_leaf(root4, tb));
    bs.e_begin = (int)o_emit[i];
    int32_t* em = emit.data() + o_emit[i];
    if (d[i].n_emitters >= 0) {
      for (int k = 0; k < d[i].n_emitters; ++k) em[k] = d[i].emitters[k] + tb;
      bs.n_emitters = d[i].n_emitters;
    } else {
      for (size_t k = 0; k < h.emitters.size(); ++k) em[k] = h.emitters[k] + tb;
      bs.n_emitters = (int)h.emitters.size();
    }
    bs.n_tris = h.n_tris;
    bs.keyb = sort_key_bounds(h.b.nodes4, h.b.root4);
    for (int k = 0; k < 3; ++k) {
      bs.sky[k] = h.sky[k];
      bs.ground[k] = h.ground[k];
    }
  });
  double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if ((r = upload_buf(c, c->b_nodes, nodes.data(), nodes.size() * sizeof(float4), "upload batch nodes"))) return r;
  if ((r = upload_buf(c, c->b_nodes4, nodes4.data(), nodes4.size() * sizeof(float4), "upload batch nodes4")))
    return r;
  if ((r = upload_buf(c, c->b_tris, tris.data(), tris.size() * sizeof(float4), "upload batch tris"))) return r;
  if ((r = upload_buf(c, c->b_shade, shade.data(), shade.size() * sizeof(float4), "upload batch shade"))) return r;
  if ((r = upload_buf(c, c->b_geo, geo.data(), geo.size() * sizeof(float4), "upload batch geo"))) return r;
  if ((r = upload_buf(c, c->b_mats, mats.data(), mats.size() * sizeof(float), "upload batch mats"))) return r;
  if ((r = upload_buf(c, c->b_emit, emit.data(), emit.size() * sizeof(int32_t), "upload batch emitters"))) return r;
  DeviceScene& s = c->bds;
  s = DeviceScene{};
  s.stack_limit = c->stack_limit;
  s.nodes = (const float4*)c->b_nodes.p;
  s.nodes4 = (const float4*)c->b_nodes4.p;
  s.root4 = kEmptyRoot;
  s.tris = (const float4*)c->b_tris.p;
  s.shade = (const float4*)c->b_shade.p;
  s.geo = (const float4*)c->b_geo.p;
  s.mats = (const float*)c->b_mats.p;
  s.emitters = (const int*)c->b_emit.p;
  s.perm = (const uint8_t*)c->perm.p;
  s.root = kEmptyRoot;
  s.n_tris = tri_base;
  s.n_emitters = (int)emit.size();
  s.n_mats = mat_base;
  s.textured = 0;
  for (size_t m = 0; m < mats.size() / RTX_MATERIAL_FLOATS; ++m)
    s.textured |= mats[RTX_MATERIAL_FLOATS * m + 21] != 0.0f;
  s.lobes = material_lobes(mats.data(), (int)(mats.size() / RTX_MATERIAL_FLOATS));
  c->has_batch = true;
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    c->graph_key.clear();
  }
  c->stats.bvh_build_ms = ms;
  c->stats.bvh_nodes = (int32_t)(nodes.size() / 4);
  c->stats.node_bytes = 64;
  c->stats.tri_bytes = 48;
  return RTX_OK;
}

int rtx_batch_upload(rtx_context* c, int n_scenes, const rtx_scene_desc* d) {
  return host_guard(c, [&] { return batch_upload(c, n_scenes, d); });
}

int rtx_scene_emitters(rtx_context* c, int32_t* out, int cap, int* n_out) {
  if (!c || !n_out) return RTX_ERR_INVALID;
  if (!c->has_scene) return fail(c, RTX_ERR_NO_SCENE, "no scene uploaded");
  *n_out = (int)c->emitters.size();
  if (out)
    for (int i = 0; i < *n_out && i < cap; ++i) out[i] = c->emitters[i];
  return RTX_OK;
}

int rtx_scene_set_emitters(rtx_context* c, const int32_t* ids, int n) {
  if (!c) return RTX_ERR_INVALID;
  if (!c->has_scene) return fail(c, RTX_ERR_NO_SCENE, "no scene uploaded");
  if (n < 0 || (n > 0 && !ids)) return fail(c, RTX_ERR_INVALID, "bad emitter list");
  for (int i = 0; i < n; ++i)
    if (ids[i] < 0 || ids[i] >= c->ds.n_tris) return fail(c, RTX_ERR_INVALID, "emitter id out of range");
  RTX_CUDA(cudaSetDevice(c->device), "cudaSetDevice");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  c->emitters.assign(ids, ids + n);
  RTX_CUDA(c->emit.ensure((size_t)n * sizeof(int32_t)), "emitter alloc");
  if (n) RTX_CUDA(cudaMemcpy(c->emit.p, ids, (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice), "emitter upload");
  c->ds.emitters = (const int*)c->emit.p;
  c->ds.n_emitters = n;
  return RTX_OK;
}

int rtx_scene_set_texture_table(rtx_context* c, const uint8_t* perm) {
  if (!c) return RTX_ERR_INVALID;
  if (!perm) return fail(c, RTX_ERR_INVALID, "table is NULL");
  int seen[256] = {0};
  for (int i = 0; i < 256; ++i)
    if (seen[perm[i]]++) return fail(c, RTX_ERR_INVALID, "the table is not a permutation of 0..255");
  RTX_CUDA(cudaSetDevice(c->device), "cudaSetDevice");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  RTX_CUDA(cudaMemcpy(c->perm.p, perm, 256, cudaMemcpyHostToDevice), "table upload");
  return RTX_OK;
}

int rtx_texture_sample(rtx_context* c, int kind, float param, int n, const float* uv, float* out) {
  if (!c) return RTX_ERR_INVALID;
  if (kind < 1 || kind > 3) return fail(c, RTX_ERR_INVALID, "kind must be 1, 2 or 3");
  if (kind == 1 && !(std::fabs(param) < 1e6f)) return fail(c, RTX_ERR_INVALID, "checkerboard scale out of range");
  if (n < 0 || (n > 0 && (!uv || !out))) return fail(c, RTX_ERR_INVALID, "bad point arrays");
  int r;
  if ((r = begin(c))) return r;
  Arg ai, ao;
  if ((r = bind_in(c, uv, (size_t)n * 8, 0, ai))) return r;
  if ((r = bind_out(c, out, (size_t)n * 4, 1, ao))) return r;
  cudaError_t e = launch_texture_sample(kind, param, (const uint8_t*)c->perm.p, n, (const float*)ai.dev,
                                        (float*)ao.dev, c->stream);
  c->stats.kernel_launches = n > 0 ? 1 : 0;
  if (e != cudaSuccess) return cuda_fail(c, e, "texture kernel");
  if ((r = copy_back(c, ao))) return r;
  return finish(c, all_device({&ai, &ao}));
}

// A display resolve requested by the caller (see Resolve).
struct ResolveReq {
  float limit, gamma;
  float* display;
  uint8_t* bytes;
  int format;
};

static int check_resolve(rtx_context* c, const ResolveReq& q) {
  if (!(q.limit == q.limit) || !(q.gamma == q.gamma)) return fail(c, RTX_ERR_INVALID, "limit / gamma is NaN");
  if (q.format != kResolveBmp && q.format != kResolveRgb) return fail(c, RTX_ERR_INVALID, "unknown byte format");
  return RTX_OK;
}

static size_t resolve_bytes(int W, int H, int format) {
  return format == kResolveBmp ? bmp_row_bytes(W) * (size_t)H : (size_t)W * H * 3;
}

// bind the resolve outputs to stage slots s, s + 1
static int bind_resolve(rtx_context* c, const ResolveReq& q, int W, int H, int slot, Arg& ad, Arg& ab,
                        Resolve& r) {
  int e;
  if ((e = bind_out(c, q.display, q.display ? (size_t)W * H * 12 : 0, slot, ad))) return e;
  if ((e = bind_out(c, q.bytes, q.bytes ? resolve_bytes(W, H, q.format) : 0, slot + 1, ab))) return e;
  r.limit = q.limit;
  r.ratio = q.gamma > 0.0f ? 1.0f / q.gamma : 0.0f;  // GammaCorrection: ratio = 1.0f / gamma
  r.display = (float*)ad.dev;
  r.bytes = (uint8_t*)ab.dev;
  r.format = q.format;
  r.W = W;
  return RTX_OK;
}

static int render_paths(rtx_context* c, const float* cam, int W, int H, int first, int n_samples,
                        int spp, int max_depth, uint64_t seed, float* out, bool per_path,
                        const ResolveReq* rq = nullptr) {
  if (!c) return RTX_ERR_INVALID;
  int r;
  if ((r = check_cam(c, cam, W, H))) return r;
  if (!out) return fail(c, RTX_ERR_INVALID, "output is NULL");
  if (n_samples < 0 || spp < 0 || first < 0) return fail(c, RTX_ERR_INVALID, "negative sample count");
  if (max_depth < 1 || max_depth > 63) return fail(c, RTX_ERR_INVALID, "max_depth must be in [1, 63]");
  size_t npix = (size_t)W * H;
  size_t out_elems = per_path ? npix * (size_t)n_samples : npix;
  if ((r = begin(c))) return r;
  Arg o;
  bool acc = c->accumulate && !per_path;
  if (acc) {
    // the caller's image is read as well as written
    if ((r = bind_in(c, out, out_elems * 3 * sizeof(float), 0, o))) return r;
    if (!is_device_ptr(out)) o.host = out;
  } else if ((r = bind_out(c, out, out_elems * 3 * sizeof(float), 0, o))) {
    return r;
  }
  Arg ad, ab;
  Resolve rs{};
  if (rq) {
    if ((r = check_resolve(c, *rq))) return r;
    if ((r = bind_resolve(c, *rq, W, H, 1, ad, ab, rs))) return r;
  }
  CamParams cp = make_cam_params(cam, W, H);
  PtParams p;
  p.resolve = rs;
  p.W = W;
  p.H = H;
  p.spp = spp;
  p.first_sample = first;
  p.n_samples = n_samples;
  p.max_depth = max_depth;
  p.seed = seed;
  p.wave_paths = (int)c->wave_paths;
  p.block = c->block;
  p.per_path = per_path;
  p.accumulate = acc;
  p.count_visits = c->count_visits;
  p.primary_cache = c->primary_cache;
  p.sort_material = sort_material_for(c, c->ds);
  p.sort_rays = sort_rays_for(c, c->ds.n_tris);
  p.overlap = c->overlap;
  p.traversal = c->traversal;
  p.min_busy = c->min_busy;
  RTX_CUDA(cudaMemsetAsync(c->d_counters, 0, sizeof(Counters), c->stream), "reset counters");
  int launches = 0, ext_launches = 0, vtx_launches = 0;
  std::string why;
  c->timer.reset();  // times are per render; rtx_get_stats collects them
  cudaError_t e = pt_render(c->pt, c->ds, cp, p, (float*)o.dev, c->d_err, c->d_counters,
                            &c->timer, c->stream, &launches, &ext_launches, &vtx_launches, &why);
  c->stats.kernel_launches = launches;
  c->stats.extend_launches = ext_launches;
  c->stats.shade_launches = vtx_launches;
  c->stats.connect_launches = vtx_launches;
  if (e != cudaSuccess) {
    if (!why.empty()) return fail(c, RTX_ERR_INVALID, why);
    return cuda_fail(c, e, "pt_render");
  }
  if ((r = copy_back(c, o))) return r;
  if ((r = copy_back(c, ad))) return r;
  if ((r = copy_back(c, ab))) return r;
  return finish(c, all_device({&o, &ad, &ab}));
}

int rtx_render_pt(rtx_context* c, const float* cam, int W, int H, int spp, int max_depth,
                  uint64_t seed, float* out) {
  if (c && spp <= 0) return fail(c, RTX_ERR_INVALID, "spp must be positive");
  return render_paths(c, cam, W, H, 0, spp, spp, max_depth, seed, out, false);
}

int rtx_render_pt_progressive(rtx_context* c, const float* cam, int W, int H, int first_sample, int n_samples,
                              int spp, int max_depth, uint64_t seed, float* out) {
  if (!c) return RTX_ERR_INVALID;
  if (spp <= 0 || n_samples <= 0 || first_sample < 0 || (long long)first_sample + n_samples > spp)
    return fail(c, RTX_ERR_INVALID, "need 0 <= first_sample < first_sample + n_samples <= spp");
  // samples after the first add to the image rendered so far
  const bool saved = c->accumulate;
  c->accumulate = first_sample > 0;
  int r = render_paths(c, cam, W, H, first_sample, n_samples, spp, max_depth, seed, out, false);
  c->accumulate = saved;
  return r;
}

int rtx_render_pt_resolved(rtx_context* c, const float* cam, int W, int H, int spp, int max_depth,
                           uint64_t seed, float* out, float limit, float gamma, float* display,
                           uint8_t* bytes, int format) {
  if (c && spp <= 0) return fail(c, RTX_ERR_INVALID, "spp must be positive");
  ResolveReq q{limit, gamma, display, bytes, format};
  return render_paths(c, cam, W, H, 0, spp, spp, max_depth, seed, out, false, &q);
}

// ---- multi-scene batch ------------------------------------------------------------
int rtx_render_batch(rtx_context* c, int n_jobs, const rtx_job* jobs, int max_depth, float* out) {
  if (!c) return RTX_ERR_INVALID;
  if (!c->has_batch) return fail(c, RTX_ERR_NO_SCENE, "no batch uploaded (rtx_batch_upload)");
  if (n_jobs < 1 || !jobs || !out) return fail(c, RTX_ERR_INVALID, "no frames or NULL output");
  if (max_depth < 1 || max_depth > 63) return fail(c, RTX_ERR_INVALID, "max_depth must be in [1, 63]");
  if (c->traversal == 1) return fail(c, RTX_ERR_INVALID, "batches use the batch traversals (RTX_OPT_TRAVERSAL 0 or 2)");
  std::vector<PtJob> hj((size_t)n_jobs);
  long long q = 0, pix = 0;
  for (int j = 0; j < n_jobs; ++j) {
    const rtx_job& J = jobs[j];
    if (J.scene < 0 || J.scene >= (int)c->bscenes.size())
      return fail(c, RTX_ERR_INVALID, "frame " + std::to_string(j) + ": scene index out of range");
    if (J.W <= 0 || J.H <= 0 || J.spp <= 0 || (long long)J.W * J.H > (1LL << 28))
      return fail(c, RTX_ERR_INVALID, "frame " + std::to_string(j) + ": bad size or spp");
    const rtx_context::BatchScene& bs = c->bscenes[J.scene];
    PtJob& P = hj[j];
    P.q_begin = q;
    P.pix_begin = pix;
    P.npix = J.W * J.H;
    P.W = J.W;
    P.spp = J.spp;
    P.first_sample = 0;
    P.root = bs.root;
    P.root4 = bs.root4;
    P.e_begin = bs.e_begin;
    P.n_emitters = bs.n_emitters;
    P.k0 = (uint32_t)J.seed;
    P.k1 = (uint32_t)(J.seed >> 32);
    for (int k = 0; k < 3; ++k) {
      P.sky[k] = bs.sky[k];
      P.ground[k] = bs.ground[k];
    }
    P.cam = make_cam_params(J.camera, J.W, J.H);
    P.keyb = bs.keyb;
    q += (long long)P.npix * J.spp;
    pix += P.npix;
  }
  if (pix > (1LL << 30)) return fail(c, RTX_ERR_INVALID, "more than 2^30 pixels in one batch frame");
  int r;
  if ((r = begin(c))) return r;
  // the job table through pinned staging (the copy a replayed graph needs)
  if (c->pinned_cap < n_jobs) {
    if (c->h_jobs_pinned) cudaFreeHost(c->h_jobs_pinned);
    if (c->h_jobq_pinned) cudaFreeHost(c->h_jobq_pinned);
    c->h_jobs_pinned = nullptr;
    c->h_jobq_pinned = nullptr;
    c->pinned_cap = 0;
    RTX_CUDA(cudaMallocHost(&c->h_jobs_pinned, sizeof(PtJob) * n_jobs), "pinned jobs");
    RTX_CUDA(cudaMallocHost(&c->h_jobq_pinned, sizeof(long long) * n_jobs), "pinned jobs");
    c->pinned_cap = n_jobs;
  }
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");  // staging reuse
  std::memcpy(c->h_jobs_pinned, hj.data(), sizeof(PtJob) * n_jobs);
  for (int j = 0; j < n_jobs; ++j) c->h_jobq_pinned[j] = hj[j].q_begin;
  RTX_CUDA(c->b_jobs.ensure(sizeof(PtJob) * n_jobs), "job table");
  RTX_CUDA(c->b_jobq.ensure(sizeof(long long) * n_jobs), "job table");
  RTX_CUDA(cudaMemcpyAsync(c->b_jobs.p, c->h_jobs_pinned, sizeof(PtJob) * n_jobs, cudaMemcpyHostToDevice,
                           c->stream),
           "job table H2D");
  RTX_CUDA(cudaMemcpyAsync(c->b_jobq.p, c->h_jobq_pinned, sizeof(long long) * n_jobs, cudaMemcpyHostToDevice,
                           c->stream),
           "job table H2D");
  Arg o;
  if ((r = bind_out(c, out, (size_t)pix * 12, 0, o))) return r;
  PtParams p{};
  p.max_depth = max_depth;
  p.wave_paths = (int)c->wave_paths;
  p.block = c->block;
  p.count_visits = c->count_visits;
  p.primary_cache = c->primary_cache;
  p.sort_material = sort_material_for(c, c->bds);
  p.sort_rays = sort_rays_for(c, c->bds.n_tris);
  p.overlap = c->overlap;
  p.traversal = c->traversal;
  p.min_busy = c->min_busy;
  p.accumulate = c->accumulate;
  p.n_jobs = n_jobs;
  p.d_jobs = (const PtJob*)c->b_jobs.p;
  p.d_job_q = (const long long*)c->b_jobq.p;
  p.h_jobs = hj.data();
  RTX_CUDA(cudaMemsetAsync(c->d_counters, 0, sizeof(Counters), c->stream), "reset counters");
  c->timer.reset();
  // the launch shape: everything the captured kernels bake in
  std::vector<int64_t> key = {n_jobs, max_depth, c->wave_paths, c->block, c->primary_cache, c->count_visits,
                              c->accumulate, (int64_t)p.sort_material, (int64_t)p.sort_rays, c->traversal, c->overlap,
                              c->stack_limit, (int64_t)(intptr_t)o.dev};
  for (int j = 0; j < n_jobs; ++j) key.insert(key.end(), {jobs[j].scene, jobs[j].W, jobs[j].H, jobs[j].spp});
  int launches = 0, ext_launches = 0, vtx_launches = 0;
  std::string why;
  cudaError_t e = cudaSuccess;
  const bool graphable = c->use_graph && !c->timer.on;
  if (graphable && c->graph && key == c->graph_key) {
    e = cudaGraphLaunch(c->graph, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphLaunch");
    c->stats.kernel_launches = 0;  // kernels are graph nodes
  } else {
    e = pt_render(c->pt, c->bds, CamParams{}, p, (float*)o.dev, c->d_err, c->d_counters, &c->timer, c->stream,
                  &launches, &ext_launches, &vtx_launches, &why);
    c->stats.kernel_launches = launches;
    c->stats.extend_launches = ext_launches;
    c->stats.shade_launches = vtx_launches;
    c->stats.connect_launches = vtx_launches;
    if (e != cudaSuccess) {
      if (!why.empty()) return fail(c, RTX_ERR_INVALID, why);
      return cuda_fail(c, e, "pt_render (batch)");
    }
    if (graphable) {
      // capture the same launch sequence (the wave size this render used)
      if (c->graph) {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
      }
      PtParams pc = p;
      pc.wave_paths = (int)pt_last_wave(c->pt);
      cudaGraph_t g = nullptr;
      int l2 = 0, x2 = 0, v2 = 0;
      RTX_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
      cudaError_t ec = pt_render(c->pt, c->bds, CamParams{}, pc, (float*)o.dev, c->d_err, c->d_counters,
                                 &c->timer, c->stream, &l2, &x2, &v2, &why);
      cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
      if (ec != cudaSuccess || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(c, ec != cudaSuccess ? ec : ee, "graph capture");
      }
      ee = cudaGraphInstantiate(&c->graph, g, 0);
      cudaGraphDestroy(g);
      if (ee != cudaSuccess) {
        c->graph = nullptr;
        return cuda_fail(c, ee, "cudaGraphInstantiate");
      }
      c->graph_key = key;
    }
  }
  if ((r = copy_back(c, o))) return r;
  return finish(c, all_device({&o}));
}

// Autotuner: frame time of a batch over BVH leaf sizes (each a rebuild of the
// batch), then threads per block x paths per wave, coordinate-wise; each
// candidate renders the frame twice and keeps the faster device time.
static int time_frame(rtx_context* c, int n_jobs, const rtx_job* jobs, int max_depth, float* d_out, double* ms) {
  double best = 1e30;
  for (int rep = 0; rep < 2; ++rep) {
    int r = rtx_render_batch(c, n_jobs, jobs, max_depth, d_out);
    if (r) return r;
    best = std::min(best, c->stats.last_gpu_ms);
  }
  *ms = best;
  return RTX_OK;
}

static int batch_autotune(rtx_context* c, int n_scenes, const rtx_scene_desc* scenes, int n_jobs,
                          const rtx_job* jobs, int max_depth, rtx_tune_result* out) {
  if (!c) return RTX_ERR_INVALID;
  if (!out || !jobs || n_jobs < 1) return fail(c, RTX_ERR_INVALID, "NULL argument");
  const bool saved_graph = c->use_graph, saved_timer = c->timer.on;
  c->use_graph = false;
  c->timer.on = false;
  int r = RTX_OK;
  long long pix = 0;
  for (int j = 0; j < n_jobs; ++j) pix += (long long)std::max(jobs[j].W, 0) * std::max(jobs[j].H, 0);
  float* d_out = nullptr;
  rtx_tune_result res{};
  res.trials = 0;
  if (c->traversal == 1) c->traversal = 2;  // batches take the batch traversals
  auto done = [&](int code) {
    if (d_out) cudaFree(d_out);
    c->use_graph = saved_graph;
    c->timer.on = saved_timer;
    return code;
  };
  cudaError_t e = cudaMalloc(&d_out, (size_t)std::max(pix, 1LL) * 12);
  if (e != cudaSuccess) return done(cuda_fail(c, e, "autotune output"));
  double ms = 0.0;
  // the starting point: the context's current options
  if (scenes && (r = rtx_batch_upload(c, n_scenes, scenes))) return done(r);
  if ((r = time_frame(c, n_jobs, jobs, max_depth, d_out, &ms))) return done(r);
  res.ms_default = ms;
  res.block = c->block;
  res.wave_paths = c->wave_paths;
  res.leaf_size = c->leaf_size;
  res.ms = ms;
  ++res.trials;
  if (scenes) {
    for (int leaf : {2, 4, 8}) {
      if (leaf == res.leaf_size) continue;
      c->leaf_size = leaf;
      if ((r = rtx_batch_upload(c, n_scenes, scenes)) || (r = time_frame(c, n_jobs, jobs, max_depth, d_out, &ms)))
        return done(r);
      ++res.trials;
      if (ms < res.ms) {
        res.ms = ms;
        res.leaf_size = leaf;
      }
    }
    c->leaf_size = (int)res.leaf_size;
    if ((r = rtx_batch_upload(c, n_scenes, scenes))) return done(r);
  }
  for (int block : {64, 128})
    for (long long wave : {1LL << 20, 1LL << 22, 1LL << 24, 0LL}) {
      if (block == res.block && wave == res.wave_paths) continue;
      c->block = block;
      c->wave_paths = wave;
      if ((r = time_frame(c, n_jobs, jobs, max_depth, d_out, &ms))) return done(r);
      ++res.trials;
      if (ms < res.ms) {
        res.ms = ms;
        res.block = block;
        res.wave_paths = wave;
      }
    }
  c->block = (int)res.block;
  c->wave_paths = res.wave_paths;
  // binary or 4-wide tree
  res.traversal = c->traversal;
  c->traversal = c->traversal == 2 ? 0 : 2;
  if ((r = time_frame(c, n_jobs, jobs, max_depth, d_out, &ms))) return done(r);
  ++res.trials;
  if (ms < res.ms) {
    res.ms = ms;
    res.traversal = c->traversal;
  }
  c->traversal = res.traversal;
  // material-sorted shading helps scenes with many materials and costs a
  // little where there are few: keep whichever is faster
  res.sort_material = sort_material_for(c, c->bds) ? 1 : 0;
  c->sort_material = res.sort_material ? 0 : 1;
  if ((r = time_frame(c, n_jobs, jobs, max_depth, d_out, &ms))) return done(r);
  ++res.trials;
  if (ms < res.ms) {
    res.ms = ms;
    res.sort_material = c->sort_material;
  }
  c->sort_material = res.sort_material;
  // ray-sorted traversal: its sorts cost a fixed few launches per vertex
  res.sort_rays = sort_rays_for(c, c->bds.n_tris) ? 1 : 0;
  c->sort_rays = res.sort_rays ? 0 : 1;
  if ((r = time_frame(c, n_jobs, jobs, max_depth, d_out, &ms))) return done(r);
  ++res.trials;
  if (ms < res.ms) {
    res.ms = ms;
    res.sort_rays = c->sort_rays;
  }
  c->sort_rays = res.sort_rays;
  // occlusion launches beside the next vertex's closest-hit launches
  res.overlap = c->overlap ? 1 : 0;
  c->overlap = !c->overlap;
  if ((r = time_frame(c, n_jobs, jobs, max_depth, d_out, &ms))) return done(r);
  ++res.trials;
  if (ms < res.ms) {
    res.ms = ms;
    res.overlap = c->overlap ? 1 : 0;
  }
  c->overlap = res.overlap != 0;
  *out = res;
  return done(RTX_OK);
}

int rtx_batch_autotune(rtx_context* c, int n_scenes, const rtx_scene_desc* scenes, int n_jobs,
                       const rtx_job* jobs, int max_depth, rtx_tune_result* out) {
  return host_guard(c, [&] { return batch_autotune(c, n_scenes, scenes, n_jobs, jobs, max_depth, out); });
}

// ---- display resolve and image files --------------------------------------------
static int resolve_image(rtx_context* c, const float* in, int W, int H, const ResolveReq& q) {
  if (!c) return RTX_ERR_INVALID;
  int r;
  if (!in) return fail(c, RTX_ERR_INVALID, "input is NULL");
  if (W <= 0 || H <= 0 || (long long)W * H > (1LL << 30)) return fail(c, RTX_ERR_INVALID, "bad image size");
  if ((r = check_resolve(c, q))) return r;
  if ((r = begin(c))) return r;
  Arg ai, ad, ab;
  Resolve rs{};
  if ((r = bind_in(c, in, (size_t)W * H * 12, 0, ai))) return r;
  if ((r = bind_resolve(c, q, W, H, 1, ad, ab, rs))) return r;
  cudaError_t e = launch_resolve((const float*)ai.dev, W, H, rs, c->stream);
  c->stats.kernel_launches = 1;
  if (e != cudaSuccess) return cuda_fail(c, e, "resolve kernel");
  if ((r = copy_back(c, ad))) return r;
  if ((r = copy_back(c, ab))) return r;
  return finish(c, all_device({&ai, &ad, &ab}));
}

int rtx_image_tonemap(rtx_context* c, const float* in, float* out, int W, int H, float limit) {
  if (c && !(limit > 0.0f)) return fail(c, RTX_ERR_INVALID, "limit must be positive");
  if (c && !out) return fail(c, RTX_ERR_INVALID, "output is NULL");
  return resolve_image(c, in, W, H, ResolveReq{limit, 0.0f, out, nullptr, kResolveRgb});
}

int rtx_image_gamma(rtx_context* c, const float* in, float* out, int W, int H, float gamma) {
  if (c && !(gamma > 0.0f)) return fail(c, RTX_ERR_INVALID, "gamma must be positive");
  if (c && !out) return fail(c, RTX_ERR_INVALID, "output is NULL");
  return resolve_image(c, in, W, H, ResolveReq{0.0f, gamma, out, nullptr, kResolveRgb});
}

int rtx_image_resolve(rtx_context* c, const float* in, int W, int H, float limit, float gamma,
                      float* display, uint8_t* bytes, int format) {
  return resolve_image(c, in, W, H, ResolveReq{limit, gamma, display, bytes, format});
}

namespace {
void put32(uint8_t* p, uint32_t v) {
  for (int k = 0; k < 4; ++k) p[k] = (uint8_t)(v >> (8 * k));
}
void put16(uint8_t* p, uint16_t v) {
  p[0] = (uint8_t)v;
  p[1] = (uint8_t)(v >> 8);
}
}  // namespace

int rtx_encode_bmp(rtx_context* c, const float* in, int W, int H, uint8_t* file, size_t cap,
                   size_t* size) {
  if (!c) return RTX_ERR_INVALID;
  if (!size) return fail(c, RTX_ERR_INVALID, "size is NULL");
  if (W <= 0 || H <= 0 || (long long)W * H > (1LL << 30)) return fail(c, RTX_ERR_INVALID, "bad image size");
  const size_t pixels = bmp_row_bytes(W) * (size_t)H;
  *size = 54 + pixels;
  if (!file) return RTX_OK;  // size query
  if (cap < *size) return fail(c, RTX_ERR_INVALID, "file buffer too small");
  // BITMAPFILEHEADER + BITMAPINFOHEADER as BMPExporter writes them
  // (src/exporter.cpp:38-77), except that the file size counts the row padding
  std::memset(file, 0, 54);
  file[0] = 'B';
  file[1] = 'M';
  put32(file + 2, (uint32_t)*size);
  put32(file + 10, 54);
  put32(file + 14, 40);
  put32(file + 18, (uint32_t)W);
  put32(file + 22, (uint32_t)H);
  put16(file + 26, 1);
  put16(file + 28, 24);
  put32(file + 38, 3780);
  put32(file + 42, 3780);
  return resolve_image(c, in, W, H, ResolveReq{0.0f, 0.0f, nullptr, file + 54, kResolveBmp});
}

int rtx_encode_ppm(rtx_context* c, const float* in, int W, int H, char* file, size_t cap,
                   size_t* size) {
  if (!c) return RTX_ERR_INVALID;
  if (!size) return fail(c, RTX_ERR_INVALID, "size is NULL");
  if (W <= 0 || H <= 0 || (long long)W * H > (1LL << 28)) return fail(c, RTX_ERR_INVALID, "bad image size");
  std::vector<uint8_t> rgb((size_t)W * H * 3);
  int r = resolve_image(c, in, W, H, ResolveReq{0.0f, 0.0f, nullptr, rgb.data(), kResolveRgb});
  if (r) return r;
  // PPMExporter (src/exporter.cpp:8-29): "P3", "W H", "255", then one
  // "r g b" line per pixel, buffer row 0 first
  std::string txt = "P3\n" + std::to_string(W) + ' ' + std::to_string(H) + "\n255\n";
  txt.reserve(txt.size() + rgb.size() * 4);
  char line[16];
  for (size_t i = 0; i < (size_t)W * H; ++i) {
    int n = std::snprintf(line, sizeof line, "%d %d %d\n", rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
    txt.append(line, (size_t)n);
  }
  *size = txt.size();
  if (!file) return RTX_OK;
  if (cap < txt.size()) return fail(c, RTX_ERR_INVALID, "file buffer too small");
  std::memcpy(file, txt.data(), txt.size());
  return RTX_OK;
}

int rtx_trace_paths(rtx_context* c, const float* cam, int W, int H, int first_sample,
                    int n_samples, int max_depth, uint64_t seed, float* out) {
  return render_paths(c, cam, W, H, first_sample, n_samples, 1, max_depth, seed, out, true);
}

static int primary_pass(rtx_context* c, const float* cam, int W, int H, int mode, float near_,
                        float far_, float* n_out, float* a_out, float* d_out, int32_t* tri_out,
                        float* tuv_out) {
  if (!c) return RTX_ERR_INVALID;
  int r;
  if ((r = check_cam(c, cam, W, H))) return r;
  size_t npix = (size_t)W * H;
  if ((r = begin(c))) return r;
  Arg an, aa, ad, at, au;
  if ((r = bind_out(c, n_out, npix * 12, 0, an))) return r;
  if ((r = bind_out(c, a_out, npix * 12, 1, aa))) return r;
  if ((r = bind_out(c, d_out, npix * 12, 2, ad))) return r;
  if (mode & 2) {
    if (!tri_out || !tuv_out) return fail(c, RTX_ERR_INVALID, "hit outputs are NULL");
    if ((r = bind_out(c, tri_out, npix * 4, 0, at))) return r;
    if ((r = bind_out(c, tuv_out, npix * 12, 1, au))) return r;
  }
  CamParams cp = make_cam_params(cam, W, H);
  int launches = 0;
  cudaError_t e = launch_primary(c->ds, cp, mode, near_, far_, (float*)an.dev, (float*)aa.dev,
                                 (float*)ad.dev, (int*)at.dev, (float*)au.dev, c->d_err,
                                 c->stream, &launches);
  c->stats.kernel_launches = launches;
  if (e != cudaSuccess) return cuda_fail(c, e, "primary kernel");
  for (const Arg* a : {&an, &aa, &ad, &at, &au})
    if ((r = copy_back(c, *a))) return r;
  return finish(c, all_device({&an, &aa, &ad, &at, &au}));
}

int rtx_render_aov(rtx_context* c, const float* cam, int W, int H, float near_, float far_,
                   float* n_out, float* a_out, float* d_out) {
  return primary_pass(c, cam, W, H, 1, near_, far_, n_out, a_out, d_out, nullptr, nullptr);
}

int rtx_primary_hits(rtx_context* c, const float* cam, int W, int H, int32_t* tri, float* tuv) {
  return primary_pass(c, cam, W, H, 2, 0.0f, 1.0f, nullptr, nullptr, nullptr, tri, tuv);
}

int rtx_intersect(rtx_context* c, int n, const float* rays, const int32_t* exclude,
                  int32_t* tri_out, float* tuv_out) {
  if (!c) return RTX_ERR_INVALID;
  if (n < 0) return fail(c, RTX_ERR_INVALID, "negative ray count");
  if (!c->has_scene) return fail(c, RTX_ERR_NO_SCENE, "no scene uploaded");
  if (n == 0) return RTX_OK;
  if (!rays || !tri_out || !tuv_out) return fail(c, RTX_ERR_INVALID, "NULL buffer");
  int r;
  if ((r = begin(c))) return r;
  Arg ar, ae, at, au;
  if ((r = bind_in(c, rays, (size_t)n * 24, 0, ar))) return r;
  if ((r = bind_in(c, exclude, exclude ? (size_t)n * 4 : 0, 1, ae))) return r;
  if ((r = bind_out(c, tri_out, (size_t)n * 4, 2, at))) return r;
  if ((r = bind_out(c, tuv_out, (size_t)n * 12, 3, au))) return r;
  int launches = 0;
  cudaError_t e = launch_intersect(c->ds, n, (const float*)ar.dev, (const int*)ae.dev,
                                   (int*)at.dev, (float*)au.dev, c->d_err, c->stream, &launches);
  c->stats.kernel_launches = launches;
  if (e != cudaSuccess) return cuda_fail(c, e, "intersect kernel");
  if ((r = copy_back(c, at))) return r;
  if ((r = copy_back(c, au))) return r;
  return finish(c, all_device({&ar, &ae, &at, &au}));
}

static int check_bsdf_args(rtx_context* c, int n, const float* mats, const float* eta,
                           const float* N, const float* dir) {
  if (!c) return RTX_ERR_INVALID;
  if (n < 0 || n > (1 << 26)) return fail(c, RTX_ERR_INVALID, "case count out of range");
  if (n > 0 && (!mats || !eta || !N || !dir)) return fail(c, RTX_ERR_INVALID, "NULL buffer");
  // material records are read as float4 vectors
  if (n > 0 && is_device_ptr(mats) && ((uintptr_t)mats & 15))
    return fail(c, RTX_ERR_INVALID, "device material array not 16-byte aligned");
  return RTX_OK;
}

int rtx_bsdf_eval(rtx_context* c, int n, const float* mats, const float* eta, const float* N,
                  const float* V, const float* L, float* out_f, float* out_pdf) {
  int r;
  if ((r = check_bsdf_args(c, n, mats, eta, N, V))) return r;
  if (n > 0 && (!L || !out_f || !out_pdf)) return fail(c, RTX_ERR_INVALID, "NULL buffer");
  if (n == 0) return RTX_OK;
  if ((r = begin(c))) return r;
  Arg am, ae, an, av, al, af, ap;
  if ((r = bind_in(c, mats, (size_t)n * 96, 0, am))) return r;
  if ((r = bind_in(c, eta, (size_t)n * 4, 1, ae))) return r;
  if ((r = bind_in(c, N, (size_t)n * 12, 2, an))) return r;
  if ((r = bind_in(c, V, (size_t)n * 12, 3, av))) return r;
  if ((r = bind_in(c, L, (size_t)n * 12, 4, al))) return r;
  if ((r = bind_out(c, out_f, (size_t)n * 12, 5, af))) return r;
  if ((r = bind_out(c, out_pdf, (size_t)n * 4, 6, ap))) return r;
  cudaError_t e = launch_bsdf_eval(n, (const float*)am.dev, (const float*)ae.dev, (const float*)an.dev,
                                   (const float*)av.dev, (const float*)al.dev, (float*)af.dev,
                                   (float*)ap.dev, c->stream);
  c->stats.kernel_launches = 1;
  if (e != cudaSuccess) return cuda_fail(c, e, "bsdf eval kernel");
  if ((r = copy_back(c, af))) return r;
  if ((r = copy_back(c, ap))) return r;
  return finish(c, all_device({&am, &ae, &an, &av, &al, &af, &ap}));
}

int rtx_bsdf_sample(rtx_context* c, int n, const float* mats, const float* eta, const float* N,
                    const float* in_dir, uint64_t seed, int sample, int32_t* out_ok,
                    float* out_dir, float* out_color, float* out_pdf) {
  int r;
  if ((r = check_bsdf_args(c, n, mats, eta, N, in_dir))) return r;
  if (n > 0 && (!out_ok || !out_dir || !out_color || !out_pdf))
    return fail(c, RTX_ERR_INVALID, "NULL buffer");
  if (n == 0) return RTX_OK;
  if ((r = begin(c))) return r;
  Arg am, ae, an, ai, ao, ad, ac, ap;
  if ((r = bind_in(c, mats, (size_t)n * 96, 0, am))) return r;
  if ((r = bind_in(c, eta, (size_t)n * 4, 1, ae))) return r;
  if ((r = bind_in(c, N, (size_t)n * 12, 2, an))) return r;
  if ((r = bind_in(c, in_dir, (size_t)n * 12, 3, ai))) return r;
  if ((r = bind_out(c, out_ok, (size_t)n * 4, 4, ao))) return r;
  if ((r = bind_out(c, out_dir, (size_t)n * 12, 5, ad))) return r;
  if ((r = bind_out(c, out_color, (size_t)n * 12, 6, ac))) return r;
  if ((r = bind_out(c, out_pdf, (size_t)n * 4, 7, ap))) return r;
  cudaError_t e = launch_bsdf_sample(n, (const float*)am.dev, (const float*)ae.dev,
                                     (const float*)an.dev, (const float*)ai.dev, seed, sample,
                                     (int*)ao.dev, (float*)ad.dev, (float*)ac.dev, (float*)ap.dev,
                                     c->stream);
  c->stats.kernel_launches = 1;
  if (e != cudaSuccess) return cuda_fail(c, e, "bsdf sample kernel");
  for (const Arg* a : {&ao, &ad, &ac, &ap})
    if ((r = copy_back(c, *a))) return r;
  return finish(c, all_device({&am, &ae, &an, &ai, &ao, &ad, &ac, &ap}));
}

int rtx_probe_read_bandwidth(rtx_context* c, size_t bytes, int passes, double* gbs) {
  if (!c) return RTX_ERR_INVALID;
  if (!gbs || passes < 1 || passes > 100000 || bytes < 4096 || bytes > ((size_t)1 << 34) || (bytes & 15))
    return fail(c, RTX_ERR_INVALID, "bad probe size");
  int r;
  if ((r = begin(c))) return r;
  int sms = 0;
  RTX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device), "attribute");
  RTX_CUDA(c->stage[0].ensure(bytes), "probe buffer");
  RTX_CUDA(c->stage[1].ensure(1024), "probe sink");
  RTX_CUDA(cudaMemsetAsync(c->stage[0].p, 0x5a, bytes, c->stream), "memset");
  // one pass first, so that an L2-sized buffer is resident when timing starts
  RTX_CUDA(launch_read_probe(c->stage[0].p, bytes, 1, (uint32_t*)c->stage[1].p, sms, c->stream),
           "probe kernel");
  RTX_CUDA(cudaEventRecord(c->ev0, c->stream), "cudaEventRecord");
  RTX_CUDA(launch_read_probe(c->stage[0].p, bytes, passes, (uint32_t*)c->stage[1].p, sms, c->stream),
           "probe kernel");
  RTX_CUDA(cudaEventRecord(c->ev1, c->stream), "cudaEventRecord");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  float ms = 0.0f;
  RTX_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "cudaEventElapsedTime");
  c->stats.last_gpu_ms = ms;
  c->stats.kernel_launches = 2;
  *gbs = (double)bytes * passes / (ms * 1e-3) / 1e9;
  return RTX_OK;
}

int rtx_selftest_wait_timeout(rtx_context* c, int polls) {
  if (!c) return RTX_ERR_INVALID;
  if (polls < 1 || polls > (1 << 20)) return fail(c, RTX_ERR_INVALID, "polls must be in [1, 2^20]");
  int r;
  if ((r = begin(c))) return r;
  RTX_CUDA(launch_wait_timeout(polls, c->d_err, c->stream), "wait kernel");
  c->stats.kernel_launches = 1;
  return finish(c, false);
}

// Bind an image input; when it aliases the output (the reference filters in
// place) it is first copied so that no kernel reads what it writes.
static int bind_image_in(rtx_context* c, const float* in, float* out, size_t bytes, int slot,
                         Arg& a) {
  int r;
  if ((r = bind_in(c, in, bytes, slot, a))) return r;
  if (a.dev == out) {
    RTX_CUDA(c->stage[slot].ensure(bytes), "stage alloc");
    RTX_CUDA(cudaMemcpyAsync(c->stage[slot].p, in, bytes, cudaMemcpyDeviceToDevice, c->stream), "copy");
    a.dev = c->stage[slot].p;
  }
  return RTX_OK;
}

static int check_image(rtx_context* c, const float* in, float* out, int W, int H) {
  if (!c) return RTX_ERR_INVALID;
  if (!in || !out) return fail(c, RTX_ERR_INVALID, "NULL image");
  if (W <= 0 || H <= 0) return fail(c, RTX_ERR_INVALID, "image size must be positive");
  if ((long long)W * H > (1LL << 30)) return fail(c, RTX_ERR_INVALID, "image too large");
  if (H > 65535) return fail(c, RTX_ERR_INVALID, "image taller than 65535 rows");
  return RTX_OK;
}

int rtx_image_convolve(rtx_context* c, const float* in, float* out, int W, int H,
                       const float* kernel, int kr, int kc, int normalize, int length,
                       int absval) {
  int r;
  if ((r = check_image(c, in, out, W, H))) return r;
  if (!kernel || kr <= 0 || kc <= 0 || (long long)kr * kc > (1 << 20))
    return fail(c, RTX_ERR_INVALID, "bad kernel");
  size_t bytes = (size_t)W * H * 12;
  if ((r = begin(c))) return r;
  Arg ai, ao;
  if ((r = bind_out(c, out, bytes, 1, ao))) return r;
  if ((r = bind_image_in(c, in, (float*)ao.dev, bytes, 0, ai))) return r;
  if ((r = upload_weights(c, kernel, (size_t)kr * kc))) return r;
  int flags = (absval ? 1 : 0) | (length ? 2 : 0) | (normalize ? 4 : 0);
  int launches = 0;
  cudaError_t e = launch_convolve((const float*)ai.dev, (float*)ao.dev, W, H,
                                  (const float*)c->weights.p, kr, kc, flags, c->compositor_fma, c->stream,
                                  &launches);
  c->stats.kernel_launches = launches;
  if (e != cudaSuccess) return cuda_fail(c, e, "convolve kernel");
  if ((r = copy_back(c, ao))) return r;
  return finish(c, all_device({&ai, &ao}));
}

static int gaussian_common(rtx_context* c, const float* in, float* out, int W, int H, int size,
                           float sigma, bool bloom, float threshold) {
  int r;
  if ((r = check_image(c, in, out, W, H))) return r;
  if (size <= 0 || size > (1 << 16)) return fail(c, RTX_ERR_INVALID, "bad kernel size");
  size_t bytes = (size_t)W * H * 12;
  if ((r = begin(c))) return r;
  Arg ai, ao;
  if ((r = bind_out(c, out, bytes, 1, ao))) return r;
  if ((r = bind_image_in(c, in, (float*)ao.dev, bytes, 0, ai))) return r;
  std::vector<float> w(size);
  gaussian_weights(size, sigma, w.data());
  if ((r = upload_weights(c, w.data(), w.size()))) return r;
  RTX_CUDA(c->stage[2].ensure(bytes), "stage alloc");
  if (bloom) RTX_CUDA(c->stage[3].ensure(bytes), "stage alloc");
  int launches = 0;
  cudaError_t e = launch_gaussian((const float*)ai.dev, (float*)c->stage[2].p,
                                  bloom ? (float*)c->stage[3].p : nullptr, (float*)ao.dev, W, H,
                                  (const float*)c->weights.p, size, bloom ? 1 : 0, threshold,
                                  c->compositor_fma, c->stream, &launches);
  c->stats.kernel_launches = launches;
  if (e != cudaSuccess) return cuda_fail(c, e, "gaussian kernels");
  if ((r = copy_back(c, ao))) return r;
  return finish(c, all_device({&ai, &ao}));
}

int rtx_image_gaussian_blur(rtx_context* c, const float* in, float* out, int W, int H, int size,
                            float sigma) {
  return gaussian_common(c, in, out, W, H, size, sigma, false, 0.0f);
}

int rtx_image_bloom(rtx_context* c, const float* in, float* out, int W, int H, int size,
                    float sigma, float threshold) {
  return gaussian_common(c, in, out, W, H, size, sigma, true, threshold);
}

int rtx_nn_gemm_bf16(rtx_context* c, int M, int N, int K, const void* A, const void* B, float* C,
                     int a_mn, int b_mn) {
  if (!c) return RTX_ERR_INVALID;
  if (M <= 0 || N <= 0 || K <= 0) return fail(c, RTX_ERR_INVALID, "M, N, K must be positive");
  if ((a_mn ? M : K) % 8 || (b_mn ? N : K) % 8)
    return fail(c, RTX_ERR_INVALID, "the contiguous dimension of each operand must be a multiple of 8");
  if (!A || !B || !C) return fail(c, RTX_ERR_INVALID, "NULL operand");
  int r;
  if ((r = begin(c))) return r;
  Arg aa, ab, ac;
  if ((r = bind_in(c, A, (size_t)M * K * 2, 0, aa))) return r;
  if ((r = bind_in(c, B, (size_t)N * K * 2, 1, ab))) return r;
  if ((r = bind_out(c, C, (size_t)M * N * 4, 2, ac))) return r;
  cudaError_t e = launch_gemm_bf16(aa.dev, ab.dev, (float*)ac.dev, M, N, K, a_mn, b_mn, c->d_err, c->stream);
  c->stats.kernel_launches = 1;
  if (e != cudaSuccess) return cuda_fail(c, e, "gemm kernel");
  if ((r = copy_back(c, ac))) return r;
  return finish(c, all_device({&aa, &ab, &ac}));
}

// ---- denoiser operators ------------------------------------------------------
static int check_conv_srcs(rtx_context* c, int N, int H, int W, const void* x1, int C1, int up1,
                           const void* x2, int C2) {
  if (N <= 0 || H <= 0 || W <= 0) return fail(c, RTX_ERR_INVALID, "N, H, W must be positive");
  if ((long long)N * H * W > (1LL << 31)) return fail(c, RTX_ERR_INVALID, "tensor too large");
  if (!x1 || C1 <= 0 || C1 % 8) return fail(c, RTX_ERR_INVALID, "x1 must be given with C1 a multiple of 8");
  if (C2 < 0 || C2 % 8 || (C2 > 0) != (x2 != nullptr))
    return fail(c, RTX_ERR_INVALID, "x2 must be given exactly when C2 > 0, C2 a multiple of 8");
  if (up1 && (H % 2 || W % 2)) return fail(c, RTX_ERR_INVALID, "an upsampled source needs even H and W");
  return RTX_OK;
}

static int bind_srcs(rtx_context* c, int N, int H, int W, const void* x1, int C1, int up1, const void* x2,
                     int C2, int slot, Arg& a1, Arg& a2, rtx::nn::Src& s1, rtx::nn::Src& s2) {
  int r;
  size_t p1 = up1 ? (size_t)N * (H / 2) * (W / 2) : (size_t)N * H * W;
  if ((r = bind_in(c, x1, p1 * C1 * 2, slot, a1))) return r;
  if ((r = bind_in(c, x2, (size_t)N * H * W * C2 * 2, slot + 1, a2))) return r;
  s1 = rtx::nn::Src{(const rtx::nn::bf16*)a1.dev, C1, up1 ? 1 : 0};
  s2 = rtx::nn::Src{(const rtx::nn::bf16*)a2.dev, C2, 0};
  return RTX_OK;
}

int rtx_nn_conv3x3_fwd(rtx_context* c, int N, int H, int W, const void* x1, int C1, int up1,
                       const void* x2, int C2, const void* w, const float* bias, int Cout, int relu,
                       float* out) {
  if (!c) return RTX_ERR_INVALID;
  int r;
  if ((r = check_conv_srcs(c, N, H, W, x1, C1, up1, x2, C2))) return r;
  if (Cout <= 0 || Cout % 16 || Cout > 256) return fail(c, RTX_ERR_INVALID, "Cout must be a multiple of 16, <= 256");
  if (!w || !out) return fail(c, RTX_ERR_INVALID, "NULL weight or output");
  const int Cin = C1 + C2;
  const size_t P = (size_t)N * H * W;
  if ((r = begin(c))) return r;
  Arg a1, a2, aw, ab, ao;
  rtx::nn::Src s1, s2;
  if ((r = bind_srcs(c, N, H, W, x1, C1, up1, x2, C2, 0, a1, a2, s1, s2))) return r;
  if ((r = bind_in(c, w, (size_t)Cout * 9 * Cin * 2, 2, aw))) return r;
  if ((r = bind_in(c, bias, bias ? (size_t)Cout * 4 : 0, 3, ab))) return r;
  if ((r = bind_out(c, out, P * Cout * 4, 4, ao))) return r;
  rtx::nn::ConvFwd a{};
  a.s1 = s1;
  a.s2 = s2;
  a.N = N;
  a.H = H;
  a.W = W;
  a.Cin = Cin;
  a.Cout = Cout;
  a.w = (const rtx::nn::bf16*)aw.dev;
  a.bias = (const float*)ab.dev;
  a.relu = relu;
  a.out = nullptr;
  a.out_f32 = (float*)ao.dev;
  a.err = c->d_err;
  cudaError_t e = rtx::nn::conv_fwd(a, c->stream);
  c->stats.kernel_launches = 1;
  if (e != cudaSuccess) return cuda_fail(c, e, "conv forward kernel");
  if ((r = copy_back(c, ao))) return r;
  return finish(c, all_device({&a1, &a2, &aw, &ab, &ao}));
}

int rtx_nn_conv3x3_dgrad(rtx_context* c, int N, int H, int W, const void* dout, int Cout, const void* wt,
                         const void* x1, int C1, int up1, const void* x2, int C2, int mask_relu,
                         void* din) {
  if (!c) return RTX_ERR_INVALID;
  int r;
  if ((r = check_conv_srcs(c, N, H, W, x1, C1, up1, x2, C2))) return r;
  const int Cin = C1 + C2;
  if (Cin % 16) return fail(c, RTX_ERR_INVALID, "C1 + C2 must be a multiple of 16");
  if (Cout <= 0 || Cout % 8) return fail(c, RTX_ERR_INVALID, "Cout must be a positive multiple of 8");
  if (!dout || !wt || !din) return fail(c, RTX_ERR_INVALID, "NULL gradient, weight or output");
  const size_t P = (size_t)N * H * W;
  if ((r = begin(c))) return r;
  Arg a1, a2, ad, aw, ao;
  rtx::nn::Src s1, s2;
  if ((r = bind_srcs(c, N, H, W, x1, C1, up1, x2, C2, 0, a1, a2, s1, s2))) return r;
  if ((r = bind_in(c, dout, P * Cout * 2, 2, ad))) return r;
  if ((r = bind_in(c, wt, (size_t)Cin * 9 * Cout * 2, 3, aw))) return r;
  if ((r = bind_out(c, din, P * Cin * 2, 4, ao))) return r;
  rtx::nn::ConvDgrad a{};
  a.dout = (const rtx::nn::bf16*)ad.dev;
  a.Cout = Cout;
  a.wt = (const rtx::nn::bf16*)aw.dev;
  a.N = N;
  a.H = H;
  a.W = W;
  a.Cin = Cin;
  a.s1 = s1;
  a.s2 = s2;
  a.mask_relu = mask_relu;
  a.din = (rtx::nn::bf16*)ao.dev;
  a.err = c->d_err;
  cudaError_t e = rtx::nn::conv_dgrad(a, c->stream);
  c->stats.kernel_launches = 1;
  if (e != cudaSuccess) return cuda_fail(c, e, "conv data-gradient kernel");
  if ((r = copy_back(c, ao))) return r;
  return finish(c, all_device({&a1, &a2, &ad, &aw, &ao}));
}

int rtx_nn_conv3x3_wgrad(rtx_context* c, int N, int H, int W, const void* dout, int Cout, const void* x1,
                         int C1, int up1, const void* x2, int C2, float* dw) {
  if (!c) return RTX_ERR_INVALID;
  int r;
  if ((r = check_conv_srcs(c, N, H, W, x1, C1, up1, x2, C2))) return r;
  if (Cout <= 0 || Cout % 16 || Cout > 256)
    return fail(c, RTX_ERR_INVALID, "Cout must be a multiple of 16, <= 256");
  if (!dout || !dw) return fail(c, RTX_ERR_INVALID, "NULL gradient or output");
  const int Cin = C1 + C2;
  const long long P = (long long)N * H * W;
  if ((r = begin(c))) return r;
  Arg a1, a2, ad, ao;
  rtx::nn::Src s1, s2;
  if ((r = bind_srcs(c, N, H, W, x1, C1, up1, x2, C2, 0, a1, a2, s1, s2))) return r;
  if ((r = bind_in(c, dout, (size_t)P * Cout * 2, 2, ad))) return r;
  if ((r = bind_out(c, dw, (size_t)Cout * 9 * Cin * 4, 4, ao))) return r;
  RTX_CUDA(cudaMemsetAsync(ao.dev, 0, ao.bytes, c->stream), "zero dw");
  rtx::nn::ConvWgrad a{};
  a.dout = (const rtx::nn::bf16*)ad.dev;
  a.Cout = Cout;
  a.s1 = s1;
  a.s2 = s2;
  a.N = N;
  a.H = H;
  a.W = W;
  a.Cin = Cin;
  a.pix_per_cta = rtx::nn::wgrad_pixels_per_cta(P, Cout, Cin);
  a.dw = (float*)ao.dev;
  a.err = c->d_err;
  cudaError_t e = rtx::nn::conv_wgrad(a, c->stream);
  c->stats.kernel_launches = 1;
  if (e != cudaSuccess) return cuda_fail(c, e, "conv weight-gradient kernel");
  if ((r = copy_back(c, ao))) return r;
  return finish(c, all_device({&a1, &a2, &ad, &ao}));
}

// ---- denoiser ------------------------------------------------------------------
static int need_dn(rtx_context* c) {
  if (!c) return RTX_ERR_INVALID;
  if (!c->dn) return fail(c, RTX_ERR_INVALID, "denoiser not initialised (rtx_dn_init)");
  return RTX_OK;
}

static int check_batch(rtx_context* c, int N, int H, int W) {
  if (N <= 0 || H <= 0 || W <= 0) return fail(c, RTX_ERR_INVALID, "N, H, W must be positive");
  if (H % 16 || W % 16) return fail(c, RTX_ERR_INVALID, "H and W must be multiples of 16");
  if ((long long)N * H * W > (1LL << 28)) return fail(c, RTX_ERR_INVALID, "batch too large");
  return RTX_OK;
}

int rtx_dn_init(rtx_context* c, uint64_t seed) {
  if (!c) return RTX_ERR_INVALID;
  RTX_CUDA(cudaSetDevice(c->device), "cudaSetDevice");
  delete c->dn;
  c->dn = new (std::nothrow) rtx::nn::UNet();
  if (!c->dn) return fail(c, RTX_ERR_NOMEM, "host allocation");
  cudaError_t e = c->dn->init(seed, c->stream);
  if (e != cudaSuccess) {
    delete c->dn;
    c->dn = nullptr;
    return cuda_fail(c, e, "denoiser init");
  }
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  return RTX_OK;
}

int rtx_dn_info(rtx_context* c, int64_t* n_params, int64_t* n_real, int* n_layers, int* step) {
  int r;
  if ((r = need_dn(c))) return r;
  if (n_params) *n_params = c->dn->num_params();
  if (n_real) *n_real = c->dn->num_real_params();
  if (n_layers) *n_layers = rtx::nn::UNet::num_layers();
  if (step) *step = c->dn->step();
  return RTX_OK;
}

int rtx_dn_layer(rtx_context* c, int layer, int64_t info[11]) {
  int r;
  if ((r = need_dn(c))) return r;
  if (layer < 0 || layer >= rtx::nn::UNet::num_layers() || !info)
    return fail(c, RTX_ERR_INVALID, "layer out of range");
  c->dn->layer_info(layer, info);
  return RTX_OK;
}

int rtx_dn_get_params(rtx_context* c, float* out) {
  int r;
  if ((r = need_dn(c))) return r;
  if (!out || is_device_ptr(out)) return fail(c, RTX_ERR_INVALID, "out must be a host buffer");
  RTX_CUDA(c->dn->get_params(out, c->stream), "get params");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  return RTX_OK;
}

int rtx_dn_set_params(rtx_context* c, const float* in) {
  int r;
  if ((r = need_dn(c))) return r;
  if (!in || is_device_ptr(in)) return fail(c, RTX_ERR_INVALID, "in must be a host buffer");
  RTX_CUDA(c->dn->set_params(in, c->stream), "set params");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  return RTX_OK;
}

int rtx_dn_get_grads(rtx_context* c, float* out) {
  int r;
  if ((r = need_dn(c))) return r;
  if (!out || is_device_ptr(out)) return fail(c, RTX_ERR_INVALID, "out must be a host buffer");
  RTX_CUDA(c->dn->get_grads(out, c->stream), "get grads");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  return RTX_OK;
}

int rtx_dn_get_adam(rtx_context* c, float* m, float* v) {
  int r;
  if ((r = need_dn(c))) return r;
  if (!m || !v || is_device_ptr(m) || is_device_ptr(v))
    return fail(c, RTX_ERR_INVALID, "m and v must be host buffers");
  RTX_CUDA(c->dn->get_state(m, v, c->stream), "get Adam state");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  return RTX_OK;
}

int rtx_dn_set_adam(rtx_context* c, const float* m, const float* v, int step) {
  int r;
  if ((r = need_dn(c))) return r;
  if (!m || !v || is_device_ptr(m) || is_device_ptr(v))
    return fail(c, RTX_ERR_INVALID, "m and v must be host buffers");
  if (step < 0) return fail(c, RTX_ERR_INVALID, "step must be >= 0");
  RTX_CUDA(c->dn->set_state(m, v, step, c->stream), "set Adam state");
  RTX_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  return RTX_OK;
}

static int dn_run(rtx_context* c, const float* input, const float* target, int N, int H, int W, bool update,
                  float lr, double* loss) {
  int r;
  if ((r = need_dn(c))) return r;
  if ((r = check_batch(c, N, H, W))) return r;
  if (!input || !target) return fail(c, RTX_ERR_INVALID, "NULL input or target");
  const size_t P = (size_t)N * H * W;
  if ((r = begin(c))) return r;
  Arg ai, at;
  if ((r = bind_in(c, input, P * 4 * rtx::nn::kRawCh, 0, ai))) return r;
  if ((r = bind_in(c, target, P * 12, 1, at))) return r;
  RTX_CUDA(c->dn->reserve((long long)P), "denoiser buffers");
  double l = 0.0;
  cudaError_t e = update ? c->dn->train_step((const float*)ai.dev, (const float*)at.dev, N, H, W, lr, &l,
                                             c->d_err, c->stream)
                         : c->dn->loss_and_grads((const float*)ai.dev, (const float*)at.dev, N, H, W, &l,
                                                 c->d_err, c->stream);
  c->stats.kernel_launches = c->dn->last_launches();
  if (e != cudaSuccess) return cuda_fail(c, e, update ? "denoiser train step" : "denoiser gradients");
  if ((r = finish(c, false))) return r;
  if (loss) *loss = l;
  return RTX_OK;
}

int rtx_dn_loss_grads(rtx_context* c, const float* input, const float* target, int N, int H, int W,
                      double* loss) {
  return dn_run(c, input, target, N, H, W, false, 0.0f, loss);
}

int rtx_dn_train_step(rtx_context* c, const float* input, const float* target, int N, int H, int W, float lr,
                      double* loss) {
  if (c && !(lr > 0.0f)) return fail(c, RTX_ERR_INVALID, "lr must be positive");
  return dn_run(c, input, target, N, H, W, true, lr, loss);
}

int rtx_dn_infer(rtx_context* c, const float* input, float* out, int N, int H, int W) {
  int r;
  if ((r = need_dn(c))) return r;
  if ((r = check_batch(c, N, H, W))) return r;
  if (!input || !out) return fail(c, RTX_ERR_INVALID, "NULL input or output");
  const size_t P = (size_t)N * H * W;
  if ((r = begin(c))) return r;
  Arg ai, ao;
  if ((r = bind_in(c, input, P * 4 * rtx::nn::kRawCh, 0, ai))) return r;
  if ((r = bind_out(c, out, P * 12, 1, ao))) return r;
  RTX_CUDA(c->dn->reserve((long long)P), "denoiser buffers");
  cudaError_t e = c->dn->forward((const float*)ai.dev, N, H, W, c->d_err, c->stream);
  if (e == cudaSuccess) e = c->dn->decode((const float*)ai.dev, (float*)ao.dev, N, H, W, H, W, c->stream);
  c->stats.kernel_launches = c->dn->last_launches() + 1;
  if (e != cudaSuccess) return cuda_fail(c, e, "denoiser inference");
  if ((r = copy_back(c, ao))) return r;
  return finish(c, all_device({&ai, &ao}));
}

int rtx_denoise(rtx_context* c, const float* radiance, const float* albedo, const float* normal,
                const float* depth, int spp, float* out, int W, int H) {
  int r;
  if ((r = need_dn(c))) return r;
  if (W <= 0 || H <= 0 || (long long)W * H > (1LL << 28)) return fail(c, RTX_ERR_INVALID, "bad image size");
  if (!radiance || !albedo || !normal || !depth || !out) return fail(c, RTX_ERR_INVALID, "NULL image");
  if (spp < 1) return fail(c, RTX_ERR_INVALID, "spp must be >= 1");
  const int Wp = (W + 15) / 16 * 16, Hp = (H + 15) / 16 * 16;
  const size_t bytes = (size_t)W * H * 12;
  if ((r = begin(c))) return r;
  Arg ar, aa, an, ad, ao;
  if ((r = bind_in(c, radiance, bytes, 0, ar))) return r;
  if ((r = bind_in(c, albedo, bytes, 1, aa))) return r;
  if ((r = bind_in(c, normal, bytes, 2, an))) return r;
  if ((r = bind_in(c, depth, bytes, 3, ad))) return r;
  if ((r = bind_out(c, out, bytes, 4, ao))) return r;
  RTX_CUDA(c->stage[5].ensure((size_t)Wp * Hp * 4 * rtx::nn::kRawCh), "stage alloc");
  RTX_CUDA(c->dn->reserve((long long)Wp * Hp), "denoiser buffers");
  float* raw = (float*)c->stage[5].p;
  cudaError_t e = rtx::nn::pack_passes((const float*)ar.dev, (const float*)aa.dev, (const float*)an.dev,
                                       (const float*)ad.dev, (float)spp, raw, W, H, Wp, Hp, c->stream);
  if (e == cudaSuccess) e = c->dn->forward(raw, 1, Hp, Wp, c->d_err, c->stream);
  if (e == cudaSuccess) e = c->dn->decode(raw, (float*)ao.dev, 1, H, W, Hp, Wp, c->stream);
  c->stats.kernel_launches = c->dn->last_launches() + 2;
  if (e != cudaSuccess) return cuda_fail(c, e, "denoise");
  if ((r = copy_back(c, ao))) return r;
  return finish(c, all_device({&ar, &aa, &an, &ad, &ao}));
}

int rtx_image_edge_detect(rtx_context* c, const float* in, float* out, int W, int H) {
  int r;
  if ((r = check_image(c, in, out, W, H))) return r;
  size_t bytes = (size_t)W * H * 12;
  if ((r = begin(c))) return r;
  Arg ai, ao;
  if ((r = bind_out(c, out, bytes, 1, ao))) return r;
  if ((r = bind_image_in(c, in, (float*)ao.dev, bytes, 0, ai))) return r;
  int launches = 0;
  cudaError_t e = launch_edge((const float*)ai.dev, (float*)ao.dev, W, H, c->stream, &launches);
  c->stats.kernel_launches = launches;
  if (e != cudaSuccess) return cuda_fail(c, e, "edge kernel");
  if ((r = copy_back(c, ao))) return r;
  return finish(c, all_device({&ai, &ao}));
}

}  // extern "C"
