// rtx_internal.h — librtx internals shared by the host API (api.cpp), the BVH
// builder (bvh_build.cpp) and the CUDA kernels (*.cu).
//
// Scene layout in HBM (all arrays 16-byte aligned, read through the
// non-coherent cache with 16-byte vector loads):
//   nodes   : binary BVH, 4 x float4 = 64 B per inner node:
//             [0] c0.lo.x c0.hi.x c0.lo.y c0.hi.y
//             [1] c1.lo.x c1.hi.x c1.lo.y c1.hi.y
//             [2] c0.lo.z c0.hi.z c1.lo.z c1.hi.z
//             [3] child0 child1 (int bits; >= 0 inner node, < 0 leaf ref)
//             leaf ref = ~((first_tri << 3) | (count - 1)), count 1..8
//   tris    : leaf-ordered triangles, 3 x float4 = 48 B each:
//             (v0.xyz, triangle id) (e1.xyz, 0) (e2.xyz, 0)
//             e1 = v1 - v0, e2 = v2 - v0 (Triangle::v0v1_w / v0v2_w)
//   shade   : per triangle id, 4 x float4 = 64 B:
//             (flat normal.xyz, area) (n0.xyz, info) (n1.xyz, 0) (n2.xyz, 0)
//             info = material index | 0x80000000 when the mesh is smooth
//   nodes4  : the same tree collapsed to 4 children per node, 7 x float4 =
//             112 B per node: lo.x[4] hi.x[4] lo.y[4] hi.y[4] lo.z[4] hi.z[4]
//             and the four child refs (int bits, as above); an unused slot
//             holds a degenerate box at 1e30 that no ray reaches before 1e7
//   geo     : per triangle id, 3 x float4 (v0, e1, e2): emitter sampling
//   mats    : 24 floats per material; emitters: triangle ids.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/rtx.h"

namespace rtx {

constexpr int kMaxLeaf = 8;
constexpr int kStackSize = 64;
constexpr int kEmptyRoot = -2147483647 - 1;  // INT_MIN: scene without triangles

// Device error word bits (set by kernels, read back by the host)
enum DeviceError : int {
  kErrStackOverflow = 1,
  kErrQueueOverflow = 2,
  kErrBadIndex = 4,
};

// A 4-wide node: six float4 of child planes (min x, max x, min y, max y,
// min z, max z of the four children), then one float4 of child references
// (112 B; padding nodes to one aligned 128-byte line measured 5 % slower
// traversal: the larger tree fits the L2 less well).
constexpr int kNode4Vecs = 7;

// Principled-BSDF lobes a scene's materials use beyond diffuse and specular
// reflection (DeviceScene::lobes)
#ifndef RTX_LOBE_BITS
#define RTX_LOBE_BITS
constexpr int kLobeTrans = 1, kLobeCoat = 2, kLobeAll = 3;
#endif
// kLobeTrans when some record (24 floats) has spec_trans (float 15) != 0,
// kLobeCoat when some has clearcoat (float 13) != 0; NaN counts as nonzero
inline int material_lobes(const float* mats, int n) {
  int r = 0;
  for (int m = 0; m < n; ++m) {
    if (!(mats[24 * (size_t)m + 15] == 0.0f)) r |= kLobeTrans;
    if (!(mats[24 * (size_t)m + 13] == 0.0f)) r |= kLobeCoat;
  }
  return r;
}

// The ray sort's origin grids over a scene: its bounds' low corner and the
// cells per unit length of the 4^3 and 16^3 grids; ok = 0 when the tree has
// no inner root (every key 0)
struct SortKeyBounds {
  float lo[3] = {0.0f, 0.0f, 0.0f}, inv4[3] = {0.0f, 0.0f, 0.0f}, inv16[3] = {0.0f, 0.0f, 0.0f};
  int ok = 0;
};

struct DeviceScene {
  const float4* __restrict__ nodes;
  const float4* __restrict__ nodes4;
  int root4;  // root of nodes4 (>= 0), a leaf ref (< 0) or kEmptyRoot
  const float4* __restrict__ tris;
  const float4* __restrict__ shade;
  const float4* __restrict__ geo;
  const float* __restrict__ mats;
  const int* __restrict__ emitters;
  const uint8_t* __restrict__ perm;  // 256-entry permutation of the Perlin texture
  int root;  // node index (>= 0), leaf ref (< 0) or kEmptyRoot
  int n_tris, n_emitters, n_mats;
  int textured;  // some material has a procedural texture
  int lobes;     // kLobeTrans: some material has spec_trans != 0; kLobeCoat: clearcoat != 0
  float sky[3], ground[3];
  // traversal stack entries a ray may use before it reports kErrStackOverflow
  // (kStackSize; lower only through RTX_OPT_STACK_LIMIT, to exercise that path)
  int stack_limit = kStackSize;
  SortKeyBounds keyb;  // the ray sort's origin grids over this scene
};

// Camera reduced to what ray generation needs (src/renderer.cpp:103-124,
// 252-259): the top three rows of the object-to-world matrix and the film
// half extents.
struct CamParams {
  float m[12];
  float top, right;
  float inv_w, inv_h;
  int W, H;
};

// Allocator of the BVH builder's arrays: sizing an array leaves its new
// elements uninitialised (the builder writes every one), so that sizing
// ~100 MB of output costs no pass of zero stores.
template <class T>
struct UninitAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = UninitAlloc<U>;
  };
  UninitAlloc() = default;
  template <class U>
  UninitAlloc(const UninitAlloc<U>&) noexcept {}
  template <class U>
  void construct(U* p) noexcept {
    ::new ((void*)p) U;
  }
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new ((void*)p) U(std::forward<A>(a)...);
  }
};
using Float4Array = std::vector<float4, UninitAlloc<float4>>;

struct BvhBuildResult {
  Float4Array nodes;   // 4 per node
  Float4Array nodes4;  // kNode4Vecs per 4-wide node
  Float4Array tris;    // 3 per triangle, leaf order
  int root = kEmptyRoot;
  int root4 = kEmptyRoot;
  int n_nodes = 0, n_nodes4 = 0, n_leaves = 0, depth = 0, depth4 = 0;
  double ms = 0.0;
};

// Host binned-SAH build over world-space triangles (verts: n x 9 floats) on
// `threads` threads (0: one per hardware thread, at most 64); the result is
// the same bits for every thread count.
BvhBuildResult build_bvh(const float* verts, int n, int max_leaf, int threads = 0);

// Host-side camera preparation, restating Renderer::PrepareScreenSpace
CamParams make_cam_params(const float* cam, int W, int H);

// Visit counters (RTX_OPT_COUNT_VISITS)
struct Counters {
  unsigned long long ext_node_visits;
  unsigned long long ext_tri_tests;
  unsigned long long sh_node_visits;
  unsigned long long sh_tri_tests;
  unsigned long long ext_rays;
  unsigned long long shadow_rays;
  unsigned long long ext_rays_by_depth[16];
};

// Per-kernel CUDA-event timing of a render (RTX_OPT_KERNEL_TIMING)
struct KernelTimer {
  std::vector<cudaEvent_t> pool;
  std::vector<std::pair<int, int>> marks;  // (kind, event index of the start)
  size_t used = 0;
  bool on = false;
  double ms[3] = {0, 0, 0};  // extend, shade, connect
  cudaError_t mark(int kind, cudaStream_t st, bool start);
  cudaError_t collect();  // after the stream is synchronised
  void reset() {
    used = 0;
    marks.clear();
    ms[0] = ms[1] = ms[2] = 0;
  }
  ~KernelTimer();
};

// ---- kernel launchers (implemented in the .cu files) ----------------------
cudaError_t launch_primary(const DeviceScene& s, const CamParams& cam, int mode,
                           float near_, float far_, float* normal, float* albedo,
                           float* depth, int* tri, float* tuv, int* err,
                           cudaStream_t st, int* launches);
cudaError_t launch_intersect(const DeviceScene& s, int n, const float* rays,
                             const int* exclude, int* tri, float* tuv, int* err,
                             cudaStream_t st, int* launches);

struct PtWorkspace;  // defined in pt_kernels.cu
// Display resolve of a radiance image: Image::Tonemap<kITURBT709>(limit)
// (include/RenderToy/compositor.h:220-226, rtmath.h:1142-1177), then
// Image::GammaCorrection(gamma) (src/compositor.cpp:94-100), then the
// exporters' quantisation int(255.99 * clamp(x, 0, 1)) (src/exporter.cpp).
// limit <= 0 skips the tonemap, ratio <= 0 the gamma (ratio = 1 / gamma).
struct Resolve {
  float limit, ratio;
  float* display;   // W x H RGB FP32 or nullptr
  uint8_t* bytes;   // quantised pixels or nullptr
  int format;       // 0: BMP pixel array (BGR rows of 4-byte multiples), 1: RGB in buffer order
  int W;
};
constexpr int kResolveBmp = 0, kResolveRgb = 1;
__host__ __device__ inline size_t bmp_row_bytes(int W) { return ((size_t)W * 3 + 3) & ~(size_t)3; }

// One frame of a multi-scene batch: a camera over one of the merged scenes.
// Paths of all frames share one index space: frame j owns
// [q_begin, q_begin + W * H * spp), sample-major like a single render, and
// pixels [pix_begin, pix_begin + W * H) of the concatenated output.  The
// random stream of each frame is the one rtx_render_pt would use for its
// scene, seed and camera, so a batched frame equals the frame rendered alone.
struct PtJob {
  long long q_begin, pix_begin;
  int npix, W, spp, first_sample;
  int root, root4, e_begin, n_emitters;
  uint32_t k0, k1;
  float sky[3], ground[3];
  CamParams cam;
  SortKeyBounds keyb;  // the frame's scene's ray sort grids
};

struct PtParams {
  int W, H, spp, first_sample, n_samples, max_depth;
  uint64_t seed;
  int wave_paths;  // paths per wave (<= capacity)
  int block;
  bool per_path;   // write L(p, s) instead of accumulating
  bool accumulate; // add the mean to the output instead of overwriting it
  bool count_visits;
  bool primary_cache;
  bool sort_material = false;  // counting-sort the shading queue by material
  bool sort_rays = false;      // counting-sort the extension queue by ray key
  bool overlap = false;        // a vertex's occlusion launch beside the next vertex's closest-hit launch
  int traversal;  // RTX_OPT_TRAVERSAL
  int min_busy;   // RTX_OPT_MIN_BUSY
  Resolve resolve;  // fused into the last accumulation when display or bytes is set
  // multi-scene batch (n_jobs > 0): device job table and its q_begin column,
  // the host copy for launch sizing; W, H, spp, n_samples, seed are unused
  int n_jobs = 0;
  const PtJob* d_jobs = nullptr;
  const long long* d_job_q = nullptr;
  const PtJob* h_jobs = nullptr;
};
PtWorkspace* pt_workspace_create();
long long pt_last_wave(const PtWorkspace* ws);
void pt_workspace_destroy(PtWorkspace* ws);
cudaError_t pt_render(PtWorkspace* ws, const DeviceScene& s, const CamParams& cam,
                      const PtParams& p, float* d_out, int* err, Counters* d_counters,
                      KernelTimer* timer, cudaStream_t st, int* launches, int* extend_launches,
                      int* vertex_launches, std::string* why);

cudaError_t launch_resolve(const float* in, int W, int H, const Resolve& r, cudaStream_t st);
// fma: each tap's multiply-add fused (RTX_OPT_COMPOSITOR_FMA) in the
// register-blocked kernels (3 x 3, 5 x 5, separable passes); false keeps the
// reference's separately rounded multiply and add
cudaError_t launch_convolve(const float* in, float* out, int W, int H, const float* d_k,
                            int kr, int kc, int flags, bool fma, cudaStream_t st, int* launches);
cudaError_t launch_gaussian(const float* in, float* tmp, float* tmp2, float* out, int W, int H,
                            const float* d_w, int size, int extract_mode, float threshold, bool fma,
                            cudaStream_t st, int* launches);
cudaError_t launch_edge(const float* in, float* out, int W, int H, cudaStream_t st,
                        int* launches);
cudaError_t launch_texture_sample(int kind, float param, const uint8_t* perm, int n, const float* uv,
                                  float* out, cudaStream_t st);
cudaError_t launch_bsdf_eval(int n, const float* mats, const float* eta, const float* N,
                             const float* V, const float* L, float* f, float* pdf, cudaStream_t st);
cudaError_t launch_bsdf_sample(int n, const float* mats, const float* eta, const float* N,
                               const float* in_dir, uint64_t seed, int sample, int* ok, float* dir,
                               float* color, float* pdf, cudaStream_t st);
cudaError_t launch_read_probe(const void* buf, size_t bytes, int passes, uint32_t* sink, int sms,
                              cudaStream_t st);
cudaError_t launch_wait_timeout(int polls, int* err, cudaStream_t st);
cudaError_t launch_gemm_bf16(const void* A, const void* B, float* C, int M, int N, int K, int a_mn,
                             int b_mn, int* err, cudaStream_t st);

}  // namespace rtx
