// pt_kernels.cu — wavefront path tracer restating RenderToy's
// PathTracingRenderer (src/renderer.cpp:236-384) for the GPU.
//
// The reference evaluates one path per recursion (Radiance, renderer.cpp:272)
// with the light sample of DirectLight (renderer.cpp:335) in the middle.  Here
// a wave of paths advances one vertex per step through four kernels:
//
//   raygen   primary ray of each (pixel, sample)            renderer.cpp:252-259
//   extend   closest hit of every live path                 renderer.cpp:282
//   shade    emission + MIS, light sample + BSDF Eval,      renderer.cpp:284-325
//            BSDF Sample -> next ray; emits a shadow record  renderer.cpp:341-371
//   connect  occlusion of each shadow record; adds the light renderer.cpp:352-379
//            contribution to its path
//   accumulate  image += L / spp in sample order            renderer.cpp:261
//
// Radiance is accumulated forward (sum over vertices of throughput x
// (emission + light)) instead of the reference's backward recursion; the two
// agree to rounding.  Paths live in structure-of-arrays float4 buffers in HBM
// (96 B per path); live paths and shadow records are compacted into queues with
// warp-aggregated atomics, and queue lengths stay on the device, so the host
// issues a fixed launch sequence per wave with no synchronisation.
// Traversal kernels run persistent warps that fetch 32 rays at a time; with
// RTX_OPT_SORT_RAYS (the default) they visit the extension rays and the
// shadow records in ray-key order (origin cell, direction cell), while the
// shading kernel keeps the path order (see the ray-sort section below).
#include <algorithm>

#include "traverse.cuh"

namespace rtx {

constexpr int kMaxDepthSlots = 64;
constexpr int kCounterInts = 4 * kMaxDepthSlots;
// material sort: at most this many materials (+1 bin for misses)
constexpr int kMaxSortBins = 4096;
// Minimum resident blocks of 128 threads per SM, i.e. the register budget
// (measured on the 1.3M-triangle frame: the traversal kernels are latency
// bound and gain from more warps until spills begin; shading, with the
// lobe-set variants, is fastest at 7 blocks (72 registers): 1.7 % faster
// than 8, 4 % faster than 6).
#ifndef RTX_SHADE_MINB
#define RTX_SHADE_MINB 7
#endif
// the batch variants (frames of several scenes in one wavefront): 8 blocks,
// 64 registers (1.4 % faster than 7 on the 16-scene batch)
#ifndef RTX_SHADE_MINB_JOBS
#define RTX_SHADE_MINB_JOBS 8
#endif
#ifndef RTX_EXTEND_MINB
#define RTX_EXTEND_MINB 10
#endif
#ifndef RTX_CONNECT_MINB
#define RTX_CONNECT_MINB 8
#endif
// path state 6 x 16 B + shadow record 4 x 16 B + six 4-byte entries (two
// queues, the material order, the ray order, the ray keys, the shadow order)
constexpr size_t kPathBytes = 6 * 16 + 4 * 16 + 7 * 4;

struct PtWorkspace {
  size_t cap = 0;
  float4* prim = nullptr;  // per-pixel primary hits
  size_t prim_cap = 0;
  float4 *ray_o = nullptr, *ray_d = nullptr, *thr = nullptr, *rad = nullptr, *absb = nullptr,
         *hit = nullptr;
  int* queue[2] = {nullptr, nullptr};
  int* sorted = nullptr;    // the shading queue ordered by material
  int* ray_sorted = nullptr;  // the extension queue ordered by ray key
  int* keys = nullptr;        // ray keys of the extension queue / shadow records
  int* shadow_order = nullptr;  // shadow records ordered by ray key
  int* mat_hist = nullptr;  // kMaxSortBins + 1 bins: counts, then write offsets
  // The occlusion launch of a vertex runs on `side`, beside the next vertex's
  // ray sort and closest-hit launch (RTX_OPT_OVERLAP): its shadow-ray sort
  // has its own keys and histogram, and two events order the streams.
  int* keys2 = nullptr;
  int* mat_hist2 = nullptr;
  cudaStream_t side = nullptr;
  cudaEvent_t ev_shaded = nullptr, ev_connected = nullptr;
  float4* shadow = nullptr;
  int* counters = nullptr;  // counts[64] | shadow_counts[64] | work[2 * 64]
  int num_sms = 0;
  int occ_extend = 0, occ_connect = 0, occ_shade = 0, occ_shade_jobs = 0, block_cached = 0;
  long long last_wave = 0;  // paths per wave of the last render
};

long long pt_last_wave(const PtWorkspace* ws) { return ws->last_wave; }

PtWorkspace* pt_workspace_create() { return new PtWorkspace(); }

static void ws_free(PtWorkspace* w) {
  float4* f[] = {w->ray_o, w->ray_d, w->thr, w->rad, w->absb, w->hit, w->shadow};
  for (float4* p : f)
    if (p) cudaFree(p);
  if (w->queue[0]) cudaFree(w->queue[0]);
  if (w->queue[1]) cudaFree(w->queue[1]);
  if (w->sorted) cudaFree(w->sorted);
  if (w->ray_sorted) cudaFree(w->ray_sorted);
  if (w->keys) cudaFree(w->keys);
  if (w->shadow_order) cudaFree(w->shadow_order);
  w->shadow_order = nullptr;
  if (w->mat_hist) cudaFree(w->mat_hist);
  if (w->keys2) cudaFree(w->keys2);
  if (w->mat_hist2) cudaFree(w->mat_hist2);
  w->sorted = w->ray_sorted = w->keys = w->mat_hist = w->keys2 = w->mat_hist2 = nullptr;
  if (w->counters) cudaFree(w->counters);
  w->ray_o = w->ray_d = w->thr = w->rad = w->absb = w->hit = w->shadow = nullptr;
  w->queue[0] = w->queue[1] = nullptr;
  w->counters = nullptr;
  w->cap = 0;
}

void pt_workspace_destroy(PtWorkspace* ws) {
  if (!ws) return;
  ws_free(ws);
  if (ws->prim) cudaFree(ws->prim);
  if (ws->ev_shaded) cudaEventDestroy(ws->ev_shaded);
  if (ws->ev_connected) cudaEventDestroy(ws->ev_connected);
  if (ws->side) cudaStreamDestroy(ws->side);
  delete ws;
}

static cudaError_t ws_reserve(PtWorkspace* w, size_t cap) {
  if (w->cap >= cap && w->counters) return cudaSuccess;
  ws_free(w);
  cudaError_t e;
  float4** f[] = {&w->ray_o, &w->ray_d, &w->thr, &w->rad, &w->absb, &w->hit};
  for (float4** p : f)
    if ((e = cudaMalloc(p, cap * sizeof(float4))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&w->shadow, cap * 4 * sizeof(float4))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&w->queue[0], cap * sizeof(int))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&w->queue[1], cap * sizeof(int))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&w->sorted, cap * sizeof(int))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&w->ray_sorted, cap * sizeof(int))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&w->keys, cap * sizeof(int))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&w->shadow_order, cap * sizeof(int))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&w->mat_hist, 2 * (kMaxSortBins + 1) * sizeof(int))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&w->keys2, cap * sizeof(int))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&w->mat_hist2, 2 * (kMaxSortBins + 1) * sizeof(int))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&w->counters, kCounterInts * sizeof(int))) != cudaSuccess) return e;
  w->cap = cap;
  return cudaSuccess;
}

struct PtArgs {
  float4 *ray_o, *ray_d, *thr, *rad, *absb, *hit, *shadow;
  int *queue_in, *queue_out;
  const int* shadow_order = nullptr;  // occlusion: record visiting order (nullptr: record order)
  // ray sort keys written by the shading kernel beside each new extension
  // ray (at its slot of the next queue) and each shadow record (nullptr:
  // rays not sorted)
  int *ekeys = nullptr, *skeys = nullptr;
  int *counts, *shadow_counts, *work;
  // a single render's camera (batches: each frame's, in its job) and the
  // per-pixel primary hits: the first shading launch makes its paths'
  // camera rays itself (k_shade<.., kFirst>)
  CamParams cam{};
  const float4* prim = nullptr;
  int* err;
  Counters* ctr;
  long long q0;
  int n_wave, npix, W, first_sample, max_depth, depth, min_busy;
  uint32_t k0, k1;
  // multi-scene batch: frames and their first paths (ascending)
  const PtJob* jobs;
  const long long* job_q;
  int n_jobs;
};

// The per-frame quantities of global path q: for a single render the scene's
// and the render's own; in a batch those of q's frame (binary search on the
// frames' first paths).
struct JobView {
  int job;  // the frame's index in the job table (batches; 0 otherwise)
  int root, root4, n_emitters;
  const int* emitters;
  float sky[3], ground[3];
  uint32_t k0, k1;
  long long q;  // path index within the frame
  int npix, first_sample;
};

template <bool kJobs>
RTX_DEV int job_index(const PtArgs& a, long long q) {
  if (!kJobs) return 0;
  int lo = 0, hi = a.n_jobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(a.job_q + mid) <= q)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

template <bool kJobs>
RTX_DEV JobView job_of(const PtArgs& a, const DeviceScene& s, long long q) {
  JobView v;
  v.job = 0;
  if (!kJobs) {
    v.root = s.root;
    v.root4 = s.root4;
    v.n_emitters = s.n_emitters;
    v.emitters = s.emitters;
    for (int k = 0; k < 3; ++k) {
      v.sky[k] = s.sky[k];
      v.ground[k] = s.ground[k];
    }
    v.k0 = a.k0;
    v.k1 = a.k1;
    v.q = q;
    v.npix = a.npix;
    v.first_sample = a.first_sample;
  } else {
    v.job = job_index<true>(a, q);
    const PtJob& J = a.jobs[v.job];
    v.root = J.root;
    v.root4 = J.root4;
    v.n_emitters = J.n_emitters;
    v.emitters = s.emitters + J.e_begin;
    for (int k = 0; k < 3; ++k) {
      v.sky[k] = J.sky[k];
      v.ground[k] = J.ground[k];
    }
    v.k0 = J.k0;
    v.k1 = J.k1;
    v.q = q - J.q_begin;
    v.npix = J.npix;
    v.first_sample = J.first_sample;
  }
  return v;
}

// the scene as one frame's traversal sees it (its own tree roots)
template <bool kJobs>
RTX_DEV DeviceScene scene_of(const DeviceScene& s, const PtArgs& a, long long q) {
  if (!kJobs) return s;
  DeviceScene r = s;
  const PtJob& J = a.jobs[job_index<true>(a, q)];
  r.root = J.root;
  r.root4 = J.root4;
  return r;
}

// Append with one atomic per warp; returns this thread's slot.
RTX_DEV int warp_append(int* counter) {
  unsigned mask = __activemask();
  int lane = threadIdx.x & 31;
  int leader = __ffs(mask) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(mask));
  base = __shfl_sync(mask, base, leader);
  return base + __popc(mask & ((1u << lane) - 1u));
}

// Persistent-warp work fetch: returns the first item of this warp's batch.
// (32 rays per fetch: 64, each lane tracing two rays in turn, measured 17 %
// slower per frame)
RTX_DEV int warp_fetch(int* work) {
  int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0) base = atomicAdd(work, 32);
  return __shfl_sync(0xffffffffu, base, 0);
}

template <bool kJobs>
__global__ void k_raygen(PtArgs a, CamParams cam, const float4* __restrict__ prim) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) a.counts[0] = a.n_wave;
  if (i >= a.n_wave) return;
  long long q = a.q0 + i;
  int pix, W;
  long long pix_base = 0;
  if (kJobs) {
    const PtJob& J = a.jobs[job_index<true>(a, q)];
    pix = (int)((q - J.q_begin) % J.npix);
    W = J.W;
    pix_base = J.pix_begin;
    cam = J.cam;
  } else {
    pix = (int)(q % a.npix);
    W = a.W;
  }
  if (prim) a.hit[i] = prim[pix_base + pix];
  F3 o, d;
  camera_ray(cam, pix % W, pix / W, o, d);
  a.ray_o[i] = make_float4(o.x, o.y, o.z, 0.0f);
  a.ray_d[i] = make_float4(d.x, d.y, d.z, __int_as_float(-1));
  a.thr[i] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(0u));
  a.rad[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  a.absb[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  a.queue_in[i] = i;
}

// Lanes of a warp that need a ray take the next ones from the queue; a lane
// finds none left when the queue is exhausted.
RTX_DEV int warp_refill(bool need, int* work, int n, bool& retired) {
  unsigned m = __ballot_sync(0xffffffffu, need);
  int item = -1;
  if (m) {
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(work, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (need) {
      int i = base + __popc(m & ((1u << lane) - 1u));
      if (i < n)
        item = i;
      else
        retired = true;
    }
  }
  return item;
}

// Closest hit of every live path (BVH::Intersect, renderer.cpp:282): persistent
// warps; a lane whose ray finishes takes a new one (dynamic fetch).
template <bool kCount>
__global__ void __launch_bounds__(128) k_extend(PtArgs a, DeviceScene s) {
  const int n = a.counts[a.depth];
  int* work = a.work + 2 * a.depth;
  VisitCount vc;
  Trav r;
  int stack[kStackSize];
  int p = -1;
  bool retired = false;
  while (true) {
    int i = warp_refill(p < 0 && !retired, work, n, retired);
    if (i >= 0) {
      p = a.queue_in[i];
      float4 ro = a.ray_o[p], rd = a.ray_d[p];
      trav_begin(r, stack, s, f3(ro.x, ro.y, ro.z), f3(rd.x, rd.y, rd.z), __float_as_int(rd.w), -1,
                 kInf);
    }
    if (__all_sync(0xffffffffu, p < 0)) break;
    if (p >= 0 && trav_run<false, kCount>(r, stack, s, a.err, vc, a.min_busy)) {
      a.hit[p] = make_float4(__int_as_float(r.best), r.tmax, r.u, r.v);
      p = -1;
    }
  }
  if (kCount) {
    atomicAdd(&a.ctr->ext_node_visits, (unsigned long long)vc.nodes);
    atomicAdd(&a.ctr->ext_tri_tests, (unsigned long long)vc.tris);
  }
}

// Variant: a warp takes 32 rays at a time and each lane traces its ray to the
// end before the warp takes the next batch.
template <bool kCount, bool kWide, bool kJobs>
__global__ void __launch_bounds__(128, RTX_EXTEND_MINB) k_extend_batch(PtArgs a, DeviceScene s0) {
  const int n = a.counts[a.depth];
  VisitCount vc;
  int lane = threadIdx.x & 31;
  while (true) {
    int base = warp_fetch(a.work + 2 * a.depth);
    if (base >= n) break;
    int i = base + lane;
    if (i < n) {
      int p = a.queue_in[i];
      const DeviceScene s = scene_of<kJobs>(s0, a, a.q0 + p);
      float4 ro = a.ray_o[p], rd = a.ray_d[p];
      float t, u, v;
      int h = kWide ? trace4<false, kCount>(s, f3(ro.x, ro.y, ro.z), f3(rd.x, rd.y, rd.z),
                                            __float_as_int(rd.w), -1, t, u, v, a.err, vc)
                    : closest_hit<kCount>(s, f3(ro.x, ro.y, ro.z), f3(rd.x, rd.y, rd.z),
                                          __float_as_int(rd.w), t, u, v, a.err, vc);
      a.hit[p] = make_float4(__int_as_float(h), t, u, v);
    }
  }
  if (kCount) {
    atomicAdd(&a.ctr->ext_node_visits, (unsigned long long)vc.nodes);
    atomicAdd(&a.ctr->ext_tri_tests, (unsigned long long)vc.tris);
  }
}

// Primary hits of every pixel, traced once per render: all samples of a pixel
// share its primary ray (renderer.cpp:255-259 has no per-sample jitter).
RTX_DEV void primary_px(const DeviceScene& s, const CamParams& cam, float4* out, int* err, Counters* ctr) {
  int tiles_x = (cam.W + 7) >> 3;
  int x = (blockIdx.x % tiles_x) * 8 + (threadIdx.x & 7);
  int y = (blockIdx.x / tiles_x) * 8 + (threadIdx.x >> 3);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(&ctr->ext_rays, (unsigned long long)cam.W * cam.H);
    atomicAdd(&ctr->ext_rays_by_depth[0], (unsigned long long)cam.W * cam.H);
  }
  if (x >= cam.W || y >= cam.H) return;
  F3 o, d;
  camera_ray(cam, x, y, o, d);
  float t, u, v;
  VisitCount vc;
  int h = closest_hit<false>(s, o, d, -1, t, u, v, err, vc);
  out[(size_t)y * cam.W + x] = make_float4(__int_as_float(h), t, u, v);
}

__global__ void __launch_bounds__(64) k_primary_cache(DeviceScene s, CamParams cam, float4* out, int* err,
                                                      Counters* ctr) {
  primary_px(s, cam, out, err, ctr);
}

// A frame of a batch: camera and tree root from the device job table, so that
// a replayed graph picks up new cameras.
__global__ void __launch_bounds__(64) k_primary_cache_job(DeviceScene s, const PtJob* jobs, int j, float4* prim,
                                                          int* err, Counters* ctr) {
  const PtJob& J = jobs[j];
  DeviceScene sj = s;
  sj.root = J.root;
  primary_px(sj, J.cam, prim + J.pix_begin, err, ctr);
}

// Sort keys (12 bits, 4,096 bins) from the scene bounds the host computed
// (SortKeyBounds).  Extension rays: the Morton code of the origin's cell in
// a 4^3 grid, then the direction's cube face (major axis and sign) and its
// 3 x 3 cell on that face; shadow rays (which all head for the lights, so the
// origin says most about the path): the origin's cell in a 16^3 grid
// (measured against 8^3 cells + octant for both: 552.7 -> 567.6 Msamples/s).
// Cheap enough to inline into the shading kernel; the direction cell takes
// a fast reciprocal, since a key only orders rays.
template <int G>
RTX_DEV uint32_t origin_cell(const SortKeyBounds& kb, F3 o) {
  const float* inv = G == 4 ? kb.inv4 : kb.inv16;
  auto cell = [](float v, float a, float iv) { return (uint32_t)min(max((int)((v - a) * iv), 0), G - 1); };
  auto spread = [](uint32_t v) { return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6); };
  return spread(cell(o.x, kb.lo[0], inv[0])) | (spread(cell(o.y, kb.lo[1], inv[1])) << 1) |
         (spread(cell(o.z, kb.lo[2], inv[2])) << 2);
}
RTX_DEV int shadow_sort_key(const SortKeyBounds& kb, F3 o) { return kb.ok ? (int)origin_cell<16>(kb, o) : 0; }
RTX_DEV int ext_sort_key(const SortKeyBounds& kb, F3 o, F3 d) {
  if (!kb.ok) return 0;
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  const bool fx = ax >= ay && ax >= az, fy = !fx && ay >= az;
  const int face = fx ? (d.x < 0.0f) : (fy ? 2 + (d.y < 0.0f) : 4 + (d.z < 0.0f));
  const float u = fx ? d.y : d.x, v = fx || fy ? d.z : d.y, mj = fx ? ax : (fy ? ay : az);
  const float inv = __fdividef(1.0f, fmaxf(mj, 1e-30f));
  const int cu = min(max((int)((u * inv + 1.0f) * 1.5f), 0), 2);
  const int cv = min(max((int)((v * inv + 1.0f) * 1.5f), 0), 2);
  return (int)((origin_cell<4>(kb, o) << 6) | (uint32_t)(face * 9 + cu * 3 + cv));
}

// Beer-Lambert factors pow(e, -absorption * distance) per channel and the
// log of a material's extinction: out of line, so that the shading kernel's
// common path (no absorption, extinction 1) does not carry six inlined
// transcendental functions through the instruction cache.
static __device__ __noinline__ F3 transmittance(F3 expo) {
  return f3(expo.x == 0.0f ? 1.0f : powf(kE, expo.x), expo.y == 0.0f ? 1.0f : powf(kE, expo.y),
            expo.z == 0.0f ? 1.0f : powf(kE, expo.z));
}
static __device__ __noinline__ F3 log_extinction(F3 ext) {
  return f3(ext.x == 1.0f ? 0.0f : logf(ext.x), ext.y == 1.0f ? 0.0f : logf(ext.y),
            ext.z == 1.0f ? 0.0f : logf(ext.z));
}

// kFeat: the scene's lobe set (kLobeTrans, kLobeCoat) | kShadeTex when some
// material has a procedural texture
constexpr int kShadeTex = 4;
// kFirst (renders with the primary-hit cache): the wave's first vertex,
// path i of the wave taking its camera ray and cached primary hit directly
// -- the state k_raygen would have written and this launch would have read
// back.
template <bool kJobs, int kFeat, bool kFirst = false>
__global__ void __launch_bounds__(128, kJobs ? RTX_SHADE_MINB_JOBS : RTX_SHADE_MINB) k_shade(PtArgs a, DeviceScene s) {
  constexpr bool kTex = (kFeat & kShadeTex) != 0;
  constexpr int kLobes = kFeat & kLobeAll;
  const int n = kFirst ? a.n_wave : a.counts[a.depth];
  if (kFirst && blockIdx.x == 0 && threadIdx.x == 0) a.counts[0] = a.n_wave;
  const int depth = a.depth;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int p = kFirst ? i : a.queue_in[i];
    const JobView J = job_of<kJobs>(a, s, a.q0 + p);
    float4 ro, rd, h, th;
    if (kFirst) {
      // the frame's pixel of the path, as k_raygen numbers it
      const PtJob* pj = kJobs ? a.jobs + J.job : nullptr;
      const int pix = kJobs ? (int)(J.q % pj->npix) : (int)((a.q0 + p) % a.npix);
      const int W = kJobs ? pj->W : a.W;
      F3 co, cd;
      camera_ray(kJobs ? pj->cam : a.cam, pix % W, pix / W, co, cd);
      ro = make_float4(co.x, co.y, co.z, 0.0f);
      rd = make_float4(cd.x, cd.y, cd.z, __int_as_float(-1));
      h = __ldg(a.prim + (kJobs ? pj->pix_begin : 0) + pix);
      th = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(0u));
    } else {
      ro = a.ray_o[p];
      rd = a.ray_d[p];
      h = a.hit[p];
      th = a.thr[p];
    }
    F3 o = f3(ro.x, ro.y, ro.z), d = f3(rd.x, rd.y, rd.z);
    float last_pdf = ro.w;
    int tri = __float_as_int(h.x);
    F3 T = f3(th.x, th.y, th.z);
    // The path's radiance is read and written back only when this vertex
    // adds a term that is not exactly zero: the sum starts at +0 and never
    // becomes -0 (x + y is -0 only when both are), so adding +-0 leaves it
    // unchanged, bit for bit; a NaN term is added.  The first vertex always
    // writes it (no earlier value exists).
    F3 acc = f3s(0.0f);
    bool touched = kFirst;
    auto add_rad = [&](F3 x) {
      if (x.x == 0.0f && x.y == 0.0f && x.z == 0.0f) return;
      if (!touched) {
        const float4 r0 = a.rad[p];
        acc = f3(r0.x, r0.y, r0.z);
        touched = true;
      }
      acc = acc + x;
    };
    if (tri < 0) {
      // World::GetDefaultEmission (world.cpp:39-42) of -direction
      F3 env = (-d.z < 0.0f) ? f3(J.sky[0], J.sky[1], J.sky[2])
                             : f3(J.ground[0], J.ground[1], J.ground[2]);
      add_rad(T * env);
      if (touched) a.rad[p] = make_float4(acc.x, acc.y, acc.z, 0.0f);
      continue;
    }
    // bit 31 of the RNG counter word: the path carries an absorption that
    // is not +-0 (only then was it stored); +-0 reads as +0, which gives
    // the same transmittance (pow(e, +-0) = 1, and +-0 * inf = NaN either way)
    const uint32_t thw = __float_as_uint(th.w);
    float4 ab = (kFirst || !(thw >> 31)) ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : a.absb[p];
    F3 absorption = f3(ab.x, ab.y, ab.z);
    float t = h.y, u = h.z, v = h.w;
    float4 s0 = __ldg(s.shade + 4 * (size_t)tri), s1 = __ldg(s.shade + 4 * (size_t)tri + 1);
    int info = __float_as_int(s1.w);
    const float* mrec = s.mats + 24 * (size_t)(info & 0x7fffffff);
    Mat m = load_mat(mrec);
    F3 pos = o + d * t;  // BVH::Intersect: src + t * direction
    F3 N = shading_normal(s, tri, u, v, s0, s1, info < 0);
    if (kTex && __ldg(mrec + 21) != 0.0f) m.base_color = textured_base(mrec, pos, N, s.perm);
    F3 ff = N;
    float eta;
    if (dot(d, ff) > 0.0f) {  // renderer.cpp:288-298
      ff = -ff;
      eta = m.ior;
      absorption = f3s(0.0f);
    } else {
      eta = 1.0f / m.ior;
    }
    // SurfacePoint::GetEmission<true> (surfacepoint.h:21-45) toward the ray source
    F3 re = o - pos;
    float d2 = dot(re, re);
    float cos_area = dot(-d, N) * s0.w;
    float self_pdf = fabsf(d2 / cos_area);
    F3 E = m.emission;
    if (depth > 0) E = E * PowerHeuristic(last_pdf, self_pdf);
    add_rad(T * E);
    float dist = length(pos - o);
    F3 expo = (-absorption) * dist;
    // pow(e, +-0) is exactly 1: no call for the common no-absorption case
    F3 br = (expo.x == 0.0f && expo.y == 0.0f && expo.z == 0.0f) ? f3s(1.0f) : transmittance(expo);
    ShadingFrame fr = make_frame(m, eta, ff, -d);

    long long q = J.q;
    Rng rng{J.k0, J.k1, (uint32_t)(q % J.npix), (uint32_t)(J.first_sample + q / J.npix),
            thw & 0x7fffffffu};
    // the vertex's draws, in the reference's order: Int (emitter), Float,
    // Float (point on it) when there are emitters, then Float, Float (BSDF)
    uint32_t dv[5];
    rng.draw5(dv);
    const bool nee = J.n_emitters > 0;
    rng.draw += nee ? 5u : 2u;
    if (nee) {
      // World::SampleEmitter + Triangle::GetSamplePoint (world.cpp:5-17, object.cpp:169-178)
      int e = __ldg(J.emitters + Rng::to_int(dv[0], 0, J.n_emitters - 1));
      float sqr1 = sqrtf(Rng::to_uniform(dv[1]));
      float r2 = Rng::to_uniform(dv[2]);
      float aa = 1.0f - sqr1;
      float bb = (1.0f - r2) * sqr1;
      const float4* g = s.geo + 3 * (size_t)e;
      float4 g0 = __ldg(g), g1 = __ldg(g + 1), g2 = __ldg(g + 2);
      F3 emit_pos = (f3(g1.x, g1.y, g1.z) * aa + f3(g2.x, g2.y, g2.z) * bb) + f3(g0.x, g0.y, g0.z);
      F3 dl = normalized(emit_pos - pos);
      float bpdf;
      F3 f = BsdfEvalFrame<kLobes>(m, eta, fr, dl, bpdf);
      if (bpdf > 0.0f) {
        int slot = warp_append(a.shadow_counts + depth);
        F3 tb = T * br;
        float4* r = a.shadow + 4 * (size_t)slot;
        r[0] = make_float4(pos.x, pos.y, pos.z, __int_as_float(p));
        r[1] = make_float4(emit_pos.x, emit_pos.y, emit_pos.z, __int_as_float(e));
        r[2] = make_float4(f.x, f.y, f.z, bpdf);
        r[3] = make_float4(tb.x, tb.y, tb.z, __int_as_float(tri));
        if (a.skeys) a.skeys[slot] = shadow_sort_key(kJobs ? a.jobs[J.job].keyb : s.keyb, pos);
      }
    }
    float r1 = Rng::to_uniform(nee ? dv[3] : dv[0]);
    float r2 = Rng::to_uniform(nee ? dv[4] : dv[1]);
    F3 nd, color;
    float pdf;
    bool cont = false;
    if (BsdfSampleFrame<kLobes>(m, eta, fr, r1, r2, nd, color, pdf)) {
      // log(1) is exactly +0: no call for the default extinction
      F3 lg = (m.extinction.x == 1.0f && m.extinction.y == 1.0f && m.extinction.z == 1.0f)
                  ? f3s(0.0f)
                  : log_extinction(m.extinction);
      absorption = (-lg) / m.at_distance;
      if (pdf > 0.0f) {
        F3 w = (br * color) / pdf;
        if (depth + 1 < a.max_depth) {
          T = T * w;
          cont = true;
        } else {
          // the reference multiplies by the (zero) radiance beyond the cap,
          // which keeps an infinite or NaN weight visible as NaN
          add_rad(T * (w * 0.0f));
        }
      }
    }
    if (touched) a.rad[p] = make_float4(acc.x, acc.y, acc.z, 0.0f);
    if (cont) {
      a.ray_o[p] = make_float4(pos.x, pos.y, pos.z, pdf);
      a.ray_d[p] = make_float4(nd.x, nd.y, nd.z, __int_as_float(tri));
      const bool ab_zero = absorption.x == 0.0f && absorption.y == 0.0f && absorption.z == 0.0f;
      a.thr[p] = make_float4(T.x, T.y, T.z, __uint_as_float(rng.draw | (ab_zero ? 0u : 0x80000000u)));
      if (!ab_zero) a.absb[p] = make_float4(absorption.x, absorption.y, absorption.z, 0.0f);
      int slot = warp_append(a.counts + depth + 1);
      a.queue_out[slot] = p;
      if (a.ekeys) a.ekeys[slot] = ext_sort_key(kJobs ? a.jobs[J.job].keyb : s.keyb, pos, nd);
    }
  }
}

// The shading variant a scene needs: its lobe set and whether it is textured.
static int shade_features(const DeviceScene& s) { return (s.lobes & kLobeAll) | (s.textured ? kShadeTex : 0); }

template <bool kJobs>
static void launch_shade(int feat, dim3 grid, dim3 block, cudaStream_t st, const PtArgs& a, const DeviceScene& s,
                         bool first = false) {
  if (first) {
    switch (feat) {
      case 0: k_shade<kJobs, 0, true><<<grid, block, 0, st>>>(a, s); return;
      case 1: k_shade<kJobs, 1, true><<<grid, block, 0, st>>>(a, s); return;
      case 2: k_shade<kJobs, 2, true><<<grid, block, 0, st>>>(a, s); return;
      case 3: k_shade<kJobs, 3, true><<<grid, block, 0, st>>>(a, s); return;
      case 4: k_shade<kJobs, 4, true><<<grid, block, 0, st>>>(a, s); return;
      case 5: k_shade<kJobs, 5, true><<<grid, block, 0, st>>>(a, s); return;
      case 6: k_shade<kJobs, 6, true><<<grid, block, 0, st>>>(a, s); return;
      default: k_shade<kJobs, 7, true><<<grid, block, 0, st>>>(a, s); return;
    }
  }
  switch (feat) {
    case 0: k_shade<kJobs, 0><<<grid, block, 0, st>>>(a, s); break;
    case 1: k_shade<kJobs, 1><<<grid, block, 0, st>>>(a, s); break;
    case 2: k_shade<kJobs, 2><<<grid, block, 0, st>>>(a, s); break;
    case 3: k_shade<kJobs, 3><<<grid, block, 0, st>>>(a, s); break;
    case 4: k_shade<kJobs, 4><<<grid, block, 0, st>>>(a, s); break;
    case 5: k_shade<kJobs, 5><<<grid, block, 0, st>>>(a, s); break;
    case 6: k_shade<kJobs, 6><<<grid, block, 0, st>>>(a, s); break;
    default: k_shade<kJobs, 7><<<grid, block, 0, st>>>(a, s); break;
  }
}

// resident blocks per SM of the least-resident shading variant
template <bool kJobs>
static int shade_occupancy(int block) {
  int occ = 1 << 30, o = 0;
  for (auto k : {k_shade<kJobs, 0>, k_shade<kJobs, 1>, k_shade<kJobs, 2>, k_shade<kJobs, 3>, k_shade<kJobs, 4>,
                 k_shade<kJobs, 5>, k_shade<kJobs, 6>, k_shade<kJobs, 7>}) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k, block, 0);
    occ = std::min(occ, o);
  }
  return occ;
}

// Emitter's own exact test for a shadow record: the emitter is the target of
// the occlusion query when the ray reaches it (t < 1e7); otherwise any hit
// occludes.
RTX_DEV bool emitter_hit(const DeviceScene& s, F3 pos, F3 dir, int e, int ex, float& te, float& ue,
                         float& ve) {
  te = kInf;
  ue = 0.0f;
  ve = 0.0f;
  if (e == ex) return false;
  const float4* g = s.geo + 3 * (size_t)e;
  float4 g0 = __ldg(g), g1 = __ldg(g + 1), g2 = __ldg(g + 2);
  float tt, uu, vv;
  if (tri_hit(pos, dir, f3(g0.x, g0.y, g0.z), f3(g1.x, g1.y, g1.z), f3(g2.x, g2.y, g2.z), tt, uu, vv) &&
      tt < kInf) {
    te = tt;
    ue = uu;
    ve = vv;
    return true;
  }
  return false;
}

// Visibility of each light sample (renderer.cpp:352-354: the light is seen
// when the closest hit is the sampled emitter or nothing) as an occlusion
// query, then the MIS-weighted contribution (renderer.cpp:356-379).
RTX_DEV void add_light(const PtArgs& a, const DeviceScene& s, int rec, int n_emitters);

template <bool kCount, bool kWide, bool kJobs>
__global__ void __launch_bounds__(128, RTX_CONNECT_MINB) k_connect_batch(PtArgs a, DeviceScene s0) {
  const int n = a.shadow_counts[a.depth];
  VisitCount vc;
  int lane = threadIdx.x & 31;
  while (true) {
    int base = warp_fetch(a.work + 2 * a.depth + 1);
    if (base >= n) break;
    int i = base + lane;
    if (i >= n) continue;
    if (a.shadow_order) i = a.shadow_order[i];
    const float4* q = a.shadow + 4 * (size_t)i;
    float4 q0 = q[0], q1 = q[1], q3 = q[3];
    const DeviceScene s = scene_of<kJobs>(s0, a, a.q0 + __float_as_int(q0.w));
    F3 pos = f3(q0.x, q0.y, q0.z);
    F3 dir = normalized(f3(q1.x, q1.y, q1.z) - pos);
    int e = __float_as_int(q1.w), ex = __float_as_int(q3.w);
    float te, ue, ve;
    bool he = emitter_hit(s, pos, dir, e, ex, te, ue, ve);
    bool occ;
    if (kWide) {
      float uu, vv;
      occ = trace4<true, kCount>(s, pos, dir, ex, he ? e : -1, te, uu, vv, a.err, vc) == 1;
    } else {
      occ = occluded<kCount>(s, pos, dir, ex, he ? e : -1, te, a.err, vc);
    }
    if (!occ) add_light(a, s, i, job_of<kJobs>(a, s, a.q0 + __float_as_int(q0.w)).n_emitters);
  }
  if (kCount) {
    atomicAdd(&a.ctr->sh_node_visits, (unsigned long long)vc.nodes);
    atomicAdd(&a.ctr->sh_tri_tests, (unsigned long long)vc.tris);
  }
}

template <bool kCount>
__global__ void __launch_bounds__(128) k_connect(PtArgs a, DeviceScene s) {
  const int n = a.shadow_counts[a.depth];
  int* work = a.work + 2 * a.depth + 1;
  VisitCount vc;
  Trav r;
  int stack[kStackSize];
  int rec = -1;
  bool retired = false;
  while (true) {
    int i = warp_refill(rec < 0 && !retired, work, n, retired);
    if (i >= 0) {
      rec = i;
      const float4* q = a.shadow + 4 * (size_t)rec;
      float4 q0 = q[0], q1 = q[1], q3 = q[3];
      F3 pos = f3(q0.x, q0.y, q0.z);
      F3 dir = normalized(f3(q1.x, q1.y, q1.z) - pos);
      int e = __float_as_int(q1.w), ex = __float_as_int(q3.w);
      float te, ue, ve;
      bool he = emitter_hit(s, pos, dir, e, ex, te, ue, ve);
      trav_begin(r, stack, s, pos, dir, ex, he ? e : -1, te);
    }
    if (__all_sync(0xffffffffu, rec < 0)) break;
    if (rec >= 0 && trav_run<true, kCount>(r, stack, s, a.err, vc, a.min_busy)) {
      if (r.best != 1) add_light(a, s, rec, s.n_emitters);
      rec = -1;
    }
  }
  if (kCount) {
    atomicAdd(&a.ctr->sh_node_visits, (unsigned long long)vc.nodes);
    atomicAdd(&a.ctr->sh_tri_tests, (unsigned long long)vc.tris);
  }
}

// MIS-weighted light contribution of a visible light sample
// (renderer.cpp:356-379), added to its path's radiance.
RTX_DEV void add_light(const PtArgs& a, const DeviceScene& s, int rec, int n_emitters) {
  const float4* q = a.shadow + 4 * (size_t)rec;
  float4 q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
  F3 pos = f3(q0.x, q0.y, q0.z), emit_pos = f3(q1.x, q1.y, q1.z);
  int p = __float_as_int(q0.w), e = __float_as_int(q1.w), ex = __float_as_int(q3.w);
  F3 dir = normalized(emit_pos - pos);
  float te, ue, ve;
  emitter_hit(s, pos, dir, e, ex, te, ue, ve);  // (u, v) of the emitter hit, or (0, 0)
  float4 s0 = __ldg(s.shade + 4 * (size_t)e), s1 = __ldg(s.shade + 4 * (size_t)e + 1);
  int info = __float_as_int(s1.w);
  F3 Ne = shading_normal(s, e, ue, ve, s0, s1, info < 0);
  F3 rv = pos - emit_pos;
  float d2 = dot(rv, rv);
  float cos_area = dot(-dir, Ne) * s0.w;
  float lpdf = fabsf(d2 / cos_area);
  const float* me = s.mats + 24 * (size_t)(info & 0x7fffffff);
  F3 Le = f3(__ldg(me + 3), __ldg(me + 4), __ldg(me + 5));
  float w = PowerHeuristic(lpdf, q2.w);
  F3 c = f3(q2.x, q2.y, q2.z) * w;
  c = c * Le;
  c = c * (float)n_emitters;
  c = c / lpdf;
  float4 acc = a.rad[p];
  F3 tb = f3(q3.x, q3.y, q3.z) * c;
  a.rad[p] = make_float4(acc.x + tb.x, acc.y + tb.y, acc.z + tb.z, 0.0f);
}

// One pixel of the display resolve (see Resolve).
__device__ __forceinline__ uint8_t quantise(float x) {
  // std::clamp keeps NaN; int(NaN) stores 0 in the exporters' 8-bit fields
  if (!(x == x)) return 0;
  float c = x < 0.0f ? 0.0f : (1.0f < x ? 1.0f : x);
  return (uint8_t)(int)(255.99f * c);
}

__device__ void resolve_px(F3 c, int i, const Resolve& r) {
  if (r.limit > 0.0f) {
    float luma = 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z;
    float s = 1.0f + luma / r.limit;
    c = f3(c.x * 1.0f / s, c.y * 1.0f / s, c.z * 1.0f / s);
  }
  if (r.ratio > 0.0f) c = f3(powf(c.x, r.ratio), powf(c.y, r.ratio), powf(c.z, r.ratio));
  if (r.display) {
    r.display[3 * (size_t)i] = c.x;
    r.display[3 * (size_t)i + 1] = c.y;
    r.display[3 * (size_t)i + 2] = c.z;
  }
  if (r.bytes) {
    int y = i / r.W, x = i - y * r.W;
    if (r.format == kResolveBmp) {
      size_t row = bmp_row_bytes(r.W);
      uint8_t* px = r.bytes + (size_t)y * row + 3 * (size_t)x;
      px[0] = quantise(c.z);
      px[1] = quantise(c.y);
      px[2] = quantise(c.x);
      if (x == r.W - 1)
        for (size_t k = 3 * (size_t)r.W; k < row; ++k) r.bytes[(size_t)y * row + k] = 0;
    } else {
      uint8_t* px = r.bytes + 3 * (size_t)i;
      px[0] = quantise(c.x);
      px[1] = quantise(c.y);
      px[2] = quantise(c.z);
    }
  }
}

__global__ void k_resolve(const float* __restrict__ in, int n, Resolve r) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) resolve_px(f3(in[3 * (size_t)i], in[3 * (size_t)i + 1], in[3 * (size_t)i + 2]), i, r);
}

cudaError_t launch_resolve(const float* in, int W, int H, const Resolve& r, cudaStream_t st) {
  int n = W * H;
  if (n > 0) k_resolve<<<(n + 255) / 256, 256, 0, st>>>(in, n, r);
  return cudaGetLastError();
}

// Batch: pixel i of the concatenated output belongs to the frame whose
// pixels begin at or before it; its paths are q_begin + s * npix + pixel.
__global__ void k_accumulate_jobs(const float4* rad, long long q0, int n_wave, const PtJob* jobs,
                                  int n_jobs, long long total_pix, float* out) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= total_pix) return;
  int lo = 0, hi = n_jobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].pix_begin <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  const PtJob& J = jobs[lo];
  long long pix = i - J.pix_begin;
  long long first = J.q_begin + pix;                 // sample 0 of this pixel
  long long last = first + (long long)(J.spp - 1) * J.npix;
  if (last < q0 || first >= q0 + n_wave) return;
  long long qs = first;
  if (qs < q0) qs = first + (q0 - first + J.npix - 1) / J.npix * J.npix;
  float* o = out + 3 * (size_t)i;
  F3 acc = f3(o[0], o[1], o[2]);
  const float spp = (float)J.spp;
  for (long long q = qs; q <= last && q < q0 + n_wave; q += J.npix) {
    float4 r = rad[q - q0];
    acc = acc + f3(r.x, r.y, r.z) / spp;
  }
  o[0] = acc.x;
  o[1] = acc.y;
  o[2] = acc.z;
}

__global__ void k_accumulate(const float4* rad, long long q0, int n_wave, int npix, float spp,
                             float* out, int per_path, Resolve rs, int last) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (per_path) {
    if (i >= n_wave) return;
    float4 r = rad[i];
    size_t q = (size_t)(q0 + i);
    out[3 * q] = r.x;
    out[3 * q + 1] = r.y;
    out[3 * q + 2] = r.z;
    return;
  }
  if (i >= npix) return;
  long long off = ((long long)i - q0 % npix + npix) % npix;
  long long qs = q0 + off;
  float* o = out + 3 * (size_t)i;
  F3 acc = f3(o[0], o[1], o[2]);
  if (qs < q0 + n_wave) {
    for (long long q = qs; q < q0 + n_wave; q += npix) {
      float4 r = rad[q - q0];
      acc = acc + f3(r.x, r.y, r.z) / spp;
    }
    o[0] = acc.x;
    o[1] = acc.y;
    o[2] = acc.z;
  }
  // the last wave resolves every pixel for display in the same pass
  if (last) resolve_px(acc, i, rs);
}

__global__ void k_tally(const int* counts, const int* shadow_counts, int max_depth, int first_traced,
                        Counters* c) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned long long e = 0, sh = 0;
  for (int d = 0; d < max_depth; ++d) {
    sh += (unsigned)shadow_counts[d];
    if (d < first_traced) continue;  // primary hits came from the per-pixel cache
    e += (unsigned)counts[d];
    if (d < 16) c->ext_rays_by_depth[d] += (unsigned)counts[d];
  }
  c->ext_rays += e;
  c->shadow_rays += sh;
}

KernelTimer::~KernelTimer() {
  for (cudaEvent_t e : pool) cudaEventDestroy(e);
}

cudaError_t KernelTimer::mark(int kind, cudaStream_t st, bool start) {
  if (!on) return cudaSuccess;
  if (used == pool.size()) {
    cudaEvent_t e;
    cudaError_t r = cudaEventCreate(&e);
    if (r != cudaSuccess) return r;
    pool.push_back(e);
  }
  if (start) marks.emplace_back(kind, (int)used);
  return cudaEventRecord(pool[used++], st);
}

cudaError_t KernelTimer::collect() {
  for (auto& m : marks) {
    float t = 0.0f;
    cudaError_t r = cudaEventElapsedTime(&t, pool[m.second], pool[m.second + 1]);
    if (r != cudaSuccess) return r;
    ms[m.first] += t;
  }
  marks.clear();
  used = 0;
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Material sort of the shading queue (RTX_OPT_SORT_MATERIAL): a counting sort
// of the live paths by the material of their hit (misses last), so that the
// warps of the shading kernel meet fewer materials.  Paths keep their state
// slots; only the order the shading kernel visits them changes.
// ---------------------------------------------------------------------------
RTX_DEV int mat_key(const DeviceScene& s, const float4* hit, int p) {
  int tri = __float_as_int(hit[p].x);
  if (tri < 0) return s.n_mats;
  return __float_as_int(__ldg(s.shade + 4 * (size_t)tri + 1).w) & 0x7fffffff;
}

__global__ void __launch_bounds__(256) k_sort_hist(PtArgs a, DeviceScene s, int* hist) {
  extern __shared__ int sh[];
  const int bins = s.n_mats + 1;
  for (int b = threadIdx.x; b < bins; b += blockDim.x) sh[b] = 0;
  __syncthreads();
  const int n = a.counts[a.depth];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    atomicAdd(&sh[mat_key(s, a.hit, a.queue_in[i])], 1);
  __syncthreads();
  for (int b = threadIdx.x; b < bins; b += blockDim.x)
    if (sh[b]) atomicAdd(&hist[b], sh[b]);
}

// exclusive prefix sum of the bins into hist[kMaxSortBins + 1 + b]; one block
__global__ void __launch_bounds__(1024) k_sort_scan(int bins, int* hist) {
  __shared__ int part[1024];
  const int per = (bins + 1023) / 1024;
  const int b0 = threadIdx.x * per;
  int sum = 0;
  for (int b = b0; b < b0 + per && b < bins; ++b) sum += hist[b];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = part[threadIdx.x] - sum;  // exclusive
  int* offs = hist + kMaxSortBins + 1;
  for (int b = b0; b < b0 + per && b < bins; ++b) {
    offs[b] = run;
    run += hist[b];
  }
}

// lanes with equal keys take consecutive slots with one atomic per key
__global__ void __launch_bounds__(256) k_sort_scatter(PtArgs a, DeviceScene s, int* hist, int* sorted) {
  int* offs = hist + kMaxSortBins + 1;
  const int n = a.counts[a.depth];
  for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    int i = base + threadIdx.x;
    bool live = i < n;
    int p = live ? a.queue_in[i] : 0;
    int key = live ? mat_key(s, a.hit, p) : -1;
    unsigned act = __ballot_sync(0xffffffffu, live);
    if (!live) continue;
    unsigned peers = __match_any_sync(act, key);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    int slot0 = 0;
    if (lane == leader) slot0 = atomicAdd(&offs[key], __popc(peers));
    slot0 = __shfl_sync(peers, slot0, leader);
    sorted[slot0 + __popc(peers & ((1u << lane) - 1u))] = p;
  }
}

// ---------------------------------------------------------------------------
// Ray sort (RTX_OPT_SORT_RAYS): counting sorts by a 12-bit key of the ray's
// origin cell and direction (ext_sort_key / shadow_sort_key, written by the
// shading kernel beside each ray), so that a warp of a traversal kernel
// takes rays that start close together and head the same way: fewer
// divergent node visits and more cache hits.  Two sorts per path vertex: the extension
// queue before the closest-hit kernel, and the shadow records before the
// occlusion kernel.  The shading kernel keeps visiting paths in the order
// the previous vertex wrote them, which keeps its path-state reads
// coalesced (shading in key order measured 8 % slower per frame).  Only the
// order in which paths and records are visited changes, never a result.
// Measured on the 1.3M-triangle frame: 434 -> 519 Msamples/s, the
// closest-hit launch 5.12 -> 3.44 ms.
// ---------------------------------------------------------------------------
constexpr int kRayKeyBins = 4096;

// Count `key` in a shared-memory histogram; returns the counter's value
// before this lane's add (a rank unique among the lanes and warps that add to
// the same key).  Plain shared atomics measured 3.3 % faster per frame than
// aggregating equal keys per warp with __match_any_sync.
RTX_DEV int count_key(int* counter, int key) { return atomicAdd(counter + key, 1); }

// Histogram of the sort keys the shading kernel wrote beside the items
// (kShadow = false: the extension queue, keys[i] for queue entry i; true:
// the shadow records, keys[i] for record i).  Each thread takes kHistPer
// keys per step and issues their loads before counting any.
constexpr int kHistPer = 4;

template <bool kShadow>
__global__ void __launch_bounds__(256) k_raykey_hist(PtArgs a, const int* keys, int* hist) {
  __shared__ int sh[kRayKeyBins];
  for (int b = threadIdx.x; b < kRayKeyBins; b += blockDim.x) sh[b] = 0;
  __syncthreads();
  const int n = kShadow ? a.shadow_counts[a.depth] : a.counts[a.depth];
  const int step = gridDim.x * blockDim.x * kHistPer;
  for (int base = blockIdx.x * blockDim.x * kHistPer; base < n; base += step) {
    int k[kHistPer];
#pragma unroll
    for (int j = 0; j < kHistPer; ++j) {
      const int i = base + j * blockDim.x + threadIdx.x;
      k[j] = i < n ? keys[i] : -1;
    }
#pragma unroll
    for (int j = 0; j < kHistPer; ++j)
      if (k[j] >= 0) count_key(sh, k[j]);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kRayKeyBins; b += blockDim.x)
    if (sh[b]) atomicAdd(&hist[b], sh[b]);
}

// Scatter in chunks of kScatterChunk queue entries per block: count the
// chunk's keys in shared memory, reserve each key's run with one global
// atomic per (chunk, key), then write every path to its slot.
constexpr int kScatterPer = 16, kScatterChunk = 256 * kScatterPer;

template <bool kShadow>
__global__ void __launch_bounds__(256) k_raykey_scatter(PtArgs a, const int* keys, int* hist, int* sorted) {
  __shared__ int cnt[kRayKeyBins], run[kRayKeyBins];
  int* offs = hist + kMaxSortBins + 1;
  const int n = kShadow ? a.shadow_counts[a.depth] : a.counts[a.depth];
  const int tid = threadIdx.x;
  for (int c0 = blockIdx.x * kScatterChunk; c0 < n; c0 += gridDim.x * kScatterChunk) {
    for (int b = tid; b < kRayKeyBins; b += 256) cnt[b] = 0;
    __syncthreads();
    int key[kScatterPer], rank[kScatterPer], path[kScatterPer];
#pragma unroll
    for (int j = 0; j < kScatterPer; ++j) {
      const int i = c0 + j * 256 + tid;
      key[j] = -1;
      if (i < n) {
        key[j] = keys[i];
        path[j] = kShadow ? i : a.queue_in[i];
        rank[j] = count_key(cnt, key[j]);
      }
    }
    __syncthreads();
    for (int b = tid; b < kRayKeyBins; b += 256)
      if (cnt[b]) run[b] = atomicAdd(&offs[b], cnt[b]);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kScatterPer; ++j)
      if (key[j] >= 0) sorted[run[key[j]] + rank[j]] = path[j];
    __syncthreads();
  }
}

// The launch sequence of one wave: raygen, then per vertex extend (skipped at
// depth 0 when the primary hits are cached), shade and connect.
template <bool kJobs>
static cudaError_t wave_launches(const PtParams& p, PtArgs& a, const DeviceScene& s, const CamParams& cam,
                                 const float4* prim, PtWorkspace* ws, KernelTimer* timer, cudaStream_t st,
                                 int grid_ext, int grid_con, int grid_sh, int block, int nw, int* launches,
                                 int* extend_launches, int* vertex_launches, bool overlap) {
  cudaError_t e;
  a.queue_in = ws->queue[0];
  a.queue_out = ws->queue[1];
  a.depth = 0;
  // A render with cached primary hits and path-order shading needs no path
  // state before its first shading launch, which makes the camera rays
  // itself; otherwise k_raygen writes the state (and the cached hits).
  const bool first_in_shade = prim && !p.sort_material;
  a.cam = cam;
  a.prim = prim;
  // with ray sorting, the shading kernel writes the extension rays' keys to
  // `keys` and the shadow records' to `keys2` (from each frame's scene
  // grids); each is read by its sort before the next shading launch writes
  // it again
  a.ekeys = p.sort_rays ? ws->keys : nullptr;
  a.skeys = p.sort_rays ? ws->keys2 : nullptr;
  if (!first_in_shade) {
    k_raygen<kJobs><<<(nw + 255) / 256, 256, 0, st>>>(a, cam, prim);
    ++*launches;
  }
  for (int depth = 0; depth < p.max_depth; ++depth) {
    a.depth = depth;
    a.queue_in = ws->queue[depth & 1];
    a.queue_out = ws->queue[(depth + 1) & 1];
    int* const path_order = a.queue_in;  // the queue as the previous vertex wrote it (shading order)
    if (p.sort_rays && depth > 0) {
      static_assert(kRayKeyBins <= kMaxSortBins, "ray keys use the sort histogram");
      if ((e = cudaMemsetAsync(ws->mat_hist, 0, (kMaxSortBins + 1) * sizeof(int), st))) return e;
      k_raykey_hist<false><<<grid_sh, 256, 0, st>>>(a, ws->keys, ws->mat_hist);
      k_sort_scan<<<1, 1024, 0, st>>>(kRayKeyBins, ws->mat_hist);
      k_raykey_scatter<false><<<grid_sh, 256, 0, st>>>(a, ws->keys, ws->mat_hist, ws->ray_sorted);
      *launches += 3;
      a.queue_in = ws->ray_sorted;  // the closest-hit kernel visits paths in key order
    }
    if (!(prim && depth == 0)) {
      if ((e = timer->mark(0, st, true))) return e;
      if (p.traversal == 2) {
        if (p.count_visits)
          k_extend_batch<true, true, kJobs><<<grid_ext, block, 0, st>>>(a, s);
        else
          k_extend_batch<false, true, kJobs><<<grid_ext, block, 0, st>>>(a, s);
      } else if (p.traversal == 0 || kJobs) {
        if (p.count_visits)
          k_extend_batch<true, false, kJobs><<<grid_ext, block, 0, st>>>(a, s);
        else
          k_extend_batch<false, false, kJobs><<<grid_ext, block, 0, st>>>(a, s);
      } else if (p.count_visits) {
        k_extend<true><<<grid_ext, block, 0, st>>>(a, s);
      } else {
        k_extend<false><<<grid_ext, block, 0, st>>>(a, s);
      }
      if ((e = timer->mark(0, st, false))) return e;
      ++*extend_launches;
      ++*launches;
    }
    // the previous vertex's occlusion launch (on the side stream) adds to the
    // radiance this vertex's shading reads and writes: wait for it here
    if (overlap && depth > 0 && (e = cudaStreamWaitEvent(st, ws->ev_connected, 0))) return e;
    if ((e = timer->mark(1, st, true))) return e;
    a.queue_in = path_order;
    if (p.sort_material && s.n_mats + 1 <= kMaxSortBins) {
      // the shading kernel reads the sorted queue; its output queue is unchanged
      if ((e = cudaMemsetAsync(ws->mat_hist, 0, (kMaxSortBins + 1) * sizeof(int), st))) return e;
      size_t shm = (size_t)(s.n_mats + 1) * sizeof(int);
      k_sort_hist<<<grid_sh, 256, shm, st>>>(a, s, ws->mat_hist);
      k_sort_scan<<<1, 1024, 0, st>>>(s.n_mats + 1, ws->mat_hist);
      k_sort_scatter<<<grid_sh, 256, 0, st>>>(a, s, ws->mat_hist, ws->sorted);
      *launches += 3;
      PtArgs as = a;
      as.queue_in = ws->sorted;
      launch_shade<kJobs>(shade_features(s), grid_sh, block, st, as, s);
    } else {
      launch_shade<kJobs>(shade_features(s), grid_sh, block, st, a, s, first_in_shade && depth == 0);
    }
    if ((e = timer->mark(1, st, false))) return e;
    // The vertex's shadow rays: sorted and traced on the side stream, beside
    // the next vertex's sort and closest-hit launch, which touch neither the
    // shadow records nor the radiance.
    cudaStream_t cs = st;
    int* shist = ws->mat_hist;
    if (overlap) {
      if ((e = cudaEventRecord(ws->ev_shaded, st))) return e;
      if ((e = cudaStreamWaitEvent(ws->side, ws->ev_shaded, 0))) return e;
      cs = ws->side;
      shist = ws->mat_hist2;
    }
    a.shadow_order = nullptr;
    if (p.sort_rays) {
      if ((e = cudaMemsetAsync(shist, 0, (kMaxSortBins + 1) * sizeof(int), cs))) return e;
      k_raykey_hist<true><<<grid_sh, 256, 0, cs>>>(a, ws->keys2, shist);
      k_sort_scan<<<1, 1024, 0, cs>>>(kRayKeyBins, shist);
      k_raykey_scatter<true><<<grid_sh, 256, 0, cs>>>(a, ws->keys2, shist, ws->shadow_order);
      *launches += 3;
      a.shadow_order = ws->shadow_order;  // the occlusion kernel visits records in key order
    }
    if ((e = timer->mark(2, cs, true))) return e;
    if (p.traversal == 2) {
      if (p.count_visits)
        k_connect_batch<true, true, kJobs><<<grid_con, block, 0, cs>>>(a, s);
      else
        k_connect_batch<false, true, kJobs><<<grid_con, block, 0, cs>>>(a, s);
    } else if (p.traversal == 0 || kJobs) {
      if (p.count_visits)
        k_connect_batch<true, false, kJobs><<<grid_con, block, 0, cs>>>(a, s);
      else
        k_connect_batch<false, false, kJobs><<<grid_con, block, 0, cs>>>(a, s);
    } else if (p.count_visits) {
      k_connect<true><<<grid_con, block, 0, cs>>>(a, s);
    } else {
      k_connect<false><<<grid_con, block, 0, cs>>>(a, s);
    }
    if ((e = timer->mark(2, cs, false))) return e;
    if (overlap && (e = cudaEventRecord(ws->ev_connected, cs))) return e;
    *launches += 2;
    ++*vertex_launches;  // one shading and one occlusion launch per path vertex
  }
  // the last occlusion launch before the accumulation reads the radiance
  if (overlap && (e = cudaStreamWaitEvent(st, ws->ev_connected, 0))) return e;
  return cudaSuccess;
}

cudaError_t pt_render(PtWorkspace* ws, const DeviceScene& s, const CamParams& cam,
                      const PtParams& p, float* d_out, int* err, Counters* d_counters,
                      KernelTimer* timer, cudaStream_t st, int* launches, int* extend_launches,
                      int* vertex_launches, std::string* why) {
  cudaError_t e;
  if (p.max_depth < 1 || p.max_depth > kMaxDepthSlots - 1) {
    *why = "max_depth must be in [1, 63]";
    return cudaErrorInvalidValue;
  }
  const bool jobs = p.n_jobs > 0;
  if (jobs && (p.per_path || p.traversal == 1)) {
    *why = "a batch renders images with the binary or 4-wide batch traversal";
    return cudaErrorInvalidValue;
  }
  long long npix = (long long)p.W * p.H;
  long long total = npix * p.n_samples;
  if (jobs) {
    const PtJob& L = p.h_jobs[p.n_jobs - 1];
    npix = L.pix_begin + L.npix;
    total = L.q_begin + (long long)L.npix * L.spp;
  }
  if (!p.per_path && !p.accumulate &&
      (e = cudaMemsetAsync(d_out, 0, (size_t)npix * 3 * sizeof(float), st)))
    return e;
  if (total == 0) return cudaSuccess;
  // Paths in flight: the whole render when it fits (every vertex launch has an
  // idle tail, so fewer, larger waves are faster), at most 2^26 paths and a
  // quarter of the free device memory (kPathBytes = 188 B per path).
  long long wave = p.wave_paths;
  if (wave <= 0) {
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    long long fit = (long long)(free_b / 4 / kPathBytes);
    wave = std::max(1LL << 20, std::min(1LL << 26, fit));
  }
  wave = std::min(wave, total);
  ws->last_wave = wave;
  if ((e = ws_reserve(ws, (size_t)wave)) != cudaSuccess) return e;
  int block = p.block > 0 ? p.block : 128;
  if (ws->num_sms == 0 || ws->block_cached != block) {
    int dev;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&ws->num_sms, cudaDevAttrMultiProcessorCount, dev);
    int o1 = 0, o2 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ws->occ_extend, k_extend<false>, block, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, k_extend_batch<false, false, false>, block, 0);
    ws->occ_extend = std::min(ws->occ_extend, o1);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, k_extend_batch<false, true, false>, block, 0);
    ws->occ_extend = std::min(ws->occ_extend, o1);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, k_extend_batch<false, false, true>, block, 0);
    ws->occ_extend = std::min(ws->occ_extend, o1);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, k_extend_batch<false, true, true>, block, 0);
    ws->occ_extend = std::min(ws->occ_extend, o1);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ws->occ_connect, k_connect<false>, block, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, k_connect_batch<false, false, false>, block, 0);
    ws->occ_connect = std::min(ws->occ_connect, o2);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, k_connect_batch<false, true, false>, block, 0);
    ws->occ_connect = std::min(ws->occ_connect, o2);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, k_connect_batch<false, false, true>, block, 0);
    ws->occ_connect = std::min(ws->occ_connect, o2);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, k_connect_batch<false, true, true>, block, 0);
    ws->occ_connect = std::min(ws->occ_connect, o2);
    ws->occ_shade = shade_occupancy<false>(block);
    ws->occ_shade_jobs = shade_occupancy<true>(block);
    ws->block_cached = block;
  }
  // The side stream and its events are made outside any stream capture (a
  // render captured before any uncaptured one runs without the overlap).
  bool overlap = p.overlap;
  if (overlap && !ws->side) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if ((e = cudaStreamIsCapturing(st, &cap))) return e;
    if (cap != cudaStreamCaptureStatusNone) {
      overlap = false;
    } else {
      if ((e = cudaStreamCreateWithFlags(&ws->side, cudaStreamNonBlocking))) return e;
      if ((e = cudaEventCreateWithFlags(&ws->ev_shaded, cudaEventDisableTiming))) return e;
      if ((e = cudaEventCreateWithFlags(&ws->ev_connected, cudaEventDisableTiming))) return e;
    }
  }
  int grid_ext = ws->num_sms * std::max(ws->occ_extend, 1);
  int grid_con = ws->num_sms * std::max(ws->occ_connect, 1);
  // the shading grid (also the sorts' grid) at the residency of the variant
  // this render launches
  int grid_sh = ws->num_sms * std::max(jobs ? ws->occ_shade_jobs : ws->occ_shade, 1);

  PtArgs a;
  a.ray_o = ws->ray_o;
  a.ray_d = ws->ray_d;
  a.thr = ws->thr;
  a.rad = ws->rad;
  a.absb = ws->absb;
  a.hit = ws->hit;
  a.shadow = ws->shadow;
  a.counts = ws->counters;
  a.shadow_counts = ws->counters + kMaxDepthSlots;
  a.work = ws->counters + 2 * kMaxDepthSlots;
  a.err = err;
  a.ctr = d_counters;
  a.npix = (int)npix;
  a.W = p.W;
  a.first_sample = p.first_sample;
  a.max_depth = p.max_depth;
  a.k0 = (uint32_t)p.seed;
  a.k1 = (uint32_t)(p.seed >> 32);
  a.min_busy = p.min_busy;
  a.jobs = p.d_jobs;
  a.job_q = p.d_job_q;
  a.n_jobs = p.n_jobs;
  float spp = (float)p.spp;

  const float4* prim = nullptr;
  if (p.primary_cache) {
    if (ws->prim_cap < (size_t)npix) {
      if (ws->prim) cudaFree(ws->prim);
      ws->prim = nullptr;
      ws->prim_cap = 0;
      if ((e = cudaMalloc(&ws->prim, (size_t)npix * sizeof(float4))) != cudaSuccess) return e;
      ws->prim_cap = (size_t)npix;
    }
    if (jobs) {
      for (int j = 0; j < p.n_jobs; ++j) {
        const PtJob& J = p.h_jobs[j];  // the launch shape only (W, H)
        int tiles = ((J.cam.W + 7) >> 3) * ((J.cam.H + 7) >> 3);
        k_primary_cache_job<<<tiles, 64, 0, st>>>(s, p.d_jobs, j, ws->prim, err, d_counters);
        ++*launches;
      }
    } else {
      int tiles = ((p.W + 7) >> 3) * ((p.H + 7) >> 3);
      k_primary_cache<<<tiles, 64, 0, st>>>(s, cam, ws->prim, err, d_counters);
      ++*launches;
    }
    prim = ws->prim;
  }

  for (long long q0 = 0; q0 < total; q0 += wave) {
    int nw = (int)std::min(wave, total - q0);
    a.q0 = q0;
    a.n_wave = nw;
    if ((e = cudaMemsetAsync(ws->counters, 0, kCounterInts * sizeof(int), st))) return e;
    e = jobs ? wave_launches<true>(p, a, s, cam, prim, ws, timer, st, grid_ext, grid_con, grid_sh, block, nw, launches,
                                   extend_launches, vertex_launches, overlap)
             : wave_launches<false>(p, a, s, cam, prim, ws, timer, st, grid_ext, grid_con, grid_sh, block, nw, launches,
                                    extend_launches, vertex_launches, overlap);
    if (e) return e;
    if (jobs) {
      k_accumulate_jobs<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(ws->rad, q0, nw, p.d_jobs, p.n_jobs,
                                                                        npix, d_out);
    } else {
      int acc_n = p.per_path ? nw : (int)npix;
      const bool last = !p.per_path && (p.resolve.display || p.resolve.bytes) && q0 + nw >= total;
      k_accumulate<<<(acc_n + 255) / 256, 256, 0, st>>>(ws->rad, q0, nw, (int)npix, spp, d_out,
                                                       p.per_path ? 1 : 0, p.resolve, last ? 1 : 0);
    }
    k_tally<<<1, 32, 0, st>>>(a.counts, a.shadow_counts, p.max_depth, prim ? 1 : 0, d_counters);
    *launches += 2;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace rtx
