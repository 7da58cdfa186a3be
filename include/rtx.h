/*
 * rtx.h — C ABI of librtx, the GB300 (sm_103a) implementation of RenderToy's
 * path-tracing hot path: camera rays, closest-hit traversal, Moller-Trumbore,
 * the principled BSDF with MIS and direct-light sampling, accumulation, the
 * normal / albedo / depth passes and the Compositor filters.
 *
 * Plain C: pointers, sizes and int status codes; no C++ or torch types.
 * Every entry point returns RTX_OK (0) or an RTX_ERR_* code; the message of the
 * last failure on a context is rtx_last_error().  Nothing throws.
 *
 * Buffers: image, ray and hit arrays may be HOST or DEVICE memory; each call
 * detects which (cudaPointerGetAttributes) and copies host data through its
 * own device buffers.  Images are packed float3, row-major, pixel (x, y) at
 * index y*W + x, row 0 at the bottom of the film (RenderToy's
 * RenderContext::buffer, include/RenderToy/renderer.h:44-62).
 *
 * Threading: a context is used by one host thread at a time.  Work runs on the
 * context's CUDA stream (rtx_get_stream / rtx_set_stream).  By default every
 * call returns after its work is complete; with RTX_OPT_ASYNC = 1, calls whose
 * buffers are all device memory return once their work is enqueued.
 *
 * Records shared with the caller:
 *   material (RTX_MATERIAL_FLOATS = 24 floats) — PrincipledBSDF,
 *     include/RenderToy/material.h:14-30:
 *       [0..2] base_color  [3..5] emission  [6] roughness  [7] metallic
 *       [8] anisotropic (unused by the BSDF, as in the reference)
 *       [9] subsurface  [10] specular_tint  [11] sheen  [12] sheen_tint
 *       [13] clearcoat  [14] clearcoat_roughness  [15] spec_trans  [16] ior
 *       [17] at_distance  [18..20] extinction
 *       [21] texture kind: 0 none, 1 checkerboard, 2 wave, 3 Perlin
 *       [22] the texture's parameter (CheckerBoard::scale, an integer;
 *            Wave::period; PerlinNoise::scale)  [23] texture units per world
 *            unit.  A textured material's base_color is scaled by
 *            0.25 + 0.75 * Sample(p), p = the hit point's two world
 *            coordinates across the dominant axis of the shading normal
 *            (x: (y, z); y: (x, z); z: (x, y)) times [23].  RenderToy's
 *            textures (src/procedural.cpp) only rasterise to images; this
 *            binding is an extension.  Zero in all three = untextured.
 *   camera (RTX_CAMERA_FLOATS = 21 floats) — Camera,
 *     include/RenderToy/object.h:69-95:
 *       [0..15] object-to-world 4x4, row-major  [16] focal length (mm)
 *       [17..18] gate dimension (inches)  [19] near  [20] far
 *   ray (6 floats): source xyz, direction xyz (not necessarily unit).
 *
 * Random numbers: RenderToy's shared mt19937 (src/rtmath.cpp:355-373) is
 * replaced by a counter-based stream.  Draw k of the path (pixel p, sample s)
 * is word (k & 3) of Philox4x32-10 (Salmon et al., SC'11) with key
 * (seed low, seed high) and counter (k >> 2, s, p, 0); Random::Float is
 * (w >> 8) * 2^-24 and Random::Int(a, b) is a + ((w * (b - a + 1)) >> 32).
 * Each shaded vertex draws, in order: emitter index, two for the point on the
 * emitter, two for the BSDF sample (src/world.cpp:9, src/object.cpp:171-172,
 * src/material.cpp:214-215).
 */
#ifndef RTX_H
#define RTX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RTX_VERSION 2
#define RTX_MATERIAL_FLOATS 24
#define RTX_CAMERA_FLOATS 21

enum rtx_status {
  RTX_OK = 0,
  RTX_ERR_INVALID = 1,   /* bad argument */
  RTX_ERR_CUDA = 2,      /* CUDA runtime error */
  RTX_ERR_NOMEM = 3,     /* device or host allocation failed */
  RTX_ERR_NO_SCENE = 4,  /* render or trace before rtx_scene_upload */
  RTX_ERR_DEVICE = 5     /* a kernel reported an error (see rtx_last_error) */
};

enum rtx_option {
  RTX_OPT_ASYNC = 1,          /* 0/1: return before device-only work ends */
  RTX_OPT_WAVE_PATHS = 2,     /* max paths in flight per wavefront (0 = auto:
                                 the whole render up to 2^26 paths and a
                                 quarter of the free device memory) */
  RTX_OPT_BLOCK = 3,          /* threads per block of the persistent wavefront
                                 kernels (extend, shade, connect): 64 or 128
                                 (their register budgets cap blocks at 128) */
  RTX_OPT_SORT_MATERIAL = 4,  /* 0 off, 1 on, 2 (default) on for scenes with a
                                 refracting material (spec_trans != 0) or 8
                                 materials or more: sort hits by material
                                 before shading (results unchanged) */
  RTX_OPT_COUNT_VISITS = 5,   /* 0/1: count node visits and triangle tests */
  RTX_OPT_LEAF_SIZE = 6,      /* max triangles per BVH leaf (1..8), next upload */
  RTX_OPT_PRIMARY_CACHE = 7,  /* 0/1: trace each pixel's primary ray once */
  RTX_OPT_KERNEL_TIMING = 8,  /* 0/1: CUDA events around each traversal and
                                 shading launch (rtx_stats.*_ms) */
  RTX_OPT_ACCUMULATE = 9,     /* 0/1: rtx_render_pt adds its mean to out_rgb
                                 (RenderToy's buffer +=, renderer.cpp:261)
                                 instead of overwriting it */
  RTX_OPT_TRAVERSAL = 10,     /* traversal kernels: 0 = binary tree, one ray per
                                 lane until the warp's batch is done; 1 = binary
                                 tree, lanes take new rays as theirs finish
                                 (while-while; single scenes only); 2 (default) =
                                 4-wide tree, batch */
  RTX_OPT_MIN_BUSY = 11,      /* with RTX_OPT_TRAVERSAL = 1: refill a warp once
                                 fewer lanes than this are traversing (0..32) */
  RTX_OPT_GRAPH = 12,         /* 0/1: rtx_render_batch captures its launch
                                 sequence as a CUDA graph and replays it for
                                 later frames of the same shape */
  RTX_OPT_SORT_RAYS = 13,     /* 0 off, 1 on, 2 (default) on for scenes of
                                 4,096 triangles or more: counting-sort the
                                 extension rays after the primary ones and
                                 the shadow rays by origin cell and direction
                                 before they are traced (results unchanged;
                                 only the visiting order; below ~4,000
                                 triangles the tree sits in L1 and the sorts
                                 cost more than they save) */
  RTX_OPT_STACK_LIMIT = 14,   /* traversal stack entries a ray may use, 2..64
                                 (default 64, the whole stack).  A ray that
                                 needs more stops, and the call returns
                                 RTX_ERR_DEVICE "traversal stack overflow".
                                 Lower values exist to exercise that error
                                 path; results are undefined after it. */
  RTX_OPT_COMPOSITOR_FMA = 15,/* 0/1 (default 0): the 3 x 3 and 5 x 5
                                 convolutions and the separable Gaussian /
                                 bloom passes fuse each tap's multiply and
                                 add (one rounding instead of two).  Results
                                 then differ from RenderToy's by at most
                                 ~1e-5 of the sum of the taps' magnitudes;
                                 0 keeps them bit-exact.  Other kernel shapes
                                 are always computed unfused. */
  RTX_OPT_OVERLAP = 16        /* 0/1 (default 1): each path vertex's shadow-ray
                                 sort and occlusion launch run on a second
                                 stream beside the next vertex's ray sort and
                                 closest-hit launch (they share no data), so
                                 one fills the other's idle tail; shading
                                 waits for both.  Results are unchanged. */
};

typedef struct rtx_context rtx_context;

typedef struct rtx_stats {
  uint64_t extension_rays;   /* closest-hit rays of the last render */
  uint64_t shadow_rays;      /* occlusion rays of the last render */
  uint64_t ext_node_visits;  /* with RTX_OPT_COUNT_VISITS: BVH nodes fetched */
  uint64_t ext_tri_tests;    /*   and triangles tested by closest-hit rays */
  uint64_t shadow_node_visits; /* ... and by occlusion rays */
  uint64_t shadow_tri_tests;
  uint64_t kernel_launches;  /* kernels launched by the last call */
  uint64_t extend_launches;  /* closest-hit traversal launches (last call) */
  double last_gpu_ms;        /* device time of the last call (CUDA events) */
  double extend_ms;          /* with RTX_OPT_KERNEL_TIMING: summed device time */
  double shade_ms;           /*   of the closest-hit, shading and occlusion */
  double connect_ms;         /*   launches of the last call */
  double bvh_build_ms;       /* host time of the last BVH build */
  int32_t bvh_nodes;         /* inner nodes of the current BVH */
  int32_t bvh_leaves;
  int32_t bvh_depth;
  int32_t node_bytes;        /* bytes per BVH node record of the tree in use
                                (64 binary, 112 4-wide) */
  int32_t tri_bytes;         /* bytes per triangle record */
  int32_t reserved;
  uint64_t ext_rays_by_depth[16]; /* closest-hit rays per path vertex 0..15 */
  uint64_t shade_launches;   /* shading launches of the last call (one per */
  uint64_t connect_launches; /*   path vertex and wave), occlusion launches */
} rtx_stats;

/* ---- context ------------------------------------------------------------ */
int rtx_create(rtx_context** out, int device);
void rtx_destroy(rtx_context* ctx);
const char* rtx_last_error(const rtx_context* ctx);
int rtx_version(void);
int rtx_set_option(rtx_context* ctx, int option, int64_t value);
int rtx_get_option(rtx_context* ctx, int option, int64_t* value);
/* the CUDA stream (a cudaStream_t) work is enqueued on */
void* rtx_get_stream(rtx_context* ctx);
int rtx_set_stream(rtx_context* ctx, void* stream);
int rtx_synchronize(rtx_context* ctx);
int rtx_get_stats(rtx_context* ctx, rtx_stats* out);

/* ---- scene ---------------------------------------------------------------
 * Replaces RenderContext::RenderContext's BVH build (src/renderer.cpp:77-85,
 * BVH::BVH src/bvh.cpp:242-264) and World::PrepareDirectLightSampling
 * (src/world.cpp:24-37).  verts: n_tris x 9 world-space floats (v0, v1, v2 of
 * World::triangles in order, Triangle::vert_w, include/RenderToy/object.h:161);
 * norms: n_tris x 9 per-vertex normals (Triangle::norm; may be NULL when no
 * mesh is smooth); tri_mesh: the mesh (Triangle::parent) of each triangle;
 * mesh_mat / mesh_smooth: Mesh::tex as an index into materials, Mesh::smooth;
 * sky / ground: World::sky_emission / ground_reflection.  Emitters are the
 * triangles of meshes whose emission is not zero, in mesh order then triangle
 * order, as the reference collects them.  The arrays are copied; the
 * caller's buffers may be released on return.  The BVH is built on host
 * threads (the same tree for any thread count).  A triangle with a
 * non-finite vertex is accepted and never hit.  A host allocation that fails
 * returns RTX_ERR_NOMEM, as rtx_batch_upload and rtx_batch_autotune do. */
int rtx_scene_upload(rtx_context* ctx, int n_tris, const float* verts,
                     const float* norms, const int32_t* tri_mesh, int n_meshes,
                     const int32_t* mesh_mat, const uint8_t* mesh_smooth,
                     int n_materials, const float* materials, const float* sky,
                     const float* ground);
/* emitter triangle ids in sampling order; returns the count in *n_out */
int rtx_scene_emitters(rtx_context* ctx, int32_t* out, int cap, int* n_out);
/* Replace the emitter list by an explicit one (ids in sampling order), as
 * World::PrepareDirectLightSampling left it (src/world.cpp:24-37); n = 0
 * disables light sampling, as in a World where it was never called. */
int rtx_scene_set_emitters(rtx_context* ctx, const int32_t* ids, int n);
/* The 256-entry permutation the Perlin texture hashes through
 * (siv::BasicPerlinNoise's m_permutation; default: a fixed seeded shuffle).
 * Applies to the current and later scenes of the context. */
int rtx_scene_set_texture_table(rtx_context* ctx, const uint8_t* perm);
/* RenderToy's ProceduralTexture samplers at n points (uv: n x 2 floats):
 * kind 1 CheckerBoard(scale = (int)param), 2 Wave(period = param),
 * 3 PerlinNoise with scale = param, time 0, 4 octaves (src/procedural.cpp:
 * 8-46), evaluated by the device code that shades textured materials. */
int rtx_texture_sample(rtx_context* ctx, int kind, float param, int n,
                       const float* uv, float* out);

/* ---- OBJ / MTL import --------------------------------------------------------
 * OBJModelImporter::Import and MTLImporter::Import (src/importer.cpp:29-229)
 * straight into the arrays rtx_scene_upload takes, with RenderToy's token
 * rules, fan triangulation (Polygon::ConvertToTriangle, src/object.cpp:
 * 333-342) and triangle order: triangles in World::triangles order; each
 * mesh's triangle list in Mesh::tris order (every face's block PREPENDED,
 * importer.cpp:136), which is the order its emitters are sampled in -- pass
 * it to rtx_scene_set_emitters.  Like the reference, an "s" value other than
 * 0 / 1 or an unreadable number ends the import silently with what was read;
 * "usemtl" is ignored (materials are assigned by the caller, by name).  Where
 * the reference has undefined behaviour (face index out of range, more than
 * three '/' fields, "s" / "f" before any "o", an MTL key before any
 * "newmtl") the import fails with RTX_ERR_INVALID and a message in msg. */
typedef struct rtx_obj rtx_obj;
int rtx_obj_import(const char* obj_path /* or NULL: MTL only */,
                   const char* mtl_path /* or NULL */, rtx_obj** out,
                   char* msg, size_t msg_len);
void rtx_obj_free(rtx_obj* obj);
int rtx_obj_info(const rtx_obj* obj, int* n_tris, int* n_meshes,
                 int* n_materials);
/* verts / norms: n_tris x 9 floats (world space, v0 v1 v2), uvs n_tris x 6,
 * tri_mesh n_tris; any pointer may be NULL */
int rtx_obj_triangles(const rtx_obj* obj, float* verts, float* norms,
                      float* uvs, int32_t* tri_mesh);
/* mesh `mesh`: its name (valid until rtx_obj_free), smooth flag and its
 * triangle ids in Mesh::tris order (tris may be NULL to query *n_tris) */
int rtx_obj_mesh(const rtx_obj* obj, int mesh, const char** name,
                 uint8_t* smooth, int32_t* tris, int* n_tris);
/* material `mat` of the MTL file: its name and 24-float record */
int rtx_obj_material(const rtx_obj* obj, int mat, const char** name,
                     float* record);

/* ---- multi-scene batches ------------------------------------------------------
 * No counterpart in RenderToy (one World per RenderContext).  Several scenes
 * are merged into one set of device arrays (each with its own BVH, materials
 * and emitter list); rtx_render_batch then traces frames over any of them --
 * uneven sizes, resolutions and spp -- through one wavefront: every kernel
 * launch of the frame serves the rays of all frames.  Each frame's random
 * stream is the one rtx_render_pt uses for its scene, camera and seed, so a
 * frame of a batch equals the frame rendered alone.  The batch is separate
 * from the context's single scene (rtx_scene_upload). */
typedef struct rtx_scene_desc {
  int n_tris;
  const float* verts;          /* as rtx_scene_upload */
  const float* norms;
  const int32_t* tri_mesh;
  int n_meshes;
  const int32_t* mesh_mat;
  const uint8_t* mesh_smooth;
  int n_materials;
  const float* materials;
  const float* sky;
  const float* ground;
  const int32_t* emitters;     /* sampling order, or NULL with n_emitters = -1
                                  for World::PrepareDirectLightSampling's */
  int n_emitters;
} rtx_scene_desc;
int rtx_batch_upload(rtx_context* ctx, int n_scenes, const rtx_scene_desc* scenes);

typedef struct rtx_job {
  int scene;                   /* index into the uploaded batch */
  float camera[RTX_CAMERA_FLOATS];
  int W, H, spp;
  uint64_t seed;
} rtx_job;
/* out: the frames' images one after another (sum of W * H * 3 floats) */
int rtx_render_batch(rtx_context* ctx, int n_jobs, const rtx_job* jobs,
                     int max_depth, float* out);

/* Autotuner: times the batch frame `jobs` (device time of rtx_render_batch,
 * best of two) over BVH leaf sizes 2 / 4 / 8 -- rebuilding the batch from
 * `scenes` for each; scenes = NULL keeps the uploaded batch and its leaf
 * size -- then threads per block 64 / 128 x paths per wave 2^20, 2^22, 2^24,
 * auto, then the binary or 4-wide tree, then material-sorted shading on /
 * off, then ray-sorted traversal on / off, then the occlusion / closest-hit
 * overlap on / off, coordinate-wise from the context's current options.  The
 * fastest setting stays on the context (RTX_OPT_LEAF_SIZE, RTX_OPT_BLOCK,
 * RTX_OPT_WAVE_PATHS, RTX_OPT_TRAVERSAL, RTX_OPT_SORT_MATERIAL,
 * RTX_OPT_SORT_RAYS, RTX_OPT_OVERLAP) and the batch is left built with it. */
typedef struct rtx_tune_result {
  int64_t block, wave_paths, leaf_size;
  double ms, ms_default;       /* frame time chosen / at the starting options */
  int trials;
  int sort_material;           /* RTX_OPT_SORT_MATERIAL chosen */
  int traversal;               /* RTX_OPT_TRAVERSAL chosen (0 or 2) */
  int sort_rays;               /* RTX_OPT_SORT_RAYS chosen */
  int overlap;                 /* RTX_OPT_OVERLAP chosen */
} rtx_tune_result;
int rtx_batch_autotune(rtx_context* ctx, int n_scenes,
                       const rtx_scene_desc* scenes, int n_jobs,
                       const rtx_job* jobs, int max_depth,
                       rtx_tune_result* out);

/* ---- renderers ------------------------------------------------------------
 * PathTracingRenderer::Render (src/renderer.cpp:236-270): out_rgb[p] =
 * sum over samples s = 0..spp-1 of L(p, s) / spp, summed in sample order;
 * max_depth = shaded vertices per path (the reference's fixed value is 5,
 * src/renderer.cpp:274). */
int rtx_render_pt(rtx_context* ctx, const float* camera, int W, int H, int spp,
                  int max_depth, uint64_t seed, float* out_rgb);
/* Progressive rendering, checkpoint and resume.  RenderToy renders all of a
 * frame's samples in one call (src/renderer.cpp:236-270) and keeps nothing to
 * resume from.  Here out[p] += sum over s = first_sample ..
 * first_sample + n_samples - 1 of L(p, s) / spp, in sample order
 * (first_sample = 0 overwrites out instead), 0 <= first_sample <
 * first_sample + n_samples <= spp.  A checkpoint is the image, the next
 * sample index and the call's camera, size, spp, max_depth and seed;
 * continuing from it -- in this or any other context with the same scene --
 * gives, bit for bit, the image one rtx_render_pt(spp) call renders. */
int rtx_render_pt_progressive(rtx_context* ctx, const float* camera, int W,
                              int H, int first_sample, int n_samples, int spp,
                              int max_depth, uint64_t seed, float* out_rgb);
/* Per-path radiance L(p, s) for samples first_sample .. first_sample+n-1:
 * out[(s - first_sample) * W*H + p] (PathTracingRenderer::Radiance,
 * src/renderer.cpp:272-333, one call per (pixel, sample)). */
int rtx_trace_paths(rtx_context* ctx, const float* camera, int W, int H,
                    int first_sample, int n_samples, int max_depth,
                    uint64_t seed, float* out_rgb);
/* NormalRenderer / AlbedoRenderer / DepthBufferRenderer::Render
 * (src/renderer.cpp:138-229, 391-427) in one primary pass; any output may be
 * NULL.  near/far as DepthBufferRenderer(ctx, near, far). */
int rtx_render_aov(rtx_context* ctx, const float* camera, int W, int H,
                   float near_, float far_, float* out_normal,
                   float* out_albedo, float* out_depth);
/* BVH::Intersect (src/bvh.cpp:266-341) of the W x H primary rays:
 * out_tri[p] (-1 on a miss), out_tuv[3p..3p+2] = t, u, v (1e7, 0, 0 on miss) */
int rtx_primary_hits(rtx_context* ctx, const float* camera, int W, int H,
                     int32_t* out_tri, float* out_tuv);
/* BVH::Intersect of n arbitrary rays; exclude[i] = triangle skipped (-1 none;
 * exclude may be NULL). */
int rtx_intersect(rtx_context* ctx, int n, const float* rays,
                  const int32_t* exclude, int32_t* out_tri, float* out_tuv);

/* PrincipledBSDF::Eval (src/material.cpp:143-204) of n independent cases,
 * by the device code the shading kernel inlines -- for checking the BSDF on
 * its own.  Case i: mats[24 i ..] (a material record; a device array must be
 * 16-byte aligned), eta[i], shading normal N[3 i ..], outgoing V[3 i ..] and
 * incoming L[3 i ..] (world space); out_f[3 i ..] = f * |L.z| and
 * out_pdf[i], as Eval returns them. */
int rtx_bsdf_eval(rtx_context* ctx, int n, const float* mats, const float* eta,
                  const float* N, const float* V, const float* L, float* out_f,
                  float* out_pdf);
/* PrincipledBSDF::Sample (src/material.cpp:206-295) of n cases: case i
 * samples from direction in_dir[3 i ..] with the two numbers that path
 * (pixel i, sample `sample`) of seed `seed` draws first (the Random::Float
 * calls of material.cpp:214-215).  out_ok[i] = Sample's return value. */
int rtx_bsdf_sample(rtx_context* ctx, int n, const float* mats, const float* eta,
                    const float* N, const float* in_dir, uint64_t seed, int sample,
                    int32_t* out_ok, float* out_dir, float* out_color,
                    float* out_pdf);

/* Measurement aid, no RenderToy counterpart: the read bandwidth (GB/s) of a
 * plain streaming kernel over one `bytes` device buffer (a multiple of 16),
 * read `passes` times in one launch after one untimed pass.  A buffer that
 * fits the L2 cache measures L2 bandwidth: the bound of traversal over a tree
 * and triangle array that stay L2-resident. */
int rtx_probe_read_bandwidth(rtx_context* ctx, size_t bytes, int passes,
                             double* gbs);

/* Diagnostic, no RenderToy counterpart: one block waits on a shared-memory
 * mbarrier that nothing arrives on, through the bounded wait every
 * tensor-core kernel uses, giving up after `polls` polls (1..2^20).  The
 * call then returns what such a kernel's failed wait returns:
 * RTX_ERR_DEVICE with "tensor-core barrier wait timed out", and the context
 * stays usable. */
int rtx_selftest_wait_timeout(rtx_context* ctx, int polls);

/* rtx_render_pt, and in the same pass as the last accumulation the display
 * resolve of the mean (see rtx_image_resolve): display (W x H RGB FP32) and
 * bytes (format as rtx_image_resolve) may each be NULL; out is the radiance. */
int rtx_render_pt_resolved(rtx_context* ctx, const float* camera, int W, int H,
                           int spp, int max_depth, uint64_t seed, float* out,
                           float limit, float gamma, float* display,
                           uint8_t* bytes, int format);

/* ---- display resolve and image files ----------------------------------------
 * Image::Tonemap<kITURBT709>(limit): p * 1 / (1 + Luma709(p) / limit)
 * (include/RenderToy/compositor.h:220-226, rtmath.h:1142-1177), then
 * Image::GammaCorrection(gamma): p^(1 / gamma) per channel
 * (src/compositor.cpp:94-100), then the exporters' quantisation
 * int(255.99 * clamp(x, 0, 1)), NaN -> 0 (src/exporter.cpp:8-95; there
 * int(NaN) is undefined: on x86 the BMP gets 0 and the PPM -2147483648).
 * limit <= 0 skips the tonemap and gamma <= 0 the gamma correction. */
#define RTX_BYTES_BMP 0 /* BMP pixel array: rows of B, G, R bytes, buffer row 0
                           first, each row zero-padded to a multiple of 4 */
#define RTX_BYTES_RGB 1 /* R, G, B bytes per pixel in buffer order */
int rtx_image_resolve(rtx_context* ctx, const float* in, int W, int H,
                      float limit, float gamma, float* display, uint8_t* bytes,
                      int format);
int rtx_image_tonemap(rtx_context* ctx, const float* in, float* out, int W,
                      int H, float limit);
int rtx_image_gamma(rtx_context* ctx, const float* in, float* out, int W, int H,
                    float gamma);
/* BMPExporter::Export (src/exporter.cpp:38-95) into memory: 54-byte header +
 * the BMP pixel array of the image (quantised as above, no tonemap).  The
 * padding bytes are zeros (the reference writes them from a null pointer)
 * and the header's file size counts them.  file = NULL queries *size. */
int rtx_encode_bmp(rtx_context* ctx, const float* in, int W, int H,
                   uint8_t* file, size_t cap, size_t* size);
/* PPMExporter::Export (src/exporter.cpp:8-29) into memory: "P3" text, one
 * "r g b" line per pixel, buffer row 0 first.  file = NULL queries *size. */
int rtx_encode_ppm(rtx_context* ctx, const float* in, int W, int H, char* file,
                   size_t cap, size_t* size);

/* ---- compositor ------------------------------------------------------------
 * Image operations (include/RenderToy/compositor.h:107-178,
 * src/compositor.cpp:42-77) on packed float3 W x H images (H <= 65535:
 * the row passes launch one block row per image row; RTX_ERR_INVALID above).
 * in == out is allowed (the input is copied first, as RenderToy filters a
 * copy of the image).  Edge taps use the reference's reflect mapping
 * (compositor.h:25-39); a tap whose linear index falls outside the image
 * reads zero. */
/* Image::Convolute<normalize, length, abs>(k): k is kr x kc, row-major */
int rtx_image_convolve(rtx_context* ctx, const float* in, float* out, int W,
                       int H, const float* kernel, int kr, int kc,
                       int normalize, int length, int absval);
/* Image::GaussianBlur(size, sigma) */
int rtx_image_gaussian_blur(rtx_context* ctx, const float* in, float* out,
                            int W, int H, int size, float sigma);
/* Image::EdgeDetection<Orientation::All>() */
int rtx_image_edge_detect(rtx_context* ctx, const float* in, float* out, int W,
                          int H);
/* Image::Bloom(size, sigma, threshold) */
int rtx_image_bloom(rtx_context* ctx, const float* in, float* out, int W,
                    int H, int size, float sigma, float threshold);

/* ---- denoiser building blocks (no RenderToy counterpart) --------------------
 * C[M x N] (FP32) = A * B^T on the tcgen05 tensor cores with BF16 operands:
 * A is M x K row-major (K contiguous), or K x M (M contiguous) when a_mn;
 * B is N x K, or K x N when b_mn.  The contiguous dimension must be a
 * multiple of 8. */
int rtx_nn_gemm_bf16(rtx_context* ctx, int M, int N, int K, const void* A,
                     const void* B, float* C, int a_mn, int b_mn);

/* One 3 x 3 "same" convolution of the denoiser, for validating its kernels
 * operator by operator.  Tensors are NHWC BF16 (uint16 bit patterns): the
 * input is the channel concatenation of x1 (C1 channels; stored at half
 * resolution and read upsampled by nearest neighbour when up1 != 0) and x2
 * (C2 channels, may be NULL with C2 = 0); Cin = C1 + C2.  C1, C2 multiples
 * of 8; Cout a multiple of 16 and <= 256.
 *   fwd  : out[P][Cout] (FP32) = relu?(bias + conv(x, w)), w [Cout][9][Cin]
 *   dgrad: din[P][Cin] (BF16) = conv^T(dout, wt) * (x > 0 if mask_relu),
 *          wt [Cin][9][Cout], Cin a multiple of 16
 *   wgrad: dw[Cout][9][Cin] (FP32) = sum_p dout[p] x[p + tap]; Cout a
 *          multiple of 16 and <= 256
 * P = N * H * W at the convolution's resolution. */
int rtx_nn_conv3x3_fwd(rtx_context* ctx, int N, int H, int W, const void* x1,
                       int C1, int up1, const void* x2, int C2, const void* w,
                       const float* bias, int Cout, int relu, float* out);
int rtx_nn_conv3x3_dgrad(rtx_context* ctx, int N, int H, int W,
                         const void* dout, int Cout, const void* wt,
                         const void* x1, int C1, int up1, const void* x2,
                         int C2, int mask_relu, void* din);
int rtx_nn_conv3x3_wgrad(rtx_context* ctx, int N, int H, int W,
                         const void* dout, int Cout, const void* x1, int C1,
                         int up1, const void* x2, int C2, float* dw);

/* ---- learned denoiser -------------------------------------------------------
 * No counterpart in RenderToy: its demos hand the path tracer's buffer to
 * Intel OIDN, a closed binary (demo/WithOIDN/main.cpp:60).  This is a 5-level
 * U-Net (3 x 3 convolutions of 32 / 64 / 96 / 128 / 160 channels, 2 x 2
 * average pooling, nearest upsampling, skip concatenation; 14 layers), run
 * and trained on the tensor cores in BF16 with FP32 accumulation.
 * Input, per pixel, 11 FP32 channels: radiance RGB (linear), albedo RGB,
 * normal RGB (encoded (n + 1) / 2 as the normal pass writes it), depth, and
 * the radiance's samples per pixel (the same over a frame).  The network
 * predicts, per pixel, a 5 x 5 filter (the softmax of 25 logits) that is
 * applied to the input radiance (taps clamped to the frame): the denoised
 * radiance is a weighted mean of input pixels.  Training minimises the
 * relative squared error (o - t)^2 / (o^2 + 0.01) of the filtered radiance o
 * against the target t, the prediction in the denominator held constant, with
 * Adam (beta 0.9 / 0.999, eps 1e-8).
 * Batches are [N][H][W][11] with H and W multiples of 16.  Parameters are one
 * FP32 array in the padded layout rtx_dn_layer describes. */
int rtx_dn_init(rtx_context* ctx, uint64_t seed);
/* n_params: FP32 entries of the padded array; n_real: parameters of the
 * network proper; n_layers: 14; step: Adam steps taken */
int rtx_dn_info(rtx_context* ctx, int64_t* n_params, int64_t* n_real,
                int* n_layers, int* step);
/* info[11] = cout_pad, cout, cin_pad, cin, c1_pad (channels of the first
 * source; the rest come from the skip connection), up1 (first source read
 * upsampled), relu, level (resolution = full >> level), w_off, b_off (float
 * offsets of w [cout_pad][9][cin_pad] and b [cout_pad]), first source id */
int rtx_dn_layer(rtx_context* ctx, int layer, int64_t info[11]);
int rtx_dn_get_params(rtx_context* ctx, float* out);
int rtx_dn_set_params(rtx_context* ctx, const float* in);
int rtx_dn_get_grads(rtx_context* ctx, float* out);
int rtx_dn_get_adam(rtx_context* ctx, float* m, float* v);
int rtx_dn_set_adam(rtx_context* ctx, const float* m, const float* v,
                    int step);
/* forward + loss + backward without an update (the gradients stay readable
 * with rtx_dn_get_grads); *loss = mean over pixels and channels */
int rtx_dn_loss_grads(rtx_context* ctx, const float* input, const float* target,
                      int N, int H, int W, double* loss);
/* one Adam step on a minibatch; *loss = the minibatch loss before the step */
int rtx_dn_train_step(rtx_context* ctx, const float* input, const float* target,
                      int N, int H, int W, float lr, double* loss);
/* out [N][H][W][3] = the denoised radiance */
int rtx_dn_infer(rtx_context* ctx, const float* input, float* out, int N, int H,
                 int W);
/* Denoise one frame from the renderer's passes, each W x H RGB FP32 as
 * rtx_render_pt / rtx_render_aov write them (depth: channel 0 is used), the
 * radiance rendered at `spp` samples per pixel.  Any W, H: the frame is
 * padded to multiples of 16 on the device (the filters never read the
 * padding). */
int rtx_denoise(rtx_context* ctx, const float* radiance, const float* albedo,
                const float* normal, const float* depth, int spp, float* out,
                int W, int H);

/* ---- without allocation -----------------------------------------------------
 * No counterpart in RenderToy.  Image::GaussianBlur (as rtx_image_gaussian_blur)
 * for callers that cannot allocate device memory when they call in: a plugin
 * whose host application owns the device-memory budget, or a real-time loop in
 * which cudaMalloc / cudaFree would synchronise the device.  d_in / d_out are
 * device images on the current device (in == out allowed); the work is
 * enqueued on `stream` (a cudaStream_t; NULL = the default stream) and the
 * call returns without waiting.  The intermediate image lives in a fixed
 * 24 MiB device array that the library keeps on every GPU that loads it until
 * the process exits: W * H <= 2097152, H <= 65535 and size <= 255, otherwise
 * RTX_ERR_INVALID.  All calls share that array, so calls whose work overlaps
 * on the GPU race: serialise them.  The first call on a device looks the
 * array's address up (cudaGetSymbolAddress) and keeps it for the process:
 * make that first call before any stream capture, and do not call across a
 * cudaDeviceReset.  If a CUDA error of earlier work is pending on the calling
 * thread, the call enqueues nothing, leaves that error in place and returns
 * RTX_ERR_CUDA.  msg (may be NULL) receives a message on failure.  Calls no
 * cudaMalloc, cudaFree or other allocating routine. */
int rtx_image_gaussian_blur_noalloc(const float* d_in, float* d_out, int W,
                                    int H, int size, float sigma, void* stream,
                                    char* msg, size_t msg_len);

#ifdef __cplusplus
}
#endif
#endif /* RTX_H */
