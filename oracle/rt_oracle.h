/*
 * rt_oracle.h — C API of the CPU oracle for RenderToy's path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a CPU restatement of the reference
 * algorithm (RenderToy, src/bvh.cpp, src/object.cpp, src/material.cpp,
 * src/rtmath.cpp, src/renderer.cpp, src/world.cpp, include/RenderToy/
 * compositor.h, src/compositor.cpp).  It is used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg, always as the
 * checker or as the timed CPU baseline; it is never linked into, or called by,
 * the product library (librtx).
 *
 * The same entry points (prefix ref_ instead of orc_) are exported by the
 * harness in oracle/ref_harness.cpp, which links the reference's own sources;
 * that is how the restatement is pinned to the reference (tests/golden).
 *
 * Conventions shared with the product C-ABI (include/rtx.h):
 *   - material = 24 floats, see RTX_MATERIAL_FLOATS in include/rtx.h;
 *   - camera   = 21 floats: o2w[16] row-major, focal_mm, gate_x_in, gate_y_in,
 *                near, far;
 *   - ray      = 6 floats: src xyz, dir xyz;
 *   - images   = packed float3, row-major, pixel (x, y) at index y*W + x.
 *   - RNG: Philox4x32-10 keyed by the 64-bit seed, counter
 *     (draw >> 2, sample, pixel, 0), word draw & 3 (see rtx.h).
 */
#ifndef RT_ORACLE_H
#define RT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

void* orc_scene_create(int n_tris, const float* verts, const float* norms,
                       const int32_t* tri_mesh, int n_meshes,
                       const int32_t* mesh_mat, const uint8_t* mesh_smooth,
                       int n_mat, const float* mats, const float* sky,
                       const float* ground);
void orc_scene_destroy(void* scene);
int orc_scene_emitters(void* scene, int32_t* out, int cap);
/* display resolve (limit / gamma <= 0 skip) and the exporters' files */
void orc_tonemap_gamma(const float* in, int W, int H, float limit, float gamma,
                       float* out);
long orc_encode(int bmp, const float* in, int W, int H, uint8_t* out, long cap);
/* the Perlin texture's permutation (default: include/rtx.h's seeded shuffle) */
void orc_scene_set_texture_table(void* scene, const uint8_t* perm);
/* procedural texture samplers at n points (perm NULL = the default table) */
void orc_texture_sample(int kind, float param, const uint8_t* perm, int n,
                        const float* uv, float* out);

/* closest hit of n rays; exclude[i] = triangle id to skip (-1 none).
 * out_tri[i] = id or -1, out_tuv[3i..] = t,u,v (t = 1e7 and u=v=0 on miss). */
void orc_intersect(void* scene, int n, const float* rays, const int32_t* exclude,
                   int32_t* out_tri, float* out_tuv, int threads);

/* primary hits of the W x H camera rays */
void orc_primary(void* scene, const float* cam, int W, int H, int32_t* out_tri,
                 float* out_tuv, int threads);

/* AOV passes (any output pointer may be NULL) */
void orc_render_aov(void* scene, const float* cam, int W, int H, float near_,
                    float far_, float* normal, float* albedo, float* depth,
                    int threads);

/* per-path radiance: out[(s*npix + p)*3] for samples first..first+n_samples-1
 * of the pixels listed in pixels[] (NULL = all W*H pixels, npix = W*H). */
void orc_trace_paths(void* scene, const float* cam, int W, int H,
                     const int32_t* pixels, int npix, int first_sample,
                     int n_samples, int max_depth, uint64_t seed, float* out,
                     int threads);

/* accumulated image: out[p] = sum_s L(p,s) / spp, summed in sample order */
void orc_render_pt(void* scene, const float* cam, int W, int H, int spp,
                   int max_depth, uint64_t seed, float* out, int threads);

/* BSDF entry points for unit parity (material = 24 floats) */
void orc_bsdf_eval(const float* mat, float eta, const float* N, const float* V,
                   const float* L, float* f_out, float* pdf_out);
int orc_bsdf_sample(const float* mat, float eta, const float* N,
                    const float* in_dir, uint64_t seed, uint32_t pixel,
                    uint32_t sample, float* out_dir, float* color,
                    float* pdf_out);

/* Compositor (images packed float3, W x H) */
void orc_convolve(const float* in, float* out, int W, int H, const float* k,
                  int kr, int kc, int normalize, int length, int absval);
void orc_gaussian_blur(const float* in, float* out, int W, int H, int size,
                       float sigma);
void orc_edge_detect(const float* in, float* out, int W, int H);
void orc_bloom(const float* in, float* out, int W, int H, int size, float sigma,
               float threshold);
void orc_gaussian_weights(int size, float sigma, float* out);

/* RNG spec check: n uniform floats of path (seed, pixel, sample) */
void orc_rng_floats(uint64_t seed, uint32_t pixel, uint32_t sample, int n,
                    float* out);

#ifdef __cplusplus
}
#endif
#endif
