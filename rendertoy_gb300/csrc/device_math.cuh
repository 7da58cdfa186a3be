// device_math.cuh — float3 arithmetic, principled BSDF and RNG on the device,
// in RenderToy's evaluation order.
//
// This header is compiled with --fmad=false: no multiply-add is fused unless
// written as __fmaf_rn, so +, -, *, / and sqrtf round exactly as in the
// reference's x86/Arm builds; only the transcendental functions (sinf, cosf,
// powf, logf) may differ by an ulp from the host C library.
//
// Each function names the reference function it restates
// (RenderToy src/rtmath.cpp, src/material.cpp, include/RenderToy/rtmath.h).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rtx {

#define RTX_DEV __device__ __forceinline__
// The BSDF lobes are called from both Eval and Sample.  Inlined (the
// default) the shading kernel is larger but avoids the call sequences and
// their register saves: measured 3.3 % more samples per second on GB300 than
// compiling each lobe once (RTX_LOBE_NOINLINE).
#ifdef RTX_LOBE_NOINLINE
#define RTX_LOBE static __device__ __noinline__
#else
#define RTX_LOBE RTX_DEV
#endif

// Two FP32 lanes in one 64-bit register: Blackwell's packed FP32
// instructions (.f32x2) round each lane exactly as the scalar instruction
// does.  They occupy the FMA pipe for two cycles, so they save issue slots,
// not FMA throughput.
typedef unsigned long long f2_t;
RTX_DEV f2_t f2_pack(float lo, float hi) {
  f2_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
RTX_DEV void f2_unpack(f2_t v, float& lo, float& hi) { asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v)); }
// a * b + c, one rounding per lane
RTX_DEV f2_t f2_fma(f2_t a, f2_t b, f2_t c) {
  f2_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
RTX_DEV f2_t f2_add(f2_t a, f2_t b) {
  f2_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
// three-input minimum / maximum (one instruction on sm_100 and later)
RTX_DEV float fmin3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
RTX_DEV float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

struct F3 {
  float x, y, z;
};
RTX_DEV F3 f3(float x, float y, float z) { return F3{x, y, z}; }
RTX_DEV F3 f3s(float s) { return F3{s, s, s}; }
RTX_DEV F3 operator+(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
RTX_DEV F3 operator-(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
RTX_DEV F3 operator-(F3 a) { return F3{-a.x, -a.y, -a.z}; }
RTX_DEV F3 operator*(F3 a, F3 b) { return F3{a.x * b.x, a.y * b.y, a.z * b.z}; }
RTX_DEV F3 operator*(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
RTX_DEV F3 operator/(F3 a, float s) { return F3{a.x / s, a.y / s, a.z / s}; }
// Vector::Dot (rtmath.h:328-338): accumulate from zero, x, y, z
RTX_DEV float dot(F3 a, F3 b) {
  float r = 0.0f;
  r = r + a.x * b.x;
  r = r + a.y * b.y;
  r = r + a.z * b.z;
  return r;
}
RTX_DEV float length(F3 a) { return sqrtf(dot(a, a)); }
// Vector::Normalize (rtmath.h:144-150): divide by the length
RTX_DEV F3 normalized(F3 a) {
  float l = length(a);
  return F3{a.x / l, a.y / l, a.z / l};
}
RTX_DEV F3 cross(F3 a, F3 b) {
  return F3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// Vector::operator== (rtmath.h:296-308): epsilon test; NaN compares equal
RTX_DEV bool eq_zero_eps(F3 a) {
  if (fabsf(a.x) > 1e-7f) return false;
  if (fabsf(a.y) > 1e-7f) return false;
  if (fabsf(a.z) > 1e-7f) return false;
  return true;
}
RTX_DEV float lerp(float x, float y, float a) { return x * (1.0f - a) + y * a; }
RTX_DEV F3 lerpv(F3 x, F3 y, F3 a) { return x * (f3s(1.0f) - a) + y * a; }
RTX_DEV float luma(F3 v) { return 0.2126f * v.x + 0.7152f * v.y + 0.0722f * v.z; }

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInf = 1e7f;
constexpr float kE = 2.718281828459045235360287471352662498f;

// ---------------------------------------------------------------------------
// Philox4x32-10 stream (see include/rtx.h)
// ---------------------------------------------------------------------------
RTX_DEV uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

struct Rng {
  uint32_t k0, k1, pixel, sample, draw;
  RTX_DEV uint32_t next_u32() {
    uint4 r = philox4x32_10(make_uint4(draw >> 2, sample, pixel, 0u), k0, k1);
    uint32_t s = draw & 3u;
    ++draw;
    return s == 0 ? r.x : (s == 1 ? r.y : (s == 2 ? r.z : r.w));
  }
  RTX_DEV float uniform() { return to_uniform(next_u32()); }
  RTX_DEV int uniform_int(int a, int b) { return to_int(next_u32(), a, b); }
  static RTX_DEV float to_uniform(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }
  static RTX_DEV int to_int(uint32_t u, int a, int b) {
    uint32_t n = (uint32_t)(b - a + 1);
    return a + (int)(((uint64_t)u * (uint64_t)n) >> 32);
  }
  // The next five draws (a shading vertex makes at most five): they lie in
  // the two consecutive Philox blocks from draw >> 2, computed here by one
  // copy of the rounds; draw advances by `used` afterwards.
  RTX_DEV void draw5(uint32_t (&v)[5]) {
    const uint32_t c = draw >> 2, s = draw & 3u;
    uint4 w0 = make_uint4(0u, 0u, 0u, 0u), w1 = w0;
#pragma unroll 1
    for (uint32_t b = 0; b < 2; ++b) {
      const uint4 r = philox4x32_10(make_uint4(c + b, sample, pixel, 0u), k0, k1);
      if (b == 0)
        w0 = r;
      else
        w1 = r;
    }
    const uint32_t w[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
    for (int k = 0; k < 5; ++k)
      v[k] = s == 0 ? w[k] : (s == 1 ? w[k + 1] : (s == 2 ? w[k + 2] : w[k + 3]));
  }
};

// ---------------------------------------------------------------------------
// Material record (24 floats, include/rtx.h)
// ---------------------------------------------------------------------------
struct Mat {
  F3 base_color, emission;
  float roughness, metallic, subsurface, specular_tint, sheen, sheen_tint,
      clearcoat, clearcoat_roughness, spec_trans, ior, at_distance;
  F3 extinction;
};

RTX_DEV Mat load_mat(const float* __restrict__ m) {
  // the 24-float record is 16-byte aligned: six vector loads
  const float4* q = reinterpret_cast<const float4*>(m);
  float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3), e = __ldg(q + 4);
  float4 f = __ldg(q + 5);
  Mat r;
  r.base_color = f3(a.x, a.y, a.z);
  r.emission = f3(a.w, b.x, b.y);
  r.roughness = b.z;
  r.metallic = b.w;
  r.subsurface = c.y;
  r.specular_tint = c.z;
  r.sheen = c.w;
  r.sheen_tint = d.x;
  r.clearcoat = d.y;
  r.clearcoat_roughness = d.z;
  r.spec_trans = d.w;
  r.ior = e.x;
  r.at_distance = e.y;
  r.extinction = f3(e.z, e.w, f.x);
  return r;
}

// ---------------------------------------------------------------------------
// Procedural textures (RenderToy src/procedural.cpp:8-46).  The samplers take
// the reference's 2D coordinate p; a surface point maps to p by its two world
// coordinates across the dominant axis of the shading normal, times the
// material's texture scale, and the sample scales base_color by
// 0.25 + 0.75 s (the binding to materials is an extension: RenderToy only
// rasterises textures to images).
// ---------------------------------------------------------------------------

// CheckerBoard::Sample (procedural.cpp:8-16): int() truncates toward zero
RTX_DEV float tex_checker(float x, float y, int scale) {
  return (((int)(x * (float)scale) & 1) ^ ((int)(y * (float)scale) & 1)) == 1 ? 1.0f : 0.0f;
}

// Wave::Sample (procedural.cpp:22-25)
RTX_DEV float tex_wave(float x, float period) {
  return (sinf(2.0f * kPi * period * x) + 1.0f) / 2.0f;
}

// Improved gradient noise (K. Perlin, "Improving Noise", SIGGRAPH 2002) as
// siv::PerlinNoise v3.0.0 evaluates it in FP32: lattice indices masked to
// 8 bits, hashes through a 256-entry permutation, quintic fade, gradient
// selection by the low 4 bits of the hash.
RTX_DEV float perlin_fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
RTX_DEV float perlin_lerp(float a, float b, float t) { return a + (b - a) * t; }
RTX_DEV float perlin_grad(uint32_t hash, float x, float y, float z) {
  uint32_t h = hash & 15u;
  float u = h < 8u ? x : y;
  float v = h < 4u ? y : (h == 12u || h == 14u ? x : z);
  return ((h & 1u) == 0u ? u : -u) + ((h & 2u) == 0u ? v : -v);
}
RTX_DEV float perlin_noise3(const uint8_t* __restrict__ perm, float x, float y, float z) {
  float fx0 = floorf(x), fy0 = floorf(y), fz0 = floorf(z);
  int ix = (int)fx0 & 255, iy = (int)fy0 & 255, iz = (int)fz0 & 255;
  float fx = x - fx0, fy = y - fy0, fz = z - fz0;
  float u = perlin_fade(fx), v = perlin_fade(fy), w = perlin_fade(fz);
  uint32_t A = (__ldg(perm + (ix & 255)) + iy) & 255, B = (__ldg(perm + ((ix + 1) & 255)) + iy) & 255;
  uint32_t AA = (__ldg(perm + A) + iz) & 255, AB = (__ldg(perm + ((A + 1) & 255)) + iz) & 255;
  uint32_t BA = (__ldg(perm + B) + iz) & 255, BB = (__ldg(perm + ((B + 1) & 255)) + iz) & 255;
  float p0 = perlin_grad(__ldg(perm + AA), fx, fy, fz);
  float p1 = perlin_grad(__ldg(perm + BA), fx - 1.0f, fy, fz);
  float p2 = perlin_grad(__ldg(perm + AB), fx, fy - 1.0f, fz);
  float p3 = perlin_grad(__ldg(perm + BB), fx - 1.0f, fy - 1.0f, fz);
  float p4 = perlin_grad(__ldg(perm + ((AA + 1) & 255)), fx, fy, fz - 1.0f);
  float p5 = perlin_grad(__ldg(perm + ((BA + 1) & 255)), fx - 1.0f, fy, fz - 1.0f);
  float p6 = perlin_grad(__ldg(perm + ((AB + 1) & 255)), fx, fy - 1.0f, fz - 1.0f);
  float p7 = perlin_grad(__ldg(perm + ((BB + 1) & 255)), fx - 1.0f, fy - 1.0f, fz - 1.0f);
  float q0 = perlin_lerp(p0, p1, u), q1 = perlin_lerp(p2, p3, u);
  float q2 = perlin_lerp(p4, p5, u), q3 = perlin_lerp(p6, p7, u);
  float r0 = perlin_lerp(q0, q1, v), r1 = perlin_lerp(q2, q3, v);
  return perlin_lerp(r0, r1, w);
}

// PerlinNoise::Sample (procedural.cpp:43-46): octave3D_01(p.x * scale,
// p.y * scale, time = 0, octaves = 4, persistence 0.5), clamped to [0, 1]
RTX_DEV float tex_perlin(const uint8_t* __restrict__ perm, float px, float py, float scale) {
  float x = px * scale, y = py * scale, z = 0.0f;
  float result = 0.0f, amplitude = 1.0f;
  for (int i = 0; i < 4; ++i) {
    result += perlin_noise3(perm, x, y, z) * amplitude;
    x *= 2.0f;
    y *= 2.0f;
    z *= 2.0f;
    amplitude *= 0.5f;
  }
  if (result <= -1.0f) return 0.0f;
  if (1.0f <= result) return 1.0f;
  return result * 0.5f + 0.5f;
}

RTX_DEV float texture_sample(int kind, float param, const uint8_t* __restrict__ perm, float px, float py) {
  if (kind == 1) return tex_checker(px, py, (int)param);
  if (kind == 2) return tex_wave(px, param);
  if (kind == 3) return tex_perlin(perm, px, py, param);
  return 1.0f;
}

// base_color of the material record m (floats 21..23: kind, parameter,
// texture scale; kind != 0) at surface point pos with normal n
static __device__ __noinline__ F3 textured_base(const float* __restrict__ m, F3 pos, F3 n,
                                                const uint8_t* __restrict__ perm) {
  float4 a = __ldg(reinterpret_cast<const float4*>(m)), f = __ldg(reinterpret_cast<const float4*>(m) + 5);
  float ax = fabsf(n.x), ay = fabsf(n.y), az = fabsf(n.z);
  float px, py;
  if (ax >= ay && ax >= az) {
    px = pos.y;
    py = pos.z;
  } else if (ay >= az) {
    px = pos.x;
    py = pos.z;
  } else {
    px = pos.x;
    py = pos.y;
  }
  float s = texture_sample((int)f.y, f.z, perm, px * f.w, py * f.w);
  return f3(a.x, a.y, a.z) * (0.25f + 0.75f * s);
}

// ---------------------------------------------------------------------------
// PBR helpers (src/rtmath.cpp:169-353)
// ---------------------------------------------------------------------------
// std::clamp(x, 0, 1): NaN passes through as in the reference
RTX_DEV float clamp01(float x) { return x < 0.0f ? 0.0f : (1.0f < x ? 1.0f : x); }
RTX_DEV float GTR1(float NdotH, float a) {
  if (a >= 1.0f) return 1.0f / kPi;
  float a2 = a * a;
  float t = 1.0f + (a2 - 1.0f) * NdotH * NdotH;
  return (a2 - 1.0f) / (kPi * logf(a2) * t);
}
// The three sampling routines below take sin and cos of their azimuth phi
// from the caller (the *_sc forms), so that a BSDF sample evaluates them
// once whichever lobe it picked; the plain forms compute them as the
// reference does.
RTX_DEV F3 SampleGTR1_sc(float rgh, float r1, float sin_phi, float cos_phi) {
  float a = fmaxf(0.001f, rgh);
  float a2 = a * a;
  float cos_theta = sqrtf((1.0f - powf(a2, 1.0f - r1)) / (1.0f - a2));
  float sin_theta = clamp01(sqrtf(1.0f - (cos_theta * cos_theta)));
  return f3(sin_theta * cos_phi, sin_theta * sin_phi, cos_theta);
}
RTX_DEV float GTR1_phi(float r1) { return r1 * 2.0f * kPi; }
RTX_DEV F3 SampleGTR1(float rgh, float r1) {
  float phi = GTR1_phi(r1);
  return SampleGTR1_sc(rgh, r1, sinf(phi), cosf(phi));
}
RTX_DEV float GTR2(float NdotH, float a) {
  float a2 = a * a;
  float t = 1.0f + (a2 - 1.0f) * NdotH * NdotH;
  return a2 / (kPi * t * t);
}
// azimuth of the cosine-weighted and GGX visible-normal samples
RTX_DEV float azimuth(float r2) { return 2.0f * kPi * r2; }
RTX_LOBE F3 SampleGGXVNDF_sc(F3 V, float rgh, float r1, float sin_phi, float cos_phi) {
  F3 Vh = normalized(f3(rgh * V.x, rgh * V.y, V.z));
  float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
  F3 T1 = lensq > 0.0f ? f3(-Vh.y, Vh.x, 0.0f) * (1.0f / sqrtf(lensq)) : f3(1.0f, 0.0f, 0.0f);
  F3 T2 = cross(Vh, T1);
  float r = sqrtf(r1);
  float t1 = r * cos_phi;
  float t2 = r * sin_phi;
  float s = 0.5f * (1.0f + Vh.z);
  t2 = (1.0f - s) * sqrtf(1.0f - t1 * t1) + s * t2;
  F3 Nh = (T1 * t1 + T2 * t2) + Vh * sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2));
  return normalized(f3(rgh * Nh.x, rgh * Nh.y, fmaxf(0.0f, Nh.z)));
}
RTX_LOBE F3 SampleGGXVNDF(F3 V, float rgh, float r1, float r2) {
  float phi = azimuth(r2);
  return SampleGGXVNDF_sc(V, rgh, r1, sinf(phi), cosf(phi));
}
RTX_DEV float SmithG(float NdotV, float alpha_g) {
  float a = alpha_g * alpha_g;
  float b = NdotV * NdotV;
  return (2.0f * NdotV) / (NdotV + sqrtf(a + b - a * b));
}
RTX_DEV float SchlickFresnel(float u) {
  float m = clamp01(1.0f - u);
  float m2 = m * m;
  return m2 * m2 * m;
}
// std::max(a, b) returns a unless a < b
RTX_DEV float smax(float a, float b) { return (a < b) ? b : a; }
RTX_DEV float DielectricFresnel(float cos_theta_i, float eta) {
  float sin_theta_t_sq = eta * eta * (1.0f - cos_theta_i * cos_theta_i);
  if (sin_theta_t_sq > 1.0f) return 1.0f;
  float cos_theta_t = sqrtf(smax(1.0f - sin_theta_t_sq, 0.0f));
  float rs = (eta * cos_theta_t - cos_theta_i) / (eta * cos_theta_t + cos_theta_i);
  float rp = (eta * cos_theta_i - cos_theta_t) / (eta * cos_theta_i + cos_theta_t);
  return 0.5f * (rs * rs + rp * rp);
}
RTX_DEV F3 CosineSampleHemisphere_sc(float r1, float sin_phi, float cos_phi) {
  F3 d;
  float r = sqrtf(r1);
  d.x = r * cos_phi;
  d.y = r * sin_phi;
  d.z = sqrtf(smax(0.0f, 1.0f - d.x * d.x - d.y * d.y));
  return d;
}
RTX_DEV F3 CosineSampleHemisphere(float r1, float r2) {
  float phi = azimuth(r2);
  return CosineSampleHemisphere_sc(r1, sinf(phi), cosf(phi));
}
RTX_DEV float PowerHeuristic(float a, float b) {
  float t = a * a;
  return t / (b * b + t);
}
RTX_DEV void Onb(F3 N, F3& T, F3& B) {
  F3 up = fabsf(N.z) < 0.999f ? f3(0.0f, 0.0f, 1.0f) : f3(1.0f, 0.0f, 0.0f);
  T = normalized(cross(up, N));
  B = cross(N, T);
}
RTX_DEV F3 ToWorld(F3 X, F3 Y, F3 Z, F3 V) { return (X * V.x + Y * V.y) + Z * V.z; }
RTX_DEV F3 ToLocal(F3 X, F3 Y, F3 Z, F3 V) { return f3(dot(V, X), dot(V, Y), dot(V, Z)); }
RTX_DEV F3 Reflect(F3 I, F3 N) { return I - N * (2.0f * dot(I, N)); }
RTX_DEV F3 Refract(F3 I, F3 N, float eta) {
  float NdotI = dot(N, I);
  float k = 1.f - eta * eta * (1.f - NdotI * NdotI);
  if (k < 0.f) return f3(0.f, 0.f, 0.f);
  return I * eta - N * (eta * NdotI + sqrtf(k));
}

// ---------------------------------------------------------------------------
// PrincipledBSDF (src/material.cpp:35-295)
// ---------------------------------------------------------------------------
RTX_DEV float FresnelMix(const Mat& m, float eta, float VdotH) {
  float mf = SchlickFresnel(VdotH);
  float df = DielectricFresnel(VdotH, eta);
  return lerp(df, mf, m.metallic);
}
RTX_LOBE F3 EvalDiffuse(const Mat& m, F3 Csheen, F3 V, F3 L, F3 H, float& pdf) {
  pdf = 0.0f;
  if (L.z <= 0.0f) return f3s(0.0f);
  float FL = SchlickFresnel(L.z);
  float FV = SchlickFresnel(V.z);
  float FH = SchlickFresnel(dot(L, H));
  float Fd90 = 0.5f + 2.0f * dot(L, H) * dot(L, H) * m.roughness;
  float Fd = lerp(1.0f, Fd90, FL) * lerp(1.0f, Fd90, FV);
  float Fss90 = dot(L, H) * dot(L, H) * m.roughness;
  float Fss = lerp(1.0f, Fss90, FL) * lerp(1.0f, Fss90, FV);
  float ss = 1.25f * (Fss * (1.0f / (L.z + V.z) - 0.5f) + 0.5f);
  F3 Fsheen = Csheen * (FH * m.sheen);
  pdf = L.z * (1.0f / kPi);
  F3 r = m.base_color * ((1.0f / kPi) * lerp(Fd, ss, m.subsurface));
  r = r + Fsheen;
  r = r * (1.0f - m.metallic);
  r = r * (1.0f - m.spec_trans);
  return r;
}
RTX_LOBE F3 EvalSpecReflection(const Mat& m, float eta, F3 specCol, F3 V, F3 L, F3 H,
                              float& pdf) {
  pdf = 0.0f;
  if (L.z <= 0.0f) return f3s(0.0f);
  float FM = FresnelMix(m, eta, dot(L, H));
  F3 F = lerpv(specCol, f3s(1.0f), f3s(FM));
  float D = GTR2(H.z, m.roughness);
  float G1 = SmithG(fabsf(V.z), m.roughness);
  float G2 = G1 * SmithG(fabsf(L.z), m.roughness);
  float jacobian = 1.0f / (4.0f * dot(V, H));
  pdf = G1 * smax(0.0f, dot(V, H)) * D * jacobian / V.z;
  F3 r = F * D;
  r = r * G2;
  return r / (4.0f * L.z * V.z);
}
RTX_LOBE F3 EvalSpecRefraction(const Mat& m, float eta, F3 V, F3 L, F3 H, float& pdf) {
  pdf = 0.0f;
  if (L.z >= 0.0f) return f3s(0.0f);
  float F = DielectricFresnel(fabsf(dot(V, H)), eta);
  float D = GTR2(H.z, m.roughness);
  float denom = dot(L, H) + dot(V, H) * eta;
  denom *= denom;
  float G1 = SmithG(fabsf(V.z), m.roughness);
  float G2 = G1 * SmithG(fabsf(L.z), m.roughness);
  float jacobian = fabsf(dot(L, H)) / denom;
  pdf = G1 * smax(0.0f, dot(V, H)) * D * jacobian / V.z;
  F3 spec_color = f3(powf(m.base_color.x, 0.5f), powf(m.base_color.y, 0.5f),
                     powf(m.base_color.z, 0.5f));
  F3 r = spec_color * (1.0f - m.metallic);
  r = r * m.spec_trans;
  r = r * (1.0f - F);
  r = r * D;
  r = r * G2;
  r = r * fabsf(dot(V, H));
  r = r * fabsf(dot(L, H));
  r = r * eta;
  r = r * eta;
  return r / (denom * fabsf(L.z) * fabsf(V.z));
}
RTX_LOBE F3 EvalClearcoat(const Mat& m, F3 V, F3 L, F3 H, float& pdf) {
  pdf = 0.0f;
  if (L.z <= 0.0f) return f3s(0.0f);
  float FH = DielectricFresnel(dot(V, H), 1.0f / 1.5f);
  float F = lerp(0.04f, 1.0f, FH);
  float D = GTR1(H.z, m.clearcoat_roughness);
  float G = SmithG(L.z, 0.25f) * SmithG(V.z, 0.25f);
  float jacobian = 1.0f / (4.0f * dot(V, H));
  pdf = D * H.z * jacobian;
  F3 r = f3s(0.25f) * m.clearcoat;
  r = r * F;
  r = r * D;
  r = r * G;
  return r / (4.0f * L.z * V.z);
}
RTX_DEV void GetSpecColor(const Mat& m, float eta, F3& spec_col, F3& sheen_col) {
  float lum = luma(m.base_color);
  F3 ctint = lum > 0.0f ? m.base_color / lum : f3s(1.0f);
  float F0 = (1.0f - eta) / (1.0f + eta);
  spec_col = lerpv(lerpv(f3s(1.0f), ctint, f3s(m.specular_tint)) * (F0 * F0), m.base_color,
                   f3s(m.metallic));
  sheen_col = lerpv(f3s(1.0f), ctint, f3s(m.sheen_tint));
}
RTX_DEV void GetLobeProbabilities(const Mat& m, F3 spec_col, float af, float& dw, float& srw,
                                  float& strw, float& cw) {
  dw = luma(m.base_color) * (1.0f - m.metallic) * (1.0f - m.spec_trans);
  srw = luma(lerpv(spec_col, f3s(1.0f), f3s(af)));
  strw = (1.0f - af) * (1.0f - m.metallic) * m.spec_trans * luma(m.base_color);
  cw = m.clearcoat * (1.0f - m.metallic);
  float total = dw + srw + strw + cw;
  dw /= total;
  srw /= total;
  strw /= total;
  cw /= total;
}
// What Eval and Sample both derive from the shading normal, the outgoing
// direction and the material: the same operations, done once per vertex.
struct ShadingFrame {
  F3 T, B, N, V;  // tangent frame and the outgoing direction in it
  F3 spec_col, sheen_col;
};

RTX_DEV ShadingFrame make_frame(const Mat& m, float eta, F3 N, F3 V) {
  ShadingFrame fr;
  Onb(N, fr.T, fr.B);
  fr.N = N;
  fr.V = ToLocal(fr.T, fr.B, N, V);
  GetSpecColor(m, eta, fr.spec_col, fr.sheen_col);
  return fr;
}

// Lobe sets.  A material with spec_trans == 0 (either sign) has a refraction
// weight strw of +-0 or NaN, and one with clearcoat == 0 a clearcoat weight
// cw of +-0 or NaN: Eval never adds those lobes (each needs its weight > 0),
// Sample never takes the refraction branch (cdf2 = cdf1 + strw compares as
// cdf1), and Sample's clearcoat branch multiplies its pdf by cw, so it returns
// pdf +-0 or NaN.  The shading kernel uses neither Eval's value nor Sample's
// direction unless the pdf is > 0, so when no material of the scene has the
// lobe, leaving it out (kTrans / kCoat false) changes no result; it shrinks
// the inlined shading code.
#ifndef RTX_LOBE_BITS
#define RTX_LOBE_BITS
constexpr int kLobeTrans = 1, kLobeCoat = 2, kLobeAll = 3;
#endif

template <int kLobes = kLobeAll>
RTX_DEV F3 BsdfEvalFrame(const Mat& m, float eta, const ShadingFrame& fr, F3 L, float& bsdf_pdf) {
  constexpr bool kTrans = (kLobes & kLobeTrans) != 0, kCoat = (kLobes & kLobeCoat) != 0;
  bsdf_pdf = 0.0f;
  F3 f = f3s(0.0f);
  F3 V = fr.V;
  L = ToLocal(fr.T, fr.B, fr.N, L);
  // without refraction every lobe needs L.z > 0: pdf 0 below the horizon
  if (!kTrans && !(L.z > 0.0f)) return f;
  F3 H;
  if (L.z > 0.0f)
    H = normalized(L + V);
  else
    H = normalized(L + V * eta);
  if (H.z < 0.0f) H = -H;
  F3 spec_color = fr.spec_col, sheen_color = fr.sheen_col;
  float dw, srw, strw, cw;
  float fresnel = FresnelMix(m, eta, dot(V, H));
  GetLobeProbabilities(m, spec_color, fresnel, dw, srw, strw, cw);
  float pdf;
  if (dw > 0.0f && L.z > 0.0f) {
    f = f + EvalDiffuse(m, sheen_color, V, L, H, pdf);
    bsdf_pdf = bsdf_pdf + pdf * dw;
  }
  if (srw > 0.0f && L.z > 0.0f && V.z > 0.0f) {
    f = f + EvalSpecReflection(m, eta, spec_color, V, L, H, pdf);
    bsdf_pdf = bsdf_pdf + pdf * srw;
  }
  if (kTrans && strw > 0.0f && L.z < 0.0f) {
    f = f + EvalSpecRefraction(m, eta, V, L, H, pdf);
    bsdf_pdf = bsdf_pdf + pdf * strw;
  }
  if (kCoat && cw > 0.0f && L.z > 0.0f && V.z > 0.0f) {
    f = f + EvalClearcoat(m, V, L, H, pdf);
    bsdf_pdf = bsdf_pdf + pdf * cw;
  }
  return f * fabsf(L.z);
}
template <int kLobes = kLobeAll>
RTX_DEV bool BsdfSampleFrame(const Mat& m, float eta, const ShadingFrame& fr, float r1, float r2,
                             F3& out_dir, F3& color_o, float& pdf) {
  constexpr bool kTrans = (kLobes & kLobeTrans) != 0, kCoat = (kLobes & kLobeCoat) != 0;
  pdf = 0.0f;
  F3 f = f3s(0.0f);
  F3 V = fr.V;
  F3 T = fr.T, B = fr.B, N = fr.N;
  F3 specCol = fr.spec_col, sheenCol = fr.sheen_col;
  float dw, srw, strw, cw;
  float approxFresnel = FresnelMix(m, eta, V.z);
  GetLobeProbabilities(m, specCol, approxFresnel, dw, srw, strw, cw);
  float cdf0 = dw;
  float cdf1 = cdf0 + srw;
  float cdf2 = cdf1 + strw;
  // pick the lobe and rescale r1 as the reference's branches do, then one
  // sin / cos of the lobe's azimuth for every branch (one inlined copy of
  // them instead of one per lobe: 5 % less shading time, measured)
  int lobe;
  float phi;
  if (r1 < cdf0) {
    lobe = 0;
    r1 /= cdf0;
    phi = azimuth(r2);
  } else if (r1 < cdf1) {
    lobe = 1;
    r1 = (r1 - cdf0) / (cdf1 - cdf0);
    phi = azimuth(r2);
  } else if (kTrans && r1 < cdf2) {
    lobe = 2;
    r1 = (r1 - cdf1) / (cdf2 - cdf1);
    phi = azimuth(r2);
  } else if (!kCoat) {
    return false;  // the clearcoat branch's pdf would be +-0 or NaN
  } else {
    lobe = 3;
    // material.cpp:279 divides in double and narrows to float
    float num = r1 - cdf2;
    r1 = (float)(__ddiv_rn((double)num, __dsub_rn(1.0, (double)cdf2)));
    phi = GTR1_phi(r1);
  }
  const float sp = sinf(phi), cp = cosf(phi);
  if (lobe == 0) {
    out_dir = CosineSampleHemisphere_sc(r1, sp, cp);
    F3 H = normalized(out_dir + V);
    f = EvalDiffuse(m, sheenCol, V, out_dir, H, pdf);
    pdf *= dw;
  } else if (lobe == 1) {
    F3 H = SampleGGXVNDF_sc(V, m.roughness, r1, sp, cp);
    if (H.z < 0.0f) H = -H;
    out_dir = normalized(Reflect(-V, H));
    f = EvalSpecReflection(m, eta, specCol, V, out_dir, H, pdf);
    pdf *= srw;
  } else if (kTrans && lobe == 2) {
    F3 H = SampleGGXVNDF_sc(V, m.roughness, r1, sp, cp);
    if (H.z < 0.0f) H = -H;
    out_dir = normalized(Refract(-V, H, eta));
    f = EvalSpecRefraction(m, eta, V, out_dir, H, pdf);
    pdf *= strw;
  } else if (kCoat) {
    F3 H = SampleGTR1_sc(m.clearcoat_roughness, r1, sp, cp);
    if (H.z < 0.0f) H = -H;
    out_dir = normalized(Reflect(-V, H));
    f = EvalClearcoat(m, V, out_dir, H, pdf);
    pdf *= cw;
  }
  out_dir = ToWorld(T, B, N, out_dir);
  color_o = f * fabsf(dot(N, out_dir));
  return !eq_zero_eps(out_dir);
}

// PrincipledBSDF::Eval / Sample with their own frame (material.cpp:143, 206)
RTX_DEV F3 BsdfEval(const Mat& m, float eta, F3 V, F3 N, F3 L, float& bsdf_pdf) {
  return BsdfEvalFrame(m, eta, make_frame(m, eta, N, V), L, bsdf_pdf);
}
RTX_DEV bool BsdfSample(const Mat& m, float eta, F3 N, F3 in_dir, float r1, float r2,
                        F3& out_dir, F3& color_o, float& pdf) {
  return BsdfSampleFrame(m, eta, make_frame(m, eta, N, in_dir), r1, r2, out_dir, color_o, pdf);
}

}  // namespace rtx
