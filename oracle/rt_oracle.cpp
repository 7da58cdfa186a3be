/*
 * rt_oracle.cpp — CPU restatement of RenderToy's path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker): used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The product
 * library never links or calls this file.
 *
 * Every function restates one reference function and keeps its floating-point
 * operation order (the build uses -ffp-contract=off, no fast-math), so that it
 * reproduces the reference bit for bit on the same machine.  The reference
 * file:line each function follows is given beside it; paths are relative to
 * the RenderToy source tree.
 *
 * Deliberate, documented deviations (both also apply to the harness that
 * links the reference, so the golden vectors pin them):
 *   - Random::Int / Random::Float (src/rtmath.cpp:355-373, a shared global
 *     mt19937) are replaced by the counter-based Philox stream of
 *     (seed, pixel, sample, draw index);
 *   - the recursion cap `depth > 4` (src/renderer.cpp:274) is a parameter
 *     (max_depth = number of shaded vertices; the reference value is 5);
 *   - compositor taps whose reflected linear index falls outside the image
 *     (an out-of-bounds read in the reference, include/RenderToy/
 *     compositor.h:25-39) read zero;
 *   - the shadow-ray (u, v) used for a smooth emitter's normal when the shadow
 *     ray hits nothing is (0, 0) (uninitialised in src/renderer.cpp:351-358).
 */
#include "rt_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <queue>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ----------------------------------------------------------------------------
// Vector arithmetic with the reference's evaluation order
// (include/RenderToy/rtmath.h:74-534).
// ----------------------------------------------------------------------------
struct V3 {
  float x, y, z;
};

inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 v3s(float s) { return V3{s, s, s}; }
inline V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 neg(V3 a) { return V3{-a.x, -a.y, -a.z}; }
inline V3 mul(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 scl(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
inline V3 dvs(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
inline V3 dvv(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
// rtmath.h:328-338 — accumulate from zero, x then y then z
inline float dot(V3 a, V3 b) {
  float r = 0.0f;
  r += a.x * b.x;
  r += a.y * b.y;
  r += a.z * b.z;
  return r;
}
// rtmath.h:124-141
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
// rtmath.h:144-150 — divide each component by the length
inline V3 normalized(V3 a) {
  float l = length(a);
  return V3{a.x / l, a.y / l, a.z / l};
}
// rtmath.h:388-395
inline V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// rtmath.h:296-308 — epsilon equality; NaN components compare "equal"
inline bool eq_eps(V3 a, V3 b) {
  if (std::fabs(a.x - b.x) > 1e-7f) return false;
  if (std::fabs(a.y - b.y) > 1e-7f) return false;
  if (std::fabs(a.z - b.z) > 1e-7f) return false;
  return true;
}
inline float get(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
inline float& ref(V3& a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
// rtmath.h:1245-1249: x * (1 - a) + y * a
inline float lerp(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline V3 lerpv(V3 x, V3 y, V3 a) {
  return add(mul(x, sub(v3s(1.0f), a)), mul(y, a));
}
// rtmath.h:1140-1147 (BT.709)
inline float luma(V3 v) {
  return 0.2126f * v.x + 0.7152f * v.y + 0.0722f * v.z;
}

const float kPi = 3.14159265358979323846f;
const float kInf = 1e7f;            // kFloatInfinity, rtmath.h:23
const float kE = 2.718281828459045235360287471352662498f;  // M_Ef32

// ----------------------------------------------------------------------------
// Counter-based RNG (Philox4x32-10, Salmon et al., SC'11).  Replaces the
// reference's global mt19937 (src/rtmath.cpp:355-373) on both sides.
// ----------------------------------------------------------------------------
inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k0;
    uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

struct Rng {
  uint64_t seed;
  uint32_t pixel, sample, draw;
  uint32_t next_u32() {
    uint32_t c[4] = {draw >> 2, sample, pixel, 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    uint32_t w = c[draw & 3u];
    ++draw;
    return w;
  }
  // Random::Float — uniform in [0, 1) with 24 bits
  float uniform() { return (float)(next_u32() >> 8) * (1.0f / 16777216.0f); }
  // Random::Int(a, b) — inclusive range
  int uniform_int(int a, int b) {
    uint32_t n = (uint32_t)(b - a + 1);
    return a + (int)(((uint64_t)next_u32() * (uint64_t)n) >> 32);
  }
};

// ----------------------------------------------------------------------------
// Material (include/RenderToy/material.h:14-30), 24-float layout of rtx.h.
// ----------------------------------------------------------------------------
struct Mat {
  V3 base_color, emission;
  float roughness, metallic, anisotropic, subsurface, specular_tint, sheen,
      sheen_tint, clearcoat, clearcoat_roughness, spec_trans, ior, at_distance;
  V3 extinction;
};

Mat load_mat(const float* m) {
  Mat r;
  r.base_color = v3(m[0], m[1], m[2]);
  r.emission = v3(m[3], m[4], m[5]);
  r.roughness = m[6];
  r.metallic = m[7];
  r.anisotropic = m[8];
  r.subsurface = m[9];
  r.specular_tint = m[10];
  r.sheen = m[11];
  r.sheen_tint = m[12];
  r.clearcoat = m[13];
  r.clearcoat_roughness = m[14];
  r.spec_trans = m[15];
  r.ior = m[16];
  r.at_distance = m[17];
  r.extinction = v3(m[18], m[19], m[20]);
  return r;
}

// ----------------------------------------------------------------------------
// PBR helpers (src/rtmath.cpp:169-353)
// ----------------------------------------------------------------------------
float GTR1(float NdotH, float a) {  // rtmath.cpp:169-176
  if (a >= 1.0f) return 1.0f / kPi;
  float a2 = a * a;
  float t = 1.0f + (a2 - 1.0f) * NdotH * NdotH;
  return (a2 - 1.0f) / (kPi * std::log(a2) * t);
}
V3 SampleGTR1(float rgh, float r1, float r2) {  // rtmath.cpp:178-191
  (void)r2;
  float a = std::max(0.001f, rgh);
  float a2 = a * a;
  float phi = r1 * 2.0f * kPi;
  float cos_theta = std::sqrt((1.0f - std::pow(a2, 1.0f - r1)) / (1.0f - a2));
  float sin_theta =
      std::clamp(std::sqrt(1.0f - (cos_theta * cos_theta)), 0.0f, 1.0f);
  float sin_phi = std::sin(phi);
  float cos_phi = std::cos(phi);
  return v3(sin_theta * cos_phi, sin_theta * sin_phi, cos_theta);
}
float GTR2(float NdotH, float a) {  // rtmath.cpp:193-198
  float a2 = a * a;
  float t = 1.0f + (a2 - 1.0f) * NdotH * NdotH;
  return a2 / (kPi * t * t);
}
V3 SampleGGXVNDF(V3 V, float rgh, float r1, float r2) {  // rtmath.cpp:214-232
  V3 Vh = normalized(v3(rgh * V.x, rgh * V.y, V.z));
  float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
  V3 T1 = lensq > 0.0f ? scl(v3(-Vh.y, Vh.x, 0.0f), 1.0f / std::sqrt(lensq))
                       : v3(1.0f, 0.0f, 0.0f);
  V3 T2 = cross(Vh, T1);
  float r = std::sqrt(r1);
  float phi = 2.0f * kPi * r2;
  float t1 = r * std::cos(phi);
  float t2 = r * std::sin(phi);
  float s = 0.5f * (1.0f + Vh.z);
  t2 = (1.0f - s) * std::sqrt(1.0f - t1 * t1) + s * t2;
  V3 Nh = add(add(scl(T1, t1), scl(T2, t2)),
              scl(Vh, std::sqrt(std::max(0.0f, 1.0f - t1 * t1 - t2 * t2))));
  return normalized(v3(rgh * Nh.x, rgh * Nh.y, std::max(0.0f, Nh.z)));
}
float SmithG(float NdotV, float alpha_g) {  // rtmath.cpp:253-258
  float a = alpha_g * alpha_g;
  float b = NdotV * NdotV;
  return (2.0f * NdotV) / (NdotV + std::sqrt(a + b - a * b));
}
float SchlickFresnel(float u) {  // rtmath.cpp:268-273
  float m = std::clamp(1.0f - u, 0.0f, 1.0f);
  float m2 = m * m;
  return m2 * m2 * m;
}
float DielectricFresnel(float cos_theta_i, float eta) {  // rtmath.cpp:275-289
  float sin_theta_t_sq = eta * eta * (1.0f - cos_theta_i * cos_theta_i);
  if (sin_theta_t_sq > 1.0f) return 1.0f;
  float cos_theta_t = std::sqrt(std::max(1.0f - sin_theta_t_sq, 0.0f));
  float rs = (eta * cos_theta_t - cos_theta_i) / (eta * cos_theta_t + cos_theta_i);
  float rp = (eta * cos_theta_i - cos_theta_t) / (eta * cos_theta_i + cos_theta_t);
  return 0.5f * (rs * rs + rp * rp);
}
V3 CosineSampleHemisphere(float r1, float r2) {  // rtmath.cpp:291-300
  V3 d;
  float r = std::sqrt(r1);
  float phi = 2.0f * kPi * r2;
  d.x = r * std::cos(phi);
  d.y = r * std::sin(phi);
  d.z = std::sqrt(std::max(0.0f, 1.0f - d.x * d.x - d.y * d.y));
  return d;
}
float PowerHeuristic(float a, float b) {  // rtmath.cpp:317-321
  float t = a * a;
  return t / (b * b + t);
}
void Onb(V3 N, V3& T, V3& B) {  // rtmath.cpp:323-328
  V3 up = std::fabs(N.z) < 0.999f ? v3(0.0f, 0.0f, 1.0f) : v3(1.0f, 0.0f, 0.0f);
  T = normalized(cross(up, N));
  B = cross(N, T);
}
V3 ToWorld(V3 X, V3 Y, V3 Z, V3 V) {  // rtmath.cpp:330-333
  return add(add(scl(X, V.x), scl(Y, V.y)), scl(Z, V.z));
}
V3 ToLocal(V3 X, V3 Y, V3 Z, V3 V) {  // rtmath.cpp:335-338
  return v3(dot(V, X), dot(V, Y), dot(V, Z));
}
V3 Reflect(V3 I, V3 N) {  // rtmath.cpp:340-343
  return sub(I, scl(N, 2.0f * dot(I, N)));
}
V3 Refract(V3 I, V3 N, float eta) {  // rtmath.cpp:345-353
  float NdotI = dot(N, I);
  float k = 1.f - eta * eta * (1.f - NdotI * NdotI);
  if (k < 0.f) return v3(0.f, 0.f, 0.f);
  return sub(scl(I, eta), scl(N, eta * NdotI + std::sqrt(k)));
}

// ----------------------------------------------------------------------------
// PrincipledBSDF (src/material.cpp:35-295)
// ----------------------------------------------------------------------------
float FresnelMix(const Mat& m, float eta, float VdotH) {  // material.cpp:35-40
  float metallic_fresnel = SchlickFresnel(VdotH);
  float dielectric_fresnel = DielectricFresnel(VdotH, eta);
  return lerp(dielectric_fresnel, metallic_fresnel, m.metallic);
}
V3 EvalDiffuse(const Mat& m, V3 Csheen, V3 V, V3 L, V3 H, float& pdf) {  // 42-65
  pdf = 0.0f;
  if (L.z <= 0.0f) return v3s(0.0f);
  float FL = SchlickFresnel(L.z);
  float FV = SchlickFresnel(V.z);
  float FH = SchlickFresnel(dot(L, H));
  float Fd90 = 0.5f + 2.0f * dot(L, H) * dot(L, H) * m.roughness;
  float Fd = lerp(1.0f, Fd90, FL) * lerp(1.0f, Fd90, FV);
  float Fss90 = dot(L, H) * dot(L, H) * m.roughness;
  float Fss = lerp(1.0f, Fss90, FL) * lerp(1.0f, Fss90, FV);
  float ss = 1.25f * (Fss * (1.0f / (L.z + V.z) - 0.5f) + 0.5f);
  V3 Fsheen = scl(Csheen, FH * m.sheen);
  pdf = L.z * (1.0f / kPi);
  V3 r = scl(m.base_color, (1.0f / kPi) * lerp(Fd, ss, m.subsurface));
  r = add(r, Fsheen);
  r = scl(r, 1.0f - m.metallic);
  r = scl(r, 1.0f - m.spec_trans);
  return r;
}
V3 EvalSpecReflection(const Mat& m, float eta, V3 specCol, V3 V, V3 L, V3 H,
                      float& pdf) {  // material.cpp:67-82
  pdf = 0.0f;
  if (L.z <= 0.0f) return v3s(0.0f);
  float FM = FresnelMix(m, eta, dot(L, H));
  V3 F = lerpv(specCol, v3s(1.0f), v3s(FM));
  float D = GTR2(H.z, m.roughness);
  float G1 = SmithG(std::fabs(V.z), m.roughness);
  float G2 = G1 * SmithG(std::fabs(L.z), m.roughness);
  float jacobian = 1.0f / (4.0f * dot(V, H));
  pdf = G1 * std::max(0.0f, dot(V, H)) * D * jacobian / V.z;
  V3 r = scl(F, D);
  r = scl(r, G2);
  return dvs(r, 4.0f * L.z * V.z);
}
V3 EvalSpecRefraction(const Mat& m, float eta, V3 V, V3 L, V3 H,
                      float& pdf) {  // material.cpp:84-102
  pdf = 0.0f;
  if (L.z >= 0.0f) return v3s(0.0f);
  float F = DielectricFresnel(std::fabs(dot(V, H)), eta);
  float D = GTR2(H.z, m.roughness);
  float denom = dot(L, H) + dot(V, H) * eta;
  denom *= denom;
  float G1 = SmithG(std::fabs(V.z), m.roughness);
  float G2 = G1 * SmithG(std::fabs(L.z), m.roughness);
  float jacobian = std::fabs(dot(L, H)) / denom;
  pdf = G1 * std::max(0.0f, dot(V, H)) * D * jacobian / V.z;
  V3 spec_color = v3(std::pow(m.base_color.x, 0.5f), std::pow(m.base_color.y, 0.5f),
                     std::pow(m.base_color.z, 0.5f));
  // `(1.0 - x)` is evaluated in double and narrowed; for float x in [0, 1]
  // that equals the float subtraction.
  V3 r = scl(spec_color, (float)(1.0 - (double)m.metallic));
  r = scl(r, m.spec_trans);
  r = scl(r, (float)(1.0 - (double)F));
  r = scl(r, D);
  r = scl(r, G2);
  r = scl(r, std::fabs(dot(V, H)));
  r = scl(r, std::fabs(dot(L, H)));
  r = scl(r, eta);
  r = scl(r, eta);
  return dvs(r, denom * std::fabs(L.z) * std::fabs(V.z));
}
V3 EvalClearcoat(const Mat& m, V3 V, V3 L, V3 H, float& pdf) {  // 104-118
  pdf = 0.0f;
  if (L.z <= 0.0f) return v3s(0.0f);
  float FH = DielectricFresnel(dot(V, H), 1.0f / 1.5f);
  float F = lerp(0.04f, 1.0f, FH);
  float D = GTR1(H.z, m.clearcoat_roughness);
  float G = SmithG(L.z, 0.25f) * SmithG(V.z, 0.25f);
  float jacobian = 1.0f / (4.0f * dot(V, H));
  pdf = D * H.z * jacobian;
  V3 r = scl(v3s(0.25f), m.clearcoat);
  r = scl(r, F);
  r = scl(r, D);
  r = scl(r, G);
  return dvs(r, 4.0f * L.z * V.z);
}
void GetSpecColor(const Mat& m, float eta, V3& spec_col, V3& sheen_col) {  // 120-127
  float lum = luma(m.base_color);
  V3 ctint = lum > 0.0f ? dvs(m.base_color, lum) : v3s(1.0f);
  float F0 = (1.0f - eta) / (1.0f + eta);
  spec_col = lerpv(scl(lerpv(v3s(1.0f), ctint, v3s(m.specular_tint)), F0 * F0),
                   m.base_color, v3s(m.metallic));
  sheen_col = lerpv(v3s(1.0f), ctint, v3s(m.sheen_tint));
}
void GetLobeProbabilities(const Mat& m, V3 spec_col, float approx_fresnel,
                          float& dw, float& srw, float& strw,
                          float& cw) {  // material.cpp:129-141
  dw = luma(m.base_color) * (1.0f - m.metallic) * (1.0f - m.spec_trans);
  srw = luma(lerpv(spec_col, v3s(1.0f), v3s(approx_fresnel)));
  strw = (1.0f - approx_fresnel) * (1.0f - m.metallic) * m.spec_trans *
         luma(m.base_color);
  cw = m.clearcoat * (1.0f - m.metallic);
  float total = dw + srw + strw + cw;
  dw /= total;
  srw /= total;
  strw /= total;
  cw /= total;
}
V3 BsdfEval(const Mat& m, float eta, V3 V, V3 N, V3 L,
            float& bsdf_pdf) {  // material.cpp:143-204
  bsdf_pdf = 0.0f;
  V3 f = v3s(0.0f);
  V3 T, B;
  Onb(N, T, B);
  V = ToLocal(T, B, N, V);
  L = ToLocal(T, B, N, L);
  V3 H;
  if (L.z > 0.0f)
    H = normalized(add(L, V));
  else
    H = normalized(add(L, scl(V, eta)));
  if (H.z < 0.0f) H = neg(H);
  V3 spec_color, sheen_color;
  GetSpecColor(m, eta, spec_color, sheen_color);
  float dw, srw, strw, cw;
  float fresnel = FresnelMix(m, eta, dot(V, H));
  GetLobeProbabilities(m, spec_color, fresnel, dw, srw, strw, cw);
  float pdf;
  if (dw > 0.0f && L.z > 0.0f) {
    f = add(f, EvalDiffuse(m, sheen_color, V, L, H, pdf));
    bsdf_pdf += pdf * dw;
  }
  if (srw > 0.0f && L.z > 0.0f && V.z > 0.0f) {
    f = add(f, EvalSpecReflection(m, eta, spec_color, V, L, H, pdf));
    bsdf_pdf += pdf * srw;
  }
  if (strw > 0.0f && L.z < 0.0f) {
    f = add(f, EvalSpecRefraction(m, eta, V, L, H, pdf));
    bsdf_pdf += pdf * strw;
  }
  if (cw > 0.0f && L.z > 0.0f && V.z > 0.0f) {
    f = add(f, EvalClearcoat(m, V, L, H, pdf));
    bsdf_pdf += pdf * cw;
  }
  return scl(f, std::fabs(L.z));
}
bool BsdfSample(const Mat& m, float eta, V3 N, V3 in_dir, Rng& rng, V3& out_dir,
                V3& color_o, float& pdf) {  // material.cpp:206-295
  pdf = 0.0f;
  V3 f = v3s(0.0f);
  V3 V = in_dir;
  float r1 = rng.uniform();
  float r2 = rng.uniform();
  V3 T, B;
  Onb(N, T, B);
  V = ToLocal(T, B, N, V);
  V3 specCol, sheenCol;
  GetSpecColor(m, eta, specCol, sheenCol);
  float dw, srw, strw, cw;
  float approxFresnel = FresnelMix(m, eta, V.z);
  GetLobeProbabilities(m, specCol, approxFresnel, dw, srw, strw, cw);
  float cdf0 = dw;
  float cdf1 = cdf0 + srw;
  float cdf2 = cdf1 + strw;
  if (r1 < cdf0) {
    r1 /= cdf0;
    out_dir = CosineSampleHemisphere(r1, r2);
    V3 H = normalized(add(out_dir, V));
    f = EvalDiffuse(m, sheenCol, V, out_dir, H, pdf);
    pdf *= dw;
  } else if (r1 < cdf1) {
    r1 = (r1 - cdf0) / (cdf1 - cdf0);
    V3 H = SampleGGXVNDF(V, m.roughness, r1, r2);
    if (H.z < 0.0f) H = neg(H);
    out_dir = normalized(Reflect(neg(V), H));
    f = EvalSpecReflection(m, eta, specCol, V, out_dir, H, pdf);
    pdf *= srw;
  } else if (r1 < cdf2) {
    r1 = (r1 - cdf1) / (cdf2 - cdf1);
    V3 H = SampleGGXVNDF(V, m.roughness, r1, r2);
    if (H.z < 0.0f) H = neg(H);
    out_dir = normalized(Refract(neg(V), H, eta));
    f = EvalSpecRefraction(m, eta, V, out_dir, H, pdf);
    pdf *= strw;
  } else {
    // material.cpp:279 divides in double, then narrows to float
    r1 = (float)((double)(r1 - cdf2) / (1.0 - (double)cdf2));
    V3 H = SampleGTR1(m.clearcoat_roughness, r1, r2);
    if (H.z < 0.0f) H = neg(H);
    out_dir = normalized(Reflect(neg(V), H));
    f = EvalClearcoat(m, V, out_dir, H, pdf);
    pdf *= cw;
  }
  out_dir = ToWorld(T, B, N, out_dir);
  color_o = scl(f, std::fabs(dot(N, out_dir)));
  return !eq_eps(out_dir, v3s(0.0f));
}

// ----------------------------------------------------------------------------
// Geometry (src/object.cpp:83-243) and the octree (src/bvh.cpp).
// ----------------------------------------------------------------------------
struct Box {
  V3 lo{0.0f, 0.0f, 0.0f}, hi{0.0f, 0.0f, 0.0f};  // bvh.cpp:9-12: origin box
  void extend(const Box& b) {  // bvh.cpp:76-84
    lo = v3(std::min(lo.x, b.lo.x), std::min(lo.y, b.lo.y), std::min(lo.z, b.lo.z));
    hi = v3(std::max(hi.x, b.hi.x), std::max(hi.y, b.hi.y), std::max(hi.z, b.hi.z));
  }
  V3 centroid() const { return scl(add(lo, hi), 0.5f); }  // bvh.cpp:86-89
  // bvh.cpp:19-74 — slab test with divisions; writes the entry distance only
  bool intersect(V3 o, V3 d, float& t_min) const {
    float tmin = (lo.x - o.x) / d.x;
    float tmax = (hi.x - o.x) / d.x;
    if (tmin > tmax) std::swap(tmin, tmax);
    float tymin = (lo.y - o.y) / d.y;
    float tymax = (hi.y - o.y) / d.y;
    if (tymin > tymax) std::swap(tymin, tymax);
    if ((tmin > tymax) || (tymin > tmax)) return false;
    if (tymin > tmin) tmin = tymin;
    if (tymax < tmax) tmax = tymax;
    float tzmin = (lo.z - o.z) / d.z;
    float tzmax = (hi.z - o.z) / d.z;
    if (tzmin > tzmax) std::swap(tzmin, tzmax);
    if ((tmin > tzmax) || (tzmin > tmax)) return false;
    if (tzmin > tmin) tmin = tzmin;
    if (tzmax < tmax) tmax = tzmax;
    t_min = tmin;
    return true;
  }
};

struct Tri {
  V3 v0, v1, v2;
  V3 n0, n1, n2;
  V3 e1, e2;  // v0v1_w, v0v2_w
  float area;
  V3 normal;
  int mesh;
};

struct OctNode {
  int child[8];
  std::vector<int> items;
  Box box;
  bool leaf = true;
  OctNode() {
    for (int i = 0; i < 8; ++i) child[i] = -1;
  }
};

struct Scene {
  std::vector<Tri> tris;
  std::vector<Box> tri_box;
  std::vector<int> mesh_mat;
  std::vector<uint8_t> mesh_smooth;
  std::vector<Mat> mats;
  std::vector<V3> mat_tex;  // per material: texture kind, parameter, scale (floats 21..23)
  uint8_t perm[256];        // Perlin texture permutation
  std::vector<int> emitters;
  V3 sky, ground;
  std::vector<OctNode> nodes;
  Box tree_box;

  void insert(int node, int item, const Box& bbox, int depth);  // bvh.cpp:127-195
  void build(int node, const Box& bbox);                        // bvh.cpp:197-228
  int intersect(V3 o, V3 d, int exclude, float& t, float& u, float& v,
                V3* pos) const;                                 // bvh.cpp:266-341
  V3 normal_at(int tri, float u, float v) const;                // object.cpp:207-217
  Mat shade_mat(int tri, V3 pos, V3 n) const;                   // textured material at a hit
};

// ----------------------------------------------------------------------------
// Procedural textures, src/procedural.cpp:8-46 (bound to materials by floats
// 21..23 of the record: an extension, see include/rtx.h).  The Perlin sampler
// is improved gradient noise (K. Perlin, SIGGRAPH 2002) as siv::PerlinNoise
// v3.0.0 (include/PerlinNoise/PerlinNoise.hpp:281-300, 365-400, 489-534,
// 611-614) evaluates it in float.
// ----------------------------------------------------------------------------
float tex_checker(float x, float y, int scale) {
  return (((int)(x * (float)scale) & 1) ^ ((int)(y * (float)scale) & 1)) == 1 ? 1.0f : 0.0f;
}
float tex_wave(float x, float period) { return (std::sin(2.0f * kPi * period * x) + 1.0f) / 2.0f; }
float pfade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
float plerp(float a, float b, float t) { return a + (b - a) * t; }
float pgrad(uint32_t hash, float x, float y, float z) {
  uint32_t h = hash & 15u;
  float u = h < 8u ? x : y;
  float v = h < 4u ? y : (h == 12u || h == 14u ? x : z);
  return ((h & 1u) == 0u ? u : -u) + ((h & 2u) == 0u ? v : -v);
}
float perlin_noise3(const uint8_t* perm, float x, float y, float z) {
  float x0 = std::floor(x), y0 = std::floor(y), z0 = std::floor(z);
  int ix = (int)x0 & 255, iy = (int)y0 & 255, iz = (int)z0 & 255;
  float fx = x - x0, fy = y - y0, fz = z - z0;
  float u = pfade(fx), v = pfade(fy), w = pfade(fz);
  uint32_t A = (perm[ix & 255] + iy) & 255, B = (perm[(ix + 1) & 255] + iy) & 255;
  uint32_t AA = (perm[A] + iz) & 255, AB = (perm[(A + 1) & 255] + iz) & 255;
  uint32_t BA = (perm[B] + iz) & 255, BB = (perm[(B + 1) & 255] + iz) & 255;
  float q0 = plerp(pgrad(perm[AA], fx, fy, fz), pgrad(perm[BA], fx - 1.0f, fy, fz), u);
  float q1 = plerp(pgrad(perm[AB], fx, fy - 1.0f, fz), pgrad(perm[BB], fx - 1.0f, fy - 1.0f, fz), u);
  float q2 = plerp(pgrad(perm[(AA + 1) & 255], fx, fy, fz - 1.0f), pgrad(perm[(BA + 1) & 255], fx - 1.0f, fy, fz - 1.0f), u);
  float q3 = plerp(pgrad(perm[(AB + 1) & 255], fx, fy - 1.0f, fz - 1.0f),
                   pgrad(perm[(BB + 1) & 255], fx - 1.0f, fy - 1.0f, fz - 1.0f), u);
  return plerp(plerp(q0, q1, v), plerp(q2, q3, v), w);
}
float tex_perlin(const uint8_t* perm, float px, float py, float scale) {
  float x = px * scale, y = py * scale, z = 0.0f, result = 0.0f, amplitude = 1.0f;
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
float texture_sample(int kind, float param, const uint8_t* perm, float px, float py) {
  if (kind == 1) return tex_checker(px, py, (int)param);
  if (kind == 2) return tex_wave(px, param);
  if (kind == 3) return tex_perlin(perm, px, py, param);
  return 1.0f;
}

Mat Scene::shade_mat(int tri, V3 pos, V3 n) const {
  int mi = mesh_mat[tris[tri].mesh];
  Mat m = mats[mi];
  V3 tx = mat_tex[mi];
  if (tx.x != 0.0f) {
    float ax = std::fabs(n.x), ay = std::fabs(n.y), az = std::fabs(n.z);
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
    float sm = texture_sample((int)tx.x, tx.y, perm, px * tx.z, py * tx.z);
    m.base_color = scl(m.base_color, 0.25f + 0.75f * sm);
  }
  return m;
}

// the default texture permutation (include/rtx.h): Fisher-Yates over 0..255
// driven by splitmix64 from 0
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
    std::swap(p[i], p[j]);
  }
}

// object.cpp:107-167 — two-sided Moller-Trumbore variant
bool tri_intersect(const Tri& tr, V3 o, V3 d, float& t, float& u, float& v) {
  V3 pvec = cross(d, tr.e2);
  float det = dot(tr.e1, pvec);
  if (det > 0.0f) {
    V3 tvec = sub(o, tr.v0);
    float alpha = dot(pvec, tvec);
    if (alpha < 0.0f || alpha > det) return false;
    V3 qvec = cross(tvec, tr.e1);
    float beta = dot(qvec, d);
    if (beta < 0.0f || alpha + beta > det) return false;
    float inv_det = 1.0f / det;
    t = dot(tr.e2, qvec) * inv_det;
    if (t < 0.0f) return false;
    u = alpha * inv_det;
    v = beta * inv_det;
    return true;
  } else if (det < 0.0f) {
    V3 tvec = sub(o, tr.v0);
    float alpha = dot(pvec, tvec);
    if (alpha > 0.0f || alpha < det) return false;
    V3 qvec = cross(tvec, tr.e1);
    float beta = dot(qvec, d);
    if (beta > 0.0f || alpha + beta < det) return false;
    float inv_det = 1.0f / det;
    t = dot(tr.e2, qvec) * inv_det;
    if (t < 0.0f) return false;
    u = alpha * inv_det;
    v = beta * inv_det;
    return true;
  }
  return false;
}

void Scene::insert(int node, int item, const Box& bbox, int depth) {
  if (nodes[node].leaf) {
    if (nodes[node].items.empty() || depth == 8) {
      nodes[node].items.push_back(item);
    } else {
      nodes[node].leaf = false;
      while (!nodes[node].items.empty()) {
        int back = nodes[node].items.back();
        insert(node, back, bbox, depth);
        nodes[node].items.pop_back();
      }
      insert(node, item, bbox, depth);
    }
    return;
  }
  V3 c = tri_box[item].centroid();
  V3 nc = bbox.centroid();
  Box cb;
  int idx = 0;
  if (c.x > nc.x) {
    idx = 4;
    cb.lo.x = nc.x;
    cb.hi.x = bbox.hi.x;
  } else {
    cb.lo.x = bbox.lo.x;
    cb.hi.x = nc.x;
  }
  if (c.y > nc.y) {
    idx += 2;
    cb.lo.y = nc.y;
    cb.hi.y = bbox.hi.y;
  } else {
    cb.lo.y = bbox.lo.y;
    cb.hi.y = nc.y;
  }
  if (c.z > nc.z) {
    idx += 1;
    cb.lo.z = nc.z;
    cb.hi.z = bbox.hi.z;
  } else {
    cb.lo.z = bbox.lo.z;
    cb.hi.z = nc.z;
  }
  if (nodes[node].child[idx] < 0) {
    int nid = (int)nodes.size();
    nodes.emplace_back();
    nodes[node].child[idx] = nid;
  }
  insert(nodes[node].child[idx], item, cb, depth + 1);
}

void Scene::build(int node, const Box& bbox) {
  if (nodes[node].leaf) {
    for (int it : nodes[node].items) nodes[node].box.extend(tri_box[it]);
    return;
  }
  for (int i = 0; i < 8; ++i) {
    int ch = nodes[node].child[i];
    if (ch < 0) continue;
    Box cb;
    V3 c = bbox.centroid();
    cb.lo.x = (i & 4) ? c.x : bbox.lo.x;
    cb.hi.x = (i & 4) ? bbox.hi.x : c.x;
    cb.lo.y = (i & 2) ? c.y : bbox.lo.y;
    cb.hi.y = (i & 2) ? bbox.hi.y : c.y;
    cb.lo.z = (i & 1) ? c.z : bbox.lo.z;
    cb.hi.z = (i & 1) ? bbox.hi.z : c.z;
    build(ch, cb);
    nodes[node].box.extend(nodes[ch].box);
  }
}

struct QueueElement {  // bvh.h:54-63 — min-heap on t
  int node;
  float t;
  friend bool operator<(const QueueElement& a, const QueueElement& b) {
    return a.t > b.t;
  }
};

int Scene::intersect(V3 o, V3 d, int exclude, float& t, float& u, float& v,
                     V3* pos) const {
  t = kInf;
  int hit = -1;
  float t_min;
  float t_max = kInf;
  if (!nodes[0].box.intersect(o, d, t_min) || t_max < 0.0f) return -1;
  t = t_max;
  std::priority_queue<QueueElement> queue;
  queue.push(QueueElement{0, 0.0f});
  while (!queue.empty() && queue.top().t < t) {
    int node = queue.top().node;
    queue.pop();
    const OctNode& nd = nodes[node];
    if (nd.leaf) {
      for (int it : nd.items) {
        float it_t, iu, iv;
        if (it != exclude && tri_intersect(tris[it], o, d, it_t, iu, iv)) {
          if (it_t < t) {
            t = it_t;
            u = iu;
            v = iv;
            hit = it;
          }
        }
      }
    } else {
      for (int i = 0; i < 8; ++i) {
        int ch = nd.child[i];
        if (ch < 0) continue;
        float tc;
        if (nodes[ch].box.intersect(o, d, tc)) queue.push(QueueElement{ch, tc});
      }
    }
  }
  if (pos) *pos = add(o, scl(d, t));
  return hit;
}

V3 Scene::normal_at(int tri, float u, float v) const {
  const Tri& tr = tris[tri];
  if (mesh_smooth[tr.mesh]) {
    float w = 1 - u - v;
    return normalized(add(add(scl(tr.n0, w), scl(tr.n1, u)), scl(tr.n2, v)));
  }
  return tr.normal;
}

// ----------------------------------------------------------------------------
// Camera (src/renderer.cpp:103-124, src/object.cpp:42-64)
// ----------------------------------------------------------------------------
struct Cam {
  float m[16];
  float focal, gx, gy, near_, far_;
  float top, right;
};

Cam load_cam(const float* c, int W, int H) {
  Cam k;
  std::memcpy(k.m, c, 16 * sizeof(float));
  k.focal = c[16];
  k.gx = c[17];
  k.gy = c[18];
  k.near_ = c[19];
  k.far_ = c[20];
  // PrepareScreenSpace, renderer.cpp:103-124; InchToMM multiplies by float(25.4)
  k.top = ((k.gy * 25.4f) / 2.0f) / k.focal;
  k.right = ((k.gx * 25.4f) / 2.0f) / k.focal;
  float gate_aspr = k.gx / k.gy;
  float film_aspr = float(W) / float(H);
  float xscale = 1.0f, yscale = 1.0f;
  if (gate_aspr >= film_aspr)
    xscale = film_aspr / gate_aspr;
  else
    yscale = gate_aspr / film_aspr;
  k.right *= xscale;
  k.top *= yscale;
  return k;
}

// Matrix * (x, y, z, 1): row dot products accumulated from zero
// (rtmath.h:724-733, object.cpp:42-48)
inline V3 xform_point(const float* m, V3 p) {
  float r[3];
  for (int i = 0; i < 3; ++i) {
    float a = 0.0f;
    a += m[4 * i + 0] * p.x;
    a += m[4 * i + 1] * p.y;
    a += m[4 * i + 2] * p.z;
    a += m[4 * i + 3] * 1.0f;
    r[i] = a;
  }
  return v3(r[0], r[1], r[2]);
}

// renderer.cpp:252-259 (+ object.cpp:58-64)
void camera_ray(const Cam& k, int W, int H, int x, int y, V3& o, V3& d) {
  float dw = 1.0f / float(W);
  float dh = 1.0f / float(H);
  float nx = float(x) * dw, ny = float(y) * dh;
  float sx = 2.0f * k.right * nx - k.right;
  float sy = 2.0f * k.top * ny - k.top;
  o = xform_point(k.m, v3(0.0f, 0.0f, 0.0f));
  V3 p = xform_point(k.m, v3(sx, sy, -1.0f));
  d = normalized(sub(p, o));
}

// ----------------------------------------------------------------------------
// Path tracer (src/renderer.cpp:272-384)
// ----------------------------------------------------------------------------
struct RayState {
  float eta;
  V3 absorption{0.0f, 0.0f, 0.0f};
  V3 ffnormal{0.0f, 0.0f, 0.0f};
};

V3 emission_pdf(const Scene& s, int tri, V3 position, float u, float v, V3 to_pos,
                V3 out_dir, float& pdf) {  // surfacepoint.h:21-45
  V3 ray = sub(to_pos, position);
  float distance2 = dot(ray, ray);
  float cos_area = dot(out_dir, s.normal_at(tri, u, v)) * s.tris[tri].area;
  pdf = std::fabs(distance2 / cos_area);
  return s.mats[s.mesh_mat[s.tris[tri].mesh]].emission;
}

V3 DirectLight(const Scene& s, const RayState& state, V3 orig_dir, int tri,
               V3 pos, const Mat& m, Rng& rng) {  // renderer.cpp:335-384
  V3 ret = v3s(0.0f);
  if (s.emitters.empty()) return ret;  // world.cpp:7-16 (no draws)
  int e = s.emitters[rng.uniform_int(0, (int)s.emitters.size() - 1)];
  const Tri& et = s.tris[e];
  // object.cpp:169-178
  float sqr1 = std::sqrt(rng.uniform());
  float r2 = rng.uniform();
  float a = 1.0f - sqr1;
  float b = (1.0f - r2) * sqr1;
  V3 emit_pos = add(add(scl(et.e1, a), scl(et.e2, b)), et.v0);

  V3 dir = normalized(sub(emit_pos, pos));
  float t, u = 0.0f, v = 0.0f;
  int test = s.intersect(pos, dir, tri, t, u, v, nullptr);
  if (test < 0 || test == e) {
    if (test < 0) u = v = 0.0f;
    float lightpdf;
    V3 em = emission_pdf(s, e, emit_pos, u, v, pos, neg(dir), lightpdf);
    float bsdfpdf;
    V3 f = BsdfEval(m, state.eta, neg(orig_dir), state.ffnormal, dir, bsdfpdf);
    float weight = PowerHeuristic(lightpdf, bsdfpdf);
    if (bsdfpdf > 0.0f) {
      V3 c = scl(f, weight);
      c = mul(c, em);
      c = scl(c, (float)s.emitters.size());
      c = dvs(c, lightpdf);
      ret = add(ret, c);
    }
  }
  return ret;
}

V3 Radiance(const Scene& s, V3 o, V3 d, int last_hit, RayState& state, int depth,
            float last_bsdfpdf, int max_depth, Rng& rng) {  // renderer.cpp:272-333
  if (depth > max_depth - 1) return v3s(0.0f);
  float t, u, v;
  V3 hitpos;
  int hit = s.intersect(o, d, last_hit, t, u, v, &hitpos);
  V3 radiance = v3s(0.0f);
  if (hit >= 0) {
    state.ffnormal = s.normal_at(hit, u, v);
    const Mat m = s.shade_mat(hit, hitpos, state.ffnormal);
    if (dot(d, state.ffnormal) > 0.0f) {
      state.ffnormal = neg(state.ffnormal);
      state.eta = m.ior;
      state.absorption = v3s(0.0f);
    } else {
      state.eta = 1.0f / m.ior;
    }
    float self_pdf;
    V3 self_em = emission_pdf(s, hit, hitpos, u, v, o, neg(d), self_pdf);
    if (depth == 0)
      radiance = add(radiance, self_em);
    else
      radiance = add(radiance, scl(self_em, PowerHeuristic(last_bsdfpdf, self_pdf)));
    float dist = length(sub(hitpos, o));
    V3 expo = scl(neg(state.absorption), dist);
    V3 bounce_ratio = v3(std::pow(kE, expo.x), std::pow(kE, expo.y), std::pow(kE, expo.z));
    radiance = add(radiance, mul(DirectLight(s, state, d, hit, hitpos, m, rng), bounce_ratio));
    V3 next_dir, color;
    float bsdfpdf;
    if (BsdfSample(m, state.eta, state.ffnormal, neg(d), rng, next_dir, color, bsdfpdf)) {
      V3 lg = v3(std::log(m.extinction.x), std::log(m.extinction.y), std::log(m.extinction.z));
      state.absorption = dvs(neg(lg), m.at_distance);
      if (bsdfpdf > 0.0f) {
        V3 w = dvs(mul(bounce_ratio, color), bsdfpdf);
        V3 li = Radiance(s, hitpos, next_dir, hit, state, depth + 1, bsdfpdf, max_depth, rng);
        radiance = add(radiance, mul(w, li));
      }
    }
  } else {
    // world.cpp:39-42
    radiance = (-d.z < 0.0f) ? s.sky : s.ground;
  }
  return radiance;
}

inline int nthreads(int threads) {
#ifdef _OPENMP
  return threads > 0 ? threads : omp_get_max_threads();
#else
  (void)threads;
  return 1;
#endif
}

// ----------------------------------------------------------------------------
// Compositor (include/RenderToy/compositor.h:25-178, src/compositor.cpp:42-77)
// ----------------------------------------------------------------------------
// compositor.h:25-39: reflect without edge repeat; p == size maps to size.
// Returns the linear index, or -1 when it falls outside the buffer.
inline long reflect_index(long row, long col, long W, long H) {
  if (row < 0) row = -row;
  if (col < 0) col = -col;
  if (col >= W) col = 2 * W - col;
  if (row >= H) row = 2 * H - row;
  long idx = row * W + col;
  if (idx < 0 || idx >= W * H) return -1;
  return idx;
}

void convolve(const float* in, float* out, int W, int H, const float* k, int kr,
              int kc, bool normalize, bool lengthf, bool absval, int threads) {
  std::vector<float> tmp(in, in + (size_t)W * H * 3);
  long r2 = kr >> 1, c2 = kc >> 1;
#pragma omp parallel for num_threads(nthreads(threads)) schedule(static)
  for (long i = 0; i < H; ++i) {
    for (long j = 0; j < W; ++j) {
      V3 acc = v3s(0.0f);
      for (long ii = 0; ii < kr; ++ii) {
        for (long jj = 0; jj < kc; ++jj) {
          long idx = reflect_index(i - r2 + ii, j - c2 + jj, W, H);
          V3 p = idx < 0 ? v3s(0.0f) : v3(tmp[3 * idx], tmp[3 * idx + 1], tmp[3 * idx + 2]);
          acc = add(acc, scl(p, k[ii * kc + jj]));
        }
      }
      if (absval) acc = v3(std::fabs(acc.x), std::fabs(acc.y), std::fabs(acc.z));
      if (lengthf) acc = v3s(length(acc));
      if (normalize) acc = normalized(acc);
      float* o = out + 3 * (i * W + j);
      o[0] = acc.x;
      o[1] = acc.y;
      o[2] = acc.z;
    }
  }
}

// rtmath.h:1019-1059 (X and Y variants produce the same weights)
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

void gaussian_blur(const float* in, float* out, int W, int H, int size, float sigma,
                   int threads) {  // compositor.cpp:42-48
  std::vector<float> w(size), mid((size_t)W * H * 3);
  gaussian_weights(size, sigma, w.data());
  convolve(in, mid.data(), W, H, w.data(), 1, size, false, false, false, threads);
  convolve(mid.data(), out, W, H, w.data(), size, 1, false, false, false, threads);
}

}  // namespace

// ============================================================================
// C API
// ============================================================================
extern "C" {

void* orc_scene_create(int n_tris, const float* verts, const float* norms,
                       const int32_t* tri_mesh, int n_meshes,
                       const int32_t* mesh_mat, const uint8_t* mesh_smooth,
                       int n_mat, const float* mats, const float* sky,
                       const float* ground) {
  Scene* s = new Scene();
  s->tris.resize(n_tris);
  s->tri_box.resize(n_tris);
  for (int i = 0; i < n_tris; ++i) {
    Tri& t = s->tris[i];
    const float* p = verts + 9 * (size_t)i;
    t.v0 = v3(p[0], p[1], p[2]);
    t.v1 = v3(p[3], p[4], p[5]);
    t.v2 = v3(p[6], p[7], p[8]);
    if (norms) {
      const float* q = norms + 9 * (size_t)i;
      t.n0 = v3(q[0], q[1], q[2]);
      t.n1 = v3(q[3], q[4], q[5]);
      t.n2 = v3(q[6], q[7], q[8]);
    } else {
      t.n0 = t.n1 = t.n2 = v3s(0.0f);
    }
    t.mesh = tri_mesh[i];
    // Triangle::UpdateCache, object.cpp:224-243
    t.e1 = sub(t.v1, t.v0);
    t.e2 = sub(t.v2, t.v0);
    t.area = length(cross(t.e1, t.e2)) * 0.5f;
    V3 tangent = normalized(t.e1);
    t.normal = normalized(cross(tangent, sub(t.v2, t.v1)));
    // Triangle::BBox, object.cpp:83-99
    Box& b = s->tri_box[i];
    b.hi = v3(std::max(t.v0.x, std::max(t.v1.x, t.v2.x)),
              std::max(t.v0.y, std::max(t.v1.y, t.v2.y)),
              std::max(t.v0.z, std::max(t.v1.z, t.v2.z)));
    b.lo = v3(std::min(t.v0.x, std::min(t.v1.x, t.v2.x)),
              std::min(t.v0.y, std::min(t.v1.y, t.v2.y)),
              std::min(t.v0.z, std::min(t.v1.z, t.v2.z)));
  }
  s->mesh_mat.assign(mesh_mat, mesh_mat + n_meshes);
  s->mesh_smooth.assign(mesh_smooth, mesh_smooth + n_meshes);
  for (int i = 0; i < n_mat; ++i) {
    s->mats.push_back(load_mat(mats + 24 * (size_t)i));
    s->mat_tex.push_back(v3(mats[24 * (size_t)i + 21], mats[24 * (size_t)i + 22], mats[24 * (size_t)i + 23]));
  }
  default_texture_table(s->perm);
  s->sky = v3(sky[0], sky[1], sky[2]);
  s->ground = v3(ground[0], ground[1], ground[2]);
  // World::PrepareDirectLightSampling, world.cpp:24-37: meshes in order, their
  // triangles in id order, when the emission differs from zero (epsilon test)
  std::vector<std::vector<int>> mesh_tris(n_meshes);
  for (int i = 0; i < n_tris; ++i) mesh_tris[tri_mesh[i]].push_back(i);
  for (int mi = 0; mi < n_meshes; ++mi) {
    if (!eq_eps(s->mats[mesh_mat[mi]].emission, v3s(0.0f)))
      for (int t : mesh_tris[mi]) s->emitters.push_back(t);
  }
  // BVH::BVH, bvh.cpp:242-264
  Box tree;
  for (int i = 0; i < n_tris; ++i) tree.extend(s->tri_box[i]);
  s->tree_box = tree;
  s->nodes.emplace_back();
  for (int i = 0; i < n_tris; ++i) s->insert(0, i, tree, 0);
  s->build(0, tree);
  return s;
}

void orc_scene_destroy(void* scene) { delete (Scene*)scene; }

// Display resolve: Image::Tonemap<kITURBT709> (compositor.h:220-226,
// rtmath.h:1142-1177), Image::GammaCorrection (compositor.cpp:94-100)
void orc_tonemap_gamma(const float* in, int W, int H, float limit, float gamma, float* out) {
  float ratio = gamma > 0.0f ? 1.0f / gamma : 0.0f;
  for (size_t i = 0; i < (size_t)W * H; ++i) {
    float c[3] = {in[3 * i], in[3 * i + 1], in[3 * i + 2]};
    if (limit > 0.0f) {
      float luma = 0.2126f * c[0] + 0.7152f * c[1] + 0.0722f * c[2];
      float s = 1.0f + luma / limit;
      for (float& x : c) x = x * 1.0f / s;
    }
    if (gamma > 0.0f)
      for (float& x : c) x = std::pow(x, ratio);
    for (int k = 0; k < 3; ++k) out[3 * i + k] = c[k];
  }
}

// the exporters' quantisation (exporter.cpp:20-25, 82-88): int(255.99 *
// clamp(x, 0, 1)); std::clamp passes NaN through and int(NaN) is undefined
// (x86: INT_MIN, which the BMP's 8-bit field truncates to 0 and the PPM
// prints; Arm: 0) -- defined here as 0 for both files
static uint8_t quantise(float x) {
  if (!(x == x)) return 0;
  return (uint8_t)(int)(255.99f * std::clamp(x, 0.0f, 1.0f));
}

// BMPExporter / PPMExporter (exporter.cpp:8-95) into out; returns the size.
// BMP rows are zero-padded to 4 bytes and the header's size counts them.
long orc_encode(int bmp, const float* in, int W, int H, uint8_t* out, long cap) {
  std::string s;
  if (bmp) {
    size_t row = ((size_t)W * 3 + 3) & ~(size_t)3;
    s.assign(54 + row * H, '\0');
    auto p32 = [&](size_t o, uint32_t v) { for (int k = 0; k < 4; ++k) s[o + k] = (char)(v >> (8 * k)); };
    s[0] = 'B';
    s[1] = 'M';
    p32(2, (uint32_t)s.size());
    p32(10, 54);
    p32(14, 40);
    p32(18, (uint32_t)W);
    p32(22, (uint32_t)H);
    s[26] = 1;
    s[28] = 24;
    p32(38, 3780);
    p32(42, 3780);
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const float* c = in + 3 * ((size_t)y * W + x);
        size_t o = 54 + y * row + 3 * (size_t)x;
        s[o] = (char)quantise(c[2]);
        s[o + 1] = (char)quantise(c[1]);
        s[o + 2] = (char)quantise(c[0]);
      }
  } else {
    s = "P3\n" + std::to_string(W) + ' ' + std::to_string(H) + "\n255\n";
    for (size_t i = 0; i < (size_t)W * H; ++i)
      s += std::to_string(quantise(in[3 * i])) + ' ' + std::to_string(quantise(in[3 * i + 1])) + ' ' +
           std::to_string(quantise(in[3 * i + 2])) + '\n';
  }
  if ((long)s.size() <= cap) std::memcpy(out, s.data(), s.size());
  return (long)s.size();
}

void orc_scene_set_texture_table(void* scene, const uint8_t* perm) {
  std::memcpy(((Scene*)scene)->perm, perm, 256);
}

void orc_texture_sample(int kind, float param, const uint8_t* perm, int n, const float* uv, float* out) {
  uint8_t def[256];
  if (!perm) {
    default_texture_table(def);
    perm = def;
  }
  for (int i = 0; i < n; ++i) out[i] = texture_sample(kind, param, perm, uv[2 * i], uv[2 * i + 1]);
}

int orc_scene_emitters(void* scene, int32_t* out, int cap) {
  Scene* s = (Scene*)scene;
  int n = (int)s->emitters.size();
  for (int i = 0; i < n && i < cap; ++i) out[i] = s->emitters[i];
  return n;
}

void orc_intersect(void* scene, int n, const float* rays, const int32_t* exclude,
                   int32_t* out_tri, float* out_tuv, int threads) {
  const Scene* s = (const Scene*)scene;
#pragma omp parallel for num_threads(nthreads(threads)) schedule(dynamic, 64)
  for (int i = 0; i < n; ++i) {
    const float* r = rays + 6 * (size_t)i;
    float t, u = 0.0f, v = 0.0f;
    int h = s->intersect(v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]),
                         exclude ? exclude[i] : -1, t, u, v, nullptr);
    out_tri[i] = h;
    out_tuv[3 * i] = t;
    out_tuv[3 * i + 1] = h >= 0 ? u : 0.0f;
    out_tuv[3 * i + 2] = h >= 0 ? v : 0.0f;
  }
}

void orc_primary(void* scene, const float* cam, int W, int H, int32_t* out_tri,
                 float* out_tuv, int threads) {
  const Scene* s = (const Scene*)scene;
  Cam k = load_cam(cam, W, H);
#pragma omp parallel for num_threads(nthreads(threads)) schedule(dynamic, 4)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      V3 o, d;
      camera_ray(k, W, H, x, y, o, d);
      float t, u = 0.0f, v = 0.0f;
      int h = s->intersect(o, d, -1, t, u, v, nullptr);
      size_t p = (size_t)y * W + x;
      out_tri[p] = h;
      out_tuv[3 * p] = t;
      out_tuv[3 * p + 1] = h >= 0 ? u : 0.0f;
      out_tuv[3 * p + 2] = h >= 0 ? v : 0.0f;
    }
}

// renderer.cpp:138-229, 391-427
void orc_render_aov(void* scene, const float* cam, int W, int H, float near_,
                    float far_, float* normal, float* albedo, float* depth,
                    int threads) {
  const Scene* s = (const Scene*)scene;
  Cam k = load_cam(cam, W, H);
  float inv_range = 1.0f / (far_ - near_);
#pragma omp parallel for num_threads(nthreads(threads)) schedule(dynamic, 4)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      V3 o, d;
      camera_ray(k, W, H, x, y, o, d);
      float t, u = 0.0f, v = 0.0f;
      V3 pos;
      int h = s->intersect(o, d, -1, t, u, v, &pos);
      size_t p = 3 * ((size_t)y * W + x);
      V3 nv = v3s(0.0f), av = v3s(0.0f), dv = v3s(1.0f);
      if (h >= 0) {
        V3 n = s->normal_at(h, u, v);
        if (dot(s->tris[h].normal, neg(d)) < 0.0f) n = neg(n);
        nv = dvs(add(n, v3s(1.0f)), 2.0f);
        av = s->shade_mat(h, pos, n).base_color;
        dv = v3s(std::clamp((t - near_) * inv_range, 0.0f, 1.0f));
      }
      if (normal) { normal[p] = nv.x; normal[p + 1] = nv.y; normal[p + 2] = nv.z; }
      if (albedo) { albedo[p] = av.x; albedo[p + 1] = av.y; albedo[p + 2] = av.z; }
      if (depth) { depth[p] = dv.x; depth[p + 1] = dv.y; depth[p + 2] = dv.z; }
    }
}

void orc_trace_paths(void* scene, const float* cam, int W, int H,
                     const int32_t* pixels, int npix, int first_sample,
                     int n_samples, int max_depth, uint64_t seed, float* out,
                     int threads) {
  const Scene* s = (const Scene*)scene;
  Cam k = load_cam(cam, W, H);
  if (!pixels) npix = W * H;
  long total = (long)npix * n_samples;
#pragma omp parallel for num_threads(nthreads(threads)) schedule(dynamic, 16)
  for (long q = 0; q < total; ++q) {
    int si = (int)(q / npix);
    int pi = (int)(q % npix);
    int pix = pixels ? pixels[pi] : pi;
    int x = pix % W, y = pix / W;
    V3 o, d;
    camera_ray(k, W, H, x, y, o, d);
    Rng rng{seed, (uint32_t)pix, (uint32_t)(first_sample + si), 0u};
    RayState st;
    st.eta = 1.0f;
    V3 L = Radiance(*s, o, d, -1, st, 0, 0.0f, max_depth, rng);
    out[3 * q] = L.x;
    out[3 * q + 1] = L.y;
    out[3 * q + 2] = L.z;
  }
}

// renderer.cpp:236-270, accumulated race-free: sample order per pixel
void orc_render_pt(void* scene, const float* cam, int W, int H, int spp,
                   int max_depth, uint64_t seed, float* out, int threads) {
  const Scene* s = (const Scene*)scene;
  Cam k = load_cam(cam, W, H);
  long npix = (long)W * H;
#pragma omp parallel for num_threads(nthreads(threads)) schedule(dynamic, 8)
  for (long pix = 0; pix < npix; ++pix) {
    int x = (int)(pix % W), y = (int)(pix / W);
    V3 o, d;
    camera_ray(k, W, H, x, y, o, d);
    V3 acc = v3s(0.0f);
    for (int i = 0; i < spp; ++i) {
      Rng rng{seed, (uint32_t)pix, (uint32_t)i, 0u};
      RayState st;
      st.eta = 1.0f;
      V3 L = Radiance(*s, o, d, -1, st, 0, 0.0f, max_depth, rng);
      acc = add(acc, dvs(L, (float)spp));
    }
    out[3 * pix] = acc.x;
    out[3 * pix + 1] = acc.y;
    out[3 * pix + 2] = acc.z;
  }
}

void orc_bsdf_eval(const float* mat, float eta, const float* N, const float* V,
                   const float* L, float* f_out, float* pdf_out) {
  Mat m = load_mat(mat);
  float pdf;
  V3 f = BsdfEval(m, eta, v3(V[0], V[1], V[2]), v3(N[0], N[1], N[2]),
                  v3(L[0], L[1], L[2]), pdf);
  f_out[0] = f.x;
  f_out[1] = f.y;
  f_out[2] = f.z;
  *pdf_out = pdf;
}

int orc_bsdf_sample(const float* mat, float eta, const float* N,
                    const float* in_dir, uint64_t seed, uint32_t pixel,
                    uint32_t sample, float* out_dir, float* color,
                    float* pdf_out) {
  Mat m = load_mat(mat);
  Rng rng{seed, pixel, sample, 0u};
  V3 od = v3s(0.0f), c = v3s(0.0f);
  float pdf;
  bool ok = BsdfSample(m, eta, v3(N[0], N[1], N[2]), v3(in_dir[0], in_dir[1], in_dir[2]),
                       rng, od, c, pdf);
  out_dir[0] = od.x;
  out_dir[1] = od.y;
  out_dir[2] = od.z;
  color[0] = c.x;
  color[1] = c.y;
  color[2] = c.z;
  *pdf_out = pdf;
  return ok ? 1 : 0;
}

void orc_convolve(const float* in, float* out, int W, int H, const float* k,
                  int kr, int kc, int normalize, int lengthf, int absval) {
  convolve(in, out, W, H, k, kr, kc, normalize != 0, lengthf != 0, absval != 0, 0);
}

void orc_gaussian_weights(int size, float sigma, float* out) {
  gaussian_weights(size, sigma, out);
}

void orc_gaussian_blur(const float* in, float* out, int W, int H, int size,
                       float sigma) {
  gaussian_blur(in, out, W, H, size, sigma, 0);
}

// compositor.h:153-178: Sobel-X on a copy, Sobel-Y on self, |y + x| broadcast
void orc_edge_detect(const float* in, float* out, int W, int H) {
  static const float sx[9] = {-1, 0, 1, -2, 0, 2, -1, 0, 1};
  static const float sy[9] = {1, 2, 1, 0, 0, 0, -1, -2, -1};
  size_t n = (size_t)W * H * 3;
  std::vector<float> gx(n), gy(n);
  convolve(in, gx.data(), W, H, sx, 3, 3, false, false, false, 0);
  convolve(in, gy.data(), W, H, sy, 3, 3, false, false, false, 0);
  for (size_t p = 0; p < (size_t)W * H; ++p) {
    V3 a = v3(gy[3 * p], gy[3 * p + 1], gy[3 * p + 2]);
    V3 b = v3(gx[3 * p], gx[3 * p + 1], gx[3 * p + 2]);
    float l = length(add(a, b));
    out[3 * p] = out[3 * p + 1] = out[3 * p + 2] = l;
  }
}

// compositor.cpp:51-77
void orc_bloom(const float* in, float* out, int W, int H, int size, float sigma,
               float threshold) {
  size_t n = (size_t)W * H * 3;
  std::vector<float> layer(n), blurred(n);
  for (size_t p = 0; p < (size_t)W * H; ++p) {
    V3 c = v3(in[3 * p], in[3 * p + 1], in[3 * p + 2]);
    V3 e = luma(c) > threshold ? c : v3s(0.0f);
    layer[3 * p] = e.x;
    layer[3 * p + 1] = e.y;
    layer[3 * p + 2] = e.z;
  }
  gaussian_blur(layer.data(), blurred.data(), W, H, size, sigma, 0);
  for (size_t i = 0; i < n; ++i) out[i] = in[i] + blurred[i];
}

void orc_rng_floats(uint64_t seed, uint32_t pixel, uint32_t sample, int n,
                    float* out) {
  Rng rng{seed, pixel, sample, 0u};
  for (int i = 0; i < n; ++i) out[i] = rng.uniform();
}

}  // extern "C"
