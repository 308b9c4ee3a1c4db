// Scalar and vector arithmetic shared by every device stage of the renderer.
//
// Every expression here is written with an explicit evaluation order and with
// explicit fused multiply-adds (fmaf) where a fused form is wanted.  The whole
// library is compiled with implicit contraction switched off (nvcc -fmad=false,
// g++ -ffp-contract=off), so the same arithmetic produces the same bits on the
// GPU and in a CPU restatement that follows the same order.  Division and
// square root are the IEEE correctly rounded forms on both sides.
//
// Transcendentals are our own (Taylor / atanh series evaluated in float with a
// fixed Horner order) so that nothing depends on a vendor math library.
#pragma once

#include <stdint.h>
#include <math.h>
#include <vector_types.h>

#if defined(__CUDACC__)
#define MSC_HD __host__ __device__ __forceinline__
#else
#define MSC_HD static inline
#endif

namespace mscg {

// Constants of the reference renderer (include/core/Constants.h:12-17).
#define MSC_PI 3.14159265358979323846f
#define MSC_INV_PI 0.31830988618379067154f
#define MSC_PI_180 0.01745329251994329577f
#define MSC_EPSILON 1.1920928955078125e-07f /* FLT_EPSILON */
#define MSC_TNEAR 0.001f   /* RayDecompress.cpp:15 */
#define MSC_TFAR 100000.f  /* RayDecompress.cpp:16 */

MSC_HD float3 f3(float x, float y, float z) { float3 r; r.x = x; r.y = y; r.z = z; return r; }
MSC_HD float3 f3(float4 a) { return f3(a.x, a.y, a.z); }
MSC_HD float3 v_add(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
MSC_HD float3 v_sub(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
MSC_HD float3 v_mul(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
MSC_HD float3 v_cmul(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
MSC_HD float3 v_neg(float3 a) { return f3(-a.x, -a.y, -a.z); }

// dot(a,b) = fma(az,bz, fma(ay,by, ax*bx))
MSC_HD float v_dot(float3 a, float3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }

// cross(a,b)_i = fma(a_j, b_k, -(a_k*b_j))
MSC_HD float3 v_cross(float3 a, float3 b) {
  return f3(fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x)));
}

MSC_HD float v_len(float3 a) { return sqrtf(v_dot(a, a)); }

// normalize(a) = a * (1 / sqrt(dot(a,a)))
MSC_HD float3 v_normalize(float3 a) {
  float inv = 1.0f / sqrtf(v_dot(a, a));
  return v_mul(a, inv);
}

MSC_HD float v_maxc(float3 a) { return fmaxf(fmaxf(a.x, a.y), a.z); }

// Affine map stored row-major: p' = L p + t with L = m[r][0..2], t = m[r][3].
// Product order per row: fma(m2, p.z, fma(m1, p.y, m0*p.x)) + t.
struct Affine3 { float m[3][4]; };

MSC_HD float3 xf_point(const Affine3& a, float3 p) {
  return f3(fmaf(a.m[0][2], p.z, fmaf(a.m[0][1], p.y, a.m[0][0] * p.x)) + a.m[0][3],
            fmaf(a.m[1][2], p.z, fmaf(a.m[1][1], p.y, a.m[1][0] * p.x)) + a.m[1][3],
            fmaf(a.m[2][2], p.z, fmaf(a.m[2][1], p.y, a.m[2][0] * p.x)) + a.m[2][3]);
}

// sin and cos of the angle 2*pi*t for t in [0,1).  The quadrant k = floor(4t)
// is split off exactly (t - k/4 is exact by Sterbenz' lemma), the remainder
// x = 2*pi*r lies in [0, pi/2) and sin/cos are Taylor polynomials in x
// (truncation error below 1e-9 on that interval), evaluated by Horner.
MSC_HD void sincos_turns(float t, float* s_out, float* c_out) {
  float q = t * 4.0f;
  int k = (int)q;
  if (k < 0) k = 0;
  if (k > 3) k = 3;
  float r = t - (float)k * 0.25f;
  float x = r * 6.28318530717958647692f;
  float x2 = x * x;
  // sin x = x (1 - x^2/6 (1 - x^2/20 (1 - x^2/42 (1 - x^2/72 (1 - x^2/110 (1 - x^2/156))))))
  float ps = 1.0f - x2 * (1.0f / 156.0f);
  ps = 1.0f - x2 * (1.0f / 110.0f) * ps;
  ps = 1.0f - x2 * (1.0f / 72.0f) * ps;
  ps = 1.0f - x2 * (1.0f / 42.0f) * ps;
  ps = 1.0f - x2 * (1.0f / 20.0f) * ps;
  ps = 1.0f - x2 * (1.0f / 6.0f) * ps;
  float sn = x * ps;
  // cos x = 1 - x^2/2 (1 - x^2/12 (1 - x^2/30 (1 - x^2/56 (1 - x^2/90 (1 - x^2/132 (1 - x^2/182))))))
  float pc = 1.0f - x2 * (1.0f / 182.0f);
  pc = 1.0f - x2 * (1.0f / 132.0f) * pc;
  pc = 1.0f - x2 * (1.0f / 90.0f) * pc;
  pc = 1.0f - x2 * (1.0f / 56.0f) * pc;
  pc = 1.0f - x2 * (1.0f / 30.0f) * pc;
  pc = 1.0f - x2 * (1.0f / 12.0f) * pc;
  pc = 1.0f - x2 * (1.0f / 2.0f) * pc;
  float cs = pc;
  float so, co;
  if (k == 0) { so = sn; co = cs; }
  else if (k == 1) { so = cs; co = -sn; }
  else if (k == 2) { so = -sn; co = -cs; }
  else { so = -cs; co = sn; }
  *s_out = so;
  *c_out = co;
}

// log2(x) for finite x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)),
// log2(m) = (2/ln 2) atanh(s), s = (m-1)/(m+1), |s| < 0.1716, series to s^11.
MSC_HD float log2_pos(float x) {
  union { float f; uint32_t u; } b;
  b.f = x;
  int e = (int)((b.u >> 23) & 0xff) - 127;
  b.u = (b.u & 0x007fffffu) | 0x3f800000u;  // m in [1,2)
  float m = b.f;
  if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float p = 1.0f / 11.0f;
  p = p * s2 + 1.0f / 9.0f;
  p = p * s2 + 1.0f / 7.0f;
  p = p * s2 + 1.0f / 5.0f;
  p = p * s2 + 1.0f / 3.0f;
  p = p * s2 + 1.0f;
  return (float)e + s * p * 2.88539008177792681472f;  // 2/ln2
}

// 2^x for x in [-126, 127]: 2^x = 2^k e^(f ln2), f in [-0.5, 0.5], Taylor to f^8.
MSC_HD float exp2_f(float x) {
  if (x < -126.0f) return 0.0f;
  if (x > 127.0f) x = 127.0f;
  float kf = floorf(x + 0.5f);
  float f = (x - kf) * 0.69314718055994530942f;
  float p = 1.0f / 40320.0f;
  p = p * f + 1.0f / 5040.0f;
  p = p * f + 1.0f / 720.0f;
  p = p * f + 1.0f / 120.0f;
  p = p * f + 1.0f / 24.0f;
  p = p * f + 1.0f / 6.0f;
  p = p * f + 0.5f;
  p = p * f + 1.0f;
  p = p * f + 1.0f;
  union { float f; uint32_t u; } b;
  b.u = (uint32_t)((int)kf + 127) << 23;
  return p * b.f;
}

// x^y for x >= 0 (x == 0 gives 0 for y > 0).
MSC_HD float pow_pos(float x, float y) {
  if (x <= 0.0f) return 0.0f;
  return exp2_f(y * log2_pos(x));
}

// Counter-based generator: the 4-lane PCG hash of Jarzynski and Olano,
// "Hash Functions for GPU Rendering" (JCGT 9(3), 2020).
MSC_HD uint4 pcg4d(uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
  x = x * 1664525u + 1013904223u;
  y = y * 1664525u + 1013904223u;
  z = z * 1664525u + 1013904223u;
  w = w * 1664525u + 1013904223u;
  x += y * w; y += z * x; z += x * y; w += y * z;
  x ^= x >> 16; y ^= y >> 16; z ^= z >> 16; w ^= w >> 16;
  x += y * w; y += z * x; z += x * y; w += y * z;
  uint4 r; r.x = x; r.y = y; r.z = z; r.w = w;
  return r;
}

// Uniform float in [0,1) from the top 24 bits (exact).
MSC_HD float u01(uint32_t v) { return (float)(v >> 8) * 5.9604644775390625e-08f; }

// Per-path draws: `slot` 0 is the camera, slot d+1 the hit at depth d;
// `lane` selects one of several independent 4-draw blocks of that slot.  The
// iteration and the scene seed enter the third word so every process() call
// draws afresh.
MSC_HD uint4 path_draws(uint32_t sample_id, uint32_t iter_seed, uint32_t slot, uint32_t lane) {
  return pcg4d(sample_id, slot, iter_seed, lane);
}

MSC_HD uint32_t iteration_seed(uint32_t seed, uint32_t iteration) {
  return seed * 0x85ebca6bu ^ (iteration * 0xc2b2ae35u + 0x27d4eb2fu);
}

// Cardinal direction bin: dominant axis by magnitude (ties to the lower axis),
// then sign; matches Camera.cpp:42-44 and Integrator.cpp:240-242.
MSC_HD int cardinal_bin(float3 d) {
  int m = (fabsf(d.x) < fabsf(d.y)) ? 1 : 0;
  float dm = (m == 1) ? d.y : d.x;
  int axis = (fabsf(dm) < fabsf(d.z)) ? 2 : m;
  float da = (axis == 0) ? d.x : ((axis == 1) ? d.y : d.z);
  return (da < 0.f) ? axis : axis + 3;
}

// Direction bin among 6 (cardinal_bin), 26 or 98: the surface cells of an
// m^3 cube (m = 3 or 5) over [-1,1]^3, the direction scaled so that its
// largest component has magnitude 1.  Cells are numbered in x-major order
// with the (m-2)^3 interior cells skipped.
MSC_HD int ray_bin(float3 d, int nbins) {
  if (nbins == 6) return cardinal_bin(d);
  const int m = nbins == 26 ? 3 : 5;
  const float mx = fmaxf(fmaxf(fabsf(d.x), fabsf(d.y)), fabsf(d.z));
  if (!(mx > 0.f)) return 0;
  const float inv = 1.0f / mx;
  const float half_m = 0.5f * (float)m;
  int c[3];
  const float v[3] = {d.x * inv, d.y * inv, d.z * inv};
  for (int a = 0; a < 3; ++a) {
    int q = (int)floorf((v[a] + 1.0f) * half_m);
    c[a] = q < 0 ? 0 : (q > m - 1 ? m - 1 : q);
  }
  const int n_in = m - 2;
  auto below = [&](int x) { return x - 1 < 0 ? 0 : (x - 1 > n_in ? n_in : x - 1); };
  auto inner = [&](int x) { return (x >= 1 && x <= m - 2) ? 1 : 0; };
  const int interior_before =
      below(c[0]) * n_in * n_in + inner(c[0]) * (below(c[1]) * n_in + inner(c[1]) * below(c[2]));
  return (c[0] * m + c[1]) * m + c[2] - interior_before;
}

MSC_HD uint32_t spread_bits_3(uint32_t v) {  // 10 bits -> every third bit
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

MSC_HD int clamp_i(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Quantise v in [lo, lo + 1/scale] to [0, cells-1].
MSC_HD uint32_t quantise(float v, float lo, float scale, int cells) {
  float q = (v - lo) * scale;
  int i = (int)floorf(q);
  return (uint32_t)clamp_i(i, 0, cells - 1);
}

// 32-bit ray sort key: a five-dimensional Morton code of the origin (3 x 6
// bits, in the batch origin box) and the direction (2 x 7 bits: the two minor
// direction components divided by the dominant one, each in [-1,1]).  From
// the top, each of six levels holds one bit of x, y, z, u, v (coarse to
// fine), and the last two bits are the finest u, v bits; so every prefix of
// the key refines origin and direction together, and a sort on its top bits
// alone already groups rays that start close together and point the same
// way.  Sorting by origin and direction is the order the reference's median
// split refines a batch in (RaySort.cpp:11-117).
MSC_HD uint32_t ray_sort_key(float3 o, float3 d, float3 lo, float3 scale) {
  const uint32_t qx = quantise(o.x, lo.x, scale.x, 64);
  const uint32_t qy = quantise(o.y, lo.y, scale.y, 64);
  const uint32_t qz = quantise(o.z, lo.z, scale.z, 64);
  const int c = cardinal_bin(d) % 3;
  const float da = (c == 0) ? d.x : ((c == 1) ? d.y : d.z);
  const float du = (c == 0) ? d.y : ((c == 1) ? d.z : d.x);
  const float dv = (c == 0) ? d.z : ((c == 1) ? d.x : d.y);
  const float inv = 1.0f / fabsf(da);
  const uint32_t qu = quantise(du * inv, -1.0f, 64.0f, 128);
  const uint32_t qv = quantise(dv * inv, -1.0f, 64.0f, 128);
  uint32_t key = 0u;
  for (int l = 0; l < 6; ++l) {
    key = (key << 5) | (((qx >> (5 - l)) & 1u) << 4) | (((qy >> (5 - l)) & 1u) << 3) |
          (((qz >> (5 - l)) & 1u) << 2) | (((qu >> (6 - l)) & 1u) << 1) | ((qv >> (6 - l)) & 1u);
  }
  return (key << 2) | ((qu & 1u) << 1) | (qv & 1u);
}

}  // namespace mscg
