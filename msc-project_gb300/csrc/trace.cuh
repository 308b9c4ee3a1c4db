// Binary LBVH layout and the stack-in-registers traversal used for both the
// closest-hit query (replacing rtcIntersect, src/core/RayIntersect.cpp:7-12)
// and the occlusion query (replacing rtcOccluded with the light mask
// 0x0FFFFFFF, src/core/Integrator.cpp:153-174).
//
// Node i (internal) = 4 float4:
//   n0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   n1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   n2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   n3 = (child0, child1, 0, 0) as ints; a child >= 0 is an internal node,
//        a child < 0 is the leaf ~k holding triangle k (in leaf order).
// Triangle k = 3 float4: (v0, geomID), (e1 = v1 - v0, is_light), (e2 = v2 - v0, global prim).
#pragma once

#include "dmath.h"

namespace mscg {

constexpr int kTraceStack = 64;
constexpr int kTraceStepCap = 1 << 22;

struct TriHit {
  float t, u, v;
  int tri;  // leaf-order triangle index, -1 for a miss
};

// Moller-Trumbore with u, v the weights of v1 and v2 (the barycentric
// convention PolygonObject::texture relies on, src/core/PolygonObject.cpp:45-63).
// Accepts tmin < t < tmax, or tmin < t <= tmax when CLOSED (the closest-hit
// queries, which settle equal distances by the triangle's scene index).
// Before the IEEE reciprocal, candidates are rejected in det-scaled terms only
// where the exact test below would reject them too: the signs of u and v are
// exact, and the upper bounds keep a margin far above the rounding of the
// scaled sums, so the accepted set and every result are unchanged.
template <bool CLOSED>
__device__ __forceinline__ bool tri_intersect(float3 o, float3 d, float3 v0, float3 e1, float3 e2, float tmin,
                                              float tmax, float* t_out, float* u_out, float* v_out) {
  float3 p = v_cross(d, e2);
  float det = v_dot(e1, p);
  if (det == 0.0f) return false;
  float3 s = v_sub(o, v0);
  const float us = v_dot(s, p);  // u * det
  const float adet = fabsf(det);
  const float su = det > 0.0f ? us : -us;  // u * |det|
  if (su < 0.0f || su > adet * 1.00001f) return false;
  float3 q = v_cross(s, e1);
  const float vs = v_dot(d, q);  // v * det
  const float sv = det > 0.0f ? vs : -vs;
  if (sv < 0.0f || su + sv > adet * 1.00001f) return false;
  float inv = 1.0f / det;
  float u = us * inv;
  if (u < 0.0f || u > 1.0f) return false;
  float v = vs * inv;
  if (v < 0.0f || u + v > 1.0f) return false;
  float t = v_dot(e2, q) * inv;
  if (!(t > tmin && (CLOSED ? t <= tmax : t < tmax))) return false;
  *t_out = t;
  *u_out = u;
  *v_out = v;
  return true;
}

// Closest-hit acceptance of a candidate at distance t <= tmax with scene
// triangle index g: nearer, or as near with a smaller index (best_g < 0 until
// the first hit, so a first hit must be strictly inside tmax).  The result is
// then the same whatever order the candidates are met in.
__device__ __forceinline__ bool closer_hit(float t, int g, float tmax, int best_g) {
  return t < tmax || g < best_g;
}

__device__ __forceinline__ float safe_rcp(float x) {
  const float tiny = 1e-12f;
  if (fabsf(x) < tiny) x = x < 0.0f ? -tiny : tiny;
  return 1.0f / x;
}

// Returns true on a hit.  ANY: stop at the first hit, skipping light triangles.
// *overflow is set to 1 when the traversal stack would overflow (the ray is then
// answered from the part of the tree already visited) and to 2 at the step cap.
template <bool ANY>
__device__ __forceinline__ bool bvh_trace(const float4* __restrict__ nodes, const float4* __restrict__ tris, float3 o,
                                          float3 d, float tmin, float tmax, TriHit* hit, int* overflow) {
  const float3 id = f3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
  const float3 ood = f3(o.x * id.x, o.y * id.y, o.z * id.z);
  int stack[kTraceStack];
  int sp = 0;
  int node = 0;
  bool found = false;
  // box test bound widened by a few ulps so rounding never culls a true hit
  const float widen = 1.0000004f;
  // a well-formed tree visits far fewer nodes; the cap only guards against a
  // malformed one (reported through *overflow = 2)
  int steps = 0;
  int best_g = -1;
  while (true) {
    while (node >= 0) {
      if (++steps > kTraceStepCap) {
        *overflow = 2;
        return found;
      }
      const float4 n0 = __ldg(&nodes[4 * node + 0]);
      const float4 n1 = __ldg(&nodes[4 * node + 1]);
      const float4 n2 = __ldg(&nodes[4 * node + 2]);
      const float4 n3 = __ldg(&nodes[4 * node + 3]);
      const float c0lx = fmaf(n0.x, id.x, -ood.x), c0hx = fmaf(n0.y, id.x, -ood.x);
      const float c0ly = fmaf(n0.z, id.y, -ood.y), c0hy = fmaf(n0.w, id.y, -ood.y);
      const float c0lz = fmaf(n2.x, id.z, -ood.z), c0hz = fmaf(n2.y, id.z, -ood.z);
      const float c1lx = fmaf(n1.x, id.x, -ood.x), c1hx = fmaf(n1.y, id.x, -ood.x);
      const float c1ly = fmaf(n1.z, id.y, -ood.y), c1hy = fmaf(n1.w, id.y, -ood.y);
      const float c1lz = fmaf(n2.z, id.z, -ood.z), c1hz = fmaf(n2.w, id.z, -ood.z);
      const float c0min = fmaxf(fmaxf(fminf(c0lx, c0hx), fminf(c0ly, c0hy)), fmaxf(fminf(c0lz, c0hz), tmin));
      const float c0max = fminf(fminf(fmaxf(c0lx, c0hx), fmaxf(c0ly, c0hy)), fminf(fmaxf(c0lz, c0hz), tmax)) * widen;
      const float c1min = fmaxf(fmaxf(fminf(c1lx, c1hx), fminf(c1ly, c1hy)), fmaxf(fminf(c1lz, c1hz), tmin));
      const float c1max = fminf(fminf(fmaxf(c1lx, c1hx), fmaxf(c1ly, c1hy)), fminf(fmaxf(c1lz, c1hz), tmax)) * widen;
      const bool t0 = c0min <= c0max;
      const bool t1 = c1min <= c1max;
      const int ch0 = __float_as_int(n3.x), ch1 = __float_as_int(n3.y);
      if (t0 && t1) {
        int nearc = ch0, farc = ch1;
        if (c1min < c0min) { nearc = ch1; farc = ch0; }
        if (sp < kTraceStack) stack[sp++] = farc;
        else *overflow = 1;
        node = nearc;
      } else if (t0) {
        node = ch0;
      } else if (t1) {
        node = ch1;
      } else {
        if (sp == 0) return found;
        node = stack[--sp];
      }
    }
    // leaf
    {
      const int k = ~node;
      const float4 a = __ldg(&tris[3 * k + 0]);
      const float4 b = __ldg(&tris[3 * k + 1]);
      const float4 c = __ldg(&tris[3 * k + 2]);
      if (!ANY || __float_as_int(b.w) == 0) {
        float t, u, v;
        if (tri_intersect<!ANY>(o, d, f3(a), f3(b), f3(c), tmin, tmax, &t, &u, &v)) {
          if (ANY) return true;
          const int g = __float_as_int(c.w);
          if (closer_hit(t, g, tmax, best_g)) {
            found = true;
            tmax = t;
            best_g = g;
            hit->t = t;
            hit->u = u;
            hit->v = v;
            hit->tri = k;
          }
        }
      }
    }
    if (sp == 0) return found;
    node = stack[--sp];
  }
}

// ------------------------------------------------------------ 8-wide BVH
// Node = 5 uint4 (80 bytes):
//   w0..w2  node box origin p (float bits)
//   w3      per-axis step exponents e+127 (bits 0-23) and the internal-child mask (bits 24-31)
//   w4      index of the first internal child node (internal children are consecutive)
//   w5      index of the first leaf triangle (leaf triangles of a node are consecutive)
//   w6      valid triangle bits: slot s owns bits 2s, 2s + 1 (one per triangle of a
//           leaf slot); the triangle of bit b is w5 + popc(w6 & ((1 << b) - 1))
//   w7      0
//   w8..w19 quantised child boxes, one byte per slot: lo.x, lo.y, lo.z, hi.x, hi.y, hi.z,
//           two words each (slots 0-3, 4-7); child box = p + q * 2^e per axis.
// Traversal keeps node groups, not single children (Ylitie, Karras and Laine,
// HPG 2017): a group is a node's child base, its internal-child mask and the
// children still to visit, as bits in the ray's octant order (bit j = slot
// j ^ octant).  The slots were assigned by octant at build time, so taking
// the lowest bit first visits the children roughly front to back.  Each
// visited node also yields a triangle group (triangle base, the node's valid
// triangle bits and the bits of its hit leaf slots), intersected before the
// next node.
constexpr int kWideStack = 64;

// Three-input minimum and maximum (PTX ISA 8.8, sm_100 and later); like
// fminf / fmaxf they return the other inputs when one is NaN.
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Moves bit s of an 8-bit mask to bit s ^ oct: one masked delta swap per
// octant bit (adjacent bits, bit pairs, nibbles); m1, m2, m4 are 0x55, 0x33,
// 0x0f where the ray's octant has that bit, else 0.  t holds bits only where
// the multiply's shifted copy cannot carry into them.
__device__ __forceinline__ uint32_t octant_order(uint32_t x, uint32_t m1, uint32_t m2, uint32_t m4) {
  uint32_t t = (x ^ (x >> 1)) & m1;
  x ^= t * 3u;
  t = (x ^ (x >> 2)) & m2;
  x ^= t * 5u;
  t = (x ^ (x >> 4)) & m4;
  x ^= t * 17u;
  return x;
}

// Bit s of an 8-bit mask onto bits 2s and 2s + 1.
__device__ __forceinline__ uint32_t spread_pairs(uint32_t x) {
  x = (x | (x << 4)) & 0x0f0fu;
  x = (x | (x << 2)) & 0x3333u;
  x = (x | (x << 1)) & 0x5555u;
  return x * 3u;
}

// Byte s of the pair as the float 1 + byte * 2^-15, exactly: one byte
// permute places the byte in the mantissa of 1.0f.  A plane at p + q * step
// then meets the ray at (1 + q * 2^-15) * A + (b - A) with A = 2^15 * step / d
// and b = (p - o) / d, so the conversion's subtraction moves out of the
// per-slot work into one per-axis bias per node.
__device__ __forceinline__ float byte_unit(uint32_t lo_word, uint32_t hi_word, int s) {
  return __uint_as_float(__byte_perm(s < 4 ? lo_word : hi_word, 0x3F800000u, 0x7604u | ((uint32_t)(s & 3) << 4)));
}

// The eight child boxes of wide node `node` against the ray: returns the node
// group (child base, internal mask, hit internal children in octant order)
// and the triangle group (base, the node's valid triangle bits, the bits of
// the hit leaf slots).  Entry distances are rounded down and exit distances
// up, bias included (A * f is exact in the fused multiply-add, the bias is
// the only other rounding), so every distance bounds the one computed from
// the exact byte value: no true intersection of a box is culled.
struct Node8Result {
  uint32_t g_base, g_imask, g_hits, t_base, t_valid, t_mask;
};

__device__ __forceinline__ Node8Result node8_test(const uint4* __restrict__ wn, int node, float3 o, float3 id,
                                                  uint32_t oct, float tmin, float tmax) {
  const uint4 A = __ldg(&wn[5 * node + 0]);
  const uint4 B = __ldg(&wn[5 * node + 1]);
  const uint4 Q0 = __ldg(&wn[5 * node + 2]);
  const uint4 Q1 = __ldg(&wn[5 * node + 3]);
  const uint4 Q2 = __ldg(&wn[5 * node + 4]);
  const float sx = __int_as_float((int)((A.w & 0xffu) << 23));
  const float sy = __int_as_float((int)(((A.w >> 8) & 0xffu) << 23));
  const float sz = __int_as_float((int)(((A.w >> 16) & 0xffu) << 23));
  const uint32_t imask = A.w >> 24;
  // per axis: the step in ray distance, scaled by 2^15 (exact), and the bias
  // b - A rounded down for entries and up for exits
  const float ax = (sx * id.x) * 32768.0f, ay = (sy * id.y) * 32768.0f, az = (sz * id.z) * 32768.0f;
  const float bx = (__uint_as_float(A.x) - o.x) * id.x;
  const float by = (__uint_as_float(A.y) - o.y) * id.y;
  const float bz = (__uint_as_float(A.z) - o.z) * id.z;
  const float bnx = __fsub_rd(bx, ax), bny = __fsub_rd(by, ay), bnz = __fsub_rd(bz, az);
  const float bfx = __fsub_ru(bx, ax), bfy = __fsub_ru(by, ay), bfz = __fsub_ru(bz, az);
  // per axis, the entry plane of a child box is its low plane when the
  // inverse direction is positive and its high plane otherwise (the step
  // scale is positive), so the slab min/max reduce to a choice per node
  const bool nx = id.x < 0.f, ny = id.y < 0.f, nz = id.z < 0.f;
  // quantised planes: lo x (Q0.x, Q0.y), lo y (Q0.z, Q0.w), lo z (Q1.x, Q1.y),
  // hi x (Q1.z, Q1.w), hi y (Q2.x, Q2.y), hi z (Q2.z, Q2.w); words for slots 0-3, 4-7
  const uint32_t enx0 = nx ? Q1.z : Q0.x, enx1 = nx ? Q1.w : Q0.y, exx0 = nx ? Q0.x : Q1.z, exx1 = nx ? Q0.y : Q1.w;
  const uint32_t eny0 = ny ? Q2.x : Q0.z, eny1 = ny ? Q2.y : Q0.w, exy0 = ny ? Q0.z : Q2.x, exy1 = ny ? Q0.w : Q2.y;
  const uint32_t enz0 = nz ? Q2.z : Q1.x, enz1 = nz ? Q2.w : Q1.y, exz0 = nz ? Q1.x : Q2.z, exz1 = nz ? Q1.y : Q2.w;
  const float widen = 1.0000004f;
  uint32_t hm = 0u;  // bit s: the box of slot s is hit
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    const float tnx = __fmaf_rd(byte_unit(enx0, enx1, s), ax, bnx);
    const float tny = __fmaf_rd(byte_unit(eny0, eny1, s), ay, bny);
    const float tnz = __fmaf_rd(byte_unit(enz0, enz1, s), az, bnz);
    const float tfx = __fmaf_ru(byte_unit(exx0, exx1, s), ax, bfx);
    const float tfy = __fmaf_ru(byte_unit(exy0, exy1, s), ay, bfy);
    const float tfz = __fmaf_ru(byte_unit(exz0, exz1, s), az, bfz);
    const float tn = fmax3(tnx, tny, fmaxf(tnz, tmin));
    const float tf = fmin3(tfx, tfy, fminf(tfz, tmax)) * widen;
    if (tn <= tf) hm |= 1u << s;
  }
  Node8Result r;
  r.g_base = B.x;
  r.g_imask = imask;
  r.g_hits = octant_order(hm & imask, (oct & 1u) ? 0x55u : 0u, (oct & 2u) ? 0x33u : 0u, (oct & 4u) ? 0x0fu : 0u);
  r.t_base = B.y;
  r.t_valid = B.z;
  // empty slots own no valid bits, so their (degenerate) boxes add nothing
  r.t_mask = spread_pairs(hm & ~imask) & B.z;
  return r;
}

// Triangle of the lowest bit of a node's triangle mask, which it clears.
__device__ __forceinline__ int take_triangle(uint32_t& t_mask, uint32_t t_base, uint32_t t_valid) {
  const uint32_t lb = t_mask & (0u - t_mask);
  t_mask ^= lb;
  return (int)(t_base + (uint32_t)__popc(t_valid & (lb - 1u)));
}

// Node and triangle indices are checked against num_nodes / num_tris before
// every fetch; a bad index ends the ray with *overflow = 3 instead of reading
// outside the arrays.
template <bool ANY>
__device__ __forceinline__ bool bvh8_trace(const uint4* __restrict__ wn, const float4* __restrict__ tris,
                                           int num_nodes, int num_tris, float3 o, float3 d, float tmin, float tmax,
                                           TriHit* hit, int* overflow) {
  const float3 id = f3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
  const uint32_t oct = (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
  uint2 stack[kWideStack];
  int sp = 0;
  // the root as the only child of a virtual group: base 0, slot 0 internal
  uint32_t g_base = 0, g_imask = 1u, g_hits = 1u << oct;
  uint32_t t_base = 0, t_valid = 0, t_mask = 0;
  bool found = false;
  int steps = 0;
  int best_g = -1;
  while (true) {
    if (g_hits != 0u && t_mask == 0u) {
      const uint32_t j = (uint32_t)(__ffs(g_hits) - 1);
      g_hits &= g_hits - 1u;
      const uint32_t slot = j ^ oct;
      const int node = (int)(g_base + __popc(g_imask & ((1u << slot) - 1u)));
      if (g_hits != 0u) {
        if (sp < kWideStack) stack[sp++] = make_uint2(g_base, (g_imask << 8) | g_hits);
        else *overflow = 1;
      }
      if (++steps > kTraceStepCap) {
        *overflow = 2;
        return found;
      }
      if (node >= num_nodes) {
        *overflow = 3;
        return found;
      }
      const Node8Result r = node8_test(wn, node, o, id, oct, tmin, tmax);
      g_base = r.g_base;
      g_imask = r.g_imask;
      g_hits = r.g_hits;
      t_base = r.t_base;
      t_valid = r.t_valid;
      t_mask = r.t_mask;
    }
    while (t_mask != 0u) {
      const int k = take_triangle(t_mask, t_base, t_valid);
      if (k >= num_tris) {
        *overflow = 3;
        return found;
      }
      const float4 a = __ldg(&tris[3 * k + 0]);
      const float4 b = __ldg(&tris[3 * k + 1]);
      const float4 c = __ldg(&tris[3 * k + 2]);
      if (ANY && __float_as_int(b.w) != 0) continue;
      float t, u, v;
      if (tri_intersect<!ANY>(o, d, f3(a), f3(b), f3(c), tmin, tmax, &t, &u, &v)) {
        if (ANY) return true;
        const int g = __float_as_int(c.w);
        if (closer_hit(t, g, tmax, best_g)) {
          found = true;
          tmax = t;
          best_g = g;
          hit->t = t;
          hit->u = u;
          hit->v = v;
          hit->tri = k;
        }
      }
    }
    if (g_hits == 0u) {
      if (sp == 0) return found;
      const uint2 e = stack[--sp];
      g_base = e.x;
      g_imask = e.y >> 8;
      g_hits = e.y & 0xffu;
    }
  }
}

// ------------------------------------------------- stepwise 8-wide traversal
// The same traversal as bvh8_trace, one step at a time: a step tests one
// triangle, visits one node, or pops one node group.  A persistent kernel
// keeps one ray per lane and, when a lane's ray ends, hands the lane a new ray
// (Aila and Laine, "Understanding the Efficiency of Ray Traversal on GPUs",
// HPG 2009), so warps stay full instead of waiting for their slowest ray.
// Hits are identical to bvh8_trace's: both return the nearest candidate,
// equal distances settled by the smaller scene triangle index.
struct Trav8 {
  float3 o, d, id;
  float tmin, tmax;
  uint32_t oct;
  uint32_t g_base, g_imask, g_hits, t_base, t_valid, t_mask;
  int sp, steps, best_g;
  bool found;
};

__device__ __forceinline__ void trav8_init(Trav8& s, float3 o, float3 d, float tmin, float tmax) {
  s.o = o;
  s.d = d;
  s.id = f3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
  s.tmin = tmin;
  s.tmax = tmax;
  s.oct = (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
  s.g_base = 0;
  s.g_imask = 1u;
  s.g_hits = 1u << s.oct;
  s.t_base = 0;
  s.t_valid = 0;
  s.t_mask = 0;
  s.sp = 0;
  s.steps = 0;
  s.best_g = -1;
  s.found = false;
}

// One step; returns true when the ray is finished (*overflow set on errors).
template <bool ANY>
__device__ __forceinline__ bool trav8_step(Trav8& s, uint2* stack, const uint4* __restrict__ wn,
                                           const float4* __restrict__ tris, int num_nodes, int num_tris, TriHit* hit,
                                           int* overflow) {
  if (s.t_mask != 0u) {
    const int k = take_triangle(s.t_mask, s.t_base, s.t_valid);
    if (k >= num_tris) {
      *overflow = 3;
      return true;
    }
    const float4 a = __ldg(&tris[3 * k + 0]);
    const float4 b = __ldg(&tris[3 * k + 1]);
    const float4 c = __ldg(&tris[3 * k + 2]);
    if (ANY && __float_as_int(b.w) != 0) return false;
    float t, u, v;
    if (tri_intersect<!ANY>(s.o, s.d, f3(a), f3(b), f3(c), s.tmin, s.tmax, &t, &u, &v)) {
      if (ANY) {
        s.found = true;
        return true;
      }
      const int g = __float_as_int(c.w);
      if (closer_hit(t, g, s.tmax, s.best_g)) {
        s.found = true;
        s.tmax = t;
        s.best_g = g;
        hit->t = t;
        hit->u = u;
        hit->v = v;
        hit->tri = k;
      }
    }
    return false;
  }
  if (s.g_hits != 0u) {
    const uint32_t j = (uint32_t)(__ffs(s.g_hits) - 1);
    s.g_hits &= s.g_hits - 1u;
    const uint32_t slot = j ^ s.oct;
    const int node = (int)(s.g_base + __popc(s.g_imask & ((1u << slot) - 1u)));
    if (s.g_hits != 0u) {
      if (s.sp < kWideStack) stack[s.sp++] = make_uint2(s.g_base, (s.g_imask << 8) | s.g_hits);
      else *overflow = 1;
    }
    if (++s.steps > kTraceStepCap) {
      *overflow = 2;
      return true;
    }
    if (node >= num_nodes) {
      *overflow = 3;
      return true;
    }
    const Node8Result r = node8_test(wn, node, s.o, s.id, s.oct, s.tmin, s.tmax);
    s.g_base = r.g_base;
    s.g_imask = r.g_imask;
    s.g_hits = r.g_hits;
    s.t_base = r.t_base;
    s.t_valid = r.t_valid;
    s.t_mask = r.t_mask;
    return false;
  }
  if (s.sp == 0) return true;
  const uint2 e = stack[--s.sp];
  s.g_base = e.x;
  s.g_imask = e.y >> 8;
  s.g_hits = e.y & 0xffu;
  return false;
}

}  // namespace mscg
