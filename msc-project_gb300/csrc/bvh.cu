// Device LBVH build (Karras, "Maximizing Parallelism in the Construction of
// BVHs, Octrees, and k-d Trees", HPG 2012), replacing the Embree scene build
// of the reference (rtcNewTriangleMesh/rtcCommit, src/core/Pathtracer.cpp:171-201,
// 242-274).  Steps: centroid bounds -> 30-bit Morton codes -> stable radix
// sort -> one thread per internal node finds its range and split -> one
// thread per leaf walks to the root, the second arrival at each node
// forming its box -> treelet restructuring rounds (SAH) -> pack into the
// traversal layout of trace.cuh.
#include <algorithm>
#include <array>
#include <functional>
#include <limits>
#include <cmath>
#include <cstring>
#include <vector>

#include "bvh.h"
#include "dmath.h"
#include "radix.cuh"

namespace mscg {

namespace {

__device__ __forceinline__ uint32_t f2ord(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// bounds[0..2] = min (ordered ints), bounds[3..5] = max
__global__ void k_centroid_bounds(const float* __restrict__ v, int n, uint32_t* bounds) {
  float mn[3] = {3.0e38f, 3.0e38f, 3.0e38f}, mx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float c = (v[9 * t + a] + v[9 * t + 3 + a] + v[9 * t + 6 + a]) * (1.0f / 3.0f);
      mn[a] = fminf(mn[a], c);
      mx[a] = fmaxf(mx[a], c);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      atomicMin(&bounds[a], f2ord(mn[a]));
      atomicMax(&bounds[3 + a], f2ord(mx[a]));
    }
  }
}

__device__ __forceinline__ uint32_t morton30(float3 c, float3 lo, float3 sc) {
  uint32_t x = (uint32_t)min(max((int)floorf((c.x - lo.x) * sc.x), 0), 1023);
  uint32_t y = (uint32_t)min(max((int)floorf((c.y - lo.y) * sc.y), 0), 1023);
  uint32_t z = (uint32_t)min(max((int)floorf((c.z - lo.z) * sc.z), 0), 1023);
  return (spread_bits_3(x) << 2) | (spread_bits_3(y) << 1) | spread_bits_3(z);
}

__global__ void k_morton(const float* __restrict__ v, int n, const uint32_t* __restrict__ bounds,
                         uint32_t* __restrict__ codes) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  float3 lo = f3(ord2f(bounds[0]), ord2f(bounds[1]), ord2f(bounds[2]));
  float3 hi = f3(ord2f(bounds[3]), ord2f(bounds[4]), ord2f(bounds[5]));
  float ex = hi.x - lo.x, ey = hi.y - lo.y, ez = hi.z - lo.z;
  float3 sc = f3(ex > 0.f ? 1024.0f / ex : 0.f, ey > 0.f ? 1024.0f / ey : 0.f, ez > 0.f ? 1024.0f / ez : 0.f);
  float3 c;
  c.x = (v[9 * t + 0] + v[9 * t + 3] + v[9 * t + 6]) * (1.0f / 3.0f);
  c.y = (v[9 * t + 1] + v[9 * t + 4] + v[9 * t + 7]) * (1.0f / 3.0f);
  c.z = (v[9 * t + 2] + v[9 * t + 5] + v[9 * t + 8]) * (1.0f / 3.0f);
  codes[t] = morton30(c, lo, sc);
}

__device__ __forceinline__ int lcp(const uint32_t* __restrict__ codes, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  uint32_t a = codes[i], b = codes[j];
  if (a == b) return 32 + __clz((uint32_t)(i ^ j));
  return __clz(a ^ b);
}

// parent[] holds the parents of internal nodes [0, n-1) then of leaves [n-1, 2n-1).
__global__ void k_karras(const uint32_t* __restrict__ codes, int n, int2* __restrict__ children,
                         int* __restrict__ parent) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int d = (lcp(codes, n, i, i + 1) - lcp(codes, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = lcp(codes, n, i, i - d);
  int lmax = 2;
  while (lcp(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (lcp(codes, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = lcp(codes, n, i, j);
  int s = 0;
  int t = l;
  do {
    t = (t + 1) >> 1;
    if (lcp(codes, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  int gamma = i + s * d + min(d, 0);
  int left = (min(i, j) == gamma) ? ~gamma : gamma;
  int right = (max(i, j) == gamma + 1) ? ~(gamma + 1) : gamma + 1;
  children[i] = make_int2(left, right);
  parent[left >= 0 ? left : (n - 1) + ~left] = i;
  parent[right >= 0 ? right : (n - 1) + ~right] = i;
  if (i == 0) parent[0] = -1;
}

// Leaf k holds triangle order[k]; writes the traversal triangle record and the leaf box.
__global__ void k_leaves(const float* __restrict__ v, const int* __restrict__ geom, const uint8_t* __restrict__ is_light,
                         const uint32_t* __restrict__ order, int n, float4* __restrict__ tris, int* __restrict__ tri_orig,
                         float4* __restrict__ leaf_box) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int t = (int)order[k];
  float3 v0 = f3(v[9 * t + 0], v[9 * t + 1], v[9 * t + 2]);
  float3 v1 = f3(v[9 * t + 3], v[9 * t + 4], v[9 * t + 5]);
  float3 v2 = f3(v[9 * t + 6], v[9 * t + 7], v[9 * t + 8]);
  float3 e1 = v_sub(v1, v0), e2 = v_sub(v2, v0);
  tris[3 * k + 0] = make_float4(v0.x, v0.y, v0.z, __int_as_float(geom[t]));
  tris[3 * k + 1] = make_float4(e1.x, e1.y, e1.z, __int_as_float((int)is_light[t]));
  tris[3 * k + 2] = make_float4(e2.x, e2.y, e2.z, __int_as_float(t));
  tri_orig[k] = t;
  leaf_box[2 * k + 0] = make_float4(fminf(fminf(v0.x, v1.x), v2.x), fminf(fminf(v0.y, v1.y), v2.y),
                                    fminf(fminf(v0.z, v1.z), v2.z), 0.f);
  leaf_box[2 * k + 1] = make_float4(fmaxf(fmaxf(v0.x, v1.x), v2.x), fmaxf(fmaxf(v0.y, v1.y), v2.y),
                                    fmaxf(fmaxf(v0.z, v1.z), v2.z), 0.f);
}

__device__ __forceinline__ void load_box(int c, const float4* leaf_box, const float4* node_box, float4* lo, float4* hi) {
  if (c < 0) {
    *lo = leaf_box[2 * (~c) + 0];
    *hi = leaf_box[2 * (~c) + 1];
  } else {
    *lo = __ldcg(&node_box[2 * c + 0]);
    *hi = __ldcg(&node_box[2 * c + 1]);
  }
}

// One thread per leaf; the second thread to reach a node builds its box and
// continues upward.  No thread waits on another.
__global__ void k_refit(const int2* __restrict__ children, const int* __restrict__ parent, int n,
                        const float4* __restrict__ leaf_box, float4* node_box, int* flags, int* err) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int p = parent[(n - 1) + k];
  int level = 0;
  while (p >= 0) {
    if (++level > n) {  // a parent chain longer than the tree can only come from a malformed hierarchy
      atomicOr(err, 1);
      return;
    }
    __threadfence();
    if (atomicAdd(&flags[p], 1) == 0) return;
    __threadfence();
    int2 ch = children[p];
    float4 l0, h0, l1, h1;
    load_box(ch.x, leaf_box, node_box, &l0, &h0);
    load_box(ch.y, leaf_box, node_box, &l1, &h1);
    float4 lo = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.f);
    float4 hi = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.f);
    __stcg(&node_box[2 * p + 0], lo);
    __stcg(&node_box[2 * p + 1], hi);
    p = parent[p];
  }
}

// ------------------------------------------------------------ treelet restructuring
// Karras and Aila, "Fast Parallel Construction of High-Quality Bounding Volume
// Hierarchies" (HPG 2013): bottom-up over the LBVH, every node with at least
// 7 leaves below roots a treelet of 7 leaves (grown by opening the treelet leaf
// of largest surface area); the SAH-optimal binary tree over those 7 leaves is
// found by dynamic programming over their 127 subsets and replaces the
// treelet when it is cheaper, reusing the treelet's 6 internal nodes.  One
// thread per treelet; a round is one bottom-up pass.
constexpr int kTreeletRounds = 6;
constexpr float kCostNode = 1.2f;  // SAH cost of a node visit relative to a triangle test
constexpr float kCostTri = 1.0f;

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
  const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
  return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ void box_of(int c, const float4* leaf_box, const float4* node_box, float4* lo, float4* hi) {
  if (c < 0) {
    *lo = __ldcg(&leaf_box[2 * (~c) + 0]);
    *hi = __ldcg(&leaf_box[2 * (~c) + 1]);
  } else {
    *lo = __ldcg(&node_box[2 * c + 0]);
    *hi = __ldcg(&node_box[2 * c + 1]);
  }
}

__global__ void k_treelet(int2* children, int* parent, int n, const float4* __restrict__ leaf_box, float4* node_box,
                          float* cost, int* leaves, int* flags, int* err) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int p = parent[(n - 1) + k];
  int level = 0;
  float s_area[128], s_cost[128];
  uint8_t s_best[128];
  while (p >= 0) {
    if (++level > n) {
      atomicOr(err, 1);
      return;
    }
    __threadfence();
    if (atomicAdd(&flags[p], 1) == 0) return;
    __threadfence();
    const int2 ch = __ldcg(&children[p]);
    float4 l0, h0, l1, h1;
    box_of(ch.x, leaf_box, node_box, &l0, &h0);
    box_of(ch.y, leaf_box, node_box, &l1, &h1);
    const float4 lo = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.f);
    const float4 hi = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.f);
    const int nl = (ch.x < 0 ? 1 : __ldcg(&leaves[ch.x])) + (ch.y < 0 ? 1 : __ldcg(&leaves[ch.y]));
    const float cl = ch.x < 0 ? kCostTri * half_area(l0, h0) : __ldcg(&cost[ch.x]);
    const float cr = ch.y < 0 ? kCostTri * half_area(l1, h1) : __ldcg(&cost[ch.y]);
    float cp = kCostNode * half_area(lo, hi) + cl + cr;
    if (nl >= 7) {
      // grow the treelet: open the internal treelet leaf of largest area until 7 leaves
      int tl[7], inner[6];
      tl[0] = ch.x;
      tl[1] = ch.y;
      int ntl = 2, ninner = 0;
      while (ntl < 7) {
        int bi = -1;
        float ba = -1.f;
        for (int i = 0; i < ntl; ++i) {
          if (tl[i] < 0) continue;
          float4 a, b;
          box_of(tl[i], leaf_box, node_box, &a, &b);
          const float ar = half_area(a, b);
          if (ar > ba) { ba = ar; bi = i; }
        }
        if (bi < 0) break;
        const int2 c2 = __ldcg(&children[tl[bi]]);
        inner[ninner++] = tl[bi];
        tl[bi] = c2.x;
        tl[ntl++] = c2.y;
      }
      if (ntl == 7) {
        // subset areas and optimal costs
        for (int S = 1; S < 128; ++S) {
          float4 a = make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.f), b = make_float4(-3.0e38f, -3.0e38f, -3.0e38f, 0.f);
          for (int i = 0; i < 7; ++i) {
            if (!((S >> i) & 1)) continue;
            float4 x, y;
            box_of(tl[i], leaf_box, node_box, &x, &y);
            a = make_float4(fminf(a.x, x.x), fminf(a.y, x.y), fminf(a.z, x.z), 0.f);
            b = make_float4(fmaxf(b.x, y.x), fmaxf(b.y, y.y), fmaxf(b.z, y.z), 0.f);
          }
          s_area[S] = half_area(a, b);
        }
        for (int i = 0; i < 7; ++i) {
          const int S = 1 << i;
          s_cost[S] = tl[i] < 0 ? kCostTri * s_area[S] : __ldcg(&cost[tl[i]]);
          s_best[S] = 0;
        }
        for (int S = 1; S < 128; ++S) {
          if ((S & (S - 1)) == 0) continue;
          const int low = S & -S;
          float best = 3.0e38f;
          int bp = 0;
          // partitions (P, S \ P) with the lowest element in P
          const int rest = S ^ low;
          for (int Q = rest;; Q = (Q - 1) & rest) {
            const int P = low | Q;
            if (P != S) {
              const float c = s_cost[P] + s_cost[S ^ P];
              if (c < best) { best = c; bp = P; }
            }
            if (Q == 0) break;
          }
          s_cost[S] = kCostNode * s_area[S] + best;
          s_best[S] = (uint8_t)bp;
        }
        if (s_cost[127] < cp * 0.9999f) {
          // rebuild: subsets in creation order, the treelet root keeps node p
          int sets[6], ids[6], nsets = 1, next = 0;
          sets[0] = 127;
          ids[0] = p;
          for (int q = 0; q < nsets; ++q) {
            const int S = sets[q], P = s_best[S];
            int cid[2];
            const int part[2] = {P, S ^ P};
            for (int h = 0; h < 2; ++h) {
              const int X = part[h];
              if ((X & (X - 1)) == 0) {
                cid[h] = tl[__ffs(X) - 1];
              } else {
                cid[h] = inner[next++];
                sets[nsets] = X;
                ids[nsets] = cid[h];
                ++nsets;
              }
              const int c = cid[h];
              if (c < 0) parent[(n - 1) + ~c] = ids[q];
              else parent[c] = ids[q];
            }
            __stcg(&children[ids[q]], make_int2(cid[0], cid[1]));
          }
          // boxes, costs and leaf counts bottom-up (children were created after their parents)
          for (int q = nsets - 1; q >= 0; --q) {
            const int id = ids[q];
            const int2 cc = __ldcg(&children[id]);
            float4 a0, b0, a1, b1;
            box_of(cc.x, leaf_box, node_box, &a0, &b0);
            box_of(cc.y, leaf_box, node_box, &a1, &b1);
            const float4 bl = make_float4(fminf(a0.x, a1.x), fminf(a0.y, a1.y), fminf(a0.z, a1.z), 0.f);
            const float4 bh = make_float4(fmaxf(b0.x, b1.x), fmaxf(b0.y, b1.y), fmaxf(b0.z, b1.z), 0.f);
            __stcg(&node_box[2 * id + 0], bl);
            __stcg(&node_box[2 * id + 1], bh);
            __stcg(&cost[id], s_cost[sets[q]]);
            __stcg(&leaves[id], __popc(sets[q]) == 7 ? nl : (cc.x < 0 ? 1 : __ldcg(&leaves[cc.x])) +
                                                               (cc.y < 0 ? 1 : __ldcg(&leaves[cc.y])));
          }
          cp = s_cost[127];
        }
      }
    }
    __stcg(&node_box[2 * p + 0], lo);  // a restructured treelet keeps its leaf set, so its box
    __stcg(&node_box[2 * p + 1], hi);
    __stcg(&cost[p], cp);
    __stcg(&leaves[p], nl);
    p = __ldcg(&parent[p]);
  }
}

__global__ void k_pack(const int2* __restrict__ children, int n, const float4* __restrict__ leaf_box,
                       const float4* __restrict__ node_box, float4* __restrict__ nodes) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int2 ch = children[i];
  float4 l0, h0, l1, h1;
  load_box(ch.x, leaf_box, node_box, &l0, &h0);
  load_box(ch.y, leaf_box, node_box, &l1, &h1);
  nodes[4 * i + 0] = make_float4(l0.x, h0.x, l0.y, h0.y);
  nodes[4 * i + 1] = make_float4(l1.x, h1.x, l1.y, h1.y);
  nodes[4 * i + 2] = make_float4(l0.z, h0.z, l1.z, h1.z);
  nodes[4 * i + 3] = make_float4(__int_as_float(ch.x), __int_as_float(ch.y), 0.f, 0.f);
}

// Scene bounds of all vertices (used to place direction-only tests and for stats).
__global__ void k_scene_bounds(const float4* __restrict__ node_box, float* out) {
  out[0] = node_box[0].x; out[1] = node_box[0].y; out[2] = node_box[0].z;
  out[3] = node_box[1].x; out[4] = node_box[1].y; out[5] = node_box[1].z;
}

size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

// ------------------------------------------------------------------ 8-wide collapse
// The binary LBVH is collapsed top-down: a wide node starts from the two
// children of a binary node and repeatedly opens the child with the largest
// surface area until it has 8 children or none is left to open.  A binary
// subtree of at most kWideLeafMax triangles becomes one leaf child; its
// triangles are re-emitted so that a node's leaf triangles are contiguous
// from the node's triangle base.  Child boxes are quantised to 8 bits per
// axis against the node box with power-of-two steps, rounded outward so the
// decoded box always contains the child.  Children are placed in slots by
// direction octant (Ylitie, Karras and Laine, "Efficient Incoherent Ray
// Traversal on GPUs Through Compressed Wide BVHs", HPG 2017): slot s prefers
// the child that lies farthest back along the octant-s direction, so a ray of
// octant o that visits slots o ^ 0, o ^ 1, ..., o ^ 7 meets the children
// roughly front to back without sorting them.
constexpr int kWideLeafMax = 2;
// SAH weights of the collapse: a wide-node visit (eight box tests), and one
// triangle test relative to it (0.6 measured best of 0.15, 0.3 and 0.6).
constexpr float kCollapseNode = 1.0f;
constexpr float kCollapseTri = 0.6f;
// slot s of a node owns the two triangle bits 2s, 2s + 1 (the traversal
// spreads its 8-bit leaf-hit mask onto them)
static_assert(kWideLeafMax <= 2, "a leaf slot owns two triangle bits");

struct WideBuild {
  std::vector<uint32_t> words;  // 20 words per node
  std::vector<int> tri_perm;    // new triangle order -> leaf index of the binary tree
};

float surface(const float4& lo, const float4& hi) {
  float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
  return dx * dy + dy * dz + dz * dx;
}

void quantise_axis(float lo, float hi, int* e_out, float* scale_out) {
  double ext = (double)hi - (double)lo;
  int e = -126;
  if (ext > 0.0) {
    e = (int)std::ceil(std::log2(ext / 255.0));
    while (std::ldexp(255.0, e) < ext) ++e;
    if (e < -126) e = -126;
    if (e > 127) e = 127;
  }
  *e_out = e;
  *scale_out = (float)std::ldexp(1.0, e);
}

uint32_t q_lo(float p, float s, float v) {
  double q = std::floor(((double)v - (double)p) / (double)s);
  int qi = (int)std::max(0.0, std::min(255.0, q));
  while (qi > 0 && std::fma((float)qi, s, p) > v) --qi;
  return (uint32_t)qi;
}

uint32_t q_hi(float p, float s, float v) {
  double q = std::ceil(((double)v - (double)p) / (double)s);
  int qi = (int)std::max(0.0, std::min(255.0, q));
  while (qi < 255 && std::fma((float)qi, s, p) < v) ++qi;
  return (uint32_t)qi;
}

void collapse_wide(int n, const std::vector<int2>& ch, const std::vector<float4>& nbox, const std::vector<float4>& lbox,
                   WideBuild* out) {
  // leaf count of every internal node, children before parents
  std::vector<int> count(n - 1), bfs;
  bfs.reserve(n - 1);
  bfs.push_back(0);
  for (size_t i = 0; i < bfs.size(); ++i) {
    int2 c = ch[bfs[i]];
    if (c.x >= 0) bfs.push_back(c.x);
    if (c.y >= 0) bfs.push_back(c.y);
  }
  for (size_t i = bfs.size(); i-- > 0;) {
    int b = bfs[i];
    int2 c = ch[b];
    const int cl = c.x < 0 ? 1 : count[c.x], cr = c.y < 0 ? 1 : count[c.y];
    count[b] = cl + cr;
  }
  auto box_lo = [&](int c) { return c < 0 ? lbox[2 * (~c)] : nbox[2 * c]; };
  auto box_hi = [&](int c) { return c < 0 ? lbox[2 * (~c) + 1] : nbox[2 * c + 1]; };
  // SAH-optimal collapse (Ylitie, Karras and Laine, HPG 2017), children before
  // parents: cost[b][i-1] is the least SAH cost of covering b's subtree with at
  // most i roots, each a leaf slot (at most kWideLeafMax triangles) or a wide
  // node; split[b][i-1] is the number of roots the left child gets in the best
  // split into exactly i (0: fewer roots are cheaper); leaf[b] marks a subtree
  // that is cheapest as one leaf slot.
  std::vector<std::array<float, 8>> cost((size_t)(n - 1));
  std::vector<std::array<uint8_t, 8>> split((size_t)(n - 1));
  std::vector<uint8_t> leaf((size_t)(n - 1), 0);
  auto child_cost = [&](int c, int i) {  // a triangle is one leaf slot at any i
    if (c < 0) {
      const float4 lo = lbox[2 * (~c)], hi = lbox[2 * (~c) + 1];
      return kCollapseTri * surface(lo, hi);
    }
    return cost[c][i - 1];
  };
  for (size_t q = bfs.size(); q-- > 0;) {
    const int b = bfs[q];
    const int l = ch[b].x, r = ch[b].y;
    float dist[9];
    int dsplit[9];
    for (int j = 2; j <= 8; ++j) {
      dist[j] = std::numeric_limits<float>::infinity();
      dsplit[j] = 1;
      for (int k = 1; k < j; ++k) {
        const float c = child_cost(l, k) + child_cost(r, j - k);
        if (c < dist[j]) { dist[j] = c; dsplit[j] = k; }
      }
    }
    const float area = surface(nbox[2 * b], nbox[2 * b + 1]);
    float best_dist = dist[2];
    for (int j = 3; j <= 8; ++j) best_dist = std::min(best_dist, dist[j]);
    const float c_int = kCollapseNode * area + best_dist;
    const float c_leaf = count[b] <= kWideLeafMax ? kCollapseTri * area * (float)count[b]
                                                   : std::numeric_limits<float>::infinity();
    leaf[b] = c_leaf <= c_int ? 1 : 0;
    cost[b][0] = std::min(c_leaf, c_int);
    split[b][0] = 0;
    for (int i = 2; i <= 8; ++i) {
      if (dist[i] < cost[b][i - 2]) {
        cost[b][i - 1] = dist[i];
        split[b][i - 1] = (uint8_t)dsplit[i];
      } else {
        cost[b][i - 1] = cost[b][i - 2];
        split[b][i - 1] = 0;
      }
    }
  }
  // the roots covering subtree c with at most i of them, per the decisions
  std::function<void(int, int, int*, int*)> roots = [&](int c, int i, int* C, int* k) {
    if (c < 0 || i == 1) {
      C[(*k)++] = c;
      return;
    }
    while (i > 1 && split[c][i - 1] == 0) --i;
    if (i == 1) {
      C[(*k)++] = c;
      return;
    }
    const int kl = split[c][i - 1];
    roots(ch[c].x, kl, C, k);
    roots(ch[c].y, i - kl, C, k);
  };
  auto is_leafish = [&](int c) { return c < 0 || leaf[c] != 0; };
  out->words.clear();
  out->tri_perm.clear();
  out->tri_perm.reserve(n);
  std::vector<int> queue;  // binary node of each wide node, in wide-node order
  queue.push_back(0);
  out->words.resize(20);
  for (size_t w = 0; w < queue.size(); ++w) {
    const int b = queue[w];
    int C[8];
    int k = 0;
    {  // the best split of b into 2..8 roots
      const int l = ch[b].x, r = ch[b].y;
      float best = std::numeric_limits<float>::infinity();
      int bj = 2, bk = 1;
      for (int j = 2; j <= 8; ++j)
        for (int kk = 1; kk < j; ++kk) {
          const float c = child_cost(l, kk) + child_cost(r, j - kk);
          if (c < best) { best = c; bj = j; bk = kk; }
        }
      roots(l, bk, C, &k);
      roots(r, bj - bk, C, &k);
    }
    const float4 lo = nbox[2 * b], hi = nbox[2 * b + 1];
    // octant slots: greedy assignment of (child, slot) pairs by increasing
    // projection of the child's centre offset on the slot's direction
    bool filled[8] = {false, false, false, false, false, false, false, false};
    {
      float cost[8][8];
      const float ncx = 0.5f * (lo.x + hi.x), ncy = 0.5f * (lo.y + hi.y), ncz = 0.5f * (lo.z + hi.z);
      for (int i = 0; i < k; ++i) {
        const float4 cl = box_lo(C[i]), chh = box_hi(C[i]);
        const float ox = 0.5f * (cl.x + chh.x) - ncx, oy = 0.5f * (cl.y + chh.y) - ncy, oz = 0.5f * (cl.z + chh.z) - ncz;
        for (int sl = 0; sl < 8; ++sl)
          cost[i][sl] = ((sl & 1) ? -ox : ox) + ((sl & 2) ? -oy : oy) + ((sl & 4) ? -oz : oz);
      }
      int slot_child[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      bool used[8] = {false, false, false, false, false, false, false, false};
      for (int round = 0; round < k; ++round) {
        int bi = -1, bs = -1;
        float bc = 0.f;
        for (int i = 0; i < k; ++i) {
          if (used[i]) continue;
          for (int sl = 0; sl < 8; ++sl)
            if (!filled[sl] && (bi < 0 || cost[i][sl] < bc)) { bi = i; bs = sl; bc = cost[i][sl]; }
        }
        used[bi] = true;
        filled[bs] = true;
        slot_child[bs] = C[bi];
      }
      for (int sl = 0; sl < 8; ++sl) C[sl] = slot_child[sl];
      k = 8;
    }
    int e[3];
    float s[3];
    quantise_axis(lo.x, hi.x, &e[0], &s[0]);
    quantise_axis(lo.y, hi.y, &e[1], &s[1]);
    quantise_axis(lo.z, hi.z, &e[2], &s[2]);
    uint32_t imask = 0, valid = 0, q[6][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
    const uint32_t child_base = (uint32_t)queue.size();
    const uint32_t tri_base = (uint32_t)out->tri_perm.size();
    for (int i = 0; i < k; ++i) {
      const int c = C[i];
      if (!filled[i]) continue;  // an empty slot
      if (is_leafish(c)) {
        // the subtree's leaves (restructured treelets need not hold a
        // contiguous leaf range, so they are collected by a walk)
        int walk[2 * kWideLeafMax], nw = 0, cnt = 0;
        walk[nw++] = c;
        while (nw > 0) {
          const int x = walk[--nw];
          if (x < 0) {
            out->tri_perm.push_back(~x);
            ++cnt;
          } else {
            walk[nw++] = ch[x].y;
            walk[nw++] = ch[x].x;
          }
        }
        // slot i owns triangle bits 2i and 2i + 1; the triangles themselves
        // are stored in slot order, so a bit's triangle is the count of
        // valid bits below it past the node's triangle base
        valid |= ((1u << cnt) - 1u) << (2 * i);
      } else {
        imask |= 1u << i;
        queue.push_back(c);
      }
      const float4 cl = box_lo(c), chh = box_hi(c);
      const float cll[3] = {cl.x, cl.y, cl.z}, chl[3] = {chh.x, chh.y, chh.z}, pl[3] = {lo.x, lo.y, lo.z};
      for (int a = 0; a < 3; ++a) {
        q[a][i >> 2] |= q_lo(pl[a], s[a], cll[a]) << (8 * (i & 3));
        q[3 + a][i >> 2] |= q_hi(pl[a], s[a], chl[a]) << (8 * (i & 3));
      }
    }
    out->words.resize(20 * queue.size());
    uint32_t* W = &out->words[20 * w];
    memcpy(&W[0], &lo.x, 4);
    memcpy(&W[1], &lo.y, 4);
    memcpy(&W[2], &lo.z, 4);
    W[3] = (uint32_t)(e[0] + 127) | ((uint32_t)(e[1] + 127) << 8) | ((uint32_t)(e[2] + 127) << 16) | (imask << 24);
    W[4] = child_base;
    W[5] = tri_base;
    W[6] = valid;
    W[7] = 0;
    // q_lo x, y, z then q_hi x, y, z, two words (slots 0-3, 4-7) each
    for (int a = 0; a < 6; ++a) {
      W[8 + 2 * a] = q[a][0];
      W[9 + 2 * a] = q[a][1];
    }
  }
}

}  // namespace

int bvh_build(const float* d_v, const int* d_geom, const uint8_t* d_light, int n, bool wide, DeviceBvh* out,
              cudaStream_t stream, std::string* err) {
  if (n < 2) { *err = "the BVH needs at least two triangles"; return -1; }
  int launches = 0;
  out->num_tris = n;
  out->num_nodes = n - 1;
  // persistent buffers
  if (cudaMalloc(&out->nodes, (size_t)(n - 1) * 4 * sizeof(float4)) != cudaSuccess ||
      cudaMalloc(&out->tris, (size_t)n * 3 * sizeof(float4)) != cudaSuccess ||
      cudaMalloc(&out->tri_orig, (size_t)n * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&out->bounds_dev, 8 * sizeof(float)) != cudaSuccess) {
    *err = "out of device memory for the BVH";
    return -1;
  }
  // build scratch
  size_t bytes = al(6 * 4) + al((size_t)n * 4) * 2 + al((size_t)(n - 1) * sizeof(int2)) + al((size_t)(2 * n) * 4) +
                 al((size_t)n * 2 * sizeof(float4)) + al((size_t)(n - 1) * 2 * sizeof(float4)) + 3 * al((size_t)n * 4) +
                 sort_scratch_bytes(n);
  char* scratch = nullptr;
  if (cudaMalloc(&scratch, bytes) != cudaSuccess) { *err = "out of device memory for the BVH build"; return -1; }
  char* p = scratch;
  uint32_t* bounds = (uint32_t*)p; p += al(6 * 4);
  uint32_t* codes = (uint32_t*)p; p += al((size_t)n * 4);
  uint32_t* order = (uint32_t*)p; p += al((size_t)n * 4);
  int2* children = (int2*)p; p += al((size_t)(n - 1) * sizeof(int2));
  int* parent = (int*)p; p += al((size_t)(2 * n) * 4);
  float4* leaf_box = (float4*)p; p += al((size_t)n * 2 * sizeof(float4));
  float4* node_box = (float4*)p; p += al((size_t)(n - 1) * 2 * sizeof(float4));
  int* flags = (int*)p; p += al((size_t)n * 4);
  float* tcost = (float*)p; p += al((size_t)n * 4);
  int* tleaves = (int*)p; p += al((size_t)n * 4);
  SortScratch ss;
  sort_scratch_bind(&ss, p, n);

  cudaMemsetAsync(bounds, 0xff, 12, stream);
  cudaMemsetAsync(bounds + 3, 0x00, 20, stream);  // max words and the error word bounds[7]
  cudaMemsetAsync(flags, 0, (size_t)n * 4, stream);
  const int tb = 256;
  const int g = (n + tb - 1) / tb;
  k_centroid_bounds<<<min(g, 1024), tb, 0, stream>>>(d_v, n, bounds);
  k_morton<<<g, tb, 0, stream>>>(d_v, n, bounds, codes);
  launches += 2;
  launches += sort_pairs(codes, nullptr, codes, order, n, 30, ss, stream);
  k_karras<<<(n - 1 + tb - 1) / tb, tb, 0, stream>>>(codes, n, children, parent);
  k_leaves<<<g, tb, 0, stream>>>(d_v, d_geom, d_light, order, n, out->tris, out->tri_orig, leaf_box);
  k_refit<<<g, tb, 0, stream>>>(children, parent, n, leaf_box, node_box, flags, (int*)(bounds + 7));
  for (int round = 0; round < kTreeletRounds && n >= 7; ++round) {
    cudaMemsetAsync(flags, 0, (size_t)n * 4, stream);
    k_treelet<<<g, tb, 0, stream>>>(children, parent, n, leaf_box, node_box, tcost, tleaves, flags,
                                    (int*)(bounds + 7));
    ++launches;
  }
  k_pack<<<(n - 1 + tb - 1) / tb, tb, 0, stream>>>(children, n, leaf_box, node_box, out->nodes);
  k_scene_bounds<<<1, 1, 0, stream>>>(node_box, out->bounds_dev);
  launches += 5;
  int refit_err = 0;
  cudaMemcpyAsync(&refit_err, bounds + 7, 4, cudaMemcpyDeviceToHost, stream);
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) {
    cudaFree(scratch);
    *err = std::string("BVH build failed: ") + cudaGetErrorString(e);
    return -1;
  }
  if (refit_err != 0) {
    cudaFree(scratch);
    *err = "BVH build produced a malformed hierarchy";
    return -1;
  }
  if (wide) {
    std::vector<int2> h_ch((size_t)(n - 1));
    std::vector<float4> h_nb((size_t)(n - 1) * 2), h_lb((size_t)n * 2), h_tris((size_t)n * 3);
    std::vector<int> h_orig((size_t)n);
    bool ok = cudaMemcpy(h_ch.data(), children, h_ch.size() * sizeof(int2), cudaMemcpyDeviceToHost) == cudaSuccess &&
              cudaMemcpy(h_nb.data(), node_box, h_nb.size() * sizeof(float4), cudaMemcpyDeviceToHost) == cudaSuccess &&
              cudaMemcpy(h_lb.data(), leaf_box, h_lb.size() * sizeof(float4), cudaMemcpyDeviceToHost) == cudaSuccess &&
              cudaMemcpy(h_tris.data(), out->tris, h_tris.size() * sizeof(float4), cudaMemcpyDeviceToHost) ==
                  cudaSuccess &&
              cudaMemcpy(h_orig.data(), out->tri_orig, h_orig.size() * sizeof(int), cudaMemcpyDeviceToHost) ==
                  cudaSuccess;
    cudaFree(scratch);
    if (!ok) { *err = "BVH collapse: device copy failed"; return -1; }
    WideBuild wb;
    collapse_wide(n, h_ch, h_nb, h_lb, &wb);
    if ((int)wb.tri_perm.size() != n) { *err = "BVH collapse lost triangles"; return -1; }
    std::vector<float4> p_tris((size_t)n * 3);
    std::vector<int> p_orig((size_t)n);
    for (int i = 0; i < n; ++i) {
      const int s = wb.tri_perm[i];
      p_tris[3 * i + 0] = h_tris[3 * s + 0];
      p_tris[3 * i + 1] = h_tris[3 * s + 1];
      p_tris[3 * i + 2] = h_tris[3 * s + 2];
      p_orig[i] = h_orig[s];
    }
    out->num_wnodes = (int)(wb.words.size() / 20);
    if (cudaMalloc(&out->wnodes, wb.words.size() * 4) != cudaSuccess ||
        cudaMemcpy(out->wnodes, wb.words.data(), wb.words.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(out->tris, p_tris.data(), p_tris.size() * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(out->tri_orig, p_orig.data(), p_orig.size() * sizeof(int), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
      *err = "out of device memory for the wide BVH";
      return -1;
    }
    cudaFree(out->nodes);  // the binary nodes are not traversed in the wide form
    out->nodes = nullptr;
    return launches;
  }
  cudaFree(scratch);
  return launches;
}

void bvh_free(DeviceBvh* b) {
  if (b->nodes) cudaFree(b->nodes);
  if (b->wnodes) cudaFree(b->wnodes);
  b->wnodes = nullptr;
  if (b->tris) cudaFree(b->tris);
  if (b->tri_orig) cudaFree(b->tri_orig);
  if (b->bounds_dev) cudaFree(b->bounds_dev);
  b->bounds_dev = nullptr;
  b->nodes = nullptr;
  b->tris = nullptr;
  b->tri_orig = nullptr;
}

}  // namespace mscg
