// CPU oracle of the sorted deferred-shading path tracer - TEST INFRASTRUCTURE
// (see oracle.h).  Restates, per path and without batching, the reference's
//   camera      src/core/Camera.cpp:6-59, src/core/StratifiedSampler.cpp:5-17,
//               src/core/PinHoleCamera.cpp:5-32, src/core/ThinLensCamera.cpp:5-56
//   integrator  src/core/Integrator.cpp:12-255 (emission, NEE, Russian roulette)
//   shaders     src/core/LambertShader.cpp:22-73, src/core/NullShader.cpp:25-54
//   light       src/core/QuadLight.cpp:5-84
//   filter      src/core/TentFilter.cpp:5-63, src/core/BoxFilter.cpp:5-37
//   scene input src/core/Pathtracer.cpp:32-275, src/core/PolygonObject.cpp:5-43,
//               thirdparty/tinyobjloader/tiny_obj_loader.cpp:131-242,309-412,643-891
//   bins        src/core/Camera.cpp:42-44, src/core/DirectionalBins.cpp:37-73
// with a per-path counter-based random sequence in place of the reference's
// per-thread mt19937 (whose per-path order depends on TBB scheduling and
// cannot be reproduced), and its own SAH BVH in place of Embree.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace orc {

const float kPi = 3.14159265358979323846f;
const float kInvPi = 0.31830988618379067154f;
const float kPi180 = 0.01745329251994329577f;
const float kEps = 1.1920928955078125e-07f;
const float kTnear = 0.001f;
const float kTfar = 100000.f;

// ------------------------------------------------------------ random draws
// 4-lane PCG hash (Jarzynski & Olano, JCGT 2020): key (sampleID, slot, iteration seed, lane).
struct U4 { uint32_t x, y, z, w; };
U4 pcg4d(uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
  x = x * 1664525u + 1013904223u;
  y = y * 1664525u + 1013904223u;
  z = z * 1664525u + 1013904223u;
  w = w * 1664525u + 1013904223u;
  x += y * w; y += z * x; z += x * y; w += y * z;
  x ^= x >> 16; y ^= y >> 16; z ^= z >> 16; w ^= w >> 16;
  x += y * w; y += z * x; z += x * y; w += y * z;
  return {x, y, z, w};
}
float u01(uint32_t v) { return (float)(v >> 8) * 5.9604644775390625e-08f; }
uint32_t iter_seed(uint32_t seed, uint32_t it) { return seed * 0x85ebca6bu ^ (it * 0xc2b2ae35u + 0x27d4eb2fu); }

// ------------------------------------------------------------ arithmetic
template <class T> struct V { T x, y, z; };
template <class T> V<T> mk(T x, T y, T z) { return V<T>{x, y, z}; }
template <class T> V<T> add(V<T> a, V<T> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> V<T> sub(V<T> a, V<T> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> V<T> mul(V<T> a, T s) { return mk(a.x * s, a.y * s, a.z * s); }
template <class T> V<T> neg(V<T> a) { return mk(-a.x, -a.y, -a.z); }
template <class T> T dot(V<T> a, V<T> b) { return std::fma(a.z, b.z, std::fma(a.y, b.y, a.x * b.x)); }
template <class T> V<T> cross(V<T> a, V<T> b) {
  return mk(std::fma(a.y, b.z, -(a.z * b.y)), std::fma(a.z, b.x, -(a.x * b.z)), std::fma(a.x, b.y, -(a.y * b.x)));
}
template <class T> V<T> normalize(V<T> a) { T inv = T(1) / std::sqrt(dot(a, a)); return mul(a, inv); }
template <class T> T len(V<T> a) { return std::sqrt(dot(a, a)); }
template <class T> T maxc(V<T> a) { return std::max(std::max(a.x, a.y), a.z); }

struct Aff { float m[3][4]; };
template <class T> V<T> xf(const Aff& a, V<T> p) {
  T r[3];
  for (int i = 0; i < 3; ++i)
    r[i] = std::fma((T)a.m[i][2], p.z, std::fma((T)a.m[i][1], p.y, (T)a.m[i][0] * p.x)) + (T)a.m[i][3];
  return mk(r[0], r[1], r[2]);
}

// sin/cos of 2*pi*t.  float: quadrant split plus Taylor polynomials in the
// fixed Horner order of the device code; double: the library functions.
void sincos_turns(float t, float* s, float* c) {
  float q = t * 4.0f;
  int k = (int)q;
  if (k < 0) k = 0;
  if (k > 3) k = 3;
  float r = t - (float)k * 0.25f;
  float x = r * 6.28318530717958647692f;
  float x2 = x * x;
  float ps = 1.0f - x2 * (1.0f / 156.0f);
  ps = 1.0f - x2 * (1.0f / 110.0f) * ps;
  ps = 1.0f - x2 * (1.0f / 72.0f) * ps;
  ps = 1.0f - x2 * (1.0f / 42.0f) * ps;
  ps = 1.0f - x2 * (1.0f / 20.0f) * ps;
  ps = 1.0f - x2 * (1.0f / 6.0f) * ps;
  float sn = x * ps;
  float pc = 1.0f - x2 * (1.0f / 182.0f);
  pc = 1.0f - x2 * (1.0f / 132.0f) * pc;
  pc = 1.0f - x2 * (1.0f / 90.0f) * pc;
  pc = 1.0f - x2 * (1.0f / 56.0f) * pc;
  pc = 1.0f - x2 * (1.0f / 30.0f) * pc;
  pc = 1.0f - x2 * (1.0f / 12.0f) * pc;
  pc = 1.0f - x2 * (1.0f / 2.0f) * pc;
  float cs = pc;
  if (k == 0) { *s = sn; *c = cs; }
  else if (k == 1) { *s = cs; *c = -sn; }
  else if (k == 2) { *s = -sn; *c = -cs; }
  else { *s = -cs; *c = sn; }
}
void sincos_turns(double t, double* s, double* c) {
  double a = 2.0 * 3.14159265358979323846 * t;
  *s = std::sin(a);
  *c = std::cos(a);
}

float log2_pos(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  int e = (int)((u >> 23) & 0xff) - 127;
  u = (u & 0x007fffffu) | 0x3f800000u;
  float m;
  memcpy(&m, &u, 4);
  if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float p = 1.0f / 11.0f;
  p = p * s2 + 1.0f / 9.0f;
  p = p * s2 + 1.0f / 7.0f;
  p = p * s2 + 1.0f / 5.0f;
  p = p * s2 + 1.0f / 3.0f;
  p = p * s2 + 1.0f;
  return (float)e + s * p * 2.88539008177792681472f;
}
float exp2_f(float x) {
  if (x < -126.0f) return 0.0f;
  if (x > 127.0f) x = 127.0f;
  float kf = std::floor(x + 0.5f);
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
  uint32_t b = (uint32_t)((int)kf + 127) << 23;
  float sc;
  memcpy(&sc, &b, 4);
  return p * sc;
}
float pow_pos(float x, float y) { return x <= 0.0f ? 0.0f : exp2_f(y * log2_pos(x)); }
double pow_pos(double x, double y) { return x <= 0.0 ? 0.0 : std::pow(x, y); }

int cardinal(float dx, float dy, float dz) {  // Camera.cpp:42-44
  float d[3] = {dx, dy, dz};
  int m = (std::fabs(d[0]) < std::fabs(d[1])) ? 1 : 0;
  int axis = (std::fabs(d[m]) < std::fabs(d[2])) ? 2 : m;
  return (d[axis] < 0.f) ? axis : axis + 3;
}

// ------------------------------------------------------------ YAML subset
struct Node {
  int kind = 0;  // 0 null, 1 scalar, 2 seq, 3 map
  std::string s;
  std::vector<Node> seq;
  std::vector<std::pair<std::string, Node>> map;
  const Node* get(const std::string& k) const {
    for (auto& kv : map)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
  size_t size() const { return kind == 3 ? map.size() : seq.size(); }
};

std::string trim(std::string s) {
  size_t b = s.find_first_not_of(" \t\r");
  if (b == std::string::npos) return "";
  size_t e = s.find_last_not_of(" \t\r");
  return s.substr(b, e - b + 1);
}

bool parse_flow(const std::string& s, size_t& p, Node* out) {
  while (p < s.size() && s[p] == ' ') ++p;
  if (p < s.size() && s[p] == '[') {
    ++p;
    out->kind = 2;
    while (true) {
      while (p < s.size() && s[p] == ' ') ++p;
      if (p < s.size() && s[p] == ']') { ++p; return true; }
      Node it;
      if (!parse_flow(s, p, &it)) return false;
      out->seq.push_back(it);
      while (p < s.size() && s[p] == ' ') ++p;
      if (p < s.size() && s[p] == ',') ++p;
      else if (p < s.size() && s[p] == ']') { ++p; return true; }
      else return false;
    }
  }
  size_t b = p;
  while (p < s.size() && s[p] != ',' && s[p] != ']') ++p;
  out->kind = 1;
  out->s = trim(s.substr(b, p - b));
  if (out->s.size() >= 2 && (out->s[0] == '"' || out->s[0] == '\'')) out->s = out->s.substr(1, out->s.size() - 2);
  return true;
}

struct Line { int ind; std::string t; };

bool parse_map(const std::vector<Line>& L, size_t& i, int ind, Node* out) {
  out->kind = 3;
  while (i < L.size() && L[i].ind == ind) {
    const std::string& t = L[i].t;
    size_t c = std::string::npos;
    for (size_t k = 0; k < t.size(); ++k)
      if (t[k] == ':' && (k + 1 == t.size() || t[k + 1] == ' ')) { c = k; break; }
    if (c == std::string::npos) return false;
    std::string key = trim(t.substr(0, c)), rest = trim(t.substr(c + 1));
    ++i;
    Node v;
    if (!rest.empty()) {
      if (rest[0] == '[') {
        size_t p = 0;
        if (!parse_flow(rest, p, &v)) return false;
      } else {
        v.kind = 1;
        v.s = rest;
        if (v.s.size() >= 2 && (v.s[0] == '"' || v.s[0] == '\'')) v.s = v.s.substr(1, v.s.size() - 2);
      }
    } else if (i < L.size() && L[i].ind > ind) {
      if (!parse_map(L, i, L[i].ind, &v)) return false;
    }
    out->map.emplace_back(key, v);
  }
  return !(i < L.size() && L[i].ind > ind);
}

bool parse_docs(const std::string& text, std::vector<Node>* docs) {
  std::vector<std::vector<Line>> g(1);
  std::istringstream in(text);
  std::string raw;
  bool content = false;
  while (std::getline(in, raw)) {
    size_t h = raw.find(" #");
    if (!raw.empty() && raw[0] == '#') raw.clear();
    else if (h != std::string::npos) raw = raw.substr(0, h);
    std::string t = trim(raw);
    if (t == "---") { if (content) g.emplace_back(); content = true; continue; }
    if (t.empty() || t == "...") continue;
    int ind = 0;
    while (ind < (int)raw.size() && raw[ind] == ' ') ++ind;
    g.back().push_back({ind, t});
    content = true;
  }
  for (auto& lines : g) {
    Node d;
    if (!lines.empty()) {
      size_t i = 0;
      if (!parse_map(lines, i, lines[0].ind, &d) || i != lines.size()) return false;
    }
    docs->push_back(d);
  }
  return true;
}

bool num(const Node* n, float* f) {
  if (!n || n->kind != 1) return false;
  char* e = nullptr;
  *f = strtof(n->s.c_str(), &e);
  return e != n->s.c_str();
}
bool inum(const Node* n, int* v) {
  if (!n || n->kind != 1) return false;
  char* e = nullptr;
  *v = (int)strtol(n->s.c_str(), &e, 10);
  return e != n->s.c_str();
}
bool vecn(const Node* n, int k, float* f) {
  if (!n || n->kind != 2 || (int)n->seq.size() != k) return false;
  for (int i = 0; i < k; ++i)
    if (!num(&n->seq[i], &f[i])) return false;
  return true;
}
std::string str(const Node* n) { return n && n->kind == 1 ? n->s : ""; }

// ------------------------------------------------------------ OBJ (tinyobj rules)
double parse_number(const char* s, const char* end) {  // tiny_obj_loader.cpp:131-242
  if (s >= end) return 0.0;
  double mant = 0.0;
  int ex = 0, read = 0;
  char sign = '+', esign = '+';
  const char* c = s;
  bool more = false;
  if (*c == '+' || *c == '-') { sign = *c; ++c; }
  else if (!isdigit((unsigned char)*c)) return 0.0;
  while ((more = (c != end)) && isdigit((unsigned char)*c)) { mant *= 10; mant += (int)(*c - '0'); ++c; ++read; }
  if (read == 0) return 0.0;
  if (more) {
    bool do_exp = false;
    if (*c == '.') {
      ++c;
      read = 1;
      while ((more = (c != end)) && isdigit((unsigned char)*c)) { mant += (int)(*c - '0') * std::pow(10.0, -read); ++read; ++c; }
      do_exp = more;
    } else if (*c == 'e' || *c == 'E') {
      do_exp = true;
    }
    if (do_exp && (*c == 'e' || *c == 'E')) {
      ++c;
      if ((more = (c != end)) && (*c == '+' || *c == '-')) { esign = *c; ++c; }
      else if (!isdigit((unsigned char)*c)) return 0.0;
      read = 0;
      while ((more = (c != end)) && isdigit((unsigned char)*c)) { ex *= 10; ex += (int)(*c - '0'); ++c; ++read; }
      ex *= (esign == '+' ? 1 : -1);
      if (read == 0) return 0.0;
    }
  }
  return (sign == '+' ? 1 : -1) * std::ldexp(mant * std::pow(5.0, ex), ex);
}

struct Obj {
  std::vector<float> pos, tex;
  std::vector<uint32_t> idx;
};

struct Key { int v, vt, vn; bool operator==(const Key& o) const { return v == o.v && vt == o.vt && vn == o.vn; } };
struct KeyHash { size_t operator()(const Key& k) const { return ((size_t)(uint32_t)k.v * 73856093u) ^ ((size_t)(uint32_t)k.vt * 19349663u) ^ ((size_t)(uint32_t)k.vn * 83492791u); } };

bool load_obj(const std::string& path, Obj* o) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  std::vector<float> v, vt, vn;
  std::vector<std::vector<Key>> faces;
  size_t p = 0;
  auto fix = [](int i, int n) { return i > 0 ? i - 1 : (i == 0 ? 0 : n + i); };
  auto flt = [](const char*& t) {
    t += strspn(t, " \t");
    const char* e = t + strcspn(t, " \t\r");
    float r = (float)parse_number(t, e);
    t = e;
    return r;
  };
  std::string line;
  while (p < text.size()) {
    size_t e = text.find('\n', p);
    if (e == std::string::npos) e = text.size();
    line.assign(text, p, e - p);
    p = e + 1;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.size() > 8191) line.resize(8191);
    const char* t = line.c_str();
    t += strspn(t, " \t");
    if (t[0] == 'v' && (t[1] == ' ' || t[1] == '\t')) {
      t += 2;
      float a = flt(t), b = flt(t), c = flt(t);
      v.insert(v.end(), {a, b, c});
    } else if (t[0] == 'v' && t[1] == 'n' && (t[2] == ' ' || t[2] == '\t')) {
      t += 3;
      float a = flt(t), b = flt(t), c = flt(t);
      vn.insert(vn.end(), {a, b, c});
    } else if (t[0] == 'v' && t[1] == 't' && (t[2] == ' ' || t[2] == '\t')) {
      t += 3;
      float a = flt(t), b = flt(t);
      vt.insert(vt.end(), {a, b});
    } else if (t[0] == 'f' && (t[1] == ' ' || t[1] == '\t')) {
      t += 2;
      t += strspn(t, " \t");
      std::vector<Key> face;
      while (!(t[0] == '\r' || t[0] == '\n' || t[0] == '\0')) {
        Key k{-1, -1, -1};
        k.v = fix(atoi(t), (int)(v.size() / 3));
        t += strcspn(t, "/ \t\r");
        if (t[0] == '/') {
          ++t;
          if (t[0] == '/') {
            ++t;
            k.vn = fix(atoi(t), (int)(vn.size() / 3));
            t += strcspn(t, "/ \t\r");
          } else {
            k.vt = fix(atoi(t), (int)(vt.size() / 2));
            t += strcspn(t, "/ \t\r");
            if (t[0] == '/') {
              ++t;
              k.vn = fix(atoi(t), (int)(vn.size() / 3));
              t += strcspn(t, "/ \t\r");
            }
          }
        }
        face.push_back(k);
        t += strspn(t, " \t\r");
      }
      faces.push_back(face);
    }
  }
  std::unordered_map<Key, uint32_t, KeyHash> cache;
  auto vert = [&](const Key& k) -> int64_t {
    auto it = cache.find(k);
    if (it != cache.end()) return it->second;
    if (k.v < 0 || (size_t)(3 * k.v + 2) >= v.size()) return -1;
    o->pos.insert(o->pos.end(), {v[3 * k.v], v[3 * k.v + 1], v[3 * k.v + 2]});
    if (k.vt >= 0 && (size_t)(2 * k.vt + 1) < vt.size()) o->tex.insert(o->tex.end(), {vt[2 * k.vt], vt[2 * k.vt + 1]});
    uint32_t id = (uint32_t)(o->pos.size() / 3 - 1);
    cache[k] = id;
    return id;
  };
  for (auto& fc : faces) {
    if (fc.size() < 3) continue;
    for (size_t k = 2; k < fc.size(); ++k) {  // fan (tiny_obj_loader.cpp:380-405)
      int64_t a = vert(fc[0]), b = vert(fc[k - 1]), c = vert(fc[k]);
      if (a < 0 || b < 0 || c < 0) return false;
      o->idx.insert(o->idx.end(), {(uint32_t)a, (uint32_t)b, (uint32_t)c});
    }
  }
  return true;
}

// ------------------------------------------------------------ scene
struct M3 { float a[3][3]; };
M3 mm(const M3& x, const M3& y) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = (x.a[i][0] * y.a[0][j] + x.a[i][1] * y.a[1][j]) + x.a[i][2] * y.a[2][j];
  return r;
}
M3 rot(int axis, float deg) {
  float ang = deg * kPi180;
  float c = std::cos(ang), s = std::sin(ang);
  M3 r = {{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}};
  int u = (axis + 1) % 3, v = (axis + 2) % 3;
  r.a[u][u] = c; r.a[u][v] = -s; r.a[v][u] = s; r.a[v][v] = c;
  return r;
}
Aff affine(const M3& l, const float t[3]) {
  Aff a;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) a.m[i][j] = l.a[i][j];
    a.m[i][3] = t[i];
  }
  return a;
}
// Eigen compositions of PolygonObject.cpp:17-22 / QuadLight.cpp:25-31 (T Rx Ry Rz S)
// and PinHoleCamera.cpp:7-11 (T Ry Rx Rz).
Aff trs_xyz(const float t[3], const float r[3], const float s[3]) {
  M3 l = mm(mm(rot(0, r[0]), rot(1, r[1])), rot(2, r[2]));
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) l.a[i][j] = l.a[i][j] * s[j];
  return affine(l, t);
}
Aff tr_yxz(const float t[3], const float r[3]) { return affine(mm(mm(rot(1, r[1]), rot(0, r[0])), rot(2, r[2])), t); }
// normalize(L^-T X) via the first cofactor column, signed by det(L).
void x_normal(const Aff& a, float out[3]) {
  const float(*L)[4] = a.m;
  float c0 = L[1][1] * L[2][2] - L[1][2] * L[2][1];
  float c1 = -(L[0][1] * L[2][2] - L[0][2] * L[2][1]);
  float c2 = L[0][1] * L[1][2] - L[0][2] * L[1][1];
  float det = (L[0][0] * c0 + L[1][0] * c1) + L[2][0] * c2;
  if (det < 0.f) { c0 = -c0; c1 = -c1; c2 = -c2; }
  float inv = 1.0f / std::sqrt((c0 * c0 + c1 * c1) + c2 * c2);
  out[0] = c0 * inv; out[1] = c1 * inv; out[2] = c2 * inv;
}
void point(const Aff& a, const float p[3], float o[3]) {
  for (int i = 0; i < 3; ++i) o[i] = ((a.m[i][0] * p[0] + a.m[i][1] * p[1]) + a.m[i][2] * p[2]) + a.m[i][3];
}

enum { LAMBERT = 0, NULLSH = 1, PHONG = 2 };
struct Shader { int type = LAMBERT; int light = -1; float refl = 1.f, ex = 0.f; float col[3] = {0, 0, 0}; int tex = 0; int tex_root = -1; };
// Texture trees (ConstantTexture / StandardTexture / LayeredTexture, include/core/*Texture.h).
struct TNode { int type = 0; int image = -1, upper = -1, lower = -1, mask = -1; float col[3] = {0, 0, 0}; };
struct OImage { int w = 0, h = 0; std::vector<float> rgb; };  // rows top first
struct Geom { int shader = 0, first = 0, count = 0, light = -1; };
struct Light { int type = 0; float inten = 100.f; float scale[2] = {1, 1}; Aff m; float n[3]; float c[3]; float rad = 0.f; };

struct BNode { float lo[3], hi[3]; int left, right, start, count; };

}  // namespace orc

using namespace orc;

struct oracle_scene {
  int W = 700, H = 500, base = 8, spp = 64, gx = 8, gy = 8;
  int min_depth = 2, max_depth = 100;
  float threshold = 0.01f;
  int cam_type = 1;  // 0 pinhole, 1 thin lens
  Aff cam;
  float cam_n[3], cam_t[3] = {0, 0, 0};
  float focal = 55.f, fdist = 1000.f, aperture = 5.6f;
  int sampler = 0, filter = 0, mis_power = 0;
  uint32_t seed = 0;
  std::vector<Shader> shaders;
  std::vector<Geom> geoms;
  std::vector<Light> lights;
  std::vector<int> sphere_lights;  // light index of each sphere light (extension)
  int texel_res = 0;           // per-face texels (extension)
  uint32_t texel_seed = 0;
  std::vector<TNode> tnodes;   // image textures
  std::vector<OImage> images;
  std::vector<std::string> image_paths;
  std::vector<float> tuv;      // 6 per triangle: texcoords of v0, v1, v2
  std::vector<float> tv;       // 9 per triangle
  std::vector<int> tgeom;
  std::vector<uint8_t> tlight;
  // BVH
  std::vector<BNode> nodes;
  std::vector<int> order;      // leaf triangle order
};

namespace orc {

// PFM ("PF"/"Pf", rows bottom first, scale < 0 little endian) and binary PPM
// ("P6", maxval < 256: bytes, else 16-bit big endian), both stored top first.
// binary16 -> binary32, exact.
float h2f(uint16_t h) {
  const int e = (h >> 10) & 31, m = h & 1023;
  float v;
  if (e == 0) v = std::ldexp((float)m, -24);
  else if (e == 31) v = m ? NAN : INFINITY;
  else v = std::ldexp((float)(1024 + m), e - 25);
  return (h & 0x8000) ? -v : v;
}

// Uncompressed single-part scanline OpenEXR: R, G, B (or Y) of HALF / FLOAT.
bool read_exr(const std::string& d, OImage* im) {
  auto u32 = [&](size_t p) { return (uint32_t)(unsigned char)d[p] | ((uint32_t)(unsigned char)d[p + 1] << 8) |
                                    ((uint32_t)(unsigned char)d[p + 2] << 16) | ((uint32_t)(unsigned char)d[p + 3] << 24); };
  if (d.size() < 8 || u32(0) != 20000630u || (u32(4) & 0xff) != 2 || (u32(4) & 0x1e00)) return false;
  size_t p = 8;
  std::vector<std::pair<std::string, int>> ch;
  int comp = -1, x0 = 0, y0 = 0, x1 = -1, y1 = -1;
  while (p < d.size() && d[p]) {
    std::string name, type;
    while (p < d.size() && d[p]) name.push_back(d[p++]);
    ++p;
    while (p < d.size() && d[p]) type.push_back(d[p++]);
    ++p;
    if (p + 4 > d.size()) return false;
    size_t sz = u32(p);
    p += 4;
    size_t end = p + sz;
    if (end > d.size()) return false;
    if (name == "channels") {
      size_t q = p;
      while (q < end && d[q]) {
        std::string cn;
        while (q < end && d[q]) cn.push_back(d[q++]);
        ++q;
        ch.push_back({cn, (int)u32(q)});
        q += 16;
      }
    } else if (name == "compression") comp = (unsigned char)d[p];
    else if (name == "dataWindow") { x0 = (int)u32(p); y0 = (int)u32(p + 4); x1 = (int)u32(p + 8); y1 = (int)u32(p + 12); }
    p = end;
  }
  ++p;
  const int w = x1 - x0 + 1, h = y1 - y0 + 1;
  if (comp != 0 || w <= 0 || h <= 0 || ch.empty()) return false;
  size_t line = 0;
  std::vector<size_t> off;
  int idx[3] = {-1, -1, -1}, iy = -1;
  for (size_t c = 0; c < ch.size(); ++c) {
    if (ch[c].second != 1 && ch[c].second != 2) return false;
    off.push_back(line);
    line += (size_t)w * (ch[c].second == 1 ? 2 : 4);
    if (ch[c].first == "R") idx[0] = (int)c;
    if (ch[c].first == "G") idx[1] = (int)c;
    if (ch[c].first == "B") idx[2] = (int)c;
    if (ch[c].first == "Y") iy = (int)c;
  }
  if (idx[0] < 0 || idx[1] < 0 || idx[2] < 0) { if (iy < 0) return false; idx[0] = idx[1] = idx[2] = iy; }
  im->w = w; im->h = h;
  im->rgb.assign((size_t)w * h * 3, 0.f);
  for (int k = 0; k < h; ++k) {
    const size_t bo = (size_t)u32(p + 8 * (size_t)k) | ((size_t)u32(p + 8 * (size_t)k + 4) << 32);
    if (bo + 8 + line > d.size()) return false;
    const int y = (int)u32(bo) - y0;
    if (y < 0 || y >= h) return false;
    for (int x = 0; x < w; ++x)
      for (int c = 0; c < 3; ++c) {
        const int t = ch[idx[c]].second;
        const size_t q = bo + 8 + off[idx[c]] + (size_t)x * (t == 1 ? 2 : 4);
        float v;
        if (t == 1) v = h2f((uint16_t)((unsigned char)d[q] | ((unsigned char)d[q + 1] << 8)));
        else { uint32_t u = u32(q); memcpy(&v, &u, 4); }
        im->rgb[((size_t)y * w + x) * 3 + c] = v;
      }
  }
  return true;
}

bool read_image(const std::string& path, OImage* im) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::string d((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  if (d.size() >= 4 && (unsigned char)d[0] == 0x76 && (unsigned char)d[1] == 0x2f) return read_exr(d, im);
  size_t p = 0;
  auto tok = [&]() {
    while (p < d.size() && (isspace((unsigned char)d[p]) || d[p] == '#')) {
      if (d[p] == '#') while (p < d.size() && d[p] != '\n') ++p;
      else ++p;
    }
    size_t b = p;
    while (p < d.size() && !isspace((unsigned char)d[p])) ++p;
    return d.substr(b, p - b);
  };
  std::string mg = tok();
  long w = atol(tok().c_str()), h = atol(tok().c_str());
  std::string third = tok();
  ++p;
  if (w <= 0 || h <= 0) return false;
  im->w = (int)w; im->h = (int)h;
  im->rgb.assign((size_t)w * h * 3, 0.f);
  const unsigned char* r = (const unsigned char*)d.data() + p;
  if (mg == "PF" || mg == "Pf") {
    int ch = mg == "PF" ? 3 : 1;
    bool le = atof(third.c_str()) < 0;
    if (d.size() - p < (size_t)w * h * ch * 4) return false;
    for (long y = 0; y < h; ++y)
      for (long x = 0; x < w; ++x)
        for (int k = 0; k < 3; ++k) {
          const unsigned char* q = r + 4 * ((y * w + x) * ch + (ch == 3 ? k : 0));
          uint32_t u = le ? (q[0] | (q[1] << 8) | (q[2] << 16) | ((uint32_t)q[3] << 24))
                          : (q[3] | (q[2] << 8) | (q[1] << 16) | ((uint32_t)q[0] << 24));
          float v; memcpy(&v, &u, 4);
          im->rgb[((h - 1 - y) * w + x) * 3 + k] = v;
        }
    return true;
  }
  if (mg == "P6") {
    long mv = atol(third.c_str());
    int bps = mv < 256 ? 1 : 2;
    if (mv <= 0 || d.size() - p < (size_t)w * h * 3 * bps) return false;
    for (size_t i = 0; i < (size_t)w * h * 3; ++i) {
      uint32_t v = bps == 1 ? r[i] : ((uint32_t)r[2 * i] << 8) | r[2 * i + 1];
      im->rgb[i] = (float)v / (float)mv;
    }
    return true;
  }
  return false;
}

int tex_node(const Node* n, oracle_scene* S, const std::string& dir) {
  if (!n) return -1;
  std::string ty = str(n->get("type"));
  TNode t;
  if (ty == "Constant") {
    if (!vecn(n->get("colour"), 3, t.col)) return -1;
  } else if (ty == "Standard") {
    t.type = 1;
    std::string path = dir + "/" + str(n->get("string"));
    for (size_t i = 0; i < S->image_paths.size(); ++i) if (S->image_paths[i] == path) t.image = (int)i;
    if (t.image < 0) {
      OImage im;
      if (!read_image(path, &im)) return -1;
      S->images.push_back(im);
      S->image_paths.push_back(path);
      t.image = (int)S->images.size() - 1;
    }
  } else if (ty == "Layered") {
    t.type = 2;
    t.upper = tex_node(n->get("upper"), S, dir);
    t.lower = tex_node(n->get("lower"), S, dir);
    t.mask = tex_node(n->get("mask"), S, dir);
    if (t.upper < 0 || t.lower < 0 || t.mask < 0) return -1;
  } else {
    return -1;
  }
  S->tnodes.push_back(t);
  return (int)S->tnodes.size() - 1;
}

// Periodic bilinear lookup between texel centres, t = 0 on the top row (the
// stand-in for OpenImageIO's texture() with periodic wrap, StandardTexture.cpp:18-34).
void image_lookup(const OImage& im, float s, float t, float out[3]) {
  const int w = im.w, h = im.h;
  s = s - std::floor(s);
  t = t - std::floor(t);
  const float x = s * (float)w - 0.5f, y = t * (float)h - 0.5f;
  const float fx0 = std::floor(x), fy0 = std::floor(y);
  const float fx = x - fx0, fy = y - fy0;
  int x0 = (int)fx0, y0 = (int)fy0;
  x0 = x0 < 0 ? x0 + w : (x0 >= w ? x0 - w : x0);
  y0 = y0 < 0 ? y0 + h : (y0 >= h ? y0 - h : y0);
  const int x1 = x0 + 1 == w ? 0 : x0 + 1, y1 = y0 + 1 == h ? 0 : y0 + 1;
  const float gx = 1.f - fx, gy = 1.f - fy;
  for (int k = 0; k < 3; ++k) {
    const float c00 = im.rgb[((size_t)y0 * w + x0) * 3 + k], c10 = im.rgb[((size_t)y0 * w + x1) * 3 + k];
    const float c01 = im.rgb[((size_t)y1 * w + x0) * 3 + k], c11 = im.rgb[((size_t)y1 * w + x1) * 3 + k];
    out[k] = (c00 * gx + c10 * fx) * gy + (c01 * gx + c11 * fx) * fy;
  }
}

// LayeredTexture.cpp:14-37: upper * mask + lower * (1 - mask).
void tex_eval(const oracle_scene* S, int node, float s, float t, float out[3]) {
  const TNode& n = S->tnodes[node];
  if (n.type == 0) { out[0] = n.col[0]; out[1] = n.col[1]; out[2] = n.col[2]; return; }
  if (n.type == 1) { image_lookup(S->images[n.image], s, t, out); return; }
  float u[3], l[3], m[3];
  tex_eval(S, n.upper, s, t, u);
  tex_eval(S, n.lower, s, t, l);
  tex_eval(S, n.mask, s, t, m);
  for (int k = 0; k < 3; ++k) out[k] = u[k] * m[k] + l[k] * (1.f - m[k]);
}

bool load(const std::string& path, oracle_scene* S, std::string* err) {
  std::ifstream f(path, std::ios::binary);
  if (!f) { *err = "cannot open " + path; return false; }
  std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  std::vector<Node> docs;
  if (!parse_docs(text, &docs) || docs.size() < 2) { *err = "malformed scene yaml"; return false; }
  std::string dir = ".";
  size_t sl = path.find_last_of('/');
  if (sl != std::string::npos) dir = path.substr(0, sl);
  const Node& su = docs[0];
  const Node& sc = docs[1];
  float t0[3] = {0, 0, 0}, r0[3] = {0, 0, 0};
  S->cam = tr_yxz(t0, r0);
  x_normal(S->cam, S->cam_n);
  if (const Node* n = su.get("image")) {
    if (n->size() != 3 || !inum(n->get("width"), &S->W) || !inum(n->get("height"), &S->H) || !inum(n->get("sample base"), &S->base)) { *err = "image"; return false; }
  }
  if (const Node* n = su.get("settings")) {
    int dummy;
    if (n->size() != 6 || !inum(n->get("min depth"), &S->min_depth) || !inum(n->get("max depth"), &S->max_depth) ||
        !num(n->get("threshold"), &S->threshold) || !inum(n->get("bucket size"), &dummy) ||
        !inum(n->get("shading size"), &dummy) || !inum(n->get("bin exponent"), &dummy)) { *err = "settings"; return false; }
  }
  if (const Node* n = su.get("camera")) {
    float t[3], r[3];
    std::string ty = str(n->get("type"));
    if (!vecn(n->get("translation"), 3, t) || !vecn(n->get("rotation"), 3, r) || !num(n->get("focal length"), &S->focal)) { *err = "camera"; return false; }
    if (ty == "PinHole") S->cam_type = 0;
    else if (ty == "ThinLens") {
      S->cam_type = 1;
      if (!num(n->get("focal distance"), &S->fdist) || !num(n->get("aperture"), &S->aperture)) { *err = "camera"; return false; }
    } else { *err = "camera type"; return false; }
    S->cam = tr_yxz(t, r);
    x_normal(S->cam, S->cam_n);
    for (int i = 0; i < 3; ++i) S->cam_t[i] = t[i];
  }
  if (const Node* n = su.get("filter")) S->filter = str(n->get("type")) == "Box" ? 1 : 0;
  if (const Node* n = su.get("sampler")) {
    std::string ty = str(n->get("type"));
    S->sampler = ty == "Independent" ? 1 : (ty == "Grid" ? 2 : 0);
  }
  int spp_ext = 0;
  if (docs.size() >= 3)
    if (const Node* e = docs[2].get("extensions")) {
      for (auto& kv : e->map) {
        if (kv.first == "samples per pixel") inum(&kv.second, &spp_ext);
        else if (kv.first == "mis") S->mis_power = str(&kv.second) == "power" ? 1 : 0;
        else if (kv.first == "seed") { int v = 0; inum(&kv.second, &v); S->seed = (uint32_t)v; }
      }
    }
  if (spp_ext > 0) {
    S->spp = spp_ext;
    int a = 1;
    for (int d = 1; d * d <= spp_ext; ++d)
      if (spp_ext % d == 0) a = d;
    S->gx = a;
    S->gy = spp_ext / a;
  } else {
    S->spp = S->base * S->base;
    S->gx = S->gy = S->base;
  }
  auto add_tris = [&](const std::vector<float>& p, const std::vector<uint32_t>& idx, int g, bool light,
                      const std::vector<float>& uv) {
    for (size_t t = 0; t + 2 < idx.size(); t += 3) {
      for (int k = 0; k < 3; ++k) {
        for (int a = 0; a < 3; ++a) S->tv.push_back(p[3 * idx[t + k] + a]);
        const size_t vi = idx[t + k];
        const bool has = 2 * vi + 1 < uv.size();
        S->tuv.push_back(has ? uv[2 * vi] : 0.f);
        S->tuv.push_back(has ? uv[2 * vi + 1] : 0.f);
      }
      S->tgeom.push_back(g);
      S->tlight.push_back(light ? 1 : 0);
    }
  };
  for (auto& kv : sc.map) {  // Pathtracer.cpp:166-217
    const Node& n = kv.second;
    if (kv.first == "object" && str(n.get("type")) == "Polygon") {
      float t[3], r[3], s[3];
      int sh = 0;
      if (n.size() != 6 || !vecn(n.get("translation"), 3, t) || !vecn(n.get("rotation"), 3, r) ||
          !vecn(n.get("scale"), 3, s) || !inum(n.get("shader"), &sh)) { *err = "object"; return false; }
      Obj o;
      if (!load_obj(dir + "/" + str(n.get("filename")), &o)) { *err = "obj " + str(n.get("filename")); return false; }
      Aff m = trs_xyz(t, r, s);
      std::vector<float> p(o.pos.size());
      for (size_t i = 0; i + 2 < o.pos.size(); i += 3) point(m, &o.pos[i], &p[i]);
      Geom g;
      g.shader = sh;
      g.first = (int)S->tgeom.size();
      g.count = (int)(o.idx.size() / 3);
      S->geoms.push_back(g);
      add_tris(p, o.idx, (int)S->geoms.size() - 1, false, o.tex);
    } else if (kv.first == "shader") {
      std::string ty = str(n.get("type"));
      Shader s;
      const Node* tex = n.get("texture");
      if (ty == "Lambert" || ty == "Phong") {
        s.type = ty == "Lambert" ? LAMBERT : PHONG;
        const std::string tt = tex ? str(tex->get("type")) : "";
        if (!num(n.get("reflectance"), &s.refl)) { *err = "shader"; return false; }
        if (tt == "Standard" || tt == "Layered") {
          s.tex = 2;
          s.tex_root = tex_node(tex, S, dir);
          if (s.tex_root < 0) { *err = "texture"; return false; }
        } else if ((tt != "Constant" && tt != "FaceTexels") || !vecn(tex->get("colour"), 3, s.col)) {
          *err = "shader";
          return false;
        }
        if (tt == "FaceTexels") {  // extension: per-face FP16 texels from a seed
          int res = 0, sd = 0;
          if (!inum(tex->get("resolution"), &res) || !inum(tex->get("seed"), &sd)) { *err = "texture"; return false; }
          S->texel_res = res;
          S->texel_seed = (uint32_t)sd;
          s.tex = 1;
        }
        if (s.type == PHONG && !num(n.get("exponent"), &s.ex)) { *err = "shader"; return false; }
        S->shaders.push_back(s);
      }
    }
  }
  for (auto& kv : sc.map) {  // Pathtracer.cpp:219-272
    const Node& n = kv.second;
    if (kv.first == "light" && str(n.get("type")) == "Sphere") {  // extension: no triangle geometry
      Light L;
      L.type = 1;
      if (!vecn(n.get("translation"), 3, L.c) || !num(n.get("radius"), &L.rad) || !num(n.get("intensity"), &L.inten)) {
        *err = "light";
        return false;
      }
      Shader ns;
      ns.type = NULLSH;
      ns.light = (int)S->lights.size();
      S->sphere_lights.push_back(ns.light);
      S->shaders.push_back(ns);
      S->lights.push_back(L);
      continue;
    }
    if (kv.first != "light" || str(n.get("type")) != "Quad") continue;
    Light L;
    float t[3], r[3];
    if (!vecn(n.get("translation"), 3, t) || !vecn(n.get("rotation"), 3, r) || !vecn(n.get("scale"), 2, L.scale) ||
        !num(n.get("intensity"), &L.inten)) { *err = "light"; return false; }
    float s3[3] = {1.f, L.scale[0], L.scale[1]};
    L.m = trs_xyz(t, r, s3);
    x_normal(L.m, L.n);
    Shader ns;
    ns.type = NULLSH;
    ns.light = (int)S->lights.size();
    Geom g;
    g.shader = (int)S->shaders.size();
    g.first = (int)S->tgeom.size();
    g.count = 2;
    g.light = ns.light;
    S->shaders.push_back(ns);
    S->geoms.push_back(g);
    S->lights.push_back(L);
    const float q[6][3] = {{0.f, -0.5f, -0.5f}, {0.f, 0.5f, -0.5f}, {0.f, 0.5f, 0.5f},
                           {0.f, 0.5f, 0.5f}, {0.f, -0.5f, 0.5f}, {0.f, -0.5f, -0.5f}};
    std::vector<float> p(18);
    for (int i = 0; i < 6; ++i) point(L.m, q[i], &p[3 * i]);
    add_tris(p, {0, 1, 2, 3, 4, 5}, (int)S->geoms.size() - 1, true, std::vector<float>());
  }
  for (auto& g : S->geoms)
    if (g.shader < 0 || g.shader >= (int)S->shaders.size()) { *err = "object shader index"; return false; }
  return true;
}

// ------------------------------------------------------------ SAH BVH
void tri_box(const oracle_scene* S, int t, float lo[3], float hi[3]) {
  const float* v = &S->tv[9 * t];
  for (int a = 0; a < 3; ++a) {
    lo[a] = std::min(std::min(v[a], v[3 + a]), v[6 + a]);
    hi[a] = std::max(std::max(v[a], v[3 + a]), v[6 + a]);
  }
}

void build_bvh(oracle_scene* S) {
  const int n = (int)S->tgeom.size();
  S->order.resize(n);
  for (int i = 0; i < n; ++i) S->order[i] = i;
  std::vector<float> cen((size_t)n * 3), blo((size_t)n * 3), bhi((size_t)n * 3);
  for (int i = 0; i < n; ++i) {
    tri_box(S, i, &blo[3 * i], &bhi[3 * i]);
    for (int a = 0; a < 3; ++a) cen[3 * i + a] = 0.5f * (blo[3 * i + a] + bhi[3 * i + a]);
  }
  S->nodes.clear();
  S->nodes.reserve(2 * (size_t)n + 1);
  struct Job { int node, start, count; };
  std::vector<Job> stack;
  S->nodes.push_back(BNode());
  stack.push_back({0, 0, n});
  const int BINS = 16;
  while (!stack.empty()) {
    Job j = stack.back();
    stack.pop_back();
    BNode nd;
    float clo[3] = {1e30f, 1e30f, 1e30f}, chi[3] = {-1e30f, -1e30f, -1e30f};
    for (int a = 0; a < 3; ++a) { nd.lo[a] = 1e30f; nd.hi[a] = -1e30f; }
    for (int k = j.start; k < j.start + j.count; ++k) {
      int t = S->order[k];
      for (int a = 0; a < 3; ++a) {
        nd.lo[a] = std::min(nd.lo[a], blo[3 * t + a]);
        nd.hi[a] = std::max(nd.hi[a], bhi[3 * t + a]);
        clo[a] = std::min(clo[a], cen[3 * t + a]);
        chi[a] = std::max(chi[a], cen[3 * t + a]);
      }
    }
    nd.left = nd.right = -1;
    nd.start = j.start;
    nd.count = j.count;
    int best_axis = -1, best_split = -1;
    if (j.count > 4) {
      double best = 1e300;
      for (int a = 0; a < 3; ++a) {
        float ext = chi[a] - clo[a];
        if (!(ext > 0.f)) continue;
        int cnt[BINS] = {0};
        float bl[BINS][3], bh[BINS][3];
        for (int b = 0; b < BINS; ++b)
          for (int c = 0; c < 3; ++c) { bl[b][c] = 1e30f; bh[b][c] = -1e30f; }
        for (int k = j.start; k < j.start + j.count; ++k) {
          int t = S->order[k];
          int b = std::min(BINS - 1, (int)((cen[3 * t + a] - clo[a]) / ext * BINS));
          cnt[b]++;
          for (int c = 0; c < 3; ++c) { bl[b][c] = std::min(bl[b][c], blo[3 * t + c]); bh[b][c] = std::max(bh[b][c], bhi[3 * t + c]); }
        }
        auto area = [](const float l[3], const float h[3]) {
          double dx = h[0] - l[0], dy = h[1] - l[1], dz = h[2] - l[2];
          return (dx < 0 || dy < 0 || dz < 0) ? 0.0 : dx * dy + dy * dz + dz * dx;
        };
        double rarea[BINS];
        int rcnt[BINS];
        float rl[3] = {1e30f, 1e30f, 1e30f}, rh[3] = {-1e30f, -1e30f, -1e30f};
        int rc = 0;
        for (int b = BINS - 1; b > 0; --b) {
          rc += cnt[b];
          for (int c = 0; c < 3; ++c) { rl[c] = std::min(rl[c], bl[b][c]); rh[c] = std::max(rh[c], bh[b][c]); }
          rarea[b] = area(rl, rh);
          rcnt[b] = rc;
        }
        float ll[3] = {1e30f, 1e30f, 1e30f}, lh[3] = {-1e30f, -1e30f, -1e30f};
        int lc = 0;
        for (int b = 0; b < BINS - 1; ++b) {
          lc += cnt[b];
          for (int c = 0; c < 3; ++c) { ll[c] = std::min(ll[c], bl[b][c]); lh[c] = std::max(lh[c], bh[b][c]); }
          if (lc == 0 || rcnt[b + 1] == 0) continue;
          double cost = area(ll, lh) * lc + rarea[b + 1] * rcnt[b + 1];
          if (cost < best) { best = cost; best_axis = a; best_split = b; }
        }
      }
    }
    int mid = -1;
    if (best_axis >= 0) {
      float ext = chi[best_axis] - clo[best_axis];
      auto it = std::partition(S->order.begin() + j.start, S->order.begin() + j.start + j.count, [&](int t) {
        int b = std::min(BINS - 1, (int)((cen[3 * t + best_axis] - clo[best_axis]) / ext * BINS));
        return b <= best_split;
      });
      mid = (int)(it - S->order.begin());
      if (mid == j.start || mid == j.start + j.count) mid = -1;
    }
    if (mid < 0 && j.count > 8) mid = j.start + j.count / 2;  // degenerate centroids: split in the middle
    if (mid >= 0) {
      nd.left = (int)S->nodes.size();
      nd.right = nd.left + 1;
      S->nodes.push_back(BNode());
      S->nodes.push_back(BNode());
      stack.push_back({nd.left, j.start, mid - j.start});
      stack.push_back({nd.right, mid, j.start + j.count - mid});
    }
    S->nodes[j.node] = nd;
  }
}

// Moller-Trumbore in the documented order (fused multiply-adds inside dot and cross).
// Accepts tmin < t < tmax, or tmin < t <= tmax when closed (closest-hit
// queries, which settle equal distances by the smaller scene triangle index,
// so the answer does not depend on the order the tree presents candidates in).
template <class T>
bool tri_hit(const oracle_scene* S, int tri, V<T> o, V<T> d, T tmin, T tmax, bool closed, T* tt, T* uu, T* vv) {
  const float* p = &S->tv[9 * tri];
  V<T> v0 = mk<T>(p[0], p[1], p[2]);
  V<T> e1 = sub(mk<T>(p[3], p[4], p[5]), v0);
  V<T> e2 = sub(mk<T>(p[6], p[7], p[8]), v0);
  V<T> pv = cross(d, e2);
  T det = dot(e1, pv);
  if (det == T(0)) return false;
  T inv = T(1) / det;
  V<T> s = sub(o, v0);
  T u = dot(s, pv) * inv;
  if (u < T(0) || u > T(1)) return false;
  V<T> q = cross(s, e1);
  T v = dot(d, q) * inv;
  if (v < T(0) || u + v > T(1)) return false;
  T t = dot(e2, q) * inv;
  if (!(t > tmin && (closed ? t <= tmax : t < tmax))) return false;
  *tt = t; *uu = u; *vv = v;
  return true;
}

// Slab test in double with a relative margin: never culls a box the ray touches.
inline bool box_hit(const BNode& n, const double o[3], const double id[3], double tmin, double tmax) {
  double t0 = tmin, t1 = tmax;
  for (int a = 0; a < 3; ++a) {
    double l = (n.lo[a] - o[a]) * id[a], h = (n.hi[a] - o[a]) * id[a];
    if (std::isnan(l) || std::isnan(h)) continue;
    if (l > h) std::swap(l, h);
    t0 = std::max(t0, l);
    t1 = std::min(t1, h);
  }
  return t0 <= t1 * (1.0 + 1e-9) + 1e-12;
}

template <class T>
int trace(const oracle_scene* S, V<T> o, V<T> d, T tmin, T tmax, bool any, T* th, T* uh, T* vh) {
  double od[3] = {(double)o.x, (double)o.y, (double)o.z};
  double dd[3] = {(double)d.x, (double)d.y, (double)d.z};
  double id[3];
  for (int a = 0; a < 3; ++a) id[a] = dd[a] != 0.0 ? 1.0 / dd[a] : (std::signbit(dd[a]) ? -1e300 : 1e300);
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  int hit = -1;
  while (sp > 0) {
    const BNode& n = S->nodes[stack[--sp]];
    if (!box_hit(n, od, id, (double)tmin, (double)tmax)) continue;
    if (n.left < 0) {
      for (int k = n.start; k < n.start + n.count; ++k) {
        int tri = S->order[k];
        if (any && S->tlight[tri]) continue;
        T t, u, v;
        if (tri_hit<T>(S, tri, o, d, tmin, tmax, !any, &t, &u, &v)) {
          if (any) return tri;
          if (t < tmax || (hit >= 0 && tri < hit)) {
            tmax = t;
            *th = t; *uh = u; *vh = v;
            hit = tri;
          }
        }
      }
    } else {
      if (sp + 2 > 128) continue;
      stack[sp++] = n.right;
      stack[sp++] = n.left;
    }
  }
  return hit;
}

// ------------------------------------------------------------ sphere lights (extension)
// First intersection of o + t d with the sphere (c, r) in (tmin, tmax), else -1.
template <class T>
T sphere_t(V<T> o, V<T> d, const float c[3], float r, T tmin, T tmax) {
  const V<T> oc = sub(o, mk<T>(c[0], c[1], c[2]));
  const T a = dot(d, d);
  const T b = dot(oc, d);
  const T cc = dot(oc, oc) - (T)r * (T)r;
  const T disc = b * b - a * cc;
  if (disc < T(0)) return T(-1);
  const T q = std::sqrt(disc);
  const T t0 = (-b - q) / a;
  if (t0 > tmin && t0 < tmax) return t0;
  const T t1 = (-b + q) / a;
  if (t1 > tmin && t1 < tmax) return t1;
  return T(-1);
}

// Uniform cone sampling pdf of the sphere seen from p: 1 / (2 pi (1 - cos theta_max)).
template <class T>
T sphere_pdf(V<T> p, const float c[3], float r) {
  const V<T> wc = sub(mk<T>(c[0], c[1], c[2]), p);
  const T d2 = dot(wc, wc);
  const T r2 = (T)r * (T)r;
  if (!(d2 > r2)) return T(0);
  const T s2 = r2 / d2;
  const T omc = s2 / (T(1) + std::sqrt(T(1) - s2));
  return T(1) / ((T(2) * T(kPi)) * omc);
}

// Closest hit: triangles, then sphere lights nearer than the triangle (a
// sphere hit is returned as -2 - sphere index).
template <class T>
int closest(const oracle_scene* S, V<T> o, V<T> d, T* th, T* uh, T* vh) {
  int hit = trace<T>(S, o, d, T(kTnear), T(kTfar), false, th, uh, vh);
  T tmax = hit >= 0 ? *th : T(kTfar);
  for (size_t q = 0; q < S->sphere_lights.size(); ++q) {
    const Light& L = S->lights[S->sphere_lights[q]];
    const T t = sphere_t<T>(o, d, L.c, L.rad, T(kTnear), tmax);
    if (t > T(0)) {
      tmax = t;
      *th = t; *uh = T(0); *vh = T(0);
      hit = -2 - (int)q;
    }
  }
  return hit;
}

// Face texel colour factor (extension): k / 1024 with k from the texel hash.
inline float face_texel(uint32_t seed, uint32_t face, uint32_t texel, uint32_t ch) {
  return (float)(pcg4d(seed, face, texel, ch).w >> 22) / 1024.0f;
}

// ------------------------------------------------------------ integrator
template <class T>
T misw(T a, T b, int power) {
  if (power) { T a2 = a * a; return a2 / (a2 + b * b); }
  return a / (a + b);  // Common.h:45-48
}

template <class T>
V<T> frame_dir(V<T> a, T x, T y, T z) {  // LambertShader.cpp:63-67
  V<T> tmp = a.x > T(0.99f) ? mk<T>(0, 1, 0) : mk<T>(1, 0, 0);
  V<T> s = normalize(cross(tmp, a));
  V<T> t = normalize(cross(a, s));
  return add(add(mul(t, x), mul(s, y)), mul(a, z));
}

template <class T>
struct Eval { V<T> f; T cs, pdf; };

template <class T>
Eval<T> evaluate(const Shader& s, V<T> col, V<T> wi, V<T> wo, V<T> n) {  // LambertShader.cpp:27-47, NullShader.cpp:25-39
  Eval<T> e;
  T ci = dot(n, wi), co = dot(n, wo);
  if (s.type == NULLSH) { e.f = mk<T>(0, 0, 0); e.cs = T(1); e.pdf = T(1) * T(kInvPi) * T(0.5f); return e; }
  if (s.type == PHONG) {
    V<T> r = sub(mul(n, T(2) * co), wo);
    T ca = std::max(T(0), dot(r, wi));
    T lobe = pow_pos(ca, (T)s.ex);
    if (ci < T(0) || co < T(0)) e.f = mk<T>(0, 0, 0);
    else e.f = mul(mul(col, (T)s.refl), (((T)s.ex + T(2)) * T(kInvPi) * T(0.5f)) * lobe);
    e.cs = ci < T(0) ? T(0) : ci;
    e.pdf = (((T)s.ex + T(1)) * T(kInvPi) * T(0.5f)) * lobe;
    return e;
  }
  if (ci < T(0) || co < T(0)) e.f = mk<T>(0, 0, 0);
  else e.f = mul(mul(col, (T)s.refl), T(kInvPi));
  e.cs = ci < T(0) ? T(0) : ci;
  e.pdf = e.cs * T(kInvPi);
  return e;
}

struct Counts { uint64_t closest = 0, shadow = 0; };

template <class T>
void render_path(const oracle_scene* S, uint32_t sid, uint32_t seed, T* rgb, T* xy, Counts* cnt) {
  const uint32_t col = (uint32_t)S->H * (uint32_t)S->spp;
  const uint32_t x = sid / col, rem = sid - x * col, y = rem / (uint32_t)S->spp, i = rem - y * (uint32_t)S->spp;
  const U4 r = pcg4d(sid, 0u, seed, 0u);
  const uint32_t ix = i / (uint32_t)S->gy, iy = i - ix * (uint32_t)S->gy;
  // StratifiedSampler.cpp:13-14 / IndependentSampler.cpp:11-12 / GridSampler.cpp:13-14
  T sx, sy;
  const T cx = T(1.f / (float)S->gx), cy = T(1.f / (float)S->gy);
  if (S->sampler == 1) { sx = (T)u01(r.x); sy = (T)u01(r.y); }
  else if (S->sampler == 2) { sx = (T)ix * cx + T(0.5f) * cx; sy = (T)iy * cy + T(0.5f) * cy; }
  else { sx = (T)ix * cx + (T)u01(r.x) * cx; sy = (T)iy * cy + (T)u01(r.y) * cy; }
  const T px = (T)x + sx, py = (T)y + sy;
  if (xy) { xy[0] = px; xy[1] = py; }
  const T W = (T)S->W, H = (T)S->H;
  const T fx = ((px * T(2) - W) / W) * T(36);   // Camera.cpp:34-35
  const T fy = ((py * T(2) - H) / W) * T(36);
  const V<T> cn = mk<T>(S->cam_n[0], S->cam_n[1], S->cam_n[2]);
  const V<T> ct = mk<T>(S->cam_t[0], S->cam_t[1], S->cam_t[2]);
  const V<T> nodal = add(ct, mul(cn, (T)S->focal));
  const V<T> film = xf<T>(S->cam, mk<T>(0, fy, fx));
  V<T> o, d;
  if (S->cam_type == 1) {  // ThinLensCamera.cpp:16-56
    const T ratio = (T)S->fdist / (T)S->focal;
    const V<T> focal = add(film, mul(sub(nodal, film), ratio));
    T ax = 0, ay = 0;
    U4 q = r;
    for (int at = 0; at < 64; ++at) {
      uint32_t a, b;
      if (at == 0) { a = r.z; b = r.w; }
      else {
        if (at & 1) q = pcg4d(sid, 0u, seed, 1u + (uint32_t)(at >> 1));
        a = (at & 1) ? q.x : q.z;
        b = (at & 1) ? q.y : q.w;
      }
      const T tx = (T)(u01(a) - 0.5f), ty = (T)(u01(b) - 0.5f);
      if (std::sqrt(tx * tx + ty * ty) < T(0.5f)) { ax = tx; ay = ty; break; }
    }
    const T sc = (T)S->focal / (T)S->aperture;
    const V<T> ap = xf<T>(S->cam, mk<T>(0, ax * sc, ay * sc));
    o = add(ap, mul(cn, (T)S->focal));
    d = normalize(sub(focal, o));
  } else {  // PinHoleCamera.cpp:18-30
    o = nodal;
    d = normalize(sub(nodal, film));
  }
  V<T> w = mk<T>(1, 1, 1);
  T last_pdf = T(1);
  int depth = 0;
  V<T> L = mk<T>(0, 0, 0);
  const int nl = (int)S->lights.size();
  const T pick = nl > 0 ? (T)(1.f / (float)nl) : T(0);
  while (true) {
    T t = 0, hu = 0, hv = 0;
    cnt->closest++;
    const int tri = closest<T>(S, o, d, &t, &hu, &hv);
    if (tri < -1) {  // sphere light (extension): uniform radiance on its outside
      const Light& Lt = S->lights[S->sphere_lights[-2 - tri]];
      const V<T> dn = normalize(d);
      const V<T> pos = add(o, mul(dn, t));
      const V<T> nl = mul(sub(pos, mk<T>(Lt.c[0], Lt.c[1], Lt.c[2])), T(1) / (T)Lt.rad);
      const T le = dot(nl, neg(dn)) < T(0) ? T(0) : (T)Lt.inten;
      T mis = T(1);
      if (depth > 0) mis = misw(last_pdf, sphere_pdf<T>(o, Lt.c, Lt.rad) * pick, S->mis_power);
      if (le > T(kEps)) {
        L.x += le * mis * w.x;
        L.y += le * mis * w.y;
        L.z += le * mis * w.z;
      }
      break;
    }
    if (tri < 0) break;  // Integrator.cpp:26-27
    const Geom& g = S->geoms[S->tgeom[tri]];
    const Shader& sh = S->shaders[g.shader];
    const V<T> dn = normalize(d);
    if (sh.light >= 0) {  // Integrator.cpp:37-76, QuadLight.cpp:69-84
      const Light& Lt = S->lights[sh.light];
      const V<T> ln = mk<T>(Lt.n[0], Lt.n[1], Lt.n[2]);
      const T cosl = dot(ln, neg(dn));
      const T le = cosl < T(0) ? T(0) : (T)Lt.inten;
      const T pdfa = T(1) / ((T)Lt.scale[0] * (T)Lt.scale[1]);
      T mis = T(1);
      if (depth > 0) {
        const T pdfw = pdfa * (t * t) / std::fabs(cosl);
        mis = misw(last_pdf, pdfw * pick, S->mis_power);
      }
      if (le > T(kEps)) {
        L.x += le * mis * w.x;
        L.y += le * mis * w.y;
        L.z += le * mis * w.z;
      }
      break;
    }
    const float* tv = &S->tv[9 * tri];
    const V<T> v0 = mk<T>(tv[0], tv[1], tv[2]);
    const V<T> e1 = sub(mk<T>(tv[3], tv[4], tv[5]), v0), e2 = sub(mk<T>(tv[6], tv[7], tv[8]), v0);
    const V<T> nrm = normalize(cross(e1, e2));  // = -normalize(Ng), Integrator.cpp:121-125
    const V<T> pos = add(o, mul(dn, t));
    const V<T> wo = neg(dn);
    V<T> colr = mk<T>(sh.col[0], sh.col[1], sh.col[2]);  // ConstantTexture.cpp:22-25
    if (sh.tex == 2) {  // Standard / Layered (PolygonObject.cpp:45-63 texture coordinates)
      const float* uv = &S->tuv[6 * (size_t)tri];
      const float fs = (float)hu, ft = (float)hv;
      const float su = (((1.f - fs) - ft) * uv[0] + fs * uv[2]) + ft * uv[4];
      const float sv = (((1.f - fs) - ft) * uv[1] + fs * uv[3]) + ft * uv[5];
      float c3[3];
      tex_eval(S, sh.tex_root, su, sv, c3);
      colr = mk<T>(c3[0], c3[1], c3[2]);
    } else if (sh.tex == 1 && S->texel_res > 0) {  // face texels (extension)
      const int res = S->texel_res;
      const int ti = std::min(res - 1, std::max(0, (int)((float)hu * (float)res)));
      const int tj = std::min(res - 1, std::max(0, (int)((float)hv * (float)res)));
      const uint32_t tx = (uint32_t)(tj * res + ti);
      colr = mk<T>(colr.x * (T)face_texel(S->texel_seed, (uint32_t)tri, tx, 0u),
                   colr.y * (T)face_texel(S->texel_seed, (uint32_t)tri, tx, 1u),
                   colr.z * (T)face_texel(S->texel_seed, (uint32_t)tri, tx, 2u));
    }
    const U4 ra = pcg4d(sid, (uint32_t)depth + 1u, seed, 0u);
    if (nl > 0) {  // Integrator.cpp:103-178, QuadLight.cpp:41-67
      int li = (int)((T)nl * (T)u01(ra.x));
      if (li >= nl) li = nl - 1;
      const Light& Lt = S->lights[li];
      V<T> wi;
      T dist, pdfw, le;
      if (Lt.type == 1) {  // sphere light (extension): uniform in its cone, distance to its near side
        const V<T> wc = sub(mk<T>(Lt.c[0], Lt.c[1], Lt.c[2]), pos);
        const T d2 = dot(wc, wc);
        const T r2 = (T)Lt.rad * (T)Lt.rad;
        le = T(0); dist = T(0); pdfw = T(1); wi = mk<T>(0, 0, 1);
        if (d2 > r2) {
          const T s2 = r2 / d2;
          const T omc = s2 / (T(1) + std::sqrt(T(1) - s2));
          const T ct = T(1) - (T)u01(ra.y) * omc;
          const T st = std::sqrt(std::max(T(0), T(1) - ct * ct));
          T sp, cp;
          sincos_turns((T)u01(ra.z), &sp, &cp);
          wi = frame_dir(mul(wc, T(1) / std::sqrt(d2)), cp * st, sp * st, ct);
          const T b = dot(wc, wi);
          const T disc = b * b - (d2 - r2);
          dist = disc > T(0) ? b - std::sqrt(disc) : b;
          pdfw = T(1) / ((T(2) * T(kPi)) * omc);
          le = dist > T(0) ? (T)Lt.inten : T(0);
        }
      } else {
        const V<T> smp = xf<T>(Lt.m, mk<T>(0, (T)(u01(ra.y) - 0.5f), (T)(u01(ra.z) - 0.5f)));
        const V<T> ln = mk<T>(Lt.n[0], Lt.n[1], Lt.n[2]);
        T cosl = dot(normalize(sub(pos, smp)), ln);
        le = cosl < T(0) ? T(0) : (T)Lt.inten;
        cosl = cosl < T(0) ? T(0) : cosl;
        const V<T> tol = sub(smp, pos);
        wi = normalize(tol);
        dist = len(tol);
        pdfw = (dot(tol, tol) / cosl) / ((T)Lt.scale[0] * (T)Lt.scale[1]);
      }
      if (le > T(kEps)) {
        const Eval<T> e = evaluate(sh, colr, wi, wo, nrm);
        if (maxc(e.f) > T(kEps)) {
          const T a = pdfw * pick;
          const T mis = misw(a, e.pdf, S->mis_power);
          const T k0 = (mis * e.cs) / a;
          const V<T> c = mk(k0 * (le * e.f.x), k0 * (le * e.f.y), k0 * (le * e.f.z));
          cnt->shadow++;
          T st, su, sv;
          if (trace<T>(S, pos, wi, T(kTnear), dist, true, &st, &su, &sv) < 0) {
            L.x += c.x * w.x;
            L.y += c.y * w.y;
            L.z += c.z * w.z;
          }
        }
      }
    }
    if (!(depth < S->max_depth) || sh.type == NULLSH) break;  // Integrator.cpp:184-185
    T q = std::min(T(1), (T)sh.refl / (T)S->threshold);      // Integrator.cpp:187-191
    if (depth < S->min_depth) q = T(1);
    if ((T)u01(ra.w) > q) break;
    const U4 rb = pcg4d(sid, (uint32_t)depth + 1u, seed, 1u);
    T sp, cp;
    sincos_turns((T)u01(rb.x), &sp, &cp);
    V<T> wi;
    Eval<T> e;
    bool ok;
    if (sh.type == PHONG) {
      const T ca = pow_pos((T)u01(rb.y), T(1) / ((T)sh.ex + T(1)));
      const T sa = std::sqrt(std::max(T(0), T(1) - ca * ca));
      const V<T> rr = sub(mul(nrm, T(2) * dot(nrm, wo)), wo);
      wi = frame_dir(normalize(rr), cp * sa, sp * sa, ca);
      e = evaluate(sh, colr, wi, wo, nrm);
      ok = e.cs > T(0) && e.pdf > T(0);
    } else {  // LambertShader.cpp:49-73
      const T st = std::sqrt(T(1) - (T)u01(rb.y));
      const T ct2 = std::sqrt((T)u01(rb.y));
      wi = frame_dir(nrm, cp * st, sp * st, ct2);
      e.f = mul(mul(colr, (T)sh.refl), T(kInvPi));
      e.cs = dot(nrm, wi);
      e.pdf = e.cs * T(kInvPi);
      ok = e.pdf > T(0);
    }
    if (!ok) break;
    const T g0 = e.cs / e.pdf;
    w = mk(((w.x * e.f.x) * g0) / q, ((w.y * e.f.y) * g0) / q, ((w.z * e.f.z) * g0) / q);
    o = pos;
    d = wi;
    last_pdf = e.pdf;
    depth += 1;
  }
  rgb[0] = L.x;
  rgb[1] = L.y;
  rgb[2] = L.z;
}

// Paths [first, first + n); path sid writes rgb[3 * (sid - out_base)] and
// xy[2 * (sid - out_base)] when those are given.
template <class T>
void parallel_paths(oracle_scene* S, int iteration, int threads, uint64_t first, uint64_t n, T* rgb, T* xy, Counts* total,
                    uint64_t out_base = 0) {
  const uint32_t seed = iter_seed(S->seed, (uint32_t)iteration);
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<uint64_t> next(0);
  const uint64_t chunk = 1024;
  std::vector<Counts> cs((size_t)threads);
  auto work = [&](int tid) {
    T dummy_rgb[3], dummy_xy[2];
    while (true) {
      uint64_t b = next.fetch_add(chunk);
      if (b >= n) break;
      uint64_t e = std::min(n, b + chunk);
      for (uint64_t k = b; k < e; ++k) {
        uint64_t sid = first + k;
        const uint64_t o = sid - out_base;
        render_path<T>(S, (uint32_t)sid, seed, rgb ? rgb + 3 * o : dummy_rgb, xy ? xy + 2 * o : dummy_xy, &cs[tid]);
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
  for (auto& c : cs) { total->closest += c.closest; total->shadow += c.shadow; }
}

template <class T>
void filter_image(const oracle_scene* S, const T* rgb, const T* xy, T* pixels) {
  const int W = S->W, H = S->H, spp = S->spp;
  for (int x = 0; x < W; ++x)
    for (int y = 0; y < H; ++y) {
      T sr = 0, sg = 0, sb = 0;
      T* px = pixels + 3 * ((size_t)y * W + x);
      if (S->filter == 1) {  // BoxFilter.cpp:16-34
        size_t b = ((size_t)x * H + y) * spp;
        for (int s = 0; s < spp; ++s) { sr += rgb[3 * (b + s)]; sg += rgb[3 * (b + s) + 1]; sb += rgb[3 * (b + s) + 2]; }
        T ns = (T)spp;
        px[0] += sr / ns; px[1] += sg / ns; px[2] += sb / ns;
        continue;
      }
      // TentFilter.cpp:20-61
      const T cx = (T)x + T(0.5f), cy = (T)y + T(0.5f);
      T den = 0;
      for (int mx = -1; mx < 2; ++mx)
        for (int my = -1; my < 2; ++my) {
          int qx = x + mx, qy = y + my;
          if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
          size_t b = ((size_t)qx * H + qy) * spp;
          for (int s = 0; s < spp; ++s) {
            const T* p = xy + 2 * (b + s);
            const T* c = rgb + 3 * (b + s);
            T dx = std::max(T(0), T(1) - std::fabs(p[0] - cx));
            T dy = std::max(T(0), T(1) - std::fabs(p[1] - cy));
            T m = dx * dy;
            den = den + m;
            sr += c[0] * m;
            sg += c[1] * m;
            sb += c[2] * m;
          }
        }
      px[0] += sr / den; px[1] += sg / den; px[2] += sb / den;
    }
}

template <class T>
int render_full(oracle_scene* S, int iteration, int threads, T* rgb, T* xy, T* pixels, uint64_t* counts) {
  const uint64_t P = (uint64_t)S->W * S->H * S->spp;
  std::vector<T> r2, x2;
  if (!rgb) { r2.resize(P * 3); rgb = r2.data(); }
  if (!xy) { x2.resize(P * 2); xy = x2.data(); }
  Counts c;
  parallel_paths<T>(S, iteration, threads, 0, P, rgb, xy, &c);
  if (pixels) filter_image<T>(S, rgb, xy, pixels);
  if (counts) { counts[0] = c.closest; counts[1] = c.shadow; }
  return 0;
}

// Quantisation of the 32-bit origin/direction ray key (oracle_ray_keys), the
// device key's restatement.
uint32_t quant(float v, float lo, float sc, int cells) {
  int i = (int)std::floor((v - lo) * sc);
  return (uint32_t)std::min(std::max(i, 0), cells - 1);
}

}  // namespace orc

// ================================================================ C API
extern "C" {

oracle_scene* oracle_load(const char* yaml_path, char* err, int errcap) {
  oracle_scene* s = new oracle_scene();
  std::string e;
  if (!orc::load(yaml_path, s, &e)) {
    if (err && errcap > 0) snprintf(err, errcap, "%s", e.c_str());
    delete s;
    return nullptr;
  }
  if (s->tgeom.empty()) {
    if (err && errcap > 0) snprintf(err, errcap, "scene has no triangles");
    delete s;
    return nullptr;
  }
  orc::build_bvh(s);
  return s;
}

void oracle_free(oracle_scene* s) { delete s; }

void oracle_triangles(const oracle_scene* s, float* v9, int32_t* geom) {
  if (v9) memcpy(v9, s->tv.data(), s->tv.size() * sizeof(float));
  if (geom)
    for (size_t i = 0; i < s->tgeom.size(); ++i) geom[i] = s->tgeom[i];
}

int oracle_set_job(oracle_scene* s, int width, int height, int spp, int min_depth, int max_depth,
                   const float* cam_t, const float* cam_r, float focal, uint32_t seed) {
  if (width > 0) s->W = width;
  if (height > 0) s->H = height;
  if (spp > 0) {
    s->spp = spp;
    int a = 1;
    for (int d = 1; d * d <= spp; ++d)
      if (spp % d == 0) a = d;
    s->gx = a;
    s->gy = spp / a;
    if (a * a == spp) s->base = a;
  }
  if (min_depth >= 0) s->min_depth = min_depth;
  if (max_depth >= 0) s->max_depth = max_depth;
  if (cam_t && cam_r && focal > 0.f) {  // a pinhole camera (PinHoleCamera.cpp:5-14)
    s->cam_type = 0;
    s->cam = orc::tr_yxz(cam_t, cam_r);
    orc::x_normal(s->cam, s->cam_n);
    for (int i = 0; i < 3; ++i) s->cam_t[i] = cam_t[i];
    s->focal = focal;
  }
  s->seed = seed;
  return 0;
}

void oracle_info(const oracle_scene* s, int* o) {
  o[0] = s->W; o[1] = s->H; o[2] = s->spp; o[3] = (int)s->tgeom.size(); o[4] = (int)s->lights.size();
}

int oracle_render_f32(oracle_scene* s, int iteration, int threads, float* rgb, float* xy, float* pixels, uint64_t* counts) {
  return orc::render_full<float>(s, iteration, threads, rgb, xy, pixels, counts);
}
int oracle_render_f64(oracle_scene* s, int iteration, int threads, double* rgb, double* xy, double* pixels, uint64_t* counts) {
  return orc::render_full<double>(s, iteration, threads, rgb, xy, pixels, counts);
}
int oracle_render_range_f32(oracle_scene* s, int iteration, int threads, uint64_t first, uint64_t n, uint64_t* counts) {
  orc::Counts c;
  orc::parallel_paths<float>(s, iteration, threads, first, n, nullptr, nullptr, &c);
  if (counts) { counts[0] = c.closest; counts[1] = c.shadow; }
  return 0;
}

int oracle_render_range_rgb_f32(oracle_scene* s, int iteration, int threads, uint64_t first, uint64_t n, float* rgb,
                                float* xy, uint64_t* counts) {
  orc::Counts c;
  orc::parallel_paths<float>(s, iteration, threads, first, n, rgb, xy, &c, first);
  if (counts) { counts[0] = c.closest; counts[1] = c.shadow; }
  return 0;
}

int oracle_trace_f32(const oracle_scene* s, const float* org, const float* dir, int n, float* t, float* u, float* v,
                     int32_t* geom, int32_t* prim) {
  for (int i = 0; i < n; ++i) {
    orc::V<float> o = orc::mk(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
    orc::V<float> d = orc::mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
    float th = orc::kTfar, uh = 0, vh = 0;
    int tri = orc::trace<float>(s, o, d, orc::kTnear, orc::kTfar, false, &th, &uh, &vh);
    if (tri < 0) { t[i] = orc::kTfar; u[i] = 0; v[i] = 0; geom[i] = -1; prim[i] = -1; continue; }
    t[i] = th; u[i] = uh; v[i] = vh;
    geom[i] = s->tgeom[tri];
    prim[i] = tri - s->geoms[geom[i]].first;
  }
  return 0;
}

int oracle_occluded_f32(const oracle_scene* s, const float* org, const float* dir, const float* tmax, int n,
                        int32_t* occ) {
  for (int i = 0; i < n; ++i) {
    orc::V<float> o = orc::mk(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
    orc::V<float> d = orc::mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
    float a, b, c;
    occ[i] = orc::trace<float>(s, o, d, orc::kTnear, tmax[i], true, &a, &b, &c) >= 0 ? 1 : 0;
  }
  return 0;
}

void oracle_cardinal(const float* dirs, int n, int32_t* bins) {
  for (int i = 0; i < n; ++i) bins[i] = orc::cardinal(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
}

void oracle_ray_keys(const float* org, const float* dir, int n, uint32_t* keys) {
  if (n <= 0) return;
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) { lo[a] = org[a]; hi[a] = org[a]; }
  for (int i = 0; i < n; ++i)  // RayBoundingbox.cpp:10-35
    for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], org[3 * i + a]); hi[a] = std::max(hi[a], org[3 * i + a]); }
  float sc[3];
  for (int a = 0; a < 3; ++a) { float e = hi[a] - lo[a]; sc[a] = e > 0.f ? 64.0f / e : 0.f; }
  for (int i = 0; i < n; ++i) {
    const float* o = org + 3 * i;
    const float* d = dir + 3 * i;
    // five-dimensional Morton code, six levels of (x, y, z, u, v) bits from the
    // top, then the finest u, v bits
    const uint32_t q[3] = {orc::quant(o[0], lo[0], sc[0], 64), orc::quant(o[1], lo[1], sc[1], 64),
                           orc::quant(o[2], lo[2], sc[2], 64)};
    int c = orc::cardinal(d[0], d[1], d[2]) % 3;
    float da = d[c], du = d[(c + 1) % 3], dv = d[(c + 2) % 3];
    float inv = 1.0f / std::fabs(da);
    uint32_t qu = orc::quant(du * inv, -1.0f, 64.0f, 128), qv = orc::quant(dv * inv, -1.0f, 64.0f, 128);
    uint32_t key = 0;
    for (int l = 0; l < 6; ++l) {
      for (int a = 0; a < 3; ++a) key = (key << 1) | ((q[a] >> (5 - l)) & 1u);
      key = (key << 1) | ((qu >> (6 - l)) & 1u);
      key = (key << 1) | ((qv >> (6 - l)) & 1u);
    }
    keys[i] = (key << 2) | ((qu & 1u) << 1) | (qv & 1u);
  }
}

void oracle_stable_sort_pairs(uint32_t* keys, uint32_t* vals, int n, int bits) {
  const uint32_t mask = bits >= 32 ? 0xffffffffu : ((1u << bits) - 1u);
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return (keys[a] & mask) < (keys[b] & mask); });
  std::vector<uint32_t> k2(n), v2(n);
  for (int i = 0; i < n; ++i) { k2[i] = keys[idx[i]]; v2[i] = vals[idx[i]]; }
  memcpy(keys, k2.data(), (size_t)n * 4);
  memcpy(vals, v2.data(), (size_t)n * 4);
}

// The reference's ray order within a batch, RaySort::operator() of
// src/core/RaySort.cpp:7-118 after RayBoundingbox (src/core/RayBoundingbox.cpp:5-50):
// a range of more than 4096 rays is sorted by origin along the widest axis of
// its box and halved at the middle; a half of more than 4096 rays keeps the box
// cut at the median origin, a smaller half takes the box of its directions; a
// range of 65..4096 rays is sorted by direction along the widest axis of its
// (direction) box and halved, the halves keeping the parent's box except for
// the first half's bound, as the reference sets it (its second half keeps the
// parent's box unchanged).  Ranges of 64 rays or fewer stay as they are.  The
// reference's tbb::parallel_sort is not stable; std::stable_sort here fixes
// the order among equal coordinates.  Coherence comparisons only.
namespace orc {
struct Box3 { float lo[3], hi[3]; };
int widest(const Box3& b) {
  int t = (b.hi[0] - b.lo[0]) < (b.hi[1] - b.lo[1]) ? 1 : 0;
  return (t < (b.hi[2] - b.lo[2])) ? 2 : t;  // the reference compares the index with the extent
}
void median_split(const float* org, const float* dir, uint32_t* ix, size_t b, size_t e, Box3 lim) {
  const size_t size = e - b;
  if (size > 4096) {
    const int axis = widest(lim);
    std::stable_sort(ix + b, ix + e, [&](uint32_t x, uint32_t y) { return org[3 * x + axis] < org[3 * y + axis]; });
    const size_t mid = b + size / 2;
    Box3 l, r;
    auto dir_box = [&](size_t s0, size_t s1, Box3* o) {
      for (int a = 0; a < 3; ++a) o->lo[a] = o->hi[a] = dir[3 * ix[s0] + a];
      for (size_t k = s0; k < s1; ++k)
        for (int a = 0; a < 3; ++a) {
          const float v = dir[3 * ix[k] + a];
          if (v < o->lo[a]) o->lo[a] = v;
          if (v > o->hi[a]) o->hi[a] = v;
        }
    };
    if (mid - b > 4096) { l = lim; l.hi[axis] = org[3 * ix[mid - 1] + axis]; }
    else dir_box(b, mid, &l);
    if (e - mid > 4096) { r = lim; r.lo[axis] = org[3 * ix[mid] + axis]; }
    else dir_box(mid, e, &r);
    median_split(org, dir, ix, b, mid, l);
    median_split(org, dir, ix, mid, e, r);
  } else if (size > 64) {
    const int axis = widest(lim);
    std::stable_sort(ix + b, ix + e, [&](uint32_t x, uint32_t y) { return dir[3 * x + axis] < dir[3 * y + axis]; });
    const size_t mid = b + size / 2;
    Box3 l = lim, r = lim;
    l.hi[axis] = dir[3 * ix[mid - 1] + axis];
    l.lo[axis] = dir[3 * ix[mid] + axis];
    median_split(org, dir, ix, b, mid, l);
    median_split(org, dir, ix, mid, e, r);
  }
}
}  // namespace orc

void oracle_median_split_order(const float* org, const float* dir, int n, uint32_t* order) {
  for (int i = 0; i < n; ++i) order[i] = (uint32_t)i;
  if (n <= 0) return;
  orc::Box3 lim;  // RayBoundingbox: the batch's origin box
  for (int a = 0; a < 3; ++a) lim.lo[a] = lim.hi[a] = org[a];
  for (int i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      lim.lo[a] = std::min(lim.lo[a], org[3 * i + a]);
      lim.hi[a] = std::max(lim.hi[a], org[3 * i + a]);
    }
  orc::median_split(org, dir, order, 0, (size_t)n, lim);
}

// 26 / 98 bins (extension, no reference counterpart): the surface cells of
// an m^3 cube over [-1,1]^3 (m = 3 or 5), the direction scaled so its largest
// component has magnitude 1; cells in x-major order, interior cells skipped.
int orc_ray_bin(float x, float y, float z, int nbins) {
  if (nbins == 6) return orc::cardinal(x, y, z);
  const int m = nbins == 26 ? 3 : 5;
  const float mx = std::max(std::max(std::fabs(x), std::fabs(y)), std::fabs(z));
  if (!(mx > 0.f)) return 0;
  const float inv = 1.0f / mx;
  const float half_m = 0.5f * (float)m;
  const float v[3] = {x * inv, y * inv, z * inv};
  int c[3];
  for (int a = 0; a < 3; ++a) c[a] = std::min(m - 1, std::max(0, (int)std::floor((v[a] + 1.0f) * half_m)));
  const int n_in = m - 2;
  int interior_before = 0;  // interior cells (all coordinates in [1, m-2]) with a smaller index
  for (int i = 1; i <= m - 2; ++i)
    for (int j = 1; j <= m - 2; ++j)
      for (int k = 1; k <= m - 2; ++k)
        if ((i * m + j) * m + k < (c[0] * m + c[1]) * m + c[2]) ++interior_before;
  (void)n_in;
  return (c[0] * m + c[1]) * m + c[2] - interior_before;
}

int oracle_image_lookup(const char* path, int n, const float* s, const float* t, float* rgb) {
  OImage im;
  if (!read_image(path, &im)) return -1;
  for (int i = 0; i < n; ++i) image_lookup(im, s[i], t[i], rgb + 3 * i);
  return 0;
}

void oracle_ray_bins(const float* dirs, int n, int nbins, int32_t* bins) {
  for (int i = 0; i < n; ++i) bins[i] = orc_ray_bin(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2], nbins);
}

void oracle_bin_partition_n(const float* rays, int n, int nbins, int cap, float* out, int32_t* counts) {
  for (int b = 0; b < nbins; ++b) counts[b] = 0;
  memset(out, 0, sizeof(float) * 12 * (size_t)nbins * (size_t)cap);
  for (int i = 0; i < n; ++i) {
    const float* r = rays + 12 * i;
    int32_t depth;
    memcpy(&depth, &r[7], 4);
    if (depth < 0) continue;
    int b = orc_ray_bin(r[4], r[5], r[6], nbins);
    if (counts[b] >= cap) continue;
    memcpy(out + 12 * ((size_t)b * cap + counts[b]), r, 48);
    counts[b]++;
  }
}

void oracle_bin_partition(const float* rays, int n, int cap, float* out, int32_t* counts) {
  oracle_bin_partition_n(rays, n, 6, cap, out, counts);
}

void oracle_tent_filter(const float* rgb, const float* xy, int w, int h, int spp, float* pixels) {
  oracle_scene s;
  s.W = w; s.H = h; s.spp = spp; s.filter = 0;
  orc::filter_image<float>(&s, rgb, xy, pixels);
}

int oracle_obj_load(const char* path, float* positions, float* texcoords, uint32_t* indices, int64_t* sizes) {
  orc::Obj o;
  if (!orc::load_obj(path, &o)) return -1;
  sizes[0] = (int64_t)o.pos.size();
  sizes[1] = (int64_t)o.tex.size();
  sizes[2] = (int64_t)o.idx.size();
  if (positions) memcpy(positions, o.pos.data(), o.pos.size() * 4);
  if (texcoords) memcpy(texcoords, o.tex.data(), o.tex.size() * 4);
  if (indices) memcpy(indices, o.idx.data(), o.idx.size() * 4);
  return 0;
}

}  // extern "C"
