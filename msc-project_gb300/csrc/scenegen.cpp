// Seeded synthetic scenes written as YAML + OBJ in the reference's scene
// schema (src/core/Pathtracer.cpp:32-275), so the reference renderer and this
// one read identical inputs.  No public benchmark scene exists for the
// reference; these stand in for it.
//
//   config 0  Cornell-style box: 5 wall quads, two rotated boxes, one
//             subdivision-3 icosphere (1280 tris), one quad light of
//             radiance 15; Lambert albedos U[0.2,0.8]^3; 40 degree pinhole;
//             256x256, 16 spp, max depth 4, batch 2^16.
//   config 1  terrain of 1024x1024 quads displaced by 5-octave value noise,
//             300 instances of a subdivision-4 icosphere, 4 Lambert + 4 Phong
//             shaders, 8 quad lights; 1024x1024, 64 spp, max depth 8,
//             Russian roulette from depth 3, batch 2^20, power heuristic.
//   config 2  hit-sort stress: 2000 randomly placed subdivided tori of 4000
//             triangles each (8 M triangles, every torus two 2000-triangle
//             halves with their own shader), a floor quad, 4096 shader ids
//             (Lambert and Phong) whose texture is per-face 16x16 FP16 RGB
//             texels from the seed, 64 sphere lights of log-uniform power;
//             1024x1024, 32 spp (4 x 8 grid), max depth 6, 64-bit hit key.
//   config 100 a tiny box scene for tests.
// `scale` in (0,1] shrinks resolution (and for config 1 the geometry).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <vector>
#include <sys/stat.h>

#include "scene.h"

namespace mscg {

namespace {

struct V3 { double x, y, z; };
V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 mul(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
V3 nrm(V3 a) { double l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); return mul(a, 1.0 / l); }

struct ObjWriter {
  std::string text;
  int nv = 0;
  char buf[160];
  int vertex(V3 p, double u, double v) {
    int n = snprintf(buf, sizeof(buf), "v %.6f %.6f %.6f\nvt %.6f %.6f\n", p.x, p.y, p.z, u, v);
    text.append(buf, n);
    return ++nv;
  }
  void tri(int a, int b, int c) {
    int n = snprintf(buf, sizeof(buf), "f %d/%d %d/%d %d/%d\n", a, a, b, b, c, c);
    text.append(buf, n);
  }
  void quad(int a, int b, int c, int d) {
    int n = snprintf(buf, sizeof(buf), "f %d/%d %d/%d %d/%d %d/%d\n", a, a, b, b, c, c, d, d);
    text.append(buf, n);
  }
  // quad centred at c spanning +-u, +-v; normal = u x v
  void quad_uv(V3 c, V3 u, V3 v) {
    int a = vertex(sub(sub(c, u), v), 0, 0);
    int b = vertex(sub(add(c, u), v), 1, 0);
    int e = vertex(add(add(c, u), v), 1, 1);
    int d = vertex(add(sub(c, u), v), 0, 1);
    quad(a, b, e, d);
  }
  bool save(const std::string& path) const {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) return false;
    size_t w = fwrite(text.data(), 1, text.size(), f);
    fclose(f);
    return w == text.size();
  }
};

// Unit cube [-0.5,0.5]^3 with outward normals.
void write_cube(ObjWriter& o) {
  const V3 X{0.5, 0, 0}, Y{0, 0.5, 0}, Z{0, 0, 0.5};
  o.quad_uv(X, Y, Z);              // +x: y x z = +x
  o.quad_uv(mul(X, -1), Z, Y);     // -x
  o.quad_uv(Y, Z, X);              // +y: z x x = +y
  o.quad_uv(mul(Y, -1), X, Z);     // -y
  o.quad_uv(Z, X, Y);              // +z: x x y = +z
  o.quad_uv(mul(Z, -1), Y, X);     // -z
}

// Unit icosphere with `sub` subdivisions (20 * 4^sub faces), outward winding,
// spherical uv.
void write_icosphere(ObjWriter& o, int sub) {
  const double t = (1.0 + std::sqrt(5.0)) / 2.0;
  std::vector<V3> v = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                       {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
  for (auto& p : v) p = nrm(p);
  std::vector<int> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6,
                        7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7,
                        9, 8, 1};
  for (int s = 0; s < sub; ++s) {
    std::vector<int> nf;
    std::map<uint64_t, int> cache;
    auto mid = [&](int a, int b) {
      uint64_t key = a < b ? ((uint64_t)a << 32 | (uint32_t)b) : ((uint64_t)b << 32 | (uint32_t)a);
      auto it = cache.find(key);
      if (it != cache.end()) return it->second;
      v.push_back(nrm(mul(add(v[a], v[b]), 0.5)));
      cache[key] = (int)v.size() - 1;
      return (int)v.size() - 1;
    };
    for (size_t i = 0; i < f.size(); i += 3) {
      int a = f[i], b = f[i + 1], c = f[i + 2];
      int ab = mid(a, b), bc = mid(b, c), ca = mid(c, a);
      int q[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
      nf.insert(nf.end(), q, q + 12);
    }
    f.swap(nf);
  }
  int base = o.nv;
  for (auto& p : v) {
    double u = 0.5 + std::atan2(p.z, p.x) / (2 * M_PI);
    double w = 0.5 - std::asin(std::max(-1.0, std::min(1.0, p.y))) / M_PI;
    o.vertex(p, u, w);
  }
  for (size_t i = 0; i < f.size(); i += 3) o.tri(base + f[i] + 1, base + f[i + 1] + 1, base + f[i + 2] + 1);
}

struct Noise {  // value noise on an integer lattice, smoothstep interpolation
  std::vector<float> lat;
  int n = 256;
  explicit Noise(std::mt19937_64& rng) : lat(256 * 256) {
    std::uniform_real_distribution<float> U(0.f, 1.f);
    for (auto& x : lat) x = U(rng);
  }
  float at(int i, int j) const { return lat[((i & 255) << 8) | (j & 255)]; }
  float eval(double x, double y) const {
    double fx = std::floor(x), fy = std::floor(y);
    int i = (int)fx, j = (int)fy;
    double tx = x - fx, ty = y - fy;
    tx = tx * tx * (3 - 2 * tx);
    ty = ty * ty * (3 - 2 * ty);
    double a = at(i, j) + (at(i + 1, j) - at(i, j)) * tx;
    double b = at(i, j + 1) + (at(i + 1, j + 1) - at(i, j + 1)) * tx;
    return (float)(a + (b - a) * ty);
  }
  float fbm(double x, double y, int oct) const {
    double s = 0, amp = 0.5, f = 1;
    for (int o = 0; o < oct; ++o) { s += amp * eval(x * f, y * f); amp *= 0.5; f *= 2; }
    return (float)s;
  }
};

std::string fmt(const char* f, double a) { char b[64]; snprintf(b, sizeof(b), f, a); return b; }
std::string vec3s(double a, double b, double c) {
  char buf[128];
  snprintf(buf, sizeof(buf), "[%.6f, %.6f, %.6f]", a, b, c);
  return buf;
}

// The reference's pinhole sits at translation + normal * focal length
// (PinHoleCamera.cpp:18), so the translation is placed one focal length
// behind the wanted eye point along the view normal R * X, R = Ry Rx Rz.
V3 camera_translation(V3 eye, V3 r_deg, double focal) {
  const double d2r = M_PI / 180.0;
  double rx = r_deg.x * d2r, ry = r_deg.y * d2r, rz = r_deg.z * d2r;
  V3 v{std::cos(rz), std::sin(rz), 0.0};
  v = {v.x, v.y * std::cos(rx) - v.z * std::sin(rx), v.y * std::sin(rx) + v.z * std::cos(rx)};
  v = {v.x * std::cos(ry) + v.z * std::sin(ry), v.y, -v.x * std::sin(ry) + v.z * std::cos(ry)};
  return sub(eye, mul(v, focal));
}

std::string setup_doc(int w, int h, int base, int mind, int maxd, double thr, int binexp, V3 eye, V3 cam_r,
                      double focal) {
  std::string s;
  V3 cam_t = camera_translation(eye, cam_r, focal);
  s += "# setup\nimage:\n  width: " + std::to_string(w) + "\n  height: " + std::to_string(h) +
       "\n  sample base: " + std::to_string(base) + "\n";
  s += "settings:\n  min depth: " + std::to_string(mind) + "\n  max depth: " + std::to_string(maxd) +
       "\n  threshold: " + fmt("%g", thr) + "\n  bucket size: 16\n  shading size: 4096\n  bin exponent: " +
       std::to_string(binexp) + "\n";
  s += "camera:\n  type: PinHole\n  translation: " + vec3s(cam_t.x, cam_t.y, cam_t.z) +
       "\n  rotation: " + vec3s(cam_r.x, cam_r.y, cam_r.z) + "\n  focal length: " + fmt("%.6f", focal) + "\n";
  s += "filter:\n  type: Tent\nsampler:\n  type: Stratified\n";
  return s;
}

std::string lambert(double r, double g, double b, double refl) {
  return "shader:\n  type: Lambert\n  texture:\n    type: Constant\n    colour: " + vec3s(r, g, b) +
         "\n  reflectance: " + fmt("%.6f", refl) + "\n";
}
std::string phong(double r, double g, double b, double refl, double ex) {
  return "shader:\n  type: Phong\n  texture:\n    type: Constant\n    colour: " + vec3s(r, g, b) +
         "\n  reflectance: " + fmt("%.6f", refl) + "\n  exponent: " + fmt("%.6f", ex) + "\n";
}
std::string object(const std::string& file, V3 t, V3 r, V3 s, int shader) {
  return "object:\n  type: Polygon\n  filename: " + file + "\n  translation: " + vec3s(t.x, t.y, t.z) +
         "\n  rotation: " + vec3s(r.x, r.y, r.z) + "\n  scale: " + vec3s(s.x, s.y, s.z) +
         "\n  shader: " + std::to_string(shader) + "\n";
}
std::string quad_light(V3 t, V3 r, double sx, double sy, double inten) {
  char buf[64];
  snprintf(buf, sizeof(buf), "[%.6f, %.6f]", sx, sy);
  return "light:\n  type: Quad\n  translation: " + vec3s(t.x, t.y, t.z) + "\n  rotation: " + vec3s(r.x, r.y, r.z) +
         "\n  scale: " + buf + "\n  intensity: " + fmt("%.6f", inten) + "\n";
}

std::string face_texel_shader(bool glossy, double r, double g, double b, double refl, double ex, int res,
                              uint32_t seed) {
  std::string tex = "  texture:\n    type: FaceTexels\n    resolution: " + std::to_string(res) +
                    "\n    seed: " + std::to_string(seed) + "\n    colour: " + vec3s(r, g, b) + "\n";
  if (!glossy) return "shader:\n  type: Lambert\n" + tex + "  reflectance: " + fmt("%.6f", refl) + "\n";
  return "shader:\n  type: Phong\n" + tex + "  reflectance: " + fmt("%.6f", refl) + "\n  exponent: " +
         fmt("%.6f", ex) + "\n";
}
std::string sphere_light(V3 c, double radius, double inten) {
  return "light:\n  type: Sphere\n  translation: " + vec3s(c.x, c.y, c.z) + "\n  radius: " + fmt("%.6f", radius) +
         "\n  intensity: " + fmt("%.6f", inten) + "\n";
}

// Half of a torus of ring radius 1 and tube radius `tube`: the tube angle
// runs over [half * pi, (half + 1) * pi); 50 x 20 quads = 2000 triangles,
// outward winding.
void write_torus_half(ObjWriter& o, double tube, int half) {
  const int NU = 50, NV = 20;
  const int base = o.nv;
  for (int i = 0; i <= NU; ++i)
    for (int j = 0; j <= NV; ++j) {
      const double u = 2.0 * M_PI * i / NU, v = M_PI * (half + (double)j / NV);
      const double rr = 1.0 + tube * std::cos(v);
      o.vertex({rr * std::cos(u), tube * std::sin(v), rr * std::sin(u)}, (double)i / NU, (double)j / NV);
    }
  for (int i = 0; i < NU; ++i)
    for (int j = 0; j < NV; ++j) {
      const int a = base + i * (NV + 1) + j + 1;  // (i, j)
      const int b = a + 1;                        // (i, j+1): along the tube first
      const int c = a + (NV + 1) + 1;             // (i+1, j+1)
      const int d = a + (NV + 1);                 // (i+1, j)
      o.quad(a, b, c, d);
    }
}

bool write_text(const std::string& path, const std::string& s) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return false;
  size_t w = fwrite(s.data(), 1, s.size(), f);
  fclose(f);
  return w == s.size();
}

int scaled(int v, double scale, int lo) { int r = (int)std::lround(v * scale); return r < lo ? lo : r; }

bool gen_box(uint32_t seed, double scale, const std::string& dir, bool tiny, std::string* yaml) {
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  auto alb = [&]() { return 0.2 + 0.6 * U(rng); };
  std::string scene;
  // walls: floor, ceiling, back, left, right with inward normals
  struct Wall { const char* name; V3 c, u, v; };
  Wall walls[5] = {{"floor.obj", {0, 0, 0}, {0, 0, 1}, {1, 0, 0}},      // z x x = +y
                   {"ceiling.obj", {0, 2, 0}, {1, 0, 0}, {0, 0, 1}},    // x x z = -y
                   {"back.obj", {0, 1, -1}, {1, 0, 0}, {0, 1, 0}},      // x x y = +z
                   {"left.obj", {-1, 1, 0}, {0, 1, 0}, {0, 0, 1}},      // y x z = +x
                   {"right.obj", {1, 1, 0}, {0, 0, 1}, {0, 1, 0}}};     // z x y = -x
  int shader = 0;
  for (auto& w : walls) {
    ObjWriter o;
    o.quad_uv(w.c, w.u, w.v);
    if (!o.save(dir + "/" + w.name)) return false;
    scene += lambert(alb(), alb(), alb(), 1.0);
    scene += object(w.name, {0, 0, 0}, {0, 0, 0}, {1, 1, 1}, shader++);
  }
  ObjWriter cube;
  write_cube(cube);
  if (!cube.save(dir + "/box.obj")) return false;
  for (int b = 0; b < 2; ++b) {
    double sx = 0.3 + 0.4 * U(rng), sy = 0.3 + 0.9 * U(rng), sz = 0.3 + 0.4 * U(rng);
    double px = (b == 0 ? -0.45 : 0.45) + 0.1 * (U(rng) - 0.5), pz = -0.3 + 0.4 * U(rng);
    double yaw = 360.0 * U(rng);
    scene += lambert(alb(), alb(), alb(), 1.0);
    scene += object("box.obj", {px, sy * 0.5, pz}, {0, yaw, 0}, {sx, sy, sz}, shader++);
  }
  ObjWriter ico;
  write_icosphere(ico, tiny ? 1 : 3);
  if (!ico.save(dir + "/icosphere.obj")) return false;
  {
    double r = 0.25 + 0.1 * U(rng);
    scene += lambert(alb(), alb(), alb(), 1.0);
    scene += object("icosphere.obj", {0.05, 1.2 + 0.3 * U(rng), 0.2}, {0, 0, 0}, {r, r, r}, shader++);
  }
  scene += quad_light({0, 1.99, 0}, {0, 0, -90}, 0.5, 0.5, 15.0);
  const double focal = 36.0 / std::tan(20.0 * M_PI / 180.0);  // 40 degree field of view
  int res = tiny ? scaled(32, scale, 4) : scaled(256, scale, 4);
  int base = tiny ? 2 : 4;
  int depth = tiny ? 3 : 4;
  std::string setup = setup_doc(res, res, base, depth, depth, 0.01, tiny ? 10 : 16, {0, 1, 3.75}, {0, 90, 0}, focal);
  std::string ext = "extensions:\n  mis: balance\n  seed: " + std::to_string(seed) + "\n";
  *yaml = dir + "/scene.yaml";
  return write_text(*yaml, setup + "---\n" + scene + "---\n" + ext);
}

bool gen_terrain(uint32_t seed, double scale, const std::string& dir, std::string* yaml) {
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  Noise noise(rng);
  const int N = scaled(1024, scale, 8);           // quads per side
  const int spheres = scaled(300, scale, 4);
  const double size = 200.0, hscale = 30.0;
  auto height = [&](double x, double z) {
    return hscale * (noise.fbm((x / size + 0.5) * 8.0, (z / size + 0.5) * 8.0, 5) - 0.5);
  };
  {
    ObjWriter o;
    o.text.reserve((size_t)(N + 1) * (N + 1) * 60 + (size_t)N * N * 50);
    for (int i = 0; i <= N; ++i)
      for (int j = 0; j <= N; ++j) {
        double x = ((double)i / N - 0.5) * size, z = ((double)j / N - 0.5) * size;
        o.vertex({x, height(x, z), z}, (double)i / N, (double)j / N);
      }
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        int a = i * (N + 1) + j + 1;
        int b = a + 1;
        int c = a + (N + 1) + 1;
        int d = a + (N + 1);
        o.quad(a, b, c, d);  // (0,0,dz) x (dx,0,dz) = +y
      }
    if (!o.save(dir + "/terrain.obj")) return false;
  }
  ObjWriter ico;
  write_icosphere(ico, 4);
  if (!ico.save(dir + "/icosphere.obj")) return false;
  std::string scene;
  for (int s = 0; s < 4; ++s) scene += lambert(0.2 + 0.6 * U(rng), 0.2 + 0.6 * U(rng), 0.2 + 0.6 * U(rng), 0.9);
  for (int s = 0; s < 4; ++s)
    scene += phong(0.2 + 0.6 * U(rng), 0.2 + 0.6 * U(rng), 0.2 + 0.6 * U(rng), 0.9, 10.0 + 190.0 * U(rng));
  scene += object("terrain.obj", {0, 0, 0}, {0, 0, 0}, {1, 1, 1}, 0);
  for (int k = 0; k < spheres; ++k) {
    double x = (U(rng) - 0.5) * size * 0.9, z = (U(rng) - 0.5) * size * 0.9;
    double r = 0.5 + 3.5 * U(rng);
    double y = height(x, z) + r * (0.3 + 0.9 * U(rng));
    int sh = (int)(U(rng) * 8) % 8;
    scene += object("icosphere.obj", {x, y, z}, {0, 0, 0}, {r, r, r}, sh);
  }
  for (int l = 0; l < 8; ++l) {
    double x = (U(rng) - 0.5) * size * 0.8, z = (U(rng) - 0.5) * size * 0.8;
    double s = 8.0 + 10.0 * U(rng);
    scene += quad_light({x, 45.0 + 20.0 * U(rng), z}, {0, 360.0 * U(rng), -90}, s, s, 60.0 + 60.0 * U(rng));
  }
  const double focal = 36.0 / std::tan(30.0 * M_PI / 180.0);  // 60 degree field of view
  int res = scaled(1024, scale, 8);
  int base = scale < 1.0 ? 2 : 8;
  std::string setup = setup_doc(res, res, base, 3, 8, 1.0, 20, {0, 60, 150}, {0, 90, -25}, focal);
  std::string ext = "extensions:\n  mis: power\n  seed: " + std::to_string(seed) + "\n";
  *yaml = dir + "/scene.yaml";
  return write_text(*yaml, setup + "---\n" + scene + "---\n" + ext);
}

bool gen_stress(uint32_t seed, double scale, const std::string& dir, std::string* yaml) {
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  const int kShapes = 8;
  double tubes[kShapes];
  for (int k = 0; k < kShapes; ++k) {
    tubes[k] = 0.2 + 0.3 * U(rng);
    for (int h = 0; h < 2; ++h) {
      ObjWriter o;
      write_torus_half(o, tubes[k], h);
      if (!o.save(dir + "/torus" + std::to_string(k) + "_" + std::to_string(h) + ".obj")) return false;
    }
  }
  {
    ObjWriter o;
    o.quad_uv({0, 0, 0}, {0, 0, 120}, {120, 0, 0});  // z x x = +y
    if (!o.save(dir + "/floor.obj")) return false;
  }
  const int kShaders = 4096, res = 16;
  std::string scene;
  for (int s = 0; s < kShaders; ++s) {
    const bool glossy = (s & 1) != 0;
    scene += face_texel_shader(glossy, 0.4 + 0.6 * U(rng), 0.4 + 0.6 * U(rng), 0.4 + 0.6 * U(rng), 0.9,
                               10.0 + 190.0 * U(rng), res, seed);
  }
  scene += object("floor.obj", {0, 0, 0}, {0, 0, 0}, {1, 1, 1}, kShaders - 1);
  const int meshes = scaled(2000, scale, 4);
  for (int m = 0; m < meshes; ++m) {
    const int k = (int)(U(rng) * kShapes) % kShapes;
    const double r = 1.0 + 2.0 * U(rng);
    const V3 t{(U(rng) - 0.5) * 120.0, r * (1.0 + tubes[k]) + 40.0 * U(rng), (U(rng) - 0.5) * 120.0};
    const V3 rot{360.0 * U(rng), 360.0 * U(rng), 360.0 * U(rng)};
    for (int h = 0; h < 2; ++h)
      scene += object("torus" + std::to_string(k) + "_" + std::to_string(h) + ".obj", t, rot, {r, r, r},
                      (2 * m + h) % (kShaders - 1));
  }
  const int lights = scaled(64, scale, 2);
  for (int l = 0; l < lights; ++l) {
    const double radius = 0.5 + U(rng);
    const double power = std::exp(std::log(1.0e2) + (std::log(1.0e4) - std::log(1.0e2)) * U(rng));
    const double inten = power / (4.0 * M_PI * M_PI * radius * radius);  // radiance of a uniform sphere emitter
    scene += sphere_light({(U(rng) - 0.5) * 110.0, 20.0 + 45.0 * U(rng), (U(rng) - 0.5) * 110.0}, radius, inten);
  }
  const double focal = 36.0 / std::tan(30.0 * M_PI / 180.0);  // 60 degree field of view
  const int img = scaled(1024, scale, 8);
  const int spp = scale < 1.0 ? 2 : 32;
  std::string setup = setup_doc(img, img, 8, 3, 6, 1.0, 20, {0, 45, 110}, {0, 90, -18}, focal);
  std::string ext = "extensions:\n  mis: power\n  seed: " + std::to_string(seed) +
                    "\n  samples per pixel: " + std::to_string(spp) + "\n  hit key bits: 64\n";
  *yaml = dir + "/scene.yaml";
  return write_text(*yaml, setup + "---\n" + scene + "---\n" + ext);
}

}  // namespace

bool generate_scene(int config, uint32_t seed, double scale, const std::string& dir, std::string* yaml,
                    std::string* err) {
  mkdir(dir.c_str(), 0755);
  if (!(scale > 0.0 && scale <= 1.0)) { *err = "scale must lie in (0, 1]"; return false; }
  bool ok = false;
  if (config == 0) ok = gen_box(seed, scale, dir, false, yaml);
  else if (config == 100) ok = gen_box(seed, scale, dir, true, yaml);
  else if (config == 1) ok = gen_terrain(seed, scale, dir, yaml);
  else if (config == 2) ok = gen_stress(seed, scale, dir, yaml);
  else { *err = "unknown scene config " + std::to_string(config); return false; }
  if (!ok) *err = "could not write the scene files into " + dir;
  return ok;
}

}  // namespace mscg
