// Image output for the headless path: the reference writes the accumulated
// image as an RGBA half-float OpenEXR file (src/main.cpp:199-213, alpha 1).
// OpenEXR is not available here, so this writes that file layout directly
// from the public format description: a single-part scanline image,
// uncompressed, channels A,B,G,R (alphabetical) of HALF, one scanline per
// block, plus the offset table.  PFM (portable float map) is also offered.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace mscg {

// float -> IEEE binary16 with round-to-nearest-even, overflow to infinity.
uint16_t float_to_half(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t mag = x & 0x7fffffffu;
  if (mag >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (mag > 0x7f800000u ? 0x200u : 0u));  // inf / nan
  if (mag >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // rounds past 65504
  if (mag < 0x38800000u) {  // subnormal half (or zero)
    if (mag < 0x33000000u) return (uint16_t)sign;
    uint32_t m = (mag & 0x7fffffu) | 0x800000u;
    int shift = 126 - (int)(mag >> 23);  // 14..24
    uint32_t h = m >> shift;
    uint32_t rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1);
    if (rem > half || (rem == half && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
  }
  uint32_t h = ((mag >> 13) - ((127u - 15u) << 10));
  uint32_t rem = mag & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
  return (uint16_t)(sign | h);
}

namespace {

void put_u32(std::string& s, uint32_t v) { for (int i = 0; i < 4; ++i) s.push_back((char)((v >> (8 * i)) & 0xff)); }
void put_i32(std::string& s, int32_t v) { put_u32(s, (uint32_t)v); }
void put_u64(std::string& s, uint64_t v) { for (int i = 0; i < 8; ++i) s.push_back((char)((v >> (8 * i)) & 0xff)); }
void put_f32(std::string& s, float f) { uint32_t v; memcpy(&v, &f, 4); put_u32(s, v); }
void attr(std::string& s, const char* name, const char* type, const std::string& value) {
  s.append(name); s.push_back('\0');
  s.append(type); s.push_back('\0');
  put_i32(s, (int32_t)value.size());
  s.append(value);
}

}  // namespace

bool write_exr_rgba_half(const std::string& path, int w, int h, const float* rgb, std::string* err) {
  std::string head;
  put_u32(head, 20000630u);  // magic
  put_u32(head, 2u);         // version 2, single-part scanline
  std::string ch;
  for (const char* c : {"A", "B", "G", "R"}) {
    ch.append(c); ch.push_back('\0');
    put_i32(ch, 1);           // HALF
    ch.push_back(0); ch.push_back(0); ch.push_back(0); ch.push_back(0);  // pLinear + reserved
    put_i32(ch, 1); put_i32(ch, 1);  // x/y sampling
  }
  ch.push_back('\0');
  attr(head, "channels", "chlist", ch);
  attr(head, "compression", "compression", std::string(1, '\0'));
  std::string box;
  put_i32(box, 0); put_i32(box, 0); put_i32(box, w - 1); put_i32(box, h - 1);
  attr(head, "dataWindow", "box2i", box);
  attr(head, "displayWindow", "box2i", box);
  attr(head, "lineOrder", "lineOrder", std::string(1, '\0'));
  std::string par; put_f32(par, 1.f);
  attr(head, "pixelAspectRatio", "float", par);
  std::string swc; put_f32(swc, 0.f); put_f32(swc, 0.f);
  attr(head, "screenWindowCenter", "v2f", swc);
  std::string sww; put_f32(sww, 1.f);
  attr(head, "screenWindowWidth", "float", sww);
  head.push_back('\0');
  const uint64_t line_bytes = (uint64_t)w * 4 * 2;
  const uint64_t block = 8 + line_bytes;
  uint64_t first = head.size() + 8ull * h;
  for (int y = 0; y < h; ++y) put_u64(head, first + block * y);
  std::string body;
  body.reserve(block * h);
  std::vector<uint16_t> line((size_t)w * 4);
  for (int y = 0; y < h; ++y) {
    put_i32(body, y);
    put_i32(body, (int32_t)line_bytes);
    const float* row = rgb + (size_t)3 * w * y;
    for (int x = 0; x < w; ++x) {
      line[0 * w + x] = float_to_half(1.f);             // A
      line[1 * w + x] = float_to_half(row[3 * x + 2]);  // B
      line[2 * w + x] = float_to_half(row[3 * x + 1]);  // G
      line[3 * w + x] = float_to_half(row[3 * x + 0]);  // R
    }
    for (uint16_t v : line) { body.push_back((char)(v & 0xff)); body.push_back((char)(v >> 8)); }
  }
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { *err = "cannot write " + path; return false; }
  bool ok = fwrite(head.data(), 1, head.size(), f) == head.size() && fwrite(body.data(), 1, body.size(), f) == body.size();
  fclose(f);
  if (!ok) *err = "short write to " + path;
  return ok;
}

// IEEE binary16 -> binary32 (exact).
float half_to_float(uint16_t h) {
  const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  const uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
  uint32_t x;
  if (e == 0) {
    if (m == 0) {
      x = sign;
    } else {  // subnormal: normalise
      int k = 0;
      uint32_t mm = m;
      while (!(mm & 0x400u)) { mm <<= 1; ++k; }
      x = sign | ((uint32_t)(127 - 15 + 1 - k) << 23) | ((mm & 0x3ffu) << 13);
    }
  } else if (e == 31) {
    x = sign | 0x7f800000u | (m << 13);
  } else {
    x = sign | ((e + 127u - 15u) << 23) | (m << 13);
  }
  float f;
  memcpy(&f, &x, 4);
  return f;
}

namespace {
uint32_t get_u32(const unsigned char* p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24); }
uint64_t get_u64(const unsigned char* p) { return (uint64_t)get_u32(p) | ((uint64_t)get_u32(p + 4) << 32); }
}  // namespace

// A single-part scanline OpenEXR file without compression, channels of HALF or
// FLOAT (the layout write_exr_rgba_half produces): R, G, B (a lone Y channel
// is read as grey).  Rows top first; 3 floats per pixel.
bool read_exr_rgb(const std::string& path, int* w_out, int* h_out, std::vector<float>* rgb, std::string* err) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) { *err = "cannot open " + path; return false; }
  std::vector<unsigned char> d;
  unsigned char buf[65536];
  size_t got;
  while ((got = fread(buf, 1, sizeof(buf), f)) > 0) d.insert(d.end(), buf, buf + got);
  fclose(f);
  auto fail = [&](const char* why) { *err = std::string("EXR [") + path + "]: " + why; return false; };
  if (d.size() < 8 || get_u32(&d[0]) != 20000630u) return fail("not an OpenEXR file");
  if ((get_u32(&d[4]) & 0xffu) != 2u || (get_u32(&d[4]) & 0x1e00u)) return fail("only single-part scanline files");
  size_t p = 8;
  struct Ch { std::string name; int type; };
  std::vector<Ch> chans;
  int compression = -1, x0 = 0, y0 = 0, x1 = -1, y1 = -1;
  auto cstr = [&](std::string* s) {
    s->clear();
    while (p < d.size() && d[p]) s->push_back((char)d[p++]);
    if (p >= d.size()) return false;
    ++p;
    return true;
  };
  while (true) {
    std::string name, type;
    if (!cstr(&name)) return fail("truncated header");
    if (name.empty()) break;
    if (!cstr(&type) || p + 4 > d.size()) return fail("truncated header");
    const uint32_t size = get_u32(&d[p]);
    p += 4;
    if (p + size > d.size()) return fail("truncated attribute");
    const size_t end = p + size;
    if (name == "channels") {
      while (p < end && d[p]) {
        Ch c;
        while (p < end && d[p]) c.name.push_back((char)d[p++]);
        ++p;
        if (p + 16 > end) return fail("bad channel list");
        c.type = (int)get_u32(&d[p]);
        if (get_u32(&d[p + 8]) != 1u || get_u32(&d[p + 12]) != 1u) return fail("subsampled channels");
        p += 16;
        chans.push_back(c);
      }
    } else if (name == "compression") {
      compression = d[p];
    } else if (name == "dataWindow" && size == 16) {
      x0 = (int)get_u32(&d[p]); y0 = (int)get_u32(&d[p + 4]);
      x1 = (int)get_u32(&d[p + 8]); y1 = (int)get_u32(&d[p + 12]);
    }
    p = end;
  }
  if (compression != 0) return fail("only uncompressed files");
  const int w = x1 - x0 + 1, h = y1 - y0 + 1;
  if (w <= 0 || h <= 0 || w > 65536 || h > 65536 || chans.empty()) return fail("bad data window or channels");
  int ir = -1, ig = -1, ib = -1, iy = -1;
  size_t line = 0;
  std::vector<size_t> off(chans.size());
  for (size_t c = 0; c < chans.size(); ++c) {
    if (chans[c].type != 1 && chans[c].type != 2) return fail("only HALF or FLOAT channels");
    off[c] = line;
    line += (size_t)w * (chans[c].type == 1 ? 2 : 4);
    if (chans[c].name == "R") ir = (int)c;
    if (chans[c].name == "G") ig = (int)c;
    if (chans[c].name == "B") ib = (int)c;
    if (chans[c].name == "Y") iy = (int)c;
  }
  if ((ir < 0 || ig < 0 || ib < 0) && iy < 0) return fail("no R, G, B or Y channel");
  if (ir < 0 || ig < 0 || ib < 0) ir = ig = ib = iy;
  if (p + 8ull * h > d.size()) return fail("truncated offset table");
  *w_out = w;
  *h_out = h;
  rgb->assign((size_t)3 * w * h, 0.f);
  auto value = [&](const unsigned char* q, int type) {
    if (type == 1) return half_to_float((uint16_t)(q[0] | (q[1] << 8)));
    uint32_t u = get_u32(q);
    float v;
    memcpy(&v, &u, 4);
    return v;
  };
  for (int k = 0; k < h; ++k) {
    const uint64_t bo = get_u64(&d[p + 8ull * k]);
    if (bo + 8 > d.size()) return fail("bad block offset");
    const int y = (int)get_u32(&d[bo]) - y0;
    const uint32_t size = get_u32(&d[bo + 4]);
    if (y < 0 || y >= h || size < line || bo + 8 + line > d.size()) return fail("bad scanline block");
    const unsigned char* q = &d[bo + 8];
    const int idx[3] = {ir, ig, ib};
    for (int x = 0; x < w; ++x)
      for (int k3 = 0; k3 < 3; ++k3) {
        const Ch& c = chans[idx[k3]];
        (*rgb)[((size_t)y * w + x) * 3 + k3] = value(q + off[idx[k3]] + (size_t)x * (c.type == 1 ? 2 : 4), c.type);
      }
  }
  return true;
}

// PFM: "PF\n<w> <h>\n-1.0\n" then little-endian float RGB rows, bottom row first.
bool write_pfm(const std::string& path, int w, int h, const float* rgb, std::string* err) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { *err = "cannot write " + path; return false; }
  fprintf(f, "PF\n%d %d\n-1.0\n", w, h);
  bool ok = true;
  for (int y = h - 1; y >= 0 && ok; --y) ok = fwrite(rgb + (size_t)3 * w * y, sizeof(float), (size_t)3 * w, f) == (size_t)3 * w;
  fclose(f);
  if (!ok) *err = "short write to " + path;
  return ok;
}

}  // namespace mscg
