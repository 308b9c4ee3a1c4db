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
