// Host-side scene description: the reference's YAML/OBJ input parsed into
// plain tables, and the POD records the device stages read.
//
// Reference layout being mirrored:
//   Pathtracer::construct   src/core/Pathtracer.cpp:32-275   (two-document YAML)
//   Image / Settings        include/core/Image.h:56-69, include/core/Settings.h:30-45
//   PinHoleCamera           src/core/PinHoleCamera.cpp:5-32, include/core/PinHoleCamera.h:98-113
//   ThinLensCamera          src/core/ThinLensCamera.cpp:5-56
//   PolygonObject           src/core/PolygonObject.cpp:5-63, include/core/PolygonObject.h:171-189
//   LambertShader           src/core/LambertShader.cpp:22-73, include/core/LambertShader.h:140-174
//   NullShader              src/core/NullShader.cpp:25-54
//   QuadLight               src/core/QuadLight.cpp:5-84, include/core/QuadLight.h:153-169
//   tinyobj::LoadObj        thirdparty/tinyobjloader/tiny_obj_loader.cpp:309-412,643-891
#pragma once

#include <stdint.h>
#include <string>
#include <vector>
#include <utility>

#include "dmath.h"

namespace mscg {

// ----------------------------------------------------------------- YAML subset
struct YNode {
  enum Kind { Null, Scalar, Seq, Map } kind = Null;
  std::string scalar;
  std::vector<YNode> seq;
  std::vector<std::pair<std::string, YNode>> map;  // duplicate keys kept, in order
  const YNode* get(const std::string& key) const;
  size_t size() const { return kind == Map ? map.size() : (kind == Seq ? seq.size() : 0); }
};

// Parses block maps/sequences, flow sequences/maps, scalars, comments and
// '---' document separators.  Returns false with a message on malformed input.
bool yaml_parse_documents(const std::string& text, std::vector<YNode>* docs, std::string* err);

// ------------------------------------------------------------------ OBJ (tinyobj semantics)
struct ObjMesh {
  std::vector<float> positions;    // 3 per vertex
  std::vector<float> normals;      // 3 per vertex that carried a normal index
  std::vector<float> texcoords;    // 2 per vertex that carried a texcoord index
  std::vector<uint32_t> indices;   // 3 per triangle (fan triangulation)
};
bool obj_load_file(const std::string& path, ObjMesh* out, std::string* err);
bool obj_load_text(const char* text, size_t len, ObjMesh* out);
double obj_parse_number(const char* s, const char* end);  // tinyobj tryParseDouble rules

// ------------------------------------------------------------------ device tables
enum ShaderType : int { SHADER_LAMBERT = 0, SHADER_NULL = 1, SHADER_PHONG = 2 };
enum TextureType : int { TEXTURE_CONSTANT = 0, TEXTURE_FACE = 1, TEXTURE_TREE = 2 };
enum TexNodeType : int { TEXNODE_CONSTANT = 0, TEXNODE_STANDARD = 1, TEXNODE_LAYERED = 2 };

// A node of a texture tree (ConstantTexture, StandardTexture, LayeredTexture;
// include/core/*Texture.h): Layered = upper * mask + lower * (1 - mask).
struct TexNode {
  int type;          // TexNodeType
  int image;         // Standard: index into the scene's images
  int upper, lower, mask;  // Layered: node indices
  float colour[3];   // Constant
};

// An RGB image, rows top first (image row 0 is texture coordinate t = 0).
struct TexImage {
  int width = 0, height = 0;
  std::vector<float> rgb;  // 3 per texel
};
// Reads PFM (PF/Pf), PPM (P6, 8 or 16 bit) and uncompressed scanline OpenEXR images.
bool image_load(const std::string& path, TexImage* out, std::string* err);
enum LightType : int { LIGHT_QUAD = 0, LIGHT_SPHERE = 1 };
enum CameraType : int { CAMERA_PINHOLE = 0, CAMERA_THINLENS = 1 };
enum SamplerType : int { SAMPLER_STRATIFIED = 0, SAMPLER_INDEPENDENT = 1, SAMPLER_GRID = 2 };
enum FilterType : int { FILTER_TENT = 0, FILTER_BOX = 1 };

struct ShaderRec {
  int type;          // ShaderType
  int light;         // light index when this is the Null shader of an emitter, else -1
  float reflectance; // LambertShader::continuation() returns it (LambertShader.cpp:22-25)
  float exponent;    // Phong exponent (extension)
  float colour[3];   // ConstantTexture colour (ConstantTexture.cpp:22-25); tint of face texels
  int texture;       // TextureType
  int tex_root;      // TEXTURE_TREE: root node of the shader's texture tree
  int tex_prog;      // TEXTURE_TREE: first op of its post-order program (device)
  int tex_len;       // and the number of ops
  int pad;
};

// Per-face texels (extension): every triangle of the scene owns res x res RGB
// texels; texel (i, j) of face f, channel c, is k / 1024 with
// k = face_texel_code(seed, f, j * res + i, c), exact in FP16.  A FaceTexels
// texture looks up i = min(res-1, floor(u res)), j = min(res-1, floor(v res))
// at the hit's barycentric weights (u, v) of v1 and v2.
struct FaceTexels {
  int res = 0;        // 0: the scene has none
  uint32_t seed = 0;
};

MSC_HD uint32_t face_texel_code(uint32_t seed, uint32_t face, uint32_t texel, uint32_t ch) {
  return pcg4d(seed, face, texel, ch).w >> 22;  // 10 bits
}

struct GeomRec {     // one per reference geomID (Scene::objects index)
  int shader;
  int first_prim;    // global index of the object's first triangle
  int prim_count;
  int light;         // light index for emitter geometry, else -1
};

struct LightRec {
  int type;          // LightType
  float intensity;
  float scale[2];    // quad extents (QuadLight::m_scale)
  Affine3 xf;        // T * Rx * Ry * Rz * diag(1, sx, sy)  (QuadLight.cpp:25-31)
  float normal[3];   // normalize(L^-T * X)                   (QuadLight.cpp:33)
  float centre[3];   // sphere lights (extension): uniform radiance `intensity` leaving the surface
  float radius;
};

struct CameraRec {
  int type;          // CameraType
  Affine3 xf;        // T * Ry * Rx * Rz (PinHoleCamera.cpp:7-11)
  float normal[3];   // normalize(L^-T * X)
  float translation[3];
  float focal_length;
  float focal_distance;
  float aperture;
};

struct Settings {    // include/core/Settings.h:16-24, defaults Pathtracer.cpp:74-79
  int min_depth = 2;
  int max_depth = 100;
  float threshold = 0.01f;
  int bucket_size = 16;
  int shading_size = 4096;
  int bin_exponent = 25;
};

struct Extensions {  // optional third YAML document; the reference ignores it
  int spp = 0;             // non-square sample count (0 = base^2)
  int mis_power = 0;       // 1 = power heuristic, 0 = balance (Common.h:45-48)
  int ray_sort = 1;        // sort batches on the origin/direction key
  int hit_sort = 1;        // sort hits on (geomID, primID)
  uint32_t seed = 0;       // mixes into every per-path draw
  int generation = 0;      // paths per camera generation (0 = automatic)
  int wide_bvh = 1;        // 1: 8-wide quantised BVH, 0: binary LBVH
  int hit_key_bits = 32;   // 32: (geomID, primID); 64: (shader 12 b, face 23 b, quantised uv 29 b)
  int bins = 6;            // direction bins: 6 (the reference's), 26 or 98
  int autotune = 1;        // 1: the batch loop tunes itself online from the settings above
};

struct SceneDesc {
  // document 0
  int width = 700, height = 500, base = 8;
  Settings settings;
  CameraRec camera;
  int sampler = SAMPLER_STRATIFIED;
  int filter = FILTER_TENT;
  Extensions ext;
  // document 1
  std::vector<ShaderRec> shaders;
  std::vector<GeomRec> geoms;
  std::vector<LightRec> lights;
  std::vector<int> sphere_lights;    // light index of each sphere light, in light order
  FaceTexels texels;
  std::vector<TexNode> tex_nodes;    // texture trees of Standard / Layered textures
  std::vector<TexImage> images;
  std::vector<std::string> image_paths;
  // flattened triangles in geomID order, positions after the object transform
  std::vector<float> tri_v;          // 9 per triangle: v0, v1, v2
  std::vector<float> tri_uv;         // 6 per triangle: uv0, uv1, uv2 (0 when absent)
  std::vector<int> tri_geom;         // geomID per triangle
  std::vector<uint8_t> tri_is_light; // 1 for emitter geometry (Embree mask 0xF0000000)
  int spp() const { return ext.spp > 0 ? ext.spp : base * base; }
};

// Loads the two-document YAML scene (plus the optional extension document)
// and every OBJ it names; relative OBJ paths resolve against the YAML's folder.
bool load_scene(const std::string& yaml_path, SceneDesc* out, std::string* err);

// Transforms exactly as the reference composes them.
Affine3 make_trs_xyz(const float t[3], const float r_deg[3], const float s[3]);  // T Rx Ry Rz S
Affine3 make_tr_yxz(const float t[3], const float r_deg[3]);                     // T Ry Rx Rz
void normal_of_x_axis(const Affine3& a, float out[3]);                           // normalize(L^-T X)

}  // namespace mscg
