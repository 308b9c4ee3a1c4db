// Scene input: a YAML subset parser, an OBJ reader with tinyobjloader's
// semantics, and the assembly of the reference's scene tables.
// See scene.h for the reference files each part follows.
#include "scene.h"

#include <algorithm>
#include <cctype>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <unordered_map>
#include <sstream>
#include <thread>

namespace mscg {

// =============================================================== YAML subset

const YNode* YNode::get(const std::string& key) const {
  if (kind != Map) return nullptr;
  for (const auto& kv : map)
    if (kv.first == key) return &kv.second;
  return nullptr;
}

namespace {

struct YLine {
  int indent;
  std::string text;  // without indentation and comments
  int lineno;
};

std::string rtrim(const std::string& s) {
  size_t e = s.size();
  while (e > 0 && (s[e - 1] == ' ' || s[e - 1] == '\t' || s[e - 1] == '\r')) --e;
  return s.substr(0, e);
}

std::string trim(const std::string& s) {
  size_t b = 0;
  while (b < s.size() && (s[b] == ' ' || s[b] == '\t')) ++b;
  return rtrim(s.substr(b));
}

// Removes a '#' comment that is not inside quotes.
std::string strip_comment(const std::string& s) {
  bool sq = false, dq = false;
  for (size_t i = 0; i < s.size(); ++i) {
    char c = s[i];
    if (c == '\'' && !dq) sq = !sq;
    else if (c == '"' && !sq) dq = !dq;
    else if (c == '#' && !sq && !dq && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) return s.substr(0, i);
  }
  return s;
}

std::string unquote(const std::string& s) {
  if (s.size() >= 2 && ((s.front() == '"' && s.back() == '"') || (s.front() == '\'' && s.back() == '\'')))
    return s.substr(1, s.size() - 2);
  return s;
}

// Position of the "key: " separator of a block mapping line, or npos.
size_t find_map_colon(const std::string& s) {
  bool sq = false, dq = false;
  int depth = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    char c = s[i];
    if (c == '\'' && !dq) sq = !sq;
    else if (c == '"' && !sq) dq = !dq;
    else if (!sq && !dq) {
      if (c == '[' || c == '{') ++depth;
      else if (c == ']' || c == '}') --depth;
      else if (c == ':' && depth == 0 && (i + 1 == s.size() || s[i + 1] == ' ' || s[i + 1] == '\t')) return i;
    }
  }
  return std::string::npos;
}

struct FlowParser {
  const std::string& s;
  size_t p = 0;
  std::string err;
  explicit FlowParser(const std::string& str) : s(str) {}
  void ws() { while (p < s.size() && (s[p] == ' ' || s[p] == '\t')) ++p; }
  bool parse(YNode* out) {
    ws();
    if (p >= s.size()) { out->kind = YNode::Null; return true; }
    if (s[p] == '[') {
      ++p;
      out->kind = YNode::Seq;
      ws();
      if (p < s.size() && s[p] == ']') { ++p; return true; }
      while (true) {
        YNode item;
        if (!parse(&item)) return false;
        out->seq.push_back(item);
        ws();
        if (p < s.size() && s[p] == ',') { ++p; continue; }
        if (p < s.size() && s[p] == ']') { ++p; return true; }
        err = "unterminated flow sequence";
        return false;
      }
    }
    if (s[p] == '{') {
      ++p;
      out->kind = YNode::Map;
      ws();
      if (p < s.size() && s[p] == '}') { ++p; return true; }
      while (true) {
        ws();
        size_t k0 = p;
        while (p < s.size() && s[p] != ':' && s[p] != ',' && s[p] != '}') ++p;
        if (p >= s.size() || s[p] != ':') { err = "bad flow mapping"; return false; }
        std::string key = unquote(trim(s.substr(k0, p - k0)));
        ++p;
        YNode val;
        if (!parse(&val)) return false;
        out->map.emplace_back(key, val);
        ws();
        if (p < s.size() && s[p] == ',') { ++p; continue; }
        if (p < s.size() && s[p] == '}') { ++p; return true; }
        err = "unterminated flow mapping";
        return false;
      }
    }
    size_t b = p;
    bool sq = false, dq = false;
    while (p < s.size()) {
      char c = s[p];
      if (c == '\'' && !dq) sq = !sq;
      else if (c == '"' && !sq) dq = !dq;
      else if (!sq && !dq && (c == ',' || c == ']' || c == '}')) break;
      ++p;
    }
    out->kind = YNode::Scalar;
    out->scalar = unquote(trim(s.substr(b, p - b)));
    return true;
  }
};

bool parse_inline_value(const std::string& text, YNode* out, std::string* err) {
  std::string t = trim(text);
  if (t.empty()) { out->kind = YNode::Null; return true; }
  if (t[0] == '[' || t[0] == '{') {
    FlowParser fp(t);
    if (!fp.parse(out)) { *err = fp.err; return false; }
    fp.ws();
    if (fp.p != t.size()) { *err = "trailing characters after flow collection"; return false; }
    return true;
  }
  out->kind = YNode::Scalar;
  out->scalar = unquote(t);
  return true;
}

bool parse_block(const std::vector<YLine>& lines, size_t* i, int indent, YNode* out, std::string* err);

// Parses the value that follows "key:" (inline text or a nested block).
bool parse_after_key(const std::vector<YLine>& lines, size_t* i, int indent, const std::string& rest,
                     YNode* out, std::string* err) {
  if (!trim(rest).empty()) return parse_inline_value(rest, out, err);
  if (*i < lines.size() && (lines[*i].indent > indent ||
                            (lines[*i].indent == indent && lines[*i].text.rfind("- ", 0) == 0)))
    return parse_block(lines, i, lines[*i].indent, out, err);
  out->kind = YNode::Null;
  return true;
}

bool parse_block(const std::vector<YLine>& lines, size_t* i, int indent, YNode* out, std::string* err) {
  if (*i >= lines.size()) { out->kind = YNode::Null; return true; }
  bool is_seq = lines[*i].text == "-" || lines[*i].text.rfind("- ", 0) == 0;
  out->kind = is_seq ? YNode::Seq : YNode::Map;
  while (*i < lines.size() && lines[*i].indent == indent) {
    const YLine& ln = lines[*i];
    if (is_seq) {
      if (!(ln.text == "-" || ln.text.rfind("- ", 0) == 0)) break;
      std::string rest = ln.text.size() > 1 ? ln.text.substr(2) : std::string();
      ++*i;
      YNode item;
      size_t colon = find_map_colon(trim(rest));
      if (!trim(rest).empty() && colon != std::string::npos && trim(rest)[0] != '[' && trim(rest)[0] != '{') {
        // "- key: value" starts a mapping whose further keys sit at indent + 2
        std::vector<YLine> sub;
        YLine first{indent + 2, trim(rest), ln.lineno};
        sub.push_back(first);
        size_t j = *i;
        while (j < lines.size() && lines[j].indent > indent) sub.push_back(lines[j++]);
        size_t k = 0;
        if (!parse_block(sub, &k, indent + 2, &item, err)) return false;
        *i = j;
      } else if (trim(rest).empty()) {
        if (*i < lines.size() && lines[*i].indent > indent) {
          if (!parse_block(lines, i, lines[*i].indent, &item, err)) return false;
        }
      } else if (!parse_inline_value(rest, &item, err)) {
        return false;
      }
      out->seq.push_back(item);
    } else {
      size_t colon = find_map_colon(ln.text);
      if (colon == std::string::npos) {
        *err = "line " + std::to_string(ln.lineno) + ": expected 'key: value'";
        return false;
      }
      std::string key = unquote(trim(ln.text.substr(0, colon)));
      std::string rest = ln.text.substr(colon + 1);
      ++*i;
      YNode val;
      if (!parse_after_key(lines, i, indent, rest, &val, err)) return false;
      out->map.emplace_back(key, val);
    }
  }
  if (*i < lines.size() && lines[*i].indent > indent) {
    *err = "line " + std::to_string(lines[*i].lineno) + ": bad indentation";
    return false;
  }
  return true;
}

}  // namespace

bool yaml_parse_documents(const std::string& text, std::vector<YNode>* docs, std::string* err) {
  docs->clear();
  std::vector<std::vector<YLine>> groups(1);
  std::istringstream in(text);
  std::string raw;
  int lineno = 0;
  bool any_content = false;
  while (std::getline(in, raw)) {
    ++lineno;
    std::string s = rtrim(strip_comment(raw));
    std::string t = trim(s);
    if (t == "---" || t.rfind("--- ", 0) == 0) {
      if (any_content || !groups.back().empty()) groups.emplace_back();
      any_content = true;
      continue;
    }
    if (t == "...") continue;
    if (t.empty()) continue;
    if (!s.empty() && s[0] == '%') continue;  // directives
    int ind = 0;
    while (ind < (int)s.size() && s[ind] == ' ') ++ind;
    if (ind < (int)s.size() && s[ind] == '\t') {
      *err = "line " + std::to_string(lineno) + ": tab indentation";
      return false;
    }
    groups.back().push_back(YLine{ind, t, lineno});
    any_content = true;
  }
  for (auto& g : groups) {
    YNode doc;
    if (!g.empty()) {
      size_t i = 0;
      if (!parse_block(g, &i, g[0].indent, &doc, err)) return false;
      if (i != g.size()) {
        *err = "line " + std::to_string(g[i].lineno) + ": unexpected content";
        return false;
      }
    }
    docs->push_back(doc);
  }
  while (!docs->empty() && docs->back().kind == YNode::Null) docs->pop_back();
  return true;
}

// ================================================================ OBJ reader

// tryParseDouble's grammar and arithmetic (tiny_obj_loader.cpp:131-242):
// integer digits accumulate as m = m*10 + d, fraction digits add d*10^-k,
// and the result is sign * ldexp(m * 5^e, e).  A malformed number yields 0.
double obj_parse_number(const char* s, const char* end) {
  if (s >= end) return 0.0;
  double mantissa = 0.0;
  int exponent = 0;
  char sign = '+', exp_sign = '+';
  const char* c = s;
  int read = 0;
  bool more = false;
  if (*c == '+' || *c == '-') { sign = *c; ++c; }
  else if (!isdigit((unsigned char)*c)) return 0.0;
  while ((more = (c != end)) && isdigit((unsigned char)*c)) {
    mantissa *= 10;
    mantissa += (int)(*c - '0');
    ++c; ++read;
  }
  if (read == 0) return 0.0;
  if (!more) goto assemble;
  if (*c == '.') {
    ++c;
    read = 1;
    while ((more = (c != end)) && isdigit((unsigned char)*c)) {
      mantissa += (int)(*c - '0') * pow(10.0, -read);
      ++read; ++c;
    }
  } else if (*c == 'e' || *c == 'E') {
  } else {
    goto assemble;
  }
  if (!more) goto assemble;
  if (*c == 'e' || *c == 'E') {
    ++c;
    if ((more = (c != end)) && (*c == '+' || *c == '-')) { exp_sign = *c; ++c; }
    else if (isdigit((unsigned char)*c)) {}
    else return 0.0;
    read = 0;
    while ((more = (c != end)) && isdigit((unsigned char)*c)) {
      exponent *= 10;
      exponent += (int)(*c - '0');
      ++c; ++read;
    }
    exponent *= (exp_sign == '+' ? 1 : -1);
    if (read == 0) return 0.0;
  }
assemble:
  return (sign == '+' ? 1 : -1) * ldexp(mantissa * pow(5.0, exponent), exponent);
}

namespace {

struct VIdx { int v, vt, vn; };
// tinyobj keys its vertex cache on the (v, vt, vn) triple (tiny_obj_loader.cpp:58-67);
// only equality matters for the output, so a hash map gives the same result.
struct VIdxHash {
  size_t operator()(const VIdx& a) const {
    uint64_t h = (uint64_t)(uint32_t)a.v * 0x9e3779b97f4a7c15ull;
    h ^= (uint64_t)(uint32_t)a.vt * 0xc2b2ae3d27d4eb4full + (h << 6) + (h >> 2);
    h ^= (uint64_t)(uint32_t)a.vn * 0x165667b19e3779f9ull + (h << 6) + (h >> 2);
    return (size_t)h;
  }
};
struct VIdxEq {
  bool operator()(const VIdx& a, const VIdx& b) const { return a.v == b.v && a.vt == b.vt && a.vn == b.vn; }
};

inline bool is_sp(char c) { return c == ' ' || c == '\t'; }
inline bool is_nl(char c) { return c == '\r' || c == '\n' || c == '\0'; }
inline int fix_index(int idx, int n) { return idx > 0 ? idx - 1 : (idx == 0 ? 0 : n + idx); }

float next_float(const char*& tok) {
  tok += strspn(tok, " \t");
  const char* e = tok + strcspn(tok, " \t\r");
  float f = (float)obj_parse_number(tok, e);
  tok = e;
  return f;
}

// One face corner as written: the atoi value of each index, kAbsent where the
// corner has no such index.  Negative (relative) indices are resolved once the
// element counts before the face line are known.
constexpr int kAbsent = INT_MIN;
struct RawCorner { int v, vt, vn; };

// parseTriple's token rules (tiny_obj_loader.cpp:309-345): "v", "v/vt", "v//vn", "v/vt/vn".
RawCorner parse_triple_raw(const char*& tok) {
  RawCorner r{atoi(tok), kAbsent, kAbsent};
  tok += strcspn(tok, "/ \t\r");
  if (tok[0] != '/') return r;
  ++tok;
  if (tok[0] == '/') {
    ++tok;
    r.vn = atoi(tok);
    tok += strcspn(tok, "/ \t\r");
    return r;
  }
  r.vt = atoi(tok);
  tok += strcspn(tok, "/ \t\r");
  if (tok[0] != '/') return r;
  ++tok;
  r.vn = atoi(tok);
  tok += strcspn(tok, "/ \t\r");
  return r;
}

// What one contiguous run of whole lines holds, in file order.
struct ObjChunk {
  std::vector<float> v, vn, vt;
  std::vector<RawCorner> corners;
  std::vector<uint32_t> face_first;           // first corner of each face
  std::vector<int> face_nv, face_nvn, face_nvt;  // this chunk's element counts before each face line
};

// The line loop of LoadObj (tiny_obj_loader.cpp:643-891) for the v, vn, vt and
// f records over text[begin, end), which starts at a line start.
void parse_obj_lines(const char* text, size_t begin, size_t end, ObjChunk* c) {
  std::string line;
  size_t pos = begin;
  while (pos < end) {
    size_t e = pos;
    while (e < end && text[e] != '\n') ++e;
    line.assign(text + pos, e - pos);
    pos = e + 1;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.size() > 8191) line.resize(8191);  // tinyobj reads lines into an 8192-byte buffer
    if (line.empty()) continue;
    const char* tok = line.c_str();
    tok += strspn(tok, " \t");
    if (tok[0] == '\0' || tok[0] == '#') continue;
    if (tok[0] == 'v' && is_sp(tok[1])) {
      tok += 2;
      float x = next_float(tok), y = next_float(tok), z = next_float(tok);
      c->v.push_back(x); c->v.push_back(y); c->v.push_back(z);
      continue;
    }
    if (tok[0] == 'v' && tok[1] == 'n' && is_sp(tok[2])) {
      tok += 3;
      float x = next_float(tok), y = next_float(tok), z = next_float(tok);
      c->vn.push_back(x); c->vn.push_back(y); c->vn.push_back(z);
      continue;
    }
    if (tok[0] == 'v' && tok[1] == 't' && is_sp(tok[2])) {
      tok += 3;
      float x = next_float(tok), y = next_float(tok);
      c->vt.push_back(x); c->vt.push_back(y);
      continue;
    }
    if (tok[0] == 'f' && is_sp(tok[1])) {
      tok += 2;
      tok += strspn(tok, " \t");
      c->face_first.push_back((uint32_t)c->corners.size());
      c->face_nv.push_back((int)(c->v.size() / 3));
      c->face_nvn.push_back((int)(c->vn.size() / 3));
      c->face_nvt.push_back((int)(c->vt.size() / 2));
      while (!is_nl(tok[0])) {
        c->corners.push_back(parse_triple_raw(tok));
        tok += strspn(tok, " \t\r");
      }
      continue;
    }
  }
}

template <class F>
void parallel_for(int workers, F&& fn) {
  std::vector<std::thread> pool;
  for (int w = 1; w < workers; ++w) pool.emplace_back(fn, w);
  fn(0);
  for (auto& t : pool) t.join();
}

}  // namespace

// LoadObj with tinyobjloader's results (positions, texcoords, normals, fan
// triangles with one vertex per distinct (v, vt, vn) triple in first-use
// order), read in parallel:
//   1. the text is cut at line starts into one run per worker, and each run's
//      v / vn / vt / f records are parsed on their own;
//   2. per-run element counts give every face line the global counts that
//      resolve its relative (negative) indices;
//   3. distinct corners are found by hash shards: worker w keeps the corners
//      whose triple hashes to w, in file order, so the first use of a triple
//      is known; a prefix sum over first uses numbers the vertices in
//      first-use order (the fan visits a face's corners in their written
//      order, so first use in corner order is first use in fan order);
//   4. vertices, normals, texcoords and fan indices are written at offsets
//      from prefix sums.
bool obj_load_text(const char* text, size_t len, ObjMesh* out) {
  unsigned hw = std::thread::hardware_concurrency();
  const int workers = len < (1u << 20) ? 1 : (int)std::max(1u, std::min(hw ? hw : 1u, 32u));
  // 1. runs of whole lines
  std::vector<size_t> cut((size_t)workers + 1, len);
  cut[0] = 0;
  for (int w = 1; w < workers; ++w) {
    size_t p = std::max(cut[w - 1], len * (size_t)w / (size_t)workers);
    while (p < len && p > 0 && text[p - 1] != '\n') ++p;
    cut[w] = p;
  }
  std::vector<ObjChunk> ch((size_t)workers);
  parallel_for(workers, [&](int w) { parse_obj_lines(text, cut[w], cut[w + 1], &ch[w]); });
  // 2. global element counts and concatenated arrays
  std::vector<size_t> ov(workers + 1, 0), ovn(workers + 1, 0), ovt(workers + 1, 0), oc(workers + 1, 0),
      of(workers + 1, 0);
  for (int w = 0; w < workers; ++w) {
    ov[w + 1] = ov[w] + ch[w].v.size();
    ovn[w + 1] = ovn[w] + ch[w].vn.size();
    ovt[w + 1] = ovt[w] + ch[w].vt.size();
    oc[w + 1] = oc[w] + ch[w].corners.size();
    of[w + 1] = of[w] + ch[w].face_first.size();
  }
  const size_t C = oc[workers], F = of[workers];
  std::vector<float> v(ov[workers]), vn(ovn[workers]), vt(ovt[workers]);
  std::vector<VIdx> corner(C);
  std::vector<uint32_t> face_first(F + 1);
  face_first[F] = (uint32_t)C;
  parallel_for(workers, [&](int w) {
    const ObjChunk& c = ch[w];
    std::copy(c.v.begin(), c.v.end(), v.begin() + ov[w]);
    std::copy(c.vn.begin(), c.vn.end(), vn.begin() + ovn[w]);
    std::copy(c.vt.begin(), c.vt.end(), vt.begin() + ovt[w]);
    const size_t nf = c.face_first.size();
    for (size_t f = 0; f < nf; ++f) {
      const uint32_t b = c.face_first[f], e = f + 1 < nf ? c.face_first[f + 1] : (uint32_t)c.corners.size();
      face_first[of[w] + f] = (uint32_t)(oc[w] + b);
      const int nv = (int)(ov[w] / 3) + c.face_nv[f], nvn = (int)(ovn[w] / 3) + c.face_nvn[f],
                nvt = (int)(ovt[w] / 2) + c.face_nvt[f];
      for (uint32_t k = b; k < e; ++k) {
        const RawCorner& r = c.corners[k];
        VIdx& x = corner[oc[w] + k];
        x.v = fix_index(r.v, nv);
        x.vt = r.vt == kAbsent ? -1 : fix_index(r.vt, nvt);
        x.vn = r.vn == kAbsent ? -1 : fix_index(r.vn, nvn);
      }
    }
  });
  ch.clear();
  ch.shrink_to_fit();
  // faces of fewer than three corners are dropped before any vertex is made
  std::vector<uint8_t> live(C, 0);
  parallel_for(workers, [&](int w) {
    for (size_t f = F * (size_t)w / workers; f < F * (size_t)(w + 1) / workers; ++f)
      if (face_first[f + 1] - face_first[f] >= 3)
        for (uint32_t k = face_first[f]; k < face_first[f + 1]; ++k) live[k] = 1;
  });
  // 3. first use of each distinct triple, by hash shard
  std::vector<uint32_t> first(C, UINT32_MAX);  // corner -> the corner of its triple's first use
  VIdxHash hasher;
  parallel_for(workers, [&](int w) {
    std::unordered_map<VIdx, uint32_t, VIdxHash, VIdxEq> seen;
    seen.reserve(v.size() / 3 / workers + 16);
    for (size_t k = 0; k < C; ++k) {
      if (!live[k]) continue;
      const VIdx& x = corner[k];
      if ((int)(hasher(x) % (size_t)workers) != w) continue;
      auto it = seen.emplace(x, (uint32_t)k).first;
      first[k] = it->second;
    }
  });
  std::vector<uint32_t> vid(C, UINT32_MAX);  // vertex number of a first-use corner
  uint32_t nverts = 0;
  for (size_t k = 0; k < C; ++k)
    if (live[k] && first[k] == (uint32_t)k) {
      const VIdx& x = corner[k];
      if (x.v < 0 || (size_t)(3 * x.v + 2) >= v.size()) return false;  // a face names a missing vertex
      vid[k] = nverts++;
    }
  // 4. vertex attributes (normals / texcoords only where the triple names a valid one)
  out->positions.assign((size_t)3 * nverts, 0.f);
  out->normals.clear();
  out->texcoords.clear();
  out->indices.clear();
  std::vector<uint32_t> rep(nverts);
  for (size_t k = 0; k < C; ++k)
    if (vid[k] != UINT32_MAX) rep[vid[k]] = (uint32_t)k;
  for (uint32_t i = 0; i < nverts; ++i) {
    const VIdx& x = corner[rep[i]];
    out->positions[3 * i + 0] = v[3 * x.v + 0];
    out->positions[3 * i + 1] = v[3 * x.v + 1];
    out->positions[3 * i + 2] = v[3 * x.v + 2];
    if (x.vn >= 0 && (size_t)(3 * x.vn + 2) < vn.size()) {
      out->normals.push_back(vn[3 * x.vn + 0]);
      out->normals.push_back(vn[3 * x.vn + 1]);
      out->normals.push_back(vn[3 * x.vn + 2]);
    }
    if (x.vt >= 0 && (size_t)(2 * x.vt + 1) < vt.size()) {
      out->texcoords.push_back(vt[2 * x.vt + 0]);
      out->texcoords.push_back(vt[2 * x.vt + 1]);
    }
  }
  // fan triangles (exportFaceGroupToShape, tiny_obj_loader.cpp:366-412)
  std::vector<size_t> tri_at(F + 1, 0);
  for (size_t f = 0; f < F; ++f) {
    const uint32_t k = face_first[f + 1] - face_first[f];
    tri_at[f + 1] = tri_at[f] + (k >= 3 ? k - 2 : 0);
  }
  out->indices.resize(3 * tri_at[F]);
  parallel_for(workers, [&](int w) {
    for (size_t f = F * (size_t)w / workers; f < F * (size_t)(w + 1) / workers; ++f) {
      const uint32_t b = face_first[f], e = face_first[f + 1];
      if (e - b < 3) continue;
      uint32_t* o = out->indices.data() + 3 * tri_at[f];
      const uint32_t i0 = vid[first[b]];
      for (uint32_t k = b + 2; k < e; ++k) {
        *o++ = i0;
        *o++ = vid[first[k - 1]];
        *o++ = vid[first[k]];
      }
    }
  });
  return true;
}

bool obj_load_file(const std::string& path, ObjMesh* out, std::string* err) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) { *err = "cannot open OBJ file [" + path + "]"; return false; }
  std::string s;
  if (fseek(f, 0, SEEK_END) == 0) {
    const long size = ftell(f);
    if (size > 0) {
      s.resize((size_t)size);
      rewind(f);
      s.resize(fread(&s[0], 1, (size_t)size, f));
    }
  }
  fclose(f);
  if (!obj_load_text(s.data(), s.size(), out)) { *err = "OBJ face references a missing vertex in [" + path + "]"; return false; }
  return true;
}

// ================================================================ transforms

namespace {
struct M3 { float a[3][3]; };
M3 m3_mul(const M3& x, const M3& y) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = (x.a[i][0] * y.a[0][j] + x.a[i][1] * y.a[1][j]) + x.a[i][2] * y.a[2][j];
  return r;
}
M3 rot_axis(int axis, float deg) {
  float ang = deg * MSC_PI_180;
  float c = std::cos(ang), s = std::sin(ang);
  M3 r = {{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}};
  int u = (axis + 1) % 3, v = (axis + 2) % 3;
  r.a[u][u] = c; r.a[u][v] = -s;
  r.a[v][u] = s; r.a[v][v] = c;
  return r;
}
Affine3 to_affine(const M3& l, const float t[3]) {
  Affine3 a;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) a.m[i][j] = l.a[i][j];
    a.m[i][3] = t[i];
  }
  return a;
}
}  // namespace

Affine3 make_trs_xyz(const float t[3], const float r_deg[3], const float s[3]) {
  M3 l = m3_mul(m3_mul(rot_axis(0, r_deg[0]), rot_axis(1, r_deg[1])), rot_axis(2, r_deg[2]));
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) l.a[i][j] = l.a[i][j] * s[j];
  return to_affine(l, t);
}

Affine3 make_tr_yxz(const float t[3], const float r_deg[3]) {
  M3 l = m3_mul(m3_mul(rot_axis(1, r_deg[1]), rot_axis(0, r_deg[0])), rot_axis(2, r_deg[2]));
  return to_affine(l, t);
}

// normalize(L^-T X): the first column of the cofactor matrix, signed by det(L).
void normal_of_x_axis(const Affine3& a, float out[3]) {
  const float(*L)[4] = a.m;
  float c0 = L[1][1] * L[2][2] - L[1][2] * L[2][1];
  float c1 = -(L[0][1] * L[2][2] - L[0][2] * L[2][1]);
  float c2 = L[0][1] * L[1][2] - L[0][2] * L[1][1];
  float det = (L[0][0] * c0 + L[1][0] * c1) + L[2][0] * c2;
  if (det < 0.f) { c0 = -c0; c1 = -c1; c2 = -c2; }
  float inv = 1.0f / std::sqrt((c0 * c0 + c1 * c1) + c2 * c2);
  out[0] = c0 * inv; out[1] = c1 * inv; out[2] = c2 * inv;
}

static void xf_host_point(const Affine3& a, const float p[3], float out[3]) {
  for (int i = 0; i < 3; ++i) out[i] = ((a.m[i][0] * p[0] + a.m[i][1] * p[1]) + a.m[i][2] * p[2]) + a.m[i][3];
}

// ============================================================ scene assembly

namespace {

bool as_float(const YNode* n, float* out) {
  if (!n || n->kind != YNode::Scalar) return false;
  const char* s = n->scalar.c_str();
  char* e = nullptr;
  float v = strtof(s, &e);
  if (e == s) return false;
  while (*e == ' ') ++e;
  if (*e != '\0') return false;
  *out = v;
  return true;
}
bool as_int(const YNode* n, int* out) {
  if (!n || n->kind != YNode::Scalar) return false;
  const char* s = n->scalar.c_str();
  char* e = nullptr;
  long v = strtol(s, &e, 10);
  if (e == s) return false;
  while (*e == ' ') ++e;
  if (*e != '\0') return false;
  *out = (int)v;
  return true;
}
bool as_vec(const YNode* n, int k, float* out) {
  if (!n || n->kind != YNode::Seq || (int)n->seq.size() != k) return false;
  for (int i = 0; i < k; ++i)
    if (!as_float(&n->seq[i], &out[i])) return false;
  return true;
}
std::string as_str(const YNode* n) { return (n && n->kind == YNode::Scalar) ? n->scalar : std::string(); }

struct Ctx {
  std::string* err;
  bool fail(const std::string& m) { *err = m; return false; }
};

// One texture node (Constant / Standard / Layered, recursively), appended to
// the scene's node table; returns its index or -1 after c.fail.
int decode_tex_node(const YNode* n, SceneDesc* S, const std::string& dir, Ctx& c, int depth) {
  if (depth > 16) { c.fail("texture layers nest deeper than 16"); return -1; }
  std::string ty = as_str(n ? n->get("type") : nullptr);
  TexNode t;
  memset(&t, 0, sizeof(t));
  t.image = t.upper = t.lower = t.mask = -1;
  if (ty == "Constant") {  // ConstantTexture.h:74-85
    t.type = TEXNODE_CONSTANT;
    if (n->size() != 2 || !as_vec(n->get("colour"), 3, t.colour)) { c.fail("bad Constant texture"); return -1; }
  } else if (ty == "Standard") {  // StandardTexture.h:69-81: the path is relative to the scene's folder
    t.type = TEXNODE_STANDARD;
    std::string rel = as_str(n->get("string"));
    if (n->size() != 2 || rel.empty()) { c.fail("bad Standard texture (needs string)"); return -1; }
    const std::string path = dir + "/" + rel;
    int found = -1;
    for (size_t i = 0; i < S->image_paths.size(); ++i)
      if (S->image_paths[i] == path) found = (int)i;
    if (found < 0) {
      TexImage img;
      if (!image_load(path, &img, c.err)) return -1;
      S->images.push_back(std::move(img));
      S->image_paths.push_back(path);
      found = (int)S->images.size() - 1;
    }
    t.image = found;
  } else if (ty == "Layered") {  // LayeredTexture.h:101-178
    t.type = TEXNODE_LAYERED;
    if (n->size() != 4) { c.fail("bad Layered texture (needs upper, lower, mask)"); return -1; }
    const int u = decode_tex_node(n->get("upper"), S, dir, c, depth + 1);
    if (u < 0) return -1;
    const int l = decode_tex_node(n->get("lower"), S, dir, c, depth + 1);
    if (l < 0) return -1;
    const int m = decode_tex_node(n->get("mask"), S, dir, c, depth + 1);
    if (m < 0) return -1;
    t.upper = u;
    t.lower = l;
    t.mask = m;
  } else {
    c.fail("unknown texture type '" + ty + "'");
    return -1;
  }
  S->tex_nodes.push_back(t);
  return (int)S->tex_nodes.size() - 1;
}

bool decode_texture(const YNode* n, ShaderRec* sh, SceneDesc* S, const std::string& dir, Ctx& c) {
  FaceTexels* ft = &S->texels;
  std::string ty = as_str(n ? n->get("type") : nullptr);
  sh->texture = TEXTURE_CONSTANT;
  sh->tex_root = -1;
  if (ty == "Constant") {  // include/core/ConstantTexture.h:74-85
    if (n->size() != 2 || !as_vec(n->get("colour"), 3, sh->colour)) return c.fail("bad Constant texture");
    return true;
  }
  if (ty == "FaceTexels") {  // extension: per-face res x res FP16 RGB texels, tinted by colour
    int res = 0, seed = 0;
    if (n->size() != 4 || !as_int(n->get("resolution"), &res) || !as_int(n->get("seed"), &seed) ||
        !as_vec(n->get("colour"), 3, sh->colour) || res < 1 || res > 256)
      return c.fail("bad FaceTexels texture (needs resolution 1-256, seed, colour)");
    if (ft->res != 0 && (ft->res != res || ft->seed != (uint32_t)seed))
      return c.fail("every FaceTexels texture of a scene must share one resolution and seed");
    ft->res = res;
    ft->seed = (uint32_t)seed;
    sh->texture = TEXTURE_FACE;
    return true;
  }
  if (ty == "Standard" || ty == "Layered") {
    const int root = decode_tex_node(n, S, dir, c, 0);
    if (root < 0) return false;
    sh->texture = TEXTURE_TREE;
    sh->tex_root = root;
    return true;
  }
  return c.fail("unknown texture type '" + ty + "'");
}

}  // namespace

// ---------------------------------------------------------------- images
// PFM: "PF" (RGB) or "Pf" (grey), width height, scale (< 0: little endian),
// rows bottom first.  PPM: "P6", width height, maxval (< 256: 8 bit, else 16
// bit big endian), rows top first, values / maxval.  OpenEXR: uncompressed
// scanline files (read_exr_rgb).  All end up top first.
bool read_exr_rgb(const std::string& path, int* w, int* h, std::vector<float>* rgb, std::string* err);

bool image_load(const std::string& path, TexImage* out, std::string* err) {
  std::ifstream f(path, std::ios::binary);
  if (!f) { *err = "cannot open texture image [" + path + "]"; return false; }
  std::string data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  if (data.size() >= 4 && (unsigned char)data[0] == 0x76 && (unsigned char)data[1] == 0x2f &&
      (unsigned char)data[2] == 0x31 && (unsigned char)data[3] == 0x01)
    return read_exr_rgb(path, &out->width, &out->height, &out->rgb, err);
  size_t p = 0;
  auto token = [&]() {
    while (p < data.size()) {
      if (data[p] == '#') { while (p < data.size() && data[p] != '\n') ++p; }
      else if (isspace((unsigned char)data[p])) ++p;
      else break;
    }
    size_t b = p;
    while (p < data.size() && !isspace((unsigned char)data[p])) ++p;
    return data.substr(b, p - b);
  };
  const std::string magic = token();
  const long w = atol(token().c_str()), h = atol(token().c_str());
  const std::string third = token();
  if (p < data.size()) ++p;  // the single whitespace before the raster
  if (w <= 0 || h <= 0 || w > 65536 || h > 65536) { *err = "bad image size in [" + path + "]"; return false; }
  out->width = (int)w;
  out->height = (int)h;
  out->rgb.assign((size_t)w * h * 3, 0.f);
  const unsigned char* r = (const unsigned char*)data.data() + p;
  const size_t left = data.size() - p;
  if (magic == "PF" || magic == "Pf") {
    const int ch = magic == "PF" ? 3 : 1;
    const bool little = atof(third.c_str()) < 0.0;
    if (left < (size_t)w * h * ch * 4) { *err = "truncated PFM [" + path + "]"; return false; }
    for (long y = 0; y < h; ++y)
      for (long x = 0; x < w; ++x)
        for (int k = 0; k < 3; ++k) {
          const unsigned char* q = r + 4 * (((size_t)y * w + x) * ch + (ch == 3 ? k : 0));
          uint32_t u = little ? (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16) | ((uint32_t)q[3] << 24)
                              : (uint32_t)q[3] | ((uint32_t)q[2] << 8) | ((uint32_t)q[1] << 16) | ((uint32_t)q[0] << 24);
          float v;
          memcpy(&v, &u, 4);
          out->rgb[(((size_t)(h - 1 - y)) * w + x) * 3 + k] = v;  // bottom row first in the file
        }
    return true;
  }
  if (magic == "P6") {
    const long maxv = atol(third.c_str());
    if (maxv <= 0 || maxv > 65535) { *err = "bad PPM maxval in [" + path + "]"; return false; }
    const int bps = maxv < 256 ? 1 : 2;
    if (left < (size_t)w * h * 3 * bps) { *err = "truncated PPM [" + path + "]"; return false; }
    for (size_t i = 0; i < (size_t)w * h * 3; ++i) {
      const uint32_t v = bps == 1 ? r[i] : ((uint32_t)r[2 * i] << 8) | r[2 * i + 1];
      out->rgb[i] = (float)v / (float)maxv;
    }
    return true;
  }
  *err = "texture image [" + path + "] is not PFM, binary PPM or OpenEXR";
  return false;
}

bool load_scene(const std::string& yaml_path, SceneDesc* out, std::string* err) {
  std::ifstream f(yaml_path, std::ios::binary);
  if (!f) { *err = "cannot open scene file [" + yaml_path + "]"; return false; }
  std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  std::vector<YNode> docs;
  if (!yaml_parse_documents(text, &docs, err)) return false;
  Ctx c{err};
  if (docs.size() < 2) return c.fail("scene file needs a setup document and a scene document");
  std::string dir = ".";
  size_t slash = yaml_path.find_last_of('/');
  if (slash != std::string::npos) dir = yaml_path.substr(0, slash);
  *out = SceneDesc();
  SceneDesc& S = *out;
  const YNode& setup = docs[0];
  const YNode& scene = docs[1];

  // camera default: ThinLens with the default constructor's values
  {
    float t[3] = {0, 0, 0}, r[3] = {0, 0, 0};
    S.camera.type = CAMERA_THINLENS;
    S.camera.xf = make_tr_yxz(t, r);
    normal_of_x_axis(S.camera.xf, S.camera.normal);
    for (int i = 0; i < 3; ++i) S.camera.translation[i] = 0;
    S.camera.focal_length = 55.f;
    S.camera.aperture = 5.6f;
    S.camera.focal_distance = 1000.f;
  }
  if (const YNode* n = setup.get("image")) {  // Image.h:56-69
    if (n->kind != YNode::Map || n->size() != 3 || !as_int(n->get("width"), &S.width) ||
        !as_int(n->get("height"), &S.height) || !as_int(n->get("sample base"), &S.base))
      return c.fail("bad image block (needs width, height, sample base)");
    if (S.width <= 0 || S.height <= 0 || S.base <= 0) return c.fail("image sizes must be positive");
  }
  if (const YNode* n = setup.get("settings")) {  // Settings.h:30-45
    Settings& st = S.settings;
    if (n->kind != YNode::Map || n->size() != 6 || !as_int(n->get("min depth"), &st.min_depth) ||
        !as_int(n->get("max depth"), &st.max_depth) || !as_float(n->get("threshold"), &st.threshold) ||
        !as_int(n->get("bucket size"), &st.bucket_size) || !as_int(n->get("shading size"), &st.shading_size) ||
        !as_int(n->get("bin exponent"), &st.bin_exponent))
      return c.fail("bad settings block");
    if (st.bin_exponent < 6 || st.bin_exponent > 26) return c.fail("bin exponent must lie in [6, 26]");
  }
  if (const YNode* n = setup.get("camera")) {
    std::string ty = as_str(n->get("type"));
    float t[3], r[3];
    if (ty == "PinHole") {  // PinHoleCamera.h:98-113
      if (n->size() != 4 || !as_vec(n->get("translation"), 3, t) || !as_vec(n->get("rotation"), 3, r) ||
          !as_float(n->get("focal length"), &S.camera.focal_length))
        return c.fail("bad PinHole camera");
      S.camera.type = CAMERA_PINHOLE;
    } else if (ty == "ThinLens") {  // ThinLensCamera.h:132-149
      if (n->size() != 6 || !as_vec(n->get("translation"), 3, t) || !as_vec(n->get("rotation"), 3, r) ||
          !as_float(n->get("focal length"), &S.camera.focal_length) ||
          !as_float(n->get("focal distance"), &S.camera.focal_distance) ||
          !as_float(n->get("aperture"), &S.camera.aperture))
        return c.fail("bad ThinLens camera");
      S.camera.type = CAMERA_THINLENS;
    } else {
      return c.fail("unknown camera type '" + ty + "'");
    }
    S.camera.xf = make_tr_yxz(t, r);
    normal_of_x_axis(S.camera.xf, S.camera.normal);
    for (int i = 0; i < 3; ++i) S.camera.translation[i] = t[i];
  }
  if (const YNode* n = setup.get("filter")) {
    std::string ty = as_str(n->get("type"));
    if (n->size() != 1) return c.fail("bad filter block");
    if (ty == "Tent") S.filter = FILTER_TENT;
    else if (ty == "Box") S.filter = FILTER_BOX;
    else return c.fail("unknown filter type '" + ty + "'");
  }
  if (const YNode* n = setup.get("sampler")) {
    std::string ty = as_str(n->get("type"));
    if (n->size() != 1) return c.fail("bad sampler block");
    if (ty == "Stratified") S.sampler = SAMPLER_STRATIFIED;
    else if (ty == "Independent") S.sampler = SAMPLER_INDEPENDENT;
    else if (ty == "Grid") S.sampler = SAMPLER_GRID;
    else return c.fail("unknown sampler type '" + ty + "'");
  }
  if (docs.size() >= 3) {
    const YNode* e = docs[2].get("extensions");
    if (e) {
      for (const auto& kv : e->map) {
        int iv = 0;
        if (kv.first == "samples per pixel") { if (!as_int(&kv.second, &S.ext.spp) || S.ext.spp <= 0) return c.fail("bad samples per pixel"); }
        else if (kv.first == "mis") {
          std::string m = as_str(&kv.second);
          if (m == "power") S.ext.mis_power = 1;
          else if (m == "balance") S.ext.mis_power = 0;
          else return c.fail("mis must be power or balance");
        }
        else if (kv.first == "ray sort") { if (!as_int(&kv.second, &S.ext.ray_sort)) return c.fail("bad ray sort"); }
        else if (kv.first == "hit sort") { if (!as_int(&kv.second, &S.ext.hit_sort)) return c.fail("bad hit sort"); }
        else if (kv.first == "autotune") { if (!as_int(&kv.second, &S.ext.autotune)) return c.fail("bad autotune"); }
        else if (kv.first == "direction bins") {
          if (!as_int(&kv.second, &S.ext.bins) || (S.ext.bins != 6 && S.ext.bins != 26 && S.ext.bins != 98))
            return c.fail("direction bins must be 6, 26 or 98");
        }
        else if (kv.first == "seed") { if (!as_int(&kv.second, &iv)) return c.fail("bad seed"); S.ext.seed = (uint32_t)iv; }
        else if (kv.first == "bvh") {
          std::string m = as_str(&kv.second);
          if (m == "wide") S.ext.wide_bvh = 1;
          else if (m == "binary") S.ext.wide_bvh = 0;
          else return c.fail("bvh must be wide or binary");
        }
        else if (kv.first == "hit key bits") {
          if (!as_int(&kv.second, &S.ext.hit_key_bits) || (S.ext.hit_key_bits != 32 && S.ext.hit_key_bits != 64))
            return c.fail("hit key bits must be 32 or 64");
        }
        else if (kv.first == "paths per generation") { if (!as_int(&kv.second, &S.ext.generation) || S.ext.generation < 0) return c.fail("bad paths per generation"); }
        else return c.fail("unknown extension '" + kv.first + "'");
      }
    }
  }

  const int workers = (int)std::max(1u, std::min(std::thread::hardware_concurrency(), 32u));
  auto add_tris = [&](const std::vector<float>& pos3, const std::vector<uint32_t>& idx, const std::vector<float>& uv,
                      int geom, bool light) {
    const size_t nt = idx.size() / 3, b = S.tri_geom.size();
    S.tri_v.resize(9 * (b + nt));
    S.tri_uv.resize(6 * (b + nt));
    S.tri_geom.resize(b + nt, geom);
    S.tri_is_light.resize(b + nt, light ? 1 : 0);
    auto fill = [&](size_t t0, size_t t1) {
      for (size_t t = t0; t < t1; ++t) {
        float* tv = &S.tri_v[9 * (b + t)];
        float* tu = &S.tri_uv[6 * (b + t)];
        for (int k = 0; k < 3; ++k) {
          const uint32_t vi = idx[3 * t + k];
          for (int a = 0; a < 3; ++a) tv[3 * k + a] = pos3[3 * vi + a];
          const bool has_uv = (size_t)(2 * vi + 1) < uv.size();
          tu[2 * k + 0] = has_uv ? uv[2 * vi + 0] : 0.f;
          tu[2 * k + 1] = has_uv ? uv[2 * vi + 1] : 0.f;
        }
      }
    };
    if (nt < (1u << 16)) fill(0, nt);
    else parallel_for(workers, [&](int w) { fill(nt * w / workers, nt * (w + 1) / workers); });
  };

  if (scene.kind != YNode::Map && scene.kind != YNode::Null) return c.fail("scene document must be a mapping");
  // OBJ files named by several objects are read once
  std::vector<std::pair<std::string, ObjMesh>> obj_cache;
  // First pass: objects and shaders in document order (Pathtracer.cpp:166-217).
  for (const auto& kv : scene.map) {
    const YNode& n = kv.second;
    if (kv.first == "object") {
      std::string ty = as_str(n.get("type"));
      if (ty != "Polygon") continue;
      float t[3], r[3], s[3];
      int shader = 0;
      std::string fname = as_str(n.get("filename"));
      if (n.size() != 6 || fname.empty() || !as_vec(n.get("translation"), 3, t) || !as_vec(n.get("rotation"), 3, r) ||
          !as_vec(n.get("scale"), 3, s) || !as_int(n.get("shader"), &shader))
        return c.fail("bad Polygon object");
      const ObjMesh* found = nullptr;
      for (const auto& e : obj_cache)
        if (e.first == fname) found = &e.second;
      if (!found) {
        ObjMesh m;
        if (!obj_load_file(dir + "/" + fname, &m, err)) return false;
        obj_cache.emplace_back(fname, std::move(m));
        found = &obj_cache.back().second;
      }
      const ObjMesh& mesh = *found;
      Affine3 xf = make_trs_xyz(t, r, s);  // PolygonObject.cpp:17-22
      std::vector<float> pos(mesh.positions.size());
      const size_t nvert = mesh.positions.size() / 3;
      auto xf_range = [&](size_t v0, size_t v1) {
        for (size_t i = v0; i < v1; ++i) xf_host_point(xf, &mesh.positions[3 * i], &pos[3 * i]);
      };
      if (nvert < (1u << 16)) xf_range(0, nvert);
      else parallel_for(workers, [&](int w) { xf_range(nvert * w / workers, nvert * (w + 1) / workers); });
      GeomRec g;
      g.shader = shader;
      g.first_prim = (int)S.tri_geom.size();
      g.prim_count = (int)(mesh.indices.size() / 3);
      g.light = -1;
      S.geoms.push_back(g);
      add_tris(pos, mesh.indices, mesh.texcoords, (int)S.geoms.size() - 1, false);
    } else if (kv.first == "shader") {
      std::string ty = as_str(n.get("type"));
      ShaderRec sh;
      memset(&sh, 0, sizeof(sh));
      sh.light = -1;
      if (ty == "Lambert") {  // LambertShader.h:140-174
        sh.type = SHADER_LAMBERT;
        if (n.size() != 3 || !as_float(n.get("reflectance"), &sh.reflectance)) return c.fail("bad Lambert shader");
        if (!decode_texture(n.get("texture"), &sh, &S, dir, c)) return false;
      } else if (ty == "Phong") {  // extension: modified Phong lobe
        sh.type = SHADER_PHONG;
        if (n.size() != 4 || !as_float(n.get("reflectance"), &sh.reflectance) ||
            !as_float(n.get("exponent"), &sh.exponent) || sh.exponent < 0.f)
          return c.fail("bad Phong shader");
        if (!decode_texture(n.get("texture"), &sh, &S, dir, c)) return false;
      } else {
        continue;
      }
      S.shaders.push_back(sh);
    }
  }
  // Second pass: lights (Pathtracer.cpp:219-272).  Each adds a Null shader,
  // an empty object pointing at it, and the emitter triangles.
  for (const auto& kv : scene.map) {
    if (kv.first != "light") continue;
    const YNode& n = kv.second;
    std::string ty = as_str(n.get("type"));
    if (ty == "Sphere") {  // extension: a sphere of uniform radiance, not triangle geometry
      LightRec L;
      memset(&L, 0, sizeof(L));
      L.type = LIGHT_SPHERE;
      if (n.size() != 4 || !as_vec(n.get("translation"), 3, L.centre) || !as_float(n.get("radius"), &L.radius) ||
          !as_float(n.get("intensity"), &L.intensity) || !(L.radius > 0.f))
        return c.fail("bad Sphere light (needs translation, radius > 0, intensity)");
      const int light_id = (int)S.lights.size();
      ShaderRec ns;
      memset(&ns, 0, sizeof(ns));
      ns.type = SHADER_NULL;
      ns.light = light_id;
      ns.reflectance = 1.f;
      S.shaders.push_back(ns);
      S.lights.push_back(L);
      S.sphere_lights.push_back(light_id);
      continue;
    }
    if (ty != "Quad") continue;
    LightRec L;
    memset(&L, 0, sizeof(L));
    L.type = LIGHT_QUAD;
    float t[3], r[3];
    if (n.size() != 5 || !as_vec(n.get("translation"), 3, t) || !as_vec(n.get("rotation"), 3, r) ||
        !as_vec(n.get("scale"), 2, L.scale) || !as_float(n.get("intensity"), &L.intensity))
      return c.fail("bad Quad light");
    float s3[3] = {1.f, L.scale[0], L.scale[1]};
    L.xf = make_trs_xyz(t, r, s3);
    normal_of_x_axis(L.xf, L.normal);
    int light_id = (int)S.lights.size();
    int shader_id = (int)S.shaders.size();
    ShaderRec ns;
    memset(&ns, 0, sizeof(ns));
    ns.type = SHADER_NULL;
    ns.light = light_id;
    ns.reflectance = 1.f;
    S.shaders.push_back(ns);
    GeomRec g;
    g.shader = shader_id;
    g.first_prim = (int)S.tri_geom.size();
    g.prim_count = 2;
    g.light = light_id;
    S.geoms.push_back(g);
    S.lights.push_back(L);
    // unit quad in the local YZ plane (QuadLight.cpp:7-21)
    const float quad[6][3] = {{0.f, -0.5f, -0.5f}, {0.f, 0.5f, -0.5f}, {0.f, 0.5f, 0.5f},
                              {0.f, 0.5f, 0.5f},   {0.f, -0.5f, 0.5f}, {0.f, -0.5f, -0.5f}};
    std::vector<float> pos(18);
    for (int i = 0; i < 6; ++i) xf_host_point(L.xf, quad[i], &pos[3 * i]);
    std::vector<uint32_t> idx = {0, 1, 2, 3, 4, 5};
    add_tris(pos, idx, std::vector<float>(), (int)S.geoms.size() - 1, true);
  }
  for (size_t g = 0; g < S.geoms.size(); ++g) {
    int sh = S.geoms[g].shader;
    if (sh < 0 || sh >= (int)S.shaders.size())
      return c.fail("object " + std::to_string(g) + " names shader " + std::to_string(sh) + " which does not exist");
  }
  return true;
}

}  // namespace mscg
