// Model::Model(model_folder, model_name, skyMap_name) (src/model.cpp:124-215,
// src/material.cpp:150-336, src/component.cpp:69-114) for Wavefront OBJ/MTL
// models: rmn_model_read parses the files, decodes the textures and the sky
// map (image_io.cpp) and lays the result out as an rmn_scene_desc.
//
// The reference imports with assimp (aiProcess_Triangulate |
// PreTransformVertices | SortByPType | FixInfacingNormals, with
// AI_CONFIG_PP_PTV_KEEP_HIERARCHY); the library does not use assimp. What it
// does for OBJ files is restated from its documented behaviour:
//  * one mesh per run of faces with the same object/group and material; a
//    vertex per face corner; polygons as a fan from their first corner;
//    lines and points dropped;
//  * materials: assimp's default material first, then the MTL files' in
//    definition order, then usemtl names no MTL defines; per material only
//    what Material::loadMaterialProperties reads -- the name, the opacity (d,
//    or 1 - Tr; below 0.99 the glass parameters by name) and the textures
//    map_Kd (diffuse), map_Ks (specular), map_Ke (emissive), norm / map_Kn
//    (normal map); texture paths are folder + path with backslashes made
//    slashes and %XX decoded (urlDecode, src/material.cpp:9-24), dispatched
//    on the extension (loadImageFromFile, src/material.cpp:287-298);
//  * FixInfacingNormals' bounding-box test flips a mesh's normals.
// Corners without a normal in a mesh give the whole mesh geometric normals,
// corners without texture coordinates (0, 0) (the reference dereferences
// assimp's missing arrays). RGB images become RGBA with opaque alpha (the
// reference leaves ImageData::channels unset for PNG files).
#include <algorithm>
#include <array>
#include <atomic>
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <map>
#include <string>
#include <string_view>
#include <thread>
#include <vector>

#include "rmn_host.h"

struct rmn_model {
  std::vector<float> positions, normals, uvs, env;
  std::vector<int32_t> indices, mesh_first, mesh_material, material_textures;
  std::vector<rmn_material> materials;
  std::vector<std::string> material_names;
  std::vector<std::vector<uint8_t>> texels;
  std::vector<rmn_texture> textures;
  int32_t env_w = 0, env_h = 0;
};

namespace {

using rmn::fail;

const char* const kDefaultMaterial = "DefaultMaterial";

using rmn::run_threads;

bool read_text(const std::string& path, std::string& out) { return rmn::read_whole_file(path.c_str(), out); }

// Lines as a text reader sees them: "\r\n" and "\r" end lines too, and a
// backslash before the end of a line continues it (OBJ only).
std::vector<std::string> split_lines(const std::string& text, bool continuation) {
  std::string t;
  t.reserve(text.size());
  for (size_t i = 0; i < text.size(); ++i) {
    char c = text[i];
    if (c == '\r') {
      if (i + 1 < text.size() && text[i + 1] == '\n') continue;
      c = '\n';
    }
    if (continuation && c == '\n' && !t.empty() && t.back() == '\\') {
      t.back() = ' ';
      continue;
    }
    t.push_back(c);
  }
  std::vector<std::string> lines;
  size_t start = 0;
  for (size_t i = 0; i <= t.size(); ++i) {
    const char c = i < t.size() ? t[i] : '\n';
    if (c == '\n' || c == '\v' || c == '\f' || c == '\x1c' || c == '\x1d' || c == '\x1e') {
      if (i < t.size() || start < t.size()) lines.emplace_back(t, start, i - start);
      start = i + 1;
    }
  }
  return lines;
}

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\v' || c == '\f' || c == '\r' || c == '\n'; }

std::vector<std::string> tokens(const std::string& s) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < s.size()) {
    while (i < s.size() && is_space(s[i])) ++i;
    size_t j = i;
    while (j < s.size() && !is_space(s[j])) ++j;
    if (j > i) out.emplace_back(s, i, j - i);
    i = j;
  }
  return out;
}

std::string strip(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && is_space(s[a])) ++a;
  while (b > a && is_space(s[b - 1])) --b;
  return s.substr(a, b - a);
}

// (key, rest) of a stripped line: the first token and the stripped remainder.
void key_rest(const std::string& line, std::string& key, std::string& rest) {
  size_t i = 0;
  while (i < line.size() && !is_space(line[i])) ++i;
  key = line.substr(0, i);
  rest = strip(line.substr(i));
}

using sv = std::string_view;

// A sign '+' is allowed before a number, as a text reader allows it.
sv drop_plus(sv t) {
  if (t.size() > 1 && t[0] == '+' && t[1] != '+' && t[1] != '-') t.remove_prefix(1);
  return t;
}

// A decimal number, the whole token (std::from_chars: correctly rounded to
// double; hexadecimal and "nan(...)" forms are not numbers here; a value
// beyond double's range is +-inf or 0 as strtod gives it).
bool sv_double(sv t, double* v) {
  if (t.empty() || t.find_first_of("xX(") != sv::npos) return false;
  t = drop_plus(t);
  const auto r = std::from_chars(t.data(), t.data() + t.size(), *v);
  if (r.ptr != t.data() + t.size()) return false;
  if (r.ec == std::errc::result_out_of_range) {
    const std::string z(t);
    *v = std::strtod(z.c_str(), nullptr);
    return true;
  }
  return r.ec == std::errc();
}

bool sv_long(sv t, long long* v) {
  t = drop_plus(t);
  if (t.empty()) return false;
  const auto r = std::from_chars(t.data(), t.data() + t.size(), *v);
  return r.ec == std::errc() && r.ptr == t.data() + t.size();
}

bool parse_double(const std::string& t, double* v) { return sv_double(sv(t), v); }

std::string lower(std::string s) {
  for (char& c : s)
    if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
  return s;
}

// urlDecode: %XX (the leading hex digits of the next two characters) to a byte.
std::string url_decode(const std::string& s) {
  std::string out;
  for (size_t i = 0; i < s.size();) {
    if (s[i] == '%') {
      int n = 0;
      for (size_t k = i + 1; k < i + 3 && k < s.size(); ++k) {
        const char c = s[k];
        int d = c >= '0' && c <= '9' ? c - '0' : c >= 'a' && c <= 'f' ? c - 'a' + 10 : c >= 'A' && c <= 'F' ? c - 'A' + 10 : -1;
        if (d < 0) break;
        n = n * 16 + d;
      }
      out.push_back((char)(n & 0xFF));
      i += 3;
    } else {
      out.push_back(s[i++]);
    }
  }
  return out;
}

// The file name of a texture statement after its options (each option takes
// its arguments as long as a file name is left after them; -o/-s/-t/-mm stop
// at the first non-number).
std::string texture_path(const std::string& rest) {
  static const std::map<std::string, int> kOptions = {
      {"-blendu", 1}, {"-blendv", 1}, {"-cc", 1}, {"-clamp", 1}, {"-imfchan", 1}, {"-texres", 1}, {"-bm", 1},
      {"-boost", 1},  {"-mm", 2},     {"-o", 3},  {"-s", 3},     {"-t", 3},       {"-type", 1}};
  const std::vector<std::string> t = tokens(rest);
  size_t i = 0;
  while (i + 1 < t.size()) {
    auto it = kOptions.find(lower(t[i]));
    if (it == kOptions.end()) break;
    ++i;
    for (int k = 0; k < it->second; ++k) {
      if (i >= t.size() - 1) break;
      double dummy;
      if (k > 0 && !parse_double(t[i], &dummy)) break;
      ++i;
    }
  }
  std::string out;
  for (size_t k = i; k < t.size(); ++k) out += (k > i ? " " : "") + t[k];
  return out;
}

struct MtlSpec {
  std::string name;
  float opacity = 1.0f;  // ai_real, as assimp hands AI_MATKEY_OPACITY over
  std::map<int, std::string> textures;  // slot -> file name
};

rmn_status parse_mtl(const std::string& path, std::vector<MtlSpec>& mats) {
  std::string text;
  if (!read_text(path, text)) return RMN_OK;  // a missing library is skipped
  const std::vector<std::string> lines = split_lines(text, false);
  for (size_t ln = 0; ln < lines.size(); ++ln) {
    const std::string line = strip(lines[ln]);
    if (line.empty() || line[0] == '#') continue;
    std::string key, rest;
    key_rest(line, key, rest);
    const std::string k = lower(key);
    if (k == "newmtl") {
      mats.push_back(MtlSpec{rest, 1.0f, {}});
      continue;
    }
    if (mats.empty()) continue;
    if (k == "d" || k == "tr") {
      const std::vector<std::string> t = tokens(rest);
      double v;
      if (t.empty() || !parse_double(t.back(), &v))
        return fail(RMN_ERR_INVALID_ARGUMENT, "%s:%zu: cannot read '%.60s'", path.c_str(), ln + 1, line.c_str());
      mats.back().opacity = k == "d" ? (float)v : 1.0f - (float)v;
    } else if (k == "map_kd") {
      mats.back().textures[RMN_TEX_DIFFUSE] = texture_path(rest);
    } else if (k == "map_ks") {
      mats.back().textures[RMN_TEX_SPECULAR] = texture_path(rest);
    } else if (k == "map_ke") {
      mats.back().textures[RMN_TEX_EMISSIVE] = texture_path(rest);
    } else if (k == "norm" || k == "map_kn") {
      mats.back().textures[RMN_TEX_NORMALS] = texture_path(rest);
    }
  }
  return RMN_OK;
}

struct Corner {
  long long v, t, n;
};
struct MeshRun {
  std::string mat;
  std::vector<Corner> corners;
  std::vector<int32_t> tris;  // 3 corner indices per triangle
};

// The OBJ parse works on views into the normalised text: no allocation per
// line or token.

bool sv_space(char c) { return is_space(c); }

sv sv_strip(sv s) {
  while (!s.empty() && sv_space(s.front())) s.remove_prefix(1);
  while (!s.empty() && sv_space(s.back())) s.remove_suffix(1);
  return s;
}

// The next whitespace-separated token of s (s advances past it); empty at the end.
sv next_token(sv& s) {
  while (!s.empty() && sv_space(s.front())) s.remove_prefix(1);
  size_t j = 0;
  while (j < s.size() && !sv_space(s[j])) ++j;
  sv t = s.substr(0, j);
  s.remove_prefix(j);
  return t;
}


// One piece of the OBJ text, parsed on its own: the v / vt / vn values, the
// face corners and, in order, the statements that shape the meshes. A
// negative or zero index counts back from the vertices read so far, which
// include the pieces before this one, so it is kept relative (its bit in
// `rel`) and completed when the pieces are joined.
struct ObjOp {
  enum Kind : uint8_t { kFace, kUseMtl, kClose, kMtlLib } kind;
  uint32_t a, b;  // kFace: corners [a, a + b); kUseMtl: names[a]; kMtlLib: names [a, a + b)
};
struct ObjPiece {
  std::vector<float> P, T, N;
  std::vector<Corner> corners;
  std::vector<uint8_t> rel;  // bit 0 / 1 / 2: v / t / n relative to the counts before the piece
  std::vector<ObjOp> ops;
  std::vector<std::string> names;
  size_t lines = 0;
  size_t bad_line = 0;  // line of the first statement that cannot be read (within the piece), 0: none
  std::string bad_text;
};

// The lines of text[begin, end), which starts a line and ends after a line
// end (or at the end of the text), in order.
void parse_obj_piece(sv text, ObjPiece& out) {
  std::vector<Corner> cs;
  std::vector<uint8_t> rs;
  size_t ln = 0, start = 0;
  for (size_t i = 0; i <= text.size(); ++i) {
    const char ch = i < text.size() ? text[i] : '\n';
    if (!(ch == '\n' || ch == '\v' || ch == '\f' || ch == '\x1c' || ch == '\x1d' || ch == '\x1e')) continue;
    if (i == text.size() && start >= text.size()) break;
    ++ln;
    const sv line = sv_strip(text.substr(start, i - start));
    start = i + 1;
    if (line.empty() || line[0] == '#') continue;
    auto bad = [&]() {
      out.bad_line = ln;
      out.bad_text = std::string(line.substr(0, 60));
    };
    sv rest = line;
    const sv key = next_token(rest);
    rest = sv_strip(rest);
    if (key == "v" || key == "vn") {
      std::vector<float>& dst = key == "v" ? out.P : out.N;
      bool ok = true;
      for (int k = 0; k < 3 && ok; ++k) {
        double d;
        ok = sv_double(next_token(rest), &d);
        if (ok) dst.push_back((float)d);
      }
      if (!ok) return bad();
    } else if (key == "vt") {
      double u, v = 0.0;
      if (!sv_double(next_token(rest), &u)) return bad();
      const sv second = next_token(rest);
      if (!second.empty() && !sv_double(second, &v)) return bad();
      out.T.push_back((float)u);
      out.T.push_back((float)v);
    } else if (key == "f") {
      cs.clear();
      rs.clear();
      for (sv tok = next_token(rest); !tok.empty(); tok = next_token(rest)) {
        sv parts[3];
        int np = 0;
        size_t a = 0;
        for (size_t b = 0; b <= tok.size(); ++b)
          if (b == tok.size() || tok[b] == '/') {
            if (np < 3) parts[np] = tok.substr(a, b - a);
            ++np;
            a = b + 1;
          }
        uint8_t r = 0;
        auto index = [&r](sv s, size_t n, int bit, long long* idx) {
          long long i;
          if (!sv_long(s, &i)) return false;
          if (i > 0) {
            *idx = i - 1;
          } else {
            *idx = (long long)n + i;
            r |= (uint8_t)bit;
          }
          return true;
        };
        Corner c{0, -1, -1};
        if (!index(parts[0], out.P.size() / 3, 1, &c.v)) return bad();
        if (np > 1 && !parts[1].empty() && !index(parts[1], out.T.size() / 2, 2, &c.t)) return bad();
        if (np > 2 && !parts[2].empty() && !index(parts[2], out.N.size() / 3, 4, &c.n)) return bad();
        cs.push_back(c);
        rs.push_back(r);
      }
      if (cs.size() < 3) continue;
      out.ops.push_back({ObjOp::kFace, (uint32_t)out.corners.size(), (uint32_t)cs.size()});
      out.corners.insert(out.corners.end(), cs.begin(), cs.end());
      out.rel.insert(out.rel.end(), rs.begin(), rs.end());
    } else if (key == "usemtl") {
      out.ops.push_back({ObjOp::kUseMtl, (uint32_t)out.names.size(), 1});
      out.names.emplace_back(rest);
    } else if (key == "o" || key == "g") {
      out.ops.push_back({ObjOp::kClose, 0, 0});
    } else if (key == "mtllib") {
      const uint32_t first = (uint32_t)out.names.size();
      for (sv m = next_token(rest); !m.empty(); m = next_token(rest)) out.names.emplace_back(m);
      out.ops.push_back({ObjOp::kMtlLib, first, (uint32_t)out.names.size() - first});
    }
  }
  out.lines = ln;
}

// Pieces of at least this many bytes, at most one per hardware thread (16 at most).
constexpr size_t kObjPieceBytes = 64 << 10;

rmn_status parse_obj(const std::string& path, std::vector<float>& P, std::vector<float>& T, std::vector<float>& N,
                     std::vector<MeshRun>& meshes, std::vector<std::string>& mtllibs) {
  std::string raw;
  if (!read_text(path, raw)) return fail(RMN_ERR_INVALID_ARGUMENT, "could not read %s", path.c_str());
  // the text with "\r\n" / "\r" as "\n" and continued lines joined
  std::string t;
  if (raw.find('\r') == std::string::npos && raw.find("\\\n") == std::string::npos) {
    t.swap(raw);
  } else {
    t.reserve(raw.size());
    for (size_t i = 0; i < raw.size(); ++i) {
      char c = raw[i];
      if (c == '\r') {
        if (i + 1 < raw.size() && raw[i + 1] == '\n') continue;
        c = '\n';
      }
      if (c == '\n' && !t.empty() && t.back() == '\\') {
        t.back() = ' ';
        continue;
      }
      t.push_back(c);
    }
    std::string().swap(raw);
  }
  // pieces that start at line starts, parsed on separate threads
  const size_t want = std::max<size_t>(1, std::min(rmn::host_threads(), t.size() / kObjPieceBytes));
  std::vector<size_t> cut{0};
  for (size_t k = 1; k < want; ++k) {
    size_t j = std::max(cut.back(), t.size() * k / want);
    while (j < t.size() && !(t[j] == '\n' || t[j] == '\v' || t[j] == '\f' || t[j] == '\x1c' || t[j] == '\x1d' ||
                             t[j] == '\x1e'))
      ++j;
    if (j >= t.size()) break;
    if (j + 1 > cut.back()) cut.push_back(j + 1);
  }
  cut.push_back(t.size());
  const size_t np = cut.size() - 1;
  std::vector<ObjPiece> pieces(np);
  const sv text(t);
  run_threads(np, [&](size_t k) { parse_obj_piece(text.substr(cut[k], cut[k + 1] - cut[k]), pieces[k]); });
  // joined in order: the statements replayed as one reader would meet them
  MeshRun cur{kDefaultMaterial, {}, {}};
  auto close = [&]() {
    if (!cur.tris.empty()) {
      const std::string mat = cur.mat;
      meshes.push_back(std::move(cur));
      cur = MeshRun{mat, {}, {}};
    }
    cur.corners.clear();
    cur.tris.clear();
  };
  size_t lines_before = 0;
  for (const ObjPiece& pc : pieces) {
    if (pc.bad_line)
      return fail(RMN_ERR_INVALID_ARGUMENT, "%s:%zu: cannot read '%s'", path.c_str(), lines_before + pc.bad_line,
                  pc.bad_text.c_str());
    const long long bv = (long long)(P.size() / 3), bt = (long long)(T.size() / 2), bn = (long long)(N.size() / 3);
    P.insert(P.end(), pc.P.begin(), pc.P.end());
    T.insert(T.end(), pc.T.begin(), pc.T.end());
    N.insert(N.end(), pc.N.begin(), pc.N.end());
    for (const ObjOp& op : pc.ops) {
      if (op.kind == ObjOp::kFace) {
        const int32_t base = (int32_t)cur.corners.size();
        for (uint32_t k = 0; k < op.b; ++k) {
          Corner c = pc.corners[op.a + k];
          const uint8_t r = pc.rel[op.a + k];
          if (r & 1) c.v += bv;
          if (r & 2) c.t += bt;
          if (r & 4) c.n += bn;
          cur.corners.push_back(c);
        }
        for (int32_t k = 1; k + 1 < (int32_t)op.b; ++k) {
          cur.tris.push_back(base);
          cur.tris.push_back(base + k);
          cur.tris.push_back(base + k + 1);
        }
      } else if (op.kind == ObjOp::kUseMtl) {
        if (pc.names[op.a] != cur.mat) close();
        cur.mat = pc.names[op.a];
      } else if (op.kind == ObjOp::kClose) {
        close();
      } else {
        for (uint32_t k = 0; k < op.b; ++k) mtllibs.push_back(pc.names[op.a + k]);
      }
    }
    lines_before += pc.lines;
  }
  close();
  return RMN_OK;
}

// Material::loadImageFromFile: the texels as RGBA, or empty (after the
// reference's message) for another extension or a DDS that does not decode.
rmn_status load_texture(const std::string& path, rmn::DecodedImage& img, bool* loaded) {
  *loaded = false;
  const size_t dot = path.rfind('.');
  const std::string ext = dot == std::string::npos ? path : path.substr(dot + 1);
  int kind;
  if (ext == "png" || ext == "PNG") {
    kind = RMN_IMAGE_PNG;
  } else if (ext == "dds" || ext == "DDS") {
    kind = RMN_IMAGE_DDS;
  } else {
    std::fprintf(stderr, "Unsupported file format: %s\n", path.c_str());
    return RMN_OK;
  }
  rmn_status st = rmn::decode_image_file(path.c_str(), kind, false, img);
  if (st != RMN_OK) {
    if (kind == RMN_IMAGE_PNG) return st;  // loadImageFromPNG throws
    std::fprintf(stderr, "Conversion failed: %s\n", rmn_last_error());
    rmn::clear_error();
    return RMN_OK;
  }
  if (img.channels == 3) {
    std::vector<uint8_t> rgba((size_t)img.w * img.h * 4, 255);
    for (size_t i = 0; i < (size_t)img.w * img.h; ++i) std::memcpy(&rgba[4 * i], &img.bytes[3 * i], 3);
    img.bytes.swap(rgba);
    img.channels = 4;
  }
  *loaded = true;
  return RMN_OK;
}

rmn_material default_material() {
  rmn_material m{};
  m.base_color[0] = m.base_color[1] = m.base_color[2] = 1.0f;
  m.has_base = 0.0f;  // no diffuse texel: white unless a texture is given
  m.roughness = 0.8f;
  m.opacity = 1.0f;
  m.ior = 1.0f;
  return m;
}

// loadMaterialProperties for opacity < 0.99 (src/material.cpp:307-329).
rmn_material glass_material(const std::string& name) {
  rmn_material m = default_material();
  m.opacity = 0.0f;
  m.ior = 1.25f;
  m.roughness = name == "Ice" ? 0.5f : 5e-3f;
  static const std::map<std::string, std::array<float, 3>> kColours = {
      {"TransparentGlassWine", {0.2f, 0.08f, 0.07f}}, {"TransparentGlass", {1.0f, 1.0f, 1.0f}},
      {"Water", {1.0f, 1.0f, 1.0f}},                  {"Ice", {1.0f, 1.0f, 1.0f}},
      {"Beer", {0.8f, 0.7f, 0.55f}},                  {"Red_Wine", {0.24f, 0.09f, 0.07f}},
      {"White_Wine", {0.85f, 0.78f, 0.6f}}};
  auto it = kColours.find(name);
  if (it != kColours.end())
    for (int k = 0; k < 3; ++k) m.transmitting_color[k] = it->second[k];
  return m;
}

// One mesh of the model as the importers hand it over: position, normal
// and uv per corner (normals: all_n, else geometric normals are made; uvs:
// all_t, else (0, 0)), triangles over the corners, the material's index.
struct BuildMesh {
  std::vector<float> pos, nrm, uv;
  bool all_n = false, all_t = false;
  std::vector<int32_t> tris;
  int material = 0;
};

// What both importers share: the materials (their textures decoded on up to
// 16 threads, taken in order of first use), the meshes (geometric normals
// where a mesh has none, FixInfacingNormals where it has them) and the sky.
rmn_status finish_model(const std::string& folder, const std::string& name, const std::vector<MtlSpec>& specs,
                        std::vector<BuildMesh>& meshes, const std::string& sky, rmn_model& M) {
  M.material_names.clear();
  for (const MtlSpec& sp : specs) M.material_names.push_back(sp.name);
  // texture files in order of first use, decoded on several threads; the
  // results are taken in that order, so indices and the first error are
  // those of one-by-one loading
  struct TexJob {
    std::string path;
    rmn::DecodedImage img;
    bool loaded = false;
    rmn_status st = RMN_OK;
    std::string err;
  };
  std::vector<TexJob> jobs;
  std::map<std::string, int> job_of;
  std::vector<std::array<int, 4>> mat_jobs;
  for (const MtlSpec& spec : specs) {
    std::array<int, 4> js = {-1, -1, -1, -1};
    for (const auto& kv : spec.textures) {
      std::string p = folder + kv.second;
      for (char& c : p)
        if (c == '\\') c = '/';
      p = url_decode(p);
      auto j = job_of.find(p);
      if (j == job_of.end()) {
        j = job_of.emplace(p, (int)jobs.size()).first;
        jobs.emplace_back();
        jobs.back().path = p;
      }
      js[kv.first] = j->second;
    }
    mat_jobs.push_back(js);
  }
  {
    std::atomic<size_t> next{0};
    auto work = [&]() {
      for (size_t j; (j = next.fetch_add(1)) < jobs.size();) {
        TexJob& t = jobs[j];
        t.st = load_texture(t.path, t.img, &t.loaded);
        if (t.st != RMN_OK) t.err = rmn_last_error();
      }
    };
    const size_t nthreads = std::min<size_t>(jobs.size(), rmn::host_threads());
    run_threads(nthreads, [&](size_t) { work(); });
  }
  std::vector<int> tex_of(jobs.size(), -1);
  for (size_t j = 0; j < jobs.size(); ++j) {
    if (jobs[j].st != RMN_OK) return fail(jobs[j].st, "%s", jobs[j].err.c_str());
    if (!jobs[j].loaded) continue;
    tex_of[j] = (int)M.texels.size();
    M.texels.push_back(std::move(jobs[j].img.bytes));
    M.textures.push_back(rmn_texture{jobs[j].img.w, jobs[j].img.h, 4, nullptr});
  }
  for (size_t i = 0; i < specs.size(); ++i) {
    int32_t slots[4];
    for (int k = 0; k < 4; ++k) slots[k] = mat_jobs[i][k] < 0 ? -1 : tex_of[mat_jobs[i][k]];
    M.materials.push_back(specs[i].opacity < 0.99f ? glass_material(specs[i].name) : default_material());  // float test
    M.material_textures.insert(M.material_textures.end(), slots, slots + 4);
  }

  // each mesh's normals (geometric, or its own after the infacing test) and
  // uvs, meshes on separate threads; then the meshes in order
  auto prepare = [](BuildMesh& mb) {
    std::vector<float>& pos = mb.pos;
    std::vector<float>& nrm = mb.nrm;
    const size_t nc = pos.size() / 3;
    nrm.resize(3 * nc, 0.0f);
    if (!mb.all_t) mb.uv.assign(2 * nc, 0.0f);
    const size_t nt = mb.tris.size() / 3;
    if (!mb.all_n) {  // geometric normals, written corner 0, 1, 2 of every triangle in turn
      std::vector<float> g(3 * nt);
      for (size_t t = 0; t < nt; ++t) {
        const float* a = &pos[3 * mb.tris[3 * t]];
        const float* b = &pos[3 * mb.tris[3 * t + 1]];
        const float* c = &pos[3 * mb.tris[3 * t + 2]];
        const float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        const float e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        float x = e1[1] * e2[2], y = e1[2] * e2[0], z = e1[0] * e2[1];
        x -= e1[2] * e2[1];
        y -= e1[0] * e2[2];
        z -= e1[1] * e2[0];
        float len = x * x;
        len += y * y;
        len += z * z;
        len = std::sqrt(len);
        if (len < 1e-30f) len = 1e-30f;  // max(|g|, 1e-30); NaN stays NaN
        g[3 * t] = x / len;
        g[3 * t + 1] = y / len;
        g[3 * t + 2] = z / len;
      }
      for (int k = 0; k < 3; ++k)
        for (size_t t = 0; t < nt; ++t)
          for (int j = 0; j < 3; ++j) nrm[3 * mb.tris[3 * t + k] + j] = g[3 * t + j];
    } else if (nc > 0) {  // FixInfacingNormals: moved box smaller than the vertices' box -> flip
      float lo0[3], hi0[3], lo1[3], hi1[3];
      for (int k = 0; k < 3; ++k) {
        lo0[k] = hi0[k] = pos[k];
        lo1[k] = hi1[k] = pos[k] + nrm[k];
      }
      for (size_t i = 1; i < nc; ++i)
        for (int k = 0; k < 3; ++k) {
          const float p = pos[3 * i + k], q = pos[3 * i + k] + nrm[3 * i + k];
          lo0[k] = std::fmin(lo0[k], p);
          hi0[k] = std::fmax(hi0[k], p);
          lo1[k] = std::fmin(lo1[k], q);
          hi1[k] = std::fmax(hi1[k], q);
        }
      float v0 = hi0[0] - lo0[0], v1 = hi1[0] - lo1[0];
      v0 *= hi0[1] - lo0[1];
      v0 *= hi0[2] - lo0[2];
      v1 *= hi1[1] - lo1[1];
      v1 *= hi1[2] - lo1[2];
      if (v0 > 0.0f && v1 < v0)
        for (float& v : nrm) v = -v;
    }
  };
  {
    std::atomic<size_t> next{0};
    run_threads(std::min(meshes.size(), rmn::host_threads()), [&](size_t) {
      for (size_t j; (j = next.fetch_add(1)) < meshes.size();) prepare(meshes[j]);
    });
  }
  M.mesh_first.assign(1, 0);
  for (BuildMesh& mb : meshes) {
    const std::vector<float>& pos = mb.pos;
    const std::vector<float>& nrm = mb.nrm;
    const size_t nt = mb.tris.size() / 3;
    const int32_t base = (int32_t)(M.positions.size() / 3);
    M.positions.insert(M.positions.end(), pos.begin(), pos.end());
    M.normals.insert(M.normals.end(), nrm.begin(), nrm.end());
    M.uvs.insert(M.uvs.end(), mb.uv.begin(), mb.uv.end());
    for (int32_t i : mb.tris) M.indices.push_back(base + i);
    M.mesh_first.push_back(M.mesh_first.back() + (int32_t)nt);
    M.mesh_material.push_back(mb.material);
  }
  if (M.indices.empty()) return fail(RMN_ERR_INVALID_ARGUMENT, "%s%s: no triangles", folder.c_str(), name.c_str());
  for (size_t i = 0; i < M.textures.size(); ++i) M.textures[i].texels = M.texels[i].data();
  if (M.textures.empty()) M.material_textures.clear();

  if (sky != "null") {  // SkyBox::load through hdr_to_array; a failure leaves no sky
    rmn::DecodedImage img;
    const std::string p = folder + sky;
    if (rmn::decode_image_file(p.c_str(), RMN_IMAGE_HDR, false, img) == RMN_OK) {
      M.env_w = img.w;
      M.env_h = img.h;
      M.env.resize((size_t)img.w * img.h * 3);
      std::memcpy(M.env.data(), img.bytes.data(), M.env.size() * sizeof(float));
    } else {
      std::fprintf(stderr, "Conversion failed: %s\n", rmn_last_error());
      rmn::clear_error();
    }
  }
  return RMN_OK;
}

rmn_status read_obj_model(const std::string& folder, const std::string& name, const std::string& sky,
                          rmn_model& M) {
  std::vector<float> P, T, N;
  std::vector<MeshRun> meshes;
  std::vector<std::string> mtllibs;
  rmn_status st = parse_obj(folder + name, P, T, N, meshes, mtllibs);
  if (st != RMN_OK) return st;
  std::vector<MtlSpec> lib;
  for (const std::string& m : mtllibs)
    if ((st = parse_mtl(folder + m, lib)) != RMN_OK) return st;

  // materials: the default one, the libraries' (a repeated name takes its
  // last definition), then usemtl names nobody defines, in order of use
  std::vector<MtlSpec> specs;
  std::map<std::string, const MtlSpec*> by_name;
  for (const MtlSpec& m : lib) by_name[m.name] = &m;
  std::vector<std::string> names(1, kDefaultMaterial);
  for (const MtlSpec& m : lib) names.push_back(m.name);
  std::map<std::string, int> index_of;
  for (size_t i = 0; i < names.size(); ++i) index_of[names[i]] = (int)i;
  for (const MeshRun& mr : meshes)
    if (!index_of.count(mr.mat)) {
      index_of.emplace(mr.mat, (int)names.size());
      names.push_back(mr.mat);
    }
  for (const std::string& n : names) {
    auto it = by_name.find(n);
    specs.push_back(it != by_name.end() ? *it->second : MtlSpec{n, 1.0f, {}});
  }

  std::vector<BuildMesh> built;
  for (const MeshRun& mr : meshes) {
    const size_t nc = mr.corners.size();
    bool all_n = true, all_t = true;
    for (const Corner& c : mr.corners) {
      if (c.v < 0 || c.v >= (long long)(P.size() / 3))
        return fail(RMN_ERR_INVALID_ARGUMENT, "%s%s: a face refers to a vertex that does not exist", folder.c_str(),
                    name.c_str());
      if (c.t >= (long long)(T.size() / 2) || c.n >= (long long)(N.size() / 3) || c.t < -1 || c.n < -1)
        return fail(RMN_ERR_INVALID_ARGUMENT,
                    "%s%s: a face refers to a texture coordinate or normal that does not exist", folder.c_str(),
                    name.c_str());
      all_n = all_n && c.n >= 0;
      all_t = all_t && c.t >= 0;
    }
    BuildMesh mb;
    mb.pos.resize(3 * nc);
    mb.nrm.resize(3 * nc);
    mb.uv.assign(2 * nc, 0.0f);
    for (size_t i = 0; i < nc; ++i) {
      const Corner& c = mr.corners[i];
      for (int k = 0; k < 3; ++k) mb.pos[3 * i + k] = P[3 * c.v + k];
      if (all_n)
        for (int k = 0; k < 3; ++k) mb.nrm[3 * i + k] = N[3 * c.n + k];
      if (all_t)
        for (int k = 0; k < 2; ++k) mb.uv[2 * i + k] = T[2 * c.t + k];
    }
    mb.all_n = all_n;
    mb.all_t = true;  // missing uvs are (0, 0) already
    mb.tris = mr.tris;
    mb.material = index_of[mr.mat];
    built.push_back(std::move(mb));
  }
  return finish_model(folder, name, specs, built, sky, M);
}

// A binary FBX model (fbx.cpp) through the same material, normal and sky
// steps.
rmn_status read_fbx_model(const std::string& folder, const std::string& name, const std::string& sky,
                          rmn_model& M) {
  std::vector<rmn::FbxMesh> fm;
  std::vector<rmn::FbxMaterial> fmats;
  rmn_status st = rmn::read_fbx(folder + name, fm, fmats);
  if (st != RMN_OK) return st;
  std::vector<MtlSpec> specs;
  for (const rmn::FbxMaterial& m : fmats) {
    MtlSpec sp{m.name, m.opacity, {}};
    for (int k = 0; k < 4; ++k)
      if (!m.textures[k].empty()) sp.textures[k] = m.textures[k];
    specs.push_back(sp);
  }
  std::vector<BuildMesh> built;
  for (rmn::FbxMesh& m : fm) {
    BuildMesh mb;
    mb.pos = std::move(m.pos);
    mb.nrm = std::move(m.nrm);
    mb.uv = std::move(m.uv);
    mb.all_n = m.has_nrm;
    mb.all_t = m.has_uv;
    mb.tris = std::move(m.tris);
    mb.material = m.material;
    built.push_back(std::move(mb));
  }
  return finish_model(folder, name, specs, built, sky, M);
}

rmn_status read_model(const std::string& folder, const std::string& name, const std::string& sky, rmn_model& M) {
  std::string ext = name.size() >= 4 ? lower(name.substr(name.size() - 4)) : "";
  if (ext == ".fbx") return read_fbx_model(folder, name, sky, M);
  return read_obj_model(folder, name, sky, M);
}

}  // namespace

extern "C" {

rmn_status rmn_model_read(const char* model_folder, const char* model_name, const char* skyMap_name,
                          rmn_model** out) {
  rmn::clear_error();
  if (!model_folder || !model_name || !out) return fail(RMN_ERR_INVALID_ARGUMENT, "rmn_model_read needs a folder, a name and an output");
  *out = nullptr;
  rmn_model* m = new (std::nothrow) rmn_model();
  if (!m) return fail(RMN_ERR_OUT_OF_MEMORY, "rmn_model_read");
  rmn_status st;
  try {
    st = read_model(model_folder, model_name, skyMap_name ? skyMap_name : "null", *m);
  } catch (const std::bad_alloc&) {
    st = fail(RMN_ERR_OUT_OF_MEMORY, "out of host memory reading %s%s", model_folder, model_name);
  } catch (const std::exception& e) {  // e.g. no thread for the texture decoders
    st = fail(RMN_ERR_INTERNAL, "reading %s%s: %s", model_folder, model_name, e.what());
  }
  if (st != RMN_OK) {
    delete m;
    return st;
  }
  *out = m;
  return RMN_OK;
}

rmn_status rmn_model_desc(const rmn_model* m, rmn_scene_desc* d) {
  rmn::clear_error();
  if (!m || !d) return fail(RMN_ERR_INVALID_ARGUMENT, "model or description is NULL");
  *d = rmn_scene_desc{};
  d->num_vertices = (int32_t)(m->positions.size() / 3);
  d->positions = m->positions.data();
  d->normals = m->normals.data();
  d->uvs = m->uvs.data();
  d->num_triangles = (int32_t)(m->indices.size() / 3);
  d->indices = m->indices.data();
  d->num_meshes = (int32_t)m->mesh_material.size();
  d->mesh_first = m->mesh_first.data();
  d->mesh_material = m->mesh_material.data();
  d->num_materials = (int32_t)m->materials.size();
  d->materials = m->materials.data();
  d->env_width = m->env.empty() ? 0 : m->env_w;
  d->env_height = m->env.empty() ? 0 : m->env_h;
  d->env_rgb = m->env.empty() ? nullptr : m->env.data();
  d->num_textures = (int32_t)m->textures.size();
  d->textures = m->textures.empty() ? nullptr : m->textures.data();
  d->material_textures = m->material_textures.empty() ? nullptr : m->material_textures.data();
  return RMN_OK;
}

const char* rmn_model_material_name(const rmn_model* m, int32_t material) {
  if (!m || material < 0 || material >= (int32_t)m->material_names.size()) return nullptr;
  return m->material_names[material].c_str();
}

rmn_status rmn_model_free(rmn_model* m) {
  delete m;
  return RMN_OK;
}

}  // extern "C"
