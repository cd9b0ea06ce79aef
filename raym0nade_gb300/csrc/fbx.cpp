// Binary FBX models for Model::Model (src/model.cpp:172-215), which reads
// them with assimp (aiProcess_Triangulate | PreTransformVertices |
// SortByPType | FixInfacingNormals). The library does not use assimp; what
// its FBX import does is restated here from the container's published
// description (the node-record layout Blender's and assimp's readers
// document) and assimp's documented behaviour:
//  * the file: a 27-byte header ("Kaydara FBX Binary  ", 0x1A 0x00, the
//    version), then node records -- end offset, property count, property
//    bytes (32-bit fields, 64-bit from version 7500), a name, the properties
//    (Y C I F D L scalars, S R strings, f d l i b arrays, raw or zlib) and
//    nested records ended by a null record;
//  * the scene: Objects (Geometry "Mesh", Model, Material, Texture) and
//    Connections ("OO" child -> parent, "OP" child -> parent property);
//  * a model's transform: T Roff Rp Rpre R Rpost^-1 Rp^-1 Soff Sp S Sp^-1
//    from its Properties70 (rotations in degrees, R in its RotationOrder),
//    times its parent's; the geometric translation / rotation / scaling on
//    top for the geometry alone. PreTransformVertices puts every vertex in
//    world space and every normal through the inverse transpose,
//    normalised. No unit or axis conversion (assimp's default);
//  * a geometry splits into one mesh per material it uses (ascending
//    material index), a vertex per polygon corner, polygons as a fan from
//    their first corner (assimp ear-clips polygons of more than four
//    corners: identical for convex quads); normals and the first uv set
//    from the layer elements (ByPolygonVertex / ByVertice / ByPolygon /
//    AllSame, Direct / IndexToDirect);
//  * materials: in order of first use, a "DefaultMaterial" for geometries
//    without one; per material what Material::loadMaterialProperties reads:
//    the name, the opacity ("Opacity", 1 without it) and the textures
//    connected to DiffuseColor (diffuse), SpecularColor / SpecularFactor
//    (specular), EmissiveColor / EmissiveFactor (emissive) and NormalMap
//    (normal map), by their RelativeFilename (else FileName); of several
//    textures in one slot the last connected wins, as the reference's
//    loader overwrites the slot.
// ASCII FBX files are RMN_ERR_UNSUPPORTED. Malformed files give
// RMN_ERR_INVALID_ARGUMENT: every offset and length is checked against the
// bytes present.
#include <array>
#include <cmath>
#include <cstdio>
#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <string>
#include <type_traits>
#include <vector>

#include "rmn_host.h"

namespace {

using rmn::fail;

struct Prop {
  char type = 0;
  int64_t i = 0;
  double d = 0.0;
  std::string s;
  std::vector<double> da;   // f, d arrays
  std::vector<int64_t> ia;  // i, l, b arrays
};

struct Node {
  std::string name;
  std::vector<Prop> props;
  std::vector<Node> kids;
  const Node* child(const char* n) const {
    for (const Node& k : kids)
      if (k.name == n) return &k;
    return nullptr;
  }
};
// Records are moved, never copied, when their parent's array grows, so a
// property keeps its address from the parse on (the deferred arrays below).
static_assert(std::is_nothrow_move_constructible<Node>::value, "records must move without copying");

class Reader {
 public:
  Reader(const std::vector<uint8_t>& b, uint32_t version) : b_(b), wide_(version >= 7500) {}
  const char* err = nullptr;

  // The arrays met by records(), inflated (zlib) and converted after the
  // parse, on several threads. A stream that does not inflate is
  // reported as the reader would have met it in file order: before any
  // later defect (every array here lies before the point where records()
  // stopped), and the first such stream if there are several. After a
  // parse that failed (`parsed` false) the records that held some of these
  // arrays are gone: the streams are only inflated to find such an earlier
  // defect, and nothing is written.
  bool finish_arrays(bool parsed) {
    std::atomic<size_t> next{0};
    rmn::run_threads(std::min(rmn::host_threads(), deferred_.size()), [&](size_t) {
      std::vector<uint8_t> tmp;
      for (size_t j; (j = next.fetch_add(1)) < deferred_.size();) {
        Deferred& a = deferred_[j];
        if (!a.zlib) {
          if (parsed) convert(*a.p, b_.data() + a.off, a.count);
          continue;
        }
        a.err = rmn::zlib_inflate(b_.data() + a.off, a.clen, tmp, a.raw);
        if (!a.err && parsed) convert(*a.p, tmp.data(), a.count);
      }
    });
    for (const Deferred& a : deferred_)  // in file order
      if (a.err) {
        err = a.err;
        return false;
      }
    return err == nullptr;
  }

  // Reads the records at `off` up to `end` (or a null record) into `out`.
  bool records(size_t& off, size_t end, std::vector<Node>& out, int depth) {
    if (depth > 64) return bad("nesting deeper than 64 records");
    while (off < end) {
      Node n;
      bool null_rec = false;
      if (!record(off, end, n, null_rec, depth)) return false;
      if (null_rec) return true;
      out.push_back(std::move(n));
    }
    return true;
  }

 private:
  struct Deferred {
    Prop* p;  // in its record's property array, which no longer changes size (valid while the records are)
    size_t off, raw;
    uint32_t clen, count;
    bool zlib;  // else the elements' bytes as they are
    const char* err = nullptr;
  };
  const std::vector<uint8_t>& b_;
  bool wide_;
  std::vector<Deferred> deferred_;

  // An array's elements (count of p.type) from their bytes.
  static void convert(Prop& p, const uint8_t* src, uint32_t count) {
    if (p.type == 'f' || p.type == 'd') {
      p.da.resize(count);
      for (uint32_t k = 0; k < count; ++k) {
        if (p.type == 'f') {
          float v;
          std::memcpy(&v, src + 4 * (size_t)k, 4);
          p.da[k] = v;
        } else {
          std::memcpy(&p.da[k], src + 8 * (size_t)k, 8);
        }
      }
    } else {
      p.ia.resize(count);
      for (uint32_t k = 0; k < count; ++k) {
        if (p.type == 'b') {
          p.ia[k] = src[k] != 0;
        } else if (p.type == 'i') {
          int32_t v;
          std::memcpy(&v, src + 4 * (size_t)k, 4);
          p.ia[k] = v;
        } else {
          std::memcpy(&p.ia[k], src + 8 * (size_t)k, 8);
        }
      }
    }
  }

  bool bad(const char* m) {
    if (!err) err = m;
    return false;
  }
  bool u32(size_t& off, uint32_t* v) {
    if (off + 4 > b_.size()) return bad("truncated record");
    *v = (uint32_t)b_[off] | (uint32_t)b_[off + 1] << 8 | (uint32_t)b_[off + 2] << 16 | (uint32_t)b_[off + 3] << 24;
    off += 4;
    return true;
  }
  bool u64(size_t& off, uint64_t* v) {
    uint32_t lo, hi;
    if (!u32(off, &lo) || !u32(off, &hi)) return false;
    *v = (uint64_t)hi << 32 | lo;
    return true;
  }
  bool field(size_t& off, uint64_t* v) {
    if (wide_) return u64(off, v);
    uint32_t x;
    if (!u32(off, &x)) return false;
    *v = x;
    return true;
  }
  template <class T>
  T get(size_t off) const {
    T v;
    std::memcpy(&v, b_.data() + off, sizeof(T));
    return v;
  }

  bool record(size_t& off, size_t limit, Node& n, bool& null_rec, int depth) {
    const size_t start = off;
    uint64_t end, nprops, plen;
    if (!field(off, &end) || !field(off, &nprops) || !field(off, &plen)) return false;
    if (off + 1 > b_.size()) return bad("truncated record");
    const uint8_t nlen = b_[off++];
    if (end == 0 && nprops == 0 && plen == 0 && nlen == 0) {
      null_rec = true;
      return true;
    }
    if (end <= start || end > limit || off + nlen > end) return bad("record outside its parent");
    n.name.assign(reinterpret_cast<const char*>(b_.data() + off), nlen);
    off += nlen;
    const size_t pend = off + plen;
    if (plen > end - off) return bad("properties outside their record");
    if (nprops > plen) return bad("more properties than property bytes");
    n.props.resize((size_t)nprops);
    for (Prop& p : n.props)
      if (!prop(off, pend, p)) return false;
    if (off != pend) return bad("property bytes do not add up");
    if (off < end && !records(off, end, n.kids, depth + 1)) return false;
    off = end;
    return true;
  }

  bool prop(size_t& off, size_t pend, Prop& p) {
    if (off + 1 > pend) return bad("truncated property");
    p.type = (char)b_[off++];
    auto need = [&](size_t k) { return off + k <= pend ? true : bad("truncated property"); };
    switch (p.type) {
      case 'Y': if (!need(2)) return false; p.i = get<int16_t>(off); off += 2; return true;
      case 'C': if (!need(1)) return false; p.i = b_[off] != 0; off += 1; return true;
      case 'I': if (!need(4)) return false; p.i = get<int32_t>(off); off += 4; return true;
      case 'F': if (!need(4)) return false; p.d = get<float>(off); off += 4; return true;
      case 'D': if (!need(8)) return false; p.d = get<double>(off); off += 8; return true;
      case 'L': if (!need(8)) return false; p.i = get<int64_t>(off); off += 8; return true;
      case 'S':
      case 'R': {
        uint32_t len;
        if (!need(4) || !u32(off, &len) || !need(len)) return false;
        p.s.assign(reinterpret_cast<const char*>(b_.data() + off), len);
        off += len;
        return true;
      }
      case 'f': case 'd': case 'l': case 'i': case 'b': {
        uint32_t count, enc, clen;
        if (!need(12) || !u32(off, &count) || !u32(off, &enc) || !u32(off, &clen) || !need(clen)) return false;
        const size_t esz = p.type == 'b' ? 1 : (p.type == 'f' || p.type == 'i') ? 4 : 8;
        if (count > (1u << 30) / esz) return bad("array too long");
        const size_t raw = (size_t)count * esz;
        if (enc == 0) {
          if (clen != raw) return bad("array length does not match its bytes");
          deferred_.push_back({&p, off, raw, clen, count, false});
        } else if (enc == 1) {
          deferred_.push_back({&p, off, raw, clen, count, true});
        } else {
          return bad("unknown array encoding");
        }
        off += clen;
        return true;
      }
      default:
        return bad("unknown property type");
    }
  }
};

// ------------------------------------------------------------ transforms
using M4 = std::array<double, 16>;  // row-major, column vectors: p' = M p

M4 identity() {
  M4 m{};
  m[0] = m[5] = m[10] = m[15] = 1.0;
  return m;
}
M4 mul(const M4& a, const M4& b) {
  M4 c{};
  for (int r = 0; r < 4; ++r)
    for (int k = 0; k < 4; ++k) {
      double s = a[4 * r] * b[k];
      s += a[4 * r + 1] * b[4 + k];
      s += a[4 * r + 2] * b[8 + k];
      s += a[4 * r + 3] * b[12 + k];
      c[4 * r + k] = s;
    }
  return c;
}
M4 translate(const double* t) {
  M4 m = identity();
  m[3] = t[0];
  m[7] = t[1];
  m[11] = t[2];
  return m;
}
M4 scale(const double* s) {
  M4 m = identity();
  m[0] = s[0];
  m[5] = s[1];
  m[10] = s[2];
  return m;
}
M4 axis_rot(int axis, double deg) {
  const double a = deg * 3.14159265358979323846 / 180.0, c = std::cos(a), s = std::sin(a);
  M4 m = identity();
  const int i = (axis + 1) % 3, j = (axis + 2) % 3;
  m[4 * i + i] = c;
  m[4 * i + j] = -s;
  m[4 * j + i] = s;
  m[4 * j + j] = c;
  return m;
}
// Euler angles (degrees) applied in the order the FBX RotationOrder names:
// 0 XYZ (X first), 1 XZY, 2 YZX, 3 YXZ, 4 ZXY, 5 ZYX.
M4 euler(const double* r, int order) {
  static const int seq[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 2, 0}, {1, 0, 2}, {2, 0, 1}, {2, 1, 0}};
  if (order < 0 || order > 5) order = 0;
  M4 m = identity();
  for (int k = 0; k < 3; ++k) m = mul(axis_rot(seq[order][k], r[seq[order][k]]), m);
  return m;
}
// Inverse of an affine matrix (3x3 part by the adjugate), and the inverse
// transpose of its 3x3 part for normals.
bool inverse3(const M4& m, double inv[9]) {
  const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
  const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
  const double det = a * A + b * B + c * C;
  if (!(std::fabs(det) > 0.0)) return false;
  inv[0] = A / det; inv[1] = -(b * i - c * h) / det; inv[2] = (b * f - c * e) / det;
  inv[3] = B / det; inv[4] = (a * i - c * g) / det; inv[5] = -(a * f - c * d) / det;
  inv[6] = C / det; inv[7] = -(a * h - b * g) / det; inv[8] = (a * e - b * d) / det;
  return true;
}

struct ModelInfo {
  int64_t id = 0;
  std::string name;
  M4 local = identity(), geometric = identity();
  int64_t parent = 0;
};

void vec3_prop(const Node* p70, const char* name, double* v) {
  if (!p70) return;
  for (const Node& p : p70->kids) {
    if (p.name != "P" || p.props.size() < 7 || p.props[0].s != name) continue;
    for (int k = 0; k < 3; ++k) {
      const Prop& q = p.props[4 + k];
      v[k] = (q.type == 'D' || q.type == 'F') ? q.d : (double)q.i;
    }
  }
}
bool num_prop(const Node* p70, const char* name, double* v) {
  if (!p70) return false;
  bool found = false;
  for (const Node& p : p70->kids) {
    if (p.name != "P" || p.props.size() < 5 || p.props[0].s != name) continue;
    const Prop& q = p.props[4];
    *v = (q.type == 'D' || q.type == 'F') ? q.d : (double)q.i;
    found = true;
  }
  return found;
}

// T Roff Rp Rpre R Rpost^-1 Rp^-1 Soff Sp S Sp^-1, and the geometric transform
void model_transforms(const Node& o, ModelInfo& mi) {
  const Node* p70 = o.child("Properties70");
  double T[3] = {0, 0, 0}, R[3] = {0, 0, 0}, S[3] = {1, 1, 1};
  double Roff[3] = {0, 0, 0}, Rp[3] = {0, 0, 0}, Soff[3] = {0, 0, 0}, Sp[3] = {0, 0, 0};
  double Rpre[3] = {0, 0, 0}, Rpost[3] = {0, 0, 0};
  double GT[3] = {0, 0, 0}, GR[3] = {0, 0, 0}, GS[3] = {1, 1, 1};
  double order = 0;
  vec3_prop(p70, "Lcl Translation", T);
  vec3_prop(p70, "Lcl Rotation", R);
  vec3_prop(p70, "Lcl Scaling", S);
  vec3_prop(p70, "RotationOffset", Roff);
  vec3_prop(p70, "RotationPivot", Rp);
  vec3_prop(p70, "ScalingOffset", Soff);
  vec3_prop(p70, "ScalingPivot", Sp);
  vec3_prop(p70, "PreRotation", Rpre);
  vec3_prop(p70, "PostRotation", Rpost);
  vec3_prop(p70, "GeometricTranslation", GT);
  vec3_prop(p70, "GeometricRotation", GR);
  vec3_prop(p70, "GeometricScaling", GS);
  num_prop(p70, "RotationOrder", &order);
  const double nRp[3] = {-Rp[0], -Rp[1], -Rp[2]}, nSp[3] = {-Sp[0], -Sp[1], -Sp[2]};
  M4 post = euler(Rpost, 0);
  // Rpost^-1: the transpose of a rotation
  M4 post_inv = identity();
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) post_inv[4 * r + c] = post[4 * c + r];
  M4 m = translate(T);
  m = mul(m, translate(Roff));
  m = mul(m, translate(Rp));
  m = mul(m, euler(Rpre, 0));
  m = mul(m, euler(R, (int)order));
  m = mul(m, post_inv);
  m = mul(m, translate(nRp));
  m = mul(m, translate(Soff));
  m = mul(m, translate(Sp));
  m = mul(m, scale(S));
  m = mul(m, translate(nSp));
  mi.local = m;
  mi.geometric = mul(mul(translate(GT), euler(GR, 0)), scale(GS));
}

std::string object_name(const Node& o) {
  if (o.props.size() < 2 || o.props[1].type != 'S') return "";
  const std::string& s = o.props[1].s;
  const size_t k = s.find(std::string("\x00\x01", 2));
  return k == std::string::npos ? s : s.substr(0, k);
}

// A layer element's mapping (MappingInformationType, default
// ByPolygonVertex) and reference (ReferenceInformationType, default Direct),
// read once per geometry.
struct LayerMap {
  enum Mode { kByCorner, kByVertex, kByPolygon, kAllSame, kOther } mode = kOther;
  bool indexed = false;                         // IndexToDirect / Index
  const std::vector<int64_t>* index = nullptr;  // the index array when indexed (none: every lookup fails)
};

LayerMap layer_map(const Node& le, const char* index_name) {
  const Node* mt = le.child("MappingInformationType");
  const Node* rt = le.child("ReferenceInformationType");
  const std::string map = mt && !mt->props.empty() ? mt->props[0].s : "ByPolygonVertex";
  const std::string ref = rt && !rt->props.empty() ? rt->props[0].s : "Direct";
  LayerMap m;
  if (map == "ByPolygonVertex") m.mode = LayerMap::kByCorner;
  else if (map == "ByVertice" || map == "ByVertex") m.mode = LayerMap::kByVertex;
  else if (map == "ByPolygon") m.mode = LayerMap::kByPolygon;
  else if (map == "AllSame") m.mode = LayerMap::kAllSame;
  m.indexed = ref == "IndexToDirect" || ref == "Index";
  if (m.indexed) {
    const Node* ix = le.child(index_name);
    if (ix && !ix->props.empty()) m.index = &ix->props[0].ia;
  }
  return m;
}

// The layer element's value index for corner c of polygon `poly` at control
// point v, or -1.
int64_t layer_index(const LayerMap& m, int64_t c, int64_t poly, int64_t v) {
  int64_t k;
  switch (m.mode) {
    case LayerMap::kByCorner: k = c; break;
    case LayerMap::kByVertex: k = v; break;
    case LayerMap::kByPolygon: k = poly; break;
    case LayerMap::kAllSame: k = 0; break;
    default: return -1;
  }
  if (m.indexed) {
    if (!m.index || k < 0 || k >= (int64_t)m.index->size()) return -1;
    k = (*m.index)[(size_t)k];
  }
  return k;
}

}  // namespace

namespace rmn {

rmn_status read_fbx(const std::string& path, std::vector<FbxMesh>& meshes, std::vector<FbxMaterial>& materials) {
  std::vector<uint8_t> b;
  if (!read_whole_file(path.c_str(), b)) return fail(RMN_ERR_INVALID_ARGUMENT, "could not read %s", path.c_str());
  static const char kMagic[] = "Kaydara FBX Binary  ";
  if (b.size() >= 5 && std::memcmp(b.data(), "; FBX", 5) == 0)
    return fail(RMN_ERR_UNSUPPORTED, "%s: ASCII FBX files are not read (binary only)", path.c_str());
  if (b.size() < 27 || std::memcmp(b.data(), kMagic, 20) != 0 || b[20] != 0 || b[21] != 0x1A || b[22] != 0)
    return fail(RMN_ERR_INVALID_ARGUMENT, "%s: not a binary FBX file", path.c_str());
  const uint32_t version = (uint32_t)b[23] | (uint32_t)b[24] << 8 | (uint32_t)b[25] << 16 | (uint32_t)b[26] << 24;
  Reader rd(b, version);
  std::vector<Node> top;
  size_t off = 27;
  const bool parsed = rd.records(off, b.size(), top, 0);
  if (!rd.finish_arrays(parsed) || !parsed)
    return fail(RMN_ERR_INVALID_ARGUMENT, "%s: %s", path.c_str(), rd.err ? rd.err : "malformed");

  const Node *objects = nullptr, *conns = nullptr;
  for (const Node& n : top) {
    if (n.name == "Objects") objects = &n;
    if (n.name == "Connections") conns = &n;
  }
  if (!objects) return fail(RMN_ERR_INVALID_ARGUMENT, "%s: no Objects", path.c_str());

  std::map<int64_t, const Node*> geometry, material, texture;
  std::vector<ModelInfo> models;
  std::map<int64_t, size_t> model_at;
  for (const Node& o : objects->kids) {
    if (o.props.empty() || o.props[0].type != 'L') continue;
    const int64_t id = o.props[0].i;
    const std::string cls = o.props.size() > 2 ? o.props[2].s : "";
    if (o.name == "Geometry" && cls == "Mesh") geometry[id] = &o;
    else if (o.name == "Material") material[id] = &o;
    else if (o.name == "Texture") texture[id] = &o;
    else if (o.name == "Model") {
      ModelInfo mi;
      mi.id = id;
      mi.name = object_name(o);
      model_transforms(o, mi);
      model_at[id] = models.size();
      models.push_back(mi);
    }
  }
  // connections, in file order
  std::map<int64_t, int64_t> geom_model;                    // geometry -> model
  std::map<int64_t, std::vector<int64_t>> model_mats;       // model -> materials, in connection order
  std::map<int64_t, std::vector<std::pair<int, int64_t>>> mat_tex;  // material -> (slot, texture)
  if (conns)
    for (const Node& c : conns->kids) {
      if (c.name != "C" || c.props.size() < 3) continue;
      const std::string& kind = c.props[0].s;
      const int64_t child = c.props[1].i, parent = c.props[2].i;
      if (kind == "OO") {
        if (geometry.count(child) && model_at.count(parent)) geom_model.emplace(child, parent);
        else if (material.count(child) && model_at.count(parent)) model_mats[parent].push_back(child);
        else if (model_at.count(child) && (parent == 0 || model_at.count(parent)))
          models[model_at[child]].parent = parent;
      } else if (kind == "OP" && c.props.size() >= 4 && texture.count(child) && material.count(parent)) {
        const std::string& p = c.props[3].s;
        int slot = -1;
        if (p == "DiffuseColor") slot = RMN_TEX_DIFFUSE;
        else if (p == "SpecularColor" || p == "SpecularFactor") slot = RMN_TEX_SPECULAR;
        else if (p == "EmissiveColor" || p == "EmissiveFactor") slot = RMN_TEX_EMISSIVE;
        else if (p == "NormalMap") slot = RMN_TEX_NORMALS;
        if (slot >= 0) mat_tex[parent].push_back({slot, child});
      }
    }
  // world transforms (parents first; a cycle stops at 64 levels)
  auto world = [&](const ModelInfo& m0) {
    M4 w = m0.local;
    int64_t p = m0.parent;
    for (int guard = 0; p != 0 && model_at.count(p) && guard < 64; ++guard) {
      const ModelInfo& pm = models[model_at[p]];
      w = mul(pm.local, w);
      p = pm.parent;
    }
    return w;
  };

  std::map<int64_t, int> mat_index;  // FBX material id -> output index
  int default_index = -1;
  auto use_material = [&](int64_t id) -> int {
    if (id == 0 || !material.count(id)) {
      if (default_index < 0) {
        default_index = (int)materials.size();
        FbxMaterial dm;
        dm.name = "DefaultMaterial";
        materials.push_back(dm);
      }
      return default_index;
    }
    auto it = mat_index.find(id);
    if (it != mat_index.end()) return it->second;
    const Node& mn = *material[id];
    FbxMaterial fm;
    fm.name = object_name(mn);
    double op;
    if (num_prop(mn.child("Properties70"), "Opacity", &op)) fm.opacity = (float)op;
    for (const auto& st : mat_tex[id]) {
      const Node& tn = *texture[st.second];
      const Node* rel = tn.child("RelativeFilename");
      const Node* abs = tn.child("FileName");
      std::string f = rel && !rel->props.empty() ? rel->props[0].s : "";
      if (f.empty() && abs && !abs->props.empty()) f = abs->props[0].s;
      fm.textures[st.first] = f;
    }
    const int k = (int)materials.size();
    materials.push_back(fm);
    mat_index[id] = k;
    return k;
  };

  // Per model, in order: its geometry's checks, polygons and material
  // groups, and the materials in order of first use -- everything whose
  // order matters. The corners of each (model, material) mesh are then
  // filled on several threads; the first defect in the order above is the
  // one reported.
  struct GeomWork {
    const std::vector<double>* V;
    const std::vector<int64_t>* PVI;
    const std::vector<double>* Nd;
    const std::vector<double>* Ud;
    LayerMap map_n, map_u;
    M4 W;
    double IT[9];
    bool inv_ok;
    std::vector<std::pair<int64_t, int64_t>> polys;  // [first corner, end)
  };
  struct MeshWork {
    size_t geom;
    std::vector<int64_t> polys;  // of the geometry, in order
    FbxMesh mesh;
    const char* err = nullptr;
  };
  std::vector<GeomWork> geoms;
  std::vector<MeshWork> work;
  std::string late_err;  // a defect found before the corners, after the work listed so far
  geoms.reserve(models.size());
  for (const ModelInfo& mi : models) {
    int64_t gid = 0;
    for (const auto& gm : geom_model)
      if (gm.second == mi.id) {
        gid = gm.first;
        break;
      }
    if (!gid) continue;
    const Node& g = *geometry[gid];
    const Node* vn = g.child("Vertices");
    const Node* pn = g.child("PolygonVertexIndex");
    if (!vn || !pn || vn->props.empty() || pn->props.empty()) {
      char m[96];
      std::snprintf(m, sizeof m, "geometry %lld without vertices or polygons", (long long)gid);
      late_err = m;
      break;
    }
    GeomWork gw;
    gw.V = &vn->props[0].da;
    gw.PVI = &pn->props[0].ia;
    const Node* le_n = g.child("LayerElementNormal");
    const Node* le_u = g.child("LayerElementUV");
    const Node* le_m = g.child("LayerElementMaterial");
    gw.Nd = nullptr;
    gw.Ud = nullptr;
    if (le_n && le_n->child("Normals") && !le_n->child("Normals")->props.empty())
      gw.Nd = &le_n->child("Normals")->props[0].da;
    if (le_u && le_u->child("UV") && !le_u->child("UV")->props.empty()) gw.Ud = &le_u->child("UV")->props[0].da;
    gw.map_n = le_n ? layer_map(*le_n, "NormalsIndex") : LayerMap();
    gw.map_u = le_u ? layer_map(*le_u, "UVIndex") : LayerMap();
    gw.W = mul(world(mi), mi.geometric);
    gw.inv_ok = inverse3(gw.W, gw.IT);
    const std::vector<int64_t>& PVI = *gw.PVI;
    for (size_t c = 0, first = 0; c < PVI.size(); ++c)
      if (PVI[c] < 0) {
        gw.polys.push_back({(int64_t)first, (int64_t)c + 1});
        first = c + 1;
      }
    const std::vector<int64_t>& model_mat_ids = model_mats[mi.id];
    const Node* mat_node = le_m ? le_m->child("Materials") : nullptr;
    const std::vector<int64_t>* mat_ids = mat_node && !mat_node->props.empty() ? &mat_node->props[0].ia : nullptr;
    const Node* mat_map = le_m ? le_m->child("MappingInformationType") : nullptr;
    const bool mat_same = mat_map && !mat_map->props.empty() && mat_map->props[0].s == "AllSame";
    auto poly_material = [&](int64_t poly) -> int64_t {
      if (!mat_ids) return 0;
      const int64_t k = mat_same ? 0 : poly;
      return k >= 0 && k < (int64_t)mat_ids->size() ? (*mat_ids)[(size_t)k] : 0;
    };
    std::map<int64_t, std::vector<int64_t>> by_mat;  // material index -> polygons
    for (int64_t p = 0; p < (int64_t)gw.polys.size(); ++p) by_mat[poly_material(p)].push_back(p);
    const size_t gi = geoms.size();
    const bool has_nrm = gw.Nd != nullptr && gw.inv_ok, has_uv = gw.Ud != nullptr;
    geoms.push_back(std::move(gw));
    for (auto& bm : by_mat) {
      const int64_t li = bm.first;
      const int64_t fid = li >= 0 && li < (int64_t)model_mat_ids.size() ? model_mat_ids[(size_t)li] : 0;
      MeshWork mw;
      mw.geom = gi;
      mw.polys = std::move(bm.second);
      mw.mesh.material = use_material(fid);
      mw.mesh.has_nrm = has_nrm;
      mw.mesh.has_uv = has_uv;
      work.push_back(std::move(mw));
    }
  }
  // the corners: a vertex per polygon corner in world space, its normal
  // through the inverse transpose, its uv; polygons as fans
  auto fill = [&](MeshWork& mw) {
    const GeomWork& gw = geoms[mw.geom];
    const std::vector<double>& V = *gw.V;
    const std::vector<int64_t>& PVI = *gw.PVI;
    const M4& W = gw.W;
    const double* IT = gw.IT;
    FbxMesh& mesh = mw.mesh;
    for (int64_t p : mw.polys) {
      const int64_t c0 = gw.polys[(size_t)p].first, c1 = gw.polys[(size_t)p].second;
      if (c1 - c0 < 3) continue;  // lines and points drop out
      const int32_t base = (int32_t)(mesh.pos.size() / 3);
      for (int64_t c = c0; c < c1; ++c) {
        const int64_t vi = PVI[(size_t)c] < 0 ? ~PVI[(size_t)c] : PVI[(size_t)c];
        if (vi < 0 || 3 * vi + 2 >= (int64_t)V.size()) {
          mw.err = "a polygon refers to a vertex that does not exist";
          return;
        }
        const double x = V[3 * vi], y = V[3 * vi + 1], z = V[3 * vi + 2];
        for (int r = 0; r < 3; ++r) {
          double s = W[4 * r] * x;
          s += W[4 * r + 1] * y;
          s += W[4 * r + 2] * z;
          s += W[4 * r + 3];
          mesh.pos.push_back((float)s);
        }
        if (mesh.has_nrm) {
          const int64_t k = layer_index(gw.map_n, c, p, vi);
          if (k < 0 || 3 * k + 2 >= (int64_t)gw.Nd->size()) {
            mw.err = "a normal index is out of range";
            return;
          }
          const double nx = (*gw.Nd)[3 * k], ny = (*gw.Nd)[3 * k + 1], nz = (*gw.Nd)[3 * k + 2];
          double t[3];
          for (int r = 0; r < 3; ++r) {  // inverse transpose: column r of the inverse
            double s = IT[r] * nx;
            s += IT[3 + r] * ny;
            s += IT[6 + r] * nz;
            t[r] = s;
          }
          double len = t[0] * t[0];
          len += t[1] * t[1];
          len += t[2] * t[2];
          len = std::sqrt(len);
          for (int r = 0; r < 3; ++r) mesh.nrm.push_back(len > 0.0 ? (float)(t[r] / len) : 0.0f);
        }
        if (mesh.has_uv) {
          const int64_t k = layer_index(gw.map_u, c, p, vi);
          if (k < 0 || 2 * k + 1 >= (int64_t)gw.Ud->size()) {
            mw.err = "a uv index is out of range";
            return;
          }
          mesh.uv.push_back((float)(*gw.Ud)[2 * k]);
          mesh.uv.push_back((float)(*gw.Ud)[2 * k + 1]);
        }
      }
      const int32_t nc = (int32_t)(c1 - c0);
      for (int32_t k = 1; k + 1 < nc; ++k) {  // a fan from the first corner
        mesh.tris.push_back(base);
        mesh.tris.push_back(base + k);
        mesh.tris.push_back(base + k + 1);
      }
    }
  };
  std::atomic<size_t> next{0};
  rmn::run_threads(std::min(rmn::host_threads(), work.size()), [&](size_t) {
    for (size_t j; (j = next.fetch_add(1)) < work.size();) fill(work[j]);
  });
  for (const MeshWork& mw : work)
    if (mw.err) return fail(RMN_ERR_INVALID_ARGUMENT, "%s: %s", path.c_str(), mw.err);
  if (!late_err.empty()) return fail(RMN_ERR_INVALID_ARGUMENT, "%s: %s", path.c_str(), late_err.c_str());
  for (MeshWork& mw : work)
    if (!mw.mesh.tris.empty()) meshes.push_back(std::move(mw.mesh));
  return RMN_OK;
}

}  // namespace rmn
