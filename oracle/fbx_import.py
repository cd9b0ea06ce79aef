"""Oracle for the binary FBX branch of the model importer: Model::Model
(src/model.cpp:172-215) reading a .fbx file, which the reference hands to
assimp (aiProcess_Triangulate | PreTransformVertices | SortByPType |
FixInfacingNormals). TEST INFRASTRUCTURE ONLY: tests/ check the library's
native importer (rmn_model_read on a .fbx name) against it array for array.

assimp is not installed. Its FBX import is restated from the container's
published description and assimp's documented behaviour, in the same
operations, in the same order and in double precision as the native reader,
so that both give identical floats:
  * node records: end offset, property count, property bytes (32-bit,
    64-bit from version 7500), name, typed properties (Y C I F D L, S R,
    arrays f d l i b raw or zlib), nested records ended by a null record;
  * Objects (Geometry "Mesh", Model, Material, Texture) and Connections
    (OO child -> parent, OP texture -> material property);
  * a model's transform T Roff Rp Rpre R Rpost^-1 Rp^-1 Soff Sp S Sp^-1,
    parents' on the left, the geometric transform on the right; vertices
    through it, normals through its inverse transpose, normalised;
  * a geometry splits into one mesh per material index (ascending), a
    vertex per polygon corner, polygons as a fan from their first corner,
    lines and points dropped; materials in order of first use, a
    "DefaultMaterial" for geometries without one; Opacity and the textures
    on DiffuseColor, SpecularColor / SpecularFactor, EmissiveColor /
    EmissiveFactor and NormalMap (RelativeFilename, else FileName; the
    last connected texture of a slot wins).
Parity with assimp itself is unpinned.
"""
from __future__ import annotations

import math
import os
import struct
import zlib

import numpy as np

from oracle import obj_import

MAGIC = b"Kaydara FBX Binary  \x00\x1a\x00"
TEXTURE_SLOTS = {"DiffuseColor": 0, "SpecularColor": 1, "SpecularFactor": 1, "EmissiveColor": 2,
                 "EmissiveFactor": 2, "NormalMap": 3}
_SCALAR = {"Y": ("<h", 2), "C": ("<B", 1), "I": ("<i", 4), "F": ("<f", 4), "D": ("<d", 8), "L": ("<q", 8)}
_ARRAY = {"f": ("<f", 4), "d": ("<d", 8), "l": ("<q", 8), "i": ("<i", 4), "b": ("<B", 1)}


class FbxError(ValueError):
    pass


class Node:
    __slots__ = ("name", "props", "kids")

    def __init__(self, name, props, kids):
        self.name, self.props, self.kids = name, props, kids

    def child(self, name):
        for k in self.kids:
            if k.name == name:
                return k
        return None


def _records(b, off, end, wide, depth, out):
    if depth > 64:
        raise FbxError("nesting deeper than 64 records")
    fw = 8 if wide else 4
    ff = "<Q" if wide else "<I"
    while off < end:
        start = off
        if off + 3 * fw > len(b):
            raise FbxError("truncated record")
        rec_end, nprops, plen = (struct.unpack_from(ff, b, off + k * fw)[0] for k in range(3))
        off += 3 * fw
        if off + 1 > len(b):
            raise FbxError("truncated record")
        nlen = b[off]
        off += 1
        if rec_end == 0 and nprops == 0 and plen == 0 and nlen == 0:
            return off
        if rec_end <= start or rec_end > end or off + nlen > rec_end:
            raise FbxError("record outside its parent")
        name = b[off:off + nlen].decode("latin-1")
        off += nlen
        if plen > rec_end - off:
            raise FbxError("properties outside their record")
        if nprops > plen:
            raise FbxError("more properties than property bytes")
        pend = off + plen
        props = []
        for _ in range(nprops):
            p, off = _prop(b, off, pend)
            props.append(p)
        if off != pend:
            raise FbxError("property bytes do not add up")
        kids = []
        if off < rec_end:
            _records(b, off, rec_end, wide, depth + 1, kids)
        out.append(Node(name, props, kids))
        off = rec_end
    return off


def _prop(b, off, pend):
    if off + 1 > pend:
        raise FbxError("truncated property")
    t = chr(b[off])
    off += 1

    def need(k):
        if off + k > pend:
            raise FbxError("truncated property")

    if t in _SCALAR:
        fmt, n = _SCALAR[t]
        need(n)
        v = struct.unpack_from(fmt, b, off)[0]
        if t == "C":
            v = int(v != 0)
        return (t, v), off + n
    if t in "SR":
        need(4)
        n = struct.unpack_from("<I", b, off)[0]
        off += 4
        need(n)
        return (t, b[off:off + n].decode("latin-1")), off + n
    if t in _ARRAY:
        need(12)
        count, enc, clen = struct.unpack_from("<III", b, off)
        off += 12
        need(clen)
        fmt, esz = _ARRAY[t]
        if count > (1 << 30) // esz:
            raise FbxError("array too long")
        raw = b[off:off + clen]
        if enc == 0:
            if clen != count * esz:
                raise FbxError("array length does not match its bytes")
        elif enc == 1:
            try:
                d = zlib.decompressobj()
                raw = d.decompress(raw)
            except zlib.error as e:
                raise FbxError(f"zlib: {e}") from None
            if len(raw) != count * esz:
                raise FbxError("zlib stream does not hold the array")
        else:
            raise FbxError("unknown array encoding")
        a = np.frombuffer(raw, np.dtype(fmt), count)
        if t == "b":
            a = (a != 0).astype(np.int64)
        elif t in "fd":
            a = a.astype(np.float64)
        else:
            a = a.astype(np.int64)
        return (t, a), off + clen
    raise FbxError("unknown property type")


def parse(data: bytes):
    """The top-level nodes of a binary FBX file."""
    if data[:5] == b"; FBX":
        raise NotImplementedError("ASCII FBX files are not read (binary only)")
    if len(data) < 27 or data[:23] != MAGIC:
        raise FbxError("not a binary FBX file")
    version = struct.unpack_from("<I", data, 23)[0]
    top = []
    _records(data, 27, len(data), version >= 7500, 0, top)
    return top


# ------------------------------------------------------------------ transforms
def _ident():
    return [1.0 if r == c else 0.0 for r in range(4) for c in range(4)]


def _mul(a, b):
    c = [0.0] * 16
    for r in range(4):
        for k in range(4):
            s = a[4 * r] * b[k]
            s += a[4 * r + 1] * b[4 + k]
            s += a[4 * r + 2] * b[8 + k]
            s += a[4 * r + 3] * b[12 + k]
            c[4 * r + k] = s
    return c


def _translate(t):
    m = _ident()
    m[3], m[7], m[11] = t
    return m


def _scale(s):
    m = _ident()
    m[0], m[5], m[10] = s
    return m


def _axis_rot(axis, deg):
    a = deg * 3.14159265358979323846 / 180.0
    c, s = math.cos(a), math.sin(a)
    m = _ident()
    i, j = (axis + 1) % 3, (axis + 2) % 3
    m[4 * i + i] = c
    m[4 * i + j] = -s
    m[4 * j + i] = s
    m[4 * j + j] = c
    return m


_ORDERS = ((0, 1, 2), (0, 2, 1), (1, 2, 0), (1, 0, 2), (2, 0, 1), (2, 1, 0))


def _euler(r, order):
    """Rotation by Euler angles in degrees, the first axis of FBX's
    RotationOrder (0 XYZ ... 5 ZYX) applied first."""
    if order < 0 or order > 5:
        order = 0
    m = _ident()
    for ax in _ORDERS[order]:
        m = _mul(_axis_rot(ax, r[ax]), m)
    return m


def _inverse3(m):
    a, b, c, d, e, f, g, h, i = m[0], m[1], m[2], m[4], m[5], m[6], m[8], m[9], m[10]
    A, B, C = e * i - f * h, -(d * i - f * g), d * h - e * g
    det = a * A + b * B + c * C
    if not abs(det) > 0.0:
        return None
    return [A / det, -(b * i - c * h) / det, (b * f - c * e) / det,
            B / det, (a * i - c * g) / det, -(a * f - c * d) / det,
            C / det, -(a * h - b * g) / det, (a * e - b * d) / det]


def _num(q):
    """A property as a number: a float, an integer, else 0."""
    t, v = q
    if t in "DF":
        return float(v)
    return float(v) if t in "YCIL" else 0.0


def _int(q):
    return q[1] if q[0] in "YCIL" else 0


def _str(q):
    return q[1] if q[0] in "SR" else ""


def _vec3(p70, name, v):
    if p70 is None:
        return v
    for p in p70.kids:
        if p.name != "P" or len(p.props) < 7 or _str(p.props[0]) != name:
            continue
        v = [_num(p.props[4 + k]) for k in range(3)]
    return v


def _number(p70, name):
    if p70 is None:
        return None
    out = None
    for p in p70.kids:
        if p.name != "P" or len(p.props) < 5 or _str(p.props[0]) != name:
            continue
        out = _num(p.props[4])
    return out


def model_transforms(o):
    """(local, geometric) matrices of a Model node, row-major, p' = M p."""
    p70 = o.child("Properties70")
    T = _vec3(p70, "Lcl Translation", [0.0] * 3)
    R = _vec3(p70, "Lcl Rotation", [0.0] * 3)
    S = _vec3(p70, "Lcl Scaling", [1.0] * 3)
    Roff = _vec3(p70, "RotationOffset", [0.0] * 3)
    Rp = _vec3(p70, "RotationPivot", [0.0] * 3)
    Soff = _vec3(p70, "ScalingOffset", [0.0] * 3)
    Sp = _vec3(p70, "ScalingPivot", [0.0] * 3)
    Rpre = _vec3(p70, "PreRotation", [0.0] * 3)
    Rpost = _vec3(p70, "PostRotation", [0.0] * 3)
    GT = _vec3(p70, "GeometricTranslation", [0.0] * 3)
    GR = _vec3(p70, "GeometricRotation", [0.0] * 3)
    GS = _vec3(p70, "GeometricScaling", [1.0] * 3)
    order = _number(p70, "RotationOrder")
    order = 0 if order is None else int(order)
    post = _euler(Rpost, 0)
    post_inv = _ident()
    for r in range(3):
        for c in range(3):
            post_inv[4 * r + c] = post[4 * c + r]
    m = _translate(T)
    for f in (_translate(Roff), _translate(Rp), _euler(Rpre, 0), _euler(R, order), post_inv,
              _translate([-x for x in Rp]), _translate(Soff), _translate(Sp), _scale(S),
              _translate([-x for x in Sp])):
        m = _mul(m, f)
    geometric = _mul(_mul(_translate(GT), _euler(GR, 0)), _scale(GS))
    return m, geometric


def _object_name(o):
    if len(o.props) < 2 or o.props[1][0] != "S":
        return ""
    return o.props[1][1].split("\x00\x01")[0]


def _layer_index(le, index_name, c, poly, v):
    mt, rt = le.child("MappingInformationType"), le.child("ReferenceInformationType")
    mapping = _str(mt.props[0]) if mt is not None and mt.props else "ByPolygonVertex"
    ref = _str(rt.props[0]) if rt is not None and rt.props else "Direct"
    if mapping == "ByPolygonVertex":
        k = c
    elif mapping in ("ByVertice", "ByVertex"):
        k = v
    elif mapping == "ByPolygon":
        k = poly
    elif mapping == "AllSame":
        k = 0
    else:
        return -1
    if ref in ("IndexToDirect", "Index"):
        ix = _ints(le, index_name)
        if ix is None or k < 0 or k >= len(ix):
            return -1
        k = int(ix[k])
    return k


_EMPTY = np.zeros(0)


def _floats(node, name):
    """The f / d array of a child node (empty for another type), or None."""
    n = node.child(name) if node is not None else None
    if n is None or not n.props:
        return None
    return n.props[0][1] if n.props[0][0] in "fd" else _EMPTY


def _ints(node, name):
    """The i / l / b array of a child node (empty for another type), or None."""
    n = node.child(name) if node is not None else None
    if n is None or not n.props:
        return None
    return n.props[0][1] if n.props[0][0] in "ilb" else _EMPTY


def read_fbx(path: str):
    """(meshes, materials): meshes are (material index, positions (k, 3),
    normals (k, 3) or None, uvs (k, 2) or None, indices (t, 3)); materials
    are dicts with name, opacity and textures by slot."""
    with open(path, "rb") as f:
        data = f.read()
    top = parse(data)
    conns = next((n for n in reversed(top) if n.name == "Connections"), None)
    objects = next((n for n in reversed(top) if n.name == "Objects"), None)
    if objects is None:
        raise FbxError("no Objects")
    geometry, material, texture, models, model_at = {}, {}, {}, [], {}
    for o in objects.kids:
        if not o.props or o.props[0][0] != "L":
            continue
        oid = o.props[0][1]
        cls = _str(o.props[2]) if len(o.props) > 2 else ""
        if o.name == "Geometry" and cls == "Mesh":
            geometry[oid] = o
        elif o.name == "Material":
            material[oid] = o
        elif o.name == "Texture":
            texture[oid] = o
        elif o.name == "Model":
            local, geom = model_transforms(o)
            model_at[oid] = len(models)
            models.append({"id": oid, "local": local, "geometric": geom, "parent": 0})
    geom_model, model_mats, mat_tex = {}, {}, {}
    if conns is not None:
        for c in conns.kids:
            if c.name != "C" or len(c.props) < 3:
                continue
            kind, child, parent = _str(c.props[0]), _int(c.props[1]), _int(c.props[2])
            if kind == "OO":
                if child in geometry and parent in model_at:
                    geom_model.setdefault(child, parent)
                elif child in material and parent in model_at:
                    model_mats.setdefault(parent, []).append(child)
                elif child in model_at and (parent == 0 or parent in model_at):
                    models[model_at[child]]["parent"] = parent
            elif kind == "OP" and len(c.props) >= 4 and child in texture and parent in material:
                slot = TEXTURE_SLOTS.get(_str(c.props[3]))
                if slot is not None:
                    mat_tex.setdefault(parent, []).append((slot, child))

    def world(m0):
        w = m0["local"]
        p = m0["parent"]
        guard = 0
        while p != 0 and p in model_at and guard < 64:
            pm = models[model_at[p]]
            w = _mul(pm["local"], w)
            p = pm["parent"]
            guard += 1
        return w

    materials, mat_index = [], {}
    default = [-1]

    def use_material(fid):
        if fid == 0 or fid not in material:
            if default[0] < 0:
                default[0] = len(materials)
                materials.append({"name": obj_import.DEFAULT_MATERIAL, "opacity": np.float32(1.0),
                                  "textures": {}})
            return default[0]
        if fid in mat_index:
            return mat_index[fid]
        mn = material[fid]
        op = _number(mn.child("Properties70"), "Opacity")
        # names as the library hands them over (UTF-8, bad bytes replaced);
        # file names as the bytes the file holds
        name = _object_name(mn).encode("latin-1").decode("utf-8", errors="replace")
        spec = {"name": name, "opacity": np.float32(1.0 if op is None else op), "textures": {}}
        for slot, tid in mat_tex.get(fid, []):
            tn = texture[tid]
            rel, ab = tn.child("RelativeFilename"), tn.child("FileName")
            f = _str(rel.props[0]) if rel is not None and rel.props else ""
            if not f and ab is not None and ab.props:
                f = _str(ab.props[0])
            spec["textures"][slot] = os.fsdecode(f.encode("latin-1"))
        spec["textures"] = {k: v for k, v in spec["textures"].items() if v}
        mat_index[fid] = len(materials)
        materials.append(spec)
        return mat_index[fid]

    meshes = []
    for mi in models:
        gid = next((g for g in sorted(geom_model) if geom_model[g] == mi["id"]), 0)
        if not gid:
            continue
        g = geometry[gid]
        V = _floats(g, "Vertices")
        PVI = _ints(g, "PolygonVertexIndex")
        if V is None or PVI is None:
            raise FbxError(f"geometry {gid} without vertices or polygons")
        le_n, le_u, le_m = g.child("LayerElementNormal"), g.child("LayerElementUV"), g.child("LayerElementMaterial")
        Nd, Ud = _floats(le_n, "Normals"), _floats(le_u, "UV")
        W = _mul(world(mi), mi["geometric"])
        IT = _inverse3(W)
        polys, first = [], 0
        for c in range(len(PVI)):
            if PVI[c] < 0:
                polys.append((first, c + 1))
                first = c + 1
        mids = model_mats.get(mi["id"], [])
        ms = _ints(le_m, "Materials")
        mt = le_m.child("MappingInformationType") if le_m is not None else None
        same = mt is not None and bool(mt.props) and _str(mt.props[0]) == "AllSame"

        def poly_material(p):
            if ms is None:
                return 0
            k = 0 if same else p
            return int(ms[k]) if 0 <= k < len(ms) else 0

        by_mat = {}
        for p in range(len(polys)):
            by_mat.setdefault(poly_material(p), []).append(p)
        for li in sorted(by_mat):
            fid = mids[li] if 0 <= li < len(mids) else 0
            mat = use_material(fid)
            has_n = Nd is not None and IT is not None
            has_t = Ud is not None
            pos, nrm, uv, tris = [], [], [], []
            for p in by_mat[li]:
                c0, c1 = polys[p]
                if c1 - c0 < 3:
                    continue
                base = len(pos)
                for c in range(c0, c1):
                    vi = int(PVI[c])
                    vi = ~vi if vi < 0 else vi
                    if vi < 0 or 3 * vi + 2 >= len(V):
                        raise FbxError("a polygon refers to a vertex that does not exist")
                    x, y, z = float(V[3 * vi]), float(V[3 * vi + 1]), float(V[3 * vi + 2])
                    row = []
                    for r in range(3):
                        s = W[4 * r] * x
                        s += W[4 * r + 1] * y
                        s += W[4 * r + 2] * z
                        s += W[4 * r + 3]
                        row.append(s)
                    pos.append(row)
                    if has_n:
                        k = _layer_index(le_n, "NormalsIndex", c, p, vi)
                        if k < 0 or 3 * k + 2 >= len(Nd):
                            raise FbxError("a normal index is out of range")
                        nx, ny, nz = float(Nd[3 * k]), float(Nd[3 * k + 1]), float(Nd[3 * k + 2])
                        t = []
                        for r in range(3):
                            s = IT[r] * nx
                            s += IT[3 + r] * ny
                            s += IT[6 + r] * nz
                            t.append(s)
                        ln = t[0] * t[0]
                        ln += t[1] * t[1]
                        ln += t[2] * t[2]
                        ln = math.sqrt(ln)
                        nrm.append([x_ / ln if ln > 0.0 else 0.0 for x_ in t])
                    if has_t:
                        k = _layer_index(le_u, "UVIndex", c, p, vi)
                        if k < 0 or 2 * k + 1 >= len(Ud):
                            raise FbxError("a uv index is out of range")
                        uv.append([float(Ud[2 * k]), float(Ud[2 * k + 1])])
                nc = c1 - c0
                for k in range(1, nc - 1):
                    tris.append((base, base + k, base + k + 1))
            if tris:
                meshes.append((mat, np.asarray(pos, np.float64).astype(np.float32),
                               np.asarray(nrm, np.float64).astype(np.float32) if has_n else None,
                               np.asarray(uv, np.float64).astype(np.float32) if has_t else None,
                               np.asarray(tris, np.int32)))
    return meshes, materials


def load_model(model_folder: str, model_name: str, skyMap_name: str = "null"):
    """Model::Model(model_folder, model_name, skyMap_name) for a binary FBX
    model: read_fbx, then the format-independent steps of
    oracle.obj_import.assemble_model."""
    meshes, materials = read_fbx(model_folder + model_name)
    return obj_import.assemble_model(model_folder, model_name, materials, meshes, skyMap_name)
