"""Binary FBX files written for the importer tests (rmn_model_read with a
.fbx name, and oracle/fbx_import.py).

The writer lays out the container as its published description has it: a
27-byte header (magic, 0x1A 0x00, the version), node records (end offset,
property count, property bytes -- 32-bit fields, 64-bit from version 7500
--, name, typed properties, nested records closed by a null record), arrays
raw or zlib-compressed. A scene is given as models (name, transform
properties, parent, geometry, materials) and materials (name, opacity,
textures by the property they connect to).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

_ARRAY = {"d": ("<d", 8), "f": ("<f", 4), "i": ("<i", 4), "l": ("<q", 8), "b": ("<B", 1)}


def _prop(p, compress):
    t, v = p
    if t == "S" or t == "R":
        b = v.encode("latin-1") if isinstance(v, str) else v
        return t.encode() + struct.pack("<I", len(b)) + b
    if t in "YCIFDL":
        fmt = {"Y": "<h", "C": "<?", "I": "<i", "F": "<f", "D": "<d", "L": "<q"}[t]
        return t.encode() + struct.pack(fmt, v)
    fmt, size = _ARRAY[t]
    a = np.asarray(v).astype(np.dtype(fmt)).tobytes()
    enc = 0
    if compress:
        a = zlib.compress(a)
        enc = 1
    return t.encode() + struct.pack("<III", len(v), enc, len(a)) + a


def _node(name, props, kids, offset, wide, compress):
    """The record of one node placed at absolute `offset`."""
    pb = b"".join(_prop(p, compress) for p in props)
    nb = name.encode()
    head = (8 if wide else 4) * 3 + 1 + len(nb)
    body = b""
    if kids:
        off = offset + head + len(pb)
        for k in kids:
            rec = _node(*k, off, wide, compress)
            body += rec
            off += len(rec)
        body += b"\0" * ((8 if wide else 4) * 3 + 1)
    end = offset + head + len(pb) + len(body)
    f = "<QQQB" if wide else "<IIIB"
    return struct.pack(f, end, len(props), len(pb), len(nb)) + nb + pb + body


def fbx_bytes(nodes, version=7400, compress=False):
    """nodes: top-level (name, props, kids) triples."""
    wide = version >= 7500
    out = b"Kaydara FBX Binary  \x00\x1a\x00" + struct.pack("<I", version)
    for n in nodes:
        out += _node(*n, len(out), wide, compress)
    out += b"\0" * ((8 if wide else 4) * 3 + 1)
    return out + b"\0" * 16  # footer padding, not read


def p70(entries):
    """Properties70 with P records: (name, type, values...)."""
    kids = []
    for e in entries:
        name, typ, vals = e[0], e[1], e[2:]
        props = [("S", name), ("S", typ), ("S", ""), ("S", "A")]
        for v in vals:
            props.append(("I", v) if typ == "enum" else ("D", float(v)))
        kids.append(("P", props, []))
    return ("Properties70", [], kids)


def scene_nodes(models, materials, version=7400):
    """models: dicts with name, transform (list of Properties70 entries),
    parent (model name or None), and optionally geometry = dict(vertices
    (n, 3), pvi (polygon vertex index, negative ends), normals (layer dict:
    mapping, reference, data, index), uvs (likewise), mat (layer dict:
    mapping, data)) and materials (names, in connection order).
    materials: dicts with name, opacity (or None) and textures: (property,
    file[, True: the file as FileName with an empty RelativeFilename]).
    Returns the top-level nodes."""
    ids = {}
    nid = [1000]

    def new_id(key):
        nid[0] += 7
        ids[key] = nid[0]
        return nid[0]

    objects, conns = [], []
    for m in materials:
        mid = new_id(("mat", m["name"]))
        props = []
        if m.get("opacity") is not None:
            props.append(("Opacity", "Number", m["opacity"]))
        objects.append(("Material", [("L", mid), ("S", m["name"] + "\x00\x01Material"), ("S", "")],
                        [p70(props)]))
        for tex in m.get("textures", []):
            prop, fname = tex[0], tex[1]
            only_file_name = len(tex) > 2 and tex[2]  # an empty RelativeFilename
            tid = new_id(("tex", m["name"], prop, fname))
            objects.append(("Texture", [("L", tid), ("S", "tex\x00\x01Texture"), ("S", "")],
                            [("FileName", [("S", fname if only_file_name else "C:/abs/" + fname)], []),
                             ("RelativeFilename", [("S", "" if only_file_name else fname)], [])]))
            conns.append(("C", [("S", "OP"), ("L", tid), ("L", mid), ("S", prop)], []))
    for m in models:
        model_id = new_id(("model", m["name"]))
        objects.append(("Model", [("L", model_id), ("S", m["name"] + "\x00\x01Model"), ("S", "Mesh")],
                        [p70(m.get("transform", []))]))
        g = m.get("geometry")
        if g is not None:
            gid = new_id(("geom", m["name"]))
            kids = [("Vertices", [("d", np.asarray(g["vertices"], np.float64).ravel())], []),
                    ("PolygonVertexIndex", [("i", np.asarray(g["pvi"], np.int32))], [])]
            for key, node, data_name, index_name in (("normals", "LayerElementNormal", "Normals", "NormalsIndex"),
                                                     ("uvs", "LayerElementUV", "UV", "UVIndex")):
                le = g.get(key)
                if le is None:
                    continue
                lk = [("MappingInformationType", [("S", le["mapping"])], []),
                      ("ReferenceInformationType", [("S", le["reference"])], []),
                      (data_name, [(le.get("dtype", "d"), np.asarray(le["data"], np.float64).ravel())], [])]
                if le.get("index") is not None:
                    lk.append((index_name, [("i", np.asarray(le["index"], np.int32))], []))
                kids.append((node, [("I", 0)], lk))
            if g.get("mat") is not None:
                kids.append(("LayerElementMaterial", [("I", 0)],
                             [("MappingInformationType", [("S", g["mat"]["mapping"])], []),
                              ("ReferenceInformationType", [("S", "IndexToDirect")], []),
                              ("Materials", [("i", np.asarray(g["mat"]["data"], np.int32))], [])]))
            objects.append(("Geometry", [("L", gid), ("S", m["name"] + "\x00\x01Geometry"), ("S", "Mesh")], kids))
            conns.append(("C", [("S", "OO"), ("L", gid), ("L", model_id)], []))
    for m in models:  # parents and materials after every object exists
        parent = ids[("model", m["parent"])] if m.get("parent") else 0
        conns.append(("C", [("S", "OO"), ("L", ids[("model", m["name"])]), ("L", parent)], []))
        for mat in m.get("materials", []):
            conns.append(("C", [("S", "OO"), ("L", ids[("mat", mat)]), ("L", ids[("model", m["name"])])], []))
    header = ("FBXHeaderExtension", [], [("FBXVersion", [("I", version)], [])])
    return [header, ("Objects", [], objects), ("Connections", [], conns)]


ROOM_TEXTURES = {  # the room's MTL textures as FBX texture connections
    "Walls": [("DiffuseColor", "tex/checker.png"), ("SpecularColor", "tex/spec%20map.dds"),
              ("NormalMap", "tex\\normal.png")],
    "Glow": [("EmissiveColor", "tex/glow.dds")],
    "Leaf": [("DiffuseColor", "tex/leaf.dds")],
    "Odd": [("DiffuseColor", "tex/picture.tga")],
}
ROOM_OPACITY = {"Water": 0.4}


def room_models(exp):
    """The meshes of tests/golden/model_files.write_room as FBX models, one
    model and geometry per mesh, identity transforms: positions, uvs and
    normals per polygon corner (ByPolygonVertex, Direct) where every
    corner of the mesh has them."""
    def as_obj(vals):  # the value the OBJ file holds: printed with 6 decimals, read as a float
        return np.asarray([[np.float32(float("%.6f" % x)) for x in v] for v in vals], np.float32).astype(np.float64)

    models, used = [], []
    for k, (mat, faces) in enumerate(exp["meshes"]):
        verts, pvi, nrm, uv = [], [], [], []
        for face in faces:
            for j, (p, t, n) in enumerate(face):
                verts.append(p)
                idx = len(verts) - 1
                pvi.append(~idx if j == len(face) - 1 else idx)
                nrm.append(n)
                uv.append(t)
        g = {"vertices": as_obj(verts), "pvi": pvi}
        if all(n is not None for n in nrm):
            g["normals"] = {"mapping": "ByPolygonVertex", "reference": "Direct", "data": as_obj(nrm)}
        if all(t is not None for t in uv):
            g["uvs"] = {"mapping": "ByPolygonVertex", "reference": "Direct", "data": as_obj(uv)}
        m = {"name": f"mesh{k}", "geometry": g}
        if mat != "DefaultMaterial":
            g["mat"] = {"mapping": "AllSame", "data": [0]}
            m["materials"] = [mat]
            if mat not in used:
                used.append(mat)
        models.append(m)
    materials = [{"name": n, "opacity": ROOM_OPACITY.get(n), "textures": ROOM_TEXTURES.get(n, [])} for n in used]
    return models, materials


def transform_models():
    """A hierarchy with every transform property: a parent with
    translation, rotation (ZYX order), scaling, pivots, offsets, pre- and
    post-rotation; a child with its own transform and a geometric
    transform; two materials on one geometry (ByPolygon), normals
    ByVertice with IndexToDirect, uvs ByPolygonVertex with IndexToDirect,
    a quad, a triangle and a pentagon, a line that drops out."""
    rng = np.random.default_rng(11)
    verts = rng.uniform(-1, 1, (9, 3))
    pvi = [0, 1, 2, ~3, 4, 5, ~6, 0, 2, 4, 6, ~8, 7, ~8]
    polys = 4
    nrm_data = rng.normal(0, 1, (9, 3))
    uv_data = rng.uniform(0, 1, (5, 2))
    uv_index = rng.integers(0, 5, len(pvi))
    geometry = {"vertices": verts, "pvi": pvi,
                "normals": {"mapping": "ByVertice", "reference": "IndexToDirect", "data": nrm_data,
                            "index": list(range(8, -1, -1))},
                "uvs": {"mapping": "ByPolygonVertex", "reference": "IndexToDirect", "data": uv_data,
                        "index": uv_index},
                "mat": {"mapping": "ByPolygon", "data": [1, 0, 1, 0][:polys]}}
    parent = {"name": "Parent", "transform": [
        ("Lcl Translation", "Vector3D", 1.5, -0.25, 3.0), ("Lcl Rotation", "Vector3D", 10.0, 35.0, -20.0),
        ("Lcl Scaling", "Vector3D", 1.0, 2.0, 0.5), ("RotationOrder", "enum", 5),
        ("RotationPivot", "Vector3D", 0.1, 0.2, 0.3), ("ScalingPivot", "Vector3D", -0.2, 0.1, 0.0),
        ("RotationOffset", "Vector3D", 0.05, 0.0, -0.05), ("ScalingOffset", "Vector3D", 0.0, 0.3, 0.0),
        ("PreRotation", "Vector3D", -90.0, 0.0, 0.0), ("PostRotation", "Vector3D", 0.0, 15.0, 0.0)]}
    child = {"name": "Child", "parent": "Parent", "geometry": geometry, "materials": ["Red", "Blue"],
             "transform": [("Lcl Translation", "Vector3D", 0.0, 1.0, 0.0),
                           ("Lcl Rotation", "Vector3D", 0.0, 0.0, 45.0),
                           ("GeometricTranslation", "Vector3D", 0.5, 0.0, 0.0),
                           ("GeometricScaling", "Vector3D", 2.0, 2.0, 2.0)]}
    materials = [{"name": "Red", "opacity": 1.0, "textures": []},
                 {"name": "Blue", "opacity": None, "textures": []}]
    return [parent, child], materials
