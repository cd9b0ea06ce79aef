"""A Wavefront OBJ/MTL model with PNG/DDS textures and an HDR sky, written
for the importer tests (raym0nade_gb300.assets.load_model).

The model exercises what Model::Model's import meets in practice: objects
and groups, material switches inside an object, quads and a pentagon,
absolute and negative indices, v, v//vn, v/vt and v/vt/vn corners, a line
and a point (dropped), faces before any usemtl (assimp's default material),
texture statements with options, %XX escapes and backslashes, a texture of
an unsupported type, a glass material (d < 0.99) named as the reference's
table names them, an emissive DDS texture (a light object), an alpha-cut DDS
texture, and a mesh with inward-pointing vertex normals.
"""
from __future__ import annotations

import os

import numpy as np

from tests.golden import image_files as F

MTL = """# materials of room.obj
newmtl Walls
Kd 0.8 0.8 0.8
map_Kd tex/checker.png
map_Ks -s 1 1 1 tex/spec%20map.dds
norm tex\\normal.png

newmtl Glow
map_Ke -bm 1.0 tex/glow.dds

newmtl Water
d 0.4
Ni 1.33

newmtl Leaf
map_Kd tex/leaf.dds

newmtl Plain
Kd 0.5 0.1 0.1

newmtl Unused
Tr 0.0

newmtl Odd
map_Kd tex/picture.tga
"""

# (material or None, [polygon corners (v, vt or None, vn or None)]) per face,
# with object/group markers; the room spans [0, 1]^3, front (z = 0) open.
ROOM_V = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]


def _box(lo, hi):
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    return [(x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0),
            (x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)]


def write_room(folder: str, seed: int = 3) -> dict:
    """Write room.obj, room.mtl, tex/* and sky.hdr under `folder` (which
    ends in '/'); return what the importer must produce from them."""
    rng = np.random.default_rng(seed)
    os.makedirs(folder + "tex", exist_ok=True)
    exp = {}
    # textures
    cx = (np.indices((16, 16)).sum(0) // 4) % 2
    checker = np.stack([40 + 180 * cx, 60 + 120 * cx, 200 - 150 * cx], -1).astype(np.uint8)
    open(folder + "tex/checker.png", "wb").write(F.encode_png(checker, 2, 8, filters=(4, 1, 2, 3)))
    normal = np.zeros((8, 8, 3), np.uint8)
    normal[...] = (128, 128, 255)
    normal[::2, ::2] = (170, 100, 230)
    open(folder + "tex/normal.png", "wb").write(F.encode_png(normal, 2, 8, level=1))
    spec = rng.integers(0, 256, 4 * 4 * 8).astype(np.uint8).tobytes()  # BC1, 16 x 16
    open(folder + "tex/spec map.dds", "wb").write(F.encode_dds(16, 16, spec, b"DXT1"))
    glow = rng.integers(0, 256, 2 * 2 * 16).astype(np.uint8)  # BC3, 8 x 8, opaque bright
    glow = glow.reshape(4, 16)
    glow[:, 0], glow[:, 1] = 255, 255
    glow[:, 8:10] = (0xFF, 0xFF)
    open(folder + "tex/glow.dds", "wb").write(F.encode_dds(8, 8, glow.tobytes(), b"DXT5"))
    leaf = np.zeros((4, 16), np.uint8)  # BC3, 8 x 8: left half alpha 0, right half 255
    leaf[:, 0], leaf[:, 1] = 0, 255
    leaf[:, 8:10] = (0xE0, 0x07)  # green endpoints
    for b in (1, 3):  # right-hand blocks: every alpha index 1 (a1 = 255); left: index 0 (a0 = 0)
        leaf[b, 2:8] = [0x49, 0x92, 0x24, 0x49, 0x92, 0x24]
    open(folder + "tex/leaf.dds", "wb").write(F.encode_dds(8, 8, leaf.tobytes(), b"DXT5"))
    open(folder + "tex/picture.tga", "wb").write(b"\0" * 18)
    exp["checker"] = checker
    exp["normal"] = normal
    exp["spec"] = spec
    exp["glow"] = glow.tobytes()
    exp["leaf"] = leaf.tobytes()
    # sky
    sky = np.exp(rng.normal(0.0, 1.0, (16, 32, 3))).astype(np.float32)
    rgbe = F.float_to_rgbe(sky)
    open(folder + "sky.hdr", "wb").write(F.encode_hdr(rgbe))
    exp["sky"] = F.rgbe_expected(rgbe)
    open(folder + "room.mtl", "w").write(MTL)

    # geometry
    vs, vts, vns = [], [], []
    lines = ["# room.obj", "mtllib room.mtl"]
    meshes = []  # expected: (material, corners [(pos, uv, nrm)], triangles count)

    def add_v(p):
        vs.append(p)
        lines.append("v %.6f %.6f %.6f" % p)
        return len(vs)

    def add_vt(t):
        vts.append(t)
        lines.append("vt %.6f %.6f" % t)
        return len(vts)

    def add_vn(n):
        vns.append(n)
        lines.append("vn %.6f %.6f %.6f" % n)
        return len(vns)

    def face(corners, negative=False):
        toks = []
        for v, t, n in corners:
            vv = v - len(vs) - 1 if negative else v
            tt = "" if t is None else str(t - len(vts) - 1 if negative else t)
            nn = None if n is None else str(n - len(vns) - 1 if negative else n)
            toks.append(str(vv) if (t is None and n is None) else
                        f"{vv}/{tt}" if n is None else f"{vv}/{tt}/{nn}")
        lines.append("f " + " ".join(toks))
        meshes[-1][1].append([(vs[v - 1], None if t is None else vts[t - 1], None if n is None else vns[n - 1])
                              for v, t, n in corners])

    # faces before any usemtl: assimp's default material
    lines.append("o Start")
    a, b, c = add_v((0.2, 0.01, 0.9)), add_v((0.3, 0.01, 0.9)), add_v((0.25, 0.01, 0.8))
    meshes.append(("DefaultMaterial", []))
    face([(a, None, None), (b, None, None), (c, None, None)])

    lines.append("o Room")
    rv = [add_v(p) for p in ROOM_V]
    t = [add_vt(x) for x in [(0, 0), (2, 0), (2, 2), (0, 2)]]  # wraps past 1
    n = {k: add_vn(d) for k, d in {"up": (0, 1, 0), "down": (0, -1, 0), "back": (0, 0, -1),
                                   "r": (-1, 0, 0), "l": (1, 0, 0)}.items()}  # pointing into the room
    lines.append("usemtl Walls")
    meshes.append(("Walls", []))
    quads = [((0, 1, 5, 4), "up"), ((3, 7, 6, 2), "down"), ((4, 5, 6, 7), "back"), ((0, 4, 7, 3), "l"),
             ((1, 2, 6, 5), "r")]
    for q, k in quads:
        face([(rv[i], t[j], n[k]) for j, i in enumerate(q)])

    lines.append("o Box")
    bv = [add_v(p) for p in _box((0.55, 0.0, 0.55), (0.8, 0.3, 0.8))]
    bn = add_vn((0.0, 1.0, 0.0))
    lines.append("usemtl Plain")
    meshes.append(("Plain", []))
    for q in [(3, 2, 6, 7), (0, 1, 2, 3)]:
        face([(bv[i], None, bn) for i in q], negative=True)
    lines.append("usemtl Walls")  # a switch inside the object: a new mesh
    meshes.append(("Walls", []))
    face([(bv[i], t[k], bn) for k, i in enumerate((4, 5, 6))])

    lines.append("g LightGroup")
    lv = [add_v(p) for p in [(0.4, 0.999, 0.4), (0.6, 0.999, 0.4), (0.6, 0.999, 0.6), (0.4, 0.999, 0.6)]]
    lines.append("usemtl Glow")
    meshes.append(("Glow", []))
    face([(lv[i], t[i], None) for i in range(4)])  # v/vt: no normals

    lines.append("o Glass")
    gv = [add_v((0.3 + 0.1 * np.cos(a), 0.5 + 0.1 * np.sin(a), 0.5)) for a in np.linspace(0, 2 * np.pi, 6)[:5]]
    gn = add_vn((0.0, 0.0, -1.0))
    lines.append("usemtl Water")
    meshes.append(("Water", []))
    face([(v, None, gn) for v in gv])  # a pentagon

    lines.append("o Leaf")
    fv = [add_v(p) for p in [(0.1, 0.2, 0.3), (0.4, 0.2, 0.3), (0.4, 0.5, 0.3), (0.1, 0.5, 0.3)]]
    lines.append("usemtl Leaf")
    meshes.append(("Leaf", []))
    face([(fv[i], t[i], gn) for i in range(4)])
    lines.append("l %d %d" % (fv[0], fv[1]))
    lines.append("p %d" % fv[2])

    # a closed cube with normals pointing to its centre, large enough (4 units)
    # for the bounding-box test to see them point inwards; far behind the room
    lines.append("o Inward")
    iv = [add_v(p) for p in _box((-2.0, -2.0, 8.0), (2.0, 2.0, 12.0))]
    centre = np.array([0.0, 0.0, 10.0])
    inn = [add_vn(tuple((centre - np.array(vs[i - 1])) / np.linalg.norm(centre - np.array(vs[i - 1]))))
           for i in iv]
    lines.append("usemtl Odd")
    meshes.append(("Odd", []))
    for q in [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (0, 4, 7, 3), (1, 2, 6, 5)]:
        face([(iv[i], None, inn[i]) for i in q])
    open(folder + "room.obj", "w").write("\n".join(lines) + "\n")
    exp["meshes"] = meshes
    exp["materials"] = ["DefaultMaterial", "Walls", "Glow", "Water", "Leaf", "Plain", "Unused", "Odd"]
    return exp


def room_camera(width: int = 64, height: int = 48, spp: int = 16, max_depth: int = 16):
    """In front of the open side of the room at (0.5, 0.5, -0.5), looking
    in (+z), 50 degree field of view across the width."""
    import math

    from raym0nade_gb300 import scenes
    acc = math.tan(math.radians(25.0)) / (width / 2.0)
    return scenes.Camera((0.5, 0.5, -0.5), (0.0, 0.0, 1.0), (0.0, -1.0, 0.0), (-1.0, 0.0, 0.0), acc, width, height,
                         spp, max_depth=max_depth)
