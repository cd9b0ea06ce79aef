"""Oracle for the model importer: Model::Model(model_folder, model_name,
skyMap_name) (src/model.cpp:124-215, src/material.cpp:150-336) for
Wavefront OBJ/MTL files, restated in Python with this package's own image
readers (oracle/image_codecs.py). TEST INFRASTRUCTURE ONLY: tests/ check
the library's native importer (rmn_model_read) against it array for array.

assimp, which the reference imports with (aiProcess_Triangulate |
PreTransformVertices | SortByPType | FixInfacingNormals, with
AI_CONFIG_PP_PTV_KEEP_HIERARCHY), is not installed: what it does for OBJ
files is restated from its documented behaviour -- one mesh per run of faces
with the same object and material, a vertex per face corner, polygons split
into a fan from their first corner (assimp ear-clips polygons of more than
four corners), lines and points dropped, its default material first, the
map_Kd / map_Ks / map_Ke / norm texture statements, d and Tr for opacity,
and the bounding-box test of FixInfacingNormals. Parity with assimp itself
is unpinned.
"""
from __future__ import annotations

import os

import numpy as np

from oracle import image_codecs
from raym0nade_gb300 import scenes

TEX_DIFFUSE, TEX_SPECULAR, TEX_EMISSIVE, TEX_NORMALS = 0, 1, 2, 3
MTL_TEXTURES = {"map_kd": TEX_DIFFUSE, "map_ks": TEX_SPECULAR, "map_ke": TEX_EMISSIVE, "norm": TEX_NORMALS,
                "map_kn": TEX_NORMALS}
_MTL_OPTIONS = {"-blendu": 1, "-blendv": 1, "-cc": 1, "-clamp": 1, "-imfchan": 1, "-texres": 1, "-bm": 1,
                "-boost": 1, "-mm": 2, "-o": 3, "-s": 3, "-t": 3, "-type": 1}
DEFAULT_MATERIAL = "DefaultMaterial"


def _to_rgba(img: np.ndarray) -> np.ndarray:
    if img.shape[2] == 4:
        return np.ascontiguousarray(img)
    out = np.full(img.shape[:2] + (4,), 255, np.uint8)
    out[..., :3] = img[..., :3]
    return out


def _load_texture(filename: str):
    """Material::loadImageFromFile by extension; None for other types or a
    DDS that does not decode."""
    ext = filename[filename.rfind(".") + 1:]
    if ext in ("png", "PNG"):
        return _to_rgba(image_codecs.png_read(filename))
    if ext in ("dds", "DDS"):
        try:
            return _to_rgba(image_codecs.dds_read(filename))
        except Exception:
            return None
    return None


def url_decode(src: str) -> str:
    """urlDecode (src/material.cpp:9-24): %XX sequences to bytes."""
    out = bytearray()
    b = src.encode("latin-1", errors="replace")
    i = 0
    while i < len(b):
        if b[i] == 0x25:  # '%'
            hexd = b[i + 1:i + 3].decode("latin-1")
            n = 0
            for ch in hexd:  # sscanf("%x") reads the leading hex digits
                if ch in "0123456789abcdefABCDEF":
                    n = n * 16 + int(ch, 16)
                else:
                    break
            out.append(n & 0xFF)
            i += 3
        else:
            out.append(b[i])
            i += 1
    return out.decode("latin-1")


def glass_properties(name: str):
    """Material::loadMaterialProperties for opacity < 0.99
    (src/material.cpp:307-329): (opacity, ior, roughness, transmitting
    colour) by material name."""
    roughness = 0.5 if name == "Ice" else 5e-3
    colours = {"TransparentGlassWine": (0.2, 0.08, 0.07), "TransparentGlass": (1.0, 1.0, 1.0),
               "Water": (1.0, 1.0, 1.0), "Ice": (1.0, 1.0, 1.0), "Beer": (0.8, 0.7, 0.55),
               "Red_Wine": (0.24, 0.09, 0.07), "White_Wine": (0.85, 0.78, 0.6)}
    return 0.0, 1.25, roughness, colours.get(name, (0.0, 0.0, 0.0))


def _texture_path(rest: str) -> str:
    """The file name of an MTL texture statement after its options: an
    option takes its arguments (up to three numbers for -o/-s/-t, one word
    or number for the others) as long as a file name is left after them."""
    toks = rest.split()
    i = 0
    while i < len(toks) - 1 and toks[i].lower() in _MTL_OPTIONS:
        n = _MTL_OPTIONS[toks[i].lower()]
        i += 1
        for k in range(n):
            if i >= len(toks) - 1:
                break
            if k > 0 and not _is_number(toks[i]):  # -o/-s/-t/-mm: fewer numbers than allowed
                break
            i += 1
    return " ".join(toks[i:])


def _is_number(s: str) -> bool:
    try:
        float(s)
        return True
    except ValueError:
        return False


def parse_mtl(path: str) -> list:
    """The materials of an MTL file in definition order: dicts with name,
    opacity and the texture file names by slot."""
    mats = []
    with open(path, "r", errors="replace") as f:
        lines = f.read().splitlines()
    for lineno, raw in enumerate(lines, 1):
        line = raw.strip()
        if not line or line.startswith("#"):
            continue
        key, rest = (line.split(None, 1) + [""])[:2]
        k = key.lower()
        rest = rest.strip()
        try:
            if k == "newmtl":
                mats.append({"name": rest, "opacity": np.float32(1.0), "textures": {}})
            elif not mats:
                continue
            elif k == "d":  # an ai_real (float), as assimp hands the opacity over
                mats[-1]["opacity"] = np.float32(float(rest.split()[-1]))
            elif k == "tr":
                mats[-1]["opacity"] = np.float32(1.0) - np.float32(float(rest.split()[-1]))
            elif k in MTL_TEXTURES:
                mats[-1]["textures"][MTL_TEXTURES[k]] = _texture_path(rest)
        except (ValueError, IndexError) as e:
            raise ValueError(f"{path}:{lineno}: cannot read {line[:60]!r} ({e})") from None
    return mats


def _fix_infacing(positions: np.ndarray, normals: np.ndarray) -> bool:
    """FixInfacingNormals' published test: the normals point inwards when
    the bounding box of the vertices moved along their normals has a smaller
    volume than the bounding box of the vertices. A flat mesh (volume 0) is
    left alone. The renderer turns every vertex normal toward the face's
    normal before use (getHitNormals, src/model.cpp:240-270), so the result
    changes the arrays but never an image."""
    if positions.shape[0] == 0:
        return False
    v0 = float(np.prod(positions.max(0) - positions.min(0)))
    moved = positions + normals
    v1 = float(np.prod(moved.max(0) - moved.min(0)))
    return v0 > 0.0 and v1 < v0


def load_obj(path: str):
    """Parse a Wavefront OBJ into meshes the way assimp's OBJ import leaves
    them after Triangulate / SortByPType: one mesh per run of faces with the
    same object and material, a vertex per face corner, polygons split into
    a fan from their first corner, lines and points dropped. Returns
    (meshes, mtllibs); each mesh is (material name, positions (k, 3),
    normals (k, 3) or None, uvs (k, 2) or None, indices (t, 3))."""
    v, vt, vn = [], [], []
    meshes, mtllibs = [], []
    cur = {"mat": DEFAULT_MATERIAL, "corners": [], "tris": []}

    def close():
        if cur["tris"]:
            meshes.append((cur["mat"], cur["corners"], cur["tris"]))
        cur["corners"], cur["tris"] = [], []

    def index(tok, n):
        i = int(tok)
        return i - 1 if i > 0 else n + i

    with open(path, "r", errors="replace") as f:
        lines = f.read().replace("\\\n", " ").splitlines()  # a trailing backslash continues the line
    for lineno, raw in enumerate(lines, 1):
        try:
            line = raw.strip()
            if not line or line[0] == "#":
                continue
            key, rest = (line.split(None, 1) + [""])[:2]
            if key in ("v", "vn"):
                xyz = [float(x) for x in rest.split()[:3]]
                if len(xyz) != 3:
                    raise ValueError("three coordinates expected")
                (v if key == "v" else vn).append(xyz)
            elif key == "vt":
                t = rest.split()
                vt.append([float(t[0]), float(t[1]) if len(t) > 1 else 0.0])
            elif key == "f":
                corners = []
                for tok in rest.split():
                    parts = tok.split("/")
                    pi = index(parts[0], len(v))
                    ti = index(parts[1], len(vt)) if len(parts) > 1 and parts[1] else -1
                    ni = index(parts[2], len(vn)) if len(parts) > 2 and parts[2] else -1
                    corners.append((pi, ti, ni))
                if len(corners) < 3:
                    continue
                base = len(cur["corners"])
                cur["corners"].extend(corners)
                for k in range(1, len(corners) - 1):
                    cur["tris"].append((base, base + k, base + k + 1))
            elif key == "usemtl":
                if rest.strip() != cur["mat"]:
                    close()
                cur["mat"] = rest.strip()
            elif key in ("o", "g"):
                close()
            elif key == "mtllib":
                mtllibs.extend(rest.split())
        except (ValueError, IndexError) as e:
            raise ValueError(f"{path}:{lineno}: cannot read {raw.strip()[:60]!r} ({e})") from None
    close()
    P = np.asarray(v, np.float32).reshape(-1, 3)
    T = np.asarray(vt, np.float32).reshape(-1, 2)
    N = np.asarray(vn, np.float32).reshape(-1, 3)
    out = []
    for mat, corners, tris in meshes:
        c = np.asarray(corners, np.int64)
        if (c[:, 0] < 0).any() or (c[:, 0] >= len(P)).any():
            raise ValueError(f"{path}: a face refers to a vertex that does not exist")
        if (c[:, 1] >= len(T)).any() or (c[:, 2] >= len(N)).any() or (c[:, 1] < -1).any() or (c[:, 2] < -1).any():
            raise ValueError(f"{path}: a face refers to a texture coordinate or normal that does not exist")
        pos = P[c[:, 0]]
        nrm = None if (c[:, 2] < 0).any() else N[c[:, 2]]
        uv = None if (c[:, 1] < 0).any() else T[c[:, 1]]
        out.append((mat, pos, nrm, uv, np.asarray(tris, np.int32)))
    return out, mtllibs


def load_model(model_folder: str, model_name: str, skyMap_name: str = "null") -> "scenes.Scene":
    """Model::Model(model_folder, model_name, skyMap_name) for an OBJ model:
    the file is model_folder + model_name, texture paths are
    model_folder + the MTL's path (backslashes made slashes, %XX decoded,
    src/model.cpp:146-156), the sky map is model_folder + skyMap_name unless
    that is "null", decoded by hdr_to_array (SkyBox::load).

    Faces without vertex normals get their geometric normal (the reference
    dereferences assimp's missing normal array); corners without texture
    coordinates get (0, 0)."""
    model_path = model_folder + model_name
    meshes, mtllibs = load_obj(model_path)
    lib_mats = []
    for m in mtllibs:
        p = model_folder + m
        if os.path.exists(p):
            lib_mats.extend(parse_mtl(p))
    # assimp's OBJ material list: its default material first, then the MTL's
    # (a repeated name takes its last definition), then usemtl names no MTL
    # file defines, in order of use
    names = [DEFAULT_MATERIAL] + [m["name"] for m in lib_mats]
    by_name = {m["name"]: m for m in lib_mats}
    index_of = {n: i for i, n in enumerate(names)}
    indexed = []
    for mat, pos, nrm, uv, tris in meshes:
        if mat not in index_of:
            index_of[mat] = len(names)
            names.append(mat)
        indexed.append((index_of[mat], pos, nrm, uv, tris))
    specs = [by_name.get(n, {"name": n, "opacity": np.float32(1.0), "textures": {}}) for n in names]
    return assemble_model(model_folder, model_name, specs, indexed, skyMap_name)


def assemble_model(model_folder: str, model_name: str, specs: list, meshes: list,
                   skyMap_name: str = "null") -> "scenes.Scene":
    """The steps Model::Model takes after assimp's import, whatever the file
    format (src/model.cpp:172-215, src/material.cpp:150-336): texture files
    loaded once each in order of first use, a glass material row where the
    opacity is below 0.99, vertex normals (the geometric normal where a mesh
    has none, FixInfacingNormals where it has them), (0, 0) where a mesh has
    no uvs, and the sky. specs: dicts with name, opacity and textures by
    slot; meshes: (material index, positions, normals or None, uvs or None,
    indices)."""
    model_path = model_folder + model_name
    names = [s["name"] for s in specs]
    cache, textures = {}, []
    mat_rows, mat_tex = [], []
    for spec in specs:
        name = spec["name"]
        slots = [-1, -1, -1, -1]
        for slot in sorted(spec["textures"]):
            p = url_decode((model_folder + spec["textures"][slot]).replace("\\", "/"))
            if p not in cache:
                tex = _load_texture(p)
                cache[p] = -1 if tex is None else len(textures)
                if tex is not None:
                    textures.append(tex)
            slots[slot] = cache[p]
        if spec["opacity"] < np.float32(0.99):  # loadMaterialProperties compares floats
            op, ior, rough, trans = glass_properties(name)
            row = scenes.material(roughness=rough, opacity=op, ior=ior, transmitting=trans)
        else:
            row = scenes.material()
        row[3] = 0.0  # no constant diffuse texel: white unless a texture is given
        mat_rows.append(row)
        mat_tex.append(slots)

    pos_l, nrm_l, uv_l, idx_l, first, mesh_mat = [], [], [], [], [0], []
    nv = 0
    for mat, pos, nrm, uv, tris in meshes:
        if nrm is None:
            a, b, c = pos[tris[:, 0]], pos[tris[:, 1]], pos[tris[:, 2]]
            g = np.cross(b - a, c - a)
            g /= np.maximum(np.linalg.norm(g, axis=1, keepdims=True), 1e-30)
            nrm = np.zeros_like(pos)
            for k in range(3):
                nrm[tris[:, k]] = g
        elif _fix_infacing(pos, nrm):
            nrm = -nrm
        if uv is None:
            uv = np.zeros((pos.shape[0], 2), np.float32)
        pos_l.append(pos)
        nrm_l.append(nrm.astype(np.float32))
        uv_l.append(uv)
        idx_l.append(tris + nv)
        nv += pos.shape[0]
        first.append(first[-1] + tris.shape[0])
        mesh_mat.append(mat)
    if not idx_l:
        raise ValueError(f"{model_path}: no triangles")
    env = None
    if skyMap_name != "null":
        try:
            env = np.ascontiguousarray(image_codecs.hdr_read(model_folder + skyMap_name), np.float32)
        except Exception:
            env = None
    mats = np.stack(mat_rows).astype(np.float32)
    mt = np.asarray(mat_tex, np.int32)
    scene = scenes.Scene(
        positions=np.ascontiguousarray(np.concatenate(pos_l), np.float32),
        normals=np.ascontiguousarray(np.concatenate(nrm_l), np.float32),
        uvs=np.ascontiguousarray(np.concatenate(uv_l), np.float32),
        indices=np.ascontiguousarray(np.concatenate(idx_l), np.int32),
        mesh_first=np.asarray(first, np.int32), mesh_material=np.asarray(mesh_mat, np.int32),
        materials=mats, env=env, name=os.path.splitext(model_name)[0],
        textures=textures if textures else None, mat_tex=mt if textures else None)
    scene.material_names = names
    return scene
