"""Oracle test infrastructure -- not part of the shipped library.

ctypes bindings for the two CPU checker libraries built by oracle/Makefile:

* ``port``: oracle/_build/libport.so, the CPU restatement of the reference's
  hot path (oracle/port/port.cpp);
* ``ref``:  oracle/_ref/libref.so, the reference's own sources compiled with
  shims (oracle/ref/harness.cpp); only present where the reference checkout
  was available at build time;
* ``ref_tex``: oracle/_ref/libref_tex.so, the same with the reference's own
  src/material.cpp (8-bit textures, mip chains) instead of constant texels.

Both export the same functions (prefix ``port_`` / ``ref_``), wrapped here by
``OracleLib``. Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libport.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")
REF_TEX_SO = os.path.join(HERE, "_ref", "libref_tex.so")
# the reference checkout, where one is present: from the environment
REFERENCE_DIR = os.environ.get("RMN_REFERENCE_DIR", "")
PIX_FLOATS = 40


class _SceneIn(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_int32), ("positions", C.c_void_p), ("normals", C.c_void_p), ("uvs", C.c_void_p),
        ("num_triangles", C.c_int32), ("indices", C.c_void_p),
        ("num_meshes", C.c_int32), ("mesh_first", C.c_void_p), ("mesh_material", C.c_void_p),
        ("num_materials", C.c_int32), ("materials", C.c_void_p),
        ("env_width", C.c_int32), ("env_height", C.c_int32), ("env_rgb", C.c_void_p),
        ("num_textures", C.c_int32), ("tex_dims", C.c_void_p), ("tex_data", C.c_void_p), ("mat_tex", C.c_void_p),
    ]


def build(with_reference: bool | None = None) -> None:
    """Compile the port, and the reference harness when the reference
    checkout exists (or when ``with_reference`` is True)."""
    targets = ["port"]
    if with_reference or (with_reference is None and os.path.isdir(os.path.join(REFERENCE_DIR, "src"))):
        targets.append("ref")
    env = dict(os.environ, RMN_REFERENCE_DIR=REFERENCE_DIR)
    subprocess.run(["make", "-s", "-C", HERE, "-j8"] + targets, check=True, env=env)


def _ptr(a):
    return None if a is None else a.ctypes.data


class OracleScene:
    def __init__(self, lib: "OracleLib", scene):
        self.lib = lib
        self._keep = [np.ascontiguousarray(x) for x in (scene.positions, scene.normals, scene.uvs, scene.indices,
                                                        scene.mesh_first, scene.mesh_material, scene.materials)]
        env = None if scene.env is None else np.ascontiguousarray(scene.env, np.float32)
        self._keep.append(env)
        p, n, u, i, mf, mm, mat = self._keep[:7]
        dims, texs, mtex = scene.texture_arrays()
        ptrs = (C.c_void_p * max(len(texs), 1))(*[t.ctypes.data for t in texs])
        self._keep += [dims, texs, mtex, ptrs]
        d = _SceneIn(p.shape[0], _ptr(p), _ptr(n), _ptr(u), i.shape[0], _ptr(i), mm.shape[0], _ptr(mf), _ptr(mm),
                     mat.shape[0], _ptr(mat), 0 if env is None else env.shape[1], 0 if env is None else env.shape[0],
                     _ptr(env), len(texs), _ptr(dims), C.cast(ptrs, C.c_void_p).value if texs else None, _ptr(mtex))
        self.handle = lib.fn("scene_create")(C.byref(d))
        if not self.handle:
            raise ValueError(f"{lib.kind}: scene refused")
        self.num_triangles = int(i.shape[0])

    def close(self):
        if self.handle:
            self.lib.fn("scene_destroy")(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bvh(self):
        n = self.lib.fn("bvh_size")(self.handle)
        boxes = np.empty((n, 6), np.float32)
        ranges = np.empty((n, 2), np.int32)
        order = np.empty(self.num_triangles, np.int32)
        self.lib.fn("bvh_export")(self.handle, _ptr(boxes), _ptr(ranges), _ptr(order))
        return boxes, ranges, order

    def lights(self):
        n = self.lib.fn("light_count")(self.handle)
        out = np.empty((n, 8), np.float32)
        if n:
            self.lib.fn("light_export")(self.handle, _ptr(out))
        return out

    def trace_closest(self, rays: np.ndarray, threads: int = 8):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        face = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        bc = np.empty((n, 3), np.float32)
        self.lib.fn("trace_closest")(self.handle, _ptr(rays), n, _ptr(face), _ptr(t), _ptr(bc), threads)
        return face, t, bc

    def trace_shadow(self, rays: np.ndarray, threads: int = 8):
        rays = np.ascontiguousarray(rays, np.float32)
        occ = np.empty(rays.shape[0], np.uint8)
        self.lib.fn("trace_shadow")(self.handle, _ptr(rays), rays.shape[0], _ptr(occ), threads)
        return occ

    def trace_stats(self, rays: np.ndarray, shadow: bool = False):
        rays = np.ascontiguousarray(rays, np.float32)
        out = np.zeros(3, np.uint64)
        self.lib.fn("trace_stats")(self.handle, _ptr(rays), rays.shape[0], 1 if shadow else 0, _ptr(out))
        return {"inner": int(out[0]), "leaves": int(out[1]), "tris": int(out[2])}

    def render(self, camera, seed: int, mode: int = 0, rect=None, threads: int = 8) -> np.ndarray:
        """Per-pixel records (h, w, 40) of the pixel rectangle (x0, y0, x1, y1)."""
        x0, y0, x1, y1 = rect or (0, 0, camera.width, camera.height)
        out = np.zeros((y1 - y0, x1 - x0, PIX_FLOATS), np.float32)
        args = camera.packed(threads)
        self.lib.fn("render")(self.handle, _ptr(args), C.c_uint64(seed), mode, x0, y0, x1, y1, _ptr(out), threads)
        return out

    def render_pixels(self, camera, seed: int, pixels, mode: int = 0, threads: int = 8) -> np.ndarray:
        """Per-pixel records (n, 40) of the listed pixels (row-major indices
        y * width + x), each rendered as in a whole-image render."""
        px = np.ascontiguousarray(pixels, np.int32)
        out = np.zeros((px.shape[0], PIX_FLOATS), np.float32)
        args = camera.packed(threads)
        self.lib.fn("render_pixels")(self.handle, _ptr(args), C.c_uint64(seed), mode, _ptr(px), px.shape[0],
                                     _ptr(out), threads)
        return out


class OracleLib:
    def __init__(self, kind: str = "port"):
        self.kind = kind
        path = {"port": PORT_SO, "ref": REF_SO, "ref_tex": REF_TEX_SO}[kind]
        prefix = "port" if kind == "port" else "ref"
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is not built (oracle.bindings.build())")
        self.lib = C.CDLL(path)
        self._fns = {}
        sig = {
            "scene_create": (C.c_void_p, [C.c_void_p]),
            "scene_destroy": (None, [C.c_void_p]),
            "bvh_size": (C.c_int, [C.c_void_p]),
            "bvh_export": (None, [C.c_void_p] * 4),
            "light_count": (C.c_int, [C.c_void_p]),
            "light_export": (None, [C.c_void_p, C.c_void_p]),
            "trace_closest": (None, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
            "render_pixels": (None, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_void_p, C.c_int64, C.c_void_p,
                                     C.c_int]),
            "trace_shadow": (None, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int]),
            "trace_stats": (None, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_void_p]),
            "render": (None, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                              C.c_void_p, C.c_int]),
            "compose": (None, [C.c_void_p, C.c_int64, C.c_float, C.c_int, C.c_void_p]),
            "gamma": (None, [C.c_void_p, C.c_int64, C.c_void_p]),
            "reverse_gamma": (None, [C.c_void_p, C.c_int64, C.c_void_p]),
            "fxaa": (None, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
            "photo": (None, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
            "mip_chain": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_size_t]),
            "url_decode": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int]),
            "material_properties": (None, [C.c_char_p, C.c_float, C.c_int, C.c_void_p]),
            "save_rows": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_void_p]),
        }
        for name, (res, args) in sig.items():
            f = getattr(self.lib, f"{prefix}_{name}", None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
            self._fns[name] = f

    def fn(self, name):
        return self._fns[name]

    def scene(self, scene) -> OracleScene:
        return OracleScene(self, scene)

    def mip_chain(self, tex: np.ndarray) -> list:
        """ImageData::generateMipmaps of the reference (ref_tex only): the
        levels of an (h, w, c) uint8 image."""
        tex = np.ascontiguousarray(tex, np.uint8)
        h, w, c = tex.shape
        out = np.zeros(tex.nbytes * 2, np.uint8)
        depth = self.fn("mip_chain")(_ptr(tex), w, h, c, _ptr(out), out.nbytes)
        assert depth > 0
        levels, at = [], 0
        for lv in range(depth):
            n = (h >> lv) * (w >> lv) * c
            levels.append(out[at:at + n].reshape(h >> lv, w >> lv, c).copy())
            at += n
        return levels

    def material_properties(self, name: str, opacity=None) -> np.ndarray:
        """Material::loadMaterialProperties of the reference (ref_tex only):
        (opacity, ior, roughness, transmitting rgb, hasFullyTransparentPart)."""
        out = np.zeros(7, np.float32)
        self.fn("material_properties")(name.encode(), 1.0 if opacity is None else float(opacity),
                                       0 if opacity is None else 1, _ptr(out))
        return out

    def save_rows(self, rgb: np.ndarray, path: str) -> np.ndarray:
        """The 8-bit rows the reference's Photo::save hands to libpng for an
        (h, w, 3) float32 image (ref / ref_tex only)."""
        rgb = np.ascontiguousarray(rgb, np.float32)
        h, w = rgb.shape[:2]
        out = np.zeros((h, w, 3), np.uint8)
        assert self.fn("save_rows")(_ptr(rgb), w, h, path.encode(), _ptr(out)) == 0
        return out

    def python_loaders(self):
        """(sky_load, dds_load): the reference's SkyBox::load and
        Material::loadImageFromDDS, which call the Python functions
        hdr_to_array / dds_to_array of ./scripts through the embedded
        interpreter -- here the running one, so they are called with the GIL
        held (ref_tex only)."""
        lib = C.PyDLL(REF_TEX_SO)
        sky = lib.ref_sky_load
        sky.restype, sky.argtypes = C.c_int, [C.c_char_p, C.c_void_p, C.c_long, C.c_void_p, C.c_void_p]
        dds = lib.ref_dds_load
        dds.restype, dds.argtypes = C.c_int, [C.c_char_p, C.c_void_p, C.c_long, C.c_void_p]

        def sky_load(path, capacity=1 << 24):
            out = np.zeros(capacity, np.float32)
            w, h = C.c_int(), C.c_int()
            if sky(path.encode(), _ptr(out), capacity, C.byref(w), C.byref(h)) != 0:
                return None
            return out[:w.value * h.value * 3].reshape(h.value, w.value, 3).copy()

        def dds_load(path, capacity=1 << 24):
            out = np.zeros(capacity, np.uint8)
            dims = np.zeros(3, np.int32)
            if dds(path.encode(), _ptr(out), capacity, _ptr(dims)) != 0:
                return None
            w, h, c = (int(x) for x in dims)
            return out[:w * h * c].reshape(h, w, c).copy()

        return sky_load, dds_load

    def url_decode(self, s: str) -> str:
        """urlDecode of the reference (ref_tex only)."""
        buf = C.create_string_buffer(4 * len(s) + 8)
        n = self.fn("url_decode")(s.encode("latin-1"), buf, len(buf))
        assert n >= 0
        return buf.raw[:n].decode("latin-1")

    def compose(self, recs: np.ndarray, exposure: float = 1.0, gamma: bool = True) -> np.ndarray:
        recs = np.ascontiguousarray(recs, np.float32)
        shp = recs.shape[:-1]
        n = int(np.prod(shp))
        out = np.empty(shp + (3,), np.float32)
        self.fn("compose")(_ptr(recs), n, exposure, 1 if gamma else 0, _ptr(out))
        return out

    def gamma(self, rgb: np.ndarray) -> np.ndarray:
        rgb = np.ascontiguousarray(rgb, np.float32)
        out = np.empty_like(rgb)
        self.fn("gamma")(_ptr(rgb), rgb.size // 3, _ptr(out))
        return out

    def reverse_gamma(self, rgb: np.ndarray) -> np.ndarray:
        """Photo::reverseGammaCorrection (reference build only)."""
        rgb = np.ascontiguousarray(rgb, np.float32)
        out = np.empty_like(rgb)
        self.fn("reverse_gamma")(_ptr(rgb), rgb.size // 3, _ptr(out))
        return out

    def photo(self, recs: np.ndarray, stages: int, options: int = 0, exposure: float = 1.0, focus: float = 1.0,
              coc: float = 0.0, camera=(0.0, 0.0, 0.0)):
        """Photo's post passes on render records (h, w, 40): stages 1
        spatialClamp, 2 filter (both update the records' radiance, returned
        as a new array), 4 postProcessing(options), 8 the same without gamma
        and FXAA. Returns (records, rgb (h, w, 3) or None)."""
        recs = np.array(recs, np.float32, copy=True, order="C")
        h, w = recs.shape[:2]
        rgb = np.zeros((h, w, 3), np.float32)
        post = np.array([exposure, focus, coc, *camera], np.float32)
        self.fn("photo")(_ptr(recs), w, h, stages, options, _ptr(post), _ptr(rgb))
        return recs, (rgb if stages & 12 else None)

    def fxaa(self, rgb: np.ndarray) -> np.ndarray:
        rgb = np.ascontiguousarray(rgb, np.float32)
        h, w, _ = rgb.shape
        out = np.empty_like(rgb)
        self.fn("fxaa")(_ptr(rgb), _ptr(out), w, h)
        return out


def have_ref() -> bool:
    return os.path.exists(REF_SO)


def have_ref_tex() -> bool:
    return os.path.exists(REF_TEX_SO)
