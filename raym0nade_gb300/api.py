"""Host-side mirror of the reference's render interface over the C ABI.

The reference exposes ``Model`` (include/model.h:25-43, with the ray queries
``rayHit`` / ``rayHit_test``), ``RenderArgs`` (include/render.h:8-15),
``render_multiThread(Model&, const RenderArgs&)`` (include/render.h:43) and
``Photo`` (include/image.h:15-67, with ``shade``, ``gammaCorrection``,
``FXAA``, ``postProcessing``, ``save``). This module keeps those names and
argument meanings; every call goes through librmn.so (include/rmn.h).

Arrays may be numpy (host) or torch CUDA tensors (device-resident, used in
place). Errors raise ``RmnError`` carrying the library's status and message.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _lib
from . import scenes as _scenes

try:  # torch is plumbing for device memory and streams; optional for host-only use
    import torch
except Exception:  # pragma: no cover
    torch = None

STATUS = {0: "RMN_OK", 1: "RMN_ERR_INVALID_ARGUMENT", 2: "RMN_ERR_CUDA", 3: "RMN_ERR_OUT_OF_MEMORY",
          4: "RMN_ERR_UNSUPPORTED", 5: "RMN_ERR_DEVICE_LIMIT", 6: "RMN_ERR_INTERNAL"}

# Photo::ShadeOption (include/image.h:17-34) + the ABI's gamma bit.
BaseColor, Emission, DirectLight, IndirectLight, Diffuse, Specular = 1, 2, 4, 8, 16, 32
shapeNormal, surfaceNormal, DoBloom, DoFXAA, DoDepthFieldBlur = 64, 128, 256, 512, 1024
Full = 63
Direct_Diffuse, Direct_Specular = DirectLight | Diffuse, DirectLight | Specular
Indirect_Diffuse, Indirect_Specular = IndirectLight | Diffuse, IndirectLight | Specular
GAMMA = 4096
EXPORTS, EXPORTS_DOF = 20, 5  # RMN_EXPORTS, RMN_EXPORTS_DOF
GBUFFER_FLOATS = 21


class RmnError(RuntimeError):
    def __init__(self, status: int, where: str):
        msg = _lib.load().rmn_last_error().decode(errors="replace")
        super().__init__(f"{where}: {STATUS.get(status, status)}: {msg}")
        self.status = status


def _check(status: int, where: str) -> None:
    if status != 0:
        raise RmnError(status, where)


def _ptr(a):
    if a is None:
        return None
    if torch is not None and isinstance(a, torch.Tensor):
        return a.data_ptr()
    return a.ctypes.data


def _stream(stream):
    if stream is None:
        return None
    if torch is not None and isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    return int(stream)


class Model:
    """A scene resident in HBM; what the reference's Model holds after
    Model::Model (faces, materials, light objects, sky map, BVH)."""

    def __init__(self, scene, model_name: str | None = None, skyMap_name: str = "null"):
        """Model(scene) from arrays, or Model(model_folder, model_name,
        skyMap_name) as the reference's constructor (src/model.cpp:172):
        an OBJ/MTL model imported by raym0nade_gb300.assets.load_model."""
        lib = _lib.load()
        if isinstance(scene, str):
            self._from_file(lib, scene, model_name, skyMap_name)
            return
        scene.check()
        self._keep = [np.ascontiguousarray(x) for x in (scene.positions, scene.normals, scene.uvs, scene.indices,
                                                        scene.mesh_first, scene.mesh_material, scene.materials)]
        env = None if scene.env is None else np.ascontiguousarray(scene.env, np.float32)
        self._keep.append(env)
        p, n, u, i, mf, mm, mat = self._keep[:7]
        _, texs, mtex = scene.texture_arrays()
        tarr = (_lib.Texture * max(len(texs), 1))(*[_lib.Texture(t.shape[1], t.shape[0], t.shape[2], t.ctypes.data)
                                                     for t in texs])
        self._keep += [texs, mtex, tarr]
        d = _lib.SceneDesc(p.shape[0], _ptr(p), _ptr(n), _ptr(u), i.shape[0], _ptr(i), mm.shape[0], _ptr(mf),
                           _ptr(mm), mat.shape[0], _ptr(mat), 0 if env is None else env.shape[1],
                           0 if env is None else env.shape[0], _ptr(env), len(texs),
                           C.cast(tarr, C.c_void_p).value if texs else None, _ptr(mtex))
        h = C.c_void_p()
        _check(lib.rmn_scene_create(C.byref(d), C.byref(h)), "rmn_scene_create")
        self._h = h
        self.name = scene.name
        self.num_triangles = int(i.shape[0])
        self._keep = None  # the library copied everything it needs

    def _from_file(self, lib, model_folder: str, model_name: str, skyMap_name: str) -> None:
        """rmn_model_read -> rmn_model_desc -> rmn_scene_create: the arrays
        go from the reader to the scene without a copy in Python."""
        mh = C.c_void_p()
        st = lib.rmn_model_read(os.fsencode(model_folder), os.fsencode(model_name or ""),
                                os.fsencode(skyMap_name), C.byref(mh))
        if st != 0:
            raise ValueError(lib.rmn_last_error().decode(errors="replace"))
        try:
            d = _lib.SceneDesc()
            _check(lib.rmn_model_desc(mh, C.byref(d)), "rmn_model_desc")
            h = C.c_void_p()
            _check(lib.rmn_scene_create(C.byref(d), C.byref(h)), "rmn_scene_create")
            self._h = h
            self.name = os.path.splitext(model_name or "")[0]
            self.num_triangles = int(d.num_triangles)
            self._keep = None
        finally:
            lib.rmn_model_free(mh)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().rmn_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        s = _lib.SceneInfo()
        _check(_lib.load().rmn_scene_info_get(self._h, C.byref(s)), "rmn_scene_info_get")
        return {k: getattr(s, k) for k, _ in s._fields_}

    def texture(self, index: int, level: int = 0) -> np.ndarray:
        """Mip level `level` of scene texture `index` as the device holds it
        (ImageData::data[level]): (h, w, 4) uint8 (rmn_scene_texture_get)."""
        lib = _lib.load()
        info = _lib.ImageDesc()
        _check(lib.rmn_scene_texture_get(self._h, index, level, C.byref(info), None, 0), "rmn_scene_texture_get")
        out = np.empty((info.height, info.width, 4), np.uint8)
        _check(lib.rmn_scene_texture_get(self._h, index, level, C.byref(info), out.ctypes.data, out.nbytes),
               "rmn_scene_texture_get")
        return out

    def rayHit(self, rays, hits=None, stream=None):
        """Model::rayHit over a batch. rays: (n, 8) float32 (origin, t_min,
        dir, t_max). Returns hits (n, 4): face id (int32 bits), t, alpha, beta."""
        n = int(rays.shape[0])
        if hits is None:
            hits = _empty_like_device(rays, (n, 4), np.float32)
        _check(_lib.load().rmn_trace_closest(self._h, _ptr(rays), n, _ptr(hits), _stream(stream)),
               "rmn_trace_closest")
        return hits

    def rayHit_test(self, rays, occluded=None, stream=None):
        """Model::rayHit_test over a batch; t_max of each ray is its aim depth."""
        n = int(rays.shape[0])
        if occluded is None:
            occluded = _empty_like_device(rays, (n,), np.uint8)
        _check(_lib.load().rmn_trace_shadow(self._h, _ptr(rays), n, _ptr(occluded), _stream(stream)),
               "rmn_trace_shadow")
        return occluded


def _empty_like_device(ref, shape, dtype):
    if torch is not None and isinstance(ref, torch.Tensor) and ref.is_cuda:
        tdt = {np.float32: torch.float32, np.uint8: torch.uint8}[dtype]
        return torch.empty(shape, dtype=tdt, device=ref.device)
    return np.empty(shape, dtype)


def split_hits(hits):
    """(face, t, bary(gamma, alpha, beta)) from rmn_hit records."""
    h = hits.cpu().numpy() if (torch is not None and isinstance(hits, torch.Tensor)) else np.asarray(hits)
    face = h[:, 0].copy().view(np.int32)
    al, be = h[:, 2], h[:, 3]
    ga = (np.float32(1.0) - al - be).astype(np.float32)
    return face, h[:, 1].copy(), np.stack([ga, al, be], 1)


@dataclass
class RenderArgs:
    """RenderArgs, include/render.h:8-15 (+ max_depth, seed, lanes_per_pixel)."""
    position: tuple
    direction: tuple
    up: tuple
    right: tuple
    accuracy: float
    focus: float = 1.0
    CoC: float = 0.0
    exposure: float = 1.0
    P_Direct: float = 0.7
    width: int = 256
    height: int = 256
    spp: int = 64
    threads: int = 1
    savePath: str = ""
    max_depth: int = 16
    seed: int = 1
    lanes_per_pixel: int = 0
    slots_per_unit: int = 0

    @staticmethod
    def from_camera(cam: "_scenes.Camera", seed: int = 1, savePath: str = "", lanes_per_pixel: int = 0,
                    slots_per_unit: int = 0):
        return RenderArgs(cam.position, cam.direction, cam.up, cam.right, cam.accuracy, cam.focus, cam.coc,
                          cam.exposure, cam.p_direct, cam.width, cam.height, cam.spp, 1, savePath, cam.max_depth,
                          seed, lanes_per_pixel, slots_per_unit)

    def c(self) -> "_lib.RenderArgs":
        a = _lib.RenderArgs()
        for k in ("position", "direction", "up", "right"):
            getattr(a, k)[:] = [float(x) for x in getattr(self, k)]
        a.accuracy, a.focus, a.CoC, a.exposure, a.P_Direct = (float(self.accuracy), float(self.focus),
                                                               float(self.CoC), float(self.exposure),
                                                               float(self.P_Direct))
        a.width, a.height, a.spp, a.threads = int(self.width), int(self.height), int(self.spp), int(self.threads)
        a.max_depth, a.seed, a.lanes_per_pixel = int(self.max_depth), int(self.seed), int(self.lanes_per_pixel)
        a.slots_per_unit = int(self.slots_per_unit)
        return a


def parse_render_args(text: str) -> RenderArgs:
    """A `create args` block of docs/renderArguments.txt, as
    MyConsole::createRenderArgs reads it (src/myconsole.cpp:27-67): direction,
    right, up, position as (D, R, U) in that basis, accuracy focus CoC
    exposure, width height, spp threads P_Direct, savePath."""
    tok = text.split()
    f = [float(x) for x in tok[:16]]
    direction, right, up = np.array(f[0:3]), np.array(f[3:6]), np.array(f[6:9])
    D, R, U = f[9:12]
    position = D * direction + R * right + U * up
    width, height = int(tok[16]), int(tok[17])
    spp, threads, p_direct = int(tok[18]), int(tok[19]), float(tok[20])
    save = tok[21] if len(tok) > 21 else ""
    return RenderArgs(tuple(position.astype(np.float32)), tuple(direction), tuple(up), tuple(right), f[12], f[13],
                      f[14], f[15], p_direct, width, height, spp, threads, save)


class Photo:
    """Render outputs (Photo, include/image.h:15-67): four RadianceData
    buffers (rgb + Var per pixel) and a G-buffer, on the device when torch
    CUDA is available (else host numpy)."""

    def __init__(self, width: int, height: int, exposure: float = 1.0, device=True):
        self.width, self.height, self.exposure = width, height, exposure
        n = width * height
        if device and torch is not None and torch.cuda.is_available():
            mk = lambda k: torch.zeros((n, k), dtype=torch.float32, device="cuda")
            self.dropped = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        else:
            mk = lambda k: np.zeros((n, k), np.float32)
            self.dropped = np.full((n,), -1, np.int32)
        self.radiance_Dd, self.radiance_Ds, self.radiance_Id, self.radiance_Is = mk(4), mk(4), mk(4), mk(4)
        self.Gbuffer = mk(GBUFFER_FLOATS)

    def c_image(self) -> "_lib.Image":
        return _lib.Image(_ptr(self.radiance_Dd), _ptr(self.radiance_Ds), _ptr(self.radiance_Id),
                          _ptr(self.radiance_Is), _ptr(self.Gbuffer), _ptr(getattr(self, "dropped", None)))

    def shade(self, options: int = Full, out=None, stream=None):
        """Photo::shade(options) [+ gammaCorrection with GAMMA] [+ FXAA with DoFXAA]."""
        if out is None:
            out = _empty_like_device(self.Gbuffer, (self.height, self.width, 3), np.float32)
        img = self.c_image()
        _check(_lib.load().rmn_compose(C.byref(img), self.width, self.height, float(self.exposure), int(options),
                                       _ptr(out), _stream(stream)), "rmn_compose")
        return out

    # Photo's depth-of-field state (include/image.h:36-38)
    focus, CoC, cameraPosition = 1.0, 0.0, (0.0, 0.0, 0.0)

    def _post_args(self) -> "_lib.PostArgs":
        return _lib.PostArgs(self.width, self.height, float(self.exposure), float(self.focus), float(self.CoC),
                             (C.c_float * 3)(*self.cameraPosition))

    def post_process(self, options: int, out=None, stream=None):
        """rmn_post_process: Photo::shade(options), depth of field
        (DoDepthFieldBlur) and bloom (DoBloom), gammaCorrection with GAMMA,
        FXAA with DoFXAA."""
        if out is None:
            out = _empty_like_device(self.Gbuffer, (self.height, self.width, 3), np.float32)
        img, a = self.c_image(), self._post_args()
        _check(_lib.load().rmn_post_process(C.byref(img), C.byref(a), int(options), _ptr(out), _stream(stream)),
               "rmn_post_process")
        return out

    def postProcessing(self, options: int, out=None, stream=None):
        """Photo::postProcessing (src/image.cpp:470-479): shade, depth of
        field, bloom, gammaCorrection, FXAA, as `options` asks."""
        return self.post_process(options | GAMMA, out, stream)

    def spatialClamp(self, stream=None):
        """Photo::spatialClamp (src/image.cpp:77-82), in place."""
        img = self.c_image()
        _check(_lib.load().rmn_spatial_clamp(C.byref(img), self.width, self.height, _stream(stream)),
               "rmn_spatial_clamp")

    def filter(self, stream=None):
        """Photo::filter (src/image.cpp:201-213), in place."""
        img = self.c_image()
        _check(_lib.load().rmn_filter(C.byref(img), self.width, self.height, _stream(stream)), "rmn_filter")

    def export_set(self, out=None, stream=None):
        """rmn_export_set: the images render_multiThread exports
        (src/render.cpp:641-674) as {tag: (h, w, 3)}; the radiance buffers are
        clamped and filtered on the way, as there."""
        lib = _lib.load()
        n = EXPORTS + EXPORTS_DOF
        if out is None:
            out = _empty_like_device(self.Gbuffer, (n, self.height, self.width, 3), np.float32)
        img, a, cnt = self.c_image(), self._post_args(), C.c_int32(0)
        _check(lib.rmn_export_set(C.byref(img), C.byref(a), _ptr(out), C.byref(cnt), _stream(stream)),
               "rmn_export_set")
        return {lib.rmn_export_tag(k).decode(): out[k] for k in range(cnt.value)}

    @staticmethod
    def load(file_name: str):
        """Photo(const char* file_name) / Photo::load (src/image.cpp:18,
        534-607): the PNG's RGB, every colour type and depth brought to 8
        bits as libpng's transforms there do (rmn_image_load), divided by
        255 -> (h, w, 3) float32 on the host. An interlaced (Adam7) PNG comes
        back as its whole image; the reference reads it with png_read_row
        without png_set_interlace_handling, so libpng hands it the rows of
        the separate interlace passes instead."""
        from . import assets
        return assets.load_png(file_name).astype(np.float32) / np.float32(255.0)

    @staticmethod
    def reverseGammaCorrection(rgb):
        """Photo::reverseGammaCorrection (src/image.cpp:610-613): every
        channel to the power 2.2f (the step before FXAA in the reference's
        fxaa.cpp tool). Host arrays go through rmn_reverse_gamma (the C
        library's powf, as the reference); a device tensor is raised with
        torch.pow on the GPU (CUDA's powf: within an ulp or two)."""
        if torch is not None and isinstance(rgb, torch.Tensor) and rgb.is_cuda:
            return torch.pow(rgb, 2.2)
        a = np.ascontiguousarray(np.asarray(rgb, np.float32))
        out = np.empty_like(a)
        _check(_lib.load().rmn_reverse_gamma(_ptr(a), a.size // 3, _ptr(out)), "rmn_reverse_gamma")
        return out

    @staticmethod
    def save(rgb, path: str) -> None:
        """Photo::save (src/image.cpp:481-532): an 8-bit RGB PNG through
        rmn_save_png, each channel * 255 truncated to a byte; a path ending in
        .ppm writes binary PPM with the same bytes."""
        if path.lower().endswith(".ppm"):
            a = rgb.cpu().numpy() if (torch is not None and isinstance(rgb, torch.Tensor)) else np.asarray(rgb)
            b = np.clip(a * np.float32(255.0), 0, 255).astype(np.uint8)
            with open(path, "wb") as f:
                f.write(b"P6\n%d %d\n255\n" % (b.shape[1], b.shape[0]))
                f.write(b.tobytes())
            return
        if not (torch is not None and isinstance(rgb, torch.Tensor)):
            rgb = np.ascontiguousarray(rgb, np.float32)
        h, w = int(rgb.shape[0]), int(rgb.shape[1])
        _check(_lib.load().rmn_save_png(_ptr(rgb), w, h, path.encode()), "rmn_save_png")


def render(model: Model, args: RenderArgs, photo: Photo | None = None, stream=None) -> Photo:
    """The per-pixel work of render_multiThread (src/render.cpp:593-631)."""
    if photo is None:
        photo = Photo(args.width, args.height, args.exposure)
    a = args.c()
    img = photo.c_image()
    _check(_lib.load().rmn_render(model.handle, C.byref(a), C.byref(img), _stream(stream)), "rmn_render")
    return photo


GRAD_PER_MATERIAL = 5  # base colour r, g, b; roughness; emission scale


def adjoint(model: Model, args: RenderArgs, photo: Photo, d_image, d_materials=None, stream=None):
    """rmn_adjoint: dL/d(material parameters) for dL/dI of the linear composed
    image of `photo` (a forward render of `model` with `args`). d_image:
    (H*W, 3) float32; returns (num_materials, 5) float32 (base r, g, b,
    roughness, emission scale), on the device when d_image is a CUDA tensor."""
    n = model.info()["num_materials"]
    if d_materials is None:
        if torch is not None and isinstance(d_image, torch.Tensor):
            d_materials = torch.zeros((n, GRAD_PER_MATERIAL), dtype=torch.float32, device=d_image.device)
        else:
            d_materials = np.zeros((n, GRAD_PER_MATERIAL), np.float32)
    a = args.c()
    img = photo.c_image()
    _check(_lib.load().rmn_adjoint(model.handle, C.byref(a), C.byref(img), _ptr(d_image), _ptr(d_materials),
                                   _stream(stream)), "rmn_adjoint")
    return d_materials


def render_profile(model: Model, args: RenderArgs, photo: Photo | None = None, stream=None):
    """rmn_render_profile_get: render twice (counting, then timed) and return
    (photo, dict of kernel times and visit counters)."""
    if photo is None:
        photo = Photo(args.width, args.height, args.exposure)
    a = args.c()
    img = photo.c_image()
    prof = _lib.RenderProfile()
    _check(_lib.load().rmn_render_profile_get(model.handle, C.byref(a), C.byref(img), C.byref(prof),
                                              _stream(stream)), "rmn_render_profile_get")
    return photo, {k: getattr(prof, k) for k, _ in prof._fields_}


def _batch_items(items):
    arr = (_lib.BatchItem * len(items))()
    for i, (m, a, ph) in enumerate(items):
        arr[i].scene = m.handle.value
        arr[i].args = a.c()
        arr[i].image = ph.c_image()
    return arr


def autotune(items, pixel_fraction: float = 1.0 / 16, stream=None) -> dict:
    """rmn_batch_autotune over (Model, RenderArgs, Photo) items: the fastest
    slots per unit, pool size, lanes and traversal stack on a proxy with
    `pixel_fraction` of the pixels. Pass slots_per_unit to the items'
    RenderArgs and pool_workers / lanes / stack_entries to Batch."""
    res = _lib.TuneResult()
    _check(_lib.load().rmn_batch_autotune(_batch_items(items), len(items), float(pixel_fraction), C.byref(res),
                                          _stream(stream)), "rmn_batch_autotune")
    return {k: getattr(res, k) for k, _ in res._fields_}


def batch_device_bytes(items, pool_workers: int = 0, lanes: int = 0) -> int:
    """rmn_batch_device_bytes: device bytes a Batch of these (Model,
    RenderArgs, Photo) items would take with these options (unit records and
    worker pool; scenes and images excluded)."""
    out = C.c_int64()
    opt = _lib.BatchOptions(1, int(pool_workers), int(lanes), 0, 0, 0)
    _check(_lib.load().rmn_batch_device_bytes(_batch_items(items), len(items), C.byref(opt), C.byref(out)),
           "rmn_batch_device_bytes")
    return int(out.value)


class Batch:
    """rmn_batch: many renders in one persistent launch, optionally replayed
    from a captured CUDA graph. Photos must live on the device."""

    def __init__(self, items, use_graph: bool = True, stream=None, pool_workers: int = 0, lanes: int = 0,
                 stack_entries: int = 0, ray_order: int = 0):
        """items: list of (Model, RenderArgs, Photo); pool_workers per lane;
        stack_entries 0 (library default), 23 or 27; ray_order 1 bins the
        ray queues before each traversal launch."""
        lib = _lib.load()
        arr = _batch_items(items)
        h = C.c_void_p()
        opt = _lib.BatchOptions(1 if use_graph else 0, int(pool_workers), int(lanes), int(stack_entries),
                                int(ray_order), 0)
        _check(lib.rmn_batch_create(arr, len(items), C.byref(opt), _stream(stream), C.byref(h)), "rmn_batch_create")
        self._h = h
        self.items = items

    def render(self, stream=None):
        _check(_lib.load().rmn_batch_render(self._h, _stream(stream)), "rmn_batch_render")

    def update(self, args_list, stream=None):
        """rmn_batch_update: new RenderArgs (camera, seed, exposure) per item,
        same image sizes, spp, P_Direct and depth as at creation."""
        arr = (_lib.RenderArgs * len(args_list))(*[a.c() for a in args_list])
        _check(_lib.load().rmn_batch_update(self._h, arr, len(args_list), _stream(stream)), "rmn_batch_update")

    @property
    def update_bytes(self) -> int:
        """Bytes rmn_batch_update uploads (the library's job table)."""
        return int(_lib.load().rmn_batch_update_bytes(self._h))

    def profile(self, stream=None) -> dict:
        prof = _lib.RenderProfile()
        _check(_lib.load().rmn_batch_profile(self._h, C.byref(prof), _stream(stream)), "rmn_batch_profile")
        return {k: getattr(prof, k) for k, _ in prof._fields_}

    def _from_file(self, lib, model_folder: str, model_name: str, skyMap_name: str) -> None:
        """rmn_model_read -> rmn_model_desc -> rmn_scene_create: the arrays
        go from the reader to the scene without a copy in Python."""
        mh = C.c_void_p()
        st = lib.rmn_model_read(os.fsencode(model_folder), os.fsencode(model_name or ""),
                                os.fsencode(skyMap_name), C.byref(mh))
        if st != 0:
            raise ValueError(lib.rmn_last_error().decode(errors="replace"))
        try:
            d = _lib.SceneDesc()
            _check(lib.rmn_model_desc(mh, C.byref(d)), "rmn_model_desc")
            h = C.c_void_p()
            _check(lib.rmn_scene_create(C.byref(d), C.byref(h)), "rmn_scene_create")
            self._h = h
            self.name = os.path.splitext(model_name or "")[0]
            self.num_triangles = int(d.num_triangles)
            self._keep = None
        finally:
            lib.rmn_model_free(mh)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().rmn_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_multiThread(model: Model, args: RenderArgs) -> Photo:
    """render_multiThread (include/render.h:43, src/render.cpp:593-677):
    render, then write the reference's export set (src/render.cpp:641-674:
    spatialClamp, filter, bloom, depth of field when CoC > eps, FXAA) to
    savePath + '(tag).png'; the radiance buffers end clamped and filtered,
    as the reference's Photo does."""
    photo = render(model, args)
    if args.savePath:
        d = os.path.dirname(args.savePath)
        if d:
            os.makedirs(d, exist_ok=True)
        photo.focus, photo.CoC, photo.cameraPosition = args.focus, args.CoC, tuple(args.position)
        exports = photo.export_set()
        host = {tag: (rgb.cpu().numpy() if (torch is not None and isinstance(rgb, torch.Tensor)) else rgb)
                for tag, rgb in exports.items()}
        # the PNG files are independent: encode them on several host threads
        # (the library call releases the interpreter lock)
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as pool:
            jobs = [pool.submit(Photo.save, rgb, f"{args.savePath}({tag}).png") for tag, rgb in host.items()]
            for j in jobs:
                j.result()
    return photo


def FXAA(rgb, out=None, stream=None):
    """Photo::FXAA on an (h, w, 3) float32 image."""
    h, w = int(rgb.shape[0]), int(rgb.shape[1])
    if out is None:
        out = _empty_like_device(rgb, (h, w, 3), np.float32)
    _check(_lib.load().rmn_fxaa(_ptr(rgb), _ptr(out), w, h, _stream(stream)), "rmn_fxaa")
    return out
