"""The reference's asset front-end on the host: image decoding and model
import into a ``Scene``.

* ``hdr_to_array`` / ``dds_to_array`` keep the names, arguments, return
  tuples and failure convention of scripts/hdr_to_array.py and
  scripts/dds_to_array.py, which the reference calls through embedded Python
  (call_image_to_array, src/material.cpp:150-188). They decode with
  librmn's ``rmn_image_load`` (imageio is not used).
* ``load_png`` is Material::loadImageFromPNG (src/material.cpp:217-285):
  8-bit RGB.
* ``load_texture`` is Material::loadImageFromFile (src/material.cpp:287-298):
  dispatch on the file extension, "png"/"PNG" or "dds"/"DDS", anything else
  printed as unsupported and left empty.
* ``load_model`` is Model::Model(model_folder, model_name, skyMap_name)
  (src/model.cpp:172-215) for Wavefront OBJ/MTL and binary FBX files, read
  natively by the library (rmn_model_read, csrc/model_io.cpp, csrc/fbx.cpp);
  the library does not use assimp, which the reference imports with. Materials follow
  Material::loadMaterialProperties (src/material.cpp:300-336): only the
  name, the opacity and the textures are read -- the MTL's colours (Kd, Ks,
  Ke) are not, as in the reference.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from . import scenes as _scenes

PNG, DDS, HDR = 0, 1, 2  # RMN_IMAGE_PNG, RMN_IMAGE_DDS, RMN_IMAGE_HDR


class ImageError(RuntimeError):
    def __init__(self, status: int, path: str):
        msg = _lib.load().rmn_last_error().decode(errors="replace")
        super().__init__(f"{path}: {msg}")
        self.status = status


def load_image(path: str, kind: int) -> np.ndarray:
    """Decode `path` with rmn_image_load: (height, width, channels) uint8, or
    float32 for HDR. Raises ImageError (status 1 malformed/missing, 4
    unsupported variant)."""
    lib = _lib.load()
    info = _lib.ImageDesc()
    bpath = os.fsencode(path)
    st = lib.rmn_image_load(bpath, kind, C.byref(info), None, 0)
    if st != 0:
        raise ImageError(st, path)
    dtype = np.uint8 if info.bytes_per_channel == 1 else np.float32
    out = np.empty((info.height, info.width, info.channels), dtype)
    st = lib.rmn_image_load(bpath, kind, C.byref(info), out.ctypes.data, out.nbytes)
    if st != 0:
        raise ImageError(st, path)
    return out


def hdr_to_array(input_hdr_file):
    """scripts/hdr_to_array.py: (width, height, channels, float32 (h, w, 3)),
    or four Nones after printing "Conversion failed: ..."."""
    try:
        img = load_image(input_hdr_file, HDR)
        return img.shape[1], img.shape[0], img.shape[2], img.astype(np.float32)
    except Exception as e:
        print(f"Conversion failed: {e}")
        return None, None, None, None


def dds_to_array(input_dds_file):
    """scripts/dds_to_array.py: (width, height, channels, bytes of the
    (h, w, channels) uint8 image), or four Nones after printing
    "Conversion failed: ..."."""
    try:
        img = load_image(input_dds_file, DDS)
        return img.shape[1], img.shape[0], img.shape[2], img.tobytes()
    except Exception as e:
        print(f"Conversion failed: {e}")
        return None, None, None, None


def load_png(filename: str) -> np.ndarray:
    """Material::loadImageFromPNG: (h, w, 3) uint8. The reference throws on a
    file it cannot read; so does this (ImageError)."""
    return load_image(filename, PNG)


def _to_rgba(img: np.ndarray) -> np.ndarray:
    """The library's 4-channel texel layout. The reference leaves an RGB
    image's channel count unset (loadImageFromPNG never assigns
    ImageData::channels), so its mip levels stay empty and its 4-byte-stride
    lookups read across texels; an RGB image enters here as RGBA with
    opaque alpha instead."""
    if img.shape[2] == 4:
        return np.ascontiguousarray(img)
    out = np.full(img.shape[:2] + (4,), 255, np.uint8)
    out[..., :3] = img[..., :3]
    return out


def load_texture(filename: str):
    """Material::loadImageFromFile: the texel array by extension, or None
    (after the reference's message) for an unsupported extension or a DDS
    that did not convert."""
    ext = filename[filename.rfind(".") + 1:]
    if ext in ("png", "PNG"):
        return _to_rgba(load_png(filename))
    if ext in ("dds", "DDS"):
        w, h, c, data = dds_to_array(filename)
        if w is None:
            return None
        return _to_rgba(np.frombuffer(data, np.uint8).reshape(h, w, c))
    print(f"Unsupported file format: {filename}")
    return None


def load_model(model_folder: str, model_name: str, skyMap_name: str = "null") -> "_scenes.Scene":
    """Model::Model(model_folder, model_name, skyMap_name) for a Wavefront
    OBJ/MTL or binary FBX model, read by the library (rmn_model_read): the
    file model_folder + model_name (FBX by a .fbx name), its MTL libraries,
    the PNG/DDS textures they name and the Radiance sky map
    model_folder + skyMap_name ("null": none),
    as a Scene of arrays (copies). Raises ValueError for a file that cannot
    be read or parsed (the message names file and line)."""
    lib = _lib.load()
    h = C.c_void_p()
    st = lib.rmn_model_read(os.fsencode(model_folder), os.fsencode(model_name), os.fsencode(skyMap_name),
                            C.byref(h))
    if st != 0:
        raise ValueError(lib.rmn_last_error().decode(errors="replace"))
    try:
        d = _lib.SceneDesc()
        if lib.rmn_model_desc(h, C.byref(d)) != 0:
            raise RuntimeError(lib.rmn_last_error().decode(errors="replace"))

        def arr(ptr, n, dtype, shape):
            if n == 0:
                return np.zeros(shape, dtype)
            buf = (C.c_char * (n * np.dtype(dtype).itemsize)).from_address(ptr)
            return np.frombuffer(buf, dtype).reshape(shape).copy()

        nv, nt, nm, nmat = d.num_vertices, d.num_triangles, d.num_meshes, d.num_materials
        env = None
        if d.env_rgb:
            env = arr(d.env_rgb, d.env_width * d.env_height * 3, np.float32, (d.env_height, d.env_width, 3))
        textures, mat_tex = None, None
        if d.num_textures > 0:
            recs = (_lib.Texture * d.num_textures).from_address(d.textures)
            textures = [arr(t.texels, t.width * t.height * 4, np.uint8, (t.height, t.width, 4)) for t in recs]
            mat_tex = arr(d.material_textures, nmat * 4, np.int32, (nmat, 4))
        scene = _scenes.Scene(
            positions=arr(d.positions, nv * 3, np.float32, (nv, 3)),
            normals=arr(d.normals, nv * 3, np.float32, (nv, 3)),
            uvs=arr(d.uvs, nv * 2, np.float32, (nv, 2)),
            indices=arr(d.indices, nt * 3, np.int32, (nt, 3)),
            mesh_first=arr(d.mesh_first, nm + 1, np.int32, (nm + 1,)),
            mesh_material=arr(d.mesh_material, nm, np.int32, (nm,)),
            materials=arr(d.materials, nmat * _scenes.MAT_FLOATS, np.float32, (nmat, _scenes.MAT_FLOATS)),
            env=env, name=os.path.splitext(model_name)[0], textures=textures, mat_tex=mat_tex)
        scene.material_names = [lib.rmn_model_material_name(h, i).decode(errors="replace") for i in range(nmat)]
        return scene
    finally:
        lib.rmn_model_free(h)
