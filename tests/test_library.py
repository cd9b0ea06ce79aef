"""Host-side checks of librmn.so that need no GPU: it builds for sm_103a,
loads, and exports every function include/rmn.h declares; host helpers."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from raym0nade_gb300 import _lib, build
    build.build()
    return _lib.load()


def declared_functions():
    text = open(os.path.join(ROOT, "include", "rmn.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const char\*|rmn_status|int32_t|int64_t)\s+(rmn_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("rmn_scene_create", "rmn_trace_closest", "rmn_trace_shadow", "rmn_render", "rmn_fxaa",
                 "rmn_compose", "rmn_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    from raym0nade_gb300 import _lib
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"
    assert lib.rmn_version().startswith(b"raym0nade-gb300")


def test_struct_sizes_match_header():
    from raym0nade_gb300 import _lib
    assert ctypes.sizeof(_lib.Material) == 64
    assert ctypes.sizeof(_lib.RenderArgs) == 4 * 17 + 4 * 5 + 8 + 4 * 4
    assert ctypes.sizeof(_lib.Image) == 6 * 8


# ctypes mirror -> C struct of include/rmn.h
ABI_STRUCTS = {"Material": "rmn_material", "SceneDesc": "rmn_scene_desc", "SceneInfo": "rmn_scene_info",
               "RenderArgs": "rmn_render_args", "Image": "rmn_image", "RenderProfile": "rmn_render_profile",
               "BatchItem": "rmn_batch_item", "BatchOptions": "rmn_batch_options", "TuneResult": "rmn_tune_result",
               "Texture": "rmn_texture", "PostArgs": "rmn_post_args", "ImageDesc": "rmn_image_desc"}


def test_ctypes_layouts_match_c_compiler(tmp_path):
    """Every field offset and struct size of the ctypes mirror equals what a
    C compiler makes of include/rmn.h."""
    import shutil
    import subprocess
    from raym0nade_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include "rmn.h"', "int main(void) {"]
    for py, c in ABI_STRUCTS.items():
        lines.append(f'  printf("{py} size %zu\\n", sizeof({c}));')
        for name, _ in getattr(_lib, py)._fields_:
            lines.append(f'  printf("{py} {name} %zu\\n", offsetof({c}, {name}));')
    lines.append("  return 0;\n}")
    src = tmp_path / "abi.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "abi"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    for line in filter(None, out):
        py, name, val = line.split()
        cls = getattr(_lib, py)
        got = ctypes.sizeof(cls) if name == "size" else getattr(cls, name).offset
        assert got == int(val), (py, name, got, val)


def test_c_program_links_and_decodes(lib, tmp_path):
    """A plain C program against include/rmn.h and librmn.so: it decodes a
    committed PNG with rmn_image_load (host work, no GPU) and reports the
    library's error text for a missing file."""
    import shutil
    import subprocess
    from raym0nade_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "use.c"
    src.write_text(r"""
#include <stdio.h>
#include <stdlib.h>
#include "rmn.h"
int main(int argc, char **argv) {
  rmn_image_desc d;
  if (rmn_image_load(argv[1], RMN_IMAGE_PNG, &d, NULL, 0) != RMN_OK) return 1;
  size_t n = (size_t)d.width * d.height * d.channels;
  unsigned char *px = malloc(n);
  if (rmn_image_load(argv[1], RMN_IMAGE_PNG, &d, px, n) != RMN_OK) return 2;
  unsigned long sum = 0;
  for (size_t i = 0; i < n; i++) sum += px[i];
  printf("%d %d %d %lu\n", d.width, d.height, d.channels, sum);
  if (rmn_image_load("/nonexistent.png", RMN_IMAGE_PNG, &d, NULL, 0) != RMN_ERR_INVALID_ARGUMENT) return 3;
  printf("%s\n", rmn_last_error());
  free(px);
  return 0;
}
""")
    exe = tmp_path / "use"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L", libdir, "-lrmn",
                    "-Wl,-rpath," + libdir], check=True)
    png = os.path.join(ROOT, "tests", "golden", "images", "rgb16_paeth.png")
    out = subprocess.run([str(exe), png], check=True, capture_output=True, text=True).stdout.split("\n")
    want = np.load(os.path.join(ROOT, "tests", "golden", "images.npz"))["rgb16_paeth.png"]
    assert out[0].split() == [str(want.shape[1]), str(want.shape[0]), "3", str(int(want.astype(np.int64).sum()))]
    assert "could not read" in out[1]


def test_integration_binding_compiles_against_reference_headers(tmp_path):
    """The reference-side C++ binding (tests/golden/reference_binding.cpp:
    the render_multiThread replacement, the image loaders, the model
    creation) compiles against the reference's own headers (with the
    oracle's glm / assimp / libpng stand-ins) and include/rmn.h."""
    import shutil
    import subprocess
    from oracle import bindings
    ref_inc = os.path.join(bindings.REFERENCE_DIR, "include")
    if not os.path.isdir(ref_inc):
        pytest.skip("the reference checkout is not on this machine")
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = os.path.join(ROOT, "tests", "golden", "reference_binding.cpp")
    import sysconfig
    cmd = [cxx, "-std=c++17", "-fsyntax-only", "-w", "-I", os.path.join(ROOT, "oracle", "shim"), "-I", ref_inc,
           "-I", sysconfig.get_paths()["include"], "-I", os.path.join(ROOT, "include"), str(src)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]


def test_parse_render_args_docs_block():
    from raym0nade_gb300.api import parse_render_args
    block = """0.96718 -0.2 -0.156768
0.16 0 0.987117
-0.1974234 -0.9798 0.032
-16.5 -0.5 -2.25
0.001025 15.0 32.0 200.0
2048 1152
0 12 0.7
output/Bistro"""
    a = parse_render_args(block)
    d = np.array([0.96718, -0.2, -0.156768]); r = np.array([0.16, 0, 0.987117]); u = np.array([-0.1974234, -0.9798, 0.032])
    assert np.allclose(a.position, -16.5 * d - 0.5 * r - 2.25 * u, atol=1e-5)
    assert (a.width, a.height, a.spp, a.threads) == (2048, 1152, 0, 12)
    assert a.accuracy == pytest.approx(0.001025) and a.exposure == 200.0 and a.P_Direct == pytest.approx(0.7)
    assert a.savePath == "output/Bistro"


def test_scene_generators_shapes():
    from raym0nade_gb300 import scenes
    c = scenes.cornell()
    assert c.num_triangles == 36
    s = scenes.random_soup(1000, 1)
    assert s.num_triangles == 1000
    h = scenes.heightfield(33, seed=1, extent=3.0, patch=8)
    assert h.num_triangles == 2 * 32 * 32
    e = scenes.sky_env(64, 32)
    assert e.shape == (32, 64, 3) and e.max() >= 5e4


def test_argument_checks_need_no_gpu(lib):
    """The new entry points refuse bad arguments before any device work."""
    import ctypes as C
    from raym0nade_gb300 import _lib, scenes
    img = _lib.Image()
    rgb = (C.c_float * 12)()
    pa = _lib.PostArgs(2, 2, 1.0, 1.0, 0.0, (C.c_float * 3)())
    # incomplete image, or no rgb
    assert lib.rmn_post_process(C.byref(img), C.byref(pa), 63, rgb, None) == 1
    assert lib.rmn_spatial_clamp(C.byref(img), 2, 2, None) == 1
    assert lib.rmn_filter(C.byref(img), 2, 2, None) == 1
    cnt = C.c_int32(-1)
    assert lib.rmn_export_set(C.byref(img), C.byref(pa), rgb, C.byref(cnt), None) == 1
    info = _lib.ImageDesc()
    assert lib.rmn_scene_texture_get(None, 0, 0, C.byref(info), None, 0) == 1
    # a negative or non-finite CoC, a zero size
    for bad in (_lib.PostArgs(2, 2, 1.0, 1.0, -1.0, (C.c_float * 3)()),
                _lib.PostArgs(2, 2, 1.0, 1.0, float("inf"), (C.c_float * 3)()),
                _lib.PostArgs(0, 2, 1.0, 1.0, 0.0, (C.c_float * 3)())):
        assert lib.rmn_post_process(C.byref(img), C.byref(bad), 63, rgb, None) == 1
    assert b"CoC" in lib.rmn_last_error() or b"size" in lib.rmn_last_error()
    # export table
    assert lib.rmn_export_tag(0) == b"DiffuseColor" and lib.rmn_export_tag(25) is None
    assert lib.rmn_export_options(-1) == -1
    assert lib.rmn_batch_update(None, None, 0, None) == 1 and lib.rmn_batch_update_bytes(None) == 0


def test_texture_scene_checks_need_no_gpu(lib):
    """rmn_scene_create refuses RGB textures (the reference's 4-byte lookups
    read past them) and out-of-range texture indices before uploading."""
    import ctypes as C
    from raym0nade_gb300 import _lib, scenes
    room = scenes.textured_room()

    def create(textures, mat_tex):
        keep = [np.ascontiguousarray(x) for x in (room.positions, room.normals, room.uvs, room.indices,
                                                  room.mesh_first, room.mesh_material, room.materials)]
        p, n, u, i, mf, mm, mat = keep
        tarr = (_lib.Texture * len(textures))(*[_lib.Texture(t.shape[1], t.shape[0], t.shape[2], t.ctypes.data)
                                                for t in textures])
        d = _lib.SceneDesc(p.shape[0], p.ctypes.data, n.ctypes.data, u.ctypes.data, i.shape[0], i.ctypes.data,
                           mm.shape[0], mf.ctypes.data, mm.ctypes.data, mat.shape[0], mat.ctypes.data, 0, 0, None,
                           len(textures), C.cast(tarr, C.c_void_p).value, mat_tex.ctypes.data)
        h = C.c_void_p()
        return lib.rmn_scene_create(C.byref(d), C.byref(h)), textures
    rgb = [np.ascontiguousarray(t[..., :3]) for t in room.textures]
    st, _ = create(rgb, np.ascontiguousarray(room.mat_tex))
    assert st == 4 and b"channels" in lib.rmn_last_error()
    bad = room.mat_tex.copy()
    bad[0, 0] = len(room.textures)
    st, _ = create(list(room.textures), np.ascontiguousarray(bad))
    assert st == 1 and b"out of range" in lib.rmn_last_error()


def _read_png(path):
    """Check every chunk CRC and the header of an 8-bit RGB PNG, then decode
    it with the oracle's reader (Python's zlib, all five filters)."""
    import struct
    import zlib
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xffffffff, typ
        chunks.append((typ, body))
        pos += 12 + n
    assert chunks[0][0] == b"IHDR" and chunks[-1][0] == b"IEND"
    w, h, depth, ctype, comp, filt, inter = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (depth, ctype, comp, filt, inter) == (8, 2, 0, 0, 0)
    raw = zlib.decompress(b"".join(b for t, b in chunks if t == b"IDAT"))
    assert len(raw) == h * (1 + 3 * w)
    from oracle.image_codecs import png_read
    return png_read(path)


@pytest.mark.parametrize("w,h", [(1, 1), (37, 5), (300, 260)])
def test_save_png_bytes_are_the_references(lib, tmp_path, w, h):
    """Photo::save's bytes, static_cast<png_byte>(v * 255), in a PNG any
    reader decodes (adaptive row filters, deflate by the library)."""
    from raym0nade_gb300 import api
    rng = np.random.default_rng(w * h)
    img = rng.random((h, w, 3), dtype=np.float32)
    img[0, 0] = (0.0, 1.0, 0.999)
    path = str(tmp_path / "x.png")
    api.Photo.save(img, path)
    got = _read_png(path)
    want = (img * np.float32(255)).astype(np.uint8)  # truncation, as the reference's cast
    assert np.array_equal(got, want)
    ppm = str(tmp_path / "x.ppm")
    api.Photo.save(img, ppm)
    assert open(ppm, "rb").read().endswith(want.tobytes())
