"""Binary FBX models through rmn_model_read (raym0nade_gb300.assets.load_model
with a .fbx name) against the oracle's restatement (oracle/fbx_import.py),
against the same room read from OBJ/MTL, and against an independent numpy
statement of the FBX transform chain; malformed files give a status."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import fbx_import
from raym0nade_gb300 import _lib, assets, build
from tests.golden import fbx_files, model_files
from tests.test_assets import same_scene

FORMATS = [(7400, False), (7400, True), (7500, False), (7500, True)]


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def write_fbx(folder, name, models, materials, version=7400, compress=False):
    data = fbx_files.fbx_bytes(fbx_files.scene_nodes(models, materials, version), version, compress)
    with open(folder + name, "wb") as f:
        f.write(data)
    return data


def read_status(folder, name):
    lib = _lib.load()
    h = C.c_void_p()
    st = lib.rmn_model_read(os.fsencode(folder), os.fsencode(name), b"null", C.byref(h))
    if st == 0:
        lib.rmn_model_free(h)
    return st, lib.rmn_last_error().decode(errors="replace")


@pytest.mark.parametrize("version,compress", FORMATS)
def test_fbx_room_matches_obj_room_and_oracle(tmp_path, capfd, version, compress):
    folder = str(tmp_path) + "/"
    exp = model_files.write_room(folder)
    models, materials = fbx_files.room_models(exp)
    write_fbx(folder, "room.fbx", models, materials, version, compress)
    fbx = assets.load_model(folder, "room.fbx", "sky.hdr")
    fbx.check()
    same_scene(fbx, fbx_import.load_model(folder, "room.fbx", "sky.hdr"))
    obj = assets.load_model(folder, "room.obj", "sky.hdr")
    capfd.readouterr()
    # materials in order of first use, no unused ones; meshes in the same order
    assert fbx.material_names == ["DefaultMaterial", "Walls", "Plain", "Glow", "Water", "Leaf", "Odd"]
    assert ([fbx.material_names[i] for i in fbx.mesh_material] ==
            [obj.material_names[i] for i in obj.mesh_material])
    for k in ("positions", "uvs", "indices", "mesh_first"):
        assert np.array_equal(getattr(fbx, k), getattr(obj, k)), k
    # the written normals went through the (identity) normal matrix and were
    # normalised again; the geometric ones are computed alike
    np.testing.assert_allclose(fbx.normals, obj.normals, atol=2e-6)
    for i, name in enumerate(fbx.material_names):
        j = obj.material_names.index(name)
        assert np.array_equal(fbx.materials[i], obj.materials[j]), name
        for slot in range(4):
            a, b = fbx.mat_tex[i, slot], obj.mat_tex[j, slot]
            assert (a < 0) == (b < 0), (name, slot)
            if a >= 0:
                assert np.array_equal(fbx.textures[a], obj.textures[b])
    assert np.array_equal(fbx.env, obj.env)


def _rot(axis, deg):
    a = np.radians(deg)
    c, s = np.cos(a), np.sin(a)
    m = np.eye(4)
    i, j = (axis + 1) % 3, (axis + 2) % 3
    m[i, i], m[i, j], m[j, i], m[j, j] = c, -s, s, c
    return m


def _euler(r, order):
    seq = {0: "xyz", 1: "xzy", 2: "yzx", 3: "yxz", 4: "zxy", 5: "zyx"}[order]
    m = np.eye(4)
    for ch in seq:  # the first axis named is applied first
        ax = "xyz".index(ch)
        m = _rot(ax, r[ax]) @ m
    return m


def _t(v):
    m = np.eye(4)
    m[:3, 3] = v
    return m


def _s(v):
    return np.diag([v[0], v[1], v[2], 1.0])


def _local(props):
    """Local transform from the Properties70 entries, in numpy matrices."""
    p = {e[0]: e[2:] for e in props}
    g = lambda k, d: np.asarray(p.get(k, d), np.float64)  # noqa: E731
    T, R, S = g("Lcl Translation", (0, 0, 0)), g("Lcl Rotation", (0, 0, 0)), g("Lcl Scaling", (1, 1, 1))
    Roff, Rp = g("RotationOffset", (0, 0, 0)), g("RotationPivot", (0, 0, 0))
    Soff, Sp = g("ScalingOffset", (0, 0, 0)), g("ScalingPivot", (0, 0, 0))
    pre, post = g("PreRotation", (0, 0, 0)), g("PostRotation", (0, 0, 0))
    order = int(p.get("RotationOrder", (0,))[0])
    local = (_t(T) @ _t(Roff) @ _t(Rp) @ _euler(pre, 0) @ _euler(R, order) @ np.linalg.inv(_euler(post, 0))
             @ np.linalg.inv(_t(Rp)) @ _t(Soff) @ _t(Sp) @ _s(S) @ np.linalg.inv(_t(Sp)))
    geo = _t(g("GeometricTranslation", (0, 0, 0))) @ _euler(g("GeometricRotation", (0, 0, 0)), 0) @ \
        _s(g("GeometricScaling", (1, 1, 1)))
    return local, geo


@pytest.mark.parametrize("version,compress", FORMATS)
def test_fbx_transforms_layers_and_materials(tmp_path, version, compress):
    folder = str(tmp_path) + "/"
    models, materials = fbx_files.transform_models()
    write_fbx(folder, "t.fbx", models, materials, version, compress)
    sc = assets.load_model(folder, "t.fbx")
    sc.check()
    same_scene(sc, fbx_import.load_model(folder, "t.fbx"))
    parent, child = models
    g = child["geometry"]
    # material index 0 (Red): the triangle (the line with it drops out);
    # index 1 (Blue): the quad and the pentagon
    assert sc.material_names == ["Red", "Blue"] and list(sc.mesh_material) == [0, 1]
    assert list(np.diff(sc.mesh_first)) == [1, 2 + 3]
    pl, _ = _local(parent["transform"])
    cl, cg = _local(child["transform"])
    W = pl @ cl @ cg
    polys = [[0, 1, 2, 3], [4, 5, 6], [0, 2, 4, 6, 8]]
    corner_at = [[0, 1, 2, 3], [4, 5, 6], [7, 8, 9, 10, 11]]  # their corner numbers in PolygonVertexIndex
    order = [polys[1], polys[0], polys[2]]
    corners = [corner_at[1], corner_at[0], corner_at[2]]
    V = np.asarray(g["vertices"], np.float64)
    want_p = np.concatenate([(W @ np.c_[V[p], np.ones(len(p))].T).T[:, :3] for p in order])
    np.testing.assert_allclose(sc.positions, want_p, atol=1e-5)
    nmat = np.linalg.inv(W[:3, :3]).T
    nidx = np.asarray(g["normals"]["index"])
    N = np.asarray(g["normals"]["data"])
    want_n = np.concatenate([(nmat @ N[nidx[p]].T).T for p in order])
    want_n /= np.linalg.norm(want_n, axis=1, keepdims=True)
    # FixInfacingNormals may flip a mesh as a whole (the oracle decides alike)
    for a, b in [(0, 3), (3, 3 + 9)]:
        s = np.sign((sc.normals[a:b] * want_n[a:b]).sum(1))
        assert (s == s[0]).all()
        np.testing.assert_allclose(sc.normals[a:b] * s[0], want_n[a:b], atol=1e-5)
    U = np.asarray(g["uvs"]["data"])
    uidx = np.asarray(g["uvs"]["index"])
    want_uv = np.concatenate([U[uidx[c]] for c in corners])
    np.testing.assert_allclose(sc.uvs, want_uv, atol=1e-7)
    # fans from the first corner
    assert np.array_equal(sc.indices, [[0, 1, 2], [3, 4, 5], [3, 5, 6], [7, 8, 9], [7, 9, 10], [7, 10, 11]])


def test_fbx_texture_slots_and_defaults(tmp_path):
    """Factor and colour properties share a slot, the last texture connected
    wins, FileName stands in for an empty RelativeFilename, a geometry
    without a material gets DefaultMaterial, and one without a material layer
    takes the model's first material."""
    folder = str(tmp_path) + "/"
    model_files.write_room(folder)
    quad = {"vertices": [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], "pvi": [0, 1, 2, ~3]}
    models = [{"name": "a", "geometry": dict(quad), "materials": ["M"]},
              {"name": "b", "geometry": dict(quad)},
              {"name": "c", "geometry": dict(quad), "materials": ["N", "M"]}]
    materials = [{"name": "M", "opacity": 0.5,
                  "textures": [("SpecularFactor", "tex/normal.png"), ("SpecularColor", "tex/checker.png"),
                               ("EmissiveFactor", "tex/glow.dds"), ("Bump", "tex/leaf.dds")]},
                 {"name": "N", "opacity": None, "textures": [("NormalMap", "tex/normal.png", True)]}]
    write_fbx(folder, "s.fbx", models, materials)
    sc = assets.load_model(folder, "s.fbx")
    same_scene(sc, fbx_import.load_model(folder, "s.fbx"))
    assert sc.material_names == ["M", "DefaultMaterial", "N"] and list(sc.mesh_material) == [0, 1, 2]
    checker = assets.load_model(folder, "room.obj")
    w = checker.mat_tex[checker.material_names.index("Walls")]
    assert np.array_equal(sc.textures[sc.mat_tex[0, 1]], checker.textures[w[0]])  # the colour came last
    assert sc.mat_tex[0, 0] == -1 and sc.mat_tex[0, 2] >= 0 and sc.mat_tex[0, 3] == -1
    assert sc.materials[0][11] == 0.0  # opacity 0.5: glass
    assert sc.mat_tex[2, 3] >= 0


def test_fbx_rejects_ascii_and_malformed_files(tmp_path):
    folder = str(tmp_path) + "/"
    with open(folder + "a.fbx", "w") as f:
        f.write("; FBX 7.4.0 project file\nFBXHeaderExtension:  {\n}\n")
    st, msg = read_status(folder, "a.fbx")
    assert st == 4 and "ASCII" in msg
    with open(folder + "b.fbx", "wb") as f:
        f.write(b"Kaydara FBX Binary   \x00")
    assert read_status(folder, "b.fbx")[0] == 1
    assert read_status(folder, "missing.fbx")[0] == 1
    models, materials = fbx_files.transform_models()
    data = write_fbx(folder, "t.fbx", models, materials)
    for cut in (30, len(data) // 2, len(data) - 60):
        with open(folder + "c.fbx", "wb") as f:
            f.write(data[:cut])
        st, msg = read_status(folder, "c.fbx")
        assert st == 1, (cut, msg)
    with pytest.raises(ValueError):
        fbx_import.load_model(folder, "c.fbx")
    # no geometry at all: nothing to render
    write_fbx(folder, "e.fbx", [{"name": "empty"}], [])
    assert read_status(folder, "e.fbx")[0] == 1


@pytest.mark.filterwarnings("ignore::RuntimeWarning")  # the oracle's float32 casts of huge mutated values
def test_fbx_mutated_files_native_matches_oracle(tmp_path):
    """Bit-flipped, truncated and spliced copies of both FBX scenes, raw and
    compressed: the native reader and the oracle agree on every file -- both
    reject it, or both read the same arrays."""
    folder = str(tmp_path) + "/"
    exp = model_files.write_room(folder)
    bases = []
    for version, compress in FORMATS:
        bases.append(fbx_files.fbx_bytes(fbx_files.scene_nodes(*fbx_files.room_models(exp), version), version,
                                         compress))
        bases.append(fbx_files.fbx_bytes(fbx_files.scene_nodes(*fbx_files.transform_models(), version), version,
                                         compress))
    rng = np.random.default_rng(5)
    agreed_ok = agreed_bad = 0
    for it in range(800):
        b = bytearray(bases[it % len(bases)])
        op = rng.integers(0, 3)
        if op == 0:
            for _ in range(int(rng.integers(1, 4))):
                b[int(rng.integers(27, len(b)))] = int(rng.integers(0, 256))
        elif op == 1:
            b = b[:int(rng.integers(27, len(b)))]
        else:
            at = int(rng.integers(27, len(b) - 8))
            b[at:at + 4] = int(rng.integers(0, 1 << 32)).to_bytes(4, "little")
        with open(folder + "m.fbx", "wb") as f:
            f.write(bytes(b))
        try:
            want = fbx_import.load_model(folder, "m.fbx")
        except (ValueError, OSError):  # OSError: a texture file that is not there
            want = None
        try:
            got = assets.load_model(folder, "m.fbx")
        except ValueError:
            got = None
        assert (got is None) == (want is None), it
        if got is None:
            agreed_bad += 1
        else:
            same_scene(got, want)
            agreed_ok += 1
    assert agreed_ok > 10 and agreed_bad > 10
