"""Seeded synthetic scenes, rays and cameras for the path-tracing core.

The reference loads FBX scenes through assimp (src/model.cpp:172-215) and
ships none; every workload here is generated from a seed instead:

* ``cornell``      -- unit room, front open, two rotated boxes, ceiling quad
                      light of emission (17, 12, 4); 36 triangles.
* ``random_soup``  -- N triangles with centroids uniform in [0,1]^3 and
                      vertex offsets of lognormal length (traversal workload).
* ``heightfield``  -- an n x n vertex grid with fBm heights, 64x64-cell
                      patches of Lambertian or GGX-conductor material, smooth
                      vertex normals, lit by ``sky_env``.
* ``sky_env``      -- lat-long HDR sky: horizon-to-zenith gradient plus a
                      0.5 degree sun disc of radiance 5e4.

A scene is plain arrays in the layout of ``rmn_scene_desc`` (include/rmn.h):
triangles grouped into meshes, one material per mesh (assimp's
SortByPType output, src/model.cpp:179-183), 16-float constant-texel
materials (see ``material``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

MAT_FLOATS = 16


def material(base=(1.0, 1.0, 1.0), emission=None, roughness=0.8, metallic=None, opacity=1.0, ior=1.0,
             transmitting=(0.0, 0.0, 0.0)) -> np.ndarray:
    """One constant-texel material record (16 float32).

    base      -- diffuse texel, linear RGB (Material::getDiffuseColor).
    emission  -- emissive texel, linear RGB, or None for no emissive texture.
    roughness -- Material::roughness when ``metallic`` is None (no specular
                 texel: metallic 0); otherwise the specular texel's G channel,
                 clamped to >= 1e-3 (Material::getSurfaceData).
    metallic  -- specular texel's B channel (clamped to <= 0.99), or None.
    """
    m = np.zeros(MAT_FLOATS, np.float32)
    m[0:3] = base
    m[3] = 1.0
    if emission is not None:
        m[4:7] = emission
        m[7] = 1.0
    m[8] = roughness
    if metallic is not None:
        m[9] = metallic
        m[10] = 1.0
    m[11] = opacity
    m[12] = ior
    m[13:16] = transmitting
    return m


@dataclass
class Scene:
    positions: np.ndarray            # (nv, 3) float32
    normals: np.ndarray              # (nv, 3) float32
    uvs: np.ndarray                  # (nv, 2) float32
    indices: np.ndarray              # (nt, 3) int32
    mesh_first: np.ndarray           # (nm + 1,) int32
    mesh_material: np.ndarray        # (nm,) int32
    materials: np.ndarray            # (nmat, 16) float32
    env: np.ndarray | None = None    # (h, w, 3) float32, row 0 = zenith
    name: str = "scene"
    # 8-bit RGBA textures, (h, w, 4) uint8 each, row 0 = the image's top row
    # (texture v = 1); mat_tex (nmat, 4) int32: per material the diffuse,
    # specular, emissive and normal-map texture index, -1 for none (the
    # record's constant texel, or none).
    textures: list | None = None
    mat_tex: np.ndarray | None = None

    @property
    def num_triangles(self) -> int:
        return int(self.indices.shape[0])

    def check(self) -> None:
        assert self.positions.dtype == np.float32 and self.positions.ndim == 2 and self.positions.shape[1] == 3
        assert self.normals.shape == self.positions.shape and self.uvs.shape == (self.positions.shape[0], 2)
        assert self.indices.dtype == np.int32 and self.indices.shape[1] == 3
        assert self.mesh_first[0] == 0 and self.mesh_first[-1] == self.indices.shape[0]
        assert self.materials.dtype == np.float32 and self.materials.shape[1] == MAT_FLOATS
        if self.mat_tex is not None:
            n = len(self.textures or [])
            assert self.mat_tex.dtype == np.int32 and self.mat_tex.shape == (self.materials.shape[0], 4)
            assert ((self.mat_tex >= -1) & (self.mat_tex < n)).all()
            for t in self.textures or []:
                assert t.dtype == np.uint8 and t.ndim == 3 and t.shape[2] == 4

    def texture_arrays(self):
        """(dims (n, 3) int32 of width, height, channels; contiguous byte
        arrays; mat_tex) for a C scene description, or Nones."""
        if self.mat_tex is None:
            return None, [], None
        texs = [np.ascontiguousarray(t, np.uint8) for t in self.textures or []]
        dims = np.array([[t.shape[1], t.shape[0], t.shape[2]] for t in texs], np.int32).reshape(-1, 3)
        return dims, texs, np.ascontiguousarray(self.mat_tex, np.int32)


@dataclass
class Camera:
    """RenderArgs (include/render.h:8-15) minus threads/savePath."""
    position: tuple
    direction: tuple
    up: tuple
    right: tuple
    accuracy: float
    width: int
    height: int
    spp: int
    p_direct: float = 0.7
    exposure: float = 1.0
    focus: float = 1.0
    coc: float = 0.0
    max_depth: int = 16

    def packed(self, threads: int = 1) -> np.ndarray:
        """The 24-float RenderArgs record of oracle/port/oracle_api.h."""
        a = np.zeros(24, np.float32)
        a[0:3] = self.position
        a[3:6] = self.direction
        a[6:9] = self.up
        a[9:12] = self.right
        a[12] = self.accuracy
        a[13] = self.focus
        a[14] = self.coc
        a[15] = self.exposure
        a[16] = self.p_direct
        a[17] = self.width
        a[18] = self.height
        a[19] = self.spp
        a[20] = threads
        a[21] = self.max_depth
        return a


def _assemble(meshes, mats, env=None, name="scene") -> Scene:
    """meshes: list of (positions (k*3,3), normals, uvs, material index)."""
    pos, nrm, uv, idx, first, mm = [], [], [], [], [0], []
    nv = 0
    for p, n, u, mat in meshes:
        k = p.shape[0] // 3
        pos.append(p)
        nrm.append(n)
        uv.append(u)
        idx.append(np.arange(nv, nv + 3 * k, dtype=np.int32).reshape(k, 3))
        nv += 3 * k
        first.append(first[-1] + k)
        mm.append(mat)
    s = Scene(np.concatenate(pos).astype(np.float32), np.concatenate(nrm).astype(np.float32),
              np.concatenate(uv).astype(np.float32), np.concatenate(idx), np.asarray(first, np.int32),
              np.asarray(mm, np.int32), np.stack(mats).astype(np.float32), env, name)
    s.check()
    return s


def _quad(a, b, c, d):
    """Two triangles (a,b,c), (a,c,d) with flat normals."""
    p = np.array([a, b, c, a, c, d], np.float32)
    n = np.cross(np.subtract(b, a), np.subtract(c, a)).astype(np.float64)
    n /= np.linalg.norm(n)
    return p, np.tile(n.astype(np.float32), (6, 1))


def _box(cx, cz, sx, sy, sz, angle_deg):
    """Axis box resting on y = 0, rotated about the vertical axis."""
    t = math.radians(angle_deg)
    c, s = math.cos(t), math.sin(t)

    def P(x, y, z):
        x0, z0 = x * sx - sx / 2, z * sz - sz / 2
        return (cx + c * x0 + s * z0, y * sy, cz - s * x0 + c * z0)

    faces = [
        (P(0, 1, 0), P(1, 1, 0), P(1, 1, 1), P(0, 1, 1)),  # top
        (P(0, 0, 0), P(0, 0, 1), P(1, 0, 1), P(1, 0, 0)),  # bottom
        (P(0, 0, 0), P(1, 0, 0), P(1, 1, 0), P(0, 1, 0)),  # front
        (P(1, 0, 1), P(0, 0, 1), P(0, 1, 1), P(1, 1, 1)),  # back
        (P(0, 0, 1), P(0, 0, 0), P(0, 1, 0), P(0, 1, 1)),  # left
        (P(1, 0, 0), P(1, 0, 1), P(1, 1, 1), P(1, 1, 0)),  # right
    ]
    ps, ns = zip(*[_quad(*f) for f in faces])
    return np.concatenate(ps), np.concatenate(ns)


CORNELL_RED = (0.65, 0.05, 0.05)
CORNELL_GREEN = (0.12, 0.45, 0.15)
CORNELL_GREY = (0.73, 0.73, 0.73)
CORNELL_LIGHT = (17.0, 12.0, 4.0)


def cornell(materials: list | None = None, wall_materials=None) -> Scene:
    """Procedural Cornell box, 36 triangles.

    Room [0,1]^3, front (z = 0) open; red wall at x = 1, green at x = 0, grey
    floor, ceiling and back wall; a 0.3^3 box rotated +15 degrees and a
    0.3 x 0.6 x 0.3 box rotated -18 degrees; a 0.25 x 0.25 ceiling light
    1e-3 below the ceiling with emission (17, 12, 4). Materials: 0 grey,
    1 red, 2 green, 3 light, 4 short box, 5 tall box (grey unless
    ``materials`` overrides the list).
    """
    if materials is None:
        materials = [material(CORNELL_GREY), material(CORNELL_RED), material(CORNELL_GREEN),
                     material((0.78, 0.78, 0.78), emission=CORNELL_LIGHT), material(CORNELL_GREY),
                     material(CORNELL_GREY)]
    wm = wall_materials or {"floor": 0, "ceiling": 0, "back": 0, "red": 1, "green": 2}
    meshes = []
    zero2 = lambda k: np.zeros((k, 2), np.float32)
    for key, quad in [
        ("floor", ((0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1))),
        ("ceiling", ((0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0))),
        ("back", ((0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1))),
        ("red", ((1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1))),
        ("green", ((0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0))),
    ]:
        p, n = _quad(*quad)
        meshes.append((p, n, zero2(6), wm[key]))
    for (cx, cz, sx, sy, sz, ang), mat in [((0.65, 0.35, 0.3, 0.3, 0.3, 15.0), 4), ((0.33, 0.62, 0.3, 0.6, 0.3, -18.0), 5)]:
        p, n = _box(cx, cz, sx, sy, sz, ang)
        meshes.append((p, n, zero2(36), mat))
    y = 1.0 - 1e-3
    p, n = _quad((0.375, y, 0.375), (0.625, y, 0.375), (0.625, y, 0.625), (0.375, y, 0.625))
    meshes.append((p, n, zero2(6), 3))
    return _assemble(meshes, materials, name="cornell")


def cornell_glass() -> Scene:
    """The Cornell box with a glass tall box (opacity 0, ior 1.5, roughness
    0.05, faintly blue transmitting colour, which also tints the light inside
    it) and a half-opaque short box (opacity 0.5): the reference's
    transmissive and semi-opaque paths (refraction, media, Fresnel split)."""
    mats = [material(CORNELL_GREY), material(CORNELL_RED), material(CORNELL_GREEN),
            material((0.78, 0.78, 0.78), emission=CORNELL_LIGHT),
            material((0.7, 0.6, 0.3), opacity=0.5, roughness=0.4),
            material((1.0, 1.0, 1.0), roughness=0.05, opacity=0.0, ior=1.5, transmitting=(0.95, 0.98, 1.0))]
    return cornell(mats)


CORNELL16_LIGHT = 5  # material index of the emitter in cornell16


def cornell16_params(seed: int = 11) -> np.ndarray:
    """Parameters of the 16-material Cornell variant, (16, 5) float64 rows
    (base r, g, b, roughness, emission scale): base ~ U[0.1, 0.9]^3,
    roughness ~ U[0.1, 0.8], scale 1; the emitter keeps base 0.78 and
    roughness 0.8."""
    rng = np.random.default_rng(seed)
    p = np.zeros((16, 5))
    p[:, 0:3] = rng.uniform(0.1, 0.9, (16, 3))
    p[:, 3] = rng.uniform(0.1, 0.8, 16)
    p[:, 4] = 1.0
    p[CORNELL16_LIGHT, 0:3] = 0.78
    p[CORNELL16_LIGHT, 3] = 0.8
    return p


def cornell16(params: np.ndarray | None = None) -> Scene:
    """The Cornell box with 16 materials: floor 0, ceiling 1, back wall 2,
    right wall 3, left wall 4, light 5 (emission (17, 12, 4) times its scale),
    short box top 6, front and bottom 7, back 8, left 9, right 10, tall box
    11-15 likewise. ``params`` as cornell16_params (default seed 11); every
    material is a constant texel without a specular texel (metallic 0)."""
    p = cornell16_params() if params is None else np.asarray(params, np.float64)
    mats = []
    for i in range(16):
        em = tuple(np.asarray(CORNELL_LIGHT) * p[i, 4]) if i == CORNELL16_LIGHT else None
        mats.append(material(tuple(p[i, 0:3]), emission=em, roughness=float(p[i, 3])))
    meshes = []
    zero2 = lambda k: np.zeros((k, 2), np.float32)
    for mat, quad in enumerate([
        ((0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)),
        ((0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)),
        ((0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)),
        ((1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1)),
        ((0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0)),
    ]):
        q, n = _quad(*quad)
        meshes.append((q, n, zero2(6), mat))
    y = 1.0 - 1e-3
    q, n = _quad((0.375, y, 0.375), (0.625, y, 0.375), (0.625, y, 0.625), (0.375, y, 0.625))
    meshes.append((q, n, zero2(6), CORNELL16_LIGHT))
    for first, box in [(6, (0.65, 0.35, 0.3, 0.3, 0.3, 15.0)), (11, (0.33, 0.62, 0.3, 0.6, 0.3, -18.0))]:
        q, n = _box(*box)
        # faces of _box: top, bottom, front, back, left, right (two triangles each)
        for f, mat in enumerate([first, first + 1, first + 1, first + 2, first + 3, first + 4]):
            meshes.append((q[6 * f:6 * f + 6], n[6 * f:6 * f + 6], zero2(6), mat))
    return _assemble(meshes, mats, name="cornell16")


def cornell_camera(width=256, height=256, spp=64, max_depth=16, p_direct=0.7) -> Camera:
    """Camera at (0.5, 0.5, -1.4) looking +z; 40 degree field of view across
    ``width`` pixels (accuracy = tan(20 deg) / (width / 2)); image rows run
    downwards, so ``up`` is -y, and ``right`` is -x looking along +z."""
    return Camera((0.5, 0.5, -1.4), (0.0, 0.0, 1.0), (0.0, -1.0, 0.0), (-1.0, 0.0, 0.0),
                  math.tan(math.radians(20.0)) / (width / 2.0), width, height, spp, p_direct, max_depth=max_depth)


def random_soup(n: int, seed: int = 1) -> Scene:
    """n triangles, centroids ~ U[0,1]^3, vertex offsets L*u with u uniform on
    the sphere and L ~ lognormal(ln 0.005, 0.5), re-centred on the centroid."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 1, 3))
    u = rng.standard_normal((n, 3, 3))
    u /= np.linalg.norm(u, axis=2, keepdims=True)
    L = rng.lognormal(math.log(0.005), 0.5, (n, 3, 1))
    off = u * L
    off -= off.mean(axis=1, keepdims=True)
    p = (c + off).astype(np.float32).reshape(-1, 3)
    nrm = np.cross(off[:, 1] - off[:, 0], off[:, 2] - off[:, 0])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    nrm = np.repeat(nrm, 3, axis=0).astype(np.float32)
    return _assemble([(p, nrm, np.zeros((3 * n, 2), np.float32), 0)], [material(CORNELL_GREY)], name=f"soup{n}")


def random_rays(n: int, seed: int = 2, shadow: bool = False) -> np.ndarray:
    """n rays as 8 float32 each: origin, t_min (1e-4), direction, t_max.
    Origins ~ U[0,1]^3, directions uniform on the sphere; t_max = inf, or for
    shadow rays an aim depth ~ U(0, sqrt 3)."""
    rng = np.random.default_rng(seed)
    r = np.empty((n, 8), np.float32)
    r[:, 0:3] = rng.random((n, 3))
    r[:, 3] = np.float32(1e-4)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 4:7] = d
    r[:, 7] = rng.uniform(0.0, math.sqrt(3.0), n) if shadow else np.inf
    return r


def _value_noise(n, octaves, seed, base_cells=4):
    """fBm of seeded value noise on an n x n grid over [0,1]^2 (gain 0.5,
    lacunarity 2, smoothstep interpolation), normalised to [0,1]."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, n)
    h = np.zeros((n, n))
    amp, cells, total = 1.0, base_cells, 0.0
    for _ in range(octaves):
        lat = rng.random((cells + 1, cells + 1))
        g = x * cells
        i = np.minimum(g.astype(np.int64), cells - 1)
        f = g - i
        f = f * f * (3 - 2 * f)
        a = lat[i][:, i] * (1 - f)[None, :] + lat[i][:, i + 1] * f[None, :]
        b = lat[i + 1][:, i] * (1 - f)[None, :] + lat[i + 1][:, i + 1] * f[None, :]
        h += amp * (a * (1 - f)[:, None] + b * f[:, None])
        total += amp
        amp *= 0.5
        cells *= 2
    return h / total


def heightfield(n: int = 2048, seed: int = 3, extent: float = 200.0, patch: int = 64) -> Scene:
    """n x n vertex grid over [0, extent]^2 in x/z, 2 (n-1)^2 triangles.

    Height = extent * 0.1 * fBm (6 octaves). Cells are grouped into
    patch x patch meshes, each either Lambertian (albedo U[0.2,0.8]^3) or a
    GGX conductor (metallic texel 0.99, roughness U[0.05,0.6], tint
    U[0.5,1]^3), 50/50 by seed. Smooth vertex normals from the height
    gradient; uv = (x, z) / extent.

    The extent keeps cells ~0.1 wide: the reference's absolute thresholds
    (the 1e-4 degenerate-triangle test, src/geometry.cpp:70, and the 1e-2
    smooth-normal area cut-off, src/model.cpp:250) then behave as intended
    (no grazing pass-through, smooth normals on).
    """
    rng = np.random.default_rng(seed)
    hgt = _value_noise(n, 6, seed) * (0.1 * extent)
    xs = np.linspace(0.0, extent, n)
    X, Z = np.meshgrid(xs, xs)  # row = z index, col = x index
    P = np.stack([X, hgt, Z], axis=-1)
    dx = np.gradient(hgt, xs, axis=1)
    dz = np.gradient(hgt, xs, axis=0)
    N = np.stack([-dx, np.ones_like(dx), -dz], axis=-1)
    N /= np.linalg.norm(N, axis=-1, keepdims=True)
    UV = np.stack([X / extent, Z / extent], axis=-1)
    cells = n - 1
    npatch = (cells + patch - 1) // patch
    mats = []
    for _ in range(npatch * npatch):
        if rng.random() < 0.5:
            mats.append(material(tuple(rng.uniform(0.2, 0.8, 3))))
        else:
            mats.append(material(tuple(rng.uniform(0.5, 1.0, 3)), roughness=float(rng.uniform(0.05, 0.6)),
                                 metallic=0.99))
    vid = np.arange(n * n, dtype=np.int64).reshape(n, n)
    pos = P.reshape(-1, 3).astype(np.float32)
    nrm = N.reshape(-1, 3).astype(np.float32)
    uv = UV.reshape(-1, 2).astype(np.float32)
    idx_parts, first, mm = [], [0], []
    for pz in range(npatch):
        for px in range(npatch):
            z0, z1 = pz * patch, min(cells, (pz + 1) * patch)
            x0, x1 = px * patch, min(cells, (px + 1) * patch)
            a = vid[z0:z1, x0:x1]
            b = vid[z0:z1, x0 + 1:x1 + 1]
            c = vid[z0 + 1:z1 + 1, x0:x1]
            d = vid[z0 + 1:z1 + 1, x0 + 1:x1 + 1]
            t1 = np.stack([a, c, b], -1).reshape(-1, 3)
            t2 = np.stack([b, c, d], -1).reshape(-1, 3)
            tri = np.concatenate([t1, t2])
            idx_parts.append(tri)
            first.append(first[-1] + tri.shape[0])
            mm.append(pz * npatch + px)
    s = Scene(pos, nrm, uv, np.concatenate(idx_parts).astype(np.int32), np.asarray(first, np.int32),
              np.asarray(mm, np.int32), np.stack(mats).astype(np.float32), None, f"heightfield{n}")
    s.check()
    return s


def sky_env(width: int = 2048, height: int = 1024, sun_radiance: float = 5e4, sun_diameter_deg: float = 0.5,
            sun_dir=(0.4, 0.55, 0.3)) -> np.ndarray:
    """Lat-long sky in the reference's SkyBox convention (src/component.cpp:
    120-140): texel (u, v) looks along (-sin p sin t, cos p, sin p cos t)
    with p = pi (v + 0.5) / h from the zenith and t = 2 pi (u + 0.5) / w.
    Zenith blue to horizon white above, dark ground below, plus a sun disc."""
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    phi = np.pi * v[:, None]
    th = 2.0 * np.pi * u[None, :]
    D = np.stack([-np.sin(phi) * np.sin(th), np.cos(phi) * np.ones_like(th), np.sin(phi) * np.cos(th)], -1)
    up = np.clip(D[..., 1], 0.0, 1.0)[..., None]
    zenith = np.array([0.25, 0.45, 0.95])
    horizon = np.array([0.9, 0.92, 1.0])
    ground = np.array([0.12, 0.1, 0.08])
    sky = np.where(D[..., 1:2] >= 0, horizon + (zenith - horizon) * up ** 0.5, ground)
    s = np.asarray(sun_dir, np.float64)
    s /= np.linalg.norm(s)
    cosang = D @ s
    sky = sky + (cosang >= math.cos(math.radians(sun_diameter_deg / 2.0)))[..., None] * sun_radiance
    return sky.astype(np.float32)


def heightfield_camera(width=1920, height=1080, spp=256, extent=200.0) -> Camera:
    """Oblique view over the terrain from above one corner, 60 degree field
    of view across the image width."""
    eye = np.array([0.15 * extent, 0.3 * extent, -0.05 * extent])
    tgt = np.array([0.55 * extent, 0.02 * extent, 0.6 * extent])
    f = tgt - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, [0.0, 1.0, 0.0])
    r /= np.linalg.norm(r)
    up_img = np.cross(f, r)  # image rows run downwards
    up_img /= np.linalg.norm(up_img)
    acc = math.tan(math.radians(30.0)) / (width / 2.0)
    return Camera(tuple(eye), tuple(f), tuple(up_img), tuple(r), acc, width, height, spp, max_depth=16)


def _tex_material(roughness=0.8, opacity=1.0, ior=1.0, transmitting=(0.0, 0.0, 0.0)) -> np.ndarray:
    """A material record whose colour slots all come from textures (or their
    defaults: white diffuse, no emission, roughness from the record)."""
    m = material(roughness=roughness, opacity=opacity, ior=ior, transmitting=transmitting)
    m[3] = 0.0
    return m


def _rgba(rgb, alpha=None) -> np.ndarray:
    rgb = np.clip(np.rint(np.asarray(rgb) * 255.0), 0, 255).astype(np.uint8)
    a = np.full(rgb.shape[:2] + (1,), 255, np.uint8) if alpha is None else \
        np.clip(np.rint(np.asarray(alpha) * 255.0), 0, 255).astype(np.uint8)[..., None]
    return np.concatenate([rgb, a], -1)


def texture_checker(w, h, cells, seed) -> np.ndarray:
    """RGBA8 checkerboard of two seeded colours with per-texel noise."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.15, 0.95, (2, 3))
    y, x = np.mgrid[0:h, 0:w]
    k = ((x * cells // w) + (y * cells // h)) % 2
    rgb = c[k] * rng.uniform(0.85, 1.0, (h, w, 1))
    return _rgba(rgb)


def texture_normals(w, h, seed, amp=0.35) -> np.ndarray:
    """RGBA8 tangent-space normal map (n * 0.5 + 0.5) of a sum of sines."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w] / np.array([h, w])[:, None, None]
    gx = np.zeros((h, w))
    gy = np.zeros((h, w))
    for _ in range(3):
        fx, fy = rng.integers(1, 6, 2)
        ph = rng.uniform(0, 2 * np.pi)
        arg = 2 * np.pi * (fx * x + fy * y) + ph
        gx += amp * fx * np.cos(arg) / 3
        gy += amp * fy * np.cos(arg) / 3
    n = np.stack([-gx, -gy, np.ones_like(gx)], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return _rgba(n * 0.5 + 0.5)


def texture_surface(w, h, seed) -> np.ndarray:
    """RGBA8 specular texture: G roughness in [0.05, 0.9] in smooth bands,
    B metallic 0 or 0.8 in blocks (Material::getSurfaceData's channels)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    rough = 0.05 + 0.85 * (0.5 + 0.5 * np.sin(2 * np.pi * (x / w * 2 + y / h) + rng.uniform(0, 6)))
    metal = np.where(((x * 4 // w) + (y * 4 // h)) % 3 == 0, 0.8, 0.0)
    return _rgba(np.stack([np.zeros_like(rough), rough, metal], -1))


def texture_cutout(w, h, seed, holes=5) -> np.ndarray:
    """RGBA8 leaf-like cutout: seeded colour, alpha 0 inside ``holes`` discs
    (the alpha test cuts them away) and 0.5 in a ring around each."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w] + 0.5
    alpha = np.ones((h, w))
    for _ in range(holes):
        cx, cy = rng.uniform(0, w), rng.uniform(0, h)
        r = rng.uniform(0.08, 0.2) * w
        d = np.hypot(x - cx, y - cy)
        alpha = np.where(d < 1.3 * r, np.minimum(alpha, 0.5), alpha)
        alpha = np.where(d < r, 0.0, alpha)
    rgb = rng.uniform(0.2, 0.8, 3) * rng.uniform(0.8, 1.0, (h, w, 1))
    return _rgba(rgb, alpha)


def texture_emissive(w, h, seed) -> np.ndarray:
    """RGBA8 emissive stripes of seeded colours."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.3, 1.0, (4, 3))
    x = np.arange(w)
    rgb = np.broadcast_to(c[(x * 4 // w) % 4][None], (h, w, 3))
    return _rgba(rgb)


def textured_room(seed: int = 5, sky: bool = True) -> Scene:
    """A room open to the sky exercising the reference's texture layer
    (src/material.cpp, src/model.cpp:217-330):

    * floor, 4 x 6, uvs tiled over [-3, 3] x [0, 9] (wrap-around): diffuse
      checker 128x128, specular texture 64x64, normal map 64x64;
    * back wall: diffuse 96x80 (non-power-of-two mip chain), normal map;
    * left wall: no texture (white diffuse), roughness 0.6;
    * right-hand emissive panel with a 32x16 striped emissive texture (a
      light object averaged over its 8x8 grid);
    * an alpha-tested fence (cutout discs) across the room, and a stack of
      ten cutout layers 1 cm apart whose holes line up, past the eight
      retries of Model::rayHit;
    * lit by a 64x32 sky without sun (``sky``), else by the panel alone
      (light-object sampling).
    """
    rng = np.random.default_rng(seed)
    texs = [texture_checker(128, 128, 8, seed + 1), texture_surface(64, 64, seed + 2),
            texture_normals(64, 64, seed + 3), texture_checker(96, 80, 6, seed + 4),
            texture_normals(32, 32, seed + 5, amp=0.6), texture_emissive(32, 16, seed + 6),
            texture_cutout(64, 64, seed + 7)]
    stack = np.zeros((16, 16, 4), np.uint8)
    stack[..., :3] = np.array([200, 120, 60], np.uint8)
    stack[..., 3] = 255
    stack[4:12, 4:12, 3] = 0
    texs.append(stack)
    mats = [_tex_material(0.8), _tex_material(0.7), _tex_material(0.6), _tex_material(0.8),
            _tex_material(0.5), _tex_material(0.7)]
    mat_tex = np.array([[0, 1, -1, 2],     # floor
                        [3, -1, -1, 4],    # back wall
                        [-1, -1, -1, -1],  # left wall
                        [-1, -1, 5, -1],   # emissive panel
                        [6, -1, -1, -1],   # fence
                        [7, -1, -1, -1]],  # stacked layers
                       np.int32)
    meshes = []

    def quad(a, b, c, d, uv, mat):
        q, n = _quad(a, b, c, d)
        ua, ub, uc, ud = uv
        meshes.append((q, n, np.array([ua, ub, uc, ua, uc, ud], np.float32), mat))

    quad((-2, 0, 0), (-2, 0, 6), (2, 0, 6), (2, 0, 0), [(-3, 0), (-3, 9), (3, 9), (3, 0)], 0)
    quad((-2, 0, 6), (-2, 3, 6), (2, 3, 6), (2, 0, 6), [(0, 0), (0, 1), (1, 1), (1, 0)], 1)
    quad((-2, 0, 0), (-2, 3, 0), (-2, 3, 6), (-2, 0, 6), [(0, 0), (0, 1), (1, 1), (1, 0)], 2)
    quad((1.9, 0.5, 2), (1.9, 0.5, 4), (1.9, 2.0, 4), (1.9, 2.0, 2), [(0, 0), (1, 0), (1, 1), (0, 1)], 3)
    quad((-1.5, 0, 2.5), (-1.5, 1.5, 2.5), (0.5, 1.5, 2.5), (0.5, 0, 2.5), [(0, 0), (0, 1.5), (2, 1.5), (2, 0)], 4)
    jitter = rng.uniform(-1e-3, 1e-3, 10)
    for k in range(10):
        z = 1.0 + 0.01 * k + jitter[k] * 0.1
        quad((0.6, 0.2, z), (0.6, 0.6, z), (1.0, 0.6, z), (1.0, 0.2, z), [(0, 0), (0, 1), (1, 1), (1, 0)], 5)
    sc = _assemble(meshes, mats, env=sky_env(64, 32, sun_radiance=0.0) if sky else None, name="textured_room")
    sc.textures = texs
    sc.mat_tex = mat_tex
    sc.check()
    return sc


def textured_camera(width=96, height=64, spp=16, max_depth=16, p_direct=0.7) -> Camera:
    """Inside the room at (0.3, 0.9, -0.4) looking at (0.2, 0.5, 4) across the
    floor, 70 degree field of view across the width."""
    eye = np.array([0.3, 0.9, -0.4])
    f = np.array([0.2, 0.5, 4.0]) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, [0.0, 1.0, 0.0])
    r /= np.linalg.norm(r)
    up_img = np.cross(f, r)
    up_img /= np.linalg.norm(up_img)
    acc = math.tan(math.radians(35.0)) / (width / 2.0)
    return Camera(tuple(eye), tuple(f), tuple(up_img), tuple(r), acc, width, height, spp, p_direct,
                  max_depth=max_depth)


@dataclass
class Instance:
    scene: Scene
    camera: Camera
    seed: int


def soup_camera(width, height, spp, max_depth) -> Camera:
    """Outside the unit cube, looking at its centre along +z; 45 degree view."""
    acc = math.tan(math.radians(22.5)) / (width / 2.0)
    return Camera((0.5, 0.5, -1.2), (0.0, 0.0, 1.0), (0.0, -1.0, 0.0), (-1.0, 0.0, 0.0), acc, width, height, spp,
                  max_depth=max_depth)


def batch_instances(count: int = 64, seed: int = 7, env_width: int = 1024, env_height: int = 512,
                    max_tris: int = 2_000_000) -> list:
    """The batching workload: ``count`` scene instances, each chosen by seed
    as a random soup or a heightfield with log-uniform triangle count in
    [1e3, max_tris], a square image of side U[128, 1024], spp log-uniform in
    [16, 256] and max depth U{4..16}, all lit by the synthetic sky."""
    out = []
    env = sky_env(env_width, env_height)
    for i in range(count):
        rng = np.random.default_rng(seed * 100003 + i)
        ntris = int(math.exp(rng.uniform(math.log(1e3), math.log(max_tris))))
        side = int(rng.uniform(128, 1025))
        spp = int(round(math.exp(rng.uniform(math.log(16), math.log(256)))))
        depth = int(rng.integers(4, 17))
        if rng.random() < 0.5:
            s = random_soup(ntris, seed=int(rng.integers(1 << 30)))
            cam = soup_camera(side, side, spp, depth)
        else:
            n = max(3, int(round(math.sqrt(ntris / 2.0))) + 1)
            s = heightfield(n, seed=int(rng.integers(1 << 30)), extent=200.0, patch=64)
            c = heightfield_camera(side, side, spp, extent=200.0)
            c.max_depth = depth
            cam = c
        s.env = env
        out.append(Instance(s, cam, seed * 1000 + i))
    return out
