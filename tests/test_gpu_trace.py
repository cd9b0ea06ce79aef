"""GPU parity of the ray queries and post passes, through the C ABI.

Closest-hit ids and t must be bit-identical to the oracle (which is pinned to
the reference's own BVH::rayHit); barycentrics too (same formula, no fused
multiply-add). Occlusion answers must be identical. FXAA must be
bit-identical; compose + gamma within 2 ulp-ish (rtol 2e-6) since CUDA's
powf/tanhf and glibc's may differ in the last bit.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from raym0nade_gb300 import api, scenes  # noqa: E402
from tests.golden.make_golden import edge_rays, scene_from, tie_soup  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def gpu_closest(model, rays, device_resident=True):
    r = torch.from_numpy(rays).cuda() if device_resident else rays
    return api.split_hits(model.rayHit(r))


@pytest.mark.parametrize("device_resident", [True, False])
def test_closest_matches_oracle_soup(port, device_resident):
    soup = tie_soup(20000, 41)
    rays = edge_rays(200000, 42)
    m = api.Model(soup)
    f, t, b = gpu_closest(m, rays, device_resident)
    pf, pt, pb = port.scene(soup).trace_closest(rays)
    assert np.array_equal(f, pf)
    assert np.array_equal(t, pt)
    hit = pf >= 0
    assert np.array_equal(b[hit], pb[hit])


def test_closest_golden(port):
    z = np.load(os.path.join(GOLDEN, "trace_soup.npz"))
    m = api.Model(scene_from(z))
    f, t, b = gpu_closest(m, z["rays"])
    assert np.array_equal(f, z["face"]) and np.array_equal(t, z["t"])
    hit = f >= 0
    assert np.array_equal(b[hit], z["bary"][hit])
    occ = m.rayHit_test(torch.from_numpy(z["shadow_rays"]).cuda()).cpu().numpy()
    assert np.array_equal(occ, z["occluded"])


@pytest.mark.parametrize("n", [1, 7, 10, 11])
def test_closest_tiny_scenes(port, n):
    s = scenes.random_soup(n, 50 + n)
    rays = edge_rays(4096, 51)
    tgt = s.positions.reshape(-1, 3, 3).mean(1)[np.arange(rays.shape[0]) % n]
    d = tgt - rays[:, 0:3]
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    m = api.Model(s)
    f, t, _ = gpu_closest(m, rays)
    pf, pt, _ = port.scene(s).trace_closest(rays)
    assert np.array_equal(f, pf) and np.array_equal(t, pt)
    assert (pf >= 0).any()


def test_closest_bounded_interval(port):
    s = scenes.random_soup(5000, 61)
    rays = scenes.random_rays(50000, 62)
    rays[:, 3] = np.float32(0.05)
    rays[:, 7] = np.float32(0.4)
    m = api.Model(s)
    f, t, _ = gpu_closest(m, rays)
    pf, pt, _ = port.scene(s).trace_closest(rays)
    assert np.array_equal(f, pf) and np.array_equal(t, pt)


def test_closest_exact_ties_and_zero_distances(port):
    """Every triangle twice (same vertices: every hit an exact tie, the first
    in leaf order wins), rays aimed at centroids, and rays starting on a
    triangle with t_min < 0 (distances of +-0): ids and t bit-identical to
    the oracle, whichever lanes test a leaf's triangles."""
    s = scenes.random_soup(4000, 71)
    s.indices = np.concatenate([s.indices, s.indices[::-1]]).astype(np.int32)
    s.mesh_first = np.array([0, s.indices.shape[0]], np.int32)
    rng = np.random.default_rng(72)
    cen = s.positions[s.indices].mean(1).astype(np.float32)
    n = 60000
    rays = scenes.random_rays(n, 73)
    tgt = cen[rng.integers(0, cen.shape[0], n)]
    d = tgt.astype(np.float64) - rays[:, 0:3]
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    z = n // 4  # origins on a centroid, t_min -1
    rays[:z, 0:3] = tgt[:z]
    rays[:z, 3] = np.float32(-1.0)
    m = api.Model(s)
    f, t, _ = gpu_closest(m, rays)
    pf, pt, _ = port.scene(s).trace_closest(rays)
    assert np.array_equal(f, pf) and np.array_equal(t.view(np.int32), pt.view(np.int32))
    assert (pf >= 0).mean() > 0.9 and (pt[:z] == 0).any()


def test_shadow_matches_oracle(port):
    soup = tie_soup(20000, 43)
    sr = scenes.random_rays(200000, 44, shadow=True)
    sr[:1000, 7] = np.inf
    m = api.Model(soup)
    occ = m.rayHit_test(torch.from_numpy(sr).cuda()).cpu().numpy()
    assert np.array_equal(occ, port.scene(soup).trace_shadow(sr))


def _surface_rays(sc, n, seed, shadow):
    """Rays leaving the surface of a scene: from a random point of a random
    triangle, 1e-3 along its upward normal, into the upper hemisphere;
    shadow rays with aims U(0.1, 50). Many cross the mesh near shared edges."""
    rng = np.random.default_rng(seed)
    P, I = sc.positions.astype(np.float64), sc.indices
    t = rng.integers(0, I.shape[0], n)
    a, b, c = P[I[t, 0]], P[I[t, 1]], P[I[t, 2]]
    u, v = rng.random(n), rng.random(n)
    m = u + v > 1
    u[m], v[m] = 1 - u[m], 1 - v[m]
    p = a + (b - a) * u[:, None] + (c - a) * v[:, None]
    nrm = np.cross(b - a, c - a)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm *= np.sign(nrm[:, 1:2] + 1e-12)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d * np.sign((d * nrm).sum(1, keepdims=True))
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = p + nrm * 1e-3
    r[:, 3] = 1e-4
    r[:, 4:7] = d
    r[:, 7] = np.inf if not shadow else rng.uniform(0.1, 50.0, n)
    return r


def test_heightfield_surface_rays_match_oracle(port):
    """A closed heightfield mesh (every edge shared by two triangles, often
    in different leaves) and rays leaving its surface: closest hits (the
    reference's visit order, warp-cooperative leaves) and occlusion (the
    order-free kernel with pending leaves) identical to the oracle's
    ordered search."""
    hf = scenes.heightfield(500, seed=3)
    m = api.Model(hf)
    cr = _surface_rays(hf, 400_000, 81, False)
    sr = _surface_rays(hf, 400_000, 82, True)
    ps = port.scene(hf)
    f, t, _ = gpu_closest(m, cr)
    pf, pt, _ = ps.trace_closest(cr, threads=os.cpu_count() or 8)
    assert np.array_equal(f, pf) and np.array_equal(t.view(np.int32), pt.view(np.int32))
    occ = m.rayHit_test(torch.from_numpy(sr).cuda()).cpu().numpy()
    ref = ps.trace_shadow(sr, threads=os.cpu_count() or 8)
    assert np.array_equal(occ, ref)
    assert 0.05 < ref.mean() < 0.95 and (pf >= 0).mean() > 0.05


def test_cornell_queries(port):
    c = scenes.cornell()
    rays = scenes.random_rays(100000, 45)
    rays[:, 0:3] = rays[:, 0:3] * 0.98 + 0.01
    m = api.Model(c)
    f, t, _ = gpu_closest(m, rays)
    pf, pt, _ = port.scene(c).trace_closest(rays)
    assert np.array_equal(f, pf) and np.array_equal(t, pt)


def test_full_size_traversal_microbench(port):
    """1M-triangle soup, 4M closest + 4M shadow rays: identical to the oracle."""
    soup = scenes.random_soup(1_000_000, 1)
    rays = scenes.random_rays(4_000_000, 2)
    sr = scenes.random_rays(4_000_000, 3, shadow=True)
    m = api.Model(soup)
    f, t, _ = gpu_closest(m, rays)
    ps = port.scene(soup)
    pf, pt, _ = ps.trace_closest(rays, threads=os.cpu_count() or 8)
    assert np.array_equal(f, pf) and np.array_equal(t, pt)
    occ = m.rayHit_test(torch.from_numpy(sr).cuda()).cpu().numpy()
    assert np.array_equal(occ, ps.trace_shadow(sr, threads=os.cpu_count() or 8))


def test_scene_errors():
    c = scenes.cornell()
    c.indices = c.indices.copy()
    c.indices[3, 1] = 10_000
    with pytest.raises(api.RmnError) as e:
        api.Model(c)
    assert e.value.status == 1 and "out of range" in str(e.value)
    m = scenes.cornell()
    m.mesh_material = m.mesh_material.copy()
    m.mesh_material[2] = 99  # no such material
    with pytest.raises(api.RmnError) as e:
        api.Model(m)
    assert e.value.status == 1


@pytest.mark.parametrize("shape", [(64, 96), (61, 173), (1080, 1920), (7, 5)])
def test_fxaa_bit_exact(port, shape):
    rng = np.random.default_rng(shape[0] * 1000 + shape[1])
    h, w = shape
    img = (rng.random((h, w, 3)) ** 3).astype(np.float32)
    yy, xx = np.mgrid[0:h, 0:w]
    img[(xx * 3 + yy * 2) % 37 < 9] += 0.6
    img = np.clip(img, 0, 1).astype(np.float32)
    out = api.FXAA(torch.from_numpy(img).cuda()).cpu().numpy()
    assert np.array_equal(out, port.fxaa(img))
    out_host = api.FXAA(img)
    assert np.array_equal(out_host, out)


def test_fxaa_golden():
    z = np.load(os.path.join(GOLDEN, "post.npz"))
    out = api.FXAA(torch.from_numpy(z["fxaa_in"]).cuda()).cpu().numpy()
    assert np.array_equal(out, z["fxaa_out"])


def _photo_from_records(rec):
    h, w, _ = rec.shape
    p = api.Photo(w, h, 1.0)
    r = torch.from_numpy(rec.reshape(-1, 40)).cuda()
    p.radiance_Dd.copy_(r[:, 0:4]); p.radiance_Ds.copy_(r[:, 4:8])
    p.radiance_Id.copy_(r[:, 8:12]); p.radiance_Is.copy_(r[:, 12:16])
    g = torch.zeros((h * w, api.GBUFFER_FLOATS), device="cuda")
    g[:, 0:3] = r[:, 16:19]; g[:, 3:6] = r[:, 19:22]; g[:, 6:9] = r[:, 22:25]
    g[:, 9:12] = r[:, 25:28]; g[:, 12:15] = r[:, 28:31]; g[:, 15] = r[:, 31]
    g[:, 16] = r[:, 32]; g[:, 17] = r[:, 33]; g[:, 18] = r[:, 35]; g[:, 19] = r[:, 36]; g[:, 20] = r[:, 37]
    p.Gbuffer.copy_(g)
    return p


def test_compose_matches_oracle(port):
    z = np.load(os.path.join(GOLDEN, "post.npz"))
    p = _photo_from_records(z["records"])
    lin = p.shade(api.Full).cpu().numpy()
    assert np.array_equal(lin, z["linear"])
    disp = p.shade(api.Full | api.GAMMA).cpu().numpy()
    np.testing.assert_allclose(disp, z["display"], rtol=2e-6, atol=1e-7)
    fx = p.shade(api.Full | api.GAMMA | api.DoFXAA).cpu().numpy()
    np.testing.assert_allclose(fx, port.fxaa(disp), rtol=2e-6, atol=1e-7)
