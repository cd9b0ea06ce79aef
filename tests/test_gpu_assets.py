"""GPU parity of an imported model: Model(model_folder, model_name,
skyMap_name) on an OBJ/MTL room with PNG and DDS textures (diffuse,
specular, normal map, emissive light, alpha cut-out), a glass material and
an HDR sky, through the C ABI, against the oracle on the same imported
arrays (the oracle itself matches the reference built with its own
src/material.cpp on this room: tests/test_assets.py)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from raym0nade_gb300 import api, assets  # noqa: E402
from tests.golden import model_files  # noqa: E402
from tests.golden.make_golden import room_rays  # noqa: E402
from tests.test_gpu_render import gpu_records  # noqa: E402
from tests.test_gpu_textures import compare_textured  # noqa: E402


@pytest.fixture(scope="module")
def room(tmp_path_factory):
    folder = str(tmp_path_factory.mktemp("objroom")) + "/"
    model_files.write_room(folder)
    return folder


def test_imported_queries_match_oracle(port, room):
    sc = assets.load_model(room, "room.obj", "sky.hdr")
    m = api.Model(room, "room.obj", "sky.hdr")
    ps = port.scene(sc)
    rays = room_rays(100000, 81)
    f, t, b = api.split_hits(m.rayHit(torch.from_numpy(rays).cuda()))
    pf, pt, pb = ps.trace_closest(rays)
    assert np.array_equal(f, pf) and np.array_equal(t, pt)
    assert np.array_equal(b[pf >= 0], pb[pf >= 0])
    srays = room_rays(100000, 82, shadow=True)
    occ = m.rayHit_test(torch.from_numpy(srays).cuda()).cpu().numpy()
    assert np.array_equal(occ, ps.trace_shadow(srays))


@pytest.mark.parametrize("sky", ["sky.hdr", "null"])
def test_imported_render_matches_oracle(port, room, sky):
    sc = assets.load_model(room, "room.obj", sky)
    cam = model_files.room_camera(64, 48, 12)
    g, _ = gpu_records(api.Model(room, "room.obj", sky), cam, seed=23)
    o = port.scene(sc).render(cam, seed=23, mode=1)
    compare_textured(g, o, frac=0.95)
    assert api.Model(sc).info()["num_lights"] == 1  # the emissive DDS mesh
