"""Batch configuration through the C ABI: the autotuner (rmn_batch_autotune),
the memory query it caps candidates with (rmn_batch_device_bytes), and the
library's default unit split, which must be a choice of each render alone.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from raym0nade_gb300 import _lib, api, scenes  # noqa: E402

SLOTS, POOLS, LANES, STACKS = {0, 2, 4, 8, 16}, {0, 1 << 20, 1 << 21, 1 << 22, 1 << 23}, {0, 2, 3, 4}, {23, 27}


def _photo_np(ph):
    return [x.cpu().numpy() for x in (ph.radiance_Dd, ph.radiance_Ds, ph.radiance_Id, ph.radiance_Is, ph.Gbuffer)]


def _uneven_items():
    """Four renders of uneven size: Cornell boxes, a heightfield under a sky,
    a triangle soup."""
    cor = api.Model(scenes.cornell())
    hf = scenes.heightfield(48, seed=2, extent=4.8, patch=8)
    hf.env = scenes.sky_env(64, 32, sun_radiance=100.0, sun_diameter_deg=8.0)
    sky = api.Model(hf)
    soup = api.Model(scenes.random_soup(20000, 5))
    skycam = scenes.Camera((0.3, 2.0, -0.8), (0.35, -0.45, 0.82), (0.0, -1.0, 0.0), (-1.0, 0.0, 0.0), 0.02, 96, 64, 24)
    specs = [(cor, scenes.cornell_camera(128, 128, 32), 1), (sky, skycam, 2),
             (cor, scenes.cornell_camera(64, 80, 12, max_depth=6), 3), (soup, scenes.soup_camera(96, 96, 16, 8), 4)]
    return [(m, api.RenderArgs.from_camera(c, seed=s), api.Photo(c.width, c.height)) for m, c, s in specs]


def _free_bytes():
    free, _ = torch.cuda.mem_get_info()
    return free


def test_autotune_returns_a_candidate_and_its_images_match():
    items = _uneven_items()
    free = _free_bytes()
    res = api.autotune(items, pixel_fraction=0.25)
    assert res["slots_per_unit"] in SLOTS and res["pool_workers"] in POOLS and res["lanes"] in LANES
    assert res["stack_entries"] in STACKS and res["ray_order"] in (0, 1)
    # these trees are shallow: both stack builds are admissible, the shallow
    # one is the default and the deeper one is timed once more; then binned
    # ray queues
    assert res["candidates"] >= 3
    assert 0.0 < res["best_ms"] <= res["default_ms"]
    # the choice fits the tuner's memory cap: half of the free device memory
    for m, a, ph in items:
        a.slots_per_unit = res["slots_per_unit"]
    assert api.batch_device_bytes(items, res["pool_workers"], res["lanes"]) <= free // 2
    # a batch built with the tuned settings renders every item exactly as
    # rmn_render does with the same slots per unit
    b = api.Batch(items, use_graph=True, pool_workers=res["pool_workers"], lanes=res["lanes"],
                  stack_entries=res["stack_entries"], ray_order=res["ray_order"])
    b.render()
    torch.cuda.synchronize()
    for m, a, ph in items:
        for x, y in zip(_photo_np(ph), _photo_np(api.render(m, a))):
            assert np.array_equal(x, y, equal_nan=True)


@pytest.mark.parametrize("use_graph", [True, False])
def test_stack_builds_and_ray_order_give_identical_images(use_graph):
    """Both traversal stack builds, with and without binned ray queues, give
    every item exactly its rmn_render images (twice in a row)."""
    items = _uneven_items()
    solo = [_photo_np(api.render(m, a)) for m, a, _ in items]
    for stack in (23, 27):
        for order in (0, 1):
            b = api.Batch(items, use_graph=use_graph, stack_entries=stack, ray_order=order, lanes=2)
            for _ in range(2):
                b.render()
                torch.cuda.synchronize()
                for (m, a, ph), ref in zip(items, solo):
                    for x, y in zip(_photo_np(ph), ref):
                        assert np.array_equal(x, y, equal_nan=True)
    with pytest.raises(api.RmnError) as e:
        api.Batch(items, stack_entries=24)
    assert e.value.status == 1
    with pytest.raises(api.RmnError) as e:
        api.Batch(items, ray_order=2)
    assert e.value.status == 1


def test_device_bytes_counts_units_and_workers():
    items = _uneven_items()[:1]  # 128 x 128 Cornell, 32 spp
    m, a, ph = items[0]
    a.slots_per_unit = 4
    # light-sample slots in units of max(4, 8), path slots in units of 4
    spp_d = int(32 * 0.7)
    units = 128 * 128 * ((spp_d + 7) // 8 + (32 - spp_d + 3) // 4)
    one = api.batch_device_bytes(items, 128, 1)
    two = api.batch_device_bytes(items, 256, 1)
    per_worker = (two - one) / 128
    assert 500 < per_worker < 1200
    assert one == units * 112 + 128 * per_worker
    # the pool never exceeds one worker per unit
    assert api.batch_device_bytes(items, 1 << 23, 1) == units * 112 + units * per_worker


def test_autotune_rejects_an_impossible_budget():
    """A batch whose unit records alone exceed the free device memory: the
    tuner reports RMN_ERR_OUT_OF_MEMORY instead of a configuration."""
    m = api.Model(scenes.cornell())
    cam = scenes.cornell_camera(1024, 1024, 1024)
    a = api.RenderArgs.from_camera(cam, seed=1)
    a.slots_per_unit = 1
    items = [(m, a, api.Photo(8, 8))]
    need = api.batch_device_bytes(items, 4096, 1)
    _lib.load().rmn_release_cached_memory()
    torch.cuda.empty_cache()
    free = _free_bytes()
    filler = None
    if need < free:
        filler = torch.empty(free - need // 2, dtype=torch.uint8, device="cuda")
    with pytest.raises(api.RmnError) as e:
        api.autotune([(m, a, api.Photo(cam.width, cam.height))], pixel_fraction=1.0 / 64)
    assert e.value.status == 3  # RMN_ERR_OUT_OF_MEMORY
    del filler
    torch.cuda.empty_cache()
    with pytest.raises(api.RmnError) as e:
        api.autotune(_uneven_items(), pixel_fraction=0.0)
    assert e.value.status == 1


def test_default_split_depends_on_the_render_alone():
    """The library's default unit split (slots_per_unit = 0) decides the
    float summation order of a pixel's samples, so it must not change with
    the free device memory or the batch around a render: the same render
    with most of the device memory taken, and inside a batch, is
    bit-identical."""
    m = api.Model(scenes.cornell())
    cam = scenes.cornell_camera(512, 512, 256)  # 2^26 sample slots: 33.5 M units of 112 B at 2 slots
    a = api.RenderArgs.from_camera(cam, seed=8)
    ref = _photo_np(api.render(m, a))
    _lib.load().rmn_release_cached_memory()
    torch.cuda.empty_cache()
    free = _free_bytes()
    keep = 12 << 30  # the unit records (3.75 GB) exceed a quarter of what is left
    filler = torch.empty(max(free - keep, 1), dtype=torch.uint8, device="cuda") if free > keep else None
    got = _photo_np(api.render(m, a))
    del filler
    torch.cuda.empty_cache()
    for x, y in zip(got, ref):
        assert np.array_equal(x, y, equal_nan=True)
    other = _uneven_items()
    ph = api.Photo(cam.width, cam.height)
    b = api.Batch([(m, a, ph)] + other, use_graph=True)
    b.render()
    torch.cuda.synchronize()
    for x, y in zip(_photo_np(ph), ref):
        assert np.array_equal(x, y, equal_nan=True)
