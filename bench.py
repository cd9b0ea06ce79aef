#!/usr/bin/env python3
"""Headline benchmark: Mpaths/s of the batched persistent renderer.

Workload (default ``batch64``): 64 scene instances chosen by seed -- a random
triangle soup or an fBm heightfield, triangle counts log-uniform in
[1e3, 2e6], square images of side U[128, 1024], spp log-uniform in
[16, 256], max depth U{4..16}, lit by a synthetic lat-long sky
(raym0nade_gb300.scenes.batch_instances). A step renders every instance once.

Arms measured on the GPU, each over the same step:
* batched -- one rmn_batch (all 64 renders in one primary + one persistent
  path launch) replayed from a captured CUDA graph: the headline ``value``;
* plain   -- 64 separate rmn_render launches on the same device buffers;
* e2e     -- the call a user of the reference makes, per instance: rmn_render
  into host (pinned) buffers plus rmn_compose to a display image with gamma
  and FXAA, host<->device copies inside the timed region.
Both GPU arms render identical images (same counter-based streams), so they
are compared at equal rel-MSE by construction.

``--impl reference`` times the reference's CPU path instead: the reference
compiled here (oracle/_ref) when present, else the oracle's restatement, on
all host cores, on a fixed pixel sample of every instance.

Timing: W untimed warm-up steps; K steps bracketed by a barrier and
torch.cuda.synchronize(), each step timed with CUDA events on the rendering
stream; a 256 MiB buffer is overwritten between steps (L2 flush) and the
scene data (> 1 GB) exceeds L2. With torchrun, every rank renders its own 64
instances (weak scaling) and the maximum time over ranks is reported.
"""
from __future__ import annotations

import argparse
import contextlib
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpaths/s at rel-MSE≤1e-3 (batched vs per-scene launch); adjoint/forward time"
UNIT = "Mpaths/s"
FALLBACK_HBM_GBS = 6800.0
# DRAM and L2 bytes (read + write) of the traversal launches (closest queue:
# qtrace_kernel, shadow queue: qocc_kernel) of one batch64 render at the
# launch configurations given beside them, summed from ncu captures (metrics
# dram__bytes_read.sum, dram__bytes_write.sum, lts__t_bytes.sum) of
#   python bench.py --profile-case batch --slots 2 --pool 8388608 --lanes L --stack S
# (ncu cannot run inside the timed region). The line takes the capture of
# the timed configuration, and says so, or else the first and says that.
BATCH64_TRAVERSAL_BYTES = [
    {"config": {"slots_per_unit": 2, "pool_workers": 1 << 23, "lanes": 3, "stack_entries": 23, "ray_order": 0},
     "dram": 161.6e9, "l2": 2256.7e9},
    {"config": {"slots_per_unit": 2, "pool_workers": 1 << 23, "lanes": 4, "stack_entries": 23, "ray_order": 0},
     "dram": 147.6e9, "l2": 2235.1e9},
]


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def l2_copy_gbs(stream):
    """Bytes moved per second (read + write) by a device copy of a 24 MiB
    buffer into another, both resident in the 129 MB L2, repeated: a
    reference figure for L2 bandwidth on this GPU (measured here; there is
    no published number)."""
    import torch
    a = torch.empty(24 << 20, dtype=torch.uint8, device="cuda")
    b = torch.empty_like(a)
    with torch.cuda.stream(stream):
        for _ in range(20):
            b.copy_(a)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(200):
            b.copy_(a)
        e1.record(stream)
    e1.synchronize()
    return 2.0 * a.numel() * 200 / (e0.elapsed_time(e1) / 1e3) / 1e9


def instance_paths(inst):
    c = inst.camera
    return c.width * c.height * c.spp


def workload(name, rank):
    from raym0nade_gb300 import scenes
    if name == "batch64":
        return scenes.batch_instances(64, seed=7 + 1000 * rank), "batch64: 64 seeded instances (soup or heightfield, " \
            "1e3-2e6 tris log-uniform, 128^2-1024^2, 16-256 spp, depth 4-16, synthetic sky 1024x512)"
    if name == "cornell":
        return [scenes.Instance(scenes.cornell(), scenes.cornell_camera(256, 256, 64, max_depth=16), 1 + rank)], \
            "cornell: Cornell box 36 tris, 256x256, 64 spp, max depth 16"
    if name == "heightfield":
        s = scenes.heightfield(2048, seed=3)
        s.env = scenes.sky_env(2048, 1024)
        return [scenes.Instance(s, scenes.heightfield_camera(1920, 1080, 256), 1 + rank)], \
            "heightfield: 2048^2 grid (8,380,418 tris), sky 2048x1024, 1920x1080, 256 spp, max depth 16"
    raise SystemExit(f"unknown workload {name}")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index=0):
        self.index = index
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except Exception:
                self.proc.kill()
        sm, mx, reasons = [], [], set()
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) != len(self.FIELDS):
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for name, v in zip(self.NAMES, p[2:]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        return rank, world, dist
    return 0, 1, None


def max_over_ranks(x, dist, device="cpu"):
    """The largest of every rank's x (the job's time is its slowest rank's)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(paths_per_rank, world, seconds):
    """Whole-job Mpaths/s: every rank renders paths_per_rank paths (weak
    scaling) and the job takes the slowest rank's time."""
    return paths_per_rank * world / seconds / 1e6


# CPU sample of every instance: one pixel drawn uniformly (seeded) from each
# cell of a CPU_GRID x CPU_GRID grid laid over the whole image, so the sample
# spans sky-miss and hit regions in proportion; the same pixels in both the
# reference arm and the GPU line's cpu_baseline.
CPU_GRID = 48


def cpu_sample_pixels(inst, grid=CPU_GRID):
    """Row-major pixel indices of the stratified sample of one instance."""
    c = inst.camera
    gx, gy = min(grid, c.width), min(grid, c.height)
    rng = np.random.default_rng(1_000_003 * (inst.seed + 1) + c.width * 7919 + c.height)
    xe = np.linspace(0, c.width, gx + 1).astype(np.int64)
    ye = np.linspace(0, c.height, gy + 1).astype(np.int64)
    xs = xe[:-1] + (rng.random(gx) * (xe[1:] - xe[:-1])).astype(np.int64)
    ys = ye[:-1, None] + (rng.random((gy, gx)) * (ye[1:] - ye[:-1])[:, None]).astype(np.int64)
    return (ys * c.width + xs[None, :]).ravel()


def cpu_sample_render(scs, insts, threads):
    """Render the stratified pixel sample of every instance with the CPU
    library's scenes `scs` (reference mt19937 stream, per-pixel seeds);
    returns (paths, seconds)."""
    paths, secs = 0, 0.0
    for sc, inst in zip(scs, insts):
        px = cpu_sample_pixels(inst)
        t = time.perf_counter()
        sc.render_pixels(inst.camera, inst.seed, px, mode=0, threads=threads)
        secs += time.perf_counter() - t
        paths += px.size * inst.camera.spp
    return paths, secs


@contextlib.contextmanager
def native_stdout_to_stderr():
    """Sends what native code writes to stdout (the reference's BVH::build
    prints the size of every tree it builds) to stderr for the duration, so
    that stdout carries the JSON line alone."""
    sys.stdout.flush()
    saved = os.dup(1)
    os.dup2(2, 1)
    try:
        yield
    finally:
        try:
            ctypes.CDLL(None).fflush(None)
        except (OSError, AttributeError):
            pass
        os.dup2(saved, 1)
        os.close(saved)


def cpu_baseline(insts):
    from oracle import bindings
    if not os.path.exists(bindings.PORT_SO):
        bindings.build(with_reference=False)
    kind = "reference" if bindings.have_ref() else "port"
    lib = bindings.OracleLib("ref" if kind == "reference" else "port")
    threads = os.cpu_count() or 8
    with native_stdout_to_stderr():
        scs = [lib.scene(i.scene) for i in insts]
    paths, secs = cpu_sample_render(scs, insts, threads)
    npx = sum(cpu_sample_pixels(i).size for i in insts)
    return {"value": paths / secs / 1e6, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"{npx} pixels: in each of the {len(insts)} instances one seeded uniform pixel per cell of a "
                      f"{CPU_GRID}x{CPU_GRID} grid over the whole image, at the instance's own spp and depth "
                      f"({paths} paths, {secs:.1f} s, reference mt19937 stream)"}, scs


def workload_config(insts, desc, world):
    """The workload's `config` object, identical in both arms."""
    return {"workload": desc, "instances": len(insts),
            "triangles": int(sum(i.scene.num_triangles for i in insts)),
            "pixels": int(sum(i.camera.width * i.camera.height for i in insts)),
            "paths_per_step": int(sum(instance_paths(i) for i in insts)), "parallelism": f"replicas x{world}",
            "l2": "scene data > L2 (129 MB), and a 256 MiB buffer is overwritten between GPU steps"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    insts, desc = workload(args.workload, 0)
    base, scs = cpu_baseline(insts)
    vals, secs = [], []
    for step in range(args.warmup + args.steps):
        p, s = cpu_sample_render(scs, insts, base["cores"])
        if step >= args.warmup:
            vals.append(p / s / 1e6)
            secs.append(s)
    value = float(np.mean(vals))
    base["value"] = value
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(secs)), "higher_is_better": True,
           "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scenes; no dataset)",
           "config": workload_config(insts, desc, world), "cpu_baseline": base,
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def adjoint_timing(args, stream, flush, barrier):
    """Adjoint / forward time on the 16-material Cornell box: 512x512, 32 spp,
    max depth 16; dL/dI of the L2 loss to a target rendered at parameters
    perturbed by up to +-10%. Both passes on device buffers, timed with CUDA
    events on the stream after W warm-ups, L2 flushed before each."""
    import numpy as np
    import torch
    from raym0nade_gb300 import api, scenes
    p0 = scenes.cornell16_params()
    rng = np.random.default_rng(5)
    pt = p0.copy()
    pt[:, 0:4] *= rng.uniform(0.9, 1.1, (16, 4))
    pt[:, 4] *= 1.1
    w, spp = 512, 32
    cam = scenes.cornell_camera(w, w, spp, max_depth=16)
    mt = api.Model(scenes.cornell16(pt))
    target = api.render(mt, api.RenderArgs.from_camera(cam, seed=99), stream=stream).shade(api.Full, stream=stream)
    m = api.Model(scenes.cornell16(p0))
    a = api.RenderArgs.from_camera(cam, seed=1)
    ph = api.Photo(w, w)
    api.render(m, a, ph, stream)
    g = (2.0 * (ph.shade(api.Full, stream=stream) - target)).reshape(-1, 3).contiguous()
    grad = api.adjoint(m, a, ph, g, stream=stream)

    def timeit(fn):
        for _ in range(args.warmup):
            fn()
        barrier()
        ms = []
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.current_stream().wait_stream(stream)
            stream.wait_stream(torch.cuda.current_stream())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(sum(ms)) / len(ms)

    fwd = timeit(lambda: api.render(m, a, ph, stream))
    adj = timeit(lambda: api.adjoint(m, a, ph, g, grad, stream))
    paths = w * w * spp
    return {"workload": "cornell16: 16 materials, 512x512, 32 spp, max depth 16, L2 loss to a target at "
                        "+-10% parameters; gradients of 16 x 5 parameters",
            "forward_ms": fwd, "adjoint_ms": adj, "adjoint_over_forward": adj / fwd,
            "forward_Mpaths_s": paths / fwd / 1e3, "adjoint_Mpaths_s": paths / adj / 1e3,
            "call": "rmn_render then rmn_adjoint on device buffers, CUDA events on the stream"}


def config_timings(args, stream, flush, barrier):
    """The reference's other configurations, each timed on its own (CUDA
    events on the stream, W warm-ups, L2 flushed before each step, device
    buffers):
      cornell     -- Cornell box (36 triangles), 256x256, 64 spp, depth 8;
      traversal   -- 1M-triangle random soup, 4M closest-hit + 4M shadow rays;
      heightfield -- 2048^2 heightfield (8,380,418 triangles) under a
                     2048x1024 sky, 1920x1080, 256 spp, depth 16, composed
                     with gamma and FXAA;
    then the post passes' export set, the textured room, the glass Cornell
    box and the host-side asset front-end."""
    import torch
    from raym0nade_gb300 import api, scenes

    def timeit(fn, steps=None):
        for _ in range(args.warmup):
            fn()
        barrier()
        ms = []
        for _ in range(steps or args.steps):
            flush.fill_(1)
            torch.cuda.current_stream().wait_stream(stream)
            stream.wait_stream(torch.cuda.current_stream())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(sum(ms)) / len(ms)

    out = {}
    cm = api.Model(scenes.cornell())
    cam = scenes.cornell_camera(256, 256, 64, max_depth=8)
    ca = api.RenderArgs.from_camera(cam, seed=1)
    cp = api.Photo(256, 256)
    ms = timeit(lambda: api.render(cm, ca, cp, stream))
    out["cornell"] = {"Mpaths_s": 256 * 256 * 64 / ms / 1e3, "ms": ms,
                      "workload": "Cornell box 36 tris, 256x256, 64 spp, max depth 8 (rmn_render)"}

    soup = api.Model(scenes.random_soup(1_000_000, 1))
    rays = torch.from_numpy(scenes.random_rays(4_000_000, 2)).cuda()
    srays = torch.from_numpy(scenes.random_rays(4_000_000, 3, shadow=True)).cuda()
    hits = soup.rayHit(rays, stream=stream)
    occ = soup.rayHit_test(srays, stream=stream)
    mc = timeit(lambda: soup.rayHit(rays, hits, stream))
    msh = timeit(lambda: soup.rayHit_test(srays, occ, stream))
    out["traversal"] = {"closest_Mrays_s": 4e6 / mc / 1e3, "shadow_Mrays_s": 4e6 / msh / 1e3,
                        "closest_ms": mc, "shadow_ms": msh,
                        "workload": "1M-triangle soup, 4M closest-hit + 4M shadow rays (rmn_trace_closest / _shadow)"}
    del soup, rays, srays, hits, occ

    hf = scenes.heightfield(2048, seed=3)
    hf.env = scenes.sky_env(2048, 1024)
    hm = api.Model(hf)
    hcam = scenes.heightfield_camera(1920, 1080, 256)
    ha = api.RenderArgs.from_camera(hcam, seed=1)
    hp = api.Photo(1920, 1080)
    rgb = torch.empty((1080, 1920, 3), dtype=torch.float32, device="cuda")

    def step_hf():
        api.render(hm, ha, hp, stream)
        hp.shade(api.Full | api.GAMMA | api.DoFXAA, out=rgb, stream=stream)

    ms = timeit(step_hf, steps=max(1, min(args.steps, 2)))
    out["heightfield"] = {"Mpaths_s": 1920 * 1080 * 256 / ms / 1e3, "ms": ms,
                          "workload": "2048^2 heightfield (8,380,418 tris), sky 2048x1024, 1920x1080, 256 spp, "
                                      "max depth 16, gamma + FXAA (rmn_render + rmn_compose)"}

    # the export set of render_multiThread on the heightfield's buffers, with
    # depth of field (25 images); the CPU restatement timed on a crop
    hp.focus, hp.CoC, hp.cameraPosition = 120.0, 6.0, tuple(hcam.position)
    keep = [x.clone() for x in (hp.radiance_Dd, hp.radiance_Ds, hp.radiance_Id, hp.radiance_Is)]
    recs = records_from_photo(hp, 1920, 1080)
    exports = torch.empty((25, 1080, 1920, 3), dtype=torch.float32, device="cuda")

    def step_post():
        for dst, src in zip((hp.radiance_Dd, hp.radiance_Ds, hp.radiance_Id, hp.radiance_Is), keep):
            dst.copy_(src)
        hp.export_set(out=exports, stream=stream)

    ms = timeit(step_post, steps=max(1, min(args.steps, 3)))
    cpu = post_cpu_sample(recs, hp, 240, 136)
    out["post_exports"] = {"ms": ms, "Mpixels_s": 1920 * 1080 / ms / 1e3, "images": 25,
                           "cpu_port_ms_per_Mpixel": cpu["ms_per_Mpixel"], "cpu_sample": cpu["sample"],
                           "gpu_over_cpu": cpu["ms_per_Mpixel"] * 1920 * 1080 / 1e6 / ms,
                           "workload": "render_multiThread's 25 exports of the 1920x1080 heightfield render "
                                       "(spatialClamp, filter, bloom, depth of field CoC 6, gamma, FXAA; "
                                       "rmn_export_set)"}
    del hm, hp, exports, keep

    room = api.Model(scenes.textured_room())
    tcam = scenes.textured_camera(1024, 768, 64)
    ta = api.RenderArgs.from_camera(tcam, seed=1)
    tp = api.Photo(1024, 768)
    ms = timeit(lambda: api.render(room, ta, tp, stream))
    cpu = textured_cpu_sample()
    out["textured"] = {"Mpaths_s": 1024 * 768 * 64 / ms / 1e3, "ms": ms,
                       "cpu_port_Mpaths_s": cpu["Mpaths_s"], "cpu_sample": cpu["sample"],
                       "workload": "textured room (diffuse / specular / emissive / normal-map textures with mip "
                                   "chains, alpha-tested cutouts), 1024x768, 64 spp, max depth 16 (rmn_render)"}
    try:  # glass and media; a failure here is reported, not fatal to the line
        gm = api.Model(scenes.cornell_glass())
        ga = api.RenderArgs.from_camera(scenes.cornell_camera(512, 512, 64), seed=1)
        gp = api.Photo(512, 512)
        ms = timeit(lambda: api.render(gm, ga, gp, stream))
        cpu = glass_cpu_sample()
        out["glass"] = {"Mpaths_s": 512 * 512 * 64 / ms / 1e3, "ms": ms,
                        "cpu_port_Mpaths_s": cpu["Mpaths_s"], "cpu_sample": cpu["sample"],
                        "workload": "Cornell box with a glass tall box and a half-opaque short box, 512x512, "
                                    "64 spp (x16 indirect paths behind glass), max depth 16 (rmn_render)"}
        del gm, gp
    except Exception as e:  # pragma: no cover
        out["glass"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    try:  # host-side asset front-end; a failure here is reported, not fatal to the line
        out["asset_decode"] = asset_decode_timings(max(1, min(args.steps, 3)))
    except Exception as e:  # pragma: no cover
        out["asset_decode"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    return out


def asset_decode_timings(repeats):
    """rmn_image_load (host; the threads the library takes for large files) on full-size asset files written
    here: a 2048x1024 run-length-encoded Radiance sky, a 2048x2048 DXT5 DDS
    texture and a 2048x2048 RGB PNG (zlib level 6, Sub / Up / Paeth rows).
    Best of `repeats` wall-clock decodes each."""
    import shutil
    import tempfile
    from raym0nade_gb300 import assets, scenes
    from tests.golden import image_files as F
    d = tempfile.mkdtemp()
    rng = np.random.default_rng(9)
    files = {}
    p = os.path.join(d, "sky.hdr")
    with open(p, "wb") as f:
        f.write(F.encode_hdr(F.float_to_rgbe(scenes.sky_env(2048, 1024))))
    files["hdr_2048x1024_rle"] = (p, assets.HDR)
    p = os.path.join(d, "tex.dds")
    with open(p, "wb") as f:
        f.write(F.encode_dds(2048, 2048, rng.integers(0, 256, 512 * 512 * 16, dtype=np.uint8).tobytes(), b"DXT5"))
    files["dds_dxt5_2048x2048"] = (p, assets.DDS)
    yy, xx = np.mgrid[0:2048, 0:2048]
    img = np.stack([(xx // 8) % 256, (yy // 8) % 256, ((xx + yy) // 16) % 256], -1) + rng.integers(0, 4, (2048, 2048, 3))
    p = os.path.join(d, "tex.png")
    with open(p, "wb") as f:
        f.write(F.encode_png(np.minimum(img, 255), 2, 8, filters=(1, 2, 4), level=6))
    files["png_rgb8_2048x2048"] = (p, assets.PNG)
    out = {}
    for name, (p, kind) in files.items():
        best, nbytes = float("inf"), 0
        for _ in range(repeats):
            t0 = time.perf_counter()
            a = assets.load_image(p, kind)
            best = min(best, time.perf_counter() - t0)
            nbytes = a.nbytes
        out[name] = {"ms": best * 1e3, "decoded_MB_s": nbytes / best / 1e6, "file_MB": os.path.getsize(p) / 1e6}
    shutil.rmtree(d)
    # rmn_scene_create of the textured room with its eight textures replaced
    # by 2048x2048 RGBA ones: level-0 upload (128 MiB) and the device-built
    # mip chains, beside the BVH and tables of a 30-triangle scene
    from raym0nade_gb300 import api
    room = scenes.textured_room()
    room.textures = [rng.integers(0, 256, (2048, 2048, 4), dtype=np.uint8) for _ in room.textures]
    best = float("inf")
    for _ in range(repeats):
        t0 = time.perf_counter()
        m = api.Model(room)
        best = min(best, time.perf_counter() - t0)
        del m
    out["scene_create_8_textures_2048sq"] = {"ms": best * 1e3, "texture_MB": 8 * 2048 * 2048 * 4 / 1e6}
    # rmn_model_read of a Wavefront OBJ: a 256x256 heightfield (130,050
    # triangles, v/vt/vn per corner), through assets.load_model
    hf = scenes.heightfield(256, seed=3)
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "hf.obj"), "w") as f:
        for key, a in (("v", hf.positions), ("vn", hf.normals), ("vt", hf.uvs)):
            np.savetxt(f, a, fmt=key + " %.6f" * a.shape[1])
        i = hf.indices.astype(np.int64) + 1
        np.savetxt(f, np.repeat(i, 3, axis=1), fmt="f %d/%d/%d %d/%d/%d %d/%d/%d")
    size = os.path.getsize(os.path.join(d, "hf.obj"))
    best = float("inf")
    for _ in range(repeats):
        t0 = time.perf_counter()
        sc = assets.load_model(d + "/", "hf.obj")
        best = min(best, time.perf_counter() - t0)
    assert sc.num_triangles == hf.num_triangles
    shutil.rmtree(d)
    out["obj_import_heightfield_256"] = {"ms": best * 1e3, "file_MB": size / 1e6, "triangles": hf.num_triangles,
                                         "MB_s": size / best / 1e6}
    return out


GB_TO_REC = [16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31, 32, 33, 35, 36, 37]


def records_from_photo(ph, w, h):
    """The oracle's per-pixel records (h, w, 40) of a GPU Photo."""
    import numpy as np
    r = np.zeros((h * w, 40), np.float32)
    for k, b in enumerate((ph.radiance_Dd, ph.radiance_Ds, ph.radiance_Id, ph.radiance_Is)):
        r[:, 4 * k:4 * k + 4] = b.cpu().numpy()
    r[:, GB_TO_REC] = ph.Gbuffer.cpu().numpy()
    r[:, 34] = 0.04  # HitInfo::specular
    return r.reshape(h, w, 40)


def post_cpu_sample(recs, ph, cw, ch):
    """The export sequence of the CPU restatement (single thread, as the
    reference's Photo passes except filter's four threads) on a cw x ch crop."""
    from oracle.bindings import OracleLib
    from raym0nade_gb300 import api
    port = OracleLib("port")
    y0, x0 = (recs.shape[0] - ch) // 2, (recs.shape[1] - cw) // 2
    crop = recs[y0:y0 + ch, x0:x0 + cw].copy()
    post = dict(exposure=1.0, focus=ph.focus, coc=ph.CoC, camera=ph.cameraPosition)
    lib = api._lib.load()
    opts = [lib.rmn_export_options(k) & ~api.GAMMA for k in range(api.EXPORTS + api.EXPORTS_DOF)]
    t0 = time.perf_counter()
    r = crop
    for k, o in enumerate(opts):
        if k == 4:
            r, _ = port.photo(r, 1)
        if k == 12:
            r, _ = port.photo(r, 2)
        port.photo(r, 4, o, **post)
    dt = (time.perf_counter() - t0) * 1e3
    return {"ms_per_Mpixel": dt / (cw * ch / 1e6), "sample": f"{cw}x{ch} centre crop, 25 exports, 1 thread"}


def textured_cpu_sample():
    """The CPU restatement (all host threads) of the textured room on a
    256x192 image at 64 spp."""
    import os as _os
    from oracle.bindings import OracleLib
    from raym0nade_gb300 import scenes
    port = OracleLib("port")
    sc = port.scene(scenes.textured_room())
    cam = scenes.textured_camera(256, 192, 64)
    th = _os.cpu_count() or 8
    t0 = time.perf_counter()
    sc.render(cam, seed=1, mode=0, threads=th)
    dt = time.perf_counter() - t0
    return {"Mpaths_s": 256 * 192 * 64 / dt / 1e6, "sample": f"256x192, 64 spp, {th} threads"}


def glass_cpu_sample():
    """The CPU restatement (all host threads) of the glass Cornell box on a
    96x96 image at 64 spp."""
    import os as _os
    from oracle.bindings import OracleLib
    from raym0nade_gb300 import scenes
    port = OracleLib("port")
    sc = port.scene(scenes.cornell_glass())
    cam = scenes.cornell_camera(96, 96, 64)
    th = _os.cpu_count() or 8
    t0 = time.perf_counter()
    sc.render(cam, seed=1, mode=0, threads=th)
    dt = time.perf_counter() - t0
    return {"Mpaths_s": 96 * 96 * 64 / dt / 1e6, "sample": f"96x96, 64 spp, {th} threads"}


def run_gpu(args, rank, world, dist):
    import torch
    from raym0nade_gb300 import api

    torch.cuda.init()
    dev = torch.cuda.current_device()
    insts, desc = workload(args.workload, rank)
    paths_per_step = sum(instance_paths(i) for i in insts)
    t0 = time.perf_counter()
    models = [api.Model(i.scene) for i in insts]
    build_s = time.perf_counter() - t0
    scene_bytes = sum(m.info()["device_bytes"] for m in models)
    argsl = [api.RenderArgs.from_camera(i.camera, seed=i.seed) for i in insts]
    photos = [api.Photo(i.camera.width, i.camera.height) for i in insts]
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    tune = None
    if args.autotune:
        # project autotuner: slots per work unit x worker pool x lanes, then
        # the traversal stack, timed on a 1/16-pixel proxy of the same batch
        # (untimed here)
        t0 = time.perf_counter()
        tune = api.autotune(list(zip(models, argsl, photos)), 1.0 / 16, stream)
        tune["tune_s"] = round(time.perf_counter() - t0, 2)
        for a in argsl:
            a.slots_per_unit = tune["slots_per_unit"]
    lanes = (tune["lanes"] if tune else 0) or 3  # 0: the library default, 3 lanes
    with torch.cuda.stream(stream):
        batch = api.Batch(list(zip(models, argsl, photos)), use_graph=True, stream=stream,
                          pool_workers=tune["pool_workers"] if tune else 0, lanes=tune["lanes"] if tune else 0,
                          stack_entries=tune["stack_entries"] if tune else 0,
                          ray_order=tune["ray_order"] if tune else 0)

    def step_batched():
        batch.render(stream)

    def step_plain():
        for m, a, ph in zip(models, argsl, photos):
            api.render(m, a, ph, stream)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(fn, steps, warmup, sampler=None):
        for _ in range(warmup):
            fn()
        barrier()
        if sampler:
            sampler.start()
        ms = []
        for _ in range(steps):
            flush.fill_(1)
            torch.cuda.current_stream().wait_stream(stream)
            stream.wait_stream(torch.cuda.current_stream())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        barrier()
        clocks = sampler.stop() if sampler else None
        total = max_over_ranks(float(sum(ms)), dist, "cuda")
        return total / steps, clocks

    # profile once (untimed): visit counters and per-kernel times of the batch
    prof = batch.profile(stream)
    sampler = ClockSampler(dev) if rank == 0 else None
    ms_b, clocks = timed(step_batched, args.steps, args.warmup, sampler)
    ms_p, _ = timed(step_plain, args.steps, 1)

    # End to end through the C ABI, host in and host out, wall clock: every
    # step uploads the 64 cameras and seeds from pinned host memory
    # (rmn_batch_update), renders the batch (rmn_batch_render) and brings
    # every instance's display image back to pinned host memory
    # (rmn_compose(Full | gamma | FXAA) into a host array).
    disp = [torch.empty((i.camera.height, i.camera.width, 3), dtype=torch.float32).pin_memory() for i in insts]

    def step_e2e():
        batch.update(argsl, stream)
        batch.render(stream)
        for ph, d in zip(photos, disp):
            ph.shade(api.Full | api.GAMMA | api.DoFXAA, out=d, stream=stream)

    e2e_steps = max(1, min(args.steps, 3))
    step_e2e()
    barrier()
    t = time.perf_counter()
    for _ in range(e2e_steps):
        step_e2e()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t) / e2e_steps, dist, "cuda")
    npx = sum(i.camera.width * i.camera.height for i in insts)
    d2h = npx * 12 + 4  # display images, and the batch's status word
    h2d = batch.update_bytes

    adj = adjoint_timing(args, stream, flush, barrier) if args.adjoint else None
    per_config = config_timings(args, stream, flush, barrier) if args.configs else None

    value = job_rate(paths_per_step, world, ms_b / 1e3)
    plain = job_rate(paths_per_step, world, ms_p / 1e3)
    if rank != 0:
        return
    peak, peak_src = measured_peaks()
    # Dominant kernel: the wavefront's traversal (closest + shadow queues).
    # Its algorithmic bytes: 64 B per inner-node visit (two child boxes),
    # 36 B per triangle test, 32 B ray in + 8 B answer out per ray. The
    # G-buffer kernel's primary rays are counted in the visits but not in
    # trace_ms, so they are taken out in proportion to their rays.
    rays = prof["closest_rays"] + prof["shadow_rays"]
    queued = max(1, rays - npx)
    alg_bytes = (64 * prof["inner_visits"] + 36 * prof["triangle_tests"]) * queued / max(1, rays) + 40 * queued
    total_ms = prof["primary_ms"] + prof["path_ms"]
    trace_share = prof["trace_ms"] / max(1e-9, total_ms)
    logic_share = prof["logic_ms"] / max(1e-9, total_ms)
    trace_ms_live = ms_b * trace_share
    achieved = alg_bytes / (trace_ms_live / 1e3) / 1e9
    # measured traffic of the traversal launches, where a capture of this
    # workload at this launch configuration exists
    traffic, traffic_src, l2 = None, None, None
    if args.workload == "batch64":
        timed = {"slots_per_unit": tune["slots_per_unit"] if tune else 0,
                 "pool_workers": tune["pool_workers"] if tune else 0, "lanes": tune["lanes"] if tune else 0,
                 "stack_entries": tune["stack_entries"] if tune else 0, "ray_order": tune["ray_order"] if tune else 0}
        cap = next((c for c in BATCH64_TRAVERSAL_BYTES if c["config"] == timed), BATCH64_TRAVERSAL_BYTES[0])
        cfg = cap["config"]
        same = timed == cfg
        traffic = cap["dram"]
        traffic_src = ("ncu dram__bytes_read.sum + dram__bytes_write.sum over every qtrace_kernel and qocc_kernel "
                       "launch of one "
                       "batch64 render at " + json.dumps(cfg) + ("" if same else "; NOT the timed configuration"))
        l2_peak = l2_copy_gbs(stream)
        l2_gbs = cap["l2"] / (trace_ms_live / 1e3) / 1e9
        l2 = {"bytes_per_step": cap["l2"], "achieved": l2_gbs, "unit": "GB/s",
              "copy_rate": l2_peak, "frac_of_copy_rate": l2_gbs / l2_peak, "same_config": same,
              "source": "ncu lts__t_bytes.sum over the same launches; copy_rate: a device copy between two "
                        "L2-resident 24 MiB buffers, measured here"}
    limiter = ("instruction issue and dependent-load latency: in steady state (ncu) the closest-hit traversal "
               "uses 67 % of its issue slots with 17.5 of 32 lanes active per instruction (warp-cooperative "
               "leaves), the occlusion traversal 69 % with 18.5 lanes (pending leaves), both stalled mostly on "
               "L1/L2 loads (long scoreboard 3.1-3.9 per issue) and fixed-latency dependencies (2.3-2.9); their "
               "measured DRAM traffic is a small share of the algorithmic bytes (L1/L2 hits) and neither DRAM "
               "nor L2 runs near its rate")
    base, _ = cpu_baseline(insts) if args.cpu_baseline else (None, None)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_b, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural scenes; no dataset)",
        "config": workload_config(insts, desc, world),
        "setup": {"launch": "rmn_batch: G-buffer kernel, then wavefront iterations (shade, NEE, slot, closest and "
                            "shadow traversal kernels) of every lane as parallel branches of a replayed CUDA graph",
                  "scene_bytes": scene_bytes, "scene_build_s": round(build_s, 1)},
        "plain": {"value": plain, "unit": UNIT, "ms_per_step": ms_p, "launches_per_step": 2 * len(insts),
                  "batched_over_plain": value / plain},
        "e2e": {"value": job_rate(paths_per_step, world, e2e_s), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "call": "rmn_batch_update (cameras and seeds from pinned host memory) + rmn_batch_render + "
                        "rmn_compose(Full|gamma|FXAA) of every instance into pinned host memory; wall clock"},
        # per batched step: G-buffer kernel, one seed kernel per lane, 8 kernels
        # per wavefront iteration and lane (14 with binned ray queues), finalize
        "gpu_launches": args.steps * (2 + lanes + (14 if tune and tune["ray_order"] else 8) * lanes *
                                      prof["iterations"]),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_source": traffic_src,
                     "per": "step (all traversal launches of one step)",
                     "kernel": "qtrace_kernel (closest queue) + qocc_kernel (shadow queue)", "peak_source": peak_src,
                     "bytes_model": "64 B per inner-node visit + 36 B per triangle test + 40 B per queued ray",
                     "algorithmic_bytes_per_step": alg_bytes, "trace_share": trace_share,
                     "logic_share": logic_share, "iterations": prof["iterations"],
                     "l2": l2, "limiter": limiter},
        "rays": {"closest": prof["closest_rays"], "shadow": prof["shadow_rays"], "Mrays_s": rays / ms_b / 1e3},
        "clocks": clocks,
    }
    if tune:
        out["setup"]["autotune"] = tune
    if adj:
        out["adjoint"] = adj
    if per_config:
        out["configs"] = per_config
    if base:
        out["cpu_baseline"] = base
    print(json.dumps(out))


def profile_case(a):
    """One small, self-contained case per kernel for ncu (``--profile-case``):
    each builds its scene, runs the work once as a warm-up and once more, and
    exits, so ``ncu --clock-control none -k regex:<kernel> -s <n> -c 1``
    captures a warm launch. Scene data is sized above the 129 MB L2 where the
    case allows, while the process holds a few GB at most (the batch case: the
    64-instance workload at the given launch configuration).

      render    a heightfield (--tris) under the synthetic sky, --size square,
                --spp, rendered twice as a one-item rmn_batch at --slots per
                unit, --pool workers per lane, --lanes, --stack, --order (0:
                library defaults) -- small pools over many units give a
                steady state
      trace     rmn_trace_closest / rmn_trace_shadow on a random soup (--tris,
                --rays)
      batch     the batch64 workload as one rmn_batch (--slots per unit,
                --pool workers per lane, --lanes, --stack entries), rendered
                twice
      adjoint   rmn_render then rmn_adjoint of the 16-material Cornell box,
                --size square, --spp, depth 16, twice
      fxaa      rmn_compose(Full | gamma | FXAA) of a --size WxH image
      post      the textured room at --size WxH, then rmn_export_set twice
      textured  rmn_render of the textured room at --size WxH, twice
      mips      rmn_scene_create of the textured room with its eight
                textures at 2048 x 2048, twice (device mip chains)
    """
    import torch

    from raym0nade_gb300 import api, scenes

    torch.cuda.init()
    t0 = time.time()
    if a.profile_case == "render":
        n = max(3, int(round(math.sqrt(a.tris / 2.0))) + 1)
        s = scenes.heightfield(n, seed=3)
        s.env = scenes.sky_env(1024, 512)
        side = int(a.size)
        cam = scenes.heightfield_camera(side, side, a.spp)
        m = api.Model(s)
        args = api.RenderArgs.from_camera(cam, seed=1)
        args.slots_per_unit = a.slots
        ph = api.Photo(side, side)
        b = api.Batch([(m, args, ph)], use_graph=False, pool_workers=a.pool, lanes=a.lanes, stack_entries=a.stack,
                      ray_order=a.order)
        for _ in range(2):
            b.render()
        torch.cuda.synchronize()
        prof = b.profile()
        print("render", m.info(), "pixels", side * side, "spp", a.spp, "slots", a.slots, "pool", a.pool,
              "lanes", a.lanes, "iterations", prof["iterations"])
    elif a.profile_case == "batch":
        insts = scenes.batch_instances(64, seed=7)
        models = [api.Model(i.scene) for i in insts]
        argsl = [api.RenderArgs.from_camera(i.camera, seed=i.seed) for i in insts]
        for r in argsl:
            r.slots_per_unit = a.slots
        photos = [api.Photo(i.camera.width, i.camera.height) for i in insts]
        b = api.Batch(list(zip(models, argsl, photos)), use_graph=True, pool_workers=a.pool, lanes=a.lanes,
                      stack_entries=a.stack, ray_order=a.order)
        for _ in range(2):
            b.render()
        torch.cuda.synchronize()
        print("batch", len(insts), "instances: slots", a.slots, "pool", a.pool, "lanes", a.lanes, "stack", a.stack)
    elif a.profile_case == "adjoint":
        side = int(a.size)
        cam = scenes.cornell_camera(side, side, a.spp, max_depth=16)
        m = api.Model(scenes.cornell16())
        args = api.RenderArgs.from_camera(cam, seed=1)
        ph = api.render(m, args)
        g = torch.ones((side * side, 3), dtype=torch.float32, device="cuda")
        for _ in range(2):
            api.adjoint(m, args, ph, g)
        torch.cuda.synchronize()
        print("adjoint", side, "spp", a.spp)
    elif a.profile_case == "trace":
        s = scenes.random_soup(a.tris, 1)
        m = api.Model(s)
        rays = torch.from_numpy(scenes.random_rays(a.rays, 2)).cuda()
        sr = torch.from_numpy(scenes.random_rays(a.rays, 3, shadow=True)).cuda()
        for _ in range(2):
            m.rayHit(rays)
            m.rayHit_test(sr)
        torch.cuda.synchronize()
        print("trace", m.info(), "rays", a.rays)
    elif a.profile_case == "mips":
        rng = np.random.default_rng(2)
        room = scenes.textured_room()
        room.textures = [rng.integers(0, 256, (2048, 2048, 4), dtype=np.uint8) for _ in room.textures]
        for _ in range(2):
            m = api.Model(room)
            del m
        torch.cuda.synchronize()
        print("mips", len(room.textures), "textures of 2048 x 2048")
    elif a.profile_case in ("post", "textured"):
        w, h = (int(x) for x in a.size.split("x")) if "x" in a.size else (1920, 1080)
        m = api.Model(scenes.textured_room())
        cam = scenes.textured_camera(w, h, a.spp)
        args = api.RenderArgs.from_camera(cam, seed=1)
        ph = api.Photo(w, h)
        api.render(m, args, ph)
        if a.profile_case == "textured":
            api.render(m, args, ph)
        else:
            ph.focus, ph.CoC, ph.cameraPosition = 3.0, 6.0, tuple(cam.position)
            out = torch.empty((api.EXPORTS + api.EXPORTS_DOF, h, w, 3), dtype=torch.float32, device="cuda")
            for _ in range(2):
                ph.export_set(out)
        torch.cuda.synchronize()
        print(a.profile_case, w, h, "spp", a.spp)
    else:
        w, h = (int(x) for x in a.size.split("x")) if "x" in a.size else (1920, 1080)
        rng = np.random.default_rng(1)
        ph = api.Photo(w, h)
        n = w * h
        for k in ("radiance_Dd", "radiance_Ds", "radiance_Id", "radiance_Is"):
            getattr(ph, k).copy_(torch.from_numpy(rng.random((n, 4), dtype=np.float32)))
        ph.Gbuffer.copy_(torch.from_numpy(rng.random((n, api.GBUFFER_FLOATS), dtype=np.float32)))
        for _ in range(2):
            ph.shade(api.Full | api.GAMMA | api.DoFXAA)
        torch.cuda.synchronize()
        print("fxaa", w, h)
    print(f"done in {time.time() - t0:.1f} s")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch64", choices=["batch64", "cornell", "heightfield"])
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false")
    ap.add_argument("--no-adjoint", dest="adjoint", action="store_false")
    ap.add_argument("--no-configs", dest="configs", action="store_false")
    ap.add_argument("--profile-case", choices=["render", "trace", "batch", "adjoint", "fxaa", "post", "textured", "mips"],
                    help="run one small case for a profiler instead of the benchmark (see profile_case)")
    ap.add_argument("--tris", type=int, default=2_000_000)
    ap.add_argument("--size", default="256")
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--rays", type=int, default=1_000_000)
    ap.add_argument("--slots", type=int, default=0)
    ap.add_argument("--pool", type=int, default=0)
    ap.add_argument("--lanes", type=int, default=0)
    ap.add_argument("--stack", type=int, default=0)
    ap.add_argument("--order", type=int, default=0)
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args)
        return
    if args.warmup < 3:
        raise SystemExit("at least 3 warm-up steps")
    rank, world, dist = (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), None)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    rank, world, dist = dist_setup()
    run_gpu(args, rank, world, dist)


if __name__ == "__main__":
    main()
