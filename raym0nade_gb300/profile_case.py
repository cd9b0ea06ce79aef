"""One small, self-contained case per kernel, for profilers (ncu).

Each case builds its scene, runs the kernel once as a warm-up and once more,
then exits -- so ``ncu -k regex:<kernel> -s 1 -c 1`` captures one warm
launch. Scene data is sized above the 129 MB L2 (DRAM counters stay
meaningful) while the whole process holds well under a few GB.

  python -m raym0nade_gb300.profile_case render [--tris N] [--size S] [--spp K]
      rmn_render of a heightfield (smooth normals, GGX + Lambertian patches)
      under the synthetic sky: primary_kernel + path_kernel.
  python -m raym0nade_gb300.profile_case trace [--tris N] [--rays R]
      rmn_trace_closest and rmn_trace_shadow on a random soup: trace_kernel.
  python -m raym0nade_gb300.profile_case batch [--lanes L]
      rmn_batch of the 64-instance benchmark batch (slots per unit 4, 2^21
      workers per lane), rendered twice: every wavefront kernel.
  python -m raym0nade_gb300.profile_case fxaa [--size WxH]
      rmn_compose(Full | gamma | FXAA): compose_kernel + fxaa_kernel.
  python -m raym0nade_gb300.profile_case post [--size WxH] [--spp K]
      a render of the textured room (every pixel a hit), then the export set
      of render_multiThread (rmn_export_set: spatialClamp, filter, bloom,
      depth of field, gamma, FXAA) twice.
  python -m raym0nade_gb300.profile_case textured [--size WxH] [--spp K]
      rmn_render of the textured room: the wavefront kernels with textures
      and alpha-tested traversal.
"""
from __future__ import annotations

import argparse
import math
import time

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["render", "trace", "fxaa", "batch", "post", "textured"])
    ap.add_argument("--lanes", type=int, default=2)
    ap.add_argument("--tris", type=int, default=2_000_000)
    ap.add_argument("--size", default="256")
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--rays", type=int, default=1_000_000)
    a = ap.parse_args(argv)

    import torch

    from . import api, scenes

    torch.cuda.init()
    if a.case == "render":
        n = max(3, int(round(math.sqrt(a.tris / 2.0))) + 1)
        s = scenes.heightfield(n, seed=3)
        s.env = scenes.sky_env(1024, 512)
        side = int(a.size)
        cam = scenes.heightfield_camera(side, side, a.spp)
        m = api.Model(s)
        args = api.RenderArgs.from_camera(cam, seed=1)
        ph = api.Photo(side, side)
        for _ in range(2):
            api.render(m, args, ph)
        torch.cuda.synchronize()
        print("render", m.info(), "pixels", side * side, "spp", a.spp)
    elif a.case == "batch":
        insts = scenes.batch_instances(64, seed=7)
        models = [api.Model(i.scene) for i in insts]
        argsl = [api.RenderArgs.from_camera(i.camera, seed=i.seed) for i in insts]
        for r in argsl:
            r.slots_per_unit = 4
        photos = [api.Photo(i.camera.width, i.camera.height) for i in insts]
        b = api.Batch(list(zip(models, argsl, photos)), use_graph=True, pool_workers=1 << 21, lanes=a.lanes)
        for _ in range(2):
            b.render()
        torch.cuda.synchronize()
        print("batch", len(insts), "instances, lanes", a.lanes)
    elif a.case == "trace":
        s = scenes.random_soup(a.tris, 1)
        m = api.Model(s)
        rays = torch.from_numpy(scenes.random_rays(a.rays, 2)).cuda()
        sr = torch.from_numpy(scenes.random_rays(a.rays, 3, shadow=True)).cuda()
        for _ in range(2):
            m.rayHit(rays)
            m.rayHit_test(sr)
        torch.cuda.synchronize()
        print("trace", m.info(), "rays", a.rays)
    elif a.case in ("post", "textured"):
        w, h = (int(x) for x in a.size.split("x")) if "x" in a.size else (1920, 1080)
        m = api.Model(scenes.textured_room())
        cam = scenes.textured_camera(w, h, a.spp)
        args = api.RenderArgs.from_camera(cam, seed=1)
        ph = api.Photo(w, h)
        api.render(m, args, ph)
        if a.case == "textured":
            api.render(m, args, ph)
        else:
            ph.focus, ph.CoC, ph.cameraPosition = 3.0, 6.0, tuple(cam.position)
            out = torch.empty((api.EXPORTS + api.EXPORTS_DOF, h, w, 3), dtype=torch.float32, device="cuda")
            for _ in range(2):
                ph.export_set(out)
        torch.cuda.synchronize()
        print(a.case, w, h, "spp", a.spp)
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


if __name__ == "__main__":
    t = time.time()
    main()
    print(f"done in {time.time() - t:.1f} s")
