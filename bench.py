"""Benchmark: Mrays/s of the sparse-voxel tile renderer on one GB300.

Workload (one step = one full frame): the 1280x720 full-frame render of a
4x4x1-tile scene (128^3 voxels per 3 m tile, FP16 32-dim corner features,
per-tile MLP 59 -> 64x3 -> 3, 5.1 % occupied, ~205k-triangle proxy mesh in
a BVH), cycling
through 8 seeded interior camera poses.  Seeded synthetic data stands in for
the reference's captured scenes, which are not distributed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is device-timed throughput (CUDA events per step, L2 flushed between
steps); `e2e` is the same metric through snisr_render_host (host output
buffers, device->host copies inside the timed region).  With N > 1 (torchrun)
every rank renders its own frames: rays are independent, so ranks are
replicas with no data-path collective.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "scalable-neural-indoor-scene-rendering_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Mrays/s render & fwd+bwd train, BF16-TC vs plain FP32 on GB300 @ RMSE≤1e-3"
UNIT = "Mrays/s"
WORKLOAD = ("cfg2 full-frame render 1280x720: 4x4x1 tiles of 128^3 over 3 m, 5.1% occupied (walls, floor, ceiling, "
            "40 boxes), FP16 32-dim corner features, per-tile FP16 MLP 59-64x3-3, 205k-triangle proxy BVH, "
            "8 seeded poses")
MLP_FLOP_PER_SAMPLE = 2 * (59 * 64 + 64 * 64 + 64 * 64 + 64 * 3)  # 24,320
GATHER_BYTES_PER_SAMPLE = 8 * (32 + 1) * 2                         # 528 (FP16 features + density)
# bytes of one tile's FP16 weight image for the tensor-core MLP (H = 64, L = 3):
# W_l [64][64] x 3, W_out [16][64], hidden-bias tile [64][64], output-bias tile [16][64]
TC_IMAGE_BYTES = 3 * 64 * 128 + 2048 + 64 * 128 + 2048               # 36,864
TRAIN_WORKLOAD = ("cfg3 training step (forward + backward): 1 tile of 256^3 over 4 m, ~4% occupied, FP32 32-dim "
                  "vertex features, MLP 59-64x3-3, 65,536 rays from 8 seeded 640x480 views, MSE against a "
                  "second scene's render (features + N(0, 0.02))")


# DRAM bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum) of
# the kernels of one frame / step, from one capture of the same workload; the
# summaries with their commands are under profiles/.
SAMPLE_RECORD_BYTES = 16  # SampleRec: voxel id, 24-bit pixel + weight, 16-bit fixed-point position
NCU_DRAM_BYTES_PER_LAUNCH = {
    "mlp_tc": {"bytes": 226571827,
               "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of mlp_tc_kernel<32, 64, 3>, mean of the "
                         "5 launches (5 poses) of `bench.py --profile-run render --steps 2 --warmup 1` "
                         "(profiles/launches_render_cfg2.md)"},
    "traverse": {"bytes": 88752588, "source": "same capture"},
    "scatter": {"bytes": 154275891, "source": "same capture"},
}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("gloo")
    return ws, rank, local


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(ws, v: float) -> float:
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_poses(rank: int, poses: int):
    """Pose order of one replica: every rank starts at a different pose."""
    return [(rank * 3 + p) % poses for p in range(poses)]


def job_value(ws: int, rays_per_step: int, steps: int, max_ms: float) -> float:
    """Whole-job Mrays/s: every rank renders `steps` frames; time = the slowest rank."""
    return ws * rays_per_step * steps / (max_ms * 1e-3) / 1e6


class HostPath:
    """The reference's method as a scalar host path: the oracle port in FP32,
    one ray per host thread at a time.  Per ray the same work as the GPU
    frame: the camera direction, the nearest proxy-mesh hit (through the
    oracle's own BVH when the scene has a mesh), the start 2 voxels before
    it, the march over occupied voxels, density, MLP and compositing with
    early stop."""

    def __init__(self, synth, threads: int):
        import oracle
        self.synth, self.threads = synth, threads
        self.osc = oracle.OracleScene(synth.desc)
        self.has_mesh = synth.desc.num_triangles > 0
        self.dirs = {}

    def rays(self, pose: int):
        import oracle
        if pose not in self.dirs:
            cam = self.synth.camera(pose)
            self.dirs[pose] = (oracle.camera_dirs(cam), cam)
        return self.dirs[pose]

    def run(self, pose: int, idx):
        """Render pixels `idx` (sorted indices, or None for the whole frame) of a pose."""
        import numpy as np

        import oracle
        d_all, cam = self.rays(pose)
        d = d_all if idx is None else np.ascontiguousarray(d_all[idx])
        o = oracle.camera_origins(cam, d.shape[0])
        ts = self.osc.proxy_bvh(o, d, self.threads)[0] if self.has_mesh else None
        self.osc.render(o, d, ts, 0, self.threads)
        return d.shape[0]


def cpu_baseline_run(synth, steps: int, target_s: float, threads: int, warmup: int = 1):
    """The host path (HostPath) on all host threads, on a bounded random
    sample of each pose's pixels, sized so that `steps` steps take about
    target_s seconds after `warmup` untimed steps."""
    import numpy as np
    hp = HostPath(synth, threads)
    npix = synth.cfg.width * synth.cfg.height
    rng = np.random.default_rng(0)
    probe = 4096
    # warm-up (builds the oracle's BVH, pages the scene in) and rate calibration
    rate = None
    for w in range(max(1, warmup)):
        idx = np.sort(rng.choice(npix, probe, replace=False))
        t0 = time.perf_counter()
        hp.run(w % synth.cfg.poses, idx)
        rate = probe / max(time.perf_counter() - t0, 1e-6)
    n = int(min(npix, max(probe, rate * target_s / max(steps, 1))))
    total_rays, total_t = 0, 0.0
    for s in range(steps):
        idx = np.sort(rng.choice(npix, n, replace=False)) if n < npix else None
        t0 = time.perf_counter()
        total_rays += hp.run(s % synth.cfg.poses, idx)
        total_t += time.perf_counter() - t0
    start = ("2 voxels before the nearest proxy-mesh hit (the oracle's BVH over the same mesh)" if hp.has_mesh
             else "at the scene entry (no proxy mesh)")
    what = "whole frames" if n >= npix else f"{n} random pixels per step"
    return {"value": total_rays / total_t / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{what} x {steps} steps over the {synth.cfg.poses} poses of the "
                      f"{synth.cfg.width}x{synth.cfg.height} frame ({warmup} warm-up steps), FP32 scalar oracle, "
                      f"{threads} threads; rays start {start}, as in the GPU frame"}


def train_bench(dev, steps: int, warmup: int, flush):
    """Training forward + backward (autograd through the hand-written adjoint)
    of the cfg3 workload, tensor-core form and plain FP32 form."""
    import numpy as np
    import torch

    import snisr
    from snisr.train import tile_field
    cfg = snisr.CFG3
    nrays, views = 65536, 8
    synth = snisr.SynthScene(cfg, max_pixels=1024, max_samples_per_ray=48)
    scene = snisr.Scene(synth.desc, dev.index)
    a = synth.arrays()
    vf = torch.from_numpy(a["vertex_feat"].astype(np.float32)).to(dev).requires_grad_(True)
    vd = torch.from_numpy(a["vertex_density"].astype(np.float32)).to(dev).requires_grad_(True)
    W = torch.from_numpy(a["mlp_params"].copy()).to(dev).requires_grad_(True)
    rng = np.random.default_rng(2003)
    os_, ds_ = [], []
    for v in range(views):
        cam = synth.camera(v)
        d = snisr.camera_rays(cam, dev.index).cpu().numpy()
        idx = np.sort(rng.choice(d.shape[0], nrays // views, replace=False))
        ds_.append(d[idx])
        os_.append(np.broadcast_to(np.array([cam.c2w[3], cam.c2w[7], cam.c2w[11]], np.float32), (idx.size, 3)))
    o = torch.from_numpy(np.ascontiguousarray(np.concatenate(os_))).to(dev)
    d = torch.from_numpy(np.ascontiguousarray(np.concatenate(ds_))).to(dev)
    rt = torch.zeros(nrays, dtype=torch.int32, device=dev)
    with torch.no_grad():
        vf_t = vf + 0.02 * torch.randn(vf.shape, generator=torch.Generator(device=dev).manual_seed(7), device=dev)
        target = tile_field(vf_t.contiguous(), vd.detach(), W.detach(), scene, o, d, rt, snisr.FORM_PLAIN_FP32)
    stream = torch.cuda.current_stream()
    res = {"workload": TRAIN_WORKLOAD, "unit": UNIT}
    res["tuning"], _ = scene.autotune_train(vf.detach(), vd.detach(), W.detach(), o, d, rt, reps=3)
    for name, form in (("tc", snisr.FORM_TC), ("plain_fp32", snisr.FORM_PLAIN_FP32)):
        def step():
            vf.grad = vd.grad = W.grad = None
            rgb = tile_field(vf, vd, W, scene, o, d, rt, form)
            loss = ((rgb - target) ** 2).mean()
            loss.backward()
            return loss
        for _ in range(warmup):
            step()
        scene.check()
        torch.cuda.synchronize()
        total = 0.0
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            loss = step()
            e1.record(stream)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        scene.check()
        res[name] = {"value": round(nrays * steps / (total * 1e-3) / 1e6, 3),
                     "ms_per_step": round(total / steps, 4), "loss": float(loss.detach())}
    res["speedup_tc_vs_plain"] = round(res["tc"]["value"] / res["plain_fp32"]["value"], 3)
    res["tc_grad_rel_err_vs_plain"] = _grad_err_tc_vs_plain(scene, vf, vd, W, o, d, rt, target)
    res["l2"] = "flushed before each step"
    scene.close()
    return res


def _grad_err_tc_vs_plain(scene, vf, vd, W, o, d, t, target):
    """Relative error ||g_tc - g_plain|| / ||g_plain|| per parameter group of one
    MSE step at the full benchmark shape (the plain FP32 form is within 1e-3
    of the FP64 oracle in the parity tests, so this bounds the tensor-core
    form's gradient error at the size the speed is measured on)."""
    import snisr
    from snisr.train import tile_field
    grads = {}
    for form in (snisr.FORM_TC, snisr.FORM_PLAIN_FP32):
        vf.grad = vd.grad = W.grad = None
        rgb = tile_field(vf, vd, W, scene, o, d, t, form)
        ((rgb - target) ** 2).sum().backward()
        grads[form] = [x.grad.detach().clone() for x in (vf, vd, W)]
    scene.check()
    out = {}
    for name, a, b in zip(("features", "density", "mlp"), grads[snisr.FORM_TC], grads[snisr.FORM_PLAIN_FP32]):
        out[name] = float(f"{float((a - b).norm() / b.norm().clamp_min(1e-30)):.3e}")
    vf.grad = vd.grad = W.grad = None
    return out


BATCH_WORKLOAD = ("cfg4 batched multi-tile training step (forward + backward): 32 tiles of 128^3 over 3 m, 5.0% "
                  "occupied, FP32 "
                  "32-dim vertex features, per-tile MLP 59-64x3-3; ray segments from 8 seeded 640x480 views split at "
                  "tile faces (tile DDA), log-uniform [1,024, 65,536] segments per tile, grouped by tile")


def batched_bench(dev, steps: int, warmup: int, flush):
    """cfg4: one batched forward+backward over all tiles (tensor-core form),
    the same as 32 per-tile calls, the plain FP32 form, and the batched step
    replayed from a CUDA graph."""
    import numpy as np
    import torch

    import snisr
    from snisr import batch
    from snisr.train import tile_field
    cfg = snisr.CFG4
    synth = snisr.SynthScene(cfg, max_pixels=1024, max_samples_per_ray=24)
    scene = snisr.Scene(synth.desc, dev.index)
    o, d, t, counts = batch.tile_batch(synth, views=8, seed=4004, device=dev.index)
    n = int(o.shape[0])
    a = synth.arrays()
    vf = torch.from_numpy(a["vertex_feat"].astype(np.float32)).to(dev).requires_grad_(True)
    vd = torch.from_numpy(a["vertex_density"].astype(np.float32)).to(dev).requires_grad_(True)
    W = torch.from_numpy(a["mlp_params"].copy()).to(dev).requires_grad_(True)
    with torch.no_grad():
        vf_t = vf + 0.02 * torch.randn(vf.shape, generator=torch.Generator(device=dev).manual_seed(7), device=dev)
        target = tile_field(vf_t.contiguous(), vd.detach(), W.detach(), scene, o, d, t, snisr.FORM_PLAIN_FP32)
    bounds = np.concatenate([[0], np.cumsum(counts)])
    stream = torch.cuda.current_stream()

    def step_batched(form):
        rgb = tile_field(vf, vd, W, scene, o, d, t, form)
        loss = ((rgb - target) ** 2).sum() / n
        loss.backward()

    def step_per_tile(form=snisr.FORM_TC):
        for i in range(len(counts)):
            if counts[i] == 0:
                continue
            sl = slice(int(bounds[i]), int(bounds[i + 1]))
            rgb = tile_field(vf, vd, W, scene, o[sl], d[sl], t[sl], form)
            (((rgb - target[sl]) ** 2).sum() / n).backward()

    def timed(fn, k):
        for _ in range(warmup):
            vf.grad = vd.grad = W.grad = None
            fn()
        scene.check()
        torch.cuda.synchronize()
        total = 0.0
        for _ in range(k):
            vf.grad = vd.grad = W.grad = None
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        scene.check()
        return total / k

    res = {"workload": BATCH_WORKLOAD, "unit": UNIT, "segments": n, "tiles": int((counts > 0).sum()),
           "segments_per_tile": [int(c) for c in counts]}
    res["tuning"], _ = scene.autotune_train(vf.detach(), vd.detach(), W.detach(), o, d, t, reps=2)
    ms = timed(lambda: step_batched(snisr.FORM_TC), steps)
    res["tc_batched"] = {"value": round(n / ms / 1e3, 3), "ms_per_step": round(ms, 4), "launches": "one per stage"}
    ms_pt = timed(step_per_tile, max(3, steps // 2))
    res["tc_per_tile_calls"] = {"value": round(n / ms_pt / 1e3, 3), "ms_per_step": round(ms_pt, 4),
                                "calls": int((counts > 0).sum())}
    ms_pl = timed(lambda: step_batched(snisr.FORM_PLAIN_FP32), max(3, steps // 2))
    res["plain_fp32_batched"] = {"value": round(n / ms_pl / 1e3, 3), "ms_per_step": round(ms_pl, 4)}
    # the baseline this workload is specified against: one plain FP32 call per tile
    ms_ppt = timed(lambda: step_per_tile(snisr.FORM_PLAIN_FP32), max(3, steps // 2))
    res["plain_fp32_per_tile_calls"] = {"value": round(n / ms_ppt / 1e3, 3), "ms_per_step": round(ms_ppt, 4),
                                        "calls": int((counts > 0).sum())}
    res["tc_grad_rel_err_vs_plain"] = _grad_err_tc_vs_plain(scene, vf, vd, W, o, d, t, target)
    # CUDA graph of the batched tensor-core step
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        for _ in range(2):
            vf.grad = vd.grad = W.grad = None
            step_batched(snisr.FORM_TC)
    stream.wait_stream(side)
    torch.cuda.synchronize()
    vf.grad = vd.grad = W.grad = None
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step_batched(snisr.FORM_TC)
    for _ in range(warmup):
        graph.replay()
    torch.cuda.synchronize()
    total = 0.0
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        graph.replay()
        e1.record(stream)
        torch.cuda.synchronize()
        total += e0.elapsed_time(e1)
    scene.check()
    ms_g = total / steps
    res["tc_batched_graph"] = {"value": round(n / ms_g / 1e3, 3), "ms_per_step": round(ms_g, 4)}
    res["speedup_batched_vs_per_tile"] = round(ms_pt / ms, 3)
    res["speedup_tc_vs_plain"] = round(ms_pl / ms, 3)
    res["speedup_tc_graph_vs_plain_per_tile_calls"] = round(ms_ppt / ms_g, 3)
    res["l2"] = "flushed before each step"
    del graph
    scene.close()
    return res


SMALL_WORKLOAD = ("cfg1 plain forward render, small: one tile of 64^3 over 2 m (room SDF: floor, two walls, 3 boxes), "
                  "FP32 16-dim corner features, MLP 43-32-32-3, 256x256 at 60 deg, 8 seeded poses, no proxy mesh "
                  "(rays start at the tile entry)")


def small_bench(dev, steps: int, warmup: int, flush, cpu: bool = True):
    """cfg1: the small single-tile scene, both GPU forms, and the scalar host
    path on whole 256x256 frames with its core count."""
    import torch

    import snisr
    cfg = snisr.CFG1
    synth = snisr.SynthScene(cfg)
    scene = snisr.Scene(synth.desc, dev.index)
    n = cfg.width * cfg.height
    cams = [synth.camera(p) for p in range(cfg.poses)]
    out = (torch.empty(n, 3, device=dev), torch.empty(n, device=dev), torch.empty(n, device=dev))
    stream = torch.cuda.current_stream()
    res = {"workload": SMALL_WORKLOAD, "unit": UNIT, "occupancy": round(synth.occupancy_fraction(), 4)}
    for name, form in (("tc", snisr.FORM_TC), ("plain_fp32", snisr.FORM_PLAIN_FP32)):
        for i in range(warmup):
            scene.render(cams[i % len(cams)], form, out)
        scene.check()
        torch.cuda.synchronize()
        total = 0.0
        for i in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            scene.render(cams[i % len(cams)], form, out)
            e1.record(stream)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        scene.check()
        res[name] = {"value": round(n * steps / (total * 1e-3) / 1e6, 3), "ms_per_step": round(total / steps, 4)}
    if cpu:
        threads = os.cpu_count() or 1
        hp = HostPath(synth, threads)
        hp.run(0, None)  # warm-up
        t0 = time.perf_counter()
        rays = sum(hp.run(p, None) for p in range(cfg.poses))
        dt = time.perf_counter() - t0
        res["cpu_scalar"] = {"value": round(rays / dt / 1e6, 4), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{cfg.poses} whole 256x256 frames, FP32 scalar oracle, {threads} threads"}
    scene.close()
    return res


LARGE_WORKLOAD = ("cfg5 large-scene full-frame render 1920x1080, 75 deg: 8x8x2 tiles of 128^3 over 24x24x6 m "
                  "(multi-room, 300 boxes), 4.2% occupied, FP16 32-dim corner features, per-tile FP16 MLP 59-64x3-3, "
                  "~1.0M-triangle proxy BVH, 16 seeded poses")


def large_scene_bench(dev, steps: int, warmup: int, flush):
    """cfg5: tensor-core and plain FP32 renders of 1920x1080 frames."""
    import torch

    import snisr
    cfg = snisr.CFG5
    synth = snisr.SynthScene(cfg)
    scene = snisr.Scene(synth.desc, dev.index)
    n = cfg.width * cfg.height
    cams = [synth.camera(p) for p in range(cfg.poses)]
    out = (torch.empty(n, 3, device=dev), torch.empty(n, device=dev), torch.empty(n, device=dev))
    tuning, _ = scene.autotune_render(cams[0], reps=2)
    stream = torch.cuda.current_stream()

    def timed(form, k):
        for i in range(warmup):
            scene.render(cams[i % len(cams)], form, out)
        scene.check()
        torch.cuda.synchronize()
        total = 0.0
        for i in range(k):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            scene.render(cams[i % len(cams)], form, out)
            e1.record(stream)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        scene.check()
        return total / k

    ms = timed(snisr.FORM_TC, steps)
    ms_pl = timed(snisr.FORM_PLAIN_FP32, max(2, steps // 8))
    info = scene.info
    res = {"workload": LARGE_WORKLOAD, "unit": UNIT, "tuning": tuning,
           "tc": {"value": round(n / ms / 1e3, 3), "ms_per_step": round(ms, 4), "fps": round(1e3 / ms, 2)},
           "plain_fp32": {"value": round(n / ms_pl / 1e3, 3), "ms_per_step": round(ms_pl, 4)},
           "speedup_tc_vs_plain": round(ms_pl / ms, 3), "l2": "flushed before each frame",
           "scene": {"voxels": int(info.num_voxels), "triangles": int(info.num_triangles),
                     "device_gb": round(info.device_bytes / 1e9, 2)}}
    scene.close()
    return res


SPEC_WORKLOAD = ("specular pass of a 1280x720 frame at reflection scale 2 (640x360 pixels): batching by network "
                 "(sort_by_key, assign_pixels), then 4 steps of 16 inverse-z samples -> per-group reflection MLP "
                 "63-64x5-28 with SH degree 2 (16 groups) -> compositing; seeded synthetic networks and rays")
SPEC_FLOP_PER_SAMPLE = 2 * (63 * 64 + 4 * 64 * 64 + 64 * 28)  # 44,416


def specular_bench(dev, steps: int, warmup: int, flush):
    """The reference's specular pass through the drop-in ops (FRender.render's
    loop, rendering/src/__init__.py:276-320)."""
    import numpy as np
    import torch

    from snisr import ops
    from snisr import spec_synth as sp
    P = sp.problem(seed=7, G=16, H=360, W=640)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    npix, spr = P["npix"], P["spr"]
    net0, rays_d, origin = T(P["net"]), T(P["rays_d"]), T(P["origin"])
    inv_near, centers, params = T(P["inv_near"]), T(P["centers"]), T(P["params"])
    inv_bound = T(((1.0 / (1.0 / P["inv_near"] + P["far"]) - P["inv_near"]) / 63).astype(np.float32))
    trans0 = T(P["transparency"])
    samples = torch.empty(npix, spr, 3, device=dev)
    isteps = torch.empty(npix, spr, device=dev)
    results = torch.zeros(npix, spr, 4, device=dev)
    frame = torch.zeros(npix, 3, device=dev)
    trans = torch.empty_like(trans0)
    stream = torch.cuda.current_stream()
    ev_mlp = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(4)]

    def frame_pass(record_mlp=False):
        keys = net0.clone()
        q = torch.arange(npix, dtype=torch.int32, device=dev)
        ps = torch.arange(npix, dtype=torch.int32, device=dev)
        num_net = ops.sort_by_key(keys, q, ps)
        end = torch.full((1,), npix, dtype=torch.int32, device=dev)
        counts = torch.cat([ps[1:num_net], end]) - ps[:num_net]
        bs = torch.cat([torch.zeros(1, dtype=torch.int32, device=dev), torch.cumsum(torch.ceil(counts / 64), 0).int()])
        nb = int(bs[-1])
        new_net = torch.empty(nb, dtype=torch.int16, device=dev)
        new_ps = torch.empty(nb, dtype=torch.int32, device=dev)
        ops.assign_pixels(keys[:num_net].contiguous(), torch.cat([ps[:num_net], end]), bs, 0, new_net, new_ps)
        new_ps = torch.cat([new_ps, end])
        trans.copy_(trans0)
        frame.zero_()
        for k, step in enumerate(range(0, 64, spr)):
            results.zero_()
            ops.inverse_z_sampling(origin, rays_d, inv_near, inv_bound, 0, step, spr, samples, isteps)
            if record_mlp:
                ev_mlp[k][0].record(stream)
            ops.inference_mlp(spr, nb, 0, float(P["inverse_far"]), float(P["trans_stop"]), new_net, trans, q, new_ps,
                              centers, samples, rays_d, params, results)
            if record_mlp:
                ev_mlp[k][1].record(stream)
            ops.integrate_points(results, isteps, 0, float(P["trans_stop"]), trans, frame)

    for _ in range(warmup):
        frame_pass()
    torch.cuda.synchronize()
    ops.check_errors()
    # samples the MLP evaluates: pixels with a network whose initial transmittance
    # passes the stop, 64 each (an upper bound: early-stopped pixels drop out later)
    live = int(((trans0 >= float(P["trans_stop"])) & (net0 >= 0)).sum()) * 64
    total = mlp_ms = 0.0
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        frame_pass(record_mlp=True)
        e1.record(stream)
        torch.cuda.synchronize()
        total += e0.elapsed_time(e1)
        mlp_ms += sum(a.elapsed_time(b) for a, b in ev_mlp)
    ops.check_errors()
    ms, mlp = total / steps, mlp_ms / steps
    _, tc_peak, kind = _peaks()
    tflops = live * SPEC_FLOP_PER_SAMPLE / (mlp * 1e-3) / 1e12
    return {"workload": SPEC_WORKLOAD, "unit": "Mpixels/s", "value": round(npix / ms / 1e3, 3),
            "ms_per_step": round(ms, 4), "mlp_ms_per_frame": round(mlp, 4),
            "mlp_samples_per_frame_upper_bound": live,
            "mlp_tflops": round(tflops, 2), "mlp_tensor_frac": round(tflops / tc_peak, 4),
            "note": "samples counted with the initial transmittance (an upper bound on the live samples)",
            "l2": "flushed before each frame"}


PIPE_WORKLOAD = ("the reference's whole frame (FRender.render, rendering/src/__init__.py:247-334) through the drop-in "
                 "ops at 1280x720: compute_rays -> tracing_tiles -> FP16 octree diffuse renderer on renderData format "
                 "(16 tiles of 64^3, converted synthetic scene) -> specular pass at reflection scale 2 (batching, "
                 "4 x [inverse-z sampling, reflection MLP, compositing]) -> bilinear upsampling -> clamp(diffuse + "
                 "specular); no CNN")


def reference_pipeline_bench(dev, steps: int, warmup: int, flush):
    """The reference renderer's per-frame op chain on this library's drop-ins."""
    import numpy as np
    import torch
    import torch.nn.functional as F

    import snisr
    from snisr import octree, ops
    cfg = snisr.CFG2.replace(res=64, with_mesh=False)
    synth = snisr.SynthScene(cfg)
    data = octree.from_synth(synth, groups=synth.desc.num_tiles, seed=5)
    T = octree.to_device(data, dev)
    der = octree.derived(data)
    cams = [synth.camera(p) for p in range(cfg.poses)]
    H, W, K = cfg.height, cfg.width, 30
    DH, DW = H // 2, W // 2
    far = der["far"]
    scene_size = torch.tensor(der["scene_size"], dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]

    def frame(cam, record=False):
        intr = torch.tensor([cam.cx, cam.cy, cam.inv_focal], dtype=torch.float32, device=dev)
        rot = torch.tensor([[cam.c2w[0], cam.c2w[1], cam.c2w[2]], [cam.c2w[4], cam.c2w[5], cam.c2w[6]],
                            [cam.c2w[8], cam.c2w[9], cam.c2w[10]]], dtype=torch.float32, device=dev)
        origin = torch.tensor([cam.c2w[3], cam.c2w[7], cam.c2w[11]], dtype=torch.float32, device=dev)
        if record:
            ev[0].record(stream)
        rays_d = torch.full((H, W, 3), -1.0, device=dev)
        visited = torch.full((H, W, K), -1, dtype=torch.int32, device=dev)
        diffuse = torch.full((H, W, 3), -1.0, device=dev)
        inv_near = torch.full((H, W), 1e-8, device=dev)
        net = torch.full((H, W), -1, dtype=torch.int16, device=dev)
        ops.compute_rays(intr, rot, 0, rays_d)
        ops.tracing_tiles(rays_d, T["tile_IndexMap"], origin, T["tile_shape"], T["scene_min_corner"], scene_size,
                          der["tile_size"], 0, visited)
        ops.rendering_diffuse_octree_fp16(rays_d, visited, origin, T["tile2group"], T["data_voxels"],
                                          T["block_IndexMap"], T["nodes_IndexMap"], T["nodes_sampleFlag"],
                                          T["voxels_start"], T["centers"], der["tile_size"], der["voxel_size"],
                                          der["sample_step"], der["block_num_voxel"], 256, 0.8, 0.01, False,
                                          diffuse, inv_near, net)
        if record:
            ev[1].record(stream)
        inv_s = inv_near[::2, ::2].contiguous()
        net_s = net[::2, ::2].flatten().contiguous()
        rays_s = rays_d[::2, ::2].contiguous()
        npix = DH * DW
        q = torch.arange(npix, dtype=torch.int32, device=dev)
        ps = torch.arange(npix, dtype=torch.int32, device=dev)
        num_net = ops.sort_by_key(net_s, q, ps)
        end = torch.full((1,), npix, dtype=torch.int32, device=dev)
        counts = torch.cat([ps[1:num_net], end]) - ps[:num_net]
        bs = torch.cat([torch.zeros(1, dtype=torch.int32, device=dev), torch.cumsum(torch.ceil(counts / 64), 0).int()])
        nb = int(bs[-1])
        new_net = torch.empty(nb, dtype=torch.int16, device=dev)
        new_ps = torch.empty(nb, dtype=torch.int32, device=dev)
        ops.assign_pixels(net_s[:num_net].contiguous(), torch.cat([ps[:num_net], end]), bs, 0, new_net, new_ps)
        new_ps = torch.cat([new_ps, end])
        sample_far = 1.0 / inv_s + far
        inv_bound = ((1.0 / sample_far - inv_s) / 63).contiguous()
        trans = torch.ones(DH, DW, 1, device=dev)
        spec = torch.zeros(DH, DW, 3, device=dev)
        for step in range(0, 64, 16):
            res = torch.zeros(DH, DW, 16, 4, device=dev)
            pts = torch.full((DH, DW, 16, 3), -1.0, device=dev)
            isteps = torch.zeros(DH, DW, 16, device=dev)
            ops.inverse_z_sampling(origin, rays_s, inv_s, inv_bound, 0, step, 16, pts, isteps)
            ops.inference_mlp(16, nb, 0, 1.0 / far, 0.01, new_net, trans, q, new_ps, T["group_centers"], pts, rays_s,
                              T["net_params"], res)
            ops.integrate_points(res, isteps, 0, 0.01, trans, spec)
        spec_up = F.interpolate(spec[None].permute(0, 3, 1, 2), scale_factor=2, mode="bilinear",
                                align_corners=True)[0].permute(1, 2, 0)
        final = torch.clamp(diffuse + spec_up, 0, 1)
        if record:
            ev[2].record(stream)
        return final

    for i in range(warmup):
        frame(cams[i % len(cams)])
    torch.cuda.synchronize()
    ops.check_errors()
    total = diff_ms = 0.0
    for i in range(steps):
        flush.zero_()
        frame(cams[i % len(cams)], record=True)
        torch.cuda.synchronize()
        total += ev[0].elapsed_time(ev[2])
        diff_ms += ev[0].elapsed_time(ev[1])
    ops.check_errors()
    ms = total / steps
    return {"workload": PIPE_WORKLOAD, "unit": "FPS", "value": round(1e3 / ms, 2), "ms_per_step": round(ms, 4),
            "diffuse_ms": round(diff_ms / steps, 4), "mrays_s": round(H * W / ms / 1e3, 3),
            "note": "includes sort_by_key's host synchronisation (it returns a count, as the reference's op does)",
            "l2": "flushed before each frame"}


PRUNE_WORKLOAD = ("occupancy pruning of one 128^3 tile of the 4x4x1-tile scene after an epoch (Tile.pruning, "
                  "training/scripts/tile/tile.py:297-395): transparency statistic of every camera ray of 8 "
                  "1280x720 views that crosses the tile (step 0.1 voxel), 3^3 max filter + block-maximum "
                  "thresholds (initial flags = the current occupancy) + border dilation, packing into occupancy "
                  "words")


def pruning_bench(dev, steps: int, warmup: int, flush):
    """Tile.pruning's device work on one tile: rays resident in HBM."""
    import time

    import numpy as np
    import torch

    import oracle
    import snisr
    from snisr import ops, prune
    from snisr.scene import camera_rays
    s = snisr.SynthScene(snisr.CFG2)
    a = s.arrays()
    t = 5
    sig_d, vsig, flags = prune.grids_from_arrays(s.desc, a, t)
    center_np = prune.tile_centers(s.desc, a)[t]
    tile = float(s.desc.tile_size)
    N = int(s.desc.res)
    D = N + 2
    vs = tile / N
    step = vs * 0.1
    c = torch.from_numpy(center_np).to(dev)
    ro, rd = [], []
    for v in range(8):
        cam = s.camera(v)
        d = camera_rays(cam, dev.index or 0).reshape(-1, 3)
        o = torch.tensor([cam.c2w[3], cam.c2w[7], cam.c2w[11]], dtype=torch.float32, device=dev).expand_as(d)
        inv = 1.0 / d
        t0, t1 = (c - tile / 2 - o) * inv, (c + tile / 2 - o) * inv
        lo = torch.minimum(t0, t1).nan_to_num(-1e30).amax(1)
        hi = torch.maximum(t0, t1).nan_to_num(1e30).amin(1)
        keep = hi > lo.clamp_min(0)
        ro.append(o[keep].contiguous())
        rd.append(d[keep].contiguous())
    ro, rd = torch.cat(ro).contiguous(), torch.cat(rd).contiguous()
    nrays = ro.shape[0]
    init = np.where(flags[1:-1, 1:-1, 1:-1] == 1, 1, -1).astype(np.int16)  # the current occupancy
    sig_t, vsig_t, flags_t, init_t = (torch.from_numpy(x).to(dev) for x in (sig_d, vsig, flags, init))
    T = torch.zeros(D, D, D, dtype=torch.float32, device=dev)
    out = torch.empty_like(flags_t)
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]

    def once(record=False):
        T.zero_()
        if record:
            ev[0].record(stream)
        ops.transparency_statistic(ro, rd, D, c, tile, vs, step, sig_t, flags_t, T)
        if record:
            ev[1].record(stream)
        ops.prune_flags(T, vsig_t, init_t, 4, 0.5, 0.01, out)
        w, n = ops.pack_occupancy(out)
        if record:
            ev[2].record(stream)
        return n

    for _ in range(warmup):
        once()
    torch.cuda.synchronize()
    tot = st = 0.0
    for _ in range(steps):
        flush.zero_()
        n = once(True)
        torch.cuda.synchronize()
        tot += ev[0].elapsed_time(ev[2])
        st += ev[0].elapsed_time(ev[1])
    kept = int(n)
    # CPU: the oracle's statistic (one thread) on a bounded sample of the rays
    k = min(nrays, 20000)
    idx = torch.linspace(0, nrays - 1, k, device=dev).long()
    o_s, d_s = ro[idx].cpu().numpy(), rd[idx].cpu().numpy()
    ref = np.zeros((D, D, D), np.float32)
    t0 = time.perf_counter()
    oracle.op_transparency_statistic(o_s, d_s, D, center_np, tile, vs, step, sig_d, flags, ref)
    cpu_s = time.perf_counter() - t0
    ms = tot / steps
    return {"workload": PRUNE_WORKLOAD, "unit": "Mrays/s", "value": round(nrays / ms / 1e3, 2),
            "ms_per_step": round(ms, 4), "statistic_ms": round(st / steps, 4), "rays": nrays,
            "voxels_before": int((flags == 1).sum()), "voxels_after": kept,
            "cpu_oracle": {"value": round(k / cpu_s / 1e6, 3), "unit": "Mrays/s", "cores": 1,
                           "sample": f"{k} of the rays, transparency statistic only"},
            "l2": "flushed before each step"}


PREP_WORKLOAD = ("training-data preparation of one tile of the 4x4x1-tile scene (get_trainData_v3, "
                 "training/src/cuda_func.cu:1341-1686) per 1280x720 view: training rays, tile DDA, two nearest hits "
                 "of the 207k-triangle proxy mesh per visited tile (BVH), background depth and validity, diffuse "
                 "estimate from 16 selected views (projection + depth test), 7x7 patch rows; images seeded noise, "
                 "depth maps from the proxy mesh")


def trainprep_bench(dev, steps: int, warmup: int, flush):
    """Per-view chain of get_trainData_v3 on resident images and depths."""
    import time

    import numpy as np
    import torch

    import oracle
    import snisr
    from snisr import trainprep
    s = snisr.SynthScene(snisr.CFG2)
    a = s.arrays()
    d = s.desc
    sc = snisr.Scene(d)
    H, W, M, KT, P = 720, 1280, 16, 30, 7
    Ks, C2Ws = [], []
    for v in range(M):
        cam = s.camera(v, W, H)
        f = 1.0 / cam.inv_focal
        Ks.append(np.array([f, 0, cam.cx, 0, f, cam.cy, 0, 0, 1], np.float32))
        C2Ws.append(np.array(list(cam.c2w), np.float32))
    Ks, C2Ws = np.stack(Ks), np.stack(C2Ws)
    rng = np.random.default_rng(3)
    images = torch.from_numpy(rng.random((M, H * W, 3), dtype=np.float32)).to(dev)
    depths = torch.empty(M, H * W, device=dev)
    imap = np.asarray(a["tile_index"], np.int32).reshape(-1)
    grid = (int(d.grid[0]), int(d.grid[1]), int(d.grid[2]))
    smin = np.array(list(d.scene_min), np.float32)
    tp = trainprep.TrainPrep(sc, H, W, imap, grid, smin, float(d.tile_size), KT, P, device=dev.index)
    Kt = [torch.from_numpy(Ks[j].copy()).to(dev) for j in range(M)]
    Ct = [torch.from_numpy(C2Ws[j].copy()).to(dev) for j in range(M)]
    for j in range(M):  # depth maps: proxy-mesh first hits along the training rays (camera z)
        from snisr import _lib
        _lib.check(_lib.lib().snisr_op_train_rays(Kt[j].data_ptr(), Ct[j].data_ptr(), H, W, tp.ro.data_ptr(),
                                                  tp.rd.data_ptr(), torch.cuda.current_stream().cuda_stream))
        t, _ = sc.proxy_hit(tp.ro, tp.rd)
        depths[j] = torch.where(t > 0, t, torch.full_like(t, 1e4))
    proj = torch.from_numpy(np.stack([trainprep.project_matrix(Ks[j], C2Ws[j]) for j in range(M)])).to(dev)
    origins = torch.from_numpy(C2Ws[:, [3, 7, 11]].copy()).to(dev)
    train_tile = 5
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for i in range(warmup):
        tp.view(train_tile, Kt[i % M], Ct[i % M], images[i % M], origins, images, depths, proj)
    torch.cuda.synchronize()
    tot, patches = 0.0, 0
    for i in range(steps):
        j = i % M
        flush.zero_()
        e0.record(stream)
        rows, count = tp.view(train_tile, Kt[j], Ct[j], images[j], origins, images, depths, proj)
        e1.record(stream)
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
        patches += int(count)
    sc.check()
    ms = tot / steps
    # CPU: the oracle chain on a 160x90 view (double hits and diffuse on 16 threads)
    h, w = 90, 160
    t0 = time.perf_counter()
    ro, rd = oracle.train_rays(Ks[0] * np.array([w / W, 1, w / W, 1, h / H, h / H, 1, 1, 1], np.float32),
                               C2Ws[0], h, w)
    vis = oracle.train_tracing(ro, rd, imap, grid, smin, float(d.tile_size), KT)
    osc = oracle.OracleScene(d)
    hits = osc.double_hits(ro, rd, vis)
    oracle.train_bgdepth(train_tile, vis, hits)
    cpu_s = time.perf_counter() - t0
    sc.close()
    return {"workload": PREP_WORKLOAD, "unit": "views/s", "value": round(1e3 / ms, 2), "ms_per_step": round(ms, 4),
            "mrays_s": round(H * W / ms / 1e3, 2), "patches_per_view": round(patches / steps, 1),
            "cpu_oracle": {"value": round(h * w / cpu_s / 1e6, 4), "unit": "Mrays/s", "cores": oracle.threads(),
                           "sample": f"one {w}x{h} view: rays, tile DDA, double hits, background depth"},
            "l2": "flushed before each view"}


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import snisr
    snisr.lib()
    synth = snisr.SynthScene(snisr.CFG2)
    threads = os.cpu_count() or 1
    cb = cpu_baseline_run(synth, args.steps, 60.0, threads, warmup=args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": "scalar CPU path (oracle port of the reference method)"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--max-samples-per-ray", type=int, default=48)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-train", action="store_true")
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--profile-run", choices=["render", "train", "batched", "large", "specular", "pipeline",
                                              "pruning", "trainprep", "small"],
                    default=None,
                    help="render: a few frames of both forms (small workspace); train: a few training steps of "
                         "both forms (for ncu captures)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return

    import numpy as np
    import torch

    import snisr
    snisr.build()
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.profile_run in ("train", "batched", "large", "specular", "pipeline", "pruning", "trainprep", "small"):
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
        fn = {"train": train_bench, "batched": batched_bench, "large": large_scene_bench,
              "specular": specular_bench, "pipeline": reference_pipeline_bench,
              "pruning": pruning_bench, "trainprep": trainprep_bench, "small": small_bench}[args.profile_run]
        res = fn(dev, args.steps, args.warmup, flush)
        print(json.dumps({"profile_run": args.profile_run, args.profile_run: res}))
        return
    cfg = snisr.CFG2
    synth = snisr.SynthScene(cfg, max_samples_per_ray=args.max_samples_per_ray)
    scene = snisr.Scene(synth.desc, local)
    W, H = cfg.width, cfg.height
    n = W * H
    cams = [synth.camera(p) for p in rank_poses(rank, cfg.poses)]
    stream = torch.cuda.current_stream()
    out = (torch.empty(n, 3, device=dev), torch.empty(n, device=dev), torch.empty(n, device=dev))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2

    if args.profile_run == "render":
        for i in range(args.warmup + args.steps):
            scene.render(cams[i % len(cams)], snisr.FORM_TC, out)
        scene.render(cams[0], snisr.FORM_PLAIN_FP32, out)
        scene.check()
        torch.cuda.synchronize()
        print(json.dumps({"profile_run": "ok", "frames": args.warmup + args.steps}))
        scene.close()
        return

    def timed(form, steps, warmup):
        for i in range(warmup):
            scene.render(cams[i % len(cams)], form, out)
        scene.check()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        _barrier(ws)
        torch.cuda.synchronize()
        for i in range(steps):
            flush.zero_()
            evs[i][0].record(stream)
            scene.render(cams[i % len(cams)], form, out)
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        _barrier(ws)
        scene.check()
        return sum(a.elapsed_time(b) for a, b in evs)

    # launch shapes chosen by the library's autotuner on the first pose
    tuning, tune_ms = scene.autotune_render(cams[0], reps=3)
    # headline: tensor-core batched form
    with ClockSampler(local) as clk:
        ms_tc = timed(snisr.FORM_TC, args.steps, args.warmup)
    clocks = clk.summary()
    ms_tc = _max_over_ranks(ws, ms_tc)
    value = job_value(ws, n, args.steps, ms_tc)
    # plain FP32 form (the >= 2x target's denominator)
    plain_steps = min(24, max(4, args.steps // 3))
    ms_plain = _max_over_ranks(ws, timed(snisr.FORM_PLAIN_FP32, plain_steps, 3))
    plain_value = job_value(ws, n, plain_steps, ms_plain)

    # stages and counters of the TC form, averaged over the poses
    scene.set_profiling(True)
    stage_sum = None
    stats_sum = {"samples": 0, "voxel_steps": 0, "chunks": 0, "voxels": 0, "vertices": 0}
    prof_steps = min(args.steps, 16)
    for i in range(prof_steps):
        flush.zero_()
        scene.render(cams[i % len(cams)], snisr.FORM_TC, out)
        st = scene.stage_times()
        stage_sum = st if stage_sum is None else [a + b for a, b in zip(stage_sum, st)]
        fs = {**scene.frame_stats(), **scene.frame_footprint()}
        for k in stats_sum:
            stats_sum[k] += fs[k]
    scene.set_profiling(False)
    npose = prof_steps
    stages = dict(zip(["raygen_proxy", "traverse", "scan", "scatter", "mlp_tc", "total"],
                      [round(v / npose, 4) for v in stage_sum]))
    samples = stats_sum["samples"] / npose
    vsteps = stats_sum["voxel_steps"] / npose
    chunks = stats_sum["chunks"] / npose
    dvox = stats_sum["voxels"] / npose
    dvert = stats_sum["vertices"] / npose

    hbm, tc_peak, peak_kind = _peaks()
    # The dominant kernel of the frame is the MLP stage (mlp_tc_kernel): its
    # algorithmic work per launch (one frame) is
    #   FLOP: 24,320 per sample (59-64x3-3 MLP, forward only);
    #   compulsory bytes: every distinct trilinear corner of the frame once
    #     (32 FP16 features + FP16 density), every 16-byte sample record once,
    #     every ray's 64-byte view encoding and 12 bytes of colour once, every
    #     tile's 36,864-byte weight image once.
    # roofline.frac is the larger of the tensor and compulsory-HBM fractions.
    # The "gather model" (every sample's 8 corners counted as DRAM bytes, one
    # weight image per 128-sample chunk) ignores on-chip reuse; it is reported
    # as a side figure only and can exceed the copy peak.
    img = TC_IMAGE_BYTES
    mlp_flop = samples * MLP_FLOP_PER_SAMPLE
    mlp_bytes_compulsory = (dvert * (32 + 1) * 2 + samples * SAMPLE_RECORD_BYTES + n * (64 + 12)
                            + synth.desc.num_tiles * img)
    mlp_bytes_gather = samples * (GATHER_BYTES_PER_SAMPLE + SAMPLE_RECORD_BYTES + 64 + 12) + chunks * img
    t_mlp = stages["mlp_tc"] * 1e-3
    tflops = mlp_flop / t_mlp / 1e12
    gbs = mlp_bytes_compulsory / t_mlp / 1e9
    f_tc, f_hbm = tflops / tc_peak, gbs / hbm
    if f_tc >= f_hbm:
        roof = {"bound": "tensor", "achieved": tflops, "peak": tc_peak, "unit": "TFLOP/s", "frac": f_tc}
    else:
        roof = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": f_hbm}
    traffic = NCU_DRAM_BYTES_PER_LAUNCH.get("mlp_tc")
    roof.update({
        "kernel": "mlp_tc_kernel", "launch_ms": round(t_mlp * 1e3, 4),
        "tensor": {"flop": int(mlp_flop), "tflops": round(tflops, 2), "frac": round(f_tc, 4)},
        "hbm_compulsory": {"bytes": int(mlp_bytes_compulsory), "gbs": round(gbs, 1), "frac": round(f_hbm, 4),
                           "distinct_vertices": int(dvert), "distinct_voxels": int(dvox)},
        "gather_model_side_figure": {"bytes": int(mlp_bytes_gather),
                                     "gbs": round(mlp_bytes_gather / t_mlp / 1e9, 1),
                                     "note": "every sample's 8 corners counted as DRAM bytes; L2 and L1 reuse make "
                                             "this exceed the copy peak, so it is not the roofline"},
        "peak_source": ("measured (MEASURED_PEAKS.json: hbm_gbs, bf16_tflops burst)" if peak_kind == "measured"
                        else "fallback (6.8 TB/s, 1.9 PFLOP/s)"),
        "traffic": traffic["bytes"] if traffic else None,
        "traffic_over_compulsory": (round(traffic["bytes"] / mlp_bytes_compulsory, 3) if traffic else None),
        "traffic_source": traffic["source"] if traffic else None,
    })
    for k in ("achieved", "frac"):
        roof[k] = round(roof[k], 4)

    # end to end through the C ABI with host (pinned) output buffers
    e2e = None
    if not args.no_e2e:
        rgb_h = torch.empty(n, 3, pin_memory=True)
        dep_h = torch.empty(n, pin_memory=True)
        op_h = torch.empty(n, pin_memory=True)
        for i in range(3):
            scene.render_host(cams[i], snisr.FORM_TC, rgb_h, dep_h, op_h)
        _barrier(ws)
        t0 = time.perf_counter()
        e2e_steps = min(args.steps, 200)
        for i in range(e2e_steps):
            scene.render_host(cams[i % len(cams)], snisr.FORM_TC, rgb_h, dep_h, op_h)
        t_sync = _max_over_ranks(ws, time.perf_counter() - t0)
        _barrier(ws)
        # pipelined: frame i's device->host copies overlap frame i+1's render;
        # every frame is still copied to (alternating) pinned host buffers
        hb = [(rgb_h, dep_h, op_h),
              (torch.empty(n, 3, pin_memory=True), torch.empty(n, pin_memory=True), torch.empty(n, pin_memory=True))]
        for i in range(3):
            scene.render_host_async(cams[i], snisr.FORM_TC, *hb[i % 2])
        scene.render_host_wait()
        _barrier(ws)
        t0 = time.perf_counter()
        for i in range(e2e_steps):
            scene.render_host_async(cams[i % len(cams)], snisr.FORM_TC, *hb[i % 2])
        scene.render_host_wait()
        t_e2e = _max_over_ranks(ws, time.perf_counter() - t0)
        _barrier(ws)
        e2e = {"value": round(ws * n * e2e_steps / t_e2e / 1e6, 3), "unit": UNIT, "steps": e2e_steps,
               "h2d_bytes_per_step": 68, "d2h_bytes_per_step": n * 20,
               "path": "snisr_render_host_async (camera by value -> device; rgb/depth/opacity -> pinned host, "
                       "copies of frame i overlapping the render of frame i+1; timed to the last copy)",
               "synchronous": {"value": round(ws * n * e2e_steps / t_sync / 1e6, 3),
                               "path": "snisr_render_host (render, copy, synchronise per frame)"}}

    train = batched = large = None
    small = small_bench(dev, min(40, max(4, args.steps // 4)), 3, flush, cpu=rank == 0 and not args.no_cpu_baseline)
    if not args.no_train:
        train = train_bench(dev, min(40, max(4, args.steps // 2)), args.warmup, flush)
        batched = batched_bench(dev, min(10, max(3, args.steps // 4)), 3, flush)
    if not args.no_large:
        large = large_scene_bench(dev, min(32, max(4, args.steps // 4)), 3, flush)
    specular = specular_bench(dev, min(20, max(3, args.steps // 10)), 3, flush)
    pipeline = reference_pipeline_bench(dev, min(20, max(3, args.steps // 10)), 3, flush)
    pruning = pruning_bench(dev, min(20, max(3, args.steps // 10)), 3, flush)
    prep = trainprep_bench(dev, min(16, max(3, args.steps // 10)), 3, flush)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_run(synth, 8, 15.0, os.cpu_count() or 1)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_tc / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f16", "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": "tensor-core batched (tcgen05 FP16, FP32 accumulate)",
                       "tuning": tuning, "autotune_ms_per_frame": round(tune_ms, 4),
                       "l2": "flushed between steps (256 MB write)", "poses": cfg.poses,
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "fps": round(value / (n / 1e6) / ws, 2),
            "plain_fp32": {"value": round(plain_value, 3), "unit": UNIT,
                           "ms_per_step": round(ms_plain / plain_steps, 4), "steps": plain_steps},
            "speedup_vs_plain": round(value / plain_value, 3),
            "stages_ms": stages,
            "frame_counters": {"samples": int(samples), "voxel_steps": int(vsteps), "mlp_chunks": int(chunks),
                               "distinct_voxels": int(dvox), "distinct_vertices": int(dvert)},
            "roofline": roof,
            "clocks": clocks,
            "gpu_launches": 5 * args.steps,
            "e2e": e2e,
            "small_scene": small,
            "train": train,
            "train_batched": batched,
            "large_scene": large,
            "specular_pass": specular,
            "reference_pipeline": pipeline,
            "pruning": pruning,
            "train_prep": prep,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    scene.close()


if __name__ == "__main__":
    main()
