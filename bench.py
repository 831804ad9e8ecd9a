#!/usr/bin/env python3
"""Mrays/s of the GB300 hair ray tracer: quantised and batched against plain FP32.

Default workload (c5_batched): 16 seeded hair models (strands log-uniform in [2,000, 200,000],
16-128 vertices, Phantom / LSS / DOTS in turn, 47.9 M segments in all), each with its own camera,
resolution (256x256 .. 1920x1080) and 1-4 jittered samples per pixel, Shade() plus one shadow ray
per hit. Quantised BLASes (8-bit BVH8 boxes; Phantom segments rebuilt from the strand vertex
stream), all scenes in one
CUDA-graph replay of the persistent trace kernel with autotuned settings. A step is one replay.
`value` counts primary + shadow rays per second with the BVHs resident in HBM (several GB, far
above the 129 MB L2, so no flush between steps); `plain_fp32` is the same scenes as 16
sequential launches of the FP32 tracer; `e2e` goes through the C ABI per step (cameras in,
every framebuffer copied to pinned host memory). `--config c4_phantom_quantised` is the single
Phantom precision-pattern frame (19.05 M segments, 1920x1080 x 4 spp) next to its FP32 build.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config NAME]

Under torchrun (N > 1) every rank renders its own full frame (replicas, weak scaling); rank 0
prints one JSON line. `--impl reference` times the CPU restatement of the reference's trace
path (oracle/, FP32, all host threads) on bounded samples of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s on 1 GB300: quantized/batched vs plain FP32 at >=99.99% hit agreement"
L2_BYTES = 129 * 1024 * 1024
PRECISION_DESC = ("quantised (8-bit BVH8 boxes; Phantom segments as 4-byte indices into the strand vertex stream, "
                  "control points rebuilt from the FP32 vertices in the leaf)")
DTYPE_DESC = "fp32 (8-bit node boxes)"
ORACLE_DESC = "FP64 CPU restatement on the original FP32 strands"


def prim_test_bytes(info, gtype: int, precision: int) -> int:
    """Bytes one primitive test reads: the record, and for quantised Phantom the four 16-byte
    stream entries it indexes."""
    return int(info["prim_bytes"]) + (64 if gtype == 0 and precision == 1 else 0)


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


class Dist:
    """Rank bookkeeping; torch.distributed only when WORLD_SIZE > 1."""

    def __init__(self):
        self.rank = env_int("RANK", 0)
        self.world = env_int("WORLD_SIZE", 1)
        self.local = env_int("LOCAL_RANK", 0)
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        dev = "cuda" if torch.cuda.is_available() else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # nvidia-smi's start-up (driver queries) would otherwise overlap the timed region: wait
        # for its first sample (at most 5 s)
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None and os.path.getsize(self.path) == 0:
            time.sleep(0.02)

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait(timeout=5)
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def load_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


_OVERRIDE = {}


def workload(name: str):
    import vkhrt_gb300 as H
    cfg = dict(H.CONFIGS[name])
    cfg.update(_OVERRIDE)
    sp = H.StrandParams(seed=cfg["seed"], nstrands=cfg["nstrands"], nverts=cfg["nverts"], r_root=cfg["r_root"],
                        r_tip=cfg["r_tip"])
    return cfg, sp


def uniform_lines(v, r, ns, nv):
    vv = v.reshape(ns, nv, 3)
    rr = r.reshape(ns, nv)
    lines = np.ascontiguousarray(np.concatenate([vv[:, :-1], vv[:, 1:]], axis=2).reshape(-1, 6), np.float32)
    lrad = np.ascontiguousarray(np.stack([rr[:, :-1], rr[:, 1:]], axis=2).reshape(-1, 2), np.float32)
    return lines, lrad


def oracle_scene(cfg, v, r, precision):
    """CPU oracle scene for the workload (the checker and the CPU baseline)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from hairscene import OracleScene, load_oracle, oracle_geometry
    orc = load_oracle()
    lines, lrad = uniform_lines(v, r, cfg["nstrands"], cfg["nverts"])
    data, rad = oracle_geometry(orc, int(cfg["type"]), lines, lrad, quantised=(precision == 1 and int(cfg["type"]) == 0))
    del lines, lrad
    return OracleScene(orc, [(int(cfg["type"]), data, rad)]), orc


def sample_pixels(w, h, n, seed=7):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(w * h, size=min(n, w * h), replace=False)).astype(np.uint32)


def cpu_sample_rate(osc, cam_arrays, cfg, precision, target_s=12.0, threads=0):
    """Rays/s of the oracle on a growing pixel sample until ~target_s of work; returns (Mrays/s, desc)."""
    vi, pi = cam_arrays
    w, h, spp = cfg["width"], cfg["height"], cfg["spp"]
    npx = 512
    while True:
        px = sample_pixels(w, h, npx, seed=npx)
        t0 = time.perf_counter()
        o = osc.render(vi, pi, w, h, spp=spp, jitter=1 if spp > 1 else 0, seed=17, shading=2, precision=precision,
                       pixel_list=px, threads=threads)
        dt = time.perf_counter() - t0
        rays = len(px) * spp + int((o["t"] >= 0).sum())
        if dt >= target_s or npx >= w * h:
            return rays / dt / 1e6, f"{len(px)} random pixels x {spp} spp (+{int((o['t'] >= 0).sum())} shadow rays)", dt
        npx = min(w * h, int(npx * max(2.0, min(8.0, target_s / max(dt, 1e-3)))))


def run_reference(args, dist):
    """CPU restatement of the reference's trace path (FP32 Prhi, all host threads)."""
    if dist.rank != 0:
        return
    if args.config == BATCH_CONFIG:
        return run_reference_batched(args)
    import vkhrt_gb300 as H
    cfg, sp = workload(args.config)
    v, r, off = H.generate_strands(sp)
    osc, orc = oracle_scene(cfg, v, r, int(cfg["precision"]))
    cam = H.scene_camera(cfg["width"], cfg["height"])
    vi, pi = H.camera_arrays(cam)
    threads = orc.orc_hardware_threads()
    w, h, spp = cfg["width"], cfg["height"], cfg["spp"]
    npx = args.ref_pixels
    rates = []
    total_t = 0.0
    total_rays = 0
    for step in range(args.warmup + args.steps):
        px = sample_pixels(w, h, npx, seed=1000 + step)
        t0 = time.perf_counter()
        o = osc.render(vi, pi, w, h, spp=spp, jitter=1 if spp > 1 else 0, seed=17, shading=2, precision=32,
                       pixel_list=px, threads=threads)
        dt = time.perf_counter() - t0
        rays = len(px) * spp + int((o["t"] >= 0).sum())
        if step >= args.warmup:
            total_t += dt
            total_rays += rays
            rates.append(rays / dt / 1e6)
    value = total_rays / total_t / 1e6
    sample = f"{npx} random pixels x {spp} spp per step (+ shadow rays)"
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total_t / max(args.steps, 1), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic: seeded strands (the reference's glTF hair assets are not available)",
            "config": config_block(cfg, args.config),
            "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_batched(args):
    """The oracle's FP32 tracer over every scene of the batched workload, a bounded pixel sample of
    each scene per step (all host threads)."""
    import vkhrt_gb300 as H
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from hairscene import OracleScene, load_oracle, oracle_geometry
    orc = load_oracle()
    threads = orc.orc_hardware_threads()
    models = batch_models(args)
    scenes = []
    for m, v, r, off in models:
        lines, lrad = uniform_lines(v, r, m["nstrands"], m["nverts"])
        data, rad = oracle_geometry(orc, int(m["type"]), lines, lrad, quantised=(int(m["type"]) == 0))
        cam = H.orbit_camera(m["width"], m["height"], m["azimuth"], m["elevation"])
        scenes.append((m, OracleScene(orc, [(int(m["type"]), data, rad)]), H.camera_arrays(cam)))
    # per step the same fraction of every scene's pixels (all their samples), so the rate is that
    # of the whole workload; 1/8 of the workload per step
    frac = 0.125
    total_t = 0.0
    total_rays = 0
    for step in range(args.warmup + args.steps):
        for m, osc, (vi, pi) in scenes:
            w, h, spp = m["width"], m["height"], m["spp"]
            px = sample_pixels(w, h, int(w * h * frac), seed=1000 + step)
            t0 = time.perf_counter()
            o = osc.render(vi, pi, w, h, spp=spp, jitter=1, seed=17, shading=2, precision=32, pixel_list=px,
                           threads=threads)
            dt = time.perf_counter() - t0
            if step >= args.warmup:
                total_t += dt
                total_rays += len(px) * spp + int((o["t"] >= 0).sum())
    value = total_rays / total_t / 1e6
    sample = (f"{pixel_share(frac)} of each of the {len(models)} scenes (all their samples, + shadow rays) per "
              f"step: the workload's mix")
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total_t / max(args.steps, 1), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic: seeded strands (the reference's glTF hair assets are not available)",
            "config": batch_config_block(models),
            "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_block(cfg, name):
    nseg = cfg["nstrands"] * (cfg["nverts"] - 1)
    return {"workload": f"{name}: {cfg['nstrands']} strands x {cfg['nverts']} vertices = {nseg} "
                        f"{'Bezier' if int(cfg['type']) == 0 else 'LSS' if int(cfg['type']) == 1 else 'DOTS'} segments, "
                        f"{cfg['width']}x{cfg['height']} x {cfg['spp']} spp, Shade + 1 shadow ray",
            "segments": nseg, "image": f"{cfg['width']}x{cfg['height']}", "spp": cfg["spp"],
            "precision": PRECISION_DESC if int(cfg["precision"]) else "fp32",
            "l2": "inputs larger than L2 (BVH + primitives resident, no flush)", "parallelism": "replicas"}


def time_frames(ctx, tlas, cam, frame, params, steps, warmup):
    import torch
    import vkhrt_gb300 as H
    for _ in range(warmup):
        H.trace(ctx, tlas, cam, frame, params)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        H.trace(ctx, tlas, cam, frame, params)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def run_ours(args, dist):
    import torch
    import vkhrt_gb300 as H
    dev = dist.local
    torch.cuda.set_device(dev)
    ctx = H.Context(dev)
    cfg, sp = workload(args.config)
    w, h, spp = cfg["width"], cfg["height"], cfg["spp"]
    t_gen = time.perf_counter()
    v, r, off = H.generate_strands(sp)
    t_gen = time.perf_counter() - t_gen
    # ---- build (untimed for `value`; reported) ----
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=cfg["type"], vertices=v, radius=r, strand_offsets=off, precision=cfg["precision"],
                    max_leaf=args.max_leaf), ctx)
    tlas = H.TopLevelAccelerationStructure([blas], ctx)
    build_wall = time.perf_counter() - t0
    cam = H.scene_camera(w, h)
    frame = H.Frame(ctx, w, h, spp, with_hits=True)
    params = H.trace_params(spp=spp, jitter=1, seed=17, shading=2, kernel_variant=args.variant, refill=args.refill, speculative=args.speculative, leaf_again=args.leaf_again, **{"async": 1})
    # rays per step (deterministic: fixed camera, jitter seed)
    H.trace(ctx, tlas, cam, frame, H.trace_params(spp=spp, jitter=1, seed=17, shading=2, count_stats=1,
                                                  kernel_variant=args.variant, refill=args.refill, speculative=args.speculative, leaf_again=args.leaf_again))
    st = frame.stats()
    rays_per_step = st["primary_rays"] + st["shadow_rays"]
    # ---- timed region ----
    dist.barrier()
    clocks = Clocks(dev)
    clocks.start()
    ms = time_frames(ctx, tlas, cam, frame, params, args.steps, args.warmup)
    clk = clocks.stop()
    ms_max = dist.max(ms)
    value = dist.world * rays_per_step / (ms_max * 1e-3) / 1e6
    if dist.rank != 0:
        dist.close()
        return
    info = blas.info
    # ---- roofline: algorithmic bytes per launch / launch time ----
    node_b = info["node_bytes"]
    prim_b = prim_test_bytes(info, int(cfg["type"]), int(cfg["precision"]))
    alg_bytes = st["nodes_visited"] * node_b + st["prims_tested"] * prim_b + w * h * 16
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                "bytes_per_launch": int(alg_bytes), "nodes_visited": int(st["nodes_visited"]),
                "prims_tested": int(st["prims_tested"]), "node_bytes": int(node_b), "prim_bytes": int(prim_b)}
    tot = st["warp_cycles_node"] + st["warp_cycles_leaf"] + st["warp_cycles_other"]
    phase = {k: round(st["warp_cycles_" + k] / tot, 4) for k in ("node", "leaf", "other")} if tot else None
    if args.profile:
        print(json.dumps({"profile": True, "ms_per_step": round(ms, 3), "rays_per_step": int(rays_per_step),
                          "value": round(value, 3), "roofline": roofline, "phase_share": phase}), flush=True)
        dist.close()
        return
    # ---- e2e: C ABI per frame, camera in, framebuffer to pinned host memory ----
    lib = ctx.lib
    pinned = torch.empty((h, w, 4), dtype=torch.float32, pin_memory=True)
    sync_params = H.trace_params(spp=spp, jitter=1, seed=17, shading=2, kernel_variant=args.variant, refill=args.refill, speculative=args.speculative, leaf_again=args.leaf_again)
    for _ in range(2):
        H.trace(ctx, tlas, cam, frame, sync_params)
        ctx.check(lib.hrt_frame_download(frame.handle, ctypes.c_void_p(pinned.data_ptr()), None, None))
    torch.cuda.synchronize()
    te = time.perf_counter()
    e2e_steps = max(3, args.steps // 2)
    for _ in range(e2e_steps):
        H.trace(ctx, tlas, cam, frame, sync_params)
        ctx.check(lib.hrt_frame_download(frame.handle, ctypes.c_void_p(pinned.data_ptr()), None, None))
    te = (time.perf_counter() - te) / e2e_steps
    e2e = {"value": round(rays_per_step / te / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 128,
           "d2h_bytes_per_step": w * h * 16, "ms_per_step": round(te * 1e3, 3)}
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_max, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPE_DESC,
            "data": "synthetic: seeded strands (the reference's glTF hair assets are not available)",
            "config": config_block(cfg, args.config), "rays_per_step": int(rays_per_step),
            "primary_rays_per_step": int(st["primary_rays"]), "shadow_rays_per_step": int(st["shadow_rays"]),
            "fp64_resolves_per_step": int(st["fp64_resolves"]), "gpu_launches": args.steps,
            "roofline": roofline, "phase_share": phase, "e2e": e2e, "clocks": clk,
            "build": {"blas_build_ms": round(info["build_ms"], 2), "build_wall_s": round(build_wall, 3),
                      "strand_generation_s": round(t_gen, 3), "nodes": int(info["nnodes"]),
                      "device_bytes": int(info["device_bytes"])}}
    # ---- plain FP32 tracer on the same strands (the comparison the metric names) ----
    if not args.quick and int(cfg["precision"]) == 1:
        blas32 = H.BottomLevelAccelerationStructure(
            H.BLASInput(type=cfg["type"], vertices=v, radius=r, strand_offsets=off, precision=H.Precision.FP32,
                        max_leaf=args.max_leaf), ctx)
        tlas32 = H.TopLevelAccelerationStructure([blas32], ctx)
        f32 = H.Frame(ctx, w, h, spp, with_hits=False)
        H.trace(ctx, tlas32, cam, f32, H.trace_params(spp=spp, jitter=1, seed=17, shading=2,
                                                      kernel_variant=args.variant, refill=args.refill, speculative=args.speculative, leaf_again=args.leaf_again))
        s32 = f32.stats()
        ms32 = time_frames(ctx, tlas32, cam, f32, params, args.steps, args.warmup)
        line["plain_fp32"] = {"value": round((s32["primary_rays"] + s32["shadow_rays"]) / (ms32 * 1e-3) / 1e6, 3),
                              "ms_per_step": round(ms32, 3), "build_ms": round(blas32.info["build_ms"], 2)}
        del f32, tlas32, blas32
    # ---- agreement with the FP64 oracle on 65,536 sampled rays, and the CPU baseline ----
    if not args.no_cpu:
        H.trace(ctx, tlas, cam, frame, H.trace_params(spp=spp, jitter=1, seed=17, shading=2, record_hits=1))
        rgba, hits = frame.download(hits=True)
        osc, orc = oracle_scene(cfg, v, r, int(cfg["precision"]))
        vi, pi = H.camera_arrays(cam)
        px = sample_pixels(w, h, 65536 // spp, seed=3)
        o = osc.render(vi, pi, w, h, spp=spp, jitter=1, seed=17, shading=2, precision=64, pixel_list=px)
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from hairscene import compare_hits
        gh = hits.reshape(h * w, spp)[px].reshape(-1)
        g_t = np.where(gh["t"] >= 0, gh["t"].astype(np.float64), -1.0)
        cmp = compare_hits(g_t, gh["prim"], gh["inst"], o["t"], o["prim"], o["inst"])
        same = (gh["prim"] == o["prim"]) & (((gh["flags"] & H.HIT_SHADOWED) != 0) == (o["shadow"] != 0))
        ok_px = same.reshape(-1, spp).all(axis=1)
        dpx = np.abs(rgba.reshape(-1, 4)[px] - o["fb"]).max(axis=1)
        line["agreement"] = {"rays": int(cmp["n"]), "hit_id": round(cmp["agreement"], 6), "mismatches": cmp["mismatches"],
                             "ties": cmp["ties"], "max_rel_t": cmp["max_rel_t"], "p9999_rel_t": cmp["p9999_rel_t"],
                             "pixels_agreeing": round(float(ok_px.mean()), 6),
                             "max_rgb_err_agreeing": float(dpx[ok_px].max()) if ok_px.any() else None,
                             "oracle": ORACLE_DESC}
        rate, desc, secs = cpu_sample_rate(osc, (vi, pi), cfg, 32, target_s=args.cpu_seconds)
        line["cpu_baseline"] = {"value": round(rate, 4), "unit": "Mrays/s", "cores": orc.orc_hardware_threads(),
                                "kind": "port", "sample": f"{desc}, FP32 oracle, {secs:.1f} s"}
    print(json.dumps(line), flush=True)
    dist.close()


BATCH_CONFIG = "c5_batched"


def batch_models(args):
    """The 16 models of the batched workload, with strands generated (host arrays)."""
    import vkhrt_gb300 as H
    models = []
    for m in H.batch_workload():
        sp = H.StrandParams(seed=m["seed"], nstrands=m["nstrands"], nverts=m["nverts"], r_root=m["r_root"],
                            r_tip=m["r_tip"])
        v, r, off = H.generate_strands(sp)
        models.append((m, v, r, off))
    return models


def batch_config_block(models):
    nseg = sum(m["nstrands"] * (m["nverts"] - 1) for m, *_ in models)
    px = sum(m["width"] * m["height"] * m["spp"] for m, *_ in models)
    return {"workload": f"{BATCH_CONFIG}: {len(models)} hair models (strands log-uniform in [2000, 200000], "
                        f"{{16,32,64,128}} vertices, Phantom/LSS/DOTS in turn), {nseg} segments, own cameras, "
                        f"256x256..1920x1080 at 1-4 spp ({px} primary samples), Shade + 1 shadow ray",
            "segments": nseg, "scenes": len(models), "primary_samples": px,
            "precision": PRECISION_DESC,
            "l2": "inputs larger than L2 (BVHs + primitives resident, no flush)", "parallelism": "replicas"}


def run_batched(args, dist):
    """All scenes in one CUDA-graph launch of the persistent kernel (autotuned) against 16
    sequential plain FP32 launches and 16 sequential quantised launches of the same scenes."""
    import torch
    import vkhrt_gb300 as H
    dev = dist.local
    torch.cuda.set_device(dev)
    ctx = H.Context(dev)
    t_gen = time.perf_counter()
    models = batch_models(args)
    t_gen = time.perf_counter() - t_gen

    def build(precision):
        out = []
        for m, v, r, off in models:
            b = H.BottomLevelAccelerationStructure(
                H.BLASInput(type=m["type"], vertices=v, radius=r, strand_offsets=off, precision=precision,
                            max_leaf=args.max_leaf), ctx)
            t = H.TopLevelAccelerationStructure([b], ctx)
            cam = H.orbit_camera(m["width"], m["height"], m["azimuth"], m["elevation"])
            out.append((b, t, cam, H.Frame(ctx, m["width"], m["height"], m["spp"], with_hits=not args.no_cpu)))
        return out

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    q = build(H.Precision.QUANTISED)
    build_wall = time.perf_counter() - t0
    f = build(H.Precision.FP32)
    base = H.trace_params(jitter=1, seed=17, shading=2, **{"async": 1})
    # ---- per-scene work counts (sequential, counted): rays and algorithmic bytes ----
    rays_per_step = 0
    alg_bytes = 0
    per_scene = []
    for (b, t, cam, fr), (m, *_r) in zip(q, models):
        H.trace(ctx, t, cam, fr, H.trace_params(jitter=1, seed=17, shading=2, count_stats=1))
        st = fr.stats()
        info = b.info
        prim_b = prim_test_bytes(info, int(m["type"]), 1)
        rays = st["primary_rays"] + st["shadow_rays"]
        rays_per_step += rays
        alg_bytes += st["nodes_visited"] * info["node_bytes"] + st["prims_tested"] * prim_b + \
            m["width"] * m["height"] * 16
        per_scene.append({"type": m["type"].name[1:], "segments": m["nstrands"] * (m["nverts"] - 1),
                          "image": f"{m['width']}x{m['height']}", "spp": m["spp"], "rays": int(rays)})
    # ---- autotune the batch (untimed) ----
    scenes_q = [(t, cam, fr) for (_, t, cam, fr) in q]
    tuned, tune_ms = H.autotune(ctx, scenes_q, base, reps=2, cache=args.tune_cache, key=f"{BATCH_CONFIG}/quantised")
    batch = H.Batch(ctx, scenes_q, tuned)
    dist.barrier()
    clocks = Clocks(dev)
    clocks.start()
    cams = [cam for (_, _, cam, _) in q]

    def paced(b, nsteps):
        # A step renders every scene from its cameras (their 3 KB scene-table upload starts the
        # step, as in an interactive renderer) and ends when the replay has finished, as the
        # sequential comparison's steps do. Replays queued back to back without this pacing ran
        # about 4 % slower each on GB300 (cause not found).
        for _ in range(nsteps):
            b.set_cameras(cams)
            b.launch()
            torch.cuda.current_stream().synchronize()

    paced(batch, args.warmup)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    paced(batch, args.steps)
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    ms_max = dist.max(ms)
    value = dist.world * rays_per_step / (ms_max * 1e-3) / 1e6

    def sequential(sc, params):
        """Mean over steps of the sum of per-scene launch times (each launch bracketed by events)."""
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in sc]
        for _ in range(args.warmup):
            for (_, t, cam, fr) in sc:
                H.trace(ctx, t, cam, fr, params)
        torch.cuda.synchronize()
        lat = np.zeros(len(sc))
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        total = 0.0
        for _ in range(args.steps):
            s0.record()
            for (a, z), (_, t, cam, fr) in zip(ev, sc):
                a.record()
                H.trace(ctx, t, cam, fr, params)
                z.record()
            s1.record()
            torch.cuda.synchronize()
            lat += [a.elapsed_time(z) for a, z in ev]
            total += s0.elapsed_time(s1)
        return total / args.steps, lat / args.steps

    plain_params = H.trace_params(jitter=1, seed=17, shading=2, **{"async": 1})
    ms_f32, lat_f32 = sequential(f, plain_params)
    ms_q, lat_q = sequential(q, tuned)
    # the batching pattern on FP32 BLASes too, so that precision and batching can be told apart
    scenes_f = [(t, cam, fr) for (_, t, cam, fr) in f]
    tuned_f, _ = H.autotune(ctx, scenes_f, base, reps=2, cache=args.tune_cache, key=f"{BATCH_CONFIG}/fp32")
    batch_f = H.Batch(ctx, scenes_f, tuned_f)
    paced(batch_f, args.warmup)
    torch.cuda.synchronize()
    e0.record()
    paced(batch_f, args.steps)
    e1.record()
    torch.cuda.synchronize()
    ms_bf = e0.elapsed_time(e1) / args.steps
    mem_q = sum(int(b.info["device_bytes"]) for (b, *_r) in q)
    mem_f = sum(int(b.info["device_bytes"]) for (b, *_r) in f)
    if dist.rank != 0:
        dist.close()
        return
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    for d, a, b2 in zip(per_scene, lat_f32, lat_q):
        d["plain_fp32_ms"] = round(float(a), 3)
        d["quantised_ms"] = round(float(b2), 3)
    # ---- e2e: through the C ABI, each step's cameras in and every framebuffer out to pinned host
    # memory; two frame sets on two streams, so that step k's read-back overlaps step k+1's render
    # (the renders themselves stay in order: each waits for the previous one) ----
    tparams = H.trace_params(jitter=1, seed=17, shading=2, **{"async": 1},
                             **{k: getattr(tuned, k) for k in H.TUNED_FIELDS})
    fsets = [[fr for (_, _, _, fr) in q], [H.Frame(ctx, m["width"], m["height"], m["spp"]) for m, *_ in models]]
    e2e_batches = [H.Batch(ctx, [(t, cam, fr) for (_, t, cam, _), fr in zip(q, fs)], tparams) for fs in fsets]
    pins = [[torch.empty((m["height"], m["width"], 4), dtype=torch.float32, pin_memory=True) for m, *_ in models]
            for _ in range(2)]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    rendered = [torch.cuda.Event(), torch.cuda.Event()]

    def e2e_run(nsteps):
        prev = None
        for k in range(nsteps):
            j = k & 1
            st, b = streams[j], e2e_batches[j]
            if prev is not None:
                st.wait_event(prev)
            b.set_cameras(cams, stream=st.cuda_stream)
            b.launch(stream=st.cuda_stream)
            rendered[j].record(st)
            prev = rendered[j]
            b.download(pins[j], stream=st.cuda_stream, synchronise=False)
        for st in streams:
            st.synchronize()

    e2e_run(2)
    e2e_steps = max(4, args.steps)
    te = time.perf_counter()
    e2e_run(e2e_steps)
    te = (time.perf_counter() - te) / e2e_steps
    assert all(torch.equal(a, b) for a, b in zip(pins[0], pins[1])), "the two frame sets must render alike"
    e2e_batch = e2e_batches[0]
    d2h = sum(m["width"] * m["height"] * 16 for m, *_ in models)
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_max, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPE_DESC,
            "data": "synthetic: seeded strands (the reference's glTF hair assets are not available)",
            "config": batch_config_block(models), "rays_per_step": int(rays_per_step), "gpu_launches": args.steps,
            "autotuned": {k: int(getattr(tuned, k)) for k in H.TUNED_FIELDS} | {"mean_ms": round(tune_ms, 3)},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                         "bytes_per_launch": int(alg_bytes)},
            "plain_fp32": {"value": round(rays_per_step / (ms_f32 * 1e-3) / 1e6, 3),
                           "ms_per_step": round(ms_f32, 3), "launches_per_step": len(models),
                           "what": "the same 16 scenes as 16 sequential launches of the FP32 tracer (FP32 nodes "
                                   "and records, no batching, no autotuning)"},
            "sequential_quantised": {"value": round(rays_per_step / (ms_q * 1e-3) / 1e6, 3),
                                     "ms_per_step": round(ms_q, 3), "launches_per_step": len(models)},
            "batched_fp32": {"value": round(rays_per_step / (ms_bf * 1e-3) / 1e6, 3), "ms_per_step": round(ms_bf, 3),
                             "autotuned": {k: int(getattr(tuned_f, k)) for k in H.TUNED_FIELDS},
                             "note": "the batching pattern on FP32 BLASes: on these coherent, L2-resident "
                                     "workloads the 8-bit node decode costs more ALU than the bytes it saves"},
            "device_bytes": {"quantised": mem_q, "fp32": mem_f},
            "per_scene_latency_ms": {"batched_all_scenes": round(ms, 3),
                                     "note": "a batched scene completes with the launch; sequential latencies "
                                             "are per launch"},
            "scenes": per_scene,
            "e2e": {"value": round(rays_per_step / te / 1e6, 3), "unit": "Mrays/s",
                    "h2d_bytes_per_step": e2e_batch.table_bytes, "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": round(te * 1e3, 3)},
            "clocks": clk,
            "build": {"build_wall_s_quantised": round(build_wall, 3), "strand_generation_s": round(t_gen, 3)}}
    if not args.no_cpu:
        line.update(batch_agreement_and_cpu(args, ctx, q, models))
    del q, f, batch, e2e_batch, e2e_batches, fsets, scenes_q, scenes_f, batch_f
    if not args.quick:
        line["c4_phantom_quantised"] = c4_summary(args, ctx)
    print(json.dumps(line), flush=True)
    dist.close()


def c4_summary(args, ctx):
    """The single Phantom precision-pattern frame (19.05 M segments, 1920x1080 x 4 spp): quantised
    and FP32 frame rates (no oracle legs; `--config c4_phantom_quantised` has them)."""
    import vkhrt_gb300 as H
    cfg, sp = workload("c4_phantom_quantised")
    w, h, spp = cfg["width"], cfg["height"], cfg["spp"]
    v, r, off = H.generate_strands(sp)
    cam = H.scene_camera(w, h)
    out = {}
    for name, prec in (("quantised", H.Precision.QUANTISED), ("plain_fp32", H.Precision.FP32)):
        blas = H.BottomLevelAccelerationStructure(
            H.BLASInput(type=cfg["type"], vertices=v, radius=r, strand_offsets=off, precision=prec), ctx)
        tlas = H.TopLevelAccelerationStructure([blas], ctx)
        fr = H.Frame(ctx, w, h, spp)
        H.trace(ctx, tlas, cam, fr, H.trace_params(spp=spp, jitter=1, seed=17, shading=2, count_stats=1))
        st = fr.stats()
        p = H.trace_params(spp=spp, jitter=1, seed=17, shading=2, **{"async": 1})
        ms = time_frames(ctx, tlas, cam, fr, p, max(8, args.steps // 2), args.warmup)
        out[name] = {"value": round((st["primary_rays"] + st["shadow_rays"]) / (ms * 1e-3) / 1e6, 3),
                     "ms_per_step": round(ms, 3), "nodes_visited": int(st["nodes_visited"]),
                     "prims_tested": int(st["prims_tested"]), "blas_build_ms": round(blas.info["build_ms"], 2)}
        # animated strands: the same BLAS refitted to moved vertices (topology kept)
        v2 = (v + np.float32(0.01) * np.sin(np.float32(3.0) * v[:, [1, 2, 0]])).astype(np.float32)
        blas.refit(v2, r)
        out[name]["blas_refit_ms"] = round(blas.info["build_ms"], 2)
        del fr, tlas, blas
    return out


def batch_agreement_and_cpu(args, ctx, q, models):
    """Per-scene FP64 oracle agreement on ~65,536 sampled rays in all, and the oracle's FP32 rate."""
    import vkhrt_gb300 as H
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from hairscene import OracleScene, compare_hits, load_oracle, oracle_geometry
    orc = load_oracle()
    threads = orc.orc_hardware_threads()
    n_t = n_mis = n_ties = 0
    max_rel_t = 0.0
    max_rgb = 0.0
    cpu_rays = 0
    cpu_px = 0
    cpu_s = 0.0
    cpu_frac = 1.0  # every pixel of every scene: about 10 s of CPU work
    per = max(1, 65536 // len(models))
    for (b, t, cam, fr), (m, v, r, off) in zip(q, models):
        H.trace(ctx, t, cam, fr, H.trace_params(jitter=1, seed=17, shading=2, record_hits=1))
        rgba, hits = fr.download(hits=True)
        w, h, spp = m["width"], m["height"], m["spp"]
        lines, lrad = uniform_lines(v, r, m["nstrands"], m["nverts"])
        data, rad = oracle_geometry(orc, int(m["type"]), lines, lrad, quantised=(int(m["type"]) == 0))
        del lines, lrad
        osc = OracleScene(orc, [(int(m["type"]), data, rad)])
        vi, pi = H.camera_arrays(cam)
        px = sample_pixels(w, h, per // spp, seed=3)
        o = osc.render(vi, pi, w, h, spp=spp, jitter=1, seed=17, shading=2, precision=64, pixel_list=px)
        gh = hits.reshape(h * w, spp)[px].reshape(-1)
        g_t = np.where(gh["t"] >= 0, gh["t"].astype(np.float64), -1.0)
        cmp = compare_hits(g_t, gh["prim"], gh["inst"], o["t"], o["prim"], o["inst"])
        n_t += cmp["n"]
        n_mis += cmp["mismatches"]
        n_ties += cmp["ties"]
        max_rel_t = max(max_rel_t, cmp["max_rel_t"])
        same = (gh["prim"] == o["prim"]) & (((gh["flags"] & H.HIT_SHADOWED) != 0) == (o["shadow"] != 0))
        ok_px = same.reshape(-1, spp).all(axis=1)
        if ok_px.any():
            max_rgb = max(max_rgb, float(np.abs(rgba.reshape(-1, 4)[px] - o["fb"]).max(axis=1)[ok_px].max()))
        # the oracle's FP32 tracer on the same fraction of every scene's pixels (the workload's mix;
        # at least 16,384 pixels per call, since a call has a few ms of thread start-up)
        cpx = sample_pixels(w, h, int(w * h * cpu_frac), seed=11)
        t0 = time.perf_counter()
        oc = osc.render(vi, pi, w, h, spp=spp, jitter=1, seed=17, shading=2, precision=32, pixel_list=cpx,
                        threads=threads)
        dt = time.perf_counter() - t0
        cpu_s += dt
        cpu_rays += len(cpx) * spp + int((oc["t"] >= 0).sum())
        cpu_px += len(cpx)
        del osc, data, rad
    return {"agreement": {"rays": int(n_t), "hit_id": round(1.0 - n_mis / max(n_t - n_ties, 1), 6),
                          "mismatches": int(n_mis),
                          "ties": int(n_ties), "max_rel_t": max_rel_t, "max_rgb_err_agreeing": max_rgb,
                          "oracle": ORACLE_DESC + ", per scene"},
            "cpu_baseline": {"value": round(cpu_rays / cpu_s / 1e6, 4), "unit": "Mrays/s", "cores": threads,
                             "kind": "port",
                             "sample": f"{pixel_share(cpu_frac)} of every scene ({cpu_px} pixels, all their "
                                       f"samples, {cpu_rays} rays), FP32 oracle, {cpu_s:.1f} s"}}


def pixel_share(frac: float) -> str:
    """'every pixel' or '<frac> of the pixels' for a CPU sample description."""
    return "every pixel" if frac >= 1.0 else f"{frac:g} of the pixels"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default=BATCH_CONFIG)
    ap.add_argument("--quick", action="store_true", help="skip the plain FP32 comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the oracle agreement and CPU baseline")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-pixels", type=int, default=4096)
    ap.add_argument("--width", type=int, default=0, help="override the image width (profiling)")
    ap.add_argument("--height", type=int, default=0, help="override the image height (profiling)")
    ap.add_argument("--spp", type=int, default=0, help="override samples per pixel (profiling)")
    ap.add_argument("--precision", choices=["fp32", "quantised"], default=None,
                    help="override the workload's BVH/primitive precision (profiling)")
    ap.add_argument("--variant", type=int, default=0, help="resident blocks per SM: 0/1 = 4, 2 = 3, 3 = 5")
    ap.add_argument("--max-leaf", type=int, default=1, help="primitives per BVH8 leaf (1..3)")
    ap.add_argument("--refill", type=int, default=8, help="idle lanes per warp that trigger a fetch (0 = 16)")
    ap.add_argument("--speculative", type=int, default=1, help="speculative traversal (0/1)")
    ap.add_argument("--leaf-again", type=int, default=4,
                    help="repeat the leaf phase while this many lanes hold leaves (0 = once)")
    ap.add_argument("--tune-cache", default=None, help="JSON file that keeps autotuner choices between runs")
    ap.add_argument("--profile", action="store_true",
                    help="one warm-up and the timed steps only: no e2e, FP32 comparison or CPU legs")
    args = ap.parse_args()
    for k in ("width", "height", "spp"):
        if getattr(args, k):
            _OVERRIDE[k] = getattr(args, k)
    if args.precision:
        import vkhrt_gb300 as H
        _OVERRIDE["precision"] = H.Precision.QUANTISED if args.precision == "quantised" else H.Precision.FP32
    if args.profile:
        args.quick = args.no_cpu = True
    if args.warmup < 3 and not args.profile:
        args.warmup = 3
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
        dist.close()
        return
    if args.config == BATCH_CONFIG:
        run_batched(args, dist)
        return
    run_ours(args, dist)


if __name__ == "__main__":
    main()
