#!/usr/bin/env python3
"""Mrays/s of the GB300 hair ray tracer: quantised and batched against plain FP32.

Default workload (c5_batched): 16 seeded hair models (strands log-uniform in [2,000, 200,000],
16-128 vertices, Phantom / LSS / DOTS in turn, 47.9 M segments in all), each with its own camera,
resolution (256x256 .. 1920x1080) and 1-4 jittered samples per pixel, Shade() plus one shadow ray
per hit. Quantised BLASes (8-bit BVH8 boxes; Phantom segments as indices into the strand vertex
stream), all scenes in one CUDA-graph replay of the persistent trace kernels with autotuned
settings. A step is one replay. `value` counts primary + shadow rays per second with the BVHs
resident in HBM (several GB, far above the 129 MB L2, so no flush between steps).

The line also carries, for the same scenes: `plain_fp32` (16 sequential launches of the FP32
tracer, the comparison the metric names), `sequential_quantised`, `batched_fp32`; `agreement`
(the timed graph's framebuffers and hit records of the same graph against the FP64 CPU oracle on
65,536 sampled rays, on the original FP32 strands); `e2e` through the C ABI (cameras in, every
framebuffer to pinned host memory); `cpu_baseline` (the oracle's FP32 tracer on every pixel, and
its FP64 tracer on a row sample); and `configs`: C1-C4 (Phantom FP32 512x512, LSS and DOTS
1920x1080, the 19.05 M-segment Phantom frame at 4 spp), each with both precisions, agreement and
roofline. Per-scene details go to stderr.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config NAME]

Under torchrun (N > 1) every rank renders its own views of the workload: each scene's camera is
turned about the vertical axis by 2 pi rank / N (rank_azimuth), so the ranks' work is disjoint and
of the same size (replicas, weak scaling, no device collective); after the timed steps rank 0
gathers every rank's framebuffers to its host (vkhrt_gb300.replicas) and prints the line. `--impl reference` times the CPU restatement of the reference's trace path
(oracle/, FP32, all host threads; the oracle library alone, which also carries the workload
generator) on one band of image rows of every scene per step.
"""
from __future__ import annotations

import argparse
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
sys.path.insert(0, os.path.join(ROOT, "tests"))  # hairscene: oracle scenes and hit comparison

METRIC = "Mrays/s on 1 GB300: quantized/batched vs plain FP32 at >=99.99% hit agreement"
L2_BYTES = 129 * 1024 * 1024
PRECISION_DESC = ("quantised (8-bit BVH8 boxes; Phantom segments as 4-byte indices into the strand vertex stream, "
                  "control points rebuilt from the FP32 vertices in the leaf)")
DTYPE_DESC = "fp32 (8-bit node boxes)"
BATCH_PRECISION_DESC = ("node format chosen by the autotuner: FP32 BVH8 boxes and records, or 8-bit boxes with "
                        "Phantom segments as 4-byte indices into the strand vertex stream, whichever it times faster "
                        "on the workload (the other is reported beside it)")
ORACLE_DESC = "FP64 CPU restatement on the original FP32 strands"
DATA_DESC = "synthetic: seeded strands (the reference's glTF hair assets are not available)"
BATCH_CONFIG = "c5_batched"
SINGLE_CONFIGS = ("c1_phantom_fp32", "c2_lss_fp32", "c3_dots_fp32", "c4_phantom_quantised")
AGREE_RAYS = 65536
ROW_BANDS = 4       # CPU legs: a step renders one of every ROW_BANDS image rows (scanline order)
FP64_BANDS = 16     # the FP64 CPU figure: one of every FP64_BANDS rows


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


def prim_test_bytes(info, gtype: int, precision: int) -> int:
    """Bytes one primitive test reads: the record, and for quantised Phantom the four 16-byte
    stream entries it indexes."""
    return int(info["prim_bytes"]) + (64 if gtype == 0 and precision == 1 else 0)


# ------------------------------------------------------------------------------ workload helpers
_OVERRIDE = {}


def workload(name: str):
    import vkhrt_gb300 as H
    cfg = dict(H.CONFIGS[name])
    cfg.update(_OVERRIDE)
    sp = H.StrandParams(seed=cfg["seed"], nstrands=cfg["nstrands"], nverts=cfg["nverts"], r_root=cfg["r_root"],
                        r_tip=cfg["r_tip"])
    return cfg, sp


def oracle_lib():
    """The CPU oracle's library with the workload generator's symbols declared."""
    import vkhrt_gb300 as H
    from hairscene import load_oracle
    return H.bind_workload(load_oracle())


def uniform_lines(v, r, ns, nv):
    vv = v.reshape(ns, nv, 3)
    rr = r.reshape(ns, nv)
    lines = np.ascontiguousarray(np.concatenate([vv[:, :-1], vv[:, 1:]], axis=2).reshape(-1, 6), np.float32)
    lrad = np.ascontiguousarray(np.stack([rr[:, :-1], rr[:, 1:]], axis=2).reshape(-1, 2), np.float32)
    return lines, lrad


def oracle_scene(orc, gtype: int, v, r, ns: int, nv: int):
    """The oracle's scene of one hair model: its own geometry processing of the FP32 strands."""
    from hairscene import OracleScene, oracle_geometry
    lines, lrad = uniform_lines(v, r, ns, nv)
    data, rad = oracle_geometry(orc, gtype, lines, lrad)
    del lines, lrad
    return OracleScene(orc, [(gtype, data, rad)])


def sample_pixels(w, h, n, seed=7):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(w * h, size=min(n, w * h), replace=False)).astype(np.uint32)


def row_band(w: int, h: int, k: int, nbands: int) -> np.ndarray:
    """Pixels of the rows y = k (mod nbands), in scanline order."""
    ys = np.arange(k % nbands, h, nbands, dtype=np.uint32)
    return (ys[:, None] * np.uint32(w) + np.arange(w, dtype=np.uint32)[None, :]).reshape(-1)


def compare_frame(rgba, hits, o, px, spp):
    """GPU hit records and pixels against the oracle's render of the pixels `px` (all samples)."""
    import vkhrt_gb300 as H
    from hairscene import compare_hits
    gh = hits.reshape(-1, spp)[px].reshape(-1)
    g_t = np.where(gh["t"] >= 0, gh["t"].astype(np.float64), -1.0)
    cmp = compare_hits(g_t, gh["prim"], gh["inst"], o["t"], o["prim"], o["inst"])
    same = (gh["prim"] == o["prim"]) & (((gh["flags"] & H.HIT_SHADOWED) != 0) == (o["shadow"] != 0))
    ok_px = same.reshape(-1, spp).all(axis=1)
    dpx = np.abs(rgba.reshape(-1, 4)[px] - o["fb"]).max(axis=1)
    return {"rays": int(cmp["n"]), "hits": int(cmp["hits"]), "mismatches": int(cmp["mismatches"]),
            "ties": int(cmp["ties"]), "max_rel_t": float(cmp["max_rel_t"]), "p9999_rel_t": float(cmp["p9999_rel_t"]),
            "pixels": int(len(px)), "pixels_agreeing": int(ok_px.sum()),
            "max_rgb": float(dpx[ok_px].max()) if ok_px.any() else 0.0,
            "rgb_over_1e-4": int((dpx[ok_px] > 1e-4).sum())}


def merge_compare(parts):
    n = sum(p["rays"] for p in parts)
    ties = sum(p["ties"] for p in parts)
    mis = sum(p["mismatches"] for p in parts)
    return {"rays": n, "hit_id": round(1.0 - mis / max(n - ties, 1), 6), "mismatches": mis, "ties": ties,
            "max_rel_t": max((p["max_rel_t"] for p in parts), default=0.0),
            "max_rgb_err_agreeing": max((p["max_rgb"] for p in parts), default=0.0),
            "pixels_rgb_over_1e-4": sum(p["rgb_over_1e-4"] for p in parts),
            "pixels_agreeing": round(sum(p["pixels_agreeing"] for p in parts) /
                                     max(sum(p["pixels"] for p in parts), 1), 6)}


def cpu_rate(scenes, precision: int, bands, nbands: int, threads: int, jitter: int):
    """The oracle's tracer over the given row bands of every scene: (Mrays/s, rays, pixels, seconds).
    scenes: (oracle scene, view_inv, proj_inv, width, height, spp)."""
    rays = px_n = 0
    secs = 0.0
    for osc, vi, pi, w, h, spp in scenes:
        for k in bands:
            px = row_band(w, h, k, nbands)
            t0 = time.perf_counter()
            o = osc.render(vi, pi, w, h, spp=spp, jitter=jitter, seed=17, shading=2, precision=precision,
                           pixel_list=px, threads=threads)
            secs += time.perf_counter() - t0
            rays += len(px) * spp + int((o["t"] >= 0).sum())
            px_n += len(px)
    return rays / secs / 1e6, rays, px_n, secs


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


def jitter_of(spp: int) -> int:
    """The batched scenes jitter every sample; single configurations jitter only with several
    samples per pixel (one sample at the pixel centre, as ray_gen.rgen)."""
    return 1 if spp > 1 else 0


# ------------------------------------------------------------------------------ reference arm
def run_reference(args, dist):
    """CPU restatement of the reference's trace path (FP32 Prhi / LSS / DOTS, all host threads),
    loading only the oracle's library (which carries the workload generator too): step s renders
    the rows y = s (mod 4) of every scene, all samples plus shadow rays, in scanline order."""
    if dist.rank != 0:
        return
    import vkhrt_gb300 as H
    orc = oracle_lib()
    threads = orc.orc_hardware_threads()
    if args.config == BATCH_CONFIG:
        models = [(m, *H.generate_strands(H.StrandParams(seed=m["seed"], nstrands=m["nstrands"], nverts=m["nverts"],
                                                         r_root=m["r_root"], r_tip=m["r_tip"]), lib=orc))
                  for m in H.batch_workload()]
        cams = [H.orbit_camera(m["width"], m["height"], m["azimuth"], m["elevation"], lib=orc) for m, *_ in models]
        config = batch_config_block([m for m, *_ in models])
        jit = 1
    else:
        cfg, sp = workload(args.config)
        models = [(cfg, *H.generate_strands(sp, lib=orc))]
        cams = [H.scene_camera(cfg["width"], cfg["height"], lib=orc)]
        config = single_config_block(cfg, args.config)
        jit = jitter_of(cfg["spp"])
    scenes = []
    for (m, v, r, off), cam in zip(models, cams):
        vi, pi = H.camera_arrays(cam)
        scenes.append((oracle_scene(orc, int(m["type"]), v, r, m["nstrands"], m["nverts"]), vi, pi, m["width"],
                       m["height"], m["spp"]))
    del models
    total_t = 0.0
    total_rays = 0
    for step in range(args.warmup + args.steps):
        _, rays, _, secs = cpu_rate(scenes, 32, [step % ROW_BANDS], ROW_BANDS, threads, jit)
        if step >= args.warmup:
            total_t += secs
            total_rays += rays
    value = total_rays / total_t / 1e6
    sample = (f"rows y = s (mod {ROW_BANDS}) of every scene at step s (all samples, + shadow rays, scanline order): "
              f"every pixel over {ROW_BANDS} steps")
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total_t / max(args.steps, 1), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": DATA_DESC,
            "config": config,
            "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def single_config_block(cfg, name):
    nseg = cfg["nstrands"] * (cfg["nverts"] - 1)
    kind = {0: "Bezier", 1: "LSS", 2: "DOTS"}[int(cfg["type"])]
    return {"workload": f"{name}: {cfg['nstrands']} strands x {cfg['nverts']} vertices = {nseg} {kind} segments, "
                        f"{cfg['width']}x{cfg['height']} x {cfg['spp']} spp, Shade + 1 shadow ray",
            "segments": nseg, "image": f"{cfg['width']}x{cfg['height']}", "spp": cfg["spp"],
            "precision": PRECISION_DESC if int(cfg["precision"]) else "fp32",
            "l2": "inputs larger than L2 (BVH + primitives resident, no flush)", "parallelism": "replicas"}


def batch_config_block(models):
    nseg = sum(m["nstrands"] * (m["nverts"] - 1) for m in models)
    px = sum(m["width"] * m["height"] * m["spp"] for m in models)
    return {"workload": f"{BATCH_CONFIG}: {len(models)} hair models (strands log-uniform in [2000, 200000], "
                        f"{{16,32,64,128}} vertices, Phantom/LSS/DOTS in turn), {nseg} segments, own cameras, "
                        f"256x256..1920x1080 at 1-4 spp ({px} primary samples), Shade + 1 shadow ray",
            "segments": nseg, "scenes": len(models), "primary_samples": px, "precision": BATCH_PRECISION_DESC,
            "l2": "inputs larger than L2 (BVHs + primitives resident, no flush)", "parallelism": "replicas"}


# ------------------------------------------------------------------------------ C1-C4 blocks
def run_config(ctx, name: str, args, orc) -> dict:
    """One BASELINE configuration at full size: both precisions timed (frames in HBM, K launches
    between CUDA events), per-sample hit records of each checked against the FP64 oracle on
    65,536 sampled rays (pixels within 1e-4 where hits agree), and the roofline of the
    configuration's own precision."""
    import vkhrt_gb300 as H
    cfg, sp = workload(name)
    w, h, spp, gtype = cfg["width"], cfg["height"], cfg["spp"], int(cfg["type"])
    v, r, off = H.generate_strands(sp)
    cam = H.scene_camera(w, h)
    vi, pi = H.camera_arrays(cam)
    t0 = time.perf_counter()
    osc = oracle_scene(orc, gtype, v, r, cfg["nstrands"], cfg["nverts"])
    px = sample_pixels(w, h, AGREE_RAYS // spp, seed=3)
    o = osc.render(vi, pi, w, h, spp=spp, jitter=jitter_of(spp), seed=17, shading=2, precision=64, pixel_list=px)
    oracle_s = time.perf_counter() - t0
    del osc
    peak, _ = load_peaks()
    out = {}
    for prec in (H.Precision.FP32, H.Precision.QUANTISED):
        blas = H.BottomLevelAccelerationStructure(
            H.BLASInput(type=cfg["type"], vertices=v, radius=r, strand_offsets=off, precision=prec), ctx)
        tlas = H.TopLevelAccelerationStructure([blas], ctx)
        fr = H.Frame(ctx, w, h, spp, with_hits=True)
        base = dict(spp=spp, jitter=jitter_of(spp), seed=17, shading=2)
        H.trace(ctx, tlas, cam, fr, H.trace_params(count_stats=1, **base))
        st = fr.stats()
        ms = time_frames(ctx, tlas, cam, fr, H.trace_params(**base, **{"async": 1}), args.config_steps, 3)
        H.trace(ctx, tlas, cam, fr, H.trace_params(record_hits=1, **base))
        rgba, hits = fr.download(hits=True)
        cmp = compare_frame(rgba, hits, o, px, spp)
        info = blas.info
        rays = st["primary_rays"] + st["shadow_rays"]
        alg = st["nodes_visited"] * info["node_bytes"] + st["prims_tested"] * prim_test_bytes(info, gtype, int(prec)) \
            + w * h * 16
        out[int(prec)] = {"value": round(rays / (ms * 1e-3) / 1e6, 1), "ms": round(ms, 3), "rays": int(rays),
                          "cmp": cmp, "fp64_resolves": int(st["fp64_resolves"]),
                          "frac": round(alg / (ms * 1e-3) / 1e9 / peak, 3)}
        del fr, tlas, blas
    own, other = out[int(cfg["precision"])], out[1 - int(cfg["precision"])]

    def agree(c):
        return round(1.0 - c["mismatches"] / max(c["rays"] - c["ties"], 1), 6)

    c = own["cmp"]
    return {"value": own["value"], "fp32": out[0]["value"], "quantised": out[1]["value"], "agree": agree(c),
            "rays": c["rays"], "mis": c["mismatches"], "ties": c["ties"], "max_rel_t": float(f"{c['max_rel_t']:.2e}"),
            "max_rgb": float(f"{c['max_rgb']:.2e}"), "rgb_over": c["rgb_over_1e-4"], "fp64": own["fp64_resolves"],
            "agree_other": agree(other["cmp"]), "hbm_frac": own["frac"], "oracle_s": round(oracle_s, 1)}


# ------------------------------------------------------------------------------ batched (default)
def rank_azimuth(azimuth: float, rank: int, world: int) -> float:
    """The camera azimuth of a scene on `rank` of `world` (rank 0 keeps the scene's own)."""
    import math
    return azimuth + 2.0 * math.pi * rank / world


def batch_models():
    """The 16 models of the batched workload, with strands generated (host arrays)."""
    import vkhrt_gb300 as H
    models = []
    for m in H.batch_workload():
        sp = H.StrandParams(seed=m["seed"], nstrands=m["nstrands"], nverts=m["nverts"], r_root=m["r_root"],
                            r_tip=m["r_tip"])
        v, r, off = H.generate_strands(sp)
        models.append((m, v, r, off))
    return models


def kernels_per_replay(models, params) -> int:
    """Our kernel launches in one replay of a batch graph: a frame kernel per group (one group per
    primitive type when split), plus the FP64 pass and its averaging kernel for the group that
    holds the Phantom scenes."""
    types = {int(m["type"]) for m in models}
    groups = len(types) if params.split_types else 1
    return groups + (2 if 0 in types and params.fp64_resolve else 0)


def run_batched(args, dist):
    """All scenes in one CUDA-graph replay of the persistent kernels, autotuned on FP32 and on
    quantised BLASes; the node format whose tuned batch the autotuner timed faster is the line's
    value, the other format's batch is reported beside it, with 16 sequential plain FP32 launches
    and 16 sequential launches of the chosen format. Then the timed graph's output against the
    FP64 oracle, the CPU baseline and the single configurations."""
    import torch
    import vkhrt_gb300 as H
    dev = dist.local
    torch.cuda.set_device(dev)
    ctx = H.Context(dev)
    t_gen = time.perf_counter()
    models = batch_models()
    t_gen = time.perf_counter() - t_gen
    mlist = [m for m, *_ in models]

    def build(precision, with_hits):
        out = []
        for m, v, r, off in models:
            b = H.BottomLevelAccelerationStructure(
                H.BLASInput(type=m["type"], vertices=v, radius=r, strand_offsets=off, precision=precision,
                            max_leaf=args.max_leaf), ctx)
            t = H.TopLevelAccelerationStructure([b], ctx)
            cam = H.orbit_camera(m["width"], m["height"], rank_azimuth(m["azimuth"], dist.rank, dist.world),
                                 m["elevation"])
            out.append((b, t, cam, H.Frame(ctx, m["width"], m["height"], m["spp"], with_hits=with_hits)))
        return out

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    q = build(H.Precision.QUANTISED, not args.no_cpu)
    build_wall = time.perf_counter() - t0
    f = build(H.Precision.FP32, not args.no_cpu)
    base = H.trace_params(jitter=1, seed=17, shading=2, **{"async": 1})
    # ---- per-scene work counts (sequential, counted): rays and algorithmic bytes per format ----
    rays_per_step = 0
    per_scene = []
    for (b, t, cam, fr), (bf, tf, _, frf), m in zip(q, f, mlist):
        H.trace(ctx, t, cam, fr, H.trace_params(jitter=1, seed=17, shading=2, count_stats=1))
        st = fr.stats()
        H.trace(ctx, tf, cam, frf, H.trace_params(jitter=1, seed=17, shading=2, count_stats=1))
        stf = frf.stats()
        rays = st["primary_rays"] + st["shadow_rays"]
        rays_per_step += rays
        alg = {}
        for key, s_, bl, prec in (("quantised", st, b, 1), ("fp32", stf, bf, 0)):
            alg[key] = s_["nodes_visited"] * bl.info["node_bytes"] + \
                s_["prims_tested"] * prim_test_bytes(bl.info, int(m["type"]), prec) + m["width"] * m["height"] * 16
        per_scene.append({"type": m["type"].name[1:], "segments": m["nstrands"] * (m["nverts"] - 1),
                          "image": f"{m['width']}x{m['height']}", "spp": m["spp"], "rays": int(rays),
                          "alg_bytes": {k: int(v) for k, v in alg.items()}, "fp64_resolves": int(st["fp64_resolves"])})
    # ---- autotune the batch in both node formats (untimed); the faster tuned batch is the claim ----
    scenes_q = [(t, cam, fr) for (_, t, cam, fr) in q]
    scenes_f = [(t, cam, fr) for (_, t, cam, fr) in f]
    tuned_q, tune_ms_q = H.autotune(ctx, scenes_q, base, reps=2, cache=args.tune_cache, key=f"{BATCH_CONFIG}/quantised")
    tuned_f, tune_ms_f = H.autotune(ctx, scenes_f, base, reps=2, cache=args.tune_cache, key=f"{BATCH_CONFIG}/fp32")
    fmt = "fp32" if 0.0 < tune_ms_f < tune_ms_q else "quantised"
    if args.precision:  # a fixed format instead of the autotuner's choice
        fmt = args.precision
    other = "quantised" if fmt == "fp32" else "fp32"
    main, tuned, tune_ms = (f, tuned_f, tune_ms_f) if fmt == "fp32" else (q, tuned_q, tune_ms_q)
    scenes_main = scenes_f if fmt == "fp32" else scenes_q
    batch = H.Batch(ctx, scenes_main, tuned)
    cams_all = [cam for (_, _, cam, _) in q]

    def paced(b, nsteps, cams):
        # A step renders every scene from its cameras (their 3 KB scene-table upload starts the
        # step, as in an interactive renderer) and ends when the replay has finished, as the
        # sequential comparison's steps do. Replays queued back to back without this pacing ran
        # about 4 % slower each on GB300 (cause not found).
        for _ in range(nsteps):
            b.set_cameras(cams)
            b.launch()
            torch.cuda.current_stream().synchronize()

    def timed(b, nsteps, cams):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        paced(b, nsteps, cams)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / nsteps

    dist.barrier()
    paced(batch, args.warmup, cams_all)
    clocks = Clocks(dev)
    clocks.start()
    ms = timed(batch, args.steps, cams_all)
    clk = clocks.stop()
    ms_max = dist.max(ms)
    value = dist.world * rays_per_step / (ms_max * 1e-3) / 1e6
    # the timed replay's framebuffers, checked below against the oracle
    fb_timed = [np.zeros((m["height"], m["width"], 4), np.float32) for m in mlist]
    batch.download(fb_timed)
    gathered = None
    if dist.world > 1:  # every rank's views to rank 0's host
        from vkhrt_gb300.replicas import gather_to_rank0
        gathered = gather_to_rank0({(dist.rank, i): fb for i, fb in enumerate(fb_timed)}, dist.pg)

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
    ms_seq, lat_seq = sequential(main, tuned)
    # the batching pattern in the other node format too, so that precision and batching can be
    # told apart
    scenes_o = scenes_q if fmt == "fp32" else scenes_f
    tuned_o = tuned_q if fmt == "fp32" else tuned_f
    batch_o = H.Batch(ctx, scenes_o, tuned_o)
    paced(batch_o, args.warmup, cams_all)
    ms_bo = timed(batch_o, args.steps, cams_all)
    mem_q = sum(int(b.info["device_bytes"]) for (b, *_r) in q)
    mem_f = sum(int(b.info["device_bytes"]) for (b, *_r) in f)
    del batch_o, scenes_o
    # ---- the dominant kernel alone, for the roofline: the Phantom scenes of the chosen format as
    # one batch (the Phantom group's frame launch and its FP64 pass) ----
    ph = [i for i, m in enumerate(mlist) if int(m["type"]) == 0]
    batch_ph = H.Batch(ctx, [scenes_main[i] for i in ph], tuned)
    cams_ph = [cams_all[i] for i in ph]
    paced(batch_ph, args.warmup, cams_ph)
    ms_ph = timed(batch_ph, args.steps, cams_ph)
    del batch_ph
    if dist.rank != 0:
        dist.close()
        return
    peak, peak_kind = load_peaks()
    ph_bytes = sum(per_scene[i]["alg_bytes"][fmt] for i in ph)
    ph_rays = sum(per_scene[i]["rays"] for i in ph)
    achieved = ph_bytes / (ms_ph * 1e-3) / 1e9
    kname = "FP32 nodes" if fmt == "fp32" else "8-bit nodes"
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                "kernel": f"frame_kernel<{kname}, Phantom>: the Phantom group of the batch, timed alone",
                "bytes_per_launch": int(ph_bytes), "launch_ms": round(ms_ph, 3), "rays_per_launch": int(ph_rays)}
    roofline.update(measured_bounds(ph_rays, ms_ph, clk, fmt))
    for d, a, b2 in zip(per_scene, lat_f32, lat_seq):
        d["plain_fp32_ms"] = round(float(a), 3)
        d[f"{fmt}_ms"] = round(float(b2), 3)
    # ---- e2e: through the C ABI, each step's cameras in and every framebuffer out to pinned host
    # memory; two frame sets on two streams, so that step k's read-back overlaps step k+1's render
    # (the renders themselves stay in order: each waits for the previous one) ----
    tparams = H.trace_params(jitter=1, seed=17, shading=2, **{"async": 1},
                             **{k: getattr(tuned, k) for k in H.TUNED_FIELDS})
    fsets = [[fr for (_, _, _, fr) in main], [H.Frame(ctx, m["width"], m["height"], m["spp"]) for m in mlist]]
    e2e_batches = [H.Batch(ctx, [(t, cam, fr) for (_, t, cam, _), fr in zip(main, fs)], tparams) for fs in fsets]
    pins = [[torch.empty((m["height"], m["width"], 4), dtype=torch.float32, pin_memory=True) for m in mlist]
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
            b.set_cameras(cams_all, stream=st.cuda_stream)
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
    table_bytes = e2e_batches[0].table_bytes
    del e2e_batches, fsets
    d2h = sum(m["width"] * m["height"] * 16 for m in mlist)
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_max, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32" if fmt == "fp32" else DTYPE_DESC, "data": DATA_DESC,
            "config": batch_config_block(mlist),
            "rays_per_step": int(rays_per_step), "gpu_launches": args.steps * kernels_per_replay(mlist, tuned),
            "autotuned": {"node_format": fmt} | {k: int(getattr(tuned, k)) for k in H.TUNED_FIELDS} |
                         {"mean_ms": round(tune_ms, 3), "mean_ms_fp32": round(tune_ms_f, 3),
                          "mean_ms_quantised": round(tune_ms_q, 3)},
            "clocks": clk,
            "e2e": {"value": round(rays_per_step / te / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": table_bytes,
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": round(te * 1e3, 3)},
            "roofline": roofline,
            "build": {"build_wall_s_quantised": round(build_wall, 3), "strand_generation_s": round(t_gen, 3)},
            "device_bytes": {"quantised": mem_q, "fp32": mem_f},
            "per_scene_latency_ms": {"batched_all_scenes": round(ms, 3),
                                     "plain_fp32": [round(float(x), 2) for x in lat_f32]}}
    if gathered is not None:
        line["replicas"] = {"ranks": dist.world, "frames_gathered_on_rank0": len(gathered),
                            "bytes_gathered": int(sum(v.nbytes for v in gathered.values())),
                            "views": "each scene's camera turned by 2 pi rank / N about the vertical axis"}
    if not args.no_cpu:
        line.update(batch_agreement_and_cpu(ctx, main, models, tuned, fb_timed))
    del q, f, main, batch, scenes_q, scenes_f, scenes_main
    if not args.quick:
        orc = oracle_lib()
        line["configs"] = {name.split("_")[0]: run_config(ctx, name, args, orc) for name in SINGLE_CONFIGS}
    # the comparisons the metric names, last (the line is long; its end is what a log tail keeps)
    line[f"sequential_{fmt}"] = {"value": round(rays_per_step / (ms_seq * 1e-3) / 1e6, 3),
                                 "ms_per_step": round(ms_seq, 3), "what": "the 16 scenes as 16 launches of the tuned "
                                                                          "kernels in the chosen node format"}
    line[f"batched_{other}"] = {"value": round(rays_per_step / (ms_bo * 1e-3) / 1e6, 3), "ms_per_step": round(ms_bo, 3),
                                "autotuned": {k: int(getattr(tuned_o, k)) for k in H.TUNED_FIELDS},
                                "what": f"the same batch on {other} BLASes (the format the autotuner did not choose)"}
    line["plain_fp32"] = {"value": round(rays_per_step / (ms_f32 * 1e-3) / 1e6, 3), "ms_per_step": round(ms_f32, 3),
                          "what": "the same 16 scenes as 16 sequential launches of the FP32 tracer (FP32 nodes and "
                                  "records, no batching, no autotuning)"}
    agreement = line.pop("agreement", None)
    if agreement is not None:
        line["agreement"] = agreement
    print(json.dumps({"per_scene": per_scene}), file=sys.stderr, flush=True)
    print(json.dumps(line), flush=True)
    dist.close()


# Per-ray counters of the dominant kernel (the batch's Phantom group) in each node format, from
# one ncu capture of that launch per format (profiles/frame_kernel_c5_phantom_group*.md): DRAM
# bytes (dram__bytes_read.sum + dram__bytes_write.sum), L2 bytes (lts__t_sectors.sum x 32) and
# warp instructions (smsp__inst_executed.sum), each over the launch's 4,649,742 rays.
NCU_PER_RAY = {
    "quantised": {"dram_bytes": 36.93e6 / 4649742, "l2_bytes": 97101539 * 32 / 4649742,
                  "warp_inst": 6621019102 / 4649742, "source": "profiles/frame_kernel_c5_phantom_group.md"},
    "fp32": {"dram_bytes": 58.94e6 / 4649742, "l2_bytes": 181719966 * 32 / 4649742,
             "warp_inst": 5963512049 / 4649742,
             "source": "profiles/frame_kernel_c5_phantom_group_fp32_vs_quantised.md"},
}


def measured_bounds(rays: int, ms: float, clk: dict, fmt: str = "quantised") -> dict:
    """DRAM traffic, achieved L2 bandwidth and the issue-rate fraction of the dominant kernel in
    node format `fmt`, scaled from its ncu capture's per-ray counters to this launch."""
    c = NCU_PER_RAY.get(fmt)
    if not c:
        return {}
    sm_mhz = clk.get("sm_mhz") or 2070.0
    dram = c["dram_bytes"] * rays
    l2 = c["l2_bytes"] * rays
    inst = c["warp_inst"] * rays
    issue_peak = 152 * 4 * sm_mhz * 1e6  # one warp instruction per scheduler per clock
    return {"traffic": int(dram), "l2": {"bytes_per_launch": int(l2), "achieved_gbs": round(l2 / (ms * 1e-3) / 1e9, 1)},
            "issue": {"warp_inst_per_launch": int(inst), "achieved_per_s": round(inst / (ms * 1e-3), 1),
                      "peak_per_s": issue_peak, "frac": round(inst / (ms * 1e-3) / issue_peak, 4)},
            "counters_from": c["source"]}


def batch_agreement_and_cpu(ctx, q, models, tuned, fb_timed):
    """The timed graph's output against the FP64 oracle: the same scenes, cameras and tuned
    parameters captured again with per-sample hit records, replayed once; its framebuffers must
    equal the timed replay's bit for bit, and its hits and the timed replay's pixels are compared
    with the oracle on about 65,536 sampled rays. Then the oracle's FP32 rate on every pixel of
    every scene (in the reference arm's row bands) and its FP64 rate on one of every 16 rows."""
    import vkhrt_gb300 as H
    orc = oracle_lib()
    threads = orc.orc_hardware_threads()
    rec = H.trace_params(jitter=1, seed=17, shading=2, record_hits=1,
                         **{k: getattr(tuned, k) for k in H.TUNED_FIELDS})
    batch = H.Batch(ctx, [(t, cam, fr) for (_, t, cam, fr) in q], rec)
    batch.launch()
    fb_rec = [np.zeros_like(a) for a in fb_timed]
    batch.download(fb_rec)
    same_fb = all(np.array_equal(a, b) for a, b in zip(fb_timed, fb_rec))
    parts = []
    per = max(1, AGREE_RAYS // len(models))
    scenes = []
    for (b, t, cam, fr), (m, v, r, off), rgba in zip(q, models, fb_timed):
        w, h, spp = m["width"], m["height"], m["spp"]
        _, hits = fr.download(hits=True)
        osc = oracle_scene(orc, int(m["type"]), v, r, m["nstrands"], m["nverts"])
        vi, pi = H.camera_arrays(cam)
        px = sample_pixels(w, h, per // spp, seed=3)
        o = osc.render(vi, pi, w, h, spp=spp, jitter=1, seed=17, shading=2, precision=64, pixel_list=px)
        parts.append(compare_frame(rgba, hits, o, px, spp))
        scenes.append((osc, vi, pi, w, h, spp))
    agreement = merge_compare(parts)
    agreement["graph_framebuffers_match_timed_replay"] = same_fb
    agreement["oracle"] = ORACLE_DESC + ", per scene; hits from the timed graph's parameters, pixels from the timed replay"
    rate, rays, npx, secs = cpu_rate(scenes, 32, range(ROW_BANDS), ROW_BANDS, threads, 1)
    rate64, rays64, _, secs64 = cpu_rate(scenes, 64, [0], FP64_BANDS, threads, 1)
    return {"agreement": agreement,
            "cpu_baseline": {"value": round(rate, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"every pixel of every scene ({npx} pixels, all samples, {rays} rays), FP32 "
                                       f"oracle, {secs:.1f} s, in the reference arm's row bands",
                             "fp64": {"value": round(rate64, 4),
                                      "sample": f"one of every {FP64_BANDS} rows ({rays64} rays), {secs64:.1f} s"}}}


def run_batched_profile(args, dist):
    """`--profile` on the batched workload: the Phantom scenes alone as one batch (the dominant
    kernel of the full batch, its Phantom group), quantised or with --precision fp32, replayed
    warmup + steps times for a profiler, then counted. Parameters from the tune cache when it holds
    the batch's choice for that precision, otherwise from --variant, --refill, --speculative and
    --leaf-again."""
    import torch
    import vkhrt_gb300 as H
    torch.cuda.set_device(dist.local)
    ctx = H.Context(dist.local)
    models = [x for x in batch_models() if int(x[0]["type"]) == 0]
    fp32 = args.precision == "fp32"
    prec = H.Precision.FP32 if fp32 else H.Precision.QUANTISED
    q = []
    for m, v, r, off in models:
        b = H.BottomLevelAccelerationStructure(H.BLASInput(type=m["type"], vertices=v, radius=r, strand_offsets=off,
                                                           precision=prec), ctx)
        t = H.TopLevelAccelerationStructure([b], ctx)
        q.append((b, t, H.orbit_camera(m["width"], m["height"], m["azimuth"], m["elevation"]),
                  H.Frame(ctx, m["width"], m["height"], m["spp"])))
    fields = {"kernel_variant": args.variant, "refill": args.refill, "speculative": args.speculative,
              "leaf_again": args.leaf_again}
    if args.tune_cache and os.path.exists(args.tune_cache):
        key = f"{BATCH_CONFIG}/{'fp32' if fp32 else 'quantised'}"
        fields = {k: int(v) for k, v in json.load(open(args.tune_cache)).get(key, fields).items()
                  if k in H.TUNED_FIELDS}
    p = H.trace_params(jitter=1, seed=17, shading=2, **{"async": 1}, **fields)
    batch = H.Batch(ctx, [(t, cam, fr) for (_, t, cam, fr) in q], p)
    for _ in range(args.warmup):
        batch.launch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        batch.launch()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(args.steps, 1)
    rays = nodes = prims = 0
    for (b, t, cam, fr) in q:  # counted after the replays, so a profiler's launch count starts with them
        H.trace(ctx, t, cam, fr, H.trace_params(jitter=1, seed=17, shading=2, count_stats=1))
        st = fr.stats()
        rays += st["primary_rays"] + st["shadow_rays"]
        nodes += st["nodes_visited"]
        prims += st["prims_tested"]
    print(json.dumps({"profile": "c5 Phantom group", "precision": "fp32" if fp32 else "quantised", "scenes": len(q), "ms_per_replay": round(ms, 3),
                      "rays_per_replay": int(rays), "nodes_visited": int(nodes), "prims_tested": int(prims),
                      "params": {k: int(getattr(p, k)) for k in H.TUNED_FIELDS},
                      "device_bytes": int(sum(b.info["device_bytes"] for (b, *_r) in q))}), flush=True)
    dist.close()


# ------------------------------------------------------------------------------ one configuration
def run_single(args, dist):
    """`--config NAME` (C1-C4): the configuration's frame timed in its own precision (or the
    --precision override); with --profile only the timed launches (for ncu), otherwise also the
    configuration's block (both precisions, agreement)."""
    import torch
    import vkhrt_gb300 as H
    dev = dist.local
    torch.cuda.set_device(dev)
    ctx = H.Context(dev)
    cfg, sp = workload(args.config)
    w, h, spp = cfg["width"], cfg["height"], cfg["spp"]
    v, r, off = H.generate_strands(sp)
    blas = H.BottomLevelAccelerationStructure(
        H.BLASInput(type=cfg["type"], vertices=v, radius=r, strand_offsets=off, precision=cfg["precision"],
                    max_leaf=args.max_leaf, width=args.node_width), ctx)
    tlas = H.TopLevelAccelerationStructure([blas], ctx)
    cam = H.scene_camera(w, h)
    frame = H.Frame(ctx, w, h, spp)
    knobs = dict(spp=spp, jitter=jitter_of(spp), seed=17, shading=2, kernel_variant=args.variant, refill=args.refill,
                 speculative=args.speculative, leaf_again=args.leaf_again)
    H.trace(ctx, tlas, cam, frame, H.trace_params(count_stats=1, **knobs))
    st = frame.stats()
    rays = st["primary_rays"] + st["shadow_rays"]
    dist.barrier()
    clocks = Clocks(dev)
    clocks.start()
    ms = time_frames(ctx, tlas, cam, frame, H.trace_params(**knobs, **{"async": 1}), args.steps, args.warmup)
    clk = clocks.stop()
    ms_max = dist.max(ms)
    value = dist.world * rays / (ms_max * 1e-3) / 1e6
    if dist.rank != 0:
        dist.close()
        return
    info = blas.info
    alg = st["nodes_visited"] * info["node_bytes"] + \
        st["prims_tested"] * prim_test_bytes(info, int(cfg["type"]), int(cfg["precision"])) + w * h * 16
    peak, peak_kind = load_peaks()
    achieved = alg / (ms * 1e-3) / 1e9
    tot = st["warp_cycles_node"] + st["warp_cycles_leaf"] + st["warp_cycles_other"]
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_max, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPE_DESC if int(cfg["precision"]) else "fp32", "data": DATA_DESC,
            "config": single_config_block(cfg, args.config), "rays_per_step": int(rays),
            "gpu_launches": args.steps * (3 if int(cfg["type"]) == 0 else 1),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                         "bytes_per_launch": int(alg), "nodes_visited": int(st["nodes_visited"]),
                         "prims_tested": int(st["prims_tested"])},
            "phase_share": {k: round(st["warp_cycles_" + k] / tot, 4) for k in ("node", "leaf", "other")} if tot else None,
            "clocks": clk}
    if not args.profile:
        del frame, tlas, blas
        line["block"] = run_config(ctx, args.config, args, oracle_lib())
    print(json.dumps(line), flush=True)
    dist.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default=BATCH_CONFIG)
    ap.add_argument("--quick", action="store_true", help="skip the C1-C4 configuration blocks")
    ap.add_argument("--no-cpu", action="store_true", help="skip the oracle agreement and CPU baseline")
    ap.add_argument("--config-steps", type=int, default=10, help="timed frames per precision in each C1-C4 block")
    ap.add_argument("--width", type=int, default=0, help="override the image width (profiling)")
    ap.add_argument("--height", type=int, default=0, help="override the image height (profiling)")
    ap.add_argument("--spp", type=int, default=0, help="override samples per pixel (profiling)")
    ap.add_argument("--precision", choices=["fp32", "quantised"], default=None,
                    help="override the workload's BVH/primitive precision (profiling)")
    ap.add_argument("--variant", type=int, default=0, help="resident blocks per SM: 0/1 = 4, 2 = 3, 3 = 5")
    ap.add_argument("--max-leaf", type=int, default=1, help="primitives per BVH8 leaf (1..3)")
    ap.add_argument("--node-width", type=int, default=0,
                    help="BVH node fan-out 2..8 (0 = 8; a measurement knob)")
    ap.add_argument("--refill", type=int, default=8, help="idle lanes per warp that trigger a fetch (0 = 16)")
    ap.add_argument("--speculative", type=int, default=1, help="speculative traversal (0/1)")
    ap.add_argument("--leaf-again", type=int, default=4,
                    help="repeat the leaf phase while this many lanes hold leaves (0 = once)")
    ap.add_argument("--tune-cache", default=None, help="JSON file that keeps autotuner choices between runs")
    ap.add_argument("--profile", action="store_true",
                    help="the timed launches only, for a profiler (with the batched workload: its Phantom group)")
    args = ap.parse_args()
    for k in ("width", "height", "spp"):
        if getattr(args, k):
            _OVERRIDE[k] = getattr(args, k)
    if args.precision:
        import vkhrt_gb300 as H
        _OVERRIDE["precision"] = H.Precision.QUANTISED if args.precision == "quantised" else H.Precision.FP32
    if args.warmup < 3 and not args.profile:
        args.warmup = 3
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
        dist.close()
        return
    if args.config == BATCH_CONFIG:
        if args.profile:
            run_batched_profile(args, dist)
        else:
            run_batched(args, dist)
        return
    run_single(args, dist)


if __name__ == "__main__":
    main()
