"""Replicas across GPUs: every rank holds its own copy of the scenes (BVH builds are deterministic,
so the copies are identical) and traces a disjoint share of the work; the one exchange is a
gather of the finished framebuffers to rank 0's host. Rays are independent, so no device
collective is needed and nothing in the trace waits on another rank.

Two partitions:
  * scenes: a batch's scenes are dealt to ranks by estimated work (pixels x samples), largest
    first onto the least-loaded rank, ties by index, so every rank computes the same assignment;
  * rows: one scene's image rows y = rank (mod world), interleaved so that sky and hair fall to
    every rank alike.
The gather uses torch.distributed (gloo on CPU ranks, NCCL's host-object path on GPU ranks).
"""
from __future__ import annotations

import numpy as np


def partition_scenes(work: list[int], world: int) -> list[list[int]]:
    """Scene indices per rank: greedy largest-first onto the least-loaded rank (ties: the lower
    rank, and scenes of equal work in index order). Deterministic on every rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(work)), key=lambda k: (-int(work[k]), k)):
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(i)
        load[r] += int(work[i])
    return [sorted(x) for x in out]


def row_pixels(width: int, height: int, rank: int, world: int) -> np.ndarray:
    """The pixels (row-major indices, scanline order) of the rows y = rank (mod world)."""
    ys = np.arange(rank, height, world, dtype=np.uint32)
    return (ys[:, None] * np.uint32(width) + np.arange(width, dtype=np.uint32)[None, :]).reshape(-1)


def gather_to_rank0(local: dict, dist) -> dict | None:
    """Every rank's {key: array} to rank 0 (None elsewhere); `dist` is torch.distributed with an
    initialised process group, or None for a single rank."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return dict(local)
    parts = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
    dist.gather_object(local, parts, dst=0)
    if dist.get_rank() != 0:
        return None
    merged: dict = {}
    for p in parts:
        for k, v in p.items():
            if k in merged:
                raise ValueError(f"two ranks produced {k!r}")
            merged[k] = v
    return merged


def assemble_rows(width: int, height: int, channels: int, parts: dict) -> np.ndarray:
    """A frame (height, width, channels) from per-rank row shares: parts[(rank, world)] holds
    the pixels of row_pixels(width, height, rank, world) in order."""
    out = np.zeros((height * width, channels), np.float32)
    seen = np.zeros(height * width, bool)
    for (rank, world), px in parts.items():
        idx = row_pixels(width, height, rank, world)
        if seen[idx].any():
            raise ValueError("row shares overlap")
        out[idx] = px
        seen[idx] = True
    if not seen.all():
        raise ValueError("row shares do not cover the frame")
    return out.reshape(height, width, channels)
