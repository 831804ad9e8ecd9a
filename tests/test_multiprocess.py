"""Replicas on CPU ranks (gloo, world size 2): bench.py's bookkeeping (barrier, max over ranks,
the whole-job value N x rays / max time), and the partition of a job (vkhrt_gb300.replicas):
interleaved rows of a scene and the scenes of a batch dealt to ranks, each rank rendering its
share and rank 0 gathering the framebuffers. Rays are independent, so the only exchange is that
host-side gather."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    assert d.rank == rank and d.world == world
    d.barrier()
    ms = 10.0 + 5.0 * rank          # the slower rank decides the job time
    m = d.max(ms)
    rays_per_rank = 1_000_000
    value = d.world * rays_per_rank / (m * 1e-3) / 1e6
    q.put((rank, m, value))
    d.close()


@pytest.mark.parametrize("world", [2])
def test_replica_max_over_ranks(world):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    for rank, m, value in res:
        assert m == 15.0
        assert abs(value - world * 1e6 / 15e-3 / 1e6) < 1e-9


def test_single_process_dist_is_trivial():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    d = bench.Dist()
    assert d.world == 1 and d.rank == 0 and d.max(3.5) == 3.5
    d.barrier()
    d.close()


def test_scene_partition_is_balanced_and_deterministic():
    sys.path.insert(0, ROOT)
    from vkhrt_gb300.replicas import partition_scenes
    work = [5, 90, 7, 40, 40, 3, 60, 12]
    parts = partition_scenes(work, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(work)))
    loads = [sum(work[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(work)  # greedy largest-first
    assert parts == partition_scenes(list(work), 3)
    assert partition_scenes(work, 1) == [list(range(len(work)))]


def _render_worker(rank, world, port, q):
    """Renders this rank's share with the CPU oracle: the rows y = rank (mod world) of scene 0 and
    the scenes dealt to it; rank 0 gathers and compares with its own single-rank renders."""
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    import torch.distributed as dist

    import vkhrt_gb300 as H
    from hairscene import PHANTOM, LSS, OracleScene, lines_from_strands, load_oracle, oracle_geometry
    from vkhrt_gb300.replicas import assemble_rows, gather_to_rank0, partition_scenes, row_pixels
    dist.init_process_group("gloo", rank=rank, world_size=world)
    orc = load_oracle()
    lib = H.bind_workload(orc)
    scenes = []
    for k, (gt, ns, w, h) in enumerate([(PHANTOM, 150, 48, 40), (LSS, 200, 40, 32), (PHANTOM, 120, 32, 24),
                                        (LSS, 90, 56, 24)]):
        v, r, off = H.generate_strands(H.StrandParams(seed=400 + k, nstrands=ns, nverts=16), lib=lib)
        lines, lrad = lines_from_strands(v, r, off)
        vi, pi = H.camera_arrays(H.orbit_camera(w, h, 0.5 * k, 0.1, lib=lib))
        scenes.append((OracleScene(orc, [(gt, *oracle_geometry(orc, gt, lines, lrad))]), vi, pi, w, h))

    def render(sc, px=None):
        osc, vi, pi, w, h = sc
        return osc.render(vi, pi, w, h, shading=2, precision=64, pixel_list=px, threads=2)["fb"]

    osc0, vi0, pi0, w0, h0 = scenes[0]
    local = {("rows", rank, world): render(scenes[0], row_pixels(w0, h0, rank, world))}
    mine = partition_scenes([w * h for (_, _, _, w, h) in scenes], world)[rank]
    for i in mine:
        local[("scene", i)] = render(scenes[i])
    got = gather_to_rank0(local, dist)
    ok = True
    if rank == 0:
        frame = assemble_rows(w0, h0, 4, {(k[1], k[2]): v for k, v in got.items() if k[0] == "rows"})
        ok &= np.array_equal(frame.reshape(-1, 4), render(scenes[0]))
        for i in range(len(scenes)):
            ok &= np.array_equal(got[("scene", i)], render(scenes[i]))
    else:
        ok &= got is None
    q.put((rank, bool(ok), mine))
    dist.destroy_process_group()


def test_partitioned_renders_gather_to_the_single_rank_frames():
    """Two gloo ranks render disjoint shares (interleaved rows of one scene, and the scenes dealt
    by work) with the CPU oracle; the frames gathered on rank 0 equal single-rank renders bit for
    bit."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_render_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert all(ok for _, ok, _ in res)
    assert sorted(i for _, _, mine in res for i in mine) == [0, 1, 2, 3]
