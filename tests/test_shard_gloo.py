"""Multi-GPU host logic on CPU: world_size-2 gloo ranks split a frame by ray range and an uneven
batch by whole scenes, trace their share (the oracle stands in for the GPU here), and rank 0's
gathered hits equal the single-process result bit for bit; the timing reduction takes the
slowest rank."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from bvhtracer_gb300 import shard  # noqa: E402


def test_ray_range_covers_every_ray_once():
    for n in (0, 1, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            spans = [shard.ray_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1


def test_assign_scenes_balances_and_partitions():
    rng = np.random.default_rng(0)
    costs = np.exp(rng.uniform(np.log(64e3), np.log(4e6), 64))
    for world in (2, 4, 8):
        parts = shard.assign_scenes(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(64))
        loads = [costs[p].sum() for p in parts]
        assert max(loads) <= sum(loads) / world + costs.max()  # LPT bound


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle as orc
        from bvhtracer_gb300 import scenes
        # a frame, sharded by ray range
        tris, rays, _ = scenes.icosphere_frame(seed=4, width=64, height=40)
        t, nodes, used = orc.bvh_build(tris)
        b, e = shard.ray_range(len(rays), rank, world)
        local = orc.bvh_intersect(nodes, used, t, rays[b:e])
        full = shard.gather_to_rank0(local, dist, world)
        # an uneven batch, sharded by whole scenes
        specs = [(scenes.soup(300 + 200 * k, k), 500 + 300 * k) for k in range(5)]
        built, items, all_rays, off = [], [], [], 0
        for k, (st, nr) in enumerate(specs):
            tk, nk, uk = orc.bvh_build(st)
            rk = scenes.sphere_rays(nr, 40 + k, box=6.0)
            built.append((tk, nk, uk))
            items.append((k, off, nr, 0))
            all_rays.append(rk)
            off += nr
        items = np.array(items, dtype=[("blas", "<u4"), ("ray_offset", "<u4"), ("ray_count", "<u4"),
                                       ("reserved", "<u4")])
        all_rays = np.concatenate(all_rays)
        mine = shard.assign_scenes([nr for _, nr in specs], world)[rank]
        sub, sub_rays = shard.batch_items_for(items, all_rays, mine)
        parts = []
        for k, it in zip(mine, sub):
            tk, nk, uk = built[k]
            o, c = int(it["ray_offset"]), int(it["ray_count"])
            parts.append(orc.bvh_intersect(nk, uk, tk, sub_rays[o:o + c]))
        local_b = np.concatenate(parts) if parts else np.zeros(0, orc.HIT)
        order = np.concatenate([np.arange(items[k]["ray_offset"], items[k]["ray_offset"] + items[k]["ray_count"])
                                for k in mine]) if mine else np.zeros(0, np.int64)
        got_b = shard.gather_to_rank0(local_b, dist, world)
        got_o = shard.gather_to_rank0(order, dist, world)
        slow = shard.max_over_ranks(1.0 + rank, dist)
        if rank == 0:
            ref = orc.bvh_intersect(nodes, used, t, rays)
            batch = np.zeros(len(all_rays), orc.HIT)
            batch[got_o] = got_b
            ref_b = np.concatenate([orc.bvh_intersect(nk, uk, tk, all_rays[o:o + c])
                                    for (tk, nk, uk), (_, o, c, _) in zip(built, items.tolist())])
            ok = (full.tobytes() == ref.tobytes()) and (batch.tobytes() == ref_b.tobytes()) and slow == world
            with open(os.path.join(out_dir, "ok"), "w") as f:
                f.write("1" if ok else "0")
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_the_single_process_result(tmp_path):
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    assert (tmp_path / "ok").read_text() == "1"
