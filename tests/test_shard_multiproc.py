"""World-size-2 gloo test of the N>1 path: scenes are sharded across ranks
with no data-path collective; the union of the ranks' pair sets (computed
here by the CPU oracle per shard) equals the single-process result, and
each scene lands on exactly one rank."""
import os
import socket

import numpy as np
import pytest

from gsap_gb300.shard import local_offsets, shard_scenes


def test_shard_covers_every_scene_once():
    rng = np.random.default_rng(0)
    for S in (1, 2, 3, 17, 4096):
        sizes = rng.integers(0, 500, S)
        off = np.concatenate([[0], np.cumsum(sizes)])
        for world in (1, 2, 3, 8):
            got = [shard_scenes(off, world, r) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == S
            for a, b in zip(got, got[1:]):
                assert a[1] == b[0]
            if S >= world * 4 and sizes.sum() > 0:
                loads = [off[b] - off[a] for a, b in got]
                assert max(loads) <= sizes.sum() / world + sizes.max()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist

    import oracle
    from gsap_gb300 import scenes
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mn, mx, off = scenes.batched_aabb(S=9, seed=5, lo=16, hi=800)
    s0, s1 = shard_scenes(off, world, rank)
    loc, base = local_offsets(off, s0, s1)
    pairs = []
    for s in range(s1 - s0):
        a, b = base + loc[s], base + loc[s + 1]
        p = oracle.bf_aabb(mn[a:b], mx[a:b]).astype(np.int64) + a
        pairs.append(p)
    mine = np.concatenate(pairs) if pairs else np.zeros((0, 2), np.int64)
    # only the final counts are reduced
    cnt = torch.tensor([len(mine), s1 - s0], dtype=torch.int64)
    dist.all_reduce(cnt)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine.tolist())
    if rank == 0:
        q.put((int(cnt[0]), int(cnt[1]), gathered))
    dist.destroy_process_group()


def test_two_rank_scene_shards_match_single_process():
    import multiprocessing as mp

    import oracle
    from gsap_gb300 import scenes
    oracle.build()  # once, before the workers load it
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    total, nscenes, gathered = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    mn, mx, off = scenes.batched_aabb(S=9, seed=5, lo=16, hi=800)
    want = np.concatenate([oracle.bf_aabb(mn[off[s]:off[s + 1]], mx[off[s]:off[s + 1]]).astype(np.int64) + off[s]
                           for s in range(9)])
    got = np.array([p for part in gathered for p in part], np.int64).reshape(-1, 2)
    got = got[np.lexsort((got[:, 1], got[:, 0]))]
    assert nscenes == 9
    assert total == len(want)
    assert np.array_equal(got, want)
