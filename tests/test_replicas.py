"""Multi-process paths on CPU: two gloo ranks run the replica plumbing that
bench.py uses for --gpus N (barrier, max-over-ranks timing, grid shares)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as td  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from stencil3d_gb300.replicas import Replicas, shard  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    r = Replicas()
    r.barrier()
    t = r.max(10.0 + rank)          # the slowest rank's time
    n = r.sum(len(shard(64, rank, world)))
    # each replica's context names its own GPU (bench.py: device = LOCAL_RANK)
    import stencil3d_gb300 as S
    o = S.default_opts(25, "wave", "f32", device=r.local_rank)
    dev = S.plan(S.Grid(16, 16, 16, 4, 4, 4), o).device
    r.barrier()
    r.close()
    out.put((rank, t, n, dev))


def test_two_gloo_ranks_agree_on_max_time_and_cover_all_grids():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [t for _, t, _, _ in res] == [11.0, 11.0]
    assert [n for _, _, n, _ in res] == [64.0, 64.0]
    assert [d for _, _, _, d in res] == [0, 1]


def test_shard_is_a_partition():
    for world in (1, 2, 3, 8):
        seen = sorted(i for r in range(world) for i in shard(64, r, world))
        assert seen == list(range(64))
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def test_single_process_needs_no_group():
    r = Replicas()
    assert r.world == int(os.environ.get("WORLD_SIZE", "1"))
    if r.world == 1:
        assert r.max(3.0) == 3.0 and r.sum(2.0) == 2.0
    r.close()
