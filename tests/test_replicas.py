"""bench.py's multi-GPU mode is replicas (rays are independent; no exchange
step): each rank renders its own cameras of the same world, and the job's
rate is the rays of all ranks over the slowest rank's time.  Checked here
with two gloo ranks on the CPU."""
import importlib.util
import os
import socket
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out: dict) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b = _bench()
        rays, ms, e2e = (1000.0 + rank, 5.0 * (rank + 1), 0.5 + rank)
        out[rank] = b.aggregate(torch, dist, world, torch.device("cpu"), rays, ms, e2e)
    finally:
        dist.destroy_process_group()


def test_aggregate_sums_rays_and_takes_the_slowest_rank():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
        res = dict(out)
    for r in range(world):
        assert res[r] == (2001.0, 10.0, 1.5)


def test_single_rank_is_unchanged():
    assert _bench().aggregate(torch, dist, 1, None, 7.0, 3.0, 2.0) == (7.0, 3.0, 2.0)


def test_ranks_render_distinct_cameras_of_one_world(vtlib):
    b = _bench()
    d0, _, c0, p0 = b.setup_scene(vtlib, 0)
    d1, _, c1, p1 = b.setup_scene(vtlib, 1)
    assert bytes(d0) == bytes(d1) and bytes(p0) == bytes(p1)
    assert {bytes(c) for c in c0}.isdisjoint({bytes(c) for c in c1})
