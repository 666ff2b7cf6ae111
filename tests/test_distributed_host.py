"""CPU, world size 2 over gloo: drop sharding and the end-of-run counter exchange of
the multi-GPU path (one process per GPU, no data-path collective). Each rank
simulates its shard of oracle drops; the summed counters equal one process
simulating every drop, because every draw is a Philox stream of (seed, drop)."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from hermespy_gb300.distributed import max_over_ranks, rank_base, shard, sum_counters
from oracle.link import LinkConfig, simulate_drop
from tests.configs import siso_channel, siso_frame

SEED = 2024
LEVELS = (4.0, 12.0)
TOTAL = 5  # drops per level, split 3 + 2 over the two ranks


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _counters(drop0: int, count: int) -> np.ndarray:
    cfg = LinkConfig(siso_frame(), siso_channel(), 15.36e6, 1, 1, "ls", "zf", "ebn0")
    out = np.zeros((len(LEVELS), 3), np.int64)  # errors, bits, drops
    for i, lv in enumerate(LEVELS):
        for d in range(drop0, drop0 + count):
            r = simulate_drop(cfg, SEED, i * 1000 + d, lv)
            out[i] += (r["errors"], r["bits"], 1)
    return out


def _worker(rank: int, world: int, port: int, path: str) -> None:
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, n = shard(TOTAL, rank, world)
        total = sum_counters(_counters(lo, n))
        slowest = max_over_ranks(10.0 + rank)
        if rank == 0:
            np.savez(path, total=total, slowest=slowest)
    finally:
        dist.destroy_process_group()


def test_shard_partition():
    for total in (0, 1, 5, 8192, 10001):
        for world in (1, 2, 3, 8):
            parts = [shard(total, r, world) for r in range(world)]
            assert sum(n for _, n in parts) == total
            starts = [lo for lo, _ in parts]
            assert starts == sorted(starts) and all(parts[i][0] + parts[i][1] == parts[i + 1][0]
                                                    for i in range(world - 1))
            assert max(n for _, n in parts) - min(n for _, n in parts) <= 1
    assert rank_base(1) == 1 << 44 and rank_base(0) == 0
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def test_two_ranks_match_one_process(tmp_path):
    path = str(tmp_path / "out.npz")
    mp.spawn(_worker, args=(2, _free_port(), path), nprocs=2, join=True)
    got = np.load(path)
    np.testing.assert_array_equal(got["total"], _counters(0, TOTAL))
    assert float(got["slowest"]) == 11.0


def test_single_process_helpers_without_group():
    c = np.array([[1, 2, 3]], np.int64)
    np.testing.assert_array_equal(sum_counters(c), c)
    assert max_over_ranks(3.5) == 3.5
    assert torch.distributed.is_available()
