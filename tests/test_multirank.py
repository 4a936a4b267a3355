"""The N > 1 bench path on CPU: two gloo ranks run the rank bookkeeping of bench.py.

Each rank's rounds are disjoint (no Philox stream shared), and the whole-job line takes the
slowest rank's seconds and the summed work — the only exchange between ranks.
"""

from __future__ import annotations

import os
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _rank(rank, world, port, queue):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rounds = [bench.first_round(rank, r) for r in range(1, 12)]
        seconds, scatters = bench.combine_ranks(1.0 + rank, 1000.0 * (rank + 1), "cpu")
        queue.put((rank, rounds, seconds, scatters))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_disjoint_rounds_and_combine_work():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as probe:
        probe.bind(("127.0.0.1", 0))
        port = probe.getsockname()[1]
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, r0, s0, w0), (_, r1, s1, w1) = results
    assert not set(r0) & set(r1)
    assert s0 == s1 == 2.0  # the slowest rank
    assert w0 == w1 == 3000.0  # summed over ranks
