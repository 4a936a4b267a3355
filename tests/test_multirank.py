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


def _replica(rank, world, port, queue):
    import numpy as np
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    for path in (str(ROOT), str(ROOT / "monki-gpu_gb300"), str(ROOT / "tests")):
        sys.path.insert(0, path)
    import monki.scenes as scenes
    from monki.execution import BatchControls
    from monki.replicas import RoundMoments, all_reduce, rank_rounds
    from oracle import oracle
    from oracle_backend import oracle_backend

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        scene = scenes.layered_cloud(6, 1, nx=6, ny=4)
        backend = oracle_backend(oracle, seed=77)
        backend.prepare(scene)
        mine = rank_rounds(33, rank, world)
        local = RoundMoments.of([backend.run_batch(BatchControls(r, 6)) for r in mine], 6)
        total = all_reduce(local)
        queue.put((rank, mine, total.rounds, total.stokes, total.squares, total.paths, total.weights,
                   *total.estimate()))
    finally:
        dist.destroy_process_group()


def test_two_replicas_sum_to_one_process_running_the_same_rounds(oracle):
    """Two gloo ranks run disjoint rounds of one scene (layer paths on) and all-reduce
    their FP64 round moments: the sums, the radiance and its standard error equal one
    process running all 33 rounds."""

    import socket

    import numpy as np
    import torch.multiprocessing as mp

    import monki.scenes as scenes
    from monki.execution import BatchControls
    from monki.replicas import RoundMoments
    from oracle_backend import oracle_backend

    with socket.socket() as probe:
        probe.bind(("127.0.0.1", 0))
        port = probe.getsockname()[1]
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    procs = [ctx.Process(target=_replica, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted((queue.get(timeout=300) for _ in procs), key=lambda item: item[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert not set(results[0][1]) & set(results[1][1])
    assert sorted(results[0][1] + results[1][1]) == list(range(1, 34))

    scene = scenes.layered_cloud(6, 1, nx=6, ny=4)
    backend = oracle_backend(oracle, seed=77)
    backend.prepare(scene)
    single = RoundMoments.of([backend.run_batch(BatchControls(r, 6)) for r in range(1, 34)], 6)
    radiance, error = single.estimate()
    for rank, _, rounds, stokes, squares, paths, weights, rad, err in results:
        assert rounds == 33
        for ours, theirs in ((stokes, single.stokes), (squares, single.squares), (paths, single.paths),
                             (weights, single.weights), (rad, radiance), (err, error)):
            np.testing.assert_allclose(ours, theirs, rtol=1e-12, atol=1e-300)
    assert np.all(error[0] < 999.0)
