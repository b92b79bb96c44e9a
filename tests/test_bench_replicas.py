"""bench.py's multi-GPU path runs N independent replicas (the step does not
shard: one tank per run); the whole-job figures are the slowest rank's time
and the pairs of all ranks. The aggregation is checked here with two gloo
ranks on the CPU. CPU only."""

import os
import socket



def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import sys
    from pathlib import Path

    import torch.distributed as dist

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: a timed region of (1 + r) s with 100 * (r + 1) pairs, an e2e of (3 - r) s with 10 pairs
        res = bench.aggregate_replicas(1.0 + rank, 100 * (rank + 1), 3.0 - rank, 10, dist, "cpu")
        out.put((rank, res))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_with_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        t_s, pairs, e2e_s, e2e_pairs = results[r]
        assert t_s == 2.0 and pairs == 300.0 and e2e_s == 3.0 and e2e_pairs == 20.0


def test_single_rank_aggregation_is_the_identity():
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench

    assert bench.aggregate_replicas(0.5, 7, 0.25, 3) == (0.5, 7.0, 0.25, 3.0)
