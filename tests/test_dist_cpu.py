"""The multi-rank path of bench.py on CPU: two gloo ranks (replicas, one
process each) reduce their timings and units the way torchrun ranks do on
GPUs: max of the times, sum of the units."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        import bench
        w, r = bench.dist_info()
        vals = bench.aggregate([(1.5 + rank, "max"), (10.0 * (rank + 1), "sum")], w)
        # each rank builds its own replica workload (seeded by rank)
        scs, _ = bench.workload("batch128", rank)
        q.put((r, w, vals, scs[0].num_tets))
    finally:
        dist.destroy_process_group()


def test_bench_aggregation_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    for _, _, vals, _ in out:
        assert vals == [2.5, 30.0]
    assert out[0][3] != out[1][3]  # the replicas' meshes differ
