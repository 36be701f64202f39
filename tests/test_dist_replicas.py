"""The N > 1 path of bench.py on CPU: two ranks over gloo (127.0.0.1).  Shells are independent replicas,
so the only cross-rank operations are the barrier around the timed region and the max-reduction of the
elapsed time; every rank seeds its own shell (seed + rank) and the reported value is the steps of all
ranks over the slowest rank's time (weak scaling)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from spectraldoublediffusiveconvection_gb300.seeds import seeded_state
    ws, rk, local = bench.dist_env()
    dist.init_process_group("gloo", rank=rk, world_size=ws)
    try:
        bench.barrier(ws)
        elapsed = 1.0 + rk                     # rank 1 is the slower one
        t = bench.max_over_ranks(elapsed, ws, torch.device("cpu"))
        x = seeded_state(16, 7, bench.WORKLOAD["seed"] + rk)
        steps_all = 100 * ws
        out.put((rk, ws, local, t, steps_all / t, float(x[0])))
        bench.barrier(ws)
    finally:
        dist.destroy_process_group()


def test_two_replica_ranks_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 and r[2] == r[0] for r in res)
    assert all(r[3] == 2.0 for r in res)                  # max over ranks
    assert all(r[4] == pytest.approx(100.0) for r in res)  # 200 steps of both ranks / 2 s
    assert res[0][5] != res[1][5]                          # each rank its own seeded shell


def test_reference_arm_is_rank_zero_only(monkeypatch):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class A:
        steps, warmup, gpus = 2, 3, 2
    assert bench.bench_reference(A()) == 0                # rank 1 exits 0 without work
