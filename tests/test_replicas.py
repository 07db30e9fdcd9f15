"""The multi-GPU path of the benchmark is replicas (independent windows per rank, no collective on
the data path): two gloo ranks on CPU check the barrier and max/sum reductions, the whole-job
throughput rule (summed work over the slowest rank's time) and that every rank draws its own
windows."""
import multiprocessing as mp
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    import bench
    from nav24_gb300.synth import Synth
    d = bench.Dist(2, rank, backend="gloo")
    d.barrier()
    mx, sm = d.max(float(rank + 1)), d.sum(float(rank + 1))
    rate = bench.whole_job_rate(d, work=100.0 * (rank + 1), seconds=1.0 + rank)
    digest = Synth(2, seed=bench.replica_seed(rank), n_windows=4).digest()
    q.put((rank, mx, sm, rate, digest))
    d.barrier()
    d.close()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, mx0, sm0, rate0, dg0), (_, mx1, sm1, rate1, dg1) = out
    assert mx0 == mx1 == 2.0 and sm0 == sm1 == 3.0
    assert rate0 == rate1 == pytest.approx(300.0 / 2.0)
    assert dg0 != dg1
