"""The N>1 path of bench.py on the CPU: world size 2 over gloo. Every rank
runs an independent replica (no data-path collective); the host-side
barrier and the whole-job aggregation (units of all ranks over the slowest
rank's time) go over gloo, and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    bench.barrier()
    # rank r processed (r+1) * 1e6 units in (r+1) * 10 ms
    value, ms_max = bench.aggregate((rank + 1) * 1e6, (rank + 1) * 10.0)
    ref = bench.run_reference(None) if rank == 1 else "skipped"
    bench.barrier()
    out.put((rank, value, ms_max, ref))
    bench._pg.destroy_process_group()


def test_two_rank_aggregation_and_reference_arm():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms_max, ref in res:
        assert ms_max == 20.0
        assert value == pytest.approx(3e6 / 0.020)
    assert res[1][3] is None  # the reference arm does no work off rank 0
