"""The multi-process path of bench.py on CPU (gloo, world size 2): the path
shards by replica (each rank registers its own scene), so the only
cross-rank steps are the barrier around the timed region and the max over
ranks of the step time; rank 0 alone reports."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    got_ws, got_rank, local, pg = bench.dist_setup()
    bench.barrier(pg)
    step_ms = 10.0 * (rank + 1)          # each rank's own step time
    worst = bench.allmax(pg, step_ms)    # what rank 0 reports
    bench.barrier(pg)
    out[rank] = (got_ws, got_rank, local, worst)
    pg.destroy_process_group()


def test_two_ranks_share_the_max_step_time():
    ws, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    assert res[0] == (2, 0, 0, 20.0)
    assert res[1] == (2, 1, 1, 20.0)


def test_single_process_needs_no_process_group(monkeypatch):
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    import bench
    ws, rank, local, pg = bench.dist_setup()
    assert (ws, rank, local, pg) == (1, 0, 0, None)
    assert bench.allmax(pg, 3.5) == 3.5
    bench.barrier(pg)
