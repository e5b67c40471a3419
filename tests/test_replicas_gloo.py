"""Multi-rank path of bench.py on CPU: two gloo ranks rendezvous on
127.0.0.1, meet at the barrier and agree on the max-over-ranks time that
becomes the whole-job figure (replicas only: no data-path collective)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out_dir):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    got_ws, got_rank, _ = bench.dist_setup()
    bench.barrier(got_ws)
    v = bench.allmax(got_ws, 1.5 + rank)  # each replica's own step time
    bench.barrier(got_ws)
    with open(os.path.join(out_dir, f"r{rank}"), "w") as f:
        f.write(f"{got_ws} {got_rank} {v}")
    import torch.distributed as dist
    dist.destroy_process_group()


@pytest.mark.parametrize("ws", [2])
def test_gloo_replicas_agree_on_max(tmp_path, ws):
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, str(tmp_path))) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(ws):
        got_ws, got_rank, v = open(tmp_path / f"r{r}").read().split()
        assert (int(got_ws), int(got_rank)) == (ws, r)
        assert float(v) == 1.5 + (ws - 1)
