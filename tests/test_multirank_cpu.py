"""bench.py's multi-GPU path on CPU: replicas (one independent system per
rank, no collective on the data path), a barrier around the timed steps and
the maximum of the ranks' times. Run as world size 2 on the gloo backend,
rendezvous on 127.0.0.1."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    w, r, local = bench.dist_setup()
    bench.barrier(w)
    slowest = bench.max_over_ranks(0.5 + rank, w)  # each rank's device time
    x, _ = bench.plummer(1000, 2 + r)              # replica r's system
    q.put((r, w, local, slowest, float(x[0, 0])))
    dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out) and [o[2] for o in out] == [0, 1]
    assert all(o[3] == 1.5 for o in out)  # both ranks see the slowest time
    assert out[0][4] != out[1][4]         # independent systems per replica
    # value = particles of all ranks x steps / slowest time (weak scaling)
    n, steps = 1000, 10
    assert np.isclose(n * 2 * steps / out[0][3], 13333.333, rtol=1e-6)
