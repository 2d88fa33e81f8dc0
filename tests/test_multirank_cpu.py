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


def _shard_worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path[:0] = [ROOT, os.path.join(ROOT, "vipp-nbody-bench_gb300")]
    import math

    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    import vipp_gb300
    w, r, _ = bench.dist_setup()
    rng = np.random.default_rng(3)  # the batching form's 512 systems, as bench.batch_measure draws them
    sizes = np.rint(np.exp(rng.uniform(math.log(1024), math.log(65536), 512))).astype(np.int64)
    first, last = vipp_gb300.shard_systems(sizes, w)[r]
    mine = torch.tensor([first, last, int(sizes[first:last].sum())], dtype=torch.int64)
    got = [torch.zeros(3, dtype=torch.int64) for _ in range(w)]
    dist.all_gather(got, mine)
    slowest = bench.max_over_ranks(1.0 + 0.25 * r, w)  # each rank's batch-step time
    q.put((r, [g.tolist() for g in got], slowest, int(sizes.sum())))
    dist.destroy_process_group()


def test_batch_systems_sharded_over_two_ranks_gloo():
    """The batching form over 2 ranks (bench.py --gpus 2): each rank takes a
    contiguous run of the 512 systems, the runs cover every system once, hold
    about equal particle counts, and the batch value uses the slowest rank's
    time (strong scaling: the same 512 systems whatever the rank count)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    runs = out[0][1]
    assert runs == out[1][1]  # every rank sees the same split
    assert runs[0][0] == 0 and runs[0][1] == runs[1][0] and runs[1][1] == 512
    total = out[0][3]
    assert runs[0][2] + runs[1][2] == total
    assert max(runs[0][2], runs[1][2]) <= 0.5 * total + 65536  # within one system of an even split
    assert all(o[2] == 1.25 for o in out)


def test_shard_systems_cover_and_balance():
    sys.path.insert(0, os.path.join(ROOT, "vipp-nbody-bench_gb300"))
    import vipp_gb300
    rng = np.random.default_rng(1)
    sizes = rng.integers(0, 70000, 300)
    sizes[5] = 0
    for world in (1, 2, 3, 4, 8, 16):
        runs = vipp_gb300.shard_systems(sizes, world)
        assert len(runs) == world and runs[0][0] == 0 and runs[-1][1] == len(sizes)
        assert all(runs[i][1] == runs[i + 1][0] and runs[i][0] <= runs[i][1] for i in range(world - 1))
        loads = [int(sizes[a:b].sum()) for a, b in runs]
        assert sum(loads) == int(sizes.sum())
        assert max(loads) <= sizes.sum() / world + sizes.max()
