"""Multi-rank path on CPU: instances are partitioned across 2 gloo ranks with
no data-path collective; every rank derives the same partition, each instance
is owned exactly once, and the gathered results equal a single-rank run."""
import os
import socket

import numpy as np
import pytest

from psfun_gb300.shard import shard_instances


def test_partition_properties():
    rng = np.random.default_rng(3)
    costs = rng.integers(1000, 100000, size=64)
    for world in (1, 2, 3, 8):
        parts = shard_instances(costs, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(64))
        loads = [costs[p].sum() for p in parts]
        assert max(loads) - min(loads) <= costs.max()
        assert parts == shard_instances(costs, world)  # deterministic


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from oracle import oracle as orc
    from psfun_gb300 import matrices
    from psfun_gb300.shard import gather_results, my_instances
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    orc.set_threads(1)  # fixed reduction order
    probs = matrices.uneven_batch(count=6, nrhs=1, scale=0.02)
    costs = [p.A.nnz for p in probs]
    local = {}
    for k in my_instances(costs, rank, world):
        p = probs[k]
        r = orc.krylov("LANCZOS", orc.serial("EXP", "CHBSYM", 1.0), orc.Csr.from_scipy(-p.params["t"] * p.A),
                       p.x[0], 1e-8, itmax=60)
        local[k] = r["y"]
    allres = gather_results(local, world)
    if rank == 0:
        q.put({k: v.tolist() for k, v in allres.items()})
    dist.destroy_process_group()


def test_two_rank_gloo_matches_single_rank():
    pytest.importorskip("torch")
    import multiprocessing as mp
    from oracle import oracle as orc
    from psfun_gb300 import matrices
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    probs = matrices.uneven_batch(count=6, nrhs=1, scale=0.02)
    assert sorted(res) == list(range(6))
    orc.set_threads(1)
    for k, p in enumerate(probs):
        r = orc.krylov("LANCZOS", orc.serial("EXP", "CHBSYM", 1.0), orc.Csr.from_scipy(-p.params["t"] * p.A),
                       p.x[0], 1e-8, itmax=60)
        assert np.array_equal(np.array(res[k]), r["y"])
