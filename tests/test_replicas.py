"""Replica aggregation at world size 2 on CPU (gloo): the timing reduction the
multi-GPU bench uses, and that replicas evaluate different boxes whose
oracle losses each rank computes alone (no data-path collective)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        _body(rank, world, q)
    except Exception as e:  # report instead of leaving the parent waiting
        q.put((rank, "error", repr(e)))
    finally:
        dist.destroy_process_group()


def _body(rank, world, q):
    from jerald_gb300 import replicas, synth
    from oracle.ldl import LDLOracle
    w, r, lr = replicas.world()
    ms = 10.0 + 5.0 * rank
    rate, slow = replicas.aggregate_rate(ms)
    n, box = 8, 20.0
    X = synth.zeldovich(n, box, 0.5, seed=replicas.replica_seed(rank)).astype(np.float64)
    o = LDLOracle((n,) * 3, box, kind="sm", L1=True)
    p = synth.default_params(2)
    loss, _ = o.loss_and_grad(p, X, np.ones((n,) * 3), 2)
    losses = [None] * world
    dist.all_gather_object(losses, loss)  # test-side check only
    q.put((rank, w, r, lr, rate, slow, losses))


def test_replica_aggregation_world2():
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
    out.sort(key=lambda t: t[0])
    errors = [t for t in out if t[1] == "error"]
    assert not errors, errors
    for rank, w, r, lr, rate, slow, losses in out:
        assert (w, r, lr) == (2, rank, rank)
        assert slow == 15.0                      # max over ranks
        assert abs(rate - 2 * 1000.0 / 15.0) < 1e-9
        assert losses[0] != losses[1]            # different boxes per replica


def test_single_process_is_identity():
    from jerald_gb300 import replicas
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.aggregate_rate(20.0) == (50.0, 20.0)
