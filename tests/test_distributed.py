"""The N-GPU host logic on two CPU ranks (gloo): the benchmark's max-over-ranks
timing and the sharded KL objective, whose all-reduced loss and gradient must
equal the single-process values on the whole sample set (computed here with
the oracle, so no GPU is needed)."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    from oracle import oracle as O
    from mpart_gb300.distributed import max_over_ranks, shard_range, sharded_kl_objective
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = max_over_ranks(1.0 + rank)
        om = O.OracleTriangularMap(3, 3, 2)
        coef = np.random.default_rng(0).normal(0.0, 0.1, om.num_coeffs)
        x = np.random.default_rng(1).standard_normal((3, 301))
        a, b = shard_range(x.shape[1], rank, world)
        cs = om.split(coef)
        losses, grads = [], []
        for i, c in enumerate(om.comps):
            l, g = O.fast_gaussian_reverse_kl(c, cs[i], np.ascontiguousarray(x[:c.input_dim, a:b]))
            losses.append(l)
            grads.append(g)
        loss, grad = sharded_kl_objective(losses, np.concatenate(grads), b - a)
        q.put((rank, t, loss, grad))
    finally:
        dist.destroy_process_group()


def test_two_rank_host_logic(oracle):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    O = oracle
    om = O.OracleTriangularMap(3, 3, 2)
    coef = np.random.default_rng(0).normal(0.0, 0.1, om.num_coeffs)
    x = np.random.default_rng(1).standard_normal((3, 301))
    cs = om.split(coef)
    ref = [O.fast_gaussian_reverse_kl(c, cs[i], np.ascontiguousarray(x[:c.input_dim])) for i, c in enumerate(om.comps)]
    ref_loss = np.array([r[0] for r in ref])
    ref_grad = np.concatenate([r[1] for r in ref])
    for rank, t, loss, grad in out:
        assert t == 2.0  # the slower rank's time
        np.testing.assert_allclose(loss, ref_loss, rtol=1e-12)
        np.testing.assert_allclose(grad, ref_grad, rtol=1e-10, atol=1e-14)


def test_shard_range_covers_points():
    from mpart_gb300.distributed import shard_range
    for n in (0, 1, 7, 301):
        for world in (1, 2, 3, 8):
            spans = [shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            assert max(b - a for a, b in spans) - min(b - a for a, b in spans) <= 1
