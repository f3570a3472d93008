"""Event-sharded FdF across two gloo ranks on the CPU: each rank evaluates
the FP64 oracle over its contiguous share of the events (only rank 0 adds
the normalisation and prior terms) and one all-reduce of P + 1 doubles
combines them; the result must equal the single-process FdF over all events
to FP64 rounding (1e-11 relative), with normalised and unnormalised
amplitudes and with the half-Cauchy prior."""
import os
import socket

import numpy as np
import pytest

from rootpwa_gb300 import synth
from rootpwa_gb300.sharded import ShardedFdF, shard_range

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

CASES = [dict(use_normalized=True, prior=0), dict(use_normalized=False, prior=0), dict(use_normalized=True, prior=1)]


def _oracle(w, data, total=None, root=True, **kw):
    from oracle.oracle import OracleIntegral, OracleLikelihood
    mc = w["mc"].astype(np.complex128)
    norm = OracleIntegral()
    assert norm.integrate(w["names"], mc)
    acc = OracleIntegral()
    assert acc.integrate(w["names"], mc, in_bin=w["accepted"])
    L = OracleLikelihood(kw["use_normalized"], kw["prior"], 0.5)
    if total is not None:
        L.set_shard(total, root)
    assert L.init(w["names"], w["refl"], None, w["rank"], 0.0)
    assert L.addNormIntegral(norm) and L.addAccIntegral(acc)
    for k, n in enumerate(w["names"]):
        assert L.addAmplitude(n, data[k].astype(np.complex128))
    assert L.finishInit()
    return L


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = synth.make_workload("compass15", seed=3, n_data=3001, n_mc=4000)
        N = w["data"].shape[1]
        b, e = shard_range(N, rank, world)
        res = []
        for kw in CASES:
            L = _oracle(w, w["data"][:, b:e], total=N, root=(rank == 0), **kw)
            f, g = ShardedFdF(L).FdF(w["par"])
            res.append((f, g))
        if rank == 0:
            out.put(res)
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_shard_range_covers_events():
    for n in (0, 1, 7, 1000):
        for world in (1, 2, 3, 8):
            r = [shard_range(n, k, world) for k in range(world)]
            assert r[0][0] == 0 and r[-1][1] == n
            assert all(r[k][1] == r[k + 1][0] for k in range(world - 1))


def test_two_gloo_ranks_equal_single_process():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(k, 2, port, out)) for k in range(2)]
    for p in procs:
        p.start()
    res = out.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    w = synth.make_workload("compass15", seed=3, n_data=3001, n_mc=4000)
    for kw, (f, g) in zip(CASES, res):
        L = _oracle(w, w["data"], **kw)
        f0, g0 = L.FdF(w["par"])
        assert abs(f - f0) <= 1e-11 * abs(f0), (kw, f, f0)
        assert np.max(np.abs(g - g0)) <= 1e-10 * np.max(np.abs(g0)), kw
