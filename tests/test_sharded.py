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


class _Failing:
    """A shard whose evaluation raises (a rank that fails on the host)."""

    def FdF(self, par):
        raise RuntimeError("injected shard failure")


def _dropout_worker(rank, world, port, use_store, out):
    import datetime
    from rootpwa_gb300.sharded import ShardFailure
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    store = dist.TCPStore("127.0.0.1", port + 1, world, rank == 0, timeout=datetime.timedelta(seconds=30))
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=10))
    w = synth.make_workload("compass15", seed=4, n_data=500, n_mc=2000)
    N = w["data"].shape[1]
    b, e = shard_range(N, rank, world)
    try:
        if rank == 1:
            local = _Failing()
        else:
            local = _oracle(w, w["data"][:, b:e], total=N, root=True, use_normalized=True, prior=0)
        F = ShardedFdF(local, store=store if use_store else None)
        if rank == 0 and use_store:
            # rank 0 evaluates after rank 1 has failed
            import time
            t0 = time.time()
            while not store.check([ShardedFdF.FAILED_KEY]) and time.time() - t0 < 20:
                time.sleep(0.05)
        try:
            F.FdF(w["par"])
            out.put((rank, "finished"))
        except ShardFailure as exc:
            out.put((rank, "peer failure: %s" % exc))
        except RuntimeError as exc:
            out.put((rank, "error: %s" % type(exc).__name__))
    finally:
        if rank == 0 or use_store:
            try:
                dist.destroy_process_group()
            except Exception:
                pass


@pytest.mark.parametrize("use_store", [True, False])
def test_rank_failure_is_detected(use_store):
    """Rank 1's evaluation raises.  With the store, rank 0 learns of it on
    the host and stops with ShardFailure before the all-reduce; without it,
    rank 0's all-reduce ends with an error (peer gone or group timeout)
    instead of waiting for ever."""
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_dropout_worker, args=(k, 2, port, use_store, out)) for k in range(2)]
    for p in procs:
        p.start()
    got = dict(out.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    assert got[1].startswith("error")  # the injected failure
    if use_store:
        assert got[0] == "peer failure: shard rank 1 failed"
    else:
        assert got[0].startswith("error")
