"""Event-sharded FdF across the processes of a torch.distributed group.

Every per-event term of the extended likelihood is independent, so each rank
holds a contiguous share of the data events in its own pwaLikelihood
(setShard(totalEvents, root=rank == 0): only the root shard adds the
normalisation and prior terms) and one all-reduce of P + 1 doubles per FdF
combines the shares.  This is the multi-GPU design of the hot path: one
process per GPU, no other exchange.  The reference evaluates all events in
one process (pwaLikelihood.cc:170-315).
"""
import numpy as np


def shard_range(n_events, rank, world):
    """[begin, end) of the rank's contiguous share of n_events."""
    per, extra = divmod(int(n_events), int(world))
    b = rank * per + min(rank, extra)
    return b, b + per + (1 if rank < extra else 0)


class ShardFailure(RuntimeError):
    """Another rank of the shard group reported a failure."""


class ShardedFdF:
    """FdF of the whole data set from the rank-local shard `local` (any
    object with FdF(par) -> (f, grad)); collective over `group`.

    Failure detection on the host: with a torch.distributed `store`, a rank
    whose local evaluation raises records itself under FAILED_KEY before it
    re-raises, and every rank checks that key before it enters the
    all-reduce, so the others stop with ShardFailure instead of waiting in a
    collective the failed rank never joins.  Without a store, the process
    group's own timeout ends that collective with an error."""

    FAILED_KEY = "pwa_shard_failed"

    def __init__(self, local, group=None, device="cpu", store=None):
        self.local = local
        self.group = group
        self.device = device
        self.store = store

    def _check_peers(self):
        if self.store is not None and self.store.check([self.FAILED_KEY]):
            raise ShardFailure("shard rank %s failed" % self.store.get(self.FAILED_KEY).decode())

    def FdF(self, par):
        import torch
        import torch.distributed as dist
        self._check_peers()
        try:
            f, g = self.local.FdF(par)
        except Exception:
            if self.store is not None:
                self.store.set(self.FAILED_KEY, str(dist.get_rank(self.group)))
            raise
        self._check_peers()
        buf = torch.from_numpy(np.concatenate([[f], np.asarray(g, dtype=np.float64)])).to(self.device)
        dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=self.group)
        out = buf.cpu().numpy()
        return float(out[0]), out[1:].copy()
