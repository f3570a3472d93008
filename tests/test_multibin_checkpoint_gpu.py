"""Checkpoint / resume of the batched multibin fit: a fit stopped after some
sweeps, saved to a file, loaded into a fresh batch over the same bins and
resumed ends bit for bit where the uninterrupted fit ends (the whole L-BFGS
state is on the device and the kernels are deterministic); the periodic
checkpoint written during a fit resumes the same way; a checkpoint does not
load into a batch with other bins or starts."""
import numpy as np
import pytest

import rootpwa_gb300 as R
from test_multibin_gpu import make_bins

pytestmark = pytest.mark.gpu


def batch(bins, starts):
    M = R.pwaMultibin()
    M.setOptions(gtolRel=1e-8)
    for (w, L), s in zip(bins, starts):
        M.addBin(L, s)
    return M


def same(a, b):
    for k in ("x", "f", "gnorm", "status", "iterations"):
        assert np.array_equal(a[k], b[k]), k


def test_save_load_resume_is_bitwise(tmp_path):
    bins = make_bins([1500, 6000])
    starts = [4, 3]
    M = batch(bins, starts)
    x0 = np.random.default_rng(11).standard_normal((M.nmbProblems(), M.nmbPars()))
    full = M.fit(x0, sweepsPerGraph=5)
    assert full["sweeps"] > 20
    # the same fit, stopped after 20 sweeps and checkpointed
    part = M.fit(x0, sweepsPerGraph=5, maxSweeps=20)
    assert part["sweeps"] == 20 and M.sweepsDone() == 20
    path = tmp_path / "fit.state"
    M.saveState(path)
    # a fresh batch over the same bins continues from the file
    M2 = batch(bins, starts)
    M2.loadState(path)
    assert M2.sweepsDone() == 20
    rest = M2.resume(sweepsPerGraph=5)
    same(rest, full)
    assert 20 + rest["sweeps"] == full["sweeps"]
    # resuming the original handle gives the same again
    same(M.resume(sweepsPerGraph=5), full)


def test_periodic_checkpoint_and_mismatch(tmp_path):
    bins = make_bins([2000, 2500])
    starts = [3, 3]
    M = batch(bins, starts)
    x0 = np.random.default_rng(12).standard_normal((M.nmbProblems(), M.nmbPars()))
    full = M.fit(x0, sweepsPerGraph=4)
    assert full["sweeps"] > 28
    path = tmp_path / "periodic.state"
    M.setCheckpoint(path, 8)
    M.fit(x0, sweepsPerGraph=4, maxSweeps=28)  # checkpoints after 8, 16 and 24 sweeps
    M.setCheckpoint(None, 0)
    M2 = batch(bins, starts)
    M2.loadState(path)
    assert M2.sweepsDone() == 24
    same(M2.resume(sweepsPerGraph=4), full)
    # other starts per bin: refused
    M3 = batch(bins, [3, 2])
    with pytest.raises(R.PwaError):
        M3.loadState(path)
    # nothing to resume before a fit or a load
    with pytest.raises(R.PwaError):
        batch(bins, starts).resume()
