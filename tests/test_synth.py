"""CPU tests of the synthetic workload generators: the resampled multibin data
are the same for the same seed (the multibin measurement repeats sweep for
sweep only if every process draws the same events), and the resampling
follows the model intensity."""
import numpy as np
import pytest

from rootpwa_gb300 import synth


def test_bin_draw_is_reproducible_and_importance_weighted():
    torch = pytest.importorskip("torch")
    W = 12
    model = synth.AmplitudeModel(W, 0, np.random.Generator(np.random.PCG64(5)))
    vt, fl = synth.true_production_amplitudes(W, np.random.default_rng(1))
    a = synth.draw_bin_device(model, vt, fl, 4000, seed=7, device="cpu")
    b = synth.draw_bin_device(model, vt, fl, 4000, seed=7, device="cpu")
    c = synth.draw_bin_device(model, vt, fl, 4000, seed=8, device="cpu")
    assert a.shape == (W, 4000) and a.dtype == torch.complex64 and a.is_contiguous()
    assert torch.equal(a, b)
    assert not torch.equal(a, c)
    # every drawn event comes from the seed's phase-space pool
    pool = synth.draw_device(model, 4 * 4000, seed=7, device="cpu")
    pool_cols = {np.ascontiguousarray(col).tobytes() for col in np.ascontiguousarray(pool.numpy().T)}
    drawn = np.ascontiguousarray(a.numpy().T)
    assert all(np.ascontiguousarray(col).tobytes() in pool_cols for col in drawn[:200])

    # resampled in proportion to the intensity: E_resampled[I] = E[I^2] / E[I]
    def intensity(x):
        s = torch.from_numpy(vt.astype(np.complex64)) @ x
        return (s.abs() ** 2 + fl * fl).double().numpy()

    ip = intensity(pool)
    expect = np.mean(ip ** 2) / np.mean(ip)
    got = np.mean(intensity(a))
    assert abs(got - expect) < 0.1 * expect, (got, expect)
