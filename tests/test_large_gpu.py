"""Size-independent checks at sizes beyond 32-bit byte offsets: 20,000,000
events x 15 waves (2.4 GB of complex64 amplitudes) in one likelihood equal
the sum of two event shards of 10,000,000 events (linearity of the extended
likelihood in the events: the normalisation term is added by the root shard
only), for the value and the gradient, to the reordering of FP32 tile sums
and FP64 block sums (1e-10 relative), with unnormalised amplitudes (so nEvt
is the total event count on both sides).  The same store evaluated twice is
bitwise identical."""
import numpy as np
import pytest

import rootpwa_gb300 as R
from rootpwa_gb300 import synth
import helpers

pytestmark = pytest.mark.gpu


def test_twenty_million_events_equal_two_shards():
    torch = pytest.importorskip("torch")
    names, refl = synth.wave_names(0, 15)
    rng = np.random.Generator(np.random.PCG64(5))
    model = synth.AmplitudeModel(15, 4, rng)
    n = 20_000_000
    data = synth.draw_device(model, n, seed=77)
    mc = synth.draw_device(model, 200_000, seed=78)
    norm = R.ampIntegralMatrix()
    norm.integrate(names, mc, precision="fp32")
    raw, nev = norm.matrix(), norm.nmbEvents()
    par = rng.standard_normal(synth.n_pars(0, 15, 1))

    def integral():
        I = R.ampIntegralMatrix()
        I.setWaveNames(names)
        I.setMatrix(raw)
        I.setNmbEvents(nev)
        return I

    def build(lo, hi, shard):
        L = R.pwaLikelihood()
        L.useNormalizedAmps(False)
        if shard is not None:
            L.setShard(n, shard)
        L.init(names, refl, None, 1, 0.0)
        L.addNormIntegral(integral())
        L.addAccIntegral(integral())
        for k, name in enumerate(names):
            L.addAmplitude(name, data[k, lo:hi].contiguous())
        L.finishInit()
        return L

    F = build(0, n, None)
    f, g = F.FdF(par)
    f2, g2 = F.FdF(par)
    assert f == f2 and np.array_equal(g, g2)
    del F
    torch.cuda.empty_cache()
    A = build(0, n // 2, True)
    fa, ga = A.FdF(par)
    del A
    B = build(n // 2, n, False)
    fb, gb = B.FdF(par)
    assert abs((fa + fb) - f) <= 1e-10 * abs(f), (fa + fb, f)
    assert np.max(np.abs((ga + gb) - g)) <= 1e-10 * np.max(np.abs(g))
