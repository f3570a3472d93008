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


def test_production_shape_full_size_against_oracle():
    """The production configuration at its full size -- 7 negative + 80
    positive waves + flat, rank 2, 341 parameters, 1,000,000 data events --
    against the FP64 oracle (the bit-for-bit restatement of
    pwaLikelihood::FdF, partialWaveFit/pwaLikelihood.cc:170-315) on the same
    events with the same integral sums, at two parameter points: value to
    1e-6 relative and gradient to 1e-6 normwise (FP32 contraction, FP64
    cross-tile and exact cross-block sums; measured errors are ~1e-9 / ~1e-8)."""
    import os
    names, refl = synth.wave_names(7, 80)
    rng = np.random.Generator(np.random.PCG64(21))
    model = synth.AmplitudeModel(len(names), 8, rng)
    data = model.draw(rng, 1_000_000)
    mc = model.draw(rng, 20_000)
    w = dict(names=names, refl=refl, rank=2, data=data, mc=mc, accepted=rng.random(20_000) < 0.6)
    on, oa = helpers.oracle_integrals(w)
    G = helpers.build_gpu(w, helpers.copy_oracle_integral_to_gpu(on), helpers.copy_oracle_integral_to_gpu(oa))
    O = helpers.build_oracle(w, on, oa)
    assert G.nmbPars() == O.nmbPars() == 341
    threads = len(os.sched_getaffinity(0))
    for par in (rng.standard_normal(341), 0.3 * rng.standard_normal(341)):
        f0, g0 = O.FdF(par, threads=threads)
        f1, g1 = G.FdF(par)
        assert helpers.rel(f1, f0) < 1e-6
        assert helpers.normwise(g1, g0) < 1e-6
