"""GPU test of the allocation-free Gram entry point pwa_gram_device_noalloc,
called through the C ABI.  Its raw sums must agree with the existing
integrate() entry point (same SIMT FP32 kernel, different chunking) and with
an FP64 product for weighted sums, on two calls in a row (the second call
reuses the fixed device scratch of the first).  Collected last so that it
runs after the other GPU tests as well as alone."""
import ctypes as C

import numpy as np
import pytest

import rootpwa_gb300 as R
from rootpwa_gb300 import _native as N
from rootpwa_gb300 import synth

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

# FP32 products and per-chunk FP32 sums: relative to the largest element
TOL = 2e-5


def _noalloc(dA, K, ldK, W, dW, precision, out, stream):
    N.call("pwa_gram_device_noalloc", C.c_void_p(dA.data_ptr()), K, ldK, W,
           None if dW is None else C.c_void_p(dW.data_ptr()), precision, C.c_void_p(out.data_ptr()),
           C.c_void_p(stream.cuda_stream))


def _amps(seed, n_neg, n_pos, n_events):
    rng = np.random.Generator(np.random.PCG64(seed))
    names, _ = synth.wave_names(n_neg, n_pos)
    model = synth.AmplitudeModel(len(names), 4, rng)
    return names, model.draw(rng, n_events), rng


def test_noalloc_gram_matches_integrate_twice():
    names, mc, _ = _amps(5, 3, 30, 50_000)
    W, K = mc.shape
    I = R.ampIntegralMatrix()
    I.integrate(names, mc, precision="fp32")
    ref = I.matrix()
    dA = torch.from_numpy(mc).cuda()
    out = torch.empty((W, W), dtype=torch.complex128, device="cuda")
    s = torch.cuda.Stream()
    for _ in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        _noalloc(dA, K, K, W, None, 1, out, s)
        s.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert np.abs(got - ref).max() <= TOL * np.abs(ref).max()
        assert np.array_equal(got, got.conj().T)


def test_noalloc_gram_weighted_rows_with_stride():
    names, mc, rng = _amps(6, 0, 17, 30_000)
    W, K = mc.shape
    ld = K + 40  # rows with a stride larger than the event count
    padded = np.zeros((W, ld), dtype=np.complex64)
    padded[:, :K] = mc
    w = rng.uniform(0.2, 3.0, K)
    ref = (mc.astype(np.complex128) * w) @ mc.astype(np.complex128).conj().T
    dA = torch.from_numpy(padded).cuda()
    dW = torch.from_numpy(w).cuda()
    out = torch.empty((W, W), dtype=torch.complex128, device="cuda")
    s = torch.cuda.Stream()
    for precision, tol in ((1, TOL), (0, 1e-12)):
        for _ in range(2):
            out.fill_(float("nan"))
            torch.cuda.synchronize()
            _noalloc(dA, K, ld, W, dW, precision, out, s)
            s.synchronize()
            got = out.cpu().numpy()
            assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


def test_noalloc_gram_rejects_oversized_wave_set():
    dA = torch.zeros((2, 64), dtype=torch.complex64, device="cuda")
    out = torch.zeros((2, 2), dtype=torch.complex128, device="cuda")
    s = torch.cuda.Stream()
    with pytest.raises(N.PwaError) as e:
        _noalloc(dA, 64, 64, 257, None, 1, out, s)
    assert e.value.status == 1 and "256" in str(e.value)


def test_noalloc_gram_largest_wave_set_million_events():
    """256 waves (the limit) over 1,000,000 events: more chunk partials than
    the fixed array holds, so the call runs in segments with integrate()'s
    chunk length.  Unweighted FP32 and FP64 sums agree with integrate() in
    FP64, weighted FP32 sums with the weighted FP64 sums, each on two calls in
    a row, and the calls take no device memory."""
    names, _ = synth.wave_names(0, 256)
    model = synth.AmplitudeModel(256, 8, np.random.Generator(np.random.PCG64(9)))
    mc = synth.draw_device(model, 1_000_000, seed=19)
    W, K = mc.shape
    I = R.ampIntegralMatrix()
    I.integrate(names, mc, precision="fp64")
    ref = I.matrix()
    dW = torch.rand(K, dtype=torch.float64, device="cuda") + 0.5
    out = torch.empty((W, W), dtype=torch.complex128, device="cuda")
    s = torch.cuda.Stream()

    def run(weights, precision):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        _noalloc(mc, K, K, W, weights, precision, out, s)
        s.synchronize()
        return out.cpu().numpy()

    ref_w = run(dW, 0)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        for weights, precision, expect, tol in ((None, 1, ref, TOL), (None, 0, ref, 1e-12), (dW, 1, ref_w, TOL)):
            got = run(weights, precision)
            assert np.abs(got - expect).max() <= tol * np.abs(expect).max()
    assert torch.cuda.mem_get_info()[0] == free0
