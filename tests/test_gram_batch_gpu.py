"""GPU test of pwa_gram_device_batch: the Gram sums and row sums of many bins
in one call (the moment features of the learned warm start), against an FP64
numpy product of the same complex64 amplitudes.  At the tensor-core
precisions bins of 128 events and more take the tensor-core kernel (odd
counts through the aligned copy), shorter ones the FP32 SIMT kernel; both
must match to their precision's tolerance."""
import ctypes as C

import numpy as np
import pytest

from rootpwa_gb300 import _native as N

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [("fp32", 2e-6), ("tf32x3", 2e-6), ("bf16x3", 1e-5), ("tf32", 2e-3)])
def test_gram_batch_matches_numpy(precision, tol):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    W = 23
    sizes = [1, 64, 127, 999, 4096, 20001, 30000]
    host = []
    for n in sizes:
        a = (rng.standard_normal((W, n)) + 1j * rng.standard_normal((W, n))).astype(np.complex64)
        a *= np.exp(rng.uniform(-1, 1, W)).astype(np.float32)[:, None]
        host.append(a)
    dev = [torch.from_numpy(a).cuda().contiguous() for a in host]
    nb = len(dev)
    gram = torch.full((nb, W, W), np.nan, dtype=torch.complex128, device="cuda")
    sums = torch.full((nb, W), np.nan, dtype=torch.complex128, device="cuda")
    ptrs = (C.c_void_p * nb)(*[d.data_ptr() for d in dev])
    counts = (C.c_uint64 * nb)(*sizes)
    N.call("pwa_gram_device_batch", ptrs, counts, nb, W, N.PRECISION[precision], C.c_void_p(gram.data_ptr()),
           C.c_void_p(sums.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    G, S = gram.cpu().numpy(), sums.cpu().numpy()
    for b, a in enumerate(host):
        a64 = a.astype(np.complex128)
        ref = a64 @ a64.conj().T
        assert np.max(np.abs(G[b] - ref)) <= tol * np.max(np.abs(ref)), (b, sizes[b])
        assert np.array_equal(G[b], G[b].conj().T)
        # row sums: compensated FP32 per thread, FP64 across threads
        assert np.max(np.abs(S[b] - a64.sum(axis=1))) <= 1e-6 * np.max(np.abs(a64).sum(axis=1))


def test_gram_batch_rejects_bad_arguments():
    torch = pytest.importorskip("torch")
    d = torch.zeros((3, 8), dtype=torch.complex64, device="cuda")
    g = torch.zeros((1, 3, 3), dtype=torch.complex128, device="cuda")
    ptrs = (C.c_void_p * 1)(d.data_ptr())
    with pytest.raises(N.PwaError) as e:
        N.call("pwa_gram_device_batch", ptrs, (C.c_uint64 * 1)(0), 1, 3, N.PRECISION["fp32"],
               C.c_void_p(g.data_ptr()), None, None)
    assert e.value.status == N.ERROR_INVALID_ARGUMENT
    with pytest.raises(N.PwaError) as e:
        N.call("pwa_gram_device_batch", ptrs, (C.c_uint64 * 1)(8), 1, 3, N.PRECISION["fp64"],
               C.c_void_p(g.data_ptr()), None, None)
    assert e.value.status == 7
