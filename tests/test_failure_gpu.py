"""Failure handling on the host side of the GPU path: allocation failures
injected before the CUDA allocator (pwa_debug_fail_alloc_after) surface as
PWA_ERROR_OUT_OF_MEMORY at whatever setup step they hit, leave no device
memory behind once the handles are gone and do not disturb the next
likelihood; non-finite parameters give non-finite results (as the FP64
reference does) without a device error, and the handle keeps working."""
import gc

import numpy as np
import pytest

import rootpwa_gb300 as R
from rootpwa_gb300 import _native as N
from rootpwa_gb300 import synth
import helpers

pytestmark = pytest.mark.gpu


def _build(w, norm, acc):
    return helpers.build_gpu(w, helpers.copy_oracle_integral_to_gpu(norm), helpers.copy_oracle_integral_to_gpu(acc))


def test_injected_allocation_failures():
    torch = pytest.importorskip("torch")
    w = synth.make_workload("compass15", seed=2, n_data=5000, n_mc=3000)
    norm, acc = helpers.oracle_integrals(w)
    G = _build(w, norm, acc)
    f0, g0 = G.FdF(w["par"])
    del G
    gc.collect()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failures = 0
    try:
        for n in range(64):
            N.lib().pwa_debug_fail_alloc_after(n)
            try:
                G = _build(w, norm, acc)
                f, g = G.FdF(w["par"])
            except R.PwaError as exc:
                assert exc.status == 4 and "injected allocation failure" in str(exc)
                failures += 1
                continue
            finally:
                N.lib().pwa_debug_fail_alloc_after(-1)
            # every allocation of setup and evaluation fitted in n
            assert f == f0 and np.array_equal(g, g0)
            del G
            break
        else:
            pytest.fail("setup never completed")
    finally:
        N.lib().pwa_debug_fail_alloc_after(-1)
    assert failures >= 5
    gc.collect()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert abs(free1 - free0) < (8 << 20), (free0, free1)
    # a likelihood built afterwards is unaffected
    G = _build(w, norm, acc)
    f, g = G.FdF(w["par"])
    assert f == f0 and np.array_equal(g, g0)


def test_non_finite_parameters():
    w = synth.make_workload("compass15", seed=3, n_data=4000, n_mc=3000)
    norm, acc = helpers.oracle_integrals(w)
    G = _build(w, norm, acc)
    f0, g0 = G.FdF(w["par"])
    for bad in (np.nan, np.inf):
        p = w["par"].copy()
        p[3] = bad
        f, g = G.FdF(p)
        assert not np.isfinite(f)
        assert not np.all(np.isfinite(g))
    f, g = G.FdF(w["par"])
    assert f == f0 and np.array_equal(g, g0)


def test_bounded_device_wait_expires_and_context_stays_usable():
    """The device-side failure path without a fault: a warp waits with the
    kernels' bounded-wait helper on an mbarrier armed for a transfer that is
    never issued (pwa_debug_stalled_wait).  The wait gives up after its limit,
    the call returns PWA_ERROR_DEVICE_TIMEOUT, and afterwards the same
    context evaluates a likelihood that agrees with the oracle."""
    import time
    lib = N.lib()
    assert lib.pwa_debug_stalled_wait(0) == N.ERROR_INVALID_ARGUMENT
    for limit_us in (2_000, 50_000):
        t0 = time.perf_counter()
        assert lib.pwa_debug_stalled_wait(limit_us) == N.ERROR_DEVICE_TIMEOUT
        dt = time.perf_counter() - t0
        assert dt >= limit_us * 1e-6
        assert b"expired" in N.lib().pwa_last_error()
    w = synth.make_workload("compass15", seed=6, n_data=3001, n_mc=2000)
    norm, acc = helpers.oracle_integrals(w)
    G = _build(w, norm, acc)
    O = helpers.build_oracle(w, norm, acc)
    f, g = G.FdF(w["par"])
    f0, g0 = O.FdF(w["par"])
    assert helpers.rel(f, f0) < helpers.F_RTOL and helpers.normwise(g, g0) < helpers.G_NORMWISE
