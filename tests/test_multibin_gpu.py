"""GPU tests of the batched multibin x multistart FdF and the GPU L-BFGS.

The batch evaluates many (bin, start) problems in one sweep; every problem's
value and gradient must agree with the single-likelihood path (itself checked
against the FP64 oracle) to the engine's tolerances: 1e-6 relative in f and
1e-5 normwise in the gradient (FP32 contractions in both paths, summed in a
different order).  Fits must reach the minima an FP64 reference minimiser
(scipy L-BFGS-B on the oracle) finds from the same start points."""
import numpy as np
import pytest

import rootpwa_gb300 as R
from rootpwa_gb300 import synth
import helpers

pytestmark = pytest.mark.gpu


def make_bins(sizes, seed=10, n_mc=4000):
    out = []
    for k, n in enumerate(sizes):
        w = synth.make_workload("multibin50", seed=seed + k, n_data=n, n_mc=n_mc)
        norm, acc = helpers.gpu_integrals(w)
        out.append((w, helpers.build_gpu(w, norm, acc)))
    return out


@pytest.mark.parametrize("group", [32, 8])
def test_batched_fdf_matches_single_likelihood(group):
    bins = make_bins([700, 3001, 12000])
    starts = [5, 33, 8]
    M = R.pwaMultibin()
    M.setOptions(startGroup=group)
    for (w, L), s in zip(bins, starts):
        M.addBin(L, s)
    P, Q = M.nmbPars(), M.nmbProblems()
    assert Q == sum(starts) and P == 100
    x = np.random.default_rng(3).standard_normal((Q, P))
    f, g = M.FdF(x)
    q = 0
    for (w, L), s in zip(bins, starts):
        for _ in range(s):
            f1, g1 = L.FdF(x[q])
            assert helpers.rel(f[q], f1) < 1e-6, (q, f[q], f1)
            assert helpers.normwise(g[q], g1) < 1e-5, q
            q += 1
    # deterministic
    f2, g2 = M.FdF(x)
    assert np.array_equal(f, f2) and np.array_equal(g, g2)


def test_batched_fdf_against_oracle():
    w = synth.make_workload("multibin50", seed=21, n_data=2500, n_mc=3000)
    on, oa, gn, ga = helpers.integral_pairs(w)
    O = helpers.build_oracle(w, on, oa)
    L = helpers.build_gpu(w, gn, ga)
    M = R.pwaMultibin()
    M.addBin(L, 4)
    x = np.random.default_rng(5).standard_normal((4, M.nmbPars()))
    f, g = M.FdF(x)
    for q in range(4):
        f0, g0 = O.FdF(x[q])
        assert helpers.rel(f[q], f0) < helpers.F_RTOL
        assert helpers.normwise(g[q], g0) < 1e-5


@pytest.mark.parametrize("group", [32, 8])
def test_chunking_and_autotune_keep_results(group):
    """Tiles per work item only re-partition the FP32 tile partials that are
    folded into FP64: values agree to FP32 rounding of those partials."""
    bins = make_bins([900, 20000])
    M = R.pwaMultibin()
    M.setOptions(startGroup=group)
    for (w, L) in bins:
        M.addBin(L, 6)
    x = np.random.default_rng(7).standard_normal((M.nmbProblems(), M.nmbPars()))
    f0, g0 = M.FdF(x)
    M.setChunks([1, 3, 5])
    f1, g1 = M.FdF(x)
    assert np.max(np.abs(f1 - f0) / np.abs(f0)) < 1e-7
    assert max(helpers.normwise(g1[q], g0[q]) for q in range(len(f0))) < 1e-5
    chunks = M.autotune(x)
    assert len(chunks) == 3 and all(c >= 1 for c in chunks)
    f2, _ = M.FdF(x)
    assert np.max(np.abs(f2 - f0) / np.abs(f0)) < 1e-7
    assert M.sweepMs(x) > 0


def test_fit_reaches_reference_minima_graph_and_stream():
    scipy_opt = pytest.importorskip("scipy.optimize")
    w = synth.make_workload("multibin50", seed=31, n_data=3000, n_mc=4000)
    on, oa, gn, ga = helpers.integral_pairs(w)
    O = helpers.build_oracle(w, on, oa)
    L = helpers.build_gpu(w, gn, ga)
    S = 4
    M = R.pwaMultibin()
    M.setOptions(startGroup=8, gtolRel=1e-9, maxIter=3000)
    M.addBin(L, S)
    x0 = np.random.default_rng(11).standard_normal((S, M.nmbPars()))
    res_g = M.fit(x0, useGraph=True, sweepsPerGraph=20)
    res_s = M.fit(x0, useGraph=False, sweepsPerGraph=20)
    assert np.array_equal(res_g["x"], res_s["x"]) and np.array_equal(res_g["f"], res_s["f"])
    assert np.all(np.isin(res_g["status"], [2, 4, 6])), res_g["status"]
    best = np.min(res_g["f"])
    ref = []
    for q in range(S):
        r = scipy_opt.minimize(lambda p: O.FdF(p), x0[q], jac=True, method="L-BFGS-B",
                               options=dict(maxiter=5000, gtol=1e-8, ftol=1e-15))
        ref.append(r.fun)
    assert helpers.rel(best, min(ref)) < 1e-6, (best, min(ref))
    # every start that scipy took to the global minimum reaches it here too
    for q in range(S):
        if helpers.rel(ref[q], min(ref)) < 1e-7:
            assert helpers.rel(res_g["f"][q], min(ref)) < 1e-6, (q, res_g["f"][q], min(ref))
