"""Batched multistart fits for the reference's general parameter layout:
rank 2, both reflectivities and threshold-fixed waves
(partialWaveFit/pwaLikelihood.cc:1487-1556), which the start-packed batch
kernels (rank 1, one reflectivity) do not cover.  Each (bin, start) problem
is evaluated by its bin's own FdF kernel inside the captured sweep, so the
batched value and gradient equal the likelihood's bit for bit, except that
the gradient components of fixed parameters are 0 (the minimiser's view).
Fixed parameters start and stay at 0, as in the reference's drivers
(highLevelInterface/pwaFit.cc:249-266, pwaNloptFit.cc:383-401)."""
import os

import numpy as np
import pytest

import rootpwa_gb300 as R
from rootpwa_gb300 import synth
import helpers

pytestmark = pytest.mark.gpu


def workload(n_neg, n_pos, rank, n_data, seed, n_mc=4000):
    names, refl = synth.wave_names(n_neg, n_pos)
    rng = np.random.default_rng(seed)
    model = synth.AmplitudeModel(n_neg + n_pos, 8, rng)
    return dict(names=names, refl=refl, rank=rank, data=model.draw(rng, n_data), mc=model.draw(rng, n_mc),
                accepted=rng.random(n_mc) < 0.6, par=rng.standard_normal(synth.n_pars(n_neg, n_pos, rank)))


def thresholds(n, waves, value):
    th = np.zeros(n)
    th[list(waves)] = value
    return th


def test_general_layout_batched_fdf_equals_each_bins_likelihood():
    # two bins of the production shape's structure (7 negative + 20 positive
    # waves, rank 2) with different event counts; the second bin has
    # threshold-fixed waves
    wa = workload(7, 20, 2, 3001, seed=41)
    wb = workload(7, 20, 2, 12011, seed=42)
    th = thresholds(27, [2, 9, 15], 3.0)     # at or above the bin centre 2.5: fixed
    La = helpers.build_gpu(wa, *helpers.gpu_integrals(wa))
    Lb = helpers.build_gpu(wb, *helpers.gpu_integrals(wb), thresholds=th, mass_bin_center=2.5)
    assert La.nmbParsFixed() == 0 and Lb.nmbParsFixed() > 0
    M = R.pwaMultibin()
    # different fixed flags, same layout: one batch
    M.addBin(La, 3)
    M.addBin(Lb, 2)
    P, Q = M.nmbPars(), M.nmbProblems()
    assert Q == 5 and P == La.nmbPars()
    x = np.random.default_rng(3).standard_normal((Q, P))
    f, g = M.FdF(x)
    fixed_b = np.array([Lb.parameter(k)["fixed"] for k in range(P)])
    for q in range(Q):
        L, fixed = (La, np.zeros(P, bool)) if q < 3 else (Lb, fixed_b)
        f1, g1 = L.FdF(x[q])
        assert f[q] == f1
        assert np.array_equal(g[q][~fixed], g1[~fixed])
        assert np.all(g[q][fixed] == 0.0)
    f2, g2 = M.FdF(x)
    assert np.array_equal(f, f2) and np.array_equal(g, g2)


def test_production_shape_multistart_fit_with_fixed_waves():
    """7 negative + 80 positive waves + flat, rank 2 (341 parameters), with
    three threshold-fixed waves: the batched GPU L-BFGS from four random
    starts reaches the minimum that scipy's L-BFGS-B finds on the FP64 oracle
    over the free parameters (fixed ones held at 0); the fixed parameters of
    every fitted point are exactly 0."""
    scipy_opt = pytest.importorskip("scipy.optimize")
    w = workload(7, 80, 2, 8000, seed=43, n_mc=6000)
    th = thresholds(87, [1, 30, 60], 3.5)    # at or above the bin centre 3.2: fixed
    kw = dict(thresholds=th, mass_bin_center=3.2)
    on, oa, gn, ga = helpers.integral_pairs(w)
    O = helpers.build_oracle(w, on, oa, **kw)
    L = helpers.build_gpu(w, gn, ga, **kw)
    P = L.nmbPars()
    assert P == 341
    fixed = np.array([L.parameter(k)["fixed"] for k in range(P)])
    assert fixed.sum() > 0 and np.array_equal(fixed, [O.parFixed(k) for k in range(P)])
    S = 4
    M = R.pwaMultibin()
    M.setOptions(gtolRel=1e-9, maxIter=20000)
    M.addBin(L, S)
    x0 = 0.3 * np.random.default_rng(13).standard_normal((S, P))
    res = M.fit(x0, useGraph=True, sweepsPerGraph=50, maxSweeps=200000)
    assert np.all(res["x"][:, fixed] == 0.0)
    assert np.all(np.isin(res["status"], [2, 4, 6])), res["status"]
    free = ~fixed
    threads = len(os.sched_getaffinity(0))

    def fg(p):
        full = np.zeros(P)
        full[free] = p
        f, g = O.FdF(full, threads=threads)
        return f, g[free]

    ref = []
    for q in range(S):
        r = scipy_opt.minimize(fg, x0[q][free], jac=True, method="L-BFGS-B",
                               options=dict(maxiter=20000, maxcor=20, gtol=1e-8, ftol=1e-15))
        ref.append(r.fun)
    best = np.min(res["f"])
    assert helpers.rel(best, min(ref)) < 1e-6, (best, min(ref), ref, res["f"])
    # the fitted point of the best start, evaluated by the FP64 oracle
    qb = int(np.argmin(res["f"]))
    f_o, g_o = O.FdF(res["x"][qb], threads=threads)
    assert helpers.rel(f_o, res["f"][qb]) < 1e-6
