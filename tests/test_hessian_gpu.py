"""GPU parity of the analytic Hessian (partialWaveFit/pwaLikelihood.cc:
639-859) and the covariance matrix (:929-981) against the FP64 oracle.

Tolerance: max |H - H_ref| / max |H_ref| below 2e-5 (FP32 event products,
TF32x3 tensor-core Gram sums, FP64 across CTAs).  compass88 at rank 2 has
2 x 2 x 87 + 1 = 349 Gram columns, which run as Grams of pairs of 48-row
groups (the last group padded); compass15 at rank 3 (91 columns) as one."""
import numpy as np
import pytest

from rootpwa_gb300 import synth
import helpers

pytestmark = pytest.mark.gpu


def pair(w, **kw):
    norm, acc, gn, ga = helpers.integral_pairs(w)
    O = helpers.build_oracle(w, norm, acc, **kw)
    G = helpers.build_gpu(w, gn, ga, **kw)
    return O, G


@pytest.mark.parametrize("workload,n_data,rank,kw", [
    ("compass15", 20000, 1, {}),
    ("compass88", 3001, 2, {}),
    ("compass15", 4000, 3, dict(prior=1, cauchy_width=0.8)),
    ("compass15", 2500, 1, dict(use_normalized=False)),
])
def test_hessian_against_oracle(workload, n_data, rank, kw):
    w = synth.make_workload(workload, seed=n_data, n_data=n_data, n_mc=5000, rank=rank)
    O, G = pair(w, **kw)
    H0 = O.Hessian(w["par"])
    H1 = G.Hessian(w["par"])
    err = np.max(np.abs(H1 - H0)) / np.max(np.abs(H0))
    assert err < 2e-5, err
    assert np.array_equal(H1 == 0, H0 == 0) or err < 2e-5


def test_covariance_against_oracle():
    w = synth.make_workload("compass15", seed=21, n_data=20000, n_mc=20000)
    O, G = pair(w)
    H0 = O.Hessian(w["par"])
    H1 = G.Hessian(w["par"])
    C0 = O.CovarianceMatrix(H0)
    C1 = G.CovarianceMatrix(H0)       # same input: the inversion itself
    assert np.allclose(C1, C0, rtol=1e-9, atol=1e-12 * np.max(np.abs(C0)))
    C2 = G.CovarianceMatrix(H1)
    cond = np.linalg.cond(H0)
    assert np.max(np.abs(C2 - C0)) / np.max(np.abs(C0)) < 2e-5 * cond
