"""On-the-fly binning of the oracle (pwaLikelihood.cc:1391-1440): the event
selection against a numpy restatement of the reference's rejection test
(x < lower or x >= upper drops an event, so NaN keeps it), and the
likelihood of a whole file with the selection against the likelihood of the
pre-selected events, which must agree bit for bit."""
import numpy as np

from oracle.oracle import OracleLikelihood
from rootpwa_gb300 import synth
import helpers


def reference_mask(bounds, cols):
    keep = np.ones(len(next(iter(cols.values()))), dtype=bool)
    for k, (lo, hi) in bounds.items():
        x = cols[k]
        keep &= ~((x < lo) | (x >= hi))
    return keep


def file_and_bins(n, seed):
    rng = np.random.default_rng(seed)
    cols = {"mass": rng.uniform(1.0, 2.0, n), "tPrime": rng.exponential(0.3, n)}
    # values on the bin edges and a NaN
    cols["mass"][::97] = 1.4
    cols["mass"][5::97] = 1.6
    cols["tPrime"][11] = np.nan
    bounds = {"mass": (1.4, 1.6), "tPrime": (0.1, 1.0)}
    return cols, bounds


def test_oracle_otf_selection_matches_rejection_test():
    cols, bounds = file_and_bins(5000, 3)
    cols["mass"][11] = 1.5  # the NaN event is otherwise in the bin
    keep = reference_mask(bounds, cols)
    assert keep[11]
    L = OracleLikelihood()
    assert L.setOnTheFlyBinning(bounds, cols)
    assert L.otfSelected() == int(keep.sum())
    assert 0 < keep.sum() < 5000


def test_oracle_otf_likelihood_equals_preselected():
    w = synth.make_workload("compass15", seed=5, n_data=3000, n_mc=4000, rank=2)
    n = w["data"].shape[1]
    cols, bounds = file_and_bins(n, 7)
    keep = reference_mask(bounds, cols)
    norm, acc = helpers.oracle_integrals(w)
    O = OracleLikelihood()
    assert O.init(w["names"], w["refl"], None, w["rank"], 0.0)
    assert O.addNormIntegral(norm)
    assert O.addAccIntegral(acc)
    assert O.setOnTheFlyBinning(bounds, cols)
    for k, name in enumerate(w["names"]):
        assert O.addAmplitude(name, w["data"][k].astype(np.complex128))
    assert O.finishInit()
    ws = dict(w, data=w["data"][:, keep])
    P = helpers.build_oracle(ws)
    f0, g0 = O.FdF(w["par"])
    f1, g1 = P.FdF(w["par"])
    assert f0 == f1
    assert np.array_equal(g0, g1)
    # a whole-file amplitude array of another length is refused
    Q = OracleLikelihood()
    assert Q.init(w["names"], w["refl"], None, w["rank"], 0.0)
    assert Q.addNormIntegral(norm) and Q.addAccIntegral(acc)
    assert Q.setOnTheFlyBinning(bounds, cols)
    assert not Q.addAmplitude(w["names"][0], w["data"][0][:-1].astype(np.complex128))
