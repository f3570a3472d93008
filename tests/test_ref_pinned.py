"""The restated FP64 oracle against the reference's own code.

oracle/ref.py drives ROOTPWA's partialWaveFit/pwaLikelihood.cc and
decayAmplitude/ampIntegralMatrix.cc, compiled unmodified from the reference
sources (`make -C oracle ref`).  The oracle restates the same loops in the
same order with the same compensated sums, so the two agree bit for bit on
everything that does not go through the reference's ROOT linear algebra
(the covariance inverse, agreed to rounding).  These tests run where the
reference sources are present; the golden fixtures written by
tests/golden/make_ref_golden.py carry the reference's values to places
without them.
"""
import os

import numpy as np
import pytest

from oracle import ref
from oracle.oracle import OracleIntegral, OracleLikelihood
from rootpwa_gb300 import synth
import helpers

pytestmark = pytest.mark.skipif(not ref.available(), reason="reference sources not present")

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # the single-bin config: 15 waves of positive reflectivity, rank 1
    "compass15": dict(name="compass15", seed=0, n_data=3001, n_mc=5003),
    # the production shape: 7 negative + 80 positive waves, rank 2
    "compass88": dict(name="compass88", seed=1, n_data=1501, n_mc=2003),
    "compass88_rank3": dict(name="compass88", seed=2, n_data=701, n_mc=1103, rank=3),
}


def _both(w, **kw):
    """the same set-up through the oracle and through the reference"""
    on, oa = helpers.oracle_integrals(w, OracleIntegral)
    rn, ra = helpers.oracle_integrals(w, ref.RefIntegral)
    O = helpers.build_oracle(w, on, oa, Likelihood=OracleLikelihood, **kw)
    R = helpers.build_oracle(w, rn, ra, Likelihood=ref.RefLikelihood, **kw)
    return O, R, (on, oa), (rn, ra)


@pytest.mark.parametrize("case", list(CASES))
def test_integrals_bitwise(case):
    """ampIntegralMatrix::integrate (ampIntegralMatrix.cc:299-488): raw sums
    and event counts of the normalisation and acceptance integrals."""
    w = synth.make_workload(**CASES[case])
    on, oa = helpers.oracle_integrals(w, OracleIntegral)
    rn, ra = helpers.oracle_integrals(w, ref.RefIntegral)
    for o, r in ((on, rn), (oa, ra)):
        assert o.nmb_events() == r.nmb_events()
        np.testing.assert_array_equal(o.raw(), r.raw())
        assert o.wave_names() == r.wave_names()


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("opts", [dict(), dict(use_normalized=False), dict(prior=1, cauchy_width=0.5)],
                         ids=["normalised", "unnormalised", "half-cauchy"])
def test_fdf_doeval_gradient_bitwise(case, opts):
    """FdF, DoEval and Gradient (pwaLikelihood.cc:170-636) and the parameter
    layout (buildParDataStruct, :1487-1556): identical names, fixed flags and
    bitwise-identical values at two points."""
    w = synth.make_workload(**CASES[case])
    O, R, _, _ = _both(w, **opts)
    assert O.nmbPars() == R.nmbPars() and O.nmbParsFixed() == R.nmbParsFixed()
    assert [O.parName(i) for i in range(O.nmbPars())] == [R.parName(i) for i in range(R.nmbPars())]
    assert [O.parFixed(i) for i in range(O.nmbPars())] == [R.parFixed(i) for i in range(R.nmbPars())]
    rng = np.random.default_rng(5)
    for par in (w["par"], rng.standard_normal(len(w["par"]))):
        fo, go = O.FdF(par)
        fr, gr = R.FdF(par)
        assert fo == fr
        np.testing.assert_array_equal(go, gr)
        assert O.DoEval(par) == R.DoEval(par) == fr
        np.testing.assert_array_equal(O.Gradient(par), R.Gradient(par))


def test_thresholds_override_and_zero_wave():
    """Threshold-fixed waves (pwaLikelihood.cc:1527-1530), a wave whose
    amplitudes and acceptance integral are all zero (:1248,1268-1282), and
    accEventsOverride (:1087-1090): same fixed flags and bitwise values."""
    w = synth.make_workload("compass88", seed=3, n_data=901, n_mc=1201)
    z = 11
    w["data"][z] = 0
    w["mc"][z] = 0
    th = np.zeros(len(w["names"]))
    th[[3, 20, 40]] = [1.5, 2.0, 0.9]
    O, R, _, _ = _both(w, thresholds=th, mass_bin_center=1.7, acc_override=5000)
    fixed_o = [O.parFixed(i) for i in range(O.nmbPars())]
    assert fixed_o == [R.parFixed(i) for i in range(R.nmbPars())]
    assert sum(fixed_o) > 0
    fo, go = O.FdF(w["par"])
    fr, gr = R.FdF(w["par"])
    assert fo == fr
    np.testing.assert_array_equal(go, gr)


@pytest.mark.parametrize("case", ["compass15", "compass88"])
def test_hessian_covariance_signs(case):
    """Hessian (pwaLikelihood.cc:639-859) bit for bit; CovarianceMatrix
    (:916-981) to rounding (the reference inverts with ROOT, absent here: the
    shim inverts by Gauss-Jordan); CorrectParamSigns (:984-1010) bit for bit."""
    w = synth.make_workload(**CASES[case])
    O, R, _, _ = _both(w)
    H = O.Hessian(w["par"])
    np.testing.assert_array_equal(H, R.Hessian(w["par"]))
    Co, Cr = O.CovarianceMatrix(H), R.CovarianceMatrix(H)
    assert np.max(np.abs(Co - Cr)) <= 1e-9 * np.max(np.abs(Cr))
    flip = w["par"].copy()
    flip[0] = -abs(flip[0])
    np.testing.assert_array_equal(O.CorrectParamSigns(flip), R.CorrectParamSigns(flip))


def test_integral_matrices_and_derivative_cache():
    """getIntegralMatrices with and without the flat wave (pwaLikelihood.cc:
    1577-1618), and DoDerivative from the derivative cache (:438-471)."""
    w = synth.make_workload(**CASES["compass88"])
    O, R, _, _ = _both(w)
    for flat in (False, True):
        for a, b in zip(O.integralMatrices(flat), R.integralMatrices(flat)):
            np.testing.assert_array_equal(a, b)
    _, g = O.FdF(w["par"])
    assert [R.DoDerivative(w["par"], i) for i in (0, 5, len(g) - 1)] == [g[0], g[5], g[-1]]


def test_weights_bins_max_events_subamps():
    """integrate with importance-sampling weights (the reference reads them
    from a file and uses 1/w), an on-the-fly bin, maxNmbEvents and two
    incoherent sub-amplitudes."""
    rng = np.random.default_rng(7)
    W, N, S = 9, 1201, 2
    names = ["w%d" % i for i in range(W)]
    amps = (rng.standard_normal((W, N, S)) + 1j * rng.standard_normal((W, N, S))) * rng.uniform(0.2, 3, (W, 1, 1))
    inbin = rng.random(N) < 0.7
    wts = rng.uniform(0.5, 2.0, N)
    for kw in (dict(), dict(weights=wts), dict(in_bin=inbin), dict(weights=wts, in_bin=inbin),
               dict(max_nmb_events=700), dict(weights=wts, max_nmb_events=333)):
        o, r = OracleIntegral(), ref.RefIntegral()
        assert o.integrate(names, amps, **kw) and r.integrate(names, amps, **kw)
        assert o.nmb_events() == r.nmb_events()
        np.testing.assert_array_equal(o.raw(), r.raw())


def test_on_the_fly_binning_likelihood():
    """setOnTheFlyBinning (pwaLikelihood.cc:1391-1440) followed by addAmplitude
    of whole-file rows: the same events selected, bitwise the same FdF."""
    w = synth.make_workload("compass15", seed=4, n_data=2500, n_mc=3000)
    rng = np.random.default_rng(8)
    mass = rng.uniform(0.5, 2.5, 2500)
    tprime = rng.uniform(0.1, 1.0, 2500)
    bounds = {"mass": (1.0, 1.8), "tPrime": (0.2, 0.9)}
    outs = []
    for Int, Lik in ((OracleIntegral, OracleLikelihood), (ref.RefIntegral, ref.RefLikelihood)):
        n, a = helpers.oracle_integrals(w, Int)
        L = Lik()
        assert L.init(w["names"], w["refl"], None, w["rank"], 0.0)
        assert L.addNormIntegral(n) and L.addAccIntegral(a)
        assert L.setOnTheFlyBinning(bounds, {"mass": mass, "tPrime": tprime})
        for k, nm in enumerate(w["names"]):
            assert L.addAmplitude(nm, w["data"][k].astype(np.complex128))
        assert L.finishInit()
        outs.append((L.otfSelected(),) + L.FdF(w["par"]))
    assert outs[0][0] == outs[1][0] == int(np.sum((mass >= 1.0) & (mass < 1.8) & (tprime >= 0.2) & (tprime < 0.9)))
    assert outs[0][1] == outs[1][1]
    np.testing.assert_array_equal(outs[0][2], outs[1][2])


def test_ascii_integral_io_against_reference(tmp_path):
    """readAscii / writeAscii (ampIntegralMatrix.cc:503-570) on the
    reference's own fixture: both read the same matrix, and what the oracle
    writes the reference reads back to the same values."""
    fixture = os.path.join(HERE, "golden", "testIntegral.int")
    o, r = OracleIntegral(), ref.RefIntegral()
    assert o.read_ascii(fixture) and r.read_ascii(fixture)
    assert o.nmb_events() == r.nmb_events() == 20000
    np.testing.assert_array_equal(o.raw(), r.raw())
    p = str(tmp_path / "o.int")
    assert o.write_ascii(p)
    r2 = ref.RefIntegral()
    assert r2.read_ascii(p)
    np.testing.assert_array_equal(r2.raw(), o.raw())


@pytest.mark.parametrize("fixture", ["ref_compass15_seed0.npz", "ref_compass88_small_seed1.npz"])
def test_reference_golden_fixtures_reproduce(fixture):
    """The committed reference-generated fixtures (make_ref_golden.py) still
    match the reference and the oracle on the regenerated inputs."""
    import golden.make_ref_golden as G
    spec = G.GOLDEN_WORKLOADS[fixture[len("ref_"):-len(".npz")]]
    w = synth.make_workload(**spec)
    d = np.load(os.path.join(HERE, "golden", fixture))
    np.testing.assert_array_equal(d["checksum"], G.checksum(w))
    O, R, (on, _), _ = _both(w)
    f, g = R.FdF(w["par"])
    assert f == float(d["f"]) and O.FdF(w["par"])[0] == f
    np.testing.assert_array_equal(g, d["grad"])
    np.testing.assert_array_equal(on.raw(), d["norm_raw"])
