"""CPU tests of the C ABI: the library loads and exports every declared
symbol, the host-side logic (integral bookkeeping and ASCII I/O, wave list,
parameter layout, sign convention) matches the oracle, and device work fails
loudly when no GPU is present."""
import ctypes as C
import os

import numpy as np
import pytest

import rootpwa_gb300 as R
from rootpwa_gb300 import _native as N
from rootpwa_gb300 import synth
from oracle.oracle import OracleIntegral, OracleLikelihood
from test_oracle import split_ascii

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_library_exports_every_declared_symbol():
    lib = N.lib()
    declared = N.header_symbols()
    assert len(declared) >= 50
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    # and every binding signature refers to a declared function
    assert set(N.SIGNATURES) <= set(declared)
    assert lib.pwa_abi_version() == 1


def test_read_write_ascii_fixture(tmp_path):
    src = os.path.join(GOLDEN, "testIntegral.int")
    I = R.ampIntegralMatrix()
    I.readAscii(src)
    assert I.nmbWaves() == 41 and I.nmbEvents() == 20000
    out = tmp_path / "rt.int"
    I.writeAscii(out)
    assert split_ascii(out.read_text()) == split_ascii(open(src).read())
    O = OracleIntegral()
    assert O.read_ascii(src)
    assert np.array_equal(I.matrix(), O.raw())
    assert I.waveNames() == O.wave_names()
    name = I.waveName(7)
    assert I.waveIndex(name) == 7
    assert I.element(name, I.waveName(3)) == O.element(7, 3)


def test_read_ascii_rejects_truncated(tmp_path):
    src = open(os.path.join(GOLDEN, "testIntegral.int")).read()
    bad = tmp_path / "bad.int"
    bad.write_text(src[:2000])
    I = R.ampIntegralMatrix()
    with pytest.raises(R.PwaError) as e:
        I.readAscii(bad)
    assert e.value.status == 6
    with pytest.raises(R.PwaError):
        I.readAscii(tmp_path / "does_not_exist.int")


def test_integral_arithmetic_and_add_event():
    rng = np.random.default_rng(11)
    A = rng.standard_normal((5, 30)) + 1j * rng.standard_normal((5, 30))
    names = ["a", "b", "c", "d", "e"]
    I = R.ampIntegralMatrix()
    I.setWaveNames(names)
    O = OracleIntegral()
    O.set_wave_names(names)
    for e in range(30):
        I.addEvent(A[:, e])
        O.add_event(A[:, e])
    assert I.nmbEvents() == 30
    assert np.array_equal(I.matrix(), O.raw())
    J = R.ampIntegralMatrix(I)
    J += I
    assert J.nmbEvents() == 60 and np.allclose(J.matrix(), 2 * I.matrix(), rtol=1e-15)
    J -= I
    assert J.nmbEvents() == 30
    J *= 2.0
    assert J.nmbEvents() == 60
    J /= 2.0
    J.renormalize(90)
    assert J.nmbEvents() == 90 and np.allclose(J.matrix(), 3 * I.matrix(), rtol=1e-14)
    # wave sets must match for +=
    K = R.ampIntegralMatrix()
    K.setWaveNames(["a", "b", "c", "d", "x"])
    with pytest.raises(R.PwaError):
        J += K
    # a second setWaveNames with other names is refused (ampIntegralMatrix.cc:255-277)
    with pytest.raises(R.PwaError):
        I.setWaveNames(["q"] * 5)


def _layout_pair(n_neg, n_pos, rank, thresholds=None, mass=0.0):
    names, refl = synth.wave_names(n_neg, n_pos)
    L = R.pwaLikelihood()
    L.init(names, refl, thresholds, rank, mass)
    O = OracleLikelihood()
    assert O.init(names, refl, thresholds, rank, mass)
    return L, O, names


@pytest.mark.parametrize("n_neg,n_pos,rank", [(0, 15, 1), (7, 80, 2), (2, 5, 3), (1, 1, 1), (3, 0, 2), (4, 4, 4)])
def test_parameter_layout_matches_oracle(n_neg, n_pos, rank):
    """buildParDataStruct (pwaLikelihood.cc:1489-1556) and parName (:107-122)."""
    L, O, names = _layout_pair(n_neg, n_pos, rank)
    assert L.nmbPars() == O.nmbPars() == synth.n_pars(n_neg, n_pos, rank)
    for k in range(L.nmbPars()):
        assert L.parameter(k)["name"] == O.parName(k)
    assert L.parameter(L.nmbPars() - 1)["name"] == "V_flat_RE"
    assert L.nmbWaves() == n_neg + n_pos
    assert L.nmbWaves(+1) == n_pos and L.nmbWaves(-1) == n_neg
    assert L.rank() == rank


def test_threshold_fixing():
    th = [0.0, 1.5, 2.0, 0.0, 1.0]
    L, O, names = _layout_pair(2, 3, 1, thresholds=th, mass=1.7)
    fixed = [L.parameter(k)["fixed"] for k in range(L.nmbPars())]
    assert fixed == [O.parFixed(k) for k in range(O.nmbPars())]
    # only the positive-reflectivity anchor (threshold 2.0 >= 1.7) is fixed: one real parameter
    assert L.nmbParsFixed() == O.nmbParsFixed() == 1
    assert any(fixed)


@pytest.mark.parametrize("fix", [False, True])
def test_hessian_eigenvectors(fix):
    """HessianEigenVectors (pwaLikelihood.cc:864-912): the eigen-decomposition
    of the free-parameter block of the Hessian, checked against LAPACK's
    symmetric solver (numpy.linalg.eigh)."""
    th = [0.0, 1.5, 2.0, 0.0, 1.0, 0.0, 0.0] if fix else None
    L, O, names = _layout_pair(3, 4, 2, thresholds=th, mass=1.7)
    P = L.nmbPars()
    free = [k for k in range(P) if not L.parameter(k)["fixed"]]
    assert len(free) == P - L.nmbParsFixed()
    assert (L.nmbParsFixed() > 0) == fix
    rng = np.random.default_rng(5)
    X = rng.standard_normal((P, P))
    H = X @ X.T + np.diag(np.linspace(0.1, 3.0, P))
    H[0, 1] += 1e-13        # asymmetric at rounding level: symmetrised
    pairs = L.HessianEigenVectors(H)
    assert len(pairs) == len(free)
    Hr = H[np.ix_(free, free)]
    Hr = 0.5 * (Hr + Hr.T)
    w, U = np.linalg.eigh(Hr)
    w, U = w[::-1], U[:, ::-1]
    vals = np.array([v for _, v in pairs])
    assert np.all(np.diff(vals) <= 0)
    np.testing.assert_allclose(vals, w, rtol=1e-12, atol=1e-12 * abs(w).max())
    fixed = [k for k in range(P) if k not in free]
    for k, (vec, val) in enumerate(pairs):
        assert vec.shape == (P,)
        assert np.all(vec[fixed] == 0.0)
        assert abs(np.linalg.norm(vec) - 1.0) < 1e-12
        assert abs(abs(vec[free] @ U[:, k]) - 1.0) < 1e-10
        r = Hr @ vec[free] - val * vec[free]
        assert np.linalg.norm(r) < 1e-11 * abs(w).max()
    # degenerate eigenvalues: the identity has every vector as eigenvector
    pairs = L.HessianEigenVectors(np.eye(P))
    V = np.array([v[free] for v, _ in pairs])
    np.testing.assert_allclose(V @ V.T, np.eye(len(free)), atol=1e-14)
    assert all(v == 1.0 for _, v in pairs)
    with pytest.raises(R.PwaError):
        Hb = H.copy()
        Hb[free[0], free[0]] = np.nan
        L.HessianEigenVectors(Hb)


def test_correct_param_signs_and_prod_amps_match_oracle():
    L, O, names = _layout_pair(3, 6, 2)
    rng = np.random.default_rng(1)
    for _ in range(5):
        p = rng.standard_normal(L.nmbPars())
        p[0] = -abs(p[0])
        p[-1] = -abs(p[-1])
        assert np.array_equal(L.CorrectParamSigns(p), O.CorrectParamSigns(p))
    amps, idx = L.buildProdAmpArrays(p, withFlat=True)
    assert idx[-1] == (L.nmbPars() - 1, -1)
    assert amps[-1] == p[-1]
    assert len(amps) == sum(1 for k in range(L.nmbPars()) if L.parameter(k)["realPart"])


def test_setup_order_is_enforced():
    """addNormIntegral before init, addAcc before addNorm, evaluation before
    finishInit are refused as in pwaLikelihood.cc:1066-1107, :177-180."""
    names, refl = synth.wave_names(0, 3)
    I = R.ampIntegralMatrix()
    I.setWaveNames(names)
    L = R.pwaLikelihood()
    with pytest.raises(R.PwaError) as e:
        L.addNormIntegral(I)
    assert e.value.status == 2
    L.init(names, refl, None, 1, 0.0)
    with pytest.raises(R.PwaError):
        L.addAccIntegral(I)
    with pytest.raises(R.PwaError) as e:
        L.FdF(np.zeros(L.nmbPars()))
    assert e.value.status == 2
    with pytest.raises(R.PwaError):
        R.pwaLikelihood().init(["a", "a"], [1, 1])
    with pytest.raises(R.PwaError):
        R.pwaLikelihood().init(["a"], [0])
    with pytest.raises(R.PwaError):
        R.pwaLikelihood().setStoreBlock(100)  # 64 or 128 events only
    R.pwaLikelihood().setStoreBlock(64)


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU failure path")
def test_device_work_fails_loudly_without_gpu():
    w = synth.make_workload("compass15", n_data=50, n_mc=50)
    L = R.pwaLikelihood()
    L.init(w["names"], w["refl"], None, 1, 0.0)
    I = R.ampIntegralMatrix()
    I.setWaveNames(w["names"])
    I.setMatrix(np.eye(15))
    I.setNmbEvents(10)
    L.addNormIntegral(I)
    L.addAccIntegral(I)
    with pytest.raises(R.PwaError) as e:
        L.addAmplitude(w["names"][0], w["data"][0])
    assert e.value.status == 3
    J = R.ampIntegralMatrix()
    with pytest.raises(R.PwaError):
        J.integrate(w["names"], w["mc"])


def test_reference_accessors_without_gpu():
    """normalizedAmpsUsed / priorType / cauchyWidth, enableCuda / cudaEnabled,
    dLcache before any evaluation, clear and Clone (pwaLikelihood.h:160-224,
    pwaLikelihood.cc:1670-1674)."""
    L, O, names = _layout_pair(2, 3, 1)
    assert L.normalizedAmpsUsed() and L.priorType() == 0 and L.cauchyWidth() == 0.5
    L.useNormalizedAmps(False)
    L.setPriorType(1)
    L.setCauchyWidth(0.25)
    assert (L.normalizedAmpsUsed(), L.priorType(), L.cauchyWidth()) == (False, 1, 0.25)
    assert L.cudaEnabled()
    L.enableCuda(True)
    with pytest.raises(R.PwaError):
        L.enableCuda(False)
    with pytest.raises(R.PwaError) as e:
        L.dLcache(0)
    assert e.value.status == 2
    assert L.ncalls() == 0 and L.Ltime() == 0.0 and L.Ntime() == 0.0
    L.clear()
    with pytest.raises(R.PwaError):
        L.Clone()


def test_integral_comparison_and_clear():
    """containsWave, hasIdenticalWaveSet, operator == and clear
    (ampIntegralMatrix.cc:93-103, :188-191, :633-646; .h:179-195)."""
    rng = np.random.default_rng(4)
    A = rng.standard_normal((3, 20)) + 1j * rng.standard_normal((3, 20))

    def build(names, amps):
        I = R.ampIntegralMatrix()
        I.setWaveNames(names)
        for e in range(amps.shape[1]):
            I.addEvent(amps[:, e])
        return I
    I1 = build(["a", "b", "c"], A)
    I2 = build(["c", "a", "b"], A[[2, 0, 1]])          # same sums, other wave order
    assert I1.containsWave("b") and not I1.containsWave("d")
    assert I1.hasIdenticalWaveSet(I2) and I1 == I2 and not (I1 != I2)
    I3 = build(["a", "b", "c"], A[:, :19])
    assert I1.hasIdenticalWaveSet(I3) and I1 != I3
    I4 = build(["a", "b", "x"], A)
    assert not I1.hasIdenticalWaveSet(I4) and I1 != I4
    I1.clear()
    assert I1.nmbWaves() == 0 and I1.nmbEvents() == 0 and not I1.containsWave("a")


def test_gram_batch_rejects_bad_arguments_without_device_work():
    """pwa_gram_device_batch checks its arguments before any device call."""
    one = (C.c_void_p * 1)(C.c_void_p(16))
    with pytest.raises(N.PwaError) as e:
        N.call("pwa_gram_device_batch", None, None, 1, 8, N.PRECISION["fp32"], None, None, None)
    assert e.value.status == N.ERROR_INVALID_ARGUMENT
    with pytest.raises(N.PwaError) as e:
        N.call("pwa_gram_device_batch", one, (C.c_uint64 * 1)(8), 1, 1025, N.PRECISION["fp32"],
               C.c_void_p(16), None, None)
    assert e.value.status == N.ERROR_INVALID_ARGUMENT and "1024" in str(e.value)
    with pytest.raises(N.PwaError) as e:
        N.call("pwa_gram_device_batch", one, (C.c_uint64 * 1)(0), 1, 8, N.PRECISION["fp32"],
               C.c_void_p(16), None, None)
    assert e.value.status == N.ERROR_INVALID_ARGUMENT
    with pytest.raises(N.PwaError) as e:
        N.call("pwa_gram_device_batch", one, (C.c_uint64 * 1)(8), 1, 8, N.PRECISION["fp64"],
               C.c_void_p(16), None, None)
    assert e.value.status == 7
