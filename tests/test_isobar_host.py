"""CPU tests of the isobar decay amplitudes: the GPU kernel's per-event
arithmetic (rootpwa_gb300/csrc/isobar_math.cuh) and the wave-plan builder,
compiled as host code by g++ (tests/isobar_host_shim.cpp), against the FP64
oracle for every option of isobarAmplitude (isobarAmplitude.h:68-75); the
library's spin-algebra utilities against the oracle; argument checks of the
C ABI; and the loud failure of the evaluation without a GPU."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import isobar_oracle as O
from rootpwa_gb300 import _native as N
from rootpwa_gb300 import isobar as I
from isobar_cases import NAMES, SPECIES, TOL, TOL32, events, rel_err, tolerances, waves

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("isobar") / "shim.so")
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-o", out,
                    os.path.join(HERE, "isobar_host_shim.cpp")], check=True)
    return C.CDLL(out)


def _c_waves(ws):
    arr = (N.IsobarWave * len(ws))()
    for k, (_, kw) in enumerate(ws):
        arr[k] = N.IsobarWave(J=kw["J"], P=kw["P"], M=kw["M"], refl=kw["refl"], L=kw["L"], S=kw["S"],
                              isobarJ=kw["isobarJ"], isobarL=kw["isobarL"], isobarS=0,
                              massDependence=I.MASS_DEPENDENCES[kw["massDependence"]],
                              isobarMass=kw["isobarMass"], isobarWidth=kw["isobarWidth"],
                              isobarDaughter1=kw["isobarDaughters"][0], isobarDaughter2=kw["isobarDaughters"][1],
                              bachelor=kw["bachelor"], bachelorFirst=int(kw.get("bachelorFirst", False)),
                              isospin=kw.get("isospin", 2), isobarIsospin=kw.get("isobarIsospin", 0),
                              binLower=kw.get("bounds", (0.0, 0.0))[0], binUpper=kw.get("bounds", (0.0, 0.0))[1])
        for j, v in enumerate(kw.get("massDepParams", ())):
            arr[k].massDepParams[j] = v
    return arr


def _shim_amps(lib, ws, beam, fs, masses, mb, opts, dtype=np.complex128):
    n = beam.shape[0]
    b = np.ascontiguousarray(beam.T)
    f = np.ascontiguousarray(np.transpose(fs, (0, 2, 1)))
    out = np.zeros((len(ws), n), dtype=dtype)
    m = np.ascontiguousarray(masses, dtype=np.float64)
    sp = np.ascontiguousarray(opts.get("species", SPECIES), dtype=np.int32)
    iso = None
    if opts.get("isospin"):
        I, I3, P = opts["isospin"]
        iso = np.ascontiguousarray(np.array([I, I3, P]).T, dtype=np.int32)
    rc = lib.shim_amplitudes(_c_waves(ws), len(ws), m.ctypes.data_as(C.c_void_p), sp.ctypes.data_as(C.c_void_p),
                             C.c_double(mb), int(opts.get("reflectivity_basis", True)), int(opts.get("bose", True)),
                             int(opts.get("space_inversion", False)), int(opts.get("reflection", False)),
                             b.ctypes.data_as(C.c_void_p), f.ctypes.data_as(C.c_void_p), C.c_uint64(n),
                             out.ctypes.data_as(C.c_void_p), int(dtype == np.complex64),
                             int(opts.get("formalism", "helicity") == "canonical"),
                             iso.ctypes.data_as(C.c_void_p) if iso is not None else None)
    assert rc == 0
    return out


OPTIONS = [{}, {"bose": False}, {"space_inversion": True}, {"reflection": True},
           {"space_inversion": True, "reflection": True}, {"formalism": "canonical"},
           {"formalism": "canonical", "bose": False, "reflection": True}]
OPTION_IDS = ["default", "no-bose", "inversion", "reflection", "both", "canonical", "canonical-no-bose-reflection"]


@pytest.mark.parametrize("opts", OPTIONS, ids=OPTION_IDS)
def test_kernel_arithmetic_matches_oracle(shim, opts):
    ws = waves()
    beam, fs, masses, mb = events(1500, seed=5)
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, SPECIES, **opts)
    got = _shim_amps(shim, ws, beam, fs, masses, mb, opts)
    err = rel_err(ref, got)
    assert np.all(err < tolerances(ws, TOL)), err
    # the parity-forbidden combination of the last wave is exactly zero in both
    assert np.all(ref[-1] == 0) and np.all(got[-1] == 0)


@pytest.mark.parametrize("opts", [OPTIONS[0], OPTIONS[1], OPTIONS[5]], ids=["default", "no-bose", "canonical"])
def test_kernel_arithmetic_complex64_mode(shim, opts):
    """FP64 frames and kinematics, FP32 per-wave arithmetic, complex64 out."""
    ws = waves()
    beam, fs, masses, mb = events(1500, seed=7)
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, SPECIES, **opts)
    got = _shim_amps(shim, ws, beam, fs, masses, mb, opts, np.complex64)
    err = rel_err(ref, got.astype(np.complex128))
    assert np.all(err < tolerances(ws, TOL32)), err
    assert np.all(got[-1] == 0)


@pytest.mark.parametrize("formalism", ["helicity", "canonical"])
def test_kernel_arithmetic_without_reflectivity_basis(shim, formalism):
    """without the reflectivity basis M may be negative (DFunctionConj)."""
    ws = [(dict(w, M=-w["M"]), dict(kw, M=-kw["M"])) for w, kw in waves()[:4]]
    beam, fs, masses, mb = events(500, seed=6)
    opts = {"reflectivity_basis": False, "formalism": formalism}
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, SPECIES, **opts)
    got = _shim_amps(shim, ws, beam, fs, masses, mb, opts)
    assert np.all(rel_err(ref, got) < tolerances(ws, TOL))


def test_spin_algebra_utilities_match_oracle():
    for j1 in range(0, 7):
        for j2 in range(0, 5):
            for J in range(abs(j1 - j2), j1 + j2 + 1, 2):
                for m1 in range(-j1, j1 + 1, 2):
                    for m2 in range(-j2, j2 + 1, 2):
                        assert abs(I.clebschGordanCoeff(j1, m1, j2, m2, J, m1 + m2)
                                   - O.clebsch_gordan(j1, m1, j2, m2, J, m1 + m2)) < 1e-13
    for j in range(0, 17):
        for m in range(-j, j + 1, 2):
            for n in range(-j, j + 1, 2):
                for t in (0.0, 0.4, 2.2, np.pi):
                    assert abs(I.dFunction(j, m, n, t) - float(O.wigner_d(j, m, n, t))) < 1e-12
    # barrier factors: the library's integer polynomials against the oracle's
    # spherical Hankel functions
    for L in range(0, 16, 2):
        for q in (0.0, 0.05, 0.1973, 0.4, 1.3, 5.0):
            assert abs(I.barrierFactor(L, q) - float(O.barrier_factor(L, q))) < 1e-12 * max(1.0, I.barrierFactor(L, q))
    with pytest.raises(N.PwaError):
        I.dFunction(2, 3, 0, 0.1)
    with pytest.raises(N.PwaError):
        I.barrierFactor(16, 0.1)


def test_wave_checks_and_state():
    A = I.isobarHelicityAmplitudes()
    kw = waves()[0][1]
    with pytest.raises(N.PwaError) as e:
        A.amplitudes(np.zeros((1, 3)), np.zeros((3, 1, 3)))
    assert e.value.status == 2                      # no final state, no waves
    A.setFinalState(NAMES, [0.1396] * 3, 0.1396)
    with pytest.raises(N.PwaError):
        A.nmbSymTerms(0)                            # no wave yet
    bad = [dict(kw, J=3), dict(kw, M=-2), dict(kw, P=0), dict(kw, L=16), dict(kw, bachelor=1),
           dict(kw, isobarDaughters=(0, 3)), dict(kw, massDependence=13), dict(kw, isobarWidth=0.0),
           dict(kw, M=6)]
    for b in bad:
        with pytest.raises(N.PwaError) as e:
            A.addWave(**b)
        assert e.value.status == 1, b
    assert A.nmbWaves() == 0
    A.addWave(**kw)
    assert A.nmbWaves() == 1
    assert A.nmbSymTerms(0) == 2                    # the two pi- exchange
    A.enableBoseSymmetrization(False)
    assert A.nmbSymTerms(0) == 1
    A.enableBoseSymmetrization(True)
    assert A.waveName(0) == "[1-,1++,0+]=[isobar=[pi+[1,0]pi-][0,1]pi-]"
    with pytest.raises(N.PwaError):
        A.setFinalState(["pi-", "pi+", "pi-"], [0.1396, 0.1396, 0.14], 0.1396)   # identical, unequal masses
    with pytest.raises(N.PwaError):
        A.setFinalState(["a", "b"], [0.1, 0.2], 0.1)                          # not three particles
    # the helicity basis admits M < 0; switching the reflectivity basis back on is refused then
    A.enableReflectivityBasis(False)
    A.addWave(**dict(kw, M=-2))
    with pytest.raises(N.PwaError):
        A.enableReflectivityBasis(True)
    assert not A.reflectivityBasis()
    with pytest.raises(N.PwaError):
        N.call("pwa_isobar_set_stream", None, None)


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour without a GPU")
def test_evaluation_fails_loudly_without_gpu():
    A = I.isobarHelicityAmplitudes()
    A.setFinalState(NAMES, [0.1396] * 3, 0.1396)
    A.addWave(**waves()[0][1])
    beam, fs, masses, mb = events(10, seed=1)
    with pytest.raises(N.PwaError) as e:
        A.amplitudes(beam, fs)
    assert e.value.status == 3
    # no events: nothing to do, no device needed
    out = A.amplitudes(np.zeros((0, 3)), np.zeros((3, 0, 3)))
    assert out.shape == (1, 0)


def test_three_pion_wave_set(shim):
    """the 88-wave benchmark set (rootpwa_gb300.synth.three_pion_waves):
    accepted by the library, parity-conserving, and the kernel arithmetic
    matches the oracle on every wave."""
    from rootpwa_gb300 import synth
    kws = synth.three_pion_waves()
    A = I.isobarHelicityAmplitudes()
    A.setFinalState(NAMES, [synth.M_PI] * 3, synth.M_PI)
    for kw in kws:
        A.addWave(**kw)
    assert A.nmbWaves() == 88
    assert len({A.waveName(k) for k in range(88)}) == 88
    ws = [(O.wave(kw["J"], kw["P"], kw["M"], kw["refl"], kw["L"], kw["S"], kw["isobarJ"], kw["isobarL"],
                  I.MASS_DEPENDENCES[kw["massDependence"]], kw["isobarMass"], kw["isobarWidth"],
                  kw["isobarDaughters"], kw["bachelor"]), kw) for kw in kws]
    beam, fs, masses, mb = events(300, seed=8)
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, SPECIES)
    got = _shim_amps(shim, ws, beam, fs, masses, mb, {})
    assert np.all(rel_err(ref, got) < tolerances(ws, TOL))
    assert np.all(np.abs(ref).max(axis=1) > 0)          # no wave vanishes identically
    par = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, SPECIES, space_inversion=True)
    for k, (w, _) in enumerate(ws):
        assert np.abs(par[k] + w["P"] * ref[k]).max() < 1e-10 * np.abs(ref[k]).max()


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("formalism", ["helicity", "canonical"])
def test_kernel_arithmetic_isospin_symmetrisation(shim, dtype, formalism):
    """pi- pi0 pi0 with isospin symmetrisation (isobarDecayTopology.cc:505-630)
    combined with the Bose terms of the two pi0."""
    from isobar_cases import NEUTRAL_ISOSPIN, NEUTRAL_SPECIES, neutral_events, neutral_waves
    ws = neutral_waves()
    beam, fs, masses, mb = neutral_events(1000, seed=10)
    opts = {"isospin": NEUTRAL_ISOSPIN, "formalism": formalism}
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, NEUTRAL_SPECIES, **opts)
    got = _shim_amps(shim, ws, beam, fs, masses, mb, dict(opts, species=NEUTRAL_SPECIES), dtype)
    tol = TOL if dtype == np.complex128 else TOL32
    assert np.all(rel_err(ref, got.astype(np.complex128)) < tolerances(ws, tol))


def test_isospin_api():
    from isobar_cases import NEUTRAL_NAMES, NEUTRAL_MASSES, neutral_waves
    A = I.isobarHelicityAmplitudes()
    A.setFinalState(NEUTRAL_NAMES, NEUTRAL_MASSES, 0.1396)        # pion isospins filled in
    for _, kw in neutral_waves():
        A.addWave(**kw)
    assert not A.isospinSymmetrization()
    assert [A.nmbSymTerms(k) for k in range(5)] == [2] * 5          # Bose: the two pi0
    A.enableIsospinSymmetrization(True)
    assert [A.nmbSymTerms(k) for k in range(5)] == [4, 4, 2, 2, 4]  # isospin x Bose terms
    B = I.isobarHelicityAmplitudes()
    B.setFinalState(["a", "b", "c"], [0.1, 0.2, 0.3], 0.1)           # no isospins known
    with pytest.raises(N.PwaError) as e:
        B.enableIsospinSymmetrization(True)
    assert e.value.status == 2
    with pytest.raises(N.PwaError):
        B.setFinalState(["a", "b", "c"], [0.1, 0.2, 0.3], 0.1, isospins=[(1, 3, 1)] * 3)   # |2I_3| > 2I


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_kernel_arithmetic_kpipi(shim, dtype):
    """K- pi+ pi- with the K pi S-wave forms (massDependence.cc:700-828)."""
    from isobar_cases import KPIPI_SPECIES, kpipi_events, kpipi_waves
    ws = kpipi_waves()
    beam, fs, masses, mb = kpipi_events(1500, seed=12)
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, KPIPI_SPECIES)
    got = _shim_amps(shim, ws, beam, fs, masses, mb, {"species": KPIPI_SPECIES}, dtype)
    tol = TOL if dtype == np.complex128 else TOL32
    assert np.all(np.abs(ref).max(axis=1) > 0)
    assert np.all(rel_err(ref, got.astype(np.complex128)) < tolerances(ws, tol))


def test_shape_checks():
    """mismatched event counts are refused before any buffer is read."""
    A = I.isobarHelicityAmplitudes()
    A.setFinalState(NAMES, [0.1396] * 3, 0.1396)
    A.addWave(**waves()[0][1])
    with pytest.raises(ValueError):
        A.amplitudes(np.zeros((5, 3)), np.zeros((3, 4, 3)))
    with pytest.raises(ValueError):
        A.amplitudes(np.zeros((5, 2)), np.zeros((3, 5, 3)))
    with pytest.raises(ValueError):
        A.amplitudes(np.zeros((5, 3)), np.zeros((2, 5, 3)))


def test_native_amplitude_file_header_without_events(tmp_path):
    """pwa_isobar_write_amp_file with no events writes a valid file (header,
    the "mass" variable and the caller's variables) without touching the
    GPU; argument and state errors are refused."""
    from rootpwa_gb300 import ampFileInfo
    A = I.isobarHelicityAmplitudes()
    with pytest.raises(N.PwaError):
        I.writeAmplitudeFileNative(A, tmp_path / "x.amp", np.zeros((0, 3)), np.zeros((3, 0, 3)), ["w"])
    A.setFinalState(NAMES, [0.1396] * 3, 0.1396)
    for _, kw in waves()[:3]:
        A.addWave(**kw)
    names = I.writeAmplitudeFileNative(A, tmp_path / "e.amp", np.zeros((0, 3)), np.zeros((3, 0, 3)),
                                       binVars={"tPrime": np.zeros(0)})
    waves_, n, vars_ = ampFileInfo(tmp_path / "e.amp")
    assert waves_ == names and n == 0 and vars_ == ["mass", "tPrime"]
