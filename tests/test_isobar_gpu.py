"""GPU parity of the three-body isobar amplitude kernel (isobar.cu) against
the FP64 oracle (oracle/isobar_oracle.py, which restates
isobarHelicityAmplitude / isobarAmplitude, decayAmplitude/isobarAmplitude.cc:
98-262, isobarHelicityAmplitude.cc:64-195), through the C ABI with host and
device buffers; ragged and large event counts; and the chain events ->
amplitudes -> integrals -> likelihood against the same chain in the oracle.

Tolerance: max |A_gpu - A_oracle| per wave below 1e-9 of the wave's largest
|A| (FP64 throughout; the frames boost ~190 GeV/c momenta by gamma ~ 100);
5e-6 in the complex64 mode (FP32 per-wave arithmetic)."""
import numpy as np
import pytest

import rootpwa_gb300 as R
from oracle import isobar_oracle as O
from rootpwa_gb300 import isobar as I
import helpers
from helpers import F_RTOL, G_NORMWISE, normwise, rel
from isobar_cases import NAMES, SPECIES, TOL, TOL32, events, rel_err, tolerances, waves

pytestmark = pytest.mark.gpu

OPTIONS = [{}, {"bose": False}, {"space_inversion": True}, {"reflection": True},
           {"space_inversion": True, "reflection": True}, {"formalism": "canonical"},
           {"formalism": "canonical", "bose": False, "reflection": True}]
OPTION_IDS = ["default", "no-bose", "inversion", "reflection", "both", "canonical", "canonical-no-bose-reflection"]
SETTERS = {"bose": "enableBoseSymmetrization", "space_inversion": "enableSpaceInversion",
           "reflection": "enableReflection", "reflectivity_basis": "enableReflectivityBasis"}


def _amp(ws, masses, mb, opts=None):
    opts = dict(opts or {})
    canonical = opts.pop("formalism", "helicity") == "canonical"
    A = I.isobarCanonicalAmplitudes() if canonical else I.isobarHelicityAmplitudes()
    A.setFinalState(NAMES, masses, mb)
    for k, v in opts.items():
        getattr(A, SETTERS[k])(v)
    for _, kw in ws:
        A.addWave(**kw)
    return A


@pytest.mark.parametrize("opts", OPTIONS, ids=OPTION_IDS)
def test_amplitudes_match_oracle_host_buffers(opts):
    ws = waves()
    beam, fs, masses, mb = events(2000, seed=11)
    A = _amp(ws, masses, mb, opts)
    got = A.amplitudes(beam, fs)
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, SPECIES, **opts)
    assert got.shape == ref.shape and got.dtype == np.complex128
    err = rel_err(ref, got)
    assert np.all(err < tolerances(ws, TOL)), err
    assert np.all(got[-1] == 0)                       # zero by reflectivity (M = 0, f = +1)


@pytest.mark.parametrize("opts", [OPTIONS[0], OPTIONS[1], OPTIONS[5]], ids=["default", "no-bose", "canonical"])
def test_complex64_mode_matches_oracle(opts):
    import torch
    ws = waves()
    beam, fs, masses, mb = events(3000, seed=17)
    A = _amp(ws, masses, mb, opts)
    got = A.amplitudes(beam, fs, dtype="complex64")
    assert got.dtype == np.complex64
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, SPECIES, **opts)
    err = rel_err(ref, got.astype(np.complex128))
    assert np.all(err < tolerances(ws, TOL32)), err
    dev = A.amplitudes(torch.from_numpy(beam).cuda(), torch.from_numpy(fs).cuda(), dtype="complex64")
    assert dev.dtype == torch.complex64
    assert np.array_equal(dev.cpu().numpy(), got)


def test_amplitudes_device_buffers_equal_host_buffers():
    import torch
    ws = waves()
    beam, fs, masses, mb = events(3000, seed=12)
    A = _amp(ws, masses, mb)
    host = A.amplitudes(beam, fs)
    dev = A.amplitudes(torch.from_numpy(beam).cuda(), torch.from_numpy(fs).cuda())
    assert dev.is_cuda and dev.dtype == torch.complex128
    assert np.array_equal(dev.cpu().numpy(), host)    # same kernel, same inputs: bitwise


@pytest.mark.parametrize("n", [1, 31, 127, 129, 4099])
def test_ragged_event_counts(n):
    ws = waves()[:4]
    beam, fs, masses, mb = events(n, seed=13)
    got = _amp(ws, masses, mb).amplitudes(beam, fs)
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, SPECIES)
    assert np.all(rel_err(ref, got) < tolerances(ws, TOL))


def test_helicity_basis_negative_projection():
    ws = [(dict(w, M=-w["M"]), dict(kw, M=-kw["M"])) for w, kw in waves()[:4]]
    beam, fs, masses, mb = events(1000, seed=14)
    got = _amp(ws, masses, mb, {"reflectivity_basis": False}).amplitudes(beam, fs)
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, SPECIES, reflectivity_basis=False)
    assert np.all(rel_err(ref, got) < tolerances(ws, TOL))


def test_large_event_count_by_tiling():
    """3,000,000 events (grid-stride loop well past one pass of the grid):
    a 2,000-event block tiled 1,500 times gives 1,500 bitwise copies of the
    block's amplitudes, and the block matches the oracle."""
    import torch
    ws = waves()
    beam, fs, masses, mb = events(2000, seed=15)
    A = _amp(ws, masses, mb)
    small = A.amplitudes(torch.from_numpy(beam).cuda(), torch.from_numpy(fs).cuda())
    reps = 1500
    big = A.amplitudes(torch.from_numpy(beam).cuda().repeat(reps, 1), torch.from_numpy(fs).cuda().repeat(1, reps, 1))
    assert big.shape == (len(ws), 2000 * reps)
    assert torch.equal(big.view(len(ws), reps, 2000), small.unsqueeze(1).expand(-1, reps, -1))
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, SPECIES)
    assert np.all(rel_err(ref, small.cpu().numpy()) < tolerances(ws, TOL))


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_events_to_likelihood_chain(dtype):
    """amplitudes of data and MC events on the GPU -> GPU integrals -> GPU
    likelihood, against oracle amplitudes -> oracle integrals -> oracle
    likelihood; FdF within the likelihood's tolerances.  In the complex64
    mode the oracle chain starts from the GPU's complex64 amplitudes (cast to
    complex128), whose own error the tests above bound."""
    import torch
    ws = waves()[:8]                                   # the non-zero waves
    data = events(4000, seed=21)
    mc = events(20000, seed=22)
    masses, mb = data[2], data[3]
    A = _amp(ws, masses, mb)
    names = ["w%d_%s" % (k, A.waveName(k)) for k in range(len(ws))]
    refl = [kw["refl"] for _, kw in ws]
    accepted = np.random.default_rng(23).random(20000) < 0.7
    Ow = [w for w, _ in ws]
    w_or = dict(names=names, refl=refl, rank=1,
                data=O.amplitudes(Ow, data[0], data[1], masses, mb, SPECIES),
                mc=O.amplitudes(Ow, mc[0], mc[1], masses, mb, SPECIES), accepted=accepted)
    Lo = helpers.build_oracle(w_or)
    d_data = A.amplitudes(torch.from_numpy(data[0]).cuda(), torch.from_numpy(data[1]).cuda(), dtype=dtype)
    d_mc = A.amplitudes(torch.from_numpy(mc[0]).cuda(), torch.from_numpy(mc[1]).cuda(), dtype=dtype)
    if dtype == "complex64":
        w_or = dict(w_or, data=d_data.cpu().numpy().astype(np.complex128),
                    mc=d_mc.cpu().numpy().astype(np.complex128))
        Lo = helpers.build_oracle(w_or)
    w_gpu = dict(w_or, data=d_data, mc=d_mc)
    norm, acc = helpers.gpu_integrals(w_gpu, precision="fp64")
    Lg = helpers.build_gpu(w_gpu, norm, acc, amps=[d_data[k] for k in range(len(ws))])
    p = np.random.default_rng(24).standard_normal(Lg.nmbPars())
    f0, g0 = Lo.FdF(p)
    f1, g1 = Lg.FdF(p)
    assert rel(f1, f0) < F_RTOL
    assert normwise(g1, g0) < G_NORMWISE


def test_no_events():
    ws = waves()[:2]
    beam, fs, masses, mb = events(10, seed=1)
    out = _amp(ws, masses, mb).amplitudes(np.zeros((0, 3)), np.zeros((3, 0, 3)))
    assert out.shape == (2, 0)


def test_caller_stream():
    """pwa_isobar_set_stream: device-buffer calls run asynchronously on the
    caller's stream; results equal the synchronous host-buffer call's."""
    import torch
    ws = waves()[:4]
    beam, fs, masses, mb = events(5000, seed=16)
    A = _amp(ws, masses, mb)
    host = A.amplitudes(beam, fs)
    s = torch.cuda.Stream()
    A.setStream(s)
    with torch.cuda.stream(s):
        dev = A.amplitudes(torch.from_numpy(beam).cuda(), torch.from_numpy(fs).cuda())
    s.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)
    assert np.array_equal(A.amplitudes(beam, fs), host)       # host buffers: synchronous on that stream


def test_evt_file_to_amplitude_file_to_likelihood(tmp_path):
    """events in an .evt file -> calcAmplitudes (GPU, complex64) -> raw
    amplitude file with the 3pi mass -> likelihood with on-the-fly binning
    on that mass, against the same likelihood fed the selected events'
    amplitudes directly."""
    from rootpwa_gb300 import evtfile, synth
    ws = waves()[:8]
    beam, fs, masses, mb = events(6000, seed=41)
    evt = tmp_path / "ev.evt"
    evtfile.writeEvtFile(evt, 9, beam, [9, 8, 9], fs)
    A = _amp(ws, masses, mb)
    names = I.calcAmplitudes(A, evt, tmp_path / "ev.amp")
    assert len(names) == len(ws) and len(set(names)) == len(ws)
    amps = A.amplitudes(beam, fs, dtype="complex64")
    m3 = I.finalStateMass(evtfile.readEvtFile(evt))
    keep = (m3 >= 1.2) & (m3 < 1.6)
    refl = [kw["refl"] for _, kw in ws]
    mc = A.amplitudes(*events(20000, seed=42)[:2], dtype="complex64")
    norm = R.ampIntegralMatrix()
    norm.integrate(names, mc, precision="fp64")
    p = np.random.default_rng(43)

    def lik(load):
        L = R.pwaLikelihood()
        L.init(names, refl, None, 1, 0.0)
        n2 = R.ampIntegralMatrix()
        n2.setWaveNames(names)
        n2.setMatrix(norm.matrix())
        n2.setNmbEvents(norm.nmbEvents())
        a2 = R.ampIntegralMatrix()
        a2.setWaveNames(names)
        a2.setMatrix(norm.matrix())
        a2.setNmbEvents(norm.nmbEvents())
        L.addNormIntegral(n2)
        L.addAccIntegral(a2)
        load(L)
        L.finishInit()
        return L
    Lf = lik(lambda L: L.loadAmplitudeFiles([tmp_path / "ev.amp"], {"mass": (1.2, 1.6)}))
    Ld = lik(lambda L: [L.addAmplitude(n, np.ascontiguousarray(amps[k][keep])) for k, n in enumerate(names)])
    assert Lf.nmbEvents() == Ld.nmbEvents() == int(keep.sum())
    x = p.standard_normal(Lf.nmbPars())
    f1, g1 = Lf.FdF(x)
    f2, g2 = Ld.FdF(x)
    assert f1 == f2 and np.array_equal(g1, g2)


@pytest.mark.parametrize("formalism", ["helicity", "canonical"])
@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_isospin_symmetrisation_matches_oracle(formalism, dtype):
    """pi- pi0 pi0 with isospin symmetrisation: per-term frames where the
    permutation exchanges the pi- and a pi0 (different masses)."""
    from isobar_cases import (NEUTRAL_ISOSPIN, NEUTRAL_NAMES, NEUTRAL_SPECIES, neutral_events,
                              neutral_waves)
    ws = neutral_waves()
    beam, fs, masses, mb = neutral_events(2500, seed=18)
    A = I.isobarCanonicalAmplitudes() if formalism == "canonical" else I.isobarHelicityAmplitudes()
    A.setFinalState(NEUTRAL_NAMES, masses, mb)
    for _, kw in ws:
        A.addWave(**kw)
    A.enableIsospinSymmetrization(True)
    got = A.amplitudes(beam, fs, dtype=dtype).astype(np.complex128)
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, NEUTRAL_SPECIES, isospin=NEUTRAL_ISOSPIN,
                       formalism=formalism)
    tol = TOL if dtype == "complex128" else TOL32
    assert np.all(rel_err(ref, got) < tolerances(ws, tol))


def test_golden_fixture():
    """the kernel against the committed oracle amplitudes
    (tests/golden/isobar3pi_oracle.npz): pi- pi+ pi- in both formalisms and
    pi- pi0 pi0 with isospin symmetrisation."""
    import os
    from isobar_cases import NEUTRAL_NAMES, neutral_waves
    gold = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "isobar3pi_oracle.npz"))
    ws = waves()
    for formalism in ("helicity", "canonical"):
        A = _amp(ws, gold["masses"], float(gold["beam_mass"]), {"formalism": formalism})
        got = A.amplitudes(gold["beam"], gold["fs"])
        assert np.all(rel_err(gold[formalism], got) < tolerances(ws, TOL)), formalism
    nws = neutral_waves()
    B = I.isobarHelicityAmplitudes()
    B.setFinalState(NEUTRAL_NAMES, gold["neutral_masses"], float(gold["neutral_beam_mass"]))
    for _, kw in nws:
        B.addWave(**kw)
    B.enableIsospinSymmetrization(True)
    got = B.amplitudes(gold["neutral_beam"], gold["neutral_fs"])
    assert np.all(rel_err(gold["neutral_isospin"], got) < tolerances(nws, TOL))


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_kpipi_matches_oracle(dtype):
    """K- pi+ pi- with the K pi S-wave forms (massDependence.cc:700-828)."""
    from isobar_cases import KPIPI_NAMES, KPIPI_SPECIES, kpipi_events, kpipi_waves
    ws = kpipi_waves()
    beam, fs, masses, mb = kpipi_events(2000, seed=19)
    A = I.isobarHelicityAmplitudes()
    A.setFinalState(KPIPI_NAMES, masses, mb)
    for _, kw in ws:
        A.addWave(**kw)
    got = A.amplitudes(beam, fs, dtype=dtype).astype(np.complex128)
    ref = O.amplitudes([w for w, _ in ws], beam, fs, masses, mb, KPIPI_SPECIES)
    assert np.all(rel_err(ref, got) < tolerances(ws, TOL if dtype == "complex128" else TOL32))


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_host_buffers_in_slabs(dtype):
    """host-buffer calls split into device passes of at most chunk events
    (pwa_isobar_set_chunk_events) give the single-pass result bit for bit."""
    ws = waves()
    beam, fs, masses, mb = events(4099, seed=20)
    A = _amp(ws, masses, mb)
    whole = A.amplitudes(beam, fs, dtype=dtype)
    A.setChunkEvents(1000)
    assert np.array_equal(A.amplitudes(beam, fs, dtype=dtype), whole)
    A.setChunkEvents(1)
    assert np.array_equal(A.amplitudes(beam[:7], fs[:, :7], dtype=dtype), whole[:, :7])


def test_native_amplitude_file_equals_python_path(tmp_path):
    """pwa_isobar_write_amp_file (slabs of 1,000 events) writes the same
    amplitudes bit for bit as calcAmplitudes (one pass) for the same events,
    the same names and binning variables (the final-state mass computed in
    C++ and numpy agrees to rounding)."""
    from rootpwa_gb300 import evtfile
    ws = waves()[:6]
    beam, fs, masses, mb = events(3500, seed=44)
    evt = tmp_path / "ev.evt"
    evtfile.writeEvtFile(evt, 9, beam, [9, 8, 9], fs)
    ev = evtfile.readEvtFile(evt)
    A = _amp(ws, ev["fs_masses"], ev["beam_mass"])
    tp = np.random.default_rng(45).random(3500)
    names = I.calcAmplitudes(A, evt, tmp_path / "py.amp", binVars={"tPrime": tp})
    A.setChunkEvents(1000)
    I.writeAmplitudeFileNative(A, tmp_path / "native.amp", ev["beam"], ev["fs"], names, {"tPrime": tp})
    from rootpwa_gb300 import readAmplitudeFile
    w1, a1, v1 = readAmplitudeFile(tmp_path / "py.amp")
    w2, a2, v2 = readAmplitudeFile(tmp_path / "native.amp")
    assert w1 == w2 == names and list(v1) == list(v2) == ["mass", "tPrime"]
    assert np.array_equal(np.asarray(a1), np.asarray(a2))
    assert np.array_equal(np.asarray(v1["tPrime"]), np.asarray(v2["tPrime"]))
    # m = sqrt(E^2 - p^2) with E ~ 190 GeV and m ~ 1 GeV: a rounding of E^2
    # moves m by ~eps E^2 / m; both sides sum in the same order without FMA
    # contraction, so they agree far inside that bound
    p = ev["fs"].sum(axis=0)
    E = np.sum(np.sqrt(ev["fs_masses"][:, None] ** 2 + np.sum(ev["fs"] ** 2, axis=2)), axis=0)
    m1 = np.asarray(v1["mass"])
    bound = 8 * np.finfo(np.float64).eps * (E * E + np.sum(p * p, axis=1)) / np.maximum(m1, 1e-3)
    assert np.all(np.abs(m1 - np.asarray(v2["mass"])) <= bound)
