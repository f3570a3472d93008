"""Decay amplitudes of three spinless final-state particles in the isobar
model (helicity formalism), evaluated on the GPU.

Mirrors isobarHelicityAmplitude / isobarAmplitude
(decayAmplitude/isobarAmplitude.h:53-120): the option switches
enableReflectivityBasis, enableBoseSymmetrization, enableSpaceInversion and
enableReflection, and the amplitude of every wave for every event.  A wave is
what a three-body key file describes (waveDescription.cc:880-932): the X
quantum numbers, X -> isobar + bachelor with (L, S), the isobar's spin, its
decay's (L, S) and its mass dependence.  Spins, projections and orbital
angular momenta are given in units of 1/2 (2J, 2M, 2L), as in the reference.

    amp = isobarHelicityAmplitudes()
    amp.setFinalState(["pi-", "pi+", "pi-"], [m_pi] * 3, beamMass=m_pi)
    amp.addWave(J=2, P=+1, M=0, refl=+1, L=0, S=2, isobarJ=2, isobarL=2,
                massDependence="relativisticBreitWigner", isobarMass=0.769,
                isobarWidth=0.150, isobarDaughters=(1, 2), bachelor=0,
                isobarName="rho(770)")
    A = amp.amplitudes(beam, fs)       # complex128 [wave, event]

beam is (N, 3) and fs (3, N, 3) lab momenta in GeV/c: numpy arrays (host)
or CUDA tensors (device; the result is then a CUDA tensor).  Each row of the
result goes straight into pwaLikelihood.addAmplitude.
"""
import ctypes as C

import numpy as np

from . import _native as N

# (2I, 2I_3, intrinsic parity) of the pions
PION_ISOSPINS = {"pi-": (2, -2, -1), "pi0": (2, 0, -1), "pi+": (2, 2, -1)}
MASS_DEPENDENCES = {"flat": 0, "relativisticBreitWigner": 1, "constWidthBreitWigner": 2, "rhoBreitWigner": 3,
                    "f0980BreitWigner": 4, "f0980FlatteBesII": 5, "piPiSWaveAuMorganPenningtonM": 6,
                    "piPiSWaveAuMorganPenningtonVes": 7, "piPiSWaveAuMorganPenningtonKachaev": 8, "binned": 9,
                    "rhoPrime": 10, "KPiSGLASS": 11, "KPiSPalanoPennington": 12}


def _qn(x):
    """spinQn (utilities/conversionUtils.hpp:121-124) as printed: 0.5 * x."""
    return ("%d" % (x // 2)) if x % 2 == 0 else ("%g" % (0.5 * x))


def _par(x):
    return "" if x == 0 else ("+" if x > 0 else "-")


class isobarHelicityAmplitudes:
    def __init__(self):
        h = C.c_void_p()
        N.call("pwa_isobar_create", C.byref(h))
        self._h = h
        self._names = None
        self._waves = []
        self._opts = [1, 1, 0, 0]
        self._async = False
        self._stream = 0
        self._isospin = False

    def __del__(self):
        if getattr(self, "_h", None):
            try:
                N.lib().pwa_isobar_destroy(self._h)
            except Exception:
                pass
            self._h = None

    # -- final state and options ---------------------------------------------------
    def setFinalState(self, names, masses, beamMass, species=None, isospins=None):
        """names of the three final-state particles (equal names are identical
        particles unless species says otherwise), their masses and the beam
        mass in GeV/c^2; isospins [(2I, 2I_3, intrinsic parity)] for isospin
        symmetrisation (filled in for pions when not given)."""
        names = list(names)
        if species is None:
            ids = {}
            species = [ids.setdefault(n, len(ids)) for n in names]
        m = np.ascontiguousarray(masses, dtype=np.float64)
        sp = np.ascontiguousarray(species, dtype=np.int32)
        N.call("pwa_isobar_set_final_state", self._h, len(names), m.ctypes.data_as(N.pd),
               sp.ctypes.data_as(C.POINTER(C.c_int32)), float(beamMass))
        self._names = names
        if isospins is None and all(n in PION_ISOSPINS for n in names):
            isospins = [PION_ISOSPINS[n] for n in names]
        if isospins is not None:
            I, I3, P = (np.ascontiguousarray([x[k] for x in isospins], dtype=np.int32) for k in range(3))
            N.call("pwa_isobar_set_isospins", self._h, *(a.ctypes.data_as(C.POINTER(C.c_int32)) for a in (I, I3, P)))

    def enableIsospinSymmetrization(self, flag=True):
        """isobarAmplitude::enableIsospinSymmetrization (isobarAmplitude.h:70);
        off by default here (it needs the final-state isospins)."""
        N.call("pwa_isobar_enable_isospin_symmetrization", self._h, 1 if flag else 0)
        self._isospin = bool(flag)

    def isospinSymmetrization(self):
        return self._isospin

    def _set_opts(self, k, flag):
        o = list(self._opts)
        o[k] = 1 if flag else 0
        N.call("pwa_isobar_set_options", self._h, *o)
        self._opts = o

    def enableReflectivityBasis(self, flag=True):
        self._set_opts(0, flag)

    def enableBoseSymmetrization(self, flag=True):
        self._set_opts(1, flag)

    def enableSpaceInversion(self, flag=True):
        self._set_opts(2, flag)

    def enableReflection(self, flag=True):
        self._set_opts(3, flag)

    def reflectivityBasis(self):
        return bool(self._opts[0])

    def boseSymmetrization(self):
        return bool(self._opts[1])

    def doSpaceInversion(self):
        return bool(self._opts[2])

    def doReflection(self):
        return bool(self._opts[3])

    def setStream(self, stream):
        """run on this CUDA stream (a torch.cuda.Stream, a raw handle or None
        for the default stream); device-buffer calls are then asynchronous."""
        h = getattr(stream, "cuda_stream", stream)
        N.call("pwa_isobar_set_stream", self._h, C.c_void_p(h or 0))
        self._async = True
        self._stream = h or 0

    def setChunkEvents(self, events):
        """host-buffer calls process at most this many events per device pass
        (0: 1 GiB of device buffers)."""
        N.call("pwa_isobar_set_chunk_events", self._h, int(events))

    # -- waves ---------------------------------------------------------------------
    def addWave(self, J, P, M, refl, L, S, isobarJ, isobarL, massDependence="flat", isobarMass=0.0,
                isobarWidth=0.0, isobarDaughters=(0, 1), bachelor=2, bachelorFirst=False, isobarS=0,
                isobarName="isobar", isospin=2, G=-1, C_=+1, isobarIsospin=0, bounds=(0.0, 0.0),
                massDepParams=()):
        """adds one wave (all spins and isospins doubled); returns its index.
        isospin and isobarIsospin (2I of X and of the isobar) enter isospin
        symmetrisation and the wave name; bounds is the isobar mass bin of
        the binned mass dependence, massDepParams the parameters of the K pi
        S-wave forms (KPiSGLASS: a, r, M0, G0, phiF, phiR, phiRsin, F, R,
        MMax; KPiSPalanoPennington: MMax)."""
        md = MASS_DEPENDENCES[massDependence] if isinstance(massDependence, str) else int(massDependence)
        w = N.IsobarWave(J=J, P=P, M=M, refl=refl, L=L, S=S, isobarJ=isobarJ, isobarL=isobarL, isobarS=isobarS,
                         massDependence=md, isobarMass=isobarMass, isobarWidth=isobarWidth,
                         isobarDaughter1=isobarDaughters[0], isobarDaughter2=isobarDaughters[1],
                         bachelor=bachelor, bachelorFirst=1 if bachelorFirst else 0, isospin=isospin,
                         isobarIsospin=isobarIsospin, binLower=float(bounds[0]), binUpper=float(bounds[1]))
        if len(massDepParams) > 10:
            raise ValueError("at most 10 mass-dependence parameters")
        for k, v in enumerate(massDepParams):
            w.massDepParams[k] = float(v)
        N.call("pwa_isobar_add_wave", self._h, C.byref(w))
        self._waves.append(dict(J=J, P=P, M=M, refl=refl, L=L, S=S, isobarJ=isobarJ, isobarL=isobarL,
                                isobarS=isobarS, isobarDaughters=tuple(isobarDaughters), bachelor=bachelor,
                                bachelorFirst=bool(bachelorFirst), isobarName=isobarName, isospin=isospin, G=G,
                                C=C_))
        return len(self._waves) - 1

    def nmbWaves(self):
        n = C.c_uint32()
        N.call("pwa_isobar_nmb_waves", self._h, C.byref(n))
        return n.value

    def nmbSymTerms(self, wave=0):
        """symmetrisation terms (Bose times isospin) of one wave."""
        n = C.c_uint32()
        N.call("pwa_isobar_nmb_sym_terms", self._h, int(wave), C.byref(n))
        return n.value

    def waveName(self, i):
        """wave name in the layout of waveDescription::waveNameFromTopology
        (waveDescription.cc:540-590): [I G,J P C,M refl]=[isobar=[a[L,S]b][L,S]bachelor]
        with parentheses replaced by underscores."""
        w = self._waves[i]
        names = self._names or ["fs0", "fs1", "fs2"]
        a, b = w["isobarDaughters"]
        iso = "%s=[%s[%s,%s]%s]" % (w["isobarName"], names[a], _qn(w["isobarL"]), _qn(w["isobarS"]), names[b])
        d1, d2 = (names[w["bachelor"]], iso) if w["bachelorFirst"] else (iso, names[w["bachelor"]])
        s = "[%s%s,%s%s%s,%s%s]=[%s[%s,%s]%s]" % (_qn(w["isospin"]), _par(w["G"]), _qn(w["J"]), _par(w["P"]),
                                                 _par(w["C"]), _qn(w["M"]), _par(w["refl"]), d1, _qn(w["L"]),
                                                 _qn(w["S"]), d2)
        return s.replace("(", "_").replace(")", "_")

    # -- evaluation ----------------------------------------------------------------
    def amplitudes(self, beam, fs, dtype="complex128"):
        """[wave, event] amplitudes for beam (N, 3) and final-state (3, N, 3)
        lab momenta.  CUDA tensors in, CUDA tensor out.  dtype complex128:
        FP64 throughout; complex64: FP64 frames, FP32 per-wave arithmetic."""
        W = self.nmbWaves()
        if dtype not in ("complex128", "complex64"):
            raise ValueError("dtype must be complex128 or complex64")
        ampType = N.COMPLEX64 if dtype == "complex64" else N.COMPLEX128
        if hasattr(beam, "__cuda_array_interface__"):
            import torch
            if not hasattr(fs, "__cuda_array_interface__"):
                raise ValueError("beam and fs must both be CUDA tensors or both host arrays")
            # the kernel reads N events from every row: the shapes must agree
            # (device buffer sizes cannot be checked behind the C ABI)
            if beam.dim() != 2 or beam.shape[1] != 3 or tuple(fs.shape) != (3, beam.shape[0], 3):
                raise ValueError("beam must be (N, 3) and fs (3, N, 3)")
            b = beam.to(torch.float64).t().contiguous()                  # [3][N]
            f = fs.to(torch.float64).permute(0, 2, 1).contiguous()       # [3][3][N]
            n = b.shape[1]
            out = torch.empty((W, n), dtype=getattr(torch, dtype), device=b.device)
            if self._async and self._stream:
                # the kernel runs on the caller's stream: order it after the
                # layout copies above and keep their memory until it has run
                es = torch.cuda.ExternalStream(self._stream, device=b.device)
                es.wait_stream(torch.cuda.current_stream(b.device))
                for buf in (b, f, out):
                    buf.record_stream(es)
            N.call("pwa_isobar_amplitudes", self._h, C.c_void_p(b.data_ptr()), C.c_void_p(f.data_ptr()), n,
                   C.c_void_p(out.data_ptr()), ampType, N.MEMORY_DEVICE)
            return out
        beam = np.asarray(beam, dtype=np.float64)
        fs = np.asarray(fs, dtype=np.float64)
        if beam.ndim != 2 or beam.shape[1] != 3 or fs.shape != (3, beam.shape[0], 3):
            raise ValueError("beam must be (N, 3) and fs (3, N, 3)")
        b = np.ascontiguousarray(beam.T)
        f = np.ascontiguousarray(np.transpose(fs, (0, 2, 1)))
        n = b.shape[1]
        out = np.empty((W, n), dtype=np.dtype(dtype))
        N.call("pwa_isobar_amplitudes", self._h, b.ctypes.data_as(C.c_void_p), f.ctypes.data_as(C.c_void_p), n,
               out.ctypes.data_as(C.c_void_p), ampType, N.MEMORY_HOST)
        return out


class isobarCanonicalAmplitudes(isobarHelicityAmplitudes):
    """The same wave set in the canonical formalism (isobarCanonicalAmplitude,
    decayAmplitude/isobarCanonicalAmplitude.cc:64-190)."""

    def __init__(self):
        super().__init__()
        N.call("pwa_isobar_set_formalism", self._h, 1)


def _cstrs(names):
    return (C.c_char_p * len(names))(*[n.encode() for n in names])


def writeAmplitudeFileNative(amp, path, beam, fs, waveNames=None, binVars=None):
    """pwa_isobar_write_amp_file: the calcAmplitudes step in native code --
    amplitudes of host momenta beam (N, 3), fs (3, N, 3) computed in slabs and
    streamed into one raw amplitude file with the final-state mass and
    binVars {name: [N]} as binning variables.  Returns the wave names."""
    beam = np.asarray(beam, dtype=np.float64)
    fs = np.asarray(fs, dtype=np.float64)
    if beam.ndim != 2 or beam.shape[1] != 3 or fs.shape != (3, beam.shape[0], 3):
        raise ValueError("beam must be (N, 3) and fs (3, N, 3)")
    n = beam.shape[0]
    names = waveNames or [amp.waveName(k) for k in range(amp.nmbWaves())]
    b = np.ascontiguousarray(beam.T)
    f = np.ascontiguousarray(np.transpose(fs, (0, 2, 1)))
    binVars = binVars or {}
    vn = list(binVars)
    v = np.ascontiguousarray(np.stack([np.asarray(binVars[k], dtype=np.float64) for k in vn])) if vn else None
    N.call("pwa_isobar_write_amp_file", amp._h, str(path).encode(), _cstrs(names), b.ctypes.data_as(C.c_void_p),
           f.ctypes.data_as(C.c_void_p), n, len(vn), _cstrs(vn) if vn else None,
           v.ctypes.data_as(C.c_void_p) if v is not None else None)
    return names


def finalStateMass(ev):
    """invariant mass of the final state of every event of an .evt file
    (readEvtFile), the usual on-the-fly binning variable ("mass")."""
    p = np.sum(ev["fs"], axis=0)
    E = np.sum(np.sqrt(ev["fs_masses"][:, None] ** 2 + np.sum(ev["fs"] ** 2, axis=2)), axis=0)
    return np.sqrt(np.maximum(E * E - np.sum(p * p, axis=1), 0.0))


def calcAmplitudes(amp, evtPath, ampPath, dtype="complex64", binVars=None):
    """The calcAmplitudes step (pyInterface/scripts/calcAmplitudes.py): the
    amplitudes of every wave of `amp` (a wave set whose final state is set)
    for the events of an .evt file, written as one raw amplitude file with the
    final-state mass (and any further binVars {name: [N]}) as binning
    variables, ready for pwaLikelihood.loadAmplitudeFiles.  Returns the wave
    names written."""
    from . import evtfile
    from .ampfile import writeAmplitudeFile
    ev = evtfile.readEvtFile(evtPath)
    A = amp.amplitudes(ev["beam"], ev["fs"], dtype=dtype)
    names = [amp.waveName(k) for k in range(amp.nmbWaves())]
    bv = {"mass": finalStateMass(ev)}
    bv.update(binVars or {})
    writeAmplitudeFile(ampPath, names, A, bv)
    return names


def clebschGordanCoeff(j1, m1, j2, m2, J, M):
    """(j1 m1 j2 m2 | J M), arguments doubled (utilities/spinUtils.hpp:241-330)."""
    v = C.c_double()
    N.call("pwa_clebsch_gordan", j1, m1, j2, m2, J, M, C.byref(v))
    return v.value


def dFunction(j, m, n, theta):
    """Wigner d^j_{m n}(theta), arguments doubled (utilities/dFunction.hpp:52-170)."""
    v = C.c_double()
    N.call("pwa_wigner_d", j, m, n, float(theta), C.byref(v))
    return v.value


def barrierFactor(L, q):
    """Blatt-Weisskopf barrier factor, 2L and breakup momentum q in GeV/c
    (utilities/physUtils.hpp:265-278)."""
    v = C.c_double()
    N.call("pwa_barrier_factor", L, float(q), C.byref(v))
    return v.value
