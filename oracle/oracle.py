"""ctypes wrapper of the FP64 CPU oracle -- TEST INFRASTRUCTURE ONLY.

The oracle (pwa_oracle.cpp in this directory) restates ROOTPWA's
pwaLikelihood (partialWaveFit/pwaLikelihood.cc) and ampIntegralMatrix
(decayAmplitude/ampIntegralMatrix.cc) in plain C++ FP64 with the reference's
compensated summation.  Only the tests, the smoke check and the CPU-baseline
leg of bench.py use it, and only as the checker; the product never does.

Parity status: pinned against the reference itself -- oracle/ref.py drives
the reference's own pwaLikelihood.cc and ampIntegralMatrix.cc (compiled from
their sources by `make -C oracle ref`) through the same class API, and
tests/test_ref_pinned.py checks this restatement against it; also pinned by
the reference's ASCII integral fixture, finite differences and the analytic
identities of the reference's likelihood write-up.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libpwa_oracle.so")
_lib = None


def build(force=False):
    """Compile the oracle shared library with its Makefile."""
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "pwa_oracle.cpp"))):
        subprocess.run(["make", "-C", _HERE, "-s"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        vp, u, ul, d, i = C.c_void_p, C.c_uint, C.c_ulong, C.c_double, C.c_int
        pd = C.POINTER(C.c_double)
        sig = {
            "oracle_int_create": (vp, []),
            "oracle_int_destroy": (None, [vp]),
            "oracle_int_set_wave_names": (i, [vp, u, C.POINTER(C.c_char_p)]),
            "oracle_int_integrate": (i, [vp, u, C.POINTER(C.c_char_p), pd, ul, u, pd, ul, C.c_void_p, C.c_long]),
            "oracle_int_add_event": (i, [vp, pd]),
            "oracle_int_element": (None, [vp, u, u, pd]),
            "oracle_int_raw": (None, [vp, pd]),
            "oracle_int_set_raw": (None, [vp, pd]),
            "oracle_int_nmb_events": (ul, [vp]),
            "oracle_int_set_nmb_events": (None, [vp, ul]),
            "oracle_int_nmb_waves": (u, [vp]),
            "oracle_int_add": (i, [vp, vp]),
            "oracle_int_read_ascii": (i, [vp, C.c_char_p]),
            "oracle_int_write_ascii": (i, [vp, C.c_char_p]),
            "oracle_int_wave_name": (i, [vp, u, C.c_char_p, u]),
            "oracle_lik_create": (vp, []),
            "oracle_lik_destroy": (None, [vp]),
            "oracle_lik_set_options": (None, [vp, i, i, d]),
            "oracle_lik_set_shard": (None, [vp, ul, i]),
            "oracle_lik_set_otf_binning": (i, [vp, u, pd, pd, C.POINTER(C.c_void_p), ul]),
            "oracle_lik_otf_selected": (ul, [vp]),
            "oracle_lik_init": (i, [vp, u, C.POINTER(C.c_char_p), C.POINTER(C.c_int), pd, u, d]),
            "oracle_lik_add_norm_integral": (i, [vp, vp]),
            "oracle_lik_add_acc_integral": (i, [vp, vp, ul]),
            "oracle_lik_add_amplitude": (i, [vp, C.c_char_p, pd, ul]),
            "oracle_lik_finish_init": (i, [vp]),
            "oracle_lik_nmb_pars": (u, [vp]),
            "oracle_lik_nmb_pars_fixed": (u, [vp]),
            "oracle_lik_par_fixed": (i, [vp, u]),
            "oracle_lik_par_name": (i, [vp, u, C.c_char_p, u]),
            "oracle_lik_tot_acc": (d, [vp]),
            "oracle_lik_fdf": (None, [vp, pd, pd, pd, u]),
            "oracle_lik_doeval": (d, [vp, pd, u]),
            "oracle_lik_gradient": (None, [vp, pd, pd, u]),
            "oracle_lik_hessian": (None, [vp, pd, pd]),
            "oracle_lik_covariance": (i, [vp, pd, pd]),
            "oracle_lik_correct_param_signs": (None, [vp, pd, pd]),
            "oracle_lik_integral_matrices": (None, [vp, pd, pd, pd, i]),
            "oracle_lik_nmb_waves": (u, [vp, i]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _pd(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _names(names):
    arr = (C.c_char_p * len(names))()
    arr[:] = [n.encode() for n in names]
    return arr


class OracleIntegral:
    """ampIntegralMatrix restatement (decayAmplitude/ampIntegralMatrix.h:67-173)."""

    _lib = staticmethod(lib)

    def __init__(self):
        self._h = self._lib().oracle_int_create()

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib().oracle_int_destroy(self._h)
            self._h = None

    def integrate(self, names, amps, weights=None, in_bin=None, max_nmb_events=0):
        """amps: complex array [wave][event] or [wave][event][sub]."""
        a = np.asarray(amps)
        if a.ndim == 2:
            a = a[:, :, None]
        nw, ne, ns = a.shape
        a = np.ascontiguousarray(a.astype(np.complex128)).view(np.float64)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        b = None if in_bin is None else np.ascontiguousarray(in_bin, dtype=np.uint8)
        ok = self._lib().oracle_int_integrate(self._h, nw, _names(names), _pd(a), ne, ns,
                                        None if w is None else _pd(w), 0 if w is None else len(w),
                                        None if b is None else b.ctypes.data, int(max_nmb_events))
        return bool(ok)

    def set_wave_names(self, names):
        return bool(self._lib().oracle_int_set_wave_names(self._h, len(names), _names(names)))

    def add_event(self, amps):
        a = np.ascontiguousarray(np.asarray(amps, dtype=np.complex128)).view(np.float64)
        return bool(self._lib().oracle_int_add_event(self._h, _pd(a)))

    def nmb_waves(self):
        return self._lib().oracle_int_nmb_waves(self._h)

    def nmb_events(self):
        return self._lib().oracle_int_nmb_events(self._h)

    def set_nmb_events(self, n):
        self._lib().oracle_int_set_nmb_events(self._h, int(n))

    def element(self, i, j):
        out = np.zeros(2)
        self._lib().oracle_int_element(self._h, i, j, _pd(out))
        return complex(out[0], out[1])

    def raw(self):
        n = self.nmb_waves()
        out = np.zeros(2 * n * n)
        self._lib().oracle_int_raw(self._h, _pd(out))
        return out.view(np.complex128).reshape(n, n)

    def set_raw(self, m):
        m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128)).view(np.float64)
        self._lib().oracle_int_set_raw(self._h, _pd(m))

    def matrix(self):
        return self.raw() / float(self.nmb_events())

    def wave_names(self):
        buf = C.create_string_buffer(4096)
        out = []
        for i in range(self.nmb_waves()):
            self._lib().oracle_int_wave_name(self._h, i, buf, 4096)
            out.append(buf.value.decode())
        return out

    def __iadd__(self, other):
        if not self._lib().oracle_int_add(self._h, other._h):
            raise ValueError("integral matrices have different wave sets")
        return self

    def read_ascii(self, path):
        return bool(self._lib().oracle_int_read_ascii(self._h, path.encode()))

    def write_ascii(self, path):
        return bool(self._lib().oracle_int_write_ascii(self._h, path.encode()))


class OracleLikelihood:
    """pwaLikelihood<complex<double>> restatement (partialWaveFit/pwaLikelihood.h:66-320)."""

    _lib = staticmethod(lib)

    def __init__(self, use_normalized_amps=True, prior=0, cauchy_width=0.5):
        self._h = self._lib().oracle_lik_create()
        self._lib().oracle_lik_set_options(self._h, int(use_normalized_amps), int(prior), float(cauchy_width))

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib().oracle_lik_destroy(self._h)
            self._h = None

    def set_shard(self, total_events, root):
        self._lib().oracle_lik_set_shard(self._h, int(total_events), 1 if root else 0)

    def setOnTheFlyBinning(self, boundaries, bin_vars):
        """pwaLikelihood::setOnTheFlyBinning (pwaLikelihood.cc:1391-1440)."""
        names = list(boundaries)
        lo = np.array([boundaries[k][0] for k in names], dtype=np.float64)
        hi = np.array([boundaries[k][1] for k in names], dtype=np.float64)
        cols = [np.ascontiguousarray(bin_vars[k], dtype=np.float64) for k in names]
        n = len(cols[0]) if cols else 0
        ptrs = (C.c_void_p * max(1, len(cols)))(*[c.ctypes.data for c in cols])
        return bool(self._lib().oracle_lik_set_otf_binning(self._h, len(names), _pd(lo), _pd(hi), ptrs, n))

    def otfSelected(self):
        return int(self._lib().oracle_lik_otf_selected(self._h))

    def init(self, names, refl, thresholds=None, rank=1, mass_bin_center=0.0):
        r = (C.c_int * len(names))(*[int(x) for x in refl])
        th = np.zeros(len(names)) if thresholds is None else np.ascontiguousarray(thresholds, dtype=np.float64)
        return bool(self._lib().oracle_lik_init(self._h, len(names), _names(names), r, _pd(th), rank,
                                          float(mass_bin_center)))

    def addNormIntegral(self, integral):
        return bool(self._lib().oracle_lik_add_norm_integral(self._h, integral._h))

    def addAccIntegral(self, integral, acc_events_override=0):
        return bool(self._lib().oracle_lik_add_acc_integral(self._h, integral._h, int(acc_events_override)))

    def addAmplitude(self, name, amps):
        a = np.ascontiguousarray(np.asarray(amps, dtype=np.complex128)).view(np.float64)
        return bool(self._lib().oracle_lik_add_amplitude(self._h, name.encode(), _pd(a), len(amps)))

    def finishInit(self):
        return bool(self._lib().oracle_lik_finish_init(self._h))

    def nmbPars(self):
        return self._lib().oracle_lik_nmb_pars(self._h)

    def nmbParsFixed(self):
        return self._lib().oracle_lik_nmb_pars_fixed(self._h)

    def parFixed(self, i):
        return bool(self._lib().oracle_lik_par_fixed(self._h, i))

    def parName(self, i):
        buf = C.create_string_buffer(4096)
        self._lib().oracle_lik_par_name(self._h, i, buf, 4096)
        return buf.value.decode()

    def totAcc(self):
        return self._lib().oracle_lik_tot_acc(self._h)

    def FdF(self, par, threads=1):
        p = np.ascontiguousarray(par, dtype=np.float64)
        f = np.zeros(1)
        g = np.zeros(self.nmbPars())
        self._lib().oracle_lik_fdf(self._h, _pd(p), _pd(f), _pd(g), threads)
        return float(f[0]), g

    def DoEval(self, par, threads=1):
        p = np.ascontiguousarray(par, dtype=np.float64)
        return self._lib().oracle_lik_doeval(self._h, _pd(p), threads)

    def Gradient(self, par, threads=1):
        p = np.ascontiguousarray(par, dtype=np.float64)
        g = np.zeros(self.nmbPars())
        self._lib().oracle_lik_gradient(self._h, _pd(p), _pd(g), threads)
        return g

    def Hessian(self, par):
        p = np.ascontiguousarray(par, dtype=np.float64)
        n = self.nmbPars()
        H = np.zeros((n, n))
        self._lib().oracle_lik_hessian(self._h, _pd(p), _pd(H))
        return H

    def CovarianceMatrix(self, H):
        H = np.ascontiguousarray(H, dtype=np.float64)
        n = self.nmbPars()
        Cm = np.zeros((n, n))
        if not self._lib().oracle_lik_covariance(self._h, _pd(H), _pd(Cm)):
            raise ValueError("singular Hessian")
        return Cm

    def CorrectParamSigns(self, par):
        p = np.ascontiguousarray(par, dtype=np.float64)
        out = np.zeros_like(p)
        self._lib().oracle_lik_correct_param_signs(self._h, _pd(p), _pd(out))
        return out

    def nmbWaves(self, refl=0):
        return self._lib().oracle_lik_nmb_waves(self._h, int(refl))

    def integralMatrices(self, with_flat=False):
        """(norm, acc, phaseSpace) in likelihood wave order (pwaLikelihood.cc:1577-1618)."""
        sz = self.nmbWaves(0) + (1 if with_flat else 0)
        n = np.zeros(2 * sz * sz)
        a = np.zeros(2 * sz * sz)
        ps = np.zeros(sz)
        self._lib().oracle_lik_integral_matrices(self._h, _pd(n), _pd(a), _pd(ps), int(with_flat))
        return n.view(np.complex128).reshape(sz, sz), a.view(np.complex128).reshape(sz, sz), ps
