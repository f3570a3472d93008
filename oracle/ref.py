"""ctypes wrapper of the reference's own likelihood and integral code --
TEST INFRASTRUCTURE ONLY.

`make -C oracle ref` compiles ROOTPWA's partialWaveFit/pwaLikelihood.cc and
decayAmplitude/ampIntegralMatrix.cc unmodified, from the reference source
tree, against the shims in oracle/ref_shim (Boost multi_array / tuple /
accumulator framework, ROOT stand-ins, in-memory amplitude and event trees),
plus the C-ABI driver ref_driver.cpp, into oracle/_ref/libpwa_ref.so.  The
arithmetic that runs -- event loops, Kahan sums (the reference's own
compensatedSumAccumulator), parameter layout, normalisation, Hessian -- is the
reference's; only CovarianceMatrix's inverse and HessianEigenVectors'
eigen-decomposition go through the shim's own linear algebra (ROOT's TMatrixT
is absent).

RefIntegral / RefLikelihood have the API of OracleIntegral /
OracleLikelihood, so a test can run the same steps through both.  The
library builds only where the reference sources are present; available()
says whether it is there.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from . import oracle as O

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_ref", "libpwa_ref.so")
REFERENCE = os.environ.get("PWA_REFERENCE_DIR", "/root/reference")
_lib = None


def buildable():
    return os.path.exists(os.path.join(REFERENCE, "partialWaveFit", "pwaLikelihood.cc"))


def build(force=False):
    """Compile the reference library with the oracle Makefile's `ref` target
    (only where the reference source tree is present)."""
    if not buildable():
        return None
    cmd = ["make", "-C", _HERE, "-s", "ref", "REFERENCE=" + REFERENCE]
    if force:
        cmd.insert(3, "-B")
    subprocess.run(cmd, check=True)
    return _LIB_PATH


def available():
    if os.path.exists(_LIB_PATH):
        return True
    try:
        return build() is not None
    except subprocess.CalledProcessError:
        return False


class _Prefixed:
    """the reference library under the oracle's entry-point names"""

    def __init__(self, L):
        self._L = L

    def __getattr__(self, name):
        return getattr(self._L, name.replace("oracle_", "ref_", 1))


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("reference library not built: the reference sources are not present")
        L = C.CDLL(_LIB_PATH)
        vp, u, ul, d, i = C.c_void_p, C.c_uint, C.c_ulong, C.c_double, C.c_int
        pd = C.POINTER(C.c_double)
        sig = {
            "ref_int_create": (vp, []),
            "ref_int_destroy": (None, [vp]),
            "ref_int_set_wave_names": (i, [vp, u, C.POINTER(C.c_char_p)]),
            "ref_int_integrate": (i, [vp, u, C.POINTER(C.c_char_p), pd, ul, u, pd, ul, C.c_void_p, C.c_long]),
            "ref_int_add_event": (i, [vp, pd]),
            "ref_int_element": (None, [vp, u, u, pd]),
            "ref_int_raw": (None, [vp, pd]),
            "ref_int_set_raw": (None, [vp, pd]),
            "ref_int_nmb_events": (ul, [vp]),
            "ref_int_set_nmb_events": (None, [vp, ul]),
            "ref_int_nmb_waves": (u, [vp]),
            "ref_int_add": (i, [vp, vp]),
            "ref_int_read_ascii": (i, [vp, C.c_char_p]),
            "ref_int_write_ascii": (i, [vp, C.c_char_p]),
            "ref_int_wave_name": (i, [vp, u, C.c_char_p, u]),
            "ref_lik_create": (vp, []),
            "ref_lik_destroy": (None, [vp]),
            "ref_lik_set_options": (None, [vp, i, i, d]),
            "ref_lik_set_otf_binning": (i, [vp, u, pd, pd, C.POINTER(C.c_void_p), ul, C.POINTER(C.c_char_p)]),
            "ref_lik_otf_selected": (ul, [vp]),
            "ref_lik_init": (i, [vp, u, C.POINTER(C.c_char_p), C.POINTER(C.c_int), pd, u, d]),
            "ref_lik_add_norm_integral": (i, [vp, vp]),
            "ref_lik_add_acc_integral": (i, [vp, vp, ul]),
            "ref_lik_add_amplitude": (i, [vp, C.c_char_p, pd, ul]),
            "ref_lik_finish_init": (i, [vp]),
            "ref_lik_nmb_pars": (u, [vp]),
            "ref_lik_nmb_pars_fixed": (u, [vp]),
            "ref_lik_par_fixed": (i, [vp, u]),
            "ref_lik_par_name": (i, [vp, u, C.c_char_p, u]),
            "ref_lik_nmb_waves": (u, [vp, i]),
            "ref_lik_nmb_events": (u, [vp]),
            "ref_lik_fdf": (None, [vp, pd, pd, pd, u]),
            "ref_lik_doeval": (d, [vp, pd, u]),
            "ref_lik_gradient": (None, [vp, pd, pd, u]),
            "ref_lik_doderivative": (d, [vp, pd, u]),
            "ref_lik_dlcache": (d, [vp, u]),
            "ref_lik_hessian": (None, [vp, pd, pd]),
            "ref_lik_covariance": (i, [vp, pd, pd]),
            "ref_lik_correct_param_signs": (None, [vp, pd, pd]),
            "ref_lik_integral_matrices": (None, [vp, pd, pd, pd, i]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = _Prefixed(L)
    return _lib


class RefIntegral(O.OracleIntegral):
    """the reference's ampIntegralMatrix (decayAmplitude/ampIntegralMatrix.cc)"""

    _lib = staticmethod(lib)


class RefLikelihood(O.OracleLikelihood):
    """the reference's pwaLikelihood<complex<double>> (partialWaveFit/pwaLikelihood.cc)"""

    _lib = staticmethod(lib)

    def setOnTheFlyBinning(self, boundaries, bin_vars):
        """pwaLikelihood::setOnTheFlyBinning over one event file (pwaLikelihood.cc:1391-1440)."""
        names = list(boundaries)
        lo = np.array([boundaries[k][0] for k in names], dtype=np.float64)
        hi = np.array([boundaries[k][1] for k in names], dtype=np.float64)
        cols = [np.ascontiguousarray(bin_vars[k], dtype=np.float64) for k in names]
        self._otf_cols = cols
        n = len(cols[0]) if cols else 0
        ptrs = (C.c_void_p * max(1, len(cols)))(*[c.ctypes.data for c in cols])
        return bool(self._lib().oracle_lik_set_otf_binning(self._h, len(names), O._pd(lo), O._pd(hi), ptrs, n,
                                                           O._names(names)))

    def nmbEvents(self):
        return int(self._lib().oracle_lik_nmb_events(self._h))

    def DoDerivative(self, par, i):
        p = np.ascontiguousarray(par, dtype=np.float64)
        return self._lib().oracle_lik_doderivative(self._h, O._pd(p), int(i))

    def dLcache(self, i):
        return self._lib().oracle_lik_dlcache(self._h, int(i))

    def totAcc(self):
        raise NotImplementedError("the reference keeps the total acceptance private")
