"""Shared set-up for parity tests: one workload -> oracle and GPU likelihoods
built through the same call sequence as the reference's initLikelihood
(pyInterface/module/_likelihood.py:17-71)."""
import numpy as np

from oracle.oracle import OracleIntegral, OracleLikelihood
from rootpwa_gb300 import synth

# tolerances of the FP32-contraction / FP64-reduction engine against the FP64 oracle
F_RTOL = 1e-6          # relative error of the function value
G_NORMWISE = 1e-6      # max |g - g_ref| / max |g_ref|


def oracle_integrals(w, Integral=OracleIntegral):
    """Normalisation (all MC events) and acceptance (accepted events) integrals
    (Integral: the oracle's class, or the reference's own, oracle.ref.RefIntegral)."""
    mc = w["mc"].astype(np.complex128)
    norm = Integral()
    assert norm.integrate(w["names"], mc)
    acc = Integral()
    assert acc.integrate(w["names"], mc, in_bin=w["accepted"])
    return norm, acc


def build_oracle(w, norm=None, acc=None, use_normalized=True, prior=0, cauchy_width=0.5, thresholds=None,
                 mass_bin_center=0.0, acc_override=0, Likelihood=OracleLikelihood):
    if norm is None:
        norm, acc = oracle_integrals(w)
    L = Likelihood(use_normalized, prior, cauchy_width)
    assert L.init(w["names"], w["refl"], thresholds, w["rank"], mass_bin_center)
    assert L.addNormIntegral(norm)
    assert L.addAccIntegral(acc, acc_override)
    for k, n in enumerate(w["names"]):
        assert L.addAmplitude(n, w["data"][k].astype(np.complex128))
    assert L.finishInit()
    return L


def gpu_integrals(w, precision="fp32"):
    import rootpwa_gb300 as R
    norm = R.ampIntegralMatrix()
    norm.integrate(w["names"], w["mc"], precision=precision)
    acc = R.ampIntegralMatrix()
    acc.integrate(w["names"], w["mc"], inBin=w["accepted"], precision=precision)
    return norm, acc


def integral_pairs(w):
    """(oracle norm, oracle acc, GPU norm, GPU acc) holding identical sums.

    The GPU copies are taken before any likelihood sees the integrals: like
    the reference, addAccIntegral overwrites the acceptance integral's event
    count (pwaLikelihood.cc:1099-1101)."""
    norm, acc = oracle_integrals(w)
    return norm, acc, copy_oracle_integral_to_gpu(norm), copy_oracle_integral_to_gpu(acc)


def copy_oracle_integral_to_gpu(oi):
    """Product integral object holding exactly the oracle's sums."""
    import rootpwa_gb300 as R
    I = R.ampIntegralMatrix()
    I.setWaveNames(oi.wave_names())
    I.setMatrix(oi.raw())
    I.setNmbEvents(oi.nmb_events())
    return I


def build_gpu(w, norm=None, acc=None, use_normalized=True, prior=0, cauchy_width=0.5, thresholds=None,
              mass_bin_center=0.0, acc_override=0, amps=None):
    import rootpwa_gb300 as R
    L = R.pwaLikelihood()
    L.useNormalizedAmps(use_normalized)
    if prior:
        L.setPriorType(prior)
        L.setCauchyWidth(cauchy_width)
    L.init(w["names"], w["refl"], thresholds, w["rank"], mass_bin_center)
    L.addNormIntegral(norm)
    L.addAccIntegral(acc, acc_override)
    data = w["data"] if amps is None else amps
    for k, n in enumerate(w["names"]):
        L.addAmplitude(n, data[k])
    L.finishInit()
    return L


def normwise(g, ref):
    return float(np.max(np.abs(g - ref)) / max(np.max(np.abs(ref)), 1e-300))


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)
