"""Generates the reference-made golden fixtures ref_<workload>.npz.

The values come from the reference's own pwaLikelihood and
ampIntegralMatrix code, compiled from its sources by `make -C oracle ref`
(oracle/ref.py): the integrals' raw sums and event counts, FdF value and
gradient, DoEval and, for small parameter counts, the Hessian, on seeded
synthetic workloads, with a checksum of the generated inputs so that a change
of the random streams is detected.  GPU tests compare the product with these
numbers on machines where the reference sources are absent.

Run from the repository root:
    python tests/golden/make_ref_golden.py [path to the reference checkout]
(or set PWA_REFERENCE_DIR).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from rootpwa_gb300 import synth  # noqa: E402

GOLDEN_WORKLOADS = {
    # the single-bin config at its full size: 20,000 data and 100,000 MC events, 15 waves, rank 1
    "compass15_seed0": dict(name="compass15", seed=0),
    # the production shape (7 + 80 waves, rank 2, 341 parameters) on few events
    "compass88_small_seed1": dict(name="compass88", seed=1, n_data=5003, n_mc=8000),
}


def checksum(w):
    d = w["data"].astype(np.complex128)
    m = w["mc"].astype(np.complex128)
    return np.array([np.sum(np.abs(d) ** 2), np.sum(np.abs(m) ** 2), float(np.sum(w["accepted"])),
                     np.sum(w["par"] ** 2), d[0, 0].real, m[-1, -1].imag])


def make(name, spec):
    from oracle import ref
    import helpers
    w = synth.make_workload(**spec)
    norm, acc = helpers.oracle_integrals(w, ref.RefIntegral)
    norm_raw, norm_n = norm.raw(), norm.nmb_events()
    acc_raw, acc_n = acc.raw(), acc.nmb_events()
    L = helpers.build_oracle(w, norm, acc, Likelihood=ref.RefLikelihood)
    f, g = L.FdF(w["par"])
    out = dict(checksum=checksum(w), norm_raw=norm_raw, norm_n=norm_n, acc_raw=acc_raw, acc_n=acc_n, f=f, grad=g,
               doeval=L.DoEval(w["par"]))
    if len(w["par"]) <= 64:
        out["hessian"] = L.Hessian(w["par"])
    np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % name), **out)
    print(name, "f =", f)


def main():
    if len(sys.argv) > 1:
        os.environ["PWA_REFERENCE_DIR"] = sys.argv[1]
    from oracle import ref
    if not ref.available():
        sys.exit("reference sources not found (pass the checkout path or set PWA_REFERENCE_DIR)")
    for name, spec in GOLDEN_WORKLOADS.items():
        make(name, spec)


if __name__ == "__main__":
    main()
