"""Generates the golden fixtures in this directory.

1. testIntegral.int -- the reference's own ASCII integral fixture
   (test/decayAmplitude/testIntegral.int of ROOTPWA: 41 waves, 20,000 events,
   raw sums), copied verbatim.  It pins the readAscii/writeAscii format and
   supplies a realistic 41 x 41 Hermitian integral matrix.
2. oracle_<workload>.npz -- FP64 oracle values (integrals, FdF, DoEval,
   Hessian) on seeded synthetic workloads, with a checksum of the generated
   inputs so that a change of the random streams is detected.

Run from the repository root:
    python tests/golden/make_golden.py [path to the reference checkout]
(step 1 needs the reference checkout: the argument, else PWA_REFERENCE_DIR).
"""
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from rootpwa_gb300 import synth  # noqa: E402
import helpers  # noqa: E402

REF_FIXTURE = os.path.join("test", "decayAmplitude", "testIntegral.int")

GOLDEN_WORKLOADS = {
    "compass15_seed0": dict(name="compass15", seed=0),
    "compass88_small_seed1": dict(name="compass88", seed=1, n_data=5003, n_mc=8000),
}


def checksum(w):
    d = w["data"].astype(np.complex128)
    m = w["mc"].astype(np.complex128)
    return np.array([np.sum(np.abs(d) ** 2), np.sum(np.abs(m) ** 2), float(np.sum(w["accepted"])),
                     np.sum(w["par"] ** 2), d[0, 0].real, m[-1, -1].imag])


def make(name, spec):
    w = synth.make_workload(**spec)
    norm, acc = helpers.oracle_integrals(w)
    norm_raw, norm_n = norm.raw(), norm.nmb_events()
    acc_raw, acc_n = acc.raw(), acc.nmb_events()
    L = helpers.build_oracle(w, norm, acc)
    f, g = L.FdF(w["par"])
    out = dict(checksum=checksum(w), norm_raw=norm_raw, norm_n=norm_n, acc_raw=acc_raw, acc_n=acc_n, f=f, grad=g,
               doeval=L.DoEval(w["par"]), tot_acc=L.totAcc())
    if len(w["par"]) <= 64:
        H = L.Hessian(w["par"])
        out["hessian"] = H
    np.savez_compressed(os.path.join(HERE, "oracle_%s.npz" % name), **out)
    print(name, "f =", f)


def main():
    refdir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PWA_REFERENCE_DIR")
    if refdir and os.path.exists(os.path.join(refdir, REF_FIXTURE)):
        shutil.copyfile(os.path.join(refdir, REF_FIXTURE), os.path.join(HERE, "testIntegral.int"))
    for name, spec in GOLDEN_WORKLOADS.items():
        make(name, spec)


if __name__ == "__main__":
    main()
