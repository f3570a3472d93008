"""Generates tests/golden/isobar3pi_oracle.npz: FP64 oracle amplitudes
(oracle/isobar_oracle.py) of the test wave sets of tests/isobar_cases.py on
seeded synthetic events -- pi- pi+ pi- with the default options and in the
canonical formalism, pi- pi0 pi0 with isospin symmetrisation -- together with
the event momenta, so that the fixture pins the oracle against later changes
and the GPU tests can check the kernel without running the oracle.

Run from the repository root:  python tests/golden/make_isobar_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import isobar_oracle as O  # noqa: E402
from isobar_cases import (NEUTRAL_ISOSPIN, NEUTRAL_SPECIES, SPECIES, events, neutral_events,  # noqa: E402
                          neutral_waves, waves)

N_EVENTS = 200


def compute():
    beam, fs, masses, mb = events(N_EVENTS, seed=101)
    W = [w for w, _ in waves()]
    nbeam, nfs, nmasses, nmb = neutral_events(N_EVENTS, seed=102)
    NW = [w for w, _ in neutral_waves()]
    return dict(
        beam=beam, fs=fs, masses=masses, beam_mass=mb,
        helicity=O.amplitudes(W, beam, fs, masses, mb, SPECIES),
        canonical=O.amplitudes(W, beam, fs, masses, mb, SPECIES, formalism="canonical"),
        neutral_beam=nbeam, neutral_fs=nfs, neutral_masses=nmasses, neutral_beam_mass=nmb,
        neutral_isospin=O.amplitudes(NW, nbeam, nfs, nmasses, nmb, NEUTRAL_SPECIES, isospin=NEUTRAL_ISOSPIN),
    )


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "isobar3pi_oracle.npz"), **compute())
    print("wrote isobar3pi_oracle.npz")
