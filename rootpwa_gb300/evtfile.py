"""Event files in the reference's ASCII .evt format, the input of the
decay-amplitude step.

Layout (decayAmplitude/evtTreeHelper.cc:350-440,
pyInterface/scripts/convertEvtToTree.py:8-30): per event one line with the
number of particles n, one line for the beam and n - 1 lines for the
final-state particles, each ``geantId charge px py pz E`` (GeV).  The reader
keeps the momenta; energies follow from the particle masses when the
amplitudes are computed, as in particle::setMomentum.  All events must list
the same particles in the same order (the reference reorders them to a
common order first, convertEvtToTree.py:39-55).

    ev = readEvtFile("events.evt")
    amp.setFinalState(ev["fs_names"], ev["fs_masses"], ev["beam_mass"])
    A = amp.amplitudes(ev["beam"], ev["fs"])
"""
import re

import numpy as np

# GEANT3 particle codes: name, charge, mass (GeV/c^2, PDG)
GEANT_PARTICLES = {
    1: ("gamma", 0, 0.0), 2: ("e+", +1, 0.00051099895), 3: ("e-", -1, 0.00051099895),
    5: ("mu+", +1, 0.1056583755), 6: ("mu-", -1, 0.1056583755), 7: ("pi0", 0, 0.1349768),
    8: ("pi+", +1, 0.13957039), 9: ("pi-", -1, 0.13957039), 10: ("K0_L", 0, 0.497611),
    11: ("K+", +1, 0.493677), 12: ("K-", -1, 0.493677), 13: ("n", 0, 0.93956542052),
    14: ("p+", +1, 0.93827208816), 15: ("pbar-", -1, 0.93827208816), 16: ("K0_S", 0, 0.497611),
    17: ("eta", 0, 0.547862),
}


# anything but numbers and whitespace: let the slow path raise a clear error
_BAD = re.compile(r"[^0-9eE+\-.\s]")


def _particle(gid):
    if gid not in GEANT_PARTICLES:
        raise ValueError("unknown GEANT particle code %d" % gid)
    return GEANT_PARTICLES[gid]


def readEvtFile(path):
    """Reads an .evt file.  Returns a dict with beam (N, 3) and fs (n_fs, N, 3)
    momenta, the GEANT codes, names, charges and masses of the beam and the
    final-state particles."""
    with open(path) as f:
        text = f.read()
    # numbers straight into one float array (a token list would cost ~60
    # bytes per number: gigabytes for millions of events)
    values = np.array(text.split(), dtype=np.float64) if _BAD.search(text) else \
        np.fromstring(text, dtype=np.float64, sep=" ")
    if values.size == 0:
        raise ValueError("%s: no events" % path)
    n = int(values[0])
    if n < 2 or n != values[0]:
        raise ValueError("%s: an event needs a beam and at least one final-state particle" % path)
    width = 1 + 6 * n
    if values.size % width:
        raise ValueError("%s: truncated file or events with different particle counts" % path)
    rows = values.reshape(-1, width)
    if np.any(rows[:, 0] != n):
        raise ValueError("%s: events with different particle counts" % path)
    parts = rows[:, 1:].reshape(rows.shape[0], n, 6)
    ids = parts[:, :, 0].astype(np.int64)
    charges = parts[:, :, 1].astype(np.int64)
    if np.any(ids != ids[0]) or np.any(charges != charges[0]):
        raise ValueError("%s: events list different particles (reorder them to one common order)" % path)
    info = [_particle(int(g)) for g in ids[0]]
    for (name, q, _), qf in zip(info, charges[0]):
        if q != qf:
            raise ValueError("%s: charge %d of %s does not match its GEANT code" % (path, qf, name))
    return {
        "beam": np.ascontiguousarray(parts[:, 0, 2:5]),
        "fs": np.ascontiguousarray(np.transpose(parts[:, 1:, 2:5], (1, 0, 2))),
        "beam_id": int(ids[0, 0]), "fs_ids": [int(g) for g in ids[0, 1:]],
        "beam_name": info[0][0], "fs_names": [x[0] for x in info[1:]],
        "beam_mass": info[0][2], "fs_masses": np.array([x[2] for x in info[1:]]),
        "fs_charges": [x[1] for x in info[1:]],
    }


def writeEvtFile(path, beam_id, beam, fs_ids, fs):
    """Writes beam (N, 3) and final-state (n_fs, N, 3) momenta as an .evt
    file, energies from the particles' masses, 17 significant digits."""
    beam = np.asarray(beam, dtype=np.float64)
    fs = np.asarray(fs, dtype=np.float64)
    ids = [int(beam_id)] + [int(g) for g in fs_ids]
    if fs.shape[0] != len(ids) - 1 or fs.shape[1] != beam.shape[0]:
        raise ValueError("beam must be (N, 3) and fs (n_fs, N, 3) with n_fs = len(fs_ids)")
    info = [_particle(g) for g in ids]
    mom = np.concatenate([beam[None], fs], axis=0)                         # (n, N, 3)
    mass = np.array([x[2] for x in info])[:, None]
    E = np.sqrt(mass ** 2 + np.sum(mom ** 2, axis=2))                      # (n, N)
    n = len(ids)
    with open(path, "w") as f:
        for e in range(beam.shape[0]):
            f.write("%d\n" % n)
            for k in range(n):
                f.write("%d %d %.17g %.17g %.17g %.17g\n" % (ids[k], info[k][1], mom[k, e, 0], mom[k, e, 1],
                                                             mom[k, e, 2], E[k, e]))
