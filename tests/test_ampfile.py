"""Raw amplitude files (the replacement of the per-wave amplitude trees,
storageFormats/amplitudeTreeLeaf.h:51-118): the native writer against the
numpy reader of the documented layout, the header accessors, and rejection
of files that are not amplitude files or are truncated.  Host code only."""
import numpy as np
import pytest

import rootpwa_gb300 as R


def sample(n=1001, w=5, seed=0):
    rng = np.random.default_rng(seed)
    names = ["1-(1++)0+ rho pi S", "1-(0-+)0+ f0 pi S", "wave_c", "wé", "x" * 300][:w]
    amps = (rng.standard_normal((w, n)) + 1j * rng.standard_normal((w, n))).astype(np.complex64)
    bv = {"mass": rng.uniform(1, 2, n), "tPrime": rng.exponential(0.3, n)}
    return names, amps, bv


def test_write_read_round_trip(tmp_path):
    names, amps, bv = sample()
    p = tmp_path / "a.amp"
    R.writeAmplitudeFile(p, names, amps, bv)
    w, a, v = R.readAmplitudeFile(p)
    assert w == names
    assert np.array_equal(np.asarray(a), amps)
    assert list(v) == list(bv)
    for k in bv:
        assert np.array_equal(np.asarray(v[k]), bv[k])
    wn, n, vn = R.ampFileInfo(p)
    assert (wn, n, vn) == (names, amps.shape[1], list(bv))
    size = p.stat().st_size
    assert size % 4096 == (amps.shape[1] * 8 * (len(names) + len(bv))) % 4096


def test_no_variables_and_empty(tmp_path):
    names, amps, _ = sample(n=7, w=2)
    p = tmp_path / "b.amp"
    R.writeAmplitudeFile(p, names, amps)
    w, a, v = R.readAmplitudeFile(p)
    assert w == names and v == {} and np.array_equal(np.asarray(a), amps)
    q = tmp_path / "e.amp"
    R.writeAmplitudeFile(q, names, np.zeros((2, 0), np.complex64))
    assert R.ampFileInfo(q) == (names, 0, [])


def test_rejects_bad_files(tmp_path):
    names, amps, bv = sample(n=100, w=2)
    p = tmp_path / "c.amp"
    R.writeAmplitudeFile(p, names, amps, bv)
    raw = p.read_bytes()
    t = tmp_path / "trunc.amp"
    t.write_bytes(raw[:-8])
    with pytest.raises(R.PwaError):
        R.ampFileInfo(t)
    m = tmp_path / "magic.amp"
    m.write_bytes(b"X" + raw[1:])
    with pytest.raises(R.PwaError):
        R.ampFileInfo(m)
    with pytest.raises(R.PwaError):
        R.ampFileInfo(tmp_path / "missing.amp")
    with pytest.raises(ValueError):
        R.writeAmplitudeFile(p, names[:1], amps, bv)
