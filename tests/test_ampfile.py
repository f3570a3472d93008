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


def test_duplicate_names_rejected_and_nothing_written(tmp_path):
    """Waves and binning variables are looked up by name: a repeated wave or
    variable name is refused before anything is written."""
    names, amps, bv = sample(n=50, w=3)
    p = tmp_path / "d.amp"
    with pytest.raises(R.PwaError) as e:
        R.writeAmplitudeFile(p, [names[0], names[1], names[0]], amps, bv)
    assert e.value.status == 1 and "duplicate" in str(e.value)
    assert not p.exists() and not (tmp_path / "d.amp.tmp").exists()
    # one name may be a wave and a variable at once (separate tables)
    R.writeAmplitudeFile(p, ["mass", names[1], names[2]], amps, bv)
    assert R.ampFileInfo(p)[0][0] == "mass"


def test_failed_write_leaves_no_file(tmp_path):
    """A write that fails part-way (here: the process's file-size limit) leaves
    neither the file nor its temporary behind; an existing file of that name
    is kept until a write succeeds."""
    import subprocess
    import sys
    import textwrap
    p = tmp_path / "big.amp"
    code = textwrap.dedent("""
        import resource, signal, sys
        import numpy as np
        sys.path.insert(0, %r)
        import rootpwa_gb300 as R
        signal.signal(signal.SIGXFSZ, signal.SIG_IGN)
        resource.setrlimit(resource.RLIMIT_FSIZE, (65536, 65536))
        amps = np.ones((4, 100000), np.complex64)
        try:
            R.writeAmplitudeFile(%r, ["a", "b", "c", "d"], amps)
        except R.PwaError as e:
            print("status", e.status)
    """) % (str(__import__("pathlib").Path(__file__).resolve().parents[1]), str(p))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert "status 6" in r.stdout, r.stdout + r.stderr
    assert not p.exists() and not (tmp_path / "big.amp.tmp").exists()
    names, amps, bv = sample(n=20, w=2)
    R.writeAmplitudeFile(p, names, amps, bv)
    before = p.read_bytes()
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert "status 6" in r.stdout, r.stdout + r.stderr
    assert p.read_bytes() == before and not (tmp_path / "big.amp.tmp").exists()
