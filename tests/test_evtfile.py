"""The reference's ASCII .evt event format (decayAmplitude/evtTreeHelper.cc:
350-440): write and read back seeded three-pion events, read a hand-written
file, and refuse malformed ones."""
import numpy as np
import pytest

from rootpwa_gb300 import evtfile, synth


def test_round_trip(tmp_path):
    beam, fs, masses, mb = synth.three_pion_events(200, seed=4)
    p = tmp_path / "ev.evt"
    evtfile.writeEvtFile(p, 9, beam, [9, 8, 9], fs)
    ev = evtfile.readEvtFile(p)
    assert np.array_equal(ev["beam"], beam) and np.array_equal(ev["fs"], fs)   # %.17g round-trips FP64
    assert ev["fs_names"] == ["pi-", "pi+", "pi-"] and ev["beam_name"] == "pi-"
    assert np.allclose(ev["fs_masses"], masses) and ev["beam_mass"] == pytest.approx(mb)
    assert ev["fs_charges"] == [-1, +1, -1]


def test_hand_written_file(tmp_path):
    text = ("4\n9 -1 0.1 0.0 190.0 190.00008\n9 -1 0.2 -0.1 31.0 31.0011\n"
            "8 1 0.0 0.1 4.0 4.0037\n9 -1 -0.1 -0.1 6.0 6.0029\n") * 3
    p = tmp_path / "hand.evt"
    p.write_text(text)
    ev = evtfile.readEvtFile(p)
    assert ev["beam"].shape == (3, 3) and ev["fs"].shape == (3, 3, 3)
    assert ev["fs"][1, 2].tolist() == [0.0, 0.1, 4.0]
    assert ev["beam"][0].tolist() == [0.1, 0.0, 190.0]


@pytest.mark.parametrize("text,why", [
    ("4\n9 -1 0 0 190 190\n9 -1 0 0 1 1\n8 1 0 0 1 1\n", "truncated"),
    ("3\n9 -1 0 0 190 190\n9 -1 0 0 1 1\n8 1 0 0 1 1\n"
     "3\n9 -1 0 0 190 190\n8 1 0 0 1 1\n9 -1 0 0 1 1\n", "different particles"),
    ("3\n9 1 0 0 190 190\n9 -1 0 0 1 1\n8 1 0 0 1 1\n", "charge"),
    ("3\n9 -1 0 0 190 190\n99 0 0 0 1 1\n8 1 0 0 1 1\n", "unknown"),
])
def test_malformed_files_are_refused(tmp_path, text, why):
    p = tmp_path / "bad.evt"
    p.write_text(text)
    with pytest.raises(ValueError, match=why):
        evtfile.readEvtFile(p)


def test_large_file_is_read_quickly(tmp_path):
    import time
    beam, fs, masses, mb = synth.three_pion_events(100_000, seed=5)
    p = tmp_path / "big.evt"
    evtfile.writeEvtFile(p, 9, beam, [9, 8, 9], fs)
    t = time.perf_counter()
    ev = evtfile.readEvtFile(p)
    assert time.perf_counter() - t < 10.0
    assert np.array_equal(ev["fs"], fs)


def test_non_numeric_content_is_refused(tmp_path):
    p = tmp_path / "text.evt"
    p.write_text("4\n9 -1 0.1 0 190 190\nfoo\n")
    with pytest.raises(ValueError):
        evtfile.readEvtFile(p)
