"""Persistent autotuner cache: a handwritten cache file loads, saves back
to the same content and rejects malformed entries (host code only); on the
GPU a likelihood whose shape is in the cache takes the cached plan at
finishInit without timing launches."""
import numpy as np
import pytest

import rootpwa_gb300 as R
from rootpwa_gb300 import _native as N

CACHE = """{"device": "", "fdf_plans": [
{"waves": 15, "negative_waves": 0, "rank": 1, "event_class": 17, "stages": 3, "variant": 1},
{"waves": 87, "negative_waves": 7, "rank": 2, "event_class": 20, "stages": 2, "variant": 2}
]}
"""


def test_cache_round_trip_and_rejects_malformed(tmp_path):
    R.autotune.clear()
    p = tmp_path / "tune.json"
    p.write_text(CACHE)
    R.autotune.load(p)
    assert R.autotune.size() == 2
    q = tmp_path / "again.json"
    R.autotune.save(q)
    body = q.read_text().splitlines()
    assert body[1:] == CACHE.splitlines()[1:]
    bad = tmp_path / "bad.json"
    bad.write_text(CACHE.replace('"stages": 3', '"stages": 9'))
    with pytest.raises(R.PwaError):
        R.autotune.load(bad)
    with pytest.raises(R.PwaError):
        R.autotune.load(tmp_path / "missing.json")
    R.autotune.clear()
    assert R.autotune.size() == 0


@pytest.mark.gpu
def test_cached_plan_skips_timing(tmp_path):
    from rootpwa_gb300 import synth
    import helpers
    w = synth.make_workload("compass88", seed=6, n_data=70_000, n_mc=3000)
    norm, acc = helpers.oracle_integrals(w)

    def build():
        return helpers.build_gpu(w, helpers.copy_oracle_integral_to_gpu(norm),
                                 helpers.copy_oracle_integral_to_gpu(acc))

    R.autotune.clear()
    lib = N.lib()
    n0 = lib.pwa_kernel_launch_count()
    G = build()  # 70,000 events: tuned at finishInit
    tuned_launches = lib.pwa_kernel_launch_count() - n0
    plan = (G.plan(), G.planVariant())
    path = tmp_path / "tune.json"
    R.autotune.save(path)
    R.autotune.clear()
    R.autotune.load(path)
    assert R.autotune.size() >= 1
    n1 = lib.pwa_kernel_launch_count()
    H = build()
    cached_launches = lib.pwa_kernel_launch_count() - n1
    assert (H.plan(), H.planVariant()) == plan
    assert cached_launches < tuned_launches - 20  # no timing runs
    f0, g0 = G.FdF(w["par"])
    f1, g1 = H.FdF(w["par"])
    assert f0 == f1 and np.array_equal(g0, g1)
