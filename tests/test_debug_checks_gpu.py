"""The debug build (rootpwa_gb300.build.build_debug(): FdF kernels compiled
with -DPWA_DEBUG_CHECKS, every shared-memory load and store of the fused
kernels checked against its region) runs the FdF parity cases of every
kernel variant without a single failed check.  This is the race- and
bounds-checking stand-in for a memory checker: a failed check sets a device
flag that the host turns into an error, and the access is skipped.  It runs
in a child process because the debug library replaces the release one for
the whole process."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import sys
sys.path.insert(0, %(root)r)
sys.path.insert(0, %(tests)r)
import numpy as np
import rootpwa_gb300 as R
from rootpwa_gb300 import _native as N
assert N.LIB_PATH.endswith("libpwa_gb300_debug.so")
from test_fdf_gpu import stress_workload, pair, check_point
shapes = [(0, 15, 1, 20000), (7, 80, 2, 30001), (3, 5, 1, 127), (2, 9, 3, 129), (20, 120, 1, 4099), (10, 54, 4, 3000),
          (5, 0, 2, 1000)]
runs = 0
for n_neg, n_pos, rank, n in shapes:
    w = stress_workload(n_neg, n_pos, rank, n, flat=1.0)
    O, G = pair(w)
    stages = G.plan()[1]
    for ne in (1, 2, 3, 4, 5):
        try:
            G.setPlan(stages, ne)
        except R.PwaError:
            continue
        check_point(O, G, w["par"])
        G.DoEval(w["par"])
        runs += 1
print("debug-checked runs", runs)
assert runs >= 15
'''


def test_debug_build_passes_bounds_checks():
    from rootpwa_gb300 import build as b
    b.build_debug()
    env = dict(os.environ, PWA_GB300_DEBUG="1")
    code = CHILD % dict(root=ROOT, tests=os.path.join(ROOT, "tests"))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "debug-checked runs" in r.stdout
