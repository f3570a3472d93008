"""Batched multibin x multistart fits over the C ABI (pwa_multibin_*).

A multibin batch holds several kinematic bins (each a finished
pwaLikelihood with the same wave set, rank 1, one reflectivity) and a number
of start points per bin.  Every (bin, start) pair is one problem with its own
parameter vector in the pwaLikelihood layout.  The batch evaluates the FdF of
all problems in one sweep (each amplitude tile is read once for a group of
start points) and fits all of them with an L-BFGS that runs on the GPU,
optionally replayed from a CUDA graph.  The reference fits one bin per
process (pwaFit.py:18,51-57) and its start points one after another
(_fit.py:131-165); there is no reference counterpart of the batch itself.
"""
import ctypes as C

import numpy as np

from . import _native as N

STATUS = {0: "active", 1: "searching", 2: "converged", 3: "max_iter", 4: "stalled", 5: "failed", 6: "floor"}


def _pd(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class pwaMultibin:
    """Batch of bins x start points (see module docstring)."""

    def __init__(self):
        h = C.c_void_p()
        N.call("pwa_multibin_create", C.byref(h))
        self._h = h
        self._keep = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and N._lib is not None:
            N.lib().pwa_multibin_destroy(h)
            self._h = None

    def addBin(self, likelihood, nStarts):
        """Adds a finished pwaLikelihood with nStarts start points (the batch
        keeps the likelihood alive)."""
        N.call("pwa_multibin_add_bin", self._h, likelihood._h, int(nStarts))
        self._keep.append(likelihood)

    def setOptions(self, startGroup=32, lbfgsMemory=8, gtolAbs=0.0, gtolRel=1e-6, maxIter=5000):
        N.call("pwa_multibin_set_options", self._h, int(startGroup), int(lbfgsMemory), float(gtolAbs),
               float(gtolRel), int(maxIter))

    def setFloorWindow(self, iterations):
        """Stop a problem whose gradient norm has not improved by 1% for this
        many iterations (status 'floor'; 0 disables)."""
        N.call("pwa_multibin_set_floor_window", self._h, int(iterations))

    def setChunks(self, tiles):
        arr = (C.c_uint32 * 3)(*[int(t) for t in tiles])
        N.call("pwa_multibin_set_chunks", self._h, arr)

    def chunks(self):
        arr = (C.c_uint32 * 3)()
        N.call("pwa_multibin_chunks", self._h, arr)
        return list(arr)

    def nmbProblems(self):
        q = C.c_uint32()
        N.call("pwa_multibin_nmb_problems", self._h, C.byref(q))
        return q.value

    def nmbPars(self):
        p = C.c_uint32()
        N.call("pwa_multibin_nmb_pars", self._h, C.byref(p))
        return p.value

    def _x(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.shape != (self.nmbProblems(), self.nmbPars()):
            raise ValueError("parameters must have shape (problems, parameters) = (%d, %d)" %
                             (self.nmbProblems(), self.nmbPars()))
        return x

    def autotune(self, x):
        x = self._x(x)
        N.call("pwa_multibin_autotune", self._h, _pd(x))
        return self.chunks()

    def FdF(self, x):
        """(f [Q], grad [Q][P]) of every problem at x [Q][P]."""
        x = self._x(x)
        f = np.zeros(x.shape[0])
        g = np.zeros_like(x)
        N.call("pwa_multibin_fdf", self._h, _pd(x), _pd(f), _pd(g))
        return f, g

    def sweepMs(self, x, reps=3):
        """Device time of one evaluation sweep of all problems at x."""
        x = self._x(x)
        ms = C.c_double()
        N.call("pwa_multibin_sweep_ms", self._h, _pd(x), int(reps), C.byref(ms))
        return ms.value

    def trace(self):
        """(seconds [checks], f [checks][Q]) recorded by the last fit."""
        n = C.c_uint32()
        N.call("pwa_multibin_trace", self._h, 0, None, None, C.byref(n))
        t = np.zeros(n.value)
        f = np.zeros((n.value, self.nmbProblems()))
        N.call("pwa_multibin_trace", self._h, n.value, _pd(t), _pd(f), C.byref(n))
        return t, f

    def fit(self, x0, useGraph=True, sweepsPerGraph=25, maxSweeps=1_000_000):
        """L-BFGS of every problem from x0; returns a dict with x, f, gnorm,
        status, iterations and sweeps."""
        x0 = self._x(x0)
        Q = x0.shape[0]
        x = np.zeros_like(x0)
        f = np.zeros(Q)
        gn = np.zeros(Q)
        st = np.zeros(Q, dtype=np.int32)
        it = np.zeros(Q, dtype=np.uint32)
        sw = C.c_uint32()
        N.call("pwa_multibin_fit", self._h, _pd(x0), 1 if useGraph else 0, int(sweepsPerGraph), int(maxSweeps),
               _pd(x), _pd(f), _pd(gn), st.ctypes.data_as(C.POINTER(C.c_int32)),
               it.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(sw))
        return dict(x=x, f=f, gnorm=gn, status=st, iterations=it, sweeps=sw.value)

    def resume(self, useGraph=True, sweepsPerGraph=25, maxSweeps=1_000_000):
        """Continues the fit held on the device (after fit() stopped at
        maxSweeps, or after loadState); same outputs as fit()."""
        Q, P = self.nmbProblems(), self.nmbPars()
        x = np.zeros((Q, P))
        f = np.zeros(Q)
        gn = np.zeros(Q)
        st = np.zeros(Q, dtype=np.int32)
        it = np.zeros(Q, dtype=np.uint32)
        sw = C.c_uint32()
        N.call("pwa_multibin_resume", self._h, 1 if useGraph else 0, int(sweepsPerGraph), int(maxSweeps),
               _pd(x), _pd(f), _pd(gn), st.ctypes.data_as(C.POINTER(C.c_int32)),
               it.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(sw))
        return dict(x=x, f=f, gnorm=gn, status=st, iterations=it, sweeps=sw.value)

    def saveState(self, path):
        """Writes the device-side fit state to a checkpoint file."""
        N.call("pwa_multibin_save_state", self._h, str(path).encode())

    def loadState(self, path):
        """Reads a checkpoint written for a batch with the same bins, starts and options."""
        N.call("pwa_multibin_load_state", self._h, str(path).encode())

    def setCheckpoint(self, path, everySweeps):
        """fit()/resume() write the checkpoint file every `everySweeps` sweeps (0: off)."""
        N.call("pwa_multibin_set_checkpoint", self._h, str(path).encode() if path else None, int(everySweeps))

    def sweepsDone(self):
        v = C.c_uint32()
        N.call("pwa_multibin_sweeps_done", self._h, C.byref(v))
        return v.value
