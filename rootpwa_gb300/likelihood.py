"""Python mirror of ROOTPWA's pwaLikelihood and ampIntegralMatrix over the C ABI.

Method names, argument order and semantics follow the reference's Python
bindings (pyInterface/bindings/partialWaveFit/pwaLikelihood_py.cc:243-312 and
pyInterface/bindings/decayAmplitude/ampIntegralMatrix_py.cc), so code written
against pyRootPwa.core.pwaLikelihood reads the same.  Differences:

* addAmplitude takes (waveName, amplitudes) instead of amplitudeMetadata
  objects (ROOT trees are out of scope); amplitudes are a numpy array
  (complex64 or complex128, host) or any CUDA array exposing
  __cuda_array_interface__ (device).
* init takes (waveNames, reflectivities, thresholds, rank, massBinCenter)
  instead of wave descriptions (the reference reads the reflectivity from the
  decay topology).
* Failures raise PwaError instead of returning False / printErr.

Every evaluation runs in libpwa_gb300.so on the GPU; nothing here computes.
"""
import ctypes as C

import numpy as np

from . import _native as N


def _pd(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _names(names):
    arr = (C.c_char_p * len(names))()
    arr[:] = [n.encode() for n in names]
    return arr


def _amp_buffer(amps):
    """(pointer, n, type, memory, keepalive) for a host or device complex array."""
    cai = getattr(amps, "__cuda_array_interface__", None)
    if cai is not None:
        typestr = cai["typestr"]
        if typestr.endswith("c8"):
            t = N.COMPLEX64
        elif typestr.endswith("c16"):
            t = N.COMPLEX128
        else:
            raise TypeError("device amplitudes must be complex64 or complex128, got %s" % typestr)
        if cai.get("strides") not in (None,):
            item = 8 if t == N.COMPLEX64 else 16
            exp = [item]
            for s in reversed(cai["shape"][1:]):
                exp.insert(0, exp[0] * s)
            if tuple(cai["strides"]) != tuple(exp):
                raise ValueError("device amplitudes must be contiguous")
        n = int(np.prod(cai["shape"])) if cai["shape"] else 1
        return C.c_void_p(cai["data"][0]), n, t, N.MEMORY_DEVICE, amps
    a = np.asarray(amps)
    if a.dtype == np.complex64:
        t = N.COMPLEX64
    elif a.dtype == np.complex128:
        t = N.COMPLEX128
    else:
        a = a.astype(np.complex128)
        t = N.COMPLEX128
    a = np.ascontiguousarray(a)
    return C.c_void_p(a.ctypes.data), a.size, t, N.MEMORY_HOST, a


class ampIntegralMatrix:
    """rpwa::ampIntegralMatrix (decayAmplitude/ampIntegralMatrix.h:67-173)."""

    def __init__(self, other=None):
        h = C.c_void_p()
        N.call("pwa_integral_create", C.byref(h))
        self._h = h
        if other is not None:
            N.call("pwa_integral_copy", self._h, other._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and N._lib is not None:
            N.lib().pwa_integral_destroy(h)
            self._h = None

    # -- construction ------------------------------------------------------
    def setWaveNames(self, names):
        N.call("pwa_integral_set_wave_names", self._h, len(names), _names(names))
        return True

    def integrate(self, waveNames, amplitudes, maxNmbEvents=0, weights=None, inBin=None, precision="fp32",
                  nmbSubAmps=1):
        """integrate (ampIntegralMatrix.cc:300-489) on the GPU.

        amplitudes: complex array [wave][event] (or [wave][event][subAmp]),
        host numpy or device (__cuda_array_interface__).  weights: the
        importance-sampling weight stream (one per selected event), inBin:
        per-event bin flags, precision: 'fp64', 'fp32', 'tf32', 'tf32x3',
        'bf16x3'."""
        ptr, n, t, mem, keep = _amp_buffer(amplitudes)
        nw = len(waveNames)
        if n % (nw * nmbSubAmps):
            raise ValueError("amplitude array size is not a multiple of the wave count")
        n_ev = n // (nw * nmbSubAmps)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        b = None if inBin is None else np.ascontiguousarray(inBin, dtype=np.uint8)
        prec = N.PRECISION[precision] if isinstance(precision, str) else int(precision)
        N.call("pwa_integral_integrate", self._h, nw, _names(waveNames), ptr, n_ev, nmbSubAmps, t, mem,
               None if w is None else _pd(w), 0 if w is None else len(w),
               None if b is None else C.c_void_p(b.ctypes.data), int(maxNmbEvents), prec)
        del keep
        return True

    def addEvent(self, amplitudes):
        """addEvent (ampIntegralMatrix.cc:280-297): dict name -> complex, or array in wave order."""
        if isinstance(amplitudes, dict):
            amplitudes = [amplitudes[n] for n in self.waveNames()]
        a = np.ascontiguousarray(np.asarray(amplitudes, dtype=np.complex128)).view(np.float64)
        N.call("pwa_integral_add_event", self._h, _pd(a))
        return True

    # -- accessors -----------------------------------------------------------
    def nmbWaves(self):
        n = C.c_uint32()
        N.call("pwa_integral_nmb_waves", self._h, C.byref(n))
        return n.value

    def nmbEvents(self):
        n = C.c_uint64()
        N.call("pwa_integral_nmb_events", self._h, C.byref(n))
        return n.value

    def setNmbEvents(self, n):
        N.call("pwa_integral_set_nmb_events", self._h, int(n))

    def waveName(self, i):
        buf = C.create_string_buffer(4096)
        N.call("pwa_integral_wave_name", self._h, int(i), buf, 4096)
        return buf.value.decode()

    def waveNames(self):
        return [self.waveName(i) for i in range(self.nmbWaves())]

    def containsWave(self, name):
        """containsWave (ampIntegralMatrix.cc:188-191)."""
        c = C.c_int()
        N.call("pwa_integral_contains_wave", self._h, name.encode(), C.byref(c))
        return bool(c.value)

    def hasIdenticalWaveSet(self, other):
        """hasIdenticalWaveSet (ampIntegralMatrix.cc:633-646)."""
        same = C.c_int()
        N.call("pwa_integral_compare", self._h, other._h, C.byref(same), None)
        return bool(same.value)

    def __eq__(self, other):
        """operator == (ampIntegralMatrix.h:179-195)."""
        if not isinstance(other, ampIntegralMatrix):
            return NotImplemented
        eq = C.c_int()
        N.call("pwa_integral_compare", self._h, other._h, None, C.byref(eq))
        return bool(eq.value)

    def __ne__(self, other):
        r = self.__eq__(other)
        return r if r is NotImplemented else not r

    __hash__ = None

    def clear(self):
        """clear (ampIntegralMatrix.cc:93-103)."""
        N.call("pwa_integral_clear", self._h)

    def waveIndex(self, name):
        k = C.c_uint32()
        N.call("pwa_integral_wave_index", self._h, name.encode(), C.byref(k))
        return k.value

    def element(self, i, j):
        if isinstance(i, str):
            i = self.waveIndex(i)
        if isinstance(j, str):
            j = self.waveIndex(j)
        re, im = C.c_double(), C.c_double()
        N.call("pwa_integral_element", self._h, int(i), int(j), C.byref(re), C.byref(im))
        return complex(re.value, im.value)

    def matrix(self):
        """Raw sums (before division by nmbEvents), complex128 [nWaves][nWaves]."""
        n = self.nmbWaves()
        out = np.zeros(2 * n * n)
        N.call("pwa_integral_matrix", self._h, _pd(out))
        return out.view(np.complex128).reshape(n, n)

    def setMatrix(self, m):
        m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128)).view(np.float64)
        N.call("pwa_integral_set_matrix", self._h, _pd(m))

    # -- arithmetic ------------------------------------------------------------
    def __iadd__(self, other):
        N.call("pwa_integral_add", self._h, other._h)
        return self

    def __isub__(self, other):
        N.call("pwa_integral_subtract", self._h, other._h)
        return self

    def __imul__(self, f):
        N.call("pwa_integral_scale", self._h, float(f))
        return self

    def __itruediv__(self, f):
        N.call("pwa_integral_divide", self._h, float(f))
        return self

    def renormalize(self, n):
        N.call("pwa_integral_renormalize", self._h, int(n))

    # -- I/O -----------------------------------------------------------------------
    def readAscii(self, path):
        N.call("pwa_integral_read_ascii", self._h, str(path).encode())
        return True

    def writeAscii(self, path):
        N.call("pwa_integral_write_ascii", self._h, str(path).encode())
        return True


class pwaLikelihood:
    """rpwa::pwaLikelihood<std::complex<double>> (partialWaveFit/pwaLikelihood.h:66-320) on the GPU."""

    FLAT = N.PRIOR_FLAT
    HALF_CAUCHY = N.PRIOR_HALF_CAUCHY

    def __init__(self):
        h = C.c_void_p()
        N.call("pwa_likelihood_create", C.byref(h))
        self._h = h
        self._P = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and N._lib is not None:
            N.lib().pwa_likelihood_destroy(h)
            self._h = None

    # -- options -------------------------------------------------------------
    def useNormalizedAmps(self, flag=True):
        N.call("pwa_likelihood_use_normalized_amps", self._h, int(bool(flag)))

    def setPriorType(self, prior):
        N.call("pwa_likelihood_set_prior_type", self._h, int(prior))

    def setOnTheFlyBinning(self, boundaries, binVars):
        """setOnTheFlyBinning (pwaLikelihood.cc:1391-1440).  boundaries:
        {name: (lower, upper)}; binVars: {name: per-event values of the data
        file} (numpy or CUDA arrays, all of the file's length).  Events with
        lower <= x < upper for every variable are kept, in file order;
        addAmplitude then takes whole-file amplitude arrays."""
        names = list(boundaries)
        lo = np.array([boundaries[k][0] for k in names], dtype=np.float64)
        hi = np.array([boundaries[k][1] for k in names], dtype=np.float64)
        keep, ptrs, n, mem = [], [], None, None
        for k in names:
            v = binVars[k]
            cai = getattr(v, "__cuda_array_interface__", None)
            if cai is not None:
                if not cai["typestr"].endswith("f8"):
                    raise TypeError("device binning variables must be float64")
                if cai.get("strides") not in (None, (8,)):
                    raise ValueError("device binning variables must be contiguous")
                ptrs.append(cai["data"][0])
                m, size = N.MEMORY_DEVICE, int(np.prod(cai["shape"]))
            else:
                a = np.ascontiguousarray(v, dtype=np.float64)
                keep.append(a)
                ptrs.append(a.ctypes.data)
                m, size = N.MEMORY_HOST, a.size
            if n is None:
                n, mem = size, m
            elif size != n or m != mem:
                raise ValueError("binning variables must have one length and one residence")
        arr = (C.c_void_p * max(1, len(ptrs)))(*ptrs)
        N.call("pwa_likelihood_set_otf_binning", self._h, len(names), _pd(lo), _pd(hi), arr, int(n), mem)

    def loadAmplitudeFiles(self, paths, boundaries=None):
        """addAmplitude for every wave of the wave list from raw amplitude
        files (rootpwa_gb300.ampfile), their events concatenated in the
        order given, with on-the-fly binning {variable: (lower, upper)} on
        the files' binning variables when boundaries are given."""
        if isinstance(paths, (str, bytes)) or hasattr(paths, "__fspath__"):
            paths = [paths]
        ps = [str(p).encode() for p in paths]
        boundaries = boundaries or {}
        names = list(boundaries)
        lo = np.array([boundaries[k][0] for k in names] or [0.0], dtype=np.float64)
        hi = np.array([boundaries[k][1] for k in names] or [0.0], dtype=np.float64)
        pa = (C.c_char_p * len(ps))(*ps)
        na = (C.c_char_p * max(1, len(names)))(*[k.encode() for k in names])
        N.call("pwa_likelihood_load_amp_files", self._h, len(ps), pa, len(names), na, _pd(lo), _pd(hi))
        return True

    def otfSelected(self):
        n = C.c_uint64()
        N.call("pwa_likelihood_otf_selected", self._h, C.byref(n))
        return n.value

    def setShard(self, totalEvents, root):
        """Event-sharded evaluation: this likelihood holds one share of the
        events; only the root shard adds the normalisation and prior terms
        (no reference counterpart; see rootpwa_gb300.sharded)."""
        N.call("pwa_likelihood_set_shard", self._h, int(totalEvents), 1 if root else 0)

    def setCauchyWidth(self, width):
        N.call("pwa_likelihood_set_cauchy_width", self._h, float(width))

    def _options(self):
        u, p, w = C.c_int(), C.c_int(), C.c_double()
        N.call("pwa_likelihood_options", self._h, C.byref(u), C.byref(p), C.byref(w))
        return bool(u.value), p.value, w.value

    def normalizedAmpsUsed(self):
        return self._options()[0]

    def priorType(self):
        return self._options()[1]

    def cauchyWidth(self):
        return self._options()[2]

    def enableCuda(self, flag=True):
        """enableCuda (pwaLikelihood.h:212): every evaluation runs on the GPU;
        there is no CPU path to switch to."""
        if not flag:
            raise N.PwaError(7, "the GB300 engine has no CPU evaluation path")

    def cudaEnabled(self):
        return True

    def dLcache(self, i):
        """dLcache (pwaLikelihood.h:200): component i of the gradient of the
        last FdF / Gradient call."""
        g = np.zeros(self.nmbPars())
        N.call("pwa_likelihood_deriv_cache", self._h, _pd(g))
        return float(g[i])

    def clear(self):
        """clear (pwaLikelihood.cc:1670-1674): releases the amplitude store."""
        N.call("pwa_likelihood_clear", self._h)

    def Clone(self):
        """Clone (pwaLikelihood.h:160): the handle owns device memory; build a
        second likelihood instead."""
        raise N.PwaError(7, "pwaLikelihood handles cannot be cloned; create a new one")

    @staticmethod
    def setQuiet(flag=True):
        """The engine prints nothing; kept for call compatibility."""
        return None

    def setStream(self, stream_handle):
        """CUDA stream (integer handle, e.g. torch.cuda.Stream().cuda_stream) for all launches."""
        N.call("pwa_likelihood_set_stream", self._h, C.c_void_p(int(stream_handle)))

    def setReduction(self, mode):
        """cross-tile reduction: 'fp64' (default: FP32 partials of 64 tiles
        folded into FP64), 'kahan_fp32' (every tile into compensated FP32) or
        'fp32' (plain FP32 over all tiles)."""
        m = {"fp64": N.REDUCE_FP64, "kahan_fp32": N.REDUCE_KAHAN_FP32,
             "fp32": N.REDUCE_FP32}[mode] if isinstance(mode, str) else int(mode)
        N.call("pwa_likelihood_set_reduction", self._h, m)

    def setAutotune(self, enable=True):
        """Time the compiled FdF kernel plans at finishInit and keep the fastest (default on)."""
        N.call("pwa_likelihood_set_autotune", self._h, int(bool(enable)))

    def plan(self):
        """(events per tile, pipeline stages, grid blocks) of the FdF kernel in use."""
        e, s, b = C.c_int(), C.c_int(), C.c_int()
        N.call("pwa_likelihood_plan", self._h, C.byref(e), C.byref(s), C.byref(b))
        return e.value, s.value, b.value

    def setPlan(self, stages, phase1Events=0):
        """Select the FdF kernel pipeline depth and coherent-sum variant (1 or
        2 events per lane; 0 keeps the current one) by hand (after finishInit)."""
        N.call("pwa_likelihood_set_plan_variant", self._h, int(stages), int(phase1Events))

    def setStoreBlock(self, events):
        """Events per amplitude-store block / FdF tile (64 or 128; 0 automatic),
        before the first addAmplitude."""
        N.call("pwa_likelihood_set_store_block", self._h, int(events))

    def planVariant(self):
        """Events per lane of the FdF kernel's coherent-sum phase (1 or 2)."""
        v = C.c_int()
        N.call("pwa_likelihood_plan_variant", self._h, C.byref(v))
        return v.value

    # -- setup (order as _likelihood.py:17-71) -------------------------------
    def init(self, waveNames, reflectivities, thresholds=None, rank=1, massBinCenter=0.0):
        n = len(waveNames)
        refl = (C.c_int32 * n)(*[int(r) for r in reflectivities])
        th = None if thresholds is None else np.ascontiguousarray(thresholds, dtype=np.float64)
        N.call("pwa_likelihood_init", self._h, n, _names(waveNames), refl, None if th is None else _pd(th),
               int(rank), float(massBinCenter))
        self._P = None
        return True

    def addNormIntegral(self, normMatrix):
        N.call("pwa_likelihood_add_norm_integral", self._h, normMatrix._h)
        return True

    def addAccIntegral(self, accMatrix, accEventsOverride=0):
        N.call("pwa_likelihood_add_acc_integral", self._h, accMatrix._h, int(accEventsOverride))
        return True

    def addAmplitude(self, waveName, amplitudes):
        ptr, n, t, mem, keep = _amp_buffer(amplitudes)
        N.call("pwa_likelihood_add_amplitude", self._h, waveName.encode(), ptr, n, t, mem)
        del keep
        return True

    def finishInit(self):
        N.call("pwa_likelihood_finish_init", self._h)
        return True

    # -- accessors -------------------------------------------------------------
    def nmbPars(self):
        if self._P is None:
            n = C.c_uint32()
            N.call("pwa_likelihood_nmb_pars", self._h, C.byref(n))
            self._P = n.value
        return self._P

    NDim = nmbPars

    def nmbParsFixed(self):
        n = C.c_uint32()
        N.call("pwa_likelihood_nmb_pars_fixed", self._h, C.byref(n))
        return n.value

    def nmbEvents(self):
        n = C.c_uint64()
        N.call("pwa_likelihood_nmb_events", self._h, C.byref(n))
        return n.value

    def rank(self):
        n = C.c_uint32()
        N.call("pwa_likelihood_rank", self._h, C.byref(n))
        return n.value

    def nmbWaves(self, reflectivity=0):
        n = C.c_uint32()
        N.call("pwa_likelihood_nmb_waves", self._h, int(reflectivity), C.byref(n))
        return n.value

    def totAcc(self):
        t = C.c_double()
        N.call("pwa_likelihood_tot_acc", self._h, C.byref(t))
        return t.value

    def parameter(self, i):
        buf = C.create_string_buffer(4096)
        fixed, real, rank = C.c_int(), C.c_int(), C.c_int32()
        th = C.c_double()
        N.call("pwa_likelihood_parameter", self._h, int(i), buf, 4096, C.byref(fixed), C.byref(real),
               C.byref(rank), C.byref(th))
        return {"name": buf.value.decode(), "fixed": bool(fixed.value), "realPart": bool(real.value),
                "rank": rank.value, "threshold": th.value}

    def parameters(self):
        return [self.parameter(k) for k in range(self.nmbPars())]

    # -- evaluation -------------------------------------------------------------
    def _par(self, par):
        p = np.ascontiguousarray(par, dtype=np.float64)
        if p.shape != (self.nmbPars(),):
            raise ValueError("expected %d parameters, got %s" % (self.nmbPars(), p.shape))
        return p

    def FdF(self, par):
        p = self._par(par)
        f = C.c_double()
        g = np.zeros(self.nmbPars())
        N.call("pwa_likelihood_fdf", self._h, _pd(p), C.byref(f), _pd(g))
        return f.value, g

    def DoEval(self, par):
        p = self._par(par)
        f = C.c_double()
        N.call("pwa_likelihood_doeval", self._h, _pd(p), C.byref(f))
        return f.value

    def Gradient(self, par):
        p = self._par(par)
        g = np.zeros(self.nmbPars())
        N.call("pwa_likelihood_gradient", self._h, _pd(p), _pd(g))
        return g

    def DoDerivative(self, par, index):
        p = self._par(par)
        d = C.c_double()
        N.call("pwa_likelihood_doderivative", self._h, _pd(p), int(index), C.byref(d))
        return d.value

    def FdFBatch(self, pars):
        p = np.ascontiguousarray(pars, dtype=np.float64)
        n = p.shape[0]
        f = np.zeros(n)
        g = np.zeros((n, self.nmbPars()))
        N.call("pwa_likelihood_fdf_batch", self._h, n, _pd(p), _pd(f), _pd(g))
        return f, g

    def FdFDevice(self, d_par_ptr, d_out_ptr, with_gradient=True, stream=0):
        """Asynchronous device-resident FdF: P doubles at d_par_ptr -> (P+2) doubles at d_out_ptr."""
        N.call("pwa_likelihood_fdf_device", self._h, C.c_void_p(int(d_par_ptr)), C.c_void_p(int(d_out_ptr)),
               int(bool(with_gradient)), C.c_void_p(int(stream)))

    def Hessian(self, par):
        p = self._par(par)
        n = self.nmbPars()
        H = np.zeros((n, n))
        N.call("pwa_likelihood_hessian", self._h, _pd(p), _pd(H))
        return H

    def CovarianceMatrix(self, hessian_or_par):
        a = np.asarray(hessian_or_par, dtype=np.float64)
        H = self.Hessian(a) if a.ndim == 1 else np.ascontiguousarray(a)
        n = self.nmbPars()
        Cm = np.zeros((n, n))
        N.call("pwa_likelihood_covariance_matrix", self._h, _pd(H), _pd(Cm))
        return Cm

    def HessianEigenVectors(self, hessian):
        """HessianEigenVectors (pwaLikelihood.cc:864-912): [(eigenvector [P],
        eigenvalue)] of the Hessian restricted to the free parameters,
        eigenvalues descending, eigenvectors zero at fixed parameters."""
        H = np.ascontiguousarray(hessian, dtype=np.float64)
        n = self.nmbPars()
        vals = np.zeros(n)
        vecs = np.zeros((n, n))
        k = C.c_uint32()
        N.call("pwa_likelihood_hessian_eigenvectors", self._h, _pd(H), _pd(vals), _pd(vecs), C.byref(k))
        return [(vecs[i].copy(), float(vals[i])) for i in range(k.value)]

    def CorrectParamSigns(self, par):
        p = self._par(par)
        out = np.zeros_like(p)
        N.call("pwa_likelihood_correct_param_signs", self._h, _pd(p), _pd(out))
        return out

    def integralMatrices(self, withFlat=False):
        sz = self.nmbWaves() + (1 if withFlat else 0)
        n = np.zeros(2 * sz * sz)
        a = np.zeros(2 * sz * sz)
        ps = np.zeros(sz)
        N.call("pwa_likelihood_integral_matrices", self._h, _pd(n), _pd(a), _pd(ps), int(bool(withFlat)))
        return n.view(np.complex128).reshape(sz, sz), a.view(np.complex128).reshape(sz, sz), ps

    def buildProdAmpArrays(self, par, withFlat=True):
        p = self._par(par)
        n = self.nmbPars()
        amps = np.zeros(2 * n)
        idx = np.zeros(2 * n, dtype=np.int32)
        k = C.c_uint32()
        N.call("pwa_likelihood_build_prod_amp_arrays", self._h, _pd(p), _pd(amps),
               idx.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(k), int(bool(withFlat)))
        m = k.value
        return amps[:2 * m].view(np.complex128).copy(), [tuple(x) for x in idx[:2 * m].reshape(m, 2)]

    def funcCallInfo(self, call=N.CALL_FDF):
        n = C.c_uint64()
        t, fn, nm = C.c_double(), C.c_double(), C.c_double()
        N.call("pwa_likelihood_func_call_info", self._h, int(call), C.byref(n), C.byref(t), C.byref(fn), C.byref(nm))
        return {"nmbCalls": n.value, "totalTime": t.value, "funcTime": fn.value, "normTime": nm.value}

    def ncalls(self, func=N.CALL_FDF):
        """ncalls (pwaLikelihood.h:199)."""
        return self.funcCallInfo(func)["nmbCalls"]

    def Ltime(self, func=N.CALL_FDF):
        """Ltime (pwaLikelihood.h:201): seconds in the event kernels."""
        return self.funcCallInfo(func)["funcTime"]

    def Ntime(self, func=N.CALL_FDF):
        """Ntime (pwaLikelihood.h:203): seconds in the normalisation term."""
        return self.funcCallInfo(func)["normTime"]

    def resetFuncCallInfo(self):
        N.call("pwa_likelihood_reset_func_call_info", self._h)

    def printFuncInfo(self, out=None):
        """printFuncInfo (pwaLikelihood.cc:1765-1779): calls and times per
        evaluation type, one line each (to `out`, default stdout)."""
        import sys
        out = out or sys.stdout
        for name, call in (("FdF", N.CALL_FDF), ("Gradient", N.CALL_GRADIENT), ("DoEval", N.CALL_DOEVAL),
                           ("DoDerivative", N.CALL_DODERIVATIVE), ("Hessian", N.CALL_HESSIAN)):
            i = self.funcCallInfo(call)
            out.write("%-12s: %d calls, %.6f s total, %.6f s in the event kernels, %.6f s normalisation\n"
                      % (name, i["nmbCalls"], i["totalTime"], i["funcTime"], i["normTime"]))

    getIntegralMatrices = integralMatrices

    def setTiming(self, enable=True):
        """Record CUDA events around each evaluation's two kernels."""
        N.call("pwa_likelihood_set_timing", self._h, int(bool(enable)))

    def kernelTimes(self):
        """(event-kernel ms, finalize ms, evaluations) summed since the last read."""
        a, b = C.c_double(), C.c_double()
        n = C.c_uint64()
        N.call("pwa_likelihood_kernel_times", self._h, C.byref(a), C.byref(b), C.byref(n))
        return a.value, b.value, n.value
