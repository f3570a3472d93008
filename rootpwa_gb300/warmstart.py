"""Learned warm start for multibin fits.

A 3-layer perceptron (pwa_mlp_*, hand-written CUDA kernels, BF16 with FP32
accumulation) maps a bin's data-averaged moment matrix
    M_ij = < a_i conj(a_j) >_data,  a = (A_w / sqrt(N_ww), 1)
(the normalised decay amplitudes of the likelihood plus the flat wave, all
real and imaginary parts) and log N to the production amplitudes at the
likelihood minimum, V / sqrt(N) (real and imaginary parts of the waves and
the flat wave).  The plain fit always refines the prediction; random start
points remain the fallback.  There is no reference counterpart: ROOTPWA
starts its fits from random amplitudes (pwaFit.cc:231-257).
"""
import ctypes as C

import numpy as np

from . import _native as N


def _pf(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class pwaMLP:
    """nIn -> nHidden1 -> nHidden2 -> nOut perceptron on the GPU."""

    def __init__(self, nIn, nHidden1=512, nHidden2=512, nOut=102, seed=0):
        h = C.c_void_p()
        N.call("pwa_mlp_create", C.byref(h), int(nIn), int(nHidden1), int(nHidden2), int(nOut), int(seed))
        self._h = h
        self.shape = (int(nIn), int(nHidden1), int(nHidden2), int(nOut))
        # input standardisation (set by fit_standardisation)
        self.mu = np.zeros(nIn, dtype=np.float32)
        self.sd = np.ones(nIn, dtype=np.float32)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and N._lib is not None:
            N.lib().pwa_mlp_destroy(h)
            self._h = None

    def nmbParams(self):
        n = C.c_uint64()
        N.call("pwa_mlp_nmb_params", self._h, C.byref(n))
        return n.value

    def params(self):
        p = np.zeros(self.nmbParams(), dtype=np.float32)
        N.call("pwa_mlp_get_params", self._h, _pf(p))
        return p

    def setParams(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nmbParams()
        N.call("pwa_mlp_set_params", self._h, _pf(p))

    def _X(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        assert X.ndim == 2 and X.shape[1] == self.shape[0]
        return X

    def forward(self, X):
        X = self._X(X)
        Y = np.zeros((X.shape[0], self.shape[3]), dtype=np.float32)
        N.call("pwa_mlp_forward", self._h, _pf(X), X.shape[0], _pf(Y))
        return Y

    def gradient(self, X, T):
        """(mean squared error, gradient in the parameter layout)."""
        X = self._X(X)
        T = np.ascontiguousarray(T, dtype=np.float32)
        loss = C.c_double()
        g = np.zeros(self.nmbParams(), dtype=np.float32)
        N.call("pwa_mlp_gradient", self._h, _pf(X), _pf(T), X.shape[0], C.byref(loss), _pf(g))
        return loss.value, g

    def train(self, X, T, batch=256, epochs=50, lr=1e-3, seed=0):
        """Adam on standardised inputs; returns the mean loss of each epoch."""
        X = self._X(X)
        T = np.ascontiguousarray(T, dtype=np.float32)
        hist = np.zeros(epochs)
        N.call("pwa_mlp_train", self._h, _pf(X), _pf(T), X.shape[0], int(batch), int(epochs), float(lr), int(seed),
               hist.ctypes.data_as(C.POINTER(C.c_double)))
        return hist

    # -- standardised use ------------------------------------------------------
    def fit_standardisation(self, F):
        self.mu = F.mean(axis=0).astype(np.float32)
        self.sd = (F.std(axis=0) + 1e-6).astype(np.float32)

    def standardise(self, F):
        return ((F - self.mu) / self.sd).astype(np.float32)


# ---------------------------------------------------------------------------
# features and targets
# ---------------------------------------------------------------------------
def moment_features(names, data, norm_diag, precision="tf32x3"):
    """Features of one bin: the real and imaginary parts of the moment matrix
    of (A_w / sqrt(N_ww), 1) over the data events and log N.

    data: complex64 [W][N] device array (torch); norm_diag: the
    normalisation integral's diagonal per event (element(w, w))."""
    import torch
    from .likelihood import ampIntegralMatrix
    W, n = data.shape
    ext = torch.cat([data, torch.ones((1, n), dtype=data.dtype, device=data.device)], dim=0).contiguous()
    I = ampIntegralMatrix()
    I.integrate(list(names) + ["flat"], ext, precision=precision)
    M = I.matrix() / n
    s = np.concatenate([1.0 / np.sqrt(np.asarray(norm_diag, dtype=np.float64)), [1.0]])
    M = M * s[:, None] * s[None, :]
    return np.concatenate([M.real.ravel(), M.imag.ravel(), [np.log(n)]]).astype(np.float32)


def moment_features_batch(datas, norm_diags, precision="tf32x3"):
    """moment_features of many bins at once, from device amplitudes in place:
    the W x W sums A conj(A)^T and the sums of A of every bin by one call of
    pwa_gram_device_batch (the integral's Gram kernels, by default the same
    TF32x3 precision as moment_features), one download at the end."""
    import torch
    W = datas[0].shape[0]
    nb = len(datas)
    gram = torch.empty((nb, W, W), dtype=torch.complex128, device=datas[0].device)
    sums = torch.empty((nb, W), dtype=torch.complex128, device=datas[0].device)
    for d in datas:
        assert d.is_contiguous() and d.dtype == torch.complex64 and d.shape[0] == W
    ptrs = (C.c_void_p * nb)(*[d.data_ptr() for d in datas])
    counts = (C.c_uint64 * nb)(*[d.shape[1] for d in datas])
    N.call("pwa_gram_device_batch", ptrs, counts, nb, W, N.PRECISION[precision], C.c_void_p(gram.data_ptr()),
           C.c_void_p(sums.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    # assembled on the device (the same FP64 operations as moment_features),
    # one download of the FP32 features
    dev = gram.device
    n = torch.tensor([d.shape[1] for d in datas], dtype=torch.float64, device=dev)
    sc = torch.ones((nb, W + 1), dtype=torch.float64, device=dev)
    sc[:, :W] = 1.0 / torch.sqrt(torch.as_tensor(np.asarray(norm_diags, dtype=np.float64).reshape(nb, W), device=dev))
    M = torch.empty((nb, W + 1, W + 1), dtype=torch.complex128, device=dev)
    M[:, :W, :W] = gram
    M[:, :W, W] = sums
    M[:, W, :W] = sums.conj()
    M[:, W, W] = n
    M /= n[:, None, None]
    M *= sc[:, :, None] * sc[:, None, :]
    F = torch.cat([M.real.reshape(nb, -1), M.imag.reshape(nb, -1), torch.log(n)[:, None]], dim=1)
    return F.to(torch.float32).cpu().numpy()


def prod_amp_indices(L):
    """Parameter indices (re, im or -1) of the production amplitudes and the
    flat wave, in wave order (pwaLikelihood::buildProdAmpArrays)."""
    _, idx = L.buildProdAmpArrays(np.zeros(L.nmbPars()), withFlat=True)
    return idx


def params_to_complex(L, x):
    idx = prod_amp_indices(L)
    return np.array([(x[r] if r >= 0 else 0.0) + 1j * (x[i] if i >= 0 else 0.0) for r, i in idx])


def complex_to_params(L, v):
    """Parameter vector from complex amplitudes (waves then flat), rotated so
    that the first wave is real and positive (the layout's convention)."""
    idx = prod_amp_indices(L)
    v = np.asarray(v, dtype=np.complex128)
    ph = np.exp(-1j * np.angle(v[0])) if abs(v[0]) > 0 else 1.0
    v = v.copy()
    v[:-1] *= ph
    v[-1] = abs(v[-1])
    x = np.zeros(L.nmbPars())
    for (r, i), c in zip(idx, v):
        if r >= 0:
            x[r] = c.real
        if i >= 0:
            x[i] = c.imag
    return x


def targets_from_params(L, x, n_events):
    v = params_to_complex(L, L.CorrectParamSigns(x)) / np.sqrt(n_events)
    return np.concatenate([v.real, v.imag]).astype(np.float32)


def params_from_targets(L, y, n_events):
    k = len(y) // 2
    v = (np.asarray(y[:k], dtype=np.float64) + 1j * np.asarray(y[k:], dtype=np.float64)) * np.sqrt(n_events)
    return complex_to_params(L, v)


def start_from_truth(L, v_true, flat, n_events, norm_diag):
    """The true amplitudes in the likelihood's normalisation: each wave
    scaled by sqrt(N_ww) (norm_diag: the normalisation integral's diagonal
    per event, as the likelihood divides the amplitudes by it), all scaled so
    that the expected number of accepted events equals n_events."""
    _, accM, _ = L.integralMatrices(withFlat=False)  # normalised acceptance integral
    v = np.asarray(v_true) * np.sqrt(np.asarray(norm_diag, dtype=np.float64))
    expected = np.real(np.conj(v) @ (accM @ v)) + flat * flat * L.totAcc()
    s = np.sqrt(n_events / max(expected, 1e-300))
    return complex_to_params(L, np.concatenate([v * s, [flat * s]]))


def generate_training_set(names, draw_bin, norm, acc, counts, rng, chunk=1000, precision="tf32x3",
                          gtolRel=1e-8, maxIter=3000):
    """Training pairs (features, targets) produced by the method itself.

    For each bin k: true amplitudes V_true (re/im ~ N(0, 1)) and a flat
    amplitude are drawn, draw_bin(v_true, flat, counts[k], k) returns the
    bin's data amplitudes (complex64 [W][N] on the device, drawn in
    proportion to the model intensity), a likelihood is built with the shared
    normalisation and acceptance integrals, and the plain batched L-BFGS fits
    it from the true amplitudes; the target is the minimum (CorrectParamSigns
    convention, divided by sqrt(N)) and the features the data moments.
    Returns (F [n][(W+1)^2 * 2 + 1], Y [n][2 (W+1)], V_true [n][W])."""
    from .likelihood import ampIntegralMatrix, pwaLikelihood
    from .multibin import pwaMultibin
    diag = np.real(np.diag(norm.matrix())) / norm.nmbEvents()
    F, Y, VT = [], [], []
    for c0 in range(0, len(counts), chunk):
        bins = []
        for k in range(c0, min(len(counts), c0 + chunk)):
            vt, fl = synth_true(len(names), rng)
            n = int(counts[k])
            data = draw_bin(vt, fl, n, k)
            L = pwaLikelihood()
            L.init(names, [1] * len(names), None, 1, 0.0)
            L.addNormIntegral(ampIntegralMatrix(norm))
            L.addAccIntegral(ampIntegralMatrix(acc))
            for w, nm in enumerate(names):
                L.addAmplitude(nm, data[w])
            L.finishInit()
            F.append(moment_features(names, data, diag, precision))
            del data
            bins.append((L, vt, fl, n))
        M = pwaMultibin()
        M.setOptions(startGroup=8, gtolRel=gtolRel, maxIter=maxIter)
        for L, _, _, _ in bins:
            M.addBin(L, 1)
        x0 = np.stack([start_from_truth(L, vt, fl, n, diag) for L, vt, fl, n in bins])
        res = M.fit(x0)
        for k, (L, vt, fl, n) in enumerate(bins):
            Y.append(targets_from_params(L, res["x"][k], n))
            VT.append(vt)
        del M, bins
    return np.stack(F), np.stack(Y), np.stack(VT)


def synth_true(n_waves, rng):
    v = rng.standard_normal(n_waves) + 1j * rng.standard_normal(n_waves)
    return v, float(abs(rng.standard_normal()))


def augment_phases(F, Y, n_waves, copies, rng):
    """Training-set augmentation by per-wave phase rotations.

    When the phase-space amplitudes of each wave are distributed invariantly
    under a phase rotation, rotating wave w by theta_w maps a bin's moments
    to M_ij exp(i (theta_i - theta_j)) and its minimum to
    V_w exp(i (theta_0 - theta_w)) (the first wave stays real, the flat wave
    is unchanged).  Returns the original rows followed by `copies` rotated
    copies of each."""
    n = n_waves + 1
    F = np.asarray(F, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    M = (F[:, :n * n] + 1j * F[:, n * n:2 * n * n]).reshape(-1, n, n)
    v = Y[:, :n] + 1j * Y[:, n:2 * n]
    outF, outY = [F], [Y]
    for _ in range(copies):
        th = np.zeros((len(F), n))
        th[:, :n_waves] = rng.uniform(0, 2 * np.pi, (len(F), n_waves))
        e = np.exp(1j * th)
        M2 = M * e[:, :, None] * np.conj(e)[:, None, :]
        rot = np.exp(1j * (th[:, :1] - th))
        rot[:, -1] = 1.0
        v2 = v * rot
        outF.append(np.concatenate([M2.real.reshape(len(F), -1), M2.imag.reshape(len(F), -1), F[:, 2 * n * n:]],
                                   axis=1))
        outY.append(np.concatenate([v2.real, v2.imag], axis=1))
    return np.concatenate(outF).astype(np.float32), np.concatenate(outY).astype(np.float32)
