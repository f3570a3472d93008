"""GPU tests of the warm-start network and of what it gains.

The network's kernels (BF16 operands, FP32 accumulation) must reproduce the
NumPy restatement in oracle/mlp_oracle.py, which rounds at the same points:
loss within 1e-4 relative, gradient within 1e-2 normwise (a BF16 rounding of
an FP32 sum can fall on the other side of a tie than the FP64 sum's).  A
network trained on fitted bins must then give start points from which the
plain fit reaches the bins' minima in far fewer iterations than from random
start points."""
import numpy as np
import pytest

import rootpwa_gb300 as R
from rootpwa_gb300 import synth
from rootpwa_gb300 import warmstart as WS
from oracle import mlp_oracle as MO
import helpers

pytestmark = pytest.mark.gpu


# batches of 33 and 300 rows: one and three 128-row tiles of the tensor-core
# GEMM (and K of 33 / 300 in the weight-gradient products dY^T X)
@pytest.mark.parametrize("shape,B", [((37, 64, 48, 10), 33), ((37, 64, 48, 10), 300), ((5203, 512, 512, 102), 64)])
def test_mlp_gradient_matches_oracle(shape, B):
    rng = np.random.default_rng(1)
    net = R.pwaMLP(*shape, seed=3)
    p = net.params()
    assert p.size == net.nmbParams()
    X = rng.standard_normal((B, shape[0])).astype(np.float32)
    T = rng.standard_normal((B, shape[3])).astype(np.float32)
    loss, g = net.gradient(X, T)
    l0, g0 = MO.loss_and_gradient(p, shape, X, T)
    assert abs(loss - l0) <= 1e-4 * l0
    assert helpers.normwise(g, g0) < 1e-2
    Y = net.forward(X)
    Y0 = MO.forward(p, shape, X)
    assert np.max(np.abs(Y - Y0)) <= 1e-2 * np.max(np.abs(Y0))


def test_training_reduces_loss():
    rng = np.random.default_rng(2)
    A = rng.standard_normal((20, 6))
    X = rng.standard_normal((2048, 20)).astype(np.float32)
    T = np.tanh(X @ A).astype(np.float32)
    net = R.pwaMLP(20, 64, 64, 6, seed=1)
    hist = net.train(X, T, batch=128, epochs=100, lr=3e-3)
    assert hist[-1] < 0.05 * hist[0]


def _bins(n_bins, names, model, norm, acc, rng, seed0, lo=2000, hi=8000):
    out = []
    for b in range(n_bins):
        n = int(rng.integers(lo, hi))
        vt, fl = synth.true_production_amplitudes(len(names), rng)
        data = synth.draw_bin_device(model, vt, fl, n, seed=seed0 + b)
        L = R.pwaLikelihood()
        L.init(names, [1] * len(names), None, 1, 0.0)
        L.addNormIntegral(R.ampIntegralMatrix(norm))
        L.addAccIntegral(R.ampIntegralMatrix(acc))
        for k, nm in enumerate(names):
            L.addAmplitude(nm, data[k])
        L.finishInit()
        out.append(dict(L=L, n=n, vt=vt, flat=fl, data=data))
    return out


def test_warm_start_gains_over_random_starts():
    torch = pytest.importorskip("torch")
    names, _ = synth.wave_names(0, 8)
    rng = np.random.default_rng(7)
    model = synth.AmplitudeModel(8, 0, np.random.Generator(np.random.PCG64(5)))
    mc = synth.draw_device(model, 40000, seed=99)
    norm = R.ampIntegralMatrix()
    norm.integrate(names, mc, precision="tf32x3")
    acc = R.ampIntegralMatrix()
    acc.integrate(names, mc, inBin=(torch.rand(40000, device="cuda") < 0.6).cpu().numpy(), precision="tf32x3")
    diag = np.real(np.diag(norm.matrix())) / norm.nmbEvents()

    def features(bins):
        F = np.stack([WS.moment_features(names, b["data"], diag) for b in bins])
        # the batched, allocation-free path gives the same features
        Fb = WS.moment_features_batch([b["data"] for b in bins], [diag] * len(bins))
        assert np.max(np.abs(Fb - F)) <= 1e-5 * np.max(np.abs(F))
        return F

    def fit(bins, x0, starts):
        M = R.pwaMultibin()
        M.setOptions(startGroup=8, gtolRel=1e-8, maxIter=2000)
        for b in bins:
            M.addBin(b["L"], starts)
        return M.fit(x0)

    train = _bins(400, names, model, norm, acc, rng, 1000)
    test = _bins(24, names, model, norm, acc, rng, 5000)
    # labels: minima reached from the true amplitudes
    x0 = np.stack([WS.start_from_truth(b["L"], b["vt"], b["flat"], b["n"], diag) for b in train])
    res = fit(train, x0, 1)
    Y = np.stack([WS.targets_from_params(b["L"], res["x"][k], b["n"]) for k, b in enumerate(train)])
    F, Y = WS.augment_phases(features(train), Y, len(names), 64, np.random.default_rng(1))
    net = R.pwaMLP(F.shape[1], 128, 128, Y.shape[1], seed=4)
    net.fit_standardisation(F)
    hist = net.train(net.standardise(F), Y, batch=64, epochs=30, lr=1e-3)
    assert hist[-1] < 0.05 * hist[0]
    # test bins: warm start vs random starts
    Yp = net.forward(net.standardise(features(test)))
    xw = np.stack([WS.params_from_targets(b["L"], Yp[k], b["n"]) for k, b in enumerate(test)])
    warm = fit(test, xw, 1)
    S = 8
    xr = np.random.default_rng(9).standard_normal((len(test) * S, xw.shape[1]))
    rand = fit(test, xr, S)
    best = rand["f"].reshape(len(test), S).min(axis=1)
    # the single warm start reaches the best minimum of 8 random starts
    same = np.abs(warm["f"] - best) <= 1e-6 * np.abs(best)
    assert same.mean() >= 0.9, same
    # its start point is much closer to that minimum than random points
    d_w = np.linalg.norm(xw - warm["x"], axis=1) / np.linalg.norm(warm["x"], axis=1)
    d_r = np.linalg.norm(xr - rand["x"], axis=1) / np.linalg.norm(rand["x"], axis=1)
    assert np.median(d_w) < 0.5 * np.median(d_r), (np.median(d_w), np.median(d_r))
    # fewer iterations per start, and far fewer in total than the multi-start
    it_w, it_r = np.median(warm["iterations"]), np.median(rand["iterations"])
    assert it_w < 0.8 * it_r, (it_w, it_r)
    assert warm["iterations"].sum() < 0.2 * rand["iterations"].sum()
