"""GPU parity of the fused FdF / DoEval / Gradient kernels against the FP64
oracle (partialWaveFit/pwaLikelihood.cc:170-636).

Tolerances (FP32 contraction, FP64 cross-tile and cross-block reductions):
function value relative 1e-6, gradient max-abs error relative to the largest
gradient component 1e-6."""
import os

import numpy as np
import pytest

import rootpwa_gb300 as R
from rootpwa_gb300 import synth
import helpers
from helpers import F_RTOL, G_NORMWISE, normwise, rel

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def pair(w, **kw):
    """Oracle and GPU likelihoods on identical integrals (the oracle's)."""
    norm, acc, gn, ga = helpers.integral_pairs(w)
    O = helpers.build_oracle(w, norm, acc, **kw)
    G = helpers.build_gpu(w, gn, ga, **kw)
    return O, G


def check_point(O, G, p, frtol=F_RTOL, gtol=G_NORMWISE):
    f0, g0 = O.FdF(p)
    f1, g1 = G.FdF(p)
    assert rel(f1, f0) < frtol, (f1, f0)
    assert normwise(g1, g0) < gtol, normwise(g1, g0)
    return f0, g0, f1, g1


def _golden_gpu(fixture, spec):
    gold = np.load(os.path.join(GOLDEN, fixture))
    w = synth.make_workload(**spec)
    gn = R.ampIntegralMatrix()
    gn.setWaveNames(w["names"])
    gn.setMatrix(gold["norm_raw"])
    gn.setNmbEvents(int(gold["norm_n"]))
    ga = R.ampIntegralMatrix()
    ga.setWaveNames(w["names"])
    ga.setMatrix(gold["acc_raw"])
    ga.setNmbEvents(int(gold["acc_n"]))
    return gold, w, helpers.build_gpu(w, gn, ga)


@pytest.mark.parametrize("source", ["ref", "oracle"])
def test_golden_compass15(source):
    """The single-bin config at full size (20,000 events, 15 waves) against
    fixtures written by the reference's own code (ref_*, make_ref_golden.py)
    and by the oracle (oracle_*): value, DoEval, gradient, Hessian, and the
    GPU integrals of the same MC events against the fixture's raw sums."""
    from golden.make_ref_golden import GOLDEN_WORKLOADS
    gold, w, G = _golden_gpu("%s_compass15_seed0.npz" % source, GOLDEN_WORKLOADS["compass15_seed0"])
    f, g = G.FdF(w["par"])
    assert rel(f, float(gold["f"])) < F_RTOL
    assert normwise(g, gold["grad"]) < G_NORMWISE
    assert rel(G.DoEval(w["par"]), float(gold["doeval"])) < F_RTOL
    if "tot_acc" in gold:
        assert G.totAcc() == pytest.approx(float(gold["tot_acc"]), rel=1e-15)
    H = G.Hessian(w["par"])
    assert np.max(np.abs(H - gold["hessian"])) < 1e-5 * np.max(np.abs(gold["hessian"]))
    gn, ga = helpers.gpu_integrals(w, precision="fp64")
    assert gn.nmbEvents() == int(gold["norm_n"]) and ga.nmbEvents() == int(gold["acc_n"])
    for m, key in ((gn, "norm_raw"), (ga, "acc_raw")):
        assert np.max(np.abs(m.matrix() - gold[key])) < 1e-12 * np.max(np.abs(gold[key]))


@pytest.mark.parametrize("source", ["ref", "oracle"])
def test_golden_compass88_small(source):
    """The production shape (7 + 80 waves, rank 2, 341 parameters) against the
    reference-made and the oracle-made fixtures."""
    from golden.make_ref_golden import GOLDEN_WORKLOADS
    gold, w, G = _golden_gpu("%s_compass88_small_seed1.npz" % source, GOLDEN_WORKLOADS["compass88_small_seed1"])
    f, g = G.FdF(w["par"])
    assert rel(f, float(gold["f"])) < F_RTOL
    assert normwise(g, gold["grad"]) < G_NORMWISE


def stress_workload(n_neg, n_pos, rank, n_data, flat=None):
    names, refl = synth.wave_names(n_neg, n_pos)
    rng = np.random.default_rng(n_data + 31 * rank)
    model = synth.AmplitudeModel(n_neg + n_pos, 4, rng)
    w = dict(names=names, refl=refl, rank=rank, data=model.draw(rng, n_data), mc=model.draw(rng, 3000),
             accepted=rng.random(3000) < 0.6, par=rng.standard_normal(synth.n_pars(n_neg, n_pos, rank)))
    if flat is not None:
        w["par"][-1] = flat
    return w


@pytest.mark.parametrize("n_neg,n_pos,rank,n_data", [
    (0, 15, 1, 20_000),      # compass15 shape
    (7, 80, 2, 30_001),      # compass88 shape, ragged tail
    (7, 80, 2, 1),           # a single event
    (3, 5, 1, 127),          # less than one tile
    (2, 9, 3, 129),          # rank above the negative wave count
    (5, 0, 2, 1000),         # negative reflectivity only
    (1, 1, 1, 256),          # one wave per reflectivity
    (20, 120, 1, 4099),      # 140 waves -> 64-event tiles
    (10, 54, 4, 3000),       # rank 4
    (0, 200, 1, 2000),       # 200 waves
])
def test_shapes_against_oracle(n_neg, n_pos, rank, n_data):
    # a flat amplitude of order one keeps every L_i away from zero, so the
    # comparison measures the kernels and not the conditioning (see below)
    w = stress_workload(n_neg, n_pos, rank, n_data, flat=1.0)
    O, G = pair(w)
    stages = G.plan()[1]
    # every kernel variant the shape supports: one, two or four (rank <= 2,
    # 128-event tiles) events per lane in the coherent-sum phase, the
    # fused-gradient kernel (rank <= 2, 128-event tiles) and the narrow
    # kernel (one event per thread; rank 1 up to 16 waves, rank 2 up to 8)
    fused_ok = rank <= 2 and G.plan()[0] == 128 and n_neg <= 16 and 1 <= n_pos <= 104
    four_ok = rank <= 2 and G.plan()[0] == 128
    narrow_ok = G.plan()[0] == 128 and n_neg + n_pos <= {1: 16, 2: 8}.get(rank, 0)
    for ne in (1, 2, 3, 4, 5):
        if (ne == 3 and not fused_ok) or (ne == 4 and not four_ok) or (ne == 5 and not narrow_ok):
            with pytest.raises(R.PwaError):
                G.setPlan(stages, ne)
            continue
        G.setPlan(stages, ne)
        assert G.planVariant() == ne
        check_point(O, G, w["par"])
        # a second point on the same handle (no stale state)
        q = 0.5 * w["par"][::-1].copy()
        q[-1] = -0.8
        check_point(O, G, q)
        # value-only and gradient-only launches of the same variant agree bitwise
        f, g = G.FdF(q)
        assert G.DoEval(q) == f
        assert np.array_equal(G.Gradient(q), g)


def test_ill_conditioned_point():
    """200 waves, rank 1 and a flat amplitude of 0.034: the smallest L_i is
    1e-4 of the median, and the few events with small L_i dominate the
    gradient.  Rounding the normalised amplitudes and V to FP32 alone moves
    the gradient by 1.2e-6 of its largest component (FP64 emulation with
    FP32-rounded inputs), FP32 coherent sums by 4.8e-6; the stated tolerance
    for such points is 2e-5 on the gradient, 1e-6 on the value."""
    w = stress_workload(0, 200, 1, 2000)
    assert abs(w["par"][-1]) < 0.05
    O, G = pair(w)
    check_point(O, G, w["par"], frtol=1e-6, gtol=2e-5)


def test_doeval_gradient_doderivative_consistent():
    w = synth.make_workload("compass88", seed=3, n_data=9000, n_mc=4000)
    O, G = pair(w)
    p = w["par"]
    f, g = G.FdF(p)
    assert G.DoEval(p) == f           # same kernels, same order: bitwise
    assert np.array_equal(G.Gradient(p), g)
    assert G.DoDerivative(p, 5) == g[5]   # cached
    q = p * 1.01
    d = G.DoDerivative(q, 7)
    assert d == pytest.approx(O.Gradient(q)[7], rel=1e-5, abs=1e-6 * np.max(np.abs(g)))
    info = G.funcCallInfo(0)
    assert info["nmbCalls"] >= 2 and info["funcTime"] > 0
    import io
    buf = io.StringIO()
    G.printFuncInfo(buf)
    lines = buf.getvalue().splitlines()
    assert len(lines) == 5 and lines[0].startswith("FdF") and " calls," in lines[0]


def test_deterministic_and_batch():
    w = synth.make_workload("compass88", seed=4, n_data=20000, n_mc=4000)
    O, G = pair(w)
    p = w["par"]
    f1, g1 = G.FdF(p)
    f2, g2 = G.FdF(p)
    assert f1 == f2 and np.array_equal(g1, g2)
    pts = np.stack([p, 0.3 * p, -p, p + 0.1])
    fb, gb = G.FdFBatch(pts)
    for k in range(len(pts)):
        fk, gk = G.FdF(pts[k])
        assert fb[k] == fk and np.array_equal(gb[k], gk)


@pytest.mark.parametrize("mode", ["fp64", "kahan_fp32", "fp32"])
def test_reduction_modes(mode):
    """The three cross-tile reduction modes at 50,000 events: each within the
    engine's tolerances of the FP64 oracle and bitwise reproducible.  The
    compensated mode folds every tile, so its sums differ from the FP64
    mode's; here every block holds fewer than 64 tiles, so the FP64 mode (a
    fold every 64 tiles of the main kernel, 32 of the narrow one) and the
    plain FP32 mode (one fold after the last tile) fold at the same point and
    agree bitwise."""
    w = synth.make_workload("compass88", seed=5, n_data=50000, n_mc=4000)
    O, G = pair(w)
    G.setReduction(mode)
    check_point(O, G, w["par"])
    f1, g1 = G.FdF(w["par"])
    f2, g2 = G.FdF(w["par"])
    assert f1 == f2 and np.array_equal(g1, g2)
    if mode != "fp64":
        G.setReduction("fp64")
        f0, g0 = G.FdF(w["par"])
        same = f0 == f1 and np.array_equal(g0, g1)
        assert same == (mode == "fp32")


def test_options_prior_unnormalised_thresholds_override():
    w = synth.make_workload("compass15", seed=6, n_data=5000, n_mc=8000)
    th = np.zeros(15)
    th[3] = 2.5
    th[9] = 1.0
    kw = dict(use_normalized=False, prior=1, cauchy_width=0.7, thresholds=th, mass_bin_center=2.0,
              acc_override=12345)
    O, G = pair(w, **kw)
    assert [G.parameter(k)["fixed"] for k in range(G.nmbPars())] == [O.parFixed(k) for k in range(O.nmbPars())]
    check_point(O, G, w["par"])
    assert G.totAcc() == pytest.approx(O.totAcc(), rel=1e-15)


def test_zero_amplitude_wave_is_fixed():
    """addAmplitude fixes the parameters of an all-zero wave whose acceptance
    diagonal is zero (pwaLikelihood.cc:1300-1334)."""
    w = synth.make_workload("compass15", seed=8, n_data=2000, n_mc=3000)
    w["mc"][4] = 0
    w["data"][4] = 0
    O, G = pair(w)
    assert [G.parameter(k)["fixed"] for k in range(G.nmbPars())] == [O.parFixed(k) for k in range(O.nmbPars())]
    assert G.nmbParsFixed() == O.nmbParsFixed() == 2
    check_point(O, G, w["par"])


def test_complex128_host_and_device_input():
    torch = pytest.importorskip("torch")
    w = synth.make_workload("compass88", seed=9, n_data=7000, n_mc=3000)
    norm, acc, gn, ga = helpers.integral_pairs(w)
    gn2, ga2 = helpers.copy_oracle_integral_to_gpu(norm), helpers.copy_oracle_integral_to_gpu(acc)
    O = helpers.build_oracle(w, norm, acc)
    G64 = helpers.build_gpu(w, gn, ga, amps=w["data"].astype(np.complex128))
    dev = torch.from_numpy(w["data"]).cuda()
    Gd = helpers.build_gpu(w, gn2, ga2, amps=dev)
    f0, g0 = O.FdF(w["par"])
    for G in (G64, Gd):
        f, g = G.FdF(w["par"])
        assert rel(f, f0) < F_RTOL and normwise(g, g0) < G_NORMWISE


def test_device_resident_fdf_and_graph_capture():
    torch = pytest.importorskip("torch")
    w = synth.make_workload("compass88", seed=10, n_data=12000, n_mc=3000)
    O, G = pair(w)
    P = G.nmbPars()
    s = torch.cuda.Stream()
    G.setStream(s.cuda_stream)
    dpar = torch.from_numpy(w["par"]).cuda()
    dout = torch.zeros(P + 2, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    G.FdFDevice(dpar.data_ptr(), dout.data_ptr(), True, s.cuda_stream)
    s.synchronize()
    f0, g0 = O.FdF(w["par"])
    out = dout.cpu().numpy()
    assert out[P + 1] == 0.0
    assert rel(out[0], f0) < F_RTOL and normwise(out[1:P + 1], g0) < G_NORMWISE
    # the same two launches captured in a CUDA graph and replayed
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        G.FdFDevice(dpar.data_ptr(), dout.data_ptr(), True, s.cuda_stream)
    dout.zero_()
    dpar.mul_(0.5)
    graph.replay()
    torch.cuda.synchronize()
    f1, g1 = O.FdF(0.5 * w["par"])
    out = dout.cpu().numpy()
    assert rel(out[0], f1) < F_RTOL and normwise(out[1:P + 1], g1) < G_NORMWISE


def test_error_paths_on_gpu():
    w = synth.make_workload("compass15", seed=12, n_data=300, n_mc=600)
    norm, acc = helpers.oracle_integrals(w)
    G = R.pwaLikelihood()
    G.init(w["names"], w["refl"], None, 1, 0.0)
    G.addNormIntegral(helpers.copy_oracle_integral_to_gpu(norm))
    G.addAccIntegral(helpers.copy_oracle_integral_to_gpu(acc))
    G.addAmplitude(w["names"][0], w["data"][0])
    with pytest.raises(R.PwaError):
        G.addAmplitude(w["names"][1], w["data"][1][:100])   # size mismatch
    with pytest.raises(R.PwaError):
        G.addAmplitude("not_a_wave", w["data"][1])
    with pytest.raises(R.PwaError) as e:
        G.finishInit()                                        # waves missing
    assert e.value.status == 2


def test_autotuned_plan_matches_oracle():
    """finishInit times the compiled tile/pipeline plans (>= 65536 events) and
    keeps the fastest; any plan it picks must give the oracle's FdF."""
    w = synth.make_workload("compass88", seed=13, n_data=70_001, n_mc=3000)
    O, G = pair(w)
    E, stages, blocks = G.plan()
    assert E in (64, 128) and 2 <= stages <= 4 and blocks >= 1
    check_point(O, G, w["par"])
    G2 = helpers.build_gpu(w, *helpers.integral_pairs(w)[2:])
    assert G2.plan() == (E, stages, blocks)   # cached per shape


def test_zero_intensity_event_gives_non_finite_value():
    """An event with all amplitudes zero and a zero flat amplitude has L_i = 0.
    The reference's compensated sum turns the -log 0 = inf sample into NaN on
    the next addition (c = (inf - s) - inf), and its gradient is NaN
    (-(2/0) * 0).  The engine must report a non-finite value and gradient as
    well (it keeps +inf), not wrap around in its fixed-point sums."""
    w = synth.make_workload("compass15", seed=14, n_data=3000, n_mc=3000)
    w["data"][:, 17] = 0
    O, G = pair(w)
    p = w["par"].copy()
    p[-1] = 0.0
    f0, g0 = O.FdF(p)
    f1, g1 = G.FdF(p)
    assert not np.isfinite(f0) and not np.isfinite(f1)
    assert np.array_equal(np.isfinite(g1), np.isfinite(g0))


@pytest.mark.parametrize("use_normalized,prior", [(True, 0), (False, 0), (True, 1)])
def test_event_shards_sum_to_full_fdf(use_normalized, prior):
    """pwa_likelihood_set_shard: two shard likelihoods over contiguous halves
    of the events sum to the full FdF (FP32 contractions: 1e-6 / 1e-5)."""
    from rootpwa_gb300.sharded import shard_range
    w = synth.make_workload("compass15", seed=4, n_data=20001, n_mc=5000)
    norm, acc = helpers.gpu_integrals(w)
    full = helpers.build_gpu(w, R.ampIntegralMatrix(norm), R.ampIntegralMatrix(acc), use_normalized=use_normalized,
                             prior=prior)
    N = w["data"].shape[1]
    f, g = 0.0, 0.0
    for k in range(2):
        b, e = shard_range(N, k, 2)
        L = R.pwaLikelihood()
        L.useNormalizedAmps(use_normalized)
        if prior:
            L.setPriorType(prior)
        L.setShard(N, k == 0)
        L.init(w["names"], w["refl"], None, w["rank"], 0.0)
        L.addNormIntegral(R.ampIntegralMatrix(norm))
        L.addAccIntegral(R.ampIntegralMatrix(acc))
        for j, n in enumerate(w["names"]):
            L.addAmplitude(n, np.ascontiguousarray(w["data"][j, b:e]))
        L.finishInit()
        fk, gk = L.FdF(w["par"])
        f, g = f + fk, g + gk
    f0, g0 = full.FdF(w["par"])
    assert helpers.rel(f, f0) < 1e-6
    assert helpers.normwise(g, g0) < 1e-5


def test_store_block_64_matches_oracle():
    """The 64-event store/tile layout (chosen automatically for wide wave
    sets, or by setStoreBlock) gives the same FdF as the oracle."""
    w = stress_workload(7, 80, 2, 30_001, flat=1.0)
    norm, acc, gn, ga = helpers.integral_pairs(w)
    O = helpers.build_oracle(w, norm, acc)
    G = R.pwaLikelihood()
    G.setStoreBlock(64)
    G.init(w["names"], w["refl"], None, w["rank"], 0.0)
    G.addNormIntegral(gn)
    G.addAccIntegral(ga)
    for k, n in enumerate(w["names"]):
        G.addAmplitude(n, w["data"][k])
    G.finishInit()
    assert G.plan()[0] == 64
    check_point(O, G, w["par"])
    with pytest.raises(R.PwaError):
        G.setStoreBlock(128)  # fixed by the first addAmplitude


def test_dlcache_and_clear():
    """dLcache (pwaLikelihood.h:200) holds the last gradient; clear
    (pwaLikelihood.cc:1670-1674) releases the amplitude store and evaluation
    is refused afterwards."""
    w = synth.make_workload("compass15", seed=3, n_data=5000, n_mc=20000)
    O, G = pair(w)
    f, g = G.FdF(w["par"])
    assert [G.dLcache(i) for i in range(G.nmbPars())] == list(g)
    assert G.ncalls() >= 1
    G.clear()
    with pytest.raises(R.PwaError) as e:
        G.FdF(w["par"])
    assert e.value.status == 2
