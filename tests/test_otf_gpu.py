"""On-the-fly binning on the GPU (pwaLikelihood.cc:1391-1440): the selection
kernels keep the events of a whole data file with lower <= x < upper for
every binning variable (NaN kept, as in the reference's rejection test), in
file order.  The likelihood of the whole file with the selection must equal
the likelihood of the pre-selected events bit for bit (same events, same
order, same kernels), for host and device inputs, and agree with the
oracle's on-the-fly binning within the FdF tolerances."""
import numpy as np
import pytest

import rootpwa_gb300 as R
from rootpwa_gb300 import synth
import helpers
from helpers import F_RTOL, G_NORMWISE, normwise, rel
from oracle.oracle import OracleLikelihood

pytestmark = pytest.mark.gpu


def reference_mask(bounds, cols):
    keep = np.ones(len(next(iter(cols.values()))), dtype=bool)
    for k, (lo, hi) in bounds.items():
        x = cols[k]
        keep &= ~((x < lo) | (x >= hi))
    return keep


def file_columns(n, seed):
    rng = np.random.default_rng(seed)
    cols = {"mass": rng.uniform(1.0, 2.0, n), "tPrime": rng.exponential(0.3, n), "phi": rng.uniform(-3, 3, n)}
    cols["mass"][::97] = 1.4   # on the lower edge: kept
    cols["mass"][5::97] = 1.6  # on the upper edge: dropped
    cols["tPrime"][11] = np.nan
    cols["mass"][11] = 1.5
    bounds = {"mass": (1.4, 1.6), "tPrime": (0.1, 1.0), "phi": (-2.5, 2.9)}
    return cols, bounds


def gpu_otf(w, norm, acc, bounds, cols, amps):
    L = R.pwaLikelihood()
    L.init(w["names"], w["refl"], None, w["rank"], 0.0)
    L.addNormIntegral(helpers.copy_oracle_integral_to_gpu(norm))
    L.addAccIntegral(helpers.copy_oracle_integral_to_gpu(acc))
    L.setOnTheFlyBinning(bounds, cols)
    for k, name in enumerate(w["names"]):
        L.addAmplitude(name, amps[k])
    L.finishInit()
    return L


@pytest.mark.parametrize("n_data", [100, 3 * 4096 + 17, 200_003])
def test_otf_equals_preselected_host(n_data):
    w = synth.make_workload("compass15", seed=n_data % 7, n_data=n_data, n_mc=4000, rank=2)
    cols, bounds = file_columns(n_data, n_data)
    keep = reference_mask(bounds, cols)
    assert keep[11] and 0 < keep.sum() < n_data
    norm, acc = helpers.oracle_integrals(w)
    G = gpu_otf(w, norm, acc, bounds, cols, w["data"])
    assert G.otfSelected() == int(keep.sum())
    assert G.nmbEvents() == int(keep.sum())
    P = helpers.build_gpu(dict(w, data=w["data"][:, keep]), helpers.copy_oracle_integral_to_gpu(norm),
                          helpers.copy_oracle_integral_to_gpu(acc))
    f0, g0 = P.FdF(w["par"])
    f1, g1 = G.FdF(w["par"])
    assert f0 == f1
    assert np.array_equal(g0, g1)


def test_otf_device_inputs_and_oracle_parity():
    torch = pytest.importorskip("torch")
    n_data = 150_001
    w = synth.make_workload("compass15", seed=4, n_data=n_data, n_mc=5000, rank=1)
    cols, bounds = file_columns(n_data, 9)
    keep = reference_mask(bounds, cols)
    norm, acc = helpers.oracle_integrals(w)
    dcols = {k: torch.from_numpy(v).cuda() for k, v in cols.items()}
    damps = [torch.from_numpy(np.ascontiguousarray(w["data"][k])).cuda() for k in range(len(w["names"]))]
    G = gpu_otf(w, norm, acc, bounds, dcols, damps)
    H = gpu_otf(w, norm, acc, bounds, cols, w["data"])
    assert G.otfSelected() == int(keep.sum())
    f0, g0 = H.FdF(w["par"])
    f1, g1 = G.FdF(w["par"])
    assert f0 == f1 and np.array_equal(g0, g1)
    # the oracle's on-the-fly binning of the same file
    O = OracleLikelihood()
    assert O.init(w["names"], w["refl"], None, w["rank"], 0.0)
    assert O.addNormIntegral(norm) and O.addAccIntegral(acc)
    assert O.setOnTheFlyBinning(bounds, cols)
    for k, name in enumerate(w["names"]):
        assert O.addAmplitude(name, w["data"][k].astype(np.complex128))
    assert O.finishInit()
    assert O.otfSelected() == G.otfSelected()
    fo, go = O.FdF(w["par"])
    assert rel(f1, fo) < F_RTOL
    assert normwise(g1, go) < G_NORMWISE


def test_otf_errors():
    w = synth.make_workload("compass15", seed=1, n_data=5000, n_mc=3000, rank=1)
    cols, bounds = file_columns(5000, 2)
    norm, acc = helpers.oracle_integrals(w)

    def fresh():
        L = R.pwaLikelihood()
        L.init(w["names"], w["refl"], None, w["rank"], 0.0)
        L.addNormIntegral(helpers.copy_oracle_integral_to_gpu(norm))
        L.addAccIntegral(helpers.copy_oracle_integral_to_gpu(acc))
        return L

    L = fresh()
    L.setOnTheFlyBinning(bounds, cols)
    with pytest.raises(R.PwaError):
        L.addAmplitude(w["names"][0], w["data"][0][:-1])  # not the file's length
    L = fresh()
    L.setOnTheFlyBinning({"mass": (5.0, 6.0)}, cols)  # empty bin
    assert L.otfSelected() == 0
    with pytest.raises(R.PwaError):
        L.addAmplitude(w["names"][0], w["data"][0])
    L = fresh()
    L.addAmplitude(w["names"][0], w["data"][0])
    with pytest.raises(R.PwaError):
        L.setOnTheFlyBinning(bounds, cols)  # after the first amplitude


def test_amplitude_files_with_binning(tmp_path):
    """Two amplitude files (ragged sizes, waves stored in another order and
    one extra wave) loaded with on-the-fly binning equal the pre-selected
    arrays bit for bit; without binning they equal the whole arrays."""
    n1, n2 = 70_001, 4096 * 5 + 3
    w = synth.make_workload("compass15", seed=8, n_data=n1 + n2, n_mc=4000, rank=2)
    cols, bounds = file_columns(n1 + n2, 13)
    keep = reference_mask(bounds, cols)
    norm, acc = helpers.oracle_integrals(w)
    names = list(w["names"])
    order = list(reversed(range(len(names))))
    extra = np.ones((1, n1 + n2), np.complex64)
    paths = []
    for k, sl in enumerate([slice(0, n1), slice(n1, n1 + n2)]):
        p = tmp_path / ("f%d.amp" % k)
        amps = np.concatenate([w["data"][order, sl], extra[:, sl]])
        R.writeAmplitudeFile(p, [names[i] for i in order] + ["not in the wave list"], amps,
                             {"phi": cols["phi"][sl], "tPrime": cols["tPrime"][sl], "mass": cols["mass"][sl]})
        paths.append(p)

    def loaded(boundaries):
        L = R.pwaLikelihood()
        L.init(w["names"], w["refl"], None, w["rank"], 0.0)
        L.addNormIntegral(helpers.copy_oracle_integral_to_gpu(norm))
        L.addAccIntegral(helpers.copy_oracle_integral_to_gpu(acc))
        L.loadAmplitudeFiles(paths, boundaries)
        L.finishInit()
        return L

    G = loaded(bounds)
    assert G.nmbEvents() == int(keep.sum())
    P = helpers.build_gpu(dict(w, data=w["data"][:, keep]), helpers.copy_oracle_integral_to_gpu(norm),
                          helpers.copy_oracle_integral_to_gpu(acc))
    f0, g0 = P.FdF(w["par"])
    f1, g1 = G.FdF(w["par"])
    assert f0 == f1 and np.array_equal(g0, g1)
    A = loaded(None)
    Q = helpers.build_gpu(w, helpers.copy_oracle_integral_to_gpu(norm), helpers.copy_oracle_integral_to_gpu(acc))
    f0, g0 = Q.FdF(w["par"])
    f1, g1 = A.FdF(w["par"])
    assert A.nmbEvents() == n1 + n2
    assert f0 == f1 and np.array_equal(g0, g1)
    # a binning variable or a wave that a file lacks
    with pytest.raises(R.PwaError):
        loaded({"energy": (0.0, 1.0)})
    R.writeAmplitudeFile(tmp_path / "short.amp", names[:-1], w["data"][:-1, :10])
    L = R.pwaLikelihood()
    L.init(w["names"], w["refl"], None, w["rank"], 0.0)
    L.addNormIntegral(helpers.copy_oracle_integral_to_gpu(norm))
    L.addAccIntegral(helpers.copy_oracle_integral_to_gpu(acc))
    with pytest.raises(R.PwaError):
        L.loadAmplitudeFiles([tmp_path / "short.amp"])
