"""CPU tests of the FP64 oracle: the reference's ASCII integral fixture,
analytic identities of the likelihood, finite differences, hand-computed
cases and the committed golden values."""
import os

import numpy as np
import pytest

from oracle.oracle import OracleIntegral, OracleLikelihood
from rootpwa_gb300 import synth
import helpers

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def split_ascii(text):
    """(header + matrix lines, set of 'name index' lines) of an ASCII integral."""
    lines = text.split("\n")
    n = int(lines[0])
    head = lines[:3 + n]
    return "\n".join(head), set(x for x in lines[4 + n:] if x), lines[3 + n]


def test_reference_integral_fixture_round_trip(tmp_path):
    """readAscii/writeAscii (ampIntegralMatrix.cc:503-570) reproduce the
    reference's fixture: matrix section byte for byte, wave-name map as a
    set (the fixture lists it sorted by name, the writer by index)."""
    src = os.path.join(GOLDEN, "testIntegral.int")
    I = OracleIntegral()
    assert I.read_ascii(src)
    assert I.nmb_waves() == 41 and I.nmb_events() == 20000
    out = tmp_path / "rt.int"
    assert I.write_ascii(str(out))
    assert split_ascii(out.read_text()) == split_ascii(open(src).read())


def test_reference_integral_fixture_is_hermitian():
    I = OracleIntegral()
    assert I.read_ascii(os.path.join(GOLDEN, "testIntegral.int"))
    m = I.raw()
    assert np.allclose(m, m.conj().T, rtol=1e-12, atol=1e-9 * np.max(np.abs(m)))
    assert np.all(np.real(np.diag(m)) > 0)
    # element() divides by the event count (ampIntegralMatrix.cc:238-252)
    assert I.element(3, 5) == pytest.approx(m[3, 5] / 20000, rel=1e-15)


def test_integrate_matches_numpy():
    rng = np.random.default_rng(3)
    A = (rng.standard_normal((6, 500)) + 1j * rng.standard_normal((6, 500)))
    I = OracleIntegral()
    names = ["w%d" % k for k in range(6)]
    assert I.integrate(names, A)
    ref = A @ A.conj().T
    assert np.allclose(I.raw(), ref, rtol=1e-13, atol=1e-10)
    assert I.nmb_events() == 500


def test_integrate_weights_bins_subamps():
    """weights 1/w, renormalised by their mean over selected events; weight
    stream consumed by selected events only (ampIntegralMatrix.cc:408-483)."""
    rng = np.random.default_rng(4)
    A = rng.standard_normal((4, 300, 2)) + 1j * rng.standard_normal((4, 300, 2))
    sel = rng.random(300) < 0.5
    w = rng.uniform(0.5, 2.0, sel.sum())
    I = OracleIntegral()
    assert I.integrate(["a", "b", "c", "d"], A, weights=w, in_bin=sel, max_nmb_events=250)
    keep = np.nonzero(sel[:250])[0]
    ws = 1.0 / w[:len(keep)]
    ref = np.einsum("ies,jes,e->ij", A[:, keep], A[:, keep].conj(), ws)
    ref *= 1.0 / (ws.sum() / len(keep))
    assert I.nmb_events() == len(keep)
    assert np.allclose(I.raw(), ref, rtol=1e-12)


def test_add_event_and_iadd():
    rng = np.random.default_rng(5)
    A = rng.standard_normal((3, 20)) + 1j * rng.standard_normal((3, 20))
    names = ["x", "y", "z"]
    I = OracleIntegral()
    assert I.set_wave_names(names)
    for e in range(20):
        I.add_event(A[:, e])
    J = OracleIntegral()
    assert J.integrate(names, A)
    assert np.allclose(I.raw(), J.raw(), rtol=1e-13)
    I += J
    assert I.nmb_events() == 40
    assert np.allclose(I.raw(), 2 * J.raw(), rtol=1e-13)


def _tiny():
    """N = 1 event, one wave, rank 1: everything by hand."""
    a = 0.7 - 0.4j
    names, refl = ["w"], [1]
    norm = OracleIntegral()
    assert norm.integrate(names, np.array([[1.5 + 0.5j, -0.3 + 1.0j]]))
    acc = OracleIntegral()
    assert acc.integrate(names, np.array([[1.5 + 0.5j]]))
    L = OracleLikelihood(use_normalized_amps=True)
    assert L.init(names, refl, None, 1, 0.0)
    assert L.addNormIntegral(norm) and L.addAccIntegral(acc) and L.addAmplitude("w", np.array([a]))
    assert L.finishInit()
    return L, a


def test_hand_computed_single_event():
    L, a = _tiny()
    n_ww = (abs(1.5 + 0.5j) ** 2 + abs(-0.3 + 1.0j) ** 2) / 2  # element = raw / nmbEvents
    acc_ww = abs(1.5 + 0.5j) ** 2 / 2                         # acc nmbEvents set to 2 generated
    tot_acc = 1 / 2
    an = a / np.sqrt(n_ww)
    acc_n = acc_ww / n_ww
    v, flat = 0.9, 0.6
    Li = abs(v * an) ** 2 + flat ** 2
    f_ref = -np.log(Li) + (v * v * acc_n + flat ** 2 * tot_acc)
    f, g = L.FdF(np.array([v, flat]))
    assert f == pytest.approx(f_ref, rel=1e-14)
    dv = -2 / Li * (v * abs(an) ** 2) + 2 * v * acc_n
    dflat = -2 / Li * flat + 2 * flat * tot_acc
    assert g == pytest.approx([dv, dflat], rel=1e-13)
    assert L.totAcc() == pytest.approx(0.5)


@pytest.fixture(scope="module")
def small():
    w = synth.make_workload("compass88", seed=7, n_data=700, n_mc=1500, rank=2)
    L = helpers.build_oracle(w)
    return w, L


def test_fdf_equals_doeval_and_gradient(small):
    """FdF = (DoEval, Gradient) to the last bit (same summation order)."""
    w, L = small
    f, g = L.FdF(w["par"])
    assert f == L.DoEval(w["par"])
    assert np.array_equal(g, L.Gradient(w["par"]))


def test_gradient_finite_differences(small):
    w, L = small
    p = w["par"].copy()
    g = L.Gradient(p)
    for k in list(range(0, len(p), 17)) + [len(p) - 1]:
        h = 1e-5 * max(1.0, abs(p[k]))
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (L.DoEval(pp) - L.DoEval(pm)) / (2 * h)
        assert fd == pytest.approx(g[k], rel=1e-6, abs=1e-6 * np.max(np.abs(g)))


def test_hessian_finite_differences():
    w = synth.make_workload("compass15", seed=2, n_data=400, n_mc=900)
    L = helpers.build_oracle(w)
    p = w["par"]
    H = L.Hessian(p)
    assert np.allclose(H, H.T, rtol=1e-10, atol=1e-8 * np.max(np.abs(H)))
    for k in (0, 3, 8, len(p) - 1):
        h = 1e-5 * max(1.0, abs(p[k]))
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        col = (L.Gradient(pp) - L.Gradient(pm)) / (2 * h)
        assert np.allclose(H[:, k], col, rtol=1e-5, atol=1e-6 * np.max(np.abs(H)))


def test_threaded_restatement_matches_single_thread(small):
    w, L = small
    f1, g1 = L.FdF(w["par"], threads=1)
    f4, g4 = L.FdF(w["par"], threads=4)
    assert f4 == pytest.approx(f1, rel=1e-13)
    assert np.allclose(g4, g1, rtol=1e-11, atol=1e-11 * np.max(np.abs(g1)))


def test_normalisation_identity(small):
    """Scaling all amplitudes by c scales every L_i by c^2 and the
    normalisation by c^2 (doc/tex/likelihood.tex eq. 1):
    f(cV) = f(V) - 2 N ln c + (c^2 - 1) N(V).  N(V) from two scalings must
    equal sum Re(V_a conj(V_b) I_ab) + V_flat^2 eta_tot built from the
    likelihood's own (normalised) acceptance matrix."""
    w, L = small
    p = w["par"]
    n = len(w["data"][0])
    f1, f2, f3 = L.DoEval(p), L.DoEval(2 * p), L.DoEval(3 * p)
    n2 = (f2 - f1 + 2 * n * np.log(2.0)) / 3
    n3 = (f3 - f1 + 2 * n * np.log(3.0)) / 8
    assert n2 == pytest.approx(n3, rel=1e-9)
    _, acc, _ = L.integralMatrices(with_flat=False)
    V = _prod_amps(w, p)
    direct = 0.0
    for r in range(w["rank"]):
        v = V[r]
        direct += np.real(v @ acc @ v.conj())
    direct += p[-1] ** 2 * L.totAcc()
    assert n2 == pytest.approx(direct, rel=1e-9)


def _prod_amps(w, p):
    """V[rank][wave] from the reference parameter layout (pwaLikelihood.cc:1682-1710)."""
    nw = len(w["names"])
    counts = [w["refl"].count(-1), w["refl"].count(1)]
    V = np.zeros((w["rank"], nw), dtype=np.complex128)
    k = 0
    for r in range(w["rank"]):
        off = 0
        for e in (0, 1):
            for i in range(counts[e]):
                if i < r:
                    pass
                elif i == r:
                    V[r, off + i] = p[k]
                    k += 1
                else:
                    V[r, off + i] = p[k] + 1j * p[k + 1]
                    k += 2
            off += counts[e]
    assert k == len(p) - 1
    return V


def test_correct_param_signs(small):
    w, L = small
    p = w["par"].copy()
    p[0] = -abs(p[0])        # anchor of rank 0, negative reflectivity
    p[-1] = -abs(p[-1])      # flat
    q = L.CorrectParamSigns(p)
    assert q[-1] == abs(p[-1])
    assert q[0] == -p[0]
    # flipping all amplitudes of a (rank, reflectivity) block leaves f unchanged
    assert L.DoEval(q) == pytest.approx(L.DoEval(p), rel=1e-12)


@pytest.mark.parametrize("name", sorted(f[len("oracle_"):-4] for f in os.listdir(GOLDEN) if f.startswith("oracle_")))
def test_oracle_matches_golden(name):
    from golden.make_golden import GOLDEN_WORKLOADS, checksum
    gold = np.load(os.path.join(GOLDEN, "oracle_%s.npz" % name))
    w = synth.make_workload(**GOLDEN_WORKLOADS[name])
    assert np.allclose(checksum(w), gold["checksum"], rtol=1e-12), "synthetic input streams changed"
    norm, acc = helpers.oracle_integrals(w)
    assert np.array_equal(norm.raw(), gold["norm_raw"])
    assert np.array_equal(acc.raw(), gold["acc_raw"])
    L = helpers.build_oracle(w, norm, acc)
    f, g = L.FdF(w["par"])
    assert f == gold["f"]
    assert np.array_equal(g, gold["grad"])
    if "hessian" in gold:
        assert np.array_equal(L.Hessian(w["par"]), gold["hessian"])


@pytest.mark.parametrize("name,rank,seed", [("compass15", 1, 3), ("compass88", 2, 4), ("compass88", 3, 5)])
def test_independent_numpy_restatement_of_the_value(name, rank, seed):
    """A second, independent restatement of the extended likelihood in numpy
    (pwaLikelihood.cc:209-276 with the normalisation of :1253-1260 and
    :1311-1334, nEvt = 1) gives the oracle's value to 1e-12: the event term
    -sum ln(sum_r sum_e |sum_{w in e} V_rw A_w / sqrt(N_ww)|^2 + V_flat^2) and
    sum_r sum_e sum_ij Re(V_ri conj(V_rj) I_ij / sqrt(N_ii N_jj)) +
    V_flat^2 eta over same-reflectivity blocks."""
    w = synth.make_workload(name, seed=seed, n_data=600, n_mc=1200, rank=rank)
    norm, acc = helpers.oracle_integrals(w)
    n_gen = norm.nmb_events()
    n_acc = acc.nmb_events()
    N = norm.matrix()
    I_acc = acc.raw() / float(n_gen)       # addAccIntegral sets the count to the generated events
    eta = n_acc / float(n_gen)
    L = helpers.build_oracle(w, norm, acc)
    p = w["par"]
    V = _prod_amps(w, p)                   # [rank][wave], reference layout
    refl = np.array(w["refl"])
    d = np.sqrt(np.real(np.diag(N)))
    A = w["data"].astype(np.complex128) / d[:, None]
    Ihat = I_acc / np.outer(d, d)
    flat = p[-1]
    intensity = np.full(A.shape[1], flat * flat)
    norm_term = flat * flat * eta
    for r in range(w["rank"]):
        for e in (-1, 1):
            m = refl == e
            if not m.any():
                continue
            S = V[r, m] @ A[m]
            intensity += np.abs(S) ** 2
            Ie = Ihat[np.ix_(m, m)]
            norm_term += np.real(V[r, m] @ Ie @ V[r, m].conj())
    f_np = -np.sum(np.log(intensity)) + norm_term
    assert L.DoEval(p) == pytest.approx(f_np, rel=1e-12)
