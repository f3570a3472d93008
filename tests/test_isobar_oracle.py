"""Pins of the isobar-amplitude oracle (oracle/isobar_oracle.py): its
Clebsch-Gordan coefficients against sympy, its Wigner d functions against
the PDG closed forms and the group properties, its barrier factors against
the closed forms of F_1..F_3 (utilities/physUtils.hpp:200-262 quotes the same
functions), and its amplitudes against the symmetries the frames must have:
invariance under a rotation of the whole event, the reflectivity eigenvalue
under reflection through the production plane (isobarAmplitude.cc:188-203),
the parity eigenvalue under space inversion (:174-186) and Bose symmetry."""
import math

import numpy as np
import pytest

from oracle import isobar_oracle as O
from isobar_cases import SPECIES, events, waves


def test_clebsch_gordan_against_sympy():
    cg = pytest.importorskip("sympy.physics.quantum.cg")
    from sympy import Rational
    n = 0
    for j1 in range(0, 7):
        for j2 in range(0, 5):
            for J in range(abs(j1 - j2), j1 + j2 + 1, 2):
                for m1 in range(-j1, j1 + 1, 2):
                    for m2 in range(-j2, j2 + 1, 2):
                        if abs(m1 + m2) > J:
                            continue
                        ref = float(cg.CG(Rational(j1, 2), Rational(m1, 2), Rational(j2, 2), Rational(m2, 2),
                                          Rational(J, 2), Rational(m1 + m2, 2)).doit())
                        assert abs(O.clebsch_gordan(j1, m1, j2, m2, J, m1 + m2) - ref) < 1e-13
                        n += 1
    assert n > 1000
    # selection rules give exact zeros
    assert O.clebsch_gordan(2, 0, 2, 0, 2, 0) == 0.0          # (1 0 1 0 | 1 0)
    assert O.clebsch_gordan(2, 2, 2, 0, 2, 0) == 0.0          # M != m1 + m2


@pytest.mark.parametrize("theta", [0.0, 0.3, 1.2, 2.5, math.pi])
def test_wigner_d_closed_forms(theta):
    c, s = math.cos(theta), math.sin(theta)
    table = {  # PDG: Clebsch-Gordan coefficients, spherical harmonics and d functions
        (1, 1, 1): math.cos(theta / 2), (1, 1, -1): -math.sin(theta / 2),
        (2, 2, 2): (1 + c) / 2, (2, 2, 0): -s / math.sqrt(2), (2, 2, -2): (1 - c) / 2, (2, 0, 0): c,
        (4, 4, 4): ((1 + c) / 2) ** 2, (4, 4, 2): -(1 + c) * s / 2, (4, 4, 0): math.sqrt(6) / 4 * s * s,
        (4, 2, 2): (1 + c) * (2 * c - 1) / 2, (4, 2, 0): -math.sqrt(1.5) * s * c, (4, 0, 0): 1.5 * c * c - 0.5,
        (3, 3, 3): math.cos(theta / 2) ** 3, (3, 3, 1): -math.sqrt(3) * (1 + c) / 2 * math.sin(theta / 2),
        (6, 0, 0): (5 * c ** 3 - 3 * c) / 2,
    }
    for (j, m, n), v in table.items():
        assert abs(O.wigner_d(j, m, n, theta) - v) < 1e-14, (j, m, n)


@pytest.mark.parametrize("j", [1, 2, 3, 4, 6, 8])
def test_wigner_d_group_properties(j):
    ms = list(range(-j, j + 1, 2))
    a, b = 0.7, 1.9

    def mat(t):
        return np.array([[O.wigner_d(j, m, n, t) for n in ms] for m in ms])
    D = mat(a)
    assert np.allclose(D @ D.T, np.eye(len(ms)), atol=1e-13)             # orthogonal
    assert np.allclose(mat(a) @ mat(b), mat(a + b), atol=1e-13)          # d(a) d(b) = d(a + b)
    for i, m in enumerate(ms):
        for k, n in enumerate(ms):
            assert abs(D[i, k] - (-1) ** ((m - n) // 2) * D[k, i]) < 1e-14   # d_mn = (-1)^(m-n) d_nm
            assert abs(D[i, k] - D[len(ms) - 1 - k, len(ms) - 1 - i]) < 1e-14  # d_mn = d_{-n,-m}


def test_barrier_factor_closed_forms():
    for q in [0.01, 0.1, 0.1973, 0.35, 0.8, 2.0]:
        z = (q / O.PR_DEFAULT) ** 2
        forms = {2: 2 * z / (z + 1), 4: 13 * z * z / (z * (z + 3) + 9),
                 6: 277 * z ** 3 / (z * (z * (z + 6) + 45) + 225)}
        assert float(O.barrier_factor(0, q)) == 1.0
        for L, f2 in forms.items():
            assert abs(float(O.barrier_factor(L, q)) ** 2 - f2) < 1e-12 * max(1.0, f2)
    for L in range(0, 16, 2):
        assert abs(float(O.barrier_factor(L, O.PR_DEFAULT)) - 1.0) < 1e-13


def test_breit_wigner_forms():
    m = np.linspace(0.3, 1.5, 50)
    bw = O.const_width_bw(m, 0.77, 0.15)
    assert np.allclose(bw, 0.77 * 0.15 / (0.77 ** 2 - m ** 2 - 1j * 0.77 * 0.15))
    rel = O.relativistic_bw(m, 0.1396, 0.1396, 0.77, 0.15, 2)
    k = np.argmin(abs(m - 0.77))
    assert abs(rel[k].imag) > abs(rel[k].real)                               # on the peak: ~ i
    assert np.allclose(abs(O.relativistic_bw(np.array([0.77]), 0.1396, 0.1396, 0.77, 0.15, 2)), 1.0)


@pytest.fixture(scope="module")
def sample():
    beam, fs, masses, mb = events(600, seed=3)
    W = [w for w, _ in waves()]
    return W, beam, fs, masses, mb, O.amplitudes(W, beam, fs, masses, mb, SPECIES)


def test_rotation_invariance(sample):
    W, beam, fs, masses, mb, A = sample
    R = O._rot("z", np.full(1, 0.4))[0] @ O._rot("y", np.full(1, 1.1))[0] @ O._rot("x", np.full(1, -0.3))[0]
    B = O.amplitudes(W, beam @ R.T, np.einsum("ij,knj->kni", R, fs), masses, mb, SPECIES)
    assert np.abs(A - B).max() < 1e-9 * np.abs(A).max()


def test_reflection_and_parity_eigenvalues(sample):
    """reflection through the production plane multiplies a wave of
    reflectivity refl by refl; space inversion by -P (P times the intrinsic
    parity (-1)^3 of three pseudoscalars, which the amplitudes leave out)."""
    W, beam, fs, masses, mb, A = sample
    Ar = O.amplitudes(W, beam, fs, masses, mb, SPECIES, reflection=True)
    Ap = O.amplitudes(W, beam, fs, masses, mb, SPECIES, space_inversion=True)
    for k, w in enumerate(W):
        s = np.abs(A[k]).max()
        if s == 0:
            continue
        assert np.abs(Ar[k] - w["refl"] * A[k]).max() < 1e-10 * s
        assert np.abs(Ap[k] + w["P"] * A[k]).max() < 1e-10 * s


def test_bose_symmetry(sample):
    W, beam, fs, masses, mb, A = sample
    swapped = fs[[2, 1, 0]]
    B = O.amplitudes(W, beam, swapped, masses, mb, SPECIES)
    assert np.abs(A - B).max() < 1e-12 * np.abs(A).max()
    # the symmetrised amplitude is the normalised sum of the two terms
    A0 = O.amplitudes(W, beam, fs, masses, mb, SPECIES, bose=False)
    A1 = O.amplitudes(W, beam, swapped, masses, mb, SPECIES, bose=False)
    assert np.abs(A - (A0 + A1) / math.sqrt(2)).max() < 1e-12 * np.abs(A).max()


def test_reflectivity_basis_combination(sample):
    """DFunctionReflConj: A(M, refl) = (A(+M) - f A(-M)) / sqrt 2 with the
    plain helicity basis, f = refl P (-1)^(J - M)."""
    W, beam, fs, masses, mb, A = sample
    for k, w in enumerate(W):
        if w["M"] == 0:
            continue
        plus = O.amplitudes([w], beam, fs, masses, mb, SPECIES, reflectivity_basis=False)[0]
        minus = O.amplitudes([dict(w, M=-w["M"])], beam, fs, masses, mb, SPECIES, reflectivity_basis=False)[0]
        f = O.reflectivity_factor(w["J"], w["P"], w["M"], w["refl"])
        assert np.abs(A[k] - (plus - f * minus) / math.sqrt(2)).max() < 1e-12 * np.abs(A[k]).max()


def test_canonical_equals_helicity_up_to_a_sign(sample):
    """for spinless final-state particles the canonical amplitudes
    (isobarCanonicalAmplitude: boost-only isobar frame, sum over mL of
    couplings times Y_L^mL) equal the helicity ones (rotated helicity frame,
    D functions): two independent routes through the frames and the spin
    algebra.  With the bachelor as the X vertex's daughter 1 the two
    conventions differ by a sign that is constant per wave (the order of the
    spins in the S coupling); with the isobar first they are equal."""
    W, beam, fs, masses, mb, A = sample
    Cn = O.amplitudes(W, beam, fs, masses, mb, SPECIES, formalism="canonical")
    for k, w in enumerate(W):
        s = np.abs(A[k]).max()
        if s == 0:
            assert np.all(Cn[k] == 0)
            continue
        sign = -1.0 if np.abs(Cn[k] + A[k]).max() < np.abs(Cn[k] - A[k]).max() else 1.0
        assert np.abs(Cn[k] - sign * A[k]).max() < 1e-9 * s    # the frames' FP64 rounding
        if not w["bachelor_first"]:
            assert sign == 1.0


def test_canonical_eigenvalues(sample):
    W, beam, fs, masses, mb, A = sample
    Cn = O.amplitudes(W, beam, fs, masses, mb, SPECIES, formalism="canonical")
    Cr = O.amplitudes(W, beam, fs, masses, mb, SPECIES, formalism="canonical", reflection=True)
    Cp = O.amplitudes(W, beam, fs, masses, mb, SPECIES, formalism="canonical", space_inversion=True)
    for k, w in enumerate(W):
        s = np.abs(Cn[k]).max()
        if s == 0:
            continue
        assert np.abs(Cr[k] - w["refl"] * Cn[k]).max() < 1e-10 * s
        assert np.abs(Cp[k] + w["P"] * Cn[k]).max() < 1e-10 * s


def test_isospin_terms_hand_derived():
    """isobarDecayTopology::getIsospinSymmetrization on two cases worked out by
    hand: pi- pi+ pi- through rho0 pi- keeps one term (factor 1); pi- pi0 pi0
    through rho- pi0 keeps the identity with (1 -1 1 0 | 1 -1)^2 / sqrt 2 =
    1 / (2 sqrt 2) and the rho0 -> pi0 pi0 partner with factor 0."""
    from isobar_cases import NEUTRAL_ISOSPIN, NEUTRAL_SPECIES, neutral_waves
    w = O.wave(2, 1, 0, 1, 0, 2, 2, 2, 1, 0.77, 0.15, (1, 2), 0, isospin=2, isobar_isospin=2)
    assert O.isospin_terms(w, [0, 1, 0], [2, 2, 2], [-2, 2, -2], [-1, -1, -1]) == [([0, 1, 2], 1.0)]
    rho_minus = neutral_waves()[0][0]
    t = O.isospin_terms(rho_minus, NEUTRAL_SPECIES, *NEUTRAL_ISOSPIN)
    assert [p for p, _ in t] == [[0, 1, 2], [2, 1, 0]]
    assert abs(t[0][1] - 0.5 / math.sqrt(2)) < 1e-15 and t[1][1] == 0.0
    # the wave keyed rho0 pi-: the rho0 -> pi0 pi0 term vanishes, a rho- pi0 term appears
    t = O.isospin_terms(neutral_waves()[4][0], NEUTRAL_SPECIES, *NEUTRAL_ISOSPIN)
    assert t[0] == ([0, 1, 2], 0.0) and t[1][0] == [1, 0, 2] and abs(t[1][1] - 0.5 / math.sqrt(2)) < 1e-15


def test_isospin_symmetrised_amplitudes():
    """for rho- pi0 the isospin-symmetrised amplitude is the Bose-symmetrised
    one times +-1 / (2 sqrt 2) (the sign of the X vertex's isospin coupling
    follows the daughters' order); the f0 and f2 waves (isospin 0 to
    pi0 pi0) keep one isospin term; the amplitudes stay reflectivity and
    parity eigenstates."""
    from isobar_cases import NEUTRAL_ISOSPIN, NEUTRAL_SPECIES, neutral_events, neutral_waves
    W = [w for w, _ in neutral_waves()]
    beam, fs, masses, mb = neutral_events(400, seed=9)
    A0 = O.amplitudes(W, beam, fs, masses, mb, NEUTRAL_SPECIES)
    A1 = O.amplitudes(W, beam, fs, masses, mb, NEUTRAL_SPECIES, isospin=NEUTRAL_ISOSPIN)
    for k, sign in ((0, +1), (1, -1)):
        assert np.abs(A1[k] - sign * A0[k] / (2 * math.sqrt(2))).max() < 1e-13 * np.abs(A0[k]).max()
    for k in (2, 3):
        assert np.abs(A1[k] - A0[k]).max() < 1e-13 * np.abs(A0[k]).max()
    Ar = O.amplitudes(W, beam, fs, masses, mb, NEUTRAL_SPECIES, isospin=NEUTRAL_ISOSPIN, reflection=True)
    Ap = O.amplitudes(W, beam, fs, masses, mb, NEUTRAL_SPECIES, isospin=NEUTRAL_ISOSPIN, space_inversion=True)
    for k, w in enumerate(W):
        s = np.abs(A1[k]).max()
        assert s > 0
        assert np.abs(Ar[k] - w["refl"] * A1[k]).max() < 1e-10 * s
        assert np.abs(Ap[k] + w["P"] * A1[k]).max() < 1e-10 * s


def test_pipi_s_wave_unitarity_and_f0_dip():
    """the AMP pi pi S-wave (massDependence.cc:505-625): below the K K
    threshold T_00 = 1 / (M_00 - i rho_00) with real M_00, so elastic
    unitarity Im(1 / T) = -rho_00 holds exactly (rho the mean of the charged
    and neutral pi pi phase-space factors); the M solution has the f0(980)
    dip just below the K K threshold."""
    m = np.linspace(0.3, 0.98, 40)
    for variant in ("m", "kachaev"):
        T = O.pipi_s_wave(m, variant)
        rho = ((2 * O._q_complex(m, O.M_PI_CHARGED) / m + 2 * O._q_complex(m, O.M_PI_NEUTRAL) / m) / 2).real
        assert np.allclose((1 / T).imag, -rho, rtol=1e-12, atol=1e-14)
    grid = np.linspace(0.9, 1.05, 301)
    a = np.abs(O.pipi_s_wave(grid, "m"))
    assert 0.97 < grid[np.argmin(a)] < 1.0 and a.min() < 0.2 * a.max()


def test_golden_fixture():
    """tests/golden/isobar3pi_oracle.npz (make_isobar_golden.py): the oracle
    and the seeded event generator reproduce the committed amplitudes."""
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import make_isobar_golden as G
    gold = np.load(os.path.join(here, "golden", "isobar3pi_oracle.npz"))
    now = G.compute()
    for k in ("beam", "fs", "neutral_beam", "neutral_fs"):
        assert np.array_equal(now[k], gold[k]), k
    for k in ("helicity", "canonical", "neutral_isospin"):
        scale = np.abs(gold[k]).max(axis=1, keepdims=True) + 1e-300
        assert np.all(np.abs(now[k] - gold[k]) <= 1e-12 * scale), k


def test_kpi_s_wave_unitarity():
    """the K pi S-wave forms (massDependence.cc:700-828): LASS with F = R = 1
    and no phases is elastic, |1 + 2 i t| = 1 for t = amp 2q / M; the
    Palano-Pennington T_11 obeys Im(1 / T_11) = -rho_Kpi below the K eta
    threshold (the K eta channel then only renormalises K_11)."""
    from isobar_cases import GLASS
    m = np.linspace(0.7, 1.85, 60)
    q = np.sqrt(O.breakup_momentum_squared(m, O.M_K_CHARGED, O.M_PI_CHARGED))
    t = O.kpi_s_glass(m, GLASS) * 2 * q / m
    assert np.allclose(np.abs(1 + 2j * t), 1.0, atol=1e-12)
    m = np.linspace(0.65, 1.03, 40)
    T = O.kpi_s_palano(m)
    rho = (2 * O._q_complex2(m, O.M_K_CHARGED, O.M_PI_CHARGED) / m).real
    assert np.allclose((1 / T).imag, -rho, rtol=1e-10, atol=1e-13)
