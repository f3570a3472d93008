"""FP64 restatement of the reference's isobar decay amplitudes for three
spinless final-state particles (X -> isobar + bachelor, isobar -> a + b) in
the helicity and the canonical formalism.

TEST INFRASTRUCTURE ONLY: this module is the checker of the GPU amplitude
kernel (rootpwa_gb300/csrc/isobar.cu).  Only tests, the smoke check and the
benchmark's CPU-baseline leg may import it; the product never calls it.

It follows the reference step by step, vectorised over events with numpy:

* Gottfried-Jackson frame: isobarAmplitude::gjTransform
  (decayAmplitude/isobarAmplitude.cc:137-171) -- rotate so that beam x X is
  the y axis, boost into the X rest frame, rotate about y so that the beam is
  the z axis; the same sequence of ROOT-style active rotations and boosts.
* helicity frame of the isobar: isobarHelicityAmplitude::hfTransform
  (decayAmplitude/isobarHelicityAmplitude.cc:64-84), applied to the isobar's
  daughters after the Gottfried-Jackson transformation
  (transformDaughters, :87-126).
* two-body amplitude: isobarHelicityAmplitude::twoBodyDecayAmplitude
  (:130-195) = sqrt(L+1) * D*(phi, theta, 0) * (L 0 S lambda | J lambda)
  * (s1 lambda1 s2 -lambda2 | S lambda) * F_L(q) * mass dependence, with the
  reflectivity-basis D function at the X vertex (utilities/dFunction.hpp
  DFunctionReflConj) and the sum over the isobar's helicities
  (isobarAmplitude::twoBodyDecayAmplitudeSum, isobarAmplitude.cc:206-262).
* canonical formalism (formalism="canonical"): isobarCanonicalAmplitude
  (decayAmplitude/isobarCanonicalAmplitude.cc:64-190): the isobar's rest
  frame by a boost alone, sqrt(4 pi) (s1 m1 s2 m2 | S mS) F_L(q) * sum over
  mL of the (reflectivity-combined) (L mL S mS | J M) Y_L^mL(theta, phi).
* symmetrisation terms: slot i takes the momentum of particle p[i] with slot
  i's own mass (decayTopology::revertMomenta, particle::setMomentum), and the
  frames are built per term.
* Bose symmetrisation: sum over the permutations of identical final-state
  particles with factor 1/sqrt(prod n_k!) (isobarDecayTopology.cc:638-670,
  isobarAmplitude.cc:98-111); isospin symmetrisation over permutations of
  isospin partners with isospin Clebsch-Gordan factors
  (isobarDecayTopology.cc:505-630), combined with the Bose terms as in
  isobarAmplitude.cc:265-330; space inversion and reflection through the
  production plane as in isobarAmplitude.cc:174-203.
* mass dependences: flat, relativistic Breit-Wigner with the PWA2000 rule
  q0 = sqrt|q0^2| (massDependence.cc:254-296, utilities/physUtils.hpp:283-300),
  constant-width Breit-Wigner (massDependence.cc:300-320), the rho and
  f0(980) Breit-Wigners (:324-390), the f0(980) Flatte form with the BES II
  parameters (:395-445), the pi pi S-wave of Au, Morgan and Pennington
  (M, VES and Kachaev variants, :449-625), the K pi S-wave forms (LASS and
  Palano-Pennington, :700-828), rho' (:830-862) and the binned mass
  dependence (:187-230).

The building blocks are restated from the published formulas, not from the
reference's arrangement of them: Clebsch-Gordan coefficients by Racah's
formula, Wigner d functions by Wigner's formula, Blatt-Weisskopf barrier
factors from spherical Hankel functions (scipy), normalised to 1 at q equal
to the momentum scale 0.1973 GeV/c (utilities/physUtils.hpp:200-275).

Parity unpinned against the reference itself: its decay-amplitude library
needs ROOT and boost and does not build here, and its tests hold no
amplitude values (test/decayAmplitude/testAmplitude.cc compares runs).  The
building blocks are pinned against sympy and against the PDG closed forms,
and the frames against rotation invariance and the reflectivity and parity
eigenvalues, in tests/test_isobar_oracle.py.

All spins, spin projections and orbital angular momenta are integers in
units of 1/2 (2J, 2M, 2L), as in the reference.
"""
import math
from itertools import permutations

import numpy as np

PR_DEFAULT = 0.1973        # GeV/c, 1 fm interaction radius
(MASSDEP_FLAT, MASSDEP_REL_BW, MASSDEP_CONST_BW, MASSDEP_RHO_BW, MASSDEP_F0980_BW, MASSDEP_F0980_FLATTE,
 MASSDEP_PIPIS_M, MASSDEP_PIPIS_VES, MASSDEP_PIPIS_KACHAEV, MASSDEP_BINNED, MASSDEP_RHO_PRIME, MASSDEP_KPIS_GLASS,
 MASSDEP_KPIS_PALANO) = range(13)
M_ETA = 0.547862
M_PI_CHARGED, M_K_CHARGED = 0.13957039, 0.493677   # GeV/c^2 (the particle table's pi+ and K+)
M_PI_NEUTRAL, M_K_NEUTRAL = 0.1349768, 0.497611

# Au, Morgan, Pennington, Phys. Rev. D 35 (1987) 1633, Table 1, M solution, as
# used by piPiSWaveAuMorganPenningtonImpl (massDependence.cc:449-500): pole
# residues a_i (2 x 2), pole positions s_i, background polynomial c_n (2 x 2)
AMP_F = np.array([0.1968, -0.0154])
AMP_A = [np.array([[0.1131, 0.0150], [0.0150, -0.3216]]), np.outer(AMP_F, AMP_F)]
AMP_C = [np.array([[0.0337, -0.2826], [-0.2826, 0.3010]]), np.array([[-0.3185, 0.0918], [0.0918, -0.5140]]),
         np.array([[-0.0942, 0.1669], [0.1669, 0.1176]]), np.array([[-0.5927, -0.2082], [-0.2082, 0.5204]]),
         np.array([[0.1957, -0.1386], [-0.1386, -0.3977]])]
AMP_SP = [-0.0074, 0.9828]


# -- spin algebra ---------------------------------------------------------------

def _f(n):
    return math.factorial(n)


def clebsch_gordan(j1, m1, j2, m2, J, M):
    """(j1 m1 j2 m2 | J M), arguments doubled; Racah's formula
    (clebschGordanCoeff, utilities/spinUtils.hpp:241-330)."""
    def ok(j, m):
        return j >= 0 and abs(m) <= j and (j - m) % 2 == 0
    if not (ok(j1, m1) and ok(j2, m2) and ok(J, M)):
        return 0.0
    if not (abs(j1 - j2) <= J <= j1 + j2) or (j1 + j2 + J) % 2:
        return 0.0
    if m1 + m2 != M:
        return 0.0
    def h(x):                 # every combination below is even
        return x // 2
    pre = ((J + 1) * _f(h(J + j1 - j2)) * _f(h(J - j1 + j2)) * _f(h(j1 + j2 - J))
           / _f(h(j1 + j2 + J) + 1))
    pre *= _f(h(J + M)) * _f(h(J - M)) * _f(h(j1 - m1)) * _f(h(j1 + m1)) * _f(h(j2 - m2)) * _f(h(j2 + m2))
    s = 0.0
    for k in range(0, h(j1 + j2 + J) + 1):
        den = [k, h(j1 + j2 - J) - k, h(j1 - m1) - k, h(j2 + m2) - k,
               h(J - j2 + m1) + k, h(J - j1 - m2) + k]
        if min(den) < 0:
            continue
        s += (-1) ** k / float(np.prod([_f(x) for x in den]))
    return math.sqrt(pre) * s


def wigner_d_terms(j, m, n):
    """d^j_{m n}(theta) = sum of coef * cos(theta/2)^a * sin(theta/2)^b,
    arguments doubled; Wigner's formula in the PDG sign convention
    (dFunction, utilities/dFunction.hpp:52-170)."""
    J, Mp, Mm = j, m, n
    jpm, jmm, jpn, jmn = (J + Mp) // 2, (J - Mp) // 2, (J + Mm) // 2, (J - Mm) // 2
    root = math.sqrt(_f(jpm) * _f(jmm) * _f(jpn) * _f(jmn))
    d = (Mp - Mm) // 2            # m' - m in units of 1
    out = []
    for s in range(0, J + 1):
        den = [jpn - s, s, d + s, jmm - s]
        if min(den) < 0:
            continue
        coef = (-1) ** (d + s) * root / float(np.prod([_f(x) for x in den]))
        out.append((coef, jpn + jmm - 2 * s, d + 2 * s))
    return out


def wigner_d(j, m, n, theta):
    theta = np.asarray(theta, dtype=np.float64)
    c, s = np.cos(theta / 2), np.sin(theta / 2)
    return sum(coef * c ** a * s ** b for coef, a, b in wigner_d_terms(j, m, n)) + 0 * theta


def D_conj(j, m, n, phi, theta):
    """conj(D^j_{m n}(phi, theta, 0)) = exp(+i m phi / 2) d^j_{m n}(theta)."""
    return np.exp(1j * (m / 2.0) * phi) * wigner_d(j, m, n, theta)


def reflectivity_factor(J, P, M, refl):
    """refl * P * (-1)^((J - M) / 2) (utilities/physUtils.hpp:172-196)."""
    return refl * P * (-1) ** ((J - M) // 2)


def D_refl_conj(J, M, n, P, refl, phi, theta):
    """conj of the reflectivity-basis D function (utilities/dFunction.hpp
    DFunctionRefl / DFunctionReflConj)."""
    f = reflectivity_factor(J, P, M, refl)
    if M == 0:
        if f == +1:
            return np.zeros_like(phi, dtype=np.complex128)
        return D_conj(J, 0, n, phi, theta)
    return (D_conj(J, M, n, phi, theta) - f * D_conj(J, -M, n, phi, theta)) / math.sqrt(2.0)


# -- barrier factors and mass dependences -----------------------------------------

def _hankel_abs2(l, x):
    from scipy.special import spherical_jn, spherical_yn
    return spherical_jn(l, x) ** 2 + spherical_yn(l, x) ** 2


def barrier_factor(L, q, Pr=PR_DEFAULT):
    """Blatt-Weisskopf factor F_L(q), L doubled: F_L^2 = |h_l(1)|^2 / (x^2 |h_l(x)|^2),
    x = q / Pr (utilities/physUtils.hpp:200-275)."""
    l = L // 2
    q = np.asarray(q, dtype=np.float64)
    if l == 0:
        return np.ones_like(q)
    x = q / Pr
    with np.errstate(divide="ignore", invalid="ignore"):
        f2 = _hankel_abs2(l, 1.0) / (x * x * _hankel_abs2(l, x))
    f2 = np.where(x == 0, 0.0, f2)
    return np.sqrt(f2)


def breakup_momentum_squared(M, m1, m2):
    """(utilities/physUtils.hpp:75-96), sub-threshold values allowed."""
    return (M - (m1 + m2)) * (M + (m1 + m2)) * (M - (m1 - m2)) * (M + (m1 - m2)) / (4 * M * M)


def relativistic_bw(M, m1, m2, M0, G0, L):
    """relativisticBreitWigner::amp (massDependence.cc:254-296) with
    breitWigner (utilities/physUtils.hpp:283-300)."""
    q = np.sqrt(np.maximum(breakup_momentum_squared(M, m1, m2), 0.0))
    q0 = math.sqrt(abs(breakup_momentum_squared(M0, m1, m2)))
    if q0 == 0:
        return np.zeros_like(M, dtype=np.complex128)
    G = G0 * (M0 / M) * (q / q0) * (barrier_factor(L, q) ** 2 / barrier_factor(L, q0) ** 2)
    A, B, C = M0 * G0, M0 * M0 - M * M, M0 * G
    return (A / (B * B + C * C)) * (B + 1j * C)


def rho_bw(M, m1, m2, M0, G0):
    """rhoBreitWigner::amp (massDependence.cc:324-359): F = 2 q^2 / (q0^2 + q^2)."""
    q2 = np.maximum(breakup_momentum_squared(M, m1, m2), 0.0)
    q02 = breakup_momentum_squared(M0, m1, m2)
    q, q0 = np.sqrt(q2), math.sqrt(q02)
    F = 2 * q2 / (q02 + q2)
    G = G0 * (M0 / M) * (q / q0) * F
    A, B, C = M0 * G0 * np.sqrt(F), M0 * M0 - M * M, M0 * G
    return (A / (B * B + C * C)) * (B + 1j * C)


def f0980_bw(M, m1, m2, M0, G0):
    """f0980BreitWigner::amp (massDependence.cc:363-390): Gamma = Gamma0 q / q0,
    numerator M0 Gamma M / q."""
    q = np.sqrt(np.maximum(breakup_momentum_squared(M, m1, m2), 0.0))
    q0 = math.sqrt(max(breakup_momentum_squared(M0, m1, m2), 0.0))
    G = G0 * (q / q0)
    C = M0 * G
    A, B = C * M / q, M0 * M0 - M * M
    return (A / (B * B + C * C)) * (B + 1j * C)


def f0980_flatte(M):
    """f0980FlatteBesII::amp (massDependence.cc:395-445): the BES II Flatte
    parameters M0 = 0.965, g1 = 0.165, g2/g1 = 4.21; complex breakup momenta
    of pi+ pi- and K+ K- (imaginary below threshold, physUtils.hpp:108-120)."""
    def kc(m):
        q2 = breakup_momentum_squared(M, m, m)
        q = np.sqrt(np.abs(q2))
        return np.where(q2 < 0, 1j * q, q + 0j)
    rho_pi, rho_k = 2 * kc(M_PI_CHARGED) / M, 2 * kc(M_K_CHARGED) / M
    denom = (0.965 ** 2 - M * M) + 0j - 1j * 0.165 * (rho_pi + 4.21 * rho_k)
    return 1.0 / denom


def _q_complex(M, m):
    """breakupMomentumComplex (utilities/physUtils.hpp:108-120) for equal masses."""
    q2 = breakup_momentum_squared(M, m, m)
    q = np.sqrt(np.abs(q2))
    return np.where(q2 < 0, 1j * q, q + 0j)


def pipi_s_wave(M, variant):
    """piPiSWaveAuMorganPennington{M,Ves,Kachaev}::amp (massDependence.cc:
    505-625): M(s) = sum_i a_i / (s - s_i) + sum_n c_n (s / 4 m_K^2 - 1)^n with
    the off-diagonal elements set to zero, T = (M - i rho)^-1, amp = T_00;
    rho from the charged and neutral pi pi (K K) breakup momenta, or the
    charged ones only on the VES sheet, which also subtracts an f0(980)
    Breit-Wigner; the Kachaev variant drops c_4 (diagonal), the off-diagonal
    a_0 and a_1."""
    a = [x.copy() for x in AMP_A]
    c = [x.copy() for x in AMP_C]
    if variant == "kachaev":
        c[4][0, 0] = c[4][1, 1] = 0.0
        a[0][0, 1] = a[0][1, 0] = 0.0
        a[1][:] = 0.0
    M = np.asarray(M, dtype=np.float64)
    out = np.zeros(M.shape, dtype=np.complex128)
    mk = (M_K_CHARGED + M_K_NEUTRAL) / 2
    for e, m in np.ndenumerate(M):
        s = m * m
        if abs(s - AMP_SP[1]) < 1e-6:
            m += 1e-6
            s = m * m
        rho = np.zeros((2, 2), dtype=np.complex128)
        if variant == "ves":
            rho[0, 0] = 2 * _q_complex(m, M_PI_CHARGED) / m
            rho[1, 1] = 2 * _q_complex(m, mk) / m
        else:
            rho[0, 0] = (2 * _q_complex(m, M_PI_CHARGED) / m + 2 * _q_complex(m, M_PI_NEUTRAL) / m) / 2
            rho[1, 1] = (2 * _q_complex(m, M_K_CHARGED) / m + 2 * _q_complex(m, M_K_NEUTRAL) / m) / 2
        scale = s / (4 * mk * mk) - 1
        Mm = sum(a[i] / (s - AMP_SP[i]) for i in range(2)) + sum(c[n] * scale ** n for n in range(5))
        Mm = Mm.astype(np.complex128)
        Mm[0, 1] = Mm[1, 0] = 0
        amp = np.linalg.inv(Mm - 1j * rho)[0, 0]
        if variant == "ves" and m > 2 * M_PI_CHARGED:
            f0m, f0w, coupling = 0.9837, 0.0376, -0.3743 + 0.3197j
            q = math.sqrt(breakup_momentum_squared(m, M_PI_CHARGED, M_PI_CHARGED))
            q0 = math.sqrt(breakup_momentum_squared(f0m, M_PI_CHARGED, M_PI_CHARGED))
            C = f0m * f0w * q / q0
            A, B = C * m / q, f0m * f0m - m * m
            amp = amp - coupling * (A / (B * B + C * C)) * (B + 1j * C)
        out[e] = amp
    return out


def kpi_s_glass(M, p):
    """KPiSGLASS::amp (massDependence.cc:700-722); p = a, r, M0, G0, phiF,
    phiR, phiRsin, F, R, MMax."""
    a, r, M0, G0, phiF, phiR, phiRsin, F, R, MMax = p
    out = np.zeros(np.shape(M), dtype=np.complex128)
    for e, m in np.ndenumerate(np.asarray(M, dtype=np.float64)):
        if not (M_K_CHARGED + M_PI_CHARGED < m < MMax):
            continue
        q = math.sqrt(breakup_momentum_squared(m, M_K_CHARGED, M_PI_CHARGED))
        q0 = math.sqrt(breakup_momentum_squared(M0, M_K_CHARGED, M_PI_CHARGED))
        G = G0 * M0 / m * q / q0
        dR = math.atan(M0 * G / (M0 * M0 - m * m))
        dF = math.atan(2.0 * a * q / (2.0 + a * r * q * q))
        amp = (F * math.sin(dF + phiF) * np.exp(1j * (dF + phiF))
               + R * math.sin(dR + phiRsin) * np.exp(1j * (dR + phiR)) * np.exp(2j * (dF + phiF)))
        out[e] = amp * 0.5 * m / q
    return out


def _q_complex2(M, m1, m2):
    q2 = breakup_momentum_squared(M, m1, m2)
    q = np.sqrt(np.abs(q2))
    return np.where(q2 < 0, 1j * q, q + 0j)


def kpi_s_palano(M, MMax=2.4):
    """KPiSPalanoPennington::amp (massDependence.cc:770-828): T_11 of the
    (K pi, K eta) K-matrix with an Adler zero."""
    sTop, sBot, sa, sb = 5.832, 0.36, 1.7991, 8.3627
    ga, gb = (0.3139, -0.00775), (1.1804, -0.22335)
    C = (((-0.1553, 0.0909, 0.8618, 0.0629), (0.0738, 0.3866, 1.2195, 0.8390)),
         ((0.0738, 0.3866, 1.2195, 0.8390), (-0.0036, 0.2590, 1.6950, 2.2300)))
    sKpi = M_K_CHARGED ** 2 + M_PI_CHARGED ** 2
    sA = 0.87753 * sKpi
    out = np.zeros(np.shape(M), dtype=np.complex128)
    for e, m in np.ndenumerate(np.asarray(M, dtype=np.float64)):
        if not (M_K_CHARGED + M_PI_CHARGED < m < MMax):
            continue
        s = m * m
        rho1 = 2 * _q_complex2(m, M_K_CHARGED, M_PI_CHARGED) / m
        rho2 = 2 * _q_complex2(m, M_K_CHARGED, M_ETA) / m
        x = (2 * s - (sTop + sBot)) / (sTop - sBot)

        def K(i, j):
            return (s - sA) / sKpi * (ga[i] * ga[j] / (sa - s) + gb[i] * gb[j] / (sb - s)
                                      + sum(C[i][j][n] * x ** n for n in range(4)))
        K11, K12, K22 = K(0, 0), K(0, 1), K(1, 1)
        detK = K11 * K22 - K12 * K12
        delta = 1.0 - 1j * rho1 * K11 - 1j * rho2 * K22 - rho1 * rho2 * detK
        out[e] = (K11 - 1j * rho2 * detK) / delta
    return out


def const_width_bw(M, M0, G0):
    """constWidthBreitWigner::amp (massDependence.cc:300-320)."""
    A, B = M0 * G0, M0 * M0 - M * M
    return (A / (B * B + A * A)) * (B + 1j * A)


# -- ROOT-style rotations and boosts (vectorised over events) ----------------------

def _phi(v):
    return np.where((v[..., 0] == 0) & (v[..., 1] == 0), 0.0, np.arctan2(v[..., 1], v[..., 0]))


def _theta(v):
    perp = np.hypot(v[..., 0], v[..., 1])
    return np.where((perp == 0) & (v[..., 2] == 0), 0.0, np.arctan2(perp, v[..., 2]))


def _rot(axis, a):
    c, s = np.cos(a), np.sin(a)
    o, z = np.ones_like(a), np.zeros_like(a)
    if axis == "x":
        m = [[o, z, z], [z, c, -s], [z, s, c]]
    elif axis == "y":
        m = [[c, z, s], [z, o, z], [-s, z, c]]
    else:
        m = [[c, -s, z], [s, c, z], [z, z, o]]
    return np.moveaxis(np.array(m), (0, 1), (-2, -1))       # (N, 3, 3)


def _apply_rot(R, lv):
    out = lv.copy()
    out[..., :3] = np.einsum("nij,nj->ni", R, lv[..., :3])
    return out


def _boost(lv, b):
    """TLorentzVector::Boost(b)."""
    b2 = np.sum(b * b, axis=-1)
    g = 1.0 / np.sqrt(1.0 - b2)
    bp = np.sum(b * lv[..., :3], axis=-1)
    g2 = np.where(b2 > 0, (g - 1.0) / np.where(b2 > 0, b2, 1.0), 0.0)
    out = np.empty_like(lv)
    out[..., :3] = lv[..., :3] + (g2 * bp)[..., None] * b + (g * lv[..., 3])[..., None] * b
    out[..., 3] = g * (lv[..., 3] + bp)
    return out


def _ytransform(yaxis):
    """rotation taking yaxis to +y with the old z axis in the (x, z) plane:
    RotateZ(pi/2 - phi_y) followed by RotateX(theta_y - pi/2)."""
    return np.einsum("nij,njk->nik", _rot("x", _theta(yaxis) - math.pi / 2), _rot("z", math.pi / 2 - _phi(yaxis)))


def gj_transform(beam, X, lvs):
    """isobarAmplitude::gjTransform (isobarAmplitude.cc:137-171) applied to
    the Lorentz vectors lvs [(N, 4), ...]."""
    R1 = _ytransform(np.cross(beam[:, :3], X[:, :3]))
    b1, X1 = _apply_rot(R1, beam), _apply_rot(R1, X)
    bx = -X1[:, :3] / X1[:, 3:4]
    b2 = _boost(b1, bx)
    R2 = _rot("y", -np.sign(b2[:, 0]) * _theta(b2))
    return [_apply_rot(R2, _boost(_apply_rot(R1, v), bx)) for v in lvs]


def hf_transform(parent, lvs):
    """isobarHelicityAmplitude::hfTransform (isobarHelicityAmplitude.cc:64-84)."""
    z = np.zeros_like(parent[:, :3])
    z[:, 2] = 1.0
    R1 = _ytransform(np.cross(z, parent[:, :3]))
    d1 = _apply_rot(R1, parent)
    R2 = _rot("y", -np.sign(d1[:, 0]) * _theta(d1))
    d2 = _apply_rot(R2, d1)
    R = np.einsum("nij,njk->nik", R2, R1)
    bx = -d2[:, :3] / d2[:, 3:4]
    return [_boost(_apply_rot(R, v), bx) for v in lvs]


def _lv(p, m):
    return np.concatenate([p, np.sqrt(m * m + np.sum(p * p, axis=-1))[:, None]], axis=-1)


def _mass(lv):
    return np.sqrt(lv[:, 3] ** 2 - np.sum(lv[:, :3] ** 2, axis=-1))


# -- amplitudes --------------------------------------------------------------------

def _can_couple(j1, m1, j2, m2, J, M):
    """spinStatesCanCouple(j1, m1, j2, m2, J, M) (utilities/spinUtils.hpp:167):
    valid projections, triangle rule, M = m1 + m2 (arguments doubled)."""
    def ok(j, m):
        return j >= 0 and abs(m) <= j and (j - m) % 2 == 0
    return (ok(j1, m1) and ok(j2, m2) and ok(J, M) and abs(j1 - j2) <= J <= j1 + j2
            and (j1 + j2 - J) % 2 == 0 and M == m1 + m2)


def isospin_terms(w, species, isospins, isospin_projs, parities):
    """isobarDecayTopology::getIsospinSymmetrization (isobarDecayTopology.cc:
    505-630) for X -> isobar(a, b) + bachelor c: permutations within groups of
    final-state particles of equal isospin and parity (all spin 0), in the
    order of getAllGroupPermutations (:889-923); a permutation is dropped if,
    against an accepted one, it exchanges particles of equal species or two
    particles of one vertex, or if the permuted isospin projections cannot
    couple at a vertex; the factor is the product of the isospin
    Clebsch-Gordan coefficients of both vertices, divided by sqrt(number of
    terms), or 1 when only one term survives.  Returns [(perm, factor)],
    slot i taking particle perm[i]."""
    n = len(species)
    keys = []
    for i in range(n):
        k = (isospins[i], parities[i])
        if k not in keys:
            keys.append(k)
    groups = [[i for i in range(n) if (isospins[i], parities[i]) == k] for k in keys]

    def group_perms(gs):
        cur = sorted(gs[-1])
        curs = list(permutations(cur))            # lexicographic, like next_permutation
        if len(gs) == 1:
            return [[list(c)] for c in curs]
        sub = group_perms(gs[:-1])
        return [sp + [list(c)] for c in curs for sp in sub]
    a, b, c = w["isobar_daughters"][0], w["isobar_daughters"][1], w["bachelor"]
    vertex = {a: 1, b: 1, c: 0}                   # the vertex each final-state slot comes from
    I_iso, I_X = w["isobar_isospin"], w["isospin"]
    accepted = []
    for gp in group_perms(groups):
        perm = [0] * n
        for g, pg in zip(groups, gp):
            for slot, part in zip(g, pg):
                perm[slot] = part
        discard = False
        for q, _ in accepted:
            for i in range(n):
                if q[i] == perm[i]:
                    continue
                if species[q[i]] == species[perm[i]]:
                    discard = True
                    break
                for j in range(i + 1, n):
                    if q[j] == perm[j]:
                        continue
                    if vertex[q[i]] == vertex[q[j]] == vertex[perm[i]] == vertex[perm[j]]:
                        discard = True
                        break
                if discard:
                    break
            if discard:
                break
        if discard:
            continue
        I3 = [isospin_projs[perm[i]] for i in range(n)]
        I3_iso = I3[a] + I3[b]
        I3_X = sum(isospin_projs)
        d = [(I_iso, I3_iso), (isospins[c], I3[c])]
        if w["bachelor_first"]:
            d = d[::-1]
        if not (_can_couple(isospins[a], I3[a], isospins[b], I3[b], I_iso, I3_iso)
                and _can_couple(d[0][0], d[0][1], d[1][0], d[1][1], I_X, I3_X)):
            continue
        f = (clebsch_gordan(d[0][0], d[0][1], d[1][0], d[1][1], I_X, I3_X)
             * clebsch_gordan(isospins[a], I3[a], isospins[b], I3[b], I_iso, I3_iso))
        accepted.append((perm, f))
    if len(accepted) == 1:
        return [(accepted[0][0], 1.0)]            # a single term keeps factor 1 (isobarAmplitude.cc:276-279)
    return [(p, f / math.sqrt(len(accepted))) for p, f in accepted]


def bose_terms(species):
    """all permutations that exchange identical final-state particles, with the
    factor 1/sqrt(prod n_k!) (isobarDecayTopology.cc:638-670)."""
    n = len(species)
    perms = [p for p in permutations(range(n)) if all(species[p[i]] == species[i] for i in range(n))]
    return perms, 1.0 / math.sqrt(len(perms))


def Y(l, m, theta, phi):
    """spherical harmonic Y_l^m, arguments doubled (sphericalHarmonic,
    utilities/dFunction.hpp:176-192): sqrt((2l+1)/4pi) e^{i m phi} d^l_{m 0}."""
    return math.sqrt((l + 1) / (4 * math.pi)) * np.exp(1j * (m / 2.0) * phi) * wigner_d(l, m, 0, theta)


def _canonical_two_body(J, M, P, refl, L, S, s1, m1, s2, m2, theta, phi, q, bw, top, refl_basis):
    """isobarCanonicalAmplitude::twoBodyDecayAmplitude (isobarCanonicalAmplitude.cc:
    118-190): sqrt(4 pi) (s1 m1 s2 m2 | S mS) F_L(q) bw sum_mL C_LS(mL) Y_L^mL."""
    mS = m1 + m2
    ss = clebsch_gordan(s1, m1, s2, m2, S, mS)
    if ss == 0:
        return np.zeros_like(theta, dtype=np.complex128)
    amp = np.zeros_like(theta, dtype=np.complex128)
    for mL in range(-L, L + 1, 2):
        if refl_basis and top:
            f = reflectivity_factor(J, P, M, refl)
            if M == 0:
                c = 0.0 if f == +1 else clebsch_gordan(L, mL, S, mS, J, 0)
            else:
                c = (clebsch_gordan(L, mL, S, mS, J, M) - f * clebsch_gordan(L, mL, S, mS, J, -M)) / math.sqrt(2)
        else:
            c = clebsch_gordan(L, mL, S, mS, J, M)
        if c == 0:
            continue
        amp = amp + c * Y(L, mL, theta, phi)
    return amp * (math.sqrt(4 * math.pi) * ss * barrier_factor(L, q) * bw)


def _sym_term(w, beam, fs, masses, opts):
    a, b, c = w["isobar_daughters"][0], w["isobar_daughters"][1], w["bachelor"]
    X = fs[0] + fs[1] + fs[2]
    gj = gj_transform(beam, X, fs)
    if opts.get("space_inversion"):
        gj = [np.concatenate([-v[:, :3], v[:, 3:]], axis=1) for v in gj]
    if opts.get("reflection"):
        gj = [v * np.array([1.0, -1.0, 1.0, 1.0]) for v in gj]
    iso = gj[a] + gj[b]
    bach = gj[c]
    # X vertex: daughter 1 is the analyser
    d1 = bach if w["bachelor_first"] else iso
    phi, theta = _phi(d1[:, :3]), _theta(d1[:, :3])
    qX = np.sqrt(np.sum(d1[:, :3] ** 2, axis=-1))
    canonical = opts.get("formalism", "helicity") == "canonical"
    # isobar vertex: helicity frame of the isobar (canonical: its rest frame
    # by a boost alone, isobarCanonicalAmplitude.cc:94-108), analyser = isobar daughter 1
    ha, = ([_boost(gj[a], -iso[:, :3] / iso[:, 3:4])] if canonical else hf_transform(iso, [gj[a]]))
    phih, thetah = _phi(ha[:, :3]), _theta(ha[:, :3])
    qI = np.sqrt(np.sum(ha[:, :3] ** 2, axis=-1))
    mI = _mass(iso)
    J, P, M, refl, L, S = w["J"], w["P"], w["M"], w["refl"], w["L"], w["S"]
    j, l, s = w["isobar_J"], w["isobar_L"], w["isobar_S"]
    md = w["mass_dep"]
    if md == MASSDEP_REL_BW:
        bw = relativistic_bw(mI, masses[a], masses[b], w["isobar_mass"], w["isobar_width"], l)
    elif md == MASSDEP_CONST_BW:
        bw = const_width_bw(mI, w["isobar_mass"], w["isobar_width"])
    elif md == MASSDEP_RHO_BW:
        bw = rho_bw(mI, masses[a], masses[b], w["isobar_mass"], w["isobar_width"])
    elif md == MASSDEP_F0980_BW:
        bw = f0980_bw(mI, masses[a], masses[b], w["isobar_mass"], w["isobar_width"])
    elif md == MASSDEP_F0980_FLATTE:
        bw = f0980_flatte(mI)
    elif md == MASSDEP_RHO_PRIME:
        # rhoPrimeMassDep::amp (massDependence.cc:830-862)
        bw = (4 * const_width_bw(mI, 1.465, 0.235) - 3 * const_width_bw(mI, 1.700, 0.220)) / 7
    elif md == MASSDEP_KPIS_GLASS:
        bw = kpi_s_glass(mI, w["mass_dep_params"])
    elif md == MASSDEP_KPIS_PALANO:
        p = w.get("mass_dep_params") or (2.4,)
        bw = kpi_s_palano(mI, p[0] if p[0] > 0 else 2.4)
    elif md == MASSDEP_BINNED:
        # binnedMassDependence::amp (massDependence.cc:212-230)
        lo, hi = w["bounds"]
        bw = np.where((mI >= lo) & (mI < hi), 1.0 + 0j, 0j)
    elif md in (MASSDEP_PIPIS_M, MASSDEP_PIPIS_VES, MASSDEP_PIPIS_KACHAEV):
        bw = pipi_s_wave(mI, {MASSDEP_PIPIS_M: "m", MASSDEP_PIPIS_VES: "ves", MASSDEP_PIPIS_KACHAEV: "kachaev"}[md])
    else:
        bw = np.ones_like(mI, dtype=np.complex128)
    amp = np.zeros(len(phi), dtype=np.complex128)
    if canonical:
        rb = opts.get("reflectivity_basis", True)
        for m in range(-j, j + 1, 2):
            if w["bachelor_first"]:
                s1, m1, s2, m2 = 0, 0, j, m
            else:
                s1, m1, s2, m2 = j, m, 0, 0
            top = _canonical_two_body(J, M, P, refl, L, S, s1, m1, s2, m2, theta, phi, qX, 1.0, True, rb)
            iso_amp = _canonical_two_body(j, m, 0, 0, l, s, 0, 0, 0, 0, thetah, phih, qI, bw, False, rb)
            amp += top * iso_amp
        return amp
    fX = math.sqrt(L + 1) * barrier_factor(L, qX)
    fI = math.sqrt(l + 1) * barrier_factor(l, qI) * bw
    for lam_iso in range(-j, j + 1, 2):
        # X -> daughter1 + daughter2: helicities (lambda1, lambda2)
        if w["bachelor_first"]:
            s1, l1, s2, l2 = 0, 0, j, lam_iso
        else:
            s1, l1, s2, l2 = j, lam_iso, 0, 0
        lam = l1 - l2
        cg = clebsch_gordan(L, 0, S, lam, J, lam) * clebsch_gordan(s1, l1, s2, -l2, S, lam)
        if cg == 0:
            continue
        if opts.get("reflectivity_basis", True):
            DX = D_refl_conj(J, M, lam, P, refl, phi, theta)
        else:
            DX = D_conj(J, M, lam, phi, theta)
        cgI = clebsch_gordan(l, 0, s, 0, j, 0) * clebsch_gordan(0, 0, 0, 0, s, 0)
        if cgI == 0:
            continue
        DI = D_conj(j, lam_iso, 0, phih, thetah)
        amp += (fX * cg * DX) * (fI * cgI * DI)
    return amp


def sym_terms(w, species, opts):
    """isobarAmplitude::initSymTermMaps (isobarAmplitude.cc:265-330): every
    isospin term combined with every Bose term, map[i] = bose[iso[i]],
    factor iso * bose."""
    n = len(species)
    if opts.get("isospin"):
        iso = isospin_terms(w, species, *opts["isospin"])
    else:
        iso = [(list(range(n)), 1.0)]
    if opts.get("bose", True):
        perms, fb = bose_terms(species)
        bose = [(list(p), fb) for p in perms]
    else:
        bose = [(list(range(n)), 1.0)]
    return [([pb[pi[i]] for i in range(n)], fi * fb) for pi, fi in iso for pb, fb in bose]


def amplitudes(waves, beam_p, fs_p, masses, beam_mass, species, **opts):
    """complex128 [W, N] amplitudes of the waves for events given by the beam
    momentum (N, 3) and the final-state momenta (3, N, 3).  opts: bose,
    reflectivity_basis, space_inversion, reflection, formalism ("helicity" or
    "canonical"), isospin = (isospins, isospin projections, parities) of the
    final-state particles (doubled) to isospin-symmetrise (the waves then
    carry "isospin" and "isobar_isospin")."""
    beam = _lv(np.asarray(beam_p, dtype=np.float64), beam_mass)
    fs_p = np.asarray(fs_p, dtype=np.float64)
    out = np.zeros((len(waves), beam.shape[0]), dtype=np.complex128)
    for k, w in enumerate(waves):
        for p, factor in sym_terms(w, species, opts):
            if factor == 0:
                continue
            # slot i takes the momentum of particle p[i] (decayTopology::revertMomenta)
            fs = [_lv(fs_p[p[i]], masses[i]) for i in range(len(masses))]
            out[k] += factor * _sym_term(w, beam, fs, masses, opts)
    return out


def wave(J, P, M, refl, L, S, isobar_J, isobar_L, mass_dep, isobar_mass=0.0, isobar_width=0.0,
         isobar_daughters=(0, 1), bachelor=2, bachelor_first=False, isobar_S=0, isospin=2, isobar_isospin=0,
         bounds=(0.0, 0.0), mass_dep_params=()):
    """one wave's description (all spins and isospins doubled; bounds: the
    isobar mass bin of the binned mass dependence; mass_dep_params: those of
    the K pi S-wave forms)."""
    return dict(J=J, P=P, M=M, refl=refl, L=L, S=S, isobar_J=isobar_J, isobar_L=isobar_L, isobar_S=isobar_S,
                mass_dep=mass_dep, isobar_mass=isobar_mass, isobar_width=isobar_width,
                isobar_daughters=tuple(isobar_daughters), bachelor=bachelor, bachelor_first=bool(bachelor_first),
                isospin=isospin, isobar_isospin=isobar_isospin, bounds=tuple(bounds),
                mass_dep_params=tuple(mass_dep_params))
