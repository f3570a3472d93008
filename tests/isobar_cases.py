"""Wave sets and events shared by the isobar-amplitude tests: seeded
synthetic diffractive three-pion events (pi- pi+ pi-) and waves covering
every mass dependence, both daughter orders at the X vertex, spins 0..4 of X
and 0..3 of the isobar, M = 0..2 and both reflectivities.  Every wave
conserves parity (P = (-1)^(L + l + 1) for three pseudoscalars)."""
import numpy as np

from oracle import isobar_oracle as O
from rootpwa_gb300 import synth

M_RHO, G_RHO = 0.7690, 0.1509
M_F2, G_F2 = 1.2751, 0.1851
M_RHO3, G_RHO3 = 1.6888, 0.161
SPECIES = [0, 1, 0]              # pi-, pi+, pi-
NAMES = ["pi-", "pi+", "pi-"]


def waves():
    """(oracle description, keyword arguments of isobarHelicityAmplitudes.addWave)."""
    specs = [
        # J  P  M refl L  S  j  l  massdep          mass    width  daughters bachelor first
        (2, +1, 0, +1, 0, 2, 2, 2, O.MASSDEP_REL_BW, M_RHO, G_RHO, (1, 2), 0, False),   # 1++0+ rho S
        (2, +1, 2, +1, 0, 2, 2, 2, O.MASSDEP_REL_BW, M_RHO, G_RHO, (1, 2), 0, False),   # 1++1+ rho S
        (4, -1, 2, +1, 2, 2, 2, 2, O.MASSDEP_REL_BW, M_RHO, G_RHO, (1, 2), 0, False),   # 2-+1+ rho P
        (4, +1, 2, -1, 4, 2, 2, 2, O.MASSDEP_REL_BW, M_RHO, G_RHO, (1, 2), 0, True),    # 2++1- rho D, bachelor first
        (0, -1, 0, +1, 0, 0, 0, 0, O.MASSDEP_FLAT, 0.0, 0.0, (1, 2), 0, False),          # 0-+0+ flat isobar
        (4, -1, 0, +1, 4, 4, 4, 4, O.MASSDEP_CONST_BW, M_F2, G_F2, (1, 2), 0, False),   # 2-+0+ f2 S (const width)
        (8, +1, 2, +1, 4, 6, 6, 6, O.MASSDEP_REL_BW, M_RHO3, G_RHO3, (2, 1), 0, False),  # 4++1+ rho3 D
        (4, -1, 4, -1, 0, 4, 4, 4, O.MASSDEP_REL_BW, M_F2, G_F2, (0, 1), 2, False),     # 2-+2- f2 S, other pair
        (2, +1, 2, +1, 0, 2, 2, 2, O.MASSDEP_RHO_BW, M_RHO, G_RHO, (1, 2), 0, False),   # 1++1+ rho S (rho BW)
        (0, -1, 0, +1, 0, 0, 0, 0, O.MASSDEP_F0980_BW, 0.980, 0.070, (1, 2), 0, False),  # 0-+0+ f0(980) S
        (2, +1, 2, +1, 2, 0, 0, 0, O.MASSDEP_F0980_FLATTE, 0.0, 0.0, (1, 2), 0, True),   # 1++1+ f0(980) P (Flatte)
        (0, -1, 0, +1, 0, 0, 0, 0, O.MASSDEP_PIPIS_M, 0.0, 0.0, (1, 2), 0, False),      # 0-+0+ (pi pi)_S AMP M
        (4, -1, 0, +1, 4, 0, 0, 0, O.MASSDEP_PIPIS_VES, 0.0, 0.0, (2, 1), 0, False),    # 2-+0+ (pi pi)_S D, VES
        (2, +1, 2, +1, 2, 0, 0, 0, O.MASSDEP_PIPIS_KACHAEV, 0.0, 0.0, (1, 2), 0, True),  # 1++1+ (pi pi)_S P, Kachaev
        (0, -1, 0, +1, 0, 0, 0, 0, O.MASSDEP_BINNED, 0.6, 0.9, (1, 2), 0, False),       # 0-+0+ freed (pi pi)_S bin
        (2, -1, 2, +1, 2, 2, 2, 2, O.MASSDEP_RHO_PRIME, 0.0, 0.0, (1, 2), 0, False),    # 1-+1+ rho' P (exotic)
        (2, +1, 0, -1, 0, 2, 2, 2, O.MASSDEP_REL_BW, M_RHO, G_RHO, (1, 2), 0, False),   # 1++0- (zero by reflectivity)
    ]
    out = []
    md = {O.MASSDEP_FLAT: "flat", O.MASSDEP_REL_BW: "relativisticBreitWigner",
          O.MASSDEP_CONST_BW: "constWidthBreitWigner", O.MASSDEP_RHO_BW: "rhoBreitWigner",
          O.MASSDEP_F0980_BW: "f0980BreitWigner", O.MASSDEP_F0980_FLATTE: "f0980FlatteBesII",
          O.MASSDEP_PIPIS_M: "piPiSWaveAuMorganPenningtonM", O.MASSDEP_PIPIS_VES: "piPiSWaveAuMorganPenningtonVes",
          O.MASSDEP_PIPIS_KACHAEV: "piPiSWaveAuMorganPenningtonKachaev", O.MASSDEP_BINNED: "binned",
          O.MASSDEP_RHO_PRIME: "rhoPrime"}
    for J, P, M, r, L, S, j, l, m, mass, width, dau, bach, first in specs:
        bounds = (mass, width) if m == O.MASSDEP_BINNED else (0.0, 0.0)
        ow = O.wave(J, P, M, r, L, S, j, l, m, mass, width, dau, bach, first, bounds=bounds)
        kw = dict(J=J, P=P, M=M, refl=r, L=L, S=S, isobarJ=j, isobarL=l, massDependence=md[m], isobarMass=mass,
                  isobarWidth=width, isobarDaughters=dau, bachelor=bach, bachelorFirst=first, bounds=bounds)
        out.append((ow, kw))
    return out


def events(n, seed=0):
    return synth.three_pion_events(n, seed=seed)


def rel_err(A, B):
    """max |A - B| per wave, relative to the wave's largest |A| (0 for a zero wave)."""
    out = []
    for a, b in zip(A, B):
        s = np.abs(a).max()
        out.append(np.abs(a - b).max() / s if s > 0 else np.abs(b).max())
    return np.array(out)


# FP64 tolerance: the lab momenta are ~190 GeV/c and the frames boost by
# gamma ~ 100, so both FP64 restatements carry ~1e-10 relative rounding
# (the oracle's own rotation invariance holds to ~6e-11)
TOL = 1e-9
# complex64 mode (FP64 frames, FP32 per-wave arithmetic): measured <= 5e-7
TOL32 = 5e-6


def tolerances(ws, base):
    """per-wave tolerance: base, ten times base for the f0(980) Flatte form,
    whose K K threshold cusp (d amp / dm ~ 1/sqrt(m - 2 m_K)) turns the
    ~1e-11 differences between the two restatements' isobar masses into up
    to ~3e-9 of the amplitude for events next to the threshold."""
    return np.array([base * (10 if w["mass_dep"] == O.MASSDEP_F0980_FLATTE else 1) for w, _ in ws])


# pi- pi0 pi0: slot 0 pi-, slots 1 and 2 pi0 (identical)
NEUTRAL_SPECIES = [0, 1, 1]
NEUTRAL_NAMES = ["pi-", "pi0", "pi0"]
NEUTRAL_MASSES = (0.13957039, 0.1349768, 0.1349768)
NEUTRAL_ISOSPIN = ([2, 2, 2], [-2, 0, 0], [-1, -1, -1])     # 2I, 2I_3, intrinsic parity


def neutral_waves():
    """pi- pi0 pi0 waves with X isospin 1: rho- pi0 (the isobar from the pi-
    and one pi0), f2 and f0(980) to pi0 pi0, and a wave keyed as rho0 pi- that
    isospin symmetrisation turns into rho- pi0 terms."""
    specs = [
        # J  P  M refl L  S  j  l  massdep             mass   width  daughters bachelor first  I_isobar
        (2, +1, 0, +1, 0, 2, 2, 2, O.MASSDEP_REL_BW, M_RHO, G_RHO, (0, 1), 2, False, 2),   # 1++0+ rho- pi0 S
        (4, +1, 2, +1, 4, 2, 2, 2, O.MASSDEP_REL_BW, M_RHO, G_RHO, (0, 1), 2, True, 2),    # 2++1+ rho- pi0 D
        (4, -1, 0, +1, 0, 4, 4, 4, O.MASSDEP_REL_BW, M_F2, G_F2, (1, 2), 0, False, 0),     # 2-+0+ f2 pi- S
        (0, -1, 0, +1, 0, 0, 0, 0, O.MASSDEP_F0980_BW, 0.980, 0.070, (1, 2), 0, False, 0),  # 0-+0+ f0 pi- S
        (2, +1, 0, +1, 0, 2, 2, 2, O.MASSDEP_REL_BW, M_RHO, G_RHO, (1, 2), 0, False, 2),   # 1++0+ "rho0" pi- S
    ]
    md = {O.MASSDEP_REL_BW: "relativisticBreitWigner", O.MASSDEP_F0980_BW: "f0980BreitWigner"}
    out = []
    for J, P, M, r, L, S, j, l, m, mass, width, dau, bach, first, Ii in specs:
        ow = O.wave(J, P, M, r, L, S, j, l, m, mass, width, dau, bach, first, isospin=2, isobar_isospin=Ii)
        kw = dict(J=J, P=P, M=M, refl=r, L=L, S=S, isobarJ=j, isobarL=l, massDependence=md[m], isobarMass=mass,
                  isobarWidth=width, isobarDaughters=dau, bachelor=bach, bachelorFirst=first, isospin=2,
                  isobarIsospin=Ii)
        out.append((ow, kw))
    return out


def neutral_events(n, seed=0):
    return synth.three_pion_events(n, seed=seed, masses=NEUTRAL_MASSES)


# K- pi+ pi-: slot 0 K-, slot 1 pi+, slot 2 pi- (no identical particles)
KPIPI_SPECIES = [0, 1, 2]
KPIPI_NAMES = ["K-", "pi+", "pi-"]
KPIPI_MASSES = (0.493677, 0.13957039, 0.13957039)
# LASS-type K pi S-wave parameters: a, r, M0, G0, phiF, phiR, phiRsin, F, R, MMax
GLASS = (1.95, 1.76, 1.435, 0.279, 0.0, 0.0, 0.0, 1.0, 1.0, 1.9)


def kpipi_waves():
    """K- pi+ pi- waves: K*(892) pi S, the K pi S-wave (LASS and
    Palano-Pennington forms) pi S, and rho(770) K S."""
    specs = [
        (2, +1, 0, +1, 0, 2, 2, 2, O.MASSDEP_REL_BW, 0.8955, 0.0473, (0, 1), 2, False, ()),
        (0, -1, 0, +1, 0, 0, 0, 0, O.MASSDEP_KPIS_GLASS, 0.0, 0.0, (0, 1), 2, False, GLASS),
        (0, -1, 0, +1, 0, 0, 0, 0, O.MASSDEP_KPIS_PALANO, 0.0, 0.0, (1, 0), 2, False, ()),
        (2, +1, 2, +1, 0, 2, 2, 2, O.MASSDEP_REL_BW, M_RHO, G_RHO, (1, 2), 0, True, ()),
    ]
    md = {O.MASSDEP_REL_BW: "relativisticBreitWigner", O.MASSDEP_KPIS_GLASS: "KPiSGLASS",
          O.MASSDEP_KPIS_PALANO: "KPiSPalanoPennington"}
    out = []
    for J, P, M, r, L, S, j, l, m, mass, width, dau, bach, first, par in specs:
        ow = O.wave(J, P, M, r, L, S, j, l, m, mass, width, dau, bach, first, mass_dep_params=par)
        kw = dict(J=J, P=P, M=M, refl=r, L=L, S=S, isobarJ=j, isobarL=l, massDependence=md[m], isobarMass=mass,
                  isobarWidth=width, isobarDaughters=dau, bachelor=bach, bachelorFirst=first, massDepParams=par)
        out.append((ow, kw))
    return out


def kpipi_events(n, seed=0):
    return synth.three_pion_events(n, seed=seed, masses=KPIPI_MASSES, m_lo=1.0, m_hi=2.4)
