"""Seeded synthetic amplitude sets that stand in for ROOTPWA's amplitude files.

No public dataset exists for the likelihood path (the reference's own
benchmark inputs are downloaded at run time), so tests and the benchmark use
synthetic decay amplitudes with the shapes of the standard workloads:

* ``compass15``: 15 positive-reflectivity waves + flat, rank 1, 20,000 data
  and 100,000 MC events; A_w = sigma_w (x + i y), x, y ~ N(0, 1),
  sigma_w log-uniform in [0.1, 10]; acceptance Bernoulli(0.6) on MC events.
* ``compass88``: the 88-wave COMPASS 3pi wave-set shape, 7 negative + 80
  positive reflectivity waves + flat, rank 2, 1,000,000 data and 5,000,000 MC
  events; A_w = sigma_w (z_w + sum_k B_wk C_k) / sqrt(2) with independent
  z_w ~ CN(0, 1), an 8-dimensional complex latent C ~ CN(0, 1) per event and a
  fixed complex mixing B (entries CN(0, 1/8)), which correlates the waves
  while keeping the integral matrix full rank.
* ``multibin50``: 50 positive waves + flat, rank 1 (per mass / t' bin).

Production amplitudes have re/im ~ N(0, 1) in the reference's parameter
layout.  All draws are float32 (the device store is complex64); the FP64
oracle receives the complex128 cast of the very same values.

For the decay-amplitude step: ``three_pion_events`` draws diffractive
pi- p -> (pi- pi+ pi-) p events (lab momenta) and ``three_pion_waves`` lists a
COMPASS-like 3pi isobar wave set.
"""
import numpy as np

WORKLOADS = {
    "compass15": dict(n_neg=0, n_pos=15, rank=1, n_data=20_000, n_mc=100_000, mixing=0),
    "compass88": dict(n_neg=7, n_pos=80, rank=2, n_data=1_000_000, n_mc=5_000_000, mixing=8),
    "multibin50": dict(n_neg=0, n_pos=50, rank=1, n_data=40_000, n_mc=200_000, mixing=0),
}


def wave_names(n_neg, n_pos):
    """Wave names and reflectivities in wave-list order (negative waves first)."""
    names = ["wave%03d_neg" % i for i in range(n_neg)] + ["wave%03d_pos" % i for i in range(n_pos)]
    refl = [-1] * n_neg + [+1] * n_pos
    return names, refl


def n_pars(n_neg, n_pos, rank):
    """Parameter count of the reference layout (pwaLikelihood.cc:1495-1516)."""
    p = 0
    for r in range(rank):
        pos, neg = n_pos - r, n_neg - r
        p += 2 * (max(pos - 1, 0) + max(neg - 1, 0))
        p += (1 if pos > 0 else 0) + (1 if neg > 0 else 0)
    return p + 1


class AmplitudeModel:
    """Per-wave scales and (optionally) the low-rank mixing of one workload."""

    def __init__(self, n_waves, mixing, rng):
        self.n_waves = n_waves
        self.sigma = np.exp(rng.uniform(np.log(0.1), np.log(10.0), n_waves)).astype(np.float32)
        self.mixing = mixing
        if mixing:
            B = (rng.standard_normal((n_waves, mixing)) + 1j * rng.standard_normal((n_waves, mixing)))
            self.B = (B / np.sqrt(2.0 * mixing)).astype(np.complex64)

    def draw(self, rng, n_events, chunk=1 << 18):
        """complex64 amplitudes [wave][event]."""
        W = self.n_waves
        out = np.empty((W, n_events), dtype=np.complex64)
        for b in range(0, n_events, chunk):
            m = min(chunk, n_events - b)
            z = np.empty((W, m), dtype=np.complex64)
            z.real = rng.standard_normal((W, m), dtype=np.float32)
            z.imag = rng.standard_normal((W, m), dtype=np.float32)
            if self.mixing:
                c = np.empty((self.mixing, m), dtype=np.complex64)
                c.real = rng.standard_normal((self.mixing, m), dtype=np.float32)
                c.imag = rng.standard_normal((self.mixing, m), dtype=np.float32)
                z = (z + self.B @ c) * np.float32(1.0 / np.sqrt(2.0))
            out[:, b:b + m] = z * self.sigma[:, None]
        return out


def draw_device(model, n_events, seed, device="cuda"):
    """Same distribution as AmplitudeModel.draw, generated on the GPU with
    torch (for workloads too large to draw on the host quickly); returns a
    contiguous complex64 tensor [wave][event]."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    W = model.n_waves
    z = torch.complex(torch.randn(W, n_events, generator=g, device=device),
                      torch.randn(W, n_events, generator=g, device=device))
    if model.mixing:
        c = torch.complex(torch.randn(model.mixing, n_events, generator=g, device=device),
                          torch.randn(model.mixing, n_events, generator=g, device=device))
        z = (z + torch.from_numpy(model.B).to(device) @ c) * (1.0 / np.sqrt(2.0))
    z = z * torch.from_numpy(model.sigma).to(device)[:, None]
    return z.to(torch.complex64).contiguous()


def make_workload(name="compass15", seed=0, n_data=None, n_mc=None, rank=None, acceptance=0.6):
    """Builds one synthetic workload.

    Returns a dict with names, refl, rank, data [W][N] complex64,
    mc [W][M] complex64, accepted [M] bool and par [P] float64."""
    cfg = dict(WORKLOADS[name])
    if n_data is not None:
        cfg["n_data"] = n_data
    if n_mc is not None:
        cfg["n_mc"] = n_mc
    if rank is not None:
        cfg["rank"] = rank
    rng = np.random.Generator(np.random.PCG64(seed))
    names, refl = wave_names(cfg["n_neg"], cfg["n_pos"])
    model = AmplitudeModel(len(names), cfg["mixing"], rng)
    data = model.draw(rng, cfg["n_data"])
    mc = model.draw(rng, cfg["n_mc"])
    accepted = rng.random(cfg["n_mc"]) < acceptance
    P = n_pars(cfg["n_neg"], cfg["n_pos"], cfg["rank"])
    par = rng.standard_normal(P)
    return dict(name=name, names=names, refl=refl, rank=cfg["rank"], data=data, mc=mc, accepted=accepted,
                par=par, n_neg=cfg["n_neg"], n_pos=cfg["n_pos"])


# ---------------------------------------------------------------------------
# Multibin workloads: bins whose data follow the model intensity of a known
# production-amplitude vector
# ---------------------------------------------------------------------------
def multibin_event_counts(n_bins=400, median=40_000, sigma_ln=1.0, lo=2_000, hi=400_000, seed=0):
    """Events per bin: LogNormal(ln median, sigma_ln) truncated to [lo, hi]
    (draws outside the range are redrawn)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = np.empty(n_bins, dtype=np.int64)
    k = 0
    while k < n_bins:
        n = int(round(np.exp(rng.normal(np.log(median), sigma_ln))))
        if lo <= n <= hi:
            out[k] = n
            k += 1
    return out


def true_production_amplitudes(n_waves, rng):
    """V_true: re/im ~ N(0, 1) per wave, flat amplitude |N(0, 1)|."""
    v = rng.standard_normal(n_waves) + 1j * rng.standard_normal(n_waves)
    return v.astype(np.complex128), float(abs(rng.standard_normal()))


def draw_bin_device(model, v_true, flat, n_events, seed, pool_factor=4, device="cuda"):
    """Data events of one bin, importance-resampled from phase-space draws in
    proportion to the rank-1 intensity |sum_w V_w A_w|^2 + flat^2 (multinomial
    resampling with replacement from a pool of pool_factor * n_events draws).
    Returns complex64 [wave][event] on the device.

    The same seed gives the same events in every process: the intensities
    come from elementwise products and fixed-order reductions, the
    cumulative distribution and the uniform draws from numpy on the host (a
    library matrix-vector product or a device-side cumulative sum may round
    differently from run to run, which moves a few resampled events)."""
    import torch
    pool = draw_device(model, pool_factor * n_events, seed=seed, device=device)
    vr = torch.from_numpy(v_true.real.astype(np.float32)).to(device)[:, None]
    vi = torch.from_numpy(v_true.imag.astype(np.float32)).to(device)[:, None]
    pr, pi = pool.real, pool.imag
    sr = (vr * pr - vi * pi).sum(dim=0)
    si = (vr * pi + vi * pr).sum(dim=0)
    inten = (sr * sr + si * si + np.float32(flat * flat)).double().cpu().numpy()
    cdf = np.cumsum(inten)
    u = np.random.Generator(np.random.PCG64(int(seed) + 7919)).random(n_events) * cdf[-1]
    idx = np.minimum(np.searchsorted(cdf, u, side="right"), len(cdf) - 1)
    return pool[:, torch.from_numpy(idx).to(device)].contiguous()


# -- three-pion events and waves for the decay-amplitude step ---------------------

M_PI = 0.13957039


def _rotation(axis, a):
    c, s = np.cos(a), np.sin(a)
    o, z = np.ones_like(a), np.zeros_like(a)
    m = {"y": [[c, z, s], [z, o, z], [-s, z, c]], "z": [[c, -s, z], [s, c, z], [z, z, o]]}[axis]
    return np.moveaxis(np.array(m), (0, 1), (-2, -1))


def _boost(p, E, b):
    b2 = np.sum(b * b, axis=-1)
    g = 1.0 / np.sqrt(1.0 - b2)
    bp = np.sum(b * p, axis=-1)
    g2 = np.where(b2 > 0, (g - 1.0) / np.where(b2 > 0, b2, 1.0), 0.0)
    return p + (g2 * bp)[:, None] * b + (g * E)[:, None] * b


def three_pion_events(n, seed=0, beam_momentum=190.0, m_lo=0.9, m_hi=2.2, masses=None):
    """Seeded diffractive events pi- p -> (pi- pi+ pi-) p: the beam along z
    with a small divergence, X of mass uniform in [m_lo, m_hi] GeV/c^2 with a
    small transverse momentum, decaying by three-body phase space (uniform in
    the Dalitz plane).  Returns beam (N, 3), final state (3, N, 3) lab
    momenta in GeV/c (particle order pi-, pi+, pi-), the three masses and the
    beam mass.  masses: other final-state masses (e.g. pi- pi0 pi0)."""
    rng = np.random.default_rng(seed)
    m1, m2, m3 = (M_PI, M_PI, M_PI) if masses is None else masses
    beam = np.stack([rng.normal(0, 0.05, n), rng.normal(0, 0.05, n), np.full(n, beam_momentum)], axis=1)
    MX = rng.uniform(m_lo, m_hi, n)
    pX = beam.copy()
    pX[:, 0] += rng.normal(0, 0.3, n)
    pX[:, 1] += rng.normal(0, 0.3, n)
    pX[:, 2] *= rng.uniform(0.95, 1.0, n)
    EX = np.sqrt(MX ** 2 + np.sum(pX ** 2, axis=1))
    rest = np.zeros((3, n, 4))
    todo = np.arange(n)
    while todo.size:
        M = MX[todo]
        s12 = rng.uniform((m1 + m2) ** 2, (M - m3) ** 2)
        s23 = rng.uniform((m2 + m3) ** 2, (M - m1) ** 2)
        E3 = (M * M + m3 * m3 - s12) / (2 * M)
        E1 = (M * M + m1 * m1 - s23) / (2 * M)
        E2 = M - E1 - E3
        p1, p2, p3 = [np.sqrt(np.maximum(E * E - mm * mm, 0)) for E, mm in ((E1, m1), (E2, m2), (E3, m3))]
        ok = (E1 > m1) & (E2 > m2) & (E3 > m3)
        with np.errstate(invalid="ignore", divide="ignore"):
            c13 = (p2 ** 2 - p1 ** 2 - p3 ** 2) / (2 * p1 * p3)
        ok &= np.abs(c13) < 1
        good = np.nonzero(ok)[0]
        if good.size:
            idx = todo[good]
            c = c13[good]
            z0 = np.zeros(good.size)
            v1 = np.stack([z0, z0, p1[good]], axis=1)
            v3 = p3[good][:, None] * np.stack([np.sqrt(1 - c * c), z0, c], axis=1)
            v2 = -(v1 + v3)
            a, b, g = (rng.uniform(0, 2 * np.pi, good.size), np.arccos(rng.uniform(-1, 1, good.size)),
                       rng.uniform(0, 2 * np.pi, good.size))
            R = np.einsum("nij,njk->nik", _rotation("z", a),
                          np.einsum("nij,njk->nik", _rotation("y", b), _rotation("z", g)))
            for i, (v, E) in enumerate(((v1, E1), (v2, E2), (v3, E3))):
                rest[i, idx, :3] = np.einsum("nij,nj->ni", R, v)
                rest[i, idx, 3] = E[good]
        todo = todo[~ok]
    bX = pX / EX[:, None]
    fs = np.stack([_boost(rest[i, :, :3], rest[i, :, 3], bX) for i in range(3)])
    return beam, fs, np.array([m1, m2, m3]), M_PI


# isobars of the 3pi wave sets: (name, 2J, mass, width, mass dependence;
# mass and width unused by the fixed-parameter pi pi S-wave)
PIPI_ISOBARS = [
    ("sigma", 0, 0.0, 0.0, "piPiSWaveAuMorganPenningtonKachaev"),      # the (pi pi)_S isobar
    ("rho(770)", 2, 0.7690, 0.1509, "relativisticBreitWigner"),
    ("f0(980)", 0, 0.980, 0.070, "relativisticBreitWigner"),
    ("f2(1270)", 4, 1.2751, 0.1851, "relativisticBreitWigner"),
    ("f0(1500)", 0, 1.505, 0.109, "relativisticBreitWigner"),
    ("rho3(1690)", 6, 1.6888, 0.161, "relativisticBreitWigner"),
]


def three_pion_waves(n_waves=88, n_neg=8, max_J=6, max_L=8):
    """A COMPASS-like pi- pi+ pi- wave set: X -> isobar(pi+ pi-) + pi- with
    every isobar above, J = 0..3, M = 0..2, parity-conserving L
    (P = (-1)^(L + l + 1) for three pseudoscalars), L <= 4, ordered by J,
    isobar and L: the first n_waves - n_neg waves of reflectivity +1 and the
    first n_neg of reflectivity -1.  Returns keyword arguments of
    isobarHelicityAmplitudes.addWave (spins doubled)."""
    out = []
    for refl, n in ((+1, n_waves - n_neg), (-1, n_neg)):
        out += _waves_of_reflectivity(refl, max_J, max_L)[:n]
    return out


def _waves_of_reflectivity(refl, max_J, max_L):
    waves = []
    for J in range(0, max_J + 1, 2):
        for P in (-1, +1):
            for M in range(0, min(J, 4) + 1, 2):
                # reflectivity basis: M = 0 exists only for refl * P * (-1)^J = -1
                if M == 0 and refl * P * (-1) ** (J // 2) == +1:
                    continue
                for name, j, mass, width, md in PIPI_ISOBARS:
                    for L in range(0, max_L + 1, 2):
                        # parity of three pseudoscalars; J from L x S with S = isobar spin
                        if (-1) ** (L // 2 + j // 2 + 1) != P or not (abs(L - j) <= J <= L + j):
                            continue
                        waves.append(dict(J=J, P=P, M=M, refl=refl, L=L, S=j, isobarJ=j, isobarL=j,
                                          massDependence=md, isobarMass=mass, isobarWidth=width,
                                          isobarDaughters=(1, 2), bachelor=0, isobarName=name))
    return waves
