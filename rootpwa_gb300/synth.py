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
    Returns complex64 [wave][event] on the device."""
    import torch
    pool = draw_device(model, pool_factor * n_events, seed=seed, device=device)
    v = torch.from_numpy(v_true.astype(np.complex64)).to(device)
    s = v @ pool
    inten = (s.real * s.real + s.imag * s.imag + flat * flat).float()
    g = torch.Generator(device=device)
    g.manual_seed(int(seed) + 7919)
    idx = torch.multinomial(inten, n_events, replacement=True, generator=g)
    return pool[:, idx].contiguous()
