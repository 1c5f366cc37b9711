"""Seeded synthetic clustered particle sets (NFW halos + background).

skid ships no benchmark data; the workloads are synthetic stand-ins shaped
like the snapshots skid is run on: a periodic unit box centred on 0 (skid's
``-p 1``), total mass 1 (mean density 1) and G = 1.

Halo masses are log-uniform over ``dex`` decades and normalised so the halos
hold ``halo_frac`` of the particles; r200 scales as M^(1/3) with the largest
equal to ``r200_max``; concentrations are uniform in ``conc``; radii come from
the inverse CDF of the truncated NFW enclosed mass mu(x) = ln(1+x) - x/(1+x),
x <= c; directions are isotropic and centres uniform.  Halo particles get an
isotropic Gaussian velocity of dispersion sqrt(G M / (2 r200)) about a bulk
velocity; the background is uniform with small Gaussian velocities.  Dark
softening is eps = 0.02 N^(-1/3).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import tipsy

SEED_BASE = 0x5C1D


@dataclasses.dataclass(frozen=True)
class HaloSpec:
    n: int                   # particles
    n_halo: int              # number of halos
    dex: float               # halo mass range in decades
    conc: tuple              # concentration range
    r200_max: float          # r200 of the most massive halo
    halo_frac: float         # fraction of particles in halos
    seed: int
    gas_frac: float = 0.0    # fraction of particles that are gas (mixed runs)
    gas_mass_ratio: float = 0.2
    gas_temp: float = 1.0e4
    background: str = "uniform"   # or "grf": Zel'dovich-displaced Gaussian random field


# The workloads.  Skid flags that go with each are in WORKLOAD_FLAGS.
CONFIGS = {
    0: HaloSpec(32768, 20, 1.5, (5.0, 15.0), 0.05, 0.60, SEED_BASE + 0),
    1: HaloSpec(1 << 21, 800, 3.0, (4.0, 20.0), 0.02, 0.55, SEED_BASE + 1),
    3: HaloSpec(1 << 20, 400, 3.0, (4.0, 20.0), 0.02, 0.55, SEED_BASE + 3),
    4: HaloSpec(1 << 24, 6000, 3.5, (4.0, 20.0), 0.02, 0.50, SEED_BASE + 4, gas_frac=0.5,
                background="grf"),
}


def config1_spec(n: int) -> HaloSpec:
    """The 2^21 clustered workload's generator at another particle count in the
    same unit box: halos in proportion to N (800 at 2^21), the same mass
    range, concentrations, largest r200 and seed."""
    if n == CONFIGS[1].n:
        return CONFIGS[1]
    return HaloSpec(n, max(1, round(800 * n / CONFIGS[1].n)), 3.0, (4.0, 20.0), 0.02, 0.55,
                    SEED_BASE + 1)


# A 32768-particle slice of the mixed-species generator (12 halos, the same
# species mix, mass range, concentrations and background as the 2^24
# workload, largest r200 0.05) and its flags (tau scaled to the slice's
# spacing): a case small enough for reference skid on one core.
CONFIG4_SLICE = HaloSpec(1 << 15, 12, 3.5, (4.0, 20.0), 0.05, 0.50, SEED_BASE + 4, gas_frac=0.5,
                         background="grf")


def config4_slice_flags() -> list:
    return ["-tau", "0.016", "-s", "64", "-m", "16", "-p", "1", "-O", "0.3", "-Lambda", "0.7",
            "-z", "0.5", "-gd", "-H", f"{hubble_for(0.3):.6g}"]


def hubble_for(omega0: float) -> float:
    """Self-consistent H0 for G=1, mean density 1: H0 = sqrt(8 pi / (3 Omega0))."""
    return math.sqrt(8.0 * math.pi / (3.0 * omega0))


def _nfw_x(u: np.ndarray, c: np.ndarray) -> np.ndarray:
    """Solve mu(x) = u mu(c) for x in [0, c] by bisection (mu is increasing)."""
    mu = lambda x: np.log1p(x) - x / (1.0 + x)
    target = u * mu(c)
    lo = np.zeros_like(u)
    hi = np.array(c, dtype=np.float64, copy=True)
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        below = mu(mid) < target
        lo = np.where(below, mid, lo)
        hi = np.where(below, hi, mid)
    return 0.5 * (lo + hi)


def grf_displacement(rng, ngrid: int, slope: float = -2.0, rms_cells: float = 0.5):
    """Zel'dovich displacement field of a Gaussian random field with power
    spectrum P(k) ~ k^slope on an ngrid^3 periodic grid: psi(k) = i k / k^2
    delta(k), scaled so the rms displacement is rms_cells grid cells.
    Returns an (ngrid, ngrid, ngrid, 3) float32 array in box units."""
    k1 = np.fft.fftfreq(ngrid) * ngrid
    kr = np.fft.rfftfreq(ngrid) * ngrid
    kx, ky, kz = np.meshgrid(k1, k1, kr, indexing="ij")
    k2 = kx * kx + ky * ky + kz * kz
    k2[0, 0, 0] = 1.0
    amp = np.sqrt(k2 ** (0.5 * slope))
    amp[0, 0, 0] = 0.0
    noise = rng.normal(size=(ngrid, ngrid, ngrid))
    delta = np.fft.rfftn(noise) * amp
    psi = np.empty((ngrid, ngrid, ngrid, 3), np.float32)
    for d, kd in enumerate((kx, ky, kz)):
        psi[..., d] = np.fft.irfftn(1j * kd / k2 * delta, s=(ngrid, ngrid, ngrid)).astype(np.float32)
    rms = float(np.sqrt(np.mean(np.sum(psi.astype(np.float64) ** 2, axis=-1))))
    if rms > 0:
        psi *= np.float32(rms_cells / ngrid / rms)
    return psi


def _wrap32(x: np.ndarray) -> np.ndarray:
    """Wrap float64 coordinates into [-0.5, 0.5) and round to float32 in range."""
    w = x - np.floor(x + 0.5)
    f = w.astype(np.float32)
    f[f >= np.float32(0.5)] = np.float32(-0.5)
    f[f < np.float32(-0.5)] = np.float32(-0.5)
    return f


def make_halos(spec: HaloSpec):
    """Return (pos, vel, mass, soft, temp, n_gas) in iOrder (gas first)."""
    rng = np.random.default_rng(spec.seed)
    n = spec.n
    n_halo_p = int(round(spec.halo_frac * n))
    # Halo masses and particle counts.
    logm = rng.uniform(0.0, spec.dex, spec.n_halo)
    m = 10.0 ** logm
    counts = np.floor(n_halo_p * m / m.sum()).astype(np.int64)
    rem = n_halo_p - counts.sum()
    order = np.argsort(-(n_halo_p * m / m.sum() - counts))
    counts[order[:rem]] += 1
    r200 = spec.r200_max * (m / m.max()) ** (1.0 / 3.0)
    conc = rng.uniform(spec.conc[0], spec.conc[1], spec.n_halo)
    centres = rng.uniform(-0.5, 0.5, (spec.n_halo, 3))
    bulk = rng.normal(0.0, 0.1, (spec.n_halo, 3))
    hid = np.repeat(np.arange(spec.n_halo), counts)
    u = rng.uniform(0.0, 1.0, n_halo_p)
    x = _nfw_x(u, conc[hid])
    r = x * (r200[hid] / conc[hid])
    costh = rng.uniform(-1.0, 1.0, n_halo_p)
    phi = rng.uniform(0.0, 2.0 * math.pi, n_halo_p)
    sinth = np.sqrt(1.0 - costh * costh)
    d = np.stack([sinth * np.cos(phi), sinth * np.sin(phi), costh], axis=1)
    hpos = centres[hid] + r[:, None] * d
    mhalo = counts.astype(np.float64) / n        # halo mass in units of total mass 1
    sig = np.sqrt(mhalo / (2.0 * r200))
    hvel = bulk[hid] + rng.normal(0.0, 1.0, (n_halo_p, 3)) * sig[hid][:, None]
    nb = n - n_halo_p
    bpos = rng.uniform(-0.5, 0.5, (nb, 3))
    bvel = rng.normal(0.0, 0.05, (nb, 3))
    if spec.background == "grf" and nb > 0:
        # uniform points displaced by the field at their nearest grid cell;
        # velocities follow the displacement (linear growth, unit factor)
        ngrid = int(min(256, max(16, 2 ** round(math.log2(nb ** (1.0 / 3.0))))))
        psi = grf_displacement(rng, ngrid)
        cell = np.floor((bpos + 0.5) * ngrid).astype(np.int64) % ngrid
        disp = psi[cell[:, 0], cell[:, 1], cell[:, 2]].astype(np.float64)
        bpos = bpos + disp
        bvel = bvel + disp
    pos = np.concatenate([hpos, bpos])
    vel = np.concatenate([hvel, bvel])
    perm = rng.permutation(n)
    pos, vel = pos[perm], vel[perm]
    n_gas = int(round(spec.gas_frac * n))
    eps = 0.02 * n ** (-1.0 / 3.0)
    mass = np.full(n, 1.0, np.float64)
    mass[:n_gas] = spec.gas_mass_ratio
    mass /= mass.sum()
    temp = np.zeros(n, np.float32)
    temp[:n_gas] = spec.gas_temp
    return (_wrap32(pos), vel.astype(np.float32), mass.astype(np.float32),
            np.full(n, eps, np.float32), temp, n_gas)


def make_snapshot(spec: HaloSpec, time: float = 1.0) -> tipsy.Snapshot:
    pos, vel, mass, soft, temp, n_gas = make_halos(spec)
    n = len(mass)
    return tipsy.Snapshot(time, n_gas, n - n_gas, 0, pos, vel, mass, soft, temp)


def write_snapshot(path, snap: tipsy.Snapshot, standard: bool = False) -> None:
    gas, dark, star = tipsy.snapshot_records(snap)
    tipsy.write_tipsy(path, snap.time, gas, dark, star, standard=standard)


def subvolume_specs(n_vol: int = 96, seed: int = SEED_BASE + 2, lo: int = 14, hi: int = 20):
    """Uneven independent subvolumes: N log-uniform in [2^lo, 2^hi], halos
    proportional to N, nSmooth from {32, 64, 128}, tau = 0.5 N^(-1/3)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_vol):
        n = int(round(2.0 ** rng.uniform(lo, hi)))
        n_halo = max(1, int(round(800 * n / (1 << 21))))
        k = int(rng.choice([32, 64, 128]))
        tau = 0.5 * n ** (-1.0 / 3.0)
        spec = HaloSpec(n, n_halo, 3.0, (4.0, 20.0), 0.02, 0.55, seed * 1000 + i)
        out.append((spec, k, tau))
    return out


def config1_subvolume(index: int, parts: int = 16):
    """One of `parts` independent periodic cubes that together sample the
    2^21 clustered workload: each holds 2^21 / parts particles in a cube of
    side L = parts^(-1/3) centred on 0, so the particle mass (2^-21), number
    density, softening and flags other than -p are the full workload's.

    Halos follow the full workload's population rather than being
    renormalised per cube: 800 / parts halos per cube, masses log-uniform
    over 3 decades with the full box's expected particles per unit mass
    (so a cube's halo fraction fluctuates about 55 %), r200 = 0.02 (M /
    10^3)^(1/3), concentrations 4-20; the rest of the cube is uniform
    background.  Returns (snapshot, L as float32)."""
    full = CONFIGS[1]
    n = full.n // parts
    L = np.float32((1.0 / parts) ** (1.0 / 3.0))
    rng = np.random.default_rng(full.seed * 1000 + 7 * parts + index)
    n_halo = max(1, round(full.n_halo / parts))
    logm = rng.uniform(0.0, full.dex, n_halo)
    m = 10.0 ** logm
    mean_m = (10.0 ** full.dex - 1.0) / (full.dex * math.log(10.0))
    per_m = full.halo_frac * full.n / (full.n_halo * mean_m)
    counts = np.maximum(1, np.round(m * per_m)).astype(np.int64)
    while counts.sum() > n:                       # a cube never overfills
        counts[np.argmax(counts)] -= counts.sum() - n
    n_halo_p = int(counts.sum())
    r200 = full.r200_max * (m / 10.0 ** full.dex) ** (1.0 / 3.0)
    conc = rng.uniform(full.conc[0], full.conc[1], n_halo)
    centres = rng.uniform(-0.5, 0.5, (n_halo, 3)) * float(L)
    bulk = rng.normal(0.0, 0.1, (n_halo, 3))
    hid = np.repeat(np.arange(n_halo), counts)
    x = _nfw_x(rng.uniform(0.0, 1.0, n_halo_p), conc[hid])
    r = x * (r200[hid] / conc[hid])
    costh = rng.uniform(-1.0, 1.0, n_halo_p)
    phi = rng.uniform(0.0, 2.0 * math.pi, n_halo_p)
    sinth = np.sqrt(1.0 - costh * costh)
    d = np.stack([sinth * np.cos(phi), sinth * np.sin(phi), costh], axis=1)
    hpos = centres[hid] + r[:, None] * d
    sig = np.sqrt((counts.astype(np.float64) / full.n) / (2.0 * r200))
    hvel = bulk[hid] + rng.normal(0.0, 1.0, (n_halo_p, 3)) * sig[hid][:, None]
    nb = n - n_halo_p
    bpos = rng.uniform(-0.5, 0.5, (nb, 3)) * float(L)
    bvel = rng.normal(0.0, 0.05, (nb, 3))
    perm = rng.permutation(n)
    pos = np.concatenate([hpos, bpos])[perm] / float(L)
    vel = np.concatenate([hvel, bvel])[perm]
    pos = (_wrap32(pos).astype(np.float64) * float(L)).astype(np.float32)
    half = np.float32(0.5) * L
    pos[pos >= half] = -half
    pos[pos < -half] = -half
    eps = 0.02 * full.n ** (-1.0 / 3.0)
    snap = tipsy.Snapshot(1.0, 0, n, 0, pos, vel.astype(np.float32),
                          np.full(n, 1.0 / full.n, np.float32), np.full(n, eps, np.float32),
                          np.zeros(n, np.float32))
    return snap, L


def config1_subvolume_flags(L) -> list:
    """The 2^21 workload's flags for one of its periodic sub-volume cubes."""
    f = list(WORKLOAD_FLAGS[1])
    f[f.index("-p") + 1] = repr(float(L))
    return f


# skid command-line flags for each workload (the reference's own flag names).
WORKLOAD_FLAGS = {
    0: ["-tau", "0.01", "-s", "64", "-m", "16", "-p", "1", "-H", f"{hubble_for(1.0):.6g}"],
    1: ["-tau", "0.004", "-s", "64", "-m", "16", "-p", "1", "-O", "0.3", "-Lambda", "0.7",
        "-H", f"{hubble_for(0.3):.6g}"],
    3: ["-tau", "0.005", "-s", "64", "-m", "16", "-p", "1", "-O", "0.3", "-Lambda", "0.7",
        "-H", f"{hubble_for(0.3):.6g}"],
    4: ["-tau", "0.002", "-s", "64", "-m", "16", "-p", "1", "-O", "0.3", "-Lambda", "0.7",
        "-z", "0.5", "-gd", "-H", f"{hubble_for(0.3):.6g}"],
}
