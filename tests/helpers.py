"""Shared test inputs: small seeded clustered snapshots."""
import numpy as np

from skid_gb300 import synth, tipsy


def small_snapshot(n=4096, n_halo=8, seed=11, r200=0.08, frac=0.6, dex=1.5, gas_frac=0.0,
                   n_star=0):
    spec = synth.HaloSpec(n, n_halo, dex, (5.0, 15.0), r200, frac, seed, gas_frac=gas_frac)
    snap = synth.make_snapshot(spec)
    if n_star:
        # turn the last n_star particles into stars (iOrder order gas, dark, star)
        snap = tipsy.Snapshot(snap.time, snap.n_gas, snap.n_dark - n_star, n_star, snap.pos,
                              snap.vel, snap.mass, snap.soft, snap.temp)
    return snap


def rel_err(a, b, floor=0.0):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)
