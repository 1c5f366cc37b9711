"""The unbinding potentials' pair factor (kdCellPot/kdSubPot/kdAddScoopPot,
grav.c:25-30,50-55,118-124; SPLINE_POT, grav.h:11-31) on the GPU.

The reference forms it as a float assigned from FP64 arithmetic.  The GPU
takes a float-float form inside the softening and a float-float reciprocal
square root beyond it, and falls back to the FP64 expression only where
those cannot decide the rounding; every value must be the FP64 expression's,
bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ref_dir(d2, twoh, plummer=False):
    """The reference's expression in numpy FP64 (IEEE sqrt, divide, multiply
    and add, each correctly rounded, in grav.h's order), rounded to float."""
    r2 = d2.astype(np.float64)
    h = twoh.astype(np.float64)
    if plummer:
        return (1.0 / np.sqrt(r2 + 0.25 * h * h)).astype(np.float32)
    r = np.sqrt(r2)
    out = np.empty(len(r), np.float64)
    far = ~(r < h)
    with np.errstate(divide="ignore"):
        out[far] = 1.0 / r[far]
    i = ~far
    dih = 2.0 / h[i]
    u = r[i] * dih
    lo = u < 1.0
    ul, dl = u[lo], dih[lo]
    a = 2.0 / 3.0 * ul * ul
    b = 3.0 / 10.0 * ul * ul * ul * ul
    c = 1.0 / 10.0 * ul * ul * ul * ul * ul
    v_lo = dl * (7.0 / 5.0 - a + b - c)
    uh, dh, rh = u[~lo], dih[~lo], r[i][~lo]
    a = 4.0 / 3.0 * uh * uh
    b = uh * uh * uh
    c = 3.0 / 10.0 * uh * uh * uh * uh
    e = 1.0 / 30.0 * uh * uh * uh * uh * uh
    v_hi = -1.0 / 15.0 * (1.0 / rh) + dh * (8.0 / 5.0 - a + b - c + e)
    vi = np.empty(int(i.sum()), np.float64)
    vi[lo] = v_lo
    vi[~lo] = v_hi
    out[i] = vi
    return out.astype(np.float32)


def _inputs(seed=5):
    rng = np.random.default_rng(seed)
    n = 1 << 21
    twoh = np.exp(rng.uniform(np.log(1e-6), np.log(1e-1), n)).astype(np.float32)
    # r / 2h: mostly inside the softening, around u = 1 (r = h) and r = 2h
    t = np.concatenate([rng.uniform(0.0, 1.05, n // 2),
                        0.5 * (1.0 + rng.uniform(-1e-5, 1e-5, n // 4)),
                        1.0 + rng.uniform(-1e-6, 1e-6, n - n // 2 - n // 4)])
    d2 = ((t * twoh.astype(np.float64)) ** 2).astype(np.float32)
    # exactly representable edges: r = h (u = 1) and r = 2h, and the floats
    # next to them; d2 = 0
    k = rng.integers(1, 4096, 4096).astype(np.float64)
    h2 = (k * 2.0 ** -14).astype(np.float32)
    e_d2 = np.concatenate([(h2.astype(np.float64) / 2) ** 2, h2.astype(np.float64) ** 2]).astype(np.float32)
    e_tw = np.concatenate([h2, h2])
    e_d2 = np.concatenate([e_d2, np.nextafter(e_d2, np.float32(0)), np.nextafter(e_d2, np.float32(1)),
                           np.zeros(16, np.float32)])
    e_tw = np.concatenate([e_tw, e_tw, e_tw, np.full(16, 1e-3, np.float32)])
    return np.concatenate([d2, e_d2]), np.concatenate([twoh, e_tw])


def test_pair_factor_bit_exact(gpu_ready):
    from skid_gb300 import gpu
    d2, twoh = _inputs()
    used = gpu.pair_factor(d2, twoh, mode=gpu.PAIR_USED)
    fp64 = gpu.pair_factor(d2, twoh, mode=gpu.PAIR_FP64)
    bad = np.flatnonzero(used.view(np.uint32) != fp64.view(np.uint32))
    assert bad.size == 0, (bad.size, d2[bad[:5]], twoh[bad[:5]], used[bad[:5]], fp64[bad[:5]])
    # the FP64 expression on the GPU is the reference's (numpy restatement)
    sel = np.random.default_rng(9).choice(len(d2), 200000, replace=False)
    sel = np.concatenate([sel, np.arange(len(d2) - 3 * 8192 - 16, len(d2))])
    want = ref_dir(d2[sel], twoh[sel])
    assert np.array_equal(fp64[sel].view(np.uint32), want.view(np.uint32))
    # the float-float spline decides almost every pair inside the softening
    ff = gpu.pair_factor(d2, twoh, mode=gpu.PAIR_SPLINE_FF)
    inner = np.sqrt(d2[: 1 << 20].astype(np.float64)) < 0.98 * twoh[: 1 << 20]
    declined = np.isnan(ff[: 1 << 20][inner]).mean()
    assert declined < 0.02, declined
    ok = ~np.isnan(ff)
    assert np.array_equal(ff[ok].view(np.uint32), fp64[ok].view(np.uint32))


def test_pair_factor_plummer_and_far(gpu_ready):
    from skid_gb300 import gpu
    rng = np.random.default_rng(6)
    n = 1 << 18
    twoh = np.exp(rng.uniform(np.log(1e-6), np.log(1e-1), n)).astype(np.float32)
    d2 = ((rng.uniform(0.0, 50.0, n) * twoh.astype(np.float64)) ** 2).astype(np.float32)
    for plummer in (False, True):
        used = gpu.pair_factor(d2, twoh, plummer=plummer, mode=gpu.PAIR_USED)
        want = ref_dir(d2, twoh, plummer=plummer)
        assert np.array_equal(used.view(np.uint32), want.view(np.uint32)), plummer
