"""Adjoints of the density, the density field and the group potential energy.

CPU tests pin the FP64 references: analytic gradients against central finite
differences (step 1e-6 box units), and the density-field gradient against
the oracle's restatement of the reference's move field (smAccDensity), which
is minus that gradient.  GPU tests compare the hand-written adjoint kernels
(FP32) with those references on random particles: the error norm of each
gradient over the sum of the norms of its terms must stay below 1e-5.
"""
import numpy as np
import pytest

from oracle import oracle
from tests.helpers import small_snapshot

TOL = 1e-5          # GPU FP32 adjoint vs FP64, norm-wise over sum |term|
FD_TOL = 1e-6       # FP64 analytic vs FP64 central differences


def _rel(a, b, absterm):
    return np.linalg.norm(np.asarray(a, np.float64) - b, axis=1) / np.maximum(absterm, 1e-300)


# ---- FP64 pair potential of kdCellPot (grav.h:11-31) and psi'(r)/r ----

def psi_fp64(r, twoh, plummer):
    r = np.asarray(r, np.float64)
    twoh = np.broadcast_to(np.asarray(twoh, np.float64), r.shape)
    if plummer:
        t = 1.0 / np.sqrt(r * r + 0.25 * twoh * twoh)
        return t, -t ** 3
    dih = 2.0 / twoh
    u = r * dih
    psi = np.empty_like(r)
    gr = np.empty_like(r)
    a = u < 1.0
    b = (u >= 1.0) & (r < twoh)
    c = r >= twoh
    ua = u[a]
    psi[a] = dih[a] * (1.4 - 2.0 / 3.0 * ua ** 2 + 0.3 * ua ** 4 - 0.1 * ua ** 5)
    gr[a] = dih[a] ** 3 * (-4.0 / 3.0 + 1.2 * ua ** 2 - 0.5 * ua ** 3)
    ub, rb = u[b], r[b]
    psi[b] = -1.0 / 15.0 / rb + dih[b] * (1.6 - 4.0 / 3.0 * ub ** 2 + ub ** 3 - 0.3 * ub ** 4
                                          + ub ** 5 / 30.0)
    gr[b] = 1.0 / 15.0 / rb ** 3 + dih[b] ** 3 * (-8.0 / 3.0 + 3.0 * ub - 1.2 * ub ** 2 + ub ** 3 / 6.0)
    psi[c] = 1.0 / r[c]
    gr[c] = -1.0 / r[c] ** 3
    return psi, gr


def group_energy_fp64(x, m, eps, G, plummer, chunk=256):
    """E = -1/2 sum_{i != j} G m_i m_j psi(r_ij, eps_i + eps_j), dE/dx and the
    sum of |term| per member, FP64 (row chunks keep memory bounded)."""
    x = np.asarray(x, np.float64)
    m = np.asarray(m, np.float64)
    eps = np.asarray(eps, np.float64)
    n = len(x)
    E = 0.0
    grad = np.zeros((n, 3))
    absterm = np.zeros(n)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        d = x[a:b, None, :] - x[None, :, :]
        r = np.sqrt((d * d).sum(-1))
        off = np.ones_like(r, dtype=bool)
        off[np.arange(b - a), np.arange(a, b)] = False
        rr = np.where(off, r, 1.0)
        psi, gr = psi_fp64(rr, eps[a:b, None] + eps[None, :], plummer)
        mm = m[a:b, None] * m[None, :]
        E += -0.5 * G * (mm * psi * off).sum()
        t = (mm * gr * off)[:, :, None] * d
        grad[a:b] = -G * t.sum(1)
        absterm[a:b] = G * np.linalg.norm(t, axis=2).sum(1)
    return E, grad, absterm


def energy_change_fp64(x, m, eps, G, plummer, i, xi_new):
    """E(x with x_i -> xi_new) - E(x): only the pairs with i change."""
    x = np.asarray(x, np.float64)
    mask = np.arange(len(x)) != i

    def part(xi):
        r = np.sqrt(((x[mask] - xi) ** 2).sum(-1))
        psi, _ = psi_fp64(r, eps[i] + eps[mask], plummer)
        return -G * m[i] * (m[mask] * psi).sum()
    return part(np.asarray(xi_new, np.float64)) - part(x[i])


def _wrap_rel(x, rel, L):
    d = (x - rel).astype(np.float32)
    h = np.float32(0.5 * L)
    d = np.where(d > h, d - np.float32(2) * h, d)
    d = np.where(d <= -h, d + np.float32(2) * h, d)
    return d.astype(np.float32)


# ---- CPU: the FP64 references themselves ----

@pytest.mark.parametrize("period", [1.0, None])
def test_fp64_density_adjoint_matches_central_differences(period):
    snap = small_snapshot(n=6000, n_halo=6, seed=21, r200=0.08)
    rng = np.random.default_rng(5)
    w = rng.standard_normal(snap.n).astype(np.float32)
    sel = rng.choice(snap.n, 200, replace=False)
    an, fd, ab = oracle.density_adjoint_check(snap.pos, snap.mass, w, 32, period, sel, h=1e-6)
    assert _rel(an, fd, ab).max() < FD_TOL


def test_fp64_field_gradient_is_minus_the_reference_move_field():
    snap = small_snapshot(n=6000, n_halo=6, seed=22, r200=0.08)
    b2 = oracle.knn_ball2(snap.pos, 32, 1.0)
    rng = np.random.default_rng(6)
    y = snap.pos[rng.choice(snap.n, 200, replace=False)] + rng.normal(0, 0.003, (200, 3))
    y = ((y + 0.5) % 1.0 - 0.5).astype(np.float32)
    an, fd, ab = oracle.field_grad_check(snap.pos, snap.mass, b2, 1.0, y, h=1e-6)
    assert _rel(an, fd, ab).max() < FD_TOL
    alive = oracle.replica_mask(snap.pos, b2, 1.0)
    acc, absacc, _ = oracle.field(snap.pos, snap.mass, b2, alive, y, 1.0)
    assert _rel(-acc, an, ab).max() < TOL


@pytest.mark.parametrize("plummer", [False, True])
def test_fp64_potential_gradient_matches_central_differences(plummer):
    rng = np.random.default_rng(7)
    n = 300
    x = rng.normal(0, 0.01, (n, 3))
    m = rng.uniform(0.5, 1.5, n) / n
    eps = np.full(n, 0.004)
    E, grad, ab = group_energy_fp64(x, m, eps, 1.0, plummer)
    h = 1e-6
    for i in rng.choice(n, 20, replace=False):
        for d in range(3):
            xp = x.copy(); xp[i, d] += h
            xm = x.copy(); xm[i, d] -= h
            fd = (group_energy_fp64(xp, m, eps, 1.0, plummer)[0]
                  - group_energy_fp64(xm, m, eps, 1.0, plummer)[0]) / (2 * h)
            assert abs(fd - grad[i, d]) < FD_TOL * ab[i]
            e = np.zeros(3); e[d] = h
            fd2 = (energy_change_fp64(x, m, eps, 1.0, plummer, i, x[i] + e)
                   - energy_change_fp64(x, m, eps, 1.0, plummer, i, x[i] - e)) / (2 * h)
            assert abs(fd2 - grad[i, d]) < FD_TOL * ab[i]


# ---- GPU: the adjoint kernels ----

def _density_ctx(snap, k, period):
    from skid_gb300 import gpu
    ctx = gpu.Context(period=period, nSmooth=k)
    ctx.set_particles(snap)
    ctx.scatter_active(False, False)
    ctx.density()
    return ctx


@pytest.mark.gpu
@pytest.mark.parametrize("period,k", [(1.0, 64), (None, 32)])
def test_density_adjoint_vs_fp64(gpu_ready, period, k):
    from skid_gb300 import gpu
    snap = small_snapshot(n=32768, n_halo=20, seed=23, r200=0.05)
    rng = np.random.default_rng(8)
    w = rng.standard_normal(snap.n).astype(np.float32)
    sel = rng.choice(snap.n, 1024, replace=False)
    an, fd, ab = oracle.density_adjoint_check(snap.pos, snap.mass, w, k, period, sel, h=1e-6)
    with _density_ctx(snap, k, period) as ctx:
        g_walk = ctx.density_adjoint(w, gpu.ADJ_RECOMPUTE)
        g_list = ctx.density_adjoint(w, gpu.ADJ_STORED)
        g_list2 = ctx.density_adjoint(w, gpu.ADJ_STORED)    # reuses the stored lists
    for g in (g_walk, g_list):
        assert _rel(g[sel], an, ab).max() < TOL
        assert _rel(g[sel], fd, ab).max() < TOL
    assert np.array_equal(g_list, g_list2) or _rel(g_list[sel], g_list2[sel], ab).max() < 1e-6


@pytest.mark.gpu
def test_density_adjoint_other_cotangent_and_linearity(gpu_ready):
    """L is linear in w: the adjoint of w1 + 2 w2 is the sum of the adjoints."""
    from skid_gb300 import gpu
    snap = small_snapshot(n=20000, n_halo=10, seed=24, r200=0.06)
    rng = np.random.default_rng(9)
    w1 = rng.standard_normal(snap.n).astype(np.float32)
    w2 = rng.standard_normal(snap.n).astype(np.float32)
    with _density_ctx(snap, 64, 1.0) as ctx:
        a = ctx.density_adjoint(w1).astype(np.float64)
        b = ctx.density_adjoint(w2).astype(np.float64)
        c = ctx.density_adjoint(w1 + 2 * w2).astype(np.float64)
    scale = np.abs(a).max() + 2 * np.abs(b).max()
    assert np.abs(c - (a + 2 * b)).max() < 1e-5 * scale


@pytest.mark.gpu
def test_field_adjoint_vs_fp64_and_reference_field(gpu_ready):
    snap = small_snapshot(n=32768, n_halo=20, seed=25, r200=0.05)
    k = 64
    rng = np.random.default_rng(10)
    y = snap.pos[rng.choice(snap.n, 1024, replace=False)] + rng.normal(0, 0.002, (1024, 3))
    y = ((y + 0.5) % 1.0 - 0.5).astype(np.float32)
    w = rng.standard_normal(1024).astype(np.float32)
    with _density_ctx(snap, k, 1.0) as ctx:
        _, b2 = ctx.get_density()
        g = ctx.field_adjoint(y, w)
    an, fd, ab = oracle.field_grad_check(snap.pos, snap.mass, b2, 1.0, y, h=1e-6)
    alive = oracle.replica_mask(snap.pos, b2, 1.0)
    acc, _, _ = oracle.field(snap.pos, snap.mass, b2, alive, y, 1.0)
    assert _rel(g, w[:, None] * an, np.abs(w) * ab).max() < TOL
    assert _rel(g, w[:, None] * fd, np.abs(w) * ab).max() < TOL
    assert _rel(g, -w[:, None] * acc, np.abs(w) * ab).max() < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("soft_type", [2, 1])
def test_potential_adjoint_vs_fp64(gpu_ready, soft_type):
    from skid_gb300 import gpu, pipeline
    from skid_gb300.options import Options
    snap = small_snapshot(n=32768, n_halo=24, seed=26, r200=0.05)
    opts = Options.parse(["-tau", "0.01", "-s", "64", "-m", "16", "-p", "1"])
    with gpu.Context(period=1.0, nSmooth=64) as ctx:
        ctx.set_particles(snap)
        ctx.scatter_active(False, False)
        ctx.density()
        ctx.init_move(opts.fDensMin, opts.fTempMax, opts.fMassMax, False, False)
        ctx.move_step(opts.fStep, True, False)
        n_act = 1
        while n_act:
            n_act, _ = ctx.move_iterate(opts.fStep, opts.fCvg, False)
        ng = ctx.fof(opts.fTau)
        ctx.group_centers()
        grp, rec = ctx.get_groups(ng)
        sizes = np.bincount(grp, minlength=ng + 1)[1:]
        sel = (np.argsort(-sizes, kind="stable")[:200] + 1).astype(np.int32)
        rng = np.random.default_rng(11)
        v = rng.standard_normal(len(sel)).astype(np.float32)
        E, grad = ctx.potential_adjoint(sel, v, G=1.0, soft_type=soft_type)
    plummer = soft_type == 1
    members = {int(g): np.flatnonzero(grp == g) for g in sel}
    xs, abs_ = {}, {}
    for s, g in enumerate(sel):
        idx = members[int(g)]
        x = _wrap_rel(snap.pos[idx], rec["rel"][g], 1.0)
        e64, g64, ab = group_energy_fp64(x, snap.mass[idx], snap.soft[idx], 1.0, plummer)
        assert abs(E[s] - e64) <= 1e-5 * abs(e64)
        assert _rel(grad[idx], v[s] * g64, abs(v[s]) * ab).max() < TOL
        xs[s], abs_[s] = x.astype(np.float64), ab
    # central differences (step 1e-6) of the FP64 energy at 1024 random members
    picks = [(s, i) for s in range(len(sel)) for i in range(len(members[int(sel[s])]))]
    rng = np.random.default_rng(12)
    h = 1e-6
    for k in rng.choice(len(picks), min(1024, len(picks)), replace=False):
        s, i = picks[k]
        idx = members[int(sel[s])]
        x = xs[s]
        for d in range(3):
            e = np.zeros(3); e[d] = h
            fd = (energy_change_fp64(x, snap.mass[idx], snap.soft[idx], 1.0, plummer, i, x[i] + e)
                  - energy_change_fp64(x, snap.mass[idx], snap.soft[idx], 1.0, plummer, i, x[i] - e)) / (2 * h)
            assert abs(grad[idx[i], d] - v[s] * fd) < TOL * abs(v[s]) * abs_[s][i]
