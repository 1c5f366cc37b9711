"""The torch.autograd.Function wrappers: a backward pass through torch gives
the adjoint kernels' gradients (the same library calls, driven by torch)."""
import numpy as np
import pytest

from tests.helpers import small_snapshot

pytestmark = pytest.mark.gpu


def test_sph_density_backward_is_the_density_adjoint(gpu_ready):
    torch = pytest.importorskip("torch")
    from skid_gb300 import autograd, gpu
    snap = small_snapshot(n=16384, n_halo=10, seed=31, r200=0.06)
    rng = np.random.default_rng(13)
    w = rng.standard_normal(snap.n).astype(np.float32)
    pos = torch.tensor(snap.pos, requires_grad=True)
    rho = autograd.sph_density(pos, torch.tensor(snap.mass), nSmooth=64, period=1.0)
    (torch.tensor(w) * rho).sum().backward()
    with gpu.Context(period=1.0, nSmooth=64) as ctx:
        ctx.set_particles(snap)
        ctx.scatter_active(False, False)
        ctx.density()
        want_rho, _ = ctx.get_density()
        want = ctx.density_adjoint(w, gpu.ADJ_RECOMPUTE)
    assert np.array_equal(rho.detach().numpy(), want_rho)
    got = pos.grad.numpy()
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


def test_group_potential_backward_is_the_potential_adjoint(gpu_ready):
    torch = pytest.importorskip("torch")
    from skid_gb300 import autograd
    from tests.test_adjoint import group_energy_fp64, _wrap_rel
    rng = np.random.default_rng(14)
    n = 3000
    centres = rng.uniform(-0.4, 0.4, (5, 3))
    grp = rng.integers(0, 6, n).astype(np.int32)          # 0 = ungrouped
    pos = (centres[np.maximum(grp, 1) - 1] + rng.normal(0, 0.01, (n, 3))).astype(np.float32)
    mass = np.full(n, 1.0 / n, np.float32)
    soft = np.full(n, 0.002, np.float32)
    sel = np.array([1, 3, 5], np.int32)
    v = rng.standard_normal(3).astype(np.float32)
    tpos = torch.tensor(pos, requires_grad=True)
    E = autograd.group_potential(tpos, torch.tensor(mass), torch.tensor(soft), torch.tensor(grp),
                                 torch.tensor(sel), G=1.0, period=1.0)
    (torch.tensor(v, dtype=torch.float64) * E).sum().backward()
    g = tpos.grad.numpy()
    for s, gid in enumerate(sel):
        idx = np.flatnonzero(grp == gid)
        rel = pos[idx[-1]]                                  # the largest-iOrder member
        x = _wrap_rel(pos[idx], rel, 1.0)
        e64, g64, ab = group_energy_fp64(x, mass[idx], soft[idx], 1.0, False)
        assert abs(float(E[s]) - e64) <= 1e-5 * abs(e64)
        err = np.linalg.norm(g[idx] - v[s] * g64, axis=1) / (abs(v[s]) * ab)
        assert err.max() < 1e-5
    assert np.all(g[grp == 0] == 0) and np.all(g[grp == 2] == 0) and np.all(g[grp == 4] == 0)
