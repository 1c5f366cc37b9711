"""kNN ball radii and SPH density on the GPU against the oracle.

fBall2 must be bit-exact (it is the k-th smallest float distance, whatever
the search order); densities within 1e-5 relative of the FP64 restatement of
smooth1.c:248-263.
"""
import numpy as np
import pytest

from oracle import oracle
from tests.helpers import rel_err, small_snapshot

pytestmark = pytest.mark.gpu

CASES = [
    (4096, 64, 1.0, 3),
    (4096, 32, None, 4),
    (3000, 128, 1.0, 5),
    (40000, 64, 1.0, 6),
]


@pytest.mark.parametrize("n,k,period,seed", CASES)
def test_ball2_and_density(gpu_ready, n, k, period, seed):
    from skid_gb300 import gpu
    snap = small_snapshot(n=n, seed=seed)
    with gpu.Context(period=period, nSmooth=k) as ctx:
        ctx.set_particles(snap)
        assert ctx.scatter_active() == n
        nextra = ctx.density()
        rho, b = ctx.get_density()
    b_or = oracle.knn_ball2(snap.pos, k, period)
    mism = np.count_nonzero(b != b_or)
    assert mism == 0, f"{mism} fBall2 values differ"
    rho_or = oracle.density(snap.pos, snap.mass, b_or, period)
    err = rel_err(rho, rho_or)
    assert err.max() < 1e-5, f"density max rel err {err.max():.3g}"
    if period is not None:
        mask = oracle.replica_mask(snap.pos, b_or, period)
        assert nextra == int(sum(bin(int(m)).count("1") - 1 for m in mask))
    else:
        assert nextra == 0


def test_knn_probe_brute(gpu_ready):
    from skid_gb300 import gpu
    rng = np.random.default_rng(7)
    pos = rng.uniform(-0.5, 0.5, (700, 3)).astype(np.float32)
    with gpu.Context(period=1.0, nSmooth=16) as ctx:
        for k in (1, 16, 100, 700):
            b = ctx.knn_ball2(pos, k)
            assert np.array_equal(b, oracle.knn_ball2(pos, k, 1.0, brute=True))


@pytest.mark.parametrize("period,G", [(1.0, 64), (None, 64), (1.0, 32), (None, 32), (1.0, 16),
                                      (1.0, 8), (None, 4), (1.0, 1)])
def test_move_field(gpu_ready, period, G):
    """The move field (minus grad rho, smooth1.c:447-459) at every particle,
    for each number of movers per warp the move step uses."""
    from skid_gb300 import gpu
    snap = small_snapshot(n=8192, seed=21)
    with gpu.Context(period=period, nSmooth=64) as ctx:
        ctx.set_option("field_movers_per_warp", G)
        ctx.set_particles(snap)
        ctx.scatter_active()
        ctx.density()
        rho, b = ctx.get_density()
        ctx.init_move()
        probe = np.concatenate([snap.pos, snap.pos[:500] + np.float32(0.003)])
        if period is not None:
            probe = (probe + 0.5) % 1.0 - 0.5
        probe = probe.astype(np.float32)
        acc = ctx.field(probe)
    mask = oracle.replica_mask(snap.pos, b, period) if period else np.full(len(b), 1 << 13, np.uint32)
    acc_or, absacc, _ = oracle.field(snap.pos, snap.mass, b, mask, probe, period)
    err = np.linalg.norm(acc - acc_or, axis=1) / np.maximum(absacc, 1e-30)
    assert err.max() < 1e-5, f"field norm-wise err {err.max():.3g}"


@pytest.mark.parametrize("period", [1.0, None])
def test_move_field_two_movers_per_lane_is_one(gpu_ready, period):
    """With 64 movers per warp each lane holds two movers, and with 32 one;
    either way a mover's hits are summed by one lane in the same order (leaves
    depth first, candidates in leaf order), so the fields are bit-identical."""
    from skid_gb300 import gpu
    snap = small_snapshot(n=8192, seed=22)
    out = []
    for G in (32, 64):
        with gpu.Context(period=period, nSmooth=64) as ctx:
            ctx.set_option("field_movers_per_warp", G)
            ctx.set_particles(snap)
            ctx.scatter_active()
            ctx.density()
            ctx.init_move()
            out.append(ctx.field(snap.pos))
    assert np.array_equal(out[0], out[1])
