"""Edge cases of the whole pipeline on the GPU against the oracle: boxes
whose particle count is not a multiple of the 32-point leaves, a uniform box
(groups only from noise) whose groups are all too small for -m, and an empty
or negative particle count, which the library refuses."""
import numpy as np
import pytest

from oracle import oracle
from tests.helpers import small_snapshot

pytestmark = pytest.mark.gpu

H = ["-p", "1", "-H", "2.89441"]


def _vs_oracle(snap, flags):
    from skid_gb300 import compare, pipeline
    from skid_gb300.options import Options
    opts = Options.parse(flags + H)
    res = pipeline.run(snap, opts)
    ref = oracle.run(snap, opts)
    m = compare.match_groups(ref["grp"], res.grp)
    assert m.agreement >= 0.999, m.agreement
    assert m.same_groups()
    for key in ("nGroupFoF", "nGroup", "nIter"):
        assert res.counts[key] == ref[key], (key, res.counts[key], ref[key])
    assert abs(res.counts["nUnbound"] - ref["nUnbound"]) <= 2
    return res, ref


@pytest.mark.parametrize("n,k,seed", [(257, 32, 72), (1000, 64, 73), (2049, 32, 74)])
def test_ragged_small_boxes(gpu_ready, n, k, seed):
    snap = small_snapshot(n=n, n_halo=3, seed=seed, r200=0.08, frac=0.7)
    res, ref = _vs_oracle(snap, ["-tau", "0.03", "-s", str(k), "-m", "8"])
    assert res.n_group > 0


def test_uniform_box_every_group_too_small(gpu_ready):
    snap = small_snapshot(n=5000, n_halo=1, seed=71, frac=0.0)
    res, ref = _vs_oracle(snap, ["-tau", "0.02", "-s", "32", "-m", "5001"])
    assert res.counts["nGroupFoF"] > 0
    assert res.n_group == 0 and not res.grp.any()
    assert len(res.groups) == 1


def test_empty_or_negative_counts_are_refused(gpu_ready):
    from skid_gb300 import gpu, tipsy
    z = np.zeros((0, 3), np.float32)
    e = np.zeros(0, np.float32)
    with gpu.Context(period=1.0, nSmooth=32) as ctx:
        with pytest.raises(gpu.SkidError) as info:
            ctx.set_particles(tipsy.Snapshot(0.0, 0, 0, 0, z, z, e, e, e))
        assert info.value.code == -1
    lib = gpu.load()
    h = gpu.Context(period=1.0, nSmooth=32)
    try:
        one = np.zeros(3, np.float32)
        f = one.ctypes.data_as(gpu.C.POINTER(gpu.C.c_float))
        assert lib.skid_set_particles(h.h, -1, 2, 0, 0.0, f, f, f, f, f) == -1
    finally:
        h.close()
