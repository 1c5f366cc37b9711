"""skid_batch_run: many uneven volumes at once give, volume by volume, the
results of running each volume alone."""
import numpy as np
import pytest

from tests.helpers import small_snapshot

pytestmark = pytest.mark.gpu


def test_batch_matches_single_volume_runs(gpu_ready):
    from skid_gb300 import gpu, pipeline
    from skid_gb300.options import Options
    rng = np.random.default_rng(41)
    vols = []
    for i, n in enumerate([3000, 20000, 6000, 12000, 4500, 9000]):
        snap = small_snapshot(n=n, n_halo=max(2, n // 1500), seed=100 + i, r200=0.06)
        k = int(rng.choice([32, 64, 128]))
        tau = float(np.float32(0.5 * n ** (-1.0 / 3.0)))
        vols.append((snap, k, tau))
    base = Options.parse(["-tau", "0.01", "-m", "8", "-p", "1", "-H", "2.89441"])
    out = gpu.batch_run(vols, base, n_workers=3)
    for (snap, k, tau), r in zip(vols, out):
        assert r["status"] == 0
        opts = Options.parse(["-tau", repr(tau), "-s", str(k), "-m", "8", "-p", "1",
                              "-H", "2.89441"])
        single = pipeline.run(snap, opts)
        assert np.array_equal(r["grp"], single.grp)
        assert r["nGroup"] == single.n_group
        assert r["nGroupFoF"] == single.counts["nGroupFoF"]
        assert r["nUnbound"] == single.counts["nUnbound"]
        for f in ("nMembers", "fMass", "rCenter", "vcm", "rBound", "fRadius"):
            assert np.array_equal(r["groups"][f], single.groups[f]), f


def test_batch_rejects_bad_arguments(gpu_ready):
    from skid_gb300 import gpu
    lib = gpu.load()
    assert lib.skid_batch_run(None, 1, None, 1, 0) == -1


def test_batch_volumes_match_the_oracle(gpu_ready):
    """Three volumes of the uneven-subvolume workload's generator (each its
    own N, halo count, nSmooth and tau = 0.5 N^(-1/3), with the workload's
    cosmology flags), run together through skid_batch_run, each against the
    oracle's restatement of reference skid on the same volume."""
    from oracle import oracle
    from skid_gb300 import compare, gpu, synth
    from skid_gb300.options import Options
    specs = synth.subvolume_specs(3, seed=synth.SEED_BASE + 12, lo=12.5, hi=13.5)
    vols = [(synth.make_snapshot(spec), k, tau) for spec, k, tau in specs]
    rest = ["-m", "16", "-p", "1", "-O", "0.3", "-Lambda", "0.7",
            "-H", f"{synth.hubble_for(0.3):.6g}"]
    out = gpu.batch_run(vols, Options.parse(["-tau", "0.01"] + rest), n_workers=3)
    for (snap, k, tau), r in zip(vols, out):
        assert r["status"] == 0
        opts = Options.parse(["-tau", repr(float(np.float32(tau))), "-s", str(k)] + rest)
        ref = oracle.run(snap, opts)
        m = compare.match_groups(ref["grp"], r["grp"])
        assert m.agreement >= 0.999, (snap.n, k, m.agreement)
        assert m.same_groups(), (snap.n, k)
        assert r["nGroupFoF"] == ref["nGroupFoF"], (snap.n, k)
        assert r["nGroup"] == ref["nGroup"], (snap.n, k)
        assert r["nIter"] == ref["nIter"], (snap.n, k)
        assert abs(r["nUnbound"] - ref["nUnbound"]) <= max(2, snap.n // 1000), (snap.n, k)
