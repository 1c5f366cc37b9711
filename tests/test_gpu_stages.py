"""Stage-by-stage parity with the oracle on the golden inputs.

After the move phase the friends-of-friends groups must be identical
(membership and numbering); unbinding fed the oracle's own groups and
centres (through the unbind-only entry point, kdInGroup/kdReadCenter) must
unbind exactly the same particles."""
import numpy as np
import pytest

from oracle import oracle
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu

STAGE_CASES = ["dark4k_open_dmin", "dark4k_periodic", "dark8k_lcdm", "gasdark6k_gd", "mixed6k",
               "dark4k_plummer_eps"]


def _ctx(opts):
    from skid_gb300 import gpu
    return gpu.Context(period=opts.period if opts.periodic else None, periodic=opts.periodic,
                       nSmooth=opts.nSmooth)


@pytest.mark.parametrize("name", STAGE_CASES)
def test_fof_groups_identical(gpu_ready, name):
    from skid_gb300 import pipeline
    snap, opts, ref, counts, meta = gc.load(name)
    r1 = oracle.run(snap, opts, stop_after=1)
    with _ctx(opts) as ctx:
        ctx.set_particles(snap)
        ctx.scatter_active(opts.bGasAndDark, opts.bGasOnly)
        ctx.density()
        na = ctx.init_move(opts.fDensMin, opts.fTempMax, opts.fMassMax, opts.bGasAndDark,
                           opts.bGasOnly)
        initial = (snap.n_gas == 0 and snap.n_star == 0) or opts.bForceInitialCut
        ctx.move_step(opts.fStep, initial, opts.bNoScatterCut)
        it = 0
        while na:
            na, _ = ctx.move_iterate(opts.fStep, opts.fCvg, opts.bNoScatterCut)
            it += 1
        ng = ctx.fof(opts.fTau)
        ctx.reactivate_move()
        for _ in range(pipeline.PRUNE_STEPS):
            ctx.move_step(np.float32(pipeline.MICRO_STEP * opts.fStep), False, opts.bNoScatterCut)
        ctx.group_centers()
        grp, rec = ctx.get_groups(ng)
    assert ng == r1["nGroupFoF"]
    assert np.array_equal(grp, r1["grp"])
    og = r1["groups"]
    # moved particles end jittering about their peak by up to a step, and the
    # float field sums differ in order from the oracle's FP64 ones
    assert np.abs(rec["rCenter"][1:] - og["rCenter"][1:]).max() < 0.1 * opts.fStep
    np.testing.assert_allclose(rec["fMass"][1:], og["fMass"][1:], rtol=1e-6)
    np.testing.assert_allclose(rec["vcm"][1:], og["vcm"][1:], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("name", STAGE_CASES)
def test_unbind_isolated(gpu_ready, name):
    from skid_gb300 import gpu
    snap, opts, ref, counts, meta = gc.load(name)
    r1 = oracle.run(snap, opts, stop_after=1)
    # the groups go in as in unbind-only mode (each group's reference point is
    # then its largest-iOrder member), so the oracle runs that mode too
    centers = np.concatenate([r1["groups"]["rCenter"][1:], r1["groups"]["vcm"][1:]], axis=1)
    r2 = oracle.run_unbind(snap, opts, r1["grp"], centers, stop_after=2)
    ng = r1["nGroupFoF"]
    cen = np.zeros(ng + 1, gpu.GROUP_DTYPE)
    cen["rCenter"] = r1["groups"]["rCenter"]
    cen["vcm"] = r1["groups"]["vcm"]
    with _ctx(opts) as ctx:
        ctx.set_particles(snap)
        ctx.set_groups(r1["grp"], cen)
        if opts.bEps:
            ctx.set_soft(opts.fEps)
        nu = ctx.unbind(opts.iSoftType, opts.fScoop, opts.bGasAndDark, opts.bNoUnbind,
                        opts.nMaxMembers, opts.G, opts.z, opts.a_shift, opts.a_hubble)
        grp, rec = ctx.get_groups(ng)
    assert nu == r2["nUnbound"]
    assert np.array_equal(grp, r2["grp"])
    og = r2["groups"]
    keep = og["nMembers"][1:] > 0
    np.testing.assert_allclose(rec["fMass"][1:][keep], og["fMass"][1:][keep], rtol=1e-6)
    np.testing.assert_allclose(rec["vcm"][1:][keep], og["vcm"][1:][keep], rtol=1e-4, atol=1e-6)
    assert np.abs(rec["rBound"][1:][keep] - og["rBound"][1:][keep]).max() < 1e-5


@pytest.mark.parametrize("name", ["dark4k_periodic", "mixed6k"])
def test_schedules_and_unfused_forms_agree(gpu_ready, name):
    """Every removal schedule the autotuner can pick, the per-group launch
    loop, and the unfused field-then-move form give the same catalogue."""
    from skid_gb300 import pipeline
    snap, opts, ref, counts, meta = gc.load(name)
    settings = [{}, {"unbind_warp_max": 0, "unbind_block": 256},
                {"unbind_warp_max": 128, "unbind_block": 1024},
                {"unbind_warp_max": 32, "unbind_block": 512},
                {"unbind_warp_max": 64, "unbind_block": 128},
                {"unbind_warp_max": 1024, "unbind_block": 256},
                {"unbind_per_group": 1}, {"field_unfused": 1}]
    outs = []
    for setting in settings:
        with _ctx(opts) as ctx:
            for k, v in setting.items():
                ctx.set_option(k, v)
            res = pipeline.run(snap, opts, ctx=ctx)
            outs.append((res.grp.copy(), res.groups.copy(), ctx.get_option("unbind_warp_max"),
                         ctx.get_option("unbind_block"), ctx.get_option("unbind_tune_candidates")))
    base_grp, base_rec = outs[0][0], outs[0][1]
    assert outs[0][2] in (0, 32, 128, 256, 512, 1024) and outs[0][3] in (256, 512, 1024)
    assert outs[0][4] == 18
    for (grp, rec, *_), setting in zip(outs[1:], settings[1:]):
        assert np.array_equal(grp, base_grp), setting
        for f in ("nMembers", "fMass", "rCenter", "rBound", "vcm", "fRadius"):
            assert np.array_equal(rec[f], base_rec[f]), (setting, f)


def test_unbind_large_groups_fp32_path(gpu_ready):
    """Groups above 1024 members take the staged-energy removal paths (one
    block per group, or one thread-block cluster per group with the members
    in the blocks' shared memory): unbind-only mode on three groups of
    1790-4075 members, with a twelfth of their members sped up fourfold so
    that each loses 89-203 of them one by one, must unbind exactly the
    particles the oracle's FP64 loop unbinds, for every block size."""
    from skid_gb300 import gpu, tipsy
    from skid_gb300.options import Options
    from tests.helpers import small_snapshot
    snap = small_snapshot(n=12288, n_halo=3, seed=41, r200=0.1, frac=0.85, dex=0.5)
    opts = Options.parse(["-tau", "0.012", "-s", "64", "-m", "16", "-p", "1", "-O", "0.3",
                          "-Lambda", "0.7", "-H", "5.28444", "-z", "0.5"])
    r1 = oracle.run(snap, opts, stop_after=1)
    cnt = np.bincount(r1["grp"])
    big = np.nonzero(cnt[1:] > 1024)[0] + 1
    assert len(big) >= 2
    rng = np.random.default_rng(5)
    vel = snap.vel.copy()
    for g in big:
        m = np.nonzero(r1["grp"] == g)[0]
        vel[rng.choice(m, len(m) // 12, replace=False)] *= 4.0
    snap = tipsy.Snapshot(snap.time, snap.n_gas, snap.n_dark, snap.n_star, snap.pos, vel,
                          snap.mass, snap.soft, snap.temp)
    centers = np.concatenate([r1["groups"]["rCenter"][1:], r1["groups"]["vcm"][1:]], axis=1)
    r2 = oracle.run_unbind(snap, opts, r1["grp"], centers, stop_after=2)
    ng = r1["nGroupFoF"]
    cen = np.zeros(ng + 1, gpu.GROUP_DTYPE)
    cen["rCenter"] = r1["groups"]["rCenter"]
    cen["vcm"] = r1["groups"]["vcm"]
    removed = cnt[big] - np.bincount(r2["grp"], minlength=len(cnt))[big]
    assert removed.min() >= 50
    # block sizes, and the thread-block-cluster path (groups above 1025
    # members shared by a cluster of blocks holding them in shared memory)
    for bs, tw, cmin in ((256, 1024, 0), (512, 1024, 0), (1024, 1024, 0), (256, 512, 1025),
                         (512, 512, 1025), (1024, 256, 1025)):
        with _ctx(opts) as ctx:
            ctx.set_option("unbind_warp_max", tw)
            ctx.set_option("unbind_block", bs)
            ctx.set_option("unbind_cluster_min", cmin)
            ctx.set_particles(snap)
            ctx.set_groups(r1["grp"], cen)
            nu = ctx.unbind(opts.iSoftType, opts.fScoop, opts.bGasAndDark, opts.bNoUnbind,
                            opts.nMaxMembers, opts.G, opts.z, opts.a_shift, opts.a_hubble)
            grp, rec = ctx.get_groups(ng)
            nclu = ctx.get_option("unbind_cluster_groups")
        assert (nclu >= len(big)) if cmin else (nclu == 0), (bs, cmin, nclu)
        assert nu == r2["nUnbound"], (bs, cmin)
        assert np.array_equal(grp, r2["grp"]), (bs, cmin)
        og = r2["groups"]
        np.testing.assert_allclose(rec["fMass"][big], og["fMass"][big], rtol=1e-6)
        np.testing.assert_allclose(rec["vcm"][big], og["vcm"][big], rtol=1e-4, atol=1e-6)


def test_unbind_isolated_config1_2e21(gpu_ready):
    """Unbinding at the benchmarked size: the 2^21 clustered workload's
    friends-of-friends groups and centres (from the GPU's own move phase) go
    into the GPU's unbind-only path and the oracle's; both must unbind
    exactly the same particles.  Hundreds of its groups hold more than 1024
    members (up to about 10^4, with hundreds of removals each), so this
    covers the staged FP32-filtered removal path at scale, every pair factor
    against the oracle's FP64 one, and the scoop terms."""
    from skid_gb300 import gpu, pipeline
    snap, opts, ref, counts, meta = gc.load("config1_2e21")
    with _ctx(opts) as ctx:
        ctx.set_particles(snap)
        ctx.scatter_active(opts.bGasAndDark, opts.bGasOnly)
        ctx.density()
        na = ctx.init_move(opts.fDensMin, opts.fTempMax, opts.fMassMax, opts.bGasAndDark,
                           opts.bGasOnly)
        ctx.move_step(opts.fStep, True, opts.bNoScatterCut)
        while na:
            na, _ = ctx.move_iterate(opts.fStep, opts.fCvg, opts.bNoScatterCut)
        ng = ctx.fof(opts.fTau)
        ctx.reactivate_move()
        for _ in range(pipeline.PRUNE_STEPS):
            ctx.move_step(np.float32(pipeline.MICRO_STEP * opts.fStep), False, opts.bNoScatterCut)
        ctx.group_centers()
        grp0, rec0 = ctx.get_groups(ng)
    # the groups fed to both unbinders are the GPU's own; their count is the
    # reference's to within the pipeline test's tolerance
    assert abs(ng - counts["nGroupFoF"]) <= int(1e-4 * counts["nGroupFoF"])
    sizes = np.bincount(grp0, minlength=ng + 1)[1:]
    assert np.count_nonzero(sizes > 1024) >= 100
    centers = np.concatenate([rec0["rCenter"][1:], rec0["vcm"][1:]], axis=1)
    r2 = oracle.run_unbind(snap, opts, grp0, centers, stop_after=2)
    cen = np.zeros(ng + 1, gpu.GROUP_DTYPE)
    cen["rCenter"] = rec0["rCenter"]
    cen["vcm"] = rec0["vcm"]
    big = np.nonzero(sizes > 1024)[0] + 1
    lost_big = int(np.sum(sizes[big - 1] - np.bincount(r2["grp"], minlength=ng + 1)[big]))
    assert lost_big > 10000
    og = r2["groups"]
    keep = og["nMembers"][1:] > 0
    # the tuned schedule; the fixed one the skid tool uses (no clusters
    # unless asked for); and that one with the largest groups on
    # thread-block clusters (their members in the blocks' shared memory)
    fixed = {"unbind_warp_max": 1024, "unbind_block": 512}
    for setting in ({}, fixed, dict(fixed, unbind_cluster_min=2048)):
        with _ctx(opts) as ctx:
            for k, v in setting.items():
                ctx.set_option(k, v)
            ctx.set_particles(snap)
            ctx.set_groups(grp0, cen)
            nu = ctx.unbind(opts.iSoftType, opts.fScoop, opts.bGasAndDark, opts.bNoUnbind,
                            opts.nMaxMembers, opts.G, opts.z, opts.a_shift, opts.a_hubble)
            grp, rec = ctx.get_groups(ng)
            if "unbind_cluster_min" in setting:
                assert ctx.get_option("unbind_cluster_groups") > 0
            elif setting:
                assert ctx.get_option("unbind_cluster_groups") == 0
        assert nu == r2["nUnbound"], setting
        assert np.array_equal(grp, r2["grp"]), setting
        np.testing.assert_allclose(rec["fMass"][1:][keep], og["fMass"][1:][keep], rtol=1e-6)
        assert np.abs(rec["rBound"][1:][keep] - og["rBound"][1:][keep]).max() < 1e-5
