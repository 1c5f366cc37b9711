"""The skid pipeline (main.c:347-495) driven through libskidgpu.

``run(snapshot, options)`` makes the reference's calls in the reference's
order and returns the catalogue and the per-particle outputs; ``write_outputs``
writes the .grp/.gtp/.den/.ray/.stat files like kd.c:1502-1839.  Progress
lines match the reference's stdout (main.c:402,416,436; kd.c:158,1326,1461,
1509; smooth1.c:304).
"""
from __future__ import annotations

import dataclasses
import math
import os
import sys
import time

import numpy as np

from . import gpu, tipsy
from .options import FLT_MAX, Options

PRUNE_STEPS = 5      # main.c:13
MICRO_STEP = 0.1     # main.c:14
DARK, GAS, STAR = 1, 2, 4


@dataclasses.dataclass
class Result:
    grp: np.ndarray              # final group id by iOrder
    groups: np.ndarray           # gpu.GROUP_DTYPE records, index 0 = ungrouped
    n_group: int
    rho: np.ndarray | None       # initial densities (for .den)
    stats: np.ndarray | None     # gpu.STAT_DTYPE per-group .stat columns (device)
    moved: np.ndarray | None     # moved positions (for .ray)
    counts: dict
    timings: dict
    lines: list


def _f32(x) -> float:
    return float(np.float32(x))


def run(snap: tipsy.Snapshot, opts: Options, ctx: gpu.Context | None = None, log=None,
        want_density: bool | None = None, want_moved: bool | None = None,
        upload: bool = True) -> Result:
    """upload=False re-runs on the particles already on the context's device
    (skid_restart) instead of copying the snapshot again."""
    lines = []

    def say(s):
        lines.append(s)
        if log:
            log(s)

    own = ctx is None
    if own:
        ctx = gpu.Context(period=opts.period if opts.periodic else None, center=opts.center,
                          periodic=opts.periodic, nSmooth=opts.nSmooth)
    t0 = time.perf_counter()
    try:
        say(f"nDark:{snap.n_dark} nGas:{snap.n_gas} nStar:{snap.n_star}")
        if upload:
            ctx.set_particles(snap)
        else:
            ctx.restart()
        in_type = (DARK if snap.n_dark else 0) | (GAS if snap.n_gas else 0) | (STAR if snap.n_star else 0)
        counts = {}
        rho = moved = None
        want_density = opts.bOutDens if want_density is None else want_density
        want_moved = opts.bOutRay if want_moved is None else want_moved
        if opts.bUnbindOnly:
            grp_in, centers = read_unbind_inputs(opts, snap)
            ctx.set_groups(grp_in, centers)
            n_fof = int(grp_in.max(initial=0))
        else:
            counts["nScatter"] = ctx.scatter_active(opts.bGasAndDark, opts.bGasOnly)
            nextra = ctx.density()
            counts["nExtraScat"] = nextra
            if opts.periodic:
                say(f"nExtraScat:{nextra}")
            if want_density:
                rho, _ = ctx.get_density()
            n_active = ctx.init_move(opts.fDensMin, opts.fTempMax, opts.fMassMax,
                                     opts.bGasAndDark, opts.bGasOnly)
            counts["nMove"] = n_active
            initial = in_type == DARK or opts.bForceInitialCut
            nscat = ctx.move_step(opts.fStep, initial, opts.bNoScatterCut)
            say(f"Ittr:0 nActive:{n_active} nScatter:{nscat}")
            it = 1
            while n_active:
                if opts.maxIter and it > opts.maxIter:
                    break
                n_active, nscat = ctx.move_iterate(opts.fStep, opts.fCvg, opts.bNoScatterCut)
                say(f"Ittr:{it} nActive:{n_active} nScatter:{nscat}")
                it += 1
            counts["nIter"] = it - 1
            n_fof = ctx.fof(opts.fTau)
            ctx.reactivate_move()
            micro = _f32(MICRO_STEP * opts.fStep)
            for i in range(PRUNE_STEPS):
                nscat = ctx.move_step(micro, False, opts.bNoScatterCut)
                say(f"Microstep:{i + 1} nScatter:{nscat}")
            counts["nScatFinal"] = nscat
            if want_moved:
                moved = ctx.get_moved()
            ctx.group_centers()
        if opts.bEps:
            ctx.set_soft(opts.fEps)
        say(f"Groups before Unbind:{n_fof}")
        counts["nGroupFoF"] = n_fof
        nu = ctx.unbind(opts.iSoftType, opts.fScoop, opts.bGasAndDark, opts.bNoUnbind,
                        opts.nMaxMembers, opts.G, opts.z, opts.a_shift, opts.a_hubble)
        say(f"Number of particles Unbound:{nu}")
        counts["nUnbound"] = nu
        ng = ctx.too_small(opts.nMembers)
        counts["nGroup"] = ng
        grp, rec = ctx.get_groups(ng)
        say(f"Number of Groups:{ng}")
        stats = None
        if opts.bOutStats:
            stats = ctx.group_stats(ng, opts.G, opts.a_shift, opts.a_hubble, opts.fDensMin,
                                    opts.fTempMax)
        tm = ctx.timings()
        tm["wall_s"] = time.perf_counter() - t0
        return Result(grp, rec, ng, rho, stats, moved, counts, tm, lines)
    finally:
        if own:
            ctx.close()


def read_unbind_inputs(opts: Options, snap: tipsy.Snapshot):
    """kdInGroup (kd.c:920-962) and kdReadCenter (kd.c:1083-1196) inputs."""
    name = opts.achGroup
    if name.endswith(".grp"):
        name = name[:-4]
    grp = tipsy.read_grp(name + ".grp")
    if len(grp) != snap.n:
        raise ValueError(f"ERROR: Mismatched number of particles: {len(grp)} in {name}.grp, "
                         f"{snap.n} in the TIPSY input")
    ng = int(grp.max(initial=0)) + 1
    centers = None
    gtp = name + ".gtp"
    if os.path.exists(gtp):
        star = tipsy.read_gtp(gtp, standard=opts.bStandard)
        if len(star) != ng - 1:
            raise ValueError(f"ERROR: grp and gtp files don't match: {len(star)} vs. {ng - 1}.")
        centers = np.zeros(ng, gpu.GROUP_DTYPE)
        centers["rCenter"][1:] = star["pos"]
        centers["vcm"][1:] = star["vel"]
    return grp, centers


# ---------------------------------------------------------------------------
# output files

def _fmt_lines(fmt: str, values) -> str:
    """One printf-formatted value per line (numpy's vectorised formatting)."""
    return "".join(np.char.add(np.char.mod(fmt, np.asarray(values, np.float64)), "\n"))


def write_outputs(res: Result, snap: tipsy.Snapshot, opts: Options, outdir: str = ".") -> list:
    base = os.path.join(outdir, opts.achName)
    written = []
    tipsy.write_grp(base + ".grp", res.grp)
    written.append(base + ".grp")
    star = np.zeros(res.n_group, tipsy.STAR_DT)
    g = res.groups[1:res.n_group + 1]
    star["mass"] = g["fMass"]
    star["pos"] = g["rCenter"]
    star["vel"] = g["vcm"]
    star["eps"] = g["fRadius"]
    star["tform"] = np.float32(snap.time)
    tipsy.write_tipsy(base + ".gtp", snap.time, star=star, standard=opts.bStandard)
    written.append(base + ".gtp")
    if opts.bOutDens and res.rho is not None:
        with open(base + ".den", "w") as f:
            f.write(f"{snap.n}\n")
            f.write(_fmt_lines("%.10g", res.rho))
        written.append(base + ".den")
    if opts.bOutRay and res.moved is not None:
        write_ray(base + ".ray", res.moved, snap, opts)
        written.append(base + ".ray")
    if opts.bOutStats and res.stats is not None:
        write_stats(base + ".stat", res)
        written.append(base + ".stat")
    return written


def write_ray(path, moved, snap, opts):
    """kdOutVector (kd.c:1550-1608): displacement moved - initial, wrapped."""
    with open(path, "w") as f:
        f.write(f"{snap.n}\n")
        for d in range(3):
            h = np.float32(0.5 * opts.period[d])
            dx = (moved[:, d] - snap.pos[:, d]).astype(np.float32)
            dx = np.where(dx > h, dx - np.float32(2) * h, dx).astype(np.float32)
            dx = np.where(dx <= -h, dx + np.float32(2) * h, dx).astype(np.float32)
            f.write(_fmt_lines("%g", dx))


def stat_rows(res: Result) -> np.ndarray:
    """The .stat table (kdOutStats, kd.c:1819-1833) as float64 rows: the
    device's per-group columns, sqrt of the squared ones taken in double as
    the reference's printf arguments are, and the records' centre, vcm and
    most bound particle."""
    rows = []
    for g in range(1, res.n_group + 1):
        q = res.stats[g]
        r = res.groups[g]
        if q["nMembers"] <= 0:
            continue
        rows.append([g, q["nMembers"], q["fTotMass"], q["fGasMass"], q["fStarMass"],
                     math.sqrt(q["fVcirc2Max"]), math.sqrt(q["fVcirc2Half"]),
                     math.sqrt(q["fVcirc2Outer"]), q["fRVmax"], q["fRHalf"],
                     math.sqrt(q["fROuter2"]), q["fVdisp"], *r["rCenter"], *r["vcm"],
                     *r["rBound"]])
    return np.asarray(rows, np.float64).reshape(-1, 21)


def write_stats(path, res):
    with open(path, "w") as f:
        for r in stat_rows(res):
            f.write(f"{int(r[0])} {int(r[1])} " + " ".join("%g" % float(x) for x in r[2:]) + "\n")


def main(argv=None) -> int:
    """`python -m skid_gb300.pipeline <skid flags> < input` (reads stdin like skid)."""
    argv = sys.argv[1:] if argv is None else argv
    try:
        opts = Options.parse(argv)
    except Exception as e:
        print(f"USAGE: skid -tau <fLinkLength> [OPTIONAL ARGUMENTS] ({e})", file=sys.stderr)
        return 1
    print("SKID v1.4.1 (GB300)")
    data = sys.stdin.buffer.read()
    snap = tipsy.read_tipsy(data, standard=opts.bStandard)
    res = run(snap, opts, log=lambda s: print(s, flush=True))
    write_outputs(res, snap, opts)
    t = res.timings
    print("SKID GPU Time (device ms):")
    if not opts.bUnbindOnly:
        print(f"   Initial Density:    {t['density_ms']:.3f}")
        print(f"   Moving Particles:   {t['moving_ms']:.3f}")
        print(f"   Friends of Friends: {t['fof_ms']:.3f}")
        print(f"   Microstepping:      {t['micro_ms']:.3f}")
    if not opts.bNoUnbind:
        print(f"   Unbinding:          {t['unbind_ms']:.3f}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
