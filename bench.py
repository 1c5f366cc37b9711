#!/usr/bin/env python3
"""Benchmark: end-to-end SKID group finding, particles/s, on GB300.

One step = one complete skid run (density, moves with scatterer removal,
friends-of-friends, micro-steps, centres, unbinding, too-small) over the
N = 2^21 clustered workload with skid's flags
``-tau 0.004 -s 64 -m 16 -p 1 -O 0.3 -Lambda 0.7 -H 5.2845`` (seeded
synthetic NFW halos + background; skid ships no benchmark data).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

``value``: particles/s with the snapshot already in HBM (skid_restart keeps
it on the device), device time by CUDA events on the library's stream.
``e2e``: the same through the C ABI from pinned host buffers: each step
copies the snapshot in (skid_set_particles) and reads the group ids and
records back.  L2 (126 MB) is flushed before every timed step.  With N
ranks (torchrun), every rank runs an independent replica on its own GPU
(the path does not shard within one snapshot): value = N x particles / max
time over ranks.

The metric compares two GPU forms at identical accuracy: the default form
(moves driven by the fused density-field adjoint kernel, every unbinding
group in one autotuned launch) is ``value``; the plain form (a separate
gradient pass then a move kernel every step, and one potential and one
removal launch per group, the reference's serial loop) is timed the same way
and reported under ``config.plain`` with its per-particle catalogue agreement
with the default form.  A run with ``-nsp`` (every scatterer kept) is
reported under ``config.nsp``.

``--impl reference`` times reference skid itself on the host cores, built
from its own sources (staged untracked under baseline/_ref/src, compiled by
oracle/build_ref.sh for the host).  skid is single-threaded, so each step
runs the 2^21 workload as 16 independent periodic sub-volume cubes of 2^17
particles with the workload's density, halo population and flags, one
process per core; value = 2^21 / the step's wall time.  The same step, once,
is the default run's ``cpu_baseline``.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "particles/s end-to-end SKID @2^21: batched+adjoint vs plain GPU, same accuracy"
UNIT = "particles/s"
N_DEFAULT = 1 << 21
FALLBACK_HBM = 6800.0


CONFIG = 1   # 1: the 2^21 dark-matter workload; 4: the 2^24 mixed-species one


def workload(n):
    from skid_gb300 import synth
    if CONFIG == 4:
        return synth.CONFIGS[4]
    if n == N_DEFAULT:
        spec = synth.CONFIGS[1]
    else:
        spec = synth.HaloSpec(n, max(1, round(800 * n / N_DEFAULT)), 3.0, (4.0, 20.0), 0.02, 0.55,
                              synth.SEED_BASE + 1)
    return spec


def flags():
    from skid_gb300 import synth
    return list(synth.WORKLOAD_FLAGS[CONFIG])


PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "field_kernel_skid_config1_2e21.md")


def field_traffic():
    """Mean DRAM bytes (read + write) per field_kernel launch over one full
    run, from the committed ncu launch capture (or None)."""
    import re
    try:
        with open(PROFILE_TRAFFIC) as f:
            m = re.search(r"traffic_bytes_per_launch_mean:\s*([0-9.eE+]+)", f.read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


def field_issue():
    """Instruction-issue utilisation of one full-activity field_kernel launch
    (fraction of peak issue slots, ncu `issue active`), from the committed
    full-section capture, or None.  The kernel is issue-bound; this is its
    roofline in the resource that binds it."""
    import re
    try:
        with open(PROFILE_TRAFFIC) as f:
            m = re.search(r"\|\s*issue active\s*\|\s*([0-9.]+)\s*%", f.read())
        return float(m.group(1)) / 100.0 if m else None
    except OSError:
        return None


def roofline_e2e(counts, n, field_bytes, ms, peak, peak_kind):
    """The whole run against the HBM roofline: its algorithmic bytes (the
    compulsory traffic of each stage, per unit: tree build 40 B and density
    24 B per scatterer; every move step the field kernel's 24 B per active
    mover and 20 B per live scatterer copy, as the library counts them;
    friends-of-friends 24 B per mover; group reductions 48 B, unbinding 36 B
    and outputs 4 B per particle) over the run's time."""
    ns = counts.get("nScatter", n)
    nm = counts.get("nMove", n)
    parts = {"tree_and_density": 64.0 * ns, "move_steps": float(field_bytes),
             "fof": 24.0 * nm, "groups_unbinding_outputs": 88.0 * n}
    tot = sum(parts.values())
    achieved = tot / (ms / 1000.0) / 1e9 if ms > 0 else 0.0
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_kind": peak_kind, "algorithmic_bytes_per_step": tot,
            "components": {k: round(v) for k, v in parts.items()}}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


REF_PARTS = 16     # periodic sub-volume cubes that together make one 2^21 step


def reference_binary():
    """Reference skid built from its own sources for this host (staged under
    baseline/_ref/src), or None with the reason."""
    from oracle import oracle
    try:
        exe = oracle.build_reference()
    except Exception as e:          # a compiler error on this host
        return None, f"reference build failed: {e}"
    if exe is None or not os.path.exists(exe):
        return None, "reference sources not present on this host"
    return exe, None


def write_subvolumes(dirpath, parts=REF_PARTS):
    """The 2^21 workload as `parts` independent periodic cubes of 2^21/parts
    particles each (synth.config1_subvolume), written as native TIPSY files.
    Returns [(path, flags)]."""
    from skid_gb300 import synth
    out = []
    for i in range(parts):
        snap, L = synth.config1_subvolume(i, parts)
        path = os.path.join(dirpath, f"sub{i:02d}.bin")
        synth.write_snapshot(path, snap)
        out.append((path, synth.config1_subvolume_flags(L)))
    return out


def _run_reference_file(exe, path, fl, cwd):
    """One reference skid process on one input file (stdin), outputs written
    to cwd.  Returns (seconds, stdout counts)."""
    t = time.perf_counter()
    with open(path, "rb") as f:
        r = subprocess.run([exe, *fl, "-o", os.path.splitext(os.path.basename(path))[0]],
                           stdin=f, cwd=cwd, capture_output=True, text=True)
    dt = time.perf_counter() - t
    if r.returncode:
        raise RuntimeError(f"reference skid failed on {path}: {r.stderr[-400:]}")
    counts = {}
    for line in r.stdout.splitlines():
        for key, tag in (("groups_before_unbind", "Groups before Unbind:"),
                         ("unbound", "Number of particles Unbound:"),
                         ("groups", "Number of Groups:")):
            if line.startswith(tag):
                counts[key] = int(line.split(":")[1])
    return dt, counts


def _run_port_file(path, fl):
    """The oracle's C restatement on one input file (fallback when the
    reference binary cannot be built here)."""
    from oracle import oracle
    from skid_gb300 import tipsy
    from skid_gb300.options import Options
    snap = tipsy.read_tipsy(path)
    t = time.perf_counter()
    r = oracle.run(snap, Options.parse(fl))
    return time.perf_counter() - t, {"groups_before_unbind": r["nGroupFoF"],
                                     "unbound": r["nUnbound"], "groups": r["nGroup"]}


def reference_step(exe, inputs, workers, cwd):
    """All sub-volumes through reference skid (or the port when exe is None),
    `workers` processes at a time.  Returns (wall seconds, per-run seconds,
    summed counts)."""
    import concurrent.futures as cf
    t = time.perf_counter()
    if exe is not None:
        with cf.ThreadPoolExecutor(workers) as ex:
            res = list(ex.map(lambda a: _run_reference_file(exe, a[0], a[1], cwd), inputs))
    else:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(workers) as pool:
            res = pool.starmap(_run_port_file, inputs, chunksize=1)
    wall = time.perf_counter() - t
    tot = {}
    for _, c in res:
        for k, v in c.items():
            tot[k] = tot.get(k, 0) + v
    return wall, [r[0] for r in res], tot


def _subvolume_sample_text(kind, parts, workers, per_run, why=None):
    from skid_gb300 import synth
    n_sub = synth.CONFIGS[1].n // parts
    what = ("reference skid v1.4.1 built from its own sources on this host (gcc -O2 "
            "-ffp-contract=off)" if kind == "reference" else
            f"the oracle's C restatement of skid ({why})")
    return (f"{what}: the 2^21 workload as {parts} independent periodic cubes of {n_sub} "
            f"particles (side {parts}^(-1/3), the workload's particle density, halo population "
            f"and flags, -p set to the side), {workers} processes at a time, each "
            f"single-threaded; {statistics.mean(per_run):.1f} s per cube")


def cpu_baseline(steps=1):
    """Reference skid on the host cores over one 2^21 step of sub-volumes
    (about 15 s of wall time with 16 cores)."""
    import tempfile
    exe, why = reference_binary()
    cores = os.cpu_count() or 1
    workers = min(cores, REF_PARTS)
    with tempfile.TemporaryDirectory() as tmp:
        inputs = write_subvolumes(tmp)
        walls, per_run = [], []
        for _ in range(steps):
            w, pr, counts = reference_step(exe, inputs, workers, tmp)
            walls.append(w)
            per_run += pr
    kind = "reference" if exe else "port"
    n = N_DEFAULT
    return {"value": n * len(walls) / sum(walls), "unit": UNIT, "cores": workers, "kind": kind,
            "per_core_value": (n / REF_PARTS) / statistics.mean(per_run),
            "n_particles": n, "sample": _subvolume_sample_text(kind, REF_PARTS, workers,
                                                               per_run, why),
            "catalogue": counts}


def cli_process_wall(snap, repeats=3):
    """The skid command-line tool as a user runs it: one process per run,
    reading the TIPSY snapshot on stdin (the file read once beforehand, so it
    is in the page cache) and writing .grp and .gtp.  Returns particles per
    second of process wall time (best of `repeats`) and the stage split the
    tool prints."""
    import tempfile
    from skid_gb300 import build, synth
    exe = build.build_cli()
    with tempfile.TemporaryDirectory() as tmp:
        inp = os.path.join(tmp, "input.bin")
        synth.write_snapshot(inp, snap)
        with open(inp, "rb") as f:
            f.read()
        cmd = [exe, *flags(), "-o", "out"]
        walls, out = [], ""
        for _ in range(repeats):
            t = time.perf_counter()
            with open(inp, "rb") as f:
                r = subprocess.run(cmd, stdin=f, cwd=tmp, capture_output=True, text=True)
            walls.append(time.perf_counter() - t)
            if r.returncode:
                raise RuntimeError(f"skid CLI failed: {r.stderr[-400:]}")
            out = r.stdout
        # one more run for the wall-clock phases the tool reports on request
        # (with a CUDA start-up probe first, so start-up and reading separate)
        phases = {}
        with open(inp, "rb") as f:
            r = subprocess.run(cmd, stdin=f, cwd=tmp, capture_output=True, text=True,
                               env=dict(os.environ, SKID_WALL_TIMES="2"))
        for line in r.stderr.splitlines():
            parts = line.split()
            if len(parts) == 3 and parts[0] == "wall_ms":
                phases[parts[1]] = round(float(parts[2]), 3)
        files = sorted(f for f in os.listdir(tmp) if f.startswith("out."))
    device = {}
    for line in out.splitlines():
        for key in ("Initial Density", "Moving Particles", "Friends of Friends", "Microstepping",
                    "Unbinding"):
            if line.strip().startswith(key + ":"):
                device[key] = float(line.split(":")[1])
    best = min(walls)
    return {"value": snap.n / best, "unit": UNIT, "wall_s": best, "walls_s": walls,
            "n_particles": snap.n, "files": files, "device_stage_ms": device,
            "host_phases_ms": phases,
            "command": "skid_gb300/bin/skid " + " ".join(flags()) + " -o out < input.bin"}


def reduce_max(x: float, world: int, device="cpu") -> float:
    """Max of x over ranks (the slowest replica sets the job's time)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world: int, n: int, steps: int, total_ms: float) -> float:
    """Whole-job particles/s: every rank processes its own n-particle replica per step."""
    return world * n * steps / (total_ms / 1000.0)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    """Reference skid itself on the host cores: each step runs the 2^21
    workload as REF_PARTS periodic sub-volume cubes, one single-threaded
    process per core; value = 2^21 particles / wall time of the step.  Falls
    back to the oracle's C restatement (labelled "port") only where the
    reference cannot be built."""
    import tempfile
    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    exe, why = reference_binary()
    cores = os.cpu_count() or 1
    workers = min(cores, REF_PARTS)
    n = N_DEFAULT
    with tempfile.TemporaryDirectory() as tmp:
        inputs = write_subvolumes(tmp)
        for _ in range(min(args.warmup, 1)):     # page cache; the CPU needs no warm-up
            reference_step(exe, inputs, workers, tmp)
        walls, per_run = [], []
        for _ in range(args.steps):
            w, pr, counts = reference_step(exe, inputs, workers, tmp)
            walls.append(w)
            per_run += pr
    tot = sum(walls)
    value = n * len(walls) / tot
    kind = "reference" if exe else "port"
    sample = _subvolume_sample_text(kind, REF_PARTS, workers, per_run, why)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / len(walls),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"skid config 1 (N=2^21 clustered, 800 NFW halos + uniform "
                                   f"background) as {REF_PARTS} periodic sub-volume cubes of "
                                   f"{n // REF_PARTS} particles",
                       "flags": " ".join(flags()) + f" (-p = cube side)", "n_particles": n,
                       "sub_volumes": REF_PARTS, "processes": workers, "catalogue": counts},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": kind,
                             "per_core_value": (n / REF_PARTS) / statistics.mean(per_run),
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import torch
    from skid_gb300 import build, gpu, pipeline, synth
    from skid_gb300.options import Options

    world, rank, local = dist_setup()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    build.build_lib()
    n = args.n
    snap = synth.make_snapshot(workload(n))
    opts = Options.parse(flags())

    # pinned host copies: the e2e copies are from page-locked memory
    def pinned(a, dtype):
        t = torch.from_numpy(np.ascontiguousarray(a, dtype)).pin_memory()
        return t.numpy()
    from skid_gb300 import tipsy
    snap = tipsy.Snapshot(snap.time, snap.n_gas, snap.n_dark, snap.n_star,
                          pinned(snap.pos, np.float32), pinned(snap.vel, np.float32),
                          pinned(snap.mass, np.float32), pinned(snap.soft, np.float32),
                          pinned(snap.temp, np.float32))

    ctx = gpu.Context(period=1.0, nSmooth=opts.nSmooth, device=local)
    stream = torch.cuda.ExternalStream(ctx.stream_ptr(), device=torch.device("cuda", local))
    flush_buf = torch.empty(64 << 20, dtype=torch.float32, device="cuda")   # 256 MB > L2

    def flush_l2():
        flush_buf.zero_()
        torch.cuda.synchronize()

    # warm-up (also instantiates the captured outer-iteration graph)
    res = None
    for _ in range(args.warmup):
        res = pipeline.run(snap, opts, ctx=ctx)
    ctx.set_particles(snap)

    # ---- resident: inputs in HBM when the timed region starts ----
    t_before = ctx.timings()
    l0 = t_before["kernel_launches"]
    step_ms = []
    barrier()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush_l2()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res = pipeline.run(snap, opts, ctx=ctx, upload=False)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
    barrier()
    t_after = ctx.timings()
    launches = t_after["kernel_launches"] - l0
    tot_ms = reduce_max(sum(step_ms), world, "cuda")
    value = job_value(world, n, args.steps, tot_ms)

    # roofline of the dominant kernel (move field): algorithmic bytes / event
    # time, from the library's figures, which restart with every run: those
    # of the last timed run (the launch count above is cumulative)
    f_ms = t_after["field_ms"]
    f_bytes = t_after["field_bytes"]
    f_launch = t_after["gather_launches"]
    peak, peak_kind = measured_peak()
    achieved = (f_bytes / f_launch) / (f_ms / f_launch / 1000.0) / 1e9 if f_ms > 0 else 0.0

    # ---- e2e: host buffers, copies inside the timed region ----
    e2e_ms = []
    barrier()
    for _ in range(args.steps):
        flush_l2()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = pipeline.run(snap, opts, ctx=ctx)   # skid_set_particles from pinned memory ... D2H
        e1.record(stream)
        e1.synchronize()
        e2e_ms.append(e0.elapsed_time(e1))
    barrier()
    e2e_tot = reduce_max(sum(e2e_ms), world, "cuda")
    h2d = n * (3 + 3 + 1 + 1 + 1) * 4
    d2h = n * 4 + (r.n_group + 1) * gpu.GROUP_DTYPE.itemsize

    # ---- the plain GPU form, same workload, same timing ----
    def timed_runs(c, o, k):
        strm = torch.cuda.ExternalStream(c.stream_ptr(), device=torch.device("cuda", local))
        ms, out = [], None
        for _ in range(k):
            flush_l2()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(strm)
            out = pipeline.run(snap, o, ctx=c, upload=False)
            e1.record(strm)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms, out

    plain = nsp = None
    if not args.no_compare:
        from skid_gb300 import compare
        pctx = gpu.Context(period=1.0, nSmooth=opts.nSmooth, device=local)
        pctx.set_option("field_unfused", 1)
        pctx.set_option("unbind_per_group", 1)
        pipeline.run(snap, opts, ctx=pctx)            # warm-up, uploads the snapshot
        p_ms, pres = timed_runs(pctx, opts, args.steps)
        pl = pctx.timings()["kernel_launches"]
        pctx.close()
        m = compare.match_groups(res.grp, pres.grp)
        plain = {"form": "separate gradient pass then move kernel every step; one potential "
                         "and one removal launch per group",
                 "value": world * n * len(p_ms) / (sum(p_ms) / 1000.0),
                 "ms_per_step": sum(p_ms) / len(p_ms), "agreement": m.agreement,
                 "same_groups": bool(m.same_groups()), "groups": pres.n_group,
                 "unbind_ms": round(float(pres.timings["unbind_ms"]), 3),
                 "moving_ms": round(float(pres.timings["moving_ms"]), 3)}
        opts_nsp = Options.parse(flags() + ["-nsp"])
        pipeline.run(snap, opts_nsp, ctx=ctx, upload=False)   # warm-up (graphs for -nsp)
        n_ms, nres = timed_runs(ctx, opts_nsp, min(args.steps, 5))
        nsp = {"value": world * n * len(n_ms) / (sum(n_ms) / 1000.0),
               "ms_per_step": sum(n_ms) / len(n_ms), "steps": len(n_ms),
               "groups": nres.n_group, "iterations": nres.counts.get("nIter"),
               "stage_ms": {k: round(float(nres.timings[k]), 3) for k in
                            ("density_ms", "moving_ms", "unbind_ms")}}
    sched = {"unbind_warp_max": ctx.get_option("unbind_warp_max"),
             "unbind_block": ctx.get_option("unbind_block"),
             "pot_ms": round(ctx.get_option("unbind_pot_ms"), 3),
             "remove_ms": round(ctx.get_option("unbind_remove_ms"), 3),
             "candidates_ms": [round(ctx.get_option(f"unbind_tune_ms{k}"), 3)
                               for k in range(int(ctx.get_option("unbind_tune_candidates")))]}

    if rank != 0:
        ctx.close()
        return 0
    cpu = None if args.no_cpu_baseline else cpu_baseline()
    cli = None if args.no_cli else cli_process_wall(snap)
    extra = None
    if not args.no_extra and world == 1 and CONFIG == 1:
        extra = {"adjoint_2e20": adjoint_workload(3),
                 "mixed_2e24": mixed_workload(2, cpu=not args.no_cpu_baseline),
                 "batch_96": batch_workload(96, 12, 1, cpu=not args.no_cpu_baseline)}
    tm = res.timings
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": (f"skid config 1: N={n} periodic unit box, 800 NFW halos "
                                f"(3 dex, c 4-20, r200max 0.02, 55%) + uniform background"
                                if CONFIG == 1 else
                                f"skid config 4: N={n} (50% gas of mass 0.2, 50% dark), 6000 NFW "
                                f"halos (3.5 dex, c 4-20, 50%) + Zel'dovich-displaced k^-2 "
                                f"Gaussian random field background, z = 0.5, -gd"),
                   "flags": " ".join(flags()), "n_particles": n, "l2": "flushed before each step",
                   "parallelism": f"replicas x{world}", "groups": res.n_group,
                   "groups_before_unbind": res.counts.get("nGroupFoF"),
                   "unbound": res.counts.get("nUnbound"), "iterations": res.counts.get("nIter"),
                   "stage_ms": {k: round(float(tm[k]), 3) for k in
                                ("density_ms", "moving_ms", "fof_ms", "micro_ms", "groups_ms",
                                 "unbind_ms", "toosmall_ms")},
                   "step_ms": [round(x, 3) for x in step_ms],
                   "e2e_step_ms": [round(x, 3) for x in e2e_ms],
                   "form": "fused density-field adjoint + move kernel; every unbinding group "
                           "in one autotuned launch",
                   "unbind_schedule": sched, "plain": plain, "nsp": nsp},
        "e2e": {"value": job_value(world, n, args.steps, e2e_tot), "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_tot / args.steps},
        "roofline": {"bound": "hbm", "kernel": "field_kernel (move-field gather + move)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": field_traffic(),
                     "traffic_source": "static: mean DRAM read+write bytes per launch from the "
                                       "committed ncu capture "
                                       "(profiles/field_kernel_skid_config1_2e21.md)",
                     "launches": f_launch, "avg_launch_ms": f_ms / max(f_launch, 1),
                     "algorithmic_bytes_per_launch": f_bytes / max(f_launch, 1),
                     "issue": {"frac": field_issue(), "unit": "fraction of peak issue slots",
                               "source": "static: ncu issue active of one launch at full "
                                         "activity (profiles/field_kernel_skid_config1_2e21.md)"}},
        "roofline_e2e": roofline_e2e(res.counts, n, f_bytes, tot_ms / args.steps, peak, peak_kind),
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if cli:
        line["cli_process"] = cli
    if extra:
        line["configs"] = extra
    print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def synth_n(config):
    from skid_gb300 import synth
    return synth.CONFIGS[config].n


def run_adjoint(args):
    """Config 3 alone: prints adjoint_workload's line."""
    print(json.dumps(adjoint_workload(args.steps, args.check)), flush=True)
    return 0


def adjoint_workload(steps, check_fd=False):
    """Config 3: N = 2^20.  Times the density adjoint (dL/dx of sum w_i rho_i,
    both neighbour modes) and the potential-energy adjoint of the 200 largest
    groups, after the ordinary pipeline up to the group centres; with check_fd,
    compares 1024 random particles with FP64 central differences (h = 1e-6)."""
    import torch
    from skid_gb300 import build, gpu, synth
    from skid_gb300.options import Options
    build.build_lib()
    snap = synth.make_snapshot(synth.CONFIGS[3])
    opts = Options.parse(synth.WORKLOAD_FLAGS[3])
    rng = np.random.default_rng(synth.SEED_BASE + 30)
    w = rng.standard_normal(snap.n).astype(np.float32)
    ctx = gpu.Context(period=1.0, nSmooth=opts.nSmooth)
    strm = torch.cuda.ExternalStream(ctx.stream_ptr())

    def timed(fn, k):
        ms = []
        out = None
        for _ in range(k):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(strm)
            out = fn()
            e1.record(strm)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return min(ms), out

    ctx.set_particles(snap)
    ctx.scatter_active(False, False)
    ctx.density()
    dens_ms, _ = timed(lambda: (ctx.restart(), ctx.scatter_active(False, False), ctx.density()), 3)
    walk_ms, g_walk = timed(lambda: ctx.density_adjoint(w, gpu.ADJ_RECOMPUTE), max(2, steps))
    list_ms, g_list = timed(lambda: ctx.density_adjoint(w, gpu.ADJ_STORED), max(2, steps))
    ctx.init_move(opts.fDensMin, opts.fTempMax, opts.fMassMax, False, False)
    ctx.move_step(opts.fStep, True, False)
    na = 1
    while na:
        na, _ = ctx.move_iterate(opts.fStep, opts.fCvg, False)
    ng = ctx.fof(opts.fTau)
    ctx.group_centers()
    grp, _ = ctx.get_groups(ng)
    sizes = np.bincount(grp, minlength=ng + 1)[1:]
    sel = (np.argsort(-sizes, kind="stable")[:200] + 1).astype(np.int32)
    v = rng.standard_normal(len(sel)).astype(np.float32)
    pot_ms, (E, gpot) = timed(lambda: ctx.potential_adjoint(sel, v, G=opts.G), max(2, steps))
    ctx.close()
    check = None
    if check_fd:
        from oracle import oracle
        pick = rng.choice(snap.n, 1024, replace=False)
        an, fd, ab = oracle.density_adjoint_check(snap.pos, snap.mass, w, opts.nSmooth, 1.0, pick)
        _, fdr, _ = oracle.density_adjoint_check(snap.pos, snap.mass, w, opts.nSmooth, 1.0, pick,
                                                 richardson=True)
        def rel(a, ref):
            return float(np.max(np.linalg.norm(np.asarray(a, np.float64) - ref, axis=1) / ab))
        check = {"particles": len(pick), "fd_step": 1e-6,
                 "density_vs_fp64": rel(g_walk[pick], an), "density_vs_fd": rel(g_walk[pick], fd),
                 "density_vs_fd_richardson": rel(g_walk[pick], fdr),
                 "stored_vs_fp64": rel(g_list[pick], an), "fp64_analytic_vs_fd": rel(an, fd),
                 "fp64_analytic_vs_fd_richardson": rel(an, fdr)}
    pairs = float(np.sum(np.minimum(sizes[sel - 1], 10 ** 9).astype(np.float64) ** 2))
    line = {"metric": "adjoint throughput, N=2^20", "unit": "particles/s",
            "value": snap.n / (walk_ms / 1000.0), "n_gpus": 1, "data": "synthetic",
            "config": {"workload": "config 3: N=2^20 periodic unit box, 400 NFW halos + background",
                       "density_ms": dens_ms, "density_adjoint_recompute_ms": walk_ms,
                       "density_adjoint_stored_ms": list_ms,
                       "potential_adjoint_ms": pot_ms, "potential_groups": len(sel),
                       "potential_pairs": pairs, "check": check}}
    return line


def mixed_cpu_baseline():
    """Reference skid on one host core over the 32768-particle slice of the
    mixed-species generator (the 2^24 run itself would take it the better part
    of an hour)."""
    import tempfile
    from skid_gb300 import synth
    exe, why = reference_binary()
    snap = synth.make_snapshot(synth.CONFIG4_SLICE)
    fl = synth.config4_slice_flags()
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "slice.bin")
        synth.write_snapshot(path, snap)
        _, per_run, counts = reference_step(exe, [(path, fl)], 1, tmp)
    kind = "reference" if exe else "port"
    what = ("reference skid v1.4.1 built from its own sources on this host (gcc -O2 "
            "-ffp-contract=off)" if kind == "reference" else
            f"the oracle's C restatement of skid ({why})")
    return {"value": snap.n / per_run[0], "unit": UNIT, "cores": 1, "kind": kind,
            "per_core_value": snap.n / per_run[0], "n_particles": snap.n,
            "sample": f"{what}: the {snap.n}-particle slice of the mixed-species generator "
                      f"(12 halos, 50 % gas, Gaussian-random-field background; "
                      f"{' '.join(fl)}), one single-threaded process, {per_run[0]:.2f} s",
            "catalogue": counts}


def mixed_workload(steps=2, cpu=False):
    """Config 4 at full size: 2^24 gas + dark particles (-gd, z = 0.5,
    Zel'dovich k^-2 background), resident and end-to-end particles/s over
    `steps` runs after one warm-up (whose first unbinding tunes the schedule).
    Its parity case is the 32768-particle slice of the same generator run by
    reference skid (tests/golden/config4_slice_32k)."""
    import torch
    from skid_gb300 import gpu, pipeline, synth, tipsy
    from skid_gb300.options import Options
    t = time.perf_counter()
    snap = synth.make_snapshot(synth.CONFIGS[4])
    gen_s = time.perf_counter() - t

    def pinned(a):
        return torch.from_numpy(np.ascontiguousarray(a, np.float32)).pin_memory().numpy()
    snap = tipsy.Snapshot(snap.time, snap.n_gas, snap.n_dark, snap.n_star, pinned(snap.pos),
                          pinned(snap.vel), pinned(snap.mass), pinned(snap.soft),
                          pinned(snap.temp))
    opts = Options.parse(synth.WORKLOAD_FLAGS[4])
    ctx = gpu.Context(period=1.0, nSmooth=opts.nSmooth)
    strm = torch.cuda.ExternalStream(ctx.stream_ptr())
    res = pipeline.run(snap, opts, ctx=ctx)

    def timed(upload):
        ms = []
        out = None
        for _ in range(steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(strm)
            out = pipeline.run(snap, opts, ctx=ctx, upload=upload)
            e1.record(strm)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return sum(ms) / len(ms), out
    r_ms, res = timed(False)
    e_ms, _ = timed(True)
    ctx.close()
    tm = res.timings
    line = {"workload": "config 4: N=2^24 (50% gas of mass 0.2, 50% dark), 6000 NFW halos "
                        "(3.5 dex, c 4-20, 50%) + Zel'dovich-displaced k^-2 Gaussian random "
                        "field background, z = 0.5, -gd",
            "flags": " ".join(synth.WORKLOAD_FLAGS[4]), "n_particles": snap.n,
            "value": snap.n / (r_ms / 1000.0), "ms_per_step": r_ms,
            "e2e_value": snap.n / (e_ms / 1000.0), "e2e_ms_per_step": e_ms, "steps": steps,
            "groups": res.n_group, "groups_before_unbind": res.counts.get("nGroupFoF"),
            "unbound": res.counts.get("nUnbound"), "iterations": res.counts.get("nIter"),
            "stage_ms": {k: round(float(tm[k]), 3) for k in
                         ("density_ms", "moving_ms", "fof_ms", "micro_ms", "unbind_ms")},
            "generation_s": round(gen_s, 1)}
    if cpu:
        line["cpu_baseline"] = mixed_cpu_baseline()
    return line


def batch_cpu_baseline(vols, rest):
    """Reference skid on the host cores over the 16 volumes of the batch
    nearest its median size (each single-threaded, 16 processes at a time:
    the batch's largest volumes would take a minute each on one core)."""
    import tempfile
    from skid_gb300 import synth
    exe, why = reference_binary()
    cores = os.cpu_count() or 1
    ln = np.log2([v[0].n for v in vols])
    pick = sorted(np.argsort(np.abs(ln - np.median(ln)), kind="stable")[:16])
    workers = min(cores, len(pick))
    with tempfile.TemporaryDirectory() as tmp:
        inputs = []
        for i in pick:
            snap, k, tau = vols[i]
            path = os.path.join(tmp, f"vol{i:02d}.bin")
            synth.write_snapshot(path, snap)
            inputs.append((path, ["-tau", repr(float(np.float32(tau))), "-s", str(k)] + rest))
        wall, per_run, counts = reference_step(exe, inputs, workers, tmp)
    ns = [vols[i][0].n for i in pick]
    kind = "reference" if exe else "port"
    what = ("reference skid v1.4.1 built from its own sources on this host (gcc -O2 "
            "-ffp-contract=off)" if kind == "reference" else
            f"the oracle's C restatement of skid ({why})")
    return {"value": sum(ns) / wall, "unit": UNIT, "cores": workers, "kind": kind,
            "per_core_value": sum(ns) / sum(per_run), "n_particles": int(sum(ns)),
            "sample": f"{what}: the {len(pick)} volumes of the batch nearest its median size "
                      f"(N {min(ns)}-{max(ns)}, each with its own nSmooth and tau), {workers} "
                      f"processes at a time, each single-threaded; {wall:.1f} s wall",
            "catalogue": counts}


def batch_workload(n_vol=96, workers=12, steps=1, cpu=False):
    """Config 2: independent periodic subvolumes of uneven sizes (N log-uniform
    in [2^14, 2^20], halos proportional to N, nSmooth from {32, 64, 128},
    tau = 0.5 N^(-1/3)) through skid_batch_run, host buffers in and out
    (end to end).  Compares nWorkers concurrent pipelines with one."""
    from skid_gb300 import build, gpu, synth
    from skid_gb300.options import Options
    build.build_lib()
    specs = synth.subvolume_specs(n_vol)
    t0 = time.perf_counter()
    vols = [(synth.make_snapshot(spec), k, tau) for spec, k, tau in specs]
    gen_s = time.perf_counter() - t0
    ntot = sum(v[0].n for v in vols)
    rest = ["-m", "16", "-p", "1", "-O", "0.3", "-Lambda", "0.7", "-H", f"{synth.hubble_for(0.3):.6g}"]
    base = Options.parse(["-tau", "0.01"] + rest)
    gpu.batch_run(vols[:4], base, n_workers=min(4, workers))     # warm-up
    out = {}
    for w in (workers, 1):
        best = None
        for _ in range(max(1, steps)):
            t = time.perf_counter()
            res = gpu.batch_run(vols, base, n_workers=w)
            dt = time.perf_counter() - t
            best = dt if best is None else min(best, dt)
        out[w] = (best, res)
    wbest, res = out[workers]
    sbest, sres = out[1]
    same = all(np.array_equal(a["grp"], b["grp"]) for a, b in zip(res, sres))
    line = {"metric": "particles/s end-to-end SKID, batched subvolumes", "value": ntot / wbest,
            "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": 1,
            "ms_per_step": 1000 * wbest, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{len(vols)} periodic subvolumes, N log-uniform in [2^14, 2^20] "
                                   f"({ntot} particles), halos proportional to N, nSmooth in "
                                   f"{{32, 64, 128}}, tau = 0.5 N^(-1/3)",
                       "workers": workers, "sequential_value": ntot / sbest,
                       "sequential_ms": 1000 * sbest, "identical_to_sequential": bool(same),
                       "groups": int(sum(r["nGroup"] for r in res)),
                       "device_ms_sum": float(sum(r["device_ms"] for r in res)),
                       "generation_s": gen_s}}
    if cpu:
        line["cpu_baseline"] = batch_cpu_baseline(vols, rest)
    return line


def run_batch(args):
    """Config 2 alone: prints batch_workload's line."""
    print(json.dumps(batch_workload(args.n_vol, args.workers, args.steps)), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT, help="particles (default 2^21)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cli", action="store_true",
                    help="skip the skid command-line process wall-time runs")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the adjoint (2^20), mixed-species (2^24) and batched-subvolume "
                         "workload runs")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the plain-form and -nsp comparison runs")
    ap.add_argument("--workload", default="single", choices=["single", "batch", "mixed", "adjoint"],
                    help="batch: the uneven-subvolume workload through skid_batch_run; mixed: "
                         "2^24 gas + dark with a Zel'dovich background (-gd, z = 0.5); adjoint: "
                         "density and potential adjoints at 2^20")
    ap.add_argument("--n-vol", type=int, default=96)
    ap.add_argument("--check", action="store_true", help="adjoint: FP64 finite-difference check")
    ap.add_argument("--workers", type=int, default=12)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "mixed":
        global CONFIG
        CONFIG = 4
        args.n = synth_n(4)
        args.no_compare = True          # per-group unbinding of ~10^5 groups: minutes
        args.no_cpu_baseline = True     # the CPU port would take hours at 2^24
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
