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

``--impl reference`` times the reference algorithm on the host cores: the
reference's own binary cannot be built on this host (its sources are not
here), so the oracle's C restatement of it runs, single-threaded like skid.
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
CPU_SAMPLE_N = 1 << 16
FALLBACK_HBM = 6800.0


def workload(n):
    from skid_gb300 import synth
    if n == N_DEFAULT:
        spec = synth.CONFIGS[1]
    else:
        spec = synth.HaloSpec(n, max(1, round(800 * n / N_DEFAULT)), 3.0, (4.0, 20.0), 0.02, 0.55,
                              synth.SEED_BASE + 1)
    return spec


def flags():
    from skid_gb300 import synth
    return list(synth.WORKLOAD_FLAGS[1])


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


def cpu_baseline(n_sample=CPU_SAMPLE_N, repeats=1):
    """The oracle's restatement of skid on a bounded sample, one host core."""
    from oracle import oracle
    from skid_gb300 import synth
    from skid_gb300.options import Options
    oracle.build()
    snap = synth.make_snapshot(workload(n_sample))
    opts = Options.parse(flags())
    best = None
    for _ in range(repeats):
        t = time.perf_counter()
        oracle.run(snap, opts)
        dt = time.perf_counter() - t
        best = dt if best is None else min(best, dt)
    return {"value": n_sample / best, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"oracle C restatement of skid, single-threaded, one run on a "
                      f"{n_sample}-particle box generated like the 2^21 workload "
                      f"({max(1, round(800 * n_sample / N_DEFAULT))} halos), same flags; "
                      f"{best:.1f} s"}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    from oracle import oracle
    from skid_gb300 import synth
    from skid_gb300.options import Options
    oracle.build()
    n = CPU_SAMPLE_N
    snap = synth.make_snapshot(workload(n))
    opts = Options.parse(flags())
    for _ in range(args.warmup if args.warmup < 1 else 1):
        oracle.run(snap, opts)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        oracle.run(snap, opts)
        times.append(time.perf_counter() - t)
    tot = sum(times)
    value = n * len(times) / tot
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"skid on a {n}-particle sample of the 2^21 workload "
                                   f"(NFW halos + background), periodic unit box",
                       "flags": " ".join(flags()), "n_particles": n},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"{n} particles per step, oracle C restatement of "
                                       f"skid (the reference binary is not buildable here), "
                                       f"single-threaded like skid"},
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
    tot_ms = sum(step_ms)
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([tot_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        tot_ms = float(tt.item())
    value = world * n * args.steps / (tot_ms / 1000.0)

    # roofline of the dominant kernel (move field): algorithmic bytes / event time
    f_ms = t_after["field_ms"] - t_before["field_ms"]
    f_bytes = t_after["field_bytes"] - t_before["field_bytes"]
    f_launch = t_after["gather_launches"] - t_before["gather_launches"]
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
    e2e_tot = sum(e2e_ms)
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([e2e_tot], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_tot = float(tt.item())
    h2d = n * (3 + 3 + 1 + 1 + 1) * 4
    d2h = n * 4 + (r.n_group + 1) * gpu.GROUP_DTYPE.itemsize

    if rank != 0:
        ctx.close()
        return 0
    cpu = None if args.no_cpu_baseline else cpu_baseline()
    tm = res.timings
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"skid config 1: N={n} periodic unit box, 800 NFW halos "
                               f"(3 dex, c 4-20, r200max 0.02, 55%) + uniform background",
                   "flags": " ".join(flags()), "n_particles": n, "l2": "flushed before each step",
                   "parallelism": f"replicas x{world}", "groups": res.n_group,
                   "groups_before_unbind": res.counts.get("nGroupFoF"),
                   "unbound": res.counts.get("nUnbound"), "iterations": res.counts.get("nIter"),
                   "stage_ms": {k: round(float(tm[k]), 3) for k in
                                ("density_ms", "moving_ms", "fof_ms", "micro_ms", "groups_ms",
                                 "unbind_ms", "toosmall_ms")}},
        "e2e": {"value": world * n * args.steps / (e2e_tot / 1000.0), "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_tot / args.steps},
        "roofline": {"bound": "hbm", "kernel": "field_kernel (move-field gather + move)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                     "launches": f_launch, "avg_launch_ms": f_ms / max(f_launch, 1),
                     "algorithmic_bytes_per_launch": f_bytes / max(f_launch, 1)},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT, help="particles (default 2^21)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
