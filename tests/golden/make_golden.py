"""Generate the golden fixtures: seeded inputs run through the reference skid.

    python tests/golden/make_golden.py [path/to/reference/skid]

The reference binary is oracle/_ref/skid (built from the reference sources by
oracle/build_ref.sh); cases with -nsp, which v1.4.1 lacks, run the patched
oracle/_ref/skid_nsp (every scatterer kept) without the flag.  Each case stores its input snapshot (native TIPSY),
the flags, the reference's stdout lines and its output files
(.grp/.gtp/.den/.stat/.ray as the flags ask).  The unbind-only cases
(-unbind) reuse another case's input snapshot ("input_from") and take that
case's reference .grp (and .gtp, when "with_gtp") as their group input,
stored beside them as in.grp / in.gtp.  The reference writes the native
TIPSY header's four pad bytes uninitialised, so a regenerated ref.gtp can
differ from the stored one in bytes 28-31 only.  The fixtures are what the GPU
tests compare against on machines where the reference is not present.

The workload-scale cases (LARGE_CASES) run the benchmark configurations
themselves: the 32768-particle demo-size configuration, the reference's own
fixture dark.std with the flags of its demo script (read through -std, as
the reference's XDR reader takes it), and the 2^21 clustered configuration
(also at 2^18).  Their outputs are stored gzip-compressed.  An input is either
stored gzip-compressed beside them ("input.bin.gz" / "input.std.gz") or, when
too large to keep, regenerated from the workload generator; case.json then
records the SHA-256 of the TIPSY bytes, and a host whose numpy regenerates
other floats fails that check instead of comparing different inputs.

    python tests/golden/make_golden.py [skid] [--only name,name]
"""
import gzip
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from skid_gb300 import synth, tipsy  # noqa: E402

H1 = f"{synth.hubble_for(1.0):.6g}"
H3 = f"{synth.hubble_for(0.3):.6g}"

# name: (n, n_halo, dex, r200max, halo_frac, seed, gas_frac, n_star, flags)
CASES = {
    "dark4k_periodic": (4096, 8, 1.5, 0.08, 0.6, 101, 0.0, 0,
                        ["-tau", "0.02", "-s", "32", "-m", "8", "-p", "1", "-H", H1,
                         "-den", "-stats", "-ray"]),
    "dark8k_lcdm": (8192, 16, 2.0, 0.06, 0.55, 102, 0.0, 0,
                    ["-tau", "0.012", "-s", "64", "-m", "16", "-p", "1", "-O", "0.3",
                     "-Lambda", "0.7", "-H", H3, "-z", "0.5", "-den", "-stats"]),
    "dark4k_open_dmin": (4096, 8, 1.5, 0.08, 0.6, 103, 0.0, 0,
                         ["-tau", "0.02", "-s", "32", "-m", "8", "-d", "3", "-H", H1, "-den",
                          "-stats"]),
    "gasdark6k_gd": (6000, 10, 1.5, 0.08, 0.6, 104, 0.5, 0,
                     ["-tau", "0.02", "-s", "32", "-m", "8", "-p", "1", "-gd", "-H", H1,
                      "-den", "-stats"]),
    "mixed6k": (6000, 10, 1.5, 0.08, 0.6, 105, 0.4, 1200,
                ["-tau", "0.02", "-s", "32", "-m", "8", "-p", "1", "-t", "2e4", "-H", H1,
                 "-stats"]),
    "dark4k_plummer_eps": (4096, 8, 1.5, 0.08, 0.6, 106, 0.0, 0,
                           ["-tau", "0.02", "-s", "32", "-m", "8", "-p", "1", "-plummer",
                            "-e", "0.002", "-maxgroup", "300", "-H", H1, "-stats"]),
    "dark4k_nu": (4096, 8, 1.5, 0.08, 0.6, 107, 0.0, 0,
                  ["-tau", "0.02", "-s", "32", "-m", "8", "-p", "1", "-nu", "-H", H1]),
    "dark6k_nsp": (6144, 12, 1.5, 0.07, 0.6, 108, 0.0, 0,
                   ["-tau", "0.016", "-s", "64", "-m", "8", "-p", "1", "-nsp", "-O", "0.3",
                    "-Lambda", "0.7", "-H", H3, "-den", "-stats"]),
    # flag branches of CutCriterion / ScatterCriterion and the driver
    # (kd.c:555-627, main.c:203-315)
    "mixed6k_go": (6000, 10, 1.5, 0.08, 0.6, 109, 0.4, 1200,
                   ["-tau", "0.02", "-s", "32", "-m", "8", "-p", "1", "-go", "-t", "2e4",
                    "-H", H1, "-stats"]),
    "gasdark6k_fic": (6000, 10, 1.5, 0.08, 0.6, 110, 0.5, 0,
                      ["-tau", "0.02", "-s", "32", "-m", "8", "-p", "1", "-fic", "-H", H1,
                       "-den", "-stats"]),
    "mixed6k_gd_M": (6000, 10, 1.5, 0.08, 0.6, 111, 0.4, 1200,
                     ["-tau", "0.02", "-s", "32", "-m", "8", "-p", "1", "-gd", "-M", "1e-4",
                      "-H", H1, "-stats"]),
    "dark4k_cvg_scoop": (4096, 8, 1.5, 0.08, 0.6, 112, 0.0, 0,
                         ["-tau", "0.02", "-s", "32", "-m", "8", "-p", "1", "-cvg", "0.006",
                          "-scoop", "0.05", "-H", H1, "-stats"]),
    "dark4k_center": (4096, 8, 1.5, 0.08, 0.6, 113, 0.0, 0,
                      ["-tau", "0.02", "-s", "32", "-m", "8", "-p", "1", "-c", "0.1",
                       "-cx", "0.3", "-cz", "-0.2", "-H", H1, "-den", "-stats"]),
}

# Cases whose box is centred off the origin: the generator's [-0.5, 0.5)
# positions are shifted by the centre the flags name.
CENTRE_SHIFT = {"dark4k_center": (0.3, 0.1, -0.2)}


# name: (source case, with_gtp, flags); "-unbind" names the stored in.grp
UNBIND_CASES = {
    "dark4k_unbind_gtp": ("dark4k_nu", True,
                          ["-tau", "0.02", "-m", "8", "-p", "1", "-H", H1, "-unbind", "in",
                           "-stats"]),
    "mixed6k_unbind_com": ("mixed6k", False,
                           ["-tau", "0.02", "-m", "8", "-p", "1", "-H", H1, "-unbind", "in.grp"]),
}


def make_input(name):
    n, nh, dex, r200, frac, seed, gas_frac, n_star, _ = CASES[name]
    spec = synth.HaloSpec(n, nh, dex, (5.0, 15.0), r200, frac, seed, gas_frac=gas_frac)
    snap = synth.make_snapshot(spec)
    if n_star:
        snap = tipsy.Snapshot(snap.time, snap.n_gas, snap.n_dark - n_star, n_star, snap.pos,
                              snap.vel, snap.mass, snap.soft, snap.temp)
    if name in CENTRE_SHIFT:
        c = np.asarray(CENTRE_SHIFT[name], np.float64)
        p = (snap.pos.astype(np.float64) + c).astype(np.float32)
        hi = (c + 0.5).astype(np.float32)
        p = np.where(p >= hi, (p.astype(np.float64) - 1.0).astype(np.float32), p)
        snap = tipsy.Snapshot(snap.time, snap.n_gas, snap.n_dark, snap.n_star, p, snap.vel,
                              snap.mass, snap.soft, snap.temp)
    return snap


# Workload-scale cases.  "spec": a generator spec (synth.HaloSpec) or
# "dark.std" (the reference's own demo fixture, XDR); "store": "gz" keeps the
# input compressed beside the outputs, "regen" keeps only its SHA-256.
C4_SLICE = synth.CONFIG4_SLICE
LARGE_CASES = {
    "config0_32k": dict(spec=synth.CONFIGS[0], store="gz",
                        flags=synth.WORKLOAD_FLAGS[0] + ["-den", "-stats"]),
    "demo_dark_std": dict(spec="dark.std", store="gz",
                          flags=["-std", "-tau", "9e-4", "-s", "64", "-d", "170", "-m", "8",
                                 "-H", "2.8944", "-p", "1", "-ray", "-den", "-stats"]),
    "config4_slice_32k": dict(spec=C4_SLICE, store="gz",
                              flags=synth.config4_slice_flags() + ["-stats"]),
    "config1_2e18": dict(spec=synth.config1_spec(1 << 18), store="regen",
                         flags=synth.WORKLOAD_FLAGS[1]),
    "config1_2e21": dict(spec=synth.CONFIGS[1], store="regen", flags=synth.WORKLOAD_FLAGS[1]),
}


def large_input_bytes(name, ref_dir=None):
    """The TIPSY bytes of a workload-scale case as the reference reads them."""
    spec = LARGE_CASES[name]["spec"]
    if spec == "dark.std":
        with open(os.path.join(ref_dir, "dark.std"), "rb") as f:
            return f.read()
    snap = synth.make_snapshot(spec)
    gas, dark, star = tipsy.snapshot_records(snap)
    with tempfile.NamedTemporaryFile(suffix=".bin") as t:
        tipsy.write_tipsy(t.name, snap.time, gas, dark, star)
        with open(t.name, "rb") as f:
            return f.read()


def _stdout_lines(text):
    return [l for l in text.splitlines() if not l.startswith(("SKID", "   ")) and "Time" not in l]


def make_large(name, ref, ref_dir):
    case = LARGE_CASES[name]
    flags = case["flags"]
    d = os.path.join(HERE, name)
    os.makedirs(d, exist_ok=True)
    data = large_input_bytes(name, ref_dir)
    std = "-std" in flags
    if case["store"] == "gz":
        with gzip.open(os.path.join(d, "input.std.gz" if std else "input.bin.gz"), "wb", 9) as f:
            f.write(data)
    snap = tipsy.read_tipsy(data, standard=std)
    with tempfile.TemporaryDirectory() as tmp:
        r = subprocess.run([ref, *flags, "-o", "ref"], input=data, cwd=tmp,
                           capture_output=True, check=True)
        outs = []
        for ext in ("grp", "gtp", "den", "stat", "ray"):
            p = os.path.join(tmp, "ref." + ext)
            if not os.path.exists(p):
                continue
            outs.append(ext)
            if ext in ("gtp", "stat"):
                shutil.copy(p, os.path.join(d, "ref." + ext))
            else:
                with open(p, "rb") as fi, gzip.open(os.path.join(d, f"ref.{ext}.gz"), "wb", 9) as fo:
                    shutil.copyfileobj(fi, fo)
    lines = _stdout_lines(r.stdout.decode())
    meta = {"flags": flags, "n": snap.n, "n_gas": snap.n_gas, "n_dark": snap.n_dark,
            "n_star": snap.n_star, "outputs": outs, "compressed": True, "stdout": lines,
            "input": case["store"], "input_sha256": hashlib.sha256(data).hexdigest()}
    if case["store"] == "regen":
        meta["generator"] = dict(vars(case["spec"]), conc=list(case["spec"].conc))
    with open(os.path.join(d, "case.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, snap.n, [l for l in lines if not l.startswith(("Ittr", "Micro"))], flush=True)


def main():
    args = sys.argv[1:]
    only = None
    if "--only" in args:
        k = args.index("--only")
        only = set(args[k + 1].split(","))
        del args[k:k + 2]
    ref = args[0] if args else os.path.join(ROOT, "oracle", "_ref", "skid")
    ref_dir = os.environ.get("SKID_REF_DIR", os.path.join(ROOT, "baseline", "_ref", "src"))
    if not os.path.exists(ref):
        raise SystemExit(f"reference binary not found: {ref} (run oracle/build_ref.sh)")
    for name in LARGE_CASES:
        if only is None or name in only:
            make_large(name, ref, ref_dir)
    for name, case in CASES.items():
        if only is not None and name not in only:
            continue
        flags = case[-1]
        snap = make_input(name)
        d = os.path.join(HERE, name)
        os.makedirs(d, exist_ok=True)
        inp = os.path.join(d, "input.bin")
        synth.write_snapshot(inp, snap)
        exe, rflags = ref, flags
        if "-nsp" in flags:
            exe = os.path.join(os.path.dirname(ref), "skid_nsp")
            rflags = [f for f in flags if f != "-nsp"]
        with tempfile.TemporaryDirectory() as tmp:
            with open(inp, "rb") as f:
                r = subprocess.run([exe, *rflags, "-o", "ref"], stdin=f, cwd=tmp,
                                   capture_output=True, text=True, check=True)
            outs = []
            for ext in ("grp", "gtp", "den", "stat", "ray"):
                p = os.path.join(tmp, "ref." + ext)
                if os.path.exists(p):
                    shutil.copy(p, os.path.join(d, "ref." + ext))
                    outs.append(ext)
        lines = [l for l in r.stdout.splitlines()
                 if not l.startswith(("SKID", "   ")) and "Time" not in l]
        meta = {"flags": flags, "n": snap.n, "n_gas": snap.n_gas, "n_dark": snap.n_dark,
                "n_star": snap.n_star, "outputs": outs, "stdout": lines}
        with open(os.path.join(d, "case.json"), "w") as f:
            json.dump(meta, f, indent=1)
        print(name, snap.n, [l for l in lines if not l.startswith(("Ittr", "Micro"))])
    for name, (src, with_gtp, flags) in UNBIND_CASES.items():
        if only is not None and name not in only:
            continue
        d = os.path.join(HERE, name)
        sd = os.path.join(HERE, src)
        os.makedirs(d, exist_ok=True)
        shutil.copy(os.path.join(sd, "ref.grp"), os.path.join(d, "in.grp"))
        if with_gtp:
            shutil.copy(os.path.join(sd, "ref.gtp"), os.path.join(d, "in.gtp"))
        elif os.path.exists(os.path.join(d, "in.gtp")):
            os.remove(os.path.join(d, "in.gtp"))
        with open(os.path.join(sd, "case.json")) as f:
            smeta = json.load(f)
        with tempfile.TemporaryDirectory() as tmp:
            for ext in ("grp", "gtp"):
                if os.path.exists(os.path.join(d, "in." + ext)):
                    shutil.copy(os.path.join(d, "in." + ext), os.path.join(tmp, "in." + ext))
            with open(os.path.join(sd, "input.bin"), "rb") as f:
                r = subprocess.run([ref, *flags, "-o", "ref"], stdin=f, cwd=tmp,
                                   capture_output=True, text=True, check=True)
            outs = []
            for ext in ("grp", "gtp", "stat"):
                p = os.path.join(tmp, "ref." + ext)
                if os.path.exists(p):
                    shutil.copy(p, os.path.join(d, "ref." + ext))
                    outs.append(ext)
        lines = [l for l in r.stdout.splitlines()
                 if not l.startswith(("SKID", "   ")) and "Time" not in l]
        meta = {"flags": flags, "n": smeta["n"], "n_gas": smeta["n_gas"],
                "n_dark": smeta["n_dark"], "n_star": smeta["n_star"], "outputs": outs,
                "stdout": lines, "input_from": src, "warnings": r.stderr.splitlines()}
        with open(os.path.join(d, "case.json"), "w") as f:
            json.dump(meta, f, indent=1)
        print(name, smeta["n"], lines)


if __name__ == "__main__":
    main()
