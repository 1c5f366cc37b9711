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
"""
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

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
}


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
    return snap


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "oracle", "_ref", "skid")
    if not os.path.exists(ref):
        raise SystemExit(f"reference binary not found: {ref} (run oracle/build_ref.sh)")
    for name, case in CASES.items():
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
