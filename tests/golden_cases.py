"""Loading and checking the golden fixtures (reference skid outputs).

Small cases keep their input as input.bin.  Workload-scale cases keep their
outputs gzip-compressed and their input either compressed (input.bin.gz,
or input.std.gz for an XDR input read with -std) or not at all: then the
input is regenerated from the workload generator named in case.json, and
its TIPSY bytes must hash to the recorded SHA-256 before anything is
compared."""
import gzip
import hashlib
import json
import os

import numpy as np

from skid_gb300 import compare, synth, tipsy
from skid_gb300.options import Options

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names(max_n=None):
    """Case names, optionally only those of at most max_n particles."""
    out = []
    for d in sorted(os.listdir(GOLDEN)):
        p = os.path.join(GOLDEN, d, "case.json")
        if not os.path.isfile(p):
            continue
        if max_n is not None:
            with open(p) as f:
                if json.load(f)["n"] > max_n:
                    continue
        out.append(d)
    return out


def meta_of(name):
    with open(os.path.join(GOLDEN, name, "case.json")) as f:
        return json.load(f)


def input_bytes(name, meta=None):
    """The exact TIPSY bytes the reference read for this case."""
    meta = meta or meta_of(name)
    d = os.path.join(GOLDEN, meta.get("input_from", name))
    kind = meta.get("input", "bin")
    if kind == "regen":
        g = dict(meta["generator"])
        g["conc"] = tuple(g["conc"])
        spec = synth.HaloSpec(**g)
        snap = synth.make_snapshot(spec)
        gas, dark, star = tipsy.snapshot_records(snap)
        import tempfile
        with tempfile.NamedTemporaryFile(suffix=".bin") as t:
            tipsy.write_tipsy(t.name, snap.time, gas, dark, star)
            with open(t.name, "rb") as f:
                data = f.read()
    elif kind == "gz":
        std = "-std" in meta["flags"]
        with gzip.open(os.path.join(d, "input.std.gz" if std else "input.bin.gz"), "rb") as f:
            data = f.read()
    else:
        with open(os.path.join(d, "input.bin"), "rb") as f:
            data = f.read()
    want = meta.get("input_sha256")
    if want is not None:
        got = hashlib.sha256(data).hexdigest()
        assert got == want, (f"{name}: input differs from the one the reference ran on "
                             f"(sha256 {got} != {want}); this host's numpy regenerates "
                             "other floats")
    return data


def ref_path(name, ext, meta=None):
    meta = meta or meta_of(name)
    p = os.path.join(GOLDEN, name, "ref." + ext)
    if meta.get("compressed") and ext not in ("gtp", "stat"):
        p += ".gz"
    return p


def load(name):
    d = os.path.join(GOLDEN, name)
    meta = meta_of(name)
    snap = tipsy.read_tipsy(input_bytes(name, meta), standard="-std" in meta["flags"])
    ref = {"grp": tipsy.read_grp(ref_path(name, "grp", meta)),
           "gtp": tipsy.read_gtp(os.path.join(d, "ref.gtp"), standard="-std" in meta["flags"])}
    if "den" in meta["outputs"]:
        ref["den"] = tipsy.read_den(ref_path(name, "den", meta))
    if "stat" in meta["outputs"]:
        ref["stat"] = tipsy.read_stat(os.path.join(d, "ref.stat"))
    opts = Options.parse(meta["flags"])
    if opts.bUnbindOnly:
        opts.achGroup = os.path.join(d, opts.achGroup)
    counts = {}
    for line in meta["stdout"]:
        for key, tag in (("nExtraScat", "nExtraScat:"), ("nGroupFoF", "Groups before Unbind:"),
                         ("nUnbound", "Number of particles Unbound:"), ("nGroup", "Number of Groups:")):
            if line.startswith(tag):
                counts[key] = int(line.split(":")[1])
    counts["nIter"] = sum(1 for l in meta["stdout"] if l.startswith("Ittr")) - 1
    return snap, opts, ref, counts, meta


def unbind_inputs(opts):
    """Group ids and (n-1, 6) centres (rCenter, vcm; None without a .gtp) of
    an unbind-only case, read the way kdInGroup/kdReadCenter read them."""
    base = opts.achGroup[:-4] if opts.achGroup.endswith(".grp") else opts.achGroup
    grp = tipsy.read_grp(base + ".grp")
    centers = None
    if os.path.exists(base + ".gtp"):
        star = tipsy.read_gtp(base + ".gtp", standard=opts.bStandard)
        centers = np.concatenate([star["pos"], star["vel"]], axis=1).astype(np.float32)
    return grp, centers


def check_catalogue(grp, groups, ref, opts, min_agree=0.999, tol_pos=None, tol_mean=None):
    """Per-particle agreement, same groups above -m, and matched .gtp records.
    groups: dict-like with fMass, rCenter, vcm, fRadius indexed by group id.

    A density centre is the mean of the members' final moved positions.
    Converged particles oscillate about their density peak by up to a step,
    and summing the move field in another order (the reference sums in tree
    order, the GPU per lane) can shift the phase of that oscillation for a
    few members, which moves a small group's centre by a fraction of fStep.
    So every matched group's centre (and radius, the largest member distance
    from it) must be within tol_pos (default fStep / 4) and their mean
    deviation within tol_mean (default 2 % of fStep)."""
    if tol_pos is None:
        tol_pos = 0.25 * opts.fStep
    if tol_mean is None:
        tol_mean = 0.02 * opts.fStep
    m = compare.match_groups(ref["grp"], grp)
    assert m.agreement >= min_agree, f"agreement {m.agreement:.5f}"
    assert m.same_groups(), f"unmatched groups ref={m.unmatched_a} new={m.unmatched_b}"
    gtp = ref["gtp"]
    worst = {"mass": 0.0, "pos": 0.0, "vel": 0.0, "rad": 0.0}
    dpos, drad = [], []
    for a, b in m.pairs.items():
        r = gtp[a - 1]
        same = np.count_nonzero((ref["grp"] == a) & (grp == b)) == np.count_nonzero(ref["grp"] == a) \
            == np.count_nonzero(grp == b)
        if not same:
            continue   # membership differs: records legitimately differ
        worst["mass"] = max(worst["mass"], abs(float(groups["fMass"][b]) - r["mass"]) / r["mass"])
        dpos.append(float(np.max(np.abs(groups["rCenter"][b] - r["pos"]))))
        vscale = max(float(np.max(np.abs(r["vel"]))), 1e-3)
        worst["vel"] = max(worst["vel"], float(np.max(np.abs(groups["vcm"][b] - r["vel"]))) / vscale)
        drad.append(abs(float(groups["fRadius"][b]) - r["eps"]))
    if dpos:
        worst["pos"] = max(dpos)
        worst["rad"] = max(drad)
        worst["pos_mean"] = float(np.mean(dpos))
        worst["rad_mean"] = float(np.mean(drad))
    assert worst["mass"] < 1e-5, worst
    assert worst["vel"] < 1e-4, worst
    assert worst["pos"] < tol_pos and worst["rad"] < tol_pos, (worst, tol_pos)
    assert worst.get("pos_mean", 0.0) < tol_mean and worst.get("rad_mean", 0.0) < tol_mean, \
        (worst, tol_mean)
    return m, worst
