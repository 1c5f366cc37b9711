"""Loading and checking the golden fixtures (reference skid outputs)."""
import json
import os

import numpy as np

from skid_gb300 import compare, tipsy
from skid_gb300.options import Options

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(d for d in os.listdir(GOLDEN) if os.path.isfile(os.path.join(GOLDEN, d, "case.json")))


def load(name):
    d = os.path.join(GOLDEN, name)
    with open(os.path.join(d, "case.json")) as f:
        meta = json.load(f)
    src = os.path.join(GOLDEN, meta["input_from"]) if "input_from" in meta else d
    snap = tipsy.read_tipsy(os.path.join(src, "input.bin"))
    ref = {"grp": tipsy.read_grp(os.path.join(d, "ref.grp")),
           "gtp": tipsy.read_gtp(os.path.join(d, "ref.gtp"))}
    if "den" in meta["outputs"]:
        ref["den"] = tipsy.read_den(os.path.join(d, "ref.den"))
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


def check_catalogue(grp, groups, ref, opts, min_agree=0.999, tol_pos=None):
    """Per-particle agreement, same groups above -m, and matched .gtp records.
    groups: dict-like with fMass, rCenter, vcm, fRadius indexed by group id.

    A density centre is the mean of the members' final moved positions, and
    each of those is only defined to within the last step's size: summing
    the move field in another order (the reference sums in tree order, the
    GPU per lane) changes where a particle stops by a fraction of fStep.  The
    default centre tolerance is therefore 2 % of fStep."""
    if tol_pos is None:
        tol_pos = 0.02 * opts.fStep
    m = compare.match_groups(ref["grp"], grp)
    assert m.agreement >= min_agree, f"agreement {m.agreement:.5f}"
    assert m.same_groups(), f"unmatched groups ref={m.unmatched_a} new={m.unmatched_b}"
    gtp = ref["gtp"]
    worst = {"mass": 0.0, "pos": 0.0, "vel": 0.0, "rad": 0.0}
    for a, b in m.pairs.items():
        r = gtp[a - 1]
        same = np.count_nonzero((ref["grp"] == a) & (grp == b)) == np.count_nonzero(ref["grp"] == a) \
            == np.count_nonzero(grp == b)
        if not same:
            continue   # membership differs: records legitimately differ
        worst["mass"] = max(worst["mass"], abs(float(groups["fMass"][b]) - r["mass"]) / r["mass"])
        worst["pos"] = max(worst["pos"], float(np.max(np.abs(groups["rCenter"][b] - r["pos"]))))
        vscale = max(float(np.max(np.abs(r["vel"]))), 1e-3)
        worst["vel"] = max(worst["vel"], float(np.max(np.abs(groups["vcm"][b] - r["vel"]))) / vscale)
        worst["rad"] = max(worst["rad"], abs(float(groups["fRadius"][b]) - r["eps"]))
    assert worst["mass"] < 1e-5, worst
    assert worst["pos"] < tol_pos, worst
    assert worst["vel"] < 1e-4, worst
    assert worst["rad"] < tol_pos, worst
    return m, worst
