"""The `skid` command-line tool (C, over the C ABI): same flags, stdin input,
progress lines and output files as the reference's driver.

CPU tests cover the host side only (argument errors, malformed TIPSY input,
which fail before any device call).  GPU tests run it on the golden cases
and compare its files with the reference's and with the Python pipeline's.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

from tests import golden_cases as gc


@pytest.fixture(scope="module")
def cli():
    from skid_gb300 import build
    build.build_lib()
    path = build.build_cli()
    assert path and os.path.exists(path)
    return path


def _run(cli, args, stdin_bytes, cwd):
    return subprocess.run([cli, *args], input=stdin_bytes, cwd=cwd, capture_output=True,
                          timeout=600)


def test_cli_usage_errors(cli, tmp_path):
    r = _run(cli, [], b"", tmp_path)
    assert r.returncode == 1 and b"USAGE" in r.stderr          # -tau is mandatory
    r = _run(cli, ["-tau", "0.1", "-bogus"], b"", tmp_path)
    assert r.returncode == 1 and b"USAGE" in r.stderr
    r = _run(cli, ["-tau"], b"", tmp_path)                      # a flag without its value
    assert r.returncode == 1 and b"USAGE" in r.stderr


def test_cli_rejects_malformed_tipsy(cli, tmp_path):
    r = _run(cli, ["-tau", "0.1"], b"\0" * 10, tmp_path)
    assert r.returncode == 2 and b"truncated TIPSY header" in r.stderr
    hdr = struct.pack("<diiiiii", 1.0, 100, 3, 0, 100, 0, 0)
    r = _run(cli, ["-tau", "0.1"], hdr + b"\0" * (36 * 5), tmp_path)
    assert r.returncode == 2 and b"truncated TIPSY particle records" in r.stderr
    hdr = struct.pack("<diiiiii", 1.0, 0, 3, -4, 0, 0, 0)
    r = _run(cli, ["-tau", "0.1"], hdr, tmp_path)
    assert r.returncode == 2 and b"bad particle counts" in r.stderr
    assert not any(p.name.endswith(".grp") for p in tmp_path.iterdir())


def _stdout_counts(text):
    out = {}
    for line in text.splitlines():
        for key, tag in (("nExtraScat", "nExtraScat:"), ("nGroupFoF", "Groups before Unbind:"),
                         ("nUnbound", "Number of particles Unbound:"), ("nGroup", "Number of Groups:")):
            if line.startswith(tag):
                out[key] = int(line.split(":")[1])
    out["nIter"] = sum(1 for l in text.splitlines() if l.startswith("Ittr")) - 1
    return out


def _flags_for(meta, case_dir):
    flags = list(meta["flags"])
    if "-unbind" in flags:
        i = flags.index("-unbind") + 1
        flags[i] = os.path.join(case_dir, flags[i])
    return flags


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["dark4k_periodic", "mixed6k", "dark8k_lcdm", "dark6k_nsp", "dark4k_unbind_gtp",
                                  "mixed6k_unbind_com", "demo_dark_std", "config0_32k",
                                  "mixed6k_go", "dark4k_center"])
def test_cli_vs_reference(gpu_ready, cli, tmp_path, name):
    from skid_gb300 import tipsy
    snap, opts, ref, counts, meta = gc.load(name)
    case_dir = os.path.join(gc.GOLDEN, name)
    data = gc.input_bytes(name, meta)
    r = _run(cli, [*_flags_for(meta, case_dir), "-o", "out"], data, tmp_path)
    assert r.returncode == 0, r.stderr.decode()
    got = _stdout_counts(r.stdout.decode())
    for key in ("nExtraScat", "nGroupFoF", "nGroup"):
        if key in counts:
            assert got[key] == counts[key], (key, got, counts)
    assert abs(got["nUnbound"] - counts["nUnbound"]) <= max(2, 0.001 * snap.n)
    if not opts.bUnbindOnly:
        assert got["nIter"] == counts["nIter"]
    grp = tipsy.read_grp(tmp_path / "out.grp")
    gtp = tipsy.read_gtp(tmp_path / "out.gtp", standard=opts.bStandard)
    groups = {"fMass": np.r_[0, gtp["mass"]].astype(np.float32),
              "rCenter": np.r_[np.zeros((1, 3)), gtp["pos"]].astype(np.float32),
              "vcm": np.r_[np.zeros((1, 3)), gtp["vel"]].astype(np.float32),
              "fRadius": np.r_[0, gtp["eps"]].astype(np.float32)}
    gc.check_catalogue(grp, groups, ref, opts)
    if "den" in ref:
        den = tipsy.read_den(tmp_path / "out.den")
        rel = np.abs(den - ref["den"]) / np.maximum(ref["den"], 1e-30)
        assert rel[ref["den"] > 0].max() < 1e-5
    if "stat" in ref:
        st = tipsy.read_stat(tmp_path / "out.stat")
        assert st.shape == ref["stat"].shape
        same = np.array_equal(grp, ref["grp"])
        if same:   # identical membership: every column agrees to float rounding
            np.testing.assert_allclose(st[:, :2], ref["stat"][:, :2])
            np.testing.assert_allclose(st[:, 2:], ref["stat"][:, 2:], rtol=2e-4, atol=2e-5)
    if "ray" in ref:
        ray = np.loadtxt(tmp_path / "out.ray", dtype=np.float64)
        want = np.loadtxt(gc.ref_path(name, "ray", meta), dtype=np.float64)
        assert ray[0] == want[0]
        assert np.abs(ray[1:] - want[1:]).max() < 0.2 * opts.fStep


@pytest.mark.gpu
def test_cli_matches_python_pipeline_and_xdr(gpu_ready, cli, tmp_path):
    """The C tool and the Python pipeline make the same calls: identical .grp
    and .gtp bytes; a -std (XDR) copy of the input gives the same groups."""
    from skid_gb300 import pipeline, synth, tipsy
    snap, opts, ref, counts, meta = gc.load("dark4k_periodic")
    with open(os.path.join(gc.GOLDEN, "dark4k_periodic", "input.bin"), "rb") as f:
        data = f.read()
    r = _run(cli, [*meta["flags"], "-o", "c"], data, tmp_path)
    assert r.returncode == 0, r.stderr.decode()
    opts.achName = "py"
    res = pipeline.run(snap, opts)
    pipeline.write_outputs(res, snap, opts, outdir=str(tmp_path))
    assert (tmp_path / "c.grp").read_bytes() == (tmp_path / "py.grp").read_bytes()
    assert (tmp_path / "c.gtp").read_bytes() == (tmp_path / "py.gtp").read_bytes()
    xdr = tmp_path / "input_xdr.bin"
    synth.write_snapshot(str(xdr), snap, standard=True)
    r = _run(cli, [*meta["flags"], "-std", "-o", "x"], xdr.read_bytes(), tmp_path)
    assert r.returncode == 0, r.stderr.decode()
    assert (tmp_path / "x.grp").read_bytes() == (tmp_path / "c.grp").read_bytes()
    a = tipsy.read_gtp(tmp_path / "x.gtp", standard=True)
    b = tipsy.read_gtp(tmp_path / "c.gtp")
    for f in ("mass", "pos", "vel", "eps", "tform"):
        assert np.array_equal(a[f], b[f])
