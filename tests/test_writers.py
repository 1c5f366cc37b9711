"""The skid tool's text writers (.grp, .den, .ray; kd.c:1502-1608) format
their lines in parallel chunks and write them in order: the files must be
byte for byte what one printf per line gives (here Python's formatting of
the same values, which rounds correctly as glibc's printf does), on both
sides of the threaded size and across the writers' block of 2^22 lines."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "skid_gb300", "host")


class Snapshot(C.Structure):
    _fields_ = [("time", C.c_double), ("nGas", C.c_int), ("nDark", C.c_int), ("nStar", C.c_int),
                ("n", C.c_int), ("pos", C.POINTER(C.c_float)), ("vel", C.POINTER(C.c_float)),
                ("mass", C.POINTER(C.c_float)), ("soft", C.POINTER(C.c_float)),
                ("temp", C.POINTER(C.c_float))]


@pytest.fixture(scope="module")
def writers(tmp_path_factory):
    """tipsy_io.c as a shared object (its reader links against libskidgpu)."""
    from skid_gb300 import build
    lib = build.build_lib()
    out = str(tmp_path_factory.mktemp("writers") / "libtipsyio.so")
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off",
                           "-fPIC", "-shared", "-I" + os.path.join(ROOT, "include"), "-o", out,
                           os.path.join(HOST, "tipsy_io.c"), "-L" + os.path.dirname(lib),
                           "-lskidgpu", "-Wl,-rpath," + os.path.dirname(lib), "-lm", "-pthread"])
    return C.CDLL(out)


def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


@pytest.mark.parametrize("n", [5, 70001, (1 << 21) + 3])   # .ray of the last: 3n > 2^22 lines
def test_text_writers_match_printf(writers, tmp_path, n):
    rng = np.random.default_rng(n)
    grp = rng.integers(-5000, 40000, n).astype(np.int32)
    grp[: min(n, 2)] = [-2**31, 2**31 - 1][: min(n, 2)]
    rho = rng.standard_normal(n).astype(np.float32) * np.float32(10.0) ** rng.integers(-30, 30, n)
    rho = rho.astype(np.float32)
    pos = rng.uniform(-0.5, 0.5, (n, 3)).astype(np.float32)
    moved = (pos + rng.uniform(-0.7, 0.7, (n, 3))).astype(np.float32)
    flag = (rng.random(n) < 0.7).astype(np.int32)
    period = np.array([1.0, 1.0, 2.0], np.float32)

    p_grp, p_den, p_ray = (str(tmp_path / f) for f in ("o.grp", "o.den", "o.ray"))
    assert writers.write_grp(p_grp.encode(), n, grp.ctypes.data_as(C.POINTER(C.c_int))) == 0
    assert writers.write_den(p_den.encode(), n, _f(rho)) == 0
    snap = Snapshot(0.0, 0, n, 0, n, _f(pos), None, None, None, None)
    assert writers.write_ray(p_ray.encode(), C.byref(snap), _f(moved),
                             flag.ctypes.data_as(C.POINTER(C.c_int)), _f(period)) == 0

    with open(p_grp, "rb") as f:
        assert f.read() == (f"{n}\n" + "".join(f"{v}\n" for v in grp.tolist())).encode()
    with open(p_den, "rb") as f:
        assert f.read() == (f"{n}\n" + "".join("%.10g\n" % v for v in rho.tolist())).encode()
    lines = [f"{n}\n"]
    for d in range(3):
        h = np.float32(0.5 * float(period[d]))
        dx = (moved[:, d] - pos[:, d]).astype(np.float32)
        dx = np.where(dx > h, dx - np.float32(2) * h, dx).astype(np.float32)
        dx = np.where(dx <= -h, dx + np.float32(2) * h, dx).astype(np.float32)
        lines += ["%g\n" % v if m else "0\n" for v, m in zip(dx.tolist(), flag.tolist())]
    with open(p_ray, "rb") as f:
        assert f.read() == "".join(lines).encode()
