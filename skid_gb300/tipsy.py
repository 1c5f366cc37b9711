"""TIPSY binary snapshots and skid's output files, in numpy.

Formats follow the reference reader/writers:

* header ``struct dump`` {double time; int nbodies, ndim, nsph, ndark, nstar}
  (tipsydefs.h:39-46) -- 28 bytes, padded to 32 in native files; the XDR
  ("-std") form writes an explicit zero pad word (kd.c:16-28);
* gas records of 12 floats, dark of 9, star of 11 (tipsydefs.h:6-37), in the
  order gas, dark, star; that order defines iOrder and particle type
  (kd.c:113-119, 164-217);
* ``.grp``: N, then one group id per line in iOrder (kd.c:1518-1519);
* ``.gtp``: a TIPSY file holding nGroup-1 star particles (kd.c:1648-1682);
* ``.den``: N, then ``%.10g`` density per line in iOrder (kd.c:1541-1545).
"""
from __future__ import annotations

import dataclasses
import io
import os

import numpy as np

GAS_DT = np.dtype([("mass", "f4"), ("pos", "f4", 3), ("vel", "f4", 3), ("rho", "f4"),
                   ("temp", "f4"), ("hsmooth", "f4"), ("metals", "f4"), ("phi", "f4")])
DARK_DT = np.dtype([("mass", "f4"), ("pos", "f4", 3), ("vel", "f4", 3), ("eps", "f4"),
                    ("phi", "f4")])
STAR_DT = np.dtype([("mass", "f4"), ("pos", "f4", 3), ("vel", "f4", 3), ("metals", "f4"),
                    ("tform", "f4"), ("eps", "f4"), ("phi", "f4")])
HEADER_NATIVE = np.dtype([("time", "<f8"), ("nbodies", "<i4"), ("ndim", "<i4"),
                          ("nsph", "<i4"), ("ndark", "<i4"), ("nstar", "<i4"),
                          ("pad", "<i4")])
HEADER_XDR = np.dtype([("time", ">f8"), ("nbodies", ">i4"), ("ndim", ">i4"),
                       ("nsph", ">i4"), ("ndark", ">i4"), ("nstar", ">i4"),
                       ("pad", ">i4")])


class TipsyError(ValueError):
    """Malformed or truncated TIPSY input."""


@dataclasses.dataclass
class Snapshot:
    """Particles in iOrder (gas, then dark, then star), as the reference reads them.

    ``soft`` is hsmooth for gas and eps for dark/star; ``temp`` is 0 for non-gas
    (kd.c:176-214).
    """
    time: float
    n_gas: int
    n_dark: int
    n_star: int
    pos: np.ndarray      # (N, 3) float32
    vel: np.ndarray      # (N, 3) float32
    mass: np.ndarray     # (N,) float32
    soft: np.ndarray     # (N,) float32
    temp: np.ndarray     # (N,) float32
    gas: np.ndarray | None = None
    dark: np.ndarray | None = None
    star: np.ndarray | None = None

    @property
    def n(self) -> int:
        return self.n_gas + self.n_dark + self.n_star


def _endian(dt: np.dtype, big: bool) -> np.dtype:
    return dt.newbyteorder(">") if big else dt.newbyteorder("<")


def read_tipsy(path_or_bytes, standard: bool = False) -> Snapshot:
    """Read a native (little-endian) or XDR (``standard=True``) TIPSY file."""
    if isinstance(path_or_bytes, (bytes, bytearray, memoryview)):
        buf = bytes(path_or_bytes)
    else:
        with open(path_or_bytes, "rb") as f:
            buf = f.read()
    hdt = HEADER_XDR if standard else HEADER_NATIVE
    if len(buf) < hdt.itemsize:
        raise TipsyError("truncated TIPSY header")
    h = np.frombuffer(buf, dtype=hdt, count=1)[0]
    ng, nd, ns = int(h["nsph"]), int(h["ndark"]), int(h["nstar"])
    if min(ng, nd, ns) < 0:
        raise TipsyError("negative particle count in TIPSY header")
    off = hdt.itemsize
    parts = []
    for cnt, dt in ((ng, GAS_DT), (nd, DARK_DT), (ns, STAR_DT)):
        dte = _endian(dt, standard)
        need = cnt * dte.itemsize
        if off + need > len(buf):
            raise TipsyError("truncated TIPSY particle records")
        parts.append(np.frombuffer(buf, dtype=dte, count=cnt, offset=off).astype(dt.newbyteorder("=")))
        off += need
    gas, dark, star = parts
    n = ng + nd + ns
    pos = np.empty((n, 3), np.float32)
    vel = np.empty((n, 3), np.float32)
    mass = np.empty(n, np.float32)
    soft = np.empty(n, np.float32)
    temp = np.zeros(n, np.float32)
    s = 0
    for arr, softname in ((gas, "hsmooth"), (dark, "eps"), (star, "eps")):
        e = s + len(arr)
        pos[s:e] = arr["pos"]
        vel[s:e] = arr["vel"]
        mass[s:e] = arr["mass"]
        soft[s:e] = arr[softname]
        s = e
    temp[:ng] = gas["temp"]
    return Snapshot(float(h["time"]), ng, nd, ns, pos, vel, mass, soft, temp, gas, dark, star)


def write_tipsy(path, time: float, gas=None, dark=None, star=None, standard: bool = False) -> None:
    """Write record arrays (GAS_DT/DARK_DT/STAR_DT) as one TIPSY file."""
    gas = np.zeros(0, GAS_DT) if gas is None else gas
    dark = np.zeros(0, DARK_DT) if dark is None else dark
    star = np.zeros(0, STAR_DT) if star is None else star
    hdt = HEADER_XDR if standard else HEADER_NATIVE
    h = np.zeros(1, hdt)
    h["time"] = time
    h["nbodies"] = len(gas) + len(dark) + len(star)
    h["ndim"] = 3
    h["nsph"] = len(gas)
    h["ndark"] = len(dark)
    h["nstar"] = len(star)
    with open(path, "wb") as f:
        f.write(h.tobytes())
        for arr, dt in ((gas, GAS_DT), (dark, DARK_DT), (star, STAR_DT)):
            f.write(np.asarray(arr, dt).astype(_endian(dt, standard)).tobytes())


def snapshot_records(snap: Snapshot):
    """Rebuild gas/dark/star record arrays from a Snapshot's iOrder arrays."""
    ng, nd, ns = snap.n_gas, snap.n_dark, snap.n_star
    gas = np.zeros(ng, GAS_DT)
    dark = np.zeros(nd, DARK_DT)
    star = np.zeros(ns, STAR_DT)
    sl = (slice(0, ng), slice(ng, ng + nd), slice(ng + nd, ng + nd + ns))
    for arr, s in zip((gas, dark, star), sl):
        arr["mass"] = snap.mass[s]
        arr["pos"] = snap.pos[s]
        arr["vel"] = snap.vel[s]
    gas["hsmooth"] = snap.soft[sl[0]]
    gas["temp"] = snap.temp[sl[0]]
    dark["eps"] = snap.soft[sl[1]]
    star["eps"] = snap.soft[sl[2]]
    return gas, dark, star


def read_grp(path) -> np.ndarray:
    """Read a ``.grp`` file (N then one id per line)."""
    a = np.loadtxt(path, dtype=np.int64)
    a = np.atleast_1d(a)
    n = int(a[0])
    if len(a) != n + 1:
        raise TipsyError(f"{path}: header says {n} particles, found {len(a) - 1}")
    return a[1:].astype(np.int32)


def write_grp(path, grp: np.ndarray) -> None:
    with open(path, "w") as f:
        f.write(f"{len(grp)}\n")
        if len(grp):
            f.write("\n".join(map(str, np.asarray(grp).tolist())))
            f.write("\n")


def read_den(path) -> np.ndarray:
    a = np.loadtxt(path, dtype=np.float64)
    a = np.atleast_1d(a)
    n = int(a[0])
    if len(a) != n + 1:
        raise TipsyError(f"{path}: header says {n} particles, found {len(a) - 1}")
    return a[1:]


def read_gtp(path, standard: bool = False) -> np.ndarray:
    """Group centres as star records: mass, pos=centre, vel=vcm, eps=radius."""
    snap = read_tipsy(path, standard)
    return snap.star


def read_stat(path) -> np.ndarray:
    """The 21-column ``.stat`` table (kd.c:1811-1833) as float64 rows."""
    if os.path.getsize(path) == 0:
        return np.zeros((0, 21))
    a = np.loadtxt(path, dtype=np.float64, ndmin=2)
    return a
