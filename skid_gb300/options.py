"""skid's command-line options, with the reference's defaults and rules.

Flags, defaults and derived values follow main.c:82-345 (semantics in
man1/skid.1:43-268): ``-tau`` is mandatory; fCvg = tau/2 and fScoop = 2 tau
unless given; fStep = fCvg/2; ``-p`` sets all three periods and switches on
periodic replica scatterers; nBucket is fixed.  Two flags are new: ``-nsp``
(no scatterer removal, README:29-30 describes it but v1.4.1 lacks it) and
``-maxiter`` (cap on outer move iterations; the reference loop has none,
main.c:409).  Values are parsed like C's atof/atoi: a malformed number gives 0.
"""
from __future__ import annotations

import dataclasses
import math
import re

import numpy as np

FLT_MAX = float(np.finfo(np.float32).max)
INT_MAX = 2**31 - 1
PLUMMER = 1
SPLINE = 2


class UsageError(ValueError):
    """Bad command line (the reference prints usage and exits 1, main.c:17-42)."""


def _atof(s: str) -> float:
    m = re.match(r"\s*[+-]?((\d+\.?\d*)|(\.\d+))([eE][+-]?\d+)?", s)
    if not m:
        m2 = re.match(r"\s*[+-]?(inf|infinity|nan)", s, re.I)
        return float(m2.group(0)) if m2 else 0.0
    return float(m.group(0))


def _atoi(s: str) -> int:
    m = re.match(r"\s*[+-]?\d+", s)
    return int(m.group(0)) if m else 0


def _f32(x: float) -> float:
    return float(np.float32(x))


@dataclasses.dataclass
class Options:
    fTau: float = 0.0
    z: float = 0.0
    Omega0: float = 1.0
    Lambda: float = 0.0
    fQuintess: float = 0.0
    G: float = 1.0
    H0: float = 0.0
    nSmooth: int = 64
    fDensMin: float = 0.0
    fTempMax: float = FLT_MAX
    fMassMax: float = FLT_MAX
    fCvg: float = 0.0
    fScoop: float = 0.0
    fStep: float = 0.0
    nMembers: int = 8
    nMaxMembers: int = INT_MAX
    bNoUnbind: bool = False
    bGasAndDark: bool = False
    bGasOnly: bool = False
    bUnbindOnly: bool = False
    achGroup: str = ""
    bForceInitialCut: bool = False
    periodic: bool = False
    iSoftType: int = SPLINE
    bEps: bool = False
    fEps: float = 0.0
    period: tuple = (FLT_MAX, FLT_MAX, FLT_MAX)
    center: tuple = (0.0, 0.0, 0.0)
    achName: str = "skid"
    bOutRay: bool = False
    bOutDens: bool = False
    bOutStats: bool = False
    bOutDiag: bool = False
    bStandard: bool = False
    bNoScatterCut: bool = False
    maxIter: int = 0

    @classmethod
    def parse(cls, argv) -> "Options":
        """Parse a skid argument list (without the program name)."""
        o = cls()
        argv = [str(a) for a in argv]
        period = [FLT_MAX] * 3
        center = [0.0] * 3
        bTau = bCvg = bScoop = False
        i = 0
        n = len(argv)

        def val():
            nonlocal i
            i += 1
            if i >= n:
                raise UsageError(f"{argv[i - 1]} needs a value")
            v = argv[i]
            i += 1
            return v

        while i < n:
            a = argv[i]
            if a == "-tau":
                o.fTau = _f32(_atof(val())); bTau = True
            elif a == "-z":
                o.z = _f32(_atof(val()))
            elif a == "-O":
                o.Omega0 = _f32(_atof(val()))
            elif a == "-Lambda":
                o.Lambda = _f32(_atof(val()))
            elif a == "-Q":
                o.fQuintess = _f32(_atof(val()))
            elif a == "-G":
                o.G = _f32(_atof(val()))
            elif a == "-H":
                o.H0 = _f32(_atof(val()))
            elif a == "-s":
                o.nSmooth = _atoi(val())
            elif a == "-d":
                o.fDensMin = _f32(_atof(val()))
            elif a == "-t":
                o.fTempMax = _f32(_atof(val()))
            elif a == "-M":
                o.fMassMax = _f32(_atof(val()))
            elif a == "-fic":
                o.bForceInitialCut = True; i += 1
            elif a == "-cvg":
                o.fCvg = _f32(_atof(val())); bCvg = True
            elif a == "-scoop":
                o.fScoop = _f32(_atof(val())); bScoop = True
            elif a == "-m":
                o.nMembers = _atoi(val())
            elif a == "-maxgroup":
                o.nMaxMembers = _atoi(val())
            elif a == "-nu":
                o.bNoUnbind = True; i += 1
            elif a == "-gd":
                o.bGasAndDark = True; i += 1
            elif a == "-go":
                o.bGasOnly = True; i += 1
            elif a == "-unbind":
                o.achGroup = val(); o.bUnbindOnly = True
            elif a == "-spline":
                o.iSoftType = SPLINE; i += 1
            elif a == "-plummer":
                o.iSoftType = PLUMMER; i += 1
            elif a == "-e":
                o.fEps = _f32(_atof(val())); o.bEps = True
            elif a == "-p":
                v = _f32(_atof(val())); period = [v, v, v]; o.periodic = True
            elif a == "-c":
                v = _f32(_atof(val())); center = [v, v, v]
            elif a == "-cx":
                center[0] = _f32(_atof(val()))
            elif a == "-cy":
                center[1] = _f32(_atof(val()))
            elif a == "-cz":
                center[2] = _f32(_atof(val()))
            elif a == "-o":
                o.achName = val()
            elif a == "-ray":
                o.bOutRay = True; i += 1
            elif a == "-den":
                o.bOutDens = True; i += 1
            elif a == "-stats":
                o.bOutStats = True; i += 1
            elif a == "-diag":
                o.bOutDiag = True; i += 1
            elif a == "-std":
                o.bStandard = True; i += 1
            elif a == "-nsp":
                o.bNoScatterCut = True; i += 1
            elif a == "-maxiter":
                o.maxIter = _atoi(val())
            else:
                raise UsageError(f"unknown argument {a}")
        if not bTau:
            raise UsageError("-tau is required")
        if not bCvg:
            o.fCvg = _f32(0.5 * o.fTau)
        if not bScoop:
            o.fScoop = _f32(2.0 * o.fTau)
        o.fStep = _f32(0.5 * o.fCvg)
        o.period = tuple(period)
        o.center = tuple(center)
        return o

    @property
    def a_shift(self) -> float:
        """Expansion factor a = 1/(1+z) as float (kd.c:1317)."""
        return _f32(1.0 / (1.0 + self.z))

    @property
    def a_hubble(self) -> float:
        """a*H(a) as float (kd.c:1318; cosmo.c:46-58 with no radiation)."""
        a = 1.0 / (1.0 + self.z)
        a32 = float(np.float32(a))
        curv = 1.0 - self.Omega0 - self.Lambda - self.fQuintess
        h = self.H0 * math.sqrt(self.Omega0 * a32 + curv * a32 * a32
                                + self.fQuintess * a32 * a32 * math.sqrt(a32)
                                + self.Lambda * a32 ** 4) / (a32 * a32)
        return _f32(a32 * h)
