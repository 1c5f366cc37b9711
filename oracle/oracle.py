"""ORACLE -- TEST INFRASTRUCTURE ONLY.

ctypes front end of the CPU restatement in skid_oracle.c.  Only the tests,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libskidoracle.so")
SRC = os.path.join(HERE, "skid_oracle.c")
REF_SKID = os.path.join(HERE, "_ref", "skid")
REF_NSP = os.path.join(HERE, "_ref", "skid_nsp")
# Staged copy of the reference's sources: untracked (gitignored), it travels
# with the working tree to hosts that have no reference checkout, where
# build_ref.sh compiles it for that host.
REF_SRC = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "src")
REF_FILES = ("main.c", "kd.c", "kd.h", "smooth1.c", "smooth1.h", "grav.c", "grav.h", "cosmo.c",
             "cosmo.h", "romberg.c", "runge.c", "runge.h", "tipsydefs.h", "totipnat.c",
             "Makefile", "README", "demo", "dark.std")

FLT_MAX = float(np.finfo(np.float32).max)


def build(force: bool = False) -> str:
    """Compile the restatement (gcc, no FMA contraction)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "skid_oracle.h"))):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                               "-o", tmp, SRC, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def stage_reference(checkout: str | None = None) -> str | None:
    """Copy the reference checkout's files into baseline/_ref/src, unchanged.

    The checkout is $SKID_REF_CHECKOUT, else the read-only checkout mounted
    at /root/reference where this repository is developed.  Returns the
    staged directory, or None when neither a checkout nor a staged copy
    exists."""
    checkout = checkout or os.environ.get("SKID_REF_CHECKOUT") or "/root/reference"
    if os.path.exists(os.path.join(checkout, "kd.c")):
        os.makedirs(REF_SRC, exist_ok=True)
        for f in REF_FILES:
            src = os.path.join(checkout, f)
            dst = os.path.join(REF_SRC, f)
            if os.path.exists(src) and (not os.path.exists(dst)
                                        or os.path.getmtime(dst) < os.path.getmtime(src)):
                shutil.copyfile(src, dst)
    return REF_SRC if os.path.exists(os.path.join(REF_SRC, "kd.c")) else None


def _ref_stale() -> bool:
    if not (os.path.exists(REF_SKID) and os.path.exists(REF_NSP)):
        return True
    t = min(os.path.getmtime(REF_SKID), os.path.getmtime(REF_NSP))
    deps = [os.path.join(REF_SRC, f) for f in REF_FILES if f.endswith((".c", ".h"))]
    deps += [os.path.join(HERE, "build_ref.sh"), os.path.join(HERE, "nsp_shim.c")]
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def build_reference(force: bool = False) -> str | None:
    """Build the unmodified reference into oracle/_ref from the staged sources
    (staging them first when a checkout is present).  Returns the binary, or
    None when no sources are available on this host."""
    src = stage_reference()
    if src is None:
        return None
    if force or _ref_stale():
        subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), src],
                              stdout=subprocess.DEVNULL)
    return REF_SKID


class Params(C.Structure):
    _fields_ = [("period", C.c_float * 3), ("center", C.c_float * 3), ("periodic", C.c_int),
                ("nSmooth", C.c_int), ("fTau", C.c_float), ("fCvg", C.c_float),
                ("fScoop", C.c_float), ("fStep", C.c_float), ("fDensMin", C.c_float),
                ("fTempMax", C.c_float), ("fMassMax", C.c_float), ("bGasAndDark", C.c_int),
                ("bGasOnly", C.c_int), ("bForceInitialCut", C.c_int),
                ("bNoScatterCut", C.c_int), ("nMinMembers", C.c_int), ("nMaxMembers", C.c_int),
                ("bNoUnbind", C.c_int), ("iSoftType", C.c_int), ("bEps", C.c_int),
                ("fEps", C.c_float), ("G", C.c_float), ("Omega0", C.c_float),
                ("Lambda", C.c_float), ("fQuintess", C.c_float), ("H0", C.c_float),
                ("z", C.c_float), ("maxIter", C.c_int), ("verbose", C.c_int),
                ("stopAfter", C.c_int)]


class Group(C.Structure):
    _fields_ = [("nMembers", C.c_int), ("fMass", C.c_float), ("rel", C.c_float * 3),
                ("rCenter", C.c_float * 3), ("rBound", C.c_float * 3), ("vcm", C.c_float * 3),
                ("fRadius", C.c_float)]


class Result(C.Structure):
    _fields_ = [("nScatterInit", C.c_int), ("nExtraScat", C.c_int), ("nMove", C.c_int),
                ("nIter", C.c_int), ("nGroupFoF", C.c_int), ("nUnbound", C.c_int),
                ("nGroup", C.c_int), ("nScatFinal", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        f = C.POINTER(C.c_float)
        d = C.POINTER(C.c_double)
        i = C.POINTER(C.c_int)
        u = C.POINTER(C.c_uint)
        _lib.or_knn_ball2.argtypes = [C.c_int, f, C.c_int, f, f]
        _lib.or_knn_ball2_brute.argtypes = [C.c_int, f, C.c_int, f, f]
        _lib.or_density.argtypes = [C.c_int, f, f, f, f, d]
        _lib.or_replica_mask.argtypes = [C.c_int, f, f, f, f, C.c_int, u]
        _lib.or_field.argtypes = [C.c_int, f, f, f, u, C.c_int, f, f, d, d, u]
        _lib.or_fof.argtypes = [C.c_int, f, f, C.c_float, i, i]
        _lib.or_d2.argtypes = [f, f, f]
        _lib.or_d2.restype = C.c_float
        _lib.or_run.argtypes = [C.POINTER(Params), C.c_int, C.c_int, C.c_int, C.c_double,
                                f, f, f, f, f, i, C.POINTER(Group), C.c_int, f, f, f,
                                C.POINTER(Result)]
        _lib.or_density_adjoint_check.argtypes = [C.c_int, f, f, f, C.c_int, f, C.c_int, i,
                                                  C.c_double, d, d, d, i]
        _lib.or_density_adjoint_check2.argtypes = [C.c_int, f, f, f, C.c_int, f, C.c_int, i,
                                                   C.c_double, d, d, d, d, i]
        _lib.or_field_grad_check.argtypes = [C.c_int, f, f, f, f, C.c_int, f, C.c_double, d, d, d]
        _lib.or_run_unbind.argtypes = [C.POINTER(Params), C.c_int, C.c_int, C.c_int, f, f, f, f,
                                       i, f, C.POINTER(Group), C.c_int, C.POINTER(Result)]
    return _lib


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _up(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint))


def _period(period):
    if period is None:
        return np.full(3, FLT_MAX, np.float32)
    p = np.asarray(period, np.float32)
    return np.full(3, p, np.float32) if p.ndim == 0 else p.copy()


def knn_ball2(pos, k, period=None, brute=False):
    pos = np.ascontiguousarray(pos, np.float32)
    out = np.empty(len(pos), np.float32)
    fn = lib().or_knn_ball2_brute if brute else lib().or_knn_ball2
    rc = fn(len(pos), _fp(pos), int(k), _fp(_period(period)), _fp(out))
    if rc:
        raise ValueError("oracle knn failed")
    return out


def density(pos, mass, ball2, period=None):
    pos = np.ascontiguousarray(pos, np.float32)
    mass = np.ascontiguousarray(mass, np.float32)
    ball2 = np.ascontiguousarray(ball2, np.float32)
    out = np.empty(len(pos), np.float64)
    lib().or_density(len(pos), _fp(pos), _fp(mass), _fp(ball2), _fp(_period(period)), _dp(out))
    return out


def replica_mask(pos, ball2, period=None, center=(0, 0, 0), periodic=True):
    pos = np.ascontiguousarray(pos, np.float32)
    ball2 = np.ascontiguousarray(ball2, np.float32)
    out = np.empty(len(pos), np.uint32)
    lib().or_replica_mask(len(pos), _fp(pos), _fp(ball2), _fp(_period(period)),
                          _fp(np.asarray(center, np.float32)), int(periodic), _up(out))
    return out


def field(spos, smass, sball2, alive, mpos, period=None):
    """Move field (minus the SPH density gradient) at mover positions, FP64.
    Returns (acc, sum of |term| per mover, touched copy bits per scatterer)."""
    spos = np.ascontiguousarray(spos, np.float32)
    smass = np.ascontiguousarray(smass, np.float32)
    sball2 = np.ascontiguousarray(sball2, np.float32)
    alive = np.ascontiguousarray(alive, np.uint32)
    mpos = np.ascontiguousarray(mpos, np.float32)
    acc = np.empty((len(mpos), 3), np.float64)
    absacc = np.empty(len(mpos), np.float64)
    touched = np.empty(len(spos), np.uint32)
    lib().or_field(len(spos), _fp(spos), _fp(smass), _fp(sball2), _up(alive), len(mpos),
                   _fp(mpos), _fp(_period(period)), _dp(acc), _dp(absacc), _up(touched))
    return acc, absacc, touched


def fof(pos, tau, period=None, iorder=None):
    pos = np.ascontiguousarray(pos, np.float32)
    n = len(pos)
    io = np.arange(n, dtype=np.int32) if iorder is None else np.ascontiguousarray(iorder, np.int32)
    grp = np.empty(n, np.int32)
    ng = lib().or_fof(n, _fp(pos), _fp(_period(period)), float(tau), _ip(io), _ip(grp))
    return grp, ng


def d2(q, c, period=None):
    q = np.ascontiguousarray(q, np.float32)
    c = np.ascontiguousarray(c, np.float32)
    return float(lib().or_d2(_fp(q), _fp(c), _fp(_period(period))))


def _params(flags, verbose=False, max_iter=0, stop_after=0):
    from skid_gb300.options import Options
    o = flags if isinstance(flags, Options) else Options.parse(flags)
    p = Params()
    for d in range(3):
        p.period[d] = o.period[d]
        p.center[d] = o.center[d]
    p.periodic = int(o.periodic)
    p.nSmooth = o.nSmooth
    p.fTau, p.fCvg, p.fScoop, p.fStep = o.fTau, o.fCvg, o.fScoop, o.fStep
    p.fDensMin, p.fTempMax, p.fMassMax = o.fDensMin, o.fTempMax, o.fMassMax
    p.bGasAndDark, p.bGasOnly, p.bForceInitialCut = int(o.bGasAndDark), int(o.bGasOnly), int(o.bForceInitialCut)
    p.bNoScatterCut = int(o.bNoScatterCut)
    p.nMinMembers, p.nMaxMembers, p.bNoUnbind = o.nMembers, o.nMaxMembers, int(o.bNoUnbind)
    p.iSoftType = o.iSoftType
    p.bEps, p.fEps = int(o.bEps), o.fEps
    p.G, p.Omega0, p.Lambda, p.fQuintess, p.H0, p.z = o.G, o.Omega0, o.Lambda, o.fQuintess, o.H0, o.z
    p.maxIter = max_iter or o.maxIter
    p.verbose = int(verbose)
    p.stopAfter = int(stop_after)
    return o, p


def _groups(groups, ng):
    return {
        "nMembers": np.array([groups[g].nMembers for g in range(ng)], np.int64),
        "fMass": np.array([groups[g].fMass for g in range(ng)], np.float32),
        "rCenter": np.array([list(groups[g].rCenter) for g in range(ng)], np.float32),
        "vcm": np.array([list(groups[g].vcm) for g in range(ng)], np.float32),
        "rBound": np.array([list(groups[g].rBound) for g in range(ng)], np.float32),
        "fRadius": np.array([groups[g].fRadius for g in range(ng)], np.float32),
    }


def run(snap, flags, verbose=False, max_iter=0, stop_after=0):
    """Run the whole pipeline on a Snapshot with skid-style options (a
    ``skid_gb300.options.Options``).  Returns a dict of arrays.  stop_after=1
    stops after the group centres (FoF groups), 2 after unbinding."""
    o, p = _params(flags, verbose, max_iter, stop_after)
    n = snap.n
    pos = np.ascontiguousarray(snap.pos, np.float32)
    vel = np.ascontiguousarray(snap.vel, np.float32)
    mass = np.ascontiguousarray(snap.mass, np.float32)
    soft = np.ascontiguousarray(snap.soft, np.float32)
    temp = np.ascontiguousarray(snap.temp, np.float32)
    grp = np.empty(n, np.int32)
    cap = n + 1
    groups = (Group * cap)()
    rho = np.empty(n, np.float32)
    ball2 = np.empty(n, np.float32)
    moved = np.empty((n, 3), np.float32)
    res = Result()
    rc = lib().or_run(C.byref(p), snap.n_gas, snap.n_dark, snap.n_star, snap.time,
                      _fp(pos), _fp(vel), _fp(mass), _fp(soft), _fp(temp), _ip(grp), groups, cap,
                      _fp(rho), _fp(ball2), _fp(moved), C.byref(res))
    if rc:
        raise ValueError(f"oracle run failed: {rc}")
    gr = _groups(groups, res.nGroup + 1)
    return {"grp": grp, "groups": gr, "rho": rho, "ball2": ball2, "moved": moved,
            "nScatterInit": res.nScatterInit, "nExtraScat": res.nExtraScat,
            "nMove": res.nMove, "nIter": res.nIter, "nGroupFoF": res.nGroupFoF,
            "nUnbound": res.nUnbound, "nGroup": res.nGroup, "nScatFinal": res.nScatFinal}


def run_unbind(snap, flags, grp, centers=None, verbose=False, stop_after=0):
    """Unbind-only mode (-unbind): grp holds the input group ids by iOrder,
    centers is None (centre of mass) or an array (nGroup-1, 6) of rCenter and
    vcm from a .gtp file.  stop_after=2 stops after unbinding (no too-small)."""
    o, p = _params(flags, verbose, 0, stop_after)
    pos = np.ascontiguousarray(snap.pos, np.float32)
    vel = np.ascontiguousarray(snap.vel, np.float32)
    mass = np.ascontiguousarray(snap.mass, np.float32)
    soft = np.ascontiguousarray(snap.soft, np.float32)
    g = np.array(grp, np.int32)
    cap = int(g.max(initial=0)) + 2
    groups = (Group * cap)()
    cptr = None
    if centers is not None:
        c = np.ascontiguousarray(centers, np.float32).reshape(-1, 6)
        cptr = _fp(c)
    res = Result()
    rc = lib().or_run_unbind(C.byref(p), snap.n_gas, snap.n_dark, snap.n_star, _fp(pos), _fp(vel),
                             _fp(mass), _fp(soft), _ip(g), cptr, groups, cap, C.byref(res))
    if rc:
        raise ValueError(f"oracle unbind-only run failed: {rc}")
    return {"grp": g, "groups": _groups(groups, res.nGroup + 1), "nGroupFoF": res.nGroupFoF,
            "nUnbound": res.nUnbound, "nGroup": res.nGroup}


def density_adjoint_check(pos, mass, w, k, period, sel, h=1e-6, richardson=False):
    """FP64 gradient of L = sum w_i rho_i at particles sel: (analytic, central
    differences of step h, sum of |term|), neighbour sets held fixed.  With
    richardson, the differences are (4 D(h/2) - D(h)) / 3, which cancels their
    O(h^2) truncation error (it reaches 1e-5 of the gradient where smoothing
    lengths are only ~100 h)."""
    pos = np.ascontiguousarray(pos, np.float32)
    mass = np.ascontiguousarray(mass, np.float32)
    w = np.ascontiguousarray(w, np.float32)
    sel = np.ascontiguousarray(sel, np.int32)
    an = np.empty((len(sel), 3))
    fd = np.empty((len(sel), 3))
    ab = np.empty(len(sel))
    ok = C.c_int(0)
    fd2 = np.empty((len(sel), 3)) if richardson else None
    rc = lib().or_density_adjoint_check2(len(pos), _fp(pos), _fp(mass), _fp(w), int(k),
                                         _fp(_period(period)), len(sel), _ip(sel), h, _dp(an),
                                         _dp(fd), _dp(fd2) if richardson else None, _dp(ab),
                                         C.byref(ok))
    if rc:
        raise ValueError(f"density adjoint check failed: {rc} (lists_ok={ok.value})")
    if richardson:
        fd = (4.0 * fd2 - fd) / 3.0
    return an, fd, ab


def field_grad_check(spos, smass, sball2, period, ypos, h=1e-6):
    """FP64 gradient of the density field at ypos: (analytic, central
    differences, sum of |term|)."""
    spos = np.ascontiguousarray(spos, np.float32)
    smass = np.ascontiguousarray(smass, np.float32)
    sball2 = np.ascontiguousarray(sball2, np.float32)
    ypos = np.ascontiguousarray(ypos, np.float32)
    an = np.empty((len(ypos), 3))
    fd = np.empty((len(ypos), 3))
    ab = np.empty(len(ypos))
    lib().or_field_grad_check(len(spos), _fp(spos), _fp(smass), _fp(sball2), _fp(_period(period)),
                              len(ypos), _fp(ypos), h, _dp(an), _dp(fd), _dp(ab))
    return an, fd, ab
