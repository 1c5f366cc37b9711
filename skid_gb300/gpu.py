"""ctypes binding of libskidgpu (include/skid_gpu.h).

There is no CPU fallback: if the library is missing or cannot load, every
call raises.  Arrays are numpy, indexed by iOrder.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .options import FLT_MAX

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libskidgpu.so")

SKID_ERRORS = {
    -1: "invalid argument", -2: "out of memory", -3: "CUDA runtime error",
    -4: "bounded device wait ran out", -5: "internal capacity exceeded",
    -6: "no usable sm_103 device", -7: "call made in the wrong pipeline state",
    -8: "request exceeds a fixed capacity",
}


class SkidError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        super().__init__(f"{where}: {SKID_ERRORS.get(code, 'error')} ({code})")


class Params(C.Structure):
    _fields_ = [("period", C.c_float * 3), ("center", C.c_float * 3), ("periodic", C.c_int),
                ("nSmooth", C.c_int), ("device", C.c_int)]


class Group(C.Structure):
    _fields_ = [("nMembers", C.c_int), ("fMass", C.c_float), ("rel", C.c_float * 3),
                ("rCenter", C.c_float * 3), ("rBound", C.c_float * 3), ("vcm", C.c_float * 3),
                ("fRadius", C.c_float)]


class Timings(C.Structure):
    _fields_ = [("density_ms", C.c_float), ("moving_ms", C.c_float), ("fof_ms", C.c_float),
                ("micro_ms", C.c_float), ("groups_ms", C.c_float), ("unbind_ms", C.c_float),
                ("toosmall_ms", C.c_float), ("gather_launches", C.c_longlong),
                ("kernel_launches", C.c_longlong), ("field_ms", C.c_double),
                ("field_bytes", C.c_double)]


class Volume(C.Structure):
    _fields_ = [("nGas", C.c_int), ("nDark", C.c_int), ("nStar", C.c_int), ("time", C.c_double),
                ("pos", C.c_void_p), ("vel", C.c_void_p), ("mass", C.c_void_p),
                ("soft", C.c_void_p), ("temp", C.c_void_p), ("period", C.c_float * 3),
                ("center", C.c_float * 3), ("periodic", C.c_int), ("nSmooth", C.c_int),
                ("fTau", C.c_float), ("fCvg", C.c_float), ("fScoop", C.c_float),
                ("grp", C.c_void_p), ("groups", C.c_void_p), ("groups_cap", C.c_int),
                ("nGroup", C.c_int), ("nGroupFoF", C.c_int), ("nUnbound", C.c_int),
                ("nIter", C.c_int), ("device_ms", C.c_float), ("status", C.c_int),
                ("message", C.c_char * 96)]


class BatchFlags(C.Structure):
    _fields_ = [("fDensMin", C.c_float), ("fTempMax", C.c_float), ("fMassMax", C.c_float),
                ("nMembers", C.c_int), ("nMaxMembers", C.c_int), ("bGasAndDark", C.c_int),
                ("bGasOnly", C.c_int), ("bForceInitialCut", C.c_int), ("bNoUnbind", C.c_int),
                ("bNoCut", C.c_int), ("iSoftType", C.c_int), ("bEps", C.c_int),
                ("fEps", C.c_float), ("G", C.c_float), ("z", C.c_float), ("a", C.c_float),
                ("aH", C.c_float), ("maxIter", C.c_int)]


GROUP_DTYPE = np.dtype([("nMembers", "<i4"), ("fMass", "<f4"), ("rel", "<f4", 3),
                        ("rCenter", "<f4", 3), ("rBound", "<f4", 3), ("vcm", "<f4", 3),
                        ("fRadius", "<f4")])
assert GROUP_DTYPE.itemsize == C.sizeof(Group)
# skid_stat (kdOutStats' per-group columns)
STAT_DTYPE = np.dtype([("nMembers", "<i4"), ("fTotMass", "<f4"), ("fGasMass", "<f4"),
                       ("fStarMass", "<f4"), ("fVcirc2Max", "<f4"), ("fVcirc2Half", "<f4"),
                       ("fVcirc2Outer", "<f4"), ("fRVmax", "<f4"), ("fRHalf", "<f4"),
                       ("fROuter2", "<f4"), ("fVdisp", "<f4")])

_I = C.POINTER(C.c_int)
_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_V = C.c_void_p

# entry point -> argtypes (all return int status)
SIGNATURES = {
    "skid_create": [C.POINTER(C.c_void_p), C.POINTER(Params)],
    "skid_destroy": [_V],
    "skid_last_error": [_V],
    "skid_set_particles": [_V, C.c_int, C.c_int, C.c_int, C.c_double, _F, _F, _F, _F, _F],
    "skid_scatter_active": [_V, C.c_int, C.c_int, _I],
    "skid_density": [_V, _I],
    "skid_get_density": [_V, _F, _F],
    "skid_init_move": [_V, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, _I],
    "skid_move_step": [_V, C.c_float, C.c_int, C.c_int, _I],
    "skid_prune_inactive": [_V, C.c_float, _I],
    "skid_move_iterate": [_V, C.c_float, C.c_float, C.c_int, _I, _I],
    "skid_reactivate_move": [_V],
    "skid_fof": [_V, C.c_float, _I],
    "skid_group_centers": [_V],
    "skid_set_groups": [_V, _I, C.c_int, C.c_void_p],
    "skid_set_soft": [_V, C.c_float],
    "skid_unbind": [_V, C.c_int, C.c_float, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                    C.c_float, C.c_float, _I],
    "skid_too_small": [_V, C.c_int, _I],
    "skid_get_groups": [_V, _I, C.c_void_p],
    "skid_group_stats": [_V, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p],
    "skid_get_moved": [_V, _F],
    "skid_get_final_density": [_V, _F],
    "skid_get_timings": [_V, C.POINTER(Timings)],
    "skid_stream": [_V, C.POINTER(C.c_void_p)],
    "skid_restart": [_V],
    "skid_field_stats": [_V, C.c_int, C.POINTER(C.c_ulonglong)],
    "skid_set_option": [_V, C.c_char_p, C.c_double],
    "skid_get_option": [_V, C.c_char_p, _D],
    "skid_knn_ball2": [_V, C.c_int, _F, C.c_int, _F],
    "skid_field": [_V, C.c_int, _F, _F],
    "skid_fof_points": [_V, C.c_int, _F, C.c_float, _I, _I],
    "skid_density_adjoint": [_V, _F, _F, C.c_int],
    "skid_field_adjoint": [_V, C.c_int, _F, _F, _F],
    "skid_potential_adjoint": [_V, C.c_int, C.c_float, C.c_int, _I, _F, _D, _F],
    "skid_batch_run": [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int],
    "skid_pair_factor": [C.c_int, _F, _F, C.c_int, C.c_int, _F],
}

PAIR_USED = 0
PAIR_FP64 = 1
PAIR_SPLINE_FF = 2

ADJ_RECOMPUTE = 0
ADJ_STORED = 1
ADJ_AUTO = 2

_lib = None


def load(path: str = LIB_PATH):
    """Load libskidgpu; raises if it is missing (there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"libskidgpu not built ({path}); run skid_gb300.build")
        lib = C.CDLL(path)
        for name, args in SIGNATURES.items():
            f = getattr(lib, name, None)
            if f is None:
                continue
            f.argtypes = args
            f.restype = C.c_int
        lib.skid_strerror.argtypes = [C.c_int]
        lib.skid_strerror.restype = C.c_char_p
        lib.skid_last_cuda_error.argtypes = [C.c_void_p]
        lib.skid_last_cuda_error.restype = C.c_char_p
        _lib = lib
    return _lib


def exported_symbols(path: str = LIB_PATH):
    lib = C.CDLL(path)
    return {name for name in list(SIGNATURES) + ["skid_strerror", "skid_last_cuda_error"]
            if hasattr(lib, name)}


def _f(a):
    return a.ctypes.data_as(_F) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_I) if a is not None else None


def _c32(a, shape=None):
    a = np.ascontiguousarray(a, np.float32)
    if shape is not None:
        a = a.reshape(shape)
    return a


class Context:
    """One libskidgpu context (one GPU stream).  Methods mirror the C ABI."""

    def __init__(self, period=None, center=(0.0, 0.0, 0.0), periodic=None, nSmooth=64, device=0):
        self.lib = load()
        p = Params()
        per = [FLT_MAX] * 3 if period is None else (list(period) if np.ndim(period) else [float(period)] * 3)
        for d in range(3):
            p.period[d] = per[d]
            p.center[d] = center[d]
        p.periodic = int(period is not None) if periodic is None else int(periodic)
        p.nSmooth = int(nSmooth)
        p.device = int(device)
        self.params = p
        h = C.c_void_p()
        self._call("skid_create", C.byref(h), C.byref(p))
        self.h = h
        self.n = 0

    def _call(self, name, *args):
        rc = getattr(self.lib, name)(*args)
        if rc != 0:
            where = name
            if rc == -3 and getattr(self, "h", None):
                where += " [" + self.lib.skid_last_cuda_error(self.h).decode() + "]"
            raise SkidError(rc, where)
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.skid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- pipeline ----
    def set_particles(self, snap):
        self.n = snap.n
        self._pos = _c32(snap.pos, (-1, 3))
        self._vel = _c32(snap.vel, (-1, 3))
        self._mass = _c32(snap.mass)
        self._soft = _c32(snap.soft)
        self._temp = _c32(snap.temp)
        self._call("skid_set_particles", self.h, snap.n_gas, snap.n_dark, snap.n_star,
                   float(snap.time), _f(self._pos), _f(self._vel), _f(self._mass), _f(self._soft),
                   _f(self._temp))

    def restart(self):
        """Back to the freshly loaded state, particles kept on the device."""
        self._call("skid_restart", self.h)

    def set_option(self, name: str, value: float):
        self._call("skid_set_option", self.h, name.encode(), float(value))

    def get_option(self, name: str) -> float:
        v = C.c_double()
        self._call("skid_get_option", self.h, name.encode(), C.byref(v))
        return v.value

    def field_stats(self, enable=True):
        """Counts so far (nodes, leaves, tests, hits); then restart counting."""
        out = (C.c_ulonglong * 4)()
        self._call("skid_field_stats", self.h, int(enable), out)
        return tuple(int(x) for x in out)

    def stream_ptr(self) -> int:
        s = C.c_void_p()
        self._call("skid_stream", self.h, C.byref(s))
        return s.value or 0

    def scatter_active(self, bGasAndDark=False, bGasOnly=False) -> int:
        n = C.c_int()
        self._call("skid_scatter_active", self.h, int(bGasAndDark), int(bGasOnly), C.byref(n))
        return n.value

    def density(self) -> int:
        n = C.c_int()
        self._call("skid_density", self.h, C.byref(n))
        return n.value

    def get_density(self):
        rho = np.empty(self.n, np.float32)
        b = np.empty(self.n, np.float32)
        self._call("skid_get_density", self.h, _f(rho), _f(b))
        return rho, b

    def get_final_density(self):
        rho = np.empty(self.n, np.float32)
        self._call("skid_get_final_density", self.h, _f(rho))
        return rho

    def init_move(self, fDensMin=0.0, fTempMax=FLT_MAX, fMassMax=FLT_MAX, bGasAndDark=False,
                  bGasOnly=False) -> int:
        n = C.c_int()
        self._call("skid_init_move", self.h, fDensMin, fTempMax, fMassMax, int(bGasAndDark),
                   int(bGasOnly), C.byref(n))
        return n.value

    def move_step(self, fStep, bInitial=False, bNoCut=False) -> int:
        n = C.c_int()
        self._call("skid_move_step", self.h, fStep, int(bInitial), int(bNoCut), C.byref(n))
        return n.value

    def prune_inactive(self, fCvg) -> int:
        n = C.c_int()
        self._call("skid_prune_inactive", self.h, fCvg, C.byref(n))
        return n.value

    def move_iterate(self, fStep, fCvg, bNoCut=False):
        a, s = C.c_int(), C.c_int()
        self._call("skid_move_iterate", self.h, fStep, fCvg, int(bNoCut), C.byref(a), C.byref(s))
        return a.value, s.value

    def reactivate_move(self):
        self._call("skid_reactivate_move", self.h)

    def fof(self, fTau) -> int:
        n = C.c_int()
        self._call("skid_fof", self.h, fTau, C.byref(n))
        return n.value

    def group_centers(self):
        self._call("skid_group_centers", self.h)

    def set_groups(self, grp, centers=None):
        grp = np.ascontiguousarray(grp, np.int32)
        ng = int(grp.max(initial=0)) + 1
        cptr = None
        if centers is not None:
            centers = np.ascontiguousarray(centers, GROUP_DTYPE)
            cptr = centers.ctypes.data_as(C.c_void_p)
        self._call("skid_set_groups", self.h, _i(grp), ng, cptr)

    def set_soft(self, fEps):
        self._call("skid_set_soft", self.h, fEps)

    def unbind(self, iSoftType, fScoop, bGasAndDark, bNoUnbind, nMaxMembers, G, z, a, aH) -> int:
        n = C.c_int()
        self._call("skid_unbind", self.h, int(iSoftType), fScoop, int(bGasAndDark), int(bNoUnbind),
                   int(min(nMaxMembers, 2**31 - 1)), G, z, a, aH, C.byref(n))
        return n.value

    def too_small(self, nMembers) -> int:
        n = C.c_int()
        self._call("skid_too_small", self.h, int(nMembers), C.byref(n))
        return n.value

    def get_groups(self, ngroups: int):
        grp = np.empty(self.n, np.int32)
        rec = np.zeros(ngroups + 1, GROUP_DTYPE)
        self._call("skid_get_groups", self.h, _i(grp), rec.ctypes.data_as(C.c_void_p))
        return grp, rec

    def group_stats(self, ngroups: int, G, fExp, fExpHub, fDensMin, fTempMax):
        """kdOutStats' per-group columns (skid_stat records, index 0 unused)."""
        out = np.zeros(ngroups + 1, STAT_DTYPE)
        self._call("skid_group_stats", self.h, float(G), float(fExp), float(fExpHub),
                   float(fDensMin), float(fTempMax), out.ctypes.data_as(C.c_void_p))
        return out

    def get_moved(self):
        out = np.empty((self.n, 3), np.float32)
        self._call("skid_get_moved", self.h, _f(out))
        return out

    def timings(self) -> dict:
        t = Timings()
        self._call("skid_get_timings", self.h, C.byref(t))
        return {k: getattr(t, k) for k, _ in Timings._fields_}

    # ---- stage probes ----
    def knn_ball2(self, pos, k):
        pos = _c32(pos, (-1, 3))
        out = np.empty(len(pos), np.float32)
        self._call("skid_knn_ball2", self.h, len(pos), _f(pos), int(k), _f(out))
        return out

    def field(self, mpos):
        mpos = _c32(mpos, (-1, 3))
        acc = np.empty((len(mpos), 3), np.float32)
        self._call("skid_field", self.h, len(mpos), _f(mpos), _f(acc))
        return acc

    def density_adjoint(self, w, mode=ADJ_RECOMPUTE):
        """dL/dx (n, 3) by iOrder for L = sum_i w_i rho_i (after density())."""
        w = _c32(w)
        out = np.empty((len(w), 3), np.float32)
        self._call("skid_density_adjoint", self.h, _f(w), _f(out), int(mode))
        return out

    def field_adjoint(self, ypos, w):
        """w_i * grad rho_f(y_i), (nm, 3), over the live scatterer copies."""
        ypos = _c32(ypos, (-1, 3))
        w = _c32(w)
        out = np.empty((len(ypos), 3), np.float32)
        self._call("skid_field_adjoint", self.h, len(ypos), _f(ypos), _f(w), _f(out))
        return out

    def potential_adjoint(self, sel, v=None, G=1.0, soft_type=2, n=None):
        """Potential energies E[s] of groups sel (FP64) and, with v, the
        gradient of sum_s v[s] E[s] by iOrder (n, 3)."""
        sel = np.ascontiguousarray(sel, np.int32)
        E = np.zeros(len(sel), np.float64)
        grad = None
        vp = gp = None
        if v is not None:
            v = _c32(v)
            grad = np.empty((self.n if n is None else n, 3), np.float32)
            vp, gp = _f(v), _f(grad)
        self._call("skid_potential_adjoint", self.h, int(soft_type), G, len(sel), _i(sel), vp,
                   E.ctypes.data_as(_D), gp)
        return E, grad

    def fof_points(self, pos, tau):
        pos = _c32(pos, (-1, 3))
        grp = np.empty(len(pos), np.int32)
        ng = C.c_int()
        self._call("skid_fof_points", self.h, len(pos), _f(pos), tau, _i(grp), C.byref(ng))
        return grp, ng.value


def pair_factor(d2, twoh, plummer=False, mode=PAIR_USED):
    """The unbinding potentials' float pair factor for squared distances d2
    and summed softenings twoh, computed on the device (skid_pair_factor)."""
    lib = load()
    d2 = _c32(d2)
    twoh = _c32(twoh)
    if d2.shape != twoh.shape:
        raise ValueError("d2 and twoh differ in length")
    out = np.empty(len(d2), np.float32)
    rc = lib.skid_pair_factor(len(d2), _f(d2), _f(twoh), int(plummer), int(mode), _f(out))
    if rc:
        raise SkidError(rc, "skid_pair_factor")
    return out


def batch_run(volumes, opts, n_workers=8, device=0, group_cap=None):
    """Run many independent volumes in one skid_batch_run call.

    volumes: list of (snapshot, nSmooth, tau); opts: an Options holding the
    shared flags (its tau/nSmooth are ignored).  Returns one dict per volume
    with grp, groups (GROUP_DTYPE, index 0 = ungrouped), counts and status."""
    lib = load()
    nv = len(volumes)
    arr = (Volume * nv)()
    keep = []
    outs = []
    for i, (snap, k, tau) in enumerate(volumes):
        v = arr[i]
        pos = _c32(snap.pos, (-1, 3)); vel = _c32(snap.vel, (-1, 3))
        mass = _c32(snap.mass); soft = _c32(snap.soft); temp = _c32(snap.temp)
        grp = np.empty(snap.n, np.int32)
        cap = (snap.n + 1) if group_cap is None else group_cap
        groups = np.zeros(cap, GROUP_DTYPE)
        keep.extend([pos, vel, mass, soft, temp])
        v.nGas, v.nDark, v.nStar, v.time = snap.n_gas, snap.n_dark, snap.n_star, float(snap.time)
        v.pos, v.vel, v.mass = pos.ctypes.data, vel.ctypes.data, mass.ctypes.data
        v.soft, v.temp = soft.ctypes.data, temp.ctypes.data
        for d in range(3):
            v.period[d] = opts.period[d]
            v.center[d] = opts.center[d]
        v.periodic = int(opts.periodic)
        v.nSmooth = int(k)
        v.fTau = float(tau)
        v.fCvg = v.fScoop = 0.0
        v.grp, v.groups, v.groups_cap = grp.ctypes.data, groups.ctypes.data, cap
        outs.append((grp, groups))
    f = BatchFlags()
    f.fDensMin, f.fTempMax, f.fMassMax = opts.fDensMin, opts.fTempMax, opts.fMassMax
    f.nMembers, f.nMaxMembers = opts.nMembers, min(opts.nMaxMembers, 2**31 - 1)
    f.bGasAndDark, f.bGasOnly = int(opts.bGasAndDark), int(opts.bGasOnly)
    f.bForceInitialCut, f.bNoUnbind, f.bNoCut = (int(opts.bForceInitialCut), int(opts.bNoUnbind),
                                                 int(opts.bNoScatterCut))
    f.iSoftType, f.bEps, f.fEps = opts.iSoftType, int(opts.bEps), opts.fEps
    f.G, f.z, f.a, f.aH = opts.G, opts.z, opts.a_shift, opts.a_hubble
    f.maxIter = opts.maxIter
    rc = lib.skid_batch_run(C.addressof(arr), nv, C.addressof(f), int(n_workers), int(device))
    res = []
    for i, (grp, groups) in enumerate(outs):
        v = arr[i]
        res.append({"grp": grp, "groups": groups[:v.nGroup + 1], "nGroup": v.nGroup,
                    "nGroupFoF": v.nGroupFoF, "nUnbound": v.nUnbound, "nIter": v.nIter,
                    "device_ms": v.device_ms, "status": v.status,
                    "message": v.message.decode(errors="replace")})
    if rc:
        msgs = sorted({r["message"] for r in res if r["message"]})
        raise SkidError(rc, "skid_batch_run" + (f" [{'; '.join(msgs)}]" if msgs else ""))
    return res
