"""libskidgpu loads here (no GPU needed) and exports every entry point that
include/skid_gpu.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    with open(os.path.join(ROOT, "include", "skid_gpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(skid_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared()
    assert "skid_create" in names and "skid_unbind" in names and len(names) >= 25


def test_library_exports_every_declared_symbol():
    from skid_gb300 import build
    lib = build.build_lib()
    h = ctypes.CDLL(lib)
    missing = [n for n in declared() if not hasattr(h, n)]
    assert not missing, missing


def test_no_device_is_an_error_not_a_crash():
    from skid_gb300 import gpu
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(gpu.SkidError) as e:
        gpu.Context(period=1.0, nSmooth=32)
    assert e.value.code == -6


def test_bad_parameters_are_refused_before_any_device_work():
    """A smoothing count below 1 or a period that is not positive (NaN
    included) is SKID_EINVAL from skid_create, checked before the device is
    looked at, here or on a GPU host."""
    from skid_gb300 import gpu
    lib = gpu.load()
    for period, k in (((1.0, 1.0, 1.0), 0), ((0.0, 0.0, 0.0), 32), ((1.0, -1.0, 1.0), 32),
                      ((float("nan"),) * 3, 32)):
        p = gpu.Params()
        for d in range(3):
            p.period[d] = period[d]
        p.periodic = 1
        p.nSmooth = k
        h = ctypes.c_void_p()
        assert lib.skid_create(ctypes.byref(h), ctypes.byref(p)) == -1, (period, k)
        assert not h.value
