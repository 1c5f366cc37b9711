"""skid_knn_ball2_noalloc, the allocation-free entry point, against the
context-based skid_knn_ball2.

The allocation-free form exists for callers that cannot allocate device
memory themselves -- a framework that owns the device allocator, or a loop
that cannot afford cudaMalloc's implicit synchronisation -- so this test
hands it device buffers it allocated elsewhere (torch) and checks the
results against the ordinary entry point on two calls in a row (the second
reuses the static scratch the first one left behind).  fBall2 is compared
exactly, the tolerance every fBall2 test here uses.  It also checks the
promise itself: after a first call on the device, a further call on a side
stream leaves the device's free memory unchanged.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLT_MAX = float(np.finfo(np.float32).max)
EINVAL = -1
ETOOLARGE = -8
MAX_POINTS = 65536
MAX_K = 256


def _entry():
    from skid_gb300 import build
    lib = C.CDLL(build.build_lib())
    fn = lib.skid_knn_ball2_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def _points(rng, n):
    pos = rng.uniform(-0.5, 0.5, (n, 3)).astype(np.float32)
    pos[: n // 4] *= np.float32(0.05)   # a dense clump among a uniform background
    return pos


def test_noalloc_matches_context_entry_point_on_two_calls(gpu_ready):
    torch = pytest.importorskip("torch")
    from skid_gb300 import gpu
    fn = _entry()
    rng = np.random.default_rng(2024)
    for n, k, period in [(20000, 64, 1.0), (30000, 32, None)]:
        pos = _points(rng, n)
        with gpu.Context(period=period, nSmooth=k) as ctx:
            want = ctx.knn_ball2(pos, k)
        d_pos = torch.from_numpy(pos.reshape(-1)).cuda()
        d_out = torch.full((n,), -1.0, dtype=torch.float32, device="cuda")
        per = (C.c_float * 3)(*([period] * 3 if period is not None else [FLT_MAX] * 3))
        torch.cuda.synchronize()
        rc = fn(d_pos.data_ptr(), n, k, per, d_out.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} of {n} differ"


def test_noalloc_refuses_sizes_beyond_its_scratch(gpu_ready):
    torch = pytest.importorskip("torch")
    fn = _entry()
    per = (C.c_float * 3)(1.0, 1.0, 1.0)
    big = torch.zeros(3 * (MAX_POINTS + 1), dtype=torch.float32, device="cuda")
    out = torch.zeros(MAX_POINTS + 1, dtype=torch.float32, device="cuda")
    assert fn(big.data_ptr(), MAX_POINTS + 1, 16, per, out.data_ptr(), None) == ETOOLARGE
    assert fn(big.data_ptr(), 1000, MAX_K + 1, per, out.data_ptr(), None) == ETOOLARGE
    torch.cuda.synchronize()


def test_noalloc_allocates_nothing_on_a_side_stream(gpu_ready):
    torch = pytest.importorskip("torch")
    from skid_gb300 import gpu
    fn = _entry()
    rng = np.random.default_rng(77)
    n, k = 40000, 48
    pos = _points(rng, n)
    with gpu.Context(period=1.0, nSmooth=k) as ctx:
        want = ctx.knn_ball2(pos, k)
    d_pos = torch.from_numpy(pos.reshape(-1)).cuda()
    d_out = torch.full((n,), -1.0, dtype=torch.float32, device="cuda")
    per = (C.c_float * 3)(1.0, 1.0, 1.0)
    side = torch.cuda.Stream()
    assert fn(d_pos.data_ptr(), n, k, per, d_out.data_ptr(), side.cuda_stream) == 0
    side.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    d_out.fill_(-1.0)
    torch.cuda.synchronize()
    assert fn(d_pos.data_ptr(), n, k, per, d_out.data_ptr(), side.cuda_stream) == 0
    side.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
    assert np.array_equal(d_out.cpu().numpy(), want)


def test_noalloc_rejects_bad_k(gpu_ready):
    torch = pytest.importorskip("torch")
    fn = _entry()
    per = (C.c_float * 3)(1.0, 1.0, 1.0)
    pts = torch.zeros(3 * 100, dtype=torch.float32, device="cuda")
    out = torch.zeros(100, dtype=torch.float32, device="cuda")
    assert fn(pts.data_ptr(), 100, 0, per, out.data_ptr(), None) == EINVAL
    assert fn(pts.data_ptr(), 100, 101, per, out.data_ptr(), None) == EINVAL
    assert fn(pts.data_ptr(), -1, 8, per, out.data_ptr(), None) == EINVAL
