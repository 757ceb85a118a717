"""simall_gpu_dot_noalloc: the dot product for callers that cannot allocate
device memory (see its declaration in include/simall_gpu.h).  It must give
the allocating simall_gpu_dot's result, call after call, without changing
the device's free memory once its one-time set-up has run.  Collected last so
that a failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 16777216  # SIMALL_DOT_NOALLOC_MAX_N


def _fn(L):
    f = L.simall_gpu_dot_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.POINTER(C.c_double)]
    return f


def test_noalloc_dot_matches_allocating_dot_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    import simall_gb300 as sg

    L = sg.load()
    noalloc = _fn(L)
    dev = torch.device("cuda:0")
    cases = [(1, 1_000_003), (2, 4096), (3, MAX_N)]
    for seed, n in cases:
        rng = np.random.default_rng(seed)
        xh = rng.standard_normal(n)
        yh = rng.standard_normal(n)
        x = torch.from_numpy(xh).to(dev)
        y = torch.from_numpy(yh).to(dev)
        torch.cuda.synchronize()
        got = C.c_double()
        ref = C.c_double()
        assert noalloc(x.data_ptr(), y.data_ptr(), n, None, C.byref(got)) == 0
        assert L.simall_gpu_dot(x.data_ptr(), y.data_ptr(), n, None, C.byref(ref)) == 0
        scale = float(np.abs(xh * yh).sum())
        assert abs(got.value - ref.value) <= 1e-12 * scale, (n, got.value, ref.value)
        # a second call on the same data agrees with the first bit for bit
        again = C.c_double()
        assert noalloc(x.data_ptr(), y.data_ptr(), n, None, C.byref(again)) == 0
        assert again.value == got.value


def test_noalloc_dot_keeps_device_memory_constant_and_rejects_oversize():
    torch = pytest.importorskip("torch")
    import simall_gb300 as sg

    L = sg.load()
    noalloc = _fn(L)
    dev = torch.device("cuda:0")
    x = torch.ones(1 << 20, dtype=torch.float64, device=dev)
    out = C.c_double()
    assert noalloc(x.data_ptr(), x.data_ptr(), x.numel(), None, C.byref(out)) == 0  # one-time set-up
    assert out.value == float(x.numel())
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert noalloc(x.data_ptr(), x.data_ptr(), x.numel(), None, C.byref(out)) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert noalloc(x.data_ptr(), x.data_ptr(), MAX_N + 1, None, C.byref(out)) == 8  # SIMALL_ERR_SIZE_MISMATCH
    assert noalloc(x.data_ptr(), x.data_ptr(), 0, None, C.byref(out)) == 0 and out.value == 0.0


def test_noalloc_dot_on_a_caller_stream():
    """The ticket reset, the kernel and the result copy all run on the stream
    the caller passes: a torch stream other than the default, one call at a
    time, with the operands written on that stream just before."""
    torch = pytest.importorskip("torch")
    import simall_gb300 as sg

    L = sg.load()
    noalloc = _fn(L)
    dev = torch.device("cuda:0")
    side = torch.cuda.Stream(device=dev)
    n = 3_000_017
    rng = np.random.default_rng(11)
    xh, yh = rng.standard_normal(n), rng.standard_normal(n)
    for k in range(3):
        with torch.cuda.stream(side):
            x = torch.from_numpy(xh * (k + 1)).to(dev, non_blocking=False)
            y = torch.from_numpy(yh).to(dev, non_blocking=False)
            x.mul_(0.5)  # queued on the side stream right before the call
        got = C.c_double()
        assert noalloc(x.data_ptr(), y.data_ptr(), n, C.c_void_p(side.cuda_stream), C.byref(got)) == 0
        side.synchronize()
        ref = C.c_double()
        assert L.simall_gpu_dot(x.data_ptr(), y.data_ptr(), n, None, C.byref(ref)) == 0
        scale = float(np.abs(0.5 * (k + 1) * xh * yh).sum())
        assert abs(got.value - ref.value) <= 1e-12 * scale, (k, got.value, ref.value)
