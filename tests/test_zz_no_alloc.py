"""mdft_get_delta_f_noalloc: the energy/gradient reduction for callers that
cannot allocate device memory during their solve (e.g. an application whose
pool allocator owns the whole GPU, or a loop that must not pay for an
allocation call).  Its scratch is a fixed array inside the library, so it
must give what mdft_get_delta_f gives, call after call, and draw nothing from
a stream-ordered memory pool: neither the device's default pool nor the
library's own (mdft_scratch_pool, the pool mdft_get_delta_f takes its
temporary from).

Collected last (file name) so that a run stopping at the first failure has
run every other test first.  Calls go straight through the C ABI."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_POINTS = 1 << 21  # 2,097,152 grid points (128^3): the fixed scratch limit

# CUmemPool_attribute value of CU_MEMPOOL_ATTR_USED_MEM_HIGH (cuda.h)
_USED_MEM_HIGH = 8


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _run(L, fn, xi, vexc, w, df, ff, prec, stream):
    no = w.numel()
    rc = fn(_ptr(xi), _ptr(vexc), _ptr(w), _ptr(df), _ptr(ff), xi.numel() // no, no,
            0.000424, -15.7, prec, stream)
    return rc


class _PoolWatermark:
    """High-water mark of a stream-ordered memory pool, read through the
    driver API: the current device's default pool (the one cudaMallocAsync
    draws from), or the given one."""

    def __init__(self, pool=None):
        self.cu = C.CDLL("libcuda.so.1")
        if pool is None:
            dev = C.c_int(0)
            assert self.cu.cuCtxGetDevice(C.byref(dev)) == 0
            pool = C.c_void_p(0)
            assert self.cu.cuDeviceGetMemPool(C.byref(pool), dev) == 0
        self.pool = pool

    def reset(self):
        zero = C.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, _USED_MEM_HIGH, C.byref(zero)) == 0

    def high(self):
        v = C.c_uint64(0)
        assert self.cu.cuMemPoolGetAttribute(self.pool, _USED_MEM_HIGH, C.byref(v)) == 0
        return v.value


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_noalloc_matches_allocating_entry_point_twice(gpu_lib, prec):
    """FP64 (0), FP32 (1) and double-float on FP64 fields (2): two calls in a
    row through the fixed scratch give the allocating call's df bit for bit
    and its ff; the high-water marks of the default pool and of the
    library's pool stay zero across them, and a positive control shows the
    allocating call does move the library pool's."""
    import torch
    L = gpu_lib.lib()
    dt = torch.float32 if prec == 1 else torch.float64
    rng = np.random.default_rng(2024)
    shape = (40, 40, 40, 84)
    xi = torch.from_numpy(rng.uniform(0.9, 1.1, shape)).to("cuda", dt)
    vexc = torch.from_numpy(rng.uniform(-1.0, 1.0, shape)).to("cuda", dt)
    w = torch.from_numpy(rng.uniform(0.0, 1.0, 84)).to("cuda", torch.float64)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    lp = C.c_void_p()
    assert L.mdft_scratch_pool(C.byref(lp)) == 0 and lp.value
    pools = (_PoolWatermark(), _PoolWatermark(lp))

    df_ref = torch.zeros_like(xi)
    ff_ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for pool in pools:
        pool.reset()
    assert _run(L, L.mdft_get_delta_f, xi, vexc, w, df_ref, ff_ref, prec, stream) == 0
    torch.cuda.synchronize()
    assert pools[1].high() > 0  # the allocating entry point draws its temporary from the library's pool

    for _ in range(2):  # two calls in a row share the fixed scratch
        df = torch.full_like(xi, 7.0)
        ff = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for pool in pools:
            pool.reset()
        assert _run(L, L.mdft_get_delta_f_noalloc, xi, vexc, w, df, ff, prec, stream) == 0, \
            L.mdft_last_error()
        torch.cuda.synchronize()
        assert all(pool.high() == 0 for pool in pools)
        assert torch.equal(df, df_ref)
        a, b = float(ff.item()), float(ff_ref.item())
        assert abs(a - b) <= 1e-12 * abs(b)


def test_noalloc_rejects_grids_beyond_the_limit(gpu_lib):
    import torch
    L = gpu_lib.lib()
    no = 1
    n = MAX_POINTS + 1
    xi = torch.ones(n, dtype=torch.float64, device="cuda")
    vexc = torch.ones(n, dtype=torch.float64, device="cuda")
    w = torch.ones(no, dtype=torch.float64, device="cuda")
    df = torch.zeros(n, dtype=torch.float64, device="cuda")
    ff = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.mdft_get_delta_f_noalloc(_ptr(xi), _ptr(vexc), _ptr(w), _ptr(df), _ptr(ff), n, no,
                                    0.3, 0.3, 0, stream)
    assert rc == 4
    assert b"fixed scratch limit" in L.mdft_last_error()
    # the largest accepted grid still runs
    rc = L.mdft_get_delta_f_noalloc(_ptr(xi), _ptr(vexc), _ptr(w), _ptr(df), _ptr(ff),
                                    MAX_POINTS, no, 0.3, 0.3, 0, stream)
    assert rc == 0, L.mdft_last_error()
    torch.cuda.synchronize()
    assert float(ff.item()) == 0.0  # xi = 1 -> xi^2 - 1 = 0
