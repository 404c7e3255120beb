"""The allocation-free range filter (buff_range_filter_noalloc) against the
regular buff_range_filter.

It serves callers that must not allocate device memory while answering a
query (a server whose HBM budget is fully reserved for resident columns, or a
process whose device memory belongs to another allocator).  Its bitmap and
count are staged in a fixed scratch array inside the library, so two calls in
a row must not see each other's results, and a call must leave the device's
memory where it found it.  This file sorts last so that a run stopping at its
first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(col, pred, device_out=False):
    """Calls the entry point with host (numpy) or device (torch) outputs."""
    import torch

    from buff_gb300 import capi

    n = col.n
    nw = (n + 31) // 32
    if device_out:
        words = torch.full((max(nw, 1),), -559038737, dtype=torch.int32, device="cuda")
        cnt = torch.full((1,), 12345, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        st = capi.lib().buff_range_filter_noalloc(col.handle, float(pred), words.data_ptr(),
                                                  cnt.data_ptr(), None)
        return st, words.cpu().numpy().view(np.uint32)[:nw], int(cnt.cpu()[0])
    words = np.full(max(nw, 1), 0xDEADBEEF, dtype=np.uint32)
    cnt = np.full(1, 12345, dtype=np.uint64)
    st = capi.lib().buff_range_filter_noalloc(col.handle, float(pred), words.ctypes.data,
                                              cnt.ctypes.data, None)
    return st, words[:nw], int(cnt[0])


def _check_same(col, pred, device_out):
    from buff_gb300 import capi

    want = col.range_filter(pred)
    st, words, cnt = _noalloc(col, pred, device_out)
    assert st == capi.OK
    assert np.array_equal(words, np.asarray(want.words, dtype=np.uint32))
    assert cnt == want.count


@pytest.mark.parametrize("device_out", [False, True], ids=["host_out", "device_out"])
def test_noalloc_matches_range_filter_twice(gpu, device_out):
    from buff_gb300 import Column
    from buff_gb300.workloads import gaussian_walk

    x = gaussian_walk(1_000_003, seed=21)
    col = Column.encode(x, 10000)
    # two calls in a row with different predicates: the shared scratch must
    # hold only the current call's result
    for q in (0.9, 0.2):
        _check_same(col, float(np.quantile(x, q)), device_out)
    # predicate below the column minimum: every row, as buff_range_filter
    _check_same(col, float(x.min()) - 1.0, device_out)


@pytest.mark.parametrize("device_out", [False, True], ids=["host_out", "device_out"])
def test_noalloc_narrow_intended_and_empty_columns(gpu, device_out):
    from buff_gb300 import Column, capi

    rng = np.random.default_rng(22)
    # codes narrower than a byte: the full compare of every row
    narrow = np.round(rng.uniform(0.0, 3.0, 40_001), 1)
    col = Column.encode(narrow, 10)
    assert col.info.fixed_len < 8
    for pred in (1.05, 2.95, -1.0, 7.0):
        _check_same(col, pred, device_out)
    # intended semantics: rows after the last full 32-row block are set too
    x = np.round(np.cumsum(rng.normal(0, 0.01, 70_017)) + 3.0, 4)
    icol = Column.encode(x, 10000, capi.FLAG_INTENDED)
    for pred in (float(np.quantile(x, 0.5)), float(x.max()) + 5.0):
        _check_same(icol, pred, device_out)
    # an empty column answers 0 rows into host or device counts alike
    ecol = Column.encode(np.zeros(0), 10000)
    st, _, cnt = _noalloc(ecol, 1.0, device_out)
    assert st == capi.OK and cnt == 0


def _driver():
    import torch

    cu = C.CDLL("libcuda.so.1")
    dev = C.c_int(0)
    assert cu.cuDeviceGet(C.byref(dev), torch.cuda.current_device()) == 0
    pool = C.c_void_p()
    assert cu.cuDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    return cu, pool


def _pool_attr(cu, pool, attr):
    v = C.c_uint64(0)
    assert cu.cuMemPoolGetAttribute(pool, attr, C.byref(v)) == 0
    return v.value


def test_noalloc_allocates_nothing(gpu):
    """After a warm-up call (which loads the library's scratch on this device),
    a call moves neither the high watermark of the device's stream-ordered pool
    (which the other entry points allocate from) nor the device's free memory."""
    import torch

    from buff_gb300 import Column, capi
    from buff_gb300.workloads import gaussian_walk

    used_current, used_high = 7, 8  # CU_MEMPOOL_ATTR_USED_MEM_CURRENT / _HIGH
    x = gaussian_walk(500_000, seed=23)
    col = Column.encode(x, 10000)
    pred = float(np.quantile(x, 0.5))
    words = np.zeros((x.size + 31) // 32, dtype=np.uint32)
    cnt = np.zeros(1, dtype=np.uint64)
    lib = capi.lib()
    assert lib.buff_range_filter_noalloc(col.handle, pred, words.ctypes.data, cnt.ctypes.data,
                                         None) == capi.OK
    torch.cuda.synchronize()
    cu, pool = _driver()
    zero = C.c_uint64(0)
    assert cu.cuMemPoolSetAttribute(pool, used_high, C.byref(zero)) == 0
    before = _pool_attr(cu, pool, used_current)
    free0, total = C.c_size_t(0), C.c_size_t(0)
    assert cu.cuMemGetInfo_v2(C.byref(free0), C.byref(total)) == 0
    for q in (0.1, 0.9):
        assert lib.buff_range_filter_noalloc(col.handle, float(np.quantile(x, q)),
                                             words.ctypes.data, cnt.ctypes.data, None) == capi.OK
    free1 = C.c_size_t(0)
    assert cu.cuMemGetInfo_v2(C.byref(free1), C.byref(total)) == 0
    assert _pool_attr(cu, pool, used_high) == before
    assert free1.value == free0.value
    assert int(cnt[0]) == col.range_filter(float(np.quantile(x, 0.9))).count


def test_noalloc_rejects_columns_above_its_scratch(gpu):
    import torch

    from buff_gb300 import Column, capi

    n = capi.NOALLOC_MAX_ROWS + 1
    x = torch.arange(n, dtype=torch.float64, device="cuda") * 0.001
    col = Column.encode(x, 1000)
    st, _, _ = _noalloc(col, 1.0)
    assert st == capi.ESCRATCH
    assert b"scratch" in capi.lib().buff_status_string(st)
