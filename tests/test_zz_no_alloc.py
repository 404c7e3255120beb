"""The allocation-free range filter (buff_range_filter_noalloc) against the
regular buff_range_filter.

It serves callers that must not allocate device memory while answering a
query (a server whose HBM budget is fully reserved for resident columns, or a
process whose device memory belongs to another allocator).  Its bitmap and
count are staged in a fixed scratch array inside the library, so two calls in
a row must not see each other's results.  This file sorts last so that a run
stopping at its first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(col, pred):
    from buff_gb300 import capi

    n = col.n
    words = np.full(max((n + 31) // 32, 1), 0xDEADBEEF, dtype=np.uint32)
    cnt = np.zeros(1, dtype=np.uint64)
    st = capi.lib().buff_range_filter_noalloc(col.handle, float(pred), words.ctypes.data,
                                              cnt.ctypes.data, None)
    return st, words[: (n + 31) // 32], int(cnt[0])


def test_noalloc_matches_range_filter_twice(gpu):
    from buff_gb300 import Column, capi
    from buff_gb300.workloads import gaussian_walk

    x = gaussian_walk(1_000_003, seed=21)
    col = Column.encode(x, 10000)
    # two calls in a row with different predicates: the shared scratch must
    # hold only the current call's result
    for q in (0.9, 0.2):
        pred = float(np.quantile(x, q))
        want = col.range_filter(pred)
        st, words, cnt = _noalloc(col, pred)
        assert st == capi.OK
        assert np.array_equal(words, np.asarray(want.words, dtype=np.uint32))
        assert cnt == want.count
    # predicate below the column minimum: every row, as buff_range_filter
    pred = float(x.min()) - 1.0
    st, words, cnt = _noalloc(col, pred)
    assert st == capi.OK and cnt == x.size
    assert np.array_equal(words, np.asarray(col.range_filter(pred).words, dtype=np.uint32))


def test_noalloc_rejects_columns_above_its_scratch(gpu):
    import torch

    from buff_gb300 import Column, capi

    n = capi.NOALLOC_MAX_ROWS + 1
    x = torch.arange(n, dtype=torch.float64, device="cuda") * 0.001
    col = Column.encode(x, 1000)
    st, _, _ = _noalloc(col, 1.0)
    assert st == capi.ESCRATCH
    assert b"scratch" in capi.lib().buff_status_string(st)
