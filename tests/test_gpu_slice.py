"""GPU parity of the buff-slice layout (compress/buff_slice.rs) against the
oracle: the byte image both ways, decode, the filters, sums and maxima."""
import numpy as np
import pytest

from tests.test_oracle_cond import cond_cases

pytestmark = pytest.mark.gpu


def _cases():
    rng = np.random.default_rng(31)
    big = np.round(np.cumsum(rng.uniform(-0.5, 0.5, 2_000_003)) + 100, 4)
    wide = np.round(rng.normal(0, 1e4, 100_000), 5)        # 5 slices: the *_sum/max panic
    const = np.full(4096, 2.5)
    dec = np.round(np.linspace(100, 0, 4001), 2)            # strictly decreasing: width 0
    f32 = np.round(rng.normal(10, 3, 70_001), 2).astype(np.float32)
    return cond_cases() + [("big", big, 10000), ("wide", wide, 100000), ("const", const, 100),
                           ("decreasing", dec, 100), ("f32", f32, 100)]


CASES = _cases()


@pytest.mark.parametrize("case", range(len(CASES)))
def test_slice_layout(oracle, gpu, case):
    from buff_gb300 import capi
    from buff_gb300.compress import SliceColumn

    name, x, scale = CASES[case]
    xd = x.astype(np.float64)
    img = oracle.slice_encode(xd, scale)
    col = SliceColumn.encode(x, scale)
    assert col.serialize() == img, name
    back = SliceColumn.deserialize(img, scale)
    assert back.serialize() == img
    ref_vals = oracle.slice_decode(img, scale)
    assert np.array_equal(col.decode(), ref_vals)
    n = xd.size
    preds = [float(np.quantile(xd, q)) for q in (0.1, 0.5, 0.9)] + \
        [float(xd[5]), float(xd.min()) - 1, float(xd.max()) + 2]
    for p in preds:
        for fn, ofn in ((col.range_filter, oracle.slice_range_filter),
                        (col.equal_filter, oracle.slice_equal_filter)):
            try:
                w, c, _ = ofn(img, scale, p)
            except oracle.OraclePanic:
                with pytest.raises(capi.ReferencePanic):
                    fn(p)
                continue
            r = fn(p)
            assert np.array_equal(r.words, w) and r.count == c, (name, p)
    for any_width in (False, True):
        try:
            s = oracle.slice_sum(img, scale, any_width)
        except oracle.OraclePanic:
            with pytest.raises(capi.ReferencePanic):
                col.slice_sum(any_width)
        else:
            assert col.slice_sum(any_width) == s, (name, any_width)
        try:
            mv, mw, mc = oracle.slice_max(img, scale, any_width)
        except oracle.OraclePanic:
            with pytest.raises(capi.ReferencePanic):
                col.slice_max(any_width)
        else:
            m = col.slice_max(any_width)
            assert m.value == mv and np.array_equal(m.argmax_words, mw) and m.argmax_count == mc
    del n


def test_slice_rejects_other_calls(gpu):
    from buff_gb300 import capi
    from buff_gb300.compress import Column, SliceColumn

    x = np.round(np.cumsum(np.random.default_rng(3).normal(0, 1, 10_000)), 2)
    col = SliceColumn.encode(x, 100)
    for fn in (lambda: Column.decode(col), lambda: Column.range_filter(col, 1.0),
               lambda: Column.sum(col)):
        with pytest.raises(capi.BuffError) as e:
            fn()
        assert e.value.status == capi.ENOTSUP
    plain = Column.encode(x, 100)
    with pytest.raises(capi.BuffError):
        SliceColumn.decode(plain)


@pytest.mark.parametrize("case", range(len(CASES)))
def test_slice_max_range(oracle, gpu, case):
    from buff_gb300 import capi
    from buff_gb300.compress import SliceColumn

    name, x, scale = CASES[case]
    xd = x.astype(np.float64)
    img = oracle.slice_encode(xd, scale)
    col = SliceColumn.encode(x, scale)
    n = xd.size
    windows = [(0, 1000, 100), (13, 13 + 128 * 7, 128), (5, 8, 3), (0, n, 1), (31, 231, 200),
               (0, n // 3, 7), (0, n // 1000 * 1000, 1000), (n - 50, n + 50, 100),
               (n - 50, n + 150, 100), (n + 5, n + 105, 100), (10, 5, 3), (0, 100, 0),
               (7, 7 + 3 * 64 + 1, 64), (12345, 12345 + 97 * 333, 333)]
    for s, e, w in windows:
        if s > n and e <= n:
            continue
        try:
            exp = oracle.slice_max_range(img, scale, s, e, w)
        except oracle.OraclePanic:
            with pytest.raises(capi.ReferencePanic):
                col.max_range(s, e, w)
            continue
        assert np.array_equal(col.max_range(s, e, w), exp), (name, s, e, w)
    if n > 4096:  # device output
        import torch

        out = torch.empty(n // 1000 + 1, dtype=torch.float64, device="cuda")
        e = n // 1000 * 1000
        try:
            exp = oracle.slice_max_range(img, scale, 0, e, 1000)
        except oracle.OraclePanic:
            return
        _, k = col.max_range(0, e, 1000, out=out)
        assert k == exp.size and np.array_equal(out.cpu().numpy()[:k], exp)
