"""GPU parity of the scalar filters of the `buff` and `buff-slice-scalar`
profiler arms against the oracle: buff_range_filter / buff_equal_filter
(compress/buff_simd.rs:4507-4679, :4925-5094) on the buff layout, and
buff_slice_range_filter_nosimd / _equal_filter_nosimd / buff_slice_decode_bs
(compress/buff_slice.rs:1753-1991, :1184-1262).  Unlike the SIMD forms they
compare every row, including those after the last full 32-row block."""
import numpy as np
import pytest

from tests.test_gpu_parity import CASES, _pred_list, gen

pytestmark = pytest.mark.gpu


def _same(got, words, cnt):
    return got.count == cnt and np.array_equal(np.asarray(got.words, dtype=np.uint32), words)


@pytest.mark.parametrize("kind,n,scale", CASES)
def test_buff_layout_scalar_filters(oracle, gpu, kind, n, scale):
    from buff_gb300 import capi
    from buff_gb300.compress import FLAG_BUFF_LAYOUT, Column

    x = gen(kind, n, 31)
    try:
        img = oracle.encode(x, scale, flipped=False)
    except oracle.OraclePanic:
        with pytest.raises(capi.ReferencePanic):
            Column.encode(x, scale, FLAG_BUFF_LAYOUT)
        return
    col = Column.encode(x, scale, FLAG_BUFF_LAYOUT)
    assert col.serialize() == img
    back = Column.deserialize(img, scale, FLAG_BUFF_LAYOUT)
    for p in _pred_list(x):
        for c in (col, back):
            w, cnt, _ = oracle.scalar_range_filter(img, scale, p)
            assert _same(c.scalar_range_filter(p), w, cnt), ("range", p)
            w, cnt, _ = oracle.scalar_equal_filter(img, scale, p)
            assert _same(c.scalar_equal_filter(p), w, cnt), ("equal", p)


@pytest.mark.parametrize("n", [7, 31, 33, 1000, 65_537])
@pytest.mark.parametrize("scale,offset,step", [(10000, 3.0, 0.01), (100, -50.0, 0.3),
                                               (10, 0.0, 0.05), (1000000, 1e3, 1.0)])
def test_slice_nosimd_filters_and_decode_bs(oracle, gpu, n, scale, offset, step):
    from buff_gb300 import capi
    from buff_gb300.compress import SliceColumn

    rng = np.random.default_rng(n)
    dec = len(str(scale)) - 1
    x = np.round(offset + np.cumsum(rng.normal(0, step, n)), dec)
    img = oracle.slice_encode(x, scale)
    col = SliceColumn.encode(x, scale)
    assert col.serialize() == img
    xs = np.sort(x)
    for p in (float(x[n // 2]), float(np.quantile(x, 0.8)), float(xs[0]) - 1.0,
              float(xs[-1]) + 1.0, float(xs[-1]), float(x[0])):
        w, cnt, _ = oracle.slice_range_filter_nosimd(img, scale, p)
        assert _same(col.range_filter_nosimd(p), w, cnt), ("range", p)
        w, cnt, _ = oracle.slice_equal_filter_nosimd(img, scale, p)
        assert _same(col.equal_filter_nosimd(p), w, cnt), ("equal", p)
    try:
        want = oracle.slice_decode_bs(img, scale)
    except oracle.OraclePanic:
        with pytest.raises(capi.ReferencePanic):
            col.decode_bs()
    else:
        assert np.array_equal(col.decode_bs(), want)


def test_slice_scalar_panics(oracle, gpu):
    """Codes wider than 4 slices: decode_bs panics as the reference's
    `_ => panic!`; a constant column panics in the filters."""
    from buff_gb300 import capi
    from buff_gb300.compress import SliceColumn

    rng = np.random.default_rng(5)
    x = np.round(rng.uniform(-1e6, 1e6, 5000), 6)  # 41-bit codes: 6 slices
    img = oracle.slice_encode(x, 1000000)
    col = SliceColumn.encode(x, 1000000)
    with pytest.raises(oracle.OraclePanic):
        oracle.slice_decode_bs(img, 1000000)
    with pytest.raises(capi.ReferencePanic):
        col.decode_bs()
    p = float(x[10])
    w, cnt, _ = oracle.slice_range_filter_nosimd(img, 1000000, p)
    assert _same(col.range_filter_nosimd(p), w, cnt)
    const = SliceColumn.encode(np.full(100, 2.5), 10)
    with pytest.raises(oracle.OraclePanic):
        oracle.slice_range_filter_nosimd(oracle.slice_encode(np.full(100, 2.5), 10), 10, 3.0)
    with pytest.raises(capi.ReferencePanic):
        const.range_filter_nosimd(3.0)
