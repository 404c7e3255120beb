"""GPU parity of the buff-major (outlier) format against the oracle.

Columns with 0-3 sparse leading byte columns are encoded on the GPU and by the
oracle; with raw outlier bitmaps the byte images must be identical, with
snappy bitmaps both images must decode to the same column.  Every query
(decode, range/equal filter, sum, max) on the GPU column must equal the
oracle's answer on the reference image.
"""
import numpy as np
import pytest

from tests.test_oracle_major import major_case

pytestmark = pytest.mark.gpu

RAW = 1
SNAPPY = 0


def _preds(x):
    xs = np.sort(x)
    return [float(x[100]), float(np.quantile(x, 0.3)), float(np.quantile(x, 0.99)),
            float(xs[-2]), float(x.max()), float(x.max()) + 1, float(x.min()) - 1,
            float(x.min()), float(np.median(x)), float(x[7]) + 1e-9]


def _check_queries(oracle, col, ref, scale, mode, x):
    from buff_gb300 import capi

    n = x.size
    ncols, majors, nouts, _ = oracle.majority_layout(ref, mode)
    assert col.info.outlier_cols == ncols
    if all(nouts):
        assert np.array_equal(col.decode(), oracle.decode_majority(ref, scale, mode))
    else:
        with pytest.raises(capi.ReferencePanic):
            col.decode()
    for p in _preds(x):
        w, c, _ = oracle.range_filter_majority(ref, scale, p, mode)
        r = col.range_filter(p)
        assert np.array_equal(r.words, w), ("range", p)
        assert r.count == c
        w, c, _ = oracle.equal_filter_majority(ref, scale, p, mode)
        r = col.equal_filter(p)
        assert np.array_equal(r.words, w), ("equal", p)
        assert r.count == c
    s, parts = oracle.sum_majority(ref, scale, mode)
    res = col.sum()
    assert res.sum == s
    assert list(res.partials[: res.n_partials]) == parts[: res.n_partials]
    mv, mc, aw, ac = oracle.max_majority(ref, scale, mode)
    m = col.max(argmax=True)
    assert m.code == mc and m.value == mv
    assert np.array_equal(m.argmax_words, aw) and m.argmax_count == ac
    _check_async(col, s, parts[: res.n_partials], mc)
    assert n == col.n


def _check_async(col, s, parts, mc):
    """buff_sum_majority_async (the f64 sum and the partials combined on the
    device) and buff_max_majority_async into device memory."""
    import torch

    from buff_gb300 import capi

    L = capi.lib()
    dsum = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    dparts = torch.full((9,), -1, dtype=torch.int64, device="cuda")
    dmax = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    st = torch.cuda.Stream()
    assert L.buff_sum_majority_async(col.handle, dsum.data_ptr(), dparts.data_ptr(),
                                     st.cuda_stream) == capi.OK
    assert L.buff_sum_majority_async(col.handle, dsum.data_ptr(), None, st.cuda_stream) == capi.OK
    assert L.buff_max_majority_async(col.handle, dmax.data_ptr(), st.cuda_stream) == capi.OK
    st.synchronize()
    assert float(dsum.item()).hex() == float(s).hex()
    got = dparts.cpu().numpy().view(np.uint64)
    assert list(got[: len(parts)]) == list(parts)
    assert int(dmax.cpu().numpy().view(np.uint64)[0]) == mc
    # the value alone through the synchronous call (no arg-max requested)
    import ctypes as C

    mv, code = C.c_double(0), C.c_uint64(0)
    assert L.buff_max_majority(col.handle, C.byref(mv), C.byref(code), None, None,
                               None) == capi.OK
    assert code.value == mc


@pytest.mark.parametrize("kind", ["one", "two", "three", "none"])
@pytest.mark.parametrize("n", [4099, 300_001])
def test_major_raw_bitmaps_bit_exact(oracle, gpu, kind, n):
    from buff_gb300.compress import FLAG_RAW_BITMAPS, MajorColumn

    x, scale = major_case(kind, n, 11)
    ref = oracle.encode_majority(x, scale, RAW)
    col = MajorColumn.encode(x, scale, FLAG_RAW_BITMAPS)
    assert col.serialize() == ref
    _check_queries(oracle, col, ref, scale, RAW, x)
    back = MajorColumn.deserialize(ref, scale, FLAG_RAW_BITMAPS)
    assert back.serialize() == ref
    _check_queries(oracle, back, ref, scale, RAW, x)


@pytest.mark.parametrize("kind", ["one", "two", "three", "none"])
def test_major_snappy_bitmaps(oracle, gpu, kind):
    from buff_gb300.compress import MajorColumn

    x, scale = major_case(kind, 200_003, 12)
    ref = oracle.encode_majority(x, scale, SNAPPY)
    col = MajorColumn.encode(x, scale)
    img = col.serialize()
    # both snappy streams hold the same bitmaps: the decoded layouts agree
    assert oracle.majority_layout(img, SNAPPY) == oracle.majority_layout(ref, SNAPPY)
    nouts = oracle.majority_layout(ref, SNAPPY)[2]
    if all(nouts):
        assert np.array_equal(oracle.decode_majority(img, scale, SNAPPY),
                              oracle.decode_majority(ref, scale, SNAPPY))
    _check_queries(oracle, col, ref, scale, SNAPPY, x)
    back = MajorColumn.deserialize(ref, scale)
    _check_queries(oracle, back, ref, scale, SNAPPY, x)


def test_major_outlier_workload(oracle, gpu):
    """A 1% outlier column with 6 decimals: one sparse byte column."""
    from buff_gb300 import workloads
    from buff_gb300.compress import FLAG_RAW_BITMAPS, MajorColumn

    x = workloads.outlier_column(1_000_003, seed=4)
    ref = oracle.encode_majority(x, 1000000, RAW)
    col = MajorColumn.encode(x, 1000000, FLAG_RAW_BITMAPS)
    assert col.serialize() == ref
    _check_queries(oracle, col, ref, 1000000, RAW, x)


def test_major_dense_outlier_runs(oracle, gpu):
    """One sparse byte column (the first 2,000 rows vote) with 512-row
    chunks that are outliers in every row or in half of them: the decode
    reads those chunks' outlier bytes one by one instead of as one window."""
    from buff_gb300.compress import FLAG_RAW_BITMAPS, MajorColumn

    x, scale = major_case("one", 70_001, 13)
    rng = np.random.default_rng(14)
    pos = np.concatenate([np.arange(6_000, 10_100),
                          40_000 + np.nonzero(rng.uniform(size=30_001) < 0.5)[0]])
    x[pos] = np.round(rng.uniform(-1e4, 1e4, pos.size), 6)
    ref = oracle.encode_majority(x, scale, RAW)
    assert oracle.majority_layout(ref, RAW)[0] == 1
    col = MajorColumn.encode(x, scale, FLAG_RAW_BITMAPS)
    assert col.serialize() == ref
    _check_queries(oracle, col, ref, scale, RAW, x)


@pytest.mark.parametrize("vmax,scale", [(5, 10), (10, 10), (3, 100), (5, 100), (10, 100),
                                        (3, 1000), (5, 1000), (10, 1000)])
def test_major_sparse_byte_only(oracle, gpu, vmax, scale):
    """Columns whose code is one sparse byte and 0-7 tail bits (fixed_len
    8-15, no dense slice): 90 % of the rows hold one value, the rest are
    uniform.  Every query against the oracle."""
    from buff_gb300.compress import FLAG_RAW_BITMAPS, MajorColumn

    rng = np.random.default_rng(vmax * 7 + scale)
    n = 50_003
    dec = {10: 1, 100: 2, 1000: 3}[scale]
    x = np.where(rng.uniform(size=n) < 0.9, vmax * 0.7,
                 np.round(rng.uniform(0, vmax, n), dec))
    ref = oracle.encode_majority(x, scale, RAW)
    fl = oracle.header(ref).fixed_len
    assert 8 <= fl < 16 and oracle.majority_layout(ref, RAW)[0] == 1
    col = MajorColumn.encode(x, scale, FLAG_RAW_BITMAPS)
    assert col.serialize() == ref
    _check_queries(oracle, col, ref, scale, RAW, x)
    for p in (vmax * 0.7, vmax * 0.7 + 10.0 ** -dec, vmax * 0.35, 0.0):
        w, c, _ = oracle.range_filter_majority(ref, scale, p, RAW)
        r = col.range_filter(p)
        assert np.array_equal(r.words, w) and r.count == c, ("range", p)
        w, c, _ = oracle.equal_filter_majority(ref, scale, p, RAW)
        r = col.equal_filter(p)
        assert np.array_equal(r.words, w) and r.count == c, ("equal", p)


def test_major_f32_and_device_input(oracle, gpu):
    import torch

    from buff_gb300.compress import FLAG_RAW_BITMAPS, MajorColumn

    x, scale = major_case("two", 50_001, 13)
    x32 = x.astype(np.float32)
    ref = oracle.encode_majority(x32.astype(np.float64), scale, RAW)
    assert MajorColumn.encode(x32, scale, FLAG_RAW_BITMAPS).serialize() == ref
    dev = torch.from_numpy(x).cuda()
    ref64 = oracle.encode_majority(x, scale, RAW)
    col = MajorColumn.encode(dev, scale, FLAG_RAW_BITMAPS)
    assert col.serialize() == ref64
    out = torch.empty(x.size, dtype=torch.float64, device="cuda")
    nouts = oracle.majority_layout(ref64, RAW)[2]
    if all(nouts):
        col.decode(out=out)
        assert np.array_equal(out.cpu().numpy(), oracle.decode_majority(ref64, scale, RAW))


def test_major_errors(gpu):
    from buff_gb300 import capi
    from buff_gb300.compress import FLAG_INTENDED, Column, MajorColumn

    with pytest.raises(capi.ReferencePanic):  # fewer rows than the 2000-row sample
        MajorColumn.encode(np.arange(1999.0), 100)
    with pytest.raises(capi.BuffError) as e:
        MajorColumn.encode(np.arange(5000.0), 100, FLAG_INTENDED)
    assert e.value.status == capi.ENOTSUP
    x, scale = major_case("one", 5000, 3)
    col = MajorColumn.encode(x, scale)
    for fn in (lambda: Column.decode(col), lambda: Column.range_filter(col, 1.0),
               lambda: Column.sum(col), lambda: Column.max(col)):
        with pytest.raises(capi.BuffError) as e:
            fn()
        assert e.value.status == capi.ENOTSUP
    plain = Column.encode(x, scale)
    with pytest.raises(capi.BuffError) as e:
        MajorColumn.sum(plain)
    assert e.value.status == capi.ENOTSUP
    ref = col.serialize()
    with pytest.raises(capi.BuffError) as e:  # truncated image
        MajorColumn.deserialize(ref[: len(ref) // 2], scale)
    assert e.value.status == capi.ECORRUPT
