"""GPU parity of the row-conditioned reads against the oracle:
buff_decode_condition, buff_range_filter_condition, their buff-major forms,
the bitmap-driven decode and the fused filter->decode call, plus the buff
layout image (byte_fixed_encode) both ways."""
import numpy as np
import pytest

from tests.test_oracle_cond import cond_cases
from tests.test_oracle_major import major_case

pytestmark = pytest.mark.gpu


def _rows(rng, n, frac):
    return np.sort(rng.choice(n, max(1, int(n * frac)), replace=False)).astype(np.uint32)


def _rows_of(words, n):
    bits = np.unpackbits(np.asarray(words, dtype="<u4").view(np.uint8), bitorder="little")[:n]
    return np.nonzero(bits)[0].astype(np.uint32)


def _big_case():
    rng = np.random.default_rng(77)
    x = np.round(np.cumsum(rng.normal(0, 0.01, 1_000_003)) + 3, 4)
    return ("walk_big", x, 10000)


CASES = cond_cases() + [_big_case()]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_buff_layout_image_both_ways(oracle, gpu, case):
    from buff_gb300.compress import FLAG_BUFF_LAYOUT, Column

    _, x, scale = CASES[case]
    img = oracle.encode(x, scale, flipped=False)
    col = Column.encode(x, scale, FLAG_BUFF_LAYOUT)
    assert col.serialize() == img
    back = Column.deserialize(img, scale, FLAG_BUFF_LAYOUT)
    assert back.serialize() == img
    assert np.array_equal(back.decode(), oracle.decode(img, scale, flipped=False))


@pytest.mark.parametrize("case", range(len(CASES)))
def test_decode_condition(oracle, gpu, case):
    import torch

    from buff_gb300 import capi
    from buff_gb300.compress import Column

    name, x, scale = CASES[case]
    img = oracle.encode(x, scale, flipped=False)
    col = Column.encode(x, scale)
    rng = np.random.default_rng(case)
    for frac in (0.0001, 0.01, 0.5, 1.0):
        rows = _rows(rng, x.size, frac)
        exp = oracle.decode_condition(img, scale, rows.astype(np.uint64))
        assert np.array_equal(col.decode_condition(rows), exp), (name, frac)
        drows = torch.from_numpy(rows.view(np.int32)).cuda()
        dout = torch.empty(rows.size, dtype=torch.float64, device="cuda")
        col.decode_condition(drows, out=dout)
        assert np.array_equal(dout.cpu().numpy(), exp), (name, frac, "device")
        words = np.zeros((x.size + 31) // 32, dtype=np.uint32)
        np.bitwise_or.at(words, rows // 32, (np.uint32(1) << (rows % 32)).astype(np.uint32))
        assert np.array_equal(col.decode_selected(words), exp), (name, frac, "bitmap")
    with pytest.raises(capi.ReferencePanic):
        col.decode_condition(np.zeros(0, dtype=np.uint32))
    for bad in ([5, 3], [1, 1], [x.size]):
        with pytest.raises(capi.BuffError) as e:
            col.decode_condition(np.array(bad, dtype=np.uint32))
        assert e.value.status == capi.EINVAL
    assert col.decode_selected(np.zeros((x.size + 31) // 32, dtype=np.uint32)).size == 0


@pytest.mark.parametrize("case", range(len(CASES)))
def test_range_filter_condition(oracle, gpu, case):
    from buff_gb300.compress import Column

    name, x, scale = CASES[case]
    img = oracle.encode(x, scale, flipped=False)
    col = Column.encode(x, scale)
    rng = np.random.default_rng(50 + case)
    preds = [float(np.quantile(x, q)) for q in (0.05, 0.5, 0.95)] + \
        [float(x.min()) - 1, float(x.max()) + 5, float(x[3]), float(x.max())]
    for frac in (0.001, 0.2, 1.0):
        rows = _rows(rng, x.size, frac)
        for p in preds:
            w, c = oracle.range_filter_condition(img, scale, p, rows.astype(np.uint64))
            r = col.range_filter_condition(p, rows)
            assert np.array_equal(r.words, w), (name, frac, p)
            assert r.count == c


@pytest.mark.parametrize("case", range(len(CASES)))
def test_range_filter_decode(oracle, gpu, case):
    from buff_gb300.compress import Column

    name, x, scale = CASES[case]
    img = oracle.encode(x, scale, flipped=False)
    col = Column.encode(x, scale)
    for q in (0.5, 0.99, 0.999):
        p = float(np.quantile(x, q))
        res, vals = col.range_filter_decode(p)
        plain = col.range_filter(p)
        assert np.array_equal(res.words, plain.words) and res.count == plain.count
        rows = _rows_of(plain.words, x.size)
        if rows.size:
            exp = oracle.decode_condition(img, scale, rows.astype(np.uint64))
            assert np.array_equal(vals, exp), (name, q)
        else:
            assert vals.size == 0


@pytest.mark.parametrize("case", range(4))
def test_decode_condition_intended(oracle, gpu, case):
    from buff_gb300.compress import FLAG_INTENDED, Column

    _, x, scale = CASES[case]
    col = Column.encode(x, scale, FLAG_INTENDED)
    full = col.decode()
    rows = _rows(np.random.default_rng(9), x.size, 0.1)
    assert np.array_equal(col.decode_condition(rows), full[rows])
    assert col.decode_condition(np.zeros(0, dtype=np.uint32)).size == 0


@pytest.mark.parametrize("kind", ["one", "two", "none"])
def test_major_condition(oracle, gpu, kind):
    from buff_gb300.compress import FLAG_RAW_BITMAPS, MajorColumn

    x, scale = major_case(kind, 20_011, 17)
    img = oracle.encode_majority(x, scale, 1)
    col = MajorColumn.deserialize(img, scale, FLAG_RAW_BITMAPS)
    rows = _rows(np.random.default_rng(4), x.size, 0.03)
    exp = oracle.major_decode_condition(img, scale, rows.astype(np.uint64))
    got = col.decode_condition(rows)
    assert got.size == exp.size and np.array_equal(got, exp)
    for q in (0.2, 0.7):
        p = float(np.quantile(x, q))
        w, c = oracle.range_filter_majority_condition(img, scale, p, rows.astype(np.uint64))
        r = col.range_filter_condition(p, rows)
        assert np.array_equal(r.words, w) and r.count == c


@pytest.mark.parametrize("case", range(len(CASES)))
def test_max_range(oracle, gpu, case):
    from buff_gb300 import capi
    from buff_gb300.compress import FLAG_INTENDED, Column

    name, x, scale = CASES[case]
    img = oracle.encode(x, scale, flipped=False)
    col = Column.encode(x, scale)
    n = x.size
    fl = oracle.header(img).fixed_len
    for s, w in ((0, 1000), (13, 128), (5, 3), (0, 1), (100, 4096), (0, n // 3), (31, 200),
                 (0, 1024), (7, 1500), (1000, 5000), (33, 2048)):
        if w == 0 or s + w > n:
            continue
        e = s + (n - s) // w * w
        exp = oracle.max_range(img, scale, s, e, w)
        got = col.max_range(s, e, w)
        assert np.array_equal(got, exp), (name, s, e, w)
    e = min(n, 1000 + 37)
    if fl > 8:
        with pytest.raises(capi.ReferencePanic):
            col.max_range(0, e, 100)
    else:
        assert np.array_equal(col.max_range(0, e, 100), oracle.max_range(img, scale, 0, e, 100))
    with pytest.raises(capi.ReferencePanic):
        col.max_range(0, n + 1, 10)
    ci = Column.encode(x, scale, FLAG_INTENDED)
    full = ci.decode()
    got = ci.max_range(3, e, 100)
    exp = np.array([full[a:min(a + 100, e)].max() for a in range(3, e, 100)])
    assert np.array_equal(got, exp)
    if n > 4000:  # windows of >= 1,024 rows, the last one ragged
        e2 = n - 17
        got = ci.max_range(5, e2, 1700)
        exp = np.array([full[a:min(a + 1700, e2)].max() for a in range(5, e2, 1700)])
        assert np.array_equal(got, exp)


@pytest.mark.parametrize("kind", ["none", "one"])
def test_max_majority_range(oracle, gpu, kind):
    from buff_gb300 import capi
    from buff_gb300.compress import FLAG_RAW_BITMAPS, MajorColumn

    x, scale = major_case(kind, 70_001, 21)
    img = oracle.encode_majority(x, scale, 1)
    col = MajorColumn.deserialize(img, scale, FLAG_RAW_BITMAPS)
    n = x.size
    for s, e, w in ((0, 1000, 100), (13, 13 + 128 * 70, 128), (5, 8, 3), (0, n // 1000 * 1000, 1000),
                    (31, 31 + 40 * 333, 333)):
        try:
            exp = oracle.max_majority_range(img, scale, s, e, w)
        except oracle.OraclePanic:
            with pytest.raises(capi.ReferencePanic):
                col.max_range(s, e, w)
            continue
        assert np.array_equal(col.max_range(s, e, w), exp), (kind, s, e, w)
