"""CPU checks of the oracle's buff-slice layout (compress/buff_slice.rs)
against the whole-array model in tests/model.py."""
import numpy as np
import pytest

from tests import model as M
from tests.test_oracle_cond import cond_cases


def _layout(x, scale):
    prec = M.prec_of_scale(scale)
    q = M.fetch_fixed(x, M.precision_exp(prec), M.PRECISION_MAP[prec])
    return M.layout(q, scale, False)


@pytest.mark.parametrize("case", range(4))
def test_slice_layout_vs_model(oracle, case):
    name, x, scale = cond_cases()[case]
    L = _layout(x, scale)
    buf = oracle.slice_encode(x, scale)
    fl = L["fl"]
    num = 1 if fl < 8 else (fl + 7) // 8
    pad = 8 * num - fl
    assert len(buf) == 20 + num * x.size
    codes = [int(c) for c in L["codes"].tolist()]
    # every slice byte is (code << pad) >> 8*(num-1-j), flipped
    for j in range(num):
        sl = np.frombuffer(buf[20 + j * x.size: 20 + (j + 1) * x.size], dtype=np.uint8)
        exp = np.array([((c << pad) >> (8 * (num - 1 - j))) & 0xFF for c in codes], dtype=np.uint8)
        assert np.array_equal(sl ^ 0x80, exp), (name, j)
    vals = np.array([float(M.wrap64(L["base"] + c)) / 2.0 ** L["dlen"] for c in codes])
    assert np.array_equal(oracle.slice_decode(buf, scale), vals)
    # sums: sequential f64 (the model adds in row order too)
    s = 0.0
    for v in vals:
        s += v
    if num <= 4:
        assert oracle.slice_sum(buf, scale) == s
    assert oracle.slice_sum(buf, scale, any_width=True) == s
    mv, words, cnt = oracle.slice_max(buf, scale, any_width=True)
    assert mv == vals.max() and cnt == int((vals == vals.max()).sum())
    # filters: compare of the padded code's first min(num, 4) bytes with the
    # target's bytes, rows of full 32-row blocks only
    for p in (float(np.quantile(x, 0.3)), float(np.quantile(x, 0.9)), float(x[11]),
              float(x.min()) - 1, float(x.max()) + 3):
        fp = int(M.fetch_fixed(np.array([p]), L["pexp"], L["dlen"])[0])
        wr, cr, er = oracle.slice_range_filter(buf, scale, p)
        we, ce, ee = oracle.slice_equal_filter(buf, scale, p)
        if fp < L["base"]:
            assert er and ee and cr == ce == x.size
            continue
        t = fp - L["base"]
        used = min(num, 4)

        def key(v):
            return tuple(((v << pad) >> (8 * (num - 1 - j))) & 0xFF for j in range(used))

        tk = tuple((t >> (fl - 8 * (j + 1))) & 0xFF if fl - 8 * j >= 8 else (t << (8 * (j + 1) - fl)) & 0xFF
                   for j in range(used))
        full = x.size // 32 * 32
        gt = np.array([key(c) > tk and i < full for i, c in enumerate(codes)], dtype=np.uint8)
        eq = np.array([key(c) == tk and i < full for i, c in enumerate(codes)], dtype=np.uint8)
        assert np.array_equal(wr, M.bits_to_words(gt)), (name, p)
        assert np.array_equal(we, M.bits_to_words(eq)), (name, p)
        # the nosimd forms of the buff-slice-scalar arm: every row
        wr, cr, _ = oracle.slice_range_filter_nosimd(buf, scale, p)
        we, ce, _ = oracle.slice_equal_filter_nosimd(buf, scale, p)
        gt = np.array([key(c) > tk for c in codes], dtype=np.uint8)
        eq = np.array([key(c) == tk for c in codes], dtype=np.uint8)
        assert np.array_equal(wr, M.bits_to_words(gt)) and cr == int(gt.sum()), (name, p)
        assert np.array_equal(we, M.bits_to_words(eq)) and ce == int(eq.sum()), (name, p)
    # decode_bs: the full decode for 1-4 slices, a panic beyond
    if num <= 4 and fl > 0:
        assert np.array_equal(oracle.slice_decode_bs(buf, scale), vals)
    else:
        with pytest.raises(oracle.OraclePanic):
            oracle.slice_decode_bs(buf, scale)


def _model_max_range(vals, n, fl, num, s, e, w):
    """Window maxima as buff_slice.rs:930-1099 states them; None = panic."""
    if fl == 0 or num > 4 or w == 0:
        return None
    hi = min(e, n)
    if hi > s:
        nwin = -(-(hi - s) // w)
        out = [vals[s + j * w: min(s + (j + 1) * w, hi)].max() for j in range(nwin)]
    else:
        nwin, out = 1, [-np.finfo(np.float64).max]
    if nwin != ((e - s) % 2**32) // w:
        return None
    return np.array(out)


@pytest.mark.parametrize("case", range(4))
def test_slice_max_range_vs_model(oracle, case):
    name, x, scale = cond_cases()[case]
    buf = oracle.slice_encode(x, scale)
    h = oracle.header(buf)
    fl = h.fixed_len
    num = 1 if fl < 8 else (fl + 7) // 8
    vals = oracle.slice_decode(buf, scale)
    n = x.size
    windows = [(0, 1000, 100), (13, 13 + 128 * 7, 128), (5, 8, 3), (0, n, 1), (31, 31 + 200, 200),
               (0, n // 3, 7), (0, n, 100), (n - 50, n + 50, 100), (n - 50, n + 150, 100),
               (n + 5, n + 105, 100), (n + 5, n + 5, 10), (10, 5, 3), (0, 100, 0),
               (7, 7 + 3 * 64 + 1, 64)]
    for s, e, w in windows:
        exp = _model_max_range(vals, n, fl, num, s, e, w)
        if exp is None:
            with pytest.raises(oracle.OraclePanic):
                oracle.slice_max_range(buf, scale, s, e, w)
        else:
            got = oracle.slice_max_range(buf, scale, s, e, w)
            assert np.array_equal(got, exp), (name, s, e, w)
