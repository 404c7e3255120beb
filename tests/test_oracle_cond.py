"""CPU checks of the oracle's row-conditioned reads (buff_decode_condition,
buff_range_filter_condition and their buff-major forms) against the
whole-array model in tests/model.py."""
import numpy as np
import pytest

from tests import model as M
from tests.test_oracle_major import major_case


def cond_cases():
    rng = np.random.default_rng(21)
    walk = np.round(np.cumsum(rng.normal(0, 0.5, 5003)) + 40, 3)
    small = np.round(rng.uniform(0, 0.06, 3001), 2)           # fixed_len < 8
    byte8 = np.round(rng.uniform(0, 2.5, 2049), 2)            # fixed_len 8
    return [("walk_r", walk, 1000), ("small", small, 100), ("byte8", byte8, 100),
            ("gauss", np.round(rng.normal(0, 100, 4097), 4), 10000)]


def _rows(rng, n, frac):
    return np.sort(rng.choice(n, max(1, int(n * frac)), replace=False)).astype(np.uint64)


@pytest.mark.parametrize("case", range(4))
def test_decode_condition_vs_model(oracle, case):
    name, x, scale = cond_cases()[case]
    buf = oracle.encode(x, scale, flipped=False)
    L = M.layout(M.fetch_fixed(x, M.precision_exp(M.prec_of_scale(scale)),
                               M.PRECISION_MAP[M.prec_of_scale(scale)]), scale, False)
    rng = np.random.default_rng(case)
    for frac in (0.001, 0.1, 1.0):
        rows = _rows(rng, x.size, frac)
        got = oracle.decode_condition(buf, scale, rows)
        assert np.array_equal(got, M.cond_decode(L, rows.tolist(), True)), (name, frac)
    with pytest.raises(oracle.OraclePanic):
        oracle.decode_condition(buf, scale, [])


@pytest.mark.parametrize("case", range(4))
def test_range_filter_condition_vs_model(oracle, case):
    name, x, scale = cond_cases()[case]
    buf = oracle.encode(x, scale, flipped=False)
    L = M.layout(M.fetch_fixed(x, M.precision_exp(M.prec_of_scale(scale)),
                               M.PRECISION_MAP[M.prec_of_scale(scale)]), scale, False)
    rng = np.random.default_rng(100 + case)
    preds = [float(np.quantile(x, q)) for q in (0.1, 0.5, 0.9)] + \
        [float(x.min()) - 1, float(x.max()) + 5, float(x[3])]
    for frac in (0.0, 0.01, 0.3, 1.0):
        rows = _rows(rng, x.size, frac) if frac else np.zeros(0, dtype=np.uint64)
        for p in preds:
            w, c = oracle.range_filter_condition(buf, scale, p, rows)
            exp = M.cond_range(L, p, rows.tolist())
            assert np.array_equal(w, exp), (name, frac, p)
            assert c == int(np.unpackbits(exp.view(np.uint8)).sum())


@pytest.mark.parametrize("kind", ["one", "none"])
def test_major_condition_vs_model(oracle, kind):
    x, scale = major_case(kind, 4099, 9)
    buf = oracle.encode_majority(x, scale, 1)
    ncols = oracle.majority_layout(buf, 1)[0]
    L = M.layout(M.fetch_fixed(x, M.precision_exp(M.prec_of_scale(scale)),
                               M.PRECISION_MAP[M.prec_of_scale(scale)]), scale, True)
    rows = _rows(np.random.default_rng(3), x.size, 0.05)
    got = oracle.major_decode_condition(buf, scale, rows)
    p = float(np.quantile(x, 0.4))
    w, c = oracle.range_filter_majority_condition(buf, scale, p, rows)
    if ncols:
        assert got.size == 0 and c == 0 and not w.any()
    else:
        assert np.array_equal(got, M.cond_decode(L, rows.tolist(), False))
        assert np.array_equal(w, M.cond_range(L, p, rows.tolist()))


def test_condition_rejects_unsorted_rows(oracle):
    x = np.round(np.linspace(0, 10, 100), 1)
    buf = oracle.encode(x, 10, flipped=False)
    with pytest.raises(RuntimeError):
        oracle.decode_condition(buf, 10, [5, 3])
    with pytest.raises(RuntimeError):
        oracle.decode_condition(buf, 10, [5, 100])


@pytest.mark.parametrize("case", range(4))
def test_max_range_vs_model(oracle, case):
    name, x, scale = cond_cases()[case]
    buf = oracle.encode(x, scale, flipped=False)
    L = M.layout(M.fetch_fixed(x, M.precision_exp(M.prec_of_scale(scale)),
                               M.PRECISION_MAP[M.prec_of_scale(scale)]), scale, False)
    n = x.size
    for s, e, w in ((0, n // 100 * 100, 100), (7, 7 + 3 * min(1000, (n - 7) // 3), 3),
                    (0, n - n % 64, 64), (5, 5 + 512, 512)):
        got = oracle.max_range(buf, scale, s, e, w)
        assert np.array_equal(got, M.max_range(L, s, e, w)), (name, s, e, w)
    # a ragged last window: dropped when the code fits one byte, a panic otherwise
    if L["fl"] <= 8:
        assert oracle.max_range(buf, scale, 0, 105, 10).size == 10
    else:
        with pytest.raises(oracle.OraclePanic):
            oracle.max_range(buf, scale, 0, 105, 10)
    with pytest.raises(oracle.OraclePanic):
        oracle.max_range(buf, scale, 0, n + 1, 10)


@pytest.mark.parametrize("kind", ["none", "one"])
def test_max_majority_range_vs_max_range(oracle, kind):
    """buff_max_majority_range: buff_max_range on the slices after the count
    byte, no windows with sparse columns."""
    from tests.test_oracle_major import major_case

    x, scale = major_case(kind, 5003, 9)
    img = oracle.encode_majority(x, scale, 1)
    ncols = oracle.majority_layout(img, 1)[0]
    plain = oracle.encode(x, scale, flipped=False)
    for s, e, w in ((0, 1000, 100), (13, 13 + 128 * 7, 128), (7, 7 + 40 * 33, 33), (0, 4096, 4096)):
        got = oracle.max_majority_range(img, scale, s, e, w)
        if ncols:
            assert got.size == 0
        else:
            assert np.array_equal(got, oracle.max_range(plain, scale, s, e, w)), (s, e, w)
