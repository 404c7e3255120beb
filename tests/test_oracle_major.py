"""CPU checks of the oracle's buff-major (outlier) format: snappy round trips
and the oracle against the whole-array model in tests/model.py."""
import numpy as np
import pytest

from tests import model as M


def test_snappy_round_trips(oracle):
    rng = np.random.default_rng(0)
    cases = [b"", b"a", bytes(1000), bytes(rng.integers(0, 4, 100000, dtype=np.uint8)),
             bytes(rng.integers(0, 256, 70000, dtype=np.uint8)), b"abcabcabcabc" * 5000,
             bytes(rng.integers(0, 2, 300000, dtype=np.uint8) * 255)]
    for data in cases:
        c = oracle.snappy_compress(data)
        assert oracle.snappy_decompress(c) == data
    # a hand-made stream: literal "ab", then a 2-byte-offset copy of length 4
    assert oracle.snappy_decompress(bytes([6, 0x04, 97, 98, 0x0E, 2, 0])) == b"ababab"


def major_case(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "one":      # one sparse leading byte
        x = np.round(rng.normal(100, 5, n), 6)
        pos = rng.choice(n, n // 100, replace=False)
        x[pos] = np.round(rng.uniform(-1e4, 1e4, pos.size), 6)
        return x, 1000000
    if kind == "two":      # two sparse bytes (outliers far out, values tight)
        x = np.round(rng.normal(100, 0.05, n), 4)
        pos = rng.choice(n, n // 50, replace=False)
        x[pos] = np.round(rng.uniform(-5e3, 5e3, pos.size), 4)
        return x, 10000
    if kind == "three":
        x = np.round(rng.normal(7, 0.0001, n), 6)
        pos = rng.choice(n, n // 40, replace=False)
        x[pos] = np.round(rng.uniform(-1e3, 1e3, pos.size), 6)
        return x, 1000000
    if kind == "none":     # no majority: plain buff layout one byte later
        return np.round(np.cumsum(rng.normal(0, 1, n)), 2), 100
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["one", "two", "three", "none"])
@pytest.mark.parametrize("mode", [0, 1])
def test_majority_oracle_vs_model(oracle, kind, mode):
    x, scale = major_case(kind, 4099, 5)
    L = M.major_layout(x, scale)
    buf = oracle.encode_majority(x, scale, mode)
    ncols, majors, nouts, _ = oracle.majority_layout(buf, mode)
    assert majors == L["majors"][:ncols] and ncols == len(L["majors"])
    h = oracle.header(buf)
    assert h.base == L["base"] and h.fixed_len == L["fl"]
    if ncols:
        codes = M.major_decode_codes(L)
        exp = np.array([float(M.wrap64(L["base"] + c)) / 2.0 ** L["dlen"] for c in codes])
        if all(nouts):
            assert np.array_equal(oracle.decode_majority(buf, scale, mode), exp)
    preds = [float(x[100]), float(np.quantile(x, 0.3)), float(np.quantile(x, 0.99)),
             float(x.max()) + 1, float(x.min()) - 1, float(x.max())]
    for p in preds:
        w, c, _ = oracle.range_filter_majority(buf, scale, p, mode)
        assert np.array_equal(w, M.major_filter(L, p, True)), p
        w, c, _ = oracle.equal_filter_majority(buf, scale, p, mode)
        assert np.array_equal(w, M.major_filter(L, p, False)), p
    s, _ = oracle.sum_majority(buf, scale, mode)
    assert s == M.major_sum(L)
    mv, mc, aw, ac = oracle.max_majority(buf, scale, mode)
    assert mc == M.major_max_code(L)


def test_majority_small_column_panics(oracle):
    with pytest.raises(oracle.OraclePanic):
        oracle.encode_majority(np.arange(100.0), 100)
