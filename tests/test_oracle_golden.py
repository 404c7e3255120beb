"""CPU checks of the oracle: the reference's own known-answer tests, then the
oracle against the independent numpy model (tests/model.py) and the
documented quirks."""
import math
import os

import numpy as np
import pytest

from tests import model as M


# ---- known-answer tests carried by the reference --------------------------

def test_bitpack_doc_vector(oracle):
    # methods/bit_packing.rs:57-71 and :297-312
    assert oracle.bitpack_write([(10, 4), (1021, 10), (3, 2)]) == bytes([218, 255])
    assert oracle.bitpack_read(bytes([218, 255]), [4, 10, 2]) == [10, 1021, 3]


def test_bitpack_smallbit(oracle):
    # test_smallbit, methods/bit_packing.rs:770-783
    buf = oracle.bitpack_write([(1, 1), (0, 1), (0, 1), (1, 1)])
    assert oracle.bitpack_read(buf, [1, 1, 1, 1]) == [1, 0, 0, 1]


def test_bitpack_bigbit(oracle):
    # test_bigbit, methods/bit_packing.rs:785-800
    pairs = [(255, 8), (65535, 16), (65535, 16), (255, 8), (65535, 16)]
    buf = oracle.bitpack_write(pairs)
    assert oracle.bitpack_read(buf, [b for _, b in pairs]) == [v for v, _ in pairs]


def test_bitpack_moresmallbit(oracle):
    # test_moresmallbit, methods/bit_packing.rs:802-819
    inp = [1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 1, 1, 1, 1, 0, 0, 1, 1, 0,
           1, 1, 1, 0, 0, 0, 1, 1, 0, 1, 0, 0, 0, 1, 0, 0, 1, 0, 0, 1,
           0, 0, 0, 1, 0, 1, 1, 0, 0, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 1]
    buf = oracle.bitpack_write([(b, 1) for b in inp])
    assert oracle.bitpack_read(buf, [1] * len(inp)) == inp


def test_bitvec_binary(oracle):
    # test_bit_vec_ser_deser, simd/vectorize_query.rs:562-573
    words = np.full(10, 32, dtype=np.uint32)
    b = oracle.bitvec_to_binary(words, 330)
    assert int.from_bytes(b[:8], "little") == 330
    assert np.frombuffer(b[8:], dtype="<u4").tolist() == [32] * 10
    assert sum(bin(int(w)).count("1") for w in words) == 10


def test_bviter_order(oracle):
    # test_BVIter, query/bit_vec_iter.rs:79-91, over BitVec::from_bytes
    # (bit-vec lib.rs:314-328): MSB-first bytes [0b10100000, 0b00010010]
    def rev(b):
        return int(f"{b:08b}"[::-1], 2)
    word = rev(0b10100000) | (rev(0b00010010) << 8)
    assert oracle.bviter(np.array([word], dtype=np.uint32)) == [0, 2, 11, 14]


def test_movemask_lane_order(oracle):
    # test_ceil, compress/buff_slice.rs:1995-2017: lane b <-> mask bit b
    buf = bytearray(32)
    buf[12] = 5
    gt, eq = oracle.movemask(bytes(buf), 5 ^ 0x80)
    assert eq == 4096
    buf = bytes([0x80 ^ i for i in range(32)])  # flipped 0..31
    gt, eq = oracle.movemask(buf, 10)
    assert eq == 1 << 10 and gt == ((1 << 32) - 1) ^ ((1 << 11) - 1)


def test_precision_bound_exponents(oracle):
    # get_precision_bound + PrecisionBound::new: exp = -dlen for p = 1..8
    assert [oracle.precision_exp(p) for p in range(1, 9)] == [-5, -8, -11, -15, -18, -21, -25, -28]
    assert [oracle.precision_exp(p) for p in range(16)] == [M.precision_exp(p) for p in range(16)]
    assert [oracle.dlen_of_prec(p) for p in range(1, 16)] == [M.PRECISION_MAP[p] for p in range(1, 16)]
    assert oracle.dlen_of_prec(0) == -1


def test_fetch_fixed_matches_model(oracle):
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.normal(0, 1000, 500), rng.uniform(-1e-3, 1e-3, 100),
                        [0.0, -0.0, 1.0, -1.0, 1e300, -1e300, 1e-300, float("inf")]])
    for dlen, pexp in [(15, -15), (5, -5), (50, -41), (10, -44)]:
        got = [oracle.fetch_fixed_aligned(float(v), pexp, dlen) for v in x]
        assert got == M.fetch_fixed(x, pexp, dlen).tolist()
    # trunc(v * 2^dlen) where exp + dlen <= 63
    v = rng.normal(0, 100, 1000)
    assert M.fetch_fixed(v, -15, 15).tolist() == np.trunc(v * 2.0 ** 15).astype(np.int64).tolist()


# ---- oracle vs the numpy model ------------------------------------------

def precision_bits(ilen, dlen, precision):
    """Bits a precision-limited read rebuilds (split_double.rs:1642-1664)."""
    if precision == 0:
        return ilen if ilen % 8 == 0 else (ilen // 8 + 1) * 8
    need = M.PRECISION_MAP[precision]
    rm = ilen + need
    if rm // 8 < (ilen + dlen) // 8 and rm % 8:
        rm = (rm // 8 + 1) * 8
    return rm


CASES = [
    # (generator, n, scale)
    ("walk", 1000, 10000), ("walk", 1003, 10000), ("walk", 777, 100), ("walk", 31, 1000),
    ("walk", 64, 10), ("narrow", 500, 100), ("narrow", 333, 10000), ("wide", 1000, 1000000),
    ("wide", 257, 100000000), ("neg", 640, 1000), ("updown", 515, 1000),
]


def make(kind, n, seed=11):
    rng = np.random.default_rng(seed + n)
    if kind == "walk":
        return np.round(1.0 + np.cumsum(rng.normal(0, 0.5, n)), 4)
    if kind == "narrow":
        return np.round(rng.uniform(3.0, 3.06, n), 2)
    if kind == "wide":
        return np.round(rng.normal(100, 5, n), 6)
    if kind == "neg":
        return np.round(-50 + np.cumsum(rng.normal(0, 0.1, n)), 3)
    if kind == "updown":
        x = np.round(np.cumsum(rng.normal(0, 1, n)), 3)
        x[0] = x.max() + 5  # first row is the column max (the `else if` max skips it)
        return x
    raise ValueError(kind)


@pytest.mark.parametrize("kind,n,scale", CASES)
@pytest.mark.parametrize("intended", [False, True])
def test_oracle_vs_model(oracle, kind, n, scale, intended):
    x = make(kind, n)
    flags = oracle.INTENDED if intended else 0
    prec = M.prec_of_scale(scale)
    q = M.fetch_fixed(x, M.precision_exp(prec), M.PRECISION_MAP[prec])
    L = M.layout(q, scale, intended)
    if L["fl"] == 0 and n > 0 and not intended:
        with pytest.raises(oracle.OraclePanic):
            oracle.encode(x, scale, True, flags)
        return
    buf = oracle.encode(x, scale, True, flags)
    h = oracle.header(buf)
    assert (h.base, h.n, h.fixed_len, h.k, h.r) == (L["base"], n, L["fl"], L["k"], L["r"])
    assert len(buf) == 20 + L["k"] * n + (n * L["r"] + 7) // 8
    d = oracle.decode(buf, scale)
    exp = np.array([float(M.wrap64(L["base"] + int(c))) / 2.0 ** L["dlen"] for c in L["codes"]])
    assert np.array_equal(d, exp)
    for p in [x[n // 3], x[0], float(np.quantile(x, 0.9)), float(x.max()) + 1.0,
              float(x.min()) - 1.0, float(x.min())]:
        w, c, _ = oracle.range_filter(buf, scale, p, flags)
        assert np.array_equal(w, M.filter_words(L, p, True, intended)), p
        w, c, _ = oracle.equal_filter(buf, scale, p, flags)
        assert np.array_equal(w, M.filter_words(L, p, False, intended)), p
    if not intended:
        # the scalar buff-layout filters of the `buff` profiler arm
        # (buff_simd.rs:4507-4679, :4925-5094) on the byte_fixed_encode image
        bbuf = oracle.encode(x, scale, False)
        for p in [x[n // 3], x[0], float(np.quantile(x, 0.9)), float(x.max()) + 1.0,
                  float(x.min()) - 1.0, float(x.min())]:
            w, c, _ = oracle.scalar_range_filter(bbuf, scale, p)
            assert np.array_equal(w, M.filter_words(L, p, True, False, False)), p
            w, c, _ = oracle.scalar_equal_filter(bbuf, scale, p)
            assert np.array_equal(w, M.filter_words(L, p, False, False, False)), p
    s, parts, exact = oracle.buff_sum(buf, scale, True, flags)
    assert s == M.ref_sum(L, n, intended)
    assert exact == n * L["base"] + sum(int(c) for c in L["codes"])
    mv, mc, aw, ac = oracle.buff_max(buf, scale, True, flags)
    assert mc == int(L["codes"].max())


def test_quirk_else_if_max(oracle):
    # Q1: the first row never updates max; [10, 3, 5] -> max 5, width ceil(log2(2)) = 1
    x = np.array([10.0, 3.0, 5.0] + [4.0] * 61)
    buf = oracle.encode(x, 10)
    h = oracle.header(buf)
    q = M.fetch_fixed(x, -5, 5)
    assert h.base == q.min() and h.fixed_len == math.ceil(math.log2(q[2] - q.min()))
    # the decoded first row is truncated to the stored width
    assert oracle.decode(buf, 10)[0] != 10.0
    buf2 = oracle.encode(x, 10, True, oracle.INTENDED)
    assert oracle.decode(buf2, 10)[0] == 10.0


def test_quirk_width_power_of_two(oracle):
    # Q2: delta = 2^j gives j bits, the max code loses its top bit
    x = np.array([0.0, 8.0] + [1.0] * 62)  # scale 10: dlen 5 -> delta 256 = 2^8
    buf = oracle.encode(x, 10)
    assert oracle.header(buf).fixed_len == 8
    assert oracle.decode(buf, 10)[1] == 0.0


def test_quirk_constant_column_panics(oracle):
    with pytest.raises(oracle.OraclePanic):
        oracle.encode(np.full(100, 3.5), 100)
    buf = oracle.encode(np.full(100, 3.5), 100, True, oracle.INTENDED)
    assert oracle.header(buf).fixed_len == 0
    assert np.all(oracle.decode(buf, 100) == 3.5)


def test_quirk_scale_without_precision_panics(oracle):
    with pytest.raises(oracle.OraclePanic):
        oracle.encode(np.arange(10.0), 1)


def test_quirk_tail_rows_never_set(oracle):
    # Q3: rows after the last full 32-row block are never set
    x = np.round(np.linspace(0, 100, 100), 2)
    buf = oracle.encode(x, 100)
    w, c, _ = oracle.range_filter(buf, 100, 50.0)
    rows = np.nonzero(np.unpackbits(w.view(np.uint8), bitorder="little")[:100])[0]
    assert rows.max() < 96 and c == np.sum(x[:96] > 50.0)


def test_quirk_early_return(oracle):
    x = np.round(np.linspace(10, 20, 64), 2)
    buf = oracle.encode(x, 100)
    w, c, early = oracle.range_filter(buf, 100, 5.0)
    assert early and c == 64
    w, c, early = oracle.equal_filter(buf, 100, 5.0)
    assert early and c == 0
    w, c, early = oracle.equal_filter_with_slice(buf, 100, 5.0)
    assert early and c == 64


def test_with_slice_matches_plain_for_four_slices(oracle):
    x = make("wide", 4096)
    buf = oracle.encode(x, 1000000)
    assert oracle.header(buf).k <= 4
    for p in [float(np.quantile(x, q)) for q in (0.1, 0.5, 0.99)] + [float(x[17])]:
        assert np.array_equal(oracle.range_filter(buf, 1000000, p)[0],
                              oracle.range_filter_with_slice(buf, 1000000, p)[0])
        assert np.array_equal(oracle.equal_filter(buf, 1000000, p)[0],
                              oracle.equal_filter_with_slice(buf, 1000000, p)[0])


def test_precision_decode_semantics(oracle):
    x = make("walk", 640)
    buf = oracle.encode(x, 10000)
    h = oracle.header(buf)
    full = oracle.decode(buf, 10000)
    assert np.array_equal(oracle.decode_at_precision(buf, 10000, 4), full)
    # intended: keep the top R bits in place -> error below 2^-8 at 2 decimals
    d2 = oracle.decode_at_precision(buf, 10000, 2, True, oracle.INTENDED)
    assert np.all(np.abs(d2 - full) < 2.0 ** -8 * 2) and np.all(d2 <= full)
    # reference: bits not shifted back (Q6) when R < fixed_len
    dr = oracle.decode_at_precision(buf, 10000, 2)
    R = precision_bits(h.ilen, h.dlen, 2)
    assert R < h.fixed_len and R % 8 == 0
    L = M.layout(M.fetch_fixed(x, -15, 15), 10000, False)
    exp = np.array([float(L["base"] + (int(c) >> (h.fixed_len - R))) / 2.0 ** 15
                    for c in L["codes"]])
    assert np.array_equal(dr, exp)
    with pytest.raises(oracle.OraclePanic):
        oracle.decode_at_precision(buf, 10000, 5)  # dlen 15 < bits for 5 decimals


def test_reference_fixture_readme_query(oracle, readme_input):
    """The README quick-start input (database/data/randomwalkdatasample1k-1k,
    scale 10000, pred 1.1509): the oracle's results agree with the model and
    with the committed digests in tests/golden/fixture_digest.json."""
    import json

    from tests.golden.make_golden import fixture_digest, load_fixture

    x = load_fixture(readme_input)
    assert x.size == 500000
    got = fixture_digest(oracle, x)
    with open(os.path.join(os.path.dirname(__file__), "golden", "fixture_digest.json")) as f:
        want = json.load(f)
    assert got == want
