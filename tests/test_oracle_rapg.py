"""CPU checks of the oracle's RAPG byte_residue restatement
(compress/split_double.rs:624-955, 1353-1893, 2211-2630).

The roaring serializer is pinned to byte images worked out by hand from the
published Roaring portable format; the codec against an independent
whole-array model of the image layout, the decoders and the sums.
"""
import math

import numpy as np
import pytest

from tests import model as M

SAMPLE = 2000


# ---------------------------------------------------------------- roaring

def _hex(s):
    return bytes.fromhex(s.replace(" ", ""))


def test_roaring_known_images(oracle):
    # one array container (4 values, 2 runs: the run form is not smaller)
    assert oracle.roaring_serialize([1, 2, 3, 1000]) == _hex(
        "3a300000 01000000 00000300 10000000 0100 0200 0300 e803")
    # one run container [5, 14]: cookie with size-1 in the high half, run flag
    # byte, key/card-1, no offsets below 4 containers, n_runs, (start, len-1)
    assert oracle.roaring_serialize(list(range(5, 15))) == _hex(
        "3b300000 01 00000900 0100 0500 0900")
    # empty bitmap
    assert oracle.roaring_serialize([]) == _hex("3a300000 00000000")
    # 4 run containers: offsets present from 4 containers on
    rows = [k * 65536 + v for k in range(4) for v in range(10, 20)]
    img = oracle.roaring_serialize(rows)
    assert img[:4] == _hex("3b300300") and img[4] == 0x0F
    start = 4 + 1 + 8 * 4
    offs = [int.from_bytes(img[5 + 16 + 4 * k: 9 + 16 + 4 * k], "little") for k in range(4)]
    assert offs == [start + 6 * k for k in range(4)]
    assert len(img) == start + 4 * 6


def test_roaring_container_choice(oracle):
    rng = np.random.default_rng(5)
    dense = np.sort(rng.choice(65536, 5000, replace=False)).astype(np.uint32)
    img = oracle.roaring_serialize(dense)  # > 4096 values, many runs: bitset
    assert len(img) == 8 + 8 + 8192 and img[:4] == _hex("3a300000")
    bits = np.unpackbits(np.frombuffer(img[16:], dtype=np.uint8), bitorder="little")
    assert np.array_equal(np.nonzero(bits)[0], dense)
    img = oracle.roaring_serialize(np.arange(6000, dtype=np.uint32))  # bitset -> one run
    assert img == _hex("3b300000 01 00006f17 0100 0000 6f17")
    # array vs run at the threshold: 2 runs cost 10 bytes, 5 values 12
    assert oracle.roaring_serialize([0, 1, 2, 10, 11])[:4] == _hex("3b300000")
    assert oracle.roaring_serialize([0, 1, 10, 11])[:4] == _hex("3a300000")


@pytest.mark.parametrize("seed", range(6))
def test_roaring_round_trip(oracle, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 300_000))
    dens = rng.uniform(0.0001, 0.9)
    rows = np.nonzero(rng.uniform(size=n) < dens)[0].astype(np.uint32)
    if seed % 2:
        rows = np.unique(np.concatenate([rows, np.arange(1000, 9000, dtype=np.uint32)]))
    img = oracle.roaring_serialize(rows)
    assert np.array_equal(oracle.roaring_parse(img), rows)
    with pytest.raises(oracle.OraclePanic):
        oracle.roaring_parse(b"\x01\x02\x03\x04\x05")


# ---------------------------------------------------------------- model

def _fl(delta):
    if delta == 0:
        return 0
    c = math.ceil(math.log2(float(delta))) if delta > 0 else float("nan")
    return 0 if (c != c or c <= 0) else int(c)


def rapg_model(x, scale):
    """Layout of byte_residue_encode for the values x (None: it panics)."""
    prec = M.prec_of_scale(scale)
    dlen = M.PRECISION_MAP[prec]
    q = [int(v) for v in M.fetch_fixed(np.asarray(x, dtype=np.float64), M.precision_exp(prec),
                                       dlen).tolist()]
    n = len(q)
    mn, mx = min(q), max(q)
    fl = _fl(M.wrap64(mx - mn))
    u = [(v - mn) & (2**64 - 1) for v in q]
    ilen = (fl - dlen) % 2**64
    cols = 0
    if ilen > 15:
        if n < SAMPLE:
            return None
        # samples with a set bit in the top 8(c+1) bits of the fixed_len-bit code
        for c in range(ilen // 8):
            if c >= 4:
                return None  # bits_counter[32]
            top = sum(1 for v in u[:SAMPLE] if v < (1 << fl) and v.bit_length() > fl - 8 * (c + 1))
            if top < int(np.float32(SAMPLE) * np.float32(0.1)):
                cols += 1
            else:
                break
    return dict(base=mn, fl=fl, dlen=dlen, ilen=ilen, u=u, n=n, cols=cols)


def _value(L, v):
    return float(M.wrap64(L["base"] + v)) / 2.0 ** L["dlen"]


def _tail_field(L, tail, i, width):
    return (tail >> (i * width)) & ((1 << width) - 1)


def _precision_bits(L, p):
    ilen, dlen = L["ilen"] & 0xFFFFFFFF, L["dlen"]
    if p is None:
        return (ilen + dlen) & 0xFFFFFFFF
    if p == 0:
        return ilen if ilen % 8 == 0 else (ilen // 8 + 1) * 8
    need = M.PRECISION_MAP[p]
    if dlen < need:
        return None
    R = ilen + need
    if R // 8 < (dlen + ilen) // 8 and R % 8:
        R = (R // 8 + 1) * 8
    return R


def rapg_decode_model(L, p=None):
    """Values byte_residue_decode(_with_precision) returns for a sane image
    (fixed_len >= 8): the top R bits of each code, not shifted back."""
    R = _precision_bits(L, p)
    if R is None:
        return None
    fl, cols, n = L["fl"], L["cols"], L["n"]
    remain = R
    fixed = [0] * n
    for c in range(cols):
        remain -= 8
        for i, v in enumerate(L["u"]):
            fixed[i] |= ((v >> (fl - 8 * (c + 1))) & 0xFF) << remain
    if remain == 0 and cols:
        return np.zeros(0)
    d = 0
    k_dense = (fl - 8 * cols) // 8
    r = fl - 8 * cols - 8 * k_dense
    while remain >= 8:
        remain -= 8
        for i, v in enumerate(L["u"]):
            fixed[i] |= ((v >> (fl - 8 * (cols + d + 1))) & 0xFF) << remain
        d += 1
    if remain:
        tail = 0
        for i, v in enumerate(L["u"]):
            tail |= (v & ((1 << r) - 1)) << (i * r)
        for i in range(n):
            fixed[i] |= _tail_field(L, tail, i, remain)
    return np.array([_value(L, f) for f in fixed])


def rapg_sum_model(L, p=None):
    R = _precision_bits(L, p)
    if R is None:
        return None
    fl, cols, n, ilen = L["fl"], L["cols"], L["n"], L["ilen"] & 0xFFFFFFFF
    ilen32 = ilen - (1 << 32) if ilen >> 31 else ilen
    remain, processed, s = R, 0, 0.0
    sum_base = (float(n) * float(L["base"])) / 2.0 ** L["dlen"]
    for c in range(cols):
        remain -= 8
        processed += 8
        part = sum((v >> (fl - 8 * (c + 1))) & 0xFF for v in L["u"])
        s = s + float(part) / 2.0 ** (processed - ilen32)
    k_dense = (fl - 8 * cols) // 8
    r = fl - 8 * cols - 8 * k_dense
    d = 0
    while remain >= 8:
        remain -= 8
        processed += 8
        part = sum((v >> (fl - 8 * (cols + d + 1))) & 0xFF for v in L["u"])
        s = s + float(part) / 2.0 ** (processed - ilen32)
        d += 1
        if remain == 0:
            return s
    if remain:
        processed += remain
        tail = 0
        for i, v in enumerate(L["u"]):
            tail |= (v & ((1 << r) - 1)) << (i * r)
        part = sum(_tail_field(L, tail, i, remain) for i in range(n))
        s = s + float(part) / 2.0 ** (processed - ilen32)
    return s + sum_base


def rapg_cases():
    rng = np.random.default_rng(41)
    walk = np.round(1 + np.cumsum(rng.normal(0, 0.3, 5000)), 4)           # ilen <= 15
    wide = np.round(np.cumsum(rng.normal(0, 1000, 4001)), 2)               # ilen > 15, dense top
    one = np.round(rng.normal(100, 5, 6000), 6)                             # 1 outlier column
    pos = np.nonzero(rng.uniform(size=one.size) < 0.01)[0]
    one[pos] = np.round(rng.uniform(1e5, 1e6, pos.size), 6)
    two = np.round(rng.normal(100, 0.5, 7001), 6)                           # 2 outlier columns
    pos = np.nonzero(rng.uniform(size=two.size) < 0.02)[0]
    two[pos] = np.round(rng.uniform(1e4, 1e6, pos.size), 6)
    three = np.round(rng.uniform(0, 1, 5000), 2)                           # 3 columns
    pos = np.nonzero(rng.uniform(size=three.size) < 0.005)[0]
    three[pos] = np.round(rng.uniform(1e6, 1e7, pos.size), 2)
    const = np.full(3000, 7.25)
    return [("walk", walk, 10000), ("wide", wide, 100), ("one", one, 1000000),
            ("two", two, 1000000), ("three", three, 100), ("const", const, 100)]


@pytest.mark.parametrize("case", range(6))
def test_rapg_layout_vs_model(oracle, case):
    name, x, scale = rapg_cases()[case]
    L = rapg_model(x, scale)
    img = oracle.rapg_encode(x, scale)
    h = oracle.header(img)
    assert (h.base, h.n, h.ilen, h.dlen) == (L["base"], L["n"], L["ilen"] & 0xFFFFFFFF, L["dlen"])
    cols, sizes, nouts, offs = oracle.rapg_layout(img)
    assert cols == L["cols"], name
    fl, n, u = L["fl"], L["n"], L["u"]
    pos = 20 + (1 if L["ilen"] > 15 else 0)
    for c in range(cols):
        byte = [(v >> (fl - 8 * (c + 1))) & 0xFF for v in u]
        rows = np.array([i for i, b in enumerate(byte) if b], dtype=np.uint32)
        assert offs[c] == pos + 4
        bm = img[offs[c]: offs[c] + sizes[c]]
        assert bm == oracle.roaring_serialize(rows)
        assert nouts[c] == rows.size
        ob = img[offs[c] + sizes[c] + 4: offs[c] + sizes[c] + 4 + nouts[c]]
        assert list(ob) == [byte[i] for i in rows]
        pos = offs[c] + sizes[c] + 4 + nouts[c]
    if cols:
        pos += 1  # the pad byte left by the last column
    k_dense = (fl - 8 * cols) // 8 if fl >= 8 else 0
    for d in range(k_dense):
        sl = np.frombuffer(img[pos + d * n: pos + (d + 1) * n], dtype=np.uint8)
        exp = np.array([(v >> (fl - 8 * (cols + d + 1))) & 0xFF for v in u], dtype=np.uint8)
        assert np.array_equal(sl, exp), (name, d)
    r = fl - 8 * cols - 8 * k_dense
    tail_len = max(1, (n * r + 7) // 8) if r else 0
    assert len(img) == pos + k_dense * n + tail_len
    # decoders and sums, full and at every precision
    # (precision reads of a code narrower than a byte take the wrapped ilen;
    # the model covers the full read only)
    for p in [None] + (list(range(16)) if fl >= 8 else []):
        want = rapg_decode_model(L, p)
        prec = -1 if p is None else p
        if want is None:
            with pytest.raises(oracle.OraclePanic):
                oracle.rapg_decode(img, scale, prec)
            continue
        got = oracle.rapg_decode(img, scale, prec)
        assert np.array_equal(got, want), (name, p)
        assert oracle.rapg_sum(img, scale, prec) == rapg_sum_model(L, p), (name, p)


def test_rapg_full_decode_is_exact(oracle):
    for name, x, scale in rapg_cases():
        img = oracle.rapg_encode(x, scale)
        L = rapg_model(x, scale)
        want = np.array([_value(L, v) for v in L["u"]])
        assert np.array_equal(oracle.rapg_decode(img, scale), want), name


def test_rapg_panics(oracle):
    rng = np.random.default_rng(3)
    # ilen > 15 with fewer than 2000 rows: fixed_vec[0..SAMPLE]
    with pytest.raises(oracle.OraclePanic):
        oracle.rapg_encode(np.round(np.cumsum(rng.normal(0, 1000, 1999)), 2), 100)
    # four sparse leading bytes of a 48-bit code: bits_counter[32]
    x = np.round(rng.uniform(0, 1, 4000), 2)
    x[::500] = 1e12
    with pytest.raises(oracle.OraclePanic):
        oracle.rapg_encode(x, 100)
    # scale without a PRECISION_MAP entry
    with pytest.raises(oracle.OraclePanic):
        oracle.rapg_encode(np.arange(10.0), 1)
    # codes narrower than dlen: the count byte is overwritten by packed codes,
    # which the decoders read one byte late and past the end
    x = np.round(rng.uniform(3.0, 3.06, 5000), 2)
    img = oracle.rapg_encode(x, 100)
    fl = rapg_model(x, 100)["fl"]
    assert fl < 8 and len(img) == 20 + (5000 * fl + 7) // 8
    with pytest.raises(oracle.OraclePanic):
        oracle.rapg_decode(img, 100)
    # precision finer than the column
    name, x, scale = rapg_cases()[0]
    with pytest.raises(oracle.OraclePanic):
        oracle.rapg_decode(oracle.rapg_encode(x, scale), scale, 5)


# ---------------------------------------------------------------- RAPG-major

def outlieru8_case(ratio, n, seed, scale):
    """outlier_exp's input (outlier/mod.rs:13-60): byte values, MAJOR = 69
    with probability `ratio`, otherwise uniform in [0, 256), one 0 and one
    255 at random rows; as f64."""
    rng = np.random.default_rng(seed)
    v = np.where(rng.uniform(size=n) < ratio, 69, rng.integers(0, 256, n))
    i0, i255 = rng.choice(n, 2, replace=False)
    v[i0], v[i255] = 0, 255
    return v.astype(np.float64), scale


@pytest.mark.parametrize("ratio,scale", [(0.9, 10), (0.99, 100), (0.5, 1000), (0.999, 10000)])
def test_outlieru8_vs_model(oracle, ratio, scale):
    """byte_residue_encode_outlieru8 is the buff-major image with MAJOR as
    the one sparse byte and a roaring bitmap; with one sparse column the
    byte_residue_*_majority queries are the buff-major ones."""
    x, scale = outlieru8_case(ratio, 5003, 7, scale)
    L = M.major_layout(x, scale)
    L["majors"] = [69]
    buf = oracle.encode_outlieru8(x, scale)
    ncols, majors, nouts, _ = oracle.majority_layout(buf, oracle.BM_ROARING)
    assert ncols == 1 and majors == [69]
    codes = M.major_decode_codes(L)
    exp = np.array([float(M.wrap64(L["base"] + c)) / 2.0 ** L["dlen"] for c in codes])
    assert np.array_equal(oracle.decode_majority(buf, scale, oracle.BM_ROARING), exp)
    assert nouts[0] == int(np.sum([((c >> (L["fl"] - 8)) & 0xFF) != 69 for c in L["codes"]]))
    for p in (float(x[3]), 69.0, 68.5, 200.0, -1.0, 255.0, 70.0):
        w, _, _ = oracle.range_filter_majority(buf, scale, p, oracle.BM_ROARING)
        assert np.array_equal(w, M.major_filter(L, p, True)), p
        w, _, _ = oracle.equal_filter_majority(buf, scale, p, oracle.BM_ROARING)
        assert np.array_equal(w, M.major_filter(L, p, False)), p
    s, _ = oracle.sum_majority(buf, scale, oracle.BM_ROARING)
    assert s == M.major_sum(L)
    _, mc, _, _ = oracle.max_majority(buf, scale, oracle.BM_ROARING)
    assert mc == M.major_max_code(L)


def test_outlieru8_panics(oracle):
    with pytest.raises(oracle.OraclePanic):  # fewer than 2000 rows
        oracle.encode_outlieru8(np.full(1999, 69.0), 10)
    with pytest.raises(oracle.OraclePanic):  # codes narrower than a byte: `remain -= 8` wraps
        oracle.encode_outlieru8(np.round(np.random.default_rng(1).uniform(0, 3, 3000), 0), 10)
