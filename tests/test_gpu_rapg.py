"""GPU parity of the RAPG byte_residue layout (compress/split_double.rs:
624-2630) against the oracle: the image from the GPU encode and after a
round trip through buff_rapg_deserialize byte for byte, and the full and
precision-limited decodes and sums on both handles, panics included."""
import numpy as np
import pytest

from tests.test_oracle_rapg import rapg_cases

pytestmark = pytest.mark.gpu


def _cases():
    rng = np.random.default_rng(17)
    big = np.round(rng.normal(100, 5, 300_001), 6)           # one sparse byte, bitset/run rows
    pos = np.nonzero(rng.uniform(size=big.size) < 0.01)[0]
    big[pos] = np.round(rng.uniform(1e5, 1e6, pos.size), 6)
    runs = np.round(rng.normal(100, 0.5, 200_003), 6)         # two sparse bytes, clustered rows
    runs[70_000:74_000] = np.round(rng.uniform(1e4, 1e6, 4000), 6)
    runs[150_000:150_050] = 5e5
    narrow = np.round(rng.uniform(3.0, 3.06, 5000), 2)        # codes narrower than dlen
    narrow0 = narrow.copy()                                     # ... whose first packed byte is 0
    narrow0[:2] = 3.0
    narrow0[2:] = np.maximum(narrow0[2:], 3.01)
    tenth = np.round(rng.uniform(0.0, 1.9, 4097), 1)          # scale 10: packed codes, no count byte
    tiny = np.array([0.1, 0.5, 1.2])
    f32 = np.round(rng.normal(10, 3, 50_001), 2).astype(np.float32)
    # codes wider than 52 bits: values past 2^53 / 2^dlen, where the decode
    # rounds and outlier rows are rebuilt from the slices, not patched
    wide = np.round(rng.normal(3e6, 50, 20_011), 9)
    pos = np.nonzero(rng.uniform(size=wide.size) < 0.01)[0]
    wide[pos] = np.round(rng.uniform(1e8, 4e9, pos.size), 9)
    # one sparse byte (the first 2,000 rows decide) with 512-row chunks that
    # are outliers throughout or in half their rows: chunks whose outlier
    # bytes exceed one 128-byte window of the decode
    dense = np.round(rng.normal(100, 5, 60_001), 6)
    pos = np.nonzero(rng.uniform(size=dense.size) < 0.01)[0]
    pos = np.concatenate([pos, np.arange(5_000, 9_000), 30_000 + np.nonzero(
        rng.uniform(size=30_001) < 0.5)[0]])
    dense[pos] = np.round(rng.uniform(1e5, 1e6, pos.size), 6)
    return rapg_cases() + [("big", big, 1000000), ("dense_runs", dense, 1000000),
                           ("runs", runs, 1000000),
                           ("narrow", narrow, 100), ("narrow0", narrow0, 100),
                           ("tenth", tenth, 10), ("tiny", tiny, 10),
                           ("f32", f32, 100), ("wide_codes", wide, 10 ** 9)]


CASES = _cases()


def _check(oracle, col, img, scale, name):
    from buff_gb300 import capi

    for p in [None] + list(range(16)):
        prec = -1 if p is None else p
        try:
            want = oracle.rapg_decode(img, scale, prec)
        except oracle.OraclePanic:
            with pytest.raises(capi.ReferencePanic):
                col.decode() if p is None else col.decode_at_precision(p)
            with pytest.raises(capi.ReferencePanic):
                col.rapg_sum(p)
            continue
        got = col.decode() if p is None else col.decode_at_precision(p)
        assert got.size == want.size and np.array_equal(got, want), (name, p)
        want_s = oracle.rapg_sum(img, scale, prec)
        got_s = col.rapg_sum(p)
        assert got_s == want_s or (np.isnan(got_s) and np.isnan(want_s)), (name, p)


@pytest.mark.parametrize("case", range(len(CASES)))
def test_rapg_parity(oracle, gpu, case):
    from buff_gb300 import capi
    from buff_gb300.compress import RapgColumn

    name, x, scale = CASES[case]
    xd = np.asarray(x, dtype=np.float64)
    try:
        img = oracle.rapg_encode(xd, scale)
    except oracle.OraclePanic:
        with pytest.raises(capi.ReferencePanic):
            RapgColumn.encode(x, scale)
        return
    col = RapgColumn.encode(x, scale)
    assert col.serialize() == img, name
    try:
        cols = oracle.rapg_layout(img)[0]
    except oracle.OraclePanic:  # packed codes read as a column directory
        cols = 0
    assert col.info.outlier_cols == cols
    back = RapgColumn.deserialize(img, scale)
    assert back.serialize() == img
    _check(oracle, col, img, scale, name)
    _check(oracle, back, img, scale, name + "/image")


def test_rapg_device_input_and_output(oracle, gpu):
    import torch

    from buff_gb300.compress import RapgColumn

    name, x, scale = CASES[6]
    img = oracle.rapg_encode(x, scale)
    col = RapgColumn.encode(torch.from_numpy(x).cuda(), scale)
    assert col.serialize() == img
    out = torch.empty(x.size, dtype=torch.float64, device="cuda")
    _, k = col.decode(out=out)
    assert k == x.size and np.array_equal(out.cpu().numpy(), oracle.rapg_decode(img, scale))
    odd = torch.empty(x.size + 1, dtype=torch.float64, device="cuda")  # 8-byte aligned view
    _, k = col.decode(out=odd[1:])
    assert np.array_equal(odd[1:].cpu().numpy(), oracle.rapg_decode(img, scale))
    dimg = torch.from_numpy(np.frombuffer(img, dtype=np.uint8).copy()).cuda()
    back = RapgColumn.deserialize(dimg, scale)
    assert back.serialize() == img


def test_rapg_errors(oracle, gpu):
    from buff_gb300 import capi
    from buff_gb300.compress import Column, RapgColumn

    name, x, scale = CASES[2]  # one sparse byte
    img = oracle.rapg_encode(x, scale)
    for bad in (img[:-1], img + b"\x00", img[:30]):
        with pytest.raises(capi.BuffError) as e:
            RapgColumn.deserialize(bad, scale)
        assert e.value.status == capi.ECORRUPT
    col = RapgColumn.encode(x, scale)
    for fn in (lambda: Column.decode(col), lambda: Column.range_filter(col, 1.0),
               lambda: Column.sum(col)):
        with pytest.raises(capi.BuffError) as e:
            fn()
        assert e.value.status == capi.ENOTSUP
    import ctypes as C

    plain = Column.encode(x, scale)
    out = np.empty(x.size, dtype=np.float64)
    k = C.c_uint64(0)
    v = C.c_double(0)
    L = capi.lib()
    assert L.buff_rapg_decode(plain.handle, out.ctypes.data, C.byref(k), None) == capi.ENOTSUP
    assert L.buff_rapg_sum(plain.handle, C.byref(v), None) == capi.ENOTSUP


# ---------------------------------------------------------------- RAPG-major

@pytest.mark.parametrize("ratio,n,scale", [(0.9, 5003, 10), (0.99, 300_001, 100),
                                           (0.5, 70_001, 1000), (0.999, 1_000_003, 10000)])
def test_rapg_major_parity(oracle, gpu, ratio, n, scale):
    """byte_residue_encode_outlieru8 image byte for byte from the GPU encode
    and after a deserialize round trip; every byte_residue_*_majority query
    against the oracle on both handles."""
    from buff_gb300.compress import RapgMajorColumn
    from tests.test_gpu_major import _check_queries
    from tests.test_oracle_rapg import outlieru8_case

    x, scale = outlieru8_case(ratio, n, 11, scale)
    img = oracle.encode_outlieru8(x, scale)
    col = RapgMajorColumn.encode(x, scale)
    assert col.serialize() == img
    assert col.info.outlier_cols == 1
    _check_queries(oracle, col, img, scale, oracle.BM_ROARING, x)
    back = RapgMajorColumn.deserialize(img, scale)
    assert back.serialize() == img
    _check_queries(oracle, back, img, scale, oracle.BM_ROARING, x)
    col32 = RapgMajorColumn.encode(x.astype(np.float32), scale)
    assert col32.serialize() == img


def test_rapg_major_errors(oracle, gpu):
    from buff_gb300 import capi
    from buff_gb300.compress import MajorColumn, RapgMajorColumn
    from tests.test_oracle_major import major_case
    from tests.test_oracle_rapg import outlieru8_case

    with pytest.raises(capi.ReferencePanic):
        RapgMajorColumn.encode(np.full(1999, 69.0), 10)
    with pytest.raises(capi.ReferencePanic):
        RapgMajorColumn.encode(np.round(np.random.default_rng(1).uniform(0, 3, 3000), 0), 10)
    x, scale = outlieru8_case(0.9, 5003, 3, 10)
    with pytest.raises(capi.ReferencePanic):  # outlier_exp's scale 0: no PRECISION_MAP entry
        RapgMajorColumn.encode(x, 0)
    with pytest.raises(oracle.OraclePanic):
        oracle.encode_outlieru8(x, 0)
    img = oracle.encode_outlieru8(x, scale)
    for bad in (img[:-1], img[:40]):
        with pytest.raises(capi.BuffError):
            RapgMajorColumn.deserialize(bad, scale)
    # a buff-major handle is not a RAPG-major one
    y, s2 = major_case("one", 5000, 3)
    plain = MajorColumn.encode(y, s2)
    out = np.empty(y.size, dtype=np.float64)
    assert capi.lib().buff_rapg_decode_majority(plain.handle, out.ctypes.data, None) == capi.ENOTSUP
    # images with two sparse columns are buff-major images, not RAPG-major ones
    y, s2 = major_case("two", 5000, 3)
    two = oracle.encode_majority(y, s2, oracle.BM_SNAPPY)
    with pytest.raises(capi.BuffError):
        RapgMajorColumn.deserialize(two, s2)
