"""GPU parity at the benchmark configurations' full sizes, against the oracle
bit for bit, and on the reference's own README input.

- 1,000,000-row Gaussian walk (scale 10^4): the six operations of the
  reference's profiler run (encode, equality on a value drawn from the
  column, range at the 90th percentile, sum, max, full decode).
- 268,435,456-row bounded walk (scale 10^4, 25-bit codes): the byte image,
  range filters at 0.1 / 1 / 10 / 50 % selectivity (alone and in the one-pass
  filter + sum), equality on a drawn value, the f64 sum bit pattern and its
  partials, max with its arg-max bitmap, and decode at full precision and at
  1, 2 and 4 decimals.
- 67,108,864-row outlier column (1 % of rows in +-1e6, scale 10^6): the
  buff-major image with raw bitmaps and every buff_*_majority query; the
  plain image of the same values.
- randomwalkdatasample1k-1k (the reference README's input; scale 10000,
  pred 1.1509): every query against the oracle and against the committed
  digests in tests/golden/fixture_digest.json.
"""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _sha(a) -> str:
    if isinstance(a, np.ndarray):
        a = np.ascontiguousarray(a).tobytes()
    return hashlib.sha256(a).hexdigest()


def _same_words(got, want):
    return np.array_equal(np.asarray(got, dtype=np.uint32), np.asarray(want, dtype=np.uint32))


def _check_sum(oracle, col, ref, scale):
    s, parts, exact = oracle.buff_sum(ref, scale)
    g = col.sum()
    assert g.sum.hex() == s.hex()
    assert list(g.partials[: g.n_partials]) == parts
    assert g.exact_num == exact
    return g


def _check_max(oracle, col, ref, scale):
    mv, mc, aw, ac = oracle.buff_max(ref, scale)
    g = col.max(argmax=True)
    assert g.value.hex() == mv.hex() and g.code == mc
    assert _same_words(g.argmax_words, aw) and g.argmax_count == ac


def test_profiler_column_one_million(oracle, gpu):
    """The 1,000,000-value Gaussian walk at scale 10^4."""
    from buff_gb300 import Column
    from buff_gb300.workloads import gaussian_walk

    x = gaussian_walk(1_000_000, seed=1)
    ref = oracle.encode(x, 10000)
    col = Column.encode(x, 10000)
    assert col.serialize() == ref
    rng = np.random.default_rng(1)
    drawn = float(x[int(rng.integers(0, x.size))])
    w, c, _ = oracle.equal_filter(ref, 10000, drawn)
    g = col.equal_filter(drawn)
    assert _same_words(g.words, w) and g.count == c
    q90 = float(np.quantile(x, 0.9))
    w, c, _ = oracle.range_filter(ref, 10000, q90)
    g = col.range_filter(q90)
    assert _same_words(g.words, w) and g.count == c
    _check_sum(oracle, col, ref, 10000)
    _check_max(oracle, col, ref, 10000)
    assert np.array_equal(col.decode(), oracle.decode(ref, 10000))


@pytest.mark.slow
def test_bounded_walk_full_size_bit_exact(oracle, gpu):
    """The 268,435,456-row bounded walk, every result against the oracle."""
    import torch

    from buff_gb300 import Column
    from buff_gb300.workloads import bounded_walk_torch

    n = 1 << 28
    xd = bounded_walk_torch(n, seed=2)
    x = xd.cpu().numpy()
    col = Column.encode(xd, 10000)
    del xd
    torch.cuda.empty_cache()
    ref = oracle.encode(x, 10000)
    inf = col.info
    assert inf.fixed_len == 25 and inf.k == 3 and inf.r == 1
    assert col.serialize() == ref
    sample = x[:: 1 << 8]
    for sel in (0.001, 0.01, 0.1, 0.5):
        p = float(np.quantile(sample, 1.0 - sel))
        w, c, _ = oracle.range_filter(ref, 10000, p)
        assert 0.5 * sel * n < c < 2.0 * sel * n
        g = col.range_filter(p)
        assert _same_words(g.words, w) and g.count == c, sel
        fr, fs = col.range_filter_sum(p)
        assert _same_words(fr.words, w) and fr.count == c, sel
    drawn = float(x[n // 3])
    w, c, _ = oracle.equal_filter(ref, 10000, drawn)
    g = col.equal_filter(drawn)
    assert c > 0 and _same_words(g.words, w) and g.count == c
    s = _check_sum(oracle, col, ref, 10000)
    assert fs.sum.hex() == s.sum.hex() and fs.exact_num == s.exact_num
    _check_max(oracle, col, ref, 10000)
    del x, sample
    got = col.decode()
    assert np.array_equal(got, oracle.decode(ref, 10000))
    del got
    for p in (1, 2, 4):
        got = col.decode_at_precision(p)
        assert np.array_equal(got, oracle.decode_at_precision(ref, 10000, p)), p
        del got


@pytest.mark.slow
def test_outlier_column_full_size_bit_exact(oracle, gpu):
    """The 67,108,864-row outlier column: buff-major image (raw bitmaps) and
    every majority query, then the plain image of the same values."""
    import torch

    from buff_gb300 import Column
    from buff_gb300.compress import FLAG_RAW_BITMAPS, MajorColumn
    from buff_gb300.workloads import outlier_column_torch

    raw = 1
    n, scale = 1 << 26, 1000000
    xd = outlier_column_torch(n, seed=3)
    x = xd.cpu().numpy()
    col = MajorColumn.encode(xd, scale, FLAG_RAW_BITMAPS)
    ref = oracle.encode_majority(x, scale, raw)
    assert col.serialize() == ref
    ncols, majors, nouts, _ = oracle.majority_layout(ref, raw)
    assert col.info.outlier_cols == ncols == 1 and all(nouts)
    sample = x[:: 1 << 6]
    preds = [float(np.quantile(sample, 1.0 - s)) for s in (0.001, 0.01, 0.1, 0.5)]
    outl = x[np.abs(x - 100.0) > 1000.0]
    preds += [float(outl[len(outl) // 2]), float(x.max()), float(x.min()) - 1.0]
    for p in preds:
        w, c, _ = oracle.range_filter_majority(ref, scale, p, raw)
        g = col.range_filter(p)
        assert _same_words(g.words, w) and g.count == c, ("range", p)
    for p in (float(x[n // 3]), float(outl[3]), float(np.median(sample))):
        w, c, _ = oracle.equal_filter_majority(ref, scale, p, raw)
        g = col.equal_filter(p)
        assert _same_words(g.words, w) and g.count == c, ("equal", p)
    s, parts = oracle.sum_majority(ref, scale, raw)
    g = col.sum()
    assert g.sum.hex() == s.hex()
    assert list(g.partials[: g.n_partials]) == parts[: g.n_partials]
    mv, mc, aw, ac = oracle.max_majority(ref, scale, raw)
    m = col.max(argmax=True)
    assert m.value.hex() == mv.hex() and m.code == mc
    assert _same_words(m.argmax_words, aw) and m.argmax_count == ac
    # the device-only sum and max, and the max value without its arg-max rows
    from tests.test_gpu_major import _check_async

    _check_async(col, s, parts[: g.n_partials], mc)
    assert np.array_equal(col.decode(), oracle.decode_majority(ref, scale, raw))
    col.free()
    # the plain (buff-simd) image of the same column
    plain = Column.encode(xd, scale)
    del xd
    torch.cuda.empty_cache()
    pref = oracle.encode(x, scale)
    assert plain.serialize() == pref
    w, c, _ = oracle.range_filter(pref, scale, preds[2])
    g = plain.range_filter(preds[2])
    assert _same_words(g.words, w) and g.count == c
    _check_sum(oracle, plain, pref, scale)
    _check_max(oracle, plain, pref, scale)


def test_readme_input_on_gpu(oracle, gpu, readme_input):
    """randomwalkdatasample1k-1k at scale 10000 with pred 1.1509 (the
    reference README's quick start): every query equals the oracle's, and the
    oracle equals the committed digests."""
    from buff_gb300 import Column
    from buff_gb300.compress import filter_image, range_filter_sum_image
    from tests.golden.make_golden import load_fixture

    with open(os.path.join(HERE, "golden", "fixture_digest.json")) as f:
        want = json.load(f)
    scale, pred = 10000, 1.1509
    x = load_fixture(readme_input)
    assert x.size == want["n"] == 500000
    ref = oracle.encode(x, scale)
    assert _sha(ref) == want["sha256"]
    col = Column.encode(x, scale)
    img = col.serialize()
    assert img == ref
    for name, fn in (("range", col.range_filter), ("equal", col.equal_filter),
                     ("range_with_slice", col.range_filter_with_slice),
                     ("equal_with_slice", col.equal_filter_with_slice)):
        g = fn(pred)
        words = np.asarray(g.words, dtype=np.uint32)
        assert g.count == want[name]["count"], name
        assert _sha(words) == want[name]["sha256"], name
    hi = filter_image(np.frombuffer(ref, dtype=np.uint8), scale, pred)
    assert hi.count == want["range"]["count"]
    assert _sha(np.asarray(hi.words, dtype=np.uint32)) == want["range"]["sha256"]
    g = col.sum()
    assert g.sum.hex() == float.fromhex(want["sum"]).hex()
    assert list(g.partials[: g.n_partials]) == want["sum_partials"]
    assert g.exact_num == int(want["sum_exact_num"])
    fr, fs = range_filter_sum_image(np.frombuffer(ref, dtype=np.uint8), scale, pred)
    assert fr.count == want["range"]["count"] and fs.sum == g.sum
    m = col.max(argmax=True)
    assert m.value.hex() == float.fromhex(want["max"]).hex()
    assert m.code == want["max_code"] and m.argmax_count == want["argmax_count"]
    assert _sha(col.decode()) == want["decode_sha256"]
    for p in (1, 2, 3, 4):
        assert _sha(col.decode_at_precision(p)) == want[f"decode_p{p}_sha256"], p
