"""The comp_profiler driver mirror (buff_gb300/profiler.py): its input
parsing, sizes and output formats on the CPU, and one run of each arm on the
GPU against the oracle."""
import io
import os

import numpy as np
import pytest

from buff_gb300 import profiler as P


def test_rust_f64_tokens():
    ok = {"1.5": 1.5, "-2": -2.0, "1e3": 1000.0, ".5": 0.5, "1.": 1.0, "+3": 3.0,
          "2.5E-2": 0.025, "-0": -0.0}
    for tok, v in ok.items():
        assert P.parse_rust_f64(tok) == v, tok
    for tok in ("inf", "-Infinity", "+INF"):
        assert np.isinf(P.parse_rust_f64(tok)), tok
    assert np.isnan(P.parse_rust_f64("NaN"))
    for tok in ("", " 1", "1 ", "1_0", "abc", "1e", "0x10", ".", "e5", "1.2.3", "--1"):
        assert P.parse_rust_f64(tok) is None, tok


def test_read_values(tmp_path):
    f = tmp_path / "in.csv"
    f.write_bytes(b"0,1.5,x,-2\r\n\n3e1,, 4,5\n\xff\xfe,6\n7")
    got = P.read_values(str(f))
    assert got.tolist() == [0.0, 1.5, -2.0, 30.0, 5.0, 7.0]
    assert P.read_values(str(f), skip=1).tolist() == [1.5, -2.0, 5.0]


def test_read_values_reference_fixture(readme_input):
    from tests.golden.make_golden import load_fixture

    x = P.read_values(readme_input)
    assert x.size == 500000
    assert np.array_equal(x, load_fixture(readme_input))


def test_segment_size_and_formats():
    assert P.segment_byte_size(0) == 31
    assert P.segment_byte_size(500000) == 4000031
    dur = {999: "999ns", 1000: "1µs", 850_200: "850.2µs", 1_500_000: "1.5ms",
           1_234_567: "1.234567ms", 2_000_000_000: "2s", 1_000_000_001: "1.000000001s",
           61_250_000_000: "61.25s"}
    for ns, s in dur.items():
        assert P.rust_duration_debug(ns) == s, ns
    f = {2.0: "2", 1.1509: "1.1509", 1e-7: "0.0000001", 0.1 + 0.2: "0.30000000000000004",
         -0.5: "-0.5", 1e20: "100000000000000000000", float("nan"): "NaN", float("-inf"): "-inf"}
    for v, s in f.items():
        assert P.rust_f64_display(v) == s, v


def test_unknown_arm_rejected(tmp_path):
    f = tmp_path / "in.csv"
    f.write_text("1,2,3\n")
    with pytest.raises(ValueError):
        P.run(str(f), "buff-zip", 10, 1.0)
    with pytest.raises(SystemExit):
        P.main([str(f), "buff-simd", "10", "1.0 "])


def _csv(tmp_path, x, junk=True):
    lines = []
    for i in range(0, x.size, 1000):
        toks = [repr(float(v)) for v in x[i:i + 1000]]
        if junk and i % 3000 == 0:
            toks.insert(3, "n/a")
        lines.append(",".join(toks) + ",")
    f = tmp_path / "walk.csv"
    f.write_text("\n".join(lines) + "\n")
    return str(f)


def _perf_fields(text):
    line = [ln for ln in text.splitlines() if ln.startswith("Performance:")]
    assert len(line) == 1
    return line[0][len("Performance:"):].split(",")


@pytest.mark.gpu
@pytest.mark.parametrize("from_bytes", [False, True])
def test_profiler_arms(oracle, gpu, tmp_path, from_bytes):
    rng = np.random.default_rng(77)
    x = np.round(100 + np.cumsum(rng.uniform(-0.5, 0.5, 70_000)), 4)
    path = _csv(tmp_path, x)
    assert np.array_equal(P.read_values(path), x)
    scale, pred = 10000, float(np.quantile(x, 0.8))
    org = P.segment_byte_size(x.size)

    out = io.StringIO()
    r = P.run(path, "buff-simd", scale, pred, from_bytes, out)
    img = oracle.encode(x, scale)
    assert r["image"] == img and r["comp_size"] == len(img)
    f = _perf_fields(out.getvalue())
    assert len(f) == 10 and f[0] == path and f[1] == str(scale) and float(f[2]) == pred
    assert float(f[3]) == len(img) / org
    assert all(float(v) > 0 for v in f[4:])
    res = r["results"]
    assert np.array_equal(res["decode"], oracle.decode(img, scale))
    for name, fn in (("range", oracle.range_filter), ("equal", oracle.equal_filter),
                     ("range_with_slice", oracle.range_filter_with_slice),
                     ("equal_with_slice", oracle.equal_filter_with_slice)):
        words, cnt = fn(img, scale, pred)[:2]
        assert res[name].count == cnt and np.array_equal(res[name].words, words), name

    out = io.StringIO()
    r = P.run(path, "buff-slice", scale, pred, from_bytes, out)
    img = oracle.slice_encode(x, scale)
    assert r["image"] == img
    res = r["results"]
    assert np.array_equal(res["decode"], oracle.slice_decode(img, scale))
    words, cnt = oracle.slice_range_filter(img, scale, pred)[:2]
    assert res["range"].count == cnt and np.array_equal(res["range"].words, words)
    assert res["buffsum"] == oracle.slice_sum(img, scale, True)
    assert res["buffmax"].value == oracle.slice_max(img, scale, True)[0]
    assert len(_perf_fields(out.getvalue())) == 10

    # the `buff` arm: the buff-layout image and the scalar filters
    out = io.StringIO()
    r = P.run(path, "buff", scale, pred, from_bytes, out)
    img = oracle.encode(x, scale, flipped=False)
    assert r["image"] == img
    text = out.getvalue()
    assert text.splitlines()[0] == "no min/max"
    assert "Time elapsed in splitbd byte range filter function() is:" in text
    res = r["results"]
    assert np.array_equal(res["decode"], oracle.decode(img, scale, flipped=False))
    for name, fn in (("range", oracle.scalar_range_filter), ("equal", oracle.scalar_equal_filter)):
        words, cnt = fn(img, scale, pred)[:2]
        assert res[name].count == cnt and np.array_equal(res[name].words, words), name
    assert res["sum"] == oracle.buff_sum(img, scale, flipped=False)[0]
    mv, mc, aw, ac = oracle.buff_max(img, scale, flipped=False)
    assert res["max"].value == mv and res["max"].argmax_count == ac
    assert len(_perf_fields(text)) == 10

    # the `buff-slice-scalar` arm: decode_bs, the row-by-row filters, sum, max
    out = io.StringIO()
    r = P.run(path, "buff-slice-scalar", scale, pred, from_bytes, out)
    img = oracle.slice_encode(x, scale)
    assert r["image"] == img
    res = r["results"]
    assert np.array_equal(res["decode"], oracle.slice_decode_bs(img, scale))
    for name, fn in (("range", oracle.slice_range_filter_nosimd),
                     ("equal", oracle.slice_equal_filter_nosimd)):
        words, cnt = fn(img, scale, pred)[:2]
        assert res[name].count == cnt and np.array_equal(res[name].words, words), name
    assert res["sum"] == oracle.slice_sum(img, scale)
    assert res["max"].value == oracle.slice_max(img, scale)[0]
    assert len(_perf_fields(out.getvalue())) == 10

    out = io.StringIO()
    r = P.run(path, "buff-major", scale, pred, from_bytes, out)
    img = r["image"]
    res = r["results"]
    assert np.array_equal(res["decode"], oracle.decode_majority(img, scale))
    words, cnt = oracle.range_filter_majority(img, scale, pred)[:2]
    assert res["range"].count == cnt and np.array_equal(res["range"].words, words)
    assert res["sum"] == oracle.sum_majority(img, scale)[0]
    assert len(_perf_fields(out.getvalue())) == 10
