"""GPU parity: every entry point of the C ABI against the CPU oracle (the
reference algorithm) on the same seeded inputs, bit for bit; the committed
golden vectors; and size-independent properties at the full benchmark size.
"""
import ctypes as C

import numpy as np
import pytest

from tests import model as M

pytestmark = pytest.mark.gpu


def words_equal(a, b):
    return np.array_equal(np.asarray(a, dtype=np.uint32), np.asarray(b, dtype=np.uint32))


def gen(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "walk":
        return np.round(1.0 + np.cumsum(rng.normal(0, 0.3, n)), 4)
    if kind == "walk_neg":
        return np.round(-40.0 + np.cumsum(rng.normal(0, 0.05, n)), 3)
    if kind == "narrow":
        return np.round(rng.uniform(3.0, 3.06, n), 2)
    if kind == "wide":
        return np.round(rng.normal(100, 5, n), 6)
    if kind == "huge":  # wide codes: 7-8 slices
        return np.round(rng.uniform(-1e6, 1e6, n), 9)
    if kind == "updown":
        x = np.round(np.cumsum(rng.normal(0, 1, n)), 3)
        if n:
            x[0] = x.max() + 3
        return x
    if kind == "decreasing":  # long strictly decreasing prefix
        x = np.round(np.cumsum(rng.normal(0, 1, n)), 3)
        m = min(n, 700)
        x[:m] = np.round(1000.0 - np.arange(m) * 0.5, 3)
        return x
    if kind == "tiny":  # magnitudes whose quantizer shift wraps at 13-15 decimals
        return np.round(rng.normal(0, 1e-6, n), 14)
    if kind == "clustered":  # many equal prefixes -> deep refinement
        base = np.round(rng.uniform(0, 1, n // 64 + 1), 4)
        return np.repeat(base, 64)[:n] + np.round(rng.uniform(0, 1e-3, n), 6)
    raise ValueError(kind)


CASES = [
    ("walk", 100000, 10000), ("walk", 99999, 10000), ("walk", 4097, 100), ("walk", 31, 1000),
    ("walk", 1, 1000), ("walk", 2, 1000), ("walk", 33, 10), ("walk_neg", 50000, 1000),
    ("narrow", 20000, 100), ("narrow", 777, 10), ("wide", 65536, 1000000),
    ("wide", 12345, 100000000), ("huge", 30000, 1000000000), ("updown", 10000, 1000),
    ("decreasing", 5000, 1000), ("clustered", 70000, 1000000), ("walk", 5000, 10 ** 13),
    ("walk", 3000, 10 ** 12), ("tiny", 4000, 10 ** 14),
]


def _pred_list(x):
    if x.size == 0:
        return [0.0]
    return [float(x[x.size // 3]), float(x[0]), float(x.max()), float(x.min()),
            float(np.quantile(x, 0.9)), float(np.quantile(x, 0.999)), float(x.max()) + 1.0,
            float(x.min()) - 1.0, float(np.quantile(x, 0.5)) + 1e-7]


def _encode_both(oracle, x, scale, flags):
    from buff_gb300 import Column, ReferencePanic

    try:
        ref = oracle.encode(x, scale, True, flags)
    except oracle.OraclePanic:
        with pytest.raises(ReferencePanic):
            Column.encode(x, scale, flags)
        return None, None
    col = Column.encode(x, scale, flags)
    return ref, col


@pytest.mark.parametrize("kind,n,scale", CASES)
@pytest.mark.parametrize("intended", [0, 1])
def test_column_parity(gpu, oracle, kind, n, scale, intended):
    from buff_gb300 import ReferencePanic

    x = gen(kind, n, 1000 + n)
    ref, col = _encode_both(oracle, x, scale, intended)
    if ref is None:
        return
    # encode: byte-identical reference image
    assert col.serialize() == ref
    # decode
    assert np.array_equal(col.decode(), oracle.decode(ref, scale))
    # filters
    for p in _pred_list(x):
        for name in ("range_filter", "equal_filter"):
            w, c, _ = getattr(oracle, name)(ref, scale, p, intended)
            g = getattr(col, name)(p)
            assert words_equal(g.words, w), (name, p)
            assert g.count == c
        for name in ("range_filter_with_slice", "equal_filter_with_slice"):
            if intended:
                continue
            try:
                w, c, _ = getattr(oracle, name)(ref, scale, p)
            except oracle.OraclePanic:
                with pytest.raises(ReferencePanic):
                    getattr(col, name)(p)
                continue
            g = getattr(col, name)(p)
            assert words_equal(g.words, w), (name, p)
            assert g.count == c
    # sum: the reference's f64 bit for bit, and the exact integer
    s, parts, exact = oracle.buff_sum(ref, scale, True, intended)
    r = col.sum()
    assert r.sum == s or (np.isnan(r.sum) and np.isnan(s))
    # the range filter and the sum from one pass
    for p in _pred_list(x):
        w, c, _ = oracle.range_filter(ref, scale, p, intended)
        fr, fs = col.range_filter_sum(p)
        assert words_equal(fr.words, w) and fr.count == c, ("one pass", p)
        assert fs.sum == s or (np.isnan(fs.sum) and np.isnan(s))
        assert fs.exact_num == exact
    assert list(r.partials[: r.n_partials]) == parts
    assert r.exact_num == exact
    # max (+ arg-max bitmap)
    mv, mc, aw, ac = oracle.buff_max(ref, scale, True, intended)
    g = col.max(argmax=True)
    assert g.code == mc and (g.value == mv or (np.isnan(g.value) and np.isnan(mv)))
    assert words_equal(g.argmax_words, aw) and g.argmax_count == ac
    # precision-limited decode and sum
    for p in range(0, 16):
        try:
            want = oracle.decode_at_precision(ref, scale, p, True, intended)
        except oracle.OraclePanic:
            with pytest.raises(ReferencePanic):
                col.decode_at_precision(p)
            continue
        assert np.array_equal(col.decode_at_precision(p), want), p
        want_s = oracle.sum_at_precision(ref, scale, p, True, intended)
        assert col.sum_at_precision(p) == want_s, p


def test_gaussian_walk_million(gpu, oracle):
    """The 1,000,000-row CPU-runnable workload (gaussian walk, x0 = 1, steps
    N(0, 0.01), 4 decimals, seed 1, scale 10^4): every op against the oracle."""
    from buff_gb300.compress import Column
    from buff_gb300.workloads import gaussian_walk

    x = gaussian_walk(1_000_000, seed=1)
    ref = oracle.encode(x, 10000)
    col = Column.encode(x, 10000)
    assert col.serialize() == ref
    assert np.array_equal(col.decode(), oracle.decode(ref, 10000))
    idx = int(np.random.default_rng(1).integers(0, x.size))
    for name, p in (("equal_filter", float(x[idx])), ("range_filter", float(np.quantile(x, 0.9)))):
        w, c, _ = getattr(oracle, name)(ref, 10000, p)
        g = getattr(col, name)(p)
        assert words_equal(g.words, w) and g.count == c, name
    s, parts, exact = oracle.buff_sum(ref, 10000, True)
    r = col.sum()
    assert r.sum == s and r.exact_num == exact
    mv, mc, aw, ac = oracle.buff_max(ref, 10000, True)
    g = col.max(argmax=True)
    assert g.code == mc and g.value == mv and words_equal(g.argmax_words, aw)
    for p in (1, 2, 4):
        assert np.array_equal(col.decode_at_precision(p),
                              oracle.decode_at_precision(ref, 10000, p, True))


def test_golden_vectors(gpu):
    import os

    from buff_gb300 import Column

    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "vectors.npz"))
    names = sorted({k.split(".")[0] for k in z.files})
    assert names
    for nm in names:
        x, scale = z[f"{nm}.x"], int(z[f"{nm}.scale"][0])
        col = Column.encode(x, scale)
        assert col.serialize() == z[f"{nm}.bytes"].tobytes(), nm
        assert np.array_equal(col.decode(), z[f"{nm}.decode"]), nm
        for j, p in enumerate(z[f"{nm}.preds"]):
            assert words_equal(col.range_filter(float(p)).words, z[f"{nm}.range{j}"]), (nm, j)
            assert words_equal(col.equal_filter(float(p)).words, z[f"{nm}.equal{j}"]), (nm, j)
        assert col.sum().sum == z[f"{nm}.sum"][0]
        m = col.max()
        assert m.value == z[f"{nm}.max"][0] and m.code == int(z[f"{nm}.max_code"][0])


def test_deserialize_reference_image(gpu, oracle):
    from buff_gb300 import Column, SplitBDDoubleCompress

    x = gen("walk", 54321, 5)
    ref = oracle.encode(x, 10000)
    comp = SplitBDDoubleCompress(10, 10, 10000)
    col = Column.deserialize(ref, 10000)
    assert col.serialize() == ref
    p = float(np.quantile(x, 0.7))
    w, c, _ = oracle.range_filter(ref, 10000, p)
    # the mirror accepts the byte image like the reference's Vec<u8>
    g = comp.buff_simd_range_filter(ref, p)
    assert words_equal(g.words, w) and g.count == c
    assert np.array_equal(comp.buff_simd256_decode(ref), oracle.decode(ref, 10000))
    assert comp.byte_fixed_sum(ref) == oracle.buff_sum(ref, 10000)[0]


def test_corrupt_image_rejected(gpu, oracle):
    from buff_gb300 import BuffError, Column

    ref = oracle.encode(gen("walk", 1000, 9), 10000)
    with pytest.raises(BuffError):
        Column.deserialize(ref[:-5], 10000)


def test_f32_input(gpu, oracle):
    from buff_gb300 import Column

    x = gen("walk", 30001, 3).astype(np.float32)
    ref = oracle.encode(x, 1000)
    col = Column.encode(x, 1000)
    assert col.serialize() == ref


def test_nonfinite_and_special_values(gpu, oracle):
    from buff_gb300 import Column

    x = gen("walk", 20000, 6)
    x[[5, 700, 19999]] = [np.inf, -np.inf, np.nan]
    x[[9, 10]] = [0.0, -0.0]
    for scale in (10000, 10 ** 14):
        try:
            ref = oracle.encode(x, scale)
        except oracle.OraclePanic:
            continue
        assert Column.encode(x, scale).serialize() == ref
    xf = gen("walk", 9000, 7).astype(np.float32)
    xf[[3, 4, 5]] = [np.float32(1e-42), np.float32(-3e-45), np.float32(-0.0)]
    xf[[6, 7]] = [np.float32(np.inf), np.float32(-2.5e38)]
    ref = oracle.encode(xf, 1000)
    assert Column.encode(xf, 1000).serialize() == ref


def test_empty_column(gpu, oracle):
    from buff_gb300 import Column

    x = np.zeros(0)
    ref = oracle.encode(x, 10000)
    col = Column.encode(x, 10000)
    assert col.serialize() == ref and len(ref) == 20
    assert col.decode().size == 0
    assert col.range_filter(1.0).count == 0


def test_device_pointers_and_alignment(gpu, oracle):
    import torch

    from buff_gb300 import Column

    x = gen("wide", 40000, 4)
    ref = oracle.encode(x, 1000000)
    t = torch.from_numpy(np.concatenate([[0.0], x])).cuda()
    col_a = Column.encode(t[1:], 1000000)  # 8-byte aligned device view
    assert col_a.serialize() == ref
    col = Column.encode(t[1:].clone(), 1000000)
    assert col.serialize() == ref
    n = x.size
    # device outputs
    words = torch.zeros((n + 31) // 32, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    from buff_gb300 import capi

    p = float(np.quantile(x, 0.4))
    capi.check(capi.lib().buff_range_filter(col.handle, p, capi.ptr(words), capi.ptr(cnt), None))
    torch.cuda.synchronize()
    w, c, _ = oracle.range_filter(ref, 1000000, p)
    assert words_equal(words.cpu().numpy().view(np.uint32), w) and int(cnt.item()) == c
    out = torch.empty(n + 1, dtype=torch.float64, device="cuda")
    col.decode(out=out[1:])  # misaligned device output
    torch.cuda.synchronize()
    assert np.array_equal(out[1:].cpu().numpy(), oracle.decode(ref, 1000000))
    # device serialize/deserialize
    img = torch.empty(len(ref), dtype=torch.uint8, device="cuda")
    col.serialize(out=img)
    assert img.cpu().numpy().tobytes() == ref
    col2 = Column.deserialize(img, 1000000)
    assert col2.serialize() == ref


def test_async_partials_on_stream(gpu, oracle):
    import torch

    from buff_gb300 import Column, capi

    x = gen("walk", 200000, 8)
    ref = oracle.encode(x, 10000)
    col = Column.encode(x, 10000)
    s = torch.cuda.Stream()
    parts = torch.zeros(9, dtype=torch.int64, device="cuda")
    mx = torch.zeros(1, dtype=torch.int64, device="cuda")
    with torch.cuda.stream(s):
        capi.check(capi.lib().buff_sum_partials_async(col.handle, capi.ptr(parts), s.cuda_stream))
        capi.check(capi.lib().buff_max_async(col.handle, capi.ptr(mx), s.cuda_stream))
    s.synchronize()
    host = np.ascontiguousarray(parts.cpu().numpy().view(np.uint64))
    res = capi.SumResult()
    capi.check(capi.lib().buff_sum_finish(col.handle, host.ctypes.data, C.byref(res)))
    assert res.sum == oracle.buff_sum(ref, 10000)[0]
    assert int(mx.item()) == oracle.buff_max(ref, 10000)[1]


@pytest.mark.slow
def test_full_size_properties(gpu):
    """268,435,456-row bounded walk (the benchmark column): decode round trip,
    filter counts, exact sum and max against torch on the quantized values."""
    import torch

    from buff_gb300 import Column
    from buff_gb300.workloads import bounded_walk_torch

    n = 1 << 28
    x = bounded_walk_torch(n, seed=2)
    q = torch.trunc(x * 32768.0).to(torch.int64)  # exact: |x| <= 500
    col = Column.encode(x, 10000)
    inf = col.info
    base = int(q.min().item())
    assert inf.base == base and inf.fixed_len == 25 and inf.k == 3 and inf.r == 1
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    col.decode(out=out)
    assert torch.equal(out, q.to(torch.float64) / 32768.0)
    del out
    for sel in (0.001, 0.01, 0.1, 0.5):
        p = float(torch.quantile(x[:: 1 << 8], 1.0 - sel).item())
        t = int(np.trunc(p * 32768.0)) - base
        g = col.range_filter(p)
        assert g.count == int(((q - base) > t).sum().item())
        e = col.equal_filter(p)
        assert e.count == int(((q - base) == t).sum().item())
    s = col.sum()
    assert s.exact_num == int(q.sum().item())
    fr, fs = col.range_filter_sum(p)
    assert fr.count == g.count and np.array_equal(fr.words, g.words)
    assert fs.exact_num == s.exact_num and fs.sum == s.sum
    assert col.max().code == int(q.max().item()) - base


@pytest.mark.parametrize("offset,scale,n", [(0.0, 10000, 300_017), (1e6, 10000, 300_017),
                                            (-3e5, 1000, 65_539), (0.0, 100, 100_000),
                                            (50.0, 10, 4_099)])
def test_decode_paths_and_output_alignment(oracle, gpu, offset, scale, n):
    """Full and precision decodes through every output placement (host,
    32-byte and 16-byte aligned device buffers), with codes that carry tail
    bits and bases inside and outside the 32-bit range."""
    import torch

    from buff_gb300.compress import Column

    rng = np.random.default_rng(n)
    x = np.round(offset + np.cumsum(rng.uniform(-0.5, 0.5, n)), 4)
    img = oracle.encode(x, scale)
    col = Column.encode(x, scale)
    assert col.serialize() == img
    want = oracle.decode(img, scale)
    assert np.array_equal(col.decode(), want)
    buf = torch.empty(n + 4, dtype=torch.float64, device="cuda")
    for shift in (0, 2):  # 32-byte aligned, then 16-byte aligned
        o = buf[shift: shift + n]
        col.decode(out=o)
        assert np.array_equal(o.cpu().numpy(), want), shift
    for p in range(0, 5):
        try:
            want_p = oracle.decode_at_precision(img, scale, p)
        except oracle.OraclePanic:
            continue
        assert np.array_equal(col.decode_at_precision(p), want_p), p
        o = buf[2: 2 + n]
        col.decode_at_precision(p, out=o)
        assert np.array_equal(o.cpu().numpy(), want_p), p
