"""buff_range_filter_sum_image: the range filter and sum read straight from a
serialized image (pageable host, pinned host or device memory), against the
oracle's filter and sum of the same image, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _walk(n, seed, step=0.5, dec=4):
    rng = np.random.default_rng(seed)
    return np.round(100 + np.cumsum(rng.uniform(-step, step, n)), dec)


# (values, scale): slice / tail splits k = 1..7, r = 0..7, ragged row counts
CASES = [
    ("walk_2p20", _walk(1 << 20, 1), 10000),           # fixed_len 25: k 3, r 1
    ("walk_ragged", _walk(100_003, 2), 10000),
    ("walk_4095", _walk(4095, 3), 10000),
    ("walk_4096", _walk(4096, 4), 10000),
    ("walk_4097", _walk(4097, 5), 10000),
    ("walk_31", _walk(31, 6), 10000),
    ("walk_33", _walk(33, 7), 10000),
    ("narrow_k1", np.round(np.random.default_rng(8).uniform(3, 40, 50_001), 1), 10),
    ("wide", np.round(np.random.default_rng(9).normal(100, 5, 70_000), 6), 1000000),
    ("huge", np.round(np.random.default_rng(10).uniform(-1e6, 1e6, 30_001), 9), 10 ** 9),
    ("r0", np.round(np.random.default_rng(11).uniform(0, 255.0, 9000), 1) , 10),
    ("f32", np.round(np.random.default_rng(12).normal(10, 3, 65_537), 2).astype(np.float32), 100),
]


def _expect(oracle, img, scale, pred):
    words, cnt = oracle.range_filter(img, scale, pred)[:2]
    s, parts, exact = oracle.buff_sum(img, scale)
    return words, cnt, s, parts


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("where", ["pageable", "pinned", "device"])
def test_image_query_matches_oracle(oracle, gpu, case, where):
    import torch

    from buff_gb300.compress import range_filter_sum_image

    name, x, scale = CASES[case]
    img = oracle.encode(x.astype(np.float64), scale)
    xs = np.sort(x.astype(np.float64))
    preds = [float(xs[len(xs) // 2]), float(xs[-1]), float(xs[0]) - 1.0,
             float(xs[int(len(xs) * 0.9)])]
    if where == "pageable":
        src = np.frombuffer(img, dtype=np.uint8).copy()
    elif where == "pinned":
        src = torch.frombuffer(bytearray(img), dtype=torch.uint8).pin_memory()
    else:
        src = torch.frombuffer(bytearray(img), dtype=torch.uint8).cuda()
    for pred in preds:
        words, cnt, s, parts = _expect(oracle, img, scale, pred)
        fr, sr = range_filter_sum_image(src, scale, pred)
        assert fr.count == cnt, (name, pred)
        assert np.array_equal(np.asarray(fr.words, dtype=np.uint32), words), (name, pred)
        assert sr.sum == s or (np.isnan(s) and np.isnan(sr.sum)), (name, pred)
        assert list(sr.partials[: sr.n_partials]) == parts, (name, pred)


@pytest.mark.parametrize("case", [0, 1, 4, 8])
def test_image_buff_layout_and_device_words(oracle, gpu, case):
    """The unflipped buff layout (BUFF_FLAG_BUFF_LAYOUT) gives the same
    results; bitmap words may be a device buffer."""
    import torch

    from buff_gb300.capi import FLAG_BUFF_LAYOUT
    from buff_gb300.compress import range_filter_sum_image

    name, x, scale = CASES[case]
    flipped = oracle.encode(x.astype(np.float64), scale)
    plain = oracle.encode(x.astype(np.float64), scale, flipped=False)
    pred = float(np.quantile(x, 0.3))
    words, cnt, s, parts = _expect(oracle, flipped, scale, pred)
    fr, sr = range_filter_sum_image(np.frombuffer(plain, dtype=np.uint8), scale, pred,
                                    flags=FLAG_BUFF_LAYOUT)
    assert fr.count == cnt and np.array_equal(fr.words, words) and sr.sum == s
    dw = torch.zeros(max((x.size + 31) // 32, 1), dtype=torch.int32, device="cuda")
    fr, sr = range_filter_sum_image(torch.frombuffer(bytearray(flipped), dtype=torch.uint8).cuda(),
                                    scale, pred, words=dw)
    assert fr.count == cnt and sr.sum == s
    assert np.array_equal(dw.cpu().numpy().view(np.uint32)[: words.size], words)


def test_image_matches_resident_call(gpu):
    """The one-pass image call and the resident column's one-pass call agree."""
    from buff_gb300.compress import Column, range_filter_sum_image

    x = _walk(3_000_001, 21)
    col = Column.encode(x, 10000)
    img = col.serialize()
    for q in (0.01, 0.5, 0.99):
        pred = float(np.quantile(x, q))
        f1, s1 = col.range_filter_sum(pred)
        f2, s2 = range_filter_sum_image(np.frombuffer(img, dtype=np.uint8), 10000, pred)
        assert f1.count == f2.count and np.array_equal(f1.words, f2.words)
        assert s1.sum == s2.sum and s1.exact == s2.exact


def test_image_errors(gpu):
    from buff_gb300 import capi
    from buff_gb300.compress import range_filter_sum_image

    with pytest.raises(capi.BuffError):
        range_filter_sum_image(b"\x00" * 10, 10000, 1.0)
    x = _walk(1000, 3)
    from buff_gb300.compress import Column

    img = Column.encode(x, 10000).serialize()
    with pytest.raises(capi.BuffError):  # truncated image
        range_filter_sum_image(img[:-5], 10000, 100.0)


KINDS = ["range", "equal", "range_with_slice", "equal_with_slice"]


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("where", ["pageable", "pinned", "device"])
def test_filter_image_matches_oracle(oracle, gpu, case, where):
    """The four filters on an image in place: bitmaps and counts as the
    oracle's (and the same panics), for every memory kind."""
    import torch

    from buff_gb300 import capi
    from buff_gb300.compress import filter_image

    name, x, scale = CASES[case]
    xd = x.astype(np.float64)
    img = oracle.encode(xd, scale)
    xs = np.sort(xd)
    preds = [float(xs[len(xs) // 2]), float(xs[-1]), float(xs[0]) - 1.0,
             float(xs[int(len(xs) * 0.9)]), float(xd[len(xd) // 3])]
    if where == "pageable":
        src = np.frombuffer(img, dtype=np.uint8).copy()
    elif where == "pinned":
        src = torch.frombuffer(bytearray(img), dtype=torch.uint8).pin_memory()
    else:
        src = torch.frombuffer(bytearray(img), dtype=torch.uint8).cuda()
    fns = {"range": oracle.range_filter, "equal": oracle.equal_filter,
           "range_with_slice": oracle.range_filter_with_slice,
           "equal_with_slice": oracle.equal_filter_with_slice}
    for kind in KINDS:
        for pred in preds:
            try:
                words, cnt = fns[kind](img, scale, pred)[:2]
            except oracle.OraclePanic:
                with pytest.raises(capi.ReferencePanic):
                    filter_image(src, scale, pred, kind)
                continue
            fr = filter_image(src, scale, pred, kind)
            assert fr.count == cnt, (name, kind, pred)
            assert np.array_equal(np.asarray(fr.words, dtype=np.uint32), words), (name, kind, pred)


def test_filter_image_layout_intended_and_device_words(oracle, gpu):
    import torch

    from buff_gb300.capi import FLAG_BUFF_LAYOUT, FLAG_INTENDED
    from buff_gb300.compress import Column, filter_image

    x = _walk(200_003, 31)
    flipped = oracle.encode(x, 10000)
    plain = oracle.encode(x, 10000, flipped=False)
    for pred in (float(np.quantile(x, 0.2)), float(x[777])):
        for kind in KINDS:
            a = filter_image(np.frombuffer(flipped, dtype=np.uint8), 10000, pred, kind)
            b = filter_image(np.frombuffer(plain, dtype=np.uint8), 10000, pred, kind,
                             flags=FLAG_BUFF_LAYOUT)
            assert a.count == b.count and np.array_equal(a.words, b.words), kind
            dw = torch.zeros((x.size + 31) // 32, dtype=torch.int32, device="cuda")
            c = filter_image(torch.frombuffer(bytearray(flipped), dtype=torch.uint8).cuda(), 10000,
                             pred, kind, words=dw)
            assert c.count == a.count
            assert np.array_equal(dw.cpu().numpy().view(np.uint32), a.words), kind
        # the intended semantics: same as the column call with the flag
        col = Column.deserialize(flipped, 10000, FLAG_INTENDED)
        for kind, fn in (("range", col.range_filter), ("equal", col.equal_filter)):
            want = fn(pred)
            got = filter_image(np.frombuffer(flipped, dtype=np.uint8), 10000, pred, kind,
                               flags=FLAG_INTENDED)
            assert got.count == want.count and np.array_equal(got.words, want.words), kind


def test_image_edge_plans(oracle, gpu):
    """Plans without the image kernel: no rows, packed codes (fixed_len < 8),
    the early return, bad kinds and truncated images."""
    from buff_gb300 import capi
    from buff_gb300.compress import Column, filter_image, range_filter_sum_image

    empty = Column.encode(np.zeros(0), 10000).serialize()
    fr = filter_image(empty, 10000, 1.0)
    assert fr.count == 0 and fr.n == 0
    fr, sr = range_filter_sum_image(empty, 10000, 1.0)
    assert fr.count == 0 and sr.n_partials == Column.deserialize(empty, 10000).sum().n_partials
    rng = np.random.default_rng(3)
    packed = np.round(rng.uniform(1.0, 1.5, 1000), 1)  # scale 10: 3-bit codes, no slice
    img = oracle.encode(packed, 10)
    h = oracle.header(img)
    assert (h.ilen + h.dlen) & 0xFFFFFFFF < 8  # ilen is stored wrapped when fixed_len < dlen
    for kind, fn in (("range", oracle.range_filter), ("equal", oracle.equal_filter)):
        words, cnt = fn(img, 10, 1.2)[:2]
        got = filter_image(img, 10, 1.2, kind)
        assert got.count == cnt and np.array_equal(got.words, words), kind
    words, cnt = oracle.range_filter(img, 10, 1.2)[:2]
    fr, sr = range_filter_sum_image(img, 10, 1.2)
    assert fr.count == cnt and sr.sum == oracle.buff_sum(img, 10)[0]
    walk = _walk(5000, 9)
    wimg = oracle.encode(walk, 10000)
    for kind, fn in (("range", oracle.range_filter), ("equal", oracle.equal_filter),
                     ("range_with_slice", oracle.range_filter_with_slice)):
        words, cnt = fn(wimg, 10000, -1e6)[:2]  # below the base: the early return
        got = filter_image(wimg, 10000, -1e6, kind)
        assert got.count == cnt and np.array_equal(got.words, words), kind
    with pytest.raises(capi.BuffError):
        capi.check(capi.lib().buff_filter_image(np.frombuffer(wimg, dtype=np.uint8).ctypes.data,
                                                len(wimg), 10000, 0, 7, 1.0, None, None, None))
    with pytest.raises(capi.BuffError):
        filter_image(wimg[:-3], 10000, 100.0)
    small = oracle.encode(walk[:20], 10000)  # _with_slice on fewer than 32 rows panics
    with pytest.raises(capi.ReferencePanic):
        filter_image(small, 10000, float(walk[5]), "equal_with_slice")


def test_concurrent_streams_on_one_column(oracle, gpu):
    """Queries on one resident column from two streams at once return what
    each returns alone (the handle is read-only after encode)."""
    import torch

    from buff_gb300 import capi
    from buff_gb300.compress import Column

    x = _walk(2_000_003, 77)
    img = oracle.encode(x, 10000)
    col = Column.encode(x, 10000)
    L = capi.lib()
    preds = [float(np.quantile(x, q)) for q in (0.05, 0.5, 0.95, 0.3)]
    nw = (x.size + 31) // 32
    streams = [torch.cuda.Stream() for _ in preds]
    words = [torch.zeros(nw, dtype=torch.int32, device="cuda") for _ in preds]
    counts = [torch.zeros(1, dtype=torch.int64, device="cuda") for _ in preds]
    for _ in range(3):
        for st, p, w, c in zip(streams, preds, words, counts):
            with torch.cuda.stream(st):
                capi.check(L.buff_range_filter(col.handle, p, w.data_ptr(), c.data_ptr(),
                                               st.cuda_stream))
        torch.cuda.synchronize()
        for p, w, c in zip(preds, words, counts):
            ow, oc = oracle.range_filter(img, 10000, p)[:2]
            assert int(c.item()) == oc
            assert np.array_equal(w.cpu().numpy().view(np.uint32), ow)
