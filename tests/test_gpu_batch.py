"""GPU parity of the batched form: batch encode against the oracle's bytes,
and every batched query (plain launch and CUDA-graph replay) against the
single-column entry points and the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _columns(seed=5, ncols=40):
    rng = np.random.default_rng(seed)
    cols, scales = [], []
    for i in range(ncols):
        n = int(np.exp(rng.uniform(np.log(64), np.log(300_000))))
        dec = int(rng.integers(2, 7))
        x = np.round(np.cumsum(rng.normal(0, rng.uniform(0.01, 5), n)) + rng.uniform(-1e3, 1e3),
                     dec)
        cols.append(x)
        scales.append(10 ** dec)
    # edge columns: strictly decreasing head, decreasing throughout, 1 row,
    # a NaN, n % 32 != 0 with few rows, an exact power-of-two span
    cols.append(np.round(np.concatenate([np.linspace(50, 10, 5000), np.linspace(10, 30, 999)]), 2))
    cols.append(np.round(np.linspace(100, 0, 4001), 2))
    cols.append(np.array([3.25]))
    z = np.round(np.cumsum(rng.normal(0, 1, 3000)), 2)
    z[17] = np.nan
    cols.append(z)
    cols.append(np.round(rng.uniform(0, 9, 37), 1))
    cols.append(np.array([0.0, 2.56] * 600))
    scales += [100, 100, 100, 100, 10, 100]
    return cols, scales


def _encode_batch(cols, scales, flags=0, offset=False):
    import torch

    from buff_gb300 import batch

    dev = []
    keep = []
    for i, x in enumerate(cols):
        t = torch.from_numpy(x).cuda()
        if offset and i % 7 == 3 and x.size > 1:  # an unaligned start: single-column path
            buf = torch.empty(x.size + 1, dtype=torch.float64, device="cuda")
            buf[1:] = t
            keep.append(buf)
            dev.append((buf.data_ptr() + 8, x.size))
        else:
            keep.append(t)
            dev.append(t)
    out = batch.batch_encode(dev, scales, flags)
    torch.cuda.synchronize()
    return out, keep


@pytest.mark.parametrize("flags", [0, 1])
def test_batch_encode_bytes(oracle, gpu, flags):
    from buff_gb300 import capi

    cols, scales = _columns()
    # edge columns are the last six: decreasing head, decreasing, 1 row, NaN,
    # 37 rows, alternating.  The reference panics on the strictly decreasing
    # column (its max is never set and the width is taken of a negative
    # delta); the NaN column is checked in the exact-reference mode only.
    e = len(cols) - 6
    drop = {e + 3} if flags else {e + 1}
    keep = [i for i in range(len(cols)) if i not in drop]
    cols, scales = [cols[i] for i in keep], [scales[i] for i in keep]
    out, _ = _encode_batch(cols, scales, flags, offset=True)
    for x, s, c in zip(cols, scales, out):
        assert c.serialize() == oracle.encode(x, s, flags=flags), (x.size, s)
    with pytest.raises(capi.ReferencePanic):
        _encode_batch([np.arange(100.0), np.round(np.linspace(100, 0, 4001), 2)], [100, 100])


def _plan_queries(cols, scales, out, rng):
    import torch

    from buff_gb300 import batch, capi
    from buff_gb300.capi import Q_DECODE, Q_EQUAL, Q_MAX, Q_RANGE, Q_SUM

    qs, meta = [], []
    for x, s, c in zip(cols, scales, out):
        n = x.size
        nw = max((n + 31) // 32, 1)
        fin = x[np.isfinite(x)]
        for ops in (Q_RANGE | Q_SUM, Q_EQUAL, Q_RANGE, Q_SUM | Q_MAX, Q_DECODE):
            pred = float(np.quantile(fin, rng.uniform(0.5, 0.999))) if ops & (Q_RANGE | Q_EQUAL) else 0.0
            if ops == Q_EQUAL:
                pred = float(fin[rng.integers(0, fin.size)])
            words = torch.zeros(nw, dtype=torch.int32, device="cuda")
            vals = torch.zeros(max(n, 1), dtype=torch.float64, device="cuda")
            prec = int(rng.integers(0, 3)) if ops == Q_DECODE else 0
            if prec:
                try:  # precisions the single-column call rejects are skipped
                    c.decode_at_precision(prec)
                except capi.BuffError:
                    prec = 0
            qs.append(batch.query(c, ops, pred, words, vals, prec))
            meta.append((c, ops, pred, words, vals, prec, n))
    return qs, meta


def _check_results(res, meta):
    from buff_gb300 import capi
    from buff_gb300.capi import Q_DECODE, Q_EQUAL, Q_MAX, Q_RANGE, Q_SUM

    for r, (c, ops, pred, words, vals, prec, n) in zip(res, meta):
        nw = (n + 31) // 32
        if ops & (Q_RANGE | Q_EQUAL):
            ref = c.range_filter(pred) if ops & Q_RANGE else c.equal_filter(pred)
            got = words.cpu().numpy().view(np.uint32)[:nw]
            assert np.array_equal(got, ref.words) and r.count == ref.count, (n, ops, pred)
        if ops & Q_SUM:
            s = c.sum()
            assert r.sum == s.sum and list(r.partials[: r.n_partials]) == \
                list(s.partials[: s.n_partials]), (n, ops)
        if ops & Q_MAX:
            m = c.max()
            assert r.max_code == m.code and r.max_value == m.value
        if ops & Q_DECODE:
            ref = c.decode_at_precision(prec) if prec else c.decode()
            assert np.array_equal(vals.cpu().numpy()[:n], ref), (n, prec)


def test_batch_plan_matches_single_column(oracle, gpu):
    import torch

    from buff_gb300 import batch

    cols, scales = _columns(seed=8, ncols=30)
    keep = [i for i in range(len(cols)) if i != len(cols) - 5]
    cols, scales = [cols[i] for i in keep], [scales[i] for i in keep]
    out, _keep = _encode_batch(cols, scales)
    rng = np.random.default_rng(3)
    qs, meta = _plan_queries(cols, scales, out, rng)
    for tn in (batch.tune(4096, 2, 1), batch.tune(32768, 4, 2), batch.tune(131072, 8, 2)):
        p = batch.Plan(qs, tn)
        p.launch()
        _check_results(p.results(), meta)
        for _, _, _, w, v, _, _ in meta:
            w.zero_()
            v.zero_()
        s = torch.cuda.Stream()
        p.capture(s)
        for _ in range(2):
            p.replay(s)
        _check_results(p.results(s), meta)
        p.free()


def test_batch_plan_set_preds_and_replay(oracle, gpu):
    import torch

    from buff_gb300 import batch
    from buff_gb300.capi import Q_RANGE, Q_SUM

    cols, scales = _columns(seed=9, ncols=12)
    cols, scales = cols[:12], scales[:12]
    out, _keep = _encode_batch(cols, scales)
    qs, meta = [], []
    for x, c in zip(cols, out):
        w = torch.zeros(max((x.size + 31) // 32, 1), dtype=torch.int32, device="cuda")
        qs.append(batch.query(c, Q_RANGE | Q_SUM, float(np.median(x)), w))
        meta.append([c, Q_RANGE | Q_SUM, float(np.median(x)), w, None, 0, x.size])
    p = batch.Plan(qs)
    s = torch.cuda.Stream()
    p.capture(s)
    for q in (0.1, 0.9, 0.999):
        preds = [float(np.quantile(x, q)) for x in cols]
        p.set_preds(preds)
        p.replay(s)
        res = p.results(s)
        for m, pr in zip(meta, preds):
            m[2] = pr
        _check_results(res, meta)
    p.free()


def test_batch_errors_and_autotune(gpu):
    import torch

    from buff_gb300 import batch, capi
    from buff_gb300.capi import Q_EQUAL, Q_RANGE
    from buff_gb300.compress import Column, MajorColumn

    x = np.round(np.cumsum(np.random.default_rng(1).normal(0, 1, 50_000)), 2)
    c = Column.encode(x, 100)
    w = torch.zeros((x.size + 31) // 32, dtype=torch.int32, device="cuda")
    with pytest.raises(capi.BuffError):
        batch.Plan([batch.query(c, Q_RANGE | Q_EQUAL, 1.0, w)])
    with pytest.raises(capi.BuffError):
        batch.Plan([batch.query(c, Q_RANGE, 1.0)])  # no bitmap
    with pytest.raises(capi.BuffError):
        batch.Plan([batch.query(c, Q_RANGE, 1.0, w)], batch.tune(1000, 4, 1))
    m = MajorColumn.encode(np.round(np.random.default_rng(2).normal(100, 0.01, 5000), 4), 10000)
    with pytest.raises(capi.BuffError):
        batch.Plan([batch.query(m, Q_RANGE, 1.0, w)])
    best, ms = batch.autotune([batch.query(c, Q_RANGE, float(np.median(x)), w)])
    assert best.tile_rows % 1024 == 0 and ms > 0
