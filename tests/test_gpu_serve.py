"""Serving loop on the GPU: every request's result is the same alone and in a
mixed, overlapping stream, in batched and one-query-per-launch mode, and
under an output budget that forces requests to wait."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _store(seed=11, ncols=24):
    from buff_gb300.compress import Column

    rng = np.random.default_rng(seed)
    cols, data = [], []
    for i in range(ncols):
        n = int(np.exp(rng.uniform(np.log(1000), np.log(400_000))))
        dec = int(rng.integers(2, 7))
        x = np.round(np.cumsum(rng.normal(0, 0.3, n)) + rng.uniform(-50, 50), dec)
        cols.append(Column.encode(x, 10 ** dec))
        data.append(x)
    return cols, data


def _mix(data, nreq, seed):
    from buff_gb300.capi import Q_DECODE, Q_EQUAL, Q_MAX, Q_RANGE, Q_SUM
    from buff_gb300.serve import request

    rng = np.random.default_rng(seed)
    reqs = []
    for t in range(nreq):
        c = int(rng.integers(0, len(data)))
        x = data[c]
        u = rng.uniform()
        if u < 0.5:
            ops, pred, prec = Q_RANGE, float(x[rng.integers(0, x.size)]), 0
        elif u < 0.7:
            ops, pred, prec = Q_EQUAL, float(x[rng.integers(0, x.size)]), 0
        elif u < 0.9:
            ops, pred, prec = (Q_SUM if rng.uniform() < 0.5 else Q_MAX), 0.0, 0
        else:
            ops, pred, prec = Q_DECODE, 0.0, int(rng.integers(0, 2))
        reqs.append(request(c, ops, pred, prec, tag=t))
    return reqs


def _snapshot(c, req, n):
    """Result and device outputs of one completion, copied to the host."""
    from buff_gb300.capi import Q_DECODE, Q_EQUAL, Q_RANGE, copy_bytes

    out = {"status": c.status, "count": c.result.count, "sum": c.result.sum,
           "max": (c.result.max_code, c.result.max_value),
           "parts": tuple(c.result.partials[: c.result.n_partials])}
    if req.ops & (Q_RANGE | Q_EQUAL) and c.words:
        out["words"] = copy_bytes(c.words, 4 * ((n + 31) // 32))
    if req.ops & Q_DECODE and c.values:
        out["values"] = copy_bytes(c.values, 8 * n)
    return out


def _run(server, reqs, data, one_at_a_time):
    snaps = {}
    if one_at_a_time:
        for r in reqs:
            server.submit([r])
            (c,) = server.wait(1)
            snaps[c.tag] = _snapshot(c, r, data[r.column].size)
            server.release(c)
    else:
        server.submit(reqs)
        done = server.wait(len(reqs))
        for c in done:
            r = reqs[c.tag]
            snaps[c.tag] = _snapshot(c, r, data[r.column].size)
            server.release(c)
    return snaps


@pytest.mark.parametrize("batched", [True, False])
def test_alone_equals_mixed(gpu, batched):
    from buff_gb300.serve import Server

    cols, data = _store()
    reqs = _mix(data, 300, 5)
    s = Server(1 << 30, max_batch=64, max_inflight=3, batched=batched, auto_release=False)
    for c in cols:
        s.add_column(c)
    s.start()
    alone = _run(s, reqs, data, True)
    mixed = _run(s, reqs, data, False)
    s.stop()
    s.free()
    assert alone.keys() == mixed.keys() == set(range(len(reqs)))
    for t in range(len(reqs)):
        assert alone[t] == mixed[t], t


def test_results_match_single_column(gpu):
    from buff_gb300.capi import Q_DECODE, Q_EQUAL, Q_MAX, Q_RANGE, Q_SUM
    from buff_gb300.serve import Server

    cols, data = _store(seed=12, ncols=10)
    reqs = _mix(data, 120, 6)
    s = Server(1 << 30, max_batch=32, max_inflight=2, batched=True, auto_release=False)
    for c in cols:
        s.add_column(c)
    s.start()
    got = _run(s, reqs, data, False)
    s.stop()
    s.free()
    for t, r in enumerate(reqs):
        col, n, g = cols[r.column], data[r.column].size, got[t]
        assert g["status"] == 0
        if r.ops & (Q_RANGE | Q_EQUAL):
            ref = col.range_filter(r.pred) if r.ops & Q_RANGE else col.equal_filter(r.pred)
            assert g["count"] == ref.count
            assert g["words"] == ref.words.astype("<u4").tobytes()
        if r.ops & Q_SUM:
            assert g["sum"] == col.sum().sum
        if r.ops & Q_MAX:
            m = col.max()
            assert g["max"] == (m.code, m.value)
        if r.ops & Q_DECODE:
            ref = col.decode_at_precision(r.precision) if r.precision else col.decode()
            assert g["values"] == np.ascontiguousarray(ref).tobytes()


def test_requests_that_fail(gpu):
    """A request asking for both filters is refused at submission in either
    mode; a batch whose requests all fail planning (a decode at a precision
    the reference has no bound for) still completes, each request with the
    single-column call's status; in a batch mixing them with valid requests
    the valid ones get their single-column results."""
    import ctypes as C

    import torch

    from buff_gb300 import capi
    from buff_gb300.capi import Q_DECODE, Q_EQUAL, Q_RANGE
    from buff_gb300.serve import Server, request

    cols, data = _store(seed=14, ncols=6)
    out = torch.empty(max(x.size for x in data), dtype=torch.float64, device="cuda")
    want = capi.lib().buff_decode_at_precision(cols[0].handle, 99, C.c_void_p(out.data_ptr()),
                                               None)
    assert want != 0
    for batched in (True, False):
        s = Server(1 << 30, max_batch=64, max_inflight=2, batched=batched, auto_release=False)
        for c in cols:
            s.add_column(c)
        s.start()
        s.submit([request(0, Q_RANGE | Q_EQUAL, 1.0, tag=0)])
        (c,) = s.wait(1)
        assert c.status == capi.EINVAL
        s.release(c)
        bad = [request(i % 6, Q_DECODE, 0.0, 99, tag=i) for i in range(40)]
        s.submit(bad)
        done = s.wait(len(bad))
        assert sorted(c.tag for c in done) == list(range(40))
        assert all(c.status == want for c in done)
        for c in done:
            s.release(c)
        reqs = []
        for i in range(40):
            x = data[i % 6]
            if i % 2:
                reqs.append(request(i % 6, Q_DECODE, 0.0, 99, tag=i))
            else:
                reqs.append(request(i % 6, Q_RANGE, float(x[x.size // 3]), tag=i))
        s.submit(reqs)
        got = {c.tag: c for c in s.wait(len(reqs))}
        for i, r in enumerate(reqs):
            c = got[i]
            if i % 2:
                assert c.status == want, i
            else:
                assert c.status == 0, i
                assert c.result.count == cols[i % 6].range_filter(r.pred).count
            s.release(c)
        s.stop()
        s.free()


def test_budget_forces_waits_and_efull(gpu):
    from buff_gb300.capi import Q_DECODE, Q_SUM
    from buff_gb300.compress import Column
    from buff_gb300.serve import Server, request

    rng = np.random.default_rng(2)
    x = np.round(np.cumsum(rng.normal(0, 1, 200_000)), 2)
    col = Column.encode(x, 100)
    # budget for two decodes at a time: 24 decodes must queue for memory
    s = Server(2 * (1 << 21), max_batch=8, max_inflight=4, batched=True, auto_release=True)
    cid = s.add_column(col)
    s.start()
    reqs = [request(cid, Q_DECODE, tag=i) for i in range(24)] + \
        [request(cid, Q_SUM, tag=24)]
    s.submit(reqs)
    done = s.wait(len(reqs))
    assert sorted(c.tag for c in done) == list(range(25))
    assert all(c.status == 0 for c in done)
    assert s.stats()["output_bytes_in_use"] == 0
    s.stop()
    s.free()
    tiny = Server(1 << 20, batched=True)
    cid = tiny.add_column(col)
    tiny.start()
    tiny.submit([request(cid, Q_DECODE, tag=7)])
    (c,) = tiny.wait(1)
    assert c.status == 8  # BUFF_EFULL: the outputs exceed the whole budget
    tiny.stop()
    tiny.free()


def test_replay_reports_latency(gpu):
    from buff_gb300.serve import Server

    cols, data = _store(seed=13, ncols=8)
    reqs = _mix(data, 2000, 9)
    arrivals = np.cumsum(np.random.default_rng(1).exponential(20_000, len(reqs))).astype(np.uint64)
    for batched in (True, False):
        s = Server(1 << 30, max_batch=256, max_inflight=4, batched=batched)
        for c in cols:
            s.add_column(c)
        s.start()
        lat, res, wall = s.replay(reqs, arrivals)
        s.stop()
        s.free()
        assert lat.size == len(reqs) and (lat > 0).all() and wall > 0
        assert all(r.status == 0 for r in res)


def _encode_inputs(seed):
    """Host f64 / f32 arrays and one device array to encode while serving."""
    import torch

    rng = np.random.default_rng(seed)
    out = []
    for i, n in enumerate((70_001, 250_000, 3_000, 131_072)):
        dec = int(rng.integers(2, 7))
        x = np.round(np.cumsum(rng.normal(0, 0.2, n)) + rng.uniform(-20, 20), dec)
        out.append((x, 10 ** dec))
    x32 = np.round(rng.uniform(-5, 5, 40_000), 2).astype(np.float32)
    out.append((x32, 100))
    xd = np.round(np.cumsum(rng.normal(0, 1.0, 90_000)), 3)
    out.append((torch.from_numpy(xd).cuda(), 1000))
    return out


def test_encode_requests_while_serving(oracle, gpu):
    """Encode requests mixed into a query stream: each new column is the
    oracle's byte image, queries on it then match a column encoded alone, and
    every query of the mix is the same as when it runs alone."""
    import torch

    from buff_gb300.capi import Q_RANGE, Q_SUM
    from buff_gb300.compress import Column
    from buff_gb300.serve import Server, encode_request, request

    cols, data = _store(seed=14, ncols=10)
    queries = _mix(data, 200, 10)
    inputs = _encode_inputs(15)
    s = Server(1 << 30, max_batch=32, max_inflight=3, batched=True, auto_release=False)
    for c in cols:
        s.add_column(c)
    base_bytes = s.stats()["store_bytes"]
    s.start()
    torch.cuda.synchronize()
    mixed_reqs = list(queries)
    enc_tag = {}
    for i, (x, scale) in enumerate(inputs):
        tag = 10_000 + i
        enc_tag[tag] = i
        mixed_reqs.insert(30 * i + 7, encode_request(x, scale, tag=tag))
    s.submit(mixed_reqs)
    done = s.wait(len(mixed_reqs))
    mixed, new_ids = {}, {}
    for c in done:
        if c.tag in enc_tag:
            assert c.status == 0, c.status
            new_ids[enc_tag[c.tag]] = c.column
            continue
        r = queries[c.tag]
        mixed[c.tag] = _snapshot(c, r, data[r.column].size)
        s.release(c)
    assert sorted(new_ids) == list(range(len(inputs)))
    alone = _run(s, queries, data, True)
    for t in range(len(queries)):
        assert alone[t] == mixed[t], t
    # every new column is the oracle's image; queries on it match a column
    # encoded alone through the single-column call
    grown = 0
    follow, refs = [], {}
    for i, (x, scale) in enumerate(inputs):
        xh = x.cpu().numpy() if hasattr(x, "cpu") else x
        col = s.column(new_ids[i])
        assert col.serialize() == oracle.encode(xh, scale), i
        grown += col.info.device_bytes
        ref = Column.encode(xh, scale)
        p = float(np.quantile(xh.astype(np.float64), 0.6))
        follow.append(request(new_ids[i], Q_RANGE | Q_SUM, p, tag=20_000 + i))
        refs[20_000 + i] = (ref.range_filter(p), ref.sum(), xh.size)
    assert s.stats()["store_bytes"] == base_bytes + grown
    s.submit(follow)
    for c in s.wait(len(follow)):
        f, sm, n = refs[c.tag]
        assert c.status == 0 and c.result.count == f.count and c.result.sum == sm.sum
        from buff_gb300.capi import copy_bytes

        assert copy_bytes(c.words, 4 * ((n + 31) // 32)) == f.words.astype("<u4").tobytes()
        s.release(c)
    s.stop()
    s.free()


def test_encode_budgets(oracle, gpu):
    """Resident columns are charged to the store budget (an encode that can
    never fit fails with BUFF_EFULL and charges nothing); an encode's host
    input is staged in the arena in arrival order with the queries' outputs."""
    import torch

    from buff_gb300.capi import Q_DECODE
    from buff_gb300.compress import Column
    from buff_gb300.serve import Server, encode_request, request

    rng = np.random.default_rng(3)
    x = np.round(np.cumsum(rng.normal(0, 1, 200_000)), 2)
    col = Column.encode(x, 100)
    cb = col.info.device_bytes
    small = np.round(rng.uniform(0, 1, 5_000), 2)
    big = np.round(np.cumsum(rng.normal(0, 1, 400_000)), 2)
    # store budget: the resident column plus room for the small encode only
    s = Server(1 << 26, max_batch=8, max_inflight=2, store_budget_bytes=cb + (1 << 16))
    cid = s.add_column(col)
    s.start()
    s.submit([encode_request(big, 100, tag=1), encode_request(small, 100, tag=2)])
    got = {c.tag: c for c in s.wait(2)}
    assert got[1].status == 8 and got[2].status == 0  # BUFF_EFULL, then OK
    st = s.stats()
    assert st["columns"] == 2
    assert st["store_bytes"] == cb + s.column(got[2].column).info.device_bytes
    assert s.column(got[2].column).serialize() == oracle.encode(small, 100)
    s.stop()
    s.free()
    # arena of 4 MiB: each 2 MiB decode output and each host input's staging
    # (1.6 MB -> a 2 MiB class) wait for one another in arrival order
    s = Server(4 << 20, max_batch=8, max_inflight=4, auto_release=True)
    cid = s.add_column(col)
    s.start()
    ins = [np.round(np.cumsum(rng.normal(0, 1, 200_000)), 2) for _ in range(4)]
    reqs = []
    for i in range(12):
        reqs.append(request(cid, Q_DECODE, tag=i))
        if i % 3 == 0:
            reqs.append(encode_request(ins[i // 3], 100, tag=100 + i // 3))
    s.submit(reqs)
    done = {c.tag: c for c in s.wait(len(reqs))}
    assert all(c.status == 0 for c in done.values())
    for j in range(4):
        assert s.column(done[100 + j].column).serialize() == oracle.encode(ins[j], 100)
    assert s.stats()["output_bytes_in_use"] == 0
    # host input larger than the whole arena: BUFF_EFULL; device input needs
    # no staging and is encoded
    huge = np.round(np.cumsum(rng.normal(0, 1, 1_000_000)), 2)
    dev = torch.from_numpy(huge).cuda()
    s.submit([encode_request(huge, 100, tag=200), encode_request(dev, 100, tag=201)])
    got = {c.tag: c for c in s.wait(2)}
    assert got[200].status == 8 and got[201].status == 0
    assert s.column(got[201].column).serialize() == oracle.encode(huge, 100)
    s.stop()
    s.free()
