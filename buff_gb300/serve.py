"""Serving form (buff_server_* in the C ABI): resident columns, a request
loop with continuous batching under a memory budget (transient outputs and
encode inputs in one arena, resident columns in a store budget), encode
requests that add columns while queries run, and a load replay that reports
per-request latency."""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from .capi import Completion, QueryResult, Request, ServerConfig, check, lib
from .batch import tune as _tune


class Server:
    def __init__(self, output_budget_bytes: int, max_batch: int = 1024, max_inflight: int = 4,
                 batched: bool = True, auto_release: bool = True, tune=None,
                 store_budget_bytes: int = 0):
        cfg = ServerConfig(output_budget_bytes, store_budget_bytes, max_batch, max_inflight,
                           1 if batched else 0, 1 if auto_release else 0,
                           tune if tune is not None else _tune(0, 0, 0))
        if tune is None:
            cfg.tune.tile_rows = 0
        self._h = C.c_void_p()
        check(lib().buff_server_create(C.byref(cfg), C.byref(self._h)), "server_create")
        self.columns = []

    def add_column(self, col) -> int:
        cid = C.c_uint32(0)
        check(lib().buff_server_add_column(self._h, col.handle, C.byref(cid)), "add_column")
        self.columns.append(col)
        return cid.value

    def start(self):
        check(lib().buff_server_start(self._h), "server_start")

    def submit(self, reqs):
        arr = (Request * max(len(reqs), 1))(*reqs)
        check(lib().buff_server_submit(self._h, arr, len(reqs)), "server_submit")

    def poll(self, cap: int = 1024):
        out = (Completion * cap)()
        n = C.c_uint32(0)
        check(lib().buff_server_poll(self._h, out, cap, C.byref(n)), "server_poll")
        return list(out[: n.value])

    def wait(self, count: int, timeout_s: float = 60.0):
        got = []
        t0 = time.time()
        while len(got) < count:
            got += self.poll()
            if time.time() - t0 > timeout_s:
                raise TimeoutError(f"{len(got)} of {count} requests completed")
            if len(got) < count:
                time.sleep(0.0002)
        return got

    def release(self, c: Completion):
        check(lib().buff_server_release(self._h, C.byref(c)), "server_release")

    def stats(self):
        b, r, u = C.c_uint64(0), C.c_uint64(0), C.c_uint64(0)
        check(lib().buff_server_stats(self._h, C.byref(b), C.byref(r), C.byref(u)), "stats")
        sb, nc = C.c_uint64(0), C.c_uint32(0)
        check(lib().buff_server_store_stats(self._h, C.byref(sb), C.byref(nc)), "store_stats")
        return {"batches": b.value, "requests": r.value, "output_bytes_in_use": u.value,
                "store_bytes": sb.value, "columns": nc.value}

    def column(self, cid: int):
        """A store column as a Column view (the server keeps ownership of
        columns made by encode requests)."""
        from .compress import Column

        h = C.c_void_p()
        check(lib().buff_server_column(self._h, cid, C.byref(h)), "server_column")
        return Column.borrow(h.value)

    def replay(self, reqs, arrival_ns: np.ndarray, results: bool = True):
        """Plays requests (a list of Request or an array of REQ_DTYPE) at
        their arrival times; returns (latencies ns, results, wall seconds)."""
        n = len(reqs)
        if isinstance(reqs, np.ndarray):
            assert reqs.dtype == REQ_DTYPE
            arr = np.ascontiguousarray(reqs).ctypes.data
        else:
            arr = (Request * max(n, 1))(*reqs)
        arrival = np.ascontiguousarray(arrival_ns, dtype=np.uint64)
        lat = np.zeros(max(n, 1), dtype=np.uint64)
        res = (QueryResult * max(n, 1))() if results else None
        wall = C.c_double(0)
        check(lib().buff_server_replay(self._h, arr, arrival.ctypes.data, n, lat.ctypes.data,
                                       res, C.byref(wall)), "server_replay")
        return lat[:n], (list(res[:n]) if results else None), wall.value

    def stop(self):
        if self._h and self._h.value:
            check(lib().buff_server_stop(self._h), "server_stop")

    def free(self):
        if self._h and self._h.value:
            lib().buff_server_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# numpy layout of buff_request (for request streams built as arrays)
REQ_DTYPE = np.dtype([("column", "<u4"), ("ops", "<u4"), ("precision", "<u4"),
                      ("reserved", "<u4"), ("pred", "<f8"), ("tag", "<u8"),
                      ("values", "<u8"), ("n", "<u8"), ("scale", "<u8"), ("flags", "<u4"),
                      ("is_f32", "<u4")])
assert REQ_DTYPE.itemsize == C.sizeof(Request)


def request(column: int, ops: int, pred: float = 0.0, precision: int = 0, tag: int = 0):
    return Request(column, ops, precision, 0, float(pred), tag)


def encode_request(values, scale: int, flags: int = 0, tag: int = 0):
    """BUFF_Q_ENCODE of a host (numpy) or device (torch) f64/f32 array; the
    array must stay alive and unchanged until the request completes."""
    from .capi import Q_ENCODE

    if hasattr(values, "data_ptr"):
        ptr, n = values.data_ptr(), values.numel()
        f32 = str(values.dtype) == "torch.float32"
    else:
        a = np.asarray(values)
        assert a.flags.c_contiguous and a.dtype in (np.float64, np.float32)
        ptr, n, f32 = a.ctypes.data, a.size, a.dtype == np.float32
    r = Request(0, Q_ENCODE, 0, 0, 0.0, tag)
    r.values, r.n, r.scale, r.flags, r.is_f32 = ptr, n, scale, flags, 1 if f32 else 0
    return r


__all__ = ["Server", "request", "encode_request", "REQ_DTYPE"]
