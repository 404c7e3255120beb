"""Batched form: many columns per launch (buff_batch_* / buff_plan_* in the C ABI).

``batch_encode`` encodes a list of device-resident f64 columns with two
persistent launches; ``Plan`` runs a list of queries (range/equality filter,
optionally with the sum; sum; max; decode at a precision) over many columns
as one persistent launch, optionally recorded into a CUDA graph and replayed.
"""
from __future__ import annotations

import ctypes as C

from . import capi
from .capi import BatchTune, Query, QueryResult, check, lib, ptr, stream_handle
from .compress import Column


def tune(tile_rows: int = 32768, blocks_per_sm: int = 4, stage: int = 2) -> BatchTune:
    return BatchTune(tile_rows, blocks_per_sm, stage, 0)


def batch_encode(columns, scales, flags: int = 0, tune_: BatchTune | None = None,
                 stream=None) -> list[Column]:
    """Encodes every column (torch float64 tensors or raw device pointers with
    lengths) with its own scale; returns one Column per input."""
    n = len(columns)
    ptrs = (C.c_void_p * n)()
    lens = (C.c_uint64 * n)()
    for i, col in enumerate(columns):
        if isinstance(col, tuple):
            ptrs[i], lens[i] = col
        else:
            ptrs[i], lens[i] = col.data_ptr(), col.numel()
    sc = (C.c_uint64 * n)(*[int(s) for s in scales])
    out = (C.c_void_p * n)()
    check(lib().buff_batch_encode_f64(ptrs, lens, sc, n, flags,
                                      C.byref(tune_) if tune_ is not None else None,
                                      stream_handle(stream), out), "batch_encode")
    return [Column(out[i]) for i in range(n)]


def query(col: Column, ops: int, pred: float = 0.0, words=None, values=None,
          precision: int = 0) -> Query:
    return Query(col.handle.value, ops, precision, float(pred),
                 ptr(words) if words is not None else None,
                 ptr(values) if values is not None else None)


class Plan:
    """A batch of queries as one persistent launch."""

    def __init__(self, queries, tune_: BatchTune | None = None, stream=None):
        self.n = len(queries)
        self._q = (Query * max(self.n, 1))(*queries)
        self._h = C.c_void_p()
        check(lib().buff_plan_create(self._q, self.n,
                                     C.byref(tune_) if tune_ is not None else None,
                                     stream_handle(stream), C.byref(self._h)), "plan_create")

    def set_preds(self, preds):
        arr = (C.c_double * self.n)(*[float(p) for p in preds])
        check(lib().buff_plan_set_preds(self._h, arr), "plan_set_preds")

    def launch(self, stream=None):
        check(lib().buff_plan_launch(self._h, stream_handle(stream)), "plan_launch")

    def capture(self, stream):
        check(lib().buff_plan_capture(self._h, stream_handle(stream)), "plan_capture")

    def replay(self, stream):
        check(lib().buff_plan_replay(self._h, stream_handle(stream)), "plan_replay")

    def results(self, stream=None) -> list[QueryResult]:
        out = (QueryResult * max(self.n, 1))()
        check(lib().buff_plan_results(self._h, out, stream_handle(stream)), "plan_results")
        return list(out[: self.n])

    def free(self):
        if self._h and self._h.value:
            lib().buff_plan_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def autotune(queries, stream=None):
    qs = (Query * max(len(queries), 1))(*queries)
    best = BatchTune()
    ms = C.c_float(0)
    check(lib().buff_batch_autotune(qs, len(queries), stream_handle(stream), C.byref(best),
                                    C.byref(ms)), "autotune")
    return best, ms.value


__all__ = ["batch_encode", "Plan", "query", "autotune", "tune", "BatchTune", "QueryResult",
           "capi"]
