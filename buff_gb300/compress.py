"""Host-side mirror of the reference's ``SplitBDDoubleCompress`` buff-simd API.

``SplitBDDoubleCompress(chunksize, batchsize, scale)`` keeps the reference's
constructor (database/src/compress/split_double.rs:29-39) and method names
(database/src/compress/buff_simd.rs); every method runs on the GPU through
the C ABI of ``include/buff_gpu.h``.  Where the reference takes the encoded
``Vec<u8>`` by value, these methods accept either a device-resident
:class:`Column` or the reference byte image (``bytes``/``np.uint8``), which is
uploaded once per call.  Where the reference only prints a result (filters,
max), the methods return it.  Where the reference panics, they raise
:class:`~buff_gb300.capi.ReferencePanic`.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi
from .capi import (FLAG_BUFF_LAYOUT, FLAG_INTENDED, FLAG_RAW_BITMAPS, check, lib, ptr,
                   stream_handle)


@dataclass
class FilterResult:
    """A BitVec<u32>-shaped result: ceil(n/32) words, bit i%32 of word i/32."""

    words: object  # np.ndarray[uint32] (host) or a device tensor
    count: int
    n: int

    def rows(self) -> np.ndarray:
        w = np.asarray(self.words if isinstance(self.words, np.ndarray) else self.words.cpu())
        bits = np.unpackbits(w.astype("<u4").view(np.uint8), bitorder="little")
        return np.nonzero(bits[: self.n])[0]


def rows_to_words(rows, n: int) -> np.ndarray:
    """A BitVec<u32> bitmap with the listed rows set."""
    bits = np.zeros(((n + 31) // 32) * 32, dtype=np.uint8)
    bits[np.asarray(rows, dtype=np.int64)] = 1
    return np.packbits(bits, bitorder="little").view("<u4").astype(np.uint32)


def _row_list(rows):
    if hasattr(rows, "data_ptr"):  # torch tensor (uint32 / int32), host or device
        return rows.contiguous(), rows.numel()
    arr = np.ascontiguousarray(np.asarray(rows, dtype=np.uint32).reshape(-1))
    return arr, arr.size


@dataclass
class MaxResult:
    value: float
    code: int
    argmax_words: object
    argmax_count: int


class Column:
    """A BUFF column resident in HBM (opaque ``buff_col*``)."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    # -- lifetime -------------------------------------------------------
    _ENCODE = ("buff_encode_f32", "buff_encode_f64")
    _DESERIALIZE = "buff_deserialize"

    @classmethod
    def encode(cls, values, scale: int, flags: int = 0, stream=None) -> "Column":
        h = C.c_void_p()
        f32, f64 = (getattr(lib(), nm) for nm in cls._ENCODE)
        if isinstance(values, np.ndarray):
            arr = np.ascontiguousarray(values)
            if arr.dtype == np.float32:
                fn = f32
            else:
                arr = np.ascontiguousarray(arr, dtype=np.float64)
                fn = f64
            check(fn(ptr(arr), arr.size, scale, flags, stream_handle(stream), C.byref(h)), "encode")
        else:  # torch tensor (host or device)
            import torch

            t = values.contiguous()
            if t.dtype == torch.float32:
                fn = f32
            elif t.dtype == torch.float64:
                fn = f64
            else:
                raise TypeError("values must be float32 or float64")
            check(fn(ptr(t), t.numel(), scale, flags, stream_handle(stream), C.byref(h)), "encode")
        return cls(h.value)

    @classmethod
    def deserialize(cls, data, scale: int, flags: int = 0, stream=None) -> "Column":
        h = C.c_void_p()
        if isinstance(data, (bytes, bytearray)):
            arr = np.frombuffer(bytes(data), dtype=np.uint8)
            n = arr.size
        elif isinstance(data, np.ndarray):
            arr = np.ascontiguousarray(data, dtype=np.uint8)
            n = arr.size
        else:
            arr = data
            n = data.numel()
        check(getattr(lib(), cls._DESERIALIZE)(ptr(arr), n, scale, flags, stream_handle(stream),
                                               C.byref(h)), "deserialize")
        return cls(h.value)

    @classmethod
    def borrow(cls, handle: int) -> "Column":
        """A view of a handle owned elsewhere (a server's store): never freed
        through this object."""
        c = cls(handle)
        c._borrowed = True
        return c

    def free(self):
        if getattr(self, "_borrowed", False):
            self._h = C.c_void_p()
            return
        if self._h and self._h.value:
            lib().buff_col_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def info(self) -> capi.ColInfo:
        inf = capi.ColInfo()
        check(lib().buff_col_get_info(self._h, C.byref(inf)), "info")
        return inf

    @property
    def n(self) -> int:
        return self.info.n

    # -- image ----------------------------------------------------------
    def serialize(self, out=None, stream=None) -> bytes:
        need = self.info.serialized_bytes
        ln = C.c_uint64(0)
        if need == 0:  # buff-major: the size is known after compressing the bitmaps
            lib().buff_serialize(self._h, None, 0, C.byref(ln), stream_handle(stream))
            need = ln.value
        if out is None:
            buf = np.empty(max(need, 1), dtype=np.uint8)
            check(lib().buff_serialize(self._h, ptr(buf), need, C.byref(ln),
                                       stream_handle(stream)), "serialize")
            return buf[: ln.value].tobytes()
        check(lib().buff_serialize(self._h, ptr(out), need, C.byref(ln), stream_handle(stream)),
              "serialize")
        return out

    # -- queries --------------------------------------------------------
    def decode(self, out=None, stream=None):
        if out is None:
            out = np.empty(max(self.n, 1), dtype=np.float64)
            check(lib().buff_decode(self._h, ptr(out), stream_handle(stream)), "decode")
            return out[: self.n]
        check(lib().buff_decode(self._h, ptr(out), stream_handle(stream)), "decode")
        return out

    def decode_at_precision(self, precision: int, out=None, stream=None):
        if out is None:
            out = np.empty(max(self.n, 1), dtype=np.float64)
            check(lib().buff_decode_at_precision(self._h, precision, ptr(out),
                                                 stream_handle(stream)), "decode_at_precision")
            return out[: self.n]
        check(lib().buff_decode_at_precision(self._h, precision, ptr(out), stream_handle(stream)),
              "decode_at_precision")
        return out

    def _filter(self, fn, pred: float, out=None, stream=None) -> FilterResult:
        n = self.n
        nw = (n + 31) // 32
        cnt = np.zeros(1, dtype=np.uint64)
        words = out if out is not None else np.zeros(max(nw, 1), dtype=np.uint32)
        check(fn(self._h, float(pred), ptr(words), ptr(cnt), stream_handle(stream)), fn.__name__)
        if out is None:
            words = words[:nw]
        return FilterResult(words, int(cnt[0]), n)

    def range_filter(self, pred, out=None, stream=None):
        return self._filter(lib().buff_range_filter, pred, out, stream)

    def equal_filter(self, pred, out=None, stream=None):
        return self._filter(lib().buff_equal_filter, pred, out, stream)

    def range_filter_with_slice(self, pred, out=None, stream=None):
        return self._filter(lib().buff_range_filter_with_slice, pred, out, stream)

    def scalar_range_filter(self, pred, out=None, stream=None):
        """buff_range_filter (buff_simd.rs:4507-4679): every row compared."""
        return self._filter(lib().buff_scalar_range_filter, pred, out, stream)

    def scalar_equal_filter(self, pred, out=None, stream=None):
        """buff_equal_filter (buff_simd.rs:4925-5094): every row compared."""
        return self._filter(lib().buff_scalar_equal_filter, pred, out, stream)

    def equal_filter_with_slice(self, pred, out=None, stream=None):
        return self._filter(lib().buff_equal_filter_with_slice, pred, out, stream)

    def sum(self, stream=None) -> capi.SumResult:
        res = capi.SumResult()
        check(lib().buff_sum(self._h, C.byref(res), stream_handle(stream)), "sum")
        return res

    def range_filter_sum(self, pred, stream=None):
        """Range filter and sum in one pass: (FilterResult, SumResult)."""
        n = self.n
        nw = (n + 31) // 32
        words = np.zeros(max(nw, 1), dtype=np.uint32)
        cnt = np.zeros(1, dtype=np.uint64)
        parts = np.zeros(9, dtype=np.uint64)
        check(lib().buff_range_filter_sum(self._h, float(pred), ptr(words), ptr(cnt), ptr(parts),
                                          stream_handle(stream)), "range_filter_sum")
        res = capi.SumResult()
        check(lib().buff_sum_finish(self._h, parts.ctypes.data, C.byref(res)), "sum_finish")
        return FilterResult(words[:nw], int(cnt[0]), n), res

    # -- row-conditioned reads -------------------------------------------
    _DECODE_CONDITION = "buff_decode_condition"
    _FILTER_CONDITION = "buff_range_filter_condition"

    def decode_condition(self, rows, out=None, stream=None):
        """Values of the listed rows (strictly ascending ids)."""
        r, m = _row_list(rows)
        dst = out if out is not None else np.empty(max(m, 1), dtype=np.float64)
        if self._DECODE_CONDITION == "buff_decode_condition":
            check(lib().buff_decode_condition(self._h, ptr(r), m, ptr(dst), stream_handle(stream)),
                  "decode_condition")
            return dst if out is not None else dst[:m]
        nout = C.c_uint64(0)
        check(lib().buff_major_decode_condition(self._h, ptr(r), m, ptr(dst), C.byref(nout),
                                                stream_handle(stream)), "decode_condition")
        return dst[: nout.value] if out is None else dst

    def decode_selected(self, words, out=None, stream=None):
        """Values of the rows set in a bitmap (e.g. a FilterResult's words)."""
        if isinstance(words, FilterResult):
            words = words.words
        cnt = C.c_uint64(0)
        dst = out if out is not None else np.empty(max(self.n, 1), dtype=np.float64)
        check(lib().buff_decode_selected(self._h, ptr(words), ptr(dst), C.byref(cnt),
                                         stream_handle(stream)), "decode_selected")
        return dst[: cnt.value] if out is None else (dst, cnt.value)

    def range_filter_condition(self, pred, cand, out=None, stream=None) -> FilterResult:
        """Range predicate on candidate rows (a bitmap or a row list)."""
        n = self.n
        nw = (n + 31) // 32
        if isinstance(cand, FilterResult):
            cand = cand.words
        elif not (hasattr(cand, "data_ptr") or
                  (isinstance(cand, np.ndarray) and cand.dtype == np.uint32 and cand.size == nw)):
            cand = rows_to_words(cand, n)
        cnt = np.zeros(1, dtype=np.uint64)
        words = out if out is not None else np.zeros(max(nw, 1), dtype=np.uint32)
        fn = getattr(lib(), self._FILTER_CONDITION)
        check(fn(self._h, float(pred), ptr(cand), ptr(words), ptr(cnt), stream_handle(stream)),
              self._FILTER_CONDITION)
        if out is None:
            words = words[:nw]
        return FilterResult(words, int(cnt[0]), n)

    def max_range(self, start: int, end: int, window: int, out=None, stream=None):
        """Maximum of every window of `window` rows in [start, end)."""
        nwin = (end - start) // window + 1 if window and end >= start else 1
        dst = out if out is not None else np.empty(max(nwin, 1), dtype=np.float64)
        cnt = C.c_uint64(0)
        check(lib().buff_max_range(self._h, start, end, window, ptr(dst), C.byref(cnt),
                                   stream_handle(stream)), "max_range")
        return dst[: cnt.value] if out is None else (dst, cnt.value)

    def range_filter_decode(self, pred, stream=None):
        """Range filter, then the selected rows' values (one call)."""
        n = self.n
        words = np.zeros(max((n + 31) // 32, 1), dtype=np.uint32)
        vals = np.empty(max(n, 1), dtype=np.float64)
        cnt = C.c_uint64(0)
        check(lib().buff_range_filter_decode(self._h, float(pred), ptr(words), ptr(vals),
                                             C.byref(cnt), stream_handle(stream)),
              "range_filter_decode")
        return FilterResult(words[: (n + 31) // 32], cnt.value, n), vals[: cnt.value]

    def sum_at_precision(self, precision: int, stream=None) -> float:
        v = C.c_double(0)
        check(lib().buff_sum_at_precision(self._h, precision, C.byref(v), stream_handle(stream)),
              "sum_at_precision")
        return v.value

    def max(self, argmax: bool = False, stream=None) -> MaxResult:
        v = C.c_double(0)
        code = C.c_uint64(0)
        cnt = C.c_uint64(0)
        words = np.zeros(max((self.n + 31) // 32, 1), dtype=np.uint32) if argmax else None
        check(lib().buff_max(self._h, C.byref(v), C.byref(code), ptr(words),
                             C.byref(cnt) if argmax else None, stream_handle(stream)), "max")
        if words is not None:
            words = words[: (self.n + 31) // 32]
        return MaxResult(v.value, code.value, words, cnt.value)


def _maj_fn(col, i):
    """The i-th majority entry point for `col`'s kind (a plain handle gets
    the buff-major ones, which reject it)."""
    names = getattr(col, "_MAJ", None) or MajorColumn._MAJ
    return getattr(lib(), names[i])


class MajorColumn(Column):
    """A buff-major (outlier) column resident in HBM: sparse leading byte
    columns kept as (major byte, outlier bitmap, outlier bytes), the rest as
    slices (compress/buff_simd.rs:317-630)."""

    _ENCODE = ("buff_encode_majority_f32", "buff_encode_majority_f64")
    _DESERIALIZE = "buff_deserialize_majority"
    _DECODE_CONDITION = "buff_major_decode_condition"
    _FILTER_CONDITION = "buff_range_filter_majority_condition"
    _MAJ = ("buff_decode_majority", "buff_range_filter_majority", "buff_equal_filter_majority",
            "buff_sum_majority", "buff_max_majority")

    def decode(self, out=None, stream=None):
        fn = _maj_fn(self, 0)
        if out is None:
            out = np.empty(max(self.n, 1), dtype=np.float64)
            check(fn(self._h, ptr(out), stream_handle(stream)), "decode")
            return out[: self.n]
        check(fn(self._h, ptr(out), stream_handle(stream)), "decode")
        return out

    def range_filter(self, pred, out=None, stream=None):
        return self._filter(_maj_fn(self, 1), pred, out, stream)

    def equal_filter(self, pred, out=None, stream=None):
        return self._filter(_maj_fn(self, 2), pred, out, stream)

    def sum(self, stream=None) -> capi.SumResult:
        res = capi.SumResult()
        check(_maj_fn(self, 3)(self._h, C.byref(res), stream_handle(stream)), "sum")
        return res

    def max(self, argmax: bool = False, stream=None) -> MaxResult:
        v = C.c_double(0)
        code = C.c_uint64(0)
        cnt = C.c_uint64(0)
        words = np.zeros(max((self.n + 31) // 32, 1), dtype=np.uint32) if argmax else None
        check(_maj_fn(self, 4)(self._h, C.byref(v), C.byref(code), ptr(words),
                                           C.byref(cnt) if argmax else None,
                                           stream_handle(stream)), "max")
        if words is not None:
            words = words[: (self.n + 31) // 32]
        return MaxResult(v.value, code.value, words, cnt.value)

    def max_range(self, start: int, end: int, window: int, out=None, stream=None):
        """buff_max_majority_range: windowed maxima (none with sparse columns)."""
        nwin = (end - start) // window + 1 if window and end >= start else 1
        dst = out if out is not None else np.empty(max(nwin, 1), dtype=np.float64)
        cnt = C.c_uint64(0)
        check(lib().buff_max_majority_range(self._h, start, end, window, ptr(dst), C.byref(cnt),
                                            stream_handle(stream)), "max_majority_range")
        return dst[: cnt.value] if out is None else (dst, cnt.value)

    def _unsupported(self, *a, **k):
        raise capi.BuffError(capi.ENOTSUP, "not defined on buff-major columns")

    decode_at_precision = sum_at_precision = _unsupported
    range_filter_with_slice = equal_filter_with_slice = _unsupported
    decode_selected = range_filter_decode = _unsupported


class RapgMajorColumn(MajorColumn):
    """A RAPG-major column (compress/split_double.rs:957-1240,
    byte_residue_encode_outlieru8): the buff-major layout with the leading
    byte as the one sparse column, major byte 69, croaring bitmap in the
    image; queried through the byte_residue_*_majority entry points."""

    _ENCODE = ("buff_rapg_encode_outlieru8_f32", "buff_rapg_encode_outlieru8_f64")
    _DESERIALIZE = "buff_rapg_major_deserialize"
    _MAJ = ("buff_rapg_decode_majority", "buff_rapg_range_filter_majority",
            "buff_rapg_equal_filter_majority", "buff_rapg_sum_majority", "buff_rapg_max_majority")

    def _unsupported(self, *a, **k):
        raise capi.BuffError(capi.ENOTSUP, "not defined on RAPG-major columns")

    decode_condition = range_filter_condition = max_range = _unsupported


class SliceColumn(Column):
    """A buff-slice column resident in HBM (compress/buff_slice.rs:298-437):
    ceil(fixed_len/8) byte slices, the last holding the low code bits
    left-aligned."""

    _ENCODE = ("buff_slice_encode_f32", "buff_slice_encode_f64")
    _DESERIALIZE = "buff_slice_deserialize"

    def decode(self, out=None, stream=None):
        dst = out if out is not None else np.empty(max(self.n, 1), dtype=np.float64)
        check(lib().buff_slice_decode(self._h, ptr(dst), stream_handle(stream)), "decode")
        return dst[: self.n] if out is None else dst

    def range_filter(self, pred, out=None, stream=None):
        return self._filter(lib().buff_slice_range_filter, pred, out, stream)

    def equal_filter(self, pred, out=None, stream=None):
        return self._filter(lib().buff_slice_equal_filter, pred, out, stream)

    def range_filter_nosimd(self, pred, out=None, stream=None):
        return self._filter(lib().buff_slice_range_filter_nosimd, pred, out, stream)

    def equal_filter_nosimd(self, pred, out=None, stream=None):
        return self._filter(lib().buff_slice_equal_filter_nosimd, pred, out, stream)

    def decode_bs(self, out=None, stream=None):
        dst = out if out is not None else np.empty(max(self.n, 1), dtype=np.float64)
        check(lib().buff_slice_decode_bs(self._h, ptr(dst), stream_handle(stream)), "decode_bs")
        return dst[: self.n] if out is None else dst

    def slice_sum(self, any_width: bool = False, stream=None) -> float:
        v = C.c_double(0)
        fn = lib().buff_slice_buffsum if any_width else lib().buff_slice_sum
        check(fn(self._h, C.byref(v), stream_handle(stream)), "slice_sum")
        return v.value

    def slice_max(self, any_width: bool = False, stream=None):
        v = C.c_double(0)
        cnt = C.c_uint64(0)
        words = np.zeros(max((self.n + 31) // 32, 1), dtype=np.uint32)
        fn = lib().buff_slice_buffmax if any_width else lib().buff_slice_max
        check(fn(self._h, C.byref(v), ptr(words), C.byref(cnt), stream_handle(stream)),
              "slice_max")
        return MaxResult(v.value, 0, words[: (self.n + 31) // 32], cnt.value)

    def max_range(self, start: int, end: int, window: int, out=None, stream=None):
        """Maximum of every window of `window` rows in [start, end)
        (buff_slice_max_range)."""
        hi = min(end, self.n)
        nwin = (hi - start + window - 1) // window + 1 if window and hi > start else 1
        dst = out if out is not None else np.empty(nwin, dtype=np.float64)
        cnt = C.c_uint64(0)
        check(lib().buff_slice_max_range(self._h, start, end, window, ptr(dst), C.byref(cnt),
                                         stream_handle(stream)), "slice_max_range")
        return dst[: cnt.value] if out is None else (dst, cnt.value)

    def _unsupported(self, *a, **k):
        raise capi.BuffError(capi.ENOTSUP, "not defined on buff-slice columns")

    sum = max = decode_at_precision = sum_at_precision = _unsupported
    range_filter_with_slice = equal_filter_with_slice = _unsupported
    decode_condition = decode_selected = range_filter_condition = _unsupported
    range_filter_decode = _unsupported


class RapgColumn(Column):
    """A RAPG byte_residue column resident in HBM
    (compress/split_double.rs:624-955): sparse leading bytes as row sets
    (major byte 0) plus nonzero bytes, dense slices, packed tail."""

    _ENCODE = ("buff_rapg_encode_f32", "buff_rapg_encode_f64")
    _DESERIALIZE = "buff_rapg_deserialize"

    def _decode(self, precision, out, stream):
        dst = out if out is not None else np.empty(max(self.n, 1), dtype=np.float64)
        cnt = C.c_uint64(0)
        if precision is None:
            check(lib().buff_rapg_decode(self._h, ptr(dst), C.byref(cnt), stream_handle(stream)),
                  "rapg_decode")
        else:
            check(lib().buff_rapg_decode_at_precision(self._h, precision, ptr(dst), C.byref(cnt),
                                                      stream_handle(stream)), "rapg_decode")
        return dst[: cnt.value] if out is None else (dst, cnt.value)

    def decode(self, out=None, stream=None):
        """byte_residue_decode (split_double.rs:1353-1610)."""
        return self._decode(None, out, stream)

    def decode_at_precision(self, precision: int, out=None, stream=None):
        """byte_residue_decode_with_precision (split_double.rs:1612-1893)."""
        return self._decode(precision, out, stream)

    def rapg_sum(self, precision=None, stream=None) -> float:
        """byte_residue_sum / byte_residue_sum_with_precision."""
        v = C.c_double(0)
        if precision is None:
            check(lib().buff_rapg_sum(self._h, C.byref(v), stream_handle(stream)), "rapg_sum")
        else:
            check(lib().buff_rapg_sum_at_precision(self._h, precision, C.byref(v),
                                                   stream_handle(stream)), "rapg_sum")
        return v.value

    def _unsupported(self, *a, **k):
        raise capi.BuffError(capi.ENOTSUP, "not defined on RAPG columns")

    sum = max = sum_at_precision = range_filter = equal_filter = _unsupported
    range_filter_with_slice = equal_filter_with_slice = _unsupported
    decode_condition = decode_selected = range_filter_condition = _unsupported
    range_filter_decode = max_range = range_filter_sum = _unsupported


class BuffSliceCompress:
    """GPU mirror of ``BuffSliceCompress`` (compress/buff_slice.rs:222-296)."""

    def __init__(self, chunksize: int, batchsize: int, scale: int):
        self.chunksize = chunksize
        self.batchsize = batchsize
        self.scale = scale

    def _col(self, data) -> SliceColumn:
        return data if isinstance(data, SliceColumn) else SliceColumn.deserialize(data, self.scale)

    def buff_slice_encode(self, values, stream=None) -> SliceColumn:
        return SliceColumn.encode(values, self.scale, 0, stream)

    def buff_slice_decode(self, data, stream=None):
        return self._col(data).decode(stream=stream)

    def buff_slice_range_filter(self, data, pred, stream=None) -> FilterResult:
        return self._col(data).range_filter(pred, stream=stream)

    def buff_slice_equal_filter(self, data, pred, stream=None) -> FilterResult:
        return self._col(data).equal_filter(pred, stream=stream)

    # buff_slice.rs:1184-1262, :1753-1871, :1873-1991 (the buff-slice-scalar arm)
    def buff_slice_decode_bs(self, data, stream=None):
        return self._col(data).decode_bs(stream=stream)

    def buff_slice_range_filter_nosimd(self, data, pred, stream=None) -> FilterResult:
        return self._col(data).range_filter_nosimd(pred, stream=stream)

    def buff_slice_equal_filter_nosimd(self, data, pred, stream=None) -> FilterResult:
        return self._col(data).equal_filter_nosimd(pred, stream=stream)

    def buff_slice_sum(self, data, stream=None) -> float:
        return self._col(data).slice_sum(False, stream=stream)

    def buff_slice_buffsum(self, data, stream=None) -> float:
        return self._col(data).slice_sum(True, stream=stream)

    def buff_slice_max(self, data, stream=None) -> MaxResult:
        return self._col(data).slice_max(False, stream=stream)

    def buff_slice_buffmax(self, data, stream=None) -> MaxResult:
        return self._col(data).slice_max(True, stream=stream)

    def buff_slice_max_range(self, data, s: int, e: int, window: int, stream=None):
        return self._col(data).max_range(s, e, window, stream=stream)


def _image_arg(image):
    """(address-bearing array, length, header bytes) of a serialized image."""
    if isinstance(image, (bytes, bytearray)):
        arr = np.frombuffer(bytes(image), dtype=np.uint8)
    elif isinstance(image, np.ndarray):
        arr = np.ascontiguousarray(image, dtype=np.uint8)
    else:
        arr = image
    ln = arr.size if isinstance(arr, np.ndarray) else arr.numel()
    if ln < 20:
        raise capi.BuffError(capi.ECORRUPT, "image")
    if isinstance(arr, np.ndarray):
        hdr = arr[:20].tobytes()
    elif getattr(arr, "is_cuda", False):
        hdr = capi.copy_bytes(ptr(arr), 20)
    else:
        hdr = arr[:20].numpy().tobytes()
    return arr, ln, hdr


FILTER_KINDS = {"range": 0, "equal": 1, "range_with_slice": 2, "equal_with_slice": 3}


def filter_image(image, scale: int, pred: float, kind: str = "range", flags: int = 0,
                 words=None, stream=None) -> FilterResult:
    """A buff-simd filter straight from a serialized image (host or device
    memory), without a resident column.  kind: range, equal,
    range_with_slice or equal_with_slice."""
    arr, ln, hdr = _image_arg(image)
    n = int.from_bytes(hdr[8:12], "little")
    nw = (n + 31) // 32
    out = words if words is not None else np.zeros(max(nw, 1), dtype=np.uint32)
    cnt = np.zeros(1, dtype=np.uint64)
    check(lib().buff_filter_image(ptr(arr), ln, scale, flags, FILTER_KINDS[kind], float(pred),
                                  ptr(out), ptr(cnt), stream_handle(stream)), "filter_image")
    if words is None:
        out = out[:nw]
    return FilterResult(out, int(cnt[0]), n)


def range_filter_sum_image(image, scale: int, pred: float, flags: int = 0, words=None,
                           stream=None):
    """Range filter and sum straight from a serialized image (host or device
    memory) in one pass, without a resident column: (FilterResult, SumResult).

    ``image``: bytes, a uint8 numpy array, or a uint8 torch tensor (pinned host
    or device).  ``words``: optional output buffer of ceil(n/32) uint32 (numpy
    or torch); a new host array by default."""
    arr, ln, hdr = _image_arg(image)
    n = int.from_bytes(hdr[8:12], "little")
    nw = (n + 31) // 32
    out = words if words is not None else np.zeros(max(nw, 1), dtype=np.uint32)
    cnt = np.zeros(1, dtype=np.uint64)
    res = capi.SumResult()
    check(lib().buff_range_filter_sum_image(ptr(arr), ln, scale, flags, float(pred), ptr(out),
                                            ptr(cnt), C.byref(res), stream_handle(stream)),
          "range_filter_sum_image")
    if words is None:
        out = out[:nw]
    return FilterResult(out, int(cnt[0]), n), res


def _as_major(comp: "SplitBDDoubleCompress", data) -> MajorColumn:
    if isinstance(data, MajorColumn):
        return data
    return MajorColumn.deserialize(data, comp.scale, comp.flags)


def _as_rapg(comp: "SplitBDDoubleCompress", data) -> RapgColumn:
    if isinstance(data, RapgColumn):
        return data
    return RapgColumn.deserialize(data, comp.scale, comp.flags)


def _as_column(comp: "SplitBDDoubleCompress", data) -> Column:
    if isinstance(data, Column):
        return data
    return Column.deserialize(data, comp.scale, comp.flags)


class SplitBDDoubleCompress:
    """GPU mirror of ``SplitBDDoubleCompress`` (compress/split_double.rs:29-39)."""

    def __init__(self, chunksize: int, batchsize: int, scale: int, flags: int = 0):
        self.chunksize = chunksize  # unused by the reference's buff-simd path
        self.batchsize = batchsize  # unused by the reference's buff-simd path
        self.scale = scale
        self.flags = flags

    # compress/buff_simd.rs:3116-3250
    def buff_simd256_encode(self, values, stream=None) -> Column:
        return Column.encode(values, self.scale, self.flags, stream)

    # compress/buff_simd.rs:3252-3357
    def buff_simd256_decode(self, data, stream=None):
        return _as_column(self, data).decode(stream=stream)

    # compress/buff_simd.rs:3361-3547 (the reference prints the count)
    def buff_simd_range_filter(self, data, pred, stream=None) -> FilterResult:
        return _as_column(self, data).range_filter(pred, stream=stream)

    # compress/buff_simd.rs:3549-3733
    def buff_simd_equal_filter(self, data, pred, stream=None) -> FilterResult:
        return _as_column(self, data).equal_filter(pred, stream=stream)

    # compress/buff_simd.rs:3736-3884
    def buff_simd_range_filter_with_slice(self, data, pred, stream=None) -> FilterResult:
        return _as_column(self, data).range_filter_with_slice(pred, stream=stream)

    # compress/buff_simd.rs:3888-4025
    def buff_simd_equal_filter_with_slice(self, data, pred, stream=None) -> FilterResult:
        return _as_column(self, data).equal_filter_with_slice(pred, stream=stream)

    # ---- buff layout (the `buff` profiler arm, buff_simd.rs:167-245) ----
    # compress/split_double.rs:298-432: the image without the ^0x80 flip
    def byte_fixed_encode(self, values, stream=None) -> Column:
        return Column.encode(values, self.scale, self.flags | FLAG_BUFF_LAYOUT, stream)

    # compress/split_double.rs:1243-1350
    def byte_fixed_decode(self, data, stream=None):
        return self._buff_layout(data).decode(stream=stream)

    # compress/buff_simd.rs:4507-4679 (the reference prints the count)
    def buff_range_filter(self, data, pred, stream=None) -> FilterResult:
        return self._buff_layout(data).scalar_range_filter(pred, stream=stream)

    # compress/buff_simd.rs:4925-5094
    def buff_equal_filter(self, data, pred, stream=None) -> FilterResult:
        return self._buff_layout(data).scalar_equal_filter(pred, stream=stream)

    def _buff_layout(self, data) -> Column:
        if isinstance(data, Column):
            return data
        return Column.deserialize(data, self.scale, self.flags | FLAG_BUFF_LAYOUT)

    # compress/split_double.rs:2127-2208 (on the unflipped slices)
    def byte_fixed_sum(self, data, stream=None) -> float:
        return _as_column(self, data).sum(stream=stream).sum

    # compress/split_double.rs:3919-4105 (the reference prints the max)
    def byte_fixed_max(self, data, stream=None) -> MaxResult:
        return _as_column(self, data).max(argmax=True, stream=stream)

    # ---- RAPG byte_residue format -----------------------------------
    # compress/split_double.rs:624-955
    def byte_residue_encode(self, values, stream=None) -> RapgColumn:
        return RapgColumn.encode(values, self.scale, self.flags, stream)

    # compress/split_double.rs:1353-1610
    def byte_residue_decode(self, data, stream=None):
        return _as_rapg(self, data).decode(stream=stream)

    # compress/split_double.rs:1612-1893 (a buff-simd column: the same
    # precision-limited read of its codes)
    def byte_residue_decode_with_precision(self, data, precision: int, stream=None):
        if isinstance(data, Column) and not isinstance(data, RapgColumn):
            return data.decode_at_precision(precision, stream=stream)
        return _as_rapg(self, data).decode_at_precision(precision, stream=stream)

    # compress/split_double.rs:2211-2407
    def byte_residue_sum(self, data, stream=None) -> float:
        return _as_rapg(self, data).rapg_sum(stream=stream)

    # compress/split_double.rs:957-1240 (outlier_exp's encoder)
    def byte_residue_encode_outlieru8(self, values, stream=None) -> RapgMajorColumn:
        return RapgMajorColumn.encode(values, self.scale, self.flags, stream)

    def _rapg_major(self, data) -> RapgMajorColumn:
        if isinstance(data, RapgMajorColumn):
            return data
        return RapgMajorColumn.deserialize(data, self.scale, self.flags)

    # compress/split_double.rs:1897-2125
    def byte_residue_decode_majority(self, data, stream=None):
        return self._rapg_major(data).decode(stream=stream)

    # compress/split_double.rs:2958-3370 (the reference prints the count)
    def byte_residue_range_filter_majority(self, data, pred, stream=None) -> FilterResult:
        return self._rapg_major(data).range_filter(pred, stream=stream)

    # compress/split_double.rs:3541-3918
    def byte_residue_equal_filter_majority(self, data, pred, stream=None) -> FilterResult:
        return self._rapg_major(data).equal_filter(pred, stream=stream)

    # compress/split_double.rs:2632-2782
    def byte_residue_sum_majority(self, data, stream=None) -> float:
        return self._rapg_major(data).sum(stream=stream).sum

    # compress/split_double.rs:4107-4676 (the reference prints the max)
    def byte_residue_max_majority(self, data, stream=None) -> MaxResult:
        return self._rapg_major(data).max(argmax=True, stream=stream)

    # compress/split_double.rs:2409-2630
    def byte_residue_sum_with_precision(self, data, precision: int, stream=None) -> float:
        if isinstance(data, Column) and not isinstance(data, RapgColumn):
            return data.sum_at_precision(precision, stream=stream)
        return _as_rapg(self, data).rapg_sum(precision, stream=stream)

    # compress/buff_simd.rs:1528-1712 (buff layout; rows strictly ascending)
    def buff_decode_condition(self, data, rows, stream=None):
        return _as_column(self, data).decode_condition(rows, stream=stream)

    # compress/buff_simd.rs:4683-4921 (returns the BitVec<u32>)
    def buff_range_filter_condition(self, data, pred, rows, stream=None) -> FilterResult:
        return _as_column(self, data).range_filter_condition(pred, rows, stream=stream)

    # compress/buff_simd.rs:5096-5334 (the reference prints the count)
    def buff_max_range(self, data, s: int, e: int, window: int, stream=None):
        return _as_column(self, data).max_range(s, e, window, stream=stream)

    # ---- buff-major (outlier) format --------------------------------
    # compress/buff_simd.rs:317-630
    def buff_encode_majority(self, values, stream=None) -> MajorColumn:
        return MajorColumn.encode(values, self.scale, self.flags, stream)

    # compress/buff_simd.rs:633-861
    def buff_decode_majority(self, data, stream=None):
        return _as_major(self, data).decode(stream=stream)

    # compress/buff_simd.rs:863-1277 (the reference prints the count)
    def buff_range_filter_majority(self, data, pred, stream=None) -> FilterResult:
        return _as_major(self, data).range_filter(pred, stream=stream)

    # compress/buff_simd.rs:1916-2292
    def buff_equal_filter_majority(self, data, pred, stream=None) -> FilterResult:
        return _as_major(self, data).equal_filter(pred, stream=stream)

    # compress/buff_simd.rs:2294-2442
    def buff_sum_majority(self, data, stream=None) -> float:
        return _as_major(self, data).sum(stream=stream).sum

    # compress/buff_simd.rs:2444-2861 (the reference prints the max)
    def buff_max_majority(self, data, stream=None) -> MaxResult:
        return _as_major(self, data).max(argmax=True, stream=stream)

    # compress/buff_simd.rs:2863-3115 (the reference prints the count)
    def buff_max_majority_range(self, data, s: int, e: int, window: int, stream=None):
        return _as_major(self, data).max_range(s, e, window, stream=stream)

    # compress/buff_simd.rs:1714-1914
    def buff_major_decode_condition(self, data, rows, stream=None):
        return _as_major(self, data).decode_condition(rows, stream=stream)

    # compress/buff_simd.rs:1279-1526
    def buff_range_filter_majority_condition(self, data, pred, rows, stream=None) -> FilterResult:
        return _as_major(self, data).range_filter_condition(pred, rows, stream=stream)


__all__ = ["SplitBDDoubleCompress", "BuffSliceCompress", "Column", "MajorColumn", "SliceColumn",
           "range_filter_sum_image", "filter_image",
           "RapgColumn", "RapgMajorColumn",
           "FilterResult", "MaxResult",
           "FLAG_INTENDED", "FLAG_RAW_BITMAPS", "FLAG_BUFF_LAYOUT", "rows_to_words"]
