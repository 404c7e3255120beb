"""ctypes binding of the C ABI in ``include/buff_gpu.h``.

The library is the in-tree ``buff_gb300/_build/libbuffgpu.so`` built by
``buff_gb300.build``.  There is no fallback: if the library is missing or
fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

OK, EINVAL, ENOMEM, ECUDA, EREFPANIC, ECORRUPT, ETIMEDOUT, ENOTSUP, EFULL, ESCRATCH = range(10)
NOALLOC_MAX_ROWS = 1 << 26
MAX_ROWS = (1 << 32) - 512  # BUFF_MAX_ROWS
FLAG_INTENDED = 0x1
FLAG_RAW_BITMAPS = 0x2
FLAG_BUFF_LAYOUT = 0x4

EXPORTED = [
    "buff_encode_f64", "buff_encode_f32", "buff_col_free", "buff_col_free_async",
    "buff_col_get_info",
    "buff_serialize", "buff_deserialize", "buff_decode", "buff_decode_at_precision",
    "buff_range_filter", "buff_equal_filter", "buff_scalar_range_filter",
    "buff_scalar_equal_filter", "buff_slice_range_filter_nosimd",
    "buff_slice_equal_filter_nosimd", "buff_slice_decode_bs", "buff_range_filter_with_slice",
    "buff_equal_filter_with_slice", "buff_sum", "buff_sum_at_precision",
    "buff_sum_partials_async", "buff_sum_finish", "buff_max", "buff_max_async",
    "buff_range_filter_sum", "buff_range_filter_sum_image", "buff_filter_image",
    "buff_status_string", "buff_last_cuda_error", "buff_kernel_launches",
    "buff_range_filter_noalloc",
    "buff_encode_majority_f64", "buff_encode_majority_f32", "buff_deserialize_majority",
    "buff_decode_majority", "buff_range_filter_majority", "buff_equal_filter_majority",
    "buff_sum_majority", "buff_max_majority", "buff_sum_majority_async",
    "buff_max_majority_async",
    "buff_decode_condition", "buff_major_decode_condition", "buff_decode_selected",
    "buff_range_filter_condition", "buff_range_filter_majority_condition",
    "buff_range_filter_decode",
    "buff_batch_encode_f64", "buff_plan_create", "buff_plan_set_preds", "buff_plan_launch",
    "buff_plan_capture", "buff_plan_replay", "buff_plan_results", "buff_plan_free",
    "buff_batch_autotune",
    "buff_server_create", "buff_server_add_column", "buff_server_start", "buff_server_submit",
    "buff_server_poll", "buff_server_release", "buff_server_stop", "buff_server_free",
    "buff_server_stats", "buff_server_replay", "buff_server_column", "buff_server_store_stats", "buff_copy", "buff_max_range", "buff_slice_max_range", "buff_max_majority_range",
    "buff_slice_encode_f64", "buff_slice_encode_f32", "buff_slice_deserialize",
    "buff_slice_decode", "buff_slice_range_filter", "buff_slice_equal_filter", "buff_slice_sum",
    "buff_slice_buffsum", "buff_slice_max", "buff_slice_buffmax",
    "buff_rapg_encode_f64", "buff_rapg_encode_f32", "buff_rapg_deserialize", "buff_rapg_decode",
    "buff_rapg_decode_at_precision", "buff_rapg_sum", "buff_rapg_sum_at_precision",
    "buff_rapg_encode_outlieru8_f64", "buff_rapg_encode_outlieru8_f32",
    "buff_rapg_major_deserialize", "buff_rapg_decode_majority", "buff_rapg_range_filter_majority",
    "buff_rapg_equal_filter_majority", "buff_rapg_sum_majority", "buff_rapg_max_majority",
]

Q_RANGE, Q_EQUAL, Q_SUM, Q_MAX, Q_DECODE, Q_ENCODE = 0x1, 0x2, 0x4, 0x8, 0x10, 0x20


class BuffError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = _status_string(status)
        if status == ECUDA:
            msg += f" (cudaError {lib().buff_last_cuda_error()})"
        super().__init__(f"{what}: {msg}" if what else msg)


class ReferencePanic(BuffError):
    """The reference implementation panics on this input."""


class ColInfo(C.Structure):
    _fields_ = [("base", C.c_int64), ("n", C.c_uint32), ("ilen", C.c_uint32),
                ("dlen", C.c_uint32), ("fixed_len", C.c_uint32), ("k", C.c_uint32),
                ("r", C.c_uint32), ("scale", C.c_uint64), ("prec", C.c_int32),
                ("precision_exp", C.c_int32), ("flags", C.c_uint32), ("outlier_cols", C.c_uint32),
                ("serialized_bytes", C.c_uint64), ("device_bytes", C.c_uint64)]


class SumResult(C.Structure):
    _fields_ = [("sum", C.c_double), ("exact", C.c_double), ("exact_num_lo", C.c_int64),
                ("exact_num_hi", C.c_int64), ("partials", C.c_uint64 * 9),
                ("n_partials", C.c_uint32), ("reserved", C.c_uint32)]

    @property
    def exact_num(self) -> int:
        return (int(self.exact_num_hi) << 64) | (int(self.exact_num_lo) & ((1 << 64) - 1))


class BatchTune(C.Structure):
    _fields_ = [("tile_rows", C.c_uint32), ("blocks_per_sm", C.c_uint32),
                ("stage", C.c_uint32), ("reserved", C.c_uint32)]

    def __repr__(self):
        return (f"BatchTune(tile_rows={self.tile_rows}, blocks_per_sm={self.blocks_per_sm}, "
                f"stage={self.stage})")


class Query(C.Structure):
    _fields_ = [("col", C.c_void_p), ("ops", C.c_uint32), ("precision", C.c_uint32),
                ("pred", C.c_double), ("words", C.c_void_p), ("values", C.c_void_p)]


class QueryResult(C.Structure):
    _fields_ = [("count", C.c_uint64), ("sum", C.c_double), ("max_value", C.c_double),
                ("max_code", C.c_uint64), ("partials", C.c_uint64 * 9),
                ("n_partials", C.c_uint32), ("status", C.c_int32)]


class ServerConfig(C.Structure):
    _fields_ = [("output_budget_bytes", C.c_uint64), ("store_budget_bytes", C.c_uint64),
                ("max_batch", C.c_uint32), ("max_inflight", C.c_uint32),
                ("batched", C.c_uint32), ("auto_release", C.c_uint32), ("tune", BatchTune)]


class Request(C.Structure):
    _fields_ = [("column", C.c_uint32), ("ops", C.c_uint32), ("precision", C.c_uint32),
                ("reserved", C.c_uint32), ("pred", C.c_double), ("tag", C.c_uint64),
                ("values", C.c_void_p), ("n", C.c_uint64), ("scale", C.c_uint64),
                ("flags", C.c_uint32), ("is_f32", C.c_uint32)]


class Completion(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("status", C.c_int32), ("column", C.c_uint32),
                ("result", QueryResult), ("words", C.c_void_p), ("values", C.c_void_p),
                ("submit_ns", C.c_uint64), ("done_ns", C.c_uint64),
                ("out_off", C.c_uint64 * 2), ("out_cls", C.c_int32 * 2)]


_lib = None


def lib_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True):
    """Loads libbuffgpu.so; builds it first when it is missing and nvcc exists."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run buff_gb300.build.build()")
        _build.build()
    L = C.CDLL(path)
    P = C.c_void_p
    pp = C.POINTER(C.c_void_p)
    L.buff_encode_f64.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_encode_f32.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_col_free.argtypes = [P]
    L.buff_col_free_async.argtypes = [P, P]
    L.buff_col_get_info.argtypes = [P, C.POINTER(ColInfo)]
    L.buff_serialize.argtypes = [P, P, C.c_uint64, C.POINTER(C.c_uint64), P]
    L.buff_deserialize.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_decode.argtypes = [P, P, P]
    L.buff_decode_at_precision.argtypes = [P, C.c_uint32, P, P]
    for nm in ("buff_range_filter", "buff_equal_filter", "buff_range_filter_with_slice",
               "buff_equal_filter_with_slice", "buff_scalar_range_filter",
               "buff_scalar_equal_filter", "buff_slice_range_filter_nosimd",
               "buff_slice_equal_filter_nosimd"):
        getattr(L, nm).argtypes = [P, C.c_double, P, P, P]
    L.buff_slice_decode_bs.argtypes = [P, P, P]
    L.buff_range_filter_noalloc.argtypes = [P, C.c_double, P, P, P]
    L.buff_sum.argtypes = [P, C.POINTER(SumResult), P]
    L.buff_sum_at_precision.argtypes = [P, C.c_uint32, P, P]
    L.buff_sum_partials_async.argtypes = [P, P, P]
    L.buff_sum_finish.argtypes = [P, P, C.POINTER(SumResult)]
    L.buff_range_filter_sum.argtypes = [P, C.c_double, P, P, P, P]
    L.buff_range_filter_sum_image.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, C.c_double,
                                              P, P, C.POINTER(SumResult), P]
    L.buff_filter_image.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, C.c_int, C.c_double,
                                    P, P, P]
    L.buff_max.argtypes = [P, P, P, P, P, P]
    L.buff_max_async.argtypes = [P, P, P]
    L.buff_encode_majority_f64.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_encode_majority_f32.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_deserialize_majority.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_decode_majority.argtypes = [P, P, P]
    L.buff_range_filter_majority.argtypes = [P, C.c_double, P, P, P]
    L.buff_equal_filter_majority.argtypes = [P, C.c_double, P, P, P]
    L.buff_sum_majority.argtypes = [P, C.POINTER(SumResult), P]
    L.buff_max_majority.argtypes = [P, P, P, P, P, P]
    L.buff_sum_majority_async.argtypes = [P, P, P, P]
    L.buff_max_majority_async.argtypes = [P, P, P]
    L.buff_decode_condition.argtypes = [P, P, C.c_uint64, P, P]
    L.buff_major_decode_condition.argtypes = [P, P, C.c_uint64, P, P, P]
    L.buff_decode_selected.argtypes = [P, P, P, P, P]
    L.buff_range_filter_condition.argtypes = [P, C.c_double, P, P, P, P]
    L.buff_range_filter_majority_condition.argtypes = [P, C.c_double, P, P, P, P]
    L.buff_range_filter_decode.argtypes = [P, C.c_double, P, P, P, P]
    L.buff_batch_encode_f64.argtypes = [P, P, P, C.c_uint32, C.c_uint32, P, P, P]
    L.buff_plan_create.argtypes = [P, C.c_uint32, P, P, pp]
    L.buff_plan_set_preds.argtypes = [P, P]
    L.buff_plan_launch.argtypes = [P, P]
    L.buff_plan_capture.argtypes = [P, P]
    L.buff_plan_replay.argtypes = [P, P]
    L.buff_plan_results.argtypes = [P, P, P]
    L.buff_plan_free.argtypes = [P]
    L.buff_batch_autotune.argtypes = [P, C.c_uint32, P, P, P]
    L.buff_server_create.argtypes = [C.POINTER(ServerConfig), pp]
    L.buff_server_add_column.argtypes = [P, P, C.POINTER(C.c_uint32)]
    L.buff_server_start.argtypes = [P]
    L.buff_server_submit.argtypes = [P, P, C.c_uint32]
    L.buff_server_poll.argtypes = [P, P, C.c_uint32, C.POINTER(C.c_uint32)]
    L.buff_server_release.argtypes = [P, P]
    L.buff_server_stop.argtypes = [P]
    L.buff_server_free.argtypes = [P]
    L.buff_server_stats.argtypes = [P, P, P, P]
    L.buff_server_column.argtypes = [P, C.c_uint32, pp]
    L.buff_server_store_stats.argtypes = [P, P, P]
    L.buff_server_replay.argtypes = [P, P, P, C.c_uint32, P, P, P]
    L.buff_copy.argtypes = [P, P, C.c_uint64, P]
    L.buff_max_range.argtypes = [P, C.c_uint32, C.c_uint32, C.c_uint32, P, P, P]
    L.buff_slice_max_range.argtypes = [P, C.c_uint32, C.c_uint32, C.c_uint32, P, P, P]
    L.buff_max_majority_range.argtypes = [P, C.c_uint32, C.c_uint32, C.c_uint32, P, P, P]
    L.buff_slice_encode_f64.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_slice_encode_f32.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_slice_deserialize.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_slice_decode.argtypes = [P, P, P]
    L.buff_slice_range_filter.argtypes = [P, C.c_double, P, P, P]
    L.buff_slice_equal_filter.argtypes = [P, C.c_double, P, P, P]
    L.buff_slice_sum.argtypes = [P, P, P]
    L.buff_slice_buffsum.argtypes = [P, P, P]
    L.buff_slice_max.argtypes = [P, P, P, P, P]
    L.buff_slice_buffmax.argtypes = [P, P, P, P, P]
    L.buff_rapg_encode_f64.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_rapg_encode_f32.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_rapg_deserialize.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_rapg_decode.argtypes = [P, P, P, P]
    L.buff_rapg_decode_at_precision.argtypes = [P, C.c_uint32, P, P, P]
    L.buff_rapg_sum.argtypes = [P, P, P]
    L.buff_rapg_sum_at_precision.argtypes = [P, C.c_uint32, P, P]
    L.buff_rapg_encode_outlieru8_f64.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_rapg_encode_outlieru8_f32.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_rapg_major_deserialize.argtypes = [P, C.c_uint64, C.c_uint64, C.c_uint32, P, pp]
    L.buff_rapg_decode_majority.argtypes = [P, P, P]
    L.buff_rapg_range_filter_majority.argtypes = [P, C.c_double, P, P, P]
    L.buff_rapg_equal_filter_majority.argtypes = [P, C.c_double, P, P, P]
    L.buff_rapg_sum_majority.argtypes = [P, C.POINTER(SumResult), P]
    L.buff_rapg_max_majority.argtypes = [P, P, P, P, P, P]
    L.buff_status_string.argtypes = [C.c_int]
    L.buff_status_string.restype = C.c_char_p
    L.buff_last_cuda_error.restype = C.c_int
    L.buff_kernel_launches.restype = C.c_uint64
    _lib = L
    return L


def _status_string(st: int) -> str:
    try:
        return lib().buff_status_string(st).decode()
    except Exception:  # pragma: no cover - library unavailable
        return f"status {st}"


def check(st: int, what: str = ""):
    if st == OK:
        return
    if st == EREFPANIC:
        raise ReferencePanic(st, what)
    raise BuffError(st, what)


def ptr(x):
    """Raw address of a numpy array, a torch tensor, an int or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    raise TypeError(f"cannot take the address of {type(x)}")


def stream_handle(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


def copy_bytes(src: int, nbytes: int) -> bytes:
    """Bytes at a device (or host) address, copied to the host."""
    buf = np.empty(max(nbytes, 1), dtype=np.uint8)
    check(lib().buff_copy(buf.ctypes.data, src, nbytes, None), "copy")
    return buf[:nbytes].tobytes()


def kernel_launches() -> int:
    return int(lib().buff_kernel_launches())
