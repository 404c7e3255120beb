"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only the test suite, the smoke check and the benchmark's CPU-baseline leg
import this module.  Parity of the codec outputs is unpinned (no reference
test asserts them); the bit-packing and bitmap helpers are pinned to the
reference's known-answer tests.  It builds ``oracle/_build/libbuff_oracle.so`` from
``buff_oracle.c`` on first use when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libbuff_oracle.so")
_lib = None

OK, PANIC, EINVAL, ENOMEM = 0, 1, 2, 3
INTENDED = 1


class OraclePanic(RuntimeError):
    """The reference panics on this input (unwrap/assert/index failure)."""


def build() -> str:
    srcs = [os.path.join(_HERE, f) for f in ("buff_oracle.c", "buff_oracle_major.c",
                                             "buff_oracle_cond.c", "buff_oracle_slice.c", "buff_oracle_rapg.c",
                                             "buff_oracle.h",
                                             "Makefile")]
    if (not os.path.exists(_LIB_PATH)) or any(os.path.getmtime(_LIB_PATH) < os.path.getmtime(s)
                                               for s in srcs):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class Header(C.Structure):
    _fields_ = [("base", C.c_int64), ("n", C.c_uint32), ("ilen", C.c_uint32),
                ("dlen", C.c_uint32), ("fixed_len", C.c_uint32), ("k", C.c_uint32),
                ("r", C.c_uint32), ("slice_off", C.c_size_t), ("tail_off", C.c_size_t)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        P = C.c_void_p
        u8p = C.POINTER(C.c_uint8)
        L.or_prec_of_scale.argtypes = [C.c_uint64]
        L.or_dlen_of_prec.argtypes = [C.c_int]
        L.or_precision_exp.argtypes = [C.c_int]
        L.or_fetch_fixed_aligned.argtypes = [C.c_double, C.c_int32, C.c_uint64]
        L.or_fetch_fixed_aligned.restype = C.c_int64
        L.or_fixed_len_of_delta.argtypes = [C.c_int64]
        L.or_fixed_len_of_delta.restype = C.c_uint32
        L.or_bitpack_write_seq.argtypes = [P, P, C.c_size_t, P, C.c_size_t, P]
        L.or_bitpack_read_seq.argtypes = [P, C.c_size_t, P, C.c_size_t, P]
        L.or_bviter_positions.argtypes = [P, C.c_size_t, P, C.c_size_t]
        L.or_bviter_positions.restype = C.c_size_t
        L.or_bitvec_to_binary.argtypes = [P, C.c_size_t, C.c_uint64, P]
        L.or_bitvec_to_binary.restype = C.c_size_t
        L.or_movemask_gt.argtypes = [P, C.c_uint8]
        L.or_movemask_gt.restype = C.c_uint32
        L.or_movemask_eq.argtypes = [P, C.c_uint8]
        L.or_movemask_eq.restype = C.c_uint32
        L.or_encode.argtypes = [P, C.c_uint32, C.c_uint64, C.c_int, C.c_uint, C.POINTER(u8p),
                                C.POINTER(C.c_size_t)]
        L.or_encode_f32.argtypes = L.or_encode.argtypes
        L.or_free.argtypes = [P]
        L.or_parse_header.argtypes = [P, C.c_size_t, C.POINTER(Header)]
        L.or_decode.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, P]
        for nm in ("or_range_filter", "or_equal_filter"):
            getattr(L, nm).argtypes = [P, C.c_size_t, C.c_uint64, C.c_double, C.c_uint, P, P, P]
        for nm in ("or_range_filter_with_slice", "or_equal_filter_with_slice"):
            getattr(L, nm).argtypes = [P, C.c_size_t, C.c_uint64, C.c_double, P, P, P]
        for nm in ("or_scalar_range_filter", "or_scalar_equal_filter"):
            getattr(L, nm).argtypes = [P, C.c_size_t, C.c_uint64, C.c_double, C.c_int, P, P, P]
        L.or_sum.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, C.c_uint, P, P, P]
        L.or_max.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, C.c_uint, P, P, P, P]
        L.or_decode_at_precision.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, C.c_uint32,
                                             C.c_uint, P]
        L.or_sum_at_precision.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, C.c_uint32,
                                          C.c_uint, P]
        L.or_snappy_max_compressed.argtypes = [C.c_size_t]
        L.or_snappy_max_compressed.restype = C.c_size_t
        L.or_snappy_compress.argtypes = [P, C.c_size_t, P, C.c_size_t, P]
        L.or_snappy_decompress.argtypes = [P, C.c_size_t, P, C.c_size_t, P]
        L.or_encode_outlieru8.argtypes = [P, C.c_uint32, C.c_uint64, C.POINTER(u8p),
                                          C.POINTER(C.c_size_t)]
        L.or_encode_majority.argtypes = [P, C.c_uint32, C.c_uint64, C.c_int, C.POINTER(u8p),
                                         C.POINTER(C.c_size_t)]
        L.or_majority_layout.argtypes = [P, C.c_size_t, C.c_int, P, P, P, P]
        L.or_decode_majority.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, P]
        for nm in ("or_range_filter_majority", "or_equal_filter_majority"):
            getattr(L, nm).argtypes = [P, C.c_size_t, C.c_uint64, C.c_double, C.c_int, P, P, P]
        L.or_sum_majority.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, P, P]
        L.or_max_majority.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, P, P, P, P]
        L.or_decode_condition.argtypes = [P, C.c_size_t, C.c_uint64, P, C.c_size_t, P]
        L.or_major_decode_condition.argtypes = [P, C.c_size_t, C.c_uint64, P, C.c_size_t, P, P]
        for nm in ("or_range_filter_condition", "or_range_filter_majority_condition"):
            getattr(L, nm).argtypes = [P, C.c_size_t, C.c_uint64, C.c_double, P, C.c_size_t, P, P]
        L.or_slice_encode.argtypes = [P, C.c_uint32, C.c_uint64, C.POINTER(u8p),
                                      C.POINTER(C.c_size_t)]
        L.or_slice_decode.argtypes = [P, C.c_size_t, C.c_uint64, P]
        for nm in ("or_slice_range_filter", "or_slice_equal_filter",
                   "or_slice_range_filter_nosimd", "or_slice_equal_filter_nosimd"):
            getattr(L, nm).argtypes = [P, C.c_size_t, C.c_uint64, C.c_double, P, P, P]
        L.or_slice_decode_bs.argtypes = [P, C.c_size_t, C.c_uint64, P]
        L.or_slice_sum.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, P]
        L.or_slice_max.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, P, P, P]
        L.or_roaring_serialize.argtypes = [P, C.c_size_t, C.POINTER(u8p), C.POINTER(C.c_size_t)]
        L.or_roaring_parse.argtypes = [P, C.c_size_t, C.POINTER(C.POINTER(C.c_uint32)),
                                       C.POINTER(C.c_size_t)]
        L.or_rapg_encode.argtypes = [P, C.c_uint32, C.c_uint64, C.POINTER(u8p),
                                     C.POINTER(C.c_size_t)]
        L.or_rapg_decode.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, P, P]
        L.or_rapg_sum.argtypes = [P, C.c_size_t, C.c_uint64, C.c_int, P]
        L.or_rapg_layout.argtypes = [P, C.c_size_t, P, P, P, P]
        L.or_slice_max_range.argtypes = [P, C.c_size_t, C.c_uint64, C.c_uint32, C.c_uint32,
                                         C.c_uint32, P, C.c_size_t, P]
        L.or_max_range.argtypes = [P, C.c_size_t, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                   P, P]
        L.or_max_majority_range.argtypes = [P, C.c_size_t, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                   P, P]
        L.or_bench_filter_sum.argtypes = [P, C.c_size_t, C.c_uint64, C.c_double, C.c_int,
                                          C.c_int, P, P]
        L.or_bench_filter_sum.restype = C.c_double
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _check(rc: int):
    if rc == PANIC:
        raise OraclePanic("reference panics on this input")
    if rc != OK:
        raise RuntimeError(f"oracle error {rc}")


# --- scalar helpers -------------------------------------------------------
def prec_of_scale(scale: int) -> int:
    return lib().or_prec_of_scale(scale)


def dlen_of_prec(prec: int) -> int:
    return lib().or_dlen_of_prec(prec)


def precision_exp(prec: int) -> int:
    return lib().or_precision_exp(prec)


def fetch_fixed_aligned(v: float, pexp: int, dlen: int) -> int:
    return lib().or_fetch_fixed_aligned(v, pexp, dlen)


# --- BitPack / BitVec known-answer helpers --------------------------------
def bitpack_write(pairs):
    vals = np.array([p[0] for p in pairs], dtype=np.uint32)
    bits = np.array([p[1] for p in pairs], dtype=np.uint32)
    out = np.zeros(64 + 8 * len(pairs), dtype=np.uint8)
    ln = C.c_size_t(0)
    _check(lib().or_bitpack_write_seq(_ptr(vals), _ptr(bits), len(pairs), _ptr(out), out.size,
                                      C.byref(ln)))
    return out[: ln.value].tobytes()


def bitpack_read(buf: bytes, bits):
    b = np.frombuffer(buf, dtype=np.uint8).copy()
    bb = np.array(bits, dtype=np.uint32)
    out = np.zeros(len(bits), dtype=np.uint32)
    _check(lib().or_bitpack_read_seq(_ptr(b), b.size, _ptr(bb), len(bits), _ptr(out)))
    return [int(x) for x in out]


def bviter(words: np.ndarray):
    w = np.ascontiguousarray(words, dtype=np.uint32)
    cap = int(sum(bin(int(x)).count("1") for x in w)) + 1
    out = np.zeros(cap, dtype=np.uint64)
    cnt = lib().or_bviter_positions(_ptr(w), w.size, _ptr(out), cap)
    return [int(x) for x in out[:cnt]]


def bitvec_to_binary(words: np.ndarray, nbits: int) -> bytes:
    w = np.ascontiguousarray(words, dtype=np.uint32)
    out = np.zeros(8 + 4 * w.size, dtype=np.uint8)
    ln = lib().or_bitvec_to_binary(_ptr(w), w.size, nbits, _ptr(out))
    return out[:ln].tobytes()


def movemask(bytes32: bytes, pred: int):
    b = np.frombuffer(bytes32, dtype=np.uint8).copy()
    return lib().or_movemask_gt(_ptr(b), pred), lib().or_movemask_eq(_ptr(b), pred)


# --- codec ----------------------------------------------------------------
def encode(x, scale: int, flipped: bool = True, flags: int = 0) -> bytes:
    x = np.asarray(x)
    if x.dtype == np.float32:
        fn, arr = lib().or_encode_f32, np.ascontiguousarray(x, dtype=np.float32)
    else:
        fn, arr = lib().or_encode, np.ascontiguousarray(x, dtype=np.float64)
    out = C.POINTER(C.c_uint8)()
    ln = C.c_size_t(0)
    _check(fn(_ptr(arr), arr.size, scale, int(flipped), flags, C.byref(out), C.byref(ln)))
    try:
        return C.string_at(out, ln.value)
    finally:
        lib().or_free(out)


def header(buf: bytes) -> Header:
    b = np.frombuffer(buf, dtype=np.uint8)
    h = Header()
    _check(lib().or_parse_header(_ptr(b), b.size, C.byref(h)))
    return h


def _buf(buf: bytes):
    return np.frombuffer(buf, dtype=np.uint8)


def decode(buf: bytes, scale: int, flipped: bool = True) -> np.ndarray:
    b = _buf(buf)
    out = np.zeros(max(header(buf).n, 1), dtype=np.float64)
    _check(lib().or_decode(_ptr(b), b.size, scale, int(flipped), _ptr(out)))
    return out[: header(buf).n]


def _filter(fn, buf, scale, pred, flags=None):
    b = _buf(buf)
    n = header(buf).n
    words = np.zeros(max((n + 31) // 32, 1), dtype=np.uint32)
    cnt = np.zeros(1, dtype=np.uint64)
    early = np.zeros(1, dtype=np.int32)
    if flags is None:
        rc = fn(_ptr(b), b.size, scale, pred, _ptr(words), _ptr(cnt), _ptr(early))
    else:
        rc = fn(_ptr(b), b.size, scale, pred, flags, _ptr(words), _ptr(cnt), _ptr(early))
    _check(rc)
    return words[: (n + 31) // 32], int(cnt[0]), bool(early[0])


def range_filter(buf, scale, pred, flags=0):
    return _filter(lib().or_range_filter, buf, scale, pred, flags)


def equal_filter(buf, scale, pred, flags=0):
    return _filter(lib().or_equal_filter, buf, scale, pred, flags)


def range_filter_with_slice(buf, scale, pred):
    return _filter(lib().or_range_filter_with_slice, buf, scale, pred)


def equal_filter_with_slice(buf, scale, pred):
    return _filter(lib().or_equal_filter_with_slice, buf, scale, pred)


def scalar_range_filter(buf, scale, pred, flipped=False):
    """buff_range_filter (buff_simd.rs:4507-4679) on a buff-layout image."""
    return _filter(lambda *a: lib().or_scalar_range_filter(*a[:4], int(flipped), *a[4:]),
                   buf, scale, pred)


def scalar_equal_filter(buf, scale, pred, flipped=False):
    """buff_equal_filter (buff_simd.rs:4925-5094) on a buff-layout image."""
    return _filter(lambda *a: lib().or_scalar_equal_filter(*a[:4], int(flipped), *a[4:]),
                   buf, scale, pred)


def buff_sum(buf, scale, flipped=True, flags=0):
    """Returns (reference f64 sum, partials list, exact numerator int)."""
    b = _buf(buf)
    s = np.zeros(1, dtype=np.float64)
    parts = np.zeros(16, dtype=np.uint64)
    ex = np.zeros(2, dtype=np.int64)
    _check(lib().or_sum(_ptr(b), b.size, scale, int(flipped), flags, _ptr(s), _ptr(parts),
                        _ptr(ex)))
    h = header(buf)
    exact = (int(ex[1]) << 64) | (int(ex[0]) & ((1 << 64) - 1))
    return float(s[0]), [int(p) for p in parts[: h.k + (1 if h.r else 0)]], exact


def buff_max(buf, scale, flipped=True, flags=0):
    """Returns (max value, max code, argmax words, argmax count)."""
    b = _buf(buf)
    n = header(buf).n
    mv = np.zeros(1, dtype=np.float64)
    mc = np.zeros(1, dtype=np.uint64)
    words = np.zeros(max((n + 31) // 32, 1), dtype=np.uint32)
    cnt = np.zeros(1, dtype=np.uint64)
    _check(lib().or_max(_ptr(b), b.size, scale, int(flipped), flags, _ptr(mv), _ptr(mc),
                        _ptr(words), _ptr(cnt)))
    return float(mv[0]), int(mc[0]), words[: (n + 31) // 32], int(cnt[0])


def decode_at_precision(buf, scale, precision, flipped=True, flags=0):
    b = _buf(buf)
    n = header(buf).n
    out = np.zeros(max(n, 1), dtype=np.float64)
    _check(lib().or_decode_at_precision(_ptr(b), b.size, scale, int(flipped), precision, flags,
                                        _ptr(out)))
    return out[:n]


def sum_at_precision(buf, scale, precision, flipped=True, flags=0):
    b = _buf(buf)
    s = np.zeros(1, dtype=np.float64)
    _check(lib().or_sum_at_precision(_ptr(b), b.size, scale, int(flipped), precision, flags,
                                     _ptr(s)))
    return float(s[0])


def bench_filter_sum(buf, scale, pred, nthreads=1, reps=1):
    """Times the CPU restatement of range filter + sum (seconds, count, sum)."""
    b = _buf(buf)
    cnt = np.zeros(1, dtype=np.uint64)
    s = np.zeros(1, dtype=np.float64)
    t = lib().or_bench_filter_sum(_ptr(b), b.size, scale, pred, nthreads, reps, _ptr(cnt), _ptr(s))
    return t, int(cnt[0]), float(s[0])


# --- buff-major (outlier) format -------------------------------------------
BM_SNAPPY, BM_RAW, BM_ROARING = 0, 1, 2


def snappy_compress(data: bytes) -> bytes:
    b = np.frombuffer(data, dtype=np.uint8).copy() if data else np.zeros(1, dtype=np.uint8)
    cap = lib().or_snappy_max_compressed(len(data))
    out = np.zeros(cap, dtype=np.uint8)
    ln = C.c_size_t(0)
    _check(lib().or_snappy_compress(_ptr(b), len(data), _ptr(out), cap, C.byref(ln)))
    return out[: ln.value].tobytes()


def snappy_decompress(data: bytes) -> bytes:
    b = np.frombuffer(data, dtype=np.uint8).copy()
    ln = C.c_size_t(0)
    _check(lib().or_snappy_decompress(_ptr(b), b.size, None, 0, C.byref(ln)))
    out = np.zeros(max(ln.value, 1), dtype=np.uint8)
    _check(lib().or_snappy_decompress(_ptr(b), b.size, _ptr(out), out.size, C.byref(ln)))
    return out[: ln.value].tobytes()


def encode_majority(x, scale: int, bm_mode: int = BM_SNAPPY) -> bytes:
    arr = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    out = C.POINTER(C.c_uint8)()
    ln = C.c_size_t(0)
    _check(lib().or_encode_majority(_ptr(arr), arr.size, scale, bm_mode, C.byref(out),
                                    C.byref(ln)))
    try:
        return C.string_at(out, ln.value)
    finally:
        lib().or_free(out)


def encode_outlieru8(x, scale: int) -> bytes:
    """byte_residue_encode_outlieru8 (split_double.rs:957-1240): read the
    image with bm_mode=BM_ROARING."""
    arr = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    out = C.POINTER(C.c_uint8)()
    ln = C.c_size_t(0)
    _check(lib().or_encode_outlieru8(_ptr(arr), arr.size, scale, C.byref(out), C.byref(ln)))
    try:
        return C.string_at(out, ln.value)
    finally:
        lib().or_free(out)


def majority_layout(buf: bytes, bm_mode: int = BM_SNAPPY):
    b = _buf(buf)
    nc = np.zeros(1, dtype=np.uint32)
    maj = np.zeros(8, dtype=np.uint8)
    nout = np.zeros(8, dtype=np.uint32)
    off = np.zeros(1, dtype=np.uint64)
    _check(lib().or_majority_layout(_ptr(b), b.size, bm_mode, _ptr(nc), _ptr(maj), _ptr(nout),
                                    _ptr(off)))
    k = int(nc[0])
    return k, [int(v) for v in maj[:k]], [int(v) for v in nout[:k]], int(off[0])


def decode_majority(buf, scale, bm_mode=BM_SNAPPY):
    b = _buf(buf)
    n = header(buf).n
    out = np.zeros(max(n, 1), dtype=np.float64)
    _check(lib().or_decode_majority(_ptr(b), b.size, scale, bm_mode, _ptr(out)))
    return out[:n]


def _filter_major(fn, buf, scale, pred, bm_mode):
    b = _buf(buf)
    n = header(buf).n
    words = np.zeros(max((n + 31) // 32, 1), dtype=np.uint32)
    cnt = np.zeros(1, dtype=np.uint64)
    early = np.zeros(1, dtype=np.int32)
    _check(fn(_ptr(b), b.size, scale, pred, bm_mode, _ptr(words), _ptr(cnt), _ptr(early)))
    return words[: (n + 31) // 32], int(cnt[0]), bool(early[0])


def range_filter_majority(buf, scale, pred, bm_mode=BM_SNAPPY):
    return _filter_major(lib().or_range_filter_majority, buf, scale, pred, bm_mode)


def equal_filter_majority(buf, scale, pred, bm_mode=BM_SNAPPY):
    return _filter_major(lib().or_equal_filter_majority, buf, scale, pred, bm_mode)


def sum_majority(buf, scale, bm_mode=BM_SNAPPY):
    b = _buf(buf)
    s = np.zeros(1, dtype=np.float64)
    parts = np.zeros(16, dtype=np.uint64)
    _check(lib().or_sum_majority(_ptr(b), b.size, scale, bm_mode, _ptr(s), _ptr(parts)))
    return float(s[0]), [int(p) for p in parts]


def max_majority(buf, scale, bm_mode=BM_SNAPPY):
    b = _buf(buf)
    n = header(buf).n
    mv = np.zeros(1, dtype=np.float64)
    mc = np.zeros(1, dtype=np.uint64)
    words = np.zeros(max((n + 31) // 32, 1), dtype=np.uint32)
    cnt = np.zeros(1, dtype=np.uint64)
    _check(lib().or_max_majority(_ptr(b), b.size, scale, bm_mode, _ptr(mv), _ptr(mc),
                                 _ptr(words), _ptr(cnt)))
    return float(mv[0]), int(mc[0]), words[: (n + 31) // 32], int(cnt[0])


# --- row-conditioned reads of the buff layout (buff_oracle_cond.c) ---------

def _rows(rows):
    return np.ascontiguousarray(np.asarray(rows, dtype=np.uint64).reshape(-1))


def decode_condition(buf, scale, rows):
    """buff_decode_condition (buff_simd.rs:1528-1712) on a buff-layout image."""
    b = _buf(buf)
    r = _rows(rows)
    out = np.zeros(max(r.size, 1), dtype=np.float64)
    _check(lib().or_decode_condition(_ptr(b), b.size, scale, _ptr(r), r.size, _ptr(out)))
    return out[: r.size]


def major_decode_condition(buf, scale, rows):
    """buff_major_decode_condition (buff_simd.rs:1714-1914)."""
    b = _buf(buf)
    r = _rows(rows)
    out = np.zeros(max(r.size, 1), dtype=np.float64)
    nout = C.c_size_t(0)
    _check(lib().or_major_decode_condition(_ptr(b), b.size, scale, _ptr(r), r.size, _ptr(out),
                                           C.byref(nout)))
    return out[: nout.value]


def _filter_cond(fn, buf, scale, pred, rows):
    b = _buf(buf)
    r = _rows(rows)
    n = header(buf).n
    words = np.zeros(max((n + 31) // 32, 1), dtype=np.uint32)
    cnt = np.zeros(1, dtype=np.uint64)
    _check(fn(_ptr(b), b.size, scale, pred, _ptr(r), r.size, _ptr(words), _ptr(cnt)))
    return words[: (n + 31) // 32], int(cnt[0])


def range_filter_condition(buf, scale, pred, rows):
    """buff_range_filter_condition (buff_simd.rs:4683-4921)."""
    return _filter_cond(lib().or_range_filter_condition, buf, scale, pred, rows)


def range_filter_majority_condition(buf, scale, pred, rows):
    """buff_range_filter_majority_condition (buff_simd.rs:1279-1526)."""
    return _filter_cond(lib().or_range_filter_majority_condition, buf, scale, pred, rows)


def max_range(buf, scale, s, e, window):
    """buff_max_range (buff_simd.rs:5096-5334) on a buff-layout image."""
    b = _buf(buf)
    nw = (e - s) // window if (window and e >= s) else 0
    out = np.zeros(max(nw, 1), dtype=np.float64)
    n = C.c_size_t(0)
    _check(lib().or_max_range(_ptr(b), b.size, scale, s, e, window, _ptr(out), C.byref(n)))
    return out[: n.value]


# --- buff-slice layout (buff_oracle_slice.c) --------------------------------

def slice_encode(x, scale: int) -> bytes:
    """buff_slice_encode (buff_slice.rs:298-437)."""
    arr = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    out = C.POINTER(C.c_uint8)()
    ln = C.c_size_t(0)
    _check(lib().or_slice_encode(_ptr(arr), arr.size, scale, C.byref(out), C.byref(ln)))
    try:
        return C.string_at(out, ln.value)
    finally:
        lib().or_free(out)


def slice_decode(buf, scale):
    b = _buf(buf)
    n = header(buf).n
    out = np.zeros(max(n, 1), dtype=np.float64)
    _check(lib().or_slice_decode(_ptr(b), b.size, scale, _ptr(out)))
    return out[:n]


def _slice_filter(fn, buf, scale, pred):
    b = _buf(buf)
    n = header(buf).n
    words = np.zeros(max((n + 31) // 32, 1), dtype=np.uint32)
    cnt = np.zeros(1, dtype=np.uint64)
    early = np.zeros(1, dtype=np.int32)
    _check(fn(_ptr(b), b.size, scale, pred, _ptr(words), _ptr(cnt), _ptr(early)))
    return words[: (n + 31) // 32], int(cnt[0]), bool(early[0])


def slice_range_filter(buf, scale, pred):
    return _slice_filter(lib().or_slice_range_filter, buf, scale, pred)


def slice_equal_filter(buf, scale, pred):
    return _slice_filter(lib().or_slice_equal_filter, buf, scale, pred)


def slice_range_filter_nosimd(buf, scale, pred):
    """buff_slice_range_filter_nosimd (buff_slice.rs:1753-1871)."""
    return _slice_filter(lib().or_slice_range_filter_nosimd, buf, scale, pred)


def slice_equal_filter_nosimd(buf, scale, pred):
    """buff_slice_equal_filter_nosimd (buff_slice.rs:1873-1991)."""
    return _slice_filter(lib().or_slice_equal_filter_nosimd, buf, scale, pred)


def slice_decode_bs(buf, scale):
    """buff_slice_decode_bs (buff_slice.rs:1184-1262)."""
    b = _buf(buf)
    n = header(buf).n
    out = np.zeros(max(n, 1), dtype=np.float64)
    _check(lib().or_slice_decode_bs(_ptr(b), b.size, scale, _ptr(out)))
    return out[:n]


def slice_sum(buf, scale, any_width=False):
    b = _buf(buf)
    s = np.zeros(1, dtype=np.float64)
    _check(lib().or_slice_sum(_ptr(b), b.size, scale, 1 if any_width else 0, _ptr(s)))
    return float(s[0])


def slice_max(buf, scale, any_width=False):
    b = _buf(buf)
    n = header(buf).n
    mv = np.zeros(1, dtype=np.float64)
    words = np.zeros(max((n + 31) // 32, 1), dtype=np.uint32)
    cnt = np.zeros(1, dtype=np.uint64)
    _check(lib().or_slice_max(_ptr(b), b.size, scale, 1 if any_width else 0, _ptr(mv),
                              _ptr(words), _ptr(cnt)))
    return float(mv[0]), words[: (n + 31) // 32], int(cnt[0])


def slice_max_range(buf, scale, s, e, window):
    """buff_slice_max_range (buff_slice.rs:930-1099): per-window maxima."""
    b = _buf(buf)
    n = header(buf).n
    cap = (min(e, n) - s + window - 1) // window + 1 if (window and min(e, n) > s) else 1
    out = np.zeros(cap, dtype=np.float64)
    k = C.c_size_t(0)
    _check(lib().or_slice_max_range(_ptr(b), b.size, scale, s, e, window, _ptr(out), cap,
                                    C.byref(k)))
    return out[: k.value]


# --- RAPG byte_residue formats (buff_oracle_rapg.c) --------------------------

def roaring_serialize(rows) -> bytes:
    """croaring Bitmap::create + ascending add + run_optimize + serialize."""
    r = np.ascontiguousarray(np.asarray(rows, dtype=np.uint32))
    out = C.POINTER(C.c_uint8)()
    ln = C.c_size_t(0)
    _check(lib().or_roaring_serialize(_ptr(r), r.size, C.byref(out), C.byref(ln)))
    try:
        return C.string_at(out, ln.value)
    finally:
        lib().or_free(out)


def roaring_parse(buf) -> np.ndarray:
    b = _buf(buf)
    out = C.POINTER(C.c_uint32)()
    n = C.c_size_t(0)
    _check(lib().or_roaring_parse(_ptr(b), b.size, C.byref(out), C.byref(n)))
    try:
        return np.ctypeslib.as_array(out, shape=(n.value,)).copy() if n.value else \
            np.zeros(0, dtype=np.uint32)
    finally:
        lib().or_free(out)


def rapg_encode(x, scale: int) -> bytes:
    """byte_residue_encode (split_double.rs:624-955)."""
    arr = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    out = C.POINTER(C.c_uint8)()
    ln = C.c_size_t(0)
    _check(lib().or_rapg_encode(_ptr(arr), arr.size, scale, C.byref(out), C.byref(ln)))
    try:
        return C.string_at(out, ln.value)
    finally:
        lib().or_free(out)


def rapg_decode(buf, scale, precision=-1):
    """byte_residue_decode (precision -1) / byte_residue_decode_with_precision."""
    b = _buf(buf)
    n = header(buf).n
    out = np.zeros(max(n, 1), dtype=np.float64)
    k = C.c_size_t(0)
    _check(lib().or_rapg_decode(_ptr(b), b.size, scale, precision, _ptr(out), C.byref(k)))
    return out[: k.value]


def rapg_sum(buf, scale, precision=-1) -> float:
    """byte_residue_sum (precision -1) / byte_residue_sum_with_precision."""
    b = _buf(buf)
    s = np.zeros(1, dtype=np.float64)
    _check(lib().or_rapg_sum(_ptr(b), b.size, scale, precision, _ptr(s)))
    return float(s[0])


def rapg_layout(buf):
    """(columns, bitmap sizes, outlier counts, bitmap byte offsets)."""
    b = _buf(buf)
    nc = np.zeros(1, dtype=np.uint32)
    sizes = np.zeros(8, dtype=np.uint32)
    nouts = np.zeros(8, dtype=np.uint32)
    offs = np.zeros(8, dtype=np.uint64)
    _check(lib().or_rapg_layout(_ptr(b), b.size, _ptr(nc), _ptr(sizes), _ptr(nouts), _ptr(offs)))
    c = int(nc[0])
    return c, sizes[:c].tolist(), nouts[:c].tolist(), offs[:c].tolist()


def max_majority_range(buf, scale, s, e, window):
    """buff_max_majority_range (buff_simd.rs:2863-3115) on a buff-major image."""
    b = _buf(buf)
    nw = (e - s) // window if (window and e >= s) else 0
    out = np.zeros(max(nw, 1), dtype=np.float64)
    n = C.c_size_t(0)
    _check(lib().or_max_majority_range(_ptr(b), b.size, scale, s, e, window, _ptr(out),
                                       C.byref(n)))
    return out[: n.value]
