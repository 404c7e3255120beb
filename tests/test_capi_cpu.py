"""CPU-side checks of the C ABI library: it loads without a GPU, exports every
function include/buff_gpu.h declares, and its host-only entry points behave."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from buff_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for hdr in os.listdir(os.path.join(ROOT, "include")):
        if not hdr.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", hdr)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(buff_[a-z_0-9]+)\s*\(", src, re.M)
    return sorted(set(names))


def test_header_declares_the_documented_entry_points():
    decl = declared_functions()
    assert len(decl) >= len(capi.EXPORTED)
    for nm in capi.EXPORTED:
        assert nm in decl


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    missing = [nm for nm in declared_functions() if not hasattr(L, nm)]
    assert not missing, missing


def test_status_strings_and_counters():
    L = capi.lib()
    assert L.buff_status_string(0) == b"ok"
    assert b"panics" in L.buff_status_string(capi.EREFPANIC)
    assert L.buff_status_string(999) == b"unknown status"
    assert capi.kernel_launches() >= 0


def test_null_arguments_rejected_without_gpu():
    L = capi.lib()
    assert L.buff_col_free(None) == capi.EINVAL
    assert L.buff_col_get_info(None, None) == capi.EINVAL
    h = C.c_void_p()
    assert L.buff_encode_f64(None, 5, 10000, 0, None, C.byref(h)) == capi.EINVAL
    assert L.buff_encode_f64(None, 1 << 32, 10000, 0, None, C.byref(h)) == capi.EINVAL
    assert L.buff_deserialize(None, 0, 10000, 0, None, C.byref(h)) == capi.EINVAL
    buf = np.zeros(8, dtype=np.uint8)
    assert L.buff_deserialize(buf.ctypes.data, 8, 10000, 0, None, C.byref(h)) == capi.ECORRUPT


def test_scale_without_precision_entry_is_a_reference_panic():
    # PRECISION_MAP has no entry for 0 decimals (compress/mod.rs:29-46); this
    # is decided on the host before any device work.
    L = capi.lib()
    h = C.c_void_p()
    x = np.arange(4, dtype=np.float64)
    assert L.buff_encode_f64(x.ctypes.data, 4, 5, 0, None, C.byref(h)) == capi.EREFPANIC


def test_mirror_class_shape():
    from buff_gb300 import SplitBDDoubleCompress

    comp = SplitBDDoubleCompress(10, 10, 10000)
    for nm in ("buff_simd256_encode", "buff_simd256_decode", "buff_simd_range_filter",
               "buff_simd_equal_filter", "buff_simd_range_filter_with_slice",
               "buff_simd_equal_filter_with_slice", "byte_fixed_sum", "byte_fixed_max",
               "byte_residue_decode_with_precision", "byte_residue_sum_with_precision"):
        assert callable(getattr(comp, nm))


def test_product_path_does_not_import_the_oracle():
    pkg = os.path.join(ROOT, "buff_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".h", ".cuh", ".cpp")):
                src = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in src.replace("oracle.", "").lower() or f == "__init__.py", f


def test_row_limit_is_refused_before_any_device_work():
    """Columns of more than BUFF_MAX_ROWS rows (2^32 - 512) are refused: on
    encode as EINVAL, from an image header as ENOTSUP."""
    L = capi.lib()
    h = C.c_void_p()
    x = np.zeros(4)
    assert L.buff_encode_f64(x.ctypes.data, capi.MAX_ROWS + 1, 10000, 0, None,
                             C.byref(h)) == capi.EINVAL
    assert L.buff_encode_majority_f64(x.ctypes.data, capi.MAX_ROWS + 1, 10000, 0, None,
                                      C.byref(h)) == capi.EINVAL
    hdr = np.zeros(64, dtype=np.uint8)
    hdr[8:12] = np.frombuffer(np.uint32(0xFFFFFFFF).tobytes(), dtype=np.uint8)
    hdr[16] = 15
    for fn in ("buff_deserialize", "buff_slice_deserialize"):
        assert getattr(L, fn)(hdr.ctypes.data, hdr.size, 10000, 0, None,
                              C.byref(h)) == capi.ENOTSUP, fn
    cnt = np.zeros(1, dtype=np.uint64)
    assert L.buff_filter_image(hdr.ctypes.data, hdr.size, 10000, 0, 0, 1.0, None,
                               cnt.ctypes.data, None) == capi.ENOTSUP
