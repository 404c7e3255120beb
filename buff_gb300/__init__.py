"""GB300-native (sm_103a) implementation of BUFF's buff-simd hot path.

The compute path is the CUDA library ``buff_gb300/_build/libbuffgpu.so``
(C ABI: ``include/buff_gpu.h``); this package is its Python front end.
"""
from .capi import BuffError, ReferencePanic, FLAG_INTENDED  # noqa: F401
from .compress import Column, FilterResult, MaxResult, SplitBDDoubleCompress  # noqa: F401

__all__ = ["SplitBDDoubleCompress", "Column", "FilterResult", "MaxResult", "BuffError",
           "ReferencePanic", "FLAG_INTENDED"]
