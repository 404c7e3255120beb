"""``comp_profiler`` for the GPU library: the reference's codec driver, same
arguments and the same ``Performance:`` line.

The reference binary (database/src/compress/main.rs:7-36) takes
``<file> <compression> <int_scale> <pred>``, reads every comma-separated
token of the file that parses as f64 (client.rs:163-182), multiplies it by
``SCALE`` = 1.0 (methods/compress.rs:46), encodes it, runs five queries on
the encoded bytes and prints one CSV line of throughputs in MiB/s of the
input's bincode size.  This module does the same through the GPU library's
public calls for the arms it covers:

- ``buff-simd``  -> run_buff_simd_encoding_decoding (compress/buff_simd.rs:28-95):
  encode, decode, range filter, equality filter, and both ``_with_slice`` filters;
- ``buff-slice`` -> run_buff_slice_encoding_decoding (compress/buff_slice.rs:30-101):
  encode, decode, range, equality, buffsum, buffmax;
- ``buff-major`` -> run_buff_majority_encoding_decoding (compress/buff_simd.rs:246-312):
  the outlier encode, decode, range, equality, sum, max;
- ``buff`` -> run_buff_encoding_decoding_mybitvec (compress/buff_simd.rs:167-245):
  byte_fixed_encode (the buff layout, without the ^0x80 flip), decode, the
  scalar range and equality filters (buff_simd.rs:4507-4679, :4925-5094),
  byte_fixed_sum, byte_fixed_max.  The reference takes its min/max from a
  table of its authors' file paths (FILE_MIN_MAX, compress/mod.rs:50-67) when
  the input is one of them; for every other path it prints ``no min/max`` and
  runs byte_fixed_encode, which is what this arm does;
- ``buff-slice-scalar`` -> run_buff_slice_scalar_encoding_decoding
  (compress/buff_slice.rs:103-171): encode, buff_slice_decode_bs, the
  row-by-row range and equality filters, buff_slice_sum, buff_slice_max.

Each operation is timed on the host clock around the call, with the device
synchronised on both sides, as ``Instant::now()``/``elapsed()`` brackets it in
the reference.  By default the encode reads the host array and every query
returns its result in host memory, as the reference's calls take and return
``Vec``s; the encoded column stays resident in device memory between calls
(the reference clones the encoded ``Vec<u8>`` outside its timed regions).
``--from-bytes`` hands every query the serialized image instead, the closest
analogue of taking ``Vec<u8>`` by value: the buff-simd filters read it in
place (buff_filter_image: slice 0 and the candidates' later bytes cross the
host link, nothing else), the other queries upload it first.

An unknown compression name is rejected, as the reference rejects it.
"""
from __future__ import annotations

import argparse
import math
import re
import sys
import time

import numpy as np

# methods/compress.rs:46
SCALE = 1.0

# A token that Rust's `str::parse::<f64>` accepts: an optional sign, then a
# decimal with optional exponent, or inf / infinity / nan in any case.  No
# surrounding whitespace and no digit separators.
_RUST_F64 = re.compile(
    r"[+-]?(?:(?:[0-9]+\.?[0-9]*|\.[0-9]+)(?:[eE][+-]?[0-9]+)?|inf|infinity|nan)\Z",
    re.IGNORECASE)


def parse_rust_f64(tok: str):
    """The value of ``tok`` as Rust's f64 parser reads it, or None when it rejects it."""
    if not _RUST_F64.match(tok):
        return None
    return float(tok)


def read_values(path: str, skip: int = 0, delim: str = ",") -> np.ndarray:
    """construct_file_iterator_skip_newline::<f64> (client.rs:163-182).

    Lines are split on ``delim``, the first ``skip`` fields of each line are
    dropped and every field that parses as f64 is kept, in file order.  Lines
    end at ``\\n`` with an optional ``\\r`` before it, as ``BufRead::lines``
    strips them; a line that is not UTF-8 is skipped (``filter_map(Result::ok)``).
    """
    out = []
    with open(path, "rb") as f:
        data = f.read()
    for raw in data.split(b"\n"):
        if raw.endswith(b"\r"):
            raw = raw[:-1]
        try:
            line = raw.decode("utf-8")
        except UnicodeDecodeError:
            continue
        for tok in line.split(delim)[skip:]:
            v = parse_rust_f64(tok)
            if v is not None:
                out.append(v * SCALE)
    return np.asarray(out, dtype=np.float64)


def segment_byte_size(n: int) -> int:
    """``Segment::get_byte_size`` (segment.rs:90-95) of an n-value f64 segment.

    bincode 1.x sizes the struct (segment.rs:35-43) field by field: the
    ``method: Option<Methods>`` None tag (1 B), ``timestamp: SystemTime``
    (u64 seconds + u32 nanoseconds, 12 B), ``signal: u64`` (8 B), ``data:
    Vec<f64>`` (u64 length + 8 B per value), and the ``time_lapse`` and
    ``prev_seg_offset`` None tags (1 B each).
    """
    return 1 + 12 + 8 + 8 + 8 * n + 1 + 1


def rust_f64_display(x: float) -> str:
    """``format!("{}", x)`` for an f64: the shortest round-trip digits, positional."""
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    return np.format_float_positional(x, unique=True, trim="-")


def rust_duration_debug(ns: int) -> str:
    """``format!("{:?}", Duration::from_nanos(ns))``: s, ms, µs or ns, no trailing zeros."""
    for unit, scale in (("s", 10**9), ("ms", 10**6), ("µs", 10**3)):
        if ns >= scale:
            whole, frac = divmod(ns, scale)
            digits = len(str(scale)) - 1
            f = str(frac).rjust(digits, "0").rstrip("0")
            return f"{whole}.{f}{unit}" if f else f"{whole}{unit}"
    return f"{ns}ns"


# (encode label, [(query label, method name)]) per arm, in the reference's order.
ARMS = {
    "buff-simd": ("splitbd byte compress function()", [
        ("buff simd decompress function()", "decode"),
        ("buff simd range filter function()", "range"),
        ("buff simd equal filter function()", "equal"),
        ("buff simd range in BS way", "range_with_slice"),
        ("buff simd equal in BS way", "equal_with_slice"),
    ]),
    "buff-slice": ("buff slice compress function()", [
        ("buff slice decompress function()", "decode"),
        ("buff slice range filter function()", "range"),
        ("buff slice equal filter function()", "equal"),
        ("buff slice sum function()", "buffsum"),
        ("buff slice max function()", "buffmax"),
    ]),
    "buff-major": ("buff-major byte compress function()", [
        ("buff-major byte decompress function()", "decode"),
        ("buff-major byte range filter function()", "range"),
        ("buff-major byte equal filter function()", "equal"),
        ("buff-major sum function()", "sum"),
        ("buff-major max function()", "max"),
    ]),
    "buff": ("splitbd byte compress function()", [
        ("splitbd byte decompress function()", "decode"),
        ("splitbd byte range filter function()", "range"),
        ("splitbd byte equal filter function()", "equal"),
        ("byte_splitbd sum function()", "sum"),
        ("byte_splitbd max function()", "max"),
    ]),
    "buff-slice-scalar": ("buff slice compress function()", [
        ("buff slice decompress function()", "decode"),
        ("buff slice range filter function()", "range"),
        ("buff slice equal filter function()", "equal"),
        ("buff slice sum function()", "sum"),
        ("buff slice max function()", "max"),
    ]),
}

# Lines the reference prints inside the encode's timed region, before its
# `Time elapsed` line (buff_simd.rs:183-186: the input is not one of its
# FILE_MIN_MAX paths).
PRE_ENCODE = {"buff": "no min/max"}


def _ops(arm: str, scale: int):
    """(encode(values) -> column, deserialize(image) -> column, {query: fn(column, pred)})."""
    from .compress import BuffSliceCompress, SplitBDDoubleCompress

    if arm == "buff-slice":
        comp = BuffSliceCompress(10, 10, scale)
        from .compress import SliceColumn as Col
        enc = comp.buff_slice_encode
        q = {"decode": lambda c, p: comp.buff_slice_decode(c),
             "range": lambda c, p: comp.buff_slice_range_filter(c, p),
             "equal": lambda c, p: comp.buff_slice_equal_filter(c, p),
             "buffsum": lambda c, p: comp.buff_slice_buffsum(c),
             "buffmax": lambda c, p: comp.buff_slice_buffmax(c)}
        return enc, (lambda b: Col.deserialize(b, scale)), q
    if arm == "buff-slice-scalar":
        comp = BuffSliceCompress(10, 10, scale)
        from .compress import SliceColumn as Col
        enc = comp.buff_slice_encode
        q = {"decode": lambda c, p: comp.buff_slice_decode_bs(c),
             "range": lambda c, p: comp.buff_slice_range_filter_nosimd(c, p),
             "equal": lambda c, p: comp.buff_slice_equal_filter_nosimd(c, p),
             "sum": lambda c, p: comp.buff_slice_sum(c),
             "max": lambda c, p: comp.buff_slice_max(c)}
        return enc, (lambda b: Col.deserialize(b, scale)), q
    comp = SplitBDDoubleCompress(10, 10, scale)
    if arm == "buff":
        from .compress import FLAG_BUFF_LAYOUT
        from .compress import Column as Col
        enc = comp.byte_fixed_encode
        q = {"decode": lambda c, p: comp.byte_fixed_decode(c),
             "range": lambda c, p: comp.buff_range_filter(c, p),
             "equal": lambda c, p: comp.buff_equal_filter(c, p),
             "sum": lambda c, p: comp.byte_fixed_sum(c),
             "max": lambda c, p: comp.byte_fixed_max(c)}
        return enc, (lambda b: Col.deserialize(b, scale, FLAG_BUFF_LAYOUT)), q
    if arm == "buff-major":
        from .compress import MajorColumn as Col
        enc = comp.buff_encode_majority
        q = {"decode": lambda c, p: comp.buff_decode_majority(c),
             "range": lambda c, p: comp.buff_range_filter_majority(c, p),
             "equal": lambda c, p: comp.buff_equal_filter_majority(c, p),
             "sum": lambda c, p: comp.buff_sum_majority(c),
             "max": lambda c, p: comp.buff_max_majority(c)}
        return enc, (lambda b: Col.deserialize(b, scale)), q
    from .compress import Column as Col
    enc = comp.buff_simd256_encode
    q = {"decode": lambda c, p: comp.buff_simd256_decode(c),
         "range": lambda c, p: comp.buff_simd_range_filter(c, p),
         "equal": lambda c, p: comp.buff_simd_equal_filter(c, p),
         "range_with_slice": lambda c, p: comp.buff_simd_range_filter_with_slice(c, p),
         "equal_with_slice": lambda c, p: comp.buff_simd_equal_filter_with_slice(c, p)}
    return enc, (lambda b: Col.deserialize(b, scale)), q


def run(test_file: str, compression: str, scl: int, pred: float, from_bytes: bool = False,
        out=sys.stdout, values: np.ndarray | None = None) -> dict:
    """One driver run; prints the reference's lines and returns the figures."""
    import torch

    if compression not in ARMS:
        raise ValueError(f"Compression not supported yet: {compression}")
    vals = read_values(test_file) if values is None else np.asarray(values, dtype=np.float64)
    org_size = segment_byte_size(vals.size)
    enc_label, queries = ARMS[compression]
    encode, deserialize, qfn = _ops(compression, scl)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter_ns()
        r = fn()
        torch.cuda.synchronize()
        return r, max(time.perf_counter_ns() - t0, 1)

    if compression in PRE_ENCODE:
        print(PRE_ENCODE[compression], file=out)
    col, t_enc = timed(lambda: encode(vals))
    image = col.serialize()
    comp_size = len(image)
    print(f"Time elapsed in {enc_label} is: {rust_duration_debug(t_enc)}", file=out)
    times = [t_enc]
    results = {}
    from .compress import FILTER_KINDS, filter_image

    in_place = {"range": "range", "equal": "equal", "range_with_slice": "range_with_slice",
                "equal_with_slice": "equal_with_slice"} if compression == "buff-simd" else {}
    host_image = np.frombuffer(image, dtype=np.uint8)
    for label, name in queries:
        if from_bytes and name in in_place:
            assert in_place[name] in FILTER_KINDS
            r, t = timed(lambda: filter_image(host_image, scl, pred, in_place[name]))
        elif from_bytes:
            r, t = timed(lambda: qfn[name](deserialize(image), pred))
        else:
            r, t = timed(lambda: qfn[name](col, pred))
        results[name] = r
        times.append(t)
        print(f"Time elapsed in {label} is: {rust_duration_debug(t)}", file=out)
    mib = [1e9 * org_size / t / 1024.0 / 1024.0 for t in times]
    fields = [test_file, str(scl), rust_f64_display(pred),
              rust_f64_display(comp_size / org_size)] + [rust_f64_display(v) for v in mib]
    print("Performance:" + ",".join(fields), file=out)
    return {"org_size": org_size, "comp_size": comp_size, "ns": times, "mib_s": mib,
            "results": results, "image": image}


def _pred_arg(tok: str) -> float:
    v = parse_rust_f64(tok)
    if v is None:  # the reference's `args[4].parse::<f64>().unwrap()` panics
        raise argparse.ArgumentTypeError(f"not an f64: {tok!r}")
    return v


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m buff_gb300.profiler",
                                 description="comp_profiler on the GPU library")
    ap.add_argument("input_file")
    ap.add_argument("compression",
                    help="buff | buff-simd | buff-slice | buff-slice-scalar | buff-major")
    ap.add_argument("int_scale", type=int)
    ap.add_argument("pred", type=_pred_arg)
    ap.add_argument("--from-bytes", action="store_true",
                    help="upload the serialized image before every query")
    a = ap.parse_args(argv)
    print(f"ARGS: {a.input_file}, {a.compression}, {a.int_scale}, {rust_f64_display(a.pred)}, ")
    run(a.input_file, a.compression, a.int_scale, a.pred, a.from_bytes)
    return 0


if __name__ == "__main__":
    sys.exit(main())
