"""Generates the committed golden fixtures of tests/golden/ from the CPU oracle.

    python tests/golden/make_golden.py

- ``vectors.npz``: small seeded columns with the oracle's byte images, decoded
  values, filter bitmaps, sums and maxima (the GPU tests compare against these
  as well as against the live oracle).
- ``randomwalkdatasample1k-1k.xz``: the reference's own README input
  (database/data/randomwalkdatasample1k-1k, 500,000 comma-separated values),
  an xz-compressed byte-for-byte copy of the reference-held test vector, so
  the tests and the GPU machine need no reference checkout.  The copy is made
  from ``$BUFF_REFERENCE_DIR`` (default: the reference checkout below) and
  only where that file exists.
- ``fixture_digest.json``: digests of the oracle's outputs on that input
  (scale 10000, pred 1.1509, README.md:11 of the reference).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

REFERENCE_DIR = os.environ.get("BUFF_REFERENCE_DIR", "/root/reference")
FIXTURE = os.path.join(REFERENCE_DIR, "database", "data", "randomwalkdatasample1k-1k")
FIXTURE_XZ = os.path.join(HERE, "randomwalkdatasample1k-1k.xz")
_FIXTURE_CACHE = {}


def fixture_path() -> str:
    """Path of the README input, decompressed once per process from the
    committed copy into a temporary file (the CSV readers take a path)."""
    if "path" not in _FIXTURE_CACHE:
        import lzma
        import tempfile

        with lzma.open(FIXTURE_XZ, "rb") as f:
            data = f.read()
        fd, path = tempfile.mkstemp(prefix="randomwalkdatasample1k-1k.")
        with os.fdopen(fd, "wb") as f:
            f.write(data)
        _FIXTURE_CACHE["path"] = path
    return _FIXTURE_CACHE["path"]


def load_fixture(path: str) -> np.ndarray:
    """construct_file_iterator_skip_newline::<f64>(file, 0, ',') (client.rs:163-182):
    every comma-separated token that parses as f64, in file order."""
    vals = []
    with open(path) as f:
        for line in f.read().splitlines():
            for tok in line.split(","):
                try:
                    vals.append(float(tok))
                except ValueError:
                    pass
    return np.array(vals, dtype=np.float64)


def _h(b) -> str:
    if isinstance(b, np.ndarray):
        b = np.ascontiguousarray(b).tobytes()
    return hashlib.sha256(b).hexdigest()


def fixture_digest(O, x: np.ndarray, scale: int = 10000, pred: float = 1.1509) -> dict:
    buf = O.encode(x, scale)
    h = O.header(buf)
    out = {"n": int(h.n), "base": int(h.base), "ilen": int(h.ilen), "dlen": int(h.dlen),
           "bytes": len(buf), "sha256": _h(buf)}
    d = O.decode(buf, scale)
    out["decode_sha256"] = _h(d)
    for name, fn in [("range", O.range_filter), ("equal", O.equal_filter)]:
        w, c, e = fn(buf, scale, pred)
        out[name] = {"count": c, "early": e, "sha256": _h(w)}
    for name, fn in [("range_with_slice", O.range_filter_with_slice),
                     ("equal_with_slice", O.equal_filter_with_slice)]:
        w, c, e = fn(buf, scale, pred)
        out[name] = {"count": c, "early": e, "sha256": _h(w)}
    s, parts, exact = O.buff_sum(buf, scale)
    out["sum"] = s.hex()
    out["sum_partials"] = parts
    out["sum_exact_num"] = str(exact)
    mv, mc, aw, ac = O.buff_max(buf, scale)
    out["max"] = mv.hex()
    out["max_code"] = mc
    out["argmax_count"] = ac
    for p in (1, 2, 3, 4):
        out[f"decode_p{p}_sha256"] = _h(O.decode_at_precision(buf, scale, p))
    return out


CASES = [
    # name, generator, n, scale
    ("walk4", "walk", 4099, 10000),
    ("walk2", "walk", 1000, 100),
    ("narrow", "narrow", 640, 100),
    ("wide6", "wide", 2048, 1000000),
    ("small", "walk", 40, 1000),
    ("tiny_width", "narrow", 96, 10),
]


def make_case(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "walk":
        return np.round(1.0 + np.cumsum(rng.normal(0, 0.3, n)), 4)
    if kind == "narrow":
        return np.round(rng.uniform(3.0, 3.1, n), 2)
    if kind == "wide":
        return np.round(rng.normal(100, 5, n), 6)
    raise ValueError(kind)


def make_vectors(O) -> dict:
    arrays = {}
    for i, (name, kind, n, scale) in enumerate(CASES):
        x = make_case(kind, n, 100 + i)
        buf = np.frombuffer(O.encode(x, scale), dtype=np.uint8)
        preds = [float(x[n // 2]), float(np.quantile(x, 0.9)), float(np.quantile(x, 0.5)),
                 float(x.max()) + 0.5]
        arrays[f"{name}.x"] = x
        arrays[f"{name}.scale"] = np.array([scale], dtype=np.uint64)
        arrays[f"{name}.bytes"] = buf
        arrays[f"{name}.decode"] = O.decode(buf.tobytes(), scale)
        arrays[f"{name}.preds"] = np.array(preds)
        for j, p in enumerate(preds):
            arrays[f"{name}.range{j}"] = O.range_filter(buf.tobytes(), scale, p)[0]
            arrays[f"{name}.equal{j}"] = O.equal_filter(buf.tobytes(), scale, p)[0]
        s, parts, exact = O.buff_sum(buf.tobytes(), scale)
        arrays[f"{name}.sum"] = np.array([s])
        mv, mc, aw, ac = O.buff_max(buf.tobytes(), scale)
        arrays[f"{name}.max"] = np.array([mv])
        arrays[f"{name}.max_code"] = np.array([mc], dtype=np.uint64)
    return arrays


def main():
    from oracle import oracle as O

    O.lib()
    arrays = make_vectors(O)
    np.savez_compressed(os.path.join(HERE, "vectors.npz"), **arrays)
    print("wrote vectors.npz with", len(CASES), "cases")
    if os.path.exists(FIXTURE):
        import lzma

        with open(FIXTURE, "rb") as f:
            raw = f.read()
        with lzma.open(FIXTURE_XZ, "wb", preset=9 | lzma.PRESET_EXTREME) as f:
            f.write(raw)
        print("wrote", os.path.basename(FIXTURE_XZ))
    if os.path.exists(FIXTURE_XZ):
        dig = fixture_digest(O, load_fixture(fixture_path()))
        with open(os.path.join(HERE, "fixture_digest.json"), "w") as f:
            json.dump(dig, f, indent=1, sort_keys=True)
        print("wrote fixture_digest.json:", dig["range"], dig["equal"])


if __name__ == "__main__":
    main()
