"""A second, independent statement of the buff-simd semantics in numpy/Python.

The oracle (oracle/buff_oracle.c) follows the reference's control flow
(BitPack cursor, progressive candidate refinement, SIMD threshold).  This model
states the same results as whole-array formulas, so the two cross-check each
other.  Small inputs only.
"""
from __future__ import annotations

import math

import numpy as np

PRECISION_MAP = {1: 5, 2: 8, 3: 11, 4: 15, 5: 18, 6: 21, 7: 25, 8: 28, 9: 31, 10: 35, 11: 38,
                 12: 50, 13: 10, 14: 10, 15: 10}


def prec_of_scale(scale: int) -> int:
    if scale == 0:
        return 0
    return int(np.log10(np.float32(scale)))


def precision_exp(prec: int) -> int:
    v = float("0." + "0" * max(prec, 0) + "49")
    return math.frexp(v)[1] - 1


def fetch_fixed(x: np.ndarray, pexp: int, dlen: int) -> np.ndarray:
    """fetch_fixed_aligned (methods/prec_double.rs:190-205), vectorized."""
    b = np.ascontiguousarray(x, dtype=np.float64).view(np.uint64)
    exp = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64) - 1023
    sh = ((63 - exp - dlen) & 63).astype(np.uint64)
    m = ((b << np.uint64(11)) | np.uint64(1 << 63)) >> sh
    neg = (b >> np.uint64(63)) != 0
    m = np.where(neg, (~(m - np.uint64(1))), m)
    m = np.where(exp < pexp, np.uint64(0), m)
    return m.view(np.int64)


def ref_minmax(q: np.ndarray):
    """The reference's `if x<min {..} else if x>max {..}` loop (buff_simd.rs:3139-3148)."""
    mn, mx = (1 << 63) - 1, -(1 << 63)
    for v in q.tolist():
        if v < mn:
            mn = v
        elif v > mx:
            mx = v
    return mn, mx


def wrap64(v: int) -> int:
    v &= (1 << 64) - 1
    return v - (1 << 64) if v >> 63 else v


def layout(q: np.ndarray, scale: int, intended: bool):
    prec = prec_of_scale(scale)
    dlen = PRECISION_MAP[prec]
    if intended:
        mn, mx = int(q.min()), int(q.max())
        delta = mx - mn
        fl = 0 if delta == 0 else delta.bit_length()
    else:
        mn, mx = ref_minmax(q)
        delta = wrap64(mx - mn)
        if delta == 0:
            fl = 0
        else:
            c = math.ceil(math.log2(float(delta))) if delta > 0 else float("nan")
            fl = 0 if (c != c or c <= 0) else int(c)
    k, r = (0, fl) if fl < 8 else (fl // 8, fl % 8)
    codes = np.array([(int(v) - mn) & ((1 << fl) - 1) if fl else 0 for v in q.tolist()],
                     dtype=np.uint64)
    return dict(base=mn, fl=fl, k=k, r=r, dlen=dlen, codes=codes,
                ilen=(fl - dlen) & 0xFFFFFFFF, pexp=precision_exp(prec))


def bits_to_words(bits: np.ndarray) -> np.ndarray:
    n = bits.size
    nw = (n + 31) // 32
    pad = np.zeros(nw * 32, dtype=np.uint8)
    pad[:n] = bits
    return np.packbits(pad, bitorder="little").view("<u4")[:nw].astype(np.uint32)


def filter_words(L, pred: float, is_range: bool, intended: bool,
                 full_blocks: bool = True) -> np.ndarray:
    """The range / equality filter bitmap.  full_blocks: the SIMD filters
    never set rows after the last full 32-row block; the scalar buff-layout
    filters (full_blocks=False) cover every row."""
    n = L["codes"].size
    fp = int(fetch_fixed(np.array([pred]), L["pexp"], L["dlen"])[0])
    if fp < L["base"]:
        return bits_to_words(np.full(n, 1 if is_range else 0, dtype=np.uint8))
    t = fp - L["base"]
    codes = [int(c) for c in L["codes"].tolist()]
    fl, k, r = L["fl"], L["k"], L["r"]
    if intended or k == 0:
        hit = [(c > t) if is_range else (c == t) for c in codes]
        return bits_to_words(np.array(hit, dtype=np.uint8))
    tt = t & ((1 << fl) - 1)
    full = n // 32 * 32 if full_blocks else n
    if (not is_range) and r == 0:
        return bits_to_words(np.zeros(n, dtype=np.uint8))
    hit = [((c > tt) if is_range else (c == tt)) and i < full for i, c in enumerate(codes)]
    return bits_to_words(np.array(hit, dtype=np.uint8))


def ref_sum(L, n: int, intended: bool = False) -> float:
    codes = [int(c) for c in L["codes"].tolist()]
    fl, k, r, dlen = L["fl"], L["k"], L["r"], L["dlen"]
    ilen_i = L["ilen"] - (1 << 32) if L["ilen"] >> 31 else L["ilen"]
    sum_base = float(n) * float(L["base"]) / 2.0 ** dlen
    s = 0.0
    processed = 0
    for j in range(k):
        sh = fl - 8 * (j + 1)
        S = sum((c >> sh) & 0xFF for c in codes)
        processed += 8
        s = s + float(S) / 2.0 ** (processed - ilen_i)
        if j == k - 1 and r == 0 and not intended:
            return s
    if r:
        S = sum(c & ((1 << r) - 1) for c in codes)
        processed += r
        s = s + float(S) / 2.0 ** (processed - ilen_i)
    return s + sum_base


# --- buff-major (outlier) format: whole-array statement of the reference ----

def _bm_vote(vals):
    freq, major = 0, 0
    for b in vals:
        if freq == 0:
            major, freq = b, 1
        elif major == b:
            freq += 1
        else:
            freq -= 1
    return major, freq


def major_layout(x: np.ndarray, scale: int):
    """Columns, majors and outlier masks of buff_encode_majority (buff_simd.rs:317-630)."""
    prec = prec_of_scale(scale)
    dlen = PRECISION_MAP[prec]
    pexp = precision_exp(prec)
    q = fetch_fixed(x, pexp, dlen)
    mn, mx = int(q.min()), int(q.max())
    delta = mx - mn
    fl = 0 if delta == 0 else int(math.ceil(math.log2(float(delta))))
    codes = [(int(v) - mn) & ((1 << 64) - 1) for v in q.tolist()]
    rsf = fl - 8 if fl >= 8 else 0
    majors = []
    maj, freq = _bm_vote([(c >> rsf) & 0xFF for c in codes[:2000]])
    if freq > 1200:
        majors.append(maj)
        while rsf > 7:
            rsf -= 8
            maj, freq = _bm_vote([(c >> rsf) & 0xFF for c in codes[:2000]])
            if freq > 1200:
                majors.append(maj)
            else:
                break
    return dict(base=mn, fl=fl, dlen=dlen, pexp=pexp, codes=codes, majors=majors,
                ilen=(fl - dlen) & 0xFFFFFFFF)


def _byte(c, fl, j):
    return (c >> (fl - 8 * (j + 1))) & 0xFF


def major_decode_codes(L):
    """buff_decode_majority's codes (buff_simd.rs:633-861): the 2nd+ sparse
    column ORs its major shifted twice, and only before its last outlier."""
    fl, codes, majors = L["fl"], L["codes"], L["majors"]
    n = len(codes)
    out = []
    m = len(majors)
    last = []
    for c in range(m):
        rows = [i for i in range(n) if _byte(codes[i], fl, c) != majors[c]]
        last.append(rows[-1] if rows else -1)
    mask64 = (1 << 64) - 1
    for i, code in enumerate(codes):
        v = 0
        for c in range(m):
            sh = fl - 8 * (c + 1)
            b = _byte(code, fl, c)
            if c == 0:
                v = (b << sh) if b != majors[0] else (majors[0] << sh)
            else:
                if b != majors[c]:
                    v |= b << sh
                elif i < last[c]:
                    v |= ((majors[c] << sh) << sh) & mask64
        low = fl - 8 * m
        v |= code & ((1 << low) - 1)
        out.append(v & mask64)
    return out


def major_filter(L, pred: float, is_range: bool):
    fl, codes, majors, base = L["fl"], L["codes"], L["majors"], L["base"]
    n = len(codes)
    fp = int(fetch_fixed(np.array([pred]), L["pexp"], L["dlen"])[0])
    if fp < base:
        return bits_to_words(np.full(n, 1 if is_range else 0, dtype=np.uint8))
    t = fp - base
    m = len(majors)
    gt = [False] * n
    eq = [True] * n
    for c in range(m):
        T = (t >> (fl - 8 * (c + 1))) & 0xFF
        M = majors[c]
        for i in range(n):
            b = _byte(codes[i], fl, c)
            out = b != M
            if not is_range:
                eq[i] = eq[i] and b == T
                continue
            if c == 0:
                gt[i] = b > T
                eq[i] = b == T
            elif T == 0 and M == 0:
                if eq[i] and out:
                    gt[i] = True
                eq[i] = False                      # the candidates are dropped
            else:
                if out and b > T:
                    gt[i] = True                   # not restricted to candidates
                if not out and T < M and eq[i]:
                    gt[i] = True
                eq[i] = eq[i] and ((out and b == T) or (not out and T == M))
    low = fl - 8 * m
    if low > 0:
        r = low % 8
        for i in range(n):
            if not eq[i]:
                continue
            lowv = codes[i] & ((1 << low) - 1)
            tlow = t & ((1 << low) - 1)
            if (low >= 8) or r:
                if is_range:
                    gt[i] = gt[i] or lowv > tlow
            eq[i] = lowv == tlow
    res = gt if is_range else ([e and (fl - 8 * m) % 8 != 0 for e in eq] if fl - 8 * m > 0 else [False] * n)
    return bits_to_words(np.array(res, dtype=np.uint8))


def major_sum(L) -> float:
    fl, codes, majors, base, dlen = L["fl"], L["codes"], L["majors"], L["base"], L["dlen"]
    n = len(codes)
    ilen_i = L["ilen"] - (1 << 32) if L["ilen"] >> 31 else L["ilen"]
    sum_base = float(n) * float(base) / 2.0 ** dlen
    s, processed = 0.0, 0
    k = fl // 8
    for j in range(k):
        S = sum(_byte(c, fl, j) for c in codes)
        processed += 8
        s = s + float(S) / 2.0 ** (processed - ilen_i)
        if j >= len(majors) and j == k - 1 and fl % 8 == 0:
            return s
    r = fl % 8
    if r:
        processed += r
        s = s + float(sum(c & ((1 << r) - 1) for c in codes)) / 2.0 ** (processed - ilen_i)
    return s + sum_base


def major_max_code(L) -> int:
    fl, codes, majors = L["fl"], L["codes"], L["majors"]
    n = len(codes)
    m = len(majors)
    cand = list(range(n))
    mx = 0
    for c in range(m):
        sh = fl - 8 * (c + 1)
        M = majors[c]
        bytes_ = {i: _byte(codes[i], fl, c) for i in cand}
        outs = [i for i in cand if bytes_[i] != M]
        if c == 0:
            best = max(bytes_.values())
            cand = [i for i in cand if bytes_[i] == best]
            mx |= best << sh
            continue
        if not outs:
            continue                               # the major never reaches max
        best = max(bytes_[i] for i in outs)
        if best > M:
            cand = [i for i in outs if bytes_[i] == best]
            mx |= best << sh
        else:
            cand = [i for i in cand if bytes_[i] == M]
            mx |= M << sh
    for j in range(m, fl // 8):
        sh = fl - 8 * (j + 1)
        if not cand:
            continue
        best = max(_byte(codes[i], fl, j) for i in cand)
        cand = [i for i in cand if _byte(codes[i], fl, j) == best]
        mx |= best << sh
    r = fl % 8
    if r and cand:
        mx |= max(codes[i] & ((1 << r) - 1) for i in cand)
    return mx


# --- row-conditioned reads (buff layout) ------------------------------------

def cond_decode(L, rows, tail_shift: bool):
    """buff_decode_condition (tail_shift, Q8) / buff_major_decode_condition."""
    fl, r, base, dlen = L["fl"], L["r"], L["base"], L["dlen"]
    out = []
    for i in rows:
        c = int(L["codes"][i])
        if fl >= 8 and r and tail_shift:
            c = (c >> r << r) | ((c & ((1 << r) - 1)) << r)
        out.append(float(wrap64(base + c)) / 2.0 ** dlen)
    return np.array(out, dtype=np.float64)


def cond_range(L, pred: float, rows):
    """buff_range_filter_condition: lexicographic compare of the (bytes, tail)
    tuple with the truncated target tuple, on the listed rows only."""
    n = L["codes"].size
    fp = int(fetch_fixed(np.array([pred]), L["pexp"], L["dlen"])[0])
    hit = np.zeros(n, dtype=np.uint8)
    if fp < L["base"]:
        return bits_to_words(hit)
    t = fp - L["base"]
    fl, k, r = L["fl"], L["k"], L["r"]

    def tup(v):
        if fl < 8:
            return (v & ((1 << fl) - 1),)
        return tuple((v >> (fl - 8 * (j + 1))) & 0xFF for j in range(k)) + \
            ((v & ((1 << r) - 1),) if r else ())

    if fl < 8:
        tt = (t & 0xFF,)
    else:
        tt = tup(t)
    for i in rows:
        if tup(int(L["codes"][i])) > tt:
            hit[i] = 1
    return bits_to_words(hit)


def max_range(L, s, e, w):
    """Per full window of w rows in [s, e): the largest code, as a value."""
    codes = [int(c) for c in L["codes"].tolist()]
    out = []
    for a in range(s, e - w + 1, w):
        m = max(codes[a:a + w])
        out.append(float(wrap64(L["base"] + m)) / 2.0 ** L["dlen"])
    return np.array(out)
