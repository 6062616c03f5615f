"""The algorithm of the GPU's sequential FP64 sums (the k_gs_* kernels and
chunk_split in mglc_gb300/csrc/k_particle2d.cu), modelled in Python
with the kernel's integer operations on IEEE bit patterns, checked on the CPU
against the plain left-to-right loop.  While the running sum s lies in the
binade [2^e, 2^(e+1)), s = S u with u = 2^(e-52), and adding a finite
non-negative addend rounds it onto the grid of u: an integer increment, except
that an exact half-ulp tie goes to the even S.  An addend is therefore a map
(incoming parity -> increment, outgoing parity); maps compose associatively.
The kernel splits a chunk at the first warp, and inside it at the first lane,
whose addend cannot take that path, adds that addend the plain way and starts
the rest over; the model does the same with small warps so splits are frequent."""
import math
import struct

import numpy as np
import pytest

MANT = (1 << 52) - 1
NO_BINADE = None


def bits(x):
    return struct.unpack("<q", struct.pack("<d", x))[0]


def dbl(b):
    return struct.unpack("<d", struct.pack("<q", b))[0]


def seg_of(x, e):
    """(i0, i1, o0, o1), upper bound of the increment; None for the plain path."""
    xb = bits(x)
    if xb < 0:
        return None
    ex = xb >> 52
    if ex == 2047:
        return None
    m_full = (xb & MANT) | ((1 << 52) if ex else 0)
    sh = max(ex, 1) - 1023 - e
    if sh > 0:
        return None
    cls = 0
    if sh == 0:
        m = m_full
    elif sh >= -62:
        k = -sh
        m = m_full >> k
        rem, half = m_full & ((1 << k) - 1), 1 << (k - 1)
        cls = 1 if rem > half else (2 if rem == half else 0)
    else:
        m = 0
    if cls == 2:
        return (m + (m & 1), m + ((m + 1) & 1), 0, 0), m + 1
    v = m + cls
    return (v, v, v & 1, (v + 1) & 1), v


IDENT = (0, 0, 0, 1)


def cat(a, b):
    return (a[0] + (b[1] if a[2] else b[0]), a[1] + (b[1] if a[3] else b[0]),
            b[3] if a[2] else b[2], b[3] if a[3] else b[2])


def binade(acc):
    e = ((bits(acc) >> 52) & 0x7FF) - 1023
    return e if acc > 0.0 and -900 <= e <= 1000 else NO_BINADE


def mant_s(acc):
    return (bits(acc) & MANT) | (1 << 52)


def apply(acc, e, h, hb):
    s = mant_s(acc)
    assert hb < (1 << 53) - s
    s1 = s + (h[1] if s & 1 else h[0])
    return dbl(((e + 1023) << 52) | (s1 & MANT))


def split_sum(xs, lanes, units):
    """Add xs (None = not kept) in order: the units (warps, or lanes) up to the
    first that cannot take the grid path as one map, that unit the plain way
    (recursively at lane level), the rest again on the new binade."""
    acc = 0.0
    plain = 0
    pos = 0
    while pos < len(xs):
        chunk = xs[pos:pos + lanes * units]
        start = 0
        while start < len(chunk):
            e = binade(acc)
            s = mant_s(acc) if e is not None else 0
            h, incl, stop = IDENT, 0, None
            for u in range(start, len(chunk), units):
                g, ub, bad = IDENT, 0, False
                for x in chunk[u:u + units]:
                    if x is None:
                        continue
                    r = seg_of(x, e) if e is not None else None
                    if r is None:
                        bad = True
                        break
                    g, ub = cat(g, r[0]), ub + r[1]
                if bad or (e is None and any(x is not None for x in chunk[u:u + units])) \
                        or incl + ub >= (1 << 53) - s:
                    stop = u
                    break
                h, incl = cat(h, g), incl + ub
            if e is not None and incl:
                acc = apply(acc, e, h, incl)
            if stop is None:
                break
            if units == 1:  # the lane itself: the plain FP64 add
                acc = acc + chunk[stop]
                plain += 1
            else:
                sub = [x for x in chunk[stop:stop + units]]
                acc2, p2 = split_from(acc, sub)
                acc, plain = acc2, plain + p2
            start = stop + units
        pos += lanes * units
    return acc, plain


def split_from(acc, xs):
    """Lane-level split of one unit's addends starting from acc."""
    plain = 0
    start = 0
    while start < len(xs):
        e = binade(acc)
        s = mant_s(acc) if e is not None else 0
        h, incl, stop = IDENT, 0, None
        for q in range(start, len(xs)):
            x = xs[q]
            if x is None:
                continue
            r = seg_of(x, e) if e is not None else None
            if r is None or incl + r[1] >= (1 << 53) - s:
                stop = q
                break
            h, incl = cat(h, r[0]), incl + r[1]
        if e is not None and incl:
            acc = apply(acc, e, h, incl)
        if stop is None:
            break
        acc = acc + xs[stop]
        plain += 1
        start = stop + 1
    return acc, plain


def loop_sum(xs):
    acc = 0.0
    for x in xs:
        if x is not None:
            acc = acc + x
    return acc


def same(a, b):
    return (math.isnan(a) and math.isnan(b)) or bits(a) == bits(b)


def addends(kind, n, rng):
    if kind == "near_one":
        x = 1.0 + 1e-3 * (rng.random(n) - 0.5)
    elif kind == "ties":
        x = np.ldexp(rng.integers(0, 4096, n).astype(np.float64), -12) + 0.5
    elif kind == "scales":
        x = np.ldexp(rng.random(n), rng.integers(-20, 20, n))
    elif kind == "negative":
        x = 3.0 * rng.random(n)
        x[rng.random(n) < 0.01] *= -1.0
    elif kind == "tiny":
        x = 1.0 + 1e-6 * rng.random(n)
        x[1::2] = 1e-300 * rng.random(x[1::2].size)
        x[::7] = 0.0
        x[::11] = np.ldexp(1.0, -1070)
    elif kind == "specials":
        x = np.ones(n)
        x[::500] = np.inf
        x[::333] = np.nan
    else:
        x = np.full(n, -0.0)
        x[n // 2:] = 1.0
    keep = rng.random(n) >= 0.1
    return [float(v) if k else None for v, k in zip(x, keep)]


@pytest.mark.parametrize("kind", ["near_one", "ties", "scales", "negative", "tiny", "specials",
                                  "signed_zero"])
def test_grid_maps_with_splits_equal_the_loop_sum(kind):
    rng = np.random.default_rng(len(kind))
    for n in (1, 7, 200, 3000):
        xs = addends(kind, n, rng)
        got, _ = split_sum(xs, lanes=4, units=8)
        assert same(got, loop_sum(xs)), (kind, n)


def test_splits_are_rare_on_densities():
    """Near-one addends leave a binade once per power of two: the plain adds
    are a handful, not one per addend."""
    rng = np.random.default_rng(7)
    xs = addends("near_one", 20000, rng)
    got, plain = split_sum(xs, lanes=32, units=32)
    assert same(got, loop_sum(xs))
    assert plain <= 20


def test_tie_rounds_to_even():
    # s = 2^52 + 1 (odd, u = 1): adding 0.5 ties, so it goes to 2^52 + 2
    s = float(2 ** 52 + 1)
    e = binade(s)
    (i0, i1, o0, o1), ub = seg_of(0.5, e)
    assert (i0, i1, o0, o1, ub) == (0, 1, 0, 0, 1)
    assert apply(s, e, (i0, i1, o0, o1), ub) == s + 0.5


def pipeline_sum(xs, chunk, lanes, units, predict):
    """The multi-block form: every chunk's map is built on the binade that
    predict(prefix estimate) names; a walk adds a chunk as its map only when
    that binade is the exact running sum's, every kept addend took the grid
    path and the bound keeps the sum inside the binade, else it re-adds the
    chunk with the split (split_sum from the running sum)."""
    chunks = [xs[p:p + chunk] for p in range(0, len(xs), chunk)] or [[]]
    parts = [sum(x for x in c if x is not None) for c in chunks]
    pre = [sum(parts[:k]) for k in range(len(chunks))]
    recs = []
    for c, est in zip(chunks, pre):
        e = predict(est)
        h, ub, ok = IDENT, 0, e is not None
        kept = [x for x in c if x is not None]
        for x in kept:
            r = seg_of(x, e) if ok else None
            if r is None:
                ok = False
                break
            h, ub = cat(h, r[0]), ub + r[1]
        recs.append((e, h, min(ub, 1 << 61), ok, bool(kept)))
    acc, redone = 0.0, 0
    for c, (e, h, ub, ok, kept) in zip(chunks, recs):
        if not kept:
            continue
        ea = binade(acc)
        if ok and ea is not None and ea == e and ub < (1 << 53) - mant_s(acc):
            acc = apply(acc, e, h, ub)
            continue
        redone += 1
        acc = split_from_acc(acc, c, lanes, units)
    return acc, redone


def split_from_acc(acc, xs, lanes, units):
    """split_sum over one chunk, starting from the running sum acc."""
    start = 0
    while start < len(xs):
        e = binade(acc)
        s = mant_s(acc) if e is not None else 0
        h, incl, stop = IDENT, 0, None
        for u in range(start, len(xs), units):
            g, ub, bad = IDENT, 0, False
            for x in xs[u:u + units]:
                if x is None:
                    continue
                r = seg_of(x, e) if e is not None else None
                if r is None:
                    bad = True
                    break
                g, ub = cat(g, r[0]), ub + r[1]
            if bad or incl + ub >= (1 << 53) - s:
                stop = u
                break
            h, incl = cat(h, g), incl + ub
        if e is not None and incl:
            acc = apply(acc, e, h, incl)
        if stop is None:
            break
        acc, _ = split_from(acc, xs[stop:stop + units])
        start = stop + units
    return acc


@pytest.mark.parametrize("kind", ["near_one", "ties", "scales", "negative", "tiny", "specials",
                                  "signed_zero"])
@pytest.mark.parametrize("predict", ["estimate", "off_by_one", "none"])
def test_chunk_walk_equals_the_loop_sum_for_any_prediction(kind, predict):
    """The walk never trusts a prediction it cannot confirm: right, wrong by one
    binade, or absent, the result is the loop's sum bit for bit."""
    fn = {"estimate": binade,
          "off_by_one": lambda est: None if binade(est) is None else binade(est) + 1,
          "none": lambda est: None}[predict]
    rng = np.random.default_rng(3 + len(kind) + len(predict))
    for n in (1, 50, 700):
        xs = addends(kind, n, rng)
        got, _ = pipeline_sum(xs, chunk=64, lanes=4, units=4, predict=fn)
        assert same(got, loop_sum(xs)), (kind, predict, n)


def test_chunk_walk_redoes_only_crossings_on_densities():
    rng = np.random.default_rng(11)
    xs = addends("near_one", 40000, rng)
    got, redone = pipeline_sum(xs, chunk=1024, lanes=32, units=32, predict=binade)
    assert same(got, loop_sum(xs))
    # the first chunk (empty running sum) and the chunks holding 2^11 .. 2^15
    assert redone <= 8
