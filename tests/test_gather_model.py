"""Index model of the batch gather (csrc/ingest.cu, gather_inputs_kernel), on the CPU.

The kernel cuts the destination of a batch (or of a contiguous range of its inputs) into
8 KiB windows, finds each window's first input by a binary search of the offsets, takes
the inputs that overlap the window 32 at a time, copies pieces under 64 bytes with one lane
each and longer pieces with the warp (head bytes, whole 16-byte blocks made of two aligned
source loads, tail bytes). This model replays those index computations and checks, for
ragged batches with empty inputs, tiny inputs, inputs longer than a window and unaligned
sources, that every destination byte of the range is written exactly once with the right
source byte, that nothing outside the range is written, and that every aligned 16-byte
source block a load touches holds at least one byte of its input.
"""

from __future__ import annotations

import numpy as np
import pytest

WINDOW, SMALL = 8192, 64


def _ld16_blocks(p: int) -> list[int]:
    """Aligned 16-byte blocks read for 16 bytes at address p."""
    blk = p & ~15
    return [blk] if p == blk else [blk, blk + 16]


def gather_model(src: list[int], offsets: np.ndarray, n: int, touched: list):
    """Returns {dst index: source address} of every write; ``touched`` collects
    (input, aligned source block) for every 16-byte load."""
    writes: dict[int, int] = {}

    def put(k: int, addr: int) -> None:
        assert k not in writes, f"byte {k} written twice"
        writes[k] = addr

    first, last = int(offsets[0]), int(offsets[n])
    if last <= first:
        return writes
    w0 = first & ~15
    windows = -(-(last - w0) // WINDOW)
    for w in range(windows):
        wl = w0 + w * WINDOW
        wh = min(wl + WINDOW, last)
        lo, hi = 0, n - 1
        while lo < hi:
            mid = (lo + hi) >> 1
            if offsets[mid + 1] > wl:
                hi = mid
            else:
                lo = mid + 1
        g = lo
        while g < n:
            lanes = []
            for lane in range(32):
                i = g + lane
                d0 = d1 = wh
                if i < n:
                    d0, d1 = int(offsets[i]), int(offsets[i + 1])
                past = d0 >= wh
                a, b = max(d0, wl), min(d1, wh)
                live = (not past) and a < b
                s = src[i] + (a - d0) if live else None
                lanes.append((i, past, a, b, live, s))
            for i, past, a, b, live, s in lanes:
                if live and b - a < SMALL:
                    for k in range(a, b):
                        put(k, s + (k - a))
            for i, past, a, b, live, s in lanes:
                if not (live and b - a >= SMALL):
                    continue
                za, zz = (a + 15) & ~15, b & ~15
                if za >= zz:
                    for k in range(a, b):
                        put(k, s + (k - a))
                    continue
                for k in range(a, za):
                    put(k, s + (k - a))
                for k in range(zz, b):
                    put(k, s + (k - a))
                for blk in range(za, zz, 16):
                    p = s + (blk - a)
                    for q in _ld16_blocks(p):
                        touched.append((i, q))
                    for k in range(16):
                        put(blk + k, p + k)
            if any(t[1] for t in lanes):
                break
            g += 32
    return writes


def _batch(rng, kinds: str, n: int):
    if kinds == "tiny":
        lens = rng.integers(0, 40, n)
    elif kinds == "long":
        lens = rng.integers(5000, 30000, n)
    else:
        lens = np.where(rng.random(n) < 0.3, 0, rng.integers(1, 20000, n))
    src, addr = [], 1 << 20
    for m in lens:  # sources at arbitrary alignments, far apart
        addr += int(rng.integers(0, 64)) + 4096
        src.append(addr)
        addr += int(m)
    off = np.zeros(n + 1, np.int64)
    off[1:] = np.cumsum(lens)
    return src, off


@pytest.mark.parametrize("kinds", ["tiny", "long", "mixed"])
@pytest.mark.parametrize("seed", range(3))
def test_every_byte_written_once_from_its_input(kinds, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 90))
    src, off = _batch(rng, kinds, n)
    # the whole batch, then two ranges of it gathered separately (pipelined slices)
    cut = int(rng.integers(0, n + 1))
    for a, b in ((0, n), (0, cut), (cut, n)):
        if b <= a:
            continue
        touched: list = []
        writes = gather_model(src[a:], off[a:], b - a, touched)
        assert sorted(writes) == list(range(int(off[a]), int(off[b])))
        for i in range(a, b):
            for k in range(int(off[i]), int(off[i + 1])):
                assert writes[k] == src[i] + (k - int(off[i]))
        for i, q in touched:
            lo, hi = src[a + i], src[a + i] + int(off[a + i + 1] - off[a + i])
            assert q < hi and q + 16 > lo, "a load touched a block without input bytes"


def test_empty_range_writes_nothing():
    off = np.array([5, 5, 5], np.int64)
    assert gather_model([100, 200], off, 2, []) == {}
