"""Host-side packing: the reference's helpers plus the engine's byte-batch layout.

Reference-compatible (``src/gpufsm/core/packing.py:21-98``; same names, dtypes and
errors, so callers of gpufsm's packing keep working):

* ``WORD_BITS``, ``words_for`` -- 64-bit words of the packed active set;
* ``symbols`` -- one input as int32 symbols;
* ``pack_inputs`` -- a batch as int32 symbols + int32 offsets, ``ValueError`` past 2 GiB;
* ``pack_accept`` / ``accept_bitmask`` -- state ``s`` is bit ``s % 64`` of word ``s // 64``.

Engine layout (what actually crosses to the device):

* ``pack_bytes`` -- a batch as **uint8** bytes (one byte per symbol instead of four) with
  **int64** offsets (no 2 GiB limit), the data padded to a 16-byte multiple so the
  kernels' 16-byte vector loads never leave the buffer.
"""

from __future__ import annotations

from typing import Any

import numpy as np

WORD_BITS = 64
"""Bits per word of the packed state set (the kernels' word type is uint64)."""

PAD = 16
"""Byte alignment of a packed batch (the width of one vector load)."""


def words_for(num_states: int) -> int:
    """Number of ``WORD_BITS``-bit words that hold ``num_states`` bits."""
    return -(-int(num_states) // WORD_BITS)


def symbols(input_bytes: bytes) -> np.ndarray:
    """One input as the int32 symbol array the reference's kernels index with."""
    return np.frombuffer(bytes(input_bytes), dtype=np.uint8).astype(np.int32)


def pack_inputs(inputs: list[bytes]) -> tuple[np.ndarray, np.ndarray]:
    """Flat int32 symbols plus int32 offsets (``len(inputs) + 1`` entries).

    Reference behaviour (core/packing.py:35-63): an all-empty batch gives an empty
    buffer, and a batch above the int32 offset range raises ``ValueError``.
    """
    lens = np.fromiter((len(b) for b in inputs), dtype=np.int64, count=len(inputs))
    total = int(lens.sum()) if lens.size else 0
    limit = int(np.iinfo(np.int32).max)
    if total > limit:
        raise ValueError(
            f"batch of {total} bytes exceeds the int32 offset range ({limit}); "
            f"split it into smaller batches"
        )
    offsets = np.zeros(len(inputs) + 1, dtype=np.int32)
    if lens.size:
        np.cumsum(lens, out=offsets[1:])
    if total:
        data = np.frombuffer(b"".join(inputs), dtype=np.uint8).astype(np.int32)
    else:
        data = np.zeros(0, dtype=np.int32)
    return data, offsets


def pack_bytes(inputs, out: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
    """Flat uint8 bytes (padded to ``PAD``) plus int64 offsets.

    ``inputs`` is a list of bytes-like objects. When ``out`` (a uint8 array, e.g. a
    pinned staging buffer viewed through numpy) is given and large enough, the bytes are
    written into it and a view of it is returned, so no intermediate copy is made.
    """
    n = len(inputs)
    offsets = np.zeros(n + 1, dtype=np.int64)
    if n:
        np.cumsum(np.fromiter((len(b) for b in inputs), dtype=np.int64, count=n),
                  out=offsets[1:])
    total = int(offsets[-1])
    padded = max(PAD, -(-total // PAD) * PAD)
    if out is not None and out.size >= padded:
        data = out[:padded]
    else:
        data = np.empty(padded, dtype=np.uint8)
    pos = 0
    for b in inputs:
        k = len(b)
        if k:
            data[pos:pos + k] = np.frombuffer(b, dtype=np.uint8)
        pos += k
    data[total:padded] = 0
    return data, offsets


def pack_accept(nfa: Any, dtype: type = np.uint64, nwords: int | None = None) -> np.ndarray:
    """Accept set as ``nwords`` bit words (reference: core/packing.py:66-85).

    ``dtype`` is the word type (``uint64`` for CUDA, ``int64`` where only signed types
    exist); ``nwords`` defaults to ``words_for(num_states)``.
    """
    n = int(nfa.num_states)
    if nwords is None:
        nwords = words_for(n)
    bits = np.zeros(int(nwords) * WORD_BITS, dtype=np.uint8)
    bits[:n] = np.asarray(nfa.accept[:n], dtype=bool)
    packed = np.packbits(bits, bitorder="little").view("<u8")
    return packed.astype(dtype, copy=False) if dtype is not np.uint64 else packed.copy()


def accept_bitmask(nfa: Any) -> int:
    """The accept set as one Python int (bit ``s`` for state ``s``)."""
    mask = 0
    for s in np.flatnonzero(np.asarray(nfa.accept, dtype=bool)):
        mask |= 1 << int(s)
    return mask
