"""Host->device staging of byte batches.

The reference widens every input byte to an int32 and copies the batch synchronously
from pageable memory on every call (src/gpufsm/core/packing.py:35-63,
native/include/common.cuh:150-159). Here a batch becomes one uint8 device buffer (1 byte
per symbol, int64 offsets, 16-byte padding) in one of two ways:

* on a device that reads pageable host memory coherently (GB300 over NVLink-C2C,
  ``gbfsm_pageable_access``), and for batches of at least ``GATHER_MIN_BYTES``, the GPU
  copies every input from the caller's own buffer (the ``bytes`` objects themselves):
  only their addresses and the offsets cross the link as a table, the bytes are read by
  ``gbfsm_gather_inputs``, and nothing is packed on the host;
* otherwise the batch is packed into a pinned buffer and copied with
  ``cudaMemcpyAsync``.

Buffers grow geometrically and are reused.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from .packing import PAD

GATHER_MIN_BYTES = 1 << 20  # smaller batches: packing costs less than the extra launch


def _address(b) -> int:
    """Address of the bytes of a buffer-protocol object (its own storage, no copy)."""
    if isinstance(b, bytes):
        return ctypes.cast(b, ctypes.c_void_p).value or 0
    return int(np.frombuffer(b, dtype=np.uint8).ctypes.data)


def _bytes_data_offset() -> int | None:
    """Offset of a ``bytes`` object's data from its ``id()`` in this interpreter (the
    object header; the same for every ``bytes``), or None where ``id()`` is not the
    object's address or the offset differs between probes."""
    probes = [b"", b"x", bytes(100), bytes(range(256)) * 40]
    offs = {(ctypes.cast(p, ctypes.c_void_p).value or 0) - id(p) for p in probes}
    if len(offs) != 1:
        return None
    off = offs.pop()
    return off if 0 < off < 256 else None


_BYTES_OFFSET = _bytes_data_offset()


def addresses(inputs, out: np.ndarray) -> None:
    """Write the data address of every input into ``out`` (int64). A batch of plain
    ``bytes`` takes the addresses from ``id()`` at once (a few microseconds per thousand
    inputs instead of one ``ctypes`` call each)."""
    n = len(inputs)
    if _BYTES_OFFSET is not None and set(map(type, inputs)) == {bytes}:
        out[:n] = np.fromiter(map(id, inputs), dtype=np.int64, count=n)
        out[:n] += _BYTES_OFFSET
        return
    for i, b in enumerate(inputs):
        out[i] = _address(b)


def _grow(cap: int, need: int) -> int:
    cap = max(cap, 1 << 12)
    while cap < need:
        cap *= 2
    return cap


class Staging:
    """Pinned host + device buffers for one in-flight batch at a time.

    ``put`` may be called again only after the previous batch's copies completed (the
    executors synchronise on their results before returning, which guarantees it).
    """

    def __init__(self, device: torch.device, gather: bool | None = None) -> None:
        """``gather``: None = read the inputs in place when the device can, False = always
        pack, True = always read in place (the device must read pageable memory)."""
        self.device = device
        self._h_data = self._d_data = None
        self._h_off = self._d_off = None
        self._h_ptr = self._d_ptr = None
        self._cap_data = self._cap_off = 0
        self.gather = gather
        self._pageable = None
        self.last_path = None
        self.deferred = False  # the last put left its gather to the caller

    def _can_gather(self) -> bool:
        if self._pageable is None:
            from . import native

            with torch.cuda.device(self.device):
                self._pageable = native.lib().gbfsm_pageable_access() > 0
            if self.gather and not self._pageable:
                raise ValueError("this device does not read pageable host memory: inputs "
                                 "cannot be gathered in place")
        return self._pageable if self.gather is None else bool(self.gather)

    def _ensure(self, nbytes: int, n_off: int) -> None:
        if nbytes > self._cap_data:
            self._cap_data = _grow(self._cap_data, nbytes)
            self._h_data = torch.empty(self._cap_data, dtype=torch.uint8, pin_memory=True)
            self._d_data = torch.empty(self._cap_data, dtype=torch.uint8, device=self.device)
        if n_off > self._cap_off:
            self._cap_off = _grow(self._cap_off, n_off)
            self._h_off = torch.empty(self._cap_off, dtype=torch.int64, pin_memory=True)
            self._d_off = torch.empty(self._cap_off, dtype=torch.int64, device=self.device)
            self._h_ptr = torch.empty(self._cap_off, dtype=torch.int64, pin_memory=True)
            self._d_ptr = torch.empty(self._cap_off, dtype=torch.int64, device=self.device)

    def put(self, inputs, stream: torch.cuda.Stream, defer: bool = False, lengths=None):
        """Pack ``inputs`` (bytes-like objects) and start their copy on ``stream``.

        Returns ``(d_data, d_offsets, h_offsets, total_bytes)``; device tensors are views
        of the staging buffers (valid until the next ``put``). ``defer``: when the batch
        is gathered in place, enqueue only its address and offset tables and set
        ``deferred``; the caller then runs ``gather_range`` over every input (in ranges, on
        streams that follow ``stream``). ``lengths``: the inputs' lengths (int64), when
        the caller has them already.
        """
        self.deferred = False
        n = len(inputs)
        lens = lengths if lengths is not None else \
            np.fromiter((len(b) for b in inputs), dtype=np.int64, count=n)
        total = int(lens.sum()) if n else 0
        padded = max(PAD, -(-total // PAD) * PAD)
        self._ensure(padded, n + 1)
        h_off = self._h_off.numpy()[: n + 1]
        h_off[0] = 0
        if n:
            np.cumsum(lens, out=h_off[1:])
        if n and total >= GATHER_MIN_BYTES and self._can_gather():
            # the GPU reads each input where it lies; the caller keeps ``inputs`` alive
            # until the stream has passed this copy (the executors synchronise first)
            addresses(inputs, self._h_ptr.numpy())
            with torch.cuda.stream(stream):
                self._d_off[: n + 1].copy_(self._h_off[: n + 1], non_blocking=True)
                self._d_ptr[:n].copy_(self._h_ptr[:n], non_blocking=True)
                if padded > total:
                    self._d_data[total:padded].zero_()
            self.last_path = "gather"
            self.deferred = defer
            if not defer:
                self.gather_range(0, n, stream)
            return self._d_data[:padded], self._d_off[: n + 1], h_off, total
        self.last_path = "pack"
        h_data = self._h_data.numpy()
        pos = 0
        for b in inputs:
            k = len(b)
            if k:
                h_data[pos:pos + k] = np.frombuffer(b, dtype=np.uint8)
            pos += k
        h_data[total:padded] = 0
        with torch.cuda.stream(stream):
            self._d_data[:padded].copy_(self._h_data[:padded], non_blocking=True)
            self._d_off[: n + 1].copy_(self._h_off[: n + 1], non_blocking=True)
        return self._d_data[:padded], self._d_off[: n + 1], h_off, total


    def gather_range(self, first: int, last: int, stream: torch.cuda.Stream) -> None:
        """Enqueue on ``stream`` the copy of inputs [first, last) of the last ``put`` (a
        gathered batch) into their places in the device buffer."""
        from . import native

        if last <= first:
            return
        native.check(native.lib().gbfsm_gather_inputs(
            self._d_ptr.data_ptr() + 8 * first, self._d_off.data_ptr() + 8 * first,
            last - first, self._d_data.data_ptr(), stream.cuda_stream), "gbfsm_gather_inputs")


class Results:
    """Device result arrays plus pinned host mirrors, reused across batches."""

    def __init__(self, device: torch.device) -> None:
        self.device = device
        self._cap = 0

    def ensure(self, n: int) -> None:
        if n > self._cap:
            self._cap = _grow(self._cap, n)
            self.d = torch.zeros((3, self._cap), dtype=torch.int32, device=self.device)
            self.h = torch.zeros((3, self._cap), dtype=torch.int32, pin_memory=True)

    def fetch(self, n: int, stream: torch.cuda.Stream) -> None:
        with torch.cuda.stream(stream):
            for r in range(3):
                self.h[r, :n].copy_(self.d[r, :n], non_blocking=True)
