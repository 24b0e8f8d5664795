"""Host->device staging of byte batches through reusable pinned buffers.

The reference widens every input byte to an int32 and copies the batch synchronously
from pageable memory on every call (src/gpufsm/core/packing.py:35-63,
native/include/common.cuh:150-159). Here a batch is packed once into a pinned uint8
buffer (1 byte per symbol, int64 offsets, 16-byte padding) and copied with
``cudaMemcpyAsync`` on the caller's stream; buffers grow geometrically and are reused.
"""

from __future__ import annotations

import numpy as np
import torch

from .packing import PAD


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

    def __init__(self, device: torch.device) -> None:
        self.device = device
        self._h_data = self._d_data = None
        self._h_off = self._d_off = None
        self._cap_data = self._cap_off = 0

    def _ensure(self, nbytes: int, n_off: int) -> None:
        if nbytes > self._cap_data:
            self._cap_data = _grow(self._cap_data, nbytes)
            self._h_data = torch.empty(self._cap_data, dtype=torch.uint8, pin_memory=True)
            self._d_data = torch.empty(self._cap_data, dtype=torch.uint8, device=self.device)
        if n_off > self._cap_off:
            self._cap_off = _grow(self._cap_off, n_off)
            self._h_off = torch.empty(self._cap_off, dtype=torch.int64, pin_memory=True)
            self._d_off = torch.empty(self._cap_off, dtype=torch.int64, device=self.device)

    def put(self, inputs, stream: torch.cuda.Stream):
        """Pack ``inputs`` (bytes-like objects) and start their copy on ``stream``.

        Returns ``(d_data, d_offsets, h_offsets, total_bytes)``; device tensors are views
        of the staging buffers (valid until the next ``put``).
        """
        n = len(inputs)
        lens = np.fromiter((len(b) for b in inputs), dtype=np.int64, count=n)
        total = int(lens.sum()) if n else 0
        padded = max(PAD, -(-total // PAD) * PAD)
        self._ensure(padded, n + 1)
        h_off = self._h_off.numpy()[: n + 1]
        h_off[0] = 0
        if n:
            np.cumsum(lens, out=h_off[1:])
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
