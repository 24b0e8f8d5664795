"""Result and benchmark-statistics types (reference: ``src/gpufsm/core/result.py:11-94``).

Same fields, same equality rule (``matches`` compares the verdict only) and the same
batch timing convention: a batched launch has one kernel time, reported on the first
result of the batch, with zeros on the rest, so ``results[0].kernel_ms`` is always the
batch time.
"""

from __future__ import annotations

import math
from collections.abc import Sequence
from dataclasses import dataclass, field
from typing import Any


@dataclass
class Result:
    """Verdict and timings of one input on one backend/technique."""

    accepted: bool
    match_len: int
    kernel_ms: float = 0.0
    total_ms: float = 0.0
    transfer_ms: float = 0.0
    mem_bytes: int = 0

    def matches(self, other: Result) -> bool:
        """True when both verdicts agree; timings are not compared."""
        return self.accepted == other.accepted and self.match_len == other.match_len


def batch_results(
    flags: Sequence[Any],
    lens: Sequence[Any],
    kernel_ms: float,
    transfer_ms: float = 0.0,
) -> list[Result]:
    """One :class:`Result` per input, with the batch's times on the first one only."""
    # verdicts as plain Python bools and ints, converted in bulk, then positional
    # construction: about half the time of per-item conversion and keyword construction
    f = (flags != 0).tolist() if hasattr(flags, "tolist") else [bool(x) for x in flags]
    m = lens.tolist() if hasattr(lens, "tolist") else [int(x) for x in lens]
    out = [Result(a, b) for a, b in zip(f, m)]
    if out:
        first = out[0]
        first.kernel_ms = kernel_ms
        first.total_ms = kernel_ms + transfer_ms
        first.transfer_ms = transfer_ms
    return out


def blank_results(n: int, result_cls=Result) -> list:
    """``n`` results with empty verdicts and zero times, for ``fill_results``: a batch's
    executor builds them while the device runs, so that only the verdicts are written
    once the device has finished."""
    return [result_cls(False, 0) for _ in range(n)]


def fill_results(out: list, flags, lens, kernel_ms: float, transfer_ms: float = 0.0) -> list:
    """Write a batch's verdicts into ``out`` (from ``blank_results``) with the timing
    convention of ``batch_results``; the objects equal those ``batch_results`` builds."""
    f = (flags != 0).tolist() if hasattr(flags, "tolist") else [bool(x) for x in flags]
    m = lens.tolist() if hasattr(lens, "tolist") else [int(x) for x in lens]
    if len(out) != len(f):
        raise ValueError(f"{len(out)} results for {len(f)} verdicts")
    for r, a, b in zip(out, f, m):
        r.accepted = a
        r.match_len = b
    if out:
        first = out[0]
        first.kernel_ms = kernel_ms
        first.total_ms = kernel_ms + transfer_ms
        first.transfer_ms = transfer_ms
    return out


@dataclass
class BenchmarkStats:
    """Timings of ``n`` repeated runs after warm-up: mean, sample std, normal CI95."""

    backend: str
    technique: str
    accepted: bool
    match_len: int
    n: int
    raw_ms: list[float] = field(default_factory=list)

    @property
    def mean_ms(self) -> float:
        return sum(self.raw_ms) / len(self.raw_ms) if self.raw_ms else 0.0

    @property
    def std_ms(self) -> float:
        k = len(self.raw_ms)
        if k < 2:
            return 0.0
        m = self.mean_ms
        return math.sqrt(sum((x - m) ** 2 for x in self.raw_ms) / (k - 1))

    @property
    def ci95_ms(self) -> float:
        """Half-width of the normal-approximation 95% interval of the mean."""
        k = len(self.raw_ms)
        return 1.96 * self.std_ms / math.sqrt(k) if k >= 2 else 0.0

    def as_row(self) -> dict[str, float | str | int | bool]:
        return {
            "backend": self.backend,
            "technique": self.technique,
            "accepted": self.accepted,
            "match_len": self.match_len,
            "n": self.n,
            "mean_ms": round(self.mean_ms, 6),
            "std_ms": round(self.std_ms, 6),
            "ci95_ms": round(self.ci95_ms, 6),
        }
