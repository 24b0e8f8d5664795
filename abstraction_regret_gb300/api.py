"""Public API: ``run``, ``run_batch``, ``benchmark`` (reference: ``src/gpufsm/api.py:15-97``).

Same signatures, dispatch and timing contract as the reference: the automaton's kind
selects the technique table, ``run_batch`` uses the executor's native batch path (every
executor here has one) and ``results[0].kernel_ms`` is the batch time. One deliberate
difference: the default backend is ``Backend.CUDA``, because this package is the CUDA
backend and registers nothing else (``backend="cpu"`` raises the reference's
"has no ... technique" ``KeyError``).
"""

from __future__ import annotations

from . import executors as _executors  # noqa: F401  (registers the CUDA techniques)
from .registry import Backend, Kind, get_factory
from .result import BenchmarkStats, Result, batch_results


def run(automaton, input_bytes: bytes, backend: Backend | str = Backend.CUDA,
        technique: str | None = None) -> Result:
    """Run ``automaton`` over one input."""
    backend = Backend(backend)
    technique, factory = get_factory(Kind.of(automaton), backend, technique)
    return factory(automaton, technique).run(input_bytes)


def run_batch(automaton, inputs: list[bytes], backend: Backend | str = Backend.CUDA,
              technique: str | None = None) -> list[Result]:
    """Run ``automaton`` over a batch; one :class:`Result` per input, batch time on [0]."""
    backend = Backend(backend)
    technique, factory = get_factory(Kind.of(automaton), backend, technique)
    executor = factory(automaton, technique)
    batch = getattr(executor, "run_batch", None)
    if callable(batch):
        return batch(inputs)
    per_input = [executor.run(b) for b in inputs]
    if not per_input:
        return []
    return batch_results([r.accepted for r in per_input], [r.match_len for r in per_input],
                         kernel_ms=sum(r.kernel_ms for r in per_input),
                         transfer_ms=sum(r.transfer_ms for r in per_input))


def benchmark(automaton, input_bytes: bytes, backend: Backend | str = Backend.CUDA,
              technique: str | None = None, repeats: int = 10, warmup: int = 3) -> BenchmarkStats:
    """Time ``repeats`` runs after ``warmup``; mean / std / CI95 of ``kernel_ms``."""
    if repeats < 1:
        raise ValueError("repeats must be >= 1")
    backend = Backend(backend)
    technique, factory = get_factory(Kind.of(automaton), backend, technique)
    executor = factory(automaton, technique)
    last = None
    for _ in range(max(0, warmup)):
        last = executor.run(input_bytes)
    raw = []
    for _ in range(repeats):
        last = executor.run(input_bytes)
        raw.append(last.kernel_ms)
    return BenchmarkStats(backend=backend.value, technique=technique, accepted=last.accepted,
                          match_len=last.match_len, n=repeats, raw_ms=raw)
