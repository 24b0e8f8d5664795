"""CUDA executors and their registration under ``Backend.CUDA``.

An executor owns one automaton resident on the device and runs batches of inputs
through one technique. ``run(bytes)`` is ``run_batch([bytes])[0]``; ``run_batch`` makes
one launch for the whole batch and reports with the convention of ``batch_results`` (the
batch's kernel time on result 0, reference core/result.py:27-50): its ``Result`` objects
are built while the device runs (``blank_results``) and given their verdicts once it has
finished (``fill_results``).

Technique names. The reference's CUDA names are registered with the meaning they have
there (src/gpufsm/backends/cuda/nfa.py:26-41, dfa.py:50-53), so callers and the
reference's own GPU tests keep working, each mapped onto this engine's kernels:

====================  ===========================================================
NFA name              engine kernel
====================  ===========================================================
auto (default)        per batch: the persistent engine (chunked, see below) when
                      inputs are long enough to cut, else the autotuned plain
                      launch (bitmap / warp / compact, block shape, staging)
bitmap, worklist,     thread per input, packed bitmap in shared memory
multistream, dense,   (``worklist`` and ``multistream_shared`` stage the edge rows
bitpacked,            in shared memory with TMA bulk copies; ``multistream_async``
multistream_shared,   reports end-to-end time in ``kernel_ms`` as the reference's
multistream_async     async pipeline does)
warp, worklist_warp,  warp per input, dense bitmap, ballot/popc/shuffle expansion
worklist_global,      (``worklist_shared`` stages the edge rows)
worklist_shared
compact,              warp per input, sparse member list (dense on overflow)
worklist_compact
persistent            the persistent batched engine (one resident launch)
====================  ===========================================================

DFA names: ``gather`` (default; the table walk, staged in shared memory when it fits)
and ``persistent``.
"""

from __future__ import annotations

import ctypes
import time
import weakref
from collections import OrderedDict

import numpy as np
import torch

from . import native
from .autotune import choose_nfa_plan, prefer_engine
from .device import DeviceDFA, DeviceNFA, resolve_device
from .engine import NfaChoice, PersistentEngine
from .registry import Backend, Kind, register, register_availability, set_unavailable_reason
from .result import Result, blank_results, fill_results
from .staging import Results, Staging

# technique -> (engine technique, stage edge rows, end-to-end timing)
NFA_TECHNIQUES: dict[str, tuple[int, int, bool]] = {
    "bitmap": (native.TECH_BITMAP, 0, False),
    "warp": (native.TECH_WARP, 0, False),
    "compact": (native.TECH_COMPACT, 0, False),
    "dense": (native.TECH_BITMAP, 1, False),
    "bitpacked": (native.TECH_BITMAP, 1, False),
    "multistream": (native.TECH_BITMAP, 0, False),
    "multistream_shared": (native.TECH_BITMAP, 1, False),
    "multistream_async": (native.TECH_BITMAP, 0, True),
    "worklist": (native.TECH_BITMAP, 1, False),
    "worklist_global": (native.TECH_WARP, 0, False),
    "worklist_warp": (native.TECH_WARP, 0, False),
    "worklist_shared": (native.TECH_WARP, 1, False),
    "worklist_compact": (native.TECH_COMPACT, 0, False),
}

MAX_INPUT_BYTES = (1 << 31) - 1  # match_len is int32, as in the reference


def _lengths(inputs) -> np.ndarray:
    """The inputs' lengths (int64); raises when one exceeds the int32 match_len range."""
    lens = np.fromiter(map(len, inputs), dtype=np.int64, count=len(inputs))
    if lens.size and int(lens.max()) > MAX_INPUT_BYTES:
        raise ValueError(f"an input of {int(lens.max())} bytes exceeds the int32 match_len range")
    return lens


class _BatchExecutor:
    """Shared host path: stage inputs, launch, fetch verdicts, time with CUDA events."""

    end_to_end = False

    def __init__(self, device) -> None:
        self.device = resolve_device(device)
        self._staging = Staging(self.device)
        self._results = Results(self.device)

    def _launch(self, d_data, d_off, n, d_flags, d_lens, d_examined, stream) -> None:
        raise NotImplementedError

    def run_arrays(self, inputs, with_examined: bool = False, lengths=None, idle=None):
        """``(flags, lens, examined | None, kernel_ms, transfer_ms)`` for a batch;
        ``idle`` is called once the launch is enqueued, before the host waits for it."""
        if lengths is None:
            lengths = _lengths(inputs)
        t0 = time.perf_counter()
        n = len(inputs)
        stream = torch.cuda.current_stream(self.device)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if self.end_to_end:
            e0.record(stream)
        d_data, d_off, _, _ = self._staging.put(inputs, stream, lengths=lengths)
        self._results.ensure(max(n, 1))
        r = self._results
        if not self.end_to_end:
            e0.record(stream)
        self._launch(d_data, d_off, n, r.d[0], r.d[1], r.d[2] if with_examined else None, stream)
        if not self.end_to_end:
            e1.record(stream)
        r.fetch(n, stream)
        if self.end_to_end:
            e1.record(stream)
        if idle is not None:
            idle()
        stream.synchronize()
        kernel_ms = e0.elapsed_time(e1)
        wall_ms = (time.perf_counter() - t0) * 1e3
        h = r.h.numpy()
        flags, lens = h[0, :n].copy(), h[1, :n].copy()
        if n and flags.min() < 0:
            raise TimeoutError("a bounded device wait gave up (shared-memory staging)")
        examined = h[2, :n].copy() if with_examined else None
        return flags, lens, examined, kernel_ms, max(0.0, wall_ms - kernel_ms)

    def run_batch(self, inputs) -> list[Result]:
        return run_batch_results(self, inputs)

    def run(self, input_bytes: bytes) -> Result:
        return self.run_batch([input_bytes])[0]


def run_batch_results(executor, inputs, result_cls=Result) -> list:
    """``executor.run_arrays`` on ``inputs`` as one ``result_cls`` per input, built while
    the device runs and filled with the verdicts afterwards."""
    if not inputs:
        return []
    out: list = []
    flags, lens, _, kms, tms = executor.run_arrays(
        inputs, idle=lambda: out.extend(blank_results(len(inputs), result_cls)))
    if not out:  # a path that did not call idle
        out = blank_results(len(inputs), result_cls)
    return fill_results(out, flags, lens, float(kms), float(tms))


class CudaNFAExecutor(_BatchExecutor):
    """One NFA resident on the device, one plain launch per batch."""

    def __init__(self, nfa, technique: str = "auto", device=None, plan=None) -> None:
        super().__init__(device)
        self.nfa = nfa
        self.technique = technique
        self.dev = DeviceNFA(nfa, self.device)
        self._auto = technique == "auto" and plan is None
        if plan is not None:
            self.plan = plan
        elif self._auto:
            self.plan = None
        else:
            tech, stage, e2e = NFA_TECHNIQUES[technique]
            self.plan = native.make_plan(tech, stage=stage)
            self.end_to_end = e2e
        self._ws = None

    def _workspace(self, n: int):
        lib = native.lib()
        need = int(lib.gbfsm_nfa_workspace_bytes(ctypes.byref(self.dev.desc), n,
                                                 ctypes.byref(self.plan)))
        if need and (self._ws is None or self._ws.numel() < need):
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        return (self._ws.data_ptr() if need else None), need

    def _launch(self, d_data, d_off, n, d_flags, d_lens, d_examined, stream) -> None:
        if self._auto and self.plan is None:
            self.plan = choose_nfa_plan(self.dev, n)
        ws, ws_bytes = self._workspace(n)
        st = native.lib().gbfsm_nfa_run(
            ctypes.byref(self.dev.desc), d_data.data_ptr(), d_off.data_ptr(), n,
            ctypes.byref(self.plan), d_flags.data_ptr(), d_lens.data_ptr(),
            d_examined.data_ptr() if d_examined is not None else None, ws, ws_bytes,
            stream.cuda_stream)
        native.check(st, "gbfsm_nfa_run")

    def launch(self, d_data, d_off, n, d_flags, d_lens, d_examined=None, stream=None) -> None:
        """Enqueue one launch on resident device buffers (no synchronisation)."""
        self._launch(d_data, d_off, n, d_flags, d_lens, d_examined,
                     stream or torch.cuda.current_stream(self.device))


class CudaDFAExecutor(_BatchExecutor):
    """One DFA resident on the device as a packed table, one launch per batch."""

    def __init__(self, dfa, technique: str = "gather", device=None, plan=None) -> None:
        super().__init__(device)
        self.dfa = dfa
        self.technique = technique
        self.dev = DeviceDFA(dfa, self.device)
        self.plan = plan if plan is not None else native.make_plan(native.TECH_DFA_WALK, stage=1)

    def _launch(self, d_data, d_off, n, d_flags, d_lens, d_examined, stream) -> None:
        st = native.lib().gbfsm_dfa_run(
            ctypes.byref(self.dev.desc), d_data.data_ptr(), d_off.data_ptr(), n,
            ctypes.byref(self.plan), d_flags.data_ptr(), d_lens.data_ptr(),
            d_examined.data_ptr() if d_examined is not None else None, stream.cuda_stream)
        native.check(st, "gbfsm_dfa_run")

    def launch(self, d_data, d_off, n, d_flags, d_lens, d_examined=None, stream=None) -> None:
        self._launch(d_data, d_off, n, d_flags, d_lens, d_examined,
                     stream or torch.cuda.current_stream(self.device))


class CudaPersistentExecutor:
    """A single automaton run through the persistent batched engine."""

    def __init__(self, automaton, technique: str = "persistent", device=None,
                 resident=None) -> None:
        self.automaton = automaton
        self.technique = technique
        choice = NfaChoice()
        if Kind.of(automaton) is Kind.NFA:
            choice = choose_nfa_plan(automaton, 0, persistent=True)
        self.engine = PersistentEngine([automaton], device, choices=[choice],
                                       resident=[resident] if resident is not None else None)

    def run_arrays(self, inputs, with_examined: bool = False, lengths=None, idle=None):
        if lengths is None:
            lengths = _lengths(inputs)
        return self.engine.run_requests(np.zeros(len(inputs), dtype=np.int64), inputs,
                                        with_examined, lengths=lengths, idle=idle)

    def run_batch(self, inputs) -> list[Result]:
        return run_batch_results(self, inputs)

    def run(self, input_bytes: bytes) -> Result:
        return self.run_batch([input_bytes])[0]


class CudaAutoNFAExecutor:
    """The default NFA technique: per batch, one plain launch or the chunked engine.

    A plain launch simulates each input serially (one warp per input), so its time grows
    with the longest input; the engine cuts long inputs into chunks that run in parallel
    and resolves them exactly, at the cost of a few more launches. ``prefer_engine``
    (autotune.py) makes the choice from the automaton's features and the batch's lengths;
    both paths share one resident device layout."""

    def __init__(self, nfa, device=None) -> None:
        self.nfa = nfa
        self.technique = "auto"
        self.plain = CudaNFAExecutor(nfa, "auto", device)
        self.device = self.plain.device
        self._engine: CudaPersistentExecutor | None = None
        self.last_path = None

    def engine(self) -> CudaPersistentExecutor:
        if self._engine is None:
            self._engine = CudaPersistentExecutor(self.nfa, "persistent", self.device,
                                                  resident=self.plain.dev)
        return self._engine

    def run_arrays(self, inputs, with_examined: bool = False, idle=None):
        lengths = _lengths(inputs)
        if prefer_engine(self.plain.dev, lengths):
            self.last_path = "engine"
            return self.engine().run_arrays(inputs, with_examined, lengths, idle)
        self.last_path = "plain"
        return self.plain.run_arrays(inputs, with_examined, lengths, idle)

    def run_batch(self, inputs) -> list[Result]:
        return run_batch_results(self, inputs)

    def run(self, input_bytes: bytes) -> Result:
        return self.run_batch([input_bytes])[0]

    def launch(self, d_data, d_off, n, d_flags, d_lens, d_examined=None, stream=None) -> None:
        """One plain launch on resident device buffers (no synchronisation)."""
        self.plain.launch(d_data, d_off, n, d_flags, d_lens, d_examined, stream)


# ---- executor cache -------------------------------------------------------------------
#
# gpufsm.api.run/run_batch build a new executor on every call (reference
# src/gpufsm/api.py:45-52); a device-resident automaton would then be re-uploaded per
# call. Executors are cached per (automaton identity, technique) and dropped when the
# automaton is garbage-collected.

CACHE_LIMIT = 64  # executors kept alive at once (least recently used are dropped)

_CACHE: OrderedDict[tuple[int, str, int], tuple] = OrderedDict()


def _cached(automaton, technique: str, build):
    dev = resolve_device(None).index  # raises first when no CUDA device is visible
    key = (id(automaton), technique, dev)
    hit = _CACHE.get(key)
    if hit is not None and hit[0]() is automaton:
        _CACHE.move_to_end(key)
        return hit[1]
    ex = build()
    try:
        ref = weakref.ref(automaton, lambda _r, k=key: _CACHE.pop(k, None))
    except TypeError:  # not weak-referenceable: do not cache
        return ex
    _CACHE[key] = (ref, ex)
    while len(_CACHE) > CACHE_LIMIT:
        _CACHE.popitem(last=False)
    return ex


def clear_cache() -> None:
    _CACHE.clear()


def make_nfa_executor(automaton, technique: str):
    if Kind.of(automaton) is not Kind.NFA:
        raise TypeError("an NFA technique was asked to run a DFA")
    if technique == "persistent":
        return _cached(automaton, technique, lambda: CudaPersistentExecutor(automaton, technique))
    if technique == "auto":
        return _cached(automaton, technique, lambda: CudaAutoNFAExecutor(automaton))
    return _cached(automaton, technique, lambda: CudaNFAExecutor(automaton, technique))


def make_dfa_executor(automaton, technique: str):
    if Kind.of(automaton) is not Kind.DFA:
        raise TypeError("a DFA technique was asked to run an NFA")
    if technique == "persistent":
        return _cached(automaton, technique, lambda: CudaPersistentExecutor(automaton, technique))
    return _cached(automaton, technique, lambda: CudaDFAExecutor(automaton, technique))


def available() -> bool:
    """CUDA backend probe: the library loads and a CUDA device is visible."""
    try:
        native.lib()
    except Exception as exc:  # noqa: BLE001 - the reason is recorded, not swallowed
        set_unavailable_reason(Backend.CUDA, f"{type(exc).__name__}: {exc}")
        return False
    if not torch.cuda.is_available():
        set_unavailable_reason(Backend.CUDA, "no CUDA device visible to PyTorch")
        return False
    return True


NFA_NAMES = ["auto", *NFA_TECHNIQUES, "persistent"]
DFA_NAMES = ["gather", "persistent"]


def register_all(register_fn=register, availability_fn=register_availability,
                 kind_enum=Kind, backend_enum=Backend) -> None:
    """Register every technique (into this package's registry, or gpufsm's)."""
    for name in NFA_NAMES:
        register_fn(kind_enum.NFA, backend_enum.CUDA, name, default=(name == "auto"))(
            make_nfa_executor)
    for name in DFA_NAMES:
        register_fn(kind_enum.DFA, backend_enum.CUDA, name, default=(name == "gather"))(
            make_dfa_executor)
    availability_fn(backend_enum.CUDA, available)

# register every CUDA technique into this package registry at import time
register_all()
