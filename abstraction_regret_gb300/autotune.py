"""Technique / block-shape / staging choice per automaton.

Two layers:

* ``choose_nfa_plan`` -- a rule from the automaton's features (state count, set words,
  edges, epsilon and wildcard use, resident bytes) and the batch size; used when nothing
  has been measured for that feature bucket yet.
* ``Autotuner`` -- times candidate plans on a probe batch (CUDA events, after a warm-up
  launch), keeps the fastest per feature bucket, and persists the table as JSON so a
  later process reuses it.

The reference has no tuner: its CUDA default technique is fixed (``dense``,
src/gpufsm/backends/cuda/nfa.py:136-137) and the state-count caps of its register and
shared-memory kernels are hard errors (bitpacked.cu:183-186, worklist_global.cu:542-556).
"""

from __future__ import annotations

import ctypes
import json
import math
import os
import threading
from dataclasses import asdict, dataclass
from pathlib import Path

import numpy as np

from . import costmodel, native

BITMAP_MAX_WORDS = 8  # thread-per-input bitmaps beyond 512 states scan too many words


@dataclass(frozen=True)
class Features:
    num_states: int
    num_words: int
    num_edges: int
    num_eps: int
    uses_any: bool
    resident_bytes: int

    @property
    def mean_degree(self) -> float:
        return self.num_edges / max(1, self.num_states)

    def bucket(self) -> str:
        """Coarse key: log2 of states and of mean degree, epsilon and wildcard flags."""
        return (f"n{int(math.log2(max(1, self.num_states)))}"
                f"-d{int(math.log2(max(1.0, self.mean_degree)))}"
                f"-e{int(self.num_eps > 0)}-a{int(self.uses_any)}")


def features(dev_nfa) -> Features:
    """Features of a ``DeviceNFA`` (or of any object with the same attributes)."""
    return Features(
        num_states=int(dev_nfa.num_states),
        num_words=int(dev_nfa.num_words),
        num_edges=int(dev_nfa.num_sym_edges),
        num_eps=int(dev_nfa.num_eps_edges),
        uses_any=bool(dev_nfa.uses_any),
        resident_bytes=int(getattr(dev_nfa, "edge_bytes", 0)),
    )


def features_of(nfa) -> Features:
    """Features straight from a CSR NFA (no device layout needed)."""
    n = int(nfa.num_states)
    ssy = np.asarray(nfa.sym_symbols)
    nnz = int(np.asarray(nfa.sym_targets).size)
    nne = int(np.asarray(nfa.eps_targets).size)
    return Features(n, -(-n // 64), nnz, nne, bool(np.any(ssy == 256)) if nnz else False,
                    16 * (nnz + nne) + 8 * (n + 1))


def _sm_count() -> int:
    try:
        import torch

        return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    except Exception:  # noqa: BLE001 - a rule needs a number, not a device
        return 152


def rule_plan(f: Features, n_inputs: int) -> native.Plan:
    """The rule used before (or instead of) measurement."""
    sms = _sm_count()
    # Many inputs and a small state set: one thread per input keeps every lane busy, as
    # long as its sets stay in shared memory (the cost model's residency: otherwise each
    # symbol moves 4 words of set per state-word through global memory) and its word
    # scan per symbol stays short.
    bitmap_ws = costmodel.working_set_traffic_per_symbol(
        f, costmodel.residency(f, native.TECH_BITMAP, 128))
    if (f.num_words <= BITMAP_MAX_WORDS and bitmap_ws == 0 and n_inputs >= 8 * sms * 32
            and not f.uses_any):
        return native.make_plan(native.TECH_BITMAP, block_threads=128, stage=1)
    # Otherwise a warp per input; the sparse list falls back to the dense bitmap itself.
    threads = 128 if n_inputs >= 4 * sms * 4 else 64
    return native.make_plan(native.TECH_COMPACT, block_threads=threads,
                            list_capacity=256 if (f.uses_any or f.num_eps) else 128, stage=1)


def choose_nfa_plan(dev_nfa, n_inputs: int, persistent: bool = False):
    """A plan for a plain launch, or an ``NfaChoice`` for the persistent engine."""
    f = features(dev_nfa) if hasattr(dev_nfa, "num_sym_edges") else features_of(dev_nfa)
    tuned = default_tuner().lookup(f, persistent)
    if persistent:
        from .engine import NfaChoice

        if tuned is not None:
            return NfaChoice(technique=tuned["technique"], list_capacity=tuned["list_capacity"])
        return NfaChoice(technique=native.TECH_COMPACT,
                         list_capacity=256 if (f.uses_any or f.num_eps) else 128)
    if tuned is not None:
        return native.make_plan(tuned["technique"], block_threads=tuned["block_threads"],
                                list_capacity=tuned["list_capacity"], stage=tuned["stage"])
    return rule_plan(f, n_inputs)


def prefer_engine(dev_nfa, lengths, model=None) -> bool:
    """Run this batch through the chunked engine rather than one plain launch? The cost
    model's answer (costmodel.py): a plain launch takes at least its longest input's
    chain of dependent steps; the engine adds planning and three launches but cuts every
    input into chunks that run in parallel. Only automata with speculative start sets
    can be chunked."""
    lengths = np.asarray(lengths)
    if lengths.size == 0 or not getattr(dev_nfa, "speculative", False):
        return False
    f = features(dev_nfa) if hasattr(dev_nfa, "num_sym_edges") else features_of(dev_nfa)
    m = model or costmodel.DEFAULT
    return m.predict_engine_ms(f, lengths) < m.predict_plain_ms(f, lengths)


def candidate_plans(f: Features) -> list[native.Plan]:
    """The plain-launch search space for one automaton."""
    out = []
    if f.num_words <= 2 * BITMAP_MAX_WORDS:
        for threads in (64, 128, 256):
            for stage in (0, 1):
                out.append(native.make_plan(native.TECH_BITMAP, threads, 0, stage))
    for tech in (native.TECH_WARP, native.TECH_COMPACT):
        for threads in (64, 128, 256):
            for stage in (0, 1):
                for cap in ((0,) if tech == native.TECH_WARP else (64, 256)):
                    out.append(native.make_plan(tech, threads, cap, stage))
    return out


def plan_dict(p: native.Plan) -> dict:
    return {"technique": int(p.technique), "block_threads": int(p.block_threads),
            "list_capacity": int(p.list_capacity), "stage": int(p.stage)}


class Autotuner:
    """Measured technique table keyed by feature bucket (and plain vs persistent)."""

    def __init__(self, path: str | os.PathLike | None = None) -> None:
        self.path = Path(path) if path else None
        self.table: dict[str, dict] = {}
        self._lock = threading.Lock()
        if self.path and self.path.exists():
            try:
                self.table = json.loads(self.path.read_text())
            except (OSError, ValueError):
                self.table = {}

    @staticmethod
    def _key(f: Features, persistent: bool) -> str:
        return ("persistent:" if persistent else "plain:") + f.bucket()

    def lookup(self, f: Features, persistent: bool = False) -> dict | None:
        return self.table.get(self._key(f, persistent))

    def record(self, f: Features, persistent: bool, choice: dict) -> None:
        with self._lock:
            self.table[self._key(f, persistent)] = choice
            if self.path:
                self.path.parent.mkdir(parents=True, exist_ok=True)
                self.path.write_text(json.dumps(self.table, indent=1, sort_keys=True))

    def tune_plain(self, dev_nfa, d_data, d_off, n_inputs: int, repeats: int = 3) -> dict:
        """Time every candidate plan on a resident probe batch; keep the fastest."""
        import torch

        lib = native.lib()
        f = features(dev_nfa)
        dev = dev_nfa.device
        out = torch.zeros((3, max(1, n_inputs)), dtype=torch.int32, device=dev)
        stream = torch.cuda.current_stream(dev)
        best, best_ms, timings = None, float("inf"), []
        for plan in candidate_plans(f):
            need = int(lib.gbfsm_nfa_workspace_bytes(ctypes.byref(dev_nfa.desc), n_inputs,
                                                     ctypes.byref(plan)))
            ws = torch.empty(max(need, 16), dtype=torch.uint8, device=dev)

            def launch():
                st = lib.gbfsm_nfa_run(ctypes.byref(dev_nfa.desc), d_data.data_ptr(),
                                       d_off.data_ptr(), n_inputs, ctypes.byref(plan),
                                       out[0].data_ptr(), out[1].data_ptr(), None,
                                       ws.data_ptr(), need, stream.cuda_stream)
                native.check(st, "gbfsm_nfa_run (autotune)")

            try:
                launch()
            except (ValueError, RuntimeError):
                continue
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(repeats):
                launch()
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / repeats
            timings.append((plan_dict(plan), ms))
            if ms < best_ms:
                best, best_ms = plan, ms
        if best is None:
            raise RuntimeError("no candidate plan could be launched")
        choice = plan_dict(best)
        choice["ms"] = best_ms
        self.record(f, False, choice)
        return {"best": choice, "timings": timings}


_DEFAULT: Autotuner | None = None


def default_tuner() -> Autotuner:
    """Process-wide tuner; persisted at $GBFSM_TUNE_CACHE when that is set."""
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Autotuner(os.environ.get("GBFSM_TUNE_CACHE"))
    return _DEFAULT


__all__ = ["Autotuner", "Features", "choose_nfa_plan", "default_tuner", "features",
           "features_of", "rule_plan", "candidate_plans", "plan_dict", "asdict"]
