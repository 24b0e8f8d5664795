"""Persistent batched engine: many automata, many uneven inputs, one launch.

``PersistentEngine`` keeps a pool of automata resident on the device (NFAs and DFAs of
any size) together with a device table of their descriptors. A batch is a list of
``(automaton index, input)`` requests; it becomes a task queue sorted longest first
(NFA inputs one task each, DFA inputs grouped up to 32 per task for one lane each), and
``gbfsm_persistent_run`` drains the queue with resident CTAs in a single launch.

``GraphRunner`` captures one batch shape (host->device copies of the inputs and the
task queue, the persistent launch, and the device->host copy of the verdicts) into a
CUDA graph, so a repeated batch costs one graph launch.

The reference has no counterpart: it builds one executor per call and launches once
per automaton (src/gpufsm/api.py:27-52, backends/cuda/nfa.py:105-121).
"""

from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import native
from .device import DeviceDFA, DeviceNFA, resolve_device
from .registry import Kind
from .result import Result, batch_results
from .staging import Results, Staging

DFA_GROUP = 32
NFA_BYTE_WEIGHT = 4  # task-ordering weight of an NFA byte relative to a DFA byte


@dataclass
class NfaChoice:
    """Per-automaton technique inside a persistent launch."""

    technique: int = native.TECH_COMPACT  # TECH_COMPACT or TECH_WARP
    list_capacity: int = 128


class PersistentEngine:
    """A resident automaton pool plus the persistent launch over it."""

    def __init__(self, automata, device=None, choices=None, block_threads: int = 256,
                 list_capacity: int | None = None, ctas_per_sm: int = 0) -> None:
        self.device = resolve_device(device)
        self.automata = list(automata)
        if not self.automata:
            raise ValueError("the engine needs at least one automaton")
        self.kinds = [Kind.of(a) for a in self.automata]
        self.dev = []
        for a, k in zip(self.automata, self.kinds):
            self.dev.append(DeviceNFA(a, self.device) if k is Kind.NFA else DeviceDFA(a, self.device))
        choices = list(choices) if choices is not None else [NfaChoice() for _ in self.automata]
        self.choices = choices
        caps = [c.list_capacity for c, k in zip(choices, self.kinds) if k is Kind.NFA]
        cap = list_capacity if list_capacity else (max(caps) if caps else 32)
        self.max_words = max([d.num_words for d in self.dev if isinstance(d, DeviceNFA)] or [1])
        self.plan = native.make_plan(native.TECH_COMPACT, block_threads=block_threads,
                                     list_capacity=cap, ctas_per_sm=ctas_per_sm)
        lib = native.lib()
        with torch.cuda.device(self.device):
            self.ctas_per_sm = int(lib.gbfsm_persistent_ctas_per_sm(self.max_words,
                                                                    ctypes.byref(self.plan)))
            if self.ctas_per_sm <= 0:
                raise ValueError(
                    f"persistent launch does not fit: {block_threads} threads with "
                    f"{self.max_words} set words and list capacity {cap}")
            self.ws_bytes = int(lib.gbfsm_persistent_workspace_bytes(self.max_words,
                                                                     ctypes.byref(self.plan)))
            self.workspace = torch.zeros(self.ws_bytes, dtype=torch.uint8, device=self.device)
            table = (native.Automaton * len(self.automata))()
            for i, (d, k, c) in enumerate(zip(self.dev, self.kinds, choices)):
                if k is Kind.NFA:
                    table[i].kind = 0
                    table[i].technique = c.technique
                    table[i].list_capacity = min(c.list_capacity, cap)
                    table[i].nfa = d.desc
                else:
                    table[i].kind = 1
                    table[i].dfa = d.desc
            raw = np.frombuffer(bytes(table), dtype=np.uint8).copy()
            self.table = torch.from_numpy(raw).to(self.device)
        self._staging = Staging(self.device)
        self._results = Results(self.device)
        self._task_cap = 0

    # ---- task queue ---------------------------------------------------------------------

    def make_tasks(self, aut_ids: np.ndarray, lengths: np.ndarray):
        """Task queue (int32 ``[n_tasks, 4]``) and input-id list, most work first.

        NFA inputs are one task each; a DFA's inputs are sorted longest first and grouped
        32 to a task (one per lane). Tasks are ordered by estimated cost (bytes, with an
        NFA byte weighted ``NFA_BYTE_WEIGHT`` DFA bytes) so the longest serial chains
        start first.
        """
        aut_ids = np.asarray(aut_ids, dtype=np.int64)
        lengths = np.asarray(lengths, dtype=np.int64)
        n = aut_ids.size
        if n == 0:
            return np.zeros((0, 4), dtype=np.int32), np.zeros(1, dtype=np.int32)
        if aut_ids.min() < 0 or aut_ids.max() >= len(self.automata):
            raise ValueError("request names an automaton outside the pool")
        is_dfa = np.array([k is Kind.DFA for k in self.kinds], dtype=bool)[aut_ids]
        nfa_idx = np.flatnonzero(~is_dfa)
        dfa_idx = np.flatnonzero(is_dfa)
        dfa_idx = dfa_idx[np.lexsort((-lengths[dfa_idx], aut_ids[dfa_idx]))]
        input_ids = np.concatenate([nfa_idx, dfa_idx]).astype(np.int32)
        rows = [np.stack([aut_ids[nfa_idx], np.arange(nfa_idx.size), np.ones_like(nfa_idx),
                          lengths[nfa_idx] * NFA_BYTE_WEIGHT], axis=1)]
        if dfa_idx.size:
            sa = aut_ids[dfa_idx]
            seg_starts = np.flatnonzero(np.r_[True, sa[1:] != sa[:-1]])
            seg_ends = np.r_[seg_starts[1:], sa.size]
            firsts, counts = [], []
            for s, e in zip(seg_starts.tolist(), seg_ends.tolist()):
                for gs in range(s, e, DFA_GROUP):
                    firsts.append(gs)
                    counts.append(min(DFA_GROUP, e - gs))
            g = np.asarray(firsts, dtype=np.int64)
            rows.append(np.stack([sa[g], nfa_idx.size + g, np.asarray(counts, dtype=np.int64),
                                  lengths[dfa_idx[g]]], axis=1))
        t = np.concatenate(rows)
        t = t[np.argsort(-t[:, 3], kind="stable")]
        t[:, 3] = 0
        return t.astype(np.int32), input_ids

    # ---- launches -------------------------------------------------------------------------

    def new_workspace(self) -> torch.Tensor:
        """A separate workspace (queue ticket + dense scratch) for a concurrent launch."""
        return torch.zeros(self.ws_bytes, dtype=torch.uint8, device=self.device)

    def launch(self, d_data, d_off, d_tasks, n_tasks, d_ids, d_flags, d_lens, d_examined=None,
               stream=None, d_ends=None, workspace=None) -> None:
        """Enqueue the persistent launch (no synchronisation).

        ``d_data`` is a device tensor or a raw address (e.g. of pinned host memory the
        device reads directly); with ``d_ends`` input i spans ``[d_off[i], d_ends[i])``.
        """
        stream = stream or torch.cuda.current_stream(self.device)
        ws = self.workspace if workspace is None else workspace
        data_ptr = d_data if isinstance(d_data, int) else d_data.data_ptr()
        st = native.lib().gbfsm_persistent_run(
            self.table.data_ptr(), len(self.automata), self.max_words, d_tasks.data_ptr(),
            int(n_tasks), d_ids.data_ptr(), data_ptr, d_off.data_ptr(),
            d_ends.data_ptr() if d_ends is not None else None,
            d_flags.data_ptr(), d_lens.data_ptr(),
            d_examined.data_ptr() if d_examined is not None else None,
            ws.data_ptr(), self.ws_bytes, ctypes.byref(self.plan), stream.cuda_stream)
        native.check(st, "gbfsm_persistent_run")

    def _upload_tasks(self, tasks: np.ndarray, ids: np.ndarray, stream):
        need_t = max(1, tasks.shape[0]) * 4
        need_i = max(1, ids.size)
        if need_t > self._task_cap or need_i > getattr(self, "_id_cap", 0):
            self._task_cap = max(need_t, 2 * self._task_cap)
            self._id_cap = max(need_i, 2 * getattr(self, "_id_cap", 0))
            self._h_tasks = torch.empty(self._task_cap, dtype=torch.int32, pin_memory=True)
            self._d_tasks = torch.empty(self._task_cap, dtype=torch.int32, device=self.device)
            self._h_ids = torch.empty(self._id_cap, dtype=torch.int32, pin_memory=True)
            self._d_ids = torch.empty(self._id_cap, dtype=torch.int32, device=self.device)
        nt = tasks.size
        self._h_tasks.numpy()[:nt] = tasks.reshape(-1)
        self._h_ids.numpy()[:ids.size] = ids
        with torch.cuda.stream(stream):
            self._d_tasks[:max(nt, 1)].copy_(self._h_tasks[:max(nt, 1)], non_blocking=True)
            self._d_ids[:ids.size].copy_(self._h_ids[:ids.size], non_blocking=True)
        return self._d_tasks, self._d_ids

    def run_requests(self, aut_ids, inputs, with_examined: bool = False):
        """Host path: ``inputs[i]`` runs on automaton ``aut_ids[i]``.

        Returns ``(flags, lens, examined | None, kernel_ms, transfer_ms)`` as numpy arrays
        indexed like ``inputs``.
        """
        t0 = time.perf_counter()
        n = len(inputs)
        stream = torch.cuda.current_stream(self.device)
        lengths = np.fromiter((len(b) for b in inputs), dtype=np.int64, count=n)
        tasks, ids = self.make_tasks(np.asarray(aut_ids), lengths)
        d_data, d_off, _, _ = self._staging.put(inputs, stream)
        d_tasks, d_ids = self._upload_tasks(tasks, ids, stream)
        self._results.ensure(max(n, 1))
        res = self._results
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        self.launch(d_data, d_off, d_tasks, tasks.shape[0], d_ids, res.d[0], res.d[1],
                    res.d[2] if with_examined else None, stream)
        e1.record(stream)
        res.fetch(n, stream)
        stream.synchronize()
        kernel_ms = e0.elapsed_time(e1)
        total_ms = (time.perf_counter() - t0) * 1e3
        h = res.h.numpy()
        flags = h[0, :n].copy()
        lens = h[1, :n].copy()
        if n and flags.min() < 0:
            raise TimeoutError("a bounded device wait gave up during the persistent launch")
        examined = h[2, :n].copy() if with_examined else None
        return flags, lens, examined, kernel_ms, max(0.0, total_ms - kernel_ms)

    def run(self, requests) -> list[Result]:
        """``requests`` is a list of ``(automaton index, bytes)``; one Result each."""
        if not requests:
            return []
        aut = [r[0] for r in requests]
        data = [r[1] for r in requests]
        flags, lens, _, kms, tms = self.run_requests(aut, data)
        return batch_results(flags, lens, kms, tms)


class GraphRunner:
    """A fixed batch captured as one CUDA graph: H2D inputs, persistent launch, D2H verdicts.

    The batch (flat uint8 data + int64 offsets + automaton ids) is fixed at construction;
    ``replay`` re-runs it end to end. ``set_inputs`` may rewrite the pinned input bytes
    in place (same lengths) between replays.
    """

    def __init__(self, engine: PersistentEngine, aut_ids, data: np.ndarray, offsets: np.ndarray,
                 with_examined: bool = False) -> None:
        self.engine = engine
        dev = engine.device
        n = len(offsets) - 1
        self.n = n
        lengths = np.diff(np.asarray(offsets, dtype=np.int64))
        tasks, ids = engine.make_tasks(np.asarray(aut_ids), lengths)
        self.n_tasks = tasks.shape[0]
        total = int(offsets[-1])
        padded = max(16, -(-total // 16) * 16)
        self.h_data = torch.zeros(padded, dtype=torch.uint8, pin_memory=True)
        self.h_data.numpy()[:total] = np.asarray(data[:total], dtype=np.uint8)
        self.h_off = torch.from_numpy(np.asarray(offsets, dtype=np.int64).copy()).pin_memory()
        self.h_tasks = torch.from_numpy(tasks.reshape(-1).copy() if tasks.size else
                                        np.zeros(4, np.int32)).pin_memory()
        self.h_ids = torch.from_numpy(ids.copy()).pin_memory()
        self.h_out = torch.zeros((3, max(n, 1)), dtype=torch.int32, pin_memory=True)
        self.d_data = torch.empty_like(self.h_data, device=dev)
        self.d_off = torch.empty_like(self.h_off, device=dev)
        self.d_tasks = torch.empty_like(self.h_tasks, device=dev)
        self.d_ids = torch.empty_like(self.h_ids, device=dev)
        self.d_out = torch.zeros((3, max(n, 1)), dtype=torch.int32, device=dev)
        self.with_examined = with_examined
        self.h2d_bytes = padded + self.h_off.numel() * 8 + self.h_tasks.numel() * 4 + \
            self.h_ids.numel() * 4
        self.d2h_bytes = self.h_out.numel() * 4
        self.stream = torch.cuda.Stream(dev)
        # warm-up outside capture (sets kernel attributes, loads modules)
        with torch.cuda.stream(self.stream):
            self._body()
        self.stream.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream):
            self._body()
        torch.cuda.synchronize(dev)

    def _body(self) -> None:
        s = torch.cuda.current_stream(self.engine.device)
        self.d_data.copy_(self.h_data, non_blocking=True)
        self.d_off.copy_(self.h_off, non_blocking=True)
        self.d_tasks.copy_(self.h_tasks, non_blocking=True)
        self.d_ids.copy_(self.h_ids, non_blocking=True)
        self.engine.launch(self.d_data, self.d_off, self.d_tasks, self.n_tasks, self.d_ids,
                           self.d_out[0], self.d_out[1],
                           self.d_out[2] if self.with_examined else None, s)
        self.h_out.copy_(self.d_out, non_blocking=True)

    def replay(self, stream=None) -> None:
        """Launch the captured graph (asynchronous)."""
        self.graph.replay()

    def kernel_only(self, stream=None) -> None:
        """The persistent launch alone on resident inputs (for device-side timing)."""
        stream = stream or torch.cuda.current_stream(self.engine.device)
        self.engine.launch(self.d_data, self.d_off, self.d_tasks, self.n_tasks, self.d_ids,
                           self.d_out[0], self.d_out[1],
                           self.d_out[2] if self.with_examined else None, stream)

    def verdicts(self):
        h = self.h_out.numpy()
        return h[0, :self.n].copy(), h[1, :self.n].copy(), h[2, :self.n].copy()
