"""Persistent batched engine: many automata, many uneven inputs, one resident launch.

``PersistentEngine`` keeps a pool of automata resident on the device (NFAs and DFAs of
any size) together with a device table of their descriptors. A batch is a list of
``(automaton index, input)`` requests. ``make_tasks`` turns it into a task queue sorted
by estimated work, longest first:

* DFA inputs are grouped up to 32 per task (one table walk per lane);
* short NFA inputs are one task each (a warp per input);
* long NFA inputs are cut into chunks that run **speculatively in parallel**: an
  input's first chunk runs exactly from the start configuration; every later chunk
  starts from a superset of the true active set (the targets of every edge labelled
  with the byte two positions before the chunk, then one step) and records its set
  sizes at checkpoints 1, 2, 4, ..., 32 bytes in, its first accept / death after each
  checkpoint and its final set. A second launch of FIXUP tasks resolves each input
  exactly: it re-runs a chunk from the true set only until the true set is as large as
  the recorded superset at a checkpoint -- then they are equal, because the superset
  always contains the true set and simulation preserves inclusion -- and continues
  from the record. The verdicts are exactly those of a serial run.

``gbfsm_persistent_run`` drains a queue with resident CTAs (one atomic ticket per task).
``GraphRunner`` captures a whole batch (host->device copies, both launches, the
device->host copy of the verdicts) in one CUDA graph.

The reference has no counterpart: it builds one executor per call and launches once per
automaton, one thread or warp per whole input (src/gpufsm/api.py:27-52,
backends/cuda/nfa.py:105-121).
"""

from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import native
from .device import DeviceDFA, DeviceNFA, resolve_device
from .registry import Kind
from .result import Result, blank_results, fill_results
from .staging import Results, Staging

DFA_GROUP = 32
NFA_BYTE_WEIGHT = 4  # task-ordering weight of an NFA byte relative to a DFA byte
MIN_CHUNK = 256      # shortest speculative chunk (bytes)
# shortest chunk of a pool whose NFAs all run in lanes with two-byte start sets of at
# most one state on average: their chunk starts are cheap, so a small batch gains from
# more, finer chunks (c1-live: 0.090 ms per step at 64 B against 0.151 ms at 256 B; a
# c3 batch, whose starts often widen, is fastest at 192-256 B)
MIN_CHUNK_SMALL_STARTS = 64
LANE_GROUP = 32      # chunks per LANES task (one per lane)
# an automaton's chunks run one per lane when its two-byte supersets are this small on
# average: a lane starts from the superset when it has at most native.LANE_CAPACITY
# states, else from the superset two bytes earlier stepped over the two bytes (up to 64
# states streamed once); sets that outgrow the lane spill to warps
LANE_PAIR_MEAN = 32.0
# resident warps per SM of the lane launch when the device is not asked (128-thread
# CTAs, 8 per SM: csrc/lanes.cu)
LANE_WARPS_PER_SM = 32
# DFA chunking (csrc/dfa_chunks.cu): the largest DFA whose inputs are chunked (2-byte
# table entries), and the shortest DFA chunk: at least DFA_CHUNK_MIN bytes and
# DFA_CHUNK_PER_STATE bytes per state. A random DFA's set of all states collapses after
# about 2n bytes, with a tail of about e^(-t/n) beyond; at 8n a chunk rarely ends before
# it collapses (at 2n about half do, and their fix-up turns serial). The planner
# lengthens the chunks of a batch with many long DFA inputs to one wave of the chunk
# launch.
DFA_CHUNK_MAX_STATES = 32768
DFA_CHUNK_MIN = 16 << 10
DFA_CHUNK_FLOOR = 4096  # the shortest DFA chunk a caller may ask for
DFA_CHUNK_PER_STATE = 8
# the most a DFA chunk's exact walk continues into the next chunk, as a share of the
# shortest chunk; 1 or more: no limit but the next chunk's end (the walk stops at that
# chunk's collapse, or covers it whole when it never collapses)
DFA_OVERLAP_CHUNKS = 1.0
# a host batch the device gathers in place (staging.py) of at least PIPELINE_MIN_BYTES is
# gathered in PIPELINE_PARTS slices of contiguous inputs, each slice's lane tasks starting
# as soon as its bytes are in (run_requests); PIPELINE_LANE_WAVES as in GraphRunner.
# Measured per run_batch call on c3-sustained inputs, whole gather / 8 slices: 8 MB 0.75 /
# 0.90 ms, 32 MB 1.12 / 1.17, 129 MB 2.48 / 2.57, 261 MB 4.47 / 4.23 (the shorter chunks
# of two lane waves and the extra launches outweigh the overlap below about 160 MiB)
PIPELINE_PARTS = 8
PIPELINE_MIN_BYTES = 160 << 20
PIPELINE_LANE_WAVES = 2


def dfa_chunk_length(num_states: int) -> int:
    """Shortest chunk for the long inputs of a DFA of ``num_states`` states (a multiple of
    64 bytes); an input is chunked when it holds two chunks."""
    return -(-max(DFA_CHUNK_MIN, DFA_CHUNK_PER_STATE * int(num_states)) // 64) * 64


def dfa_overlap_bytes(chunk_length: int) -> int:
    """Most bytes a DFA chunk's exact walk continues into the next chunk."""
    if DFA_OVERLAP_CHUNKS >= 1.0:
        return 1 << 30
    return int(DFA_OVERLAP_CHUNKS * int(chunk_length))


@dataclass
class NfaChoice:
    """Per-automaton technique inside a persistent launch."""

    technique: int = native.TECH_COMPACT  # TECH_COMPACT or TECH_WARP
    list_capacity: int = 128
    speculate: bool = True                # allow chunked speculation for long inputs
    lanes: bool = True                    # allow one-lane-per-chunk speculation


@dataclass
class TaskPlan:
    """Host-side task queue of one batch."""

    tasks_a: np.ndarray    # int32 [na, 4]: WHOLE and CHUNK tasks (persistent launch)
    tasks_b: np.ndarray    # int32 [nb, 4]: FIXUP tasks (last launch)
    input_ids: np.ndarray  # int32 [n]
    chunks: np.ndarray     # CHUNK_DTYPE [nc] (lane chunks first)
    chunk_bytes: int       # chunk size of warp-simulated chunks (0: none)
    lane_chunks: int = 0   # chunks run one per lane (the first lane_chunks of `chunks`)
    lane_chunk_bytes: int = 0
    tasks_l: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))
    # int32 [nl, 4]: LANES tasks (lane launch, before the persistent one)


class DeviceTasks:
    """Pinned + device buffers for task plans, grown on demand and reused."""

    def __init__(self, device) -> None:
        self.device = device
        self.cap_t = self.cap_i = self.cap_c = 0
        self.nl = self.na = self.nb = self.nc = 0
        self.n_lane_chunks = 0

    def chunk_io(self, overflow_count: bool = False) -> native.ChunkIO:
        io = native.ChunkIO()
        if self.nc:
            io.chunks = self.d_chunks.data_ptr()
            io.records = self.d_records.data_ptr()
            io.overflow_tasks = self.d_overflow.data_ptr()
            io.overflow_count = self.d_overflow_count.data_ptr()
            io.n_chunks = self.nc
            if overflow_count:
                io.task_count = self.d_overflow_count.data_ptr()
        return io

    def _ensure(self, n_tasks: int, n_ids: int, n_chunks: int) -> None:
        dev = self.device
        if n_tasks > self.cap_t:
            self.cap_t = max(n_tasks, 2 * self.cap_t, 256)
            self.h_tasks = torch.empty(self.cap_t * 4, dtype=torch.int32, pin_memory=True)
            self.d_tasks = torch.empty(self.cap_t * 4, dtype=torch.int32, device=dev)
        if n_ids > self.cap_i:
            self.cap_i = max(n_ids, 2 * self.cap_i, 256)
            self.h_ids = torch.empty(self.cap_i, dtype=torch.int32, pin_memory=True)
            self.d_ids = torch.empty(self.cap_i, dtype=torch.int32, device=dev)
        if n_chunks > self.cap_c:
            self.cap_c = max(n_chunks, 2 * self.cap_c, 64)
            self.h_chunks = torch.empty(self.cap_c * 24, dtype=torch.uint8, pin_memory=True)
            self.d_chunks = torch.empty(self.cap_c * 24, dtype=torch.uint8, device=dev)
            self.d_records = torch.empty(self.cap_c * native.CHUNK_RECORD_BYTES,
                                         dtype=torch.uint8, device=dev)
            self.d_overflow = torch.empty(self.cap_c * 4, dtype=torch.int32, device=dev)
            self.d_overflow_count = torch.zeros(4, dtype=torch.int32, device=dev)

    def upload(self, plan: TaskPlan, stream) -> None:
        """Copy a plan into the pinned buffers and enqueue its host->device copies. The
        task buffer holds the LANES, persistent and FIXUP tasks back to back."""
        nl, na, nb = plan.tasks_l.shape[0], plan.tasks_a.shape[0], plan.tasks_b.shape[0]
        nc = plan.chunks.shape[0]
        self._ensure(nl + na + nb + 1, plan.input_ids.size + 1, nc + 1)
        h = self.h_tasks.numpy()
        if nl:
            h[: nl * 4] = plan.tasks_l.reshape(-1)
        if na:
            h[nl * 4:(nl + na) * 4] = plan.tasks_a.reshape(-1)
        if nb:
            h[(nl + na) * 4:(nl + na + nb) * 4] = plan.tasks_b.reshape(-1)
        self.h_ids.numpy()[: plan.input_ids.size] = plan.input_ids
        if nc:
            self.h_chunks.numpy()[: nc * 24] = plan.chunks.view(np.uint8)
        with torch.cuda.stream(stream):
            nt = max(1, nl + na + nb) * 4
            self.d_tasks[:nt].copy_(self.h_tasks[:nt], non_blocking=True)
            ni = max(1, plan.input_ids.size)
            self.d_ids[:ni].copy_(self.h_ids[:ni], non_blocking=True)
            if nc:
                self.d_chunks[: nc * 24].copy_(self.h_chunks[: nc * 24], non_blocking=True)
        self.nl, self.na, self.nb, self.nc = nl, na, nb, nc
        self.n_lane_chunks = int(plan.lane_chunks)


class DevicePlan:
    """Buffers of a batch planned on the device (gbfsm_batch_plan) and its launches.

    Sized for up to ``n_inputs`` inputs of ``total_bytes`` in all. ``plan`` enqueues the
    two planning launches; ``launch`` then enqueues the lane launch, the persistent
    launch, the overflow pass and the fix-up, each reading its task count from the plan
    header on the device -- no host work depends on the batch's lengths, so the whole
    step (planning included) can be captured once and replayed for new inputs of the
    same sizes. ``slices`` (input indices where slices start, plus ``n_inputs``) gives
    each slice's lane tasks their own range in the header, for pipelined ingest.
    ``lane_waves``: how many waves of the lane launch the lane chunks fill (1: one chunk
    per resident lane; more: shorter chunks that the slices of a pipelined step hand to
    whichever lanes are free as their bytes arrive).
    """

    def __init__(self, engine: PersistentEngine, n_inputs: int, total_bytes: int,
                 slices=None, shrink: float = 0.0, lane_waves: int = 1) -> None:
        self.engine = engine
        dev = engine.device
        self.n = int(n_inputs)
        self.total_bytes = int(total_bytes)
        self.slices = list(slices) if slices is not None and len(slices) > 2 else None
        if self.slices is not None and len(self.slices) - 1 > native.PLAN_MAX_SLICES:
            raise ValueError(f"at most {native.PLAN_MAX_SLICES} slices")
        self.shrink = float(shrink) if self.slices else 0.0
        self.lane_waves = max(1, int(lane_waves))
        lw = engine.sm_count * engine.lane_warps_per_sm * self.lane_waves
        pw = engine.resident_warps
        fixed = engine.fixed_chunk
        n = max(self.n, 1)
        if fixed > 0:
            cap = int(total_bytes) // max(1, fixed // 2) + 2 * n + 64
        else:
            # lane chunks fill at most one wave (32 per resident warp) unless even 1 MiB
            # chunks do not; slices scale lane chunks down by up to 1 - shrink; warp
            # chunks number fewer than 8 per resident persistent warp plus one per input
            factor = 1.25 / (1.0 - max(self.shrink, 0.0))
            cap = int(factor * (LANE_GROUP * lw + int(total_bytes) // (1 << 20) + n)) + \
                8 * pw + 2 * n + 64
        self.cap_dfa_chunks, self.cap_dfa_fixup = self.dfa_caps(engine, n, total_bytes)
        self.cap_lanes = cap // LANE_GROUP + 2
        self.cap_persist = n + cap
        self.cap_fixup = n
        cap += self.cap_dfa_chunks
        self.cap_chunks = cap
        i32 = torch.int32
        self.chunks = torch.empty(cap * 24, dtype=torch.uint8, device=dev)
        self.records = torch.empty(cap * native.CHUNK_RECORD_BYTES, dtype=torch.uint8, device=dev)
        self.overflow = torch.empty(cap * 4, dtype=i32, device=dev)
        self.tasks = torch.empty((self.cap_lanes + self.cap_persist + self.cap_fixup +
                                  self.cap_dfa_chunks + self.cap_dfa_fixup) * 4,
                                 dtype=i32, device=dev)
        self.input_ids = torch.empty(n, dtype=i32, device=dev)
        # per input: the lowest chunk index that found an accept (chunked DFA inputs)
        self.dfa_latch = torch.empty(n if self.cap_dfa_chunks else 1, dtype=i32, device=dev)
        self.header = torch.zeros(native.PLAN_HEADER_WORDS, dtype=i32, device=dev)
        self.h_header = torch.zeros(native.PLAN_HEADER_WORDS, dtype=i32, pin_memory=True)
        lib = native.lib()
        self.scratch = torch.empty(max(16, int(lib.gbfsm_batch_plan_scratch_bytes(n))),
                                   dtype=torch.uint8, device=dev)
        base = self.tasks.data_ptr()
        self.tasks_lanes = base
        self.tasks_persist = base + self.cap_lanes * 16
        self.tasks_fixup = base + (self.cap_lanes + self.cap_persist) * 16
        self.tasks_dfa_chunk = self.tasks_fixup + self.cap_fixup * 16
        self.tasks_dfa_fixup = self.tasks_dfa_chunk + self.cap_dfa_chunks * 16

    @staticmethod
    def dfa_caps(engine: PersistentEngine, n: int, total_bytes: int) -> tuple[int, int]:
        """Capacities for DFA chunks and DFA fix-ups: an input is chunked when it holds
        at least two chunks of its DFA, so it has at most 1.5 x its bytes / chunk chunks."""
        if engine.aut_dfa_chunk is None:
            return 0, 0
        c = engine.min_dfa_chunk
        return (3 * int(total_bytes) // (2 * c) + 2,
                min(int(n), int(total_bytes) // (2 * c)) + 1)

    @staticmethod
    def device_bytes(engine: PersistentEngine, n_inputs: int, total_bytes: int) -> int:
        """Device memory a plan of this size takes (chunk table, records, task queues)."""
        lw = engine.sm_count * engine.lane_warps_per_sm
        n = max(int(n_inputs), 1)
        cap = int(1.25 * (LANE_GROUP * lw + int(total_bytes) // (1 << 20) + n)) + \
            8 * engine.resident_warps + 2 * n + 64
        dc, df = DevicePlan.dfa_caps(engine, n, total_bytes)
        return (cap + dc) * (24 + native.CHUNK_RECORD_BYTES + 16 + 16) + (dc + df) * 16 + \
            n * (68 if dc else 64)

    def _hdr(self, word: int) -> int:
        return self.header.data_ptr() + 4 * word

    def plan(self, d_off, d_ends, d_aut, stream, n_inputs: int | None = None,
             slices=None) -> None:
        """Enqueue planning for the inputs at ``d_off`` (``d_ends``, ``d_aut``: device
        tensors or None). ``slices``: this batch's slice starts (plus ``n_inputs``), in
        place of the ones the plan was built with."""
        eng = self.engine
        n = self.n if n_inputs is None else int(n_inputs)
        if n > self.n:
            raise ValueError(f"{n} inputs above the plan's capacity of {self.n}")
        if slices is not None:
            slices = list(slices)
            if not 2 < len(slices) <= native.PLAN_MAX_SLICES + 1:
                raise ValueError(f"2 to {native.PLAN_MAX_SLICES} slices")
            self.slices = slices
        a = native.BatchPlanArgs()
        a.n_inputs = n
        a.n_automata = len(eng.automata)
        a.offsets = d_off.data_ptr()
        a.ends = d_ends.data_ptr() if d_ends is not None else None
        a.aut_ids = d_aut.data_ptr() if d_aut is not None else None
        a.aut_class = eng.aut_class.data_ptr()
        if eng.aut_dfa_chunk is not None:
            a.aut_dfa_chunk = eng.aut_dfa_chunk.data_ptr()
            a.tasks_dfa_chunk = self.tasks_dfa_chunk
            a.tasks_dfa_fixup = self.tasks_dfa_fixup
            a.dfa_latch = self.dfa_latch.data_ptr()
        a.cap_dfa_chunk_tasks = self.cap_dfa_chunks
        a.cap_dfa_fixup_tasks = self.cap_dfa_fixup
        a.lane_warps = eng.sm_count * eng.lane_warps_per_sm * self.lane_waves
        a.persist_warps = eng.resident_warps
        a.dfa_warps = eng.dfa_warps
        a.min_chunk = eng.min_chunk
        a.fixed_chunk = eng.fixed_chunk
        if self.slices:
            a.n_slices = len(self.slices) - 1
            a.shrink = self.shrink
            for k, v in enumerate(self.slices):
                a.slice_first[k] = int(v)
        a.cap_chunks = self.cap_chunks
        a.cap_lane_tasks = self.cap_lanes
        a.cap_persist_tasks = self.cap_persist
        a.cap_fixup_tasks = self.cap_fixup
        a.chunks = self.chunks.data_ptr()
        a.tasks_lanes = self.tasks_lanes
        a.tasks_persist = self.tasks_persist
        a.tasks_fixup = self.tasks_fixup
        a.input_ids = self.input_ids.data_ptr()
        a.header = self.header.data_ptr()
        a.scratch = self.scratch.data_ptr()
        self._d_aut = d_aut
        native.check(native.lib().gbfsm_batch_plan(ctypes.byref(a), stream.cuda_stream),
                     "gbfsm_batch_plan")

    def chunk_io(self, task_count_word: int | None) -> native.ChunkIO:
        io = native.ChunkIO()
        io.chunks = self.chunks.data_ptr()
        io.records = self.records.data_ptr()
        io.overflow_tasks = self.overflow.data_ptr()
        io.overflow_count = self._hdr(native.PLAN_OVERFLOW)
        io.n_chunks = self.cap_chunks
        io.aut_ids = self._d_aut.data_ptr() if self._d_aut is not None else None
        if task_count_word is not None:
            io.task_count = self._hdr(task_count_word)
        return io

    def launch(self, data_ptr: int, d_off, d_ends, d_flags, d_lens, d_examined, stream,
               workspace=None, phases: dict | None = None, lane_slices=None) -> int:
        """Enqueue the launches of a planned batch (four, six when the pool chunks long DFA
        inputs); returns their number.
        ``lane_slices``: ``[(side stream, ready event)]`` per slice (pipelined ingest);
        slice k's lane tasks run on its side stream once its event has fired."""
        eng = self.engine
        lib = native.lib()

        def mark(name):
            if phases is not None:
                e = torch.cuda.Event(enable_timing=True)
                e.record(stream)
                phases.setdefault(name, []).append(e)

        ws = eng.workspace if workspace is None else workspace
        table, n_aut = eng.table.data_ptr(), len(eng.automata)
        io = self.chunk_io(None)
        launches = 0
        if lane_slices:
            fork = torch.cuda.Event()
            fork.record(stream)
            joins = []
            for k, (side, ready) in enumerate(lane_slices):
                side.wait_event(fork)
                side.wait_event(ready)
                st = lib.gbfsm_lanes_run_range(table, n_aut, self.tasks_lanes, self.cap_lanes,
                                               self._hdr(native.PLAN_SLICES + 2 * k), data_ptr,
                                               d_off.data_ptr(), ctypes.byref(io),
                                               side.cuda_stream)
                native.check(st, "gbfsm_lanes_run_range")
                done = torch.cuda.Event()
                done.record(side)
                joins.append(done)
                launches += 1
            for done in joins:
                stream.wait_event(done)
            for _, ready in lane_slices:
                stream.wait_event(ready)
        else:
            mark("lanes")
            st = lib.gbfsm_lanes_run_range(table, n_aut, self.tasks_lanes, self.cap_lanes,
                                           self._hdr(native.PLAN_LANE_FIRST), data_ptr,
                                           d_off.data_ptr(), ctypes.byref(io), stream.cuda_stream)
            native.check(st, "gbfsm_lanes_run_range")
            mark("lanes")
            launches += 1

        def dfa_chunks(name, tasks_ptr, max_tasks, count_word):
            mark(name)
            st = lib.gbfsm_dfa_chunks_run(
                table, n_aut, tasks_ptr, int(max_tasks), self._hdr(count_word), data_ptr,
                d_off.data_ptr(), d_ends.data_ptr() if d_ends is not None else None,
                ctypes.byref(io), eng.dfa_max_states, d_flags.data_ptr(), d_lens.data_ptr(),
                d_examined.data_ptr() if d_examined is not None else None,
                self.dfa_latch.data_ptr(), stream.cuda_stream)
            native.check(st, "gbfsm_dfa_chunks_run")
            mark(name)

        chunked_dfa = eng.aut_dfa_chunk is not None and self.cap_dfa_chunks > 0
        if chunked_dfa:
            dfa_chunks("dfa_chunks", self.tasks_dfa_chunk, self.cap_dfa_chunks,
                       native.PLAN_DFA_CHUNKS)
            launches += 1

        def persist(name, tasks_ptr, max_tasks, count_word):
            mark(name)
            cio = self.chunk_io(count_word)
            st = lib.gbfsm_persistent_run(
                table, n_aut, eng.max_words, tasks_ptr, int(max_tasks),
                self.input_ids.data_ptr(), data_ptr, d_off.data_ptr(),
                d_ends.data_ptr() if d_ends is not None else None, ctypes.byref(cio),
                d_flags.data_ptr(), d_lens.data_ptr(),
                d_examined.data_ptr() if d_examined is not None else None,
                ws.data_ptr(), eng.ws_bytes, ctypes.byref(eng.plan), stream.cuda_stream)
            native.check(st, "gbfsm_persistent_run")
            mark(name)

        persist("persistent", self.tasks_persist, self.cap_persist, native.PLAN_PERSIST_TASKS)
        persist("overflow", self.overflow.data_ptr(), self.cap_chunks, native.PLAN_OVERFLOW)
        persist("fixup", self.tasks_fixup, self.cap_fixup, native.PLAN_FIXUP_TASKS)
        if chunked_dfa:
            dfa_chunks("dfa_fixup", self.tasks_dfa_fixup, self.cap_dfa_fixup,
                       native.PLAN_DFA_FIXUPS)
            launches += 1
        return launches + 3

    def fetch_header(self, stream) -> None:
        """Enqueue the header's copy to pinned host memory (read it after the stream)."""
        with torch.cuda.stream(stream):
            self.h_header.copy_(self.header, non_blocking=True)

    def check(self) -> None:
        """Raise if the last plan (its header fetched and the stream finished) failed."""
        st = int(self.h_header[native.PLAN_STATUS])
        if st == 1:
            raise RuntimeError("device plan: a plan buffer was too small for this batch")
        if st == 2:
            raise ValueError("device plan: a request names an automaton outside the pool")


class PersistentEngine:
    """A resident automaton pool plus the persistent launch over it."""

    def __init__(self, automata, device=None, choices=None, block_threads: int = 256,
                 list_capacity: int | None = None, ctas_per_sm: int = 0,
                 chunk_bytes: int | None = 0, lane_pair_mean: float = LANE_PAIR_MEAN,
                 resident=None, dfa_chunk_bytes: int | None = None) -> None:
        """``chunk_bytes``: 0 = chosen per batch, None = never chunk, else a fixed size.
        ``dfa_chunk_bytes``: chunk length of long DFA inputs; None = from each DFA's size
        (dfa_chunk_length()), 0 = DFA inputs always run whole, else this length (rounded up
        to 64 bytes, at least DFA_CHUNK_FLOOR) for every DFA.
        ``lane_pair_mean``: largest mean two-byte superset for one-lane-per-chunk tasks.
        ``resident``: device layouts already built for ``automata`` (DeviceNFA /
        DeviceDFA, same order), shared instead of built again."""
        self.device = resolve_device(device)
        self.automata = list(automata)
        if not self.automata:
            raise ValueError("the engine needs at least one automaton")
        self.kinds = [Kind.of(a) for a in self.automata]
        if resident is not None:
            self.dev = list(resident)
            if len(self.dev) != len(self.automata):
                raise ValueError("one resident layout per automaton is needed")
        else:
            self.dev = [DeviceNFA(a, self.device) if k is Kind.NFA else DeviceDFA(a, self.device)
                        for a, k in zip(self.automata, self.kinds)]
        choices = list(choices) if choices is not None else [NfaChoice() for _ in self.automata]
        self.choices = choices
        self.chunk_bytes = chunk_bytes
        self.can_chunk = np.array([k is Kind.NFA and d.speculative and c.speculate
                                   for k, d, c in zip(self.kinds, self.dev, choices)], dtype=bool)
        self.lane_ok = np.array([bool(self.can_chunk[i]) and c.lanes and d.lanes and
                                 d.pair_mean <= lane_pair_mean
                                 for i, (d, c) in enumerate(zip(self.dev, choices))], dtype=bool)
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
            # long DFA inputs are cut into chunks walked in parallel (DFA_CHUNK tasks): a
            # chunk of an n-state DFA spans at least max(16 KiB, 8n) bytes, and its exact
            # walk continues into the next chunk until it passes that chunk's collapse
            # (about 2n bytes in for a random DFA), or over all of it when it never
            # collapses
            dfa_chunk = [0] * len(self.automata)
            if chunk_bytes is not None and dfa_chunk_bytes != 0:
                for i, (d, k) in enumerate(zip(self.dev, self.kinds)):
                    if k is Kind.DFA and d.entry_bytes == 2 and \
                            d.num_states <= DFA_CHUNK_MAX_STATES:
                        dfa_chunk[i] = (dfa_chunk_length(d.num_states) if dfa_chunk_bytes is None
                                        else -(-max(DFA_CHUNK_FLOOR, int(dfa_chunk_bytes))
                                               // 64) * 64)
            self.dfa_chunk = dfa_chunk
            self.dfa_max_states = max([d.num_states for d, c in zip(self.dev, dfa_chunk) if c]
                                      or [0])
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
                    table[i].dfa_overlap = dfa_overlap_bytes(dfa_chunk[i])
            raw = np.frombuffer(bytes(table), dtype=np.uint8).copy()
            self.table = torch.from_numpy(raw).to(self.device)
            props = torch.cuda.get_device_properties(self.device)
        self.sm_count = props.multi_processor_count
        with torch.cuda.device(self.device):
            self.lane_warps_per_sm = int(lib.gbfsm_lanes_warps_per_sm()) or LANE_WARPS_PER_SM
        self.resident_warps = self.sm_count * self.ctas_per_sm * (block_threads // 32)
        self._staging = Staging(self.device)
        self._results = Results(self.device)
        self._tasks = DeviceTasks(self.device)
        # planning classes of the automata (gbfsm_batch_plan) and the chunk-size rule
        cls = []
        for i, k in enumerate(self.kinds):
            if k is Kind.DFA:
                cls.append(native.PLAN_DFA)
            elif self.lane_ok[i]:
                cls.append(native.PLAN_NFA_LANES)
            elif self.can_chunk[i]:
                cls.append(native.PLAN_NFA_WARP)
            else:
                cls.append(native.PLAN_NFA_WHOLE)
        self.aut_class = torch.tensor(cls, dtype=torch.int32, device=self.device)
        nfa_ix = [i for i, k in enumerate(self.kinds) if k is Kind.NFA]
        small_starts = bool(nfa_ix) and all(
            bool(self.lane_ok[i]) and self.dev[i].pair_mean <= 1.0 for i in nfa_ix)
        self.min_chunk = MIN_CHUNK_SMALL_STARTS if small_starts else MIN_CHUNK
        self.aut_dfa_chunk = (torch.tensor(self.dfa_chunk, dtype=torch.int32, device=self.device)
                              if any(self.dfa_chunk) else None)
        self.min_dfa_chunk = min([c for c in self.dfa_chunk if c] or [0])
        # chunk lengths follow the batch (one wave of the chunk launch) unless fixed
        self.dfa_warps = 0
        if self.aut_dfa_chunk is not None and dfa_chunk_bytes is None:
            with torch.cuda.device(self.device):
                self.dfa_warps = self.sm_count * int(
                    lib.gbfsm_dfa_chunks_warps_per_sm(max(1, self.dfa_max_states)))
        self.fixed_chunk = -1 if chunk_bytes is None else max(0, int(chunk_bytes))
        if self.fixed_chunk > 0:
            self.fixed_chunk = max(self.fixed_chunk, self.min_chunk)
        self._dplan: DevicePlan | None = None
        self._pplan: DevicePlan | None = None  # pipelined host batches (run_requests)
        self._copy_stream = None
        self._slice_streams: list = []
        self.pipeline_parts = PIPELINE_PARTS  # 0 or 1: gather a host batch whole first
        self.last_slices = 0  # slices of the last run_requests batch (0: not pipelined)
        self._h_aut = self._d_aut = None

    # ---- task queue ---------------------------------------------------------------------

    def auto_chunk_bytes(self, nfa_bytes: int) -> int:
        """Warp chunks: about four per resident warp of the persistent launch (a power of
        two in [the shortest chunk, 1 MiB])."""
        per = nfa_bytes // max(1, 4 * self.resident_warps)
        size = max(getattr(self, "min_chunk", MIN_CHUNK),
                   1 << max(0, int(per).bit_length() - 1))
        return int(min(size, 1 << 20))

    def auto_lane_chunk_bytes(self, lengths: np.ndarray, aut: np.ndarray) -> int:
        """Lane chunks: the smallest size (a multiple of 64 bytes, at least the shortest
        chunk)
        whose LANES tasks (32 chunks each, per automaton) fit the lane launch's resident
        warps, so the batch runs in one full wave. A lane's steps are dependent L2 round
        trips: once every lane is busy, finer chunks only add per-chunk work, and a second
        partial wave adds its whole duration."""
        warps = self.sm_count * getattr(self, "lane_warps_per_sm", LANE_WARPS_PER_SM)
        floor = getattr(self, "min_chunk", MIN_CHUNK)
        lengths = np.asarray(lengths, dtype=np.int64)
        aut = np.asarray(aut, dtype=np.int64)
        if lengths.size == 0:
            return floor
        total = int(lengths.sum())
        size = max(floor, -(-total // (warps * LANE_GROUP) // 64) * 64)
        order = np.argsort(aut, kind="stable")
        a_sorted, l_sorted = aut[order], lengths[order]
        seg = np.flatnonzero(np.r_[True, a_sorted[1:] != a_sorted[:-1]])
        while size < (1 << 20):
            chunks = np.maximum(1, -(-l_sorted // size))
            per_aut = np.add.reduceat(chunks, seg) if seg.size else np.zeros(0, np.int64)
            if int((-(-per_aut // LANE_GROUP)).sum()) <= warps:
                break
            size += 64
        return int(min(size, 1 << 20))

    def make_tasks(self, aut_ids, lengths, starts=None, lane_chunk=None,
                   warp_chunk: int | None = None) -> TaskPlan:
        """Task plan for a batch: input i is ``lengths[i]`` bytes at ``starts[i]`` (default:
        packed back to back from 0) on automaton ``aut_ids[i]``. Chunk bounds are nominal:
        the kernels move each later chunk's start a few bytes forward to where the
        two-byte superset is small (chunk_bounds in csrc/chunks.cuh)."""
        aut_ids = np.asarray(aut_ids, dtype=np.int64)
        lengths = np.asarray(lengths, dtype=np.int64)
        n = aut_ids.size
        empty = np.zeros((0, 4), dtype=np.int32)
        no_chunks = np.zeros(0, dtype=native.CHUNK_DTYPE)
        if n == 0:
            return TaskPlan(empty, empty, np.zeros(1, np.int32), no_chunks, 0)
        if aut_ids.min() < 0 or aut_ids.max() >= len(self.automata):
            raise ValueError("request names an automaton outside the pool")
        if starts is None:
            starts = np.zeros(n, dtype=np.int64)
            np.cumsum(lengths[:-1], out=starts[1:])
        starts = np.asarray(starts, dtype=np.int64)
        is_dfa = np.array([k is Kind.DFA for k in self.kinds], dtype=bool)[aut_ids]
        nfa_idx = np.flatnonzero(~is_dfa)
        dfa_idx = np.flatnonzero(is_dfa)
        dfa_idx = dfa_idx[np.lexsort((-lengths[dfa_idx], aut_ids[dfa_idx]))]
        input_ids = np.concatenate([nfa_idx, dfa_idx]).astype(np.int32)
        rows = []
        # NFA inputs: whole, or chunked when long and the automaton allows speculation;
        # chunks of automata with small two-byte supersets run one per lane
        lane_in = self.lane_ok[aut_ids] & ~is_dfa
        warp_in = self.can_chunk[aut_ids] & ~lane_in & ~is_dfa
        csize = np.zeros(n, dtype=np.int64)
        chunk_w = chunk_l = 0
        if self.chunk_bytes is not None and nfa_idx.size:
            if self.chunk_bytes:
                chunk_w = chunk_l = max(int(self.chunk_bytes),
                                        getattr(self, "min_chunk", MIN_CHUNK))
            else:
                chunk_w = warp_chunk or self.auto_chunk_bytes(int(lengths[warp_in].sum()))
                if isinstance(lane_chunk, np.ndarray):
                    chunk_l = int(lane_chunk.max()) if lane_chunk.size else 0
                else:
                    chunk_l = lane_chunk or self.auto_lane_chunk_bytes(lengths[lane_in],
                                                                       aut_ids[lane_in])
            csize[warp_in] = chunk_w
            if isinstance(lane_chunk, np.ndarray) and not self.chunk_bytes:
                csize[lane_in] = np.maximum(np.asarray(lane_chunk, np.int64)[lane_in],
                                            getattr(self, "min_chunk", MIN_CHUNK))
            else:
                csize[lane_in] = chunk_l
        # every input of a lane automaton is chunked (a short one is a single exact
        # chunk); warp-chunked inputs are split when they span two chunks or more
        split = (csize > 0) & ((lengths >= 2 * np.maximum(csize, 1)) | lane_in)
        whole = nfa_idx[~split[nfa_idx]]
        pos_of = np.empty(n, dtype=np.int64)
        pos_of[nfa_idx] = np.arange(nfa_idx.size)
        rows.append(np.stack([aut_ids[whole], pos_of[whole], np.ones_like(whole),
                              np.full_like(whole, native.TASK_WHOLE),
                              lengths[whole] * NFA_BYTE_WEIGHT], axis=1))
        chunk_list, fix_rows, lane_rows = [], [], []
        n_lane = 0
        if split.any():
            # lane-chunked inputs first (grouped by automaton), then warp-chunked ones
            sl = np.flatnonzero(split & lane_in)
            sl = sl[np.argsort(aut_ids[sl], kind="stable")]
            sw = np.flatnonzero(split & ~lane_in)
            sidx = np.concatenate([sl, sw])
            cs = csize[sidx]
            # ceil(length / size) chunks of even length (each in (size/2, size])
            counts = np.maximum(1, -(-lengths[sidx] // cs))
            first = np.zeros(sidx.size, dtype=np.int64)
            np.cumsum(counts[:-1], out=first[1:])
            total = int(counts.sum())
            ch = np.zeros(total, dtype=native.CHUNK_DTYPE)
            inp = np.repeat(sidx, counts)
            idx = np.arange(total) - np.repeat(first, counts)
            cnt = np.repeat(counts, counts)
            ln = lengths[inp]
            ch["input"] = inp
            ch["index"] = idx
            ch["begin"] = starts[inp] + idx * ln // cnt
            ch["end"] = starts[inp] + (idx + 1) * ln // cnt
            n_lane = int(counts[:sl.size].sum())
            chunk_list.append(ch)
            clen = ch["end"] - ch["begin"]
            # LANES tasks: up to 32 consecutive lane chunks of one automaton
            if n_lane:
                la = aut_ids[inp[:n_lane]]
                seg = np.flatnonzero(np.r_[True, la[1:] != la[:-1]])
                seg_end = np.r_[seg[1:], n_lane]
                g0, gc = [], []
                for s0, e0 in zip(seg.tolist(), seg_end.tolist()):
                    for g in range(s0, e0, LANE_GROUP):
                        g0.append(g)
                        gc.append(min(LANE_GROUP, e0 - g))
                g0 = np.asarray(g0, dtype=np.int64)
                gc = np.asarray(gc, dtype=np.int64)
                lane_rows.append(np.stack([la[g0], g0, gc, np.full(g0.size, native.TASK_LANES)],
                                          axis=1))
            wc = np.arange(n_lane, total)
            if wc.size:
                rows.append(np.stack([aut_ids[inp[wc]], wc, np.ones(wc.size, np.int64),
                                      np.full(wc.size, native.TASK_CHUNK),
                                      clen[wc] * NFA_BYTE_WEIGHT], axis=1))
            fix_rows.append(np.stack([aut_ids[sidx], first, counts,
                                      np.full(sidx.size, native.TASK_FIXUP), counts], axis=1))
        if dfa_idx.size:
            sa = aut_ids[dfa_idx]
            seg_starts = np.flatnonzero(np.r_[True, sa[1:] != sa[:-1]])
            seg_ends = np.r_[seg_starts[1:], sa.size]
            firsts, cnts = [], []
            for s, e in zip(seg_starts.tolist(), seg_ends.tolist()):
                for gs in range(s, e, DFA_GROUP):
                    firsts.append(gs)
                    cnts.append(min(DFA_GROUP, e - gs))
            g = np.asarray(firsts, dtype=np.int64)
            rows.append(np.stack([sa[g], nfa_idx.size + g, np.asarray(cnts, dtype=np.int64),
                                  np.full(g.size, native.TASK_WHOLE), lengths[dfa_idx[g]]], axis=1))
        t = np.concatenate(rows)
        t = t[np.argsort(-t[:, 4], kind="stable")][:, :4]
        lanes = np.concatenate(lane_rows) if lane_rows else empty
        if fix_rows:
            f = np.concatenate(fix_rows)
            f = f[np.argsort(-f[:, 4], kind="stable")][:, :4]
        else:
            f = empty
        chunks = np.concatenate(chunk_list) if chunk_list else no_chunks
        return TaskPlan(np.ascontiguousarray(t, dtype=np.int32),
                        np.ascontiguousarray(f, dtype=np.int32), input_ids, chunks, chunk_w,
                        n_lane, chunk_l, np.ascontiguousarray(lanes, dtype=np.int32))

    # ---- launches -------------------------------------------------------------------------

    def new_workspace(self) -> torch.Tensor:
        """A separate workspace (queue ticket + dense scratch) for a concurrent launch."""
        return torch.zeros(self.ws_bytes, dtype=torch.uint8, device=self.device)

    def _run(self, tasks_ptr, n_tasks, dt: DeviceTasks, data_ptr, d_off, d_ends, d_flags, d_lens,
             d_examined, ws, stream, overflow_pass: bool = False) -> None:
        io = dt.chunk_io(overflow_pass)
        st = native.lib().gbfsm_persistent_run(
            self.table.data_ptr(), len(self.automata), self.max_words, tasks_ptr, int(n_tasks),
            dt.d_ids.data_ptr(), data_ptr, d_off.data_ptr(),
            d_ends.data_ptr() if d_ends is not None else None,
            ctypes.byref(io) if dt.nc else None,
            d_flags.data_ptr(), d_lens.data_ptr(),
            d_examined.data_ptr() if d_examined is not None else None,
            ws.data_ptr(), self.ws_bytes, ctypes.byref(self.plan), stream.cuda_stream)
        native.check(st, "gbfsm_persistent_run")

    def launch(self, d_data, d_off, dt: DeviceTasks, d_flags, d_lens, d_examined=None,
               stream=None, d_ends=None, workspace=None, phases: dict | None = None,
               lane_slices=None) -> int:
        """Enqueue the batch's launches; returns how many kernels were launched:
        the lane launch (LANES tasks), the persistent launch (WHOLE / CHUNK tasks), the
        overflow pass (lane chunks that outgrew their lane, run by warps) and the fix-up
        (FIXUP tasks), each only when it has work. ``d_data`` is a device tensor or a raw
        device address (e.g. of pinned host memory read in place); with ``d_ends`` input
        i spans ``[d_off[i], d_ends[i])``. ``phases`` (optional) collects a pair of timing
        events around each launch, keyed "lanes", "persistent", "overflow", "fixup".

        ``lane_slices`` (optional) splits the lane launch: a list of ``(first task, task
        count, side stream, event)``; each range of LANES tasks runs on its side stream
        once the event (e.g. "its input bytes have arrived") has fired, and the rest of
        the step waits for all of them, and for every event, on ``stream``."""
        stream = stream or torch.cuda.current_stream(self.device)

        def mark(name):
            if phases is None:
                return None
            e = torch.cuda.Event(enable_timing=True)
            e.record(stream)
            phases.setdefault(name, []).append(e)
            return e
        ws = self.workspace if workspace is None else workspace
        data_ptr = d_data if isinstance(d_data, int) else d_data.data_ptr()
        base = dt.d_tasks.data_ptr()
        launches = 0
        if dt.nl:
            with torch.cuda.stream(stream):
                dt.d_overflow_count.zero_()
            io = dt.chunk_io()
            lib = native.lib()
            if lane_slices:
                fork = torch.cuda.Event()
                fork.record(stream)
                joins = []
                for first, count, side, ready in lane_slices:
                    if count <= 0:
                        continue
                    side.wait_event(fork)
                    side.wait_event(ready)
                    st = lib.gbfsm_lanes_run(
                        self.table.data_ptr(), len(self.automata), base + int(first) * 16,
                        int(count), data_ptr, d_off.data_ptr(), ctypes.byref(io),
                        side.cuda_stream)
                    native.check(st, "gbfsm_lanes_run")
                    done = torch.cuda.Event()
                    done.record(side)
                    joins.append(done)
                    launches += 1
                for done in joins:
                    stream.wait_event(done)
                for _, _, _, ready in lane_slices:  # the launches below may read any slice
                    stream.wait_event(ready)
            else:
                mark("lanes")
                st = lib.gbfsm_lanes_run(
                    self.table.data_ptr(), len(self.automata), base, dt.nl, data_ptr,
                    d_off.data_ptr(), ctypes.byref(io), stream.cuda_stream)
                native.check(st, "gbfsm_lanes_run")
                mark("lanes")
                launches += 1
        if dt.na or not (dt.nl or dt.nb):
            mark("persistent")
            self._run(base + dt.nl * 16, dt.na, dt, data_ptr, d_off, d_ends, d_flags, d_lens,
                      d_examined, ws, stream)
            mark("persistent")
            launches += 1
        if dt.nl:
            mark("overflow")
            self._run(dt.d_overflow.data_ptr(), dt.n_lane_chunks, dt, data_ptr, d_off, d_ends,
                      d_flags, d_lens, d_examined, ws, stream, overflow_pass=True)
            mark("overflow")
            launches += 1
        if dt.nb:
            mark("fixup")
            self._run(base + (dt.nl + dt.na) * 16, dt.nb, dt, data_ptr, d_off, d_ends, d_flags,
                      d_lens, d_examined, ws, stream)
            mark("fixup")
            launches += 1
        return launches

    def device_plan(self, n_inputs: int, total_bytes: int, pipelined: bool = False) -> DevicePlan:
        """Plan buffers for a batch of this size (kept and reused while batches fit);
        ``pipelined``: the plan of sliced host batches (its slices given per batch)."""
        p = self._pplan if pipelined else self._dplan
        if p is None or p.n < n_inputs or p.total_bytes < total_bytes:
            n = max(int(n_inputs), 2 * (p.n if p else 0), 64)
            total = max(int(total_bytes), 2 * (p.total_bytes if p else 0), 1 << 20)
            if pipelined:
                self._pplan = None  # free the old buffers first
                p = DevicePlan(self, n, total, slices=[0, 1, 2], lane_waves=PIPELINE_LANE_WAVES)
                self._pplan = p
            else:
                self._dplan = None
                p = DevicePlan(self, n, total)
                self._dplan = p
        return p

    def _pipelined_launch(self, n: int, h_off: np.ndarray, total: int, d_data, d_off, d_aut,
                          res, with_examined: bool, stream) -> DevicePlan | None:
        """Gather a deferred host batch in slices on a copy stream, each slice's lane tasks
        on a stream of its own once its bytes are in, the rest of the step on ``stream``;
        None (nothing enqueued) when the batch makes fewer than two slices."""
        spans = slice_bounds(h_off, min(self.pipeline_parts, native.PLAN_MAX_SLICES))
        if len(spans) < 2:
            return None
        if self._copy_stream is None:
            self._copy_stream = torch.cuda.Stream(self.device)
            self._slice_streams = [torch.cuda.Stream(self.device)
                                   for _ in range(native.PLAN_MAX_SLICES)]
        plan = self.device_plan(n, total, pipelined=True)
        fork = torch.cuda.Event()
        fork.record(stream)
        self._copy_stream.wait_event(fork)
        ready = []
        for a, b in spans:
            self._staging.gather_range(a, b, self._copy_stream)
            ev = torch.cuda.Event()
            ev.record(self._copy_stream)
            ready.append(ev)
        plan.plan(d_off, None, d_aut, stream, n, slices=[a for a, _ in spans] + [n])
        plan.launch(d_data.data_ptr(), d_off, None, res.d[0], res.d[1],
                    res.d[2] if with_examined else None, stream,
                    lane_slices=list(zip(self._slice_streams, ready)))
        self.last_slices = len(spans)
        return plan

    def upload_aut_ids(self, aut_ids, stream):
        """Device int32 copy of the batch's automaton ids (None for a one-automaton pool,
        whose requests all name automaton 0)."""
        aut = np.asarray(aut_ids, dtype=np.int64)
        if aut.size and (aut.min() < 0 or aut.max() >= len(self.automata)):
            raise ValueError("request names an automaton outside the pool")
        if len(self.automata) == 1:
            return None
        n = max(int(aut.size), 1)
        if self._h_aut is None or self._h_aut.numel() < n:
            cap = max(n, 2 * (self._h_aut.numel() if self._h_aut is not None else 0), 256)
            self._h_aut = torch.empty(cap, dtype=torch.int32, pin_memory=True)
            self._d_aut = torch.empty(cap, dtype=torch.int32, device=self.device)
        self._h_aut.numpy()[: aut.size] = aut
        with torch.cuda.stream(stream):
            self._d_aut[:n].copy_(self._h_aut[:n], non_blocking=True)
        return self._d_aut

    def run_requests(self, aut_ids, inputs, with_examined: bool = False, lengths=None,
                     idle=None):
        """Host path: ``inputs[i]`` runs on automaton ``aut_ids[i]``; the batch is planned
        on the device.

        Returns ``(flags, lens, examined | None, kernel_ms, transfer_ms)`` as numpy arrays
        indexed like ``inputs``; ``kernel_ms`` covers the planning and simulation launches
        (and, for a batch the device gathers in slices, the gather they overlap).
        A batch the device gathers in place, of at least PIPELINE_MIN_BYTES, is gathered
        in ``pipeline_parts`` slices, each slice's lane tasks running as its bytes arrive.
        ``lengths``: the inputs' lengths (int64), when the caller has them already.
        ``idle``: called once every launch is enqueued, before the host waits for them.
        """
        t0 = time.perf_counter()
        n = len(inputs)
        stream = torch.cuda.current_stream(self.device)
        d_aut = self.upload_aut_ids(aut_ids, stream)
        d_data, d_off, h_off, total = self._staging.put(inputs, stream,
                                                        defer=self.pipeline_parts > 1,
                                                        lengths=lengths)
        self._results.ensure(max(n, 1))
        res = self._results
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        sliced = self._staging.deferred and n > 1 and total >= PIPELINE_MIN_BYTES
        if self._staging.deferred and not sliced:
            self._staging.gather_range(0, n, stream)  # ingest, outside kernel_ms
        e0.record(stream)
        plan = None
        self.last_slices = 0
        if sliced:
            plan = self._pipelined_launch(n, h_off, total, d_data, d_off, d_aut, res,
                                          with_examined, stream)
            if plan is None:  # a single slice: the batch is gathered whole
                self._staging.gather_range(0, n, stream)
        if plan is None and n:
            plan = self.device_plan(n, total)
            plan.plan(d_off, None, d_aut, stream, n)
            plan.launch(d_data.data_ptr(), d_off, None, res.d[0], res.d[1],
                        res.d[2] if with_examined else None, stream)
        e1.record(stream)
        res.fetch(n, stream)
        if n:
            plan.fetch_header(stream)
        if idle is not None:
            idle()
        stream.synchronize()
        if n:
            plan.check()
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
        out: list = []
        flags, lens, _, kms, tms = self.run_requests(
            aut, data, idle=lambda: out.extend(blank_results(len(data))))
        return fill_results(out, flags, lens, kms, tms)


def slice_bounds(offsets: np.ndarray, parts: int) -> list[tuple[int, int]]:
    """Contiguous input ranges [a, b) covering every input, cut where the cumulative bytes
    cross multiples of total / parts (empty ranges dropped)."""
    offsets = np.asarray(offsets, dtype=np.int64)
    n = offsets.size - 1
    total = int(offsets[-1])
    cut = np.searchsorted(offsets[1:], total * np.arange(1, parts) / parts) + 1
    bounds = np.unique(np.concatenate([[0], np.minimum(cut, n), [n]]))
    return [(int(a), int(b)) for a, b in zip(bounds[:-1], bounds[1:]) if b > a]


class GraphRunner:
    """A batch captured as one CUDA graph: H2D inputs, planning, the launches, D2H verdicts.

    The batch (flat uint8 data + int64 offsets + automaton ids) is staged at construction;
    ``replay`` re-runs it end to end, planning included (gbfsm_batch_plan), so the same
    graph also serves any new batch of the same sizes written into ``h_data`` / ``h_off``.
    """

    INGEST = ("copy", "zero_copy", "pipelined")

    def __init__(self, engine: PersistentEngine, aut_ids, data: np.ndarray, offsets: np.ndarray,
                 with_examined: bool = False, ingest: str = "copy", parts: int = 8,
                 shrink: float = 0.0, lane_waves: int = 2) -> None:
        """``ingest`` says how each replay moves the inputs from the pinned host buffer:

        * ``copy``: one copy-engine transfer, then planning and the launches;
        * ``zero_copy``: no copy, the simulation kernels read the bytes in place over the
          host link (NVLink-C2C on GB300);
        * ``pipelined``: the inputs are copied in ``parts`` slices of contiguous inputs
          with about equal bytes. The lane tasks of each slice run on a stream of their
          own as soon as the slice's bytes have arrived, concurrently with the copies of
          later slices; the overflow pass and the fix-up then run once for the whole
          batch. Inputs of slice k of P get the whole batch's lane chunk size scaled by
          1 - shrink * k / P: a slice that arrives later has less time left, so its lanes
          get shorter chunks. ``lane_waves`` > 1 cuts the lane chunks shorter, to fill
          that many waves of the lane launch, so that each arriving slice finds free lanes.
          Measured on c3-sustained (2.76 ms per step): 8 slices, no shrink, 2 waves; one
          wave with shrink 0.75 took 2.81 ms, 4 waves 2.87 ms (per-chunk work grows: the
          resident step takes 1.92 / 2.22 / 2.61 ms at 1 / 2 / 4 waves).

        ``kernel_only`` plans and runs the batch on the device copy of the inputs."""
        if ingest not in self.INGEST:
            raise ValueError(f"ingest must be one of {self.INGEST}")
        self.engine = engine
        dev = engine.device
        n = len(offsets) - 1
        self.n = n
        offsets = np.asarray(offsets, dtype=np.int64)
        aut_ids = np.asarray(aut_ids, dtype=np.int64)
        total = int(offsets[-1])
        self.slices: list[tuple[int, int]] = []  # byte range [lo, hi) of each slice's copy
        slice_first = None
        if ingest == "pipelined" and n:
            spans = slice_bounds(offsets, parts)
            slice_first = [a for a, _ in spans] + [n]
            total_b = max(16, -(-total // 16) * 16)
            # slice k ends at the 16-byte block holding its last input's end and the next
            # slice starts there, so no block is copied twice (a block shared by two inputs
            # arrives with the earlier slice, which the later slice's copy follows)
            lo = 0
            for a, b in spans:
                hi = min(total_b, -(-int(offsets[b]) // 16) * 16)
                self.slices.append((lo, hi))
                lo = hi
        self.plan = DevicePlan(engine, max(n, 1), total, slices=slice_first, shrink=shrink,
                               lane_waves=lane_waves if slice_first else 1)
        # the resident copy for kernel_only (no slices: every lane task in one range)
        self.kplan = DevicePlan(engine, max(n, 1), total) if self.slices else self.plan
        padded = max(16, -(-total // 16) * 16)
        self.h_data = torch.zeros(padded, dtype=torch.uint8, pin_memory=True)
        self.h_data.numpy()[:total] = np.asarray(data[:total], dtype=np.uint8)
        self.h_off = torch.from_numpy(offsets.copy()).pin_memory()
        self.h_out = torch.zeros((3, max(n, 1)), dtype=torch.int32, pin_memory=True)
        self.d_data = torch.empty_like(self.h_data, device=dev)
        self.d_data.copy_(self.h_data)
        self.d_off = torch.empty_like(self.h_off, device=dev)
        self.d_off.copy_(self.h_off)
        self.multi = len(engine.automata) > 1
        if self.multi:
            if aut_ids.size and (aut_ids.min() < 0 or aut_ids.max() >= len(engine.automata)):
                raise ValueError("request names an automaton outside the pool")
            self.h_aut = torch.from_numpy(aut_ids.astype(np.int32)).pin_memory()
            self.d_aut = self.h_aut.to(dev)
        else:
            self.h_aut = self.d_aut = None
        self.ingest = ingest
        self.host_ptr = (native.device_pointer(self.h_data.data_ptr())
                         if ingest == "zero_copy" else None)
        self.d_out = torch.zeros((3, max(n, 1)), dtype=torch.int32, device=dev)
        self.with_examined = with_examined
        self.stream = torch.cuda.Stream(dev)
        if self.slices:
            self.copy_stream = torch.cuda.Stream(dev)
            self.slice_streams = [torch.cuda.Stream(dev) for _ in self.slices]
            self.slice_events = [torch.cuda.Event() for _ in self.slices]
        self.h2d_bytes = (0 if ingest == "zero_copy" else padded) + self.h_off.numel() * 8 + \
            (self.h_aut.numel() * 4 if self.multi else 0)
        self.d2h_bytes = self.h_out.numel() * 4 + native.PLAN_HEADER_WORDS * 4
        self.launches_per_step = 0
        # warm-up outside capture (kernel attributes, occupancy queries, module load); the
        # plan must fit its buffers
        with torch.cuda.stream(self.stream):
            self._body()
        self.stream.synchronize()
        self.plan.check()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream):
            self._body()
        torch.cuda.synchronize(dev)

    def _outputs(self, first: int):
        ex = self.d_out[2][first:] if self.with_examined else None
        return self.d_out[0][first:], self.d_out[1][first:], ex

    def _body(self) -> None:
        s = torch.cuda.current_stream(self.engine.device)
        self.d_off.copy_(self.h_off, non_blocking=True)
        if self.multi:
            self.d_aut.copy_(self.h_aut, non_blocking=True)
        f, l, ex = self._outputs(0)
        if self.slices:
            start = torch.cuda.Event()
            start.record(s)
            self.copy_stream.wait_event(start)
            with torch.cuda.stream(self.copy_stream):
                for (lo, hi), ev in zip(self.slices, self.slice_events):
                    self.d_data[lo:hi].copy_(self.h_data[lo:hi], non_blocking=True)
                    ev.record(self.copy_stream)
            self.plan.plan(self.d_off, None, self.d_aut, s, self.n)
            self.launches_per_step = 2 + self.plan.launch(
                self.d_data.data_ptr(), self.d_off, None, f, l, ex, s,
                lane_slices=list(zip(self.slice_streams, self.slice_events)))
        else:
            if self.ingest == "copy":
                self.d_data.copy_(self.h_data, non_blocking=True)
            self.plan.plan(self.d_off, None, self.d_aut, s, self.n)
            data_ptr = self.host_ptr if self.ingest == "zero_copy" else self.d_data.data_ptr()
            self.launches_per_step = 2 + self.plan.launch(data_ptr, self.d_off, None, f, l, ex, s)
        self.h_out.copy_(self.d_out, non_blocking=True)
        self.plan.fetch_header(s)

    def replay(self) -> None:
        """Launch the captured graph on the runner's stream (asynchronous)."""
        with torch.cuda.stream(self.stream):
            self.graph.replay()

    def kernel_only(self, stream=None, phases: dict | None = None) -> int:
        """Planning and the launches alone, on the device copy of the inputs (for
        device-side timing); returns the number of kernels launched."""
        stream = stream or torch.cuda.current_stream(self.engine.device)
        f, l, ex = self._outputs(0)
        if phases is not None:
            e = torch.cuda.Event(enable_timing=True)
            e.record(stream)
            phases.setdefault("plan", []).append(e)
        self.kplan.plan(self.d_off, None, self.d_aut, stream, self.n)
        if phases is not None:
            e = torch.cuda.Event(enable_timing=True)
            e.record(stream)
            phases["plan"].append(e)
        return 2 + self.kplan.launch(self.d_data.data_ptr(), self.d_off, None, f, l, ex, stream,
                                     phases=phases)

    def plan_info(self) -> dict:
        """Chunk sizes and counts of the last plan (after the stream has finished)."""
        h = self.plan.h_header.numpy()
        return {"lane_chunk_bytes": int(h[native.PLAN_LANE_BYTES]),
                "warp_chunk_bytes": int(h[native.PLAN_WARP_BYTES]),
                "lane_chunks": int(h[native.PLAN_LANE_CHUNKS]),
                "chunks": int(h[native.PLAN_CHUNKS]),
                "lane_tasks": int(h[native.PLAN_LANE_TASKS]),
                "persistent_tasks": int(h[native.PLAN_PERSIST_TASKS]),
                "fixup_tasks": int(h[native.PLAN_FIXUP_TASKS]),
                "dfa_chunks": int(h[native.PLAN_DFA_CHUNKS]),
                "dfa_fixups": int(h[native.PLAN_DFA_FIXUPS]),
                "dfa_chunk_bytes": int(h[native.PLAN_DFA_CHUNK_BYTES])}

    def verdicts(self):
        """(flags, lens, examined) of the last replay, once it has finished."""
        self.stream.synchronize()
        self.plan.check()
        h = self.h_out.numpy()
        return h[0, :self.n].copy(), h[1, :self.n].copy(), h[2, :self.n].copy()
