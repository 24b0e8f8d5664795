"""Continuous-batching serving loop over a resident automaton pool.

The pool (NFAs and DFAs of any size) stays resident in a ``PersistentEngine``. Requests
``(automaton index, bytes)`` arrive over time; the loop:

1. admits arrived requests into a FIFO queue;
2. whenever one of its ``slots`` is free, forms a batch from the head of the queue under
   the slot's device-memory budget (``batch_bytes`` of input; a request larger than the
   budget is rejected) and enqueues, on that slot's stream, the host->device copies, one
   persistent launch (longest work first) and the device->host copy of the verdicts;
3. harvests finished slots (CUDA event query), stamping each request's completion time.

With two or more slots, a batch is staged and launched while earlier ones are still on
the GPU, so requests that arrive meanwhile join the next launch as soon as a slot and
its memory free up, and consecutive launches overlap on the device (each slot has its
own stream, buffers and engine workspace). Latency is completion minus arrival on the
host's monotonic clock.

Ingest modes: ``copy`` packs each batch into the slot's pinned buffer and copies it to
the device; ``zero_copy`` leaves requests in place in a pinned host pool and the kernel
reads their bytes over the host link directly (GB300's coherent NVLink-C2C), so only
the bytes a simulation actually examines cross it -- a latching or dying input stops
reading early.

The reference has no serving path; its closest analogue is a per-call executor
(src/gpufsm/api.py:27-52). ``serve_plain`` is that baseline on the same trace: one plain
launch per request, in arrival order.
"""

from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import native
from .engine import DevicePlan, PersistentEngine
from .packing import PAD
from .registry import Kind


@dataclass
class ServeStats:
    requests: int
    wall_s: float
    offered_bytes: int
    examined_bytes: int
    p50_ms: float
    p99_ms: float
    mean_ms: float
    max_ms: float
    batches: int
    mean_batch: float
    rejected: int
    mode: str
    extra: dict = field(default_factory=dict)

    @property
    def offered_GBps(self) -> float:
        return self.offered_bytes / max(self.wall_s, 1e-9) / 1e9

    @property
    def examined_GBps(self) -> float:
        """Bytes the simulations consumed (up to each latch or death) per second."""
        return self.examined_bytes / max(self.wall_s, 1e-9) / 1e9

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k in ("requests", "wall_s", "offered_bytes",
                                           "examined_bytes", "p50_ms", "p99_ms", "mean_ms",
                                           "max_ms", "batches", "mean_batch", "rejected",
                                           "mode")}
        d["offered_GBps"] = self.offered_GBps
        d["examined_GBps"] = self.examined_GBps
        d.update(self.extra)
        return d


class _Slot:
    def __init__(self, engine: PersistentEngine, batch_bytes: int, max_requests: int,
                 zero_copy: bool) -> None:
        dev = engine.device
        self.stream = torch.cuda.Stream(dev)
        self.event = torch.cuda.Event()
        self.workspace = engine.new_workspace()
        self.zero_copy = zero_copy
        if not zero_copy:
            self.h_data = torch.empty(batch_bytes + PAD, dtype=torch.uint8, pin_memory=True)
            self.d_data = torch.empty(batch_bytes + PAD, dtype=torch.uint8, device=dev)
        self.h_off = torch.empty(2 * max_requests + 1, dtype=torch.int64, pin_memory=True)
        self.d_off = torch.empty(2 * max_requests + 1, dtype=torch.int64, device=dev)
        self.h_aut = torch.empty(max_requests, dtype=torch.int32, pin_memory=True)
        self.d_aut = torch.empty(max_requests, dtype=torch.int32, device=dev)
        self.plan = DevicePlan(engine, max_requests, batch_bytes)
        self.h_out = torch.zeros((3, max_requests), dtype=torch.int32, pin_memory=True)
        self.d_out = torch.zeros((3, max_requests), dtype=torch.int32, device=dev)
        self.reqs: list[int] = []


class Server:
    """Continuous batching over ``engine`` with ``slots`` concurrent launches."""

    def __init__(self, automata=None, device=None, slots: int = 3, batch_bytes: int = 64 << 20,
                 max_requests: int = 2048, engine: PersistentEngine | None = None,
                 zero_copy: bool = False, memory_fraction: float = 0.5) -> None:
        self.engine = engine or PersistentEngine(automata, device)
        dev = self.engine.device
        free, _total = torch.cuda.mem_get_info(dev)
        # admission budget: the slots' input buffers must fit a fraction of free memory
        budget = int(free * memory_fraction)
        plan_bytes = DevicePlan.device_bytes(self.engine, max_requests, batch_bytes)
        per_slot = batch_bytes + 64 * max_requests + self.engine.ws_bytes + plan_bytes
        if slots * per_slot > budget:
            slots = max(1, budget // per_slot)
        self.batch_bytes = batch_bytes
        self.max_requests = max_requests
        self.zero_copy = zero_copy
        self.slots = [_Slot(self.engine, batch_bytes, max_requests, zero_copy)
                      for _ in range(slots)]
        self.is_dfa = np.array([k is Kind.DFA for k in self.engine.kinds])

    # ---- one batch ----------------------------------------------------------------------

    def _launch(self, slot: _Slot, reqs: list[int], aut_ids: np.ndarray, starts: np.ndarray,
                lengths: np.ndarray, pool: np.ndarray, pool_dev_ptr: int | None) -> None:
        n = len(reqs)
        ln = lengths[reqs]
        slot.h_aut.numpy()[:n] = aut_ids[reqs]
        off = slot.h_off.numpy()
        if self.zero_copy:
            off[:n] = starts[reqs]
            off[n:2 * n] = starts[reqs] + ln
        else:
            off[0] = 0
            np.cumsum(ln, out=off[1:n + 1])
            h = slot.h_data.numpy()
            pos = 0
            for r, k in zip(reqs, ln.tolist()):
                s = int(starts[r])
                h[pos:pos + k] = pool[s:s + k]
                pos += k
            h[pos:pos + PAD] = 0
        with torch.cuda.stream(slot.stream):
            if self.zero_copy:
                slot.d_off[:2 * n].copy_(slot.h_off[:2 * n], non_blocking=True)
                d_off = slot.d_off[:n]
                d_ends = slot.d_off[n:2 * n]
                data = pool_dev_ptr
            else:
                used = int(off[n]) + PAD
                slot.d_data[:used].copy_(slot.h_data[:used], non_blocking=True)
                slot.d_off[:n + 1].copy_(slot.h_off[:n + 1], non_blocking=True)
                d_off, d_ends, data = slot.d_off, None, slot.d_data.data_ptr()
            slot.d_aut[:n].copy_(slot.h_aut[:n], non_blocking=True)
            slot.plan.plan(d_off, d_ends, slot.d_aut, slot.stream, n)
            slot.plan.launch(data, d_off, d_ends, slot.d_out[0], slot.d_out[1], slot.d_out[2],
                             slot.stream, workspace=slot.workspace)
            for r in range(3):
                slot.h_out[r, :n].copy_(slot.d_out[r, :n], non_blocking=True)
            slot.plan.fetch_header(slot.stream)
            slot.event.record(slot.stream)
        slot.reqs = reqs

    # ---- the loop -------------------------------------------------------------------------

    def serve(self, trace, time_scale: float = 1.0, pinned_pool: torch.Tensor | None = None):
        """Serve every request of ``trace`` (a ``workloads.ServingTrace``) at its arrival
        times (scaled by ``time_scale``). Returns ``(flags, lens, latency_ms, stats)``."""
        n = len(trace.aut_ids)
        arrivals = np.asarray(trace.arrivals, dtype=np.float64) * time_scale
        aut_ids = np.asarray(trace.aut_ids, dtype=np.int64)
        starts = np.asarray(trace.starts, dtype=np.int64)
        lengths = np.asarray(trace.lengths, dtype=np.int64)
        pool = trace.pool
        pool_ptr = None
        if self.zero_copy:
            if pinned_pool is None:
                pinned_pool = torch.from_numpy(pool).pin_memory()
            pool = pinned_pool.numpy()
            pool_ptr = native.device_pointer(pinned_pool.data_ptr())
        flags = np.zeros(n, np.int32)
        lens = np.zeros(n, np.int32)
        examined = np.zeros(n, np.int64)
        done_at = np.zeros(n, np.float64)
        rejected = np.zeros(n, dtype=bool)
        pending: deque[int] = deque()
        free = list(self.slots)
        busy: list[_Slot] = []
        nxt = 0
        finished = 0
        batches = 0
        batch_sizes = []
        t0 = time.perf_counter()
        while finished < n:
            now = time.perf_counter() - t0
            while nxt < n and arrivals[nxt] <= now:
                if lengths[nxt] > self.batch_bytes:
                    rejected[nxt] = True
                    done_at[nxt] = now
                    finished += 1
                else:
                    pending.append(nxt)
                nxt += 1
            progressed = False
            for slot in list(busy):
                if slot.event.query():
                    k = len(slot.reqs)
                    t = time.perf_counter() - t0
                    slot.plan.check()
                    h = slot.h_out.numpy()
                    flags[slot.reqs] = h[0, :k]
                    lens[slot.reqs] = h[1, :k]
                    examined[slot.reqs] = h[2, :k]
                    done_at[slot.reqs] = t
                    finished += k
                    busy.remove(slot)
                    free.append(slot)
                    progressed = True
            while free and pending:
                slot = free.pop()
                reqs, used = [], 0
                while pending and len(reqs) < self.max_requests:
                    r = pending[0]
                    if reqs and used + lengths[r] > self.batch_bytes:
                        break
                    reqs.append(pending.popleft())
                    used += int(lengths[r])
                self._launch(slot, reqs, aut_ids, starts, lengths, pool, pool_ptr)
                busy.append(slot)
                batches += 1
                batch_sizes.append(len(reqs))
                progressed = True
            if not progressed:
                if not busy and not pending and nxt < n:
                    wait = arrivals[nxt] - (time.perf_counter() - t0)
                    if wait > 2e-4:
                        time.sleep(wait - 1e-4)
                else:
                    time.sleep(2e-5)
        wall = time.perf_counter() - t0
        lat = (done_at - arrivals) * 1e3
        ok = ~rejected
        if n and flags.min() < 0:
            raise TimeoutError("a bounded device wait gave up during serving")
        stats = ServeStats(
            requests=n, wall_s=wall, offered_bytes=int(lengths[ok].sum()),
            examined_bytes=int(examined[ok].sum()), p50_ms=float(np.percentile(lat[ok], 50)) if ok.any() else 0.0,
            p99_ms=float(np.percentile(lat[ok], 99)) if ok.any() else 0.0,
            mean_ms=float(lat[ok].mean()) if ok.any() else 0.0,
            max_ms=float(lat[ok].max()) if ok.any() else 0.0,
            batches=batches, mean_batch=float(np.mean(batch_sizes)) if batch_sizes else 0.0,
            rejected=int(rejected.sum()), mode="zero_copy" if self.zero_copy else "copy")
        return flags, lens, lat, stats


def serve_plain(engine: PersistentEngine, trace, executors: dict, time_scale: float = 1.0):
    """Baseline: one plain launch per request, in arrival order, on one stream.

    ``executors[k]`` is a plain executor for automaton ``k`` (``run_arrays`` interface).
    Returns ``(flags, lens, latency_ms, stats)``.
    """
    n = len(trace.aut_ids)
    arrivals = np.asarray(trace.arrivals, dtype=np.float64) * time_scale
    flags = np.zeros(n, np.int32)
    lens = np.zeros(n, np.int32)
    examined = np.zeros(n, np.int64)
    done_at = np.zeros(n)
    t0 = time.perf_counter()
    for i in range(n):
        now = time.perf_counter() - t0
        if arrivals[i] > now:
            time.sleep(arrivals[i] - now)
        a, data = trace.request(i)
        f, l, e, _, _ = executors[a].run_arrays([data], with_examined=True)
        flags[i], lens[i], examined[i] = f[0], l[0], e[0]
        done_at[i] = time.perf_counter() - t0
    wall = time.perf_counter() - t0
    lat = (done_at - arrivals) * 1e3
    stats = ServeStats(requests=n, wall_s=wall, offered_bytes=int(np.sum(trace.lengths)),
                       examined_bytes=int(examined.sum()), p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)),
                       mean_ms=float(lat.mean()), max_ms=float(lat.max()), batches=n,
                       mean_batch=1.0, rejected=0, mode="plain per request")
    return flags, lens, lat, stats
