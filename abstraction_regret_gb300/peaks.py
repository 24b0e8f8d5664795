"""Measured on-chip peaks: the denominators of the L2 and shared-memory rooflines.

The simulation kernels gather edge records and DFA table entries that stay on chip, so
their bound is L2 (or shared memory), not HBM. These figures come from the probe kernels
of ``csrc/peaks.cu``, timed with CUDA events (best of several launches after a warm-up):

* ``l2_read_GBps``: streaming 16-byte L2-only loads over a 32 MiB buffer, every SM busy;
* ``l2_gather16_*``: independent 16-byte loads at random entries of a 1 MiB table (the
  size of the c3 lane records) through L2 only and through L1, as records per second and
  as GB/s of 16-byte records;
* ``l2_latency_ns``: one dependent 4-byte L2 load (a pointer chase over a random cycle of
  a 4 MiB table);
* ``smem_GBps``: bank-conflict-free 16-byte shared-memory loads, 4 CTAs of 256 threads
  per SM;
* ``h2d_*_GBps``: the host link, 256 MiB from page-locked memory: one copy-engine
  transfer (``dma``), four concurrent ones (``dma4``), and a copy driven by the SMs
  reading the mapped host buffer (``sm2`` / ``sm8``: 2 or 8 CTAs of 256 threads per SM).

    python -m abstraction_regret_gb300.peaks     # prints the figures as one JSON line
"""

from __future__ import annotations

import ctypes
import json

import numpy as np

from . import native


def _best_ms(fn, stream, reps: int = 5) -> float:
    import torch

    fn()
    stream.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def measure(device=None) -> dict:
    """Run every probe on ``device`` (default: the current CUDA device)."""
    import torch

    lib = native.lib()
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else \
        torch.device(device)
    sm = torch.cuda.get_device_properties(dev).multi_processor_count
    out: dict = {"device": torch.cuda.get_device_name(dev), "sm_count": sm}
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev)
        s = stream.cuda_stream
        sink = torch.zeros(1, dtype=torch.int64, device=dev)

        def call(st, what):
            native.check(st, what)

        # L2 streaming read bandwidth
        nbytes, passes = 32 << 20, 16
        buf = torch.randint(0, 255, (nbytes,), dtype=torch.uint8, device=dev)
        ms = _best_ms(lambda: call(lib.gbfsm_probe_l2_read(buf.data_ptr(), nbytes, passes,
                                                           sink.data_ptr(), s),
                                   "gbfsm_probe_l2_read"), stream)
        out["l2_read_GBps"] = nbytes * passes / (ms * 1e-3) / 1e9
        # random 16-byte gathers from a 1 MiB table
        tbytes, loads = 1 << 20, 1024
        threads = sm * 8 * 256
        for via_l1, key in ((0, "l2_gather16"), (1, "l1_gather16")):
            ms = _best_ms(lambda: call(lib.gbfsm_probe_gather16(buf.data_ptr(), tbytes, loads,
                                                                via_l1, sink.data_ptr(), s),
                                       "gbfsm_probe_gather16"), stream)
            per_s = threads * (-(-loads // 8) * 8) / (ms * 1e-3)
            out[key + "_Grecords_per_s"] = per_s / 1e9
            out[key + "_GBps"] = per_s * 16 / 1e9
        # dependent-load latency: a random single cycle over 1 Mi entries (4 MiB)
        n = 1 << 20
        perm = np.random.default_rng(0).permutation(n).astype(np.uint32)
        nxt = np.empty(n, dtype=np.uint32)
        nxt[perm] = np.roll(perm, -1)
        d_next = torch.from_numpy(nxt.view(np.int32)).to(dev)
        steps = 100_000
        ms = _best_ms(lambda: call(lib.gbfsm_probe_chase(d_next.data_ptr(), n, steps, 1,
                                                         sink.data_ptr(), s),
                                   "gbfsm_probe_chase"), stream, reps=3)
        out["l2_latency_ns"] = ms * 1e6 / steps
        # shared-memory bandwidth
        iters, blocks = 1 << 14, 4
        ms = _best_ms(lambda: call(lib.gbfsm_probe_smem(iters, blocks, sink.data_ptr(), s),
                                   "gbfsm_probe_smem"), stream)
        out["smem_GBps"] = sm * blocks * 4096 * iters / (ms * 1e-3) / 1e9
        del buf, d_next
        # host -> device ingest of 256 MiB from page-locked memory: one copy-engine
        # transfer, four concurrent transfers of a quarter each, and an SM-driven copy
        # reading the mapped host buffer over the host link
        nbytes = 256 << 20
        h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        h.fill_(7)
        d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        ms = _best_ms(lambda: d.copy_(h, non_blocking=True), stream, reps=3)
        out["h2d_dma_GBps"] = nbytes / (ms * 1e-3) / 1e9
        side = [torch.cuda.Stream(dev) for _ in range(4)]
        q = nbytes // 4

        def four():
            ev = torch.cuda.Event()
            ev.record(stream)
            for k, st in enumerate(side):
                st.wait_event(ev)
                with torch.cuda.stream(st):
                    d[k * q:(k + 1) * q].copy_(h[k * q:(k + 1) * q], non_blocking=True)
            for st in side:
                stream.wait_stream(st)

        ms = _best_ms(four, stream, reps=3)
        out["h2d_dma4_GBps"] = nbytes / (ms * 1e-3) / 1e9
        hp = native.device_pointer(h.data_ptr())
        for blocks in (2, 8):
            ms = _best_ms(lambda: call(lib.gbfsm_probe_copy(d.data_ptr(), hp, nbytes, blocks, s),
                                       "gbfsm_probe_copy"), stream, reps=3)
            out[f"h2d_sm{blocks}_GBps"] = nbytes / (ms * 1e-3) / 1e9
        del h, d
        out["pageable_access"] = int(lib.gbfsm_pageable_access())
    out["method"] = ("CUDA events, best of 5 launches after a warm-up: L2 streaming read of "
                     "32 MiB x 16 passes (ld.global.cg); 16-byte random gathers from 1 MiB; "
                     "pointer chase over a 4 MiB random cycle (1 chain, 100k steps); "
                     "shared-memory 16-byte loads, 4 CTAs x 256 threads per SM; host->device "
                     "256 MiB from pinned memory by copy engines and by an SM copy kernel "
                     "(best of 3)")
    return out


if __name__ == "__main__":
    print(json.dumps(measure()))
