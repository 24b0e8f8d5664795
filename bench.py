"""Benchmark: bit-exact input GB/s of the persistent batched engine vs the plain kernels.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c3-sustained|c3-live|c3-literal]

One "step" is one pass of the hot path over the whole batch of the uneven-input NFA
configuration (16384-state NFA, Poisson(4) out-degree, 2048 inputs with log-uniform
lengths in [256 B, 1 MiB]; c3). The default variant is "sustained": random-walk inputs
that keep the active set alive and no accepting state, so every offered byte is
examined (the literal configuration's uniform bytes kill the active set after about one
byte). Inputs are larger than L2 (261 MB > 129 MB).

Printed (rank 0, one JSON line):
  value       GB/s of input through the engine's launches (lane launch, persistent
              launch, overflow pass, fix-up), inputs resident in HBM (CUDA events
              around K steps on the launching stream);
  e2e         the same batch through the public engine path: a captured CUDA graph
              that moves the inputs from pinned host memory, runs the launches and
              copies the verdicts back, every step; the fastest of three ingest paths
              (one host->device copy first; read in place over NVLink-C2C by the
              kernels; copied in slices overlapped with the simulation of the previous
              slice), the others beside it as ``e2e_other_ingest``;
  plain_*     the plain kernels on the same batch: one launch per input (sample,
              sequential on one stream, scaled by bytes) and one launch for the batch;
  dfa         the plain DFA walk on the c2 configuration (4096 states, 4096 x 64 KiB);
  serving     the continuous-batching loop on the c5 trace (p50 / p99 latency, offered
              GB/s, against one plain launch per request);
  roofline    the dominant kernel (the lane launch) against the measured HBM copy
              bandwidth, with the input stream alone beside it;
  cpu_baseline the CPU oracle port on this host's cores on a bounded sample.

With ``--impl reference`` the reference's CPU algorithm (the C port of
gpufsm.reference.simulate in oracle/, all host threads) is timed on a bounded sample of
the same workload instead. With torchrun (N > 1) each rank runs an independent replica
on its own GPU ("replicas only": inputs are independent, nothing is exchanged).
"""

from __future__ import annotations

import argparse
import dataclasses
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "bit-exact input GB/s, persistent-batched vs plain, 1 GB300; serving p50/p99 ms"


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="c3-sustained",
                    choices=["c3-sustained", "c3-live", "c3-literal"])
    ap.add_argument("--skip-extras", action="store_true",
                    help="only the headline measurement (used for profiling)")
    ap.add_argument("--extras", default="plain,run_batch,refgpu,c1,dfa,dfa_chunks,c4,serving",
                    help="comma-separated extra sections after the headline")
    ap.add_argument("--serve-requests", type=int, default=20000,
                    help="requests of the c5 serving trace (0: skip the serving section)")
    ap.add_argument("--slo-ms", type=float, default=50.0,
                    help="p99 latency objective of the serving section")
    return ap.parse_args(argv)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def load_workload(name: str, reference_arm: bool = False):
    """The named batch. The CPU reference arm generates its random-walk inputs with the
    oracle's walker (byte-identical), so that it loads no product library."""
    from abstraction_regret_gb300 import workloads as W

    config, variant = name.split("-", 1)
    walk = None
    if reference_arm:
        from oracle import oracle as O

        walk = O.walk_bytes
    return {"c1": W.c1, "c3": W.c3}[config](variant, walk=walk)


def workload_config(workload: str) -> str:
    """The workload string both arms print (same configuration, same words)."""
    return (f"{workload}: 16384-state NFA, Poisson(4) degree, 0.1% accepting (cleared when "
            "sustained), 2048 inputs log-uniform 256 B..1 MiB")


# ---- clocks during the timed region -------------------------------------------------------


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, period_ms: int = 20) -> None:
        self.gpu = gpu_index
        self.period_ms = period_ms
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        # wait (bounded) for the first sample, so the timed region that follows is covered
        t0 = time.monotonic()
        while self.proc is not None and time.monotonic() - t0 < 5.0:
            if self.proc.poll() is not None:
                break
            try:
                if os.path.getsize(self.path) > 0:
                    break
            except OSError:
                pass
            time.sleep(0.01)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ---- measurements ---------------------------------------------------------------------------


def max_over_ranks(x: float, device, world: int) -> float:
    """The slowest rank's time: every replica's step must be over for the job's step."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(offered_bytes: int, ms: float, world: int) -> float:
    """Whole-job GB/s of `world` replicas, each processing `offered_bytes` per step, at
    the slowest rank's step time (replicas only: inputs are independent, nothing is
    exchanged)."""
    return offered_bytes * world / (ms * 1e-3) / 1e9


def step_stats(samples, total_bytes: int, iters: int = 2000, seed: int = 0) -> dict:
    """Median step time with a percentile-bootstrap 95 % interval of the median
    (``iters`` resamples of the steps with replacement, seeded so a rerun gives the same
    interval), and the throughput at the median. Step times are skewed by the odd slow
    step, so the median and its interval describe them better than a mean and a standard
    deviation."""
    a = np.asarray(samples, dtype=np.float64)
    if a.size == 0:
        return {"n": 0}
    med = float(np.median(a))
    if a.size > 1:
        draws = np.random.default_rng(seed).integers(0, a.size, size=(iters, a.size))
        meds = np.median(a[draws], axis=1)
        lo, hi = float(np.percentile(meds, 2.5)), float(np.percentile(meds, 97.5))
    else:
        lo = hi = med
    return {"median_ms": med, "ci95_ms": [lo, hi], "n": int(a.size),
            "median_GBps": total_bytes / (med * 1e-3) / 1e9,
            "method": f"median of {a.size} step times, percentile bootstrap CI95 of the "
                      f"median ({iters} resamples, seed {seed})"}


def time_launches(fn, stream, steps: int, warmup: int):
    """Mean ms per call of ``fn`` over ``steps`` calls (CUDA events on ``stream``)."""
    import torch

    for _ in range(warmup):
        fn()
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def cpu_port(one_pass, offered: int, what: str, budget_s: float = 5.0) -> dict:
    """The oracle port on this host's cores for one extra configuration: whole passes
    (``one_pass()`` runs the batch once, inputs spread over every thread) until
    ``budget_s`` of wall time has gone; at least one pass. Offered bytes per second, the
    unit of the extras."""
    threads = os.cpu_count() or 1
    passes = 0
    t0 = time.perf_counter()
    while True:
        one_pass(threads)
        passes += 1
        dt = time.perf_counter() - t0
        if dt >= budget_s:
            break
    return {"value": offered * passes / dt / 1e9, "unit": "GB/s", "cores": threads,
            "kind": "port", "sample": f"{passes} whole passes over {what} in {dt:.1f} s"}


def nfa_roofline(counts: dict, ms: float, onchip: dict | None) -> dict:
    """Roofline of an NFA engine step from the oracle's counts (same rule as the
    headline: per examined symbol 1 input byte, 8 bytes per active state, 8 per scanned
    edge, 12 bytes of verdicts per input) against the L2 read bandwidth, with the latency
    bound of its chains (lane chunks or whole inputs: one dependent L2 load per byte)."""
    algo = counts["examined"] + 8 * counts["states"] + 8 * counts["edges"] + 12 * counts["n"]
    achieved = algo / (ms * 1e-3) / 1e9
    l2 = onchip.get("l2_read_GBps") if onchip else None
    lat = onchip.get("l2_latency_ns") if onchip else None
    sym = counts["examined"] / (ms * 1e-3) / 1e9
    bound_sym = counts["chains"] / lat if lat and counts["chains"] else None
    smem = onchip.get("smem_GBps") if onchip else None
    return {"bound": "l2", "achieved": achieved, "peak": l2, "unit": "GB/s",
            "frac": achieved / l2 if l2 else None, "algorithmic_bytes": int(algo),
            "smem_peak": smem, "frac_of_smem_peak": achieved / smem if smem else None,
            "latency": {"chains": counts["chains"], "l2_latency_ns": lat,
                        "bound_Gsymbols_per_s": bound_sym, "achieved_Gsymbols_per_s": sym,
                        "frac": sym / bound_sym if bound_sym else None},
            "peak_source": "measured in this run: L2 streaming read (gbfsm_probe_l2_read)"}


def dfa_roofline(examined: int, chains: int, ms: float, onchip: dict | None,
                 hbm: float) -> dict:
    """Roofline of a DFA walk: every examined symbol is one dependent lookup of a 2-byte
    table entry held on chip, so ``chains`` walks run at most chains / L2 latency symbols
    per second; the input stream (1 byte per symbol) against HBM beside it."""
    lat = onchip.get("l2_latency_ns") if onchip else None
    l2 = onchip.get("l2_read_GBps") if onchip else None
    sym = examined / (ms * 1e-3) / 1e9
    bound = chains / lat if lat else None
    # the bandwidth view: per examined symbol 1 input byte from HBM and one table entry
    # (counted as 4 bytes, the reference's int32 table, and as a whole 32-byte L2 sector)
    bw_bound = min(hbm / 1.0, l2 / 4.0) if l2 else hbm
    return {"bound": "latency", "achieved": sym, "peak": bound, "unit": "Gsymbols/s",
            "frac": sym / bound if bound else None, "chains": chains, "l2_latency_ns": lat,
            "algorithmic_bytes": 3 * int(examined),
            "bandwidth": {"bound_Gsymbols_per_s": bw_bound, "frac": sym / bw_bound,
                          "frac_at_32B_per_sector": sym / (l2 / 32.0) if l2 else None,
                          "rule": "min(HBM/1 B, L2/4 B) per examined symbol"},
            "input_stream": {"achieved": sym, "peak": hbm, "unit": "GB/s",
                             "frac": sym / hbm},
            "peak_source": "chains / L2 dependent-load latency measured in this run "
                           "(gbfsm_probe_chase)"}


def attach_rooflines(extras: dict, onchip: dict | None, hbm: float) -> None:
    """Give the c1, c2 and c4 extras their roofline entries once the on-chip peaks have
    been measured (the counts were stored by their sections)."""
    for key in ("c1_plain_nfa", "c4_multi_automaton"):
        for v in extras.get(key, {}).values():
            c = v.pop("_counts", None)
            if isinstance(v, dict) and c:
                v["roofline"] = nfa_roofline(c, v["engine_ms"] if "engine_ms" in v else v["ms"],
                                             onchip)
    for key in ("dfa_c2_literal", "dfa_c2_sustained"):
        v = extras.get(key)
        if v and "_counts" in v:
            c = v.pop("_counts")
            v["roofline"].update(dfa_roofline(c["examined"], c["chains"], v["ms"], onchip, hbm))


def cpu_reference(batch, budget_s: float = 15.0, threads: int | None = None):
    """The oracle port on this host's cores: whole passes over the batch (inputs spread
    over all threads) until ``budget_s`` of wall time has gone; at least one pass."""
    from oracle import oracle as O

    threads = threads or os.cpu_count() or 1
    a = batch.automata[0]
    passes, examined = 0, 0
    t0 = time.perf_counter()
    while True:
        _, _, ex, _ = O.nfa_batch(a, batch.data, batch.offsets, threads)
        passes += 1
        examined += int(ex.sum())
        dt = time.perf_counter() - t0
        if dt >= budget_s:
            break
    return {"value": passes * batch.total_bytes / dt / 1e9, "unit": "GB/s",
            "cores": int(threads), "kind": "port",
            "sample": f"{passes} whole passes over the {batch.n_inputs}-input batch "
                      f"({passes * batch.total_bytes / 1e6:.0f} MB offered, "
                      f"{examined / 1e6:.0f} MB examined) in {dt:.1f} s"}


def run_reference(args, world, rank):
    """--impl reference: the reference algorithm (C port of the oracle) on host cores."""
    if rank != 0:
        return 0
    batch = load_workload(args.workload, reference_arm=True)
    samples = []
    info = None
    for i in range(args.warmup + args.steps):
        info = cpu_reference(batch, budget_s=10.0 if i >= args.warmup else 1.0)
        if i >= args.warmup:
            samples.append(info["value"])
    value = float(np.median(samples))
    info["value"] = value
    # a step is one pass over the batch: its time at the median rate
    ms_step = batch.total_bytes / (value * 1e9) * 1e3 if value > 0 else None
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": workload_config(args.workload),
                       "sample": info["sample"]},
            "cpu_baseline": info,
            "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "each step times whole passes of the C port over the batch for about "
                    "10 s (median of the steps); ms_per_step is one pass at that rate"}
    print(json.dumps(line), flush=True)
    return 0


def main(argv=None) -> int:
    args = parse_args(argv)
    world, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch
    import torch.distributed as dist

    import abstraction_regret_gb300 as G
    from abstraction_regret_gb300.engine import GraphRunner, PersistentEngine
    from abstraction_regret_gb300.executors import CudaDFAExecutor, CudaNFAExecutor
    from abstraction_regret_gb300 import native
    from abstraction_regret_gb300 import workloads as W

    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)

    batch = load_workload(args.workload)
    nfa = batch.automata[0]
    eng = PersistentEngine([nfa], dev)
    runners = {ing: GraphRunner(eng, batch.aut_ids, batch.data, batch.offsets,
                                with_examined=True, ingest=ing)
               for ing in GraphRunner.INGEST}
    runner = runners["copy"]
    stream = runner.stream

    # ---- oracle gate before any timing (full batch, bit-exact, every ingest path) ----------
    verdicts = []
    for r in runners.values():
        with torch.cuda.stream(r.stream):
            r.replay()
        r.stream.synchronize()
        verdicts.append(r.verdicts())
    flags, lens, examined = verdicts[0]
    gate = {"checked": 0}
    if rank == 0:
        from oracle import oracle as O

        f, l, ex, _, work, visits = O.nfa_batch(nfa, batch.data, batch.offsets, with_work=True)
        for fl, le, exa in verdicts:
            if not (np.array_equal(fl, f) and np.array_equal(le, l) and np.array_equal(exa, ex)):
                bad = np.flatnonzero((fl != f) | (le != l) | (exa != ex))
                raise SystemExit(f"oracle gate failed on {bad.size} inputs "
                                 f"(first {bad[:5].tolist()})")
        gate = {"checked": int(flags.size), "paths": list(runners),
                "accepted": int(f.sum()), "examined_bytes": int(ex.sum()),
                "edges_scanned": int(work.sum()), "states_stepped": int(visits.sum())}

    offered = batch.total_bytes
    examined_bytes = int(examined.sum())

    # ---- headline: the engine's launches on resident inputs ------------------------------
    def barrier():
        if world > 1:
            dist.barrier()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            runner.kernel_only(stream)
    phases: dict = {}
    # clocks are sampled over the headline's and the e2e paths' timed regions
    clk = ClockSampler(local).__enter__()
    barrier()
    torch.cuda.synchronize()
    # an event between consecutive steps gives per-step times for the median and its
    # interval; the mean over the K steps (first to last event) is the headline
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with torch.cuda.stream(stream):
        marks[0].record(stream)
        launches = 0
        for k in range(args.steps):
            launches += runner.kernel_only(stream, phases=phases)
            marks[k + 1].record(stream)
    marks[-1].synchronize()
    ms = marks[0].elapsed_time(marks[-1]) / args.steps
    step_samples = [marks[k].elapsed_time(marks[k + 1]) for k in range(args.steps)]
    torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(ms, dev, world)
    value = replica_throughput(offered, ms, world)
    phase_ms = {k: float(np.mean([ev[2 * i].elapsed_time(ev[2 * i + 1])
                                  for i in range(len(ev) // 2)]))
                for k, ev in phases.items()}

    # ---- e2e: graph replay, inputs from pinned host memory, verdicts back every step ----
    describe = {
        "copy": "CUDA graph: inputs + tables H2D from pinned memory, launches, verdicts D2H",
        "zero_copy": "CUDA graph: tables H2D, kernels read the inputs from pinned host "
                     "memory over NVLink-C2C, verdicts D2H",
        "pipelined": "CUDA graph: the inputs copied H2D from pinned memory in 8 slices on "
                     "a copy stream; each slice's lane tasks (chunks for two waves of the "
                     "lane launch) run on their own stream as soon as its bytes arrive; "
                     "overflow pass and fix-up once for the batch; verdicts D2H"}
    paths = {}
    for name, r in runners.items():
        with torch.cuda.stream(r.stream):
            e2e_ms = time_launches(r.replay, r.stream, args.steps, args.warmup)
        e2e_ms = max_over_ranks(e2e_ms, dev, world)
        paths[name] = {"value": replica_throughput(offered, e2e_ms, world), "unit": "GB/s",
                       "h2d_bytes_per_step": int(r.h2d_bytes),
                       "d2h_bytes_per_step": int(r.d2h_bytes), "ms_per_step": e2e_ms,
                       "path": describe[name]}
    clk.__exit__(None, None, None)
    best = max(paths, key=lambda k: paths[k]["value"])
    e2e = paths[best]
    e2e_other = {k: v for k, v in paths.items() if k != best}

    extras = {}
    sections = set() if args.skip_extras else set(filter(None, args.extras.split(",")))
    if "plain" in sections and rank == 0:
        # plain single launch over the whole batch (the autotuned plain plan)
        plain = CudaNFAExecutor(nfa, "compact", dev)
        d_out = torch.zeros((3, batch.n_inputs), dtype=torch.int32, device=dev)
        with torch.cuda.stream(stream):
            single_ms = time_launches(
                lambda: plain.launch(runner.d_data, runner.d_off, batch.n_inputs, d_out[0],
                                     d_out[1], None, stream), stream, max(2, args.steps // 2), 3)
        assert np.array_equal(d_out[0].cpu().numpy(), flags)
        # plain launch per input, one stream (sample of inputs spread over the lengths)
        lens_all = np.diff(batch.offsets)
        order = np.argsort(lens_all)
        sample = order[np.linspace(0, len(order) - 1, 24).astype(int)]
        per_ms = 0.0
        per_bytes = 0
        one = torch.zeros((3, 1), dtype=torch.int32, device=dev)
        for i in sample:
            off = torch.tensor([0, int(lens_all[i])], dtype=torch.int64, device=dev)
            d = runner.d_data[int(batch.offsets[i]):]
            with torch.cuda.stream(stream):
                per_ms += time_launches(lambda: plain.launch(d, off, 1, one[0], one[1], None, stream),
                                        stream, 1, 1)
            per_bytes += int(lens_all[i])
        per_input_gbps = per_bytes / (per_ms * 1e-3) / 1e9
        extras["plain_single_launch"] = {"value": offered / (single_ms * 1e-3) / 1e9,
                                         "unit": "GB/s", "ms": single_ms,
                                         "technique": "compact, one launch"}
        extras["plain_per_input"] = {"value": per_input_gbps, "unit": "GB/s",
                                     "sample_inputs": int(sample.size), "sample_bytes": per_bytes,
                                     "note": "one launch per input, sequential on one stream"}
        extras["speedup_vs_plain_per_input"] = value / world / per_input_gbps
        extras["speedup_vs_plain_single_launch"] = value / world / extras["plain_single_launch"]["value"]
        del plain, d_out
    for k in [k for k in runners if k != "copy"]:
        del runners[k]
    if "dfa" in sections and rank == 0:
        # DFA walk on c2 (literal and sustained)
        for variant in ("literal", "sustained"):
            b2 = W.c2(variant)
            ex2 = CudaDFAExecutor(b2.automata[0], device=dev)
            r2 = GraphRunnerLike(ex2, b2, dev)
            d_ms = r2.time(stream, max(2, args.steps // 2))
            f2, l2, e2 = r2.verdicts()
            from oracle import oracle as O

            of, ol, oe = O.dfa_batch(b2.automata[0], b2.data, b2.offsets)
            assert np.array_equal(f2, of) and np.array_equal(l2, ol), f"DFA c2-{variant} parity"
            cpu2 = cpu_port(lambda t, b2=b2: O.dfa_batch(b2.automata[0], b2.data, b2.offsets, t),
                            b2.total_bytes, f"c2-{variant} (4096 x 64 KiB)")
            examined_gbps = int(oe.sum()) / (d_ms * 1e-3) / 1e9
            hbm_peak = float(json.loads((REPO / "MEASURED_PEAKS.json").read_text())
                             .get("hbm_gbs", 6800.0)) \
                if (REPO / "MEASURED_PEAKS.json").exists() else 6800.0
            # per examined symbol: 1 input byte (HBM stream) + one 2-byte table entry read
            # from on-chip memory; each input is one chain of dependent lookups
            longest = int(np.diff(b2.offsets).max())
            extras[f"dfa_c2_{variant}"] = {
                "offered_GBps": b2.total_bytes / (d_ms * 1e-3) / 1e9,
                "examined_GBps": examined_gbps,
                "ms": d_ms, "examined_bytes": int(oe.sum()), "checked": int(of.size),
                "roofline": {"bound": "latency (one dependent lookup per symbol per input)",
                             "hbm_frac_input_stream": examined_gbps / hbm_peak,
                             "chains": int(b2.n_inputs),
                             "ns_per_lookup_longest_chain": d_ms * 1e6 / max(1, longest)
                             if variant == "sustained" else None},
                "cpu_baseline": cpu2,
                "_counts": {"examined": int(oe.sum()), "chains": int(b2.n_inputs)}}
            del r2, ex2, b2
    if "run_batch" in sections and rank == 0:
        extras["run_batch_default"] = run_batch_section(batch, flags, lens, steps=3)
    if "refgpu" in sections and rank == 0:
        extras["reference_gpu_kernels"] = reference_gpu_section(dev, max(2, args.steps // 4))
    if "c1" in sections and rank == 0:
        extras["c1_plain_nfa"] = c1_section(dev, max(2, args.steps // 2))
    if "c4" in sections and rank == 0:
        extras["c4_multi_automaton"] = c4_section(dev, max(2, args.steps // 2))
    if "dfa_chunks" in sections and rank == 0:
        extras["dfa_chunks"] = dfa_chunks_section(dev, max(2, args.steps // 4))
    if "serving" in sections and rank == 0 and args.serve_requests > 0:
        extras["serving"] = serving_section(dev, args.serve_requests, args.slo_ms)

    cpu = cpu_reference(batch) if rank == 0 else None
    onchip = None
    if rank == 0:
        from abstraction_regret_gb300 import peaks as P

        onchip = P.measure(dev)
        attach_rooflines(extras, onchip, float(json.loads(
            (REPO / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs", 6800.0))
            if (REPO / "MEASURED_PEAKS.json").exists() else 6800.0)

    # ---- roofline of the dominant kernel ----------------------------------------------
    peaks = {}
    try:
        peaks = json.loads((REPO / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    top = max(phase_ms, key=phase_ms.get) if phase_ms else "lanes"
    kernel_ms = phase_ms.get(top, ms)
    kernel_name = {"lanes": "lanes_kernel", "persistent": "persistent_kernel",
                   "overflow": "persistent_kernel", "fixup": "persistent_kernel",
                   "plan": "plan_scan_kernel"}[top]
    # algorithmic bytes of the exact simulation (CSR view): per examined symbol 1 input
    # byte, per active state an 8-byte row range, per scanned edge 8 bytes (symbol +
    # target); 12 bytes of verdicts per input. Counted by the oracle on the same batch.
    algo = gate.get("examined_bytes", examined_bytes) + 8 * gate.get("states_stepped", 0) + \
        8 * gate.get("edges_scanned", 0) + 12 * batch.n_inputs
    achieved = algo / (kernel_ms * 1e-3) / 1e9
    traffic = None  # DRAM bytes per launch from the committed ncu summary, when one exists
    tpath = REPO / "profiles" / "traffic.txt"
    if tpath.exists():
        for line in tpath.read_text().splitlines():
            parts = line.split()
            if len(parts) == 3 and parts[0] == kernel_name and parts[1] == args.workload:
                traffic = int(parts[2])
    # the bound: the edge gathers are served on chip (a 1 MiB record table), so the
    # algorithmic bytes are held against the L2 read bandwidth measured in this run; the
    # input stream alone against HBM; and a latency bound: every lane chain waits for one
    # dependent L2 record load per byte, so at most chains / L2 latency symbols per second
    l2 = onchip.get("l2_read_GBps") if onchip else None
    info = runner.plan_info()
    chains = min(info["lane_chunks"], eng.sm_count * eng.lane_warps_per_sm * 32)
    lat_ns = onchip.get("l2_latency_ns") if onchip else None
    symbols = gate.get("examined_bytes", examined_bytes)
    roofline = {"bound": "l2", "achieved": achieved, "peak": l2, "unit": "GB/s",
                "frac": achieved / l2 if l2 else None, "traffic": traffic,
                "peak_source": "measured in this run: L2 streaming read (gbfsm_probe_l2_read)",
                "kernel": kernel_name, "kernel_ms": kernel_ms,
                "algorithmic_bytes_per_launch": int(algo),
                "input_stream": {"achieved": examined_bytes / (kernel_ms * 1e-3) / 1e9,
                                 "peak": hbm, "frac": examined_bytes / (kernel_ms * 1e-3) / 1e9 / hbm,
                                 "peak_source": "MEASURED_PEAKS.json hbm_gbs"
                                 if "hbm_gbs" in peaks else "fallback"},
                "latency": {"chains": chains, "l2_latency_ns": lat_ns,
                            "bound_Gsymbols_per_s": chains / lat_ns if chains and lat_ns else None,
                            "achieved_Gsymbols_per_s": symbols / (kernel_ms * 1e-3) / 1e9,
                            "frac": (symbols / (kernel_ms * 1e-3) / 1e9) / (chains / lat_ns)
                            if chains and lat_ns else None},
                # every active state of a step is one 16-byte record gathered by its lane
                # at the step before: the oracle's count of states stepped is the number
                # of random gathers, held against the measured random-gather rates
                "gathers": {"records": int(gate.get("states_stepped", 0)),
                            "achieved_Grecords_per_s":
                                gate.get("states_stepped", 0) / (kernel_ms * 1e-3) / 1e9,
                            "peak_l1_path_Grecords_per_s":
                                onchip.get("l1_gather16_Grecords_per_s") if onchip else None,
                            "peak_l2_only_Grecords_per_s":
                                onchip.get("l2_gather16_Grecords_per_s") if onchip else None,
                            "frac_l1_path": (gate.get("states_stepped", 0) / (kernel_ms * 1e-3)
                                             / 1e9 / onchip["l1_gather16_Grecords_per_s"])
                            if onchip and onchip.get("l1_gather16_Grecords_per_s") else None},
                "onchip_peaks": onchip,
                "note": "algorithmic bytes (per symbol: 1 input byte, 8 per active state, 8 "
                        "per scanned edge) are mostly edge gathers from a 1 MiB table held "
                        "in L1/L2; DRAM carries the input stream"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "u8", "data": "synthetic (seeded; random-walk inputs for live/sustained)",
                "config": {"workload": workload_config(args.workload),
                           "offered_bytes": offered, "examined_bytes": examined_bytes,
                           "l2": "inputs larger than L2 (no flush)",
                           "parallelism": f"replicas x{world}",
                           "technique": f"planned on the device: lane chunks of "
                                        f"{info['lane_chunk_bytes']} B ({info['lane_chunks']} "
                                        f"of {info['chunks']} chunks), overlap-linked "
                                        "parallel fix-up"},
                "phases_ms": phase_ms,
                "step_stats": step_stats(step_samples, offered),
                "e2e": e2e, "e2e_other_ingest": e2e_other, "gpu_launches": launches,
                "oracle_gate": gate,
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clk.summary()}
        line.update(extras)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_batch_section(batch, flags, lens, steps: int = 3) -> dict:
    """The drop-in call with host bytes: ``run_batch(nfa, inputs)`` with the default
    technique (what ``gpufsm.run_batch(nfa, inputs, backend="cuda")`` runs once the plugin
    is installed), wall-clock per call: packing the bytes into pinned memory, planning,
    the copies, the launches and the verdicts back."""
    import abstraction_regret_gb300 as G
    from abstraction_regret_gb300.executors import make_nfa_executor

    nfa = batch.automata[0]
    inputs = batch.inputs()
    res = G.run_batch(nfa, inputs)  # warm-up (executor build, buffers)
    got_f = np.fromiter((r.accepted for r in res), dtype=np.int32, count=len(res))
    got_l = np.fromiter((r.match_len for r in res), dtype=np.int32, count=len(res))
    if not (np.array_equal(got_f, flags) and np.array_equal(got_l, lens)):
        raise SystemExit("run_batch default technique differs from the gated verdicts")
    times, kern = [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        r = G.run_batch(nfa, inputs)
        times.append(time.perf_counter() - t0)
        kern.append(float(r[0].kernel_ms))
    ms = float(np.median(times)) * 1e3
    ex = make_nfa_executor(nfa, "auto")
    ingest = None
    if ex.last_path == "engine":
        eng = ex.engine().engine
        ingest = eng._staging.last_path
        if eng.last_slices:
            ingest += f" in {eng.last_slices} slices, each slice's lanes starting on arrival"
    return {"value": batch.total_bytes / (ms * 1e-3) / 1e9, "unit": "GB/s", "ms": ms,
            "calls": steps, "path": ex.last_path, "ingest": ingest,
            "kernel_ms": float(np.median(kern)),
            "note": "wall clock per call (median), host bytes in, verdicts out; kernel_ms: "
                    "planning and simulation launches, with the gather they overlap when "
                    "the batch is gathered in slices (the rest is host work, the address "
                    "and offset tables, verdicts)"}


def reference_gpu_section(dev, steps: int) -> dict:
    """The reference's own CUDA kernels (built from its sources for sm_103a, oracle/_ref)
    on the same GPU and workloads: dfa_kernel on c2-sustained and worklist_warp_kernel on
    c3-sustained and c1-live, launched as its host functions launch them, with int32
    symbols and offsets; verdicts checked against the oracle."""
    import torch

    from abstraction_regret_gb300 import workloads as W
    from abstraction_regret_gb300.packing import pack_accept
    from oracle import oracle as O
    from oracle import ref_cuda as R

    try:
        dfa_img, wl_img = R.Kernels("dfa"), R.Kernels("worklist_global")
        dfa_fn, wl_fn = dfa_img.fn("dfa_kernel"), wl_img.fn("worklist_warp_kernel")
    except (OSError, RuntimeError, KeyError) as exc:
        return {"unavailable": f"{type(exc).__name__}: {exc}"}
    stream = torch.cuda.current_stream(dev)

    def timed(run, reps):
        run()
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            run()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    out = {"built_from": "src/gpufsm/backends/cuda/native/{dfa,worklist_global}.cu, nvcc "
                         "-cubin sm_103a", "input_layout": "int32 symbols, int32 offsets"}
    b = W.c2("sustained")
    dfa = b.automata[0]
    n = b.n_inputs
    trans = torch.from_numpy(dfa.trans.astype(np.int32)).to(dev)
    acc = torch.from_numpy(dfa.accept.astype(np.int8)).to(dev)
    data = torch.from_numpy(b.data).to(dev).to(torch.int32)
    off = torch.from_numpy(b.offsets.astype(np.int32)).to(dev)
    res = torch.zeros((2, n), dtype=torch.int32, device=dev)
    args = R.dfa_kernel_args(trans.data_ptr(), acc.data_ptr(), data.data_ptr(), off.data_ptr(),
                             n, dfa.num_states, dfa.start_state, res[0].data_ptr(),
                             res[1].data_ptr())
    ms = timed(lambda: R.launch(dfa_fn, (n + 255) // 256, 256, args, stream.cuda_stream), steps)
    of, ol, oe = O.dfa_batch(dfa, b.data, b.offsets)
    h = res.cpu().numpy()
    if not (np.array_equal(h[0], of) and np.array_equal(h[1], ol)):
        raise SystemExit("reference dfa_kernel differs from the oracle on c2-sustained")
    out["dfa_c2_sustained"] = {"kernel": "dfa_kernel", "ms": ms,
                               "offered_GBps": b.total_bytes / (ms * 1e-3) / 1e9,
                               "examined_GBps": int(oe.sum()) / (ms * 1e-3) / 1e9,
                               "checked": int(n)}
    del trans, acc, data, off, res
    for name, batch, reps in (("worklist_warp_c3_sustained", W.c3("sustained"), 1),
                              ("worklist_warp_c1_live", W.c1("live"), steps)):
        nfa = batch.automata[0]
        n = batch.n_inputs
        nwords = (nfa.num_states + 63) // 64
        t = lambda a, dt=torch.int32: torch.from_numpy(np.ascontiguousarray(a).astype(  # noqa: E731
            np.int32 if dt == torch.int32 else np.int64)).to(dev)
        srp, stg, ssy = t(nfa.sym_row_ptr), t(nfa.sym_targets), t(nfa.sym_symbols)
        erp, etg = t(nfa.eps_row_ptr), t(nfa.eps_targets)
        if etg.numel() == 0:
            etg = torch.zeros(1, dtype=torch.int32, device=dev)
        words = torch.from_numpy(pack_accept(nfa).view(np.int64)).to(dev)
        data = torch.from_numpy(batch.data).to(dev).to(torch.int32)
        off = torch.from_numpy(batch.offsets.astype(np.int32)).to(dev)
        bufs = torch.zeros((4, n * nwords), dtype=torch.int64, device=dev)
        res = torch.zeros((2, n), dtype=torch.int32, device=dev)
        args = R.worklist_warp_args(srp.data_ptr(), stg.data_ptr(), ssy.data_ptr(),
                                    erp.data_ptr(), etg.data_ptr(), words.data_ptr(),
                                    data.data_ptr(), off.data_ptr(), n, nfa.start_state,
                                    int(nfa.uses_any_symbol), nwords, bufs[0].data_ptr(),
                                    bufs[1].data_ptr(), bufs[2].data_ptr(), bufs[3].data_ptr(),
                                    res[0].data_ptr(), res[1].data_ptr())
        ms = timed(lambda: R.launch(wl_fn, (n * 32 + 255) // 256, 256, args,
                                    stream.cuda_stream), reps)
        f, l, ex, _ = O.nfa_batch(nfa, batch.data, batch.offsets)
        h = res.cpu().numpy()
        if not (np.array_equal(h[0], f) and np.array_equal(h[1], l)):
            raise SystemExit(f"reference worklist_warp_kernel differs from the oracle ({name})")
        out[name] = {"kernel": "worklist_warp_kernel", "ms": ms,
                     "offered_GBps": batch.total_bytes / (ms * 1e-3) / 1e9,
                     "examined_GBps": int(ex.sum()) / (ms * 1e-3) / 1e9, "checked": int(n)}
        del srp, stg, ssy, erp, etg, words, data, off, bufs, res
    return out


def launch_phases(runner) -> dict:
    """Device time of each launch of one engine step (CUDA events around each)."""
    import torch

    phases: dict = {}
    with torch.cuda.stream(runner.stream):
        runner.kernel_only(runner.stream, phases=phases)
    runner.stream.synchronize()
    return {k: ev[0].elapsed_time(ev[1]) for k, ev in phases.items() if len(ev) >= 2}


def c1_section(dev, steps: int) -> dict:
    """c1: the 1024-state NFA on 64 inputs of 4 KiB (live and sustained random walks;
    the literal inputs die after about one byte), one engine step and one plain launch,
    both checked against the oracle first."""
    import torch

    from abstraction_regret_gb300 import workloads as W
    from abstraction_regret_gb300.engine import GraphRunner, PersistentEngine
    from abstraction_regret_gb300.executors import CudaNFAExecutor
    from oracle import oracle as O

    out = {}
    for variant in ("live", "sustained"):
        b = W.c1(variant)
        nfa = b.automata[0]
        of, ol, oe, _, work, visits = O.nfa_batch(nfa, b.data, b.offsets, with_work=True)
        r = GraphRunner(PersistentEngine([nfa], dev), b.aut_ids, b.data, b.offsets,
                        with_examined=True)
        with torch.cuda.stream(r.stream):
            r.replay()
        r.stream.synchronize()
        f, l, ex = r.verdicts()
        if not (np.array_equal(f, of) and np.array_equal(l, ol) and np.array_equal(ex, oe)):
            raise SystemExit(f"c1-{variant}: engine differs from the oracle")
        with torch.cuda.stream(r.stream):
            ms = time_launches(lambda: r.kernel_only(r.stream), r.stream, steps, 3)
        phases = launch_phases(r)
        plain = CudaNFAExecutor(nfa, "auto", dev)
        d_out = torch.zeros((3, b.n_inputs), dtype=torch.int32, device=dev)
        with torch.cuda.stream(r.stream):
            plain_ms = time_launches(lambda: plain.launch(r.d_data, r.d_off, b.n_inputs,
                                                          d_out[0], d_out[1], None, r.stream),
                                     r.stream, steps, 3)
        if not np.array_equal(d_out[0].cpu().numpy(), of):
            raise SystemExit(f"c1-{variant}: plain launch differs from the oracle")
        info = r.plan_info()
        out[variant] = {"engine_GBps": b.total_bytes / (ms * 1e-3) / 1e9, "engine_ms": ms,
                        "phases_ms": phases,
                        "plain_GBps": b.total_bytes / (plain_ms * 1e-3) / 1e9,
                        "plain_ms": plain_ms, "offered_bytes": int(b.total_bytes),
                        "checked": int(f.size),
                        "cpu_baseline": cpu_port(
                            lambda t: O.nfa_batch(nfa, b.data, b.offsets, t),
                            b.total_bytes, f"c1-{variant} (64 x 4 KiB)"),
                        "_counts": {"examined": int(oe.sum()), "states": int(visits.sum()),
                                    "edges": int(work.sum()), "n": int(b.n_inputs),
                                    "chains": int(info["lane_chunks"] or b.n_inputs)}}
        del r, plain
    return out


def c4_section(dev, steps: int) -> dict:
    """c4: 64 NFAs of 256..65536 states, 16 inputs each, one persistent engine step per
    batch (live and sustained random-walk inputs), against one plain launch per
    automaton; bit-exact against the oracle on all 1024 pairs first."""
    import torch

    from abstraction_regret_gb300 import workloads as W
    from abstraction_regret_gb300.engine import GraphRunner, PersistentEngine
    from abstraction_regret_gb300.executors import make_nfa_executor
    from oracle import oracle as O

    out = {}
    for variant in ("live", "sustained"):
        b = W.c4(variant)
        eng = PersistentEngine(b.automata, dev)
        r = GraphRunner(eng, b.aut_ids, b.data, b.offsets, with_examined=True)
        with torch.cuda.stream(r.stream):
            r.replay()
        r.stream.synchronize()
        f, l, ex = r.verdicts()
        counts = {"examined": 0, "states": 0, "edges": 0, "n": int(b.n_inputs)}
        subsets = []
        for k, a in enumerate(b.automata):
            sel = np.flatnonzero(b.aut_ids == k)
            sub = b.subset(sel)
            subsets.append((a, sub))
            of, ol, oe, _, work, visits = O.nfa_batch(a, sub.data, sub.offsets, with_work=True)
            counts["examined"] += int(oe.sum())
            counts["states"] += int(visits.sum())
            counts["edges"] += int(work.sum())
            if not (np.array_equal(f[sel], of) and np.array_equal(l[sel], ol)
                    and np.array_equal(ex[sel], oe)):
                raise SystemExit(f"c4-{variant}: automaton {k} differs from the oracle")
        with torch.cuda.stream(r.stream):
            ms = time_launches(lambda: r.kernel_only(r.stream), r.stream, steps, 3)
        phases = launch_phases(r)
        # plain: one launch per automaton (its 16 inputs), back to back on one stream
        plains, subs = [], []
        for k, a in enumerate(b.automata):
            sel = np.flatnonzero(b.aut_ids == k)
            plains.append(make_nfa_executor(a, "auto"))
            lo, hi = int(b.offsets[sel[0]]), int(b.offsets[sel[-1] + 1])
            subs.append((r.d_data[lo:], torch.from_numpy(b.offsets[sel[0]:sel[-1] + 2] - lo)
                         .to(dev), sel.size))
        d_out = torch.zeros((3, 16), dtype=torch.int32, device=dev)

        def plain_all():
            for ex_, (d, off, n) in zip(plains, subs):
                ex_.launch(d, off, n, d_out[0], d_out[1], None, r.stream)

        with torch.cuda.stream(r.stream):
            plain_ms = time_launches(plain_all, r.stream, 1, 1)
        info = r.plan_info()
        counts["chains"] = int(info["lane_chunks"] + info["persistent_tasks"])

        def cpu_pass(t, subsets=subsets):
            for a_, sub_ in subsets:
                O.nfa_batch(a_, sub_.data, sub_.offsets, t)

        out[variant] = {"offered_GBps": b.total_bytes / (ms * 1e-3) / 1e9,
                        "examined_GBps": int(ex.sum()) / (ms * 1e-3) / 1e9, "ms": ms,
                        "phases_ms": phases, "plan": r.plan_info(),
                        "plain_per_automaton_ms": plain_ms,
                        "speedup_vs_plain_per_automaton": plain_ms / ms,
                        "offered_bytes": int(b.total_bytes), "checked": int(f.size),
                        "cpu_baseline": cpu_port(cpu_pass, b.total_bytes,
                                                 f"c4-{variant} (64 NFAs x 16 inputs)"),
                        "_counts": counts}
        del r, eng, plains
    return out


def dfa_chunks_section(dev, steps: int) -> dict:
    """Chunked DFA walks (DFA_CHUNK / DFA_FIXUP tasks) against whole-input walks (one lane
    per input) in one engine step, no accepting state: 64 inputs of 4 MiB on the c2 DFA
    (4096 states); one 4 MiB input on a 16384-state DFA (the latency of a lone long
    request); c2-sustained itself (4096 inputs of 64 KiB: the engine's own choice, which
    runs them whole) and with 16 KiB chunks forced. Verdicts and examined counts
    bit-exact against the oracle first; device time per step (planning included)."""
    import torch

    from abstraction_regret_gb300 import engine as E
    from abstraction_regret_gb300 import workloads as W
    from abstraction_regret_gb300.engine import GraphRunner, PersistentEngine
    from oracle import oracle as O

    from abstraction_regret_gb300.automata import random_dfa

    c2 = W.c2("sustained")
    long_n, long_len = 64, 4 << 20
    big = random_dfa(16384, accept_prob=0.0, seed=17)
    cases = {
        "long_4MiB": (c2.automata[0], W.offsets_of(np.full(long_n, long_len, dtype=np.int64)),
                      W.uniform_bytes([1, 3], long_n * long_len), None),
        "one_4MiB_16384_states": (big, np.array([0, long_len], np.int64),
                                  W.uniform_bytes([1, 5], long_len), None),
        "c2_sustained": (c2.automata[0], c2.offsets, c2.data, None),
        "c2_sustained_16KiB": (c2.automata[0], c2.offsets, c2.data, 16 << 10),
    }
    out = {}
    for name, (dfa, offsets, data, forced) in cases.items():
        of, ol, oe = O.dfa_batch(dfa, data, offsets)
        row = {"inputs": int(len(offsets) - 1), "bytes": int(offsets[-1])}
        for mode, chunk in (("chunked", forced), ("whole", 0)):
            eng = PersistentEngine([dfa], dev, dfa_chunk_bytes=chunk)
            r = GraphRunner(eng, np.zeros(len(offsets) - 1, np.int64), data, offsets,
                            with_examined=True)
            with torch.cuda.stream(r.stream):
                r.replay()
            r.stream.synchronize()
            f, l, ex = r.verdicts()
            if not (np.array_equal(f, of) and np.array_equal(l, ol) and np.array_equal(ex, oe)):
                raise SystemExit(f"DFA chunks {name}/{mode}: verdicts differ from the oracle")
            info = r.plan_info()
            with torch.cuda.stream(r.stream):
                ms = time_launches(lambda: r.kernel_only(r.stream), r.stream,
                                   steps if mode == "chunked" else 1, 1)
            phases: dict = {}
            with torch.cuda.stream(r.stream):
                r.kernel_only(r.stream, phases=phases)
            r.stream.synchronize()
            row[mode] = {"ms": ms, "GBps": int(offsets[-1]) / (ms * 1e-3) / 1e9,
                         "dfa_chunks": info.get("dfa_chunks", 0),
                         "min_chunk_bytes": int(eng.dfa_chunk[0]),
                         "batch_chunk_bytes": info.get("dfa_chunk_bytes", 0),
                         "phases_ms": {k: ev[0].elapsed_time(ev[1]) for k, ev in phases.items()
                                       if len(ev) >= 2}}
            del r, eng
        row["speedup"] = row["whole"]["ms"] / row["chunked"]["ms"]
        row["states"] = int(dfa.num_states)
        out[name] = row
    return out


def serving_section(dev, n_requests: int, slo_ms: float) -> dict:
    """c5: the serving loop over the resident 32-automaton pool at swept arrival rates,
    against one plain launch per request; verdicts equal to the plain path on every
    request and to the oracle on a sample."""
    import torch

    from abstraction_regret_gb300 import workloads as W
    from abstraction_regret_gb300.engine import PersistentEngine
    from abstraction_regret_gb300.executors import make_dfa_executor, make_nfa_executor
    from abstraction_regret_gb300.serving import Server, serve_plain
    from oracle import oracle as O

    pool = W.c5_pool()
    engine = PersistentEngine(pool, dev)
    out = {"pool": "16 NFAs (c4 distribution) + 16 DFAs (1024..16384 states)",
           "requests": n_requests, "slo_p99_ms": slo_ms, "rates": []}
    base = W.c5(rate_per_s=1.0, n_requests=n_requests, automata=pool)
    pinned = torch.from_numpy(base.pool).pin_memory()
    # plain baseline: one launch per request, arrivals ignored (back to back)
    ex = {k: (make_dfa_executor(a, "gather") if hasattr(a, "trans") else
              make_nfa_executor(a, "compact")) for k, a in enumerate(pool)}
    pf, pl, plat, pstats = serve_plain(engine, base, ex, time_scale=0.0)
    out["plain_per_request"] = {"offered_GBps": pstats.offered_GBps, "wall_s": pstats.wall_s,
                                "note": "one plain launch per request, back to back"}
    # oracle on a sample of requests
    rng = np.random.default_rng(0)
    sample = rng.choice(n_requests, min(400, n_requests), replace=False)
    for i in sample:
        a, data = base.request(int(i))
        want = O.verdicts(pool[a], [bytes(data)])[0]
        if (int(pf[i]), int(pl[i])) != (int(want[0]), int(want[1])):
            raise SystemExit(f"serving: plain path disagrees with the oracle on request {i}")
    # swept Poisson rates, then every request at once (the loop's saturation throughput)
    for rate in (2000.0, 8000.0, 32000.0, 128000.0, None):
        tr = dataclasses.replace(base, arrivals=base.arrivals / (rate or 1.0))
        srv = Server(engine=engine, slots=3, batch_bytes=256 << 20, max_requests=4096,
                     zero_copy=True)
        warm = dataclasses.replace(tr, aut_ids=tr.aut_ids[:256], arrivals=tr.arrivals[:256],
                                   starts=tr.starts[:256], lengths=tr.lengths[:256])
        srv.serve(warm, time_scale=0.0, pinned_pool=pinned)  # untimed warm-up
        f, l, lat, st = srv.serve(tr, time_scale=1.0 if rate else 0.0, pinned_pool=pinned)
        if not (np.array_equal(f, pf) and np.array_equal(l, pl)):
            raise SystemExit(f"serving at {rate}/s: verdicts differ from the plain path")
        d = st.as_dict()
        d.update({"rate_per_s": rate if rate else "all at t=0",
                  "slo_met": bool(st.p99_ms <= slo_ms)})
        out["rates"].append(d)
        del srv
    out["checked"] = {"plain_equal": n_requests, "oracle_sample": int(sample.size)}
    # live and sustained traces: random-walk NFA requests (and, sustained, every accept
    # bit cleared), so the simulations examine the bytes instead of dying or latching
    out["examined_traces"] = {}
    for variant in ("live", "sustained"):
        base = W.c5(rate_per_s=1.0, n_requests=n_requests, automata=pool, variant=variant)
        eng = engine if variant == "live" else PersistentEngine(base.automata, dev)
        pinned = torch.from_numpy(base.pool).pin_memory()
        runs, first = [], None
        # the sustained trace also runs its first 2000 requests at lower rates, to find
        # where every-byte-examined load meets the SLO
        rates = (8000.0, 32000.0, None) + ((2000.0, 500.0) if variant == "sustained" else ())
        for rate in rates:
            # the same requests; only the arrival times scale with the rate
            k = n_requests if rate is None or rate >= 8000.0 else min(n_requests, 2000)
            tr = dataclasses.replace(base, arrivals=base.arrivals[:k] / (rate or 1.0),
                                     aut_ids=base.aut_ids[:k], starts=base.starts[:k],
                                     lengths=base.lengths[:k])
            srv = Server(engine=eng, slots=3, batch_bytes=256 << 20, max_requests=4096,
                         zero_copy=True)
            warm = dataclasses.replace(tr, aut_ids=tr.aut_ids[:256], arrivals=tr.arrivals[:256],
                                       starts=tr.starts[:256], lengths=tr.lengths[:256])
            srv.serve(warm, time_scale=0.0, pinned_pool=pinned)  # untimed warm-up
            f, l, lat, st = srv.serve(tr, time_scale=1.0 if rate else 0.0, pinned_pool=pinned)
            if first is None:
                first = (f, l)
                for i in sample[:200]:
                    a, data = base.request(int(i))
                    want = O.verdicts(base.automata[a], [bytes(data)])[0]
                    if (int(f[i]), int(l[i])) != (int(want[0]), int(want[1])):
                        raise SystemExit(f"serving {variant}: request {i} differs from the oracle")
            elif not (np.array_equal(f, first[0][:k]) and np.array_equal(l, first[1][:k])):
                raise SystemExit(f"serving {variant} at {rate}/s: verdicts changed")
            d = st.as_dict()
            d.update({"rate_per_s": rate if rate else "all at t=0",
                      "slo_met": bool(st.p99_ms <= slo_ms)})
            runs.append(d)
            del srv
        out["examined_traces"][variant] = {
            "trace": ("NFA requests: prefixes of random walks of their automaton; DFA "
                      "requests: uniform bytes" + ("; every accept bit cleared"
                                                   if variant == "sustained" else "")),
            "rates": runs, "oracle_sample": 200}
        del pinned, base
    return out


class GraphRunnerLike:
    """Resident-input timing helper for a plain DFA executor."""

    def __init__(self, executor, batch, dev):
        import torch

        self.ex = executor
        self.batch = batch
        total = batch.total_bytes
        padded = -(-total // 16) * 16 + 16
        self.d_data = torch.zeros(padded, dtype=torch.uint8, device=dev)
        self.d_data[:total].copy_(torch.from_numpy(batch.data[:total]))
        self.d_off = torch.from_numpy(batch.offsets.copy()).to(dev)
        self.out = torch.zeros((3, batch.n_inputs), dtype=torch.int32, device=dev)

    def launch(self, stream):
        self.ex.launch(self.d_data, self.d_off, self.batch.n_inputs, self.out[0], self.out[1],
                       self.out[2], stream)

    def time(self, stream, steps):
        import torch

        with torch.cuda.stream(stream):
            return time_launches(lambda: self.launch(stream), stream, steps, 3)

    def verdicts(self):
        h = self.out.cpu().numpy()
        return h[0], h[1], h[2]


if __name__ == "__main__":
    raise SystemExit(main())
