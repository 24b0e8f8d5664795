"""Time the reference's own CPU path, ``gpufsm.run_batch(..., backend="cpu")``, one core.

    python oracle/time_reference_cpu.py --reference /root/reference

The reference package (gpufsm 0.1.0) is pure Python and runs single-threaded
(``api.run_batch`` loops ``run``, src/gpufsm/api.py:54-62; ``backends/cpu.py:28-32``
registers ``reference`` and, for NFAs, ``bitmap``). It is imported from its checkout, so
this runs where the checkout is (the development container), not on the GPU machines.
For each workload it times a fixed deterministic sample -- the first inputs of the batch,
cut to a byte budget -- checks the verdicts against this repository's oracle, and prints
one JSON line per (workload, technique) with the examined bytes per second: on one core,
and fanned out over one process per host core (inputs dealt round-robin; the worker
processes are started and loaded before the clock starts).
"""

from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))


_W = {}


def _init(reference: str, automaton, inputs) -> None:
    sys.path.insert(0, str(Path(reference) / "src"))
    import gpufsm

    _W.update(gpufsm=gpufsm, automaton=automaton, inputs=inputs)


def _run(job):
    tech, idx = job
    res = _W["gpufsm"].run_batch(_W["automaton"], [_W["inputs"][i] for i in idx],
                                 backend="cpu", technique=tech)
    return [(i, r.accepted, r.match_len) for i, r in zip(idx, res)]


def fan_out(reference: str, automaton, inputs, tech: str, procs: int):
    """Seconds for all inputs over ``procs`` worker processes, and their verdicts."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    jobs = [(tech, list(range(k, len(inputs), procs))) for k in range(procs)]
    with ctx.Pool(procs, initializer=_init, initargs=(reference, automaton, inputs)) as pool:
        pool.map(_run, [(tech, []) for _ in range(procs)])  # every worker loaded
        t0 = time.perf_counter()
        parts = pool.map(_run, jobs)
        dt = time.perf_counter() - t0
    got = [None] * len(inputs)
    for part in parts:
        for i, a, m in part:
            got[i] = (a, m)
    return dt, got


def sample(batch, budget: int, cap: int):
    out, used = [], 0
    for i in range(batch.n_inputs):
        x = batch.data[batch.offsets[i]:batch.offsets[i + 1]][:cap].tobytes()
        if used + len(x) > budget:
            break
        out.append(x)
        used += len(x)
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--budget", type=int, default=1 << 18, help="bytes per sample")
    args = ap.parse_args()
    sys.path.insert(0, str(Path(args.reference) / "src"))
    import gpufsm

    from abstraction_regret_gb300 import workloads as W
    from oracle import oracle as O

    cases = [("c3-sustained", W.c3("sustained", n_inputs=64, walk=O.walk_bytes),
              ("reference", "bitmap")),
             ("c1-live", W.c1("live", walk=O.walk_bytes), ("reference", "bitmap")),
             ("c2-sustained", W.c2("sustained", n_inputs=8), ("reference",))]
    for name, batch, techs in cases:
        a = batch.automata[0]
        if hasattr(a, "trans"):
            ref = gpufsm.DFA(num_states=a.num_states, start_state=a.start_state,
                             accept=np.asarray(a.accept), trans=np.asarray(a.trans))
        else:
            ref = gpufsm.NFA(num_states=a.num_states, start_state=a.start_state,
                             accept=np.asarray(a.accept), sym_row_ptr=a.sym_row_ptr,
                             sym_targets=a.sym_targets, sym_symbols=a.sym_symbols,
                             eps_row_ptr=a.eps_row_ptr, eps_targets=a.eps_targets)
        inputs = sample(batch, args.budget, 1 << 16)
        want = O.verdicts(a, inputs)
        data, off = O.flatten(inputs)
        examined = int((O.dfa_batch(a, data, off)[2] if hasattr(a, "trans")
                        else O.nfa_batch(a, data, off)[2]).sum())
        for tech in techs:
            t0 = time.perf_counter()
            res = gpufsm.run_batch(ref, inputs, backend="cpu", technique=tech)
            dt = time.perf_counter() - t0
            got = [(r.accepted, r.match_len) for r in res]
            assert got == want, f"{name}/{tech}: the reference disagrees with the oracle"
            print(json.dumps({"workload": name, "technique": tech, "inputs": len(inputs),
                              "bytes": int(off[-1]), "examined": examined, "seconds": dt,
                              "examined_MBps": examined / dt / 1e6, "cores": 1,
                              "host": platform.processor() or platform.machine(),
                              "cpus": os.cpu_count()}), flush=True)
            procs = os.cpu_count() or 1
            dt, got = fan_out(args.reference, ref, inputs, tech, procs)
            assert got == want, f"{name}/{tech}: the fan-out disagrees with the oracle"
            print(json.dumps({"workload": name, "technique": tech, "inputs": len(inputs),
                              "bytes": int(off[-1]), "examined": examined, "seconds": dt,
                              "examined_MBps": examined / dt / 1e6, "cores": procs,
                              "processes": procs, "host": platform.processor() or
                              platform.machine(), "cpus": os.cpu_count()}), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
