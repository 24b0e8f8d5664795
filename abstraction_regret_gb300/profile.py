"""One small step of a named workload, for a profiler to capture.

    python -m abstraction_regret_gb300.profile CASE [--steps N]

Each case builds its batch, checks the verdicts of its first step against the oracle
(the process exits non-zero on a difference), then runs ``--steps`` more steps and
exits. Sizes are chosen so that a capture of every launch ends in seconds while the
inputs stay larger than L2 where the case's kernel streams them:

* ``c1-live``        the engine on c1 (1024-state NFA, 64 x 4 KiB random walks);
* ``c1-plain``       the plain warp-per-input launch (``nfa_warp_kernel``) on c1;
* ``c2-sustained``   the DFA cluster walk on c2-sustained (4096 x 64 KiB);
* ``c4-sustained``   the engine on c4-sustained (64 NFAs, 1024 inputs; lanes and
                     persistent launches);
* ``dfa-long``       chunked DFA walks (``dfa_chunks_kernel``): 8 inputs of 2 MiB on
                     the c2 DFA (4096 states, no accepting state);
* ``c5-live``        the serving loop over the c5 pool (16 NFAs, 16 DFAs): the first
                     2000 requests of the live trace, all arriving at once (the oracle
                     checks 100 of them);
* ``c3-warps``       the engine on the first 512 inputs of c3-sustained with lane chunks
                     turned off, so that warp chunks in ``persistent_kernel`` do the work
                     (the design the lane launch replaced);
* ``gather``         the batch gather (``gather_inputs_kernel``) of the first 1024
                     c3-sustained inputs as Python ``bytes`` (130 MB, read in place from
                     pageable host memory); the device buffer is checked byte for byte
                     against the packed batch instead of the oracle;
* ``run-batch``      the drop-in call ``run_batch(nfa, inputs)`` on c3-sustained with
                     Python ``bytes`` and the default technique (gather, planning, lanes,
                     fix-up, verdicts); ``--time`` prints its wall clock per call.
"""

from __future__ import annotations

import argparse
import sys

import numpy as np


def _check(name, got, want) -> None:
    for g, w, what in zip(got, want, ("flags", "lens", "examined")):
        if g is not None and not np.array_equal(np.asarray(g), np.asarray(w)):
            raise SystemExit(f"{name}: {what} differ from the oracle")


def run(case: str, steps: int) -> float | None:
    """Run the case; returns the mean device time (ms) of its timed engine steps, when
    it has any."""
    import torch

    from oracle import oracle as O

    from . import workloads as W
    from .engine import GraphRunner, PersistentEngine
    from .executors import CudaDFAExecutor, CudaNFAExecutor

    dev = torch.device("cuda", torch.cuda.current_device())
    if case == "run-batch":
        import time

        from .api import run_batch

        b = W.c3("sustained")
        nfa, inputs = b.automata[0], b.inputs()
        res = run_batch(nfa, inputs)
        want = O.nfa_batch(nfa, b.data, b.offsets)[:2]
        _check(case, ([r.accepted for r in res], [r.match_len for r in res]), want)
        t0 = time.perf_counter()
        for _ in range(steps):
            run_batch(nfa, inputs)
        return (time.perf_counter() - t0) * 1e3 / steps if steps else None
    if case == "gather":
        from .staging import Staging

        b = W.c3("sustained").subset(np.arange(1024))
        inputs = b.inputs()
        st = Staging(dev, gather=True)
        stream = torch.cuda.current_stream(dev)
        d_data, _, _, total = st.put(inputs, stream)
        stream.synchronize()
        if not np.array_equal(d_data[:total].cpu().numpy(), b.data[:total]):
            raise SystemExit("gather: the device buffer differs from the packed batch")
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            st.put(inputs, stream)
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / steps if steps else None
    if case == "c5-live":
        from .serving import Server

        k = 2000
        t = W.c5(rate_per_s=1.0, n_requests=k, variant="live")
        eng = PersistentEngine(t.automata, dev)
        pinned = torch.from_numpy(t.pool).pin_memory()
        for step in range(1 + steps):
            srv = Server(engine=eng, slots=3, batch_bytes=256 << 20, max_requests=4096,
                         zero_copy=True)
            f, l, _, _ = srv.serve(t, time_scale=0.0, pinned_pool=pinned)
            if step == 0:
                for i in range(0, k, k // 100):
                    a, data = t.request(i)
                    want = O.verdicts(t.automata[a], [bytes(data)])[0]
                    if (int(f[i]), int(l[i])) != (int(want[0]), int(want[1])):
                        raise SystemExit(f"c5-live: request {i} differs from the oracle")
        return
    if case in ("c1-live", "c4-sustained", "dfa-long", "c3-warps"):
        choices = None
        if case == "c1-live":
            b = W.c1("live")
        elif case == "c4-sustained":
            b = W.c4("sustained")
        elif case == "c3-warps":
            from .engine import NfaChoice

            b = W.c3("sustained", n_inputs=512)
            choices = [NfaChoice(lanes=False)]
        else:
            b = W.c2("sustained")
            n, length = 8, 2 << 20
            b = W.Batch("dfa-long", b.automata, np.zeros(n, np.int64),
                        W.uniform_bytes([1, 4], n * length),
                        W.offsets_of(np.full(n, length, dtype=np.int64)), {})
        r = GraphRunner(PersistentEngine(b.automata, dev, choices=choices), b.aut_ids, b.data,
                        b.offsets, with_examined=True)
        with torch.cuda.stream(r.stream):
            r.replay()
        r.stream.synchronize()
        got = r.verdicts()
        want = [np.zeros(b.n_inputs, np.int64) for _ in range(3)]
        for k, a in enumerate(b.automata):
            sel = np.flatnonzero(b.aut_ids == k)
            if sel.size == 0:
                continue
            sub = b.subset(sel)
            res = O.dfa_batch(a, sub.data, sub.offsets) if case == "dfa-long" else \
                O.nfa_batch(a, sub.data, sub.offsets)[:3]
            for w, v in zip(want, res):
                w[sel] = v
        _check(case, got, want)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(r.stream):
            e0.record(r.stream)
            for _ in range(steps):
                r.kernel_only(r.stream)
            e1.record(r.stream)
        r.stream.synchronize()
        return e0.elapsed_time(e1) / steps if steps else None
    if case == "c1-plain":
        b = W.c1("live")
        ex = CudaNFAExecutor(b.automata[0], "auto", dev)
        want = O.nfa_batch(b.automata[0], b.data, b.offsets)[:2]
    elif case == "c2-sustained":
        b = W.c2("sustained")
        ex = CudaDFAExecutor(b.automata[0], device=dev)
        want = O.dfa_batch(b.automata[0], b.data, b.offsets)[:2]
    else:
        raise SystemExit(f"unknown case {case!r}")
    stream = torch.cuda.current_stream(dev)
    d = torch.from_numpy(b.data).to(dev)
    off = torch.from_numpy(b.offsets).to(dev)
    out = torch.zeros((2, b.n_inputs), dtype=torch.int32, device=dev)
    ex.launch(d, off, b.n_inputs, out[0], out[1], None, stream)
    stream.synchronize()
    _check(case, (out[0].cpu().numpy(), out[1].cpu().numpy()), want)
    for _ in range(steps):
        ex.launch(d, off, b.n_inputs, out[0], out[1], None, stream)
    stream.synchronize()


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("case", choices=["c1-live", "c1-plain", "c2-sustained", "c4-sustained",
                                     "dfa-long", "c5-live", "c3-warps", "gather",
                                     "run-batch"])
    ap.add_argument("--time", action="store_true",
                    help="also print the mean device time of the timed steps")
    ap.add_argument("--steps", type=int, default=2)
    args = ap.parse_args(argv)
    ms = run(args.case, args.steps)
    checked = "device buffer equal to the packed batch" if args.case == "gather" else \
        "verdicts equal to the oracle"
    print(f"{args.case}: {checked}; {args.steps} more steps run")
    if args.time and ms is not None:
        what = "call (wall clock)" if args.case == "run-batch" else "engine step"
        print(f"{args.case}: {ms:.4f} ms per {what} (mean of {args.steps})")
    return 0


if __name__ == "__main__":
    sys.exit(main())
