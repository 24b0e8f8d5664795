"""Serving loop: continuous batching over a resident pool of NFAs and DFAs (GPU).

Checks that every request's verdict is the oracle's, that it is the same when the
request runs alone (its own launch) and in the mix (batched with whatever arrived
around it, on overlapping slots), and that both ingest modes agree.
"""

from __future__ import annotations

import numpy as np
import pytest

from abstraction_regret_gb300 import workloads as W
from abstraction_regret_gb300.engine import PersistentEngine
from abstraction_regret_gb300.serving import Server, serve_plain
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    pool = W.c5_pool()
    trace = W.c5(rate_per_s=20000.0, n_requests=600, pool_bytes=1 << 22, automata=pool)
    engine = PersistentEngine(pool)
    want_f = np.zeros(len(trace.aut_ids), np.int32)
    want_l = np.zeros(len(trace.aut_ids), np.int32)
    for k, a in enumerate(pool):
        sel = np.flatnonzero(trace.aut_ids == k)
        got = O.verdicts(a, [bytes(trace.request(int(i))[1]) for i in sel])
        for i, (f, l) in zip(sel, got):
            want_f[i], want_l[i] = int(f), l
    return pool, trace, engine, want_f, want_l


@pytest.mark.parametrize("zero_copy", [False, True])
def test_served_verdicts_match_the_oracle(setup, zero_copy):
    pool, trace, engine, want_f, want_l = setup
    srv = Server(engine=engine, slots=3, batch_bytes=16 << 20, max_requests=256,
                 zero_copy=zero_copy)
    flags, lens, lat, stats = srv.serve(trace)
    assert np.array_equal(flags, want_f) and np.array_equal(lens, want_l)
    assert stats.rejected == 0 and stats.batches >= 2
    assert (lat >= 0).all() and stats.p99_ms >= stats.p50_ms


def test_same_alone_and_in_the_mix(setup):
    pool, trace, engine, want_f, want_l = setup
    srv = Server(engine=engine, slots=2, batch_bytes=8 << 20, max_requests=128)
    flags, lens, _, stats = srv.serve(trace, time_scale=0.25)  # denser arrivals: bigger mixes
    assert stats.mean_batch > 1.0
    rng = np.random.default_rng(0)
    for i in rng.choice(len(trace.aut_ids), 60, replace=False):
        a, data = trace.request(int(i))
        f, l, _, _, _ = engine.run_requests([a], [bytes(data)])
        assert (f[0], l[0]) == (flags[i], lens[i]) == (want_f[i], want_l[i])


def test_plain_per_request_baseline_agrees(setup):
    pool, trace, engine, want_f, want_l = setup
    from abstraction_regret_gb300.executors import make_dfa_executor, make_nfa_executor

    ex = {k: (make_dfa_executor(a, "gather") if hasattr(a, "trans") else
              make_nfa_executor(a, "compact")) for k, a in enumerate(pool)}
    sub = W.ServingTrace(pool, trace.aut_ids[:100], trace.arrivals[:100], trace.pool,
                         trace.starts[:100], trace.lengths[:100])
    flags, lens, _, stats = serve_plain(engine, sub, ex)
    assert np.array_equal(flags, want_f[:100]) and np.array_equal(lens, want_l[:100])
    assert stats.batches == 100


def test_live_trace_served_alone_and_in_the_mix():
    """The live trace (random-walk NFA requests, whose sets stay alive for many
    kilobytes): verdicts and examined bytes equal the oracle's, batched and alone."""
    pool = W.c5_pool()
    trace = W.c5(rate_per_s=20000.0, n_requests=400, pool_bytes=1 << 22, automata=pool,
                 variant="live", walks_per_nfa=2)
    engine = PersistentEngine(pool)
    srv = Server(engine=engine, slots=3, batch_bytes=32 << 20, max_requests=256,
                 zero_copy=True)
    flags, lens, _, stats = srv.serve(trace, time_scale=0.25)
    want, examined = [], 0
    for i in range(len(trace.aut_ids)):
        a, data = trace.request(i)
        d, off = O.flatten([bytes(data)])
        if hasattr(pool[a], "trans"):
            f, l, e = O.dfa_batch(pool[a], d, off)
        else:
            f, l, e, _ = O.nfa_batch(pool[a], d, off)
        want.append((int(f[0]), int(l[0])))
        examined += int(e[0])
    assert list(zip(flags.tolist(), lens.tolist())) == want
    assert stats.examined_bytes == examined and examined > stats.offered_bytes // 20
    rng = np.random.default_rng(1)
    for i in rng.choice(len(trace.aut_ids), 40, replace=False):
        a, data = trace.request(int(i))
        f, l, _, _, _ = engine.run_requests([a], [bytes(data)])
        assert (int(f[0]), int(l[0])) == want[i]


def test_sustained_trace_chunks_long_dfa_requests():
    """The sustained trace (every accept bit cleared, every byte examined): long DFA
    requests are walked in chunks inside the serving batches, and every verdict and the
    examined total equal the oracle's."""
    pool = W.c5_pool()
    trace = W.c5(rate_per_s=20000.0, n_requests=300, pool_bytes=1 << 24, automata=pool,
                 variant="sustained", walks_per_nfa=2)
    engine = PersistentEngine(trace.automata)
    assert engine.aut_dfa_chunk is not None
    srv = Server(engine=engine, slots=2, batch_bytes=64 << 20, max_requests=256,
                 zero_copy=True)
    flags, lens, _, stats = srv.serve(trace, time_scale=0.25)
    examined = 0
    long_dfa = 0
    for i in range(len(trace.aut_ids)):
        a, data = trace.request(i)
        d, off = O.flatten([bytes(data)])
        if hasattr(trace.automata[a], "trans"):
            f, l, e = O.dfa_batch(trace.automata[a], d, off)
            long_dfa += len(data) >= 2 * engine.dfa_chunk[a]
        else:
            f, l, e, _ = O.nfa_batch(trace.automata[a], d, off)
        assert (int(flags[i]), int(lens[i])) == (int(f[0]), int(l[0])), i
        examined += int(e[0])
    assert long_dfa > 0
    assert stats.examined_bytes == examined == stats.offered_bytes
