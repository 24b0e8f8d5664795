"""Ingest that the GPU drives: inputs copied from the caller's own buffers (GPU).

On a device that reads pageable host memory (GB300 over NVLink-C2C), ``Staging`` lets
``gbfsm_gather_inputs`` read every input where it lies -- Python ``bytes``, ``bytearray``,
``memoryview`` slices at any alignment, numpy arrays -- instead of packing the batch on
the host. The device buffer must be byte for byte the packed one -- gathered whole or as
ranges of inputs on streams of their own -- and the verdicts the oracle's, also when the
engine gathers a batch in slices that its lane tasks start on as they arrive. Skipped on
a device that cannot read pageable memory (nothing is tried there).
"""

from __future__ import annotations

import numpy as np
import pytest

from abstraction_regret_gb300 import engine as E
from abstraction_regret_gb300 import native, staging
from abstraction_regret_gb300 import workloads as W
from abstraction_regret_gb300.automata import DFA, random_dfa
from abstraction_regret_gb300.engine import PersistentEngine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pageable():
    import torch

    with torch.cuda.device(0):
        if native.lib().gbfsm_pageable_access() <= 0:
            pytest.skip("this device does not read pageable host memory")


def _mixed_inputs(seed: int):
    rng = np.random.default_rng(seed)
    store = bytearray(rng.integers(0, 256, 3 << 20, dtype=np.uint8).tobytes())
    out = []
    for k in range(300):
        length = int(rng.choice([0, 1, 7, 15, 16, 17, 31, 33, 1000, 4093, 65537,
                                 int(rng.integers(0, 40000))]))
        kind = k % 4
        if kind == 0:
            out.append(rng.integers(0, 256, length, dtype=np.uint8).tobytes())
        elif kind == 1:
            start = int(rng.integers(0, len(store) - length))
            out.append(memoryview(store)[start:start + length])
        elif kind == 2:
            out.append(bytearray(rng.integers(0, 256, length, dtype=np.uint8).tobytes()))
        else:
            a = rng.integers(0, 256, length + 9, dtype=np.uint8)
            out.append(a[int(rng.integers(0, 9)):][:length])
    return out


def test_gathered_batch_equals_the_packed_batch(pageable, monkeypatch):
    import torch

    monkeypatch.setattr(staging, "GATHER_MIN_BYTES", 0)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    inputs = _mixed_inputs(3)
    got = staging.Staging(dev, gather=True)
    want = staging.Staging(dev, gather=False)
    for _ in range(2):  # reused buffers
        d1, o1, _, t1 = got.put(inputs, stream)
        assert got.last_path == "gather"
        d2, o2, _, t2 = want.put(inputs, stream)
        assert want.last_path == "pack"
        stream.synchronize()
        assert t1 == t2 and torch.equal(o1, o2)
        assert torch.equal(d1[:t1 + 16 - t1 % 16].cpu(), d2[:t2 + 16 - t2 % 16].cpu())


def test_engine_batch_read_in_place_matches_the_oracle(pageable):
    b = W.c3("live", n_inputs=96)
    eng = PersistentEngine(b.automata)
    inputs = b.inputs()
    assert sum(map(len, inputs)) >= staging.GATHER_MIN_BYTES
    f, l, e, _, _ = eng.run_requests(np.zeros(b.n_inputs), inputs, with_examined=True)
    assert eng._staging.last_path == "gather"
    of, ol, oe, _ = O.nfa_batch(b.automata[0], b.data, b.offsets)
    assert np.array_equal(f, of) and np.array_equal(l, ol) and np.array_equal(e, oe)


def test_gathered_in_ranges_on_several_streams(pageable, monkeypatch):
    """Ranges of one batch gathered concurrently write every byte once: the result is the
    packed batch (blocks shared by two ranges' inputs included)."""
    import torch

    monkeypatch.setattr(staging, "GATHER_MIN_BYTES", 0)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    inputs = _mixed_inputs(4)
    want = staging.Staging(dev, gather=False)
    d2, _, _, t2 = want.put(inputs, stream)
    got = staging.Staging(dev, gather=True)
    n = len(inputs)
    for cuts in ([0, n], [0, 1, n], [0, 37, 38, 200, n], [0, n - 1, n]):
        d1, _, _, t1 = got.put(inputs, stream, defer=True)
        assert got.deferred
        d1.fill_(0xAB)  # stale bytes must all be overwritten
        fork = torch.cuda.Event()
        fork.record(stream)
        sides = [torch.cuda.Stream(dev) for _ in cuts[1:]]
        for side, a, b in zip(sides, cuts[:-1], cuts[1:]):
            side.wait_event(fork)
            got.gather_range(a, b, side)
        for side in sides:
            stream.wait_stream(side)
        stream.synchronize()
        assert t1 == t2
        assert torch.equal(d1[:t1].cpu(), d2[:t2].cpu()), cuts


def _alarm_dfa(n: int, seed: int) -> DFA:
    rng = np.random.default_rng(seed)
    trans = rng.integers(0, n - 1, size=(n, 256), dtype=np.int32)
    trans[:, 255] = n - 1
    accept = np.zeros(n, dtype=bool)
    accept[n - 1] = True
    return DFA(num_states=n, start_state=0, accept=accept, trans=trans.reshape(-1))


@pytest.mark.parametrize("parts", [2, 8, 16])
def test_engine_pipelined_gather_matches_the_oracle(pageable, monkeypatch, parts):
    """A mixed pool (lane-chunked NFA, chunked DFAs) run through the sliced gather: every
    verdict and examined count is the oracle's."""
    monkeypatch.setattr(E, "PIPELINE_MIN_BYTES", 0)
    rng = np.random.default_rng(parts)
    nfa = W.random_nfa(1024, seed=0, degree=2, accept_prob=0.001)
    automata = [nfa, random_dfa(256, accept_prob=1e-5, seed=1), _alarm_dfa(300, 2)]
    eng = PersistentEngine(automata)
    eng.pipeline_parts = parts
    aut_ids, inputs = [], []
    for i in range(240):
        a = int(rng.integers(0, 3))
        m = int(rng.choice([0, 5, 100, 70000, int(rng.integers(1, 200000))]))
        x = rng.integers(0, 256 if a == 0 else 255, m, dtype=np.uint8)
        if a == 2 and m and i % 3 == 0:
            x[int(rng.integers(0, m))] = 255
        aut_ids.append(a)
        inputs.append(x.tobytes())
    f, l, e, _, _ = eng.run_requests(aut_ids, inputs, with_examined=True)
    assert eng._staging.last_path == "gather" and eng.last_slices >= 2
    for a, aut in enumerate(automata):
        idx = [i for i, x in enumerate(aut_ids) if x == a]
        data, off = O.flatten([inputs[i] for i in idx])
        want = O.dfa_batch(aut, data, off) if isinstance(aut, DFA) else \
            O.nfa_batch(aut, data, off)[:3]
        for g, w, what in zip((f, l, e), want, ("flags", "lens", "examined")):
            bad = np.flatnonzero(np.asarray(g)[idx] != np.asarray(w))
            assert bad.size == 0, (parts, a, what, bad[:5].tolist())
