"""Randomised parity of the batched engine against the oracle (GPU).

Many small random automata -- NFAs with epsilon edges, ANY edges, dead ends and
accepting starts; DFAs of a few to a few hundred states -- in mixed pools, with inputs
that keep the sets alive (random walks over a small alphabet) or kill them (uniform
bytes), of every length from 0 up. Each pool runs through the engine with short fixed
chunks, so that every path is taken: lane chunks, warp chunks, whole inputs, DFA groups,
DFA chunks and their fix-ups. Verdicts and examined counts must equal the oracle's.
"""

from __future__ import annotations

import numpy as np
import pytest

import abstraction_regret_gb300 as G
from abstraction_regret_gb300.automata import DFA
from abstraction_regret_gb300.engine import PersistentEngine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _random_nfa(rng: np.random.Generator, alphabet: int):
    n = int(rng.integers(2, 300))
    p = float(rng.choice([0.0, 0.005, 0.05]))
    b = G.NFABuilder()
    for k in range(n):
        b.add_state(accept=bool(rng.random() < p))
    b.set_start(int(rng.integers(0, n)))
    for s in range(n):
        for _ in range(int(rng.poisson(2.5))):
            sym = G.ANY_SYMBOL if rng.random() < 0.01 else int(rng.integers(0, alphabet))
            b.add_transition(s, sym, int(rng.integers(0, n)))
        if rng.random() < 0.05:
            b.add_epsilon(s, int(rng.integers(0, n)))
    return b.build()


def _random_dfa(rng: np.random.Generator, alphabet: int) -> DFA:
    n = int(rng.integers(2, 400))
    trans = rng.integers(0, n, (n, 256), dtype=np.int32)
    trans[:, alphabet:] = trans[:, :1]  # bytes outside the alphabet act like byte 0
    accept = rng.random(n) < float(rng.choice([0.0, 0.0005, 0.005]))
    return DFA(num_states=n, start_state=int(rng.integers(0, n)), accept=accept,
               trans=trans.reshape(-1))


def _inputs(rng: np.random.Generator, count: int, alphabet: int, long_len: int):
    out = []
    for _ in range(count):
        r = rng.random()
        m = 0 if r < 0.05 else int(rng.integers(1, 64)) if r < 0.4 else \
            int(rng.integers(64, long_len))
        out.append(rng.integers(0, alphabet, m, dtype=np.uint8).tobytes())
    return out


def _oracle(automata, aut_ids, inputs):
    f = np.zeros(len(inputs), np.int32)
    ln = np.zeros(len(inputs), np.int32)
    ex = np.zeros(len(inputs), np.int64)
    for a, aut in enumerate(automata):
        idx = [i for i, x in enumerate(aut_ids) if x == a]
        if not idx:
            continue
        data, off = O.flatten([inputs[i] for i in idx])
        res = O.dfa_batch(aut, data, off) if isinstance(aut, DFA) else \
            O.nfa_batch(aut, data, off)[:3]
        f[idx], ln[idx], ex[idx] = res
    return f, ln, ex


@pytest.mark.parametrize("seed", range(12))
def test_random_pools_every_engine_path(seed):
    rng = np.random.default_rng(1000 + seed)
    alphabet = int(rng.choice([2, 4, 16, 256]))
    automata = [_random_nfa(rng, alphabet) for _ in range(int(rng.integers(1, 5)))] + \
        [_random_dfa(rng, alphabet) for _ in range(int(rng.integers(1, 4)))]
    n_inputs = int(rng.integers(40, 160))
    aut_ids = [int(a) for a in rng.integers(0, len(automata), n_inputs)]
    inputs = _inputs(rng, n_inputs, alphabet, long_len=int(rng.choice([2000, 20000])))
    want = _oracle(automata, aut_ids, inputs)
    for chunk, dfa_chunk in ((256, 4096), (0, None), (None, 0)):
        eng = PersistentEngine(automata, chunk_bytes=chunk, dfa_chunk_bytes=dfa_chunk)
        got = eng.run_requests(aut_ids, inputs, with_examined=True)[:3]
        for g, w, what in zip(got, want, ("flags", "lens", "examined")):
            bad = np.flatnonzero(np.asarray(g) != np.asarray(w))
            assert bad.size == 0, (seed, chunk, what, bad[:5].tolist())
