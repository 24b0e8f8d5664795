"""ANML automata on the GPU: every NFA technique and the persistent engine against the
oracle (GPU).

Automata loaded from ANML have the reference loader's shape (src/gpufsm/io/anml.py:
166-212): a start state with epsilon edges to an all-input state (an ANY self-loop, so
the active set never empties) and a start-of-data state, then one state per STE with
sparse pattern chains. They exercise the epsilon-closure and wildcard paths of every
kernel; long inputs go through the engine's warp chunks (the automata have epsilon
edges, so they do not run in lanes).
"""

from __future__ import annotations

import numpy as np
import pytest

import abstraction_regret_gb300 as G
from abstraction_regret_gb300 import anml
from abstraction_regret_gb300 import workloads as W
from abstraction_regret_gb300.engine import PersistentEngine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pairs(res):
    return [(r.accepted, r.match_len) for r in res]


@pytest.mark.parametrize("patterns", [20, 300])
def test_every_technique_on_anml_automata(patterns):
    nfa = anml.load_anml_string(W.anml_patterns(patterns, seed=patterns))
    inputs = W.anml_inputs(nfa, 48, 3000, seed=patterns + 1) + [b"", b"\x00"]
    want = O.verdicts(nfa, inputs)
    assert any(a for a, _ in want) and not all(a for a, _ in want)
    for technique in G.list_techniques(G.Backend.CUDA, G.Kind.NFA):
        assert _pairs(G.run_batch(nfa, inputs, technique=technique)) == want, technique


def test_engine_chunks_long_inputs_of_anml_automata():
    """Long inputs (warp chunks, speculative starts from one-byte supersets) and a pool
    of several ANML automata with an ordinary NFA in one batch."""
    pool = [anml.load_anml_string(W.anml_patterns(k, seed=10 + k)) for k in (40, 120, 400)]
    pool.append(W.random_nfa(1024, seed=0, degree=2, accept_prob=0.01))
    rng = np.random.default_rng(5)
    aut, inputs = [], []
    for i in range(96):
        a = int(rng.integers(0, len(pool)))
        length = int(W.log_uniform_lengths(rng, 1, 100, 300_000)[0])
        if a < 3:
            inputs += W.anml_inputs(pool[a], 1, length, seed=1000 + i, plant=0.3)
        else:
            inputs.append(W.walk_bytes(pool[a], W.offsets_of(np.array([length])), seed=i).tobytes())
        aut.append(a)
    aut = np.asarray(aut)
    for chunk in (0, 4096):
        eng = PersistentEngine(pool, chunk_bytes=chunk)
        f, l, e, _, _ = eng.run_requests(aut, inputs, with_examined=True)
        for k, a in enumerate(pool):
            sel = np.flatnonzero(aut == k)
            data, off = O.flatten([inputs[i] for i in sel])
            of, ol, oe, _ = O.nfa_batch(a, data, off)
            assert np.array_equal(f[sel], of) and np.array_equal(l[sel], ol), (chunk, k)
            assert np.array_equal(e[sel], oe), (chunk, k)
