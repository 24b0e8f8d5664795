"""The reference's own GPU test suite, restated against this engine (GPU).

Same generators, seeds, sizes and checks as the reference's tests/test_gpu_backends.py
(examples, 40 fuzz NFAs of <= 8 states, batches of <= 64 states, multi-word 65/130/300),
tests/test_dfa_gpu.py (n = 16/256/4096, accept 0.02, 48 inputs) and
tests/test_worklist_warp.py (warp == oracle up to 64 states; warp == global,
shared == warp and compact == global up to 2048 states). Like the reference, each check
iterates every technique registered under ``Backend.CUDA``.
"""

from __future__ import annotations

import random

import pytest

from abstraction_regret_gb300 import (
    ANY_SYMBOL,
    Backend,
    Kind,
    NFABuilder,
    available_backends,
    list_techniques,
    random_dfa,
    run,
    run_batch,
)
from oracle.oracle import simulate, simulate_dfa

from .golden_data import load, nfa_from

pytestmark = pytest.mark.gpu


def _techniques():
    assert Backend.CUDA in available_backends()
    return list_techniques(Backend.CUDA, Kind.NFA)


def _pairs(res):
    return [(r.accepted, r.match_len) for r in res]


def test_examples_every_technique():
    cases = [c for c in load("reference_corpus.json.gz")["nfa_cases"]
             if c["id"].startswith("example:")]
    assert len(cases) == 16
    for technique in _techniques():
        for c in cases:
            nfa, data = nfa_from(c["nfa"]), bytes.fromhex(c["input_hex"])
            res = run(nfa, data, backend="cuda", technique=technique)
            assert (res.accepted, res.match_len) == simulate(nfa, data), (technique, c["id"])


def test_fuzz_every_technique():
    rng = random.Random(7)
    for technique in _techniques():
        for _ in range(40):
            b = NFABuilder()
            n = rng.randint(1, 8)
            for _ in range(n):
                b.add_state(accept=rng.random() < 0.25)
            b.set_start(rng.randrange(n))
            for s in range(n):
                for _ in range(rng.randint(0, 2)):
                    sym = ANY_SYMBOL if rng.random() < 0.1 else rng.choice("abc")
                    b.add_transition(s, sym, rng.randrange(n))
                for _ in range(rng.randint(0, 1)):
                    b.add_epsilon(s, rng.randrange(n))
            nfa = b.build()
            data = bytes(ord(rng.choice("abc")) for _ in range(rng.randint(0, 10)))
            res = run(nfa, data, backend="cuda", technique=technique)
            assert (res.accepted, res.match_len) == simulate(nfa, data), technique


def _random_nfa(n, rng, alpha, p_acc, max_deg, max_eps, p_any):
    b = NFABuilder()
    for _ in range(n):
        b.add_state(accept=rng.random() < p_acc)
    b.set_start(rng.randrange(n))
    for s in range(n):
        for _ in range(rng.randint(0, max_deg)):
            sym = ANY_SYMBOL if rng.random() < p_any else ord(rng.choice(alpha))
            b.add_transition(s, sym, rng.randrange(n))
        for _ in range(rng.randint(0, max_eps)):
            b.add_epsilon(s, rng.randrange(n))
    return b.build()


def test_run_batch_every_technique():
    rng = random.Random(11)
    for technique in _techniques():
        for _ in range(8):
            nfa = _random_nfa(rng.randint(1, 64), rng, "abcd", 0.2, 2, 1, 0.05)
            batch = [bytes(ord(rng.choice("abcd")) for _ in range(rng.randint(0, 16)))
                     for _ in range(rng.randint(1, 24))]
            got = _pairs(run_batch(nfa, batch, backend="cuda", technique=technique))
            assert got == [simulate(nfa, d) for d in batch], technique


def test_multiword_batch_every_technique():
    rng = random.Random(23)
    for technique in _techniques():
        for n in (65, 130, 300):
            nfa = _random_nfa(n, rng, "abcde", 0.1, 2, 1, 0.05)
            batch = [bytes(ord(rng.choice("abcde")) for _ in range(rng.randint(0, 24)))
                     for _ in range(rng.randint(1, 16))]
            got = _pairs(run_batch(nfa, batch, backend="cuda", technique=technique))
            assert got == [simulate(nfa, d) for d in batch], (technique, n)


def test_dfa_matches_reference():
    rng = random.Random(0)
    for n in (16, 256, 4096):
        dfa = random_dfa(n, accept_prob=0.02, seed=n)
        batch = [bytes(rng.randint(0, 255) for _ in range(rng.randint(0, 40))) for _ in range(48)]
        for technique in list_techniques(Backend.CUDA, Kind.DFA):
            got = _pairs(run_batch(dfa, batch, backend="cuda", technique=technique))
            assert got == [simulate_dfa(dfa, b) for b in batch], (n, technique)


def test_warp_matches_reference_small():
    rng = random.Random(7)
    for _ in range(30):
        nfa = _random_nfa(rng.randint(1, 64), rng, "abcde", 0.1, 3, 2, 0.05)
        batch = [bytes(ord(rng.choice("abcde")) for _ in range(rng.randint(0, 20)))
                 for _ in range(16)]
        got = _pairs(run_batch(nfa, batch, "cuda", "worklist_warp"))
        assert got == [simulate(nfa, d) for d in batch]


@pytest.mark.parametrize("n", [65, 200, 1000, 2048])
@pytest.mark.parametrize("pair", [("worklist_warp", "worklist_global"),
                                  ("worklist_shared", "worklist_warp"),
                                  ("worklist_compact", "worklist_global")])
def test_large_technique_pairs_agree_and_match_the_oracle(n, pair):
    rng = random.Random({"worklist_warp": 100, "worklist_shared": 200,
                         "worklist_compact": 300}[pair[0]] + n)
    nfa = _random_nfa(n, rng, "abcde", 0.1, 3, 2, 0.05)
    batch = [bytes(ord(rng.choice("abcde")) for _ in range(rng.randint(0, 24))) for _ in range(24)]
    a = _pairs(run_batch(nfa, batch, "cuda", pair[0]))
    b = _pairs(run_batch(nfa, batch, "cuda", pair[1]))
    assert a == b == [simulate(nfa, d) for d in batch]
