"""The CPU oracle (oracle/) is pinned before it is trusted.

Both restatements of the reference's simulators -- the pure-Python one and the C one --
must reproduce every verdict of the reference's own golden corpus and of the extra
golden vectors labelled by the reference oracle (tests/golden/, made by
make_golden.py), and agree with each other on fuzz cases. The benchmark workload
generators are pinned by digests, so the configuration vectors stay meaningful.
"""

from __future__ import annotations

import random

import numpy as np
import pytest

from abstraction_regret_gb300 import ANY_SYMBOL, NFABuilder
from abstraction_regret_gb300 import workloads as W
from oracle import oracle as O

from .golden_data import corpus_cases, dfa_digest, load, nfa_digest, sha


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build()


def test_corpus_is_non_trivial():
    ref = load("reference_corpus.json.gz")
    assert len(ref["nfa_cases"]) >= 500 and len(ref["dfa_cases"]) >= 36
    assert any(c["accepted"] for c in ref["nfa_cases"])
    assert any(not c["accepted"] for c in ref["nfa_cases"])
    assert any(c["accepted"] and c["match_len"] > 0 for c in ref["nfa_cases"])


@pytest.mark.parametrize("kind", ["nfa", "dfa"])
def test_python_oracle_matches_golden(kind):
    sim = O.simulate if kind == "nfa" else O.simulate_dfa
    bad = [(cid, sim(a, d), v) for cid, a, d, v in corpus_cases(kind)
           if sim(a, d) != tuple(v)]
    assert not bad, bad[:5]


@pytest.mark.parametrize("kind", ["nfa", "dfa"])
def test_c_oracle_matches_golden(kind):
    bad = []
    for cid, a, d, v in corpus_cases(kind):
        got = O.verdicts(a, [d], threads=1)[0]
        if got != tuple(v):
            bad.append((cid, got, v))
    assert not bad, bad[:5]


def test_c_oracle_batches_match_python_on_fuzz():
    rng = random.Random(99)
    for _ in range(60):
        b = NFABuilder()
        n = rng.randint(1, 90)
        for _ in range(n):
            b.add_state(accept=rng.random() < 0.08)
        b.set_start(rng.randrange(n))
        for s in range(n):
            for _ in range(rng.randint(0, 3)):
                sym = ANY_SYMBOL if rng.random() < 0.05 else ord(rng.choice("abcd"))
                b.add_transition(s, sym, rng.randrange(n))
            for _ in range(rng.randint(0, 1)):
                b.add_epsilon(s, rng.randrange(n))
        nfa = b.build()
        inputs = [bytes(ord(rng.choice("abcd")) for _ in range(rng.randint(0, 40)))
                  for _ in range(12)]
        want = [O.simulate(nfa, x) for x in inputs]
        assert O.verdicts(nfa, inputs, threads=4) == want


def test_c_oracle_examined_and_peak():
    b = NFABuilder()
    s0, s1, s2 = b.add_state(), b.add_state(), b.add_state(accept=True)
    b.set_start(s0)
    b.add_transition(s0, "a", s0)
    b.add_transition(s0, "a", s1)
    b.add_transition(s1, "b", s2)
    nfa = b.build()
    data, off = O.flatten([b"aaab", b"aaxa", b"", b"aaa"])
    f, l, ex, peak = O.nfa_batch(nfa, data, off, threads=2)
    assert f.tolist() == [1, 0, 0, 0]
    assert l.tolist() == [4, 0, 0, 0]
    assert ex.tolist() == [4, 3, 0, 3]  # latch at 4; dies on 'x' (3rd byte); empty; whole input
    assert peak.tolist() == [2, 2, 1, 2]


def test_c_oracle_rejects_invalid_automata():
    b = NFABuilder()
    b.add_state()
    nfa = b.build()
    bad = type(nfa)(num_states=1, start_state=0, accept=nfa.accept,
                    sym_row_ptr=np.array([0, 1], np.int32), sym_targets=np.array([5], np.int32),
                    sym_symbols=np.array([1], np.int32), eps_row_ptr=nfa.eps_row_ptr,
                    eps_targets=nfa.eps_targets)
    with pytest.raises(ValueError):
        O.verdicts(bad, [b"a"])


# ---- configuration vectors: generators pinned, reference verdicts replayed -----------------

_SMALL = {
    "c1-literal": lambda: W.c1("literal"),
    "c1-live": lambda: W.c1("live"),
    "c1-sustained": lambda: W.c1("sustained"),
    "c2-literal": lambda: W.c2("literal", n_inputs=256),
    "c2-sustained": lambda: W.c2("sustained", n_inputs=64),
    "c3-literal": lambda: W.c3("literal"),
    "c3-live": lambda: W.c3("live"),
    "c3-sustained": lambda: W.c3("sustained"),
    "c4-literal": lambda: W.c4("literal"),
    "c4-live": lambda: W.c4("live"),
}


@pytest.mark.parametrize("name", sorted(_SMALL))
def test_generators_are_pinned_and_oracle_matches_reference(name):
    vec = load("config_vectors.json.gz")["configs"][name]
    b = _SMALL[name]()
    digests = [dfa_digest(a) if hasattr(a, "trans") else nfa_digest(a) for a in b.automata]
    assert digests == vec["automata_sha256"], "automaton generator drifted"
    assert sha(b.data) == vec["data_sha256"], "input generator drifted"
    assert sha(b.offsets) == vec["offsets_sha256"]
    idx = [v[0] for v in vec["verdicts"]]
    for k, a in enumerate(b.automata):
        sel = [i for i in idx if b.aut_ids[i] == k]
        if not sel:
            continue
        got = O.verdicts(a, b.inputs(sel))
        want = [(bool(v[1]), v[2]) for v in vec["verdicts"] if b.aut_ids[v[0]] == k]
        assert got == want


def test_oracle_walker_matches_the_library_walker():
    """The CPU reference arm generates its random-walk inputs with the oracle's walker
    (so that it loads no product code); the bytes must equal the library's."""
    cases = [(W.random_nfa(1024, seed=0, degree=2, accept_prob=0.01), 10),
             (W.random_nfa(3000, seed=5, poisson=4.0, accept_prob=0.001), 20),
             (W.c4_automaton(101), 1001)]
    b = NFABuilder()  # ANY edges and a start state outside the live core
    s = [b.add_state() for _ in range(5)]
    b.add_transition(s[0], ANY_SYMBOL, s[1])
    b.add_transition(s[1], "a", s[2])
    b.add_transition(s[2], ANY_SYMBOL, s[1])
    b.add_transition(s[1], "b", s[3])
    b.set_accept(s[3])
    cases.append((b.build(), 7))
    lengths = np.array([0, 1, 17, 300, 5000, 4096, 33, 1], dtype=np.int64)
    off = W.offsets_of(lengths)
    for nfa, seed in cases:
        for threads in (1, 3):
            ours = O.walk_bytes(nfa, off, seed=seed, threads=threads)
            lib = W.walk_bytes(nfa, off, seed=seed, threads=2)
            assert np.array_equal(ours, lib), (nfa.num_states, seed, threads)


def test_reference_arm_workload_loads_no_product_library():
    """bench.py --impl reference builds its workload and times the oracle without
    mapping libgbfsm.so."""
    import subprocess
    import sys
    from pathlib import Path

    repo = Path(__file__).resolve().parent.parent
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import bench\n"
        "b = bench.load_workload('c1-live', reference_arm=True)\n"
        "from oracle import oracle as O\n"
        "O.nfa_batch(b.automata[0], b.data, b.offsets)\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('libgbfsm' in maps, 'libfsm_oracle' in maps)\n" % str(repo))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         timeout=600, cwd=str(repo))
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.split() == ["False", "True"]
