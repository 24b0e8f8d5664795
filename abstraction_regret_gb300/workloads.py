"""Seeded synthetic workloads: the five benchmark configurations and their variants.

Every automaton and input is a deterministic function of its seed (numpy
``default_rng``); nothing is downloaded. Conventions follow the reference's generators:
uniform bytes from ``default_rng(seed).integers(0, 256, uint8)``
(src/gpufsm/bench/generators.py:139-161) and ``random_dfa``'s draw order
(src/gpufsm/core/dfa.py:44-57).

Configurations (sizes as named by the benchmark definition):

* ``c1`` plain NFA: 1024 states, 2 edges per state (uniform symbols and targets), start 0
  non-accepting, 1% of the other states accepting, seed 0; 64 inputs of 4096 uniform
  bytes. The "regenerate until the active set exceeds one state" rule is applied through
  an optional ``check`` callable (the rule is essentially never satisfiable for this
  automaton: its active set dies after about one byte of uniform input).
* ``c2`` plain DFA: 4096 states, uint32 table of 4 MiB, 0.5% accepting, seed 1; 4096
  inputs of 64 KiB uniform bytes (256 MiB).
* ``c3`` batched NFA, uneven inputs: 16384 states, Poisson(4) out-degree, 0.1% accepting,
  seed 2; 2048 inputs with log-uniform lengths in [256 B, 1 MiB].
* ``c4`` multi-automaton: 64 NFAs with log-uniform state counts in [256, 65536] and
  out-degrees uniform in 1..8, 1% accepting, seeds 100..163; 16 inputs each, log-uniform
  in [1 KiB, 256 KiB].
* ``c5`` serving: 16 NFAs from the c4 distribution and 16 DFAs with 1024..16384 states
  (accept probability 0.005, as c2); 20000 requests with Poisson arrivals, seed 7,
  lengths log-uniform in [64 B, 4 MiB].

Variants (documented deviations, for throughput): ``live`` replaces uniform input bytes
by random walks through the automaton (``gbfsm_workload_walk``), so NFA active sets stay
alive; ``sustained`` additionally clears every accept bit so no input latches early
(the reference's own latch control: ``NO_ACCEPT``, generators.py:54, and
``scripts/dfa_latch_control.py``).
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field, replace

import numpy as np

from .automata import DFA, NFA, nfa_from_edges, random_dfa


@dataclass
class Batch:
    """One automaton (or a pool) and a flat batch of inputs."""

    name: str
    automata: list
    aut_ids: np.ndarray   # int64 [n] automaton index per input
    data: np.ndarray      # uint8 [total]
    offsets: np.ndarray   # int64 [n + 1]
    meta: dict = field(default_factory=dict)

    @property
    def n_inputs(self) -> int:
        return len(self.offsets) - 1

    @property
    def total_bytes(self) -> int:
        return int(self.offsets[-1])

    def inputs(self, idx=None) -> list[bytes]:
        rng = range(self.n_inputs) if idx is None else idx
        d, o = self.data, self.offsets
        return [d[o[i]:o[i + 1]].tobytes() for i in rng]

    def subset(self, idx) -> Batch:
        idx = np.asarray(idx, dtype=np.int64)
        lens = self.offsets[idx + 1] - self.offsets[idx]
        off = np.zeros(idx.size + 1, dtype=np.int64)
        np.cumsum(lens, out=off[1:])
        data = np.concatenate([self.data[self.offsets[i]:self.offsets[i + 1]] for i in idx]) \
            if idx.size else np.zeros(0, np.uint8)
        return replace(self, aut_ids=self.aut_ids[idx], data=data, offsets=off,
                       meta=dict(self.meta, subset=int(idx.size)))


# ---- automata ----------------------------------------------------------------------------


def random_nfa(num_states: int, seed: int, *, degree=None, poisson: float | None = None,
               accept_prob: float = 0.01, start: int = 0) -> NFA:
    """Epsilon-free random NFA: per-state out-degree (fixed, uniform range or Poisson),
    uniform symbols 0..255 and targets, ``accept_prob`` of the non-start states accept."""
    rng = np.random.default_rng(seed)
    n = int(num_states)
    if poisson is not None:
        deg = rng.poisson(poisson, n)
    elif isinstance(degree, tuple):
        deg = rng.integers(degree[0], degree[1] + 1, n)
    else:
        deg = np.full(n, int(degree if degree is not None else 2), dtype=np.int64)
    total = int(deg.sum())
    syms = rng.integers(0, 256, total, dtype=np.int64)
    dst = rng.integers(0, n, total, dtype=np.int64)
    accept = rng.random(n) < accept_prob
    accept[start] = False
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    return nfa_from_edges(n, start, accept, src, syms, dst)


def without_accepts(a):
    """The same automaton with every accept bit cleared (the ``sustained`` variant)."""
    if isinstance(a, DFA) or hasattr(a, "trans"):
        return DFA(num_states=a.num_states, start_state=a.start_state,
                   accept=np.zeros(a.num_states, dtype=bool), trans=a.trans)
    return NFA(num_states=a.num_states, start_state=a.start_state,
               accept=np.zeros(a.num_states, dtype=bool), sym_row_ptr=a.sym_row_ptr,
               sym_targets=a.sym_targets, sym_symbols=a.sym_symbols,
               eps_row_ptr=a.eps_row_ptr, eps_targets=a.eps_targets)


# ---- inputs ------------------------------------------------------------------------------


def log_uniform_lengths(rng: np.random.Generator, n: int, lo: int, hi: int) -> np.ndarray:
    """``floor(exp(U(ln lo, ln hi)))`` per input, clipped to [lo, hi]."""
    x = np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), n))).astype(np.int64)
    return np.clip(x, lo, hi)


def offsets_of(lengths: np.ndarray) -> np.ndarray:
    off = np.zeros(len(lengths) + 1, dtype=np.int64)
    np.cumsum(lengths, out=off[1:])
    return off


def uniform_bytes(seed, total: int) -> np.ndarray:
    return np.random.default_rng(seed).integers(0, 256, total, dtype=np.uint8)


def walk_bytes(nfa, offsets: np.ndarray, seed: int, threads: int | None = None) -> np.ndarray:
    """Random-walk ("live") inputs for ``nfa`` (see ``gbfsm_workload_walk``)."""
    from . import native

    lib = native.lib()
    total = int(offsets[-1])
    out = np.zeros(max(total, 1), dtype=np.uint8)
    arrs = [np.ascontiguousarray(x, dtype=np.int32) for x in
            (nfa.sym_row_ptr, nfa.sym_targets, nfa.sym_symbols)]
    acc = np.ascontiguousarray(nfa.accept, dtype=np.uint8)
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    ptr = lambda a: a.ctypes.data if a.size else None  # noqa: E731
    st = lib.gbfsm_workload_walk(int(nfa.num_states), ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]),
                                 ptr(acc), int(nfa.start_state), ptr(off), len(off) - 1,
                                 int(seed) & (2**64 - 1), out.ctypes.data,
                                 int(threads or os.cpu_count() or 1))
    native.check(st, "gbfsm_workload_walk")
    return out[:total]


# ---- configurations ------------------------------------------------------------------------


def c1(variant: str = "literal", check=None, max_tries: int = 64, walk=None) -> Batch:
    """Plain NFA. ``check(nfa, data, offsets) -> bool[n]`` applies the divergence rule.
    ``walk`` generates the random-walk inputs (default ``walk_bytes``; any generator
    giving the same bytes, e.g. a CPU-only one for a process that must not load the
    library)."""
    walk = walk or walk_bytes
    nfa = random_nfa(1024, seed=0, degree=2, accept_prob=0.01)
    n, length = 64, 4096
    offsets = offsets_of(np.full(n, length, dtype=np.int64))
    meta = {"config": "c1", "variant": variant, "states": 1024, "inputs": n, "length": length}
    if variant == "literal":
        rng = np.random.default_rng([0, 1])
        data = rng.integers(0, 256, n * length, dtype=np.uint8)
        if check is not None:
            ok = np.asarray(check(nfa, data, offsets), dtype=bool)
            tries = 1
            while not ok.all() and tries < max_tries:
                bad = np.flatnonzero(~ok)
                for i in bad:
                    data[offsets[i]:offsets[i + 1]] = rng.integers(0, 256, length, dtype=np.uint8)
                ok = np.asarray(check(nfa, data, offsets), dtype=bool)
                tries += 1
            meta.update(regen_tries=tries, regen_satisfied=int(ok.sum()))
    else:
        a = nfa if variant == "live" else without_accepts(nfa)
        data = walk(nfa, offsets, seed=10)
        nfa = a
    return Batch("c1-" + variant, [nfa], np.zeros(n, np.int64), data, offsets, meta)


def c2(variant: str = "literal", n_inputs: int = 4096, length: int = 65536) -> Batch:
    """Plain DFA (4096 states, 0.5% accepting; ``sustained`` = no accepting states)."""
    p = 0.005 if variant == "literal" else 0.0
    dfa = random_dfa(4096, accept_prob=p, seed=1)
    offsets = offsets_of(np.full(n_inputs, length, dtype=np.int64))
    data = uniform_bytes([1, 1], n_inputs * length)
    meta = {"config": "c2", "variant": variant, "states": 4096, "inputs": n_inputs,
            "length": length, "table_bytes_int32": 4096 * 256 * 4}
    return Batch("c2-" + variant, [dfa], np.zeros(n_inputs, np.int64), data, offsets, meta)


def c3(variant: str = "literal", n_inputs: int = 2048, walk=None) -> Batch:
    """Batched NFA with uneven inputs (16384 states, Poisson(4) degree, 0.1% accepting).
    ``walk`` as for ``c1``."""
    walk = walk or walk_bytes
    nfa = random_nfa(16384, seed=2, poisson=4.0, accept_prob=0.001)
    lengths = log_uniform_lengths(np.random.default_rng([2, 1]), n_inputs, 256, 1 << 20)
    offsets = offsets_of(lengths)
    if variant == "literal":
        data = uniform_bytes([2, 2], int(offsets[-1]))
    else:
        data = walk(nfa, offsets, seed=20)
        if variant == "sustained":
            nfa = without_accepts(nfa)
    meta = {"config": "c3", "variant": variant, "states": 16384, "inputs": n_inputs}
    return Batch("c3-" + variant, [nfa], np.zeros(n_inputs, np.int64), data, offsets, meta)


def c4_automaton(seed: int) -> NFA:
    rng = np.random.default_rng([seed, 0])
    n = int(np.floor(math.exp(rng.uniform(math.log(256), math.log(65536)))))
    return random_nfa(n, seed=seed, degree=(1, 8), accept_prob=0.01)


def c4(variant: str = "literal", per_automaton: int = 16, walk=None) -> Batch:
    """64 NFAs (seeds 100..163), 16 inputs each, all in one persistent launch. ``walk``
    as for ``c1``."""
    walk = walk or walk_bytes
    automata, lens, ids = [], [], []
    for k, seed in enumerate(range(100, 164)):
        automata.append(c4_automaton(seed))
        rng = np.random.default_rng([seed, 1])
        lens.append(log_uniform_lengths(rng, per_automaton, 1024, 256 * 1024))
        ids.append(np.full(per_automaton, k, dtype=np.int64))
    lengths = np.concatenate(lens)
    offsets = offsets_of(lengths)
    aut_ids = np.concatenate(ids)
    if variant == "literal":
        data = uniform_bytes([100, 2], int(offsets[-1]))
    else:
        data = np.zeros(int(offsets[-1]), dtype=np.uint8)
        for k, a in enumerate(automata):
            sel = np.flatnonzero(aut_ids == k)
            sub = offsets_of(lengths[sel])
            chunk = walk(a, sub, seed=1000 + k)
            data[offsets[sel[0]]:offsets[sel[-1] + 1]] = chunk
        if variant == "sustained":
            automata = [without_accepts(a) for a in automata]
    meta = {"config": "c4", "variant": variant, "automata": 64, "inputs": int(lengths.size),
            "states": [int(a.num_states) for a in automata]}
    return Batch("c4-" + variant, automata, aut_ids, data, offsets, meta)


@dataclass
class ServingTrace:
    """A pool of automata and a request trace (arrival times in seconds)."""

    automata: list
    aut_ids: np.ndarray
    arrivals: np.ndarray
    pool: np.ndarray          # shared random bytes; request i is pool[starts[i]:+lengths[i]]
    starts: np.ndarray
    lengths: np.ndarray

    def request(self, i: int) -> tuple[int, memoryview]:
        s = int(self.starts[i])
        return int(self.aut_ids[i]), memoryview(self.pool)[s:s + int(self.lengths[i])]

    @property
    def total_bytes(self) -> int:
        return int(self.lengths.sum())


def c5_pool() -> list:
    nfas = [c4_automaton(seed) for seed in range(200, 216)]
    dfas = []
    for seed in range(300, 316):
        rng = np.random.default_rng([seed, 0])
        n = int(np.floor(math.exp(rng.uniform(math.log(1024), math.log(16384)))))
        dfas.append(random_dfa(n, accept_prob=0.005, seed=seed))
    return nfas + dfas


C5_MAX_REQUEST = 4 << 20


def c5(rate_per_s: float = 2000.0, n_requests: int = 20000, pool_bytes: int = 1 << 26,
       automata=None, variant: str = "literal", walks_per_nfa: int = 4) -> ServingTrace:
    """Serving trace: Poisson arrivals at ``rate_per_s``, seed 7, lengths log-uniform in
    64 B..4 MiB, automata drawn uniformly from the pool.

    ``literal``: request bytes are uniform random, drawn as slices of one shared random
    pool (a documented economy: 20000 independent draws would be ~7.6 GB of host memory);
    NFA requests then die within a byte or two and DFA requests latch after ~250 bytes.
    ``live``: an NFA request is a prefix of one of ``walks_per_nfa`` random walks of its
    automaton (4 MiB each, kept after the uniform pool), so its active set stays alive;
    DFA requests as in ``literal``. ``sustained``: as ``live`` with every accept bit of
    every automaton cleared (the reference's latch control), so every offered byte is
    examined.
    """
    if variant not in ("literal", "live", "sustained"):
        raise ValueError(f"unknown c5 variant {variant!r}")
    automata = list(automata) if automata is not None else c5_pool()
    rng = np.random.default_rng(7)
    gaps = rng.exponential(1.0 / rate_per_s, n_requests)
    arrivals = np.cumsum(gaps) - gaps[0]
    aut_ids = rng.integers(0, len(automata), n_requests)
    lengths = log_uniform_lengths(rng, n_requests, 64, C5_MAX_REQUEST)
    starts = rng.integers(0, pool_bytes, n_requests)
    uniform = uniform_bytes([7, 1], pool_bytes + C5_MAX_REQUEST)
    if variant == "literal":
        return ServingTrace(automata, aut_ids.astype(np.int64), arrivals, uniform, starts,
                            lengths)
    nfa_ids = [k for k, a in enumerate(automata) if not hasattr(a, "trans")]
    parts = [uniform]
    base = uniform.size
    walk_start = {}
    for k in nfa_ids:
        off = offsets_of(np.full(walks_per_nfa, C5_MAX_REQUEST, dtype=np.int64))
        parts.append(walk_bytes(automata[k], off, seed=5000 + k))
        walk_start[k] = base
        base += int(off[-1])
    pool = np.concatenate(parts)
    for i in range(n_requests):
        k = int(aut_ids[i])
        if k in walk_start:
            starts[i] = walk_start[k] + (i % walks_per_nfa) * C5_MAX_REQUEST
    if variant == "sustained":
        automata = [without_accepts(a) for a in automata]
    return ServingTrace(automata, aut_ids.astype(np.int64), arrivals, pool, starts, lengths)


CONFIGS = {"c1": c1, "c2": c2, "c3": c3, "c4": c4}


# ---- ANML automata ---------------------------------------------------------------------------


def _anml_set(rng: np.random.Generator) -> str:
    """A symbol set as pattern-matching ANML files write them: mostly one byte, else a
    small range, a negated byte, or any byte."""
    u = rng.random()
    if u < 0.70:
        return f"\\x{int(rng.integers(0, 256)):02x}"
    if u < 0.90:
        lo = int(rng.integers(0, 240))
        return f"[\\x{lo:02x}-\\x{lo + int(rng.integers(1, 16)):02x}]"
    if u < 0.96:
        return f"[^\\x{int(rng.integers(0, 256)):02x}]"
    return "*"


def anml_patterns(n_patterns: int, seed: int, min_len: int = 4, max_len: int = 24,
                  start_of_data: float = 0.1, loop: float = 0.08, branch: float = 0.05) -> str:
    """A synthetic homogeneous ANML automaton of signature patterns, the shape of the
    pattern-matching families the reference loads (sparse active sets): each pattern is
    a chain of ``min_len..max_len`` STEs, started at every position (``all-input``) or
    only at the start (``start-of-data``), reporting at its last STE; a few STEs keep
    themselves active (a ``[...]+`` loop) and a few branch to a second successor."""
    rng = np.random.default_rng(seed)
    out = ['<anml version="1.0"><automata-network id="patterns">']
    for p in range(n_patterns):
        length = int(rng.integers(min_len, max_len + 1))
        names = [f"p{p}_{k}" for k in range(length)]
        for k, name in enumerate(names):
            attrs = f'id="{name}" symbol-set="{_anml_set(rng)}"'
            if k == 0:
                attrs += ' start="start-of-data"' if rng.random() < start_of_data \
                    else ' start="all-input"'
            body = []
            if k + 1 < length:
                body.append(f'<activate-on-match element="{names[k + 1]}"/>')
                if k + 2 < length and rng.random() < branch:
                    body.append(f'<activate-on-match element="{names[k + 2]}"/>')
            else:
                body.append(f'<report-on-match reportcode="{p}"/>')
            if rng.random() < loop:
                body.append(f'<activate-on-match element="{name}"/>')
            out.append(f'<state-transition-element {attrs}>{"".join(body)}'
                       f'</state-transition-element>')
    out.append("</automata-network></anml>")
    return "\n".join(out)


def anml_inputs(nfa, n_inputs: int, length: int, seed: int, plant: float = 0.5) -> list[bytes]:
    """Inputs for an ANML automaton: uniform bytes, with a random walk of the automaton
    (from the all-input seeding state) planted at a random position in a ``plant``
    fraction of them, so that some inputs match."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_inputs):
        x = rng.integers(0, 256, length, dtype=np.uint8)
        if length and rng.random() < plant:
            k = int(rng.integers(1, min(length, 64) + 1))
            walk = _walk_from(nfa, 1, k, rng)
            at = int(rng.integers(0, length - walk.size + 1))
            x[at:at + walk.size] = walk
        out.append(x.tobytes())
    return out


def _walk_from(nfa, state: int, k: int, rng: np.random.Generator) -> np.ndarray:
    """Up to k bytes read along symbol edges from ``state`` (ANY edges: a uniform byte),
    leaving state 1's ANY self-loop on the first step."""
    rp, tg, sy = nfa.sym_row_ptr, nfa.sym_targets, nfa.sym_symbols
    out = []
    s = state
    for step in range(k):
        lo, hi = int(rp[s]), int(rp[s + 1])
        if hi <= lo:
            break
        e = int(rng.integers(lo, hi))
        if step == 0 and s == 1 and hi - lo > 1:
            e = int(rng.integers(lo + 1, hi))
        sym = int(sy[e])
        out.append(int(rng.integers(0, 256)) if sym > 255 else sym)
        s = int(tg[e])
    return np.asarray(out, dtype=np.uint8)
