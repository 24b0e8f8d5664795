"""Loaders for the golden fixtures in tests/golden/ (made by tests/golden/make_golden.py
from the reference's own oracle and corpus)."""

from __future__ import annotations

import gzip
import hashlib
import json
from functools import lru_cache
from pathlib import Path

import numpy as np

from abstraction_regret_gb300.automata import DFA, NFA, random_dfa

GOLDEN = Path(__file__).resolve().parent / "golden"


@lru_cache(maxsize=None)
def load(name: str) -> dict:
    return json.loads(gzip.decompress((GOLDEN / name).read_bytes()))


def nfa_from(d: dict) -> NFA:
    return NFA(num_states=int(d["num_states"]), start_state=int(d["start_state"]),
               accept=np.array(d["accept"], dtype=bool),
               sym_row_ptr=np.array(d["sym_row_ptr"], dtype=np.int32),
               sym_targets=np.array(d["sym_targets"], dtype=np.int32),
               sym_symbols=np.array(d["sym_symbols"], dtype=np.int32),
               eps_row_ptr=np.array(d["eps_row_ptr"], dtype=np.int32),
               eps_targets=np.array(d["eps_targets"], dtype=np.int32))


def dfa_from(d: dict) -> DFA:
    return DFA(num_states=int(d["num_states"]), start_state=int(d["start_state"]),
               accept=np.array(d["accept"], dtype=bool),
               trans=np.array(d["trans"], dtype=np.int32))


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def dfa_digest(a) -> str:
    return sha(np.asarray(a.accept, bool), np.asarray(a.trans, np.int32),
               np.asarray([a.num_states, a.start_state], np.int64))


def nfa_digest(a) -> str:
    return sha(np.asarray(a.accept, bool), np.asarray(a.sym_row_ptr, np.int32),
               np.asarray(a.sym_targets, np.int32), np.asarray(a.sym_symbols, np.int32),
               np.asarray(a.eps_row_ptr, np.int32), np.asarray(a.eps_targets, np.int32),
               np.asarray([a.num_states, a.start_state], np.int64))


def corpus_cases(kind: str):
    """``[(id, automaton, input bytes, (accepted, match_len))]`` from both corpora."""
    out = []
    ref = load("reference_corpus.json.gz")
    same: dict[str, object] = {}  # identical serialised automata share one object
    for c in ref[f"{kind}_cases"]:
        key = json.dumps(c[kind], sort_keys=True)
        if key not in same:
            same[key] = nfa_from(c["nfa"]) if kind == "nfa" else dfa_from(c["dfa"])
        a = same[key]
        out.append((c["id"], a, bytes.fromhex(c["input_hex"]), (c["accepted"], c["match_len"])))
    edge = load("edge_cases.json.gz")
    built = {}
    for c in edge[f"{kind}_cases"]:
        k = c["automaton"]
        if k not in built:
            spec = edge["automata"][k]
            if "nfa" in spec:
                built[k] = nfa_from(spec["nfa"])
            elif "dfa" in spec:
                built[k] = dfa_from(spec["dfa"])
            else:
                g = spec["random_dfa"]
                a = random_dfa(g["num_states"], accept_prob=g["accept_prob"], seed=g["seed"])
                assert dfa_digest(a) == spec["sha256"], "random_dfa drifted from the reference"
                built[k] = a
        out.append((c["id"], built[k], bytes.fromhex(c["input_hex"]),
                    (c["accepted"], c["match_len"])))
    return out


def grouped(kind: str):
    """Cases grouped by automaton identity: ``[(automaton, [(id, input, verdict)])]``."""
    groups: dict[int, tuple] = {}
    for cid, a, data, v in corpus_cases(kind):
        key = id(a)
        if key not in groups:
            groups[key] = (a, [])
        groups[key][1].append((cid, data, v))
    return list(groups.values())
