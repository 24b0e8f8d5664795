"""Generate the golden fixtures under tests/golden/ by running the reference itself.

Run in a checkout that has the reference package gpufsm 0.1.0 (alepot55/abstraction-regret)
available, e.g.::

    python tests/golden/make_golden.py --reference /root/reference

It writes three gzip'd JSON files. Every verdict in them comes from the reference's own
oracle (``gpufsm.reference.simulate`` / ``simulate_dfa``), imported from the given
checkout; nothing here is computed by this repository's code.

* ``reference_corpus.json.gz`` -- the reference's pinned corpus
  (``tests/data/golden.json``: 516 NFA and 36 DFA cases, automata serialised in full),
  re-serialised and re-verified against the reference oracle.
* ``edge_cases.json.gz`` -- extra cases drawn here and labelled by the reference oracle:
  multi-word NFAs (65..2048 states) with epsilon cycles and ANY edges, empty inputs,
  start-accepting automata, DFAs from the reference's ``DFABuilder`` (dead state) and
  ``random_dfa``.
* ``config_vectors.json.gz`` -- for each benchmark configuration and variant: SHA-256
  digests of the generated automata and inputs (pinning this repository's generators),
  and reference-oracle verdicts on a deterministic subset of inputs.
"""

from __future__ import annotations

import argparse
import gzip
import hashlib
import json
import random
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def nfa_digest(a) -> str:
    return sha(np.asarray(a.accept, bool), np.asarray(a.sym_row_ptr, np.int32),
               np.asarray(a.sym_targets, np.int32), np.asarray(a.sym_symbols, np.int32),
               np.asarray(a.eps_row_ptr, np.int32), np.asarray(a.eps_targets, np.int32),
               np.asarray([a.num_states, a.start_state], np.int64))


def dfa_digest(a) -> str:
    return sha(np.asarray(a.accept, bool), np.asarray(a.trans, np.int32),
               np.asarray([a.num_states, a.start_state], np.int64))


def nfa_json(a) -> dict:
    return {"num_states": int(a.num_states), "start_state": int(a.start_state),
            "accept": [int(x) for x in a.accept],
            "sym_row_ptr": [int(x) for x in a.sym_row_ptr],
            "sym_targets": [int(x) for x in a.sym_targets],
            "sym_symbols": [int(x) for x in a.sym_symbols],
            "eps_row_ptr": [int(x) for x in a.eps_row_ptr],
            "eps_targets": [int(x) for x in a.eps_targets]}


def dfa_json(a) -> dict:
    return {"num_states": int(a.num_states), "start_state": int(a.start_state),
            "accept": [int(x) for x in a.accept], "trans": [int(x) for x in a.trans]}


def write(name: str, obj) -> None:
    path = HERE / name
    raw = json.dumps(obj, separators=(",", ":")).encode()
    path.write_bytes(gzip.compress(raw, compresslevel=9, mtime=0))
    print(f"wrote {path.relative_to(REPO)} ({path.stat().st_size} bytes)")


def reference_corpus(ref_root: Path, ref) -> dict:
    src = json.loads((ref_root / "tests" / "data" / "golden.json").read_text())
    NFA, DFA = ref["NFA"], ref["DFA"]
    nfa_cases, dfa_cases = [], []
    for c in src["nfa_cases"]:
        d = c["nfa"]
        a = NFA(num_states=d["num_states"], start_state=d["start_state"],
                accept=np.array(d["accept"], dtype=bool),
                sym_row_ptr=np.array(d["sym_row_ptr"], np.int32),
                sym_targets=np.array(d["sym_targets"], np.int32),
                sym_symbols=np.array(d["sym_symbols"], np.int32),
                eps_row_ptr=np.array(d["eps_row_ptr"], np.int32),
                eps_targets=np.array(d["eps_targets"], np.int32))
        data = bytes.fromhex(c["input_hex"])
        got = ref["simulate"](a, data)
        assert got == (c["accepted"], c["match_len"]), c["id"]
        nfa_cases.append({"id": c["id"], "nfa": nfa_json(a), "input_hex": c["input_hex"],
                          "accepted": bool(got[0]), "match_len": int(got[1])})
    for c in src["dfa_cases"]:
        d = c["dfa"]
        a = DFA(num_states=d["num_states"], start_state=d["start_state"],
                accept=np.array(d["accept"], dtype=bool), trans=np.array(d["trans"], np.int32))
        data = bytes.fromhex(c["input_hex"])
        got = ref["simulate_dfa"](a, data)
        assert got == (c["accepted"], c["match_len"]), c["id"]
        dfa_cases.append({"id": c["id"], "dfa": dfa_json(a), "input_hex": c["input_hex"],
                          "accepted": bool(got[0]), "match_len": int(got[1])})
    return {"source": "reference tests/data/golden.json (format_version "
                      f"{src['format_version']}), re-verified with gpufsm.reference",
            "nfa_cases": nfa_cases, "dfa_cases": dfa_cases}


def edge_cases(ref) -> dict:
    """Automata are stored once (``automata`` list) and referenced by index; reference
    ``random_dfa`` tables are stored as their generator arguments plus a SHA-256 digest."""
    NFABuilder, DFABuilder = ref["NFABuilder"], ref["DFABuilder"]
    ANY = 256
    rng = random.Random(20261203)
    automata, nfa_cases, dfa_cases = [], [], []

    def add_nfa(tag, a, inputs):
        automata.append({"nfa": nfa_json(a)})
        k = len(automata) - 1
        for j, data in enumerate(inputs):
            acc, ml = ref["simulate"](a, data)
            nfa_cases.append({"id": f"{tag}:{j}", "automaton": k, "input_hex": data.hex(),
                              "accepted": bool(acc), "match_len": int(ml)})

    def rand_nfa(n, p_acc, max_deg, max_eps, p_any, alpha):
        b = NFABuilder()
        for _ in range(n):
            b.add_state(accept=rng.random() < p_acc)
        b.set_start(rng.randrange(n))
        for s in range(n):
            for _ in range(rng.randint(0, max_deg)):
                sym = ANY if rng.random() < p_any else ord(rng.choice(alpha))
                b.add_transition(s, sym, rng.randrange(n))
            for _ in range(rng.randint(0, max_eps)):
                b.add_epsilon(s, rng.randrange(n))
        return b.build()

    # multi-word automata with epsilon cycles and wildcards (dense and sparse sets)
    for n in (65, 130, 300, 700, 1000, 2048):
        for variant, (p_acc, deg, eps, p_any) in enumerate(
                [(0.02, 3, 1, 0.05), (0.005, 2, 2, 0.0), (0.01, 4, 0, 0.1)]):
            a = rand_nfa(n, p_acc, deg, eps, p_any, "abcde")
            inputs = [b"", *[bytes(ord(rng.choice("abcde")) for _ in range(rng.randint(1, 64)))
                            for _ in range(6)]]
            add_nfa(f"multiword:{n}:{variant}", a, inputs)
    # full-byte alphabet, long inputs, wildcard-heavy (sets grow dense)
    for k in range(6):
        a = rand_nfa(rng.choice([40, 200, 600]), 0.003, 3, 1, 0.2,
                     [chr(c) for c in range(256)])
        inputs = [bytes(rng.randrange(256) for _ in range(rng.randint(100, 400))) for _ in range(4)]
        add_nfa(f"dense:{k}", a, inputs)
    # start state accepts directly and via epsilon
    b = NFABuilder()
    s0, s1 = b.add_state(accept=True), b.add_state()
    b.set_start(s0)
    b.add_transition(s0, "a", s1)
    add_nfa("start-accepts", b.build(), [b"", b"a", b"zz"])
    b = NFABuilder()
    s0, s1, s2 = b.add_state(), b.add_state(), b.add_state(accept=True)
    b.set_start(s0)
    b.add_epsilon(s0, s1)
    b.add_epsilon(s1, s2)
    b.add_transition(s0, "x", s0)
    add_nfa("start-closure-accepts", b.build(), [b"", b"xx"])
    # no edges at all: any byte kills the set
    b = NFABuilder()
    b.add_state()
    b.set_start(0)
    add_nfa("edgeless", b.build(), [b"", b"a", b"abc"])
    # a self-loop on ANY that never accepts: runs to the end of the input
    b = NFABuilder()
    s0, s1 = b.add_state(), b.add_state(accept=True)
    b.set_start(s0)
    b.add_transition(s0, ANY, s0)
    b.add_transition(s0, 0xFF, s1)
    add_nfa("any-loop", b.build(), [bytes(range(255)) * 3, bytes(range(256)), b"\xff"])

    def add_dfa(tag, a, inputs, gen=None):
        automata.append({"random_dfa": gen, "sha256": dfa_digest(a)} if gen else {"dfa": dfa_json(a)})
        k = len(automata) - 1
        for j, data in enumerate(inputs):
            acc, ml = ref["simulate_dfa"](a, data)
            dfa_cases.append({"id": f"{tag}:{j}", "automaton": k, "input_hex": data.hex(),
                              "accepted": bool(acc), "match_len": int(ml)})

    for k in range(8):
        b = DFABuilder()
        n = rng.randint(2, 40)
        for i in range(n):
            b.add_state(accept=(i > 0 and rng.random() < 0.1))
        b.set_start(rng.randrange(n))
        for s in range(n):
            for c in range(256):
                if rng.random() < 0.3:
                    b.add_transition(s, c, rng.randrange(n))
        a = b.build()
        add_dfa(f"builder:{k}", a, [b"", *[bytes(rng.randrange(256) for _ in range(rng.randint(1, 200)))
                                           for _ in range(5)]])
    for n in (16, 256, 4096, 40000):
        a = ref["random_dfa"](n, accept_prob=0.02, seed=n)
        add_dfa(f"random_dfa:{n}", a, [bytes(rng.randrange(256) for _ in range(rng.randint(0, 300)))
                                        for _ in range(6)],
                gen={"num_states": n, "accept_prob": 0.02, "seed": n})
    b = DFABuilder()
    b.add_state(accept=True)
    b.set_start(0)
    add_dfa("start-accepts", b.build(), [b"", b"q"])
    return {"source": "drawn by tests/golden/make_golden.py, labelled by gpufsm.reference",
            "automata": automata, "nfa_cases": nfa_cases, "dfa_cases": dfa_cases}


def pick_subset(offsets: np.ndarray, budget: int, max_count: int) -> list[int]:
    """Deterministic subset: shortest inputs first, then every k-th, within a byte budget."""
    lens = np.diff(offsets)
    order = list(np.argsort(lens, kind="stable"))
    chosen, used = [], 0
    for i in order[: max_count // 2] + order[:: max(1, len(order) // max(1, max_count // 2))]:
        i = int(i)
        if i in chosen:
            continue
        if used + lens[i] > budget:
            continue
        chosen.append(i)
        used += int(lens[i])
        if len(chosen) >= max_count:
            break
    return sorted(chosen)


def config_vectors(ref) -> dict:
    from abstraction_regret_gb300 import workloads as W

    out = {}
    plans = [
        ("c1-literal", lambda: W.c1("literal"), 1 << 20, 64),
        ("c1-live", lambda: W.c1("live"), 1 << 20, 64),
        ("c1-sustained", lambda: W.c1("sustained"), 1 << 20, 64),
        ("c2-literal", lambda: W.c2("literal", n_inputs=256), 1 << 22, 256),
        ("c2-sustained", lambda: W.c2("sustained", n_inputs=64), 1 << 20, 16),
        ("c3-literal", lambda: W.c3("literal"), 1 << 22, 2048),
        ("c3-live", lambda: W.c3("live"), 1 << 20, 48),
        ("c3-sustained", lambda: W.c3("sustained"), 1 << 20, 48),
        ("c4-literal", lambda: W.c4("literal"), 1 << 22, 1024),
        ("c4-live", lambda: W.c4("live"), 1 << 20, 64),
    ]
    for name, make, budget, count in plans:
        t0 = time.time()
        b = make()
        digests = [dfa_digest(a) if hasattr(a, "trans") else nfa_digest(a) for a in b.automata]
        entry = {"automata_sha256": digests, "data_sha256": sha(b.data),
                 "offsets_sha256": sha(b.offsets), "aut_ids_sha256": sha(b.aut_ids),
                 "n_inputs": b.n_inputs, "total_bytes": b.total_bytes}
        idx = pick_subset(b.offsets, budget, count)
        verdicts = []
        for i in idx:
            a = b.automata[int(b.aut_ids[i])]
            data = b.data[b.offsets[i]:b.offsets[i + 1]].tobytes()
            sim = ref["simulate_dfa"] if hasattr(a, "trans") else ref["simulate"]
            acc, ml = sim(a, data)
            verdicts.append([int(i), int(acc), int(ml)])
        entry["verdicts"] = verdicts
        out[name] = entry
        print(f"  {name}: {len(verdicts)} reference verdicts in {time.time() - t0:.1f}s")
    return {"source": "digests of this repository's generators; verdicts by gpufsm.reference",
            "configs": out}


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--reference", default="/root/reference",
                    help="checkout of the reference (its src/ is put on sys.path)")
    ap.add_argument("--only", choices=["corpus", "edge", "configs"], default=None)
    args = ap.parse_args()
    ref_root = Path(args.reference)
    sys.path.insert(0, str(ref_root / "src"))
    import gpufsm
    from gpufsm.core.dfa import DFA, DFABuilder, random_dfa
    from gpufsm.core.nfa import NFA, NFABuilder
    from gpufsm.reference import simulate, simulate_dfa

    ref = {"NFA": NFA, "DFA": DFA, "NFABuilder": NFABuilder, "DFABuilder": DFABuilder,
           "random_dfa": random_dfa, "simulate": simulate, "simulate_dfa": simulate_dfa,
           "version": getattr(gpufsm, "__version__", "?")}
    if args.only in (None, "corpus"):
        write("reference_corpus.json.gz", reference_corpus(ref_root, ref))
    if args.only in (None, "edge"):
        write("edge_cases.json.gz", edge_cases(ref))
    if args.only in (None, "configs"):
        write("config_vectors.json.gz", config_vectors(ref))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
