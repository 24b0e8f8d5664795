"""CPU oracle for the automata-simulation hot path -- TEST INFRASTRUCTURE ONLY.

This module is the oracle the CUDA engine is compared against. Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import it; the
product package (``abstraction_regret_gb300``) never does, and it has no CPU fallback.

Two restatements of the reference package gpufsm 0.1.0 (alepot55/abstraction-regret):

* ``simulate`` / ``simulate_dfa`` / ``epsilon_closure`` -- pure-Python loops that follow
  ``src/gpufsm/reference.py:20-33`` (iterative DFS closure), ``:36-65`` (NFA,
  latch-first-match, break on an empty set) and ``:68-81`` (DFA). Use them on small cases.
* ``nfa_batch`` / ``dfa_batch`` -- the same algorithm in C (``oracle/fsm_oracle.c``),
  multi-threaded over inputs, for full-size workloads. ``build()`` compiles it with gcc
  into ``oracle/_build/``.

Both are pinned against the reference's own golden corpus and against golden vectors
produced by running the reference itself (``tests/golden/``).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

ANY_SYMBOL = 256  # src/gpufsm/core/nfa.py:16
ALPHABET = 256  # src/gpufsm/core/dfa.py:22

_HERE = Path(__file__).resolve().parent
_SRC = _HERE / "fsm_oracle.c"
_LIB = _HERE / "_build" / "libfsm_oracle.so"


# --------------------------------------------------------------------------------------
# Pure-Python restatement (small cases)
# --------------------------------------------------------------------------------------


def epsilon_closure(states, nfa) -> set[int]:
    """Epsilon closure by iterative DFS (reference.py:20-33)."""
    seen = set(int(s) for s in states)
    todo = list(seen)
    rp, tg = nfa.eps_row_ptr, nfa.eps_targets
    while todo:
        s = todo.pop()
        for k in range(int(rp[s]), int(rp[s + 1])):
            t = int(tg[k])
            if t not in seen:
                seen.add(t)
                todo.append(t)
    return seen


def simulate(nfa, data: bytes) -> tuple[bool, int]:
    """Latch-first-match NFA verdict ``(accepted, match_len)`` (reference.py:36-65)."""
    acc = nfa.accept
    active = epsilon_closure({int(nfa.start_state)}, nfa)
    if any(acc[s] for s in active):
        return True, 0
    rp, tg, sy = nfa.sym_row_ptr, nfa.sym_targets, nfa.sym_symbols
    for i, b in enumerate(bytes(data)):
        step: set[int] = set()
        for s in active:
            for k in range(int(rp[s]), int(rp[s + 1])):
                sym = int(sy[k])
                if sym == b or sym == ANY_SYMBOL:
                    step.add(int(tg[k]))
        if not step:
            return False, 0
        active = epsilon_closure(step, nfa)
        if any(acc[s] for s in active):
            return True, i + 1
    return False, 0


def simulate_dfa(dfa, data: bytes) -> tuple[bool, int]:
    """Latch-first-match DFA verdict (reference.py:68-81)."""
    cur = int(dfa.start_state)
    if dfa.accept[cur]:
        return True, 0
    tr = dfa.trans
    for i, b in enumerate(bytes(data)):
        cur = int(tr[cur * ALPHABET + b])
        if dfa.accept[cur]:
            return True, i + 1
    return False, 0


# --------------------------------------------------------------------------------------
# C restatement (full-size cases)
# --------------------------------------------------------------------------------------


def build(force: bool = False) -> Path:
    """Compile ``fsm_oracle.c`` into ``oracle/_build/libfsm_oracle.so`` (gcc, -O2)."""
    if _LIB.exists() and not force and _LIB.stat().st_mtime >= _SRC.stat().st_mtime:
        return _LIB
    _LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = _LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(
        ["gcc", "-O2", "-std=c11", "-shared", "-fPIC", "-pthread", str(_SRC), "-o", str(tmp)],
        check=True,
    )
    os.replace(tmp, _LIB)
    return _LIB


_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(build()))
        p = ctypes.c_void_p
        lib.fsm_oracle_nfa_batch.restype = ctypes.c_int
        lib.fsm_oracle_nfa_batch.argtypes = [ctypes.c_int32, ctypes.c_int32, p, p, p, p, p, p, p,
                                             p, ctypes.c_int64, ctypes.c_int32, p, p, p, p, p,
                                             p]
        lib.fsm_oracle_dfa_batch.restype = ctypes.c_int
        lib.fsm_oracle_dfa_batch.argtypes = [ctypes.c_int32, ctypes.c_int32, p, p, p, p,
                                             ctypes.c_int64, ctypes.c_int32, p, p, p]
        lib.fsm_oracle_walk.restype = ctypes.c_int
        lib.fsm_oracle_walk.argtypes = [ctypes.c_int32, p, p, p, p, ctypes.c_int32, p,
                                        ctypes.c_int64, ctypes.c_uint64, p, ctypes.c_int32]
        _lib = lib
    return _lib


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data) if a.size else ctypes.c_void_p(0)


def flatten(inputs) -> tuple[np.ndarray, np.ndarray]:
    """A list of ``bytes`` as one uint8 buffer plus int64 offsets (``len + 1`` entries)."""
    lens = np.fromiter((len(b) for b in inputs), dtype=np.int64, count=len(inputs))
    offsets = np.zeros(len(inputs) + 1, dtype=np.int64)
    np.cumsum(lens, out=offsets[1:])
    data = np.frombuffer(b"".join(inputs), dtype=np.uint8) if offsets[-1] else np.zeros(1, np.uint8)
    return data, offsets


def _threads(threads: int | None) -> int:
    return int(threads) if threads else (os.cpu_count() or 1)


def nfa_batch(nfa, data: np.ndarray, offsets: np.ndarray, threads: int | None = None,
              with_work: bool = False):
    """C oracle over a flat batch. Returns ``(flags, lens, examined, max_active)``, plus
    ``work`` (symbol edges scanned per input) and ``visits`` (active states stepped per
    input) when ``with_work``."""
    lib = _load()
    n_in = len(offsets) - 1
    acc = np.ascontiguousarray(nfa.accept, dtype=np.uint8)
    arrs = [np.ascontiguousarray(getattr(nfa, f), dtype=np.int32) for f in
            ("sym_row_ptr", "sym_targets", "sym_symbols", "eps_row_ptr", "eps_targets")]
    data = np.ascontiguousarray(data, dtype=np.uint8)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    flags = np.zeros(n_in, np.int32)
    lens = np.zeros(n_in, np.int32)
    examined = np.zeros(n_in, np.int64)
    peak = np.zeros(n_in, np.int32)
    work = np.zeros(n_in, np.int64)
    visits = np.zeros(n_in, np.int64)
    rc = lib.fsm_oracle_nfa_batch(int(nfa.num_states), int(nfa.start_state), _ptr(acc),
                                  *[_ptr(a) for a in arrs], _ptr(data), _ptr(offsets), n_in,
                                  _threads(threads), _ptr(flags), _ptr(lens), _ptr(examined),
                                  _ptr(peak), _ptr(work), _ptr(visits))
    if rc != 0:
        raise ValueError(f"oracle rejected the automaton or offsets (rc={rc})")
    if with_work:
        return flags, lens, examined, peak, work, visits
    return flags, lens, examined, peak


def dfa_batch(dfa, data: np.ndarray, offsets: np.ndarray, threads: int | None = None):
    """C oracle over a flat batch. Returns ``(flags, lens, examined)``."""
    lib = _load()
    n_in = len(offsets) - 1
    acc = np.ascontiguousarray(dfa.accept, dtype=np.uint8)
    trans = np.ascontiguousarray(dfa.trans, dtype=np.int32)
    data = np.ascontiguousarray(data, dtype=np.uint8)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    flags = np.zeros(n_in, np.int32)
    lens = np.zeros(n_in, np.int32)
    examined = np.zeros(n_in, np.int64)
    rc = lib.fsm_oracle_dfa_batch(int(dfa.num_states), int(dfa.start_state), _ptr(acc),
                                  _ptr(trans), _ptr(data), _ptr(offsets), n_in,
                                  _threads(threads), _ptr(flags), _ptr(lens), _ptr(examined))
    if rc != 0:
        raise ValueError(f"oracle rejected the automaton or offsets (rc={rc})")
    return flags, lens, examined


def walk_bytes(nfa, offsets: np.ndarray, seed: int, threads: int | None = None) -> np.ndarray:
    """Random-walk inputs for ``nfa``, byte-identical to the product library's generator;
    the CPU reference arm of the benchmark uses this one so that it loads no product code."""
    lib = _load()
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    total = int(offsets[-1])
    out = np.zeros(max(total, 1), dtype=np.uint8)
    arrs = [np.ascontiguousarray(getattr(nfa, f), dtype=np.int32) for f in
            ("sym_row_ptr", "sym_targets", "sym_symbols")]
    acc = np.ascontiguousarray(nfa.accept, dtype=np.uint8)
    rc = lib.fsm_oracle_walk(int(nfa.num_states), *[_ptr(a) for a in arrs], _ptr(acc),
                             int(nfa.start_state), _ptr(offsets), len(offsets) - 1,
                             int(seed) & (2**64 - 1), _ptr(out), _threads(threads))
    if rc != 0:
        raise ValueError(f"oracle walk rejected its arguments (rc={rc})")
    return out[:total]


def verdicts(automaton, inputs, threads: int | None = None) -> list[tuple[bool, int]]:
    """``[(accepted, match_len)]`` for a list of ``bytes`` through the C oracle."""
    data, offsets = flatten(inputs)
    if hasattr(automaton, "trans"):
        f, l, _ = dfa_batch(automaton, data, offsets, threads)
    else:
        f, l, _, _ = nfa_batch(automaton, data, offsets, threads)
    return [(bool(a), int(b)) for a, b in zip(f, l)]
