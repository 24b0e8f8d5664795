"""Automaton data model: the CSR NFA and the dense-table DFA the engine consumes.

The layouts are the reference's own, so an automaton built for gpufsm 0.1.0 runs here
unchanged (and an automaton built here is accepted by gpufsm):

* ``NFA`` -- ``src/gpufsm/core/nfa.py:43-84``. CSR over symbol edges
  (``sym_row_ptr`` int32[n+1], ``sym_targets`` / ``sym_symbols`` int32[nnz], symbols
  0..255 or ``ANY_SYMBOL`` = 256) and epsilon edges (``eps_row_ptr`` int32[n+1],
  ``eps_targets`` int32[nnz_eps]); ``accept`` bool[n]. Identity equality and hashing
  (``eq=False``), so automata key executor caches.
* ``DFA`` -- ``src/gpufsm/core/dfa.py:25-41``. ``trans`` int32[n*256] with
  ``trans[s*256 + c]`` the successor of ``s`` on byte ``c``; ``accept`` bool[n].
* ``random_dfa`` -- ``src/gpufsm/core/dfa.py:44-57``: the same draws in the same order
  from ``numpy.random.default_rng(seed)``, so a seed names the same table in both
  packages (tests pin this against the reference's own output).

The engine never reads these objects on the device; ``device.py`` derives the
GPU-resident layout from them once per automaton.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

ANY_SYMBOL = 256
"""Wildcard label: an edge with this symbol matches every input byte."""

ALPHABET = 256
"""Row width of the DFA table: one successor per byte value."""


def _symbol_id(symbol: int | str) -> int:
    """Normalise an edge label to 0..255 or ANY_SYMBOL (reference: core/nfa.py:20-40).

    A one-character string stands for its code point, which must be a byte; ``chr(256)``
    is rejected rather than silently becoming the wildcard.
    """
    if isinstance(symbol, str):
        if len(symbol) != 1:
            raise ValueError(f"symbol string must be a single char, got {symbol!r}")
        code = ord(symbol)
        if code > 255:
            raise ValueError(
                f"symbol {symbol!r} has code point {code}; edges are labelled with bytes "
                f"(0..255). Encode the text first, or pass ANY_SYMBOL for a wildcard."
            )
        return code
    value = int(symbol)
    if value == ANY_SYMBOL or 0 <= value <= 255:
        return value
    raise ValueError(f"symbol must be 0..255 or ANY_SYMBOL, got {symbol}")


@dataclass(frozen=True, eq=False)
class NFA:
    """Immutable CSR NFA. Build one with :class:`NFABuilder` or from arrays directly."""

    num_states: int
    start_state: int
    accept: np.ndarray  # bool [num_states]
    sym_row_ptr: np.ndarray  # int32 [num_states + 1]
    sym_targets: np.ndarray  # int32 [nnz_sym]
    sym_symbols: np.ndarray  # int32 [nnz_sym], 0..255 or ANY_SYMBOL
    eps_row_ptr: np.ndarray  # int32 [num_states + 1]
    eps_targets: np.ndarray  # int32 [nnz_eps]

    @property
    def uses_any_symbol(self) -> bool:
        return bool(np.any(self.sym_symbols == ANY_SYMBOL))

    @property
    def num_sym_transitions(self) -> int:
        return int(self.sym_targets.size)

    @property
    def num_eps_transitions(self) -> int:
        return int(self.eps_targets.size)

    def __repr__(self) -> str:  # pragma: no cover - cosmetic
        return (
            f"NFA(states={self.num_states}, start={self.start_state}, "
            f"accept={int(np.count_nonzero(self.accept))}, "
            f"sym={self.num_sym_transitions}, eps={self.num_eps_transitions})"
        )


def nfa_from_edges(
    num_states: int,
    start_state: int,
    accept: np.ndarray,
    src: np.ndarray,
    symbols: np.ndarray,
    dst: np.ndarray,
    eps_src: np.ndarray | None = None,
    eps_dst: np.ndarray | None = None,
) -> NFA:
    """Vectorised CSR construction from edge lists (stable in the given edge order).

    ``NFABuilder`` is a per-edge Python loop; the synthetic workloads (up to 65536 states
    and ~0.5 M edges) are built with this instead. Edge order within a row is the order of
    appearance, which is what ``NFABuilder.build`` produces as well.
    """
    n = int(num_states)
    src = np.asarray(src, dtype=np.int64)
    order = np.argsort(src, kind="stable")
    counts = np.bincount(src, minlength=n)
    row = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(counts, out=row[1:])
    if eps_src is None:
        eps_src = np.zeros(0, np.int64)
        eps_dst = np.zeros(0, np.int32)
    eps_src = np.asarray(eps_src, dtype=np.int64)
    eorder = np.argsort(eps_src, kind="stable")
    erow = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(np.bincount(eps_src, minlength=n), out=erow[1:])
    return NFA(
        num_states=n,
        start_state=int(start_state),
        accept=np.asarray(accept, dtype=bool).copy(),
        sym_row_ptr=row,
        sym_targets=np.asarray(dst, dtype=np.int32)[order].copy(),
        sym_symbols=np.asarray(symbols, dtype=np.int32)[order].copy(),
        eps_row_ptr=erow,
        eps_targets=np.asarray(eps_dst, dtype=np.int32)[eorder].copy(),
    )


class NFABuilder:
    """Mutable builder that finalises into an immutable CSR :class:`NFA`
    (reference: core/nfa.py:87-157; same method names, checks and exceptions)."""

    def __init__(self) -> None:
        self._accepting: list[bool] = []
        self._edges: list[list[tuple[int, int]]] = []
        self._eps: list[list[int]] = []
        self._start = 0

    def add_state(self, accept: bool = False) -> int:
        self._accepting.append(bool(accept))
        self._edges.append([])
        self._eps.append([])
        return len(self._accepting) - 1

    def set_start(self, state: int) -> None:
        self._require(state)
        self._start = state

    def set_accept(self, state: int, accept: bool = True) -> None:
        self._require(state)
        self._accepting[state] = bool(accept)

    def add_transition(self, src: int, symbol: int | str, dst: int) -> None:
        self._require(src)
        self._require(dst)
        self._edges[src].append((_symbol_id(symbol), dst))

    def add_epsilon(self, src: int, dst: int) -> None:
        self._require(src)
        self._require(dst)
        self._eps[src].append(dst)

    def build(self) -> NFA:
        n = len(self._accepting)
        if n == 0:
            raise ValueError("cannot build an NFA with zero states")
        row = np.zeros(n + 1, dtype=np.int32)
        row[1:] = np.cumsum([len(e) for e in self._edges])
        erow = np.zeros(n + 1, dtype=np.int32)
        erow[1:] = np.cumsum([len(e) for e in self._eps])
        flat = [edge for edges in self._edges for edge in edges]
        syms = np.array([s for s, _ in flat], dtype=np.int32)
        tgts = np.array([t for _, t in flat], dtype=np.int32)
        etgts = np.array([t for targets in self._eps for t in targets], dtype=np.int32)
        return NFA(
            num_states=n,
            start_state=self._start,
            accept=np.array(self._accepting, dtype=bool),
            sym_row_ptr=row,
            sym_targets=tgts,
            sym_symbols=syms,
            eps_row_ptr=erow,
            eps_targets=etgts,
        )

    def _require(self, state: int) -> None:
        if not 0 <= state < len(self._accepting):
            raise IndexError(f"state {state} out of range (0..{len(self._accepting) - 1})")


@dataclass(frozen=True, eq=False)
class DFA:
    """Total DFA over bytes with a dense int32 table ``trans[s * 256 + c]``.

    Identity equality and hashing, as for :class:`NFA`, so DFAs key executor caches.
    """

    num_states: int
    start_state: int
    accept: np.ndarray  # bool [num_states]
    trans: np.ndarray  # int32 [num_states * 256]

    @property
    def table_bytes(self) -> int:
        return int(self.trans.size) * self.trans.itemsize


def random_dfa(num_states: int, *, accept_prob: float = 0.05, seed: int = 0) -> DFA:
    """Random total DFA with uniform successors; start 0 is never accepting.

    Draw order matches the reference's ``random_dfa`` (core/dfa.py:44-57): the table
    first (``integers(0, n, n*256, int32)``), then one ``random()`` per state.
    """
    if num_states < 1:
        raise ValueError("num_states must be >= 1")
    rng = np.random.default_rng(seed)
    trans = rng.integers(0, num_states, size=num_states * ALPHABET, dtype=np.int32)
    accept = rng.random(num_states) < accept_prob
    accept[0] = False
    return DFA(num_states=num_states, start_state=0, accept=accept, trans=trans)


class DFABuilder:
    """Incremental DFA; unset edges lead to an extra absorbing, non-accepting dead state
    (reference: core/dfa.py:60-110, including its bounds checks)."""

    def __init__(self) -> None:
        self._accepting: list[bool] = []
        self._edges: list[dict[int, int]] = []
        self._start = 0

    def add_state(self, accept: bool = False) -> int:
        self._accepting.append(bool(accept))
        self._edges.append({})
        return len(self._accepting) - 1

    def _require(self, state: int) -> None:
        if not 0 <= state < len(self._accepting):
            raise IndexError(f"state {state} out of range (0..{len(self._accepting) - 1})")

    def set_start(self, state: int) -> None:
        self._require(state)
        self._start = state

    def add_transition(self, src: int, symbol: int, dst: int) -> None:
        self._require(src)
        self._require(dst)
        if not 0 <= symbol < ALPHABET:
            raise ValueError(f"symbol must be 0..255, got {symbol}")
        self._edges[src][symbol] = dst

    def build(self) -> DFA:
        n = len(self._accepting)
        if n == 0:
            raise ValueError("cannot build a DFA with zero states")
        dead = n
        table = np.full((n + 1, ALPHABET), dead, dtype=np.int32)
        for s, edges in enumerate(self._edges):
            for c, d in edges.items():
                table[s, c] = d
        accept = np.zeros(n + 1, dtype=bool)
        accept[:n] = self._accepting
        return DFA(num_states=n + 1, start_state=self._start, accept=accept,
                   trans=table.reshape(-1))
