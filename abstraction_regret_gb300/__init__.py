"""GB300-native automata-simulation engine (sm_103a), a drop-in for gpufsm's CUDA backend.

The same API as gpufsm 0.1.0 (alepot55/abstraction-regret, ``src/gpufsm/__init__.py``)::

    from abstraction_regret_gb300 import NFABuilder, run, run_batch, random_dfa

    b = NFABuilder()
    s0 = b.add_state(); s1 = b.add_state(accept=True)
    b.set_start(s0); b.add_transition(s0, "a", s1)
    nfa = b.build()
    run(nfa, b"a")                         # Result(accepted=True, match_len=1, ...)
    run_batch(random_dfa(1024, seed=0), [b"abc", b"xyz"])

Every technique runs on the GPU through ``libgbfsm.so`` (hand-written sm_103a kernels
behind a C ABI, ``include/gbfsm.h``); there is no CPU path. To serve gpufsm's own API,
``abstraction_regret_gb300.plugin.install()`` registers the same techniques into
gpufsm's registry under ``Backend.CUDA``.
"""

from __future__ import annotations

from .api import benchmark, run, run_batch
from .automata import ANY_SYMBOL, DFA, NFA, DFABuilder, NFABuilder, nfa_from_edges, random_dfa
from .engine import GraphRunner, NfaChoice, PersistentEngine
from .registry import (
    Backend,
    Kind,
    available_backends,
    is_available,
    list_kinds,
    list_techniques,
)
from .result import BenchmarkStats, Result

__version__ = "0.1.0"

__all__ = [
    "ANY_SYMBOL",
    "NFA",
    "NFABuilder",
    "DFA",
    "DFABuilder",
    "random_dfa",
    "nfa_from_edges",
    "Backend",
    "Kind",
    "Result",
    "BenchmarkStats",
    "run",
    "run_batch",
    "benchmark",
    "available_backends",
    "is_available",
    "list_kinds",
    "list_techniques",
    "PersistentEngine",
    "GraphRunner",
    "NfaChoice",
]
