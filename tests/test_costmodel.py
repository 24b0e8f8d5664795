"""The cost model behind the autotuner's rules (abstraction_regret_gb300/costmodel.py),
on the CPU: residency and modelled traffic per technique (as the reference's
tests/test_costmodel.py checks its own), the two-constant fit, and the decisions the
rules take from it."""

from __future__ import annotations

import numpy as np
import pytest

from abstraction_regret_gb300 import autotune, costmodel, executors, native
from abstraction_regret_gb300 import workloads as W


def test_every_registered_nfa_technique_has_a_residency():
    missing = set(executors.NFA_NAMES) - set(costmodel.TECHNIQUE_KIND)
    assert not missing
    f = autotune.features_of(W.random_nfa(100, seed=1, degree=2))
    for name in executors.NFA_NAMES:
        assert costmodel.traffic_per_symbol(f, name) >= 0
    with pytest.raises(KeyError, match="no working-set residency"):
        costmodel.traffic_per_symbol(f, "no-such-technique")


def test_sets_leave_shared_memory_as_automata_grow():
    small = autotune.features_of(W.random_nfa(512, seed=1, degree=2))
    big = autotune.features_of(W.random_nfa(120_000, seed=1, degree=2))
    assert costmodel.residency(small, native.TECH_BITMAP) is costmodel.Residency.SHARED
    assert costmodel.residency(big, native.TECH_BITMAP) is costmodel.Residency.GLOBAL_WORD
    assert costmodel.residency(big, native.TECH_WARP, 256) is costmodel.Residency.GLOBAL_WORD
    assert costmodel.residency(big, -1) is costmodel.Residency.REGISTER
    # global sets add 4 words of traffic per state-word and symbol; shared ones none
    t_big = costmodel.traffic_per_symbol(big, "bitmap")
    assert t_big == costmodel.WS_TOUCHES * costmodel.words(120_000) * 8 + \
        costmodel.csr_traffic_per_symbol(big)
    assert costmodel.traffic_per_symbol(small, "bitmap") == costmodel.csr_traffic_per_symbol(small)
    assert costmodel.csr_traffic_per_symbol(small, staged=True) == 0


def test_csr_traffic_is_the_algorithmic_bytes_per_active_state():
    f = autotune.features_of(W.random_nfa(1000, seed=2, degree=4))
    assert costmodel.csr_traffic_per_symbol(f) == pytest.approx(8 + 8 * 4)
    assert costmodel.csr_traffic_per_symbol(f, active=3) == pytest.approx(3 * 40)


def test_fit_recovers_the_constants():
    rng = np.random.default_rng(0)
    traffic = rng.uniform(1e6, 1e9, 20)
    chains = rng.uniform(1e3, 1e6, 20)
    seconds = traffic / 5e12 + chains * 4e-7
    m = costmodel.fit(traffic, chains, seconds)
    assert m.eff_bandwidth_bytes_per_s == pytest.approx(5e12, rel=1e-6)
    assert m.step_s == pytest.approx(4e-7, rel=1e-6)
    chain_bound = costmodel.fit(traffic, chains, chains * 4e-7 - traffic * 1e-15)
    assert chain_bound.eff_bandwidth_bytes_per_s == float("inf")


class _Spec:
    """A device layout's features without a device."""

    def __init__(self, nfa, speculative=True):
        f = autotune.features_of(nfa)
        self.num_states, self.num_words = f.num_states, f.num_words
        self.num_sym_edges, self.num_eps_edges = f.num_edges, f.num_eps
        self.uses_any, self.edge_bytes, self.speculative = f.uses_any, 0, speculative


def test_engine_is_chosen_for_inputs_long_enough_to_cut():
    d = _Spec(W.random_nfa(16384, seed=2, poisson=4.0))
    c3 = np.diff(W.c3("literal").offsets)
    assert autotune.prefer_engine(d, c3)
    assert not autotune.prefer_engine(d, np.full(8, 100))
    assert autotune.prefer_engine(d, np.full(8, 4096))
    assert not autotune.prefer_engine(_Spec(W.random_nfa(64, seed=3, degree=2), False), c3)
    assert not autotune.prefer_engine(d, np.zeros(0, np.int64))


def test_rule_keeps_bitmaps_only_while_their_sets_fit_shared_memory():
    many = 8 * 152 * 32
    small = autotune.features_of(W.random_nfa(300, seed=4, degree=2))
    assert autotune.rule_plan(small, many).technique == native.TECH_BITMAP
    assert autotune.rule_plan(small, 10).technique == native.TECH_COMPACT
    big = autotune.features_of(W.random_nfa(5000, seed=4, degree=2))
    assert autotune.rule_plan(big, many).technique == native.TECH_COMPACT
