"""Technique choice: the feature rule, the measured table and its persistence (CPU), and
measurement on a probe batch (GPU)."""

from __future__ import annotations

import json

import numpy as np
import pytest

from abstraction_regret_gb300 import autotune as T
from abstraction_regret_gb300 import native
from abstraction_regret_gb300 import workloads as W


def _f(states, edges=None, eps=0, any_=False):
    edges = 2 * states if edges is None else edges
    return T.Features(states, -(-states // 64), edges, eps, any_, 16 * (edges + eps))


def test_rule_prefers_thread_per_input_bitmaps_for_small_automata_and_many_inputs():
    many = 8 * 152 * 32
    small = T.rule_plan(_f(300), many)
    assert small.technique == native.TECH_BITMAP
    big = T.rule_plan(_f(16384), many)
    assert big.technique == native.TECH_COMPACT and big.list_capacity == 128
    wild = T.rule_plan(_f(300, any_=True), many)
    assert wild.technique == native.TECH_COMPACT and wild.list_capacity == 256
    few = T.rule_plan(_f(300), 64)
    assert few.technique == native.TECH_COMPACT and few.block_threads == 64


def test_candidate_space_offers_bitmaps_only_for_small_sets():
    small = {p.technique for p in T.candidate_plans(_f(500))}
    large = {p.technique for p in T.candidate_plans(_f(60000))}
    assert native.TECH_BITMAP in small and native.TECH_BITMAP not in large
    assert {native.TECH_WARP, native.TECH_COMPACT} <= large


def test_measured_table_persists_and_separates_plain_from_persistent(tmp_path):
    path = tmp_path / "tune.json"
    t = T.Autotuner(path)
    f = _f(1024)
    choice = {"technique": native.TECH_WARP, "block_threads": 256, "list_capacity": 0,
              "stage": 1, "ms": 0.5}
    t.record(f, False, choice)
    assert t.lookup(f) == choice and t.lookup(f, persistent=True) is None
    again = T.Autotuner(path)
    assert again.lookup(f) == choice
    assert again.lookup(_f(1100)) == choice  # same feature bucket
    assert again.lookup(_f(4096)) is None
    path.write_text("{not json")
    assert T.Autotuner(path).table == {}
    assert json.loads(json.dumps(T.plan_dict(native.make_plan(native.TECH_COMPACT, 64, 128, 1))))


def test_a_measured_choice_overrides_the_rule(monkeypatch):
    nfa = W.random_nfa(1024, seed=0, degree=2)
    tuner = T.Autotuner()
    monkeypatch.setattr(T, "_DEFAULT", tuner)
    assert T.choose_nfa_plan(nfa, 64).technique == native.TECH_COMPACT
    tuner.record(T.features_of(nfa), False, {"technique": native.TECH_WARP, "block_threads": 256,
                                             "list_capacity": 0, "stage": 0})
    p = T.choose_nfa_plan(nfa, 64)
    assert p.technique == native.TECH_WARP and p.block_threads == 256
    choice = T.choose_nfa_plan(nfa, 64, persistent=True)
    assert choice.technique == native.TECH_COMPACT  # persistent entries are separate


@pytest.mark.gpu
def test_probe_batch_measurement_picks_a_plan_that_matches_the_oracle(tmp_path, monkeypatch):
    import torch

    import abstraction_regret_gb300 as G
    from abstraction_regret_gb300.device import DeviceNFA
    from abstraction_regret_gb300.executors import clear_cache
    from oracle import oracle as O

    b = W.c1("live")
    nfa = b.automata[0]
    dev = torch.device("cuda:0")
    d = DeviceNFA(nfa, dev)
    padded = np.zeros(-(-int(b.offsets[-1]) // 16) * 16 + 16, np.uint8)
    padded[: int(b.offsets[-1])] = b.data
    d_data = torch.from_numpy(padded).to(dev)
    d_off = torch.from_numpy(b.offsets.astype(np.int64)).to(dev)
    tuner = T.Autotuner(tmp_path / "t.json")
    monkeypatch.setattr(T, "_DEFAULT", tuner)
    res = tuner.tune_plain(d, d_data, d_off, b.n_inputs, repeats=2)
    assert res["best"]["ms"] == min(ms for _, ms in res["timings"])
    assert len(res["timings"]) == len(T.candidate_plans(T.features(d)))
    assert tuner.lookup(T.features(d)) == res["best"]
    clear_cache()
    got = [(r.accepted, r.match_len) for r in G.run_batch(nfa, b.inputs(), technique="auto")]
    assert got == O.verdicts(nfa, b.inputs())
