"""The ANML loader (abstraction_regret_gb300.anml) against the reference's own loader.

tests/golden/anml_cases.json.gz holds what gpufsm 0.1.0's ``gpufsm.io.anml.load_anml``
made of each document (its CSR arrays, or the ValueError it raised) and the verdicts of
``gpufsm.reference.simulate`` on sample inputs (written by
tests/golden/make_anml_golden.py). The loader must build the same automaton -- the same
states, accept bits, epsilon edges and, row by row, the same (symbol, target) edges --
refuse the same documents, and the oracle must give the recorded verdicts on it.
"""

from __future__ import annotations

import numpy as np
import pytest

from abstraction_regret_gb300 import ANY_SYMBOL
from abstraction_regret_gb300 import anml
from abstraction_regret_gb300 import workloads as W
from oracle import oracle as O

from .golden.make_anml_golden import row_digest
from .golden_data import load, nfa_from


def _cases():
    return load("anml_cases.json.gz")["cases"]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["id"])
def test_documents_match_the_reference_loader(case):
    if "error" in case:
        with pytest.raises(ValueError) as exc:
            anml.load_anml_string(case["anml"])
        want = case["message"].replace("<file>: ", "").replace(" in <file>", "")
        assert want in str(exc.value)
        return
    ours = anml.load_anml_string(case["anml"])
    ref = nfa_from(case["nfa"])
    assert row_digest(ours) == case["digest"] == row_digest(ref)
    inputs = [bytes.fromhex(x) for x in case["inputs_hex"]]
    want = [tuple(v) for v in case["verdicts"]]
    assert [O.simulate(ours, x) for x in inputs] == want
    assert O.verdicts(ours, inputs) == want


@pytest.mark.parametrize("idx", range(3))
def test_synthetic_pattern_automata_match_the_reference_loader(idx):
    s = load("anml_cases.json.gz")["synthetic"][idx]
    nfa = anml.load_anml_string(W.anml_patterns(s["patterns"], seed=s["seed"]))
    assert nfa.num_states == s["num_states"] and nfa.sym_targets.size == s["num_edges"]
    assert row_digest(nfa) == s["digest"]
    inputs = [bytes.fromhex(x) for x in s["inputs_hex"]]
    assert O.verdicts(nfa, inputs) == [tuple(v) for v in s["verdicts"]]


def test_symbol_set_forms():
    assert anml.parse_symbol_set("*").tolist() == [ANY_SYMBOL]
    assert anml.parse_symbol_set("[0x61-0x63]").tolist() == [97, 98, 99]
    assert anml.parse_symbol_set(" [abc] ").tolist() == [97, 98, 99]
    assert anml.parse_symbol_set("\\x41").tolist() == [65]
    assert anml.parse_symbol_set("[a-]").tolist() == [45, 97]
    neg = anml.parse_symbol_set("[^0x61]")
    assert neg.size == 255 and 97 not in neg.tolist()
    assert anml.parse_symbol_set("[^]").tolist() == list(range(256))
    for bad in ("[]", "[z-a]", "[0x4]", "ab", "[\\x4g]"):
        with pytest.raises(ValueError):
            anml.parse_symbol_set(bad)


def test_file_and_string_give_the_same_automaton(tmp_path):
    text = W.anml_patterns(10, seed=4)
    path = tmp_path / "p.anml"
    path.write_text(text)
    a, b = anml.load_anml(path), anml.load_anml_string(text)
    for f in ("sym_row_ptr", "sym_targets", "sym_symbols", "eps_row_ptr", "eps_targets",
              "accept"):
        assert np.array_equal(getattr(a, f), getattr(b, f))
