"""Host-side mirror of the reference interface, without a GPU.

Follows the reference's own CPU tests for the same surface: data model and builders
(tests/test_nfa.py, test_validation.py), packing (test_packing.py:37-96), registry and
dispatch (test_registry.py:47-172), result/benchmark conventions (test_api.py).
"""

from __future__ import annotations

import numpy as np
import pytest

import abstraction_regret_gb300 as G
from abstraction_regret_gb300 import registry as R
from abstraction_regret_gb300.packing import (
    WORD_BITS,
    accept_bitmask,
    pack_accept,
    pack_bytes,
    pack_inputs,
    symbols,
    words_for,
)
from abstraction_regret_gb300.result import BenchmarkStats, Result, batch_results


def _nfa(accepting=(), n=8):
    b = G.NFABuilder()
    for i in range(n):
        b.add_state(accept=i in accepting)
    b.set_start(0)
    return b.build()


@pytest.mark.parametrize(("n", "w"), [(1, 1), (63, 1), (64, 1), (65, 2), (128, 2), (129, 3),
                                      (500, 8)])
def test_words_for_rounds_up(n, w):
    assert words_for(n) == w


def test_symbols_and_pack_inputs_match_the_reference_layout():
    assert symbols(b"\x00A\xff").tolist() == [0, 65, 255]
    assert symbols(b"\x00A\xff").dtype == np.int32
    data, off = pack_inputs([b"ab", b"", b"xyz"])
    assert off.tolist() == [0, 2, 2, 5] and off.dtype == np.int32 and data.dtype == np.int32
    data, off = pack_inputs([b"", b""])
    assert data.size == 0 and off.tolist() == [0, 0, 0]
    data, off = pack_inputs([])
    assert data.size == 0 and off.tolist() == [0]


def test_pack_bytes_is_uint8_int64_and_padded():
    data, off = pack_bytes([b"ab", b"", b"xyz"])
    assert data.dtype == np.uint8 and off.dtype == np.int64
    assert off.tolist() == [0, 2, 2, 5]
    assert data.size % 16 == 0 and bytes(data[:5]) == b"abxyz"
    data, off = pack_bytes([])
    assert off.tolist() == [0] and data.size == 16


def test_pack_accept_spans_word_boundaries():
    acc = {0, 31, 32, 63, 64, 127, 128, 199}
    nfa = _nfa(acc, n=200)
    w = pack_accept(nfa)
    assert w.dtype == np.uint64 and w.size == words_for(200)
    got = {s for s in range(200) if int(w[s // WORD_BITS]) >> (s % WORD_BITS) & 1}
    assert got == acc
    assert int(pack_accept(_nfa({1, 5, 6}))[0]) == accept_bitmask(_nfa({1, 5, 6})) == 0b1100010
    assert pack_accept(_nfa({0}), nwords=8).size == 8
    assert pack_accept(_nfa({3}), dtype=np.int64).dtype == np.int64


def test_builder_validation_matches_the_reference():
    b = G.NFABuilder()
    with pytest.raises(ValueError):
        b.build()
    s = b.add_state()
    with pytest.raises(IndexError):
        b.add_transition(s, "a", 7)
    with pytest.raises(ValueError):
        b.add_transition(s, chr(256), s)
    with pytest.raises(ValueError):
        b.add_transition(s, "ab", s)
    with pytest.raises(ValueError):
        b.add_transition(s, 300, s)
    b.add_transition(s, G.ANY_SYMBOL, s)
    nfa = b.build()
    assert nfa.uses_any_symbol and nfa.num_sym_transitions == 1
    d = G.DFABuilder()
    with pytest.raises(ValueError):
        d.build()
    d.add_state()
    with pytest.raises(IndexError):
        d.add_transition(-1, 1, 0)
    with pytest.raises(ValueError):
        d.add_transition(0, 256, 0)
    dfa = d.build()
    assert dfa.num_states == 2 and dfa.trans.tolist() == [1] * 512  # the dead state


def test_random_dfa_matches_the_reference_draws():
    a = G.random_dfa(64, accept_prob=0.2, seed=3)
    rng = np.random.default_rng(3)
    assert np.array_equal(a.trans, rng.integers(0, 64, size=64 * 256, dtype=np.int32))
    acc = rng.random(64) < 0.2
    acc[0] = False
    assert np.array_equal(a.accept, acc)


def test_nfa_from_edges_equals_the_builder():
    b = G.NFABuilder()
    for i in range(4):
        b.add_state(accept=i == 3)
    for s, c, t in [(0, 1, 1), (2, 5, 3), (0, 9, 2), (1, 256, 0)]:
        b.add_transition(s, c, t)
    b.add_epsilon(1, 2)
    ref = b.build()
    got = G.nfa_from_edges(4, 0, ref.accept, [0, 2, 0, 1], [1, 5, 9, 256], [1, 3, 2, 0], [1], [2])
    for f in ("sym_row_ptr", "sym_targets", "sym_symbols", "eps_row_ptr", "eps_targets"):
        assert np.array_equal(getattr(got, f), getattr(ref, f)), f


def test_kind_dispatch_and_identity_hashing():
    nfa, dfa = _nfa(), G.random_dfa(4)
    assert G.Kind.of(nfa) is G.Kind.NFA and G.Kind.of(dfa) is G.Kind.DFA
    with pytest.raises(TypeError, match="expected an NFA or a DFA"):
        G.Kind.of("nope")
    assert {nfa: 1}[nfa] == 1 and {dfa: 2}[dfa] == 2
    assert nfa != _nfa()


def test_cuda_registers_both_kinds_with_declared_defaults():
    assert R.list_kinds(G.Backend.CUDA) == [G.Kind.NFA, G.Kind.DFA]
    assert "worklist_warp" in R.list_techniques(G.Backend.CUDA, G.Kind.NFA)
    assert R.get_factory(G.Kind.NFA, G.Backend.CUDA, None)[0] == "auto"
    assert R.get_factory(G.Kind.DFA, G.Backend.CUDA, None)[0] == "gather"
    pairs = {(k, b) for k, b, _ in R._REGISTRY}
    assert all(p in R._DEFAULTS for p in pairs)
    for (k, b), t in R._DEFAULTS.items():
        assert (k, b, t) in R._REGISTRY


def test_registry_errors_name_the_alternatives():
    with pytest.raises(KeyError, match="available: "):
        R.get_factory(G.Kind.DFA, G.Backend.CUDA, "bitmap")
    with pytest.raises(KeyError, match="has no nfa technique"):
        G.run(_nfa(), b"a", backend="cpu")
    with pytest.raises(RuntimeError, match="two defaults"):
        R.register(G.Kind.NFA, G.Backend.CUDA, "something_else", default=True)(lambda a, t: None)


def test_no_cpu_fallback_without_a_gpu():
    """Without a device the CUDA path fails loudly instead of computing on the host."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert not G.is_available(G.Backend.CUDA)
    assert "CUDA device" in (R.unavailable_reason(G.Backend.CUDA) or "")
    with pytest.raises(RuntimeError, match="CUDA device"):
        G.run(_nfa({1}), b"a")


def test_batch_results_and_benchmark_stats_conventions():
    res = batch_results([1, 0, 1], [3, 0, 0], kernel_ms=2.0, transfer_ms=0.5)
    assert [r.kernel_ms for r in res] == [2.0, 0.0, 0.0]
    assert res[0].total_ms == 2.5 and res[1].total_ms == 0.0
    assert res[0].matches(Result(True, 3)) and not res[0].matches(Result(True, 4))
    st = BenchmarkStats("cuda", "auto", True, 3, 3, [1.0, 2.0, 3.0])
    assert st.mean_ms == 2.0 and st.std_ms == pytest.approx(1.0)
    assert st.as_row()["backend"] == "cuda"
    with pytest.raises(ValueError):
        G.benchmark(_nfa(), b"a", repeats=0)


def test_lane_state_records_pack_labels_degree_and_flags():
    """gbfsm_lane_rec of each state: packed labels for <= 16 edges without ANY, else SLOW."""
    from abstraction_regret_gb300 import native
    from abstraction_regret_gb300.device import lane_state_records

    b = G.NFABuilder()
    for k in range(4):
        b.add_state(accept=(k == 2))
    b.set_start(0)
    for sym in (5, 7, 255):          # state 0: three edges, fast form
        b.add_transition(0, sym, 1)
    for sym in range(17):            # state 1: seventeen edges, slow (degree above 16)
        b.add_transition(1, sym, 2)
    b.add_transition(2, G.ANY_SYMBOL, 3)  # state 2: ANY edge, slow
    nfa = b.build()                  # state 3: no edges, fast with degree 0
    recs, ext = lane_state_records(nfa)
    srp = np.asarray(nfa.sym_row_ptr)
    x = recs[:, 0].astype(np.int64)
    assert list(x & 0x1FFFFFF) == [0, 1, 2, 3]
    assert list((x >> 30) & 1) == [0, 1, 1, 0]
    assert list((x >> 31) & 1) == [0, 0, 1, 0]
    assert (x[0] >> native.LANE_DEG_SHIFT) & 31 == 3 and (x[3] >> native.LANE_DEG_SHIFT) & 31 == 0
    assert list(recs[:, 1]) == list(srp[:-1])
    row0 = sorted(int(s) for s in np.asarray(nfa.sym_symbols)[srp[0]:srp[1]])
    packed = [(int(recs[0, 2]) >> (8 * j)) & 0xFF for j in range(3)]
    assert sorted(packed) == row0
    assert recs[1, 2] == srp[2] and recs[2, 2] == srp[3]  # slow form: row_end


def test_lane_chunk_size_fills_one_wave():
    """The auto lane chunk size is the smallest whose LANES tasks fit the resident warps."""
    from types import SimpleNamespace

    from abstraction_regret_gb300 import workloads as W
    from abstraction_regret_gb300.engine import (LANE_GROUP, LANE_WARPS_PER_SM, MIN_CHUNK,
                                                 PersistentEngine)

    eng = SimpleNamespace(sm_count=152)
    pick = PersistentEngine.auto_lane_chunk_bytes
    assert pick(eng, np.zeros(0, np.int64), np.zeros(0, np.int64)) == MIN_CHUNK
    assert pick(eng, np.full(8, 1000), np.zeros(8, np.int64)) == MIN_CHUNK
    lengths = W.log_uniform_lengths(np.random.default_rng([2, 1]), 2048, 256, 1 << 20)
    aut = np.zeros(lengths.size, np.int64)
    size = pick(eng, lengths, aut)
    warps = 152 * LANE_WARPS_PER_SM

    def tasks(s):
        return -(-int(np.maximum(1, -(-lengths // s)).sum()) // LANE_GROUP)

    assert size % 64 == 0 and tasks(size) <= warps < tasks(size - 64)


def test_lane_records_pack_edges_8_to_15_separately():
    from abstraction_regret_gb300 import native
    from abstraction_regret_gb300.device import lane_state_records

    b = G.NFABuilder()
    b.add_state()
    b.add_state()
    b.set_start(0)
    labels = [10 + k for k in range(12)]
    for sym in labels:
        b.add_transition(0, sym, 1)
    nfa = b.build()
    recs, ext = lane_state_records(nfa)
    srp = np.asarray(nfa.sym_row_ptr)
    got = np.asarray(nfa.sym_symbols)[srp[0]:srp[1]]
    assert (int(recs[0, 0]) >> native.LANE_DEG_SHIFT) & 31 == 12
    assert not (int(recs[0, 0]) >> 30) & 1
    words = [int(recs[0, 2]), int(recs[0, 3]), int(ext[0, 0]), int(ext[0, 1])]
    packed = [(words[k // 4] >> (8 * (k % 4))) & 0xFF for k in range(12)]
    assert packed == [int(s) for s in got]


def _planner(kinds, lane_ok, can_chunk, chunk_bytes=0):
    """A PersistentEngine with only the attributes its task planner reads (no device)."""
    from abstraction_regret_gb300.engine import PersistentEngine
    from abstraction_regret_gb300.registry import Kind

    eng = PersistentEngine.__new__(PersistentEngine)
    eng.automata = [object()] * len(kinds)
    eng.kinds = [Kind.NFA if k == "nfa" else Kind.DFA for k in kinds]
    eng.lane_ok = np.asarray(lane_ok, dtype=bool)
    eng.can_chunk = np.asarray(can_chunk, dtype=bool)
    eng.chunk_bytes = chunk_bytes
    eng.sm_count, eng.lane_warps_per_sm, eng.resident_warps = 152, 32, 152 * 16
    return eng


def test_task_plan_covers_every_input_exactly_once():
    """Lane chunks tile their inputs in even chunks, LANES tasks hold <= 32 chunks of one
    automaton, warp chunks and fix-ups match, and every input is resolved exactly once."""
    from abstraction_regret_gb300 import native

    rng = np.random.default_rng(4)
    # automaton 0: lanes; 1: warp chunks only; 2: not chunkable; 3: DFA
    eng = _planner(["nfa", "nfa", "nfa", "dfa"], [1, 0, 0, 0], [1, 1, 0, 0], chunk_bytes=512)
    n = 300
    aut = rng.integers(0, 4, n)
    lengths = rng.integers(0, 6000, n)
    starts = np.zeros(n, np.int64)
    np.cumsum(lengths[:-1], out=starts[1:])
    p = eng.make_tasks(aut, lengths)
    ch = p.chunks
    resolved = np.zeros(n, np.int64)
    # fix-ups: one per chunked input, its chunks tile the input
    for a_, first, count, kind in p.tasks_b.tolist():
        assert kind == native.TASK_FIXUP
        c = ch[first:first + count]
        i = int(c["input"][0])
        assert (c["input"] == i).all() and list(c["index"]) == list(range(count))
        assert c["begin"][0] == starts[i] and c["end"][-1] == starts[i] + lengths[i]
        assert (c["begin"][1:] == c["end"][:-1]).all()
        if count > 1:
            size = c["end"] - c["begin"]
            assert size.max() <= 512 and size.min() > 256
        assert aut[i] == a_
        resolved[i] += 1
    # lane chunks first, grouped in LANES tasks of one automaton
    covered = np.zeros(ch.shape[0], np.int64)
    for a_, first, count, kind in p.tasks_l.tolist():
        assert kind == native.TASK_LANES and 1 <= count <= 32 and first + count <= p.lane_chunks
        assert (aut[ch["input"][first:first + count]] == a_).all() and a_ == 0
        covered[first:first + count] += 1
    whole_nfa = 0
    for a_, first, count, kind in p.tasks_a.tolist():
        if kind == native.TASK_CHUNK:
            assert count == 1 and first >= p.lane_chunks and a_ == 1
            covered[first] += 1
        else:
            assert kind == native.TASK_WHOLE
            ids = p.input_ids[first:first + count]
            assert (aut[ids] == a_).all()
            if a_ == 3:
                assert count <= 32
            else:
                assert count == 1
                whole_nfa += 1
            resolved[ids] += 1
    assert (covered == 1).all()
    assert (resolved == 1).all()
    assert sorted(p.input_ids.tolist()) == list(range(n))


def test_pipeline_slices_are_contiguous_and_balanced():
    from abstraction_regret_gb300.engine import slice_bounds

    lengths = np.random.default_rng(1).integers(1, 10000, 500)
    off = np.zeros(501, np.int64)
    np.cumsum(lengths, out=off[1:])
    spans = slice_bounds(off, 8)
    assert spans[0][0] == 0 and spans[-1][1] == 500
    assert all(a < b for a, b in spans) and all(spans[k][1] == spans[k + 1][0]
                                                for k in range(len(spans) - 1))
    sizes = [off[b] - off[a] for a, b in spans]
    assert len(spans) == 8 and max(sizes) < 1.3 * off[-1] / 8
    assert slice_bounds(off[:2], 8) == [(0, 1)]


def test_per_input_lane_chunk_sizes():
    """The pipelined path gives later slices shorter lane chunks, per input."""
    eng = _planner(["nfa"], [1], [1])
    lengths = np.array([10000, 10000, 10000])
    sizes = np.array([2048, 1024, 512])
    p = eng.make_tasks(np.zeros(3, np.int64), lengths, lane_chunk=sizes)
    for i, size in enumerate(sizes.tolist()):
        c = p.chunks[p.chunks["input"] == i]
        assert len(c) == -(-10000 // size)
        assert (c["end"] - c["begin"]).max() <= size


def test_input_addresses_equal_ctypes_for_every_input_kind():
    """The gather path's address table: plain bytes through id() and the header offset,
    anything else through the buffer protocol; both give each input's own storage."""
    from abstraction_regret_gb300 import staging as S

    plain = [bytes(k) for k in range(50)] + [b"", b"abc" * 100]
    mixed = plain + [bytearray(b"xyz"), memoryview(b"0123456789")[2:7]]
    for inputs in (plain, mixed):
        out = np.zeros(len(inputs), np.int64)
        S.addresses(inputs, out)
        assert [int(a) for a in out] == [S._address(b) for b in inputs]


def test_batch_results_values_and_timing_convention():
    """Verdicts from arrays or lists; the batch's times on the first result only."""
    from abstraction_regret_gb300.result import Result, batch_results

    for flags, lens in ((np.array([1, 0, 1], np.int32), np.array([3, 0, 7], np.int32)),
                        ([True, False, True], [3, 0, 7])):
        res = batch_results(flags, lens, 2.0, 0.5)
        assert [(r.accepted, r.match_len) for r in res] == [(True, 3), (False, 0), (True, 7)]
        assert all(type(r.accepted) is bool and type(r.match_len) is int for r in res)
        assert (res[0].kernel_ms, res[0].total_ms, res[0].transfer_ms) == (2.0, 2.5, 0.5)
        assert all(r.kernel_ms == r.total_ms == r.transfer_ms == 0.0 for r in res[1:])
        assert isinstance(res[0], Result)
    assert batch_results([], [], 1.0) == []


def test_fill_results_equal_batch_results():
    """Results built before the verdicts and filled afterwards equal batch_results's."""
    from abstraction_regret_gb300.executors import run_batch_results
    from abstraction_regret_gb300.result import batch_results, blank_results, fill_results

    rng = np.random.default_rng(1)
    flags = rng.integers(0, 2, 50).astype(np.int32)
    lens = rng.integers(0, 1000, 50).astype(np.int32)
    for n in (0, 1, 50):
        got = fill_results(blank_results(n), flags[:n], lens[:n], 3.0, 0.25)
        assert got == batch_results(flags[:n], lens[:n], 3.0, 0.25)
        assert got == fill_results(blank_results(n), flags[:n].tolist(), lens[:n].tolist(),
                                   3.0, 0.25)
    with pytest.raises(ValueError):
        fill_results(blank_results(2), flags[:3], lens[:3], 1.0)

    class Stand:
        calls = 0

        def run_arrays(self, inputs, idle=None):
            if idle is not None:
                Stand.calls += 1
                idle()
            return flags[:len(inputs)], lens[:len(inputs)], None, 2.0, 1.0

    assert run_batch_results(Stand(), []) == []
    assert run_batch_results(Stand(), [b"a"] * 7) == batch_results(flags[:7], lens[:7], 2.0, 1.0)
    assert Stand.calls == 1
