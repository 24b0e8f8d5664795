"""Bit-exact parity of every CUDA technique with the reference's oracle (GPU).

Verdicts are integers, so the tolerance is zero: every ``(accepted, match_len)`` must
equal the golden verdict (produced by the reference's ``simulate`` / ``simulate_dfa``)
or the CPU oracle's on the same seeded inputs. All calls go through the C ABI of
libgbfsm (the executors call ``gbfsm_nfa_run`` / ``gbfsm_dfa_run`` /
``gbfsm_persistent_run``; the host-array entry points are called directly).
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import abstraction_regret_gb300 as G
from abstraction_regret_gb300 import native
from abstraction_regret_gb300 import workloads as W
from abstraction_regret_gb300.engine import NfaChoice, PersistentEngine
from abstraction_regret_gb300.executors import CudaDFAExecutor, CudaNFAExecutor
from abstraction_regret_gb300.packing import pack_accept, pack_inputs
from oracle import oracle as O

from .golden_data import grouped

pytestmark = pytest.mark.gpu

NFA_TECHS = G.list_techniques(G.Backend.CUDA, G.Kind.NFA)
DFA_TECHS = G.list_techniques(G.Backend.CUDA, G.Kind.DFA)


def verdicts(results):
    return [(r.accepted, r.match_len) for r in results]


@pytest.mark.parametrize("technique", NFA_TECHS)
def test_nfa_golden_corpus_every_technique(technique):
    for a, cases in grouped("nfa"):
        got = verdicts(G.run_batch(a, [d for _, d, _ in cases], technique=technique))
        want = [tuple(v) for _, _, v in cases]
        bad = [(cid, g, w) for (cid, _, _), g, w in zip(cases, got, want) if g != w]
        assert not bad, f"{technique}: {bad[:3]}"


@pytest.mark.parametrize("technique", DFA_TECHS)
def test_dfa_golden_corpus_every_technique(technique):
    for a, cases in grouped("dfa"):
        got = verdicts(G.run_batch(a, [d for _, d, _ in cases], technique=technique))
        want = [tuple(v) for _, _, v in cases]
        assert got == want, technique


def test_single_run_matches_batch_and_timing_convention():
    a, cases = grouped("nfa")[0]
    res = G.run_batch(a, [d for _, d, _ in cases])
    assert res[0].kernel_ms > 0 and all(r.kernel_ms == 0 for r in res[1:])
    for (_, d, v) in cases:
        r = G.run(a, d)
        assert (r.accepted, r.match_len) == tuple(v)


def test_every_golden_automaton_in_one_persistent_launch():
    """NFAs and DFAs of different sizes mixed in a single launch (the c4/c5 shape)."""
    groups = grouped("nfa") + grouped("dfa")
    automata = [a for a, _ in groups]
    aut_ids, inputs, want = [], [], []
    for k, (_, cases) in enumerate(groups):
        for _, d, v in cases:
            aut_ids.append(k)
            inputs.append(d)
            want.append(tuple(v))
    for tech, cap in ((native.TECH_COMPACT, 8), (native.TECH_COMPACT, 128), (native.TECH_WARP, 0)):
        choices = [NfaChoice(tech, max(cap, 1)) for _ in automata]
        eng = PersistentEngine(automata, choices=choices, list_capacity=max(cap, 1))
        flags, lens, ex, _, _ = eng.run_requests(aut_ids, inputs, with_examined=True)
        got = list(zip(flags.astype(bool).tolist(), lens.tolist()))
        assert got == want, (tech, cap)
        assert all(0 <= e <= len(d) for e, d in zip(ex.tolist(), inputs))


def test_empty_and_unaligned_batches():
    a, cases = grouped("nfa")[5]
    for tech in ("bitmap", "warp", "compact", "persistent"):
        assert G.run_batch(a, [], technique=tech) == []
        res = G.run_batch(a, [b"", b"", b""], technique=tech)
        want = O.simulate(a, b"")
        assert verdicts(res) == [want] * 3
    dfa = G.random_dfa(300, accept_prob=0.01, seed=4)
    rng = np.random.default_rng(1)
    inputs = [rng.integers(0, 256, k, dtype=np.uint8).tobytes() for k in
              (0, 1, 15, 16, 17, 31, 33, 255, 1000, 4099)]
    for tech in DFA_TECHS:
        assert verdicts(G.run_batch(dfa, inputs, technique=tech)) == [O.simulate_dfa(dfa, x) for x in inputs]


def test_sparse_list_overflow_and_staging_paths():
    """Small list capacities force sparse->dense->sparse switches mid-input."""
    for a, cases in grouped("nfa")[-60:]:
        inputs = [d for _, d, _ in cases]
        want = [tuple(v) for _, _, v in cases]
        for cap in (1, 2, 5):
            for stage in (0, 1):
                for threads in (32, 96):
                    plan = native.make_plan(native.TECH_COMPACT, threads, cap, stage)
                    ex = CudaNFAExecutor(a, plan=plan)
                    assert verdicts(ex.run_batch(inputs)) == want, (cap, stage, threads)


def _host_nfa_args(nfa):
    arrs = [np.ascontiguousarray(getattr(nfa, f), dtype=np.int32) for f in
            ("sym_row_ptr", "sym_targets", "sym_symbols", "eps_row_ptr", "eps_targets")]
    return arrs, np.ascontiguousarray(pack_accept(nfa), dtype=np.uint64)


def _ptr(a):
    return a.ctypes.data if a.size else None


@pytest.mark.parametrize("entry", ["gbfsm_run_multistream", "gbfsm_run_multistream_shared",
                                   "gbfsm_run_multistream_async", "gbfsm_run_worklist",
                                   "gbfsm_run_worklist_global", "gbfsm_run_worklist_warp",
                                   "gbfsm_run_worklist_compact", "gbfsm_run_worklist_shared"])
def test_reference_shaped_host_entry_points(entry):
    """The C-ABI functions that stand in for _cuda.run_* (host arrays in and out)."""
    lib = native.lib()
    fn = getattr(lib, entry)
    for a, cases in grouped("nfa")[::7]:
        arrs, acc = _host_nfa_args(a)
        data, off = pack_inputs([d for _, d, _ in cases])
        n = len(cases)
        flags = np.zeros(n, np.int32)
        lens = np.zeros(n, np.int32)
        ms = ctypes.c_float(0)
        st = fn(*[_ptr(x) for x in arrs], _ptr(acc), _ptr(data), _ptr(off), n, a.num_states,
                a.start_state, int(a.uses_any_symbol), _ptr(flags), _ptr(lens), ctypes.byref(ms))
        native.check(st, entry)
        assert list(zip(flags.astype(bool).tolist(), lens.tolist())) == [tuple(v) for *_, v in cases]
        assert ms.value > 0


def test_reference_shaped_single_and_dfa_entry_points():
    lib = native.lib()
    for a, cases in grouped("nfa")[::11]:
        arrs, acc = _host_nfa_args(a)
        acc8 = np.ascontiguousarray(a.accept, dtype=np.int8)
        for _, d, v in cases:
            syms = np.frombuffer(d, np.uint8).astype(np.int32)
            for fn, accept in ((lib.gbfsm_run_dense, acc8), (lib.gbfsm_run_bitpacked, acc)):
                f, l, ms = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_float()
                st = fn(*[_ptr(x) for x in arrs], _ptr(accept), _ptr(syms), syms.size,
                        a.num_states, a.start_state, 0, ctypes.byref(f), ctypes.byref(l),
                        ctypes.byref(ms))
                native.check(st, "single-input entry")
                assert (bool(f.value), l.value) == tuple(v)
    for a, cases in grouped("dfa"):
        data, off = pack_inputs([d for _, d, _ in cases])
        n = len(cases)
        flags, lens, ms = np.zeros(n, np.int32), np.zeros(n, np.int32), ctypes.c_float()
        trans = np.ascontiguousarray(a.trans, np.int32)
        acc = np.ascontiguousarray(a.accept, np.int8)
        st = lib.gbfsm_run_dfa(_ptr(trans), _ptr(acc), _ptr(data), _ptr(off), n, a.num_states,
                               a.start_state, _ptr(flags), _ptr(lens), ctypes.byref(ms))
        native.check(st, "gbfsm_run_dfa")
        assert list(zip(flags.astype(bool).tolist(), lens.tolist())) == [tuple(v) for *_, v in cases]


def test_invalid_automata_are_rejected_before_any_launch():
    b = G.NFABuilder()
    b.add_state()
    good = b.build()
    bad = G.NFA(num_states=1, start_state=0, accept=good.accept,
                sym_row_ptr=np.array([0, 1], np.int32), sym_targets=np.array([3], np.int32),
                sym_symbols=np.array([7], np.int32), eps_row_ptr=good.eps_row_ptr,
                eps_targets=good.eps_targets)
    with pytest.raises(ValueError, match="invalid NFA"):
        CudaNFAExecutor(bad, "compact")
    d = G.random_dfa(8)
    bad_dfa = G.DFA(num_states=8, start_state=0, accept=d.accept, trans=d.trans.copy() + 8)
    with pytest.raises(ValueError, match="invalid DFA"):
        CudaDFAExecutor(bad_dfa)


# ---- benchmark configurations at full size, against the C oracle ------------------------

def _check_batch(b, runner, check_examined=True):
    flags, lens, ex = runner(b)
    for k, a in enumerate(b.automata):
        sel = np.flatnonzero(b.aut_ids == k)
        sb = b.subset(sel)
        if hasattr(a, "trans"):
            f, l, e = O.dfa_batch(a, sb.data, sb.offsets)
        else:
            f, l, e, _ = O.nfa_batch(a, sb.data, sb.offsets)
        assert np.array_equal(flags[sel], f), b.name
        assert np.array_equal(lens[sel], l), b.name
        if check_examined:
            assert np.array_equal(ex[sel], e), b.name


def _persistent(b):
    eng = PersistentEngine(b.automata)
    f, l, e, _, _ = eng.run_requests(b.aut_ids, b.inputs(), with_examined=True)
    return f, l, e


def _plain(tech):
    def run(b):
        ex = G.executors.make_nfa_executor(b.automata[0], tech) if not hasattr(
            b.automata[0], "trans") else G.executors.make_dfa_executor(b.automata[0], tech)
        f, l, e, _, _ = ex.run_arrays(b.inputs(), with_examined=True)
        return f, l, e
    return run


@pytest.mark.parametrize("variant", ["literal", "live", "sustained"])
def test_c1_full(variant):
    b = W.c1(variant)
    for tech in ("bitmap", "warp", "compact", "persistent", "auto"):
        _check_batch(b, _plain(tech))


@pytest.mark.parametrize("variant", ["literal", "sustained"])
def test_c2_full(variant):
    b = W.c2(variant)
    assert b.n_inputs == 4096
    for tech in DFA_TECHS:
        _check_batch(b, _plain(tech))
    _check_batch(b, _persistent)


@pytest.mark.parametrize("variant", ["literal", "live", "sustained"])
def test_c3_full(variant):
    b = W.c3(variant)
    _check_batch(b, _persistent)
    _check_batch(b, _plain("compact"))


@pytest.mark.parametrize("variant", ["literal", "live", "sustained"])
def test_c4_all_pairs_one_launch(variant):
    b = W.c4(variant)
    assert b.n_inputs == 1024
    _check_batch(b, _persistent)


# ---- speculative chunking in the persistent engine ------------------------------------

@pytest.mark.parametrize("chunk", [256, 1000, 4096])
def test_chunked_persistent_matches_oracle_on_live_walks(chunk):
    b = W.c1("live")
    for a in (b.automata[0], W.without_accepts(b.automata[0])):
        eng = PersistentEngine([a], chunk_bytes=chunk)
        plan = eng.make_tasks(np.zeros(b.n_inputs, np.int64), np.diff(b.offsets))
        # lane automata chunk every input; warp-chunked ones only inputs of two chunks
        chunked = chunk <= 2048 or bool(eng.lane_ok[0])
        assert plan.tasks_b.shape[0] == (b.n_inputs if chunked else 0)
        f, l, e, _, _ = eng.run_requests(np.zeros(b.n_inputs), b.inputs(), with_examined=True)
        of, ol, oe, _ = O.nfa_batch(a, b.data, b.offsets)
        assert np.array_equal(f, of) and np.array_equal(l, ol) and np.array_equal(e, oe)


def test_chunked_persistent_with_epsilon_and_wildcards():
    import random

    rng = random.Random(5)
    automata, reqs = [], []
    for k in range(12):
        b = G.NFABuilder()
        n = rng.randint(2, 300)
        for _ in range(n):
            b.add_state(accept=rng.random() < 0.004)
        b.set_start(rng.randrange(n))
        for s in range(n):
            for _ in range(rng.randint(1, 4)):
                sym = G.ANY_SYMBOL if rng.random() < 0.03 else ord(rng.choice("abcd"))
                b.add_transition(s, sym, rng.randrange(n))
            for _ in range(rng.randint(0, 1)):
                b.add_epsilon(s, rng.randrange(n))
        automata.append(b.build())
        for _ in range(6):
            reqs.append((k, bytes(ord(rng.choice("abcd")) for _ in range(rng.randint(0, 3000)))))
    for chunk in (256, 700):
        eng = PersistentEngine(automata, chunk_bytes=chunk)
        f, l, _, _, _ = eng.run_requests([a for a, _ in reqs], [d for _, d in reqs])
        want = [O.simulate(automata[a], d) for a, d in reqs]
        assert list(zip(f.astype(bool).tolist(), l.tolist())) == want, chunk


@pytest.mark.parametrize("variant", ["live", "sustained"])
@pytest.mark.parametrize("lanes", [True, False])
def test_c3_chunked_small_chunks(variant, lanes):
    """Lane chunks (with sets that outgrow a lane spilling to warps) and warp chunks."""
    from abstraction_regret_gb300.engine import NfaChoice

    b = W.c3(variant, n_inputs=256)
    eng = PersistentEngine(b.automata, chunk_bytes=512, choices=[NfaChoice(lanes=lanes)])
    plan = eng.make_tasks(b.aut_ids, np.diff(b.offsets))
    assert (plan.lane_chunks > 0) == lanes
    f, l, e, _, _ = eng.run_requests(b.aut_ids, b.inputs(), with_examined=True)
    of, ol, oe, _ = O.nfa_batch(b.automata[0], b.data, b.offsets)
    assert np.array_equal(f, of) and np.array_equal(l, ol) and np.array_equal(e, oe)


def test_lane_chunks_that_outgrow_the_lane_fall_back_to_warps():
    """Wildcard edges keep the true sets above a lane's capacity (about 9 states):
    chunks take the overflow path."""
    rng = np.random.default_rng(11)
    n, deg = 400, 3
    syms = np.where(rng.random(n * deg) < 0.15, G.ANY_SYMBOL, rng.integers(0, 256, n * deg))
    accept = rng.random(n) < 0.002
    accept[0] = False
    nfa = G.nfa_from_edges(n, 0, accept, np.repeat(np.arange(n), deg), syms,
                           rng.integers(0, n, n * deg))
    lengths = W.log_uniform_lengths(np.random.default_rng(3), 96, 2000, 20000)
    off = W.offsets_of(lengths)
    data = W.walk_bytes(nfa, off, seed=4)
    inputs = [data[off[i]:off[i + 1]].tobytes() for i in range(lengths.size)]
    eng = PersistentEngine([nfa], chunk_bytes=512, lane_pair_mean=float("inf"))
    assert eng.make_tasks(np.zeros(lengths.size), lengths).lane_chunks > 0
    f, l, e, _, _ = eng.run_requests(np.zeros(lengths.size), inputs, with_examined=True)
    from abstraction_regret_gb300 import native

    assert int(eng._dplan.header[native.PLAN_OVERFLOW].item()) > 0
    of, ol, oe, _ = O.nfa_batch(nfa, data, off)
    assert np.array_equal(f, of) and np.array_equal(l, ol) and np.array_equal(e, oe)


@pytest.mark.parametrize("states", [257, 300, 1000, 2049, 4096])
def test_dfa_table_split_over_a_cluster(states):
    """2-byte tables of 257..4096 states are split by rows over 2..16 CTAs of a cluster
    (distributed shared memory); verdicts equal the oracle's and the L2 path's."""
    from abstraction_regret_gb300 import native
    from abstraction_regret_gb300.executors import CudaDFAExecutor

    rng = np.random.default_rng(states)
    for p in (0.0, 0.002):
        dfa = G.random_dfa(states, accept_prob=p, seed=states)
        lengths = [0, 1, 15, 16, 17, 100, 1000, 5000] + list(rng.integers(1, 20000, 300))
        inputs = [rng.integers(0, 256, int(k), dtype=np.uint8).tobytes() for k in lengths]
        want = [O.simulate_dfa(dfa, x) for x in inputs]
        staged = CudaDFAExecutor(dfa, plan=native.make_plan(native.TECH_DFA_WALK, stage=1))
        through_l2 = CudaDFAExecutor(dfa, plan=native.make_plan(native.TECH_DFA_WALK, stage=0))
        f, l, ex, _, _ = staged.run_arrays(inputs, with_examined=True)
        assert list(zip(f.astype(bool).tolist(), l.tolist())) == want
        f2, l2, ex2, _, _ = through_l2.run_arrays(inputs, with_examined=True)
        assert np.array_equal(f, f2) and np.array_equal(l, l2) and np.array_equal(ex, ex2)
    start_acc = G.DFABuilder()
    for k in range(600):
        start_acc.add_state(accept=(k == 0))
    for s in range(600):
        for c in range(256):
            start_acc.add_transition(s, c, (s * 7 + c) % 600)
    a = start_acc.build()
    f, l, _, _, _ = CudaDFAExecutor(a).run_arrays([b"", b"xyz"])
    assert f.tolist() == [1, 1] and l.tolist() == [0, 0]


@pytest.mark.parametrize("ingest", ["copy", "zero_copy", "pipelined", "pipelined-shrink"])
def test_graph_runner_ingest_paths(ingest):
    """A captured step (H2D, launches, D2H) gives the oracle's verdicts on every ingest
    path, replayed twice; the pipelined path plans each slice on its own (two lane waves
    by default; one wave with later slices' chunks shrunk)."""
    import torch

    from abstraction_regret_gb300.engine import GraphRunner

    b = W.c3("live", n_inputs=192)
    eng = PersistentEngine(b.automata)
    extra = {"shrink": 0.75, "lane_waves": 1} if ingest == "pipelined-shrink" else {}
    ingest = ingest.split("-")[0]
    r = GraphRunner(eng, b.aut_ids, b.data, b.offsets, with_examined=True, ingest=ingest,
                    parts=3, **extra)
    of, ol, oe, _ = O.nfa_batch(b.automata[0], b.data, b.offsets)
    for _ in range(2):
        with torch.cuda.stream(r.stream):
            r.replay()
        r.stream.synchronize()
        f, l, e = r.verdicts()
        assert np.array_equal(f, of) and np.array_equal(l, ol) and np.array_equal(e, oe)
    if ingest == "pipelined":
        from abstraction_regret_gb300 import native

        assert len(r.slices) == 3
        h = r.plan.h_header.numpy()
        ranges = [(int(h[native.PLAN_SLICES + 2 * k]), int(h[native.PLAN_SLICES + 2 * k + 1]))
                  for k in range(3)]
        assert ranges[0][0] == 0
        assert all(a + c == b for (a, c), (b, _) in zip(ranges, ranges[1:]))
        assert sum(c for _, c in ranges) == int(h[native.PLAN_LANE_TASKS]) > 0
