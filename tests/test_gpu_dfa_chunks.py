"""Chunked walks of long DFA inputs (csrc/dfa_chunks.cu) against the oracle (GPU).

A DFA input at least twice its DFA's chunk length is cut into chunks walked in
parallel; verdicts and examined counts must equal the oracle's serial walk bit for bit:
for random DFAs of 64 to 16384 states, with accepts placed at, just before and just
after chunk boundaries and inside the overlaps, with no overlap at all (every chunk then
linked by a serial gap walk), for DFAs whose set of all states never collapses (every
chunk walked whole in the fix-up), and in pools that mix chunked DFAs with chunked NFAs
(their chunk records share one table).
"""

from __future__ import annotations

import numpy as np
import pytest

from abstraction_regret_gb300 import engine as E
from abstraction_regret_gb300 import native
from abstraction_regret_gb300 import workloads as W
from abstraction_regret_gb300.automata import DFA, random_dfa
from abstraction_regret_gb300.engine import PersistentEngine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _alarm_dfa(n: int, seed: int, permutation: bool) -> DFA:
    """Random transitions (or one random permutation per byte: the set of all states
    never shrinks) except byte 255, which leads every state to the one accepting state."""
    rng = np.random.default_rng(seed)
    if permutation:
        trans = np.stack([rng.permutation(n - 1) for _ in range(256)], axis=1).astype(np.int32)
    else:
        trans = rng.integers(0, n - 1, size=(n - 1, 256), dtype=np.int32)
    trans = np.vstack([trans, rng.integers(0, n - 1, size=(1, 256), dtype=np.int32)])
    trans[:, 255] = n - 1
    accept = np.zeros(n, dtype=bool)
    accept[n - 1] = True
    return DFA(num_states=n, start_state=0, accept=accept, trans=trans.reshape(-1))


def _oracle(automata, aut_ids, inputs):
    flags = np.zeros(len(inputs), np.int32)
    lens = np.zeros(len(inputs), np.int32)
    examined = np.zeros(len(inputs), np.int64)
    for a, aut in enumerate(automata):
        idx = [i for i, x in enumerate(aut_ids) if x == a]
        if not idx:
            continue
        sub = [inputs[i] for i in idx]
        off = np.zeros(len(sub) + 1, np.int64)
        off[1:] = np.cumsum([len(x) for x in sub])
        flat = np.frombuffer(b"".join(sub), np.uint8)
        if isinstance(aut, DFA):
            f, ln, ex = O.dfa_batch(aut, flat, off)
        else:
            f, ln, ex, _ = O.nfa_batch(aut, flat, off)
        flags[idx], lens[idx], examined[idx] = f, ln, ex
    return flags, lens, examined


def _run_and_check(eng, aut_ids, inputs, min_dfa_chunks=1):
    flags, lens, examined, _, _ = eng.run_requests(aut_ids, inputs, with_examined=True)
    h = eng._dplan.h_header.numpy()
    assert h[native.PLAN_STATUS] == 0
    assert int(h[native.PLAN_DFA_CHUNKS]) >= min_dfa_chunks
    of, ol, oe = _oracle(eng.automata, aut_ids, inputs)
    bad = np.flatnonzero((flags != of) | (lens != ol) | (examined != oe))
    assert bad.size == 0, [(int(i), len(inputs[i]), (int(flags[i]), int(lens[i]),
                            int(examined[i])), (int(of[i]), int(ol[i]), int(oe[i])))
                           for i in bad[:8]]
    return flags


def _boundary_inputs(chunk: int, lengths, seed: int):
    """Inputs with one alarm byte (255) at, around or after a chunk boundary (cut as the
    planner cuts: chunk k of an input of L bytes in cnt chunks starts at k L / cnt)."""
    rng = np.random.default_rng(seed)
    out = []
    for length in lengths:
        cnt = -(-length // chunk)
        starts = [k * length // cnt for k in range(1, cnt)]
        out.append(rng.integers(0, 255, length, dtype=np.uint8).tobytes())  # no accept
        for b in starts[:3] + starts[-2:]:
            for d in (-1, 0, 1, 3, 777):
                x = rng.integers(0, 255, length, dtype=np.uint8)
                x[min(length - 1, b + d)] = 255
                out.append(x.tobytes())
        x = rng.integers(0, 255, length, dtype=np.uint8)
        x[length - 1] = 255
        out.append(x.tobytes())
    return out


@pytest.mark.parametrize("permutation", [False, True])
def test_accepts_around_chunk_boundaries(permutation):
    dfa = _alarm_dfa(64, seed=1, permutation=permutation)
    chunk = E.dfa_chunk_length(64)
    eng = PersistentEngine([dfa], dfa_chunk_bytes=chunk)  # fixed: the boundaries are known
    inputs = _boundary_inputs(chunk, [2 * chunk, 5 * chunk + 123, 9 * chunk - 7], seed=2)
    flags = _run_and_check(eng, [0] * len(inputs), inputs)
    assert 0 < int(flags.sum()) < len(inputs)


def test_no_overlap_links_every_chunk_by_a_gap_walk(monkeypatch):
    monkeypatch.setattr(E, "DFA_OVERLAP_CHUNKS", 0.0)
    dfa = _alarm_dfa(200, seed=3, permutation=False)
    chunk = E.dfa_chunk_length(200)
    eng = PersistentEngine([dfa], dfa_chunk_bytes=chunk)
    inputs = _boundary_inputs(chunk, [3 * chunk + 5, 6 * chunk], seed=4)
    _run_and_check(eng, [0] * len(inputs), inputs)


@pytest.mark.parametrize("states", [64, 1024, 4096, 16384])
def test_random_dfas_long_and_short_inputs(states):
    """Long inputs (chunked) and short ones (DFA groups) in one batch; a few accepts."""
    dfa = random_dfa(states, accept_prob=2e-6 * (16384 / states) ** 0.5, seed=states)
    eng = PersistentEngine([dfa])
    rng = np.random.default_rng(states)
    chunk = E.dfa_chunk_length(states)
    lengths = list(rng.integers(2 * chunk, 12 * chunk, 12)) + \
        list(rng.integers(0, 2 * chunk, 40))
    inputs = [rng.integers(0, 256, int(m), dtype=np.uint8).tobytes() for m in lengths]
    _run_and_check(eng, [0] * len(inputs), inputs)


def test_mixed_pool_of_chunked_nfas_and_dfas():
    """Lane-chunked NFAs, warp-chunked and whole NFAs and chunked DFAs interleaved: the
    DFA chunks follow the NFA chunks in one chunk table and record array."""
    nfas = [W.random_nfa(1024, seed=0, degree=2, accept_prob=0.001),
            W.random_nfa(3000, seed=5, poisson=4.0, accept_prob=0.0005)]
    dfas = [random_dfa(1024, accept_prob=1e-5, seed=7), _alarm_dfa(300, 8, False)]
    automata = nfas + dfas
    eng = PersistentEngine(automata)
    rng = np.random.default_rng(9)
    aut_ids, inputs = [], []
    for i in range(160):
        a = int(rng.integers(0, len(automata)))
        if a >= 2:
            m = int(rng.integers(1, 6 * E.dfa_chunk_length(automata[a].num_states)))
            x = rng.integers(0, 255, m, dtype=np.uint8)
            if a == 3 and i % 3 == 0:
                x[int(rng.integers(0, m))] = 255
        else:
            m = int(rng.integers(1, 300_000))
            x = rng.integers(0, 256, m, dtype=np.uint8)
        aut_ids.append(a)
        inputs.append(x.tobytes())
    _run_and_check(eng, aut_ids, inputs)


def test_dfa_chunking_off_without_chunking():
    """chunk_bytes=None runs every input whole: no DFA chunk tasks."""
    dfa = random_dfa(256, accept_prob=0.0, seed=11)
    eng = PersistentEngine([dfa], chunk_bytes=None)
    assert eng.aut_dfa_chunk is None
    rng = np.random.default_rng(12)
    inputs = [rng.integers(0, 256, 300_000, dtype=np.uint8).tobytes() for _ in range(4)]
    _run_and_check(eng, [0] * 4, inputs, min_dfa_chunks=0)


def test_early_accept_stops_later_chunks():
    """An accept near the start of a long input (found by chunk 0) stops the input's later
    chunks (their records say p = -2); verdicts stay exact, including an input whose
    accept lies in a later chunk's overlap and one with no accept."""
    dfa = _alarm_dfa(64, seed=5, permutation=False)
    chunk = E.dfa_chunk_length(64)
    eng = PersistentEngine([dfa], dfa_chunk_bytes=chunk)
    length = 16 * chunk
    rng = np.random.default_rng(6)
    inputs = []
    for q in (10, 3000, length // 2 + 5, -1):
        x = rng.integers(0, 255, length, dtype=np.uint8)
        if q >= 0:
            x[q] = 255
        inputs.append(x.tobytes())
    _run_and_check(eng, [0] * len(inputs), inputs)
    plan = eng._dplan
    h = plan.h_header.numpy()
    n_lane = int(h[native.PLAN_LANE_CHUNKS])
    nc = int(h[native.PLAN_CHUNKS])
    chunks = plan.chunks[: nc * 24].cpu().numpy().view(native.CHUNK_DTYPE)
    recs = plan.records[: nc * native.CHUNK_RECORD_BYTES].cpu().numpy() \
        .view(np.int32).reshape(nc, -1)[:, :5]
    first = chunks[n_lane:][chunks[n_lane:]["input"] == 0]
    p_later = recs[n_lane:][chunks[n_lane:]["input"] == 0][1:, 0]
    assert first.size == 16 and (p_later == -2).mean() >= 0.9, p_later
    p_none = recs[n_lane:][chunks[n_lane:]["input"] == 3][1:, 0]
    assert (p_none >= 0).all()


def test_chunk_length_follows_the_batch():
    """Few long inputs get the DFA's shortest chunks; enough long inputs to fill the chunk
    launch get longer chunks (one wave), and verdicts stay exact either way."""
    dfa = random_dfa(256, accept_prob=0.0, seed=13)
    eng = PersistentEngine([dfa])
    minimum = E.dfa_chunk_length(256)
    assert eng.dfa_warps > 0
    rng = np.random.default_rng(14)
    few = [rng.integers(0, 256, 8 * minimum, dtype=np.uint8).tobytes() for _ in range(2)]
    _run_and_check(eng, [0] * 2, few, min_dfa_chunks=16)
    h = eng._dplan.h_header.numpy()
    assert int(h[native.PLAN_DFA_CHUNK_BYTES]) <= minimum
    n = -(-2 * minimum * eng.dfa_warps // (2 << 20))  # about two chunk-lengths per warp
    many = [rng.integers(0, 256, 2 << 20, dtype=np.uint8).tobytes() for _ in range(n)]
    _run_and_check(eng, [0] * n, many)
    h = eng._dplan.h_header.numpy()
    target = int(h[native.PLAN_DFA_CHUNK_BYTES])
    assert target > minimum
    assert int(h[native.PLAN_DFA_CHUNKS]) <= eng.dfa_warps  # one wave
