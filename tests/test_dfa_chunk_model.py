"""A CPU model of the chunked DFA walk (csrc/dfa_chunks.cuh) against the oracle's serial
walk, on small DFAs and short chunks, so that the record and fix-up rules are checked
without a GPU.

The model follows the device code step for step: chunk 0 walks from the start state;
a later chunk walks the set of all states until it holds one (the collapse), then walks
exactly to its end and on into the next chunk: ``overlap`` bytes, or (adaptive, as on
the device when the next chunk has published its collapse in time) exactly to the next
chunk's collapse, capped at ``overlap``; the fix-up links each chunk to the one before
it through the overlap, or walks the gap serially. Every verdict and examined
count must equal the serial walk's (src/gpufsm/reference.py:68-81), whatever the
overlap (zero included), for DFAs that collapse fast, slowly or never.
"""

from __future__ import annotations

import numpy as np
import pytest

from abstraction_regret_gb300.automata import DFA, random_dfa
from oracle import oracle as O


def _span(trans, acc, s, data, a, b):
    """State at b (or at the first accept q in (a, b]) and that accept, or -1."""
    for q in range(a, b):
        s = int(trans[s * 256 + data[q]])
        if acc[s]:
            return s, q + 1
    return s, -1


def _collapse(trans, n, data, b, e):
    if e <= b:
        return -1, 0
    cur = np.arange(n)
    pos = b
    while pos < e:
        cur = np.unique(trans[cur * 256 + data[pos]])
        pos += 1
        if cur.size == 1:
            return pos, int(cur[0])
    return -1, 0


def _chunk(dfa, data, length, b, e, index, overlap, next_p=None, e_next=None):
    trans, acc = dfa.trans, dfa.accept
    a = -1
    s = 0
    if index == 0:
        p, s = 0, dfa.start_state
        if acc[s]:
            a = 0
    else:
        p, s = _collapse(trans, dfa.num_states, data, b, e)
    ov_len, ov_acc, ov_state = 0, -1, 0
    if p >= 0 and a < 0:
        s, a = _span(trans, acc, s, data, p, e)
        if a < 0:
            ov_end = min(e + max(overlap, 0), length)
            if e_next is not None:  # never past the next chunk's end
                ov_end = min(ov_end, e_next)
            if next_p is not None and next_p >= 0:  # adaptive: stop at its collapse
                ov_end = min(ov_end, max(next_p, e))
            ov_state, ov_acc = _span(trans, acc, s, data, e, ov_end)
            ov_len = (ov_acc if ov_acc >= 0 else ov_end) - e
    return dict(p=p, acc=a, end_state=s, ov_len=ov_len, ov_acc=ov_acc, ov_state=ov_state)


def _fixup(dfa, data, length, bounds, recs):
    trans, acc = dfa.trans, dfa.accept
    r0 = recs[0]
    if r0["acc"] >= 0:
        return 1, r0["acc"], r0["acc"]
    s = r0["end_state"]
    prev_ok, prev_ov_len, prev_ov_acc = True, r0["ov_len"], r0["ov_acc"]
    prev_ov_state = r0["ov_state"]
    for k in range(1, len(recs)):
        if prev_ok and prev_ov_acc >= 0:
            return 1, prev_ov_acc, prev_ov_acc
        b, e = bounds[k]
        r = recs[k]
        if r["p"] >= 0:
            if not (prev_ok and r["p"] - b <= prev_ov_len):
                _, a = _span(trans, acc, s, data, b, r["p"])
                if a >= 0:
                    return 1, a, a
            if r["acc"] >= 0:
                return 1, r["acc"], r["acc"]
            s = r["end_state"]
            prev_ok, prev_ov_len, prev_ov_acc = True, r["ov_len"], r["ov_acc"]
            prev_ov_state = r["ov_state"]
        else:
            if prev_ok and prev_ov_len == e - b:
                s = prev_ov_state  # the previous overlap covered the whole chunk
            else:
                s, a = _span(trans, acc, s, data, b, e)
                if a >= 0:
                    return 1, a, a
            prev_ok = False
    return 0, 0, length


def chunked_verdict(dfa, data: np.ndarray, chunk: int, overlap: int, adaptive: bool = False):
    """Verdict of one input by the chunk model (chunk bounds as the planner cuts them)."""
    data = np.asarray(data).astype(np.int64)
    length = len(data)
    cnt = max(1, -(-length // chunk))
    bounds = [(k * length // cnt, (k + 1) * length // cnt) for k in range(cnt)]
    nxt = [None] * cnt
    if adaptive:  # the collapse positions the chunks publish
        for k in range(1, cnt):
            nxt[k - 1] = _collapse(dfa.trans, dfa.num_states, data, *bounds[k])[0]
    ends = [e for _, e in bounds[1:]] + [None]
    recs = [_chunk(dfa, data, length, b, e, k, overlap, nxt[k], ends[k] if adaptive else None)
            for k, (b, e) in enumerate(bounds)]
    return _fixup(dfa, data, length, bounds, recs), recs


def _alarm_dfa(n: int, seed: int, permutation: bool) -> DFA:
    """Random transitions (or a random permutation per byte, so the set of all states
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


def _check(dfa, inputs, chunk, overlap, adaptive=False):
    offsets = np.zeros(len(inputs) + 1, np.int64)
    offsets[1:] = np.cumsum([len(x) for x in inputs])
    flat = np.concatenate(inputs) if inputs else np.zeros(0, np.uint8)
    flags, lens, examined = O.dfa_batch(dfa, flat, offsets)
    for i, x in enumerate(inputs):
        (f, ln, ex), _ = chunked_verdict(dfa, x, chunk, overlap, adaptive)
        assert (f, ln, ex) == (flags[i], lens[i], examined[i]), (i, len(x))


@pytest.mark.parametrize("adaptive", [False, True])
@pytest.mark.parametrize("overlap", [0, 7, 64, 10_000])
@pytest.mark.parametrize("permutation", [False, True])
def test_alarm_byte_at_and_around_chunk_boundaries(overlap, permutation, adaptive):
    """Accepts placed at chunk starts, one byte either side, and inside the overlap."""
    dfa = _alarm_dfa(24, seed=1, permutation=permutation)
    rng = np.random.default_rng(2)
    chunk, length = 256, 2000
    cnt = -(-length // chunk)
    starts = [k * length // cnt for k in range(1, cnt)]
    inputs = [rng.integers(0, 255, length, dtype=np.uint8)]  # no alarm byte: no accept
    for b in starts:
        for d in (-2, -1, 0, 1, 2, 5, 40):
            x = rng.integers(0, 255, length, dtype=np.uint8)
            x[b + d] = 255
            inputs.append(x)
    for q in (0, 1, length - 1):
        x = rng.integers(0, 255, length, dtype=np.uint8)
        x[q] = 255
        inputs.append(x)
    _check(dfa, inputs, chunk, overlap, adaptive)


@pytest.mark.parametrize("adaptive", [False, True])
@pytest.mark.parametrize("n,accept_prob", [(2, 0.0), (16, 0.002), (64, 0.0005), (200, 0.0)])
@pytest.mark.parametrize("overlap", [0, 100, 1000])
def test_random_dfas(n, accept_prob, overlap, adaptive):
    dfa = random_dfa(n, accept_prob=accept_prob, seed=n)
    rng = np.random.default_rng(n + overlap)
    inputs = [rng.integers(0, 256, int(m), dtype=np.uint8)
              for m in rng.integers(512, 4000, 12)]
    _check(dfa, inputs, 256, overlap, adaptive)


@pytest.mark.parametrize("overlap", [300, 10_000])
def test_overlap_covers_chunks_that_never_collapse(overlap):
    """Permutation DFA (no collapse without the alarm byte): an overlap of a whole chunk
    carries the true state over it, so the fix-up need not walk it."""
    dfa = _alarm_dfa(24, seed=1, permutation=True)
    rng = np.random.default_rng(7)
    x = rng.integers(0, 255, 2000, dtype=np.uint8)
    x[700] = 255  # chunk 2 collapses at the alarm byte; chunks 1, 3.. never do
    x[1900] = 255
    (f, ln, ex), recs = chunked_verdict(dfa, x, 256, overlap, adaptive=True)
    want = O.dfa_batch(dfa, x, np.array([0, x.size], np.int64))
    assert (f, ln, ex) == (want[0][0], want[1][0], want[2][0])
    assert any(r["p"] == -1 for r in recs[1:])


def test_adaptive_overlap_links_exactly_at_the_collapse():
    """An adaptive overlap ends exactly at the next chunk's collapse and still links."""
    dfa = random_dfa(16, accept_prob=0.0, seed=4)
    x = np.random.default_rng(5).integers(0, 256, 4096, dtype=np.uint8)
    (f, _, ex), recs = chunked_verdict(dfa, x, 512, 4000, adaptive=True)
    assert f == 0 and ex == 4096
    bounds = [k * 4096 // 8 for k in range(8)]
    assert all(recs[k]["p"] - bounds[k] == recs[k - 1]["ov_len"] for k in range(1, 8))


def test_start_state_accepting_latches_at_zero():
    dfa = random_dfa(8, accept_prob=0.0, seed=3)
    accept = dfa.accept.copy()
    accept[0] = True
    dfa = DFA(num_states=8, start_state=0, accept=accept, trans=dfa.trans)
    x = np.random.default_rng(0).integers(0, 256, 1000, dtype=np.uint8)
    (f, ln, ex), _ = chunked_verdict(dfa, x, 256, 0)
    assert (f, ln, ex) == (1, 0, 0)


def test_collapse_links_through_the_overlap():
    """With a long overlap, a random DFA's chunks are linked: no gap is walked twice."""
    dfa = random_dfa(16, accept_prob=0.0, seed=4)
    x = np.random.default_rng(5).integers(0, 256, 4096, dtype=np.uint8)
    (f, _, ex), recs = chunked_verdict(dfa, x, 512, 400)
    assert f == 0 and ex == 4096
    assert all(r["p"] >= 0 for r in recs)
    bounds = [k * 4096 // 8 for k in range(8)]
    assert all(recs[k]["p"] - bounds[k] <= recs[k - 1]["ov_len"] for k in range(1, 8))
