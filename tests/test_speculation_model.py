"""The speculative chunk protocol, checked on the CPU with a set-based model.

``run_chunk`` / ``run_fixup`` below restate the device protocol of the persistent
engine (csrc/persistent.cu) with Python sets: a chunk after the first starts from the
epsilon closure of every target of an edge labelled with the byte two positions before
it, steps over the byte just before it, records its set sizes after 1, 2, 4, ..., 32
bytes, the first accept after each checkpoint and where it died; the fix-up re-runs each
chunk exactly until the exact set is as large as the superset at a checkpoint. The
model must give the oracle's verdict on every input, for any chunk size -- this pins the
protocol itself, independently of the kernels (the GPU tests pin the kernels against
the oracle).

``scan_fixup`` restates the parallel form of the fix-up (csrc/chunks.cuh): each chunk
also continues its run up to 32 bytes into the next chunk (the overlap), and a chunk is
linked to its predecessor when the overlap run has the next chunk's recorded size at a
checkpoint. A chain of links from the exact first chunk makes every linked chunk's
record exact, so the fix-up is a scan for the first chunk that decides (an accept or a
death) or cannot be linked; only from there does it fall back to the serial re-run.
"""

from __future__ import annotations

import random

import numpy as np
import pytest

from abstraction_regret_gb300 import ANY_SYMBOL, NFABuilder
from abstraction_regret_gb300 import workloads as W
from abstraction_regret_gb300.device import first_lists
from oracle.oracle import epsilon_closure, simulate

CHECKPOINTS = 6


def step(nfa, cur, b):
    rp, tg, sy = nfa.sym_row_ptr, nfa.sym_targets, nfa.sym_symbols
    nxt = set()
    for s in cur:
        for k in range(int(rp[s]), int(rp[s + 1])):
            if int(sy[k]) in (b, ANY_SYMBOL):
                nxt.add(int(tg[k]))
    return epsilon_closure(nxt, nfa) if nxt else set()


def accepts(nfa, cur):
    return any(nfa.accept[s] for s in cur)


def run_chunk(nfa, data, b, e, index, lists, ov_end=None):
    rec = {"counts": [0] * CHECKPOINTS, "acc_after": [-1] * CHECKPOINTS, "dead_at": -1,
           "end": None, "ov_len": 0, "ov_counts": [0] * CHECKPOINTS, "ov_acc": 0,
           "ov_dead": 0}
    ov_end = e if ov_end is None else ov_end
    if index == 0:
        cur = epsilon_closure({int(nfa.start_state)}, nfa)
        if accepts(nfa, cur):
            rec["acc_after"][0] = 0
            return rec
    else:
        row, recs = lists
        c0 = data[b - 2]
        cur = epsilon_closure({int(t) for t in recs[row[c0]:row[c0 + 1], 0]}, nfa)
        cur = step(nfa, cur, data[b - 1]) if cur else set()
        if not cur:
            rec["dead_at"] = b
            return rec
    for j in range(1, e - b + 1):
        cur = step(nfa, cur, data[b + j - 1])
        pos = b + j
        if index == 0:
            if not cur:
                rec["dead_at"] = pos
                return rec
            if accepts(nfa, cur):
                rec["acc_after"][0] = pos
                return rec
            continue
        if not cur:
            rec["dead_at"] = pos
            return rec
        if accepts(nfa, cur):
            for c in range(CHECKPOINTS):
                if j > (1 << c) and rec["acc_after"][c] < 0:
                    rec["acc_after"][c] = pos
            if j > (1 << (CHECKPOINTS - 1)):
                return rec
        if j <= (1 << (CHECKPOINTS - 1)) and (j & (j - 1)) == 0:
            rec["counts"][j.bit_length() - 1] = len(cur)
    rec["end"] = set(cur)
    if ov_end > e:  # the overlap: continue into the next chunk from the end set
        rec["ov_len"] = ov_end - e
        for j in range(1, ov_end - e + 1):
            cur = step(nfa, cur, data[e + j - 1])
            if not cur:
                rec["ov_dead"] = j
                break
            if accepts(nfa, cur):
                rec["ov_acc"] = j
                break
            if j <= 32 and (j & (j - 1)) == 0:
                rec["ov_counts"][j.bit_length() - 1] = len(cur)
    return rec


def run_fixup(nfa, data, chunks, recs, start=1):
    """Serial fix-up from chunk ``start`` (>= 1), whose predecessor's end set is exact."""
    r0 = recs[0]
    if r0["acc_after"][0] >= 0:
        return True, r0["acc_after"][0]
    if r0["dead_at"] >= 0:
        return False, 0
    cur = recs[start - 1]["end"]
    for (b, e), rk in zip(chunks[start:], recs[start:]):
        matched = -1
        j = 0
        while b + j < e:
            cur = step(nfa, cur, data[b + j])
            j += 1
            if not cur:
                return False, 0
            if accepts(nfa, cur):
                return True, b + j
            if j <= 32 and (j & (j - 1)) == 0 and len(cur) == rk["counts"][j.bit_length() - 1]:
                matched = j.bit_length() - 1
                break
        if matched >= 0:
            if rk["acc_after"][matched] >= 0:
                return True, rk["acc_after"][matched]
            if rk["dead_at"] >= 0:
                return False, 0
            if rk["end"] is not None:
                cur = rk["end"]
            else:
                while b + j < e:
                    cur = step(nfa, cur, data[b + j])
                    j += 1
    return False, 0


LINK, DECIDE, BREAK = 0, 1, 2


def classify(prev, rk, begin):
    """Chunk k against its predecessor's overlap run: LINK (exact from a checkpoint on,
    no event), DECIDE with the verdict, or BREAK (no link within the overlap)."""
    for c in range(CHECKPOINTS):
        j = 1 << c
        if j > prev["ov_len"]:
            break
        if prev["ov_acc"] and prev["ov_acc"] <= j:
            return DECIDE, (True, begin + prev["ov_acc"])
        if prev["ov_dead"] and prev["ov_dead"] <= j:
            return DECIDE, (False, 0)
        if prev["ov_counts"][c] == rk["counts"][c]:
            if rk["acc_after"][c] >= 0:
                return DECIDE, (True, rk["acc_after"][c])
            if rk["dead_at"] >= 0:
                return DECIDE, (False, 0)
            return LINK, None
    return BREAK, None


def scan_fixup(nfa, data, chunks, recs):
    r0 = recs[0]
    if r0["acc_after"][0] >= 0:
        return True, r0["acc_after"][0]
    if r0["dead_at"] >= 0:
        return False, 0
    last_rec = 0 if r0["end"] is not None else -1
    for k in range(1, len(chunks)):
        status, verdict = classify(recs[k - 1], recs[k], chunks[k][0])
        if status == DECIDE:
            return verdict
        if status == BREAK:
            if last_rec < 0:
                return simulate(nfa, data)
            return run_fixup(nfa, data, chunks, recs, start=last_rec + 1)
        if recs[k]["end"] is not None:
            last_rec = k
    return False, 0


def even_bounds(n: int, chunk: int):
    count = max(1, -(-n // chunk))
    return [(k * n // count, (k + 1) * n // count) for k in range(count)]


def speculative(nfa, data: bytes, chunk: int, scan: bool = False, even: bool = False):
    n = len(data)
    if n < 2 * chunk and not even:
        return simulate(nfa, data)
    lists = first_lists(nfa)
    if even:
        bounds = even_bounds(n, chunk)
    else:
        count = n // chunk
        bounds = [(k * chunk, (k + 1) * chunk if k < count - 1 else n) for k in range(count)]
    recs = []
    for k, (b, e) in enumerate(bounds):
        ov_end = min(e + 32, bounds[k + 1][1]) if k + 1 < len(bounds) else e
        recs.append(run_chunk(nfa, data, b, e, k, lists, ov_end))
    if scan:
        return scan_fixup(nfa, data, bounds, recs)
    return run_fixup(nfa, data, bounds, recs)


def _fuzz_nfa(rng, n, alpha, p_acc, p_any, max_eps):
    b = NFABuilder()
    for _ in range(n):
        b.add_state(accept=rng.random() < p_acc)
    b.set_start(rng.randrange(n))
    for s in range(n):
        for _ in range(rng.randint(0, 3)):
            sym = ANY_SYMBOL if rng.random() < p_any else ord(rng.choice(alpha))
            b.add_transition(s, sym, rng.randrange(n))
        for _ in range(rng.randint(0, max_eps)):
            b.add_epsilon(s, rng.randrange(n))
    return b.build()


@pytest.mark.parametrize("seed", range(6))
def test_protocol_matches_the_oracle_on_fuzz(seed):
    rng = random.Random(1000 + seed)
    for _ in range(25):
        nfa = _fuzz_nfa(rng, rng.randint(1, 40), "abc", 0.03, 0.05, rng.choice([0, 1, 2]))
        for _ in range(4):
            data = bytes(ord(rng.choice("abc")) for _ in range(rng.randint(0, 400)))
            want = simulate(nfa, data)
            for chunk in (40, 64, 97):
                assert speculative(nfa, data, chunk) == want
                assert speculative(nfa, data, chunk, scan=True) == want
            for chunk in (9, 17):  # overlaps shorter than 32 bytes
                assert speculative(nfa, data, chunk, scan=True) == want
            if len(data) >= 64:
                assert speculative(nfa, data, 64, scan=True, even=True) == want


def test_protocol_on_live_walks_of_the_large_configuration():
    b = W.c3("live", n_inputs=64)
    nfa = b.automata[0]
    idx = np.argsort(np.diff(b.offsets))[:12]
    for i in idx:
        data = b.inputs([int(i)])[0][:6000]
        want = simulate(nfa, data)
        for chunk in (256, 1000):
            assert speculative(nfa, data, chunk) == want
            assert speculative(nfa, data, chunk, scan=True, even=True) == want


def _true_sets(nfa, data):
    """Active set after each prefix of data (index p: after p bytes), until it dies."""
    cur = epsilon_closure({int(nfa.start_state)}, nfa)
    out = [set(cur)]
    for x in data:
        cur = step(nfa, cur, x) if cur else set()
        out.append(set(cur))
    return out


@pytest.mark.parametrize("seed", range(4))
def test_two_byte_and_widened_start_sets_contain_the_true_set(seed):
    """The lane start sets (csrc/chunks.cuh): the two-byte superset of x[b-2] x[b-1]
    (pair_lanes), and the widened one -- the two-byte superset of x[b-4] x[b-3] stepped
    over x[b-2] and x[b-1] -- both contain the true active set at b, for every b."""
    from abstraction_regret_gb300.device import pair_lists

    rng = random.Random(2000 + seed)
    for _ in range(20):
        nfa = _fuzz_nfa(rng, rng.randint(2, 60), "abcd", 0.02, 0.04, 0)  # no epsilon
        first = first_lists(nfa)
        pairs = pair_lists(nfa, first)
        assert pairs is not None
        prow, precs = pairs
        data = bytes(ord(rng.choice("abcd")) for _ in range(rng.randint(8, 300)))
        truth = _true_sets(nfa, data)

        def pair_set(c1, c2):
            k = c1 * 256 + c2
            return {int(t) for t in precs[prow[k]:prow[k + 1], 0]}

        for b in range(4, len(data) + 1):
            two = pair_set(data[b - 2], data[b - 1])
            assert truth[b] <= two
            wide = pair_set(data[b - 4], data[b - 3])
            for x in (data[b - 2], data[b - 1]):
                wide = step(nfa, wide, x) if wide else set()
            assert truth[b] <= wide <= two
