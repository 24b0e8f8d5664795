"""Batches planned on the device (gbfsm_batch_plan) against the host planner and the
oracle (GPU).

For one automaton the device plan must equal the host plan (``make_tasks``) exactly:
the same chunk size, the same chunk table and the same lane and fix-up tasks. For mixed
pools (lane-chunked, warp-chunked and whole-input NFAs with DFAs, interleaved) the
verdicts and examined counts must equal the oracle's. A plan that does not fit its
buffers, or names an automaton outside the pool, is reported in the header's status
and runs no task.
"""

from __future__ import annotations

import numpy as np
import pytest

import abstraction_regret_gb300 as G
from abstraction_regret_gb300 import native
from abstraction_regret_gb300 import workloads as W
from abstraction_regret_gb300.engine import NfaChoice, PersistentEngine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _device_plan(eng, offsets, aut_ids=None):
    import torch

    n = len(offsets) - 1
    stream = torch.cuda.current_stream(eng.device)
    d_off = torch.from_numpy(np.asarray(offsets, dtype=np.int64)).to(eng.device)
    d_aut = (torch.from_numpy(np.asarray(aut_ids, dtype=np.int32)).to(eng.device)
             if aut_ids is not None else None)
    plan = eng.device_plan(n, int(offsets[-1]))
    plan.plan(d_off, None, d_aut, stream, n)
    plan.fetch_header(stream)
    stream.synchronize()
    return plan


def _tasks(t, first, count):
    return t.cpu().numpy()[first * 4:(first + count) * 4].reshape(-1, 4)


@pytest.mark.parametrize("case", ["c3-live", "c1-live", "c3-fixed"])
def test_device_plan_equals_host_plan_for_one_automaton(case):
    if case.startswith("c3"):
        b = W.c3("live", n_inputs=256)
    else:
        b = W.c1("live")
    eng = PersistentEngine(b.automata, chunk_bytes=512 if case == "c3-fixed" else 0)
    lengths = np.diff(b.offsets)
    host = eng.make_tasks(np.zeros(b.n_inputs, np.int64), lengths)
    plan = _device_plan(eng, b.offsets)
    h = plan.h_header.numpy()
    assert h[native.PLAN_STATUS] == 0
    nc = int(h[native.PLAN_CHUNKS])
    assert nc == host.chunks.shape[0] and int(h[native.PLAN_LANE_CHUNKS]) == host.lane_chunks
    assert int(h[native.PLAN_LANE_BYTES]) == host.lane_chunk_bytes
    dev_chunks = plan.chunks[: nc * 24].cpu().numpy().view(native.CHUNK_DTYPE)
    assert np.array_equal(dev_chunks, host.chunks)
    nl = int(h[native.PLAN_LANE_TASKS])
    lanes = plan.tasks[: nl * 4].cpu().numpy().reshape(-1, 4)
    assert np.array_equal(lanes[:, 1:], host.tasks_l[:, 1:])
    assert (lanes[:, 0] == -1).all()
    nf = int(h[native.PLAN_FIXUP_TASKS])
    fix = plan.tasks.cpu().numpy()[(plan.cap_lanes + plan.cap_persist) * 4:].reshape(-1, 4)[:nf]
    assert sorted(map(tuple, fix.tolist())) == sorted(map(tuple, host.tasks_b.tolist()))
    # the sentinel after the last chunk ends every chunk's overlap at its input's end
    sentinel = plan.chunks[nc * 24:(nc + 1) * 24].cpu().numpy().view(native.CHUNK_DTYPE)[0]
    assert sentinel["input"] == -1 and sentinel["index"] == 0


def _mixed_pool():
    import random

    rng = random.Random(3)
    pool = [W.random_nfa(1024, seed=0, degree=2, accept_prob=0.01),       # lane chunks
            W.random_nfa(3000, seed=5, poisson=4.0, accept_prob=0.002)]   # lane chunks
    b = G.NFABuilder()  # epsilon edges: warp chunks
    n = 200
    for _ in range(n):
        b.add_state(accept=rng.random() < 0.01)
    for s in range(n):
        for _ in range(rng.randint(1, 3)):
            b.add_transition(s, ord(rng.choice("abcdef")), rng.randrange(n))
        if rng.random() < 0.3:
            b.add_epsilon(s, rng.randrange(n))
    pool.append(b.build())
    pool.append(W.random_nfa(500, seed=9, degree=3, accept_prob=0.004))   # whole inputs
    pool += [G.random_dfa(k, accept_prob=p, seed=k) for k, p in ((64, 0.01), (4096, 0.0),
                                                                 (1500, 0.002))]
    choices = [NfaChoice(), NfaChoice(), NfaChoice(), NfaChoice(speculate=False)] + \
        [NfaChoice()] * 3
    return pool, choices


def _requests(pool, n, seed):
    rng = np.random.default_rng(seed)
    aut = rng.integers(0, len(pool), n)
    lengths = np.where(rng.random(n) < 0.1, 0,
                       W.log_uniform_lengths(rng, n, 1, 40000))
    inputs = []
    for a, k in zip(aut, lengths):
        x = pool[a]
        if hasattr(x, "trans"):  # DFAs: uniform bytes
            inputs.append(rng.integers(0, 256, int(k), dtype=np.uint8).tobytes())
        elif x.eps_targets.size:  # the epsilon NFA reads 'a'..'f'
            inputs.append(rng.integers(97, 103, int(k), dtype=np.uint8).tobytes())
        else:  # random walks keep the other NFAs alive
            off = W.offsets_of(np.array([k], dtype=np.int64))
            inputs.append(W.walk_bytes(x, off, seed=int(rng.integers(1 << 30))).tobytes())
    return aut, inputs


@pytest.mark.parametrize("chunk", [0, 600, None])
def test_mixed_pool_planned_on_the_device_matches_the_oracle(chunk):
    pool, choices = _mixed_pool()
    eng = PersistentEngine(pool, choices=choices, chunk_bytes=chunk)
    assert set(eng.aut_class.cpu().tolist()) >= ({0, 3} if chunk is None else {0, 1, 2, 3})
    aut, inputs = _requests(pool, 400, seed=7)
    f, l, e, _, _ = eng.run_requests(aut, inputs, with_examined=True)
    for k, a in enumerate(pool):
        sel = np.flatnonzero(aut == k)
        data, off = O.flatten([inputs[i] for i in sel])
        if hasattr(a, "trans"):
            of, ol, oe = O.dfa_batch(a, data, off)
        else:
            of, ol, oe, _ = O.nfa_batch(a, data, off)
        assert np.array_equal(f[sel], of) and np.array_equal(l[sel], ol), k
        assert np.array_equal(e[sel], oe), k
    # a second, smaller batch reuses the plan buffers
    aut2, inputs2 = _requests(pool, 37, seed=8)
    f2, l2, _, _, _ = eng.run_requests(aut2, inputs2)
    want = [O.verdicts(pool[a], [x])[0] for a, x in zip(aut2, inputs2)]
    assert list(zip(f2.astype(bool).tolist(), l2.tolist())) == want


def test_plan_status_reports_small_buffers_and_bad_automata():
    b = W.c1("live")
    eng = PersistentEngine(b.automata)
    plan = eng.device_plan(b.n_inputs, b.total_bytes)
    import torch

    stream = torch.cuda.current_stream(eng.device)
    d_off = torch.from_numpy(b.offsets.copy()).to(eng.device)
    cap = plan.cap_chunks
    plan.cap_chunks = 3  # fewer chunks than the batch needs (the buffers stay larger)
    plan.plan(d_off, None, None, stream, b.n_inputs)
    plan.fetch_header(stream)
    stream.synchronize()
    assert int(plan.h_header[native.PLAN_STATUS]) == 1
    assert int(plan.h_header[native.PLAN_CHUNKS]) == 0
    with pytest.raises(RuntimeError, match="too small"):
        plan.check()
    plan.cap_chunks = cap
    d_aut = torch.full((b.n_inputs,), 5, dtype=torch.int32, device=eng.device)
    plan.plan(d_off, None, d_aut, stream, b.n_inputs)
    plan.fetch_header(stream)
    stream.synchronize()
    with pytest.raises(ValueError, match="outside the pool"):
        plan.check()
    # and the engine still plans and runs a valid batch afterwards
    f, l, _, _, _ = eng.run_requests(np.zeros(b.n_inputs), b.inputs())
    of, ol, _, _ = O.nfa_batch(b.automata[0], b.data, b.offsets)
    assert np.array_equal(f, of) and np.array_equal(l, ol)
