"""gbfsm_nfa_run_static: the workspace-free NFA launch, against gbfsm_nfa_run.

Collected last (file name) so it also runs after every other test in one process; it
must pass alone in a fresh process too. Each case calls the static-scratch entry point
twice in a row through the C ABI and compares both results with gbfsm_nfa_run given a
caller-allocated workspace (and with the oracle).
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from abstraction_regret_gb300 import native
from abstraction_regret_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _run(fn, nfa, d_data, d_off, n, plan, workspace=None, out=None):
    import torch

    dev = d_data.device
    if out is None:
        out = torch.full((3, n), -7, dtype=torch.int32, device=dev)
    else:
        out.fill_(-7)
    stream = torch.cuda.current_stream(dev).cuda_stream
    args = [ctypes.byref(nfa.desc), d_data.data_ptr(), d_off.data_ptr(), n, ctypes.byref(plan),
            out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr()]
    if workspace is not None:
        args += [workspace.data_ptr() if workspace.numel() else None, workspace.numel()]
    st = fn(*args, stream)
    native.check(st, fn.__name__)
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()


def _case(automaton, data, offsets, technique, block_threads=0):
    import torch

    from abstraction_regret_gb300.device import DeviceNFA

    lib = native.lib()
    dev = torch.device("cuda:0")
    nfa = DeviceNFA(automaton, dev)
    n = len(offsets) - 1
    padded = np.zeros(max(16, -(-int(offsets[-1]) // 16) * 16), dtype=np.uint8)
    padded[: int(offsets[-1])] = data[: int(offsets[-1])]
    d_data = torch.from_numpy(padded).to(dev)
    d_off = torch.from_numpy(np.asarray(offsets, dtype=np.int64)).to(dev)
    plan = native.make_plan(technique, block_threads=block_threads)
    need = int(lib.gbfsm_nfa_workspace_bytes(ctypes.byref(nfa.desc), n, ctypes.byref(plan)))
    assert 0 < need <= native.STATIC_SCRATCH_BYTES  # the case really uses scratch
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    want = _run(lib.gbfsm_nfa_run, nfa, d_data, d_off, n, plan, ws)
    first = _run(lib.gbfsm_nfa_run_static, nfa, d_data, d_off, n, plan)
    # the second call, set-up done, takes no device memory: free memory is unchanged
    out = torch.empty((3, n), dtype=torch.int32, device=dev)
    torch.cuda.synchronize(dev)
    free_before = torch.cuda.mem_get_info(dev)[0]
    second = _run(lib.gbfsm_nfa_run_static, nfa, d_data, d_off, n, plan, out=out)
    free_after = torch.cuda.mem_get_info(dev)[0]
    assert free_after == free_before
    assert np.array_equal(first, want)
    assert np.array_equal(second, want)
    of, ol, oe, _ = O.nfa_batch(automaton, data, offsets)
    assert np.array_equal(want[0], of) and np.array_equal(want[1], ol)
    assert np.array_equal(want[2], oe)


def test_static_scratch_bitmap_technique_matches_workspace_launch():
    """16384-state NFA, thread-per-input bitmap sets kept in the scratch."""
    b = W.c3("live", n_inputs=96)
    lengths = np.minimum(np.diff(b.offsets), 6000)
    off = W.offsets_of(lengths)
    data = np.concatenate([b.data[b.offsets[i]:b.offsets[i] + lengths[i]]
                           for i in range(lengths.size)])
    _case(b.automata[0], data, off, native.TECH_BITMAP)


def test_static_scratch_warp_technique_matches_workspace_launch():
    """A 120000-state NFA with eight warps per CTA: the dense sets go to the scratch."""
    nfa = W.random_nfa(120000, seed=9, degree=2, accept_prob=0.002)
    lengths = np.full(40, 3000, dtype=np.int64)
    off = W.offsets_of(lengths)
    data = W.walk_bytes(nfa, off, seed=10)
    _case(nfa, data, off, native.TECH_COMPACT, block_threads=256)


def test_static_scratch_rejects_a_batch_above_its_size():
    import torch

    from abstraction_regret_gb300.device import DeviceNFA

    lib = native.lib()
    b = W.c3("literal", n_inputs=8)
    nfa = DeviceNFA(b.automata[0], torch.device("cuda:0"))
    plan = native.make_plan(native.TECH_BITMAP)
    n = 8192  # 8 KiB of bitmap sets per input: 64 MiB
    need = int(lib.gbfsm_nfa_workspace_bytes(ctypes.byref(nfa.desc), n, ctypes.byref(plan)))
    assert need > native.STATIC_SCRATCH_BYTES
    st = lib.gbfsm_nfa_run_static(ctypes.byref(nfa.desc), None, None, n, ctypes.byref(plan),
                                  None, None, None, None)
    assert st == native.INVALID_ARG
    assert "static scratch" in native.last_error()
