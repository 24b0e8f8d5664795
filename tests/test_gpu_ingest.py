"""Ingest that the GPU drives: inputs copied from the caller's own buffers (GPU).

On a device that reads pageable host memory (GB300 over NVLink-C2C), ``Staging`` lets
``gbfsm_gather_inputs`` read every input where it lies -- Python ``bytes``, ``bytearray``,
``memoryview`` slices at any alignment, numpy arrays -- instead of packing the batch on
the host. The device buffer must be byte for byte the packed one, and the verdicts the
oracle's. Skipped on a device that cannot read pageable memory (nothing is tried there).
"""

from __future__ import annotations

import numpy as np
import pytest

from abstraction_regret_gb300 import native, staging
from abstraction_regret_gb300 import workloads as W
from abstraction_regret_gb300.engine import PersistentEngine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pageable():
    import torch

    with torch.cuda.device(0):
        if native.lib().gbfsm_pageable_access() <= 0:
            pytest.skip("this device does not read pageable host memory")


def _mixed_inputs(seed: int):
    rng = np.random.default_rng(seed)
    store = bytearray(rng.integers(0, 256, 3 << 20, dtype=np.uint8).tobytes())
    out = []
    for k in range(300):
        length = int(rng.choice([0, 1, 7, 15, 16, 17, 31, 33, 1000, 4093, 65537,
                                 int(rng.integers(0, 40000))]))
        kind = k % 4
        if kind == 0:
            out.append(rng.integers(0, 256, length, dtype=np.uint8).tobytes())
        elif kind == 1:
            start = int(rng.integers(0, len(store) - length))
            out.append(memoryview(store)[start:start + length])
        elif kind == 2:
            out.append(bytearray(rng.integers(0, 256, length, dtype=np.uint8).tobytes()))
        else:
            a = rng.integers(0, 256, length + 9, dtype=np.uint8)
            out.append(a[int(rng.integers(0, 9)):][:length])
    return out


def test_gathered_batch_equals_the_packed_batch(pageable, monkeypatch):
    import torch

    monkeypatch.setattr(staging, "GATHER_MIN_BYTES", 0)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    inputs = _mixed_inputs(3)
    got = staging.Staging(dev, gather=True)
    want = staging.Staging(dev, gather=False)
    for _ in range(2):  # reused buffers
        d1, o1, _, t1 = got.put(inputs, stream)
        assert got.last_path == "gather"
        d2, o2, _, t2 = want.put(inputs, stream)
        assert want.last_path == "pack"
        stream.synchronize()
        assert t1 == t2 and torch.equal(o1, o2)
        assert torch.equal(d1[:t1 + 16 - t1 % 16].cpu(), d2[:t2 + 16 - t2 % 16].cpu())


def test_engine_batch_read_in_place_matches_the_oracle(pageable):
    b = W.c3("live", n_inputs=96)
    eng = PersistentEngine(b.automata)
    inputs = b.inputs()
    assert sum(map(len, inputs)) >= staging.GATHER_MIN_BYTES
    f, l, e, _, _ = eng.run_requests(np.zeros(b.n_inputs), inputs, with_examined=True)
    assert eng._staging.last_path == "gather"
    of, ol, oe, _ = O.nfa_batch(b.automata[0], b.data, b.offsets)
    assert np.array_equal(f, of) and np.array_equal(l, ol) and np.array_equal(e, oe)
