"""The drop-in path on the GPU: ``plugin.install()`` into a host registry, then the host's
``run_batch`` through the factories it registered (GPU).

The reference package (gpufsm 0.1.0) can be imported only from its checkout, which
exists in the development container and not on the machines that run the GPU tests.
So the host here is a stand-in: fresh module instances of this package's ``registry``
and ``result`` modules, which restate gpufsm's registry (src/gpufsm/core/registry.py:
50-162) and result (core/result.py:11-50) contracts, and a ``run_batch`` that resolves
a factory and calls it exactly as gpufsm's does (src/gpufsm/api.py:27-62). Everything
below the registry -- the plugin's factories and adapter, the executor cache, the
executors and the kernels -- is the code that runs under gpufsm. ``test_plugin.py``
installs the same plugin into the real gpufsm registry on the CPU; where gpufsm and a
GPU are both present, ``test_reference_gpu_suite_unchanged`` runs the reference's own
GPU test files, unchanged, after the install.
"""

from __future__ import annotations

import importlib.util
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import abstraction_regret_gb300 as G
from abstraction_regret_gb300 import plugin
from abstraction_regret_gb300 import workloads as W
from oracle import oracle as O

from .golden_data import load, nfa_from

pytestmark = pytest.mark.gpu

PKG = Path(G.__file__).resolve().parent
REPO = PKG.parent


def _fresh(name: str):
    """A new instance of a module of this package (its own registry dictionaries)."""
    spec = importlib.util.spec_from_file_location(f"abstraction_regret_gb300._host_{name}",
                                                  PKG / f"{name}.py")
    mod = importlib.util.module_from_spec(spec)
    mod.__package__ = "abstraction_regret_gb300"
    sys.modules[spec.name] = mod  # dataclasses resolve their annotations through it
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def host():
    R = _fresh("registry")
    Res = _fresh("result")
    names = plugin.install(gpufsm_registry=R, gpufsm_result=Res)
    assert len(names) >= 17
    return R, Res


def _run_batch(R, automaton, inputs, technique=None):
    """gpufsm.api.run_batch's resolution and call (api.py:27-52), CUDA backend."""
    kind = R.Kind.of(automaton)
    name, factory = R.get_factory(kind, R.Backend.CUDA, technique)
    ex = factory(automaton, name)
    return ex, ex.run_batch(list(inputs))


def _pairs(res):
    return [(r.accepted, r.match_len) for r in res]


def test_probe_says_available(host):
    R, _ = host
    assert R.is_available(R.Backend.CUDA)
    assert R.Backend.CUDA in R.available_backends()


def test_every_nfa_technique_through_the_plugin(host):
    R, Res = host
    corpus = load("reference_corpus.json.gz")["nfa_cases"]
    cases = [c for c in corpus if c["id"].startswith("example:")] + \
        [c for c in corpus if c["id"].startswith("fuzz:")][:40]
    assert len(cases) == 56
    b = W.c1("live")
    live = b.inputs()
    want_live = O.verdicts(b.automata[0], live)
    for technique in R.list_techniques(R.Backend.CUDA, R.Kind.NFA):
        for c in cases:
            nfa, data = nfa_from(c["nfa"]), bytes.fromhex(c["input_hex"])
            _, res = _run_batch(R, nfa, [data], technique)
            assert _pairs(res) == O.verdicts(nfa, [data]), (technique, c["id"])
            assert type(res[0]) is Res.Result
        _, res = _run_batch(R, b.automata[0], live, technique)
        assert _pairs(res) == want_live, technique


def test_every_dfa_technique_through_the_plugin(host):
    R, Res = host
    for n in (16, 256, 4096):
        dfa = G.random_dfa(n, accept_prob=0.02, seed=n)
        rng = np.random.default_rng(n)
        inputs = [rng.integers(0, 256, int(k), dtype=np.uint8).tobytes()
                  for k in rng.integers(0, 2000, 48)]
        want = O.verdicts(dfa, inputs)
        for technique in R.list_techniques(R.Backend.CUDA, R.Kind.DFA):
            _, res = _run_batch(R, dfa, inputs, technique)
            assert _pairs(res) == want, (technique, n)
            assert type(res[0]) is Res.Result


def test_default_technique_reaches_the_chunked_engine(host):
    """run_batch(nfa, inputs) with no technique: long inputs go to the engine."""
    R, _ = host
    b = W.c3("sustained", n_inputs=64)
    inputs = b.inputs()
    ex, res = _run_batch(R, b.automata[0], inputs)
    assert ex._inner.last_path == "engine"
    of, ol, _, _ = O.nfa_batch(b.automata[0], b.data, b.offsets)
    assert _pairs(res) == list(zip(of.astype(bool).tolist(), ol.tolist()))
    # short inputs: one plain launch
    short = [x[:100] for x in inputs[:8]]
    ex, res = _run_batch(R, b.automata[0], short)
    assert ex._inner.last_path == "plain"
    assert _pairs(res) == O.verdicts(b.automata[0], short)


REF_SRC = Path(os.environ.get("GPUFSM_REFERENCE_SRC", "/nonexistent"))
REF_TESTS = REF_SRC.parent / "tests"


@pytest.mark.skipif(not (REF_SRC / "gpufsm").is_dir() or not REF_TESTS.is_dir(),
                    reason="the reference checkout (GPUFSM_REFERENCE_SRC) is not present here")
def test_reference_gpu_suite_unchanged():
    """The reference's GPU tests, unchanged, with this engine installed as its CUDA
    backend (a pytest plugin module calls plugin.install() before collection)."""
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1",
               PYTHONPATH=os.pathsep.join([str(REPO), str(REF_SRC)]))
    files = [str(REF_TESTS / f) for f in ("test_gpu_backends.py", "test_dfa_gpu.py",
                                          "test_worklist_warp.py")]
    res = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider",
                          "-p", "abstraction_regret_gb300.pytest_install", "-m", "gpu",
                          *files], capture_output=True, text=True, env=env, timeout=1800)
    assert res.returncode == 0, res.stdout[-4000:] + res.stderr[-2000:]
    assert " passed" in res.stdout and " skipped" not in res.stdout.split("\n")[-2]
