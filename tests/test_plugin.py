"""Installing the engine into the reference package's own registry (the drop-in path).

Runs only where the reference package (gpufsm 0.1.0) is importable; it is imported in a
child process (read-only checkout, no bytecode written) so this suite's own imports stay
untouched.
"""

from __future__ import annotations

import os
import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
REF_SRC = Path(os.environ.get("GPUFSM_REFERENCE_SRC", "/root/reference/src"))

pytestmark = pytest.mark.skipif(not (REF_SRC / "gpufsm").is_dir(),
                                reason="reference package not present on this machine")


def _run(code: str) -> str:
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1",
               PYTHONPATH=f"{REPO}{os.pathsep}{REF_SRC}")
    res = subprocess.run([sys.executable, "-c", textwrap.dedent(code)], capture_output=True,
                         text=True, env=env, timeout=300)
    assert res.returncode == 0, res.stderr[-3000:]
    return res.stdout


def test_install_registers_every_technique_with_declared_defaults():
    out = _run("""
        import gpufsm
        from gpufsm.core import registry as R
        import abstraction_regret_gb300.plugin as plugin
        names = plugin.install()
        nfa = R.list_techniques(R.Backend.CUDA, R.Kind.NFA)
        dfa = R.list_techniques(R.Backend.CUDA, R.Kind.DFA)
        assert {"worklist", "worklist_warp", "worklist_global", "worklist_shared",
                "worklist_compact", "multistream", "dense", "auto", "persistent"} <= set(nfa), nfa
        assert dfa == ["gather", "persistent"], dfa
        assert R.get_factory(R.Kind.NFA, R.Backend.CUDA, None)[0] == "auto"
        assert R.get_factory(R.Kind.DFA, R.Backend.CUDA, None)[0] == "gather"
        for (k, b), t in R._DEFAULTS.items():
            assert (k, b, t) in R._REGISTRY
        print(len(names))
    """)
    assert int(out.split()[-1]) >= 17


def test_availability_probe_is_replaced_and_explains_itself():
    out = _run("""
        import torch
        import gpufsm
        from gpufsm.core import registry as R
        import abstraction_regret_gb300.plugin as plugin
        plugin.install()
        ok = R.is_available(R.Backend.CUDA)
        print(ok, torch.cuda.is_available(), R.unavailable_reason(R.Backend.CUDA))
        if not ok:
            try:
                gpufsm.run_batch(gpufsm.random_dfa(8), [b"ab"], backend="cuda")
            except RuntimeError as exc:
                print("raised", "CUDA device" in str(exc))
    """)
    first = out.splitlines()[0].split()
    assert first[0] == first[1]  # available exactly when a device is visible
    if first[0] == "False":
        assert "CUDA device" in out and "raised True" in out


@pytest.mark.gpu
def test_reference_objects_run_through_the_engine_when_a_gpu_is_present():
    out = _run("""
        import torch
        if not torch.cuda.is_available():
            print("skip"); raise SystemExit(0)
        import gpufsm
        from gpufsm.examples import EXAMPLES
        import abstraction_regret_gb300.plugin as plugin
        plugin.install()
        for name, make in EXAMPLES.items():
            nfa, labelled = make()
            inputs = [d for d, _ in labelled]
            res = gpufsm.run_batch(nfa, inputs, backend="cuda")
            assert [(r.accepted, r.match_len) for r in res] == \
                [gpufsm.simulate(nfa, d) for d in inputs]
            assert type(res[0]).__module__ == "gpufsm.core.result"
        print("ok")
    """)
    assert out.strip().splitlines()[-1] in ("ok", "skip")


def test_adapter_results_equal_gpufsm_batch_results():
    """The adapter builds gpufsm's own Result objects while the device runs and fills in
    the verdicts afterwards: they must equal what gpufsm's batch_results builds from the
    same verdicts and times, field by field (a stand-in executor, no device)."""
    out = _run("""
        import numpy as np
        from gpufsm.core import result as GR
        import abstraction_regret_gb300.plugin as plugin

        rng = np.random.default_rng(0)
        flags = rng.integers(0, 2, 300).astype(np.int32)
        lens = rng.integers(0, 1 << 20, 300).astype(np.int32)

        class Stand:
            def __init__(self, call_idle):
                self.call_idle = call_idle
            def run_arrays(self, inputs, idle=None):
                if idle is not None and self.call_idle:
                    idle()
                n = len(inputs)
                return flags[:n], lens[:n], None, 1.25, 0.5

        for call_idle in (True, False):
            for n in (0, 1, 300):
                got = plugin._Adapter(Stand(call_idle), GR.Result).run_batch([b"x"] * n)
                want = GR.batch_results(flags[:n], lens[:n], 1.25, 0.5)
                assert got == want, (call_idle, n)
                assert all(type(g) is GR.Result for g in got)
                assert all(type(g.accepted) is bool and type(g.match_len) is int for g in got)
        print("ok")
    """)
    assert out.split()[-1] == "ok"
