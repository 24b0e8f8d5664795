"""The C ABI without a GPU: the library loads, exports exactly what include/gbfsm.h
declares, and rejects bad arguments with status codes (no exception crosses the ABI).

Mirrors the reference's native-surface check (tests/test_cuda_api_surface.py:60-105),
which cross-checks api.hpp declarations against the .cu definitions and bindings.
"""

from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from abstraction_regret_gb300 import build, native

REPO = Path(__file__).resolve().parent.parent
HEADER = REPO / "include" / "gbfsm.h"


def declared() -> set[str]:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    names = set(re.findall(r"\b(gbfsm_\w+)\s*\(", text))
    return {n for n in names if not n.startswith("gbfsm_status")}


@pytest.fixture(scope="module")
def lib():
    build.build()
    return native.lib()


def test_header_declares_the_reference_entry_points():
    names = declared()
    # one entry per _cuda.run_* of the reference (native/include/api.hpp:23-104)
    for ref in ("dense", "bitpacked", "multistream", "multistream_shared", "multistream_async",
                "worklist", "worklist_global", "worklist_warp", "worklist_compact",
                "worklist_shared", "dfa"):
        assert f"gbfsm_run_{ref}" in names
    for dev in ("gbfsm_nfa_run", "gbfsm_dfa_run", "gbfsm_persistent_run",
                "gbfsm_nfa_workspace_bytes", "gbfsm_last_error", "gbfsm_abi_version"):
        assert dev in names


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(native.LIB_PATH)],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (gbfsm_\w+)", out))
    missing = declared() - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    extra = {n for n in exported if n.startswith("gbfsm_")} - declared()
    assert not extra, f"exported but not declared: {sorted(extra)}"


def test_python_binding_covers_the_header(lib):
    assert set(native.SIGNATURES) == declared()
    assert lib.gbfsm_abi_version() == native.ABI_VERSION


PLAN_FIELDS = ("aut_dfa_chunk", "lane_warps", "dfa_warps", "n_slices", "slice_first",
               "cap_chunks", "cap_dfa_chunk_tasks", "cap_dfa_fixup_tasks", "chunks", "tasks_dfa_chunk",
               "tasks_dfa_fixup", "dfa_latch", "input_ids", "scratch")


def test_struct_layouts_match_the_header(tmp_path):
    """Compile a probe against include/gbfsm.h and compare every struct with ctypes."""
    pairs = {"gbfsm_edge": native.Edge, "gbfsm_nfa_dev": native.NfaDev,
             "gbfsm_dfa_dev": native.DfaDev, "gbfsm_plan": native.Plan,
             "gbfsm_automaton": native.Automaton, "gbfsm_task": native.Task,
             "gbfsm_chunk": native.Chunk, "gbfsm_chunk_io": native.ChunkIO,
             "gbfsm_lane_rec": native.LaneRec, "gbfsm_batch_plan_args": native.BatchPlanArgs}
    src = tmp_path / "probe.c"
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gbfsm.h"', "int main(void) {"]
    for name in pairs:
        lines.append(f'  printf("{name} %zu\\n", sizeof({name}));')
    lines.append('  printf("record %d\\n", GBFSM_CHUNK_RECORD_BYTES);')
    lines.append('  printf("static %u\\n", GBFSM_STATIC_SCRATCH_BYTES);')
    for name in ("STATUS", "LANE_CHUNKS", "CHUNKS", "LANE_FIRST", "LANE_TASKS",
                 "PERSIST_TASKS", "FIXUP_TASKS", "LANE_BYTES", "WARP_BYTES", "OVERFLOW",
                 "WHOLE", "DFA_INPUTS", "DFA_CHUNKS", "DFA_FIXUPS", "DFA_CHUNK_BYTES", "SLICES", "MAX_SLICES", "HEADER_WORDS", "NFA_WHOLE",
                 "NFA_WARP", "NFA_LANES", "DFA"):
        lines.append(f'  printf("PLAN_{name} %d\\n", GBFSM_PLAN_{name});')
    for name in ("DFA_GROUP", "DFA_CHUNK", "DFA_FIXUP"):
        lines.append(f'  printf("TASK_{name} %d\\n", GBFSM_TASK_{name});')
    for field in PLAN_FIELDS:
        lines.append(f'  printf("off_{field} %zu\\n", '
                     f'offsetof(gbfsm_batch_plan_args, {field}));')
    lines.append('  printf("off_aut_ids %zu\\n", offsetof(gbfsm_chunk_io, aut_ids));')
    lines.append('  printf("off_dfa_overlap %zu\\n", offsetof(gbfsm_automaton, dfa_overlap));')
    lines.append("  return 0; }")
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", str(REPO / "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    for name, cls in pairs.items():
        assert int(out[name]) == ctypes.sizeof(cls), name
    assert int(out["record"]) == native.CHUNK_RECORD_BYTES
    assert int(out["static"]) == native.STATIC_SCRATCH_BYTES
    assert np.dtype(native.CHUNK_DTYPE).itemsize == ctypes.sizeof(native.Chunk)
    for key, value in out.items():
        if key.startswith(("PLAN_", "TASK_")):
            assert int(value) == getattr(native, key), key
    for field in PLAN_FIELDS:
        assert int(out[f"off_{field}"]) == getattr(native.BatchPlanArgs, field).offset, field
    assert int(out["off_aut_ids"]) == native.ChunkIO.aut_ids.offset
    assert int(out["off_dfa_overlap"]) == native.Automaton.dfa_overlap.offset


def test_invalid_arguments_return_status_codes(lib):
    plan = native.make_plan(native.TECH_COMPACT)
    st = lib.gbfsm_nfa_run(None, None, None, 0, ctypes.byref(plan), None, None, None, None, 0,
                           None)
    assert st == native.INVALID_ARG
    assert "NULL" in native.last_error()
    d = native.NfaDev()
    d.num_states, d.start_state, d.num_words = 10, 12, 1
    st = lib.gbfsm_nfa_run(ctypes.byref(d), None, None, 0, ctypes.byref(plan), None, None, None,
                           None, 0, None)
    assert st == native.INVALID_ARG and "start_state" in native.last_error()
    st = lib.gbfsm_dfa_layout(10, None, None, 3, None, None, None, None)
    assert st == native.INVALID_ARG
    dummy = ctypes.c_int32(0)
    p = ctypes.addressof(dummy)
    st = lib.gbfsm_dfa_layout(40000, p, p, 2, p, p, p, None)
    assert st == native.UNSUPPORTED
    assert lib.gbfsm_nfa_workspace_bytes(None, 10, None) == 0
    io = native.ChunkIO()
    st = lib.gbfsm_lanes_run(p, 1, p, 4, p, p, ctypes.byref(io), None)
    assert st == native.INVALID_ARG and "NULL" in native.last_error()
    assert lib.gbfsm_lanes_run(None, 0, None, 0, None, None, None, None) == native.OK
    assert lib.gbfsm_lanes_run(p, 1, p, -1, p, p, ctypes.byref(io), None) == native.INVALID_ARG
    st = lib.gbfsm_nfa_run_static(None, None, None, 4, ctypes.byref(plan), None, None, None,
                                  None)
    assert st == native.INVALID_ARG
    # DFA chunk launches: argument checks come before any device work
    assert lib.gbfsm_dfa_chunks_run(None, 0, None, 0, None, None, None, None, None, 1, None,
                                    None, None, None, None) == native.OK
    st = lib.gbfsm_dfa_chunks_run(p, 1, p, 4, None, p, p, None, None, 16, p, p, None, None,
                                  None)
    assert st == native.INVALID_ARG and "NULL" in native.last_error()
    io.chunks, io.records, io.n_chunks = p, p, 4
    st = lib.gbfsm_dfa_chunks_run(p, 1, p, 4, None, p, p, None, ctypes.byref(io), 40000, p, p,
                                  None, None, None)
    assert st == native.INVALID_ARG and "max_states" in native.last_error()
    a = native.BatchPlanArgs()
    a.n_inputs, a.n_automata, a.min_chunk, a.cap_chunks = 4, 1, 64, 8
    for f in ("offsets", "aut_class", "chunks", "tasks_lanes", "tasks_persist", "tasks_fixup",
              "input_ids", "header", "scratch", "aut_dfa_chunk"):
        setattr(a, f, p)
    st = lib.gbfsm_batch_plan(ctypes.byref(a), None)
    assert st == native.INVALID_ARG and "aut_dfa_chunk" in native.last_error()


def test_status_mapping_raises_the_reference_exception_types():
    with pytest.raises(ValueError):
        native.check(native.INVALID_ARG, "x")
    with pytest.raises(RuntimeError):
        native.check(native.CUDA_ERROR, "x")
    with pytest.raises(MemoryError):
        native.check(native.OOM, "x")
    with pytest.raises(TimeoutError):
        native.check(native.TIMEOUT, "x")
    native.check(native.OK, "x")


def test_workload_walk_is_deterministic_and_thread_independent(lib):
    from abstraction_regret_gb300 import workloads as W

    nfa = W.random_nfa(300, seed=5, poisson=3.0, accept_prob=0.01)
    off = W.offsets_of(np.array([0, 17, 4096, 1, 999], dtype=np.int64))
    a = W.walk_bytes(nfa, off, seed=3, threads=1)
    b = W.walk_bytes(nfa, off, seed=3, threads=5)
    assert a.tobytes() == b.tobytes()
    assert W.walk_bytes(nfa, off, seed=4).tobytes() != a.tobytes()
