"""ctypes binding of ``libgbfsm.so`` (the C ABI declared in ``include/gbfsm.h``).

The library is loaded from this package directory (an in-tree build, see ``build.py``).
There is no fallback: if the library is missing or fails to load, ``lib()`` raises, and
the CUDA backend reports itself unavailable with that reason.

Status codes map onto the exceptions the reference raises for the same conditions:
``GBFSM_INVALID_ARG`` -> ``ValueError`` (as ``pack_inputs`` does, core/packing.py:49-53),
``GBFSM_OOM`` -> ``MemoryError``, ``GBFSM_TIMEOUT`` -> ``TimeoutError`` and everything
else -> ``RuntimeError`` (the reference's ``CUDA_CHECK`` -> ``std::runtime_error``,
native/include/common.cuh:63-71).
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

# The in-tree build; GBFSM_LIBRARY points at another build of the same ABI (e.g. a
# tuning variant made with ``python -m abstraction_regret_gb300.build --out``).
LIB_PATH = Path(os.environ.get("GBFSM_LIBRARY") or Path(__file__).resolve().parent / "libgbfsm.so")

OK, INVALID_ARG, UNSUPPORTED, CUDA_ERROR, TIMEOUT, OOM = range(6)

TECH_BITMAP, TECH_WARP, TECH_COMPACT, TECH_DFA_WALK = range(4)

NFA_HAS_EPS = 1
NFA_HAS_ANY = 2

EDGE_SYMBOL_MASK = 0x1FF
EDGE_ACCEPT = 1 << 9
EDGE_HAS_EPS = 1 << 10

FLAG_TIMEOUT = -1


class Edge(ctypes.Structure):
    _fields_ = [("target", ctypes.c_uint32), ("info", ctypes.c_uint32),
                ("row_begin", ctypes.c_uint32), ("row_end", ctypes.c_uint32)]


class NfaDev(ctypes.Structure):
    _fields_ = [
        ("num_states", ctypes.c_int32),
        ("start_state", ctypes.c_int32),
        ("num_words", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("sym_row", ctypes.c_void_p),
        ("sym_edges", ctypes.c_void_p),
        ("eps_row", ctypes.c_void_p),
        ("eps_edges", ctypes.c_void_p),
        ("accept_words", ctypes.c_void_p),
        ("num_sym_edges", ctypes.c_uint64),
        ("num_eps_edges", ctypes.c_uint64),
        ("first_row", ctypes.c_void_p),
        ("first_edges", ctypes.c_void_p),
        ("edge_sym", ctypes.c_void_p),
        ("pair_row", ctypes.c_void_p),
        ("pair_lanes", ctypes.c_void_p),
        ("lane_edges", ctypes.c_void_p),
        ("lane_labels_ext", ctypes.c_void_p),
    ]


class LaneRec(ctypes.Structure):
    _fields_ = [("state", ctypes.c_uint32), ("row_begin", ctypes.c_uint32),
                ("labels_lo", ctypes.c_uint32), ("labels_hi", ctypes.c_uint32)]


LANE_STATE_BITS = 25  # GBFSM_LANE_STATE_MASK
LANE_DEG_SHIFT = 25
LANE_SLOW = 1 << 30
LANE_ACCEPT = 1 << 31
LANE_FAST_DEGREE = 16  # most out-edges of a state in the packed-label form


class DfaDev(ctypes.Structure):
    _fields_ = [
        ("num_states", ctypes.c_int32),
        ("start_state", ctypes.c_int32),
        ("entry_bytes", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("table", ctypes.c_void_p),
        ("accept_bits", ctypes.c_void_p),
        ("table_bytes", ctypes.c_uint64),
    ]


class Plan(ctypes.Structure):
    _fields_ = [
        ("technique", ctypes.c_int32),
        ("block_threads", ctypes.c_int32),
        ("list_capacity", ctypes.c_int32),
        ("stage", ctypes.c_int32),
        ("ctas_per_sm", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 3),
    ]


class Automaton(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("technique", ctypes.c_int32),
        ("list_capacity", ctypes.c_int32),
        ("dfa_overlap", ctypes.c_int32),
        ("nfa", NfaDev),
        ("dfa", DfaDev),
    ]


class Task(ctypes.Structure):
    _fields_ = [("automaton", ctypes.c_int32), ("first", ctypes.c_int32),
                ("count", ctypes.c_int32), ("kind", ctypes.c_int32)]


class Chunk(ctypes.Structure):
    _fields_ = [("input", ctypes.c_int32), ("index", ctypes.c_int32),
                ("begin", ctypes.c_int64), ("end", ctypes.c_int64)]


class ChunkIO(ctypes.Structure):
    _fields_ = [("chunks", ctypes.c_void_p), ("records", ctypes.c_void_p),
                ("overflow_tasks", ctypes.c_void_p), ("overflow_count", ctypes.c_void_p),
                ("task_count", ctypes.c_void_p), ("n_chunks", ctypes.c_int32),
                ("aut_ids", ctypes.c_void_p)]


PLAN_MAX_SLICES = 16  # GBFSM_PLAN_MAX_SLICES


class BatchPlanArgs(ctypes.Structure):
    _fields_ = [
        ("n_inputs", ctypes.c_int32), ("n_automata", ctypes.c_int32),
        ("offsets", ctypes.c_void_p), ("ends", ctypes.c_void_p),
        ("aut_ids", ctypes.c_void_p), ("aut_class", ctypes.c_void_p),
        ("aut_dfa_chunk", ctypes.c_void_p),
        ("lane_warps", ctypes.c_int32), ("persist_warps", ctypes.c_int32),
        ("dfa_warps", ctypes.c_int32),
        ("min_chunk", ctypes.c_int32), ("fixed_chunk", ctypes.c_int32),
        ("n_slices", ctypes.c_int32), ("shrink", ctypes.c_float),
        ("slice_first", ctypes.c_int32 * (PLAN_MAX_SLICES + 1)),
        ("cap_chunks", ctypes.c_int32), ("cap_lane_tasks", ctypes.c_int32),
        ("cap_persist_tasks", ctypes.c_int32), ("cap_fixup_tasks", ctypes.c_int32),
        ("cap_dfa_chunk_tasks", ctypes.c_int32), ("cap_dfa_fixup_tasks", ctypes.c_int32),
        ("chunks", ctypes.c_void_p), ("tasks_lanes", ctypes.c_void_p),
        ("tasks_persist", ctypes.c_void_p), ("tasks_fixup", ctypes.c_void_p),
        ("tasks_dfa_chunk", ctypes.c_void_p), ("tasks_dfa_fixup", ctypes.c_void_p),
        ("dfa_latch", ctypes.c_void_p),
        ("input_ids", ctypes.c_void_p), ("header", ctypes.c_void_p),
        ("scratch", ctypes.c_void_p),
    ]


# automaton classes and header words of gbfsm_batch_plan
PLAN_NFA_WHOLE, PLAN_NFA_WARP, PLAN_NFA_LANES, PLAN_DFA = 0, 1, 2, 3
PLAN_HEADER_WORDS = 64
(PLAN_STATUS, PLAN_LANE_CHUNKS, PLAN_CHUNKS, PLAN_LANE_FIRST, PLAN_LANE_TASKS,
 PLAN_PERSIST_TASKS, PLAN_FIXUP_TASKS, PLAN_LANE_BYTES, PLAN_WARP_BYTES, PLAN_OVERFLOW,
 PLAN_WHOLE, PLAN_DFA_INPUTS, PLAN_DFA_CHUNKS, PLAN_DFA_FIXUPS,
 PLAN_DFA_CHUNK_BYTES) = range(15)
PLAN_SLICES = 16

(TASK_WHOLE, TASK_CHUNK, TASK_FIXUP, TASK_LANES, TASK_DFA_GROUP, TASK_DFA_CHUNK,
 TASK_DFA_FIXUP) = range(7)
LANE_CAPACITY = 4  # members a lane holds (kLaneSlots)
CHUNK_RECORD_BYTES = 256
STATIC_SCRATCH_BYTES = 32 << 20  # GBFSM_STATIC_SCRATCH_BYTES
CHUNK_DTYPE = [("input", "<i4"), ("index", "<i4"), ("begin", "<i8"), ("end", "<i8")]


_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64
_sz = ctypes.c_size_t
_P = ctypes.POINTER

# name -> (restype, argtypes). Every function declared in include/gbfsm.h.
SIGNATURES: dict[str, tuple] = {
    "gbfsm_abi_version": (ctypes.c_int, []),
    "gbfsm_last_error": (ctypes.c_char_p, []),
    "gbfsm_nfa_layout": (ctypes.c_int, [_i32, _vp, _vp, _vp, _vp, _vp, _vp, _u64, _u64, _vp, _vp,
                                        _vp, _vp, _vp, _vp, _vp]),
    "gbfsm_dfa_layout": (ctypes.c_int, [_i32, _vp, _vp, _i32, _vp, _vp, _vp, _vp]),
    "gbfsm_nfa_workspace_bytes": (_sz, [_P(NfaDev), _i32, _P(Plan)]),
    "gbfsm_nfa_run": (ctypes.c_int, [_P(NfaDev), _vp, _vp, _i32, _P(Plan), _vp, _vp, _vp, _vp,
                                     _sz, _vp]),
    "gbfsm_dfa_run": (ctypes.c_int, [_P(DfaDev), _vp, _vp, _i32, _P(Plan), _vp, _vp, _vp, _vp]),
    "gbfsm_persistent_workspace_bytes": (_sz, [_i32, _P(Plan)]),
    "gbfsm_persistent_ctas_per_sm": (_i32, [_i32, _P(Plan)]),
    "gbfsm_persistent_run": (ctypes.c_int, [_vp, _i32, _i32, _vp, _i32, _vp, _vp, _vp, _vp,
                                            _P(ChunkIO), _vp, _vp, _vp, _vp, _sz, _P(Plan), _vp]),
    "gbfsm_run_multistream": (ctypes.c_int, [_vp] * 8 + [_i32] * 4 + [_vp] * 3),
    "gbfsm_run_multistream_shared": (ctypes.c_int, [_vp] * 8 + [_i32] * 4 + [_vp] * 3),
    "gbfsm_run_multistream_async": (ctypes.c_int, [_vp] * 8 + [_i32] * 4 + [_vp] * 3),
    "gbfsm_run_worklist": (ctypes.c_int, [_vp] * 8 + [_i32] * 4 + [_vp] * 3),
    "gbfsm_run_worklist_global": (ctypes.c_int, [_vp] * 8 + [_i32] * 4 + [_vp] * 3),
    "gbfsm_run_worklist_warp": (ctypes.c_int, [_vp] * 8 + [_i32] * 4 + [_vp] * 3),
    "gbfsm_run_worklist_compact": (ctypes.c_int, [_vp] * 8 + [_i32] * 4 + [_vp] * 3),
    "gbfsm_run_worklist_shared": (ctypes.c_int, [_vp] * 8 + [_i32] * 4 + [_vp] * 3),
    "gbfsm_run_dense": (ctypes.c_int, [_vp] * 7 + [_i32] * 4 + [_vp] * 3),
    "gbfsm_run_bitpacked": (ctypes.c_int, [_vp] * 7 + [_i32] * 4 + [_vp] * 3),
    "gbfsm_run_dfa": (ctypes.c_int, [_vp] * 4 + [_i32] * 3 + [_vp] * 3),
    "gbfsm_run_nfa_bytes": (ctypes.c_int, [_vp] * 6 + [_i32] * 2 + [_vp] * 2 + [_i32] +
                            [_P(Plan)] + [_vp] * 3),
    "gbfsm_run_dfa_bytes": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp, _vp, _i32, _P(Plan), _vp, _vp,
                                           _vp]),
    "gbfsm_host_device_pointer": (ctypes.c_int, [_vp, _P(_vp)]),
    "gbfsm_lanes_warps_per_sm": (_i32, []),
    "gbfsm_lanes_run": (ctypes.c_int, [_vp, _i32, _vp, _i32, _vp, _vp, _P(ChunkIO), _vp]),
    "gbfsm_nfa_run_static": (ctypes.c_int, [_P(NfaDev), _vp, _vp, _i32, _P(Plan), _vp, _vp,
                                            _vp, _vp]),
    "gbfsm_workload_walk": (_i32, [_i32, _vp, _vp, _vp, _vp, _i32, _vp, _i32, _u64, _vp, _i32]),
    "gbfsm_lanes_run_range": (ctypes.c_int, [_vp, _i32, _vp, _i32, _vp, _vp, _vp, _P(ChunkIO),
                                             _vp]),
    "gbfsm_batch_plan_scratch_bytes": (_sz, [_i32]),
    "gbfsm_batch_plan": (ctypes.c_int, [_P(BatchPlanArgs), _vp]),
    "gbfsm_probe_l2_read": (ctypes.c_int, [_vp, _sz, _i32, _vp, _vp]),
    "gbfsm_probe_gather16": (ctypes.c_int, [_vp, _sz, _i64, _i32, _vp, _vp]),
    "gbfsm_probe_chase": (ctypes.c_int, [_vp, ctypes.c_uint32, _i64, _i32, _vp, _vp]),
    "gbfsm_probe_smem": (ctypes.c_int, [_i64, _i32, _vp, _vp]),
    "gbfsm_probe_copy": (ctypes.c_int, [_vp, _vp, _sz, _i32, _vp]),
    "gbfsm_pageable_access": (_i32, []),
    "gbfsm_gather_inputs": (ctypes.c_int, [_vp, _vp, _i32, _vp, _vp]),
    "gbfsm_dfa_chunks_warps_per_sm": (_i32, [_i32]),
    "gbfsm_dfa_chunks_run": (ctypes.c_int, [_vp, _i32, _vp, _i32, _vp, _vp, _vp, _vp,
                                            _P(ChunkIO), _i32, _vp, _vp, _vp, _vp, _vp]),
}

ABI_VERSION = 3

_lib: ctypes.CDLL | None = None


def lib() -> ctypes.CDLL:
    """The loaded library with every signature bound. Raises if it is absent or stale."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is not built; run `python -m abstraction_regret_gb300.build`"
            )
        handle = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        version = handle.gbfsm_abi_version()
        if version != ABI_VERSION:
            raise ImportError(f"libgbfsm ABI version {version}, expected {ABI_VERSION}")
        _lib = handle
    return _lib


def last_error() -> str:
    msg = lib().gbfsm_last_error()
    return msg.decode(errors="replace") if msg else ""


def check(status: int, what: str) -> None:
    """Raise the exception that corresponds to a gbfsm_status."""
    if status == OK:
        return
    msg = f"{what}: {last_error()}"
    if status == INVALID_ARG:
        raise ValueError(msg)
    if status == OOM:
        raise MemoryError(msg)
    if status == TIMEOUT:
        raise TimeoutError(msg)
    raise RuntimeError(msg)


def device_pointer(host_ptr: int) -> int:
    """Device address of page-locked host memory at ``host_ptr`` (raises if not mapped)."""
    out = ctypes.c_void_p()
    check(lib().gbfsm_host_device_pointer(host_ptr, ctypes.byref(out)), "gbfsm_host_device_pointer")
    return int(out.value or 0)


def make_plan(technique: int, block_threads: int = 0, list_capacity: int = 0, stage: int = 0,
              ctas_per_sm: int = 0) -> Plan:
    p = Plan()
    p.technique = technique
    p.block_threads = block_threads
    p.list_capacity = list_capacity
    p.stage = stage
    p.ctas_per_sm = ctas_per_sm
    return p
