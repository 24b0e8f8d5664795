"""Device-resident automata: the engine's GPU layouts, built once per automaton.

The reference re-uploads the CSR and re-packs the accept words on every call
(src/gpufsm/backends/cuda/nfa.py:44-52 and :105-121, ``dev_copy`` in
native/include/common.cuh:150-159). Here an automaton is uploaded once, converted on the
device by the layout kernels of ``libgbfsm`` (which also validate every index), and kept
resident as PyTorch tensors for as long as its executor lives.

NFA layout (``gbfsm_nfa_dev``): uint32 row arrays, 16-byte edge records
``{target, symbol | accept/eps flags of target, target's edge-row begin, end}`` and the
packed accept words (pack_accept layout). DFA layout (``gbfsm_dfa_dev``): 2-byte entries
(up to 32768 states) or 4-byte entries holding the successor with ``accept[successor]``
in the top bit, plus packed accept bits.
"""

from __future__ import annotations

import numpy as np
import torch

from . import native
from .automata import ALPHABET, ANY_SYMBOL
from .packing import words_for


def _stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _padded(n_elems: int, elem_bytes: int, device, dtype=torch.uint8) -> torch.Tensor:
    """A zero-filled device buffer of at least ``n_elems * elem_bytes`` bytes, padded to 16."""
    nbytes = max(16, -(-(n_elems * elem_bytes) // 16) * 16)
    itemsize = torch.empty((), dtype=dtype).element_size()
    return torch.zeros(nbytes // itemsize, dtype=dtype, device=device)


def _records(recs: np.ndarray, device) -> torch.Tensor:
    """uint32[k, 4] records as a 16-byte-aligned device buffer (at least one record)."""
    buf = _padded(max(1, recs.shape[0]), 16, device)
    if recs.size:
        buf[: recs.nbytes].copy_(torch.from_numpy(np.ascontiguousarray(recs, dtype=np.uint32)
                                                  .view(np.uint8).ravel()))
    return buf


def _to_dev(a: np.ndarray, dtype, device) -> torch.Tensor:
    arr = np.ascontiguousarray(a, dtype=dtype)
    if arr.size == 0:
        arr = np.zeros(4, dtype=dtype)
    return torch.from_numpy(arr).to(device)


def resolve_device(device=None) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("the CUDA backend needs a CUDA device (torch.cuda.is_available() is False)")
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    d = torch.device(device)
    if d.type != "cuda":
        raise ValueError(f"device must be a CUDA device, got {d}")
    return torch.device("cuda", d.index if d.index is not None else torch.cuda.current_device())


SUPERSET_LIMIT = 1 << 25  # records; above this an automaton is not chunked speculatively


def first_lists(nfa, limit: int = SUPERSET_LIMIT):
    """Per byte c, the distinct targets of edges labelled c or ANY, as engine state records.

    Returns ``(row int32[257], records uint32[k, 4])`` or ``None`` when the lists would
    exceed ``limit`` records (many wildcard targets). After consuming byte c an NFA's
    active set is contained in the epsilon closure of these targets, whatever the set
    before it: the starting superset of a speculative chunk.
    """
    n = int(nfa.num_states)
    syms = np.asarray(nfa.sym_symbols, dtype=np.int64)
    tgts = np.asarray(nfa.sym_targets, dtype=np.int64)
    any_t = np.unique(tgts[syms == ANY_SYMBOL])
    plain = syms != ANY_SYMBOL
    if int(plain.sum()) + 256 * any_t.size > limit:
        return None
    keys = syms[plain] * n + tgts[plain]
    if any_t.size:
        keys = np.concatenate([keys, (np.arange(256)[:, None] * n + any_t[None, :]).ravel()])
    keys = np.unique(keys)
    c, t = keys // n, keys % n
    row = np.zeros(257, dtype=np.int64)
    np.cumsum(np.bincount(c, minlength=256), out=row[1:])
    srp = np.asarray(nfa.sym_row_ptr, dtype=np.int64)
    recs = np.stack([t, _info(nfa, t), srp[t], srp[t + 1]], axis=1).astype(np.uint32)
    return row.astype(np.int32), recs


PAIR_LIMIT = 1 << 24  # records; above this an automaton gets no two-byte superset table


def _info(nfa, t: np.ndarray) -> np.ndarray:
    acc = np.asarray(nfa.accept, dtype=bool)
    erp = np.asarray(nfa.eps_row_ptr, dtype=np.int64)
    return (acc[t].astype(np.int64) << 9) | ((erp[t + 1] > erp[t]).astype(np.int64) << 10)


def pair_lists(nfa, first, limit: int = PAIR_LIMIT):
    """Two-byte supersets for an automaton without epsilon edges.

    For bytes c1, c2: the distinct targets, reachable by a c2 (or ANY) edge, of the states
    in ``first`` for c1 -- i.e. every state the automaton can occupy after reading c1 c2,
    from any set. Returns ``(row int32[65537], records uint32[k, 4])`` or ``None`` (epsilon
    edges, no first lists, or more than ``limit`` records).
    """
    if first is None or int(np.asarray(nfa.eps_targets).size):
        return None
    row1, recs1 = first
    n = int(nfa.num_states)
    srp = np.asarray(nfa.sym_row_ptr, dtype=np.int64)
    syms = np.asarray(nfa.sym_symbols, dtype=np.int64)
    tgts = np.asarray(nfa.sym_targets, dtype=np.int64)
    states = recs1[:, 0].astype(np.int64)
    c1_of = np.repeat(np.arange(256, dtype=np.int64), np.diff(row1.astype(np.int64)))
    deg = srp[states + 1] - srp[states]
    total = int(deg.sum())
    if total > 4 * limit:
        return None
    offs = np.cumsum(deg) - deg
    edge = np.arange(total, dtype=np.int64) - np.repeat(offs, deg) + np.repeat(srp[states], deg)
    c1_e = np.repeat(c1_of, deg)
    e_sym, e_tgt = syms[edge], tgts[edge]
    plain = e_sym != ANY_SYMBOL
    keys = (c1_e[plain] * 256 + e_sym[plain]) * n + e_tgt[plain]
    if (~plain).any():
        c1_a, t_a = c1_e[~plain], e_tgt[~plain]
        if c1_a.size * 256 > 4 * limit:
            return None
        keys = np.concatenate([keys, ((c1_a[:, None] * 256 + np.arange(256)[None, :]) * n
                                      + t_a[:, None]).ravel()])
    keys = np.unique(keys)
    if keys.size > limit:
        return None
    pair, t = keys // n, keys % n
    row = np.zeros(65537, dtype=np.int64)
    np.cumsum(np.bincount(pair, minlength=65536), out=row[1:])
    recs = np.stack([t, _info(nfa, t), srp[t], srp[t + 1]], axis=1).astype(np.uint32)
    return row.astype(np.int32), recs


def lane_state_records(nfa):
    """Lane record (gbfsm_lane_rec) of every state, uint32[n, 4], and the packed symbols
    of its edges 8..15, uint32[n, 2]; None when the automaton has 2^25 states or more."""
    n = int(nfa.num_states)
    if n >= 1 << native.LANE_STATE_BITS:
        return None
    srp = np.asarray(nfa.sym_row_ptr, dtype=np.int64)
    syms = np.asarray(nfa.sym_symbols, dtype=np.int64)
    nnz = int(srp[-1])
    deg = srp[1:] - srp[:-1]
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    has_any = np.bincount(src[syms == ANY_SYMBOL], minlength=n)[:n] > 0
    slow = (deg > native.LANE_FAST_DEGREE) | has_any
    j = np.arange(native.LANE_FAST_DEGREE, dtype=np.int64)
    idx = np.minimum(srp[:-1, None] + j[None, :], max(nnz - 1, 0))
    lab = np.where(j[None, :] < deg[:, None], syms[idx] if nnz else 0, 0) & 0xFF
    words = [lab[:, 4 * k] | (lab[:, 4 * k + 1] << 8) | (lab[:, 4 * k + 2] << 16)
             | (lab[:, 4 * k + 3] << 24) for k in range(4)]
    lo, hi = words[0], words[1]
    ext = np.stack([np.where(slow, 0, words[2]), np.where(slow, 0, words[3])], axis=1)
    acc = np.asarray(nfa.accept, dtype=bool)
    x = (np.arange(n, dtype=np.int64) | (np.where(slow, 0, deg) << native.LANE_DEG_SHIFT)
         | (slow.astype(np.int64) << 30) | (acc.astype(np.int64) << 31))
    recs = np.stack([x, srp[:-1], np.where(slow, srp[1:], lo), np.where(slow, 0, hi)], axis=1)
    return recs.astype(np.uint32), ext.astype(np.uint32)


class DeviceNFA:
    """An NFA (ours or gpufsm's, duck-typed on the CSR fields) resident on a GPU."""

    def __init__(self, nfa, device=None) -> None:
        dev = resolve_device(device)
        lib = native.lib()
        n = int(nfa.num_states)
        if n < 1:
            raise ValueError("cannot simulate an NFA with zero states")
        start = int(nfa.start_state)
        if not 0 <= start < n:
            raise ValueError(f"start_state {start} out of range (0..{n - 1})")
        srp = np.asarray(nfa.sym_row_ptr)
        erp = np.asarray(nfa.eps_row_ptr)
        if srp.shape != (n + 1,) or erp.shape != (n + 1,):
            raise ValueError("row pointer arrays must have num_states + 1 entries")
        ssy = np.asarray(nfa.sym_symbols)
        nnz, nne = int(srp[-1]), int(erp[-1])
        if nnz != np.asarray(nfa.sym_targets).size or nne != np.asarray(nfa.eps_targets).size:
            raise ValueError("row pointers disagree with the edge array lengths")
        self.device = dev
        self.num_states = n
        self.start_state = start
        self.num_words = words_for(n)
        self.num_sym_edges = nnz
        self.num_eps_edges = nne
        self.has_eps = nne > 0
        self.uses_any = bool(np.any(ssy == ANY_SYMBOL)) if nnz else False
        with torch.cuda.device(dev):
            src = [_to_dev(nfa.sym_row_ptr, np.int32, dev), _to_dev(nfa.sym_targets, np.int32, dev),
                   _to_dev(nfa.sym_symbols, np.int32, dev), _to_dev(nfa.eps_row_ptr, np.int32, dev),
                   _to_dev(nfa.eps_targets, np.int32, dev), _to_dev(nfa.accept, np.uint8, dev)]
            self.sym_row = _padded(n + 1, 4, dev)
            self.eps_row = _padded(n + 1, 4, dev)
            self.sym_edges = _padded(max(nnz, 1), 16, dev)
            self.eps_edges = _padded(max(nne, 1), 16, dev)
            self.accept_words = _padded(self.num_words, 8, dev)
            err = torch.zeros(4, dtype=torch.int32, device=dev)
            status = lib.gbfsm_nfa_layout(
                n, src[0].data_ptr(), src[1].data_ptr(), src[2].data_ptr(), src[3].data_ptr(),
                src[4].data_ptr(), src[5].data_ptr(), nnz, nne, self.sym_row.data_ptr(),
                self.sym_edges.data_ptr(), self.eps_row.data_ptr(), self.eps_edges.data_ptr(),
                self.accept_words.data_ptr(), err.data_ptr(), _stream_handle(dev))
            native.check(status, "gbfsm_nfa_layout")
            code = int(err[0].item())  # synchronises: the layout is checked before any use
            if code:
                raise ValueError(f"invalid NFA: layout check failed with code {code} "
                                 f"(1 row pointers, 2 target, 3 symbol, 4 epsilon target)")
        d = native.NfaDev()
        d.num_states = n
        d.start_state = start
        d.num_words = self.num_words
        d.flags = (native.NFA_HAS_EPS if self.has_eps else 0) | (
            native.NFA_HAS_ANY if self.uses_any else 0)
        d.sym_row = self.sym_row.data_ptr()
        d.sym_edges = self.sym_edges.data_ptr()
        d.eps_row = self.eps_row.data_ptr()
        d.eps_edges = self.eps_edges.data_ptr()
        d.accept_words = self.accept_words.data_ptr()
        d.num_sym_edges = nnz
        d.num_eps_edges = nne
        lists = first_lists(nfa)
        self.speculative = lists is not None
        if lists is not None:
            row, recs = lists
            with torch.cuda.device(dev):
                self.first_row = torch.from_numpy(np.ascontiguousarray(row)).to(dev)
                self.first_edges = _padded(max(1, recs.shape[0]), 16, dev)
                if recs.size:
                    self.first_edges[: recs.nbytes].copy_(
                        torch.from_numpy(np.ascontiguousarray(recs).view(np.uint8).ravel()))
            d.first_row = self.first_row.data_ptr()
            d.first_edges = self.first_edges.data_ptr()
        pairs = pair_lists(nfa, lists)
        self.lanes = pairs is not None
        self.pair_sizes = np.diff(pairs[0]).astype(np.int32) if pairs is not None else None
        self.pair_mean = float(self.pair_sizes.mean()) if pairs is not None else float("inf")
        lane = lane_state_records(nfa) if pairs is not None else None
        if lane is None:
            pairs = None
            self.lanes = False
            self.pair_sizes, self.pair_mean = None, float("inf")
        if pairs is not None:
            prow, precs = pairs
            tg = np.asarray(nfa.sym_targets, dtype=np.int64)
            with torch.cuda.device(dev):
                self.edge_sym = _padded(max(1, nnz), 2, dev, torch.int16)
                if nnz:
                    self.edge_sym[:nnz].copy_(torch.from_numpy(
                        np.ascontiguousarray(ssy, dtype=np.int16)))
                self.pair_row = torch.from_numpy(np.ascontiguousarray(prow)).to(dev)
                lane_states, lane_ext = lane
                self.pair_lanes = _records(lane_states[precs[:, 0].astype(np.int64)], dev)
                self.lane_edges = _records(lane_states[tg] if nnz else lane_states[:0], dev)
                self.lane_labels_ext = torch.from_numpy(
                    np.ascontiguousarray(lane_ext).view(np.int32).ravel()).to(dev)
            d.edge_sym = self.edge_sym.data_ptr()
            d.pair_row = self.pair_row.data_ptr()
            d.pair_lanes = self.pair_lanes.data_ptr()
            d.lane_edges = self.lane_edges.data_ptr()
            d.lane_labels_ext = self.lane_labels_ext.data_ptr()
        self.desc = d

    @property
    def edge_bytes(self) -> int:
        """Bytes of the resident layout (rows + edge records + accept words)."""
        return (self.sym_row.numel() + self.eps_row.numel() + self.sym_edges.numel()
                + self.eps_edges.numel() + self.accept_words.numel())


class DeviceDFA:
    """A DFA (ours or gpufsm's) resident on a GPU as a packed transition table."""

    def __init__(self, dfa, device=None, entry_bytes: int | None = None) -> None:
        dev = resolve_device(device)
        lib = native.lib()
        n = int(dfa.num_states)
        if n < 1:
            raise ValueError("cannot simulate a DFA with zero states")
        start = int(dfa.start_state)
        if not 0 <= start < n:
            raise ValueError(f"start_state {start} out of range (0..{n - 1})")
        trans = np.asarray(dfa.trans)
        if trans.size != n * ALPHABET:
            raise ValueError(f"trans must have num_states * 256 = {n * ALPHABET} entries")
        if entry_bytes is None:
            entry_bytes = 2 if n <= 32768 else 4
        self.device = dev
        self.num_states = n
        self.start_state = start
        self.entry_bytes = entry_bytes
        self.table_bytes = n * ALPHABET * entry_bytes
        with torch.cuda.device(dev):
            t_dev = _to_dev(trans, np.int32, dev)
            a_dev = _to_dev(dfa.accept, np.uint8, dev)
            self.table = _padded(n * ALPHABET, entry_bytes, dev)
            self.accept_bits = _padded(-(-n // 32), 4, dev)
            err = torch.zeros(4, dtype=torch.int32, device=dev)
            status = lib.gbfsm_dfa_layout(n, t_dev.data_ptr(), a_dev.data_ptr(), entry_bytes,
                                          self.table.data_ptr(), self.accept_bits.data_ptr(),
                                          err.data_ptr(), _stream_handle(dev))
            native.check(status, "gbfsm_dfa_layout")
            code = int(err[0].item())
            if code:
                raise ValueError(f"invalid DFA: a successor is outside [0, {n}) (code {code})")
        d = native.DfaDev()
        d.num_states = n
        d.start_state = start
        d.entry_bytes = entry_bytes
        d.flags = 0
        d.table = self.table.data_ptr()
        d.accept_bits = self.accept_bits.data_ptr()
        d.table_bytes = self.table_bytes
        self.desc = d
