"""ANML (Micron's Automata Network Markup Language) to the CSR ``NFA`` of this package.

Same subset and semantics as the reference's loader (src/gpufsm/io/anml.py:52-212): a
homogeneous automaton matches its symbol set on each state-transition element (STE),
so an ``activate-on-match`` edge u -> v becomes one edge u --c--> v per byte c of v's
symbol set. Three synthetic states come first:

* state 0, the start, with epsilon edges to states 1 and 2 (in that order);
* state 1 keeps itself active on every byte (an ANY self-loop, its first edge) and
  seeds the ``all-input`` STEs at every position;
* state 2 seeds the ``start-of-data`` STEs at position 0 only.

STE k of the document (in document order) is state 3 + k; ``report-on-match`` STEs
accept. Symbol sets: ``*`` (ANY), one atom (``0xHH``, ``\\xHH`` or one character), or a
bracketed class of atoms and ranges, negated by a leading ``^`` over 0..255 (``[^]`` is
every byte). Elements outside the subset (counters, boolean gates, ...), STEs without an
id or with a duplicate id, activations of unknown elements (``id:port`` resolves to
``id``), malformed atoms, empty classes and inverted ranges raise ``ValueError`` rather
than yield a different language.

The CSR is built with array operations, not one Python call per edge (real ANML
automata have tens of thousands of STEs and symbol sets of up to 256 bytes). Within a
state's row, edges keep the document order of the activations and the bytes of one
symbol set ascend; the reference orders those bytes by Python set iteration, which no
verdict depends on, so the tests compare rows as sorted (symbol, target) lists.
"""

from __future__ import annotations

import re
import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np

from .automata import ANY_SYMBOL, NFA

_HEX_ATOM = re.compile(r"(?:0x|\\x)[0-9a-fA-F]{2}", re.IGNORECASE)

# The homogeneous-STE subset; any other element changes the semantics and is refused.
ALLOWED_ELEMENTS = frozenset({"anml", "automata-network", "description",
                              "state-transition-element", "activate-on-match",
                              "report-on-match"})


def _atom(tok: str) -> int:
    if tok[:2].lower() in ("0x", "\\x"):
        return int(tok[2:], 16)
    if len(tok) == 1:
        return ord(tok)
    raise ValueError(f"unsupported ANML symbol atom: {tok!r}")


def parse_symbol_set(text: str) -> np.ndarray:
    """The bytes of an ANML symbol set, ascending (int32); ``[ANY_SYMBOL]`` for ``*``.

    An atom may denote a code point above 255 (a non-Latin-1 character); such a value is
    kept here and refused when an edge would carry it, as the reference's builder does.
    """
    s = text.strip()
    if s == "*":
        return np.array([ANY_SYMBOL], dtype=np.int32)
    if not (s.startswith("[") and s.endswith("]")):
        return np.array([_atom(s)], dtype=np.int32)
    body = s[1:-1]
    if not body:
        raise ValueError(f"empty ANML symbol-set {text!r}: the STE would be unreachable")
    negate = body.startswith("^")
    if negate:
        body = body[1:]
    atoms: list[str] = []
    i = 0
    while i < len(body):
        if body[i:i + 2].lower() in ("0x", "\\x"):
            tok = body[i:i + 4]
            if not _HEX_ATOM.fullmatch(tok):
                raise ValueError(f"malformed hex atom {tok!r} in ANML symbol-set {text!r}")
            atoms.append(tok)
            i += 4
        else:
            atoms.append(body[i])
            i += 1
    out: set[int] = set()
    j = 0
    while j < len(atoms):
        if j + 2 < len(atoms) and atoms[j + 1] == "-":
            lo, hi = _atom(atoms[j]), _atom(atoms[j + 2])
            if hi < lo:
                raise ValueError(f"inverted ANML range in {text!r}")
            out.update(range(lo, hi + 1))
            j += 3
        else:
            out.add(_atom(atoms[j]))
            j += 1
    if negate:
        mask = np.ones(256, dtype=bool)
        mask[[b for b in out if b < 256]] = False
        return np.flatnonzero(mask).astype(np.int32)
    return np.array(sorted(out), dtype=np.int32)


def _local(tag: str) -> str:
    return tag.rsplit("}", 1)[-1]


def anml_to_nfa(root: ET.Element, where: str = "<anml>") -> NFA:
    """The NFA of a parsed ANML document (see the module docstring)."""
    unsupported = sorted({_local(e.tag) for e in root.iter()} - ALLOWED_ELEMENTS)
    if unsupported:
        raise ValueError(f"{where}: unsupported ANML elements {unsupported} (only the "
                         f"homogeneous-STE subset is supported; counters/boolean gates "
                         f"change semantics)")
    stes = [e for e in root.iter() if _local(e.tag) == "state-transition-element"]
    if not stes:
        raise ValueError(f"no state-transition-element found in {where}")
    ids = [e.get("id") for e in stes]
    missing = sum(1 for i in ids if i is None)
    if missing:
        raise ValueError(f"{where}: {missing} state-transition-element(s) without an 'id' "
                         f"attribute")
    seen: set[str] = set()
    dup = sorted({i for i in ids if i in seen or seen.add(i)})
    if dup:
        raise ValueError(f"{where}: duplicate state-transition-element ids {dup[:5]}")
    index = {sid: k for k, sid in enumerate(ids)}
    cache: dict[str, np.ndarray] = {}
    symsets = []
    for e, sid in zip(stes, ids):
        raw = e.get("symbol-set", "*")
        if raw not in cache:
            try:
                cache[raw] = parse_symbol_set(raw)
            except ValueError as exc:
                raise ValueError(f"{where}: STE {sid!r}: {exc}") from None
        symsets.append(cache[raw])
    n = 3 + len(stes)
    accept = np.zeros(n, dtype=bool)
    # edge groups in insertion order: (source state, target STE index); each expands to
    # one edge per byte of the target's symbol set
    src = [1]
    tgt = [-1]  # the ANY self-loop of state 1
    for k, (e, sid) in enumerate(zip(stes, ids)):
        mode = (e.get("start") or "none").lower()
        if mode == "all-input":
            src.append(1)
            tgt.append(k)
        elif mode == "start-of-data":
            src.append(2)
            tgt.append(k)
        for child in e:
            t = _local(child.tag)
            if t == "activate-on-match":
                name = child.get("element")
                if name is None:
                    raise ValueError(f"{where}: STE {sid!r}: activate-on-match without "
                                     f"'element'")
                if name not in index and ":" in name:
                    name = name.split(":", 1)[0]
                if name not in index:
                    raise ValueError(f"{where}: STE {sid!r} activates unknown element "
                                     f"{child.get('element')!r}")
                src.append(3 + k)
                tgt.append(index[name])
            elif t == "report-on-match":
                accept[3 + k] = True
    src = np.asarray(src, dtype=np.int64)
    tgt = np.asarray(tgt, dtype=np.int64)
    sizes = np.array([1] + [symsets[t].size for t in tgt[1:]], dtype=np.int64)
    symbols = np.concatenate([np.array([ANY_SYMBOL], np.int32)] +
                             [symsets[t] for t in tgt[1:]]).astype(np.int32)
    bad = (symbols > 255) & (symbols != ANY_SYMBOL)
    if bad.any():
        raise ValueError(f"{where}: symbol must be 0..255 or ANY_SYMBOL, got "
                         f"{int(symbols[bad][0])}")
    e_src = np.repeat(src, sizes)
    e_tgt = np.repeat(np.where(tgt < 0, 1, tgt + 3), sizes)
    order = np.argsort(e_src, kind="stable")  # rows in insertion order
    row = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(np.bincount(e_src, minlength=n), out=row[1:])
    eps_row = np.zeros(n + 1, dtype=np.int32)
    eps_row[1:] = 2
    return NFA(num_states=n, start_state=0, accept=accept, sym_row_ptr=row,
               sym_targets=e_tgt[order].astype(np.int32),
               sym_symbols=symbols[order].astype(np.int32),
               eps_row_ptr=eps_row, eps_targets=np.array([1, 2], dtype=np.int32))


def load_anml(path) -> NFA:
    """Load an ANML file (the reference's ``gpufsm.io.anml.load_anml``)."""
    root = ET.parse(path).getroot()  # noqa: S314 - local automata files
    return anml_to_nfa(root, str(path))


def load_anml_string(text: str) -> NFA:
    """Load ANML from a string."""
    return anml_to_nfa(ET.fromstring(text), "<string>")  # noqa: S314


__all__ = ["ALLOWED_ELEMENTS", "anml_to_nfa", "load_anml", "load_anml_string",
           "parse_symbol_set"]
