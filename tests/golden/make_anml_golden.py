"""Generate tests/golden/anml_cases.json.gz by running the reference's ANML loader.

    python tests/golden/make_anml_golden.py --reference /root/reference

The documents are written here (hand-written ones covering each feature of the
homogeneous-STE subset and each refusal, plus synthetic pattern automata from
``workloads.anml_patterns``); everything recorded about them comes from the reference
package gpufsm 0.1.0 imported from the given checkout: ``gpufsm.io.anml.load_anml``'s
CSR arrays (or its exception) and ``gpufsm.reference.simulate``'s verdicts on sample
inputs. For the synthetic automata the CSR is recorded as a digest of its rows sorted
by (symbol, target).
"""

from __future__ import annotations

import argparse
import gzip
import hashlib
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

STE = '<state-transition-element id="{id}" symbol-set="{s}"{start}>{body}</state-transition-element>'


def ste(id_, s, start=None, to=(), report=False):
    body = "".join(f'<activate-on-match element="{t}"/>' for t in to)
    if report:
        body += '<report-on-match reportcode="7"/>'
    st = f' start="{start}"' if start else ""
    return STE.format(id=id_, s=s, start=st, body=body)


def doc(*stes, root="anml", ns=""):
    inner = "".join(stes)
    if root == "anml":
        return f'<anml{ns}><automata-network id="g">{inner}</automata-network></anml>'
    return f'<automata-network id="g"{ns}>{inner}</automata-network>'


CASES = {
    # accepted documents
    "sod-chain": (doc(ste("a", "x", "start-of-data", ["b"]), ste("b", "y", report=True)),
                  [b"", b"x", b"xy", b"xyz", b"axy", b"yx"]),
    "all-input-class": (doc(ste("d", "[0-9]", "all-input", report=True)),
                        [b"", b"abc", b"ab7", b"7", b"a\x00z9"]),
    "hex-forms": (doc(ste("h", "[0x41\\x42C]", "all-input", ["t"]), ste("t", "\\x44", report=True)),
                  [b"AD", b"BD", b"CD", b"DD", b"xxCDxx", b"C"]),
    "ranges-and-negation": (doc(ste("r", "[a-cx-z]", "all-input", ["n"]),
                                ste("n", "[^0x2e]", to=["e"]),
                                ste("e", "[\\x30-\\x39]", report=True)),
                            [b"a.1", b"aq1", b"zz9", b"b..", b"dq1", b"c\xff0"]),
    "negated-empty-is-any": (doc(ste("s", "q", "start-of-data", ["all"]),
                                 ste("all", "[^]", report=True)),
                             [b"q", b"q\x00", b"qz", b"zq"]),
    "wildcard-star": (doc(ste("s", "*", "start-of-data", ["t"]), ste("t", "!", report=True)),
                      [b"!", b"a!", b"!!", b"ab!"]),
    "port-target": (doc(ste("s", "a", "start-of-data", ["t:in"]), ste("t", "b", report=True)),
                    [b"ab", b"a", b"b", b"aab"]),
    "self-loop": (doc(ste("s", "a", "all-input", ["m"]), ste("m", "[b-d]", to=["m", "e"]),
                      ste("e", "e", report=True)),
                  [b"abe", b"abcdcde", b"ae", b"xxabbbbe", b"abf", b"a"]),
    "branch-and-both-starts": (doc(ste("s", "k", "start-of-data", ["u", "v"]),
                                   ste("g", "k", "all-input", ["v"]),
                                   ste("u", "1", report=True), ste("v", "2", to=["w"]),
                                   ste("w", "3", report=True)),
                               [b"k1", b"k23", b"xk23", b"xk1", b"kk23"]),
    "report-on-start": (doc(ste("s", "[ab]", "all-input", report=True)),
                        [b"", b"a", b"zzb", b"zz"]),
    "namespace-and-description": (
        '<anml xmlns="http://www.micron.com/anml"><description>d</description>'
        '<automata-network id="n">' + ste("s", "z", "all-input", report=True) +
        '</automata-network></anml>', [b"z", b"az", b"aa"]),
    "bare-network-root": (doc(ste("s", "0x7a", "start-of-data", report=True), root="net"),
                          [b"z", b"az"]),
    "unused-wide-char": (doc(ste("s", "a", "all-input", report=True),
                             ste("w", "[€]")), [b"a", b"b"]),
    # refused documents
    "err-gate": (doc(ste("s", "a", "all-input")) .replace(
        "</automata-network>", '<or id="g0"><report-on-match/></or></automata-network>'), None),
    "err-counter": (doc(ste("s", "a", "all-input")).replace(
        "</automata-network>", '<counter id="c" target="3"/></automata-network>'), None),
    "err-missing-id": ('<anml><automata-network><state-transition-element symbol-set="a" '
                       'start="all-input"/></automata-network></anml>', None),
    "err-duplicate-id": (doc(ste("s", "a", "all-input"), ste("s", "b")), None),
    "err-unknown-target": (doc(ste("s", "a", "all-input", ["nowhere"])), None),
    "err-empty-class": (doc(ste("s", "[]", "all-input")), None),
    "err-inverted-range": (doc(ste("s", "[z-a]", "all-input")), None),
    "err-short-hex": (doc(ste("s", "[0x4]", "all-input")), None),
    "err-two-char-atom": (doc(ste("s", "ab", "all-input")), None),
    "err-no-ste": ('<anml><automata-network id="e"></automata-network></anml>', None),
    "err-wide-char-edge": (doc(ste("s", "[€]", "all-input", report=True)), None),
}


def row_digest(a) -> str:
    """SHA-256 of the CSR with each row sorted by (symbol, target)."""
    rp = np.asarray(a.sym_row_ptr, np.int64)
    sy = np.asarray(a.sym_symbols, np.int64)
    tg = np.asarray(a.sym_targets, np.int64)
    src = np.repeat(np.arange(a.num_states), np.diff(rp))
    order = np.lexsort((tg, sy, src))
    h = hashlib.sha256()
    for arr in (np.asarray([a.num_states, a.start_state], np.int64), rp, sy[order], tg[order],
                np.asarray(a.accept, np.int64), np.asarray(a.eps_row_ptr, np.int64),
                np.asarray(a.eps_targets, np.int64)):
        h.update(np.ascontiguousarray(arr).tobytes())
    return h.hexdigest()


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    sys.path.insert(0, str(Path(args.reference) / "src"))
    from gpufsm.io.anml import load_anml
    from gpufsm.reference import simulate

    from abstraction_regret_gb300 import workloads as W
    from tests.golden.make_golden import nfa_json

    out = {"source": "gpufsm 0.1.0 gpufsm.io.anml.load_anml + gpufsm.reference.simulate",
           "cases": [], "synthetic": []}
    with tempfile.TemporaryDirectory() as tmp:
        path = Path(tmp) / "case.anml"
        for name, (text, inputs) in CASES.items():
            path.write_text(text, encoding="utf-8")
            case = {"id": name, "anml": text}
            try:
                nfa = load_anml(path)
            except Exception as exc:  # noqa: BLE001 - recorded as the expected refusal
                case["error"] = type(exc).__name__
                case["message"] = str(exc).replace(str(path), "<file>")
            else:
                case["nfa"] = nfa_json(nfa)
                case["digest"] = row_digest(nfa)
                case["inputs_hex"] = [x.hex() for x in inputs]
                case["verdicts"] = [list(simulate(nfa, x)) for x in inputs]
            out["cases"].append(case)
        for n_pat, seed, n_in, length in ((20, 1, 12, 400), (60, 2, 8, 300), (150, 3, 6, 200)):
            text = W.anml_patterns(n_pat, seed=seed)
            path.write_text(text)
            nfa = load_anml(path)
            inputs = W.anml_inputs(nfa, n_in, length, seed=seed + 100)
            out["synthetic"].append({"patterns": n_pat, "seed": seed, "digest": row_digest(nfa),
                                     "num_states": int(nfa.num_states),
                                     "num_edges": int(nfa.sym_targets.size),
                                     "inputs_hex": [x.hex() for x in inputs],
                                     "verdicts": [list(simulate(nfa, x)) for x in inputs]})
    raw = json.dumps(out, separators=(",", ":")).encode()
    (HERE / "anml_cases.json.gz").write_bytes(gzip.compress(raw, mtime=0))
    print(f"wrote {len(out['cases'])} documents and {len(out['synthetic'])} synthetic automata")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
