"""Memory cost model of this engine's techniques: the autotuner's priors.

The reference models time per input symbol as modelled memory traffic over an effective
bandwidth plus a compute term, the traffic following from where a technique keeps its
active-set working set (src/gpufsm/costmodel.py:62-142: ``Residency``, ``_RESIDENCY``,
``working_set_traffic_per_symbol``, ``csr_traffic_per_symbol``, ``traffic_per_symbol``;
two constants fitted by least squares, :171-213). The same model is stated here for this
engine's kernels, with two changes that follow from them:

* every kernel is work-efficient -- it reads only the active states' rows -- so the CSR
  traffic per symbol is that of the active states (8 bytes of row range per active state
  and 8 per scanned edge, the algorithmic bytes of the measurement), unless the rows are
  staged in shared memory (then 0 global bytes per symbol, as the reference counts
  ``multistream_shared``);
* the second term is not the reference's n^2 closure scan but the serial chain: one
  input is one chain of dependent steps, so a launch cannot finish before its longest
  input has been walked, ``max_len * step_s``.

``traffic_per_symbol`` feeds ``autotune.rule_plan`` (thread-per-input bitmaps only while
their sets stay in shared memory) and ``predict_plain_ms`` / ``predict_engine_ms`` feed
``autotune.prefer_engine`` (plain launch or chunked engine for a batch).
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from enum import Enum

import numpy as np

from . import native

WORD_BYTES = 8
WS_TOUCHES = 4  # working-set touches per symbol (clear, scatter, swap, accept test)
SHARED_BUDGET = 227 * 1024 - 1024  # opt-in shared memory per CTA less a reserve


class Residency(str, Enum):
    """Where a technique keeps the active-set working set."""

    REGISTER = "register"        # a few states in registers (lane chunks)
    SHARED = "shared"            # words or member lists in shared memory
    GLOBAL_WORD = "global_word"  # packed 64-bit words in global memory


# Every registered NFA technique of this package, and where its set lives when it fits
# shared memory (``residency`` decides from the automaton and the plan).
TECHNIQUE_KIND: dict[str, int] = {
    "bitmap": native.TECH_BITMAP, "dense": native.TECH_BITMAP,
    "bitpacked": native.TECH_BITMAP, "multistream": native.TECH_BITMAP,
    "multistream_shared": native.TECH_BITMAP, "multistream_async": native.TECH_BITMAP,
    "worklist": native.TECH_BITMAP, "warp": native.TECH_WARP,
    "worklist_global": native.TECH_WARP, "worklist_warp": native.TECH_WARP,
    "worklist_shared": native.TECH_WARP, "compact": native.TECH_COMPACT,
    "worklist_compact": native.TECH_COMPACT, "auto": native.TECH_COMPACT,
    "persistent": -1,
}


def words(num_states: int) -> int:
    return -(-int(num_states) // 64)


def residency(f, technique: int, threads: int = 128) -> Residency:
    """Working-set residency of a plain launch (the rule of make_warp_plan /
    make_bitmap_plan): a thread-per-input bitmap keeps 4 words of sets per state-word
    per thread in shared memory while ``threads`` of them fit; a warp keeps its dense
    bitmaps there while 3 words per state-word fit for its CTA; -1: the lane engine."""
    w = words(f.num_states)
    if technique < 0:
        return Residency.REGISTER
    if technique == native.TECH_BITMAP:
        return Residency.SHARED if threads * 4 * w * WORD_BYTES <= SHARED_BUDGET \
            else Residency.GLOBAL_WORD
    warps = max(1, threads // 32)
    return Residency.SHARED if warps * 4 * w * WORD_BYTES + warps * 32 * 32 <= SHARED_BUDGET \
        else Residency.GLOBAL_WORD


def working_set_traffic_per_symbol(f, res: Residency) -> int:
    """Global bytes per symbol for the working set (0 when it stays on chip)."""
    if res is not Residency.GLOBAL_WORD:
        return 0
    return WS_TOUCHES * words(f.num_states) * WORD_BYTES


def csr_traffic_per_symbol(f, staged: bool = False, active: float = 1.0) -> float:
    """Row and edge bytes per symbol of a work-efficient step over ``active`` states
    (0 when the rows are staged in shared memory)."""
    if staged:
        return 0.0
    degree = f.num_edges / max(1, f.num_states)
    return active * (8.0 + 8.0 * degree)


def traffic_per_symbol(f, technique: str, threads: int = 128, staged: bool = False,
                       active: float = 1.0) -> float:
    """Modelled global bytes per symbol of a registered technique."""
    try:
        kind = TECHNIQUE_KIND[technique]
    except KeyError:
        raise KeyError(f"no working-set residency declared for {technique!r}") from None
    res = residency(f, kind, threads)
    return working_set_traffic_per_symbol(f, res) + csr_traffic_per_symbol(f, staged, active)


@dataclass(frozen=True)
class CostModel:
    """The effective bandwidth of modelled traffic and the time of one dependent step of
    a chain (one symbol of one input) -- the two constants ``fit`` estimates -- plus the
    engine's per-lane step times, launch overhead and lane count (measured on GB300:
    the c3 lane launch, 1728-byte chunks in 1.83 ms; one warp per input, 575 ms for a
    1 MiB input)."""

    eff_bandwidth_bytes_per_s: float = 4.0e12
    step_s: float = 5.5e-7            # plain launch: one warp's step on one input
    lane_step_s: float = 1.05e-6      # lane engine: one lane's step, every lane busy
    lane_step_idle_s: float = 4.0e-7  # ... with few lanes busy (a dependent L2 trip)
    engine_overhead_s: float = 6.0e-5  # planning + four launches
    lanes: int = 152 * 1024           # resident lanes of the lane launch

    def time_per_symbol_s(self, traffic: float) -> float:
        return traffic / self.eff_bandwidth_bytes_per_s

    def predict_plain_ms(self, f, lengths, technique: str = "compact") -> float:
        """One plain launch over the batch: the longest chain, or the traffic."""
        lengths = np.asarray(lengths, dtype=np.int64)
        if lengths.size == 0:
            return 0.0
        traffic = traffic_per_symbol(f, technique) * float(lengths.sum())
        return 1e3 * max(float(lengths.max()) * self.step_s, self.time_per_symbol_s(traffic))

    def predict_engine_ms(self, f, lengths) -> float:
        """The chunked engine: its overhead, then one wave of lane chunks (the smallest
        size, a multiple of 64 bytes of at least 256, that fills the lanes at most once),
        each lane's step slower the more lanes are busy."""
        lengths = np.asarray(lengths, dtype=np.int64)
        if lengths.size == 0:
            return 0.0
        total = float(lengths.sum())
        chunk = max(256, int(math.ceil(total / self.lanes / 64.0)) * 64)
        chunks = float(np.maximum(1, -(-lengths // chunk)).sum())
        busy = min(1.0, chunks / self.lanes)
        step = self.lane_step_idle_s + (self.lane_step_s - self.lane_step_idle_s) * busy
        chain = min(int(lengths.max()), chunk) * step
        traffic = traffic_per_symbol(f, "persistent") * total
        return 1e3 * (self.engine_overhead_s + max(chain, self.time_per_symbol_s(traffic)))


def fit(traffic, chains, seconds) -> CostModel:
    """Least-squares fit of ``seconds = traffic / bandwidth + chain * step_s`` over
    measured launches (the reference's two-constant fit, costmodel.py:171-213). A
    non-positive traffic coefficient means the launches were chain-bound: the bandwidth
    is then infinite and the step time is refitted alone."""
    a = np.stack([np.asarray(traffic, float), np.asarray(chains, float)], axis=1)
    b = np.asarray(seconds, float)
    if a.shape[0] < 2:
        raise ValueError("calibration needs >= 2 points")
    coef, *_ = np.linalg.lstsq(a, b, rcond=None)
    if coef[0] <= 0:
        step, *_ = np.linalg.lstsq(a[:, 1:2], b, rcond=None)
        return CostModel(eff_bandwidth_bytes_per_s=math.inf, step_s=max(float(step[0]), 0.0))
    return CostModel(eff_bandwidth_bytes_per_s=1.0 / float(coef[0]),
                     step_s=max(float(coef[1]), 0.0))


DEFAULT = CostModel()
