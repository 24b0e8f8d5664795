// Chunked walks of long DFA inputs: one input's chunks run in parallel, with exact
// verdicts (dfa_chunks.cu, tasks GBFSM_TASK_DFA_CHUNK and GBFSM_TASK_DFA_FIXUP).
//
// A DFA walk is one dependent table lookup per byte, so a long input is a long chain. Cut
// it into chunks. Chunk 0 walks exactly from the start state. A later chunk starting at
// position b does not know its start state, so it walks the set of ALL states: after each
// byte the set becomes the distinct successors of its members, and for a random DFA it
// shrinks like 2n/t; once it holds a single state (position p, the collapse), every start
// state leads there, so from p on the chunk's walk is the true walk, whatever came before.
// The chunk records p, its first accept after p, its state at its end and -- continuing
// that exact walk past its end into the next chunk -- the first accept of this overlap.
// Positions count the bytes consumed from the start of the input.
//
// The overlap is as long as the next chunk needs: a chunk publishes its collapse position
// in its record as soon as it has it, and the previous chunk's overlap walk, polling that
// word, stops once it has passed it (at once when the next chunk stopped early), and in
// any case at the next chunk's end or after `overlap` bytes (the automaton's
// dfa_overlap). When the next chunk never collapses, the overlap covers it whole and
// records the true state at its end, so the fix-up need not walk it. A stale word (the
// next chunk's task not started yet) can only cut an overlap short; the fix-up checks
// every link against the final records, so verdicts never depend on the timing.
//
// Fix-up (one lane per input, serial over the input's chunks): the true state at each
// chunk start is known from the previous chunk's record. Chunk k is linked when chunk
// k-1's walk is exact (it is chunk 0 or it collapsed) and its overlap reached p_k: the
// overlap is then the true walk over (b_k, p_k], so its first accept (if any) is the
// input's next accept, and otherwise chunk k's record is exact from p_k on. A chunk that
// is not linked has its gap (b_k, p_k], or the whole chunk if it never collapsed, walked
// serially from the known true state. Verdicts are exactly those of a serial walk
// (src/gpufsm/reference.py:68-81).
//
// Set walk of a chunk, by one warp: while the set has more than 32 members it is a bitmap
// of the states in shared memory (each lane scans its words, looks up the successors of
// their members and sets their bits with shared atomics); then one member per lane,
// duplicates removed with __match_any_sync, until one lane is left.
//
// Early stop: an accept found by chunk 0's walk, by a collapsed chunk's walk or by its
// overlap is in the input's true walk, so the input's verdict lies at or before it. The
// chunk lowers the input's latch to its index (the overlap: to the next chunk's index),
// and every chunk of a higher index, polling the latch, stops (p = -2). The fix-up never
// reads a stopped chunk: it returns at the latching chunk or earlier. It would walk one
// whole, as a chunk that never collapsed.
#pragma once

#include "common.cuh"
#include "dfa_device.cuh"
#include "nfa_device.cuh"

namespace gbfsm {

// Record of a DFA chunk: the first 32 bytes of its GBFSM_CHUNK_RECORD_BYTES record slot.
struct DfaChunkRecord {
    int32_t p;        // collapse position (0 for an input's first chunk), -1: none,
                      // -2: stopped, kPending while the set walk runs
    int32_t acc;      // first accept in (p, end], -1: none (first chunk: in [0, end])
    int32_t end_state;
    int32_t ov_len;   // bytes walked past the chunk end (exact when p >= 0)
    int32_t ov_acc;   // first accept in the overlap, -1: none
    int32_t ov_state; // the state at the end of the overlap (when ov_acc < 0)
    int32_t pad[2];
};
static_assert(sizeof(DfaChunkRecord) == 32 && sizeof(DfaChunkRecord) <= GBFSM_CHUNK_RECORD_BYTES,
              "DFA chunk record slot");

__device__ __forceinline__ DfaChunkRecord *dfa_record(void *records, int32_t chunk) {
    return reinterpret_cast<DfaChunkRecord *>(static_cast<uint8_t *>(records) +
                                              (size_t)chunk * GBFSM_CHUNK_RECORD_BYTES);
}

__device__ __forceinline__ const DfaChunkRecord *dfa_record(const void *records,
                                                            int32_t chunk) {
    return reinterpret_cast<const DfaChunkRecord *>(static_cast<const uint8_t *>(records) +
                                                    (size_t)chunk * GBFSM_CHUNK_RECORD_BYTES);
}

template <typename Entry>
__device__ __forceinline__ uint32_t dfa_entry(const Entry *T, uint32_t s, uint32_t c) {
    return __ldg(T + (typename RowIndex<Entry>::type)s * (uint32_t)kAlphabet + c);
}

constexpr int kLatchPollBytes = 256;  // serial steps between two polls of the latch
constexpr int kLatchPollSets = 16;    // light bitmap steps between two polls
constexpr int kPollEveryStep = 512;   // set size above which every bitmap step polls
constexpr int32_t kPending = -3;      // a record's p while its chunk's set walk runs

// True when a chunk of index below `index` has latched the input (latch may be NULL).
__device__ __forceinline__ bool latched_below(const int32_t *latch, int32_t index) {
    return latch && __ldcv(latch) < index;
}

// The same for the whole warp (latch and index warp-uniform): lane 0 reads the latch and
// every lane gets its answer, so the warp leaves a collective walk together.
__device__ __forceinline__ bool warp_latched_below(const int32_t *latch, int32_t index) {
    if (!latch) return false;
    int32_t v = lane_id() == 0 ? __ldcv(latch) : 0;
    v = __shfl_sync(GBFSM_FULL_MASK, v, 0);
    return v < index;
}

// One lane: consume bytes [a, b) of `base` from state s. Returns the state at b, or at the
// first accepting position q in (a, b], which goes to `acc` (-1 when none). With a latch,
// polls it every kLatchPollBytes bytes and returns early with `stopped` set once a chunk
// below `index` has latched.
template <typename Entry>
__device__ uint32_t dfa_span(const Entry *T, uint32_t s, const uint8_t *base, int64_t a,
                             int64_t b, int64_t &acc, const int32_t *latch = nullptr,
                             int32_t index = 0, bool *stopped = nullptr) {
    constexpr uint32_t ACC = EntryTraits<Entry>::kAccept;
    acc = -1;
    if (b <= a) return s;
    ByteStream bs;
    bs.init(base + a, b - a);
    for (int64_t q0 = a; q0 < b; q0 += kLatchPollBytes) {
        if (latched_below(latch, index)) {
            *stopped = true;
            return s;
        }
        const int64_t q1 = min(b, q0 + (int64_t)kLatchPollBytes);
        for (int64_t q = q0; q < q1; ++q) {
            const uint32_t e = dfa_entry(T, s, bs.next());
            s = e & ~ACC;
            if (e & ACC) {
                acc = q + 1;
                return s;
            }
        }
    }
    return s;
}

__device__ __forceinline__ int32_t warp_sum_i32(int32_t v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(GBFSM_FULL_MASK, v, d);
    return v;
}

// The whole warp: walk the set of all n states from position b over bytes [b, e) until it
// holds one state. Returns the collapse position (the state in `sigma`, every lane), -1
// when the set still has two or more members at e, or -2 when a chunk below `index` has
// latched the input (latch may be NULL). bm0 / bm1: shared bitmaps of at least
// ceil(n / 32) words; list: 32 shared words.
template <typename Entry>
__device__ int64_t dfa_collapse(const Entry *T, uint32_t n, const uint8_t *base, int64_t b,
                                int64_t e, uint32_t *bm0, uint32_t *bm1, uint32_t *list,
                                uint32_t &sigma, const int32_t *latch, int32_t index) {
    constexpr uint32_t ACC = EntryTraits<Entry>::kAccept;
    const uint32_t lane = lane_id();
    const uint32_t nw = (n + 31u) >> 5;
    if (e <= b) return -1;
    // first byte: the successors of every state
    for (uint32_t w = lane; w < nw; w += 32) bm1[w] = 0u;
    __syncwarp();
    {
        const uint32_t c = __ldg(base + b);
        for (uint32_t s = lane; s < n; s += 32) {
            const uint32_t t = dfa_entry(T, s, c) & ~ACC;
            atomicOr(bm1 + (t >> 5), 1u << (t & 31u));
        }
    }
    __syncwarp();
    int64_t pos = b + 1;
    uint32_t *cur = bm1, *nxt = bm0;
    int32_t count = 0;
    for (uint32_t w = lane; w < nw; w += 32) count += __popc(cur[w]);
    count = warp_sum_i32(count);
    // many members: bitmaps
    while (count > 32 && pos < e) {
        if ((count > kPollEveryStep || (pos - b) % kLatchPollSets == 0) &&
            warp_latched_below(latch, index))
            return -2;
        const uint32_t c = __ldg(base + pos);
        for (uint32_t w = lane; w < nw; w += 32) nxt[w] = 0u;
        __syncwarp();
        for (uint32_t w = lane; w < nw; w += 32) {
            uint32_t bits = cur[w];
            while (bits) {  // up to four lookups in flight per lane
                uint32_t s4[4];
                int k = 0;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (bits) {
                        s4[u] = (w << 5) + (uint32_t)(__ffs(bits) - 1);
                        bits &= bits - 1u;
                        k = u + 1;
                    }
                }
                uint32_t t4[4];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (u < k) t4[u] = dfa_entry(T, s4[u], c) & ~ACC;
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (u < k) atomicOr(nxt + (t4[u] >> 5), 1u << (t4[u] & 31u));
            }
        }
        __syncwarp();
        count = 0;
        for (uint32_t w = lane; w < nw; w += 32) count += __popc(nxt[w]);
        count = warp_sum_i32(count);
        uint32_t *tmp = cur;
        cur = nxt;
        nxt = tmp;
        ++pos;
    }
    if (count > 32) return -1;
    // at most 32 members: one per lane
    int32_t mine = 0;
    for (uint32_t w = lane; w < nw; w += 32) mine += __popc(cur[w]);
    int32_t before = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int32_t y = __shfl_up_sync(GBFSM_FULL_MASK, before, d);
        if ((int)lane >= d) before += y;
    }
    before -= mine;
    for (uint32_t w = lane; w < nw; w += 32) {
        uint32_t bits = cur[w];
        while (bits) {
            list[before++] = (w << 5) + (uint32_t)(__ffs(bits) - 1);
            bits &= bits - 1u;
        }
    }
    __syncwarp();
    bool active = (int32_t)lane < count;
    uint32_t member = active ? list[lane] : 0xffffffffu;
    __syncwarp();
    uint32_t alive = __ballot_sync(GBFSM_FULL_MASK, active);
    while (__popc(alive) > 1 && pos < e) {
        if ((pos - b) % kLatchPollBytes == 0 && warp_latched_below(latch, index)) return -2;
        const uint32_t c = __ldg(base + pos);
        const uint32_t t = active ? (dfa_entry(T, member, c) & ~ACC) : 0xffffffffu;
        const uint32_t same = __match_any_sync(GBFSM_FULL_MASK, t);
        active = active && (uint32_t)(__ffs(same) - 1) == lane;
        member = t;
        alive = __ballot_sync(GBFSM_FULL_MASK, active);
        ++pos;
    }
    if (__popc(alive) != 1) return -1;
    sigma = __shfl_sync(GBFSM_FULL_MASK, member, __ffs(alive) - 1);
    return pos;
}

// One lane: the overlap walk of a chunk ending at e, from its exact state s, into the next
// chunk (record `next`, or NULL when e is the input's end): until the next chunk's
// published collapse position has been passed, or it is known that the next chunk
// stopped, or `cap` (at most the next chunk's end) is reached. Returns the overlap's
// length; its first accept goes to ov_acc (-1 when none), the state at its end to
// `s_end`, and `stopped` is set when a chunk below `index` latched the input meanwhile.
template <typename Entry>
__device__ int64_t dfa_overlap_walk(const Entry *T, uint32_t s, const uint8_t *base,
                                    int64_t e, int64_t cap, const DfaChunkRecord *next,
                                    const int32_t *latch, int32_t index, int64_t &ov_acc,
                                    uint32_t &s_end, bool &stopped) {
    constexpr uint32_t ACC = EntryTraits<Entry>::kAccept;
    ov_acc = -1;
    s_end = s;
    if (cap <= e || !next) return 0;
    ByteStream bs;
    bs.init(base + e, cap - e);
    int64_t q = e, target = cap;
    while (q < target) {
        if (latched_below(latch, index)) {
            stopped = true;
            break;
        }
        const int32_t np = __ldcv(&next->p);
        if (np >= 0) target = min(target, max((int64_t)np, q));
        else if (np == -2) target = q;  // -1 (never collapsed): on to the cap
        const int64_t q1 = min(target, q + (int64_t)kLatchPollBytes);
        for (; q < q1; ++q) {
            const uint32_t x = dfa_entry(T, s, bs.next());
            s = x & ~ACC;
            if (x & ACC) {
                ov_acc = q + 1;
                s_end = s;
                return ov_acc - e;
            }
        }
    }
    s_end = s;
    return q - e;
}

// A DFA_CHUNK task: chunk `index` of an input spanning positions [b, e) of `base` (the
// input's first byte), `len` bytes in all; the record goes to rec (the next chunk's, when
// e < len, is rec_next, and that chunk ends at e_next). latch: the input's latch word, or
// NULL.
template <typename Entry>
__device__ void dfa_chunk(const gbfsm_dfa_dev &d, int32_t overlap, const uint8_t *base,
                          int64_t len, int64_t b, int64_t e, int64_t e_next, int index,
                          uint32_t *bm0, uint32_t *bm1, uint32_t *list, DfaChunkRecord *rec,
                          const DfaChunkRecord *rec_next, int32_t *latch) {
    const Entry *T = static_cast<const Entry *>(d.table);
    const uint32_t lane = lane_id();
    int64_t p;
    uint32_t s = 0;
    int64_t acc = -1;
    if (index == 0) {
        p = 0;
        s = (uint32_t)d.start_state;
        if ((__ldg(d.accept_bits + (s >> 5)) >> (s & 31u)) & 1u) acc = 0;
    } else {
        if (lane == 0) __stcg(&rec->p, kPending);
        p = dfa_collapse<Entry>(T, (uint32_t)d.num_states, base, b, e, bm0, bm1, list, s,
                                latch, index);
        if (lane == 0) __stcg(&rec->p, (int32_t)p);  // for the previous chunk's overlap
    }
    if (lane == 0) {
        int64_t ov_len = 0, ov_acc = -1;
        uint32_t ov_state = 0;
        bool stopped = false;
        if (p >= 0 && acc < 0) {
            s = dfa_span<Entry>(T, s, base, p, e, acc, latch, index, &stopped);
            if (acc < 0 && !stopped) {
                const int64_t cap =
                    min(min(e + (int64_t)(overlap > 0 ? overlap : 0), e_next), len);
                ov_len = dfa_overlap_walk<Entry>(T, s, base, e, cap, e < len ? rec_next : nullptr,
                                                 latch, index, ov_acc, ov_state, stopped);
                if (latch && ov_acc >= 0) atomicMin(latch, index + 1);
            }
        }
        if (latch && acc >= 0) atomicMin(latch, index);
        if (stopped) {  // the verdict lies in an earlier chunk: this record is never read
            p = -2;
            acc = ov_acc = -1;
            ov_len = 0;
        }
        int4 *w = reinterpret_cast<int4 *>(rec);
        w[0] = make_int4((int32_t)p, (int32_t)acc, (int32_t)s, (int32_t)ov_len);
        w[1] = make_int4((int32_t)ov_acc, (int32_t)ov_state, 0, 0);
    }
    __syncwarp();
}

// A DFA_FIXUP task (lane 0): the verdict of an input from its chunks' records (chunks[first
// .. first + count), positions relative to the input's start `off`).
template <typename Entry>
__device__ Verdict dfa_fixup(const gbfsm_dfa_dev &d, const uint8_t *base, int64_t len,
                             const gbfsm_chunk *chunks, int64_t off, const void *records,
                             int32_t first, int32_t count) {
    const Entry *T = static_cast<const Entry *>(d.table);
    const DfaChunkRecord r0 = *dfa_record(records, first);
    if (r0.acc >= 0) return Verdict{1, r0.acc, r0.acc};
    uint32_t s = (uint32_t)r0.end_state;
    bool prev_ok = true;  // the previous chunk's walk and overlap are exact
    int64_t prev_ov_len = r0.ov_len, prev_ov_acc = r0.ov_acc;
    uint32_t prev_ov_state = (uint32_t)r0.ov_state;
    for (int32_t k = 1; k < count; ++k) {
        if (prev_ok && prev_ov_acc >= 0) return Verdict{1, (int32_t)prev_ov_acc, prev_ov_acc};
        const gbfsm_chunk ch = chunks[first + k];
        const int64_t b = ch.begin - off, e = ch.end - off;
        const DfaChunkRecord r = *dfa_record(records, first + k);
        int64_t acc;
        if (r.p >= 0) {
            if (!(prev_ok && r.p - b <= prev_ov_len)) {
                dfa_span<Entry>(T, s, base, b, r.p, acc);  // the gap before the collapse
                if (acc >= 0) return Verdict{1, (int32_t)acc, acc};
            }
            if (r.acc >= 0) return Verdict{1, r.acc, r.acc};
            s = (uint32_t)r.end_state;
            prev_ok = true;
            prev_ov_len = r.ov_len;
            prev_ov_acc = r.ov_acc;
            prev_ov_state = (uint32_t)r.ov_state;
        } else {
            if (prev_ok && prev_ov_len == e - b) {
                s = prev_ov_state;  // never collapsed, but the previous overlap covered it
            } else {
                s = dfa_span<Entry>(T, s, base, b, e, acc);  // never collapsed: walk it
                if (acc >= 0) return Verdict{1, (int32_t)acc, acc};
            }
            prev_ok = false;
        }
    }
    return Verdict{0, 0, len};
}

}  // namespace gbfsm
