// Speculative chunk-parallel NFA simulation: the chunk record, the warp and lane chunk
// runners and the exact fix-up (shared by persistent.cu and lanes.cu).
//
// An input is cut into chunks. Its first chunk runs exactly from the start configuration.
// Every later chunk starting at byte b runs from a superset of the true active set at b:
// the targets of every edge labelled x[b-2] (or ANY), stepped over x[b-1] (for automata
// without epsilon edges this two-byte superset is tabulated, pair_lanes). Because
// simulation preserves set inclusion, the speculative set contains the true set at every
// later position of the chunk, so equal sizes mean equal sets. The chunk records its set
// sizes after 1, 2, 4, ..., 32 bytes, the first accept strictly after each of those
// checkpoints, where it died, and its final set; it then continues its run up to 32 bytes
// into the next chunk (the overlap) and records that run's sizes and first event.
//
// Fix-up. Chunk k is linked to chunk k-1 when, at some checkpoint and before any event of
// the overlap run, the overlap run of chunk k-1 has the size chunk k recorded. If chunk
// k-1's run is exact, so is its overlap run, which then equals chunk k's speculative run
// from that checkpoint on: chunk k's record is exact from there. The first chunk is
// exact, so along a chain of links every record is exact, and an input's verdict is that
// of the first chunk that decides (an accept or a death, in its overlap prefix or its
// record). The fix-up is therefore a warp-parallel scan over the chunks; only at a chunk
// that cannot be linked does it fall back to re-running chunks serially from the last
// exact recorded set, checking sizes at the checkpoints the same way. Verdicts are
// exactly those of a serial run (src/gpufsm/reference.py:36-65).
#pragma once

#include "common.cuh"
#include "nfa_device.cuh"

namespace gbfsm {

constexpr int kCheckpoints = 6;  // set sizes after 1, 2, 4, 8, 16, 32 bytes of a chunk
constexpr int kOverlap = 1 << (kCheckpoints - 1);  // bytes a run continues into the next chunk
constexpr int kEndCap = 8;       // states of a chunk's final set kept in its record
constexpr int kLaneSlots = 4;    // states (and matching edges per byte) a lane handles

// Outcome of one chunk (GBFSM_CHUNK_RECORD_BYTES bytes). Positions are byte counts from
// the start of the chunk's input. acc_after[c]: first accepting position strictly after
// checkpoint c (-1: none before the run stopped); dead_at: position at which the run's
// set became empty (-1: never). For an input's first chunk (exact) acc_after[0] / dead_at
// are the input's own first accept / death. end_recs: the set at the chunk end as state
// records, when the run got there with at most kEndCap members (end_count, else -1).
// The overlap run (from the end set into the next chunk of the same input): ov_len bytes
// stepped, ov_event = +j / -j when it accepted / died at its j-th byte (0: neither),
// ov_counts[c] its size after 2^c bytes. begin / end: the bounds the chunk actually ran
// over (chunk_bounds), input-relative.
struct ChunkRecord {
    int32_t counts[kCheckpoints];
    int32_t acc_after[kCheckpoints];
    int32_t dead_at;
    int32_t end_count;
    int32_t ov_len;
    int32_t ov_event;
    int32_t ov_counts[kCheckpoints];
    int64_t begin;
    int64_t end;
    int32_t pad[6];
    uint4 end_recs[kEndCap];
};
static_assert(sizeof(ChunkRecord) == GBFSM_CHUNK_RECORD_BYTES, "chunk record layout");

// Device pointers of the chunk machinery, passed by value to the kernels.
struct ChunkIO {
    const gbfsm_chunk *chunks;
    ChunkRecord *records;
    gbfsm_task *overflow_tasks;
    int32_t *overflow_count;
    const int32_t *task_count;
    int32_t n_chunks;
    const int32_t *aut_ids;  // per-input automaton (NULL: all 0)
};

__device__ __forceinline__ uint32_t byte_at(const uint8_t *p) { return __ldg(p); }

constexpr int kShiftWindow = 32;    // bytes a chunk start may move forward
constexpr uint32_t kShiftSet = 4u;  // a two-byte superset this small ends the search

// Start of a later chunk whose nominal bounds are [nb, ne) (input-relative). For an
// automaton with a two-byte superset table the start moves forward to the first position
// of its first min(kShiftWindow, (ne - nb) / 4) bytes whose superset has at most kShiftSet
// states (the smallest superset when none does): a smaller starting superset converges
// sooner and rarely outgrows a lane. The rule is a pure function of the chunk table and
// the bytes, so the chunk and its predecessor (whose end it is) agree without exchange.
__device__ __forceinline__ int64_t chunk_start(const gbfsm_nfa_dev &A, const uint8_t *base,
                                               int64_t nb, int64_t ne) {
    if (A.pair_row == nullptr) return nb;
    const int w = (int)min((int64_t)kShiftWindow, max((int64_t)1, (ne - nb) / 4));
    uint32_t prev = byte_at(base + nb - 2), cur = byte_at(base + nb - 1);
    int best = 0;
    uint32_t best_size = 0xffffffffu;
    for (int t = 0; t < w; ++t) {
        const uint32_t key = prev * 256u + cur;
        const uint32_t size = __ldg(A.pair_row + key + 1) - __ldg(A.pair_row + key);
        if (size <= kShiftSet) {
            best = t;
            break;
        }
        if (size < best_size) {
            best_size = size;
            best = t;
        }
        prev = cur;
        cur = byte_at(base + nb + t);
    }
    return nb + best;
}

// Bounds a chunk runs over (input-relative): its start (moved by chunk_start unless it
// is the input's first chunk), its end (the next chunk's start, or the input end), and
// the end of its overlap run: up to kOverlap bytes into the next chunk, never past that
// chunk's nominal end (which its actual end cannot precede).
struct Bounds {
    int64_t b, e, ov_end;
};

__device__ __forceinline__ Bounds chunk_bounds(const ChunkIO &io, const gbfsm_nfa_dev &A,
                                               const uint8_t *base, int cid, int64_t off) {
    const gbfsm_chunk ch = io.chunks[cid];
    Bounds r;
    r.b = ch.begin - off;
    r.e = ch.end - off;
    if (ch.index > 0) r.b = chunk_start(A, base, r.b, r.e);
    r.ov_end = r.e;
    if (cid + 1 < io.n_chunks) {
        const gbfsm_chunk nx = io.chunks[cid + 1];
        if (nx.index != 0) {
            const int64_t nb = nx.begin - off, ne = nx.end - off;
            r.e = chunk_start(A, base, nb, ne);
            r.ov_end = min(r.e + (int64_t)kOverlap, ne);
        }
    }
    return r;
}

__device__ __forceinline__ int checkpoint_of(int64_t j) {
    return (j >= 1 && j <= (1 << (kCheckpoints - 1)) && (j & (j - 1)) == 0) ? 31 - __clz((int)j)
                                                                            : -1;
}

// Record an accept at position `pos` (j bytes into a speculative chunk): it is the first
// accept after every checkpoint before j that has none yet.
__device__ __forceinline__ void note_accept(int32_t (&acc_after)[kCheckpoints], int64_t j,
                                            int32_t pos) {
#pragma unroll
    for (int c = 0; c < kCheckpoints; ++c)
        if (j > (1 << c) && acc_after[c] < 0) acc_after[c] = pos;
}

// ---- warp chunk (any set size; the overflow path of lane chunks) --------------------------

__device__ __forceinline__ void write_overlap(ChunkRecord *rec, int32_t ov_len, int32_t ov_event,
                                              const int32_t (&ov_counts)[kCheckpoints]) {
    rec->ov_len = ov_len;
    rec->ov_event = ov_event;
#pragma unroll
    for (int c = 0; c < kCheckpoints; ++c) rec->ov_counts[c] = ov_counts[c];
}

// b, e, ov_end: input-relative bounds of the chunk and of its overlap run.
__device__ inline void run_chunk(const gbfsm_nfa_dev &nfa, const Rows &R, WarpScratch S,
                                 const uint8_t *base, int64_t b, int64_t e, int64_t ov_end,
                                 int index, ChunkRecord *rec) {
    const uint32_t lane = lane_id();
    WarpNfa<false> w(nfa, R, S);
    int32_t counts[kCheckpoints], acc_after[kCheckpoints];
#pragma unroll
    for (int c = 0; c < kCheckpoints; ++c) {
        counts[c] = 0;
        acc_after[c] = -1;
    }
    int32_t dead_at = -1;
    bool stopped = false;
    int ev;
    if (index == 0) {
        ev = w.init_start();
        if (ev == kAccept) {
            acc_after[0] = 0;
            stopped = true;
        }
    } else {
        const uint32_t c0 = byte_at(base + b - 2);
        ev = w.init_records(nfa.first_edges, __ldg(nfa.first_row + c0),
                            __ldg(nfa.first_row + c0 + 1));
        if (ev != kDead) ev = w.step(byte_at(base + b - 1));
        if (ev == kDead) {
            dead_at = (int32_t)b;
            stopped = true;
        }
    }
    const int64_t len = e - b;
    ByteStream bytes;
    bytes.init(base + b, stopped ? 0 : len);
    int64_t j = 0;
    while (!stopped && j < len) {
        ev = w.step(bytes.next());
        ++j;
        const int32_t pos = (int32_t)(b + j);
        if (ev == kDead) {
            dead_at = pos;
            stopped = true;
        } else if (ev == kAccept) {
            if (index == 0) {
                acc_after[0] = pos;
                stopped = true;
            } else {
                note_accept(acc_after, j, pos);
                if (j > kOverlap) stopped = true;
            }
        }
        const int c = checkpoint_of(j);
        if (c >= 0 && ev != kDead) counts[c] = w.m;
    }
    int32_t end_count = -1;
    int32_t ov_len = 0, ov_event = 0, ov_counts[kCheckpoints];
#pragma unroll
    for (int c = 0; c < kCheckpoints; ++c) ov_counts[c] = 0;
    if (!stopped) {
        end_count = w.export_recs(rec->end_recs, kEndCap);
        __syncwarp();
        for (int64_t t = 1; t <= ov_end - e; ++t) {
            const int ev2 = w.step(byte_at(base + e + t - 1));
            ov_len = (int32_t)t;
            if (ev2 == kDead) {
                ov_event = -(int32_t)t;
                break;
            }
            if (ev2 == kAccept) {
                ov_event = (int32_t)t;
                break;
            }
            const int c = checkpoint_of(t);
            if (c >= 0) ov_counts[c] = w.m;
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < kCheckpoints; ++c) {
            rec->counts[c] = counts[c];
            rec->acc_after[c] = acc_after[c];
        }
        rec->dead_at = dead_at;
        rec->end_count = end_count;
        rec->begin = b;
        rec->end = e;
        write_overlap(rec, ov_len, ov_event, ov_counts);
    }
    w.cleanup();
}

// ---- lane chunk (one chunk per thread; up to kLaneSlots states) ----------------------------

// Sequential 4-byte words of a byte range starting at any alignment: aligned 16-byte
// blocks read one block ahead (never past `end`), each word put together by one funnel
// shift of two aligned words.
struct WordStream {
    const uint8_t *blk;
    const uint8_t *end;
    uint4 cur, nxt;
    uint32_t wi;  // aligned word (0..3) of cur holding the next byte
    uint32_t sh;  // 8 x the byte offset of the next byte in that word

    __device__ __forceinline__ static uint32_t word(const uint4 &v, uint32_t i) {
        return i == 0u ? v.x : i == 1u ? v.y : i == 2u ? v.z : v.w;
    }

    __device__ __forceinline__ void init(const uint8_t *p, const uint8_t *e) {
        end = e;
        const uint64_t a = reinterpret_cast<uint64_t>(p);
        blk = reinterpret_cast<const uint8_t *>(a & ~15ull);
        wi = (uint32_t)((a >> 2) & 3u);
        sh = (uint32_t)(a & 3u) * 8u;
        cur = ld_stream16(blk);
        nxt = (blk + 16 < end) ? ld_stream16(blk + 16) : make_uint4(0, 0, 0, 0);
    }

    __device__ __forceinline__ uint32_t next_word() {
        const uint32_t lo = word(cur, wi);
        const uint32_t hi = wi == 3u ? nxt.x : word(cur, wi + 1u);
        const uint32_t w = __funnelshift_r(lo, hi, sh);
        if (++wi == 4u) {
            wi = 0u;
            blk += 16;
            cur = nxt;
            nxt = (blk + 16 < end) ? ld_stream16(blk + 16) : make_uint4(0, 0, 0, 0);
        }
        return w;
    }
};
//
// The set is kept as the lane records (gbfsm_lane_rec) of its members, slot q valid when
// bit q of `valid` is set. Per byte: find each member's edges labelled with the byte --
// two byte-wise compares of its packed labels for a state in the fast form, a scan of
// edge_sym (L1-resident) otherwise -- collecting at most kLaneSlots matching edges; load
// the lane records of their targets together (one L2 round trip); the distinct targets
// are the next set.

__device__ __forceinline__ uint4 ld_lane(const gbfsm_lane_rec *p) {
    return __ldg(reinterpret_cast<const uint4 *>(p));
}

// Lane record of state s, built from the CSR rows (the start state of a first chunk).
__device__ inline uint4 lane_record_of(const gbfsm_nfa_dev &A, uint32_t s) {
    const uint32_t rb = __ldg(A.sym_row + s), re = __ldg(A.sym_row + s + 1);
    const uint32_t deg = re - rb;
    const bool acc =
        (__ldg(reinterpret_cast<const unsigned long long *>(A.accept_words) + (s >> 6)) >>
         (s & 63u)) & 1ull;
    bool slow = deg > (uint32_t)GBFSM_LANE_FAST_DEGREE;
    uint32_t lo = 0, hi = 0;
    for (uint32_t j = 0; j < deg && !slow; ++j) {
        const uint32_t sym = __ldg(A.edge_sym + rb + j);
        if (sym == (uint32_t)GBFSM_ANY_SYMBOL) slow = true;
        if (j < 4) lo |= (sym & 0xFFu) << (8u * j);
        else if (j < 8) hi |= (sym & 0xFFu) << (8u * (j - 4));
    }
    const uint32_t x = s | (slow ? 0u : deg << GBFSM_LANE_DEG_SHIFT) |
                       (slow ? GBFSM_LANE_SLOW : 0u) | (acc ? GBFSM_LANE_ACCEPT : 0u);
    return slow ? make_uint4(x, rb, re, 0u) : make_uint4(x, rb, lo, hi);
}

__device__ __forceinline__ uint32_t lane_degree(uint32_t x) {
    return (x >> GBFSM_LANE_DEG_SHIFT) & GBFSM_LANE_DEG_MASK;
}

// The engine state record (as WarpNfa keeps it) of a lane record.
__device__ __forceinline__ uint4 warp_record_of(uint4 l) {
    const uint32_t re = (l.x & GBFSM_LANE_SLOW) ? l.z : l.y + lane_degree(l.x);
    return make_uint4(l.x & GBFSM_LANE_STATE_MASK,
                      (l.x & GBFSM_LANE_ACCEPT) ? GBFSM_EDGE_ACCEPT : 0u, l.y, re);
}

// Append edge k to the match list (kept in registers: the index is a run-time count).
__device__ __forceinline__ void add_match(uint32_t (&mk)[kLaneSlots], int &nm, uint32_t k) {
#pragma unroll
    for (int u = 0; u < kLaneSlots; ++u)
        if (u == nm) mk[u] = k;
    ++nm;
}

// Bit 7 of each byte of the result is set where the byte of x is zero (exact: the
// per-byte sum cannot carry into the next byte).
__device__ __forceinline__ uint32_t zero_bytes(uint32_t x) {
    const uint32_t t = (x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu;
    return ~(t | x) & 0x80808080u;
}

// Byte markers of the first k (< 0: none, >= 4: all four) bytes of a word.
__device__ __forceinline__ uint32_t first_bytes(int k) {
    // shr.b32 clamps shift counts above 32 to 32, which yields 0 (k <= 0)
    const uint32_t shift = 32u - 8u * (uint32_t)min(max(k, 0), 4);
    uint32_t r;
    asm("shr.b32 %0, %1, %2;" : "=r"(r) : "r"(0x80808080u), "r"(shift));
    return r;
}

// Markers (bit 7 of byte j of word w: edge 4w + j) of the labels of a fast-form record
// equal to the byte: edges 0..7 from the record, edges 8..15 from the ext table.
// Returns the number of markers.
__device__ __forceinline__ int label_matches(const uint4 &r, uint32_t sym4,
                                             const uint2 *__restrict__ ext, uint32_t (&m)[4]) {
    const int deg = (int)lane_degree(r.x);
    m[0] = zero_bytes(r.z ^ sym4) & first_bytes(deg);
    m[1] = zero_bytes(r.w ^ sym4) & first_bytes(deg - 4);
    m[2] = 0u;
    m[3] = 0u;
    int c = __popc(m[0]) + __popc(m[1]);
    if (deg > 8) {
        const uint2 h = __ldg(ext + (r.x & GBFSM_LANE_STATE_MASK));
        m[2] = zero_bytes(h.x ^ sym4) & first_bytes(deg - 8);
        m[3] = zero_bytes(h.y ^ sym4) & first_bytes(deg - 12);
        c += __popc(m[2]) + __popc(m[3]);
    }
    return c;
}

// Edge of the lowest remaining marker of m (edge 4w + j of the row starting at rb for
// bit 7 of byte j of word w), cleared from m. m must have a marker.
__device__ __forceinline__ uint32_t pop_match(uint32_t (&m)[4], uint32_t rb) {
    uint32_t w, off;
    if (m[0] | m[1]) {  // edges 0..7: almost every match
        const bool z0 = m[0] != 0u;
        w = z0 ? m[0] : m[1];
        off = z0 ? 0u : 4u;
        const uint32_t rest = w & (w - 1u);
        if (z0) m[0] = rest;
        else m[1] = rest;
    } else {
        const bool z2 = m[2] != 0u;
        w = z2 ? m[2] : m[3];
        off = z2 ? 8u : 12u;
        const uint32_t rest = w & (w - 1u);
        if (z2) m[2] = rest;
        else m[3] = rest;
    }
    return rb + off + ((uint32_t)(__ffs(w) - 1) >> 3);
}

// The set becomes the distinct targets of the matched edges mk[0 .. nm) (nm <= kLaneSlots),
// their records loaded together; returns the member count (acc: a member accepts).
__device__ __forceinline__ int load_targets(uint4 (&cur)[kLaneSlots], uint32_t &valid, bool &acc,
                                            const uint32_t (&mk)[kLaneSlots], int nm,
                                            const gbfsm_lane_rec *__restrict__ recs) {
#pragma unroll
    for (int q = 0; q < kLaneSlots; ++q)
        cur[q] = (q < nm) ? ld_lane(recs + mk[q]) : make_uint4(0, 0, 0, 0);
    valid = 0;
    acc = false;
#pragma unroll
    for (int q = 0; q < kLaneSlots; ++q) {
        bool keep = q < nm;
#pragma unroll
        for (int u = 0; u < q; ++u)
            keep = keep && ((cur[u].x ^ cur[q].x) & GBFSM_LANE_STATE_MASK) != 0u;
        if (keep) {
            valid |= 1u << q;
            acc |= (cur[q].x & GBFSM_LANE_ACCEPT) != 0u;
        }
    }
    return __popc(valid);
}

// One byte: returns the new member count (acc: a member accepts), or -1 when more than
// kLaneSlots edges match.
__device__ __forceinline__ int lane_step(uint4 (&cur)[kLaneSlots], uint32_t &valid, bool &acc,
                                         uint32_t sym, const uint16_t *__restrict__ labels,
                                         const gbfsm_lane_rec *__restrict__ recs,
                                         const uint2 *__restrict__ ext) {
    const uint32_t sym4 = sym * 0x01010101u;
    // The common cases, with little divergence between the lanes of a warp: one or two
    // members in the fast form (slots 0 and 1) with at most two matching edges between
    // them. The second member's compare and the second load run only in the lanes
    // that need them.
    const bool v1 = (valid >> 1) & 1u;
    if ((valid & ~3u) == 0u && valid != 0u && !(cur[0].x & GBFSM_LANE_SLOW) &&
        !(v1 && (cur[1].x & GBFSM_LANE_SLOW))) {
        uint32_t ma[4], mb[4] = {0u, 0u, 0u, 0u};
        const int ca = label_matches(cur[0], sym4, ext, ma);
        const int cb = v1 ? label_matches(cur[1], sym4, ext, mb) : 0;
        const int c = ca + cb;
        if (c == 0) {
            valid = 0;
            acc = false;
            return 0;
        }
        if (c <= 2) {
            const uint32_t rb0 = cur[0].y, rb1 = cur[1].y;
            const uint32_t e0 = ca > 0 ? pop_match(ma, rb0) : pop_match(mb, rb1);
            if (c == 1) {
                cur[0] = ld_lane(recs + e0);
                valid = 1u;
                acc = (cur[0].x & GBFSM_LANE_ACCEPT) != 0u;
                return 1;
            }
            const uint32_t e1 = ca > 1 ? pop_match(ma, rb0) : pop_match(mb, rb1);
            const uint4 r0 = ld_lane(recs + e0), r1 = ld_lane(recs + e1);
            const bool two = ((r0.x ^ r1.x) & GBFSM_LANE_STATE_MASK) != 0u;
            cur[0] = r0;
            cur[1] = r1;
            valid = two ? 3u : 1u;
            acc = (r0.x & GBFSM_LANE_ACCEPT) || (two && (r1.x & GBFSM_LANE_ACCEPT));
            return two ? 2 : 1;
        }
    }
    uint32_t mk[kLaneSlots];
    int nm = 0;
#pragma unroll
    for (int q = 0; q < kLaneSlots; ++q) mk[q] = 0;
#pragma unroll
    for (int q = 0; q < kLaneSlots; ++q) {
        if (!((valid >> q) & 1u)) continue;
        const uint4 r = cur[q];
        if (!(r.x & GBFSM_LANE_SLOW)) {
            uint32_t m[4];
            label_matches(r, sym4, ext, m);
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                while (m[w]) {
                    add_match(mk, nm, r.y + 4u * w + ((uint32_t)(__ffs(m[w]) - 1) >> 3));
                    m[w] &= m[w] - 1u;
                }
            }
        } else {
            for (uint32_t k = r.y; k < r.z; ++k) {
                const uint32_t es = __ldg(labels + k);
                if (es == sym || es == (uint32_t)GBFSM_ANY_SYMBOL) add_match(mk, nm, k);
            }
        }
    }
    if (nm > kLaneSlots) return -1;
    return load_targets(cur, valid, acc, mk, nm, recs);
}

// Calls f(edge) for every edge of the lane record r labelled `sym` (or ANY).
template <typename F>
__device__ __forceinline__ void for_each_match(const uint4 &r, uint32_t sym,
                                               const uint16_t *__restrict__ labels,
                                               const uint2 *__restrict__ ext, F &&f) {
    if (!(r.x & GBFSM_LANE_SLOW)) {
        uint32_t m[4];
        label_matches(r, sym * 0x01010101u, ext, m);
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            while (m[w]) {
                f(r.y + 4u * w + ((uint32_t)(__ffs(m[w]) - 1) >> 3));
                m[w] &= m[w] - 1u;
            }
        }
    } else {
        for (uint32_t k = r.y; k < r.z; ++k) {
            const uint32_t es = __ldg(labels + k);
            if (es == sym || es == (uint32_t)GBFSM_ANY_SYMBOL) f(k);
        }
    }
}

// Start set of a later chunk at b when the two-byte superset there is too large for a
// lane: the two-byte superset at b-2 (at most kWideStart members, streamed from
// pair_lanes) stepped over x[b-2] and x[b-1] -- again a superset of the true set at b,
// and usually far smaller. The intermediate set is never held: each member's targets
// on x[b-2] are expanded over x[b-1] at once, and only the final edges (distinct, at
// most kLaneSlots) are kept. Returns false when the wide set or the final set is too
// large.
constexpr uint32_t kWideStart = 64;

__device__ inline bool widened_start(const gbfsm_nfa_dev &A, const uint8_t *base, int64_t b,
                                     const uint16_t *__restrict__ labels,
                                     const gbfsm_lane_rec *__restrict__ recs,
                                     const uint2 *__restrict__ ext, uint4 (&cur)[kLaneSlots],
                                     uint32_t &valid) {
    if (b < 4) return false;
    const uint32_t key = byte_at(base + b - 4) * 256u + byte_at(base + b - 3);
    const uint32_t pr = __ldg(A.pair_row + key);
    const uint32_t cnt = __ldg(A.pair_row + key + 1) - pr;
    if (cnt > kWideStart) return false;
    const uint32_t s1 = byte_at(base + b - 2), s2 = byte_at(base + b - 1);
    uint32_t mk[kLaneSlots];
    int nm = 0;
#pragma unroll
    for (int q = 0; q < kLaneSlots; ++q) mk[q] = 0xFFFFFFFFu;
    auto add_final = [&](uint32_t k2) {
        bool seen = false;
#pragma unroll
        for (int u = 0; u < kLaneSlots; ++u) seen = seen || mk[u] == k2;
        if (!seen) add_match(mk, nm, k2);
    };
    for (uint32_t q = 0; q < cnt && nm <= kLaneSlots; ++q) {
        const uint4 r = ld_lane(A.pair_lanes + pr + q);
        for_each_match(r, s1, labels, ext, [&](uint32_t k1) {
            if (nm > kLaneSlots) return;
            for_each_match(ld_lane(recs + k1), s2, labels, ext, add_final);
        });
    }
    if (nm > kLaneSlots) return false;
    bool acc;
    load_targets(cur, valid, acc, mk, nm, recs);
    return true;
}

// Returns false, writing nothing, when a start superset or a byte's matches exceed
// kLaneSlots inside the chunk (the chunk is then run by a warp); in the overlap that only
// ends the overlap run.
__device__ inline bool lane_chunk(const gbfsm_nfa_dev &A, const uint8_t *base, int64_t b,
                                  int64_t e, int64_t ov_end, int index, ChunkRecord *rec) {
    const uint16_t *__restrict__ labels = A.edge_sym;
    const gbfsm_lane_rec *__restrict__ recs = A.lane_edges;
    const uint2 *__restrict__ ext = reinterpret_cast<const uint2 *>(A.lane_labels_ext);
    uint4 cur[kLaneSlots];
#pragma unroll
    for (int q = 0; q < kLaneSlots; ++q) cur[q] = make_uint4(0, 0, 0, 0);
    uint32_t valid = 0;
    int32_t counts[kCheckpoints], acc_after[kCheckpoints];
#pragma unroll
    for (int c = 0; c < kCheckpoints; ++c) {
        counts[c] = 0;
        acc_after[c] = -1;
    }
    int32_t dead_at = -1;
    bool stopped = false;
    if (index == 0) {
        cur[0] = lane_record_of(A, (uint32_t)A.start_state);
        valid = 1;
        if (cur[0].x & GBFSM_LANE_ACCEPT) {
            acc_after[0] = 0;
            stopped = true;
        }
    } else {
        const uint32_t key = byte_at(base + b - 2) * 256u + byte_at(base + b - 1);
        const uint32_t pr = __ldg(A.pair_row + key);
        const uint32_t cnt = __ldg(A.pair_row + key + 1) - pr;
        if (cnt <= (uint32_t)kLaneSlots) {
#pragma unroll
            for (int q = 0; q < kLaneSlots; ++q)
                if ((uint32_t)q < cnt) cur[q] = ld_lane(A.pair_lanes + pr + q);
            valid = (1u << cnt) - 1u;
        } else if (!widened_start(A, base, b, labels, recs, ext, cur, valid)) {
            return false;
        }
        if (valid == 0u) {
            dead_at = (int32_t)b;
            stopped = true;
        }
    }
    const int32_t len = (int32_t)(e - b);
    const int32_t b32 = (int32_t)b;
    ByteStream bytes;
    bytes.init(base + b, stopped ? 0 : len);
    int32_t j = 0;
    int m = __popc(valid);
    // the first kOverlap bytes: set sizes at the checkpoints; a later chunk's accept there
    // is recorded without stopping
    const int32_t head = min(len, (int32_t)kOverlap);
    while (!stopped && j < head) {
        const uint32_t sym = bytes.next();
        ++j;
        bool acc;
        m = lane_step(cur, valid, acc, sym, labels, recs, ext);
        if (m < 0) return false;
        const int32_t pos = b32 + j;
        if (m == 0) {  // reference.py:59-60
            dead_at = pos;
            stopped = true;
            break;
        }
        if (acc) {
            if (index == 0) {
                acc_after[0] = pos;
                stopped = true;
                break;
            }
            note_accept(acc_after, j, pos);
        }
        const int c = checkpoint_of(j);
#pragma unroll
        for (int q = 0; q < kCheckpoints; ++q)
            if (q == c) counts[q] = m;
    }
    // The checkpoint sizes are final now, and so are the first accepts found so far:
    // write them, keeping only which accepts are still open, so that the long loop below
    // holds no arrays.
    uint32_t open_acc = 0;  // (a first chunk records only its own first accept)
#pragma unroll
    for (int c = 0; c < kCheckpoints; ++c) {
        rec->counts[c] = counts[c];
        rec->acc_after[c] = acc_after[c];
        if (acc_after[c] < 0 && (index > 0 || c == 0)) open_acc |= 1u << c;
    }
    // The rest: no checkpoints, and any accept ends the run (it is the first accept
    // after every checkpoint still open, all of which lie before it). Four bytes per
    // word; the last (at most three) bytes one at a time. step() returns 1 to stop, -1
    // when the set outgrew the lane.
    auto step = [&](uint32_t sym) -> int {
        ++j;
        bool acc;
        m = lane_step(cur, valid, acc, sym, labels, recs, ext);
        if (m < 0) return -1;
        if (m == 0) {
            dead_at = b32 + j;
            stopped = true;
        } else if (acc) {
            for (int c = 0; c < kCheckpoints; ++c)
                if ((open_acc >> c) & 1u) rec->acc_after[c] = b32 + j;
            stopped = true;
        }
        return stopped ? 1 : 0;
    };
    if (!stopped && len - j >= 4) {
        WordStream words;
        words.init(base + b + j, base + e);
        while (!stopped && len - j >= 4) {
            const uint32_t w4 = words.next_word();
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int r = step((w4 >> (8 * t)) & 0xFFu);
                if (r < 0) return false;
                if (r) break;
            }
        }
    }
    while (!stopped && j < len)
        if (step(byte_at(base + b + j)) < 0) return false;
    rec->dead_at = dead_at;
    rec->end_count = stopped ? -1 : m;
    rec->begin = b;
    rec->end = e;
    int32_t ov_len = 0, ov_event = 0, ov_counts[kCheckpoints];
#pragma unroll
    for (int c = 0; c < kCheckpoints; ++c) ov_counts[c] = 0;
    if (!stopped) {
        int o = 0;
#pragma unroll
        for (int q = 0; q < kLaneSlots; ++q) {
            if ((valid >> q) & 1u) {
                rec->end_recs[o] = warp_record_of(cur[q]);
                ++o;
            }
        }
        for (int64_t t = 1; t <= ov_end - e; ++t) {
            bool acc;
            const int nm = lane_step(cur, valid, acc, byte_at(base + e + t - 1), labels, recs, ext);
            if (nm < 0) break;
            ov_len = (int32_t)t;
            if (nm == 0) {
                ov_event = -(int32_t)t;
                break;
            }
            if (acc) {
                ov_event = (int32_t)t;
                break;
            }
            const int c = checkpoint_of(t);
#pragma unroll
            for (int q = 0; q < kCheckpoints; ++q)
                if (q == c) ov_counts[q] = nm;
        }
    }
    write_overlap(rec, ov_len, ov_event, ov_counts);
    return true;
}

// ---- exact fix-up (one warp per chunked input) ----------------------------------------------

struct RecordHead {
    int32_t counts[kCheckpoints];
    int32_t acc_after[kCheckpoints];
    int32_t dead_at;
    int32_t end_count;
    int64_t begin;
    int64_t end;
};

__device__ __forceinline__ RecordHead load_head(const ChunkRecord *recs, int k) {
    RecordHead h;
    const ChunkRecord &r = recs[k];
#pragma unroll
    for (int c = 0; c < kCheckpoints; ++c) {
        h.counts[c] = r.counts[c];
        h.acc_after[c] = r.acc_after[c];
    }
    h.dead_at = r.dead_at;
    h.end_count = r.end_count;
    h.begin = r.begin;
    h.end = r.end;
    return h;
}

enum LinkStatus { kLink = 0, kDecide = 1, kBreak = 2 };

// Chunk `rk` (starting `begin` bytes into its input) against its predecessor's overlap
// run: kLink (its record is exact from a checkpoint on and has no event), kDecide (the
// input's verdict: accept when flag, at / examined up to `pos`), or kBreak (no link).
__device__ __forceinline__ int classify(const ChunkRecord &prev, const ChunkRecord &rk,
                                        int64_t begin, int32_t &flag, int64_t &pos) {
    const int32_t ov_len = prev.ov_len, ov_event = prev.ov_event;
    const int32_t ov_at = ov_event < 0 ? -ov_event : ov_event;
#pragma unroll
    for (int c = 0; c < kCheckpoints; ++c) {
        const int32_t j = 1 << c;
        if (ov_event != 0 && ov_at <= j) {
            flag = ov_event > 0;
            pos = begin + ov_at;
            return kDecide;
        }
        if (j > ov_len) return kBreak;
        if (prev.ov_counts[c] == rk.counts[c]) {
            if (rk.acc_after[c] >= 0) {
                flag = 1;
                pos = rk.acc_after[c];
                return kDecide;
            }
            if (rk.dead_at >= 0) {
                flag = 0;
                pos = rk.dead_at;
                return kDecide;
            }
            return kLink;
        }
    }
    return kBreak;
}

__device__ __forceinline__ Verdict decided(int32_t flag, int64_t pos) {
    Verdict v;
    v.flag = flag;
    v.len = flag ? (int32_t)pos : 0;
    v.examined = pos;
    return v;
}

// Serial re-run of chunks [start, count) from the exact set already in `w`; the part of
// the fix-up that runs only from a chunk the scan could not link.
__device__ inline Verdict serial_fixup(WarpNfa<false> &w, const uint8_t *base, int64_t len,
                                       const ChunkRecord *recs, int first, int start,
                                       int count) {
    Verdict v{0, 0, len};
    RecordHead next = load_head(recs, first + start);
    for (int k = start; k < count; ++k) {
        const RecordHead rk = next;
        if (k + 1 < count) next = load_head(recs, first + k + 1);  // prefetch
        const int64_t b = rk.begin, e = rk.end;
        int matched = -1;
        int64_t j = 0;
        while (b + j < e) {
            const int ev = w.step(byte_at(base + b + j));
            ++j;
            if (ev == kDead) return decided(0, b + j);
            if (ev == kAccept) return decided(1, b + j);
            const int c = checkpoint_of(j);
            if (c >= 0 && w.m == rk.counts[c]) {
                matched = c;
                break;
            }
        }
        if (matched >= 0) {
            if (rk.acc_after[matched] >= 0) return decided(1, rk.acc_after[matched]);
            if (rk.dead_at >= 0) return decided(0, rk.dead_at);
            if (rk.end_count >= 0) {
                w.cleanup();
                w.init_recs(recs[first + k].end_recs, min(rk.end_count, kEndCap));
            } else {
                while (b + j < e) w.step(byte_at(base + b + j++));  // no event can occur here
            }
        }
    }
    return v;
}

__device__ inline Verdict run_fixup(const gbfsm_nfa_dev &nfa, const Rows &R, WarpScratch S,
                                    const uint8_t *base, int64_t len, const ChunkRecord *recs,
                                    int first, int count) {
    const uint32_t lane = lane_id();
    const ChunkRecord &r0 = recs[first];
    if (r0.acc_after[0] >= 0) return decided(1, r0.acc_after[0]);
    if (r0.dead_at >= 0) return decided(0, r0.dead_at);
    // scan: 32 chunks per round, one per lane; stop at the first that is not linked
    int last_rec = r0.end_count >= 0 ? 0 : -1;  // last chunk with an exact recorded end set
    int brk = -1;
    for (int k0 = 1; k0 < count && brk < 0; k0 += 32) {
        const int k = k0 + (int)lane;
        int status = kLink;
        int32_t flag = 0;
        int64_t pos = 0;
        bool rec_ok = false;
        if (k < count) {
            const ChunkRecord &rk = recs[first + k];
            status = classify(recs[first + k - 1], rk, rk.begin, flag, pos);
            rec_ok = rk.end_count >= 0;
        }
        const uint32_t stop = __ballot_sync(GBFSM_FULL_MASK, status != kLink);
        const uint32_t before = stop ? (stop & (0u - stop)) - 1u : GBFSM_FULL_MASK;
        const uint32_t recm = __ballot_sync(GBFSM_FULL_MASK, rec_ok) & before;
        if (recm) last_rec = k0 + 31 - __clz(recm);
        if (stop) {
            const int src = __ffs(stop) - 1;
            status = __shfl_sync(GBFSM_FULL_MASK, status, src);
            flag = __shfl_sync(GBFSM_FULL_MASK, flag, src);
            pos = __shfl_sync(GBFSM_FULL_MASK, pos, src);
            if (status == kDecide) return decided(flag, pos);
            brk = k0 + src;
        }
    }
    if (brk < 0) return Verdict{0, 0, len};  // every chunk linked, no event: no accept
    // fall back: serial from the chunk after the last exact recorded end set
    WarpNfa<false> w(nfa, R, S);
    int start;
    if (last_rec >= 0) {
        w.init_recs(recs[first + last_rec].end_recs,
                    min(recs[first + last_rec].end_count, kEndCap));
        start = last_rec + 1;
    } else {  // the first chunk's final set was not recorded: recompute it exactly
        w.init_start();
        const int64_t e0 = recs[first].end;
        for (int64_t p = 0; p < e0; ++p) w.step(byte_at(base + p));
        start = 1;
    }
    const Verdict v = serial_fixup(w, base, len, recs, first, start, count);
    w.cleanup();
    return v;
}

}  // namespace gbfsm
