// Device-side NFA simulation (latch-first-match), shared by the plain batch kernels
// (nfa_kernels.cu) and the persistent engine (persistent.cu).
//
// Semantics: src/gpufsm/reference.py:36-65 (simulate) with the epsilon closure of
// :20-33. Per input byte the next set is the union of the targets of matching edges
// (symbol == byte or ANY); an empty next set ends the run with (0, 0); otherwise the
// set is closed under epsilon edges and an accepting member latches (1, pos + 1). The
// start configuration is the closure of {start}; if it accepts the verdict is (1, 0).
//
// Two set representations, chosen per step by a warp:
//   sparse: a list of member records (gbfsm_edge of the state: id, accept/eps flags and
//           its edge-row range) plus a dedup bitmap V that is all-zero between steps;
//           a step costs O(members + edges touched) and one dependent edge-record load;
//   dense:  the packed bitmap (pack_accept word layout, src/gpufsm/core/packing.py:
//           66-85); a step scans all W words.
// A step that overflows the list capacity continues in dense form (V already holds the
// whole next set); a dense set that shrinks to half the capacity returns to a list.
//
// Work distribution inside the warp uses ballot/popc/shuffle: the members of a batch
// (up to 32) publish their edge counts, a warp scan gives each lane flat edge indices,
// a 5-step shuffle search maps a flat index back to its member, matching edges are
// inserted with shared-memory atomicOr and new members are compacted into the next
// list with __ballot_sync + __popc.
#pragma once

#include "common.cuh"

namespace gbfsm {

constexpr int kFlagTimeout = -1;  // flags[] value written when a bounded wait gave up

// Per-warp scratch of the warp simulator.
struct WarpScratch {
    uint64_t *V;   // [W] next-set bitmap; all-zero between steps
    uint64_t *D;   // [W] dense current set; all-zero while sparse
    uint64_t *FA;  // [W] dense closure frontier; all-zero between steps
    uint64_t *FB;  // [W] dense closure frontier (next round); all-zero between steps
    uint4 *LA;     // [C] current member list
    uint4 *LB;     // [C] next member list
    int C;         // list capacity; 0 = dense only
};

struct Verdict {
    int32_t flag;
    int32_t len;
    int64_t examined;
};

template <bool kStaged>
__device__ __forceinline__ uint4 load_edge(const gbfsm_edge *p) {
    if (kStaged) return *reinterpret_cast<const uint4 *>(p);
    return ld_edge(p);
}

template <bool kStaged>
__device__ __forceinline__ uint32_t load_row(const uint32_t *p) {
    if (kStaged) return *p;
    return __ldg(p);
}

// Edge rows of the automaton (global, or staged copies in shared memory).
struct Rows {
    const uint32_t *sym_row;
    const gbfsm_edge *sym_edges;
    const uint32_t *eps_row;
    const gbfsm_edge *eps_edges;
};

// Walk the edges of a batch of up to 32 members, one member per lane: lane l owns edges
// [rb_l, rb_l + deg_l) of `edges`. Flattened over the warp. An edge whose symbol matches
// (or any edge when `filter` is false) inserts its target into V; a first insertion is
// appended to `out` (when below capacity C) and, when F is non-null, marked in F.
// Returns the number of new members; ORs their info words into `info_or`.
template <bool kStaged>
__device__ __forceinline__ int walk_batch(const gbfsm_edge *edges, uint32_t rb, uint32_t deg,
                                          bool filter, uint32_t sym, uint64_t *V, uint4 *out,
                                          int n_out, int C, uint64_t *F, uint32_t &info_or) {
    const uint32_t lane = lane_id();
    const uint32_t incl = warp_inclusive_scan(deg);
    const uint32_t total = __shfl_sync(GBFSM_FULL_MASK, incl, 31);
    const uint32_t excl = incl - deg;
    int added = 0;
    for (uint32_t f0 = 0; f0 < total; f0 += 32) {
        const uint32_t f = f0 + lane;
        // largest lane whose first flat index is <= f owns edge f
        uint32_t owner = 0;
#pragma unroll
        for (uint32_t step = 16; step >= 1; step >>= 1) {
            const uint32_t cand = owner + step;
            const uint32_t e = __shfl_sync(GBFSM_FULL_MASK, excl, cand);
            if (e <= f) owner = cand;
        }
        const uint32_t orb = __shfl_sync(GBFSM_FULL_MASK, rb, owner);
        const uint32_t oex = __shfl_sync(GBFSM_FULL_MASK, excl, owner);
        bool fresh = false;
        uint4 rec = make_uint4(0, 0, 0, 0);
        if (f < total) {
            rec = load_edge<kStaged>(edges + orb + (f - oex));
            const uint32_t s = rec.y & GBFSM_EDGE_SYMBOL_MASK;
            if (!filter || s == sym || s == GBFSM_ANY_SYMBOL) {
                const unsigned long long bit = 1ull << (rec.x & 63u);
                const unsigned long long old =
                    atomicOr(reinterpret_cast<unsigned long long *>(V + (rec.x >> 6)), bit);
                fresh = (old & bit) == 0;
                if (fresh && F) atomicOr(reinterpret_cast<unsigned long long *>(F + (rec.x >> 6)), bit);
            }
        }
        const uint32_t ball = __ballot_sync(GBFSM_FULL_MASK, fresh);
        if (fresh) {
            const int pos = n_out + added + __popc(ball & lanemask_lt());
            if (pos < C) out[pos] = rec;
            info_or |= rec.y;
        }
        added += __popc(ball);
    }
    __syncwarp();  // list entries and V words written above are visible to the warp
    return added;
}

// Sparse expansion of L[0..m) on byte `sym` into V / out. Returns the number of members.
template <bool kStaged>
__device__ __forceinline__ int sparse_expand(const Rows &R, const uint4 *L, int m, uint32_t sym,
                                             uint64_t *V, uint4 *out, int C, uint32_t &info_or) {
    int n = 0;
    for (int base = 0; base < m; base += 32) {
        const int j = base + (int)lane_id();
        uint32_t rb = 0, deg = 0;
        if (j < m) {
            const uint4 r = L[j];
            rb = r.z;
            deg = r.w - r.z;
        }
        n += walk_batch<kStaged>(R.sym_edges, rb, deg, true, sym, V, out, n, C, nullptr, info_or);
    }
    return n;
}

// Epsilon closure of the list out[0..n) (all members already in V). Processes members
// in insertion order, appending epsilon targets; stops early (returns > C) when the list
// overflows, leaving the rest to the dense closure, which rescans V.
template <bool kStaged>
__device__ __forceinline__ int sparse_closure(const Rows &R, uint4 *out, int n, int C, uint64_t *V,
                                              uint32_t &info_or) {
    int a = 0;
    while (a < n && n <= C) {
        const int b = n;
        for (int base = a; base < b; base += 32) {
            const int j = base + (int)lane_id();
            uint32_t eb = 0, deg = 0;
            if (j < b) {
                const uint4 r = out[j];
                if (r.y & GBFSM_EDGE_HAS_EPS) {
                    eb = load_row<kStaged>(R.eps_row + r.x);
                    deg = load_row<kStaged>(R.eps_row + r.x + 1) - eb;
                }
            }
            n += walk_batch<kStaged>(R.eps_edges, eb, deg, false, 0, V, out, n, C, nullptr, info_or);
            if (n > C) break;
        }
        a = b;
    }
    return n;
}

// Dense expansion: every member of bitmap D (W words) follows its matching edges into V.
// Members are taken one per lane per round (lane = word within a 32-word group).
template <bool kStaged>
__device__ __forceinline__ int dense_expand(const Rows &R, const uint64_t *D, int W, bool filter,
                                            uint32_t sym, const gbfsm_edge *edges,
                                            const uint32_t *row, uint64_t *V, uint64_t *F,
                                            uint32_t &info_or) {
    int n = 0;
    for (int g = 0; g < W; g += 32) {
        const int w = g + (int)lane_id();
        unsigned long long bits = (w < W) ? D[w] : 0ull;
        while (__any_sync(GBFSM_FULL_MASK, bits != 0ull)) {
            uint32_t rb = 0, deg = 0;
            if (bits) {
                const uint32_t s = (uint32_t)w * 64u + (uint32_t)(__ffsll((long long)bits) - 1);
                bits &= bits - 1ull;
                rb = load_row<kStaged>(row + s);
                deg = load_row<kStaged>(row + s + 1) - rb;
            }
            n += walk_batch<kStaged>(edges, rb, deg, filter, sym, V, nullptr, 0, 0, F, info_or);
        }
    }
    return n;
}

__device__ __forceinline__ void zero_words(uint64_t *p, int W) {
    for (int w = (int)lane_id(); w < W; w += 32) p[w] = 0ull;
}

// Dense epsilon closure of V. Round 0 expands every member of V; later rounds expand
// the members first inserted by the previous round (frontier FA/FB).
template <bool kStaged>
__device__ __forceinline__ int dense_closure(const Rows &R, int W, uint64_t *V, uint64_t *FA,
                                             uint64_t *FB, uint32_t &info_or) {
    int added = dense_expand<kStaged>(R, V, W, false, 0, R.eps_edges, R.eps_row, V, FA, info_or);
    int last = added;
    uint64_t *cur = FA, *nxt = FB;
    while (last > 0) {
        __syncwarp();
        last = dense_expand<kStaged>(R, cur, W, false, 0, R.eps_edges, R.eps_row, V, nxt, info_or);
        __syncwarp();
        zero_words(cur, W);
        added += last;
        uint64_t *t = cur;
        cur = nxt;
        nxt = t;
    }
    __syncwarp();
    zero_words(cur, W);  // frontier buffers are left all-zero
    return added;
}

// Build the list of the members of bitmap D (popc-compacted); clears D. Returns count.
template <bool kStaged>
__device__ __forceinline__ int bitmap_to_list(const gbfsm_nfa_dev &A, const Rows &R, uint64_t *D,
                                              int W, uint4 *out) {
    int n = 0;
    const bool has_eps = (A.flags & GBFSM_NFA_HAS_EPS) != 0;
    for (int g = 0; g < W; g += 32) {
        const int w = g + (int)lane_id();
        unsigned long long bits = (w < W) ? D[w] : 0ull;
        const uint32_t c = __popcll(bits);
        const uint32_t incl = warp_inclusive_scan(c);
        int pos = n + (int)(incl - c);
        while (bits) {
            const uint32_t s = (uint32_t)w * 64u + (uint32_t)(__ffsll((long long)bits) - 1);
            bits &= bits - 1ull;
            uint32_t info = 0;
            if ((A.accept_words[s >> 6] >> (s & 63u)) & 1ull) info |= GBFSM_EDGE_ACCEPT;
            if (has_eps && load_row<kStaged>(R.eps_row + s + 1) > load_row<kStaged>(R.eps_row + s))
                info |= GBFSM_EDGE_HAS_EPS;
            out[pos++] = make_uint4(s, info, load_row<kStaged>(R.sym_row + s),
                                    load_row<kStaged>(R.sym_row + s + 1));
        }
        if (w < W) D[w] = 0ull;
        n += (int)__shfl_sync(GBFSM_FULL_MASK, incl, 31);
    }
    return n;
}

// Simulate one input with a whole warp. All lanes call it with identical arguments and
// all receive the verdict. `R` may point at shared-memory copies of the edge rows.
template <bool kStaged>
__device__ Verdict simulate_warp(const gbfsm_nfa_dev &A, const Rows &R, const uint8_t *in,
                                 int64_t len, WarpScratch S) {
    const int W = A.num_words;
    const bool has_eps = (A.flags & GBFSM_NFA_HAS_EPS) != 0;
    const int C = S.C;
    Verdict v{0, 0, 0};

    // ---- start configuration: closure({start}) --------------------------------------
    uint32_t info_or = 0;
    int m = 0;
    bool dense = (C == 0);
    {
        const uint32_t s = (uint32_t)A.start_state;
        uint32_t info = 0;
        if ((A.accept_words[s >> 6] >> (s & 63u)) & 1ull) info |= GBFSM_EDGE_ACCEPT;
        if (has_eps && load_row<kStaged>(R.eps_row + s + 1) > load_row<kStaged>(R.eps_row + s))
            info |= GBFSM_EDGE_HAS_EPS;
        const uint4 rec = make_uint4(s, info, load_row<kStaged>(R.sym_row + s),
                                     load_row<kStaged>(R.sym_row + s + 1));
        if (lane_id() == 0) {
            S.V[s >> 6] |= 1ull << (s & 63u);
            if (C > 0) S.LB[0] = rec;
        }
        info_or = info;
        m = 1;
        __syncwarp();
        if (has_eps) {
            if (!dense) m = sparse_closure<kStaged>(R, S.LB, m, C, S.V, info_or);
            if (dense || m > C) {
                __syncwarp();
                m += dense_closure<kStaged>(R, W, S.V, S.FA, S.FB, info_or);
                dense = true;
            }
        }
    }

    int64_t pos = 0;  // bytes consumed so far
    // input bytes: 16-byte blocks, the next block loaded one block ahead of use
    const uint8_t *end = in + len;
    const uint64_t addr = reinterpret_cast<uint64_t>(in);
    const uint8_t *blk = reinterpret_cast<const uint8_t *>(addr & ~15ull);
    int k = (int)(addr & 15ull);
    uint4 chunk = make_uint4(0, 0, 0, 0), ahead = make_uint4(0, 0, 0, 0);
    if (len > 0) chunk = ld_stream16(blk);
    if (blk + 16 < end) ahead = ld_stream16(blk + 16);

    for (;;) {
        // ---- finish the step that produced the set now in V (members m) --------------
        __syncwarp();
        const uint32_t flags = __reduce_or_sync(GBFSM_FULL_MASK, info_or);
        if (flags & GBFSM_EDGE_ACCEPT) {
            v.flag = 1;
            v.len = (int32_t)pos;
            v.examined = pos;
            break;
        }
        if (!dense) {
            // V holds exactly LB[0..m): clear it, LB becomes the current list
            for (int j = (int)lane_id(); j < m; j += 32) S.V[S.LB[j].x >> 6] = 0ull;
            uint4 *t = S.LA;
            S.LA = S.LB;
            S.LB = t;
        } else {
            // V becomes the current set; the old current set (all-zero while sparse,
            // stale while dense) is cleared to serve as the next V
            uint64_t *t = S.D;
            S.D = S.V;
            S.V = t;
            __syncwarp();
            zero_words(S.V, W);
            if (C > 0 && 2 * m <= C) {
                __syncwarp();
                m = bitmap_to_list<kStaged>(A, R, S.D, W, S.LA);
                dense = false;
            }
        }
        __syncwarp();
        if (pos >= len) {
            v.examined = len;
            break;
        }

        // ---- next byte ------------------------------------------------------------
        if (k == 16) {
            blk += 16;
            k = 0;
            chunk = ahead;
            if (blk + 16 < end) ahead = ld_stream16(blk + 16);
        }
        const uint32_t sym = byte_of(chunk, k);
        ++k;
        ++pos;

        info_or = 0;
        int n;
        if (!dense) {
            n = sparse_expand<kStaged>(R, S.LA, m, sym, S.V, S.LB, C, info_or);
        } else {
            n = dense_expand<kStaged>(R, S.D, W, true, sym, R.sym_edges, R.sym_row, S.V, nullptr,
                                      info_or);
        }
        if (n == 0) {  // reference.py:59-60: the set died
            v.examined = pos;
            if (dense) {
                __syncwarp();
                zero_words(S.D, W);
            }
            break;
        }
        __syncwarp();
        if (has_eps && (__reduce_or_sync(GBFSM_FULL_MASK, info_or) & GBFSM_EDGE_HAS_EPS)) {
            if (!dense && n <= C) n = sparse_closure<kStaged>(R, S.LB, n, C, S.V, info_or);
            if (dense || n > C) {
                __syncwarp();
                n += dense_closure<kStaged>(R, W, S.V, S.FA, S.FB, info_or);
            }
        }
        if (!dense && n > C) {
            // the list overflowed: V holds the whole set; continue in dense form
            dense = true;
        }
        m = n;
    }

    // leave the scratch all-zero for the next input
    __syncwarp();
    if (!dense) {
        if (v.flag) {
            for (int j = (int)lane_id(); j < m; j += 32) S.V[S.LB[j].x >> 6] = 0ull;
        }
    } else {
        zero_words(S.V, W);
        zero_words(S.D, W);
    }
    __syncwarp();
    return v;
}

}  // namespace gbfsm
