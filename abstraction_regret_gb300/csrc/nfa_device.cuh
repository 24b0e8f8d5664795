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

// Paths taken rarely per byte (set-size changes, epsilon closure, mode switches). They
// are inlined by default: kept out of line (-DGBFSM_COLD=__noinline__) the per-byte loop
// needs fewer registers, but the stepper's state then lives in local memory, which
// measured slower on GB300 (c3-sustained: 2.9 vs 3.5 GB/s) than two CTAs per SM.
#ifndef GBFSM_COLD
#define GBFSM_COLD __forceinline__
#endif

namespace gbfsm {

constexpr int kFlagTimeout = -1;  // flags[] value written when a bounded wait gave up

// Per-warp scratch of the warp simulator.
struct WarpScratch {
    uint64_t *V;   // [W] next-set bitmap; all-zero between steps
    uint64_t *D;   // [W] dense current set; all-zero while sparse
    uint64_t *FA;  // [W] dense closure frontier; all-zero between steps
    uint64_t *FB;  // [W] dense closure frontier (next closure pass); all-zero between steps
    uint4 *LA;     // [max(C, 32)] current member list
    uint4 *LB;     // [max(C, 32)] next member list (also the REG-mode compaction buffer)
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

// Dense epsilon closure of V. The first pass expands every member of V; each later pass
// expands the members first inserted by the pass before (frontier FA/FB).
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

// Position of the k-th (0-based) set bit of `mask` (k < popc(mask)): binary search on
// popcounts, no shuffles.
__device__ __forceinline__ uint32_t select_bit(uint32_t mask, uint32_t k) {
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t w = 16; w; w >>= 1) {
        const uint32_t c = __popc((mask >> pos) & ((1u << w) - 1u));
        if (k >= c) {
            k -= c;
            pos += w;
        }
    }
    return pos;
}

__device__ __forceinline__ uint4 shfl_rec(const uint4 &r, uint32_t src) {
    return make_uint4(__shfl_sync(GBFSM_FULL_MASK, r.x, src), __shfl_sync(GBFSM_FULL_MASK, r.y, src),
                      __shfl_sync(GBFSM_FULL_MASK, r.z, src), __shfl_sync(GBFSM_FULL_MASK, r.w, src));
}

enum StepEvent { kAlive = 0, kDead = 1, kAccept = 2 };

// One warp's NFA run, advanced one byte at a time. Three representations of the
// current set, chosen per step:
//   REG   up to 32 members, member i's record held by lane i in registers; a step whose
//         members have at most 32 edges in total is one edge load per lane, deduplicated
//         with __match_any_sync and compacted with ballot/popc/select + shuffles;
//   LIST  up to C members in the shared list LA (steps through walk_batch and V);
//   DENSE the packed bitmap D (all W words scanned per step).
// V, FA, FB are all-zero between steps; D is all-zero unless the mode is DENSE.
template <bool kStaged>
struct WarpNfa {
    const gbfsm_nfa_dev &A;
    const Rows &R;
    WarpScratch S;
    int W;
    bool has_eps;
    int mode;  // 0 REG, 1 LIST, 2 DENSE
    int m;
    uint4 mine;

    static constexpr int kReg = 0, kList = 1, kDense = 2;

    __device__ __forceinline__ WarpNfa(const gbfsm_nfa_dev &a, const Rows &r, WarpScratch s)
        : A(a), R(r), S(s), W(a.num_words), has_eps((a.flags & GBFSM_NFA_HAS_EPS) != 0),
          mode(kReg), m(0), mine(make_uint4(0, 0, 0, 0)) {}

    __device__ __forceinline__ uint4 state_record(uint32_t s) const {
        uint32_t info = 0;
        if ((A.accept_words[s >> 6] >> (s & 63u)) & 1ull) info |= GBFSM_EDGE_ACCEPT;
        if (has_eps && load_row<kStaged>(R.eps_row + s + 1) > load_row<kStaged>(R.eps_row + s))
            info |= GBFSM_EDGE_HAS_EPS;
        return make_uint4(s, info, load_row<kStaged>(R.sym_row + s),
                          load_row<kStaged>(R.sym_row + s + 1));
    }

    // The set just built in V (n members; LB holds them when !dense_now) becomes current.
    __device__ GBFSM_COLD int finish_general(int n, bool dense_now, uint32_t info_or) {
        const uint32_t lane = lane_id();
        __syncwarp();
        const uint32_t flags = __reduce_or_sync(GBFSM_FULL_MASK, info_or);
        if (!dense_now) {
            for (int j = (int)lane; j < n; j += 32) S.V[S.LB[j].x >> 6] = 0ull;
            __syncwarp();
            if (n <= 32) {
                mine = ((int)lane < n) ? S.LB[lane] : make_uint4(0, 0, 0, 0);
                mode = kReg;
            } else {
                uint4 *t = S.LA;
                S.LA = S.LB;
                S.LB = t;
                mode = kList;
            }
        } else {
            uint64_t *t = S.D;  // the new set becomes D; the old D (stale or zero) is cleared
            S.D = S.V;
            S.V = t;
            __syncwarp();
            zero_words(S.V, W);
            mode = kDense;
            if (S.C > 0 && 2 * n <= S.C) {
                __syncwarp();
                n = bitmap_to_list<kStaged>(A, R, S.D, W, S.LA);
                __syncwarp();
                if (n <= 32) {
                    mine = ((int)lane < n) ? S.LA[lane] : make_uint4(0, 0, 0, 0);
                    mode = kReg;
                } else {
                    mode = kList;
                }
            }
        }
        m = n;
        __syncwarp();
        return (flags & GBFSM_EDGE_ACCEPT) ? kAccept : kAlive;
    }

    // Start configuration: closure({start}).
    __device__ GBFSM_COLD int init_start() {
        const uint4 rec = state_record((uint32_t)A.start_state);
        if (S.C > 0 && !(rec.y & GBFSM_EDGE_HAS_EPS)) {
            mode = kReg;
            m = 1;
            mine = lane_id() == 0 ? rec : make_uint4(0, 0, 0, 0);
            return (rec.y & GBFSM_EDGE_ACCEPT) ? kAccept : kAlive;
        }
        const uint32_t s = rec.x;
        if (lane_id() == 0) {
            S.V[s >> 6] |= 1ull << (s & 63u);
            if (S.C > 0) S.LB[0] = rec;
        }
        __syncwarp();
        uint32_t info_or = rec.y;
        int n = 1;
        bool dense_now = S.C == 0;
        if (has_eps && !dense_now) n = sparse_closure<kStaged>(R, S.LB, n, S.C, S.V, info_or);
        if (n > S.C) dense_now = true;
        if (has_eps && dense_now) {
            __syncwarp();
            n += dense_closure<kStaged>(R, W, S.V, S.FA, S.FB, info_or);
        }
        return finish_general(n, dense_now, info_or);
    }

    __device__ GBFSM_COLD int step_general(uint32_t sym) {
        const uint32_t lane = lane_id();
        if (mode == kReg) {
            if (m <= S.C) {
                if ((int)lane < m) S.LA[lane] = mine;
                mode = kList;
            } else {  // more members than the list holds: spill to the bitmap
                if ((int)lane < m)
                    atomicOr(reinterpret_cast<unsigned long long *>(S.D + (mine.x >> 6)),
                             1ull << (mine.x & 63u));
                mode = kDense;
            }
            __syncwarp();
        }
        uint32_t info_or = 0;
        bool dense_now = mode == kDense;
        int n;
        if (!dense_now)
            n = sparse_expand<kStaged>(R, S.LA, m, sym, S.V, S.LB, S.C, info_or);
        else
            n = dense_expand<kStaged>(R, S.D, W, true, sym, R.sym_edges, R.sym_row, S.V, nullptr,
                                      info_or);
        if (n == 0) {  // reference.py:59-60: the set died
            if (dense_now) {
                __syncwarp();
                zero_words(S.D, W);
            }
            mode = kReg;
            m = 0;
            __syncwarp();
            return kDead;
        }
        __syncwarp();
        if (has_eps && (__reduce_or_sync(GBFSM_FULL_MASK, info_or) & GBFSM_EDGE_HAS_EPS)) {
            if (!dense_now && n <= S.C) n = sparse_closure<kStaged>(R, S.LB, n, S.C, S.V, info_or);
            if (dense_now || n > S.C) {
                __syncwarp();
                n += dense_closure<kStaged>(R, W, S.V, S.FA, S.FB, info_or);
                dense_now = true;
            }
        }
        if (n > S.C) dense_now = true;
        return finish_general(n, dense_now, info_or);
    }

    // REG-mode step: at most 32 members with at most 32 edges in total. The common case
    // (at most 4 members of at most 8 edges) gives each member 8 fixed lanes, so no scan
    // is needed to spread the edges; otherwise a warp scan flattens them.
    __device__ int step_reg(uint32_t sym) {
        const uint32_t lane = lane_id();
        const uint32_t deg = ((int)lane < m) ? mine.w - mine.z : 0u;
        uint4 rec = make_uint4(0, 0, 0, 0);
        bool have;
        if (m <= 4 && __ballot_sync(GBFSM_FULL_MASK, deg > 8u) == 0u) {
            const uint32_t mem = lane >> 3;
            const uint32_t rb = __shfl_sync(GBFSM_FULL_MASK, mine.z, mem);
            const uint32_t dg = __shfl_sync(GBFSM_FULL_MASK, deg, mem);
            have = (lane & 7u) < dg;  // dg is 0 for lanes past the last member
            if (have) rec = load_edge<kStaged>(R.sym_edges + rb + (lane & 7u));
        } else {
            const uint32_t incl = warp_inclusive_scan(deg);
            const uint32_t total = __shfl_sync(GBFSM_FULL_MASK, incl, 31);
            if (total > 32u) return step_general(sym);
            const uint32_t excl = incl - deg;
            uint32_t owner = 0;
#pragma unroll
            for (uint32_t step = 16; step >= 1; step >>= 1) {
                const uint32_t cand = owner + step;
                const uint32_t e = __shfl_sync(GBFSM_FULL_MASK, excl, cand);
                if (e <= lane) owner = cand;
            }
            const uint32_t orb = __shfl_sync(GBFSM_FULL_MASK, mine.z, owner);
            const uint32_t oex = __shfl_sync(GBFSM_FULL_MASK, excl, owner);
            have = lane < total;
            if (have) rec = load_edge<kStaged>(R.sym_edges + orb + (lane - oex));
        }
        bool match = false;
        if (have) {
            const uint32_t es = rec.y & GBFSM_EDGE_SYMBOL_MASK;
            match = (es == sym) || (es == GBFSM_ANY_SYMBOL);
        }
        const uint32_t key = match ? rec.x : 0xffffffffu;
        const uint32_t grp = __match_any_sync(GBFSM_FULL_MASK, key);
        const bool fresh = match && ((uint32_t)(__ffs(grp) - 1) == lane);
        const uint32_t F = __ballot_sync(GBFSM_FULL_MASK, fresh);
        const int n = __popc(F);
        if (n == 0) {  // reference.py:59-60
            m = 0;
            return kDead;
        }
        const uint32_t info = __reduce_or_sync(GBFSM_FULL_MASK, fresh ? rec.y : 0u);
        if (has_eps && (info & GBFSM_EDGE_HAS_EPS)) {
            // epsilon closure needed: continue through the shared-memory path
            if (fresh) {
                const int pos = __popc(F & lanemask_lt());
                if (pos < S.C) S.LB[pos] = rec;
                atomicOr(reinterpret_cast<unsigned long long *>(S.V + (rec.x >> 6)),
                         1ull << (rec.x & 63u));
            }
            __syncwarp();
            uint32_t info_or = fresh ? rec.y : 0u;
            int nn = n;
            bool dense_now = false;
            if (nn <= S.C) nn = sparse_closure<kStaged>(R, S.LB, nn, S.C, S.V, info_or);
            if (nn > S.C) {
                __syncwarp();
                nn += dense_closure<kStaged>(R, W, S.V, S.FA, S.FB, info_or);
                dense_now = true;
            }
            return finish_general(nn, dense_now, info_or);
        }
        // compact the new members into lanes 0..n-1 through the (32-slot) list buffer
        if (fresh) S.LB[__popc(F & lanemask_lt())] = rec;
        __syncwarp();
        mine = ((int)lane < n) ? S.LB[lane] : make_uint4(0, 0, 0, 0);
        __syncwarp();
        m = n;
        return (info & GBFSM_EDGE_ACCEPT) ? kAccept : kAlive;
    }

    __device__ __forceinline__ int step(uint32_t sym) {
        return mode == kReg ? step_reg(sym) : step_general(sym);
    }

    // Start from the set of records recs[rb .. re) (distinct states), closed under epsilon
    // edges: the speculative superset of a chunk (first_edges of one byte).
    __device__ GBFSM_COLD int init_records(const gbfsm_edge *recs, uint32_t rb, uint32_t re) {
        const uint32_t lane = lane_id();
        const uint32_t cnt = re - rb;
        if (cnt == 0) {
            mode = kReg;
            m = 0;
            return kDead;
        }
        if (cnt <= 32u && S.C > 0) {
            mine = (lane < cnt) ? load_edge<false>(recs + rb + lane) : make_uint4(0, 0, 0, 0);
            const uint32_t eps = __ballot_sync(GBFSM_FULL_MASK, lane < cnt && (mine.y & GBFSM_EDGE_HAS_EPS));
            const uint32_t acc = __ballot_sync(GBFSM_FULL_MASK, lane < cnt && (mine.y & GBFSM_EDGE_ACCEPT));
            if (!(has_eps && eps)) {
                mode = kReg;
                m = (int)cnt;
                return acc ? kAccept : kAlive;
            }
        }
        uint32_t info_or = 0;
        int n = walk_batch<false>(recs, lane == 0 ? rb : 0u, lane == 0 ? cnt : 0u, false, 0, S.V,
                                  S.LB, 0, S.C, nullptr, info_or);
        bool dense_now = n > S.C;
        if (has_eps && (__reduce_or_sync(GBFSM_FULL_MASK, info_or) & GBFSM_EDGE_HAS_EPS)) {
            if (!dense_now) n = sparse_closure<kStaged>(R, S.LB, n, S.C, S.V, info_or);
            if (dense_now || n > S.C) {
                __syncwarp();
                n += dense_closure<kStaged>(R, W, S.V, S.FA, S.FB, info_or);
                dense_now = true;
            }
        }
        return finish_general(n, dense_now, info_or);
    }

    // Start from the state records recs[0 .. count) (distinct states, already closed
    // under epsilon, count <= 32), e.g. a chunk's recorded final set.
    __device__ __forceinline__ void init_recs(const uint4 *recs, int count) {
        const uint32_t lane = lane_id();
        mine = ((int)lane < count) ? recs[lane] : make_uint4(0, 0, 0, 0);
        mode = kReg;
        m = count;
    }

    // Write the current members' records to out[0 .. m) if there are at most `cap` of
    // them and they are listed (REG or LIST); returns m, or -1 if not written.
    __device__ int export_recs(uint4 *out, int cap) const {
        const uint32_t lane = lane_id();
        if (m > cap || mode == kDense) return -1;
        if (mode == kReg) {
            if ((int)lane < m) out[lane] = mine;
        } else {
            for (int j = (int)lane; j < m; j += 32) out[j] = S.LA[j];
        }
        return m;
    }

    // Leave V, D, FA and FB all-zero for the next input.
    __device__ void cleanup() {
        __syncwarp();
        if (mode == kDense) {
            zero_words(S.D, W);
            zero_words(S.V, W);
        }
        mode = kReg;
        m = 0;
        __syncwarp();
    }
};

// Simulate one input with a whole warp. All lanes call it with identical arguments and
// all receive the verdict. `R` may point at shared-memory copies of the edge rows.
template <bool kStaged>
__device__ Verdict simulate_warp(const gbfsm_nfa_dev &A, const Rows &R, const uint8_t *in,
                                 int64_t len, WarpScratch S) {
    WarpNfa<kStaged> w(A, R, S);
    Verdict v{0, 0, 0};
    int ev = w.init_start();
    if (ev == kAccept) {
        v.flag = 1;
        w.cleanup();
        return v;
    }
    ByteStream bytes;
    bytes.init(in, len);
    int64_t pos = 0;
    v.examined = len;
    while (pos < len) {
        const uint32_t sym = bytes.next();
        ++pos;
        ev = w.step(sym);
        if (ev == kDead) {
            v.examined = pos;
            break;
        }
        if (ev == kAccept) {
            v.flag = 1;
            v.len = (int32_t)pos;
            v.examined = pos;
            break;
        }
    }
    w.cleanup();
    return v;
}

}  // namespace gbfsm
