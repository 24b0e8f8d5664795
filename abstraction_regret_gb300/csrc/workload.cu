// Synthetic input generator for the "live" workload variants (host code; no device work).
//
// Uniform random bytes kill a random NFA within a byte or two (a set of k states
// survives a byte with probability about k * degree / 256), so the literal benchmark
// configurations barely exercise a simulator. A live input is instead a random walk
// through the automaton's "live core": the largest set of non-accepting states in which
// every state has a symbol edge to another state of the set (found by pruning states
// without such an edge until nothing changes, over reverse edges). At each position the
// walk state picks, uniformly, one of its symbol edges into the core, emits that edge's
// label (a uniform byte for an ANY edge) and moves to the target. A walk that starts
// outside the core, or an automaton whose core is empty, gives uniform random bytes.
// The simulated active set therefore always contains the walk state until the input
// ends or an accepting state is reached through other members of the set.
//
// Randomness: SplitMix64 (Steele, Lea & Flood, OOPSLA 2014) seeded per input from
// (seed, input index), so the bytes are identical on every host and thread count.
#include <stdint.h>

#include <thread>
#include <vector>

#include "../../include/gbfsm.h"

namespace {

struct SplitMix64 {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    // uniform in [0, n) for n >= 1 (multiply-shift; bias below 2^-32 for n < 2^32)
    uint32_t below(uint32_t n) { return (uint32_t)(((next() >> 32) * (uint64_t)n) >> 32); }
};

// live[s] = 1 for the states of the live core (see above).
std::vector<uint8_t> live_core(int32_t n, const int32_t *srp, const int32_t *stg,
                               const uint8_t *accept) {
    std::vector<uint8_t> live((size_t)n, 1);
    std::vector<int32_t> count((size_t)n, 0), rrow((size_t)n + 1, 0), rsrc, queue;
    const int32_t nnz = srp[n];
    for (int32_t k = 0; k < nnz; ++k)
        if (stg[k] >= 0 && stg[k] < n) ++rrow[(size_t)stg[k] + 1];
    for (int32_t s = 0; s < n; ++s) rrow[(size_t)s + 1] += rrow[s];
    rsrc.resize((size_t)rrow[n]);
    std::vector<int32_t> fill(rrow.begin(), rrow.end() - 1);
    for (int32_t s = 0; s < n; ++s)
        for (int32_t k = srp[s]; k < srp[s + 1]; ++k) {
            const int32_t t = stg[k];
            if (t < 0 || t >= n) continue;
            rsrc[(size_t)fill[t]++] = s;
            if (!accept[t]) ++count[s];
        }
    for (int32_t s = 0; s < n; ++s)
        if (accept[s] || count[s] == 0) {
            live[s] = 0;
            queue.push_back(s);
        }
    // a state that dies removes one candidate edge from each predecessor per edge into it
    for (size_t q = 0; q < queue.size(); ++q) {
        const int32_t t = queue[q];
        if (accept[t]) continue;  // edges into accepting states were never counted
        for (int32_t r = rrow[t]; r < rrow[t + 1]; ++r) {
            const int32_t s = rsrc[(size_t)r];
            if (live[s] && --count[s] == 0) {
                live[s] = 0;
                queue.push_back(s);
            }
        }
    }
    return live;
}

void walk_one(int32_t n, const int32_t *srp, const int32_t *stg, const int32_t *ssy,
              const uint8_t *live, int32_t start, uint8_t *out, int64_t len, SplitMix64 &rng,
              std::vector<int32_t> &good) {
    int32_t s = start;
    int64_t i = 0;
    for (; i < len && live[s]; ++i) {
        good.clear();
        for (int32_t k = srp[s]; k < srp[s + 1]; ++k) {
            const int32_t t = stg[k];
            if (t >= 0 && t < n && live[t]) good.push_back(k);
        }
        if (good.empty()) break;
        const int32_t k = good[rng.below((uint32_t)good.size())];
        const int32_t sym = ssy[k];
        out[i] = (sym >= 0 && sym <= 255) ? (uint8_t)sym : (uint8_t)(rng.next() & 0xffu);
        s = stg[k];
    }
    for (; i < len; ++i) out[i] = (uint8_t)(rng.next() & 0xffu);
}

}  // namespace

extern "C" int32_t gbfsm_workload_walk(int32_t num_states, const int32_t *sym_row_ptr,
                                       const int32_t *sym_targets, const int32_t *sym_symbols,
                                       const uint8_t *accept, int32_t start_state,
                                       const int64_t *offsets, int32_t n_inputs, uint64_t seed,
                                       uint8_t *out, int32_t n_threads) {
    if (num_states < 1 || start_state < 0 || start_state >= num_states || n_inputs < 0 ||
        !sym_row_ptr || !accept || !offsets || !out)
        return GBFSM_INVALID_ARG;
    if (n_threads < 1) n_threads = 1;
    const std::vector<uint8_t> live = live_core(num_states, sym_row_ptr, sym_targets, accept);
    const uint8_t *live_p = live.data();
    std::vector<std::thread> pool;
    for (int32_t t = 0; t < n_threads; ++t) {
        pool.emplace_back([=]() {
            std::vector<int32_t> good;
            for (int32_t i = t; i < n_inputs; i += n_threads) {
                SplitMix64 rng{seed * 0x100000001b3ull ^ (uint64_t)(i + 1) * 0x9e3779b97f4a7c15ull};
                walk_one(num_states, sym_row_ptr, sym_targets, sym_symbols, live_p, start_state,
                         out + offsets[i], offsets[i + 1] - offsets[i], rng, good);
            }
        });
    }
    for (auto &th : pool) th.join();
    return GBFSM_OK;
}
