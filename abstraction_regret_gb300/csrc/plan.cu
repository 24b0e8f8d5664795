// Device-side batch planning: the task queue of a batch built on the GPU from the inputs'
// offsets and automaton ids, so a step needs no host work between receiving a batch and
// its launches, and a captured graph re-plans every replay.
//
// plan_scan_kernel (one CTA of 1024 threads):
//   1. classify every input by its automaton's class (whole-input NFA, warp-chunked NFA,
//      lane-chunked NFA, DFA) and sum the bytes of the lane and warp classes;
//   2. choose the chunk sizes: DFA chunks of an input are max(its DFA's shortest chunk,
//      B / dfa_warps) bytes (B: the bytes of the DFA inputs holding two chunks of their
//      own minimum), so that a batch of few long inputs gets short chunks and a large
//      one a single wave of them; lane chunks get the smallest multiple of 64 bytes (at
//      least min_chunk) whose chunks fill at most one wave of the lane launch (32 chunks
//      per resident warp) -- found by an exponential then binary search, each probe a
//      block-wide sum; warp chunks get a power of two giving about four chunks per
//      resident warp of the persistent launch; with slices, the lane size of slice k of
//      P is scaled by 1 - shrink * k / P;
//   3. count each input's chunks, exclusive-scan the counts over the inputs in index
//      order (lane chunks first, then warp chunks, then the chunks of long DFA inputs),
//      place the FIXUP and DFA_FIXUP tasks in input
//      order, and histogram the persistent launch's tasks by log2 of their work (WHOLE
//      NFA inputs, warp chunks, groups of 32 DFA inputs) so that they can be queued
//      longest first, bucket by bucket;
//   4. write the header: counts, chunk sizes, the lane task range of each slice, and a
//      zeroed overflow counter.
// plan_fill_kernel (grid): a warp per input writes its FIXUP, DFA_FIXUP, CHUNK and WHOLE
//   tasks, its warp chunks and its input id; a thread per chunk writes the lane chunks and
//   the DFA chunks (with their tasks), finding its input by a binary search of the
//   inputs' chunk prefix counts, so that one long input's thousands of chunks do not
//   fall to one warp; then the sentinel chunk of index 0 after the last, the LANES tasks
//   (32 consecutive lane chunks each; every lane finds its own automaton) and the DFA
//   groups (32 consecutive DFA inputs of the length-bucketed order; every lane finds its
//   own DFA).
//
// The reference has no counterpart: it launches one kernel per automaton and per call
// with one thread or warp per whole input (src/gpufsm/backends/cuda/nfa.py:105-121).
#include "common.cuh"
#include "engine.hpp"

namespace gbfsm {
namespace {

constexpr int kPlanThreads = 1024;
constexpr int kBuckets = 64;
constexpr int kLaneGroup = 32;
constexpr int64_t kMaxChunk = 1 << 20;

// per-input scratch (int32 arrays of n entries) and per-bucket tables
struct PlanScratch {
    int32_t *cls;       // GBFSM_PLAN_* class of the input, or -1 (automaton out of range)
    int32_t *cnt;       // chunks of a split input (0: not split)
    int32_t *first;     // first chunk of a split input; slot of a whole NFA input
    int32_t *fix;       // FIXUP task slot of a split input
    int32_t *lpre;      // lane chunks of the inputs before i (n + 1 entries)
    int32_t *dpre;      // DFA chunks of the inputs before i (n + 1 entries)
    uint32_t *cursor;   // [kBuckets] WHOLE/CHUNK cursors, [kBuckets] DFA cursors
    int32_t *tbase;     // [kBuckets] first persistent slot of each work bucket
    int32_t *tdfa;      // [kBuckets] first persistent slot of each bucket's DFA groups
    int32_t *dbase;     // [kBuckets + 1] first DFA position of each bucket
};

size_t scratch_bytes(int32_t n) {
    return (size_t)4 * 4 * (size_t)n + 8 * ((size_t)n + 1) + 4 * (size_t)kBuckets * 2 +
           4 * (size_t)kBuckets * 2 + 4 * ((size_t)kBuckets + 1) + 256;
}

PlanScratch carve(void *p, int32_t n) {
    int32_t *w = static_cast<int32_t *>(p);
    PlanScratch s;
    s.cls = w;
    s.cnt = w + n;
    s.first = w + 2 * (size_t)n;
    s.fix = w + 3 * (size_t)n;
    s.lpre = w + 4 * (size_t)n;
    s.dpre = s.lpre + n + 1;
    s.cursor = reinterpret_cast<uint32_t *>(s.dpre + n + 1);
    s.tbase = reinterpret_cast<int32_t *>(s.cursor + 2 * kBuckets);
    s.tdfa = s.tbase + kBuckets;
    s.dbase = s.tdfa + kBuckets;
    return s;
}

__device__ __forceinline__ int bucket_of(int64_t w) {
    return 63 - __clzll((unsigned long long)(w > 0 ? w : 1));
}

struct InputInfo {
    int32_t aut;
    int32_t cls;
    int64_t start;
    int64_t len;
};

// Length of input i (an end before the start counts as empty).
__device__ __forceinline__ int64_t input_len(const gbfsm_batch_plan_args &a, int32_t i) {
    const int64_t e = a.ends ? a.ends[i] : a.offsets[i + 1];
    const int64_t l = e - a.offsets[i];
    return l > 0 ? l : 0;
}

__device__ __forceinline__ InputInfo input_info(const gbfsm_batch_plan_args &a, int32_t i) {
    InputInfo r;
    r.aut = a.aut_ids ? a.aut_ids[i] : 0;
    r.start = a.offsets[i];
    r.len = input_len(a, i);
    r.cls = (r.aut >= 0 && r.aut < a.n_automata) ? a.aut_class[r.aut] : -1;
    if (r.cls == GBFSM_PLAN_NFA_LANES && a.fixed_chunk < 0) r.cls = GBFSM_PLAN_NFA_WHOLE;
    if (r.cls == GBFSM_PLAN_NFA_WARP && a.fixed_chunk < 0) r.cls = GBFSM_PLAN_NFA_WHOLE;
    return r;
}

// Block-wide sum of an int64 (every thread gets the total).
__device__ int64_t block_sum(int64_t v, int64_t *red) {
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(GBFSM_FULL_MASK, v, d);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    int64_t t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0;
    if (w == 0)
        for (int d = 16; d > 0; d >>= 1) t += __shfl_xor_sync(GBFSM_FULL_MASK, t, d);
    if (threadIdx.x == 0) red[32] = t;
    __syncthreads();
    return red[32];
}

// Block-wide exclusive scan of K int64 values per thread (thread order); returns the
// totals in tot.
template <int K>
__device__ void block_scan(int64_t (&v)[K], int64_t (&tot)[K], int64_t *red) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    int64_t inc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        int64_t x = v[k];
        for (int d = 1; d < 32; d <<= 1) {
            const int64_t y = __shfl_up_sync(GBFSM_FULL_MASK, x, d);
            if (lane >= d) x += y;
        }
        inc[k] = x;
    }
    __syncthreads();
    if (lane == 31)
#pragma unroll
        for (int k = 0; k < K; ++k) red[k * 32 + w] = inc[k];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            int64_t x = lane < nw ? red[k * 32 + lane] : 0;
            for (int d = 1; d < 32; d <<= 1) {
                const int64_t y = __shfl_up_sync(GBFSM_FULL_MASK, x, d);
                if (lane >= d) x += y;
            }
            red[k * 32 + lane] = x;  // inclusive scan of the warp totals
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int64_t before = w > 0 ? red[k * 32 + w - 1] : 0;
        tot[k] = red[k * 32 + nw - 1];
        v[k] = before + inc[k] - v[k];
    }
    __syncthreads();
}

__device__ __forceinline__ int64_t chunks_of(int64_t len, int64_t size) {
    const int64_t c = (len + size - 1) / size;
    return c > 1 ? c : 1;
}

// Lane chunk size of input i: the base size, scaled for its slice.
__device__ __forceinline__ int64_t lane_size(const gbfsm_batch_plan_args &a, int64_t base,
                                             int32_t i) {
    if (a.n_slices <= 1 || a.fixed_chunk > 0) return base;
    int k = 0;
    while (k + 1 < a.n_slices && i >= a.slice_first[k + 1]) ++k;
    const double f = 1.0 - (double)a.shrink * (double)k / (double)a.n_slices;
    int64_t s = (int64_t)((double)base * f) / 64 * 64;
    return s > a.min_chunk ? s : a.min_chunk;
}

__global__ void __launch_bounds__(kPlanThreads) plan_scan_kernel(gbfsm_batch_plan_args a,
                                                                 PlanScratch s) {
    __shared__ int64_t red[6 * 32 + 1];
    __shared__ int32_t h_work[kBuckets], h_dfa[kBuckets], h_grp[kBuckets];
    __shared__ int32_t bad;
    const int32_t n = a.n_inputs;
    const int64_t per = ((int64_t)n + kPlanThreads - 1) / kPlanThreads;
    const int32_t lo = (int32_t)min((int64_t)n, (int64_t)threadIdx.x * per);
    const int32_t hi = (int32_t)min((int64_t)n, (int64_t)lo + per);
    for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) h_work[b] = h_dfa[b] = h_grp[b] = 0;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();

    // 1. classes and the bytes of the chunked classes
    int64_t lane_bytes = 0, warp_bytes = 0, dfa_bytes = 0, dfa_long = 0;
    for (int32_t i = lo; i < hi; ++i) {
        const InputInfo r = input_info(a, i);
        s.cls[i] = r.cls;
        if (r.cls < 0) bad = 1;
        if (r.cls == GBFSM_PLAN_NFA_LANES) lane_bytes += r.len;
        if (r.cls == GBFSM_PLAN_NFA_WARP) warp_bytes += r.len;
        if (r.cls == GBFSM_PLAN_DFA && a.aut_dfa_chunk) {
            const int64_t m = a.aut_dfa_chunk[r.aut];
            if (m > 0 && r.len >= 2 * m) {
                dfa_bytes += r.len;
                dfa_long += 1;
            }
        }
    }
    {  // the four totals in one block-wide pass
        int64_t v4[4] = {lane_bytes, warp_bytes, dfa_bytes, dfa_long}, t4[4];
        block_scan<4>(v4, t4, red);
        lane_bytes = t4[0];
        warp_bytes = t4[1];
        dfa_bytes = t4[2];
        dfa_long = t4[3];
    }
    // the batch's DFA chunk length (before each DFA's minimum): rounding each input up to
    // whole chunks adds at most one chunk per input, so B / (warps - inputs) keeps the
    // chunks within one wave
    int64_t dfa_target = 0;
    if (a.dfa_warps > 0 && dfa_bytes > 0) {
        const int64_t w = a.dfa_warps > dfa_long ? a.dfa_warps - dfa_long : 1;
        dfa_target = ((dfa_bytes + w - 1) / w + 63) / 64 * 64;
        if (dfa_target > (int64_t)1 << 30) dfa_target = (int64_t)1 << 30;
    }

    // 2. chunk sizes
    int64_t lane_base = a.min_chunk;
    if (a.fixed_chunk > 0) {
        lane_base = a.fixed_chunk > a.min_chunk ? a.fixed_chunk : a.min_chunk;
    } else if (lane_bytes > 0) {
        const int64_t target = (int64_t)kLaneGroup * (a.lane_warps > 0 ? a.lane_warps : 1);
        auto count = [&](int64_t size) {
            int64_t c = 0;
            for (int32_t i = lo; i < hi; ++i)
                if (s.cls[i] == GBFSM_PLAN_NFA_LANES) c += chunks_of(input_len(a, i), size);
            return block_sum(c, red);
        };
        int64_t start = ((lane_bytes + target - 1) / target + 63) / 64 * 64;
        if (start < a.min_chunk) start = a.min_chunk;
        if (start > kMaxChunk) start = kMaxChunk;
        if (count(start) <= target) {
            lane_base = start;
        } else {
            // exponential search for a size that fits, then binary search below it
            int64_t fail = start, step = 64, ok = -1;
            while (fail < kMaxChunk) {
                int64_t probe = fail + step;
                if (probe > kMaxChunk) probe = kMaxChunk;
                if (count(probe) <= target) {
                    ok = probe;
                    break;
                }
                fail = probe;
                step *= 2;
            }
            if (ok < 0) {
                lane_base = kMaxChunk;  // more than one wave even at the largest size
            } else {
                while (ok - fail > 64) {
                    const int64_t mid = fail + ((ok - fail) / 2 + 63) / 64 * 64;
                    const int64_t m = mid >= ok ? ok - 64 : mid;
                    if (count(m) <= target) ok = m;
                    else fail = m;
                }
                lane_base = ok;
            }
        }
    }
    int64_t warp_size = a.min_chunk;
    if (a.fixed_chunk > 0) {
        warp_size = lane_base;
    } else {
        const int64_t pw = 4 * (int64_t)(a.persist_warps > 0 ? a.persist_warps : 1);
        const int64_t per_w = warp_bytes / pw;
        int64_t p2 = 1;
        while (p2 * 2 <= per_w) p2 *= 2;
        warp_size = p2 > a.min_chunk ? p2 : a.min_chunk;
        if (warp_size > kMaxChunk) warp_size = kMaxChunk;
    }

    // 3. per-input counts, scans and bucket histograms
    // lane chunks, warp chunks, split NFA inputs, whole NFA inputs, DFA chunks, chunked
    // DFA inputs
    int64_t v[6] = {0, 0, 0, 0, 0, 0};
    for (int32_t i = lo; i < hi; ++i) {
        const int32_t c = s.cls[i];
        const int64_t len = input_len(a, i);
        int64_t cnt = 0;
        int64_t dfa_chunk = (c == GBFSM_PLAN_DFA && a.aut_dfa_chunk)
                                ? (int64_t)a.aut_dfa_chunk[a.aut_ids ? a.aut_ids[i] : 0]
                                : 0;
        if (dfa_chunk > 0 && dfa_target > dfa_chunk) dfa_chunk = dfa_target;
        if (c == GBFSM_PLAN_DFA && dfa_chunk > 0 && len >= 2 * dfa_chunk) {
            // a long DFA input: cut into chunks walked in parallel (DFA_CHUNK tasks)
            cnt = chunks_of(len, dfa_chunk);
            v[4] += cnt;
            v[5] += 1;
            s.cnt[i] = (int32_t)cnt;
            continue;
        }
        if (c == GBFSM_PLAN_NFA_LANES) {
            cnt = chunks_of(len, lane_size(a, lane_base, i));
            v[0] += cnt;
        } else if (c == GBFSM_PLAN_NFA_WARP && len >= 2 * warp_size) {
            cnt = chunks_of(len, warp_size);
            v[1] += cnt;
            atomicAdd(&h_work[bucket_of(4 * (len / cnt))], (int32_t)cnt);
        } else if (c == GBFSM_PLAN_NFA_WARP || c == GBFSM_PLAN_NFA_WHOLE) {
            v[3] += 1;
            atomicAdd(&h_work[bucket_of(4 * len)], 1);
        } else if (c == GBFSM_PLAN_DFA) {
            atomicAdd(&h_dfa[bucket_of(len)], 1);
        }
        s.cnt[i] = (int32_t)cnt;
        if (cnt > 0) v[2] += 1;
    }
    int64_t tot[6];
    int64_t ex[6] = {v[0], v[1], v[2], v[3], v[4], v[5]};
    block_scan<6>(ex, tot, red);
    const int64_t n_lane = tot[0], n_warp = tot[1], n_split = tot[2], n_whole = tot[3];
    const int64_t n_dfa_chunks = tot[4], n_dfa_split = tot[5];
    const int64_t n_chunks = n_lane + n_warp + n_dfa_chunks;
    for (int32_t i = lo; i < hi; ++i) {
        const int32_t c = s.cls[i];
        s.lpre[i] = (int32_t)ex[0];
        s.dpre[i] = (int32_t)ex[4];
        const int32_t cnt = s.cnt[i];
        if (cnt > 0 && c == GBFSM_PLAN_DFA) {
            s.first[i] = (int32_t)(n_lane + n_warp + ex[4]);
            ex[4] += cnt;
            s.fix[i] = (int32_t)ex[5];
            ex[5] += 1;
        } else if (cnt > 0) {
            if (c == GBFSM_PLAN_NFA_LANES) {
                s.first[i] = (int32_t)ex[0];
                ex[0] += cnt;
            } else {
                s.first[i] = (int32_t)(n_lane + ex[1]);
                ex[1] += cnt;
            }
            s.fix[i] = (int32_t)ex[2];
            ex[2] += 1;
        } else if (c == GBFSM_PLAN_NFA_WARP || c == GBFSM_PLAN_NFA_WHOLE) {
            s.first[i] = (int32_t)ex[3];
            ex[3] += 1;
        }
    }
    if (threadIdx.x == kPlanThreads - 1) {
        s.lpre[n] = (int32_t)n_lane;
        s.dpre[n] = (int32_t)n_dfa_chunks;
    }
    __syncthreads();

    // 4. bucket tables and the header (one warp)
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        if (lane == 0) {
            int32_t d = 0, t = 0;
            for (int b = kBuckets - 1; b >= 0; --b) {  // DFA positions, longest bucket first
                s.dbase[b] = d;
                const int32_t g0 = (d + kLaneGroup - 1) / kLaneGroup;
                d += h_dfa[b];
                h_grp[b] = (d + kLaneGroup - 1) / kLaneGroup - g0;
            }
            s.dbase[kBuckets] = d;
            for (int b = kBuckets - 1; b >= 0; --b) {  // persistent slots, longest first
                s.tbase[b] = t;
                s.tdfa[b] = t + h_work[b];
                t += h_work[b] + h_grp[b];
            }
            const int64_t n_lane_tasks = (n_lane + kLaneGroup - 1) / kLaneGroup;
            const bool over = n_chunks + 1 > a.cap_chunks || n_lane_tasks > a.cap_lane_tasks ||
                              t > a.cap_persist_tasks || n_split > a.cap_fixup_tasks ||
                              n_dfa_chunks > a.cap_dfa_chunk_tasks ||
                              n_dfa_split > a.cap_dfa_fixup_tasks ||
                              (n_dfa_chunks > 0 && (!a.tasks_dfa_chunk || !a.tasks_dfa_fixup)) ||
                              bad;
            int32_t *h = a.header;
            h[GBFSM_PLAN_STATUS] = bad ? 2 : over ? 1 : 0;
            h[GBFSM_PLAN_LANE_CHUNKS] = over ? 0 : (int32_t)n_lane;
            h[GBFSM_PLAN_CHUNKS] = over ? 0 : (int32_t)n_chunks;
            h[GBFSM_PLAN_LANE_FIRST] = 0;
            h[GBFSM_PLAN_LANE_TASKS] = over ? 0 : (int32_t)n_lane_tasks;
            h[GBFSM_PLAN_PERSIST_TASKS] = over ? 0 : t;
            h[GBFSM_PLAN_FIXUP_TASKS] = over ? 0 : (int32_t)n_split;
            h[GBFSM_PLAN_LANE_BYTES] = (int32_t)lane_base;
            h[GBFSM_PLAN_WARP_BYTES] = (int32_t)warp_size;
            h[GBFSM_PLAN_OVERFLOW] = 0;
            h[GBFSM_PLAN_WHOLE] = (int32_t)n_whole;
            h[GBFSM_PLAN_DFA_INPUTS] = d;
            h[GBFSM_PLAN_DFA_CHUNKS] = over ? 0 : (int32_t)n_dfa_chunks;
            h[GBFSM_PLAN_DFA_FIXUPS] = over ? 0 : (int32_t)n_dfa_split;
            h[GBFSM_PLAN_DFA_CHUNK_BYTES] = (int32_t)dfa_target;
            // lane task range of each slice: task t waits for the slice holding the input
            // of its last chunk, min(32 t + 31, n_lane - 1)
            const int ns = a.n_slices > 1 ? a.n_slices : 1;
            int32_t prev = 0;
            for (int k = 0; k < ns && k < GBFSM_PLAN_MAX_SLICES; ++k) {
                int32_t next = (int32_t)n_lane_tasks;
                if (k + 1 < ns) {
                    const int32_t ck = s.lpre[a.slice_first[k + 1]];
                    next = ck >= n_lane ? (int32_t)n_lane_tasks
                                        : (ck > 31 ? (ck - 31 + kLaneGroup - 1) / kLaneGroup : 0);
                }
                if (over) prev = next = 0;
                h[GBFSM_PLAN_SLICES + 2 * k] = prev;
                h[GBFSM_PLAN_SLICES + 2 * k + 1] = next - prev;
                prev = next;
            }
        }
        for (int b = lane; b < 2 * kBuckets; b += 32) s.cursor[b] = 0;
    }
}

// Chunk k of cnt of input i (bytes [st, st + len)): even cuts.
__device__ __forceinline__ gbfsm_chunk chunk_of(int32_t i, int32_t k, int32_t cnt, int64_t st,
                                                int64_t len) {
    gbfsm_chunk ch;
    ch.input = i;
    ch.index = k;
    ch.begin = st + (int64_t)k * len / cnt;
    ch.end = st + (int64_t)(k + 1) * len / cnt;
    return ch;
}

// The last input i in [0, n) with pre[i] <= c (pre: non-decreasing prefix counts).
__device__ __forceinline__ int32_t owner(const int32_t *pre, int32_t n, int32_t c) {
    int32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const int32_t mid = lo + (hi - lo + 1) / 2;
        if (pre[mid] <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(256) plan_fill_kernel(gbfsm_batch_plan_args a, PlanScratch s) {
    const int32_t *h = a.header;
    if (h[GBFSM_PLAN_STATUS] != 0) return;
    const int32_t n = a.n_inputs;
    const int32_t n_lane = h[GBFSM_PLAN_LANE_CHUNKS];
    const int32_t n_chunks = h[GBFSM_PLAN_CHUNKS];
    const int32_t n_whole = h[GBFSM_PLAN_WHOLE];
    const int32_t n_dfa = h[GBFSM_PLAN_DFA_INPUTS];
    gbfsm_task *tl = a.tasks_lanes, *tp = a.tasks_persist, *tf = a.tasks_fixup;
    const uint32_t lane = lane_id();
    const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i64 = gwarp; i64 < n; i64 += nwarps) {
        const int32_t i = (int32_t)i64;
        const int32_t c = s.cls[i];
        const int32_t aut = a.aut_ids ? a.aut_ids[i] : 0;
        const int64_t st = a.offsets[i];
        const int64_t len = input_len(a, i);
        const int32_t cnt = s.cnt[i];
        if (cnt > 0 && c == GBFSM_PLAN_DFA) {  // a long DFA input (its chunks: below)
            if (lane == 0) {
                a.tasks_dfa_fixup[s.fix[i]] =
                    gbfsm_task{aut, s.first[i], cnt, GBFSM_TASK_DFA_FIXUP};
                if (a.dfa_latch) a.dfa_latch[i] = INT32_MAX;
            }
        } else if (cnt > 0 && c == GBFSM_PLAN_NFA_LANES) {  // lane chunks: below
            if (lane == 0) tf[s.fix[i]] = gbfsm_task{aut, s.first[i], cnt, GBFSM_TASK_FIXUP};
        } else if (cnt > 0) {  // warp chunks, each with its CHUNK task
            const int32_t f = s.first[i];
            int32_t slot0 = 0;
            if (lane == 0)
                slot0 = (int32_t)atomicAdd(&s.cursor[bucket_of(4 * (len / cnt))], (uint32_t)cnt);
            slot0 = __shfl_sync(GBFSM_FULL_MASK, slot0, 0);
            const int b = bucket_of(4 * (len / cnt));
            for (int32_t k = (int32_t)lane; k < cnt; k += 32) {
                a.chunks[f + k] = chunk_of(i, k, cnt, st, len);
                tp[s.tbase[b] + slot0 + k] = gbfsm_task{aut, f + k, 1, GBFSM_TASK_CHUNK};
            }
            if (lane == 0) tf[s.fix[i]] = gbfsm_task{aut, f, cnt, GBFSM_TASK_FIXUP};
        } else if (c == GBFSM_PLAN_NFA_WARP || c == GBFSM_PLAN_NFA_WHOLE) {
            if (lane == 0) {
                const int b = bucket_of(4 * len);
                const int32_t slot = (int32_t)atomicAdd(&s.cursor[b], 1u);
                const int32_t pos = s.first[i];
                a.input_ids[pos] = i;
                tp[s.tbase[b] + slot] = gbfsm_task{aut, pos, 1, GBFSM_TASK_WHOLE};
            }
        } else if (c == GBFSM_PLAN_DFA) {
            if (lane == 0) {
                const int b = bucket_of(len);
                const int32_t pos = s.dbase[b] + (int32_t)atomicAdd(&s.cursor[kBuckets + b], 1u);
                a.input_ids[n_whole + pos] = i;
            }
        }
    }
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    // lane chunks: chunk c of the lane region belongs to the last input i with
    // lpre[i] <= c (inputs without lane chunks share their successor's prefix)
    for (int64_t c = tid; c < n_lane; c += nthreads) {
        const int32_t i = owner(s.lpre, n, (int32_t)c);
        const int32_t k = (int32_t)c - s.lpre[i];
        a.chunks[c] = chunk_of(i, k, s.cnt[i], a.offsets[i], input_len(a, i));
    }
    // DFA chunks (after the lane and warp chunks), each with its DFA_CHUNK task
    const int32_t n_dfa_chunks = h[GBFSM_PLAN_DFA_CHUNKS];
    const int32_t dfa_base = n_chunks - n_dfa_chunks;
    for (int64_t c = tid; c < n_dfa_chunks; c += nthreads) {
        const int32_t i = owner(s.dpre, n, (int32_t)c);
        const int32_t k = (int32_t)c - s.dpre[i];
        const int32_t aut = a.aut_ids ? a.aut_ids[i] : 0;
        a.chunks[dfa_base + c] = chunk_of(i, k, s.cnt[i], a.offsets[i], input_len(a, i));
        a.tasks_dfa_chunk[c] = gbfsm_task{aut, dfa_base + (int32_t)c, 1, GBFSM_TASK_DFA_CHUNK};
    }
    if (tid == 0 && n_chunks < a.cap_chunks) {  // sentinel: no next chunk of the same input
        gbfsm_chunk z;
        z.input = -1;
        z.index = 0;
        z.begin = z.end = 0;
        a.chunks[n_chunks] = z;
    }
    // LANES tasks: 32 consecutive lane chunks each, each lane finding its own automaton
    const int32_t n_lt = (n_lane + kLaneGroup - 1) / kLaneGroup;
    for (int64_t t = tid; t < n_lt; t += nthreads) {
        const int32_t first = (int32_t)t * kLaneGroup;
        tl[t] = gbfsm_task{-1, first, min(kLaneGroup, n_lane - first), GBFSM_TASK_LANES};
    }
    // DFA groups: 32 consecutive positions of the bucketed DFA order
    const int32_t n_groups = (n_dfa + kLaneGroup - 1) / kLaneGroup;
    for (int64_t g = tid; g < n_groups; g += nthreads) {
        const int32_t p = (int32_t)g * kLaneGroup;
        int b = kBuckets - 1;
        while (b > 0 && p >= s.dbase[b - 1]) --b;  // bucket b holds [dbase[b], dbase[b-1])
        const int32_t g_first = (s.dbase[b] + kLaneGroup - 1) / kLaneGroup;
        tp[s.tdfa[b] + ((int32_t)g - g_first)] =
            gbfsm_task{-1, n_whole + p, min(kLaneGroup, n_dfa - p), GBFSM_TASK_DFA_GROUP};
    }
}

}  // namespace

size_t batch_plan_scratch_bytes(int32_t n_inputs) {
    return n_inputs < 0 ? 0 : scratch_bytes(n_inputs);
}

gbfsm_status launch_batch_plan(const gbfsm_batch_plan_args &a, cudaStream_t stream) {
    const PlanScratch s = carve(a.scratch, a.n_inputs);
    plan_scan_kernel<<<1, kPlanThreads, 0, stream>>>(a, s);
    GBFSM_LAUNCH_CHECK("plan_scan_kernel launch");
    int grid = (a.n_inputs + 7) / 8;  // 8 warps per CTA, a warp per input
    const int cap = sm_count() * 4;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    plan_fill_kernel<<<grid, 256, 0, stream>>>(a, s);
    GBFSM_LAUNCH_CHECK("plan_fill_kernel launch");
    return GBFSM_OK;
}

}  // namespace gbfsm
