// Persistent batched engine: one launch for many inputs of uneven length over many
// automata (NFAs and DFAs) of different sizes.
//
// The grid is sized to the resident capacity (SMs x CTAs per SM from the occupancy
// calculator). Each warp pops tasks from a device queue with one atomicAdd ticket per
// task, in the order the host gave them (longest first, so the longest serial chains
// start first), until the queue is empty:
//   - an NFA task (one input) is simulated by the whole warp with the automaton's own
//     technique (dense bitmap or sparse list) from the device automaton table;
//   - a DFA task (1..32 inputs of one DFA) runs one table walk per lane.
// Per-warp scratch: the dedup bitmap V and the two member lists in shared memory, sized
// for the largest NFA of the launch; the dense buffers (D, FA, FB) in a global workspace
// slice per resident warp. The reference has no counterpart: it launches one kernel per
// automaton and per batch (src/gpufsm/backends/cuda/nfa.py:105-121).
#include <map>
#include <mutex>
#include <tuple>

#include "common.cuh"
#include "dfa_device.cuh"
#include "engine.hpp"
#include "nfa_device.cuh"

namespace gbfsm {
namespace {

constexpr int kPersistThreads = 256;  // 8 warps per CTA by default
// CTAs of kPersistThreads per SM the register allocation must allow (the per-byte loop is
// latency-bound: more resident warps means more chains in flight).
#ifndef GBFSM_PERSIST_MIN_BLOCKS
#define GBFSM_PERSIST_MIN_BLOCKS 2
#endif
constexpr int kPersistMinBlocks = GBFSM_PERSIST_MIN_BLOCKS;

struct PersistLayout {
    int Wmax;
    int C;
    int wpc;
    uint32_t smem_per_warp;
    uint32_t wbytes;
    size_t global_per_warp;
};

PersistLayout persist_layout(int32_t max_words, const gbfsm_plan &p) {
    PersistLayout L;
    L.Wmax = max_words > 0 ? max_words : 1;
    L.C = p.list_capacity > 0 ? p.list_capacity : kDefaultListCapacity;
    const int threads = p.block_threads > 0 ? p.block_threads : kPersistThreads;
    L.wpc = threads / 32;
    L.wbytes = pad16((uint64_t)L.Wmax * 8u);
    L.smem_per_warp = L.wbytes + 32u * (uint32_t)max(L.C, 32);
    L.global_per_warp = 3u * (size_t)L.wbytes;
    return L;
}

// Outcome of one chunk (GBFSM_CHUNK_RECORD_BYTES bytes). Positions are byte counts from
// the start of the chunk's input. For a speculative chunk the set sizes are recorded
// after 1, 2, 4, ..., 32 bytes of the chunk; acc_after[c] is the first accepting position
// strictly after checkpoint c (-1: none before the run stopped), dead_at the position at
// which the (superset) run died. For an input's first chunk (exact) acc_after[0] /
// dead_at are the input's own first accept / death. end_ids lists the set at the chunk
// end when the run got there with at most kEndCap members (end_count, else -1).
constexpr int kCheckpoints = 6;
constexpr int kEndCap = 32;
struct ChunkRecord {
    int32_t counts[kCheckpoints];
    int32_t acc_after[kCheckpoints];
    int32_t dead_at;
    int32_t end_count;
    int32_t pad[2];
    uint32_t end_ids[kEndCap];
};
static_assert(sizeof(ChunkRecord) == GBFSM_CHUNK_RECORD_BYTES, "chunk record layout");

__device__ __forceinline__ uint32_t byte_at(const uint8_t *p) { return __ldg(p); }

// CHUNK task: run one chunk (exactly when it is the input's first) and record it.
__device__ void run_chunk(const gbfsm_nfa_dev &nfa, const Rows &R, WarpScratch S,
                          const uint8_t *base, int64_t b, int64_t e, int index,
                          ChunkRecord *rec) {
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
        // superset of the true set after byte b-2, then one step on byte b-1
        const uint32_t c0 = byte_at(base + b - 2);
        ev = w.init_records(nfa.first_edges, __ldg(nfa.first_row + c0), __ldg(nfa.first_row + c0 + 1));
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
        if (index == 0) {
            if (ev == kDead) {
                dead_at = pos;
                stopped = true;
            } else if (ev == kAccept) {
                acc_after[0] = pos;
                stopped = true;
            }
            continue;
        }
        if (ev == kDead) {
            dead_at = pos;
            stopped = true;
            break;
        }
        if (ev == kAccept) {
#pragma unroll
            for (int c = 0; c < kCheckpoints; ++c)
                if (j > (1 << c) && acc_after[c] < 0) acc_after[c] = pos;
            if (j > (1 << (kCheckpoints - 1))) stopped = true;  // first accept after the last checkpoint
        }
        if (j <= (1 << (kCheckpoints - 1)) && (j & (j - 1)) == 0) counts[31 - __clz((int)j)] = w.m;
    }
    int32_t end_count = -1;
    if (!stopped) end_count = w.export_ids(rec->end_ids, kEndCap);
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < kCheckpoints; ++c) {
            rec->counts[c] = counts[c];
            rec->acc_after[c] = acc_after[c];
        }
        rec->dead_at = dead_at;
        rec->end_count = end_count;
    }
    w.cleanup();
}

// FIXUP task: resolve an input from its chunk records, re-running each chunk exactly only
// until its exact set has as many members as the speculative superset at a checkpoint
// (the superset contains the exact set, so equal sizes mean equal sets, and the rest of
// the chunk is the recorded run).
__device__ Verdict run_fixup(const gbfsm_nfa_dev &nfa, const Rows &R, WarpScratch S,
                             const uint8_t *base, int64_t len, const gbfsm_chunk *chunks,
                             const ChunkRecord *recs, int first, int count, int64_t input_off) {
    Verdict v{0, 0, len};
    const ChunkRecord &r0 = recs[first];
    if (r0.acc_after[0] >= 0) {
        v.flag = 1;
        v.len = r0.acc_after[0];
        v.examined = r0.acc_after[0];
        return v;
    }
    if (r0.dead_at >= 0) {
        v.examined = r0.dead_at;
        return v;
    }
    WarpNfa<false> w(nfa, R, S);
    if (r0.end_count >= 0) {
        w.init_ids(r0.end_ids, r0.end_count);
    } else {  // the first chunk's end set was not recorded: recompute it exactly
        w.init_start();
        const int64_t e0 = chunks[first].end - input_off;
        for (int64_t p = 0; p < e0; ++p) w.step(byte_at(base + p));
    }
    for (int k = 1; k < count; ++k) {
        const gbfsm_chunk ch = chunks[first + k];
        const ChunkRecord &rk = recs[first + k];
        const int64_t b = ch.begin - input_off, e = ch.end - input_off;
        int matched = -1;
        int64_t j = 0;
        while (b + j < e) {
            const int ev = w.step(byte_at(base + b + j));
            ++j;
            if (ev == kDead) {
                v.examined = b + j;
                w.cleanup();
                return v;
            }
            if (ev == kAccept) {
                v.flag = 1;
                v.len = (int32_t)(b + j);
                v.examined = b + j;
                w.cleanup();
                return v;
            }
            if (matched < 0 && j <= (1 << (kCheckpoints - 1)) && (j & (j - 1)) == 0 &&
                w.m == rk.counts[31 - __clz((int)j)]) {
                matched = 31 - __clz((int)j);
                break;
            }
        }
        if (matched >= 0) {
            if (rk.acc_after[matched] >= 0) {
                v.flag = 1;
                v.len = rk.acc_after[matched];
                v.examined = rk.acc_after[matched];
                w.cleanup();
                return v;
            }
            if (rk.dead_at >= 0) {
                v.examined = rk.dead_at;
                w.cleanup();
                return v;
            }
            if (rk.end_count >= 0) {
                w.cleanup();
                w.init_ids(rk.end_ids, rk.end_count);
            } else {
                while (b + j < e) w.step(byte_at(base + b + j++));  // no event can occur here
            }
        }
    }
    w.cleanup();
    return v;
}

// LANES task body: one chunk per lane, the set held in registers (at most kLaneCap
// members: id and edge-row range each). Same protocol and record as run_chunk; a chunk
// whose set outgrows the lane returns false without writing its record. The first step
// of a speculative chunk starts from the two-byte superset pair_edges of the bytes
// before it; each step scans a member's edge labels (edge_sym, uint16) and loads the
// 16-byte record only of an edge that matches.
constexpr int kLaneCap = 8;    // members a lane holds
constexpr int kLaneMatch = 8;  // matching edges a lane handles per byte

__device__ bool run_chunk_lane(const gbfsm_nfa_dev &A, const uint8_t *base, int64_t b, int64_t e,
                               int index, ChunkRecord *rec) {
    uint32_t ct[kLaneCap], crb[kLaneCap], cre[kLaneCap];
    int m = 0;
    int32_t counts[kCheckpoints], acc_after[kCheckpoints];
#pragma unroll
    for (int c = 0; c < kCheckpoints; ++c) {
        counts[c] = 0;
        acc_after[c] = -1;
    }
#pragma unroll
    for (int i = 0; i < kLaneCap; ++i) ct[i] = crb[i] = cre[i] = 0;
    int32_t dead_at = -1;
    bool stopped = false;
    if (index == 0) {
        const uint32_t s = (uint32_t)A.start_state;
        ct[0] = s;
        crb[0] = __ldg(A.sym_row + s);
        cre[0] = __ldg(A.sym_row + s + 1);
        m = 1;
        if ((__ldg(reinterpret_cast<const unsigned long long *>(A.accept_words) + (s >> 6)) >>
             (s & 63u)) & 1ull) {
            acc_after[0] = 0;
            stopped = true;
        }
    } else {
        const uint32_t key = (uint32_t)__ldg(base + b - 2) * 256u + (uint32_t)__ldg(base + b - 1);
        const uint32_t pr = __ldg(A.pair_row + key), pe = __ldg(A.pair_row + key + 1);
        if (pe - pr > (uint32_t)kLaneCap) return false;
        m = (int)(pe - pr);
#pragma unroll
        for (int i = 0; i < kLaneCap; ++i) {
            if (i < m) {
                const uint4 r = ld_edge(A.pair_edges + pr + i);
                ct[i] = r.x;
                crb[i] = r.z;
                cre[i] = r.w;
            }
        }
        if (m == 0) {
            dead_at = (int32_t)b;
            stopped = true;
        }
    }
    const int64_t len = e - b;
    ByteStream bytes;
    bytes.init(base + b, stopped ? 0 : len);
    int64_t j = 0;
    while (!stopped && j < len) {
        const uint32_t sym = bytes.next();
        ++j;
        // 1. scan the members' edge labels (L1-resident uint16) for this byte, keeping the
        //    indices of at most kLaneMatch matching edges
        uint32_t mk[kLaneMatch];
        int nm = 0;
#pragma unroll
        for (int q = 0; q < kLaneMatch; ++q) mk[q] = 0;
#pragma unroll
        for (int i = 0; i < kLaneCap; ++i) {
            if (i < m) {
                const uint32_t kb = crb[i], ke = cre[i];
#pragma unroll 4
                for (uint32_t k = kb; k < ke; ++k) {
                    const uint32_t es = __ldg(A.edge_sym + k);
                    if (es == sym || es == (uint32_t)GBFSM_ANY_SYMBOL) {
#pragma unroll
                        for (int q = 0; q < kLaneMatch; ++q)
                            if (q == nm) mk[q] = k;
                        ++nm;
                    }
                }
            }
        }
        if (nm > kLaneMatch) return false;
        // 2. load the matching edges' records together (one L2 round trip per byte)
        uint4 rr[kLaneMatch];
#pragma unroll
        for (int q = 0; q < kLaneMatch; ++q)
            rr[q] = (q < nm) ? ld_edge(A.sym_edges + mk[q]) : make_uint4(0, 0, 0, 0);
        // 3. deduplicate the targets into the next set
        uint32_t nt[kLaneCap], nrb[kLaneCap], nre[kLaneCap];
        int n = 0;
        bool acc = false, ovf = false;
#pragma unroll
        for (int q = 0; q < kLaneMatch; ++q) {
            if (q < nm) {
                const uint4 r = rr[q];
                bool dup = false;
#pragma unroll
                for (int u = 0; u < q; ++u) dup |= (rr[u].x == r.x);
                if (!dup) {
                    if (n == kLaneCap) {
                        ovf = true;
                    } else {
#pragma unroll
                        for (int u = 0; u < kLaneCap; ++u) {
                            if (u == n) {
                                nt[u] = r.x;
                                nrb[u] = r.z;
                                nre[u] = r.w;
                            }
                        }
                        ++n;
                        acc |= (r.y & GBFSM_EDGE_ACCEPT) != 0;
                    }
                }
            }
        }
        if (ovf) return false;
#pragma unroll
        for (int q = 0; q < kLaneCap; ++q) {
            ct[q] = nt[q];
            crb[q] = nrb[q];
            cre[q] = nre[q];
        }
        m = n;
        const int32_t pos = (int32_t)(b + j);
        if (index == 0) {
            if (m == 0) {
                dead_at = pos;
                stopped = true;
            } else if (acc) {
                acc_after[0] = pos;
                stopped = true;
            }
            continue;
        }
        if (m == 0) {
            dead_at = pos;
            stopped = true;
            break;
        }
        if (acc) {
#pragma unroll
            for (int c = 0; c < kCheckpoints; ++c)
                if (j > (1 << c) && acc_after[c] < 0) acc_after[c] = pos;
            if (j > (1 << (kCheckpoints - 1))) stopped = true;
        }
        if (j <= (1 << (kCheckpoints - 1)) && (j & (j - 1)) == 0) {
            const int c = 31 - __clz((int)j);
#pragma unroll
            for (int q = 0; q < kCheckpoints; ++q)
                if (q == c) counts[q] = m;
        }
    }
#pragma unroll
    for (int c = 0; c < kCheckpoints; ++c) {
        rec->counts[c] = counts[c];
        rec->acc_after[c] = acc_after[c];
    }
    rec->dead_at = dead_at;
    rec->end_count = stopped ? -1 : m;
    if (!stopped) {
#pragma unroll
        for (int q = 0; q < kLaneCap; ++q)
            if (q < m) rec->end_ids[q] = ct[q];
    }
    return true;
}

// Device pointers of the chunk machinery, passed by value to the kernel.
struct ChunkIO {
    const gbfsm_chunk *chunks;
    ChunkRecord *records;
    gbfsm_task *overflow_tasks;
    int32_t *overflow_count;
    const int32_t *task_count;
};

__global__ void __launch_bounds__(kMaxBlockThreads, kPersistMinBlocks) persistent_kernel(
    const gbfsm_automaton *__restrict__ table, const gbfsm_task *__restrict__ tasks,
    int32_t n_tasks, const int32_t *__restrict__ input_ids, const uint8_t *__restrict__ data,
    const int64_t *__restrict__ offsets, const int64_t *__restrict__ ends, ChunkIO io,
    int32_t *flags, int32_t *lens, int32_t *examined, PersistLayout L, uint32_t *ticket,
    uint8_t *gws) {
    const gbfsm_chunk *__restrict__ chunks = io.chunks;
    ChunkRecord *records = io.records;
    if (io.task_count) n_tasks = min(n_tasks, *io.task_count);
    extern __shared__ __align__(16) uint8_t smem[];
    const int warp = (int)(threadIdx.x >> 5);
    const uint32_t lane = lane_id();
    const size_t slot = (size_t)blockIdx.x * L.wpc + warp;
    uint8_t *sp = smem + (size_t)warp * L.smem_per_warp;
    uint8_t *gp = gws + slot * L.global_per_warp;
    WarpScratch S;
    S.V = reinterpret_cast<uint64_t *>(sp);
    S.LA = reinterpret_cast<uint4 *>(sp + L.wbytes);
    S.LB = S.LA + max(L.C, 32);
    S.D = reinterpret_cast<uint64_t *>(gp);
    S.FA = reinterpret_cast<uint64_t *>(gp + L.wbytes);
    S.FB = reinterpret_cast<uint64_t *>(gp + 2 * L.wbytes);
    zero_words(S.V, L.Wmax);
    zero_words(S.D, L.Wmax);
    zero_words(S.FA, L.Wmax);
    zero_words(S.FB, L.Wmax);
    __syncwarp();

    for (;;) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(ticket, 1u);
        t = __shfl_sync(GBFSM_FULL_MASK, t, 0);
        if (t >= (uint32_t)n_tasks) break;
        const gbfsm_task task = tasks[t];
        const gbfsm_automaton *A = table + task.automaton;
        if (A->kind == 0) {
            const gbfsm_nfa_dev nfa = A->nfa;
            Rows R;
            R.sym_row = nfa.sym_row;
            R.sym_edges = nfa.sym_edges;
            R.eps_row = nfa.eps_row;
            R.eps_edges = nfa.eps_edges;
            S.C = (A->technique == GBFSM_TECH_WARP) ? 0 : min(A->list_capacity, L.C);
            if (task.kind == GBFSM_TASK_LANES) {
                if ((int)lane < task.count) {
                    const int cid = task.first + (int)lane;
                    const gbfsm_chunk ch = chunks[cid];
                    const int64_t off = offsets[ch.input];
                    if (!run_chunk_lane(nfa, data + off, ch.begin - off, ch.end - off, ch.index,
                                        records + cid)) {
                        const int slot = atomicAdd(io.overflow_count, 1);
                        gbfsm_task spill;
                        spill.automaton = task.automaton;
                        spill.first = cid;
                        spill.count = 1;
                        spill.kind = GBFSM_TASK_CHUNK;
                        io.overflow_tasks[slot] = spill;
                    }
                }
                __syncwarp();
                continue;
            }
            if (task.kind == GBFSM_TASK_CHUNK) {
                const gbfsm_chunk ch = chunks[task.first];
                const int64_t off = offsets[ch.input];
                if (S.C == 0) S.C = min(L.C, 32);  // speculation keeps small sets listed
                run_chunk(nfa, R, S, data + off, ch.begin - off, ch.end - off, ch.index,
                          records + task.first);
                continue;
            }
            if (task.kind == GBFSM_TASK_FIXUP) {
                const int32_t id = chunks[task.first].input;
                const int64_t off = offsets[id];
                const int64_t e = ends ? ends[id] : offsets[id + 1];
                if (S.C == 0) S.C = min(L.C, 32);
                const Verdict v = run_fixup(nfa, R, S, data + off, e - off, chunks, records,
                                            task.first, task.count, off);
                if (lane == 0) {
                    flags[id] = v.flag;
                    lens[id] = v.len;
                    if (examined) examined[id] = (int32_t)v.examined;
                }
                continue;
            }
            const int32_t id = input_ids[task.first];
            const int64_t b = offsets[id];
            const int64_t e = ends ? ends[id] : offsets[id + 1];
            const Verdict v = simulate_warp<false>(nfa, R, data + b, e - b, S);
            if (lane == 0) {
                flags[id] = v.flag;
                lens[id] = v.len;
                if (examined) examined[id] = (int32_t)v.examined;
            }
        } else {
            const gbfsm_dfa_dev d = A->dfa;
            if ((int)lane < task.count) {
                const int32_t id = input_ids[task.first + (int)lane];
                const int64_t b = offsets[id];
                const int64_t e = ends ? ends[id] : offsets[id + 1];
                int32_t f, l;
                int64_t ex;
                if (d.entry_bytes == 2)
                    dfa_walk<uint16_t, false>(static_cast<const uint16_t *>(d.table), d.accept_bits,
                                              (uint32_t)d.start_state, data + b, e - b, f,
                                              l, ex);
                else
                    dfa_walk<uint32_t, false>(static_cast<const uint32_t *>(d.table), d.accept_bits,
                                              (uint32_t)d.start_state, data + b, e - b, f,
                                              l, ex);
                flags[id] = f;
                lens[id] = l;
                if (examined) examined[id] = (int32_t)ex;
            }
            __syncwarp();
        }
    }
}

int32_t persistent_ctas_query(const PersistLayout &L, const gbfsm_plan &p);

cudaError_t ensure_smem(size_t bytes) {
    if (bytes <= 48u * 1024u) return cudaSuccess;
    return cudaFuncSetAttribute(persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)bytes);
}

}  // namespace

size_t persistent_workspace_bytes(int32_t max_words, const gbfsm_plan &p) {
    const PersistLayout L = persist_layout(max_words, p);
    const int ctas = persistent_ctas_per_sm(max_words, p);
    if (ctas <= 0) return 0;
    return 256u + (size_t)sm_count() * (size_t)ctas * L.wpc * L.global_per_warp;
}

namespace {
// Occupancy answers per (device, layout): computed once, outside any stream capture in
// practice (the first call of a layout), and reused by later launches and graph captures.
std::mutex g_occ_mutex;
std::map<std::tuple<int, int, int, int, int>, int32_t> g_occ;
}  // namespace

int32_t persistent_ctas_per_sm(int32_t max_words, const gbfsm_plan &p) {
    const PersistLayout L = persist_layout(max_words, p);
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_tuple(dev, L.Wmax, L.C, L.wpc, p.ctas_per_sm);
    {
        std::lock_guard<std::mutex> lock(g_occ_mutex);
        const auto it = g_occ.find(key);
        if (it != g_occ.end()) return it->second;
    }
    const int32_t v = persistent_ctas_query(L, p);
    std::lock_guard<std::mutex> lock(g_occ_mutex);
    g_occ[key] = v;
    return v;
}

namespace {
int32_t persistent_ctas_query(const PersistLayout &L, const gbfsm_plan &p) {
    const size_t smem = (size_t)L.wpc * L.smem_per_warp;
    if (smem + kSmemReserve > (size_t)smem_optin()) return 0;
    if (ensure_smem(smem) != cudaSuccess) return 0;
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, persistent_kernel, L.wpc * 32,
                                                      smem) != cudaSuccess)
        return 0;
    if (p.ctas_per_sm > 0 && p.ctas_per_sm < blocks) blocks = p.ctas_per_sm;
    return blocks;
}
}  // namespace

gbfsm_status launch_persistent(const gbfsm_automaton *table, int32_t max_words,
                               const gbfsm_task *tasks, int32_t n_tasks, const int32_t *input_ids,
                               const uint8_t *data, const int64_t *offsets, const int64_t *ends,
                               const gbfsm_chunk_io *chunk_io, int32_t *flags,
                               int32_t *lens, int32_t *examined, void *workspace,
                               size_t workspace_bytes, const gbfsm_plan &p, cudaStream_t stream) {
    const PersistLayout L = persist_layout(max_words, p);
    if (L.wpc < 1 || L.wpc * 32 > kMaxBlockThreads || (p.block_threads % 32) != 0)
        return fail(GBFSM_INVALID_ARG, "block_threads must be a multiple of 32 up to 256");
    const int ctas = persistent_ctas_per_sm(max_words, p);
    if (ctas <= 0)
        return fail(GBFSM_UNSUPPORTED,
                    "persistent launch does not fit: %d warps x %u shared bytes per warp",
                    L.wpc, L.smem_per_warp);
    const size_t need = persistent_workspace_bytes(max_words, p);
    if (workspace == nullptr || workspace_bytes < need)
        return fail(GBFSM_INVALID_ARG, "persistent workspace too small: %zu < %zu bytes",
                    workspace_bytes, need);
    if (n_tasks <= 0) return GBFSM_OK;
    ChunkIO io{nullptr, nullptr, nullptr, nullptr, nullptr};
    if (chunk_io) {
        io.chunks = chunk_io->chunks;
        io.records = static_cast<ChunkRecord *>(chunk_io->records);
        io.overflow_tasks = chunk_io->overflow_tasks;
        io.overflow_count = chunk_io->overflow_count;
        io.task_count = chunk_io->task_count;
    }
    uint32_t *ticket = static_cast<uint32_t *>(workspace);
    uint8_t *gws = static_cast<uint8_t *>(workspace) + 256;
    GBFSM_CUDA_TRY(cudaMemsetAsync(ticket, 0, sizeof(uint32_t), stream));
    const size_t smem = (size_t)L.wpc * L.smem_per_warp;
    int grid = sm_count() * ctas;
    const int needed = (n_tasks + L.wpc - 1) / L.wpc;
    if (grid > needed) grid = needed;
    persistent_kernel<<<grid, L.wpc * 32, smem, stream>>>(table, tasks, n_tasks, input_ids, data,
                                                          offsets, ends, io, flags, lens,
                                                          examined, L, ticket, gws);
    GBFSM_LAUNCH_CHECK("persistent_kernel launch");
    return GBFSM_OK;
}

}  // namespace gbfsm
