// Persistent batched engine: one launch for many inputs of uneven length over many
// automata (NFAs and DFAs) of different sizes.
//
// The grid is sized to the resident capacity (SMs x CTAs per SM from the occupancy
// calculator). Each warp pops tasks from a device queue with one atomicAdd ticket per
// task, in the order the host gave them (longest first, so the longest serial chains
// start first), until the queue is empty:
//   - a WHOLE NFA task (one input) is simulated by the whole warp with the automaton's
//     own technique (dense bitmap or sparse list) from the device automaton table;
//   - a WHOLE DFA task (1..32 inputs of one DFA) runs one table walk per lane;
//   - a CHUNK task runs one speculative chunk with the warp (run_chunk, chunks.cuh):
//     chunks of automata that do not run in lanes, and lane chunks whose set outgrew
//     the lane (the overflow queue);
//   - a FIXUP task resolves one chunked input exactly from its chunk records
//     (run_fixup, chunks.cuh).
// LANES tasks belong to the lane launch (lanes.cu) and are skipped here.
// Per-warp scratch: the dedup bitmap V and the two member lists in shared memory, sized
// for the largest NFA of the launch; the dense buffers (D, FA, FB) in a global workspace
// slice per resident warp. The reference has no counterpart: it launches one kernel per
// automaton and per batch (src/gpufsm/backends/cuda/nfa.py:105-121).
#include <map>
#include <mutex>
#include <tuple>

#include "chunks.cuh"
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

__global__ void __launch_bounds__(kMaxBlockThreads, kPersistMinBlocks) persistent_kernel(
    const gbfsm_automaton *__restrict__ table, int32_t n_automata,
    const gbfsm_task *__restrict__ tasks,
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
        if (task.kind == GBFSM_TASK_DFA_GROUP) {  // one walk per lane, each on its own DFA
            if ((int)lane < task.count) {
                const int32_t id = input_ids[task.first + (int)lane];
                const int32_t aut = io.aut_ids ? io.aut_ids[id] : 0;
                if (aut >= 0 && aut < n_automata && table[aut].kind == 1) {
                    const gbfsm_dfa_dev d = table[aut].dfa;
                    const int64_t b = offsets[id];
                    const int64_t e = ends ? ends[id] : offsets[id + 1];
                    int32_t f, l;
                    int64_t ex;
                    if (d.entry_bytes == 2)
                        dfa_walk<uint16_t, false>(static_cast<const uint16_t *>(d.table),
                                                  d.accept_bits, (uint32_t)d.start_state,
                                                  data + b, e - b, f, l, ex);
                    else
                        dfa_walk<uint32_t, false>(static_cast<const uint32_t *>(d.table),
                                                  d.accept_bits, (uint32_t)d.start_state,
                                                  data + b, e - b, f, l, ex);
                    flags[id] = f;
                    lens[id] = l;
                    if (examined) examined[id] = (int32_t)ex;
                }
            }
            __syncwarp();
            continue;
        }
        if (task.automaton < 0 || task.automaton >= n_automata) continue;
        const gbfsm_automaton *A = table + task.automaton;
        if (A->kind == 0) {
            const gbfsm_nfa_dev nfa = A->nfa;
            Rows R;
            R.sym_row = nfa.sym_row;
            R.sym_edges = nfa.sym_edges;
            R.eps_row = nfa.eps_row;
            R.eps_edges = nfa.eps_edges;
            S.C = (A->technique == GBFSM_TECH_WARP) ? 0 : min(A->list_capacity, L.C);
            if (task.kind == GBFSM_TASK_LANES) continue;  // gbfsm_lanes_run's tasks
            // chunk tasks naming chunks outside the table are skipped
            if ((task.kind == GBFSM_TASK_CHUNK || task.kind == GBFSM_TASK_FIXUP) &&
                (task.first < 0 || task.count < 1 || task.first + task.count > io.n_chunks))
                continue;
            if (task.kind == GBFSM_TASK_CHUNK) {
                const gbfsm_chunk ch = chunks[task.first];
                // a later chunk needs the one-byte supersets; without them it is not run
                if (ch.index > 0 && nfa.first_row == nullptr) continue;
                const int64_t off = offsets[ch.input];
                if (S.C == 0) S.C = min(L.C, 32);  // speculation keeps small sets listed
                const Bounds bd = chunk_bounds(io, nfa, data + off, task.first, off);
                run_chunk(nfa, R, S, data + off, bd.b, bd.e, bd.ov_end, ch.index,
                          records + task.first);
                continue;
            }
            if (task.kind == GBFSM_TASK_FIXUP) {
                const int32_t id = chunks[task.first].input;
                const int64_t off = offsets[id];
                const int64_t e = ends ? ends[id] : offsets[id + 1];
                if (S.C == 0) S.C = min(L.C, 32);
                const Verdict v = run_fixup(nfa, R, S, data + off, e - off, records,
                                            task.first, task.count);
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

gbfsm_status launch_persistent(const gbfsm_automaton *table, int32_t n_automata,
                               int32_t max_words,
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
    ChunkIO io{nullptr, nullptr, nullptr, nullptr, nullptr, 0, nullptr};
    if (chunk_io) {
        io.chunks = chunk_io->chunks;
        io.records = static_cast<ChunkRecord *>(chunk_io->records);
        io.overflow_tasks = chunk_io->overflow_tasks;
        io.overflow_count = chunk_io->overflow_count;
        io.task_count = chunk_io->task_count;
        io.n_chunks = chunk_io->n_chunks;
        io.aut_ids = chunk_io->aut_ids;
    }
    uint32_t *ticket = static_cast<uint32_t *>(workspace);
    uint8_t *gws = static_cast<uint8_t *>(workspace) + 256;
    GBFSM_CUDA_TRY(cudaMemsetAsync(ticket, 0, sizeof(uint32_t), stream));
    const size_t smem = (size_t)L.wpc * L.smem_per_warp;
    int grid = sm_count() * ctas;
    const int needed = (n_tasks + L.wpc - 1) / L.wpc;
    if (grid > needed) grid = needed;
    persistent_kernel<<<grid, L.wpc * 32, smem, stream>>>(table, n_automata, tasks, n_tasks,
                                                          input_ids, data,
                                                          offsets, ends, io, flags, lens,
                                                          examined, L, ticket, gws);
    GBFSM_LAUNCH_CHECK("persistent_kernel launch");
    return GBFSM_OK;
}

}  // namespace gbfsm
