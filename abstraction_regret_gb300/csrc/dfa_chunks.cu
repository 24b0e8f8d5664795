// The launch of DFA_CHUNK and DFA_FIXUP tasks (chunked walks of long DFA inputs,
// dfa_chunks.cuh). A warp takes one task at a time from a grid-stride loop over the task
// list, whose length is read on the device (the plan header). Each warp has its own
// shared scratch for the set walk of a chunk: two bitmaps of the largest DFA's states and
// a 32-entry member list.
#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"
#include "dfa_chunks.cuh"
#include "engine.hpp"

namespace gbfsm {
namespace {

constexpr int kDfaChunkThreads = 128;  // 4 warps per CTA
constexpr int kDfaChunkWarps = kDfaChunkThreads / 32;
// resident CTAs per SM the register allocation is bounded for (0: no bound, 72 registers,
// 7 CTAs per SM). 8 gives 64 registers (16 spilled bytes) and 4864 resident warps, so a
// wave holds more, shorter chunks: 64 x 4 MiB on a 4096-state DFA took 22.8 ms against
// 26.0 ms, but the serving pool's live trace with every request at once lost 16% of its
// examined rate (p99 105 against 86-89 ms): its long DFA inputs latch within hundreds of
// bytes, and every extra chunk walks its set of all states before it sees the latch
#ifndef GBFSM_DFA_CHUNK_MIN_BLOCKS
#define GBFSM_DFA_CHUNK_MIN_BLOCKS 0
#endif
#if GBFSM_DFA_CHUNK_MIN_BLOCKS > 0
#define GBFSM_DFA_CHUNK_BOUNDS __launch_bounds__(kDfaChunkThreads, GBFSM_DFA_CHUNK_MIN_BLOCKS)
#else
#define GBFSM_DFA_CHUNK_BOUNDS __launch_bounds__(kDfaChunkThreads)
#endif

__global__ void GBFSM_DFA_CHUNK_BOUNDS dfa_chunks_kernel(
    const gbfsm_automaton *__restrict__ table, int32_t n_automata,
    const gbfsm_task *__restrict__ tasks, int32_t n_tasks, const int32_t *__restrict__ task_count,
    const uint8_t *__restrict__ data, const int64_t *__restrict__ offsets,
    const int64_t *__restrict__ ends, const gbfsm_chunk *__restrict__ chunks, int32_t n_chunks,
    void *records, uint32_t words, int32_t *flags, int32_t *lens, int32_t *examined,
    int32_t *latch) {
    extern __shared__ __align__(16) uint32_t dsm[];
    if (task_count) n_tasks = min(n_tasks, *task_count);
    const uint32_t lane = lane_id();
    const int warp_in_cta = (int)(threadIdx.x >> 5);
    uint32_t *bm0 = dsm + (size_t)warp_in_cta * (2u * words + 32u);
    uint32_t *bm1 = bm0 + words;
    uint32_t *list = bm1 + words;
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int t = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); t < n_tasks; t += nwarps) {
        const gbfsm_task task = tasks[t];
        if (task.kind != GBFSM_TASK_DFA_CHUNK && task.kind != GBFSM_TASK_DFA_FIXUP) continue;
        if (task.automaton < 0 || task.automaton >= n_automata || task.first < 0 ||
            task.count < 1 || task.first > n_chunks - task.count)
            continue;
        const gbfsm_automaton &T = table[task.automaton];
        if (T.kind != 1 || T.dfa.num_states < 1 || (uint32_t)T.dfa.num_states > words * 32u)
            continue;
        const gbfsm_dfa_dev d = T.dfa;
        const gbfsm_chunk ch = chunks[task.first];
        if (ch.input < 0) continue;
        const int64_t off = offsets[ch.input];
        const int64_t len = (ends ? ends[ch.input] : offsets[ch.input + 1]) - off;
        if (task.kind == GBFSM_TASK_DFA_CHUNK) {
            DfaChunkRecord *rec = dfa_record(records, task.first);
            // the next chunk of the input, when there is one, is the next table entry
            const DfaChunkRecord *next = nullptr;
            int64_t e_next = ch.end - off;
            if (task.first + 1 < n_chunks) {
                const gbfsm_chunk nx = chunks[task.first + 1];
                if (nx.input == ch.input && nx.index == ch.index + 1) {
                    next = dfa_record(records, task.first + 1);
                    e_next = nx.end - off;
                }
            }
            int32_t *lt = latch ? latch + ch.input : nullptr;
            if (d.entry_bytes == 2)
                dfa_chunk<uint16_t>(d, T.dfa_overlap, data + off, len, ch.begin - off,
                                    ch.end - off, e_next, ch.index, bm0, bm1, list, rec, next,
                                    lt);
            else
                dfa_chunk<uint32_t>(d, T.dfa_overlap, data + off, len, ch.begin - off,
                                    ch.end - off, e_next, ch.index, bm0, bm1, list, rec, next,
                                    lt);
        } else if (lane == 0) {
            const Verdict v =
                d.entry_bytes == 2
                    ? dfa_fixup<uint16_t>(d, data + off, len, chunks, off, records, task.first,
                                          task.count)
                    : dfa_fixup<uint32_t>(d, data + off, len, chunks, off, records, task.first,
                                          task.count);
            flags[ch.input] = v.flag;
            lens[ch.input] = v.len;
            if (examined) examined[ch.input] = (int32_t)v.examined;
        }
        __syncwarp();
    }
}

// Shared scratch of a CTA for DFAs of up to `words` x 32 states.
size_t dfa_chunks_smem(uint32_t words) {
    return (size_t)kDfaChunkWarps * (2u * words + 32u) * sizeof(uint32_t);
}

// Resident CTAs per SM for that scratch, asked once per (device, scratch size): later
// launches and graph captures reuse the answer. Opts the kernel in to the shared memory
// it needs above 48 KiB; -1 when that is more than the device has.
int dfa_chunks_blocks_per_sm(uint32_t words, gbfsm_status &st) {
    static std::mutex mu;
    static std::map<std::pair<int, uint32_t>, int> occupancy;
    st = GBFSM_OK;
    const size_t smem = dfa_chunks_smem(words);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        st = GBFSM_CUDA_ERROR;
        return 0;
    }
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(dev, words);
    const auto it = occupancy.find(key);
    if (it != occupancy.end()) return it->second;
    if (smem > 48u * 1024u) {
        if (smem + kSmemReserve > (size_t)smem_optin()) return -1;
        if (cudaFuncSetAttribute(dfa_chunks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess) {
            cudaGetLastError();
            st = GBFSM_CUDA_ERROR;
            return 0;
        }
    }
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, dfa_chunks_kernel,
                                                      kDfaChunkThreads, smem) != cudaSuccess) {
        cudaGetLastError();
        st = GBFSM_CUDA_ERROR;
        return 0;
    }
    occupancy[key] = blocks;
    return blocks;
}

}  // namespace

gbfsm_status launch_dfa_chunks(const gbfsm_automaton *table, int32_t n_automata,
                               const gbfsm_task *tasks, int32_t max_tasks,
                               const int32_t *task_count, const uint8_t *data,
                               const int64_t *offsets, const int64_t *ends,
                               const gbfsm_chunk_io &chunk_io, int32_t max_states,
                               int32_t *flags, int32_t *lens, int32_t *examined,
                               int32_t *latch, cudaStream_t stream) {
    if (max_tasks <= 0) return GBFSM_OK;
    const uint32_t words = ((uint32_t)max_states + 31u) >> 5;
    const size_t smem = dfa_chunks_smem(words);
    gbfsm_status st = GBFSM_OK;
    const int blocks = dfa_chunks_blocks_per_sm(words, st);
    if (st != GBFSM_OK) return fail(st, "dfa_chunks_kernel: occupancy query failed");
    if (blocks < 0)
        return fail(GBFSM_UNSUPPORTED, "DFA chunk walks of %d states need %zu shared bytes",
                    max_states, smem);
    int grid = sm_count() * (blocks > 0 ? blocks : 1);
    const int needed = (max_tasks + kDfaChunkWarps - 1) / kDfaChunkWarps;
    if (grid > needed) grid = needed;
    dfa_chunks_kernel<<<grid, kDfaChunkThreads, smem, stream>>>(
        table, n_automata, tasks, max_tasks, task_count, data, offsets, ends, chunk_io.chunks,
        chunk_io.n_chunks, chunk_io.records, words, flags, lens, examined, latch);
    GBFSM_LAUNCH_CHECK("dfa_chunks_kernel launch");
    return GBFSM_OK;
}

}  // namespace gbfsm

extern "C" int32_t gbfsm_dfa_chunks_warps_per_sm(int32_t max_states) {
    using namespace gbfsm;
    if (max_states < 1 || max_states > 32768) return 0;
    gbfsm_status st = GBFSM_OK;
    const int blocks = dfa_chunks_blocks_per_sm(((uint32_t)max_states + 31u) >> 5, st);
    return st == GBFSM_OK && blocks > 0 ? blocks * kDfaChunkWarps : 0;
}

extern "C" gbfsm_status gbfsm_dfa_chunks_run(const gbfsm_automaton *table, int32_t n_automata,
                                             const gbfsm_task *tasks, int32_t max_tasks,
                                             const int32_t *task_count, const uint8_t *data,
                                             const int64_t *offsets, const int64_t *ends,
                                             const gbfsm_chunk_io *chunk_io,
                                             int32_t max_states, int32_t *flags, int32_t *lens,
                                             int32_t *examined, int32_t *latch, void *stream) {
    using namespace gbfsm;
    if (max_tasks < 0 || n_automata < 0) return fail(GBFSM_INVALID_ARG, "negative task count");
    if (max_tasks == 0) return GBFSM_OK;
    if (!table || !tasks || !data || !offsets || !chunk_io || !chunk_io->chunks ||
        !chunk_io->records || !flags || !lens)
        return fail(GBFSM_INVALID_ARG, "NULL array passed to gbfsm_dfa_chunks_run");
    if (chunk_io->n_chunks < 1)
        return fail(GBFSM_INVALID_ARG, "gbfsm_dfa_chunks_run: empty chunk table");
    if (max_states < 1 || max_states > 32768)
        return fail(GBFSM_INVALID_ARG, "max_states must be in 1..32768 (got %d)", max_states);
    return launch_dfa_chunks(table, n_automata, tasks, max_tasks, task_count, data, offsets, ends,
                             *chunk_io, max_states, flags, lens, examined, latch,
                             static_cast<cudaStream_t>(stream));
}
