// One-lane-per-chunk speculative NFA launch (GBFSM_TASK_LANES tasks).
//
// Each warp takes one LANES task (up to 32 chunks of one automaton) and each lane runs one
// chunk with lane_chunk() (chunks.cuh): a set of at most kLaneSlots states held as their
// lane records in registers, matched against each byte by byte-wise compares of their
// packed edge labels, with one L2 record load per matched edge. A chunk
// that outgrows its lane is appended to the overflow queue as a CHUNK task, which the
// persistent launch then runs with a whole warp. The kernel holds no per-warp shared
// state and no warp-wide loop, so it runs in a separate, lighter launch than the
// persistent kernel and fits more resident warps per SM.
#include "chunks.cuh"
#include "common.cuh"
#include "engine.hpp"

namespace gbfsm {
namespace {

constexpr int kLanesThreads = 128;
#ifndef GBFSM_LANES_MIN_BLOCKS
#define GBFSM_LANES_MIN_BLOCKS 8
#endif
constexpr int kLanesMinBlocks = GBFSM_LANES_MIN_BLOCKS;  // 8 x 128 threads: 64 registers

__global__ void __launch_bounds__(kLanesThreads, kLanesMinBlocks) lanes_kernel(
    const gbfsm_automaton *__restrict__ table, int32_t n_automata,
    const gbfsm_task *__restrict__ tasks, int32_t n_tasks, const int32_t *__restrict__ range,
    const uint8_t *__restrict__ data, const int64_t *__restrict__ offsets, ChunkIO io) {
    int32_t first = 0;
    if (range) {  // a task range written on the device by an earlier launch
        first = range[0];
        n_tasks = min(n_tasks, range[1]);
    }
    const int lane = (int)lane_id();
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); w < n_tasks; w += nwarps) {
        const gbfsm_task task = tasks[first + w];
        if (lane >= task.count) continue;
        const int cid = task.first + lane;
        if (cid < 0 || cid >= io.n_chunks) continue;  // a task naming chunks outside the table
        const gbfsm_chunk ch = io.chunks[cid];
        if (ch.input < 0) continue;
        // automaton -1: each lane runs its chunk's input's automaton
        const int32_t aut =
            task.automaton >= 0 ? task.automaton : (io.aut_ids ? io.aut_ids[ch.input] : 0);
        if (aut < 0 || aut >= n_automata) continue;
        const int64_t off = offsets[ch.input];
        const gbfsm_automaton &T = table[aut];
        const gbfsm_nfa_dev &A = T.nfa;
        if (T.kind != 0) continue;  // LANES tasks of a DFA are ignored
        const bool lane_tables = A.lane_edges != nullptr && A.pair_row != nullptr;
        bool done = false;
        if (lane_tables) {
            const Bounds bd = chunk_bounds(io, A, data + off, cid, off);
            done = lane_chunk(A, data + off, bd.b, bd.e, bd.ov_end, ch.index, io.records + cid);
        }
        if (!done) {
            gbfsm_task spill;
            spill.automaton = aut;
            spill.first = cid;
            spill.count = 1;
            spill.kind = GBFSM_TASK_CHUNK;
            // the queue holds n_chunks entries: only a task list naming a chunk twice
            // could overflow it, and then the extra entries are dropped rather than written
            // past it
            const int slot = atomicAdd(io.overflow_count, 1);
            if (slot < io.n_chunks) io.overflow_tasks[slot] = spill;
        }
    }
}

}  // namespace

int lanes_warps_per_sm() {
    // asked once per device (the answer depends only on the kernel and the device)
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = -1;
    if (dev >= 0 && cached[dev] > 0) return cached[dev];
    // the kernel uses no shared memory: ask for the largest L1 share of the unified
    // L1/shared storage, where the lane records that miss in registers are gathered from
    cudaFuncSetAttribute(lanes_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    cudaGetLastError();
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, lanes_kernel, kLanesThreads, 0) !=
        cudaSuccess)
        blocks = 0;
    cudaGetLastError();
    const int warps = blocks * (kLanesThreads / 32);
    if (dev >= 0 && warps > 0) cached[dev] = warps;
    return warps;
}

gbfsm_status launch_lanes(const gbfsm_automaton *table, int32_t n_automata,
                          const gbfsm_task *tasks, int32_t n_tasks, const int32_t *range,
                          const uint8_t *data, const int64_t *offsets,
                          const gbfsm_chunk_io &chunk_io, cudaStream_t stream) {
    if (n_tasks <= 0) return GBFSM_OK;
    const int warps_per_sm = lanes_warps_per_sm();  // once per device: sets the L1 share
    ChunkIO io{chunk_io.chunks, static_cast<ChunkRecord *>(chunk_io.records),
               chunk_io.overflow_tasks, chunk_io.overflow_count, nullptr, chunk_io.n_chunks,
               chunk_io.aut_ids};
    const int warps_per_block = kLanesThreads / 32;
    int grid = (n_tasks + warps_per_block - 1) / warps_per_block;
    if (range) {  // at most one resident wave; the warps loop over the tasks
        const int wave = sm_count() * (warps_per_sm / warps_per_block);
        if (wave > 0 && grid > wave) grid = wave;
    }
    lanes_kernel<<<grid, kLanesThreads, 0, stream>>>(table, n_automata, tasks, n_tasks, range,
                                                      data, offsets, io);
    GBFSM_LAUNCH_CHECK("lanes_kernel launch");
    return GBFSM_OK;
}

}  // namespace gbfsm
