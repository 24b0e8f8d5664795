// Internal (host) interface between the C-ABI layer (abi.cu) and the kernel translation
// units. Not exported.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/gbfsm.h"

namespace gbfsm {

constexpr int kDefaultListCapacity = 128;
constexpr int kMaxBlockThreads = 256;  // __launch_bounds__ of every simulation kernel
constexpr size_t kSmemReserve = 1024;  // static/driver-reserved shared memory headroom

// Where the per-warp scratch of the warp simulator lives, and how shared memory is laid
// out for one CTA of the plain warp kernel.
struct WarpPlan {
    int W;                    // set words of the automaton
    int C;                    // list capacity (0 = dense only)
    int warps_per_cta;
    int staged;               // edge rows copied to shared memory
    int dense_in_smem;        // D/FA/FB in shared memory (else global workspace)
    int v_in_smem;            // V and the lists in shared memory (else global workspace)
    uint32_t stage_bytes;     // bytes of the staged region (incl. the mbarrier slot)
    uint32_t off_sym_row, off_sym_edges, off_eps_row, off_eps_edges;
    uint32_t bytes_sym_row, bytes_sym_edges, bytes_eps_row, bytes_eps_edges;
    uint32_t smem_per_warp;   // shared bytes per warp
    size_t global_per_warp;   // global workspace bytes per warp
    size_t smem_total;        // dynamic shared memory per CTA
};

// Thread-per-input bitmap kernel plan.
struct BitmapPlan {
    int W;
    int threads;        // per CTA
    int staged;
    int sets_in_smem;   // 4W words per thread in shared memory (else global)
    uint32_t stage_bytes;
    uint32_t off_sym_row, off_sym_edges, off_eps_row, off_eps_edges;
    uint32_t bytes_sym_row, bytes_sym_edges, bytes_eps_row, bytes_eps_edges;
    size_t smem_total;
};

__host__ __device__ __forceinline__ uint32_t pad16(uint64_t bytes) {
    return (uint32_t)((bytes + 15u) & ~(uint64_t)15u);
}

// Plan builders (host). Return GBFSM_UNSUPPORTED when no layout fits.
gbfsm_status make_warp_plan(const gbfsm_nfa_dev &a, int32_t n_inputs, const gbfsm_plan &p,
                            WarpPlan &out);
gbfsm_status make_bitmap_plan(const gbfsm_nfa_dev &a, int32_t n_inputs, const gbfsm_plan &p,
                              BitmapPlan &out);

// Launchers (nfa_kernels.cu, dfa_kernels.cu, persistent.cu, layout.cu).
gbfsm_status launch_nfa_warp(const gbfsm_nfa_dev &a, const WarpPlan &wp, const uint8_t *data,
                             const int64_t *offsets, int32_t n_inputs, int32_t *flags,
                             int32_t *lens, int32_t *examined, void *workspace,
                             cudaStream_t stream);
gbfsm_status launch_nfa_bitmap(const gbfsm_nfa_dev &a, const BitmapPlan &bp, const uint8_t *data,
                               const int64_t *offsets, int32_t n_inputs, int32_t *flags,
                               int32_t *lens, int32_t *examined, void *workspace,
                               cudaStream_t stream);
gbfsm_status launch_dfa_walk(const gbfsm_dfa_dev &d, const gbfsm_plan &p, const uint8_t *data,
                             const int64_t *offsets, int32_t n_inputs, int32_t *flags,
                             int32_t *lens, int32_t *examined, cudaStream_t stream);
gbfsm_status launch_persistent(const gbfsm_automaton *table, int32_t n_automata,
                               int32_t max_words,
                               const gbfsm_task *tasks, int32_t n_tasks, const int32_t *input_ids,
                               const uint8_t *data, const int64_t *offsets, const int64_t *ends,
                               const gbfsm_chunk_io *chunk_io, int32_t *flags,
                               int32_t *lens, int32_t *examined, void *workspace,
                               size_t workspace_bytes, const gbfsm_plan &p, cudaStream_t stream);
int lanes_warps_per_sm();
gbfsm_status launch_lanes(const gbfsm_automaton *table, int32_t n_automata,
                          const gbfsm_task *tasks, int32_t n_tasks, const int32_t *range,
                          const uint8_t *data, const int64_t *offsets,
                          const gbfsm_chunk_io &chunk_io, cudaStream_t stream);
size_t batch_plan_scratch_bytes(int32_t n_inputs);
gbfsm_status launch_gather_inputs(const uint64_t *src, const int64_t *offsets, int32_t n,
                                  uint8_t *dst, cudaStream_t stream);
int32_t pageable_access();
gbfsm_status launch_batch_plan(const gbfsm_batch_plan_args &args, cudaStream_t stream);

// DFA_CHUNK / DFA_FIXUP tasks (dfa_chunks.cu).
gbfsm_status launch_dfa_chunks(const gbfsm_automaton *table, int32_t n_automata,
                               const gbfsm_task *tasks, int32_t max_tasks,
                               const int32_t *task_count, const uint8_t *data,
                               const int64_t *offsets, const int64_t *ends,
                               const gbfsm_chunk_io &chunk_io, int32_t max_states,
                               int32_t *flags, int32_t *lens, int32_t *examined,
                               int32_t *latch, cudaStream_t stream);
size_t persistent_workspace_bytes(int32_t max_words, const gbfsm_plan &p);
int32_t persistent_ctas_per_sm(int32_t max_words, const gbfsm_plan &p);
gbfsm_status launch_nfa_layout(int32_t n, const int32_t *srp, const int32_t *stg,
                               const int32_t *ssy, const int32_t *erp, const int32_t *etg,
                               const uint8_t *accept, uint64_t nnz_sym, uint64_t nnz_eps,
                               uint32_t *sym_row, gbfsm_edge *sym_edges, uint32_t *eps_row,
                               gbfsm_edge *eps_edges, uint64_t *accept_words, int32_t *error,
                               cudaStream_t stream);
gbfsm_status launch_dfa_layout(int32_t n, const int32_t *trans, const uint8_t *accept,
                               int32_t entry_bytes, void *table, uint32_t *accept_bits,
                               int32_t *error, cudaStream_t stream);
gbfsm_status launch_narrow_symbols(const int32_t *src, uint8_t *dst, int64_t n,
                                   int32_t *error, cudaStream_t stream);
gbfsm_status launch_widen_offsets(const int32_t *src, int64_t *dst, int64_t n,
                                  cudaStream_t stream);

}  // namespace gbfsm
