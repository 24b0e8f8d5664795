/*
 * gbfsm.h -- C ABI of libgbfsm, the GB300 (sm_103a) automata-simulation engine.
 *
 * Drop-in for the native layer of the reference's CUDA backend: gpufsm 0.1.0
 * (alepot55/abstraction-regret), whose pybind11 module `_cuda` exposes the `run_*`
 * functions of src/gpufsm/backends/cuda/native/include/api.hpp:23-104 and
 * bindings.cu:11-39. Two layers are exported:
 *
 *  1. Reference-shaped host entry points (gbfsm_run_*): the same arguments and meaning
 *     as the `_cuda.run_*` functions they replace (host arrays in, host arrays out,
 *     synchronous, the kernel time in milliseconds), with status codes instead of C++
 *     exceptions. A ctypes/cffi stub binds them in place of the pybind11 module.
 *  2. Device entry points (gbfsm_nfa_run, gbfsm_dfa_run, gbfsm_persistent_run, ...):
 *     device pointers owned by the caller (PyTorch tensors in this package), a CUDA
 *     stream, no implicit synchronisation, no allocation. These are what the Python
 *     engine uses; they can be captured in a CUDA graph.
 *
 * Conventions for every function:
 *   - returns gbfsm_status; no exception crosses the ABI; on failure a message is left
 *     in gbfsm_last_error() (thread-local);
 *   - `stream` is a cudaStream_t passed as void* (0 = the legacy default stream);
 *   - verdicts follow the reference's latch-first-match rule (src/gpufsm/reference.py:
 *     36-81): flags[i] = 1 and lens[i] = the number of bytes consumed when the first
 *     accepting configuration is reached (0 if the start configuration accepts),
 *     flags[i] = lens[i] = 0 otherwise;
 *   - an input is bytes data[offsets[i] .. offsets[i+1]) with int64 offsets. `data`
 *     must stay readable up to the next 16-byte boundary past offsets[n_inputs] (the
 *     kernels use 16-byte vector loads); a single input is shorter than 2^31 bytes.
 */
#ifndef GBFSM_H
#define GBFSM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBFSM_ABI_VERSION 3
#define GBFSM_ANY_SYMBOL 256 /* src/gpufsm/core/nfa.py:16 */
#define GBFSM_WORD_BITS 64   /* src/gpufsm/core/packing.py:21 */

typedef enum gbfsm_status {
    GBFSM_OK = 0,
    GBFSM_INVALID_ARG = 1, /* bad pointer, size or automaton; maps to ValueError */
    GBFSM_UNSUPPORTED = 2, /* valid but beyond a technique's limits */
    GBFSM_CUDA_ERROR = 3,  /* a CUDA call failed; maps to RuntimeError */
    GBFSM_TIMEOUT = 4,     /* a bounded device wait gave up */
    GBFSM_OOM = 5          /* a host-buffer entry point could not allocate */
} gbfsm_status;

/* ---------------------------------------------------------------------------------
 * Device-resident automaton layouts
 * ------------------------------------------------------------------------------- */

/* One edge of the NFA, 16 bytes. Besides the edge's own target and label it carries
 * what the simulator needs next about the target (whether it accepts, whether it has
 * epsilon edges, and the range of its own symbol edges), so following an edge costs
 * one dependent load instead of three. The same record describes a state in the
 * engine's active-state lists (target = the state itself). */
typedef struct gbfsm_edge {
    uint32_t target;
    uint32_t info;      /* bits 0-8: symbol (0..255, 256 = ANY); GBFSM_EDGE_* flags */
    uint32_t row_begin; /* target's symbol edges: sym_edges[row_begin .. row_end) */
    uint32_t row_end;
} gbfsm_edge;

#define GBFSM_EDGE_SYMBOL_MASK 0x1FFu
#define GBFSM_EDGE_ACCEPT (1u << 9)  /* the target accepts */
#define GBFSM_EDGE_HAS_EPS (1u << 10) /* the target has epsilon edges */

#define GBFSM_NFA_HAS_EPS 1 /* the automaton has epsilon edges */
#define GBFSM_NFA_HAS_ANY 2 /* the automaton has ANY_SYMBOL edges */

/* An NFA on the device (all pointers are device pointers). Built from the reference's
 * CSR arrays (src/gpufsm/core/nfa.py:56-65) by gbfsm_nfa_layout. */
/* A state as a lane of the one-chunk-per-lane kernel holds it: the state, its accept
 * flag and its out-edges in 16 bytes. When the state has at most 16 symbol edges and no
 * ANY edge (the fast form) the symbols of its first 8 edges are packed one byte each
 * into labels_lo (edges 0..3, lowest byte first) and labels_hi (edges 4..7), and those
 * of edges 8..15 into lane_labels_ext[2*state], [2*state + 1]; a lane finds the edges
 * matching a byte with byte-wise compares. Otherwise (GBFSM_LANE_SLOW) labels_lo holds
 * row_end and the lane scans edge_sym. */
typedef struct gbfsm_lane_rec {
    uint32_t state;     /* bits 0-24 state, 25-29 out-degree (fast form), 30 SLOW, 31 ACCEPT */
    uint32_t row_begin;
    uint32_t labels_lo;
    uint32_t labels_hi;
} gbfsm_lane_rec;
#define GBFSM_LANE_STATE_MASK 0x01FFFFFFu
#define GBFSM_LANE_DEG_SHIFT 25
#define GBFSM_LANE_DEG_MASK 31u
#define GBFSM_LANE_FAST_DEGREE 16
#define GBFSM_LANE_SLOW (1u << 30)
#define GBFSM_LANE_ACCEPT (1u << 31)

typedef struct gbfsm_nfa_dev {
    int32_t num_states;
    int32_t start_state;
    int32_t num_words; /* ceil(num_states / 64) */
    int32_t flags;     /* GBFSM_NFA_* */
    const uint32_t *sym_row;        /* [num_states + 1] */
    const gbfsm_edge *sym_edges;    /* [num_sym_edges] */
    const uint32_t *eps_row;        /* [num_states + 1] */
    const gbfsm_edge *eps_edges;    /* [num_eps_edges] (info symbol bits unused) */
    const uint64_t *accept_words;   /* [num_words], pack_accept layout */
    uint64_t num_sym_edges;
    uint64_t num_eps_edges;
    /* Optional (NULL = no speculative chunking for this automaton): for each byte c, the
     * distinct targets of all edges labelled c or ANY, as state records
     * first_edges[first_row[c] .. first_row[c+1]) (first_row has 257 entries). After any
     * byte c the active set is contained in the epsilon closure of these targets, which
     * makes them a safe starting superset for a chunk that begins mid-input. */
    const uint32_t *first_row;
    const gbfsm_edge *first_edges;
    /* Optional (NULL = no lane-per-chunk speculation; automata without epsilon edges and
     * with fewer than 2^26 states): the label of every symbol edge as uint16 (0..256);
     * the two-byte supersets: for bytes c1, c2 the distinct states reachable from any
     * state by c1 then c2, as lane records pair_lanes[pair_row[c1*256 + c2] ..
     * pair_row[c1*256 + c2 + 1]) (65537 entries); for every symbol edge the lane
     * record of its target (lane_edges, indexed like sym_edges); and the packed symbols
     * of edges 8..15 of every state (lane_labels_ext, [2 * num_states]). */
    const uint16_t *edge_sym;
    const uint32_t *pair_row;
    const gbfsm_lane_rec *pair_lanes;
    const gbfsm_lane_rec *lane_edges;
    const uint32_t *lane_labels_ext;
} gbfsm_nfa_dev;

/* A DFA on the device. table[s * 256 + c] holds the successor of s on byte c in the low
 * bits and, in the top bit, whether that successor accepts; entries are 2 bytes when
 * num_states <= 32768, else 4 bytes. accept_bits[s / 32] bit s % 32 = accept[s]. */
typedef struct gbfsm_dfa_dev {
    int32_t num_states;
    int32_t start_state;
    int32_t entry_bytes; /* 2 or 4 */
    int32_t flags;
    const void *table;
    const uint32_t *accept_bits;
    uint64_t table_bytes;
} gbfsm_dfa_dev;

/* How to run a batch. Zero fields select the defaults. */
typedef struct gbfsm_plan {
    int32_t technique;     /* GBFSM_TECH_* */
    int32_t block_threads; /* threads per CTA (multiple of 32) */
    int32_t list_capacity; /* sparse active-list capacity per warp (COMPACT) */
    int32_t stage;         /* 1: stage edges / DFA table in shared memory when they fit.
                              Staging copies sym_row, sym_edges, eps_row, eps_edges (or
                              the DFA table) with bulk copies of whole 16-byte blocks: it
                              is used only when each of them starts 16-byte aligned (else
                              the launch reads them through L2), and each must then be
                              readable up to the next 16-byte boundary past its end. */
    int32_t ctas_per_sm;   /* persistent launches: CTAs per SM (0 = from occupancy) */
    int32_t reserved[3];
} gbfsm_plan;

#define GBFSM_TECH_BITMAP 0  /* thread per input, packed bitmap set in shared memory */
#define GBFSM_TECH_WARP 1    /* warp per input, dense bitmap set, ballot/popc/shfl expansion */
#define GBFSM_TECH_COMPACT 2 /* warp per input, sparse active list; dense when it overflows */
#define GBFSM_TECH_DFA_WALK 3 /* DFA: thread per input, table walk */

/* ---------------------------------------------------------------------------------
 * Library
 * ------------------------------------------------------------------------------- */

/* ABI version of the loaded library (GBFSM_ABI_VERSION). */
int gbfsm_abi_version(void);

/* Message of the last failure on the calling thread ("" if none). */
const char *gbfsm_last_error(void);

/* ---------------------------------------------------------------------------------
 * Layout builders (device). Replace the per-call host marshalling of
 * src/gpufsm/backends/cuda/nfa.py:44-52 (_csr_args), :90-100 (pack_accept) and
 * dfa.py:27-31 with a one-time, device-side build.
 * ------------------------------------------------------------------------------- */

/* Validate the reference CSR arrays (device pointers, int32 as in core/nfa.py:60-65,
 * accept as uint8) and write the engine's layout into caller-allocated device arrays:
 * sym_row/eps_row [n+1], sym_edges [nnz_sym], eps_edges [nnz_eps], accept_words
 * [ceil(n/64)]. *error (a device int32, zeroed by this call) receives a nonzero code if
 * an index or symbol is out of range or a row pointer decreases; the caller reads it
 * after the stream completes. Stream-ordered. */
gbfsm_status gbfsm_nfa_layout(int32_t num_states, const int32_t *sym_row_ptr,
                              const int32_t *sym_targets, const int32_t *sym_symbols,
                              const int32_t *eps_row_ptr, const int32_t *eps_targets,
                              const uint8_t *accept, uint64_t nnz_sym, uint64_t nnz_eps,
                              uint32_t *sym_row, gbfsm_edge *sym_edges, uint32_t *eps_row,
                              gbfsm_edge *eps_edges, uint64_t *accept_words, int32_t *error,
                              void *stream);

/* Pack the reference DFA table (device int32 [n*256], core/dfa.py:36-41) and accept
 * array (uint8 [n]) into `table` (entry_bytes per entry) and accept_bits
 * [ceil(n/32)]. *error as above (a successor out of [0, n)). */
gbfsm_status gbfsm_dfa_layout(int32_t num_states, const int32_t *trans, const uint8_t *accept,
                              int32_t entry_bytes, void *table, uint32_t *accept_bits,
                              int32_t *error, void *stream);

/* ---------------------------------------------------------------------------------
 * Plain single-launch batch kernels (device pointers). One launch covers the batch.
 * Replace the kernels behind _cuda.run_worklist / run_worklist_warp /
 * run_worklist_compact / run_dfa (worklist_register.cu:113-128,
 * worklist_global.cu:128-181 and :289-310, dfa.cu:9-29).
 * ------------------------------------------------------------------------------- */

/* Scratch bytes gbfsm_nfa_run needs for `plan` (0 when the sets fit shared memory). */
size_t gbfsm_nfa_workspace_bytes(const gbfsm_nfa_dev *nfa, int32_t n_inputs,
                                 const gbfsm_plan *plan);

/* Simulate `nfa` over a batch. examined (nullable) receives the bytes consumed per
 * input. workspace: device scratch of at least gbfsm_nfa_workspace_bytes. */
gbfsm_status gbfsm_nfa_run(const gbfsm_nfa_dev *nfa, const uint8_t *data,
                           const int64_t *offsets, int32_t n_inputs, const gbfsm_plan *plan,
                           int32_t *flags, int32_t *lens, int32_t *examined, void *workspace,
                           size_t workspace_bytes, void *stream);

/* Size of the fixed device scratch of gbfsm_nfa_run_static (32 MiB per device). */
#define GBFSM_STATIC_SCRATCH_BYTES (32u << 20)

/* gbfsm_nfa_run without a workspace argument: the scratch comes from a fixed array of
 * GBFSM_STATIC_SCRATCH_BYTES in device memory, so the call allocates nothing on the
 * device (no cudaMalloc / cudaFree, no allocator of any library). For callers that
 * cannot allocate device memory themselves, e.g. a foreign-language host without a
 * device allocator, or a service that must not grow its device footprint or wait on
 * an allocator while requests are in flight. Returns GBFSM_INVALID_ARG, writing
 * nothing, when the batch needs more scratch than that (gbfsm_nfa_workspace_bytes of
 * the same arguments). The first call on a device looks up the array's address
 * (module load); make it before any stream capture. The address is kept for the life
 * of the process and is valid only as long as the device's context: after
 * cudaDeviceReset on that device, do not call this entry point again in the same
 * process. All calls on a device share the one array: calls whose kernels overlap on the
 * GPU race on it and must be ordered (e.g. issued on one stream). Results are those of
 * gbfsm_nfa_run. No counterpart in the reference. */
gbfsm_status gbfsm_nfa_run_static(const gbfsm_nfa_dev *nfa, const uint8_t *data,
                                  const int64_t *offsets, int32_t n_inputs,
                                  const gbfsm_plan *plan, int32_t *flags, int32_t *lens,
                                  int32_t *examined, void *stream);

/* Simulate `dfa` over a batch (thread per input; table in shared memory when
 * plan->stage and it fits, else read through L2). */
gbfsm_status gbfsm_dfa_run(const gbfsm_dfa_dev *dfa, const uint8_t *data,
                           const int64_t *offsets, int32_t n_inputs, const gbfsm_plan *plan,
                           int32_t *flags, int32_t *lens, int32_t *examined, void *stream);

/* ---------------------------------------------------------------------------------
 * Persistent batched engine (device pointers). Many inputs of uneven length over many
 * automata of different sizes in ONE launch: resident CTAs pop tasks from a device
 * queue (one atomic ticket per task) in the order given (the host sorts them longest
 * first). No counterpart in the reference, which launches once per automaton.
 * ------------------------------------------------------------------------------- */

/* One entry of the device-resident automaton table. */
typedef struct gbfsm_automaton {
    int32_t kind;          /* 0 = NFA, 1 = DFA */
    int32_t technique;     /* NFA: GBFSM_TECH_WARP or GBFSM_TECH_COMPACT */
    int32_t list_capacity; /* NFA compact list capacity (<= the launch's capacity) */
    int32_t dfa_overlap;   /* DFA: the most bytes a DFA_CHUNK task's exact walk continues
                              past its chunk's end, never past the next chunk's end (0 =
                              none: every chunk then links by a serial walk) */
    gbfsm_nfa_dev nfa;     /* valid when kind == 0 */
    gbfsm_dfa_dev dfa;     /* valid when kind == 1 */
} gbfsm_automaton;

/* One task. kind GBFSM_TASK_LANES: up to 32 chunks of one automaton, each simulated by a
 * single lane with a small register-resident set (the automaton needs edge_sym and
 * pair_row); a chunk whose set outgrows the lane is appended as a CHUNK task to the
 * overflow queue of gbfsm_chunk_io. kind GBFSM_TASK_WHOLE: `count` inputs of automaton `automaton`, whose input
 * indices are input_ids[first .. first + count); an NFA task has count 1 (a warp runs it),
 * a DFA task 1..32 inputs (one lane each). kind GBFSM_TASK_CHUNK: chunk `first` of the
 * chunk table, simulated speculatively (or exactly when it is an input's first chunk);
 * its outcome goes to the chunk records. kind GBFSM_TASK_FIXUP: input whose chunks are
 * chunks[first .. first + count), resolved exactly from the chunk records of an earlier
 * launch; writes the input's verdict. */
typedef struct gbfsm_task {
    int32_t automaton;
    int32_t first;
    int32_t count;
    int32_t kind;
} gbfsm_task;

#define GBFSM_TASK_WHOLE 0
#define GBFSM_TASK_CHUNK 1
#define GBFSM_TASK_FIXUP 2
#define GBFSM_TASK_LANES 3 /* chunks[first .. first + count), count <= 32, one per lane; with
                              automaton -1 each lane runs its chunk's input's automaton
                              (gbfsm_chunk_io.aut_ids) */
#define GBFSM_TASK_DFA_GROUP 4 /* inputs input_ids[first .. first + count), count <= 32, one
                                  DFA walk per lane, each on its input's own DFA
                                  (gbfsm_chunk_io.aut_ids); automaton is -1 */
#define GBFSM_TASK_DFA_CHUNK 5 /* chunk `first` (count 1) of a long input of DFA `automaton`,
                                  walked by a warp from the set of all states until it
                                  collapses to one; its record goes to the chunk records
                                  (gbfsm_dfa_chunks_run) */
#define GBFSM_TASK_DFA_FIXUP 6 /* input whose DFA chunks are chunks[first .. first + count):
                                  its exact verdict from their records, gaps walked
                                  serially (gbfsm_dfa_chunks_run) */

/* A piece of an NFA input: bytes data[begin .. end) of input `input`; `index` counts the
 * input's chunks from 0. Chunks after the first must start at least 2 bytes into the
 * input and span at least 32 bytes. */
typedef struct gbfsm_chunk {
    int32_t input;
    int32_t index;
    int64_t begin;
    int64_t end;
} gbfsm_chunk;

/* Bytes of one chunk record (device scratch written by CHUNK tasks, read by FIXUP). */
#define GBFSM_CHUNK_RECORD_BYTES 256

/* Device buffers of the speculative-chunk machinery (all device pointers; passed by
 * host pointer, NULL when a launch has no CHUNK, LANES or FIXUP task). */
typedef struct gbfsm_chunk_io {
    const gbfsm_chunk *chunks;    /* chunk table */
    void *records;                /* GBFSM_CHUNK_RECORD_BYTES per chunk */
    gbfsm_task *overflow_tasks;   /* LANES tasks append CHUNK tasks here (capacity: chunks) */
    int32_t *overflow_count;      /* entries of overflow_tasks; the caller zeroes it before
                                     the launch that runs LANES tasks */
    const int32_t *task_count;    /* non-NULL: run min(*task_count, n_tasks) tasks, a count
                                     written on the device by an earlier launch */
    int32_t n_chunks;             /* entries of the chunk table (its capacity, when a
                                     device-built table ends with a sentinel chunk whose
                                     index is 0) */
    const int32_t *aut_ids;       /* per-input automaton (device, n_inputs), for LANES tasks
                                     with automaton -1 and DFA_GROUP tasks; NULL = all 0 */
} gbfsm_chunk_io;

/* Scratch bytes for a persistent launch whose largest NFA has `max_words` set words. */
size_t gbfsm_persistent_workspace_bytes(int32_t max_words, const gbfsm_plan *plan);

/* Run `n_tasks` WHOLE, CHUNK and FIXUP tasks (LANES tasks are skipped: they belong to
 * gbfsm_lanes_run). table/tasks/input_ids (and the chunk_io buffers, needed only by
 * CHUNK and FIXUP tasks) are device arrays. Speculative chunking takes up to four calls on
 * one stream: gbfsm_lanes_run for the LANES tasks; this call for the CHUNK tasks (with
 * any WHOLE tasks); this call for the overflow queue (tasks = overflow_tasks,
 * task_count = overflow_count); then this call for the FIXUP tasks. Input i is
 * data[offsets[i] .. ends[i]) when `ends` is non-NULL (spans anywhere in `data`, e.g.
 * requests left in place in a pinned host pool that the device reads directly), else
 * data[offsets[i] .. offsets[i+1]). Results are written by input index. workspace
 * (device, >= gbfsm_persistent_workspace_bytes) holds the queue ticket, which this call
 * resets in-stream, so the launch can be replayed from a graph; concurrent launches need
 * separate workspaces. */
gbfsm_status gbfsm_persistent_run(const gbfsm_automaton *table, int32_t n_automata,
                                  int32_t max_words, const gbfsm_task *tasks, int32_t n_tasks,
                                  const int32_t *input_ids, const uint8_t *data,
                                  const int64_t *offsets, const int64_t *ends,
                                  const gbfsm_chunk_io *chunk_io, int32_t *flags, int32_t *lens,
                                  int32_t *examined, void *workspace, size_t workspace_bytes,
                                  const gbfsm_plan *plan, void *stream);

/* Device address of page-locked host memory (cudaHostGetDevicePointer), for kernels that
 * read request bytes in place over the host link instead of copying them first. No
 * counterpart in the reference (which copies every input, common.cuh:150-159). */
gbfsm_status gbfsm_host_device_pointer(void *host, void **device);

/* Whether the current device reads pageable host memory coherently, without registering
 * it: 0 no, 1 yes, 2 yes through the host's page tables (address translation services, as
 * GB300 over NVLink-C2C); -1 when the device cannot be asked. A query: nothing is
 * accessed. No counterpart in the reference. */
int32_t gbfsm_pageable_access(void);

/* Copy n_inputs inputs into the contiguous device layout of a batch: input i, the bytes
 * src_ptrs[i] .. src_ptrs[i] + (offsets[i+1] - offsets[i]), goes to
 * dst[offsets[i] .. offsets[i+1]). src_ptrs (uint64 addresses) and offsets are device
 * arrays; dst is device memory of at least offsets[n_inputs] rounded up to 16 bytes. A
 * source may be device memory, page-locked host memory mapped into the device, or, where
 * gbfsm_pageable_access() > 0, any pageable host memory; it is read in aligned 16-byte
 * blocks that each hold at least one of its bytes. offsets must not decrease; the copy
 * covers dst[offsets[0] .. offsets[n_inputs]), so a contiguous range of a batch's inputs
 * (src_ptrs + k, offsets + k) is gathered alone, every byte written once (ranges may be
 * gathered concurrently). Warps take 8 KiB windows of the destination; stream-ordered.
 * No counterpart in the reference (which packs and copies every batch on the host). */
gbfsm_status gbfsm_gather_inputs(const uint64_t *src_ptrs, const int64_t *offsets,
                                 int32_t n_inputs, uint8_t *dst, void *stream);

/* Resident warps per SM of the lane launch on the current device (0 when it cannot run):
 * a batch whose LANES tasks fit sm_count times this runs in one wave. No counterpart in
 * the reference. */
int32_t gbfsm_lanes_warps_per_sm(void);

/* Run LANES tasks (one warp per task, one chunk per lane), writing chunk records and
 * appending chunks that outgrow a lane to chunk_io->overflow_tasks (the caller zeroes
 * overflow_count first). A task whose automaton is an NFA without lane tables
 * (gbfsm_nfa_dev.lane_edges and pair_row) sends all its chunks to the overflow queue; a
 * task of a DFA is ignored. data/offsets as for gbfsm_persistent_run (contiguous inputs:
 * input i starts at offsets[i]). No counterpart in the reference. */
gbfsm_status gbfsm_lanes_run(const gbfsm_automaton *table, int32_t n_automata,
                             const gbfsm_task *tasks, int32_t n_tasks, const uint8_t *data,
                             const int64_t *offsets, const gbfsm_chunk_io *chunk_io,
                             void *stream);

/* gbfsm_lanes_run with the task range read on the device: tasks[range[0] .. range[0] +
 * min(range[1], max_tasks)) run, `range` a device int32[2] written by an earlier launch
 * (e.g. a slice's range in a gbfsm_batch_plan header). Resident warps loop over the tasks,
 * so any count runs. No counterpart in the reference. */
gbfsm_status gbfsm_lanes_run_range(const gbfsm_automaton *table, int32_t n_automata,
                                   const gbfsm_task *tasks, int32_t max_tasks,
                                   const int32_t *range, const uint8_t *data,
                                   const int64_t *offsets, const gbfsm_chunk_io *chunk_io,
                                   void *stream);

/* ---------------------------------------------------------------------------------
 * Device-side batch planning (no counterpart in the reference, which launches once per
 * automaton with a thread or warp per whole input). gbfsm_batch_plan builds a batch's
 * whole task queue on the GPU from its offsets and automaton ids -- chunk sizes, the
 * chunk table, the LANES, persistent (WHOLE / CHUNK / DFA_GROUP, longest work first by
 * log2 buckets) and FIXUP tasks, and the input ids -- and writes the counts into a
 * device header that the launches read (gbfsm_lanes_run_range and the task_count of
 * gbfsm_chunk_io), so a step needs no host work and a captured graph re-plans on every
 * replay. Planning costs two small launches (one CTA, then a warp per input).
 * ------------------------------------------------------------------------------- */

/* Automaton classes for planning (gbfsm_batch_plan_args.aut_class). */
#define GBFSM_PLAN_NFA_WHOLE 0 /* NFA inputs run whole, a warp each */
#define GBFSM_PLAN_NFA_WARP 1  /* NFA: inputs of two chunks or more cut into warp chunks
                                  (the automaton needs first_row / first_edges) */
#define GBFSM_PLAN_NFA_LANES 2 /* NFA: every input cut into lane chunks (the automaton
                                  needs the lane tables) */
#define GBFSM_PLAN_DFA 3       /* DFA inputs, 32 per task, one walk per lane; inputs of at
                                  least two DFA chunks (gbfsm_batch_plan_args.aut_dfa_chunk,
                                  dfa_warps) are cut into DFA chunks instead */

/* Words of the plan header (int32, device). */
#define GBFSM_PLAN_HEADER_WORDS 64
#define GBFSM_PLAN_STATUS 0        /* 0 ok; 1 a capacity was too small; 2 an automaton id
                                      out of range. Not 0: every count below is 0. */
#define GBFSM_PLAN_LANE_CHUNKS 1   /* chunks run one per lane: chunks[0 .. this) */
#define GBFSM_PLAN_CHUNKS 2        /* all chunks (lane chunks, warp chunks, DFA chunks) */
#define GBFSM_PLAN_LANE_FIRST 3    /* always 0: {LANE_FIRST, LANE_TASKS} is the range of
                                      every LANES task for gbfsm_lanes_run_range */
#define GBFSM_PLAN_LANE_TASKS 4
#define GBFSM_PLAN_PERSIST_TASKS 5 /* task_count of the persistent launch */
#define GBFSM_PLAN_FIXUP_TASKS 6   /* task_count of the fix-up launch */
#define GBFSM_PLAN_LANE_BYTES 7    /* chosen lane chunk size (before slice scaling) */
#define GBFSM_PLAN_WARP_BYTES 8    /* chosen warp chunk size */
#define GBFSM_PLAN_OVERFLOW 9      /* zeroed: the overflow_count of the lane launch */
#define GBFSM_PLAN_WHOLE 10        /* whole NFA inputs: input_ids[0 .. this) */
#define GBFSM_PLAN_DFA_INPUTS 11   /* DFA inputs: input_ids[WHOLE .. WHOLE + this) */
#define GBFSM_PLAN_DFA_CHUNKS 12   /* task_count of the DFA chunk launch (chunks of long DFA
                                      inputs, after the lane and warp chunks) */
#define GBFSM_PLAN_DFA_FIXUPS 13   /* task_count of the DFA fix-up launch */
#define GBFSM_PLAN_DFA_CHUNK_BYTES 14 /* the batch's DFA chunk length before each DFA's
                                         minimum (0: from aut_dfa_chunk alone) */
#define GBFSM_PLAN_SLICES 16       /* {first, count} LANES task range of slice k at
                                      16 + 2k, for gbfsm_lanes_run_range */
#define GBFSM_PLAN_MAX_SLICES 16

typedef struct gbfsm_batch_plan_args {
    int32_t n_inputs;
    int32_t n_automata;
    const int64_t *offsets;   /* device [n_inputs + 1]: input i starts at offsets[i] */
    const int64_t *ends;      /* device [n_inputs] or NULL: input i ends at ends[i], else at
                                 offsets[i + 1] */
    const int32_t *aut_ids;   /* device [n_inputs] or NULL (all automaton 0) */
    const int32_t *aut_class; /* device [n_automata]: GBFSM_PLAN_* */
    const int32_t *aut_dfa_chunk; /* device [n_automata] or NULL: shortest DFA chunk of each
                                     automaton, bytes (0 = run the DFA's inputs whole) */
    int32_t lane_warps;       /* resident warps of the lane launch (SMs x
                                 gbfsm_lanes_warps_per_sm) */
    int32_t persist_warps;    /* resident warps of the persistent launch */
    int32_t dfa_warps;        /* resident warps of the DFA chunk launch (SMs x
                                 gbfsm_dfa_chunks_warps_per_sm), or 0. An input of DFA a is
                                 cut into chunks of max(aut_dfa_chunk[a], B / dfa_warps)
                                 bytes, B the bytes of the batch's DFA inputs that hold two
                                 chunks of their own minimum, when it holds two of them:
                                 short chunks when few long inputs leave warps idle, one
                                 wave of chunks otherwise */
    int32_t min_chunk;        /* shortest chunk (bytes) */
    int32_t fixed_chunk;      /* > 0: every chunk size; 0: chosen; < 0: never chunk */
    int32_t n_slices;         /* 0 or 1: one lane range; else inputs cut into slices at
                                 slice_first (host values, ascending, slice_first[0] = 0,
                                 slice_first[n_slices] = n_inputs) */
    float shrink;             /* lane chunks of slice k get the size x (1 - shrink k / n),
                                 -4 < shrink < 1 (below 0: later slices get longer chunks) */
    int32_t slice_first[GBFSM_PLAN_MAX_SLICES + 1];
    int32_t cap_chunks;       /* capacities of the output arrays */
    int32_t cap_lane_tasks;
    int32_t cap_persist_tasks;
    int32_t cap_fixup_tasks;
    int32_t cap_dfa_chunk_tasks;
    int32_t cap_dfa_fixup_tasks;
    gbfsm_chunk *chunks;          /* device [cap_chunks] */
    gbfsm_task *tasks_lanes;      /* device [cap_lane_tasks] */
    gbfsm_task *tasks_persist;    /* device [cap_persist_tasks] */
    gbfsm_task *tasks_fixup;      /* device [cap_fixup_tasks] */
    gbfsm_task *tasks_dfa_chunk;  /* device [cap_dfa_chunk_tasks] (needed with aut_dfa_chunk) */
    gbfsm_task *tasks_dfa_fixup;  /* device [cap_dfa_fixup_tasks] (needed with aut_dfa_chunk) */
    int32_t *dfa_latch;           /* device [n_inputs] or NULL: set to INT32_MAX for every
                                     chunked DFA input (the latch of gbfsm_dfa_chunks_run) */
    int32_t *input_ids;           /* device [n_inputs] */
    int32_t *header;              /* device [GBFSM_PLAN_HEADER_WORDS] */
    void *scratch;                /* device, gbfsm_batch_plan_scratch_bytes(n_inputs) */
} gbfsm_batch_plan_args;

/* Scratch bytes gbfsm_batch_plan needs for n_inputs inputs. */
size_t gbfsm_batch_plan_scratch_bytes(int32_t n_inputs);

/* Enqueue the planning launches on `stream`. Validates the arguments on the host;
 * device-side failures (capacity, automaton ids) are reported in the header's status. */
gbfsm_status gbfsm_batch_plan(const gbfsm_batch_plan_args *args, void *stream);

/* Resident warps per SM of gbfsm_dfa_chunks_run for DFAs of up to max_states states (its
 * shared scratch grows with them); 0 when the query fails. */
int32_t gbfsm_dfa_chunks_warps_per_sm(int32_t max_states);

/* Run DFA_CHUNK or DFA_FIXUP tasks (others are skipped): min(*task_count, max_tasks)
 * tasks of `tasks` when task_count is non-NULL, else max_tasks. A step runs the DFA_CHUNK
 * tasks of a batch first, then its DFA_FIXUP tasks in a later launch on the same stream;
 * both read chunk_io->chunks and share chunk_io->records (the first 32 bytes of each
 * chunk's record). max_states: the most states of any DFA the tasks name (1..32768; each
 * warp holds two bitmaps of that many bits in shared memory). A DFA_FIXUP task writes its
 * input's flags / lens (and examined) entries. Input i is data[offsets[i] .. ends[i]) when
 * `ends` is non-NULL, else data[offsets[i] .. offsets[i + 1]). latch (device [n_inputs] or
 * NULL) lets an input's chunks stop early: a chunk that finds an accept certain to be in
 * the input's true walk lowers latch[input] to its index (atomicMin), and a chunk of a
 * higher index stops walking once it sees that -- the verdict lies before it. Its entries
 * must hold INT32_MAX for the chunked inputs when the DFA_CHUNK launch starts
 * (gbfsm_batch_plan writes them when given dfa_latch). No counterpart in the
 * reference, whose DFA kernel walks each input serially with one thread
 * (src/gpufsm/backends/cuda/native/dfa.cu). */
gbfsm_status gbfsm_dfa_chunks_run(const gbfsm_automaton *table, int32_t n_automata,
                                  const gbfsm_task *tasks, int32_t max_tasks,
                                  const int32_t *task_count, const uint8_t *data,
                                  const int64_t *offsets, const int64_t *ends,
                                  const gbfsm_chunk_io *chunk_io, int32_t max_states,
                                  int32_t *flags, int32_t *lens, int32_t *examined,
                                  int32_t *latch, void *stream);

/* Occupancy query for persistent launches: CTAs of `plan` resident per SM. */
int32_t gbfsm_persistent_ctas_per_sm(int32_t max_words, const gbfsm_plan *plan);

/* ---------------------------------------------------------------------------------
 * Reference-shaped host entry points: one per `_cuda.run_*` of
 * src/gpufsm/backends/cuda/native/include/api.hpp:23-104, same argument order and
 * meaning. Arrays are HOST pointers: the CSR as int32 (nfa.py:44-52), accept words as
 * uint64 (packing.py:66-85), the batch as int32 symbols with int32 offsets
 * (packing.py:35-63, num_strings = len(offsets) - 1). Outputs are host arrays of
 * num_strings int32 and *kernel_ms (device time of the simulation launch). The call is
 * synchronous on the legacy default stream, like the reference. Each allocates its
 * device buffers per call and frees them before returning.
 * ------------------------------------------------------------------------------- */

#define GBFSM_HOST_NFA_BATCH_ARGS                                                          \
    const int32_t *sym_row_ptr, const int32_t *sym_targets, const int32_t *sym_symbols,    \
        const int32_t *eps_row_ptr, const int32_t *eps_targets, const uint64_t *accept_words, \
        const int32_t *input_data, const int32_t *input_offsets, int32_t num_strings,     \
        int32_t num_states, int32_t start_state, int32_t uses_any, int32_t *out_flags,     \
        int32_t *out_lens, float *kernel_ms

/* api.hpp:39-44  run_multistream         (bitpacked.cu:233-307)      -> GBFSM_TECH_BITMAP */
gbfsm_status gbfsm_run_multistream(GBFSM_HOST_NFA_BATCH_ARGS);
/* api.hpp:46-51  run_multistream_shared  (bitpacked.cu:310-411)      -> BITMAP, staged edges */
gbfsm_status gbfsm_run_multistream_shared(GBFSM_HOST_NFA_BATCH_ARGS);
/* api.hpp:53-58  run_multistream_async   (bitpacked.cu:420-526)      -> BITMAP, pinned async copies; *kernel_ms is end to end */
gbfsm_status gbfsm_run_multistream_async(GBFSM_HOST_NFA_BATCH_ARGS);
/* api.hpp:62-67  run_worklist            (worklist_register.cu:132-205) -> GBFSM_TECH_BITMAP */
gbfsm_status gbfsm_run_worklist(GBFSM_HOST_NFA_BATCH_ARGS);
/* api.hpp:71-76  run_worklist_global     (worklist_global.cu:347-405) -> GBFSM_TECH_WARP, sets in global scratch */
gbfsm_status gbfsm_run_worklist_global(GBFSM_HOST_NFA_BATCH_ARGS);
/* api.hpp:78-83  run_worklist_warp       (worklist_global.cu:409-468) -> GBFSM_TECH_WARP */
gbfsm_status gbfsm_run_worklist_warp(GBFSM_HOST_NFA_BATCH_ARGS);
/* api.hpp:85-90  run_worklist_compact    (worklist_global.cu:472-528) -> GBFSM_TECH_COMPACT */
gbfsm_status gbfsm_run_worklist_compact(GBFSM_HOST_NFA_BATCH_ARGS);
/* api.hpp:92-97  run_worklist_shared     (worklist_global.cu:533-600) -> GBFSM_TECH_WARP, sets in shared memory */
gbfsm_status gbfsm_run_worklist_shared(GBFSM_HOST_NFA_BATCH_ARGS);

/* api.hpp:23-28 run_dense and api.hpp:32-37 run_bitpacked (one input; dense.cu:66-110,
 * bitpacked.cu:191-231): (accepted, match_len, kernel_ms) for input_symbols[0..input_len). */
gbfsm_status gbfsm_run_dense(const int32_t *sym_row_ptr, const int32_t *sym_targets,
                             const int32_t *sym_symbols, const int32_t *eps_row_ptr,
                             const int32_t *eps_targets, const int8_t *accept,
                             const int32_t *input_symbols, int32_t input_len,
                             int32_t num_states, int32_t start_state, int32_t uses_any,
                             int32_t *accepted, int32_t *match_len, float *kernel_ms);
gbfsm_status gbfsm_run_bitpacked(const int32_t *sym_row_ptr, const int32_t *sym_targets,
                                 const int32_t *sym_symbols, const int32_t *eps_row_ptr,
                                 const int32_t *eps_targets, const uint64_t *accept_words,
                                 const int32_t *input_symbols, int32_t input_len,
                                 int32_t num_states, int32_t start_state, int32_t uses_any,
                                 int32_t *accepted, int32_t *match_len, float *kernel_ms);

/* api.hpp:101-104 run_dfa (dfa.cu:32-71): trans int32 [num_states*256], accept int8. */
gbfsm_status gbfsm_run_dfa(const int32_t *trans, const int8_t *accept, const int32_t *input_data,
                           const int32_t *input_offsets, int32_t num_strings, int32_t num_states,
                           int32_t start_state, int32_t *out_flags, int32_t *out_lens,
                           float *kernel_ms);

/* Byte-batch variants of the host path (no counterpart in the reference): uint8 input
 * bytes and int64 offsets, so 1 byte per symbol crosses the host link instead of 4.
 * `technique` is a GBFSM_TECH_* value; `plan` may be NULL. */
gbfsm_status gbfsm_run_nfa_bytes(const int32_t *sym_row_ptr, const int32_t *sym_targets,
                                 const int32_t *sym_symbols, const int32_t *eps_row_ptr,
                                 const int32_t *eps_targets, const uint8_t *accept,
                                 int32_t num_states, int32_t start_state, const uint8_t *data,
                                 const int64_t *offsets, int32_t num_strings,
                                 const gbfsm_plan *plan, int32_t *out_flags, int32_t *out_lens,
                                 float *kernel_ms);
gbfsm_status gbfsm_run_dfa_bytes(const int32_t *trans, const uint8_t *accept, int32_t num_states,
                                 int32_t start_state, const uint8_t *data, const int64_t *offsets,
                                 int32_t num_strings, const gbfsm_plan *plan, int32_t *out_flags,
                                 int32_t *out_lens, float *kernel_ms);

/* ---------------------------------------------------------------------------------
 * On-chip peak probes (no counterpart in the reference, whose rooflines use nominal
 * DRAM figures). The simulation kernels read edge records and DFA tables that stay in
 * L1/L2/shared memory, so their rooflines need measured L2 and shared-memory figures.
 * Each call enqueues one launch on `stream`; the caller times it with events. Buffers
 * are device buffers owned by the caller; `sink` is a device uint64 that a launch
 * writes only when its checksum equals a fixed constant (it keeps the loads alive).
 * ------------------------------------------------------------------------------- */

/* `passes` passes of 16-byte L2-only loads (ld.global.cg) over `bytes` of `buf` (16-byte
 * aligned) by 8 CTAs of 256 threads per SM: bytes * passes read. */
gbfsm_status gbfsm_probe_l2_read(const void *buf, size_t bytes, int32_t passes, uint64_t *sink,
                                 void *stream);
/* Independent 16-byte loads at pseudo-random entries of `table` (a power-of-two number of
 * 16-byte entries, 16-byte aligned): 8 CTAs of 256 threads per SM, each making
 * loads_per_thread rounded up to a multiple of 8 loads; via_l1 = 0 reads through L2
 * only, 1 through L1 (ld.global.nc). */
gbfsm_status gbfsm_probe_gather16(const void *table, size_t table_bytes, int64_t loads_per_thread,
                                  int32_t via_l1, uint64_t *sink, void *stream);
/* `chains` threads of one CTA each follow p = next[p] & (n - 1) for `steps` dependent
 * L2-only 4-byte loads (n a power of two): the duration / steps is the latency of one
 * dependent load. */
gbfsm_status gbfsm_probe_chase(const uint32_t *next, uint32_t n, int64_t steps, int32_t chains,
                               uint64_t *sink, void *stream);
/* Copy `bytes` (a multiple of 16, both pointers 16-byte aligned) from `src` to `dst` with
 * blocks_per_sm (1..8) CTAs of 256 threads per SM streaming 16-byte vectors. `src` may be
 * page-locked host memory mapped into the device (gbfsm_host_device_pointer): the copy is
 * then driven by the SMs over the host link instead of by a copy engine. */
gbfsm_status gbfsm_probe_copy(void *dst, const void *src, size_t bytes, int32_t blocks_per_sm,
                              void *stream);
/* blocks_per_sm (1..8) CTAs of 256 threads per SM, each thread making `iters` 16-byte
 * bank-conflict-free shared-memory loads: 4096 * iters bytes per CTA. */
gbfsm_status gbfsm_probe_smem(int64_t iters, int32_t blocks_per_sm, uint64_t *sink, void *stream);

/* ---------------------------------------------------------------------------------
 * Synthetic workload generator (host only; no counterpart in the reference, which
 * draws uniform bytes, src/gpufsm/bench/generators.py:139-161). Writes "live" inputs:
 * random walks along symbol edges whose targets do not accept and have symbol edges,
 * so the simulated active set stays non-empty (uniform bytes kill a random NFA within a
 * byte or two). out[offsets[i] .. offsets[i+1]) receives input i; the bytes depend only
 * on (automaton, seed, i). Arrays are HOST arrays in the reference CSR layout.
 * ------------------------------------------------------------------------------- */
int32_t gbfsm_workload_walk(int32_t num_states, const int32_t *sym_row_ptr,
                            const int32_t *sym_targets, const int32_t *sym_symbols,
                            const uint8_t *accept, int32_t start_state, const int64_t *offsets,
                            int32_t n_inputs, uint64_t seed, uint8_t *out, int32_t n_threads);

#ifdef __cplusplus
}
#endif

#endif /* GBFSM_H */
