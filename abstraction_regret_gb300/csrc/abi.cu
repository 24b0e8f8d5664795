// The C ABI of libgbfsm (include/gbfsm.h): argument validation, status codes and the
// thread-local error message, plus the reference-shaped host entry points that stand in
// for the pybind11 functions of src/gpufsm/backends/cuda/native/bindings.cu:11-39.
//
// No C++ exception crosses this boundary: every failure becomes a gbfsm_status and a
// message for gbfsm_last_error() (the reference throws std::runtime_error from
// CUDA_CHECK, common.cuh:63-71, which pybind11 turns into RuntimeError; the Python layer
// of this package maps GBFSM_CUDA_ERROR back to RuntimeError and GBFSM_INVALID_ARG to
// ValueError).
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "engine.hpp"

namespace gbfsm {

namespace {
thread_local char g_error[1024] = "";
constexpr int kMaxDevices = 64;
int g_sm_count[kMaxDevices] = {0};
int g_smem_optin[kMaxDevices] = {0};

int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
    return dev;
}
}  // namespace

gbfsm_status fail(gbfsm_status code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
    return code;
}

gbfsm_status cuda_fail(cudaError_t err, const char *what) {
    snprintf(g_error, sizeof(g_error), "CUDA error in %s: %s (%s)", what, cudaGetErrorString(err),
             cudaGetErrorName(err));
    (void)cudaGetLastError();  // clear a non-sticky error so the next call starts clean
    if (err == cudaErrorMemoryAllocation) return GBFSM_OOM;
    return GBFSM_CUDA_ERROR;
}

int sm_count() {
    const int dev = current_device();
    if (g_sm_count[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
            v = 1;
        g_sm_count[dev] = v;
    }
    return g_sm_count[dev];
}

int smem_optin() {
    const int dev = current_device();
    if (g_smem_optin[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            v <= 0)
            v = 48 * 1024;
        g_smem_optin[dev] = v;
    }
    return g_smem_optin[dev];
}

namespace {

gbfsm_status check_nfa(const gbfsm_nfa_dev *a) {
    if (!a) return fail(GBFSM_INVALID_ARG, "nfa descriptor is NULL");
    if (a->num_states < 1) return fail(GBFSM_INVALID_ARG, "num_states must be >= 1");
    if (a->start_state < 0 || a->start_state >= a->num_states)
        return fail(GBFSM_INVALID_ARG, "start_state %d out of range (0..%d)", a->start_state,
                    a->num_states - 1);
    if (a->num_words != (a->num_states + 63) / 64)
        return fail(GBFSM_INVALID_ARG, "num_words %d != ceil(num_states / 64)", a->num_words);
    if (!a->sym_row || !a->eps_row || !a->accept_words ||
        (a->num_sym_edges && !a->sym_edges) || (a->num_eps_edges && !a->eps_edges))
        return fail(GBFSM_INVALID_ARG, "nfa descriptor has a NULL array");
    if (a->num_sym_edges > 0xffffffffull || a->num_eps_edges > 0xffffffffull)
        return fail(GBFSM_UNSUPPORTED, "more than 2^32 edges");
    return GBFSM_OK;
}

gbfsm_status check_batch(const uint8_t *data, const int64_t *offsets, int32_t n_inputs,
                         const int32_t *flags, const int32_t *lens) {
    if (n_inputs < 0) return fail(GBFSM_INVALID_ARG, "n_inputs must be >= 0");
    if (n_inputs > 0 && (!data || !offsets || !flags || !lens))
        return fail(GBFSM_INVALID_ARG, "data, offsets, flags and lens must be non-NULL");
    return GBFSM_OK;
}

gbfsm_plan plan_or_default(const gbfsm_plan *p, int32_t technique) {
    gbfsm_plan q;
    memset(&q, 0, sizeof(q));
    if (p) q = *p;
    else q.technique = technique;
    return q;
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// The staged launches copy arrays into shared memory with cp.async.bulk, whose source
// must be 16-byte aligned. A plan asking for staging of an NFA whose row or edge arrays
// are not (e.g. views into a larger allocation) runs unstaged, reading them through L2;
// the workspace query and the launch apply the same rule, so they agree.
gbfsm_plan nfa_plan(const gbfsm_nfa_dev &a, const gbfsm_plan *plan) {
    gbfsm_plan p = plan_or_default(plan, GBFSM_TECH_COMPACT);
    const bool eps = (a.flags & GBFSM_NFA_HAS_EPS) != 0;
    if (p.stage && !(aligned16(a.sym_row) && aligned16(a.sym_edges) &&
                     (!eps || (aligned16(a.eps_row) && aligned16(a.eps_edges)))))
        p.stage = 0;
    return p;
}

}  // namespace
}  // namespace gbfsm

using namespace gbfsm;

extern "C" {

int gbfsm_abi_version(void) { return GBFSM_ABI_VERSION; }

const char *gbfsm_last_error(void) { return g_error; }

gbfsm_status gbfsm_nfa_layout(int32_t num_states, const int32_t *sym_row_ptr,
                              const int32_t *sym_targets, const int32_t *sym_symbols,
                              const int32_t *eps_row_ptr, const int32_t *eps_targets,
                              const uint8_t *accept, uint64_t nnz_sym, uint64_t nnz_eps,
                              uint32_t *sym_row, gbfsm_edge *sym_edges, uint32_t *eps_row,
                              gbfsm_edge *eps_edges, uint64_t *accept_words, int32_t *error,
                              void *stream) {
    if (num_states < 1) return fail(GBFSM_INVALID_ARG, "num_states must be >= 1");
    if (!sym_row_ptr || !eps_row_ptr || !accept || !sym_row || !eps_row || !accept_words || !error)
        return fail(GBFSM_INVALID_ARG, "NULL array passed to gbfsm_nfa_layout");
    if (nnz_sym && (!sym_targets || !sym_symbols || !sym_edges))
        return fail(GBFSM_INVALID_ARG, "NULL symbol-edge array with nnz_sym > 0");
    if (nnz_eps && (!eps_targets || !eps_edges))
        return fail(GBFSM_INVALID_ARG, "NULL epsilon-edge array with nnz_eps > 0");
    if (nnz_sym > 0xffffffffull || nnz_eps > 0xffffffffull)
        return fail(GBFSM_UNSUPPORTED, "more than 2^32 edges");
    return launch_nfa_layout(num_states, sym_row_ptr, sym_targets, sym_symbols, eps_row_ptr,
                             eps_targets, accept, nnz_sym, nnz_eps, sym_row, sym_edges, eps_row,
                             eps_edges, accept_words, error, static_cast<cudaStream_t>(stream));
}

gbfsm_status gbfsm_dfa_layout(int32_t num_states, const int32_t *trans, const uint8_t *accept,
                              int32_t entry_bytes, void *table, uint32_t *accept_bits,
                              int32_t *error, void *stream) {
    if (num_states < 1) return fail(GBFSM_INVALID_ARG, "num_states must be >= 1");
    if (!trans || !accept || !table || !accept_bits || !error)
        return fail(GBFSM_INVALID_ARG, "NULL array passed to gbfsm_dfa_layout");
    if (entry_bytes != 2 && entry_bytes != 4)
        return fail(GBFSM_INVALID_ARG, "entry_bytes must be 2 or 4 (got %d)", entry_bytes);
    if (entry_bytes == 2 && num_states > 32768)
        return fail(GBFSM_UNSUPPORTED, "2-byte entries hold at most 32768 states (got %d)",
                    num_states);
    return launch_dfa_layout(num_states, trans, accept, entry_bytes, table, accept_bits, error,
                             static_cast<cudaStream_t>(stream));
}

size_t gbfsm_nfa_workspace_bytes(const gbfsm_nfa_dev *nfa, int32_t n_inputs,
                                 const gbfsm_plan *plan) {
    if (check_nfa(nfa) != GBFSM_OK || n_inputs <= 0) return 0;
    const gbfsm_plan p = nfa_plan(*nfa, plan);
    if (p.technique == GBFSM_TECH_BITMAP) {
        BitmapPlan bp;
        if (make_bitmap_plan(*nfa, n_inputs, p, bp) != GBFSM_OK || bp.sets_in_smem) return 0;
        const size_t grid = (size_t)((n_inputs + bp.threads - 1) / bp.threads);
        return grid * (size_t)bp.threads * (size_t)bp.W * 32u;
    }
    WarpPlan wp;
    if (make_warp_plan(*nfa, n_inputs, p, wp) != GBFSM_OK) return 0;
    return (size_t)n_inputs * wp.global_per_warp;
}

gbfsm_status gbfsm_nfa_run(const gbfsm_nfa_dev *nfa, const uint8_t *data, const int64_t *offsets,
                           int32_t n_inputs, const gbfsm_plan *plan, int32_t *flags,
                           int32_t *lens, int32_t *examined, void *workspace,
                           size_t workspace_bytes, void *stream) {
    gbfsm_status st = check_nfa(nfa);
    if (st != GBFSM_OK) return st;
    if ((st = check_batch(data, offsets, n_inputs, flags, lens)) != GBFSM_OK) return st;
    const gbfsm_plan p = nfa_plan(*nfa, plan);
    const size_t need = gbfsm_nfa_workspace_bytes(nfa, n_inputs, &p);
    if (need > 0 && (workspace == nullptr || workspace_bytes < need))
        return fail(GBFSM_INVALID_ARG, "workspace too small: %zu < %zu bytes", workspace_bytes,
                    need);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (p.technique) {
        case GBFSM_TECH_BITMAP: {
            BitmapPlan bp;
            if ((st = make_bitmap_plan(*nfa, n_inputs, p, bp)) != GBFSM_OK) return st;
            return launch_nfa_bitmap(*nfa, bp, data, offsets, n_inputs, flags, lens, examined,
                                     workspace, s);
        }
        case GBFSM_TECH_WARP:
        case GBFSM_TECH_COMPACT: {
            WarpPlan wp;
            if ((st = make_warp_plan(*nfa, n_inputs, p, wp)) != GBFSM_OK) return st;
            return launch_nfa_warp(*nfa, wp, data, offsets, n_inputs, flags, lens, examined,
                                   workspace, s);
        }
        default:
            return fail(GBFSM_INVALID_ARG, "unknown NFA technique %d", p.technique);
    }
}

gbfsm_status gbfsm_dfa_run(const gbfsm_dfa_dev *dfa, const uint8_t *data, const int64_t *offsets,
                           int32_t n_inputs, const gbfsm_plan *plan, int32_t *flags,
                           int32_t *lens, int32_t *examined, void *stream) {
    if (!dfa) return fail(GBFSM_INVALID_ARG, "dfa descriptor is NULL");
    if (dfa->num_states < 1 || dfa->start_state < 0 || dfa->start_state >= dfa->num_states)
        return fail(GBFSM_INVALID_ARG, "bad DFA descriptor (num_states %d, start %d)",
                    dfa->num_states, dfa->start_state);
    if (!dfa->table || !dfa->accept_bits)
        return fail(GBFSM_INVALID_ARG, "dfa descriptor has a NULL array");
    if (dfa->entry_bytes == 2 && dfa->num_states > 32768)
        return fail(GBFSM_INVALID_ARG, "2-byte entries hold at most 32768 states");
    gbfsm_status st = check_batch(data, offsets, n_inputs, flags, lens);
    if (st != GBFSM_OK) return st;
    gbfsm_plan p = plan_or_default(plan, GBFSM_TECH_DFA_WALK);
    if (!aligned16(dfa->table)) p.stage = 0;  // cp.async.bulk needs an aligned source
    return launch_dfa_walk(*dfa, p, data, offsets, n_inputs, flags, lens, examined,
                           static_cast<cudaStream_t>(stream));
}

gbfsm_status gbfsm_host_device_pointer(void *host, void **device) {
    if (!host || !device) return fail(GBFSM_INVALID_ARG, "NULL pointer");
    *device = nullptr;
    GBFSM_CUDA_TRY(cudaHostGetDevicePointer(device, host, 0));
    return GBFSM_OK;
}

int32_t gbfsm_lanes_warps_per_sm(void) { return lanes_warps_per_sm(); }

gbfsm_status gbfsm_lanes_run(const gbfsm_automaton *table, int32_t n_automata,
                             const gbfsm_task *tasks, int32_t n_tasks, const uint8_t *data,
                             const int64_t *offsets, const gbfsm_chunk_io *chunk_io,
                             void *stream) {
    if (n_tasks < 0 || n_automata < 0) return fail(GBFSM_INVALID_ARG, "negative task count");
    if (n_tasks == 0) return GBFSM_OK;
    if (!table || !tasks || !data || !offsets || !chunk_io || !chunk_io->chunks ||
        !chunk_io->records || !chunk_io->overflow_tasks || !chunk_io->overflow_count)
        return fail(GBFSM_INVALID_ARG, "NULL array passed to gbfsm_lanes_run");
    return launch_lanes(table, n_automata, tasks, n_tasks, nullptr, data, offsets, *chunk_io,
                        static_cast<cudaStream_t>(stream));
}

gbfsm_status gbfsm_lanes_run_range(const gbfsm_automaton *table, int32_t n_automata,
                                   const gbfsm_task *tasks, int32_t max_tasks,
                                   const int32_t *range, const uint8_t *data,
                                   const int64_t *offsets, const gbfsm_chunk_io *chunk_io,
                                   void *stream) {
    if (max_tasks < 0 || n_automata < 0) return fail(GBFSM_INVALID_ARG, "negative task count");
    if (max_tasks == 0) return GBFSM_OK;
    if (!table || !tasks || !range || !data || !offsets || !chunk_io || !chunk_io->chunks ||
        !chunk_io->records || !chunk_io->overflow_tasks || !chunk_io->overflow_count)
        return fail(GBFSM_INVALID_ARG, "NULL array passed to gbfsm_lanes_run_range");
    return launch_lanes(table, n_automata, tasks, max_tasks, range, data, offsets, *chunk_io,
                        static_cast<cudaStream_t>(stream));
}

size_t gbfsm_batch_plan_scratch_bytes(int32_t n_inputs) {
    return batch_plan_scratch_bytes(n_inputs);
}

gbfsm_status gbfsm_batch_plan(const gbfsm_batch_plan_args *a, void *stream) {
    if (!a) return fail(GBFSM_INVALID_ARG, "gbfsm_batch_plan: NULL arguments");
    if (a->n_inputs < 0 || a->n_automata < 1)
        return fail(GBFSM_INVALID_ARG, "gbfsm_batch_plan: %d inputs, %d automata", a->n_inputs,
                    a->n_automata);
    if (a->n_inputs == 0) return GBFSM_OK;
    if (!a->offsets || !a->aut_class || !a->chunks || !a->tasks_lanes || !a->tasks_persist ||
        !a->tasks_fixup || !a->input_ids || !a->header || !a->scratch)
        return fail(GBFSM_INVALID_ARG, "gbfsm_batch_plan: NULL array");
    if (a->min_chunk < 64)
        return fail(GBFSM_INVALID_ARG, "gbfsm_batch_plan: min_chunk %d below 64", a->min_chunk);
    if (a->cap_chunks < 1 || a->cap_lane_tasks < 0 || a->cap_persist_tasks < 0 ||
        a->cap_fixup_tasks < 0 || a->cap_dfa_chunk_tasks < 0 || a->cap_dfa_fixup_tasks < 0)
        return fail(GBFSM_INVALID_ARG, "gbfsm_batch_plan: negative capacity");
    if (a->aut_dfa_chunk && (!a->tasks_dfa_chunk || !a->tasks_dfa_fixup))
        return fail(GBFSM_INVALID_ARG,
                    "gbfsm_batch_plan: aut_dfa_chunk needs tasks_dfa_chunk and tasks_dfa_fixup");
    if (a->n_slices > GBFSM_PLAN_MAX_SLICES)
        return fail(GBFSM_INVALID_ARG, "gbfsm_batch_plan: more than %d slices",
                    GBFSM_PLAN_MAX_SLICES);
    if (a->n_slices > 1) {
        if (a->slice_first[0] != 0 || a->slice_first[a->n_slices] != a->n_inputs)
            return fail(GBFSM_INVALID_ARG, "gbfsm_batch_plan: slices must cover the inputs");
        for (int k = 0; k < a->n_slices; ++k)
            if (a->slice_first[k + 1] < a->slice_first[k])
                return fail(GBFSM_INVALID_ARG, "gbfsm_batch_plan: slices out of order");
        if (!(a->shrink > -4.0f && a->shrink < 1.0f))
            return fail(GBFSM_INVALID_ARG, "gbfsm_batch_plan: shrink must be in (-4, 1)");
    }
    return launch_batch_plan(*a, static_cast<cudaStream_t>(stream));
}

size_t gbfsm_persistent_workspace_bytes(int32_t max_words, const gbfsm_plan *plan) {
    const gbfsm_plan p = plan_or_default(plan, GBFSM_TECH_COMPACT);
    return persistent_workspace_bytes(max_words, p);
}

int32_t gbfsm_persistent_ctas_per_sm(int32_t max_words, const gbfsm_plan *plan) {
    const gbfsm_plan p = plan_or_default(plan, GBFSM_TECH_COMPACT);
    return persistent_ctas_per_sm(max_words, p);
}

gbfsm_status gbfsm_persistent_run(const gbfsm_automaton *table, int32_t n_automata,
                                  int32_t max_words, const gbfsm_task *tasks, int32_t n_tasks,
                                  const int32_t *input_ids, const uint8_t *data,
                                  const int64_t *offsets, const int64_t *ends,
                                  const gbfsm_chunk_io *chunk_io, int32_t *flags, int32_t *lens,
                                  int32_t *examined, void *workspace, size_t workspace_bytes,
                                  const gbfsm_plan *plan, void *stream) {
    if (n_tasks < 0 || n_automata < 0) return fail(GBFSM_INVALID_ARG, "negative task count");
    if (n_tasks > 0 && (!table || !tasks || !input_ids || !data || !offsets || !flags || !lens))
        return fail(GBFSM_INVALID_ARG, "NULL array passed to gbfsm_persistent_run");
    if (max_words < 1) return fail(GBFSM_INVALID_ARG, "max_words must be >= 1");
    const gbfsm_plan p = plan_or_default(plan, GBFSM_TECH_COMPACT);
    return launch_persistent(table, n_automata, max_words, tasks, n_tasks, input_ids, data,
                             offsets, ends,
                             chunk_io, flags, lens, examined, workspace,
                             workspace_bytes, p,
                             static_cast<cudaStream_t>(stream));
}

}  // extern "C"

// -------------------------------------------------------------------------------------
// Reference-shaped host entry points
// -------------------------------------------------------------------------------------

namespace {

// Device buffers of one host call, freed on every exit path.
struct DeviceBuffers {
    std::vector<void *> ptrs;
    ~DeviceBuffers() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <typename T>
    gbfsm_status alloc(T **out, size_t bytes) {
        void *p = nullptr;
        const cudaError_t e = cudaMalloc(&p, bytes < 16 ? 16 : bytes);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        ptrs.push_back(p);
        *out = static_cast<T *>(p);
        return GBFSM_OK;
    }
    template <typename T>
    gbfsm_status upload(T **out, const void *host, size_t bytes) {
        gbfsm_status st = alloc(out, bytes);
        if (st != GBFSM_OK) return st;
        if (bytes) GBFSM_CUDA_TRY(cudaMemcpy(*out, host, bytes, cudaMemcpyHostToDevice));
        return GBFSM_OK;
    }
};

struct Events {
    cudaEvent_t a = nullptr, b = nullptr;
    ~Events() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    gbfsm_status create() {
        GBFSM_CUDA_TRY(cudaEventCreate(&a));
        GBFSM_CUDA_TRY(cudaEventCreate(&b));
        return GBFSM_OK;
    }
};

#define GBFSM_TRY(expr)                         \
    do {                                        \
        gbfsm_status _s = (expr);               \
        if (_s != GBFSM_OK) return _s;          \
    } while (0)

// Upload the reference CSR (host int32 arrays, host uint8 accept) and build the device
// layout. On success *desc describes it; buffers are owned by `buf`.
gbfsm_status build_nfa(DeviceBuffers &buf, const int32_t *srp, const int32_t *stg,
                       const int32_t *ssy, const int32_t *erp, const int32_t *etg,
                       const uint8_t *accept_bytes, int32_t n, int32_t start,
                       gbfsm_nfa_dev *desc) {
    if (n < 1) return fail(GBFSM_INVALID_ARG, "num_states must be >= 1");
    if (start < 0 || start >= n)
        return fail(GBFSM_INVALID_ARG, "start_state %d out of range (0..%d)", start, n - 1);
    if (!srp || !erp || !accept_bytes) return fail(GBFSM_INVALID_ARG, "NULL CSR array");
    const int64_t nnz = srp[n], nne = erp[n];
    if (nnz < 0 || nne < 0) return fail(GBFSM_INVALID_ARG, "negative edge count in row pointers");
    if ((nnz && (!stg || !ssy)) || (nne && !etg)) return fail(GBFSM_INVALID_ARG, "NULL edge array");
    int32_t *d_srp, *d_stg, *d_ssy, *d_erp, *d_etg, *d_err;
    uint8_t *d_acc;
    GBFSM_TRY(buf.upload(&d_srp, srp, sizeof(int32_t) * (n + 1)));
    GBFSM_TRY(buf.upload(&d_stg, stg, sizeof(int32_t) * nnz));
    GBFSM_TRY(buf.upload(&d_ssy, ssy, sizeof(int32_t) * nnz));
    GBFSM_TRY(buf.upload(&d_erp, erp, sizeof(int32_t) * (n + 1)));
    GBFSM_TRY(buf.upload(&d_etg, etg, sizeof(int32_t) * nne));
    GBFSM_TRY(buf.upload(&d_acc, accept_bytes, (size_t)n));
    GBFSM_TRY(buf.alloc(&d_err, sizeof(int32_t)));
    uint32_t *sym_row, *eps_row;
    gbfsm_edge *sym_edges, *eps_edges;
    uint64_t *acc_words;
    const int32_t W = (n + 63) / 64;
    GBFSM_TRY(buf.alloc(&sym_row, pad16(sizeof(uint32_t) * (n + 1))));
    GBFSM_TRY(buf.alloc(&eps_row, pad16(sizeof(uint32_t) * (n + 1))));
    GBFSM_TRY(buf.alloc(&sym_edges, sizeof(gbfsm_edge) * (size_t)nnz));
    GBFSM_TRY(buf.alloc(&eps_edges, sizeof(gbfsm_edge) * (size_t)nne));
    GBFSM_TRY(buf.alloc(&acc_words, pad16(sizeof(uint64_t) * W)));
    GBFSM_TRY(gbfsm_nfa_layout(n, d_srp, d_stg, d_ssy, d_erp, d_etg, d_acc, (uint64_t)nnz,
                               (uint64_t)nne, sym_row, sym_edges, eps_row, eps_edges, acc_words,
                               d_err, nullptr));
    int32_t err = 0;
    GBFSM_CUDA_TRY(cudaMemcpy(&err, d_err, sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (err) return fail(GBFSM_INVALID_ARG, "invalid NFA (layout check code %d)", err);
    bool uses_any = false, has_eps = nne > 0;
    for (int64_t k = 0; k < nnz; ++k) uses_any |= (ssy[k] == GBFSM_ANY_SYMBOL);
    desc->num_states = n;
    desc->start_state = start;
    desc->num_words = W;
    desc->flags = (has_eps ? GBFSM_NFA_HAS_EPS : 0) | (uses_any ? GBFSM_NFA_HAS_ANY : 0);
    desc->sym_row = sym_row;
    desc->sym_edges = sym_edges;
    desc->eps_row = eps_row;
    desc->eps_edges = eps_edges;
    desc->accept_words = acc_words;
    desc->num_sym_edges = (uint64_t)nnz;
    desc->num_eps_edges = (uint64_t)nne;
    return GBFSM_OK;
}

// Upload a reference-format batch (int32 symbols + int32 offsets) as uint8 + int64.
gbfsm_status upload_int32_batch(DeviceBuffers &buf, const int32_t *input_data,
                                const int32_t *input_offsets, int32_t num_strings,
                                uint8_t **d_data, int64_t **d_off) {
    if (num_strings < 0) return fail(GBFSM_INVALID_ARG, "num_strings must be >= 0");
    if (!input_offsets) return fail(GBFSM_INVALID_ARG, "input_offsets is NULL");
    const int64_t total = input_offsets[num_strings];
    if (input_offsets[0] < 0 || total < input_offsets[0])
        return fail(GBFSM_INVALID_ARG, "input offsets are not monotone");
    for (int32_t i = 0; i < num_strings; ++i)
        if (input_offsets[i + 1] < input_offsets[i])
            return fail(GBFSM_INVALID_ARG, "input offsets are not monotone at %d", i);
    if (total > 0 && !input_data) return fail(GBFSM_INVALID_ARG, "input_data is NULL");
    int32_t *d_sym, *d_off32, *d_err;
    GBFSM_TRY(buf.upload(&d_sym, input_data, sizeof(int32_t) * (size_t)total));
    GBFSM_TRY(buf.upload(&d_off32, input_offsets, sizeof(int32_t) * (size_t)(num_strings + 1)));
    GBFSM_TRY(buf.alloc(d_data, pad16((uint64_t)total + 16)));
    GBFSM_TRY(buf.alloc(d_off, sizeof(int64_t) * (size_t)(num_strings + 1)));
    GBFSM_TRY(buf.alloc(&d_err, sizeof(int32_t)));
    GBFSM_CUDA_TRY(cudaMemset(d_err, 0, sizeof(int32_t)));
    GBFSM_TRY(launch_narrow_symbols(d_sym, *d_data, total, d_err, nullptr));
    GBFSM_TRY(launch_widen_offsets(d_off32, *d_off, num_strings + 1, nullptr));
    int32_t err = 0;
    GBFSM_CUDA_TRY(cudaMemcpy(&err, d_err, sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (err) return fail(GBFSM_INVALID_ARG, "input symbol outside 0..255");
    return GBFSM_OK;
}

std::vector<uint8_t> unpack_accept_words(const uint64_t *words, int32_t n) {
    std::vector<uint8_t> out((size_t)n);
    for (int32_t s = 0; s < n; ++s) out[s] = (uint8_t)((words[s >> 6] >> (s & 63)) & 1ull);
    return out;
}

// Time the simulation launch on the legacy default stream (events around it), then copy
// the verdicts back. `end_to_end` times the input upload and result download too.
gbfsm_status run_nfa_host(int32_t technique, int32_t stage, bool end_to_end,
                          const int32_t *srp, const int32_t *stg, const int32_t *ssy,
                          const int32_t *erp, const int32_t *etg, const uint8_t *accept_bytes,
                          int32_t num_states, int32_t start_state, bool int32_batch,
                          const void *data, const void *offsets, int32_t num_strings,
                          int32_t *out_flags, int32_t *out_lens, float *kernel_ms,
                          const gbfsm_plan *plan_in) {
    if (num_strings < 0) return fail(GBFSM_INVALID_ARG, "num_strings must be >= 0");
    if (num_strings > 0 && (!out_flags || !out_lens))
        return fail(GBFSM_INVALID_ARG, "output arrays are NULL");
    DeviceBuffers buf;
    gbfsm_nfa_dev desc;
    GBFSM_TRY(build_nfa(buf, srp, stg, ssy, erp, etg, accept_bytes, num_states, start_state, &desc));
    Events ev;
    GBFSM_TRY(ev.create());
    if (end_to_end) GBFSM_CUDA_TRY(cudaEventRecord(ev.a, nullptr));
    uint8_t *d_data = nullptr;
    int64_t *d_off = nullptr;
    if (int32_batch) {
        GBFSM_TRY(upload_int32_batch(buf, static_cast<const int32_t *>(data),
                                     static_cast<const int32_t *>(offsets), num_strings, &d_data,
                                     &d_off));
    } else {
        const int64_t *off = static_cast<const int64_t *>(offsets);
        if (!off) return fail(GBFSM_INVALID_ARG, "offsets is NULL");
        const int64_t total = off[num_strings];
        GBFSM_TRY(buf.alloc(&d_data, pad16((uint64_t)total + 16)));
        if (total) GBFSM_CUDA_TRY(cudaMemcpy(d_data, data, (size_t)total, cudaMemcpyHostToDevice));
        GBFSM_TRY(buf.upload(&d_off, off, sizeof(int64_t) * (size_t)(num_strings + 1)));
    }
    int32_t *d_flags, *d_lens;
    GBFSM_TRY(buf.alloc(&d_flags, sizeof(int32_t) * (size_t)num_strings));
    GBFSM_TRY(buf.alloc(&d_lens, sizeof(int32_t) * (size_t)num_strings));
    gbfsm_plan p = plan_or_default(plan_in, technique);
    if (!plan_in) p.stage = stage;
    const size_t ws = gbfsm_nfa_workspace_bytes(&desc, num_strings, &p);
    void *d_ws = nullptr;
    if (ws) GBFSM_TRY(buf.alloc(&d_ws, ws));
    if (!end_to_end) GBFSM_CUDA_TRY(cudaEventRecord(ev.a, nullptr));
    GBFSM_TRY(gbfsm_nfa_run(&desc, d_data, d_off, num_strings, &p, d_flags, d_lens, nullptr, d_ws,
                            ws, nullptr));
    if (!end_to_end) GBFSM_CUDA_TRY(cudaEventRecord(ev.b, nullptr));
    if (num_strings) {
        GBFSM_CUDA_TRY(cudaMemcpy(out_flags, d_flags, sizeof(int32_t) * num_strings,
                                  cudaMemcpyDeviceToHost));
        GBFSM_CUDA_TRY(cudaMemcpy(out_lens, d_lens, sizeof(int32_t) * num_strings,
                                  cudaMemcpyDeviceToHost));
    }
    if (end_to_end) GBFSM_CUDA_TRY(cudaEventRecord(ev.b, nullptr));
    GBFSM_CUDA_TRY(cudaEventSynchronize(ev.b));
    float ms = 0.0f;
    GBFSM_CUDA_TRY(cudaEventElapsedTime(&ms, ev.a, ev.b));
    if (kernel_ms) *kernel_ms = ms;
    for (int32_t i = 0; i < num_strings; ++i)
        if (out_flags[i] < 0) return fail(GBFSM_TIMEOUT, "a shared-memory staging wait gave up");
    return GBFSM_OK;
}

gbfsm_status run_nfa_int32(int32_t technique, int32_t stage, bool e2e, const int32_t *srp,
                           const int32_t *stg, const int32_t *ssy, const int32_t *erp,
                           const int32_t *etg, const uint64_t *accept_words,
                           const int32_t *input_data, const int32_t *input_offsets,
                           int32_t num_strings, int32_t num_states, int32_t start_state,
                           int32_t *out_flags, int32_t *out_lens, float *kernel_ms) {
    if (num_states < 1) return fail(GBFSM_INVALID_ARG, "num_states must be >= 1");
    if (!accept_words) return fail(GBFSM_INVALID_ARG, "accept_words is NULL");
    const std::vector<uint8_t> acc = unpack_accept_words(accept_words, num_states);
    return run_nfa_host(technique, stage, e2e, srp, stg, ssy, erp, etg, acc.data(), num_states,
                        start_state, true, input_data, input_offsets, num_strings, out_flags,
                        out_lens, kernel_ms, nullptr);
}

gbfsm_status run_dfa_host(const int32_t *trans, const uint8_t *accept, int32_t num_states,
                          int32_t start_state, bool int32_batch, const void *data,
                          const void *offsets, int32_t num_strings, const gbfsm_plan *plan,
                          int32_t *out_flags, int32_t *out_lens, float *kernel_ms) {
    if (num_states < 1) return fail(GBFSM_INVALID_ARG, "num_states must be >= 1");
    if (start_state < 0 || start_state >= num_states)
        return fail(GBFSM_INVALID_ARG, "start_state %d out of range", start_state);
    if (!trans || !accept) return fail(GBFSM_INVALID_ARG, "NULL DFA array");
    if (num_strings < 0) return fail(GBFSM_INVALID_ARG, "num_strings must be >= 0");
    if (num_strings > 0 && (!out_flags || !out_lens))
        return fail(GBFSM_INVALID_ARG, "output arrays are NULL");
    DeviceBuffers buf;
    const int32_t eb = num_states <= 32768 ? 2 : 4;
    const uint64_t entries = (uint64_t)num_states * kAlphabet;
    int32_t *d_trans, *d_err;
    uint8_t *d_acc;
    void *d_table;
    uint32_t *d_bits;
    GBFSM_TRY(buf.upload(&d_trans, trans, sizeof(int32_t) * entries));
    GBFSM_TRY(buf.upload(&d_acc, accept, (size_t)num_states));
    GBFSM_TRY(buf.alloc(&d_err, sizeof(int32_t)));
    GBFSM_TRY(buf.alloc(&d_table, pad16(entries * (uint64_t)eb)));
    GBFSM_TRY(buf.alloc(&d_bits, pad16(sizeof(uint32_t) * (size_t)((num_states + 31) / 32))));
    GBFSM_TRY(gbfsm_dfa_layout(num_states, d_trans, d_acc, eb, d_table, d_bits, d_err, nullptr));
    int32_t err = 0;
    GBFSM_CUDA_TRY(cudaMemcpy(&err, d_err, sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (err) return fail(GBFSM_INVALID_ARG, "invalid DFA (layout check code %d)", err);
    gbfsm_dfa_dev desc;
    memset(&desc, 0, sizeof(desc));
    desc.num_states = num_states;
    desc.start_state = start_state;
    desc.entry_bytes = eb;
    desc.table = d_table;
    desc.accept_bits = d_bits;
    desc.table_bytes = entries * (uint64_t)eb;
    uint8_t *d_data = nullptr;
    int64_t *d_off = nullptr;
    if (int32_batch) {
        GBFSM_TRY(upload_int32_batch(buf, static_cast<const int32_t *>(data),
                                     static_cast<const int32_t *>(offsets), num_strings, &d_data,
                                     &d_off));
    } else {
        const int64_t *off = static_cast<const int64_t *>(offsets);
        if (!off) return fail(GBFSM_INVALID_ARG, "offsets is NULL");
        const int64_t total = off[num_strings];
        GBFSM_TRY(buf.alloc(&d_data, pad16((uint64_t)total + 16)));
        if (total) GBFSM_CUDA_TRY(cudaMemcpy(d_data, data, (size_t)total, cudaMemcpyHostToDevice));
        GBFSM_TRY(buf.upload(&d_off, off, sizeof(int64_t) * (size_t)(num_strings + 1)));
    }
    int32_t *d_flags, *d_lens;
    GBFSM_TRY(buf.alloc(&d_flags, sizeof(int32_t) * (size_t)num_strings));
    GBFSM_TRY(buf.alloc(&d_lens, sizeof(int32_t) * (size_t)num_strings));
    gbfsm_plan p = plan_or_default(plan, GBFSM_TECH_DFA_WALK);
    if (!plan) p.stage = 1;
    Events ev;
    GBFSM_TRY(ev.create());
    GBFSM_CUDA_TRY(cudaEventRecord(ev.a, nullptr));
    GBFSM_TRY(gbfsm_dfa_run(&desc, d_data, d_off, num_strings, &p, d_flags, d_lens, nullptr,
                            nullptr));
    GBFSM_CUDA_TRY(cudaEventRecord(ev.b, nullptr));
    GBFSM_CUDA_TRY(cudaEventSynchronize(ev.b));
    float ms = 0.0f;
    GBFSM_CUDA_TRY(cudaEventElapsedTime(&ms, ev.a, ev.b));
    if (kernel_ms) *kernel_ms = ms;
    if (num_strings) {
        GBFSM_CUDA_TRY(cudaMemcpy(out_flags, d_flags, sizeof(int32_t) * num_strings,
                                  cudaMemcpyDeviceToHost));
        GBFSM_CUDA_TRY(cudaMemcpy(out_lens, d_lens, sizeof(int32_t) * num_strings,
                                  cudaMemcpyDeviceToHost));
    }
    for (int32_t i = 0; i < num_strings; ++i)
        if (out_flags[i] < 0) return fail(GBFSM_TIMEOUT, "a shared-memory staging wait gave up");
    return GBFSM_OK;
}

}  // namespace

extern "C" {

#define GBFSM_FORWARD_NFA_BATCH(TECH, STAGE, E2E)                                            \
    return run_nfa_int32(TECH, STAGE, E2E, sym_row_ptr, sym_targets, sym_symbols, eps_row_ptr, \
                         eps_targets, accept_words, input_data, input_offsets, num_strings,  \
                         num_states, start_state, out_flags, out_lens, kernel_ms)

gbfsm_status gbfsm_run_multistream(GBFSM_HOST_NFA_BATCH_ARGS) {
    (void)uses_any;
    GBFSM_FORWARD_NFA_BATCH(GBFSM_TECH_BITMAP, 0, false);
}
gbfsm_status gbfsm_run_multistream_shared(GBFSM_HOST_NFA_BATCH_ARGS) {
    (void)uses_any;
    GBFSM_FORWARD_NFA_BATCH(GBFSM_TECH_BITMAP, 1, false);
}
gbfsm_status gbfsm_run_multistream_async(GBFSM_HOST_NFA_BATCH_ARGS) {
    (void)uses_any;
    GBFSM_FORWARD_NFA_BATCH(GBFSM_TECH_BITMAP, 0, true);
}
gbfsm_status gbfsm_run_worklist(GBFSM_HOST_NFA_BATCH_ARGS) {
    (void)uses_any;
    GBFSM_FORWARD_NFA_BATCH(GBFSM_TECH_BITMAP, 1, false);
}
gbfsm_status gbfsm_run_worklist_global(GBFSM_HOST_NFA_BATCH_ARGS) {
    (void)uses_any;
    GBFSM_FORWARD_NFA_BATCH(GBFSM_TECH_WARP, 0, false);
}
gbfsm_status gbfsm_run_worklist_warp(GBFSM_HOST_NFA_BATCH_ARGS) {
    (void)uses_any;
    GBFSM_FORWARD_NFA_BATCH(GBFSM_TECH_WARP, 0, false);
}
gbfsm_status gbfsm_run_worklist_compact(GBFSM_HOST_NFA_BATCH_ARGS) {
    (void)uses_any;
    GBFSM_FORWARD_NFA_BATCH(GBFSM_TECH_COMPACT, 0, false);
}
gbfsm_status gbfsm_run_worklist_shared(GBFSM_HOST_NFA_BATCH_ARGS) {
    (void)uses_any;
    GBFSM_FORWARD_NFA_BATCH(GBFSM_TECH_WARP, 1, false);
}

static gbfsm_status run_single(int32_t technique, const int32_t *srp, const int32_t *stg,
                               const int32_t *ssy, const int32_t *erp, const int32_t *etg,
                               const uint8_t *acc, const int32_t *input_symbols, int32_t input_len,
                               int32_t num_states, int32_t start_state, int32_t *accepted,
                               int32_t *match_len, float *kernel_ms) {
    if (input_len < 0) return fail(GBFSM_INVALID_ARG, "input_len must be >= 0");
    if (!accepted || !match_len) return fail(GBFSM_INVALID_ARG, "output pointers are NULL");
    const int32_t off[2] = {0, input_len};
    return run_nfa_host(technique, 1, false, srp, stg, ssy, erp, etg, acc, num_states,
                        start_state, true, input_symbols, off, 1, accepted, match_len, kernel_ms,
                        nullptr);
}

gbfsm_status gbfsm_run_dense(const int32_t *sym_row_ptr, const int32_t *sym_targets,
                             const int32_t *sym_symbols, const int32_t *eps_row_ptr,
                             const int32_t *eps_targets, const int8_t *accept,
                             const int32_t *input_symbols, int32_t input_len,
                             int32_t num_states, int32_t start_state, int32_t uses_any,
                             int32_t *accepted, int32_t *match_len, float *kernel_ms) {
    (void)uses_any;
    if (num_states < 1 || !accept) return fail(GBFSM_INVALID_ARG, "bad num_states or accept");
    std::vector<uint8_t> acc((size_t)num_states);
    for (int32_t s = 0; s < num_states; ++s) acc[s] = accept[s] != 0;
    return run_single(GBFSM_TECH_BITMAP, sym_row_ptr, sym_targets, sym_symbols, eps_row_ptr,
                      eps_targets, acc.data(), input_symbols, input_len, num_states, start_state,
                      accepted, match_len, kernel_ms);
}

gbfsm_status gbfsm_run_bitpacked(const int32_t *sym_row_ptr, const int32_t *sym_targets,
                                 const int32_t *sym_symbols, const int32_t *eps_row_ptr,
                                 const int32_t *eps_targets, const uint64_t *accept_words,
                                 const int32_t *input_symbols, int32_t input_len,
                                 int32_t num_states, int32_t start_state, int32_t uses_any,
                                 int32_t *accepted, int32_t *match_len, float *kernel_ms) {
    (void)uses_any;
    if (num_states < 1 || !accept_words) return fail(GBFSM_INVALID_ARG, "bad num_states or accept");
    const std::vector<uint8_t> acc = unpack_accept_words(accept_words, num_states);
    return run_single(GBFSM_TECH_BITMAP, sym_row_ptr, sym_targets, sym_symbols, eps_row_ptr,
                      eps_targets, acc.data(), input_symbols, input_len, num_states, start_state,
                      accepted, match_len, kernel_ms);
}

gbfsm_status gbfsm_run_dfa(const int32_t *trans, const int8_t *accept, const int32_t *input_data,
                           const int32_t *input_offsets, int32_t num_strings, int32_t num_states,
                           int32_t start_state, int32_t *out_flags, int32_t *out_lens,
                           float *kernel_ms) {
    if (num_states < 1 || !accept) return fail(GBFSM_INVALID_ARG, "bad num_states or accept");
    std::vector<uint8_t> acc((size_t)num_states);
    for (int32_t s = 0; s < num_states; ++s) acc[s] = accept[s] != 0;
    return run_dfa_host(trans, acc.data(), num_states, start_state, true, input_data,
                        input_offsets, num_strings, nullptr, out_flags, out_lens, kernel_ms);
}

gbfsm_status gbfsm_run_nfa_bytes(const int32_t *sym_row_ptr, const int32_t *sym_targets,
                                 const int32_t *sym_symbols, const int32_t *eps_row_ptr,
                                 const int32_t *eps_targets, const uint8_t *accept,
                                 int32_t num_states, int32_t start_state, const uint8_t *data,
                                 const int64_t *offsets, int32_t num_strings,
                                 const gbfsm_plan *plan, int32_t *out_flags, int32_t *out_lens,
                                 float *kernel_ms) {
    return run_nfa_host(plan ? plan->technique : GBFSM_TECH_COMPACT, 0, false, sym_row_ptr,
                        sym_targets, sym_symbols, eps_row_ptr, eps_targets, accept, num_states,
                        start_state, false, data, offsets, num_strings, out_flags, out_lens,
                        kernel_ms, plan);
}

gbfsm_status gbfsm_run_dfa_bytes(const int32_t *trans, const uint8_t *accept, int32_t num_states,
                                 int32_t start_state, const uint8_t *data, const int64_t *offsets,
                                 int32_t num_strings, const gbfsm_plan *plan, int32_t *out_flags,
                                 int32_t *out_lens, float *kernel_ms) {
    return run_dfa_host(trans, accept, num_states, start_state, false, data, offsets, num_strings,
                        plan, out_flags, out_lens, kernel_ms);
}

}  // extern "C"
