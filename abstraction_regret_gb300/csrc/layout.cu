// Device-side construction of the engine's automaton layouts from the reference's arrays,
// with validation (an out-of-range index would otherwise be read unchecked by the
// simulation kernels, the hazard noted at src/gpufsm/core/dfa.py:74-84).
//
//   NFA: CSR (core/nfa.py:60-65) -> row arrays (uint32) + 16-byte edge records carrying
//        the target's accept/epsilon flags and edge-row range + packed accept words
//        (the pack_accept layout, core/packing.py:66-85).
//   DFA: int32 table (core/dfa.py:36-41) -> 2- or 4-byte entries with accept[successor]
//        in the top bit + packed accept bits.
// Error codes written to *error (first one wins): 1 row pointers, 2 symbol target,
// 3 symbol label, 4 epsilon target, 5 DFA successor, 6 input symbol outside 0..255.
#include "common.cuh"
#include "engine.hpp"

namespace gbfsm {
namespace {

constexpr int kLayoutThreads = 256;

__device__ __forceinline__ void flag_error(int32_t *error, int32_t code) {
    atomicCAS(error, 0, code);
}

__global__ void nfa_rows_kernel(int32_t n, const int32_t *srp, const int32_t *erp,
                                uint64_t nnz_sym, uint64_t nnz_eps, uint32_t *sym_row,
                                uint32_t *eps_row, int32_t *error) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s <= n;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = srp[s], e = erp[s];
        bool bad = a < 0 || e < 0 || (uint64_t)a > nnz_sym || (uint64_t)e > nnz_eps;
        if (s == 0) bad |= (a != 0) || (e != 0);
        if (s == n) bad |= ((uint64_t)a != nnz_sym) || ((uint64_t)e != nnz_eps);
        if (s < n) bad |= (srp[s + 1] < a) || (erp[s + 1] < e);
        if (bad) flag_error(error, 1);
        sym_row[s] = (uint32_t)a;
        eps_row[s] = (uint32_t)e;
    }
}

__device__ __forceinline__ uint32_t state_flags(int32_t t, const uint8_t *accept,
                                                const int32_t *erp) {
    uint32_t f = 0;
    if (accept[t]) f |= GBFSM_EDGE_ACCEPT;
    if (erp[t + 1] > erp[t]) f |= GBFSM_EDGE_HAS_EPS;
    return f;
}

__global__ void nfa_edges_kernel(int32_t n, const int32_t *srp, const int32_t *targets,
                                 const int32_t *symbols, const int32_t *erp,
                                 const uint8_t *accept, uint64_t nnz, bool labelled,
                                 gbfsm_edge *out, int32_t *error) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nnz;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t t = targets[k];
        uint32_t sym = GBFSM_EDGE_SYMBOL_MASK;
        if (labelled) {
            const int32_t s = symbols[k];
            if (s < 0 || s > GBFSM_ANY_SYMBOL) {
                flag_error(error, 3);
                continue;
            }
            sym = (uint32_t)s;
        }
        if (t < 0 || t >= n) {
            flag_error(error, labelled ? 2 : 4);
            continue;
        }
        gbfsm_edge r;
        r.target = (uint32_t)t;
        r.info = sym | state_flags(t, accept, erp);
        r.row_begin = (uint32_t)srp[t];
        r.row_end = (uint32_t)srp[t + 1];
        out[k] = r;
    }
}

__global__ void accept_words_kernel(int32_t n, const uint8_t *accept, uint64_t *words, int32_t W) {
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < W; w += gridDim.x * blockDim.x) {
        uint64_t x = 0;
        const int base = w * 64;
        for (int b = 0; b < 64 && base + b < n; ++b)
            if (accept[base + b]) x |= 1ull << b;
        words[w] = x;
    }
}

template <typename Entry>
__global__ void dfa_table_kernel(int32_t n, const int32_t *trans, const uint8_t *accept,
                                 Entry *table, int32_t *error) {
    const uint64_t total = (uint64_t)n * kAlphabet;
    const uint32_t acc_bit = 1u << (sizeof(Entry) * 8 - 1);
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < total;
         k += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t t = trans[k];
        if (t < 0 || t >= n) {
            flag_error(error, 5);
            table[k] = 0;
            continue;
        }
        table[k] = (Entry)((uint32_t)t | (accept[t] ? acc_bit : 0u));
    }
}

__global__ void accept_bits_kernel(int32_t n, const uint8_t *accept, uint32_t *bits) {
    const int words = (n + 31) / 32;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < words; w += gridDim.x * blockDim.x) {
        uint32_t x = 0;
        for (int b = 0; b < 32 && w * 32 + b < n; ++b)
            if (accept[w * 32 + b]) x |= 1u << b;
        bits[w] = x;
    }
}

__global__ void narrow_kernel(const int32_t *src, uint8_t *dst, int64_t n, int32_t *error) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = src[k];
        if (v < 0 || v > 255) flag_error(error, 6);
        dst[k] = (uint8_t)v;
    }
}

__global__ void widen_kernel(const int32_t *src, int64_t *dst, int64_t n) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        dst[k] = (int64_t)src[k];
}

unsigned grid_for(uint64_t n) {
    const uint64_t want = (n + kLayoutThreads - 1) / kLayoutThreads;
    const uint64_t cap = (uint64_t)sm_count() * 8u;
    return (unsigned)(want < 1 ? 1 : (want > cap ? cap : want));
}

}  // namespace

gbfsm_status launch_nfa_layout(int32_t n, const int32_t *srp, const int32_t *stg,
                               const int32_t *ssy, const int32_t *erp, const int32_t *etg,
                               const uint8_t *accept, uint64_t nnz_sym, uint64_t nnz_eps,
                               uint32_t *sym_row, gbfsm_edge *sym_edges, uint32_t *eps_row,
                               gbfsm_edge *eps_edges, uint64_t *accept_words, int32_t *error,
                               cudaStream_t stream) {
    GBFSM_CUDA_TRY(cudaMemsetAsync(error, 0, sizeof(int32_t), stream));
    nfa_rows_kernel<<<grid_for((uint64_t)n + 1), kLayoutThreads, 0, stream>>>(
        n, srp, erp, nnz_sym, nnz_eps, sym_row, eps_row, error);
    if (nnz_sym)
        nfa_edges_kernel<<<grid_for(nnz_sym), kLayoutThreads, 0, stream>>>(
            n, srp, stg, ssy, erp, accept, nnz_sym, true, sym_edges, error);
    if (nnz_eps)
        nfa_edges_kernel<<<grid_for(nnz_eps), kLayoutThreads, 0, stream>>>(
            n, srp, etg, nullptr, erp, accept, nnz_eps, false, eps_edges, error);
    const int32_t W = (n + 63) / 64;
    accept_words_kernel<<<grid_for((uint64_t)W), kLayoutThreads, 0, stream>>>(n, accept,
                                                                              accept_words, W);
    GBFSM_LAUNCH_CHECK("NFA layout kernels");
    return GBFSM_OK;
}

gbfsm_status launch_dfa_layout(int32_t n, const int32_t *trans, const uint8_t *accept,
                               int32_t entry_bytes, void *table, uint32_t *accept_bits,
                               int32_t *error, cudaStream_t stream) {
    GBFSM_CUDA_TRY(cudaMemsetAsync(error, 0, sizeof(int32_t), stream));
    const uint64_t total = (uint64_t)n * kAlphabet;
    if (entry_bytes == 2)
        dfa_table_kernel<uint16_t><<<grid_for(total), kLayoutThreads, 0, stream>>>(
            n, trans, accept, static_cast<uint16_t *>(table), error);
    else
        dfa_table_kernel<uint32_t><<<grid_for(total), kLayoutThreads, 0, stream>>>(
            n, trans, accept, static_cast<uint32_t *>(table), error);
    accept_bits_kernel<<<grid_for((uint64_t)(n + 31) / 32), kLayoutThreads, 0, stream>>>(
        n, accept, accept_bits);
    GBFSM_LAUNCH_CHECK("DFA layout kernels");
    return GBFSM_OK;
}

gbfsm_status launch_narrow_symbols(const int32_t *src, uint8_t *dst, int64_t n, int32_t *error,
                                   cudaStream_t stream) {
    if (n <= 0) return GBFSM_OK;
    narrow_kernel<<<grid_for((uint64_t)n), kLayoutThreads, 0, stream>>>(src, dst, n, error);
    GBFSM_LAUNCH_CHECK("narrow_kernel");
    return GBFSM_OK;
}

gbfsm_status launch_widen_offsets(const int32_t *src, int64_t *dst, int64_t n,
                                  cudaStream_t stream) {
    if (n <= 0) return GBFSM_OK;
    widen_kernel<<<grid_for((uint64_t)n), kLayoutThreads, 0, stream>>>(src, dst, n);
    GBFSM_LAUNCH_CHECK("widen_kernel");
    return GBFSM_OK;
}

}  // namespace gbfsm
