// Plain single-launch DFA batch kernel (GBFSM_TECH_DFA_WALK): one thread per input,
// the packed transition table staged in shared memory by the TMA engine when it fits
// the opt-in budget (plan.stage), read through L2 with ld.global.nc otherwise.
// Replaces dfa_kernel / run_dfa of the reference (dfa.cu:9-71), which reads an int32
// table and an int8 accept array from global memory and int32 input symbols.
#include "common.cuh"
#include "dfa_device.cuh"
#include "engine.hpp"

namespace gbfsm {
namespace {

template <typename Entry, bool kStaged>
__global__ void __launch_bounds__(kMaxBlockThreads) dfa_walk_kernel(gbfsm_dfa_dev d,
                                                        const uint8_t *__restrict__ data,
                                                        const int64_t *__restrict__ offsets,
                                                        int32_t n_inputs, int32_t *flags,
                                                        int32_t *lens, int32_t *examined,
                                                        uint32_t staged_bytes) {
    extern __shared__ __align__(16) uint8_t smem[];
    const Entry *table = static_cast<const Entry *>(d.table);
    bool ok = true;
    if (kStaged) {
        const StageCopy c{16u, d.table, staged_bytes};
        ok = stage_to_smem(smem, reinterpret_cast<uint64_t *>(smem), &c, 1);
        table = reinterpret_cast<const Entry *>(smem + 16);
    }
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n_inputs) return;
    if (!ok) {
        flags[i] = -1;
        lens[i] = 0;
        if (examined) examined[i] = 0;
        return;
    }
    const int64_t b = offsets[i];
    int32_t f, l;
    int64_t ex;
    dfa_walk<Entry, kStaged>(table, d.accept_bits, (uint32_t)d.start_state, data + b,
                             offsets[i + 1] - b, f, l, ex);
    flags[i] = f;
    lens[i] = l;
    if (examined) examined[i] = (int32_t)ex;
}

template <typename K>
cudaError_t allow_smem(K kernel, size_t bytes) {
    if (bytes <= 48u * 1024u) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename Entry>
gbfsm_status launch_typed(const gbfsm_dfa_dev &d, bool staged, int threads, const uint8_t *data,
                          const int64_t *offsets, int32_t n, int32_t *flags, int32_t *lens,
                          int32_t *examined, cudaStream_t stream) {
    const dim3 grid((unsigned)((n + threads - 1) / threads));
    const dim3 block((unsigned)threads);
    if (staged) {
        const uint32_t bytes = pad16(d.table_bytes);
        const size_t smem = 16u + bytes;
        GBFSM_CUDA_TRY(allow_smem(dfa_walk_kernel<Entry, true>, smem));
        dfa_walk_kernel<Entry, true><<<grid, block, smem, stream>>>(d, data, offsets, n, flags,
                                                                    lens, examined, bytes);
    } else {
        dfa_walk_kernel<Entry, false><<<grid, block, 0, stream>>>(d, data, offsets, n, flags, lens,
                                                                  examined, 0u);
    }
    GBFSM_LAUNCH_CHECK("dfa_walk_kernel launch");
    return GBFSM_OK;
}

}  // namespace

gbfsm_status launch_dfa_walk(const gbfsm_dfa_dev &d, const gbfsm_plan &p, const uint8_t *data,
                             const int64_t *offsets, int32_t n_inputs, int32_t *flags,
                             int32_t *lens, int32_t *examined, cudaStream_t stream) {
    if (n_inputs <= 0) return GBFSM_OK;
    int threads = p.block_threads;
    if (threads <= 0) {
        // spread the chains over every SM before stacking them in one CTA
        const int per_sm = (n_inputs + sm_count() - 1) / sm_count();
        threads = ((per_sm + 31) / 32) * 32;
        if (threads < 32) threads = 32;
        if (threads > 256) threads = 256;
    }
    if (threads % 32 != 0 || threads > kMaxBlockThreads)
        return fail(GBFSM_INVALID_ARG, "block_threads must be a multiple of 32 up to 256 (got %d)",
                    threads);
    const size_t budget = (size_t)smem_optin() - kSmemReserve;
    const bool staged = p.stage && (16u + (size_t)pad16(d.table_bytes) <= budget);
    if (d.entry_bytes == 2)
        return launch_typed<uint16_t>(d, staged, threads, data, offsets, n_inputs, flags, lens,
                                      examined, stream);
    if (d.entry_bytes == 4)
        return launch_typed<uint32_t>(d, staged, threads, data, offsets, n_inputs, flags, lens,
                                      examined, stream);
    return fail(GBFSM_INVALID_ARG, "DFA entry_bytes must be 2 or 4 (got %d)", d.entry_bytes);
}

}  // namespace gbfsm
