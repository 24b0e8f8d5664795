// Plain single-launch DFA batch kernels (GBFSM_TECH_DFA_WALK): one thread per input.
// With plan.stage the packed transition table goes to shared memory by the TMA engine:
//   - dfa_walk_kernel<kStaged = true>: the whole table in each CTA, when it fits the
//     opt-in budget;
//   - dfa_cluster_kernel: a 2-byte table of up to 16 x 256 states split by rows over
//     the CTAs of a thread-block cluster (256 states = 128 KiB per CTA), each lookup a
//     distributed-shared-memory load from the CTA that holds the state's row;
// otherwise (or without plan.stage) it is read through L2 with ld.global.nc.
// Replaces dfa_kernel / run_dfa of the reference (dfa.cu:9-71), which reads an int32
// table and an int8 accept array from global memory and int32 input symbols.
#include <map>
#include <mutex>
#include <utility>

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

// ---- cluster-distributed table --------------------------------------------------------

constexpr uint32_t kSliceStatesLog2 = 8;  // states per CTA slice: 256
constexpr uint32_t kSliceBytes = (1u << kSliceStatesLog2) * kAlphabet * 2u;  // 128 KiB
constexpr int kMaxClusterCtas = 16;
constexpr uint32_t kSliceOffset = 16;  // mbarrier (8 B) + staging flag (4 B) + pad

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ uint32_t cluster_size() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}

// Every thread of every CTA of the cluster; orders shared-memory writes before it with
// reads after it across the cluster.
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

__device__ __forceinline__ uint32_t remote_u32(uint32_t local, uint32_t rank) {
    uint32_t remote, v;
    asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(rank));
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(remote));
    return v;
}

// Entry of (state, byte): row state % 256 of the slice held by CTA state / 256 (clamped
// to the cluster, so a corrupt table cannot address a CTA that does not exist).
struct ClusterTable {
    uint32_t slice;     // shared-memory address of the slice (the same offset in every CTA)
    uint32_t last_rank;
    __device__ __forceinline__ uint32_t operator()(uint32_t state, uint32_t byte) const {
        const uint32_t local =
            slice + ((((state & ((1u << kSliceStatesLog2) - 1u)) << 8) | byte) << 1);
        uint32_t remote;
        unsigned short v;
        asm("mapa.shared::cluster.u32 %0, %1, %2;"
            : "=r"(remote)
            : "r"(local), "r"(min(state >> kSliceStatesLog2, last_rank)));
        asm volatile("ld.shared::cluster.u16 %0, [%1];" : "=h"(v) : "r"(remote));
        return v;
    }
};

__global__ void __launch_bounds__(kMaxBlockThreads) dfa_cluster_kernel(
    gbfsm_dfa_dev d, const uint8_t *__restrict__ data, const int64_t *__restrict__ offsets,
    int32_t n_inputs, int32_t *flags, int32_t *lens, int32_t *examined) {
    extern __shared__ __align__(16) uint8_t smem[];
    const uint32_t rank = cluster_rank();
    const uint64_t from = (uint64_t)rank * kSliceBytes;
    const uint32_t bytes =
        from < d.table_bytes ? (uint32_t)min((uint64_t)kSliceBytes, d.table_bytes - from) : 0u;
    const StageCopy c{kSliceOffset, static_cast<const uint8_t *>(d.table) + from, bytes};
    const bool ok = stage_to_smem(smem, reinterpret_cast<uint64_t *>(smem), &c, 1);
    if (threadIdx.x == 0) reinterpret_cast<volatile uint32_t *>(smem)[2] = ok ? 1u : 0u;
    cluster_barrier();
    bool all_ok = true;
    const uint32_t flag_addr = smem_addr(smem + 8);
    for (uint32_t r = 0; r < cluster_size(); ++r) all_ok = all_ok && remote_u32(flag_addr, r);
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i < n_inputs) {
        if (!all_ok) {
            flags[i] = -1;
            lens[i] = 0;
            if (examined) examined[i] = 0;
        } else {
            const int64_t b = offsets[i];
            int32_t f, l;
            int64_t ex;
            dfa_walk_with<uint16_t>(ClusterTable{smem_addr(smem + kSliceOffset),
                                                 cluster_size() - 1u},
                                    d.accept_bits,
                                    (uint32_t)d.start_state, data + b, offsets[i + 1] - b, f, l,
                                    ex);
            flags[i] = f;
            lens[i] = l;
            if (examined) examined[i] = (int32_t)ex;
        }
    }
    cluster_barrier();  // this CTA's slice stays in place until the whole cluster is done
}

// Co-resident clusters of `ctas` CTAs with `threads` threads (0: the cluster shape cannot
// run here), cached per device and shape.
int cluster_capacity(int ctas, int threads) {
    static std::mutex mu;
    static std::map<std::pair<int, int>, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_pair(dev * 1000 + ctas, threads);
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int n = 0;
    const size_t smem = kSliceOffset + kSliceBytes;
    if (cudaFuncSetAttribute(dfa_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) == cudaSuccess &&
        cudaFuncSetAttribute(dfa_cluster_kernel,
                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)ctas);
        cfg.blockDim = dim3((unsigned)threads);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeClusterDimension;
        attr.val.clusterDim.x = (unsigned)ctas;
        attr.val.clusterDim.y = 1;
        attr.val.clusterDim.z = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        if (cudaOccupancyMaxActiveClusters(&n, dfa_cluster_kernel, &cfg) != cudaSuccess) n = 0;
    }
    cudaGetLastError();  // a refused shape is an answer, not a sticky error
    cache[key] = n;
    return n;
}

gbfsm_status launch_cluster(const gbfsm_dfa_dev &d, int ctas, int threads, const uint8_t *data,
                            const int64_t *offsets, int32_t n, int32_t *flags, int32_t *lens,
                            int32_t *examined, cudaStream_t stream) {
    const int per_cluster = ctas * threads;
    const int clusters = (n + per_cluster - 1) / per_cluster;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(clusters * ctas));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = kSliceOffset + kSliceBytes;
    cfg.stream = stream;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = (unsigned)ctas;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    GBFSM_CUDA_TRY(cudaLaunchKernelEx(&cfg, dfa_cluster_kernel, d, data, offsets, n, flags,
                                      lens, examined));
    return GBFSM_OK;
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
    // a 2-byte table too large for one CTA: split over the CTAs of a cluster
    const int ctas = (int)((d.num_states + (1 << kSliceStatesLog2) - 1) >> kSliceStatesLog2);
    if (p.stage && !staged && d.entry_bytes == 2 && ctas >= 2 && ctas <= kMaxClusterCtas &&
        kSliceOffset + kSliceBytes <= budget && p.block_threads <= 0) {
        const int fit = cluster_capacity(ctas, 32);
        if (fit > 0) {
            // spread the inputs over every co-resident cluster before stacking them
            // (a partial warp is fine: every co-resident cluster gets chains)
            const int per_cta = (n_inputs + fit * ctas - 1) / (fit * ctas);
            const int t = per_cta < 32 ? 32 : per_cta > 256 ? 256 : per_cta;
            if (t == 32 || cluster_capacity(ctas, t) > 0)
                return launch_cluster(d, ctas, t, data, offsets, n_inputs, flags, lens,
                                      examined, stream);
        }
    }
    if (d.entry_bytes == 2)
        return launch_typed<uint16_t>(d, staged, threads, data, offsets, n_inputs, flags, lens,
                                      examined, stream);
    if (d.entry_bytes == 4)
        return launch_typed<uint32_t>(d, staged, threads, data, offsets, n_inputs, flags, lens,
                                      examined, stream);
    return fail(GBFSM_INVALID_ARG, "DFA entry_bytes must be 2 or 4 (got %d)", d.entry_bytes);
}

}  // namespace gbfsm
