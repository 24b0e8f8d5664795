// On-chip peak microbenchmarks: the denominators of the L2 and shared-memory rooflines.
//
// The simulation kernels are bound by on-chip memory (edge records and DFA tables that
// stay in L1/L2/shared memory), not by HBM, so their rooflines need measured on-chip
// figures. Each entry point below enqueues one launch on the caller's stream over
// caller-allocated device buffers; the caller times it with CUDA events. Every kernel
// folds what it loads into a value that is written to `sink` only when it equals a
// constant it practically never equals, so the loads cannot be dropped.
//
//   gbfsm_probe_l2_read:   streaming 16-byte loads (ld.global.cg: cached in L2 only) over
//                          an L2-resident buffer, every SM busy -> L2 read bandwidth;
//   gbfsm_probe_gather16:  independent 16-byte loads at pseudo-random addresses of a table
//                          (through L2 only, or through L1 as the lane kernel reads its
//                          records) -> gathered records per second;
//   gbfsm_probe_chase:     a dependent chain of 4-byte loads over a permutation given by
//                          the caller -> latency of one dependent L2 load;
//   gbfsm_probe_smem:      16-byte conflict-free shared-memory loads -> shared bandwidth.
//
// No counterpart in the reference, whose roofline uses nominal DRAM figures only.
#include "common.cuh"
#include "engine.hpp"

namespace gbfsm {
namespace {

constexpr uint32_t kSinkMagic = 0x9e3779b9u;

__device__ __forceinline__ uint4 ld_l2_only16(const uint4 *p) {
    uint4 v;
    asm volatile("ld.global.cg.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

__device__ __forceinline__ uint4 ld_l1_16(const uint4 *p) {
    uint4 v;
    asm volatile("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

__device__ __forceinline__ uint32_t ld_l2_only4(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.global.cg.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ void sink_if(uint32_t x, uint64_t *sink) {
    if (x == kSinkMagic) sink[0] = x;
}

__global__ void __launch_bounds__(256) l2_read_kernel(const uint4 *__restrict__ buf,
                                                      uint64_t n_vec, int32_t passes,
                                                      uint64_t *sink) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t acc = 0;
    for (int32_t p = 0; p < passes; ++p) {
        uint64_t i = tid;
        // four independent loads in flight per thread
        for (; i + 3 * stride < n_vec; i += 4 * stride) {
            const uint4 a = ld_l2_only16(buf + i);
            const uint4 b = ld_l2_only16(buf + i + stride);
            const uint4 c = ld_l2_only16(buf + i + 2 * stride);
            const uint4 d = ld_l2_only16(buf + i + 3 * stride);
            acc ^= a.x ^ b.y ^ c.z ^ d.w;
        }
        for (; i < n_vec; i += stride) acc ^= ld_l2_only16(buf + i).x;
    }
    sink_if(acc, sink);
}

__device__ __forceinline__ uint32_t xorshift32(uint32_t &s) {
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return s;
}

template <bool kViaL1>
__global__ void __launch_bounds__(256) gather16_kernel(const uint4 *__restrict__ table,
                                                       uint32_t mask, int64_t loads,
                                                       uint64_t *sink) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t s = tid * 2654435761u + 0x2545F491u;
    if (s == 0) s = 1;
    uint32_t acc = 0;
    for (int64_t k = 0; k < loads; k += 8) {
        uint32_t idx[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) idx[u] = xorshift32(s) & mask;
        uint4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = kViaL1 ? ld_l1_16(table + idx[u]) : ld_l2_only16(table + idx[u]);
#pragma unroll
        for (int u = 0; u < 8; ++u) acc ^= v[u].x ^ v[u].w;
    }
    sink_if(acc, sink);
}

__global__ void chase_kernel(const uint32_t *__restrict__ next, uint32_t mask, int64_t steps,
                             uint64_t *sink) {
    // one chain per thread, started at different entries; each load depends on the last
    // (the mask keeps every index inside the n = mask + 1 entries whatever they hold)
    uint32_t p = (threadIdx.x * 2654435761u) & mask;
    for (int64_t k = 0; k < steps; ++k) p = ld_l2_only4(next + p) & mask;
    sink_if(p, sink);
}

constexpr int kSmemVecs = 2048;  // 32 KiB of 16-byte vectors per CTA

__global__ void __launch_bounds__(256) smem_kernel(int64_t iters, uint64_t *sink) {
    __shared__ uint4 buf[kSmemVecs];
    for (int i = threadIdx.x; i < kSmemVecs; i += blockDim.x)
        buf[i] = make_uint4(i, i * 3u, i * 5u, i * 7u);
    __syncthreads();
    const uint32_t base = smem_addr(buf);
    uint32_t acc = 0;
    uint32_t slot = threadIdx.x;
    for (int64_t it = 0; it < iters; ++it) {
        // consecutive lanes read consecutive vectors: no bank conflicts
        uint32_t x, y, z, w;
        asm volatile("ld.shared.v4.u32 {%0,%1,%2,%3}, [%4];"
                     : "=r"(x), "=r"(y), "=r"(z), "=r"(w)
                     : "r"(base + (slot & (kSmemVecs - 1)) * 16u));
        acc ^= x ^ y ^ z ^ w;
        slot += 32u;
    }
    sink_if(acc, sink);
}

// Copy `n_vec` 16-byte vectors from `src` (device memory, or page-locked host memory
// mapped into the device's address space) to `dst`: every thread streams its vectors
// with four independent loads in flight.
__global__ void __launch_bounds__(256) copy16_kernel(uint4 *__restrict__ dst,
                                                     const uint4 *__restrict__ src,
                                                     uint64_t n_vec) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t i = tid;
    for (; i + 3 * stride < n_vec; i += 4 * stride) {
        const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride],
                    d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n_vec; i += stride) dst[i] = src[i];
}

int probe_grid(int blocks_per_sm) { return sm_count() * blocks_per_sm; }

}  // namespace
}  // namespace gbfsm

using namespace gbfsm;

extern "C" {

gbfsm_status gbfsm_probe_l2_read(const void *buf, size_t bytes, int32_t passes, uint64_t *sink,
                                 void *stream) {
    if (!buf || !sink || bytes < 16 || passes < 1)
        return fail(GBFSM_INVALID_ARG, "gbfsm_probe_l2_read: bad buffer, size or passes");
    if ((reinterpret_cast<uintptr_t>(buf) & 15u) != 0)
        return fail(GBFSM_INVALID_ARG, "gbfsm_probe_l2_read: buffer not 16-byte aligned");
    l2_read_kernel<<<probe_grid(8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const uint4 *>(buf), (uint64_t)(bytes / 16), passes, sink);
    GBFSM_LAUNCH_CHECK("l2_read_kernel launch");
    return GBFSM_OK;
}

gbfsm_status gbfsm_probe_gather16(const void *table, size_t table_bytes, int64_t loads_per_thread,
                                  int32_t via_l1, uint64_t *sink, void *stream) {
    const size_t n_vec = table_bytes / 16;
    if (!table || !sink || n_vec == 0 || (n_vec & (n_vec - 1)) != 0 || n_vec > (1ull << 31) ||
        loads_per_thread < 8)
        return fail(GBFSM_INVALID_ARG,
                    "gbfsm_probe_gather16: table of a power-of-two number of 16-byte entries "
                    "and at least 8 loads per thread");
    if ((reinterpret_cast<uintptr_t>(table) & 15u) != 0)
        return fail(GBFSM_INVALID_ARG, "gbfsm_probe_gather16: table not 16-byte aligned");
    const uint32_t mask = (uint32_t)(n_vec - 1);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (via_l1)
        gather16_kernel<true><<<probe_grid(8), 256, 0, s>>>(static_cast<const uint4 *>(table),
                                                            mask, loads_per_thread, sink);
    else
        gather16_kernel<false><<<probe_grid(8), 256, 0, s>>>(static_cast<const uint4 *>(table),
                                                             mask, loads_per_thread, sink);
    GBFSM_LAUNCH_CHECK("gather16_kernel launch");
    return GBFSM_OK;
}

gbfsm_status gbfsm_probe_chase(const uint32_t *next, uint32_t n, int64_t steps, int32_t chains,
                               uint64_t *sink, void *stream) {
    if (!next || !sink || n == 0 || (n & (n - 1)) != 0 || steps < 1 || chains < 1 ||
        chains > 1024)
        return fail(GBFSM_INVALID_ARG,
                    "gbfsm_probe_chase: a power-of-two entry count, steps >= 1, 1..1024 chains");
    chase_kernel<<<1, chains, 0, static_cast<cudaStream_t>(stream)>>>(next, n - 1, steps, sink);
    GBFSM_LAUNCH_CHECK("chase_kernel launch");
    return GBFSM_OK;
}

gbfsm_status gbfsm_probe_copy(void *dst, const void *src, size_t bytes, int32_t blocks_per_sm,
                              void *stream) {
    if (!dst || !src || bytes == 0 || (bytes & 15u) != 0 || blocks_per_sm < 1 ||
        blocks_per_sm > 8)
        return fail(GBFSM_INVALID_ARG,
                    "gbfsm_probe_copy: buffers, a multiple of 16 bytes and 1..8 CTAs per SM");
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15u) != 0)
        return fail(GBFSM_INVALID_ARG, "gbfsm_probe_copy: buffers not 16-byte aligned");
    copy16_kernel<<<probe_grid(blocks_per_sm), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<uint4 *>(dst), static_cast<const uint4 *>(src), (uint64_t)(bytes / 16));
    GBFSM_LAUNCH_CHECK("copy16_kernel launch");
    return GBFSM_OK;
}

gbfsm_status gbfsm_probe_smem(int64_t iters, int32_t blocks_per_sm, uint64_t *sink, void *stream) {
    if (!sink || iters < 1 || blocks_per_sm < 1 || blocks_per_sm > 8)
        return fail(GBFSM_INVALID_ARG, "gbfsm_probe_smem: bad iterations or blocks per SM");
    smem_kernel<<<probe_grid(blocks_per_sm), 256, 0, static_cast<cudaStream_t>(stream)>>>(iters,
                                                                                         sink);
    GBFSM_LAUNCH_CHECK("smem_kernel launch");
    return GBFSM_OK;
}

}  // extern "C"
