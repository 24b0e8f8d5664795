// Shared definitions of the libgbfsm translation units (sm_103a).
//
// The library is compiled without relocatable device code, so device helpers used by
// more than one translation unit live in headers (this one, nfa_device.cuh,
// dfa_device.cuh) and are inlined into each kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbfsm.h"

#define GBFSM_FULL_MASK 0xffffffffu

namespace gbfsm {

constexpr int kWarp = 32;
constexpr int kAlphabet = 256;

// Status plumbing shared by the entry points (defined in abi.cu).
gbfsm_status fail(gbfsm_status code, const char *fmt, ...);
gbfsm_status cuda_fail(cudaError_t err, const char *what);

#define GBFSM_CUDA_TRY(call)                                      \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return ::gbfsm::cuda_fail(_e, #call); \
    } while (0)

// Kernel launch + launch-error check.
#define GBFSM_LAUNCH_CHECK(what)                                  \
    do {                                                          \
        cudaError_t _e = cudaGetLastError();                      \
        if (_e != cudaSuccess) return ::gbfsm::cuda_fail(_e, what); \
    } while (0)

// Number of SMs of the current device (cached per device).
int sm_count();
// Opt-in shared memory per block of the current device (cached per device).
int smem_optin();

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// 16-byte read-only load that does not allocate in L1 (streamed input bytes).
__device__ __forceinline__ uint4 ld_stream16(const uint8_t *p) {
    uint4 v;
    asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

// 16-byte read-only load through L1 (edge records: re-read across steps and warps).
__device__ __forceinline__ uint4 ld_edge(const gbfsm_edge *p) {
    return __ldg(reinterpret_cast<const uint4 *>(p));
}

__device__ __forceinline__ uint32_t byte_of(const uint4 &v, int k) {
    uint32_t w = (k < 4) ? v.x : (k < 8) ? v.y : (k < 12) ? v.z : v.w;
    return (w >> ((k & 3) * 8)) & 0xffu;
}

// Sequential reader of one input's bytes: 16-byte loads (L1::no_allocate), the next
// block fetched one block ahead of use; bytes are shifted out of four 32-bit words with
// funnel shifts. Reads never leave the 16-byte blocks that contain input bytes.
struct ByteStream {
    const uint8_t *blk;
    const uint8_t *end;
    uint4 ahead;
    uint32_t w0, w1, w2, w3;
    int left;

    __device__ __forceinline__ void shift_bytes(int r) {
        w0 = __funnelshift_r(w0, w1, r);
        w1 = __funnelshift_r(w1, w2, r);
        w2 = __funnelshift_r(w2, w3, r);
        w3 >>= r;
    }

    __device__ __forceinline__ void init(const uint8_t *in, int64_t len) {
        end = in + len;
        const uint64_t a = reinterpret_cast<uint64_t>(in);
        blk = reinterpret_cast<const uint8_t *>(a & ~15ull);
        const int skip = (int)(a & 15ull);
        uint4 c = make_uint4(0, 0, 0, 0);
        ahead = make_uint4(0, 0, 0, 0);
        if (len > 0) c = ld_stream16(blk);
        if (blk + 16 < end) ahead = ld_stream16(blk + 16);
        w0 = c.x;
        w1 = c.y;
        w2 = c.z;
        w3 = c.w;
        for (int q = 0; q < (skip >> 2); ++q) {
            w0 = w1;
            w1 = w2;
            w2 = w3;
            w3 = 0;
        }
        if (skip & 3) shift_bytes((skip & 3) * 8);
        left = 16 - skip;
    }

    __device__ __forceinline__ uint32_t next() {
        if (left == 0) {
            blk += 16;
            w0 = ahead.x;
            w1 = ahead.y;
            w2 = ahead.z;
            w3 = ahead.w;
            if (blk + 16 < end) ahead = ld_stream16(blk + 16);
            left = 16;
        }
        const uint32_t b = w0 & 0xffu;
        shift_bytes(8);
        --left;
        return b;
    }
};

// Inclusive warp prefix sum of `x` (all 32 lanes participate).
__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t x) {
    const uint32_t lane = lane_id();
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(GBFSM_FULL_MASK, x, d);
        if (lane >= (uint32_t)d) x += y;
    }
    return x;
}

}  // namespace gbfsm

// ---------------------------------------------------------------------------------
// Bulk staging of read-only arrays into shared memory with the TMA engine
// (cp.async.bulk, no multicast, completion counted on an mbarrier). Every wait is
// bounded: after kStageSpinLimit polls the CTA gives up and reports a timeout instead
// of spinning forever.
// ---------------------------------------------------------------------------------
namespace gbfsm {

constexpr uint32_t kStageSpinLimit = 1u << 24;
constexpr uint32_t kBulkChunk = 32768;  // bytes per cp.async.bulk instruction

struct StageCopy {
    uint32_t dst_off;   // byte offset in dynamic shared memory (16-byte aligned)
    const void *src;    // global source (16-byte aligned)
    uint32_t bytes;     // multiple of 16
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity) {
    for (uint32_t i = 0; i < kStageSpinLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Copy up to 4 arrays into shared memory. All threads of the CTA call it; returns false
// (for every thread) if the copies did not complete within the bounded wait.
__device__ __forceinline__ bool stage_to_smem(uint8_t *smem, uint64_t *mbar_slot,
                                              const StageCopy *copies, int n_copies) {
    const uint32_t mbar = smem_addr(mbar_slot);
    uint32_t total = 0;
    for (int c = 0; c < n_copies; ++c) total += copies[c].bytes;
    if (total == 0) return true;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(total)
                     : "memory");
        for (int c = 0; c < n_copies; ++c) {
            const uint8_t *src = static_cast<const uint8_t *>(copies[c].src);
            const uint32_t dst = smem_addr(smem + copies[c].dst_off);
            for (uint32_t off = 0; off < copies[c].bytes; off += kBulkChunk) {
                const uint32_t n = min(kBulkChunk, copies[c].bytes - off);
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
                    "[%0], [%1], %2, [%3];" ::"r"(dst + off),
                    "l"(src + off), "r"(n), "r"(mbar)
                    : "memory");
            }
        }
    }
    __syncthreads();
    bool ok = mbar_wait_bounded(mbar, 0);
    if (!ok) ok = mbar_wait_bounded(mbar, 0);  // second bounded wait for copies in flight
    return __syncthreads_and(ok) != 0;
}

}  // namespace gbfsm
