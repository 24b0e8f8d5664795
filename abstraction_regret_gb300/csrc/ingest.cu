// Host-to-device ingest of a batch driven by the GPU: every input is copied from where the
// caller keeps it (one host buffer per input, e.g. the Python `bytes` objects passed to
// run_batch) into the contiguous device layout the kernels read, without packing the
// batch on the host first.
//
// On a device that reads pageable host memory coherently (GB300 with NVLink-C2C: address
// translation through the host's page tables), the source buffers need no registration:
// the copy kernel loads them directly. One warp copies one input: each lane writes whole
// 16-byte blocks of the destination, each made of two aligned 16-byte source loads joined
// by shifts (the source and destination need not share an alignment);
// the partial blocks at the two ends of an input are written byte by byte. A load never
// touches an aligned 16-byte block that holds no byte of its input, so it never touches a
// page the input does not.
//
// The reference packs every batch on the host and copies it synchronously from pageable
// memory, widened to int32 (src/gpufsm/core/packing.py:35-63,
// native/include/common.cuh:150-159).
#include "common.cuh"
#include "engine.hpp"

namespace gbfsm {
namespace {

__device__ __forceinline__ uint4 ld16(const uint8_t *p) {
    return *reinterpret_cast<const uint4 *>(p);
}

// 16 bytes starting at p (any alignment), from the aligned blocks holding them.
__device__ __forceinline__ uint4 ld16_unaligned(const uint8_t *p) {
    const uint64_t a = reinterpret_cast<uint64_t>(p);
    const uint32_t sh = (uint32_t)(a & 15u);
    const uint8_t *blk = reinterpret_cast<const uint8_t *>(a & ~15ull);
    const uint4 x = ld16(blk);
    if (sh == 0) return x;
    const uint4 y = ld16(blk + 16);
    // bytes sh .. sh + 15 of the 32-byte window x:y, as 64-bit words: the three words
    // from the one holding byte sh, shifted right by 8 * (sh % 8) bits
    const uint64_t w0 = ((uint64_t)x.y << 32) | x.x, w1 = ((uint64_t)x.w << 32) | x.z;
    const uint64_t w2 = ((uint64_t)y.y << 32) | y.x, w3 = ((uint64_t)y.w << 32) | y.z;
    const uint64_t u = sh >= 8 ? w1 : w0, v = sh >= 8 ? w2 : w1, z = sh >= 8 ? w3 : w2;
    const uint32_t t = (sh & 7u) * 8u;
    const uint64_t o0 = t ? (u >> t) | (v << (64u - t)) : u;
    const uint64_t o1 = t ? (v >> t) | (z << (64u - t)) : v;
    return make_uint4((uint32_t)o0, (uint32_t)(o0 >> 32), (uint32_t)o1, (uint32_t)(o1 >> 32));
}

__global__ void __launch_bounds__(256) gather_inputs_kernel(const uint64_t *__restrict__ src,
                                                            const int64_t *__restrict__ offsets,
                                                            int32_t n, uint8_t *__restrict__ dst) {
    const uint32_t lane = lane_id();
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nwarps) {
        const uint8_t *s = reinterpret_cast<const uint8_t *>(src[i]);
        const int64_t d0 = offsets[i], d1 = offsets[i + 1];
        if (d1 <= d0) continue;
        const int64_t b0 = d0 & ~(int64_t)15, b1 = (d1 + 15) & ~(int64_t)15;
        for (int64_t b = b0 + 16 * (int64_t)lane; b < b1; b += 16 * 32) {
            const int64_t lo = b > d0 ? b : d0, hi = b + 16 < d1 ? b + 16 : d1;
            if (lo == b && hi == b + 16) {
                *reinterpret_cast<uint4 *>(dst + b) = ld16_unaligned(s + (b - d0));
            } else {
                for (int64_t k = lo; k < hi; ++k) dst[k] = s[k - d0];
            }
        }
    }
}

}  // namespace

gbfsm_status launch_gather_inputs(const uint64_t *src, const int64_t *offsets, int32_t n,
                                  uint8_t *dst, cudaStream_t stream) {
    if (n <= 0) return GBFSM_OK;
    int grid = (n + 7) / 8;  // 8 warps per CTA, a warp per input
    const int cap = sm_count() * 8;
    if (grid > cap) grid = cap;
    gather_inputs_kernel<<<grid, 256, 0, stream>>>(src, offsets, n, dst);
    GBFSM_LAUNCH_CHECK("gather_inputs_kernel launch");
    return GBFSM_OK;
}

int32_t pageable_access() {
    int dev = 0, v = 0, host_tables = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    if (cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                               dev) != cudaSuccess) {
        cudaGetLastError();
        host_tables = 0;
    }
    return v ? (host_tables ? 2 : 1) : 0;
}

}  // namespace gbfsm

extern "C" {

int32_t gbfsm_pageable_access(void) { return gbfsm::pageable_access(); }

gbfsm_status gbfsm_gather_inputs(const uint64_t *src_ptrs, const int64_t *offsets,
                                 int32_t n_inputs, uint8_t *dst, void *stream) {
    using namespace gbfsm;
    if (n_inputs < 0) return fail(GBFSM_INVALID_ARG, "gbfsm_gather_inputs: n_inputs < 0");
    if (n_inputs > 0 && (!src_ptrs || !offsets || !dst))
        return fail(GBFSM_INVALID_ARG, "gbfsm_gather_inputs: NULL array");
    return launch_gather_inputs(src_ptrs, offsets, n_inputs, dst,
                                static_cast<cudaStream_t>(stream));
}

}  // extern "C"
