// Host-to-device ingest of a batch driven by the GPU: every input is copied from where the
// caller keeps it (one host buffer per input, e.g. the Python `bytes` objects passed to
// run_batch) into the contiguous device layout the kernels read, without packing the
// batch on the host first.
//
// On a device that reads pageable host memory coherently (GB300 with NVLink-C2C: address
// translation through the host's page tables), the source buffers need no registration:
// the copy kernel loads them directly. The destination is cut into 8 KiB windows, taken by
// the warps of the grid in turn, so that a long input is copied by many warps and a batch
// of unequal inputs keeps every warp busy to the end (one warp per input left a 1 MiB
// input to one warp). In a window, the inputs that overlap it are taken 32 at a time:
// pieces under 64 bytes are copied byte by byte by one lane each, longer ones by the whole
// warp, each lane writing whole 16-byte blocks of the destination made of two aligned
// 16-byte source loads joined by shifts (the source and destination need not share an
// alignment), and the partial blocks at the two ends of a piece byte by byte. Every
// destination byte is written once. A load never touches an aligned 16-byte block that
// holds no byte of its input, so it never touches a page the input does not.
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

constexpr int64_t kGatherWindow = 8192;  // destination bytes per warp task
constexpr int64_t kGatherSmall = 64;     // pieces shorter than this: one lane each
#ifndef GBFSM_GATHER_THREADS
#define GBFSM_GATHER_THREADS 256
#endif
#ifndef GBFSM_GATHER_CTAS_PER_SM
#define GBFSM_GATHER_CTAS_PER_SM 2  // the host link saturates at 2 CTAs of 256 per SM
#endif
constexpr int kGatherThreads = GBFSM_GATHER_THREADS;
constexpr int kGatherCtasPerSm = GBFSM_GATHER_CTAS_PER_SM;

// The warp copies dst[lo, hi) from s (s holds the byte of dst[lo]).
__device__ __forceinline__ void copy_piece(const uint8_t *s, uint8_t *__restrict__ dst,
                                           int64_t lo, int64_t hi, uint32_t lane) {
    const int64_t a = (lo + 15) & ~(int64_t)15, z = hi & ~(int64_t)15;
    if (a >= z) {  // no whole block: fewer than 32 bytes
        const int64_t k = lo + lane;
        if (k < hi) dst[k] = s[k - lo];
        return;
    }
    if (lo + lane < a) dst[lo + lane] = s[lane];                  // head, under 16 bytes
    if (z + lane < hi) dst[z + lane] = s[z + lane - lo];          // tail, under 16 bytes
    for (int64_t b = a + 16 * (int64_t)lane; b < z; b += 16 * 32 * 4) {
        uint4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (b + 512 * u < z) v[u] = ld16_unaligned(s + (b + 512 * u - lo));
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (b + 512 * u < z) *reinterpret_cast<uint4 *>(dst + b + 512 * u) = v[u];
    }
}

__global__ void __launch_bounds__(kGatherThreads) gather_inputs_kernel(
    const uint64_t *__restrict__ src, const int64_t *__restrict__ offsets, int32_t n,
    uint8_t *__restrict__ dst) {
    const uint32_t lane = lane_id();
    const int64_t first = offsets[0], last = offsets[n];
    if (last <= first) return;
    const int64_t w0 = first & ~(int64_t)15;  // windows start on 16-byte blocks
    const int64_t windows = (last - w0 + kGatherWindow - 1) / kGatherWindow;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < windows;
         w += nwarps) {
        const int64_t wl = w0 + w * kGatherWindow;
        const int64_t wh = wl + kGatherWindow < last ? wl + kGatherWindow : last;
        // the first input that ends after wl (input n - 1 does: wl < last)
        int32_t lo = 0, hi = n - 1;
        while (lo < hi) {
            const int32_t mid = (lo + hi) >> 1;
            if (offsets[mid + 1] > wl) hi = mid;
            else lo = mid + 1;
        }
        for (int64_t g = lo; g < n; g += 32) {
            const int64_t i = g + (int64_t)lane;
            int64_t d0 = wh, d1 = wh;
            if (i < n) {
                d0 = offsets[i];
                d1 = offsets[i + 1];
            }
            const bool past = d0 >= wh;  // this input and every later one start after the window
            const int64_t a = d0 > wl ? d0 : wl, b = d1 < wh ? d1 : wh;
            const bool live = !past && a < b;
            const uint8_t *s = live ? reinterpret_cast<const uint8_t *>(src[i]) + (a - d0) : nullptr;
            if (live && b - a < kGatherSmall)
                for (int64_t k = a; k < b; ++k) dst[k] = s[k - a];
            uint32_t big = __ballot_sync(0xffffffffu, live && b - a >= kGatherSmall);
            while (big) {
                const int j = __ffs(big) - 1;
                big &= big - 1;
                const int64_t aj = __shfl_sync(0xffffffffu, a, j);
                const int64_t bj = __shfl_sync(0xffffffffu, b, j);
                const uint8_t *sj = reinterpret_cast<const uint8_t *>(
                    __shfl_sync(0xffffffffu, reinterpret_cast<uint64_t>(s), j));
                copy_piece(sj, dst, aj, bj, lane);
            }
            if (__any_sync(0xffffffffu, past)) break;
        }
    }
}

}  // namespace

gbfsm_status launch_gather_inputs(const uint64_t *src, const int64_t *offsets, int32_t n,
                                  uint8_t *dst, cudaStream_t stream) {
    if (n <= 0) return GBFSM_OK;
    gather_inputs_kernel<<<sm_count() * kGatherCtasPerSm, kGatherThreads, 0, stream>>>(
        src, offsets, n, dst);
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
