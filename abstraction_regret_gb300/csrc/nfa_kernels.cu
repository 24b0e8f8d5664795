// Plain single-launch NFA batch kernels and their launch plans.
//
//   nfa_warp_kernel    one warp per input (GBFSM_TECH_WARP: dense bitmap only;
//                      GBFSM_TECH_COMPACT: sparse member list, dense on overflow).
//                      Replaces worklist_warp / worklist_shared / worklist_compact /
//                      worklist_global of the reference (worklist_global.cu:128-181,
//                      :289-342), whose sets live in global memory or shared memory with
//                      a 48 KB cap; here the per-warp scratch is placed in shared memory
//                      when it fits the opt-in budget and in a global workspace otherwise.
//   nfa_bitmap_kernel  one thread per input with a packed bitmap set (GBFSM_TECH_BITMAP).
//                      Replaces the register worklist / multistream kernels
//                      (worklist_register.cu:113-128, bitpacked.cu:105-166); no state cap.
//
// With plan.stage the edge rows are copied into shared memory by the TMA engine
// (cp.async.bulk) once per CTA when they fit next to the per-warp scratch.
#include <algorithm>

#include "common.cuh"
#include "engine.hpp"
#include "nfa_device.cuh"

namespace gbfsm {

namespace {

__device__ __forceinline__ Rows staged_rows(uint8_t *smem, uint32_t o_sr, uint32_t o_se,
                                            uint32_t o_er, uint32_t o_ee) {
    Rows r;
    r.sym_row = reinterpret_cast<const uint32_t *>(smem + o_sr);
    r.sym_edges = reinterpret_cast<const gbfsm_edge *>(smem + o_se);
    r.eps_row = reinterpret_cast<const uint32_t *>(smem + o_er);
    r.eps_edges = reinterpret_cast<const gbfsm_edge *>(smem + o_ee);
    return r;
}

__device__ __forceinline__ Rows global_rows(const gbfsm_nfa_dev &a) {
    Rows r;
    r.sym_row = a.sym_row;
    r.sym_edges = a.sym_edges;
    r.eps_row = a.eps_row;
    r.eps_edges = a.eps_edges;
    return r;
}

template <bool kStaged>
__global__ void __launch_bounds__(kMaxBlockThreads) nfa_warp_kernel(gbfsm_nfa_dev a, WarpPlan wp,
                                                        const uint8_t *__restrict__ data,
                                                        const int64_t *__restrict__ offsets,
                                                        int32_t n_inputs, int32_t *flags,
                                                        int32_t *lens, int32_t *examined,
                                                        uint8_t *gws) {
    extern __shared__ __align__(16) uint8_t smem[];
    Rows R;
    bool ok = true;
    if (kStaged) {
        StageCopy c[4] = {{wp.off_sym_row, a.sym_row, wp.bytes_sym_row},
                          {wp.off_sym_edges, a.sym_edges, wp.bytes_sym_edges},
                          {wp.off_eps_row, a.eps_row, wp.bytes_eps_row},
                          {wp.off_eps_edges, a.eps_edges, wp.bytes_eps_edges}};
        ok = stage_to_smem(smem, reinterpret_cast<uint64_t *>(smem), c, 4);
        R = staged_rows(smem, wp.off_sym_row, wp.off_sym_edges, wp.off_eps_row, wp.off_eps_edges);
    } else {
        R = global_rows(a);
    }
    const int warp = (int)(threadIdx.x >> 5);
    const int input = (int)blockIdx.x * wp.warps_per_cta + warp;
    if (input >= n_inputs) return;
    if (!ok) {
        if (lane_id() == 0) {
            flags[input] = kFlagTimeout;
            lens[input] = 0;
            if (examined) examined[input] = 0;
        }
        return;
    }
    const int W = wp.W;
    const uint32_t wbytes = pad16((uint64_t)W * 8u);
    uint8_t *sp = smem + wp.stage_bytes + (size_t)warp * wp.smem_per_warp;
    uint8_t *gp = gws + (size_t)input * wp.global_per_warp;
    WarpScratch S;
    S.C = wp.C;
    // V and the lists first, then D/FA/FB, each in shared memory or the global slice
    const size_t vpart = wbytes + (size_t)32u * (uint32_t)max(wp.C, 32);
    uint8_t *vp = wp.v_in_smem ? sp : gp;
    uint8_t *dp = wp.dense_in_smem ? sp + vpart : (wp.v_in_smem ? gp : gp + vpart);
    S.V = reinterpret_cast<uint64_t *>(vp);
    S.LA = reinterpret_cast<uint4 *>(vp + wbytes);
    S.LB = S.LA + max(wp.C, 32);
    S.D = reinterpret_cast<uint64_t *>(dp);
    S.FA = reinterpret_cast<uint64_t *>(dp + wbytes);
    S.FB = reinterpret_cast<uint64_t *>(dp + 2 * wbytes);
    zero_words(S.V, W);
    zero_words(S.D, W);
    zero_words(S.FA, W);
    zero_words(S.FB, W);
    __syncwarp();
    const int64_t b = offsets[input];
    const Verdict v = simulate_warp<kStaged>(a, R, data + b, offsets[input + 1] - b, S);
    if (lane_id() == 0) {
        flags[input] = v.flag;
        lens[input] = v.len;
        if (examined) examined[input] = (int32_t)v.examined;
    }
}

// Thread-per-input bitmap simulation. Word w of a set of thread t is at X[w * stride + t]
// (interleaved, so a warp touching word w hits 32 consecutive words).
struct TSet {
    uint64_t *p;
    int stride;
    int t;
    __device__ __forceinline__ uint64_t &word(int w) const { return p[(size_t)w * stride + t]; }
    // returns true if the bit was not set before
    __device__ __forceinline__ bool insert(uint32_t s) const {
        uint64_t &x = word((int)(s >> 6));
        const uint64_t b = 1ull << (s & 63u);
        const bool fresh = (x & b) == 0;
        x |= b;
        return fresh;
    }
};

template <bool kStaged>
__device__ __forceinline__ void thread_closure(const Rows &R, int W, TSet nxt, TSet f1, TSet f2,
                                               uint32_t &info_or) {
    for (;;) {
        bool more = false;
        for (int w = 0; w < W; ++w) {
            uint64_t bits = f1.word(w);
            if (!bits) continue;
            f1.word(w) = 0ull;
            while (bits) {
                const uint32_t s = (uint32_t)w * 64u + (uint32_t)(__ffsll((long long)bits) - 1);
                bits &= bits - 1ull;
                const uint32_t eb = load_row<kStaged>(R.eps_row + s);
                const uint32_t ee = load_row<kStaged>(R.eps_row + s + 1);
                for (uint32_t k = eb; k < ee; ++k) {
                    const uint4 rec = load_edge<kStaged>(R.eps_edges + k);
                    if (nxt.insert(rec.x)) {
                        info_or |= rec.y;
                        if (rec.y & GBFSM_EDGE_HAS_EPS) {
                            f2.insert(rec.x);
                            more = true;
                        }
                    }
                }
            }
        }
        if (!more) break;
        const TSet t = f1;
        f1 = f2;
        f2 = t;
    }
}

template <bool kStaged>
__device__ Verdict simulate_thread(const gbfsm_nfa_dev &a, const Rows &R, const uint8_t *in,
                                   int64_t len, TSet cur, TSet nxt, TSet f1, TSet f2) {
    const int W = a.num_words;
    const bool has_eps = (a.flags & GBFSM_NFA_HAS_EPS) != 0;
    Verdict v{0, 0, 0};
    uint32_t info_or = 0;
    {
        const uint32_t s = (uint32_t)a.start_state;
        uint32_t info = 0;
        if ((a.accept_words[s >> 6] >> (s & 63u)) & 1ull) info |= GBFSM_EDGE_ACCEPT;
        nxt.insert(s);
        if (has_eps && load_row<kStaged>(R.eps_row + s + 1) > load_row<kStaged>(R.eps_row + s)) {
            info |= GBFSM_EDGE_HAS_EPS;
            f1.insert(s);
        }
        info_or = info;
        if (info & GBFSM_EDGE_HAS_EPS) thread_closure<kStaged>(R, W, nxt, f1, f2, info_or);
    }
    if (info_or & GBFSM_EDGE_ACCEPT) {
        v.flag = 1;
        for (int w = 0; w < W; ++w) nxt.word(w) = 0ull;
        return v;
    }
    {
        const TSet t = cur;
        cur = nxt;
        nxt = t;
    }
    const uint8_t *end = in + len;
    const uint64_t addr = reinterpret_cast<uint64_t>(in);
    const uint8_t *blk = reinterpret_cast<const uint8_t *>(addr & ~15ull);
    int k = (int)(addr & 15ull);
    uint4 chunk = make_uint4(0, 0, 0, 0), ahead = make_uint4(0, 0, 0, 0);
    if (len > 0) chunk = ld_stream16(blk);
    if (blk + 16 < end) ahead = ld_stream16(blk + 16);
    int64_t pos = 0;
    bool live = true;
    while (pos < len) {
        if (k == 16) {
            blk += 16;
            k = 0;
            chunk = ahead;
            if (blk + 16 < end) ahead = ld_stream16(blk + 16);
        }
        const uint32_t sym = byte_of(chunk, k);
        ++k;
        ++pos;
        info_or = 0;
        bool any = false;
        for (int w = 0; w < W; ++w) {
            uint64_t bits = cur.word(w);
            if (!bits) continue;
            cur.word(w) = 0ull;  // cur is consumed; it becomes the next step's empty set
            while (bits) {
                const uint32_t s = (uint32_t)w * 64u + (uint32_t)(__ffsll((long long)bits) - 1);
                bits &= bits - 1ull;
                const uint32_t rb = load_row<kStaged>(R.sym_row + s);
                const uint32_t re = load_row<kStaged>(R.sym_row + s + 1);
                for (uint32_t e = rb; e < re; ++e) {
                    const uint4 rec = load_edge<kStaged>(R.sym_edges + e);
                    const uint32_t es = rec.y & GBFSM_EDGE_SYMBOL_MASK;
                    if (es == sym || es == GBFSM_ANY_SYMBOL) {
                        if (nxt.insert(rec.x)) {
                            any = true;
                            info_or |= rec.y;
                            if (has_eps && (rec.y & GBFSM_EDGE_HAS_EPS)) f1.insert(rec.x);
                        }
                    }
                }
            }
        }
        if (!any) {  // reference.py:59-60
            live = false;
            break;
        }
        if (info_or & GBFSM_EDGE_HAS_EPS) thread_closure<kStaged>(R, W, nxt, f1, f2, info_or);
        const TSet t = cur;
        cur = nxt;
        nxt = t;
        if (info_or & GBFSM_EDGE_ACCEPT) {
            v.flag = 1;
            v.len = (int32_t)pos;
            break;
        }
    }
    v.examined = pos;
    if (live) {
        for (int w = 0; w < W; ++w) cur.word(w) = 0ull;
    }
    return v;
}

template <bool kStaged, bool kSmemSets>
__global__ void __launch_bounds__(kMaxBlockThreads) nfa_bitmap_kernel(gbfsm_nfa_dev a, BitmapPlan bp,
                                                          const uint8_t *__restrict__ data,
                                                          const int64_t *__restrict__ offsets,
                                                          int32_t n_inputs, int32_t *flags,
                                                          int32_t *lens, int32_t *examined,
                                                          uint64_t *gws) {
    extern __shared__ __align__(16) uint8_t smem[];
    Rows R;
    bool ok = true;
    if (kStaged) {
        StageCopy c[4] = {{bp.off_sym_row, a.sym_row, bp.bytes_sym_row},
                          {bp.off_sym_edges, a.sym_edges, bp.bytes_sym_edges},
                          {bp.off_eps_row, a.eps_row, bp.bytes_eps_row},
                          {bp.off_eps_edges, a.eps_edges, bp.bytes_eps_edges}};
        ok = stage_to_smem(smem, reinterpret_cast<uint64_t *>(smem), c, 4);
        R = staged_rows(smem, bp.off_sym_row, bp.off_sym_edges, bp.off_eps_row, bp.off_eps_edges);
    } else {
        R = global_rows(a);
    }
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n_inputs) return;
    if (!ok) {
        flags[i] = kFlagTimeout;
        lens[i] = 0;
        if (examined) examined[i] = 0;
        return;
    }
    const int W = bp.W;
    TSet base;
    if (kSmemSets) {
        base.p = reinterpret_cast<uint64_t *>(smem + bp.stage_bytes);
        base.stride = (int)blockDim.x;
        base.t = (int)threadIdx.x;
    } else {
        base.p = gws;
        base.stride = (int)(gridDim.x * blockDim.x);
        base.t = i;
    }
    TSet sets[4];
    for (int q = 0; q < 4; ++q) {
        sets[q] = base;
        sets[q].p = base.p + (size_t)q * W * base.stride;
        for (int w = 0; w < W; ++w) sets[q].word(w) = 0ull;
    }
    const int64_t b = offsets[i];
    const Verdict v = simulate_thread<kStaged>(a, R, data + b, offsets[i + 1] - b, sets[0], sets[1],
                                               sets[2], sets[3]);
    flags[i] = v.flag;
    lens[i] = v.len;
    if (examined) examined[i] = (int32_t)v.examined;
}

template <typename K>
cudaError_t allow_smem(K kernel, size_t bytes) {
    if (bytes <= 48u * 1024u) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Byte layout of staged rows after the 16-byte mbarrier slot; returns the region size.
uint32_t stage_layout(const gbfsm_nfa_dev &a, uint32_t &o_sr, uint32_t &o_se, uint32_t &o_er,
                      uint32_t &o_ee, uint32_t &b_sr, uint32_t &b_se, uint32_t &b_er,
                      uint32_t &b_ee) {
    const uint64_t n = (uint64_t)a.num_states;
    const bool eps = (a.flags & GBFSM_NFA_HAS_EPS) != 0;
    b_sr = pad16((n + 1) * 4);
    b_se = pad16(a.num_sym_edges * sizeof(gbfsm_edge));
    b_er = eps ? pad16((n + 1) * 4) : 0;
    b_ee = eps ? pad16(a.num_eps_edges * sizeof(gbfsm_edge)) : 0;
    o_sr = 16;
    o_se = o_sr + b_sr;
    o_er = o_se + b_se;
    o_ee = o_er + b_er;
    return o_ee + b_ee;
}

}  // namespace

gbfsm_status make_warp_plan(const gbfsm_nfa_dev &a, int32_t n_inputs, const gbfsm_plan &p,
                            WarpPlan &wp) {
    (void)n_inputs;
    wp = WarpPlan{};
    wp.W = a.num_words;
    wp.C = (p.technique == GBFSM_TECH_WARP) ? 0
           : (p.list_capacity > 0)          ? p.list_capacity
                                            : kDefaultListCapacity;
    int threads = p.block_threads > 0 ? p.block_threads : 128;
    if (threads % 32 != 0 || threads > kMaxBlockThreads)
        return fail(GBFSM_INVALID_ARG, "block_threads must be a multiple of 32 up to 256 (got %d)",
                    threads);
    wp.warps_per_cta = threads / 32;
    const size_t budget = (size_t)smem_optin() - kSmemReserve;
    const uint32_t wbytes = pad16((uint64_t)wp.W * 8u);
    const size_t vpart = wbytes + (size_t)32u * (uint32_t)std::max(wp.C, 32);
    const size_t dpart = 3u * (size_t)wbytes;
    uint32_t stage = 0;
    if (p.stage) {
        uint64_t need = (uint64_t)16 + pad16(((uint64_t)a.num_states + 1) * 4) +
                        pad16(a.num_sym_edges * sizeof(gbfsm_edge));
        if (a.flags & GBFSM_NFA_HAS_EPS)
            need += pad16(((uint64_t)a.num_states + 1) * 4) +
                    pad16(a.num_eps_edges * sizeof(gbfsm_edge));
        if (need + (uint64_t)wp.warps_per_cta * vpart <= budget) {
            stage = stage_layout(a, wp.off_sym_row, wp.off_sym_edges, wp.off_eps_row,
                                 wp.off_eps_edges, wp.bytes_sym_row, wp.bytes_sym_edges,
                                 wp.bytes_eps_row, wp.bytes_eps_edges);
            wp.staged = 1;
        }
    }
    wp.stage_bytes = stage;
    const size_t wpc = (size_t)wp.warps_per_cta;
    if (stage + wpc * (vpart + dpart) <= budget) {
        wp.v_in_smem = wp.dense_in_smem = 1;
    } else if (stage + wpc * vpart <= budget) {
        wp.v_in_smem = 1;
    }
    wp.smem_per_warp = (uint32_t)((wp.v_in_smem ? vpart : 0) + (wp.dense_in_smem ? dpart : 0));
    wp.global_per_warp = (wp.v_in_smem ? 0 : vpart) + (wp.dense_in_smem ? 0 : dpart);
    wp.smem_total = stage + wpc * wp.smem_per_warp;
    return GBFSM_OK;
}

gbfsm_status make_bitmap_plan(const gbfsm_nfa_dev &a, int32_t n_inputs, const gbfsm_plan &p,
                              BitmapPlan &bp) {
    (void)n_inputs;
    bp = BitmapPlan{};
    bp.W = a.num_words;
    int threads = p.block_threads > 0 ? p.block_threads : 128;
    if (threads % 32 != 0 || threads > kMaxBlockThreads)
        return fail(GBFSM_INVALID_ARG, "block_threads must be a multiple of 32 up to 256 (got %d)",
                    threads);
    const size_t budget = (size_t)smem_optin() - kSmemReserve;
    const size_t per_thread = (size_t)bp.W * 32u;
    uint32_t stage = 0;
    if (p.stage) {
        uint32_t o[4], b[4];
        const uint32_t need = stage_layout(a, o[0], o[1], o[2], o[3], b[0], b[1], b[2], b[3]);
        if (need + 32u * per_thread <= budget) {
            stage = stage_layout(a, bp.off_sym_row, bp.off_sym_edges, bp.off_eps_row,
                                 bp.off_eps_edges, bp.bytes_sym_row, bp.bytes_sym_edges,
                                 bp.bytes_eps_row, bp.bytes_eps_edges);
            bp.staged = 1;
        }
    }
    bp.stage_bytes = stage;
    while (threads > 32 && stage + threads * per_thread > budget) threads -= 32;
    bp.threads = threads;
    bp.sets_in_smem = (stage + threads * per_thread <= budget) ? 1 : 0;
    bp.smem_total = stage + (bp.sets_in_smem ? threads * per_thread : 0);
    return GBFSM_OK;
}

gbfsm_status launch_nfa_warp(const gbfsm_nfa_dev &a, const WarpPlan &wp, const uint8_t *data,
                             const int64_t *offsets, int32_t n_inputs, int32_t *flags,
                             int32_t *lens, int32_t *examined, void *workspace,
                             cudaStream_t stream) {
    if (n_inputs <= 0) return GBFSM_OK;
    const dim3 grid((unsigned)((n_inputs + wp.warps_per_cta - 1) / wp.warps_per_cta));
    const dim3 block((unsigned)(wp.warps_per_cta * 32));
    uint8_t *gws = static_cast<uint8_t *>(workspace);
    if (wp.staged) {
        GBFSM_CUDA_TRY(allow_smem(nfa_warp_kernel<true>, wp.smem_total));
        nfa_warp_kernel<true><<<grid, block, wp.smem_total, stream>>>(
            a, wp, data, offsets, n_inputs, flags, lens, examined, gws);
    } else {
        GBFSM_CUDA_TRY(allow_smem(nfa_warp_kernel<false>, wp.smem_total));
        nfa_warp_kernel<false><<<grid, block, wp.smem_total, stream>>>(
            a, wp, data, offsets, n_inputs, flags, lens, examined, gws);
    }
    GBFSM_LAUNCH_CHECK("nfa_warp_kernel launch");
    return GBFSM_OK;
}

gbfsm_status launch_nfa_bitmap(const gbfsm_nfa_dev &a, const BitmapPlan &bp, const uint8_t *data,
                               const int64_t *offsets, int32_t n_inputs, int32_t *flags,
                               int32_t *lens, int32_t *examined, void *workspace,
                               cudaStream_t stream) {
    if (n_inputs <= 0) return GBFSM_OK;
    const dim3 grid((unsigned)((n_inputs + bp.threads - 1) / bp.threads));
    const dim3 block((unsigned)bp.threads);
    uint64_t *gws = static_cast<uint64_t *>(workspace);
#define GBFSM_BITMAP_LAUNCH(ST, SM)                                                          \
    do {                                                                                     \
        GBFSM_CUDA_TRY(allow_smem(nfa_bitmap_kernel<ST, SM>, bp.smem_total));                \
        nfa_bitmap_kernel<ST, SM><<<grid, block, bp.smem_total, stream>>>(                   \
            a, bp, data, offsets, n_inputs, flags, lens, examined, gws);                     \
    } while (0)
    if (bp.staged && bp.sets_in_smem) GBFSM_BITMAP_LAUNCH(true, true);
    else if (bp.staged) GBFSM_BITMAP_LAUNCH(true, false);
    else if (bp.sets_in_smem) GBFSM_BITMAP_LAUNCH(false, true);
    else GBFSM_BITMAP_LAUNCH(false, false);
#undef GBFSM_BITMAP_LAUNCH
    GBFSM_LAUNCH_CHECK("nfa_bitmap_kernel launch");
    return GBFSM_OK;
}

}  // namespace gbfsm
