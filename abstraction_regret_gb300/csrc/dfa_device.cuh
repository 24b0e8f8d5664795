// Device-side DFA table walk (latch-first-match), shared by the plain DFA kernel
// (dfa_kernels.cu) and the persistent engine (persistent.cu).
//
// Semantics: src/gpufsm/reference.py:68-81 (simulate_dfa): accept[start] gives (1, 0);
// then cur = trans[cur * 256 + byte] per byte and the first accepting cur gives
// (1, pos + 1); running off the end gives (0, 0). The device table folds accept[next]
// into the top bit of each entry, so one load per byte yields both the successor and
// the latch test (the reference reads trans and then accept, dfa.cu:21-22).
//
// Input bytes are streamed with 16-byte loads (L1::no_allocate) one block ahead of use.
#pragma once

#include "common.cuh"

namespace gbfsm {

template <typename Entry>
struct EntryTraits;
template <>
struct EntryTraits<uint16_t> {
    static constexpr uint32_t kAccept = 0x8000u;
};
template <>
struct EntryTraits<uint32_t> {
    static constexpr uint32_t kAccept = 0x80000000u;
};

// Row index type: 32-bit for 2-byte tables (at most 32768 states), 64-bit otherwise.
template <typename Entry>
struct RowIndex {
    using type = uint64_t;
};
template <>
struct RowIndex<uint16_t> {
    using type = uint32_t;
};

// Table entry lookup from one array: shared memory of this CTA (kStaged) or global
// memory read through L2.
template <typename Entry, bool kStaged>
struct ArrayTable {
    const Entry *t;
    __device__ __forceinline__ uint32_t operator()(uint32_t state, uint32_t byte) const {
        const typename RowIndex<Entry>::type idx =
            (typename RowIndex<Entry>::type)state * (uint32_t)kAlphabet + byte;
        if (kStaged) return t[idx];
        return __ldg(t + idx);
    }
};

// One input, one thread, table entries through `lookup(state, byte)`. Returns (flag,
// len, examined) through references.
template <typename Entry, typename Lookup>
__device__ __forceinline__ void dfa_walk_with(const Lookup &table_at, const uint32_t *accept_bits,
                                              uint32_t start, const uint8_t *in, int64_t len,
                                              int32_t &flag, int32_t &mlen, int64_t &examined) {
    constexpr uint32_t ACC = EntryTraits<Entry>::kAccept;
    flag = 0;
    mlen = 0;
    examined = len;
    if ((__ldg(accept_bits + (start >> 5)) >> (start & 31u)) & 1u) {
        flag = 1;
        examined = 0;
        return;
    }
    if (len <= 0) return;
    const uint8_t *end = in + len;
    const uint64_t addr = reinterpret_cast<uint64_t>(in);
    const uint8_t *blk = reinterpret_cast<const uint8_t *>(addr & ~15ull);
    int k = (int)(addr & 15ull);
    uint4 cur4 = ld_stream16(blk);
    uint4 nxt4 = make_uint4(0, 0, 0, 0);
    if (blk + 16 < end) nxt4 = ld_stream16(blk + 16);
    uint32_t cur = start;
    int64_t pos = -(int64_t)k;  // position of byte 0 of the current block
    for (;;) {
        const int64_t remain = len - pos;  // bytes from the block start to the end
        if (k == 0 && remain >= 16) {
            // full block: 16 dependent lookups, latch tested per byte
            const uint32_t w[4] = {cur4.x, cur4.y, cur4.z, cur4.w};
#pragma unroll
            for (int b = 0; b < 16; ++b) {
                const uint32_t e = table_at(cur, (w[b >> 2] >> ((b & 3) * 8)) & 0xffu);
                cur = e & ~ACC;
                if (e & ACC) {
                    flag = 1;
                    mlen = (int32_t)(pos + b + 1);
                    examined = pos + b + 1;
                    return;
                }
            }
        } else {
            const int hi = remain < 16 ? (int)remain : 16;
            for (int b = k; b < hi; ++b) {
                const uint32_t e = table_at(cur, byte_of(cur4, b));
                cur = e & ~ACC;
                if (e & ACC) {
                    flag = 1;
                    mlen = (int32_t)(pos + b + 1);
                    examined = pos + b + 1;
                    return;
                }
            }
        }
        pos += 16;
        k = 0;
        if (pos >= len) return;
        blk += 16;
        cur4 = nxt4;
        if (blk + 16 < end) nxt4 = ld_stream16(blk + 16);
    }
}

template <typename Entry, bool kStaged>
__device__ __forceinline__ void dfa_walk(const Entry *table, const uint32_t *accept_bits,
                                         uint32_t start, const uint8_t *in, int64_t len,
                                         int32_t &flag, int32_t &mlen, int64_t &examined) {
    dfa_walk_with<Entry>(ArrayTable<Entry, kStaged>{table}, accept_bits, start, in, len, flag,
                         mlen, examined);
}

}  // namespace gbfsm
