// Triangle count (the reference's triangleCountPullGraphCSR,
// triangleCount.c:254-334): on a (src,dst)-sorted CSR,
//   total = sum over edges u->v with v <= u,
//           over w in N(v) with w <= v, of [w in N(u)].
// On a symmetric, deduplicated, loop-free graph this counts each triangle
// once (w < v < u); after degree reordering (highest degree = id 0) it is the
// degree-ordered DAG count.
//
// Write N+(x) = N(x) ∩ [0, x], a prefix of the sorted row (its length is
// cached per graph). Every w in N+(v) is <= v, so the term of the pair (u, v)
// is |N+(v) ∩ N(u)|.
//
// Fast path -- rows without repeated neighbours on a symmetric CSR (both
// checked once per graph): the pair term equals the number of w in the prefix
// N(u) ∩ [0, v] that lie in N+(v), and the pairs of a fixed v are exactly the
// u >= v in N(v) (symmetry). So the kernel is centred on v: N+(v) goes into
// an open-addressing hash table in shared memory once, and for every upper
// neighbour u the prefix N(u) ∩ [0, v] is streamed with consecutive lanes on
// consecutive elements (coalesced), one or two shared-memory probes each.
// Summed over pairs that streams |N(u) ∩ [0, v]| elements instead of |N+(v)|
// (3.5x fewer on RMAT-20). The prefix length |N(u) ∩ [0, v]| of every pair
// is found by a search of u's row in the first count of a graph, and from
// the second count on read from the plan (pre_len, one word per edge). A v
// with many upper neighbours is cut into units of kUpperChunk of them, dealt
// to warps by an atomic cursor, so hubs are spread over the GPU; the rest
// are one warp per v. A v whose N+(v) is
// longer than the per-warp table (up to 16384 ids) goes to tc_wide_kernel:
// one CTA per unit of its upper neighbours, N+(v) in a CTA-wide table, so no
// element is searched in global memory. The prefixes are read as aligned
// 16-byte quads.
//
// Hub pivots (fast path, v below the hub range H, at most 4,096): every
// vertex x keeps the bitmap of N(x) ∩ [0, H) (H/32 words, built once per
// graph), and the pair term is popc(bits(u) & bits(v)) over the words that
// cover [0, v) -- at most H/32 words per pair instead of |N(u) ∩ [0, v]|
// streamed elements. These low ids are the highest-degree vertices of the
// degree order, which hold most of the pairs' prefix work. Lanes take one
// word each, several pairs per warp step when v needs fewer than 32 words.
//
// General path (repeated neighbours, or a CSR that is not symmetric): the
// reference's multiplicities, centred on u, with a binary search of N+(u) in
// global memory per element of N+(v).
#include <algorithm>

#include "gbx_internal.cuh"

namespace gbx {

constexpr int kTcThreads = 256;
constexpr int kTcWarps = kTcThreads / 32;
constexpr uint32_t kTcTableMax = 512;   // |N+(v)| that fits a per-warp table
constexpr uint32_t kTcWarpSlots = 1024;  // hash slots per warp
constexpr uint32_t kUpperChunk = 256;   // upper neighbours per work unit
constexpr uint32_t kEmptySlot = 0xFFFFFFFFu;
// hybrid membership for pivots above the bitmap range: ids below
// kHybridSplit (the high-degree end of the degree order, which holds most of
// N+(v) and of the streamed prefixes) in the warp's bitmap, the rest in a
// second per-warp hash table of at most kHybridSlots slots
constexpr uint32_t kHybridSplit = kTcWarpSlots * 32;
constexpr uint32_t kHybridSlots = 256;

// number of elements <= x (or < x) in sorted a[0..n)
__device__ __forceinline__ uint32_t count_le(const uint32_t *a, uint32_t n, uint32_t x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(a + mid) <= x) lo = mid + 1; else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ uint32_t count_lt(const uint32_t *a, uint32_t n, uint32_t x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// count_le by galloping from the front: 2*log2(answer) loads instead of
// log2(n), for lists whose prefix <= x is short (x a high-degree id)
__device__ __forceinline__ uint32_t count_le_front(const uint32_t *a, uint32_t n, uint32_t x) {
    if (n == 0 || __ldg(a) > x) return 0;
    uint32_t lo = 1, hi = 2;  // a[lo-1] <= x
    while (hi <= n && __ldg(a + hi - 1) <= x) {
        lo = hi;
        hi *= 2;
    }
    hi = min(hi - 1, n);  // answer in [lo, hi]
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(a + mid - 1) <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ bool sorted_contains(const uint32_t *a, uint32_t n, uint32_t x) {
    uint32_t i = count_lt(a, n, x);
    return i < n && __ldg(a + i) == x;
}

__device__ __forceinline__ uint32_t hash_slot(uint32_t x, uint32_t mask) {
    return (x * 0x9E3779B1u >> 7) & mask;
}

__device__ __forceinline__ void hash_insert(uint32_t *table, uint32_t mask, uint32_t x) {
    uint32_t h = hash_slot(x, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        uint32_t old = atomicCAS(table + h, kEmptySlot, x);
        if (old == kEmptySlot || old == x) return;
        h = (h + 1) & mask;
    }
}

__device__ __forceinline__ bool hash_contains(const uint32_t *table, uint32_t mask, uint32_t x) {
    uint32_t h = hash_slot(x, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        uint32_t t = table[h];
        if (t == x) return true;
        if (t == kEmptySlot) return false;
        h = (h + 1) & mask;
    }
    return false;
}

__device__ __forceinline__ uint32_t table_mask(uint32_t n) {
    uint32_t t = 64;
    while (t < 2 * n && t < kTcWarpSlots) t <<= 1;
    return t - 1;
}

// per vertex: |N+(v)| (elements <= v)
__global__ void tc_low_count_kernel(const uint32_t *off, const uint32_t *dest, uint32_t V, uint32_t *low) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        uint32_t b = off[v];
        low[v] = count_le(dest + b, off[v + 1] - b, v);
    }
}

__device__ __forceinline__ unsigned long long pair_hash(uint32_t a, uint32_t b) {
    // splitmix64 finaliser (Steele, Lea, Flood 2014) of the packed pair
    unsigned long long z = ((unsigned long long)a << 32 | b) + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// flags: bit 0 = some row repeats a neighbour. *asym accumulates, over all
// edges v->u, hash(v,u) - hash(u,v) (mod 2^64): zero when the edge multiset
// equals its reverse (the CSR is symmetric); a non-symmetric CSR sums to zero
// only by a 64-bit hash coincidence. One streaming pass instead of a search
// per edge.
__global__ void tc_shape_check_kernel(const uint32_t *off, const uint32_t *dest, uint32_t V, uint32_t E,
                                      unsigned *flags, unsigned long long *asym) {
    // the edge array in fixed chunks per warp (rows of any length spread
    // over many warps); each lane finds the row of its first edge by binary
    // search over the offsets and then walks forward with its edges
    constexpr uint32_t kChunk = 8192;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    unsigned f = 0;
    unsigned long long h = 0;
    for (uint64_t c0 = (uint64_t)gw * kChunk; c0 < E; c0 += (uint64_t)nw * kChunk) {
        const uint32_t c1 = c0 + kChunk < (uint64_t)E ? (uint32_t)(c0 + kChunk) : E;
        uint32_t j = (uint32_t)c0 + lane;
        if (j >= c1) continue;
        uint32_t lo = 0, hi = V - 1;  // last row r with off[r] <= j (E > j, so one exists)
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (__ldg(off + mid) <= j) lo = mid; else hi = mid - 1;
        }
        uint32_t r = lo;
        for (; j < c1; j += 32) {
            while (__ldg(off + r + 1) <= j) ++r;
            const uint32_t u = __ldcs(dest + j);
            if (j > __ldg(off + r) && u == __ldg(dest + j - 1)) f |= 1u;
            h += pair_hash(r, u) - pair_hash(u, r);
        }
    }
    f = __reduce_or_sync(0xffffffffu, f);
    h = warp_sum(h);
    if (lane == 0) {
        if (f) atomicOr(flags, f);
        if (h) atomicAdd(asym, h);
    }
}

// Prefix lengths of the fast path, kept in the plan: for every edge v->u
// with u >= v, pre_len = |N(u) ∩ [0, v]| (v's position in the sorted row of
// u, plus one, on a symmetric deduplicated CSR). The count kernels read it
// next to u instead of searching u's row for v on every count. Edges in
// fixed chunks per warp, each lane walking the rows of its edges.
__global__ void tc_prefix_len_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ dest, uint32_t V,
                                     uint32_t E, uint32_t *__restrict__ pre_len) {
    constexpr uint32_t kChunk = 2048;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint64_t c0 = (uint64_t)gw * kChunk; c0 < E; c0 += (uint64_t)nw * kChunk) {
        const uint32_t c1 = c0 + kChunk < (uint64_t)E ? (uint32_t)(c0 + kChunk) : E;
        uint32_t j = (uint32_t)c0 + lane;
        if (j >= c1) continue;
        uint32_t lo = 0, hi = V - 1;  // last row r with off[r] <= j
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (__ldg(off + mid) <= j) lo = mid; else hi = mid - 1;
        }
        uint32_t r = lo;
        for (; j < c1; j += 32) {
            while (__ldg(off + r + 1) <= j) ++r;
            const uint32_t u = __ldg(dest + j);
            uint32_t n = 0;
            if (u >= r) {
                const uint32_t b = __ldg(off + u);
                n = count_le_front(dest + b, __ldg(off + u + 1) - b, r);
            }
            pre_len[j] = n;
        }
    }
}

// Count the elements of the lanes' lists (base_k, len_k), flattened over the
// warp, that `member` accepts. Every lane calls with its own list (len 0 when
// it has none).
template <class Member>
__device__ __forceinline__ unsigned long long count_flat(const uint32_t *__restrict__ dest, uint32_t base,
                                                        uint32_t len, uint32_t *s_pre, uint32_t *s_base,
                                                        const Member &member) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    s_pre[lane] = incl - len;
    s_base[lane] = base;
    if (lane == 31) s_pre[32] = incl;
    __syncwarp();
    const uint32_t tot = s_pre[32];
    unsigned long long count = 0;
    uint32_t k = 0;  // owner lane of this lane's current item, advanced monotonically
    for (uint32_t i0 = 0; i0 < tot; i0 += 128) {
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t i = i0 + q * 32 + lane;
            w[q] = kEmptySlot;
            if (i < tot) {
                while (s_pre[k + 1] <= i) ++k;
                w[q] = __ldg(dest + s_base[k] + (i - s_pre[k]));
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (w[q] != kEmptySlot && member(w[q])) count++;
    }
    __syncwarp();
    return count;
}

// Same count with 16-byte loads: each lane's list [base, base+len) is read as
// the aligned quads that cover it (the neighbour array is 16-byte aligned and
// padded by four ids), four quads per lane per step, and the elements of a
// quad outside the list are masked. Four times fewer load instructions and
// four times the bytes in flight of count_flat.
template <class Member>
__device__ __forceinline__ unsigned long long count_flat4(const uint32_t *__restrict__ dest, uint32_t base,
                                                         uint32_t len, uint32_t *s_pre, uint32_t *s_base,
                                                         uint32_t *s_end, const Member &member) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t q0 = base >> 2;
    const uint32_t nq = len ? ((base + len + 3) >> 2) - q0 : 0u;
    uint32_t incl = nq;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    s_pre[lane] = incl - nq;
    s_base[lane] = base;
    s_end[lane] = base + len;
    if (lane == 31) s_pre[32] = incl;
    __syncwarp();
    const uint32_t tot = s_pre[32];
    const uint4 *d4 = reinterpret_cast<const uint4 *>(dest);
    unsigned long long count = 0;
    uint32_t k = 0;  // owner lane of this lane's current quad, advanced monotonically
    for (uint32_t i0 = 0; i0 < tot; i0 += 128) {
        uint4 w[4];
        uint32_t e0[4], lo[4], hi[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t i = i0 + q * 32 + lane;
            lo[q] = hi[q] = e0[q] = 0;
            w[q] = make_uint4(0u, 0u, 0u, 0u);
            if (i < tot) {
                while (s_pre[k + 1] <= i) ++k;
                const uint32_t qa = (s_base[k] >> 2) + (i - s_pre[k]);
                w[q] = __ldg(d4 + qa);
                e0[q] = qa * 4;
                lo[q] = s_base[k];
                hi[q] = s_end[k];
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            // the quad's elements inside [lo, hi) as a 4-bit mask; the
            // membership bits of all four, then one popcount
            const uint32_t x[4] = {w[q].x, w[q].y, w[q].z, w[q].w};
            const uint32_t from = lo[q] > e0[q] ? min(lo[q] - e0[q], 4u) : 0u;
            const uint32_t to = hi[q] > e0[q] ? min(hi[q] - e0[q], 4u) : 0u;
            const uint32_t valid = (0xFu >> (4u - to)) & (0xFu << from) & 0xFu;
            uint32_t hit = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                // a bitmap bit is cheaper to read than to branch around
                if (Member::kProbeAll || ((valid >> j) & 1u)) hit |= member.bit(x[j]) << j;
            }
            count += __popc(hit & valid);
        }
    }
    __syncwarp();
    return count;
}

struct HashMember {
    static constexpr bool kProbeAll = false;
    const uint32_t *table;
    uint32_t mask;
    __device__ __forceinline__ bool operator()(uint32_t w) const { return hash_contains(table, mask, w); }
    __device__ __forceinline__ uint32_t bit(uint32_t w) const { return hash_contains(table, mask, w) ? 1u : 0u; }
};

// Exact bitmap over [0, nbits) with nbits a power of two. Ids are masked
// into that range before the read: count_flat4 probes every id of a quad,
// including ids outside the list (other rows, padding), whose bits it then
// discards; a list's own ids are <= v < nbits and read their true bit.
struct HybridMember {
    static constexpr bool kProbeAll = true;  // both reads stay in range for any id
    const uint32_t *bits;   // ids below kHybridSplit
    const uint32_t *table;  // the others
    uint32_t mask;
    __device__ __forceinline__ uint32_t bit(uint32_t w) const {
        if (w < kHybridSplit) return (bits[w >> 5] >> (w & 31)) & 1u;
        return hash_contains(table, mask, w) ? 1u : 0u;
    }
    __device__ __forceinline__ bool operator()(uint32_t w) const { return bit(w) != 0u; }
};

struct BitmapMember {
    static constexpr bool kProbeAll = true;
    const uint32_t *bits;
    uint32_t id_mask;  // nbits - 1
    __device__ __forceinline__ uint32_t bit(uint32_t w) const {
        const uint32_t x = w & id_mask;
        return (bits[x >> 5] >> (x & 31)) & 1u;
    }
    __device__ __forceinline__ bool operator()(uint32_t w) const { return bit(w) != 0u; }
};

// For the upper neighbours u in [ub, ue) of v's row nv, 32 at a time: the
// prefix N(u) ∩ [0, v] of each (its length pl[] from the plan, read next to
// u, or a binary search of u's row before the plan has them), counted
// against m.
template <class Member>
__device__ __forceinline__ unsigned long long stream_pairs(const uint32_t *__restrict__ off,
                                                          const uint32_t *__restrict__ dest, const uint32_t *nv,
                                                          const uint32_t *pl, uint32_t v, uint32_t ub, uint32_t ue,
                                                          uint32_t *s_pre, uint32_t *s_base, uint32_t *s_end,
                                                          const Member &m) {
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long count = 0;
    for (uint32_t a0 = ub; a0 < ue; a0 += 32) {
        uint32_t base = 0, len = 0;
        if (a0 + lane < ue) {
            const uint32_t u = __ldg(nv + a0 + lane);
            base = __ldg(off + u);
            len = pl ? __ldg(pl + a0 + lane) : count_le(dest + base, __ldg(off + u + 1) - base, v);
        }
        count += count_flat4(dest, base, len, s_pre, s_base, s_end, m);
    }
    return count;
}

// stream_pairs for a CTA sharing one unit: warps take 32-neighbour chunks of
// [ub, ue) from a shared-memory counter (zeroed before the CTA barrier that
// precedes the call), so a warp with light prefixes takes more chunks and
// the CTA's wait at the end of the unit is one chunk long.
template <class Member>
__device__ __forceinline__ unsigned long long stream_pairs_dealt(const uint32_t *__restrict__ off,
                                                                const uint32_t *__restrict__ dest,
                                                                const uint32_t *nv, const uint32_t *pl, uint32_t v,
                                                                uint32_t ub, uint32_t ue, uint32_t *s_pre,
                                                                uint32_t *s_base,
                                                                uint32_t *s_end, const Member &m,
                                                                unsigned *s_next) {
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long count = 0;
    for (;;) {
        uint32_t c = 0;
        if (lane == 0) c = atomicAdd(s_next, 1u);
        const uint32_t a0 = ub + 32 * __shfl_sync(0xffffffffu, c, 0);
        if (a0 >= ue) break;
        uint32_t base = 0, len = 0;
        if (a0 + lane < ue) {
            const uint32_t u = __ldg(nv + a0 + lane);
            base = __ldg(off + u);
            len = pl ? __ldg(pl + a0 + lane) : count_le_front(dest + base, __ldg(off + u + 1) - base, v);
        }
        count += count_flat4(dest, base, len, s_pre, s_base, s_end, m);
    }
    return count;
}

struct SortedMember {
    static constexpr bool kProbeAll = false;
    const uint32_t *list;
    uint32_t n;
    __device__ __forceinline__ bool operator()(uint32_t w) const { return sorted_contains(list, n, w); }
    __device__ __forceinline__ uint32_t bit(uint32_t w) const { return sorted_contains(list, n, w) ? 1u : 0u; }
};

// One v, upper neighbours [ub, ue) of its row: build the membership test of
// N+(v) (warp table, or the sorted list when it is too long) and count.
__device__ __forceinline__ unsigned long long v_unit(const uint32_t *__restrict__ off,
                                                    const uint32_t *__restrict__ dest,
                                                    const uint32_t *__restrict__ pre_len, uint32_t v, uint32_t pv,
                                                    uint32_t ub, uint32_t ue, uint32_t *table, uint32_t *htable,
                                                    uint32_t *s_pre, uint32_t *s_base, uint32_t *s_end) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t row = __ldg(off + v);
    const uint32_t *nv = dest + row, *pl = pre_len ? pre_len + row : nullptr;
    unsigned long long count = 0;
    if (v < kTcWarpSlots * 32) {
        // exact bitmap of N+(v) over [0, v]: the warp's words are all zero
        // on entry and are zeroed again on exit
        for (uint32_t i = lane; i < pv; i += 32) {
            const uint32_t w = __ldg(nv + i);
            atomicOr(table + (w >> 5), 1u << (w & 31));
        }
        __syncwarp();
        count = stream_pairs(off, dest, nv, pl, v, ub, ue, s_pre, s_base, s_end,
                             BitmapMember{table, kTcWarpSlots * 32 - 1});
        __syncwarp();
        for (uint32_t i = lane; i < pv; i += 32) table[__ldg(nv + i) >> 5] = 0u;
        __syncwarp();
    } else if (pv <= kTcTableMax) {
        uint32_t nh = 0;  // ids of N+(v) at or above kHybridSplit
        for (uint32_t i = lane; i < pv; i += 32) nh += __ldg(nv + i) >= kHybridSplit ? 1u : 0u;
        nh = warp_sum(nh);
        if (2 * nh <= kHybridSlots) {
            uint32_t hmask = 31;
            while (hmask + 1 < 2 * nh) hmask = 2 * hmask + 1;
            for (uint32_t i = lane; i <= hmask; i += 32) htable[i] = kEmptySlot;
            __syncwarp();
            for (uint32_t i = lane; i < pv; i += 32) {
                const uint32_t w = __ldg(nv + i);
                if (w < kHybridSplit) atomicOr(table + (w >> 5), 1u << (w & 31));
                else hash_insert(htable, hmask, w);
            }
            __syncwarp();
            count = stream_pairs(off, dest, nv, pl, v, ub, ue, s_pre, s_base, s_end,
                                 HybridMember{table, htable, hmask});
            __syncwarp();
            for (uint32_t i = lane; i < pv; i += 32) {
                const uint32_t w = __ldg(nv + i);
                if (w < kHybridSplit) table[w >> 5] = 0u;
            }
            __syncwarp();
            return count;
        }
        const uint32_t mask = table_mask(pv);
        for (uint32_t i = lane; i <= mask; i += 32) table[i] = kEmptySlot;
        __syncwarp();
        for (uint32_t i = lane; i < pv; i += 32) hash_insert(table, mask, __ldg(nv + i));
        __syncwarp();
        count = stream_pairs(off, dest, nv, pl, v, ub, ue, s_pre, s_base, s_end, HashMember{table, mask});
        __syncwarp();
        for (uint32_t i = lane; i <= mask; i += 32) table[i] = 0u;
        __syncwarp();
    } else {
        count = stream_pairs(off, dest, nv, pl, v, ub, ue, s_pre, s_base, s_end, SortedMember{nv, pv});
    }
    return count;
}

struct TcBig {  // a v whose upper neighbours are dealt out in kUpperChunk units
    uint32_t v, ub, ue, first_unit;
};

constexpr uint32_t kHubWordsMax = 128;          // H = 32 * words <= 4,096
constexpr uint64_t kHubBytesMax = 1ull << 31;   // bitmap rows of all vertices <= 2 GiB
constexpr uint32_t kHubStepsPerUnit = 64;       // warp steps of pair work per unit

// pairs per warp step for a pivot whose prefix needs nw words (<= 32: lane
// groups of the next power of two; above: one pair, lanes striding words)
__host__ __device__ __forceinline__ uint32_t hub_group(uint32_t nw) {
    uint32_t gs = 1;
    while (gs < nw && gs < 32) gs <<= 1;
    return gs;
}
__host__ __device__ __forceinline__ uint32_t hub_uppers_per_unit(uint32_t v) {
    const uint32_t nw = (v >> 5) + 1;
    return nw <= 32 ? kHubStepsPerUnit * (32 / hub_group(nw)) : kHubStepsPerUnit / ((nw + 31) / 32);
}

// bits[x * hw + k] bit b: 32k + b is a neighbour of x below 32 hw (rows are
// sorted, so those neighbours are a prefix of the row); bits zeroed before
__global__ void tc_hub_bits_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ dest, uint32_t V,
                                   uint32_t hw, uint32_t *bits) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t H = hw * 32;
    for (uint32_t x = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; x < V; x += nwarps) {
        const uint32_t b = __ldg(off + x), e = __ldg(off + x + 1);
        uint32_t *row = bits + (size_t)x * hw;
        for (uint32_t j0 = b; j0 < e; j0 += 32) {
            const uint32_t j = j0 + lane;
            const uint32_t w = j < e ? __ldg(dest + j) : 0xFFFFFFFFu;
            if (w < H) atomicOr(row + (w >> 5), 1u << (w & 31));
            if (!__any_sync(0xffffffffu, w < H) || __ldg(dest + min(j0 + 31, e - 1)) >= H) break;
        }
    }
}

// Units of hub pivots: for v and its upper neighbours [ub, ue), the sum over
// u of popc(bits(u) & bits(v)) over the words covering [0, v).
__global__ void __launch_bounds__(kTcThreads)
    tc_hub_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ dest,
                  const uint32_t *__restrict__ bits, uint32_t hw, const TcBig *__restrict__ hub, uint32_t n_hub,
                  uint32_t n_units, unsigned *cursor, unsigned long long *total) {
    __shared__ unsigned long long sred[32];
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long count = 0;
    for (;;) {
        uint32_t unit = 0;
        if (lane == 0) unit = atomicAdd(cursor, 1u);
        unit = __shfl_sync(0xffffffffu, unit, 0);
        if (unit >= n_units) break;
        uint32_t lo = 0, hi = n_hub - 1;  // last entry with first_unit <= unit
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (hub[mid].first_unit <= unit) lo = mid; else hi = mid - 1;
        }
        const TcBig hv = hub[lo];
        const uint32_t v = hv.v;
        const uint32_t per = hub_uppers_per_unit(v);
        const uint32_t ub = hv.ub + (unit - hv.first_unit) * per;
        const uint32_t ue = min(ub + per, hv.ue);
        const uint32_t *nv = dest + __ldg(off + v);
        const uint32_t *vb = bits + (size_t)v * hw;
        const uint32_t nw = (v >> 5) + 1;                  // words covering [0, v]
        const uint32_t last = (1u << (v & 31)) - 1u;       // ids below v in the last word
        if (nw <= 32) {
            const uint32_t gs = hub_group(nw), ppw = 32 / gs;
            const uint32_t j = lane & (gs - 1), grp = lane / gs;
            uint32_t pw = 0;
            if (j < nw) pw = __ldg(vb + j) & (j == nw - 1 ? last : 0xFFFFFFFFu);
            // eight steps' neighbour ids, then their words, in flight per lane
            for (uint32_t a0 = ub; a0 < ue; a0 += 8 * ppw) {
                uint32_t u[8], w[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const uint32_t a = a0 + q * ppw + grp;
                    u[q] = (a < ue && j < nw) ? __ldg(nv + a) : 0xFFFFFFFFu;
                }
#pragma unroll
                for (int q = 0; q < 8; ++q) w[q] = u[q] != 0xFFFFFFFFu ? __ldg(bits + (size_t)u[q] * hw + j) : 0u;
#pragma unroll
                for (int q = 0; q < 8; ++q) count += __popc(w[q] & pw);
            }
        } else {
            uint32_t pw[kHubWordsMax / 32];
#pragma unroll
            for (uint32_t q = 0; q < kHubWordsMax / 32; ++q) {
                const uint32_t k = q * 32 + lane;
                pw[q] = k < nw ? (__ldg(vb + k) & (k == nw - 1 ? last : 0xFFFFFFFFu)) : 0u;
            }
            // two pairs' neighbour ids, then all their words, in flight
            for (uint32_t a = ub; a < ue; a += 2) {
                const uint32_t u0 = __ldg(nv + a);
                const uint32_t u1 = a + 1 < ue ? __ldg(nv + a + 1) : 0xFFFFFFFFu;
                const uint32_t *r0 = bits + (size_t)u0 * hw;
                const uint32_t *r1 = bits + (size_t)(u1 != 0xFFFFFFFFu ? u1 : u0) * hw;
                uint32_t w0[kHubWordsMax / 32], w1[kHubWordsMax / 32];
#pragma unroll
                for (uint32_t q = 0; q < kHubWordsMax / 32; ++q) {
                    const uint32_t k = q * 32 + lane;
                    w0[q] = k < nw ? __ldg(r0 + k) : 0u;
                    w1[q] = (k < nw && u1 != 0xFFFFFFFFu) ? __ldg(r1 + k) : 0u;
                }
#pragma unroll
                for (uint32_t q = 0; q < kHubWordsMax / 32; ++q) count += __popc(w0[q] & pw[q]) + __popc(w1[q] & pw[q]);
            }
        }
    }
    count = block_sum(count, sred);
    if (threadIdx.x == 0 && count) atomicAdd(total, count);
}

__global__ void __launch_bounds__(kTcThreads, 4)
    tc_vcentric_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ dest,
                       const uint32_t *__restrict__ low, const uint32_t *__restrict__ pre_len,
                       const TcBig *__restrict__ big, uint32_t n_big,
                       uint32_t n_units, const TcBig *__restrict__ small, uint32_t n_small, unsigned *cursor,
                       unsigned long long *total) {
    __shared__ uint32_t tables[kTcWarps][kTcWarpSlots];
    __shared__ uint32_t htables[kTcWarps][kHybridSlots];
    __shared__ uint32_t s_pre[kTcWarps][33];
    __shared__ uint32_t s_base[kTcWarps][32];
    __shared__ uint32_t s_end[kTcWarps][32];
    __shared__ unsigned long long sred[32];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long count = 0;
    for (uint32_t i = lane; i < kTcWarpSlots; i += 32) tables[wid][i] = 0u;  // v_unit keeps it zero
    __syncwarp();
    // big v's: units from an atomic cursor
    for (;;) {
        uint32_t unit = 0;
        if (lane == 0) unit = atomicAdd(cursor, 1u);
        unit = __shfl_sync(0xffffffffu, unit, 0);
        if (unit >= n_units) break;
        uint32_t lo = 0, hi = n_big - 1;  // last big entry with first_unit <= unit
        while (lo < hi) {
            uint32_t mid = (lo + hi + 1) >> 1;
            if (big[mid].first_unit <= unit) lo = mid; else hi = mid - 1;
        }
        const TcBig bg = big[lo];
        const uint32_t ub = bg.ub + (unit - bg.first_unit) * kUpperChunk;
        const uint32_t ue = min(ub + kUpperChunk, bg.ue);
        count += v_unit(off, dest, pre_len, bg.v, __ldg(low + bg.v), ub, ue, tables[wid], htables[wid],
                        s_pre[wid], s_base[wid], s_end[wid]);
    }
    // the other pivots with work (the plan's compact list, with the first
    // upper neighbour precomputed): one warp each
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = gw; i < n_small; i += nw) {
        const TcBig sm = small[i];
        count += v_unit(off, dest, pre_len, sm.v, __ldg(low + sm.v), sm.ub, sm.ue, tables[wid], htables[wid],
                        s_pre[wid], s_base[wid], s_end[wid]);
    }
    count = block_sum(count, sred);
    if (threadIdx.x == 0 && count) atomicAdd(total, count);
}

// The reference's multiplicities: for each v in N+(u) (with repeats) and each
// w in N+(v) (with repeats), w counts when it is in N(u).
__global__ void __launch_bounds__(kTcThreads)
    tc_multiset_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ dest,
                       const uint32_t *__restrict__ low, uint32_t V, unsigned long long *total) {
    __shared__ uint32_t s_pre[kTcWarps][33];
    __shared__ uint32_t s_base[kTcWarps][32];
    __shared__ unsigned long long sred[32];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long count = 0;
    for (uint32_t u = gw; u < V; u += nw) {
        const uint32_t pu = __ldg(low + u);
        if (pu == 0) continue;
        const uint32_t *nu = dest + __ldg(off + u);
        SortedMember m{nu, pu};
        for (uint32_t a0 = 0; a0 < pu; a0 += 32) {
            uint32_t base = 0, len = 0;
            if (a0 + lane < pu) {
                const uint32_t v = __ldg(nu + a0 + lane);
                base = __ldg(off + v);
                len = __ldg(low + v);
            }
            count += count_flat(dest, base, len, s_pre[wid], s_base[wid], m);
        }
    }
    count = block_sum(count, sred);
    if (threadIdx.x == 0 && count) atomicAdd(total, count);
}

// Long N+(v) (above the per-warp table): one CTA per unit of kWideChunk upper
// neighbours, N+(v) hashed once into a CTA-wide shared table of `slots`
// entries (load factor <= 1/2), every warp streaming 32 upper neighbours'
// prefixes at a time against it.
constexpr int kWideThreads = 1024;
constexpr uint32_t kWideChunk = 4096;
constexpr uint32_t kWideSlotsMax = 32768;  // 128 KiB: |N+(v)| <= 16384
static_assert((kWideSlotsMax & (kWideSlotsMax - 1)) == 0 && (kTcWarpSlots & (kTcWarpSlots - 1)) == 0,
              "bitmap tables must cover a power-of-two id range (BitmapMember masks ids)");

__global__ void __launch_bounds__(kWideThreads, 1)
    tc_wide_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ dest,
                   const uint32_t *__restrict__ low, const uint32_t *__restrict__ pre_len,
                   const TcBig *__restrict__ wide, uint32_t n_wide,
                   uint32_t n_units, uint32_t slots, unsigned *cursor, unsigned long long *total) {
    extern __shared__ uint32_t s_table[];
    __shared__ uint32_t s_pre[kWideThreads / 32][33];
    __shared__ uint32_t s_base[kWideThreads / 32][32];
    __shared__ uint32_t s_end[kWideThreads / 32][32];
    __shared__ uint32_t s_unit;
    __shared__ unsigned s_next;
    __shared__ unsigned long long sred[32];
    const uint32_t wid = threadIdx.x >> 5;
    unsigned long long count = 0;
    for (uint32_t i = threadIdx.x; i < slots; i += blockDim.x) s_table[i] = 0u;  // kept zero between units
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_unit = atomicAdd(cursor, 1u);
        __syncthreads();
        const uint32_t unit = s_unit;
        if (unit >= n_units) break;
        uint32_t lo = 0, hi = n_wide - 1;  // last entry with first_unit <= unit
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (wide[mid].first_unit <= unit) lo = mid; else hi = mid - 1;
        }
        const TcBig bg = wide[lo];
        const uint32_t v = bg.v, pv = __ldg(low + v);
        const uint32_t ub = bg.ub + (unit - bg.first_unit) * kWideChunk;
        const uint32_t ue = min(ub + kWideChunk, bg.ue);
        const uint32_t row = __ldg(off + v);
        const uint32_t *nv = dest + row, *pl = pre_len ? pre_len + row : nullptr;
        if (threadIdx.x == 0) s_next = 0;
        if (v < slots * 32) {
            // exact bitmap of N+(v) over [0, v]
            for (uint32_t i = threadIdx.x; i < pv; i += blockDim.x) {
                const uint32_t w = __ldg(nv + i);
                atomicOr(s_table + (w >> 5), 1u << (w & 31));
            }
            __syncthreads();
            count += stream_pairs_dealt(off, dest, nv, pl, v, ub, ue, s_pre[wid], s_base[wid], s_end[wid],
                                        BitmapMember{s_table, slots * 32 - 1}, &s_next);
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < pv; i += blockDim.x) s_table[__ldg(nv + i) >> 5] = 0u;
        } else {
            uint32_t mask = 63;
            while (mask + 1 < 2 * pv && mask + 1 < slots) mask = 2 * mask + 1;
            for (uint32_t i = threadIdx.x; i <= mask; i += blockDim.x) s_table[i] = kEmptySlot;
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < pv; i += blockDim.x) hash_insert(s_table, mask, __ldg(nv + i));
            __syncthreads();
            count += stream_pairs_dealt(off, dest, nv, pl, v, ub, ue, s_pre[wid], s_base[wid], s_end[wid],
                                        HashMember{s_table, mask}, &s_next);
            __syncthreads();
            for (uint32_t i = threadIdx.x; i <= mask; i += blockDim.x) s_table[i] = 0u;
        }
    }
    count = block_sum(count, sred);
    if (threadIdx.x == 0 && count) atomicAdd(total, count);
}

// Work lists of the v-centric count. kind 3: v's below the hub range H with
// pairs (units of hub_uppers_per_unit(v), tc_hub_kernel); for the others,
// kind 0: v's with more than kUpperChunk upper neighbours and |N+(v)| within
// the warp table (units of kUpperChunk); kind 1: v's with |N+(v)| above the
// warp table and within the CTA table (units of kWideChunk, for
// tc_wide_kernel); kind 2: every other v with N+(v) and an upper neighbour
// (one warp each). v's without both have no pairs and are in no list.
__global__ void tc_plan_flags_kernel(const uint32_t *off, const uint32_t *dest, const uint32_t *low, uint32_t V,
                                     uint32_t H, uint32_t *flag /* 4V: kinds 0, 1, 2, 3 */,
                                     uint32_t *units /* 3V: kinds 0, 1, 3 */, uint32_t *ub_out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const uint32_t b = off[v], d = off[v + 1] - b;
        const uint32_t ub = count_lt(dest + b, d, v);
        const uint32_t up = d - ub, pv = low[v];
        const bool pairs = pv > 0 && up > 0;
        const bool hub = v < H;
        const bool wide = !hub && pv > kTcTableMax && pv <= kWideSlotsMax / 2;
        const bool big = !hub && !wide && (up > kUpperChunk || pv > kTcTableMax);
        flag[v] = pairs && big ? 1u : 0u;
        flag[(size_t)V + v] = pairs && wide ? 1u : 0u;
        flag[2 * (size_t)V + v] = pairs && !hub && !big && !wide ? 1u : 0u;
        flag[3 * (size_t)V + v] = pairs && hub ? 1u : 0u;
        units[v] = pairs && big ? (up + kUpperChunk - 1) / kUpperChunk : 0u;
        units[(size_t)V + v] = pairs && wide ? (up + kWideChunk - 1) / kWideChunk : 0u;
        const uint32_t per = hub_uppers_per_unit(v);
        units[2 * (size_t)V + v] = pairs && hub ? (up + per - 1) / per : 0u;
        ub_out[v] = ub;
    }
}

__global__ void tc_plan_scatter_kernel(const uint32_t *off, const uint32_t *flag, const uint32_t *pos,
                                       const uint32_t *unit_pre, const uint32_t *ub, uint32_t V, TcBig *big,
                                       TcBig *wide, TcBig *small, TcBig *hub) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const uint32_t d = off[v + 1] - off[v];
        if (flag[v]) big[pos[v]] = TcBig{v, ub[v], d, unit_pre[v]};
        if (flag[(size_t)V + v]) wide[pos[(size_t)V + v]] = TcBig{v, ub[v], d, unit_pre[(size_t)V + v]};
        if (flag[2 * (size_t)V + v]) small[pos[2 * (size_t)V + v]] = TcBig{v, ub[v], d, 0u};
        if (flag[3 * (size_t)V + v]) hub[pos[3 * (size_t)V + v]] = TcBig{v, ub[v], d, unit_pre[2 * (size_t)V + v]};
    }
}

}  // namespace gbx

// Per-graph cache of the fast path's work decomposition.
struct gbx_tc_plan {
    gbx::TcBig *big = nullptr;   // warp-table v's with many upper neighbours
    gbx::TcBig *wide = nullptr;  // CTA-table v's (|N+(v)| above the warp table)
    gbx::TcBig *small = nullptr; // the other v's with pairs, one warp each
    gbx::TcBig *hub = nullptr;   // v's below the hub range (bitmap rows)
    uint32_t *hub_bits = nullptr;  // V rows of hub_words words: N(x) ∩ [0, 32 hub_words)
    uint32_t *pre_len = nullptr;   // per edge v->u with u >= v: |N(u) ∩ [0, v]|
    uint32_t hub_words = 0;
    uint32_t n_big = 0, n_units = 0;
    uint32_t n_wide = 0, n_wunits = 0;
    uint32_t n_small = 0;
    uint32_t n_hub = 0, n_hunits = 0;
};

using namespace gbx;

static int tc_prepare(gbx_graph *g, cudaStream_t s) {
    const uint32_t V = g->V;
    const unsigned grid = std::min<unsigned>(ceil_div(V, 256), (unsigned)num_sms() * 8);
    const unsigned wgrid = std::min<unsigned>(ceil_div((uint64_t)V * 32, kTcThreads), (unsigned)num_sms() * 8);
    if (!g->low_count) {
        void *lp = nullptr;
        GBX_TRY(dev_alloc(&lp, (size_t)V * 4, s));
        uint32_t *low = static_cast<uint32_t *>(lp);
        tc_low_count_kernel<<<grid, 256, 0, s>>>(g->offsets, g->dest, V, low);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            cudaStreamSynchronize(s);
            dev_free(low);
            return cuda_fail(e, "tc_low_count_kernel", __FILE__, __LINE__);
        }
        note_launch();
        g->low_count = low;
    }
    if (g->simple_rows < 0) {
        DevBuf<unsigned long long> flags;  // [0] repeat flags, [1] asymmetry hash sum
        GBX_TRY(flags.alloc(2, s));
        GBX_CUDA(cudaMemsetAsync(flags.p, 0, 16, s));
        tc_shape_check_kernel<<<wgrid, kTcThreads, 0, s>>>(g->offsets, g->dest, V, g->E,
                                                           reinterpret_cast<unsigned *>(flags.p), flags.p + 1);
        GBX_LAUNCH_CHECK();
        unsigned long long h[2] = {0, 0};
        GBX_CUDA(cudaMemcpyAsync(h, flags.p, 16, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        g->simple_rows = (h[0] & 1u) ? 0 : 1;
        g->symmetric = h[1] ? 0 : 1;
    }
    if (g->simple_rows == 1 && g->symmetric == 1 && !g->tc_plan) {
        DevBuf<uint32_t> flag, pos, units, unit_pre, ub, tot;
        GBX_TRY(flag.alloc(4 * (size_t)V, s));
        GBX_TRY(pos.alloc(4 * (size_t)V, s));
        GBX_TRY(units.alloc(3 * (size_t)V, s));
        GBX_TRY(unit_pre.alloc(3 * (size_t)V, s));
        GBX_TRY(ub.alloc(V, s));
        GBX_TRY(tot.alloc(7, s));
        gbx_tc_plan *p = new gbx_tc_plan();
        // hub range: 32 hw ids, hw a power of two <= kHubWordsMax with the
        // bitmap rows of all V vertices within kHubBytesMax
        uint32_t hw = kHubWordsMax;
        while (hw > 1 && (uint64_t)V * hw * 4 > kHubBytesMax) hw >>= 1;
        if ((uint64_t)V * hw * 4 > kHubBytesMax) hw = 0;
        const uint32_t H = hw * 32;
        auto build = [&]() -> int {
            // the four work lists in one classification pass, seven scans
            // and one host round trip for the list sizes
            tc_plan_flags_kernel<<<grid, 256, 0, s>>>(g->offsets, g->dest, g->low_count, V, H, flag.p, units.p,
                                                      ub.p);
            GBX_LAUNCH_CHECK();
            for (int k = 0; k < 4; ++k)
                GBX_TRY(exclusive_scan_u32(flag.p + (size_t)k * V, pos.p + (size_t)k * V, V, s, tot.p + k));
            for (int k = 0; k < 3; ++k)
                GBX_TRY(exclusive_scan_u32(units.p + (size_t)k * V, unit_pre.p + (size_t)k * V, V, s, tot.p + 4 + k));
            uint32_t h[7];
            GBX_CUDA(cudaMemcpyAsync(h, tot.p, sizeof(h), cudaMemcpyDeviceToHost, s));
            GBX_CUDA(cudaStreamSynchronize(s));
            p->n_big = h[0];
            p->n_wide = h[1];
            p->n_small = h[2];
            p->n_hub = h[3];
            p->n_units = h[4];
            p->n_wunits = h[5];
            p->n_hunits = h[6];
            GBX_TRY(dev_alloc((void **)&p->big, sizeof(TcBig) * (h[0] ? h[0] : 1), s));
            GBX_TRY(dev_alloc((void **)&p->wide, sizeof(TcBig) * (h[1] ? h[1] : 1), s));
            GBX_TRY(dev_alloc((void **)&p->small, sizeof(TcBig) * (h[2] ? h[2] : 1), s));
            GBX_TRY(dev_alloc((void **)&p->hub, sizeof(TcBig) * (h[3] ? h[3] : 1), s));
            tc_plan_scatter_kernel<<<grid, 256, 0, s>>>(g->offsets, flag.p, pos.p, unit_pre.p, ub.p, V, p->big,
                                                        p->wide, p->small, p->hub);
            GBX_LAUNCH_CHECK();
            if (p->n_hub) {
                const size_t bytes = (size_t)V * hw * 4;
                GBX_TRY(dev_alloc((void **)&p->hub_bits, bytes, s));
                GBX_CUDA(cudaMemsetAsync(p->hub_bits, 0, bytes, s));
                tc_hub_bits_kernel<<<wgrid, 256, 0, s>>>(g->offsets, g->dest, V, hw, p->hub_bits);
                GBX_LAUNCH_CHECK();
                p->hub_words = hw;
            }
            return GBX_OK;
        };
        const int st = build();
        if (st != GBX_OK) {
            cudaStreamSynchronize(s);
            gbx_free_tc_plan(p);
            return st;
        }
        g->tc_plan = p;
    } else if (g->tc_plan && !g->tc_plan->pre_len && g->E) {
        // the graph is counted again: from now on its counts read the
        // prefix lengths (building them costs about as much as the row
        // searches of one count, so a graph counted once never pays for them)
        gbx_tc_plan *p = g->tc_plan;
        GBX_TRY(dev_alloc((void **)&p->pre_len, (size_t)g->E * 4, s));
        const unsigned egrid =
            std::min<unsigned>(ceil_div(ceil_div((uint64_t)g->E, 2048) * 32, 256), (unsigned)num_sms() * 8);
        tc_prefix_len_kernel<<<egrid, 256, 0, s>>>(g->offsets, g->dest, V, g->E, p->pre_len);
        GBX_LAUNCH_CHECK();
    }
    return GBX_OK;
}

void gbx_free_tc_plan(gbx_tc_plan *p) {
    if (!p) return;
    dev_free(p->big);
    dev_free(p->wide);
    dev_free(p->small);
    dev_free(p->hub);
    dev_free(p->hub_bits);
    dev_free(p->pre_len);
    delete p;
}

extern "C" int gbx_tc(gbx_graph *g, uint64_t *total, void *stream) {
    clear_error();
    GBX_REQUIRE(g && total, GBX_ERR_INVALID, "graph or total is NULL");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V;
    GBX_TRY(tc_prepare(g, s));
    DevBuf<unsigned long long> d;
    DevBuf<unsigned> cursor;
    GBX_TRY(d.alloc(1, s));
    GBX_TRY(cursor.alloc(3, s));
    GBX_CUDA(cudaMemsetAsync(d.p, 0, 8, s));
    GBX_CUDA(cudaMemsetAsync(cursor.p, 0, 12, s));
    if (g->tc_plan) {
        int per_sm = 0;
        GBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc_vcentric_kernel, kTcThreads, 0));
        const unsigned grid = (unsigned)std::max(1, per_sm) * (unsigned)num_sms();
        const gbx_tc_plan *p = g->tc_plan;
        tc_vcentric_kernel<<<grid, kTcThreads, 0, s>>>(g->offsets, g->dest, g->low_count, p->pre_len, p->big,
                                                       p->n_big, p->n_big ? p->n_units : 0u, p->small, p->n_small,
                                                       cursor.p, d.p);
        GBX_LAUNCH_CHECK();
        if (p->n_wide) {
            const size_t smem = (size_t)kWideSlotsMax * 4;
            GBX_CUDA(cudaFuncSetAttribute(tc_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            int wper = 0;
            GBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&wper, tc_wide_kernel, kWideThreads, smem));
            const unsigned wgrid = std::min<unsigned>((unsigned)std::max(1, wper) * (unsigned)num_sms(), p->n_wunits);
            tc_wide_kernel<<<wgrid, kWideThreads, smem, s>>>(g->offsets, g->dest, g->low_count, p->pre_len,
                                                              p->wide, p->n_wide, p->n_wunits, kWideSlotsMax,
                                                              cursor.p + 1, d.p);
        }
        if (p->n_hub) {
            GBX_LAUNCH_CHECK();
            int hper = 0;
            GBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&hper, tc_hub_kernel, kTcThreads, 0));
            const unsigned hgrid = std::min<unsigned>((unsigned)std::max(1, hper) * (unsigned)num_sms(),
                                                      ceil_div(p->n_hunits, kTcWarps));
            tc_hub_kernel<<<hgrid, kTcThreads, 0, s>>>(g->offsets, g->dest, p->hub_bits, p->hub_words, p->hub,
                                                       p->n_hub, p->n_hunits, cursor.p + 2, d.p);
        }
    } else {
        const unsigned wgrid = std::min<unsigned>(ceil_div((uint64_t)V * 32, kTcThreads), (unsigned)num_sms() * 8);
        tc_multiset_kernel<<<wgrid, kTcThreads, 0, s>>>(g->offsets, g->dest, g->low_count, V, d.p);
    }
    GBX_LAUNCH_CHECK();
    if (is_device_ptr(total)) {
        GBX_CUDA(cudaMemcpyAsync(total, d.p, 8, cudaMemcpyDeviceToDevice, s));
        return GBX_OK;
    }
    unsigned long long h = 0;
    GBX_CUDA(cudaMemcpyAsync(&h, d.p, 8, cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    *total = h;
    return GBX_OK;
}
