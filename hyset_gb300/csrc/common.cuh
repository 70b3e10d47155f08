// common.cuh — device-side views and helpers shared by the join kernels.
//
// Layout in HBM (all uint32, CSR):
//   tokens[T]  the sets' tokens, each set sorted ascending
//   starts[n]  offset of set i in tokens
//   sizes[n]   |set i|, non-decreasing in i (the reference's size-sorted order)
// Bounds are looked up in tables the host fills with the reference's own double
// expressions (include/hyset/similarity.hpp:11-54); no floating point runs on
// the device, so every bound is bit-identical to the reference's.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace hs {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr uint32_t NOWN = 0xFFFFFFFFu;  // "no ownership constraint"

enum Sim : int { SIM_JACCARD = 0, SIM_COSINE = 1, SIM_DICE = 2 };

struct CollView {
    const uint32_t* __restrict__ tokens;
    const uint32_t* __restrict__ starts;
    const uint32_t* __restrict__ sizes;
    const uint2* __restrict__ meta;  // (start, size) per set: one 8-byte load instead of two
    uint32_t n;
};

// Host-computed bound tables over set lengths 0..L.
struct BoundsView {
    const uint32_t* __restrict__ minsize;       // [L+1]  Similarity::minsize
    const uint32_t* __restrict__ probe_prefix;  // [L+1]  maxprefix
    const uint32_t* __restrict__ index_prefix;  // [L+1]  midprefix (self-join) or maxprefix (R-S)
    const uint32_t* __restrict__ max_partner;   // [L+1]  largest l with minsize(l) <= len
    const uint32_t* __restrict__ mid_prefix;    // [L+1]  midprefix
    const uint32_t* __restrict__ mo_sum;        // [2L+1] raw minoverlap by l1+l2 (jaccard, dice)
    const uint64_t* __restrict__ mo_row;        // [L+2]  cosine: row offsets by larger length
    const uint32_t* __restrict__ mo_tab;        // cosine: raw minoverlap at (big, small)
    uint32_t L;
    int sim;
    // [L+1] jaccard, dice: the largest l1 + l2 whose raw minoverlap is at most
    // v (nullptr for cosine or a table that is not monotone)
    const uint32_t* __restrict__ max_sum = nullptr;
    // cosine: bound fields by (size, position), rows lp_row[l] (see Bounds)
    const uint32_t* __restrict__ lp_row = nullptr;
    const uint32_t* __restrict__ lp_tab = nullptr;
};

// Copy chunks of a host-input join (in tokens): 64 MB while more than three
// remain, then a third of what is left, at least 16 MB, so the work left when
// the last chunk lands is small.  The next chunk's size when `rem` tokens are
// left (the host schedules the copies with it, the size scan finds the sets
// each chunk completes with it).
constexpr uint64_t PIPE_CHUNK_TOKENS = 16ull << 20;
constexpr uint64_t PIPE_TAIL_TOKENS = 4ull << 20;
constexpr uint32_t PIPE_MAX_CHUNKS = 1024;  // 2^32 tokens take at most 259
__host__ __device__ inline uint64_t pipe_chunk(uint64_t rem) {
    uint64_t c = (rem / 3 + 0xFFFFu) & ~0xFFFFull;
    c = c > PIPE_TAIL_TOKENS ? c : PIPE_TAIL_TOKENS;
    c = c < PIPE_CHUNK_TOKENS ? c : PIPE_CHUNK_TOKENS;
    return c < rem ? c : rem;
}

// The low field of a bound-layout index entry (a self-join's midprefix index,
// jaccard or dice) for position pos of a set of size len: the longest probe lp
// (lp >= len, as every probe of a self-join window) whose positional bound this
// side of the pair admits, len - pos >= minoverlap(lp, len).  For pos > 0 that
// is raw minoverlap(lp + len) <= len - pos, i.e. lp + len <= max_sum[len - pos];
// pos 0 admits every probe (maxf, at least the longest set).
__device__ __forceinline__ uint32_t bound_field(const uint32_t* __restrict__ max_sum, uint32_t len, uint32_t pos,
                                                uint32_t maxf) {
    if (pos == 0) return maxf;
    const uint32_t s = max_sum[len - pos];
    return s <= len ? 0u : min(maxf, s - len);
}
// The tables a bound-layout index build reads (all null: positions).
struct BoundFields {
    const uint32_t* __restrict__ max_sum;  // jaccard, dice
    const uint32_t* __restrict__ lp_row;   // cosine
    const uint32_t* __restrict__ lp_tab;
    __host__ __device__ bool on() const { return max_sum || lp_tab; }
};
// The field from either table (any similarity with monotone minoverlap).
__device__ __forceinline__ uint32_t bound_field_of(const BoundFields& F, uint32_t len, uint32_t pos, uint32_t maxf) {
    if (F.max_sum) return bound_field(F.max_sum, len, pos, maxf);
    return min(maxf, F.lp_tab[F.lp_row[len] + pos]);
}

// generic_similarity::minoverlap (similarity.hpp:21-23): min(l2, min(l1, raw)).
// Requires big >= small >= minsize(big) (guaranteed by every caller's length window).
__device__ __forceinline__ uint32_t minoverlap(const BoundsView& B, uint32_t big, uint32_t small) {
    uint32_t raw;
    if (B.sim == SIM_COSINE)
        raw = B.mo_tab[B.mo_row[big] + (small - B.minsize[big])];
    else
        raw = B.mo_sum[big + small];
    return min(small, min(big, raw));
}

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t* a, uint32_t lo, uint32_t hi, uint32_t key) {
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Two lower bounds over the same sorted range, searched in lockstep: each
// step issues both probes' loads together, so the two dependent chains cost
// one chain's latency.
__device__ __forceinline__ void lower_bound2_u32(const uint32_t* __restrict__ a, uint32_t lo, uint32_t hi,
                                                 uint32_t k1, uint32_t k2, uint32_t& r1, uint32_t& r2) {
    uint32_t l1 = lo, h1 = hi, l2 = lo, h2 = hi;
    while (l1 < h1 || l2 < h2) {
        const uint32_t m1 = (l1 + h1) >> 1, m2 = (l2 + h2) >> 1;
        const uint32_t v1 = l1 < h1 ? __ldg(a + m1) : 0u, v2 = l2 < h2 ? __ldg(a + m2) : 0u;
        if (l1 < h1) {
            if (v1 < k1) l1 = m1 + 1;
            else h1 = m1;
        }
        if (l2 < h2) {
            if (v2 < k2) l2 = m2 + 1;
            else h2 = m2;
        }
    }
    r1 = l1;
    r2 = l2;
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += y;
    }
    return v;
}

__device__ __forceinline__ unsigned lanemask_lt(int lane) { return (1u << lane) - 1u; }

// Result sink.  `count` always advances (so the host learns the true count);
// pairs past `cap` are dropped and the host re-runs with a larger buffer.
struct Sink {
    uint2* pairs;
    unsigned long long* count;
    unsigned long long cap;
    int count_only;
    int swap;  // store (second, first): an R-S join run with the collections' roles exchanged
};

// Warp-aggregated append; every lane of the warp must call it.
__device__ __forceinline__ void emit(const Sink& out, bool want, uint32_t first, uint32_t second, int lane) {
    unsigned m = __ballot_sync(FULL, want);
    if (!m) return;
    int leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(out.count, (unsigned long long)__popc(m));
    base = __shfl_sync(FULL, base, leader);
    if (want && !out.count_only) {
        unsigned long long pos = base + __popc(m & lanemask_lt(lane));
        if (pos < out.cap) out.pairs[pos] = out.swap ? make_uint2(second, first) : make_uint2(first, second);
    }
}

// One lane, two-pointer merge with the reference's early-exit bounds
// (include/hyset/verification.hpp:35-58), from the start of both sets.
// own_a != NOWN: the pair belongs to the caller only if the smallest common
// token sits at a[own_a]; otherwise the function returns false at the first
// common token (another work item owns the pair).
// *used (optional) receives the number of tokens read from a and b.
__device__ __forceinline__ bool verify_serial(const uint32_t* a, uint32_t na, const uint32_t* __restrict__ b,
                                              uint32_t nb, uint32_t thr, uint32_t own_a, uint32_t* used = nullptr) {
    uint32_t i = 0, k = 0, found = 0, maxa = na, maxb = nb;
    bool ok = true;
    while (maxa >= thr && maxb >= thr && found < thr) {
        uint32_t x = a[i], y = __ldg(b + k);
        if (x == y) {
            if (found == 0 && own_a != NOWN && i != own_a) {
                ok = false;
                break;
            }
            ++i; ++k; ++found;
        } else if (x < y) {
            ++i; --maxa;
        } else {
            ++k; --maxb;
        }
    }
    if (used) *used = i + k + (ok ? 0u : 1u);
    return ok && found >= thr;
}

// Whole warp, merge-path style: 32 tokens of b per step (one coalesced 128-byte
// load), each lane locates its token in a by binary search, matches are counted
// with __ballot_sync.  After each step the exact remaining upper bound
// found + min(|b| - consumed_b, |a| - consumed_a) ends the loop as soon as the
// pair can no longer reach thr, and the loop also ends once found >= thr.
// own_b != NOWN: a match at b[k], k < own_b, means a smaller common token
// exists, so the pair is owned by another work item and false is returned.
// All 32 lanes must call it with the same arguments.
// *used (optional) receives the number of tokens of b read plus the positions
// of a searched past (a bound on the tokens of a read).
__device__ __forceinline__ bool verify_warp(const uint32_t* a, uint32_t na, const uint32_t* __restrict__ b,
                                            uint32_t nb, uint32_t thr, uint32_t own_b, int lane,
                                            uint32_t* used = nullptr) {
    uint32_t found = 0, alo = 0;
    if (used) *used = nb;
    for (uint32_t k0 = 0; k0 < nb; k0 += 32) {
        if (used) *used = min(nb, k0 + 32) + alo;
        uint32_t k = k0 + lane;
        bool valid = k < nb;
        uint32_t y = valid ? __ldg(b + k) : 0xFFFFFFFFu;
        uint32_t pos = valid ? lower_bound_u32(a, alo, na, y) : na;
        bool hit = valid && pos < na && a[pos] == y;
        unsigned m = __ballot_sync(FULL, hit);
        if (own_b != NOWN && own_b > k0) {
            uint32_t lim = own_b - k0;
            unsigned early = lim >= 32 ? FULL : ((1u << lim) - 1u);
            if (m & early) return false;
        }
        found += __popc(m);
        uint32_t last = min(31u, nb - 1 - k0);
        uint32_t consumed_a = __shfl_sync(FULL, pos + (hit ? 1u : 0u), last);
        uint32_t consumed_b = k0 + last + 1;
        if (found >= thr) return true;
        if (found + min(nb - consumed_b, na - consumed_a) < thr) return false;
        alo = consumed_a;
    }
    return found >= thr;
}

}  // namespace hs
