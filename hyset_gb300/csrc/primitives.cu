// primitives.cu — HBM-bound building blocks of the inverted index and the
// signatures: device-wide scan, stable radix sort, warp-aggregated histogram and
// scatter, prefix-entry emission, XOR bitmaps.
//
// Replaces the reference's index::histogram / thrust::exclusive_scan /
// index::create_index / thrust::sort (include/hyset/index.hpp:217-313) and
// bitmap::generate (include/hyset/device_algorithms.hpp:58-74).
#include "kernels.h"

#include <algorithm>
#include <atomic>

namespace hs {

static std::atomic<unsigned long long> g_launches{0};
unsigned long long launches() { return g_launches.load(); }
void note_launches(unsigned n) { g_launches += n; }

namespace {

// Index lists of at most LIST_SHORT entries are filled by atomic slots and put
// back in set order inside one warp (k_list_scatter, k_list_rank); longer
// ones go through the radix passes.
constexpr uint32_t LIST_SHORT = 64;
constexpr int RANK_THREADS = 256;
constexpr uint32_t RANK_CAP = 1024;  // staged entries per warp (16 lists of up to LIST_SHORT always fit)

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr uint32_t SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 2048

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* warp_sums, uint32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = warp_incl_scan(v, lane);
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (SCAN_THREADS / 32) ? warp_sums[lane] : 0;
        uint32_t wi = warp_incl_scan(w, lane);
        if (lane < (SCAN_THREADS / 32)) warp_sums[lane] = wi - w;
        if (lane == (SCAN_THREADS / 32) - 1) warp_sums[SCAN_THREADS / 32] = wi;
    }
    __syncthreads();
    uint32_t r = warp_sums[warp] + incl - v;
    total = warp_sums[SCAN_THREADS / 32];
    __syncthreads();
    return r;
}

// gate: when non-null, the scans (and the radix kernels) run only when the
// word is above LIST_SHORT: an index whose lists are not all short is sorted
// by the radix passes, the others by k_list_scatter and k_list_rank
__device__ __forceinline__ bool gated_off(const uint32_t* gate) { return gate && *gate <= LIST_SHORT; }

__global__ void __launch_bounds__(SCAN_THREADS) k_tile_reduce(const uint32_t* in, uint64_t n, uint32_t* sums,
                                                              const uint32_t* gate) {
    if (gated_off(gate)) return;
    __shared__ uint32_t ws[SCAN_THREADS / 32 + 1];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i)
        if (base + i < n) s += in[base + i];
    uint32_t total;
    block_excl_scan(s, ws, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// in/out may alias: every tile reads all its inputs before writing.
__global__ void __launch_bounds__(SCAN_THREADS) k_tile_scan(const uint32_t* in, uint32_t* out, uint64_t n,
                                                            const uint32_t* tile_off, const uint32_t* gate) {
    if (gated_off(gate)) return;
    __shared__ uint32_t ws[SCAN_THREADS / 32 + 1];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        v[i] = base + i < n ? in[base + i] : 0;
        s += v[i];
    }
    uint32_t total;
    uint32_t run = block_excl_scan(s, ws, total) + (tile_off ? tile_off[blockIdx.x] : 0);
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
}

// ---- radix sort -----------------------------------------------------------
// Digits of up to 10 bits (a 20-bit token key sorts in two passes).
constexpr int RADIX_THREADS = 512;
constexpr int RADIX_WARPS = RADIX_THREADS / 32;
constexpr int RADIX_ROUNDS = 8;                                   // 32-item rounds per warp
constexpr uint32_t RADIX_TILE = RADIX_THREADS * RADIX_ROUNDS;     // 4096
constexpr int RADIX_MAX_BITS = 10;
constexpr int RADIX_BINS = 1 << RADIX_MAX_BITS;

__global__ void __launch_bounds__(RADIX_THREADS) k_radix_upsweep(const uint32_t* keys, uint64_t n, int shift,
                                                                 uint32_t mask, uint32_t* tile_counts,
                                                                 uint32_t tiles, const uint32_t* gate) {
    if (gated_off(gate)) return;
    __shared__ uint32_t hist[RADIX_BINS];
    const uint64_t base = (uint64_t)blockIdx.x * RADIX_TILE + threadIdx.x;
    uint32_t k[RADIX_ROUNDS];  // loads first, in flight under the zeroing
#pragma unroll
    for (int r = 0; r < RADIX_ROUNDS; ++r) {
        const uint64_t idx = base + (uint64_t)r * RADIX_THREADS;
        k[r] = idx < n ? keys[idx] : 0u;
    }
    for (uint32_t d = threadIdx.x; d <= mask; d += RADIX_THREADS) hist[d] = 0;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RADIX_ROUNDS; ++r)
        if (base + (uint64_t)r * RADIX_THREADS < n) atomicAdd(&hist[(k[r] >> shift) & mask], 1u);
    __syncthreads();
    for (uint32_t d = threadIdx.x; d <= mask; d += RADIX_THREADS)
        tile_counts[(uint64_t)d * tiles + blockIdx.x] = hist[d];
}

// Stable scatter: an item's rank inside its tile is the number of equal digits
// before it (warp w owns items [w*512, w*512+512) of the tile, processed in
// order, 32 at a time, peers found with __match_any_sync).  The tile is first
// reordered by digit in shared memory, so each digit's run of the tile leaves
// as consecutive addresses (coalesced stores instead of one sector per item).
constexpr int RADIX_THREAD_BINS = RADIX_BINS / RADIX_THREADS;  // 2
struct RadixSmem {
    union {
        uint32_t whist[RADIX_WARPS][RADIX_BINS];  // per-warp digit counts, then per-warp bases
        struct {
            uint32_t k[RADIX_TILE], v[RADIX_TILE];  // the tile ordered by digit
        } tile;
    } u;
    uint32_t start[RADIX_BINS];  // tile-local first position of each digit
    uint32_t gpos[RADIX_BINS];   // global first position of each digit for this tile
    uint32_t wsum[RADIX_THREAD_BINS][RADIX_WARPS];
};

#ifndef HS_RADIX_MIN_BLOCKS
#define HS_RADIX_MIN_BLOCKS 2  // 54 registers, no spills; two 72 KB blocks per SM
#endif
__global__ void __launch_bounds__(RADIX_THREADS, HS_RADIX_MIN_BLOCKS) k_radix_downsweep(const uint32_t* __restrict__ keys,
                                                                   const uint32_t* __restrict__ vals, uint64_t n,
                                                                   int shift, uint32_t mask,
                                                                   const uint32_t* __restrict__ tile_off,
                                                                   uint32_t tiles, uint32_t* keys_out,
                                                                   uint32_t* vals_out, const uint32_t* gate) {
    if (gated_off(gate)) return;
    extern __shared__ __align__(16) uint8_t radix_smem[];
    RadixSmem& sm = *reinterpret_cast<RadixSmem*>(radix_smem);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t bins = mask + 1;
    const uint64_t tile_base = (uint64_t)blockIdx.x * RADIX_TILE;
    const uint64_t base = tile_base + (uint64_t)warp * (32 * RADIX_ROUNDS);
    uint32_t k[RADIX_ROUNDS], v[RADIX_ROUNDS], rank[RADIX_ROUNDS];
    // the warp's key loads first (8 in flight per thread, under the zeroing
    // below), then the ranking rounds, whose warp barriers would otherwise hold
    // each round's load behind the previous round; the values follow later
#pragma unroll
    for (int r = 0; r < RADIX_ROUNDS; ++r) {
        const uint64_t idx = base + (uint64_t)r * 32 + lane;
        k[r] = idx < n ? keys[idx] : 0u;
    }
    {  // zero the per-warp counts, 16 bytes a store
        uint4* z = reinterpret_cast<uint4*>(&sm.u.whist[0][0]);
        for (uint32_t q = threadIdx.x; q < RADIX_WARPS * RADIX_BINS / 4; q += RADIX_THREADS)
            z[q] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RADIX_ROUNDS; ++r) {
        const bool valid = base + (uint64_t)r * 32 + lane < n;
        const uint32_t d = valid ? ((k[r] >> shift) & mask) : 0xFFFFFFFFu;
        const unsigned peers = __match_any_sync(FULL, d);
        const int leader = __ffs(peers) - 1;
        const uint32_t cnt = valid ? sm.u.whist[warp][d] : 0;
        __syncwarp();
        if (valid && lane == leader) sm.u.whist[warp][d] = cnt + __popc(peers);
        __syncwarp();
        rank[r] = cnt + __popc(peers & lanemask_lt(lane));
    }
    __syncthreads();
    // per digit: warp bases (exclusive over warps) and the digit's tile total.
    // Thread t owns digits t and t + 512, so a warp's accesses are 32
    // consecutive words (no bank conflicts).
    uint32_t tot[RADIX_THREAD_BINS];
#pragma unroll
    for (int j = 0; j < RADIX_THREAD_BINS; ++j) {
        const uint32_t d = threadIdx.x + j * RADIX_THREADS;
        uint32_t acc = 0;
#pragma unroll
        for (int w = 0; w < RADIX_WARPS; ++w) {
            const uint32_t c = sm.u.whist[w][d];
            sm.u.whist[w][d] = acc;
            acc += c;
        }
        tot[j] = acc;
    }
    // tile-local digit starts: an exclusive scan over the digits in order,
    // digits [0, 512) in thread order, then [512, 1024) after all of them
    uint32_t incl[RADIX_THREAD_BINS];
#pragma unroll
    for (int j = 0; j < RADIX_THREAD_BINS; ++j) {
        incl[j] = warp_incl_scan(tot[j], lane);
        if (lane == 31) sm.wsum[j][warp] = incl[j];
    }
#pragma unroll
    for (int r = 0; r < RADIX_ROUNDS; ++r) {
        const uint64_t idx = base + (uint64_t)r * 32 + lane;
        v[r] = idx < n ? vals[idx] : 0u;
    }
    __syncthreads();
    uint32_t carry = 0;
#pragma unroll
    for (int j = 0; j < RADIX_THREAD_BINS; ++j) {
        uint32_t before = carry + incl[j] - tot[j];
#pragma unroll
        for (int w = 0; w < RADIX_WARPS; ++w) {
            const uint32_t ws = sm.wsum[j][w];
            if (w < warp) before += ws;
            carry += ws;
        }
        const uint32_t d = threadIdx.x + j * RADIX_THREADS;
        sm.start[d] = before;
        sm.gpos[d] = d < bins ? tile_off[(uint64_t)d * tiles + blockIdx.x] : 0u;
    }
    __syncthreads();
    // tile-local sorted position of every item (registers), then the tile in
    // digit order over the (now free) counts
#pragma unroll
    for (int r = 0; r < RADIX_ROUNDS; ++r) {  // rank becomes the tile-local position
        const uint64_t idx = base + (uint64_t)r * 32 + lane;
        const uint32_t d = (k[r] >> shift) & mask;
        rank[r] = idx < n ? sm.start[d] + sm.u.whist[warp][d] + rank[r] : 0xFFFFFFFFu;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RADIX_ROUNDS; ++r) {
        if (rank[r] != 0xFFFFFFFFu) {
            sm.u.tile.k[rank[r]] = k[r];
            sm.u.tile.v[rank[r]] = v[r];
        }
    }
    __syncthreads();
    const uint32_t in_tile = n - tile_base < RADIX_TILE ? (uint32_t)(n - tile_base) : RADIX_TILE;
    for (uint32_t i = threadIdx.x; i < in_tile; i += RADIX_THREADS) {
        const uint32_t key = sm.u.tile.k[i];
        const uint32_t d = (key >> shift) & mask;
        const uint32_t pos = sm.gpos[d] + (i - sm.start[d]);
        if (keys_out) keys_out[pos] = key;
        vals_out[pos] = sm.u.tile.v[i];
    }
}

// ---- index and signatures --------------------------------------------------
__global__ void k_prefix_len(CollView c, const uint32_t* __restrict__ tab, uint32_t lo, uint32_t hi,
                             uint32_t* out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; lo + i < hi; i += gridDim.x * blockDim.x)
        out[i] = tab[c.sizes[lo + i]];
}

// One warp per set: the first len tokens become entries (token, set, position).
__global__ void k_emit_entries(CollView c, uint32_t lo, uint32_t hi, const uint32_t* __restrict__ off,
                               const uint32_t* __restrict__ len, uint32_t* e_token, uint32_t* e_set,
                               uint32_t* e_pos) {
    const int lane = threadIdx.x & 31;
    uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; lo + w < hi; w += warps) {
        uint32_t s = lo + w, l = len[w], o = off[w];
        const uint32_t* t = c.tokens + c.starts[s];
        for (uint32_t i = lane; i < l; i += 32) {
            e_token[o + i] = t[i];
            e_set[o + i] = s;
            e_pos[o + i] = i;
        }
    }
}

// (token, (set << pos_bits) | position) for the first len tokens of every set,
// and the token histogram (one atomic per entry).  A warp takes 32 consecutive
// sets: their entries are contiguous in the output (off is the scan of len),
// so the warp walks them flattened, 32 entries per round, each lane finding
// its set from one ballot (the sets ending before the round) and one OR of the
// positions where sets start inside the round.  Every lane
// carries an entry in every round (prefixes are far shorter than 32), the
// stores coalesce, and the token loads of EMIT_ROUNDS (8) rounds are issued before
// any of their stores.  Sets [lo, c.n): c, off and len are indexed by absolute
// set id.  counts may be nullptr (no histogram).
// REC: instead of the entry arrays, each entry goes straight into its token's
// record (the histogram atomic returns its slot; tokens at or above `limit`
// and slots past REC_ENTRIES are dropped); len is then the prefix-length table
// indexed by set size and off is not read.
constexpr int EMIT_ROUNDS = 8;
#ifndef HS_REC_EMIT_ROUNDS
#define HS_REC_EMIT_ROUNDS 4  // rounds of slot atomics in flight per lane (record emit)
#endif
#ifndef HS_REC_EMIT_MINB
#define HS_REC_EMIT_MINB 6  // resident blocks per SM the record emit is compiled for
#endif
template <bool REC>
__global__ void __launch_bounds__(256, REC ? HS_REC_EMIT_MINB : 1) k_emit_packed(CollView c, uint32_t lo, const uint32_t* __restrict__ off,
                              const uint32_t* __restrict__ len, uint32_t pos_bits, uint32_t* __restrict__ e_token,
                              uint32_t* __restrict__ e_val, uint32_t* __restrict__ counts, uint32_t limit,
                              BoundFields bf, uint32_t spw) {
    constexpr int ROUNDS = REC ? HS_REC_EMIT_ROUNDS : EMIT_ROUNDS;
    const uint32_t maxf = (1u << pos_bits) - 1u;
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t s0 = lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * spw; s0 < c.n; s0 += warps * spw) {
        const uint32_t s = s0 + lane;
        const bool has = (uint32_t)lane < spw && s < c.n;
        uint32_t l, start, o0 = 0, size = 0;
        if constexpr (REC) {  // len is the prefix table by size; no offsets
            const uint2 m = has ? c.meta[s] : make_uint2(0, 0);
            l = has ? len[m.y] : 0u;
            start = m.x;
            size = m.y;
        } else {
            l = has ? len[s] : 0u;
            start = has ? c.meta[s].x : 0u;
            o0 = __shfl_sync(FULL, has ? off[s] : 0u, 0);
        }
        const uint32_t incl = warp_incl_scan(l, lane);
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        for (uint32_t j0 = 0; j0 < total; j0 += 32 * ROUNDS) {
            uint32_t tok[ROUNDS], val[ROUNDS];
#pragma unroll
            for (int u = 0; u < ROUNDS; ++u) {
                const uint32_t j = j0 + 32u * u + lane;
                // the set of the round's first entry r0 (sets ending at or before
                // r0 come first), plus the sets that start inside the round up to j
                const uint32_t r0 = j0 + 32u * u, excl = incl - l;
                const int kf = __popc(__ballot_sync(FULL, incl <= r0));
                const uint32_t starts =
                    __reduce_or_sync(FULL, (l && excl > r0 && excl < r0 + 32u) ? 1u << (excl - r0) : 0u);
                const int k = (kf + __popc(starts & ((2u << lane) - 1u))) & 31;
                const uint32_t excl_k = __shfl_sync(FULL, excl, k);
                const uint32_t start_k = __shfl_sync(FULL, start, k);
                const uint32_t i = j - excl_k;
                tok[u] = j < total ? __ldg(c.tokens + start_k + i) : 0u;
                uint32_t low = i;
                if constexpr (REC) {
                    const uint32_t size_k = __shfl_sync(FULL, size, k);
                    if (bf.on() && j < total) low = bound_field_of(bf, size_k, i, maxf);
                }
                val[u] = ((s0 + (uint32_t)k) << pos_bits) | low;
            }
            if constexpr (REC) {
                // every round's slot atomic is in flight before the first store
                uint32_t slot[ROUNDS];
#pragma unroll
                for (int u = 0; u < ROUNDS; ++u) {
                    const uint32_t j = j0 + 32u * u + lane;
                    slot[u] = j < total && tok[u] < limit ? atomicAdd(&counts[tok[u]], 1u) : 0xFFFFFFFFu;
                }
#pragma unroll
                for (int u = 0; u < ROUNDS; ++u)
                    if (slot[u] < REC_ENTRIES) e_val[(uint64_t)tok[u] * REC_CAP + 1 + slot[u]] = val[u];
                continue;
            }
#pragma unroll
            for (int u = 0; u < ROUNDS; ++u) {
                const uint32_t j = j0 + 32u * u + lane;
                if (j < total) {
                    e_token[o0 + j] = tok[u];
                    e_val[o0 + j] = val[u];
                    // tokens inside one set are distinct: one atomic per entry
                    if (counts && tok[u] < limit) atomicAdd(&counts[tok[u]], 1u);
                }
            }
        }
    }
}

// gate = the longest list: the maximum of the per-token counts of tokens
// below U, reduced per block (one atomic per block on the single word; the
// caller zeroes it).
__global__ void k_list_max(const uint32_t* __restrict__ counts, uint32_t U, uint32_t* gate) {
    __shared__ uint32_t wm[32];
    uint32_t m = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < U; t += stride) m = max(m, counts[t]);
    m = __reduce_max_sync(FULL, m);
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? wm[threadIdx.x] : 0u;
        m = __reduce_max_sync(FULL, m);
        if (threadIdx.x == 0 && m) atomicMax(gate, m);
    }
}

// Short-list index build, step 1 (runs when every list is short): each entry
// (token t, value v) takes the next slot of list t from an atomic on the
// list's cursor (initialised to the list offsets), so each list holds its
// entries in arbitrary order.  Tokens at or above U are left out (the counts
// did not count them).
constexpr int SCATTER_ITEMS = 8;  // entries per thread per step: eight atomics in flight
__global__ void k_list_scatter(const uint32_t* __restrict__ tok, const uint32_t* __restrict__ val, uint64_t n,
                               uint32_t U, uint32_t* __restrict__ cursor, uint32_t* __restrict__ out,
                               const uint32_t* gate, bool vec) {
    if (gate && *gate > LIST_SHORT) return;  // gate == nullptr: run
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * SCATTER_ITEMS;
    for (uint64_t i0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * SCATTER_ITEMS; i0 < n; i0 += stride) {
        uint32_t t[SCATTER_ITEMS], v[SCATTER_ITEMS], at[SCATTER_ITEMS];
        if (SCATTER_ITEMS % 4 == 0 && vec && i0 + SCATTER_ITEMS <= n) {  // 16-byte loads (both arrays aligned)
#pragma unroll
            for (int q = 0; q < SCATTER_ITEMS / 4; ++q) {
                const uint4 tt = *reinterpret_cast<const uint4*>(tok + i0 + 4 * q);
                const uint4 vv = *reinterpret_cast<const uint4*>(val + i0 + 4 * q);
                t[4 * q] = tt.x, t[4 * q + 1] = tt.y, t[4 * q + 2] = tt.z, t[4 * q + 3] = tt.w;
                v[4 * q] = vv.x, v[4 * q + 1] = vv.y, v[4 * q + 2] = vv.z, v[4 * q + 3] = vv.w;
            }
        } else {
#pragma unroll
            for (int u = 0; u < SCATTER_ITEMS; ++u) {
                t[u] = i0 + u < n ? tok[i0 + u] : 0xFFFFFFFFu;
                v[u] = i0 + u < n ? val[i0 + u] : 0u;
            }
        }
#pragma unroll
        for (int u = 0; u < SCATTER_ITEMS; ++u) at[u] = t[u] < U ? atomicAdd(&cursor[t[u]], 1u) : 0xFFFFFFFFu;
#pragma unroll
        for (int u = 0; u < SCATTER_ITEMS; ++u)
            if (at[u] != 0xFFFFFFFFu) out[at[u]] = v[u];
    }
}

// Step 2: a warp orders 32 consecutive lists.  Their entries are contiguous;
// the warp stages them in shared memory, lane k orders list k there by
// insertion sort (the scatter leaves lists nearly in emission order, since
// earlier entries mostly take their slots first, so this is close to one pass
// per list), and the warp writes the range back with coalesced stores.  When
// the 32 lists overflow the stage they go as two halves of 16 (16 lists of at
// most LIST_SHORT entries always fit); a half that still overflows (lists
// longer than LIST_SHORT) is sorted in place in global memory, a lane per list.
__device__ __forceinline__ void order_lists(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                            uint32_t* stage, uint32_t ls, uint32_t le, int k0, int k1, int lane) {
    const uint32_t a = __shfl_sync(FULL, ls, k0), b = __shfl_sync(FULL, le, k1 - 1), m = b - a;
    const bool mine = lane >= k0 && lane < k1;
    if (m <= RANK_CAP) {
        for (uint32_t j0 = 0; j0 < m; j0 += 256) {  // eight loads in flight per lane
            uint32_t x[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t j = j0 + 32u * u + lane;
                x[u] = j < m ? in[a + j] : 0u;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t j = j0 + 32u * u + lane;
                if (j < m) stage[j] = x[u];
            }
        }
        __syncwarp();
        if (mine) {
            const uint32_t lo = ls - a, hi = le - a;
            for (uint32_t i = lo + 1; i < hi; ++i) {
                const uint32_t x = stage[i];
                uint32_t j = i;
                for (; j > lo; --j) {
                    const uint32_t y = stage[j - 1];
                    if (y < x) break;
                    stage[j] = y;
                }
                stage[j] = x;
            }
        }
        __syncwarp();
        for (uint32_t j = lane; j < m; j += 32) out[a + j] = stage[j];
        __syncwarp();
    } else if (mine) {
        for (uint32_t i = ls; i < le; ++i) out[i] = in[i];
        for (uint32_t i = ls + 1; i < le; ++i) {
            const uint32_t x = out[i];
            uint32_t j = i;
            for (; j > ls; --j) {
                const uint32_t y = out[j - 1];
                if (y < x) break;
                out[j] = y;
            }
            out[j] = x;
        }
    }
}

__global__ void __launch_bounds__(RANK_THREADS) k_list_rank(const uint32_t* __restrict__ list_off, uint32_t U,
                                                           const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                           const uint32_t* gate) {
    if (gate && *gate > LIST_SHORT) return;  // gate == nullptr: run
    __shared__ uint32_t stage_all[RANK_THREADS / 32][RANK_CAP];
    const int lane = threadIdx.x & 31;
    uint32_t* stage = stage_all[threadIdx.x >> 5];
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint64_t t0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5 << 5; t0 < U; t0 += (uint64_t)warps * 32) {
        const uint64_t t = t0 + lane;
        const uint32_t ls = list_off[t < U ? t : U];
        const uint32_t le = list_off[t + 1 < U ? t + 1 : U];
        const uint32_t a = __shfl_sync(FULL, ls, 0), b = __shfl_sync(FULL, le, 31);
        if (b - a <= RANK_CAP) {
            order_lists(in, out, stage, ls, le, 0, 32, lane);
        } else {
            order_lists(in, out, stage, ls, le, 0, 16, lane);
            order_lists(in, out, stage, ls, le, 16, 32, lane);
        }
    }
}

// Orders the token records: a warp takes 32 consecutive records, stages in
// shared memory (a record per 33 words, so the lanes' sorts hit distinct
// banks) the 16-byte quarters that hold its length word and entries, lane k
// sorts record k by insertion (the atomic slots mostly follow emission order,
// which is set order), pads it and writes its length word, and the warp
// stores back every 32-byte piece a probe reads for that length (the piece
// holding word 0 and as many more as the entries reach; see record_window).
// Pieces past them are neither read nor written.
constexpr int REC_THREADS = 256;
__host__ __device__ constexpr uint32_t record_pieces(uint32_t n) { return n > 7u ? 1u + (n - 7u + 7u) / 8u : 1u; }
__global__ void __launch_bounds__(REC_THREADS) k_order_records(const uint32_t* __restrict__ counts, uint32_t U,
                                                               uint32_t* __restrict__ rec, uint32_t* overflow,
                                                               uint32_t* __restrict__ prev) {
    __shared__ uint32_t stage_all[REC_THREADS / 32][32 * 33];
    const int lane = threadIdx.x & 31;
    uint32_t* stage = stage_all[threadIdx.x >> 5];
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint64_t t0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5 << 5; t0 < U;
         t0 += (uint64_t)warps * 32) {
        const uint32_t nrec = U - t0 < 32 ? (uint32_t)(U - t0) : 32u;
        const uint32_t cnt = (uint32_t)lane < nrec ? counts[t0 + lane] : 0u;
        if (prev) {  // incremental pass: only groups with new entries
            const bool changed = (uint32_t)lane < nrec && prev[t0 + lane] != cnt;
            if (!__any_sync(FULL, changed)) continue;
            if (changed) prev[t0 + lane] = cnt;
        }
        if (overflow && __any_sync(FULL, cnt > REC_ENTRIES) && lane == 0) atomicOr(overflow, REC_OVERFLOW);
        const uint32_t mine = min(cnt, REC_ENTRIES);
        uint4* g = reinterpret_cast<uint4*>(rec + t0 * REC_CAP);
        // quarter k: record k / 8, words 4 (k % 8) .. +3; read if it holds the length or an entry
#pragma unroll
        for (uint32_t it = 0; it < 8; ++it) {  // every lane takes every round: the shuffles stay converged
            const uint32_t k = (uint32_t)lane + 32u * it;
            const uint32_t n = __shfl_sync(FULL, mine, k >> 3);
            if (k < nrec * 8 && 4 * (k & 7) < n + 1) {
                const uint4 x = g[k];
                uint32_t* d = stage + (k >> 3) * 33 + (k & 7) * 4;
                d[0] = x.x, d[1] = x.y, d[2] = x.z, d[3] = x.w;
            }
        }
        __syncwarp();
        if ((uint32_t)lane < nrec) {
            uint32_t* r = stage + lane * 33 + 1;  // the entries follow the length word
            const uint32_t n = mine;
            for (uint32_t i = 1; i < n; ++i) {
                const uint32_t x = r[i];
                uint32_t j = i;
                for (; j > 0; --j) {
                    const uint32_t y = r[j - 1];
                    if (y < x) break;
                    r[j] = y;
                }
                r[j] = x;
            }
            for (uint32_t i = n; i < 8 * record_pieces(n) - 1; ++i) r[i] = 0xFFFFFFFFu;
            r[-1] = n;
        }
        __syncwarp();
#pragma unroll
        for (uint32_t it = 0; it < 8; ++it) {
            const uint32_t k = (uint32_t)lane + 32u * it;
            const uint32_t n = __shfl_sync(FULL, mine, k >> 3);
            if (k < nrec * 8 && 4 * (k & 7) < 8 * record_pieces(n)) {
                const uint32_t* d = stage + (k >> 3) * 33 + (k & 7) * 4;
                g[k] = make_uint4(d[0], d[1], d[2], d[3]);
            }
        }
        __syncwarp();
    }
}

// Records from built lists: a warp per token, lane 0 writes the length, lane
// i > 0 entry i - 1 or the pad.
__global__ void k_records_from_lists(const uint32_t* __restrict__ list_off, const uint32_t* __restrict__ vals,
                                     uint32_t U, uint32_t* __restrict__ rec, BoundFields bf,
                                     const uint32_t* __restrict__ sizes, uint32_t list_bits, uint32_t rec_bits) {
    const int lane = threadIdx.x & 31;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t t = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < U; t += warps) {
        const uint32_t a = list_off[t], b = list_off[t + 1];
        uint32_t w = lane == 0 ? b - a : (a + lane - 1 < b ? vals[a + lane - 1] : 0xFFFFFFFFu);
        if (bf.on() && lane > 0 && a + lane - 1 < b) {  // (set, position) -> (set, bound field)
            const uint32_t set = w >> list_bits, pos = w & ((1u << list_bits) - 1u);
            w = (set << rec_bits) | bound_field_of(bf, sizes[set], pos, (1u << rec_bits) - 1u);
        }
        rec[t * REC_CAP + lane] = w;
    }
}

// counts has `limit` entries; tokens at or above it are not counted.
__global__ void k_histogram(const uint32_t* __restrict__ tok, uint64_t n, uint32_t* counts, uint32_t limit) {
    const int lane = threadIdx.x & 31;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        uint64_t i = i0 + threadIdx.x;
        bool valid = i < n;
        uint32_t t = valid ? tok[i] : 0xFFFFFFFFu;
        unsigned peers = __match_any_sync(FULL, t);
        if (valid && t < limit && lane == __ffs(peers) - 1) atomicAdd(&counts[t], (uint32_t)__popc(peers));
    }
}

__global__ void k_scatter(const uint32_t* __restrict__ tok, const uint32_t* __restrict__ eset,
                          const uint32_t* __restrict__ epos, uint64_t n, uint32_t* cursor, uint32_t* idx_set,
                          uint32_t* idx_pos) {
    const int lane = threadIdx.x & 31;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        uint64_t i = i0 + threadIdx.x;
        bool valid = i < n;
        uint32_t t = valid ? tok[i] : 0xFFFFFFFFu;
        unsigned peers = __match_any_sync(FULL, t);
        int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (valid && lane == leader) base = atomicAdd(&cursor[t], (uint32_t)__popc(peers));
        base = __shfl_sync(FULL, base, leader);
        if (valid) {
            uint32_t at = base + __popc(peers & lanemask_lt(lane));
            idx_set[at] = eset[i];
            idx_pos[at] = epos[i];
        }
    }
}

__global__ void k_gather(const uint32_t* __restrict__ order, uint64_t n, const uint32_t* __restrict__ eset,
                         const uint32_t* __restrict__ epos, uint32_t* idx_set, uint32_t* idx_pos) {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint32_t e = order[i];
        idx_set[i] = eset[e];
        idx_pos[i] = epos[e];
    }
}

__global__ void k_iota(uint32_t* out, uint64_t n) {
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) out[i] = (uint32_t)i;
}

// Eight lanes per set (four sets per warp).  The group's 2W 32-bit signature
// words live in shared memory; every token flips its bit there with one
// shared-memory XOR (a register fold would cost a compare and select per word
// per token), four token loads in flight per lane; the group's lanes then
// store the words (coalesced).  Bit b of the signature is bit b%32 of 32-bit
// word b/32 (the popcount of a XOR of two signatures does not depend on the
// bit layout).
constexpr int BITMAP_THREADS = 256;
constexpr int BITMAP_UNROLL = 4;
template <int W>
__global__ void __launch_bounds__(BITMAP_THREADS) k_bitmaps(CollView c, uint64_t* out) {
    constexpr int NW = 2 * W;
    __shared__ uint32_t sw[BITMAP_THREADS / 8][NW];
    const int lane = threadIdx.x & 31, g = lane & 7;
    uint32_t* mine = sw[threadIdx.x >> 3];
    const uint32_t mask = 64u * W - 1u;
    const uint32_t groups = (gridDim.x * blockDim.x) >> 3;
    uint32_t* out32 = reinterpret_cast<uint32_t*>(out);
    // every lane iterates the same number of times so the warp barriers match
    const uint32_t rounds = (c.n + groups - 1) / groups;
    uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    for (uint32_t r = 0; r < rounds; ++r, s += groups) {
#pragma unroll
        for (int q = g; q < NW; q += 8) mine[q] = 0u;
        __syncwarp();
        const bool live = s < c.n;
        uint2 m = make_uint2(0, 0);
        if (live) m = c.meta[s];
        const uint32_t* t = c.tokens + m.x;
        for (uint32_t i0 = g; i0 < m.y; i0 += 8 * BITMAP_UNROLL) {
            uint32_t tok[BITMAP_UNROLL];
#pragma unroll
            for (int u = 0; u < BITMAP_UNROLL; ++u) {
                const uint32_t i = i0 + 8u * u;
                tok[u] = i < m.y ? __ldg(t + i) : 0xFFFFFFFFu;
            }
#pragma unroll
            for (int u = 0; u < BITMAP_UNROLL; ++u) {
                if (i0 + 8u * u < m.y) {
                    const uint32_t b = tok[u] & mask;
                    atomicXor(&mine[b >> 5], 1u << (b & 31));
                }
            }
        }
        __syncwarp();
        if (live) {
#pragma unroll
            for (int q = g; q < NW; q += 8) out32[(uint64_t)s * NW + q] = mine[q];
        }
        __syncwarp();
    }
}

// The checks of k_validate and the signatures of k_bitmaps in one pass over
// the tokens of the sets of c (LPS lanes per set: eight as k_bitmaps, or a
// warp for parts of long sets, which would otherwise leave most SMs idle):
// the set's meta pair is written from its start and size, and its tokens are
// read once for both (the order check reads each token's successor, an L1
// hit).
template <int W, int LPS>
__global__ void __launch_bounds__(BITMAP_THREADS) k_validate_bitmaps(CollView c, uint64_t n_tokens, uint32_t* flags,
                                                                    uint2* meta, uint64_t* out) {
    static_assert(LPS == 8 || LPS == 32, "lanes per set");
    constexpr int NW = 2 * W;
    constexpr int SH = LPS == 8 ? 3 : 5;
    __shared__ uint32_t sw[BITMAP_THREADS / LPS][NW];
    const int lane = threadIdx.x & 31, g = lane & (LPS - 1);
    uint32_t* mine = sw[threadIdx.x >> SH];
    const uint32_t mask = 64u * W - 1u;
    const uint32_t groups = (gridDim.x * blockDim.x) >> SH;
    uint32_t* out32 = reinterpret_cast<uint32_t*>(out);
    uint32_t f = 0, mx = 0;
    const uint32_t rounds = (c.n + groups - 1) / groups;  // the same for every lane: the warp barriers match
    uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> SH;
    for (uint32_t r = 0; r < rounds; ++r, s += groups) {
#pragma unroll
        for (int q = g; q < NW; q += LPS) mine[q] = 0u;
        __syncwarp();
        const bool live = s < c.n;
        uint32_t st = 0, l = 0;
        if (live) {
            st = c.starts[s];
            l = c.sizes[s];
            if (g == 0) meta[s] = make_uint2(st, l);
            if (l == 0) f |= 1;
            if (s > 0 && c.sizes[s - 1] > l) f |= 4;
            if ((uint64_t)st + l > n_tokens) {
                f |= 8;
                l = 0;
            } else if (l > 0 && g == 0) {
                mx = max(mx, c.tokens[st + l - 1]);
            }
        }
        const uint32_t* t = c.tokens + st;
        for (uint32_t i0 = g; i0 < l; i0 += LPS * BITMAP_UNROLL) {
            uint32_t tok[BITMAP_UNROLL], nxt[BITMAP_UNROLL];
#pragma unroll
            for (int u = 0; u < BITMAP_UNROLL; ++u) {
                const uint32_t i = i0 + (uint32_t)LPS * u;
                tok[u] = i < l ? __ldg(t + i) : 0xFFFFFFFFu;
                nxt[u] = i + 1 < l ? __ldg(t + i + 1) : 0xFFFFFFFFu;
            }
#pragma unroll
            for (int u = 0; u < BITMAP_UNROLL; ++u) {
                const uint32_t i = i0 + (uint32_t)LPS * u;
                if (i < l) {
                    if (i + 1 < l && tok[u] >= nxt[u]) f |= 2;
                    const uint32_t b = tok[u] & mask;
                    atomicXor(&mine[b >> 5], 1u << (b & 31));
                }
            }
        }
        __syncwarp();
        if (live) {
#pragma unroll
            for (int q = g; q < NW; q += LPS) out32[(uint64_t)s * NW + q] = mine[q];
        }
        __syncwarp();
    }
    f = __reduce_or_sync(FULL, f);
    mx = __reduce_max_sync(FULL, mx);
    if (lane == 0) {
        if (f) atomicOr(&flags[0], f);
        atomicMax(&flags[1], mx);
    }
}

// One warp per set: checks the input contract and writes the set's (start,
// size) pair.  The largest token is kept per lane and reduced once per warp, so
// the kernel makes one atomic per warp, not one per set.
__global__ void k_validate(CollView c, uint64_t n_tokens, uint32_t* flags, uint2* meta) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t f = 0, mx = 0;
    for (uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < c.n; s += warps) {
        const uint32_t l = c.sizes[s], st = c.starts[s];
        if (lane == 0) meta[s] = make_uint2(st, l);
        if (l == 0) f |= 1;
        if (s > 0 && c.sizes[s - 1] > l) f |= 4;
        if ((uint64_t)st + l > n_tokens) {
            f |= 8;
        } else if (l > 0) {
            const uint32_t* t = c.tokens + st;
            for (uint32_t i = lane; i + 1 < l; i += 32)
                if (t[i] >= t[i + 1]) f |= 2;
            if (lane == 0) mx = max(mx, t[l - 1]);
        }
    }
    f = __reduce_or_sync(FULL, f);
    mx = __reduce_max_sync(FULL, mx);
    if (lane == 0) {
        if (f) atomicOr(&flags[0], f);
        atomicMax(&flags[1], mx);
    }
}

unsigned grid_for(uint64_t n, unsigned threads, unsigned cap = 152u * 32u) {
    uint64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

}  // namespace

size_t scan_scratch_words(uint64_t n) {
    size_t words = 0;
    while (n > SCAN_TILE) {
        n = (n + SCAN_TILE - 1) / SCAN_TILE;
        words += n;
    }
    return words + 1;
}

cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* scratch, cudaStream_t s,
                           const uint32_t* gate) {
    if (n == 0) return cudaSuccess;
    if (n <= SCAN_TILE) {
        note_launches();
        k_tile_scan<<<1, SCAN_THREADS, 0, s>>>(in, out, n, nullptr, gate);
        return cudaGetLastError();
    }
    uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    uint32_t* sums = scratch;
    note_launches(2);
    k_tile_reduce<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n, sums, gate);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = scan_exclusive(sums, sums, tiles, scratch + tiles, s, gate);
    if (e != cudaSuccess) return e;
    k_tile_scan<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, out, n, sums, gate);
    return cudaGetLastError();
}

size_t radix_scratch_words(uint64_t n) {
    uint64_t tiles = (n + RADIX_TILE - 1) / RADIX_TILE;
    uint64_t counts = tiles * RADIX_BINS;
    return counts + scan_scratch_words(counts);
}

cudaError_t prepare_kernels() {
    // the downsweep's per-warp digit counts need more than the default 48 KB
    return cudaFuncSetAttribute(k_radix_downsweep, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sizeof(RadixSmem));
}

namespace {
__global__ void k_copy_gated(uint32_t* dst, const uint32_t* __restrict__ src, uint64_t n, const uint32_t* gate) {
    if (gated_off(gate)) return;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = src[i];
}
}  // namespace

cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* alt_keys, uint32_t* alt_vals, uint64_t n,
                             int key_bits, uint32_t* scratch, cudaStream_t s, bool keep_keys, const uint32_t* gate) {
    if (n <= 1) return cudaSuccess;
    uint32_t tiles = (uint32_t)((n + RADIX_TILE - 1) / RADIX_TILE);
    int passes = (key_bits + RADIX_MAX_BITS - 1) / RADIX_MAX_BITS;
    if (passes < 1) passes = 1;
    const int digit = (key_bits + passes - 1) / passes;
    uint32_t *kin = keys, *vin = vals, *kout = alt_keys, *vout = alt_vals;
    for (int p = 0; p < passes; ++p) {
        const int shift = digit * p;
        const int width = std::min(digit, key_bits - shift);
        const uint32_t mask = (1u << width) - 1u;
        const uint64_t counts = (uint64_t)tiles * (mask + 1);
        uint32_t* tile_counts = scratch;
        uint32_t* scan_tmp = scratch + counts;
        note_launches(2);
        k_radix_upsweep<<<tiles, RADIX_THREADS, 0, s>>>(kin, n, shift, mask, tile_counts, tiles, gate);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        e = scan_exclusive(tile_counts, tile_counts, counts, scan_tmp, s, gate);
        if (e != cudaSuccess) return e;
        const bool last = p + 1 == passes;
        k_radix_downsweep<<<tiles, RADIX_THREADS, sizeof(RadixSmem), s>>>(
            kin, vin, n, shift, mask, tile_counts, tiles, last && !keep_keys ? nullptr : kout, vout, gate);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        uint32_t* t;
        t = kin; kin = kout; kout = t;
        t = vin; vin = vout; vout = t;
    }
    if (vin != vals) {
        if (gate) {  // the copy back obeys the gate too
            note_launches(keep_keys ? 2 : 1);
            if (keep_keys) k_copy_gated<<<grid_for(n, 256), 256, 0, s>>>(keys, kin, n, gate);
            k_copy_gated<<<grid_for(n, 256), 256, 0, s>>>(vals, vin, n, gate);
            return cudaGetLastError();
        }
        cudaError_t e = keep_keys ? cudaMemcpyAsync(keys, kin, n * 4, cudaMemcpyDeviceToDevice, s) : cudaSuccess;
        if (e != cudaSuccess) return e;
        e = cudaMemcpyAsync(vals, vin, n * 4, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t set_prefix_lengths(CollView c, const uint32_t* prefix_tab, uint32_t lo, uint32_t hi, uint32_t* out_len,
                               cudaStream_t s) {
    if (hi <= lo) return cudaSuccess;
    note_launches();
    k_prefix_len<<<grid_for(hi - lo, 256), 256, 0, s>>>(c, prefix_tab, lo, hi, out_len);
    return cudaGetLastError();
}

cudaError_t emit_prefix_entries(CollView c, uint32_t lo, uint32_t hi, const uint32_t* entry_off, const uint32_t* len,
                                uint32_t* e_token, uint32_t* e_set, uint32_t* e_pos, cudaStream_t s) {
    if (hi <= lo) return cudaSuccess;
    note_launches();
    k_emit_entries<<<grid_for((uint64_t)(hi - lo) * 32, 256), 256, 0, s>>>(c, lo, hi, entry_off, len, e_token,
                                                                            e_set, e_pos);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) k_size_scan(const uint32_t* __restrict__ sizes,
                                                   const uint32_t* __restrict__ starts, int starts_given, uint32_t n,
                                                   uint32_t L, uint64_t n_tokens, uint32_t* out,
                                                   uint32_t* __restrict__ first_ge, uint32_t* __restrict__ chunk_hi) {
    __shared__ uint64_t ends[PIPE_MAX_CHUNKS];
    __shared__ uint32_t n_ends;
    __shared__ uint32_t bflags;
    __shared__ unsigned long long bsum;
    if (threadIdx.x == 0) {  // the copy schedule, as the host makes it
        uint32_t k = 0;
        for (uint64_t t = 0; t < n_tokens && k < PIPE_MAX_CHUNKS;) {
            t += pipe_chunk(n_tokens - t);
            ends[k++] = t;
        }
        n_ends = k;
        bflags = 0;
        bsum = 0;
    }
    __syncthreads();
    uint32_t flags = 0;
    unsigned long long sum = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += stride) {
        // first_ge[l] = i for l in (sizes[i-1], sizes[i]] (from 0 for i = 0; up to L + 1 for i = n)
        const uint32_t lo = i == 0 ? 0u : min(sizes[i - 1], L + 1u) + 1u;
        const uint32_t hi = i == n ? L + 1u : min(sizes[i], L + 1u);
        for (uint32_t l = lo; l <= hi; ++l) first_ge[l] = i;
        if (i == n) continue;
        const uint32_t z = sizes[i];
        sum += z;
        if (i > 0 && z < sizes[i - 1]) flags |= 1u;
        if (starts_given && starts[i] != (i ? starts[i - 1] + sizes[i - 1] : 0u)) flags |= 2u;
        // the chunks whose end lies in [end of set i - 1, end of set i): set i is the first to end past them
        const uint64_t e1 = (uint64_t)starts[i] + z, e0 = i ? (uint64_t)starts[i - 1] + sizes[i - 1] : 0ull;
        uint32_t a = 0, b = n_ends;  // first chunk with end >= e0
        while (a < b) {
            const uint32_t m = (a + b) >> 1;
            if (ends[m] < e0) a = m + 1;
            else b = m;
        }
        for (uint32_t k = a; k < n_ends && ends[k] < e1; ++k) chunk_hi[k] = i;
    }
    if (flags) atomicOr(&bflags, flags);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(FULL, sum, o);
    if ((threadIdx.x & 31) == 0 && sum) atomicAdd(&bsum, sum);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (bflags) atomicOr(out, bflags);
        if (bsum) atomicAdd(reinterpret_cast<unsigned long long*>(out + 2), bsum);
    }
}

cudaError_t size_scan(const uint32_t* sizes, const uint32_t* starts, bool starts_given, uint32_t n, uint32_t L,
                      uint64_t n_tokens, uint32_t* out, uint32_t* first_ge, uint32_t* chunk_hi, cudaStream_t s) {
    note_launches();
    k_size_scan<<<grid_for((uint64_t)n + 1, 256, 152u * 8u), 256, 0, s>>>(sizes, starts, starts_given ? 1 : 0, n, L,
                                                                        n_tokens, out, first_ge, chunk_hi);
    return cudaGetLastError();
}

namespace {
// Sets [lo, hi) in two launches: below big_lo a warp per 32 sets, from big_lo
// on (the sets with long prefixes) a warp per set, so that no warp walks 32
// long prefixes alone while the others have finished.
template <bool REC>
cudaError_t launch_emit(CollView c, uint32_t lo, uint32_t hi, uint32_t big_lo, const uint32_t* off,
                        const uint32_t* len, uint32_t pos_bits, uint32_t* e_token, uint32_t* e_val, uint32_t* counts,
                        uint32_t limit, BoundFields bf, cudaStream_t s) {
    if (hi == 0xFFFFFFFFu) hi = c.n;
    const uint32_t mid = std::min(std::max(lo, big_lo), hi);
    CollView v = c;
    if (mid > lo) {
        note_launches();
        v.n = mid;  // the kernel walks ids [lo, mid)
        k_emit_packed<REC><<<grid_for((uint64_t)(mid - lo), 256), 256, 0, s>>>(v, lo, off, len, pos_bits, e_token,
                                                                             e_val, counts, limit, bf, 32u);
    }
    if (hi > mid) {
        note_launches();
        v.n = hi;
        k_emit_packed<REC><<<grid_for((uint64_t)(hi - mid) * 32u, 256), 256, 0, s>>>(v, mid, off, len, pos_bits,
                                                                                   e_token, e_val, counts, limit,
                                                                                   bf, 1u);
    }
    return cudaGetLastError();
}
}  // namespace

cudaError_t emit_packed_entries(CollView c, const uint32_t* entry_off, const uint32_t* len, uint32_t pos_bits,
                                uint32_t* e_token, uint32_t* e_val, uint32_t* counts, cudaStream_t s, uint32_t lo,
                                uint32_t hi, uint32_t limit, uint32_t big_lo) {
    return launch_emit<false>(c, lo, hi, big_lo, entry_off, len, pos_bits, e_token, e_val, counts, limit,
                              BoundFields{}, s);
}

cudaError_t emit_records(CollView c, const uint32_t* prefix_tab, uint32_t pos_bits, uint32_t* counts, uint32_t* rec,
                         uint32_t limit, cudaStream_t s, uint32_t lo, uint32_t hi, BoundFields bf,
                         uint32_t big_lo) {
    return launch_emit<true>(c, lo, hi, big_lo, nullptr, prefix_tab, pos_bits, nullptr, rec, counts, limit, bf, s);
}

cudaError_t order_records(const uint32_t* counts, uint32_t U, uint32_t* rec, cudaStream_t s, uint32_t* overflow,
                          uint32_t* prev) {
    if (U == 0) return cudaSuccess;
    note_launches();
    k_order_records<<<grid_for(((uint64_t)U + 31) / 32 * 32, REC_THREADS), REC_THREADS, 0, s>>>(counts, U, rec,
                                                                                              overflow, prev);
    return cudaGetLastError();
}

cudaError_t records_from_lists(const uint32_t* list_off, const uint32_t* vals, uint32_t U, uint32_t* rec,
                               cudaStream_t s, BoundFields bf, const uint32_t* sizes, uint32_t list_bits,
                               uint32_t rec_bits) {
    if (U == 0) return cudaSuccess;
    note_launches();
    k_records_from_lists<<<grid_for((uint64_t)U * 32, 256), 256, 0, s>>>(list_off, vals, U, rec, bf, sizes,
                                                                         list_bits, rec_bits);
    return cudaGetLastError();
}

cudaError_t index_lists(uint32_t* e_token, uint32_t* e_val, uint64_t n, uint32_t U, uint32_t* counts,
                        uint32_t* list_off, uint32_t* alt_keys, uint32_t* alt_vals, uint32_t* gate, int key_bits,
                        uint32_t* scratch, cudaStream_t s, int* path, uint32_t* h_gate) {
    cudaError_t e = scan_exclusive(counts, list_off, (uint64_t)U + 1, scratch, s);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    int p = path ? *path : 0;
    const uint32_t* g = nullptr;  // the kernels' device-side choice (p == 0 only)
    if (p == 0) {
        e = cudaMemsetAsync(gate, 0, 4, s);
        if (e != cudaSuccess) return e;
        note_launches();
        k_list_max<<<grid_for(U, 256, 4 * 152), 256, 0, s>>>(counts, U, gate);
        if (h_gate) {  // one host read settles the path for later builds
            e = cudaMemcpyAsync(h_gate, gate, 4, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return e;
            p = *h_gate <= LIST_SHORT ? 1 : 2;
            if (path) *path = p;
        } else {
            g = gate;
        }
    }
    if (p != 2) {
        // short lists: scatter into alt_vals (the counts become the cursors),
        // order back into e_val
        e = cudaMemcpyAsync(counts, list_off, (size_t)U * 4, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
        const bool vec = ((reinterpret_cast<uintptr_t>(e_token) | reinterpret_cast<uintptr_t>(e_val)) & 15u) == 0;
        note_launches(2);
        k_list_scatter<<<grid_for((n + SCATTER_ITEMS - 1) / SCATTER_ITEMS, 256), 256, 0, s>>>(
            e_token, e_val, n, U, counts, alt_vals, g, vec);
        k_list_rank<<<grid_for(U, RANK_THREADS), RANK_THREADS, 0, s>>>(list_off, U, alt_vals, e_val, g);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    // long lists: the radix passes (gated when the choice is the device's)
    if (p != 1) return radix_sort_pairs(e_token, e_val, alt_keys, alt_vals, n, key_bits, scratch, s, false, g);
    return cudaSuccess;
}

cudaError_t token_histogram(const uint32_t* e_token, uint64_t n, uint32_t* counts, uint32_t limit, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    note_launches();
    k_histogram<<<grid_for(n, 256), 256, 0, s>>>(e_token, n, counts, limit);
    return cudaGetLastError();
}

cudaError_t scatter_entries(const uint32_t* e_token, const uint32_t* e_set, const uint32_t* e_pos, uint64_t n,
                            uint32_t* cursor, uint32_t* idx_set, uint32_t* idx_pos, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    note_launches();
    k_scatter<<<grid_for(n, 256), 256, 0, s>>>(e_token, e_set, e_pos, n, cursor, idx_set, idx_pos);
    return cudaGetLastError();
}

cudaError_t gather_entries(const uint32_t* order, uint64_t n, const uint32_t* e_set, const uint32_t* e_pos,
                           uint32_t* idx_set, uint32_t* idx_pos, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    note_launches();
    k_gather<<<grid_for(n, 256), 256, 0, s>>>(order, n, e_set, e_pos, idx_set, idx_pos);
    return cudaGetLastError();
}

cudaError_t iota_u32(uint32_t* out, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    note_launches();
    k_iota<<<grid_for(n, 256), 256, 0, s>>>(out, n);
    return cudaGetLastError();
}

namespace {

__global__ void k_split_pairs(const uint2* __restrict__ pairs, uint64_t n, uint32_t* __restrict__ first,
                              uint32_t* __restrict__ second) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint2 p = pairs[i];
        first[i] = p.x;
        second[i] = p.y;
    }
}

__global__ void k_zip_pairs(const uint32_t* __restrict__ first, const uint32_t* __restrict__ second, uint64_t n,
                            uint2* __restrict__ pairs) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        pairs[i] = make_uint2(first[i], second[i]);
}

}  // namespace

cudaError_t sort_pair_list(uint2* pairs, uint64_t n, int first_bits, int second_bits, uint32_t* a, uint32_t* b,
                           uint32_t* c, uint32_t* d, uint32_t* scratch, cudaStream_t s) {
    if (n <= 1) return cudaSuccess;
    note_launches();
    k_split_pairs<<<grid_for(n, 256), 256, 0, s>>>(pairs, n, a, b);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // keys = second, values = first; then keys = first, values = second (stable)
    e = radix_sort_pairs(b, a, c, d, n, second_bits < 1 ? 1 : second_bits, scratch, s);
    if (e != cudaSuccess) return e;
    e = radix_sort_pairs(a, b, c, d, n, first_bits < 1 ? 1 : first_bits, scratch, s);
    if (e != cudaSuccess) return e;
    note_launches();
    k_zip_pairs<<<grid_for(n, 256), 256, 0, s>>>(a, b, n, pairs);
    return cudaGetLastError();
}

cudaError_t validate_collection(CollView c, uint64_t n_tokens, uint32_t* flags, uint2* meta, cudaStream_t s) {
    if (c.n == 0) return cudaSuccess;
    note_launches();
    k_validate<<<grid_for((uint64_t)c.n * 32, 256), 256, 0, s>>>(c, n_tokens, flags, meta);
    return cudaGetLastError();
}

namespace {
template <int LPS>
cudaError_t launch_validate_bitmaps(CollView c, uint64_t n_tokens, uint32_t* flags, uint2* meta, int words,
                                    uint64_t* out, cudaStream_t s) {
    const unsigned g = grid_for((uint64_t)c.n * LPS, BITMAP_THREADS);
    note_launches();
    switch (words) {
    case 1: k_validate_bitmaps<1, LPS><<<g, BITMAP_THREADS, 0, s>>>(c, n_tokens, flags, meta, out); break;
    case 2: k_validate_bitmaps<2, LPS><<<g, BITMAP_THREADS, 0, s>>>(c, n_tokens, flags, meta, out); break;
    case 4: k_validate_bitmaps<4, LPS><<<g, BITMAP_THREADS, 0, s>>>(c, n_tokens, flags, meta, out); break;
    case 8: k_validate_bitmaps<8, LPS><<<g, BITMAP_THREADS, 0, s>>>(c, n_tokens, flags, meta, out); break;
    case 16: k_validate_bitmaps<16, LPS><<<g, BITMAP_THREADS, 0, s>>>(c, n_tokens, flags, meta, out); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
}  // namespace

cudaError_t validate_with_bitmaps(CollView c, uint64_t n_tokens, uint32_t* flags, uint2* meta, int words, uint64_t* out,
                                  cudaStream_t s, uint32_t min_size) {
    if (c.n == 0) return cudaSuccess;
    constexpr uint32_t WARP_SET_SIZE = 128;  // sets this long (all of the part) take a warp each
    return min_size >= WARP_SET_SIZE ? launch_validate_bitmaps<32>(c, n_tokens, flags, meta, words, out, s)
                                     : launch_validate_bitmaps<8>(c, n_tokens, flags, meta, words, out, s);
}

cudaError_t generate_bitmaps(CollView c, int words, uint64_t* out, cudaStream_t s, unsigned max_blocks) {
    if (c.n == 0) return cudaSuccess;
    unsigned g = grid_for((uint64_t)c.n * 8, BITMAP_THREADS);
    if (max_blocks && g > max_blocks) g = max_blocks;
    note_launches();
    switch (words) {
    case 1: k_bitmaps<1><<<g, BITMAP_THREADS, 0, s>>>(c, out); break;
    case 2: k_bitmaps<2><<<g, BITMAP_THREADS, 0, s>>>(c, out); break;
    case 4: k_bitmaps<4><<<g, BITMAP_THREADS, 0, s>>>(c, out); break;
    case 8: k_bitmaps<8><<<g, BITMAP_THREADS, 0, s>>>(c, out); break;
    case 16: k_bitmaps<16><<<g, BITMAP_THREADS, 0, s>>>(c, out); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace hs
