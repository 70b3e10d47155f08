// join_tm.cu — token-major prefix-filter join (the whole-join FGSS path).
//
// The prefix entries of every set (its maxprefix tokens) are grouped by token
// with one histogram, one scan and one warp-aggregated atomic scatter — no sort.
// A work unit is one token's group: a warp stages the group's candidate entries
// in shared memory (one coalesced load) and pairs them with the group's probe
// entries, 32 probes per step (lane per probe), in registers:
//   self-join:  c < p, |c| >= minsize(|p|), c's entry lies in its midprefix
//               (the reference's index holds midprefix entries only,
//               include/hyset/collection.hpp:128-135);
//   R-S join:   |r| within [minsize(|s|), max_partner(|s|)];
//   both:       positional bound 1 + min(|p|-jp-1, |c|-pc-1) >= minoverlap.
// Surviving (probe, candidate) items are queued in shared memory and, 32 at a
// time, checked against the XOR-bitmap bound and verified one lane per item
// with the ownership rule (a pair is verified only from its smallest common
// token, so it is emitted once).  Every pair the reference's allpairs finds
// shares a token in the probe's maxprefix and the candidate's midprefix, so it
// appears in that token's group; the output set is the reference's.
// Replaces fgssjoin::prefix_filter + verify_pairs (device_algorithms.hpp:265-303,
// verification.hpp:60-138) and the dense B x B count matrix between them.
#include "kernels.h"

namespace hs {

namespace {

constexpr int TM_THREADS = 256;
constexpr int TM_WARPS = TM_THREADS / 32;
constexpr uint32_t TM_CAND = 128;   // candidate entries staged per warp and step
constexpr uint32_t TM_QUEUE = 64;   // queued items per warp (flushed at >= 32)

struct Item {
    uint32_t p, c, pos, len, mo;  // pos = jp | pc << 16, len = lp | lc << 16
};

struct WarpSmem {
    uint2 cand[TM_CAND];  // (set, size | pos << 16); pos = 0xFFFF marks a non-index entry
    Item q[TM_QUEUE];
};

__device__ __forceinline__ void stat_add(const TokenJoinParams& P, int k, uint32_t v, int lane) {
    if (P.stats == nullptr) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    if (lane == 0 && v) atomicAdd(P.stats + k, (unsigned long long)v);
}

// Bitmap bound + verification of the first `cnt` queued items (lane per item).
template <int W>
__device__ __forceinline__ void flush(const TokenJoinParams& P, WarpSmem& S, uint32_t cnt, int lane) {
    bool keep = (uint32_t)lane < cnt;
    Item it{0, 0, 0, 0, 0};
    if (keep) it = S.q[lane];
    __syncwarp();
    const uint32_t lp = it.len & 0xFFFFu, lc = it.len >> 16, jp = it.pos & 0xFFFFu;
    if constexpr (W > 0) {
        if (keep) {
            const uint64_t* bs = P.bits_S + (uint64_t)it.p * W;
            const uint64_t* bc = P.bits_R + (uint64_t)it.c * W;
            uint32_t pop = 0;
#pragma unroll
            for (int w = 0; w < W; ++w) pop += __popcll(__ldg(bs + w) ^ __ldg(bc + w));
            keep = lp + lc - pop >= 2u * it.mo;
        }
    }
    stat_add(P, 1, keep ? 1u : 0u, lane);
    stat_add(P, 2, keep ? lc : 0u, lane);
    bool ok = false;
    uint32_t used = 0;
    if (keep) {
        const uint2 pm = P.S.meta[it.p];
        const uint2 cm = P.R.meta[it.c];
        ok = verify_serial(P.S.tokens + pm.x, lp, P.R.tokens + cm.x, lc, it.mo, jp, &used);
    }
    stat_add(P, 6, used, lane);
    emit(P.out, ok, it.p, it.c, lane);
}

template <int W>
__global__ void __launch_bounds__(TM_THREADS) k_join_tm(TokenJoinParams P) {
    __shared__ WarpSmem smem_all[TM_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpSmem& S = smem_all[warp];
    const uint32_t U = P.universe;
    uint32_t qn = 0;  // queued items (warp-uniform)
    for (;;) {
        uint32_t t0 = 0;
        if (lane == 0) t0 = atomicAdd(P.work, P.grab);
        t0 = __shfl_sync(FULL, t0, 0);
        if (t0 >= U) break;
        const uint32_t t1 = min(U, t0 + P.grab);
        for (uint32_t i = t0; i < t1; ++i) {
            const uint32_t t = U - 1 - i;  // frequent (heavy) tokens have the largest ids: start there
            const uint32_t g0 = P.gs_off[t], g1 = P.gs_off[t + 1];  // probe entries
            const uint32_t h0 = P.gr_off[t], h1 = P.gr_off[t + 1];  // candidate entries
            if (g0 == g1 || h0 == h1 || (P.self && g1 - g0 < 2)) continue;
            for (uint32_t pb = g0; pb < g1; pb += 32) {
                // lane = one probe entry
                const uint32_t pe = pb + lane;
                const bool pv = pe < g1;
                // an invalid lane gets an empty size window, so every test fails for it
                uint32_t p = 0, jp = 0, lp = 0, ms = 1, mx = 0, plim = 0;
                if (pv) {
                    p = P.gs_set[pe];
                    const uint32_t ps = P.gs_ps[pe];
                    jp = ps & 0xFFFFu;
                    lp = ps >> 16;
                    ms = P.B.minsize[lp];
                    mx = P.self ? lp : P.B.max_partner[lp];
                    plim = P.self ? p : 0xFFFFFFFFu;  // self-join: candidates precede the probe
                }
                for (uint32_t cb = h0; cb < h1; cb += TM_CAND) {
                    const uint32_t cn = min(TM_CAND, h1 - cb);
                    __syncwarp();
                    for (uint32_t k = lane; k < cn; k += 32) {
                        const uint32_t cps = P.gr_ps[cb + k];
                        const uint32_t pc = cps & 0xFFFFu, lc = cps >> 16;
                        // self-join candidates are midprefix entries only
                        const bool idx = !P.self || pc < P.B.index_prefix[lc];
                        S.cand[k] = make_uint2(P.gr_set[cb + k], lc | ((idx ? pc : 0xFFFFu) << 16));
                    }
                    __syncwarp();
                    uint32_t checks = 0;
                    for (uint32_t k = 0; k < cn; ++k) {
                        const uint2 ck = S.cand[k];
                        const uint32_t c = ck.x, lc = ck.y & 0xFFFFu, pc = ck.y >> 16;
                        bool pass = (c < plim) & (lc >= ms) & (lc <= mx) & (pc != 0xFFFFu);
                        if (!__any_sync(FULL, pass)) continue;
                        uint32_t mo = 0;
                        if (pass) {
                            ++checks;
                            mo = minoverlap(P.B, max(lp, lc), min(lp, lc));
                            pass = 1u + min(lp - jp - 1u, lc - pc - 1u) >= mo;
                        }
                        const unsigned m = __ballot_sync(FULL, pass);
                        if (m) {
                            if (pass) {
                                const uint32_t slot = qn + __popc(m & lanemask_lt(lane));
                                S.q[slot] = Item{p, c, jp | (pc << 16), lp | (lc << 16), mo};
                            }
                            qn += __popc(m);
                            if (qn >= 32) {
                                __syncwarp();
                                flush<W>(P, S, 32, lane);
                                // move the overflow (at most 31 items) to the front
                                const uint32_t rest = qn - 32;
                                Item mv{0, 0, 0, 0, 0};
                                if ((uint32_t)lane < rest) mv = S.q[32 + lane];
                                __syncwarp();
                                if ((uint32_t)lane < rest) S.q[lane] = mv;
                                __syncwarp();
                                qn = rest;
                            }
                        }
                    }
                    stat_add(P, 0, checks, lane);
                }
            }
        }
    }
    __syncwarp();
    if (qn) flush<W>(P, S, qn, lane);
}

// ---- group build ---------------------------------------------------------

// One warp per set: counts[token]++ for the first pre[size] tokens.
__global__ void k_group_count(CollView c, const uint32_t* __restrict__ pre, uint32_t* counts) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < c.n; s += warps) {
        const uint2 m = c.meta[s];
        const uint32_t l = pre[m.y];
        for (uint32_t i = lane; i < l; i += 32) atomicAdd(&counts[__ldg(c.tokens + m.x + i)], 1u);
    }
}

// One warp per set: scatter (set, pos | size << 16) into its token's group.
__global__ void k_group_scatter(CollView c, const uint32_t* __restrict__ pre, uint32_t* cursor, uint32_t* gset,
                                uint32_t* gps) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < c.n; s += warps) {
        const uint2 m = c.meta[s];
        const uint32_t l = pre[m.y];
        for (uint32_t i = lane; i < l; i += 32) {
            const uint32_t at = atomicAdd(&cursor[__ldg(c.tokens + m.x + i)], 1u);
            gset[at] = s;
            gps[at] = i | (m.y << 16);
        }
    }
}

unsigned grid_sets(uint32_t n) {
    uint64_t g = ((uint64_t)n * 32 + 255) / 256;
    if (g < 1) g = 1;
    if (g > 152u * 64u) g = 152u * 64u;
    return (unsigned)g;
}

}  // namespace

cudaError_t group_count(CollView c, const uint32_t* pre, uint32_t* counts, cudaStream_t s) {
    if (c.n == 0) return cudaSuccess;
    note_launches();
    k_group_count<<<grid_sets(c.n), 256, 0, s>>>(c, pre, counts);
    return cudaGetLastError();
}

cudaError_t group_scatter(CollView c, const uint32_t* pre, uint32_t* cursor, uint32_t* gset, uint32_t* gps,
                          cudaStream_t s) {
    if (c.n == 0) return cudaSuccess;
    note_launches();
    k_group_scatter<<<grid_sets(c.n), 256, 0, s>>>(c, pre, cursor, gset, gps);
    return cudaGetLastError();
}

cudaError_t launch_join_tm(const TokenJoinParams& P, int sm_count, cudaStream_t s) {
    if (P.universe == 0) return cudaSuccess;
    note_launches();
    int per_sm = 0;
    cudaError_t e;
    switch (P.bits_R ? P.words : 0) {
#define HS_TM_CASE(WW)                                                                                 \
    case WW:                                                                                           \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_join_tm<WW>, TM_THREADS, 0);      \
        if (e != cudaSuccess) return e;                                                                \
        k_join_tm<WW><<<sm_count * (per_sm ? per_sm : 1), TM_THREADS, 0, s>>>(P);                      \
        break;
        HS_TM_CASE(0)
        HS_TM_CASE(1)
        HS_TM_CASE(2)
        HS_TM_CASE(4)
        HS_TM_CASE(8)
#undef HS_TM_CASE
    default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace hs
