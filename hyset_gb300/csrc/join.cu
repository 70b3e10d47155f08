// join.cu — the filter + verify kernels of the exact set-similarity join.
//
// One persistent launch per join (or per block pair in the reference-shaped
// handlers).  Every warp steals probe ids from a global counter, so heavy
// probes (long sets, long inverted lists) balance dynamically across the 152
// SMs.  Per probe the warp:
//   1. derives the candidate id window from the size-sorted order and the
//      length bounds (replaces device::length_filter per pair,
//      include/hyset/device_algorithms.hpp:21-53 and the minsize tests at :100, :297);
//   2. FGSS: walks the inverted lists of its maxprefix tokens (one lane per
//      token, binary search of the window in set-id-sorted lists), turning each
//      entry into a work item (candidate, probe position, candidate position)
//      (replaces fgssjoin::prefix_filter, :265-303);
//      BITMAP / DIRECT: enumerates the window 32 candidates at a time
//      (replaces bitmap::filter, :76-118);
//   3. filters items by the positional bound and, optionally, the XOR-bitmap
//      bound (|r| + |s| - popc(b_r ^ b_s)) / 2 >= minoverlap (:104-113);
//   4. verifies survivors — one lane per candidate (two-pointer merge) or one
//      warp per candidate (32-token coalesced steps, ballot counting, early
//      termination) — and appends (probe, candidate) with one atomic per warp
//      (replaces verification::device::verify_pairs, verification.hpp:60-138,
//      and hybrid::kernels::scenario_1/2, hybrid_kernels.hpp:14-165).
// A pair reached through several shared prefix tokens is emitted once: only the
// item at its smallest common token verifies it (the other items stop at the
// first common token they see).  No dense B x B filter matrix exists.
#include "join_impl.cuh"
#include "verify_impl.cuh"

#ifndef HS_ITEM_CARRY
#define HS_ITEM_CARRY 1  // probe-major FGSS: items carried until a round of 32 is full (fgss_carry)
#endif

namespace hs {

namespace {

// BD: the index is token records in the bound layout (IndexView::bound;
// prefix-index joins only).
template <int TECH, int VMODE, int W, bool ST, bool BD = false>
__global__ void __launch_bounds__(JOIN_THREADS, HS_JOIN_MIN_BLOCKS) k_join(JoinParams P) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* sbuf = smem + warp * MAXP;
    const uint32_t nprobe = P.p_hi - P.p_lo;
    const uint32_t grab = P.grab ? P.grab : 1;
    uint32_t i = 0, i_end = 0;
    ItemCarry ic;  // FGSS with HS_ITEM_CARRY: items pending across slot rounds and batches
    ic.q = sbuf;   // its queue for bound-layout indexes (QSLOTS * QF_N <= MAXP words)
    static_assert(QSLOTS * QF_N <= MAXP, "item queue exceeds the warp's shared-memory slot");
    uint32_t nheavy = 0;  // the longest probes (the first from the top) go as slot segments, one per steal
    if constexpr (TECH == TECH_FGSS && HS_ITEM_CARRY) {
        const uint32_t hf = max(P.heavy_from, P.p_lo);
        nheavy = P.p_hi > hf ? P.p_hi - hf : 0u;
        const uint32_t units = nheavy * P.segs;
        for (;;) {
            uint32_t u = 0;
            if (lane == 0) u = atomicAdd(P.work + 1, 1u);
            u = __shfl_sync(FULL, u, 0);
            if (u >= units) break;
            const uint32_t h = u / P.segs, g = u - h * P.segs;
            fgss_carry<VMODE, W, ST, BD>(P, h, 1, lane, ic, g * P.seg_slots, (g + 1) * P.seg_slots);
        }
    }
    for (;;) {
        if (i >= i_end) {
            const uint32_t steal = grab * HS_JOIN_STEAL;  // probes per atomic on the shared counter
            if (lane == 0) i = atomicAdd(P.work, steal);
            i = __shfl_sync(FULL, i, 0) + nheavy;
            i_end = min(nprobe, i + steal);
        }
        if (i >= nprobe) break;
        const uint32_t end = min(i_end, i + grab);
        // largest sets first: the heaviest probes start early, the tail is light
        if constexpr (TECH == TECH_FGSS) {
            if constexpr (HS_ITEM_CARRY) fgss_carry<VMODE, W, ST, BD>(P, i, end - i, lane, ic);
            else fgss_batch<VMODE, W, ST, true, BD>(P, i, end - i, lane);
        } else {
            for (uint32_t q = i; q < end; ++q) enum_probe<VMODE, W, ST>(P, P.p_hi - 1 - q, sbuf, lane);
        }
        i = end;
    }
    if constexpr (TECH == TECH_FGSS && HS_ITEM_CARRY) flush_items<VMODE, W, ST, BD>(P, ic, lane);
}

#ifndef HS_VREVERSE
#define HS_VREVERSE 1
#endif

#ifndef HS_VCLAIM
#define HS_VCLAIM 1
#endif
constexpr uint32_t VCLAIM = HS_VCLAIM;  // probes a warp of the batch verifier takes per atomic

// Explicit candidate lists: probes[i] owns candidates [offsets[i-1], offsets[i]).
template <int VMODE, int W>
__global__ void __launch_bounds__(JOIN_THREADS) k_verify_candidates(CollView R, CollView S, BoundsView B,
                                                                    const uint64_t* __restrict__ sig_R,
                                                                    const uint64_t* __restrict__ sig_S,
                                                                    const uint32_t* __restrict__ probes,
                                                                    const uint32_t* __restrict__ offsets,
                                                                    const uint32_t* __restrict__ cands,
                                                                    uint32_t n_probes, Sink out, unsigned int* work) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* sbuf = smem + warp * verify_smem_words(VMODE, VMAXP);
    uint32_t i = 0, i_end = 0;
    for (;; ++i) {
        if (i >= i_end) {  // VCLAIM probes per atomic on the shared counter
            if (lane == 0) i = atomicAdd(work, (unsigned)VCLAIM);
            i = __shfl_sync(FULL, i, 0);
            i_end = min(n_probes, i + VCLAIM);
        }
        if (i >= n_probes) break;
        // lists from the last: callers list probes by id, so the longest sets
        // (the longest merges) start first and the launch's tail is light
        const uint32_t li = HS_VREVERSE ? n_probes - 1 - i : i;
        const uint32_t cb = li ? offsets[li - 1] : 0, ce = offsets[li];
        const uint32_t* list = cands + cb;
        verify_probe_list<VMODE, W, VMAXP>(R, S, B, sig_R, sig_S, probes[li], [list](uint32_t k) { return list[k]; },
                                           ce - cb, out, sbuf, lane);
    }
}

template <int VMODE, int W>
cudaError_t launch_verify_w(CollView R, CollView S, BoundsView B, const uint64_t* sig_R, const uint64_t* sig_S,
                            const uint32_t* probes, const uint32_t* offsets, const uint32_t* cands, uint32_t n_probes,
                            Sink out, unsigned int* work, int sm_count, cudaStream_t s) {
    const size_t smem = JOIN_WARPS * verify_smem_words(VMODE, VMAXP) * sizeof(uint32_t);
    int per_sm = 0;
    const cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_verify_candidates<VMODE, W>, JOIN_THREADS, smem);
    if (e != cudaSuccess) return e;
    k_verify_candidates<VMODE, W><<<sm_count * (per_sm ? per_sm : 1), JOIN_THREADS, smem, s>>>(
        R, S, B, sig_R, sig_S, probes, offsets, cands, n_probes, out, work);
    return cudaGetLastError();
}

template <int VMODE>
cudaError_t launch_verify_v(int words, CollView R, CollView S, BoundsView B, const uint64_t* sig_R,
                            const uint64_t* sig_S, const uint32_t* probes, const uint32_t* offsets,
                            const uint32_t* cands, uint32_t n_probes, Sink out, unsigned int* work, int sm_count,
                            cudaStream_t s) {
    switch (sig_R && sig_S ? words : 0) {
    case 0: return launch_verify_w<VMODE, 0>(R, S, B, sig_R, sig_S, probes, offsets, cands, n_probes, out, work, sm_count, s);
    case 1: return launch_verify_w<VMODE, 1>(R, S, B, sig_R, sig_S, probes, offsets, cands, n_probes, out, work, sm_count, s);
    case 2: return launch_verify_w<VMODE, 2>(R, S, B, sig_R, sig_S, probes, offsets, cands, n_probes, out, work, sm_count, s);
    case 4: return launch_verify_w<VMODE, 4>(R, S, B, sig_R, sig_S, probes, offsets, cands, n_probes, out, work, sm_count, s);
    case 8: return launch_verify_w<VMODE, 8>(R, S, B, sig_R, sig_S, probes, offsets, cands, n_probes, out, work, sm_count, s);
    default: return cudaErrorInvalidValue;
    }
}

template <typename K>
cudaError_t launch_persistent(K kernel, int sm_count, cudaStream_t s, const JoinParams& P) {
    note_launches();
    const size_t smem = JOIN_WARPS * MAXP * sizeof(uint32_t);
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, JOIN_THREADS, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    kernel<<<sm_count * per_sm, JOIN_THREADS, smem, s>>>(P);
    return cudaGetLastError();
}

template <int TECH, int VMODE, bool ST, bool BD>
cudaError_t dispatch_words_bd(const JoinParams& P, int sm_count, cudaStream_t s) {
    switch (P.bits_R ? P.words : 0) {
    case 0: return launch_persistent(k_join<TECH, VMODE, 0, ST, BD>, sm_count, s, P);
    case 1: return launch_persistent(k_join<TECH, VMODE, 1, ST, BD>, sm_count, s, P);
    case 2: return launch_persistent(k_join<TECH, VMODE, 2, ST, BD>, sm_count, s, P);
    case 4: return launch_persistent(k_join<TECH, VMODE, 4, ST, BD>, sm_count, s, P);
    case 8: return launch_persistent(k_join<TECH, VMODE, 8, ST, BD>, sm_count, s, P);
    case 16:  // 1024-bit signatures: the prefix filter only
        if constexpr (TECH == TECH_FGSS) return launch_persistent(k_join<TECH, VMODE, 16, ST, BD>, sm_count, s, P);
        return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
    }
}

template <int TECH, int VMODE, bool ST>
cudaError_t dispatch_words_st(const JoinParams& P, int sm_count, cudaStream_t s) {
    if constexpr (TECH == TECH_FGSS) {
        if (P.X.bound) return dispatch_words_bd<TECH, VMODE, ST, true>(P, sm_count, s);
    }
    return dispatch_words_bd<TECH, VMODE, ST, false>(P, sm_count, s);
}

template <int TECH, int VMODE>
cudaError_t dispatch_words(const JoinParams& P, int sm_count, cudaStream_t s) {
    return P.stats ? dispatch_words_st<TECH, VMODE, true>(P, sm_count, s)
                   : dispatch_words_st<TECH, VMODE, false>(P, sm_count, s);
}

}  // namespace

uint32_t join_resident_warps(int sm_count) { return (uint32_t)sm_count * HS_JOIN_MIN_BLOCKS * JOIN_WARPS; }

cudaError_t launch_join(const JoinParams& P, int technique, int vmode, int sm_count, cudaStream_t s) {
    if (P.p_hi <= P.p_lo) return cudaSuccess;
    if (technique == TECH_FGSS)
        return vmode == 2 ? dispatch_words<TECH_FGSS, 2>(P, sm_count, s) : dispatch_words<TECH_FGSS, 1>(P, sm_count, s);
    // BITMAP and DIRECT share the enumeration kernel; DIRECT runs without signatures.
    JoinParams Q = P;
    if (technique == TECH_DIRECT) Q.bits_R = Q.bits_S = nullptr;
    return vmode == 2 ? dispatch_words<TECH_BITMAP, 2>(Q, sm_count, s) : dispatch_words<TECH_BITMAP, 1>(Q, sm_count, s);
}

cudaError_t launch_verify_candidates(CollView R, CollView S, BoundsView B, const uint32_t* probes,
                                     const uint32_t* offsets, const uint32_t* cands, uint32_t n_probes, int vmode,
                                     Sink out, unsigned int* work, int sm_count, cudaStream_t s, const uint64_t* sig_R,
                                     const uint64_t* sig_S, int words) {
    if (n_probes == 0) return cudaSuccess;
    note_launches();
    if (vmode == 3)
        return launch_verify_v<3>(words, R, S, B, sig_R, sig_S, probes, offsets, cands, n_probes, out, work, sm_count, s);
    if (vmode == 2)
        return launch_verify_v<2>(words, R, S, B, sig_R, sig_S, probes, offsets, cands, n_probes, out, work, sm_count, s);
    return launch_verify_v<1>(words, R, S, B, sig_R, sig_S, probes, offsets, cands, n_probes, out, work, sm_count, s);
}

}  // namespace hs
