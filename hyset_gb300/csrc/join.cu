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

namespace hs {

namespace {

template <int TECH, int VMODE, int W, bool ST>
__global__ void __launch_bounds__(JOIN_THREADS, HS_JOIN_MIN_BLOCKS) k_join(JoinParams P) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* sbuf = smem + warp * MAXP;
    const uint32_t nprobe = P.p_hi - P.p_lo;
    const uint32_t grab = P.grab ? P.grab : 1;
    const uint32_t steal = grab * HS_JOIN_STEAL;  // probes per atomic on the shared counter
    uint32_t i = 0, i_end = 0;
    for (;;) {
        if (i >= i_end) {
            if (lane == 0) i = atomicAdd(P.work, steal);
            i = __shfl_sync(FULL, i, 0);
            i_end = min(nprobe, i + steal);
        }
        if (i >= nprobe) break;
        const uint32_t end = min(i_end, i + grab);
        // largest sets first: the heaviest probes start early, the tail is light
        if constexpr (TECH == TECH_FGSS) {
            fgss_batch<VMODE, W, ST>(P, i, end - i, lane);
        } else {
            for (uint32_t q = i; q < end; ++q) enum_probe<VMODE, W, ST>(P, P.p_hi - 1 - q, sbuf, lane);
        }
        i = end;
    }
}

// Staged lane-serial merge: b's first VSTAGE tokens are in `head` (shared
// memory), the rest in global memory; same early-exit bounds as verify_serial.
constexpr uint32_t VSTAGE = 16;            // candidate tokens staged per candidate
constexpr uint32_t VSTRIDE = VSTAGE + 1;   // padded row: the 32 lanes' rows fall in distinct banks
__device__ __forceinline__ bool verify_staged(const uint32_t* a, uint32_t na, const uint32_t* head,
                                              const uint32_t* __restrict__ b, uint32_t nb, uint32_t thr) {
    uint32_t i = 0, k = 0, found = 0, maxa = na, maxb = nb;
    while (maxa >= thr && maxb >= thr && found < thr) {
        const uint32_t x = a[i], y = k < VSTAGE ? head[k] : __ldg(b + k);
        if (x == y) {
            ++i;
            ++k;
            ++found;
        } else if (x < y) {
            ++i;
            --maxa;
        } else {
            ++k;
            --maxb;
        }
    }
    return found >= thr;
}

// Explicit candidate lists: probes[i] owns candidates [offsets[i-1], offsets[i]).
template <int VMODE>
__global__ void __launch_bounds__(JOIN_THREADS) k_verify_candidates(CollView R, CollView S, BoundsView B,
                                                                    const uint32_t* __restrict__ probes,
                                                                    const uint32_t* __restrict__ offsets,
                                                                    const uint32_t* __restrict__ cands,
                                                                    uint32_t n_probes, Sink out, unsigned int* work) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* sbuf = smem + warp * (MAXP + (VMODE == 3 ? 32 * VSTRIDE : 0));
    for (;;) {
        uint32_t i = 0;
        if (lane == 0) i = atomicAdd(work, 1u);
        i = __shfl_sync(FULL, i, 0);
        if (i >= n_probes) break;
        const uint32_t p = probes[i];
        const uint2 pm = S.meta[p];
        const uint32_t lp = pm.y;
        const uint32_t cb = i ? offsets[i - 1] : 0, ce = offsets[i];
        const uint32_t* pg = S.tokens + pm.x;
        const uint32_t* a = pg;
        if (lp <= MAXP) {
            for (uint32_t k = lane; k < lp; k += 32) sbuf[k] = pg[k];
            __syncwarp();
            a = sbuf;
        }
        for (uint32_t k0 = cb; k0 < ce; k0 += 32) {
            const uint32_t k = k0 + lane;
            bool keep = k < ce;
            uint32_t c = 0, lc = 0, mo = 0, cs = 0;
            if (keep) {
                c = cands[k];
                const uint2 cm = R.meta[c];
                cs = cm.x;
                lc = cm.y;
                // hybrid_kernels.hpp:50: minoverlap(probe, candidate),
                // for any pair (an incompatible length pair gets min(lp, lc)).
                const uint32_t big = max(lp, lc), small = min(lp, lc);
                if (small >= B.minsize[big]) mo = minoverlap(B, big, small);
                else mo = small;
            }
            if constexpr (VMODE == 1) {
                bool ok = keep && verify_serial(a, lp, R.tokens + cs, lc, mo, NOWN);
                emit(out, ok, p, c, lane);
            } else if constexpr (VMODE == 3) {
                // the first VSTAGE tokens of the round's 32 candidates arrive with
                // 16 coalesced loads (two candidates per load, one per half-warp);
                // each lane then merges its candidate out of shared memory and
                // reads global memory only past the staged prefix
                uint32_t* tile = sbuf + MAXP;
                const uint32_t t = lane & (VSTAGE - 1);
#pragma unroll
                for (int r = 0; r < 16; ++r) {
                    const int j = 2 * r + (lane >> 4);
                    const uint32_t cj = __shfl_sync(FULL, cs, j), lj = __shfl_sync(FULL, keep ? lc : 0u, j);
                    if (t < lj) tile[j * VSTRIDE + t] = __ldg(R.tokens + cj + t);
                }
                __syncwarp();
                const bool ok = keep && verify_staged(a, lp, tile + lane * VSTRIDE, R.tokens + cs, lc, mo);
                __syncwarp();
                emit(out, ok, p, c, lane);
            } else {
                unsigned m = __ballot_sync(FULL, keep);
                while (m) {
                    int src = __ffs(m) - 1;
                    m &= m - 1;
                    uint32_t cc = __shfl_sync(FULL, c, src);
                    uint32_t c2 = __shfl_sync(FULL, cs, src);
                    uint32_t ll = __shfl_sync(FULL, lc, src);
                    uint32_t mm = __shfl_sync(FULL, mo, src);
                    bool ok = verify_warp(a, lp, R.tokens + c2, ll, mm, NOWN, lane);
                    emit(out, ok && lane == 0, p, cc, lane);
                }
            }
        }
        __syncwarp();
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

template <int TECH, int VMODE, bool ST>
cudaError_t dispatch_words_st(const JoinParams& P, int sm_count, cudaStream_t s) {
    switch (P.bits_R ? P.words : 0) {
    case 0: return launch_persistent(k_join<TECH, VMODE, 0, ST>, sm_count, s, P);
    case 1: return launch_persistent(k_join<TECH, VMODE, 1, ST>, sm_count, s, P);
    case 2: return launch_persistent(k_join<TECH, VMODE, 2, ST>, sm_count, s, P);
    case 4: return launch_persistent(k_join<TECH, VMODE, 4, ST>, sm_count, s, P);
    case 8: return launch_persistent(k_join<TECH, VMODE, 8, ST>, sm_count, s, P);
    default: return cudaErrorInvalidValue;
    }
}

template <int TECH, int VMODE>
cudaError_t dispatch_words(const JoinParams& P, int sm_count, cudaStream_t s) {
    return P.stats ? dispatch_words_st<TECH, VMODE, true>(P, sm_count, s)
                   : dispatch_words_st<TECH, VMODE, false>(P, sm_count, s);
}

}  // namespace

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
                                     Sink out, unsigned int* work, int sm_count, cudaStream_t s) {
    if (n_probes == 0) return cudaSuccess;
    note_launches();
    const size_t smem = JOIN_WARPS * (MAXP + (vmode == 3 ? 32 * VSTRIDE : 0)) * sizeof(uint32_t);
    int per_sm = 0;
    cudaError_t e;
    if (vmode == 3) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_verify_candidates<3>, JOIN_THREADS, smem);
        if (e != cudaSuccess) return e;
        k_verify_candidates<3><<<sm_count * (per_sm ? per_sm : 1), JOIN_THREADS, smem, s>>>(
            R, S, B, probes, offsets, cands, n_probes, out, work);
    } else if (vmode == 2) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_verify_candidates<2>, JOIN_THREADS, smem);
        if (e != cudaSuccess) return e;
        k_verify_candidates<2><<<sm_count * (per_sm ? per_sm : 1), JOIN_THREADS, smem, s>>>(
            R, S, B, probes, offsets, cands, n_probes, out, work);
    } else {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_verify_candidates<1>, JOIN_THREADS, smem);
        if (e != cudaSuccess) return e;
        k_verify_candidates<1><<<sm_count * (per_sm ? per_sm : 1), JOIN_THREADS, smem, s>>>(
            R, S, B, probes, offsets, cands, n_probes, out, work);
    }
    return cudaGetLastError();
}

}  // namespace hs
