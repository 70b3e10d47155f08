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
#include "kernels.h"

namespace hs {

namespace {

constexpr int JOIN_THREADS = 256;
constexpr int JOIN_WARPS = JOIN_THREADS / 32;
constexpr uint32_t MAXP = 1024;  // probe tokens staged in shared memory per warp

struct Window {
    uint32_t lo, hi;
};

__device__ __forceinline__ Window candidate_window(const JoinParams& P, uint32_t p, uint32_t lp) {
    Window w;
    const uint32_t ms = P.B.minsize[lp];
    w.lo = max(P.first_ge[min(ms, P.R_L + 1)], P.r_lo);
    if (P.self) {
        w.hi = min(p, P.r_hi);
    } else {
        uint32_t mx = P.B.max_partner[lp];
        w.hi = min(P.first_ge[min(mx + 1, P.R_L + 1)], P.r_hi);
    }
    return w;
}

__device__ __forceinline__ void count_stat(const JoinParams& P, int k, uint32_t v, int lane) {
    if (P.stats == nullptr) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    if (lane == 0 && v) atomicAdd(P.stats + k, (unsigned long long)v);
}

template <int W>
__device__ __forceinline__ bool bitmap_pass(const JoinParams& P, const uint64_t (&bp)[W > 0 ? W : 1], uint32_t c,
                                            uint32_t lp, uint32_t lc, uint32_t mo) {
    if constexpr (W == 0) {
        return true;
    } else {
        uint32_t pop = 0;
        const uint64_t* bc = P.bits_R + (uint64_t)c * W;
#pragma unroll
        for (int q = 0; q < W; ++q) pop += __popcll(bp[q] ^ __ldg(bc + q));
        return lp + lc - pop >= 2u * mo;
    }
}

// Verifies the warp's surviving items and appends the accepted pairs.
// own: per-lane ownership position (a-index for lane mode, b-index for warp
// mode) or NOWN.
template <int VMODE>
__device__ __forceinline__ void verify_and_emit(const JoinParams& P, uint32_t p, const uint32_t* a, uint32_t lp,
                                                bool keep, uint32_t c, uint32_t lc, uint32_t mo, uint32_t own_a,
                                                uint32_t own_b, int lane) {
    uint32_t used = 0;
    if constexpr (VMODE == 1) {
        bool ok = false;
        if (keep) ok = verify_serial(a, lp, P.R.tokens + P.R.starts[c], lc, mo, own_a, &used);
        emit(P.out, ok, p, c, lane);
    } else {
        unsigned m = __ballot_sync(FULL, keep);
        while (m) {
            int src = __ffs(m) - 1;
            m &= m - 1;
            uint32_t cc = __shfl_sync(FULL, c, src);
            uint32_t ll = __shfl_sync(FULL, lc, src);
            uint32_t mm = __shfl_sync(FULL, mo, src);
            uint32_t ob = __shfl_sync(FULL, own_b, src);
            uint32_t u = 0;
            bool ok = verify_warp(a, lp, P.R.tokens + P.R.starts[cc], ll, mm, ob, lane, &u);
            if (lane == 0) used += u;
            emit(P.out, ok && lane == 0, p, cc, lane);
        }
    }
    count_stat(P, 6, used, lane);
}

template <int VMODE, int W>
__device__ void fgss_probe(const JoinParams& P, uint32_t p, uint32_t* sbuf, int lane) {
    const uint32_t lp = P.S.sizes[p];
    if (lp == 0) return;
    const Window win = candidate_window(P, p, lp);
    if (win.lo >= win.hi) return;
    const uint32_t* pg = P.S.tokens + P.S.starts[p];
    const uint32_t* a = pg;
    if (lp <= MAXP) {
        for (uint32_t i = lane; i < lp; i += 32) sbuf[i] = pg[i];
        __syncwarp();
        a = sbuf;
    }
    uint64_t bp[W > 0 ? W : 1];
    if constexpr (W > 0) {
#pragma unroll
        for (int q = 0; q < W; ++q) bp[q] = __ldg(P.bits_S + (uint64_t)p * W + q);
    }
    const uint32_t mp = P.B.probe_prefix[lp];
    for (uint32_t j0 = 0; j0 < mp; j0 += 32) {
        const uint32_t j = j0 + lane;
        uint32_t first = 0, cnt = 0;
        if (j < mp) {
            uint32_t t = a[j];
            if (t < P.X.universe) {
                uint32_t b0 = P.X.list_off[t], b1 = P.X.list_off[t + 1];
                if (P.X.sorted) {
                    b0 = lower_bound_u32(P.X.set, b0, b1, win.lo);
                    b1 = lower_bound_u32(P.X.set, b0, b1, win.hi);
                }
                first = b0;
                cnt = b1 - b0;
            }
        }
        const uint32_t incl = warp_incl_scan(cnt, lane);
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        for (uint32_t q0 = 0; q0 < total; q0 += 32) {
            const uint32_t q = q0 + lane;
            bool keep = q < total;
            const uint32_t qq = keep ? q : 0;
            int jj = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                uint32_t v = __shfl_sync(FULL, incl, jj + step - 1);
                if (v <= qq) jj += step;
            }
            const uint32_t f_jj = __shfl_sync(FULL, first, jj);
            const uint32_t i_jj = __shfl_sync(FULL, incl, jj);
            const uint32_t c_jj = __shfl_sync(FULL, cnt, jj);
            const uint32_t e = f_jj + (qq - (i_jj - c_jj));
            const uint32_t jp = j0 + (uint32_t)jj;
            uint32_t c = 0, pc = 0, lc = 0, mo = 0;
            if (keep) {
                c = P.X.set[e];
                pc = P.X.pos[e];
                if (!P.X.sorted) keep = c >= win.lo && c < win.hi;
            }
            if (keep) {
                lc = P.R.sizes[c];
                const uint32_t big = max(lp, lc), small = min(lp, lc);
                mo = minoverlap(P.B, big, small);
                keep = 1u + min(lp - jp - 1u, lc - pc - 1u) >= mo;  // positional bound
            }
            count_stat(P, 0, q < total ? 1u : 0u, lane);
            count_stat(P, 5, (W > 0 && keep) ? 1u : 0u, lane);
            if (keep) keep = bitmap_pass<W>(P, bp, c, lp, lc, mo);
            count_stat(P, 1, keep ? 1u : 0u, lane);
            count_stat(P, 2, keep ? lc : 0u, lane);
            verify_and_emit<VMODE>(P, p, a, lp, keep, c, lc, mo, jp, pc, lane);
        }
    }
    __syncwarp();
}

template <int VMODE, int W>
__device__ void enum_probe(const JoinParams& P, uint32_t p, uint32_t* sbuf, int lane) {
    const uint32_t lp = P.S.sizes[p];
    if (lp == 0) return;
    const Window win = candidate_window(P, p, lp);
    if (win.lo >= win.hi) return;
    const uint32_t* pg = P.S.tokens + P.S.starts[p];
    const uint32_t* a = pg;
    if (lp <= MAXP) {
        for (uint32_t i = lane; i < lp; i += 32) sbuf[i] = pg[i];
        __syncwarp();
        a = sbuf;
    }
    uint64_t bp[W > 0 ? W : 1];
    if constexpr (W > 0) {
#pragma unroll
        for (int q = 0; q < W; ++q) bp[q] = __ldg(P.bits_S + (uint64_t)p * W + q);
    }
    for (uint32_t c0 = win.lo; c0 < win.hi; c0 += 32) {
        const uint32_t c = c0 + lane;
        bool keep = c < win.hi;
        uint32_t lc = 0, mo = 0;
        if (keep) {
            lc = P.R.sizes[c];
            const uint32_t big = max(lp, lc), small = min(lp, lc);
            mo = minoverlap(P.B, big, small);
            keep = bitmap_pass<W>(P, bp, c, lp, lc, mo);
        }
        count_stat(P, 0, c < win.hi ? 1u : 0u, lane);
        count_stat(P, 5, (W > 0 && c < win.hi) ? 1u : 0u, lane);
        count_stat(P, 1, keep ? 1u : 0u, lane);
        count_stat(P, 2, keep ? lc : 0u, lane);
        verify_and_emit<VMODE>(P, p, a, lp, keep, c, lc, mo, NOWN, NOWN, lane);
    }
    __syncwarp();
}

template <int TECH, int VMODE, int W>
__global__ void __launch_bounds__(JOIN_THREADS) k_join(JoinParams P) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* sbuf = smem + warp * MAXP;
    const uint32_t nprobe = P.p_hi - P.p_lo;
    for (;;) {
        uint32_t i = 0;
        if (lane == 0) i = atomicAdd(P.work, 1u);
        i = __shfl_sync(FULL, i, 0);
        if (i >= nprobe) break;
        if constexpr (TECH == TECH_FGSS)
            fgss_probe<VMODE, W>(P, P.p_lo + i, sbuf, lane);
        else
            enum_probe<VMODE, W>(P, P.p_lo + i, sbuf, lane);
    }
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
    uint32_t* sbuf = smem + warp * MAXP;
    for (;;) {
        uint32_t i = 0;
        if (lane == 0) i = atomicAdd(work, 1u);
        i = __shfl_sync(FULL, i, 0);
        if (i >= n_probes) break;
        const uint32_t p = probes[i];
        const uint32_t lp = S.sizes[p];
        const uint32_t cb = i ? offsets[i - 1] : 0, ce = offsets[i];
        const uint32_t* pg = S.tokens + S.starts[p];
        const uint32_t* a = pg;
        if (lp <= MAXP) {
            for (uint32_t k = lane; k < lp; k += 32) sbuf[k] = pg[k];
            __syncwarp();
            a = sbuf;
        }
        for (uint32_t k0 = cb; k0 < ce; k0 += 32) {
            const uint32_t k = k0 + lane;
            bool keep = k < ce;
            uint32_t c = 0, lc = 0, mo = 0;
            if (keep) {
                c = cands[k];
                lc = R.sizes[c];
                // verification.hpp:346-348 / hybrid_kernels.hpp:50: minoverlap(probe, candidate),
                // for any pair (an incompatible length pair gets min(lp, lc)).
                const uint32_t big = max(lp, lc), small = min(lp, lc);
                if (small >= B.minsize[big]) mo = minoverlap(B, big, small);
                else mo = small;
            }
            if constexpr (VMODE == 1) {
                bool ok = keep && verify_serial(a, lp, R.tokens + R.starts[c], lc, mo, NOWN);
                emit(out, ok, p, c, lane);
            } else {
                unsigned m = __ballot_sync(FULL, keep);
                while (m) {
                    int src = __ffs(m) - 1;
                    m &= m - 1;
                    uint32_t cc = __shfl_sync(FULL, c, src);
                    uint32_t ll = __shfl_sync(FULL, lc, src);
                    uint32_t mm = __shfl_sync(FULL, mo, src);
                    bool ok = verify_warp(a, lp, R.tokens + R.starts[cc], ll, mm, NOWN, lane);
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

template <int TECH, int VMODE>
cudaError_t dispatch_words(const JoinParams& P, int sm_count, cudaStream_t s) {
    switch (P.bits_R ? P.words : 0) {
    case 0: return launch_persistent(k_join<TECH, VMODE, 0>, sm_count, s, P);
    case 1: return launch_persistent(k_join<TECH, VMODE, 1>, sm_count, s, P);
    case 2: return launch_persistent(k_join<TECH, VMODE, 2>, sm_count, s, P);
    case 4: return launch_persistent(k_join<TECH, VMODE, 4>, sm_count, s, P);
    case 8: return launch_persistent(k_join<TECH, VMODE, 8>, sm_count, s, P);
    default: return cudaErrorInvalidValue;
    }
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
    const size_t smem = JOIN_WARPS * MAXP * sizeof(uint32_t);
    int per_sm = 0;
    cudaError_t e;
    if (vmode == 2) {
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
