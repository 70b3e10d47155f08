// verify_impl.cuh — verification of explicit candidate lists
// (hybrid::kernels::scenario_1 / scenario_2, include/hyset/hybrid_kernels.hpp:14-165):
// one warp takes a probe and its candidates, 32 at a time.  Shared by the
// batch verifier (k_verify_candidates, join.cu) and the persistent consumer of
// the candidate ring (ring.cu).
#pragma once
#include "join_impl.cuh"

namespace hs {
namespace {

// Staged lane-serial merge: b's first VSTAGE tokens are in `head` (shared
// memory), the rest in global memory; same early-exit bounds as verify_serial.
#ifndef HS_VSTAGE
#define HS_VSTAGE 8
#endif
constexpr uint32_t VSTAGE = HS_VSTAGE;     // candidate tokens staged per candidate (a power of two, 2..32)
static_assert(VSTAGE >= 2 && VSTAGE <= 32 && (VSTAGE & (VSTAGE - 1)) == 0, "VSTAGE: a power of two up to 32");
constexpr uint32_t VSTRIDE = VSTAGE + 1;   // padded row: the 32 lanes' rows fall in distinct banks

#ifndef HS_VMAXP
#define HS_VMAXP 384
#endif
// Probe tokens the batch verifier stages in shared memory (longer probes are
// merged from L1/L2).  Smaller than the join kernels' stage so that more warps
// fit an SM: the verifier waits on gathers, and more resident warps hide them.
constexpr uint32_t VMAXP = HS_VMAXP;

#ifndef HS_VLONG
#define HS_VLONG 256
#endif
constexpr uint32_t VLONG = HS_VLONG;  // merges of two sets at least this long run on the whole warp

// Shared-memory words one warp needs: the probe (pmax tokens), plus the
// staged candidate prefixes in mode 3.
__host__ __device__ constexpr uint32_t verify_smem_words(int vmode, uint32_t pmax = MAXP) {
    return pmax + (vmode == 3 ? 32 * VSTRIDE : 0);
}

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

// Verifies probe p of S against the n candidates cand_at(0..n-1) of R and
// appends (p, c) for every pair with overlap >= minoverlap.  VMODE 1: a lane
// per candidate; 2: the warp per candidate (merge-path steps of 32 tokens);
// 3: a lane per candidate, merging from 16-token prefixes staged with
// coalesced loads.  W > 0: before any merge, the XOR-signature bound of the
// reference's bitmap filter (|r ∩ s| <= (|r| + |s| - popc(b_r ^ b_s)) / 2,
// include/hyset/device_algorithms.hpp:104-113) drops candidates that cannot
// reach minoverlap (W words per signature in sig_R / sig_S); a round whose
// candidates all fail it stages and merges nothing, and the probe's tokens are
// staged only when a round first needs them.  The bound is sound, so the pairs
// do not change.  sbuf: this warp's verify_smem_words(VMODE, PMAX) words.
// All 32 lanes call it with the same arguments.
template <int VMODE, int W, uint32_t PMAX, typename CandAt>
__device__ __forceinline__ void verify_probe_list(const CollView& R, const CollView& S, const BoundsView& B,
                                                  const uint64_t* __restrict__ sig_R,
                                                  const uint64_t* __restrict__ sig_S, uint32_t p, CandAt cand_at,
                                                  uint32_t n, const Sink& out, uint32_t* sbuf, int lane) {
    const uint2 pm = S.meta[p];
    const uint32_t lp = pm.y;
    const uint32_t* pg = S.tokens + pm.x;
    const uint32_t* a = pg;
    bool staged = false;
    uint64_t ps[W > 0 ? W : 1];
    if constexpr (W > 0) {
#pragma unroll
        for (int w = 0; w < W; ++w) ps[w] = __ldg(sig_S + (uint64_t)p * W + w);
    }
    for (uint32_t k0 = 0; k0 < n; k0 += 32) {
        const uint32_t k = k0 + lane;
        bool keep = k < n;
        uint32_t c = 0, lc = 0, mo = 0, cs = 0;
        if (keep) {
            c = cand_at(k);
            const uint2 cm = R.meta[c];
            cs = cm.x;
            lc = cm.y;
            // hybrid_kernels.hpp:50: minoverlap(probe, candidate), for any pair
            // (an incompatible length pair gets min(lp, lc)).
            const uint32_t big = max(lp, lc), small = min(lp, lc);
            if (small >= B.minsize[big]) mo = minoverlap(B, big, small);
            else mo = small;
            if constexpr (W > 0) {
                uint32_t pop = 0;
                const uint64_t* bc = sig_R + (uint64_t)c * W;
                if constexpr (W % 2 == 0) {
#pragma unroll
                    for (int w = 0; w < W; w += 2) {
                        const ulonglong2 y = __ldg(reinterpret_cast<const ulonglong2*>(bc + w));
                        pop += __popcll(ps[w] ^ y.x) + __popcll(ps[w + 1] ^ y.y);
                    }
                } else {
#pragma unroll
                    for (int w = 0; w < W; ++w) pop += __popcll(ps[w] ^ __ldg(bc + w));
                }
                keep = lp + lc - pop >= 2u * mo;
            }
        }
        if constexpr (W > 0) {
            if (!__ballot_sync(FULL, keep)) continue;  // no candidate of the round can reach minoverlap
        }
        if (!staged) {  // the probe's tokens, once, when a round first merges
            if (lp <= PMAX) {
                for (uint32_t q = lane; q < lp; q += 32) sbuf[q] = pg[q];
                __syncwarp();
                a = sbuf;
            }
            staged = true;
        }
        // Long merges (both sets of at least VLONG tokens) run on the whole
        // warp in 32-token steps: a lane-serial merge of two similar sets of
        // 2,000 tokens holds its warp for about 4,000 dependent steps, and
        // one such pair at the end of a launch was its tail.
        const bool lng = VMODE != 2 && keep && min(lp, lc) >= VLONG;
        if (VMODE != 2) {
            unsigned ml = __ballot_sync(FULL, lng);
            while (ml) {
                const int src = __ffs(ml) - 1;
                ml &= ml - 1;
                const uint32_t cc = __shfl_sync(FULL, c, src), c2 = __shfl_sync(FULL, cs, src);
                const uint32_t ll = __shfl_sync(FULL, lc, src), mm = __shfl_sync(FULL, mo, src);
                const bool ok = verify_warp(a, lp, R.tokens + c2, ll, mm, NOWN, lane);
                emit(out, ok && lane == 0, p, cc, lane);
            }
            keep = keep && !lng;
        }
        if constexpr (VMODE == 1) {
            bool ok = keep && verify_serial(a, lp, R.tokens + cs, lc, mo, NOWN);
            emit(out, ok, p, c, lane);
        } else if constexpr (VMODE == 3) {
            // the first VSTAGE tokens of the round's 32 candidates arrive with
            // VSTAGE coalesced loads (32 / VSTAGE candidates per load, VSTAGE
            // lanes each); each lane then merges its candidate out of shared
            // memory and reads global memory only past the staged prefix
            uint32_t* tile = sbuf + PMAX;
            const uint32_t t = lane & (VSTAGE - 1);
            constexpr int PER = 32 / VSTAGE;  // candidates per load
#pragma unroll
            for (int r = 0; r < (int)VSTAGE; ++r) {
                const int j = PER * r + lane / (int)VSTAGE;
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

}  // namespace
}  // namespace hs
