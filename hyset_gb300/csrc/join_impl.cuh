// join_impl.cuh — per-probe filter + verify routines of the single-join kernel
// (join.cu: fgss_carry, enum_probe) and the batched multi-join kernel
// (batch.cu: fgss_batch, enum_probe).
#pragma once
#include "kernels.h"

namespace hs {
namespace {

#ifndef HS_JOIN_MIN_BLOCKS
#define HS_JOIN_MIN_BLOCKS 5  // resident blocks per SM the join kernels are compiled for (48 registers)
#endif
#ifndef HS_JOIN_THREADS
#define HS_JOIN_THREADS 256  // threads per block of the join kernels
#endif
constexpr int JOIN_THREADS = HS_JOIN_THREADS;
constexpr int JOIN_WARPS = JOIN_THREADS / 32;
constexpr uint32_t MAXP = 768;       // probe tokens staged in shared memory per warp
#ifndef HS_JOIN_STEAL
#define HS_JOIN_STEAL 1  // probe batches taken per atomic on the work counter
#endif
#ifndef HS_SHORT_LIST
#define HS_SHORT_LIST 8
#endif

constexpr uint32_t SHORT_LIST = HS_SHORT_LIST;  // inverted lists this short are windowed without bisection

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

// ST (compile time): the launch collects work counters.  Without them the
// counter code is not compiled in at all.
template <bool ST>
__device__ __forceinline__ void count_stat(const JoinParams& P, int k, uint32_t v, int lane) {
    if constexpr (!ST) return;
    if (P.stats == nullptr) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    if (lane == 0 && v) atomicAdd(P.stats + k, (unsigned long long)v);
}

// Per-lane counter update (divergent-safe; stats runs only).
template <bool ST>
__device__ __forceinline__ void count_stat_lane(const JoinParams& P, int k, uint32_t v) {
    if constexpr (!ST) return;
    if (P.stats != nullptr && v) atomicAdd(P.stats + k, (unsigned long long)v);
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

// Stages the probe's tokens in this warp's shared-memory slot (once per probe,
// and only when an item survives the filters); long probes stay in HBM/L2.
__device__ __forceinline__ const uint32_t* stage_probe(const uint32_t* pg, uint32_t lp, uint32_t* sbuf,
                                                       bool& staged, int lane) {
    if (lp > MAXP) return pg;
    if (!staged) {
        for (uint32_t i = lane; i < lp; i += 32) sbuf[i] = pg[i];
        __syncwarp();
        staged = true;
    }
    return sbuf;
}

template <int W>
__device__ __forceinline__ uint32_t bitmap_xor_pop(const JoinParams& P, const uint64_t (&bp)[W], uint32_t c) {
    uint32_t pop = 0;
    const uint64_t* bc = P.bits_R + (uint64_t)c * W;
#pragma unroll
    for (int q = 0; q < W; ++q) pop += __popcll(bp[q] ^ __ldg(bc + q));
    return pop;
}

// Verifies the warp's surviving items and appends the accepted pairs.
// own_a / own_b: the item's position in the probe / candidate (ownership test)
// or NOWN.
template <int VMODE, bool ST>
__device__ __forceinline__ void verify_and_emit(const JoinParams& P, uint32_t p, const uint32_t* pg, uint32_t lp,
                                                uint32_t* sbuf, bool& staged, bool keep, uint32_t cstart,
                                                uint32_t c, uint32_t lc, uint32_t mo, uint32_t own_a,
                                                uint32_t own_b, int lane) {
    unsigned m = __ballot_sync(FULL, keep);
    uint32_t used = 0;
    if (m) {
        const bool before = staged;
        const uint32_t* a = stage_probe(pg, lp, sbuf, staged, lane);
        if (!before) count_stat<ST>(P, 4, lane == 0 ? lp : 0u, lane);  // probe tokens read for verification
        if constexpr (VMODE == 1) {
            bool ok = false;
            if (keep) ok = verify_serial(a, lp, P.R.tokens + cstart, lc, mo, own_a, &used);
            emit(P.out, ok, p, c, lane);
        } else {
            while (m) {
                int src = __ffs(m) - 1;
                m &= m - 1;
                uint32_t cc = __shfl_sync(FULL, c, src);
                uint32_t cs = __shfl_sync(FULL, cstart, src);
                uint32_t ll = __shfl_sync(FULL, lc, src);
                uint32_t mm = __shfl_sync(FULL, mo, src);
                uint32_t ob = __shfl_sync(FULL, own_b, src);
                uint32_t u = 0;
                bool ok = verify_warp(a, lp, P.R.tokens + cs, ll, mm, ob, lane, &u);
                if (lane == 0) used += u;
                emit(P.out, ok && lane == 0, p, cc, lane);
            }
        }
    }
    count_stat<ST>(P, 6, used, lane);
}

// Hamming distance of two W-word signatures.  A set's signature starts on a
// multiple of 8 W bytes (the array is 256-byte aligned), so for even W the
// words are read 16 bytes at a time.
template <int W>
__device__ __forceinline__ uint32_t sig_distance(const uint64_t* __restrict__ a, const uint64_t* __restrict__ b) {
    uint32_t pop = 0;
    if constexpr (W % 2 == 0) {
#pragma unroll
        for (int w = 0; w < W; w += 2) {
            const ulonglong2 x = __ldg(reinterpret_cast<const ulonglong2*>(a + w));
            const ulonglong2 y = __ldg(reinterpret_cast<const ulonglong2*>(b + w));
            pop += __popcll(x.x ^ y.x) + __popcll(x.y ^ y.y);
        }
    } else {
#pragma unroll
        for (int w = 0; w < W; ++w) pop += __popcll(__ldg(a + w) ^ __ldg(b + w));
    }
    return pop;
}

// One 32-byte load (sm_100 and later), non-coherent path: p must be 32-byte aligned.
__device__ __forceinline__ void ldg256(const uint32_t* p, uint32_t (&w)[8]) {
    asm("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]), "=r"(w[7])
        : "l"(p));
}

// Window [klo, khi) of a token record (length word, then ascending entries
// padded with 0xFFFFFFFF; 128-byte aligned): the entries below each bound,
// counted over 32-byte pieces of the one line, the first piece giving the
// length and the others read only as far as it reaches (no search).
__device__ __forceinline__ void record_window(const uint32_t* __restrict__ r, uint32_t klo, uint32_t khi,
                                              uint32_t& nlo, uint32_t& nhi) {
    uint32_t w[8];
    ldg256(r, w);
    const uint32_t len = w[0];
    nlo = 0;
    nhi = 0;
#pragma unroll
    for (int q = 1; q < 8; ++q) {
        nlo += w[q] < klo;
        nhi += w[q] < khi;
    }
#pragma unroll
    for (int k = 1; k < 4; ++k) {
        if (len > 8u * k - 1u) {
            ldg256(r + 8 * k, w);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                nlo += w[q] < klo;
                nhi += w[q] < khi;
            }
        }
    }
}

// Lane k of the warp holds the k-th value of a non-decreasing inclusive scan;
// returns the first lane whose value exceeds q (q < the warp total).
__device__ __forceinline__ int scan_owner(uint32_t incl, uint32_t q) {
    int jj = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
        uint32_t v = __shfl_sync(FULL, incl, jj + step - 1);
        if (v <= q) jj += step;
    }
    return jj;
}

// FGSS for a batch of up to 32 probes per warp.  The probes' prefix slots
// (probe, position) are flattened across lanes, then the index entries their
// inverted lists contribute; every round trip to memory is shared by the whole
// batch, so a warp keeps several probes' loads in flight at once.
//
// Banded R-S joins (P.X2.set != nullptr, k <= 16): lane t < k takes the
// candidates of probe t at least as long as the probe (its midprefix tokens
// against the maxprefix index X), lane k + t the shorter ones (its maxprefix
// tokens against the midprefix index X2).
// RC: the index may be token records (IndexView::rec, checked per launch);
// without it the record path is not compiled.
template <int VMODE, int W, bool ST, bool RC = true, bool BD = false>
__device__ void fgss_batch(const JoinParams& P, uint32_t i0, uint32_t k, int lane) {
    // lane t < k: probe t of the batch (largest sets first)
    uint32_t p = 0, lp = 0, pst = 0, mp = 0, lo = 0, hi = 0, band = 0;
    const bool banded = P.X2.set != nullptr;
    const uint32_t t_probe = banded && (uint32_t)lane >= k ? (uint32_t)lane - k : (uint32_t)lane;
    if (t_probe < k && (banded || (uint32_t)lane < k)) {
        band = (uint32_t)lane >= k ? 1u : 0u;
        p = P.p_hi - 1 - (i0 + t_probe);
        const uint2 pm = P.S.meta[p];
        lp = pm.y;
        pst = pm.x;
        if (lp) {
            const Window w = candidate_window(P, p, lp);
            lo = w.lo;
            hi = w.hi;
            if (banded) {
                const uint32_t mid = P.first_ge[min(lp, P.R_L + 1)];  // first candidate with size >= lp
                if (band == 0) lo = max(lo, mid);
                else hi = min(hi, mid);
            }
            if (lo < hi) mp = banded && band == 0 ? P.B.mid_prefix[lp] : P.B.probe_prefix[lp];
        }
    }
    count_stat<ST>(P, 4, mp, lane);  // prefix tokens read by the filter
    const uint32_t mp_incl = warp_incl_scan(mp, lane);
    const uint32_t slots = __shfl_sync(FULL, mp_incl, 31);
    for (uint32_t s0 = 0; s0 < slots; s0 += 32) {
        // ---- slot = (probe t, prefix position j): window of the token's list
        const uint32_t sl = s0 + lane;
        const bool sv = sl < slots;
        const int t = scan_owner(mp_incl, sv ? sl : 0);
        const uint32_t t_incl = __shfl_sync(FULL, mp_incl, t), t_mp = __shfl_sync(FULL, mp, t);
        const uint32_t j = (sv ? sl : 0) - (t_incl - t_mp);
        const uint32_t t_pst = __shfl_sync(FULL, pst, t);
        const uint32_t t_lo = __shfl_sync(FULL, lo, t), t_hi = __shfl_sync(FULL, hi, t);
        const uint32_t t_band = __shfl_sync(FULL, band, t);
        const uint32_t* __restrict__ x_off = t_band ? P.X2.list_off : P.X.list_off;
        const uint32_t* __restrict__ x_set = t_band ? P.X2.set : P.X.set;
        uint32_t first = 0, cnt = 0;
        if (sv) {
            const uint32_t tok = __ldg(P.S.tokens + t_pst + j);
            if (RC && tok < P.X.universe && (t_band ? P.X2.rec : P.X.rec)) {
                static_assert(REC_CAP == 32, "record_window reads four 32-byte pieces");
                const uint32_t klo = t_lo << P.X.pos_bits, khi = t_hi << P.X.pos_bits;
                uint32_t nlo, nhi;
                record_window(x_set + ((uint64_t)tok << 5), klo, khi, nlo, nhi);
                first = (tok << 5) + 1 + nlo;
                cnt = nhi - nlo;
            } else if (tok < P.X.universe) {
                uint32_t b0 = x_off[tok], b1 = x_off[tok + 1];
                if (P.X.sorted) {
                    const uint32_t klo = t_lo << P.X.pos_bits, khi = t_hi << P.X.pos_bits;
                    const uint32_t len = b1 - b0;
                    if (len <= SHORT_LIST) {
                        // one round trip: independent loads instead of dependent bisection
                        uint32_t v[SHORT_LIST];
#pragma unroll
                        for (int q = 0; q < (int)SHORT_LIST; ++q)
                            v[q] = (uint32_t)q < len ? __ldg(x_set + b0 + q) : 0xFFFFFFFFu;
                        uint32_t nlo = 0, nhi = 0;
#pragma unroll
                        for (int q = 0; q < (int)SHORT_LIST; ++q) {
                            nlo += v[q] < klo;
                            nhi += v[q] < khi;
                        }
                        b1 = b0 + nhi;
                        b0 = b0 + nlo;
                    } else {
                        lower_bound2_u32(x_set, b0, b1, klo, khi, b0, b1);
                    }
                }
                first = b0;
                cnt = b1 - b0;
            }
        }
        const uint32_t incl = warp_incl_scan(cnt, lane);
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        for (uint32_t q0 = 0; q0 < total; q0 += 32) {
            // ---- item = one index entry of one slot
            const uint32_t q = q0 + lane;
            bool keep = q < total;
            const int jj = scan_owner(incl, keep ? q : 0);
            const uint32_t f_jj = __shfl_sync(FULL, first, jj);
            const uint32_t i_jj = __shfl_sync(FULL, incl, jj);
            const uint32_t c_jj = __shfl_sync(FULL, cnt, jj);
            const uint32_t jp = __shfl_sync(FULL, j, jj);
            const int it = __shfl_sync(FULL, t, jj);
            const uint32_t ip = __shfl_sync(FULL, p, it);
            const uint32_t ilp = __shfl_sync(FULL, lp, it);
            const uint32_t ipst = __shfl_sync(FULL, pst, it);
            const uint32_t ilo = __shfl_sync(FULL, lo, it), ihi = __shfl_sync(FULL, hi, it);
            const uint32_t iband = __shfl_sync(FULL, band, it);
            const uint32_t e = f_jj + ((keep ? q : 0) - (i_jj - c_jj));
            uint32_t c = 0, pc = 0, lc = 0, mo = 0, cstart = 0, pop = 0;
            if (keep) {
                const uint32_t v = (iband ? P.X2.set : P.X.set)[e];
                if (P.X.pos) {
                    c = v;
                    pc = (iband ? P.X2.pos : P.X.pos)[e];
                } else {
                    c = v >> P.X.pos_bits;
                    pc = v & ((1u << P.X.pos_bits) - 1u);
                }
                if (!P.X.sorted) keep = c >= ilo && c < ihi;
                if constexpr (BD) keep = keep && ilp <= pc;  // pc: the longest probe the entry admits
            }
            // Signatures up to 256 bits are loaded with the candidate's meta (one
            // round trip); wider ones only for items that pass the positional
            // bound (their reads outweigh the extra round trip).
            constexpr bool early_sig = W > 0 && W <= 4;
            if (keep) {
                const uint2 cm = P.R.meta[c];
                if constexpr (early_sig) {
                    pop = sig_distance<W>(P.bits_S + (uint64_t)ip * W, P.bits_R + (uint64_t)c * W);
                }
                cstart = cm.x;
                lc = cm.y;
                const uint32_t big = max(ilp, lc), small = min(ilp, lc);
                mo = minoverlap(P.B, big, small);
                keep = BD ? ilp - jp >= mo : 1u + min(ilp - jp - 1u, lc - pc - 1u) >= mo;  // positional bound
            }
            count_stat<ST>(P, 0, q < total ? 1u : 0u, lane);
            count_stat<ST>(P, 5, (W > 0 && keep) ? 1u : 0u, lane);
            if constexpr (W > 4) {
                if (keep) pop = sig_distance<W>(P.bits_S + (uint64_t)ip * W, P.bits_R + (uint64_t)c * W);
            }
            if constexpr (W > 0) keep = keep && ilp + lc - pop >= 2u * mo;

            count_stat<ST>(P, 1, keep ? 1u : 0u, lane);
            count_stat<ST>(P, 2, keep ? lc : 0u, lane);
            // ---- verification: the probe is read from HBM/L2 (it was just touched)
            uint32_t used = 0;
            const uint32_t* a = P.S.tokens + ipst;
            if constexpr (VMODE == 1) {
                bool ok = false;
                if (keep) ok = verify_serial(a, ilp, P.R.tokens + cstart, lc, mo, jp, &used);
                emit(P.out, ok, ip, c, lane);
            } else {
                unsigned m = __ballot_sync(FULL, keep);
                while (m) {
                    const int src = __ffs(m) - 1;
                    m &= m - 1;
                    const uint32_t cc = __shfl_sync(FULL, c, src), cs = __shfl_sync(FULL, cstart, src);
                    const uint32_t ll = __shfl_sync(FULL, lc, src), mm = __shfl_sync(FULL, mo, src);
                    const uint32_t ob = __shfl_sync(FULL, BD ? jp : pc, src), pp = __shfl_sync(FULL, ip, src);
                    const uint32_t pl = __shfl_sync(FULL, ilp, src), ps = __shfl_sync(FULL, ipst, src);
                    uint32_t u = 0;
                    const bool ok = BD
                                        ? verify_warp(P.R.tokens + cs, ll, P.S.tokens + ps, pl, mm, ob, lane, &u)
                                        : verify_warp(P.S.tokens + ps, pl, P.R.tokens + cs, ll, mm, ob, lane, &u);
                    if (lane == 0) used += u;
                    emit(P.out, ok && lane == 0, pp, cc, lane);
                }
            }
            count_stat<ST>(P, 6, used, lane);
        }
    }
}

// ---- probe-major FGSS with full item rounds ---------------------------------
//
// fgss_batch runs the items of each slot round as soon as the round is
// windowed, so most item rounds are partial (about 1.1 items per slot: one
// full round and one of a few items per slot round, half the lanes idle).
// fgss_carry keeps the last partial round's items in the lanes instead, each
// lane holding everything its item needs (candidate, positions, probe id,
// length and token offset), and fills the rest of the round from the next
// slot round, or the next probe batch of the same launch: only full rounds
// run until the warp's work ends (flush_items).

constexpr uint32_t NO_ITEM = 0xFFFFFFFFu;

struct ItemLane {  // one lane's pending item (c == NO_ITEM: none)
    uint32_t c = NO_ITEM, pc = 0, jp = 0, ip = 0, ilp = 0, ipst = 0;
};

// Filters and verifies one round of items (the lanes whose c != NO_ITEM) and
// appends the accepted pairs; every lane's item is consumed.
template <int VMODE, int W, bool ST, bool BD>
__device__ __forceinline__ void run_items(const JoinParams& P, ItemLane& it, int lane) {
    bool keep = it.c != NO_ITEM;
    const uint32_t c = keep ? it.c : 0u, pc = it.pc, jp = it.jp, ip = it.ip, ilp = it.ilp;
    uint32_t lc = 0, mo = 0, cstart = 0, pop = 0;
    count_stat<ST>(P, 0, keep ? 1u : 0u, lane);
    // as in fgss_batch; with bound-layout entries almost every item here has
    // passed the positional bound already, so every width loads early
    constexpr bool early_sig = W > 0 && (W <= 4 || BD);
    if (keep) {
        const uint2 cm = P.R.meta[c];
        if constexpr (early_sig) pop = sig_distance<W>(P.bits_S + (uint64_t)ip * W, P.bits_R + (uint64_t)c * W);
        cstart = cm.x;
        lc = cm.y;
        const uint32_t big = max(ilp, lc), small = min(ilp, lc);
        mo = minoverlap(P.B, big, small);
        // positional bound; with bound-layout entries the candidate's side was
        // checked when the item was taken
        keep = BD ? ilp - jp >= mo : 1u + min(ilp - jp - 1u, lc - pc - 1u) >= mo;
    }
    count_stat<ST>(P, 5, (W > 0 && keep) ? 1u : 0u, lane);
    if constexpr (W > 4) {
        if (keep) pop = sig_distance<W>(P.bits_S + (uint64_t)ip * W, P.bits_R + (uint64_t)c * W);
    }
    if constexpr (W > 0) keep = keep && ilp + lc - pop >= 2u * mo;
    count_stat<ST>(P, 1, keep ? 1u : 0u, lane);
    count_stat<ST>(P, 2, keep ? lc : 0u, lane);
    uint32_t used = 0;
    if constexpr (VMODE == 1) {
        bool ok = false;
        if (keep) ok = verify_serial(P.S.tokens + it.ipst, ilp, P.R.tokens + cstart, lc, mo, jp, &used);
        emit(P.out, ok, ip, c, lane);
    } else {
        unsigned m = __ballot_sync(FULL, keep);
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const uint32_t cc = __shfl_sync(FULL, c, src), cs = __shfl_sync(FULL, cstart, src);
            const uint32_t ll = __shfl_sync(FULL, lc, src), mm = __shfl_sync(FULL, mo, src);
            const uint32_t ob = __shfl_sync(FULL, BD ? jp : pc, src), pp = __shfl_sync(FULL, ip, src);
            const uint32_t pl = __shfl_sync(FULL, ilp, src), ps = __shfl_sync(FULL, it.ipst, src);
            uint32_t u = 0;
            // ownership by the candidate's position, or (bound layout: no
            // candidate position) by the probe's, with the merge's sides swapped
            const bool ok = BD ? verify_warp(P.R.tokens + cs, ll, P.S.tokens + ps, pl, mm, ob, lane, &u)
                                      : verify_warp(P.S.tokens + ps, pl, P.R.tokens + cs, ll, mm, ob, lane, &u);
            if (lane == 0) used += u;
            emit(P.out, ok && lane == 0, pp, cc, lane);
        }
    }
    count_stat<ST>(P, 6, used, lane);
    it.c = NO_ITEM;
}

// The pending items of a warp (fewer than 32) and how many there are.
// Bound-layout indexes keep them in the warp's shared-memory queue instead
// (QSLOTS slots of the fields below, one array per field), because the items
// that pass the candidate's side of the positional bound are compacted there.
struct ItemCarry {
    ItemLane lane_item;
    uint32_t pending = 0;  // warp-uniform: lanes [0, pending) hold an item (or queue slots [0, pending))
    uint32_t* q = nullptr;  // the warp's queue (bound layout)
};
constexpr uint32_t QSLOTS = 64;  // pending (< 32) plus one window's survivors (<= 32)
enum : uint32_t { QF_C = 0, QF_JP, QF_IP, QF_ILP, QF_IPST, QF_N };

__device__ __forceinline__ ItemLane queue_item(const uint32_t* q, uint32_t slot) {
    ItemLane x;
    x.c = q[QF_C * QSLOTS + slot];
    x.pc = 0;
    x.jp = q[QF_JP * QSLOTS + slot];
    x.ip = q[QF_IP * QSLOTS + slot];
    x.ilp = q[QF_ILP * QSLOTS + slot];
    x.ipst = q[QF_IPST * QSLOTS + slot];
    return x;
}

template <int VMODE, int W, bool ST, bool BD>
__device__ __forceinline__ void flush_items(const JoinParams& P, ItemCarry& ic, int lane) {
    if constexpr (BD) {
        if (ic.pending) {
            ItemLane x;
            if ((uint32_t)lane < ic.pending) x = queue_item(ic.q, lane);
            run_items<VMODE, W, ST, BD>(P, x, lane);
        }
    } else {
        if (ic.pending) run_items<VMODE, W, ST, BD>(P, ic.lane_item, lane);
    }
    ic.pending = 0;
}

// [jb, je): the prefix slots of each probe to run (all by default; a heavy
// probe's segment otherwise).
template <int VMODE, int W, bool ST, bool BD>
__device__ void fgss_carry(const JoinParams& P, uint32_t i0, uint32_t k, int lane, ItemCarry& ic, uint32_t jb = 0,
                           uint32_t je = 0xFFFFFFFFu) {
    // probes as in fgss_batch: lane t < k (banded R-S: lanes k + t too)
    uint32_t p = 0, lp = 0, pst = 0, mp = 0, lo = 0, hi = 0, band = 0;
    const bool banded = P.X2.set != nullptr;
    const uint32_t t_probe = banded && (uint32_t)lane >= k ? (uint32_t)lane - k : (uint32_t)lane;
    if (t_probe < k && (banded || (uint32_t)lane < k)) {
        band = (uint32_t)lane >= k ? 1u : 0u;
        p = P.p_hi - 1 - (i0 + t_probe);
        const uint2 pm = P.S.meta[p];
        lp = pm.y;
        pst = pm.x;
        if (lp) {
            const Window w = candidate_window(P, p, lp);
            lo = w.lo;
            hi = w.hi;
            if (banded) {
                const uint32_t mid = P.first_ge[min(lp, P.R_L + 1)];
                if (band == 0) lo = max(lo, mid);
                else hi = min(hi, mid);
            }
            if (lo < hi) mp = banded && band == 0 ? P.B.mid_prefix[lp] : P.B.probe_prefix[lp];
            mp = min(mp, je);
            mp = mp > jb ? mp - jb : 0u;  // the slots [jb, je) of the prefix
        }
    }
    count_stat<ST>(P, 4, mp, lane);
    const uint32_t mp_incl = warp_incl_scan(mp, lane);
    const uint32_t slots = __shfl_sync(FULL, mp_incl, 31);
    for (uint32_t s0 = 0; s0 < slots; s0 += 32) {
        // ---- slot = (probe t, prefix position j): window of the token's list
        const uint32_t sl = s0 + lane;
        const bool sv = sl < slots;
        const int t = scan_owner(mp_incl, sv ? sl : 0);
        const uint32_t t_incl = __shfl_sync(FULL, mp_incl, t), t_mp = __shfl_sync(FULL, mp, t);
        const uint32_t j = (sv ? sl : 0) - (t_incl - t_mp) + jb;
        const uint32_t t_pst = __shfl_sync(FULL, pst, t);
        const uint32_t t_lo = __shfl_sync(FULL, lo, t), t_hi = __shfl_sync(FULL, hi, t);
        const uint32_t t_band = __shfl_sync(FULL, band, t);
        const uint32_t* __restrict__ x_off = t_band ? P.X2.list_off : P.X.list_off;
        const uint32_t* __restrict__ x_set = t_band ? P.X2.set : P.X.set;
        uint32_t first = 0, cnt = 0;
        if (sv) {
            const uint32_t tok = __ldg(P.S.tokens + t_pst + j);
            if (tok < P.X.universe && (t_band ? P.X2.rec : P.X.rec)) {
                const uint32_t klo = t_lo << P.X.pos_bits, khi = t_hi << P.X.pos_bits;
                uint32_t nlo, nhi;
                record_window(x_set + ((uint64_t)tok << 5), klo, khi, nlo, nhi);
                first = (tok << 5) + 1 + nlo;
                cnt = nhi - nlo;
            } else if (tok < P.X.universe) {
                uint32_t b0 = x_off[tok], b1 = x_off[tok + 1];
                if (P.X.sorted) {
                    const uint32_t klo = t_lo << P.X.pos_bits, khi = t_hi << P.X.pos_bits;
                    const uint32_t len = b1 - b0;
                    if (len <= SHORT_LIST) {
                        uint32_t v[SHORT_LIST];
#pragma unroll
                        for (int q = 0; q < (int)SHORT_LIST; ++q)
                            v[q] = (uint32_t)q < len ? __ldg(x_set + b0 + q) : 0xFFFFFFFFu;
                        uint32_t nlo = 0, nhi = 0;
#pragma unroll
                        for (int q = 0; q < (int)SHORT_LIST; ++q) {
                            nlo += v[q] < klo;
                            nhi += v[q] < khi;
                        }
                        b1 = b0 + nhi;
                        b0 = b0 + nlo;
                    } else {
                        lower_bound2_u32(x_set, b0, b1, klo, khi, b0, b1);
                    }
                }
                first = b0;
                cnt = b1 - b0;
            }
        }
        const uint32_t incl = warp_incl_scan(cnt, lane);
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        if constexpr (BD) {
            // ---- bound layout: 32 of the round's items at a time are checked
            // against the candidate's side of the positional bound (the entry
            // carries the longest probe it admits); the survivors are appended
            // to the warp's queue and every full round of 32 runs
            uint32_t* q = ic.q;
            for (uint32_t taken = 0; taken < total; taken += 32) {
                const uint32_t qi = taken + (uint32_t)lane;
                const bool has = qi < total;
                const int jj = scan_owner(incl, has ? qi : 0u);
                const uint32_t f_jj = __shfl_sync(FULL, first, jj);
                const uint32_t i_jj = __shfl_sync(FULL, incl, jj);
                const uint32_t c_jj = __shfl_sync(FULL, cnt, jj);
                const uint32_t jp = __shfl_sync(FULL, j, jj);
                const int it = __shfl_sync(FULL, t, jj);
                const uint32_t ip = __shfl_sync(FULL, p, it);
                const uint32_t ilp = __shfl_sync(FULL, lp, it);
                const uint32_t ipst = __shfl_sync(FULL, pst, it);
                bool ok = false;
                uint32_t c = 0;
                count_stat<ST>(P, 7, has ? 1u : 0u, lane);  // index entries in windows, before the bound
                if (has) {
                    const uint32_t v = x_set[f_jj + (qi - (i_jj - c_jj))];
                    c = v >> P.X.pos_bits;
                    ok = ilp <= (v & ((1u << P.X.pos_bits) - 1u));
                }
                const unsigned m = __ballot_sync(FULL, ok);
                if (ok) {
                    const uint32_t slot = ic.pending + __popc(m & lanemask_lt(lane));
                    q[QF_C * QSLOTS + slot] = c;
                    q[QF_JP * QSLOTS + slot] = jp;
                    q[QF_IP * QSLOTS + slot] = ip;
                    q[QF_ILP * QSLOTS + slot] = ilp;
                    q[QF_IPST * QSLOTS + slot] = ipst;
                }
                ic.pending += __popc(m);
                __syncwarp();
                if (ic.pending >= 32u) {
                    ItemLane x = queue_item(q, lane);
                    // slots [32, pending) move to the front for the next round
                    const uint32_t rest = ic.pending - 32u;
                    ItemLane y;
                    if ((uint32_t)lane < rest) y = queue_item(q, 32u + lane);
                    __syncwarp();
                    if ((uint32_t)lane < rest) {
                        q[QF_C * QSLOTS + lane] = y.c;
                        q[QF_JP * QSLOTS + lane] = y.jp;
                        q[QF_IP * QSLOTS + lane] = y.ip;
                        q[QF_ILP * QSLOTS + lane] = y.ilp;
                        q[QF_IPST * QSLOTS + lane] = y.ipst;
                    }
                    ic.pending = rest;
                    __syncwarp();
                    run_items<VMODE, W, ST, BD>(P, x, lane);
                }
            }
        } else {
        // ---- the round's items join the pending ones; every full round runs
        uint32_t taken = 0;
        while (taken < total) {
            const uint32_t room = 32u - ic.pending;
            const uint32_t take = min(room, total - taken);
            // lanes [pending, pending + take) take items taken .. taken + take - 1
            const bool mine = (uint32_t)lane >= ic.pending && (uint32_t)lane < ic.pending + take;
            const uint32_t q = mine ? taken + (uint32_t)lane - ic.pending : 0u;
            const int jj = scan_owner(incl, q);
            const uint32_t f_jj = __shfl_sync(FULL, first, jj);
            const uint32_t i_jj = __shfl_sync(FULL, incl, jj);
            const uint32_t c_jj = __shfl_sync(FULL, cnt, jj);
            const uint32_t jp = __shfl_sync(FULL, j, jj);
            const int it = __shfl_sync(FULL, t, jj);
            const uint32_t ip = __shfl_sync(FULL, p, it);
            const uint32_t ilp = __shfl_sync(FULL, lp, it);
            const uint32_t ipst = __shfl_sync(FULL, pst, it);
            const uint32_t ilo = __shfl_sync(FULL, lo, it), ihi = __shfl_sync(FULL, hi, it);
            const uint32_t iband = __shfl_sync(FULL, band, it);
            if (mine) {
                const uint32_t e = f_jj + (q - (i_jj - c_jj));
                const uint32_t v = (iband ? P.X2.set : P.X.set)[e];
                uint32_t c, pc;
                if (P.X.pos) {
                    c = v;
                    pc = (iband ? P.X2.pos : P.X.pos)[e];
                } else {
                    c = v >> P.X.pos_bits;
                    pc = v & ((1u << P.X.pos_bits) - 1u);
                }
                ItemLane& x = ic.lane_item;
                x.c = (!P.X.sorted && (c < ilo || c >= ihi)) ? NO_ITEM : c;
                x.pc = pc;
                x.jp = jp;
                x.ip = ip;
                x.ilp = ilp;
                x.ipst = ipst;
            }
            taken += take;
            ic.pending += take;
            if (ic.pending == 32u) {
                run_items<VMODE, W, ST, BD>(P, ic.lane_item, lane);
                ic.pending = 0;
            }
        }
        }  // BD
    }
}

template <int VMODE, int W, bool ST>
__device__ void enum_probe(const JoinParams& P, uint32_t p, uint32_t* sbuf, int lane) {
    const uint2 pm = P.S.meta[p];
    const uint32_t lp = pm.y;
    if (lp == 0) return;
    const Window win = candidate_window(P, p, lp);
    if (win.lo >= win.hi) return;
    const uint32_t* pg = P.S.tokens + pm.x;
    bool staged = false;
    uint64_t bp[W > 0 ? W : 1];
    if constexpr (W > 0) {
#pragma unroll
        for (int q = 0; q < W; ++q) bp[q] = __ldg(P.bits_S + (uint64_t)p * W + q);
    }
    for (uint32_t c0 = win.lo; c0 < win.hi; c0 += 32) {
        const uint32_t c = c0 + lane;
        bool keep = c < win.hi;
        uint32_t lc = 0, mo = 0, cstart = 0;
        if (keep) {
            const uint2 cm = P.R.meta[c];
            cstart = cm.x;
            lc = cm.y;
            const uint32_t big = max(lp, lc), small = min(lp, lc);
            mo = minoverlap(P.B, big, small);
            keep = bitmap_pass<W>(P, bp, c, lp, lc, mo);
        }
        count_stat<ST>(P, 0, c < win.hi ? 1u : 0u, lane);
        count_stat<ST>(P, 5, (W > 0 && c < win.hi) ? 1u : 0u, lane);
        count_stat<ST>(P, 1, keep ? 1u : 0u, lane);
        count_stat<ST>(P, 2, keep ? lc : 0u, lane);
        verify_and_emit<VMODE, ST>(P, p, pg, lp, sbuf, staged, keep, cstart, c, lc, mo, NOWN, NOWN, lane);
    }
    __syncwarp();
}

}  // namespace
}  // namespace hs
