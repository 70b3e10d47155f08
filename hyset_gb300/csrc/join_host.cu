// join_host.cu — one join: technique and configuration, index and
// signatures, the persistent filter + verify launch (re-run once with an
// exact buffer when the pairs overflowed), the optional device sort of the
// pairs, and the self-join / R-S join entry points.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "host.h"

namespace hs {

// Orders n result pairs by (probe id, indexed id) on the device, in place.
hyset_status sort_device_pairs(hyset_ctx* ctx, uint2* pairs, uint64_t n, uint32_t n_probe, uint32_t n_indexed) {
    if (n <= 1) return HYSET_OK;
    cudaStream_t s = ctx->stream;
    Scratch& sc = ctx->own;
    const size_t b = (size_t)n * 4;
    CK(sc.tok.ensure(b, s));
    CK(sc.set.ensure(b, s));
    CK(sc.altk.ensure(b, s));
    CK(sc.altv.ensure(b, s));
    CK(sc.scan.ensure(radix_scratch_words(n) * 4, s));
    CK(sort_pair_list(pairs, n, (int)bits_for(n_probe), (int)bits_for(n_indexed), sc.tok.as<uint32_t>(),
                      sc.set.as<uint32_t>(), sc.altk.as<uint32_t>(), sc.altv.as<uint32_t>(), sc.scan.as<uint32_t>(),
                      s));
    return HYSET_OK;
}

// R-S joins are symmetric in the two collections (the bounds take the larger
// and smaller size of a pair, both sides keep maxprefix tokens), so the
// collections' roles may be exchanged: the indexed side is the smaller one
// (a cheaper index build) and the probe side the larger one (more work units
// for the persistent launch).  Output pairs are written back in the caller's
// (probe, indexed) order.  Probe ranges shard the caller's probe side and keep
// the given orientation.
bool swap_sides(const hyset_coll* R, const hyset_coll* S, const hyset_join_opts* o) {
    if (R == S || o->probe_end) return false;
    if (o->orientation == 2) return true;
    return o->orientation == 0 && S->n < R->n;
}

// Runs one configured join launch into the context's pair buffer, growing the
// buffer and re-running when the first pass overflowed.
hyset_status run_join(hyset_ctx* ctx, JoinParams P, int tech, int vmode, const hyset_join_opts* o,
                      hyset_result* res, bool timed_from_ev0, TokenJoinParams* T) {
    cudaStream_t s = ctx->stream;
    const int count_only = o->count_only ? 1 : 0;
    uint64_t cap = o->pair_capacity ? o->pair_capacity : std::max<uint64_t>(1u << 20, 4ull * P.S.n);
    if (count_only) cap = 0;
    CK(ctx->s_count.ensure(16, s));
    CK(ctx->s_work.ensure(16, s));
    CK(ctx->s_stats.ensure(64, s));
    P.stats = o->collect_stats ? ctx->s_stats.as<unsigned long long>() : nullptr;
    for (int attempt = 0; attempt < 2; ++attempt) {
        if (!count_only) CK(ctx->s_pairs.ensure(std::max<uint64_t>(cap, 1) * sizeof(uint2), s));
        P.out.pairs = count_only ? nullptr : ctx->s_pairs.as<uint2>();
        P.out.count = ctx->s_count.as<unsigned long long>();
        P.out.cap = cap;
        P.out.count_only = count_only;
        P.work = ctx->s_work.as<unsigned int>();
        if (!timed_from_ev0 || attempt > 0) CK(cudaEventRecord(ctx->ev0, s));
        CK(cudaMemsetAsync(ctx->s_count.p, 0, 16, s));
        CK(cudaMemsetAsync(ctx->s_work.p, 0, 16, s));
        if (P.stats) CK(cudaMemsetAsync(P.stats, 0, 64, s));
        CK(cudaEventRecord(ctx->ek0, s));
        if (T) {
            T->out = P.out;
            T->work = P.work;
            T->stats = P.stats;
            CK(launch_join_tm(*T, ctx->sm_count, s));
        } else {
            CK(launch_join(P, tech, vmode, ctx->sm_count, s));
        }
        CK(cudaEventRecord(ctx->ek1, s));
        CK(cudaEventRecord(ctx->ev1, s));
        unsigned long long count = 0;
        CK(cudaMemcpyAsync(&count, ctx->s_count.p, 8, cudaMemcpyDeviceToHost, s));
        if (P.stats) CK(cudaMemcpyAsync(res->stats, P.stats, 64, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        float ms = 0, kms = 0;
        CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        CK(cudaEventElapsedTime(&kms, ctx->ek0, ctx->ek1));
        res->device_ms = ms;
        res->kernel_ms = kms;
        res->count = count;
        if (count_only || count <= cap) break;
        cap = count + count / 8 + 1024;  // overflow: retry once with room for everything
        if (attempt == 1) return fail(ctx, HYSET_E_OVERFLOW, "pair buffer overflow after resize");
    }
    return deliver_pairs(ctx, P, o, res);
}

void split_heavy(const hyset_coll* S, const Bounds* b, JoinParams& P) {
    constexpr uint32_t HEAVY_SLOTS = 128;  // probes with longer prefixes are split
    constexpr uint32_t SEG_SLOTS = 64;     // prefix slots per unit of a split probe
    P.heavy_from = 0xFFFFFFFFu;
    P.segs = 0;
    P.seg_slots = SEG_SLOTS;
    if (P.X2.set) return;  // banded R-S joins keep two lanes per probe
    const uint32_t L = std::min(S->max_size, b->L);
    for (uint32_t l = 0; l <= L; ++l)
        if (b->probe_prefix[l] > HEAVY_SLOTS) {
            P.heavy_from = S->h_first_ge[l];
            P.segs = (b->probe_prefix[L] + SEG_SLOTS - 1) / SEG_SLOTS;
            return;
        }
}

hyset_status deliver_pairs(hyset_ctx* ctx, const JoinParams& P, const hyset_join_opts* o, hyset_result* res) {
    cudaStream_t s = ctx->stream;
    const bool count_only = o->count_only != 0;
    if (!count_only && o->sort_pairs)
        ST(sort_device_pairs(ctx, ctx->s_pairs.as<uint2>(), res->count, P.out.swap ? P.R.n : P.S.n,
                             P.out.swap ? P.S.n : P.R.n));
    if (!count_only && o->device_pairs) {
        if (o->sort_pairs) CK(cudaStreamSynchronize(s));  // device pairs are final when the call returns
        res->device_pairs = ctx->s_pairs.p;
    } else if (!count_only) {
        res->pairs.resize(res->count);
        if (res->count)
            CK(cudaMemcpyAsync(res->pairs.data(), ctx->s_pairs.p, res->count * sizeof(hyset_pair),
                               cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        res->has_pairs = 1;
    }
    return HYSET_OK;
}

hyset_status do_join(hyset_ctx* ctx, hyset_coll* R, hyset_coll* S, const hyset_join_opts* o, hyset_result* res) {
    ST(check_opts(ctx, o));
    const bool swapped = swap_sides(R, S, o);
    if (swapped) std::swap(R, S);
    const bool self = (S == R);
    if (self) {
        uint32_t split_at = 0;
        hyset_technique low = HYSET_TECH_AUTO, high = HYSET_TECH_AUTO;
        ST(plan_split(ctx, R, o, &split_at, &low, &high));
        if (split_at) {  // two probe ranges, each with its technique; pairs of the low range first
            hyset_result part[2];
            for (int k = 0; k < 2; ++k) {
                hyset_join_opts q = *o;
                q.technique = k == 0 ? low : high;
                q.probe_major = 1;
                q.probe_begin = k == 0 ? 0 : split_at;
                q.probe_end = k == 0 ? split_at : R->n;
                ST(do_join(ctx, R, S, &q, &part[k]));
            }
            res->count = part[0].count + part[1].count;
            res->has_pairs = part[0].has_pairs;
            res->pairs = std::move(part[0].pairs);
            res->pairs.insert(res->pairs.end(), part[1].pairs.begin(), part[1].pairs.end());
            res->device_ms = part[0].device_ms + part[1].device_ms;
            res->kernel_ms = part[0].kernel_ms + part[1].kernel_ms;
            for (int k = 0; k < 8; ++k) res->stats[k] = part[0].stats[k] + part[1].stats[k];
            res->launches = part[0].launches + part[1].launches;
            res->technique = part[1].technique;
            res->bitmap_bits = part[1].bitmap_bits;
            res->verify_mode = part[1].verify_mode;
            res->probe_batch = part[1].probe_batch;
            res->selector = 2;
            res->split_at = split_at;
            res->split_low = part[0].technique;
            return HYSET_OK;
        }
    }
    const uint32_t L = std::max(R->max_size, S->max_size);
    Bounds* b = nullptr;
    ST(get_bounds(ctx, o->sim, o->threshold, L, self ? 0 : 1, &b));
    hyset_technique selected = HYSET_TECH_AUTO;
    ST(select_technique(ctx, R, S, o, &selected, &res->selector));
    Tuned tn = tune(R, S, o, selected);
    const hyset_technique tech = tn.tech;
    res->technique = tech;
    {
        const uint32_t a_lo = o->probe_end ? o->probe_begin : 0, a_hi = o->probe_end ? o->probe_end : S->n;
        if (o->technique == HYSET_TECH_AUTO && o->bitmap_bits == 0 && tech == HYSET_TECH_FGSS && tn.probe_major &&
            a_hi - a_lo >= TUNE_MIN_PROBES)
            ST(autotune_bits(ctx, R, S, o, b, self, a_lo, a_hi, &tn.bits, o->verify_mode ? nullptr : &tn.vmode,
                             o->fgss_batch ? nullptr : &tn.batch));
    }
    const int vmode = tn.vmode;
    res->verify_mode = (uint32_t)vmode;
    res->bitmap_bits = tech == HYSET_TECH_DIRECT ? 0 : (tn.bits > 512 && !(tech == HYSET_TECH_FGSS && tn.probe_major) ? 512 : tn.bits);
    if (o->probe_end > S->n || o->probe_begin > o->probe_end)
        return fail(ctx, HYSET_E_INVALID, "probe range outside the probe collection");
    const unsigned long long launches0 = launches();
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    JoinParams P{};
    P.R = R->view();
    P.S = S->view();
    P.B = b->view;
    P.first_ge = R->first_ge.as<uint32_t>();
    P.R_L = R->max_size;
    P.self = self ? 1 : 0;
    P.grab = tech == HYSET_TECH_FGSS ? std::min<uint32_t>(tn.batch, 32) : 1;
    res->probe_batch = tech == HYSET_TECH_FGSS && tn.probe_major ? P.grab : 0;
    P.p_lo = o->probe_end ? o->probe_begin : 0;
    P.p_hi = o->probe_end ? o->probe_end : S->n;
    P.r_lo = 0;
    P.r_hi = R->n;
    P.out.swap = swapped ? 1 : 0;
    const bool token_major = tech == HYSET_TECH_FGSS && L < 65536 && !tn.probe_major;
    uint64_t group_entries = 0;
    TokenJoinParams T{};
    if (token_major) {
        // probes: maxprefix entries of S; candidates: the same groups (self-join,
        // midprefix filter in the kernel) or R's maxprefix entries (R-S join)
        const uint32_t U = std::max(R->universe, S->universe);
        ST(build_groups(ctx, S, b->view.probe_prefix, b->probe_prefix, U, &group_entries));
        if (!self) {
            uint64_t er = 0;
            ST(build_groups(ctx, R, b->view.index_prefix, b->index_prefix, U, &er));
            group_entries += er;
        }
        T.R = R->view();
        T.S = S->view();
        T.B = b->view;
        T.gs_off = S->g_off.as<uint32_t>();
        T.gs_set = S->g_set.as<uint32_t>();
        T.gs_ps = S->g_ps.as<uint32_t>();
        T.gr_off = R->g_off.as<uint32_t>();
        T.gr_set = R->g_set.as<uint32_t>();
        T.gr_ps = R->g_ps.as<uint32_t>();
        T.universe = U;
        T.self = self ? 1 : 0;
        T.grab = 16;
    }
    // signatures do not depend on the index: they are generated on the
    // auxiliary stream while the index builds on the context's stream
    // 1024-bit signatures serve the probe-major prefix filter; the window
    // techniques and the token-major kernel take 512 at most
    const int words = (int)(tn.bits / 64) > 8 && !(tech == HYSET_TECH_FGSS && tn.probe_major) ? 8 : (int)(tn.bits / 64);
    if (words) {
        const uint64_t *br = nullptr, *bs = nullptr;
        ST(get_bitmaps(ctx, R, words, &br, ctx->aux));
        if (self) bs = br;
        else ST(get_bitmaps(ctx, S, words, &bs, ctx->aux));
        CK(cudaEventRecord(ctx->ev_join, ctx->aux));
        P.bits_R = br;
        P.bits_S = bs;
        P.words = words;
    }
    if (!token_major && tech == HYSET_TECH_FGSS) {
        ST(build_fgss_indexes(ctx, R, b, self, R->index, R->index_mid, P));
        if (P.X2.set) P.grab = std::min<uint32_t>(P.grab, 16);  // two bands per probe share a warp batch
        split_heavy(S, b, P);
    }
    if (words) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
    int ktech = tech == HYSET_TECH_FGSS ? TECH_FGSS : (tech == HYSET_TECH_DIRECT ? TECH_DIRECT : TECH_BITMAP);
    if (token_major) {
        T.bits_R = P.bits_R;
        T.bits_S = P.bits_S;
        T.words = P.words;
        if (o->probe_end && (o->probe_begin || o->probe_end != S->n))
            return fail(ctx, HYSET_E_UNSUPPORTED, "probe ranges need the probe-major kernel (probe_major = 1)");
        ST(run_join(ctx, P, ktech, vmode, o, res, true, &T));
        res->stats[3] = group_entries;
    } else {
        ST(run_join(ctx, P, ktech, vmode, o, res, true));
    }
    if (P.X.set && o->collect_stats && !token_major) {
        res->stats[3] = R->index.entries;
    }
    res->launches = launches() - launches0;
    return HYSET_OK;
}

}  // namespace hs

using namespace hs;

extern "C" {

hyset_status hyset_self_join(hyset_ctx* ctx, const hyset_coll* coll, const hyset_join_opts* opts,
                             hyset_result** out) {
    if (!ctx || !coll || !out) return fail(ctx, HYSET_E_INVALID, "null argument");
    *out = nullptr;
    CK(cudaSetDevice(ctx->device));
    auto res = std::make_unique<hyset_result>();
    hyset_coll* c = const_cast<hyset_coll*>(coll);  // caches (index, signatures) live in the collection
    ST(do_join(ctx, c, c, opts, res.get()));
    *out = res.release();
    return HYSET_OK;
}

hyset_status hyset_rs_join(hyset_ctx* ctx, const hyset_coll* indexed, const hyset_coll* probe,
                           const hyset_join_opts* opts, hyset_result** out) {
    if (!ctx || !indexed || !probe || !out) return fail(ctx, HYSET_E_INVALID, "null argument");
    *out = nullptr;
    CK(cudaSetDevice(ctx->device));
    auto res = std::make_unique<hyset_result>();
    hyset_coll* R = const_cast<hyset_coll*>(indexed);
    hyset_coll* S = const_cast<hyset_coll*>(probe);
    if (R == S) return fail(ctx, HYSET_E_INVALID, "use hyset_self_join for R join R");
    ST(do_join(ctx, R, S, opts, res.get()));
    *out = res.release();
    return HYSET_OK;
}

}  // extern "C"
