// capi.cu — the C ABI (include/hyset_gb300.h): contexts, collections, bound
// tables, index builds, joins, the reference-shaped handlers and the candidate
// verifier.  Host code; every device step runs on the context's stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "internal.h"

using namespace hs;

namespace {

// ---------------------------------------------------------------- errors
hyset_status fail(hyset_ctx* ctx, hyset_status st, const char* what, cudaError_t e = cudaSuccess) {
    if (ctx) {
        char buf[512];
        if (e != cudaSuccess)
            std::snprintf(buf, sizeof buf, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
        else
            std::snprintf(buf, sizeof buf, "%s", what);
        ctx->err = buf;
    }
    return st;
}

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t _e = (call);                                                        \
        if (_e != cudaSuccess)                                                          \
            return fail(ctx, _e == cudaErrorMemoryAllocation ? HYSET_E_NOMEM : HYSET_E_CUDA, #call, _e); \
    } while (0)

#define ST(call)                                \
    do {                                        \
        hyset_status _s = (call);               \
        if (_s != HYSET_OK) return _s;          \
    } while (0)

// ---------------------------------------------------------------- bounds
// The reference's similarity bounds (include/hyset/similarity.hpp:11-54) in the
// same double expressions; this translation unit is compiled without
// multiply-add contraction so the doubles match the reference bit for bit.
// Cosine and dice have no reference code and follow the same style.
int imin(int a, int b) { return (a > b) ? b : a; }

uint32_t sim_minoverlap(int sim, uint32_t l1, uint32_t l2, double t) {
    switch (sim) {
    case SIM_COSINE: return (uint32_t)(std::ceil(t * std::sqrt((double)l1 * (double)l2)));
    case SIM_DICE: return (uint32_t)(std::ceil(t * (double)(l1 + l2) / 2.0));
    default: return (uint32_t)(std::ceil((double)(l1 + l2) * t / (1 + t)));
    }
}
uint32_t minsize_of(int sim, uint32_t len, double t) {
    switch (sim) {
    case SIM_COSINE: return (uint32_t)(std::ceil(t * t * (double)len));
    case SIM_DICE: return (uint32_t)(std::ceil(t * (double)len / (2.0 - t)));
    default: return (uint32_t)(std::ceil(t * (double)len));
    }
}
uint32_t minoverlap_of(int sim, uint32_t l1, uint32_t l2, double t) {
    return (uint32_t)imin((int)l2, imin((int)l1, (int)sim_minoverlap(sim, l1, l2, t)));
}
uint32_t maxprefix_of(int sim, uint32_t len, double t) {
    return (uint32_t)imin((int)len, (int)(len - minsize_of(sim, len, t) + 1));
}
uint32_t midprefix_of(int sim, uint32_t len, double t) {
    return (uint32_t)imin((int)len, (int)(len - minoverlap_of(sim, len, len, t) + 1));
}

constexpr uint64_t MAX_COSINE_TABLE = 64ull << 20;  // entries

hyset_status get_bounds(hyset_ctx* ctx, int sim, double tau, uint32_t L, int index_maxprefix, Bounds** out) {
    auto key = std::make_tuple(sim, tau, L, index_maxprefix);
    auto it = ctx->bounds.find(key);
    if (it != ctx->bounds.end()) {
        *out = it->second.get();
        return HYSET_OK;
    }
    auto b = std::make_unique<Bounds>();
    b->sim = sim;
    b->tau = tau;
    b->L = L;
    b->index_maxprefix = index_maxprefix;
    b->minsize.resize(L + 1);
    b->probe_prefix.resize(L + 1);
    b->index_prefix.resize(L + 1);
    b->max_partner.resize(L + 1);
    b->mid_prefix.resize(L + 1);
    for (uint32_t l = 0; l <= L; ++l) {
        b->minsize[l] = minsize_of(sim, l, tau);
        b->probe_prefix[l] = l ? maxprefix_of(sim, l, tau) : 0;
        b->mid_prefix[l] = l ? midprefix_of(sim, l, tau) : 0;
        b->index_prefix[l] = l ? (index_maxprefix ? b->probe_prefix[l] : b->mid_prefix[l]) : 0;
        if (b->minsize[l] > l) return fail(ctx, HYSET_E_INVALID, "threshold yields minsize > set size");
    }
    uint32_t q = 0;
    for (uint32_t l = 0; l <= L; ++l) {
        while (q + 1 <= L && b->minsize[q + 1] <= l) ++q;
        b->max_partner[l] = q;
    }
    if (sim == SIM_COSINE) {
        b->mo_row.resize((size_t)L + 2);
        uint64_t run = 0;
        for (uint32_t big = 0; big <= L; ++big) {
            b->mo_row[big] = run;
            run += (uint64_t)(big - b->minsize[big] + 1);
        }
        b->mo_row[L + 1] = run;
        if (run > MAX_COSINE_TABLE)
            return fail(ctx, HYSET_E_UNSUPPORTED, "cosine bound table too large for the longest set");
        b->mo_tab.resize(run);
        for (uint32_t big = 0; big <= L; ++big)
            for (uint32_t small = b->minsize[big]; small <= big; ++small)
                b->mo_tab[b->mo_row[big] + (small - b->minsize[big])] = sim_minoverlap(sim, big, small, tau);
        b->mo_sum.assign(1, 0);
        // non-decreasing along rows (small) and along columns (big)
        b->mo_monotone = true;
        for (uint32_t big = 1; big <= L && b->mo_monotone; ++big)
            for (uint32_t small = b->minsize[big]; small <= big; ++small) {
                const uint32_t v = b->mo_tab[b->mo_row[big] + (small - b->minsize[big])];
                if (small > b->minsize[big] && b->mo_tab[b->mo_row[big] + (small - 1 - b->minsize[big])] > v)
                    b->mo_monotone = false;
                if (big > 1 && small >= b->minsize[big - 1] && small <= big - 1 &&
                    b->mo_tab[b->mo_row[big - 1] + (small - b->minsize[big - 1])] > v)
                    b->mo_monotone = false;
            }
    } else {
        b->mo_sum.resize(2 * (size_t)L + 1);
        for (uint32_t s = 0; s <= 2 * L; ++s) b->mo_sum[s] = sim_minoverlap(sim, s, 0, tau);
        b->mo_row.assign(1, 0);
        b->mo_tab.assign(1, 0);
        b->mo_monotone = true;
        for (uint32_t s = 1; s <= 2 * L; ++s)
            if (b->mo_sum[s] < b->mo_sum[s - 1]) b->mo_monotone = false;
    }
    // one device allocation holding all tables
    size_t n32 = 5 * ((size_t)L + 1) + b->mo_sum.size() + b->mo_tab.size();
    size_t bytes = b->mo_row.size() * 8 + n32 * 4;
    CK(b->dev.ensure(bytes, ctx->stream));
    uint8_t* base = b->dev.as<uint8_t>();
    uint64_t* d_row = (uint64_t*)base;
    uint32_t* p = (uint32_t*)(base + b->mo_row.size() * 8);
    auto put = [&](const std::vector<uint32_t>& v, uint32_t*& dst) -> cudaError_t {
        uint32_t* d = p;
        p += v.size();
        dst = d;
        return cudaMemcpyAsync(d, v.data(), v.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    };
    uint32_t *d_minsize, *d_pp, *d_ip, *d_mp, *d_mid, *d_sum, *d_tab;
    CK(cudaMemcpyAsync(d_row, b->mo_row.data(), b->mo_row.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(put(b->minsize, d_minsize));
    CK(put(b->probe_prefix, d_pp));
    CK(put(b->index_prefix, d_ip));
    CK(put(b->max_partner, d_mp));
    CK(put(b->mid_prefix, d_mid));
    CK(put(b->mo_sum, d_sum));
    CK(put(b->mo_tab, d_tab));
    CK(cudaStreamSynchronize(ctx->stream));
    b->view = BoundsView{d_minsize, d_pp, d_ip, d_mp, d_mid, d_sum, d_row, d_tab, L, sim};
    *out = b.get();
    ctx->bounds.emplace(key, std::move(b));
    return HYSET_OK;
}

// Host size statistics from host-resident sizes (the caller's array, or the
// pinned copy of device sizes): the per-size histogram and first_ge[l] = first
// set id with size >= l (sizes are non-decreasing), whose device copy is
// enqueued on the stream (the host array is a member, so no synchronisation is
// needed here).  The collection keeps no per-set host array: sizes of single
// sets and of id ranges come from first_ge.
hyset_status build_size_meta(hyset_ctx* ctx, hyset_coll* c, const uint32_t* sizes) {
    // run lengths: sorted sizes repeat, so the count stays in a register
    std::vector<uint64_t>& hist = c->size_hist;
    hist.assign(c->n ? (size_t)sizes[c->n - 1] + 1 : 1, 0);
    uint32_t i = 0;
    while (i < c->n) {
        const uint32_t v = sizes[i];
        uint32_t j = i + 1;
        while (j < c->n && sizes[j] == v) ++j;
        if (v >= hist.size()) hist.resize((size_t)v + 1, 0);
        hist[v] += j - i;
        i = j;
    }
    const uint32_t L = (uint32_t)hist.size() - 1;
    c->max_size = L;
    std::vector<uint32_t>& f = c->h_first_ge;
    f.resize((size_t)L + 2);
    uint64_t run = 0;
    for (uint32_t l = 0; l <= L + 1; ++l) {
        f[l] = (uint32_t)run;
        if (l <= L) run += c->size_hist[l];
    }
    CK(c->first_ge.ensure(f.size() * 4, ctx->stream));
    CK(cudaMemcpyAsync(c->first_ge.p, f.data(), f.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    return HYSET_OK;
}

// Size of set i (sizes are non-decreasing: the last l with first_ge[l] <= i).
uint32_t size_at(const hyset_coll* c, uint32_t i) {
    const auto& f = c->h_first_ge;
    return (uint32_t)(std::upper_bound(f.begin(), f.end(), i) - f.begin()) - 1;
}

// Sets per size among ids [lo, hi).
std::vector<uint64_t> range_hist(const hyset_coll* c, uint32_t lo, uint32_t hi) {
    std::vector<uint64_t> ph((size_t)c->max_size + 1, 0);
    const auto& f = c->h_first_ge;
    for (uint32_t l = 0; l <= c->max_size; ++l) {
        const uint32_t a = std::max(lo, f[l]), b = std::min(hi, f[l + 1]);
        if (b > a) ph[l] = b - a;
    }
    return ph;
}

// Prefix entries of sets [lo, hi) (all sets when hi == n) from the size histogram.
uint64_t prefix_entries(const hyset_coll* c, const std::vector<uint32_t>& pre) {
    uint64_t E = 0;
    for (size_t l = 0; l < c->size_hist.size(); ++l) E += c->size_hist[l] * (uint64_t)pre[l];
    return E;
}

// Bits needed to represent v (at least 1).
uint32_t bits_for(uint64_t v) {
    uint32_t b = 1;
    while (b < 64 && (v >> b)) ++b;
    return b;
}

uint32_t pre_len(const Bounds* b, uint32_t l) { return b->index_prefix[l]; }

int key_bits_for(uint32_t universe) {
    int bits = 1;
    while (bits < 32 && (universe - 1) >> bits) ++bits;
    return bits;
}

// Global inverted index over the prefix entries of every set, lists ordered by
// set id: histogram + scan give the list offsets; the entries (emitted in set
// order) go into their lists by atomic slots and each list is put back in set
// order in shared memory when every list is short, or by a stable radix sort
// by token otherwise (index_lists).
// pre / d_pre: the prefix length table (default: the bounds' index prefix);
// force_pb >= 0 fixes the layout (0 = unpacked, > 0 = packed with that many
// position bits) so that two indexes of one join share it.
hyset_status build_sorted_index(hyset_ctx* ctx, hyset_coll* c, const Bounds* b, int kind, Index& ix,
                                const std::vector<uint32_t>* pre = nullptr, const uint32_t* d_pre = nullptr,
                                int force_pb = -1) {
    // Rebuilt on every join (buffers are reused): a join's timed device work
    // always includes its own index build.  Only asynchronous stream work once
    // the buffers are large enough, so a batch can capture it into a graph.
    if (!pre) {
        pre = &b->index_prefix;
        d_pre = b->view.index_prefix;
    }
    cudaStream_t s = ctx->stream;
    const uint32_t n = c->n, U = c->universe;
    const uint64_t E = prefix_entries(c, *pre);
    if (E >= (1ull << 32)) return fail(ctx, HYSET_E_UNSUPPORTED, "more than 2^32 prefix entries");
    const uint64_t E1 = E ? E : 1;
    CK(ctx->sc->len.ensure((size_t)n * 4 + 4, s));
    CK(ctx->sc->off.ensure((size_t)n * 4 + 4, s));
    CK(ctx->sc->tok.ensure(E1 * 4, s));
    CK(ctx->sc->set.ensure(E1 * 4, s));
    CK(ctx->sc->pos.ensure(E1 * 4, s));
    CK(ctx->sc->order.ensure(E1 * 4, s));
    CK(ctx->sc->altk.ensure(E1 * 4, s));
    CK(ctx->sc->altv.ensure(E1 * 4, s));
    CK(ctx->sc->counts.ensure(((size_t)U + 1) * 4, s));
    size_t scan_words = std::max(std::max(scan_scratch_words(n), scan_scratch_words((uint64_t)U + 1)),
                                 radix_scratch_words(E1));
    CK(ctx->sc->scan.ensure(scan_words * 4, s));
    CK(ix.list_off.ensure(((size_t)U + 1) * 4, s));
    CK(ix.set.ensure(E1 * 4, s));
    CK(ix.pos.ensure(E1 * 4, s));
    CollView v = c->view();
    uint32_t* len = ctx->sc->len.as<uint32_t>();
    uint32_t* off = ctx->sc->off.as<uint32_t>();
    uint32_t* scr = ctx->sc->scan.as<uint32_t>();
    CK(set_prefix_lengths(v, d_pre, 0, n, len, s));
    CK(scan_exclusive(len, off, n, scr, s));
    // Packed entries (set << pb | position) when set ids up to n and positions
    // below the longest prefix fit 32 bits: the sorted values are the index.
    uint32_t max_pre = 1;
    for (size_t l = 0; l < c->size_hist.size(); ++l)
        if (c->size_hist[l]) max_pre = std::max(max_pre, (*pre)[l]);
    const uint32_t pb = force_pb > 0 ? (uint32_t)force_pb : bits_for(max_pre), sb = bits_for(n);
    if (force_pb != 0 && pb + sb <= 32) {
        uint32_t* counts = ctx->sc->counts.as<uint32_t>();
        CK(ctx->sc->gate.ensure(4, s));
        CK(cudaMemsetAsync(counts, 0, ((size_t)U + 1) * 4, s));
        CK(emit_packed_entries(v, off, len, pb, ctx->sc->tok.as<uint32_t>(), ix.set.as<uint32_t>(), counts, s));
        // the list build's path is read back once per collection and prefix
        // table (not while a batch is being captured into a graph)
        cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(s, &capturing));
        int& path = c->list_path[d_pre];
        CK(index_lists(ctx->sc->tok.as<uint32_t>(), ix.set.as<uint32_t>(), E, U, counts, ix.list_off.as<uint32_t>(),
                       ctx->sc->altk.as<uint32_t>(), ctx->sc->altv.as<uint32_t>(), ctx->sc->gate.as<uint32_t>(),
                       key_bits_for(U), scr, s, &path,
                       capturing == cudaStreamCaptureStatusNone ? ctx->h_flags + 15 : nullptr));
        ix.sim = b->sim;
        ix.tau = b->tau;
        ix.kind = kind;
        ix.universe = U;
        ix.entries = E;
        ix.pos_bits = pb;
        return HYSET_OK;
    }
    CK(emit_prefix_entries(v, 0, n, off, len, ctx->sc->tok.as<uint32_t>(), ctx->sc->set.as<uint32_t>(),
                           ctx->sc->pos.as<uint32_t>(), s));
    uint32_t* counts = ctx->sc->counts.as<uint32_t>();
    CK(cudaMemsetAsync(counts, 0, ((size_t)U + 1) * 4, s));
    CK(token_histogram(ctx->sc->tok.as<uint32_t>(), E, counts, U + 1, s));
    CK(scan_exclusive(counts, ix.list_off.as<uint32_t>(), (uint64_t)U + 1, scr, s));
    CK(iota_u32(ctx->sc->order.as<uint32_t>(), E, s));
    CK(radix_sort_pairs(ctx->sc->tok.as<uint32_t>(), ctx->sc->order.as<uint32_t>(), ctx->sc->altk.as<uint32_t>(),
                        ctx->sc->altv.as<uint32_t>(), E, key_bits_for(U), scr, s, false));
    CK(gather_entries(ctx->sc->order.as<uint32_t>(), E, ctx->sc->set.as<uint32_t>(), ctx->sc->pos.as<uint32_t>(),
                      ix.set.as<uint32_t>(), ix.pos.as<uint32_t>(), s));
    ix.sim = b->sim;
    ix.tau = b->tau;
    ix.kind = kind;
    ix.universe = U;
    ix.entries = E;
    ix.pos_bits = 0;
    return HYSET_OK;
}

// R-S prefix-index joins split each probe's length window in two bands:
// candidates at least as long as the probe need only the probe's midprefix
// tokens (against R's maxprefix index), shorter candidates need only their
// own midprefix entries (a second, midprefix index of R, against the probe's
// maxprefix tokens).  Both hold because minoverlap does not decrease when
// either length grows, which get_bounds checks on the bound tables.
bool use_bands(const Bounds* b, bool self) { return !self && b->mo_monotone; }

// The prefix index (and for banded R-S joins the midprefix index) of R, and
// their views in P.
hyset_status build_fgss_indexes(hyset_ctx* ctx, hyset_coll* R, const Bounds* b, bool self, Index& ix,
                                 Index& ix_mid, JoinParams& P) {
    ST(build_sorted_index(ctx, R, b, self ? 0 : 1, ix));
    P.X = ix.view();
    P.X2 = IndexView{};
    if (use_bands(b, self)) {
        ST(build_sorted_index(ctx, R, b, 2, ix_mid, &b->mid_prefix, b->view.mid_prefix, (int)ix.pos_bits));
        P.X2 = ix_mid.view();
    }
    return HYSET_OK;
}

// Token groups of the first pre[size] tokens of every set (histogram, scan,
// atomic scatter).  Rebuilt on every join; buffers are reused.
hyset_status build_groups(hyset_ctx* ctx, hyset_coll* c, const uint32_t* d_pre, const std::vector<uint32_t>& pre,
                          uint32_t U, uint64_t* entries) {
    cudaStream_t s = ctx->stream;
    const uint64_t E = prefix_entries(c, pre);
    if (E >= (1ull << 32)) return fail(ctx, HYSET_E_UNSUPPORTED, "more than 2^32 prefix entries");
    CK(c->g_off.ensure(((size_t)U + 1) * 4, s));
    CK(c->g_cursor.ensure(((size_t)U + 1) * 4, s));
    CK(c->g_set.ensure((E ? E : 1) * 4, s));
    CK(c->g_ps.ensure((E ? E : 1) * 4, s));
    CK(ctx->sc->scan.ensure(scan_scratch_words((uint64_t)U + 1) * 4, s));
    uint32_t* cnt = c->g_cursor.as<uint32_t>();
    CK(cudaMemsetAsync(cnt, 0, ((size_t)U + 1) * 4, s));
    CK(group_count(c->view(), d_pre, cnt, s));
    CK(scan_exclusive(cnt, c->g_off.as<uint32_t>(), (uint64_t)U + 1, ctx->sc->scan.as<uint32_t>(), s));
    CK(cudaMemcpyAsync(cnt, c->g_off.p, ((size_t)U + 1) * 4, cudaMemcpyDeviceToDevice, s));
    CK(group_scatter(c->view(), d_pre, cnt, c->g_set.as<uint32_t>(), c->g_ps.as<uint32_t>(), s));
    *entries = E;
    return HYSET_OK;
}

// Signatures are regenerated on every join (the buffer is reused); the buffer
// is sized on the context's stream, the generation runs on `gen` (default: the
// same stream).
hyset_status get_bitmaps(hyset_ctx* ctx, hyset_coll* c, int words, const uint64_t** out,
                         cudaStream_t gen = nullptr) {
    DevBuf& d = c->bitmaps[words];
    CK(d.ensure((size_t)c->n * words * 8 + 8, ctx->stream));
    if (gen && gen != ctx->stream) {
        CK(cudaEventRecord(ctx->ev_fork, ctx->stream));
        CK(cudaStreamWaitEvent(gen, ctx->ev_fork, 0));
    }
    CK(generate_bitmaps(c->view(), words, d.as<uint64_t>(), gen ? gen : ctx->stream));
    *out = d.as<uint64_t>();
    return HYSET_OK;
}

hyset_status check_opts(hyset_ctx* ctx, const hyset_join_opts* o) {
    if (!o) return fail(ctx, HYSET_E_INVALID, "null options");
    if (!(o->threshold > 0.0 && o->threshold <= 1.0)) return fail(ctx, HYSET_E_INVALID, "threshold must be in (0, 1]");
    if (o->sim < HYSET_JACCARD || o->sim > HYSET_DICE) return fail(ctx, HYSET_E_INVALID, "unknown similarity");
    if (o->technique < HYSET_TECH_AUTO || o->technique > HYSET_TECH_DIRECT)
        return fail(ctx, HYSET_E_INVALID, "unknown technique");
    if (o->bitmap_bits != 0 && o->bitmap_bits != 64 && o->bitmap_bits != 128 && o->bitmap_bits != 256 &&
        o->bitmap_bits != 512)
        return fail(ctx, HYSET_E_INVALID, "bitmap_bits must be 0, 64, 128, 256 or 512");
    if (o->verify_mode > 3) return fail(ctx, HYSET_E_INVALID, "verify_mode must be 0, 1, 2 or 3");
    if (o->orientation > 2) return fail(ctx, HYSET_E_INVALID, "orientation must be 0, 1 or 2");
    return HYSET_OK;
}

// The autotuner's per-join configuration (technique, kernel variant, signature
// width, batch, verification mode).  Explicit options always win; AUTO fills
// the rest from collection statistics with rules measured on GB300
// (1M-set long-set workload: probe-major, batch 3, 256-bit signatures; 200K-set
// short-set workload: 128-bit signatures; token-major only on request, it wins
// only where every token group is small, i.e. high thresholds; enumerating the
// length window only for small collections).
struct Tuned {
    hyset_technique tech;
    int probe_major;
    uint32_t batch;
    uint32_t bits;
    int vmode;
};

Tuned tune(const hyset_coll* R, const hyset_coll* S, const hyset_join_opts* o,
           hyset_technique selected = HYSET_TECH_AUTO) {
    Tuned t{};
    const double avg = R->n ? (double)R->n_tokens / (double)R->n : 0.0;
    const uint64_t pairs_window = (uint64_t)R->n * (uint64_t)S->n;
    t.tech = o->technique;
    if (t.tech == HYSET_TECH_AUTO) t.tech = selected;
    if (t.tech == HYSET_TECH_AUTO) t.tech = (pairs_window <= 4000000ull) ? HYSET_TECH_BITMAP : HYSET_TECH_FGSS;
    // explicit FGSS defaults to the token-major kernel; AUTO to probe-major
    t.probe_major = (o->technique == HYSET_TECH_FGSS && !o->probe_major) ? 0 : 1;
    t.batch = o->fgss_batch ? o->fgss_batch : 3;
    t.bits = o->bitmap_bits;
    if (o->technique == HYSET_TECH_AUTO && t.bits == 0) t.bits = avg <= 48.0 ? 128 : 256;
    if (t.tech == HYSET_TECH_BITMAP && t.bits == 0) t.bits = 64;
    if (t.tech == HYSET_TECH_DIRECT) t.bits = 0;
    t.vmode = o->verify_mode ? (int)o->verify_mode : 1;
    if (t.vmode == 3) t.vmode = 1;  // the staged mode exists for explicit candidate lists only
    return t;
}

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
                      hyset_result* res, bool timed_from_ev0, TokenJoinParams* T = nullptr) {
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

// ---------------------------------------------------------------- selector

// Length-compatible candidate pairs (the enumeration techniques' work) from the
// size histograms: per probe size l, the indexed sets of size [minsize(l), upper(l)].
double window_pairs(const hyset_coll* R, const std::vector<uint64_t>& probe_hist, const Bounds* b, bool self) {
    std::vector<uint64_t> cum(R->size_hist.size() + 1, 0);
    for (size_t l = 0; l < R->size_hist.size(); ++l) cum[l + 1] = cum[l] + R->size_hist[l];
    auto count_le = [&](uint64_t l) -> uint64_t { return cum[std::min<uint64_t>(l + 1, cum.size() - 1)]; };
    double pairs = 0;
    for (size_t l = 0; l < probe_hist.size(); ++l) {
        if (!probe_hist[l]) continue;
        const uint64_t lo = b->minsize[l];
        const uint64_t hi = self ? l : b->max_partner[l];
        if (hi < lo) continue;
        double w = (double)(count_le(hi) - (lo ? count_le(lo - 1) : 0));
        if (self) w -= 0.5 * (double)(probe_hist[l] + 1);  // only smaller ids among equal sizes
        pairs += (double)probe_hist[l] * std::max(0.0, w);
    }
    return pairs;
}

hyset_status compute_features(hyset_ctx* ctx, hyset_coll* R, hyset_coll* S, const hyset_join_opts* o, float* f,
                              double* base) {
    ST(check_opts(ctx, o));
    const bool self = R == S;
    const uint32_t L = std::max(R->max_size, S->max_size);
    Bounds* b = nullptr;
    ST(get_bounds(ctx, o->sim, o->threshold, L, self ? 0 : 1, &b));
    if (o->probe_end > S->n || o->probe_begin > o->probe_end)
        return fail(ctx, HYSET_E_INVALID, "probe range outside the probe collection");
    const uint32_t p_lo = o->probe_end ? o->probe_begin : 0, p_hi = o->probe_end ? o->probe_end : S->n;
    const uint32_t np = p_hi - p_lo;
    const uint32_t U = std::max(R->universe, S->universe);
    cudaStream_t s = ctx->stream;
    CK(ctx->d_moments.ensure(64, s));
    CK(ctx->d_hist.ensure(((size_t)U + 1) * 4, s));
    unsigned long long* mom = ctx->d_moments.as<unsigned long long>();
    CK(cudaMemsetAsync(mom, 0, 64, s));
    CK(cudaMemsetAsync(ctx->d_hist.p, 0, ((size_t)U + 1) * 4, s));
    CollView part = S->view();  // the probe partition as a collection of its own
    part.sizes += p_lo;
    part.starts += p_lo;
    part.meta += p_lo;
    part.n = np;
    if (np) {
        CK(moments_u32(S->d_sizes + p_lo, np, mom, s));
        CK(group_count(part, b->view.probe_prefix, ctx->d_hist.as<uint32_t>(), s));
        CK(moments_u32(ctx->d_hist.as<uint32_t>(), U, mom + 4, s));
    }
    unsigned long long m[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    CK(cudaMemcpyAsync(m, mom, 64, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const std::vector<uint64_t> ph = np == S->n ? S->size_hist : range_hist(S, p_lo, p_hi);
    double pre = 0;
    for (size_t l = 0; l < ph.size(); ++l) pre += (double)ph[l] * b->probe_prefix[l];
    const double n_d = np ? (double)np : 1.0;
    const double mean = (double)m[0] / n_d;
    const double var = std::max(0.0, (double)m[1] / n_d - mean * mean);
    const double tmean = (double)m[4] / (double)U;
    const double tvar = std::max(0.0, (double)m[5] / (double)U - tmean * tmean);  // over the whole universe
    const double index_entries = (double)prefix_entries(R, b->index_prefix);
    const double pairs = window_pairs(R, ph, b, self);
    const double v[MLP_IN] = {std::log2(1.0 + np), mean, std::sqrt(var), std::log2(1.0 + (double)m[2]),
                              std::log2(1.0 + U), o->threshold, (double)o->sim / 2.0, pre / n_d,
                              std::log2(1.0 + index_entries), std::log2(1.0 + std::sqrt(tvar)),
                              std::log2(1.0 + (double)m[6]), std::log2(1.0 + pairs)};
    for (int k = 0; k < MLP_IN; ++k) f[k] = (float)v[k];
    if (base) {
        base[0] = std::sqrt(var);
        base[1] = mean;
        base[2] = std::sqrt(tvar);
        base[3] = np;
        base[4] = U;
        base[5] = index_entries;
        base[6] = pairs;
        base[7] = pre / n_d;
    }
    return HYSET_OK;
}

// Content signature of a collection for the selector and autotuner caches: the
// decisions depend only on the collection's statistics, so a re-uploaded copy
// of the same data reuses them.
std::string coll_signature(const hyset_coll* c) {
    uint64_t h = 1469598103934665603ull;  // FNV-1a over the size histogram
    for (uint64_t v : c->size_hist) {
        h ^= v;
        h *= 1099511628211ull;
    }
    char buf[96];
    std::snprintf(buf, sizeof buf, "%u:%llu:%u:%016llx", c->n, (unsigned long long)c->n_tokens, c->max_size,
                  (unsigned long long)h);
    return buf;
}

std::string join_key(const hyset_coll* R, const hyset_coll* S, const hyset_join_opts* o) {
    char buf[96];
    std::snprintf(buf, sizeof buf, "|%d|%.17g|%u|%u|%d", (int)o->sim, o->threshold, o->probe_begin, o->probe_end,
                  R == S ? 1 : 0);
    return coll_signature(R) + "/" + coll_signature(S) + buf;
}

const hyset_technique kSelectable[3] = {HYSET_TECH_BITMAP, HYSET_TECH_FGSS, HYSET_TECH_DIRECT};

// cost.hpp:28-58 / statistics.hpp:150-160: |c . (1, std, avg, tokfreq, n, n^2, U, index, bitmap)|
double analytic_cost(const double* c, const double* base, double bitmap_bits) {
    const double x[9] = {1.0, base[0], base[1], base[2], base[3], base[3] * base[3], base[4], base[5], bitmap_bits};
    double s = 0;
    for (int k = 0; k < 9; ++k) s += c[k] * x[k];
    return std::fabs(s);
}

// The technique AUTO runs: the learned network's argmin of predicted log-time,
// else the analytic cost model's argmin, else fixed rules (AUTO passed on).
// Decided once per (collections, similarity, threshold, probe range) and reused.
hyset_status select_technique(hyset_ctx* ctx, hyset_coll* R, hyset_coll* S, const hyset_join_opts* o,
                              hyset_technique* out, int* selector) {
    *out = HYSET_TECH_AUTO;
    *selector = 0;
    if (o->technique != HYSET_TECH_AUTO) {
        *selector = -1;
        return HYSET_OK;
    }
    if (!ctx->has_mlp && !ctx->has_cost) return HYSET_OK;
    const std::string key = join_key(R, S, o);
    auto it = ctx->select_cache.find(key);
    if (it != ctx->select_cache.end()) {
        *out = it->second.first;
        *selector = it->second.second;
        return HYSET_OK;
    }
    float f[MLP_IN];
    double base[8];
    ST(compute_features(ctx, R, S, o, f, base));
    if (ctx->has_mlp) {
        float x[MLP_IN], y[MLP_OUT] = {0, 0, 0};
        for (int k = 0; k < MLP_IN; ++k) x[k] = (f[k] - ctx->feat_mean[k]) / ctx->feat_scale[k];
        cudaStream_t s = ctx->stream;
        CK(ctx->d_feat.ensure(256, s));
        float* dx = ctx->d_feat.as<float>();
        CK(cudaMemcpyAsync(dx, x, sizeof x, cudaMemcpyHostToDevice, s));
        CK(mlp_forward(ctx->d_mlp.as<float>(), dx, 1, dx + 32, ctx->sm_count, s));
        CK(cudaMemcpyAsync(y, dx + 32, sizeof y, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        int best = 0;
        for (int k = 1; k < MLP_OUT; ++k)
            if (y[k] < y[best]) best = k;
        *out = kSelectable[best];
        *selector = 2;
    } else {
        const double avg = base[1];
        const double bits = avg <= 48.0 ? 128.0 : 256.0;
        int best = 0;
        double bc = 0;
        for (int k = 0; k < 3; ++k) {
            const double c = analytic_cost(ctx->cost[k], base, k == 0 ? bits : 0.0);
            if (k == 0 || c < bc) { bc = c; best = k; }
        }
        *out = kSelectable[best];
        *selector = 1;
    }
    ctx->select_cache[key] = {*out, *selector};
    return HYSET_OK;
}

// Partition split (the selector's second decision, dichotomy.cu's split of a
// join into partitions handled by different techniques): the learned network
// predicts each technique's time for the whole probe range and for its two
// halves; when the halves prefer different techniques and their predicted sum
// is at least 10 % below the whole's best, the join runs as two probe ranges.
// Self-joins from 40,000 probes with technique AUTO and the network installed;
// the plan is cached with the technique choice.  The pair set does not change.
constexpr uint32_t SPLIT_MIN_PROBES = 40000;
constexpr float SPLIT_MARGIN = 0.9f;

hyset_status plan_split(hyset_ctx* ctx, hyset_coll* R, const hyset_join_opts* o, uint32_t* split_at,
                        hyset_technique* low, hyset_technique* high) {
    *split_at = 0;
    if (o->technique != HYSET_TECH_AUTO || !ctx->has_mlp || o->probe_end || o->device_pairs ||
        R->n < SPLIT_MIN_PROBES)
        return HYSET_OK;
    const std::string key = "split|" + join_key(R, R, o);
    auto it = ctx->split_cache.find(key);
    if (it != ctx->split_cache.end()) {
        *split_at = it->second.at;
        *low = it->second.low;
        *high = it->second.high;
        return HYSET_OK;
    }
    const uint32_t mid = R->n / 2;
    float x[3][MLP_IN], y[3][MLP_OUT];
    for (int part = 0; part < 3; ++part) {
        hyset_join_opts q = *o;
        q.probe_begin = part == 2 ? mid : 0;
        q.probe_end = part == 0 ? 0 : (part == 1 ? mid : R->n);
        float f[MLP_IN];
        ST(compute_features(ctx, R, R, &q, f, nullptr));
        for (int k = 0; k < MLP_IN; ++k) x[part][k] = (f[k] - ctx->feat_mean[k]) / ctx->feat_scale[k];
    }
    cudaStream_t s = ctx->stream;
    CK(ctx->d_feat.ensure(512, s));
    float* dx = ctx->d_feat.as<float>();
    CK(cudaMemcpyAsync(dx, x, sizeof x, cudaMemcpyHostToDevice, s));
    CK(mlp_forward(ctx->d_mlp.as<float>(), dx, 3, dx + 64, ctx->sm_count, s));
    CK(cudaMemcpyAsync(y, dx + 64, sizeof y, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    int best[3];
    for (int part = 0; part < 3; ++part) {
        best[part] = 0;
        for (int k = 1; k < MLP_OUT; ++k)
            if (y[part][k] < y[part][best[part]]) best[part] = k;
    }
    const double whole = std::exp((double)y[0][best[0]]);
    const double parts = std::exp((double)y[1][best[1]]) + std::exp((double)y[2][best[2]]);
    hyset_ctx::SplitPlan plan{0, kSelectable[best[1]], kSelectable[best[2]]};
    if (best[1] != best[2] && parts < SPLIT_MARGIN * whole) plan.at = mid;
    ctx->split_cache[key] = plan;
    *split_at = plan.at;
    *low = plan.low;
    *high = plan.high;
    return HYSET_OK;
}

// Autotuner for the prefix-index join's signature width: on the first AUTO join
// of a (collections, similarity, threshold), the probe-major kernel runs on
// three probe samples spread over the probe range with no signatures and with
// 128-, 256- and 512-bit signatures; the samples' time scaled to the whole
// probe range plus the width's signature generation decides, and the width is
// kept for that join.  Measured on GB300: 256 bits wins on long sets at high thresholds, 512
// on long sets at low thresholds, 128 on short ones, none on some collections.
constexpr uint32_t TUNE_MIN_PROBES = 60000, TUNE_SAMPLE = 16384;  // a sample fills the GPU for about two waves
constexpr float TUNE_MARGIN = 0.92f;  // leave the rule's width only for an estimated gain of 8 % or more
constexpr float TUNE_VMODE_MARGIN = 0.97f;  // warp verification only for an estimated gain of 3 % or more

// The signature width (and, when vmode is given, the verification mode) of a
// prefix-index join, from timed samples of its probe range; cached per join
// key as bits | vmode << 16.
hyset_status autotune_bits(hyset_ctx* ctx, hyset_coll* R, hyset_coll* S, const hyset_join_opts* o, Bounds* b,
                           bool self, uint32_t p_lo, uint32_t p_hi, uint32_t* bits, int* vmode = nullptr) {
    const std::string key = join_key(R, S, o);
    auto it = ctx->bits_cache.find(key);
    if (it != ctx->bits_cache.end() && (!vmode || (it->second >> 16))) {
        *bits = it->second & 0xFFFFu;
        if (vmode) *vmode = (int)(it->second >> 16);
        return HYSET_OK;
    }
    cudaStream_t s = ctx->stream;
    JoinParams P{};
    ST(build_fgss_indexes(ctx, R, b, self, R->index, R->index_mid, P));
    P.R = R->view();
    P.S = S->view();
    P.B = b->view;
    P.first_ge = R->first_ge.as<uint32_t>();
    P.R_L = R->max_size;
    P.self = self ? 1 : 0;
    P.r_lo = 0;
    P.r_hi = R->n;
    P.grab = 4;
    CK(ctx->s_count.ensure(16, s));
    CK(ctx->s_work.ensure(16, s));
    P.out = Sink{nullptr, ctx->s_count.as<unsigned long long>(), 0, 1};
    P.work = ctx->s_work.as<unsigned int>();
    const uint32_t cand[4] = {0, 128, 256, 512};
    float est[4] = {0, 0, 0, 0}, kern_est[4] = {0, 0, 0, 0};
    float best_ms = 0;
    uint32_t best = 256;
    // estimated kernel time of the whole probe range with signature words w and
    // verification mode vm, from three samples (start, middle, end)
    auto sample = [&](int vm, float* out) -> hyset_status {
        float total = 0;
        uint32_t sampled = 0;
        for (int c = 0; c < 3; ++c) {
            const uint32_t span = p_hi - p_lo, len = std::min(TUNE_SAMPLE, span / 3);
            P.p_lo = p_lo + (uint32_t)((uint64_t)(span - len) * c / 2);
            P.p_hi = P.p_lo + len;
            sampled += len;
            CK(cudaMemsetAsync(ctx->s_count.p, 0, 16, s));
            CK(cudaMemsetAsync(ctx->s_work.p, 0, 16, s));
            CK(cudaEventRecord(ctx->ek0, s));
            CK(launch_join(P, TECH_FGSS, vm, ctx->sm_count, s));
            CK(cudaEventRecord(ctx->ek1, s));
            CK(cudaEventSynchronize(ctx->ek1));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, ctx->ek0, ctx->ek1));
            total += ms;
        }
        *out = total * (float)(p_hi - p_lo) / (float)(sampled ? sampled : 1);
        return HYSET_OK;
    };
    for (int k = 0; k < 4; ++k) {
        const int words = (int)(cand[k] / 64);
        P.words = words;
        P.bits_R = P.bits_S = nullptr;
        float gen_ms = 0;  // the width's signature generation, paid once per join
        if (words) {
            const uint64_t *br = nullptr, *bs = nullptr;
            CK(cudaEventRecord(ctx->ek0, s));
            ST(get_bitmaps(ctx, R, words, &br));
            if (self) bs = br;
            else ST(get_bitmaps(ctx, S, words, &bs));
            CK(cudaEventRecord(ctx->ek1, s));
            CK(cudaEventSynchronize(ctx->ek1));
            CK(cudaEventElapsedTime(&gen_ms, ctx->ek0, ctx->ek1));
            P.bits_R = br;
            P.bits_S = bs;
        }
        float total = 0;
        ST(sample(1, &total));
        kern_est[k] = total;
        total += gen_ms;  // the whole probe range's estimated kernel time plus the generation
        est[k] = total;
        if (k == 0 || total < best_ms) {
            best_ms = total;
            best = cand[k];
        }
    }
    // the rule's width (mean size <= 48: 128 bits, else 256) unless another is clearly faster
    const uint32_t rule = (double)R->n_tokens / (double)std::max<uint32_t>(R->n, 1) <= 48.0 ? 128u : 256u;
    const float rule_ms = est[rule == 128u ? 1 : 2];
    if (best != rule && best_ms > TUNE_MARGIN * rule_ms) best = rule;
    // verification: a lane per surviving item, or the warp per item when the
    // samples show it faster at the chosen width (long merges: low thresholds,
    // cosine)
    int vm = 1;
    if (vmode) {
        const int kb = best == 0 ? 0 : best == 128 ? 1 : best == 256 ? 2 : 3;
        const int words = (int)(best / 64);
        P.words = words;
        P.bits_R = P.bits_S = nullptr;
        if (words) {
            const uint64_t *br = nullptr, *bs = nullptr;
            ST(get_bitmaps(ctx, R, words, &br));
            if (self) bs = br;
            else ST(get_bitmaps(ctx, S, words, &bs));
            P.bits_R = br;
            P.bits_S = bs;
        }
        float warp_ms = 0;
        ST(sample(2, &warp_ms));
        if (warp_ms < TUNE_VMODE_MARGIN * kern_est[kb]) vm = 2;
        *vmode = vm;
    }
    ctx->bits_cache[key] = best | (vmode ? (uint32_t)vm << 16 : 0u);
    *bits = best;
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
            ST(autotune_bits(ctx, R, S, o, b, self, a_lo, a_hi, &tn.bits, o->verify_mode ? nullptr : &tn.vmode));
    }
    const int vmode = tn.vmode;
    res->verify_mode = (uint32_t)vmode;
    res->bitmap_bits = tech == HYSET_TECH_DIRECT ? 0 : tn.bits;
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
    const int words = (int)(tn.bits / 64);
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

// Validates an uploaded collection and derives its metadata.  The device
// check (one pass over the tokens, which also writes the meta pairs) is
// enqueued behind the caller's copies; with host sizes the histogram work runs
// on the host while the copies are in flight, and one synchronisation ends it.
// Pinned host memory of at least `bytes`, kept by the context for
// device-to-host reads that must not wait on a pageable copy.
hyset_status host_stage(hyset_ctx* ctx, size_t bytes, void** out) {
    if (bytes > ctx->h_stage_bytes) {
        const size_t want = std::max(bytes, 2 * ctx->h_stage_bytes);
        if (ctx->h_stage) CK(cudaFreeHost(ctx->h_stage));
        ctx->h_stage = nullptr;
        ctx->h_stage_bytes = 0;
        CK(cudaMallocHost(&ctx->h_stage, want));
        ctx->h_stage_bytes = want;
    }
    *out = ctx->h_stage;
    return HYSET_OK;
}

// Enqueues the checks of a new collection (one pass over the tokens, which also
// writes the meta pairs) and the read-back of their flags (and of the sizes,
// when they are only on the device).  With host sizes the histogram work runs
// on the host while the copies and the check are in flight.
hyset_status enqueue_collection_checks(hyset_ctx* ctx, hyset_coll* c, const uint32_t* h_sizes_or_null) {
    cudaStream_t s = ctx->stream;
    if (!h_sizes_or_null && c->n) {
        void* stage = nullptr;
        ST(host_stage(ctx, (size_t)c->n * 4, &stage));
        CK(cudaMemcpyAsync(stage, c->d_sizes, (size_t)c->n * 4, cudaMemcpyDeviceToHost, s));
    }
    CK(ctx->s_flags.ensure(16, s));
    CK(cudaMemsetAsync(ctx->s_flags.p, 0, 16, s));
    CK(c->meta.ensure((size_t)c->n * sizeof(uint2) + 8, s));
    CK(validate_collection(c->view(), c->n_tokens, ctx->s_flags.as<uint32_t>(), c->meta.as<uint2>(), s));
    if (c->n && h_sizes_or_null) ST(build_size_meta(ctx, c, h_sizes_or_null));
    uint32_t* f = ctx->h_flags;
    f[0] = f[1] = 0;
    CK(cudaMemcpyAsync(f, ctx->s_flags.p, 8, cudaMemcpyDeviceToHost, s));
    return HYSET_OK;
}

// After the stream has synchronised: the verdict of the checks, then the host
// size statistics of a collection whose sizes came from the device.
hyset_status finish_collection_checks(hyset_ctx* ctx, hyset_coll* c, const uint32_t* h_sizes_or_null) {
    const uint32_t* f = ctx->h_flags;
    if (f[0] & 8) return fail(ctx, HYSET_E_INVALID, "a set reaches past the end of the token array");
    if (f[0] & 1) return fail(ctx, HYSET_E_INVALID, "empty set in collection");
    if (f[0] & 2) return fail(ctx, HYSET_E_INVALID, "set tokens must be strictly ascending");
    if (f[0] & 4) return fail(ctx, HYSET_E_INVALID, "sets must be ordered by non-decreasing size");
    if (f[1] == 0xFFFFFFFFu) return fail(ctx, HYSET_E_INVALID, "token 0xFFFFFFFF is reserved");
    c->universe = c->n ? f[1] + 1 : 1;
    if (!h_sizes_or_null || !c->n)
        ST(build_size_meta(ctx, c, c->n ? static_cast<const uint32_t*>(ctx->h_stage) : nullptr));
    return HYSET_OK;
}

hyset_status make_collection(hyset_ctx* ctx, hyset_coll* c, const uint32_t* h_sizes_or_null) {
    ST(enqueue_collection_checks(ctx, c, h_sizes_or_null));
    CK(cudaStreamSynchronize(ctx->stream));
    return finish_collection_checks(ctx, c, h_sizes_or_null);
}

// ---------------------------------------------------------------- batches

std::string opts_key(const hyset_join_desc& d) {
    std::string k((const char*)&d.indexed, sizeof(d.indexed));
    k.append((const char*)&d.probe, sizeof(d.probe));
    k.append((const char*)&d.opts, sizeof(d.opts));
    return k;
}

void batch_release(hyset_ctx* ctx) {
    if (!ctx->batch) return;
    BatchPlan& bp = *ctx->batch;
    cudaStream_t s = ctx->stream;
    if (bp.exec) cudaGraphExecDestroy(bp.exec);
    if (bp.graph) cudaGraphDestroy(bp.graph);
    for (auto& bj : bp.joins) {
        DevBuf* bufs[] = {&bj->ix.list_off, &bj->ix.set, &bj->ix.pos, &bj->ix_mid.list_off, &bj->ix_mid.set,
                          &bj->ix_mid.pos, &bj->bits_r, &bj->bits_s, &bj->pairs};
        for (DevBuf* d : bufs) d->release(s);
    }
    DevBuf* bufs[] = {&bp.desc, &bp.unit_off, &bp.counts, &bp.work};
    for (DevBuf* d : bufs) d->release(s);
    bp.sc.release(s);
    cudaStreamSynchronize(s);
    ctx->batch.reset();
}

// The device work of a batch: per join its index build and signatures, then
// one persistent launch over the units of every join.  Asynchronous only.
hyset_status batch_record(hyset_ctx* ctx, BatchPlan& bp) {
    cudaStream_t s = ctx->stream;
    const uint32_t n = (uint32_t)bp.joins.size();
    CK(cudaMemsetAsync(bp.counts.p, 0, n * sizeof(unsigned long long), s));
    CK(cudaMemsetAsync(bp.work.p, 0, 16, s));
    for (auto& bjp : bp.joins) {
        BatchJoin& bj = *bjp;
        if (bj.ktech == TECH_FGSS) {
            ST(build_sorted_index(ctx, bj.R, bj.b, bj.self ? 0 : 1, bj.ix));
            if (use_bands(bj.b, bj.self))
                ST(build_sorted_index(ctx, bj.R, bj.b, 2, bj.ix_mid, &bj.b->mid_prefix, bj.b->view.mid_prefix,
                                      (int)bj.ix.pos_bits));
        }
        if (bj.words) {
            CK(generate_bitmaps(bj.R->view(), bj.words, bj.bits_r.as<uint64_t>(), s));
            if (!bj.self) CK(generate_bitmaps(bj.S->view(), bj.words, bj.bits_s.as<uint64_t>(), s));
        }
    }
    CK(launch_batch_join(bp.desc.as<BatchDesc>(), bp.unit_off.as<uint32_t>(), n, bp.work.as<unsigned int>(),
                         ctx->sm_count, s));
    return HYSET_OK;
}

hyset_status batch_prepare(hyset_ctx* ctx, const hyset_join_desc* joins, uint32_t n) {
    std::vector<std::string> sig(n);
    for (uint32_t j = 0; j < n; ++j) sig[j] = opts_key(joins[j]);
    if (ctx->batch && ctx->batch->sig == sig) return HYSET_OK;  // same batch: replay its graph
    batch_release(ctx);
    auto plan = std::make_unique<BatchPlan>();
    plan->sig = sig;
    // index builds of the batch use the plan's own scratch, so later joins that
    // grow the context's scratch cannot free memory the graph still addresses
    struct ScratchSwitch {
        hyset_ctx* c;
        ~ScratchSwitch() { c->sc = &c->own; }
    } sw{ctx};
    ctx->sc = &plan->sc;
    cudaStream_t s = ctx->stream;
    std::vector<BatchDesc> desc(n);
    std::vector<double> cost(n);
    uint64_t maxE = 1, maxU = 1, maxN = 1;
    for (uint32_t j = 0; j < n; ++j) {
        const hyset_join_desc& d = joins[j];
        if (!d.indexed) return fail(ctx, HYSET_E_INVALID, "batch join without an indexed collection");
        auto bj = std::make_unique<BatchJoin>();
        bj->R = const_cast<hyset_coll*>(d.indexed);
        bj->S = const_cast<hyset_coll*>(d.probe ? d.probe : d.indexed);
        bj->self = bj->S == bj->R;
        bj->o = d.opts;
        ST(check_opts(ctx, &bj->o));
        bj->swapped = swap_sides(bj->R, bj->S, &bj->o);
        if (bj->swapped) std::swap(bj->R, bj->S);
        const hyset_join_opts* o = &bj->o;
        hyset_coll* R = bj->R;
        hyset_coll* S = bj->S;
        if (o->probe_end > S->n || o->probe_begin > o->probe_end)
            return fail(ctx, HYSET_E_INVALID, "probe range outside the probe collection");
        const uint32_t L = std::max(R->max_size, S->max_size);
        ST(get_bounds(ctx, o->sim, o->threshold, L, bj->self ? 0 : 1, &bj->b));
        hyset_technique selected = HYSET_TECH_AUTO;
        int selector = 0;
        ST(select_technique(ctx, R, S, o, &selected, &selector));
        Tuned tn = tune(R, S, o, selected);
        tn.probe_major = 1;  // the batched kernel runs the probe-major form
        {
            const uint32_t a_lo = o->probe_end ? o->probe_begin : 0, a_hi = o->probe_end ? o->probe_end : S->n;
            if (o->technique == HYSET_TECH_AUTO && o->bitmap_bits == 0 && tn.tech == HYSET_TECH_FGSS &&
                a_hi - a_lo >= TUNE_MIN_PROBES)
                ST(autotune_bits(ctx, R, S, o, bj->b, bj->self, a_lo, a_hi, &tn.bits));
        }
        bj->tech = tn.tech;
        bj->ktech = tn.tech == HYSET_TECH_FGSS ? TECH_FGSS : (tn.tech == HYSET_TECH_DIRECT ? TECH_DIRECT : TECH_BITMAP);
        bj->words = (int)(tn.bits / 64);
        if (bj->ktech == TECH_DIRECT) bj->words = 0;
        JoinParams& P = desc[j].P;
        P = JoinParams{};
        P.R = R->view();
        P.S = S->view();
        P.B = bj->b->view;
        P.first_ge = R->first_ge.as<uint32_t>();
        P.R_L = R->max_size;
        P.self = bj->self ? 1 : 0;
        P.p_lo = o->probe_end ? o->probe_begin : 0;
        P.p_hi = o->probe_end ? o->probe_end : S->n;
        P.r_lo = 0;
        P.r_hi = R->n;
        P.grab = 1;
        if (bj->ktech == TECH_FGSS) {
            const uint64_t E = prefix_entries(R, bj->b->index_prefix);
            if (E >= (1ull << 32)) return fail(ctx, HYSET_E_UNSUPPORTED, "more than 2^32 prefix entries");
            maxE = std::max<uint64_t>(maxE, E);
            maxU = std::max<uint64_t>(maxU, (uint64_t)R->universe + 1);
            maxN = std::max<uint64_t>(maxN, R->n);
            CK(bj->ix.list_off.ensure(((size_t)R->universe + 1) * 4, s));
            CK(bj->ix.set.ensure((E ? E : 1) * 4, s));
            CK(bj->ix.pos.ensure((E ? E : 1) * 4, s));
            uint32_t max_pre = 1;
            for (size_t l = 0; l < R->size_hist.size(); ++l)
                if (R->size_hist[l]) max_pre = std::max(max_pre, pre_len(bj->b, (uint32_t)l));
            const uint32_t pb = bits_for(max_pre), sb = bits_for(R->n);
            bj->ix.universe = R->universe;
            bj->ix.pos_bits = pb + sb <= 32 ? pb : 0;
            P.X = bj->ix.view();
            if (use_bands(bj->b, bj->self)) {  // the midprefix index, same layout
                const uint64_t E2 = prefix_entries(R, bj->b->mid_prefix);
                CK(bj->ix_mid.list_off.ensure(((size_t)R->universe + 1) * 4, s));
                CK(bj->ix_mid.set.ensure((E2 ? E2 : 1) * 4, s));
                CK(bj->ix_mid.pos.ensure((E2 ? E2 : 1) * 4, s));
                bj->ix_mid.universe = R->universe;
                bj->ix_mid.pos_bits = bj->ix.pos_bits;
                P.X2 = bj->ix_mid.view();
            }
        }
        if (bj->words) {
            CK(bj->bits_r.ensure((size_t)R->n * bj->words * 8 + 8, s));
            if (!bj->self) CK(bj->bits_s.ensure((size_t)S->n * bj->words * 8 + 8, s));
            P.bits_R = bj->bits_r.as<uint64_t>();
            P.bits_S = bj->self ? P.bits_R : bj->bits_s.as<uint64_t>();
            P.words = bj->words;
        }
        bj->cap = o->count_only ? 0 : (o->pair_capacity ? o->pair_capacity : std::max<uint64_t>(4096, 2ull * S->n));
        if (!o->count_only) CK(bj->pairs.ensure(std::max<uint64_t>(bj->cap, 1) * sizeof(uint2), s));
        desc[j].tech = (uint32_t)bj->ktech;
        desc[j].words = (uint32_t)bj->words;
        desc[j].unit_probes = bj->ktech == TECH_FGSS ? std::min<uint32_t>(tn.batch, P.X2.set ? 16 : 32) : 1;
        const uint32_t np = P.p_hi - P.p_lo;
        bj->units = (np + desc[j].unit_probes - 1) / desc[j].unit_probes;
        cost[j] = (double)np * (double)(R->n_tokens / std::max<uint32_t>(R->n, 1) + 1) *
                  (bj->ktech == TECH_FGSS ? 1.0 : (double)R->n);
        plan->joins.push_back(std::move(bj));
    }
    // scratch for the largest index build, sized before capture
    CK(ctx->sc->len.ensure((size_t)maxN * 4 + 4, s));
    CK(ctx->sc->off.ensure((size_t)maxN * 4 + 4, s));
    const size_t e4 = (size_t)maxE * 4;
    CK(ctx->sc->tok.ensure(e4, s));
    CK(ctx->sc->set.ensure(e4, s));
    CK(ctx->sc->pos.ensure(e4, s));
    CK(ctx->sc->order.ensure(e4, s));
    CK(ctx->sc->altk.ensure(e4, s));
    CK(ctx->sc->altv.ensure(e4, s));
    CK(ctx->sc->gate.ensure(4, s));
    CK(ctx->sc->counts.ensure((size_t)maxU * 4, s));
    const size_t scan_words = std::max(std::max(scan_scratch_words(maxN), scan_scratch_words(maxU)),
                                       radix_scratch_words(maxE));
    CK(ctx->sc->scan.ensure(scan_words * 4, s));
    // heaviest joins first, so the tail of the launch is light
    plan->order.resize(n);
    for (uint32_t j = 0; j < n; ++j) plan->order[j] = j;
    std::stable_sort(plan->order.begin(), plan->order.end(), [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
    CK(plan->counts.ensure(n * sizeof(unsigned long long), s));
    CK(plan->work.ensure(16, s));
    std::vector<BatchDesc> ordered(n);
    std::vector<uint32_t> unit_off(n + 1, 0);
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t j = plan->order[k];
        ordered[k] = desc[j];
        BatchJoin& bj = *plan->joins[j];
        ordered[k].P.out = Sink{bj.o.count_only ? nullptr : bj.pairs.as<uint2>(),
                                plan->counts.as<unsigned long long>() + j, bj.cap, bj.o.count_only ? 1 : 0,
                                bj.swapped ? 1 : 0};
        unit_off[k + 1] = unit_off[k] + bj.units;
    }
    CK(plan->desc.ensure(n * sizeof(BatchDesc), s));
    CK(plan->unit_off.ensure((n + 1) * 4, s));
    CK(cudaMemcpyAsync(plan->desc.p, ordered.data(), n * sizeof(BatchDesc), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(plan->unit_off.p, unit_off.data(), (n + 1) * 4, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    ctx->batch = std::move(plan);
    BatchPlan& bp = *ctx->batch;
    // indexes whose list path is not known yet are built once here, outside
    // the capture, so that the path is read back and remembered: the graph then
    // holds only the kernels of the path each index takes
    for (auto& bjp : bp.joins) {
        BatchJoin& bj = *bjp;
        if (bj.ktech != TECH_FGSS) continue;
        const uint32_t* index_tab = bj.b->view.index_prefix;
        const uint32_t* mid_tab = bj.b->view.mid_prefix;
        if (!bj.R->list_path.count(index_tab)) ST(build_sorted_index(ctx, bj.R, bj.b, bj.self ? 0 : 1, bj.ix));
        if (use_bands(bj.b, bj.self) && !bj.R->list_path.count(mid_tab))
            ST(build_sorted_index(ctx, bj.R, bj.b, 2, bj.ix_mid, &bj.b->mid_prefix, bj.b->view.mid_prefix,
                                  (int)bj.ix.pos_bits));
    }
    // capture the device work once; later calls with the same batch replay it
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    hyset_status st = batch_record(ctx, bp);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (st != HYSET_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        batch_release(ctx);
        return st != HYSET_OK ? st : fail(ctx, HYSET_E_CUDA, "batch graph capture", e);
    }
    bp.graph = g;
    e = cudaGraphInstantiate(&bp.exec, g, 0);
    if (e != cudaSuccess) {
        batch_release(ctx);
        return fail(ctx, HYSET_E_CUDA, "batch graph instantiation", e);
    }
    return HYSET_OK;
}

}  // namespace


// ====================================================================== ABI

extern "C" {

void hyset_default_opts(hyset_join_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->sim = HYSET_JACCARD;
    o->threshold = 0.8;
    o->technique = HYSET_TECH_AUTO;
}

hyset_status hyset_create(int device, hyset_ctx** out) {
    if (!out) return HYSET_E_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return HYSET_E_NODEVICE;
    }
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return HYSET_E_NODEVICE;
    if (device >= count) return HYSET_E_INVALID;
    hyset_ctx* ctx = new (std::nothrow) hyset_ctx();
    if (!ctx) return HYSET_E_NOMEM;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = prepare_kernels();
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ek0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ek1);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&ctx->h_flags, 64);
    if (e == cudaSuccess) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    if (e != cudaSuccess) {
        hyset_destroy(ctx);
        return HYSET_E_CUDA;
    }
    *out = ctx;
    return HYSET_OK;
}

void hyset_destroy(hyset_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) {
        cudaStream_t s = ctx->stream;
        batch_release(ctx);
        for (auto& kv : ctx->bounds) kv.second->dev.release(s);
        ctx->own.release(s);
        DevBuf* bufs[] = {&ctx->s_pairs, &ctx->s_count, &ctx->s_work, &ctx->s_stats, &ctx->s_flags,
                          &ctx->d_mlp, &ctx->d_feat, &ctx->d_moments, &ctx->d_hist};
        for (DevBuf* b : bufs) b->release(s);
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    if (ctx->aux) {
        cudaStreamSynchronize(ctx->aux);
        cudaStreamDestroy(ctx->aux);
    }
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    for (cudaEvent_t e : ctx->pipe_ev) cudaEventDestroy(e);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->ek0) cudaEventDestroy(ctx->ek0);
    if (ctx->ek1) cudaEventDestroy(ctx->ek1);
    if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    delete ctx;
}

const char* hyset_last_error(const hyset_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

hyset_status hyset_collection_upload(hyset_ctx* ctx, const uint32_t* tokens, uint64_t n_tokens,
                                     const uint32_t* starts, const uint32_t* sizes, uint32_t n_sets,
                                     hyset_coll** out) {
    if (!ctx || !out || (n_sets && (!sizes || (!tokens && n_tokens))))
        return fail(ctx, HYSET_E_INVALID, "null argument");
    if (n_tokens >= (1ull << 32)) return fail(ctx, HYSET_E_INVALID, "n_tokens must be < 2^32");
    *out = nullptr;
    CK(cudaSetDevice(ctx->device));
    auto c = std::make_unique<hyset_coll>();
    c->ctx = ctx;
    c->n = n_sets;
    c->n_tokens = n_tokens;
    cudaStream_t s = ctx->stream;
    std::vector<uint32_t> st;
    if (!starts && n_sets) {
        st.resize(n_sets);
        uint64_t run = 0;
        for (uint32_t i = 0; i < n_sets; ++i) {
            st[i] = (uint32_t)run;
            run += sizes[i];
        }
        if (run > n_tokens) return fail(ctx, HYSET_E_INVALID, "sizes sum past n_tokens");
        starts = st.data();
    }
    CK(c->tokens.ensure(n_tokens * 4 + 4, s));
    CK(c->starts.ensure((size_t)n_sets * 4 + 4, s));
    CK(c->sizes.ensure((size_t)n_sets * 4 + 4, s));
    if (n_tokens) CK(cudaMemcpyAsync(c->tokens.p, tokens, n_tokens * 4, cudaMemcpyHostToDevice, s));
    if (n_sets) {
        CK(cudaMemcpyAsync(c->starts.p, starts, (size_t)n_sets * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(c->sizes.p, sizes, (size_t)n_sets * 4, cudaMemcpyHostToDevice, s));
    }
    c->d_tokens = c->tokens.as<uint32_t>();
    c->d_starts = c->starts.as<uint32_t>();
    c->d_sizes = c->sizes.as<uint32_t>();
    hyset_status stt = make_collection(ctx, c.get(), sizes);
    if (stt != HYSET_OK) {
        hyset_collection_free(ctx, c.release());
        return stt;
    }
    *out = c.release();
    return HYSET_OK;
}

hyset_status hyset_collection_from_device(hyset_ctx* ctx, const uint32_t* d_tokens, uint64_t n_tokens,
                                          const uint32_t* d_starts, const uint32_t* d_sizes, uint32_t n_sets,
                                          hyset_coll** out) {
    if (!ctx || !out || (n_sets && (!d_sizes || !d_starts || !d_tokens)))
        return fail(ctx, HYSET_E_INVALID, "null argument");
    if (n_tokens >= (1ull << 32)) return fail(ctx, HYSET_E_INVALID, "n_tokens must be < 2^32");
    *out = nullptr;
    CK(cudaSetDevice(ctx->device));
    auto c = std::make_unique<hyset_coll>();
    c->ctx = ctx;
    c->n = n_sets;
    c->n_tokens = n_tokens;
    c->d_tokens = d_tokens;
    c->d_starts = d_starts;
    c->d_sizes = d_sizes;
    hyset_status stt = make_collection(ctx, c.get(), nullptr);
    if (stt != HYSET_OK) {
        hyset_collection_free(ctx, c.release());
        return stt;
    }
    *out = c.release();
    return HYSET_OK;
}

namespace {
constexpr uint64_t PIPE_CHUNK_TOKENS = 16ull << 20;  // 64 MB of tokens per copy chunk

cudaEvent_t pipe_event(hyset_ctx* ctx, size_t k) {
    while (ctx->pipe_ev.size() <= k) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        ctx->pipe_ev.push_back(e);
    }
    return ctx->pipe_ev[k];
}
}  // namespace

hyset_status hyset_collection_parse(hyset_ctx* ctx, const char* text, uint64_t n_bytes, hyset_coll** out) {
    if (!ctx || !out || (n_bytes && !text)) return fail(ctx, HYSET_E_INVALID, "null argument");
    if (n_bytes >= (1ull << 33)) return fail(ctx, HYSET_E_UNSUPPORTED, "text of 2^33 bytes or more");
    *out = nullptr;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    // the text: used in place when it is device memory, else copied
    const uint8_t* d_text = reinterpret_cast<const uint8_t*>(text);
    DevBuf staged, counts, err;
    struct Release {  // scratch goes back to the pool on every return path
        DevBuf* b[3];
        cudaStream_t s;
        ~Release() {
            for (DevBuf* d : b) d->release(s);
        }
    } rel{{&staged, &counts, &err}, s};
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, text) != cudaSuccess) cudaGetLastError();
    // host text travels in 64 MB chunks on the auxiliary stream; the tiles of a
    // chunk are counted once it and the next chunk (a tile reads one byte past
    // its end) have landed, so counting overlaps the copy
    constexpr uint64_t PARSE_CHUNK = 64ull << 20;  // a multiple of the 4 KiB tile
    uint64_t n_chunks = 0;
    if (n_bytes && attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) {
        CK(staged.ensure(n_bytes + 16, s));
        CK(cudaEventRecord(ctx->ev_fork, s));
        CK(cudaStreamWaitEvent(ctx->aux, ctx->ev_fork, 0));
        n_chunks = (n_bytes + PARSE_CHUNK - 1) / PARSE_CHUNK;
        for (uint64_t k = 0; k < n_chunks; ++k) {
            const uint64_t b0 = k * PARSE_CHUNK, b1 = std::min(n_bytes, b0 + PARSE_CHUNK);
            CK(cudaMemcpyAsync(staged.as<uint8_t>() + b0, text + b0, b1 - b0, cudaMemcpyHostToDevice, ctx->aux));
            cudaEvent_t e = pipe_event(ctx, k);
            if (!e) {
                cudaStreamSynchronize(ctx->aux);
                return fail(ctx, HYSET_E_CUDA, "event creation");
            }
            CK(cudaEventRecord(e, ctx->aux));
        }
        d_text = staged.as<uint8_t>();
    }
    if (n_bytes && (reinterpret_cast<uintptr_t>(d_text) & 15u)) {  // tiles load 16-byte words
        DevBuf aligned;
        CK(aligned.ensure(n_bytes + 16, s));
        CK(cudaMemcpyAsync(aligned.p, d_text, n_bytes, cudaMemcpyDeviceToDevice, s));
        staged.release(s);
        staged = aligned;
        aligned.p = nullptr;
        d_text = staged.as<uint8_t>();
    }
    const uint64_t tiles = parse_tiles(n_bytes);
    CK(counts.ensure((2 * tiles + 2) * 4 + (2 * n_chunks + 2) * 4, s));
    CK(err.ensure(16, s));
    uint32_t* tile_toks = counts.as<uint32_t>();
    uint32_t* tile_lines = tile_toks + tiles + 1;
    uint32_t* carry = tile_lines + tiles + 1;  // per chunk: tokens and lines before it
    uint32_t* flags = err.as<uint32_t>();
    unsigned long long* first_bad = reinterpret_cast<unsigned long long*>(err.as<uint8_t>() + 8);
    CK(cudaMemsetAsync(flags, 0, 8, s));
    CK(cudaMemsetAsync(first_bad, 0xFF, 8, s));
    CK(cudaMemsetAsync(tile_toks, 0, (2 * tiles + 2) * 4 + (2 * n_chunks + 2) * 4, s));
    uint32_t* h = ctx->h_flags + 8;  // [0] flags, [2..3] first bad offset, [4] tokens, [5] lines
    auto parse_error = [&](uint32_t f, unsigned long long at) {
        char msg[160];
        const char* what = (f & PARSE_E_CHAR) ? "unexpected byte"
                           : (f & PARSE_E_EMPTY_ITEM) ? "empty item (two spaces, a leading space or a space before CR)"
                           : (f & PARSE_E_LINE_END) ? "CR not ending a line, or a line of only CR"
                                                    : "number of more than 10 digits or >= 2^32";
        std::snprintf(msg, sizeof msg, "parse error at byte %llu: %s", at, what);
        return fail(ctx, HYSET_E_INVALID, msg);
    };
    auto c = std::make_unique<hyset_coll>();
    c->ctx = ctx;
    struct CollGuard {  // the collection's buffers go back on every early return
        hyset_ctx* ctx;
        std::unique_ptr<hyset_coll>& c;
        ~CollGuard() {
            if (c) hyset_collection_free(ctx, c.release());
        }
    } cguard{ctx, c};
    uint32_t n_tokens = 0, n_lines = 0;
    if (n_chunks) {
        // each chunk is counted, scanned on top of the previous chunks' totals
        // and emitted as soon as it and the next chunk have landed, so the
        // whole parse overlaps the copy.  The output is sized from the first
        // chunk's density (one wait); a text denser further on overflows that
        // estimate and is emitted again at its exact size.
        const uint64_t per = PARSE_CHUNK / 4096;  // tiles per chunk
        uint32_t tok_cap = 0, line_cap = 0;
        for (uint64_t k = 0; k < n_chunks; ++k) {
            CK(cudaStreamWaitEvent(s, pipe_event(ctx, std::min(k + 1, n_chunks - 1)), 0));
            CK(parse_count(d_text, n_bytes, tile_toks, tile_lines, flags, first_bad, s, k * per, (k + 1) * per));
            CK(parse_chunk_scan(tile_toks, tile_lines, k * per, std::min(tiles, (k + 1) * per), carry, k, s));
            if (k == 0) {
                CK(cudaMemcpyAsync(h + 4, carry + 2, 8, cudaMemcpyDeviceToHost, s));
                CK(cudaStreamSynchronize(s));
                const double scale = (double)n_bytes / (double)std::min<uint64_t>(n_bytes, PARSE_CHUNK);
                const double bound = (double)(n_bytes / 2 + 2);  // a token or a line takes two bytes
                tok_cap = (uint32_t)std::min({bound, 1.25 * scale * h[4] + 4096.0, 4294967295.0});
                line_cap = (uint32_t)std::min({bound, 1.25 * scale * h[5] + 4096.0, 4294967295.0});
                CK(c->tokens.ensure((size_t)tok_cap * 4 + 4, s));
                CK(c->starts.ensure((size_t)line_cap * 4 + 4, s));
            }
            CK(parse_emit(d_text, n_bytes, tile_toks, tile_lines, c->tokens.as<uint32_t>(), c->starts.as<uint32_t>(),
                          flags, first_bad, s, k * per, (k + 1) * per, tok_cap, line_cap));
        }
        CK(cudaMemcpyAsync(h, err.p, 16, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(h + 4, carry + 2 * n_chunks, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (h[0] & ~PARSE_E_CAPACITY) return parse_error(h[0], *reinterpret_cast<unsigned long long*>(h + 2));
        n_tokens = h[4];
        n_lines = h[5];
        if (h[0] & PARSE_E_CAPACITY) {  // the estimate was short: every tile again, exact sizes
            CK(c->tokens.ensure((size_t)n_tokens * 4 + 4, s));
            CK(c->starts.ensure((size_t)n_lines * 4 + 4, s));
            CK(cudaMemsetAsync(flags, 0, 4, s));
            CK(parse_emit(d_text, n_bytes, tile_toks, tile_lines, c->tokens.as<uint32_t>(), c->starts.as<uint32_t>(),
                          flags, first_bad, s));
        }
        c->n = n_lines;
        c->n_tokens = n_tokens;
        CK(c->sizes.ensure((size_t)n_lines * 4 + 4, s));
    } else {
        CK(parse_count(d_text, n_bytes, tile_toks, tile_lines, flags, first_bad, s));
        CK(ctx->sc->scan.ensure(scan_scratch_words(tiles + 1) * 4, s));
        CK(scan_exclusive(tile_toks, tile_toks, tiles + 1, ctx->sc->scan.as<uint32_t>(), s));
        CK(scan_exclusive(tile_lines, tile_lines, tiles + 1, ctx->sc->scan.as<uint32_t>(), s));
        CK(cudaMemcpyAsync(h, err.p, 16, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(h + 4, tile_toks + tiles, 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(h + 5, tile_lines + tiles, 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (h[0]) return parse_error(h[0], *reinterpret_cast<unsigned long long*>(h + 2));
        n_tokens = h[4];
        n_lines = h[5];
        c->n = n_lines;
        c->n_tokens = n_tokens;
        CK(c->tokens.ensure((size_t)n_tokens * 4 + 4, s));
        CK(c->starts.ensure((size_t)n_lines * 4 + 4, s));
        CK(c->sizes.ensure((size_t)n_lines * 4 + 4, s));
        CK(parse_emit(d_text, n_bytes, tile_toks, tile_lines, c->tokens.as<uint32_t>(), c->starts.as<uint32_t>(),
                      flags, first_bad, s));
    }
    CK(parse_line_sizes(c->starts.as<uint32_t>(), n_lines, n_tokens, c->starts.as<uint32_t>(),
                        c->sizes.as<uint32_t>(), s));
    CK(cudaMemcpyAsync(h, err.p, 16, cudaMemcpyDeviceToHost, s));
    c->d_tokens = c->tokens.as<uint32_t>();
    c->d_starts = c->starts.as<uint32_t>();
    c->d_sizes = c->sizes.as<uint32_t>();
    // the collection checks go behind the parse on the stream: one synchronisation
    hyset_status stt = enqueue_collection_checks(ctx, c.get(), nullptr);
    if (stt == HYSET_OK) {
        CK(cudaStreamSynchronize(s));
        if (h[0]) stt = parse_error(h[0], *reinterpret_cast<unsigned long long*>(h + 2));
        else stt = finish_collection_checks(ctx, c.get(), nullptr);
    }
    if (stt != HYSET_OK) {
        hyset_collection_free(ctx, c.release());
        return stt;
    }
    *out = c.release();
    return HYSET_OK;
}

uint64_t hyset_collection_num_tokens(const hyset_coll* c) { return c ? c->n_tokens : 0; }

hyset_status hyset_collection_download(hyset_ctx* ctx, const hyset_coll* c, uint32_t* tokens, uint32_t* starts,
                                       uint32_t* sizes) {
    if (!ctx || !c) return fail(ctx, HYSET_E_INVALID, "null argument");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    if (tokens && c->n_tokens) CK(cudaMemcpyAsync(tokens, c->d_tokens, c->n_tokens * 4, cudaMemcpyDeviceToHost, s));
    if (starts && c->n) CK(cudaMemcpyAsync(starts, c->d_starts, (size_t)c->n * 4, cudaMemcpyDeviceToHost, s));
    if (sizes && c->n) CK(cudaMemcpyAsync(sizes, c->d_sizes, (size_t)c->n * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return HYSET_OK;
}

void hyset_collection_free(hyset_ctx* ctx, hyset_coll* c) {
    if (!c) return;
    hyset_ctx* owner = ctx ? ctx : c->ctx;
    if (owner && owner->batch) {  // a captured batch that reads this collection is dropped with it
        for (const auto& bj : owner->batch->joins)
            if (bj->R == c || bj->S == c) {
                batch_release(owner);
                break;
            }
    }
    cudaStream_t s = ctx ? ctx->stream : c->ctx->stream;
    c->tokens.release(s);
    c->starts.release(s);
    c->sizes.release(s);
    c->meta.release(s);
    c->index.list_off.release(s);
    c->index.set.release(s);
    c->index.pos.release(s);
    c->index_mid.list_off.release(s);
    c->index_mid.set.release(s);
    c->index_mid.pos.release(s);
    c->first_ge.release(s);
    c->g_off.release(s);
    c->g_set.release(s);
    c->g_ps.release(s);
    c->g_cursor.release(s);
    for (auto& kv : c->bitmaps) kv.second.release(s);
    cudaStreamSynchronize(s);
    delete c;
}

uint32_t hyset_collection_num_sets(const hyset_coll* c) { return c ? c->n : 0; }

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

// ---------------------------------------------------------------- joins from host arrays



// The upload and the self-join in one call.  The tokens go to the device in
// 64 MB chunks on the auxiliary stream; while the later chunks are in flight,
// the sets of the chunks already on the device are checked, their prefix
// entries emitted and their signatures generated on the context's stream.
// After the last chunk only the index sort and the join launch remain.  The
// pipeline needs the join's configuration before the tokens arrive: an explicit
// probe-major prefix-index join, or one whose technique and signature width
// the context has already chosen for a collection with the same size profile;
// every other join runs as hyset_collection_upload + hyset_self_join.
hyset_status hyset_self_join_host(hyset_ctx* ctx, const uint32_t* tokens, uint64_t n_tokens, const uint32_t* starts,
                                  const uint32_t* sizes, uint32_t n_sets, const hyset_join_opts* opts,
                                  hyset_coll** coll_out, hyset_result** out) {
    if (!ctx || !out || !opts || (n_sets && (!sizes || (!tokens && n_tokens))))
        return fail(ctx, HYSET_E_INVALID, "null argument");
    *out = nullptr;
    if (coll_out) *coll_out = nullptr;
    ST(check_opts(ctx, opts));
    if (n_tokens >= (1ull << 32)) return fail(ctx, HYSET_E_INVALID, "n_tokens must be < 2^32");
    if (opts->probe_end) return fail(ctx, HYSET_E_INVALID, "probe ranges need an uploaded collection");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream, cp = ctx->aux;
    auto res = std::make_unique<hyset_result>();
    auto c = std::make_unique<hyset_coll>();
    c->ctx = ctx;
    c->n = n_sets;
    c->n_tokens = n_tokens;
    hyset_coll* C = c.get();
    auto bail = [&](hyset_status st) {
        cudaStreamSynchronize(cp);
        hyset_collection_free(ctx, c.release());
        return st;
    };
    const unsigned long long launches0 = launches();
    CK(cudaEventRecord(ctx->ev0, s));
    if (C->tokens.ensure(n_tokens * 4 + 4, s) != cudaSuccess || C->starts.ensure((size_t)n_sets * 4 + 4, s) ||
        C->sizes.ensure((size_t)n_sets * 4 + 4, s) || C->meta.ensure((size_t)n_sets * sizeof(uint2) + 8, s))
        return bail(fail(ctx, HYSET_E_NOMEM, "device allocation"));
    C->d_tokens = C->tokens.as<uint32_t>();
    C->d_starts = C->starts.as<uint32_t>();
    C->d_sizes = C->sizes.as<uint32_t>();
    // 1. on the copy stream: the sizes (and starts, when given) first, then every
    //    token chunk with an event after each; the sizes go first so the
    //    per-set work is not queued behind the tokens on the copy engine
    CK(cudaEventRecord(ctx->ev_fork, s));
    CK(cudaStreamWaitEvent(cp, ctx->ev_fork, 0));
    const bool starts_given = starts != nullptr;
    if (n_sets) {
        CK(cudaMemcpyAsync(C->sizes.p, sizes, (size_t)n_sets * 4, cudaMemcpyHostToDevice, cp));
        if (starts_given) CK(cudaMemcpyAsync(C->starts.p, starts, (size_t)n_sets * 4, cudaMemcpyHostToDevice, cp));
    }
    CK(cudaEventRecord(ctx->ev_join, cp));
    CK(cudaStreamWaitEvent(s, ctx->ev_join, 0));
    if (!starts_given && n_sets) {  // contiguous sets: starts are the exclusive scan of the sizes
        CK(ctx->sc->scan.ensure(scan_scratch_words(n_sets) * 4, s));
        CK(scan_exclusive(C->d_sizes, C->starts.as<uint32_t>(), n_sets, ctx->sc->scan.as<uint32_t>(), s));
    }
    const uint64_t n_chunks = n_tokens ? (n_tokens + PIPE_CHUNK_TOKENS - 1) / PIPE_CHUNK_TOKENS : 0;
    for (uint64_t k = 0; k < n_chunks; ++k) {
        const uint64_t t0 = k * PIPE_CHUNK_TOKENS, t1 = std::min(n_tokens, t0 + PIPE_CHUNK_TOKENS);
        CK(cudaMemcpyAsync(C->tokens.as<uint32_t>() + t0, tokens + t0, (t1 - t0) * 4, cudaMemcpyHostToDevice, cp));
        cudaEvent_t e = pipe_event(ctx, k);
        if (!e) return bail(fail(ctx, HYSET_E_CUDA, "event creation"));
        CK(cudaEventRecord(e, cp));
    }
    // 2. on the host meanwhile, one pass over the sizes: contiguity of the given
    //    starts, size order, and for every chunk the first set that ends past it
    //    (sets before it are complete once the chunk has landed)
    bool contiguous = true, ordered = true;
    std::vector<uint32_t> chunk_hi(n_chunks, n_sets);
    {
        uint64_t run = 0, bound = PIPE_CHUNK_TOKENS, k = 0;
        uint32_t prev = 0;
        for (uint32_t i = 0; i < n_sets; ++i) {
            const uint32_t z = sizes[i];
            if (starts_given) contiguous &= starts[i] == run;
            ordered &= z >= prev;
            prev = z;
            const uint64_t end = run + z;
            while (k < n_chunks && end > bound) {
                chunk_hi[k++] = i;
                bound += PIPE_CHUNK_TOKENS;
            }
            run = end;
        }
        if (!starts_given && run > n_tokens) return bail(fail(ctx, HYSET_E_INVALID, "sizes sum past n_tokens"));
    }
    if (!ordered) return bail(fail(ctx, HYSET_E_INVALID, "sets must be ordered by non-decreasing size"));
    ST(build_size_meta(ctx, C, sizes));
    // 3. the configuration, from the options or the context's earlier choices
    const hyset_join_opts* o = opts;
    bool pipelined = contiguous && n_sets > 0;
    hyset_technique selected = HYSET_TECH_AUTO;
    int selector = -1;
    const std::string key = join_key(C, C, o);
    if (o->technique == HYSET_TECH_AUTO) {
        auto it = ctx->select_cache.find(key);
        if (it == ctx->select_cache.end()) pipelined = false;
        else {
            selected = it->second.first;
            selector = it->second.second;
        }
    }
    Tuned tn = tune(C, C, o, selected);
    if (tn.tech != HYSET_TECH_FGSS || !tn.probe_major) pipelined = false;
    if (o->technique == HYSET_TECH_AUTO && o->bitmap_bits == 0 && n_sets >= TUNE_MIN_PROBES) {
        auto it = ctx->bits_cache.find(key);
        if (it == ctx->bits_cache.end()) pipelined = false;
        else {
            tn.bits = it->second & 0xFFFFu;
            if (!o->verify_mode && (it->second >> 16)) tn.vmode = (int)(it->second >> 16);
        }
    }
    Bounds* b = nullptr;
    ST(get_bounds(ctx, o->sim, o->threshold, C->max_size, 0, &b));
    uint32_t max_pre = 1;
    for (size_t l = 0; l < C->size_hist.size(); ++l)
        if (C->size_hist[l]) max_pre = std::max(max_pre, b->index_prefix[l]);
    const uint32_t pb = bits_for(max_pre);
    const uint64_t E = prefix_entries(C, b->index_prefix);
    if (pb + bits_for(n_sets) > 32 || E >= (1ull << 32)) pipelined = false;  // packed layout only
    if (!pipelined) {
        // the plain sequence: all tokens, the checks, then the join
        CK(cudaStreamWaitEvent(s, pipe_event(ctx, n_chunks ? n_chunks - 1 : 0), 0));
        hyset_status stt = enqueue_collection_checks(ctx, C, sizes);
        if (stt == HYSET_OK) {
            CK(cudaStreamSynchronize(s));
            stt = finish_collection_checks(ctx, C, sizes);
        }
        if (stt == HYSET_OK) stt = do_join(ctx, C, C, o, res.get());
        if (stt != HYSET_OK) return bail(stt);
    } else {
        // 4. per chunk: checks, prefix entries (no histogram yet) and signatures
        const uint32_t n = n_sets;
        CK(ctx->sc->len.ensure((size_t)n * 4 + 4, s));
        CK(ctx->sc->off.ensure((size_t)n * 4 + 4, s));
        CK(ctx->sc->tok.ensure(E ? E * 4 : 4, s));
        CK(ctx->sc->altk.ensure(E ? E * 4 : 4, s));
        CK(ctx->sc->altv.ensure(E ? E * 4 : 4, s));
        CK(ctx->sc->gate.ensure(4, s));
        Index& ix = C->index;
        CK(ix.set.ensure(E ? E * 4 : 4, s));
        CK(ix.pos.ensure(4, s));
        CK(ctx->s_flags.ensure(16, s));
        CK(cudaMemsetAsync(ctx->s_flags.p, 0, 16, s));
        const size_t scan_words = std::max(scan_scratch_words(n), radix_scratch_words(E ? E : 1));
        CK(ctx->sc->scan.ensure(scan_words * 4, s));
        uint32_t* len = ctx->sc->len.as<uint32_t>();
        uint32_t* off = ctx->sc->off.as<uint32_t>();
        CollView v = C->view();
        CK(set_prefix_lengths(v, b->view.index_prefix, 0, n, len, s));
        CK(scan_exclusive(len, off, n, ctx->sc->scan.as<uint32_t>(), s));
        const int words = (int)(tn.bits / 64);
        DevBuf& bits = C->bitmaps[words];
        if (words) CK(bits.ensure((size_t)n * words * 8 + 8, s));
        // A collection with the same size profile joined before: its universe
        // is assumed, so the token histogram is counted as the chunks land and
        // the checks are read after the join (one synchronisation); a larger
        // token than assumed means the index is built again and the join re-run.
        const std::string ukey = coll_signature(C);
        auto uit = ctx->universe_cache.find(ukey);
        bool assumed = uit != ctx->universe_cache.end();
        uint32_t U = assumed ? uit->second : 0;
        uint32_t* counts = nullptr;
        if (assumed) {
            CK(ctx->sc->counts.ensure(((size_t)U + 1) * 4, s));
            counts = ctx->sc->counts.as<uint32_t>();
            CK(cudaMemsetAsync(counts, 0, ((size_t)U + 1) * 4, s));
        }
        uint32_t lo = 0;
        for (uint64_t k = 0; k < n_chunks && lo < n; ++k) {
            // sets whose tokens end inside the chunks copied so far
            const uint32_t hi = k + 1 == n_chunks ? n : std::max(lo, chunk_hi[k]);
            CK(cudaStreamWaitEvent(s, pipe_event(ctx, k), 0));
            if (hi <= lo) continue;
            CollView part = v;
            part.sizes += lo;
            part.starts += lo;
            part.meta += lo;
            part.n = hi - lo;
            CK(validate_collection(part, n_tokens, ctx->s_flags.as<uint32_t>(), C->meta.as<uint2>() + lo, s));
            CK(emit_packed_entries(v, off, len, pb, ctx->sc->tok.as<uint32_t>(), ix.set.as<uint32_t>(), counts, s, lo,
                                   hi, U + 1));
            if (words) CK(generate_bitmaps(part, words, bits.as<uint64_t>() + (size_t)lo * words, s));
            lo = hi;
        }
        if (n_chunks) CK(cudaStreamWaitEvent(s, pipe_event(ctx, n_chunks - 1), 0));  // every copy has landed
        // 5. the index and the join.  The universe (largest token + 1) sizes the
        //    list offsets: assumed (above), or read with the checks.
        uint32_t* f = ctx->h_flags;
        auto verdict = [&]() -> hyset_status {
            if (f[0] & 8) return fail(ctx, HYSET_E_INVALID, "a set reaches past the end of the token array");
            if (f[0] & 1) return fail(ctx, HYSET_E_INVALID, "empty set in collection");
            if (f[0] & 2) return fail(ctx, HYSET_E_INVALID, "set tokens must be strictly ascending");
            if (f[1] == 0xFFFFFFFFu) return fail(ctx, HYSET_E_INVALID, "token 0xFFFFFFFF is reserved");
            return HYSET_OK;
        };
        if (!assumed) {
            CK(cudaMemcpyAsync(f, ctx->s_flags.p, 8, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            const hyset_status vs = verdict();
            if (vs != HYSET_OK) return bail(vs);
            U = f[1] + 1;
        }
        JoinParams P{};
        for (int attempt = 0; attempt < 2; ++attempt) {
            C->universe = U;
            CK(ctx->sc->counts.ensure(((size_t)U + 1) * 4, s));
            CK(ix.list_off.ensure(((size_t)U + 1) * 4, s));
            CK(ctx->sc->scan.ensure(std::max(scan_words, scan_scratch_words((uint64_t)U + 1)) * 4, s));
            if (attempt > 0)  // the list build reordered the entries: emit them again
                CK(emit_packed_entries(v, off, len, pb, ctx->sc->tok.as<uint32_t>(), ix.set.as<uint32_t>(), nullptr, s));
            counts = ctx->sc->counts.as<uint32_t>();
            if (!(assumed && attempt == 0)) {  // not counted while the chunks landed
                CK(cudaMemsetAsync(counts, 0, ((size_t)U + 1) * 4, s));
                CK(token_histogram(ctx->sc->tok.as<uint32_t>(), E, counts, U + 1, s));
            }
            CK(index_lists(ctx->sc->tok.as<uint32_t>(), ix.set.as<uint32_t>(), E, U, counts,
                           ix.list_off.as<uint32_t>(), ctx->sc->altk.as<uint32_t>(), ctx->sc->altv.as<uint32_t>(),
                           ctx->sc->gate.as<uint32_t>(), key_bits_for(U), ctx->sc->scan.as<uint32_t>(), s));
            ix.sim = b->sim;
            ix.tau = b->tau;
            ix.kind = 0;
            ix.universe = U;
            ix.entries = E;
            ix.pos_bits = pb;
            P = JoinParams{};
            P.R = C->view();
            P.S = P.R;
            P.B = b->view;
            P.first_ge = C->first_ge.as<uint32_t>();
            P.R_L = C->max_size;
            P.self = 1;
            P.grab = std::min<uint32_t>(tn.batch, 32);
            P.p_lo = 0;
            P.p_hi = n;
            P.r_lo = 0;
            P.r_hi = n;
            P.X = ix.view();
            if (words) {
                P.bits_R = P.bits_S = bits.as<uint64_t>();
                P.words = words;
            }
            if (assumed) CK(cudaMemcpyAsync(f, ctx->s_flags.p, 8, cudaMemcpyDeviceToHost, s));
            const hyset_status js = run_join(ctx, P, TECH_FGSS, tn.vmode, o, res.get(), true);  // synchronises
            if (js != HYSET_OK) return bail(js);
            if (!assumed) break;
            const hyset_status vs = verdict();
            if (vs != HYSET_OK) return bail(vs);
            if (f[1] + 1 <= U) break;  // every token was indexed: the join stands
            U = f[1] + 1;              // a larger token: index and join again
            assumed = false;
        }
        C->universe = f[1] + 1;
        ctx->universe_cache[ukey] = C->universe;
        res->technique = HYSET_TECH_FGSS;
        res->bitmap_bits = tn.bits;
        res->verify_mode = (uint32_t)tn.vmode;
        res->selector = selector;
        if (o->collect_stats) res->stats[3] = E;
        res->launches = launches() - launches0;
    }
    if (coll_out) *coll_out = c.release();
    else hyset_collection_free(ctx, c.release());
    *out = res.release();
    return HYSET_OK;
}

hyset_status hyset_batch_join(hyset_ctx* ctx, const hyset_join_desc* joins, uint32_t n_joins,
                              hyset_result** results) {
    if (!ctx || (n_joins && (!joins || !results))) return fail(ctx, HYSET_E_INVALID, "null argument");
    for (uint32_t i = 0; i < n_joins; ++i) results[i] = nullptr;
    if (n_joins == 0) return HYSET_OK;
    CK(cudaSetDevice(ctx->device));
    ST(batch_prepare(ctx, joins, n_joins));
    BatchPlan& bp = *ctx->batch;
    cudaStream_t s = ctx->stream;
    CK(cudaEventRecord(ctx->ev0, s));
    CK(cudaGraphLaunch(bp.exec, s));
    CK(cudaEventRecord(ctx->ev1, s));
    std::vector<unsigned long long> counts(n_joins);
    CK(cudaMemcpyAsync(counts.data(), bp.counts.p, n_joins * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    std::vector<std::unique_ptr<hyset_result>> out(n_joins);
    hyset_status st = HYSET_OK;
    for (uint32_t j = 0; j < n_joins && st == HYSET_OK; ++j) {
        BatchJoin& bj = *bp.joins[j];
        out[j] = std::make_unique<hyset_result>();
        hyset_result* r = out[j].get();
        r->technique = bj.tech;
        r->bitmap_bits = (uint32_t)bj.words * 64u;
        r->device_ms = ms;  // the whole batch: one launch sequence
        r->count = counts[j];
        if (!bj.o.count_only && counts[j] > bj.cap) {
            // the join's buffer overflowed: run it alone with room for every pair
            hyset_join_opts o2 = bj.o;
            o2.pair_capacity = counts[j] + 1024;
            st = do_join(ctx, bj.swapped ? bj.S : bj.R, bj.swapped ? bj.R : bj.S, &o2, r);
            continue;
        }
        if (bj.o.count_only) continue;
        if (bj.o.sort_pairs) {
            st = sort_device_pairs(ctx, bj.pairs.as<uint2>(), counts[j], bj.swapped ? bj.R->n : bj.S->n,
                                   bj.swapped ? bj.S->n : bj.R->n);
            if (st != HYSET_OK) break;
        }
        if (bj.o.device_pairs) {
            r->device_pairs = bj.pairs.p;
            continue;
        }
        r->pairs.resize(counts[j]);
        r->has_pairs = 1;
        if (counts[j]) {
            cudaError_t e = cudaMemcpyAsync(r->pairs.data(), bj.pairs.p, counts[j] * sizeof(hyset_pair),
                                            cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) st = fail(ctx, HYSET_E_CUDA, "batch pair copy", e);
        }
    }
    if (st == HYSET_OK) CK(cudaStreamSynchronize(s));
    if (st != HYSET_OK) return st;
    for (uint32_t j = 0; j < n_joins; ++j) results[j] = out[j].release();
    return HYSET_OK;
}

hyset_status hyset_join_features(hyset_ctx* ctx, const hyset_coll* indexed, const hyset_coll* probe,
                                 const hyset_join_opts* opts, float* features, double* base_stats) {
    if (!ctx || !indexed || !opts || !features) return fail(ctx, HYSET_E_INVALID, "null argument");
    CK(cudaSetDevice(ctx->device));
    hyset_coll* R = const_cast<hyset_coll*>(indexed);
    hyset_coll* S = const_cast<hyset_coll*>(probe ? probe : indexed);
    return compute_features(ctx, R, S, opts, features, base_stats);
}

namespace {
struct MlpBufs {
    DevBuf w, x, t, m, y, g, mom, vel, loss;
};
hyset_status mlp_upload(hyset_ctx* ctx, MlpBufs& B, const float* params, const float* x, const float* t,
                        const float* mask, uint32_t n) {
    cudaStream_t s = ctx->stream;
    CK(B.w.ensure(MLP_PARAMS * 4, s));
    CK(B.x.ensure((size_t)n * MLP_IN * 4 + 4, s));
    CK(B.y.ensure((size_t)n * MLP_OUT * 4 + 4, s));
    CK(cudaMemcpyAsync(B.w.p, params, MLP_PARAMS * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(B.x.p, x, (size_t)n * MLP_IN * 4, cudaMemcpyHostToDevice, s));
    if (t) {
        CK(B.t.ensure((size_t)n * MLP_OUT * 4 + 4, s));
        CK(B.m.ensure((size_t)n * MLP_OUT * 4 + 4, s));
        CK(cudaMemcpyAsync(B.t.p, t, (size_t)n * MLP_OUT * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(B.m.p, mask, (size_t)n * MLP_OUT * 4, cudaMemcpyHostToDevice, s));
    }
    return HYSET_OK;
}
void mlp_release(hyset_ctx* ctx, MlpBufs& B) {
    DevBuf* bufs[] = {&B.w, &B.x, &B.t, &B.m, &B.y, &B.g, &B.mom, &B.vel, &B.loss};
    for (DevBuf* d : bufs) d->release(ctx->stream);
    cudaStreamSynchronize(ctx->stream);
}
float mask_sum(const float* mask, uint32_t n) {
    double d = 0;
    for (size_t i = 0; i < (size_t)n * MLP_OUT; ++i) d += mask[i];
    return (float)d;
}
}  // namespace

hyset_status hyset_mlp_forward(hyset_ctx* ctx, const float* params, const float* x, uint32_t n, float* y) {
    if (!ctx || !params || (n && (!x || !y))) return fail(ctx, HYSET_E_INVALID, "null argument");
    if (n == 0) return HYSET_OK;
    CK(cudaSetDevice(ctx->device));
    MlpBufs B;
    hyset_status st = mlp_upload(ctx, B, params, x, nullptr, nullptr, n);
    if (st == HYSET_OK) {
        cudaError_t e = mlp_forward(B.w.as<float>(), B.x.as<float>(), (int)n, B.y.as<float>(), ctx->sm_count,
                                    ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(y, B.y.p, (size_t)n * MLP_OUT * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = fail(ctx, HYSET_E_CUDA, "mlp forward", e);
    }
    mlp_release(ctx, B);
    return st;
}

hyset_status hyset_mlp_grad(hyset_ctx* ctx, const float* params, const float* x, const float* t, const float* mask,
                            uint32_t n, float* grad, float* loss) {
    if (!ctx || !params || !x || !t || !mask || !grad || !loss || n == 0)
        return fail(ctx, HYSET_E_INVALID, "null argument");
    const float denom = mask_sum(mask, n);
    if (!(denom > 0.f)) return fail(ctx, HYSET_E_INVALID, "mask selects no output");
    CK(cudaSetDevice(ctx->device));
    MlpBufs B;
    hyset_status st = mlp_upload(ctx, B, params, x, t, mask, n);
    cudaError_t e = cudaSuccess;
    if (st == HYSET_OK) {
        e = B.g.ensure(MLP_PARAMS * 4, ctx->stream);
        if (e == cudaSuccess) e = B.loss.ensure(16, ctx->stream);
        if (e == cudaSuccess)
            e = mlp_grad(B.w.as<float>(), B.x.as<float>(), B.t.as<float>(), B.m.as<float>(), (int)n, denom,
                         B.g.as<float>(), B.loss.as<float>(), ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(grad, B.g.p, MLP_PARAMS * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(loss, B.loss.p, 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = fail(ctx, HYSET_E_CUDA, "mlp gradient", e);
    }
    mlp_release(ctx, B);
    return st;
}

hyset_status hyset_mlp_train(hyset_ctx* ctx, float* params, const float* x, const float* t, const float* mask,
                             uint32_t n, uint32_t steps, float lr, float weight_decay, float* loss_trace) {
    if (!ctx || !params || !x || !t || !mask || n == 0) return fail(ctx, HYSET_E_INVALID, "null argument");
    const float denom = mask_sum(mask, n);
    if (!(denom > 0.f)) return fail(ctx, HYSET_E_INVALID, "mask selects no output");
    CK(cudaSetDevice(ctx->device));
    MlpBufs B;
    hyset_status st = mlp_upload(ctx, B, params, x, t, mask, n);
    cudaError_t e = cudaSuccess;
    cudaStream_t s = ctx->stream;
    if (st == HYSET_OK) {
        e = B.g.ensure(MLP_PARAMS * 4, s);
        if (e == cudaSuccess) e = B.mom.ensure(MLP_PARAMS * 4, s);
        if (e == cudaSuccess) e = B.vel.ensure(MLP_PARAMS * 4, s);
        if (e == cudaSuccess) e = B.loss.ensure((size_t)steps * 4 + 4, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(B.mom.p, 0, MLP_PARAMS * 4, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(B.vel.p, 0, MLP_PARAMS * 4, s);
        if (e == cudaSuccess)
            e = mlp_train(B.w.as<float>(), B.mom.as<float>(), B.vel.as<float>(), B.g.as<float>(), B.x.as<float>(),
                          B.t.as<float>(), B.m.as<float>(), (int)n, denom, (int)steps, lr, weight_decay,
                          B.loss.as<float>(), s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(params, B.w.p, MLP_PARAMS * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && loss_trace && steps)
            e = cudaMemcpyAsync(loss_trace, B.loss.p, (size_t)steps * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = fail(ctx, HYSET_E_CUDA, "mlp training", e);
    }
    mlp_release(ctx, B);
    return st;
}

hyset_status hyset_selector_set(hyset_ctx* ctx, const float* params, const float* feature_mean,
                                const float* feature_scale, const double* cost_coefficients) {
    if (!ctx) return HYSET_E_INVALID;
    CK(cudaSetDevice(ctx->device));
    ctx->select_cache.clear();
    ctx->split_cache.clear();
    ctx->has_mlp = false;
    if (params) {
        if (!feature_mean || !feature_scale) return fail(ctx, HYSET_E_INVALID, "normalisation missing");
        for (int k = 0; k < MLP_IN; ++k)
            if (!(feature_scale[k] > 0.f)) return fail(ctx, HYSET_E_INVALID, "feature scale must be > 0");
        ctx->mlp_params.assign(params, params + MLP_PARAMS);
        std::memcpy(ctx->feat_mean, feature_mean, sizeof ctx->feat_mean);
        std::memcpy(ctx->feat_scale, feature_scale, sizeof ctx->feat_scale);
        CK(ctx->d_mlp.ensure(MLP_PARAMS * 4, ctx->stream));
        CK(cudaMemcpyAsync(ctx->d_mlp.p, ctx->mlp_params.data(), MLP_PARAMS * 4, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        ctx->has_mlp = true;
    }
    ctx->has_cost = cost_coefficients != nullptr;
    if (cost_coefficients) std::memcpy(ctx->cost, cost_coefficients, sizeof ctx->cost);
    return HYSET_OK;
}

int hyset_result_selector(const hyset_result* r) { return r ? r->selector : -1; }

uint64_t hyset_result_count(const hyset_result* r) { return r ? r->count : 0; }
const hyset_pair* hyset_result_pairs(const hyset_result* r) {
    static const hyset_pair none = {0, 0};
    if (!r || !r->has_pairs) return nullptr;
    return r->pairs.empty() ? &none : r->pairs.data();
}
uint64_t hyset_result_launches(const hyset_result* r) { return r ? r->launches : 0; }
hyset_technique hyset_result_technique(const hyset_result* r) { return r ? r->technique : HYSET_TECH_AUTO; }
uint32_t hyset_result_bitmap_bits(const hyset_result* r) { return r ? r->bitmap_bits : 0; }
uint32_t hyset_result_verify_mode(const hyset_result* r) { return r ? r->verify_mode : 0; }
uint32_t hyset_result_split(const hyset_result* r, hyset_technique* low_technique) {
    if (low_technique) *low_technique = r ? r->split_low : HYSET_TECH_AUTO;
    return r ? r->split_at : 0;
}
double hyset_result_device_ms(const hyset_result* r) { return r ? r->device_ms : 0.0; }
double hyset_result_kernel_ms(const hyset_result* r) { return r ? r->kernel_ms : 0.0; }
const void* hyset_result_device_pairs(const hyset_result* r) { return r ? r->device_pairs : nullptr; }
uint32_t hyset_result_stats(const hyset_result* r, uint64_t* out, uint32_t n) {
    if (!r || !out) return 0;
    uint32_t k = n < 8 ? n : 8;
    for (uint32_t i = 0; i < k; ++i) out[i] = r->stats[i];
    return k;
}
void hyset_result_free(hyset_result* r) { delete r; }

// ---------------------------------------------------------------- handlers

hyset_status hyset_handler_create(hyset_ctx* ctx, const hyset_coll* coll, hyset_technique technique, hyset_sim sim,
                                  uint32_t bitmap_size, uint32_t block_size, int aggregate, double threshold,
                                  hyset_handler** out) {
    if (!ctx || !coll || !out) return fail(ctx, HYSET_E_INVALID, "null argument");
    *out = nullptr;
    if (technique != HYSET_TECH_BITMAP && technique != HYSET_TECH_FGSS)
        return fail(ctx, HYSET_E_INVALID, "handler technique must be BITMAP or FGSS");
    if (block_size == 0) return fail(ctx, HYSET_E_INVALID, "block size must be > 0");
    hyset_join_opts o;
    hyset_default_opts(&o);
    o.sim = sim;
    o.threshold = threshold;
    ST(check_opts(ctx, &o));
    if (technique == HYSET_TECH_BITMAP && bitmap_size != 64 && bitmap_size != 128 && bitmap_size != 256 &&
        bitmap_size != 512)
        return fail(ctx, HYSET_E_INVALID, "bitmap size must be 64, 128, 256 or 512");
    CK(cudaSetDevice(ctx->device));
    auto h = std::make_unique<hyset_handler>();
    h->ctx = ctx;
    h->coll = coll;
    h->technique = technique;
    h->sim = sim;
    h->tau = threshold;
    h->block_size = block_size;
    h->aggregate = aggregate ? 1 : 0;
    ST(get_bounds(ctx, sim, threshold, coll->max_size, 0, &h->bounds));
    cudaStream_t s = ctx->stream;
    if (technique == HYSET_TECH_BITMAP) {
        // bitmap::handler ctor generates every signature up front (device_algorithms.hpp:144-156)
        h->words = (int)(bitmap_size / 64);
        CK(h->bits.ensure((size_t)coll->n * h->words * 8 + 8, s));
        CK(generate_bitmaps(coll->view(), h->words, h->bits.as<uint64_t>(), s));
    }
    CK(h->count.ensure(16, s));
    CK(h->work.ensure(16, s));
    h->cap = aggregate ? 0 : std::max<uint64_t>(1u << 16, (uint64_t)block_size * 4);
    if (!aggregate) CK(h->pairs.ensure(h->cap * sizeof(uint2), s));
    CK(cudaStreamSynchronize(s));
    *out = h.release();
    return HYSET_OK;
}

namespace {

// Per-indexed-block inverted index in the reference's layout
// (include/hyset/index.hpp:284-313): zero universe-sized counts, histogram of
// the block's prefix entries, exclusive scan, atomic scatter (lists unsorted).
hyset_status build_block_index(hyset_handler* h, const hyset_block& blk) {
    hyset_ctx* ctx = h->ctx;
    cudaStream_t s = ctx->stream;
    const hyset_coll* c = h->coll;
    const uint32_t lo = blk.start_id, hi = blk.end_id + 1, nb = hi - lo, U = c->universe;
    uint64_t E = 0;  // the block's prefix entries (block.entries in the reference)
    const std::vector<uint64_t> bh = range_hist(c, lo, hi);
    for (size_t l = 0; l < bh.size(); ++l) E += bh[l] * h->bounds->index_prefix[l];
    const uint64_t E1 = E ? E : 1;
    CK(h->counts.ensure(((size_t)U + 1) * 4, s));
    CK(h->list_off.ensure(((size_t)U + 1) * 4, s));
    CK(h->e_len.ensure((size_t)nb * 4 + 4, s));
    CK(h->e_off.ensure((size_t)nb * 4 + 4, s));
    CK(h->e_tok.ensure(E1 * 4, s));
    CK(h->e_set.ensure(E1 * 4, s));
    CK(h->e_pos.ensure(E1 * 4, s));
    CK(h->idx_set.ensure(E1 * 4, s));
    CK(h->idx_pos.ensure(E1 * 4, s));
    CK(h->scan.ensure(std::max(scan_scratch_words(nb), scan_scratch_words((uint64_t)U + 1)) * 4, s));
    CollView v = c->view();
    uint32_t* scr = h->scan.as<uint32_t>();
    CK(set_prefix_lengths(v, h->bounds->view.index_prefix, lo, hi, h->e_len.as<uint32_t>(), s));
    CK(scan_exclusive(h->e_len.as<uint32_t>(), h->e_off.as<uint32_t>(), nb, scr, s));
    CK(emit_prefix_entries(v, lo, hi, h->e_off.as<uint32_t>(), h->e_len.as<uint32_t>(), h->e_tok.as<uint32_t>(),
                           h->e_set.as<uint32_t>(), h->e_pos.as<uint32_t>(), s));
    CK(cudaMemsetAsync(h->counts.p, 0, ((size_t)U + 1) * 4, s));
    CK(token_histogram(h->e_tok.as<uint32_t>(), E, h->counts.as<uint32_t>(), U + 1, s));
    CK(scan_exclusive(h->counts.as<uint32_t>(), h->list_off.as<uint32_t>(), (uint64_t)U + 1, scr, s));
    // the scatter advances a cursor copy of the list starts
    CK(cudaMemcpyAsync(h->counts.p, h->list_off.p, ((size_t)U + 1) * 4, cudaMemcpyDeviceToDevice, s));
    CK(scatter_entries(h->e_tok.as<uint32_t>(), h->e_set.as<uint32_t>(), h->e_pos.as<uint32_t>(), E,
                       h->counts.as<uint32_t>(), h->idx_set.as<uint32_t>(), h->idx_pos.as<uint32_t>(), s));
    h->indexed_block = blk.id;
    return HYSET_OK;
}

hyset_status check_block(hyset_ctx* ctx, const hyset_coll* c, const hyset_block* b) {
    if (!b || b->start_id > b->end_id || b->end_id >= c->n) return fail(ctx, HYSET_E_INVALID, "bad block range");
    return HYSET_OK;
}

}  // namespace

hyset_status hyset_handler_join_blocks(hyset_handler* h, const hyset_block* first, const hyset_block* second) {
    if (!h) return HYSET_E_INVALID;
    hyset_ctx* ctx = h->ctx;
    ST(check_block(ctx, h->coll, first));
    ST(check_block(ctx, h->coll, second));
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    if (h->technique == HYSET_TECH_FGSS && h->indexed_block != first->id) ST(build_block_index(h, *first));
    JoinParams P{};
    P.R = h->coll->view();
    P.S = P.R;
    P.B = h->bounds->view;
    P.first_ge = h->coll->first_ge.as<uint32_t>();
    P.R_L = h->coll->max_size;
    P.self = 1;
    P.grab = h->technique == HYSET_TECH_FGSS ? 4 : 1;
    P.p_lo = second->start_id;
    P.p_hi = second->end_id + 1;
    P.r_lo = first->start_id;
    P.r_hi = first->end_id + 1;
    if (h->technique == HYSET_TECH_FGSS) {
        P.X.list_off = h->list_off.as<uint32_t>();
        P.X.set = h->idx_set.as<uint32_t>();
        P.X.pos = h->idx_pos.as<uint32_t>();
        P.X.universe = h->coll->universe;
        P.X.sorted = 0;
    } else {
        P.bits_R = P.bits_S = h->bits.as<uint64_t>();
        P.words = h->words;
    }
    const int tech = h->technique == HYSET_TECH_FGSS ? TECH_FGSS : TECH_BITMAP;
    const int vmode = 1;
    for (int attempt = 0; attempt < 2; ++attempt) {
        P.out.pairs = h->aggregate ? nullptr : h->pairs.as<uint2>();
        P.out.count = h->count.as<unsigned long long>();
        P.out.cap = h->cap;
        P.out.count_only = h->aggregate;
        P.work = h->work.as<unsigned int>();
        CK(cudaMemsetAsync(h->count.p, 0, 16, s));
        CK(cudaMemsetAsync(h->work.p, 0, 16, s));
        CK(launch_join(P, tech, vmode, ctx->sm_count, s));
        unsigned long long count = 0;
        CK(cudaMemcpyAsync(&count, h->count.p, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (h->aggregate) {
            h->out_count += count;
            return HYSET_OK;
        }
        if (count <= h->cap) {
            size_t old = h->out_pairs.size();
            h->out_pairs.resize(old + count);
            if (count)
                CK(cudaMemcpyAsync(h->out_pairs.data() + old, h->pairs.p, count * sizeof(hyset_pair),
                                   cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            h->out_count += count;
            return HYSET_OK;
        }
        h->cap = count + count / 4 + 1024;
        CK(h->pairs.ensure(h->cap * sizeof(uint2), s));
    }
    return fail(ctx, HYSET_E_OVERFLOW, "handler pair buffer overflow after resize");
}

hyset_status hyset_handler_join_partitions(hyset_handler* h, const hyset_block* first, uint32_t n_first,
                                           const hyset_block* second, uint32_t n_second) {
    if (!h || (n_first && !first) || (n_second && !second)) return HYSET_E_INVALID;
    // device::length_filter (device_algorithms.hpp:21-53): probe block id >= indexed
    // block id and size[last indexed] >= minsize(size[first probe]).
    for (uint32_t i = 0; i < n_first; ++i) {
        ST(check_block(h->ctx, h->coll, &first[i]));
        for (uint32_t k = 0; k < n_second; ++k) {
            ST(check_block(h->ctx, h->coll, &second[k]));
            if (second[k].id < first[i].id) continue;
            uint32_t last_indexed = size_at(h->coll, first[i].end_id);
            uint32_t first_probe = size_at(h->coll, second[k].start_id);
            if (last_indexed >= h->bounds->minsize[first_probe]) ST(hyset_handler_join_blocks(h, &first[i], &second[k]));
        }
    }
    return HYSET_OK;
}

hyset_status hyset_handler_output(const hyset_handler* h, uint64_t* count, const hyset_pair** pairs) {
    if (!h) return HYSET_E_INVALID;
    if (count) *count = h->out_count;
    if (pairs) *pairs = h->aggregate ? nullptr : h->out_pairs.data();
    return HYSET_OK;
}

hyset_status hyset_handler_clear_output(hyset_handler* h) {
    if (!h) return HYSET_E_INVALID;
    h->out_count = 0;
    h->out_pairs.clear();
    return HYSET_OK;
}

void hyset_handler_destroy(hyset_handler* h) {
    if (!h) return;
    cudaStream_t s = h->ctx->stream;
    DevBuf* bufs[] = {&h->counts, &h->list_off, &h->e_len, &h->e_off, &h->e_tok, &h->e_set, &h->e_pos,
                      &h->idx_set, &h->idx_pos, &h->scan, &h->bits, &h->pairs, &h->count, &h->work};
    for (DevBuf* b : bufs) b->release(s);
    cudaStreamSynchronize(s);
    delete h;
}

// ---------------------------------------------------------------- verifier

hyset_status hyset_verifier_create(hyset_ctx* ctx, const hyset_coll* indexed, const hyset_coll* probe, hyset_sim sim,
                                   uint32_t threads, uint32_t scenario, int aggregate, uint32_t max_probes,
                                   uint32_t max_candidates, double threshold, hyset_verifier** out) {
    (void)threads;  // the reference's CTA width; here one warp verifies a probe's candidates
    if (!ctx || !indexed || !probe || !out) return fail(ctx, HYSET_E_INVALID, "null argument");
    *out = nullptr;
    if (scenario != 1 && scenario != 2) return fail(ctx, HYSET_E_INVALID, "scenario must be 1 or 2");
    if (max_probes == 0 || max_candidates == 0) return fail(ctx, HYSET_E_INVALID, "capacities must be > 0");
    hyset_join_opts o;
    hyset_default_opts(&o);
    o.sim = sim;
    o.threshold = threshold;
    ST(check_opts(ctx, &o));
    CK(cudaSetDevice(ctx->device));
    auto v = std::make_unique<hyset_verifier>();
    v->ctx = ctx;
    v->indexed = indexed;
    v->probe = probe;
    v->scenario = scenario;
    v->aggregate = aggregate ? 1 : 0;
    v->max_probes = max_probes;
    v->max_candidates = max_candidates;
    ST(get_bounds(ctx, sim, threshold, std::max(indexed->max_size, probe->max_size), 0, &v->bounds));
    cudaStream_t s = ctx->stream;
    CK(v->d_probes.ensure((size_t)max_probes * 4 + 8, s));
    CK(v->d_offsets.ensure((size_t)max_probes * 4 + 8, s));
    CK(v->d_cands.ensure((size_t)max_candidates * 4 + 4, s));
    CK(v->pairs.ensure((size_t)max_candidates * sizeof(uint2), s));
    CK(v->count.ensure(16, s));
    CK(v->work.ensure(16, s));
    CK(cudaStreamSynchronize(s));
    *out = v.release();
    return HYSET_OK;
}

namespace {
hyset_status verifier_run(hyset_verifier* v) {
    hyset_ctx* ctx = v->ctx;
    cudaStream_t s = ctx->stream;
    const uint32_t np = (uint32_t)v->h_probes.size();
    if (np == 0) return HYSET_OK;
    CK(cudaMemcpyAsync(v->d_probes.p, v->h_probes.data(), (size_t)np * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(v->d_offsets.p, v->h_offsets.data(), (size_t)np * 4, cudaMemcpyHostToDevice, s));
    if (!v->h_cands.empty())
        CK(cudaMemcpyAsync(v->d_cands.p, v->h_cands.data(), v->h_cands.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(v->count.p, 0, 16, s));
    CK(cudaMemsetAsync(v->work.p, 0, 16, s));
    Sink out{v->aggregate ? nullptr : v->pairs.as<uint2>(), v->count.as<unsigned long long>(),
             (unsigned long long)v->max_candidates, v->aggregate};
    CK(launch_verify_candidates(v->indexed->view(), v->probe->view(), v->bounds->view, v->d_probes.as<uint32_t>(),
                                v->d_offsets.as<uint32_t>(), v->d_cands.as<uint32_t>(), np,
                                v->scenario == 1 ? 3 : 2,  // scenario 1 (lane per candidate) runs staged
                                out,
                                v->work.as<unsigned int>(), ctx->sm_count, s));
    unsigned long long count = 0;
    CK(cudaMemcpyAsync(&count, v->count.p, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (!v->aggregate && count) {
        size_t old = v->out_pairs.size();
        v->out_pairs.resize(old + count);
        CK(cudaMemcpyAsync(v->out_pairs.data() + old, v->pairs.p, count * sizeof(hyset_pair), cudaMemcpyDeviceToHost,
                           s));
        CK(cudaStreamSynchronize(s));
    }
    v->out_count += count;
    v->h_probes.clear();
    v->h_offsets.clear();
    v->h_cands.clear();
    return HYSET_OK;
}
}  // namespace

hyset_status hyset_verifier_add_candidates(hyset_verifier* v, uint32_t probe_id, const uint32_t* candidates,
                                           uint32_t n) {
    if (!v || (n && !candidates)) return HYSET_E_INVALID;
    hyset_ctx* ctx = v->ctx;
    if (probe_id >= v->probe->n) return fail(ctx, HYSET_E_INVALID, "probe id out of range");
    for (uint32_t k = 0; k < n; ++k)
        if (candidates[k] >= v->indexed->n) return fail(ctx, HYSET_E_INVALID, "candidate id out of range");
    // addCandidates (hybrid_algorithms.hpp:71-105): a candidate set that does not
    // fit is split; the full batch is verified before the rest is queued.
    uint32_t done = 0;
    do {
        if (v->h_probes.size() >= v->max_probes || v->h_cands.size() >= v->max_candidates) ST(verifier_run(v));
        uint32_t room = v->max_candidates - (uint32_t)v->h_cands.size();
        uint32_t take = std::min(room, n - done);
        v->h_probes.push_back(probe_id);
        v->h_cands.insert(v->h_cands.end(), candidates + done, candidates + done + take);
        v->h_offsets.push_back((uint32_t)v->h_cands.size());
        done += take;
    } while (done < n);
    return HYSET_OK;
}

hyset_status hyset_verify_device(hyset_ctx* ctx, const hyset_coll* indexed, const hyset_coll* probe,
                                 const uint32_t* d_probes, const uint32_t* d_offsets, const uint32_t* d_candidates,
                                 uint32_t n_probes, const hyset_join_opts* opts, hyset_result** out) {
    if (!ctx || !indexed || !opts || !out || (n_probes && (!d_probes || !d_offsets || !d_candidates)))
        return fail(ctx, HYSET_E_INVALID, "null argument");
    *out = nullptr;
    ST(check_opts(ctx, opts));
    CK(cudaSetDevice(ctx->device));
    const hyset_coll* R = indexed;
    const hyset_coll* S = probe ? probe : indexed;
    Bounds* b = nullptr;
    ST(get_bounds(ctx, opts->sim, opts->threshold, std::max(R->max_size, S->max_size), 0, &b));
    auto res = std::make_unique<hyset_result>();
    cudaStream_t s = ctx->stream;
    const int vmode = opts->verify_mode ? (int)opts->verify_mode : 3;
    const int count_only = opts->count_only ? 1 : 0;
    uint64_t cap = opts->pair_capacity ? opts->pair_capacity : (1u << 20);
    CK(ctx->s_count.ensure(16, s));
    CK(ctx->s_work.ensure(16, s));
    for (int attempt = 0; attempt < 2; ++attempt) {
        if (!count_only) CK(ctx->s_pairs.ensure(std::max<uint64_t>(cap, 1) * sizeof(uint2), s));
        Sink sk{count_only ? nullptr : ctx->s_pairs.as<uint2>(), ctx->s_count.as<unsigned long long>(),
                count_only ? 0ull : (unsigned long long)cap, count_only};
        CK(cudaMemsetAsync(ctx->s_count.p, 0, 16, s));
        CK(cudaMemsetAsync(ctx->s_work.p, 0, 16, s));
        CK(cudaEventRecord(ctx->ek0, s));
        CK(launch_verify_candidates(R->view(), S->view(), b->view, d_probes, d_offsets, d_candidates, n_probes, vmode,
                                    sk, ctx->s_work.as<unsigned int>(), ctx->sm_count, s));
        CK(cudaEventRecord(ctx->ek1, s));
        unsigned long long count = 0;
        CK(cudaMemcpyAsync(&count, ctx->s_count.p, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        float kms = 0;
        CK(cudaEventElapsedTime(&kms, ctx->ek0, ctx->ek1));
        res->kernel_ms = res->device_ms = kms;
        res->verify_mode = (uint32_t)vmode;
        res->count = count;
        if (count_only || count <= cap) break;
        cap = count + count / 8 + 1024;
        if (attempt == 1) return fail(ctx, HYSET_E_OVERFLOW, "pair buffer overflow after resize");
    }
    if (!count_only && opts->device_pairs) {
        res->device_pairs = ctx->s_pairs.p;
    } else if (!count_only) {
        res->pairs.resize(res->count);
        if (res->count)
            CK(cudaMemcpyAsync(res->pairs.data(), ctx->s_pairs.p, res->count * sizeof(hyset_pair),
                               cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        res->has_pairs = 1;
    }
    res->technique = HYSET_TECH_DIRECT;
    *out = res.release();
    return HYSET_OK;
}

hyset_status hyset_verifier_flush(hyset_verifier* v) {
    if (!v) return HYSET_E_INVALID;
    return verifier_run(v);
}

hyset_status hyset_verifier_output(const hyset_verifier* v, uint64_t* count, const hyset_pair** pairs) {
    if (!v) return HYSET_E_INVALID;
    if (count) *count = v->out_count;
    if (pairs) *pairs = v->aggregate ? nullptr : v->out_pairs.data();
    return HYSET_OK;
}

void hyset_verifier_destroy(hyset_verifier* v) {
    if (!v) return;
    cudaStream_t s = v->ctx->stream;
    DevBuf* bufs[] = {&v->d_probes, &v->d_offsets, &v->d_cands, &v->pairs, &v->count, &v->work};
    for (DevBuf* b : bufs) b->release(s);
    cudaStreamSynchronize(s);
    delete v;
}

}  // extern "C"
