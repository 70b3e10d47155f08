// index_host.cu — host orchestration of the index builds: size statistics of
// a collection, the global set-id-sorted prefix index (and the R-S midprefix
// index), token groups, and the XOR signatures.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "host.h"

namespace hs {

// Host size statistics from host-resident sizes (the caller's array, or the
// pinned copy of device sizes): the per-size histogram and first_ge[l] = first
// set id with size >= l (sizes are non-decreasing), whose device copy is
// enqueued on the stream (the host array is a member, so no synchronisation is
// needed here).  The collection keeps no per-set host array: sizes of single
// sets and of id ranges come from first_ge.
hyset_status build_size_meta(hyset_ctx* ctx, hyset_coll* c, const uint32_t* sizes) {
    std::vector<uint64_t>& hist = c->size_hist;
    hist.assign(c->n ? (size_t)sizes[c->n - 1] + 1 : 1, 0);
    uint32_t i = 0;
    // run lengths: sorted sizes repeat, so the count stays in a register
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

void size_meta_from_first_ge(hyset_coll* c, const uint32_t* first_ge, uint32_t L) {
    c->max_size = L;
    c->h_first_ge.assign(first_ge, first_ge + (size_t)L + 2);
    c->size_hist.assign((size_t)L + 1, 0);
    for (uint32_t l = 0; l <= L; ++l) c->size_hist[l] = first_ge[l + 1] - first_ge[l];
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

BoundFields bound_fields(const Bounds* b) {
    return BoundFields{b->view.max_sum, b->view.lp_row, b->view.lp_tab};
}

uint32_t first_long_prefix(const hyset_coll* c, const std::vector<uint32_t>& pre) {
    constexpr uint32_t LONG_PREFIX = 32;  // longer prefixes are emitted a warp per set
    uint64_t id = 0;
    for (size_t l = 0; l < c->size_hist.size(); ++l) {
        if (l < pre.size() && pre[l] > LONG_PREFIX) return (uint32_t)id;
        id += c->size_hist[l];
    }
    return 0xFFFFFFFFu;
}

void record_layout(const hyset_coll* c, const Bounds* b, int kind, uint32_t pb, uint32_t* rec_bits, bool* bound) {
    const uint32_t fb = bits_for(b->L);  // a field that holds every probe length
    *bound = kind == 0 && (b->view.max_sum != nullptr || b->view.lp_tab != nullptr) && fb + bits_for(c->n) <= 32;
    *rec_bits = *bound ? fb : pb;
}

// Bits needed to represent v (at least 1).
uint32_t bits_for(uint64_t v) {
    uint32_t b = 1;
    while (b < 64 && (v >> b)) ++b;
    return b;
}


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
// records_ok: the caller's kernel reads token records (REC_CAP); they are
// built once the longest list of this prefix table is known to fit (it is
// read back on the collection's first build with the table; that build's
// lists are converted), afterwards directly from the prefix entries: one emit
// pass and one ordering pass, no offsets, no scan.
hyset_status build_sorted_index(hyset_ctx* ctx, hyset_coll* c, const Bounds* b, int kind, Index& ix,
                                const std::vector<uint32_t>* pre, const uint32_t* d_pre,
                                int force_pb, bool records_ok) {
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
    // Packed entries (set << pb | position) when set ids up to n and positions
    // below the longest prefix fit 32 bits: the sorted values are the index.
    uint32_t max_pre = 1;
    for (size_t l = 0; l < c->size_hist.size(); ++l)
        if (c->size_hist[l]) max_pre = std::max(max_pre, (*pre)[l]);
    const uint32_t pb = force_pb > 0 ? (uint32_t)force_pb : bits_for(max_pre), sb = bits_for(n);
    const bool packed = force_pb != 0 && pb + sb <= 32;
    // Records are sized from the longest list seen on an earlier build, so only
    // collections whose tokens the library owns (immutable once uploaded) use
    // them; a collection over caller memory can change between joins.
    const bool owned = c->tokens.p != nullptr && c->d_tokens == c->tokens.as<uint32_t>();
    const bool rec_fits = records_ok && packed && owned && (uint64_t)U <= REC_MAX_TOKENS;
    ix.sim = b->sim;
    ix.tau = b->tau;
    ix.kind = kind;
    ix.universe = U;
    ix.entries = E;
    ix.records = false;
    if (rec_fits) {
        const auto lk = c->list_longest.find(d_pre);
        if (lk != c->list_longest.end() && lk->second <= REC_ENTRIES) {
            uint32_t* counts = ctx->sc->counts.as<uint32_t>();
            record_layout(c, b, kind, pb, &ix.rec_bits, &ix.rec_bound);
            CK(ix.rec.ensure((size_t)U * REC_CAP * 4, s));
            CK(cudaMemsetAsync(counts, 0, (size_t)U * 4, s));
            CK(emit_records(v, d_pre, ix.rec_bits, counts, ix.rec.as<uint32_t>(), U, s, 0, 0xFFFFFFFFu,
                            ix.rec_bound ? bound_fields(b) : BoundFields{}, first_long_prefix(c, *pre)));
            CK(order_records(counts, U, ix.rec.as<uint32_t>(), s));
            ix.records = true;
            ix.pos_bits = pb;
            return HYSET_OK;
        }
    }
    CK(set_prefix_lengths(v, d_pre, 0, n, len, s));
    CK(scan_exclusive(len, off, n, scr, s));
    if (packed) {
        uint32_t* counts = ctx->sc->counts.as<uint32_t>();
        CK(ctx->sc->gate.ensure(4, s));
        CK(cudaMemsetAsync(counts, 0, ((size_t)U + 1) * 4, s));
        CK(emit_packed_entries(v, off, len, pb, ctx->sc->tok.as<uint32_t>(), ix.set.as<uint32_t>(), counts, s, 0,
                               0xFFFFFFFFu, 0xFFFFFFFFu, first_long_prefix(c, *pre)));
        // the list build's path is read back once per collection and prefix
        // table (not while a batch is being captured into a graph)
        cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(s, &capturing));
        int& path = c->list_path[d_pre];
        const bool read_back = path == 0 && capturing == cudaStreamCaptureStatusNone;
        CK(index_lists(ctx->sc->tok.as<uint32_t>(), ix.set.as<uint32_t>(), E, U, counts, ix.list_off.as<uint32_t>(),
                       ctx->sc->altk.as<uint32_t>(), ctx->sc->altv.as<uint32_t>(), ctx->sc->gate.as<uint32_t>(),
                       key_bits_for(U), scr, s, &path, read_back ? ctx->h_flags + 15 : nullptr));
        if (read_back && E) c->list_longest[d_pre] = ctx->h_flags[15];
        ix.pos_bits = pb;
        if (rec_fits && E && read_back && ctx->h_flags[15] <= REC_ENTRIES) {
            // this build's lists become records; later builds emit records directly
            record_layout(c, b, kind, pb, &ix.rec_bits, &ix.rec_bound);
            CK(ix.rec.ensure((size_t)U * REC_CAP * 4, s));
            CK(records_from_lists(ix.list_off.as<uint32_t>(), ix.set.as<uint32_t>(), U, ix.rec.as<uint32_t>(), s,
                                  ix.rec_bound ? bound_fields(b) : BoundFields{}, c->d_sizes, pb, ix.rec_bits));
            ix.records = true;
        }
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
    ST(build_sorted_index(ctx, R, b, self ? 0 : 1, ix, nullptr, nullptr, -1, true));
    P.X = ix.view();
    P.X2 = IndexView{};
    if (use_bands(b, self)) {
        ST(build_sorted_index(ctx, R, b, 2, ix_mid, &b->mid_prefix, b->view.mid_prefix, (int)ix.pos_bits, true));
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
                         cudaStream_t gen) {
    DevBuf& d = c->bitmaps[words];
    CK(d.ensure((size_t)c->n * words * 8 + 8, ctx->stream));
    if (gen && gen != ctx->stream) {
        CK(cudaEventRecord(ctx->ev_fork, ctx->stream));
        CK(cudaStreamWaitEvent(gen, ctx->ev_fork, 0));
    }
    // beside the index build the generation takes a few blocks per SM (it is
    // bandwidth-bound; the index build is latency-bound and needs the SMs)
    const unsigned cap = gen && gen != ctx->stream ? (unsigned)(ctx->sm_count * HS_SIG_BLOCKS_PER_SM) : 0u;
    CK(generate_bitmaps(c->view(), words, d.as<uint64_t>(), gen ? gen : ctx->stream, cap));
    *out = d.as<uint64_t>();
    return HYSET_OK;
}

}  // namespace hs
