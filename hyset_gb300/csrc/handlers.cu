// handlers.cu — the reference-shaped handlers (bitmap::handler,
// fgssjoin::handler): block pairs and partitions of one collection, with the
// reference's per-indexed-block inverted index.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "host.h"

using namespace hs;

extern "C" {

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
    auto guard = on_exit([&] {  // a failed creation releases what it allocated
        if (h) hyset_handler_destroy(h.release());
    });
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

}  // extern "C"
