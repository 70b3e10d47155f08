// pipeline.cu — calls whose input arrives from host memory in chunks while
// the device already works on the chunks that have landed: the text reader
// (hyset_collection_parse) and the upload + self-join in one call
// (hyset_self_join_host).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "host.h"

namespace hs {

namespace {
constexpr uint64_t JOIN_POINT_TOKENS = 20ull << 20;  // a host-input join runs a piece every 80 MB landed
// The small chunks at the end of the copy are checked and emitted in groups of
// at least 32 MB (or at a join point): the context's stream is behind the copy
// by then, and each group costs its launches whatever its size.
constexpr uint64_t GROUP_MIN_TOKENS = 8ull << 20;

cudaEvent_t nth_event(std::vector<cudaEvent_t>& v, size_t k) {
    while (v.size() <= k) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        v.push_back(e);
    }
    return v[k];
}

// Token offsets where the copy chunks of a host-input join end (pipe_chunk).
std::vector<uint64_t> chunk_ends(uint64_t n_tokens) {
    std::vector<uint64_t> ends;
    for (uint64_t t = 0; t < n_tokens;) {
        t += pipe_chunk(n_tokens - t);
        ends.push_back(t);
    }
    return ends;
}
}  // namespace

cudaEvent_t pipe_event(hyset_ctx* ctx, size_t k) { return nth_event(ctx->pipe_ev, k); }

}  // namespace hs

using namespace hs;

extern "C" {

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
        std::swap(staged, aligned);  // staged (released by the guard on every return): the aligned copy
        const cudaError_t e = cudaMemcpyAsync(staged.p, d_text, n_bytes, cudaMemcpyDeviceToDevice, s);
        aligned.release(s);
        CK(e);
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
    auto guard = on_exit([&] {  // every early return releases the collection (copies finished first)
        if (c) {
            cudaStreamSynchronize(cp);
            hyset_collection_free(ctx, c.release());
        }
    });
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
    const std::vector<uint64_t> ends = chunk_ends(n_tokens);
    const uint64_t n_chunks = ends.size();
    for (uint64_t k = 0; k < n_chunks; ++k) {
        const uint64_t t0 = k ? ends[k - 1] : 0, t1 = ends[k];
        CK(cudaMemcpyAsync(C->tokens.as<uint32_t>() + t0, tokens + t0, (t1 - t0) * 4, cudaMemcpyHostToDevice, cp));
        cudaEvent_t e = pipe_event(ctx, k);
        if (!e) return bail(fail(ctx, HYSET_E_CUDA, "event creation"));
        CK(cudaEventRecord(e, cp));
    }
    // 2. one device pass over the sizes (and starts) while the tokens are copied:
    //    size order, contiguity of given starts, the total size, first_ge, and
    //    for every chunk the first set that ends past it (sets before it are
    //    complete once the chunk has landed), read back with one wait (a host
    //    pass over a million sets outlasted the copy of the first chunks)
    bool contiguous = true, ordered = true;
    std::vector<uint32_t> chunk_hi(n_chunks, n_sets);
    {
        const uint32_t L = n_sets ? sizes[n_sets - 1] : 0;  // the largest size once the order is confirmed
        if (n_chunks > PIPE_MAX_CHUNKS) return bail(fail(ctx, HYSET_E_UNSUPPORTED, "too many copy chunks"));
        const size_t words = 4 + n_chunks;  // flags, spare, total size (u64), chunk_hi[n_chunks]
        CK(C->first_ge.ensure(((size_t)L + 2) * 4, s));
        CK(ctx->sc->sscan.ensure(words * 4, s));
        uint32_t* d = ctx->sc->sscan.as<uint32_t>();
        CK(cudaMemsetAsync(d, 0, 16, s));
        CK(cudaMemsetAsync(d + 4, 0xFF, n_chunks * 4, s));
        CK(size_scan(C->d_sizes, C->d_starts, starts_given, n_sets, L, n_tokens, d, C->first_ge.as<uint32_t>(), d + 4,
                     s));
        void* stage = nullptr;
        ST(host_stage(ctx, (words + L + 2) * 4, &stage));
        uint32_t* h = static_cast<uint32_t*>(stage);
        CK(cudaMemcpyAsync(h, d, words * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(h + words, C->first_ge.p, ((size_t)L + 2) * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        ordered = (h[0] & 1u) == 0;
        contiguous = !starts_given || (h[0] & 2u) == 0;
        uint64_t run = 0;
        std::memcpy(&run, h + 2, 8);
        // contiguous sets past the token array: rejected here, before any
        // kernel reads them (the device checks are read only after the join)
        if (contiguous && run > n_tokens) return bail(fail(ctx, HYSET_E_INVALID, "sizes sum past n_tokens"));
        if (!ordered) return bail(fail(ctx, HYSET_E_INVALID, "sets must be ordered by non-decreasing size"));
        for (uint64_t k = 0; k < n_chunks; ++k) chunk_hi[k] = h[4 + k] == 0xFFFFFFFFu ? n_sets : h[4 + k];
        size_meta_from_first_ge(C, h + words, L);
    }
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
        auto it = ctx->tune_cache.find(key);
        if (it == ctx->tune_cache.end()) pipelined = false;
        else {
            tn.bits = it->second.bits;
            if (!o->verify_mode && it->second.vmode) tn.vmode = it->second.vmode;
            if (!o->fgss_batch && it->second.batch) tn.batch = it->second.batch;
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
        // Token records (see build_sorted_index) when a join with this key had
        // lists short enough: the entries go straight into the records as the
        // chunks land; the ordering pass flags a list that outgrew its record
        // (this collection's tokens differ), and the join is then run again
        // over lists.
        auto lit = ctx->longest_cache.find(key);
        bool records = assumed && lit != ctx->longest_cache.end() && lit->second <= REC_ENTRIES &&
                       (uint64_t)U <= REC_MAX_TOKENS;
        if (records) {
            CK(ix.rec.ensure((size_t)U * REC_CAP * 4, s));
            record_layout(C, b, 0, pb, &ix.rec_bits, &ix.rec_bound);
        }
        const uint32_t big_lo = first_long_prefix(C, b->index_prefix);  // emitted a warp per set from here on
        bool lists_ready = false;  // prefix lengths and entry offsets computed
        auto prepare_lists = [&]() -> hyset_status {
            if (lists_ready) return HYSET_OK;
            CK(set_prefix_lengths(v, b->view.index_prefix, 0, n, len, s));
            CK(scan_exclusive(len, off, n, ctx->sc->scan.as<uint32_t>(), s));
            lists_ready = true;
            return HYSET_OK;
        };
        if (!records) ST(prepare_lists());
        // With records, the join runs in pieces while the copy goes on: once the
        // entries of every landed set are in the records and the records are
        // ordered, the landed probes have every candidate they can pair with (a
        // candidate comes before its probe in size order), so they are joined
        // then, on the context's stream (the copy engine keeps copying); the
        // pairs of all pieces go to one buffer.
        const bool streamed = records && n_chunks > 1;
        JoinParams SP{};
        uint64_t cap = 0;
        uint32_t* prev = nullptr;  // each record's count at the last ordering pass
        uint32_t join_launches = 0, join_lo = 0;  // probes [0, join_lo) are joined
        uint64_t joined_to = 0;                    // the tokens that had landed at the last join point
        if (streamed) {
            ix.records = true;
            ix.sim = b->sim;
            ix.tau = b->tau;
            ix.kind = 0;
            ix.universe = U;
            ix.entries = E;
            ix.pos_bits = pb;
            const bool count_only = o->count_only != 0;
            cap = count_only ? 0 : (o->pair_capacity ? o->pair_capacity : std::max<uint64_t>(1u << 20, 4ull * n));
            CK(ctx->s_count.ensure(16, s));
            CK(ctx->s_work.ensure((2 * n_chunks + 4) * 4, s));
            CK(ctx->s_stats.ensure(64, s));
            if (!count_only) CK(ctx->s_pairs.ensure(std::max<uint64_t>(cap, 1) * sizeof(uint2), s));
            CK(ctx->sc->order.ensure((size_t)U * 4 + 4, s));
            prev = ctx->sc->order.as<uint32_t>();
            CK(cudaMemsetAsync(prev, 0xFF, (size_t)U * 4, s));  // the first pass orders every record
            // every record word padding until written: a join reading a record
            // while a later pass orders it sees only entries of its own and
            // earlier chunks in place, padding, or entries of later sets (above
            // every window it counts), never a word left from an earlier call
            CK(cudaMemsetAsync(ix.rec.p, 0xFF, (size_t)U * REC_CAP * 4, s));
            CK(cudaMemsetAsync(ctx->s_count.p, 0, 16, s));
            CK(cudaMemsetAsync(ctx->s_work.p, 0, (2 * n_chunks + 4) * 4, s));
            if (o->collect_stats) CK(cudaMemsetAsync(ctx->s_stats.p, 0, 64, s));
            SP.R = C->view();
            SP.S = SP.R;
            SP.B = b->view;
            SP.first_ge = C->first_ge.as<uint32_t>();
            SP.R_L = C->max_size;
            SP.self = 1;
            SP.grab = std::min<uint32_t>(tn.batch, 32);
            SP.r_lo = 0;
            SP.r_hi = n;
            SP.X = ix.view();
            split_heavy(C, b, SP);
            if (words) {
                SP.bits_R = SP.bits_S = bits.as<uint64_t>();
                SP.words = words;
            }
            SP.out = Sink{count_only ? nullptr : ctx->s_pairs.as<uint2>(), ctx->s_count.as<unsigned long long>(), cap,
                          count_only ? 1 : 0, 0};
            SP.stats = o->collect_stats ? ctx->s_stats.as<unsigned long long>() : nullptr;
        }
        uint32_t lo = 0;
        uint64_t grouped_to = 0;  // the tokens that had landed at the last group
        for (uint64_t k = 0; k < n_chunks && lo < n; ++k) {
            const bool last = k + 1 == n_chunks;
            const bool join_point = streamed && (last || ends[k] - joined_to >= JOIN_POINT_TOKENS);
            if (!last && !join_point && ends[k] - grouped_to < GROUP_MIN_TOKENS) continue;  // with the next group
            // sets whose tokens end inside the chunks copied so far
            const uint32_t hi = last ? n : std::max(lo, chunk_hi[k]);
            CK(cudaStreamWaitEvent(s, pipe_event(ctx, k), 0));
            grouped_to = ends[k];
            if (hi <= lo) continue;
            CollView part = v;
            part.sizes += lo;
            part.starts += lo;
            part.meta += lo;
            part.n = hi - lo;
            // the checks (and the signatures, in the same pass over the tokens)
            if (words)
                CK(validate_with_bitmaps(part, n_tokens, ctx->s_flags.as<uint32_t>(), C->meta.as<uint2>() + lo, words,
                                         bits.as<uint64_t>() + (size_t)lo * words, s, size_at(C, lo)));
            else
                CK(validate_collection(part, n_tokens, ctx->s_flags.as<uint32_t>(), C->meta.as<uint2>() + lo, s));
            if (records)
                CK(emit_records(v, b->view.index_prefix, ix.rec_bits, counts, ix.rec.as<uint32_t>(), U, s, lo, hi,
                                ix.rec_bound ? bound_fields(b) : BoundFields{}, big_lo));
            else
                CK(emit_packed_entries(v, off, len, pb, ctx->sc->tok.as<uint32_t>(), ix.set.as<uint32_t>(), counts, s,
                                       lo, hi, U + 1, big_lo));
            // at a join point (the last chunk, or JOIN_POINT_TOKENS since the last
            // one): order the records, then join the probes not joined yet, all
            // in stream order while the next chunks are copied
            if (join_point) {
                CK(order_records(counts, U, ix.rec.as<uint32_t>(), s, ctx->s_flags.as<uint32_t>(), prev));
                if (join_launches == 0) CK(cudaEventRecord(ctx->ek0, s));
                JoinParams Q = SP;
                Q.p_lo = join_lo;
                Q.p_hi = hi;
                // the pieces of the longest sets hold few probes: with fewer than
                // four probe batches per warp the launch ends on its slowest
                // warps, so their batches are halved (down to 3)
                while (Q.grab > 3 && (uint64_t)(hi - join_lo) < 4ull * Q.grab * join_resident_warps(ctx->sm_count))
                    Q.grab = std::max(3u, (Q.grab + 1) / 2);
                Q.work = ctx->s_work.as<unsigned int>() + 2 * join_launches;  // probe batches, split probes
                CK(launch_join(Q, TECH_FGSS, tn.vmode, ctx->sm_count, s));
                ++join_launches;
                join_lo = hi;
                joined_to = ends[k];
            }
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
        bool joined = false;  // the chunk-by-chunk join stands
        if (streamed) {
            CK(cudaEventRecord(ctx->ek1, s));
            CK(cudaEventRecord(ctx->ev1, s));
            CK(cudaMemcpyAsync(f, ctx->s_flags.p, 8, cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(f + 10, ctx->s_count.p, 8, cudaMemcpyDeviceToHost, s));
            if (SP.stats) CK(cudaMemcpyAsync(res->stats, SP.stats, 64, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            const hyset_status vs = verdict();
            if (vs != HYSET_OK) return bail(vs);
            unsigned long long count = 0;
            std::memcpy(&count, f + 10, 8);
            // a list that outgrew its record, a token past the assumed universe
            // or a full pair buffer: the join is run again below (records, then lists)
            if (!(f[0] & REC_OVERFLOW) && f[1] + 1 <= U && (o->count_only || count <= cap)) {
                float ms = 0, kms = 0;
                CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
                CK(cudaEventElapsedTime(&kms, ctx->ek0, ctx->ek1));
                res->device_ms = ms;
                res->kernel_ms = kms;
                res->count = count;
                P = SP;
                ST(deliver_pairs(ctx, P, o, res.get()));
                joined = true;
            }
        }
        for (int attempt = 0; attempt < 2 && !joined; ++attempt) {
            C->universe = U;
            CK(ctx->sc->counts.ensure(((size_t)U + 1) * 4, s));
            CK(ix.list_off.ensure(((size_t)U + 1) * 4, s));
            CK(ctx->sc->scan.ensure(std::max(scan_words, scan_scratch_words((uint64_t)U + 1)) * 4, s));
            const bool rec_now = records && attempt == 0;
            if (rec_now) {
                CK(order_records(counts, U, ix.rec.as<uint32_t>(), s, ctx->s_flags.as<uint32_t>()));
            } else {
                ST(prepare_lists());
                if (attempt > 0 || records)  // the list build reordered the entries (or none were emitted): emit them
                    CK(emit_packed_entries(v, off, len, pb, ctx->sc->tok.as<uint32_t>(), ix.set.as<uint32_t>(), nullptr,
                                           s, 0, 0xFFFFFFFFu, 0xFFFFFFFFu, big_lo));
                counts = ctx->sc->counts.as<uint32_t>();
                if (!(assumed && attempt == 0)) {  // not counted while the chunks landed
                    CK(cudaMemsetAsync(counts, 0, ((size_t)U + 1) * 4, s));
                    CK(token_histogram(ctx->sc->tok.as<uint32_t>(), E, counts, U + 1, s));
                }
                CK(index_lists(ctx->sc->tok.as<uint32_t>(), ix.set.as<uint32_t>(), E, U, counts,
                               ix.list_off.as<uint32_t>(), ctx->sc->altk.as<uint32_t>(), ctx->sc->altv.as<uint32_t>(),
                               ctx->sc->gate.as<uint32_t>(), key_bits_for(U), ctx->sc->scan.as<uint32_t>(), s));
            }
            ix.records = rec_now;
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
            split_heavy(C, b, P);
            if (words) {
                P.bits_R = P.bits_S = bits.as<uint64_t>();
                P.words = words;
            }
            if (assumed) CK(cudaMemcpyAsync(f, ctx->s_flags.p, 8, cudaMemcpyDeviceToHost, s));
            // the longest list (a list build with the device's choice writes it)
            if (!rec_now) CK(cudaMemcpyAsync(f + 14, ctx->sc->gate.p, 4, cudaMemcpyDeviceToHost, s));
            const hyset_status js = run_join(ctx, P, TECH_FGSS, tn.vmode, o, res.get(), true);  // synchronises
            if (js != HYSET_OK) return bail(js);
            if (!rec_now && E) ctx->longest_cache[key] = f[14];
            if (!assumed) break;
            const hyset_status vs = verdict();
            if (vs != HYSET_OK) return bail(vs);
            const bool grown = rec_now && (f[0] & REC_OVERFLOW);  // a list outgrew its record
            if (grown) ctx->longest_cache.erase(key);
            if (f[1] + 1 <= U && !grown) break;  // every token was indexed: the join stands
            U = std::max(U, f[1] + 1);  // a larger token or a longer list: index (as lists) and join again
            assumed = false;
        }
        C->universe = f[1] + 1;
        ctx->universe_cache[ukey] = C->universe;
        res->technique = HYSET_TECH_FGSS;
        res->bitmap_bits = tn.bits;
        res->verify_mode = (uint32_t)tn.vmode;
        res->probe_batch = P.grab;
        res->selector = selector;
        if (o->collect_stats) res->stats[3] = E;
        res->launches = launches() - launches0;
    }
    if (coll_out) *coll_out = c.release();
    else hyset_collection_free(ctx, c.release());
    *out = res.release();
    return HYSET_OK;
}

}  // extern "C"
