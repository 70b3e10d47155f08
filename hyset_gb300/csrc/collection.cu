// collection.cu — uploaded collections: the input-contract checks (one pass
// over the tokens that also writes the (start, size) records), the host size
// statistics, upload from host or device arrays, download and release.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "host.h"

namespace hs {

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

}  // namespace hs

using namespace hs;

extern "C" {

hyset_status hyset_collection_upload(hyset_ctx* ctx, const uint32_t* tokens, uint64_t n_tokens,
                                     const uint32_t* starts, const uint32_t* sizes, uint32_t n_sets,
                                     hyset_coll** out) {
    if (!ctx || !out || (n_sets && (!sizes || (!tokens && n_tokens))))
        return fail(ctx, HYSET_E_INVALID, "null argument");
    if (n_tokens >= (1ull << 32)) return fail(ctx, HYSET_E_INVALID, "n_tokens must be < 2^32");
    *out = nullptr;
    CK(cudaSetDevice(ctx->device));
    auto c = std::make_unique<hyset_coll>();
    auto guard = on_exit([&] {  // a failed upload releases what it allocated
        if (c) hyset_collection_free(ctx, c.release());
    });
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
    ST(make_collection(ctx, c.get(), sizes));
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
    c->index.rec.release(s);
    c->index.set.release(s);
    c->index.pos.release(s);
    c->index_mid.list_off.release(s);
    c->index_mid.rec.release(s);
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

}  // extern "C"
