// verifier.cu — explicit candidate lists (hybrid::device_handler): the
// batched host-side verifier and verification of lists already on the device.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "host.h"

using namespace hs;

extern "C" {

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
    auto guard = on_exit([&] {  // a failed creation releases what it allocated
        if (v) hyset_verifier_destroy(v.release());
    });
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
