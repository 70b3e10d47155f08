// verifier.cu — explicit candidate lists (hybrid::device_handler): the
// streaming verifier over the candidate ring (ring.cu) and verification of
// lists already on the device.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>

#include "host.h"

using namespace hs;

namespace {

constexpr uint64_t PUBLISH_CANDS = 1u << 16;             // staged candidates that trigger a publication
constexpr uint64_t DEFAULT_WAIT_NS = 100'000'000;        // the consumer waits 100 ms for the producer
constexpr auto HOST_WAIT = std::chrono::seconds(60);     // the host waits this long for device progress
// control words in d_ctl (64-bit each)
enum : int { CTL_TAIL = 0, CTL_CLOSE = 1, CTL_CLAIM = 2, CTL_HEAD = 3, CTL_STATUS = 4, CTL_COUNT = 5, CTL_WORDS = 8 };

uint64_t pow2_at_least(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

unsigned long long* ctl(const hyset_verifier* v, int w) { return v->d_ctl.as<unsigned long long>() + w; }

RingView ring_view(const hyset_verifier* v) {
    RingView r{};
    r.tail = ctl(v, CTL_TAIL);
    r.close = ctl(v, CTL_CLOSE);
    r.claim = ctl(v, CTL_CLAIM);
    r.head = ctl(v, CTL_HEAD);
    r.done = v->d_done.as<unsigned long long>();
    r.status = reinterpret_cast<unsigned int*>(ctl(v, CTL_STATUS));
    r.recs = v->d_recs.as<RingRec>();
    r.cands = v->d_cands.as<uint32_t>();
    r.rec_cap = v->rec_cap;
    r.cand_cap = v->cand_cap;
    r.wait_ns = v->wait_ns;
    return r;
}

// Has the consumer launch ended?  (false while it runs)
bool consumer_ended(hyset_verifier* v) {
    if (!v->consumer_live) return true;
    const cudaError_t e = cudaEventQuery(v->ev_cons);
    if (e == cudaErrorNotReady) return false;
    v->consumer_live = false;
    return true;
}

// Launches the persistent consumer on its own stream, behind everything the
// publication stream has queued (ring copies, the status reset).
hyset_status launch_consumer(hyset_verifier* v) {
    hyset_ctx* ctx = v->ctx;
    CK(cudaMemsetAsync(ctl(v, CTL_STATUS), 0, 8, v->pub));
    CK(cudaEventRecord(v->ev_pub, v->pub));
    CK(cudaStreamWaitEvent(v->cons, v->ev_pub, 0));
    const Sink out{v->aggregate ? nullptr : v->pairs.as<uint2>(), ctl(v, CTL_COUNT),
                   v->aggregate ? 0ull : (unsigned long long)v->pair_cap, v->aggregate, 0};
    CK(launch_ring_consumer(v->indexed->view(), v->probe->view(), v->bounds->view, ring_view(v),
                            v->scenario == 2 ? 2 : 3, out, ctx->sm_count, v->cons));
    CK(cudaEventRecord(v->ev_cons, v->cons));
    v->consumer_live = true;
    return HYSET_OK;
}

// Reads the control words back (head, exit status).
hyset_status read_back(hyset_verifier* v) {
    hyset_ctx* ctx = v->ctx;
    CK(cudaMemcpyAsync(v->h_ctl, v->d_ctl.p, CTL_WORDS * 8, cudaMemcpyDeviceToHost, v->pub));
    CK(cudaStreamSynchronize(v->pub));
    v->head = v->h_ctl[CTL_HEAD];
    return HYSET_OK;
}

// Copies the staged records and candidates not yet on the device (a ring
// range wraps at most once: two copies each), then raises the device tail
// behind them on the same stream.  A consumer that has ended is relaunched.
hyset_status publish(hyset_verifier* v) {
    hyset_ctx* ctx = v->ctx;
    if (v->pushed == v->published) return HYSET_OK;
    auto copy_range = [&](void* dev, const void* host, uint64_t cap, uint64_t lo, uint64_t hi,
                          size_t elem) -> hyset_status {
        while (lo < hi) {
            const uint64_t at = lo & (cap - 1), n = std::min(hi - lo, cap - at);
            CK(cudaMemcpyAsync(static_cast<char*>(dev) + at * elem, static_cast<const char*>(host) + at * elem,
                               n * elem, cudaMemcpyHostToDevice, v->pub));
            lo += n;
        }
        return HYSET_OK;
    };
    ST(copy_range(v->d_recs.p, v->h_recs, v->rec_cap, v->published, v->pushed, sizeof(RingRec)));
    ST(copy_range(v->d_cands.p, v->h_cands, v->cand_cap, v->cand_published, v->cand_pushed, sizeof(uint32_t)));
    CK(ring_store(ctl(v, CTL_TAIL), v->pushed, v->pub));
    v->published = v->pushed;
    v->cand_published = v->cand_pushed;
    if (consumer_ended(v)) ST(launch_consumer(v));
    return HYSET_OK;
}

// Waits (bounded) until done() holds, reading the device's progress back and
// relaunching a consumer that ended while published records remain.
template <typename Done>
hyset_status wait_for(hyset_verifier* v, Done done) {
    hyset_ctx* ctx = v->ctx;
    auto since = std::chrono::steady_clock::now();
    uint64_t seen = v->head;
    for (int spin = 0;; ++spin) {
        ST(read_back(v));
        if (done()) return HYSET_OK;
        if (v->head != seen) {
            seen = v->head;
            since = std::chrono::steady_clock::now();
        }
        if (v->published > v->head && consumer_ended(v)) ST(launch_consumer(v));
        if (std::chrono::steady_clock::now() - since > HOST_WAIT)
            return fail(ctx, HYSET_E_TIMEOUT, "candidate ring: no verification progress");
        if (spin > 16) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

// Everything published is verified: the pairs since the last drain go to the
// host output and the device count restarts at zero.
hyset_status drain(hyset_verifier* v) {
    hyset_ctx* ctx = v->ctx;
    ST(publish(v));
    ST(wait_for(v, [v] { return v->head == v->published; }));
    const uint64_t count = v->h_ctl[CTL_COUNT];
    if (!v->aggregate && count) {
        const size_t old = v->out_pairs.size();
        v->out_pairs.resize(old + count);
        CK(cudaMemcpyAsync(v->out_pairs.data() + old, v->pairs.p, count * sizeof(hyset_pair), cudaMemcpyDeviceToHost,
                           v->pub));
    }
    CK(cudaMemsetAsync(ctl(v, CTL_COUNT), 0, 8, v->pub));
    CK(cudaStreamSynchronize(v->pub));
    v->out_count += count;
    v->undrained = 0;
    return HYSET_OK;
}

}  // namespace

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
    v->rec_cap = pow2_at_least(std::max<uint64_t>(max_probes, 64));
    v->cand_cap = pow2_at_least(std::max<uint64_t>(max_candidates, 1024));
    v->pair_cap = max_candidates;
    v->wait_ns = DEFAULT_WAIT_NS;
    ST(get_bounds(ctx, sim, threshold, std::max(indexed->max_size, probe->max_size), 0, &v->bounds));
    CK(cudaStreamCreateWithFlags(&v->pub, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&v->cons, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&v->ev_pub, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&v->ev_cons, cudaEventDisableTiming));
    CK(cudaMallocHost((void**)&v->h_recs, v->rec_cap * sizeof(RingRec)));
    CK(cudaMallocHost((void**)&v->h_cands, v->cand_cap * sizeof(uint32_t)));
    CK(cudaMallocHost((void**)&v->h_ctl, CTL_WORDS * 8));
    cudaStream_t s = v->pub;
    CK(v->d_recs.ensure(v->rec_cap * sizeof(RingRec), s));
    CK(v->d_cands.ensure(v->cand_cap * sizeof(uint32_t), s));
    CK(v->d_done.ensure(v->rec_cap * 8, s));
    CK(v->d_ctl.ensure(CTL_WORDS * 8, s));
    if (!v->aggregate) CK(v->pairs.ensure(v->pair_cap * sizeof(uint2), s));
    CK(cudaMemsetAsync(v->d_done.p, 0, v->rec_cap * 8, s));
    CK(cudaMemsetAsync(v->d_ctl.p, 0, CTL_WORDS * 8, s));
    // the consumer starts at once and waits for the producer's first records
    ST(launch_consumer(v.get()));
    CK(cudaStreamSynchronize(s));
    *out = v.release();
    return HYSET_OK;
}

/* device_handler::addCandidates (hybrid_algorithms.hpp:71-105): the
 * candidates are staged in the host ring and published in batches of 64K
 * candidates (or a quarter of the record ring); a candidate set larger than
 * half the candidate ring, or than the pair buffer, travels as several
 * records of the same probe.  The call waits only when the rings are full or
 * the pair buffer must be drained. */
hyset_status hyset_verifier_add_candidates(hyset_verifier* v, uint32_t probe_id, const uint32_t* candidates,
                                           uint32_t n) {
    if (!v || (n && !candidates)) return HYSET_E_INVALID;
    hyset_ctx* ctx = v->ctx;
    if (probe_id >= v->probe->n) return fail(ctx, HYSET_E_INVALID, "probe id out of range");
    for (uint32_t k = 0; k < n; ++k)
        if (candidates[k] >= v->indexed->n) return fail(ctx, HYSET_E_INVALID, "candidate id out of range");
    const uint64_t piece_max = std::max<uint64_t>(1, std::min(v->cand_cap / 2, v->pair_cap));
    const uint64_t rmask = v->rec_cap - 1, cmask = v->cand_cap - 1;
    uint32_t done = 0;
    while (done < n) {
        const uint64_t len = std::min<uint64_t>(n - done, piece_max);
        // each candidate yields at most one pair: the pair buffer holds every
        // pair of the candidates published since it was last drained
        if (!v->aggregate && v->undrained + len > v->pair_cap) ST(drain(v));
        auto has_room = [&] {
            const uint64_t cand_head = v->head < v->pushed ? v->h_recs[v->head & rmask].begin : v->cand_pushed;
            return v->pushed - v->head < v->rec_cap && v->cand_pushed + len - cand_head <= v->cand_cap;
        };
        if (!has_room()) {
            ST(publish(v));
            ST(wait_for(v, has_room));
        }
        RingRec& r = v->h_recs[v->pushed & rmask];
        r.probe = probe_id;
        r.n = (uint32_t)len;
        r.begin = v->cand_pushed;
        for (uint64_t k = 0; k < len;) {  // at most two copies (the ring wraps once)
            const uint64_t at = (v->cand_pushed + k) & cmask, m = std::min(len - k, v->cand_cap - at);
            std::memcpy(v->h_cands + at, candidates + done + k, m * sizeof(uint32_t));
            k += m;
        }
        v->pushed += 1;
        v->cand_pushed += len;
        v->undrained += len;
        done += (uint32_t)len;
        if (v->cand_pushed - v->cand_published >= PUBLISH_CANDS || v->pushed - v->published >= v->rec_cap / 4)
            ST(publish(v));
    }
    return HYSET_OK;
}

hyset_status hyset_verifier_set_wait(hyset_verifier* v, uint64_t microseconds) {
    if (!v || microseconds == 0) return HYSET_E_INVALID;
    v->wait_ns = microseconds * 1000ull;
    return HYSET_OK;
}

hyset_status hyset_verifier_status(hyset_verifier* v) {
    if (!v) return HYSET_E_INVALID;
    hyset_ctx* ctx = v->ctx;
    if (!consumer_ended(v)) return HYSET_OK;
    ST(read_back(v));
    return (unsigned int)v->h_ctl[CTL_STATUS] == RING_TIMEOUT
               ? fail(ctx, HYSET_E_TIMEOUT, "candidate ring: the consumer gave up waiting for the producer")
               : HYSET_OK;
}

hyset_status hyset_verify_device(hyset_ctx* ctx, const hyset_coll* indexed, const hyset_coll* probe,
                                 const uint32_t* d_probes, const uint32_t* d_offsets, const uint32_t* d_candidates,
                                 uint32_t n_probes, const hyset_join_opts* opts, hyset_result** out) {
    if (!ctx || !indexed || !opts || !out || (n_probes && (!d_probes || !d_offsets || !d_candidates)))
        return fail(ctx, HYSET_E_INVALID, "null argument");
    *out = nullptr;
    ST(check_opts(ctx, opts));
    CK(cudaSetDevice(ctx->device));
    hyset_coll* R = const_cast<hyset_coll*>(indexed);  // signature buffers live in the collections
    hyset_coll* S = const_cast<hyset_coll*>(probe ? probe : indexed);
    Bounds* b = nullptr;
    ST(get_bounds(ctx, opts->sim, opts->threshold, std::max(R->max_size, S->max_size), 0, &b));
    auto res = std::make_unique<hyset_result>();
    cudaStream_t s = ctx->stream;
    const int vmode = opts->verify_mode ? (int)opts->verify_mode : 3;
    // the signature bound first (technique AUTO or BITMAP; DIRECT merges every
    // candidate, as the reference does): width from bitmap_bits, else 128 bits
    // for mean set sizes up to 48 and 256 above; the signatures are generated
    // here, inside the call's device time
    int words = 0;
    if (opts->technique != HYSET_TECH_DIRECT && opts->technique != HYSET_TECH_FGSS) {
        const double avg = R->n ? (double)R->n_tokens / (double)R->n : 0.0;
        words = opts->bitmap_bits ? std::min(8, (int)(opts->bitmap_bits / 64)) : (avg <= 48.0 ? 2 : 4);  // 512 bits at most
    }
    CK(cudaEventRecord(ctx->ev0, s));
    const uint64_t *sig_r = nullptr, *sig_s = nullptr;
    if (words && n_probes) {
        ST(get_bitmaps(ctx, R, words, &sig_r));
        if (S == R) sig_s = sig_r;
        else ST(get_bitmaps(ctx, S, words, &sig_s));
    }
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
                                    sk, ctx->s_work.as<unsigned int>(), ctx->sm_count, s, sig_r, sig_s, words));
        CK(cudaEventRecord(ctx->ek1, s));
        unsigned long long count = 0;
        CK(cudaMemcpyAsync(&count, ctx->s_count.p, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        float kms = 0, dms = 0;
        CK(cudaEventElapsedTime(&kms, ctx->ek0, ctx->ek1));
        CK(cudaEventElapsedTime(&dms, ctx->ev0, ctx->ek1));
        res->kernel_ms = kms;
        res->device_ms = dms;  // signatures (first attempt) and the verification
        res->verify_mode = (uint32_t)vmode;
        res->bitmap_bits = (uint32_t)words * 64u;
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
    res->technique = words ? HYSET_TECH_BITMAP : HYSET_TECH_DIRECT;
    *out = res.release();
    return HYSET_OK;
}

/* device_handler::flush() (hybrid_algorithms.hpp:195-200): everything added
 * so far is verified and its pairs (or count) delivered. */
hyset_status hyset_verifier_flush(hyset_verifier* v) {
    if (!v) return HYSET_E_INVALID;
    return drain(v);
}

hyset_status hyset_verifier_output(const hyset_verifier* v, uint64_t* count, const hyset_pair** pairs) {
    if (!v) return HYSET_E_INVALID;
    if (count) *count = v->out_count;
    if (pairs) *pairs = v->aggregate ? nullptr : v->out_pairs.data();
    return HYSET_OK;
}

void hyset_verifier_destroy(hyset_verifier* v) {
    if (!v) return;
    if (v->consumer_live && v->d_ctl.p) {  // the consumer ends at the close word (it polls every few us)
        if (ring_store(ctl(v, CTL_CLOSE), 1, v->pub) == cudaSuccess) cudaStreamSynchronize(v->pub);
        cudaEventSynchronize(v->ev_cons);
    }
    cudaStream_t s = v->pub ? v->pub : v->ctx->stream;
    DevBuf* bufs[] = {&v->d_recs, &v->d_cands, &v->d_done, &v->d_ctl, &v->pairs};
    for (DevBuf* b : bufs) b->release(s);
    cudaStreamSynchronize(s);
    if (v->h_recs) cudaFreeHost(v->h_recs);
    if (v->h_cands) cudaFreeHost(v->h_cands);
    if (v->h_ctl) cudaFreeHost(v->h_ctl);
    if (v->ev_pub) cudaEventDestroy(v->ev_pub);
    if (v->ev_cons) cudaEventDestroy(v->ev_cons);
    if (v->pub) cudaStreamDestroy(v->pub);
    if (v->cons) cudaStreamDestroy(v->cons);
    delete v;
}

}  // extern "C"
