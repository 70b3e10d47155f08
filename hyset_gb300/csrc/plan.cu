// plan.cu — a join's configuration: option checks, the rule-based tuner, the
// features of a join, the learned technique selector (with the analytic cost
// model as its fallback), the partition split, the signature-width and
// verification-mode autotuner, and the host side of the MLP (upload, forward,
// gradient, training, installation).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "host.h"

namespace hs {

hyset_status check_opts(hyset_ctx* ctx, const hyset_join_opts* o) {
    if (!o) return fail(ctx, HYSET_E_INVALID, "null options");
    if (!(o->threshold > 0.0 && o->threshold <= 1.0)) return fail(ctx, HYSET_E_INVALID, "threshold must be in (0, 1]");
    if (o->sim < HYSET_JACCARD || o->sim > HYSET_DICE) return fail(ctx, HYSET_E_INVALID, "unknown similarity");
    if (o->technique < HYSET_TECH_AUTO || o->technique > HYSET_TECH_DIRECT)
        return fail(ctx, HYSET_E_INVALID, "unknown technique");
    if (o->bitmap_bits != 0 && o->bitmap_bits != 64 && o->bitmap_bits != 128 && o->bitmap_bits != 256 &&
        o->bitmap_bits != 512 && o->bitmap_bits != 1024)
        return fail(ctx, HYSET_E_INVALID, "bitmap_bits must be 0, 64, 128, 256, 512 or 1024");
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
Tuned tune(const hyset_coll* R, const hyset_coll* S, const hyset_join_opts* o, hyset_technique selected) {
    Tuned t{};
    const double avg = R->n ? (double)R->n_tokens / (double)R->n : 0.0;
    const uint64_t pairs_window = (uint64_t)R->n * (uint64_t)S->n;
    t.tech = o->technique;
    if (t.tech == HYSET_TECH_AUTO) t.tech = selected;
    if (t.tech == HYSET_TECH_AUTO) t.tech = (pairs_window <= 4000000ull) ? HYSET_TECH_BITMAP : HYSET_TECH_FGSS;
    // explicit FGSS defaults to the token-major kernel; AUTO to probe-major
    t.probe_major = (o->technique == HYSET_TECH_FGSS && !o->probe_major) ? 0 : 1;
    t.batch = o->fgss_batch ? o->fgss_batch : DEFAULT_PROBE_BATCH;
    t.bits = o->bitmap_bits;
    if (o->technique == HYSET_TECH_AUTO && t.bits == 0) t.bits = avg <= 48.0 ? 128 : 256;
    if (t.tech == HYSET_TECH_BITMAP && t.bits == 0) t.bits = 64;
    if (t.tech == HYSET_TECH_DIRECT) t.bits = 0;
    t.vmode = o->verify_mode ? (int)o->verify_mode : 1;
    if (t.vmode == 3) t.vmode = 1;  // the staged mode exists for explicit candidate lists only
    return t;
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

namespace {
const hyset_technique kSelectable[3] = {HYSET_TECH_BITMAP, HYSET_TECH_FGSS, HYSET_TECH_DIRECT};

// cost.hpp:28-58 / statistics.hpp:150-160: |c . (1, std, avg, tokfreq, n, n^2, U, index, bitmap)|
double analytic_cost(const double* c, const double* base, double bitmap_bits) {
    const double x[9] = {1.0, base[0], base[1], base[2], base[3], base[3] * base[3], base[4], base[5], bitmap_bits};
    double s = 0;
    for (int k = 0; k < 9; ++k) s += c[k] * x[k];
    return std::fabs(s);
}
}  // namespace

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
namespace {
constexpr uint32_t SPLIT_MIN_PROBES = 40000;
constexpr float SPLIT_MARGIN = 0.9f;
}  // namespace

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
namespace {
constexpr uint32_t TUNE_SAMPLE = 16384;  // a sample fills the GPU for about two waves
constexpr float TUNE_MARGIN = 0.92f;  // leave the rule's width only for an estimated gain of 8 % or more
constexpr float TUNE_VMODE_MARGIN = 0.97f;  // warp verification only for an estimated gain of 3 % or more
constexpr float TUNE_BATCH_MARGIN = 0.97f;  // a probe batch other than the default only for a gain of 3 % or more
constexpr uint32_t TUNE_BATCHES[] = {1, 2, 3, 4, 6, 8, 12};  // probe batches the autotuner times
constexpr float TUNE_BATCH_FULL_MS = 40.0f;  // batches are timed over the whole range up to this estimate
}  // namespace

// The signature width (and, when requested, the verification mode and the
// probe batch) of a prefix-index join, from timed samples of its probe range;
// cached per join key.  The batch is the tile of the probe-major kernel: the
// probes one warp filters together (its slot and item rounds are shared by
// the batch, so a larger batch keeps more loads in flight per warp but
// balances worse across warps).
hyset_status autotune_bits(hyset_ctx* ctx, hyset_coll* R, hyset_coll* S, const hyset_join_opts* o, Bounds* b,
                           bool self, uint32_t p_lo, uint32_t p_hi, uint32_t* bits, int* vmode, uint32_t* batch,
                           float* est_ms) {
    const std::string key = join_key(R, S, o);
    auto it = ctx->tune_cache.find(key);
    if (it != ctx->tune_cache.end() && (!vmode || it->second.vmode) && (!batch || it->second.batch)) {
        *bits = it->second.bits;
        if (vmode) *vmode = it->second.vmode;
        if (batch) *batch = it->second.batch;
        if (est_ms) *est_ms = it->second.est_ms;
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
    split_heavy(S, b, P);
    const uint32_t grab_cap = P.X2.set ? 16u : 32u;  // banded R-S joins: two lanes per probe
    const uint32_t base_batch = std::min(o->fgss_batch ? o->fgss_batch : DEFAULT_PROBE_BATCH, grab_cap);
    P.grab = base_batch;
    CK(ctx->s_count.ensure(16, s));
    CK(ctx->s_work.ensure(16, s));
    P.out = Sink{nullptr, ctx->s_count.as<unsigned long long>(), 0, 1};
    P.work = ctx->s_work.as<unsigned int>();
    const uint32_t cand[5] = {0, 128, 256, 512, 1024};
    float est[5] = {0, 0, 0, 0, 0}, kern_est[5] = {0, 0, 0, 0, 0};
    float best_ms = 0;
    uint32_t best = 256;
    const bool learned = ctx->has_width_mlp;  // the width network replaces the width samples
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
    auto use_width = [&](uint32_t width) -> hyset_status {
        const int words = (int)(width / 64);
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
        return HYSET_OK;
    };
    if (learned) {
        float f[MLP_IN], x[MLP_IN], y[MLP_OUT] = {0, 0, 0};
        ST(compute_features(ctx, R, S, o, f, nullptr));
        for (int k = 0; k < MLP_IN; ++k) x[k] = (f[k] - ctx->width_mean[k]) / ctx->width_scale[k];
        CK(ctx->d_feat.ensure(256, s));
        float* dx = ctx->d_feat.as<float>();
        CK(cudaMemcpyAsync(dx, x, sizeof x, cudaMemcpyHostToDevice, s));
        CK(mlp_forward(ctx->d_width_mlp.as<float>(), dx, 1, dx + 32, ctx->sm_count, s));
        CK(cudaMemcpyAsync(y, dx + 32, sizeof y, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        int w = 0;
        for (int k = 1; k < MLP_OUT; ++k)
            if (y[k] < y[w]) w = k;
        best = 128u << w;  // outputs: 128, 256, 512 bits
    }
    // the estimated time of width cand[k]: its signature generation (paid once
    // per join) plus the whole probe range's kernel time from the samples
    auto time_width = [&](int k) -> hyset_status {
        const int words = (int)(cand[k] / 64);
        P.words = words;
        P.bits_R = P.bits_S = nullptr;
        float gen_ms = 0;
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
        ST(sample(1, &kern_est[k]));
        est[k] = kern_est[k] + gen_ms;
        return HYSET_OK;
    };
    if (!learned) {
        for (int k = 0; k < 5; ++k) {
            ST(time_width(k));
            if (k == 0 || est[k] < best_ms) {
                best_ms = est[k];
                best = cand[k];
            }
        }
        // the rule's width (mean size <= 48: 128 bits, else 256) unless another is clearly faster
        const uint32_t rule = (double)R->n_tokens / (double)std::max<uint32_t>(R->n, 1) <= 48.0 ? 128u : 256u;
        const float rule_ms = est[rule == 128u ? 1 : 2];
        if (best != rule && best_ms > TUNE_MARGIN * rule_ms) best = rule;
    } else if (best == 512) {
        // the network's widest output: 1024 bits (long sets at low thresholds,
        // where 512-bit signatures pass most candidates) when clearly faster
        ST(time_width(3));
        ST(time_width(4));
        if (est[4] < TUNE_MARGIN * est[3]) best = 1024;
    }
    if (best >= 512 && std::max(kern_est[3], kern_est[4]) > 0 &&
        std::max(kern_est[3], kern_est[4]) <= TUNE_BATCH_FULL_MS) {
        // 512 against 1024 bits again over the whole probe range when that is
        // cheap: the samples weigh the heaviest probes (the largest sets, where
        // the wider signature pays) like the light ones and can misjudge it
        auto whole_at = [&](uint32_t width, float* out) -> hyset_status {
            ST(use_width(width));
            P.p_lo = p_lo;
            P.p_hi = p_hi;
            float ms = 0;
            for (int rep = 0; rep < 2; ++rep) {  // the first run warms the caches
                CK(cudaMemsetAsync(ctx->s_count.p, 0, 16, s));
                CK(cudaMemsetAsync(ctx->s_work.p, 0, 16, s));
                CK(cudaEventRecord(ctx->ek0, s));
                CK(launch_join(P, TECH_FGSS, 1, ctx->sm_count, s));
                CK(cudaEventRecord(ctx->ek1, s));
                CK(cudaEventSynchronize(ctx->ek1));
                CK(cudaEventElapsedTime(&ms, ctx->ek0, ctx->ek1));
            }
            *out = ms;
            return HYSET_OK;
        };
        float ms512 = 0, ms1024 = 0;
        ST(whole_at(512, &ms512));
        ST(whole_at(1024, &ms1024));
        best = ms1024 < TUNE_MARGIN * ms512 ? 1024u : 512u;
        kern_est[3] = ms512;
        kern_est[4] = ms1024;
    }
    const int kc = best == 0 ? 0 : best == 128 ? 1 : best == 256 ? 2 : best == 512 ? 3 : 4;
    float cur_ms = kern_est[kc];  // the chosen configuration's estimated kernel time
    // verification: a lane per surviving item, or the warp per item when the
    // samples show it faster at the chosen width (long merges: low thresholds,
    // cosine); an explicit mode is kept
    int vm = o->verify_mode == 2 ? 2 : 1;
    ST(use_width(best));
    if (learned) {  // the predicted width's own estimate (the base of the comparisons below)
        ST(sample(1, &cur_ms));  // the first run after the generation warms the caches: not kept
        ST(sample(1, &cur_ms));
    }
    if (vmode) {
        float warp_ms = 0;
        ST(sample(2, &warp_ms));
        if (warp_ms < TUNE_VMODE_MARGIN * cur_ms) {
            vm = 2;
            cur_ms = warp_ms;
        }
        *vmode = vm;
    } else if (vm == 2) {
        ST(sample(2, &cur_ms));
    }
    // probe batch: it trades loads in flight per warp against balance across
    // warps, which samples of a few thousand batches cannot show (they do not
    // fill the persistent launch), so the candidates run over the whole probe
    // range, when the range's estimated kernel time makes that cheap; a batch
    // other than the default only for a gain of 3 % or more
    uint32_t tb = base_batch;
    if (batch) {
        if (cur_ms <= TUNE_BATCH_FULL_MS) {
            auto whole = [&](uint32_t g, float* out) -> hyset_status {
                P.grab = g;
                P.p_lo = p_lo;
                P.p_hi = p_hi;
                CK(cudaMemsetAsync(ctx->s_count.p, 0, 16, s));
                CK(cudaMemsetAsync(ctx->s_work.p, 0, 16, s));
                CK(cudaEventRecord(ctx->ek0, s));
                CK(launch_join(P, TECH_FGSS, vm, ctx->sm_count, s));
                CK(cudaEventRecord(ctx->ek1, s));
                CK(cudaEventSynchronize(ctx->ek1));
                CK(cudaEventElapsedTime(out, ctx->ek0, ctx->ek1));
                return HYSET_OK;
            };
            float base_ms = 0;
            ST(whole(base_batch, &base_ms));  // warms the caches the other runs find warm too
            ST(whole(base_batch, &base_ms));
            float tb_ms = base_ms;
            for (uint32_t cand_b : TUNE_BATCHES) {
                const uint32_t g = std::min(cand_b, grab_cap);
                if (g == base_batch) continue;
                float ms = 0;
                ST(whole(g, &ms));
                if (ms < TUNE_BATCH_MARGIN * base_ms && ms < tb_ms) {
                    tb = g;
                    tb_ms = ms;
                }
            }
            cur_ms = tb_ms;  // a whole-range run: the estimate becomes a measurement
        }
        P.grab = base_batch;
        *batch = tb;
    }
    hyset_ctx::TuneChoice& ch = ctx->tune_cache[key];
    ch.bits = best;
    if (vmode) ch.vmode = vm;
    if (batch) ch.batch = tb;
    ch.est_ms = cur_ms;
    *bits = best;
    if (est_ms) *est_ms = cur_ms;
    return HYSET_OK;
}

}  // namespace hs

using namespace hs;

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

extern "C" {

hyset_status hyset_join_features(hyset_ctx* ctx, const hyset_coll* indexed, const hyset_coll* probe,
                                 const hyset_join_opts* opts, float* features, double* base_stats) {
    if (!ctx || !indexed || !opts || !features) return fail(ctx, HYSET_E_INVALID, "null argument");
    CK(cudaSetDevice(ctx->device));
    hyset_coll* R = const_cast<hyset_coll*>(indexed);
    hyset_coll* S = const_cast<hyset_coll*>(probe ? probe : indexed);
    return compute_features(ctx, R, S, opts, features, base_stats);
}

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

hyset_status hyset_width_selector_set(hyset_ctx* ctx, const float* params, const float* feature_mean,
                                      const float* feature_scale) {
    if (!ctx) return HYSET_E_INVALID;
    CK(cudaSetDevice(ctx->device));
    ctx->tune_cache.clear();
    ctx->has_width_mlp = false;
    if (!params) return HYSET_OK;
    if (!feature_mean || !feature_scale) return fail(ctx, HYSET_E_INVALID, "normalisation missing");
    for (int k = 0; k < MLP_IN; ++k)
        if (!(feature_scale[k] > 0.f)) return fail(ctx, HYSET_E_INVALID, "feature scale must be > 0");
    std::memcpy(ctx->width_mean, feature_mean, sizeof ctx->width_mean);
    std::memcpy(ctx->width_scale, feature_scale, sizeof ctx->width_scale);
    CK(ctx->d_width_mlp.ensure(MLP_PARAMS * 4, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_width_mlp.p, params, MLP_PARAMS * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->has_width_mlp = true;
    return HYSET_OK;
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

}  // extern "C"
