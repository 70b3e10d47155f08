// batch_host.cu — many joins in one persistent launch: the batch plan (per
// join its configuration, index and signature buffers, output sink, work
// units; joins ordered heaviest first), its capture into a CUDA graph keyed by
// the batch's signature, and replays.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "host.h"

namespace hs {

namespace {
constexpr float SOLO_MS = 20.0f;  // a join whose kernel is estimated this long runs as a launch of its own

std::string opts_key(const hyset_join_desc& d) {
    std::string k((const char*)&d.indexed, sizeof(d.indexed));
    k.append((const char*)&d.probe, sizeof(d.probe));
    k.append((const char*)&d.opts, sizeof(d.opts));
    return k;
}
}  // namespace

namespace {
// Gives back every buffer and graph of a plan (installed or not).
void release_plan(hyset_ctx* ctx, BatchPlan& bp) {
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
}
}  // namespace

void batch_release(hyset_ctx* ctx) {
    if (!ctx->batch) return;
    release_plan(ctx, *ctx->batch);
    ctx->batch.reset();
}

namespace {
// The device work of a batch: per join its index build and signatures, then
// one persistent launch over the units of every join.  Asynchronous only.
hyset_status batch_record(hyset_ctx* ctx, BatchPlan& bp) {
    cudaStream_t s = ctx->stream;
    const uint32_t n = (uint32_t)bp.joins.size();
    CK(cudaMemsetAsync(bp.counts.p, 0, n * sizeof(unsigned long long), s));
    CK(cudaMemsetAsync(bp.work.p, 0, 16 + 8 * (size_t)n, s));
    for (auto& bjp : bp.joins) {
        BatchJoin& bj = *bjp;
        if (bj.ktech == TECH_FGSS) {
            ST(build_sorted_index(ctx, bj.R, bj.b, bj.self ? 0 : 1, bj.ix, nullptr, nullptr, -1, bj.solo));
            if (use_bands(bj.b, bj.self))
                ST(build_sorted_index(ctx, bj.R, bj.b, 2, bj.ix_mid, &bj.b->mid_prefix, bj.b->view.mid_prefix,
                                      (int)bj.ix.pos_bits, bj.solo));
        }
        if (bj.words) {
            CK(generate_bitmaps(bj.R->view(), bj.words, bj.bits_r.as<uint64_t>(), s));
            if (!bj.self) CK(generate_bitmaps(bj.S->view(), bj.words, bj.bits_s.as<uint64_t>(), s));
        }
    }
    // the solo joins, heaviest first, each with the single-join kernel over its
    // own index (token records when its lists fit them), then the shared launch
    uint32_t q = 0;
    for (uint32_t k = 0; k < n; ++k) {
        BatchJoin& bj = *bp.joins[bp.order[k]];
        if (!bj.solo) continue;
        JoinParams P = bp.host_desc[k].P;
        P.X = bj.ix.view();
        if (use_bands(bj.b, bj.self)) P.X2 = bj.ix_mid.view();
        P.grab = std::min<uint32_t>(bj.batch, P.X2.set ? 16u : 32u);
        split_heavy(bj.S, bj.b, P);
        P.work = bp.work.as<unsigned int>() + 4 + 2 * q++;
        CK(launch_join(P, TECH_FGSS, bj.vmode, ctx->sm_count, s));
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
    auto guard = on_exit([&] {  // a plan that failed before it was installed gives its memory back
        if (plan) release_plan(ctx, *plan);
    });
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
        // owned by the plan from the start: a failure below releases its buffers
        plan->joins.push_back(std::make_unique<BatchJoin>());
        BatchJoin* bj = plan->joins.back().get();
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
        float est_ms = 0;  // the autotuner's estimate of the join kernel's time (0: not tuned)
        {
            const uint32_t a_lo = o->probe_end ? o->probe_begin : 0, a_hi = o->probe_end ? o->probe_end : S->n;
            if (o->technique == HYSET_TECH_AUTO && o->bitmap_bits == 0 && tn.tech == HYSET_TECH_FGSS &&
                a_hi - a_lo >= TUNE_MIN_PROBES)
                ST(autotune_bits(ctx, R, S, o, bj->b, bj->self, a_lo, a_hi, &tn.bits,
                                 o->verify_mode ? nullptr : &tn.vmode, o->fgss_batch ? nullptr : &tn.batch, &est_ms));
        }
        // a join whose kernel alone takes tens of milliseconds gains nothing from
        // sharing a launch and loses the single-join kernel's token records and
        // carried items: it runs as a launch of its own in the batch's graph; so
        // does one tuned to 1024-bit signatures, which the shared launch lacks
        // (their code would cost it registers)
        bj->solo = tn.tech == HYSET_TECH_FGSS && (est_ms >= SOLO_MS || tn.bits > 512);
        bj->vmode = tn.vmode;
        bj->tech = tn.tech;
        bj->ktech = tn.tech == HYSET_TECH_FGSS ? TECH_FGSS : (tn.tech == HYSET_TECH_DIRECT ? TECH_DIRECT : TECH_BITMAP);
        bj->words = (int)(tn.bits / 64);
        if (bj->ktech == TECH_DIRECT) bj->words = 0;
        if (bj->words > 8 && !bj->solo) bj->words = 8;  // explicit 1024 bits on a window technique
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
                if (R->size_hist[l]) max_pre = std::max(max_pre, bj->b->index_prefix[l]);
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
        bj->unit_probes = bj->ktech == TECH_FGSS ? desc[j].unit_probes : 0;
        bj->batch = desc[j].unit_probes;
        const uint32_t np = P.p_hi - P.p_lo;
        bj->units = bj->solo ? 0u : (np + desc[j].unit_probes - 1) / desc[j].unit_probes;
        cost[j] = (double)np * (double)(R->n_tokens / std::max<uint32_t>(R->n, 1) + 1) *
                  (bj->ktech == TECH_FGSS ? 1.0 : (double)R->n);
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
    CK(plan->work.ensure(16 + 8 * (size_t)n, s));  // the shared launch's counter, then two per solo join
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
    plan->host_desc = ordered;
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
        // a solo join builds here once more, with token records, so that the
        // records exist before the capture (the capture allocates nothing)
        if (bj.solo || !bj.R->list_path.count(index_tab))
            ST(build_sorted_index(ctx, bj.R, bj.b, bj.self ? 0 : 1, bj.ix, nullptr, nullptr, -1, bj.solo));
        if (use_bands(bj.b, bj.self) && (bj.solo || !bj.R->list_path.count(mid_tab)))
            ST(build_sorted_index(ctx, bj.R, bj.b, 2, bj.ix_mid, &bj.b->mid_prefix, bj.b->view.mid_prefix,
                                  (int)bj.ix.pos_bits, bj.solo));
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

}  // namespace hs

using namespace hs;

extern "C" {

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
        r->probe_batch = bj.unit_probes;
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

}  // extern "C"
