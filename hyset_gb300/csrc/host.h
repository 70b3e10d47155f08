// host.h — host-side functions shared by the translation units behind the C
// ABI (capi.cu, collection.cu, bounds.cu, index_host.cu, plan.cu,
// join_host.cu, pipeline.cu, batch_host.cu, handlers.cu, verifier.cu).
// Every device step they issue runs on the context's stream.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "internal.h"

namespace hs {

// Runs f when the scope ends (cleanup of partially built objects on every
// early return).
template <typename F>
struct OnExit {
    F f;
    ~OnExit() { f(); }
};
template <typename F>
OnExit<F> on_exit(F f) {
    return OnExit<F>{f};
}

// ---- errors (capi.cu) -------------------------------------------------------
// Records `what` (and the CUDA error) as the context's last error; returns st.
hyset_status fail(hyset_ctx* ctx, hyset_status st, const char* what, cudaError_t e = cudaSuccess);

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t _e = (call);                                                                        \
        if (_e != cudaSuccess)                                                                          \
            return ::hs::fail(ctx, _e == cudaErrorMemoryAllocation ? HYSET_E_NOMEM : HYSET_E_CUDA, #call, _e); \
    } while (0)

#define ST(call)                       \
    do {                               \
        hyset_status _s = (call);      \
        if (_s != HYSET_OK) return _s; \
    } while (0)

// ---- bound tables (bounds.cu) ----------------------------------------------
// The reference's bounds (include/hyset/similarity.hpp:11-54) in its double
// expressions; cosine and dice in the same style.
uint32_t sim_minoverlap(int sim, uint32_t l1, uint32_t l2, double t);
uint32_t minsize_of(int sim, uint32_t len, double t);
uint32_t minoverlap_of(int sim, uint32_t l1, uint32_t l2, double t);
uint32_t maxprefix_of(int sim, uint32_t len, double t);
uint32_t midprefix_of(int sim, uint32_t len, double t);
// Tables over lengths 0..L, cached per context; uploaded once (synchronises).
hyset_status get_bounds(hyset_ctx* ctx, int sim, double tau, uint32_t L, int index_maxprefix, Bounds** out);

// ---- collections (collection.cu) -------------------------------------------
// Pinned host memory of at least `bytes`, kept by the context.
hyset_status host_stage(hyset_ctx* ctx, size_t bytes, void** out);
hyset_status enqueue_collection_checks(hyset_ctx* ctx, hyset_coll* c, const uint32_t* h_sizes_or_null);
hyset_status finish_collection_checks(hyset_ctx* ctx, hyset_coll* c, const uint32_t* h_sizes_or_null);
hyset_status make_collection(hyset_ctx* ctx, hyset_coll* c, const uint32_t* h_sizes_or_null);

// ---- index builds and size statistics (index_host.cu) ------------------------
hyset_status build_size_meta(hyset_ctx* ctx, hyset_coll* c, const uint32_t* sizes);
// The host side of the size metadata (max_size, size_hist, h_first_ge) from a
// first_ge table computed on the device (c->first_ge holds it already).
void size_meta_from_first_ge(hyset_coll* c, const uint32_t* first_ge, uint32_t L);
uint32_t size_at(const hyset_coll* c, uint32_t i);
std::vector<uint64_t> range_hist(const hyset_coll* c, uint32_t lo, uint32_t hi);
uint64_t prefix_entries(const hyset_coll* c, const std::vector<uint32_t>& pre);
uint32_t bits_for(uint64_t v);
// The entry layout of an index's token records: the low rec_bits hold the
// longest probe the entry's positional bound admits (*bound: a self-join's
// midprefix index, kind 0, with a monotone minoverlap table, when set ids and
// that field fit 32 bits) or the entry's position (rec_bits = pb, the lists'
// layout).
void record_layout(const hyset_coll* c, const Bounds* b, int kind, uint32_t pb, uint32_t* rec_bits, bool* bound);
// The tables a bound-layout record build reads (jaccard, dice: max_sum;
// cosine: lp_row / lp_tab).
BoundFields bound_fields(const Bounds* b);
// The first set id whose prefix (pre[size] tokens) is long enough to be
// emitted a warp per set (0xFFFFFFFF: none).
uint32_t first_long_prefix(const hyset_coll* c, const std::vector<uint32_t>& pre);
int key_bits_for(uint32_t universe);
hyset_status build_sorted_index(hyset_ctx* ctx, hyset_coll* c, const Bounds* b, int kind, Index& ix,
                                const std::vector<uint32_t>* pre = nullptr, const uint32_t* d_pre = nullptr,
                                int force_pb = -1, bool records_ok = false);
bool use_bands(const Bounds* b, bool self);
hyset_status build_fgss_indexes(hyset_ctx* ctx, hyset_coll* R, const Bounds* b, bool self, Index& ix, Index& ix_mid,
                                JoinParams& P);
hyset_status build_groups(hyset_ctx* ctx, hyset_coll* c, const uint32_t* d_pre, const std::vector<uint32_t>& pre,
                          uint32_t U, uint64_t* entries);
hyset_status get_bitmaps(hyset_ctx* ctx, hyset_coll* c, int words, const uint64_t** out, cudaStream_t gen = nullptr);

// ---- configuration, selector, autotuner (plan.cu) ---------------------------
constexpr uint32_t TUNE_MIN_PROBES = 60000;  // joins this large time samples to pick their configuration
constexpr uint32_t DEFAULT_PROBE_BATCH = 3;  // probes per warp batch of the probe-major kernel, untuned
hyset_status check_opts(hyset_ctx* ctx, const hyset_join_opts* o);
struct Tuned {
    hyset_technique tech;
    int probe_major;
    uint32_t batch;
    uint32_t bits;
    int vmode;
};
Tuned tune(const hyset_coll* R, const hyset_coll* S, const hyset_join_opts* o,
           hyset_technique selected = HYSET_TECH_AUTO);
hyset_status compute_features(hyset_ctx* ctx, hyset_coll* R, hyset_coll* S, const hyset_join_opts* o, float* f,
                              double* base);
std::string coll_signature(const hyset_coll* c);
std::string join_key(const hyset_coll* R, const hyset_coll* S, const hyset_join_opts* o);
hyset_status select_technique(hyset_ctx* ctx, hyset_coll* R, hyset_coll* S, const hyset_join_opts* o,
                              hyset_technique* out, int* selector);
hyset_status plan_split(hyset_ctx* ctx, hyset_coll* R, const hyset_join_opts* o, uint32_t* split_at,
                        hyset_technique* low, hyset_technique* high);
// The autotuner: signature width (always), verification mode (vmode != NULL)
// and probe batch (batch != NULL) of a prefix-index join from timed samples.
// est_ms (optional): the join kernel's estimated time in the chosen configuration.
hyset_status autotune_bits(hyset_ctx* ctx, hyset_coll* R, hyset_coll* S, const hyset_join_opts* o, Bounds* b,
                           bool self, uint32_t p_lo, uint32_t p_hi, uint32_t* bits, int* vmode = nullptr,
                           uint32_t* batch = nullptr, float* est_ms = nullptr);

// ---- joins (join_host.cu) -----------------------------------------------------
hyset_status sort_device_pairs(hyset_ctx* ctx, uint2* pairs, uint64_t n, uint32_t n_probe, uint32_t n_indexed);
bool swap_sides(const hyset_coll* R, const hyset_coll* S, const hyset_join_opts* o);
hyset_status run_join(hyset_ctx* ctx, JoinParams P, int tech, int vmode, const hyset_join_opts* o, hyset_result* res,
                      bool timed_from_ev0, TokenJoinParams* T = nullptr);
// The probe-major prefix filter's split of the longest probes of S into slot
// segments (JoinParams::heavy_from, segs, seg_slots); none for banded joins.
// The launch's work buffer then needs two zeroed counters.
void split_heavy(const hyset_coll* S, const Bounds* b, JoinParams& P);
// The pairs of a finished join (res->count of them in the context's pair
// buffer): sorted when asked, left on the device or copied to the host.
hyset_status deliver_pairs(hyset_ctx* ctx, const JoinParams& P, const hyset_join_opts* o, hyset_result* res);
hyset_status do_join(hyset_ctx* ctx, hyset_coll* R, hyset_coll* S, const hyset_join_opts* o, hyset_result* res);

// ---- host-input pipelines (pipeline.cu) --------------------------------------
// One event per copy chunk, created on demand (nullptr on failure).
cudaEvent_t pipe_event(hyset_ctx* ctx, size_t k);


// ---- batches (batch_host.cu) --------------------------------------------------
void batch_release(hyset_ctx* ctx);

}  // namespace hs
