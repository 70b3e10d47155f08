/*
 * hyset_gb300.h — C ABI of the GB300 (sm_103a) exact set-similarity join.
 *
 * Drop-in boundary for chribell/hyset's GPU join path.  The reference exposes
 * C++ templates and structs only (no C ABI); each entry point below names the
 * reference interface it replaces (paths relative to the reference source tree).
 * Plain pointers and sizes only; no C++ or torch types cross this boundary.
 *
 * Conventions
 *   - Every call returns hyset_status; HYSET_OK is 0.  hyset_last_error(ctx)
 *     returns a human-readable message for the last failure on that context.
 *   - One context per host thread; a context owns one CUDA stream on one device.
 *   - Results are owned by the library until hyset_result_free.
 *   - Pairs are (probe set id, indexed set id).  In a self-join the ids are the
 *     positions in the size-sorted collection and first > second, exactly as the
 *     reference emits them (include/hyset/verification.hpp:128-129).
 *   - The output pair SET is bit-exact to the reference's host::allpairs on the
 *     same input; the ORDER of pairs is unspecified unless sorted on request.
 *   - The library never falls back to a CPU implementation: without a usable
 *     device every compute call fails with HYSET_E_NODEVICE.
 */
#ifndef HYSET_GB300_H
#define HYSET_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    HYSET_OK = 0,
    HYSET_E_INVALID = 1,     /* bad argument (null pointer, unsorted input, ...) */
    HYSET_E_CUDA = 2,        /* a CUDA runtime call failed */
    HYSET_E_NOMEM = 3,       /* device or host allocation failed */
    HYSET_E_OVERFLOW = 4,    /* a fixed-capacity output could not hold the result */
    HYSET_E_TIMEOUT = 5,     /* a bounded device wait gave up */
    HYSET_E_UNSUPPORTED = 6, /* option combination not implemented */
    HYSET_E_NODEVICE = 7     /* no CUDA device, or the library was built without one */
} hyset_status;

typedef enum { HYSET_JACCARD = 0, HYSET_COSINE = 1, HYSET_DICE = 2 } hyset_sim;

/* Filter technique.  BITMAP and FGSS are the reference's two GPU techniques
 * (src/bitmap.cu, src/fgss.cu); DIRECT verifies every length-compatible pair.
 * AUTO lets the library choose (learned selector, analytic cost model fallback).
 * The choice never changes the output. */
typedef enum {
    HYSET_TECH_AUTO = 0,
    HYSET_TECH_BITMAP = 1,
    HYSET_TECH_FGSS = 2,
    HYSET_TECH_DIRECT = 3
} hyset_technique;

/* hyset::structs::block (include/hyset/structs.hpp:10-54), same field order. */
typedef struct {
    uint32_t id, start_id, end_id, first_entry_position, last_entry_position, num_tokens, entries, size;
} hyset_block;

/* hyset::structs::pair (include/hyset/structs.hpp:76-81). */
typedef struct {
    uint32_t first, second;
} hyset_pair;

typedef struct {
    hyset_sim sim;
    double threshold;          /* in (0, 1] */
    hyset_technique technique;
    uint32_t bitmap_bits;      /* 64, 128, 256, 512 or 1024 (the probe-major prefix filter only; the
                                  window techniques, the token-major kernel and the candidate
                                  verifier use 512 for it); 0 = chosen by the library with technique
                                  AUTO (timed samples for joins of 60,000 probes or more, else
                                  128 bits for mean set sizes <= 48 and 256 above), no signature
                                  filter with an explicit technique */
    uint32_t count_only;       /* 1 = count result pairs, do not materialise them */
    uint32_t verify_mode;      /* 0 = auto (a lane per candidate, or a warp per candidate where
                                  the samples that choose the signature width show it faster),
                                  1 = one lane per candidate, 2 = one warp per candidate,
                                  3 = one lane per candidate from staged prefixes (explicit candidate
                                  lists; joins treat it as 1) */
    uint32_t sort_pairs;       /* 1 = return pairs sorted by (first, second) */
    uint64_t pair_capacity;    /* initial device pair buffer; 0 = automatic (grows on demand) */
    uint32_t device_pairs;     /* 1 = leave the pairs in device memory (hyset_result_device_pairs) */
    uint32_t collect_stats;    /* 1 = count filter work (hyset_result_stats); costs a few atomics */
    uint32_t probe_begin;      /* probe id range [probe_begin, probe_end) of this call; */
    uint32_t probe_end;        /* 0, 0 = every probe (a shard of a join, e.g. one rank's part) */
    uint32_t probe_major;      /* technique FGSS: 1 = probe-major kernel (set-id-sorted index, one warp
                                  per probe batch), 0 = token-major kernel (token groups in shared
                                  memory).  AUTO always uses probe-major; probe ranges need it */
    uint32_t fgss_batch;       /* probe-major FGSS: probes per warp batch (1..32); 0 = the default (3),
                                  or the autotuner's choice with technique AUTO */
    uint32_t orientation;      /* R-S joins: 0 = automatic (index the smaller collection, probe the
                                  larger), 1 = as given, 2 = swapped.  The result is the same pair
                                  set in every orientation, pairs always (probe id, indexed id) of
                                  the caller's collections; probe ranges keep the given orientation */
} hyset_join_opts;

typedef struct hyset_ctx hyset_ctx;
typedef struct hyset_coll hyset_coll;
typedef struct hyset_result hyset_result;
typedef struct hyset_handler hyset_handler;
typedef struct hyset_verifier hyset_verifier;

/* ---- context --------------------------------------------------------- */
/* Replaces the implicit cuda-api-wrappers current-device setup of every driver
 * (e.g. src/bitmap.cu:77-80).  device < 0 selects the current device. */
hyset_status hyset_create(int device, hyset_ctx** out);
void hyset_destroy(hyset_ctx* ctx);
const char* hyset_last_error(const hyset_ctx* ctx);
void hyset_default_opts(hyset_join_opts* opts);
/* No counterpart in the reference (its handlers own raw device arrays).
 * Device memory held by the library's buffers, summed over every context,
 * collection, handler and verifier alive (capacity planning, leak checks).
 * Allocation failures return HYSET_E_NOMEM and leave every object valid;
 * for tests, while the environment variable HYSET_FAULT_ALLOC holds N the
 * N-th device allocation counted from when that value was first seen fails. */
uint64_t hyset_device_bytes(void);

/* ---- collections ----------------------------------------------------- */
/* hyset::collection::device_collection(host_collection&) (include/hyset/collection.hpp:54-71):
 * uploads the CSR arrays of a collection whose sets are sorted ascending and
 * whose sets are ordered by size (the reference's input contract,
 * collection.hpp:93-177).  starts may be NULL (then sets are contiguous).
 * Returns HYSET_E_INVALID if sizes are not non-decreasing, a set is empty or
 * unsorted, or n_tokens >= 2^32. */
hyset_status hyset_collection_upload(hyset_ctx* ctx, const uint32_t* tokens, uint64_t n_tokens,
                                     const uint32_t* starts, const uint32_t* sizes, uint32_t n_sets,
                                     hyset_coll** out);
/* Same, from arrays already resident on the context's device (no host copy of tokens). */
hyset_status hyset_collection_from_device(hyset_ctx* ctx, const uint32_t* d_tokens, uint64_t n_tokens,
                                          const uint32_t* d_starts, const uint32_t* d_sizes,
                                          uint32_t n_sets, hyset_coll** out);
/* hyset::collection::read_collection (include/hyset/collection.hpp:93-177, split at :16-24)
 * on the GPU: parses the reference's text format (one set per line, tokens as
 * decimal numbers split by single spaces, '\n' or "\r\n" line ends, empty
 * lines skipped, one trailing space per line allowed) from `text` (host or
 * device memory, n_bytes long) into a device collection, validated as
 * hyset_collection_upload validates.  Items the reference would turn into
 * token 0 through atoi of an empty or non-numeric field (two spaces, a leading
 * space, a space before '\r', a line of only "\r"), other bytes, and numbers
 * of 2^32 or more return HYSET_E_INVALID; hyset_last_error names the first
 * bad byte offset.  n_bytes must be below 2^33. */
hyset_status hyset_collection_parse(hyset_ctx* ctx, const char* text, uint64_t n_bytes, hyset_coll** out);
void hyset_collection_free(hyset_ctx* ctx, hyset_coll* coll);
uint32_t hyset_collection_num_sets(const hyset_coll* coll);
/* Copies the collection's CSR arrays to host memory (each may be NULL to skip):
 * tokens[num_tokens], starts[num_sets], sizes[num_sets]. */
uint64_t hyset_collection_num_tokens(const hyset_coll* coll);
hyset_status hyset_collection_download(hyset_ctx* ctx, const hyset_coll* coll, uint32_t* tokens,
                                       uint32_t* starts, uint32_t* sizes);

/* ---- whole joins ----------------------------------------------------- */
/* Self-join R ⋈ R: what src/bitmap.cu:112-121 and src/fgss.cu:108-116 compute
 * with bitmap::handler / fgssjoin::handler over one partition of all blocks,
 * and what cpu_single computes with host::allpairs (src/cpu_single.cu:116-136). */
hyset_status hyset_self_join(hyset_ctx* ctx, const hyset_coll* coll, const hyset_join_opts* opts,
                             hyset_result** out);
/* R-S join: every (s, r), s in probe, r in indexed, with m >= minsize(b) and
 * |s ∩ r| >= minoverlap(b, m), (b, m) = (larger, smaller) size.  The reference
 * declares --foreign-input (e.g. src/bitmap.cu:31) but never reads it; this is
 * the self-join's predicate applied across two collections. */
hyset_status hyset_rs_join(hyset_ctx* ctx, const hyset_coll* indexed, const hyset_coll* probe,
                           const hyset_join_opts* opts, hyset_result** out);
/* The upload and the self-join in one call, from host arrays (the reference's
 * read_collection -> device_collection -> handler sequence, src/fgss.cu:88-116):
 * the tokens travel in chunks while the sets already on the device are checked
 * and indexed.  The arguments mean what they mean for hyset_collection_upload and
 * hyset_self_join (probe ranges are not accepted here); *coll_out (may be NULL)
 * receives the uploaded collection for later joins.  Same result and the same
 * input checks as the two calls. */
hyset_status hyset_self_join_host(hyset_ctx* ctx, const uint32_t* tokens, uint64_t n_tokens, const uint32_t* starts,
                                  const uint32_t* sizes, uint32_t n_sets, const hyset_join_opts* opts,
                                  hyset_coll** coll_out, hyset_result** out);

/* Many independent joins in one persistent, work-stealing launch (the
 * device-resident form of src/queue.cu:142-281's block-pair queue), the whole
 * sequence (index builds, signatures, launches) captured in a CUDA graph and
 * replayed when the same batch comes again.  An AUTO prefix-filter join the
 * autotuner estimates at 20 ms of kernel time or more runs as a launch of its
 * own inside the same graph (the single-join kernel: sharing a launch saves it
 * nothing).  probe == NULL (or probe == indexed) means a self-join. */
typedef struct {
    const hyset_coll* indexed;
    const hyset_coll* probe;
    hyset_join_opts opts;
} hyset_join_desc;
hyset_status hyset_batch_join(hyset_ctx* ctx, const hyset_join_desc* joins, uint32_t n_joins,
                              hyset_result** results /* [n_joins] */);

uint64_t hyset_result_count(const hyset_result* r);
const hyset_pair* hyset_result_pairs(const hyset_result* r); /* NULL when count_only */
hyset_technique hyset_result_technique(const hyset_result* r);
uint32_t hyset_result_bitmap_bits(const hyset_result* r);   /* signature width used (0 = none) */
uint32_t hyset_result_verify_mode(const hyset_result* r);   /* verification mode used (1 lane, 2 warp, 3 staged) */
/* Probes per warp batch of the probe-major prefix-filter kernel (the tile the
 * reference sizes with --block for its block-pair launches, src/fgss.cu and
 * device_algorithms.hpp:147-148); 0 when the join ran another kernel.  With
 * fgss_batch 0 and technique AUTO the autotuner picks it from timed samples
 * (joins of 60,000 probes or more). */
uint32_t hyset_result_probe_batch(const hyset_result* r);
/* Partition split chosen by the learned selector for an AUTO self-join: the
 * first probe id of the high range (0 = the join ran as one range) and, in
 * *low_technique (may be NULL), the low range's technique (the high range's is
 * hyset_result_technique). */
uint32_t hyset_result_split(const hyset_result* r, hyset_technique* low_technique);
double hyset_result_device_ms(const hyset_result* r);       /* CUDA-event time of the join's device work */
double hyset_result_kernel_ms(const hyset_result* r);       /* CUDA-event time of the filter+verify launch */
/* Device pointer to count (first, second) uint32 pairs when device_pairs was
 * set; valid until the next join on the same context. */
const void* hyset_result_device_pairs(const hyset_result* r);
/* Work counters when collect_stats was set: [0] filter items examined,
 * [1] items reaching verification, [2] candidate tokens of those items,
 * [3] index entries, [4] prefix tokens read by the filter, [5] signature
 * checks, [6] tokens read by verification (both sets); returns the number
 * written (<= n). */
uint32_t hyset_result_stats(const hyset_result* r, uint64_t* out, uint32_t n);
/* Kernel launches the join issued (index build, signatures, filter+verify). */
uint64_t hyset_result_launches(const hyset_result* r);
void hyset_result_free(hyset_result* r);

/* ---- reference-shaped handlers -------------------------------------- */
/* bitmap::handler(timer, hostCollection, deviceCollection, bitmapSize, blockSize,
 *                 aggregate, threshold)     include/hyset/device_algorithms.hpp:138-171
 * fgssjoin::handler(timer, hostCollection, deviceCollection, blockSize,
 *                   aggregate, threshold)   include/hyset/device_algorithms.hpp:322-348
 * technique selects which; bitmap_size is ignored for FGSS.  sim extends the
 * reference (which hard-codes jaccard). */
hyset_status hyset_handler_create(hyset_ctx* ctx, const hyset_coll* coll, hyset_technique technique,
                                  hyset_sim sim, uint32_t bitmap_size, uint32_t block_size,
                                  int aggregate, double threshold, hyset_handler** out);
/* handler::join(block*, block*): first = indexed block, second = probe block
 * (device_algorithms.hpp:177-229, :363-412).  Pairs/count accumulate in the
 * handler's output, like the pairs_handler / count_handler the reference
 * appends to. */
hyset_status hyset_handler_join_blocks(hyset_handler* h, const hyset_block* first, const hyset_block* second);
/* handler::join(partition*, partition*): block-level length filter, then every
 * surviving block pair (device_algorithms.hpp:21-53, :232-247, :416-432). */
hyset_status hyset_handler_join_partitions(hyset_handler* h, const hyset_block* first, uint32_t n_first,
                                           const hyset_block* second, uint32_t n_second);
/* output::pairs_handler::getPairs / count_handler::count (include/hyset/output.hpp:19-37). */
hyset_status hyset_handler_output(const hyset_handler* h, uint64_t* count, const hyset_pair** pairs);
hyset_status hyset_handler_clear_output(hyset_handler* h);
void hyset_handler_destroy(hyset_handler* h);

/* ---- candidate verifier (hybrid::device_handler) ------------------- */
/* hybrid::device_handler(indexed, probe, threads, scenario, aggregate, maxProbes,
 * maxCandidates, threshold)   include/hyset/hybrid_algorithms.hpp:41-62.
 * scenario 1 = one lane per candidate, 2 = one warp per candidate (merge-path).
 * The reference copies a host batch synchronously and verifies it on a
 * worker thread (hybrid_algorithms.hpp:107-193).  Here candidates stream
 * through device-resident rings (records: max_probes rounded up to a power of
 * two; candidate ids: max_candidates rounded up) that a persistent kernel,
 * started at creation, verifies as they are published: adding candidates
 * copies them asynchronously and returns, waiting only when the rings are
 * full or the pair buffer (max_candidates pairs) must be drained.  The kernel
 * waits for the producer at most the wait limit (default 100 ms) and then ends
 * (the next publication starts it again); every device wait is bounded. */
hyset_status hyset_verifier_create(hyset_ctx* ctx, const hyset_coll* indexed, const hyset_coll* probe,
                                   hyset_sim sim, uint32_t threads, uint32_t scenario, int aggregate,
                                   uint32_t max_probes, uint32_t max_candidates, double threshold,
                                   hyset_verifier** out);
/* device_handler::addCandidates(probeID, candidate_set&)  hybrid_algorithms.hpp:71-105 */
hyset_status hyset_verifier_add_candidates(hyset_verifier* v, uint32_t probe_id, const uint32_t* candidates,
                                           uint32_t n_candidates);
/* device_handler::flush()  hybrid_algorithms.hpp:195-200: verifies everything
 * added so far and appends its pairs (or count) to the output.  Returns
 * HYSET_E_TIMEOUT if the device made no progress for 60 s. */
hyset_status hyset_verifier_flush(hyset_verifier* v);
/* No counterpart in the reference.  How long the persistent verifier kernel
 * waits for published candidates before it ends (from its next start on). */
hyset_status hyset_verifier_set_wait(hyset_verifier* v, uint64_t microseconds);
/* No counterpart in the reference.  HYSET_E_TIMEOUT when the last verifier
 * kernel ended because the producer published nothing within the wait limit
 * (the next publication starts a new one), else HYSET_OK. */
hyset_status hyset_verifier_status(hyset_verifier* v);
hyset_status hyset_verifier_output(const hyset_verifier* v, uint64_t* count, const hyset_pair** pairs);
void hyset_verifier_destroy(hyset_verifier* v);
/* Device-resident candidate lists (the input of hybrid::device_handler's
 * kernels, hybrid_kernels.hpp:14-165, already on the device): probe
 * d_probes[i] of `probe` (NULL = indexed) owns candidates [d_offsets[i-1]
 * (0 for i = 0), d_offsets[i]) of `indexed`; pairs with overlap >= minoverlap
 * are returned as a join result (kernel_ms = the verification launch,
 * device_ms = the signatures and the launch).  Uses opts->sim, threshold,
 * verify_mode (0 = 3: one lane per candidate merging from a staged 16-token
 * prefix), count_only, pair_capacity, device_pairs, and technique: DIRECT
 * merges every candidate (the reference's scenario kernels); AUTO or BITMAP
 * first drops the candidates whose XOR signatures rule out minoverlap (the
 * bound of device_algorithms.hpp:104-113; bitmap_bits wide, 0 = 128 bits for
 * mean set sizes up to 48, else 256), which never changes the pairs. */
hyset_status hyset_verify_device(hyset_ctx* ctx, const hyset_coll* indexed, const hyset_coll* probe,
                                 const uint32_t* d_probes, const uint32_t* d_offsets, const uint32_t* d_candidates,
                                 uint32_t n_probes, const hyset_join_opts* opts, hyset_result** out);

/* ---- technique selector ------------------------------------------ */
/* statistics::extract (include/hyset/statistics.hpp:163-213) and the analytic
 * model of cost::run (include/hyset/cost.hpp:28-58) drive the reference's
 * technique choice.  Here a small FP32 network (12 -> 64 -> 64 -> 3, ReLU,
 * trained on the GPU by this library's kernels on timings this library
 * measured) predicts the log-time of the bitmap, prefix-index and
 * direct-verify techniques for a join; the analytic cost model is its
 * fallback; without either, fixed rules decide.  The choice never changes a
 * join's output. */
#define HYSET_FEATURES 12
#define HYSET_MLP_PARAMS 5187
#define HYSET_COST_TERMS 9
/* features[12]: log2(1+probes), mean size, size std, log2(1+max size),
 * log2(1+universe), threshold, sim/2, mean probe prefix, log2(1+index entries),
 * log2(1+token-frequency std), log2(1+max token frequency), log2(1+length-
 * compatible pairs).  base_stats[8] (may be NULL): the reference's
 * statistics::base — size std, mean size, token-frequency std, set count,
 * universe, index entries — then length-compatible pairs and mean prefix. */
hyset_status hyset_join_features(hyset_ctx* ctx, const hyset_coll* indexed, const hyset_coll* probe,
                                 const hyset_join_opts* opts, float* features, double* base_stats);
/* Host arrays: x[n][12], y/t/mask[n][3], params[HYSET_MLP_PARAMS]. */
hyset_status hyset_mlp_forward(hyset_ctx* ctx, const float* params, const float* x, uint32_t n, float* y);
hyset_status hyset_mlp_grad(hyset_ctx* ctx, const float* params, const float* x, const float* t, const float* mask,
                            uint32_t n, float* grad, float* loss);
/* Full-dataset Adam on the GPU; params is updated in place; loss_trace[steps] may be NULL. */
hyset_status hyset_mlp_train(hyset_ctx* ctx, float* params, const float* x, const float* t, const float* mask,
                             uint32_t n, uint32_t steps, float lr, float weight_decay, float* loss_trace);
/* Installs the selector AUTO uses: params (NULL: none) with the features'
 * normalisation x' = (x - mean) / scale, and the analytic model's coefficients
 * per technique (bitmap, fgss, direct) x HYSET_COST_TERMS in the reference's
 * form |c0 + c1 std + c2 avg + c3 tokfreq + c4 n + c5 n^2 + c6 universe +
 * c7 index + c8 bitmap| (NULL: none). */
hyset_status hyset_selector_set(hyset_ctx* ctx, const float* params, const float* feature_mean,
                                const float* feature_scale, const double* cost_coefficients);
/* No counterpart in the reference.  Installs a second network of the same
 * shape whose three outputs predict the prefix-filter join's log-time with
 * 128-, 256- and 512-bit signatures (same features and normalisation form);
 * with it, AUTO joins that tune their signature width take the predicted
 * width instead of timing samples of every width (the verification mode and
 * probe batch are still tuned).  params NULL removes it. */
hyset_status hyset_width_selector_set(hyset_ctx* ctx, const float* params, const float* feature_mean,
                                      const float* feature_scale);
/* Which selector chose the result's technique: -1 explicit, 0 rules,
 * 1 analytic cost model, 2 learned network. */
int hyset_result_selector(const hyset_result* r);

/* ---- verification without allocation ------------------------------ */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory when they verify: a host engine that owns all GPU memory through its
 * own pool and forbids allocations after start-up, or a latency-critical path
 * that cannot afford cudaMalloc's implicit device synchronisation.
 *
 * Verifies explicit candidate lists exactly like hyset_verifier (scenario 1:
 * one lane per candidate, 2: one warp per candidate): probe d_probes[i] of the
 * probe collection S owns candidates [d_offsets[i-1] (0 for i = 0),
 * d_offsets[i]) of the indexed collection R; (probe, candidate) is appended to
 * d_pairs when |probe ∩ candidate| >= minoverlap(|probe|, |candidate|).  All
 * inputs and outputs are device pointers; nothing is allocated and nothing is
 * copied from host memory: the call enqueues two kernels and two
 * device-to-device copies on `stream` (a cudaStream_t, NULL = legacy default
 * stream, on the current device) and returns without waiting.  *d_count
 * receives the number of result pairs (pairs past pair_capacity are counted
 * but not written); *d_skipped (optional) receives the number of candidates
 * skipped because a set is longer than max_set_size.  Both, and d_pairs, are
 * valid once the stream has reached the end of the call's work (for example
 * after cudaStreamSynchronize).
 *
 * Limits: Jaccard and dice only (HYSET_E_UNSUPPORTED for cosine); sets of at
 * most HYSET_NOALLOC_MAX_SET_SIZE tokens (larger max_set_size is rejected with
 * HYSET_E_UNSUPPORTED).  The scratch (counters and the minoverlap table) is one
 * HYSET_NOALLOC_SCRATCH_BYTES array in device memory that every GPU loading
 * the library keeps until exit.  All calls share it and it keeps the last
 * call's contents; each call's first kernel clears and rewrites it, so calls
 * that overlap on the GPU race and must be serialised by the caller.  The
 * first call on a device looks up the array's device address with that device
 * current (cudaGetSymbolAddress, once per device). */
#define HYSET_NOALLOC_SCRATCH_BYTES 65536
#define HYSET_NOALLOC_MAX_SET_SIZE 4096
hyset_status hyset_verify_candidates_noalloc(
    const uint32_t* d_r_tokens, const uint32_t* d_r_starts, const uint32_t* d_r_sizes,
    const uint32_t* d_s_tokens, const uint32_t* d_s_starts, const uint32_t* d_s_sizes, uint32_t max_set_size,
    const uint32_t* d_probes, const uint32_t* d_offsets, const uint32_t* d_candidates, uint32_t n_probes,
    hyset_sim sim, double threshold, uint32_t scenario, hyset_pair* d_pairs, uint64_t pair_capacity,
    unsigned long long* d_count, unsigned int* d_skipped, void* stream);

#ifdef __cplusplus
}
#endif
#endif
