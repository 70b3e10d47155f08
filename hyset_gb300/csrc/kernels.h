// kernels.h — host-side launchers of the CUDA kernels (defined in *.cu).
// Everything here is asynchronous on the given stream and returns the first
// CUDA error it sees.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace hs {

// Per-device kernel attributes (shared-memory opt-ins); call once per device
// before the first launch (hyset_create does).
cudaError_t prepare_kernels();

// Kernel launches issued by this library since load (bench bookkeeping).
unsigned long long launches();
void note_launches(unsigned n = 1);

// ---- parse.cu ------------------------------------------------------------
// The reference's text format on the device (one set per line, tokens split by
// single spaces).  Error bits of flags[0]:
constexpr uint32_t PARSE_E_CHAR = 1;        // a byte other than digit, ' ', '\r', '\n'
constexpr uint32_t PARSE_E_EMPTY_ITEM = 2;  // two spaces, a leading space, or a space before '\r'
constexpr uint32_t PARSE_E_LINE_END = 4;    // '\r' not followed by '\n', or a line of only "\r"
constexpr uint32_t PARSE_E_RANGE = 8;       // a number of more than 10 digits or >= 2^32
constexpr uint32_t PARSE_E_CAPACITY = 16;   // (not an input error) a token or line past the output capacity
uint64_t parse_tiles(uint64_t n_bytes);
// Per 4 KiB tile: token starts and line starts; flags / first_bad (byte offset,
// atomicMin) record errors.
// Tiles [tile_lo, tile_hi) only (default: all); a tile reads one byte on
// either side of its 4 KiB.
cudaError_t parse_count(const uint8_t* text, uint64_t n_bytes, uint32_t* tile_toks, uint32_t* tile_lines,
                        uint32_t* flags, unsigned long long* first_bad, cudaStream_t s, uint64_t tile_lo = 0,
                        uint64_t tile_hi = ~0ull);
// tile_tok0 / tile_line0: exclusive scans of the tile counts.  Writes every
// token and line_tok0[line] = index of the line's first token, for tiles
// [tile_lo, tile_hi) (default: all); indexes at or past tok_cap / line_cap
// are not written and set PARSE_E_CAPACITY.
cudaError_t parse_emit(const uint8_t* text, uint64_t n_bytes, const uint32_t* tile_tok0, const uint32_t* tile_line0,
                       uint32_t* tokens, uint32_t* line_tok0, uint32_t* flags, unsigned long long* first_bad,
                       cudaStream_t s, uint64_t tile_lo = 0, uint64_t tile_hi = ~0ull, uint32_t tok_cap = ~0u,
                       uint32_t line_cap = ~0u);
// In place: exclusive scans of the token and line counts of tiles [tile_lo,
// tile_hi) (at most 65,536 tiles), offset by carry[2k], carry[2k+1] (tokens,
// lines before the range); carry[2k+2], carry[2k+3] get the totals after it.
// One block: for chunks of a text scanned as they arrive.
cudaError_t parse_chunk_scan(uint32_t* tile_toks, uint32_t* tile_lines, uint64_t tile_lo, uint64_t tile_hi,
                             uint32_t* carry, uint64_t k, cudaStream_t s);
// starts[i] = line_tok0[i], sizes[i] = next line's first token - line_tok0[i].
cudaError_t parse_line_sizes(const uint32_t* line_tok0, uint32_t n_lines, uint32_t n_tokens, uint32_t* starts,
                             uint32_t* sizes, cudaStream_t s);

// ---- primitives.cu -------------------------------------------------------
// Exclusive prefix sum of n uint32 values (in may equal out).  `scratch` must
// hold scan_scratch_words(n) words.
size_t scan_scratch_words(uint64_t n);
cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* scratch, cudaStream_t s,
                           const uint32_t* gate = nullptr);

// Stable LSD radix sort of (key, value) pairs on the low `key_bits` bits of the
// keys.  Result lands in keys/vals; alt_* are ping-pong buffers of n words;
// `scratch` holds radix_scratch_words(n) words.  keep_keys = false leaves the
// keys array unsorted (only the values are wanted; the last pass skips them).
size_t radix_scratch_words(uint64_t n);
// gate: when non-null, every kernel of the sort runs only if the device word
// is above the short-list bound (see index_lists).
cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* alt_keys, uint32_t* alt_vals,
                             uint64_t n, int key_bits, uint32_t* scratch, cudaStream_t s, bool keep_keys = true,
                             const uint32_t* gate = nullptr);

// The index lists from prefix entries emitted in set order (e_token, e_val)
// and the per-token counts of tokens below U (counts[U+1]): list_off[U+1]
// (exclusive scan of counts) and e_val reordered so that each list holds its
// entries in emission order.  Without a host round trip: the longest list is
// written to *gate on the device; when every list has at most 64 entries the
// entries are scattered into their lists with atomics and each list is put
// back in emission order inside a warp (insertion sort in shared memory, the
// values being increasing in emission order), otherwise the stable radix
// passes on
// the token sort them (each kernel checks the gate and returns early when it
// is not its case).  *path (optional): 1 = only the short-list path (correct
// for any lists, slow for long ones), 2 = only the radix passes, 0 = choose:
// with h_gate (pinned) the longest list is read back once (a synchronisation)
// and *path set, otherwise both paths launch and the gate picks on the device
// (no host round trip: graph capture).  counts, e_token, alt_* and scratch
// (max of scan_scratch_words(U + 1) and radix_scratch_words(n) words) are
// clobbered.
cudaError_t index_lists(uint32_t* e_token, uint32_t* e_val, uint64_t n, uint32_t U, uint32_t* counts,
                        uint32_t* list_off, uint32_t* alt_keys, uint32_t* alt_vals, uint32_t* gate, int key_bits,
                        uint32_t* scratch, cudaStream_t s, int* path = nullptr, uint32_t* h_gate = nullptr);

// Prefix entries of sets [lo, hi): the first prefix_len(size) tokens of every
// set (include/hyset/collection.hpp:128-135).  entry_off must hold the
// exclusive scan of the per-set prefix lengths over [lo, hi) (relative to lo).
cudaError_t set_prefix_lengths(CollView c, const uint32_t* prefix_tab, uint32_t lo, uint32_t hi,
                               uint32_t* out_len, cudaStream_t s);
cudaError_t emit_prefix_entries(CollView c, uint32_t lo, uint32_t hi, const uint32_t* entry_off,
                                const uint32_t* len, uint32_t* e_token, uint32_t* e_set,
                                uint32_t* e_pos, cudaStream_t s);
// Packed form: e_token[k] = token, e_val[k] = (set << pos_bits) | position, and the
// token histogram counts[token]++ of tokens below `limit` in the same pass
// (counts may be nullptr).  Sets [lo, hi) only (hi = 0xFFFFFFFF: to the end);
// ids stay absolute.
// big_lo: sets from this id on have long prefixes and are emitted a warp
// per set (below it, a warp per 32 sets).
cudaError_t emit_packed_entries(CollView c, const uint32_t* entry_off, const uint32_t* len, uint32_t pos_bits,
                                uint32_t* e_token, uint32_t* e_val, uint32_t* counts, cudaStream_t s,
                                uint32_t lo = 0, uint32_t hi = 0xFFFFFFFFu, uint32_t limit = 0xFFFFFFFFu,
                                uint32_t big_lo = 0xFFFFFFFFu);

// Token records: when no list holds more than REC_ENTRIES entries, list t is
// the fixed REC_CAP-word record rec[REC_CAP t, REC_CAP t + REC_CAP): word 0
// the list's length, then its entries ascending and the rest 0xFFFFFFFF
// (never a valid packed entry).  A probe finds its window in one 128-byte
// line (32-byte loads, only as many as the length needs) and the build needs
// no offsets: no scan, no scatter pass.
constexpr uint32_t REC_CAP = 32;
constexpr uint32_t REC_ENTRIES = REC_CAP - 1;
constexpr uint64_t REC_MAX_TOKENS = 1ull << 25;  // records of larger universes would pass 4 GB
// Record build, pass 1: the first prefix_tab[size] tokens of every set of c
// become entries (set << pos_bits) | position, each taking slot
// atomicAdd(&counts[token], 1) of its token's record (tokens below `limit`;
// counts zeroed by the caller).  The slots follow no order.
// bf (optional, a self-join's midprefix index): the low pos_bits of each entry
// hold its bound field (bound_field_of) instead of the position.
cudaError_t emit_records(CollView c, const uint32_t* prefix_tab, uint32_t pos_bits, uint32_t* counts, uint32_t* rec,
                         uint32_t limit, cudaStream_t s, uint32_t lo = 0, uint32_t hi = 0xFFFFFFFFu,
                         BoundFields bf = BoundFields{}, uint32_t big_lo = 0xFFFFFFFFu);
// Pass 2: each record's min(counts[t], REC_ENTRIES) entries in ascending
// order after its length word, padded with 0xFFFFFFFF.  overflow (optional):
// OR-ed with REC_OVERFLOW when a token had more entries than a record holds
// (its record is then incomplete and the index must be built as lists).
// prev (optional): each record's count at the previous pass (0xFFFFFFFF
// before the first); a group of 32 records none of whose counts changed is
// skipped, and prev is brought up to date.  Entries emitted after a pass
// belong to later sets than every entry before it, so a later pass leaves
// the ordered front of each record where it was and only fills padding
// words and the length: a join reading sets below the earlier pass's bound
// may run beside it.
constexpr uint32_t REC_OVERFLOW = 16;
cudaError_t order_records(const uint32_t* counts, uint32_t U, uint32_t* rec, cudaStream_t s,
                          uint32_t* overflow = nullptr, uint32_t* prev = nullptr);
// Records from index lists already built (every list at most REC_ENTRIES long).
// bf (optional): entries (set << list_bits) | position become
// (set << rec_bits) | bound field (sizes: the indexed sets' sizes).
cudaError_t records_from_lists(const uint32_t* list_off, const uint32_t* vals, uint32_t U, uint32_t* rec,
                               cudaStream_t s, BoundFields bf = BoundFields{}, const uint32_t* sizes = nullptr,
                               uint32_t list_bits = 0, uint32_t rec_bits = 0);

// Token histogram of n entries into counts[limit] (warp-aggregated atomics;
// tokens >= limit are skipped; the counts are NOT zeroed here).
cudaError_t token_histogram(const uint32_t* e_token, uint64_t n, uint32_t* counts, uint32_t limit, cudaStream_t s);

// Reference-style scatter (include/hyset/index.hpp:233-248): each entry goes to
// cursor[token]++ (warp-aggregated); list order within a token is arbitrary.
cudaError_t scatter_entries(const uint32_t* e_token, const uint32_t* e_set, const uint32_t* e_pos, uint64_t n,
                            uint32_t* cursor, uint32_t* idx_set, uint32_t* idx_pos, cudaStream_t s);

// After a stable sort by token of entry indices: idx_set[i] = e_set[order[i]], ...
cudaError_t gather_entries(const uint32_t* order, uint64_t n, const uint32_t* e_set, const uint32_t* e_pos,
                           uint32_t* idx_set, uint32_t* idx_pos, cudaStream_t s);

cudaError_t iota_u32(uint32_t* out, uint64_t n, cudaStream_t s);

// Sorts n result pairs in place by (first, second) on the device: two stable
// LSD radix sorts (by second, then by first carrying second), so a result's
// order no longer depends on the order warps appended it.  first < 2^first_bits,
// second < 2^second_bits; a, b, c, d hold n words each, scratch
// radix_scratch_words(n) words.
cudaError_t sort_pair_list(uint2* pairs, uint64_t n, int first_bits, int second_bits, uint32_t* a, uint32_t* b,
                           uint32_t* c, uint32_t* d, uint32_t* scratch, cudaStream_t s);

// Input contract check of an uploaded collection.  flags[0] gets bit 1 for an
// empty set, 2 for a set whose tokens are not strictly ascending, 4 for a size
// smaller than the previous set's, 8 for a set reaching past n_tokens;
// flags[1] gets the largest token (atomicMax).  flags must be zeroed first.
// One pass over the n sizes (and starts: given, or the scan of the sizes) of
// a host-input collection as its copy begins: out[0] gets bit 1 where a size
// is below the one before it and bit 2 where a given start is not where the
// set before it ends (or the first start is not 0); out[2..3] the sum of the
// sizes (u64); first_ge[l] (l in [0, L+1], L the last size) the first set
// with size >= l (meaningful when the sizes are ordered); and
// chunk_hi[k] (filled with 0xFFFFFFFF first) the first set that ends past
// the end of copy chunk k of n_tokens tokens (pipe_chunk), meaningful when
// the sets are contiguous and ordered.  out must be zeroed.
cudaError_t size_scan(const uint32_t* sizes, const uint32_t* starts, bool starts_given, uint32_t n, uint32_t L,
                      uint64_t n_tokens, uint32_t* out, uint32_t* first_ge, uint32_t* chunk_hi, cudaStream_t s);


// The same pass writes meta[i] = (starts[i], sizes[i]).
cudaError_t validate_collection(CollView c, uint64_t n_tokens, uint32_t* flags, uint2* meta, cudaStream_t s);
// validate_collection and generate_bitmaps (words in {1, 2, 4, 8, 16}) in one
// pass over the tokens; min_size (optional): no set of c is shorter (sizes are
// ordered), parts of long sets are read a warp per set.
cudaError_t validate_with_bitmaps(CollView c, uint64_t n_tokens, uint32_t* flags, uint2* meta, int words, uint64_t* out,
                                  cudaStream_t s, uint32_t min_size = 0);

// XOR bitmap signatures, bit (token mod bits) per token
// (include/hyset/device_algorithms.hpp:58-74), words = bits / 64 in {1,2,4,8}.
// max_blocks > 0 caps the grid (signatures generated beside other work leave
// it SMs).
cudaError_t generate_bitmaps(CollView c, int words, uint64_t* out, cudaStream_t s, unsigned max_blocks = 0);

// ---- join.cu --------------------------------------------------------------
struct IndexView {
    const uint32_t* __restrict__ list_off;  // [universe+1]: list t = [list_off[t], list_off[t+1])
    const uint32_t* __restrict__ set;       // entry set ids, or (set << pos_bits) | position when pos == nullptr
    const uint32_t* __restrict__ pos;       // entry positions within their sets (unpacked layout)
    uint32_t universe;
    uint32_t pos_bits;                      // packed layout: bits of the position field
    int sorted;                             // lists ordered by set id
    int rec = 0;                            // token records: list t = set[REC_CAP t, REC_CAP (t + 1)) (see REC_CAP)
    // packed entries carry, in place of the position, the longest probe the
    // entry's side of the positional bound admits (see bound_field)
    int bound = 0;
};

struct JoinParams {
    CollView R;                 // indexed collection
    CollView S;                 // probe collection (== R for a self-join)
    BoundsView B;
    const uint32_t* __restrict__ first_ge;  // [R_L+2] first id of R with size >= l
    uint32_t R_L;               // largest set size in R
    int self;                   // candidates c < p inside one collection
    uint32_t p_lo, p_hi;        // probe ids [p_lo, p_hi)
    uint32_t r_lo, r_hi;        // candidate ids restricted to [r_lo, r_hi)
    IndexView X;                // FGSS only
    IndexView X2;               // R-S FGSS, banded: midprefix index of R (set == nullptr: no bands)
    const uint64_t* __restrict__ bits_R;    // signatures (nullptr = no bitmap filter)
    const uint64_t* __restrict__ bits_S;
    int words;
    Sink out;
    unsigned int* work;         // work-stealing counters, zero before launch ([2] when probes are split)
    uint32_t grab;              // probes taken per steal
    unsigned long long* stats;  // optional [8] counters (nullptr = off)
    // probe-major prefix filter: probes from heavy_from on (the longest
    // prefixes; 0xFFFFFFFF = none) are split into `segs` units of seg_slots
    // prefix slots each, taken one per steal from work[1] before the batches
    uint32_t heavy_from = 0xFFFFFFFFu;
    uint32_t segs = 0, seg_slots = 0;
};

enum Technique : int { TECH_BITMAP = 1, TECH_FGSS = 2, TECH_DIRECT = 3 };

// One persistent, work-stealing launch over probes [p_lo, p_hi).
// vmode: 1 = lane per candidate, 2 = warp per candidate.
cudaError_t launch_join(const JoinParams& P, int technique, int vmode, int sm_count, cudaStream_t s);
// Warps of one launch_join (the blocks per SM its kernels are compiled for).
uint32_t join_resident_warps(int sm_count);

// ---- join_tm.cu ------------------------------------------------------------
// Token groups: for every token, the entries (set, pos | size << 16) of the sets
// whose first pre[size] tokens contain it.  counts must be zeroed; cursor holds
// the groups' start offsets and advances.
cudaError_t group_count(CollView c, const uint32_t* pre, uint32_t* counts, cudaStream_t s);
cudaError_t group_scatter(CollView c, const uint32_t* pre, uint32_t* cursor, uint32_t* gset, uint32_t* gps,
                          cudaStream_t s);

struct TokenJoinParams {
    CollView R, S;
    BoundsView B;
    const uint32_t* __restrict__ gs_off;  // probe groups (S, maxprefix entries), [universe+1]
    const uint32_t* __restrict__ gs_set;
    const uint32_t* __restrict__ gs_ps;
    const uint32_t* __restrict__ gr_off;  // candidate groups (R), [universe+1]
    const uint32_t* __restrict__ gr_set;
    const uint32_t* __restrict__ gr_ps;
    uint32_t universe;
    int self;
    const uint64_t* __restrict__ bits_R;
    const uint64_t* __restrict__ bits_S;
    int words;
    Sink out;
    unsigned int* work;
    uint32_t grab;
    unsigned long long* stats;
};

// One persistent launch; warps steal token groups, largest token ids first.
cudaError_t launch_join_tm(const TokenJoinParams& P, int sm_count, cudaStream_t s);

// ---- batch.cu ----------------------------------------------------------------
// One join of a batch: its parameters plus how its probes split into units.
struct BatchDesc {
    JoinParams P;
    uint32_t tech;         // TECH_FGSS, TECH_BITMAP or TECH_DIRECT
    uint32_t words;        // signature words (0: none)
    uint32_t unit_probes;  // probes per work unit
    uint32_t pad;
};
// unit_off[j] = first unit of join j, unit_off[n_joins] = all units; work zeroed.
cudaError_t launch_batch_join(const BatchDesc* d_desc, const uint32_t* d_unit_off, uint32_t n_joins,
                              unsigned int* d_work, int sm_count, cudaStream_t s);

// ---- stats.cu --------------------------------------------------------------
// out4[0] += sum, [1] += sum of squares, [2] = max, [3] += non-zero count (zero out4 first)
cudaError_t moments_u32(const uint32_t* v, uint64_t n, unsigned long long* out4, cudaStream_t s);

// ---- mlp.cu ----------------------------------------------------------------
constexpr int MLP_IN = 12, MLP_HIDDEN = 64, MLP_OUT = 3;
constexpr int MLP_PARAMS = MLP_IN * MLP_HIDDEN + MLP_HIDDEN + MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN +
                           MLP_HIDDEN * MLP_OUT + MLP_OUT;  // 5187
constexpr int MLP_MAX_BATCH = 128;  // samples held in shared memory at once
constexpr int MLP_THREADS = 256;
size_t mlp_smem_bytes();
// y[n][3] = net(x[n][12])
cudaError_t mlp_forward(const float* w, const float* x, int n, float* y, int sm_count, cudaStream_t s);
// g = dLoss/dw, *loss = Loss over the dataset (t, m: [n][3] targets and 0/1 mask; denom = sum of m)
cudaError_t mlp_grad(const float* w, const float* x, const float* t, const float* m, int n, float denom, float* g,
                     float* loss, cudaStream_t s);
// `steps` Adam steps (w, mom, vel, g: MLP_PARAMS floats each; mom/vel zeroed by the caller)
cudaError_t mlp_train(float* w, float* mom, float* vel, float* g, const float* x, const float* t, const float* m,
                      int n, float denom, int steps, float lr, float weight_decay, float* loss_trace,
                      cudaStream_t s);

// ---- ring.cu ---------------------------------------------------------------
// The candidate ring: records (probe, n, begin) and candidate ids in device
// rings the host fills; see ring.cu.
struct RingRec {
    uint32_t probe;       // probe set id (of S)
    uint32_t n;           // candidates of this record
    unsigned long long begin;  // absolute position of its first candidate (mod cand_cap)
};
enum RingStatus : unsigned int { RING_RUNNING = 0, RING_CLOSED = 1, RING_TIMEOUT = 2 };
struct RingView {
    const unsigned long long* tail;   // records published by the host
    const unsigned long long* close;  // non-zero: stop once the published records are verified
    unsigned long long* claim;        // next record to verify
    unsigned long long* head;         // records verified: a contiguous prefix
    unsigned long long* done;         // [rec_cap] record index + 1 once that record is verified
    unsigned int* status;             // the launch's exit status (RingStatus, atomicMax)
    const RingRec* recs;              // [rec_cap]
    const uint32_t* cands;            // [cand_cap]
    unsigned long long rec_cap, cand_cap;  // powers of two
    unsigned long long wait_ns;       // a warp waits this long for a published record, then gives up
};
// One persistent launch (a block per SM) consuming the ring until close or
// the wait limit; vmode 2 = a warp per candidate, otherwise the staged lane mode.
cudaError_t launch_ring_consumer(CollView R, CollView S, BoundsView B, const RingView& V, int vmode, Sink out,
                                 int sm_count, cudaStream_t s);
// *word = value, ordered on stream s (publishes the ring's tail and close words).
cudaError_t ring_store(unsigned long long* word, unsigned long long value, cudaStream_t s);

// Explicit candidate lists (hybrid::device_handler): probes[i] owns candidates
// [i ? offsets[i-1] : 0, offsets[i]).
// sig_R / sig_S (words per signature, 0 = none): the XOR-signature bound drops
// candidates before any merge (the pairs do not change).
cudaError_t launch_verify_candidates(CollView R, CollView S, BoundsView B, const uint32_t* probes,
                                     const uint32_t* offsets, const uint32_t* cands, uint32_t n_probes,
                                     int vmode, Sink out, unsigned int* work, int sm_count, cudaStream_t s,
                                     const uint64_t* sig_R = nullptr, const uint64_t* sig_S = nullptr,
                                     int words = 0);

}  // namespace hs
