// internal.h — host-side state behind the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/hyset_gb300.h"
#include "kernels.h"

namespace hs {

// Device bytes held by the library's buffers (every DevBuf of every context).
unsigned long long device_bytes();
void add_device_bytes(long long delta);
// Allocation-failure injection for tests: while the environment variable
// HYSET_FAULT_ALLOC holds N, the N-th device allocation attempt counted from
// when that value was first seen fails as cudaErrorMemoryAllocation.
bool inject_alloc_failure();

// Device allocation from the stream-ordered pool; grows, never shrinks.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b, cudaStream_t s) {
        if (b <= bytes && p) return cudaSuccess;
        if (inject_alloc_failure()) return cudaErrorMemoryAllocation;
        if (p) {
            cudaFreeAsync(p, s);
            add_device_bytes(-(long long)bytes);
        }
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMallocAsync(&p, b ? b : 16, s);
        if (e == cudaSuccess) {
            bytes = b ? b : 16;
            add_device_bytes((long long)bytes);
        } else {
            p = nullptr;
        }
        return e;
    }
    void release(cudaStream_t s) {
        if (p) {
            cudaFreeAsync(p, s);
            add_device_bytes(-(long long)bytes);
        }
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

// Host-computed bound tables (exact reference doubles) and their device copy.
struct Bounds {
    int sim = 0;
    double tau = 0;
    uint32_t L = 0;
    int index_maxprefix = 0;  // 0: index midprefix (self-join), 1: maxprefix (R-S)
    std::vector<uint32_t> minsize, probe_prefix, index_prefix, max_partner, mid_prefix, mo_sum, mo_tab, max_sum;
    // cosine (monotone tables): for a set of size l and position p < maxprefix(l),
    // lp_tab[lp_row[l] + p] = the longest probe the entry's side of the
    // positional bound admits (the bound layout of token records)
    std::vector<uint32_t> lp_row, lp_tab;
    bool mo_monotone = false;  // minoverlap non-decreasing in each length (R-S bands are valid)
    std::vector<uint64_t> mo_row;
    DevBuf dev;
    BoundsView view{};
};

#ifndef HS_SIG_BLOCKS_PER_SM
#define HS_SIG_BLOCKS_PER_SM 4  // blocks per SM of signature generation beside an index build (0: no cap)
#endif
#ifndef HS_STREAM_PRIO
#define HS_STREAM_PRIO 1  // the context's stream at the highest priority, the auxiliary stream at the lowest
#endif

struct Index {
    int sim = -1;
    double tau = -1;
    int kind = -1;
    DevBuf list_off, set, pos;
    DevBuf rec;             // token records (REC_CAP words per token) when records is set
    bool records = false;
    uint32_t universe = 0;
    uint64_t entries = 0;
    uint32_t pos_bits = 0;  // > 0: packed (set << pos_bits) | position entries
    // the records' layout: low rec_bits of an entry, the position or (rec_bound)
    // the longest probe the entry's positional bound admits
    uint32_t rec_bits = 0;
    bool rec_bound = false;
    IndexView view() const {
        IndexView v;
        v.list_off = list_off.as<uint32_t>();
        v.set = records ? rec.as<uint32_t>() : set.as<uint32_t>();
        v.pos = pos_bits ? nullptr : pos.as<uint32_t>();
        v.universe = universe;
        v.pos_bits = records ? rec_bits : pos_bits;
        v.sorted = 1;
        v.rec = records ? 1 : 0;
        v.bound = records && rec_bound ? 1 : 0;
        return v;
    }
};

struct Bounds;

// One join of a batch with the buffers it owns (stable across graph replays).
struct BatchJoin {
    hyset_coll* R = nullptr;
    hyset_coll* S = nullptr;
    bool self = false;
    bool swapped = false;  // R-S join run with the roles exchanged (R, S are the kernel's roles)
    hyset_join_opts o{};
    Bounds* b = nullptr;
    Index ix, ix_mid;
    DevBuf bits_r, bits_s, pairs;
    uint64_t cap = 0;
    int words = 0;
    int ktech = 0;
    hyset_technique tech = HYSET_TECH_AUTO;
    uint32_t units = 0;
    uint32_t unit_probes = 0;  // probes per work unit of the prefix-index kernel (0: window technique)
    // a heavy prefix-index join runs as a launch of its own inside the batch's
    // graph (the single-join kernel: token records, carried items), not in the
    // shared launch
    bool solo = false;
    int vmode = 1;
    uint32_t batch = 3;
};

// Scratch of an index build (prefix lengths and offsets, entries, radix sort
// ping-pong buffers, token counts, scan/sort scratch).
struct Scratch {
    DevBuf len, off, tok, set, pos, order, altk, altv, counts, scan, gate, sscan;
    void release(cudaStream_t s) {
        DevBuf* all[] = {&len, &off, &tok, &set, &pos, &order, &altk, &altv, &counts, &scan, &gate, &sscan};
        for (DevBuf* d : all) d->release(s);
    }
};

// A captured batch: signature (collections and options), per-join buffers,
// device descriptors, and the instantiated graph of its device work.
struct BatchPlan {
    std::vector<std::string> sig;
    Scratch sc;  // owned by the plan: its graph holds these addresses
    std::vector<std::unique_ptr<BatchJoin>> joins;
    std::vector<uint32_t> order;  // joins[order[k]] is descriptor k (heaviest first)
    DevBuf desc, unit_off, counts, work;
    std::vector<BatchDesc> host_desc;  // the joins' descriptors in launch order (solo joins launch from them)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

}  // namespace hs

struct hyset_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ek0 = nullptr, ek1 = nullptr;
    cudaStream_t aux = nullptr;                         // work that overlaps the index build
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;  // fork to / join from aux
    std::vector<cudaEvent_t> pipe_ev;                   // one per copy chunk of a host-input join
    std::string err;
    std::map<std::tuple<int, double, uint32_t, int>, std::unique_ptr<hs::Bounds>> bounds;
    // scratch reused across joins; a batch being prepared points sc at its own
    hs::Scratch own;
    hs::Scratch* sc = &own;
    hs::DevBuf s_pairs, s_count, s_work, s_stats, s_flags;
    uint32_t* h_flags = nullptr;  // pinned host words for small device-to-host reads
    void* h_stage = nullptr;      // pinned staging for larger reads (grows)
    size_t h_stage_bytes = 0;
    std::unique_ptr<hs::BatchPlan> batch;
    // technique selector: learned network and/or analytic cost model
    bool has_mlp = false, has_cost = false;
    std::vector<float> mlp_params;            // MLP_PARAMS
    float feat_mean[hs::MLP_IN] = {}, feat_scale[hs::MLP_IN] = {};
    double cost[3][9] = {};                   // per technique (bitmap, fgss, direct)
    hs::DevBuf d_mlp, d_feat, d_moments, d_hist;
    // learned signature width (a second network of the same shape: log-time at 128, 256, 512 bits)
    bool has_width_mlp = false;
    float width_mean[hs::MLP_IN] = {}, width_scale[hs::MLP_IN] = {};
    hs::DevBuf d_width_mlp;
    std::map<std::string, std::pair<hyset_technique, int>> select_cache;  // decision, selector
    struct TuneChoice {
        uint32_t bits = 0;   // signature width
        int vmode = 0;       // verification mode (0: not tuned)
        uint32_t batch = 0;  // probes per warp batch of the probe-major kernel (0: not tuned)
        float est_ms = 0;    // the join kernel's estimated time in this configuration
    };
    std::map<std::string, TuneChoice> tune_cache;  // the autotuner's choices per join
    std::map<std::string, uint32_t> universe_cache;  // universe by collection size profile (host-input joins)
    std::map<std::string, uint32_t> longest_cache;   // longest index list by join key (host-input joins)
    struct SplitPlan {
        uint32_t at;  // first probe id of the high range; 0 = no split
        hyset_technique low, high;
    };
    std::map<std::string, SplitPlan> split_cache;  // partition plans of AUTO self-joins
};

struct hyset_coll {
    hyset_ctx* ctx = nullptr;
    hs::DevBuf tokens, starts, sizes, meta;
    const uint32_t* d_tokens = nullptr;  // may point at caller memory (from_device)
    const uint32_t* d_starts = nullptr;
    const uint32_t* d_sizes = nullptr;
    uint32_t n = 0;
    uint64_t n_tokens = 0;
    uint32_t max_size = 0;
    uint32_t universe = 0;  // max token + 1
    std::vector<uint64_t> size_hist;  // sets per size, [max_size+1]
    hs::DevBuf first_ge;              // [max_size+2] first id with size >= l
    std::vector<uint32_t> h_first_ge; // host copy (source of the device copy)
    hs::Index index;
    hs::Index index_mid;  // R-S bands: midprefix entries, same layout as index
    hs::DevBuf g_off, g_set, g_ps, g_cursor;  // token groups of the prefix entries (token-major join)
    std::map<int, hs::DevBuf> bitmaps;  // by words
    std::map<const uint32_t*, int> list_path;  // per prefix table: index lists built short (1) or by radix (2)
    std::map<const uint32_t*, uint32_t> list_longest;  // per prefix table: the longest index list, once read back
    hs::CollView view() const { return hs::CollView{d_tokens, d_starts, d_sizes, meta.as<uint2>(), n}; }
};

struct hyset_result {
    uint64_t count = 0;
    std::vector<hyset_pair> pairs;
    int has_pairs = 0;
    const void* device_pairs = nullptr;
    hyset_technique technique = HYSET_TECH_AUTO;
    uint32_t bitmap_bits = 0;  // signature width the join ran with
    uint32_t verify_mode = 0;  // verification mode the join ran with
    uint32_t probe_batch = 0;  // probes per warp batch of the probe-major kernel (0: not that kernel)
    uint32_t split_at = 0;     // partition split: first probe id of the high range (0 = none)
    hyset_technique split_low = HYSET_TECH_AUTO;  // the low range's technique
    double device_ms = 0;
    double kernel_ms = 0;
    uint64_t stats[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint64_t launches = 0;
    int selector = -1;  // -1 explicit technique, 0 rules, 1 analytic cost model, 2 learned network
};

struct hyset_handler {
    hyset_ctx* ctx = nullptr;
    const hyset_coll* coll = nullptr;
    hyset_technique technique = HYSET_TECH_FGSS;
    hyset_sim sim = HYSET_JACCARD;
    double tau = 0;
    uint32_t block_size = 0;
    int aggregate = 0;
    int words = 0;
    hs::Bounds* bounds = nullptr;
    // per-indexed-block inverted index (reference layout: unsorted lists)
    hs::DevBuf counts, list_off, e_len, e_off, e_tok, e_set, e_pos, idx_set, idx_pos, scan;
    uint32_t indexed_block = 0xFFFFFFFFu;
    hs::DevBuf bits, pairs, count, work;
    uint64_t cap = 0;
    uint64_t out_count = 0;
    std::vector<hyset_pair> out_pairs;
};

struct hyset_verifier {
    hyset_ctx* ctx = nullptr;
    const hyset_coll* indexed = nullptr;
    const hyset_coll* probe = nullptr;
    hs::Bounds* bounds = nullptr;
    uint32_t scenario = 1;
    int aggregate = 0;
    uint32_t max_probes = 0, max_candidates = 0;
    // the candidate ring (ring.cu): records and candidate ids in device rings,
    // staged in pinned host rings of the same layout
    uint64_t rec_cap = 0, cand_cap = 0, pair_cap = 0;
    hs::DevBuf d_recs, d_cands, d_done, d_ctl, pairs;
    hs::RingRec* h_recs = nullptr;
    uint32_t* h_cands = nullptr;
    unsigned long long* h_ctl = nullptr;  // pinned read-back of the control words
    uint64_t pushed = 0, published = 0;   // records staged / published (absolute counts)
    uint64_t cand_pushed = 0, cand_published = 0;
    uint64_t head = 0;       // records verified, as last read back
    uint64_t undrained = 0;  // candidates published since the pairs were last drained
    uint64_t wait_ns = 0;    // the consumer's wait limit for published records
    cudaStream_t pub = nullptr, cons = nullptr;  // publication copies / the persistent consumer
    cudaEvent_t ev_pub = nullptr, ev_cons = nullptr;
    bool consumer_live = false;
    unsigned int last_status = 0;  // exit status of the last consumer launch that ended
    uint64_t out_count = 0;
    std::vector<hyset_pair> out_pairs;
};
