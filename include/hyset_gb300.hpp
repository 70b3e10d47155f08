/* hyset_gb300.hpp — header-only C++ adapter over the C ABI with the shapes of
 * the reference's join-driver classes, so a driver's call sites change their
 * namespace and little else:
 *
 *   reference (include/hyset/...)                     here
 *   collection::host_collection / read_collection     hyset_gb300::host_collection / read_collection
 *   collection::device_collection                     hyset_gb300::device_collection
 *   output::handler, count_handler, pairs_handler     hyset_gb300::output::... (same members)
 *   bitmap::handler, fgssjoin::handler                hyset_gb300::bitmap::handler, fgssjoin::handler
 *   hybrid::device_handler                            hyset_gb300::hybrid::device_handler
 *
 * Constructor arguments follow device_algorithms.hpp:138-141 / :322-324 and
 * hybrid_algorithms.hpp:41-62 without the timer argument.  Errors throw
 * hyset_gb300::error (the reference's cuda-api-wrappers throw too).  Every
 * call goes through include/hyset_gb300.h; nothing here touches CUDA. */
#ifndef HYSET_GB300_HPP
#define HYSET_GB300_HPP

#include <algorithm>
#include <cstdint>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "hyset_gb300.h"

namespace hyset_gb300 {

struct error : std::runtime_error {
    hyset_status status;
    error(hyset_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(hyset_status s, const hyset_ctx* ctx) {
    if (s != HYSET_OK) throw error(s, ctx ? hyset_last_error(ctx) : "hyset_gb300: call failed");
}

// One GPU context (stream, scratch, selector); one per host thread.
class context {
  public:
    explicit context(int device = 0) { check(hyset_create(device, &h_), nullptr); }
    ~context() { hyset_destroy(h_); }
    context(const context&) = delete;
    context& operator=(const context&) = delete;
    hyset_ctx* get() const { return h_; }

  private:
    hyset_ctx* h_ = nullptr;
};

// collection::host_collection: CSR arrays of size-sorted sets.
struct host_collection {
    std::vector<uint32_t> tokens, starts, sizes;
    uint32_t universeSize = 0;
};

// collection::read_collection's parsing (collection.hpp:93-177): one set per
// line, tokens split by single spaces, empty lines skipped.
inline host_collection read_collection(const std::string& filename) {
    std::ifstream in(filename);
    if (!in) throw error(HYSET_E_INVALID, "file not found: " + filename);
    host_collection c;
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty()) continue;
        std::istringstream ss(line);
        std::string item;
        uint32_t n = 0;
        c.starts.push_back((uint32_t)c.tokens.size());
        while (std::getline(ss, item, ' ')) {
            c.tokens.push_back((uint32_t)std::stoul(item));
            ++n;
        }
        c.sizes.push_back(n);
        if (n && c.tokens.back() + 1 > c.universeSize) c.universeSize = c.tokens.back() + 1;
    }
    return c;
}

// collection::device_collection: the collection resident on the device.
class device_collection {
  public:
    device_collection(context& ctx, const host_collection& c) : ctx_(ctx.get()) {
        check(hyset_collection_upload(ctx_, c.tokens.data(), c.tokens.size(), c.starts.data(), c.sizes.data(),
                                      (uint32_t)c.sizes.size(), &h_),
              ctx_);
    }
    // The reference's text format parsed on the GPU (hyset_collection_parse).
    device_collection(context& ctx, const std::string& text) : ctx_(ctx.get()) {
        check(hyset_collection_parse(ctx_, text.data(), text.size(), &h_), ctx_);
    }
    ~device_collection() { hyset_collection_free(ctx_, h_); }
    device_collection(const device_collection&) = delete;
    device_collection& operator=(const device_collection&) = delete;
    const hyset_coll* get() const { return h_; }
    uint32_t size() const { return hyset_collection_num_sets(h_); }

  private:
    hyset_ctx* ctx_;
    hyset_coll* h_ = nullptr;
};

namespace output {
// output::handler and its two implementations (output.hpp:13-37).
struct handler {
    virtual ~handler() = default;
    virtual void addPair(const unsigned int& rec1, const unsigned int& rec2) = 0;
    virtual unsigned long getCount() const = 0;
};
struct count_handler : handler {
    unsigned long count = 0;
    void addPair(const unsigned int&, const unsigned int&) override { ++count; }
    unsigned long getCount() const override { return count; }
};
struct pairs_handler : handler {
    std::vector<hyset_pair> pairs;
    void addPair(const unsigned int& rec1, const unsigned int& rec2) override { pairs.push_back({rec1, rec2}); }
    const std::vector<hyset_pair>& getPairs() const { return pairs; }
    unsigned long getCount() const override { return (unsigned long)pairs.size(); }
};
}  // namespace output

using block = hyset_block;  // structs::block, same field order

// The blocks read_collection cuts (collection.hpp:147-171): block_size
// consecutive sets each.  The handlers read id, start_id and end_id; the
// prefix bookkeeping fields are left 0 (the library derives what it needs).
inline std::vector<block> make_blocks(const host_collection& c, uint32_t block_size) {
    std::vector<block> out;
    const uint32_t n = (uint32_t)c.sizes.size();
    for (uint32_t lo = 0; lo < n; lo += block_size) {
        block b{};
        b.id = (uint32_t)out.size();
        b.start_id = lo;
        b.end_id = std::min(n, lo + block_size) - 1;
        for (uint32_t i = b.start_id; i <= b.end_id; ++i) b.num_tokens += c.sizes[i];
        b.size = b.end_id - b.start_id + 1;
        out.push_back(b);
    }
    return out;
}

namespace detail {
// bitmap::handler / fgssjoin::handler: joins of blocks or of partitions (lists
// of blocks); the pairs (or the count) of each call go to the output handler.
class block_handler {
  public:
    block_handler(context& ctx, device_collection& coll, hyset_technique tech, uint32_t bitmap_size,
                  uint32_t block_size, bool aggregate, double threshold, hyset_sim sim)
        : ctx_(ctx.get()), aggregate_(aggregate) {
        check(hyset_handler_create(ctx_, coll.get(), tech, sim, bitmap_size, block_size, aggregate ? 1 : 0,
                                   threshold, &h_),
              ctx_);
    }
    ~block_handler() { hyset_handler_destroy(h_); }
    block_handler(const block_handler&) = delete;
    block_handler& operator=(const block_handler&) = delete;
    void setOutputHandler(std::shared_ptr<output::handler> out) { out_ = std::move(out); }
    void join(const block* first, const block* second) {
        check(hyset_handler_join_blocks(h_, first, second), ctx_);
        drain();
    }
    void join(const std::vector<block>& first, const std::vector<block>& second) {
        check(hyset_handler_join_partitions(h_, first.data(), (uint32_t)first.size(), second.data(),
                                            (uint32_t)second.size()),
              ctx_);
        drain();
    }

  private:
    void drain() {
        uint64_t n = 0;
        const hyset_pair* pairs = nullptr;
        check(hyset_handler_output(h_, &n, &pairs), ctx_);
        if (out_) {
            if (auto* c = dynamic_cast<output::count_handler*>(out_.get()); c && (aggregate_ || !pairs)) {
                c->count += n;
            } else {
                for (uint64_t i = 0; i < n && pairs; ++i) out_->addPair(pairs[i].first, pairs[i].second);
            }
        }
        check(hyset_handler_clear_output(h_), ctx_);
    }
    hyset_ctx* ctx_;
    hyset_handler* h_ = nullptr;
    bool aggregate_;
    std::shared_ptr<output::handler> out_;
};
}  // namespace detail

namespace bitmap {
// bitmap::handler(timer, hostCollection, deviceCollection, bitmap, blockSize, aggregate, threshold)
class handler : public detail::block_handler {
  public:
    handler(context& ctx, device_collection& coll, uint32_t bitmap_size, uint32_t block_size, bool aggregate,
            double threshold, hyset_sim sim = HYSET_JACCARD)
        : block_handler(ctx, coll, HYSET_TECH_BITMAP, bitmap_size, block_size, aggregate, threshold, sim) {}
};
}  // namespace bitmap

namespace fgssjoin {
// fgssjoin::handler(timer, hostCollection, deviceCollection, blockSize, aggregate, threshold)
class handler : public detail::block_handler {
  public:
    handler(context& ctx, device_collection& coll, uint32_t block_size, bool aggregate, double threshold,
            hyset_sim sim = HYSET_JACCARD)
        : block_handler(ctx, coll, HYSET_TECH_FGSS, 0, block_size, aggregate, threshold, sim) {}
};
}  // namespace fgssjoin

namespace hybrid {
// hybrid::device_handler(idx, probe, threads, scenario, aggregate, maxProbes, maxCandidates, threshold)
class device_handler {
  public:
    device_handler(context& ctx, device_collection& indexed, device_collection& probe, uint32_t threads,
                   uint32_t scenario, bool aggregate, uint32_t max_probes, uint32_t max_candidates,
                   double threshold, hyset_sim sim = HYSET_JACCARD)
        : ctx_(ctx.get()) {
        check(hyset_verifier_create(ctx_, indexed.get(), probe.get(), sim, threads, scenario, aggregate ? 1 : 0,
                                    max_probes, max_candidates, threshold, &h_),
              ctx_);
    }
    ~device_handler() { hyset_verifier_destroy(h_); }
    device_handler(const device_handler&) = delete;
    device_handler& operator=(const device_handler&) = delete;
    void setOutputHandler(std::shared_ptr<output::handler> out) { out_ = std::move(out); }
    void addCandidates(uint32_t probe_id, const std::vector<uint32_t>& candidates) {
        check(hyset_verifier_add_candidates(h_, probe_id, candidates.data(), (uint32_t)candidates.size()), ctx_);
    }
    void flush() {
        check(hyset_verifier_flush(h_), ctx_);
        uint64_t n = 0;
        const hyset_pair* pairs = nullptr;
        check(hyset_verifier_output(h_, &n, &pairs), ctx_);
        if (!out_) return;
        for (uint64_t i = delivered_; i < n && pairs; ++i) out_->addPair(pairs[i].first, pairs[i].second);
        if (!pairs)
            if (auto* c = dynamic_cast<output::count_handler*>(out_.get())) c->count += n - delivered_;
        delivered_ = n;
    }

  private:
    hyset_ctx* ctx_;
    hyset_verifier* h_ = nullptr;
    std::shared_ptr<output::handler> out_;
    uint64_t delivered_ = 0;
};
}  // namespace hybrid

// A whole self-join (the fast path): technique AUTO unless opts say otherwise.
inline std::vector<hyset_pair> self_join(context& ctx, device_collection& coll, double threshold,
                                         hyset_sim sim = HYSET_JACCARD, hyset_join_opts* opts_in = nullptr) {
    hyset_join_opts o;
    hyset_default_opts(&o);
    if (opts_in) o = *opts_in;
    o.sim = sim;
    o.threshold = threshold;
    hyset_result* r = nullptr;
    check(hyset_self_join(ctx.get(), coll.get(), &o, &r), ctx.get());
    std::vector<hyset_pair> out;
    if (const hyset_pair* p = hyset_result_pairs(r)) out.assign(p, p + hyset_result_count(r));
    hyset_result_free(r);
    return out;
}

}  // namespace hyset_gb300

#endif
