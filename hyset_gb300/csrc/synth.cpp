// Seeded synthetic set collections (host C++).  See include/hyset_gb300_synth.h.
//
// Output follows the reference's input contract (include/hyset/collection.hpp:93-177):
// every set sorted ascending, the collection sorted by set size, tokens >= 1
// (the reference indexes offsets[token - 1], include/hyset/index.hpp:111-124, so a
// zero token is undefined there).  Tokens are renumbered by ascending global
// frequency so that a set's prefix holds its rarest tokens.
//
// Determinism: every set draws from its own counter-based stream (splitmix64 of
// seed and set index), so the result does not depend on the thread count.

#include "../../include/hyset_gb300_synth.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {  // splitmix64
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    uint32_t below(uint32_t n) { return (uint32_t)(((next() >> 32) * (uint64_t)n) >> 32); }
};

uint64_t stream_seed(uint64_t seed, uint64_t index, uint64_t stream) {
    Rng r(seed ^ (0xA0761D6478BD642Full * (index + 1)) ^ (0xE7037ED1A0B428DBull * (stream + 1)));
    r.next();
    return r.next();
}

// Vose alias table over ranks 1..U with P(k) proportional to k^-s.
struct Alias {
    std::vector<double> prob;
    std::vector<uint32_t> alias;
    uint32_t n = 0;
    void build(uint32_t U, double s) {
        n = U;
        prob.assign(U, 0.0);
        alias.assign(U, 0);
        std::vector<double> w(U);
        double total = 0.0;
        for (uint32_t k = 0; k < U; ++k) { w[k] = std::pow((double)(k + 1), -s); total += w[k]; }
        std::vector<uint32_t> small, large;
        for (uint32_t k = 0; k < U; ++k) {
            w[k] = w[k] * (double)U / total;
            if (w[k] < 1.0) small.push_back(k); else large.push_back(k);
        }
        while (!small.empty() && !large.empty()) {
            uint32_t a = small.back(); small.pop_back();
            uint32_t b = large.back();
            prob[a] = w[a];
            alias[a] = b;
            w[b] = (w[b] + w[a]) - 1.0;
            if (w[b] < 1.0) { large.pop_back(); small.push_back(b); }
        }
        for (uint32_t k : large) { prob[k] = 1.0; alias[k] = k; }
        for (uint32_t k : small) { prob[k] = 1.0; alias[k] = k; }
    }
    uint32_t draw(Rng& r) const {  // returns a rank in 1..U
        uint32_t col = r.below(n);
        return (r.uniform() < prob[col] ? col : alias[col]) + 1;
    }
};

// Draws `size` distinct ranks (sampling without replacement by rejection):
// the result is the set of distinct values in the draw sequence up to the
// first point where `size` distinct values have been seen.
void draw_set(const Alias& z, Rng& r, uint32_t size, std::vector<uint32_t>& out) {
    out.clear();
    while (out.size() < size) {
        size_t need = size - out.size();
        for (size_t k = 0; k < need; ++k) out.push_back(z.draw(r));
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
    }
}

template <typename F>
void parallel_for(uint32_t n, int threads, F f) {
    if (threads <= 1 || n < 1024) { f(0u, n); return; }
    std::vector<std::thread> pool;
    uint32_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        uint32_t lo = std::min(n, chunk * (uint32_t)t), hi = std::min(n, lo + chunk);
        if (lo < hi) pool.emplace_back([=] { f(lo, hi); });
    }
    for (auto& th : pool) th.join();
}

}  // namespace

struct hyset_synth {
    std::vector<uint32_t> tokens, sizes, starts;
    uint32_t max_token = 0;
};

extern "C" int hyset_synth_generate(const hyset_synth_params* p, hyset_synth** out) {
    if (!p || !out || p->n_sets == 0 || p->universe == 0 || p->size_min == 0 ||
        p->size_min > p->size_max || p->size_max > p->universe || p->zipf_s < 0.0)
        return 1;
    int threads = p->threads > 0 ? p->threads : (int)std::max(1u, std::thread::hardware_concurrency());
    const uint32_t n = p->n_sets;

    Alias zipf;
    zipf.build(p->universe, p->zipf_s);

    // 1. sizes and duplicate roles
    std::vector<uint32_t> size(n), dup_src(n, UINT32_MAX);
    std::vector<double> dup_edit(n, 0.0);
    for (uint32_t i = 0; i < n; ++i) {
        Rng r(stream_seed(p->seed, i, 0));
        double v;
        if (p->size_dist == HYSET_SIZES_LOGNORMAL) {
            double u1 = r.uniform(), u2 = r.uniform();
            if (u1 < 1e-300) u1 = 1e-300;
            double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
            v = std::exp(p->size_a + p->size_b * z);
        } else {
            v = p->size_a + (p->size_b - p->size_a + 1.0) * r.uniform();
            v = std::floor(v);
        }
        long s = std::lround(v);
        if (s < (long)p->size_min) s = p->size_min;
        if (s > (long)p->size_max) s = p->size_max;
        size[i] = (uint32_t)s;
        if (p->dup_frac > 0.0 && i > 0 && r.uniform() < p->dup_frac) {
            dup_src[i] = r.below(i);
            dup_edit[i] = p->dup_edit_lo + (p->dup_edit_hi - p->dup_edit_lo) * r.uniform();
        }
    }
    // A duplicate copies the size of its (transitively resolved) base set.
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t s = dup_src[i];
        while (s != UINT32_MAX && dup_src[s] != UINT32_MAX) s = dup_src[s];
        dup_src[i] = s;
        if (s != UINT32_MAX) size[i] = size[s];
    }

    std::vector<uint64_t> off(n + 1, 0);
    for (uint32_t i = 0; i < n; ++i) off[i + 1] = off[i] + size[i];
    if (off[n] >= (1ull << 32)) return 1;
    std::vector<uint32_t> raw(off[n]);

    // 2. base sets
    parallel_for(n, threads, [&](uint32_t lo, uint32_t hi) {
        std::vector<uint32_t> buf;
        for (uint32_t i = lo; i < hi; ++i) {
            if (dup_src[i] != UINT32_MAX) continue;
            Rng r(stream_seed(p->seed, i, 1));
            draw_set(zipf, r, size[i], buf);
            std::copy(buf.begin(), buf.end(), raw.begin() + off[i]);
        }
    });
    // 3. near-duplicates: copy the base set and replace a fraction of its tokens
    parallel_for(n, threads, [&](uint32_t lo, uint32_t hi) {
        std::vector<uint32_t> buf;
        for (uint32_t i = lo; i < hi; ++i) {
            uint32_t s = dup_src[i];
            if (s == UINT32_MAX) continue;
            Rng r(stream_seed(p->seed, i, 2));
            buf.assign(raw.begin() + off[s], raw.begin() + off[s] + size[s]);
            uint32_t edits = (uint32_t)std::lround(dup_edit[i] * (double)size[i]);
            if (edits > size[i]) edits = size[i];
            for (uint32_t e = 0; e < edits; ++e) buf.erase(buf.begin() + r.below((uint32_t)buf.size()));
            uint32_t guard = 0;
            while (buf.size() < size[i] && guard < 1000000u) {
                uint32_t t = zipf.draw(r);
                auto it = std::lower_bound(buf.begin(), buf.end(), t);
                if (it == buf.end() || *it != t) buf.insert(it, t);
                ++guard;
            }
            for (uint32_t t = 1; buf.size() < size[i]; ++t) {  // tiny universes only
                auto it = std::lower_bound(buf.begin(), buf.end(), t);
                if (it == buf.end() || *it != t) buf.insert(it, t);
            }
            std::copy(buf.begin(), buf.end(), raw.begin() + off[i]);
        }
    });

    // 4. renumber by ascending global frequency (ties by raw rank), ids start at 1
    std::vector<uint64_t> freq(p->universe + 1, 0);
    for (uint64_t k = 0; k < off[n]; ++k) freq[raw[k]]++;
    std::vector<uint32_t> order;
    order.reserve(p->universe);
    for (uint32_t t = 1; t <= p->universe; ++t) if (freq[t]) order.push_back(t);
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return freq[a] < freq[b]; });
    std::vector<uint32_t> newid(p->universe + 1, 0);
    for (uint32_t k = 0; k < order.size(); ++k) newid[order[k]] = k + 1;
    parallel_for(n, threads, [&](uint32_t lo, uint32_t hi) {
        for (uint32_t i = lo; i < hi; ++i) {
            for (uint64_t k = off[i]; k < off[i + 1]; ++k) raw[k] = newid[raw[k]];
            std::sort(raw.begin() + off[i], raw.begin() + off[i + 1]);
        }
    });

    // 5. sort the collection by (size, tokens)
    std::vector<uint32_t> perm(n);
    for (uint32_t i = 0; i < n; ++i) perm[i] = i;
    std::sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) {
        if (size[a] != size[b]) return size[a] < size[b];
        for (uint32_t k = 0; k < size[a]; ++k) {
            uint32_t x = raw[off[a] + k], y = raw[off[b] + k];
            if (x != y) return x < y;
        }
        return a < b;
    });

    hyset_synth* h = new (std::nothrow) hyset_synth();
    if (!h) return 1;
    h->tokens.resize(off[n]);
    h->sizes.resize(n);
    h->starts.resize(n);
    uint64_t pos = 0;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t src = perm[i];
        h->sizes[i] = size[src];
        h->starts[i] = (uint32_t)pos;
        std::copy(raw.begin() + off[src], raw.begin() + off[src + 1], h->tokens.begin() + pos);
        pos += size[src];
    }
    h->max_token = (uint32_t)order.size();
    *out = h;
    return 0;
}

extern "C" uint32_t hyset_synth_num_sets(const hyset_synth* s) { return (uint32_t)s->sizes.size(); }
extern "C" uint64_t hyset_synth_num_tokens(const hyset_synth* s) { return s->tokens.size(); }
extern "C" uint32_t hyset_synth_max_token(const hyset_synth* s) { return s->max_token; }
extern "C" const uint32_t* hyset_synth_tokens(const hyset_synth* s) { return s->tokens.data(); }
extern "C" const uint32_t* hyset_synth_sizes(const hyset_synth* s) { return s->sizes.data(); }
extern "C" const uint32_t* hyset_synth_starts(const hyset_synth* s) { return s->starts.data(); }

extern "C" int hyset_synth_write_text(const hyset_synth* s, const char* path) {
    FILE* f = std::fopen(path, "w");
    if (!f) return 1;
    std::vector<char> line;
    for (size_t i = 0; i < s->sizes.size(); ++i) {
        const uint32_t* t = s->tokens.data() + s->starts[i];
        for (uint32_t k = 0; k < s->sizes[i]; ++k) std::fprintf(f, k ? " %u" : "%u", t[k]);
        std::fputc('\n', f);
    }
    return std::fclose(f) == 0 ? 0 : 1;
}

namespace {
inline uint32_t decimal_digits(uint32_t v) {
    uint32_t d = 1;
    while (v >= 10) {
        v /= 10;
        ++d;
    }
    return d;
}
}  // namespace

extern "C" uint64_t hyset_format_text(const uint32_t* tokens, const uint32_t* starts, const uint32_t* sizes,
                                      uint32_t n_sets, char* buf, uint64_t cap) {
    uint64_t total = 0;
    for (uint32_t i = 0; i < n_sets; ++i) {
        for (uint32_t k = 0; k < sizes[i]; ++k) total += decimal_digits(tokens[(uint64_t)starts[i] + k]) + 1;
        if (!sizes[i]) total += 1;
    }
    if (!buf || cap < total) return total;
    char* o = buf;
    for (uint32_t i = 0; i < n_sets; ++i) {
        for (uint32_t k = 0; k < sizes[i]; ++k) {
            uint32_t v = tokens[(uint64_t)starts[i] + k];
            const uint32_t d = decimal_digits(v);
            for (uint32_t j = d; j-- > 0;) {
                o[j] = (char)('0' + v % 10);
                v /= 10;
            }
            o += d;
            *o++ = k + 1 < sizes[i] ? ' ' : '\n';
        }
        if (!sizes[i]) *o++ = '\n';
    }
    return total;
}

extern "C" void hyset_synth_free(hyset_synth* s) { delete s; }
