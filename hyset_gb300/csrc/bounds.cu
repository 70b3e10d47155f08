// bounds.cu — the similarity bound tables the kernels look up.  The
// reference's bounds (include/hyset/similarity.hpp:11-54) are computed on the
// host in the same double expressions; this translation unit is compiled
// without multiply-add contraction so the doubles match the reference bit for
// bit.  Cosine and dice have no reference code and follow the same style.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "host.h"

namespace hs {

namespace {
int imin(int a, int b) { return (a > b) ? b : a; }
}  // namespace

uint32_t sim_minoverlap(int sim, uint32_t l1, uint32_t l2, double t) {
    switch (sim) {
    case SIM_COSINE: return (uint32_t)(std::ceil(t * std::sqrt((double)l1 * (double)l2)));
    case SIM_DICE: return (uint32_t)(std::ceil(t * (double)(l1 + l2) / 2.0));
    default: return (uint32_t)(std::ceil((double)(l1 + l2) * t / (1 + t)));
    }
}
uint32_t minsize_of(int sim, uint32_t len, double t) {
    switch (sim) {
    case SIM_COSINE: return (uint32_t)(std::ceil(t * t * (double)len));
    case SIM_DICE: return (uint32_t)(std::ceil(t * (double)len / (2.0 - t)));
    default: return (uint32_t)(std::ceil(t * (double)len));
    }
}
uint32_t minoverlap_of(int sim, uint32_t l1, uint32_t l2, double t) {
    return (uint32_t)imin((int)l2, imin((int)l1, (int)sim_minoverlap(sim, l1, l2, t)));
}
uint32_t maxprefix_of(int sim, uint32_t len, double t) {
    return (uint32_t)imin((int)len, (int)(len - minsize_of(sim, len, t) + 1));
}
uint32_t midprefix_of(int sim, uint32_t len, double t) {
    return (uint32_t)imin((int)len, (int)(len - minoverlap_of(sim, len, len, t) + 1));
}

namespace {
constexpr uint64_t MAX_COSINE_TABLE = 64ull << 20;  // entries
}  // namespace

hyset_status get_bounds(hyset_ctx* ctx, int sim, double tau, uint32_t L, int index_maxprefix, Bounds** out) {
    auto key = std::make_tuple(sim, tau, L, index_maxprefix);
    auto it = ctx->bounds.find(key);
    if (it != ctx->bounds.end()) {
        *out = it->second.get();
        return HYSET_OK;
    }
    auto b = std::make_unique<Bounds>();
    auto guard = on_exit([&] {  // tables that failed to upload give their memory back
        if (b) b->dev.release(ctx->stream);
    });
    b->sim = sim;
    b->tau = tau;
    b->L = L;
    b->index_maxprefix = index_maxprefix;
    b->minsize.resize(L + 1);
    b->probe_prefix.resize(L + 1);
    b->index_prefix.resize(L + 1);
    b->max_partner.resize(L + 1);
    b->mid_prefix.resize(L + 1);
    for (uint32_t l = 0; l <= L; ++l) {
        b->minsize[l] = minsize_of(sim, l, tau);
        b->probe_prefix[l] = l ? maxprefix_of(sim, l, tau) : 0;
        b->mid_prefix[l] = l ? midprefix_of(sim, l, tau) : 0;
        b->index_prefix[l] = l ? (index_maxprefix ? b->probe_prefix[l] : b->mid_prefix[l]) : 0;
        if (b->minsize[l] > l) return fail(ctx, HYSET_E_INVALID, "threshold yields minsize > set size");
    }
    uint32_t q = 0;
    for (uint32_t l = 0; l <= L; ++l) {
        while (q + 1 <= L && b->minsize[q + 1] <= l) ++q;
        b->max_partner[l] = q;
    }
    if (sim == SIM_COSINE) {
        b->mo_row.resize((size_t)L + 2);
        uint64_t run = 0;
        for (uint32_t big = 0; big <= L; ++big) {
            b->mo_row[big] = run;
            run += (uint64_t)(big - b->minsize[big] + 1);
        }
        b->mo_row[L + 1] = run;
        if (run > MAX_COSINE_TABLE)
            return fail(ctx, HYSET_E_UNSUPPORTED, "cosine bound table too large for the longest set");
        b->mo_tab.resize(run);
        for (uint32_t big = 0; big <= L; ++big)
            for (uint32_t small = b->minsize[big]; small <= big; ++small)
                b->mo_tab[b->mo_row[big] + (small - b->minsize[big])] = sim_minoverlap(sim, big, small, tau);
        b->mo_sum.assign(1, 0);
        // non-decreasing along rows (small) and along columns (big)
        b->mo_monotone = true;
        for (uint32_t big = 1; big <= L && b->mo_monotone; ++big)
            for (uint32_t small = b->minsize[big]; small <= big; ++small) {
                const uint32_t v = b->mo_tab[b->mo_row[big] + (small - b->minsize[big])];
                if (small > b->minsize[big] && b->mo_tab[b->mo_row[big] + (small - 1 - b->minsize[big])] > v)
                    b->mo_monotone = false;
                if (big > 1 && small >= b->minsize[big - 1] && small <= big - 1 &&
                    b->mo_tab[b->mo_row[big - 1] + (small - b->minsize[big - 1])] > v)
                    b->mo_monotone = false;
            }
        if (b->mo_monotone) {
            // bound fields: for each size l and position p of its maxprefix, the
            // largest probe length lp whose minoverlap with l leaves l - p enough
            // (monotone in lp; lengths incompatible with l count as admitted
            // below l and refused above it: no window pairs them)
            auto admits = [&](uint32_t lp, uint32_t l, uint32_t v) -> bool {
                const uint32_t big = std::max(lp, l), small = std::min(lp, l);
                if (small < b->minsize[big]) return lp < l;
                const uint32_t raw = b->mo_tab[b->mo_row[big] + (small - b->minsize[big])];
                return v >= std::min(small, std::min(big, raw));
            };
            uint64_t total = 0;
            b->lp_row.assign((size_t)L + 2, 0);
            for (uint32_t l = 0; l <= L; ++l) {
                b->lp_row[l] = (uint32_t)total;
                total += b->probe_prefix[l];
            }
            b->lp_row[L + 1] = (uint32_t)total;
            if (total <= MAX_COSINE_TABLE) {
                b->lp_tab.resize(total ? total : 1);
                for (uint32_t l = 1; l <= L; ++l)
                    for (uint32_t p = 0; p < b->probe_prefix[l]; ++p) {
                        uint32_t lo = 0, hi = L + 1;  // admits(lo), not admits(hi)
                        while (hi - lo > 1) {
                            const uint32_t mid = lo + (hi - lo) / 2;
                            if (admits(mid, l, l - p)) lo = mid;
                            else hi = mid;
                        }
                        b->lp_tab[b->lp_row[l] + p] = lo;
                    }
            } else {
                b->lp_row.clear();
            }
        }
    } else {
        b->mo_sum.resize(2 * (size_t)L + 1);
        for (uint32_t s = 0; s <= 2 * L; ++s) b->mo_sum[s] = sim_minoverlap(sim, s, 0, tau);
        b->mo_row.assign(1, 0);
        b->mo_tab.assign(1, 0);
        b->mo_monotone = true;
        for (uint32_t s = 1; s <= 2 * L; ++s)
            if (b->mo_sum[s] < b->mo_sum[s - 1]) b->mo_monotone = false;
        if (b->mo_monotone) {  // the sums whose minoverlap is <= v form the prefix [0, max_sum[v]]
            b->max_sum.resize((size_t)L + 1);
            uint32_t s = 0;
            for (uint32_t v = 0; v <= L; ++v) {
                while (s < 2 * L && b->mo_sum[s + 1] <= v) ++s;
                b->max_sum[v] = s;
            }
        }
    }
    // one device allocation holding all tables
    size_t n32 = 5 * ((size_t)L + 1) + b->mo_sum.size() + b->mo_tab.size() + b->max_sum.size() + b->lp_row.size() +
                 b->lp_tab.size();
    size_t bytes = b->mo_row.size() * 8 + n32 * 4;
    CK(b->dev.ensure(bytes, ctx->stream));
    uint8_t* base = b->dev.as<uint8_t>();
    uint64_t* d_row = (uint64_t*)base;
    uint32_t* p = (uint32_t*)(base + b->mo_row.size() * 8);
    auto put = [&](const std::vector<uint32_t>& v, uint32_t*& dst) -> cudaError_t {
        uint32_t* d = p;
        p += v.size();
        dst = d;
        return cudaMemcpyAsync(d, v.data(), v.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    };
    uint32_t *d_minsize, *d_pp, *d_ip, *d_mp, *d_mid, *d_sum, *d_tab, *d_msum = nullptr, *d_lprow = nullptr,
             *d_lptab = nullptr;
    CK(cudaMemcpyAsync(d_row, b->mo_row.data(), b->mo_row.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(put(b->minsize, d_minsize));
    CK(put(b->probe_prefix, d_pp));
    CK(put(b->index_prefix, d_ip));
    CK(put(b->max_partner, d_mp));
    CK(put(b->mid_prefix, d_mid));
    CK(put(b->mo_sum, d_sum));
    CK(put(b->mo_tab, d_tab));
    if (!b->max_sum.empty()) CK(put(b->max_sum, d_msum));
    if (!b->lp_row.empty()) {
        CK(put(b->lp_row, d_lprow));
        CK(put(b->lp_tab, d_lptab));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    b->view = BoundsView{d_minsize, d_pp, d_ip, d_mp, d_mid, d_sum, d_row, d_tab, L, sim, d_msum, d_lprow, d_lptab};
    *out = b.get();
    ctx->bounds.emplace(key, std::move(b));
    return HYSET_OK;
}

}  // namespace hs
