/*
 * oracle.c — CPU restatement of the reference's exact set-similarity self-join.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline.  The product library (hyset_gb300/) never links or calls this file.
 *
 * Restated from chribell/hyset:
 *   similarity bounds    include/hyset/similarity.hpp:11-54, helpers.hpp:36-50
 *   prefix entries       include/hyset/collection.hpp:128-135 (midprefix tokens per set)
 *   inverted index       include/hyset/index.hpp:251-282 (entries sorted by (token, setID),
 *                        list t = [offsets[t-1], offsets[t]))
 *   allpairs             include/hyset/host_algorithms.hpp:16-129
 *   ppjoin               include/hyset/host_algorithms.hpp:131-250
 *   verify_pair          include/hyset/verification.hpp:9-31
 *   cpu_multi split      src/cpu_multi.cu:118-149, :177-207
 * Compile with -ffp-contract=off so no multiply-add is fused: the bounds must be
 * the same doubles the reference computes.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* Seconds spent in the last index build / probe loop of this thread (the
 * reference times the join separately from indexing, src/cpu_single.cu:98-140). */
static _Thread_local double t_index_s, t_join_s;
static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static double g_multi_index_s, g_multi_join_s;
void oracle_last_timing(double* index_s, double* join_s) {
    if (index_s) *index_s = t_index_s;
    if (join_s) *join_s = t_join_s;
}
void oracle_last_multi_timing(double* index_s, double* join_s) {
    if (index_s) *index_s = g_multi_index_s;
    if (join_s) *join_s = g_multi_join_s;
}

/* ---------------------------------------------------------------- bounds */

static int imin(int a, int b) { return (a > b) ? b : a; } /* hyset::min, helpers.hpp:41-44 */

static uint32_t sim_minoverlap(int sim, uint32_t l1, uint32_t l2, double t) {
    switch (sim) {
    case ORACLE_COSINE: return (uint32_t)(ceil(t * sqrt((double)l1 * (double)l2)));
    case ORACLE_DICE:   return (uint32_t)(ceil(t * (double)(l1 + l2) / 2.0));
    default:            return (uint32_t)(ceil((double)(l1 + l2) * t / (1 + t))); /* similarity.hpp:40-42 */
    }
}

uint32_t oracle_minsize(int sim, uint32_t len, double t) {
    switch (sim) {
    case ORACLE_COSINE: return (uint32_t)(ceil(t * t * (double)len));
    case ORACLE_DICE:   return (uint32_t)(ceil(t * (double)len / (2.0 - t)));
    default:            return (uint32_t)(ceil(t * (double)len)); /* similarity.hpp:44-46 */
    }
}

uint32_t oracle_maxsize(int sim, uint32_t len, double t) {
    switch (sim) {
    case ORACLE_COSINE: return (uint32_t)((double)len / (t * t));
    case ORACLE_DICE:   return (uint32_t)((2.0 - t) * (double)len / t);
    default:            return (uint32_t)(((double)len / t)); /* similarity.hpp:48-50 */
    }
}

/* generic_similarity::minoverlap, similarity.hpp:21-23 */
uint32_t oracle_minoverlap(int sim, uint32_t l1, uint32_t l2, double t) {
    return (uint32_t)imin((int)l2, imin((int)l1, (int)sim_minoverlap(sim, l1, l2, t)));
}

/* generic_similarity::maxprefix, similarity.hpp:13-15 */
uint32_t oracle_maxprefix(int sim, uint32_t len, double t) {
    return (uint32_t)imin((int)len, (int)(len - oracle_minsize(sim, len, t) + 1));
}

/* generic_similarity::midprefix, similarity.hpp:17-19 */
uint32_t oracle_midprefix(int sim, uint32_t len, double t) {
    return (uint32_t)imin((int)len, (int)(len - oracle_minoverlap(sim, len, len, t) + 1));
}

/* ---------------------------------------------------------------- results */

struct oracle_pairs {
    uint32_t* data;
    uint64_t count, cap;
};

static oracle_pairs* pairs_new(void) {
    oracle_pairs* p = (oracle_pairs*)calloc(1, sizeof(oracle_pairs));
    return p;
}

static int pairs_add(oracle_pairs* p, uint32_t a, uint32_t b) {
    if (p->count == p->cap) {
        uint64_t cap = p->cap ? p->cap * 2 : 1024;
        uint32_t* d = (uint32_t*)realloc(p->data, cap * 2 * sizeof(uint32_t));
        if (!d) return 1;
        p->data = d;
        p->cap = cap;
    }
    p->data[2 * p->count] = a;
    p->data[2 * p->count + 1] = b;
    p->count++;
    return 0;
}

static int pairs_append(oracle_pairs* dst, const oracle_pairs* src) {
    for (uint64_t k = 0; k < src->count; ++k)
        if (pairs_add(dst, src->data[2 * k], src->data[2 * k + 1])) return 1;
    return 0;
}

uint64_t oracle_pairs_count(const oracle_pairs* p) { return p ? p->count : 0; }
const uint32_t* oracle_pairs_data(const oracle_pairs* p) { return p ? p->data : NULL; }
void oracle_pairs_free(oracle_pairs* p) {
    if (p) { free(p->data); free(p); }
}

/* ---------------------------------------------------------------- index */

typedef struct {
    uint32_t* list_begin; /* [universe] */
    uint32_t* list_end;   /* [universe] */
    uint32_t* set_id;     /* entry setID, lists ordered by (token, setID) */
    uint32_t* position;   /* entry position within its set */
} cpu_index;

/* The reference builds this on the GPU (histogram -> exclusive scan -> scatter ->
 * sort by (token, setID), index.hpp:251-282) and copies it back.  Entries are
 * generated in setID order, so a stable counting sort by token gives the same
 * (token, setID) order. */
static int index_build(cpu_index* ix, const uint32_t* tokens, const uint32_t* starts,
                       const uint32_t* sizes, uint32_t universe, int sim, double t,
                       uint32_t lo, uint32_t hi) {
    memset(ix, 0, sizeof(*ix));
    uint64_t entries = 0;
    for (uint32_t s = lo; s <= hi; ++s) entries += oracle_midprefix(sim, sizes[s], t);
    ix->list_begin = (uint32_t*)calloc((size_t)universe + 1, sizeof(uint32_t));
    ix->list_end = (uint32_t*)calloc((size_t)universe + 1, sizeof(uint32_t));
    ix->set_id = (uint32_t*)malloc((entries ? entries : 1) * sizeof(uint32_t));
    ix->position = (uint32_t*)malloc((entries ? entries : 1) * sizeof(uint32_t));
    if (!ix->list_begin || !ix->list_end || !ix->set_id || !ix->position) return 1;
    for (uint32_t s = lo; s <= hi; ++s) {
        uint32_t pre = oracle_midprefix(sim, sizes[s], t);
        for (uint32_t i = 0; i < pre; ++i) ix->list_end[tokens[starts[s] + i]]++;
    }
    uint32_t run = 0;
    for (uint32_t k = 0; k < universe; ++k) {
        uint32_t c = ix->list_end[k];
        ix->list_begin[k] = run;
        ix->list_end[k] = run;
        run += c;
    }
    for (uint32_t s = lo; s <= hi; ++s) {
        uint32_t pre = oracle_midprefix(sim, sizes[s], t);
        for (uint32_t i = 0; i < pre; ++i) {
            uint32_t tok = tokens[starts[s] + i];
            uint32_t at = ix->list_end[tok]++;
            ix->set_id[at] = s;
            ix->position[at] = i;
        }
    }
    return 0;
}

static void index_free(cpu_index* ix) {
    free(ix->list_begin);
    free(ix->list_end);
    free(ix->set_id);
    free(ix->position);
}

/* ---------------------------------------------------------------- verify */

/* verification.hpp:9-31 */
static int verify_pair(const uint32_t* r1, uint32_t r1size, const uint32_t* r2, uint32_t r2size,
                       uint32_t overlapthres, uint32_t posr1, uint32_t posr2, uint32_t foundoverlap) {
    uint32_t maxr1 = r1size - posr1 + foundoverlap;
    uint32_t maxr2 = r2size - posr2 + foundoverlap;
    while (maxr1 >= overlapthres && maxr2 >= overlapthres && foundoverlap < overlapthres) {
        if (r1[posr1] == r2[posr2]) {
            ++posr1;
            ++posr2;
            ++foundoverlap;
        } else if (r1[posr1] < r2[posr2]) {
            ++posr1;
            --maxr1;
        } else {
            ++posr2;
            --maxr2;
        }
    }
    return foundoverlap >= overlapthres;
}

/* ---------------------------------------------------------------- join */

typedef struct {
    uint32_t count, minoverlap, probe_pos, indexed_pos; /* structs.hpp:83-94 */
} cand_data;

static int join_range(oracle_pairs* out, const uint32_t* tokens, const uint32_t* starts,
                      const uint32_t* sizes, uint32_t n_sets, uint32_t universe, int sim,
                      double t, int algo, uint32_t index_lo, uint32_t index_hi,
                      uint32_t probe_lo, uint32_t probe_hi) {
    cpu_index ix;
    double t0 = now_s();
    if (index_build(&ix, tokens, starts, sizes, universe, sim, t, index_lo, index_hi)) {
        index_free(&ix);
        return 1;
    }
    double t1 = now_s();
    t_index_s = t1 - t0;
    cand_data* cd = (cand_data*)calloc(n_sets ? n_sets : 1, sizeof(cand_data));
    uint32_t* cands = (uint32_t*)malloc((n_sets ? n_sets : 1) * sizeof(uint32_t));
    if (!cd || !cands) {
        free(cd);
        free(cands);
        index_free(&ix);
        return 1;
    }
    int err = 0;
    for (uint32_t probe = probe_lo; probe <= probe_hi && !err; ++probe) {
        const uint32_t psize = sizes[probe];
        const uint32_t* ptok = tokens + starts[probe];
        const uint32_t minsize = oracle_minsize(sim, psize, t);
        const uint32_t prefix = oracle_maxprefix(sim, psize, t);
        const uint32_t maxsize = oracle_maxsize(sim, psize, t);
        uint32_t ncand = 0;

        /* filter: host_algorithms.hpp:47-86 (allpairs), :161-210 (ppjoin) */
        for (uint32_t pos = 0; pos < prefix; ++pos) {
            uint32_t tok = ptok[pos];
            uint32_t k = ix.list_begin[tok], end = ix.list_end[tok];
            while (k < end && sizes[ix.set_id[k]] < minsize) ++k; /* length_filter */
            for (; k < end; ++k) {
                uint32_t id = ix.set_id[k];
                if (id >= probe) break;
                uint32_t isize = sizes[id];
                if (isize > maxsize) break;
                cand_data* c = &cd[id];
                if (algo == 1) {
                    if (c->count == 0) {
                        uint32_t mo = oracle_minoverlap(sim, psize, isize, t);
                        /* position_filter, helpers.hpp:46-50 */
                        if (!(mo <= (uint32_t)imin((int)(psize - pos), (int)(isize - ix.position[k]))))
                            continue;
                        cands[ncand++] = id;
                        c->minoverlap = mo;
                    }
                    c->count += 1;
                    c->probe_pos = pos;
                    c->indexed_pos = ix.position[k];
                } else {
                    if (c->count == 0) cands[ncand++] = id;
                    c->count += 1;
                }
            }
        }

        /* verify: host_algorithms.hpp:89-127 (allpairs), :212-248 (ppjoin) */
        for (uint32_t q = 0; q < ncand; ++q) {
            uint32_t id = cands[q];
            cand_data* c = &cd[id];
            uint32_t isize = sizes[id];
            const uint32_t* itok = tokens + starts[id];
            uint32_t lastposind = oracle_midprefix(sim, isize, t);
            uint32_t lastposprobe = prefix;
            uint32_t recpreftoklast = ptok[lastposprobe - 1];
            uint32_t indrecpreftoklast = itok[lastposind - 1];
            uint32_t recpos, indrecpos, mo;
            if (algo == 1) {
                recpos = c->probe_pos;
                indrecpos = c->indexed_pos;
                if (recpreftoklast > indrecpreftoklast) {
                    recpos += 1;
                    indrecpos = lastposind;
                } else {
                    recpos = lastposprobe;
                    indrecpos += 1;
                }
                mo = c->minoverlap;
            } else {
                if (recpreftoklast > indrecpreftoklast) {
                    recpos = c->count;
                    indrecpos = lastposind;
                } else {
                    recpos = lastposprobe;
                    indrecpos = c->count;
                }
                mo = oracle_minoverlap(sim, psize, isize, t);
            }
            if (verify_pair(ptok, psize, itok, isize, mo, recpos, indrecpos, c->count))
                if (pairs_add(out, probe, id)) err = 1;
            c->count = 0;
        }
    }
    t_join_s = now_s() - t1;
    free(cd);
    free(cands);
    index_free(&ix);
    return err;
}

oracle_pairs* oracle_join(const uint32_t* tokens, const uint32_t* starts, const uint32_t* sizes,
                          uint32_t n_sets, uint32_t universe, int sim, double t, int algo,
                          uint32_t index_lo, uint32_t index_hi, uint32_t probe_lo, uint32_t probe_hi) {
    oracle_pairs* out = pairs_new();
    if (!out) return NULL;
    if (n_sets == 0 || index_lo > index_hi || probe_lo > probe_hi) return out;
    if (index_hi >= n_sets || probe_hi >= n_sets ||
        join_range(out, tokens, starts, sizes, n_sets, universe, sim, t, algo, index_lo, index_hi,
                   probe_lo, probe_hi)) {
        oracle_pairs_free(out);
        return NULL;
    }
    return out;
}

typedef struct {
    const uint32_t *tokens, *starts, *sizes;
    uint32_t n_sets, universe, lo, hi;
    int sim, algo, err;
    double t, index_s, join_s;
    oracle_pairs* out;
} worker_arg;

static void* worker(void* a) {
    worker_arg* w = (worker_arg*)a;
    w->out = pairs_new();
    if (!w->out) { w->err = 1; return NULL; }
    if (w->lo <= w->hi) {
        w->err = join_range(w->out, w->tokens, w->starts, w->sizes, w->n_sets, w->universe, w->sim,
                            w->t, w->algo, 0, w->hi, w->lo, w->hi);
        w->index_s = t_index_s;
        w->join_s = t_join_s;
    }
    return NULL;
}

oracle_pairs* oracle_join_multi(const uint32_t* tokens, const uint32_t* starts, const uint32_t* sizes,
                                uint32_t n_sets, uint32_t universe, int sim, double t, int algo,
                                int threads) {
    return oracle_join_multi_range(tokens, starts, sizes, n_sets, universe, sim, t, algo, threads, 0,
                                   n_sets ? n_sets - 1 : 0);
}

oracle_pairs* oracle_join_multi_range(const uint32_t* tokens, const uint32_t* starts, const uint32_t* sizes,
                                      uint32_t n_sets, uint32_t universe, int sim, double t, int algo,
                                      int threads, uint32_t probe_lo, uint32_t probe_hi) {
    if (threads < 1) threads = 1;
    oracle_pairs* out = pairs_new();
    if (!out || n_sets == 0 || probe_lo > probe_hi || probe_hi >= n_sets) return out;
    const uint32_t k = probe_hi - probe_lo + 1;
    worker_arg* args = (worker_arg*)calloc((size_t)threads, sizeof(worker_arg));
    pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    if (!args || !th) { free(args); free(th); oracle_pairs_free(out); return NULL; }
    /* x_i = k * sqrt((i + 1) / P), truncated: cpu_multi.cu:118-125 */
    uint32_t prev = probe_lo;
    for (int i = 0; i < threads; ++i) {
        uint32_t point = probe_lo + (uint32_t)((double)k * sqrt((double)(i + 1) / (double)threads));
        worker_arg* w = &args[i];
        w->tokens = tokens; w->starts = starts; w->sizes = sizes;
        w->n_sets = n_sets; w->universe = universe; w->sim = sim; w->algo = algo; w->t = t;
        w->lo = prev;
        w->hi = point ? point - 1 : 0;
        if (point <= prev) w->hi = 0, w->lo = 1; /* empty range */
        if (i == threads - 1 && point <= probe_hi && point > prev) w->hi = probe_hi;
        prev = point > prev ? point : prev;
    }
    int err = 0;
    for (int i = 0; i < threads; ++i)
        if (pthread_create(&th[i], NULL, worker, &args[i])) { worker(&args[i]); th[i] = 0; }
    for (int i = 0; i < threads; ++i)
        if (th[i]) pthread_join(th[i], NULL);
    g_multi_index_s = g_multi_join_s = 0;
    for (int i = 0; i < threads; ++i) {
        if (args[i].index_s > g_multi_index_s) g_multi_index_s = args[i].index_s;
        if (args[i].join_s > g_multi_join_s) g_multi_join_s = args[i].join_s;
    }
    for (int i = 0; i < threads; ++i) {
        if (args[i].err || !args[i].out || pairs_append(out, args[i].out)) err = 1;
        oracle_pairs_free(args[i].out);
    }
    free(args);
    free(th);
    if (err) { oracle_pairs_free(out); return NULL; }
    return out;
}

/* ---------------------------------------------------------------- exhaustive */

static uint32_t overlap(const uint32_t* a, uint32_t na, const uint32_t* b, uint32_t nb) {
    uint32_t i = 0, j = 0, o = 0;
    while (i < na && j < nb) {
        if (a[i] == b[j]) { ++o; ++i; ++j; }
        else if (a[i] < b[j]) ++i;
        else ++j;
    }
    return o;
}

oracle_pairs* oracle_brute(const uint32_t* tokens, const uint32_t* starts, const uint32_t* sizes,
                           uint32_t n_sets, int sim, double t) {
    oracle_pairs* out = pairs_new();
    if (!out) return NULL;
    for (uint32_t p = 0; p < n_sets; ++p) {
        uint32_t ms = oracle_minsize(sim, sizes[p], t);
        for (uint32_t c = 0; c < p; ++c) {
            if (sizes[c] < ms) continue;
            uint32_t mo = oracle_minoverlap(sim, sizes[p], sizes[c], t);
            if (overlap(tokens + starts[p], sizes[p], tokens + starts[c], sizes[c]) >= mo)
                if (pairs_add(out, p, c)) { oracle_pairs_free(out); return NULL; }
        }
    }
    return out;
}

oracle_pairs* oracle_brute_rs(const uint32_t* r_tokens, const uint32_t* r_starts, const uint32_t* r_sizes,
                              uint32_t r_n, const uint32_t* s_tokens, const uint32_t* s_starts,
                              const uint32_t* s_sizes, uint32_t s_n, int sim, double t) {
    oracle_pairs* out = pairs_new();
    if (!out) return NULL;
    for (uint32_t s = 0; s < s_n; ++s) {
        for (uint32_t r = 0; r < r_n; ++r) {
            uint32_t big = s_sizes[s] > r_sizes[r] ? s_sizes[s] : r_sizes[r];
            uint32_t small = s_sizes[s] > r_sizes[r] ? r_sizes[r] : s_sizes[s];
            if (small < oracle_minsize(sim, big, t)) continue;
            uint32_t mo = oracle_minoverlap(sim, big, small, t);
            if (overlap(s_tokens + s_starts[s], s_sizes[s], r_tokens + r_starts[r], r_sizes[r]) >= mo)
                if (pairs_add(out, s, r)) { oracle_pairs_free(out); return NULL; }
        }
    }
    return out;
}

/* ---- the reference's text reader ----------------------------------------- */

static int is_space_c(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

/* atoi of item [a, b); *digits = whether any digit was read */
static uint32_t atoi_item(const char* a, const char* b, int* digits) {
    while (a < b && is_space_c(*a)) ++a;
    int neg = 0;
    if (a < b && (*a == '+' || *a == '-')) {
        neg = *a == '-';
        ++a;
    }
    uint32_t v = 0;
    *digits = 0;
    while (a < b && *a >= '0' && *a <= '9') {
        v = v * 10u + (uint32_t)(*a - '0');
        ++a;
        *digits = 1;
    }
    return neg ? (uint32_t)(0u - v) : v;
}

uint64_t oracle_read_text(const char* text, uint64_t n, uint32_t* tokens, uint64_t tok_cap, uint32_t* sizes,
                          uint64_t size_cap, uint64_t* n_tokens, uint64_t* empty_items) {
    uint64_t sets = 0, toks = 0, empty = 0, i = 0;
    while (i < n) {
        uint64_t e = i;
        while (e < n && text[e] != '\n') ++e;
        if (e > i) { /* a non-empty line [i, e) */
            uint32_t count = 0;
            uint64_t a = i;
            for (uint64_t k = i; k <= e; ++k) {
                const int end = k == e;
                if (end && k == a) break; /* nothing after the last ' ' */
                if (end || text[k] == ' ') {
                    int digits = 0;
                    const uint32_t v = atoi_item(text + a, text + k, &digits);
                    if (!digits) ++empty;
                    if (toks < tok_cap) tokens[toks] = v;
                    ++toks;
                    ++count;
                    a = k + 1;
                }
            }
            if (sets < size_cap) sizes[sets] = count;
            ++sets;
        }
        i = e + 1;
    }
    *n_tokens = toks;
    *empty_items = empty;
    return sets;
}

/* ---- explicit candidate lists -------------------------------------------- */

/* Candidate lists verified as hybrid::device_handler's kernels do: every
 * (probe, candidate) merged from the start of both sets with the early-exit
 * bounds of verification.hpp:9-31.  *tokens_read receives the tokens the
 * merges read (positions consumed on both sides when each merge stops). */
oracle_pairs* oracle_verify_csr(const uint32_t* r_tokens, const uint32_t* r_starts, const uint32_t* r_sizes,
                                const uint32_t* s_tokens, const uint32_t* s_starts, const uint32_t* s_sizes,
                                const uint32_t* probes, const uint32_t* offsets, const uint32_t* cands,
                                uint32_t n_probes, int sim, double t, uint64_t* tokens_read) {
    oracle_pairs* out = pairs_new();
    if (!out) return NULL;
    uint64_t read = 0;
    for (uint32_t i = 0; i < n_probes; ++i) {
        const uint32_t p = probes[i], lp = s_sizes[p];
        const uint32_t* a = s_tokens + s_starts[p];
        const uint32_t cb = i ? offsets[i - 1] : 0, ce = offsets[i];
        for (uint32_t k = cb; k < ce; ++k) {
            const uint32_t c = cands[k], lc = r_sizes[c];
            const uint32_t* b = r_tokens + r_starts[c];
            const uint32_t thr = oracle_minoverlap(sim, lp, lc, t);
            uint32_t x = 0, y = 0, found = 0, maxa = lp, maxb = lc;
            while (maxa >= thr && maxb >= thr && found < thr) {
                if (a[x] == b[y]) { ++x; ++y; ++found; }
                else if (a[x] < b[y]) { ++x; --maxa; }
                else { ++y; --maxb; }
            }
            read += x + y;
            if (found >= thr && pairs_add(out, p, c)) { oracle_pairs_free(out); return NULL; }
        }
    }
    *tokens_read = read;
    return out;
}
