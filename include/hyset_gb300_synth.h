/*
 * hyset_gb300_synth.h — seeded synthetic set collections for benchmarks and tests.
 *
 * The reference reads its inputs from text files (one set per line, ascending
 * uint tokens, lines sorted by set size; include/hyset/collection.hpp:93-177).
 * It ships no data, so every workload here is generated: Zipf-distributed
 * tokens drawn without replacement inside a set, optional planted
 * near-duplicates, tokens renumbered 1..U by ascending global frequency, each
 * set sorted ascending and the collection sorted by (size, tokens).  This has
 * no counterpart in the reference's interface; it produces the inputs that the
 * reference's read_collection would have parsed.
 *
 * Host code only (C++), deterministic for a given seed on any machine and any
 * thread count.
 */
#ifndef HYSET_GB300_SYNTH_H
#define HYSET_GB300_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hyset_synth hyset_synth;

enum { HYSET_SIZES_UNIFORM = 0, HYSET_SIZES_LOGNORMAL = 1 };

typedef struct {
    uint64_t seed;
    uint32_t n_sets;
    uint32_t universe;      /* raw token ranks are 1..universe */
    double   zipf_s;        /* P(rank k) proportional to k^-zipf_s */
    int      size_dist;     /* HYSET_SIZES_* */
    double   size_a;        /* uniform: low;  lognormal: mu    */
    double   size_b;        /* uniform: high; lognormal: sigma */
    uint32_t size_min;      /* clamp after drawing */
    uint32_t size_max;
    double   dup_frac;      /* fraction of sets planted as near-duplicates */
    double   dup_edit_lo;   /* fraction of tokens replaced in a duplicate, */
    double   dup_edit_hi;   /* uniform in [lo, hi] */
    int      threads;       /* 0 = hardware concurrency */
} hyset_synth_params;

/* Returns 0 on success, nonzero on invalid parameters or allocation failure. */
int hyset_synth_generate(const hyset_synth_params* params, hyset_synth** out);
uint32_t hyset_synth_num_sets(const hyset_synth* s);
uint64_t hyset_synth_num_tokens(const hyset_synth* s);
uint32_t hyset_synth_max_token(const hyset_synth* s);
const uint32_t* hyset_synth_tokens(const hyset_synth* s);  /* CSR tokens, length num_tokens */
const uint32_t* hyset_synth_sizes(const hyset_synth* s);   /* length num_sets */
const uint32_t* hyset_synth_starts(const hyset_synth* s);  /* length num_sets */
/* Writes the reference's text format; returns 0 on success. */
int hyset_synth_write_text(const hyset_synth* s, const char* path);
/* Formats CSR arrays in the reference's text format (one set per line, tokens
 * split by one space, '\n' line ends) into buf; returns the byte count.  With
 * buf == NULL or cap too small nothing is written (the count is still returned). */
uint64_t hyset_format_text(const uint32_t* tokens, const uint32_t* starts, const uint32_t* sizes, uint32_t n_sets,
                           char* buf, uint64_t cap);
void hyset_synth_free(hyset_synth* s);

#ifdef __cplusplus
}
#endif
#endif
