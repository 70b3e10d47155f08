/*
 * oracle.h — CPU restatement of the reference's set-similarity self-join.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker for the CUDA path, and the
 * timed CPU baseline of the benchmark; the product library never links, loads
 * or calls it.  Each function cites the reference file:line it restates
 * (paths relative to the chribell/hyset source tree).
 *
 * Parity pinning: the restatement is checked against the reference's own
 * host::allpairs / host::ppjoin, compiled from its headers by oracle/Makefile
 * (target `ref`) and run on seeded inputs; the fixtures in tests/golden/ were
 * produced that way (tests/golden/make_golden.py).
 */
#ifndef HYSET_ORACLE_H
#define HYSET_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_JACCARD = 0, ORACLE_COSINE = 1, ORACLE_DICE = 2 };

/* Similarity bounds exactly as include/hyset/similarity.hpp:11-54 computes them
 * (double arithmetic, same expression order, `hyset::min(int,int)` clamps).
 * Cosine and dice have no reference code; they follow the same style. */
uint32_t oracle_minoverlap(int sim, uint32_t len1, uint32_t len2, double t); /* generic, clamped */
uint32_t oracle_minsize(int sim, uint32_t len, double t);
uint32_t oracle_maxsize(int sim, uint32_t len, double t);
uint32_t oracle_maxprefix(int sim, uint32_t len, double t);
uint32_t oracle_midprefix(int sim, uint32_t len, double t);

typedef struct oracle_pairs oracle_pairs;

/* AllPairs (algo 0) or PPJoin (algo 1) of probes [probe_lo, probe_hi] against an
 * inverted index over the midprefix entries of sets [index_lo, index_hi]
 * (include/hyset/host_algorithms.hpp:16-129 and :131-250).  Pairs are
 * (probe, indexed) with indexed < probe. */
oracle_pairs* oracle_join(const uint32_t* tokens, const uint32_t* starts, const uint32_t* sizes,
                          uint32_t n_sets, uint32_t universe, int sim, double t, int algo,
                          uint32_t index_lo, uint32_t index_hi, uint32_t probe_lo, uint32_t probe_hi);

/* cpu_multi: `threads` std::thread-style workers over sqrt-balanced probe
 * ranges, each with its own index over sets [0, end of its range]
 * (src/cpu_multi.cu:118-149, :177-207).  The union of the workers' pairs. */
oracle_pairs* oracle_join_multi(const uint32_t* tokens, const uint32_t* starts, const uint32_t* sizes,
                                uint32_t n_sets, uint32_t universe, int sim, double t, int algo,
                                int threads);

/* The same over probes [probe_lo, probe_hi] only (sqrt split within the range;
 * a bounded sample of a join). */
oracle_pairs* oracle_join_multi_range(const uint32_t* tokens, const uint32_t* starts, const uint32_t* sizes,
                                      uint32_t n_sets, uint32_t universe, int sim, double t, int algo,
                                      int threads, uint32_t probe_lo, uint32_t probe_hi);

/* Wall seconds of the last index build and probe loop on the calling thread
 * (oracle_join), or the slowest worker of the last multi-threaded join. */
void oracle_last_timing(double* index_s, double* join_s);
void oracle_last_multi_timing(double* index_s, double* join_s);

/* Exhaustive check of every pair: (p, c) with c < p, sizes[c] >= minsize(sizes[p])
 * and |p ∩ c| >= minoverlap(sizes[p], sizes[c]).  Small inputs only. */
oracle_pairs* oracle_brute(const uint32_t* tokens, const uint32_t* starts, const uint32_t* sizes,
                           uint32_t n_sets, int sim, double t);

/* R-S join by exhaustive check: (s, r) for s in S, r in R with, for
 * (b, m) = (max, min) of the two sizes, m >= minsize(b) and overlap >= minoverlap(b, m).
 * Pairs are (probe s, indexed r).  Small inputs only. */
oracle_pairs* oracle_brute_rs(const uint32_t* r_tokens, const uint32_t* r_starts, const uint32_t* r_sizes,
                              uint32_t r_n, const uint32_t* s_tokens, const uint32_t* s_starts,
                              const uint32_t* s_sizes, uint32_t s_n, int sim, double t);

/* hyset::collection::read_collection's text reading (include/hyset/collection.hpp:93-177)
 * and split (collection.hpp:16-24): lines by '\n' (the text after the last
 * '\n' too), empty lines skipped, items split at every ' ' (a space at the end
 * of a line ends the last item), each item atoi'ed (leading white space, a
 * sign, digits).  Writes up to tok_cap tokens and size_cap sizes; returns the
 * number of sets, *n_tokens the number of tokens and *empty_items the items
 * with no digits (atoi gives 0). */
uint64_t oracle_read_text(const char* text, uint64_t n, uint32_t* tokens, uint64_t tok_cap, uint32_t* sizes,
                          uint64_t size_cap, uint64_t* n_tokens, uint64_t* empty_items);

/* Explicit candidate lists (probe probes[i] owns cands[offsets[i-1], offsets[i]))
 * verified as hybrid::device_handler's kernels do; *tokens_read receives the
 * tokens the early-exit merges read. */
oracle_pairs* oracle_verify_csr(const uint32_t* r_tokens, const uint32_t* r_starts, const uint32_t* r_sizes,
                                const uint32_t* s_tokens, const uint32_t* s_starts, const uint32_t* s_sizes,
                                const uint32_t* probes, const uint32_t* offsets, const uint32_t* cands,
                                uint32_t n_probes, int sim, double t, uint64_t* tokens_read);

uint64_t oracle_pairs_count(const oracle_pairs* p);
const uint32_t* oracle_pairs_data(const oracle_pairs* p); /* 2*count: (first, second) */
void oracle_pairs_free(oracle_pairs* p);

#ifdef __cplusplus
}
#endif
#endif
