// parse.cu — the reference's collection text format parsed on the GPU.
//
// hyset::collection::read_collection (include/hyset/collection.hpp:93-177)
// reads one set per line with std::getline, skips empty lines and splits each
// line on single spaces (split, collection.hpp:16-24: std::getline with ' '
// and atoi per item); sets arrive sorted by size with ascending tokens.  Here
// the text sits in device memory and two passes over 4 KiB tiles (256 threads,
// 16 bytes each, one 16-byte load per thread) turn it into the CSR arrays:
//   pass 1  per tile: count token ends and line starts and check the bytes;
//   scan    exclusive scans of the tile counts give every tile its first
//           token and first line;
//   pass 2  per tile: a block scan places every token and line; each thread
//           parses the digit runs that end in its 16 bytes eight digits at a
//           time, continuing a number that began in the previous thread's
//           bytes, and the tile's tokens and line starts are staged in shared
//           memory and stored contiguously.
// A token belongs to the thread holding its last digit.  Byte classes are
// computed four bytes at a time and kept as 16-bit masks (bit k = byte k of
// the thread's chunk).
// Lines are "d+( d+)* ?\r?\n" (a single trailing space is dropped, as the
// reference's split drops it).  Inputs the reference turns into token 0 by
// atoi of an empty or non-numeric item (two spaces, a leading space, a space
// before '\r', a blank "\r" line) and numbers of 2^32 or more are rejected
// with their byte offset instead.
#include "kernels.h"

namespace hs {

namespace {

constexpr int PARSE_THREADS = 256;
constexpr int PARSE_BYTES = 16;                               // per thread
constexpr uint64_t PARSE_TILE = PARSE_THREADS * PARSE_BYTES;  // 4096
constexpr int PARSE_MAX_ITEMS = PARSE_TILE / 2;               // tokens (or lines) of one tile, at most

// 0x80 in every byte of x that is zero.
__device__ __forceinline__ uint32_t zero_bytes(uint32_t x) {
    const uint32_t t = (x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu;
    return ~(t | x | 0x7F7F7F7Fu);
}

// The high bits of the four bytes of m (0x80 per byte) as bits 0..3.
__device__ __forceinline__ uint32_t pack4(uint32_t m) { return ((m >> 7) * 0x00204081u >> 21) & 0xFu; }

__device__ __forceinline__ uint32_t byte_eq(uint32_t w, uint32_t c) { return pack4(zero_bytes(w ^ (c * 0x01010101u))); }

// Bytes 0x30..0x39: (b - 0x30) < 10, four bytes at a time without borrows.
__device__ __forceinline__ uint32_t digit_bytes(uint32_t w) {
    const uint32_t hi = w & 0x80808080u;     // bytes >= 0x80 are not digits
    const uint32_t lo = w & 0x7F7F7F7Fu;
    const uint32_t ge0 = (lo + 0x50505050u) & 0x80808080u;  // lo >= 0x30
    const uint32_t ge10 = (lo + 0x46464646u) & 0x80808080u; // lo >= 0x3A
    return pack4(ge0 & ~ge10 & ~hi);
}

struct Masks {
    uint32_t digit, space, nl, cr, valid;  // bit k: byte k of the chunk (valid: inside the text)
    uint32_t prev_nl, prev_sp, next_digit, next_nl, next_cr;
};

__device__ __forceinline__ uint32_t byte_at(const uint8_t* t, uint64_t n, int64_t i) {
    return (i >= 0 && (uint64_t)i < n) ? t[i] : (uint32_t)'\n';  // outside the text: a line end
}

// The chunk's four words (bytes past the text read as '\n') and its masks.
__device__ __forceinline__ void load_chunk(const uint8_t* t, uint64_t n, uint64_t base, uint32_t (&w)[4], Masks& m) {
    if (base + PARSE_BYTES <= n) {
        const uint4 v = *reinterpret_cast<const uint4*>(t + base);  // base is a multiple of 16
        w[0] = v.x;
        w[1] = v.y;
        w[2] = v.z;
        w[3] = v.w;
    } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint32_t x = 0;
#pragma unroll
            for (int b = 0; b < 4; ++b) x |= byte_at(t, n, (int64_t)(base + 4 * q + b)) << (8 * b);
            w[q] = x;
        }
    }
    m.digit = m.space = m.nl = m.cr = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        m.digit |= digit_bytes(w[q]) << (4 * q);
        m.space |= byte_eq(w[q], ' ') << (4 * q);
        m.nl |= byte_eq(w[q], '\n') << (4 * q);
        m.cr |= byte_eq(w[q], '\r') << (4 * q);
    }
    m.valid = base >= n ? 0u : (n - base >= PARSE_BYTES ? 0xFFFFu : (1u << (n - base)) - 1u);
    const uint32_t before = byte_at(t, n, (int64_t)base - 1), after = byte_at(t, n, (int64_t)(base + PARSE_BYTES));
    m.prev_nl = ((m.nl << 1) | (before == '\n' ? 1u : 0u)) & 0xFFFFu;
    m.prev_sp = ((m.space << 1) | (before == ' ' ? 1u : 0u)) & 0xFFFFu;
    m.next_digit = (m.digit >> 1) | ((after - '0' < 10u) ? 0x8000u : 0u);
    m.next_nl = (m.nl >> 1) | (after == '\n' ? 0x8000u : 0u);
    m.next_cr = (m.cr >> 1) | (after == '\r' ? 0x8000u : 0u);
}

__device__ __forceinline__ uint32_t token_ends(const Masks& m) { return m.digit & ~m.next_digit & m.valid; }
__device__ __forceinline__ uint32_t line_starts(const Masks& m) { return m.prev_nl & ~m.nl & m.valid; }

// Error bits of the chunk and the first offending byte (bit index, 16 if none).
__device__ __forceinline__ uint32_t chunk_errors(const Masks& m, int& first) {
    const uint32_t bad_char = ~(m.digit | m.space | m.nl | m.cr) & m.valid;
    const uint32_t empty_item = m.space & (m.prev_sp | m.prev_nl | m.next_cr) & m.valid;
    const uint32_t bad_cr = m.cr & (~m.next_nl | m.prev_nl) & m.valid;
    const uint32_t any = bad_char | empty_item | bad_cr;
    first = any ? __ffs(any) - 1 : PARSE_BYTES;
    return (bad_char ? PARSE_E_CHAR : 0u) | (empty_item ? PARSE_E_EMPTY_ITEM : 0u) | (bad_cr ? PARSE_E_LINE_END : 0u);
}

__device__ __forceinline__ void record_error(uint32_t err, uint64_t at, uint32_t* flags,
                                             unsigned long long* first_bad) {
    if (err) {
        atomicOr(flags, err);
        atomicMin(first_bad, (unsigned long long)at);
    }
}

__global__ void __launch_bounds__(PARSE_THREADS) k_parse_count(const uint8_t* __restrict__ t, uint64_t n,
                                                               uint64_t tile0, uint32_t* tile_toks,
                                                               uint32_t* tile_lines, uint32_t* flags,
                                                               unsigned long long* first_bad) {
    __shared__ uint32_t red[2][PARSE_THREADS / 32];
    const uint64_t tile = tile0 + blockIdx.x;
    const uint64_t base = tile * PARSE_TILE + (uint64_t)threadIdx.x * PARSE_BYTES;
    uint32_t w[4];
    Masks m;
    load_chunk(t, n, base, w, m);
    int first;
    const uint32_t err = chunk_errors(m, first);
    record_error(err, base + first, flags, first_bad);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t toks = __reduce_add_sync(FULL, __popc(token_ends(m)));
    const uint32_t lines = __reduce_add_sync(FULL, __popc(line_starts(m)));
    if (lane == 0) {
        red[0][warp] = toks;
        red[1][warp] = lines;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t a = 0, b = 0;
        for (int q = 0; q < PARSE_THREADS / 32; ++q) {
            a += red[0][q];
            b += red[1][q];
        }
        tile_toks[tile] = a;
        tile_lines[tile] = b;
    }
}

// Eight bytes of the 16-byte chunk (lo = bytes 0..7, hi = 8..15) from byte s,
// byte s in the low byte (zeros past the chunk).
__device__ __forceinline__ uint64_t bytes_from(uint64_t lo, uint64_t hi, uint32_t s) {
    if (s == 0) return lo;
    if (s < 8) return (lo >> (8 * s)) | (hi << (64 - 8 * s));
    return hi >> (8 * (s - 8));
}

// Value of len (1..8) ASCII digits in the low bytes of x, the first digit in
// the lowest byte: the digits are moved to the top bytes over a '0' fill, then
// combined pairwise, four-wise and eight-wise with three multiplies (the
// published SWAR method of simdjson's parse_eight_digits_unrolled).
__device__ __forceinline__ uint32_t digits8(uint64_t x, uint32_t len) {
    uint64_t y = len == 8 ? x : (x << (8 * (8 - len))) | (0x3030303030303030ull >> (8 * len));
    y -= 0x3030303030303030ull;
    y = ((y & 0x0F0F0F0F0F0F0F0Full) * 2561ull) >> 8;
    y = ((y & 0x00FF00FF00FF00FFull) * 6553601ull) >> 16;
    return (uint32_t)(((y & 0x0000FFFF0000FFFFull) * 42949672960001ull) >> 32);
}

// Value of the digit run of len (1..10) bytes starting at byte s.
__device__ __forceinline__ unsigned long long run_value(uint64_t lo, uint64_t hi, uint32_t s, uint32_t len) {
    if (len <= 8) return digits8(bytes_from(lo, hi, s), len);
    return (unsigned long long)digits8(bytes_from(lo, hi, s), len - 8) * 100000000ull +
           digits8(bytes_from(lo, hi, s + len - 8), 8);
}

// The digit run that leaves the chunk on the right (nd = 0: none; nd = 11:
// more than ten digits, an error wherever the number ends).
__device__ __forceinline__ void right_run(uint32_t digit, uint64_t lo, uint64_t hi, unsigned long long& acc,
                                          uint32_t& nd) {
    acc = 0;
    nd = 0;
    if (!(digit & 0x8000u)) return;
    const uint32_t nond = ~digit & 0xFFFFu;
    const uint32_t s = nond ? 32u - __clz(nond) : 0u;  // one past the last non-digit
    const uint32_t len = PARSE_BYTES - s;
    if (s == 0 || len > 10) {
        nd = 11;
        return;
    }
    acc = run_value(lo, hi, s, len);
    nd = len;
}

__global__ void __launch_bounds__(PARSE_THREADS) k_parse_emit(const uint8_t* __restrict__ t, uint64_t n,
                                                              const uint32_t* __restrict__ tile_tok0,
                                                              const uint32_t* __restrict__ tile_line0,
                                                              uint32_t* __restrict__ tokens,
                                                              uint32_t* __restrict__ line_tok0, uint32_t* flags,
                                                              unsigned long long* first_bad) {
    __shared__ uint32_t wsum[2][PARSE_THREADS / 32];
    __shared__ unsigned long long tail_acc[PARSE_THREADS / 32];
    __shared__ uint32_t tail_nd[PARSE_THREADS / 32];
    __shared__ uint32_t s_tok[PARSE_MAX_ITEMS], s_line[PARSE_MAX_ITEMS];
    const uint64_t tile = blockIdx.x;
    const uint64_t base = tile * PARSE_TILE + (uint64_t)threadIdx.x * PARSE_BYTES;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t w[4];
    Masks m;
    load_chunk(t, n, base, w, m);
    const uint32_t ends = token_ends(m), starts = line_starts(m);
    const uint32_t toks = __popc(ends), lines = __popc(starts);
    // block-wide exclusive scan of the token and line counts
    const uint32_t ti = warp_incl_scan(toks, lane), li = warp_incl_scan(lines, lane);
    if (lane == 31) {
        wsum[0][warp] = ti;
        wsum[1][warp] = li;
    }
    __syncthreads();
    uint32_t tw = 0, lw = 0;
    for (int q = 0; q < warp; ++q) {
        tw += wsum[0][q];
        lw += wsum[1][q];
    }
    const uint32_t tok_first = tile_tok0[tile], line_first = tile_line0[tile];
    const uint32_t tok0 = tw + ti - toks;  // within the tile
    uint32_t line = lw + li - lines;
    // line starts: the index of the line's first token = tokens ending before it
    uint32_t sm = starts;
    while (sm) {
        const int k = __ffs(sm) - 1;
        sm &= sm - 1;
        s_line[line++] = tok_first + tok0 + __popc(ends & ((1u << k) - 1u));
    }
    // every token ending here: its run of digits [s, k] parsed eight digits at a
    // time; a run from byte 0 may continue a number of the previous chunk and
    // waits for the carry (lead_len digits, value lead)
    const uint64_t lo = w[0] | (uint64_t)w[1] << 32, hi = w[2] | (uint64_t)w[3] << 32;
    unsigned long long lead = 0;
    uint32_t lead_len = 0, tok = tok0, bad = 0;
    int bad_k = PARSE_BYTES;
    uint32_t e = ends;
    while (e) {
        const int k = __ffs(e) - 1;
        e &= e - 1;
        const uint32_t below = ~m.digit & ((1u << k) - 1u);
        const uint32_t st = below ? 32u - __clz(below) : 0u;
        const uint32_t len = (uint32_t)k - st + 1u;
        unsigned long long v = 0;
        if (len <= 10) v = run_value(lo, hi, st, len);
        if (st == 0 && (m.digit & 1u)) {
            lead = v;
            lead_len = len;
        } else if (len > 10 || v > 0xFFFFFFFFull) {
            bad = PARSE_E_RANGE;
            bad_k = min(bad_k, k);
        }
        s_tok[tok++] = (uint32_t)v;
    }
    // carry in: the previous chunk's right run (lane - 1; the previous warp's last
    // lane through shared memory; the previous tile's last chunk from memory)
    unsigned long long racc;
    uint32_t rnd;
    right_run(m.digit, lo, hi, racc, rnd);
    unsigned long long cacc = __shfl_up_sync(FULL, racc, 1);
    uint32_t cnd = __shfl_up_sync(FULL, rnd, 1);
    if (lane == 31) {
        tail_acc[warp] = racc;
        tail_nd[warp] = rnd;
    }
    __syncthreads();
    if (lane == 0) {
        if (warp > 0) {
            cacc = tail_acc[warp - 1];
            cnd = tail_nd[warp - 1];
        } else {
            cacc = 0;
            cnd = 0;
            if (base >= PARSE_BYTES) {
                uint32_t pw[4];
                Masks pm;
                load_chunk(t, n, base - PARSE_BYTES, pw, pm);
                right_run(pm.digit, pw[0] | (uint64_t)pw[1] << 32, pw[2] | (uint64_t)pw[3] << 32, cacc, cnd);
            }
        }
    }
    if (lead_len) {  // the first token ends here with lead_len digits from byte 0
        unsigned long long p10 = 1;
        for (uint32_t q = 0; q < lead_len && q < 11; ++q) p10 *= 10u;
        const unsigned long long v = cacc * p10 + lead;
        const uint32_t digits = cnd + lead_len;
        if (digits > 10 || v > 0xFFFFFFFFull) {
            bad = PARSE_E_RANGE;
            bad_k = 0;
        }
        s_tok[tok0] = (uint32_t)v;
    }
    record_error(bad, base + (uint64_t)bad_k, flags, first_bad);
    __syncthreads();
    const uint32_t n_tok = tile_tok0[tile + 1] - tok_first, n_line = tile_line0[tile + 1] - line_first;
    for (uint32_t i = threadIdx.x; i < n_tok; i += PARSE_THREADS) tokens[tok_first + i] = s_tok[i];
    for (uint32_t i = threadIdx.x; i < n_line; i += PARSE_THREADS) line_tok0[line_first + i] = s_line[i];
}

__global__ void k_line_sizes(const uint32_t* __restrict__ line_tok0, uint32_t n_lines, uint32_t n_tokens,
                             uint32_t* __restrict__ starts, uint32_t* __restrict__ sizes) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_lines; i += gridDim.x * blockDim.x) {
        const uint32_t a = line_tok0[i], b = i + 1 < n_lines ? line_tok0[i + 1] : n_tokens;
        starts[i] = a;
        sizes[i] = b - a;
    }
}

}  // namespace

uint64_t parse_tiles(uint64_t n_bytes) { return (n_bytes + PARSE_TILE - 1) / PARSE_TILE; }

cudaError_t parse_count(const uint8_t* text, uint64_t n_bytes, uint32_t* tile_toks, uint32_t* tile_lines,
                        uint32_t* flags, unsigned long long* first_bad, cudaStream_t s, uint64_t tile_lo,
                        uint64_t tile_hi) {
    const uint64_t tiles = parse_tiles(n_bytes);
    if (tile_hi > tiles) tile_hi = tiles;
    if (tile_hi <= tile_lo) return cudaSuccess;
    if (tile_hi - tile_lo > 0x7FFFFFFFull) return cudaErrorInvalidValue;
    note_launches();
    k_parse_count<<<(unsigned)(tile_hi - tile_lo), PARSE_THREADS, 0, s>>>(text, n_bytes, tile_lo, tile_toks,
                                                                         tile_lines, flags, first_bad);
    return cudaGetLastError();
}

cudaError_t parse_emit(const uint8_t* text, uint64_t n_bytes, const uint32_t* tile_tok0, const uint32_t* tile_line0,
                       uint32_t* tokens, uint32_t* line_tok0, uint32_t* flags, unsigned long long* first_bad,
                       cudaStream_t s) {
    const uint64_t tiles = parse_tiles(n_bytes);
    if (tiles == 0) return cudaSuccess;
    note_launches();
    k_parse_emit<<<(unsigned)tiles, PARSE_THREADS, 0, s>>>(text, n_bytes, tile_tok0, tile_line0, tokens, line_tok0,
                                                           flags, first_bad);
    return cudaGetLastError();
}

cudaError_t parse_line_sizes(const uint32_t* line_tok0, uint32_t n_lines, uint32_t n_tokens, uint32_t* starts,
                             uint32_t* sizes, cudaStream_t s) {
    if (n_lines == 0) return cudaSuccess;
    note_launches();
    unsigned g = (unsigned)std::min<uint64_t>((n_lines + 255) / 256, 152u * 16u);
    k_line_sizes<<<g, 256, 0, s>>>(line_tok0, n_lines, n_tokens, starts, sizes);
    return cudaGetLastError();
}

}  // namespace hs
