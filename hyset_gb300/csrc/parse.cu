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
// Called by all lanes of a warp for consecutive chunks: the bytes just before
// and after the chunk come from the neighbouring lanes (the warp's end lanes
// read them from memory).
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
    const int lane = threadIdx.x & 31;
    const uint32_t up = __shfl_up_sync(FULL, w[3], 1), down = __shfl_down_sync(FULL, w[0], 1);
    const uint32_t before = lane > 0 ? up >> 24 : byte_at(t, n, (int64_t)base - 1);
    const uint32_t after = lane < 31 ? down & 0xFFu : byte_at(t, n, (int64_t)(base + PARSE_BYTES));
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

// Eight bytes of the staged tile from byte s (the tile is followed by eight
// bytes of '\n' so that reads near its end stay inside the stage).
__device__ __forceinline__ uint64_t stage_bytes(const uint64_t* st8, uint32_t s) {
    const uint32_t q = s >> 3, r = (s & 7u) * 8u;
    const uint64_t a = st8[q];
    return r ? (a >> r) | (st8[q + 1] << (64u - r)) : a;
}

// Pass 2, one block per 4 KiB tile.  Every thread classifies its 16 bytes and
// stages them with their digit mask in shared memory; a block scan places the
// tile's tokens and lines; the byte offset of every token's last digit is
// recorded; then the tile's tokens are parsed round-robin by all threads (no
// thread waits on a neighbour with more tokens) from the staged bytes, eight
// digits at a time, and stored contiguously.  A number that begins in the
// previous tile (at most one per tile) is read back from global memory.
__global__ void __launch_bounds__(PARSE_THREADS) k_parse_emit(const uint8_t* __restrict__ t, uint64_t n,
                                                              uint64_t tile0, const uint32_t* __restrict__ tile_tok0,
                                                              const uint32_t* __restrict__ tile_line0,
                                                              uint32_t* __restrict__ tokens,
                                                              uint32_t* __restrict__ line_tok0, uint32_t tok_cap,
                                                              uint32_t line_cap, uint32_t* flags,
                                                              unsigned long long* first_bad) {
    __shared__ uint32_t wsum[2][PARSE_THREADS / 32];
    __shared__ uint64_t s_text[PARSE_TILE / 8 + 1];
    __shared__ uint32_t s_dig[PARSE_THREADS];
    __shared__ uint16_t s_end[PARSE_MAX_ITEMS];
    __shared__ uint32_t s_line[PARSE_MAX_ITEMS];
    const uint64_t tile = tile0 + blockIdx.x;
    const uint64_t tile_base = tile * PARSE_TILE;
    const uint64_t base = tile_base + (uint64_t)threadIdx.x * PARSE_BYTES;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t w[4];
    Masks m;
    load_chunk(t, n, base, w, m);
    s_text[2 * threadIdx.x] = w[0] | (uint64_t)w[1] << 32;
    s_text[2 * threadIdx.x + 1] = w[2] | (uint64_t)w[3] << 32;
    if (threadIdx.x == 0) s_text[PARSE_TILE / 8] = 0x0A0A0A0A0A0A0A0Aull;
    s_dig[threadIdx.x] = m.digit;
    const uint32_t ends = token_ends(m), starts = line_starts(m);
    const uint32_t toks = __popc(ends), lines = __popc(starts);
    // block-wide exclusive scan of the token and line counts
    const uint32_t ti = warp_incl_scan(toks, lane), li = warp_incl_scan(lines, lane);
    if (lane == 31) {
        wsum[0][warp] = ti;
        wsum[1][warp] = li;
    }
    __syncthreads();
    uint32_t tw = 0, lw = 0, n_tok = 0, n_line = 0;
    for (int q = 0; q < PARSE_THREADS / 32; ++q) {
        if (q < warp) {
            tw += wsum[0][q];
            lw += wsum[1][q];
        }
        n_tok += wsum[0][q];
        n_line += wsum[1][q];
    }
    const uint32_t tok_first = tile_tok0[tile], line_first = tile_line0[tile];
    uint32_t tok = tw + ti - toks;  // within the tile
    uint32_t line = lw + li - lines;
    // line starts: the index of the line's first token = tokens ending before it
    for (uint32_t sm = starts; sm; sm &= sm - 1) {
        const int k = __ffs(sm) - 1;
        s_line[line++] = tok_first + tok + __popc(ends & ((1u << k) - 1u));
    }
    for (uint32_t e = ends; e; e &= e - 1) s_end[tok++] = (uint16_t)(threadIdx.x * PARSE_BYTES + __ffs(e) - 1);
    __syncthreads();
    uint32_t bad = 0;
    uint64_t bad_at = ~0ull;
    for (uint32_t i = threadIdx.x; i < n_tok; i += PARSE_THREADS) {
        const uint32_t e = s_end[i], c = e >> 4, k = e & 15u;
        // first digit of the run: after the last non-digit below byte e
        uint32_t st;
        const uint32_t below = ~s_dig[c] & ((1u << k) - 1u);
        bool from_prev_tile = false;
        if (below) {
            st = c * PARSE_BYTES + 32u - __clz(below);
        } else if (c > 0) {
            const uint32_t nondig = ~s_dig[c - 1] & 0xFFFFu;
            st = nondig ? (c - 1) * PARSE_BYTES + 32u - __clz(nondig) : 0u;
            from_prev_tile = !nondig;  // sixteen digits and more: too long, reported below
        } else {
            st = 0;
            from_prev_tile = true;
        }
        uint32_t len = e - st + 1;
        unsigned long long v = 0;
        if (from_prev_tile && c == 0 && tile_base > 0) {
            // the number may begin in the previous tile: its digits from memory
            uint32_t lead = 0;
            while (lead <= 10 && lead < tile_base && (uint32_t)t[tile_base - 1 - lead] - '0' < 10u) ++lead;
            len += lead;
            if (len <= 10)
                for (uint64_t q = tile_base - lead; q <= tile_base + e; ++q) v = v * 10u + (t[q] - '0');
        } else if (from_prev_tile && c > 0) {
            len = 11;  // a run of more than sixteen digits
        } else if (len <= 8) {
            v = digits8(stage_bytes(s_text, st), len);
        } else if (len <= 10) {
            v = (unsigned long long)digits8(stage_bytes(s_text, st), len - 8) * 100000000ull +
                digits8(stage_bytes(s_text, st + len - 8), 8);
        }
        if (len > 10 || v > 0xFFFFFFFFull) {
            bad = PARSE_E_RANGE;
            if (tile_base + e < bad_at) bad_at = tile_base + e;
        }
        if (tok_first + i < tok_cap) tokens[tok_first + i] = (uint32_t)v;
    }
    record_error(bad, bad_at, flags, first_bad);
    for (uint32_t i = threadIdx.x; i < n_line; i += PARSE_THREADS)
        if (line_first + i < line_cap) line_tok0[line_first + i] = s_line[i];
    if (threadIdx.x == 0 && ((uint64_t)tok_first + n_tok > tok_cap || (uint64_t)line_first + n_line > line_cap))
        atomicOr(flags, PARSE_E_CAPACITY);
}

// One block scans the token and line counts of up to 65,536 tiles (a chunk of
// the text) in place, on top of the totals carried from the previous chunks.
constexpr int CHUNK_SCAN_THREADS = 1024;
__global__ void __launch_bounds__(CHUNK_SCAN_THREADS) k_parse_chunk_scan(uint32_t* tile_toks, uint32_t* tile_lines,
                                                                         uint32_t n, uint32_t* carry, uint32_t k) {
    __shared__ uint32_t ws[2][CHUNK_SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t per = (n + CHUNK_SCAN_THREADS - 1) / CHUNK_SCAN_THREADS;  // consecutive tiles per thread
    const uint32_t lo = min(n, threadIdx.x * per), hi = min(n, lo + per);
    uint32_t a = 0, b = 0;
    for (uint32_t i = lo; i < hi; ++i) {
        a += tile_toks[i];
        b += tile_lines[i];
    }
    const uint32_t ia = warp_incl_scan(a, lane), ib = warp_incl_scan(b, lane);
    if (lane == 31) {
        ws[0][warp] = ia;
        ws[1][warp] = ib;
    }
    __syncthreads();
    uint32_t ra = carry[2 * k] + ia - a, rb = carry[2 * k + 1] + ib - b, ta = 0, tb = 0;
    for (int q = 0; q < CHUNK_SCAN_THREADS / 32; ++q) {
        if (q < warp) {
            ra += ws[0][q];
            rb += ws[1][q];
        }
        ta += ws[0][q];
        tb += ws[1][q];
    }
    for (uint32_t i = lo; i < hi; ++i) {
        const uint32_t x = tile_toks[i], y = tile_lines[i];
        tile_toks[i] = ra;
        tile_lines[i] = rb;
        ra += x;
        rb += y;
    }
    if (threadIdx.x == 0) {
        carry[2 * k + 2] = carry[2 * k] + ta;
        carry[2 * k + 3] = carry[2 * k + 1] + tb;
    }
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
                       cudaStream_t s, uint64_t tile_lo, uint64_t tile_hi, uint32_t tok_cap, uint32_t line_cap) {
    const uint64_t tiles = parse_tiles(n_bytes);
    if (tile_hi > tiles) tile_hi = tiles;
    if (tile_hi <= tile_lo) return cudaSuccess;
    if (tile_hi - tile_lo > 0x7FFFFFFFull) return cudaErrorInvalidValue;
    note_launches();
    k_parse_emit<<<(unsigned)(tile_hi - tile_lo), PARSE_THREADS, 0, s>>>(
        text, n_bytes, tile_lo, tile_tok0, tile_line0, tokens, line_tok0, tok_cap, line_cap, flags, first_bad);
    return cudaGetLastError();
}

cudaError_t parse_chunk_scan(uint32_t* tile_toks, uint32_t* tile_lines, uint64_t tile_lo, uint64_t tile_hi,
                             uint32_t* carry, uint64_t k, cudaStream_t s) {
    if (tile_hi <= tile_lo) return cudaSuccess;
    if (tile_hi - tile_lo > 65536u || k > 0x7FFFFFFEull) return cudaErrorInvalidValue;
    note_launches();
    k_parse_chunk_scan<<<1, CHUNK_SCAN_THREADS, 0, s>>>(tile_toks + tile_lo, tile_lines + tile_lo,
                                                       (uint32_t)(tile_hi - tile_lo), carry, (uint32_t)k);
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
