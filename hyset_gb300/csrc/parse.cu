// parse.cu — the reference's collection text format parsed on the GPU.
//
// hyset::collection::read_collection (include/hyset/collection.hpp:93-177)
// reads one set per line with std::getline, skips empty lines and splits each
// line on single spaces (split, collection.hpp:16-24: std::getline with ' '
// and atoi per item); sets arrive sorted by size with ascending tokens.  Here
// the text sits in device memory and two passes over 4 KiB tiles turn it into
// the CSR arrays:
//   pass 1  per tile: count token starts and line starts, check the bytes;
//   scan    exclusive scans of the tile counts give every tile its first
//           token and first line;
//   pass 2  per tile: a block scan of the per-thread counts places every token
//           and line; each token start parses its digits (reading past the
//           tile when a number crosses it) and writes its value; each line
//           start records the index of its first token.
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

__device__ __forceinline__ bool is_digit(uint32_t c) { return c - '0' < 10u; }

// Byte i of the text, '\n' outside [0, n).
__device__ __forceinline__ uint32_t byte_at(const uint8_t* t, uint64_t n, int64_t i) {
    return (i >= 0 && (uint64_t)i < n) ? t[i] : (uint32_t)'\n';
}

struct Chunk {
    uint32_t b[PARSE_BYTES + 2];  // b[0] = byte before the chunk, b[17] = byte after it
};

__device__ __forceinline__ void load_chunk(const uint8_t* t, uint64_t n, uint64_t base, Chunk& c) {
    c.b[0] = byte_at(t, n, (int64_t)base - 1);
    if (base + PARSE_BYTES <= n) {
        const uint4 v = *reinterpret_cast<const uint4*>(t + base);  // base is a multiple of 16
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int k = 0; k < PARSE_BYTES; ++k) c.b[1 + k] = (w[k >> 2] >> (8 * (k & 3))) & 0xFFu;
    } else {
#pragma unroll
        for (int k = 0; k < PARSE_BYTES; ++k) c.b[1 + k] = byte_at(t, n, (int64_t)(base + k));
    }
    c.b[PARSE_BYTES + 1] = byte_at(t, n, (int64_t)(base + PARSE_BYTES));
}

// Token starts and line starts in the chunk; error bits and the first bad
// offset go to err.
__device__ __forceinline__ void chunk_counts(const Chunk& c, uint64_t base, uint64_t n, uint32_t& toks,
                                             uint32_t& lines, uint32_t& err, uint64_t& err_at) {
    toks = lines = err = 0;
    err_at = ~0ull;
#pragma unroll
    for (int k = 1; k <= PARSE_BYTES; ++k) {
        if (base + k - 1 >= n) break;
        const uint32_t prev = c.b[k - 1], x = c.b[k], next = c.b[k + 1];
        const bool at_line_start = prev == '\n';
        uint32_t e = 0;
        if (is_digit(x)) {
            toks += (prev == ' ' || at_line_start) ? 1u : 0u;
        } else if (x == ' ') {
            if (prev == ' ' || at_line_start || next == '\r') e |= PARSE_E_EMPTY_ITEM;
        } else if (x == '\r') {
            if (next != '\n' || at_line_start) e |= PARSE_E_LINE_END;
        } else if (x != '\n') {
            e |= PARSE_E_CHAR;
        }
        lines += (at_line_start && x != '\n') ? 1u : 0u;
        if (e) {
            err |= e;
            const uint64_t at = base + k - 1;
            err_at = at < err_at ? at : err_at;
        }
    }
}

__device__ __forceinline__ void record_error(uint32_t err, uint64_t err_at, uint32_t* flags,
                                             unsigned long long* first_bad) {
    if (err) {
        atomicOr(flags, err);
        atomicMin(first_bad, (unsigned long long)err_at);
    }
}

__global__ void __launch_bounds__(PARSE_THREADS) k_parse_count(const uint8_t* __restrict__ t, uint64_t n,
                                                               uint32_t* tile_toks, uint32_t* tile_lines,
                                                               uint32_t* flags, unsigned long long* first_bad) {
    __shared__ uint32_t red[2][PARSE_THREADS / 32];
    const uint64_t tile = blockIdx.x;
    const uint64_t base = tile * PARSE_TILE + (uint64_t)threadIdx.x * PARSE_BYTES;
    Chunk c;
    load_chunk(t, n, base, c);
    uint32_t toks, lines, err;
    uint64_t err_at;
    chunk_counts(c, base, n, toks, lines, err, err_at);
    record_error(err, err_at, flags, first_bad);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    toks = __reduce_add_sync(FULL, toks);
    lines = __reduce_add_sync(FULL, lines);
    if (lane == 0) {
        red[0][warp] = toks;
        red[1][warp] = lines;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t a = 0, b = 0;
        for (int w = 0; w < PARSE_THREADS / 32; ++w) {
            a += red[0][w];
            b += red[1][w];
        }
        tile_toks[tile] = a;
        tile_lines[tile] = b;
    }
}

// Parses the number starting at byte i (at most 10 digits, value < 2^32).
__device__ __forceinline__ bool parse_number(const uint8_t* t, uint64_t n, uint64_t i, uint32_t& value) {
    uint64_t v = 0;
    int d = 0;
    while (i < n) {
        const uint32_t ch = t[i];
        if (!is_digit(ch)) break;
        v = v * 10u + (ch - '0');
        ++i;
        if (++d > 10) return false;
    }
    value = (uint32_t)v;
    return v <= 0xFFFFFFFFull;
}

__global__ void __launch_bounds__(PARSE_THREADS) k_parse_emit(const uint8_t* __restrict__ t, uint64_t n,
                                                              const uint32_t* __restrict__ tile_tok0,
                                                              const uint32_t* __restrict__ tile_line0,
                                                              uint32_t* __restrict__ tokens,
                                                              uint32_t* __restrict__ line_tok0, uint32_t* flags,
                                                              unsigned long long* first_bad) {
    __shared__ uint32_t wsum[2][PARSE_THREADS / 32];
    const uint64_t tile = blockIdx.x;
    const uint64_t base = tile * PARSE_TILE + (uint64_t)threadIdx.x * PARSE_BYTES;
    Chunk c;
    load_chunk(t, n, base, c);
    uint32_t toks, lines, err;
    uint64_t err_at;
    chunk_counts(c, base, n, toks, lines, err, err_at);
    // block-wide exclusive scan of (toks, lines)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t ti = warp_incl_scan(toks, lane), li = warp_incl_scan(lines, lane);
    if (lane == 31) {
        wsum[0][warp] = ti;
        wsum[1][warp] = li;
    }
    __syncthreads();
    uint32_t tw = 0, lw = 0;
    for (int w = 0; w < warp; ++w) {
        tw += wsum[0][w];
        lw += wsum[1][w];
    }
    uint32_t tok = tile_tok0[tile] + tw + ti - toks;
    uint32_t line = tile_line0[tile] + lw + li - lines;
    uint32_t bad = 0;
    uint64_t bad_at = ~0ull;
#pragma unroll
    for (int k = 1; k <= PARSE_BYTES; ++k) {
        if (base + k - 1 >= n) break;
        const uint32_t prev = c.b[k - 1], x = c.b[k];
        if (prev == '\n' && x != '\n') line_tok0[line++] = tok;
        if (is_digit(x) && (prev == ' ' || prev == '\n')) {
            uint32_t v = 0;
            if (!parse_number(t, n, base + k - 1, v)) {
                bad |= PARSE_E_RANGE;
                const uint64_t at = base + k - 1;
                bad_at = at < bad_at ? at : bad_at;
            }
            tokens[tok++] = v;
        }
    }
    record_error(bad, bad_at, flags, first_bad);
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
                        uint32_t* flags, unsigned long long* first_bad, cudaStream_t s) {
    const uint64_t tiles = parse_tiles(n_bytes);
    if (tiles == 0) return cudaSuccess;
    if (tiles > 0x7FFFFFFFull) return cudaErrorInvalidValue;
    note_launches();
    k_parse_count<<<(unsigned)tiles, PARSE_THREADS, 0, s>>>(text, n_bytes, tile_toks, tile_lines, flags, first_bad);
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
