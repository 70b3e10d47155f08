// noalloc.cu — candidate verification that allocates no memory.
//
// Some callers of this library cannot allocate device memory at the moment
// they need a join step: a host engine that owns every byte of GPU memory
// through its own pool (a database or serving process that sizes its pool at
// start-up and forbids allocations afterwards), or a latency-critical path
// where cudaMalloc's implicit device synchronisation is not acceptable.
// hyset_verify_candidates_noalloc serves them: the caller passes device inputs
// and outputs, and the kernel's scratch (work counter, pair counter,
// minoverlap table) lives in one file-scope __device__ array.  The call
// enqueues a set-up kernel, the verification kernel and two device-to-device
// copies on the caller's stream; it never waits for the stream.
//
// The array is HYSET_NOALLOC_SCRATCH_BYTES (64 KiB); every GPU that loads the
// library holds it until the process exits.  All calls share it and it keeps
// the last call's contents: each call's set-up kernel clears the counters and
// rewrites the table first, so calls that overlap on the GPU (different
// streams, or different host threads without ordering) race on it and must be
// serialised by the caller.
#include <cstddef>
#include <mutex>

#include "../../include/hyset_gb300.h"
#include "common.cuh"

namespace hs {
namespace {

constexpr uint32_t NOALLOC_MAX_LEN = HYSET_NOALLOC_MAX_SET_SIZE;  // longest set the table covers
constexpr size_t TABLE_OFFSET = 256;        // counters live below, the table above

struct ScratchHeader {
    unsigned long long count;
    unsigned int work;
    unsigned int skipped;  // pairs whose sets exceed the table (guard; zero when the caller's bound holds)
};

static_assert(TABLE_OFFSET + (2 * NOALLOC_MAX_LEN + 1) * sizeof(uint32_t) <= HYSET_NOALLOC_SCRATCH_BYTES,
              "minoverlap table does not fit the no-alloc scratch array");

static __device__ __align__(256) unsigned char g_noalloc_scratch[HYSET_NOALLOC_SCRATCH_BYTES];

// The same two-phase verification as the library's candidate verifier
// (hybrid::kernels::scenario_1/2, include/hyset/hybrid_kernels.hpp:14-165),
// reading starts[]/sizes[] directly and the minoverlap table from scratch.
template <int VMODE>
__global__ void __launch_bounds__(256) k_verify_noalloc(
    const uint32_t* __restrict__ r_tokens, const uint32_t* __restrict__ r_starts, const uint32_t* __restrict__ r_sizes,
    const uint32_t* __restrict__ s_tokens, const uint32_t* __restrict__ s_starts, const uint32_t* __restrict__ s_sizes,
    const uint32_t* __restrict__ probes, const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ cands,
    uint32_t n_probes, uint32_t max_len, uint2* pairs, unsigned long long cap, unsigned char* scratch) {
    ScratchHeader* hdr = reinterpret_cast<ScratchHeader*>(scratch);
    const uint32_t* mo_sum = reinterpret_cast<const uint32_t*>(scratch + TABLE_OFFSET);
    const Sink out{pairs, &hdr->count, cap, 0};
    const int lane = threadIdx.x & 31;
    for (;;) {
        uint32_t i = 0;
        if (lane == 0) i = atomicAdd(&hdr->work, 1u);
        i = __shfl_sync(FULL, i, 0);
        if (i >= n_probes) break;
        const uint32_t p = probes[i];
        const uint32_t lp = s_sizes[p];
        const uint32_t* a = s_tokens + s_starts[p];
        const uint32_t cb = i ? offsets[i - 1] : 0, ce = offsets[i];
        for (uint32_t k0 = cb; k0 < ce; k0 += 32) {
            const uint32_t k = k0 + lane;
            bool keep = k < ce;
            uint32_t c = 0, lc = 0, mo = 0, cs = 0;
            if (keep) {
                c = cands[k];
                lc = r_sizes[c];
                cs = r_starts[c];
                if (lp > max_len || lc > max_len) {  // beyond the table this call wrote
                    atomicAdd(&hdr->skipped, 1u);
                    keep = false;
                } else {
                    // generic_similarity::minoverlap (similarity.hpp:21-23) for any pair
                    mo = min(min(lp, lc), mo_sum[lp + lc]);
                }
            }
            if constexpr (VMODE == 1) {
                const bool ok = keep && verify_serial(a, lp, r_tokens + cs, lc, mo, NOWN);
                emit(out, ok, p, c, lane);
            } else {
                unsigned m = __ballot_sync(FULL, keep);
                while (m) {
                    const int src = __ffs(m) - 1;
                    m &= m - 1;
                    const uint32_t cc = __shfl_sync(FULL, c, src), c2 = __shfl_sync(FULL, cs, src);
                    const uint32_t ll = __shfl_sync(FULL, lc, src), mm = __shfl_sync(FULL, mo, src);
                    const bool ok = verify_warp(a, lp, r_tokens + c2, ll, mm, NOWN, lane);
                    emit(out, ok && lane == 0, p, cc, lane);
                }
            }
        }
    }
}

// Set-up of one call: clears the counters and writes the raw minoverlap by
// |a| + |b| for sums 0..entries-1.  The reference's double expression
// (include/hyset/similarity.hpp:40-42, jaccard: ceil(sum * t / (1 + t)); dice
// in the same style: ceil(t * sum / 2)) is evaluated with explicitly rounded
// IEEE operations, so no multiply-add contraction can change a value: each
// entry is the double the host computes.
__global__ void __launch_bounds__(256) k_noalloc_setup(unsigned char* scratch, uint32_t entries, int sim, double t) {
    ScratchHeader* hdr = reinterpret_cast<ScratchHeader*>(scratch);
    uint32_t* mo_sum = reinterpret_cast<uint32_t*>(scratch + TABLE_OFFSET);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        hdr->count = 0;
        hdr->work = 0;
        hdr->skipped = 0;
    }
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < entries; k += gridDim.x * blockDim.x) {
        const double sum = (double)k;
        const double v = sim == SIM_DICE ? __ddiv_rn(__dmul_rn(t, sum), 2.0)
                                         : __ddiv_rn(__dmul_rn(sum, t), __dadd_rn(1.0, t));
        mo_sum[k] = (uint32_t)ceil(v);
    }
}

// Device address of g_noalloc_scratch per device, looked up once per device
// (with that device current) on the first call made on it.
std::mutex g_mu;
void* g_scratch_ptr[64];

hyset_status scratch_for_current_device(void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return HYSET_E_NODEVICE;
    if (dev >= 64) return HYSET_E_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return HYSET_E_CUDA;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return HYSET_OK;
}

}  // namespace
}  // namespace hs

extern "C" hyset_status hyset_verify_candidates_noalloc(
    const uint32_t* d_r_tokens, const uint32_t* d_r_starts, const uint32_t* d_r_sizes,
    const uint32_t* d_s_tokens, const uint32_t* d_s_starts, const uint32_t* d_s_sizes, uint32_t max_set_size,
    const uint32_t* d_probes, const uint32_t* d_offsets, const uint32_t* d_candidates, uint32_t n_probes,
    hyset_sim sim, double threshold, uint32_t scenario, hyset_pair* d_pairs, uint64_t pair_capacity,
    unsigned long long* d_count, unsigned int* d_skipped, void* stream) {
    using namespace hs;
    if (!d_count || (n_probes && (!d_r_tokens || !d_r_starts || !d_r_sizes || !d_s_tokens || !d_s_starts ||
                                  !d_s_sizes || !d_probes || !d_offsets || !d_candidates)))
        return HYSET_E_INVALID;
    if (pair_capacity && !d_pairs) return HYSET_E_INVALID;
    if (!(threshold > 0.0 && threshold <= 1.0)) return HYSET_E_INVALID;
    if (scenario != 1 && scenario != 2) return HYSET_E_INVALID;
    if (sim != HYSET_JACCARD && sim != HYSET_DICE) return HYSET_E_UNSUPPORTED;  // cosine needs a 2-D table
    if (max_set_size > NOALLOC_MAX_LEN) return HYSET_E_UNSUPPORTED;             // beyond the scratch table
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void* scratch = nullptr;
    hyset_status st = scratch_for_current_device(&scratch);
    if (st != HYSET_OK) return st;
    // counters cleared and the minoverlap table for lengths <= max_set_size
    // written by a set-up kernel on the same stream (no host copy)
    unsigned char* base = static_cast<unsigned char*>(scratch);
    const uint32_t entries = 2 * max_set_size + 1;
    k_noalloc_setup<<<(entries + 255) / 256, 256, 0, s>>>(base, entries, (int)sim, threshold);
    if (cudaGetLastError() != cudaSuccess) return HYSET_E_CUDA;
    if (n_probes) {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return HYSET_E_CUDA;
        const unsigned grid = (unsigned)(sms * 4);
        uint2* pairs = reinterpret_cast<uint2*>(d_pairs);
        if (scenario == 1)
            k_verify_noalloc<1><<<grid, 256, 0, s>>>(d_r_tokens, d_r_starts, d_r_sizes, d_s_tokens, d_s_starts,
                                                     d_s_sizes, d_probes, d_offsets, d_candidates, n_probes, max_set_size,
                                                     pairs, pair_capacity, base);
        else
            k_verify_noalloc<2><<<grid, 256, 0, s>>>(d_r_tokens, d_r_starts, d_r_sizes, d_s_tokens, d_s_starts,
                                                     d_s_sizes, d_probes, d_offsets, d_candidates, n_probes, max_set_size,
                                                     pairs, pair_capacity, base);
        if (cudaGetLastError() != cudaSuccess) return HYSET_E_CUDA;
    }
    if (cudaMemcpyAsync(d_count, base, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return HYSET_E_CUDA;
    if (d_skipped &&
        cudaMemcpyAsync(d_skipped, base + offsetof(ScratchHeader, skipped), sizeof(unsigned int),
                        cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return HYSET_E_CUDA;
    return HYSET_OK;
}
