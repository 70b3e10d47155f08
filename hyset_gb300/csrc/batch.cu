// batch.cu — many independent joins in one persistent, work-stealing launch.
//
// The device-resident form of the reference's block-pair work queue
// (src/queue.cu:142-281, moodycamel ConcurrentQueue + one GPU consumer thread):
// every join of a batch is split into work units (a batch of probes for the
// prefix-index technique, one probe for the window-enumeration techniques);
// the units of all joins form one flat range, and the warps of a single launch
// steal units from it with one atomic each.  A unit finds its join by bisection
// over the units' prefix offsets and runs that join's filter + verify with the
// join's own descriptor (collections, bound tables, index, signatures, output
// buffer), so joins of different sizes, similarity functions, thresholds and
// signature widths share one launch and balance across all 152 SMs.
#include "join_impl.cuh"

namespace hs {

namespace {

template <int W>
__device__ __forceinline__ void run_unit_words(const BatchDesc& d, uint32_t i0, uint32_t k, uint32_t* sbuf, int lane) {
    if (d.tech == TECH_FGSS) {
        fgss_batch<1, W, false, false>(d.P, i0, k, lane);  // batches index by lists
    } else {
        for (uint32_t i = i0; i < i0 + k; ++i) enum_probe<1, W, false>(d.P, d.P.p_hi - 1 - i, sbuf, lane);
    }
}

__device__ __forceinline__ void run_unit(const BatchDesc& d, uint32_t i0, uint32_t k, uint32_t* sbuf, int lane) {
    switch (d.words) {
    case 1: run_unit_words<1>(d, i0, k, sbuf, lane); break;
    case 2: run_unit_words<2>(d, i0, k, sbuf, lane); break;
    case 4: run_unit_words<4>(d, i0, k, sbuf, lane); break;
    case 8: run_unit_words<8>(d, i0, k, sbuf, lane); break;
    default: run_unit_words<0>(d, i0, k, sbuf, lane); break;
    }
}

__global__ void __launch_bounds__(JOIN_THREADS, HS_JOIN_MIN_BLOCKS) k_batch_join(const BatchDesc* __restrict__ D,
                                                            const uint32_t* __restrict__ unit_off, uint32_t n_joins,
                                                            unsigned int* work) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* sbuf = smem + warp * MAXP;
    const uint32_t total = unit_off[n_joins];
    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(work, 1u);
        u = __shfl_sync(FULL, u, 0);
        if (u >= total) break;
        uint32_t lo = 0, hi = n_joins;  // the join: largest j with unit_off[j] <= u
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (unit_off[mid] <= u) lo = mid;
            else hi = mid;
        }
        const BatchDesc& d = D[lo];
        const uint32_t nprobe = d.P.p_hi - d.P.p_lo;
        const uint32_t i0 = (u - unit_off[lo]) * d.unit_probes;
        const uint32_t k = min(d.unit_probes, nprobe - i0);
        run_unit(d, i0, k, sbuf, lane);
    }
}

}  // namespace

cudaError_t launch_batch_join(const BatchDesc* d_desc, const uint32_t* d_unit_off, uint32_t n_joins,
                              unsigned int* d_work, int sm_count, cudaStream_t s) {
    if (n_joins == 0) return cudaSuccess;
    note_launches();
    const size_t smem = JOIN_WARPS * MAXP * sizeof(uint32_t);
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_join, JOIN_THREADS, smem);
    if (e != cudaSuccess) return e;
    k_batch_join<<<sm_count * (per_sm ? per_sm : 1), JOIN_THREADS, smem, s>>>(d_desc, d_unit_off, n_joins, d_work);
    return cudaGetLastError();
}

}  // namespace hs
