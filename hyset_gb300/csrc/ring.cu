// ring.cu — the candidate ring's persistent consumer.
//
// The reference's hybrid::device_handler (include/hyset/hybrid_algorithms.hpp:
// 71-193) collects a CPU filter's candidates in a host batch, copies the batch
// with a synchronous copy and verifies it on a worker thread, one batch in
// flight.  Here the candidates stream through two rings in device memory
// (records: probe id, candidate count, first candidate position; candidate
// ids) that the host fills by asynchronous copies and publishes by raising
// the device word `tail`.  One persistent launch verifies records as they are
// published: each warp claims the next published record, verifies the probe
// against its candidates (verify_probe_list) and marks the record done; the
// contiguous prefix of done records (`head`) tells the host which ring slots
// it may fill again.  Every wait is bounded: a warp that finds no published
// record for `wait_ns` nanoseconds of the global timer gives up and the
// launch ends with RING_TIMEOUT (the host relaunches it when more records
// arrive); a raised `close` word ends it with RING_CLOSED once the published
// records are verified.
#include "kernels.h"
#include "verify_impl.cuh"

namespace hs {
namespace {

constexpr int RING_THREADS = 256;
static_assert(sizeof(RingRec) == 16, "a ring record is read as one 16-byte load");

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned long long load_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}


template <int VMODE>
__global__ void __launch_bounds__(RING_THREADS) k_ring_consume(CollView R, CollView S, BoundsView B, RingView V,
                                                               Sink out) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* sbuf = smem + warp * verify_smem_words(VMODE);
    const unsigned long long rec_mask = V.rec_cap - 1, cand_mask = V.cand_cap - 1;
    for (;;) {
        // lane 0 claims the next published record, waiting (bounded) for one
        unsigned long long c = 0;
        unsigned int code = 0;  // 0: claimed, else the exit status
        if (lane == 0) {
            const unsigned long long since = global_ns();
            unsigned int backoff = 64;
            for (;;) {
                const unsigned long long t = load_acquire(V.tail);
                c = load_acquire(V.claim);
                if (c < t) {
                    if (atomicCAS(V.claim, c, c + 1) == c) break;
                    continue;  // another warp took it: try the next one at once
                }
                if (load_acquire(V.close)) {
                    code = RING_CLOSED;
                    break;
                }
                if (global_ns() - since > V.wait_ns) {
                    code = RING_TIMEOUT;
                    break;
                }
                __nanosleep(backoff);
                backoff = min(backoff * 2, 16384u);
            }
        }
        code = __shfl_sync(FULL, code, 0);
        if (code) {
            if (lane == 0) atomicMax(V.status, code);
            return;
        }
        c = __shfl_sync(FULL, c, 0);
        // ring data is read through L2 only (ld.cg): a slot is rewritten on
        // every lap, so no stale line may be served from L1
        const uint4 rec = __ldcg(reinterpret_cast<const uint4*>(V.recs) + (c & rec_mask));
        const uint32_t* ring = V.cands;
        const unsigned long long base = (unsigned long long)rec.z | ((unsigned long long)rec.w << 32);
        verify_probe_list<VMODE, 0, MAXP>(R, S, B, nullptr, nullptr, rec.x,
                                 [ring, base, cand_mask](uint32_t k) { return __ldcg(ring + ((base + k) & cand_mask)); },
                                 rec.y, out, sbuf, lane);
        // the record is done: its pairs are written, then the flag, then the
        // contiguous prefix of done records advances past it (and past later
        // records other warps finished first)
        if (lane == 0) {
            __threadfence();
            atomicExch(V.done + (c & rec_mask), c + 1);
            __threadfence();
            unsigned long long h = atomicAdd(V.head, 0ull);
            while (atomicAdd(V.done + (h & rec_mask), 0ull) == h + 1) {
                const unsigned long long prev = atomicCAS(V.head, h, h + 1);
                h = prev == h ? h + 1 : prev;
            }
        }
        __syncwarp();
    }
}

__global__ void k_ring_store(unsigned long long* word, unsigned long long value) { *word = value; }

}  // namespace

cudaError_t launch_ring_consumer(CollView R, CollView S, BoundsView B, const RingView& V, int vmode, Sink out,
                                 int sm_count, cudaStream_t s) {
    note_launches();
    const size_t smem = (RING_THREADS / 32) * verify_smem_words(vmode) * sizeof(uint32_t);
    // one block per SM: room is left for other work on the device while the
    // consumer waits for the producer
    if (vmode == 2)
        k_ring_consume<2><<<sm_count, RING_THREADS, smem, s>>>(R, S, B, V, out);
    else
        k_ring_consume<3><<<sm_count, RING_THREADS, smem, s>>>(R, S, B, V, out);
    return cudaGetLastError();
}

cudaError_t ring_store(unsigned long long* word, unsigned long long value, cudaStream_t s) {
    note_launches();
    k_ring_store<<<1, 1, 0, s>>>(word, value);
    return cudaGetLastError();
}

}  // namespace hs
