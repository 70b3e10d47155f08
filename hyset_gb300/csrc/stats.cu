// stats.cu — collection statistics for the technique selector.
//
// The reference's statistics::extract (include/hyset/statistics.hpp:163-213)
// computes, with thrust::transform_reduce over device arrays, the mean and
// standard deviation of the set sizes of a partition and the standard
// deviation of the token histogram of its prefix entries.  Here: one block-
// reduced pass over the sizes (sum, sum of squares, max) and one over a token
// histogram (sum, sum of squares, max, non-zero count), both with 64-bit
// integer accumulators, so the moments are exact.
#include "kernels.h"

namespace hs {

namespace {

__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

__device__ __forceinline__ unsigned long long warp_max64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long y = __shfl_xor_sync(FULL, v, o);
        v = y > v ? y : v;
    }
    return v;
}

// out[0] += sum, out[1] += sum of squares, out[2] = max, out[3] += non-zero count
__global__ void k_moments(const uint32_t* __restrict__ v, uint64_t n, unsigned long long* out) {
    unsigned long long s = 0, q = 0, mx = 0, nz = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned long long x = v[i];
        s += x;
        q += x * x;
        mx = x > mx ? x : mx;
        nz += x != 0;
    }
    s = warp_sum64(s);
    q = warp_sum64(q);
    mx = warp_max64(mx);
    nz = warp_sum64(nz);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out + 0, s);
        atomicAdd(out + 1, q);
        atomicMax(out + 2, mx);
        atomicAdd(out + 3, nz);
    }
}

}  // namespace

cudaError_t moments_u32(const uint32_t* v, uint64_t n, unsigned long long* out4, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    note_launches();
    uint64_t g = (n + 255) / 256;
    if (g > 152u * 16u) g = 152u * 16u;
    k_moments<<<(unsigned)g, 256, 0, s>>>(v, n, out4);
    return cudaGetLastError();
}

}  // namespace hs
