// mlp.cu — the technique selector's FP32 network: 12 -> 64 -> 64 -> 3, ReLU.
//
// Inputs are normalised features of a join (or of one probe partition of it);
// outputs are predicted log-milliseconds of the bitmap, prefix-index (fgss) and
// direct-verify techniques.  The network is small enough that one CTA holds a
// training chunk in shared memory, so a training run is one launch: per step
// forward and masked mean-squared-error backward over the dataset in chunks of
// MLP_MAX_BATCH samples (gradients accumulated), then one Adam update.  Parameters are one flat float array:
//   W1[12][64] b1[64] W2[64][64] b2[64] W3[64][3] b3[3]   (5187 floats)
#include "kernels.h"

namespace hs {

namespace {

constexpr int F = MLP_IN, H = MLP_HIDDEN, O = MLP_OUT;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + F * H, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
              OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H * O, NPARAM = OFF_B3 + O;
static_assert(NPARAM == MLP_PARAMS, "parameter layout");

// Activations of a batch of B samples (B <= MLP_MAX_BATCH) in shared memory.
struct Act {
    float x[MLP_MAX_BATCH][F];
    float h1[MLP_MAX_BATCH][H];
    float h2[MLP_MAX_BATCH][H];
    float y[MLP_MAX_BATCH][O];
    float d2[MLP_MAX_BATCH][H];  // dL/d(h2 pre-activation)
    float d1[MLP_MAX_BATCH][H];  // dL/d(h1 pre-activation)
};

__device__ void forward(const float* __restrict__ w, Act& A, int B) {
    for (int i = threadIdx.x; i < B * H; i += blockDim.x) {
        const int b = i / H, j = i % H;
        float s = w[OFF_B1 + j];
        for (int k = 0; k < F; ++k) s += A.x[b][k] * w[OFF_W1 + k * H + j];
        A.h1[b][j] = s > 0.f ? s : 0.f;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < B * H; i += blockDim.x) {
        const int b = i / H, j = i % H;
        float s = w[OFF_B2 + j];
        for (int k = 0; k < H; ++k) s += A.h1[b][k] * w[OFF_W2 + k * H + j];
        A.h2[b][j] = s > 0.f ? s : 0.f;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < B * O; i += blockDim.x) {
        const int b = i / O, j = i % O;
        float s = w[OFF_B3 + j];
        for (int k = 0; k < H; ++k) s += A.h2[b][k] * w[OFF_W3 + k * O + j];
        A.y[b][j] = s;
    }
    __syncthreads();
}

// Loss of a chunk = sum over masked outputs of (y - t)^2 / denom, where denom
// is the number of masked outputs of the whole dataset, so chunk losses and
// gradients add up to the dataset's.  Adds dL/dparam into g (NPARAM floats)
// and returns the chunk loss.  t and m are [B][O] in global memory.
__device__ float backward(const float* __restrict__ w, Act& A, int B, const float* __restrict__ t,
                          const float* __restrict__ m, float* __restrict__ g, float* red, float denom) {
    float loss = 0.f;
    for (int i = threadIdx.x; i < B * O; i += blockDim.x) {
        const float e = A.y[i / O][i % O] - t[i];
        loss += m[i] * e * e;
    }
    red[threadIdx.x] = loss;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    const float chunk_loss = red[0] / denom;
    __syncthreads();
    // dL/dy = 2 m (y - t) / denom, kept in A.y
    for (int i = threadIdx.x; i < B * O; i += blockDim.x) {
        const int b = i / O, j = i % O;
        A.y[b][j] = 2.f * m[i] * (A.y[b][j] - t[i]) / denom;
    }
    __syncthreads();
    // layer 3 gradients and dL/dh2
    for (int i = threadIdx.x; i < H * O; i += blockDim.x) {
        const int k = i / O, j = i % O;
        float s = 0.f;
        for (int b = 0; b < B; ++b) s += A.h2[b][k] * A.y[b][j];
        g[OFF_W3 + i] += s;
    }
    for (int j = threadIdx.x; j < O; j += blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < B; ++b) s += A.y[b][j];
        g[OFF_B3 + j] += s;
    }
    for (int i = threadIdx.x; i < B * H; i += blockDim.x) {
        const int b = i / H, k = i % H;
        float s = 0.f;
        for (int j = 0; j < O; ++j) s += A.y[b][j] * w[OFF_W3 + k * O + j];
        A.d2[b][k] = A.h2[b][k] > 0.f ? s : 0.f;
    }
    __syncthreads();
    // layer 2
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) {
        const int k = i / H, j = i % H;
        float s = 0.f;
        for (int b = 0; b < B; ++b) s += A.h1[b][k] * A.d2[b][j];
        g[OFF_W2 + i] += s;
    }
    for (int j = threadIdx.x; j < H; j += blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < B; ++b) s += A.d2[b][j];
        g[OFF_B2 + j] += s;
    }
    for (int i = threadIdx.x; i < B * H; i += blockDim.x) {
        const int b = i / H, k = i % H;
        float s = 0.f;
        for (int j = 0; j < H; ++j) s += A.d2[b][j] * w[OFF_W2 + k * H + j];
        A.d1[b][k] = A.h1[b][k] > 0.f ? s : 0.f;
    }
    __syncthreads();
    // layer 1
    for (int i = threadIdx.x; i < F * H; i += blockDim.x) {
        const int k = i / H, j = i % H;
        float s = 0.f;
        for (int b = 0; b < B; ++b) s += A.x[b][k] * A.d1[b][j];
        g[OFF_W1 + i] += s;
    }
    for (int j = threadIdx.x; j < H; j += blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < B; ++b) s += A.d1[b][j];
        g[OFF_B1 + j] += s;
    }
    __syncthreads();
    return chunk_loss;
}

// Dataset loss and gradient (g overwritten) over n samples in chunks.
__device__ float dataset_grad(const float* __restrict__ w, Act& A, const float* __restrict__ x,
                              const float* __restrict__ t, const float* __restrict__ m, int n, float* __restrict__ g,
                              float* red, float denom) {
    for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) g[i] = 0.f;
    __syncthreads();
    float loss = 0.f;
    for (int base = 0; base < n; base += MLP_MAX_BATCH) {
        const int B = min(MLP_MAX_BATCH, n - base);
        for (int i = threadIdx.x; i < B * F; i += blockDim.x) A.x[i / F][i % F] = x[(size_t)base * F + i];
        __syncthreads();
        forward(w, A, B);
        loss += backward(w, A, B, t + (size_t)base * O, m + (size_t)base * O, g, red, denom);
    }
    return loss;
}

__device__ void load_x(Act& A, const float* __restrict__ x, int B) {
    for (int i = threadIdx.x; i < B * F; i += blockDim.x) A.x[i / F][i % F] = x[i];
    __syncthreads();
}

__global__ void __launch_bounds__(MLP_THREADS) k_mlp_forward(const float* __restrict__ w, const float* __restrict__ x,
                                                              int n, float* __restrict__ y) {
    extern __shared__ float smem_f[];
    Act& A = *reinterpret_cast<Act*>(smem_f);
    for (int base = blockIdx.x * MLP_MAX_BATCH; base < n; base += gridDim.x * MLP_MAX_BATCH) {
        const int B = min(MLP_MAX_BATCH, n - base);
        load_x(A, x + (size_t)base * F, B);
        forward(w, A, B);
        for (int i = threadIdx.x; i < B * O; i += blockDim.x) y[(size_t)base * O + i] = A.y[i / O][i % O];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(MLP_THREADS) k_mlp_grad(const float* __restrict__ w, const float* __restrict__ x,
                                                           const float* __restrict__ t, const float* __restrict__ m,
                                                           int n, float denom, float* __restrict__ g,
                                                           float* __restrict__ loss) {
    extern __shared__ float smem_f[];
    Act& A = *reinterpret_cast<Act*>(smem_f);
    float* red = smem_f + sizeof(Act) / sizeof(float);
    const float l = dataset_grad(w, A, x, t, m, n, g, red, denom);
    if (threadIdx.x == 0) *loss = l;
}

// `steps` full-dataset Adam steps on one CTA; w, mom, vel and g live in global memory
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_train(float* __restrict__ w, float* __restrict__ mom,
                                                            float* __restrict__ vel, float* __restrict__ g,
                                                            const float* __restrict__ x, const float* __restrict__ t,
                                                            const float* __restrict__ m, int n, float denom,
                                                            int steps, float lr, float weight_decay,
                                                            float* __restrict__ loss_trace) {
    extern __shared__ float smem_f[];
    Act& A = *reinterpret_cast<Act*>(smem_f);
    float* red = smem_f + sizeof(Act) / sizeof(float);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int step = 1; step <= steps; ++step) {
        const float l = dataset_grad(w, A, x, t, m, n, g, red, denom);
        if (threadIdx.x == 0 && loss_trace) loss_trace[step - 1] = l;
        const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
        for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) {
            const float gi = g[i] + weight_decay * w[i];
            const float mi = b1 * mom[i] + (1.f - b1) * gi;
            const float vi = b2 * vel[i] + (1.f - b2) * gi * gi;
            mom[i] = mi;
            vel[i] = vi;
            w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        }
        __syncthreads();
    }
}

}  // namespace

size_t mlp_smem_bytes() { return sizeof(Act) + 2 * MLP_THREADS * sizeof(float); }

cudaError_t mlp_forward(const float* w, const float* x, int n, float* y, int sm_count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    note_launches();
    const size_t smem = mlp_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = (n + MLP_MAX_BATCH - 1) / MLP_MAX_BATCH;
    if (blocks > sm_count) blocks = sm_count;
    k_mlp_forward<<<blocks, MLP_THREADS, smem, s>>>(w, x, n, y);
    return cudaGetLastError();
}

cudaError_t mlp_grad(const float* w, const float* x, const float* t, const float* m, int n, float denom, float* g,
                     float* loss, cudaStream_t s) {
    if (n <= 0 || !(denom > 0.f)) return cudaErrorInvalidValue;
    note_launches();
    const size_t smem = mlp_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_mlp_grad<<<1, MLP_THREADS, smem, s>>>(w, x, t, m, n, denom, g, loss);
    return cudaGetLastError();
}

cudaError_t mlp_train(float* w, float* mom, float* vel, float* g, const float* x, const float* t, const float* m,
                      int n, float denom, int steps, float lr, float weight_decay, float* loss_trace,
                      cudaStream_t s) {
    if (n <= 0 || steps < 0 || !(denom > 0.f)) return cudaErrorInvalidValue;
    note_launches();
    const size_t smem = mlp_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_mlp_train<<<1, MLP_THREADS, smem, s>>>(w, mom, vel, g, x, t, m, n, denom, steps, lr, weight_decay,
                                             loss_trace);
    return cudaGetLastError();
}

}  // namespace hs
