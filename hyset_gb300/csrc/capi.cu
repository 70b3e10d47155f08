// capi.cu — the C ABI's contexts and results (include/hyset_gb300.h), and the
// library's error recording.  The other entry points live beside the code
// they drive: collection.cu, join_host.cu, pipeline.cu, batch_host.cu,
// plan.cu, handlers.cu, verifier.cu, noalloc.cu.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "host.h"

namespace hs {

namespace {
std::atomic<long long> g_device_bytes{0};
std::mutex g_fault_mu;
std::string g_fault_value;  // the HYSET_FAULT_ALLOC value the count started from
long long g_fault_count = 0;
}  // namespace

unsigned long long device_bytes() { return (unsigned long long)g_device_bytes.load(); }
void add_device_bytes(long long delta) { g_device_bytes += delta; }

bool inject_alloc_failure() {
    const char* v = std::getenv("HYSET_FAULT_ALLOC");
    if (!v || !*v) return false;
    std::lock_guard<std::mutex> lock(g_fault_mu);
    if (g_fault_value != v) {
        g_fault_value = v;
        g_fault_count = 0;
    }
    return ++g_fault_count == std::atoll(v);
}

hyset_status fail(hyset_ctx* ctx, hyset_status st, const char* what, cudaError_t e) {
    if (ctx) {
        char buf[512];
        if (e != cudaSuccess)
            std::snprintf(buf, sizeof buf, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
        else
            std::snprintf(buf, sizeof buf, "%s", what);
        ctx->err = buf;
    }
    return st;
}

}  // namespace hs

using namespace hs;

extern "C" {

void hyset_default_opts(hyset_join_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->sim = HYSET_JACCARD;
    o->threshold = 0.8;
    o->technique = HYSET_TECH_AUTO;
}

hyset_status hyset_create(int device, hyset_ctx** out) {
    if (!out) return HYSET_E_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return HYSET_E_NODEVICE;
    }
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return HYSET_E_NODEVICE;
    if (device >= count) return HYSET_E_INVALID;
    hyset_ctx* ctx = new (std::nothrow) hyset_ctx();
    if (!ctx) return HYSET_E_NOMEM;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = prepare_kernels();
    // The auxiliary stream runs work beside the critical path (signatures
    // during the index build): its blocks yield to the context stream's.
    int prio_lo = 0, prio_hi = 0;
    if (e == cudaSuccess && HS_STREAM_PRIO) e = cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, prio_hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&ctx->aux, cudaStreamNonBlocking, prio_lo);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ek0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ek1);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&ctx->h_flags, 64);
    if (e == cudaSuccess) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    if (e != cudaSuccess) {
        hyset_destroy(ctx);
        return HYSET_E_CUDA;
    }
    *out = ctx;
    return HYSET_OK;
}

void hyset_destroy(hyset_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) {
        cudaStream_t s = ctx->stream;
        batch_release(ctx);
        for (auto& kv : ctx->bounds) kv.second->dev.release(s);
        ctx->own.release(s);
        DevBuf* bufs[] = {&ctx->s_pairs, &ctx->s_count, &ctx->s_work, &ctx->s_stats, &ctx->s_flags,
                          &ctx->d_mlp, &ctx->d_feat, &ctx->d_moments, &ctx->d_hist, &ctx->d_width_mlp};
        for (DevBuf* b : bufs) b->release(s);
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    if (ctx->aux) {
        cudaStreamSynchronize(ctx->aux);
        cudaStreamDestroy(ctx->aux);
    }
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    for (cudaEvent_t e : ctx->pipe_ev) cudaEventDestroy(e);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->ek0) cudaEventDestroy(ctx->ek0);
    if (ctx->ek1) cudaEventDestroy(ctx->ek1);
    if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    delete ctx;
}

const char* hyset_last_error(const hyset_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

uint64_t hyset_device_bytes(void) { return device_bytes(); }

uint64_t hyset_result_count(const hyset_result* r) { return r ? r->count : 0; }
const hyset_pair* hyset_result_pairs(const hyset_result* r) {
    static const hyset_pair none = {0, 0};
    if (!r || !r->has_pairs) return nullptr;
    return r->pairs.empty() ? &none : r->pairs.data();
}
uint64_t hyset_result_launches(const hyset_result* r) { return r ? r->launches : 0; }
hyset_technique hyset_result_technique(const hyset_result* r) { return r ? r->technique : HYSET_TECH_AUTO; }
uint32_t hyset_result_bitmap_bits(const hyset_result* r) { return r ? r->bitmap_bits : 0; }
uint32_t hyset_result_verify_mode(const hyset_result* r) { return r ? r->verify_mode : 0; }
uint32_t hyset_result_probe_batch(const hyset_result* r) { return r ? r->probe_batch : 0; }
uint32_t hyset_result_split(const hyset_result* r, hyset_technique* low_technique) {
    if (low_technique) *low_technique = r ? r->split_low : HYSET_TECH_AUTO;
    return r ? r->split_at : 0;
}
double hyset_result_device_ms(const hyset_result* r) { return r ? r->device_ms : 0.0; }
double hyset_result_kernel_ms(const hyset_result* r) { return r ? r->kernel_ms : 0.0; }
const void* hyset_result_device_pairs(const hyset_result* r) { return r ? r->device_pairs : nullptr; }
uint32_t hyset_result_stats(const hyset_result* r, uint64_t* out, uint32_t n) {
    if (!r || !out) return 0;
    uint32_t k = n < 8 ? n : 8;
    for (uint32_t i = 0; i < k; ++i) out[i] = r->stats[i];
    return k;
}
void hyset_result_free(hyset_result* r) { delete r; }

}  // extern "C"
