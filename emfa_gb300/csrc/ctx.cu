// Context, status strings and HBM-budget accounting of libemfa_cuda.
#include "emfa_internal.cuh"

#include <cstdio>
#include <cstring>

namespace emfa {

// Process-wide error state, never destroyed: entry points may run from
// interpreter or static teardown, after ordinary statics are gone.
static std::mutex& err_mu()
{
    static std::mutex* m = new std::mutex;
    return *m;
}
static std::string& last_error_global()
{
    static std::string* s = new std::string;
    return *s;
}

void set_global_error(const std::string& msg)
{
    std::lock_guard<std::mutex> g(err_mu());
    last_error_global() = msg;
}

void set_error(Ctx* ctx, const std::string& msg)
{
    if (ctx) {
        std::lock_guard<std::mutex> g(ctx->mu);
        ctx->last_error = msg;
    }
    set_global_error(msg);
}

emfa_status_t ensure_smem_raw(Ctx* c, const void* func, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> limit;
    int dev = c ? c->device : 0;
    if (!c) EMFA_CUDA(c, cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(mu);
    size_t& cur = limit[std::make_pair(func, dev)];
    if (cur >= bytes) return EMFA_OK;
    EMFA_CUDA(c, cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
    return EMFA_OK;
}

emfa_status_t ctx_alloc(Ctx* c, size_t bytes, void** p)
{
    {
        std::lock_guard<std::mutex> g(c->mu);
        if (c->budget && c->used + bytes > c->budget) {
            char buf[160];
            std::snprintf(buf, sizeof buf, "HBM budget exceeded: %zu B held + %zu B requested > %zu B budget",
                          c->used, bytes, c->budget);
            c->last_error = buf;
            set_global_error(buf);
            return EMFA_ERR_OOM;
        }
        c->used += bytes;
        if (c->used > c->peak) c->peak = c->used;
    }
    cudaError_t e = !c->stream_ordered ? cudaMalloc(p, bytes)
                    : c->pool           ? cudaMallocFromPoolAsync(p, bytes, c->pool, c->stream)
                                        : cudaMallocAsync(p, bytes, c->stream);
    if (e != cudaSuccess) {
        std::lock_guard<std::mutex> g(c->mu);
        c->used -= bytes;
        c->last_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        set_global_error(c->last_error);
        *p = nullptr;
        return e == cudaErrorMemoryAllocation ? EMFA_ERR_OOM : EMFA_ERR_CUDA;
    }
    return EMFA_OK;
}

TimedLaunch::TimedLaunch(Ctx* c, int id, cudaStream_t st, double work) : c_(c), st_(st)
{
    if (!c || !c->time_kernels) return;
    std::lock_guard<std::mutex> g(c->mu);
    KernelTimer& t = c->timers[id];
    if (t.used == t.start.size()) {
        cudaEvent_t a = nullptr, b = nullptr;
        if (cudaEventCreate(&a) != cudaSuccess) return;
        if (cudaEventCreate(&b) != cudaSuccess) {
            cudaEventDestroy(a);
            return;
        }
        t.start.push_back(a);
        t.stop.push_back(b);
    }
    if (cudaEventRecord(t.start[t.used], st) != cudaSuccess) return;
    stop_ = t.stop[t.used];
    t.used += 1;
    t.work += work;
}

TimedLaunch::~TimedLaunch()
{
    if (stop_) cudaEventRecord(stop_, st_);
}

namespace {
std::mutex& refs_mutex()
{
    static std::mutex m;
    return m;
}
}  // namespace

void ctx_retain(Ctx* c)
{
    std::lock_guard<std::mutex> g(refs_mutex());
    c->refs += 1;
}

void ctx_release(Ctx* c)
{
    {
        std::lock_guard<std::mutex> g(refs_mutex());
        if (--c->refs > 0) return;
    }
    cudaSetDevice(c->device);
    if (c->stream) {
        cudaStreamSynchronize(c->stream);
        cudaStreamDestroy(c->stream);
    }
    for (auto& t : c->timers) {
        for (auto e : t.start) cudaEventDestroy(e);
        for (auto e : t.stop) cudaEventDestroy(e);
    }
    if (c->pinned) cudaFreeHost(c->pinned);
    delete static_cast<emfa_ctx_t*>(c);
}

emfa_status_t ctx_workspace(Ctx* c, int slot, size_t bytes, void** p)
{
    DevBuf& b = c->ws[slot];
    if (b.bytes < bytes) {
        if (b.ptr) cudaDeviceSynchronize();  // the old buffer may still be in use
        EMFA_TRY(b.alloc(c, bytes));
    }
    *p = b.ptr;
    return EMFA_OK;
}

void ctx_free(Ctx* c, void* p, size_t bytes)
{
    if (!p) return;
    if (c->stream_ordered)
        cudaFreeAsync(p, c->stream);
    else
        cudaFree(p);
    std::lock_guard<std::mutex> g(c->mu);
    c->used -= bytes;
}

}  // namespace emfa

using namespace emfa;

extern "C" {

const char* emfa_status_string(emfa_status_t s)
{
    switch (s) {
        case EMFA_OK: return "ok";
        case EMFA_ERR_INVALID: return "invalid argument";
        case EMFA_ERR_CUDA: return "CUDA error";
        case EMFA_ERR_OOM: return "out of device memory / HBM budget";
        case EMFA_ERR_NOT_CONVERGED: return "iteration did not converge";
        case EMFA_ERR_MESH: return "mesh error";
        case EMFA_ERR_UNSUPPORTED: return "unsupported";
        case EMFA_ERR_TIMEOUT: return "device wait timed out";
    }
    return "unknown status";
}

const char* emfa_last_error(const emfa_ctx_t* ctx)
{
    if (ctx) return ctx->last_error.c_str();
    return last_error_global().c_str();
}

const char* emfa_version(void) { return "emfa_gb300 0.1 (sm_103a)"; }

emfa_status_t emfa_ctx_create(int device, size_t hbm_budget_bytes, emfa_ctx_t** out)
{
    if (!out) return EMFA_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        set_global_error(std::string("no CUDA device: ") + cudaGetErrorString(e));
        return EMFA_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) {
        set_global_error("device index out of range");
        return EMFA_ERR_INVALID;
    }
    e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        set_global_error(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
        return EMFA_ERR_CUDA;
    }
    emfa_ctx_t* c = new emfa_ctx_t();
    c->device = device;
    c->budget = hbm_budget_bytes;
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        set_global_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
        delete c;
        return EMFA_ERR_CUDA;
    }
    e = cudaHostAlloc((void**)&c->pinned, 64 * sizeof(int), cudaHostAllocDefault);
    if (e != cudaSuccess) {
        set_global_error(std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
        cudaStreamDestroy(c->stream);
        delete c;
        return EMFA_ERR_CUDA;
    }
    *out = c;
    return EMFA_OK;
}

emfa_status_t emfa_ctx_destroy(emfa_ctx_t* ctx)
{
    if (!ctx) return EMFA_ERR_INVALID;
    cudaSetDevice(ctx->device);
    // the context's own buffers now (stream-ordered ones are freed on its
    // stream); the stream and the struct when no geometry or operator holds it
    for (auto& b : ctx->ws) b.release();
    for (auto& kv : ctx->user_bufs) ctx_free(ctx, kv.first, kv.second);
    ctx->user_bufs.clear();
    ctx_release(ctx);
    return EMFA_OK;
}

emfa_status_t emfa_ctx_memory(const emfa_ctx_t* ctx, size_t* used, size_t* peak, size_t* budget)
{
    if (!ctx) return EMFA_ERR_INVALID;
    if (used) *used = ctx->used;
    if (peak) *peak = ctx->peak;
    if (budget) *budget = ctx->budget;
    return EMFA_OK;
}

emfa_status_t emfa_ctx_launch_count(const emfa_ctx_t* ctx, int64_t* count)
{
    if (!ctx || !count) return EMFA_ERR_INVALID;
    *count = (int64_t)ctx->kernel_launches;
    return EMFA_OK;
}

emfa_status_t emfa_ctx_set_kernel_timing(emfa_ctx_t* ctx, int on)
{
    if (!ctx) return EMFA_ERR_INVALID;
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->time_kernels = on != 0;
    for (auto& t : ctx->timers) {
        t.used = 0;
        t.work = 0.0;
    }
    return EMFA_OK;
}

emfa_status_t emfa_ctx_kernel_time(emfa_ctx_t* ctx, int kernel, int64_t* launches, double* total_ms, double* work)
{
    if (!ctx || kernel < 0 || kernel >= KT_COUNT || !launches || !total_ms) return EMFA_ERR_INVALID;
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    std::lock_guard<std::mutex> g(ctx->mu);
    const KernelTimer& t = ctx->timers[kernel];
    double sum = 0.0;
    for (size_t i = 0; i < t.used; ++i) {
        EMFA_CUDA(ctx, cudaEventSynchronize(t.stop[i]));
        float ms = 0.f;
        EMFA_CUDA(ctx, cudaEventElapsedTime(&ms, t.start[i], t.stop[i]));
        sum += ms;
    }
    *launches = (int64_t)t.used;
    *total_ms = sum;
    if (work) *work = t.work;
    return EMFA_OK;
}

emfa_status_t emfa_ctx_synchronize(emfa_ctx_t* ctx)
{
    if (!ctx) return EMFA_ERR_INVALID;
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    EMFA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return EMFA_OK;
}

emfa_status_t emfa_device_alloc(emfa_ctx_t* ctx, size_t bytes, void** dev)
{
    if (!ctx || !dev || bytes == 0) return EMFA_ERR_INVALID;
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    EMFA_TRY(ctx_alloc(ctx, bytes, dev));
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->user_bufs[*dev] = bytes;
    return EMFA_OK;
}

emfa_status_t emfa_device_free(emfa_ctx_t* ctx, void* dev)
{
    if (!ctx || !dev) return EMFA_ERR_INVALID;
    size_t bytes = 0;
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        auto it = ctx->user_bufs.find(dev);
        if (it == ctx->user_bufs.end()) {
            ctx->last_error = "emfa_device_free: pointer not allocated by this context";
            return EMFA_ERR_INVALID;
        }
        bytes = it->second;
        ctx->user_bufs.erase(it);
    }
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    EMFA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx_free(ctx, dev, bytes);
    return EMFA_OK;
}

emfa_status_t emfa_memcpy(emfa_ctx_t* ctx, void* dst, const void* src, size_t bytes, int kind)
{
    if (!ctx || !dst || !src || kind < 0 || kind > 2) return EMFA_ERR_INVALID;
    cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice : kind == 1 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    EMFA_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, k, ctx->stream));
    EMFA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return EMFA_OK;
}

emfa_status_t emfa_ctx_stream(const emfa_ctx_t* ctx, void** stream)
{
    if (!ctx || !stream) return EMFA_ERR_INVALID;
    *stream = (void*)ctx->stream;
    return EMFA_OK;
}

}  // extern "C"
