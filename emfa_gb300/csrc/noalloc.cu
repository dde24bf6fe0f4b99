// emfa_matvec_tf32_noalloc: the tensor-core multi-RHS product Y = Z X of
// emfa_matvec(EMFA_F32, EMFA_MV_TF32) for callers that may not allocate device
// memory during the call.
//
// Its scratch (the packed B operand and the kernel's error word) is one
// file-scope device array, reserved when this translation unit's module is
// loaded on a device.  The first call on a device (with that device current)
// looks the array's address up with cudaGetSymbolAddress and caches it; later
// calls on that device only read the cache.  Nothing here calls cudaMalloc,
// cudaFree or any library routine that allocates.
#include "emfa_internal.cuh"
#include "gemm.cuh"

#include <mutex>

namespace {

// packed B operand: 4 floats per (RHS, unknown) pair
constexpr size_t PACK_BYTES = 16u * EMFA_NOALLOC_MAX_ELEMS;
constexpr size_t ERR_BYTES = 256;  // error word, own 256-byte line after the pack

static __device__ __align__(256) unsigned char g_scratch[PACK_BYTES + ERR_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
unsigned char* g_ptr[MAX_DEVICES] = {};

// once per device, with that device current
emfa_status_t scratch_for(int dev, unsigned char** out)
{
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) {
            emfa::set_error(nullptr, std::string("emfa_matvec_tf32_noalloc: cudaGetSymbolAddress of the static "
                                                 "scratch failed: ") +
                                         cudaGetErrorString(e));
            return EMFA_ERR_CUDA;
        }
        EMFA_TRY(emfa::cgemm_tf32_prepare());
        g_ptr[dev] = (unsigned char*)p;
    }
    *out = g_ptr[dev];
    return EMFA_OK;
}

}  // namespace

extern "C" {

emfa_status_t emfa_matvec_tf32_noalloc(const void* Z_dev, int n, const void* X_dev, int n_rhs, void* Y_dev,
                                       void* stream)
{
    if (!Z_dev || !X_dev || !Y_dev || n <= 0 || n_rhs <= 0) {
        emfa::set_error(nullptr, "emfa_matvec_tf32_noalloc: bad arguments");
        return EMFA_ERR_INVALID;
    }
    if ((size_t)n * (size_t)n_rhs > EMFA_NOALLOC_MAX_ELEMS) {
        emfa::set_error(nullptr, "emfa_matvec_tf32_noalloc: n * n_rhs = " +
                                     std::to_string((size_t)n * (size_t)n_rhs) + " exceeds the static scratch limit " +
                                     std::to_string((size_t)EMFA_NOALLOC_MAX_ELEMS) +
                                     " (use emfa_matvec for larger products)");
        return EMFA_ERR_INVALID;
    }
    if (n & 1) {
        emfa::set_error(nullptr, "emfa_matvec_tf32_noalloc: n must be even (TMA row stride)");
        return EMFA_ERR_UNSUPPORTED;
    }
    int dev = -1;
    EMFA_CUDA(nullptr, cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) {
        emfa::set_error(nullptr, "emfa_matvec_tf32_noalloc: device index out of range");
        return EMFA_ERR_INVALID;
    }
    unsigned char* s = nullptr;
    EMFA_TRY(scratch_for(dev, &s));
    cudaStream_t st = (cudaStream_t)stream;
    int* err = (int*)(s + PACK_BYTES);
    // the kernel only ever raises the error word; it starts each call at zero
    EMFA_CUDA(nullptr, cudaMemsetAsync(err, 0, sizeof(int), st));
    EMFA_TRY(emfa::cgemm_tf32_scratch(Z_dev, (size_t)n, X_dev, n, n_rhs, Y_dev, s, err, st));
    int h = 0;
    EMFA_CUDA(nullptr, cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    EMFA_CUDA(nullptr, cudaStreamSynchronize(st));
    if (h) {
        emfa::set_error(nullptr, "emfa_matvec_tf32_noalloc: a pipeline wait timed out (stage " +
                                     std::to_string(h) + ")");
        return EMFA_ERR_TIMEOUT;
    }
    return EMFA_OK;
}

}  // extern "C"
