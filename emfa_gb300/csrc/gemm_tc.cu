// Multi-RHS complex product on the 5th-generation tensor cores (tcgen05,
// TF32 operands, FP32 accumulation in tensor memory).
//
//   Y[r][f] = sum_k Z[f][k] X[r][k]        (complex, Z row-major N x N)
//
// as one real GEMM C = A B^T with
//   A = Z viewed as an N x 2N float matrix (re, im interleaved along k),
//   B rows 2r   = (Re x, -Im x) interleaved  -> C[f][2r]   = Re Y[r][f]
//   B rows 2r+1 = (Im x,  Re x) interleaved  -> C[f][2r+1] = Im Y[r][f]
// so Z is read straight from its complex64 storage and the accumulator's
// column pairs are the complex outputs.
//
// Kernel: one 128 x BN output tile per CTA, 6 warps:
//   warp 0      TMA producer: A (128 x 32) and B (BN x 32) fp32 tiles, 128-byte
//               swizzle, into a 4-stage shared-memory ring (mbarrier tx count)
//   warp 1      allocates tensor memory; one lane issues tcgen05.mma
//               (M = 128, N = BN, K = 8 per instruction, 4 per stage) and
//               tcgen05.commit frees each stage / signals the accumulator
//   warps 2..5  epilogue: tcgen05.ld 32 lanes x 16 columns per warp, writes the
//               complex64 outputs (consecutive lanes = consecutive f: coalesced)
// Every mbarrier wait is bounded (clock64); on timeout the kernel records an
// error code, drains its own copies and MMAs (bounded), frees tensor memory
// and returns, and the host reports EMFA_ERR_TIMEOUT.
#include "emfa_internal.cuh"
#include "gemm.cuh"
#include "tcgen05.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

namespace emfa {

namespace tc {

constexpr int BM = 128;
constexpr int BK = 32;          // fp32 elements per stage row = 128 bytes = one swizzle atom
constexpr int STAGES = 6;
constexpr int THREADS = 192;
template <int BN>
struct Smem {
    static constexpr int A_BYTES = BM * BK * 4;
    static constexpr int B_BYTES = BN * BK * 4;
    static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
    static constexpr int TOTAL = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
    static constexpr int TMEM_COLS = BN <= 32 ? 32 : BN <= 64 ? 64 : BN <= 128 ? 128 : 256;
};

template <int BN>
__global__ void __launch_bounds__(THREADS, 1)
    k_gemm_tf32(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                float2* __restrict__ Y, int M, int R, int kblocks, int* __restrict__ err)
{
    using S = Smem<BN>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = base;
    uint8_t* sB = base + STAGES * S::A_BYTES;
    uint64_t* full = (uint64_t*)(base + STAGES * S::STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* accum = empty + STAGES;
    uint32_t* tmem_slot = (uint32_t*)(accum + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // grid x = column tiles, y = row tiles: the CTAs sharing a row block of Z
    // run back to back, so the block is read from DRAM once and reused in L2
    const int f0 = blockIdx.y * BM, c0 = blockIdx.x * BN;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        mbar_init(accum, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(S::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int issued = 0;
            for (int kb = 0; kb < kblocks; ++kb) {
                const int s = kb % STAGES;
                if (kb >= STAGES && !mbar_wait(empty + s, ((kb / STAGES) - 1) & 1, err, 1)) break;
                if (*(volatile int*)err) break;
                mbar_expect_tx(full + s, S::STAGE_BYTES);
                tma_load_2d(sA + s * S::A_BYTES, &tmA, full + s, kb * BK, f0);
                tma_load_2d(sB + s * S::B_BYTES, &tmB, full + s, kb * BK, c0);
                issued = kb + 1;
            }
            // drain: every issued stage's copy must have landed before the CTA exits
            for (int kb = issued - STAGES > 0 ? issued - STAGES : 0; kb < issued; ++kb)
                mbar_wait(full + (kb % STAGES), (kb / STAGES) & 1, err, 2);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_tf32(BM, BN);
            bool ok = true;
            for (int kb = 0; kb < kblocks && ok; ++kb) {
                const int s = kb % STAGES;
                ok = mbar_wait(full + s, (kb / STAGES) & 1, err, 3);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint64_t da = sw128_desc(smem_u32(sA + s * S::A_BYTES));
                const uint64_t db = sw128_desc(smem_u32(sB + s * S::B_BYTES));
#pragma unroll
                for (int k = 0; k < BK / 8; ++k)  // K = 8 tf32 = 32 bytes per instruction
                    mma_tf32(tmem, da + 2 * k, db + 2 * k, idesc, (kb > 0 || k > 0) ? 1u : 0u);
                mma_commit(empty + s);
            }
            mma_commit(accum);
            // the MMAs must be complete before tensor memory is released
            mbar_wait(accum, 0, err, 4);
        }
        __syncwarp();
    } else {
        // epilogue warps 2..5: lane quadrant (warp % 4) of tensor memory
        const int q = warp & 3;
        // one lane waits, the warp follows it: tcgen05.ld is warp-collective
        int ok = lane == 0 ? (int)mbar_wait(accum, 0, err, 5) : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int f = f0 + 32 * q + lane;
#pragma unroll 1
            for (int c = 0; c < BN; c += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c, v);
                if (f < M) {
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int r = (c0 + c) / 2 + i;
                        if (r < R) Y[(size_t)r * M + f] = make_float2(v[2 * i], v[2 * i + 1]);
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(S::TMEM_COLS) : "memory");
    }
}

// B rows 2r = (Re x, -Im x), 2r+1 = (Im x, Re x), one float2 per k
__global__ void k_pack_b(const float2* __restrict__ X, int n, int nrhs, float2* __restrict__ B)
{
    size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t tot = (size_t)n * nrhs;
    for (; id < tot; id += (size_t)gridDim.x * blockDim.x) {
        size_t r = id / n, k = id % n;
        float2 x = X[id];
        B[(2 * r) * n + k] = make_float2(x.x, -x.y);
        B[(2 * r + 1) * n + k] = make_float2(x.y, x.x);
    }
}

// the pipelines' bounded wait on a barrier nothing arrives on (no copy or MMA
// in flight): records `code` once the short limit passes
__global__ void k_diag_wait(int* err, int code, long long limit)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    mbar_wait(&bar, 0, err, code, limit);
}

}  // namespace tc

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// 2-D fp32 tensor map: inner extent `inner` floats, `rows` rows `stride_bytes`
// apart, box 32 x box_rows, 128-byte swizzle, zero fill out of bounds.
static emfa_status_t make_map(Ctx* c, CUtensorMap* m, const void* ptr, uint64_t inner, uint64_t rows,
                              uint64_t stride_bytes, uint32_t box_rows)
{
    auto fn = tensor_map_encoder();
    if (!fn) {
        set_error(c, "cuTensorMapEncodeTiled unavailable");
        return EMFA_ERR_CUDA;
    }
    cuuint64_t dims[2] = {inner, rows};
    cuuint64_t strides[1] = {stride_bytes};
    cuuint32_t box[2] = {(cuuint32_t)tc::BK, box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error(c, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
        return EMFA_ERR_CUDA;
    }
    return EMFA_OK;
}

template <int BN>
static emfa_status_t launch_tc(Ctx* c, const CUtensorMap& ta, const CUtensorMap& tb, float2* Y, int n, int nrhs,
                               int* err, cudaStream_t st)
{
    using S = tc::Smem<BN>;
    EMFA_TRY(ensure_smem(c, tc::k_gemm_tf32<BN>, S::TOTAL));
    dim3 grd((2 * nrhs + BN - 1) / BN, (n + tc::BM - 1) / tc::BM);
    int kblocks = (2 * n + tc::BK - 1) / tc::BK;
    {
        TimedLaunch tl(c, KT_GEMM, st, 8.0 * n * (double)n * nrhs);
        tc::k_gemm_tf32<BN><<<grd, tc::THREADS, S::TOTAL, st>>>(ta, tb, Y, n, nrhs, kblocks, err);
    }
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    return EMFA_OK;
}

emfa_status_t cgemm_tf32(Ctx* c, const void* Z, size_t ldz, const void* X, int n, int nrhs, void* Y, cudaStream_t st)
{
    if ((n & 1) || (ldz & 1) || ((uintptr_t)Z & 15)) {
        set_error(c, "cgemm_tf32: needs even n and ldz and a 16-byte aligned matrix (TMA strides)");
        return EMFA_ERR_UNSUPPORTED;
    }
    void* bp = nullptr;
    void* ep = nullptr;
    EMFA_TRY(ctx_workspace(c, WS_GEMM_B, sizeof(float) * 4 * (size_t)n * nrhs, &bp));
    EMFA_TRY(ctx_workspace(c, WS_GEMM_ERR, 64, &ep));
    int* err = (int*)ep;
    EMFA_CUDA(c, cudaMemsetAsync(err, 0, sizeof(int), st));
    size_t tot = (size_t)n * nrhs;
    tc::k_pack_b<<<(int)std::min<size_t>((tot + 255) / 256, 8192), 256, 0, st>>>((const float2*)X, n, nrhs,
                                                                                 (float2*)bp);
    c->kernel_launches += 1;
    CUtensorMap ta, tb;
    // 144 columns: 720 outputs (360 RHS) = 5 tiles, 300 CTAs = 1.97 waves on 152 SMs
    const int BN = 2 * nrhs <= 64 ? 64 : 144;
    EMFA_TRY(make_map(c, &ta, Z, 2 * (uint64_t)n, (uint64_t)n, ldz * 8, tc::BM));
    EMFA_TRY(make_map(c, &tb, bp, 2 * (uint64_t)n, 2 * (uint64_t)nrhs, (uint64_t)n * 8, BN));
    if (BN == 64)
        EMFA_TRY(launch_tc<64>(c, ta, tb, (float2*)Y, n, nrhs, err, st));
    else
        EMFA_TRY(launch_tc<144>(c, ta, tb, (float2*)Y, n, nrhs, err, st));
    return EMFA_OK;
}

emfa_status_t gemm_check_error(Ctx* c, cudaStream_t st)
{
    void* ep = nullptr;
    EMFA_TRY(ctx_workspace(c, WS_GEMM_ERR, 64, &ep));
    int h = 0;
    EMFA_CUDA(c, cudaMemcpyAsync(&h, ep, sizeof(int), cudaMemcpyDeviceToHost, st));
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    if (h) {
        set_error(c, "tensor-core GEMM: a pipeline wait timed out (stage " + std::to_string(h) + ")");
        return EMFA_ERR_TIMEOUT;
    }
    return EMFA_OK;
}

emfa_status_t cgemm_tf32_prepare()
{
    EMFA_CUDA(nullptr, cudaFuncSetAttribute(tc::k_gemm_tf32<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            tc::Smem<64>::TOTAL));
    EMFA_CUDA(nullptr, cudaFuncSetAttribute(tc::k_gemm_tf32<144>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            tc::Smem<144>::TOTAL));
    return EMFA_OK;
}

emfa_status_t cgemm_tf32_scratch(const void* Z, size_t ldz, const void* X, int n, int nrhs, void* Y, void* bpack,
                                 int* err, cudaStream_t st)
{
    if ((n & 1) || (ldz & 1) || ((uintptr_t)Z & 15) || ((uintptr_t)bpack & 15)) {
        set_error(nullptr, "cgemm_tf32: needs even n and ldz and 16-byte aligned operands (TMA strides)");
        return EMFA_ERR_UNSUPPORTED;
    }
    size_t tot = (size_t)n * nrhs;
    tc::k_pack_b<<<(int)std::min<size_t>((tot + 255) / 256, 8192), 256, 0, st>>>((const float2*)X, n, nrhs,
                                                                                 (float2*)bpack);
    EMFA_CUDA(nullptr, cudaGetLastError());
    CUtensorMap ta, tb;
    const int BN = 2 * nrhs <= 64 ? 64 : 144;
    EMFA_TRY(make_map(nullptr, &ta, Z, 2 * (uint64_t)n, (uint64_t)n, ldz * 8, tc::BM));
    EMFA_TRY(make_map(nullptr, &tb, bpack, 2 * (uint64_t)n, 2 * (uint64_t)nrhs, (uint64_t)n * 8, BN));
    dim3 grd((2 * nrhs + BN - 1) / BN, (n + tc::BM - 1) / tc::BM);
    int kblocks = (2 * n + tc::BK - 1) / tc::BK;
    if (BN == 64)
        tc::k_gemm_tf32<64><<<grd, tc::THREADS, tc::Smem<64>::TOTAL, st>>>(ta, tb, (float2*)Y, n, nrhs, kblocks, err);
    else
        tc::k_gemm_tf32<144><<<grd, tc::THREADS, tc::Smem<144>::TOTAL, st>>>(ta, tb, (float2*)Y, n, nrhs, kblocks,
                                                                             err);
    EMFA_CUDA(nullptr, cudaGetLastError());
    return EMFA_OK;
}

}  // namespace emfa

extern "C" emfa_status_t emfa_diag_wait_timeout(emfa_ctx_t* ctx, int* code_out)
{
    using namespace emfa;
    if (!ctx || !code_out) return EMFA_ERR_INVALID;
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    void* ep = nullptr;
    EMFA_TRY(ctx_workspace(ctx, WS_GEMM_ERR, 64, &ep));
    int* err = (int*)ep;
    cudaStream_t st = ctx->stream;
    EMFA_CUDA(ctx, cudaMemsetAsync(err, 0, sizeof(int), st));
    tc::k_diag_wait<<<1, 32, 0, st>>>(err, 42, 2000000LL);  // about 1 ms
    ctx->kernel_launches += 1;
    EMFA_CUDA(ctx, cudaGetLastError());
    EMFA_CUDA(ctx, cudaMemcpyAsync(code_out, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    EMFA_CUDA(ctx, cudaStreamSynchronize(st));
    EMFA_CUDA(ctx, cudaMemsetAsync(err, 0, sizeof(int), st));  // the product kernels start from a clear word
    if (*code_out) {
        set_error(ctx, "emfa_diag_wait_timeout: the bounded wait gave up (stage " + std::to_string(*code_out) + ")");
        return EMFA_ERR_TIMEOUT;
    }
    return EMFA_OK;
}
