// Split-FP16 complex products on the 5th-generation tensor cores
// (tcgen05.mma kind::f16, FP32 accumulation in tensor memory) for the
// mixed-precision dense solver.
//
// Z (complex64) is split once per solve into two FP16 planes after scaling
// by a power of two s (max |s Z| < 2^15, so every value is in FP16 range):
//     Zh = fp16(s Z),   Zl = fp16(s Z - Zh)        Zh + Zl = s Z to ~2^-22
// each an n x 2n real matrix (re, im interleaved along k).  A right-hand side
// x_r gets its own power-of-two scale t_r (max |t_r x_r| < 2^14) and is packed
// as B rows 2r = (Re, -Im), 2r+1 = (Im, Re), so C = A B^T has the complex
// outputs in its column pairs (the layout of the TF32 kernel, gemm_tc.cu).
//
//   inner product of the Krylov iterations:  Z X  ~  Zh Xh / (s t)
//       11-bit significands on both sides: the accuracy of a TF32 product
//       at the FP16 tensor rate, reading half the bytes of Z
//   refinement residual:  B - Z X  with  Z X ~ (Zh Xh + Zh Xl + Zl Xh) / (s t)
//       k_hresid: a fresh accumulator per k-block, drained into compensated
//       FP32 sums in registers (see the kernel's comment)
//
// Kernel k_hgemm<BN, MS>: one (128 MS) x BN output tile per CTA, 6 warps:
//   warp 0      TMA producer: MS blocks of A (128 x 64 halves each) and one
//               B tile (BN x 64 halves), 128-byte swizzle, multi-stage ring
//   warp 1      allocates tensor memory (one accumulator per row block); one
//               lane issues tcgen05.mma (M = 128, N = BN, K = 16): 4 per stage
//               and row block, and commits each stage free
//   warps 2..5  epilogue: tcgen05.ld 32 lanes x 16 columns, scaled complex64
//               stores (consecutive lanes = consecutive rows: coalesced)
// Every wait is bounded (clock64): on timeout the kernel records a code in
// the error word, waits (bounded) for its own copies and MMAs, frees tensor
// memory and returns; the host reports EMFA_ERR_TIMEOUT.
#include "emfa_internal.cuh"
#include "emfa_math.cuh"
#include "gemm.cuh"
#include "tcgen05.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <map>
#include <mutex>

namespace emfa {

namespace th {

constexpr int BM = 128;
constexpr int BKH = 64;  // halves per stage row = 128 bytes = one swizzle atom
constexpr int THREADS = 192;
constexpr int SMEM_BUDGET = 216 * 1024;

// Inner product: MS row blocks of 128 (M = 128 MMAs, one accumulator each)
// share every B tile, so a 256-row tile reads 26% fewer operand bytes per
// FLOP than a 128-row one; operand delivery from L2, not the tensor pipe,
// bounds this skinny product (N = 2R = 720).
template <int BN, int MS>
struct Smem {
    static constexpr int A_BYTES = BM * 128;  // one 128-row block
    static constexpr int B_BYTES = BN * 128;
    static constexpr int STAGE_BYTES = MS * A_BYTES + B_BYTES;
    static constexpr int STAGES = SMEM_BUDGET / STAGE_BYTES > 8 ? 8 : SMEM_BUDGET / STAGE_BYTES;
    static constexpr int ACC = BN <= 32 ? 32 : BN <= 64 ? 64 : BN <= 128 ? 128 : 256;  // columns per accumulator
    static constexpr int TMEM_COLS = MS * ACC < 32 ? 32 : MS * ACC;
    static constexpr int TOTAL = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
};

template <int BN, int MS>
__global__ void __launch_bounds__(THREADS, 1)
    k_hgemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
            float2* __restrict__ Y, int M, int R, int kblocks, const float* __restrict__ inv_s,
            const float* __restrict__ inv_t, int* __restrict__ err, const int* __restrict__ skip)
{
    using S = Smem<BN, MS>;
    using namespace tc;
    // one wave: every CTA is resident, so the next launch (the Gram-Schmidt
    // coefficients) may be scheduled beside it at once and wait for its end
    griddep_launch();
    // launched as a dependent (the Krylov loop's products): the step that
    // packed B and counted the active right-hand sides must have finished
    griddep_wait();
    // no right-hand side left active (the Krylov step queued after the last
    // one): the same value in every thread, before any barrier or allocation
    if (skip && *skip == 0) return;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = base;                               // [stage][row block]
    uint8_t* sB = base + S::STAGES * MS * S::A_BYTES;  // [stage]
    uint64_t* full = (uint64_t*)(base + S::STAGES * S::STAGE_BYTES);
    uint64_t* empty = full + S::STAGES;
    uint64_t* accum = empty + S::STAGES;
    uint32_t* tmem_slot = (uint32_t*)(accum + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // grid x = column tiles, y = row tiles: CTAs sharing a row block of the
    // hi plane run back to back and reuse it from L2
    const int f0 = blockIdx.y * (BM * MS), c0 = blockIdx.x * BN;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S::STAGES; ++s) {
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
                const int s = kb % S::STAGES;
                if (kb >= S::STAGES && !mbar_wait(empty + s, ((kb / S::STAGES) - 1) & 1, err, 1)) break;
                if (*(volatile int*)err) break;
                mbar_expect_tx(full + s, S::STAGE_BYTES);
#pragma unroll
                for (int m = 0; m < MS; ++m)
                    tma_load_2d(sA + (s * MS + m) * S::A_BYTES, &tmA, full + s, kb * BKH, f0 + m * BM);
                tma_load_2d(sB + s * S::B_BYTES, &tmB, full + s, kb * BKH, c0);
                issued = kb + 1;
            }
            // every issued stage's copy must have landed before the CTA exits
            for (int kb = issued - S::STAGES > 0 ? issued - S::STAGES : 0; kb < issued; ++kb)
                mbar_wait(full + (kb % S::STAGES), (kb / S::STAGES) & 1, err, 2);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_f16(BM, BN);
            for (int kb = 0; kb < kblocks; ++kb) {
                const int s = kb % S::STAGES;
                if (!mbar_wait(full + s, (kb / S::STAGES) & 1, err, 3)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint64_t db = sw128_desc(smem_u32(sB + s * S::B_BYTES));
#pragma unroll
                for (int m = 0; m < MS; ++m) {
                    const uint64_t da = sw128_desc(smem_u32(sA + (s * MS + m) * S::A_BYTES));
#pragma unroll
                    for (int k = 0; k < BKH / 16; ++k)  // K = 16 halves = 32 bytes per instruction
                        mma_f16(tmem + (uint32_t)(m * S::ACC), da + 2 * k, db + 2 * k, idesc,
                                (kb > 0 || k > 0) ? 1u : 0u);
                }
                mma_commit(empty + s);
            }
            // every MMA issued must be complete before the epilogue and before
            // tensor memory is released
            mma_commit(accum);
            mbar_wait(accum, 0, err, 4);
        }
        __syncwarp();
    } else {
        // epilogue warps 2..5: lane quadrant (warp % 4) of tensor memory
        const int q = warp & 3;
        int ok = lane == 0 ? (int)mbar_wait(accum, 0, err, 5) : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const float is = *inv_s;
            // 48 columns a round trip where BN allows (144 = 3 x 48), else 16
            constexpr int CW = BN % 48 == 0 ? 48 : 16;
#pragma unroll 1
            for (int m = 0; m < MS; ++m) {
                const int f = f0 + m * BM + 32 * q + lane;
#pragma unroll 1
                for (int c = 0; c < BN; c += CW) {
                    float v[CW];
                    if constexpr (CW == 48)
                        tmem_ld48(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(m * S::ACC + c), v);
                    else
                        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(m * S::ACC + c), v);
                    if (f < M) {
#pragma unroll
                        for (int i = 0; i < CW / 2; ++i) {
                            const int r = (c0 + c) / 2 + i;
                            if (r < R) {
                                const float sc = is * inv_t[r];
                                Y[(size_t)r * M + f] = make_float2(v[2 * i] * sc, v[2 * i + 1] * sc);
                            }
                        }
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

// ---------------------------------------------------------------------------
// operand preparation
// ---------------------------------------------------------------------------
__device__ __forceinline__ float block_max(float m, float* red)
{
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = m;
    __syncthreads();
    if (w == 0) {
        m = l < (int)(blockDim.x >> 5) ? red[l] : 0.f;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (l == 0) red[0] = m;
    }
    __syncthreads();
    return red[0];
}

// max |Re|, |Im| over Z: non-negative floats order like their bit patterns
__global__ void k_zmax(const float2* __restrict__ Z, size_t ldz, int n, unsigned int* __restrict__ amax)
{
    __shared__ float red[32];
    float m = 0.f;
    // CTAs stride the rows, threads the columns: no index division per element
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        const float2* zr = Z + (size_t)i * ldz;
#pragma unroll 4
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const float2 z = zr[j];
            m = fmaxf(m, fmaxf(fabsf(z.x), fabsf(z.y)));
        }
    }
    m = block_max(m, red);
    if (threadIdx.x == 0) atomicMax(amax, __float_as_uint(m));
}

// Zh = fp16(s Z), Zl = fp16(s Z - Zh) with s = 2^(15 - e), max|Z| = m 2^e, m in [0.5, 1)
__global__ void k_zsplit(const float2* __restrict__ Z, size_t ldz, int n, size_t ldh,
                         const unsigned int* __restrict__ amax, __half* __restrict__ Zh, __half* __restrict__ Zl,
                         float* __restrict__ inv_s)
{
    int e = 0;
    frexpf(__uint_as_float(*amax), &e);
    const float s = ldexpf(1.f, 15 - e);
    if (blockIdx.x == 0 && threadIdx.x == 0) *inv_s = ldexpf(1.f, e - 15);
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        const float2* zr = Z + (size_t)i * ldz;
        __half2* hr = reinterpret_cast<__half2*>(Zh + (size_t)i * ldh);
        __half2* lr = reinterpret_cast<__half2*>(Zl + (size_t)i * ldh);
#pragma unroll 4
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const float2 z = zr[j];
            const float a = s * z.x, b = s * z.y;  // exact: power-of-two scaling
            const __half ha = __float2half_rn(a), hb = __float2half_rn(b);
            const __half la = __float2half_rn(a - __half2float(ha)), lb = __float2half_rn(b - __half2float(hb));
            hr[j] = __halves2half2(ha, hb);
            lr[j] = __halves2half2(la, lb);
        }
    }
}

// One CTA per right-hand side r: scale t_r = 2^(14 - e), max|x_r| = m 2^e,
// then B rows 2r = (Re, -Im), 2r+1 = (Im, Re) of t_r x_r as FP16 pairs; the
// lo plane (NP = 2) holds fp16(t_r x_r - hi).
__global__ void __launch_bounds__(256) k_hpack_f32(const float2* __restrict__ X, int n, size_t ldh,
                                                   __half* __restrict__ Bh, float* __restrict__ inv_t)
{
    __shared__ float red[32];
    const int r = blockIdx.x;
    const float2* x = X + (size_t)r * n;
    float m = 0.f;
    for (int k = threadIdx.x; k < n; k += blockDim.x) m = fmaxf(m, fmaxf(fabsf(x[k].x), fabsf(x[k].y)));
    m = block_max(m, red);
    int e = 0;
    frexpf(m, &e);
    const float t = ldexpf(1.f, 14 - e);
    if (threadIdx.x == 0) inv_t[r] = ldexpf(1.f, e - 14);
    __half2* h0 = reinterpret_cast<__half2*>(Bh + (size_t)(2 * r) * ldh);
    __half2* h1 = reinterpret_cast<__half2*>(Bh + (size_t)(2 * r + 1) * ldh);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const __half hre = __float2half_rn(t * x[k].x), him = __float2half_rn(t * x[k].y);
        h0[k] = __halves2half2(hre, __hneg(him));
        h1[k] = __halves2half2(him, hre);
    }
}

// Krylov normalisation fused with the packing: v = scale[r] w in FP32 (the
// scale rounded to FP32 once: an FP64 product per element would run on
// GB300's 1/64-rate FP64 pipe), written to Vout and packed as k_hpack_f32
// packs it.  The FP16 scale t_r comes from
// wmax[r] * scale[r] (max |w| recorded by the pass that produced w), so every
// element is independent: a grid over (chunks of 1024, RHS).
__global__ void __launch_bounds__(256) k_hpack_scale(const float2* __restrict__ W, const double* __restrict__ scale,
                                                     const double* __restrict__ wmax, int n, size_t ldh,
                                                     float2* __restrict__ Vout, __half* __restrict__ Bh,
                                                     float* __restrict__ inv_t)
{
    const int r = blockIdx.y;
    const float sc = (float)scale[r];
    const int e = hpack_exponent(wmax[r], scale[r]);
    const float t = ldexpf(1.f, 14 - e);
    if (blockIdx.x == 0 && threadIdx.x == 0) inv_t[r] = ldexpf(1.f, e - 14);
    const float2* w = W + (size_t)r * n;
    float2* v = Vout + (size_t)r * n;
    __half2* h0 = reinterpret_cast<__half2*>(Bh + (size_t)(2 * r) * ldh);
    __half2* h1 = reinterpret_cast<__half2*>(Bh + (size_t)(2 * r + 1) * ldh);
    const int k1 = min(n, (int)(blockIdx.x + 1) * 1024);
#pragma unroll 4
    for (int k = blockIdx.x * 1024 + threadIdx.x; k < k1; k += 256) {
        const float2 x = w[k];
        const float2 y = make_float2(x.x * sc, x.y * sc);
        v[k] = y;
        const __half hre = __float2half_rn(t * y.x), him = __float2half_rn(t * y.y);
        h0[k] = __halves2half2(hre, __hneg(him));
        h1[k] = __halves2half2(him, hre);
    }
}

// hi and lo FP16 planes of t x (t a power of two, so t hi and t lo are exact
// in FP32): hi = fp16(t hi), lo = fp16((t hi - hi16) + t lo), the first
// difference exact
__device__ __forceinline__ void split_f16(float2 s, float t, __half* h, __half* l)
{
    const float a = t * s.x;
    *h = __float2half_rn(a);
    *l = __float2half_rn((a - __half2float(*h)) + t * s.y);
}

__global__ void __launch_bounds__(256) k_hpack_f64(const double2* __restrict__ X, int n, size_t ldh,
                                                   __half* __restrict__ Bh, __half* __restrict__ Bl,
                                                   float* __restrict__ inv_t)
{
    __shared__ float red[32];
    const int r = blockIdx.x;
    const double2* x = X + (size_t)r * n;
    float m = 0.f;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double2 v = x[k];
        m = fmaxf(m, fmaxf(fabsf(split_f64(v.x).x), fabsf(split_f64(v.y).x)));  // = (float) max |x|
    }
    m = block_max(m, red);
    // the float max can round up to the next power of two: scale from it
    // keeps max |t x| < 2^14 either way
    int e = 0;
    frexpf(m, &e);
    const float t = ldexpf(1.f, 14 - e);
    if (threadIdx.x == 0) inv_t[r] = ldexpf(1.f, e - 14);
    __half2* h0 = reinterpret_cast<__half2*>(Bh + (size_t)(2 * r) * ldh);
    __half2* h1 = reinterpret_cast<__half2*>(Bh + (size_t)(2 * r + 1) * ldh);
    __half2* l0 = reinterpret_cast<__half2*>(Bl + (size_t)(2 * r) * ldh);
    __half2* l1 = reinterpret_cast<__half2*>(Bl + (size_t)(2 * r + 1) * ldh);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double2 v = x[k];
        __half hre, lre, him, lim;
        split_f16(split_f64(v.x), t, &hre, &lre);
        split_f16(split_f64(v.y), t, &him, &lim);
        h0[k] = __halves2half2(hre, __hneg(him));
        h1[k] = __halves2half2(him, hre);
        l0[k] = __halves2half2(lre, __hneg(lim));
        l1[k] = __halves2half2(lim, lre);
    }
}

// Two FP32 additions in one instruction (add/sub.rn.f32x2), round to nearest
// like __fadd_rn / __fsub_rn: the residual's Kahan sums run on column pairs
__device__ __forceinline__ unsigned long long pk2(float2 v)
{
    return ((unsigned long long)__float_as_uint(v.y) << 32) | __float_as_uint(v.x);
}
__device__ __forceinline__ float2 upk2(unsigned long long u)
{
    return make_float2(__uint_as_float((unsigned)u), __uint_as_float((unsigned)(u >> 32)));
}
__device__ __forceinline__ float2 fadd2_rn(float2 a, float2 b)
{
    unsigned long long z;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(z) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(z);
}
__device__ __forceinline__ float2 fsub2_rn(float2 a, float2 b)
{
    unsigned long long z;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(z) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(z);
}

// ---------------------------------------------------------------------------
// refinement residual R = B - Z X, Z X ~ (Zh Xh + Zh Xl + Zl Xh) / (s t)
//
// The tensor cores add into their FP32 accumulator with truncation, so the
// error of a long accumulation grows with its length (measured on the
// 7680-unknown CFIE matrix: 4e-6 of ||B|| for partial sums over 1024
// columns, 5e-6 over the whole row).  Here every k-block (64 real columns)
// starts a fresh accumulator, the two correction products go first (their
// partial sums are 2^-11 smaller, so truncating them costs little) and the
// hi x hi products last; eight epilogue warps drain each k-block into
// Kahan-compensated FP32 sums in registers (56 columns each) while the next
// k-block accumulates in the second buffer, and the last step forms
// B - sum / (s t) in FP64.  A drain releases the accumulator as soon as its
// 56 columns are in registers, before the sums.
// ---------------------------------------------------------------------------
constexpr int RBN = 112;
constexpr int REPI = 16;                   // epilogue warps: four per SM sub-partition
constexpr int RCOLS = RBN * 4 / REPI;      // 28 accumulator columns per epilogue warp
constexpr int RTHREADS = 32 * (2 + REPI);  // producer, MMA, epilogue

struct RSmem {
    static constexpr int A_BYTES = BM * 128;
    static constexpr int B_BYTES = RBN * 128;
    static constexpr int STAGE_BYTES = 2 * (A_BYTES + B_BYTES);
    static constexpr int STAGES = SMEM_BUDGET / STAGE_BYTES;
    static constexpr int ACC = 128;
    static constexpr int TMEM_COLS = 256;
    static constexpr int TOTAL = STAGES * STAGE_BYTES + 1024 + 256;
};

__global__ void __launch_bounds__(RTHREADS, 1)
    k_hresid(const __grid_constant__ CUtensorMap tmA0, const __grid_constant__ CUtensorMap tmA1,
             const __grid_constant__ CUtensorMap tmB0, const __grid_constant__ CUtensorMap tmB1,
             const void* __restrict__ Bv, int b_f64, double2* __restrict__ Rout, int M, int R, int kblocks,
             const float* __restrict__ inv_s, const float* __restrict__ inv_t, int* __restrict__ err)
{
    using S = RSmem;
    using namespace tc;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = base;                               // [stage][plane]
    uint8_t* sB = base + S::STAGES * 2 * S::A_BYTES;  // [stage][plane]
    uint64_t* full = (uint64_t*)(base + S::STAGES * S::STAGE_BYTES);
    uint64_t* empty = full + S::STAGES;
    uint64_t* acc_full = empty + S::STAGES;
    uint64_t* acc_empty = acc_full + 2;
    uint64_t* done = acc_empty + 2;
    uint32_t* tmem_slot = (uint32_t*)(done + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int f0 = blockIdx.y * BM, c0 = blockIdx.x * RBN;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S::STAGES; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(acc_full + a, 1);
            mbar_init(acc_empty + a, REPI);  // one arrival per epilogue warp
        }
        mbar_init(done, 1);
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
                const int s = kb % S::STAGES;
                if (kb >= S::STAGES && !mbar_wait(empty + s, ((kb / S::STAGES) - 1) & 1, err, 11)) break;
                if (*(volatile int*)err) break;
                mbar_expect_tx(full + s, S::STAGE_BYTES);
                tma_load_2d(sA + (2 * s) * S::A_BYTES, &tmA0, full + s, kb * BKH, f0);
                tma_load_2d(sA + (2 * s + 1) * S::A_BYTES, &tmA1, full + s, kb * BKH, f0);
                tma_load_2d(sB + (2 * s) * S::B_BYTES, &tmB0, full + s, kb * BKH, c0);
                tma_load_2d(sB + (2 * s + 1) * S::B_BYTES, &tmB1, full + s, kb * BKH, c0);
                issued = kb + 1;
            }
            for (int kb = issued - S::STAGES > 0 ? issued - S::STAGES : 0; kb < issued; ++kb)
                mbar_wait(full + (kb % S::STAGES), (kb / S::STAGES) & 1, err, 12);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_f16(BM, RBN);
            for (int kb = 0; kb < kblocks; ++kb) {
                const int s = kb % S::STAGES;
                const uint32_t acc = tmem + (uint32_t)((kb & 1) * S::ACC);
                if (kb >= 2) {
                    if (!mbar_wait(acc_empty + (kb & 1), ((kb >> 1) - 1) & 1, err, 16)) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                }
                if (!mbar_wait(full + s, (kb / S::STAGES) & 1, err, 13)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint64_t dah = sw128_desc(smem_u32(sA + (2 * s) * S::A_BYTES));
                const uint64_t dal = sw128_desc(smem_u32(sA + (2 * s + 1) * S::A_BYTES));
                const uint64_t dbh = sw128_desc(smem_u32(sB + (2 * s) * S::B_BYTES));
                const uint64_t dbl = sw128_desc(smem_u32(sB + (2 * s + 1) * S::B_BYTES));
#pragma unroll
                for (int k = 0; k < BKH / 16; ++k) {  // corrections: Zh Xl + Zl Xh
                    mma_f16(acc, dah + 2 * k, dbl + 2 * k, idesc, k > 0 ? 1u : 0u);
                    mma_f16(acc, dal + 2 * k, dbh + 2 * k, idesc, 1u);
                }
#pragma unroll
                for (int k = 0; k < BKH / 16; ++k) mma_f16(acc, dah + 2 * k, dbh + 2 * k, idesc, 1u);
                mma_commit(empty + s);
                mma_commit(acc_full + (kb & 1));
            }
            mma_commit(done);
            mbar_wait(done, 0, err, 14);
        }
        __syncwarp();
    } else {
        // epilogue warps 2..17: lane quadrant warp % 4, column quarter (warp - 2) / 4
        constexpr int CP = RCOLS / 2;  // column pairs (right-hand sides) per thread
        const int q = warp & 3, grp = (warp - 2) >> 2;
        const int f = f0 + 32 * q + lane;
        const int col0 = RCOLS * grp;
        // Kahan sums: sum - cmp is the running total.  cmp stays below half an
        // ulp of sum, so bf16 holds it to 2^-32 of the total.  The drain is
        // issue-bound and sets the kernel's pace: a k-block's 28 columns come
        // in one tensor-memory round trip (tmem_ld28), the accumulator is
        // released as soon as they are in registers, the sums run on column
        // pairs (f32x2: two additions an instruction), and sixteen warps (four
        // per SM sub-partition) share the work to hide the latencies
        // (0.81 ms a launch with eight warps, seven round trips and scalar
        // sums; 0.62 ms with eight warps and the rest).
        float2 sum[CP];  // columns 2i, 2i + 1
        __nv_bfloat162 cmp[CP];
#pragma unroll
        for (int i = 0; i < CP; ++i) {
            sum[i] = make_float2(0.f, 0.f);
            cmp[i] = __floats2bfloat162_rn(0.f, 0.f);
        }
        bool ok = true;
#pragma unroll 1
        for (int kb = 0; kb < kblocks; ++kb) {
            const int a = kb & 1;
            int w = lane == 0 ? (int)mbar_wait(acc_full + a, (kb >> 1) & 1, err, 15) : 0;
            w = __shfl_sync(0xffffffffu, w, 0);
            if (!w) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            float v[RCOLS];
            tmem_ld28(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(a * S::ACC + col0), v);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(acc_empty + a);
#pragma unroll
            for (int i = 0; i < CP; ++i) {
                const float2 y = fsub2_rn(make_float2(v[2 * i], v[2 * i + 1]), __bfloat1622float2(cmp[i]));
                const float2 t = fadd2_rn(sum[i], y);
                const float2 cn = fsub2_rn(fsub2_rn(t, sum[i]), y);
                cmp[i] = __floats2bfloat162_rn(cn.x, cn.y);
                sum[i] = t;
            }
        }
        if (ok && f < M) {
            // R = B - (sum - cmp) sc.  sc = (1 / s)(1 / t_r) is a power of two,
            // so sum sc and cmp sc are exact: for an FP32 B, R = (B - sum sc)
            // + cmp sc is two FMAs rounded once each (FP64 would queue on
            // GB300's 1/64-rate pipe for every output)
            const float is = *inv_s;
            // unrolled: static indices keep sum and cmp in registers
#pragma unroll
            for (int i = 0; i < CP; ++i) {
                const int r = (c0 + col0) / 2 + i;
                if (r >= R) continue;
                const float2 cf = __bfloat1622float2(cmp[i]);
                const size_t o = (size_t)r * M + f;
                if (b_f64) {
                    const double sc = (double)is * (double)inv_t[r];
                    const double re = ((double)sum[i].x - (double)cf.x) * sc;
                    const double im = ((double)sum[i].y - (double)cf.y) * sc;
                    const double2 b = reinterpret_cast<const double2*>(Bv)[o];
                    Rout[o] = make_double2(b.x - re, b.y - im);
                } else {
                    const float sc = is * inv_t[r];
                    const float2 b = reinterpret_cast<const float2*>(Bv)[o];
                    const float rr = fmaf(cf.x, sc, fmaf(-sum[i].x, sc, b.x));
                    const float ri = fmaf(cf.y, sc, fmaf(-sum[i].y, sc, b.y));
                    Rout[o] = make_double2((double)rr, (double)ri);
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

}  // namespace th

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static size_t ld_halves(int n) { return ((size_t)2 * n + 7) & ~(size_t)7; }  // 16-byte rows

static int grid_stride_blocks(Ctx* c, size_t tot)
{
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    return (int)std::max<size_t>(1, std::min<size_t>((tot + 255) / 256, (size_t)sms * 8));
}

// FP16 2-D tensor map: inner extent `inner` halves, `rows` rows `ld` halves
// apart, box 64 x box_rows, 128-byte swizzle, zero fill out of bounds.
static emfa_status_t make_map_h(Ctx* c, CUtensorMap* m, const void* ptr, uint64_t inner, uint64_t rows, size_t ld,
                                uint32_t box_rows)
{
    auto fn = tensor_map_encoder();
    if (!fn) {
        set_error(c, "cuTensorMapEncodeTiled unavailable");
        return EMFA_ERR_CUDA;
    }
    cuuint64_t dims[2] = {inner, rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {(cuuint32_t)th::BKH, box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error(c, "cuTensorMapEncodeTiled (fp16) failed (" + std::to_string((int)r) + ")");
        return EMFA_ERR_CUDA;
    }
    return EMFA_OK;
}

// timed: bracket the launch with the context's kernel timer (launches that
// may skip are not timed: their work is not known on the host)
template <int BN, int MS>
static emfa_status_t launch_h(Ctx* c, const CUtensorMap& ta, const CUtensorMap& tb, float2* Y, int n, int nrhs,
                              const float* inv_s, const float* inv_t, int* err, cudaStream_t st, bool timed,
                              const int* skip)
{
    using S = th::Smem<BN, MS>;
    EMFA_TRY(ensure_smem(c, th::k_hgemm<BN, MS>, S::TOTAL));
    dim3 grd((2 * nrhs + BN - 1) / BN, (n + th::BM * MS - 1) / (th::BM * MS));
    const int kblocks = (2 * n + th::BKH - 1) / th::BKH;
    if (timed && !skip) {
        TimedLaunch tl(c, KT_GEMM, st, 8.0 * n * (double)n * nrhs);
        th::k_hgemm<BN, MS><<<grd, th::THREADS, S::TOTAL, st>>>(ta, tb, Y, n, nrhs, kblocks, inv_s, inv_t, err,
                                                                  nullptr);
    } else if (skip) {
        // the Krylov loop's product: scheduled while the step that packed its
        // operand drains (programmatic dependent launch)
        EMFA_CUDA(c, launch_dependent(th::k_hgemm<BN, MS>, grd, dim3(th::THREADS), (size_t)S::TOTAL, st, ta, tb, Y, n,
                                      nrhs, kblocks, inv_s, inv_t, err, skip));
    } else {
        th::k_hgemm<BN, MS><<<grd, th::THREADS, S::TOTAL, st>>>(ta, tb, Y, n, nrhs, kblocks, inv_s, inv_t, err, skip);
    }
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    return EMFA_OK;
}

// error word of the split kernels: int 4 of the context's GEMM error slot
static emfa_status_t herr(Ctx* c, int** err)
{
    void* ep = nullptr;
    EMFA_TRY(ctx_workspace(c, WS_GEMM_ERR, 64, &ep));
    *err = (int*)ep + 4;
    return EMFA_OK;
}

emfa_status_t hsplit_prepare(Ctx* c, const void* Z, size_t ldz, int n, HPlanes* out, cudaStream_t st)
{
    const size_t ldh = ld_halves(n);
    const size_t plane = Carver::round(sizeof(__half) * ldh * (size_t)n);
    void* wp = nullptr;
    EMFA_TRY(ctx_workspace(c, WS_ZPLANES, 2 * plane + 256, &wp));
    Carver cv{(char*)wp};
    __half* zh = cv.take<__half>(ldh * (size_t)n);
    __half* zl = cv.take<__half>(ldh * (size_t)n);
    unsigned int* amax = cv.take<unsigned int>(1);
    float* inv_s = cv.take<float>(1);
    int* err = nullptr;
    EMFA_TRY(herr(c, &err));
    EMFA_CUDA(c, cudaMemsetAsync(err, 0, sizeof(int), st));
    EMFA_CUDA(c, cudaMemsetAsync(amax, 0, sizeof(unsigned int), st));
    const int g = std::max(1, std::min(grid_stride_blocks(c, (size_t)n * n), n));  // CTAs stride the rows
    th::k_zmax<<<g, 256, 0, st>>>((const float2*)Z, ldz, n, amax);
    th::k_zsplit<<<g, 256, 0, st>>>((const float2*)Z, ldz, n, ldh, amax, zh, zl, inv_s);
    c->kernel_launches += 2;
    EMFA_CUDA(c, cudaGetLastError());
    out->zh = zh;
    out->zl = zl;
    out->inv_s = inv_s;
    out->n = n;
    out->ldh = ldh;
    return EMFA_OK;
}

// ---------------------------------------------------------------------------
// Tile-shape autotuner of the inner product.  Shapes (BN columns, MS row
// blocks of 128): 64 x 1, 64 x 2, 144 x 1, 144 x 2.  The first product of a
// shape bucket (device, ceil(N / 256), ceil(2 n_rhs / 16)) in the process
// times every candidate twice with CUDA events on the caller's stream and
// keeps the fastest; later products of the bucket launch it directly.  Every
// shape accumulates each output over K in the same order, so the choice
// never changes the result.  EMFA_AUTOTUNE=0 in the environment keeps the
// fixed rule (the 256-row, 144-column tiles once they fill the SMs).
// ---------------------------------------------------------------------------
namespace {
struct TuneKey {
    int dev, rows, cols;
    bool operator<(const TuneKey& o) const
    {
        return dev != o.dev ? dev < o.dev : rows != o.rows ? rows < o.rows : cols < o.cols;
    }
};
struct TuneEntry {
    int variant = -1;
    float ms[HV_COUNT] = {-1.f, -1.f, -1.f, -1.f};
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneEntry> g_tune;

bool autotune_enabled()
{
    static const bool on = [] {
        const char* e = getenv("EMFA_AUTOTUNE");
        return !(e && e[0] == '0');
    }();
    return on;
}
}  // namespace

static int fixed_variant(int n, int nrhs, int sms)
{
    if (2 * nrhs <= 64) return HV_64_1;
    const int col_tiles = (2 * nrhs + 143) / 144;
    return (long)col_tiles * ((n + 255) / 256) >= (long)sms * 9 / 10 ? HV_144_2 : HV_144_1;
}

static emfa_status_t launch_variant(Ctx* c, int v, const CUtensorMap& ta, const CUtensorMap* tb, float2* Y, int n,
                                    int nrhs, const float* inv_s, const float* inv_t, int* err, cudaStream_t st,
                                    bool timed, const int* skip = nullptr)
{
    switch (v) {
    case HV_64_1: return launch_h<64, 1>(c, ta, tb[0], Y, n, nrhs, inv_s, inv_t, err, st, timed, skip);
    case HV_64_2: return launch_h<64, 2>(c, ta, tb[0], Y, n, nrhs, inv_s, inv_t, err, st, timed, skip);
    case HV_144_1: return launch_h<144, 1>(c, ta, tb[1], Y, n, nrhs, inv_s, inv_t, err, st, timed, skip);
    default: return launch_h<144, 2>(c, ta, tb[1], Y, n, nrhs, inv_s, inv_t, err, st, timed, skip);
    }
}

// times the candidates (two launches each, the faster kept) and records the
// choice; the last launch leaves the product in Y
static emfa_status_t tune_variants(Ctx* c, const TuneKey& key, const CUtensorMap& ta, const CUtensorMap* tb, float2* Y,
                                   int n, int nrhs, const float* inv_s, const float* inv_t, int* err, cudaStream_t st)
{
    TuneEntry e;
    int cand[HV_COUNT], nc = 0;
    cand[nc++] = HV_64_1;
    if (n > 128) cand[nc++] = HV_64_2;
    if (2 * nrhs > 64) {
        cand[nc++] = HV_144_1;
        if (n > 128) cand[nc++] = HV_144_2;
    }
    cudaEvent_t ev[2];
    EMFA_CUDA(c, cudaEventCreate(&ev[0]));
    EMFA_CUDA(c, cudaEventCreate(&ev[1]));
    emfa_status_t st_ = EMFA_OK;
    for (int i = 0; i < nc && st_ == EMFA_OK; ++i) {
        float best = 1e30f;
        for (int rep = 0; rep < 2 && st_ == EMFA_OK; ++rep) {
            cudaEventRecord(ev[0], st);
            st_ = launch_variant(c, cand[i], ta, tb, Y, n, nrhs, inv_s, inv_t, err, st, false);
            cudaEventRecord(ev[1], st);
            if (st_ != EMFA_OK) break;
            if (cudaEventSynchronize(ev[1]) != cudaSuccess) {
                st_ = EMFA_ERR_CUDA;
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[0], ev[1]);
            best = std::min(best, ms);
        }
        e.ms[cand[i]] = best;
        if (e.variant < 0 || best < e.ms[e.variant]) e.variant = cand[i];
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    EMFA_TRY(st_);
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        g_tune[key] = e;
    }
    // the result of the last candidate is in Y; the chosen one gives the same bits
    return EMFA_OK;
}

// the inner-product GEMM on an already packed B plane; skip (optional): an
// int that, if zero when the product starts, skips it
static emfa_status_t hgemm_run(Ctx* c, const HPlanes& h, const __half* bh, const float* inv_t, void* Y, int nrhs,
                               int* err, cudaStream_t st, const int* skip = nullptr)
{
    const int n = h.n;
    const size_t ldh = h.ldh;
    CUtensorMap ta, tb[2];  // tb[0]: 64-column boxes, tb[1]: 144-column boxes
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    EMFA_TRY(make_map_h(c, &ta, h.zh, 2 * (uint64_t)n, (uint64_t)n, ldh, th::BM));
    EMFA_TRY(make_map_h(c, &tb[0], bh, 2 * (uint64_t)n, 2 * (uint64_t)nrhs, ldh, 64));
    if (2 * nrhs > 64) EMFA_TRY(make_map_h(c, &tb[1], bh, 2 * (uint64_t)n, 2 * (uint64_t)nrhs, ldh, 144));
    int v = fixed_variant(n, nrhs, sms);
    if (autotune_enabled()) {
        const TuneKey key{c->device, (n + 255) / 256, (2 * nrhs + 15) / 16};
        int known = -1;
        {
            std::lock_guard<std::mutex> g(g_tune_mu);
            auto it = g_tune.find(key);
            if (it != g_tune.end()) known = it->second.variant;
        }
        // a product that may be skipped is never the one that tunes
        if (known < 0 && !skip) return tune_variants(c, key, ta, tb, (float2*)Y, n, nrhs, h.inv_s, inv_t, err, st);
        if (known >= 0) v = known;
    }
    return launch_variant(c, v, ta, tb, (float2*)Y, n, nrhs, h.inv_s, inv_t, err, st, true, skip);
}

emfa_status_t hgemm_tuned_shape(int device, int n, int nrhs, int* variant, float* ms)
{
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune.find(TuneKey{device, (n + 255) / 256, (2 * nrhs + 15) / 16});
    if (it == g_tune.end()) {
        *variant = -1;
        for (int i = 0; i < HV_COUNT; ++i) ms[i] = -1.f;
        return EMFA_OK;
    }
    *variant = it->second.variant;
    for (int i = 0; i < HV_COUNT; ++i) ms[i] = it->second.ms[i];
    return EMFA_OK;
}

void hgemm_tune_clear()
{
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune.clear();
}

static emfa_status_t hgemm_bplane(Ctx* c, const HPlanes& h, int nrhs, __half** bh, float** inv_t)
{
    void* wp = nullptr;
    const size_t bplane = Carver::round(sizeof(__half) * h.ldh * 2 * (size_t)nrhs);
    EMFA_TRY(ctx_workspace(c, WS_HGEMM, bplane + Carver::round(sizeof(float) * nrhs) + 256, &wp));
    Carver cv{(char*)wp};
    *bh = cv.take<__half>(h.ldh * 2 * (size_t)nrhs);
    *inv_t = cv.take<float>(nrhs);
    return EMFA_OK;
}

emfa_status_t hgemm_apply(Ctx* c, const HPlanes& h, const void* X, void* Y, int nrhs, cudaStream_t st)
{
    __half* bh = nullptr;
    float* inv_t = nullptr;
    EMFA_TRY(hgemm_bplane(c, h, nrhs, &bh, &inv_t));
    int* err = nullptr;
    EMFA_TRY(herr(c, &err));
    th::k_hpack_f32<<<nrhs, 256, 0, st>>>((const float2*)X, h.n, h.ldh, bh, inv_t);
    c->kernel_launches += 1;
    return hgemm_run(c, h, bh, inv_t, Y, nrhs, err, st);
}

emfa_status_t hgemm_normalize_apply(Ctx* c, const HPlanes& h, const void* W, const double* scale,
                                    const double* wmax, void* Vout, void* Y, int nrhs, cudaStream_t st)
{
    __half* bh = nullptr;
    float* inv_t = nullptr;
    EMFA_TRY(hgemm_bplane(c, h, nrhs, &bh, &inv_t));
    int* err = nullptr;
    EMFA_TRY(herr(c, &err));
    th::k_hpack_scale<<<dim3((h.n + 1023) / 1024, nrhs), 256, 0, st>>>((const float2*)W, scale, wmax, h.n, h.ldh,
                                                                       (float2*)Vout, bh, inv_t);
    c->kernel_launches += 1;
    return hgemm_run(c, h, bh, inv_t, Y, nrhs, err, st);
}

emfa_status_t hgemm_pack_target(Ctx* c, const HPlanes& h, int nrhs, HPack* out)
{
    EMFA_TRY(hgemm_bplane(c, h, nrhs, &out->bh, &out->inv_t));
    out->ldh = h.ldh;
    return EMFA_OK;
}

emfa_status_t hgemm_apply_packed(Ctx* c, const HPlanes& h, const HPack& p, void* Y, int nrhs, cudaStream_t st)
{
    int* err = nullptr;
    EMFA_TRY(herr(c, &err));
    return hgemm_run(c, h, p.bh, p.inv_t, Y, nrhs, err, st, p.skip);
}

emfa_status_t hgemm_pack(Ctx* c, const HPlanes& h, const void* X, const HPack& p, int nrhs, cudaStream_t st)
{
    if (!p.bh || !p.inv_t || p.ldh != h.ldh) return EMFA_ERR_INVALID;
    th::k_hpack_f32<<<nrhs, 256, 0, st>>>((const float2*)X, h.n, h.ldh, p.bh, p.inv_t);
    c->kernel_launches += 1;
    return EMFA_OK;
}

emfa_status_t hgemm_residual(Ctx* c, const HPlanes& h, const double2* X, const void* B, bool b_is_f32, double2* R,
                             int nrhs, cudaStream_t st)
{
    using S = th::RSmem;
    const int n = h.n;
    const size_t ldh = h.ldh;
    const size_t bplane = Carver::round(sizeof(__half) * ldh * 2 * (size_t)nrhs);
    void* wp = nullptr;
    EMFA_TRY(ctx_workspace(c, WS_HGEMM, 2 * bplane + Carver::round(sizeof(float) * nrhs) + 256, &wp));
    Carver cv{(char*)wp};
    __half* bh = cv.take<__half>(ldh * 2 * (size_t)nrhs);
    __half* bl = cv.take<__half>(ldh * 2 * (size_t)nrhs);
    float* inv_t = cv.take<float>(nrhs);
    int* err = nullptr;
    EMFA_TRY(herr(c, &err));
    th::k_hpack_f64<<<nrhs, 256, 0, st>>>(X, n, ldh, bh, bl, inv_t);
    c->kernel_launches += 1;
    CUtensorMap a0, a1, b0, b1;
    EMFA_TRY(make_map_h(c, &a0, h.zh, 2 * (uint64_t)n, (uint64_t)n, ldh, th::BM));
    EMFA_TRY(make_map_h(c, &a1, h.zl, 2 * (uint64_t)n, (uint64_t)n, ldh, th::BM));
    EMFA_TRY(make_map_h(c, &b0, bh, 2 * (uint64_t)n, 2 * (uint64_t)nrhs, ldh, th::RBN));
    EMFA_TRY(make_map_h(c, &b1, bl, 2 * (uint64_t)n, 2 * (uint64_t)nrhs, ldh, th::RBN));
    EMFA_TRY(ensure_smem(c, th::k_hresid, S::TOTAL));
    dim3 grd((2 * nrhs + th::RBN - 1) / th::RBN, (n + th::BM - 1) / th::BM);
    const int kblocks = (2 * n + th::BKH - 1) / th::BKH;
    {
        TimedLaunch tl(c, KT_RESIDUAL, st, 8.0 * n * (double)n * nrhs);
        th::k_hresid<<<grd, th::RTHREADS, S::TOTAL, st>>>(a0, a1, b0, b1, B, b_is_f32 ? 0 : 1, R, n, nrhs, kblocks,
                                                          h.inv_s, inv_t, err);
    }
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    return EMFA_OK;
}

emfa_status_t hgemm_check_error(Ctx* c, cudaStream_t st)
{
    int* err = nullptr;
    EMFA_TRY(herr(c, &err));
    int h = 0;
    EMFA_CUDA(c, cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    if (h) {
        set_error(c, "split-FP16 tensor-core product: a pipeline wait timed out (stage " + std::to_string(h) + ")");
        return EMFA_ERR_TIMEOUT;
    }
    return EMFA_OK;
}

}  // namespace emfa
