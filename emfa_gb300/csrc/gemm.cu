// Multi-right-hand-side dense complex product on CUDA cores:
//   Y[r][f] = sum_k Z[f][k] X[r][k]      (Z row-major N x N, X / Y RHS-major)
// the dense products of iml::BICGSTAB / iml::GMRES (EMIterative/iml.cpp:22,186)
// for many right-hand sides at once.
//
// 64 (f) x 64 (r) CTA tile, 16-wide K slices staged through shared memory,
// 4 x 4 complex outputs per thread; up to 16 right-hand sides a warp-per-row
// GEMV instead.  ACC selects the accumulation:
//   float / double : plain accumulation in that type
//   CHUNKED        : FP32 products and sums over 64-wide K chunks, chunk sums
//                    accumulated in FP64 (the refinement residual of the
//                    mixed-precision solver: ~FP32-product accuracy without
//                    FP64 FMA throughput)
#include "emfa_internal.cuh"
#include "emfa_math.cuh"
#include "gemm.cuh"

#include <algorithm>

namespace emfa {

template <typename T, bool CHUNKED>
__global__ void __launch_bounds__(256) k_cgemm(const Cx<T>* __restrict__ Z, size_t ldz, const Cx<T>* __restrict__ X,
                                               int n, int nrhs, Cx<T>* __restrict__ Y,
                                               const Cx<T>* __restrict__ Bsub, Cx<double>* __restrict__ Yd)
{
    constexpr int BM = 64, BN = 64, BK = 16;
    __shared__ Cx<T> As[BK][BM + 1];
    __shared__ Cx<T> Bs[BK][BN + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int f0 = blockIdx.x * BM, r0 = blockIdx.y * BN;
    Cx<T> acc[4][4];
    double accd[4][4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            acc[i][j] = cx(T(0), T(0));
            accd[i][j][0] = accd[i][j][1] = 0.0;
        }
    // loader mapping: 256 threads load 64 rows x 16 k: row = tid / 4, k = (tid % 4) * 4 .. +3
    const int lrow = threadIdx.x >> 2, lk = (threadIdx.x & 3) * 4;
    int kt = 0;
    for (int k0 = 0; k0 < n; k0 += BK, ++kt) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int k = k0 + lk + q;
            int f = f0 + lrow, r = r0 + lrow;
            As[lk + q][lrow] = (f < n && k < n) ? Z[(size_t)f * ldz + k] : cx(T(0), T(0));
            Bs[lk + q][lrow] = (r < nrhs && k < n) ? X[(size_t)r * n + k] : cx(T(0), T(0));
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            Cx<T> a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    acc[i][j].re = fma(a[i].re, b[j].re, acc[i][j].re);
                    acc[i][j].re = fma(-a[i].im, b[j].im, acc[i][j].re);
                    acc[i][j].im = fma(a[i].re, b[j].im, acc[i][j].im);
                    acc[i][j].im = fma(a[i].im, b[j].re, acc[i][j].im);
                }
        }
        __syncthreads();
        if (CHUNKED && ((kt & 3) == 3 || k0 + BK >= n)) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    accd[i][j][0] += (double)acc[i][j].re;
                    accd[i][j][1] += (double)acc[i][j].im;
                    acc[i][j] = cx(T(0), T(0));
                }
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        int r = r0 + ty + 16 * j;
        if (r >= nrhs) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int f = f0 + tx + 16 * i;
            if (f >= n) continue;
            size_t o = (size_t)r * n + f;
            if (CHUNKED) {
                // Yd = Bsub - Z X  (residual) when Bsub given, else Z X
                double re = accd[i][j][0], im = accd[i][j][1];
                if (Bsub) {
                    re = (double)Bsub[o].re - re;
                    im = (double)Bsub[o].im - im;
                }
                Yd[o] = cx(re, im);
            } else {
                Y[o] = acc[i][j];
            }
        }
    }
}

// Few right-hand sides (the 64-wide tile above would leave most of its RHS
// columns empty): a warp per RPW rows of Z, lanes striding k, up to RB
// right-hand sides per launch accumulated in registers, then reduced by
// shuffles.  Each warp reads its rows once (coalesced 512-byte segments for
// complex128) and the RHS entries from L1/L2; FP64 is bound by the FMA rate.
template <typename T, int RB, int RPW>
__global__ void __launch_bounds__(256) k_cgemv(const Cx<T>* __restrict__ Z, size_t ldz, const Cx<T>* __restrict__ X,
                                               int n, int nrhs, Cx<T>* __restrict__ Y)
{
    const int warp = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    const int f0 = warp * RPW;
    if (f0 >= n) return;
    T ar[RPW][RB], ai[RPW][RB];
#pragma unroll
    for (int i = 0; i < RPW; ++i)
#pragma unroll
        for (int r = 0; r < RB; ++r) ar[i][r] = ai[i][r] = T(0);
    for (int k = lane; k < n; k += 32) {
        Cx<T> z[RPW];
#pragma unroll
        for (int i = 0; i < RPW; ++i) z[i] = f0 + i < n ? Z[(size_t)(f0 + i) * ldz + k] : cx(T(0), T(0));
#pragma unroll
        for (int r = 0; r < RB; ++r)
            if (r < nrhs) {
                const Cx<T> x = X[(size_t)r * n + k];
#pragma unroll
                for (int i = 0; i < RPW; ++i) {
                    ar[i][r] = fma(z[i].re, x.re, ar[i][r]);
                    ar[i][r] = fma(-z[i].im, x.im, ar[i][r]);
                    ai[i][r] = fma(z[i].re, x.im, ai[i][r]);
                    ai[i][r] = fma(z[i].im, x.re, ai[i][r]);
                }
            }
    }
#pragma unroll
    for (int i = 0; i < RPW; ++i)
#pragma unroll
        for (int r = 0; r < RB; ++r) {
            if (r >= nrhs) break;
            T re = ar[i][r], im = ai[i][r];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                re += __shfl_xor_sync(0xffffffffu, re, o);
                im += __shfl_xor_sync(0xffffffffu, im, o);
            }
            if (lane == 0 && f0 + i < n) Y[(size_t)r * n + f0 + i] = cx(re, im);
        }
}

// up to 16 right-hand sides: GEMV launches of 8; more: the tiled kernel
template <typename T>
static emfa_status_t cgemv_chunks(Ctx* c, const void* Z, size_t ldz, const void* X, int n, int nrhs, void* Y,
                                  cudaStream_t st)
{
    constexpr int RPW = sizeof(T) == 8 ? 1 : 4;
    const int warps = (n + RPW - 1) / RPW;
    for (int r0 = 0; r0 < nrhs; r0 += 8) {
        const int nr = std::min(8, nrhs - r0);
        const Cx<T>* x = (const Cx<T>*)X + (size_t)r0 * n;
        Cx<T>* y = (Cx<T>*)Y + (size_t)r0 * n;
        const int grd = (warps + 7) / 8;
        if (nr == 1)
            k_cgemv<T, 1, RPW><<<grd, 256, 0, st>>>((const Cx<T>*)Z, ldz, x, n, nr, y);
        else if (nr <= 2)
            k_cgemv<T, 2, RPW><<<grd, 256, 0, st>>>((const Cx<T>*)Z, ldz, x, n, nr, y);
        else if (nr <= 4)
            k_cgemv<T, 4, RPW><<<grd, 256, 0, st>>>((const Cx<T>*)Z, ldz, x, n, nr, y);
        else
            k_cgemv<T, 8, RPW><<<grd, 256, 0, st>>>((const Cx<T>*)Z, ldz, x, n, nr, y);
        c->kernel_launches += 1;
        EMFA_CUDA(c, cudaGetLastError());
    }
    return EMFA_OK;
}

emfa_status_t cgemm_f32(Ctx* c, const void* Z, size_t ldz, const void* X, int n, int nrhs, void* Y, cudaStream_t st)
{
    if (nrhs <= 16) return cgemv_chunks<float>(c, Z, ldz, X, n, nrhs, Y, st);
    dim3 grd((n + 63) / 64, (nrhs + 63) / 64);
    k_cgemm<float, false><<<grd, 256, 0, st>>>((const Cx<float>*)Z, ldz, (const Cx<float>*)X, n, nrhs, (Cx<float>*)Y,
                                               nullptr, nullptr);
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    return EMFA_OK;
}

emfa_status_t cgemm_f64(Ctx* c, const void* Z, size_t ldz, const void* X, int n, int nrhs, void* Y, cudaStream_t st)
{
    if (nrhs <= 16) return cgemv_chunks<double>(c, Z, ldz, X, n, nrhs, Y, st);
    dim3 grd((n + 63) / 64, (nrhs + 63) / 64);
    k_cgemm<double, false><<<grd, 256, 0, st>>>((const Cx<double>*)Z, ldz, (const Cx<double>*)X, n, nrhs,
                                                (Cx<double>*)Y, nullptr, nullptr);
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    return EMFA_OK;
}

emfa_status_t cgemm_f32_chunked(Ctx* c, const void* Z, size_t ldz, const void* X, int n, int nrhs, const void* Bsub,
                                void* Yd, cudaStream_t st)
{
    dim3 grd((n + 63) / 64, (nrhs + 63) / 64);
    {
        TimedLaunch tl(c, KT_RESIDUAL, st, 8.0 * n * (double)n * nrhs);
        k_cgemm<float, true><<<grd, 256, 0, st>>>((const Cx<float>*)Z, ldz, (const Cx<float>*)X, n, nrhs, nullptr,
                                                  (const Cx<float>*)Bsub, (Cx<double>*)Yd);
    }
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    return EMFA_OK;
}

}  // namespace emfa
