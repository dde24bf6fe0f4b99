// Dense LU factorisation of the impedance matrix, for solves that factor once
// and then solve and refine (the batched EFIE problems, whose restarted
// Krylov solves need hundreds of iterations).  The reference has no dense
// direct solver on this path: EMSolver/EFIE.cpp:89 keeps a commented-out
// Eigen LU, and its EFIE/CFIE solves are GMRES/BiCGStab only.
//
// Factorisation, FP32 complex, blocked right-looking, block LU_NB = 64, row
// exchanges within each diagonal block (the rows of block k only trade places
// among themselves).  One step per diagonal block:
//   k_lu_diag     one CTA: pivoted LU of the diagonal block in shared memory,
//                 then explicit inverses of its unit-lower and upper factors
//   k_lu_rowperm  the block's row exchanges applied to the other columns
//   k_lu_small    U12 = L11^-1 A12 and L21 = A21 U11^-1 with those inverses
//   k_lu_update   A22 -= L21 U12, 64 x 64 CTA tiles, K = 64
// with a one-block lookahead: the next block's 64 columns are updated first,
// and that block's k_lu_diag (one CTA, latency bound) runs while a helper
// stream updates the remaining columns.
// Solve for many right-hand sides (RHS-major, (r, u) at r n + u): gather by
// the row permutation, then one launch per block for the forward (L) sweep
// and one per block for the backward (U) sweep.  Each CTA applies the block's
// explicit inverse to the block's right-hand sides and updates its own rows
// below (above) the block.
//
// A pivot that is exactly zero is replaced by 1e-30 and recorded in the
// factor's info word, so the caller can fall back to an iterative solve.
#include "emfa_internal.cuh"
#include "lu.cuh"

#include <algorithm>

namespace emfa {

namespace {

constexpr int NB = LU_NB;
constexpr int LDS = NB + 1;  // padded shared-memory row

__device__ __forceinline__ float2 cm(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c)  // c + a b
{
    return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
__device__ __forceinline__ float2 cinv(float2 a)
{
    const float d = a.x * a.x + a.y * a.y;
    return make_float2(a.x / d, -a.y / d);
}

// Pivoted LU of the diagonal block [k0, k0 + nb)^2 and the inverses of its
// factors.  perm[k0 + i] = the original row now at k0 + i (rows of earlier
// blocks never move into this one, so original = k0 + local index).
__global__ void __launch_bounds__(256) k_lu_diag(float2* __restrict__ A, int n, int k0, int nb, int* __restrict__ perm,
                                                 float2* __restrict__ linv, float2* __restrict__ uinv,
                                                 int* __restrict__ info)
{
    extern __shared__ float2 s_lu[];
    float2* D = s_lu;               // [NB][LDS] the block, then its factors
    float2* WL = D + NB * LDS;      // [NB][LDS] L^-1
    float2* WU = WL + NB * LDS;     // [NB][LDS] U^-1
    __shared__ int lp[NB];
    __shared__ int piv_row;
    __shared__ float2 invd[NB];
    const int tid = threadIdx.x;
    for (int q = tid; q < NB * NB; q += blockDim.x) {
        const int i = q / NB, j = q % NB;
        D[i * LDS + j] = (i < nb && j < nb) ? A[(size_t)(k0 + i) * n + k0 + j] : make_float2(0.f, 0.f);
    }
    if (tid < NB) lp[tid] = tid;
    __syncthreads();
    for (int j = 0; j < nb; ++j) {
        // pivot: largest |D[i][j]|^2 over i >= j (lowest index on ties), warp 0
        if (tid < 32) {
            float best = -1.f;
            int bi = j;
            for (int i = j + tid; i < nb; i += 32) {
                const float2 v = D[i * LDS + j];
                const float m = v.x * v.x + v.y * v.y;
                if (m > best) {
                    best = m;
                    bi = i;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) {
                    best = ob;
                    bi = oi;
                }
            }
            if (tid == 0) piv_row = bi;
        }
        __syncthreads();
        const int p = piv_row;
        if (p != j) {
            for (int c = tid; c < nb; c += blockDim.x) {
                const float2 t = D[j * LDS + c];
                D[j * LDS + c] = D[p * LDS + c];
                D[p * LDS + c] = t;
            }
            if (tid == 0) {
                const int t = lp[j];
                lp[j] = lp[p];
                lp[p] = t;
            }
        }
        __syncthreads();
        float2 pv = D[j * LDS + j];
        if (pv.x == 0.f && pv.y == 0.f) {
            if (tid == 0) atomicCAS(info, 0, k0 + j + 1);
            pv = make_float2(1e-30f, 0.f);
        }
        const float2 ipv = cinv(pv);
        __syncthreads();  // every thread has read the pivot
        for (int i = j + 1 + tid; i < nb; i += blockDim.x) D[i * LDS + j] = cm(D[i * LDS + j], ipv);
        if (tid == 0) D[j * LDS + j] = pv;
        __syncthreads();
        const int w = nb - j - 1;
        for (int q = tid; q < w * w; q += blockDim.x) {
            const int i = j + 1 + q / w, c = j + 1 + q % w;
            const float2 l = D[i * LDS + j], u = D[j * LDS + c];
            D[i * LDS + c] = make_float2(D[i * LDS + c].x - (l.x * u.x - l.y * u.y),
                                         D[i * LDS + c].y - (l.x * u.y + l.y * u.x));
        }
        __syncthreads();
    }
    for (int q = tid; q < nb * nb; q += blockDim.x) {
        const int i = q / nb, j = q % nb;
        A[(size_t)(k0 + i) * n + k0 + j] = D[i * LDS + j];
    }
    if (tid < nb) {
        perm[k0 + tid] = k0 + lp[tid];
        invd[tid] = cinv(D[tid * LDS + tid]);
    }
    __syncthreads();
    // column c of L^-1 (threads 0..63) and of U^-1 (threads 64..127); entries
    // outside the block (nb < NB) stay zero
    if (tid < NB) {
        const int c = tid;
        for (int i = 0; i < NB; ++i) {
            float2 s = make_float2(0.f, 0.f);
            for (int k = 0; k < i; ++k) s = cfma(D[i * LDS + k], WL[k * LDS + c], s);
            float2 x = make_float2(0.f, 0.f);
            if (c < nb && i < nb && i >= c) x = (i == c) ? make_float2(1.f, 0.f) : make_float2(-s.x, -s.y);
            WL[i * LDS + c] = x;
        }
    } else if (tid < 2 * NB) {
        const int c = tid - NB;
        for (int i = NB - 1; i >= 0; --i) {
            float2 s = make_float2(0.f, 0.f);
            for (int k = i + 1; k < NB; ++k) s = cfma(D[i * LDS + k], WU[k * LDS + c], s);
            float2 x = make_float2(0.f, 0.f);
            if (c < nb && i <= c) x = cm(make_float2((i == c ? 1.f : 0.f) - s.x, -s.y), invd[i]);
            WU[i * LDS + c] = x;
        }
    }
    __syncthreads();
    const size_t kb = (size_t)(k0 / NB) * NB * NB;
    for (int q = tid; q < NB * NB; q += blockDim.x) {
        const int i = q / NB, j = q % NB;
        linv[kb + q] = WL[i * LDS + j];
        uinv[kb + q] = WU[i * LDS + j];
    }
}

// rows [k0, k0 + nb) of the columns outside the diagonal block, reordered
// by the block's permutation; CTA per 32 columns
__global__ void __launch_bounds__(256) k_lu_rowperm(float2* __restrict__ A, int n, int k0, int nb,
                                                    const int* __restrict__ perm)
{
    __shared__ float2 T[NB][33];
    __shared__ int moved;
    if (threadIdx.x == 0) moved = 0;
    __syncthreads();
    if (threadIdx.x < nb && perm[k0 + threadIdx.x] != k0 + (int)threadIdx.x) moved = 1;
    __syncthreads();
    if (!moved) return;
    const int cc0 = blockIdx.x * 32;
    for (int q = threadIdx.x; q < nb * 32; q += blockDim.x) {
        const int r = q / 32, cl = q % 32, cc = cc0 + cl;
        if (cc >= n - nb) continue;
        const int c = cc < k0 ? cc : cc + nb;
        T[r][cl] = A[(size_t)perm[k0 + r] * n + c];
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nb * 32; q += blockDim.x) {
        const int r = q / 32, cl = q % 32, cc = cc0 + cl;
        if (cc >= n - nb) continue;
        const int c = cc < k0 ? cc : cc + nb;
        A[(size_t)(k0 + r) * n + c] = T[r][cl];
    }
}

// mode 0: U12 = L11^-1 A12 on the 64-column chunk blockIdx.x of [k0 + nb, n);
// mode 1: L21 = A21 U11^-1 on the 64-row chunk blockIdx.x of [k0 + nb, n)
__global__ void __launch_bounds__(256) k_lu_small(float2* __restrict__ A, int n, int k0, int nb,
                                                  const float2* __restrict__ inv, int mode)
{
    extern __shared__ float2 s_lu[];
    float2* X = s_lu;           // [NB][LDS] the inverse
    float2* Y = X + NB * LDS;   // [NB][LDS] the panel chunk
    const int k1 = k0 + nb, tid = threadIdx.x;
    const int e0 = k1 + blockIdx.x * NB;  // first column (mode 0) or row (mode 1) of the chunk
    const int ne = min(NB, n - e0);
    const float2* iv = inv + (size_t)(k0 / NB) * NB * NB;
    for (int q = tid; q < NB * NB; q += blockDim.x) {
        const int i = q / NB, j = q % NB;
        X[i * LDS + j] = iv[q];
        float2 v = make_float2(0.f, 0.f);
        if (mode == 0) {
            if (i < nb && j < ne) v = A[(size_t)(k0 + i) * n + e0 + j];
        } else {
            if (i < ne && j < nb) v = A[(size_t)(e0 + i) * n + k0 + j];
        }
        Y[i * LDS + j] = v;
    }
    __syncthreads();
    const int tx = tid & 15, ty = tid >> 4;
    float2 acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = make_float2(0.f, 0.f);
    for (int k = 0; k < NB; ++k) {
        float2 l[4], r[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) l[a] = mode == 0 ? X[(ty + 16 * a) * LDS + k] : Y[(ty + 16 * a) * LDS + k];
#pragma unroll
        for (int b = 0; b < 4; ++b) r[b] = mode == 0 ? Y[k * LDS + tx + 16 * b] : X[k * LDS + tx + 16 * b];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = cfma(l[a], r[b], acc[a][b]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int i = ty + 16 * a, j = tx + 16 * b;
            if (mode == 0) {
                if (i < nb && j < ne) A[(size_t)(k0 + i) * n + e0 + j] = acc[a][b];
            } else {
                if (i < ne && j < nb) A[(size_t)(e0 + i) * n + k0 + j] = acc[a][b];
            }
        }
}

// trailing update A22 -= L21 U12 on the 64 x 64 tile (blockIdx.y, blockIdx.x +
// ct0) of [k1, n)^2, K = nb <= 64
__global__ void __launch_bounds__(256) k_lu_update(float2* __restrict__ A, int n, int k0, int nb, int ct0)
{
    extern __shared__ float2 s_lu[];
    float2* As = s_lu;          // [k][LDS]: L21 tile, transposed
    float2* Bs = As + NB * LDS; // [k][LDS]: U12 tile
    const int k1 = k0 + nb, m = n - k1, tid = threadIdx.x;
    const int r0 = blockIdx.y * NB, c0 = (blockIdx.x + ct0) * NB;
    for (int q = tid; q < NB * NB; q += blockDim.x) {
        const int i = q / NB, k = q % NB;  // L21: row i, column k (coalesced along k)
        As[k * LDS + i] = (r0 + i < m && k < nb) ? A[(size_t)(k1 + r0 + i) * n + k0 + k] : make_float2(0.f, 0.f);
        const int kk = q / NB, j = q % NB;  // U12: row kk, column j (coalesced along j)
        Bs[kk * LDS + j] = (kk < nb && c0 + j < m) ? A[(size_t)(k0 + kk) * n + k1 + c0 + j] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int tx = tid & 15, ty = tid >> 4;
    float2 acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int k = 0; k < NB; ++k) {
        float2 l[4], r[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) l[a] = As[k * LDS + ty + 16 * a];
#pragma unroll
        for (int b = 0; b < 4; ++b) r[b] = Bs[k * LDS + tx + 16 * b];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = cfma(l[a], r[b], acc[a][b]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int i = r0 + ty + 16 * a, j = c0 + tx + 16 * b;
            if (i < m && j < m) {
                float2* p = A + (size_t)(k1 + i) * n + k1 + j;
                const float2 v = *p;
                *p = make_float2(v.x - acc[a][b].x, v.y - acc[a][b].y);
            }
        }
}

// W[r][i] = B[r][perm[i]]
__global__ void k_lu_gather(const float2* __restrict__ B, const int* __restrict__ perm, int n, int nrhs,
                            float2* __restrict__ W)
{
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (size_t)n * nrhs) return;
    const int r = (int)(id / n), i = (int)(id % n);
    W[id] = B[(size_t)r * n + perm[i]];
}

constexpr int RC = 8;  // right-hand sides per CTA of a sweep step

// One step of the forward (dir 0, L) or backward (dir 1, U) sweep for block
// k0: x = inv W[block] for the CTA's right-hand sides (CTA x = 0 stores it in
// Out), then W[rows] -= A[rows][block] x on the CTA's 64-row chunk of the rows
// after (dir 0) or before (dir 1) the block.  The block's inverse, then the
// chunk's 64 x 64 slice of A, are staged in shared memory.
__global__ void __launch_bounds__(256) k_lu_sweep(const float2* __restrict__ A, int n, int k0, int nb,
                                                  const float2* __restrict__ inv, int dir, int nrhs,
                                                  float2* __restrict__ W, float2* __restrict__ Out)
{
    __shared__ float2 M[NB][LDS];  // inverse of the block, then the chunk's slice of A
    __shared__ float2 ws[RC][NB];
    __shared__ float2 xs[RC][NB];
    const int tid = threadIdx.x;
    const int rb = blockIdx.y * RC, nr = min(RC, nrhs - rb);
    const float2* iv = inv + (size_t)(k0 / NB) * NB * NB;
    for (int q = tid; q < NB * NB; q += blockDim.x) M[q / NB][q % NB] = iv[q];
    for (int q = tid; q < RC * NB; q += blockDim.x) {
        const int r = q / NB, j = q % NB;
        ws[r][j] = (r < nr && j < nb) ? W[(size_t)(rb + r) * n + k0 + j] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int q = tid; q < RC * NB; q += blockDim.x) {
        const int r = q / NB, i = q % NB;
        float2 s = make_float2(0.f, 0.f);
#pragma unroll 8
        for (int j = 0; j < NB; ++j) s = cfma(M[i][j], ws[r][j], s);
        xs[r][i] = s;
    }
    __syncthreads();
    if (blockIdx.x == 0)
        for (int q = tid; q < RC * NB; q += blockDim.x) {
            const int r = q / NB, i = q % NB;
            if (r < nr && i < nb) Out[(size_t)(rb + r) * n + k0 + i] = xs[r][i];
        }
    // rows of this CTA's chunk
    const int lo = dir == 0 ? k0 + nb : 0, hi = dir == 0 ? n : k0;
    const int m0 = lo + blockIdx.x * NB;
    const int nm = min(NB, hi - m0);
    if (nm <= 0) return;  // uniform over the CTA; no barrier follows
    for (int q = tid; q < NB * NB; q += blockDim.x) {
        const int i = q / NB, j = q % NB;
        M[i][j] = (i < nm && j < nb) ? A[(size_t)(m0 + i) * n + k0 + j] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int q = tid; q < nm * nr; q += blockDim.x) {
        const int i = q % nm, r = q / nm;
        float2 s = make_float2(0.f, 0.f);
#pragma unroll 8
        for (int j = 0; j < NB; ++j) s = cfma(M[i][j], xs[r][j], s);
        float2* w = W + (size_t)(rb + r) * n + m0 + i;
        *w = make_float2(w->x - s.x, w->y - s.y);
    }
}

}  // namespace

size_t lu_bytes(int n)
{
    const size_t nblk = (size_t)(n + NB - 1) / NB;
    return sizeof(float2) * (size_t)n * n + sizeof(int) * (size_t)n + 2 * sizeof(float2) * nblk * NB * NB + 256 * 4;
}

static emfa_status_t lu_set_smem(Ctx* c)
{
    EMFA_TRY(ensure_smem(c, k_lu_diag, 3 * sizeof(float2) * NB * LDS));
    EMFA_TRY(ensure_smem(c, k_lu_small, 2 * sizeof(float2) * NB * LDS));
    return ensure_smem(c, k_lu_update, 2 * sizeof(float2) * NB * LDS);
}

emfa_status_t lu_factor(Ctx* c, const void* Z, int n, LuFactor& F, cudaStream_t st)
{
    if (n <= 0) {
        set_error(c, "lu_factor: n must be positive");
        return EMFA_ERR_INVALID;
    }
    EMFA_TRY(lu_set_smem(c));
    F.n = n;
    F.nblk = (n + NB - 1) / NB;
    EMFA_TRY(F.a.alloc(c, sizeof(float2) * (size_t)n * n));
    EMFA_TRY(F.perm.alloc(c, sizeof(int) * (size_t)n));
    EMFA_TRY(F.linv.alloc(c, sizeof(float2) * (size_t)F.nblk * NB * NB));
    EMFA_TRY(F.uinv.alloc(c, sizeof(float2) * (size_t)F.nblk * NB * NB));
    EMFA_TRY(F.info.alloc(c, 256));
    float2* A = dptr<float2>(F.a);
    if (Z != A) EMFA_CUDA(c, cudaMemcpyAsync(A, Z, sizeof(float2) * (size_t)n * n, cudaMemcpyDeviceToDevice, st));
    EMFA_CUDA(c, cudaMemsetAsync(F.info.ptr, 0, sizeof(int), st));
    const size_t s2 = 2 * sizeof(float2) * NB * LDS, s3 = 3 * sizeof(float2) * NB * LDS;
    // helper stream and events of the lookahead (released on every return)
    struct Aux {
        cudaStream_t s = nullptr;
        cudaEvent_t panel = nullptr, rest = nullptr;
        ~Aux()
        {
            if (panel) cudaEventDestroy(panel);
            if (rest) cudaEventDestroy(rest);
            if (s) cudaStreamDestroy(s);
        }
    } aux;
    if (F.nblk > 2) {
        EMFA_CUDA(c, cudaStreamCreateWithFlags(&aux.s, cudaStreamNonBlocking));
        EMFA_CUDA(c, cudaEventCreateWithFlags(&aux.panel, cudaEventDisableTiming));
        EMFA_CUDA(c, cudaEventCreateWithFlags(&aux.rest, cudaEventDisableTiming));
    }
    auto diag = [&](int kb) {
        const int k0 = kb * NB, nb = std::min(NB, n - k0);
        k_lu_diag<<<1, 256, s3, st>>>(A, n, k0, nb, dptr<int>(F.perm), dptr<float2>(F.linv), dptr<float2>(F.uinv),
                                      dptr<int>(F.info));
        c->kernel_launches += 1;
    };
    diag(0);
    for (int kb = 0; kb < F.nblk; ++kb) {
        const int k0 = kb * NB, nb = std::min(NB, n - k0), rest = n - k0 - nb;
        if (n - nb > 0) {
            k_lu_rowperm<<<(n - nb + 31) / 32, 256, 0, st>>>(A, n, k0, nb, dptr<int>(F.perm));
            c->kernel_launches += 1;
        }
        if (rest <= 0) continue;
        const unsigned ch = (unsigned)((rest + NB - 1) / NB);
        k_lu_small<<<ch, 256, s2, st>>>(A, n, k0, nb, dptr<float2>(F.linv), 0);
        k_lu_small<<<ch, 256, s2, st>>>(A, n, k0, nb, dptr<float2>(F.uinv), 1);
        c->kernel_launches += 2;
        if (aux.s && ch > 1) {
            // the next block's columns, then its diagonal block on st while
            // the other columns are updated on the helper stream
            k_lu_update<<<dim3(1, ch), 256, s2, st>>>(A, n, k0, nb, 0);
            EMFA_CUDA(c, cudaEventRecord(aux.panel, st));
            EMFA_CUDA(c, cudaStreamWaitEvent(aux.s, aux.panel, 0));
            k_lu_update<<<dim3(ch - 1, ch), 256, s2, aux.s>>>(A, n, k0, nb, 1);
            EMFA_CUDA(c, cudaEventRecord(aux.rest, aux.s));
            diag(kb + 1);
            EMFA_CUDA(c, cudaStreamWaitEvent(st, aux.rest, 0));
        } else {
            k_lu_update<<<dim3(ch, ch), 256, s2, st>>>(A, n, k0, nb, 0);
            diag(kb + 1);
        }
        c->kernel_launches += aux.s && ch > 1 ? 2 : 1;
    }
    EMFA_CUDA(c, cudaGetLastError());
    return EMFA_OK;
}

emfa_status_t lu_zero_pivot(Ctx* c, const LuFactor& F, int* first, cudaStream_t st)
{
    EMFA_CUDA(c, cudaMemcpyAsync(first, F.info.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    return EMFA_OK;
}

emfa_status_t lu_apply(Ctx* c, const LuFactor& F, const float2* B, int nrhs, float2* X, float2* work,
                       cudaStream_t st)
{
    const int n = F.n;
    const size_t tot = (size_t)n * nrhs;
    float2* W = work;           // permuted right-hand sides, then the forward sweep's residue
    float2* Y = work + tot;     // L^-1 P b
    const float2* A = dptr<float2>(F.a);
    k_lu_gather<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(B, dptr<int>(F.perm), n, nrhs, W);
    const unsigned gy = (unsigned)((nrhs + RC - 1) / RC);
    for (int kb = 0; kb < F.nblk; ++kb) {
        const int k0 = kb * NB, nb = std::min(NB, n - k0), rows = n - k0 - nb;
        k_lu_sweep<<<dim3((unsigned)std::max(1, (rows + NB - 1) / NB), gy), 256, 0, st>>>(
            A, n, k0, nb, dptr<float2>(F.linv), 0, nrhs, W, Y);
    }
    for (int kb = F.nblk - 1; kb >= 0; --kb) {
        const int k0 = kb * NB, nb = std::min(NB, n - k0);
        k_lu_sweep<<<dim3((unsigned)std::max(1, (k0 + NB - 1) / NB), gy), 256, 0, st>>>(
            A, n, k0, nb, dptr<float2>(F.uinv), 1, nrhs, Y, X);
    }
    c->kernel_launches += 1 + 2 * F.nblk;
    EMFA_CUDA(c, cudaGetLastError());
    return EMFA_OK;
}

}  // namespace emfa
