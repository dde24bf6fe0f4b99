// Dense LU factorisation of the impedance matrix, for solves that factor once
// and then solve and refine (the batched EFIE problems, whose restarted
// Krylov solves need hundreds of iterations).  The reference has no dense
// direct solver on this path: EMSolver/EFIE.cpp:89 keeps a commented-out
// Eigen LU, and its EFIE/CFIE solves are GMRES/BiCGStab only.
//
// Factorisation, FP32 complex, blocked right-looking, block LU_NB = 64, row
// exchanges within each diagonal block (the rows of block k only trade places
// among themselves).  One step per diagonal block:
//   k_lu_diag     one CTA: pivoted LU of the diagonal block in registers,
//                 then explicit inverses of its unit-lower and upper factors
//   k_lu_panels   U12 = L11^-1 P A12 and L21 = A21 U11^-1 with those
//                 inverses (P the block's row exchange, applied by reading
//                 A12 through the permutation), and their split-FP16
//                 operand planes, scaled per column / row by powers of two
//   k_lu_update_tc  A22 -= L21 U12 on the tensor cores (tcgen05, K = 128
//                 real per block), tiles of 256 rows x 64 complex columns of
//                 A22 moved through shared memory by TMA
// with a one-block lookahead: the next block's 64 columns are updated first,
// and that block's k_lu_diag (one CTA, latency bound) runs on a high-priority
// stream while the remaining columns are updated.  While two or more blocks
// follow, blocks go in pairs: the first block updates only the second
// block's columns and rows, and one pass with both blocks' panels
// (k_lu_pack2, K = 128 complex) updates the rest, so A22 is read and
// written once per two blocks.  The row exchanges reach
// the columns left of each block in one pass at the end (k_lu_rowperm_left).
// Rows of the factor are padded to an even number of complex elements
// (16-byte TMA strides).
// Solve for many right-hand sides (RHS-major, (r, u) at r n + u): gather by
// the row permutation, then one launch for the forward (L) and one for the
// backward (U) sweep (k_lu_wave): a CTA per row block, in wavefront order,
// applies the block's explicit inverse once the blocks before it are solved.
//
// A pivot that is exactly zero is replaced by 1e-30 and recorded in the
// factor's info word, so the caller can fall back to an iterative solve.
#include "emfa_internal.cuh"
#include "gemm.cuh"
#include "lu.cuh"
#include "tcgen05.cuh"

#include <cuda_fp16.h>

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
//
// Factorisation by 16-column panels.  Rows never move: a pivot row only
// leaves the active set, and its step number is its position in the factor
// (ord, pos).  Per panel:
//   1. warp 0 holds the panel (lane l: rows l and l + 32, 16 columns) in
//      registers and runs its 16 column steps with warp barriers only: the
//      pivot is the largest |.|^2 among active rows (a 64-bit key, |.|^2 bits
//      then the inverted row, so the lowest row wins ties, reduced by
//      shuffles); the pivot lane publishes its row, every lane scales and
//      updates its own rows
//   2. all warps: the panel's pivot rows on the columns to its right
//      (unit-lower triangular solve, a thread per column), then the rank-16
//      update of the active rows there
// Inverses: the 8 x 8 diagonal blocks of L and U by substitution (a thread
// per column), then three merge levels of the 2 x 2 block inverse,
//   [L11 0; L21 L22]^-1 = [X11 0; -X22 L21 X11  X22],
//   [U11 U12; 0 U22]^-1 = [Y11 -Y11 U12 Y22; 0 Y22],
// each two rounds of small products over all block pairs at once.
constexpr int DIAG_THREADS = 512;
constexpr int PW = 16;  // panel width

// One merge level of the blocked inverses: for every pair of b-blocks on the
// diagonal, T = L21 X11 and T = Y11 U12, then X21 = -X22 T and Y12 = -T Y22.
// A thread takes NI items (an entry of T, then of X21 or Y12) and runs their
// b-long sums side by side.
template <int b>
__device__ __forceinline__ void diag_merge(const float2* __restrict__ D, float2* __restrict__ WL,
                                           float2* __restrict__ WU, float2* __restrict__ TM)
{
    constexpr int pairs = (NB / 2) / b, per = pairs * b * b, NI = (2 * per + DIAG_THREADS - 1) / DIAG_THREADS;
    const int tid = threadIdx.x;
    int mat[NI], pr[NI], r[NI], c[NI];
#pragma unroll
    for (int it = 0; it < NI; ++it) {
        const int q = tid + it * DIAG_THREADS;  // 2 per is a multiple of the block: every q is an item
        const int rem = q % per;
        mat[it] = q / per;
        pr[it] = rem / (b * b);
        r[it] = (rem / b) % b;
        c[it] = rem % b;
    }
    float2 s[NI];
#pragma unroll
    for (int it = 0; it < NI; ++it) s[it] = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int k = 0; k < b; ++k)
#pragma unroll
        for (int it = 0; it < NI; ++it) {
            const int i0 = pr[it] * 2 * b;
            if (mat[it] == 0)
                s[it] = cfma(D[(i0 + b + r[it]) * LDS + i0 + k], WL[(i0 + k) * LDS + i0 + c[it]], s[it]);
            else
                s[it] = cfma(WU[(i0 + r[it]) * LDS + i0 + k], D[(i0 + k) * LDS + i0 + b + c[it]], s[it]);
        }
#pragma unroll
    for (int it = 0; it < NI; ++it) TM[tid + it * DIAG_THREADS] = s[it];
    __syncthreads();
#pragma unroll
    for (int it = 0; it < NI; ++it) s[it] = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int k = 0; k < b; ++k)
#pragma unroll
        for (int it = 0; it < NI; ++it) {
            const int i0 = pr[it] * 2 * b;
            const float2* T = TM + mat[it] * per + pr[it] * b * b;
            if (mat[it] == 0)
                s[it] = cfma(WL[(i0 + b + r[it]) * LDS + i0 + b + k], T[k * b + c[it]], s[it]);
            else
                s[it] = cfma(T[r[it] * b + k], WU[(i0 + b + k) * LDS + i0 + b + c[it]], s[it]);
        }
#pragma unroll
    for (int it = 0; it < NI; ++it) {
        const int i0 = pr[it] * 2 * b;
        if (mat[it] == 0)
            WL[(i0 + b + r[it]) * LDS + i0 + c[it]] = make_float2(-s[it].x, -s[it].y);
        else
            WU[(i0 + r[it]) * LDS + i0 + b + c[it]] = make_float2(-s[it].x, -s[it].y);
    }
    __syncthreads();
}

__global__ void __launch_bounds__(DIAG_THREADS) k_lu_diag(float2* __restrict__ A, int n, int lda, int k0, int nb,
                                                          int* __restrict__ perm, float2* __restrict__ linv,
                                                          float2* __restrict__ uinv, int* __restrict__ info)
{
    extern __shared__ float2 s_lu[];
    float2* D = s_lu;               // [NB][LDS] the factors, in factor order
    float2* WL = D + NB * LDS;      // [NB][LDS] the block by original row while it is factored, then L^-1
    float2* WU = WL + NB * LDS;     // [NB][LDS] U^-1
    float2* TM = WU + NB * LDS;     // [2048] products of a merge level
    __shared__ float2 prow[PW];     // the step's pivot row within the panel
    __shared__ int pos[NB];         // factor position of each row (NB + row while active)
    __shared__ int ord[NB];         // row at each factor position
    __shared__ float2 invd[NB];
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
    float2* W = WL;
    for (int q = tid; q < NB * NB; q += blockDim.x) {
        const int i = q / NB, j = q % NB;
        W[i * LDS + j] = (i < nb && j < nb) ? A[(size_t)(k0 + i) * lda + k0 + j] : make_float2(0.f, 0.f);
    }
    if (tid < NB) pos[tid] = NB + tid;
    __syncthreads();
    unsigned act = (l < nb ? 1u : 0u) | (l + 32 < nb ? 2u : 0u);  // warp 0: rows l, l + 32 still active
    for (int c0 = 0; c0 < nb; c0 += PW) {
        if (w == 0) {
            float2 x[2][PW];
#pragma unroll
            for (int r = 0; r < 2; ++r)
#pragma unroll
                for (int c = 0; c < PW; ++c) x[r][c] = W[(l + 32 * r) * LDS + c0 + c];
#pragma unroll
            for (int jj = 0; jj < PW; ++jj) {
                const int j = c0 + jj;
                if (j < nb) {  // uniform
                    unsigned long long key = 0ull;
#pragma unroll
                    for (int r = 0; r < 2; ++r)
                        if (act >> r & 1) {
                            const float m2 = x[r][jj].x * x[r][jj].x + x[r][jj].y * x[r][jj].y;
                            const unsigned long long kk =
                                (unsigned long long)__float_as_uint(m2) << 32 | (unsigned)(NB - 1 - (l + 32 * r));
                            key = kk > key ? kk : key;
                        }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
                        key = ok > key ? ok : key;
                    }
                    // a key is nonzero for any active row but row 63 with a zero
                    // entry, which the empty key names as well
                    const int p = NB - 1 - (int)(key & 0xffffffffull);
                    const int pl = p & 31, pr = p >> 5;
                    if (l == pl) {
#pragma unroll
                        for (int c = jj; c < PW; ++c) prow[c] = pr ? x[1][c] : x[0][c];
                    }
                    __syncwarp();
                    float2 pv = prow[jj];
                    if (pv.x == 0.f && pv.y == 0.f) {
                        if (l == 0) atomicCAS(info, 0, k0 + j + 1);
                        pv = make_float2(1e-30f, 0.f);
                        if (l == pl) {
                            if (pr)
                                x[1][jj] = pv;
                            else
                                x[0][jj] = pv;
                        }
                    }
                    if (l == pl) act &= ~(1u << pr);
                    const float2 ipv = cinv(pv);
#pragma unroll
                    for (int r = 0; r < 2; ++r)
                        if (act >> r & 1) {
                            const float2 lm = cm(x[r][jj], ipv);
                            x[r][jj] = lm;
#pragma unroll
                            for (int c = jj + 1; c < PW; ++c) {
                                const float2 u = prow[c];
                                x[r][c] = make_float2(x[r][c].x - (lm.x * u.x - lm.y * u.y),
                                                      x[r][c].y - (lm.x * u.y + lm.y * u.x));
                            }
                        }
                    if (l == 0) {
                        ord[j] = p;
                        pos[p] = j;
                    }
                    __syncwarp();
                }
            }
#pragma unroll
            for (int r = 0; r < 2; ++r)
#pragma unroll
                for (int c = 0; c < PW; ++c) W[(l + 32 * r) * LDS + c0 + c] = x[r][c];
        }
        __syncthreads();
        const int c1 = c0 + PW, pe = min(PW, nb - c0);  // columns right of the panel; its pivots
        if (c1 < nb) {
            // the panel's pivot rows on the columns right of it: forward
            // substitution with the panel's unit-lower part, four lanes per
            // column (lane sub keeps the solved entries k = sub mod 4)
            if (w < (4 * (nb - c1) + 31) / 32) {  // whole warps
                const int sub = tid & 3, c = c1 + (tid >> 2), cc = min(c, NB - 1);
                float2 u[PW / 4];
#pragma unroll
                for (int t = 0; t < PW / 4; ++t) u[t] = make_float2(0.f, 0.f);
#pragma unroll
                for (int i = 0; i < PW; ++i) {
                    if (i < pe) {  // uniform
                        const int ri = ord[c0 + i];
                        float2 part = make_float2(0.f, 0.f);
#pragma unroll
                        for (int t = 0; t < PW / 4; ++t)
                            if (sub + 4 * t < i) part = cfma(W[ri * LDS + c0 + sub + 4 * t], u[t], part);
                        part.x += __shfl_xor_sync(0xffffffffu, part.x, 1);
                        part.y += __shfl_xor_sync(0xffffffffu, part.y, 1);
                        part.x += __shfl_xor_sync(0xffffffffu, part.x, 2);
                        part.y += __shfl_xor_sync(0xffffffffu, part.y, 2);
                        const float2 a = W[ri * LDS + cc];
                        const float2 v = make_float2(a.x - part.x, a.y - part.y);
                        if ((i & 3) == sub) u[i >> 2] = v;
                        if (sub == 0 && c < nb) W[ri * LDS + c] = v;
                    }
                }
            }
            __syncthreads();
            // rank-pe update of the active rows right of the panel
            const int nc = nb - c1;
            for (int q = tid; q < NB * nc; q += blockDim.x) {
                const int r = q / nc, c = c1 + q % nc;
                if (r >= nb || pos[r] < NB) continue;
                float2 s = W[r * LDS + c];
                for (int k = 0; k < pe; ++k) {
                    const float2 lk = W[r * LDS + c0 + k], uk = W[ord[c0 + k] * LDS + c];
                    s = make_float2(s.x - (lk.x * uk.x - lk.y * uk.y), s.y - (lk.x * uk.y + lk.y * uk.x));
                }
                W[r * LDS + c] = s;
            }
            __syncthreads();
        }
    }
    // the factors in factor order: shared memory (rows and columns past nb
    // are zero) and A
    for (int q = tid; q < NB * NB; q += blockDim.x) {
        const int r = q / NB, c = q % NB;
        const int i = r < nb ? pos[r] : r;
        const float2 v = W[r * LDS + c];
        D[i * LDS + c] = v;
        if (r < nb && c < nb) A[(size_t)(k0 + i) * lda + k0 + c] = v;
    }
    if (tid < nb) perm[k0 + tid] = k0 + ord[tid];
    __syncthreads();
    for (int q = tid; q < NB * LDS; q += blockDim.x) {
        WL[q] = make_float2(0.f, 0.f);
        WU[q] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (tid < NB) invd[tid] = tid < nb ? cinv(D[tid * LDS + tid]) : make_float2(1.f, 0.f);
    if (tid >= nb && tid < NB) D[tid * LDS + tid] = make_float2(1.f, 0.f);  // identity past the block
    __syncthreads();
    // 8 x 8 diagonal blocks: threads 0..63 columns of L^-1, 64..127 of U^-1
    if (tid < 2 * NB) {
        const int t = tid & 63, b0 = t & ~7, c = t & 7;
        float2 x[8];
        if (tid < NB) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                float2 s = make_float2(0.f, 0.f);
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (k >= c && k < i) s = cfma(D[(b0 + i) * LDS + b0 + k], x[k], s);
                x[i] = i < c ? make_float2(0.f, 0.f) : i == c ? make_float2(1.f, 0.f) : make_float2(-s.x, -s.y);
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) WL[(b0 + i) * LDS + b0 + c] = x[i];
        } else {
#pragma unroll
            for (int i = 7; i >= 0; --i) {
                float2 s = make_float2(0.f, 0.f);
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (k > i && k <= c) s = cfma(D[(b0 + i) * LDS + b0 + k], x[k], s);
                x[i] = i > c ? make_float2(0.f, 0.f)
                             : cm(make_float2((i == c ? 1.f : 0.f) - s.x, -s.y), invd[b0 + i]);
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) WU[(b0 + i) * LDS + b0 + c] = x[i];
        }
    }
    __syncthreads();
    diag_merge<8>(D, WL, WU, TM);
    diag_merge<16>(D, WL, WU, TM);
    diag_merge<32>(D, WL, WU, TM);
    const size_t kb = (size_t)(k0 / NB) * NB * NB;
    for (int q = tid; q < NB * NB; q += blockDim.x) {
        const int i = q / NB, j = q % NB;
        const bool in = i < nb && j < nb;
        linv[kb + q] = in ? WL[i * LDS + j] : make_float2(0.f, 0.f);
        uinv[kb + q] = in ? WU[i * LDS + j] : make_float2(0.f, 0.f);
    }
}

// The row exchanges of every diagonal block applied to the columns left of
// the block (the factor's L part), once the factorisation is done: the
// exchanges stay within a block and those columns are final by then.  CTA
// per (32 columns, block).
__global__ void __launch_bounds__(256) k_lu_rowperm_left(float2* __restrict__ A, int n, int lda,
                                                         const int* __restrict__ perm)
{
    __shared__ float2 T[NB][33];
    __shared__ int moved;
    const int k0 = blockIdx.y * NB, nb = min(NB, n - k0), c0 = blockIdx.x * 32;
    if (c0 >= k0) return;  // uniform over the CTA
    if (threadIdx.x == 0) moved = 0;
    __syncthreads();
    if (threadIdx.x < nb && perm[k0 + threadIdx.x] != k0 + (int)threadIdx.x) moved = 1;
    __syncthreads();
    if (!moved) return;
    for (int q = threadIdx.x; q < nb * 32; q += blockDim.x) {
        const int r = q / 32, c = c0 + q % 32;
        if (c < k0) T[r][q % 32] = A[(size_t)perm[k0 + r] * lda + c];
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nb * 32; q += blockDim.x) {
        const int r = q / 32, c = c0 + q % 32;
        if (c < k0) A[(size_t)(k0 + r) * lda + c] = T[r][q % 32];
    }
}

// ---------------------------------------------------------------------------
// Trailing update on the tensor cores: A22 -= L21 U12 as one real GEMM with
// split-FP16 operands (tcgen05.mma kind::f16, FP32 accumulation in tensor
// memory).  The accumulator is laid out transposed, D[real column][row], so
// that the epilogue's 32 lanes read and write 32 consecutive floats of a row
// of A22 (coalesced):
//   U operand row 2j   = t_j (Re u_kj, -Im u_kj)_k     (K = 2 nb = 128 halves)
//   U operand row 2j+1 = t_j (Im u_kj,  Re u_kj)_k
//   L operand row i    = s_i (Re l_ik,  Im l_ik)_k
//   D[2j + e][i] = t_j s_i (Re, Im)_e (L21 U12)_ij
// with t_j, s_i powers of two per column of U12 and per row of L21 (largest
// |Re|, |Im| scaled into [2^14, 2^15)), each operand split into hi = fp16(x)
// and lo = fp16(x - hi), and D = Uh Lh + Uh Ll + Ul Lh (the lo-lo term is
// below 2^-21 of the product).
// ---------------------------------------------------------------------------
namespace lutc {
constexpr int TM = 128;                                  // real columns of A22 per tile (MMA M): 64 complex
constexpr int TN = 256;                                  // rows of A22 per tile (MMA N)
constexpr int KH = 4 * NB;                               // halves per operand row: two blocks' panels
constexpr int U_BYTES = TM * 128;                        // one 64-half K slice of one U plane
constexpr int L_BYTES = TN * 128;                        // one K slice of one L plane
constexpr int STAGE = 2 * U_BYTES + 2 * L_BYTES;         // both planes of both operands: 96 KB
constexpr int C_BYTES = 64 * 128 * 4;                    // 64 rows x 64 complex of A22: three fill the stage
constexpr int SMEM = STAGE + 1024 /*align*/ + 256 /*barriers*/;
constexpr int THREADS = 320;                             // producer, MMA, 8 epilogue warps
constexpr int TMEM_COLS = TN;
}  // namespace lutc

__device__ __forceinline__ float2 col_max_scale(float m)
{
    int e = 0;
    frexpf(m, &e);  // m = f 2^e, f in [0.5, 1); m = 0 gives e = 0
    return make_float2(ldexpf(1.f, 15 - e), ldexpf(1.f, e - 15));
}

__device__ __forceinline__ uint32_t h2_bits(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }

// hi/lo FP16 pairs of (a, b)
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo)
{
    const __half ha = __float2half_rn(a), hb = __float2half_rn(b);
    hi = h2_bits(__halves2half2(ha, hb));
    lo = h2_bits(__halves2half2(__float2half_rn(a - __half2float(ha)), __float2half_rn(b - __half2float(hb))));
}

// Panels of step k0, written to A and packed as the trailing update's
// split-FP16 operand planes (rows indexed from k1 = k0 + nb; plane p of the U
// operand starts at row p 2n, of the L operand at row p n):
//   blockIdx.y = 0: U12 = L11^-1 P A12 on the 64-column chunk blockIdx.x,
//                   P the diagonal block's row exchange (row perm[k0 + i] of
//                   A12 is read for row i)
//   blockIdx.y = 1: L21 = A21 U11^-1 on the 64-row chunk blockIdx.x
// The chunk's product is kept in shared memory, scaled per column of U12 /
// row of L21, and written as 16-byte pieces of contiguous operand rows.
__global__ void __launch_bounds__(256) k_lu_panels(float2* __restrict__ A, int n, int lda, int k0, int nb,
                                                   const int* __restrict__ perm, const float2* __restrict__ linv,
                                                   const float2* __restrict__ uinv, __half* __restrict__ Uop,
                                                   __half* __restrict__ Lop, float* __restrict__ inv_t,
                                                   float* __restrict__ inv_s, int pack)
{
    extern __shared__ float2 s_lu[];
    float2* X = s_lu;           // [NB][LDS] the inverse
    float2* Y = X + NB * LDS;   // [NB][LDS] the chunk, then the product
    __shared__ float sc[NB];    // scale of each product column (U12) or row (L21)
    const int mode = blockIdx.y;
    const int k1 = k0 + nb, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int e0 = k1 + blockIdx.x * NB;  // first column (U12) or row (L21) of the chunk
    const int ne = min(NB, n - e0);
    const float2* iv = (mode == 0 ? linv : uinv) + (size_t)(k0 / NB) * NB * NB;
    for (int q = tid; q < NB * NB; q += blockDim.x) {
        const int i = q / NB, j = q % NB;
        X[i * LDS + j] = iv[q];
        float2 v = make_float2(0.f, 0.f);
        if (mode == 0) {
            if (i < nb && j < ne) v = A[(size_t)perm[k0 + i] * lda + e0 + j];
        } else {
            if (i < ne && j < nb) v = A[(size_t)(e0 + i) * lda + k0 + j];
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
    __syncthreads();  // Y is overwritten by the product
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int i = ty + 16 * a, j = tx + 16 * b;
            // entries past the chunk or the block are zero products
            Y[i * LDS + j] = acc[a][b];
            if (mode == 0) {
                if (i < nb && j < ne) A[(size_t)(k0 + i) * lda + e0 + j] = acc[a][b];
            } else {
                if (i < ne && j < nb) A[(size_t)(e0 + i) * lda + k0 + j] = acc[a][b];
            }
        }
    if (!pack) return;  // uniform: the pair's operands are packed by k_lu_pack2
    __syncthreads();
    // scales: per column of U12 (mode 0) or row of L21 (mode 1), 8 per warp
    for (int c = warp * 8; c < warp * 8 + 8; ++c) {
        const float2 a = mode == 0 ? Y[lane * LDS + c] : Y[c * LDS + lane];
        const float2 b = mode == 0 ? Y[(lane + 32) * LDS + c] : Y[c * LDS + lane + 32];
        float mx = fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fmaxf(fabsf(b.x), fabsf(b.y)));
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) {
            const float2 s2 = col_max_scale(mx);
            sc[c] = s2.x;
            if (c < ne) (mode == 0 ? inv_t : inv_s)[e0 - k1 + c] = s2.y;
        }
    }
    __syncthreads();
    if (mode == 0) {
        // item (column c, part e, 16-byte piece ch of the 256-byte row): 4 k values
        for (int q = tid; q < NB * 2 * 16; q += blockDim.x) {
            const int c = q >> 5, e = (q >> 4) & 1, ch = q & 15;
            if (c >= ne) continue;
            const float t = sc[c];
            uint4 h, lo;
            uint32_t* hp = &h.x;
            uint32_t* lp = &lo.x;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float2 v = Y[(4 * ch + u) * LDS + c];
                if (e == 0)
                    split2(t * v.x, -(t * v.y), hp[u], lp[u]);
                else
                    split2(t * v.y, t * v.x, hp[u], lp[u]);
            }
            const size_t r = (size_t)(2 * (e0 - k1 + c) + e);
            reinterpret_cast<uint4*>(Uop + r * lutc::KH)[ch] = h;
            reinterpret_cast<uint4*>(Uop + ((size_t)2 * n + r) * lutc::KH)[ch] = lo;
        }
    } else {
        // item (row i, 16-byte piece ch): 4 k values
        for (int q = tid; q < NB * 16; q += blockDim.x) {
            const int i = q >> 4, ch = q & 15;
            if (i >= ne) continue;
            const float s = sc[i];
            uint4 h, lo;
            uint32_t* hp = &h.x;
            uint32_t* lp = &lo.x;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float2 v = Y[i * LDS + 4 * ch + u];
                split2(s * v.x, s * v.y, hp[u], lp[u]);
            }
            const size_t r = (size_t)(e0 - k1 + i);
            reinterpret_cast<uint4*>(Lop + r * lutc::KH)[ch] = h;
            reinterpret_cast<uint4*>(Lop + ((size_t)n + r) * lutc::KH)[ch] = lo;
        }
    }
}

// Operand planes of a pair of blocks s0 and s0 + 64 for the update of
// [k2, n)^2, k2 = s0 + 128: U operand rows (from k2) hold U12 of both blocks
// (rows s0 .. s0 + 127 of A), L operand rows L21 of both (columns s0 ..
// s0 + 127), K = 128 complex, with one power-of-two scale per column / row
// over both blocks.  blockIdx.y = 0: rows of L21, one warp per row;
// blockIdx.y = 1: 32 columns of U12 per CTA, staged and transposed in
// shared memory.
__global__ void __launch_bounds__(256) k_lu_pack2(const float2* __restrict__ A, int n, int lda, int s0,
                                                  __half* __restrict__ Uop, __half* __restrict__ Lop,
                                                  float* __restrict__ inv_t, float* __restrict__ inv_s)
{
    const int k2 = s0 + 2 * NB, m = n - k2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (blockIdx.y == 0) {
        const int i = blockIdx.x * 8 + warp;
        if (i >= m) return;
        const float2* row = A + (size_t)(k2 + i) * lda + s0 + 4 * lane;
        float2 v[4];
        float mx = 0.f;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            v[u] = row[u];
            mx = fmaxf(mx, fmaxf(fabsf(v[u].x), fabsf(v[u].y)));
        }
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        const float2 sc = col_max_scale(mx);
        if (lane == 0) inv_s[i] = sc.y;
        uint4 h, l;
        uint32_t* hp = &h.x;
        uint32_t* lp = &l.x;
#pragma unroll
        for (int u = 0; u < 4; ++u) split2(sc.x * v[u].x, sc.x * v[u].y, hp[u], lp[u]);
        reinterpret_cast<uint4*>(Lop + (size_t)i * lutc::KH)[lane] = h;
        reinterpret_cast<uint4*>(Lop + ((size_t)n + i) * lutc::KH)[lane] = l;
        return;
    }
    __shared__ float2 T[2 * NB][33];
    __shared__ float ts[32];
    const int j0 = blockIdx.x * 32;
    if (j0 >= m) return;  // uniform over the CTA
    for (int q = threadIdx.x; q < 2 * NB * 32; q += blockDim.x) {
        const int k = q >> 5, c = q & 31;
        T[k][c] = j0 + c < m ? A[(size_t)(s0 + k) * lda + k2 + j0 + c] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int c = warp * 4; c < warp * 4 + 4; ++c) {
        float mx = 0.f;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float2 a = T[lane + 32 * u][c];
            mx = fmaxf(mx, fmaxf(fabsf(a.x), fabsf(a.y)));
        }
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) {
            const float2 sc = col_max_scale(mx);
            ts[c] = sc.x;
            if (j0 + c < m) inv_t[j0 + c] = sc.y;
        }
    }
    __syncthreads();
    // item (column c, part e, 16-byte piece ch of the 512-byte row): 4 k values
    for (int q = threadIdx.x; q < 32 * 2 * 32; q += blockDim.x) {
        const int c = q >> 6, e = (q >> 5) & 1, ch = q & 31, j = j0 + c;
        if (j >= m) continue;
        const float t = ts[c];
        uint4 h, l;
        uint32_t* hp = &h.x;
        uint32_t* lp = &l.x;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float2 v = T[4 * ch + u][c];
            if (e == 0)
                split2(t * v.x, -(t * v.y), hp[u], lp[u]);
            else
                split2(t * v.y, t * v.x, hp[u], lp[u]);
        }
        const size_t r = (size_t)(2 * j + e);
        reinterpret_cast<uint4*>(Uop + r * lutc::KH)[ch] = h;
        reinterpret_cast<uint4*>(Uop + ((size_t)2 * n + r) * lutc::KH)[ch] = l;
    }
}

// A22 -= L21 U12 on the tile of 64 complex columns (blockIdx.x + ct0) and
// 256 rows (blockIdx.y) of [k1, n)^2, two CTAs per SM.  nslices K slices of
// 64 halves: 2 for one block's panels (K = 64 complex), 4 for two blocks'.
//   warp 0      TMA producer: each K slice, once the MMAs of the one before
//               are done, of Uh, Ul (128 rows) and Lh, Ll (256 rows), 128-byte
//               swizzle
//   warp 1      allocates 256 tensor-memory columns; one lane issues
//               tcgen05.mma M = 128, N = 256, K = 16: 12 per slice
//   warps 2..9  epilogue.  Once the MMAs are done, the operand buffer holds
//               three 64-row chunks of the tile of A22 (TMA loads, 32 KB
//               each; the fourth chunk takes the first slot once that slot's
//               store has read it).  Per chunk each warp takes a quadrant of
//               the tensor-memory lanes (32 real columns) and 32 rows and
//               subtracts the scaled accumulator in shared memory; one thread
//               stores the chunk back with TMA.  Rows and columns past the
//               matrix are zero-filled on load and clipped on store.
// Every wait is bounded; on timeout the kernel records a code in *err, skips
// the stores that would follow, drains its copies and MMAs and frees tensor
// memory.
__global__ void __launch_bounds__(lutc::THREADS, 2)
    k_lu_update_tc(const __grid_constant__ CUtensorMap tmU, const __grid_constant__ CUtensorMap tmL,
                   const __grid_constant__ CUtensorMap tmC, int n, int k1, int ct0, int nslices,
                   const float* __restrict__ inv_t, const float* __restrict__ inv_s, int* __restrict__ err)
{
    using namespace tc;
    extern __shared__ uint8_t smem_raw[];
    __shared__ float rs[lutc::TN];  // 1 / s_i of the tile's rows
    __shared__ int eok;
    uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sUh = base;
    uint8_t* sUl = sUh + lutc::U_BYTES;
    uint8_t* sLh = sUl + lutc::U_BYTES;
    uint8_t* sLl = sLh + lutc::L_BYTES;
    uint64_t* full = (uint64_t*)(base + lutc::STAGE);
    uint64_t* empty = full + 1;
    uint64_t* accum = empty + 1;
    uint64_t* cfull = accum + 1;  // [3] chunk slots of A22
    uint32_t* tmem_slot = (uint32_t*)(cfull + 3);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m = n - k1;
    const int cc0 = (blockIdx.x + ct0) * 64, r0 = blockIdx.y * lutc::TN;

    if (threadIdx.x == 0) {
        mbar_init(full, 1);
        mbar_init(empty, 1);
        mbar_init(accum, 1);
        for (int c = 0; c < 3; ++c) mbar_init(cfull + c, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fence_proxy_async();
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(lutc::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    for (int q = threadIdx.x; q < lutc::TN; q += blockDim.x) rs[q] = r0 + q < m ? inv_s[r0 + q] : 0.f;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int issued = 0;
            for (int s = 0; s < nslices; ++s) {
                if (s > 0 && !mbar_wait(empty, (s - 1) & 1, err, 11)) break;
                if (*(volatile int*)err) break;
                mbar_expect_tx(full, lutc::STAGE);
                tma_load_2d(sUh, &tmU, full, 64 * s, 2 * cc0);
                tma_load_2d(sUl, &tmU, full, 64 * s, 2 * n + 2 * cc0);
                tma_load_2d(sLh, &tmL, full, 64 * s, r0);
                tma_load_2d(sLl, &tmL, full, 64 * s, n + r0);
                issued = s + 1;
            }
            // the last issued copy must have landed before the CTA exits
            if (issued) mbar_wait(full, (issued - 1) & 1, err, 12);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_f16(lutc::TM, lutc::TN);
            for (int s = 0; s < nslices; ++s) {
                if (!mbar_wait(full, s & 1, err, 13)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint64_t uh = sw128_desc(smem_u32(sUh)), ul = sw128_desc(smem_u32(sUl));
                const uint64_t lh = sw128_desc(smem_u32(sLh)), ll = sw128_desc(smem_u32(sLl));
#pragma unroll
                for (int k = 0; k < 4; ++k)  // K = 16 halves = 32 bytes per instruction
                    mma_f16(tmem, uh + 2 * k, lh + 2 * k, idesc, (s > 0 || k > 0) ? 1u : 0u);
#pragma unroll
                for (int k = 0; k < 4; ++k) mma_f16(tmem, uh + 2 * k, ll + 2 * k, idesc, 1u);
#pragma unroll
                for (int k = 0; k < 4; ++k) mma_f16(tmem, ul + 2 * k, lh + 2 * k, idesc, 1u);
                if (s + 1 < nslices) mma_commit(empty);
            }
            // every MMA issued must be complete before the epilogue and before
            // tensor memory is released
            mma_commit(accum);
            mbar_wait(accum, 0, err, 14);
        }
        __syncwarp();
    } else {
        const int q = warp & 3, hf = (warp - 2) >> 2;
        const bool leader = threadIdx.x == 64;
        const int l = 32 * q + lane;  // lane of tensor memory: real column of the tile
        const int jc = cc0 + (l >> 1);  // complex column, from k1
        const float itj = jc < m ? inv_t[jc] : 0.f;
        const int xC = 2 * (k1 + cc0), yC = k1 + r0;  // tile origin in the float view of A
        if (leader) {
            // the operand buffer is free once the MMAs are done
            int ok = (int)mbar_wait(accum, 0, err, 15);
            if (ok) ok = *(volatile int*)err == 0;
            if (ok)
                for (int c = 0; c < 3; ++c) {
                    mbar_expect_tx(cfull + c, lutc::C_BYTES);
                    tma_load_2d(base + c * lutc::C_BYTES, &tmC, cfull + c, xC, yC + 64 * c);
                }
            eok = ok;
        }
        asm volatile("bar.sync 1, 256;" ::: "memory");
        if (eok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
            for (int c = 0; c < 4; ++c) {
                const int slot = c % 3;
                float* cs = (float*)(base + slot * lutc::C_BYTES);  // [64][128] floats
                int got = 0;
                if (lane == 0) got = *(volatile int*)err == 0 && mbar_wait(cfull + slot, c / 3, err, 16);
                got = __shfl_sync(0xffffffffu, got, 0);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int rr = 32 * hf + 16 * h;  // first row of the group, in the chunk
                    float acc[16];
                    tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * c + rr), acc);
                    if (got) {
#pragma unroll
                        for (int r = 0; r < 16; ++r) {
                            float* p = cs + (rr + r) * 128 + l;
                            *p = *p - acc[r] * (itj * rs[64 * c + rr + r]);
                        }
                    }
                }
                fence_proxy_async();
                asm volatile("bar.sync 1, 256;" ::: "memory");
                if (leader && *(volatile int*)err == 0) {
                    tma_store_2d(&tmC, cs, xC, yC + 64 * c);
                    bulk_store_commit();
                    if (c == 0) {
                        bulk_store_wait_read();  // slot 0 takes the last chunk
                        mbar_expect_tx(cfull, lutc::C_BYTES);
                        tma_load_2d(base, &tmC, cfull, xC, yC + 192);
                    }
                }
            }
            if (leader) bulk_store_wait();
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(lutc::TMEM_COLS)
                     : "memory");
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

constexpr int RC = 8;  // right-hand sides per CTA of a triangular solve

// Both triangular solves as one launch each, in wavefront order.  A CTA
// takes a ticket when it starts: ticket t is row block t of the forward (L)
// sweep, block nblk - 1 - t of the backward (U) sweep, so a CTA only waits for
// blocks whose CTAs started before it.  Row block k:
//   acc = W[block k] - sum over the blocks j before k (forward: j < k;
//         backward: j > k) of A[block k][block j] x_j
//   x_k = inv_k acc, stored in Out, then the block's flag is raised
// Each x_j is read once its flag is up (bounded wait: on timeout, or once
// any wait has given up, the kernel records an error and stops waiting); the
// 64 x 64 blocks of A stream through a cp.async double buffer.  RC right-hand
// sides per CTA (blockIdx.y).  Thread: row i = tid / 4, right-hand sides
// 2 (tid % 4) and the next.
constexpr int WLD = NB + 2;  // tile row stride in float2: 16-byte aligned, 8 rows on distinct banks

__device__ __forceinline__ void cp_async16(void* dst, const void* src, int src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(tc::smem_u32(dst)), "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// tile rows [r0, r0 + 64) x columns [c0, c0 + 64) of A into T (rows past n
// or columns past n read as zeros)
__device__ __forceinline__ void tile_async(float2* T, const float2* __restrict__ A, int n, int lda, int r0, int c0)
{
    for (int q = threadIdx.x; q < NB * (NB / 2); q += blockDim.x) {
        const int i = q / (NB / 2), c = 2 * (q % (NB / 2));  // 16-byte piece: two complex
        const int r = r0 + i, cc = c0 + c;
        const int nv = (r < n) ? max(0, min(2, n - cc)) : 0;  // valid complex in the piece
        // clamped source stays 16-byte aligned: lda and the column are even
        const float2* src = A + (size_t)min(r, n - 1) * lda + min(cc, (n - 1) & ~1);
        cp_async16(T + i * WLD + c, src, 8 * nv);
    }
}

template <int DIR>
__global__ void __launch_bounds__(256) k_lu_wave(const float2* __restrict__ A, int n, int lda, int nblk,
                                                 const float2* __restrict__ inv, int nrhs,
                                                 const float2* __restrict__ W, float2* __restrict__ Out,
                                                 int* __restrict__ ticket, int* __restrict__ flag,
                                                 int* __restrict__ err, long long limit)
{
    extern __shared__ float2 s_w[];
    float2* T0 = s_w;                 // [NB][WLD] tile buffers
    float2* T1 = T0 + NB * WLD;
    __shared__ float2 xs[NB][RC];     // x_j of the tile, then acc
    __shared__ int s_t, s_ok;
    const int tid = threadIdx.x, i = tid >> 2, r = 2 * (tid & 3);
    if (tid == 0) s_t = atomicAdd(ticket + blockIdx.y, 1);
    __syncthreads();
    const int t = s_t;
    const int k = DIR == 0 ? t : nblk - 1 - t;
    const int k0 = k * NB, nbk = min(NB, n - k0);
    const int rb = blockIdx.y * RC, nr = min(RC, nrhs - rb);
    int* fl = flag + (size_t)blockIdx.y * nblk;
    float2 acc[2];
#pragma unroll
    for (int h = 0; h < 2; ++h)
        acc[h] = (i < nbk && r + h < nr) ? W[(size_t)(rb + r + h) * n + k0 + i] : make_float2(0.f, 0.f);
    // the blocks this row block depends on, in the order they are solved
    const int nd = DIR == 0 ? k : nblk - 1 - k;
    auto dep = [&](int s) { return DIR == 0 ? s : nblk - 1 - s; };
    if (nd > 0) {
        tile_async(T0, A, n, lda, k0, dep(0) * NB);
        cp_async_commit();
    }
    bool ok = true;
    for (int s = 0; s < nd; ++s) {
        float2* T = (s & 1) ? T1 : T0;
        if (s + 1 < nd) tile_async((s & 1) ? T0 : T1, A, n, lda, k0, dep(s + 1) * NB);
        cp_async_commit();
        const int j = dep(s), j0 = j * NB, nbj = min(NB, n - j0);
        if (tid == 0) {
            int got = ok;
            if (got) {
                const long long t0 = clock64();
                while (*(volatile int*)(fl + j) == 0) {
                    if (*(volatile int*)err || clock64() - t0 > limit) {
                        atomicCAS(err, 0, 21);
                        got = 0;
                        break;
                    }
                }
            }
            __threadfence();
            s_ok = got;
        }
        __syncthreads();
        ok = s_ok;
        if (ok)
            for (int q = tid; q < NB * RC; q += blockDim.x) {
                const int c = q / RC, rr = q % RC;
                xs[c][rr] = (c < nbj && rr < nr) ? __ldcg(Out + (size_t)(rb + rr) * n + j0 + c) : make_float2(0.f, 0.f);
            }
        cp_async_wait<1>();
        __syncthreads();
        if (ok) {
            // the block's 64-term product on its own, then subtracted (the
            // rounding of a sweep that updates W block by block)
            float2 p[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll 8
            for (int c = 0; c < NB; ++c) {
                const float2 l = T[i * WLD + c];
#pragma unroll
                for (int h = 0; h < 2; ++h) p[h] = cfma(l, xs[c][r + h], p[h]);
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) acc[h] = make_float2(acc[h].x - p[h].x, acc[h].y - p[h].y);
        }
        __syncthreads();
    }
    cp_async_wait<0>();
    // x_k = inv_k acc
#pragma unroll
    for (int h = 0; h < 2; ++h) xs[i][r + h] = acc[h];
    const float2* iv = inv + (size_t)k * NB * NB;
    for (int q = tid; q < NB * NB; q += blockDim.x) T0[(q / NB) * WLD + q % NB] = iv[q];
    __syncthreads();
    float2 x[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll 8
    for (int c = 0; c < NB; ++c) {
        const float2 m = T0[i * WLD + c];
#pragma unroll
        for (int h = 0; h < 2; ++h) x[h] = cfma(m, xs[c][r + h], x[h]);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (i < nbk && r + h < nr) Out[(size_t)(rb + r + h) * n + k0 + i] = x[h];
    __threadfence();
    __syncthreads();
    if (tid == 0) atomicExch(fl + k, 1);
}

}  // namespace

// trailing-update operands: U planes [2][2n][128] and L planes [2][n][128]
// halves, then 1/t_j and 1/s_i (n floats each)
static size_t ops_bytes(int n) { return (size_t)6 * n * lutc::KH * sizeof(__half) + 2 * sizeof(float) * (size_t)n; }

size_t lu_bytes(int n)
{
    const size_t nblk = (size_t)(n + NB - 1) / NB;
    return sizeof(float2) * (size_t)(n + (n & 1)) * n + sizeof(int) * (size_t)n + 2 * sizeof(float2) * nblk * NB * NB + 256 * 4 +
           ops_bytes(n);
}

// FP16 operand map: rows of 128 halves (256 bytes), box 64 halves x box_rows,
// 128-byte swizzle, zero fill past the last row
static emfa_status_t ops_map(Ctx* c, CUtensorMap* m, const void* ptr, uint64_t rows, uint32_t box_rows)
{
    auto fn = tensor_map_encoder();
    if (!fn) {
        set_error(c, "cuTensorMapEncodeTiled unavailable");
        return EMFA_ERR_CUDA;
    }
    cuuint64_t dims[2] = {(cuuint64_t)lutc::KH, rows};
    cuuint64_t strides[1] = {(cuuint64_t)lutc::KH * sizeof(__half)};
    cuuint32_t box[2] = {64, box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error(c, "lu_factor: cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
        return EMFA_ERR_CUDA;
    }
    return EMFA_OK;
}

// A as a float matrix of `rows` rows x 2n columns, rows lda complex apart;
// box 128 floats (64 complex) x 64 rows, no swizzle; loads past the matrix
// (or past `rows`) read zeros and stores there are clipped
static emfa_status_t tile_map(Ctx* c, CUtensorMap* m, const void* A, int n, int lda, int rows)
{
    auto fn = tensor_map_encoder();
    if (!fn) {
        set_error(c, "cuTensorMapEncodeTiled unavailable");
        return EMFA_ERR_CUDA;
    }
    cuuint64_t dims[2] = {2 * (cuuint64_t)n, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)lda * sizeof(float2)};
    cuuint32_t box[2] = {128, 64};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(A), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error(c, "lu_factor: cuTensorMapEncodeTiled (A) failed (" + std::to_string((int)r) + ")");
        return EMFA_ERR_CUDA;
    }
    return EMFA_OK;
}

// three padded 64 x 64 blocks and the merge products (2048): about 116 KB,
// so the CTA fits on an SM beside one CTA of the trailing update
static size_t diag_smem() { return sizeof(float2) * (3 * NB * LDS + 2048); }

static emfa_status_t lu_set_smem(Ctx* c)
{
    EMFA_TRY(ensure_smem(c, k_lu_diag, diag_smem()));
    EMFA_TRY(ensure_smem(c, k_lu_panels, 2 * sizeof(float2) * NB * LDS));
    EMFA_TRY(ensure_smem(c, k_lu_wave<0>, sizeof(float2) * 2 * NB * WLD));
    EMFA_TRY(ensure_smem(c, k_lu_wave<1>, sizeof(float2) * 2 * NB * WLD));
    return ensure_smem(c, k_lu_update_tc, lutc::SMEM);
}

emfa_status_t lu_factor(Ctx* c, const void* Z, int n, LuFactor& F, cudaStream_t st)
{
    if (n <= 0) {
        set_error(c, "lu_factor: n must be positive");
        return EMFA_ERR_INVALID;
    }
    EMFA_TRY(lu_set_smem(c));
    F.n = n;
    F.lda = n + (n & 1);  // rows 16-byte aligned: the update moves tiles of A with TMA
    F.nblk = (n + NB - 1) / NB;
    const int lda = F.lda;
    EMFA_TRY(F.a.alloc(c, sizeof(float2) * (size_t)lda * n));
    EMFA_TRY(F.perm.alloc(c, sizeof(int) * (size_t)n));
    EMFA_TRY(F.linv.alloc(c, sizeof(float2) * (size_t)F.nblk * NB * NB));
    EMFA_TRY(F.uinv.alloc(c, sizeof(float2) * (size_t)F.nblk * NB * NB));
    EMFA_TRY(F.info.alloc(c, 256));
    EMFA_TRY(F.ops.alloc(c, ops_bytes(n)));
    float2* A = dptr<float2>(F.a);
    __half* Uop = dptr<__half>(F.ops);
    __half* Lop = Uop + (size_t)4 * n * lutc::KH;
    float* inv_t = (float*)(Lop + (size_t)2 * n * lutc::KH);
    float* inv_s = inv_t + n;
    int* info = dptr<int>(F.info);
    CUtensorMap tmU, tmL, tmC;
    EMFA_TRY(ops_map(c, &tmU, Uop, (uint64_t)4 * n, lutc::TM));
    EMFA_TRY(ops_map(c, &tmL, Lop, (uint64_t)2 * n, lutc::TN));
    EMFA_TRY(tile_map(c, &tmC, A, n, lda, n));
    EMFA_CUDA(c, cudaMemcpy2DAsync(A, sizeof(float2) * (size_t)lda, Z, sizeof(float2) * (size_t)n,
                                   sizeof(float2) * (size_t)n, (size_t)n, cudaMemcpyDeviceToDevice, st));
    EMFA_CUDA(c, cudaMemsetAsync(info, 0, 3 * sizeof(int), st));
    const size_t s2 = 2 * sizeof(float2) * NB * LDS;
    // lookahead: the next diagonal block is factored on a high-priority
    // stream while the rest of the trailing matrix is updated on st, so its
    // one CTA is scheduled ahead of the update's waiting tiles (released on
    // every return)
    struct Aux {
        cudaStream_t s = nullptr;
        cudaEvent_t panel = nullptr, diag = nullptr;
        ~Aux()
        {
            if (panel) cudaEventDestroy(panel);
            if (diag) cudaEventDestroy(diag);
            if (s) cudaStreamDestroy(s);
        }
    } aux;
    if (F.nblk > 2) {
        int lo = 0, hi = 0;
        EMFA_CUDA(c, cudaDeviceGetStreamPriorityRange(&lo, &hi));
        EMFA_CUDA(c, cudaStreamCreateWithPriority(&aux.s, cudaStreamNonBlocking, hi));
        EMFA_CUDA(c, cudaEventCreateWithFlags(&aux.panel, cudaEventDisableTiming));
        EMFA_CUDA(c, cudaEventCreateWithFlags(&aux.diag, cudaEventDisableTiming));
    }
    auto diag = [&](int kb, cudaStream_t s) {
        const int k0 = kb * NB, nb = std::min(NB, n - k0);
        k_lu_diag<<<1, DIAG_THREADS, diag_smem(), s>>>(A, n, lda, k0, nb, dptr<int>(F.perm), dptr<float2>(F.linv), dptr<float2>(F.uinv),
                                     info);
        c->kernel_launches += 1;
    };
    // A22 -= L21 U12 on column tiles [ct0, ct0 + nct) (64 complex columns
    // each) and row tiles [0, rt) of [k1, n)^2, clipped to the rows of tm
    auto update = [&](const CUtensorMap& tm, int k1, int ct0, int nct, int rt, int nslices, cudaStream_t s) {
        k_lu_update_tc<<<dim3((unsigned)nct, (unsigned)rt), lutc::THREADS, lutc::SMEM, s>>>(
            tmU, tmL, tm, n, k1, ct0, nslices, inv_t, inv_s, info + 1);
        c->kernel_launches += 1;
    };
    auto row_tiles = [&](int k1) { return (n - k1 + lutc::TN - 1) / lutc::TN; };
    auto panels = [&](int k0, int nb, int pack) {
        const unsigned ch = (unsigned)((n - k0 - nb + NB - 1) / NB);
        k_lu_panels<<<dim3(ch, 2), 256, s2, st>>>(A, n, lda, k0, nb, dptr<int>(F.perm), dptr<float2>(F.linv),
                                                   dptr<float2>(F.uinv), Uop, Lop, inv_t, inv_s, pack);
        c->kernel_launches += 1;
    };
    // the next diagonal block on the high-priority stream once st has
    // updated its columns; st waits for it before it goes on
    auto diag_aside = [&](int kb) -> emfa_status_t {
        EMFA_CUDA(c, cudaEventRecord(aux.panel, st));
        EMFA_CUDA(c, cudaStreamWaitEvent(aux.s, aux.panel, 0));
        diag(kb, aux.s);
        EMFA_CUDA(c, cudaEventRecord(aux.diag, aux.s));
        return EMFA_OK;
    };
    diag(0, st);
    int kb = 0;
    while (kb < F.nblk) {
        const int k0 = kb * NB, nb = std::min(NB, n - k0), rest = n - k0 - nb;
        if (rest <= 0) break;
        const int k1 = k0 + nb, ch = (rest + NB - 1) / NB;
        if (aux.s && F.nblk - kb - 1 >= 2) {
            // blocks kb and kb + 1 as a pair: block kb's update of the next
            // block's columns and rows only, then one K = 128 update of the
            // rest with both blocks' panels (A22 is read and written once
            // for the two)
            const int k2 = k1 + NB, ch2 = (n - k2 + NB - 1) / NB;
            panels(k0, nb, 1);
            update(tmC, k1, 0, 1, row_tiles(k1), 2, st);  // columns of block kb + 1
            EMFA_TRY(diag_aside(kb + 1));
            CUtensorMap tmR;                              // rows of block kb + 1
            EMFA_TRY(tile_map(c, &tmR, A, n, lda, k2));
            update(tmR, k1, 1, ch - 1, 1, 2, st);
            EMFA_CUDA(c, cudaStreamWaitEvent(st, aux.diag, 0));
            panels(k1, NB, 0);
            k_lu_pack2<<<dim3((unsigned)((n - k2 + 7) / 8), 2), 256, 0, st>>>(A, n, lda, k0, Uop, Lop, inv_t, inv_s);
            c->kernel_launches += 1;
            update(tmC, k2, 0, 1, row_tiles(k2), 4, st);  // columns of block kb + 2
            if (ch2 > 1) {
                EMFA_TRY(diag_aside(kb + 2));
                update(tmC, k2, 1, ch2 - 1, row_tiles(k2), 4, st);
                EMFA_CUDA(c, cudaStreamWaitEvent(st, aux.diag, 0));
            } else {
                diag(kb + 2, st);
            }
            kb += 2;
            continue;
        }
        panels(k0, nb, 1);
        if (aux.s && ch > 1) {
            // the next block's columns, then its diagonal block on the
            // high-priority stream while the other columns are updated
            update(tmC, k1, 0, 1, row_tiles(k1), 2, st);
            EMFA_TRY(diag_aside(kb + 1));
            update(tmC, k1, 1, ch - 1, row_tiles(k1), 2, st);
            EMFA_CUDA(c, cudaStreamWaitEvent(st, aux.diag, 0));
        } else {
            update(tmC, k1, 0, ch, row_tiles(k1), 2, st);
            diag(kb + 1, st);
        }
        kb += 1;
    }
    if (F.nblk > 1) {
        k_lu_rowperm_left<<<dim3((unsigned)(F.nblk - 1) * (NB / 32), (unsigned)F.nblk), 256, 0, st>>>(
            A, n, lda, dptr<int>(F.perm));
        c->kernel_launches += 1;
    }
    EMFA_CUDA(c, cudaGetLastError());
    return EMFA_OK;
}

emfa_status_t lu_check_solves(Ctx* c, const LuFactor& F, cudaStream_t st)
{
    int h = 0;
    EMFA_CUDA(c, cudaMemcpyAsync(&h, dptr<int>(F.info) + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    if (h) {
        set_error(c, "lu_apply: a wait of the triangular solves timed out (code " + std::to_string(h) + ")");
        return EMFA_ERR_TIMEOUT;
    }
    return EMFA_OK;
}

emfa_status_t lu_zero_pivot(Ctx* c, const LuFactor& F, int* first, cudaStream_t st)
{
    int h[2] = {0, 0};
    EMFA_CUDA(c, cudaMemcpyAsync(h, F.info.ptr, sizeof(h), cudaMemcpyDeviceToHost, st));
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    *first = h[0];
    if (h[1]) {
        set_error(c, "lu_factor: a wait of the tensor-core trailing update timed out (stage " + std::to_string(h[1]) +
                         ")");
        return EMFA_ERR_TIMEOUT;
    }
    return EMFA_OK;
}

emfa_status_t lu_apply(Ctx* c, const LuFactor& F, const float2* B, int nrhs, float2* X, float2* work,
                       cudaStream_t st)
{
    const int n = F.n;
    const size_t tot = (size_t)n * nrhs;
    float2* W = work;           // permuted right-hand sides
    float2* Y = work + tot;     // L^-1 P b
    const float2* A = dptr<float2>(F.a);
    const int gy = (nrhs + RC - 1) / RC;
    // tickets and flags of both sweeps: 2 (gy + gy nblk) ints
    void* wp = nullptr;
    const size_t words = 2 * ((size_t)gy + (size_t)gy * F.nblk);
    EMFA_TRY(ctx_workspace(c, WS_LU_WAVE, sizeof(int) * words, &wp));
    int* tk = (int*)wp;
    int* fl = tk + 2 * gy;
    EMFA_CUDA(c, cudaMemsetAsync(tk, 0, sizeof(int) * words, st));
    k_lu_gather<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(B, dptr<int>(F.perm), n, nrhs, W);
    const size_t sm = sizeof(float2) * 2 * NB * WLD;
    const long long limit = 2000000000LL;  // about 1 s
    k_lu_wave<0><<<dim3((unsigned)F.nblk, (unsigned)gy), 256, sm, st>>>(A, n, F.lda, F.nblk, dptr<float2>(F.linv),
                                                                        nrhs, W, Y, tk, fl, dptr<int>(F.info) + 2,
                                                                        limit);
    k_lu_wave<1><<<dim3((unsigned)F.nblk, (unsigned)gy), 256, sm, st>>>(
        A, n, F.lda, F.nblk, dptr<float2>(F.uinv), nrhs, Y, X, tk + gy, fl + (size_t)gy * F.nblk,
        dptr<int>(F.info) + 2, limit);
    c->kernel_launches += 3;
    EMFA_CUDA(c, cudaGetLastError());
    return EMFA_OK;
}

}  // namespace emfa
