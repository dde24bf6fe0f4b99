// Batched Krylov solvers: all right-hand sides advance in lockstep and share
// one multi-RHS product Z V per step.
//
// GMRES(m) (EMIterative/iml.cpp:156-207): Arnoldi by classical Gram-Schmidt
// applied twice (CGS2, FP64 coefficients), complex Givens rotations in FP64,
// per-RHS early exit when the rotated residual |g_{j+1}| meets the tolerance,
// restart from the true residual.  For the mixed-precision path the basis is
// stored in FP32, the inner product Z V_j runs in reduced precision, and each
// restart recomputes b - Z x with FP64 accumulation: restarted GMRES is then
// mixed-precision iterative refinement with GMRES as the inner solver.
//
// BiCGStab (EMIterative/iml.cpp:3-39, MLFMA.cpp:402-452): the reference's
// update order, x0 = 0, stop when ||s|| / ||b|| < tol, FP64 vectors.
//
// All reductions use fixed-order two-level sums (per-block partials, then a
// sequential sum of the partials), so a solve is run-to-run reproducible.
#include "emfa_internal.cuh"
#include "emfa_math.cuh"
#include "gemm.cuh"
#include "krylov.cuh"
#include "lu.cuh"

#include <algorithm>
#include <type_traits>
#include <cmath>

namespace emfa {

constexpr int KB = 256;     // threads per block of the vector kernels
constexpr int KE = 4;       // elements per thread per block chunk
constexpr int KCHUNK = KB * KE;

template <typename T> __device__ __forceinline__ double2 ld2(const Cx<T>* p) { Cx<T> v = *p; return make_double2((double)v.re, (double)v.im); }
__device__ __forceinline__ double2 ld2(const double2* p) { return *p; }

// partial[(i * nrhs + r) * nblk + blk] = sum_{k in chunk} conj(V_i[r][k]) W[r][k]
template <typename TV, typename TW>
__global__ void __launch_bounds__(KB) k_block_dots(const TV* __restrict__ V, size_t vstride, int nv,
                                                   const TW* __restrict__ W, int n, int nrhs, int nblk,
                                                   double2* __restrict__ partial)
{
    const int blk = blockIdx.x, r = blockIdx.y;
    const size_t base = (size_t)r * n;
    double2 w[KE];
    int kk[KE];
#pragma unroll
    for (int e = 0; e < KE; ++e) {
        int k = blk * KCHUNK + e * KB + threadIdx.x;
        kk[e] = k;
        w[e] = k < n ? ld2(W + base + k) : make_double2(0.0, 0.0);
    }
    __shared__ double2 red[32][KB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i0 = 0; i0 < nv; i0 += 32) {
        int cnt = min(32, nv - i0);
        for (int ii = 0; ii < cnt; ++ii) {
            const TV* vi = V + (size_t)(i0 + ii) * vstride + base;
            double re = 0.0, im = 0.0;
#pragma unroll
            for (int e = 0; e < KE; ++e) {
                if (kk[e] < n) {
                    double2 v = ld2(vi + kk[e]);
                    re += v.x * w[e].x + v.y * w[e].y;
                    im += v.x * w[e].y - v.y * w[e].x;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                re += __shfl_xor_sync(0xffffffffu, re, o);
                im += __shfl_xor_sync(0xffffffffu, im, o);
            }
            if (lane == 0) red[ii][wid] = make_double2(re, im);
        }
        __syncthreads();
        if (threadIdx.x < cnt) {
            double2 s = make_double2(0.0, 0.0);
            for (int q = 0; q < KB / 32; ++q) {
                s.x += red[threadIdx.x][q].x;
                s.y += red[threadIdx.x][q].y;
            }
            partial[((size_t)(i0 + threadIdx.x) * nrhs + r) * nblk + blk] = s;
        }
        __syncthreads();
    }
}

// out[i * nrhs + r] (+)= sum_blk partial[(i * nrhs + r) * nblk + blk]
__global__ void k_reduce_partials(const double2* __restrict__ partial, int nv, int nrhs, int nblk,
                                  double2* __restrict__ out, int accumulate)
{
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nv * nrhs) return;
    const double2* p = partial + (size_t)id * nblk;
    double2 s = make_double2(0.0, 0.0);
    for (int b = 0; b < nblk; ++b) {
        s.x += p[b].x;
        s.y += p[b].y;
    }
    if (accumulate) {
        s.x += out[id].x;
        s.y += out[id].y;
    }
    out[id] = s;
}

// ---------------------------------------------------------------------------
// Block reductions: per-thread sums in the storage precision (FP32 for the
// mixed path: GB300's FP64 pipe is ~1/64 of FP32), warp and block sums in
// FP64, written as the block's partials.
// ---------------------------------------------------------------------------
constexpr int MAXV = 32;  // basis vectors per pass of the block-dot kernels (BiCGStab)
constexpr int MAX_RESTART = 255;  // GMRES(m): coefficients live in dynamic shared memory

template <typename T> struct Acc { using type = float; };
template <> struct Acc<double> { using type = double; };

template <typename A>
__device__ __forceinline__ void block_reduce_write(A (&ar)[MAXV], A (&ai)[MAXV], int nv, double2* out, size_t ostride)
{
    __shared__ double2 red[MAXV][KB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < MAXV; ++i) {
        if (i < nv) {
            double re = (double)ar[i], im = (double)ai[i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                re += __shfl_xor_sync(0xffffffffu, re, o);
                im += __shfl_xor_sync(0xffffffffu, im, o);
            }
            if (lane == 0) red[i][wid] = make_double2(re, im);
        }
    }
    __syncthreads();
    if (threadIdx.x < nv) {
        double2 t = make_double2(0.0, 0.0);
        for (int q = 0; q < KB / 32; ++q) {
            t.x += red[threadIdx.x][q].x;
            t.y += red[threadIdx.x][q].y;
        }
        out[(size_t)threadIdx.x * ostride] = t;
    }
}

// squared norms of complex128 vectors: partial[r * nblk + blk]
// F32: the squares of the values rounded to FP32 (split_f64's high parts,
// integer operations) summed in FP32 within a thread: the FP32-basis
// refinement compares the norm with its target to a few digits, and FP64
// multiply-adds queue on GB300's 1/64-rate pipe.  The plain FP64 path keeps
// FP64 sums.
template <bool F32>
__global__ void __launch_bounds__(KB) k_norm2(const double2* __restrict__ X, int n, int nblk, int chunk,
                                              double2* __restrict__ partial)
{
    const int blk = blockIdx.x, r = blockIdx.y;
    const size_t base = (size_t)r * n;
    const int k1 = min(n, (blk + 1) * chunk);
    double a1[MAXV], a2[MAXV];
    a1[0] = 0.0;
    a2[0] = 0.0;
    if (F32) {
        float t = 0.f;
        for (int k = blk * chunk + threadIdx.x; k < k1; k += KB) {
            const double2 x = X[base + k];
            const float xr = split_f64(x.x).x, xi = split_f64(x.y).x;
            t += xr * xr + xi * xi;
        }
        a1[0] = (double)t;
    } else {
        for (int k = blk * chunk + threadIdx.x; k < k1; k += KB) {
            double2 x = X[base + k];
            a1[0] += x.x * x.x + x.y * x.y;
        }
    }
    block_reduce_write<double>(a1, a2, 1, partial + ((size_t)r * nblk + blk), 1);
}

// ---------------------------------------------------------------------------
// Gram-Schmidt passes, second form (low register pressure, many loads in
// flight).  k_vdots: CTA per (chunk of N, RHS); warp w takes basis vectors
// w, w+8, ...; lanes stride the chunk with 4 independent loads in flight; the
// W chunk stays in L1 across the warp's vectors.  k_vupdate: thread per
// element, W -= sum_i h_i V_i with 8 vectors in flight, optional |W|^2.
// Sums within a warp are in the storage precision, across warps and blocks
// in FP64.
// ---------------------------------------------------------------------------
constexpr int VCHUNK = 1024;

// reset (optional): an int zeroed by the first CTA, after the predecessor
// (the step's product) has finished: the step's count of active right-hand
// sides, so that no memset sits between the step's launches.
// active (optional): right-hand sides with active[r] == 0 have converged and
// are skipped (their coefficients and norms are read by nobody).
template <typename T>
__global__ void __launch_bounds__(256) k_vdots(const Cx<T>* __restrict__ V, size_t vstride, int nv,
                                               const Cx<T>* __restrict__ W, int n, int nrhs, int nblk,
                                               double2* __restrict__ partial, int* __restrict__ reset,
                                               const int* __restrict__ active)
{
    using A = typename Acc<T>::type;
    const int blk = blockIdx.x, r = blockIdx.y;
    griddep_wait();
    if (reset && blk == 0 && r == 0 && threadIdx.x == 0) *reset = 0;
    if (active && !active[r]) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t base = (size_t)r * n;
    const int k0 = blk * VCHUNK, k1 = min(n, k0 + VCHUNK);
    // two basis vectors per warp pass (i and i + 8): twice the loads in
    // flight, and one reduction's latency hides behind the other's loads
    for (int i = warp; i < nv; i += 16) {
        const bool two = i + 8 < nv;
        const Cx<T>* va = V + (size_t)i * vstride + base;
        const Cx<T>* vb = V + (size_t)(two ? i + 8 : i) * vstride + base;
        A re = 0, im = 0, re2 = 0, im2 = 0;
        for (int k = k0 + lane; k < k1; k += 128) {
            Cx<T> a[4], b[4], w[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int kk = k + 32 * u;
                const bool in = kk < k1;
                a[u] = in ? va[kk] : Cx<T>{T(0), T(0)};
                b[u] = in && two ? vb[kk] : Cx<T>{T(0), T(0)};
                w[u] = in ? W[base + kk] : Cx<T>{T(0), T(0)};
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                re += (A)a[u].re * (A)w[u].re + (A)a[u].im * (A)w[u].im;
                im += (A)a[u].re * (A)w[u].im - (A)a[u].im * (A)w[u].re;
                re2 += (A)b[u].re * (A)w[u].re + (A)b[u].im * (A)w[u].im;
                im2 += (A)b[u].re * (A)w[u].im - (A)b[u].im * (A)w[u].re;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            re += __shfl_xor_sync(0xffffffffu, re, o);
            im += __shfl_xor_sync(0xffffffffu, im, o);
            re2 += __shfl_xor_sync(0xffffffffu, re2, o);
            im2 += __shfl_xor_sync(0xffffffffu, im2, o);
        }
        if (lane == 0) {
            partial[((size_t)i * nrhs + r) * nblk + blk] = make_double2((double)re, (double)im);
            if (two) partial[((size_t)(i + 8) * nrhs + r) * nblk + blk] = make_double2((double)re2, (double)im2);
        }
    }
    griddep_launch();
}

// With `partial` (the block partials of k_vdots) the coefficients are summed
// here, over the blocks in order as k_reduce_partials does, and block 0 also
// stores them in h; without it they are read from h.  The right-hand sides
// are taken last first: k_vdots ran them first to last, so the basis slices
// it read last (up to the L2's size, ~100 MB) are read again from L2.
template <typename T, bool NORM>
__global__ void __launch_bounds__(256) k_vupdate(const Cx<T>* __restrict__ V, size_t vstride, int nv,
                                                 double2* __restrict__ h, const double2* __restrict__ partial,
                                                 Cx<T>* __restrict__ W, int n, int nrhs, int nblk,
                                                 double2* __restrict__ pnorm, const int* __restrict__ active)
{
    using A = typename Acc<T>::type;
    const int blk = blockIdx.x, r = nrhs - 1 - (int)blockIdx.y;
    griddep_wait();
    if (active && !active[r]) return;  // converged: nobody reads its coefficients or norm
    const size_t base = (size_t)r * n;
    // coefficients (dynamic shared memory: 2 nv values, any restart length)
    extern __shared__ unsigned char dyn_smem[];
    A* hs0 = reinterpret_cast<A*>(dyn_smem);
    A* hs1 = hs0 + nv;
    __shared__ A red[8], redm[8];
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        // the block partials summed in the basis precision: FP32 sums for an
        // FP32 basis (its coefficients are used in FP32; an FP64 addition
        // costs ~64 cycles a warp instruction on GB300)
        A tx, ty;
        if (partial) {
            const double2* p = partial + ((size_t)i * nrhs + r) * nblk;
            tx = 0;
            ty = 0;
            for (int b = 0; b < nblk; ++b) {
                tx += (A)p[b].x;
                ty += (A)p[b].y;
            }
            if (blk == 0) h[(size_t)i * nrhs + r] = make_double2((double)tx, (double)ty);
        } else {
            const double2 t = h[(size_t)i * nrhs + r];
            tx = (A)t.x;
            ty = (A)t.y;
        }
        hs0[i] = tx;
        hs1[i] = ty;
    }
    __syncthreads();
    A nr = 0, mx = 0;
    const int k0 = blk * VCHUNK, k1 = min(n, k0 + VCHUNK);
    // a thread's VCHUNK / 256 = 4 elements together, 4 basis vectors a pass:
    // 16 independent loads in flight at clamped in-bounds addresses (a
    // vector past the basis counts with coefficient 0), so no tail of nv
    // loads one vector at a time
    constexpr int EL = VCHUNK / 256, VG = 4;
    int kc[EL];
    Cx<T> w[EL];
#pragma unroll
    for (int e = 0; e < EL; ++e) {
        kc[e] = min(k0 + (int)threadIdx.x + 256 * e, k1 - 1);
        w[e] = W[base + kc[e]];
    }
    A sr[EL], si[EL];
#pragma unroll
    for (int e = 0; e < EL; ++e) sr[e] = si[e] = 0;
    const Cx<T>* vb = V + base;
    for (int i = 0; i < nv; i += VG) {
        Cx<T> v[VG][EL];
#pragma unroll
        for (int u = 0; u < VG; ++u) {
            const Cx<T>* vi = vb + (size_t)min(i + u, nv - 1) * vstride;
#pragma unroll
            for (int e = 0; e < EL; ++e) v[u][e] = vi[kc[e]];
        }
#pragma unroll
        for (int u = 0; u < VG; ++u) {
            const bool ok = i + u < nv;
            const A hr = ok ? hs0[i + u] : (A)0, hi = ok ? hs1[i + u] : (A)0;
#pragma unroll
            for (int e = 0; e < EL; ++e) {
                sr[e] += hr * (A)v[u][e].re - hi * (A)v[u][e].im;
                si[e] += hr * (A)v[u][e].im + hi * (A)v[u][e].re;
            }
        }
    }
#pragma unroll
    for (int e = 0; e < EL; ++e) {
        const int k = k0 + (int)threadIdx.x + 256 * e;
        if (k >= k1) continue;
        w[e].re = (T)((A)w[e].re - sr[e]);
        w[e].im = (T)((A)w[e].im - si[e]);
        W[base + k] = w[e];
        if (NORM) {
            nr += (A)w[e].re * (A)w[e].re + (A)w[e].im * (A)w[e].im;
            mx = fmax(mx, fmax(fabs((A)w[e].re), fabs((A)w[e].im)));
        }
    }
    if (NORM) {
        // |w|^2 and max |Re|, |Im| of the block (the max sets the FP16 scale
        // of the packed copy the next product reads)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            nr += __shfl_xor_sync(0xffffffffu, nr, o);
            mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        if ((threadIdx.x & 31) == 0) {
            red[threadIdx.x >> 5] = nr;
            redm[threadIdx.x >> 5] = mx;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            A t = 0, tm = 0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
                t += red[q];
                tm = fmax(tm, redm[q]);
            }
            pnorm[(size_t)r * nblk + blk] = make_double2((double)t, (double)tm);
        }
    }
    griddep_launch();
}

// X[r][k] += sum_i y_i V_i[r][k]; the sum in the basis precision, added to
// the FP64 iterate once
template <typename T>
__global__ void k_update_x2(const Cx<T>* __restrict__ V, size_t vstride, int nvmax, const double2* __restrict__ y,
                            const int* __restrict__ jlen, double2* __restrict__ X, int n, int nrhs)
{
    using A = typename Acc<T>::type;
    const int r = blockIdx.y;
    extern __shared__ unsigned char dyn_smem[];
    A* ys0 = reinterpret_cast<A*>(dyn_smem);  // 2 nvmax values
    A* ys1 = ys0 + nvmax;
    const int jl = min(jlen[r], nvmax);
    for (int i = threadIdx.x; i < jl; i += blockDim.x) {
        double2 t = y[(size_t)i * nrhs + r];
        ys0[i] = (A)t.x;
        ys1[i] = (A)t.y;
    }
    __syncthreads();
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    size_t o = (size_t)r * n + k;
    A sr = 0, si = 0;
    for (int i = 0; i < jl; ++i) {
        const Cx<T> v = V[(size_t)i * vstride + o];
        sr += ys0[i] * (A)v.re - ys1[i] * (A)v.im;
        si += ys0[i] * (A)v.im + ys1[i] * (A)v.re;
    }
    double2 x = X[o];
    X[o] = make_double2(x.x + (double)sr, x.y + (double)si);
}

// ---------------------------------------------------------------------------
// The same three passes on an FP16 basis: the operand rows of the split-FP16
// product.  Basis vector i of right-hand side r is row 2r of plane i (planes
// `plane` halves apart, rows `ldh` halves apart): the pairs (Re, -Im) of
// t v_i in FP16, t = 1 / inv_t[i nrhs + r] a power of two.  A stored pair c
// is conj(t v), so h = conj(v) w is inv_t sum c w and v = inv_t conj(c).
// The product multiplied exactly these vectors, so the Arnoldi relation
// holds for them; each read moves 4 bytes an element instead of 8.
// ---------------------------------------------------------------------------
__device__ __forceinline__ const __half2* hrow(const __half* Bh, size_t plane, size_t ldh, int i, int r)
{
    return reinterpret_cast<const __half2*>(Bh + (size_t)i * plane + (size_t)(2 * r) * ldh);
}

// unpacks two FP16 values (one stored pair) to FP32
__device__ __forceinline__ float2 h2f(unsigned int u)
{
    __half2 h;
    memcpy(&h, &u, sizeof(h));
    return __half22float2(h);
}
// the bits of an FP16 pair
__device__ __forceinline__ unsigned int h2u(__half2 h)
{
    unsigned int u;
    memcpy(&u, &h, sizeof(u));
    return u;
}

// Element pairs of a length-n row of W (elements 2q, 2q + 1).  Rows start
// 16-byte aligned for even n: one 16-byte access.  For odd n every other row
// starts 8 bytes off and the last pair is half outside the row: two 8-byte
// accesses, the second guarded (loads give 0 past the row).
template <bool ODD>
__device__ __forceinline__ float4 ld_wpair(const float2* w, int q, int n)
{
    if (!ODD) return reinterpret_cast<const float4*>(w)[q];
    const float2 a = w[2 * q];
    const float2 b = 2 * q + 1 < n ? w[2 * q + 1] : make_float2(0.f, 0.f);
    return make_float4(a.x, a.y, b.x, b.y);
}
template <bool ODD>
__device__ __forceinline__ void st_wpair(float2* w, int q, int n, float4 v)
{
    if (!ODD) {
        reinterpret_cast<float4*>(w)[q] = v;
        return;
    }
    w[2 * q] = make_float2(v.x, v.y);
    if (2 * q + 1 < n) w[2 * q + 1] = make_float2(v.z, v.w);
}
// a basis row's stored pairs for elements 2q, 2q + 1 (rows are 16-byte
// aligned and hold at least 2n + 2 halves for odd n); past the vector the
// row's padding, which is zeroed here so that it cannot carry a NaN
template <bool ODD>
__device__ __forceinline__ uint2 ld_bpair(const __half2* row, int q, int n)
{
    uint2 v = reinterpret_cast<const uint2*>(row)[q];
    if (ODD && 2 * q + 1 >= n) v.y = 0u;
    return v;
}


// conj(v) w summed over an element pair: c the stored pairs (conj of t v)
__device__ __forceinline__ void cmac2(uint2 c, float4 x, float& re, float& im)
{
    const float2 c0 = h2f(c.x), c1 = h2f(c.y);
    re += c0.x * x.x - c0.y * x.y + c1.x * x.z - c1.y * x.w;
    im += c0.x * x.y + c0.y * x.x + c1.x * x.w + c1.y * x.z;
}

// The coefficients on the FP16 basis, a warp per 128 elements of the CTA's
// chunk: a lane loads its two element pairs of W once (16-byte loads; for odd
// N 8-byte ones) and then 8 basis vectors at a time (16 independent 8-byte loads, a
// single round trip per group however short the basis).  The group's 16 sums
// (8 vectors x Re, Im) go across the warp by a transposed butterfly: at each
// level a lane keeps half its values and adds the partner's copy of them, 16
// shuffles in all against 80 for 16 separate reductions.  The warps' sums
// meet in shared memory and are added in warp order (fixed: reproducible).
constexpr int VW_MAXV = 32;  // the separate-pass FP16 step takes restarts up to 32
template <bool ODD>
__global__ void __launch_bounds__(256) k_vdots_hw(const __half* __restrict__ Bh, size_t plane, size_t ldh,
                                                  const float* __restrict__ inv_t, int nv,
                                                  const float2* __restrict__ W, int n, int nrhs, int nblk,
                                                  double2* __restrict__ partial, int* __restrict__ reset,
                                                  const int* __restrict__ active)
{
    __shared__ float sp[8][2 * VW_MAXV];
    const int blk = blockIdx.x, r = blockIdx.y;
    griddep_wait();
    if (reset && blk == 0 && r == 0 && threadIdx.x == 0) *reset = 0;
    if (active && !active[r]) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int p1 = (min(n, (blk + 1) * VCHUNK) + 1) >> 1;
    const int q0 = ((blk * VCHUNK) >> 1) + warp * 64 + lane, q1 = q0 + 32;  // this lane's pairs
    const bool in0 = q0 < p1, in1 = q1 < p1;
    const float2* w = W + (size_t)r * n;
    const float4 x0 = in0 ? ld_wpair<ODD>(w, q0, n) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 x1 = in1 ? ld_wpair<ODD>(w, q1, n) : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int g = 0; g < nv; g += 8) {
        uint2 a[8][2];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const bool ok = g + u < nv;  // uniform across the warp
            const __half2* row = hrow(Bh, plane, ldh, ok ? g + u : 0, r);
            a[u][0] = ok && in0 ? ld_bpair<ODD>(row, q0, n) : make_uint2(0u, 0u);
            a[u][1] = ok && in1 ? ld_bpair<ODD>(row, q1, n) : make_uint2(0u, 0u);
        }
        float v[16];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            float re = 0.f, im = 0.f;
            cmac2(a[u][0], x0, re, im);
            cmac2(a[u][1], x1, re, im);
            v[2 * u] = re;
            v[2 * u + 1] = im;
        }
        // after the levels 16, 8, 4, 2 lane L holds value (L >> 1) summed
        // over the lanes that share bits 4..1 of L; level 1 adds the pair
#pragma unroll
        for (int h = 8, o = 16; h >= 1; h >>= 1, o >>= 1) {
            const bool up = (lane & o) != 0;
#pragma unroll
            for (int t = 0; t < h; ++t) {
                const float send = up ? v[t] : v[t + h];
                const float keep = up ? v[t + h] : v[t];
                v[t] = keep + __shfl_xor_sync(0xffffffffu, send, o);
            }
        }
        v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
        if ((lane & 1) == 0) sp[warp][2 * g + (lane >> 1)] = v[0];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            re += sp[q][2 * i];
            im += sp[q][2 * i + 1];
        }
        const float s = inv_t[(size_t)i * nrhs + r];  // a power of two: exact
        partial[((size_t)i * nrhs + r) * nblk + blk] = make_double2((double)(re * s), (double)(im * s));
    }
    griddep_launch();
}

// W -= sum_i h_i v_i with |W|^2 and max |Re|, |Im| partials (k_vupdate<float,
// true> on the FP16 basis): the coefficients are summed from the block
// partials, block 0 stores them in h, and each is taken times inv_t once.
// A thread holds two element pairs of W (16-byte accesses; 8-byte ones for
// odd N) and loads 4 basis vectors a group, 8 bytes each (40 registers, six
// CTAs an SM).  Measured on the dense CFIE job (7680 x 360): 11.10 ms a
// solve, against 11.19 with single elements and 11.32 with 8 vectors a group
template <bool ODD>
__global__ void __launch_bounds__(256) k_vupdate_h(const __half* __restrict__ Bh, size_t plane, size_t ldh,
                                                   const float* __restrict__ inv_t, int nv, double2* __restrict__ h,
                                                   const double2* __restrict__ partial, float2* __restrict__ W, int n,
                                                   int nrhs, int nblk, double2* __restrict__ pnorm,
                                                   const int* __restrict__ active)
{
    const int blk = blockIdx.x, r = nrhs - 1 - (int)blockIdx.y;
    griddep_wait();
    if (active && !active[r]) return;
    extern __shared__ unsigned char dyn_smem[];
    float* hs0 = reinterpret_cast<float*>(dyn_smem);
    float* hs1 = hs0 + nv;
    __shared__ float red[8], redm[8];
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        const double2* p = partial + ((size_t)i * nrhs + r) * nblk;
        float tx = 0.f, ty = 0.f;
        for (int b = 0; b < nblk; ++b) {
            tx += (float)p[b].x;
            ty += (float)p[b].y;
        }
        if (blk == 0) h[(size_t)i * nrhs + r] = make_double2((double)tx, (double)ty);
        const float s = inv_t[(size_t)i * nrhs + r];
        hs0[i] = tx * s;
        hs1[i] = ty * s;
    }
    __syncthreads();
    float nr = 0.f, mx = 0.f;
    const int k0 = blk * VCHUNK, k1 = min(n, k0 + VCHUNK);
    constexpr int EP = VCHUNK / 512, VG = 4;
    const int p0 = k0 >> 1, p1 = (k1 + 1) >> 1;
    float2* w2 = W + (size_t)r * n;
    int pc[EP];
    float4 w[EP];
#pragma unroll
    for (int e = 0; e < EP; ++e) {
        pc[e] = min(p0 + (int)threadIdx.x + 256 * e, p1 - 1);
        w[e] = ld_wpair<ODD>(w2, pc[e], n);
    }
    float sr[EP][2], si[EP][2];
#pragma unroll
    for (int e = 0; e < EP; ++e) sr[e][0] = sr[e][1] = si[e][0] = si[e][1] = 0.f;
    for (int i = 0; i < nv; i += VG) {
        uint2 v[VG][EP];
#pragma unroll
        for (int u = 0; u < VG; ++u) {
            const __half2* vi = hrow(Bh, plane, ldh, min(i + u, nv - 1), r);
#pragma unroll
            for (int e = 0; e < EP; ++e) v[u][e] = ld_bpair<ODD>(vi, pc[e], n);
        }
#pragma unroll
        for (int u = 0; u < VG; ++u) {
            const bool ok = i + u < nv;
            const float hr = ok ? hs0[i + u] : 0.f, hi = ok ? hs1[i + u] : 0.f;
#pragma unroll
            for (int e = 0; e < EP; ++e) {
                // h v with v = conj(c)
                const float2 c0 = h2f(v[u][e].x), c1 = h2f(v[u][e].y);
                sr[e][0] += hr * c0.x + hi * c0.y;
                si[e][0] += hi * c0.x - hr * c0.y;
                sr[e][1] += hr * c1.x + hi * c1.y;
                si[e][1] += hi * c1.x - hr * c1.y;
            }
        }
    }
#pragma unroll
    for (int e = 0; e < EP; ++e) {
        const int p = p0 + (int)threadIdx.x + 256 * e;
        if (p >= p1) continue;
        w[e].x -= sr[e][0];
        w[e].y -= si[e][0];
        w[e].z -= sr[e][1];
        w[e].w -= si[e][1];  // past the row (odd N): 0 - 0, not stored
        st_wpair<ODD>(w2, p, n, w[e]);
        nr += w[e].x * w[e].x + w[e].y * w[e].y + w[e].z * w[e].z + w[e].w * w[e].w;
        mx = fmaxf(mx, fmaxf(fmaxf(fabsf(w[e].x), fabsf(w[e].y)), fmaxf(fabsf(w[e].z), fabsf(w[e].w))));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nr += __shfl_xor_sync(0xffffffffu, nr, o);
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = nr;
        redm[threadIdx.x >> 5] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f, tm = 0.f;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
            t += red[q];
            tm = fmaxf(tm, redm[q]);
        }
        pnorm[(size_t)r * nblk + blk] = make_double2((double)t, (double)tm);
    }
    griddep_launch();
}

// X[r][k] += sum_i y_i v_i on the FP16 basis, the sum in FP32: a thread
// takes an element pair (the second past the vector for odd N: computed from
// the zeroed padding, not stored), four basis vectors a group of loads
template <bool ODD>
__global__ void k_update_x2_h(const __half* __restrict__ Bh, size_t plane, size_t ldh, const float* __restrict__ inv_t,
                              int nvmax, const double2* __restrict__ y, const int* __restrict__ jlen,
                              double2* __restrict__ X, int n, int nrhs)
{
    const int r = blockIdx.y;
    extern __shared__ unsigned char dyn_smem[];
    float* ys0 = reinterpret_cast<float*>(dyn_smem);
    float* ys1 = ys0 + nvmax;
    const int jl = min(jlen[r], nvmax);
    for (int i = threadIdx.x; i < jl; i += blockDim.x) {
        const double2 t = y[(size_t)i * nrhs + r];
        const float s = inv_t[(size_t)i * nrhs + r];
        ys0[i] = (float)t.x * s;
        ys1[i] = (float)t.y * s;
    }
    __syncthreads();
    constexpr int VG = 4;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;  // element pair
    if (2 * q >= n) return;
    float sr[2] = {0.f, 0.f}, si[2] = {0.f, 0.f};
    for (int i = 0; i < jl; i += VG) {
        float2 c[VG][2];
#pragma unroll
        for (int u = 0; u < VG; ++u) {
            const uint2 v = ld_bpair<ODD>(hrow(Bh, plane, ldh, min(i + u, jl - 1), r), q, n);
            c[u][0] = h2f(v.x);
            c[u][1] = h2f(v.y);
        }
#pragma unroll
        for (int u = 0; u < VG; ++u) {
            const bool ok = i + u < jl;
            const float a = ok ? ys0[i + u] : 0.f, b = ok ? ys1[i + u] : 0.f;
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                sr[e] += a * c[u][e].x + b * c[u][e].y;
                si[e] += b * c[u][e].x - a * c[u][e].y;
            }
        }
    }
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        if (ODD && 2 * q + e >= n) break;
        const size_t o = (size_t)r * n + 2 * (size_t)q + e;
        const double2 x = X[o];
        X[o] = make_double2(x.x + (double)sr[e], x.y + (double)si[e]);
    }
}

// per-RHS: finish Arnoldi column j, rotate, test convergence.  A serial FP64
// chain per right-hand side: one RHS per warp (lane 0) spreads the chains
// over the SMs' FP64 units instead of packing 32 of them into one warp.
__global__ void k_arnoldi_finish(GmresDev s, int j, const double2* __restrict__ pnorm, int nblk, int two_pass)
{
    const int r = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if ((threadIdx.x & 31) != 0 || r >= s.nrhs) return;
    const int m = s.m;
    if (!s.active[r]) {
        s.scale[r] = 0.0;
        return;
    }
    double nr2 = 0.0, wm = 0.0;
    for (int b = 0; b < nblk; ++b) {
        nr2 += pnorm[(size_t)r * nblk + b].x;
        wm = fmax(wm, pnorm[(size_t)r * nblk + b].y);
    }
    s.wmax[r] = wm;
    double beta = sqrt(nr2);
    double2* H = s.H + (size_t)r * (m + 1) * m;
    // column j of H: Gram-Schmidt coefficients (sum of both passes for CGS2)
    for (int i = 0; i <= j; ++i) {
        double2 a = s.hcol[(size_t)i * s.nrhs + r];
        if (two_pass) {
            const double2 b = s.y[(size_t)i * s.nrhs + r];
            a.x += b.x;
            a.y += b.y;
        }
        H[i * m + j] = a;
    }
    H[(j + 1) * m + j] = make_double2(beta, 0.0);
    double* cs = s.cs + (size_t)r * m;
    double2* sn = s.sn + (size_t)r * m;
    double2* g = s.g + (size_t)r * (m + 1);
    // previous rotations: [x; y] <- [c x + s y; -conj(s) x + c y]
    for (int i = 0; i < j; ++i) {
        double2 x = H[i * m + j], y = H[(i + 1) * m + j];
        double c = cs[i];
        double2 sv = sn[i];
        double2 nx = make_double2(c * x.x + sv.x * y.x - sv.y * y.y, c * x.y + sv.x * y.y + sv.y * y.x);
        double2 ny = make_double2(-(sv.x * x.x + sv.y * x.y) + c * y.x, -(sv.x * x.y - sv.y * x.x) + c * y.y);
        H[i * m + j] = nx;
        H[(i + 1) * m + j] = ny;
    }
    double2 a = H[j * m + j];
    double b = beta;
    double aa = hypot(a.x, a.y);
    double nu = hypot(aa, b);
    double c;
    double2 sv;
    if (aa == 0.0) {
        c = 0.0;
        sv = make_double2(1.0, 0.0);
        H[j * m + j] = make_double2(b, 0.0);
    } else {
        c = aa / nu;
        double2 ph = make_double2(a.x / aa, a.y / aa);
        sv = make_double2(ph.x * b / nu, ph.y * b / nu);
        H[j * m + j] = make_double2(ph.x * nu, ph.y * nu);
    }
    H[(j + 1) * m + j] = make_double2(0.0, 0.0);
    cs[j] = c;
    sn[j] = sv;
    double2 gj = g[j];
    g[j + 1] = make_double2(-(sv.x * gj.x + sv.y * gj.y), -(sv.x * gj.y - sv.y * gj.x));
    g[j] = make_double2(c * gj.x, c * gj.y);
    double res = hypot(g[j + 1].x, g[j + 1].y);
    s.jlen[r] = j + 1;
    s.est[r] = res;
    double thr = fmax(s.inner * (s.tol_abs ? s.tol : s.tol * s.bnorm[r]), s.red * s.true_res[r] * s.bnorm[r]);
    bool breakdown = beta <= 1e-14 * s.bnorm[r];
    if (res < thr || breakdown || j + 1 == m) {
        s.active[r] = 0;
        s.scale[r] = 0.0;
    } else {
        s.scale[r] = 1.0 / beta;
        atomicAdd(s.step_cnt, 1);
    }
}

// V_out[r][k] = scale[r] * W[r][k]
// k_arnoldi_finish for restarts of at most 32: warp per RHS, lane i holds
// entry i of the new Hessenberg column and rotation i (loaded together), the
// previous rotations run through shuffles instead of a chain of dependent
// memory accesses, and the column is written back at once.  Same arithmetic,
// in the same order, as k_arnoldi_finish.
__device__ __forceinline__ double2 shfl_d2(double2 v, int src)
{
    return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// Arnoldi column j of right-hand side r (one warp): lane i <= j holds the
// Gram-Schmidt coefficient h_i, beta = ||w||.  Applies the previous
// rotations, forms the new one, updates g and tests convergence.
__device__ void arnoldi_column(const GmresDev& s, int r, int j, double2 h, double beta)
{
    const int lane = threadIdx.x & 31, m = s.m;
    double2* H = s.H + (size_t)r * (m + 1) * m;
    double* cs = s.cs + (size_t)r * m;
    double2* sn = s.sn + (size_t)r * m;
    const double cl = lane < j ? cs[lane] : 0.0;
    const double2 sl = lane < j ? sn[lane] : make_double2(0.0, 0.0);
    // previous rotations: [x; y] <- [c x + s y; -conj(s) x + c y] on entries (i, i + 1)
    for (int i = 0; i < j; ++i) {
        const double2 y = shfl_d2(h, i + 1), x = shfl_d2(h, i);
        const double c = __shfl_sync(0xffffffffu, cl, i);
        const double2 sv = shfl_d2(sl, i);
        if (lane == i)
            h = make_double2(c * x.x + sv.x * y.x - sv.y * y.y, c * x.y + sv.x * y.y + sv.y * y.x);
        else if (lane == i + 1)
            h = make_double2(-(sv.x * x.x + sv.y * x.y) + c * y.x, -(sv.x * x.y - sv.y * x.x) + c * y.y);
    }
    if (lane == j) {
        const double2 a = h;
        const double b = beta;
        const double aa = hypot(a.x, a.y);
        const double nu = hypot(aa, b);
        double c;
        double2 sv;
        if (aa == 0.0) {
            c = 0.0;
            sv = make_double2(1.0, 0.0);
            h = make_double2(b, 0.0);
        } else {
            c = aa / nu;
            const double2 ph = make_double2(a.x / aa, a.y / aa);
            sv = make_double2(ph.x * b / nu, ph.y * b / nu);
            h = make_double2(ph.x * nu, ph.y * nu);
        }
        H[(j + 1) * m + j] = make_double2(0.0, 0.0);
        cs[j] = c;
        sn[j] = sv;
        double2* g = s.g + (size_t)r * (m + 1);
        const double2 gj = g[j];
        g[j + 1] = make_double2(-(sv.x * gj.x + sv.y * gj.y), -(sv.x * gj.y - sv.y * gj.x));
        g[j] = make_double2(c * gj.x, c * gj.y);
        const double res = hypot(g[j + 1].x, g[j + 1].y);
        s.jlen[r] = j + 1;
        s.est[r] = res;
        const double thr =
            fmax(s.inner * (s.tol_abs ? s.tol : s.tol * s.bnorm[r]), s.red * s.true_res[r] * s.bnorm[r]);
        const bool breakdown = beta <= 1e-14 * s.bnorm[r];
        if (res < thr || breakdown || j + 1 == m) {
            s.active[r] = 0;
            s.scale[r] = 0.0;
        } else {
            s.scale[r] = 1.0 / beta;
            atomicAdd(s.step_cnt, 1);
        }
    }
    if (lane <= j) H[lane * m + j] = h;
}

// FP32 form of arnoldi_column for the FP32-basis inner solve of the
// refinement: the same steps in FP32 arithmetic, with H, cs, sn and g kept in
// FP64 memory.  GB300's FP64 pipe takes about 64 cycles a warp instruction,
// so the FP64 chain of a column (rotations, two hypot, four divisions) ran
// for 10-20 us; the coefficients of an FP32 basis carry ~1e-7 relative error
// already, and every restart recomputes the true residual in FP64.
__device__ __forceinline__ float2 shfl_f2(float2 v, int src)
{
    return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

__device__ void arnoldi_column_f32(const GmresDev& s, int r, int j, double2 hd, float beta)
{
    const int lane = threadIdx.x & 31, m = s.m;
    double2* H = s.H + (size_t)r * (m + 1) * m;
    double* cs = s.cs + (size_t)r * m;
    double2* sn = s.sn + (size_t)r * m;
    float2 h = make_float2((float)hd.x, (float)hd.y);
    const float cl = lane < j ? (float)cs[lane] : 0.f;
    const double2 sld = lane < j ? sn[lane] : make_double2(0.0, 0.0);
    const float2 sl = make_float2((float)sld.x, (float)sld.y);
    for (int i = 0; i < j; ++i) {
        const float2 y = shfl_f2(h, i + 1), x = shfl_f2(h, i);
        const float c = __shfl_sync(0xffffffffu, cl, i);
        const float2 sv = shfl_f2(sl, i);
        if (lane == i)
            h = make_float2(c * x.x + sv.x * y.x - sv.y * y.y, c * x.y + sv.x * y.y + sv.y * y.x);
        else if (lane == i + 1)
            h = make_float2(-(sv.x * x.x + sv.y * x.y) + c * y.x, -(sv.x * x.y - sv.y * x.x) + c * y.y);
    }
    if (lane == j) {
        const float2 a = h;
        const float b = beta;
        const float aa = hypotf(a.x, a.y);
        const float nu = hypotf(aa, b);
        float c;
        float2 sv;
        if (aa == 0.f) {
            c = 0.f;
            sv = make_float2(1.f, 0.f);
            h = make_float2(b, 0.f);
        } else {
            c = aa / nu;
            const float2 ph = make_float2(a.x / aa, a.y / aa);
            sv = make_float2(ph.x * b / nu, ph.y * b / nu);
            h = make_float2(ph.x * nu, ph.y * nu);
        }
        H[(j + 1) * m + j] = make_double2(0.0, 0.0);
        cs[j] = c;
        sn[j] = make_double2(sv.x, sv.y);
        double2* g = s.g + (size_t)r * (m + 1);
        const double2 gjd = g[j];
        const float2 gj = make_float2((float)gjd.x, (float)gjd.y);
        const float2 gn = make_float2(-(sv.x * gj.x + sv.y * gj.y), -(sv.x * gj.y - sv.y * gj.x));
        g[j + 1] = make_double2(gn.x, gn.y);
        g[j] = make_double2(c * gj.x, c * gj.y);
        const double res = hypotf(gn.x, gn.y);
        s.jlen[r] = j + 1;
        s.est[r] = res;
        const double thr =
            fmax(s.inner * (s.tol_abs ? s.tol : s.tol * s.bnorm[r]), s.red * s.true_res[r] * s.bnorm[r]);
        const bool breakdown = (double)beta <= 1e-14 * s.bnorm[r];
        if (res < thr || breakdown || j + 1 == m) {
            s.active[r] = 0;
            s.scale[r] = 0.0;
        } else {
            s.scale[r] = 1.0 / (double)beta;
            atomicAdd(s.step_cnt, 1);
        }
    }
    if (lane <= j) H[lane * m + j] = make_double2(h.x, h.y);
}

__global__ void k_arnoldi_finish_warp(GmresDev s, int j, const double2* __restrict__ pnorm, int nblk, int two_pass)
{
    const int r = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (r >= s.nrhs) return;  // whole warps
    if (!s.active[r]) {
        if (lane == 0) s.scale[r] = 0.0;
        return;
    }
    double beta = 0.0;
    if (lane == 0) {
        double nr2 = 0.0, wm = 0.0;
        for (int b = 0; b < nblk; ++b) {
            nr2 += pnorm[(size_t)r * nblk + b].x;
            wm = fmax(wm, pnorm[(size_t)r * nblk + b].y);
        }
        s.wmax[r] = wm;
        beta = sqrt(nr2);
    }
    beta = __shfl_sync(0xffffffffu, beta, 0);
    double2 h = make_double2(0.0, 0.0);
    if (lane <= j) {
        h = s.hcol[(size_t)lane * s.nrhs + r];
        if (two_pass) {
            const double2 b = s.y[(size_t)lane * s.nrhs + r];
            h.x += b.x;
            h.y += b.y;
        }
    }
    arnoldi_column(s, r, j, h, beta);
}

// Last kernel of the separate-pass CGS1 step (FP32 basis, restarts up to
// 32): CTA per (chunk of FP_CHUNK elements, right-hand side).  Every CTA forms
// beta = ||w|| and the FP16 scale from the update's partials (the same sums
// in the same order, so the same values) and writes its chunk of
// V_{j+1} = W / beta and, for operators that pack their input, the FP16 rows
// of the next product (as k_hpack_scale).  In the first chunk's CTA, warp 0
// finishes the Arnoldi column (as k_arnoldi_finish_warp, single pass) while
// the other warps pack: the column's serial chain (FP32) overlaps the stream.
// A right-hand side that this step finds converged is normalised all the
// same (its V_{j+1} lies past its basis length); one that was already
// inactive writes nothing.  On the FP16 basis Vout is null: the packed rows
// (plane j + 1 of the basis) are V_{j+1}.  The stream moves element pairs,
// four 16-byte loads a thread issued before any store: 0.70 -> 0.51 ms a
// job on the dense CFIE job (7680 x 360).
constexpr int FP_CHUNK = 4096;

template <bool ODD>
__global__ void __launch_bounds__(256) k_finish_pack(GmresDev s, int j, const double2* __restrict__ pnorm, int nblk,
                                                     const float2* __restrict__ W, int n, float2* __restrict__ Vout,
                                                     HPack pk)
{
    __shared__ float sbeta;
    __shared__ float nscale[2];
    const int r = blockIdx.y, chunk = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
    griddep_wait();
    if (!s.active[r]) {
        if (chunk == 0 && tid == 0) s.scale[r] = 0.0;
        return;
    }
    if (tid == 0) {
        // FP32 on one thread (FP64 would cost ~64 cycles an instruction here)
        float nr2 = 0.f, wm = 0.f;
        for (int b = 0; b < nblk; ++b) {
            nr2 += (float)pnorm[(size_t)r * nblk + b].x;
            wm = fmaxf(wm, (float)pnorm[(size_t)r * nblk + b].y);
        }
        const float beta = sqrtf(nr2);
        const float scale = beta > 0.f ? 1.f / beta : 0.f;
        sbeta = beta;
        nscale[0] = scale;
        nscale[1] = 1.f;
        int ex = 0;
        if (pk.bh) {
            ex = hpack_exponent_f(wm, scale);
            nscale[1] = ldexpf(1.f, 14 - ex);
        }
        if (chunk == 0) {
            s.wmax[r] = wm;
            if (pk.bh) pk.inv_t[r] = ldexpf(1.f, ex - 14);
        }
    }
    __syncthreads();
    const bool column = chunk == 0;
    if (column && tid < 32) {
        const double2 h = lane <= j ? s.hcol[(size_t)lane * s.nrhs + r] : make_double2(0.0, 0.0);
        arnoldi_column_f32(s, r, j, h, sbeta);
        return;
    }
    const float sc = nscale[0], t = nscale[1];
    const int k1 = min(n, (chunk + 1) * FP_CHUNK), off = column ? 32 : 0, nt = blockDim.x - off;
    // element pairs, PB of a thread's loads issued before any store (16
    // bytes each; two 8-byte loads for odd N): one round trip for a chunk
    // instead of four.  Past the vector (odd N) the pair's second element is
    // 0: V's is not stored, the rows' goes to their padding
    constexpr int PB = 4;
    const float2* w = W + (size_t)r * n;
    float2* v = Vout ? Vout + (size_t)r * n : nullptr;
    uint2* g0 = pk.bh ? reinterpret_cast<uint2*>(pk.bh + (size_t)(2 * r) * pk.ldh) : nullptr;
    uint2* g1 = pk.bh ? reinterpret_cast<uint2*>(pk.bh + (size_t)(2 * r + 1) * pk.ldh) : nullptr;
    const int q1 = (k1 + 1) >> 1;
    for (int qb = ((chunk * FP_CHUNK) >> 1) + tid - off; qb < q1; qb += PB * nt) {
        float4 x[PB];
#pragma unroll
        for (int u = 0; u < PB; ++u) {
            const int q = qb + u * nt;
            x[u] = q < q1 ? ld_wpair<ODD>(w, q, n) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < PB; ++u) {
            const int q = qb + u * nt;
            if (q >= q1) continue;
            const float4 y = make_float4(x[u].x * sc, x[u].y * sc, x[u].z * sc, x[u].w * sc);
            if (v) st_wpair<ODD>(v, q, n, y);
            if (g0) {
                const __half re0 = __float2half_rn(t * y.x), im0 = __float2half_rn(t * y.y);
                const __half re1 = __float2half_rn(t * y.z), im1 = __float2half_rn(t * y.w);
                g0[q] = make_uint2(h2u(__halves2half2(re0, __hneg(im0))), h2u(__halves2half2(re1, __hneg(im1))));
                g1[q] = make_uint2(h2u(__halves2half2(im0, re0)), h2u(__halves2half2(im1, re1)));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// One Arnoldi step in one launch (FP32 basis, CGS1): a cluster of CS <= 8
// CTAs per right-hand side, CTA `rank` owning elements [rank slice,
// (rank + 1) slice) of the N, E per thread, held in registers throughout.
//   1. w and the basis slices are staged in shared memory by asynchronous
//      copies (up to 104 KB a CTA, all in flight at once); partial
//      coefficients h_i = V_i^H w over the slice, a warp per vector (FP32
//      within the warp), published in shared memory in FP64
//   2. cluster barrier; every CTA sums the cluster's partials in rank order
//      from distributed shared memory (the same FP64 sums in every CTA)
//   3. w -= sum_i h_i V_i over the slice, from the staged slices (a restart
//      longer than the staging holds reads its earlier vectors again from
//      L2: the cluster read them microseconds before).  |w|^2 and
//      max |Re|, |Im| partials
//   4. cluster barrier; beta = ||w||; v = w / beta goes to V_{j+1} and, for
//      operators that pack their input, to the FP16 rows of the next product
//      (the packing k_hpack_scale does: same scale, same rounding)
//   5. the first CTA's warp 0 finishes the Arnoldi column (arnoldi_column)
// W is read once and never written: the next product reads the packed rows
// (or V_{j+1}).  A right-hand side that is no longer active writes nothing
// (its V_{j+1} is past its basis length; its rows in the product's operand
// still hold its last, finite vector).  Replaces k_vdots, k_vupdate,
// k_arnoldi_finish_warp and the normalisation pass: one launch instead of
// four, the basis read once from HBM, W once.  Each CTA's work is a chain
// (staging, two cluster barriers, FP64 sums on one thread, the Givens
// column on the first CTA), so the step is faster where launches and
// latency dominate (tens of right-hand sides) and the separate passes are
// faster for hundreds; the solver picks by the grid size.
// ---------------------------------------------------------------------------
constexpr int AS_THREADS = 512;
constexpr int AS_WARPS = AS_THREADS / 32;
constexpr int AS_MAXV = 32;     // restart lengths up to 32 (one coefficient per lane in arnoldi_column)
constexpr int AS_MAX_CLUSTER = 8;
constexpr int AS_STAGE_BYTES = 104 * 1024;  // staged slices a CTA: two CTAs an SM

__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
// a double2 in the shared memory of CTA `rank` of the cluster, at the
// address `local` has in this CTA
__device__ __forceinline__ double2 ld_cluster_d2(const double2* local, int rank)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(local);
    uint32_t ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    double x, y;
    asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(x), "=d"(y) : "r"(ra) : "memory");
    return make_double2(x, y);
}

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

template <int E>
__global__ void __launch_bounds__(AS_THREADS, 2)
    k_arnoldi_step(GmresDev s, int j, const float2* __restrict__ V, size_t vstride, const float2* __restrict__ W,
                   int n, int slice, int sv, float2* __restrict__ Vout, HPack pk)
{
    constexpr int SW = AS_THREADS * E;  // elements of a staged slice (>= slice)
    extern __shared__ float2 stage[];   // w, then sv basis slices
    float2* sW = stage;
    float2* sV = stage + SW;
    __shared__ double2 hpart[AS_MAXV];  // this CTA's partial coefficients (read by the cluster)
    __shared__ double2 hs[AS_MAXV];     // the cluster's sums
    __shared__ float2 hf[AS_MAXV];
    __shared__ double2 nred[AS_WARPS];
    __shared__ double2 npart;           // this CTA's |w|^2 and max (read by the cluster)
    __shared__ double2 ntot;            // beta and max |Re|, |Im| of w
    __shared__ float nscale[2];         // 1 / beta and the FP16 scale t

    const int r = blockIdx.y, rank = blockIdx.x, csize = gridDim.x;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (!s.active[r]) {  // the same branch in every CTA of the cluster: no barrier is left waiting
        if (rank == 0 && tid == 0) s.scale[r] = 0.0;
        return;
    }
    const int nv = j + 1;
    const int k0 = rank * slice, len = min(n, k0 + slice) - k0;  // len >= 1 for every rank
    const float2* Vs = V + (size_t)r * n + k0;                    // this slice of basis vector 0
    const float2* Ws = W + (size_t)r * n + k0;

    // 1. partial coefficients.  Each round stages (asynchronous copies, all
    // in flight at once) up to sv basis slices, and w in the first; warp q
    // then reduces the round's vectors q, q + 16 from shared memory.
    int vlast = 0;  // first basis vector of the last round (still staged)
    for (int v0 = 0; v0 < nv; v0 += sv) {
        const int v1 = min(nv, v0 + sv);
        vlast = v0;
        if (v0 > 0) __syncthreads();  // the previous round's reads are done
        if (v0 == 0)
            for (int k = tid; k < len; k += AS_THREADS) cp_async8(sW + k, Ws + k);
        for (int i = v0; i < v1; ++i)
            for (int k = tid; k < len; k += AS_THREADS) cp_async8(sV + (size_t)(i - v0) * SW + k, Vs + (size_t)i * vstride + k);
        cp_async_wait_all();
        __syncthreads();
        for (int i = v0 + warp; i < v1; i += AS_WARPS) {
            const float2* vi = sV + (size_t)(i - v0) * SW;
            float ar = 0.f, ai = 0.f;
#pragma unroll 4
            for (int k = lane; k < len; k += 32) {
                const float2 a = vi[k], x = sW[k];
                ar += a.x * x.x + a.y * x.y;
                ai += a.x * x.y - a.y * x.x;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                ar += __shfl_xor_sync(0xffffffffu, ar, o);
                ai += __shfl_xor_sync(0xffffffffu, ai, o);
            }
            if (lane == 0) hpart[i] = make_double2((double)ar, (double)ai);
        }
    }
    // 2. the cluster's sums (the barrier also orders this CTA's own writes)
    cluster_arrive();
    cluster_wait();
    if (tid < AS_MAXV) {
        double2 t = make_double2(0.0, 0.0);
        if (tid < nv)
            for (int c = 0; c < csize; ++c) {
                const double2 p = ld_cluster_d2(&hpart[tid], c);
                t.x += p.x;
                t.y += p.y;
            }
        hs[tid] = t;
        hf[tid] = make_float2((float)t.x, (float)t.y);
    }
    __syncthreads();

    // 3. w -= V h: the last round's slices from shared memory, earlier rounds'
    // (restarts longer than sv) again from global memory, where they were
    // read microseconds earlier
    float2 w[E];
    float nr = 0.f, mx = 0.f;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int k = tid + e * AS_THREADS;
        w[e] = make_float2(0.f, 0.f);
        if (k >= len) continue;
        float sr = 0.f, si = 0.f;
#pragma unroll 4
        for (int i = 0; i < vlast; ++i) {
            const float2 v = Vs[(size_t)i * vstride + k];
            const float2 h = hf[i];
            sr += h.x * v.x - h.y * v.y;
            si += h.x * v.y + h.y * v.x;
        }
#pragma unroll 4
        for (int i = vlast; i < nv; ++i) {
            const float2 v = sV[(size_t)(i - vlast) * SW + k];
            const float2 h = hf[i];
            sr += h.x * v.x - h.y * v.y;
            si += h.x * v.y + h.y * v.x;
        }
        const float2 x = sW[k];
        w[e] = make_float2(x.x - sr, x.y - si);
        nr += w[e].x * w[e].x + w[e].y * w[e].y;
        mx = fmaxf(mx, fmaxf(fabsf(w[e].x), fabsf(w[e].y)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nr += __shfl_xor_sync(0xffffffffu, nr, o);
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane == 0) nred[warp] = make_double2((double)nr, (double)mx);
    __syncthreads();
    if (tid == 0) {
        double t = 0.0, tm = 0.0;
        for (int q = 0; q < AS_WARPS; ++q) {
            t += nred[q].x;
            tm = fmax(tm, nred[q].y);
        }
        npart = make_double2(t, tm);
    }
    // 4. beta and the normalised vector
    cluster_arrive();
    cluster_wait();
    if (tid == 0) {
        // one thread, and FP32 for the root and the division (an FP64
        // instruction costs ~64 cycles of GB300's FP64 pipe)
        double nr2 = 0.0, wm = 0.0;
        for (int c = 0; c < csize; ++c) {
            const double2 p = ld_cluster_d2(&npart, c);
            nr2 += p.x;
            wm = fmax(wm, p.y);
        }
        const float beta = sqrtf((float)nr2);
        const float scale = beta > 0.f ? 1.f / beta : 0.f;
        ntot = make_double2(beta, wm);
        nscale[0] = scale;
        nscale[1] = 1.f;
        if (pk.bh) {
            const int ex = hpack_exponent_f((float)wm, scale);
            nscale[1] = ldexpf(1.f, 14 - ex);
            if (rank == 0) pk.inv_t[r] = ldexpf(1.f, ex - 14);
        }
    }
    __syncthreads();
    cluster_arrive();  // this CTA's reads of the others' shared memory are done
    const float sc = nscale[0], t = nscale[1];
    __half2* h0 = pk.bh ? reinterpret_cast<__half2*>(pk.bh + (size_t)(2 * r) * pk.ldh) + k0 : nullptr;
    __half2* h1 = pk.bh ? reinterpret_cast<__half2*>(pk.bh + (size_t)(2 * r + 1) * pk.ldh) + k0 : nullptr;
    float2* vo = Vout + (size_t)r * n + k0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int k = tid + e * AS_THREADS;
        if (k >= len) continue;
        const float2 y = make_float2(w[e].x * sc, w[e].y * sc);
        vo[k] = y;
        if (h0) {
            const __half hre = __float2half_rn(t * y.x), him = __float2half_rn(t * y.y);
            h0[k] = __halves2half2(hre, __hneg(him));
            h1[k] = __halves2half2(him, hre);
        }
    }
    // 5. the Arnoldi column
    if (rank == 0 && warp == 0) {
        if (lane == 0) s.wmax[r] = ntot.y;
        arnoldi_column_f32(s, r, j, lane <= j ? hs[lane] : make_double2(0.0, 0.0), (float)ntot.x);
    }
    cluster_wait();  // no CTA leaves while another may still read its shared memory
}

// out[r] = scale[r] W[r]: grid over (chunks of 1024, RHS).  An FP32 basis is
// scaled in FP32 and an FP64 source converted by split_f64 (integer
// operations): FP64 products and conversions per element would run on
// GB300's 1/64-rate FP64 pipe.
template <typename T> __device__ __forceinline__ float to_f32(T v) { return (float)v; }
template <> __device__ __forceinline__ float to_f32<double>(double v) { return split_f64(v).x; }
__device__ __forceinline__ double cre(double2 v) { return v.x; }
__device__ __forceinline__ double cim(double2 v) { return v.y; }
template <typename T> __device__ __forceinline__ T cre(Cx<T> v) { return v.re; }
template <typename T> __device__ __forceinline__ T cim(Cx<T> v) { return v.im; }

template <typename TO, typename TI>
__global__ void k_scale_store(const TI* __restrict__ W, const double* __restrict__ scale, int n, int nrhs,
                              TO* __restrict__ out)
{
    using R = decltype(out->re);
    const int r = blockIdx.y;
    const R sc = (R)scale[r];
    const size_t base = (size_t)r * n;
    const int k1 = min(n, (int)(blockIdx.x + 1) * 1024);
    for (int k = blockIdx.x * 1024 + threadIdx.x; k < k1; k += blockDim.x) {
        const TI w = W[base + k];
        if constexpr (sizeof(R) == 4)
            out[base + k] = TO{to_f32(cre(w)) * sc, to_f32(cim(w)) * sc};
        else
            out[base + k] = TO{(R)cre(w) * sc, (R)cim(w) * sc};
    }
}

// per-RHS back substitution of the rotated Hessenberg system
__global__ void k_backsolve(GmresDev s)
{
    // one RHS per warp (lane 0): the FP64 chains of the RHS spread over the SMs
    const int r = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if ((threadIdx.x & 31) != 0 || r >= s.nrhs) return;
    const int m = s.m;
    int jl = s.jlen[r];
    const double2* H = s.H + (size_t)r * (m + 1) * m;
    const double2* g = s.g + (size_t)r * (m + 1);
    double2* y = s.y;  // y[i * nrhs + r]
    for (int i = m - 1; i >= jl; --i) y[(size_t)i * s.nrhs + r] = make_double2(0.0, 0.0);
    for (int i = jl - 1; i >= 0; --i) {
        double2 acc = g[i];
        for (int q = i + 1; q < jl; ++q) {
            double2 h = H[i * m + q], yq = y[(size_t)q * s.nrhs + r];
            acc.x -= h.x * yq.x - h.y * yq.y;
            acc.y -= h.x * yq.y + h.y * yq.x;
        }
        double2 d = H[i * m + i];
        double den = d.x * d.x + d.y * d.y;
        double2 v = den > 0 ? make_double2((acc.x * d.x + acc.y * d.y) / den, (acc.y * d.x - acc.x * d.y) / den)
                            : make_double2(0.0, 0.0);
        y[(size_t)i * s.nrhs + r] = v;
    }
}

// The same for the FP32-basis inner solve (restarts up to 32): a warp per
// right-hand side, lane q holding row q of the triangle (staged in shared
// memory in FP32), column-oriented: y_i = b_i / H_ii on lane i, broadcast,
// then every lane q < i takes b_q -= H_qi y_i.  FP32 like the basis; the
// serial FP64 form spent ~60 us a launch on GB300's FP64 pipe.
constexpr int BS_WARPS = 4;

__global__ void __launch_bounds__(32 * BS_WARPS) k_backsolve_f32(GmresDev s)
{
    __shared__ float2 sh[BS_WARPS][32][33];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * BS_WARPS + w;
    if (r >= s.nrhs) return;  // whole warps
    const int m = s.m, jl = s.jlen[r];
    const double2* H = s.H + (size_t)r * (m + 1) * m;
    for (int i = 0; i < jl; ++i)
        if (lane < jl) {
            const double2 v = H[i * m + lane];
            sh[w][i][lane] = make_float2((float)v.x, (float)v.y);
        }
    __syncwarp();
    const double2 gl = lane < jl ? s.g[(size_t)r * (m + 1) + lane] : make_double2(0.0, 0.0);
    float2 b = make_float2((float)gl.x, (float)gl.y), yl = make_float2(0.f, 0.f);
    for (int i = jl - 1; i >= 0; --i) {
        float2 yi = make_float2(0.f, 0.f);
        if (lane == i) {
            const float2 d = sh[w][i][i];
            const float den = d.x * d.x + d.y * d.y;
            if (den > 0.f) yi = make_float2((b.x * d.x + b.y * d.y) / den, (b.y * d.x - b.x * d.y) / den);
            yl = yi;
        }
        yi = make_float2(__shfl_sync(0xffffffffu, yi.x, i), __shfl_sync(0xffffffffu, yi.y, i));
        if (lane < i) {
            const float2 h = sh[w][lane][i];
            b.x -= h.x * yi.x - h.y * yi.y;
            b.y -= h.x * yi.y + h.y * yi.x;
        }
    }
    if (lane < m) s.y[(size_t)lane * s.nrhs + r] = make_double2((double)yl.x, (double)yl.y);
}


// R = B - Y (all complex128; B may be complex64)
template <typename TB>
__global__ void k_residual(const TB* __restrict__ B, const double2* __restrict__ Y, double2* __restrict__ R, size_t tot)
{
    size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; id < tot; id += (size_t)gridDim.x * blockDim.x) {
        double2 b = ld2(B + id), y = Y[id];
        R[id] = make_double2(b.x - y.x, b.y - y.y);
    }
}

__global__ void k_to_f32(const double2* __restrict__ X, float2* __restrict__ Y, size_t tot)
{
    size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; id < tot; id += (size_t)gridDim.x * blockDim.x) Y[id] = make_float2((float)X[id].x, (float)X[id].y);
}

__global__ void k_to_f64(const float2* __restrict__ X, double2* __restrict__ Y, size_t tot)
{
    size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; id < tot; id += (size_t)gridDim.x * blockDim.x) Y[id] = make_double2((double)X[id].x, (double)X[id].y);
}

// start of a restart cycle: beta = ||R||, convergence test, g = beta e1
__global__ void k_cycle_init(GmresDev s, const double2* __restrict__ pnorm, int nblk, int first)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= s.nrhs) return;
    double nr2 = 0.0;
    for (int b = 0; b < nblk; ++b) nr2 += pnorm[(size_t)r * nblk + b].x;
    double beta = sqrt(nr2);
    if (first) s.bnorm[r] = beta;  // x0 = 0: first residual is b
    s.true_res[r] = s.bnorm[r] > 0 ? beta / s.bnorm[r] : 0.0;
    double thr = s.tol_abs ? s.tol : s.tol * s.bnorm[r];
    double2* g = s.g + (size_t)r * (s.m + 1);
    for (int i = 0; i <= s.m; ++i) g[i] = make_double2(0.0, 0.0);
    g[0] = make_double2(beta, 0.0);
    s.jlen[r] = 0;
    if (beta < thr || beta == 0.0) {
        s.active[r] = 0;
        s.scale[r] = 0.0;
        atomicAdd(s.counters + 1, 1);  // converged
    } else {
        s.active[r] = 1;
        s.scale[r] = 1.0 / beta;
        atomicAdd(s.counters, 1);  // active
    }
}

__global__ void k_accumulate(double2* __restrict__ a, const double2* __restrict__ b, int tot)
{
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id < tot) {
        a[id].x += b[id].x;
        a[id].y += b[id].y;
    }
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
static int dot_blocks(int n) { return (n + KCHUNK - 1) / KCHUNK; }

template <typename T>
static emfa_status_t dots(Ctx* c, const Cx<T>* V, size_t vstride, int nv, const void* W, bool w_double, int n,
                          int nrhs, double2* partial, double2* out, int accumulate, cudaStream_t st)
{
    int nblk = dot_blocks(n);
    dim3 grd(nblk, nrhs);
    if (w_double)
        k_block_dots<Cx<T>, double2><<<grd, KB, 0, st>>>(V, vstride, nv, (const double2*)W, n, nrhs, nblk, partial);
    else
        k_block_dots<Cx<T>, Cx<T>><<<grd, KB, 0, st>>>(V, vstride, nv, (const Cx<T>*)W, n, nrhs, nblk, partial);
    k_reduce_partials<<<(nv * nrhs + 127) / 128, 128, 0, st>>>(partial, nv, nrhs, nblk, out, accumulate);
    c->kernel_launches += 2;
    return EMFA_OK;
}

static int grid1(size_t tot) { return (int)std::min<size_t>((tot + 255) / 256, 8192); }

// cluster shape of the fused Arnoldi step for N unknowns: CTAs per
// right-hand side, elements per CTA and per thread (0: N too large)
struct StepShape {
    int cs = 0, slice = 0, e = 0;
};
static StepShape step_shape(int n)
{
    StepShape sh;
    sh.cs = std::min(AS_MAX_CLUSTER, std::max(1, (n + 1023) / 1024));
    sh.slice = (n + sh.cs - 1) / sh.cs;
    const int e = (sh.slice + AS_THREADS - 1) / AS_THREADS;
    sh.e = e <= 1 ? 1 : e <= 2 ? 2 : e <= 4 ? 4 : 0;
    return sh;
}

template <int E>
static emfa_status_t launch_step_e(Ctx* c, const StepShape& sh, int nrhs, cudaStream_t st, const GmresDev& s, int j,
                                   const float2* V, size_t vstride, const float2* W, int n, float2* Vout,
                                   const HPack& pk)
{
    const int sw = AS_THREADS * E;  // staged slice
    const int sv = std::min(AS_MAXV, AS_STAGE_BYTES / (int)(sizeof(float2) * sw) - 1);
    const size_t smem = sizeof(float2) * (size_t)sw * (sv + 1);
    EMFA_TRY(ensure_smem(c, k_arnoldi_step<E>, smem));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(sh.cs, nrhs);
    cfg.blockDim = dim3(AS_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = sh.cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    EMFA_CUDA(c, cudaLaunchKernelEx(&cfg, k_arnoldi_step<E>, s, j, V, vstride, W, n, sh.slice, sv, Vout, pk));
    return EMFA_OK;
}

static emfa_status_t launch_arnoldi_step(Ctx* c, const StepShape& sh, int nrhs, cudaStream_t st, const GmresDev& s,
                                         int j, const float2* V, size_t vstride, const float2* W, int n, float2* Vout,
                                         const HPack& pk)
{
    if (sh.e == 1) return launch_step_e<1>(c, sh, nrhs, st, s, j, V, vstride, W, n, Vout, pk);
    if (sh.e == 2) return launch_step_e<2>(c, sh, nrhs, st, s, j, V, vstride, W, n, Vout, pk);
    return launch_step_e<4>(c, sh, nrhs, st, s, j, V, vstride, W, n, Vout, pk);
}

template <typename T>
static emfa_status_t gmres_t(Ctx* c, LinOp& A, const void* B, int nrhs, double2* X, const emfa_solver_params_t* sp,
                             emfa_solve_info_t* info, cudaStream_t st)
{
    const int n = A.n, prec = A.prec;
    const int m = std::max(1, std::min(sp->restart > 0 ? sp->restart : 30, MAX_RESTART));
    const size_t vec = (size_t)n * nrhs;
    // residual-norm grid: at least ~2 CTAs per SM over (chunks of N) x
    // (right-hand sides), chunks of at most 2048 elements (with one CTA a
    // right-hand side, 360 of them streamed 123 KB each: 23 us a launch on
    // the dense CFIE job), and at least 4 elements a thread (1024 a CTA)
    const int sms = c->sm_count > 0 ? c->sm_count : 148;
    const int nblk = std::max(1, std::min(std::max((2 * sms + nrhs - 1) / nrhs, (n + 2047) / 2048),
                                          (n + 4 * KB - 1) / (4 * KB)));
    const int chunk = (n + nblk - 1) / nblk;
    const int vblk = (n + VCHUNK - 1) / VCHUNK;  // chunks of the Gram-Schmidt passes
    // the FP32 inner solve of the refinement only has to gain a few digits per
    // cycle: one Gram-Schmidt pass; the plain FP64 path keeps two
    const bool two_pass = sp->orth == 2 || (sp->orth == 0 && prec == EMFA_F64);
    // CGS1 on an FP32 basis: one fused launch per Arnoldi step (k_arnoldi_step)
    // where the restart and N fit it and its clusters fill at most about two
    // waves of CTAs; orth 3 keeps the separate passes.  Measured GMRES(30)
    // solves (split-FP16 products, 18 steps): fused 10-15 % faster for 1 to
    // 64 right-hand sides at N = 2000, 4000 and 7680; 4-8 % slower for 360,
    // where the separate passes' thousands of independent CTAs hide memory
    // latency better than two staged CTAs an SM between cluster barriers.
    const StepShape sh = step_shape(n);
    // orth 4 takes the fused step whatever the grid size (for measurement)
    const bool fused = std::is_same<T, float>::value && !two_pass && sp->orth != 3 && m <= AS_MAXV && sh.e > 0 &&
                       ((long)nrhs * sh.cs <= 4L * sms || sp->orth == 4);
    // separate passes on an FP32 basis with one Gram-Schmidt pass end in
    // k_finish_pack (column, normalisation and packing in one launch)
    const bool finish_pack = std::is_same<T, float>::value && !fused && !two_pass && m <= 32;
    // ... and keep the basis as the product's FP16 operand rows where the
    // operator packs its input (unless basis = 1): m + 1 planes of the
    // layout pack_target gives
    HPack pk0;
    const bool hbasis = finish_pack && sp->basis != 1 && A.pack_target(c, nrhs, &pk0);
    const size_t hplane = hbasis ? pk0.ldh * 2 * (size_t)nrhs : 0;  // halves
    const size_t vslots = hbasis ? 1 : (size_t)(m + 1);
    // one workspace for the whole solve (reused across solves of a context)
    const size_t need = Carver::round(sizeof(Cx<T>) * vec * vslots) + Carver::round(sizeof(Cx<T>) * vec) +
                        Carver::round(sizeof(__half) * hplane * (m + 1)) +
                        Carver::round(sizeof(float) * (size_t)nrhs * (m + 1)) +
                        Carver::round(sizeof(double2) * vec) + Carver::round(sizeof(float2) * vec) +
                        Carver::round(sizeof(double2) * (size_t)nrhs * (m + 1) * m) +
                        Carver::round(sizeof(double) * (size_t)nrhs * m) +
                        Carver::round(sizeof(double2) * (size_t)nrhs * m) * 2 +
                        Carver::round(sizeof(double2) * (size_t)nrhs * (m + 1)) * 2 +
                        Carver::round(sizeof(double2) * (size_t)nrhs * (m + 1) * std::max(nblk, (n + VCHUNK - 1) / VCHUNK)) +
                        Carver::round(sizeof(double2) * (size_t)nrhs * std::max(nblk, (n + VCHUNK - 1) / VCHUNK)) +
                        Carver::round(sizeof(double) * 5 * (size_t)nrhs) + Carver::round(sizeof(int) * 2 * (size_t)nrhs) +
                        Carver::round(sizeof(int) * 4) + 4096;
    void* wsp = nullptr;
    EMFA_TRY(ctx_workspace(c, WS_KRYLOV, need, &wsp));
    Carver cv{(char*)wsp};
    Cx<T>* V = cv.take<Cx<T>>(vec * vslots);
    Cx<T>* W = cv.take<Cx<T>>(vec);
    __half* Bh = cv.take<__half>(hplane * (m + 1));     // FP16 basis planes (hbasis)
    float* inv_tb = cv.take<float>((size_t)nrhs * (m + 1));  //   and their per-RHS scales
    double2* R = cv.take<double2>(vec);
    float2* Xt = cv.take<float2>(vec);
    GmresDev s;
    s.m = m;
    s.nrhs = nrhs;
    s.tol = sp->tol;
    s.tol_abs = sp->tol_absolute;
    // the inner solve of a refinement whose products are less accurate than
    // its residual stops short of the target so that the restart's true
    // residual meets it (a cycle that ended just above it would cost a whole
    // restart), and stops a cycle after a fixed reduction; plain GMRES stops
    // at the target
    s.inner = A.inner_margin();
    s.red = sp->inner_reduction > 0 ? sp->inner_reduction : sp->inner_reduction < 0 ? 0.0 : A.inner_reduction();
    s.H = cv.take<double2>((size_t)nrhs * (m + 1) * m);
    s.cs = cv.take<double>((size_t)nrhs * m);
    s.sn = cv.take<double2>((size_t)nrhs * m);
    s.y = cv.take<double2>((size_t)nrhs * m);
    s.g = cv.take<double2>((size_t)nrhs * (m + 1));
    s.hcol = cv.take<double2>((size_t)nrhs * (m + 1));
    const int pb = std::max(nblk, (n + VCHUNK - 1) / VCHUNK);
    double2* partial = cv.take<double2>((size_t)nrhs * (m + 1) * pb);
    double2* pnorm = cv.take<double2>((size_t)nrhs * pb);
    s.bnorm = cv.take<double>(5 * (size_t)nrhs);
    s.scale = s.bnorm + nrhs;
    s.est = s.scale + nrhs;
    s.true_res = s.est + nrhs;
    s.wmax = s.true_res + nrhs;
    s.jlen = cv.take<int>(2 * (size_t)nrhs);
    s.active = s.jlen + nrhs;
    s.counters = cv.take<int>(4);

    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    EMFA_CUDA(c, cudaMemsetAsync(X, 0, sizeof(double2) * vec, st));
    int max_cycles = sp->max_iter > 0 ? (sp->max_iter + m - 1) / m : 100;
    if (prec == EMFA_F32 && sp->max_refine > 0) max_cycles = std::min(max_cycles, sp->max_refine);
    int total_iters = 0, cycles = 0, converged = 0;
    int host_cnt[4];
    // Arnoldi steps are checked one step late: step j and the operator
    // application for step j + 1 are queued before the host reads step j-1's
    // count of active right-hand sides (a page-locked word behind an event),
    // so the device never waits for the host between steps.  The step queued
    // after the last active one does nothing for converged right-hand sides
    // (k_arnoldi_finish skips them).
    struct StepEvents {
        cudaEvent_t e[2] = {nullptr, nullptr};     // the host's copy of a step's count has landed
        cudaEvent_t done[2] = {nullptr, nullptr};  // a step's kernels have finished (main stream)
        cudaStream_t side = nullptr;               // the copies
        ~StepEvents()
        {
            if (side) {
                cudaStreamSynchronize(side);
                cudaStreamDestroy(side);
            }
            for (auto x : e)
                if (x) cudaEventDestroy(x);
            for (auto x : done)
                if (x) cudaEventDestroy(x);
        }
    } sev;
    for (auto& x : sev.e) EMFA_CUDA(c, cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    for (auto& x : sev.done) EMFA_CUDA(c, cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    EMFA_CUDA(c, cudaStreamCreateWithFlags(&sev.side, cudaStreamNonBlocking));
    volatile int* slot = c->pinned;
    for (int cyc = 0; cyc < max_cycles; ++cyc) {
        // true residual R = B - Z X (X = 0 on the first cycle: R = B)
        if (cyc == 0) {
            if (prec == EMFA_F64)
                EMFA_CUDA(c, cudaMemcpyAsync(R, B, sizeof(double2) * vec, cudaMemcpyDeviceToDevice, st));
            else
                k_to_f64<<<grid1(vec), 256, 0, st>>>((const float2*)B, R, vec);
        } else {
            EMFA_TRY(A.residual(c, X, B, R, nrhs, Xt, st));
        }
        k_norm2<std::is_same<T, float>::value><<<dim3(nblk, nrhs), KB, 0, st>>>(R, n, nblk, chunk, pnorm);
        EMFA_CUDA(c, cudaMemsetAsync(s.counters, 0, sizeof(int) * 4, st));
        k_cycle_init<<<(nrhs + 127) / 128, 128, 0, st>>>(s, pnorm, nblk, cyc == 0);
        EMFA_CUDA(c, cudaMemcpyAsync(host_cnt, s.counters, sizeof(int) * 4, cudaMemcpyDeviceToHost, st));
        EMFA_CUDA(c, cudaStreamSynchronize(st));
        c->kernel_launches += 3;
        converged = host_cnt[1];
        if (host_cnt[0] == 0) break;
        ++cycles;
        // V0 = R / beta (on the FP16 basis: through W into plane 0, packed as
        // the product packs its input)
        const HPack p0{Bh, inv_tb, pk0.ldh, nullptr};
        k_scale_store<Cx<T>, double2><<<dim3((n + 1023) / 1024, nrhs), 256, 0, st>>>(R, s.scale, n, nrhs,
                                                                                     hbasis ? W : V);
        if (hbasis) EMFA_TRY(A.pack(c, W, p0, nrhs, st));
        int steps = 0;
        for (int j = 0; j < m; ++j) {
            // W = A V_j (for j > 0 done by normalize_apply at the end of the previous step)
            if (j == 0) EMFA_TRY(hbasis ? A.apply_packed(c, p0, W, nrhs, st) : A.apply(c, V, W, nrhs, st));
            // CGS1: h = V^H W; W -= V h with |W|^2.  CGS2 repeats the pair
            // (h2 = V^H W; W -= V h2) and H gets h + h2.
            const dim3 vg(vblk, nrhs);
            const int nv = j + 1;
            s.step_cnt = s.counters + 2 + (j & 1);
            HPack pk;
            bool packs = false;
            // the step normalises V_{j+1} itself (fused, or separate passes
            // ending in k_finish_pack); otherwise normalize_apply does
            const bool normalises = fused || finish_pack;
            if (normalises) {
                packs = A.pack_target(c, nrhs, &pk);
                if (!packs) pk = HPack{};
                if (hbasis) {  // V_{j+1} is plane j + 1
                    pk.bh = Bh + (size_t)(j + 1) * hplane;
                    pk.inv_t = inv_tb + (size_t)(j + 1) * nrhs;
                }
                // the next product skips itself if this step leaves nothing active
                pk.skip = s.step_cnt;
            }
            if (fused) {
                // V_{j+1} and the next product's operand come out of the step
                EMFA_CUDA(c, cudaMemsetAsync(s.step_cnt, 0, sizeof(int), st));
                EMFA_TRY(launch_arnoldi_step(c, sh, nrhs, st, s, j, (const float2*)V, vec, (const float2*)W, n,
                                             (float2*)(V + (size_t)(j + 1) * vec), pk));
                c->kernel_launches += 1;
            } else {
                // the updates sum the dots' block partials themselves (block 0
                // keeps the coefficients in s.hcol / s.y for the Arnoldi finish)
                const size_t hsm = 2 * nv * sizeof(typename Acc<T>::type);
                if (finish_pack) {
                    // product -> coefficients -> update -> finish: each launch may
                    // be resident before its predecessor ends (griddep_wait); the
                    // coefficients pass zeroes the step's active count
                    // the pair kernels by the parity of N (odd N: 8-byte W accesses)
                    const auto finish = n % 2 ? k_finish_pack<true> : k_finish_pack<false>;
                    const dim3 fg((n + FP_CHUNK - 1) / FP_CHUNK, nrhs);
                    if (hbasis) {
                        const auto dots = n % 2 ? k_vdots_hw<true> : k_vdots_hw<false>;
                        const auto upd = n % 2 ? k_vupdate_h<true> : k_vupdate_h<false>;
                        EMFA_CUDA(c, launch_dependent(dots, vg, dim3(256), 0, st, (const __half*)Bh, hplane, pk0.ldh,
                                                      (const float*)inv_tb, nv, (const float2*)W, n, nrhs, vblk,
                                                      partial, s.step_cnt, (const int*)s.active));
                        EMFA_CUDA(c, launch_dependent(upd, vg, dim3(256), 2 * nv * sizeof(float), st,
                                                      (const __half*)Bh, hplane, pk0.ldh, (const float*)inv_tb, nv,
                                                      s.hcol, (const double2*)partial, (float2*)W, n, nrhs, vblk,
                                                      pnorm, (const int*)s.active));
                        EMFA_CUDA(c, launch_dependent(finish, fg, dim3(256), 0, st, s, j, (const double2*)pnorm, vblk,
                                                      (const float2*)W, n, (float2*)nullptr, pk));
                    } else {
                        EMFA_CUDA(c, launch_dependent(k_vdots<T>, vg, dim3(256), 0, st, (const Cx<T>*)V, vec, nv,
                                                      (const Cx<T>*)W, n, nrhs, vblk, partial, s.step_cnt,
                                                      (const int*)s.active));
                        EMFA_CUDA(c, launch_dependent(k_vupdate<T, true>, vg, dim3(256), hsm, st, (const Cx<T>*)V, vec,
                                                      nv, s.hcol, (const double2*)partial, W, n, nrhs, vblk, pnorm,
                                                      (const int*)s.active));
                        EMFA_CUDA(c, launch_dependent(finish, fg, dim3(256), 0, st, s, j, (const double2*)pnorm, vblk,
                                                      (const float2*)W, n, (float2*)(V + (size_t)(j + 1) * vec), pk));
                    }
                    c->kernel_launches += 3;
                } else {
                k_vdots<T><<<vg, 256, 0, st>>>(V, vec, nv, W, n, nrhs, vblk, partial, nullptr, s.active);
                if (two_pass) {
                    k_vupdate<T, false><<<vg, 256, hsm, st>>>(V, vec, nv, s.hcol, partial, W, n, nrhs, vblk, pnorm,
                                                              s.active);
                    k_vdots<T><<<vg, 256, 0, st>>>(V, vec, nv, W, n, nrhs, vblk, partial, nullptr, s.active);
                    k_vupdate<T, true><<<vg, 256, hsm, st>>>(V, vec, nv, s.y, partial, W, n, nrhs, vblk, pnorm,
                                                             s.active);
                    c->kernel_launches += 2;
                } else {
                    k_vupdate<T, true><<<vg, 256, hsm, st>>>(V, vec, nv, s.hcol, partial, W, n, nrhs, vblk, pnorm,
                                                             s.active);
                }
                EMFA_CUDA(c, cudaMemsetAsync(s.step_cnt, 0, sizeof(int), st));
                if (m <= 32)
                    k_arnoldi_finish_warp<<<(nrhs * 32 + 127) / 128, 128, 0, st>>>(s, j, pnorm, vblk, two_pass ? 1 : 0);
                else
                    k_arnoldi_finish<<<(nrhs * 32 + 127) / 128, 128, 0, st>>>(s, j, pnorm, vblk, two_pass ? 1 : 0);
                c->kernel_launches += 3;
                }
            }
            // the host reads the step's count on a side stream, so no copy sits
            // between this step's last kernel and the next product
            EMFA_CUDA(c, cudaEventRecord(sev.done[j & 1], st));
            EMFA_CUDA(c, cudaStreamWaitEvent(sev.side, sev.done[j & 1], 0));
            EMFA_CUDA(c, cudaMemcpyAsync((void*)(slot + (j & 1)), s.step_cnt, sizeof(int), cudaMemcpyDeviceToHost,
                                         sev.side));
            EMFA_CUDA(c, cudaEventRecord(sev.e[j & 1], sev.side));
            ++steps;
            if (j > 0) {
                EMFA_CUDA(c, cudaEventSynchronize(sev.e[(j - 1) & 1]));
                if (slot[(j - 1) & 1] == 0) {  // step j (queued) found nothing active
                    --steps;
                    break;
                }
            }
            if (j + 1 == m) break;
            // V_{j+1} = W / beta, then W = A V_{j+1} (one pass for operators that
            // pack; the fused step has normalised and packed already)
            if (normalises && packs)
                EMFA_TRY(A.apply_packed(c, pk, W, nrhs, st));
            else if (normalises)
                EMFA_TRY(A.apply(c, V + (size_t)(j + 1) * vec, W, nrhs, st));
            else
                EMFA_TRY(A.normalize_apply(c, W, s.scale, s.wmax, V + (size_t)(j + 1) * vec, W, nrhs, st));
        }
        total_iters += steps;
        if (std::is_same<T, float>::value && m <= 32)
            k_backsolve_f32<<<(nrhs + BS_WARPS - 1) / BS_WARPS, 32 * BS_WARPS, 0, st>>>(s);
        else
            k_backsolve<<<(nrhs * 32 + 127) / 128, 128, 0, st>>>(s);
        if (hbasis)
            (n % 2 ? k_update_x2_h<true> : k_update_x2_h<false>)<<<dim3(((n + 1) / 2 + 255) / 256, nrhs), 256,
                                                                    2 * std::max(1, steps) * sizeof(float), st>>>(
                Bh, hplane, pk0.ldh, inv_tb, steps, s.y, s.jlen, X, n, nrhs);
        else
            k_update_x2<T><<<dim3((n + 255) / 256, nrhs), 256,
                             2 * std::max(1, steps) * sizeof(typename Acc<T>::type), st>>>(V, vec, steps, s.y, s.jlen,
                                                                                            X, n, nrhs);
        c->kernel_launches += 2;
        EMFA_CUDA(c, cudaGetLastError());
    }
    EMFA_CUDA(c, cudaGetLastError());
    // the operator's device-side error word (a timed-out wait) once, after the
    // last cycle: the word is sticky, and a check per cycle cost a host
    // synchronisation in the middle of the device's queue
    EMFA_TRY(A.check(c, st));
    cudaEventRecord(e1, st);
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::vector<double> tr(nrhs);
    EMFA_CUDA(c, cudaMemcpy(tr.data(), s.true_res, sizeof(double) * nrhs, cudaMemcpyDeviceToHost));
    if (info) {
        info->iterations = total_iters;
        info->cycles = cycles;
        info->converged = converged;
        info->max_rel_residual = *std::max_element(tr.begin(), tr.end());
        info->seconds = ms * 1e-3;
    }
    return converged == nrhs ? EMFA_OK : EMFA_ERR_NOT_CONVERGED;
}


// ---------------------------------------------------------------------------
// BiCGStab, FP64 vectors, reference update order (iml.cpp:3-39)
// ---------------------------------------------------------------------------
struct BicgDev {
    int nrhs;
    double tol;
    double2 *rho0, *rho1, *alpha, *omega, *beta;
    double* bnorm;
    double* res;
    int* active;
    int* counters;
};

__device__ __forceinline__ double2 cdiv(double2 a, double2 b)
{
    double d = b.x * b.x + b.y * b.y;
    if (d == 0.0) return make_double2(0.0, 0.0);
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double2 cmuld(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

// p = r + beta (p - omega v)     (active RHS only)
__global__ void k_bicg_p(BicgDev s, const double2* __restrict__ r, double2* __restrict__ p, const double2* __restrict__ v, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x, q = blockIdx.y;
    if (k >= n || !s.active[q]) return;
    size_t o = (size_t)q * n + k;
    double2 b = s.beta[q], w = s.omega[q];
    double2 t = make_double2(p[o].x - (w.x * v[o].x - w.y * v[o].y), p[o].y - (w.x * v[o].y + w.y * v[o].x));
    double2 bt = cmuld(b, t);
    p[o] = make_double2(r[o].x + bt.x, r[o].y + bt.y);
}

// x += alpha p ; s = r - alpha v
__global__ void k_bicg_s(BicgDev s, double2* __restrict__ x, const double2* __restrict__ p, const double2* __restrict__ r,
                         const double2* __restrict__ v, double2* __restrict__ sv, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x, q = blockIdx.y;
    if (k >= n || !s.active[q]) return;
    size_t o = (size_t)q * n + k;
    double2 a = s.alpha[q];
    double2 ap = cmuld(a, p[o]), av = cmuld(a, v[o]);
    x[o] = make_double2(x[o].x + ap.x, x[o].y + ap.y);
    sv[o] = make_double2(r[o].x - av.x, r[o].y - av.y);
}

// x += omega s ; r = s - omega t
__global__ void k_bicg_r(BicgDev s, double2* __restrict__ x, const double2* __restrict__ sv, const double2* __restrict__ t,
                         double2* __restrict__ r, int n)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x, q = blockIdx.y;
    if (k >= n || !s.active[q]) return;
    size_t o = (size_t)q * n + k;
    double2 w = s.omega[q];
    double2 ws = cmuld(w, sv[o]), wt = cmuld(w, t[o]);
    x[o] = make_double2(x[o].x + ws.x, x[o].y + ws.y);
    r[o] = make_double2(sv[o].x - wt.x, sv[o].y - wt.y);
}

// scalar stages; d holds the reduced dot products of the stage
__global__ void k_bicg_scalar(BicgDev s, int stage, const double2* __restrict__ d0, const double2* __restrict__ d1)
{
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= s.nrhs) return;
    if (stage == 0) {  // init: bnorm = ||b||, rho0 = alpha = omega = 1
        s.bnorm[q] = sqrt(d0[q].x);
        s.rho0[q] = s.alpha[q] = s.omega[q] = make_double2(1.0, 0.0);
        s.active[q] = s.bnorm[q] > 0.0;
        s.res[q] = s.bnorm[q] > 0.0 ? 1.0 : 0.0;
        return;
    }
    if (!s.active[q]) return;
    if (stage == 1) {  // rho1 = <rhat, r>; beta = (rho1/rho0)(alpha/omega)
        s.rho1[q] = d0[q];
        s.beta[q] = cmuld(cdiv(d0[q], s.rho0[q]), cdiv(s.alpha[q], s.omega[q]));
    } else if (stage == 2) {  // alpha = rho1 / <rhat, v>
        s.alpha[q] = cdiv(s.rho1[q], d0[q]);
    } else if (stage == 3) {  // ||s|| / ||b|| test
        double res = sqrt(d0[q].x) / s.bnorm[q];
        s.res[q] = res;
        if (res < s.tol) {
            s.active[q] = 0;
            atomicAdd(s.counters + 1, 1);
        }
    } else if (stage == 4) {  // omega = <t, s> / <t, t>; rho0 = rho1
        s.omega[q] = cdiv(d0[q], d1[q]);
        s.rho0[q] = s.rho1[q];
        atomicAdd(s.counters, 1);
    }
}

static emfa_status_t matvec_d(Ctx* c, LinOp& A, const double2* X, int nrhs, double2* Y, float2* tmp_in,
                              float2* tmp_out, cudaStream_t st)
{
    size_t vec = (size_t)A.n * nrhs;
    if (A.prec == EMFA_F64) return A.apply(c, X, Y, nrhs, st);
    k_to_f32<<<grid1(vec), 256, 0, st>>>(X, tmp_in, vec);
    EMFA_TRY(A.apply(c, tmp_in, tmp_out, nrhs, st));
    k_to_f64<<<grid1(vec), 256, 0, st>>>(tmp_out, Y, vec);
    c->kernel_launches += 2;
    return EMFA_OK;
}

static emfa_status_t dots_d(Ctx* c, const double2* A, const double2* B, int n, int nrhs, double2* partial, double2* out,
                            cudaStream_t st)
{
    int nblk = dot_blocks(n);
    k_block_dots<double2, double2><<<dim3(nblk, nrhs), KB, 0, st>>>(A, 0, 1, B, n, nrhs, nblk, partial);
    k_reduce_partials<<<(nrhs + 127) / 128, 128, 0, st>>>(partial, 1, nrhs, nblk, out, 0);
    c->kernel_launches += 2;
    return EMFA_OK;
}

static emfa_status_t bicgstab(Ctx* c, LinOp& A, const void* B, int nrhs, double2* X, const emfa_solver_params_t* sp,
                              emfa_solve_info_t* info, cudaStream_t st)
{
    const int n = A.n, prec = A.prec;
    const size_t vec = (size_t)n * nrhs;
    const int nblk = dot_blocks(n);
    DevBuf vb, tin, tout, sc, pb, db;
    EMFA_TRY(vb.alloc(c, sizeof(double2) * vec * 6));  // r, rhat, p, v, s, t
    if (prec == EMFA_F32) {
        EMFA_TRY(tin.alloc(c, sizeof(float2) * vec));
        EMFA_TRY(tout.alloc(c, sizeof(float2) * vec));
    }
    EMFA_TRY(sc.alloc(c, sizeof(double2) * 5 * nrhs + sizeof(double) * 2 * nrhs + sizeof(int) * (nrhs + 4)));
    EMFA_TRY(pb.alloc(c, sizeof(double2) * (size_t)nrhs * nblk));
    EMFA_TRY(db.alloc(c, sizeof(double2) * 2 * nrhs));
    double2* partial = dptr<double2>(pb);
    double2* r = dptr<double2>(vb);
    double2* rh = r + vec;
    double2* p = rh + vec;
    double2* v = p + vec;
    double2* sv = v + vec;
    double2* t = sv + vec;
    BicgDev s;
    s.nrhs = nrhs;
    s.tol = sp->tol;
    s.rho0 = dptr<double2>(sc);
    s.rho1 = s.rho0 + nrhs;
    s.alpha = s.rho1 + nrhs;
    s.omega = s.alpha + nrhs;
    s.beta = s.omega + nrhs;
    s.bnorm = reinterpret_cast<double*>(s.beta + nrhs);
    s.res = s.bnorm + nrhs;
    s.active = reinterpret_cast<int*>(s.res + nrhs);
    s.counters = s.active + nrhs;
    double2* d0 = dptr<double2>(db);
    double2* d1 = d0 + nrhs;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    EMFA_CUDA(c, cudaMemsetAsync(X, 0, sizeof(double2) * vec, st));
    if (prec == EMFA_F64)
        EMFA_CUDA(c, cudaMemcpyAsync(r, B, sizeof(double2) * vec, cudaMemcpyDeviceToDevice, st));
    else
        k_to_f64<<<grid1(vec), 256, 0, st>>>((const float2*)B, r, vec);
    EMFA_CUDA(c, cudaMemcpyAsync(rh, r, sizeof(double2) * vec, cudaMemcpyDeviceToDevice, st));
    EMFA_CUDA(c, cudaMemsetAsync(p, 0, sizeof(double2) * vec * 2, st));  // p, v
    EMFA_TRY(dots_d(c, r, r, n, nrhs, partial, d0, st));
    k_bicg_scalar<<<(nrhs + 127) / 128, 128, 0, st>>>(s, 0, d0, nullptr);
    EMFA_CUDA(c, cudaMemsetAsync(s.counters, 0, sizeof(int) * 4, st));
    const int max_it = sp->max_iter > 0 ? sp->max_iter : 500;
    dim3 eg((n + 255) / 256, nrhs);
    int it = 0, hc[4] = {0, 0, 0, 0};
    int converged = 0;
    for (; it < max_it; ++it) {
        EMFA_TRY(dots_d(c, rh, r, n, nrhs, partial, d0, st));
        k_bicg_scalar<<<(nrhs + 127) / 128, 128, 0, st>>>(s, 1, d0, nullptr);
        k_bicg_p<<<eg, 256, 0, st>>>(s, r, p, v, n);
        EMFA_TRY(matvec_d(c, A, p, nrhs, v, dptr<float2>(tin), dptr<float2>(tout), st));
        EMFA_TRY(dots_d(c, rh, v, n, nrhs, partial, d0, st));
        k_bicg_scalar<<<(nrhs + 127) / 128, 128, 0, st>>>(s, 2, d0, nullptr);
        k_bicg_s<<<eg, 256, 0, st>>>(s, X, p, r, v, sv, n);
        EMFA_TRY(dots_d(c, sv, sv, n, nrhs, partial, d0, st));
        k_bicg_scalar<<<(nrhs + 127) / 128, 128, 0, st>>>(s, 3, d0, nullptr);
        EMFA_TRY(matvec_d(c, A, sv, nrhs, t, dptr<float2>(tin), dptr<float2>(tout), st));
        EMFA_TRY(dots_d(c, t, sv, n, nrhs, partial, d0, st));
        EMFA_TRY(dots_d(c, t, t, n, nrhs, partial, d1, st));
        EMFA_CUDA(c, cudaMemsetAsync(s.counters, 0, sizeof(int), st));
        k_bicg_scalar<<<(nrhs + 127) / 128, 128, 0, st>>>(s, 4, d0, d1);
        k_bicg_r<<<eg, 256, 0, st>>>(s, X, sv, t, r, n);
        c->kernel_launches += 8;
        EMFA_CUDA(c, cudaMemcpyAsync(hc, s.counters, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
        EMFA_CUDA(c, cudaStreamSynchronize(st));
        converged = hc[1];
        if (hc[0] == 0) {
            ++it;
            break;
        }
    }
    cudaEventRecord(e1, st);
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::vector<double> res(nrhs);
    EMFA_CUDA(c, cudaMemcpy(res.data(), s.res, sizeof(double) * nrhs, cudaMemcpyDeviceToHost));
    if (info) {
        info->iterations = it;
        info->cycles = 1;
        info->converged = converged;
        info->max_rel_residual = *std::max_element(res.begin(), res.end());
        info->seconds = ms * 1e-3;
    }
    return converged == nrhs ? EMFA_OK : EMFA_ERR_NOT_CONVERGED;
}

__global__ void k_add_c128(double2* __restrict__ X, const double2* __restrict__ D, size_t tot)
{
    size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id < tot) X[id] = make_double2(X[id].x + D[id].x, X[id].y + D[id].y);
}

// out[r] = ||R_r|| / ||B_r|| with B2 holding ||B_r||^2 in .x: CTA per RHS
// (256 threads), FP64 sums
__global__ void __launch_bounds__(256) k_norm_ratio(const double2* __restrict__ R, const double2* __restrict__ B2,
                                                    int n, int nrhs, double* __restrict__ out)
{
    __shared__ double ws[8];
    const int r = blockIdx.x;
    double s = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double2 v = R[(size_t)r * n + k];
        s += v.x * v.x + v.y * v.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < 8; ++w) t += ws[w];
        out[r] = B2[r].x > 0 ? sqrt(t / B2[r].x) : 0.0;
    }
}

// BiCGStab with FP32 products: the recursively updated residual drifts from
// the true one, so each pass solves for a correction A d = b - A x from the
// true FP64 residual (iterative refinement), until the true residual meets
// the tolerance.  The reference's FP32 BiCGStab stops on the recursive one.
static emfa_status_t bicgstab_refined(Ctx* c, LinOp& A, const void* B, int nrhs, double2* X,
                                      const emfa_solver_params_t* sp, emfa_solve_info_t* info, cudaStream_t st)
{
    const size_t vec = (size_t)A.n * nrhs;
    DevBuf rb, xt, db, bb, nb, rr;
    EMFA_TRY(rb.alloc(c, sizeof(double2) * vec));
    EMFA_TRY(xt.alloc(c, sizeof(float2) * vec));
    EMFA_TRY(db.alloc(c, sizeof(double2) * vec));
    EMFA_TRY(bb.alloc(c, sizeof(float2) * vec));
    EMFA_TRY(nb.alloc(c, sizeof(double2) * nrhs));
    EMFA_TRY(rr.alloc(c, sizeof(double) * nrhs));
    // ||b||^2
    k_to_f64<<<grid1(vec), 256, 0, st>>>((const float2*)B, dptr<double2>(rb), vec);
    EMFA_TRY(dots_d(c, dptr<double2>(rb), dptr<double2>(rb), A.n, nrhs, dptr<double2>(db), dptr<double2>(nb), st));
    emfa_status_t s = bicgstab(c, A, B, nrhs, X, sp, info, st);
    if (s != EMFA_OK && s != EMFA_ERR_NOT_CONVERGED) return s;
    const int passes = sp->max_refine > 0 ? sp->max_refine : 4;
    int iters = info ? info->iterations : 0;
    std::vector<double> rel(nrhs);
    for (int pass = 0; pass < passes; ++pass) {
        EMFA_TRY(A.residual(c, X, B, dptr<double2>(rb), nrhs, dptr<float2>(xt), st));
        k_norm_ratio<<<nrhs, 256, 0, st>>>(dptr<double2>(rb), dptr<double2>(nb), A.n, nrhs,
                                                         dptr<double>(rr));
        EMFA_CUDA(c, cudaMemcpyAsync(rel.data(), rr.ptr, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st));
        EMFA_CUDA(c, cudaStreamSynchronize(st));
        c->kernel_launches += 1;
        double worst = *std::max_element(rel.begin(), rel.end());
        if (info) info->max_rel_residual = worst;
        if (worst < sp->tol) {
            if (info) {
                info->converged = nrhs;
                info->iterations = iters;
                info->cycles = pass + 1;
            }
            return EMFA_OK;
        }
        // correction: A d = r (FP32 right-hand side), x += d
        k_to_f32<<<grid1(vec), 256, 0, st>>>(dptr<double2>(rb), dptr<float2>(bb), vec);
        emfa_solver_params_t sp2 = *sp;
        sp2.tol = sp->tol / std::max(worst, 1e-30);  // relative to the correction's right-hand side
        if (sp2.tol > 0.5) sp2.tol = 0.5;
        emfa_solve_info_t in2{};
        s = bicgstab(c, A, dptr<float2>(bb), nrhs, dptr<double2>(db), &sp2, &in2, st);
        if (s != EMFA_OK && s != EMFA_ERR_NOT_CONVERGED) return s;
        iters += in2.iterations;
        k_add_c128<<<grid1(vec), 256, 0, st>>>(X, dptr<double2>(db), vec);
        c->kernel_launches += 2;
    }
    if (info) {
        info->iterations = iters;
        info->cycles = passes + 1;
        info->converged = 0;
        for (double v : rel)
            if (v < sp->tol) info->converged++;
    }
    return EMFA_ERR_NOT_CONVERGED;
}

emfa_status_t solve_op(Ctx* c, LinOp& A, const void* B, int nrhs, void* X, const emfa_solver_params_t* sp,
                       emfa_solve_info_t* info, cudaStream_t st)
{
    if (sp->method == EMFA_BICGSTAB) {
        // the reference's FP32 BiCGStab (1e-2 / 1e-3 tolerances) stops on the
        // recursive residual; tighter tolerances get true-residual refinement
        if (A.prec == EMFA_F32 && sp->tol < 1e-4) return bicgstab_refined(c, A, B, nrhs, (double2*)X, sp, info, st);
        return bicgstab(c, A, B, nrhs, (double2*)X, sp, info, st);
    }
    if (A.prec == EMFA_F64) return gmres_t<double>(c, A, B, nrhs, (double2*)X, sp, info, st);
    return gmres_t<float>(c, A, B, nrhs, (double2*)X, sp, info, st);
}

emfa_status_t LinOp::normalize_apply(Ctx* c, const void* W, const double* scale, const double*, void* Vout,
                                     void* Y, int nrhs, cudaStream_t st)
{
    const size_t vec = (size_t)n * nrhs;
    if (prec == EMFA_F64)
        k_scale_store<Cx<double>, Cx<double>><<<dim3((n + 1023) / 1024, nrhs), 256, 0, st>>>((const Cx<double>*)W, scale, n, nrhs,
                                                                           (Cx<double>*)Vout);
    else
        k_scale_store<Cx<float>, Cx<float>><<<dim3((n + 1023) / 1024, nrhs), 256, 0, st>>>((const Cx<float>*)W, scale, n, nrhs,
                                                                         (Cx<float>*)Vout);
    c->kernel_launches += 1;
    return apply(c, Vout, Y, nrhs, st);
}

// Dense impedance matrix as a Krylov operator.  Mixed path: inner products
// on the tensor cores (split FP16 or TF32) or FP32 CUDA cores; refinement
// residual from the three-term split-FP16 product (F16X) or FP32 products
// with FP64 chunk sums.  Plain path: FP64 throughout.
// Measured on the 7,680-unknown CFIE job (360 right-hand sides, GMRES(30),
// tolerance 1e-6): inner reduction per cycle 1e-2 -> 47 iterations in 3
// cycles, 16.3 ms; 5e-3 -> 49 / 3; 1e-3 -> 50 / 3; 1e-4 -> 52 / 2; none ->
// 53 / 2, 18.6 ms.  A restart from the true residual gains more than the
// residual (0.8 ms) costs, down to about 1e-2 per cycle.
constexpr double kInnerReduction = 1e-2;

struct DenseOp : LinOp {
    enum Mode { SIMT = 0, TF32 = 1, F16X = 2 };
    const void* Z = nullptr;
    int mode = SIMT;
    HPlanes hp;  // F16X: planes of Z, split by prepare()
    emfa_status_t prepare(Ctx* c, cudaStream_t st)
    {
        return mode == F16X ? hsplit_prepare(c, Z, n, n, &hp, st) : EMFA_OK;
    }
    // tensor-core inner products (FP16 significands or TF32) against an
    // FP32/FP64-accurate residual: half the target, and a restart from the
    // true residual after two digits per cycle
    double inner_margin() const override { return prec == EMFA_F32 && mode != SIMT ? 0.5 : 1.0; }
    double inner_reduction() const override { return prec == EMFA_F32 && mode != SIMT ? kInnerReduction : 0.0; }
    emfa_status_t apply(Ctx* c, const void* X, void* Y, int nrhs, cudaStream_t st) override
    {
        if (prec == EMFA_F64) return cgemm_f64(c, Z, n, X, n, nrhs, Y, st);
        if (mode == F16X) return hgemm_apply(c, hp, X, Y, nrhs, st);
        if (mode == TF32) return cgemm_tf32(c, Z, n, X, n, nrhs, Y, st);
        return cgemm_f32(c, Z, n, X, n, nrhs, Y, st);
    }
    emfa_status_t residual(Ctx* c, const double2* X, const void* B, double2* R, int nrhs, float2* xt,
                           cudaStream_t st) override
    {
        const size_t vec = (size_t)n * nrhs;
        if (prec == EMFA_F32 && mode == F16X) return hgemm_residual(c, hp, X, B, true, R, nrhs, st);
        if (prec == EMFA_F64) {
            EMFA_TRY(cgemm_f64(c, Z, n, X, n, nrhs, R, st));  // R = Z X
            k_residual<double2><<<grid1(vec), 256, 0, st>>>((const double2*)B, R, R, vec);
            c->kernel_launches += 1;
            return EMFA_OK;
        }
        k_to_f32<<<grid1(vec), 256, 0, st>>>(X, xt, vec);
        c->kernel_launches += 1;
        return cgemm_f32_chunked(c, Z, n, xt, n, nrhs, B, R, st);  // R = B - Z X
    }
    emfa_status_t normalize_apply(Ctx* c, const void* W, const double* scale, const double* wmax, void* Vout,
                                  void* Y, int nrhs, cudaStream_t st) override
    {
        if (prec == EMFA_F32 && mode == F16X && wmax)
            return hgemm_normalize_apply(c, hp, W, scale, wmax, Vout, Y, nrhs, st);
        return LinOp::normalize_apply(c, W, scale, wmax, Vout, Y, nrhs, st);
    }
    bool pack_target(Ctx* c, int nrhs, HPack* p) override
    {
        return prec == EMFA_F32 && mode == F16X && hgemm_pack_target(c, hp, nrhs, p) == EMFA_OK;
    }
    emfa_status_t apply_packed(Ctx* c, const HPack& p, void* Y, int nrhs, cudaStream_t st) override
    {
        return hgemm_apply_packed(c, hp, p, Y, nrhs, st);
    }
    emfa_status_t pack(Ctx* c, const void* X, const HPack& p, int nrhs, cudaStream_t st) override
    {
        if (!(prec == EMFA_F32 && mode == F16X)) return EMFA_ERR_UNSUPPORTED;
        return hgemm_pack(c, hp, X, p, nrhs, st);
    }
    emfa_status_t check(Ctx* c, cudaStream_t st) override
    {
        if (mode == F16X) return hgemm_check_error(c, st);
        return mode == TF32 ? gemm_check_error(c, st) : EMFA_OK;
    }
};

__global__ void k_add_f32_c128(double2* __restrict__ X, const float2* __restrict__ D, size_t tot)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
        const float2 d = D[i];
        X[i].x += (double)d.x;
        X[i].y += (double)d.y;
    }
}

// Dense solve by LU with FP64 iterative refinement (EMFA_LU): factor Z once in
// FP32 (lu.cu), x = (LU)^-1 b, then per pass the true residual r = b - Z x
// from the operator's refinement residual (FP64-accurate) and x += (LU)^-1 r,
// until every right-hand side meets the tolerance.  A zero pivot, or a pass
// that fails to halve the worst residual, hands the remaining correction to
// GMRES-IR on the same operator.
static emfa_status_t lu_refined(Ctx* c, LinOp& A, const void* Z, const void* B, int nrhs, double2* X,
                                const emfa_solver_params_t* sp, emfa_solve_info_t* info, cudaStream_t st)
{
    const int n = A.n;
    const size_t vec = (size_t)n * nrhs;
    LuFactor F;
    EMFA_TRY(lu_factor(c, Z, n, F, st));
    int zero_pivot = 0;
    EMFA_TRY(lu_zero_pivot(c, F, &zero_pivot, st));
    DevBuf work, d32, r64, r32, db, nb, rr;
    EMFA_TRY(work.alloc(c, sizeof(float2) * 2 * vec));
    EMFA_TRY(d32.alloc(c, sizeof(float2) * vec));
    EMFA_TRY(r64.alloc(c, sizeof(double2) * vec));
    EMFA_TRY(r32.alloc(c, sizeof(float2) * vec));
    EMFA_TRY(db.alloc(c, sizeof(double2) * vec));
    EMFA_TRY(nb.alloc(c, sizeof(double2) * nrhs));
    EMFA_TRY(rr.alloc(c, sizeof(double) * nrhs));
    k_to_f64<<<grid1(vec), 256, 0, st>>>((const float2*)B, dptr<double2>(r64), vec);
    EMFA_TRY(dots_d(c, dptr<double2>(r64), dptr<double2>(r64), n, nrhs, dptr<double2>(db), dptr<double2>(nb), st));
    if (zero_pivot == 0) {
        EMFA_TRY(lu_apply(c, F, (const float2*)B, nrhs, dptr<float2>(d32), dptr<float2>(work), st));
        k_to_f64<<<grid1(vec), 256, 0, st>>>(dptr<float2>(d32), X, vec);
    } else {
        EMFA_CUDA(c, cudaMemsetAsync(X, 0, sizeof(double2) * vec, st));
    }
    c->kernel_launches += 2;
    const int passes = sp->max_refine > 0 ? sp->max_refine : 10;
    std::vector<double> rel(nrhs);
    double prev = 1e300, worst = 1e300;
    int pass = 0;
    for (;; ++pass) {
        EMFA_TRY(A.residual(c, X, B, dptr<double2>(r64), nrhs, dptr<float2>(r32), st));
        k_norm_ratio<<<nrhs, 256, 0, st>>>(dptr<double2>(r64), dptr<double2>(nb), n, nrhs,
                                                         dptr<double>(rr));
        EMFA_CUDA(c, cudaMemcpyAsync(rel.data(), rr.ptr, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st));
        EMFA_CUDA(c, cudaStreamSynchronize(st));
        c->kernel_launches += 1;
        worst = *std::max_element(rel.begin(), rel.end());
        if (zero_pivot == 0) EMFA_TRY(lu_check_solves(c, F, st));
        if (worst < sp->tol) {
            if (info) {
                info->converged = nrhs;
                info->iterations = pass;
                info->cycles = pass + 1;
                info->max_rel_residual = worst;
            }
            return EMFA_OK;
        }
        if (zero_pivot != 0 || pass >= passes || !(worst < 0.5 * prev)) break;
        prev = worst;
        k_to_f32<<<grid1(vec), 256, 0, st>>>(dptr<double2>(r64), dptr<float2>(r32), vec);
        EMFA_TRY(lu_apply(c, F, dptr<float2>(r32), nrhs, dptr<float2>(d32), dptr<float2>(work), st));
        k_add_f32_c128<<<grid1(vec), 256, 0, st>>>(X, dptr<float2>(d32), vec);
        c->kernel_launches += 2;
    }
    // the factor did not carry the solve: GMRES-IR on the correction A d = r
    F.release();
    work.release();
    k_to_f32<<<grid1(vec), 256, 0, st>>>(dptr<double2>(r64), dptr<float2>(r32), vec);
    c->kernel_launches += 1;
    emfa_solver_params_t sp2 = *sp;
    sp2.method = EMFA_GMRES;
    sp2.tol = std::min(0.5, sp->tol / std::max(worst, 1e-30));
    emfa_solve_info_t in2{};
    emfa_status_t s = gmres_t<float>(c, A, dptr<float2>(r32), nrhs, dptr<double2>(db), &sp2, &in2, st);
    if (s != EMFA_OK && s != EMFA_ERR_NOT_CONVERGED) return s;
    k_add_c128<<<grid1(vec), 256, 0, st>>>(X, dptr<double2>(db), vec);
    EMFA_TRY(A.residual(c, X, B, dptr<double2>(r64), nrhs, dptr<float2>(r32), st));
    k_norm_ratio<<<nrhs, 256, 0, st>>>(dptr<double2>(r64), dptr<double2>(nb), n, nrhs, dptr<double>(rr));
    EMFA_CUDA(c, cudaMemcpyAsync(rel.data(), rr.ptr, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, st));
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    c->kernel_launches += 2;
    int conv = 0;
    for (double v : rel) conv += v < sp->tol;
    if (info) {
        info->iterations = pass + in2.iterations;
        info->cycles = pass + 1 + in2.cycles;
        info->converged = conv;
        info->max_rel_residual = *std::max_element(rel.begin(), rel.end());
    }
    return conv == nrhs ? EMFA_OK : EMFA_ERR_NOT_CONVERGED;
}

// matvec mode of the dense operator; TF32 needs even n and a 16-byte aligned Z
static int dense_mode(int prec, int matvec, const void* Z, int n)
{
    if (prec != EMFA_F32) return DenseOp::SIMT;
    if (matvec == EMFA_MV_AUTO || matvec == EMFA_MV_F16X) return DenseOp::F16X;
    if (matvec == EMFA_MV_TF32 && n % 2 == 0 && ((uintptr_t)Z & 15) == 0) return DenseOp::TF32;
    return DenseOp::SIMT;
}

emfa_status_t solve_dense(Ctx* c, int prec, const void* Z, int n, const void* B, int nrhs, void* X,
                          const emfa_solver_params_t* sp, emfa_solve_info_t* info, cudaStream_t st)
{
    DenseOp A;
    A.n = n;
    A.prec = prec;
    A.Z = Z;
    A.mode = dense_mode(prec, sp->matvec, Z, n);
    EMFA_TRY(A.prepare(c, st));
    if (sp->method == EMFA_LU) return lu_refined(c, A, Z, B, nrhs, (double2*)X, sp, info, st);
    return solve_op(c, A, B, nrhs, X, sp, info, st);
}
}  // namespace emfa

using namespace emfa;

extern "C" {

emfa_status_t emfa_autotune_query(int device, int n, int n_rhs, int* shape, float* ms)
{
    if (!shape || !ms || n <= 0 || n_rhs <= 0) {
        set_global_error("emfa_autotune_query: null output or non-positive size");
        return EMFA_ERR_INVALID;
    }
    return hgemm_tuned_shape(device, n, n_rhs, shape, ms);
}

emfa_status_t emfa_autotune_clear(void)
{
    hgemm_tune_clear();
    return EMFA_OK;
}

emfa_status_t emfa_matvec(emfa_ctx_t* ctx, int prec, int matvec, const void* Z_dev, int n, const void* X_dev, int n_rhs,
                          void* Y_dev, void* stream)
{
    if (!ctx || !Z_dev || !X_dev || !Y_dev || n <= 0 || n_rhs <= 0 || n_rhs > 65535) {
        set_error(ctx, "emfa_matvec: bad arguments");
        return EMFA_ERR_INVALID;
    }
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    if (prec == EMFA_F64) return cgemm_f64(ctx, Z_dev, n, X_dev, n, n_rhs, Y_dev, st);
    if (prec != EMFA_F32) {
        set_error(ctx, "emfa_matvec: precision");
        return EMFA_ERR_INVALID;
    }
    if (matvec == EMFA_MV_TF32) {
        EMFA_TRY(cgemm_tf32(ctx, Z_dev, n, X_dev, n, n_rhs, Y_dev, st));
        return gemm_check_error(ctx, st);
    }
    if (matvec == EMFA_MV_F16X) {
        HPlanes hp;
        EMFA_TRY(hsplit_prepare(ctx, Z_dev, n, n, &hp, st));
        EMFA_TRY(hgemm_apply(ctx, hp, X_dev, Y_dev, n_rhs, st));
        return hgemm_check_error(ctx, st);
    }
    return cgemm_f32(ctx, Z_dev, n, X_dev, n, n_rhs, Y_dev, st);
}

emfa_status_t emfa_residual(emfa_ctx_t* ctx, int prec, int matvec, const void* Z_dev, int n, const void* X_dev,
                            const void* B_dev, int n_rhs, void* R_dev, void* stream)
{
    if (!ctx || !Z_dev || !X_dev || !B_dev || !R_dev || n <= 0 || n_rhs <= 0 || n_rhs > 65535 ||
        (prec != EMFA_F32 && prec != EMFA_F64) || matvec < EMFA_MV_AUTO || matvec > EMFA_MV_F16X) {
        set_error(ctx, "emfa_residual: bad arguments");
        return EMFA_ERR_INVALID;
    }
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    DenseOp A;
    A.n = n;
    A.prec = prec;
    A.Z = Z_dev;
    A.mode = dense_mode(prec, matvec, Z_dev, n);
    EMFA_TRY(A.prepare(ctx, st));
    DevBuf xt;
    if (A.mode != DenseOp::F16X) EMFA_TRY(xt.alloc(ctx, sizeof(float2) * (size_t)n * n_rhs));
    EMFA_TRY(A.residual(ctx, (const double2*)X_dev, B_dev, (double2*)R_dev, n_rhs, dptr<float2>(xt), st));
    EMFA_TRY(A.check(ctx, st));
    EMFA_CUDA(ctx, cudaStreamSynchronize(st));
    return EMFA_OK;
}

emfa_status_t emfa_solve(emfa_ctx_t* ctx, int prec, const void* Z_dev, int n, const void* B_dev, int n_rhs,
                         void* X_dev, const emfa_solver_params_t* sp, emfa_solve_info_t* info, void* stream)
{
    if (!ctx || !Z_dev || !B_dev || !X_dev || !sp || n <= 0 || n_rhs <= 0 || n_rhs > 65535 ||
        (prec != EMFA_F32 && prec != EMFA_F64) || !(sp->tol > 0)) {
        set_error(ctx, "emfa_solve: bad arguments");
        return EMFA_ERR_INVALID;
    }
    if (sp->method != EMFA_GMRES && sp->method != EMFA_BICGSTAB && sp->method != EMFA_LU) {
        set_error(ctx, "emfa_solve: method must be EMFA_GMRES, EMFA_BICGSTAB or EMFA_LU");
        return EMFA_ERR_INVALID;
    }
    if (sp->method == EMFA_LU && prec != EMFA_F32) {
        set_error(ctx, "emfa_solve: EMFA_LU factors in FP32 and refines in FP64; it takes EMFA_F32 operands");
        return EMFA_ERR_UNSUPPORTED;
    }
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return solve_dense(ctx, prec, Z_dev, n, B_dev, n_rhs, X_dev, sp, info, st);
}

}  // extern "C"
