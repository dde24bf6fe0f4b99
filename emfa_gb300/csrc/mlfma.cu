// Multilevel fast multipole CFIE operator (EMSolver/MLFMA.cpp).
//
// Host (float arithmetic, the reference's own rules, so box order, multipole
// counts, sample points and stencils are the reference's):
//   bounding cube and level count   MLFMA_Boundary::init (MLFMA_Boundary.cpp:15-35)
//   octree, box order of unknowns   buildBox / buildFirstLevel / buildCurLevel (MLFMA.cpp:688-805)
//   near / far lists                setBoxParameter (MLFMA.cpp:807-866)
//   multipoles, Gauss-Legendre      getMultipoleNumber / levelRootsAndWeights (MLFMA.cpp:877-915)
//   3x3 Lagrange stencils           calculateInterpolationMtr / lagrangeIPWeights (MLFMA.cpp:917-1002)
// Device (FP32 patterns; level patterns in 3 Cartesian components as in the
// reference, the transverse radiation / receive patterns in 2, theta and phi
// of each sample's own basis):
//   k_trans_table  translation operators (parallelLevelTrans, MLFMA.cpp:1191-1222) in FP64, once
//                  per distinct box offset (at most 7^3 per level) instead of per box pair
//   k_radrec       radiation / receive patterns (MLFMA.cpp:1244-1292,1393-1422)
//   k_near_fill    near-field CFIE blocks per (field box, near box) (MLFMA.cpp:1004-1131)
//   per mat-vec (MLFMA.cpp:454-686), up to 8 right-hand sides per pass, level patterns planar:
//     k_agg_finest    finest-level aggregation
//     k_upward        interpolation + shift, child -> parent: the 3 x 3 Lagrange stencil as two
//                     1-D passes (theta into shared memory, then phi)
//     k_downward      translation from far boxes + anterpolation from the parent (transposed
//                     stencil as two 1-D passes), by chunks of phi rows
//     k_disagg_near   disaggregation at the finest level fused with the near-field product
#include "emfa_internal.cuh"
#include "emfa_math.cuh"
#include "fill_entry.cuh"
#include "gemm.cuh"

#include <algorithm>
#include <cmath>
#include <complex>

namespace emfa {

struct C3f {
    float2 x, y, z;
};
// a transverse pattern in the (theta, phi) basis of its sample direction
struct C2f {
    float2 t, p;
};

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 caddf(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cscalef(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ C3f c3zero() { return C3f{make_float2(0, 0), make_float2(0, 0), make_float2(0, 0)}; }
__device__ __forceinline__ void c3fma(C3f& acc, float2 s, const C3f& v)
{
    acc.x = caddf(acc.x, cmulf(s, v.x));
    acc.y = caddf(acc.y, cmulf(s, v.y));
    acc.z = caddf(acc.z, cmulf(s, v.z));
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace mh {

const float PI = 3.14159265358979323846f;

struct Box {
    float c[3];
    int parent = -1;
    int oct = 0;      // child index (x*2+y)*2+z within the parent
    int offset = 0;   // first unknown (box order)
    std::vector<int> unk;
    std::vector<int> child, near, far;
};

// Legendre value / derivative recurrence of GaussLegendre::Evaluation
static void gl_eval(float x, int n, float& v, float& d)
{
    float vsub1 = x, vsub2 = 1;
    float f = 1 / (x * x - 1);
    v = 1;
    d = 0;
    for (int i = 2; i <= n; ++i) {
        v = ((2 * i - 1) * x * vsub1 - (i - 1) * vsub2) / i;
        d = i * f * (x * v - vsub1);
        vsub2 = vsub1;
        vsub1 = v;
    }
}

// GaussLegendre::set (EMComponent/Quadrature.cpp:93-112): Newton from the
// Chebyshev-like guess, float arithmetic, roots ascending
static void gauss_legendre(int n, std::vector<float>& r, std::vector<float>& w)
{
    r.assign(n, 0);
    w.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        float x = (float)std::cos((double)(PI * (i + 0.75f) / (n + 0.5f)));
        float v, d, dr;
        gl_eval(x, n, v, d);
        int guard = 0;
        do {
            dr = v / d;
            x = x - dr;
            gl_eval(x, n, v, d);
        } while (std::fabs((double)dr) > 2e-7f && ++guard < 1000);
        r[n - 1 - i] = x;
        w[n - 1 - i] = 2 / ((1 - x * x) * d * d);
    }
}

// lagrangeIPWeights (MLFMA.cpp:962-1002): 3-point stencils of the samples
// `cur` (parent level) in the samples `nxt` (child level), clamped at the ends
static void lagrange(const std::vector<float>& nxt, const std::vector<float>& cur, std::vector<int>& loc,
                     std::vector<float>& el)
{
    size_t cols = cur.size();
    loc.assign(3 * cols, 0);
    el.assign(3 * cols, 0);
    size_t nlast = nxt.size() - 1;
    size_t nid = 2;
    float low = nxt[1], high = nxt[nlast - 1];
    for (size_t cid = 0; cid < cols; ++cid) {
        const float xx = cur[cid];
        size_t p1, p2, p3;
        if (xx < low) {
            p1 = 0; p2 = 1; p3 = 2;
        } else if (xx > high) {
            p1 = nlast - 2; p2 = nlast - 1; p3 = nlast;
        } else {
            nid += nxt[nid] < xx ? 1 : 0;
            size_t off = (nxt[nid] - xx < xx - nxt[nid - 1]) ? 1 : 0;
            p1 = nid + off - 2; p2 = nid + off - 1; p3 = nid + off;
        }
        loc[3 * cid] = (int)p1; loc[3 * cid + 1] = (int)p2; loc[3 * cid + 2] = (int)p3;
        const float x0 = nxt[p1], x1 = nxt[p2], x2 = nxt[p3];
        el[3 * cid] = (xx - x1) * (xx - x2) / ((x0 - x1) * (x0 - x2));
        el[3 * cid + 1] = (xx - x0) * (xx - x2) / ((x1 - x0) * (x1 - x2));
        el[3 * cid + 2] = (xx - x0) * (xx - x1) / ((x2 - x0) * (x2 - x1));
    }
}

static float fnorm3(const float* a, const float* b)
{
    float x = a[0] - b[0], y = a[1] - b[1], z = a[2] - b[2];
    return std::sqrt(x * x + y * y + z * z);
}

}  // namespace mh

// per-level device data
struct MLevel {
    int nbox = 0, L = 0, K = 0;
    float len = 0;
    DevBuf parent, oct;                 // parent index and octant per box (int)
    DevBuf child_ptr, child_idx;        // CSR children (int)
    DevBuf far_ptr, far;                // CSR far lists: int2 {source box, offset index}
    DevBuf trans;                       // float2 [343][K]
    DevBuf up, down;                    // planar float2 [right-hand side][nbox][3][K]
    // interpolation to this level from the level below, separable: 3-point
    // Lagrange stencils in theta (per theta index of this level: child theta,
    // weight) and in phi (per phi index: child phi row, weight)
    DevBuf ip_tl, ip_te, ip_pl, ip_pe;
    // anterpolation from the level above, as two transposed 1-D Lagrange
    // stencils: theta (CSR over this level's theta index: parent theta, weight)
    // and phi (CSR over this level's phi index: parent phi, weight)
    DevBuf th_ptr, th_src, th_w, ph_ptr, ph_src, ph_w;
    size_t down_smem = 0;               // shared bytes per CTA (theta-pass rows)
    DevBuf down_win;                    // int2 per chunk: parent phi rows its phi stencils read
    DevBuf up_phase;                    // float2 [8][K]: exp(-j k k.(parent - child)) for the level below
    int up_rows = 0;                    // interpolation from the level below: phi rows per CTA,
    size_t up_child_bytes = 0;          //   shared bytes of one child's theta pass,
    int up_batch = 0;                   //   children per shared-memory pass,
    DevBuf up_win;                      //   int2 per chunk: the child phi rows it reads
};

}  // namespace emfa

struct emfa_mlfma {
    emfa::Ctx* ctx = nullptr;
    emfa::Geom* geom = nullptr;
    emfa_mlfma_params_t p{};
    int levels = 0;   // finest level number L (levels 2..L carry patterns)
    int n = 0;
    float k = 0;
    std::vector<int> perm;         // box order -> RWG index
    std::vector<int> level_boxes;  // boxes per level 0..L
    std::vector<int> poles;        // multipoles per level 2..L
    std::vector<emfa::MLevel> lv;  // index level - 2
    int rcap = 1;                  // right-hand sides the level patterns hold (one apply chunk)
    emfa::DevBuf perm_d, box_of;   // int [n]
    emfa::DevBuf rad, rec;         // C2f [n][Kf]: theta, phi components in each sample's basis
    emfa::DevBuf tp;               // float [Kf][6]: theta_hat, phi_hat of the finest samples
    emfa::DevBuf coeff;            // float [Kf]
    emfa::DevBuf box_off, box_cnt; // finest boxes: first unknown, count
    emfa::DevBuf near_ptr, near_box, near_col, row_cols;  // CSR near lists, column base per slot, C_b per box
    emfa::DevBuf row_base;         // size_t per finest box: first value of the box's rows
    emfa::DevBuf near_val;         // float2 [nnz]
    emfa::DevBuf near_cbase, near_cidx;  // per finest box: first entry, column unknowns of its near rows
    size_t nnz = 0;
    emfa::DevBuf tmp_in, tmp_out;  // complex64 scratch for residuals
    // SAI preconditioner P (CSR over box-order rows), built when p.precond
    bool precond = false;
    size_t sai_nnz = 0;
    std::vector<int> sai_rptr, sai_rows, sai_cptr, sai_cols, sai_own;  // host copies of the lists
    emfa::DevBuf csr_ptr, csr_col, csr_val;  // int [n+1], int [nnz], float2 [nnz]
    emfa::DevBuf pre_tmp, pre_b;             // complex64 scratch: Z x, P b
};

namespace emfa {

// ---------------------------------------------------------------------------
// device kernels
// ---------------------------------------------------------------------------
// radiation / receive patterns of every unknown (box order) at every finest
// sample.  Both are transverse (k . rad = 0: rad is projected off k; the
// receive pattern is alpha conj(rad) plus k x (...)), so they are stored as
// their theta and phi components in the sample's own basis (tp: theta_hat,
// phi_hat per sample), 16 bytes a sample instead of the 24 of x, y, z.
__global__ void k_radrec(const RwgPack<float>* __restrict__ rw, const int* __restrict__ perm,
                         const int* __restrict__ box_of, const float* __restrict__ centers,
                         const float* __restrict__ kdir, const float* __restrict__ tp, int n, int K, float k,
                         float alpha, C2f* __restrict__ rad, C2f* __restrict__ rec)
{
    size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (size_t)n * K) return;
    const int u = (int)(id / K), kk = (int)(id % K);
    const RwgPack<float>& R = rw[perm[u]];
    const float* c = centers + 3 * box_of[u];
    const V3<float> kh = v3(kdir[3 * kk], kdir[3 * kk + 1], kdir[3 * kk + 2]);
    const V3<float> cen = v3(c[0], c[1], c[2]);
    const float w3 = 1.0f / 3.0f;
    float2 ra[3] = {{0, 0}, {0, 0}, {0, 0}}, rh[3] = {{0, 0}, {0, 0}, {0, 0}};
    for (int s = 0; s < 2; ++s) {
        const float sg = s == 0 ? 1.0f : -1.0f;
        const V3<float> fv = v3(R.v[s][0], R.v[s][1], R.v[s][2]);
        const V3<float> nn = v3(R.n[s][0], R.n[s][1], R.n[s][2]);
        for (int q = 0; q < 3; ++q) {
            const V3<float> g = v3(R.q3[s][q][0], R.q3[s][q][1], R.q3[s][q][2]);
            const V3<float> rho = (g - fv) * (sg * w3);
            const V3<float> nr = cross(nn, rho);
            float sn, cs;
            sincos_pi(k * dot(kh, g - cen) / mh::PI, &sn, &cs);
            // rad: rho e^{+j phase}; half receive: (n x rho) e^{-j phase}
            ra[0] = caddf(ra[0], make_float2(rho.x * cs, rho.x * sn));
            ra[1] = caddf(ra[1], make_float2(rho.y * cs, rho.y * sn));
            ra[2] = caddf(ra[2], make_float2(rho.z * cs, rho.z * sn));
            rh[0] = caddf(rh[0], make_float2(nr.x * cs, -nr.x * sn));
            rh[1] = caddf(rh[1], make_float2(nr.y * cs, -nr.y * sn));
            rh[2] = caddf(rh[2], make_float2(nr.z * cs, -nr.z * sn));
        }
    }
    // rad - (k . rad) k
    float2 kd = make_float2(kh.x * ra[0].x + kh.y * ra[1].x + kh.z * ra[2].x, kh.x * ra[0].y + kh.y * ra[1].y + kh.z * ra[2].y);
    ra[0] = make_float2(ra[0].x - kd.x * kh.x, ra[0].y - kd.y * kh.x);
    ra[1] = make_float2(ra[1].x - kd.x * kh.y, ra[1].y - kd.y * kh.y);
    ra[2] = make_float2(ra[2].x - kd.x * kh.z, ra[2].y - kd.y * kh.z);
    // k x half-receive
    float2 hx = make_float2(kh.y * rh[2].x - kh.z * rh[1].x, kh.y * rh[2].y - kh.z * rh[1].y);
    float2 hy = make_float2(kh.z * rh[0].x - kh.x * rh[2].x, kh.z * rh[0].y - kh.x * rh[2].y);
    float2 hz = make_float2(kh.x * rh[1].x - kh.y * rh[0].x, kh.x * rh[1].y - kh.y * rh[0].y);
    const float h = R.len / 2;
    const float b = 1.0f - alpha;
    const float* e = tp + 6 * kk;  // theta_hat, phi_hat
    C3f o, q;
    o.x = cscalef(ra[0], h);
    o.y = cscalef(ra[1], h);
    o.z = cscalef(ra[2], h);
    q.x = make_float2(h * (alpha * ra[0].x + b * hx.x), h * (-alpha * ra[0].y + b * hx.y));
    q.y = make_float2(h * (alpha * ra[1].x + b * hy.x), h * (-alpha * ra[1].y + b * hy.y));
    q.z = make_float2(h * (alpha * ra[2].x + b * hz.x), h * (-alpha * ra[2].y + b * hz.y));
    auto proj = [](const C3f& v, const float* u) {
        return make_float2(u[0] * v.x.x + u[1] * v.y.x + u[2] * v.z.x, u[0] * v.x.y + u[1] * v.y.y + u[2] * v.z.y);
    };
    rad[id] = C2f{proj(o, e), proj(o, e + 3)};
    rec[id] = C2f{proj(q, e), proj(q, e + 3)};
}

// near-field blocks: thread per (field unknown, near-slot); values row-major
// per field box over the concatenated near-box columns
__global__ void k_near_fill(const RwgPack<float>* __restrict__ rw, const int* __restrict__ perm,
                            const int* __restrict__ box_of, const int* __restrict__ box_off,
                            const int* __restrict__ box_cnt, const int* __restrict__ near_ptr,
                            const int* __restrict__ near_box, const int* __restrict__ near_col,
                            const int* __restrict__ row_cols, const size_t* __restrict__ row_base, int n,
                            int max_near, FillConst<float> fc, const double2* __restrict__ sing,
                            float2* __restrict__ val)
{
    size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (size_t)n * max_near) return;
    const int u = (int)(id / max_near), j = (int)(id % max_near);
    const int b = box_of[u];
    const int slot = near_ptr[b] + j;
    if (slot >= near_ptr[b + 1]) return;
    const int nb = near_box[slot];
    const int s0 = box_off[nb], ns = box_cnt[nb];
    const RwgPack<float> F = rw[perm[u]];
    float2* out = val + row_base[b] + (size_t)(u - box_off[b]) * row_cols[b] + near_col[slot];
    for (int q = 0; q < ns; ++q) {
        Cx<float> z = z_entry<float, true>(F, rw[perm[s0 + q]], fc, sing);
        out[q] = make_float2(z.re, z.im);
    }
}

// Level patterns (up and down) are planar: box b's component c occupies
// float2 [(3 b + c) K, (3 b + c + 1) K), so a warp reads 32 consecutive
// samples of one plane at once.

// finest aggregation: CTA per finest box, threads over samples; each
// radiation pattern is read once for up to RB right-hand sides (nr of them:
// x[r][u] at r n + u, patterns of RHS r at out + r ostride)
// (the box's theta and phi sums, then expanded to x, y, z once per sample)
template <int RB>
__global__ void k_agg_finest(const float2* __restrict__ x, int n, int nr, const C2f* __restrict__ rad,
                             const float* __restrict__ tp, const int* __restrict__ box_off,
                             const int* __restrict__ box_cnt, int K, float2* __restrict__ out, size_t ostride)
{
    const int b = blockIdx.x;
    const int o = box_off[b], cnt = box_cnt[b];
    for (int kk = threadIdx.x; kk < K; kk += blockDim.x) {
        float2 at[RB], ap[RB];
#pragma unroll
        for (int r = 0; r < RB; ++r) at[r] = ap[r] = make_float2(0, 0);
        for (int u = 0; u < cnt; ++u) {
            const C2f rv = rad[(size_t)(o + u) * K + kk];
#pragma unroll
            for (int r = 0; r < RB; ++r)
                if (RB == 1 || r < nr) {
                    const float2 xv = x[(size_t)r * n + o + u];
                    at[r] = caddf(at[r], cmulf(xv, rv.t));
                    ap[r] = caddf(ap[r], cmulf(xv, rv.p));
                }
        }
        const float* e = tp + 6 * kk;
#pragma unroll
        for (int r = 0; r < RB; ++r)
            if (RB == 1 || r < nr) {
                float2* ob = out + r * ostride + (size_t)3 * b * K + kk;
                ob[0] = caddf(cscalef(at[r], e[0]), cscalef(ap[r], e[3]));
                ob[K] = caddf(cscalef(at[r], e[1]), cscalef(ap[r], e[4]));
                ob[2 * K] = caddf(cscalef(at[r], e[2]), cscalef(ap[r], e[5]));
            }
    }
}

// interpolation + phase shift: CTA per (parent box, chunk of parent phi rows
// [pp0, pp0 + R)); thread per parent sample (pp, t), k = pp Lp + t.  The
// Lagrange stencil is separable: per child (in batches that fit shared memory)
//   1. theta pass: u[row][t] = sum_it tel(t, it) child(row, tloc(t, it)) for
//      the child phi rows [win.x, win.y) the chunk reads, into shared memory;
//   2. phi pass: parent(pp, t) += phase_oct(pp, t) sum_ip pel(pp, ip) u[ploc(pp, ip)][t].
__global__ void k_upward(const float2* __restrict__ child, int Lc, const int* __restrict__ child_ptr,
                         const int* __restrict__ child_idx, const int* __restrict__ child_oct,
                         const int* __restrict__ tl, const float* __restrict__ te, const int* __restrict__ pl,
                         const float* __restrict__ pe, const int2* __restrict__ win, int batch,
                         const float2* __restrict__ phase, int Lp, int R, float2* __restrict__ out, size_t cstride,
                         size_t ostride)
{
    extern __shared__ float2 s_u[];  // [child in batch][3][rows of the window][Lp]
    child += blockIdx.z * cstride;  // right-hand side blockIdx.z
    out += blockIdx.z * ostride;
    const int b = blockIdx.x;
    const int Kc = 2 * Lc * Lc, K = 2 * Lp * Lp;
    const int pp0 = blockIdx.y * R;
    const int nr = min(R, 2 * Lp - pp0);
    const int2 w2 = win[blockIdx.y];
    const int usz = (w2.y - w2.x) * Lp;  // one plane of one child
    const int it = threadIdx.x;
    const bool act = it < nr * Lp;
    const int pp = pp0 + (act ? it / Lp : 0), t = act ? it % Lp : 0;
    const int kp = pp * Lp + t;
    int prow[3];
    float pw[3];
#pragma unroll
    for (int ip = 0; ip < 3; ++ip) {
        prow[ip] = (pl[3 * pp + ip] - w2.x) * Lp + t;
        pw[ip] = pe[3 * pp + ip];
    }
    const int c0 = child_ptr[b], nch = child_ptr[b + 1] - c0;
    C3f acc = c3zero();
    for (int cb = 0; cb < nch; cb += batch) {
        const int nb = min(batch, nch - cb);
        __syncthreads();  // the previous batch has been read
        for (int cc = 0; cc < nb; ++cc) {
            const float2* src = child + (size_t)3 * child_idx[c0 + cb + cc] * Kc;
            float2* dst = s_u + (size_t)cc * 3 * usz;
            for (int i = threadIdx.x; i < usz; i += blockDim.x) {
                const int r = i / Lp, tt = i - r * Lp;
                const int base = (w2.x + r) * Lc;
                float2 vx = make_float2(0, 0), vy = vx, vz = vx;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const int kc = base + tl[3 * tt + q];
                    const float w = te[3 * tt + q];
                    vx = caddf(vx, cscalef(src[kc], w));
                    vy = caddf(vy, cscalef(src[Kc + kc], w));
                    vz = caddf(vz, cscalef(src[2 * Kc + kc], w));
                }
                dst[i] = vx;
                dst[usz + i] = vy;
                dst[2 * usz + i] = vz;
            }
        }
        __syncthreads();
        if (act)
            for (int cc = 0; cc < nb; ++cc) {
                const float2* u = s_u + (size_t)cc * 3 * usz;
                C3f v = c3zero();
#pragma unroll
                for (int ip = 0; ip < 3; ++ip) {
                    v.x = caddf(v.x, cscalef(u[prow[ip]], pw[ip]));
                    v.y = caddf(v.y, cscalef(u[usz + prow[ip]], pw[ip]));
                    v.z = caddf(v.z, cscalef(u[2 * usz + prow[ip]], pw[ip]));
                }
                c3fma(acc, phase[child_oct[child_idx[c0 + cb + cc]] * K + kp], v);
            }
    }
    if (act) {
        float2* ob = out + (size_t)3 * b * K + kp;
        ob[0] = acc.x;
        ob[K] = acc.y;
        ob[2 * K] = acc.z;
    }
}

// translation from far boxes + anterpolation from the parent: CTA per (box,
// chunk of phi rows [pc0, pc0 + R)), i.e. the contiguous samples
// [pc0 L, (pc0 + R) L) of the box (samples k = pc L + tc, phi-major).
//   1. theta pass (boxes below the top level): for the parent phi rows
//      pp in [win.x, win.y) that the chunk's phi stencils read, and every theta
//      column tc: h[comp][pp - win.x][tc] = sum over the transposed theta
//      stencil of w * conj(phase_oct(pp, t)) * parent(pp, t), into shared memory;
//   2. per pair of samples (16-byte loads of the planar patterns and of the
//      translation table): the far boxes' translated patterns in far-list
//      order, then the transposed phi stencil over h.
__device__ __forceinline__ void cfma2(float4& acc, float4 t, float4 v)
{
    acc.x += t.x * v.x - t.y * v.y;
    acc.y += t.x * v.y + t.y * v.x;
    acc.z += t.z * v.z - t.w * v.w;
    acc.w += t.z * v.w + t.w * v.z;
}

__global__ void k_downward(const float4* __restrict__ up, const int* __restrict__ far_ptr,
                           const int2* __restrict__ far, const float4* __restrict__ trans, int L, int R,
                           const float2* __restrict__ pdown, int Lp, const int2* __restrict__ win,
                           const int* __restrict__ parent, const int* __restrict__ oct,
                           const float2* __restrict__ pphase, const int* __restrict__ th_ptr,
                           const int* __restrict__ th_src, const float* __restrict__ th_w,
                           const int* __restrict__ ph_ptr, const int* __restrict__ ph_src,
                           const float* __restrict__ ph_w, float4* __restrict__ out, size_t ustride, size_t pstride)
{
    extern __shared__ float2 s_h[];  // [3][rows of the window][L]
    // right-hand side blockIdx.z: strides in complex64 (this level, parent level)
    up += blockIdx.z * (ustride / 2);
    out += blockIdx.z * (ustride / 2);
    if (pdown) pdown += blockIdx.z * pstride;
    const int b = blockIdx.x;
    const int K = 2 * L * L, K2 = K >> 1;
    const int pc0 = blockIdx.y * R;
    const int npair = (min(R, 2 * L - pc0) * L) >> 1;
    int2 w2 = make_int2(0, 0);
    int hsz = 0;
    if (pdown) {
        w2 = win[blockIdx.y];
        hsz = (w2.y - w2.x) * L;
        const int Kp = 2 * Lp * Lp;
        const float2* src = pdown + (size_t)3 * parent[b] * Kp;
        const float2* ph0 = pphase + (size_t)oct[b] * Kp;
        for (int i = threadIdx.x; i < hsz; i += blockDim.x) {
            const int r = i / L, tc = i - r * L;
            const int base = (w2.x + r) * Lp;
            float2 sx = make_float2(0, 0), sy = sx, sz = sx;
            for (int a = th_ptr[tc]; a < th_ptr[tc + 1]; ++a) {
                const int kp = base + th_src[a];
                const float w = th_w[a];
                float2 ph = ph0[kp];
                ph = make_float2(ph.x * w, -ph.y * w);  // conj: exp(+j k k.(parent - child))
                sx = caddf(sx, cmulf(ph, src[kp]));
                sy = caddf(sy, cmulf(ph, src[Kp + kp]));
                sz = caddf(sz, cmulf(ph, src[2 * Kp + kp]));
            }
            s_h[i] = sx;
            s_h[hsz + i] = sy;
            s_h[2 * hsz + i] = sz;
        }
        __syncthreads();
    }
    const int f0 = far_ptr[b], f1 = far_ptr[b + 1];
    for (int i = threadIdx.x; i < npair; i += blockDim.x) {
        const int q = ((pc0 * L) >> 1) + i;  // pair index: samples 2q, 2q + 1
        float4 ax = make_float4(0, 0, 0, 0), ay = ax, az = ax;
        for (int f = f0; f < f1; ++f) {
            const int2 e = far[f];
            const float4 t = trans[(size_t)e.y * K2 + q];
            const float4* sp = up + (size_t)3 * e.x * K2 + q;
            cfma2(ax, t, sp[0]);
            cfma2(ay, t, sp[K2]);
            cfma2(az, t, sp[2 * K2]);
        }
        if (pdown) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int kk = 2 * q + h;
                const int pc = kk / L, tc = kk - pc * L;
                float2 sx = make_float2(0, 0), sy = sx, sz = sx;
                for (int a = ph_ptr[pc]; a < ph_ptr[pc + 1]; ++a) {
                    const int r = (ph_src[a] - w2.x) * L + tc;
                    const float w = ph_w[a];
                    sx = caddf(sx, cscalef(s_h[r], w));
                    sy = caddf(sy, cscalef(s_h[hsz + r], w));
                    sz = caddf(sz, cscalef(s_h[2 * hsz + r], w));
                }
                if (h == 0) {
                    ax.x += sx.x; ax.y += sx.y; ay.x += sy.x; ay.y += sy.y; az.x += sz.x; az.y += sz.y;
                } else {
                    ax.z += sx.x; ax.w += sx.y; ay.z += sy.x; ay.w += sy.y; az.z += sz.x; az.w += sz.y;
                }
            }
        }
        float4* ob = out + (size_t)3 * b * K2 + q;
        ob[0] = ax;
        ob[K2] = ay;
        ob[2 * K2] = az;
    }
}

// disaggregation + near field: warp per unknown (box order), for up to RB
// right-hand sides (nr of them; x, y at r n, down patterns at r dstride): the
// receive pattern and the near row are read once.  The near row of unknown u
// is contiguous in val (row_cols[b] values); its column unknowns are listed
// once per box in near_cidx.
template <int RB>
__global__ void k_disagg_near(const float2* __restrict__ x, int nr, const C2f* __restrict__ rec,
                              const float* __restrict__ tp, const float2* __restrict__ down, size_t dstride,
                              const float* __restrict__ coeff, int K,
                              const int* __restrict__ box_of, const int* __restrict__ box_off,
                              const int* __restrict__ row_cols, const size_t* __restrict__ row_base,
                              const int* __restrict__ near_cbase, const int* __restrict__ near_cidx,
                              const float2* __restrict__ val, int n, int skip_near, float2* __restrict__ y)
{
    const int warp = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (warp >= n) return;
    const int u = warp, b = box_of[u];
    float2 acc[RB];
#pragma unroll
    for (int r = 0; r < RB; ++r) acc[r] = make_float2(0, 0);
    const C2f* rr = rec + (size_t)u * K;
    const float2* dd = down + (size_t)3 * b * K;
#pragma unroll 4
    for (int kk = lane; kk < K; kk += 32) {
        const C2f rv = rr[kk];
        const float cf = coeff[kk];
        const float* e = tp + 6 * kk;
#pragma unroll
        for (int r = 0; r < RB; ++r)
            if (RB == 1 || r < nr) {
                const float2* d = dd + r * dstride;
                const float2 dx = d[kk], dy = d[K + kk], dz = d[2 * K + kk];
                // theta and phi components of the down pattern at this sample
                const float2 dt = caddf(caddf(cscalef(dx, e[0]), cscalef(dy, e[1])), cscalef(dz, e[2]));
                const float2 dp = caddf(caddf(cscalef(dx, e[3]), cscalef(dy, e[4])), cscalef(dz, e[5]));
                const float2 t = caddf(cmulf(rv.t, dt), cmulf(rv.p, dp));
                acc[r] = caddf(acc[r], cscalef(t, cf));
            }
    }
    if (!skip_near) {
        const int rc = row_cols[b];
        const float2* vrow = val + row_base[b] + (size_t)(u - box_off[b]) * rc;
        const int* ci = near_cidx + near_cbase[b];
#pragma unroll 4
        for (int j = lane; j < rc; j += 32) {
            const float2 v = vrow[j];
            const int cj = ci[j];
#pragma unroll
            for (int r = 0; r < RB; ++r)
                if (RB == 1 || r < nr) acc[r] = caddf(acc[r], cmulf(v, x[(size_t)r * n + cj]));
        }
    }
#pragma unroll
    for (int r = 0; r < RB; ++r) {
        if (RB > 1 && r >= nr) break;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            acc[r].x += __shfl_xor_sync(0xffffffffu, acc[r].x, o);
            acc[r].y += __shfl_xor_sync(0xffffffffu, acc[r].y, o);
        }
        if (lane == 0) y[(size_t)r * n + u] = acc[r];
    }
}

__global__ void k_gather_c64(const float2* __restrict__ src, const int* __restrict__ idx, int n, int nrhs,
                             float2* __restrict__ dst)
{
    size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (size_t)n * nrhs) return;
    size_t r = id / n, u = id % n;
    dst[id] = src[r * n + idx[u]];
}

__global__ void k_scatter_c128(const double2* __restrict__ src, const int* __restrict__ idx, int n, int nrhs,
                               double2* __restrict__ dst)
{
    size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (size_t)n * nrhs) return;
    size_t r = id / n, u = id % n;
    dst[r * n + idx[u]] = src[id];
}

__global__ void k_resid_c64(const float2* __restrict__ B, const float2* __restrict__ Y, double2* __restrict__ R, size_t tot)
{
    size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id < tot) R[id] = make_double2((double)B[id].x - (double)Y[id].x, (double)B[id].y - (double)Y[id].y);
}

__global__ void k_f64_to_f32(const double2* __restrict__ X, float2* __restrict__ Y, size_t tot)
{
    size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id < tot) Y[id] = make_float2((float)X[id].x, (float)X[id].y);
}

// ---------------------------------------------------------------------------
// SAI preconditioner (MLFMA::parallelPreconditioner, EMSolver/MLFMA.cpp:1346-1391)
// ---------------------------------------------------------------------------
// near-field entry Z(uf, us) in box order, zero when the boxes are not near
__device__ __forceinline__ float2 near_entry(int uf, int us, const int* __restrict__ box_of,
                                             const int* __restrict__ box_off, const int* __restrict__ near_ptr,
                                             const int* __restrict__ near_box, const int* __restrict__ near_col,
                                             const int* __restrict__ row_cols, const size_t* __restrict__ row_base,
                                             const float2* __restrict__ val)
{
    const int bf = box_of[uf], bs = box_of[us];
    for (int sl = near_ptr[bf]; sl < near_ptr[bf + 1]; ++sl)
        if (near_box[sl] == bs)
            return val[row_base[bf] + (size_t)(uf - box_off[bf]) * row_cols[bf] + near_col[sl] + (us - box_off[bs])];
    return make_float2(0.f, 0.f);
}

__device__ __forceinline__ float2 cconjmul(float2 a, float2 b)  // conj(a) b
{
    return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

__device__ __forceinline__ float2 warp_sum2(float2 v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// One CTA (4 warps) per finest box: A = Z_near(rows, cols) (m x n, column
// major in shared memory), complex Householder QR, then for each unknown u
// of the box the least-squares column P(cols, u) = R^-1 Q^H e_(own + u),
// written to its CSR slot.  FP32, as the reference's value_t.
__global__ void __launch_bounds__(128) k_sai(const int* __restrict__ rptr, const int* __restrict__ rows,
                                             const int* __restrict__ cptr, const int* __restrict__ cols,
                                             const int* __restrict__ own, const int* __restrict__ box_cnt,
                                             const size_t* __restrict__ ebase, const int* __restrict__ dest,
                                             const int* __restrict__ box_of, const int* __restrict__ box_off,
                                             const int* __restrict__ near_ptr, const int* __restrict__ near_box,
                                             const int* __restrict__ near_col, const int* __restrict__ row_cols,
                                             const size_t* __restrict__ row_base, const float2* __restrict__ val,
                                             int max_rows, int max_cols, float2* __restrict__ csr_val)
{
    extern __shared__ float2 sm[];
    const int b = blockIdx.x;
    const int m = rptr[b + 1] - rptr[b], n = cptr[b + 1] - cptr[b], nb = box_cnt[b], o = own[b];
    const int* R = rows + rptr[b];
    const int* C = cols + cptr[b];
    float2* A = sm;                                        // [n][m]
    float2* rd = A + (size_t)max_rows * max_cols;          // R diagonal [n]
    float* tau = reinterpret_cast<float*>(rd + max_cols);  // [n]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2* bv = reinterpret_cast<float2*>(tau + max_cols + (max_cols & 1)) + (size_t)warp * (max_rows + max_cols);
    float2* yv = bv + max_rows;
    for (int idx = threadIdx.x; idx < m * n; idx += blockDim.x) {
        const int f = idx % m, s = idx / m;
        A[idx] = near_entry(R[f], C[s], box_of, box_off, near_ptr, near_box, near_col, row_cols, row_base, val);
    }
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        float2* aj = A + (size_t)j * m;
        if (warp == 0) {
            float xs = 0.f;
            for (int i = j + lane; i < m; i += 32) xs += aj[i].x * aj[i].x + aj[i].y * aj[i].y;
#pragma unroll
            for (int q = 16; q > 0; q >>= 1) xs += __shfl_xor_sync(0xffffffffu, xs, q);
            if (lane == 0) {
                // H_j x = al e_j with al = -e^(i arg x0) |x|: no cancellation in v0
                const float xn = sqrtf(xs);
                const float2 x0 = aj[j];
                const float ax = sqrtf(x0.x * x0.x + x0.y * x0.y);
                const float2 al = ax > 0.f ? make_float2(-x0.x / ax * xn, -x0.y / ax * xn) : make_float2(-xn, 0.f);
                const float2 v0 = make_float2(x0.x - al.x, x0.y - al.y);
                const float vn = xs - ax * ax + v0.x * v0.x + v0.y * v0.y;
                aj[j] = v0;
                rd[j] = al;
                tau[j] = vn > 0.f ? 2.f / vn : 0.f;
            }
        }
        __syncthreads();
        const float t = tau[j];
        for (int k = j + 1 + warp; k < n; k += 4) {
            float2* ak = A + (size_t)k * m;
            float2 s = make_float2(0.f, 0.f);
            for (int i = j + lane; i < m; i += 32) {
                const float2 p = cconjmul(aj[i], ak[i]);
                s.x += p.x;
                s.y += p.y;
            }
            s = warp_sum2(s);
            for (int i = j + lane; i < m; i += 32) {
                const float2 v = aj[i];
                ak[i].x -= t * (s.x * v.x - s.y * v.y);
                ak[i].y -= t * (s.x * v.y + s.y * v.x);
            }
        }
        __syncthreads();
    }
    for (int u = warp; u < nb; u += 4) {
        for (int i = lane; i < m; i += 32) bv[i] = make_float2(i == o + u ? 1.f : 0.f, 0.f);
        __syncwarp();
        for (int j = 0; j < n; ++j) {  // b <- H_j b: Q^H e
            const float2* aj = A + (size_t)j * m;
            float2 s = make_float2(0.f, 0.f);
            for (int i = j + lane; i < m; i += 32) {
                const float2 p = cconjmul(aj[i], bv[i]);
                s.x += p.x;
                s.y += p.y;
            }
            s = warp_sum2(s);
            const float t = tau[j];
            for (int i = j + lane; i < m; i += 32) {
                const float2 v = aj[i];
                bv[i].x -= t * (s.x * v.x - s.y * v.y);
                bv[i].y -= t * (s.x * v.y + s.y * v.x);
            }
            __syncwarp();
        }
        for (int i = n - 1; i >= 0; --i) {  // R y = b (R above the diagonal in A, diagonal in rd)
            float2 s = make_float2(0.f, 0.f);
            for (int k = i + 1 + lane; k < n; k += 32) {
                const float2 r = A[(size_t)k * m + i], y = yv[k];
                s.x += r.x * y.x - r.y * y.y;
                s.y += r.x * y.y + r.y * y.x;
            }
            s = warp_sum2(s);
            if (lane == 0) {
                const float2 d = rd[i];
                const float dd = d.x * d.x + d.y * d.y;
                const float2 num = make_float2(bv[i].x - s.x, bv[i].y - s.y);
                yv[i] = dd > 0.f ? make_float2((num.x * d.x + num.y * d.y) / dd, (num.y * d.x - num.x * d.y) / dd)
                                 : make_float2(0.f, 0.f);
            }
            __syncwarp();
        }
        for (int c = lane; c < n; c += 32) csr_val[dest[ebase[b] + (size_t)u * n + c]] = yv[c];
        __syncwarp();
    }
}

// translation operator of every far-box offset at every sample (FP64, the
// host recurrences of parallelLevelTrans, MLFMA.cpp:1191-1222): thread per
// (offset, sample); hl holds each offset's spherical Hankel values
__global__ void k_trans_table(const double2* __restrict__ hl, const int* __restrict__ minl, int lmax,
                              const float* __restrict__ kd, int K, double len, float2* __restrict__ tr)
{
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (size_t)343 * K) return;
    const int off = (int)(id / K), kk = (int)(id % K);
    const int ml = minl[off];
    if (ml < 0) {  // near offsets: no translation
        tr[id] = make_float2(0.f, 0.f);
        return;
    }
    const int dx = off / 49 - 3, dy = (off / 7) % 7 - 3, dz = off % 7 - 3;
    const double D0 = dx * len, D1 = dy * len, D2 = dz * len;
    const double Dn = sqrt(D0 * D0 + D1 * D1 + D2 * D2);
    const double ct = ((double)kd[3 * kk] * D0 + (double)kd[3 * kk + 1] * D1 + (double)kd[3 * kk + 2] * D2) / Dn;
    const double2* h = hl + (size_t)off * (lmax + 1);
    double vr = 0.0, vi = 0.0, p0 = 1.0, p1 = ct;
    for (int q = 0; q <= ml; ++q) {
        double Pq = q == 0 ? 1.0 : ct;
        if (q >= 2) {
            Pq = ((2 * q - 1) * ct * p1 - (q - 1) * p0) / q;
            p0 = p1;
            p1 = Pq;
        }
        // (2q+1) (-j)^q h_q P_q
        const double2 hq = h[q];
        double ar, ai;
        switch (q & 3) {
            case 0: ar = hq.x; ai = hq.y; break;
            case 1: ar = hq.y; ai = -hq.x; break;
            case 2: ar = -hq.x; ai = -hq.y; break;
            default: ar = -hq.y; ai = hq.x; break;
        }
        const double w = (2.0 * q + 1) * Pq;
        vr += w * ar;
        vi += w * ai;
    }
    tr[id] = make_float2((float)vr, (float)vi);
}

// y = P x, P in CSR (row per thread)
__global__ void k_sai_apply(const int* __restrict__ ptr, const int* __restrict__ col, const float2* __restrict__ val,
                            const float2* __restrict__ x, int n, float2* __restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 acc = make_float2(0.f, 0.f);
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) acc = caddf(acc, cmulf(val[k], x[col[k]]));
    y[i] = acc;
}

// ---------------------------------------------------------------------------
// host build
// ---------------------------------------------------------------------------
// phi rows per CTA of the downward pass: an even count giving chunks of about
// 256 samples (sample pairs never straddle a chunk)
static int down_rows(int L)
{
    const int nchunk = (2 * L * L + 255) / 256;
    const int r = (2 * L + nchunk - 1) / nchunk;
    return r + (r & 1);
}

template <typename T>
static emfa_status_t upload(Ctx* c, DevBuf& b, const std::vector<T>& v, cudaStream_t st)
{
    EMFA_TRY(b.alloc(c, sizeof(T) * std::max<size_t>(v.size(), 1)));
    if (!v.empty()) EMFA_CUDA(c, cudaMemcpyAsync(b.ptr, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st));
    return EMFA_OK;
}

// Host plan: everything the reference computes before its operators, in its
// float arithmetic (tree, box order, near/far lists, multipoles, samples).
struct Plan {
    int L = 0;
    float k = 0;
    std::vector<float> blen;
    std::vector<std::vector<mh::Box>> lb;
    std::vector<int> poles;
    std::vector<std::vector<float>> gt, gp, gw, kd;
    std::vector<std::vector<float>> wt1, wp1;  // 1-D Gauss weights in theta and phi (gw = wp1 x wt1)
    std::vector<int> perm, box_of, off, cnt;
    std::vector<float> cen;
    std::vector<float> cp;  // RWG centres (v1 + v2) / 2, RWG order
};

static bool build_plan(const std::vector<double>& verts, int nv, const std::vector<int>& rwg, int n,
                       const emfa_mlfma_params_t& prm, Plan& P, std::string& err)
{
    const float freq = (float)prm.freq;
    const float cc = 299792458.0f;
    const float k = ((2.0f * mh::PI) * freq) / cc;  // PI2 * f / cc
    P.k = k;
    const float lambda = cc / freq;
    // float vertices, as the reference holds them
    std::vector<float> vf(verts.size());
    for (size_t i = 0; i < vf.size(); ++i) vf[i] = (float)verts[i];
    // MLFMA_Boundary::init
    float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int i = 0; i < nv; ++i)
        for (int d = 0; d < 3; ++d) {
            mn[d] = std::min(mn[d], vf[3 * i + d]);
            mx[d] = std::max(mx[d], vf[3 * i + d]);
        }
    float cen[3], half;
    for (int d = 0; d < 3; ++d) cen[d] = (mn[d] + mx[d]) * 0.5f;
    float maxlen = std::max(std::max(mx[0] - mn[0], mx[1] - mn[1]), mx[2] - mn[2]) + 0.1f * lambda;
    half = maxlen / 2;
    float bmin[3], bmax[3];
    for (int d = 0; d < 3; ++d) {
        bmin[d] = cen[d] - half;
        bmax[d] = cen[d] + half;
    }
    const float delta = (float)prm.box_threshold * lambda;
    int L = 0;
    for (float ml = maxlen; ml > delta; ++L) ml /= 2;
    if (L < 2) {
        err = "level number of MLFMA is too small (MLFMA box threshold is too large)";
        return false;
    }
    P.L = L;
    const float big = bmax[0] - bmin[0];
    float root[3];
    for (int d = 0; d < 3; ++d) root[d] = (bmin[d] + bmax[d]) * 0.5f;
    // RWG centres: (v1 + v2) / 2
    std::vector<float>& cp = P.cp;
    cp.assign(3 * (size_t)n, 0.f);
    for (int u = 0; u < n; ++u)
        for (int d = 0; d < 3; ++d) cp[3 * u + d] = (vf[3 * rwg[6 * u] + d] + vf[3 * rwg[6 * u + 1] + d]) * 0.5f;
    // octree (buildBox)
    auto& lb = P.lb;
    auto& blen = P.blen;
    lb.assign(L + 1, {});
    blen.assign(L + 1, 0.f);
    mh::Box rb;
    std::copy(root, root + 3, rb.c);
    for (int u = 0; u < n; ++u) rb.unk.push_back(u);
    lb[0].push_back(rb);
    float cur = big / 2;
    blen[1] = cur;
    for (int l = 1; l <= L; ++l) {
        if (l > 1) {
            cur /= 2;
            blen[l] = cur;
        }
        for (size_t pi = 0; pi < lb[l - 1].size(); ++pi) {
            mh::Box& pb = lb[l - 1][pi];
            mh::Box ch[8];
            for (int x = 0; x < 2; ++x)
                for (int y = 0; y < 2; ++y)
                    for (int z = 0; z < 2; ++z) {
                        int idx = (x * 2 + y) * 2 + z;
                        ch[idx].c[0] = pb.c[0] + (x - 0.5f) * cur;
                        ch[idx].c[1] = pb.c[1] + (y - 0.5f) * cur;
                        ch[idx].c[2] = pb.c[2] + (z - 0.5f) * cur;
                        ch[idx].parent = (int)pi;
                        ch[idx].oct = idx;
                    }
            for (int u : pb.unk) {
                int xf = cp[3 * u] < pb.c[0] ? 0 : 1, yf = cp[3 * u + 1] < pb.c[1] ? 0 : 1,
                    zf = cp[3 * u + 2] < pb.c[2] ? 0 : 1;
                ch[(xf * 2 + yf) * 2 + zf].unk.push_back(u);
            }
            int pos = pb.offset;
            for (int ci = 0; ci < 8; ++ci) {
                if (ch[ci].unk.empty()) continue;
                ch[ci].offset = pos;
                pos += (int)ch[ci].unk.size();
                pb.child.push_back((int)lb[l].size());
                lb[l].push_back(std::move(ch[ci]));
            }
        }
    }
    // setBoxParameter: level 1 all near; level >= 2 near if centre distance < 1.75 box
    for (size_t f = 0; f < lb[1].size(); ++f)
        for (size_t s2 = 0; s2 < lb[1].size(); ++s2) lb[1][f].near.push_back((int)s2);
    float clen = big / 4;
    for (int l = 2; l <= L; ++l, clen /= 2) {
        float lim = 1.75f * clen;
        for (auto& b : lb[l]) {
            for (int pn : lb[l - 1][b.parent].near)
                for (int cidx : lb[l - 1][pn].child) {
                    float dist = mh::fnorm3(lb[l][cidx].c, b.c);
                    (dist < lim ? b.near : b.far).push_back(cidx);
                }
        }
    }
    // box order of the unknowns
    const auto& fin = lb[L];
    P.perm.clear();
    P.box_of.assign(n, 0);
    for (size_t b = 0; b < fin.size(); ++b) {
        P.off.push_back(fin[b].offset);
        P.cnt.push_back((int)fin[b].unk.size());
        for (int u : fin[b].unk) {
            P.box_of[P.perm.size()] = (int)b;
            P.perm.push_back(u);
        }
        P.cen.insert(P.cen.end(), fin[b].c, fin[b].c + 3);
    }
    // multipoles, samples, weights, directions
    const int nl = L - 1;
    P.poles.assign(nl, 0);
    auto& gt = P.gt;
    auto& gp = P.gp;
    auto& gw = P.gw;
    auto& kd = P.kd;
    gt.assign(nl, {});
    P.wt1.assign(nl, {});
    P.wp1.assign(nl, {});
    gp.assign(nl, {});
    gw.assign(nl, {});
    kd.assign(nl, {});
    for (int l = 2; l <= L; ++l) {
        int i = l - 2;
        float kdl = 1.732051f * k * blen[l];
        // the reference's rule, or the excess-bandwidth rule of the
        // configuration (d0 = 3 digits: d0^(2/3) = 9^(1/3))
        int Pm = prm.truncation == 1 ? (int)(kdl + 1.8f * cbrtf(9.0f) * cbrtf(kdl)) : (int)(kdl + 6 * cbrtf(kdl));
        P.poles[i] = Pm;
        std::vector<float> rt, wt, rp, wp;
        mh::gauss_legendre(Pm, rt, wt);
        mh::gauss_legendre(2 * Pm, rp, wp);
        gt[i] = rt;
        gp[i] = rp;
        P.wt1[i] = wt;
        P.wp1[i] = wp;
        gw[i].resize(2 * (size_t)Pm * Pm);
        kd[i].resize(3 * 2 * (size_t)Pm * Pm);
        size_t q = 0;
        for (int pp = 0; pp < 2 * Pm; ++pp)
            for (int t = 0; t < Pm; ++t, ++q) gw[i][q] = wp[pp] * wt[t];
        const float PIh = 0.5f * mh::PI;
        for (int pp = 0; pp < 2 * Pm; ++pp) {
            float phi = mh::PI * (rp[pp] + 1);
            float ps = (float)std::sin((double)phi), pc = (float)std::cos((double)phi);
            for (int t = 0; t < Pm; ++t) {
                float th = PIh * (rt[t] + 1);
                float ts = (float)std::sin((double)th), tc = (float)std::cos((double)th);
                size_t kk = (size_t)pp * Pm + t;
                kd[i][3 * kk] = ts * pc;
                kd[i][3 * kk + 1] = ts * ps;
                kd[i][3 * kk + 2] = tc;
            }
        }
    }
    return true;
}

// SAI lists (MLFMA::setBoxParameter and parallelPreconditioner, EMSolver/MLFMA.cpp:719-741,1346-1370):
// per finest box, the near unknowns whose centre lies within row / col
// threshold x finest box length of the box centre, in near-box order; then
// the batched QR on the device and P in CSR over box-order rows
static emfa_status_t sai_build(emfa_mlfma* M, const Plan& P, cudaStream_t st)
{
    Ctx* c = M->ctx;
    if (!(M->p.row_threshold >= 0.87) || !(M->p.col_threshold >= 0.87)) {
        set_error(c, "MLFMA preconditioner: row_threshold and col_threshold must be >= 0.87 (a box's own "
                     "unknowns lie within sqrt(3)/2 box lengths of its centre)");
        return EMFA_ERR_INVALID;
    }
    const auto& fin = P.lb[P.L];
    const float bl = P.blen[P.L];
    const float thr_r = (float)M->p.row_threshold * bl, thr_c = (float)M->p.col_threshold * bl;
    const int nbox = (int)fin.size(), n = M->n;
    auto& rptr = M->sai_rptr;
    auto& rows = M->sai_rows;
    auto& cptr = M->sai_cptr;
    auto& cols = M->sai_cols;
    auto& own = M->sai_own;
    rptr.assign(1, 0);
    cptr.assign(1, 0);
    rows.clear();
    cols.clear();
    own.clear();
    std::vector<size_t> ebase;
    size_t nnz = 0;
    int max_rows = 1, max_cols = 1;
    for (int b = 0; b < nbox; ++b) {
        int o = -1;
        for (int nb : fin[b].near) {
            if (nb == b) o = (int)(rows.size() - rptr.back());
            for (size_t i = 0; i < fin[nb].unk.size(); ++i) {
                const float dist = mh::fnorm3(&P.cp[3 * (size_t)fin[nb].unk[i]], fin[b].c);
                const int idx = fin[nb].offset + (int)i;
                if (dist <= thr_r) rows.push_back(idx);
                if (dist <= thr_c) cols.push_back(idx);
            }
        }
        rptr.push_back((int)rows.size());
        cptr.push_back((int)cols.size());
        own.push_back(o);
        const int m = rptr[b + 1] - rptr[b], nc = cptr[b + 1] - cptr[b];
        max_rows = std::max(max_rows, m);
        max_cols = std::max(max_cols, nc);
        ebase.push_back(nnz);
        nnz += (size_t)nc * fin[b].unk.size();
    }
    // CSR of P over rows = cols[c], columns = the box's own unknowns, the
    // entries of a row in the order the boxes produce them
    std::vector<int> cnt(n + 1, 0), dest(std::max<size_t>(nnz, 1)), ccol(std::max<size_t>(nnz, 1));
    for (int b = 0; b < nbox; ++b)
        for (size_t u = 0; u < fin[b].unk.size(); ++u)
            for (int k = cptr[b]; k < cptr[b + 1]; ++k) cnt[cols[k] + 1] += 1;
    for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    std::vector<int> fillp(cnt.begin(), cnt.end() - 1);
    for (int b = 0; b < nbox; ++b)
        for (size_t u = 0; u < fin[b].unk.size(); ++u)
            for (int k = cptr[b]; k < cptr[b + 1]; ++k) {
                const size_t e = ebase[b] + u * (size_t)(cptr[b + 1] - cptr[b]) + (k - cptr[b]);
                const int pos = fillp[cols[k]]++;
                dest[e] = pos;
                ccol[pos] = fin[b].offset + (int)u;
            }
    const size_t smem = sizeof(float2) * ((size_t)max_rows * max_cols + max_cols) +
                        sizeof(float) * (max_cols + (max_cols & 1)) + sizeof(float2) * 4 * (size_t)(max_rows + max_cols);
    if (smem > 220 * 1024) {
        set_error(c, "MLFMA preconditioner: a near block of " + std::to_string(max_rows) + " x " +
                         std::to_string(max_cols) + " does not fit in shared memory (use smaller boxes)");
        return EMFA_ERR_UNSUPPORTED;
    }
    M->sai_nnz = nnz;
    DevBuf d_rptr, d_rows, d_cptr, d_cols, d_own, d_ebase, d_dest;
    EMFA_TRY(upload(c, d_rptr, rptr, st));
    EMFA_TRY(upload(c, d_rows, rows, st));
    EMFA_TRY(upload(c, d_cptr, cptr, st));
    EMFA_TRY(upload(c, d_cols, cols, st));
    EMFA_TRY(upload(c, d_own, own, st));
    EMFA_TRY(upload(c, d_ebase, ebase, st));
    EMFA_TRY(upload(c, d_dest, dest, st));
    EMFA_TRY(upload(c, M->csr_ptr, cnt, st));
    EMFA_TRY(upload(c, M->csr_col, ccol, st));
    EMFA_TRY(M->csr_val.alloc(c, sizeof(float2) * std::max<size_t>(nnz, 1)));
    EMFA_TRY(M->pre_tmp.alloc(c, sizeof(float2) * (size_t)n));
    EMFA_TRY(ensure_smem(c, k_sai, smem));
    k_sai<<<nbox, 128, smem, st>>>(dptr<int>(d_rptr), dptr<int>(d_rows), dptr<int>(d_cptr), dptr<int>(d_cols),
                                   dptr<int>(d_own), dptr<int>(M->box_cnt), dptr<size_t>(d_ebase), dptr<int>(d_dest),
                                   dptr<int>(M->box_of), dptr<int>(M->box_off), dptr<int>(M->near_ptr),
                                   dptr<int>(M->near_box), dptr<int>(M->near_col), dptr<int>(M->row_cols),
                                   dptr<size_t>(M->row_base), dptr<float2>(M->near_val), max_rows, max_cols,
                                   dptr<float2>(M->csr_val));
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    EMFA_CUDA(c, cudaStreamSynchronize(st));  // the list buffers and host vectors are released on return
    M->precond = true;
    return EMFA_OK;
}

static emfa_status_t mlfma_build(emfa_mlfma* M, cudaStream_t st)
{
    Ctx* c = M->ctx;
    Geom* g = M->geom;
    const int n = g->n;
    M->n = n;
    Plan P;
    std::string err;
    if (!build_plan(g->verts, g->nv, g->rwg, n, M->p, P, err)) {
        set_error(c, err);
        return EMFA_ERR_INVALID;
    }
    const int L = P.L;
    const float k = P.k;
    M->k = k;
    M->levels = L;
    auto& lb = P.lb;
    auto& gt = P.gt;
    auto& gp = P.gp;
    auto& gw = P.gw;
    auto& kd = P.kd;
    const auto& fin = lb[L];
    M->level_boxes.clear();
    for (int l = 0; l <= L; ++l) M->level_boxes.push_back((int)lb[l].size());
    M->perm = P.perm;
    M->poles = P.poles;
    std::vector<int>& box_of_h = P.box_of;
    std::vector<int>& off_h = P.off;
    std::vector<int>& cnt_h = P.cnt;
    std::vector<float>& cen_h = P.cen;
    const int nl = L - 1;
    M->lv.clear();
    M->lv.resize(nl);
    for (int l = 2; l <= L; ++l) {
        const int i = l - 2;
        MLevel& ml = M->lv[i];
        ml.nbox = (int)lb[l].size();
        ml.L = P.poles[i];
        ml.K = 2 * ml.L * ml.L;
        ml.len = P.blen[l];
    }
    // the interpolation and anterpolation passes may use more than the default 48 KB of shared memory
    EMFA_TRY(ensure_smem(c, k_upward, 96 * 1024));
    EMFA_TRY(ensure_smem(c, k_downward, 200 * 1024));
    // per-level device tables
    for (int l = 2; l <= L; ++l) {
        const int i = l - 2;
        MLevel& ml = M->lv[i];
        const int K = ml.K;
        std::vector<int> par, oc, cptr{0}, cidx, fptr{0}, fbox, foff;
        for (auto& b : lb[l]) {
            par.push_back(b.parent);
            oc.push_back(b.oct);
            for (int f : b.far) {
                const float* a = b.c;
                const float* o = lb[l][f].c;
                int dx = (int)std::lround((a[0] - o[0]) / ml.len), dy = (int)std::lround((a[1] - o[1]) / ml.len),
                    dz = (int)std::lround((a[2] - o[2]) / ml.len);
                fbox.push_back(f);
                foff.push_back(((dx + 3) * 7 + (dy + 3)) * 7 + (dz + 3));
            }
            fptr.push_back((int)fbox.size());
        }
        if (l < L)
            for (auto& b : lb[l]) {
                for (int ch : b.child) cidx.push_back(ch);
                cptr.push_back((int)cidx.size());
            }
        EMFA_TRY(upload(c, ml.parent, par, st));
        EMFA_TRY(upload(c, ml.oct, oc, st));
        {
            std::vector<int2> fe(fbox.size());
            for (size_t f = 0; f < fbox.size(); ++f) fe[f] = make_int2(fbox[f], foff[f]);
            EMFA_TRY(upload(c, ml.far_ptr, fptr, st));
            EMFA_TRY(upload(c, ml.far, fe, st));
        }
        EMFA_TRY(upload(c, ml.child_ptr, cptr, st));
        EMFA_TRY(upload(c, ml.child_idx, cidx, st));
        // translation operators per offset: sum_l (2l+1)(-j)^l h_l^(2)(kD) P_l(k.D/|D|),
        // l <= min(poles, floor(kD)) (MLFMA.cpp:1203-1219), in FP64: the Hankel
        // recurrence per offset here, the Legendre sums per sample on the device
        {
            const int lmax = ml.L;
            std::vector<double2> hlv((size_t)343 * (lmax + 1), make_double2(0, 0));
            std::vector<int> minl(343, -1);
            for (int dx = -3; dx <= 3; ++dx)
                for (int dy = -3; dy <= 3; ++dy)
                    for (int dz = -3; dz <= 3; ++dz) {
                        if (std::abs(dx) <= 1 && std::abs(dy) <= 1 && std::abs(dz) <= 1) continue;
                        const int off = ((dx + 3) * 7 + (dy + 3)) * 7 + (dz + 3);
                        double D[3] = {dx * (double)ml.len, dy * (double)ml.len, dz * (double)ml.len};
                        double Dn = std::sqrt(D[0] * D[0] + D[1] * D[1] + D[2] * D[2]);
                        double x = (double)k * Dn;
                        int minL = (int)std::min((float)ml.L, (float)(k * (float)Dn));
                        minL = std::min(minL, lmax);
                        std::vector<std::complex<double>> hl(minL + 1);
                        hl[0] = std::complex<double>(std::sin(x), std::cos(x)) / x;
                        if (minL >= 1)
                            hl[1] = std::complex<double>(std::sin(x) / x - std::cos(x), std::cos(x) / x + std::sin(x)) / x;
                        for (int q = 2; q <= minL; ++q) hl[q] = ((2.0 * q - 1) / x) * hl[q - 1] - hl[q - 2];
                        for (int q = 0; q <= minL; ++q)
                            hlv[(size_t)off * (lmax + 1) + q] = make_double2(hl[q].real(), hl[q].imag());
                        minl[off] = minL;
                    }
            DevBuf d_hl, d_minl, d_kd;
            EMFA_TRY(upload(c, d_hl, hlv, st));
            EMFA_TRY(upload(c, d_minl, minl, st));
            EMFA_TRY(upload(c, d_kd, kd[i], st));
            EMFA_TRY(ml.trans.alloc(c, sizeof(float2) * (size_t)343 * K));
            const size_t tot = (size_t)343 * K;
            k_trans_table<<<(unsigned)((tot + 127) / 128), 128, 0, st>>>(dptr<double2>(d_hl), dptr<int>(d_minl), lmax,
                                                                         dptr<float>(d_kd), K, (double)ml.len,
                                                                         dptr<float2>(ml.trans));
            c->kernel_launches += 1;
            EMFA_CUDA(c, cudaGetLastError());
            EMFA_CUDA(c, cudaStreamSynchronize(st));  // host vectors and the small tables are released next
        }
        EMFA_TRY(ml.up.alloc(c, sizeof(float2) * 3 * (size_t)ml.nbox * K));
        EMFA_TRY(ml.down.alloc(c, sizeof(float2) * 3 * (size_t)ml.nbox * K));
    }
    // interpolation level i+1 (child, fewer samples) -> level i (parent), i = 0..nl-2
    for (int i = 0; i + 1 < nl; ++i) {
        MLevel& pm = M->lv[i];
        MLevel& cm = M->lv[i + 1];
        std::vector<int> tloc, ploc;
        std::vector<float> tel, pel;
        mh::lagrange(gt[i + 1], gt[i], tloc, tel);
        mh::lagrange(gp[i + 1], gp[i], ploc, pel);
        const int Kp = pm.K, Lc = cm.L;
        EMFA_TRY(upload(c, pm.ip_tl, tloc, st));
        EMFA_TRY(upload(c, pm.ip_te, tel, st));
        EMFA_TRY(upload(c, pm.ip_pl, ploc, st));
        EMFA_TRY(upload(c, pm.ip_pe, pel, st));
        {
            // phi-row chunks of about 256 parent samples and the child rows each reads
            pm.up_rows = down_rows(pm.L);
            const int nchunk = (2 * pm.L + pm.up_rows - 1) / pm.up_rows;
            std::vector<int2> win(nchunk);
            int most = 0;
            for (int ch = 0; ch < nchunk; ++ch) {
                int lo = 2 * Lc, hi = 0;
                for (int pp = ch * pm.up_rows; pp < std::min(2 * pm.L, (ch + 1) * pm.up_rows); ++pp)
                    for (int ip = 0; ip < 3; ++ip) {
                        lo = std::min(lo, ploc[3 * pp + ip]);
                        hi = std::max(hi, ploc[3 * pp + ip] + 1);
                    }
                win[ch] = make_int2(lo, hi);
                most = std::max(most, hi - lo);
            }
            pm.up_child_bytes = sizeof(float2) * 3 * (size_t)most * pm.L;
            pm.up_batch = (int)std::min<size_t>(8, (96 * 1024) / pm.up_child_bytes);
            if (pm.up_batch < 1) {
                set_error(c, "mlfma: interpolation rows exceed shared memory (level too large)");
                return EMFA_ERR_UNSUPPORTED;
            }
            EMFA_TRY(upload(c, pm.up_win, win, st));
        }
        // phases for the children of level i: exp(-j k kp . (parent - child)), per octant
        std::vector<float2> ph((size_t)8 * Kp);
        for (int o = 0; o < 8; ++o) {
            int x = o >> 2, y = (o >> 1) & 1, z = o & 1;
            float rv[3] = {-(x - 0.5f) * cm.len, -(y - 0.5f) * cm.len, -(z - 0.5f) * cm.len};
            for (int kk = 0; kk < Kp; ++kk) {
                double a = (double)k * ((double)kd[i][3 * kk] * rv[0] + (double)kd[i][3 * kk + 1] * rv[1] +
                                         (double)kd[i][3 * kk + 2] * rv[2]);
                ph[(size_t)o * Kp + kk] = make_float2((float)std::cos(a), (float)-std::sin(a));
            }
        }
        EMFA_TRY(upload(c, pm.up_phase, ph, st));
        // anterpolation into level i+1: the transposed theta and phi Lagrange
        // stencils, each weight scaled by w_parent / w_child of its own axis
        // (the 2-D weights are products: gw = wp x wt)
        {
            const int Lp = pm.L;
            auto transpose = [](const std::vector<int>& loc, const std::vector<float>& el, int np, int nc,
                                const std::vector<float>& wpar, const std::vector<float>& wch, std::vector<int>& ptr,
                                std::vector<int>& src, std::vector<float>& wt) {
                std::vector<std::vector<std::pair<int, float>>> lst(nc);
                for (int x = 0; x < np; ++x)
                    for (int q = 0; q < 3; ++q) {
                        const int y = loc[3 * x + q];
                        lst[y].push_back({x, el[3 * x + q] * wpar[x] / wch[y]});
                    }
                ptr.assign(1, 0);
                src.clear();
                wt.clear();
                for (int y = 0; y < nc; ++y) {
                    for (auto& e : lst[y]) {
                        src.push_back(e.first);
                        wt.push_back(e.second);
                    }
                    ptr.push_back((int)src.size());
                }
            };
            std::vector<int> tptr, tsrc, pptr, psrc;
            std::vector<float> tw, pw;
            transpose(tloc, tel, Lp, Lc, P.wt1[i], P.wt1[i + 1], tptr, tsrc, tw);
            transpose(ploc, pel, 2 * Lp, 2 * Lc, P.wp1[i], P.wp1[i + 1], pptr, psrc, pw);
            EMFA_TRY(upload(c, cm.th_ptr, tptr, st));
            EMFA_TRY(upload(c, cm.th_src, tsrc, st));
            EMFA_TRY(upload(c, cm.th_w, tw, st));
            EMFA_TRY(upload(c, cm.ph_ptr, pptr, st));
            EMFA_TRY(upload(c, cm.ph_src, psrc, st));
            EMFA_TRY(upload(c, cm.ph_w, pw, st));
            // phi-row chunks of about 256 samples, and the parent rows each reads
            const int rows = down_rows(Lc);
            const int nchunk = (2 * Lc + rows - 1) / rows;
            std::vector<int2> dw(nchunk);
            int most = 0;
            for (int ch = 0; ch < nchunk; ++ch) {
                int lo = 2 * Lp, hi = 0;
                for (int pc = ch * rows; pc < std::min(2 * Lc, (ch + 1) * rows); ++pc)
                    for (int a = pptr[pc]; a < pptr[pc + 1]; ++a) {
                        lo = std::min(lo, psrc[a]);
                        hi = std::max(hi, psrc[a] + 1);
                    }
                if (hi <= lo) lo = hi = 0;
                dw[ch] = make_int2(lo, hi);
                most = std::max(most, hi - lo);
            }
            cm.down_smem = sizeof(float2) * 3 * (size_t)most * Lc;
            if (cm.down_smem > 200 * 1024) {
                set_error(c, "mlfma: anterpolation rows exceed shared memory (level too large)");
                return EMFA_ERR_UNSUPPORTED;
            }
            EMFA_TRY(upload(c, cm.down_win, dw, st));
        }
    }
    // finest-level data
    MLevel& fl = M->lv[nl - 1];
    const int Kf = fl.K;
    std::vector<float> coeff(Kf);
    {
        const float PIh = 0.5f * mh::PI;
        size_t q = 0;
        const int P = fl.L;
        for (int pp = 0; pp < 2 * P; ++pp)
            for (int t = 0; t < P; ++t, ++q) coeff[q] = (float)(gw[nl - 1][q] * std::sin((double)(PIh * (gt[nl - 1][t] + 1))));
        const float z0 = 120.0f * mh::PI;
        const float cn = k * k * z0 / 32;
        for (auto& v : coeff) v = cn * v;
    }
    EMFA_TRY(upload(c, M->coeff, coeff, st));
    EMFA_TRY(upload(c, M->perm_d, M->perm, st));
    EMFA_TRY(upload(c, M->box_of, box_of_h, st));
    EMFA_TRY(upload(c, M->box_off, off_h, st));
    EMFA_TRY(upload(c, M->box_cnt, cnt_h, st));
    DevBuf cen_d, kdir_d;
    EMFA_TRY(upload(c, cen_d, cen_h, st));
    EMFA_TRY(upload(c, kdir_d, kd[nl - 1], st));
    EMFA_TRY(geom_prepare_f32(g, st));
    // theta_hat, phi_hat of every finest sample direction (FP64 from the
    // sample's float direction, stored in float): phi_hat = z x k / |z x k|,
    // theta_hat = phi_hat x k (the Gauss-Legendre theta nodes avoid the poles)
    {
        std::vector<float> tp((size_t)6 * Kf);
        const auto& kv = kd[nl - 1];
        for (int kk = 0; kk < Kf; ++kk) {
            const double kx = kv[3 * kk], ky = kv[3 * kk + 1], kz = kv[3 * kk + 2];
            const double rho = std::sqrt(kx * kx + ky * ky);
            const double px = -ky / rho, py = kx / rho;
            const double tx = py * kz, ty = -px * kz, tz = px * ky - py * kx;
            const double tv[6] = {tx, ty, tz, px, py, 0.0};
            for (int j = 0; j < 6; ++j) tp[6 * (size_t)kk + j] = (float)tv[j];
        }
        EMFA_TRY(upload(c, M->tp, tp, st));
    }
    EMFA_TRY(M->rad.alloc(c, sizeof(C2f) * (size_t)n * Kf));
    EMFA_TRY(M->rec.alloc(c, sizeof(C2f) * (size_t)n * Kf));
    {
        size_t tot = (size_t)n * Kf;
        k_radrec<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(dptr<RwgPack<float>>(g->g32.rwg), dptr<int>(M->perm_d),
                                                               dptr<int>(M->box_of), dptr<float>(cen_d),
                                                               dptr<float>(kdir_d), dptr<float>(M->tp), n, Kf, k,
                                                               (float)M->p.alpha, dptr<C2f>(M->rad),
                                                               dptr<C2f>(M->rec));
        c->kernel_launches += 1;
    }
    // near field: CSR of near boxes, column bases, row bases
    std::vector<int> nptr{0}, nbox, ncol, rcols;
    std::vector<size_t> rbase;
    size_t nnz = 0;
    int max_near = 0;
    for (size_t b = 0; b < fin.size(); ++b) {
        int cols = 0;
        for (int nb : fin[b].near) {
            nbox.push_back(nb);
            ncol.push_back(cols);
            cols += (int)fin[nb].unk.size();
        }
        nptr.push_back((int)nbox.size());
        max_near = std::max(max_near, (int)fin[b].near.size());
        rcols.push_back(cols);
        rbase.push_back(nnz);
        nnz += (size_t)cols * fin[b].unk.size();
    }
    M->nnz = nnz;
    {
        // column unknowns of each box's near rows, in value order
        std::vector<int> cbase{0}, cidx;
        for (size_t b = 0; b < fin.size(); ++b) {
            for (int nb : fin[b].near)
                for (int q = 0; q < cnt_h[nb]; ++q) cidx.push_back(off_h[nb] + q);
            cbase.push_back((int)cidx.size());
        }
        EMFA_TRY(upload(c, M->near_cbase, cbase, st));
        EMFA_TRY(upload(c, M->near_cidx, cidx, st));
    }
    EMFA_TRY(upload(c, M->near_ptr, nptr, st));
    EMFA_TRY(upload(c, M->near_box, nbox, st));
    EMFA_TRY(upload(c, M->near_col, ncol, st));
    EMFA_TRY(upload(c, M->row_cols, rcols, st));
    EMFA_TRY(upload(c, M->row_base, rbase, st));
    EMFA_TRY(M->near_val.alloc(c, sizeof(float2) * std::max<size_t>(nnz, 1)));
    {
        emfa_fill_params_t fp{EMFA_CFIE, EMFA_F32, M->p.freq, M->p.alpha, 0, 0, 0};
        DevBuf tab;
        EMFA_TRY(tab.alloc(c, sizeof(double2) * (size_t)g->nt * 9));
        EMFA_TRY(build_singular_table(c, g, &fp, dptr<double2>(tab), st));
        FillConst<float> fc = make_fill_const<float>(&fp);
        size_t tot = (size_t)n * max_near;
        k_near_fill<<<(unsigned)((tot + 127) / 128), 128, 0, st>>>(
            dptr<RwgPack<float>>(g->g32.rwg), dptr<int>(M->perm_d), dptr<int>(M->box_of), dptr<int>(M->box_off),
            dptr<int>(M->box_cnt), dptr<int>(M->near_ptr), dptr<int>(M->near_box), dptr<int>(M->near_col),
            dptr<int>(M->row_cols), dptr<size_t>(M->row_base), n, max_near, fc, dptr<double2>(tab),
            dptr<float2>(M->near_val));
        c->kernel_launches += 1;
        EMFA_CUDA(c, cudaGetLastError());
        EMFA_CUDA(c, cudaStreamSynchronize(st));
    }
    if (M->p.precond) EMFA_TRY(sai_build(M, P, st));
    EMFA_CUDA(c, cudaGetLastError());
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    return EMFA_OK;
}

// right-hand sides per pass of the operator's kernels
constexpr int RHS_CHUNK = 8;

// level patterns for nr right-hand sides (scratch: grown, never copied)
static emfa_status_t reserve_rhs(emfa_mlfma* M, int nr)
{
    if (nr <= M->rcap) return EMFA_OK;
    for (auto& ml : M->lv) {
        const size_t per = sizeof(float2) * 3 * (size_t)ml.nbox * ml.K;
        EMFA_TRY(ml.up.alloc(M->ctx, per * nr));
        EMFA_TRY(ml.down.alloc(M->ctx, per * nr));
    }
    M->rcap = nr;
    return EMFA_OK;
}

template <int RB>
static void launch_agg_disagg(emfa_mlfma* M, bool agg, const float2* x, int nr, float2* y, int parts, cudaStream_t st)
{
    const int nl = M->levels - 1;
    MLevel& fl = M->lv[nl - 1];
    const int Kf = fl.K, n = M->n;
    const size_t lstride = (size_t)3 * fl.nbox * Kf;
    if (agg)
        k_agg_finest<RB><<<fl.nbox, 128, 0, st>>>(x, n, nr, dptr<C2f>(M->rad), dptr<float>(M->tp),
                                                  dptr<int>(M->box_off), dptr<int>(M->box_cnt), Kf,
                                                  dptr<float2>(fl.up), lstride);
    else
        k_disagg_near<RB><<<(unsigned)(((size_t)n * 32 + 255) / 256), 256, 0, st>>>(
            x, nr, dptr<C2f>(M->rec), dptr<float>(M->tp), dptr<float2>(fl.down), lstride, dptr<float>(M->coeff),
            parts == 1 ? 0 : Kf,
            dptr<int>(M->box_of), dptr<int>(M->box_off), dptr<int>(M->row_cols), dptr<size_t>(M->row_base),
            dptr<int>(M->near_cbase), dptr<int>(M->near_cidx), dptr<float2>(M->near_val), n, parts == 2 ? 1 : 0, y);
}

static void agg_disagg(emfa_mlfma* M, bool agg, const float2* x, int nr, float2* y, int parts, cudaStream_t st)
{
    if (nr <= 1)
        launch_agg_disagg<1>(M, agg, x, nr, y, parts, st);
    else if (nr <= 2)
        launch_agg_disagg<2>(M, agg, x, nr, y, parts, st);
    else if (nr <= 4)
        launch_agg_disagg<4>(M, agg, x, nr, y, parts, st);
    else
        launch_agg_disagg<8>(M, agg, x, nr, y, parts, st);
}

// y = Z x for nr <= RHS_CHUNK vectors (RHS-major, box order, complex64);
// parts: 0 near + far, 1 near, 2 far
static emfa_status_t mlfma_apply(emfa_mlfma* M, const float2* x, float2* y, int nr, cudaStream_t st, int parts = 0)
{
    Ctx* c = M->ctx;
    EMFA_TRY(reserve_rhs(M, nr));
    const int nl = M->levels - 1;
    agg_disagg(M, true, x, nr, y, parts, st);
    for (int i = nl - 2; i >= 0; --i) {
        MLevel& pm = M->lv[i];
        MLevel& cm = M->lv[i + 1];
        const int R = pm.up_rows;
        const int bs = 32 * ((R * pm.L + 31) / 32);
        const dim3 grid((unsigned)pm.nbox, (unsigned)((2 * pm.L + R - 1) / R), (unsigned)nr);
        k_upward<<<grid, bs, pm.up_child_bytes * pm.up_batch, st>>>(
            dptr<float2>(cm.up), cm.L, dptr<int>(pm.child_ptr), dptr<int>(pm.child_idx), dptr<int>(cm.oct),
            dptr<int>(pm.ip_tl), dptr<float>(pm.ip_te), dptr<int>(pm.ip_pl), dptr<float>(pm.ip_pe),
            dptr<int2>(pm.up_win), pm.up_batch, dptr<float2>(pm.up_phase), pm.L, R, dptr<float2>(pm.up),
            (size_t)3 * cm.nbox * cm.K, (size_t)3 * pm.nbox * pm.K);
    }
    for (int i = 0; i < nl; ++i) {
        MLevel& ml = M->lv[i];
        const bool top = i == 0;
        MLevel& pm = M->lv[top ? 0 : i - 1];
        const int R = down_rows(ml.L);
        const int bs = std::min(256, 32 * ((R * ml.L / 2 + 31) / 32));
        const dim3 grid((unsigned)ml.nbox, (unsigned)((2 * ml.L + R - 1) / R), (unsigned)nr);
        k_downward<<<grid, bs, top ? 0 : ml.down_smem, st>>>(
            dptr<float4>(ml.up), dptr<int>(ml.far_ptr), dptr<int2>(ml.far), dptr<float4>(ml.trans), ml.L, R,
            top ? nullptr : dptr<float2>(pm.down), pm.L, dptr<int2>(ml.down_win), dptr<int>(ml.parent),
            dptr<int>(ml.oct), dptr<float2>(pm.up_phase), dptr<int>(ml.th_ptr), dptr<int>(ml.th_src),
            dptr<float>(ml.th_w), dptr<int>(ml.ph_ptr), dptr<int>(ml.ph_src), dptr<float>(ml.ph_w),
            dptr<float4>(ml.down), (size_t)3 * ml.nbox * ml.K, (size_t)3 * pm.nbox * pm.K);
    }
    agg_disagg(M, false, x, nr, y, parts, st);
    c->kernel_launches += 2 * nl + 1;
    EMFA_CUDA(c, cudaGetLastError());
    return EMFA_OK;
}

// MLFMA as a Krylov operator (iteration vectors complex64, box order)
// y = P x for n_rhs vectors
static emfa_status_t sai_apply(emfa_mlfma* M, const float2* x, float2* y, int nrhs, cudaStream_t st)
{
    for (int r = 0; r < nrhs; ++r)
        k_sai_apply<<<(M->n + 255) / 256, 256, 0, st>>>(dptr<int>(M->csr_ptr), dptr<int>(M->csr_col),
                                                          dptr<float2>(M->csr_val), x + (size_t)r * M->n, M->n,
                                                          y + (size_t)r * M->n);
    M->ctx->kernel_launches += nrhs;
    EMFA_CUDA(M->ctx, cudaGetLastError());
    return EMFA_OK;
}

struct MlfmaOp : LinOp {
    emfa_mlfma* M = nullptr;
    bool pre = false;  // left-preconditioned operator P Z
    emfa_status_t apply(Ctx*, const void* X, void* Y, int nrhs, cudaStream_t st) override
    {
        if (pre) {
            // P (Z x): one right-hand side at a time through the preconditioner's scratch
            for (int r = 0; r < nrhs; ++r) {
                EMFA_TRY(mlfma_apply(M, (const float2*)X + (size_t)r * n, dptr<float2>(M->pre_tmp), 1, st));
                EMFA_TRY(sai_apply(M, dptr<float2>(M->pre_tmp), (float2*)Y + (size_t)r * n, 1, st));
            }
            return EMFA_OK;
        }
        for (int r0 = 0; r0 < nrhs; r0 += RHS_CHUNK)
            EMFA_TRY(mlfma_apply(M, (const float2*)X + (size_t)r0 * n, (float2*)Y + (size_t)r0 * n,
                                 std::min(RHS_CHUNK, nrhs - r0), st));
        return EMFA_OK;
    }
    emfa_status_t residual(Ctx* c, const double2* X, const void* B, double2* R, int nrhs, float2* xt,
                           cudaStream_t st) override
    {
        const size_t tot = (size_t)n * nrhs;
        EMFA_TRY(M->tmp_out.bytes >= sizeof(float2) * tot ? EMFA_OK : M->tmp_out.alloc(c, sizeof(float2) * tot));
        k_f64_to_f32<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(X, xt, tot);
        EMFA_TRY(apply(c, xt, M->tmp_out.ptr, nrhs, st));
        k_resid_c64<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>((const float2*)B, dptr<float2>(M->tmp_out), R, tot);
        c->kernel_launches += 2;
        return EMFA_OK;
    }
};

}  // namespace emfa

using namespace emfa;

extern "C" {

emfa_status_t emfa_mlfma_create(emfa_ctx_t* ctx, emfa_geom_t* geom, const emfa_mlfma_params_t* p, emfa_mlfma_t** out)
{
    if (!ctx || !geom || !p || !out || !(p->freq > 0) || !(p->box_threshold > 0) ||
        (p->truncation != 0 && p->truncation != 1)) {
        set_error(ctx, "emfa_mlfma_create: bad arguments");
        return EMFA_ERR_INVALID;
    }
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    emfa_mlfma_t* M = new emfa_mlfma_t();
    M->ctx = ctx;
    M->geom = geom;
    M->p = *p;
    emfa_status_t s = mlfma_build(M, ctx->stream);
    if (s != EMFA_OK) {
        delete M;
        return s;
    }
    // the operator holds its geometry (and through it the context) until it
    // is destroyed, whatever order the caller closes them in
    geom_retain(geom);
    *out = M;
    return EMFA_OK;
}

emfa_status_t emfa_mlfma_plan(const double* verts_host, int n_vert, const int* rwg_host, int n_rwg,
                              const emfa_mlfma_params_t* p, int* levels, int* level_boxes, int level_cap, int* poles,
                              int* perm)
{
    if (!verts_host || !rwg_host || !p || n_vert <= 0 || n_rwg <= 0 || !levels) return EMFA_ERR_INVALID;
    if (p->truncation != 0 && p->truncation != 1) {
        set_global_error("emfa_mlfma_plan: truncation must be 0 or 1");
        return EMFA_ERR_INVALID;
    }
    std::vector<double> v(verts_host, verts_host + 3 * (size_t)n_vert);
    std::vector<int> r(rwg_host, rwg_host + 6 * (size_t)n_rwg);
    Plan P;
    std::string err;
    if (!build_plan(v, n_vert, r, n_rwg, *p, P, err)) {
        set_global_error("emfa_mlfma_plan: " + err);
        return EMFA_ERR_INVALID;
    }
    *levels = P.L;
    if (level_boxes) {
        if (level_cap < P.L + 1) return EMFA_ERR_INVALID;
        for (int l = 0; l <= P.L; ++l) level_boxes[l] = (int)P.lb[l].size();
    }
    if (poles)
        for (size_t i = 0; i < P.poles.size(); ++i) poles[i] = P.poles[i];
    if (perm) std::copy(P.perm.begin(), P.perm.end(), perm);
    return EMFA_OK;
}

emfa_status_t emfa_mlfma_destroy(emfa_mlfma_t* M)
{
    if (!M) return EMFA_ERR_INVALID;
    cudaSetDevice(M->ctx->device);
    cudaStreamSynchronize(M->ctx->stream);
    emfa::Geom* g = M->geom;
    delete M;
    geom_release(g);
    return EMFA_OK;
}

emfa_status_t emfa_mlfma_info(const emfa_mlfma_t* M, int* levels, int* level_boxes, int* poles, size_t* near_nnz,
                              int* perm)
{
    if (!M) return EMFA_ERR_INVALID;
    if (levels) *levels = M->levels;
    if (level_boxes) std::copy(M->level_boxes.begin(), M->level_boxes.end(), level_boxes);
    if (poles) std::copy(M->poles.begin(), M->poles.end(), poles);
    if (near_nnz) *near_nnz = M->nnz;
    if (perm) std::copy(M->perm.begin(), M->perm.end(), perm);
    return EMFA_OK;
}

emfa_status_t emfa_mlfma_apply_part(emfa_mlfma_t* M, const void* x_dev, void* y_dev, int part, void* stream)
{
    if (!M || !x_dev || !y_dev || part < 0 || part > 2) return EMFA_ERR_INVALID;
    Ctx* c = M->ctx;
    EMFA_CUDA(c, cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    return mlfma_apply(M, (const float2*)x_dev, (float2*)y_dev, 1, st, part);
}

emfa_status_t emfa_mlfma_apply(emfa_mlfma_t* M, const void* x_dev, void* y_dev, int n_rhs, void* stream)
{
    if (!M || !x_dev || !y_dev || n_rhs <= 0) return EMFA_ERR_INVALID;
    Ctx* c = M->ctx;
    EMFA_CUDA(c, cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    MlfmaOp A;
    A.M = M;
    A.n = M->n;
    A.prec = EMFA_F32;
    return A.apply(c, x_dev, y_dev, n_rhs, st);
}

emfa_status_t emfa_mlfma_fill_v(emfa_mlfma_t* M, const double* angles_host, int n_inc, void* V_dev, void* stream)
{
    if (!M || !angles_host || n_inc <= 0 || !V_dev) return EMFA_ERR_INVALID;
    Ctx* c = M->ctx;
    EMFA_CUDA(c, cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    emfa_fill_params_t fp{EMFA_CFIE, EMFA_F32, M->p.freq, M->p.alpha, 0, 0, 0};
    DevBuf tmp;
    EMFA_TRY(tmp.alloc(c, sizeof(float2) * (size_t)M->n * n_inc));
    EMFA_TRY(launch_fill_v(c, M->geom, &fp, angles_host, n_inc, tmp.ptr, st));
    size_t tot = (size_t)M->n * n_inc;
    k_gather_c64<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(dptr<float2>(tmp), dptr<int>(M->perm_d), M->n, n_inc,
                                                                (float2*)V_dev);
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    return EMFA_OK;
}

emfa_status_t emfa_mlfma_solve(emfa_mlfma_t* M, const void* B_dev, int n_rhs, void* X_dev,
                               const emfa_solver_params_t* sp, emfa_solve_info_t* info, void* stream)
{
    if (!M || !B_dev || !X_dev || !sp || n_rhs <= 0 || !(sp->tol > 0)) return EMFA_ERR_INVALID;
    Ctx* c = M->ctx;
    EMFA_CUDA(c, cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    MlfmaOp A;
    A.M = M;
    A.n = M->n;
    A.prec = EMFA_F32;
    A.pre = M->precond;
    const void* B = B_dev;
    if (M->precond) {  // V <- P V (MLFMA::iterativeSolve, MLFMA.cpp:407-408)
        const size_t bytes = sizeof(float2) * (size_t)M->n * n_rhs;
        if (M->pre_b.bytes < bytes) EMFA_TRY(M->pre_b.alloc(c, bytes));
        EMFA_TRY(sai_apply(M, (const float2*)B_dev, dptr<float2>(M->pre_b), n_rhs, st));
        B = M->pre_b.ptr;
    }
    return solve_op(c, A, B, n_rhs, X_dev, sp, info, st);
}

emfa_status_t emfa_mlfma_precond_csr(const emfa_mlfma_t* M, size_t* nnz, int* ptr_host, int* col_host,
                                     void* val_host)
{
    if (!M || !nnz) return EMFA_ERR_INVALID;
    *nnz = M->precond ? M->sai_nnz : 0;
    if (!M->precond || !ptr_host) return EMFA_OK;
    Ctx* c = M->ctx;
    EMFA_CUDA(c, cudaSetDevice(c->device));
    EMFA_CUDA(c, cudaStreamSynchronize(c->stream));
    EMFA_CUDA(c, cudaMemcpy(ptr_host, M->csr_ptr.ptr, sizeof(int) * (M->n + 1), cudaMemcpyDeviceToHost));
    if (col_host) EMFA_CUDA(c, cudaMemcpy(col_host, M->csr_col.ptr, sizeof(int) * M->sai_nnz, cudaMemcpyDeviceToHost));
    if (val_host)
        EMFA_CUDA(c, cudaMemcpy(val_host, M->csr_val.ptr, sizeof(float2) * M->sai_nnz, cudaMemcpyDeviceToHost));
    return EMFA_OK;
}

emfa_status_t emfa_mlfma_precond_lists(const emfa_mlfma_t* M, int* nbox, size_t* nrows, size_t* ncols, int* rptr,
                                       int* rows, int* cptr, int* cols, int* own)
{
    if (!M || !nbox || !nrows || !ncols) return EMFA_ERR_INVALID;
    *nbox = M->precond ? (int)M->sai_own.size() : 0;
    *nrows = M->sai_rows.size();
    *ncols = M->sai_cols.size();
    if (!M->precond) return EMFA_OK;
    if (rptr) std::copy(M->sai_rptr.begin(), M->sai_rptr.end(), rptr);
    if (rows) std::copy(M->sai_rows.begin(), M->sai_rows.end(), rows);
    if (cptr) std::copy(M->sai_cptr.begin(), M->sai_cptr.end(), cptr);
    if (cols) std::copy(M->sai_cols.begin(), M->sai_cols.end(), cols);
    if (own) std::copy(M->sai_own.begin(), M->sai_own.end(), own);
    return EMFA_OK;
}

emfa_status_t emfa_mlfma_unpermute(emfa_mlfma_t* M, const void* X_box_dev, int n_rhs, void* X_rwg_dev, void* stream)
{
    if (!M || !X_box_dev || !X_rwg_dev || n_rhs <= 0) return EMFA_ERR_INVALID;
    Ctx* c = M->ctx;
    EMFA_CUDA(c, cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    size_t tot = (size_t)M->n * n_rhs;
    k_scatter_c128<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>((const double2*)X_box_dev, dptr<int>(M->perm_d),
                                                                  M->n, n_rhs, (double2*)X_rwg_dev);
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    return EMFA_OK;
}

}  // extern "C"
