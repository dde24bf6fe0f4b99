// Bistatic / monostatic RCS: far-field reduction of the surface current.
//   E_s(k_s) = sum_u I_u l_u sum_{7 pts} w rho exp(+j k k_s . r)
//   sigma = Z0^2 k^2 |0.5 k_s x (k_s x E_s)|^2 / 4 pi,  reported 10 log10
// (EMSolver/EFIE.cpp:788-832, EMSolver/CFIE.cpp:643-685, MLFMA.cpp:1573-1620).
// One CTA per (right-hand side, direction); the RWG sum is a fixed-order
// block reduction in FP64, so results are run-to-run identical.
#include "emfa_internal.cuh"
#include "emfa_math.cuh"

#include <type_traits>

namespace emfa {

// s + x with the rounding error carried in c (Kahan), FP32
__device__ __forceinline__ void kahan_add(float& s, float& c, float x)
{
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

// NT threads: 512 for FP32, three CTAs an SM at 40 registers.  The (RHS,
// direction) grid is often one CTA an incidence (monostatic: 360 CTAs on the
// dense CFIE job), so wider CTAs keep more warps an SM on the point loop:
// 160 -> 146 us there (ncu).  The FP64 path keeps 256 (at three CTAs of 512
// it would spill).
template <typename T, int NT>
__global__ void __launch_bounds__(NT, NT == 512 ? 3 : 1) k_rcs(const RwgPack<T>* __restrict__ rw, const T* __restrict__ q7, int n,
                                             const double2* __restrict__ I, const T* __restrict__ dirs, int n_dir,
                                             int per_rhs, T k, T kpi, double z0, double* __restrict__ out)
{
    const int d = blockIdx.x, a = blockIdx.y;
    const T* dp = dirs + 3 * ((size_t)(per_rhs ? a * n_dir : 0) + d);
    V3<T> ks = v3(dp[0], dp[1], dp[2]);
    double acc[6] = {0, 0, 0, 0, 0, 0};
    // FP32 geometry: each RWG's term I l E_u in FP32 and a thread's terms
    // summed with compensation, converted to FP64 once per thread (per-RWG
    // FP64 products and conversions ran on GB300's 1/64-rate FP64 pipe:
    // 215 -> 160 us on the dense CFIE job's 360 monostatic directions); the
    // current's FP64 components rounded to FP32 by integer operations.  A
    // numpy model of both sums over the 1,920-RWG sphere's 541 bistatic
    // directions differs by at most 2.5e-7 dB
    float ks32[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, kc32[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    constexpr bool F32 = std::is_same<T, float>::value;
    for (int u = threadIdx.x; u < n; u += blockDim.x) {
        const RwgPack<T>& R = rw[u];
        T ex[3] = {0, 0, 0}, ey[3] = {0, 0, 0};  // re / im of sum w rho e^{j..}
        for (int s = 0; s < 2; ++s) {
            T sgn = s == 0 ? T(1) : T(-1);
            V3<T> fv = v3(R.v[s][0], R.v[s][1], R.v[s][2]);
            const T* q = q7 + 21 * R.tri[s];
#pragma unroll
            for (int i = 0; i < 7; ++i) {
                V3<T> g = v3(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
                V3<T> rho = (g - fv) * (sgn * gauss7_weight<T>(i));
                T sn, cs;
                sincos_pi(kpi * dot(g, ks), &sn, &cs);
                ex[0] += rho.x * cs; ey[0] += rho.x * sn;
                ex[1] += rho.y * cs; ey[1] += rho.y * sn;
                ex[2] += rho.z * cs; ey[2] += rho.z * sn;
            }
        }
        double2 iu = I[(size_t)a * n + u];
        if constexpr (F32) {
            const float ir = split_f64(iu.x).x * R.len, ii = split_f64(iu.y).x * R.len;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                kahan_add(ks32[2 * c], kc32[2 * c], fmaf(ex[c], ir, -(ey[c] * ii)));
                kahan_add(ks32[2 * c + 1], kc32[2 * c + 1], fmaf(ex[c], ii, ey[c] * ir));
            }
        } else {
            double ir = iu.x * (double)R.len, ii = iu.y * (double)R.len;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                acc[2 * c] += (double)ex[c] * ir - (double)ey[c] * ii;
                acc[2 * c + 1] += (double)ex[c] * ii + (double)ey[c] * ir;
            }
        }
    }
    if constexpr (F32) {
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[c] = (double)ks32[c] - (double)kc32[c];
    }
    __shared__ double red[6][NT];
    for (int c = 0; c < 6; ++c) red[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int c = 0; c < 6; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double E[3][2] = {{red[0][0], red[1][0]}, {red[2][0], red[3][0]}, {red[4][0], red[5][0]}};
        double kx = ks.x, ky = ks.y, kz = ks.z;
        double es2 = 0.0;
        // es = 0.5 k x (k x E), per real/imag part
        for (int part = 0; part < 2; ++part) {
            double ex = E[0][part], ey = E[1][part], ez = E[2][part];
            double cx1 = ky * ez - kz * ey, cy1 = kz * ex - kx * ez, cz1 = kx * ey - ky * ex;
            double x = 0.5 * (ky * cz1 - kz * cy1), y = 0.5 * (kz * cx1 - kx * cz1), z = 0.5 * (kx * cy1 - ky * cx1);
            es2 += x * x + y * y + z * z;
        }
        double kk = (double)k;
        double pi = 3.14159265358979323846;
        double sigma = z0 * z0 * kk * kk * es2 / (4.0 * pi);
        out[(size_t)a * n_dir + d] = 10.0 * log10(sigma);
    }
}

template <typename T>
static emfa_status_t rcs_t(Ctx* c, Geom* g, GeomDev<T>& gd, const emfa_fill_params_t* p, const void* I, int n_rhs,
                           const double* dirs, int n_dir, int per_rhs, double* out_host, cudaStream_t st)
{
    size_t nd = (size_t)(per_rhs ? n_rhs : 1) * n_dir;
    std::vector<T> dh(3 * nd);
    for (size_t i = 0; i < 3 * nd; ++i) dh[i] = (T)dirs[i];
    DevBuf dd, od;
    EMFA_TRY(dd.alloc(c, sizeof(T) * dh.size()));
    EMFA_TRY(od.alloc(c, sizeof(double) * (size_t)n_rhs * n_dir));
    EMFA_CUDA(c, cudaMemcpyAsync(dd.ptr, dh.data(), dd.bytes, cudaMemcpyHostToDevice, st));
    T k = Phys<T>::wavenumber(p->freq);
    dim3 grd(n_dir, n_rhs);
    constexpr int NT = std::is_same<T, float>::value ? 512 : 256;
    k_rcs<T, NT><<<grd, NT, 0, st>>>(dptr<RwgPack<T>>(gd.rwg), dptr<T>(gd.tri_q7), g->n, (const double2*)I,
                                  dptr<T>(dd), n_dir, per_rhs, k, k / Phys<T>::pi(), (double)Phys<T>::z0(),
                                  dptr<double>(od));
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    EMFA_CUDA(c, cudaMemcpyAsync(out_host, od.ptr, od.bytes, cudaMemcpyDeviceToHost, st));
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    return EMFA_OK;
}

emfa_status_t launch_rcs(Ctx* c, Geom* g, const emfa_fill_params_t* p, const void* I, int n_rhs, const double* dirs,
                         int n_dir, int per_rhs, double* out, cudaStream_t st)
{
    if (p->precision == EMFA_F64) {
        EMFA_TRY(geom_prepare_f64(g, st));
        return rcs_t<double>(c, g, g->g64, p, I, n_rhs, dirs, n_dir, per_rhs, out, st);
    }
    EMFA_TRY(geom_prepare_f32(g, st));
    return rcs_t<float>(c, g, g->g32, p, I, n_rhs, dirs, n_dir, per_rhs, out, st);
}

}  // namespace emfa

using namespace emfa;

extern "C" emfa_status_t emfa_rcs(emfa_ctx_t* ctx, emfa_geom_t* geom, const emfa_fill_params_t* p, const void* I_dev,
                                  int n_rhs, const double* dirs_host, int n_dir, int per_rhs_dirs, double* out_host,
                                  void* stream)
{
    if (!ctx || !geom || !p || !I_dev || !dirs_host || !out_host || n_rhs <= 0 || n_dir <= 0 || n_rhs > 65535 ||
        n_dir > (1 << 30)) {
        set_error(ctx, "emfa_rcs: bad arguments");
        return EMFA_ERR_INVALID;
    }
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return launch_rcs(ctx, geom, p, I_dev, n_rhs, dirs_host, n_dir, per_rhs_dirs, out_host, st);
}
