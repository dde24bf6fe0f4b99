// Impedance-matrix fill (EFIE and CFIE) and plane-wave excitation.
//
// Z(f, s) = l_f l_s * sum over the four (field triangle a, source triangle b)
// pairs of RWG f and RWG s, with sign s_a s_b (+ side +1, - side -1):
//   regular pairs: 3x3-point Gauss rule with G = exp(-jkR)/R
//     (EMSolver/EFIE.cpp:139-160, EMSolver/Miscellaneous.cpp:6-30)
//   same-triangle pairs: singularity-extracted self terms
//     (EMSolver/EFIE.cpp:231-542, EMSolver/Miscellaneous.cpp:32-77)
// The self terms depend only on (triangle, field free vertex, source free
// vertex) and the frequency, so they are tabulated once per fill in FP64
// (9 entries per triangle) and looked up by the entry kernel; the regular
// pairs run in the fill precision (FP32 for the mixed path, FP64 plain).
#include "emfa_internal.cuh"
#include "emfa_math.cuh"
#include "fill_entry.cuh"

namespace emfa {

// ---------------------------------------------------------------------------
// singular self terms, FP64, one thread per (triangle, field corner, source corner)
// ---------------------------------------------------------------------------
struct SingConst {
    double k, inv_k2, w, alpha, z0, pi;
    double sig_re, sig_im;
    int cfie;
};

// EFIE self term without the j k Z0 / 4 pi prefactor, unsigned (field and
// source signs +1).  proj selects the projected edge-distance form of
// eZ{pm,mp,mm}Singular (EFIE.cpp:344-368) instead of eZppSingular's direct
// form (EFIE.cpp:260-283); both are the same integral.
__device__ static Cx<double> efie_self(const V3<double>* v, V3<double> vf, V3<double> vs, const SingConst& c,
                                       bool proj)
{
    V3<double> g[3];
    gauss3(v[0], v[1], v[2], g);
    double S = tri_area(v[0], v[1], v[2]);
    double k = c.k;
    Cx<double> ze1 = cx(0.0, 0.0);
    double ze2 = 0.0;
    V3<double> n = normalized(cross(v[1] - v[0], v[2] - v[0]));
    for (int p = 0; p < 3; ++p) {
        V3<double> rf = g[p] - vf;
        for (int q = 0; q < 3; ++q) {
            V3<double> rs = g[q] - vs;
            double r = norm(g[p] - g[q]);
            Cx<double> coff = cx(-0.5 * k * k * r, (k / 6.0) * (k * k * r * r - 6.0));
            double s = c.w * c.w * (0.25 * dot(rf, rs) - c.inv_k2);
            ze1 = ze1 + coff * s;
        }
        double Is2 = 0.0;
        V3<double> Is1 = v3(0.0, 0.0, 0.0);
        V3<double> rou = g[p] - n * dot(n, g[p]);
        for (int i = 0; i < 3; ++i) {
            V3<double> a = v[(i + 1) % 3], b = v[i];
            V3<double> li = a - b;
            V3<double> rou_p = a - n * dot(n, a);
            V3<double> rou_m = b - n * dot(n, b);
            V3<double> ui = normalized(cross(li, n));
            V3<double> l1 = normalized(li);
            double p0 = fabs(dot(b - g[p], ui));
            double d = dot(g[p] - b, n);
            double lp, lm, rp, rm;
            if (!proj) {
                lp = dot(a - g[p], l1);
                lm = dot(b - g[p], l1);
                rp = norm(g[p] - a);
                rm = norm(g[p] - b);
            } else {
                lp = dot(rou_p - rou, l1);
                lm = dot(rou_m - rou, l1);
                rp = sqrt(p0 * p0 + d * d + lp * lp);
                rm = sqrt(p0 * p0 + d * d + lm * lm);
            }
            if (p0 < 1e-10) continue;
            V3<double> pi = normalized((rou_p - rou) - l1 * lp);
            double r02 = p0 * p0 + d * d;
            double lg = log((rp + lp) / (rm + lm));
            Is1 = Is1 + (ui * 0.5) * (r02 * lg + lp * rp - lm * rm);
            double ad = fabs(d);
            Is2 += dot(pi, ui) * (p0 * lg - ad * (atan((p0 * lp) / (r02 + ad * rp)) - atan((p0 * lm) / (r02 + ad * rm))));
        }
        ze2 += c.w * (0.25 * dot(rf, Is1 + (g[p] - vs) * Is2) - Is2 * c.inv_k2);
    }
    return cx(ze1.re + ze2 / S, ze1.im);
}

// EFIE surface-impedance term (EFIE.cpp:297-306), identical for all four
// sign combinations in the reference.
__device__ static Cx<double> efie_sigma(const V3<double>* v, V3<double> vf, V3<double> vs, const SingConst& c)
{
    if (sqrt(c.sig_re * c.sig_re + c.sig_im * c.sig_im) <= 1e-8) return cx(0.0, 0.0);
    V3<double> g[3];
    gauss3(v[0], v[1], v[2], g);
    double S = tri_area(v[0], v[1], v[2]);
    double acc = 0.0;
    for (int i = 0; i < 3; ++i) acc += dot((g[i] - vf) * c.w, g[i] - vs);
    // pi sigma / (S j k Z0) = -j pi sigma / (S k Z0)
    double den = S * c.k * c.z0;
    return cx(c.pi * c.sig_im / den * acc, -c.pi * c.sig_re / den * acc);
}

// CFIE self term (Miscellaneous.cpp:32-77), unsigned, complete with the
// alpha / (1 - alpha) combination.  The edge-log term reuses the source
// rho of the last inner quadrature point, as the reference does.
__device__ static Cx<double> cfie_self(const V3<double>* v, V3<double> vf, V3<double> vs, const SingConst& c)
{
    V3<double> g[3];
    gauss3(v[0], v[1], v[2], g);
    double area = tri_area(v[0], v[1], v[2]);
    double k = c.k;
    Cx<double> ze1 = cx(0.0, 0.0);
    double ze2 = 0.0, zm = 0.0;
    for (int p = 0; p < 3; ++p) {
        V3<double> rf = g[p] - vf;
        V3<double> rs = v3(0.0, 0.0, 0.0);
        for (int q = 0; q < 3; ++q) {
            rs = g[q] - vs;
            double r = norm(g[p] - g[q]);
            Cx<double> coff = cx(-0.5 * k * k * r, (k / 6.0) * (k * k * r * r - 6.0));
            ze1 = ze1 + coff * (c.w * c.w * (0.25 * dot(rf, rs) - c.inv_k2));
        }
        for (int i = 0; i < 3; ++i) {
            V3<double> a = v[(i + 1) % 3], b = v[i];
            V3<double> L = normalized(a - b);
            double Lp = dot(a - g[p], L), Lm = dot(b - g[p], L);
            double Rp = norm(a - g[p]), Rm = norm(b - g[p]);
            V3<double> sj0 = b + L * dot(g[p] - b, L);
            double P0 = norm(sj0 - g[p]);
            if (P0 > 1e-10) ze2 += c.w * (0.25 * dot(rf, rs) - c.inv_k2) * P0 * log((Rp + Lp) / (Rm + Lm));
        }
        zm += c.w * dot(g[p] - vf, g[p] - vs);
    }
    double kz = k * c.z0 / (4.0 * c.pi);
    // j kz (ze1 + ze2/area)
    double er = ze1.re + ze2 / area, ei = ze1.im;
    Cx<double> ze = cx(-kz * ei, kz * er);
    double zmv = zm / (8.0 * area);
    return cx(c.alpha * ze.re + (1.0 - c.alpha) * c.z0 * zmv, c.alpha * ze.im);
}

// table layout per (t, ef, es): EFIE {A_direct, A_proj, B_sigma}, CFIE {S}
__global__ void k_singular_table(const double* __restrict__ vd, const int* __restrict__ tris, int nt, SingConst c,
                                 double2* __restrict__ tab)
{
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= 9 * nt) return;
    int t = id / 9, ef = (id % 9) / 3, es = id % 3;
    V3<double> v[3];
    for (int j = 0; j < 3; ++j) {
        int i = tris[3 * t + j];
        v[j] = v3(vd[3 * i], vd[3 * i + 1], vd[3 * i + 2]);
    }
    V3<double> vf = v[ef], vs = v[es];
    if (c.cfie) {
        Cx<double> s = cfie_self(v, vf, vs, c);
        tab[id] = make_double2(s.re, s.im);
    } else {
        Cx<double> a = efie_self(v, vf, vs, c, false);
        Cx<double> b = efie_self(v, vf, vs, c, true);
        Cx<double> sg = efie_sigma(v, vf, vs, c);
        tab[3 * id] = make_double2(a.re, a.im);
        tab[3 * id + 1] = make_double2(b.re, b.im);
        tab[3 * id + 2] = make_double2(sg.re, sg.im);
    }
}

// ---------------------------------------------------------------------------
// entry kernel: one thread per Z(f, s); a warp runs 32 consecutive s of one f
// ---------------------------------------------------------------------------
template <typename T, bool CFIE>
__global__ void __launch_bounds__(256) k_fill_z(const RwgPack<T>* __restrict__ rw, int n, FillConst<T> c,
                                                const double2* __restrict__ sing, Cx<T>* __restrict__ Z, size_t ldz)
{
    int s = blockIdx.x * 32 + threadIdx.x;
    int f = blockIdx.y * blockDim.y + threadIdx.y;
    if (s >= n || f >= n) return;
    Z[(size_t)f * ldz + s] = z_entry<T, CFIE>(rw[f], rw[s], c, sing);
}

// ---------------------------------------------------------------------------
// excitation: one thread per (incidence, RWG)
// ---------------------------------------------------------------------------
template <typename T, bool CFIE>
__global__ void k_fill_v(const RwgPack<T>* __restrict__ rw, const T* __restrict__ q7, const T* __restrict__ inc,
                         int n, int n_inc, T k, T kpi, T alpha, Cx<T>* __restrict__ V)
{
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    int a = blockIdx.y;
    if (u >= n || a >= n_inc) return;
    const RwgPack<T>& R = rw[u];
    const T* ic = inc + 9 * a;
    V3<T> kk = v3(ic[0], ic[1], ic[2]), ee = v3(ic[3], ic[4], ic[5]), hh = v3(ic[6], ic[7], ic[8]);
    Cx<T> ve = cx(T(0), T(0)), vm = cx(T(0), T(0));
    for (int s = 0; s < 2; ++s) {
        T sgn = s == 0 ? T(1) : T(-1);
        V3<T> fv = v3(R.v[s][0], R.v[s][1], R.v[s][2]);
        if (!CFIE) {
            // EFIE::eVKernel (EFIE.cpp:568-601), 7-point rule
            const T* q = q7 + 21 * R.tri[s];
            for (int i = 0; i < 7; ++i) {
                V3<T> g = v3(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
                V3<T> rho = (g - fv) * sgn;
                T sn, cs;
                sincos_pi(kpi * dot(g, kk), &sn, &cs);
                T w = gauss7_weight<T>(i) * dot(rho, ee);
                ve.re += w * cs;
                ve.im -= w * sn;
            }
        } else {
            // cfieVKernel (Miscellaneous.cpp:152-189), 3-point rule
            V3<T> nn = v3(R.n[s][0], R.n[s][1], R.n[s][2]);
            V3<T> nh = cross(nn, hh);
            T w3 = T(1) / T(3);
            for (int i = 0; i < 3; ++i) {
                V3<T> g = v3(R.q3[s][i][0], R.q3[s][i][1], R.q3[s][i][2]);
                V3<T> rho = (g - fv) * sgn;
                T sn, cs;
                sincos_pi(kpi * dot(g, kk), &sn, &cs);
                T we = w3 * dot(rho, ee), wm = w3 * dot(rho, nh);
                ve.re += we * cs;
                ve.im -= we * sn;
                vm.re += wm * cs;
                vm.im -= wm * sn;
            }
        }
    }
    Cx<T> v = CFIE ? cx(alpha * ve.re + (T(1) - alpha) * vm.re, alpha * ve.im + (T(1) - alpha) * vm.im) : ve;
    T h = T(0.5) * R.len;
    V[(size_t)a * n + u] = cx(v.re * h, v.im * h);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename T>
static emfa_status_t fill_z_t(Ctx* c, Geom* g, GeomDev<T>& d, const emfa_fill_params_t* p, void* Z, size_t ldz,
                              cudaStream_t st)
{
    const bool cfie = p->kind == EMFA_CFIE;
    // singular table (FP64), 9 (CFIE) or 27 (EFIE) double2 per triangle
    void* tab = nullptr;
    EMFA_TRY(ctx_workspace(c, WS_FILL, sizeof(double2) * (size_t)g->nt * (cfie ? 9 : 27), &tab));
    EMFA_TRY(build_singular_table(c, g, p, (double2*)tab, st));
    FillConst<T> fc = make_fill_const<T>(p);
    dim3 blk(32, 8);
    dim3 grd((g->n + 31) / 32, (g->n + 7) / 8);
    {
        TimedLaunch tl(c, KT_FILL_Z, st, (double)g->n * g->n);
        if (cfie)
            k_fill_z<T, true><<<grd, blk, 0, st>>>(dptr<RwgPack<T>>(d.rwg), g->n, fc, (const double2*)tab,
                                                   reinterpret_cast<Cx<T>*>(Z), ldz);
        else
            k_fill_z<T, false><<<grd, blk, 0, st>>>(dptr<RwgPack<T>>(d.rwg), g->n, fc, (const double2*)tab,
                                                    reinterpret_cast<Cx<T>*>(Z), ldz);
    }
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    return EMFA_OK;
}

emfa_status_t build_singular_table(Ctx* c, Geom* g, const emfa_fill_params_t* p, double2* tab, cudaStream_t st)
{
    const bool cfie = p->kind == EMFA_CFIE;
    if (p->precision == EMFA_F64)
        EMFA_TRY(geom_prepare_f64(g, st));
    else
        EMFA_TRY(geom_prepare_f32(g, st));
    // the table's vertices and k: the fill precision's k, in FP64 arithmetic
    DevBuf vd;
    EMFA_TRY(vd.alloc(c, sizeof(double) * 3 * (size_t)g->nv));
    EMFA_CUDA(c, cudaMemcpyAsync(vd.ptr, g->verts.data(), vd.bytes, cudaMemcpyHostToDevice, st));
    SingConst sc;
    sc.k = p->precision == EMFA_F64 ? Phys<double>::wavenumber(p->freq) : (double)Phys<float>::wavenumber(p->freq);
    sc.inv_k2 = 1.0 / (sc.k * sc.k);
    sc.w = 1.0 / 3.0;
    sc.alpha = p->alpha;
    sc.pi = 3.14159265358979323846;
    sc.z0 = 120.0 * sc.pi;
    sc.sig_re = p->sigma_re;
    sc.sig_im = p->sigma_im;
    sc.cfie = cfie;
    const int* tris = p->precision == EMFA_F64 ? dptr<int>(g->g64.tris) : dptr<int>(g->g32.tris);
    k_singular_table<<<(9 * g->nt + 127) / 128, 128, 0, st>>>(dptr<double>(vd), tris, g->nt, sc, tab);
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    EMFA_CUDA(c, cudaStreamSynchronize(st));  // vd is released on return
    return EMFA_OK;
}

emfa_status_t launch_fill_z(Ctx* c, Geom* g, const emfa_fill_params_t* p, void* Z, size_t ldz, cudaStream_t st)
{
    if (p->precision == EMFA_F64) {
        EMFA_TRY(geom_prepare_f64(g, st));
        return fill_z_t<double>(c, g, g->g64, p, Z, ldz, st);
    }
    EMFA_TRY(geom_prepare_f32(g, st));
    return fill_z_t<float>(c, g, g->g32, p, Z, ldz, st);
}

template <typename T>
static emfa_status_t fill_v_t(Ctx* c, Geom* g, GeomDev<T>& d, const emfa_fill_params_t* p, const double* angles,
                              int n_inc, void* V, cudaStream_t st)
{
    std::vector<T> inc((size_t)9 * n_inc);
    for (int a = 0; a < n_inc; ++a)
        incidence_vectors<T>(angles[3 * a], angles[3 * a + 1], angles[3 * a + 2], inc.data() + 9 * a);
    DevBuf dinc;
    EMFA_TRY(dinc.alloc(c, sizeof(T) * inc.size()));
    EMFA_CUDA(c, cudaMemcpyAsync(dinc.ptr, inc.data(), dinc.bytes, cudaMemcpyHostToDevice, st));
    T k = Phys<T>::wavenumber(p->freq);
    T kpi = k / Phys<T>::pi();
    dim3 grd((g->n + 127) / 128, n_inc);
    if (p->kind == EMFA_CFIE)
        k_fill_v<T, true><<<grd, 128, 0, st>>>(dptr<RwgPack<T>>(d.rwg), dptr<T>(d.tri_q7), dptr<T>(dinc), g->n, n_inc,
                                               k, kpi, (T)p->alpha, reinterpret_cast<Cx<T>*>(V));
    else
        k_fill_v<T, false><<<grd, 128, 0, st>>>(dptr<RwgPack<T>>(d.rwg), dptr<T>(d.tri_q7), dptr<T>(dinc), g->n,
                                                n_inc, k, kpi, (T)p->alpha, reinterpret_cast<Cx<T>*>(V));
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    return EMFA_OK;
}

emfa_status_t launch_fill_v(Ctx* c, Geom* g, const emfa_fill_params_t* p, const double* angles, int n_inc,
                            void* V, cudaStream_t st)
{
    if (p->precision == EMFA_F64) {
        EMFA_TRY(geom_prepare_f64(g, st));
        return fill_v_t<double>(c, g, g->g64, p, angles, n_inc, V, st);
    }
    EMFA_TRY(geom_prepare_f32(g, st));
    return fill_v_t<float>(c, g, g->g32, p, angles, n_inc, V, st);
}

}  // namespace emfa

using namespace emfa;

static emfa_status_t check_fill(emfa_ctx_t* ctx, emfa_geom_t* geom, const emfa_fill_params_t* p)
{
    if (!ctx || !geom || !p) return EMFA_ERR_INVALID;
    if (p->kind != EMFA_EFIE && p->kind != EMFA_CFIE) {
        set_error(ctx, "fill: kind must be EMFA_EFIE or EMFA_CFIE");
        return EMFA_ERR_INVALID;
    }
    if (p->precision != EMFA_F32 && p->precision != EMFA_F64) {
        set_error(ctx, "fill: precision must be EMFA_F32 or EMFA_F64");
        return EMFA_ERR_INVALID;
    }
    if (!(p->freq > 0)) {
        set_error(ctx, "fill: frequency must be positive");
        return EMFA_ERR_INVALID;
    }
    if (p->edm_mode < 0 || p->edm_mode > 2) {
        set_error(ctx, "fill: edm_mode must be 0, 1 or 2");
        return EMFA_ERR_INVALID;
    }
    return EMFA_OK;
}

extern "C" {

emfa_status_t emfa_fill_z(emfa_ctx_t* ctx, emfa_geom_t* geom, const emfa_fill_params_t* p, void* Z_dev, size_t ldz,
                          void* stream)
{
    EMFA_TRY(check_fill(ctx, geom, p));
    if (!Z_dev || ldz < (size_t)geom->n) {
        set_error(ctx, "emfa_fill_z: null matrix or ldz < n");
        return EMFA_ERR_INVALID;
    }
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return launch_fill_z(ctx, geom, p, Z_dev, ldz, st);
}

emfa_status_t emfa_fill_v(emfa_ctx_t* ctx, emfa_geom_t* geom, const emfa_fill_params_t* p, const double* angles_host,
                          int n_inc, void* V_dev, void* stream)
{
    EMFA_TRY(check_fill(ctx, geom, p));
    if (!angles_host || n_inc <= 0 || n_inc > 65535 || !V_dev) {
        set_error(ctx, "emfa_fill_v: bad incidence list or output");
        return EMFA_ERR_INVALID;
    }
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return launch_fill_v(ctx, geom, p, angles_host, n_inc, V_dev, st);
}

}  // extern "C"
