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
// FP32 entries come from tiled kernels (k_fill_tile: the kernel values of a
// 16 x 16 block's triangle pairs staged once); the EFIE one, whose regular
// part is symmetric, fills the upper triangle of tiles and mirrors it
// (k_fill_tile_sym); the CFIE one fills a tile and its mirror from the same
// staged values, the EFIE part once for both (k_fill_tile_cfie_sym).
#include "emfa_internal.cuh"
#include "emfa_math.cuh"
#include "fill_entry.cuh"

#include <algorithm>
#include <type_traits>
#include <vector>

namespace emfa {

// ---------------------------------------------------------------------------
// singular self terms, FP64, one thread per (triangle, field corner, source
// corner); for EFIE the triangle's edge integrals are evaluated once first
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
// The edge integrals of the singular EFIE term at quadrature point p of the
// triangle (Is1, a vector, and Is2), with the points' distances taken
// directly (proj false) or through their projections on the triangle's
// plane (proj true): they depend on neither RWG, so one evaluation serves
// the triangle's 9 (test edge, source edge) pairs.
__device__ static void efie_edge_integrals(const V3<double>* v, int p, bool proj, V3<double>* Is1_out,
                                           double* Is2_out)
{
    V3<double> g[3];
    gauss3(v[0], v[1], v[2], g);
    V3<double> n = normalized(cross(v[1] - v[0], v[2] - v[0]));
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
    *Is1_out = Is1;
    *Is2_out = Is2;
}

// EFIE self term (EFIE.cpp:139-296) of one (test edge, source edge) pair from
// the triangle's edge integrals Is[p] = (Is1, Is2) of one variant: the
// regular part over the 3 x 3 point pairs, then the singular part point by
// point, in the order of the reference's loops.
__device__ static Cx<double> efie_self(const V3<double>* v, V3<double> vf, V3<double> vs, const SingConst& c,
                                       const double (*Is)[4])
{
    V3<double> g[3];
    gauss3(v[0], v[1], v[2], g);
    double S = tri_area(v[0], v[1], v[2]);
    double k = c.k;
    Cx<double> ze1 = cx(0.0, 0.0);
    double ze2 = 0.0;
    for (int p = 0; p < 3; ++p) {
        V3<double> rf = g[p] - vf;
        for (int q = 0; q < 3; ++q) {
            V3<double> rs = g[q] - vs;
            double r = norm(g[p] - g[q]);
            Cx<double> coff = cx(-0.5 * k * k * r, (k / 6.0) * (k * k * r * r - 6.0));
            double s = c.w * c.w * (0.25 * dot(rf, rs) - c.inv_k2);
            ze1 = ze1 + coff * s;
        }
        const V3<double> Is1 = v3(Is[p][0], Is[p][1], Is[p][2]);
        const double Is2 = Is[p][3];
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

// table layout per (t, ef, es): EFIE {A_direct, A_proj, B_sigma}, CFIE {S}.
// A CTA of SING_TRIS triangles x 9 (ef, es) threads; for EFIE, 6 threads of
// each triangle first evaluate its edge integrals (3 points x 2 variants).
constexpr int SING_TRIS = 14;
__global__ void __launch_bounds__(9 * SING_TRIS) k_singular_table(const double* __restrict__ vd,
                                                                  const int* __restrict__ tris, int nt,
                                                                  SingConst c, double2* __restrict__ tab)
{
    __shared__ double sIs[SING_TRIS][2][3][4];  // [triangle][variant][point][Is1 xyz, Is2]
    const int tl = threadIdx.x / 9, combo = threadIdx.x % 9;
    const int t = blockIdx.x * SING_TRIS + tl;
    const bool valid = t < nt;
    V3<double> v[3];
    if (valid)
        for (int j = 0; j < 3; ++j) {
            int i = tris[3 * t + j];
            v[j] = v3(vd[3 * i], vd[3 * i + 1], vd[3 * i + 2]);
        }
    if (!c.cfie) {
        if (valid && combo < 6) {
            V3<double> Is1;
            double Is2;
            efie_edge_integrals(v, combo % 3, combo >= 3, &Is1, &Is2);
            double* o = sIs[tl][combo / 3][combo % 3];
            o[0] = Is1.x;
            o[1] = Is1.y;
            o[2] = Is1.z;
            o[3] = Is2;
        }
        __syncthreads();
    }
    if (!valid) return;
    const int id = 9 * t + combo, ef = combo / 3, es = combo % 3;
    V3<double> vf = v[ef], vs = v[es];
    if (c.cfie) {
        Cx<double> s = cfie_self(v, vf, vs, c);
        tab[id] = make_double2(s.re, s.im);
    } else {
        Cx<double> a = efie_self(v, vf, vs, c, sIs[tl][0]);
        Cx<double> b = efie_self(v, vf, vs, c, sIs[tl][1]);
        Cx<double> sg = efie_sigma(v, vf, vs, c);
        tab[3 * id] = make_double2(a.re, a.im);
        tab[3 * id + 1] = make_double2(b.re, b.im);
        tab[3 * id + 2] = make_double2(sg.re, sg.im);
    }
}

// ---------------------------------------------------------------------------
// The configuration's discretisation (EMFA_DISC_CONFIG, EFIE): 7 x 7-point
// regular pairs, and singularity extraction on self AND edge-adjacent
// triangle pairs, where the reference (Q2) extracts on self pairs only
// (EMSolver/EFIE.cpp:655-662) and uses 3 x 3 points elsewhere.
//
// For a singular pair (field triangle Tf, source triangle Ts) and field /
// source free vertices vf, vs, with G = exp(-jkR)/R = 1/R + Gs(R):
//   smooth   sum_p sum_q w_p w_q [(P_p - vf).(Q_q - vs)/4 - 1/k^2] Gs(R_pq),
//            Gs(R) = (exp(-jkR) - 1)/R = (-2 sin^2(kR/2) - j sin kR)/R,
//            Gs(0) = -jk
//   singular sum_p w_p [(P_p - vf).(I_rho(P_p) + (rho_p - vs) I_1(P_p))/4
//                       - I_1(P_p)/k^2] / A_s
// with I_1(r) = int_Ts 1/R dS', I_rho(r) = int_Ts (rho' - rho)/R dS' (rho the
// projection of r on the plane of Ts) in closed form for any r, on or off
// the plane (Wilton, Rao, Glisson, Schaubert, Al-Bundak and Butler, IEEE
// Trans. Antennas Propag. 32 (1984) 276-281, eqs. for the scalar and vector
// potential integrals).  w are the reference's 7-point weights (sum 1), so
// the value is in the units of the regular sums: the entry is
// j k Z0 / 4pi l_f l_s sum over the RWGs' four triangle pairs.
// ---------------------------------------------------------------------------
// ln((R+ + l+) / (R- + l-)) without the cancellation of R + l for l < 0:
// there R + l = R0^2 / (R - l)
__device__ static double log_ratio(double lp, double rp, double lm, double rm, double r02)
{
    const double a = lp >= 0 ? rp + lp : r02 / (rp - lp);
    const double b = lm >= 0 ? rm + lm : r02 / (rm - lm);
    return log(a / b);
}

__device__ void potential_integrals(const V3<double>* v, V3<double> r, double* I1_out, V3<double>* Irho_out)
{
    const V3<double> n = normalized(cross(v[1] - v[0], v[2] - v[0]));
    const double h = dot(r - v[0], n), ah = fabs(h);
    const V3<double> rho = r - n * h;
    double I1 = 0.0;
    V3<double> Ir = v3(0.0, 0.0, 0.0);
    for (int i = 0; i < 3; ++i) {
        const V3<double> b = v[i], a = v[(i + 1) % 3];
        const V3<double> l = normalized(a - b);
        const V3<double> u = cross(l, n);  // in-plane, pointing out of the triangle
        const double lp = dot(a - rho, l), lm = dot(b - rho, l);
        const double t = dot(b - rho, u);  // signed distance of rho from the edge's line
        const double p0 = fabs(t);
        const double r02 = p0 * p0 + h * h;
        const double rp = sqrt(r02 + lp * lp), rm = sqrt(r02 + lm * lm);
        const double lg = r02 > 0 ? log_ratio(lp, rp, lm, rm, r02) : 0.0;
        Ir = Ir + u * (0.5 * (r02 * lg + lp * rp - lm * rm));
        if (p0 > 0) {
            const double sg = t > 0 ? 1.0 : -1.0;
            I1 += sg * (p0 * lg - ah * (atan(p0 * lp / (r02 + ah * rp)) - atan(p0 * lm / (r02 + ah * rm))));
        }
    }
    *I1_out = I1;
    *Irho_out = Ir;
}

// one configuration-table value (unsigned), FP64
__device__ static Cx<double> efie_cfg_pair(const V3<double>* tf, const V3<double>* ts, V3<double> vf, V3<double> vs,
                                           bool self, const SingConst& c)
{
    V3<double> P[7], Q[7];
    gauss7(tf[0], tf[1], tf[2], P);
    gauss7(ts[0], ts[1], ts[2], Q);
    const double As = tri_area(ts[0], ts[1], ts[2]);
    const V3<double> ns = normalized(cross(ts[1] - ts[0], ts[2] - ts[0]));
    double zr = 0.0, zi = 0.0, sing = 0.0;
    for (int p = 0; p < 7; ++p) {
        const double wp = gauss7_weight<double>(p);
        const V3<double> rf = P[p] - vf;
        for (int q = 0; q < 7; ++q) {
            const double wq = gauss7_weight<double>(q);
            const double R = norm(P[p] - Q[q]);
            const double e = wp * wq * (0.25 * dot(rf, Q[q] - vs) - c.inv_k2);
            if (R > 0) {
                double sn, cs;
                sincos(0.5 * c.k * R, &sn, &cs);
                zr += e * (-2.0 * sn * sn / R);
                zi += e * (-2.0 * sn * cs / R);
            } else {
                zi += e * (-c.k);
            }
        }
        double I1;
        V3<double> Ir;
        potential_integrals(ts, P[p], &I1, &Ir);
        const V3<double> rho = P[p] - ns * dot(P[p] - ts[0], ns);
        sing += wp * (0.25 * dot(rf, Ir + (rho - vs) * I1) - I1 * c.inv_k2);
    }
    zr += sing / As;
    if (self && sqrt(c.sig_re * c.sig_re + c.sig_im * c.sig_im) > 1e-8) {
        // surface-impedance term (EFIE.cpp:297-306) with the 7-point rule
        double acc = 0.0;
        for (int i = 0; i < 7; ++i) acc += gauss7_weight<double>(i) * dot(P[i] - vf, P[i] - vs);
        const double den = As * c.k * c.z0;
        zr += c.pi * c.sig_im / den * acc;
        zi -= c.pi * c.sig_re / den * acc;
    }
    return cx(zr, zi);
}

// table: per triangle t, 4 slots (0 the triangle itself, 1..3 its edge
// neighbours in nbr order) x 9 (field corner, source corner); a thread per
// value
__global__ void __launch_bounds__(144) k_config_table(const double* __restrict__ vd, const int* __restrict__ tris,
                                                      const int* __restrict__ nbr, int nt, SingConst c,
                                                      double2* __restrict__ tab)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= 36 * nt) return;
    const int t = id / 36, slot = (id / 9) % 4, ef = (id / 3) % 3, es = id % 3;
    const int s = slot == 0 ? t : nbr[3 * t + slot - 1];
    if (s < 0) {
        tab[id] = make_double2(0.0, 0.0);
        return;
    }
    V3<double> tf[3], ts[3];
    for (int j = 0; j < 3; ++j) {
        int a = tris[3 * t + j], b = tris[3 * s + j];
        tf[j] = v3(vd[3 * a], vd[3 * a + 1], vd[3 * a + 2]);
        ts[j] = v3(vd[3 * b], vd[3 * b + 1], vd[3 * b + 2]);
    }
    const Cx<double> z = efie_cfg_pair(tf, ts, tf[ef], ts[es], slot == 0, c);
    tab[id] = make_double2(z.re, z.im);
}

// one entry in the configuration's discretisation (EFIE): the far-pair
// branch as z_entry; pairs of one triangle or of edge neighbours from the
// table, the others by the 7 x 7-point rule in T
template <typename T>
__device__ __forceinline__ Cx<T> z_entry_cfg(const RwgPack<T>& F, const RwgPack<T>& S, const FillConst<T>& c,
                                             const double2* __restrict__ tab, const int* __restrict__ nbr,
                                             const T* __restrict__ q7)
{
    if (c.edm_mode != 2) {
        V3<T> fc = divr(v3(F.cen[0][0], F.cen[0][1], F.cen[0][2]) + v3(F.cen[1][0], F.cen[1][1], F.cen[1][2]), T(2));
        V3<T> sc = divr(v3(S.cen[0][0], S.cen[0][1], S.cen[0][2]) + v3(S.cen[1][0], S.cen[1][1], S.cen[1][2]), T(2));
        if (norm(fc - sc) > c.thr_edm) return c.edm_mode == 1 ? edm_value(F, S, c) : cx(T(0), T(0));
    }
    T zr = 0, zi = 0;
    double sr = 0.0, si = 0.0;
#pragma unroll 1
    for (int a = 0; a < 2; ++a) {
        const int tf = F.tri[a];
        const T* Pp = q7 + (size_t)21 * tf;
        const V3<T> vf = v3(F.v[a][0], F.v[a][1], F.v[a][2]);
#pragma unroll 1
        for (int b = 0; b < 2; ++b) {
            const T sgn = (a == b) ? T(1) : T(-1);
            const int ts = S.tri[b];
            const int slot = ts == tf ? 0
                             : nbr[3 * tf] == ts ? 1
                             : nbr[3 * tf + 1] == ts ? 2
                             : nbr[3 * tf + 2] == ts ? 3 : -1;
            if (slot >= 0) {
                const double2 v = tab[(size_t)36 * tf + 9 * slot + 3 * F.e[a] + S.e[b]];
                sr += (double)sgn * v.x;
                si += (double)sgn * v.y;
                continue;
            }
            const T* Qp = q7 + (size_t)21 * ts;
            const V3<T> vs = v3(S.v[b][0], S.v[b][1], S.v[b][2]);
            T er = 0, ei = 0;
#pragma unroll 1
            for (int p = 0; p < 7; ++p) {
                const V3<T> P = v3(Pp[3 * p], Pp[3 * p + 1], Pp[3 * p + 2]);
                const V3<T> rf = P - vf;
                const T wp = gauss7_weight<T>(p);
#pragma unroll
                for (int q = 0; q < 7; ++q) {
                    const V3<T> Q = v3(Qp[3 * q], Qp[3 * q + 1], Qp[3 * q + 2]);
                    const V3<T> d = P - Q;
                    const T r = sqrt(dot(d, d));
                    const T rinv = T(1) / r;
                    T sn, cs;
                    sincos_pi(r * c.kpi, &sn, &cs);
                    const T e = wp * gauss7_weight<T>(q) * (T(0.25) * dot(rf, Q - vs) - c.inv_k2);
                    er += e * cs * rinv;
                    ei -= e * sn * rinv;
                }
            }
            zr += sgn * er;
            zi += sgn * ei;
        }
    }
    const T kz = (T)c.coef_efie * (F.len * S.len);
    const T re = zr + (T)sr, im = zi + (T)si;
    return cx(-kz * im, kz * re);
}

template <typename T>
__global__ void __launch_bounds__(256) k_fill_z_cfg(const RwgPack<T>* __restrict__ rw, int n, FillConst<T> c,
                                                    const double2* __restrict__ tab, const int* __restrict__ nbr,
                                                    const T* __restrict__ q7, Cx<T>* __restrict__ Z, size_t ldz)
{
    int s = blockIdx.x * 32 + threadIdx.x;
    int f = blockIdx.y * blockDim.y + threadIdx.y;
    if (s >= n || f >= n) return;
    Z[(size_t)f * ldz + s] = z_entry_cfg<T>(rw[f], rw[s], c, tab, nbr, q7);
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
// tiled FP32 fill: a CTA fills a 16 x 16 block of Z.  The 9 point-pair
// kernel values (G = e^{-jkR}/R, with R and 1/R) of every (test triangle,
// source triangle) pair of the block are computed once into shared memory,
// then each entry is assembled from them: consecutive RWGs share triangles,
// so a block needs about 18 x 18 triangle pairs instead of 16 x 16 x 4.  The
// arithmetic of every point pair, and the order of every sum, is that of
// z_entry, except that sin/cos(kR) come from the FP32 Taylor evaluation
// (sincos_pi_taylor, about 1.5 ulp).
// ---------------------------------------------------------------------------
constexpr int FT = 16;  // RWGs per tile side

template <bool CFIE>
__device__ __forceinline__ void regular_pair_staged(const float (&P)[3][3], const float4* __restrict__ Q4,
                                                    const float (&vf)[3], const float (&vs)[3],
                                                    const float (&nf)[3], const float4* __restrict__ K,
                                                    const FillConst<float>& c, Cx<float>& ze, Cx<float>& zm)
{
    V3<float> n = v3(nf[0], nf[1], nf[2]);
    float Q[9];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float4 t = Q4[q];
        Q[3 * q] = t.x;
        Q[3 * q + 1] = t.y;
        Q[3 * q + 2] = t.z;
    }
    V3<float> rs[3];
    float nrs[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        rs[q] = v3(Q[3 * q] - vs[0], Q[3 * q + 1] - vs[1], Q[3 * q + 2] - vs[2]);
        nrs[q] = dot(n, rs[q]);
    }
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        V3<float> pp = v3(P[p][0], P[p][1], P[p][2]);
        V3<float> rf = v3(P[p][0] - vf[0], P[p][1] - vf[1], P[p][2] - vf[2]);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float4 kv = K[3 * p + q];
            const float gr = kv.x, gi = kv.y;
            float rfrs = dot(rf, rs[q]);
            float e = 0.25f * rfrs - c.inv_k2;
            ze.re += e * gr;
            ze.im += e * gi;
            if (CFIE) {
                V3<float> d = v3(pp.x - Q[3 * q], pp.y - Q[3 * q + 1], pp.z - Q[3 * q + 2]);
                const float r = kv.z, rinv = kv.w;
                float m = dot(rf, d) * nrs[q] - rfrs * dot(n, d);
                float t = m * (rinv * rinv);
                float kr = r * c.k;
                float hr = gr - kr * gi, hi = gi + kr * gr;
                zm.re += t * hr;
                zm.im += t * hi;
            }
        }
    }
}

template <bool CFIE>
__global__ void __launch_bounds__(256) k_fill_tile(const RwgPack<float>* __restrict__ rw, int n, FillConst<float> c,
                                                   const double2* __restrict__ sing, const float* __restrict__ tri_q3,
                                                   const float* __restrict__ tri_n, const int* __restrict__ blk_tris,
                                                   const int* __restrict__ blk_nt, const unsigned char* __restrict__ loc,
                                                   int maxt, Cx<float>* __restrict__ Z, size_t ldz)
{
    extern __shared__ float4 sk[];  // [maxt][maxt][9] (G re, G im, R, 1/R)
    float4* sqf = sk + (size_t)maxt * maxt * 9;  // test points [maxt][3] (x y z -)
    float4* snf = sqf + maxt * 3;                 // test normals [maxt]
    float4* sqs = snf + maxt;                     // source points [maxt][3]
    const int bf = blockIdx.y, bs = blockIdx.x;
    const int ntf = blk_nt[bf], nts = blk_nt[bs];
    const int* tf_ids = blk_tris + (size_t)bf * maxt;
    const int* ts_ids = blk_tris + (size_t)bs * maxt;
    for (int i = threadIdx.x; i < ntf * 3; i += blockDim.x) {
        const float* q = tri_q3 + 9 * (size_t)tf_ids[i / 3] + 3 * (i % 3);
        sqf[i] = make_float4(q[0], q[1], q[2], 0.0f);
    }
    for (int i = threadIdx.x; i < ntf; i += blockDim.x) {
        const float* q = tri_n + 3 * (size_t)tf_ids[i];
        snf[i] = make_float4(q[0], q[1], q[2], 0.0f);
    }
    for (int i = threadIdx.x; i < nts * 3; i += blockDim.x) {
        const float* q = tri_q3 + 9 * (size_t)ts_ids[i / 3] + 3 * (i % 3);
        sqs[i] = make_float4(q[0], q[1], q[2], 0.0f);
    }
    __syncthreads();
    // phase 1: point-pair kernel values of every triangle pair (self pairs are
    // computed too, never read: their entries come from the FP64 table)
    for (int pr = threadIdx.x; pr < ntf * nts; pr += blockDim.x) {
        const int tf = pr / nts, ts = pr - tf * nts;
        float4* out = sk + ((size_t)tf * maxt + ts) * 9;
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            const float4 P = sqf[3 * tf + p];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float4 Q = sqs[3 * ts + q];
                V3<float> d = v3(P.x - Q.x, P.y - Q.y, P.z - Q.z);
                float r = sqrtf(dot(d, d));
                float rinv = 1.0f / r;
                float sn, cs;
                sincos_pi_taylor(r * c.kpi, &sn, &cs);
                out[3 * p + q] = make_float4(cs * rinv, -sn * rinv, r, rinv);
            }
        }
    }
    __syncthreads();
    // phase 2: the entries, z_entry's loop with the staged values
    const int f = bf * FT + (threadIdx.x >> 4), s = bs * FT + (threadIdx.x & 15);
    if (f >= n || s >= n) return;
    const RwgPack<float>& F = rw[f];
    const RwgPack<float>& S = rw[s];
    if (!CFIE && c.edm_mode != 2) {
        V3<float> fc = divr(v3(F.cen[0][0], F.cen[0][1], F.cen[0][2]) + v3(F.cen[1][0], F.cen[1][1], F.cen[1][2]), 2.0f);
        V3<float> sc = divr(v3(S.cen[0][0], S.cen[0][1], S.cen[0][2]) + v3(S.cen[1][0], S.cen[1][1], S.cen[1][2]), 2.0f);
        if (norm(fc - sc) > c.thr_edm) {
            Z[(size_t)f * ldz + s] = c.edm_mode == 1 ? edm_value(F, S, c) : cx(0.0f, 0.0f);
            return;
        }
    }
    Cx<float> ze = cx(0.0f, 0.0f), zm = cx(0.0f, 0.0f);
    // self terms: a pair's value formed in FP64 from the table and rounded
    // once; the sum over an entry's (at most two) self pairs in FP32, so no
    // FP64 register or conversion in the common entry
    float sr = 0.f, si = 0.f;
#pragma unroll 1
    for (int a = 0; a < 2; ++a) {
        const int lf = loc[2 * (size_t)f + a];
        float P[3][3], vf[3], nf[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float4 t = sqf[3 * lf + i];
            P[i][0] = t.x;
            P[i][1] = t.y;
            P[i][2] = t.z;
        }
        const float4 nn = snf[lf];
        nf[0] = nn.x;
        nf[1] = nn.y;
        nf[2] = nn.z;
#pragma unroll
        for (int j = 0; j < 3; ++j) vf[j] = F.v[a][j];
#pragma unroll 1
        for (int b = 0; b < 2; ++b) {
            const float sgn = (a == b) ? 1.0f : -1.0f;
            if (F.tri[a] == S.tri[b]) {
                const int id = 9 * F.tri[a] + 3 * F.e[a] + S.e[b];
                if (CFIE) {
                    const double2 v = sing[id];
                    sr += sgn * (float)v.x;
                    si += sgn * (float)v.y;
                } else {
                    const double2 v = sing[3 * id + ((a == 0 && b == 0) ? 0 : 1)];
                    const double2 g = sing[3 * id + 2];
                    sr += (float)((double)sgn * v.x + g.x);
                    si += (float)((double)sgn * v.y + g.y);
                }
                continue;
            }
            const int ls = loc[2 * (size_t)s + b];
            float vs[3] = {S.v[b][0], S.v[b][1], S.v[b][2]};
            Cx<float> e = cx(0.0f, 0.0f), m = cx(0.0f, 0.0f);
            regular_pair_staged<CFIE>(P, sqs + 3 * ls, vf, vs, nf, sk + ((size_t)lf * maxt + ls) * 9, c, e, m);
            ze.re += sgn * e.re;
            ze.im += sgn * e.im;
            if (CFIE) {
                zm.re += sgn * m.re;
                zm.im += sgn * m.im;
            }
        }
    }
    const float l = F.len * S.len;
    Cx<float> out;
    if (CFIE) {
        const float re = -c.ce * ze.im + c.cm * zm.re + sr;
        const float im = c.ce * ze.re + c.cm * zm.im + si;
        out = cx(re * l, im * l);
    } else {
        const float kz = (float)c.coef_efie * l;
        const float re = c.ce * ze.re + sr, im = c.ce * ze.im + si;
        out = cx(-kz * im, kz * re);
    }
    Z[(size_t)f * ldz + s] = out;
}

// Symmetric EFIE fill (edm_mode 0 or 2): the regular part of an EFIE entry,
//   sum over the triangle pairs of sum_pq (rf.rs/4 - 1/k^2) G(P_p, Q_q),
// does not change when test and source trade places, so a CTA fills a tile
// on or above the diagonal of tiles and, off the diagonal, the mirrored tile
// from the same regular sums (staged through shared memory and stored a row
// at a time).  The FP64 self terms of pairs that share a triangle are not
// symmetric: the mirrored entry takes them from the table with the roles of
// the two RWGs exchanged.  Far pairs zeroed under edm_mode 0 are zero both
// ways (the centre distance is the same).
__global__ void __launch_bounds__(256) k_fill_tile_sym(const RwgPack<float>* __restrict__ rw, int n,
                                                       FillConst<float> c, const double2* __restrict__ sing,
                                                       const float* __restrict__ tri_q3,
                                                       const int* __restrict__ blk_tris,
                                                       const int* __restrict__ blk_nt,
                                                       const unsigned char* __restrict__ loc, int maxt, int nb,
                                                       Cx<float>* __restrict__ Z, size_t ldz)
{
    extern __shared__ float4 sk[];  // [maxt][maxt][9] (G re, G im, R, 1/R)
    float4* sqf = sk + (size_t)maxt * maxt * 9;  // test points [maxt][3]
    float4* sqs = sqf + maxt * 3;                 // source points [maxt][3]
    __shared__ Cx<float> zt[FT][FT + 1];          // the mirrored tile, [s][f]
    // tile (bf, bs), bf <= bs, from the linear index: row bf holds nb - bf tiles
    const long long li = blockIdx.x;
    int bf = (int)(((2.0 * nb + 1.0) - sqrt((2.0 * nb + 1.0) * (2.0 * nb + 1.0) - 8.0 * (double)li)) / 2.0);
    auto row0 = [&](int b) { return (long long)b * nb - (long long)b * (b - 1) / 2; };
    while (bf > 0 && row0(bf) > li) --bf;
    while (bf + 1 < nb && row0(bf + 1) <= li) ++bf;
    const int bs = bf + (int)(li - row0(bf));
    const int ntf = blk_nt[bf], nts = blk_nt[bs];
    const int* tf_ids = blk_tris + (size_t)bf * maxt;
    const int* ts_ids = blk_tris + (size_t)bs * maxt;
    for (int i = threadIdx.x; i < ntf * 3; i += blockDim.x) {
        const float* q = tri_q3 + 9 * (size_t)tf_ids[i / 3] + 3 * (i % 3);
        sqf[i] = make_float4(q[0], q[1], q[2], 0.0f);
    }
    for (int i = threadIdx.x; i < nts * 3; i += blockDim.x) {
        const float* q = tri_q3 + 9 * (size_t)ts_ids[i / 3] + 3 * (i % 3);
        sqs[i] = make_float4(q[0], q[1], q[2], 0.0f);
    }
    __syncthreads();
    for (int pr = threadIdx.x; pr < ntf * nts; pr += blockDim.x) {
        const int tf = pr / nts, ts = pr - tf * nts;
        float4* out = sk + ((size_t)tf * maxt + ts) * 9;
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            const float4 P = sqf[3 * tf + p];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float4 Q = sqs[3 * ts + q];
                V3<float> d = v3(P.x - Q.x, P.y - Q.y, P.z - Q.z);
                float r = sqrtf(dot(d, d));
                float rinv = 1.0f / r;
                float sn, cs;
                sincos_pi_taylor(r * c.kpi, &sn, &cs);
                out[3 * p + q] = make_float4(cs * rinv, -sn * rinv, r, rinv);
            }
        }
    }
    __syncthreads();
    const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
    const int f = bf * FT + ty, s = bs * FT + tx;
    const bool mirror = bf != bs;
    Cx<float> out = cx(0.0f, 0.0f), out_t = cx(0.0f, 0.0f);
    if (f < n && s < n) {
        const RwgPack<float>& F = rw[f];
        const RwgPack<float>& S = rw[s];
        bool zeroed = false;
        if (c.edm_mode == 0) {
            V3<float> fc = divr(v3(F.cen[0][0], F.cen[0][1], F.cen[0][2]) + v3(F.cen[1][0], F.cen[1][1], F.cen[1][2]), 2.0f);
            V3<float> sc = divr(v3(S.cen[0][0], S.cen[0][1], S.cen[0][2]) + v3(S.cen[1][0], S.cen[1][1], S.cen[1][2]), 2.0f);
            zeroed = norm(fc - sc) > c.thr_edm;
        }
        if (!zeroed) {
            Cx<float> ze = cx(0.0f, 0.0f), zm = cx(0.0f, 0.0f);
            // self terms: a pair's value formed in FP64 and rounded once, the
            // sums in FP32 (no FP64 register or conversion per entry)
            float sr = 0.f, si = 0.f, sr_t = 0.f, si_t = 0.f;
#pragma unroll 1
            for (int a = 0; a < 2; ++a) {
                const int lf = loc[2 * (size_t)f + a];
                float P[3][3], vf[3], nf[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const float4 t = sqf[3 * lf + i];
                    P[i][0] = t.x;
                    P[i][1] = t.y;
                    P[i][2] = t.z;
                }
#pragma unroll
                for (int j = 0; j < 3; ++j) vf[j] = F.v[a][j];
#pragma unroll 1
                for (int b = 0; b < 2; ++b) {
                    const float sgn = (a == b) ? 1.0f : -1.0f;
                    if (F.tri[a] == S.tri[b]) {
                        const int id = 9 * F.tri[a] + 3 * F.e[a] + S.e[b];
                        const double2 v = sing[3 * id + ((a == 0 && b == 0) ? 0 : 1)];
                        const double2 g = sing[3 * id + 2];
                        sr += (float)((double)sgn * v.x + g.x);
                        si += (float)((double)sgn * v.y + g.y);
                        // the mirrored entry: test s (side b), source f (side a)
                        const int it = 9 * S.tri[b] + 3 * S.e[b] + F.e[a];
                        const double2 vt = sing[3 * it + ((b == 0 && a == 0) ? 0 : 1)];
                        const double2 gt = sing[3 * it + 2];
                        sr_t += (float)((double)sgn * vt.x + gt.x);
                        si_t += (float)((double)sgn * vt.y + gt.y);
                        continue;
                    }
                    const int ls = loc[2 * (size_t)s + b];
                    float vs[3] = {S.v[b][0], S.v[b][1], S.v[b][2]};
                    Cx<float> e = cx(0.0f, 0.0f), m = cx(0.0f, 0.0f);
                    regular_pair_staged<false>(P, sqs + 3 * ls, vf, vs, nf, sk + ((size_t)lf * maxt + ls) * 9, c, e,
                                               m);
                    ze.re += sgn * e.re;
                    ze.im += sgn * e.im;
                }
            }
            const float kz = (float)c.coef_efie * (F.len * S.len);
            float re = c.ce * ze.re + sr, im = c.ce * ze.im + si;
            out = cx(-kz * im, kz * re);
            re = c.ce * ze.re + sr_t;
            im = c.ce * ze.im + si_t;
            out_t = cx(-kz * im, kz * re);
        }
        Z[(size_t)f * ldz + s] = out;
    }
    if (!mirror) return;  // uniform over the CTA
    zt[tx][ty] = out_t;  // Z[s][f]
    __syncthreads();
    // row s = bs 16 + ty of the mirrored tile, columns f = bf 16 + tx
    const int sr_ = bs * FT + ty, fc_ = bf * FT + tx;
    if (sr_ < n && fc_ < n) Z[(size_t)sr_ * ldz + fc_] = zt[ty][tx];
}

// Symmetric-pair CFIE fill: a CTA takes a tile pair (bf <= bs) and fills
// both Z(bf, bs) and, off the diagonal, Z(bs, bf).  With d = P - Q,
// rf = P - vf and rs = Q - vs, an entry's regular pair sums
//   EFIE part  (rf.rs/4 - 1/k^2) G            (the same both ways)
//   MFIE part  m H,  m = (rf.d)(nf.rs) - (rf.rs)(nf.d)        for Z(f, s)
//              m' H, m' = (rf.rs)(ns.d) - (rs.d)(ns.rf)       for Z(s, f)
// (the test field of Z(s, f) is Q on the source triangle, its source P,
// so d changes sign), with G = e^{-jkR}/R and H = (1 + jkR) G / R^2 the
// same both ways.  G and H of every point pair of the tiles' triangle pairs
// are staged once (16 bytes a point pair, so three CTAs fit an SM); nf.d
// and ns.d are formed per entry from d.  Self pairs take the FP64 table
// with the field and source corners exchanged for the mirrored entry.  The
// mirrored tile is staged through shared memory and stored a row at a time.
__global__ void __launch_bounds__(256, 3) k_fill_tile_cfie_sym(const RwgPack<float>* __restrict__ rw, int n,
                                                               FillConst<float> c, const double2* __restrict__ sing,
                                                               const float* __restrict__ tri_q3,
                                                               const float* __restrict__ tri_n,
                                                               const int* __restrict__ blk_tris,
                                                               const int* __restrict__ blk_nt,
                                                               const unsigned char* __restrict__ loc, int maxt,
                                                               int nb, Cx<float>* __restrict__ Z, size_t ldz)
{
    extern __shared__ float4 sk[];               // [maxt][maxt][9] (G re, G im, H re, H im)
    float4* sqf = sk + (size_t)maxt * maxt * 9;  // test points [maxt][3]
    float4* sqs = sqf + maxt * 3;                // source points [maxt][3]
    float4* snf = sqs + maxt * 3;                // test normals [maxt]
    float4* sns = snf + maxt;                    // source normals [maxt]
    __shared__ Cx<float> zt[FT][FT + 1];         // the mirrored tile, [s][f]
    const long long li = blockIdx.x;
    int bf = (int)(((2.0 * nb + 1.0) - sqrt((2.0 * nb + 1.0) * (2.0 * nb + 1.0) - 8.0 * (double)li)) / 2.0);
    auto row0 = [&](int b) { return (long long)b * nb - (long long)b * (b - 1) / 2; };
    while (bf > 0 && row0(bf) > li) --bf;
    while (bf + 1 < nb && row0(bf + 1) <= li) ++bf;
    const int bs = bf + (int)(li - row0(bf));
    const int ntf = blk_nt[bf], nts = blk_nt[bs];
    const int* tf_ids = blk_tris + (size_t)bf * maxt;
    const int* ts_ids = blk_tris + (size_t)bs * maxt;
    for (int i = threadIdx.x; i < ntf * 3; i += blockDim.x) {
        const float* q = tri_q3 + 9 * (size_t)tf_ids[i / 3] + 3 * (i % 3);
        sqf[i] = make_float4(q[0], q[1], q[2], 0.0f);
    }
    for (int i = threadIdx.x; i < nts * 3; i += blockDim.x) {
        const float* q = tri_q3 + 9 * (size_t)ts_ids[i / 3] + 3 * (i % 3);
        sqs[i] = make_float4(q[0], q[1], q[2], 0.0f);
    }
    for (int i = threadIdx.x; i < ntf; i += blockDim.x) {
        const float* q = tri_n + 3 * (size_t)tf_ids[i];
        snf[i] = make_float4(q[0], q[1], q[2], 0.0f);
    }
    for (int i = threadIdx.x; i < nts; i += blockDim.x) {
        const float* q = tri_n + 3 * (size_t)ts_ids[i];
        sns[i] = make_float4(q[0], q[1], q[2], 0.0f);
    }
    __syncthreads();
    for (int pr = threadIdx.x; pr < ntf * nts; pr += blockDim.x) {
        const int tf = pr / nts, ts = pr - tf * nts;
        float4* o4 = sk + ((size_t)tf * maxt + ts) * 9;
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            const float4 P = sqf[3 * tf + p];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float4 Q = sqs[3 * ts + q];
                const float dx = P.x - Q.x, dy = P.y - Q.y, dz = P.z - Q.z;
                const float r = sqrtf(dx * dx + dy * dy + dz * dz);
                const float rinv = 1.0f / r;
                float sn, cs;
                sincos_pi_taylor(r * c.kpi, &sn, &cs);
                const float gr = cs * rinv, gi = -sn * rinv;
                const float kr = r * c.k, r2 = rinv * rinv;
                o4[3 * p + q] = make_float4(gr, gi, (gr - kr * gi) * r2, (gi + kr * gr) * r2);
            }
        }
    }
    __syncthreads();
    const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
    const int f = bf * FT + ty, s = bs * FT + tx;
    const bool mirror = bf != bs;
    Cx<float> out = cx(0.0f, 0.0f), out_t = cx(0.0f, 0.0f);
    if (f < n && s < n) {
        const RwgPack<float>& F = rw[f];
        const RwgPack<float>& S = rw[s];
        float zer = 0, zei = 0, zmr = 0, zmi = 0, ztr = 0, zti = 0;
        // self terms from the FP64 table, summed in FP32 (at most two per
        // entry; the entry is FP32): four registers, not eight
        float sr = 0.f, si = 0.f, sr_t = 0.f, si_t = 0.f;
#pragma unroll 1
        for (int a = 0; a < 2; ++a) {
            const int lf = loc[2 * (size_t)f + a];
            float P[3][3], rf[3][3];
            const float4 nf = snf[lf];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float4 t = sqf[3 * lf + i];
                P[i][0] = t.x;
                P[i][1] = t.y;
                P[i][2] = t.z;
                rf[i][0] = t.x - F.v[a][0];
                rf[i][1] = t.y - F.v[a][1];
                rf[i][2] = t.z - F.v[a][2];
            }
#pragma unroll 1
            for (int b = 0; b < 2; ++b) {
                const float sgn = (a == b) ? 1.0f : -1.0f;
                if (F.tri[a] == S.tri[b]) {
                    const double2 v = sing[9 * F.tri[a] + 3 * F.e[a] + S.e[b]];
                    sr += sgn * (float)v.x;
                    si += sgn * (float)v.y;
                    const double2 vt = sing[9 * S.tri[b] + 3 * S.e[b] + F.e[a]];
                    sr_t += sgn * (float)vt.x;
                    si_t += sgn * (float)vt.y;
                    continue;
                }
                const int ls = loc[2 * (size_t)s + b];
                const float4 ns = sns[ls];
                float Q[3][3], rs[3][3], nfrs[3], nsrf[3];
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const float4 t = sqs[3 * ls + q];
                    Q[q][0] = t.x;
                    Q[q][1] = t.y;
                    Q[q][2] = t.z;
                    rs[q][0] = t.x - S.v[b][0];
                    rs[q][1] = t.y - S.v[b][1];
                    rs[q][2] = t.z - S.v[b][2];
                    nfrs[q] = nf.x * rs[q][0] + nf.y * rs[q][1] + nf.z * rs[q][2];
                }
#pragma unroll
                for (int p = 0; p < 3; ++p) nsrf[p] = ns.x * rf[p][0] + ns.y * rf[p][1] + ns.z * rf[p][2];
                const float4* K4 = sk + ((size_t)lf * maxt + ls) * 9;
                float er = 0, ei = 0, mr = 0, mi = 0, tr = 0, ti = 0;
#pragma unroll
                for (int p = 0; p < 3; ++p)
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        const float4 g = K4[3 * p + q];
                        const float dx = P[p][0] - Q[q][0], dy = P[p][1] - Q[q][1], dz = P[p][2] - Q[q][2];
                        const float nfd = nf.x * dx + nf.y * dy + nf.z * dz;
                        const float nsd = ns.x * dx + ns.y * dy + ns.z * dz;
                        const float rfrs = rf[p][0] * rs[q][0] + rf[p][1] * rs[q][1] + rf[p][2] * rs[q][2];
                        const float rfd = rf[p][0] * dx + rf[p][1] * dy + rf[p][2] * dz;
                        const float rsd = rs[q][0] * dx + rs[q][1] * dy + rs[q][2] * dz;
                        const float e = 0.25f * rfrs - c.inv_k2;
                        er += e * g.x;
                        ei += e * g.y;
                        const float m = rfd * nfrs[q] - rfrs * nfd;
                        const float mt = rfrs * nsd - rsd * nsrf[p];
                        mr += m * g.z;
                        mi += m * g.w;
                        tr += mt * g.z;
                        ti += mt * g.w;
                    }
                zer += sgn * er;
                zei += sgn * ei;
                zmr += sgn * mr;
                zmi += sgn * mi;
                ztr += sgn * tr;
                zti += sgn * ti;
            }
        }
        const float l = F.len * S.len;
        out = cx((-c.ce * zei + c.cm * zmr + sr) * l, (c.ce * zer + c.cm * zmi + si) * l);
        out_t = cx((-c.ce * zei + c.cm * ztr + sr_t) * l, (c.ce * zer + c.cm * zti + si_t) * l);
        Z[(size_t)f * ldz + s] = out;
    }
    if (!mirror) return;  // uniform over the CTA
    zt[tx][ty] = out_t;  // Z[s][f]
    __syncthreads();
    const int sr_ = bs * FT + ty, fc_ = bf * FT + tx;
    if (sr_ < n && fc_ < n) Z[(size_t)sr_ * ldz + fc_] = zt[ty][tx];
}

static size_t tile_smem_cfie_sym(int maxt)
{
    return sizeof(float4) * ((size_t)maxt * maxt * 9 + 8 * (size_t)maxt);
}

// per-geometry plan of the tiled fill (host, once)
static emfa_status_t tile_plan(Ctx* c, Geom* g, cudaStream_t st)
{
    if (g->tile_ready) return EMFA_OK;
    const int n = g->n, nb = (n + FT - 1) / FT;
    std::vector<std::vector<int>> lists(nb);
    std::vector<unsigned char> loc(2 * (size_t)n);
    int maxt = 1;
    for (int b = 0; b < nb; ++b) {
        auto& L = lists[b];
        for (int u = b * FT; u < std::min(n, (b + 1) * FT); ++u)
            for (int a = 0; a < 2; ++a) {
                const int t = g->rwg[6 * (size_t)u + 4 + a];
                int idx = -1;
                for (int i = 0; i < (int)L.size(); ++i)
                    if (L[i] == t) {
                        idx = i;
                        break;
                    }
                if (idx < 0) {
                    idx = (int)L.size();
                    L.push_back(t);
                }
                loc[2 * (size_t)u + a] = (unsigned char)idx;
            }
        maxt = std::max(maxt, (int)L.size());
    }
    std::vector<int> flat((size_t)nb * maxt, 0), cnt(nb);
    for (int b = 0; b < nb; ++b) {
        cnt[b] = (int)lists[b].size();
        std::copy(lists[b].begin(), lists[b].end(), flat.begin() + (size_t)b * maxt);
    }
    const size_t b0 = (sizeof(int) * flat.size() + 255) & ~(size_t)255, b1 = (sizeof(int) * cnt.size() + 255) & ~(size_t)255;
    EMFA_TRY(g->tile_block.alloc(c, b0 + b1 + loc.size()));
    g->tile_tris = DevView{g->tile_block.ptr, sizeof(int) * flat.size()};
    g->tile_nt = DevView{(char*)g->tile_block.ptr + b0, sizeof(int) * cnt.size()};
    g->tile_loc = DevView{(char*)g->tile_block.ptr + b0 + b1, loc.size()};
    EMFA_CUDA(c, cudaMemcpyAsync(g->tile_tris.ptr, flat.data(), g->tile_tris.bytes, cudaMemcpyHostToDevice, st));
    EMFA_CUDA(c, cudaMemcpyAsync(g->tile_nt.ptr, cnt.data(), g->tile_nt.bytes, cudaMemcpyHostToDevice, st));
    EMFA_CUDA(c, cudaMemcpyAsync(g->tile_loc.ptr, loc.data(), g->tile_loc.bytes, cudaMemcpyHostToDevice, st));
    EMFA_CUDA(c, cudaStreamSynchronize(st));  // host staging vectors go out of scope
    g->tile_maxt = maxt;
    g->tile_ready = true;
    return EMFA_OK;
}

static size_t tile_smem(int maxt) { return sizeof(float4) * ((size_t)maxt * maxt * 9 + 7 * (size_t)maxt); }

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
static SingConst sing_const(const emfa_fill_params_t* p)
{
    SingConst sc;
    sc.k = p->precision == EMFA_F64 ? Phys<double>::wavenumber(p->freq) : (double)Phys<float>::wavenumber(p->freq);
    sc.inv_k2 = 1.0 / (sc.k * sc.k);
    sc.w = 1.0 / 3.0;
    sc.alpha = p->alpha;
    sc.pi = 3.14159265358979323846;
    sc.z0 = 120.0 * sc.pi;
    sc.sig_re = p->sigma_re;
    sc.sig_im = p->sigma_im;
    sc.cfie = p->kind == EMFA_CFIE;
    return sc;
}

// Each triangle's edge neighbours (up to 3, -1 where none), from the RWG
// table in RWG order: the RWG of an edge joins its + and - triangles.  A
// triangle with more than 3 RWG neighbours (a non-manifold mesh) keeps the
// first 3; the rest are filled as regular pairs.
static emfa_status_t geom_neighbours(Ctx* c, Geom* g, cudaStream_t st)
{
    if (g->nbr_ready) return EMFA_OK;
    std::vector<int> nb((size_t)3 * g->nt, -1);
    auto add = [&](int t, int o) {
        for (int j = 0; j < 3; ++j) {
            if (nb[3 * t + j] == o) return;
            if (nb[3 * t + j] < 0) {
                nb[3 * t + j] = o;
                return;
            }
        }
    };
    for (int u = 0; u < g->n; ++u) {
        const int tp = g->rwg[6 * u + 4], tm = g->rwg[6 * u + 5];
        add(tp, tm);
        add(tm, tp);
    }
    EMFA_TRY(g->nbr.alloc(c, sizeof(int) * nb.size()));
    EMFA_CUDA(c, cudaMemcpyAsync(g->nbr.ptr, nb.data(), sizeof(int) * nb.size(), cudaMemcpyHostToDevice, st));
    EMFA_CUDA(c, cudaStreamSynchronize(st));  // nb is a host temporary
    g->nbr_ready = true;
    return EMFA_OK;
}

// The configuration's discretisation: FP64 table of self and edge-adjacent
// pairs, then one thread per entry with 7 x 7-point regular pairs.
template <typename T>
static emfa_status_t fill_z_cfg(Ctx* c, Geom* g, GeomDev<T>& d, const emfa_fill_params_t* p, void* Z, size_t ldz,
                                cudaStream_t st)
{
    EMFA_TRY(geom_neighbours(c, g, st));
    EMFA_TRY(geom_vd(g, st));
    void* tab = nullptr;
    EMFA_TRY(ctx_workspace(c, WS_FILL, sizeof(double2) * (size_t)g->nt * 36, &tab));
    const SingConst sc = sing_const(p);
    k_config_table<<<(36 * g->nt + 143) / 144, 144, 0, st>>>(dptr<double>(g->vd), dptr<int>(d.tris),
                                                             dptr<int>(g->nbr), g->nt, sc, (double2*)tab);
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    FillConst<T> fc = make_fill_const<T>(p);
    dim3 blk(32, 8);
    dim3 grd((g->n + 31) / 32, (g->n + 7) / 8);
    {
        TimedLaunch tl(c, KT_FILL_Z, st, (double)g->n * g->n);
        k_fill_z_cfg<T><<<grd, blk, 0, st>>>(dptr<RwgPack<T>>(d.rwg), g->n, fc, (const double2*)tab,
                                             dptr<int>(g->nbr), dptr<T>(d.tri_q7), reinterpret_cast<Cx<T>*>(Z), ldz);
    }
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    return EMFA_OK;
}

template <typename T>
static emfa_status_t fill_z_t(Ctx* c, Geom* g, GeomDev<T>& d, const emfa_fill_params_t* p, void* Z, size_t ldz,
                              cudaStream_t st)
{
    const bool cfie = p->kind == EMFA_CFIE;
    if (p->discretisation == EMFA_DISC_CONFIG) return fill_z_cfg<T>(c, g, d, p, Z, ldz, st);
    // singular table (FP64), 9 (CFIE) or 27 (EFIE) double2 per triangle
    void* tab = nullptr;
    EMFA_TRY(ctx_workspace(c, WS_FILL, sizeof(double2) * (size_t)g->nt * (cfie ? 9 : 27), &tab));
    EMFA_TRY(build_singular_table(c, g, p, (double2*)tab, st));
    FillConst<T> fc = make_fill_const<T>(p);
    if (std::is_same<T, float>::value) {
        // FP32: the tiled kernel
        EMFA_TRY(tile_plan(c, g, st));
        const size_t sm = tile_smem(g->tile_maxt);
        const size_t sm_c = tile_smem_cfie_sym(g->tile_maxt);
        EMFA_TRY(ensure_smem(c, k_fill_tile<true>, sm));
        EMFA_TRY(ensure_smem(c, k_fill_tile<false>, sm));
        EMFA_TRY(ensure_smem(c, k_fill_tile_sym, sm));
        EMFA_TRY(ensure_smem(c, k_fill_tile_cfie_sym, sm_c));
        const dim3 grd((g->n + FT - 1) / FT, (g->n + FT - 1) / FT);
        const FillConst<float> fc32 = make_fill_const<float>(p);
        {
            TimedLaunch tl(c, KT_FILL_Z, st, (double)g->n * g->n);
            if (cfie) {
                const int nb = (g->n + FT - 1) / FT;
                k_fill_tile_cfie_sym<<<(unsigned)((long long)nb * (nb + 1) / 2), 256, sm_c, st>>>(
                    dptr<RwgPack<float>>(g->g32.rwg), g->n, fc32, (const double2*)tab, dptr<float>(g->g32.tri_q3),
                    dptr<float>(g->g32.tri_n), dptr<int>(g->tile_tris), dptr<int>(g->tile_nt),
                    dptr<unsigned char>(g->tile_loc), g->tile_maxt, nb, reinterpret_cast<Cx<float>*>(Z), ldz);
            } else if (p->edm_mode != 1) {
                const int nb = (g->n + FT - 1) / FT;
                k_fill_tile_sym<<<(unsigned)((long long)nb * (nb + 1) / 2), 256, sm, st>>>(
                    dptr<RwgPack<float>>(g->g32.rwg), g->n, fc32, (const double2*)tab, dptr<float>(g->g32.tri_q3),
                    dptr<int>(g->tile_tris), dptr<int>(g->tile_nt), dptr<unsigned char>(g->tile_loc), g->tile_maxt,
                    nb, reinterpret_cast<Cx<float>*>(Z), ldz);
            } else
                k_fill_tile<false><<<grd, 256, sm, st>>>(
                    dptr<RwgPack<float>>(g->g32.rwg), g->n, fc32, (const double2*)tab, dptr<float>(g->g32.tri_q3),
                    dptr<float>(g->g32.tri_n), dptr<int>(g->tile_tris), dptr<int>(g->tile_nt),
                    dptr<unsigned char>(g->tile_loc), g->tile_maxt, reinterpret_cast<Cx<float>*>(Z), ldz);
        }
        c->kernel_launches += 1;
        EMFA_CUDA(c, cudaGetLastError());
        EMFA_CUDA(c, cudaStreamSynchronize(st));
        return EMFA_OK;
    }
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
    if (p->precision == EMFA_F64)
        EMFA_TRY(geom_prepare_f64(g, st));
    else
        EMFA_TRY(geom_prepare_f32(g, st));
    // the table's vertices (the geometry's FP64 copy) and k: the fill
    // precision's k, in FP64 arithmetic
    EMFA_TRY(geom_vd(g, st));
    const SingConst sc = sing_const(p);
    const int* tris = p->precision == EMFA_F64 ? dptr<int>(g->g64.tris) : dptr<int>(g->g32.tris);
    k_singular_table<<<(g->nt + SING_TRIS - 1) / SING_TRIS, 9 * SING_TRIS, 0, st>>>(dptr<double>(g->vd), tris, g->nt,
                                                                                   sc, tab);
    c->kernel_launches += 1;
    EMFA_CUDA(c, cudaGetLastError());
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
    if (p->discretisation != EMFA_DISC_REFERENCE && p->discretisation != EMFA_DISC_CONFIG) {
        set_error(ctx, "fill: discretisation must be EMFA_DISC_REFERENCE or EMFA_DISC_CONFIG");
        return EMFA_ERR_INVALID;
    }
    if (p->discretisation == EMFA_DISC_CONFIG && p->kind != EMFA_EFIE) {
        set_error(ctx, "fill: EMFA_DISC_CONFIG (7-point rule, adjacent-pair extraction) is built for EFIE only");
        return EMFA_ERR_UNSUPPORTED;
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

// diagnostics: the FP32 sin/cos(pi x) of the tiled fill, for accuracy tests
namespace {
__global__ void k_diag_sincospi(const float* __restrict__ x, int n, float* __restrict__ s, float* __restrict__ c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) emfa::sincos_pi_taylor(x[i], s + i, c + i);
}
}  // namespace

extern "C" emfa_status_t emfa_diag_sincospi(const float* x_dev, int n, float* s_dev, float* c_dev, void* stream)
{
    if (!x_dev || !s_dev || !c_dev || n <= 0) return EMFA_ERR_INVALID;
    k_diag_sincospi<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(x_dev, n, s_dev, c_dev);
    EMFA_CUDA(nullptr, cudaGetLastError());
    EMFA_CUDA(nullptr, cudaStreamSynchronize((cudaStream_t)stream));
    return EMFA_OK;
}
