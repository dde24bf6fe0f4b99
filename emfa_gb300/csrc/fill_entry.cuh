// Per-entry impedance computation shared by the dense fill (fill.cu) and the
// MLFMA near-field fill (mlfma.cu).
#pragma once
#include "emfa_internal.cuh"
#include "emfa_math.cuh"

namespace emfa {

// ---------------------------------------------------------------------------
// entry kernel: one thread per Z(f, s); a warp runs 32 consecutive s of one f
// ---------------------------------------------------------------------------
template <typename T>
struct FillConst {
    T k, kpi, inv_k2;      // k, k / pi, 1 / k^2
    T ce, cm;              // regular-pair scale: EFIE ce = w^2; CFIE ce = alpha k Z0 w^2 / 4pi, cm = (1-alpha) Z0 w^2 / 16pi
    double coef_efie;      // EFIE: k Z0 / 4pi (the j is applied in the epilogue)
    T thr_edm;             // 3 lambda
    int edm_mode;
    T z0, pi;
};

// regular pair, unsigned: ze = sum_pq (rf.rs/4 - 1/k^2) G,
// zm = sum_pq [rf . (n x (d x rs))] (1 + j kR) G / R^2  (d = P_p - Q_q)
template <typename T, bool MFIE>
__device__ __forceinline__ void regular_pair(const T (&P)[3][3], const T (&Q)[3][3], const T (&vf)[3],
                                             const T (&vs)[3], const T (&nf)[3], const FillConst<T>& c,
                                             Cx<T>& ze, Cx<T>& zm)
{
    V3<T> n = v3(nf[0], nf[1], nf[2]);
    V3<T> rs[3];
    T nrs[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        rs[q] = v3(Q[q][0] - vs[0], Q[q][1] - vs[1], Q[q][2] - vs[2]);
        nrs[q] = dot(n, rs[q]);
    }
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        V3<T> pp = v3(P[p][0], P[p][1], P[p][2]);
        V3<T> rf = v3(P[p][0] - vf[0], P[p][1] - vf[1], P[p][2] - vf[2]);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            V3<T> d = v3(pp.x - Q[q][0], pp.y - Q[q][1], pp.z - Q[q][2]);
            // IEEE sqrt and reciprocal: the four triangle-pair terms of a far
            // RWG pair nearly cancel, so G needs every bit it can keep
            T r = sqrt(dot(d, d));
            T rinv = T(1) / r;
            T sn, cs;
            sincos_pi(r * c.kpi, &sn, &cs);
            T gr = cs * rinv, gi = -sn * rinv;
            T rfrs = dot(rf, rs[q]);
            T e = T(0.25) * rfrs - c.inv_k2;
            ze.re += e * gr;
            ze.im += e * gi;
            if (MFIE) {
                T m = dot(rf, d) * nrs[q] - rfrs * dot(n, d);
                T t = m * (rinv * rinv);
                T kr = r * c.k;
                T hr = gr - kr * gi, hi = gi + kr * gr;
                zm.re += t * hr;
                zm.im += t * hi;
            }
        }
    }
}

template <typename T>
__device__ __forceinline__ void load_side(const RwgPack<T>& pk, int s, T (&q)[3][3], T (&v)[3], T (&n)[3])
{
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) q[i][j] = pk.q3[s][i][j];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        v[j] = pk.v[s][j];
        n[j] = pk.n[s][j];
    }
}

// EFIE::EDMKernel (EFIE.cpp:544-566)
template <typename T>
__device__ Cx<T> edm_value(const RwgPack<T>& F, const RwgPack<T>& S, const FillConst<T>& c)
{
    V3<T> fcp = v3(F.cen[0][0], F.cen[0][1], F.cen[0][2]), fcm = v3(F.cen[1][0], F.cen[1][1], F.cen[1][2]);
    V3<T> scp = v3(S.cen[0][0], S.cen[0][1], S.cen[0][2]), scm = v3(S.cen[1][0], S.cen[1][1], S.cen[1][2]);
    V3<T> R = divr(fcp + fcm, T(2)) - divr(scp + scm, T(2));
    T Rn = norm(R);
    V3<T> ms = (scm - scp) * S.len;
    T ir2 = T(1) / (Rn * Rn);
    Cx<T> C = cx(ir2, -ir2 / (c.k * Rn));
    V3<T> Ms = divr(R * dot(R, ms), Rn * Rn);
    Cx<T> f1 = cx(C.re, c.k / Rn + C.im);
    T sn, cs;
    sincos_pi(Rn * c.kpi, &sn, &cs);
    Cx<T> ph = cx(cs, -sn) * (c.z0 / (T(4) * c.pi));
    V3<T> a = Ms - ms, b = Ms * T(2);
    V3<T> dl = fcm - fcp;
    // E . dl with E = (a f1 + b C) ph
    Cx<T> e = f1 * dot(a, dl) + C * dot(b, dl);
    e = e * ph;
    return e * (-F.len);
}

// One impedance entry Z(f, s) (EFIE or CFIE), regular pairs in T, self
// terms from the FP64 table: EFIE::fillZ / CFIE::fillZ loop body
// (EMSolver/EFIE.cpp:627-694, EMSolver/CFIE.cpp:515-566).
template <typename T, bool CFIE>
__device__ __forceinline__ Cx<T> z_entry(const RwgPack<T>& F, const RwgPack<T>& S, const FillConst<T>& c,
                                         const double2* __restrict__ sing)
{
    if (!CFIE && c.edm_mode != 2) {
        V3<T> fc = divr(v3(F.cen[0][0], F.cen[0][1], F.cen[0][2]) + v3(F.cen[1][0], F.cen[1][1], F.cen[1][2]), T(2));
        V3<T> sc = divr(v3(S.cen[0][0], S.cen[0][1], S.cen[0][2]) + v3(S.cen[1][0], S.cen[1][1], S.cen[1][2]), T(2));
        if (norm(fc - sc) > c.thr_edm) return c.edm_mode == 1 ? edm_value(F, S, c) : cx(T(0), T(0));
    }
    Cx<T> ze = cx(T(0), T(0)), zm = cx(T(0), T(0));
    double sr = 0.0, si = 0.0;
#pragma unroll 1
    for (int a = 0; a < 2; ++a) {
        T P[3][3], vf[3], nf[3];
        load_side(F, a, P, vf, nf);
#pragma unroll 1
        for (int b = 0; b < 2; ++b) {
            T sgn = (a == b) ? T(1) : T(-1);
            if (F.tri[a] == S.tri[b]) {
                int id = 9 * F.tri[a] + 3 * F.e[a] + S.e[b];
                if (CFIE) {
                    double2 v = sing[id];
                    sr += (double)sgn * v.x;
                    si += (double)sgn * v.y;
                } else {
                    double2 v = sing[3 * id + ((a == 0 && b == 0) ? 0 : 1)];
                    double2 g = sing[3 * id + 2];
                    sr += (double)sgn * v.x + g.x;
                    si += (double)sgn * v.y + g.y;
                }
                continue;
            }
            T Q[3][3], vs[3], ns[3];
            load_side(S, b, Q, vs, ns);
            Cx<T> e = cx(T(0), T(0)), m = cx(T(0), T(0));
            regular_pair<T, CFIE>(P, Q, vf, vs, nf, c, e, m);
            ze.re += sgn * e.re;
            ze.im += sgn * e.im;
            if (CFIE) {
                zm.re += sgn * m.re;
                zm.im += sgn * m.im;
            }
        }
    }
    T l = F.len * S.len;
    if (CFIE) {
        // lf ls [ j ce ze + cm zm + singular ]
        T re = -c.ce * ze.im + c.cm * zm.re + (T)sr;
        T im = c.ce * ze.re + c.cm * zm.im + (T)si;
        return cx(re * l, im * l);
    }
    // j (k Z0 / 4pi) lf ls (w^2 ze + singular)
    T kz = (T)c.coef_efie * l;
    T re = c.ce * ze.re + (T)sr, im = c.ce * ze.im + (T)si;
    return cx(-kz * im, kz * re);
}

// fill constants for precision T from the C ABI parameters
template <typename T>
inline FillConst<T> make_fill_const(const emfa_fill_params_t* p)
{
    FillConst<T> fc;
    const T pi = Phys<T>::pi(), z0 = Phys<T>::z0();
    T kt = Phys<T>::wavenumber(p->freq);
    T w = T(1) / T(3);
    T w2 = w * w;
    fc.k = kt;
    fc.kpi = kt / pi;
    fc.inv_k2 = T(1) / (kt * kt);
    fc.pi = pi;
    fc.z0 = z0;
    if (p->kind == EMFA_CFIE) {
        fc.ce = (T)p->alpha * (kt * z0 / (T(4) * pi)) * w2;
        fc.cm = (T(1) - (T)p->alpha) * (z0 / (T(16) * pi)) * w2;
    } else {
        fc.ce = w2;
        fc.cm = 0;
    }
    fc.coef_efie = (double)(kt * z0 / (T(4) * pi));
    fc.thr_edm = T(3) * Phys<T>::c0() / (T)p->freq;
    fc.edm_mode = p->edm_mode;
    return fc;
}

// FP64 self-term table (9 or 27 double2 per triangle), fill.cu
emfa_status_t build_singular_table(Ctx* c, Geom* g, const emfa_fill_params_t* p, double2* tab, cudaStream_t st);

}  // namespace emfa
