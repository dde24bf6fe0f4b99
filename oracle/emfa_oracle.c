/*
 * emfa_oracle.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU restatement of the reference's SIE hot path (xiangwei0909/EMFA) used
 * only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
 * the checker.  The product (libemfa_cuda.so) never links or calls it.
 *
 * Compiled twice by oracle/build_oracle.sh: REAL=float (prefix or32_) and
 * REAL=double (prefix or64_).  Each routine follows the reference's
 * operation order (vector helpers mirror EMComponent/VectorR3.h and
 * VectorC3.h: scalar division is a reciprocal multiply, dot is x+y+z in
 * order), so the float build tracks the reference's FP32 results to a few
 * ulps and the double build its FP64-promoted build.
 *
 * Pinning: tests/test_oracle.py checks this file against the reference
 * binaries built by oracle/build_ref.sh (when the reference is present) and
 * against the committed golden vectors in tests/golden/ (always).
 */
#include <tgmath.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL float
#endif
#ifndef PFX
#define PFX(name) or32_##name
#endif

typedef REAL r_t;

/* The reference calls sin/cos/log/atan/log10 unqualified on float arguments;
 * under g++ these bind to the C double functions, the float argument is
 * widened and the double result rounds back where it meets a float.  The
 * oracle does the same (std::exp of complex<float> and std::sqrt stay float). */
#define DSIN(x) sin((double)(x))
#define DCOS(x) cos((double)(x))
#define DLOG(x) log((double)(x))
#define DATAN(x) atan((double)(x))
#define DLOG10(x) log10((double)(x))
typedef struct { r_t re, im; } cx;
typedef struct { r_t x, y, z; } v3;
typedef struct { cx x, y, z; } c3;

/* ---- constants (EMComponent/Mathdef.h:14-33, Quadrature.h:20-72) ---- */
#define ONE ((r_t)1)
static const r_t PI_ = (r_t)3.14159265358979323846;
#define PI4_ ((r_t)4 * PI_)
#define Z0_ ((r_t)120 * PI_)

static r_t w3c(void) { return ONE / (r_t)3; }
static r_t w7c(int i)
{
    static const double w[7] = {0.112500000000000, 0.062969590272413, 0.062969590272413,
                                0.062969590272413, 0.066197076394253, 0.066197076394253,
                                0.066197076394253};
    return (r_t)w[i] * 2;
}

/* ---- vector helpers mirroring VectorR3.h / VectorC3.h ---- */
static inline v3 V(r_t x, r_t y, r_t z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, r_t d) { return V(a.x * d, a.y * d, a.z * d); }
static inline v3 vdivr(v3 a, r_t d) { r_t m = ONE / d; return V(a.x * m, a.y * m, a.z * m); }
static inline r_t vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b)
{
    return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline r_t vnorm(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline v3 vnormalize(v3 a) { return vdivr(a, vnorm(a)); }

static inline cx C(r_t re, r_t im) { cx r = {re, im}; return r; }
static inline cx cadd(cx a, cx b) { return C(a.re + b.re, a.im + b.im); }
static inline cx csub(cx a, cx b) { return C(a.re - b.re, a.im - b.im); }
static inline cx cmul(cx a, cx b) { return C(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cx cscale(cx a, r_t d) { return C(a.re * d, a.im * d); }
static inline cx cdivr(cx a, r_t d) { return C(a.re / d, a.im / d); }
/* exp(-j x) as std::exp(complex) gives it for a -0 real part */
static inline cx expmj(r_t x) { return C(cos(x), -sin(x)); }
static inline cx exppj(r_t x) { return C(cos(x), sin(x)); }

static inline c3 c3zero(void) { c3 r; r.x = r.y = r.z = C(0, 0); return r; }
static inline c3 c3add(c3 a, c3 b) { c3 r = {cadd(a.x, b.x), cadd(a.y, b.y), cadd(a.z, b.z)}; return r; }
static inline c3 c3sub(c3 a, c3 b) { c3 r = {csub(a.x, b.x), csub(a.y, b.y), csub(a.z, b.z)}; return r; }
static inline c3 c3_vc(v3 u, cx m) { c3 r = {cscale(m, u.x), cscale(m, u.y), cscale(m, u.z)}; return r; }
static inline c3 c3scale(c3 a, cx m) { c3 r = {cmul(a.x, m), cmul(a.y, m), cmul(a.z, m)}; return r; }
static inline c3 c3scaler(c3 a, r_t d) { c3 r = {cscale(a.x, d), cscale(a.y, d), cscale(a.z, d)}; return r; }
/* operator^(VectorR3, VectorC3): vc.x*vr.x + vc.y*vr.y + vc.z*vr.z */
static inline cx vdotc(v3 r, c3 c)
{
    return cadd(cadd(cscale(c.x, r.x), cscale(c.y, r.y)), cscale(c.z, r.z));
}
/* operator*(VectorR3, VectorC3): cross */
static inline c3 vcrossc(v3 r, c3 c)
{
    c3 o;
    o.x = csub(cscale(c.z, r.y), cscale(c.y, r.z));
    o.y = csub(cscale(c.x, r.z), cscale(c.z, r.x));
    o.z = csub(cscale(c.y, r.x), cscale(c.x, r.y));
    return o;
}
static inline c3 c3crossv(c3 c, v3 r)
{
    c3 o;
    o.x = csub(cscale(c.y, r.z), cscale(c.z, r.y));
    o.y = csub(cscale(c.z, r.x), cscale(c.x, r.z));
    o.z = csub(cscale(c.x, r.y), cscale(c.y, r.x));
    return o;
}
static inline r_t c3norm2(c3 a)
{
    return (a.x.re * a.x.re + a.x.im * a.x.im) + (a.y.re * a.y.re + a.y.im * a.y.im) +
           (a.z.re * a.z.re + a.z.im * a.z.im);
}

/* ---- quadrature (Quadrature.cpp:13-53) ---- */
static void gauss3(v3 a, v3 b, v3 c, v3* p)
{
    r_t g0 = (r_t)2 / (r_t)3, g1 = ONE / (r_t)6;
    p[0] = vadd(vadd(vmul(a, g0), vmul(b, g1)), vmul(c, g1));
    p[1] = vadd(vadd(vmul(a, g1), vmul(b, g0)), vmul(c, g1));
    p[2] = vadd(vadd(vmul(a, g1), vmul(b, g1)), vmul(c, g0));
}
static void gauss7(v3 a, v3 b, v3 c, v3* p)
{
    static const double g[7][2] = {{0.333333333333333, 0.333333333333333},
                                   {0.797426985353087, 0.101286507323456},
                                   {0.101286507323456, 0.797426985353087},
                                   {0.101286507323456, 0.101286507323456},
                                   {0.470142064105115, 0.470142064105115},
                                   {0.470142064105115, 0.059715871789770},
                                   {0.059715871789770, 0.470142064105115}};
    for (int i = 0; i < 7; ++i) {
        r_t g0 = (r_t)g[i][0], g1 = (r_t)g[i][1];
        r_t g2 = ONE - g0 - g1;
        p[i] = vadd(vadd(vmul(a, g0), vmul(b, g1)), vmul(c, g2));
    }
}
/* Heron's formula, VectorR3.h Area() */
static r_t tri_area(v3 a, v3 b, v3 c)
{
    r_t la = vnorm(vsub(a, b)), lb = vnorm(vsub(b, c)), lc = vnorm(vsub(c, a));
    r_t ls = (la + lb + lc) / (r_t)2;
    return sqrt(ls * (ls - la) * (ls - lb) * (ls - lc));
}
/* Triangle::getInfo, EMComponent/Triangle.cpp:47-61 */
static v3 tri_normal(v3 A, v3 B, v3 Cc)
{
    v3 ab = vsub(B, A), bc = vsub(Cc, B), ca = vsub(A, Cc);
    v3 n = (vdot(ab, bc) < vdot(bc, ca)) ? vcross(ab, bc) : vcross(bc, ca);
    return vdivr(n, vnorm(n));
}

/* ---- mesh access ---- */
typedef struct {
    const r_t* verts;  /* V x 3 */
    const int* tris;   /* T x 3 */
    const int* rwg;    /* N x 6: v1 v2 vxp vxm tp tm */
    const r_t* len;    /* N */
    int n;
} mesh_t;

static inline v3 vtx(const mesh_t* m, int i)
{
    return V(m->verts[3 * i], m->verts[3 * i + 1], m->verts[3 * i + 2]);
}
static void tri3(const mesh_t* m, int t, v3* o)
{
    o[0] = vtx(m, m->tris[3 * t]);
    o[1] = vtx(m, m->tris[3 * t + 1]);
    o[2] = vtx(m, m->tris[3 * t + 2]);
}

/* ---- EFIE kernels (EMSolver/EFIE.cpp:139-160, 231-566) ---- */
static cx efie_regular(r_t k, const v3* vf3, const v3* vs3, v3 vf, v3 vs)
{
    v3 vgf[3], vgs[3];
    gauss3(vf3[0], vf3[1], vf3[2], vgf);
    gauss3(vs3[0], vs3[1], vs3[2], vgs);
    cx Ze = C(0, 0);
    r_t w = w3c();
    for (int p = 0; p < 3; ++p) {
        v3 rf = vsub(vgf[p], vf);
        for (int q = 0; q < 3; ++q) {
            v3 rs = vsub(vgs[q], vs);
            r_t r = vnorm(vsub(vgf[p], vgs[q]));
            cx G = cdivr(expmj(k * r), r);
            r_t s = w * w * ((r_t)0.25 * vdot(rf, rs) - ONE / (k * k));
            Ze = cadd(Ze, cscale(G, s));
        }
    }
    return Ze;
}

/* sign pattern of eZ{pp,pm,mp,mm}Singular: fs/ss are the field/source signs;
 * proj selects the projected edge-distance form used by pm/mp/mm
 * (EFIE.cpp:344-368) instead of the direct form of pp (EFIE.cpp:260-283). */
static cx efie_singular(r_t k, cx sigma, const v3* vf3, const v3* vs3, v3 vf, v3 vs,
                        r_t fs, r_t ss, int proj)
{
    cx Ze1 = C(0, 0), Ze2 = C(0, 0), Ze3 = C(0, 0);
    v3 vgf[3], vgs[3];
    r_t S_s = tri_area(vs3[0], vs3[1], vs3[2]);
    gauss3(vf3[0], vf3[1], vf3[2], vgf);
    gauss3(vs3[0], vs3[1], vs3[2], vgs);
    r_t w = w3c();
    for (int p = 0; p < 3; ++p) {
        v3 rf = (fs > 0) ? vsub(vgf[p], vf) : vsub(vf, vgf[p]);
        for (int q = 0; q < 3; ++q) {
            v3 rs = (ss > 0) ? vsub(vgs[q], vs) : vsub(vs, vgs[q]);
            r_t r = vnorm(vsub(vgf[p], vgs[q]));
            /* coff = -0.5 k^2 r + j k/6 (k^2 r^2 - 6) */
            cx coff = C((r_t)(-0.5) * k * k * r, (k / (r_t)6) * (k * k * r * r - 6));
            r_t s = w * w * ((r_t)0.25 * vdot(rf, rs) - (fs * ss) / (k * k));
            Ze1 = cadd(Ze1, cscale(coff, s));
        }
        r_t Is2 = 0;
        v3 Is1 = V(0, 0, 0);
        v3 n = vcross(vsub(vs3[1], vs3[0]), vsub(vs3[2], vs3[0]));
        n = vnormalize(n); /* Normalize() normalizes n in place */
        v3 ni = n;
        v3 rou = vsub(vgf[p], vmul(ni, vdot(ni, vgf[p])));
        for (int i = 0; i < 3; ++i) {
            v3 a = vs3[(i + 1) % 3], b = vs3[i];
            v3 li = vsub(a, b);
            v3 rou_p = vsub(a, vmul(ni, vdot(ni, a)));
            v3 rou_m = vsub(b, vmul(ni, vdot(ni, b)));
            v3 u = vcross(li, n);
            v3 ui = vnormalize(u);
            v3 l1 = vnormalize(li);
            r_t p0 = fabs(vdot(vsub(b, vgf[p]), ui));
            r_t d = vdot(vsub(vgf[p], b), ni);
            r_t lp, lm, rp, rm;
            if (!proj) {
                lp = vdot(vsub(a, vgf[p]), l1);
                lm = vdot(vsub(b, vgf[p]), l1);
                rp = vnorm(vsub(vgf[p], a));
                rm = vnorm(vsub(vgf[p], b));
            } else {
                lp = vdot(vsub(rou_p, rou), l1);
                lm = vdot(vsub(rou_m, rou), l1);
                rp = sqrt(p0 * p0 + d * d + lp * lp);
                rm = sqrt(p0 * p0 + d * d + lm * lm);
            }
            if ((double)p0 < 1e-10) continue; /* float compared with a double literal */
            v3 pi = vnormalize(vsub(vsub(rou_p, rou), vmul(l1, lp)));
            r_t r02 = p0 * p0 + d * d;
            double lg = DLOG((rp + lp) / (rm + lm));
            Is1 = vadd(Is1, vmul(vmul(ui, (r_t)0.5), (r_t)((double)r02 * lg + (double)(lp * rp) - (double)(lm * rm))));
            r_t ad = fabs(d);
            Is2 = (r_t)((double)Is2 + (double)vdot(pi, ui) *
                   (((double)p0 * lg) - (double)ad * (DATAN((p0 * lp) / (r02 + ad * rp)) - DATAN((p0 * lm) / (r02 + ad * rm)))));
        }
        v3 rfp = vsub(vgf[p], vf); /* unsigned field rho */
        r_t dotv = vdot(rfp, vadd(Is1, vmul(vsub(vgf[p], vs), Is2)));
        r_t term = fs * ss * ((r_t)0.25 * dotv - Is2 / (k * k));
        Ze2 = cadd(Ze2, C(w * term, 0));
    }
    if (sqrt(sigma.re * sigma.re + sigma.im * sigma.im) > (r_t)1e-8) {
        r_t acc = 0;
        for (int i = 0; i < 3; ++i) acc += vdot(vmul(vsub(vgf[i], vf), w), vsub(vgf[i], vs));
        /* PI*Sigma / (S_s * j k Z0) */
        r_t den = S_s * k * Z0_;
        cx f = C(PI_ * sigma.im / den, -PI_ * sigma.re / den);
        Ze3 = cscale(f, acc);
    }
    cx Ze = cadd(cadd(Ze1, cscale(Ze2, ONE / S_s)), Ze3);
    return Ze;
}

static v3 centroid(const v3* t) { return vdivr(vadd(vadd(t[0], t[1]), t[2]), (r_t)3); }

/* EFIE::EDMKernel, EFIE.cpp:544-566 */
static cx efie_edm(r_t k, const v3* fp3, const v3* fm3, const v3* sp3, const v3* sm3, r_t lf, r_t ls)
{
    v3 fcp = centroid(fp3), fcm = centroid(fm3), scp = centroid(sp3), scm = centroid(sm3);
    v3 r_fld = vdivr(vadd(fcp, fcm), (r_t)2), r_src = vdivr(vadd(scp, scm), (r_t)2);
    v3 R = vsub(r_fld, r_src);
    r_t Rn = vnorm(R);
    v3 m_s = vmul(vsub(scm, scp), ls);
    /* C = (1/R^2)(1 + 1/(j k R)) = (1/R^2)(1 - j/(kR)) */
    cx Cc = C(ONE / (Rn * Rn), -(ONE / (Rn * Rn)) / (k * Rn));
    v3 M_s = vdivr(vmul(R, vdot(R, m_s)), Rn * Rn);
    cx jkR = C(Cc.re, k / Rn + Cc.im);
    c3 E = c3add(c3_vc(vsub(M_s, m_s), jkR), c3_vc(vmul(M_s, 2), Cc));
    cx ph = cscale(expmj(k * Rn), Z0_ / PI4_);
    E = c3scale(E, ph);
    cx dot = vdotc(vsub(fcm, fcp), E);
    return cscale(dot, -lf);
}

/* EFIE::fillZ, EFIE.cpp:603-696.  Z is N x N row-major (f, s).
 * edm_mode 0: far pairs (centre distance > 3 lambda) are zero, as in the
 * Eigen matrix the reference solves; 1: far pairs hold the EDM value (the
 * Armadillo matrix); 2: no EDM branch, quadrature everywhere. */
void PFX(fill_z_efie)(const r_t* verts, const int* tris, const int* rwg, const r_t* len, int n,
                       r_t k, r_t threshold_edm, r_t sig_re, r_t sig_im, int edm_mode, r_t* Zout)
{
    mesh_t m = {verts, tris, rwg, len, n};
    cx sigma = C(sig_re, sig_im);
    cx coef = C(0, k * Z0_ / PI4_);
    for (int f = 0; f < n; ++f) {
        const int* rf = rwg + 6 * f;
        v3 vfp = vtx(&m, rf[2]), vfm = vtx(&m, rf[3]);
        v3 fp3[3], fm3[3];
        tri3(&m, rf[4], fp3);
        tri3(&m, rf[5], fm3);
        r_t lf = len[f];
        v3 fcen = vdivr(vadd(centroid(fp3), centroid(fm3)), (r_t)2);
        for (int s = 0; s < n; ++s) {
            const int* rs = rwg + 6 * s;
            v3 vsp = vtx(&m, rs[2]), vsm = vtx(&m, rs[3]);
            v3 sp3[3], sm3[3];
            tri3(&m, rs[4], sp3);
            tri3(&m, rs[5], sm3);
            r_t ls = len[s];
            v3 scen = vdivr(vadd(centroid(sp3), centroid(sm3)), (r_t)2);
            cx z;
            if (edm_mode != 2 && vnorm(vsub(fcen, scen)) > threshold_edm) {
                z = edm_mode == 1 ? efie_edm(k, fp3, fm3, sp3, sm3, lf, ls) : C(0, 0);
            } else {
                cx zpp = rf[4] == rs[4] ? efie_singular(k, sigma, fp3, sp3, vfp, vsp, 1, 1, 0)
                                        : efie_regular(k, fp3, sp3, vfp, vsp);
                cx zpm = rf[4] == rs[5] ? efie_singular(k, sigma, fp3, sm3, vfp, vsm, 1, -1, 1)
                                        : cscale(efie_regular(k, fp3, sm3, vfp, vsm), -1);
                cx zmp = rf[5] == rs[4] ? efie_singular(k, sigma, fm3, sp3, vfm, vsp, -1, 1, 1)
                                        : cscale(efie_regular(k, fm3, sp3, vfm, vsp), -1);
                cx zmm = rf[5] == rs[5] ? efie_singular(k, sigma, fm3, sm3, vfm, vsm, -1, -1, 1)
                                        : efie_regular(k, fm3, sm3, vfm, vsm);
                cx sum = cadd(cadd(cadd(zpp, zpm), zmp), zmm);
                z = cmul(cscale(cscale(coef, lf), ls), sum);
            }
            Zout[2 * ((size_t)f * n + s)] = z.re;
            Zout[2 * ((size_t)f * n + s) + 1] = z.im;
        }
    }
}

/* ---- CFIE kernels (EMSolver/Miscellaneous.cpp:6-77) ---- */
static cx cfie_regular(r_t alpha, r_t k, const v3* vf3, const v3* vs3, v3 vf, v3 vs, v3 nf,
                       r_t fs, r_t ss)
{
    v3 vgf[3], vgs[3];
    gauss3(vf3[0], vf3[1], vf3[2], vgf);
    gauss3(vs3[0], vs3[1], vs3[2], vgs);
    cx Ze = C(0, 0), Zm = C(0, 0);
    r_t w = w3c();
    for (int p = 0; p < 3; ++p) {
        v3 rf = vmul(vsub(vgf[p], vf), fs);
        for (int q = 0; q < 3; ++q) {
            v3 rs = vmul(vsub(vgs[q], vs), ss);
            v3 dv = vsub(vgf[p], vgs[q]);
            r_t r = vnorm(dv);
            cx G = cdivr(expmj(k * r), r);
            r_t s = w * w * ((r_t)0.25 * vdot(rf, rs) - (fs * ss) / (k * k));
            Ze = cadd(Ze, cscale(G, s));
            r_t m = w * w * vdot(rf, vcross(nf, vcross(dv, rs)));
            cx t = cmul(C(m, m * (k * r)), G);
            Zm = cadd(Zm, cdivr(t, r * r));
        }
    }
    Ze = cmul(C(0, k * Z0_ / PI4_), Ze);
    Zm = cdivr(Zm, (r_t)16 * PI_);
    return cadd(cscale(Ze, alpha), cscale(Zm, (ONE - alpha) * Z0_));
}

static cx cfie_singular(r_t alpha, r_t k, const v3* vf3, const v3* vs3, v3 vf, v3 vs, r_t fs, r_t ss)
{
    v3 vgf[3], vgs[3];
    gauss3(vf3[0], vf3[1], vf3[2], vgf);
    gauss3(vs3[0], vs3[1], vs3[2], vgs);
    cx Ze1 = C(0, 0), Ze2 = C(0, 0);
    r_t Zm = 0;
    r_t area = tri_area(vf3[0], vf3[1], vf3[2]);
    r_t w = w3c();
    v3 rs = V(0, 0, 0);
    for (int p = 0; p < 3; ++p) {
        v3 rf = vmul(vsub(vgf[p], vf), fs);
        for (int q = 0; q < 3; ++q) {
            rs = vmul(vsub(vgs[q], vs), ss);
            r_t r = vnorm(vsub(vgf[p], vgs[q]));
            cx coff = C((r_t)(-0.5) * k * k * r, (k / (r_t)6) * (k * k * r * r - 6));
            r_t s = w * w * ((r_t)0.25 * vdot(rf, rs) - (fs * ss) / (k * k));
            Ze1 = cadd(Ze1, cscale(coff, s));
        }
        /* rs is left over from the last q iteration (q = 2), as in the reference */
        for (int i = 0; i < 3; ++i) {
            v3 Li = vnormalize(vsub(vs3[(i + 1) % 3], vs3[i]));
            r_t Lp = vdot(vsub(vs3[(i + 1) % 3], vgf[p]), Li);
            r_t Lm = vdot(vsub(vs3[i], vgf[p]), Li);
            r_t Rp = vnorm(vsub(vs3[(i + 1) % 3], vgf[p]));
            r_t Rm = vnorm(vsub(vs3[i], vgf[p]));
            v3 sj0 = vadd(vs3[i], vmul(Li, vdot(vsub(vgf[p], vs3[i]), Li)));
            r_t P0 = vnorm(vsub(sj0, vgf[p]));
            if (P0 > (r_t)1e-10) {
                double s = (double)(w * ((r_t)0.25 * vdot(rf, rs) - (fs * ss) / (k * k)) * P0) *
                           DLOG((Rp + Lp) / (Rm + Lm));
                Ze2 = cadd(Ze2, C((r_t)s, 0));
            }
        }
        v3 rf2 = vmul(vsub(vgf[p], vf), fs);
        v3 rs2 = vmul(vsub(vgs[p], vs), ss);
        Zm += w * vdot(rf2, rs2);
    }
    cx Ze = cmul(C(0, k * Z0_ / PI4_), cadd(Ze1, cscale(Ze2, ONE / area)));
    r_t zm = Zm / ((r_t)8 * area);
    return cadd(cscale(Ze, alpha), C((ONE - alpha) * Z0_ * zm, 0));
}

/* CFIE::fillZ, EMSolver/CFIE.cpp:485-568; normals are those of the field
 * triangles (Triangle::getNormal). */
void PFX(fill_z_cfie)(const r_t* verts, const int* tris, const int* rwg, const r_t* len, int n,
                       r_t k, r_t alpha, r_t* Zout)
{
    mesh_t m = {verts, tris, rwg, len, n};
    for (int f = 0; f < n; ++f) {
        const int* rf = rwg + 6 * f;
        v3 vfp = vtx(&m, rf[2]), vfm = vtx(&m, rf[3]);
        v3 fp3[3], fm3[3];
        tri3(&m, rf[4], fp3);
        tri3(&m, rf[5], fm3);
        v3 np = tri_normal(fp3[0], fp3[1], fp3[2]), nm = tri_normal(fm3[0], fm3[1], fm3[2]);
        r_t lf = len[f];
        for (int s = 0; s < n; ++s) {
            const int* rs = rwg + 6 * s;
            v3 vsp = vtx(&m, rs[2]), vsm = vtx(&m, rs[3]);
            v3 sp3[3], sm3[3];
            tri3(&m, rs[4], sp3);
            tri3(&m, rs[5], sm3);
            r_t ls = len[s];
            cx zpp = rf[4] == rs[4] ? cfie_singular(alpha, k, fp3, sp3, vfp, vsp, 1, 1)
                                    : cfie_regular(alpha, k, fp3, sp3, vfp, vsp, np, 1, 1);
            cx zpm = rf[4] == rs[5] ? cfie_singular(alpha, k, fp3, sm3, vfp, vsm, 1, -1)
                                    : cfie_regular(alpha, k, fp3, sm3, vfp, vsm, np, 1, -1);
            cx zmp = rf[5] == rs[4] ? cfie_singular(alpha, k, fm3, sp3, vfm, vsp, -1, 1)
                                    : cfie_regular(alpha, k, fm3, sp3, vfm, vsp, nm, -1, 1);
            cx zmm = rf[5] == rs[5] ? cfie_singular(alpha, k, fm3, sm3, vfm, vsm, -1, -1)
                                    : cfie_regular(alpha, k, fm3, sm3, vfm, vsm, nm, -1, -1);
            cx sum = cadd(cadd(cadd(zpp, zpm), zmp), zmm);
            cx z = cscale(sum, lf * ls);
            Zout[2 * ((size_t)f * n + s)] = z.re;
            Zout[2 * ((size_t)f * n + s) + 1] = z.im;
        }
    }
}

/* ---- excitation (EFIE.cpp:568-601,698-722; Miscellaneous.cpp:152-189) ----
 * inc: per incidence 9 values k_hat(3), e_hat(3), h_hat(3).  V is
 * n_inc x N row-major. */
void PFX(fill_v)(const r_t* verts, const int* tris, const int* rwg, const r_t* len, int n,
                  r_t k, int cfie, r_t alpha, const r_t* inc, int n_inc, r_t* Vout)
{
    mesh_t m = {verts, tris, rwg, len, n};
    for (int a = 0; a < n_inc; ++a) {
        v3 kk = V(inc[9 * a], inc[9 * a + 1], inc[9 * a + 2]);
        v3 ee = V(inc[9 * a + 3], inc[9 * a + 4], inc[9 * a + 5]);
        v3 hh = V(inc[9 * a + 6], inc[9 * a + 7], inc[9 * a + 8]);
        for (int u = 0; u < n; ++u) {
            const int* r = rwg + 6 * u;
            v3 vp = vtx(&m, r[2]), vm = vtx(&m, r[3]);
            v3 p3[3], m3[3];
            tri3(&m, r[4], p3);
            tri3(&m, r[5], m3);
            cx vk;
            if (!cfie) {
                v3 gp[7], gm[7];
                gauss7(p3[0], p3[1], p3[2], gp);
                gauss7(m3[0], m3[1], m3[2], gm);
                cx Vep = C(0, 0), Vem = C(0, 0);
                for (int i = 0; i < 7; ++i) {
                    r_t w = w7c(i);
                    cx G = expmj(k * vdot(gp[i], kk));
                    Vep = cadd(Vep, cscale(vdotc(vsub(gp[i], vp), c3_vc(ee, G)), w));
                    G = expmj(k * vdot(gm[i], kk));
                    Vem = cadd(Vem, cscale(vdotc(vsub(vm, gm[i]), c3_vc(ee, G)), w));
                }
                vk = cadd(Vep, Vem);
            } else {
                v3 gp[3], gm[3];
                gauss3(p3[0], p3[1], p3[2], gp);
                gauss3(m3[0], m3[1], m3[2], gm);
                v3 np = tri_normal(p3[0], p3[1], p3[2]), nm = tri_normal(m3[0], m3[1], m3[2]);
                cx Vep = C(0, 0), Vem = C(0, 0), Vmp = C(0, 0), Vmm = C(0, 0);
                r_t w = w3c();
                for (int i = 0; i < 3; ++i) {
                    v3 rp = vsub(gp[i], vp);
                    cx G = expmj(k * vdot(gp[i], kk));
                    Vep = cadd(Vep, cscale(vdotc(rp, c3_vc(ee, G)), w));
                    Vmp = cadd(Vmp, cscale(vdotc(rp, vcrossc(np, c3_vc(hh, G))), w));
                    v3 rm = vsub(vm, gm[i]);
                    G = expmj(k * vdot(gm[i], kk));
                    Vem = cadd(Vem, cscale(vdotc(rm, c3_vc(ee, G)), w));
                    Vmm = cadd(Vmm, cscale(vdotc(rm, vcrossc(nm, c3_vc(hh, G))), w));
                }
                vk = cadd(cscale(cadd(Vep, Vem), alpha), cscale(cadd(Vmp, Vmm), ONE - alpha));
            }
            cx v = cscale(vk, (r_t)0.5 * len[u]);
            Vout[2 * ((size_t)a * n + u)] = v.re;
            Vout[2 * ((size_t)a * n + u) + 1] = v.im;
        }
    }
}

/* ---- bistatic RCS (EFIE.cpp:788-832, CFIE.cpp:643-685) ----
 * I: n_rhs x N currents; dirs: n_dir x 3 scattering directions.
 * out: n_rhs x n_dir, 10 log10(sigma). */
void PFX(rcs)(const r_t* verts, const int* tris, const int* rwg, const r_t* len, int n, r_t k,
               const r_t* cur, int n_rhs, const r_t* dirs, int n_dir, r_t* out)
{
    mesh_t m = {verts, tris, rwg, len, n};
    for (int a = 0; a < n_rhs; ++a) {
        for (int d = 0; d < n_dir; ++d) {
            v3 sk = V(dirs[3 * d], dirs[3 * d + 1], dirs[3 * d + 2]);
            c3 Es = c3zero();
            for (int u = 0; u < n; ++u) {
                const int* r = rwg + 6 * u;
                v3 vp = vtx(&m, r[2]), vm = vtx(&m, r[3]);
                v3 p3[3], m3[3], gp[7], gm[7];
                tri3(&m, r[4], p3);
                tri3(&m, r[5], m3);
                gauss7(p3[0], p3[1], p3[2], gp);
                gauss7(m3[0], m3[1], m3[2], gm);
                c3 Esp = c3zero(), Esm = c3zero();
                for (int g = 0; g < 7; ++g) {
                    r_t w = w7c(g);
                    Esp = c3add(Esp, c3_vc(vmul(vsub(gp[g], vp), w), exppj(k * vdot(gp[g], sk))));
                    Esm = c3add(Esm, c3_vc(vmul(vsub(vm, gm[g]), w), exppj(k * vdot(gm[g], sk))));
                }
                cx Iu = C(cur[2 * ((size_t)a * n + u)], cur[2 * ((size_t)a * n + u) + 1]);
                Es = c3add(Es, c3scale(c3add(Esp, Esm), cscale(Iu, len[u])));
            }
            c3 es = vcrossc(vmul(sk, (r_t)0.5), vcrossc(sk, Es));
            r_t rcs = Z0_ * Z0_ * k * k * c3norm2(es) / PI4_;
            out[(size_t)a * n_dir + d] = (r_t)(10 * DLOG10(rcs));
        }
    }
}

/* ---- normals and quadrature points (geometry pack) ---- */
void PFX(tri_geometry)(const r_t* verts, const int* tris, int nt, r_t* normals, r_t* q3, r_t* q7,
                        r_t* area)
{
    mesh_t m = {verts, tris, 0, 0, 0};
    for (int t = 0; t < nt; ++t) {
        v3 v[3], g3[3], g7[7];
        tri3(&m, t, v);
        v3 nn = tri_normal(v[0], v[1], v[2]);
        normals[3 * t] = nn.x; normals[3 * t + 1] = nn.y; normals[3 * t + 2] = nn.z;
        gauss3(v[0], v[1], v[2], g3);
        gauss7(v[0], v[1], v[2], g7);
        for (int i = 0; i < 3; ++i) {
            q3[9 * t + 3 * i] = g3[i].x; q3[9 * t + 3 * i + 1] = g3[i].y; q3[9 * t + 3 * i + 2] = g3[i].z;
        }
        for (int i = 0; i < 7; ++i) {
            q7[21 * t + 3 * i] = g7[i].x; q7[21 * t + 3 * i + 1] = g7[i].y; q7[21 * t + 3 * i + 2] = g7[i].z;
        }
        area[t] = tri_area(v[0], v[1], v[2]);
    }
}

/* ---- incidence vectors (EMSolver/EM.cpp:33-38) ---- */
void PFX(incidence)(r_t theta_deg, r_t phi_deg, r_t pole_deg, r_t* out9)
{
    r_t d2r = PI_ / (r_t)180;
    r_t pol = pole_deg * d2r, th = theta_deg * d2r, ph = phi_deg * d2r;
    /* EM.cpp:33-34: products of the double-valued sin/cos, rounded once */
    v3 kk = V((r_t)(-DSIN(th) * DCOS(ph)), (r_t)(-DSIN(th) * DSIN(ph)), (r_t)(-DCOS(th)));
    v3 ee = V((r_t)(-DCOS(pol) * DCOS(th) * DCOS(ph) - DSIN(pol) * DSIN(ph)),
              (r_t)(-DCOS(pol) * DCOS(th) * DSIN(ph) + DSIN(pol) * DCOS(ph)), (r_t)(DCOS(pol) * DSIN(th)));
    v3 hh = vcross(kk, ee);
    r_t o[9] = {kk.x, kk.y, kk.z, ee.x, ee.y, ee.z, hh.x, hh.y, hh.z};
    memcpy(out9, o, sizeof o);
}

/* ---- the configurations' discretisation of the EFIE (not the reference's):
 * 7 x 7-point regular pairs, singularity extraction on self and
 * edge-adjacent triangle pairs.  For a singular pair, with
 * G = e^{-jkR}/R = 1/R + Gs(R), Gs = (e^{-jkR} - 1)/R (Gs(0) = -jk):
 *   sum_p sum_q w_p w_q [(P_p - vf).(Q_q - vs)/4 - 1/k^2] Gs(R_pq)
 * + sum_p w_p [(P_p - vf).(I_rho(P_p) + (rho_p - vs) I_1(P_p))/4
 *              - I_1(P_p)/k^2] / A_s
 * where I_1 = int 1/R and I_rho = int (rho' - rho)/R over the source
 * triangle are the closed forms of Wilton et al. (IEEE Trans. Antennas
 * Propag. 32, 1984, pp. 276-281) for an observation point anywhere.  Pairs
 * are adjacent when the triangles share two vertex indices. ---- */
void PFX(potential_integrals)(const r_t* tri9, const r_t* r3, r_t* I1_out, r_t* Irho3)
{
    v3 t[3] = {V(tri9[0], tri9[1], tri9[2]), V(tri9[3], tri9[4], tri9[5]), V(tri9[6], tri9[7], tri9[8])};
    v3 r = V(r3[0], r3[1], r3[2]);
    v3 n = vnormalize(vcross(vsub(t[1], t[0]), vsub(t[2], t[0])));
    r_t h = vdot(vsub(r, t[0]), n), ah = fabs(h);
    v3 rho = vsub(r, vmul(n, h));
    r_t I1 = 0;
    v3 Ir = V(0, 0, 0);
    for (int i = 0; i < 3; ++i) {
        v3 b = t[i], a = t[(i + 1) % 3];
        v3 l = vnormalize(vsub(a, b));
        v3 u = vcross(l, n);
        r_t lp = vdot(vsub(a, rho), l), lm = vdot(vsub(b, rho), l);
        r_t sd = vdot(vsub(b, rho), u);
        r_t p0 = fabs(sd);
        r_t r02 = p0 * p0 + h * h;
        r_t rp = sqrt(r02 + lp * lp), rm = sqrt(r02 + lm * lm);
        r_t lg = 0;
        if (r02 > 0) {
            /* R + l, written R0^2 / (R - l) where l < 0 (no cancellation) */
            r_t fa = lp >= 0 ? rp + lp : r02 / (rp - lp);
            r_t fb = lm >= 0 ? rm + lm : r02 / (rm - lm);
            lg = log(fa / fb);
        }
        Ir = vadd(Ir, vmul(u, (r_t)0.5 * (r02 * lg + lp * rp - lm * rm)));
        if (p0 > 0) {
            r_t sg = sd > 0 ? ONE : -ONE;
            I1 += sg * (p0 * lg - ah * (atan(p0 * lp / (r02 + ah * rp)) - atan(p0 * lm / (r02 + ah * rm))));
        }
    }
    *I1_out = I1;
    Irho3[0] = Ir.x;
    Irho3[1] = Ir.y;
    Irho3[2] = Ir.z;
}

static cx efie_cfg_pair(r_t k, cx sigma, const v3* vf3, const v3* vs3, v3 vf, v3 vs, int self, int singular)
{
    v3 P[7], Q[7];
    gauss7(vf3[0], vf3[1], vf3[2], P);
    gauss7(vs3[0], vs3[1], vs3[2], Q);
    r_t ik2 = ONE / (k * k);
    cx z = C(0, 0);
    for (int p = 0; p < 7; ++p) {
        v3 rf = vsub(P[p], vf);
        for (int q = 0; q < 7; ++q) {
            r_t R = vnorm(vsub(P[p], Q[q]));
            r_t e = w7c(p) * w7c(q) * ((r_t)0.25 * vdot(rf, vsub(Q[q], vs)) - ik2);
            cx g;
            if (!singular) {
                g = cdivr(expmj(k * R), R);
            } else if (R > 0) {
                r_t sh = sin((r_t)0.5 * k * R);
                g = C((r_t)-2 * sh * sh / R, -sin(k * R) / R);
            } else {
                g = C(0, -k);
            }
            z = cadd(z, cscale(g, e));
        }
    }
    if (singular) {
        r_t As = tri_area(vs3[0], vs3[1], vs3[2]);
        v3 ns = vnormalize(vcross(vsub(vs3[1], vs3[0]), vsub(vs3[2], vs3[0])));
        r_t tri9[9] = {vs3[0].x, vs3[0].y, vs3[0].z, vs3[1].x, vs3[1].y, vs3[1].z, vs3[2].x, vs3[2].y, vs3[2].z};
        r_t acc = 0;
        for (int p = 0; p < 7; ++p) {
            r_t r3[3] = {P[p].x, P[p].y, P[p].z}, I1, Ir3[3];
            PFX(potential_integrals)(tri9, r3, &I1, Ir3);
            v3 rho = vsub(P[p], vmul(ns, vdot(vsub(P[p], vs3[0]), ns)));
            v3 rs = vadd(V(Ir3[0], Ir3[1], Ir3[2]), vmul(vsub(rho, vs), I1));
            acc += w7c(p) * ((r_t)0.25 * vdot(vsub(P[p], vf), rs) - I1 * ik2);
        }
        z.re += acc / As;
        if (self && sqrt(sigma.re * sigma.re + sigma.im * sigma.im) > (r_t)1e-8) {
            r_t s2 = 0;
            for (int i = 0; i < 7; ++i) s2 += w7c(i) * vdot(vsub(P[i], vf), vsub(P[i], vs));
            r_t den = As * k * Z0_;
            z.re += PI_ * sigma.im / den * s2;
            z.im -= PI_ * sigma.re / den * s2;
        }
    }
    return z;
}

static int shares_edge(const int* a, const int* b)
{
    int c = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) c += a[i] == b[j];
    return c >= 2;
}

void PFX(fill_z_efie_cfg)(const r_t* verts, const int* tris, const int* rwg, const r_t* len, int n, r_t k,
                           r_t sig_re, r_t sig_im, r_t* Zout)
{
    mesh_t m = {verts, tris, rwg, len, n};
    cx sigma = C(sig_re, sig_im);
    cx coef = C(0, k * Z0_ / PI4_);
    for (int f = 0; f < n; ++f) {
        const int* rf = rwg + 6 * f;
        v3 vff[2] = {vtx(&m, rf[2]), vtx(&m, rf[3])};
        v3 tf[2][3];
        tri3(&m, rf[4], tf[0]);
        tri3(&m, rf[5], tf[1]);
        for (int s = 0; s < n; ++s) {
            const int* rs = rwg + 6 * s;
            v3 vss[2] = {vtx(&m, rs[2]), vtx(&m, rs[3])};
            v3 ts[2][3];
            tri3(&m, rs[4], ts[0]);
            tri3(&m, rs[5], ts[1]);
            cx sum = C(0, 0);
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b) {
                    int ia = rf[4 + a], ib = rs[4 + b];
                    int self = ia == ib;
                    int sing = self || shares_edge(tris + 3 * ia, tris + 3 * ib);
                    cx z = efie_cfg_pair(k, sigma, tf[a], ts[b], vff[a], vss[b], self, sing);
                    sum = cadd(sum, cscale(z, a == b ? ONE : -ONE));
                }
            cx zz = cmul(cscale(cscale(coef, len[f]), len[s]), sum);
            Zout[2 * ((size_t)f * n + s)] = zz.re;
            Zout[2 * ((size_t)f * n + s) + 1] = zz.im;
        }
    }
}
