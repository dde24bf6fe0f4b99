// Device-side 3-vector and complex helpers, templated on float / double.
// Vector helpers follow the operation order of EMComponent/VectorR3.h
// (dot = x*x' + y*y' + z*z' left to right; division by a scalar is a
// multiplication by its reciprocal), so geometry derived on the device
// (Gauss points, normals, lengths) equals the reference's own values.
#pragma once
#include <cuda_runtime.h>

namespace emfa {

template <typename T> struct V3 { T x, y, z; };
template <typename T> struct Cx { T re, im; };

template <typename T> __host__ __device__ __forceinline__ V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <typename T> __host__ __device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> __host__ __device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> __host__ __device__ __forceinline__ V3<T> operator*(V3<T> a, T d) { return v3(a.x * d, a.y * d, a.z * d); }
template <typename T> __host__ __device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> __host__ __device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename T> __host__ __device__ __forceinline__ T norm(V3<T> a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
template <typename T> __host__ __device__ __forceinline__ V3<T> divr(V3<T> a, T d) { T m = T(1) / d; return a * m; }
template <typename T> __host__ __device__ __forceinline__ V3<T> normalized(V3<T> a) { return divr(a, norm(a)); }

template <typename T> __host__ __device__ __forceinline__ Cx<T> cx(T re, T im) { return Cx<T>{re, im}; }
template <typename T> __host__ __device__ __forceinline__ Cx<T> operator+(Cx<T> a, Cx<T> b) { return cx(a.re + b.re, a.im + b.im); }
template <typename T> __host__ __device__ __forceinline__ Cx<T> operator-(Cx<T> a, Cx<T> b) { return cx(a.re - b.re, a.im - b.im); }
template <typename T> __host__ __device__ __forceinline__ Cx<T> operator*(Cx<T> a, Cx<T> b)
{
    return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T> __host__ __device__ __forceinline__ Cx<T> operator*(Cx<T> a, T d) { return cx(a.re * d, a.im * d); }
template <typename T> __host__ __device__ __forceinline__ Cx<T> conjmul(Cx<T> a, Cx<T> b)  // conj(a) * b
{
    return cx(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re);
}

template <typename T> __device__ __forceinline__ V3<T> ld3(const T* p) { return v3(p[0], p[1], p[2]); }
template <typename T> __device__ __forceinline__ void st3(T* p, V3<T> v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

// sin/cos of pi*x; CUDA's accurate sincospi for both precisions.
__device__ __forceinline__ void sincos_pi(float x, float* s, float* c) { sincospif(x, s, c); }

// sin/cos of pi*x in FP32 from the Taylor series of sin and cos, this
// project's own: x = n/2 + r with n = rint(2x), |r| <= 1/4 (exact in FP32),
// then sin(pi r) = r (pi - pi^3/6 r^2 + ... + pi^9/9! r^8) and
// cos(pi r) = 1 - pi^2/2 r^2 + ... - pi^10/10! r^10 (the first omitted terms
// are below 2e-9 at |pi r| = pi/4), and the quadrant n mod 4 picks and signs
// them.  All FP32 and integer: no branch, no FP64 and no float/int
// conversion (those issue on GB300's slow FP64/conversion pipe): 2x is
// rounded by adding 1.5 * 2^23, whose low mantissa bits then hold n mod 4.
// Valid for |x| < 2^21.  About 1.5 ulp against the exact values.
namespace taylor {
constexpr double PI = 3.14159265358979323846;
constexpr float S1 = (float)PI, S3 = (float)(-PI * PI * PI / 6.0), S5 = (float)(PI * PI * PI * PI * PI / 120.0);
constexpr float S7 = (float)(-PI * PI * PI * PI * PI * PI * PI / 5040.0);
constexpr float S9 = (float)(PI * PI * PI * PI * PI * PI * PI * PI * PI / 362880.0);
constexpr float C2 = (float)(-PI * PI / 2.0), C4 = (float)(PI * PI * PI * PI / 24.0);
constexpr float C6 = (float)(-PI * PI * PI * PI * PI * PI / 720.0);
constexpr float C8 = (float)(PI * PI * PI * PI * PI * PI * PI * PI / 40320.0);
constexpr float C10 = (float)(-PI * PI * PI * PI * PI * PI * PI * PI * PI * PI / 3628800.0);
}  // namespace taylor

__device__ __forceinline__ void sincos_pi_taylor(float x, float* s, float* c)
{
    using namespace taylor;
    const float big = 12582912.0f;  // 1.5 * 2^23
    const float t = fmaf(2.0f, x, big);  // big + rint(2x), one rounding
    const float n = t - big;            // rint(2x), exact
    const float r = fmaf(-0.5f, n, x);
    const float u = r * r;
    const float sv = r * fmaf(fmaf(fmaf(fmaf(S9, u, S7), u, S5), u, S3), u, S1);
    const float cv = fmaf(fmaf(fmaf(fmaf(fmaf(C10, u, C8), u, C6), u, C4), u, C2), u, 1.0f);
    const int q = __float_as_int(t) & 3;
    float a = (q & 1) ? cv : sv;
    float b = (q & 1) ? sv : cv;
    if (q & 2) a = -a;
    if ((q + 1) & 2) b = -b;
    *s = a;
    *c = b;
}
__device__ __forceinline__ void sincos_pi(double x, double* s, double* c) { sincospi(x, s, c); }
__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_t(double x) { return rsqrt(x); }

// Gauss 3-point rule (EMComponent/Quadrature.cpp:13-18): barycentric
// (2/3, 1/6, 1/6) and permutations, weights 1/3.
template <typename T>
__host__ __device__ inline void gauss3(V3<T> a, V3<T> b, V3<T> c, V3<T>* p)
{
    T g0 = T(2) / T(3), g1 = T(1) / T(6);
    p[0] = a * g0 + b * g1 + c * g1;
    p[1] = a * g1 + b * g0 + c * g1;
    p[2] = a * g1 + b * g1 + c * g0;
}

// Gauss 7-point rule (Quadrature.h:42-72, Quadrature.cpp:44-53); weights
// are twice the textbook values so that they sum to 1.
template <typename T>
__host__ __device__ inline void gauss7(V3<T> a, V3<T> b, V3<T> c, V3<T>* p)
{
    const double g[7][2] = {{0.333333333333333, 0.333333333333333}, {0.797426985353087, 0.101286507323456},
                            {0.101286507323456, 0.797426985353087}, {0.101286507323456, 0.101286507323456},
                            {0.470142064105115, 0.470142064105115}, {0.470142064105115, 0.059715871789770},
                            {0.059715871789770, 0.470142064105115}};
    for (int i = 0; i < 7; ++i) {
        T g0 = (T)g[i][0], g1 = (T)g[i][1];
        T g2 = T(1) - g0 - g1;
        p[i] = a * g0 + b * g1 + c * g2;
    }
}

template <typename T>
__host__ __device__ inline T gauss7_weight(int i)
{
    const double w[7] = {0.112500000000000, 0.062969590272413, 0.062969590272413, 0.062969590272413,
                         0.066197076394253, 0.066197076394253, 0.066197076394253};
    return (T)w[i] * 2;
}

// Heron's formula (VectorR3.h Area)
template <typename T>
__host__ __device__ inline T tri_area(V3<T> a, V3<T> b, V3<T> c)
{
    T la = norm(a - b), lb = norm(b - c), lc = norm(c - a);
    T ls = (la + lb + lc) / T(2);
    return sqrt(ls * (ls - la) * (ls - lb) * (ls - lc));
}

// Triangle::getInfo (EMComponent/Triangle.cpp:47-61)
template <typename T>
__host__ __device__ inline V3<T> tri_normal(V3<T> A, V3<T> B, V3<T> C)
{
    V3<T> ab = B - A, bc = C - B, ca = A - C;
    V3<T> n = (dot(ab, bc) < dot(bc, ca)) ? cross(ab, bc) : cross(bc, ca);
    return divr(n, norm(n));
}

template <typename T>
__host__ __device__ inline V3<T> centroid(V3<T> a, V3<T> b, V3<T> c)
{
    return divr(a + b + c, T(3));
}

// x = hi + lo, hi = x rounded to FP32 (to nearest, ties to even) and lo the
// remainder rounded to FP32, from the bits of the double with integer
// operations only: GB300's FP64 pipe takes ~64 cycles a warp instruction, and
// the FP64 form of this packing ran at 1 TB/s.  |x| below 2^-126 gives
// (0, 0); |x| of 2^128 and above, +-inf.  The remainder is exact to 2^-48 |x|.
__device__ __forceinline__ float2 split_f64(double x)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(u >> 63) << 31;
    const int ex = (int)((u >> 52) & 0x7ff) - 1023;
    if (ex < -126) return make_float2(0.f, 0.f);
    if (ex > 127) return make_float2(__uint_as_float(sign | 0x7f800000u), 0.f);
    const unsigned long long mant = u & 0xFFFFFFFFFFFFFull;  // 52 bits
    unsigned m = (unsigned)(mant >> 29);                      // the 23 bits FP32 keeps
    const int rem = (int)(mant & ((1u << 29) - 1));
    int low = rem;  // the rest, in units of 2^(ex - 52)
    int e2 = ex;
    if (rem > (1 << 28) || (rem == (1 << 28) && (m & 1u))) {
        m += 1u;
        low -= 1 << 29;
        if (m == (1u << 23)) {  // rounded up to the next power of two
            m = 0u;
            e2 += 1;
        }
    }
    if (e2 > 127) return make_float2(__uint_as_float(sign | 0x7f800000u), 0.f);
    const float hi = __uint_as_float(sign | ((unsigned)(e2 + 127) << 23) | m);
    float lo = 0.f;
    if (ex - 52 >= -126) {  // 2^(ex - 52) is a normal FP32: the scaling is exact
        lo = (float)low * __uint_as_float((unsigned)(ex - 52 + 127) << 23);
        if (sign) lo = -lo;
    }
    return make_float2(hi, lo);
}

}  // namespace emfa
