// Group and algebra arithmetic for SU(2) and SU(3) links, shared by every kernel.
//
// All functions are __host__ __device__ so the same per-site code that the
// CUDA kernels run can also be instantiated on the host by the test-only
// build (tcym_hostcheck.cu) and compared with the FP64 oracle without a GPU.
//
// Conventions (those of the reference, SUNc/):
//   SU(2): U = u3*1 + i u_k sigma_k, four reals (SU2/GroupOperations.cpp:4-14)
//   SU(3): 3x3 complex; generators t^a = lambda^a/2 (SU3/AlgebraOperations.cpp:6-7)
//   proj(V)^a = Re tr(i t^a V)  (ReTrIGenU: SU2/GroupOperations.cpp:78-84,
//                                SU3/GroupOperations.cpp:108-118)
//   iexp(c, e) = exp(i c t^a e^a) (MatrixIExp: SU2/AlgebraOperations.cpp:37-55,
//                                  SU3/AlgebraOperations.cpp:141-182)
// The SU(3) exponential here is not the reference's eigen-decomposition: it
// reduces the Taylor series of exp(iQ) with the Cayley-Hamilton identity
// Q^3 = c1 Q + c0 (traceless Hermitian Q, c1 = tr Q^2 / 2, c0 = det Q), so that
// exp(iQ) = f0 + f1 Q + f2 Q^2 with real-coefficient scalar recurrences only,
// after scaling Q by 2^-k until its spectral radius is <= 1/2 and squaring back.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#define TCYM_HD __host__ __device__ __forceinline__
// rarely taken paths of the step, compiled out of line so that they do not sit in
// the instruction stream of the common path (1) or inline like the rest (0)
#ifndef TCYM_COLD_NOINLINE
#define TCYM_COLD_NOINLINE 0
#endif
#if TCYM_COLD_NOINLINE
#define TCYM_COLD __host__ __device__ __noinline__
#else
#define TCYM_COLD TCYM_HD
#endif

namespace tcym {

// ------------------------------------------------------------------ scalars
template <class T> struct Real;
template <> struct Real<float> {
    static TCYM_HD float sqrt_(float x) { return sqrtf(x); }
    // 1/sqrt(x) to about half an ulp: the hardware approximation refined by one
    // Newton step (its own error, up to 2 ulp, need not average to zero).
    static TCYM_HD float rsqrt_(float x) {
#ifdef __CUDA_ARCH__
        const float r = rsqrtf(x);
        return fmaf(r, fmaf(-0.5f * x * r, r, 0.5f), r);
#else
        return 1.0f / sqrtf(x);
#endif
    }
    static TCYM_HD float log_(float x) { return logf(x); }
    static TCYM_HD void sincos_(float x, float *s, float *c) {
#ifdef __CUDA_ARCH__
        sincosf(x, s, c);
#else
        *s = sinf(x); *c = cosf(x);
#endif
    }
    // sin(pi x), cos(pi x)
    static TCYM_HD void sincospi_(float x, float *s, float *c) {
#ifdef __CUDA_ARCH__
        sincospif(x, s, c);
#else
        *s = (float)sin(3.14159265358979323846 * (double)x);
        *c = (float)cos(3.14159265358979323846 * (double)x);
#endif
    }
};
template <> struct Real<double> {
    static TCYM_HD double sqrt_(double x) { return sqrt(x); }
    static TCYM_HD double rsqrt_(double x) { return 1.0 / sqrt(x); }
    static TCYM_HD double log_(double x) { return log(x); }
    static TCYM_HD void sincos_(double x, double *s, double *c) {
#ifdef __CUDA_ARCH__
        sincos(x, s, c);
#else
        *s = sin(x); *c = cos(x);
#endif
    }
    static TCYM_HD void sincospi_(double x, double *s, double *c) {
#ifdef __CUDA_ARCH__
        sincospi(x, s, c);
#else
        *s = sin(3.14159265358979323846264338327950288 * x);
        *c = cos(3.14159265358979323846264338327950288 * x);
#endif
    }
};

// -------------------------------------------------------------- packed pairs
// f2: two FP32 values, one for each site of a site pair.  Every operation is
// one packed instruction on sm_100 and later (FADD2 / FMUL2 / FFMA2), each
// lane rounded exactly as the scalar operation; host code (and device code
// for older targets) does the lanes one at a time.  Packing halves the
// instructions issued for the FP32 arithmetic, which otherwise take every
// issue slot the FP32 pipe can use.
struct f2 {
    float2 v;
    f2() = default;
    TCYM_HD explicit f2(double a) : v(make_float2((float)a, (float)a)) {}
    TCYM_HD f2(float a, float b) : v(make_float2(a, b)) {}
};
TCYM_HD f2 f2_of(float2 x) { f2 r; r.v = x; return r; }
// the lanes exchanged (a pair read across the z seam holds its partner's site first)
TCYM_HD f2 swap_f2(f2 v) { return f2(v.v.y, v.v.x); }
TCYM_HD f2 operator-(f2 a) { return f2(-a.v.x, -a.v.y); }
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
#define TCYM_PACKED_FP32 1
#else
#define TCYM_PACKED_FP32 0
#endif
#if TCYM_PACKED_FP32
TCYM_HD f2 operator+(f2 a, f2 b) { return f2_of(__fadd2_rn(a.v, b.v)); }
TCYM_HD f2 operator-(f2 a, f2 b) { return f2_of(__fadd2_rn(a.v, make_float2(-b.v.x, -b.v.y))); }
TCYM_HD f2 operator*(f2 a, f2 b) { return f2_of(__fmul2_rn(a.v, b.v)); }
#else
TCYM_HD f2 operator+(f2 a, f2 b) { return f2(a.v.x + b.v.x, a.v.y + b.v.y); }
TCYM_HD f2 operator-(f2 a, f2 b) { return f2(a.v.x - b.v.x, a.v.y - b.v.y); }
TCYM_HD f2 operator*(f2 a, f2 b) { return f2(a.v.x * b.v.x, a.v.y * b.v.y); }
#endif
TCYM_HD f2 &operator+=(f2 &a, f2 b) { return a = a + b; }
TCYM_HD f2 &operator-=(f2 &a, f2 b) { return a = a - b; }
TCYM_HD f2 &operator*=(f2 &a, f2 b) { return a = a * b; }
using ::fma;
TCYM_HD f2 fma(f2 a, f2 b, f2 c) {
#if TCYM_PACKED_FP32
    return f2_of(__ffma2_rn(a.v, b.v, c.v));
#else
    return f2(fmaf(a.v.x, b.v.x, c.v.x), fmaf(a.v.y, b.v.y, c.v.y));
#endif
}
TCYM_HD float lane(f2 a, int l) { return l ? a.v.y : a.v.x; }
TCYM_HD f2 lane_swap(f2 a) { return f2(a.v.y, a.v.x); }
template <class T> struct Packed { static constexpr bool value = false; };
template <> struct Packed<f2> { static constexpr bool value = true; };
// a > t in any lane
TCYM_HD bool any_gt(float a, float t) { return a > t; }
TCYM_HD bool any_gt(double a, double t) { return a > t; }
TCYM_HD bool any_gt(f2 a, f2 t) { return a.v.x > t.v.x || a.v.y > t.v.y; }

// f = sin(d/2) / d (any finite value at d = 0, where it multiplies zeros) and
// co = cos(d/2), d = sqrt(d2): the SU(2) exponential's coefficients.
TCYM_HD void half_angle(float d2, float &f, float &co) {
    if (d2 == 0.0f) { f = 0.5f; co = 1.0f; return; }
    const float d = Real<float>::sqrt_(d2);
    float s;
    Real<float>::sincos_(0.5f * d, &s, &co);
    f = s / d;
}
TCYM_HD void half_angle(double d2, double &f, double &co) {
    if (d2 == 0.0) { f = 0.5; co = 1.0; return; }
    const double d = Real<double>::sqrt_(d2);
    double s;
    Real<double>::sincos_(0.5 * d, &s, &co);
    f = s / d;
}
TCYM_HD void half_angle(f2 d2, f2 &f, f2 &co) {  // no packed sine: lane by lane
    half_angle(d2.v.x, f.v.x, co.v.x);
    half_angle(d2.v.y, f.v.y, co.v.y);
}
TCYM_HD float quot(float a, float b) { return a / b; }
TCYM_HD double quot(double a, double b) { return a / b; }
TCYM_HD f2 quot(f2 a, f2 b) { return f2(a.v.x / b.v.x, a.v.y / b.v.y); }

template <class T> struct cx {
    T re, im;
};
template <class T> TCYM_HD cx<T> cmk(T r, T i) { return cx<T>{r, i}; }
template <class T> TCYM_HD cx<T> operator+(cx<T> a, cx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <class T> TCYM_HD cx<T> operator-(cx<T> a, cx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <class T> TCYM_HD cx<T> operator*(cx<T> a, cx<T> b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
template <class T> TCYM_HD cx<T> operator*(T s, cx<T> a) { return {s * a.re, s * a.im}; }
template <class T> TCYM_HD cx<T> conj(cx<T> a) { return {a.re, -a.im}; }
// acc + a*b, acc + a*conj(b), acc + conj(a)*conj(b)
template <class T> TCYM_HD cx<T> cfma(cx<T> a, cx<T> b, cx<T> acc) {
    return {fma(a.re, b.re, fma(-a.im, b.im, acc.re)), fma(a.re, b.im, fma(a.im, b.re, acc.im))};
}
template <class T> TCYM_HD cx<T> cfma_nc(cx<T> a, cx<T> b, cx<T> acc) {  // a * conj(b)
    return {fma(a.re, b.re, fma(a.im, b.im, acc.re)), fma(a.im, b.re, fma(-a.re, b.im, acc.im))};
}
template <class T> TCYM_HD cx<T> cfma_cc(cx<T> a, cx<T> b, cx<T> acc) {  // conj(a) * conj(b)
    return {fma(a.re, b.re, fma(-a.im, b.im, acc.re)), fma(-a.re, b.im, fma(-a.im, b.re, acc.im))};
}
template <class T> TCYM_HD cx<T> cfma_cn(cx<T> a, cx<T> b, cx<T> acc) {  // conj(a) * b
    return {fma(a.re, b.re, fma(a.im, b.im, acc.re)), fma(a.re, b.im, fma(-a.im, b.re, acc.im))};
}

// ------------------------------------------------------------------ SU(2)
template <class T> struct Q4 {
    T q[4];  // q0,q1,q2: coefficients of i sigma_k; q3: identity
};

template <class T> struct SU2 {
    using real = T;
    using Mat = Q4<T>;
    static constexpr int NA = 3;

    static TCYM_HD Mat identity() { return Mat{{T(0), T(0), T(0), T(1)}}; }
    static TCYM_HD Mat zero() { return Mat{{T(0), T(0), T(0), T(0)}}; }
    static TCYM_HD Mat dag(const Mat &u) { return Mat{{-u.q[0], -u.q[1], -u.q[2], u.q[3]}}; }
    static TCYM_HD Mat add(const Mat &a, const Mat &b) {
        return Mat{{a.q[0] + b.q[0], a.q[1] + b.q[1], a.q[2] + b.q[2], a.q[3] + b.q[3]}};
    }
    static TCYM_HD Mat scale(T s, const Mat &a) { return Mat{{s * a.q[0], s * a.q[1], s * a.q[2], s * a.q[3]}}; }
    // quaternion product (u3 + i u.s)(v3 + i v.s) = u3 v3 - u.v + i (u3 v + v3 u - u x v).s
    // with optional conjugation of either factor
    template <bool DA, bool DB> static TCYM_HD Mat mulx(const Mat &a, const Mat &b) {
        const T u0 = DA ? -a.q[0] : a.q[0], u1 = DA ? -a.q[1] : a.q[1], u2 = DA ? -a.q[2] : a.q[2], u3 = a.q[3];
        const T v0 = DB ? -b.q[0] : b.q[0], v1 = DB ? -b.q[1] : b.q[1], v2 = DB ? -b.q[2] : b.q[2], v3 = b.q[3];
        Mat w;
        w.q[0] = fma(u3, v0, fma(v3, u0, -(u1 * v2 - u2 * v1)));
        w.q[1] = fma(u3, v1, fma(v3, u1, -(u2 * v0 - u0 * v2)));
        w.q[2] = fma(u3, v2, fma(v3, u2, -(u0 * v1 - u1 * v0)));
        w.q[3] = fma(u3, v3, -fma(u0, v0, fma(u1, v1, u2 * v2)));
        return w;
    }
    static TCYM_HD Mat mul(const Mat &a, const Mat &b) { return mulx<false, false>(a, b); }
    // product of group elements (same as mulx for SU(2))
    template <bool DA, bool DB> static TCYM_HD Mat mulu(const Mat &a, const Mat &b) { return mulx<DA, DB>(a, b); }
    // exp(i c t^k e^k) u formed as u + (exp - 1) u, the real part of exp - 1 being
    // cos(d/2) - 1 = -sin^2(d/2) / (1 + cos(d/2)), without cancellation.  Near the
    // identity cos(d/2) rounds to 1 (or next to it) in FP32, which would put |exp|
    // above 1 by up to sin^2(d/2) at every update, always the same way, and a long
    // FP32 gradient flow would carry its links off the group; the increment form
    // leaves only the rounding of u's own components, of either sign.
    static TCYM_HD Mat iexp_mul(T c, const T *e, const Mat &u) {
        const T x0 = c * e[0], x1 = c * e[1], x2 = c * e[2];
        const T d2 = fma(x0, x0, fma(x1, x1, x2 * x2));
        T f, co;
        half_angle(d2, f, co);
        const T cm1 = -quot(f * f * d2, T(1) + co);
        const Mat w = mul(Mat{{f * x0, f * x1, f * x2, cm1}}, u);
        return Mat{{u.q[0] + w.q[0], u.q[1] + w.q[1], u.q[2] + w.q[2], u.q[3] + w.q[3]}};
    }
    // proj(u * a) for the force: Re tr(i t^k (u a)) = -(u a)_k
    static TCYM_HD void proj_mul(const Mat &u, const Mat &a, T *out) {
        Mat w = mulx<false, false>(u, a);
        out[0] = -w.q[0]; out[1] = -w.q[1]; out[2] = -w.q[2];
    }
    static TCYM_HD void proj(const Mat &v, T *out) { out[0] = -v.q[0]; out[1] = -v.q[1]; out[2] = -v.q[2]; }
    // proj(a b^dag): only the vector part of the product
    static TCYM_HD void proj_mul_dag(const Mat &a, const Mat &b, T *out) {
        const Mat w = mulx<false, true>(a, b);
        proj(w, out);
    }
    static TCYM_HD T retr_one_minus(const Mat &v) { return T(2) * (T(1) - v.q[3]); }
    // exp(i c t^k e^k) = cos(d/2) + i sin(d/2) (c e / d).sigma, d = |c e|
    static TCYM_HD Mat iexp(T c, const T *e) {
        T x0 = c * e[0], x1 = c * e[1], x2 = c * e[2];
        T d2 = fma(x0, x0, fma(x1, x1, x2 * x2));
        T f, co;
        half_angle(d2, f, co);
        return Mat{{f * x0, f * x1, f * x2, co}};
    }
    // components of V (e^k t^k) V^dagger: the pure quaternion (e,0) rotated
    static TCYM_HD void adjoint(const Mat &v, const T *e, T *out) {
        Mat q{{e[0], e[1], e[2], T(0)}};
        Mat w = mulx<false, true>(mulx<false, false>(v, q), v);
        out[0] = w.q[0]; out[1] = w.q[1]; out[2] = w.q[2];
    }
    static TCYM_HD void inverse_adjoint(const Mat &v, const T *e, T *out) {
        Mat q{{e[0], e[1], e[2], T(0)}};
        Mat w = mulx<false, false>(mulx<true, false>(v, q), v);
        out[0] = w.q[0]; out[1] = w.q[1]; out[2] = w.q[2];
    }
    // ||V V^dagger - 1|| over the four components (SU2/GroupOperations.cpp:172-184)
    static TCYM_HD T unitarity_norm(const Mat &v) {
        Mat c = mulx<false, true>(v, v);
        return Real<T>::sqrt_(c.q[0] * c.q[0] + c.q[1] * c.q[1] + c.q[2] * c.q[2] + (c.q[3] - T(1)) * (c.q[3] - T(1)));
    }
    static TCYM_HD Mat reunitarize(const Mat &v) {
        T n = Real<T>::rsqrt_(v.q[0] * v.q[0] + v.q[1] * v.q[1] + v.q[2] * v.q[2] + v.q[3] * v.q[3]);
        return scale(n, v);
    }
    // A^a with exp(i c A^a t^a) = V, c = +-1, principal branch (MatrixILog,
    // SU2/AlgebraOperations.cpp:56-74): V = cos t + i sin t n.sigma, A = 2 t n / c
    static TCYM_HD void ilog(T c, const Mat &v, T *out) {
        const T d = Real<T>::sqrt_(v.q[0] * v.q[0] + v.q[1] * v.q[1] + v.q[2] * v.q[2]);
        const T m = d == T(0) ? T(0) : T(2) * atan2(d, v.q[3]) / (c * d);
        out[0] = m * v.q[0]; out[1] = m * v.q[1]; out[2] = m * v.q[2];
    }
};

// ------------------------------------------------------------------ SU(3)
template <class T> struct M3 {
    cx<T> m[3][3];  // row-major m[i][j]
};

template <class T> struct SU3 {
    using real = T;
    using Mat = M3<T>;
    static constexpr int NA = 8;
    // FP32 arithmetic, one value or a packed pair (the series lengths depend on it)
    static constexpr bool kSingle = sizeof(T) == 4 || Packed<T>::value;

    static TCYM_HD Mat identity() {
        Mat r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r.m[i][j] = cx<T>{i == j ? T(1) : T(0), T(0)};
        return r;
    }
    static TCYM_HD Mat zero() {
        Mat r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r.m[i][j] = cx<T>{T(0), T(0)};
        return r;
    }
    static TCYM_HD Mat dag(const Mat &a) {
        Mat r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r.m[i][j] = conj(a.m[j][i]);
        return r;
    }
    static TCYM_HD Mat add(const Mat &a, const Mat &b) {
        Mat r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] + b.m[i][j];
        return r;
    }
    static TCYM_HD Mat scale(T s, const Mat &a) {
        Mat r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r.m[i][j] = s * a.m[i][j];
        return r;
    }
    // a^(dagger if DA) * b^(dagger if DB)
    template <bool DA, bool DB> static TCYM_HD Mat mulx(const Mat &a, const Mat &b) {
        Mat r;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                cx<T> acc{T(0), T(0)};
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    cx<T> x = DA ? a.m[k][i] : a.m[i][k];
                    cx<T> y = DB ? b.m[j][k] : b.m[k][j];
                    if (!DA && !DB) acc = cfma(x, y, acc);
                    else if (!DA && DB) acc = cfma_nc(x, y, acc);
                    else if (DA && !DB) acc = cfma_cn(x, y, acc);
                    else acc = cfma_cc(x, y, acc);
                }
                r.m[i][j] = acc;
            }
        return r;
    }
    static TCYM_HD Mat mul(const Mat &a, const Mat &b) { return mulx<false, false>(a, b); }

    // Product of two SU(3) elements: rows 0 and 1 from the factors, row 2 as
    // conj(row0 x row1).  When a caller reads only rows 0 and 1 of the result
    // (or of a factor that is not daggered), the compiler drops the rest.
    template <bool DA, bool DB> static TCYM_HD Mat mulu(const Mat &a, const Mat &b) {
        Mat r;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                cx<T> acc{T(0), T(0)};
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    cx<T> x = DA ? a.m[k][i] : a.m[i][k];
                    cx<T> y = DB ? b.m[j][k] : b.m[k][j];
                    if (!DA && !DB) acc = cfma(x, y, acc);
                    else if (!DA && DB) acc = cfma_nc(x, y, acc);
                    else if (DA && !DB) acc = cfma_cn(x, y, acc);
                    else acc = cfma_cc(x, y, acc);
                }
                r.m[i][j] = acc;
            }
        complete_row2(r);
        return r;
    }

    // Re tr(i t^a V) for all a, V given by its entries; needs Im of the diagonal and
    // both triangles off the diagonal (SU3/GroupOperations.cpp:108-118 expressions).
    static TCYM_HD void proj(const Mat &v, T *p) {
        const T is3 = T(0.57735026918962576450914878050196);
        p[0] = T(-0.5) * (v.m[0][1].im + v.m[1][0].im);
        p[1] = T(-0.5) * (v.m[0][1].re - v.m[1][0].re);
        p[2] = T(-0.5) * (v.m[0][0].im - v.m[1][1].im);
        p[3] = T(-0.5) * (v.m[0][2].im + v.m[2][0].im);
        p[4] = T(-0.5) * (v.m[0][2].re - v.m[2][0].re);
        p[5] = T(-0.5) * (v.m[1][2].im + v.m[2][1].im);
        p[6] = T(-0.5) * (v.m[1][2].re - v.m[2][1].re);
        p[7] = T(-0.5) * is3 * (v.m[0][0].im + v.m[1][1].im - T(2) * v.m[2][2].im);
    }
    // proj(u * a) computing only the entries proj reads: the six off-diagonal
    // entries in full and the imaginary part of the diagonal.
    static TCYM_HD void proj_mul(const Mat &u, const Mat &a, T *p) {
        Mat w;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                if (i == j) {
                    T im = T(0);
#pragma unroll
                    for (int k = 0; k < 3; ++k) im = fma(u.m[i][k].re, a.m[k][j].im, fma(u.m[i][k].im, a.m[k][j].re, im));
                    w.m[i][j] = cx<T>{T(0), im};
                } else {
                    cx<T> acc{T(0), T(0)};
#pragma unroll
                    for (int k = 0; k < 3; ++k) acc = cfma(u.m[i][k], a.m[k][j], acc);
                    w.m[i][j] = acc;
                }
            }
        proj(w, p);
    }
    // proj(a b^dag), W_ij = sum_k a_ik conj(b_jk), computing only the entries proj reads
    static TCYM_HD void proj_mul_dag(const Mat &a, const Mat &b, T *p) {
        Mat w;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                if (i == j) {
                    T im = T(0);  // Im(a conj(b)) = a.im b.re - a.re b.im
#pragma unroll
                    for (int k = 0; k < 3; ++k) im = fma(a.m[i][k].im, b.m[j][k].re, fma(-a.m[i][k].re, b.m[j][k].im, im));
                    w.m[i][j] = cx<T>{T(0), im};
                } else {
                    cx<T> acc{T(0), T(0)};
#pragma unroll
                    for (int k = 0; k < 3; ++k) acc = cfma_nc(a.m[i][k], b.m[j][k], acc);
                    w.m[i][j] = acc;
                }
            }
        proj(w, p);
    }
    static TCYM_HD T retr_one_minus(const Mat &v) { return T(3) - (v.m[0][0].re + v.m[1][1].re + v.m[2][2].re); }

    // Hermitian H = e^a t^a
    static TCYM_HD Mat algebra_matrix(T c, const T *e) {
        const T is3 = T(0.57735026918962576450914878050196);
        const T h = T(0.5) * c;
        Mat q;
        q.m[0][0] = cx<T>{h * (e[2] + e[7] * is3), T(0)};
        q.m[1][1] = cx<T>{h * (-e[2] + e[7] * is3), T(0)};
        q.m[2][2] = cx<T>{-c * e[7] * is3, T(0)};
        q.m[1][0] = cx<T>{h * e[0], h * e[1]};
        q.m[0][1] = cx<T>{h * e[0], -h * e[1]};
        q.m[2][0] = cx<T>{h * e[3], h * e[4]};
        q.m[0][2] = cx<T>{h * e[3], -h * e[4]};
        q.m[2][1] = cx<T>{h * e[5], h * e[6]};
        q.m[1][2] = cx<T>{h * e[5], -h * e[6]};
        return q;
    }
    // x^a = 2 tr(t^a H) for Hermitian H
    static TCYM_HD void algebra_components(const Mat &hm, T *x) {
        const T is3 = T(0.57735026918962576450914878050196);
        x[0] = hm.m[1][0].re + hm.m[0][1].re;
        x[1] = hm.m[1][0].im - hm.m[0][1].im;
        x[2] = hm.m[0][0].re - hm.m[1][1].re;
        x[3] = hm.m[2][0].re + hm.m[0][2].re;
        x[4] = hm.m[2][0].im - hm.m[0][2].im;
        x[5] = hm.m[2][1].re + hm.m[1][2].re;
        x[6] = hm.m[2][1].im - hm.m[1][2].im;
        x[7] = is3 * (hm.m[0][0].re + hm.m[1][1].re - T(2) * hm.m[2][2].re);
    }

    // exp(i Q) for traceless Hermitian Q, see the file comment.
    static TCYM_HD Mat iexp_hermitian(Mat q) {
        // Q^2 (Hermitian): compute the upper triangle and mirror
        Mat q2;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                cx<T> acc{T(0), T(0)};
#pragma unroll
                for (int k = 0; k < 3; ++k) acc = cfma(q.m[i][k], q.m[k][j], acc);
                q2.m[i][j] = acc;
                if (j != i) q2.m[j][i] = conj(acc);
            }
        T c1 = T(0.5) * (q2.m[0][0].re + q2.m[1][1].re + q2.m[2][2].re);
        // spectral radius bound r^2 <= 4 c1 / 3; halve Q until r <= 1/2
        int k = 0;
        T r2 = c1 * T(4.0 / 3.0);
        while (r2 > T(0.25) && k < 40) { r2 *= T(0.25); ++k; }
        T s = T(1);
        if (k > 0) {
            s = T(1) / T(1ull << (k < 62 ? k : 62));
            q = scale(s, q);
            q2 = scale(s * s, q2);
            c1 *= s * s;
        }
        // c0 = det Q (real for Hermitian Q)
        cx<T> d = q.m[0][0] * (q.m[1][1] * q.m[2][2] - q.m[1][2] * q.m[2][1]) -
                  q.m[0][1] * (q.m[1][0] * q.m[2][2] - q.m[1][2] * q.m[2][0]) +
                  q.m[0][2] * (q.m[1][0] * q.m[2][1] - q.m[1][1] * q.m[2][0]);
        T c0 = d.re;
        // sum_n (i^n / n!) Q^n with Q^n = a_n + b_n Q + d_n Q^2
        const int N = kSingle ? 9 : 16;
        T a = T(1), b = T(0), dd = T(0);
        T f0r = T(1), f0i = T(0), f1r = T(0), f1i = T(0), f2r = T(0), f2i = T(0);
        T fact = T(1);
#pragma unroll
        for (int n = 1; n <= N; ++n) {
            T na = dd * c0, nb = fma(dd, c1, a), nd = b;
            a = na; b = nb; dd = nd;
            fact /= T(n);
            T wa = fact * a, wb = fact * b, wd = fact * dd;
            switch (n & 3) {  // i^n = 1, i, -1, -i
                case 0: f0r += wa; f1r += wb; f2r += wd; break;
                case 1: f0i += wa; f1i += wb; f2i += wd; break;
                case 2: f0r -= wa; f1r -= wb; f2r -= wd; break;
                default: f0i -= wa; f1i -= wb; f2i -= wd; break;
            }
        }
        Mat r;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                cx<T> x = q.m[i][j], y = q2.m[i][j];
                T re = fma(f1r, x.re, fma(-f1i, x.im, fma(f2r, y.re, -f2i * y.im)));
                T im = fma(f1r, x.im, fma(f1i, x.re, fma(f2r, y.im, f2i * y.re)));
                if (i == j) { re += f0r; im += f0i; }
                r.m[i][j] = cx<T>{re, im};
            }
        for (int it = 0; it < k; ++it) r = mul(r, r);
        return r;
    }
    static TCYM_HD Mat iexp(T c, const T *e) { return iexp_hermitian(algebra_matrix(c, e)); }

    // exp(i c t^a e^a) u for a link update.  In the common case (spectral radius
    // of Q <= 1/2, no scaling) only rows 0 and 1 of exp(iQ) - 1 and of
    // u + (exp(iQ) - 1) u are formed; row 2 of the product is conj(row0 x row1).
    // The increment form keeps f0 - 1 apart from the 1: near the identity f0
    // itself rounds next to 1 in FP32, which would move every updated link's
    // norm the same way and carry a long FP32 gradient flow off the group.
    // Otherwise the scaled-and-squared exponential is used.
    static TCYM_HD Mat iexp_mul(T c, const T *e, const Mat &u) {
        const Mat q = algebra_matrix(c, e);
        // c1 = tr(Q^2)/2 = sum_ij |Q_ij|^2 / 2
        const T d0 = q.m[0][0].re, d1 = q.m[1][1].re, d2 = q.m[2][2].re;
        const T o01 = q.m[0][1].re * q.m[0][1].re + q.m[0][1].im * q.m[0][1].im;
        const T o02 = q.m[0][2].re * q.m[0][2].re + q.m[0][2].im * q.m[0][2].im;
        const T o12 = q.m[1][2].re * q.m[1][2].re + q.m[1][2].im * q.m[1][2].im;
        const T c1 = T(0.5) * (d0 * d0 + d1 * d1 + d2 * d2) + (o01 + o02 + o12);
        if (any_gt(c1 * T(4.0 / 3.0), T(0.25))) {
            if constexpr (Packed<T>::value) return iexp_mul_lanes(c, e, u);
            else return mulu<false, false>(iexp_hermitian(q), u);
        }
        // rows 0 and 1 of Q^2 (Hermitian Q)
        cx<T> q2[2][3];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                cx<T> acc{T(0), T(0)};
#pragma unroll
                for (int k = 0; k < 3; ++k) acc = cfma(q.m[i][k], q.m[k][j], acc);
                q2[i][j] = acc;
            }
        q2[1][0] = conj(q2[0][1]);
        // c0 = det Q (real for Hermitian Q)
        const T c0 = d0 * (d1 * d2 - o12) - d1 * o02 - d2 * o01 +
                     T(2) * (q.m[0][1].re * (q.m[1][2].re * q.m[2][0].re - q.m[1][2].im * q.m[2][0].im) -
                             q.m[0][1].im * (q.m[1][2].re * q.m[2][0].im + q.m[1][2].im * q.m[2][0].re));
        T f0r, f0i, f1r, f1i, f2r, f2i;
        if constexpr (kSingle) {
            // terms of the series by the spectral radius r (r^2 <= 4 c1 / 3): the first
            // omitted term r^(N+1)/(N+1)! stays below half an FP32 ulp, 3e-8, with 5
            // terms for r^2 <= 0.02 (the common case: |dt E| is small) and 8 up to r = 1/2
            if (any_gt(c1 * T(4.0 / 3.0), T(0.02))) series_coeffs<8, true>(c0, c1, f0r, f0i, f1r, f1i, f2r, f2i);
            else series_coeffs<5, true>(c0, c1, f0r, f0i, f1r, f1i, f2r, f2i);
        } else {
            series_coeffs<16, true>(c0, c1, f0r, f0i, f1r, f1i, f2r, f2i);
        }
        Mat w;  // rows 0 and 1 of exp(iQ) - 1
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const cx<T> x = q.m[i][j], y = q2[i][j];
                T re = fma(f1r, x.re, fma(-f1i, x.im, fma(f2r, y.re, -f2i * y.im)));
                T im = fma(f1r, x.im, fma(f1i, x.re, fma(f2r, y.im, f2i * y.re)));
                if (i == j) { re += f0r; im += f0i; }
                w.m[i][j] = cx<T>{re, im};
            }
        return mulu_inc(w, u);  // reads rows 0 and 1 of w only
    }
    // rows 0 and 1 of u + w u (each accumulator starts at u's entry), row 2 rebuilt
    static TCYM_HD Mat mulu_inc(const Mat &w, const Mat &u) {
        Mat r;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                cx<T> acc = u.m[i][j];
#pragma unroll
                for (int k = 0; k < 3; ++k) acc = cfma(w.m[i][k], u.m[k][j], acc);
                r.m[i][j] = acc;
            }
        complete_row2(r);
        return r;
    }
    // packed pairs whose exponent needs scaling: each lane through the scalar path
    template <class P = T> static TCYM_COLD Mat iexp_mul_lanes(P c, const P *e, const Mat &u) {
        Mat r;
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            float el[NA];
            typename SU3<float>::Mat ul;
#pragma unroll
            for (int a = 0; a < NA; ++a) el[a] = lane(e[a], l);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) ul.m[i][j] = cx<float>{lane(u.m[i][j].re, l), lane(u.m[i][j].im, l)};
            const typename SU3<float>::Mat w = SU3<float>::iexp_mul(lane(c, l), el, ul);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    if (l == 0) { r.m[i][j].re.v.x = w.m[i][j].re; r.m[i][j].im.v.x = w.m[i][j].im; }
                    else { r.m[i][j].re.v.y = w.m[i][j].re; r.m[i][j].im.v.y = w.m[i][j].im; }
                }
        }
        return r;
    }

    // f_k of exp(iQ) = f0 + f1 Q + f2 Q^2 for spectral radius <= 1/2: the Taylor
    // series reduced with Q^3 = c1 Q + c0 (Q^n = a_n + b_n Q + d_n Q^2).
    // M1: f0r returns f0 - 1 (the series without its leading 1), for the increment form
    template <int N, bool M1 = false>
    static TCYM_HD void series_coeffs(T c0, T c1, T &f0r, T &f0i, T &f1r, T &f1i, T &f2r, T &f2i) {
        static_assert(N >= 1 && N <= 16, "at most 16 terms");
        constexpr double inv_fact[17] = {1.0, 1.0, 0.5, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720, 1.0 / 5040,
                                         1.0 / 40320, 1.0 / 362880, 1.0 / 3628800, 1.0 / 39916800,
                                         1.0 / 479001600, 1.0 / 6227020800.0, 1.0 / 87178291200.0,
                                         1.0 / 1307674368000.0, 1.0 / 20922789888000.0};
        T a = T(1), b = T(0), d = T(0);
        f0r = M1 ? T(0) : T(1); f0i = T(0); f1r = T(0); f1i = T(0); f2r = T(0); f2i = T(0);
#pragma unroll
        for (int n = 1; n <= N; ++n) {
            const T na = d * c0, nb = fma(d, c1, a), nd = b;
            a = na; b = nb; d = nd;
            const T fct = T(inv_fact[n]);
            const T wa = fct * a, wb = fct * b, wd = fct * d;
            switch (n & 3) {  // i^n = 1, i, -1, -i
                case 0: f0r += wa; f1r += wb; f2r += wd; break;
                case 1: f0i += wa; f1i += wb; f2i += wd; break;
                case 2: f0r -= wa; f1r -= wb; f2r -= wd; break;
                default: f0i -= wa; f1i -= wb; f2i -= wd; break;
            }
        }
    }

    // V (e^a t^a) V^dagger and V^dagger (e^a t^a) V in components
    static TCYM_HD void adjoint(const Mat &v, const T *e, T *out) {
        Mat h = algebra_matrix(T(1), e);
        Mat w = mulx<false, true>(mulx<false, false>(v, h), v);
        algebra_components(w, out);
    }
    static TCYM_HD void inverse_adjoint(const Mat &v, const T *e, T *out) {
        Mat h = algebra_matrix(T(1), e);
        Mat w = mulx<false, false>(mulx<true, false>(v, h), v);
        algebra_components(w, out);
    }
    // ||V V^dagger - 1||_F (SU3/GroupOperations.cpp:351-363)
    static TCYM_HD T unitarity_norm(const Mat &v) {
        Mat c = mulx<false, true>(v, v);
        T n = T(0);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                T re = c.m[i][j].re - (i == j ? T(1) : T(0)), im = c.m[i][j].im;
                n = fma(re, re, fma(im, im, n));
            }
        return Real<T>::sqrt_(n);
    }
    // third row of an SU(3) matrix from the first two: r2 = conj(r0 x r1)
    static TCYM_HD void complete_row2(Mat &u) {
        const cx<T> *a = u.m[0], *b = u.m[1];
        u.m[2][0] = conj_cross(a[1], b[2], a[2], b[1]);
        u.m[2][1] = conj_cross(a[2], b[0], a[0], b[2]);
        u.m[2][2] = conj_cross(a[0], b[1], a[1], b[0]);
    }
    // conj(x y - z w) as fused multiply-adds
    static TCYM_HD cx<T> conj_cross(cx<T> x, cx<T> y, cx<T> z, cx<T> w) {
        return {fma(x.re, y.re, fma(-x.im, y.im, fma(-z.re, w.re, z.im * w.im))),
                fma(z.re, w.im, fma(z.im, w.re, fma(-x.re, y.im, -(x.im * y.re))))};
    }
    // Hermitian A = W diag(w) W^dagger by cyclic complex Jacobi rotations (the
    // rotation from tan t = sgn(tau) / (|tau| + sqrt(1 + tau^2)), no trigonometry),
    // at most 30 sweeps.
    static TCYM_HD void hermitian_eigen(Mat a, T *w, Mat &W) {
        W = identity();
        for (int sweep = 0; sweep < 30; ++sweep) {
            const T off = abs2(a.m[0][1]) + abs2(a.m[0][2]) + abs2(a.m[1][2]);
            const T diag = a.m[0][0].re * a.m[0][0].re + a.m[1][1].re * a.m[1][1].re + a.m[2][2].re * a.m[2][2].re;
            if (!(off > T(1e-32) * (diag + off))) break;
            for (int p = 0; p < 2; ++p)
                for (int q = p + 1; q < 3; ++q) {
                    const cx<T> apq = a.m[p][q];
                    const T r = Real<T>::sqrt_(abs2(apq));
                    if (r == T(0)) continue;
                    const cx<T> ph{apq.re / r, apq.im / r};  // a_pq = r e^{i phi}
                    const T tau = (a.m[q][q].re - a.m[p][p].re) / (T(2) * r);
                    const T t = (tau >= T(0) ? T(1) : T(-1)) / (fabs(tau) + Real<T>::sqrt_(T(1) + tau * tau));
                    const T cs = T(1) / Real<T>::sqrt_(T(1) + t * t), sn = t * cs;
                    // columns p, q of A and W: col_p' = c col_p - s conj(ph) col_q, col_q' = s ph col_p + c col_q
                    const cx<T> gqp{-sn * ph.re, sn * ph.im}, gpq{sn * ph.re, sn * ph.im};
                    for (int k = 0; k < 3; ++k) {
                        const cx<T> akp = a.m[k][p], akq = a.m[k][q], wkp = W.m[k][p], wkq = W.m[k][q];
                        a.m[k][p] = cx<T>{cs * akp.re, cs * akp.im} + akq * gqp;
                        a.m[k][q] = akp * gpq + cx<T>{cs * akq.re, cs * akq.im};
                        W.m[k][p] = cx<T>{cs * wkp.re, cs * wkp.im} + wkq * gqp;
                        W.m[k][q] = wkp * gpq + cx<T>{cs * wkq.re, cs * wkq.im};
                    }
                    for (int k = 0; k < 3; ++k) {  // rows: A <- G^dagger A
                        const cx<T> apk = a.m[p][k], aqk = a.m[q][k];
                        a.m[p][k] = cx<T>{cs * apk.re, cs * apk.im} + conj(gqp) * aqk;
                        a.m[q][k] = conj(gpq) * apk + cx<T>{cs * aqk.re, cs * aqk.im};
                    }
                }
        }
        w[0] = a.m[0][0].re; w[1] = a.m[1][1].re; w[2] = a.m[2][2].re;
    }
    static TCYM_HD T abs2(cx<T> z) { return z.re * z.re + z.im * z.im; }
    // A^a with exp(i c A^a t^a) = V, c = +-1, principal branch (MatrixILog,
    // SU3/AlgebraOperations.cpp:186-233, there through LAPACK zgeev): the normal V
    // shares its eigenvectors with the commuting Hermitian (V + V^dag)/2 and
    // (V - V^dag)/(2i), found as those of C = (V + V^dag)/2 + g (V - V^dag)/(2i),
    // g = 0.618... (eigenvalues cos t + g sin t keep t and -t apart);
    // H = W diag(arg(w_k^dag V w_k)) W^dag and A^a = 2 tr(t^a H) / c.
    static TCYM_HD void ilog(T c, const Mat &v, T *out) {
        const T g = T(0.6180339887498949);
        Mat h;
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) {
                const cx<T> a = v.m[i][k], b = conj(v.m[k][i]);
                // (a + b)/2 + g (a - b)/(2i) = (a + b)/2 - i g (a - b)/2
                h.m[i][k] = cx<T>{T(0.5) * (a.re + b.re) + T(0.5) * g * (a.im - b.im),
                                  T(0.5) * (a.im + b.im) - T(0.5) * g * (a.re - b.re)};
            }
        T w[3];
        Mat W;
        hermitian_eigen(h, w, W);
        T th[3];
        for (int j = 0; j < 3; ++j) {
            cx<T> z{T(0), T(0)};  // w_j^dag V w_j
            for (int i = 0; i < 3; ++i) {
                cx<T> vw{T(0), T(0)};
                for (int k = 0; k < 3; ++k) vw = cfma(v.m[i][k], W.m[k][j], vw);
                z = cfma_cn(W.m[i][j], vw, z);
            }
            th[j] = atan2(z.im, z.re);
        }
        Mat hm;  // H = W diag(th) W^dagger (Hermitian)
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) {
                cx<T> s{T(0), T(0)};
                for (int j = 0; j < 3; ++j) s = cfma_nc(cx<T>{th[j] * W.m[i][j].re, th[j] * W.m[i][j].im}, W.m[k][j], s);
                hm.m[i][k] = s;
            }
        algebra_components(hm, out);
        for (int a = 0; a < NA; ++a) out[a] = out[a] / c;
    }
    // Gram-Schmidt of rows 0 and 1, row 2 rebuilt: the nearest SU(3) matrix
    // for a link that has drifted by rounding (not a max-trace projection).
    static TCYM_HD Mat reunitarize(Mat u) {
        T n0 = T(0);
        for (int j = 0; j < 3; ++j) n0 = fma(u.m[0][j].re, u.m[0][j].re, fma(u.m[0][j].im, u.m[0][j].im, n0));
        T i0 = Real<T>::rsqrt_(n0);
        for (int j = 0; j < 3; ++j) u.m[0][j] = i0 * u.m[0][j];
        cx<T> dot{T(0), T(0)};  // <r0, r1> = sum conj(r0) r1
        for (int j = 0; j < 3; ++j) dot = cfma_cn(u.m[0][j], u.m[1][j], dot);
        for (int j = 0; j < 3; ++j) u.m[1][j] = u.m[1][j] - dot * u.m[0][j];
        T n1 = T(0);
        for (int j = 0; j < 3; ++j) n1 = fma(u.m[1][j].re, u.m[1][j].re, fma(u.m[1][j].im, u.m[1][j].im, n1));
        T i1 = Real<T>::rsqrt_(n1);
        for (int j = 0; j < 3; ++j) u.m[1][j] = i1 * u.m[1][j];
        complete_row2(u);
        return u;
    }
};

}  // namespace tcym
