// pic_math.cuh -- per-particle arithmetic of the OSIRIS push and charge-conserving deposit,
// for float (mixed-precision path) and double (plain FP64 path).
//
// Every expression keeps the rounding structure of the reference SIMD kernels: a fused
// multiply-add appears exactly where the reference uses one, every other product and sum is
// rounded on its own (the library is compiled with -fmad=false so nvcc does not contract).
// Division and square root are the IEEE-rounded operations (no fast-math), so a particle's
// new position, cell and momentum are bit-identical to the reference CPU kernels.
//
//   B-spline weights         source/simd/splines-avx2.h
//   longitudinal weights     source/simd/os-spec-current-avx2d.c:17-110
//   Boris rotation + energy  source/simd/os-spec-push-avx2d.c:98-154
//   1/gamma                  source/simd/os-spec-push-avx2d.c:163-168
//   cell trim                source/simd/os-spec-push-avx2d.c:53-64
//   trajectory split         source/simd/split-vec.h:105-265 (2D), :266-718 (3D)
#pragma once

#include <cstdint>

#include "../../include/osiris_gb300.h"

namespace osg {

__device__ __forceinline__ float fmaR(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmaR(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float sqrtR(float a) { return sqrtf(a); }
__device__ __forceinline__ double sqrtR(double a) { return sqrt(a); }

// grid offset of the interpolation stencil (1 + ORD/2, 3 for quartic)
template <int ORD> struct Stencil {
    static constexpr int NP = ORD + 1;
    static constexpr int OFS = (ORD == 1) ? 1 : (ORD == 2) ? 2 : (ORD == 3) ? 2 : 3;
};

// B-spline weights at a cell-centred offset x in [-0.5, 0.5)
template <int ORD, typename T>
__device__ __forceinline__ void spline(T x, T *w)
{
    const T c1_2 = T(0.5);
    if constexpr (ORD == 1) {
        w[0] = c1_2 - x;
        w[1] = c1_2 + x;
    } else if constexpr (ORD == 2) {
        T a = c1_2 - x, b = c1_2 + x;
        w[0] = (a * a) * c1_2;
        w[1] = fmaR(a, b, c1_2);
        w[2] = (b * b) * c1_2;
    } else if constexpr (ORD == 3) {
        T a = c1_2 - x, b = c1_2 + x;
        T a2 = a * a, b2 = b * b;
        T a3 = a * a2, b3 = b * b2;
        w[0] = T(1.0 / 6.0) * a3;
        w[1] = fmaR(c1_2, b3, T(2.0 / 3.0) - b2);
        w[2] = fmaR(c1_2, a3, T(2.0 / 3.0) - a2);
        w[3] = T(1.0 / 6.0) * b3;
    } else {
        T a = c1_2 - x, b = c1_2 + x;
        T ab = a * b, a2 = a * a, b2 = b * b;
        w[0] = T(1.0 / 24.0) * (a2 * a2);
        w[1] = T(1.0 / 6.0) * fmaR(a, fmaR(a, T(1.5) + ab, T(1.0)), T(0.25));
        w[2] = fmaR(ab, fmaR(T(0.25), ab, c1_2), T(11.0 / 24.0));
        w[3] = T(1.0 / 6.0) * fmaR(b, fmaR(b, T(1.5) + ab, T(1.0)), T(0.25));
        w[4] = T(1.0 / 24.0) * (b2 * b2);
    }
}

// weights at the half-shifted point (h = 1 when x < 0), for staggered field components
template <int ORD, typename T>
__device__ __forceinline__ void spline_h(T x, T h, T *w)
{
    T a = (T(1.0) - h) - x, b = h + x;
    if constexpr (ORD == 1) {
        w[0] = a;
        w[1] = b;
    } else if constexpr (ORD == 2) {
        w[0] = (a * a) * T(0.5);
        w[1] = fmaR(a, b, T(0.5));
        w[2] = (b * b) * T(0.5);
    } else if constexpr (ORD == 3) {
        T a2 = a * a, b2 = b * b;
        T a3 = a * a2, b3 = b * b2;
        w[0] = T(1.0 / 6.0) * a3;
        w[1] = fmaR(T(0.5), b3, T(2.0 / 3.0) - b2);
        w[2] = fmaR(T(0.5), a3, T(2.0 / 3.0) - a2);
        w[3] = T(1.0 / 6.0) * b3;
    } else {
        T ab = a * b, a2 = a * a, b2 = b * b;
        w[0] = T(1.0 / 24.0) * (a2 * a2);
        w[1] = T(1.0 / 6.0) * fmaR(a, fmaR(a, T(1.5) + ab, T(1.0)), T(0.25));
        w[2] = fmaR(ab, fmaR(T(0.25), ab, T(0.5)), T(11.0 / 24.0));
        w[3] = T(1.0 / 6.0) * fmaR(b, fmaR(b, T(1.5) + ab, T(1.0)), T(0.25));
        w[4] = T(1.0 / 24.0) * (b2 * b2);
    }
}

// charge-conserving weights along the motion (ORD values)
template <int ORD, typename T>
__device__ __forceinline__ void long_weights(T qn, T x0, T x1, T *w)
{
    T d = x1 - x0;
    if constexpr (ORD == 1) {
        w[0] = qn * d;
    } else if constexpr (ORD == 2) {
        T s = T(0.5) - x0, p = T(0.5) + x0;
        T n = qn * d;
        w[0] = n * fmaR(-T(0.5), d, s);
        w[1] = n * fmaR(T(0.5), d, p);
    } else if constexpr (ORD == 3) {
        T s = T(0.5) - x0, p = T(0.5) + x0;
        T d3 = T(1.0 / 3.0) * d;
        T a0 = T(0.5) * fmaR(s, s, -(d * (s - d3)));
        T a1 = fmaR(-d, x0 + d3, fmaR(-x0, x0, T(0.75)));
        T a2 = T(0.5) * fmaR(p, p, d * (p + d3));
        T n = qn * d;
        w[0] = n * a0;
        w[1] = n * a1;
        w[2] = n * a2;
    } else {
        T s = T(0.5) - x0, p = T(0.5) + x0;
        T t = x0 - T(1.0 / 6.0), u = x0 + T(1.0 / 6.0);
        T s2 = s * s, s3 = s2 * s, p2 = p * p, p3 = p2 * p;
        T d2 = d * T(0.5), d4 = d * T(0.25);
        T a0 = T(1.0 / 6.0) * fmaR(d, fmaR(d, s - d4, -(T(1.5) * s2)), s3);
        T a1 = fmaR(d, fmaR(d2, t + d4, fmaR(T(0.75), t * t, -T(1.0 / 3.0))),
                    fmaR(T(0.5), p3, T(2.0 / 3.0) - p2));
        T a2 = fmaR(-d, fmaR(d2, u + d4, fmaR(T(0.75), u * u, -T(1.0 / 3.0))),
                    fmaR(T(0.5), s3, T(2.0 / 3.0) - s2));
        T a3 = T(1.0 / 6.0) * fmaR(d, fmaR(d, p + d4, T(1.5) * p2), p3);
        T n = qn * d;
        w[0] = n * a0;
        w[1] = n * a1;
        w[2] = n * a2;
        w[3] = n * a3;
    }
}

// Boris momentum update; tem = dt / (2 rqm); returns the time-centred kinetic energy factor
// u^2 / (gamma + 1) of the half-kicked momentum.
template <typename T>
__device__ __forceinline__ T boris(T tem, T e1, T e2, T e3, T b1, T b2, T b3, T &u1, T &u2,
                                   T &u3)
{
    e1 = e1 * tem;
    e2 = e2 * tem;
    e3 = e3 * tem;
    T ut1 = u1 + e1, ut2 = u2 + e2, ut3 = u3 + e3;
    T utsq = fmaR(ut3, ut3, fmaR(ut2, ut2, ut1 * ut1));
    T gam = sqrtR(utsq + T(1.0));
    T ene = utsq / (gam + T(1.0));
    T tg = tem / gam;
    b1 = b1 * tg;
    b2 = b2 * tg;
    b3 = b3 * tg;
    T v1 = fmaR(b3, ut2, ut1), v2 = fmaR(b1, ut3, ut2), v3 = fmaR(b2, ut1, ut3);
    v1 = fmaR(-b2, ut3, v1);
    v2 = fmaR(-b3, ut1, v2);
    v3 = fmaR(-b1, ut2, v3);
    T ot = fmaR(b1, b1, T(1.0));
    ot = fmaR(b2, b2, ot);
    ot = fmaR(b3, b3, ot);
    ot = T(2.0) / ot;
    b1 = b1 * ot;
    b2 = b2 * ot;
    b3 = b3 * ot;
    ut1 = fmaR(b3, v2, ut1);
    ut2 = fmaR(b1, v3, ut2);
    ut3 = fmaR(b2, v1, ut3);
    ut1 = fmaR(-b2, v3, ut1);
    ut2 = fmaR(-b3, v1, ut2);
    ut3 = fmaR(-b1, v2, ut3);
    u1 = ut1 + e1;
    u2 = ut2 + e2;
    u3 = ut3 + e3;
    return ene;
}

template <typename T>
__device__ __forceinline__ T rgamma(T u1, T u2, T u3)
{
    return T(1.0) / sqrtR(fmaR(u3, u3, fmaR(u2, u2, fmaR(u1, u1, T(1.0)))));
}

// cell crossing of a pushed offset: +1 when x >= 0.5, -1 when x < -0.5
template <typename T>
__device__ __forceinline__ int trim(T x)
{
    return (x >= T(0.5) ? 1 : 0) - (x < T(-0.5) ? 1 : 0);
}

// ---------------------------------------------------------------------------------------
// Virtual particles: trajectory segments that stay inside one cell, positions relative to
// that cell (x0 start, x1 end), cell index i.  In 2D the out-of-plane velocity vz is split
// in proportion to the segment fraction (the 2D deposit needs it for j3).
// ---------------------------------------------------------------------------------------

template <typename T> struct Seg2 {
    T x0, x1, y0, y1, vz;
    int i, j;
};

template <typename T> struct Seg3 {
    T x0, x1, y0, y1, z0, z1;
    int i, j, k;
};

// Split a 2D move into <= 3 in-cell segments (split-vec.h:105-265). s[0] is the first segment;
// returns the number of segments.
template <typename T>
__device__ __forceinline__ int split2(Seg2<T> *s, int dix, int diy)
{
    Seg2<T> &v = s[0];
    if (dix == 0 && diy == 0) return 1;
    if (diy == 0) {
        T xint = T(0.5) * T(dix);
        T delta = (xint - v.x0) / (v.x1 - v.x0);
        T yint = v.y0 + (v.y1 - v.y0) * delta;
        Seg2<T> &w = s[1];
        w.x0 = -xint; w.x1 = v.x1 - T(dix);
        w.y0 = yint;  w.y1 = v.y1;
        w.i = v.i + dix; w.j = v.j;
        w.vz = v.vz * (T(1) - delta);
        v.x1 = xint; v.y1 = yint; v.vz = v.vz * delta;
        return 2;
    }
    if (dix == 0) {
        T yint = T(0.5) * T(diy);
        T delta = (yint - v.y0) / (v.y1 - v.y0);
        T xint = v.x0 + (v.x1 - v.x0) * delta;
        Seg2<T> &w = s[1];
        w.x0 = xint;  w.x1 = v.x1;
        w.y0 = -yint; w.y1 = v.y1 - T(diy);
        w.i = v.i; w.j = v.j + diy;
        w.vz = v.vz * (T(1) - delta);
        v.x1 = xint; v.y1 = yint; v.vz = v.vz * delta;
        return 2;
    }
    T xint = T(0.5) * T(dix);
    T delta = (xint - v.x0) / (v.x1 - v.x0);
    T yint = v.y0 + (v.y1 - v.y0) * delta;
    if (yint >= T(-0.5) && yint < T(0.5)) {
        // x face first, then y face inside the x-shifted cell
        T vzint = v.vz * delta;
        T vzint2 = v.vz * (T(1) - delta);
        T yint2 = T(0.5) * T(diy);
        delta = (yint2 - yint) / (v.y1 - yint);
        T xint2 = -xint + (v.x1 - xint) * delta;
        Seg2<T> &a = s[1];
        a.x0 = -xint; a.x1 = xint2; a.y0 = yint; a.y1 = yint2;
        a.i = v.i + dix; a.j = v.j; a.vz = vzint2 * delta;
        Seg2<T> &b = s[2];
        b.x0 = xint2; b.x1 = v.x1 - T(dix); b.y0 = -yint2; b.y1 = v.y1 - T(diy);
        b.i = v.i + dix; b.j = v.j + diy; b.vz = vzint2 * (T(1) - delta);
        v.x1 = xint; v.y1 = yint; v.vz = vzint;
    } else {
        // y face first
        T vzint = v.vz * delta;
        T yint2 = T(0.5) * T(diy);
        delta = (yint2 - v.y0) / (yint - v.y0);
        T xint2 = v.x0 + (xint - v.x0) * delta;
        Seg2<T> &a = s[1];
        a.x0 = xint2; a.x1 = xint; a.y0 = -yint2; a.y1 = yint - T(diy);
        a.i = v.i; a.j = v.j + diy; a.vz = vzint * (T(1) - delta);
        Seg2<T> &b = s[2];
        b.x0 = -xint; b.x1 = v.x1 - T(dix); b.y0 = yint - T(diy); b.y1 = v.y1 - T(diy);
        b.i = v.i + dix; b.j = v.j + diy; b.vz = v.vz - vzint;
        v.x1 = xint2; v.y1 = yint2; v.vz = vzint * delta;
    }
    return 3;
}

// coordinate accessors for the axis-generic 3D split
template <typename T> __device__ __forceinline__ T &c0(Seg3<T> &s, int a)
{
    return a == 0 ? s.x0 : (a == 1 ? s.y0 : s.z0);
}
template <typename T> __device__ __forceinline__ T &c1(Seg3<T> &s, int a)
{
    return a == 0 ? s.x1 : (a == 1 ? s.y1 : s.z1);
}
template <typename T> __device__ __forceinline__ int &ci(Seg3<T> &s, int a)
{
    return a == 0 ? s.i : (a == 1 ? s.j : s.k);
}

// one face crossing along axis a (split-vec.h cases 1, 2, 4)
template <typename T>
__device__ __forceinline__ void cut_one(Seg3<T> &v, Seg3<T> &w, int a, int d)
{
    T cint = T(0.5) * T(d);
    T delta = (cint - c0(v, a)) / (c1(v, a) - c0(v, a));
    T in[3];
#pragma unroll
    for (int b = 0; b < 3; b++) in[b] = (b == a) ? cint : c0(v, b) + (c1(v, b) - c0(v, b)) * delta;
    w = v;
    w.x0 = in[0]; w.y0 = in[1]; w.z0 = in[2];
    c0(w, a) = -cint;
    c1(w, a) = c1(v, a) - T(d);
    ci(w, a) += d;
    v.x1 = in[0]; v.y1 = in[1]; v.z1 = in[2];
}

// two face crossings along axes a < b (split-vec.h cases 3, 5, 6)
template <typename T>
__device__ __forceinline__ void cut_two(Seg3<T> &v, Seg3<T> &w0, Seg3<T> &w1, int a, int b,
                                        int da, int db)
{
    const int o = 3 - a - b;
    T aint = T(0.5) * T(da);
    T delta = (aint - c0(v, a)) / (c1(v, a) - c0(v, a));
    T bint = c0(v, b) + (c1(v, b) - c0(v, b)) * delta;
    T oint = c0(v, o) + (c1(v, o) - c0(v, o)) * delta;
    w0 = v;
    w1 = v;
    if (bint >= T(-0.5) && bint < T(0.5)) {
        T bint2 = T(0.5) * T(db);
        T del2 = (bint2 - bint) / (c1(v, b) - bint);
        T aint2 = -aint + (c1(v, a) - aint) * del2;
        T oint2 = oint + (c1(v, o) - oint) * del2;
        c0(w0, a) = -aint; c1(w0, a) = aint2;
        c0(w0, b) = bint;  c1(w0, b) = bint2;
        c0(w0, o) = oint;  c1(w0, o) = oint2;
        ci(w0, a) += da;
        c0(w1, a) = aint2;  c1(w1, a) = c1(v, a) - T(da);
        c0(w1, b) = -bint2; c1(w1, b) = c1(v, b) - T(db);
        c0(w1, o) = oint2;  c1(w1, o) = c1(v, o);
        ci(w1, a) += da; ci(w1, b) += db;
        c1(v, a) = aint; c1(v, b) = bint; c1(v, o) = oint;
    } else {
        T bint2 = T(0.5) * T(db);
        T del2 = (bint2 - c0(v, b)) / (bint - c0(v, b));
        T aint2 = c0(v, a) + (aint - c0(v, a)) * del2;
        T oint2 = c0(v, o) + (oint - c0(v, o)) * del2;
        c0(w0, a) = aint2;  c1(w0, a) = aint;
        c0(w0, b) = -bint2; c1(w0, b) = bint - T(db);
        c0(w0, o) = oint2;  c1(w0, o) = oint;
        ci(w0, b) += db;
        c0(w1, a) = -aint;       c1(w1, a) = c1(v, a) - T(da);
        c0(w1, b) = bint - T(db); c1(w1, b) = c1(v, b) - T(db);
        c0(w1, o) = oint;        c1(w1, o) = c1(v, o);
        ci(w1, a) += da; ci(w1, b) += db;
        c1(v, a) = aint2; c1(v, b) = bint2; c1(v, o) = oint2;
    }
}

// Split a 3D move into <= 4 in-cell segments; returns the count.
template <typename T>
__device__ __forceinline__ int split3(Seg3<T> *s, int dix, int diy, int diz)
{
    const int cross = (dix != 0) | ((diy != 0) << 1) | ((diz != 0) << 2);
    switch (cross) {
    case 0: return 1;
    case 1: cut_one(s[0], s[1], 0, dix); return 2;
    case 2: cut_one(s[0], s[1], 1, diy); return 2;
    case 4: cut_one(s[0], s[1], 2, diz); return 2;
    case 3: cut_two(s[0], s[1], s[2], 0, 1, dix, diy); return 3;
    case 5: cut_two(s[0], s[1], s[2], 0, 2, dix, diz); return 3;
    case 6: cut_two(s[0], s[1], s[2], 1, 2, diy, diz); return 3;
    default: {
        cut_two(s[0], s[1], s[2], 0, 1, dix, diy);
        T zint = T(0.5) * T(diz);
        int n = 3;
#pragma unroll 1
        for (int t = 0; t < 3; t++) {
            Seg3<T> &c = s[t];
            if (c.z1 < T(-0.5) || c.z1 >= T(0.5)) {
                T delta = (zint - c.z0) / (c.z1 - c.z0);
                T xi = c.x0 + (c.x1 - c.x0) * delta;
                T yi = c.y0 + (c.y1 - c.y0) * delta;
                Seg3<T> &w = s[3];
                w.x0 = xi; w.x1 = c.x1; w.y0 = yi; w.y1 = c.y1;
                w.z0 = -zint; w.z1 = c.z1 - T(diz);
                w.i = c.i; w.j = c.j; w.k = c.k + diz;
                c.x1 = xi; c.y1 = yi; c.z1 = zint;
                for (int r = t + 1; r < 3; r++) {
                    s[r].z0 = s[r].z0 - T(diz);
                    s[r].z1 = s[r].z1 - T(diz);
                    s[r].k += diz;
                }
                n = 4;
                break;
            }
        }
        return n;
    }
    }
}

// ---------------------------------------------------------------------------------------
// Exact momentum update (push_type = "exact"; dudt_exact, source/spec/os-spec-extpush.f03:
// 40-348, after arXiv:2007.07556): the Lorentz force in the fields seen by the particle, held
// constant over the step, is integrated analytically; the proper time of the step comes from
// Newton iterations (get_t_light :352-391, get_t :395-430; at most 10, relative tolerance
// tol).  Precision as the Fortran source: T (p_k_part) arithmetic, every double literal and
// the insides of trig_func / hyper_func (:720-803) in double, rounded to T on assignment.
// ---------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void ex_fu(const T *ep, const T *bp, const T *u, T *f)
{
    f[3] = (ep[0] * u[0] + ep[1] * u[1]) + ep[2] * u[2];
    f[0] = (ep[0] * u[3] + bp[2] * u[1]) - bp[1] * u[2];
    f[1] = (ep[1] * u[3] - bp[2] * u[0]) + bp[0] * u[2];
    f[2] = (ep[2] * u[3] + bp[1] * u[0]) - bp[0] * u[1];
}

// cos x, sin x / x, (cos x - 1) / x^2  (hyp = true: cosh x, sinh x / x, (cosh x - 1) / x^2)
template <typename T, bool HYP>
__device__ __forceinline__ void ex_circ(T x, T &c, T &sc, T &cc)
{
    const double xd = (double)x, x2 = xd * xd;
    const double s = HYP ? 1.0 : -1.0;
    if (fabs(xd) < 0.007367081148666) {
        const double x4 = x2 * x2;
        c = (T)((1.0 + s * 0.5 * x2) + 0.041666666666667 * x4);
        sc = (T)((1.0 + s * 0.166666666666667 * x2) + 0.008333333333333 * x4);
        cc = (T)((s * 0.5 + 0.041666666666667 * x2) + s * 0.001388888888889 * x4);
    } else {
        const double t1 = HYP ? tanh(0.5 * xd) : tan(0.5 * xd), t2 = t1 * t1;
        const double t3 = 1.0 / (1.0 - s * t2);
        const double cd = (1.0 + s * t2) * t3;
        c = (T)cd;
        sc = (T)(((2.0 * t1) * t3) / xd);
        cc = (T)((cd - 1.0) / x2);
    }
}

// ep, bp: interpolated fields times q/m; u: momentum (in/out); dt: the double time step.
// Returns false (momentum unchanged) in a weak field, e^2 + b^2 < 1e-12.
template <typename T>
__device__ __noinline__ bool exact_u(const T *ep, const T *bp, T *u, double dt, double tol)
{
    const T e2 = (ep[0] * ep[0] + ep[1] * ep[1]) + ep[2] * ep[2];
    const T b2 = (bp[0] * bp[0] + bp[1] * bp[1]) + bp[2] * bp[2];
    if ((double)(e2 + b2) < 1.0e-12) return false;
    const T inv1 = e2 - b2;
    const T inv2 = (ep[0] * bp[0] + ep[1] * bp[1]) + ep[2] * bp[2];
    const T tmp = sqrtR(inv1 * inv1 + (T(4.0) * inv2) * inv2);
    const T k2 = T(0.5) * (inv1 + tmp), kk = sqrtR(k2);
    const T o2 = T(0.5) * (-inv1 + tmp), oo = sqrtR(o2);
    T u0[4], fu0[4], f2u0[4];
    u0[0] = u[0];
    u0[1] = u[1];
    u0[2] = u[2];
    u0[3] = sqrtR(((T(1.0) + u0[0] * u0[0]) + u0[1] * u0[1]) + u0[2] * u0[2]);
    ex_fu(ep, bp, u0, fu0);
    ex_fu(ep, bp, fu0, f2u0);
    if ((double)k2 < 1.0e-12 && (double)o2 < 1.0e-12) {
        T f3u0[4];
        ex_fu(ep, bp, f2u0, f3u0);
        T t1 = (T)(dt / (double)u0[3]), t = t1, c1 = T(0), c2 = T(0);
        for (int iter = 1;; iter++) {
            const T t2 = t1 * t1, t3 = t2 * t1;
            c1 = (T)(0.5 * (double)t2);
            c2 = (T)(0.166666666666667 * (double)t3);
            const T fa = (t1 * u0[3] + c1 * fu0[3]) + c2 * f2u0[3];
            const double fb = ((0.041666666666667 * (double)t3) * (double)t1) * (double)f3u0[3];
            const T fun = (T)(((double)fa + fb) - dt);
            const T dfun = ((u0[3] + t1 * fu0[3]) + c1 * f2u0[3]) + c2 * f3u0[3];
            t = t1 - fun / dfun;
            const T rel = (t - t1) < T(0) ? (t1 - t) / t1 : (t - t1) / t1;
            if ((double)rel < tol || iter > 10) break;
            t1 = t;
        }
#pragma unroll
        for (int c = 0; c < 3; c++) u[c] = ((u0[c] + t * fu0[c]) + c1 * f2u0[c]) + c2 * f3u0[c];
        return true;
    }
    const T k2o2 = k2 + o2;
    T uk0[4], uo0[4], fuk0[4], fuo0[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        uk0[c] = (f2u0[c] + o2 * u0[c]) / k2o2;
        uo0[c] = u0[c] - uk0[c];
    }
    ex_fu(ep, bp, uk0, fuk0);
#pragma unroll
    for (int c = 0; c < 4; c++) fuo0[c] = fu0[c] - fuk0[c];
    T t0 = (T)(dt / (double)(uk0[3] + uo0[3])), t = t0;
    T ch_k, shc_k, chc_k, cn_o, snc_o, cnc_o;
    for (int iter = 1;; iter++) {
        ex_circ<T, false>(oo * t0, cn_o, snc_o, cnc_o);
        ex_circ<T, true>(kk * t0, ch_k, shc_k, chc_k);
        const T fa = (uk0[3] * shc_k + (fuk0[3] * chc_k) * t0) * t0 +
                     (uo0[3] * snc_o - (fuo0[3] * cnc_o) * t0) * t0;
        const T fun = (T)((double)fa - dt);
        const T dfun = ((uk0[3] * ch_k + (fuk0[3] * shc_k) * t0) + uo0[3] * cn_o) +
                       (fuo0[3] * snc_o) * t0;
        t = t0 - fun / dfun;
        const T rel = (t - t0) < T(0) ? (t0 - t) / t0 : (t - t0) / t0;
        if ((double)rel < tol || iter > 10) break;
        t0 = t;
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const T uk = uk0[c] * ch_k + (fuk0[c] * shc_k) * t;
        const T uo = uo0[c] * cn_o + (fuo0[c] * snc_o) * t;
        u[c] = uk + uo;
    }
    return true;
}

// Exact momentum update from the unscaled interpolated fields (scaled by qm = 1/rqm as
// dudt_exact does, :76-86); returns q (gamma - 1) of the new momentum (its energy, :335-344).
template <typename T>
__device__ __forceinline__ T exact_push(T qm, double dt, double tol, T e1, T e2, T e3, T b1,
                                        T b2, T b3, T q, T &u1, T &u2, T &u3)
{
    const T ep[3] = {e1 * qm, e2 * qm, e3 * qm}, bp[3] = {b1 * qm, b2 * qm, b3 * qm};
    T u[3] = {u1, u2, u3};
    exact_u<T>(ep, bp, u, dt, tol);
    u1 = u[0];
    u2 = u[1];
    u3 = u[2];
    const T g = sqrtR(((T(1.0) + u1 * u1) + u2 * u2) + u3 * u3);
    return q * (g - T(1.0));
}

// ---------------------------------------------------------------------------------------
// Vay pusher (dudt_vay, source/spec/os-spec-push.f03:636-796; tem = real(0.5 dt / rqm),
// :663) and Higuera-Cary pusher (dudt_cary, :1104-1253; tem = real(0.5 (dt / rqm)), :1132),
// operation by operation as the Fortran (x**2 = x * x, a + b + c = (a + b) + c).  Both keep a
// particle at the E x B drift velocity exactly.  They return the energy term each reference
// pusher accumulates: Vay q uc^2 / (gamma_c + 1) of the time-centred momentum (in T), HC
// q u^2 / (sqrt(1 + u^2) + 1) of the half-kicked momentum (in double).
// ---------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T vay_push(T tem, T e1, T e2, T e3, T b1, T b2, T b3, T q, T &u1,
                                      T &u2, T &u3)
{
    const T ep[3] = {e1 * tem, e2 * tem, e3 * tem};
    T bp[3] = {b1 * tem, b2 * tem, b3 * tem};
    const T uo[3] = {u1, u2, u3};
    T rgam = T(1.0) / sqrtR(((T(1.0) + u1 * u1) + u2 * u2) + u3 * u3);
    T tv[3] = {u1 * rgam, u2 * rgam, u3 * rgam};
    const T bpsq = (bp[0] * bp[0] + bp[1] * bp[1]) + bp[2] * bp[2];
    T ut[3];
    ut[0] = ((uo[0] + ep[0]) + tv[1] * bp[2]) - tv[2] * bp[1];
    ut[1] = ((uo[1] + ep[1]) + tv[2] * bp[0]) - tv[0] * bp[2];
    ut[2] = ((uo[2] + ep[2]) + tv[0] * bp[1]) - tv[1] * bp[0];
#pragma unroll
    for (int c = 0; c < 3; c++) tv[c] = ut[c] + ep[c];
    const T ustar = (tv[0] * bp[0] + tv[1] * bp[1]) + tv[2] * bp[2];
    const T sigma = (((T(1.0) + tv[0] * tv[0]) + tv[1] * tv[1]) + tv[2] * tv[2]) - bpsq;
    rgam = T(1.0) / sqrtR(T(0.5) * (sigma + sqrtR(sigma * sigma + T(4.0) * (bpsq + ustar * ustar))));
#pragma unroll
    for (int c = 0; c < 3; c++) bp[c] = bp[c] * rgam;
    const T spar = T(1.0) / (((T(1.0) + bp[0] * bp[0]) + bp[1] * bp[1]) + bp[2] * bp[2]);
    const T uptp = (tv[0] * bp[0] + tv[1] * bp[1]) + tv[2] * bp[2];
    u1 = spar * (((tv[0] + uptp * bp[0]) + tv[1] * bp[2]) - tv[2] * bp[1]);
    u2 = spar * (((tv[1] + uptp * bp[1]) + tv[2] * bp[0]) - tv[0] * bp[2]);
    u3 = spar * (((tv[2] + uptp * bp[2]) + tv[0] * bp[1]) - tv[1] * bp[0]);
    const T uc[3] = {T(0.5) * (uo[0] + u1), T(0.5) * (uo[1] + u2), T(0.5) * (uo[2] + u3)};
    const T uc2 = (uc[0] * uc[0] + uc[1] * uc[1]) + uc[2] * uc[2];
    const T gc = sqrtR(uc2 + T(1.0));
    return (q * uc2) / (gc + T(1.0));
}

// Conditional Vay pusher (dudt_cond_vay, source/spec/os-spec-push.f03:800-1100): a particle
// whose gamma of the old momentum exceeds 5 takes the Vay update (and its energy term), the
// others the Fortran Boris update of the same routine -- half kick, rotation with
// b tem / gamma and 2 / (1 + |b|^2), half kick -- with the energy q u^2 / (gamma + 1) of the
// half-kicked momentum divided in double.  tem = real(0.5 dt / rqm) for both (:835).
template <typename T>
__device__ __forceinline__ double cond_vay_push(T tem, T e1, T e2, T e3, T b1, T b2, T b3, T q,
                                                T &u1, T &u2, T &u3)
{
    const T g0 = sqrtR(((T(1.0) + u1 * u1) + u2 * u2) + u3 * u3);
    if (g0 > T(5.0)) return (double)vay_push<T>(tem, e1, e2, e3, b1, b2, b3, q, u1, u2, u3);
    const T ep[3] = {e1 * tem, e2 * tem, e3 * tem};
    T ut[3] = {u1 + ep[0], u2 + ep[1], u3 + ep[2]};
    const T usq = (ut[0] * ut[0] + ut[1] * ut[1]) + ut[2] * ut[2];
    const T gam = sqrtR(usq + T(1.0));
    const double ene = (double)(q * usq) / ((double)gam + 1.0);
    const T gt = tem / gam;
    T bp[3] = {b1 * gt, b2 * gt, b3 * gt};
    T pn[3];
    pn[0] = ut[0] + ut[1] * bp[2];
    pn[1] = ut[1] + ut[2] * bp[0];
    pn[2] = ut[2] + ut[0] * bp[1];
    pn[0] = pn[0] - ut[2] * bp[1];
    pn[1] = pn[1] - ut[0] * bp[2];
    pn[2] = pn[2] - ut[1] * bp[0];
    const T otsq = T(2.0) / (((T(1.0) + bp[0] * bp[0]) + bp[1] * bp[1]) + bp[2] * bp[2]);
#pragma unroll
    for (int c = 0; c < 3; c++) bp[c] = bp[c] * otsq;
    ut[0] = ut[0] + pn[1] * bp[2];
    ut[1] = ut[1] + pn[2] * bp[0];
    ut[2] = ut[2] + pn[0] * bp[1];
    ut[0] = ut[0] - pn[2] * bp[1];
    ut[1] = ut[1] - pn[0] * bp[2];
    ut[2] = ut[2] - pn[1] * bp[0];
    u1 = ut[0] + ep[0];
    u2 = ut[1] + ep[1];
    u3 = ut[2] + ep[2];
    return ene;
}

template <typename T>
__device__ __forceinline__ double hc_push(T tem, T e1, T e2, T e3, T b1, T b2, T b3, T q, T &u1,
                                          T &u2, T &u3)
{
    const T ep[3] = {e1 * tem, e2 * tem, e3 * tem};
    T bp[3] = {b1 * tem, b2 * tem, b3 * tem};
    T ut[3] = {u1 + ep[0], u2 + ep[1], u3 + ep[2]};
    const T usq = (ut[0] * ut[0] + ut[1] * ut[1]) + ut[2] * ut[2];
    const T gm = (T)((double)usq + 1.0);
    const double ene = (double)(q * usq) / ((double)sqrtR(gm) + 1.0);
    const T bpsq = (bp[0] * bp[0] + bp[1] * bp[1]) + bp[2] * bp[2];
    T bdu = (bp[0] * ut[0] + bp[1] * ut[1]) + bp[2] * ut[2];
    bdu = bdu * bdu;
    const T gmb = gm - bpsq;
    const T gam = sqrtR(T(0.5) * (gmb + sqrtR(gmb * gmb + T(4.0) * (bpsq + bdu))));
#pragma unroll
    for (int c = 0; c < 3; c++) bp[c] = bp[c] / gam;
    T pn[3];
    pn[0] = ut[0] + ut[1] * bp[2];
    pn[1] = ut[1] + ut[2] * bp[0];
    pn[2] = ut[2] + ut[0] * bp[1];
    pn[0] = pn[0] - ut[2] * bp[1];
    pn[1] = pn[1] - ut[0] * bp[2];
    pn[2] = pn[2] - ut[1] * bp[0];
    const T otsq = T(2.0) / (((T(1.0) + bp[0] * bp[0]) + bp[1] * bp[1]) + bp[2] * bp[2]);
#pragma unroll
    for (int c = 0; c < 3; c++) bp[c] = bp[c] * otsq;
    ut[0] = ut[0] + pn[1] * bp[2];
    ut[1] = ut[1] + pn[2] * bp[0];
    ut[2] = ut[2] + pn[0] * bp[1];
    ut[0] = ut[0] - pn[2] * bp[1];
    ut[1] = ut[1] - pn[0] * bp[2];
    ut[2] = ut[2] - pn[1] * bp[0];
    u1 = ut[0] + ep[0];
    u2 = ut[1] + ep[1];
    u3 = ut[2] + ep[2];
    return ene;
}

// ---------------------------------------------------------------------------------------
// Full-rotation pusher (dudt_fullrot, source/spec/os-spec-push.f03:83-231): Boris with the
// rotation vector scaled by tan(b)/b (the reference's rational approximation in b^2,
// evaluated in double from the T value of b^2 and rounded back to T, :166-178), so a uniform
// magnetic field turns the momentum by the exact gyration angle.  Euler-rotation pusher
// (dudt_euler, :235-352): the magnetic rotation as the matrix of the quaternion
// (cos(w/2), -sin(w/2) b/|b|), w = |B| dt / (rqm gamma), the factor dt / (rqm gamma) in
// double from the T product rqm gamma (:289).  tem = real(0.5 (dt / rqm)); both return
// q u^2 / (gamma + 1) of the half-kicked momentum in double (:144-147, :278-281).
// ---------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ double fullrot_push(T tem, T e1, T e2, T e3, T b1, T b2, T b3, T q,
                                               T &u1, T &u2, T &u3)
{
    const T ep[3] = {e1 * tem, e2 * tem, e3 * tem};
    T ut[3] = {u1 + ep[0], u2 + ep[1], u3 + ep[2]};
    const T usq = (ut[0] * ut[0] + ut[1] * ut[1]) + ut[2] * ut[2];
    const T gamma = sqrtR(usq + T(1.0));
    const double ene = (double)(q * usq) / ((double)gamma + 1.0);
    const T tg = tem / gamma;
    T bp[3] = {b1 * tg, b2 * tg, b3 * tg};
    const T bsq = (bp[0] * bp[0] + bp[1] * bp[1]) + bp[2] * bp[2];
    const double d2 = (double)bsq;
    const T r = (T)(2005892.32789228135999056 +
                    d2 * (-267559.850143894287032640 +
                          d2 * (6870.7950060474599763728 - 35.8427314349709199363798 * d2)));
    const T s = (T)(2005892.32789228136020125 +
                    d2 * (-936190.626107988089080768 +
                          d2 * (51482.0266564063006502261 + d2 * (d2 - 625.608053837898687047447))));
    const T t = s != T(0.0) ? r / s : T(1.0);
#pragma unroll
    for (int c = 0; c < 3; c++) bp[c] = bp[c] * t;
    const T p[3] = {(ut[0] + ut[1] * bp[2]) - ut[2] * bp[1], (ut[1] + ut[2] * bp[0]) - ut[0] * bp[2],
                    (ut[2] + ut[0] * bp[1]) - ut[1] * bp[0]};
    const T sc = T(2.0) / (((T(1.0) + bp[0] * bp[0]) + bp[1] * bp[1]) + bp[2] * bp[2]);
#pragma unroll
    for (int c = 0; c < 3; c++) bp[c] = bp[c] * sc;
    ut[0] = (ut[0] + p[1] * bp[2]) - p[2] * bp[1];
    ut[1] = (ut[1] + p[2] * bp[0]) - p[0] * bp[2];
    ut[2] = (ut[2] + p[0] * bp[1]) - p[1] * bp[0];
    u1 = ut[0] + ep[0];
    u2 = ut[1] + ep[1];
    u3 = ut[2] + ep[2];
    return ene;
}

__device__ __forceinline__ float sinR(float x) { return sinf(x); }
__device__ __forceinline__ double sinR(double x) { return sin(x); }
__device__ __forceinline__ float cosR(float x) { return cosf(x); }
__device__ __forceinline__ double cosR(double x) { return cos(x); }

template <typename T>
__device__ __forceinline__ double euler_push(T tem, T rqm, double dt, T e1, T e2, T e3, T b1,
                                             T b2, T b3, T q, T &u1, T &u2, T &u3)
{
    const T ep[3] = {e1 * tem, e2 * tem, e3 * tem};
    const T ut[3] = {u1 + ep[0], u2 + ep[1], u3 + ep[2]};
    const T usq = (ut[0] * ut[0] + ut[1] * ut[1]) + ut[2] * ut[2];
    const T gamma = sqrtR(usq + T(1.0));
    const double ene = (double)(q * usq) / ((double)gamma + 1.0);
    const T gt = (T)(dt / (double)(rqm * gamma));
    const T bp[3] = {b1 * gt, b2 * gt, b3 * gt};
    const T bsq = (bp[0] * bp[0] + bp[1] * bp[1]) + bp[2] * bp[2];
    const T bn = sqrtR(bsq);
    T s = sinR(bn / T(2.0));
    const T a = cosR(bn / T(2.0));
    s = bsq > T(0.0) ? -s / bn : T(-1.0);
    const T qb = bp[0] * s, qc = bp[1] * s, qd = bp[2] * s;
    const T r11 = ((a * a + qb * qb) - qc * qc) - qd * qd, r21 = T(2.0) * (qb * qc - a * qd),
            r31 = T(2.0) * (qb * qd + a * qc);
    const T r12 = T(2.0) * (qb * qc + a * qd), r22 = ((a * a + qc * qc) - qb * qb) - qd * qd,
            r32 = T(2.0) * (qc * qd - a * qb);
    const T r13 = T(2.0) * (qb * qd - a * qc), r23 = T(2.0) * (qc * qd + a * qb),
            r33 = ((a * a + qd * qd) - qb * qb) - qc * qc;
    u1 = ((r11 * ut[0] + r21 * ut[1]) + r31 * ut[2]) + ep[0];
    u2 = ((r12 * ut[0] + r22 * ut[1]) + r32 * ut[2]) + ep[1];
    u3 = ((r13 * ut[0] + r23 * ut[1]) + r33 * ut[2]) + ep[2];
    return ene;
}

// the pusher-specific tem of the Fortran pushers from the double dt and the species' rqm
// (Higuera-Cary, full and Euler rotation: 0.5 (dt / rqm); Boris and Vay: 0.5 dt / rqm)
inline double pusher_tem(int pusher, double dt, double rqm)
{
    return pusher == OSG_PUSHER_HC || pusher == OSG_PUSHER_FULLROT || pusher == OSG_PUSHER_EULER
               ? 0.5 * (dt / rqm)
               : 0.5 * dt / rqm;
}

// Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC11): ten rounds of two 32x32 -> 64-bit multiplies, the key bumped by the Weyl constants
// between rounds.  A counter-based stream: every re-emission draws from its own counter.
__device__ __forceinline__ void philox4x32_10(unsigned int c[4], unsigned int k0, unsigned int k1)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const unsigned int lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
        const unsigned int lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
        const unsigned int n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// One thermal-bath draw for a particle re-emitted at the lower (lower = true) or upper edge of
// axis d (thermal_bath, source/spec/os-spec-boundary.f03:972-1067): the momentum un[3] and the
// uniform number v3 in (0, 1) that places it along d.  One Philox4x32-10 call, counter (the
// particle's id, its high word, step, d + 4 side) and key (seed, species); the four 32-bit
// outputs r become (r + 1/2) / 2^32 in double.  thermal_type 0 "thermal": uth_c times a
// Box-Muller Gaussian for the two tangential components and uth_d times the half-Maxwellian
// sqrt(-2 ln v) pointing into the box for the normal one; 1 "random dir"; 2 "waterbag".  The
// fluid momentum ufl is then added relativistically when all three of its components are
// non-zero.
template <typename T>
__device__ __forceinline__ void bath_draw(const T *uth, const T *ufl, int type, int d,
                                          bool lower, unsigned long long id, unsigned int step,
                                          unsigned int key0, unsigned int key1, T *un,
                                          double *v3out)
{
    const double inv32 = 2.3283064365386963e-10;   // 2^-32
    const int code = lower ? 1 : 2;
    unsigned int r[4] = {(unsigned int)id, (unsigned int)(id >> 32), step,
                         (unsigned int)(d + 4 * code)};
    philox4x32_10(r, key0, key1);
    const double v0 = (r[0] + 0.5) * inv32, v1 = (r[1] + 0.5) * inv32;
    const double v2 = (r[2] + 0.5) * inv32, v3 = (r[3] + 0.5) * inv32;
    const T usign = lower ? T(1) : T(-1);
    if (type == 1) {
        // "random dir": |uth| along a random direction, u3 = upar |uth| and the other two
        // on a circle of radius sqrt(1 - upar) |uth| (the reference's expression, :1026-1041)
        const T ut = sqrt(uth[0] * uth[0] + uth[1] * uth[1] + uth[2] * uth[2]);
        const T upar = (T)(2.0 * v0 - 1.0);
        const T uperp = sqrt(T(1) - upar) * ut;
        const T th = (T)(6.283185307179586 * v1);
        un[0] = cos(th) * uperp;
        un[1] = sin(th) * uperp;
        un[2] = upar * ut;
        un[d] = usign * fabs(un[d]);
    } else if (type == 2) {
        // "waterbag": uniform in [-uth/2, uth/2) per component (:1016-1024)
        const double w[3] = {v0, v1, v2};
        for (int c = 0; c < 3; c++) un[c] = uth[c] * (T)(w[c] - 0.5);
        un[d] = usign * fabs(un[d]);
    } else {
        const double rad = sqrt(-2.0 * log(v0)), th = 6.283185307179586 * v1;
        const double gs[2] = {rad * cos(th), rad * sin(th)};
        for (int c = 0, k = 0; c < 3; c++)
            if (c != d) un[c] = uth[c] * (T)gs[k++];
        un[d] = usign * uth[d] * (T)sqrt(-2.0 * log(v2));
    }
    const T f1 = ufl[0], f2 = ufl[1], f3 = ufl[2];
    if (f1 != T(0) && f2 != T(0) && f3 != T(0)) {
        const T fa = T(1) / (T(1) + sqrt(T(1) + f1 * f1 + f2 * f2 + f3 * f3));
        const T gth = sqrt(T(1) + un[0] * un[0] + un[1] * un[1] + un[2] * un[2]);
        const T fb = gth + fa * (f1 * un[0] + f2 * un[1] + f3 * un[2]);
        un[0] = un[0] + fb * f1;
        un[1] = un[1] + fb * f2;
        un[2] = un[2] + fb * f3;
    }
    *v3out = v3;
}

} // namespace osg
