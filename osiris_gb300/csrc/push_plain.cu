// push_plain.cu -- particle push + charge-conserving current deposition on the reference
// particle layout (ix(dim,N), x(dim,N), p(3,N), q(N)) with one thread per particle and
// global atomic current accumulation: the "plain" GPU form, in float and double.
//
// Reference algorithm: FNAME(vadvance_deposit_{1d,2d,3d}_sN), source/simd/
// os-spec-push-avx2d.c:263-475 (1D), :481-775 (2D), :1127-1467 (3D) and the deposits
// source/simd/os-spec-current-avx2d.c:189-278, :476-613, :854-1013.  Each thread gathers E and
// B with the staggered B-spline stencil, does the Boris update, moves the particle, trims it
// back into [-0.5, 0.5) of its new cell, splits the trajectory at cell faces and deposits the
// charge-conserving current of every segment.
//
// Memory safety: a particle whose cell index would put any stencil point outside the arrays
// is not pushed; the kernel raises OSG_STATUS_RANGE in the status word instead.
#include <cuda_runtime.h>

#include "common.cuh"
#include "pic_math.cuh"
#include "push_plain.cuh"
#include "tile_ops.cuh"

namespace osg {

template <typename T, int ORD>
__device__ __forceinline__ void deposit1(T *pj, T jn, T q, T x0, T x1, T vy, T vz, int i)
{
    constexpr int NP = ORD + 1;
    T s0[NP], s1[NP], wl[ORD];
    spline<ORD>(x0, s0);
    spline<ORD>(x1, s1);
    T qnx = q * jn, qvy = q * vy, qvz = q * vz;
    long_weights<ORD>(qnx, x0, x1, wl);
    T *p = pj + 3 * i;
#pragma unroll
    for (int k = 0; k < ORD; k++) atomicAdd(p + 3 * k, wl[k]);
#pragma unroll
    for (int k = 0; k < NP; k++) {
        T wp = T(0.5) * (s0[k] + s1[k]);
        atomicAdd(p + 3 * k + 1, qvy * wp);
        atomicAdd(p + 3 * k + 2, qvz * wp);
    }
}

template <typename T, int ORD>
__device__ __forceinline__ void deposit2(T *pj, long Dy, T jn0, T jn1, T q, const Seg2<T> &s)
{
    constexpr int NP = ORD + 1;
    T s0x[NP], s1x[NP], s0y[NP], s1y[NP], wl1[ORD], wl2[ORD], wp1[NP], wp2[NP];
    spline<ORD>(s.x0, s0x);
    spline<ORD>(s.x1, s1x);
    spline<ORD>(s.y0, s0y);
    spline<ORD>(s.y1, s1y);
    T qnx = q * jn0, qny = q * jn1;
    T qvz = (q * s.vz) * T(1.0 / 3.0);
    long_weights<ORD>(qnx, s.x0, s.x1, wl1);
    long_weights<ORD>(qny, s.y0, s.y1, wl2);
#pragma unroll
    for (int k = 0; k < NP; k++) {
        wp1[k] = s0y[k] + s1y[k];
        wp2[k] = s0x[k] + s1x[k];
    }
    T *p = pj + 3L * s.i + Dy * s.j;
#pragma unroll
    for (int k2 = 0; k2 < NP; k2++)
#pragma unroll
        for (int k1 = 0; k1 < ORD; k1++) atomicAdd(p + 3 * k1 + Dy * k2, wl1[k1] * wp1[k2]);
#pragma unroll
    for (int k2 = 0; k2 < ORD; k2++)
#pragma unroll
        for (int k1 = 0; k1 < NP; k1++) atomicAdd(p + 3 * k1 + Dy * k2 + 1, wl2[k2] * wp2[k1]);
#pragma unroll
    for (int k2 = 0; k2 < NP; k2++)
#pragma unroll
        for (int k1 = 0; k1 < NP; k1++) {
            T t1 = fmaR(s1y[k2], s1x[k1], s0x[k1] * s0y[k2]);
            T t2 = fmaR(s0y[k2], s1x[k1], s0x[k1] * s1y[k2]);
            t1 = fmaR(t2, T(0.5), t1);
            atomicAdd(p + 3 * k1 + Dy * k2 + 2, qvz * t1);
        }
}

template <typename T, int ORD>
__device__ __forceinline__ void deposit3(T *pj, long Dy, long Dz, T jn0, T jn1, T jn2, T q,
                                         const Seg3<T> &s)
{
    constexpr int NP = ORD + 1;
    T s0x[NP], s1x[NP], s0y[NP], s1y[NP], s0z[NP], s1z[NP], wl1[ORD], wl2[ORD], wl3[ORD];
    spline<ORD>(s.x0, s0x);
    spline<ORD>(s.x1, s1x);
    spline<ORD>(s.y0, s0y);
    spline<ORD>(s.y1, s1y);
    spline<ORD>(s.z0, s0z);
    spline<ORD>(s.z1, s1z);
    long_weights<ORD>(q * jn0, s.x0, s.x1, wl1);
    long_weights<ORD>(q * jn1, s.y0, s.y1, wl2);
    long_weights<ORD>(q * jn2, s.z0, s.z1, wl3);
    T *p = pj + 3L * s.i + Dy * s.j + Dz * s.k;
    // perpendicular weights: wp(b, a) = s0a s0b + s1a s1b + (s0a s1b + s1a s0b) / 2
#pragma unroll
    for (int k3 = 0; k3 < NP; k3++)
#pragma unroll
        for (int k2 = 0; k2 < NP; k2++) {
            T t1 = s0y[k2] * s0z[k3], t2 = s0y[k2] * s1z[k3];
            t1 = fmaR(s1y[k2], s1z[k3], t1);
            t2 = fmaR(s1y[k2], s0z[k3], t2);
            T wp1 = fmaR(T(0.5), t2, t1);
#pragma unroll
            for (int k1 = 0; k1 < ORD; k1++)
                atomicAdd(p + 3 * k1 + Dy * k2 + Dz * k3, wl1[k1] * wp1);
        }
#pragma unroll
    for (int k3 = 0; k3 < NP; k3++)
#pragma unroll
        for (int k1 = 0; k1 < NP; k1++) {
            T t1 = s0x[k1] * s0z[k3], t2 = s0x[k1] * s1z[k3];
            t1 = fmaR(s1x[k1], s1z[k3], t1);
            t2 = fmaR(s1x[k1], s0z[k3], t2);
            T wp2 = fmaR(T(0.5), t2, t1);
#pragma unroll
            for (int k2 = 0; k2 < ORD; k2++)
                atomicAdd(p + 3 * k1 + Dy * k2 + Dz * k3 + 1, wl2[k2] * wp2);
        }
#pragma unroll
    for (int k2 = 0; k2 < NP; k2++)
#pragma unroll
        for (int k1 = 0; k1 < NP; k1++) {
            T t1 = s0x[k1] * s0y[k2], t2 = s0x[k1] * s1y[k2];
            t1 = fmaR(s1x[k1], s1y[k2], t1);
            t2 = fmaR(s1x[k1], s0y[k2], t2);
            T wp3 = fmaR(T(0.5), t2, t1);
#pragma unroll
            for (int k3 = 0; k3 < ORD; k3++)
                atomicAdd(p + 3 * k1 + Dy * k2 + Dz * k3 + 2, wl3[k3] * wp3);
        }
}

// A cell index c (Fortran, 1-based) is safe when every gather point and every deposit point
// of the segments that can start from it lies inside [0, size) of the array:
// points c - OFS .. c + NP - OFS + 1 map to positions c - OFS - 1 + off .. c + NP - OFS + off.
template <int ORD>
__device__ __forceinline__ bool cell_ok(int c, int off, int size)
{
    constexpr int NP = ORD + 1, OFS = Stencil<ORD>::OFS;
    return c - OFS - 1 + off >= 0 && c + NP - OFS + off < size;
}

// periodic single-node wrap of a cell index (source/spec/os-spec-boundary.f03:1280-1290);
// n = 0 leaves the index as pushed (the reference kernel itself does not wrap)
__device__ __forceinline__ int wrap_cell(int c, int n)
{
    if (n > 0) {
        if (c < 1) c += n;
        else if (c > n) c -= n;
    }
    return c;
}

// New cell and offset of a particle along axis d: periodic wrap, or specular reflection at a
// conducting wall (p_bc_specular, source/spec/os-spec-boundary.f03:1293-1310: the momentum
// along d flips, the particle goes to the edge cell at the mirrored offset), after its current
// was deposited along the unreflected path; or absorption at an open edge (p_bc_absorbing,
// :501-511: the reference removes the particle after its deposit; here it stays in the
// arrays with charge and momentum 0 at offset 0 of the edge cell, and deposits nothing more).
// A crossing of a thermal-bath edge returns 1 (lower) or 2 (upper) and leaves the cell outside
// the box; thermal_reemit then moves the particle to the edge cell and sets its momentum and
// offset (axis by axis, as the reference's boundary loop, which meets a particle crossing two
// edges with the second axis not yet processed).
template <typename T, int DIM>
__device__ __forceinline__ int store_position(const PlainPushArgs<T> &a, long p, int d, int cn,
                                              T xn)
{
    int code = 0;
    if (a.thermal[d] > 0 && (cn < 1 || cn > a.thermal[d])) {
        code = cn < 1 ? 1 : 2;
    } else if (a.absorb[d] > 0 && (cn < 1 || cn > a.absorb[d])) {
        cn = cn < 1 ? 1 : a.absorb[d];
        xn = T(0);
        a.u[3 * p + 0] = T(0);
        a.u[3 * p + 1] = T(0);
        a.u[3 * p + 2] = T(0);
        a.q_absorb[p] = T(0);
    } else if (a.reflect[d] > 0 && (cn < 1 || cn > a.reflect[d])) {
        cn = cn < 1 ? 1 : a.reflect[d];
        xn = -xn;
        a.u[3 * p + d] = -a.u[3 * p + d];
    } else {
        cn = wrap_cell(cn, a.wrap[d]);
    }
    a.x[DIM * p + d] = xn;
    a.ix[DIM * p + d] = cn;
    return code << (2 * d);
}

// Thermal-bath re-emission of particle p after it crossed the edges coded in tb (2 bits per
// axis: 1 lower, 2 upper), axis by axis (p_bc_thermal, source/spec/os-spec-boundary.f03:
// 1315-1387, with thermal_bath :972-1067; thermal_type "thermal" below, "random dir" and
// "waterbag" in the branches):
//  * momentum: uth_c times a Gaussian for the two other components, uth_d times a
//    half-Maxwellian sqrt(-2 ln v) pointing into the box for the normal one, then the fluid
//    momentum ufl added relativistically when all three of its components are non-zero;
//  * offset along d: xpos + vperp delta, xpos = -1/2 (lower) or the float just below 1/2
//    (upper), vperp = u_d / gamma dt/dx_d, delta uniform in (0, 1);
//  * current: -q moved from the new position back along -u / gamma dt/dx (rev_current :1392-
//    1440; in 2D the out-of-plane current keeps +u3, as the reference's).
// The random numbers come from one Philox4x32-10 call per re-emission, counter (p, step, d and
// side), key (seed, species): two Box-Muller Gaussians, the half-Maxwellian and delta, each
// from (r + 1/2) / 2^32 in double.  The reference draws from its one sequential generator in
// the order the boundary routine meets the particles; the distributions are the same.
template <typename T, int DIM, int ORD>
__device__ __noinline__ void thermal_reemit(const PlainPushArgs<T> &a, long p, T q, int tb)
{
    for (int d = 0; d < DIM; d++) {
        const int code = (tb >> (2 * d)) & 3;
        if (!code) continue;
        const bool lower = code == 1;
        a.ix[DIM * p + d] = lower ? 1 : a.thermal[d];
        T un[3];
        double v3;
        bath_draw<T>(a.uth_bnd, a.ufl_bnd, a.thermal_type, d, lower,
                     (unsigned long long)p, (unsigned int)*a.step, a.rng_key[0], a.rng_key[1],
                     un, &v3);
        for (int c = 0; c < 3; c++) a.u[3 * p + c] = un[c];
        const T rg = T(1) / sqrt(T(1) + un[0] * un[0] + un[1] * un[1] + un[2] * un[2]);
        const T xpos = lower ? T(-0.5) : (sizeof(T) == 4 ? T(0.49999997f) : T(0.49999999999999994));
        const T vperp = rg * un[d] * a.dtdx[d];
        a.x[DIM * p + d] = xpos + vperp * (T)v3;
        // the current of the way in: -q from the new position back to where it came from
        T xn[3], xv[3];
        int cc[3];
        for (int k = 0; k < DIM; k++) {
            xn[k] = a.x[DIM * p + k];
            cc[k] = a.ix[DIM * p + k];
            xv[k] = xn[k] - un[k] * rg * a.dtdx[k];
        }
        if constexpr (DIM == 2) {
            Seg2<T> s[3];
            s[0].x0 = xn[0]; s[0].x1 = xv[0]; s[0].y0 = xn[1]; s[0].y1 = xv[1];
            s[0].vz = un[2] * rg; s[0].i = cc[0]; s[0].j = cc[1];
            const int ns = split2(s, trim(xv[0]), trim(xv[1]));
            for (int t = 0; t < ns; t++)
                deposit2<T, ORD>(a.j, a.j_Dy, a.jn[0], a.jn[1], -q, s[t]);
        } else if constexpr (DIM == 3) {
            Seg3<T> s[4];
            s[0].x0 = xn[0]; s[0].x1 = xv[0]; s[0].y0 = xn[1]; s[0].y1 = xv[1];
            s[0].z0 = xn[2]; s[0].z1 = xv[2]; s[0].i = cc[0]; s[0].j = cc[1]; s[0].k = cc[2];
            const int ns = split3(s, trim(xv[0]), trim(xv[1]), trim(xv[2]));
            for (int t = 0; t < ns; t++)
                deposit3<T, ORD>(a.j, a.j_Dy, a.j_Dz, a.jn[0], a.jn[1], a.jn[2], -q, s[t]);
        }
    }
}

// FP32 2D orders whose per-warp value scratch (8 warps) fits 32 KB of static shared memory
// deposit their in-cell segments by warp runs (cell_runs_deposit_global2): 2x faster on the
// two-stream workload.  The others add every value with its own atomic (FP64: native double
// atomics, and the runs measured 8% slower)
template <typename T, int DIM, int ORD>
constexpr bool plain_runs()
{
    return DIM == 2 && sizeof(T) == 4 && SegVals<2, ORD>::NV * SCR_LD * sizeof(T) * 8 <= 32768;
}

template <typename T, int DIM, int ORD>
__global__ void __launch_bounds__(256) k_push_plain(PlainPushArgs<T> a)
{
    constexpr int NP = ORD + 1;
    constexpr bool RUNS = plain_runs<T, DIM, ORD>();
    constexpr int NV = SegVals<2, ORD>::NV, NC = (NV + 31) / 32;
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double my_ene = 0.0;
    // FP32 Boris: the energy term q ene in FP32 (as the reference's single-precision kernels),
    // summed per block in FP32 (FP64 arithmetic runs at a small fraction of the FP32 rate here)
    float my_ene_f = 0.f;
    long run_base = -1;   // RUNS: stencil origin of the in-cell segment in J (-1: none)
    T rv[RUNS ? NV : 1];
    if constexpr (RUNS) {
#pragma unroll
        for (int k = 0; k < NV; k++) rv[k] = T(0);
    }
    if (p < a.np) {
        int c[DIM];
        T x0[DIM];
        bool ok = true;
#pragma unroll
        for (int d = 0; d < DIM; d++) {
            c[d] = a.ix[DIM * p + d];
            x0[d] = a.x[DIM * p + d];
            ok = ok && cell_ok<ORD>(c[d], a.emf_off[d], a.emf_size[d]) &&
                 cell_ok<ORD>(c[d], a.j_off[d], a.j_size[d]);
        }
        if (!ok) {
            atomicOr(a.status, OSG_STATUS_RANGE);
        } else {
            const T q = a.q[p];
            T w[DIM][NP], wh[DIM][NP];
            int ch[DIM];
#pragma unroll
            for (int d = 0; d < DIM; d++) {
                spline<ORD>(x0[d], w[d]);
                const bool neg = x0[d] < T(0);
                ch[d] = c[d] - (neg ? 1 : 0);
                spline_h<ORD>(x0[d], neg ? T(1) : T(0), wh[d]);
            }
            const T *__restrict__ e0 = a.efield;
            const T *__restrict__ b0 = a.bfield;
            T E1 = T(0), E2 = T(0), E3 = T(0), B1 = T(0), B2 = T(0), B3 = T(0);
            if constexpr (DIM == 1) {
#pragma unroll
                for (int k = 0; k < NP; k++) {
                    E1 = fmaR(__ldg(e0 + 3 * (ch[0] + k) + 0), wh[0][k], E1);
                    E2 = fmaR(__ldg(e0 + 3 * (c[0] + k) + 1), w[0][k], E2);
                    E3 = fmaR(__ldg(e0 + 3 * (c[0] + k) + 2), w[0][k], E3);
                }
#pragma unroll
                for (int k = 0; k < NP; k++) {
                    B1 = fmaR(__ldg(b0 + 3 * (c[0] + k) + 0), w[0][k], B1);
                    B2 = fmaR(__ldg(b0 + 3 * (ch[0] + k) + 1), wh[0][k], B2);
                    B3 = fmaR(__ldg(b0 + 3 * (ch[0] + k) + 2), wh[0][k], B3);
                }
            } else if constexpr (DIM == 2) {
                const long Dy = a.emf_Dy;
#pragma unroll
                for (int k2 = 0; k2 < NP; k2++) {
                    T f1 = T(0), f2 = T(0), f3 = T(0);
#pragma unroll
                    for (int k1 = 0; k1 < NP; k1++) {
                        f1 = fmaR(__ldg(e0 + 3L * (ch[0] + k1) + Dy * (c[1] + k2) + 0), wh[0][k1], f1);
                        f2 = fmaR(__ldg(e0 + 3L * (c[0] + k1) + Dy * (ch[1] + k2) + 1), w[0][k1], f2);
                        f3 = fmaR(__ldg(e0 + 3L * (c[0] + k1) + Dy * (c[1] + k2) + 2), w[0][k1], f3);
                    }
                    E1 = fmaR(f1, w[1][k2], E1);
                    E2 = fmaR(f2, wh[1][k2], E2);
                    E3 = fmaR(f3, w[1][k2], E3);
                }
#pragma unroll
                for (int k2 = 0; k2 < NP; k2++) {
                    T f1 = T(0), f2 = T(0), f3 = T(0);
#pragma unroll
                    for (int k1 = 0; k1 < NP; k1++) {
                        f1 = fmaR(__ldg(b0 + 3L * (c[0] + k1) + Dy * (ch[1] + k2) + 0), w[0][k1], f1);
                        f2 = fmaR(__ldg(b0 + 3L * (ch[0] + k1) + Dy * (c[1] + k2) + 1), wh[0][k1], f2);
                        f3 = fmaR(__ldg(b0 + 3L * (ch[0] + k1) + Dy * (ch[1] + k2) + 2), wh[0][k1], f3);
                    }
                    B1 = fmaR(f1, wh[1][k2], B1);
                    B2 = fmaR(f2, w[1][k2], B2);
                    B3 = fmaR(f3, wh[1][k2], B3);
                }
            } else {
                const long Dy = a.emf_Dy, Dz = a.emf_Dz;
#pragma unroll
                for (int k3 = 0; k3 < NP; k3++) {
                    T g1 = T(0), g2 = T(0), g3 = T(0);
#pragma unroll
                    for (int k2 = 0; k2 < NP; k2++) {
                        T f1 = T(0), f2 = T(0), f3 = T(0);
#pragma unroll
                        for (int k1 = 0; k1 < NP; k1++) {
                            f1 = fmaR(__ldg(e0 + 3L * (ch[0] + k1) + Dy * (c[1] + k2) + Dz * (c[2] + k3) + 0), wh[0][k1], f1);
                            f2 = fmaR(__ldg(e0 + 3L * (c[0] + k1) + Dy * (ch[1] + k2) + Dz * (c[2] + k3) + 1), w[0][k1], f2);
                            f3 = fmaR(__ldg(e0 + 3L * (c[0] + k1) + Dy * (c[1] + k2) + Dz * (ch[2] + k3) + 2), w[0][k1], f3);
                        }
                        g1 = fmaR(f1, w[1][k2], g1);
                        g2 = fmaR(f2, wh[1][k2], g2);
                        g3 = fmaR(f3, w[1][k2], g3);
                    }
                    E1 = fmaR(g1, w[2][k3], E1);
                    E2 = fmaR(g2, w[2][k3], E2);
                    E3 = fmaR(g3, wh[2][k3], E3);
                }
#pragma unroll
                for (int k3 = 0; k3 < NP; k3++) {
                    T g1 = T(0), g2 = T(0), g3 = T(0);
#pragma unroll
                    for (int k2 = 0; k2 < NP; k2++) {
                        T f1 = T(0), f2 = T(0), f3 = T(0);
#pragma unroll
                        for (int k1 = 0; k1 < NP; k1++) {
                            f1 = fmaR(__ldg(b0 + 3L * (c[0] + k1) + Dy * (ch[1] + k2) + Dz * (ch[2] + k3) + 0), w[0][k1], f1);
                            f2 = fmaR(__ldg(b0 + 3L * (ch[0] + k1) + Dy * (c[1] + k2) + Dz * (ch[2] + k3) + 1), wh[0][k1], f2);
                            f3 = fmaR(__ldg(b0 + 3L * (ch[0] + k1) + Dy * (ch[1] + k2) + Dz * (c[2] + k3) + 2), wh[0][k1], f3);
                        }
                        g1 = fmaR(f1, wh[1][k2], g1);
                        g2 = fmaR(f2, w[1][k2], g2);
                        g3 = fmaR(f3, wh[1][k2], g3);
                    }
                    B1 = fmaR(g1, wh[2][k3], B1);
                    B2 = fmaR(g2, wh[2][k3], B2);
                    B3 = fmaR(g3, w[2][k3], B3);
                }
            }
            T u1 = a.u[3 * p], u2 = a.u[3 * p + 1], u3 = a.u[3 * p + 2];
            if (a.pusher == OSG_PUSHER_EXACT) {
                my_ene = (double)exact_push<T>(a.qm, a.dt_full, a.iter_tol, E1, E2, E3, B1, B2,
                                               B3, q, u1, u2, u3);
            } else if (a.pusher == OSG_PUSHER_VAY) {
                my_ene = (double)vay_push<T>(a.tem, E1, E2, E3, B1, B2, B3, q, u1, u2, u3);
            } else if (a.pusher == OSG_PUSHER_HC) {
                my_ene = hc_push<T>(a.tem, E1, E2, E3, B1, B2, B3, q, u1, u2, u3);
            } else if (a.pusher == OSG_PUSHER_FULLROT) {
                my_ene = fullrot_push<T>(a.tem, E1, E2, E3, B1, B2, B3, q, u1, u2, u3);
            } else if (a.pusher == OSG_PUSHER_EULER) {
                my_ene = euler_push<T>(a.tem, a.rqm, a.dt_full, E1, E2, E3, B1, B2, B3, q, u1,
                                       u2, u3);
            } else if (a.pusher == OSG_PUSHER_COND_VAY) {
                my_ene = cond_vay_push<T>(a.tem, E1, E2, E3, B1, B2, B3, q, u1, u2, u3);
            } else {
                const T ene = boris(a.tem, E1, E2, E3, B1, B2, B3, u1, u2, u3);
                if constexpr (sizeof(T) == 4) my_ene_f = q * ene;
                else my_ene = (double)q * (double)ene;
            }
            a.u[3 * p] = u1;
            a.u[3 * p + 1] = u2;
            a.u[3 * p + 2] = u3;
            const T rg = rgamma(u1, u2, u3);
            const T v1 = u1 * rg, v2 = u2 * rg, v3 = u3 * rg;
            if constexpr (DIM == 1) {
                T x1 = fmaR(v1, a.dtdx[0], x0[0]);
                int dix = trim(x1);
                store_position<T, 1>(a, p, 0, c[0] + dix, x1 - T(dix));
                if (dix == 0) {
                    deposit1<T, ORD>(a.j, a.jn[0], q, x0[0], x1, v2, v3, c[0]);
                } else {
                    T xint = T(0.5 * dix);
                    T delta = (xint - x0[0]) / (x1 - x0[0]);
                    deposit1<T, ORD>(a.j, a.jn[0], q, x0[0], xint, v2 * delta, v3 * delta, c[0]);
                    deposit1<T, ORD>(a.j, a.jn[0], q, -xint, x1 - T(dix), v2 * (T(1) - delta),
                                     v3 * (T(1) - delta), c[0] + dix);
                }
            } else if constexpr (DIM == 2) {
                T x1 = fmaR(v1, a.dtdx[0], x0[0]);
                T y1;
                if (a.cyl) {
                    // cylindrical radial move, in double as the reference (both precisions;
                    // source/simd/os-spec-push-avx2d.c:1029-1065, os-spec-push-avx2.c:
                    // 992-1080): from the global radius r_old the particle moves to
                    // (r_old + v2 dt, v3 dt) in the (r, theta) plane; its new radius r_new
                    // gives x2 (unchanged when r_new == r_old: cold plasma roundoff), and
                    // p_r, p_theta turn onto the new radial direction (angular momentum
                    // kept).  The deposit below keeps the Cartesian velocities.
                    const double gix2 = (double)c[1] + a.cyl_gshift;
                    const double r_old = ((double)x0[1] + gix2) * a.cyl_dr;
                    const double x2n = fma((double)v2, a.dt_full, r_old);
                    const double x3n = (double)v3 * a.dt_full;
                    const double r_new = sqrt(fma(x2n, x2n, x3n * x3n));
                    const double y1d = r_old == r_new ? (double)x0[1]
                                                      : fma(r_new, a.cyl_rdr, -gix2);
                    y1 = (T)y1d;
                    const double tmp = 1.0 / r_new;
                    a.u[3 * p + 1] = (T)(fma((double)u2, x2n, (double)u3 * x3n) * tmp);
                    a.u[3 * p + 2] = (T)((double)u3 * (r_old * tmp));
                } else {
                    y1 = fmaR(v2, a.dtdx[1], x0[1]);
                }
                int dix = trim(x1), diy = trim(y1);
                const int tb = store_position<T, 2>(a, p, 0, c[0] + dix, x1 - T(dix)) |
                               store_position<T, 2>(a, p, 1, c[1] + diy, y1 - T(diy));
                Seg2<T> s[3];
                s[0].x0 = x0[0]; s[0].x1 = x1; s[0].y0 = x0[1]; s[0].y1 = y1;
                s[0].vz = v3; s[0].i = c[0]; s[0].j = c[1];
                const int ns = split2(s, dix, diy);
                if constexpr (RUNS) {
                    seg_values2<ORD, T>(s[0], q, a.jn[0], a.jn[1], rv);
                    run_base = 3L * s[0].i + a.j_Dy * s[0].j;
                    for (int t = 1; t < ns; t++)
                        deposit2<T, ORD>(a.j, a.j_Dy, a.jn[0], a.jn[1], q, s[t]);
                } else {
                    for (int t = 0; t < ns; t++)
                        deposit2<T, ORD>(a.j, a.j_Dy, a.jn[0], a.jn[1], q, s[t]);
                }
                if (tb) thermal_reemit<T, 2, ORD>(a, p, q, tb);
            } else {
                T x1 = fmaR(v1, a.dtdx[0], x0[0]);
                T y1 = fmaR(v2, a.dtdx[1], x0[1]);
                T z1 = fmaR(v3, a.dtdx[2], x0[2]);
                int dix = trim(x1), diy = trim(y1), diz = trim(z1);
                const int tb = store_position<T, 3>(a, p, 0, c[0] + dix, x1 - T(dix)) |
                               store_position<T, 3>(a, p, 1, c[1] + diy, y1 - T(diy)) |
                               store_position<T, 3>(a, p, 2, c[2] + diz, z1 - T(diz));
                Seg3<T> s[4];
                s[0].x0 = x0[0]; s[0].x1 = x1; s[0].y0 = x0[1]; s[0].y1 = y1;
                s[0].z0 = x0[2]; s[0].z1 = z1; s[0].i = c[0]; s[0].j = c[1]; s[0].k = c[2];
                const int ns = split3(s, dix, diy, diz);
                for (int t = 0; t < ns; t++)
                    deposit3<T, ORD>(a.j, a.j_Dy, a.j_Dz, a.jn[0], a.jn[1], a.jn[2], q, s[t]);
                if (tb) thermal_reemit<T, 3, ORD>(a, p, q, tb);
            }
        }
    }
    if constexpr (RUNS) {
        __shared__ T sScr[8][NV * SCR_LD];
        __shared__ long sBase[8][16];
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        int off[NC];
#pragma unroll
        for (int c = 0; c < NC; c++)
            off[c] = lane + 32 * c < NV ? seg_offset<2, ORD>(lane + 32 * c, (int)a.j_Dy, 0) : 0;
        cell_runs_deposit_global2<T, ORD>(a.j, sScr[w], sBase[w], run_base, rv, off);
    }
    if constexpr (sizeof(T) == 4) {
        if (a.pusher == OSG_PUSHER_BORIS) {
            const float tot = block_sum_f(my_ene_f);
            if (threadIdx.x == 0 && tot != 0.f) atomicAdd(a.ene, (double)tot);
            return;
        }
    }
    const double tot = block_sum(my_ene);
    if (threadIdx.x == 0 && tot != 0.0) atomicAdd(a.ene, tot);
}

template <typename T>
PlainPushArgs<T> make_plain_args(int dim, int order, int *ix, T *x, T *u, const T *q, long np,
                                 T rqm, const T *e, const T *b, const int *emf_size,
                                 const int *emf_off, T *j, const int *j_size, const int *j_off,
                                 const double *dx, double dt, double *d_ene, int *d_status)
{
    PlainPushArgs<T> a;
    const int OFS = order == 1 ? 1 : (order == 2 ? 2 : (order == 3 ? 2 : 3));
    a.ix = ix; a.x = x; a.u = u; a.q = q; a.np = np;
    a.tem = (T)(0.5 * dt / (double)rqm);
    long eDy = 3L * emf_size[0], eDz = dim > 2 ? eDy * emf_size[1] : 0;
    long jDy = 3L * j_size[0], jDz = dim > 2 ? jDy * j_size[1] : 0;
    long eo = (emf_off[0] - OFS) * 3L, jo = (j_off[0] - OFS) * 3L;
    if (dim > 1) { eo += (emf_off[1] - OFS) * eDy; jo += (j_off[1] - OFS) * jDy; }
    if (dim > 2) { eo += (emf_off[2] - OFS) * eDz; jo += (j_off[2] - OFS) * jDz; }
    a.efield = e + eo;
    a.bfield = b + eo;
    a.j = j + jo;
    a.emf_Dy = eDy; a.emf_Dz = eDz; a.j_Dy = jDy; a.j_Dz = jDz;
    for (int d = 0; d < 3; d++) {
        a.emf_off[d] = d < dim ? emf_off[d] : 0;
        a.emf_size[d] = d < dim ? emf_size[d] : 1;
        a.j_off[d] = d < dim ? j_off[d] : 0;
        a.j_size[d] = d < dim ? j_size[d] : 1;
        a.dtdx[d] = d < dim ? (T)(dt / dx[d]) : T(0);
        const double div = dim == 1 ? 1.0 : (dim == 2 ? 2.0 : 3.0);
        a.jn[d] = d < dim ? (T)(dx[d] / dt / div) : T(0);
    }
    a.wrap[0] = a.wrap[1] = a.wrap[2] = 0;
    a.reflect[0] = a.reflect[1] = a.reflect[2] = 0;
    a.absorb[0] = a.absorb[1] = a.absorb[2] = 0;
    a.q_absorb = nullptr;
    for (int d = 0; d < 3; d++) {
        a.thermal[d] = 0;
        a.uth_bnd[d] = a.ufl_bnd[d] = T(0);
    }
    a.step = nullptr;
    a.rng_key[0] = a.rng_key[1] = 0;
    a.thermal_type = 0;
    a.pusher = OSG_PUSHER_BORIS;
    a.qm = T(1) / rqm;
    a.rqm = rqm;
    a.dt_full = dt;
    a.cyl = 0;
    a.cyl_gshift = 0.0;
    a.cyl_dr = dim > 1 ? dx[1] : 0.0;
    a.cyl_rdr = dim > 1 ? 1.0 / dx[1] : 0.0;
    a.iter_tol = 1.0e-3;
    a.ene = d_ene;
    a.status = d_status;
    return a;
}

template <typename T, int DIM, int ORD>
static void launch_one(const PlainPushArgs<T> &a, cudaStream_t st)
{
    if (a.np <= 0) return;
    k_push_plain<T, DIM, ORD><<<blocks_for(a.np, 256), 256, 0, st>>>(a);
}

template <typename T>
int launch_plain_push(int dim, int order, const PlainPushArgs<T> &a, cudaStream_t st)
{
#define OSG_CASE(D, O)                                                                        \
    if (dim == D && order == O) {                                                             \
        launch_one<T, D, O>(a, st);                                                           \
        return OSG_OK;                                                                        \
    }
    OSG_CASE(1, 1) OSG_CASE(1, 2) OSG_CASE(1, 3) OSG_CASE(1, 4)
    OSG_CASE(2, 1) OSG_CASE(2, 2) OSG_CASE(2, 3) OSG_CASE(2, 4)
    OSG_CASE(3, 1) OSG_CASE(3, 2) OSG_CASE(3, 3) OSG_CASE(3, 4)
#undef OSG_CASE
    set_error("unsupported dim %d / order %d", dim, order);
    return OSG_ERR_ARG;
}

template PlainPushArgs<float> make_plain_args<float>(int, int, int *, float *, float *,
                                                     const float *, long, float, const float *,
                                                     const float *, const int *, const int *,
                                                     float *, const int *, const int *,
                                                     const double *, double, double *, int *);
template PlainPushArgs<double> make_plain_args<double>(int, int, int *, double *, double *,
                                                       const double *, long, double,
                                                       const double *, const double *,
                                                       const int *, const int *, double *,
                                                       const int *, const int *,
                                                       const double *, double, double *, int *);
template int launch_plain_push<float>(int, int, const PlainPushArgs<float> &, cudaStream_t);
template int launch_plain_push<double>(int, int, const PlainPushArgs<double> &, cudaStream_t);

} // namespace osg
