/*
 * pic_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the OSIRIS particle-in-cell time step (push, charge-conserving current
 * deposition, periodic guard fold/replace, Yee field advance, periodic particle wrap, cell
 * sort, seeded particle load, energy and charge diagnostics).  It is the parity checker for
 * the CUDA implementation in osiris_gb300/: only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load it.  The product never links or calls it.
 *
 * The push/deposit part (oracle_push_tmpl.h) is pinned bit for bit against the reference's own
 * AVX2 kernels compiled from source (oracle/Makefile target `ref`, fixtures in tests/golden/).
 * The grid phases (oracle_fields_tmpl.h) restate Fortran code that cannot be compiled here (no
 * Fortran compiler); they are pinned by known-answer tests (periodic plane wave, fold identity,
 * charge conservation) in tests/test_oracle_*.py.
 *
 * Build: see oracle/Makefile (gcc -O2 -ffp-contract=off -fopenmp, portable C99).
 */

#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "pic_oracle.h"

/* double-precision B-spline weights (order 1..4) used by the charge deposit diagnostic */
void ora_spline_weights_f64(int order, double x, double *w)
{
    double a = 0.5 - x, b = 0.5 + x;
    switch (order) {
    case 1:
        w[0] = a; w[1] = b;
        break;
    case 2:
        w[0] = 0.5 * a * a; w[1] = fma(a, b, 0.5); w[2] = 0.5 * b * b;
        break;
    case 3:
        w[0] = a * a * a / 6.0;
        w[1] = fma(0.5, b * b * b, 2.0 / 3.0 - b * b);
        w[2] = fma(0.5, a * a * a, 2.0 / 3.0 - a * a);
        w[3] = b * b * b / 6.0;
        break;
    default: {
        double ab = a * b;
        w[0] = a * a * a * a / 24.0;
        w[1] = fma(a, fma(a, 1.5 + ab, 1.0), 0.25) / 6.0;
        w[2] = fma(ab, fma(0.25, ab, 0.5), 11.0 / 24.0);
        w[3] = fma(b, fma(b, 1.5 + ab, 1.0), 0.25) / 6.0;
        w[4] = b * b * b * b / 24.0;
    } break;
    }
}

/* ---------------------------------------------------------------- single precision ------ */
#define R float
#define SFX f32
#define VW 8
#define K(v) ((float)(v))
#define FMA fmaf
#define SQRT sqrtf
#define SIN sinf
#define COS cosf

#include "oracle_exact_tmpl.h"

#define ORD 1
#define OFS 1
#include "oracle_push_tmpl.h"
#undef ORD
#undef OFS
#define ORD 2
#define OFS 2
#include "oracle_push_tmpl.h"
#undef ORD
#undef OFS
#define ORD 3
#define OFS 2
#include "oracle_push_tmpl.h"
#undef ORD
#undef OFS
#define ORD 4
#define OFS 3
#include "oracle_push_tmpl.h"
#undef ORD
#undef OFS
#include "oracle_fields_tmpl.h"

#undef R
#undef SFX
#undef VW
#undef K
#undef FMA
#undef SQRT
#undef SIN
#undef COS

/* ---------------------------------------------------------------- double precision ------ */
#define R double
#define SFX f64
#define VW 4
#define K(v) ((double)(v))
#define FMA fma
#define SQRT sqrt
#define SIN sin
#define COS cos

#include "oracle_exact_tmpl.h"

#define ORD 1
#define OFS 1
#include "oracle_push_tmpl.h"
#undef ORD
#undef OFS
#define ORD 2
#define OFS 2
#include "oracle_push_tmpl.h"
#undef ORD
#undef OFS
#define ORD 3
#define OFS 2
#include "oracle_push_tmpl.h"
#undef ORD
#undef OFS
#define ORD 4
#define OFS 3
#include "oracle_push_tmpl.h"
#undef ORD
#undef OFS
#include "oracle_fields_tmpl.h"

#undef R
#undef SFX
#undef VW
#undef K
#undef FMA
#undef SQRT
#undef SIN
#undef COS

/* ---------------------------------------------------------------- dispatch -------------- */

typedef void (*push_f32_t)(int *, float *, float *, float *, int *, int *, float *, float *,
                           float *, int *, int *, float *, int *, int *, double *, double *,
                           double *);
typedef void (*push_f64_t)(int *, double *, double *, double *, int *, int *, double *,
                           double *, double *, int *, int *, double *, int *, int *, double *,
                           double *, double *);

static push_f32_t push_table_f32(int dim, int order)
{
    static const push_f32_t t[3][4] = {
        {ora_vadvance_deposit_1d_s1_f32, ora_vadvance_deposit_1d_s2_f32,
         ora_vadvance_deposit_1d_s3_f32, ora_vadvance_deposit_1d_s4_f32},
        {ora_vadvance_deposit_2d_s1_f32, ora_vadvance_deposit_2d_s2_f32,
         ora_vadvance_deposit_2d_s3_f32, ora_vadvance_deposit_2d_s4_f32},
        {ora_vadvance_deposit_3d_s1_f32, ora_vadvance_deposit_3d_s2_f32,
         ora_vadvance_deposit_3d_s3_f32, ora_vadvance_deposit_3d_s4_f32}};
    if (dim < 1 || dim > 3 || order < 1 || order > 4) return 0;
    return t[dim - 1][order - 1];
}

static push_f64_t push_table_f64(int dim, int order)
{
    static const push_f64_t t[3][4] = {
        {ora_vadvance_deposit_1d_s1_f64, ora_vadvance_deposit_1d_s2_f64,
         ora_vadvance_deposit_1d_s3_f64, ora_vadvance_deposit_1d_s4_f64},
        {ora_vadvance_deposit_2d_s1_f64, ora_vadvance_deposit_2d_s2_f64,
         ora_vadvance_deposit_2d_s3_f64, ora_vadvance_deposit_2d_s4_f64},
        {ora_vadvance_deposit_3d_s1_f64, ora_vadvance_deposit_3d_s2_f64,
         ora_vadvance_deposit_3d_s3_f64, ora_vadvance_deposit_3d_s4_f64}};
    if (dim < 1 || dim > 3 || order < 1 || order > 4) return 0;
    return t[dim - 1][order - 1];
}

int ora_push_f32(int dim, int order, int *ix, float *x, float *u, float *q, int i0, int i1,
                 float rqm, float *e, float *b, int *emf_size, int *emf_off, float *j,
                 int *j_size, int *j_off, double *dx, double dt, double *ene)
{
    push_f32_t f = push_table_f32(dim, order);
    if (!f) return -1;
    f(ix, x, u, q, &i0, &i1, &rqm, e, b, emf_size, emf_off, j, j_size, j_off, dx, &dt, ene);
    return 0;
}

int ora_push_f64(int dim, int order, int *ix, double *x, double *u, double *q, int i0, int i1,
                 double rqm, double *e, double *b, int *emf_size, int *emf_off, double *j,
                 int *j_size, int *j_off, double *dx, double dt, double *ene)
{
    push_f64_t f = push_table_f64(dim, order);
    if (!f) return -1;
    f(ix, x, u, q, &i0, &i1, &rqm, e, b, emf_size, emf_off, j, j_size, j_off, dx, &dt, ene);
    return 0;
}

#define ORA_CYL_DISPATCH(SFXN, RT)                                                            \
    int ora_push_cyl_##SFXN(int order, int *ix, RT *x, RT *u, RT *q, int i0, int i1, RT rqm,  \
                            int ilb2, RT *e, RT *b, int *emf_size, int *emf_off, RT *j,       \
                            int *j_size, int *j_off, double *dx, double dt, double *ene)      \
    {                                                                                         \
        switch (order) {                                                                      \
        case 1: ora_vadvance_deposit_2d_cyl_s1_##SFXN(ix, x, u, q, &i0, &i1, &rqm, &ilb2, e, \
                    b, emf_size, emf_off, j, j_size, j_off, dx, &dt, ene); return 0;          \
        case 2: ora_vadvance_deposit_2d_cyl_s2_##SFXN(ix, x, u, q, &i0, &i1, &rqm, &ilb2, e, \
                    b, emf_size, emf_off, j, j_size, j_off, dx, &dt, ene); return 0;          \
        case 3: ora_vadvance_deposit_2d_cyl_s3_##SFXN(ix, x, u, q, &i0, &i1, &rqm, &ilb2, e, \
                    b, emf_size, emf_off, j, j_size, j_off, dx, &dt, ene); return 0;          \
        case 4: ora_vadvance_deposit_2d_cyl_s4_##SFXN(ix, x, u, q, &i0, &i1, &rqm, &ilb2, e, \
                    b, emf_size, emf_off, j, j_size, j_off, dx, &dt, ene); return 0;          \
        }                                                                                     \
        return -1;                                                                            \
    }
ORA_CYL_DISPATCH(f32, float)
ORA_CYL_DISPATCH(f64, double)

/* Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random numbers: as easy as 1, 2, 3",
 * SC11): the counter-based stream the thermal-bath re-emission below draws from. */
static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; r++) {
        const uint64_t m0 = (uint64_t)0xD2511F53u * c[0], m1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(m0 >> 32), lo0 = (uint32_t)m0;
        const uint32_t hi1 = (uint32_t)(m1 >> 32), lo1 = (uint32_t)m1;
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

/* Thermal-bath particle boundary (p_bc_thermal, source/spec/os-spec-boundary.f03:1315-1387,
 * thermal_bath :972-1067 with thermal_type "thermal") on the axes in `mask`, run on the pushed
 * particles 1..np before any wrap: a particle outside [1, nx_d] is moved to the edge cell, takes
 * uth_c times a Gaussian for the two other momentum components and uth_d times the
 * half-Maxwellian sqrt(-2 ln v) into the box for the normal one, then the fluid momentum ufl
 * (added relativistically only when all three components are non-zero, :1048-1063); its offset
 * becomes xpos + u_d / gamma dt/dx_d delta (xpos = -1/2 below, the value just under 1/2
 * above); and -q is deposited from the new position back along -u / gamma dt/dx (rev_current
 * :1392-1440; in 2D the out-of-plane velocity keeps its sign), here as a Boris push of a
 * virtual particle with momentum (-u1, -u2, u3) (2D) or -u (3D) through zero fields.  Axes in
 * order.  The random numbers: one Philox4x32-10 call per re-emission, counter (p, p >> 32,
 * step, d + 4 side code), key (seed, species); two Box-Muller Gaussians, the half-Maxwellian
 * and delta from (r + 1/2) / 2^32 in double.  ttype 1 ("random dir", :1026-1041): |uth| along
 * a random direction, u3 = upar |uth|, the other two on a circle of radius
 * sqrt(1 - upar) |uth| (the reference's expression); ttype 2 ("waterbag", :1016-1024):
 * uth_c (v - 1/2) per component; both with the normal component turned into the box. */
#define THERMAL_BODY(R, SFXN)                                                                 \
    if (!mask || np <= 0) return;                                                            \
    int gsz = 3;                                                                              \
    for (int d = 0; d < dim; d++) gsz *= emf_size[d];                                        \
    R *zero = (R *)calloc((size_t)gsz, sizeof(R));                                            \
    const int saved = ora_pusher_##SFXN;                                                      \
    ora_pusher_##SFXN = 0;                                                                    \
    for (long p = 0; p < np; p++)                                                             \
        for (int d = 0; d < dim; d++) {                                                       \
            if (!((mask >> d) & 1)) continue;                                                 \
            int *c = &ix[dim * p + d];                                                        \
            if (*c >= 1 && *c <= nx[d]) continue;                                             \
            const int lower = *c < 1, code = lower ? 1 : 2;                                   \
            *c = lower ? 1 : nx[d];                                                           \
            uint32_t r[4] = {(uint32_t)p, (uint32_t)((uint64_t)p >> 32), (uint32_t)step,      \
                             (uint32_t)(d + 4 * code)};                                       \
            philox4x32_10(r, seed, (uint32_t)species);                                        \
            const double inv32 = 2.3283064365386963e-10;                                      \
            const double v0 = (r[0] + 0.5) * inv32, v1 = (r[1] + 0.5) * inv32;               \
            const double v2 = (r[2] + 0.5) * inv32, v3 = (r[3] + 0.5) * inv32;               \
            const R usign = lower ? (R)1 : (R)-1;                                             \
            R un[3];                                                                          \
            if (ttype == 1) {                                                                 \
                const R ut = (R)sqrt((R)uth[0] * (R)uth[0] + (R)uth[1] * (R)uth[1] +          \
                                     (R)uth[2] * (R)uth[2]);                                  \
                const R upar = (R)(2.0 * v0 - 1.0);                                           \
                const R uperp = (R)sqrt((R)1 - upar) * ut;                                    \
                const R th = (R)(6.283185307179586 * v1);                                     \
                un[0] = (R)cos(th) * uperp;                                                   \
                un[1] = (R)sin(th) * uperp;                                                   \
                un[2] = upar * ut;                                                            \
                un[d] = usign * (R)fabs(un[d]);                                               \
            } else if (ttype == 2) {                                                          \
                const double w[3] = {v0, v1, v2};                                             \
                for (int cc = 0; cc < 3; cc++) un[cc] = (R)uth[cc] * (R)(w[cc] - 0.5);         \
                un[d] = usign * (R)fabs(un[d]);                                               \
            } else {                                                                          \
                const double rad = sqrt(-2.0 * log(v0)), th = 6.283185307179586 * v1;         \
                const double gs[2] = {rad * cos(th), rad * sin(th)};                          \
                for (int cc = 0, k = 0; cc < 3; cc++)                                         \
                    if (cc != d) un[cc] = (R)uth[cc] * (R)gs[k++];                            \
                un[d] = usign * (R)uth[d] * (R)sqrt(-2.0 * log(v2));                          \
            }                                                                                 \
            const R f1 = (R)ufl[0], f2 = (R)ufl[1], f3 = (R)ufl[2];                           \
            if (f1 != 0 && f2 != 0 && f3 != 0) {                                              \
                const R fa = (R)1 / ((R)1 + (R)sqrt((R)1 + f1 * f1 + f2 * f2 + f3 * f3));     \
                const R gth = (R)sqrt((R)1 + un[0] * un[0] + un[1] * un[1] + un[2] * un[2]);  \
                const R fb = gth + fa * (f1 * un[0] + f2 * un[1] + f3 * un[2]);               \
                un[0] = un[0] + fb * f1;                                                      \
                un[1] = un[1] + fb * f2;                                                      \
                un[2] = un[2] + fb * f3;                                                      \
            }                                                                                 \
            for (int cc = 0; cc < 3; cc++) u[3 * p + cc] = un[cc];                            \
            const R rg = (R)1 / (R)sqrt((R)1 + un[0] * un[0] + un[1] * un[1] + un[2] * un[2]);\
            const R dtdx = (R)(dt / dx[d]);                                                   \
            const R xpos = lower ? (R)-0.5 : (sizeof(R) == 4 ? (R)0.49999997f                 \
                                                             : (R)0.49999999999999994);       \
            x[dim * p + d] = xpos + (rg * un[d] * dtdx) * (R)v3;                              \
            int vix[3];                                                                       \
            R vx[3], vu[3], vq = -q[p];                                                       \
            for (int k = 0; k < dim; k++) {                                                   \
                vix[k] = ix[dim * p + k];                                                     \
                vx[k] = x[dim * p + k];                                                       \
            }                                                                                 \
            vu[0] = -un[0];                                                                   \
            vu[1] = -un[1];                                                                   \
            vu[2] = dim == 3 ? -un[2] : un[2];                                                \
            double ev = 0.0;                                                                  \
            ora_push_##SFXN(dim, order, vix, vx, vu, &vq, 1, 1, rqm, zero, zero, emf_size,    \
                            emf_off, j, emf_size, emf_off, (double *)dx, dt, &ev);            \
        }                                                                                     \
    ora_pusher_##SFXN = saved;                                                                \
    free(zero);

void ora_particle_thermal_f32(int dim, int order, const int *nx, int np, int *ix, float *x,
                              float *u, float *q, float rqm, int *emf_size, int *emf_off,
                              float *j, const double *dx, double dt, int mask,
                              const double *uth, const double *ufl, uint32_t seed, int species,
                              uint64_t step, int ttype)
{
    THERMAL_BODY(float, f32)
}

void ora_particle_thermal_f64(int dim, int order, const int *nx, int np, int *ix, double *x,
                              double *u, double *q, double rqm, int *emf_size, int *emf_off,
                              double *j, const double *dx, double dt, int mask,
                              const double *uth, const double *ufl, uint32_t seed, int species,
                              uint64_t step, int ttype)
{
    THERMAL_BODY(double, f64)
}

/* thermal-bath parameters of the step functions below (mask 0: none) */
static int step_thermal = 0;
static uint32_t step_seed = 0;
static uint64_t step_count = 0;
static int step_ttype = 0;
static double step_uth[3], step_ufl[3];
void ora_set_thermal(int mask, const double *uth, const double *ufl, uint32_t seed,
                     uint64_t step, int ttype)
{
    step_ttype = ttype;
    step_thermal = mask;
    step_seed = seed;
    step_count = step;
    for (int c = 0; c < 3; c++) {
        step_uth[c] = uth ? uth[c] : 0.0;
        step_ufl[c] = ufl ? ufl[c] : 0.0;
    }
}

/* push with another momentum update (pusher 1 exact, 2 Vay, 3 Higuera-Cary, 4 full rotation,
 * 5 Euler rotation; the Fortran advance_deposit path): momentum with the double step dt (and
 * tolerance tol, exact pusher), position and deposit as the push above with dt */
int ora_push_pusher_f32(int pusher, int dim, int order, int *ix, float *x, float *u, float *q,
                        int i0, int i1, float rqm, float *e, float *b, int *emf_size,
                        int *emf_off, float *j, int *j_size, int *j_off, double *dx, double dt,
                        double tol, double *ene)
{
    ora_pusher_f32 = pusher;
    ora_push_dt_f32 = dt;
    ora_iter_tol_f32 = tol;
    int rc = ora_push_f32(dim, order, ix, x, u, q, i0, i1, rqm, e, b, emf_size, emf_off, j,
                          j_size, j_off, dx, dt, ene);
    ora_pusher_f32 = 0;
    return rc;
}

int ora_push_pusher_f64(int pusher, int dim, int order, int *ix, double *x, double *u,
                        double *q, int i0, int i1, double rqm, double *e, double *b,
                        int *emf_size, int *emf_off, double *j, int *j_size, int *j_off,
                        double *dx, double dt, double tol, double *ene)
{
    ora_pusher_f64 = pusher;
    ora_push_dt_f64 = dt;
    ora_iter_tol_f64 = tol;
    int rc = ora_push_f64(dim, order, ix, x, u, q, i0, i1, rqm, e, b, emf_size, emf_off, j,
                          j_size, j_off, dx, dt, ene);
    ora_pusher_f64 = 0;
    return rc;
}

int ora_push_exact_f32(int dim, int order, int *ix, float *x, float *u, float *q, int i0, int i1,
                       float rqm, float *e, float *b, int *emf_size, int *emf_off, float *j,
                       int *j_size, int *j_off, double *dx, double dt, double tol, double *ene)
{
    return ora_push_pusher_f32(1, dim, order, ix, x, u, q, i0, i1, rqm, e, b, emf_size, emf_off,
                               j, j_size, j_off, dx, dt, tol, ene);
}

int ora_push_exact_f64(int dim, int order, int *ix, double *x, double *u, double *q, int i0,
                       int i1, double rqm, double *e, double *b, int *emf_size, int *emf_off,
                       double *j, int *j_size, int *j_off, double *dx, double dt, double tol,
                       double *ene)
{
    return ora_push_pusher_f64(1, dim, order, ix, x, u, q, i0, i1, rqm, e, b, emf_size, emf_off,
                               j, j_size, j_off, dx, dt, tol, ene);
}

/* ---------------------------------------------------------------- particle phases ------- */

/* periodic single-node wrap of cell indices (source/spec/os-spec-boundary.f03:1280-1290) */
void ora_wrap(int dim, const int *nx, int np, int *ix)
{
    for (int p = 0; p < np; p++)
        for (int d = 0; d < dim; d++) {
            int *c = &ix[dim * p + d];
            if (*c < 1) *c += nx[d];
            else if (*c > nx[d]) *c -= nx[d];
        }
}

/* stable counting sort destination of each particle, by cell with x fastest
 * (source/spec/os-species.f03:388-505); new_idx is 0-based */
void ora_sort_index(int dim, const int *nx, int np, const int *ix, int *new_idx)
{
    long ncell = 1;
    for (int d = 0; d < dim; d++) ncell *= nx[d];
    long *cnt = (long *)calloc((size_t)ncell, sizeof(long));
    for (int p = 0; p < np; p++) {
        long c = ix[dim * p] - 1;
        if (dim > 1) c += (long)nx[0] * (ix[dim * p + 1] - 1);
        if (dim > 2) c += (long)nx[0] * nx[1] * (ix[dim * p + 2] - 1);
        new_idx[p] = (int)c;
        cnt[c]++;
    }
    long s = 0;
    for (long c = 0; c < ncell; c++) {
        long t = cnt[c];
        cnt[c] = s;
        s += t;
    }
    for (int p = 0; p < np; p++) new_idx[p] = (int)(cnt[new_idx[p]]++);
    free(cnt);
}

/* ---------------------------------------------------------------- seeded load ----------- */
/*
 * Mersenne Twister as seeded by OSIRIS (source/random/os-random-mt.f03:84-149): the first
 * state word is seed XOR 0x80000000 and the read index starts at N (1-based), so the first
 * draw tempers the last initialisation word before the first regeneration.
 */
void ora_mt_seed(ora_mt *r, int seed)
{
    r->mt[0] = (uint32_t)seed ^ 0x80000000u;
    for (int i = 1; i < 624; i++)
        r->mt[i] = 1812433253u * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t)i;
    r->mti = 623; /* 0-based position of the next word */
    r->have_gauss = 0;
    r->gauss = 0.0;
}

int32_t ora_mt_int32(ora_mt *r)
{
    static const uint32_t mag[2] = {0u, 0x9908b0dfu};
    if (r->mti >= 624) {
        int k;
        uint32_t y;
        for (k = 0; k < 624 - 397; k++) {
            y = (r->mt[k] & 0x80000000u) | (r->mt[k + 1] & 0x7fffffffu);
            r->mt[k] = r->mt[k + 397] ^ (y >> 1) ^ mag[y & 1u];
        }
        for (; k < 623; k++) {
            y = (r->mt[k] & 0x80000000u) | (r->mt[k + 1] & 0x7fffffffu);
            r->mt[k] = r->mt[k + (397 - 624)] ^ (y >> 1) ^ mag[y & 1u];
        }
        y = (r->mt[623] & 0x80000000u) | (r->mt[0] & 0x7fffffffu);
        r->mt[623] = r->mt[396] ^ (y >> 1) ^ mag[y & 1u];
        r->mti = 0;
    }
    uint32_t y = r->mt[r->mti++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return (int32_t)y;
}

/* polar Box-Muller gaussian (source/random/os-random-class.f03:348-392) */
double ora_gaussian(ora_mt *r)
{
    if (r->have_gauss) {
        r->have_gauss = 0;
        return r->gauss;
    }
    double v1, v2, rsq;
    do {
        v1 = ((double)ora_mt_int32(r) + 0.5) * (1.0 / 2147483648.0);
        v2 = ((double)ora_mt_int32(r) + 0.5) * (1.0 / 2147483648.0);
        rsq = v1 * v1 + v2 * v2;
    } while (!(rsq < 1.0 && rsq > 0.0));
    double fac = sqrt(-2.0 * log(rsq) / rsq);
    r->gauss = v1 * fac;
    r->have_gauss = 1;
    return v2 * fac;
}

/*
 * Regular-lattice load of one species over the whole periodic box
 * (source/spec/psource/os-psource-std.f03:759-1120): ppc_d particles per cell along each axis
 * at in-cell offsets (2i-1-n)/(2n); cells visited with x slowest; charge = den * sign(1/ppc,rqm)
 * with den = 1 + amp*cos(2 pi kmode x1_phys / L1) (amp = 0 gives a uniform plasma); momenta
 * uth*gaussian per component followed by the relativistic fluid boost ufl
 * (source/spec/os-spec-udist.f03:452-850, uniform ufl branch).  Returns the particle count.
 */
#define LOAD_BODY(R)                                                                          \
    int ppc = 1;                                                                              \
    for (int d = 0; d < dim; d++) ppc *= ppc_d[d];                                             \
    R pvol = (R)(rqm < 0 ? -1.0 : 1.0) * ((R)1.0 / (R)ppc);                                   \
    double pos[3][64];                                                                        \
    for (int d = 0; d < dim; d++) {                                                            \
        R half = (R)0.5 / (R)ppc_d[d];                                                        \
        for (int i = 1; i <= ppc_d[d]; i++) pos[d][i - 1] = (double)((R)(2 * i - 1 - ppc_d[d]) * half); \
    }                                                                                         \
    int n = 0;                                                                                \
    int c3n = dim > 2 ? nx[2] : 1, c2n = dim > 1 ? nx[1] : 1;                                  \
    int p3n = dim > 2 ? ppc_d[2] : 1, p2n = dim > 1 ? ppc_d[1] : 1;                            \
    double L1 = nx[0] * dx[0];                                                                \
    for (int c1 = 1; c1 <= nx[0]; c1++)                                                       \
        for (int c2 = 1; c2 <= c2n; c2++)                                                     \
            for (int c3 = 1; c3 <= c3n; c3++)                                                 \
                for (int a = 0; a < ppc_d[0]; a++)                                            \
                    for (int bb = 0; bb < p2n; bb++)                                          \
                        for (int cc = 0; cc < p3n; cc++) {                                    \
                            int ci[3] = {c1, c2, c3}, pi[3] = {a, bb, cc};                    \
                            for (int d = 0; d < dim; d++) {                                    \
                                x[dim * n + d] = (R)pos[d][pi[d]];                            \
                                ix[dim * n + d] = ci[d];                                      \
                            }                                                                 \
                            double xp = (c1 - 0.5 + pos[0][a]) * dx[0];                       \
                            R den = (R)(1.0 + amp * cos(2.0 * M_PI * kmode * xp / L1));        \
                            q[n] = den * pvol;                                                \
                            n++;                                                              \
                        }                                                                     \
    R ufa = (R)1.0 / (sqrtf_or_sqrt((R)1 + (R)ufl[0] * (R)ufl[0] + (R)ufl[1] * (R)ufl[1] +    \
                                     (R)ufl[2] * (R)ufl[2]) + (R)1);                           \
    for (int p = 0; p < n; p++) {                                                             \
        u[3 * p + 0] = (R)((R)uth[0] * ora_gaussian(rng));                                    \
        u[3 * p + 1] = (R)((R)uth[1] * ora_gaussian(rng));                                    \
        u[3 * p + 2] = (R)((R)uth[2] * ora_gaussian(rng));                                    \
        R g = sqrtf_or_sqrt((R)1 + u[3 * p] * u[3 * p] + u[3 * p + 1] * u[3 * p + 1] +         \
                            u[3 * p + 2] * u[3 * p + 2]);                                     \
        R bq = ufa * (u[3 * p] * (R)ufl[0] + u[3 * p + 1] * (R)ufl[1] + u[3 * p + 2] * (R)ufl[2]) + g; \
        u[3 * p + 0] = u[3 * p + 0] + bq * (R)ufl[0];                                         \
        u[3 * p + 1] = u[3 * p + 1] + bq * (R)ufl[1];                                         \
        u[3 * p + 2] = u[3 * p + 2] + bq * (R)ufl[2];                                         \
    }                                                                                         \
    return n;

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int ora_load_f32(ora_mt *rng, int dim, const int *nx, const int *ppc_d, const double *dx,
                 double rqm, const double *uth, const double *ufl, double amp, double kmode,
                 int *ix, float *x, float *u, float *q)
{
#define sqrtf_or_sqrt sqrtf
    LOAD_BODY(float)
#undef sqrtf_or_sqrt
}

int ora_load_f64(ora_mt *rng, int dim, const int *nx, const int *ppc_d, const double *dx,
                 double rqm, const double *uth, const double *ufl, double amp, double kmode,
                 int *ix, double *x, double *u, double *q)
{
#define sqrtf_or_sqrt sqrt
    LOAD_BODY(double)
#undef sqrtf_or_sqrt
}

/* ---------------------------------------------------------------- divergence ------------ */
/* div of the staggered E (or J) into div[] (one value per interior point, x fastest)
 * (source/vdf/os-vdf-math.f90:1013-1073, offset 0), in double */
#define DIV_BODY(R)                                                                           \
    int sz0 = nx[0] + gcl[0] + gcu[0];                                                        \
    int sz1 = dim > 1 ? nx[1] + gcl[1] + gcu[1] : 1;                                          \
    int n2 = dim > 1 ? nx[1] : 1, n3 = dim > 2 ? nx[2] : 1;                                   \
    long o = 0;                                                                               \
    for (int i3 = 1; i3 <= n3; i3++)                                                          \
        for (int i2 = 1; i2 <= n2; i2++)                                                      \
            for (int i1 = 1; i1 <= nx[0]; i1++) {                                             \
                long c = (i1 - 1 + gcl[0]);                                                   \
                if (dim > 1) c += (long)sz0 * (i2 - 1 + gcl[1]);                              \
                if (dim > 2) c += (long)sz0 * sz1 * (i3 - 1 + gcl[2]);                        \
                double v = ((double)f[3 * c] - (double)f[3 * (c - 1)]) / dx[0];                \
                if (dim > 1) v += ((double)f[3 * c + 1] - (double)f[3 * (c - sz0) + 1]) / dx[1]; \
                if (dim > 2)                                                                  \
                    v += ((double)f[3 * c + 2] - (double)f[3 * (c - (long)sz0 * sz1) + 2]) / dx[2]; \
                div[o++] = v;                                                                 \
            }

void ora_div_f32(int dim, const int *nx, const int *gcl, const int *gcu, const float *f,
                 const double *dx, double *div)
{
    DIV_BODY(float)
}

void ora_div_f64(int dim, const int *nx, const int *gcl, const int *gcu, const double *f,
                 const double *dx, double *div)
{
    DIV_BODY(double)
}

/* ---------------------------------------------------------------- full step ------------- */
/*
 * One time step in the phase order of iter_sim (source/os-simulation.f03:498-666) for a single
 * periodic node: E/B guard replace -> per species push+deposit (OpenMP particle split with a
 * private current grid per thread and an ordered reduction, source/particles/os-particles.f03:
 * 1416-1443 and source/spec/os-spec-vpush.f03:380-397) -> particle wrap -> optional cell sort ->
 * current guard fold -> Yee.  ene[s] receives the time-centred kinetic energy sum of species s
 * (before the rqm*dV normalisation).
 */
#define STEP_BODY(R, SFXN, PUSHER, TOL)                                                        \
    int gsz = 3;                                                                              \
    for (int d = 0; d < dim; d++) gsz *= nx[d] + gcl[d] + gcu[d];                             \
    int emf_size[3], emf_off[3];                                                              \
    for (int d = 0; d < 3; d++) {                                                             \
        emf_size[d] = d < dim ? nx[d] + gcl[d] + gcu[d] : 1;                                  \
        emf_off[d] = d < dim ? gcl[d] : 0;                                                    \
    }                                                                                         \
    /* the single-precision SIMD push gets dt rounded to p_k_part (dtcycle = real(dt, p_k_part),\
       source/spec/os-spec-vpush.f03:365); the Fortran push used with the other pushers keeps \
       the double dt (dt_dx = real(gdt/dx, p_k_part), source/spec/os-spec-push.f03:1459-1460) */\
    const double dtp = (sizeof(R) == 4 && !(PUSHER)) ? (double)(float)dt : dt;                \
    ora_pusher_##SFXN = (PUSHER);                                                             \
    ora_push_dt_##SFXN = dt;                                                                  \
    ora_iter_tol_##SFXN = (TOL);                                                              \
    const int walls = step_walls_##SFXN;                                                      \
    const int oax = step_open_##SFXN; /* Lindman axis, -1: none */                            \
    const int win = step_window_##SFXN; /* moving window along x1 */                          \
    const int pml = step_pml_##SFXN; /* PML axes (bit mask), 0: none */                      \
    const int skip = walls | (oax >= 0 ? 1 << oax : 0) | (pml & 7) | win;                     \
    if (oax >= 0) {                                                                           \
        ora_open_guards_##SFXN(dim, nx, gcl, gcu, e, b, oax, step_lind_##SFXN);               \
    } else if (pml) {                                                                         \
        ora_pml_guards_##SFXN(dim, nx, gcl, gcu, e, b, pml, step_pml_nb_##SFXN,               \
                              step_pml_st_##SFXN);                                            \
    } else {                                                                                  \
        ora_periodic_skip_##SFXN(dim, nx, gcl, gcu, e, 0, walls | win);                       \
        ora_periodic_skip_##SFXN(dim, nx, gcl, gcu, b, 0, walls | win);                       \
    }                                                                                         \
    memset(j, 0, sizeof(R) * (size_t)gsz);                                                    \
    /* the fields the particles see: E and B, or their smoothed copies */                      \
    R *ep = e, *bp = b;                                                                       \
    if (step_esmooth_ord_##SFXN[0] > 0) {                                                     \
        ep = (R *)malloc(sizeof(R) * (size_t)gsz);                                            \
        bp = (R *)malloc(sizeof(R) * (size_t)gsz);                                            \
        memcpy(ep, e, sizeof(R) * (size_t)gsz);                                               \
        memcpy(bp, b, sizeof(R) * (size_t)gsz);                                               \
        ora_smooth_##SFXN(dim, nx, gcl, gcu, ep, step_esmooth_ord_##SFXN,                     \
                          step_esmooth_coef_##SFXN);                                          \
        ora_smooth_##SFXN(dim, nx, gcl, gcu, bp, step_esmooth_ord_##SFXN,                     \
                          step_esmooth_coef_##SFXN);                                          \
    }                                                                                         \
    int nt = nthreads < 1 ? 1 : nthreads;                                                     \
    R *jt = nt > 1 ? (R *)calloc((size_t)gsz * (nt - 1), sizeof(R)) : 0;                     \
    for (int s = 0; s < nspec; s++) {                                                         \
        double *et = (double *)calloc((size_t)nt, sizeof(double));                            \
        int chunk = (np[s] + nt - 1) / nt;                                                    \
        chunk = ((chunk + 15) / 16) * 16;                                                     \
        _Pragma("omp parallel for num_threads(nt) schedule(static,1)")                        \
        for (int t = 0; t < nt; t++) {                                                        \
            int a = t * chunk + 1, bnd = (t + 1) * chunk < np[s] ? (t + 1) * chunk : np[s];    \
            R *jj = t == 0 ? j : jt + (size_t)gsz * (t - 1);                                  \
            if (bnd >= a)                                                                     \
                ora_push_##SFXN(dim, order, ix[s], x[s], u[s], q[s], a, bnd, rqm[s], ep, bp,  \
                                emf_size, emf_off, jj, emf_size, emf_off, (double *)dx, dtp,  \
                                &et[t]);                                                      \
        }                                                                                     \
        ene[s] = 0.0;                                                                         \
        for (int t = 0; t < nt; t++) ene[s] += et[t];                                         \
        free(et);                                                                             \
        ora_particle_thermal_##SFXN(dim, order, nx, np[s], ix[s], x[s], u[s], q[s], rqm[s],   \
                                    emf_size, emf_off, j, dx, dtp, step_thermal, step_uth,    \
                                    step_ufl, step_seed, s, step_count, step_ttype);          \
        if (oax >= 0)                                                                         \
            ora_particle_absorb_##SFXN(dim, nx, np[s], ix[s], x[s], u[s], q[s], oax);         \
        for (int a = 0; a < dim; a++)                                                         \
            if ((pml >> a) & 1)                                                               \
                ora_particle_absorb_##SFXN(dim, nx, np[s], ix[s], x[s], u[s], q[s], a);       \
        if (win) ora_particle_window_##SFXN(dim, nx, np[s], ix[s], x[s], u[s], q[s]);        \
        ora_particle_bound_##SFXN(dim, nx, np[s], ix[s], x[s], u[s], walls);                  \
    }                                                                                         \
    if (nt > 1) {                                                                             \
        _Pragma("omp parallel for num_threads(nt) schedule(static)")                          \
        for (long i = 0; i < gsz; i++)                                                        \
            for (int t = 1; t < nt; t++) j[i] += jt[(size_t)gsz * (t - 1) + i];                \
        free(jt);                                                                             \
    }                                                                                         \
    if (ep != e) {                                                                            \
        free(ep);                                                                             \
        free(bp);                                                                             \
    }                                                                                         \
    ora_pusher_##SFXN = 0;                                                                    \
    ora_periodic_skip_##SFXN(dim, nx, gcl, gcu, j, 1, skip);                                  \
    if (walls) ora_walls_##SFXN(dim, nx, gcl, gcu, j, 2, walls, order);                       \
    if (step_smooth_ord_##SFXN[0] > 0)                                                       \
        ora_smooth_##SFXN(dim, nx, gcl, gcu, j, step_smooth_ord_##SFXN,                      \
                          step_smooth_coef_##SFXN);                                          \
    if (walls)                                                                                \
        ora_yee_advance_walls_##SFXN(dim, nx, gcl, gcu, e, b, j, dx, dt, walls, order);      \
    else if (oax >= 0)                                                                        \
        ora_yee_advance_open_##SFXN(dim, nx, gcl, gcu, e, b, j, dx, dt, oax,                 \
                                    step_lind_##SFXN);                                        \
    else if (pml)                                                                             \
        ora_yee_advance_pml_##SFXN(dim, nx, gcl, gcu, e, b, j, dx, dt, pml,                  \
                                   step_pml_nb_##SFXN, step_pml_st_##SFXN);                   \
    else                                                                                      \
        ora_yee_advance_##SFXN(dim, nx, gcl, gcu, e, b, j, dx, dt);                           \
    return 0;

int ora_step_f32(int dim, int order, const int *nx, const int *gcl, const int *gcu,
                 const double *dx, double dt, float *e, float *b, float *j, int nspec,
                 const int *np, int **ix, float **x, float **u, float **q, const float *rqm,
                 double *ene, int nthreads)
{
    STEP_BODY(float, f32, 0, 1e-3)
}

int ora_step_f64(int dim, int order, const int *nx, const int *gcl, const int *gcu,
                 const double *dx, double dt, double *e, double *b, double *j, int nspec,
                 const int *np, int **ix, double **x, double **u, double **q,
                 const double *rqm, double *ene, int nthreads)
{
    STEP_BODY(double, f64, 0, 1e-3)
}

/* the same step with another momentum update (pusher 1 exact, 2 Vay, 3 Higuera-Cary, 4 full
 * rotation, 5 Euler rotation) */
int ora_step_pusher_f32(int pusher, int dim, int order, const int *nx, const int *gcl,
                        const int *gcu, const double *dx, double dt, float *e, float *b,
                        float *j, int nspec, const int *np, int **ix, float **x, float **u,
                        float **q, const float *rqm, double *ene, int nthreads, double tol)
{
    STEP_BODY(float, f32, pusher, tol)
}

int ora_step_pusher_f64(int pusher, int dim, int order, const int *nx, const int *gcl,
                        const int *gcu, const double *dx, double dt, double *e, double *b,
                        double *j, int nspec, const int *np, int **ix, double **x, double **u,
                        double **q, const double *rqm, double *ene, int nthreads, double tol)
{
    STEP_BODY(double, f64, pusher, tol)
}

int ora_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
