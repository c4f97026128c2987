/*
 * oracle_push_tmpl.h -- TEST INFRASTRUCTURE ONLY (parity checker, never shipped).
 *
 * Scalar CPU restatement of the OSIRIS single-pass particle advance + charge-conserving
 * current deposition ("vadvance_deposit_{1d,2d,3d}_sN").  Included by pic_oracle.c once per
 * (precision, interpolation order) with these macros set:
 *
 *   R      real type (float | double)
 *   SFX    name suffix token (f32 | f64)
 *   VW     SIMD lane count of the reference build (8 for single, 4 for double)
 *   ORD    interpolation order 1..4, NPT = ORD + 1, OFS = grid offset (1 + ORD/2, 3 for ORD 4)
 *
 * The arithmetic follows, operation by operation, the reference AVX2 kernels so that results
 * can be compared bit for bit:
 *   source/simd/os-spec-push-avx2d.c:98-154   (Boris, double)   os-spec-push-avx2.c:90-146 (single)
 *   source/simd/os-spec-push-avx2d.c:163-168  (1/gamma)
 *   source/simd/os-spec-push-avx2d.c:53-64    (trim)
 *   source/simd/os-spec-push-avx2d.c:263-475  (1D), :481-775 (2D), :1127-1467 (3D)
 *   source/simd/os-spec-push-avx2.c:255-467   (1D), :471-760 (2D), :1141-1480 (3D)
 *   source/simd/splines-avx2.h                (B-spline weights, order 1..4)
 *   source/simd/split-vec.h:46-97 (1D), :105-265 (2D), :266-718 (3D)   (trajectory split)
 *   source/simd/os-spec-current-avx2d.c:17-110 (longitudinal weights)
 *   source/simd/os-spec-current-avx2d.c:189-278 (1D), :476-613 (2D), :854-1013 (3D) (deposit)
 *
 * Ordering that matters for floating point and is reproduced here:
 *   - particles are processed in chunks of the reference cache size (64 / 464 / 160);
 *   - inside a chunk, groups of VW lanes are pushed, the VW "original" virtual particles are
 *     stored followed by the extra split segments in lane order; the chunk's virtual particles
 *     are deposited in that buffer order after the whole chunk is pushed;
 *   - the time-centred energy is accumulated per lane in R and horizontally reduced per chunk
 *     with the reference reduction tree, then added to the double accumulator.
 * Explicit FMA(a,b,c) is used exactly where the reference uses a fused intrinsic; everything
 * else is a separately rounded operation (the file must be compiled with -ffp-contract=off).
 */

#define PASTE3_(a, b, c) a##b##c
#define PASTE3(a, b, c) PASTE3_(a, b, c)
#define PASTE5_(a, b, c, d, e) a##b##c##d##e
#define PASTE5(a, b, c, d, e) PASTE5_(a, b, c, d, e)
#define OFN(name) PASTE5(name, _s, ORD, _, SFX)
#define NPT (ORD + 1)
#ifndef SKIP_VP
/* marks the slot of a padding lane (the reference fills it with a zero-charge dummy) */
#define SKIP_VP (-2147483647 - 1)
#endif

/* ------------------------------------------------------------------------------------------
 * B-spline weights at x (cell-centred offset in [-0.5, 0.5)) and at the half-shifted point
 * (h = 1 when x < 0).  splines-avx2.h restated.
 * ---------------------------------------------------------------------------------------- */
static inline void OFN(spl)(R x, R w[NPT])
{
#if ORD == 1
    w[0] = K(0.5) - x;
    w[1] = K(0.5) + x;
#elif ORD == 2
    R a = K(0.5) - x, b = K(0.5) + x;
    w[0] = (a * a) * K(0.5);
    w[1] = FMA(a, b, K(0.5));
    w[2] = (b * b) * K(0.5);
#elif ORD == 3
    R a = K(0.5) - x, b = K(0.5) + x;
    R a2 = a * a, b2 = b * b;
    R a3 = a * a2, b3 = b * b2;
    w[0] = K(1.0 / 6.0) * a3;
    w[1] = FMA(K(0.5), b3, K(2.0 / 3.0) - b2);
    w[2] = FMA(K(0.5), a3, K(2.0 / 3.0) - a2);
    w[3] = K(1.0 / 6.0) * b3;
#elif ORD == 4
    R a = K(0.5) - x, b = K(0.5) + x;
    R ab = a * b, a2 = a * a, b2 = b * b;
    w[0] = K(1.0 / 24.0) * (a2 * a2);
    w[1] = K(1.0 / 6.0) * FMA(a, FMA(a, K(1.5) + ab, K(1.0)), K(0.25));
    w[2] = FMA(ab, FMA(K(0.25), ab, K(0.5)), K(11.0 / 24.0));
    w[3] = K(1.0 / 6.0) * FMA(b, FMA(b, K(1.5) + ab, K(1.0)), K(0.25));
    w[4] = K(1.0 / 24.0) * (b2 * b2);
#endif
}

static inline void OFN(splh)(R x, R h, R w[NPT])
{
#if ORD == 1
    w[0] = (K(1.0) - h) - x;
    w[1] = h + x;
#elif ORD == 2
    R a = (K(1.0) - h) - x, b = h + x;
    w[0] = (a * a) * K(0.5);
    w[1] = FMA(a, b, K(0.5));
    w[2] = (b * b) * K(0.5);
#elif ORD == 3
    R a = (K(1.0) - h) - x, b = h + x;
    R a2 = a * a, b2 = b * b;
    R a3 = a * a2, b3 = b * b2;
    w[0] = K(1.0 / 6.0) * a3;
    w[1] = FMA(K(0.5), b3, K(2.0 / 3.0) - b2);
    w[2] = FMA(K(0.5), a3, K(2.0 / 3.0) - a2);
    w[3] = K(1.0 / 6.0) * b3;
#elif ORD == 4
    R a = (K(1.0) - h) - x, b = h + x;
    R ab = a * b, a2 = a * a, b2 = b * b;
    w[0] = K(1.0 / 24.0) * (a2 * a2);
    w[1] = K(1.0 / 6.0) * FMA(a, FMA(a, K(1.5) + ab, K(1.0)), K(0.25));
    w[2] = FMA(ab, FMA(K(0.25), ab, K(0.5)), K(11.0 / 24.0));
    w[3] = K(1.0 / 6.0) * FMA(b, FMA(b, K(1.5) + ab, K(1.0)), K(0.25));
    w[4] = K(1.0 / 24.0) * (b2 * b2);
#endif
}

/* Longitudinal (along-motion) charge-conserving weights, ORD values.
 * os-spec-current-avx2d.c:17-110 restated. */
static inline void OFN(wl)(R qn, R x0, R x1, R w[ORD])
{
#if ORD == 1
    w[0] = qn * (x1 - x0);
#elif ORD == 2
    R d = x1 - x0, s = K(0.5) - x0, p = K(0.5) + x0;
    R n = qn * d;
    w[0] = n * FMA(-K(0.5), d, s);
    w[1] = n * FMA(K(0.5), d, p);
#elif ORD == 3
    R d = x1 - x0, s = K(0.5) - x0, p = K(0.5) + x0;
    R d3 = K(1.0 / 3.0) * d;
    R a0 = K(0.5) * FMA(s, s, -(d * (s - d3)));
    R a1 = FMA(-d, x0 + d3, FMA(-x0, x0, K(0.75)));
    R a2 = K(0.5) * FMA(p, p, d * (p + d3));
    R n = qn * d;
    w[0] = n * a0;
    w[1] = n * a1;
    w[2] = n * a2;
#elif ORD == 4
    R d = x1 - x0, s = K(0.5) - x0, p = K(0.5) + x0;
    R t = x0 - K(1.0 / 6.0), u = x0 + K(1.0 / 6.0);
    R s2 = s * s, s3 = s2 * s, p2 = p * p, p3 = p2 * p;
    R d2 = d * K(0.5), d4 = d * K(0.25);
    R a0 = K(1.0 / 6.0) * FMA(d, FMA(d, s - d4, -(K(1.5) * s2)), s3);
    R a1 = FMA(d, FMA(d2, t + d4, FMA(K(0.75), t * t, -K(1.0 / 3.0))),
               FMA(K(0.5), p3, K(2.0 / 3.0) - p2));
    R a2 = FMA(-d, FMA(d2, u + d4, FMA(K(0.75), u * u, -K(1.0 / 3.0))),
               FMA(K(0.5), s3, K(2.0 / 3.0) - s2));
    R a3 = K(1.0 / 6.0) * FMA(d, FMA(d, p + d4, K(1.5) * p2), p3);
    R n = qn * d;
    w[0] = n * a0;
    w[1] = n * a1;
    w[2] = n * a2;
    w[3] = n * a3;
#endif
}

/* Boris momentum update with time-centred energy; VDUDT_BORIS restated.
 * e[] and b[] are the interpolated fields, tem = dt/(2 rqm). */
static inline void OFN(boris)(R tem, R e1, R e2, R e3, R b1, R b2, R b3,
                              R *u1, R *u2, R *u3, R *ene)
{
    e1 = e1 * tem;
    e2 = e2 * tem;
    e3 = e3 * tem;
    R ut1 = *u1 + e1, ut2 = *u2 + e2, ut3 = *u3 + e3;
    R utsq = FMA(ut3, ut3, FMA(ut2, ut2, ut1 * ut1));
    R gam = SQRT(utsq + K(1.0));
    *ene = utsq / (gam + K(1.0));
    R tg = tem / gam;
    b1 = b1 * tg;
    b2 = b2 * tg;
    b3 = b3 * tg;
    R v1 = FMA(b3, ut2, ut1), v2 = FMA(b1, ut3, ut2), v3 = FMA(b2, ut1, ut3);
    v1 = FMA(-b2, ut3, v1);
    v2 = FMA(-b3, ut1, v2);
    v3 = FMA(-b1, ut2, v3);
    R ot = FMA(b1, b1, K(1.0));
    ot = FMA(b2, b2, ot);
    ot = FMA(b3, b3, ot);
    ot = K(2.0) / ot;
    b1 = b1 * ot;
    b2 = b2 * ot;
    b3 = b3 * ot;
    ut1 = FMA(b3, v2, ut1);
    ut2 = FMA(b1, v3, ut2);
    ut3 = FMA(b2, v1, ut3);
    ut1 = FMA(-b2, v3, ut1);
    ut2 = FMA(-b3, v1, ut2);
    ut3 = FMA(-b1, v2, ut3);
    *u1 = ut1 + e1;
    *u2 = ut2 + e2;
    *u3 = ut3 + e3;
}

/* Momentum update selected for this call: Boris (time-centred energy factor u^2/(gamma+1) in
 * *en), or the exact pusher (oracle_exact_tmpl.h) with the fields scaled by q/m as dudt_exact
 * does (source/spec/os-spec-extpush.f03:76-86): *en = 0 and q (gamma - 1) of the new momentum
 * (:335-344) is added to the double accumulator *eacc. */
static inline void OFN(dudt)(R tem, R rqm, R e1, R e2, R e3, R b1, R b2, R b3,
                             R *u1, R *u2, R *u3, R *en, R qp, double *eacc)
{
    if (!EXN(ora_pusher)) {
        OFN(boris)(tem, e1, e2, e3, b1, b2, b3, u1, u2, u3, en);
        return;
    }
    if (EXN(ora_pusher) >= 2) {
        /* Vay / Higuera-Cary / full and Euler rotation / conditional Vay: their own tem from
         * the double dt,
         * energy straight to *eacc */
        const double dt = EXN(ora_push_dt);
        const R e[3] = {e1, e2, e3}, b[3] = {b1, b2, b3};
        R uu[3] = {*u1, *u2, *u3};
        if (EXN(ora_pusher) == 2)
            *eacc += (double)EXN(ora_vay_u)((R)(0.5 * dt / (double)rqm), e, b, uu, qp);
        else if (EXN(ora_pusher) == 3)
            *eacc += EXN(ora_hc_u)((R)(0.5 * (dt / (double)rqm)), e, b, uu, qp);
        else if (EXN(ora_pusher) == 4)
            *eacc += EXN(ora_fullrot_u)((R)(0.5 * (dt / (double)rqm)), e, b, uu, qp);
        else if (EXN(ora_pusher) == 6)
            *eacc += EXN(ora_cond_vay_u)((R)(0.5 * dt / (double)rqm), e, b, uu, qp);
        else
            *eacc += EXN(ora_euler_u)((R)(0.5 * (dt / (double)rqm)), rqm, dt, e, b, uu, qp);
        *u1 = uu[0]; *u2 = uu[1]; *u3 = uu[2];
        *en = K(0.0);
        return;
    }
    const R qm = K(1.0) / rqm;
    R ep[3], bp[3], uu[3];
    ep[0] = e1 * qm; ep[1] = e2 * qm; ep[2] = e3 * qm;
    bp[0] = b1 * qm; bp[1] = b2 * qm; bp[2] = b3 * qm;
    uu[0] = *u1; uu[1] = *u2; uu[2] = *u3;
    EXN(ora_exact_u)(ep, bp, uu, EXN(ora_push_dt), EXN(ora_iter_tol));
    *u1 = uu[0]; *u2 = uu[1]; *u3 = uu[2];
    const R g = SQRT(((K(1.0) + uu[0] * uu[0]) + uu[1] * uu[1]) + uu[2] * uu[2]);
    *eacc += (double)(qp * (g - K(1.0)));
    *en = K(0.0);
}

static inline R OFN(rgamma)(R u1, R u2, R u3)
{
    return K(1.0) / SQRT(FMA(u3, u3, FMA(u2, u2, FMA(u1, u1, K(1.0)))));
}

/* trim: +1 when x >= 0.5, -1 when x < -0.5, else 0 */
static inline R OFN(trim)(R x)
{
    return (x >= K(0.5) ? K(1.0) : K(0.0)) - (x < K(-0.5) ? K(1.0) : K(0.0));
}

/* horizontal reduction of the per-lane energy accumulators in the reference's tree order
 * (vector-avx2.h:80-98) */
static inline R OFN(lane_reduce)(const R *a)
{
#if VW == 4
    return (a[0] + a[1]) + (a[2] + a[3]);
#else
    return ((a[4] + a[0]) + (a[5] + a[1])) + ((a[6] + a[2]) + (a[7] + a[3]));
#endif
}

/* ========================================================================================
 * 1D
 * ====================================================================================== */

typedef struct { R x0, x1, q, vy, vz; int i; } OFN(vp1);

static void OFN(dep1d)(R *j, const int *j_off, R jn, const OFN(vp1) *vp, int nvp)
{
    R *pj = j + (j_off[0] - OFS) * 3;
    for (int n = 0; n < nvp; n++) {
        if (vp[n].i == SKIP_VP) continue;
        R s0[NPT], s1[NPT], wl[ORD];
        OFN(spl)(vp[n].x0, s0);
        OFN(spl)(vp[n].x1, s1);
        R qnx = vp[n].q * jn, qvy = vp[n].q * vp[n].vy, qvz = vp[n].q * vp[n].vz;
        OFN(wl)(qnx, vp[n].x0, vp[n].x1, wl);
        R *p0 = pj + 3 * vp[n].i;
        for (int k = 0; k < ORD; k++) p0[3 * k] += wl[k];
        for (int k = 0; k < NPT; k++) {
            R wp = K(0.5) * (s0[k] + s1[k]);
            p0[3 * k + 1] += qvy * wp;
            p0[3 * k + 2] += qvz * wp;
        }
    }
}

void OFN(ora_vadvance_deposit_1d)(int *ix, R *x, R *u, R *q, int *i0, int *i1, R *rqm,
                                  R *e, R *b, int *emf_size, int *emf_off,
                                  R *j, int *j_size, int *j_off,
                                  double *dx, double *dt, double *ene)
{
    (void)emf_size; (void)j_size;
    const R tem = (R)(0.5 * (*dt) / (*rqm));
    const R dtdx1 = (R)((*dt) / dx[0]);
    const R jn = (R)(dx[0] / (*dt));
    const R *e0 = e + (emf_off[0] - OFS) * 3;
    const R *b0 = b + (emf_off[0] - OFS) * 3;
    const int first = *i0 - 1, np = *i1 - *i0 + 1;
    const int cache = 64;
    OFN(vp1) *buf = (OFN(vp1) *)malloc(sizeof(OFN(vp1)) * 2 * cache);

    for (int c0 = 0; c0 < np; c0 += cache) {
        int cn = np - c0 < cache ? np - c0 : cache;
        R acc[VW];
        double eacc = 0.0;
        for (int l = 0; l < VW; l++) acc[l] = K(0.0);
        int nvp = 0;
        for (int g = 0; g < cn; g += VW) {
            int gn = cn - g < VW ? cn - g : VW;
            int base = nvp, extra = base + VW;
            int dix[VW];
            for (int l = 0; l < gn; l++) {
                int p = first + c0 + g + l;
                R x0 = x[p];
                int i = ix[p];
                R wx[NPT], wxh[NPT];
                OFN(spl)(x0, wx);
                R h = x0 < K(0.0) ? K(1.0) : K(0.0);
                int ih = i - (x0 < K(0.0) ? 1 : 0);
                OFN(splh)(x0, h, wxh);
                R E1 = K(0.0), E2 = K(0.0), E3 = K(0.0), B1 = K(0.0), B2 = K(0.0), B3 = K(0.0);
                for (int k = 0; k < NPT; k++) {
                    E1 = FMA(e0[3 * (ih + k) + 0], wxh[k], E1);
                    E2 = FMA(e0[3 * (i + k) + 1], wx[k], E2);
                    E3 = FMA(e0[3 * (i + k) + 2], wx[k], E3);
                }
                for (int k = 0; k < NPT; k++) {
                    B1 = FMA(b0[3 * (i + k) + 0], wx[k], B1);
                    B2 = FMA(b0[3 * (ih + k) + 1], wxh[k], B2);
                    B3 = FMA(b0[3 * (ih + k) + 2], wxh[k], B3);
                }
                R u1 = u[3 * p], u2 = u[3 * p + 1], u3 = u[3 * p + 2], en;
                OFN(dudt)(tem, *rqm, E1, E2, E3, B1, B2, B3, &u1, &u2, &u3, &en, q[p], &eacc);
                u[3 * p] = u1; u[3 * p + 1] = u2; u[3 * p + 2] = u3;
                R rg = OFN(rgamma)(u1, u2, u3);
                acc[l] = FMA(q[p], en, acc[l]);
                R v1 = u1 * rg, v2 = u2 * rg, v3 = u3 * rg;
                R x1 = FMA(v1, dtdx1, x0);
                buf[base + l].x0 = x0; buf[base + l].x1 = x1; buf[base + l].q = q[p];
                buf[base + l].vy = v2; buf[base + l].vz = v3; buf[base + l].i = i;
                R tr = OFN(trim)(x1);
                x[p] = x1 - tr;
                dix[l] = (int)tr;
                ix[p] = i + dix[l];
            }
            for (int l = gn; l < VW; l++) buf[base + l].i = SKIP_VP;
            /* split (split-vec.h:46-97) */
            for (int l = 0; l < gn; l++) {
                if (!dix[l]) continue;
                OFN(vp1) *v = &buf[base + l];
                R xint = (R)(0.5 * dix[l]);
                R delta = (xint - v->x0) / (v->x1 - v->x0);
                OFN(vp1) *w = &buf[extra++];
                w->x0 = -xint; w->x1 = v->x1 - dix[l]; w->i = v->i + dix[l]; w->q = v->q;
                w->vy = v->vy * (1 - delta); w->vz = v->vz * (1 - delta);
                v->x1 = xint; v->vy *= delta; v->vz *= delta;
            }
            nvp = extra;
        }
        OFN(dep1d)(j, j_off, jn, buf, nvp);
        *ene += (double)OFN(lane_reduce)(acc);
        *ene += eacc;
    }
    free(buf);
}

/* ========================================================================================
 * 2D
 * ====================================================================================== */

typedef struct { R x0, x1, y0, y1, q, vz; int i, j; } OFN(vp2);

static void OFN(dep2d)(R *jf, const int *j_size, const int *j_off, const R *jn,
                        const OFN(vp2) *vp, int nvp)
{
    const int Dy = 3 * j_size[0];
    R *pj = jf + (j_off[0] - OFS) * 3 + (j_off[1] - OFS) * Dy;
    for (int n = 0; n < nvp; n++) {
        const OFN(vp2) *v = &vp[n];
        if (v->i == SKIP_VP) continue;
        R s0x[NPT], s1x[NPT], s0y[NPT], s1y[NPT], wl1[ORD], wl2[ORD], wp1[NPT], wp2[NPT];
        OFN(spl)(v->x0, s0x);
        OFN(spl)(v->x1, s1x);
        OFN(spl)(v->y0, s0y);
        OFN(spl)(v->y1, s1y);
        R qnx = v->q * jn[0], qny = v->q * jn[1];
        R qvz = (v->q * v->vz) * K(1.0 / 3.0);
        OFN(wl)(qnx, v->x0, v->x1, wl1);
        OFN(wl)(qny, v->y0, v->y1, wl2);
        for (int k = 0; k < NPT; k++) {
            wp1[k] = s0y[k] + s1y[k];
            wp2[k] = s0x[k] + s1x[k];
        }
        R *p = pj + 3 * v->i + Dy * v->j;
        for (int k2 = 0; k2 < NPT; k2++)
            for (int k1 = 0; k1 < ORD; k1++) p[3 * k1 + Dy * k2 + 0] += wl1[k1] * wp1[k2];
        for (int k2 = 0; k2 < ORD; k2++)
            for (int k1 = 0; k1 < NPT; k1++) p[3 * k1 + Dy * k2 + 1] += wl2[k2] * wp2[k1];
        for (int k2 = 0; k2 < NPT; k2++)
            for (int k1 = 0; k1 < NPT; k1++) {
                R t1 = FMA(s1y[k2], s1x[k1], s0x[k1] * s0y[k2]);
                R t2 = FMA(s0y[k2], s1x[k1], s0x[k1] * s1y[k2]);
                t1 = FMA(t2, K(0.5), t1);
                p[3 * k1 + Dy * k2 + 2] += qvz * t1;
            }
    }
}

/* split-vec.h:105-265 restated; appends extra segments at buf[*extra] */
static void OFN(split2d)(OFN(vp2) *buf, int base, int gn, const int *dix, const int *diy,
                          int *extra)
{
    int ne = *extra;
    for (int l = 0; l < gn; l++) {
        OFN(vp2) *v = &buf[base + l];
        int cross = (dix[l] != 0 ? 1 : 0) | (diy[l] != 0 ? 2 : 0);
        if (cross == 0) continue;
        if (cross == 1) {
            R xint = (R)(0.5 * dix[l]);
            R delta = (xint - v->x0) / (v->x1 - v->x0);
            R yint = v->y0 + (v->y1 - v->y0) * delta;
            OFN(vp2) *w = &buf[ne++];
            w->x0 = -xint; w->x1 = v->x1 - dix[l];
            w->y0 = yint; w->y1 = v->y1;
            w->i = v->i + dix[l]; w->j = v->j; w->q = v->q;
            w->vz = v->vz * (1 - delta);
            v->x1 = xint; v->y1 = yint; v->vz *= delta;
        } else if (cross == 2) {
            R yint = (R)(0.5 * diy[l]);
            R delta = (yint - v->y0) / (v->y1 - v->y0);
            R xint = v->x0 + (v->x1 - v->x0) * delta;
            OFN(vp2) *w = &buf[ne++];
            w->x0 = xint; w->x1 = v->x1;
            w->y0 = -yint; w->y1 = v->y1 - diy[l];
            w->i = v->i; w->j = v->j + diy[l]; w->q = v->q;
            w->vz = v->vz * (1 - delta);
            v->x1 = xint; v->y1 = yint; v->vz *= delta;
        } else {
            R xint = (R)(0.5 * dix[l]);
            R delta = (xint - v->x0) / (v->x1 - v->x0);
            R yint = v->y0 + (v->y1 - v->y0) * delta;
            if (yint >= -0.5 && yint < 0.5) {
                R vzint = v->vz * delta;
                R vzint2 = v->vz * (1 - delta);
                R yint2 = (R)(0.5 * diy[l]);
                delta = (yint2 - yint) / (v->y1 - yint);
                R xint2 = -xint + (v->x1 - xint) * delta;
                OFN(vp2) *w = &buf[ne++];
                w->x0 = -xint; w->x1 = xint2; w->y0 = yint; w->y1 = yint2;
                w->i = v->i + dix[l]; w->j = v->j; w->q = v->q; w->vz = vzint2 * delta;
                w = &buf[ne++];
                w->x0 = xint2; w->x1 = v->x1 - dix[l]; w->y0 = -yint2; w->y1 = v->y1 - diy[l];
                w->i = v->i + dix[l]; w->j = v->j + diy[l]; w->q = v->q;
                w->vz = vzint2 * (1 - delta);
                v->x1 = xint; v->y1 = yint; v->vz = vzint;
            } else {
                R vzint = v->vz * delta;
                R yint2 = (R)(0.5 * diy[l]);
                delta = (yint2 - v->y0) / (yint - v->y0);
                R xint2 = v->x0 + (xint - v->x0) * delta;
                OFN(vp2) *w = &buf[ne++];
                w->x0 = xint2; w->x1 = xint; w->y0 = -yint2; w->y1 = yint - diy[l];
                w->i = v->i; w->j = v->j + diy[l]; w->q = v->q; w->vz = vzint * (1 - delta);
                w = &buf[ne++];
                w->x0 = -xint; w->x1 = v->x1 - dix[l]; w->y0 = yint - diy[l];
                w->y1 = v->y1 - diy[l];
                w->i = v->i + dix[l]; w->j = v->j + diy[l]; w->q = v->q; w->vz = v->vz - vzint;
                v->x1 = xint2; v->y1 = yint2; v->vz = vzint * delta;
            }
        }
    }
    *extra = ne;
}

/* cyl = 1: the 2D cylindrical variant (x1 = z, x2 = r; vadvance_deposit_2d_cyl_sK,
 * source/simd/os-spec-push-avx2d.c:777-1107, single precision os-spec-push-avx2.c:762-1092):
 * the radial move and the angular-momentum correction of p_r, p_theta in double, from the
 * global radial position of the particle (ilb2 = the node's lower global cell along x2) */
static void OFN(push2d)(int *ix, R *x, R *u, R *q, int *i0, int *i1, R *rqm,
                        R *e, R *b, int *emf_size, int *emf_off,
                        R *j, int *j_size, int *j_off,
                        double *dx, double *dt, double *ene, int cyl, int ilb2)
{
    const R tem = (R)(0.5 * (*dt) / (*rqm));
    const R dtdx1 = (R)((*dt) / dx[0]), dtdx2 = (R)((*dt) / dx[1]);
    R jn[2];
    jn[0] = (R)(dx[0] / (*dt) / 2);
    jn[1] = (R)(dx[1] / (*dt) / 2);
    const int Dy = 3 * emf_size[0];
    const R *e0 = e + (emf_off[0] - OFS) * 3 + (emf_off[1] - OFS) * Dy;
    const R *b0 = b + (emf_off[0] - OFS) * 3 + (emf_off[1] - OFS) * Dy;
    const int first = *i0 - 1, np = *i1 - *i0 + 1;
    const int cache = 464;
    OFN(vp2) *buf = (OFN(vp2) *)malloc(sizeof(OFN(vp2)) * 3 * cache);

    for (int c0 = 0; c0 < np; c0 += cache) {
        int cn = np - c0 < cache ? np - c0 : cache;
        R acc[VW];
        double eacc = 0.0;
        for (int l = 0; l < VW; l++) acc[l] = K(0.0);
        int nvp = 0;
        for (int g = 0; g < cn; g += VW) {
            int gn = cn - g < VW ? cn - g : VW;
            int base = nvp, extra = base + VW;
            int dix[VW], diy[VW];
            for (int l = 0; l < gn; l++) {
                int p = first + c0 + g + l;
                R x0 = x[2 * p], y0 = x[2 * p + 1];
                int i = ix[2 * p], jj = ix[2 * p + 1];
                R wx[NPT], wy[NPT], wxh[NPT], wyh[NPT];
                OFN(spl)(x0, wx);
                OFN(spl)(y0, wy);
                R hx = x0 < K(0.0) ? K(1.0) : K(0.0), hy = y0 < K(0.0) ? K(1.0) : K(0.0);
                int ih = i - (x0 < K(0.0) ? 1 : 0), jh = jj - (y0 < K(0.0) ? 1 : 0);
                OFN(splh)(x0, hx, wxh);
                OFN(splh)(y0, hy, wyh);
                /* staggered gather: E1 (ih,j) E2 (i,jh) E3 (i,j) B1 (i,jh) B2 (ih,j) B3 (ih,jh) */
                R E1 = K(0.0), E2 = K(0.0), E3 = K(0.0);
                for (int k2 = 0; k2 < NPT; k2++) {
                    R f1 = K(0.0), f2 = K(0.0), f3 = K(0.0);
                    for (int k1 = 0; k1 < NPT; k1++) {
                        f1 = FMA(e0[3 * (ih + k1) + Dy * (jj + k2) + 0], wxh[k1], f1);
                        f2 = FMA(e0[3 * (i + k1) + Dy * (jh + k2) + 1], wx[k1], f2);
                        f3 = FMA(e0[3 * (i + k1) + Dy * (jj + k2) + 2], wx[k1], f3);
                    }
                    E1 = FMA(f1, wy[k2], E1);
                    E2 = FMA(f2, wyh[k2], E2);
                    E3 = FMA(f3, wy[k2], E3);
                }
                R B1 = K(0.0), B2 = K(0.0), B3 = K(0.0);
                for (int k2 = 0; k2 < NPT; k2++) {
                    R f1 = K(0.0), f2 = K(0.0), f3 = K(0.0);
                    for (int k1 = 0; k1 < NPT; k1++) {
                        f1 = FMA(b0[3 * (i + k1) + Dy * (jh + k2) + 0], wx[k1], f1);
                        f2 = FMA(b0[3 * (ih + k1) + Dy * (jj + k2) + 1], wxh[k1], f2);
                        f3 = FMA(b0[3 * (ih + k1) + Dy * (jh + k2) + 2], wxh[k1], f3);
                    }
                    B1 = FMA(f1, wyh[k2], B1);
                    B2 = FMA(f2, wy[k2], B2);
                    B3 = FMA(f3, wyh[k2], B3);
                }
                R u1 = u[3 * p], u2 = u[3 * p + 1], u3 = u[3 * p + 2], en;
                OFN(dudt)(tem, *rqm, E1, E2, E3, B1, B2, B3, &u1, &u2, &u3, &en, q[p], &eacc);
                u[3 * p] = u1; u[3 * p + 1] = u2; u[3 * p + 2] = u3;
                R rg = OFN(rgamma)(u1, u2, u3);
                acc[l] = FMA(q[p], en, acc[l]);
                R v1 = u1 * rg, v2 = u2 * rg, v3 = u3 * rg;
                R x1 = FMA(v1, dtdx1, x0), y1;
                if (cyl) {
                    /* :1034-1065: gix2 = iy0 + gshift2 (global cell), r_old = (y0 + gix2) dr,
                     * x2_new = r_old + v2 dt, x3_new = v3 dt, r_new = |(x2_new, x3_new)|,
                     * y1 = r_new / dr - gix2 (y0 if r_new == r_old); p_r, p_theta rotated
                     * onto the new radial direction, p_theta scaled by r_old / r_new */
                    const double gshift2 = (ORD == 1 || ORD == 3) ? (double)(ilb2 - 2)
                                                                  : (double)(ilb2 - 2) - 0.5;
                    const double gix2 = (double)jj + gshift2;
                    const double r_old = ((double)y0 + gix2) * dx[1];
                    const double x2n = fma((double)v2, *dt, r_old);
                    const double x3n = (double)v3 * (*dt);
                    const double r_new = sqrt(fma(x2n, x2n, x3n * x3n));
                    const double y1d = (r_old == r_new) ? (double)y0
                                                        : fma(r_new, 1.0 / dx[1], -gix2);
                    y1 = (R)y1d;
                    const double tmp = 1.0 / r_new;
                    const double u2n = fma((double)u2, x2n, (double)u3 * x3n) * tmp;
                    const double u3n = (double)u3 * (r_old * tmp);
                    u[3 * p + 1] = (R)u2n;
                    u[3 * p + 2] = (R)u3n;
                } else {
                    y1 = FMA(v2, dtdx2, y0);
                }
                OFN(vp2) *v = &buf[base + l];
                v->x0 = x0; v->x1 = x1; v->y0 = y0; v->y1 = y1; v->q = q[p]; v->vz = v3;
                v->i = i; v->j = jj;
                R trx = OFN(trim)(x1), try_ = OFN(trim)(y1);
                x[2 * p] = x1 - trx;
                x[2 * p + 1] = y1 - try_;
                dix[l] = (int)trx;
                diy[l] = (int)try_;
                ix[2 * p] = i + dix[l];
                ix[2 * p + 1] = jj + diy[l];
            }
            for (int l = gn; l < VW; l++) buf[base + l].i = SKIP_VP;
            OFN(split2d)(buf, base, gn, dix, diy, &extra);
            nvp = extra;
        }
        OFN(dep2d)(j, j_size, j_off, jn, buf, nvp);
        *ene += (double)OFN(lane_reduce)(acc);
        *ene += eacc;
    }
    free(buf);
}

void OFN(ora_vadvance_deposit_2d)(int *ix, R *x, R *u, R *q, int *i0, int *i1, R *rqm,
                                  R *e, R *b, int *emf_size, int *emf_off,
                                  R *j, int *j_size, int *j_off,
                                  double *dx, double *dt, double *ene)
{
    OFN(push2d)(ix, x, u, q, i0, i1, rqm, e, b, emf_size, emf_off, j, j_size, j_off, dx, dt,
                ene, 0, 0);
}

void OFN(ora_vadvance_deposit_2d_cyl)(int *ix, R *x, R *u, R *q, int *i0, int *i1, R *rqm,
                                      int *ilb2, R *e, R *b, int *emf_size, int *emf_off,
                                      R *j, int *j_size, int *j_off,
                                      double *dx, double *dt, double *ene)
{
    OFN(push2d)(ix, x, u, q, i0, i1, rqm, e, b, emf_size, emf_off, j, j_size, j_off, dx, dt,
                ene, 1, *ilb2);
}

/* ========================================================================================
 * 3D
 * ====================================================================================== */

typedef struct { R x0, x1, y0, y1, z0, z1, q; int i, j, k; } OFN(vp3);

/*
 * 3D deposit.  Per grid element the contributions are added in the order the reference adds
 * them: the double-precision kernel walks the virtual particles one by one
 * (os-spec-current-avx2d.c:854-1013); the single-precision kernel (os-spec-current-avx2.c:
 * 1147-1322) takes VW virtual particles at a time and, inside that group, adds one z plane of
 * the stencil for every particle before moving to the next plane.  The single-precision
 * reference additionally offsets the plane by k3*Dy instead of k3*Dz for orders 3 and 4
 * (os-spec-current-avx2.c:1096, :1118); that is a defect of the reference and is NOT
 * reproduced: this restatement always deposits plane k3 at z offset k3.
 */
static void OFN(dep3d_one)(R *pj, int Dy, int Dz, const R *jn, const OFN(vp3) *v, int plane)
{
    if (v->i == SKIP_VP) return;
    {
        R s0x[NPT], s1x[NPT], s0y[NPT], s1y[NPT], s0z[NPT], s1z[NPT];
        R wl1[ORD], wl2[ORD], wl3[ORD];
        R wp1[NPT][NPT], wp2[NPT][NPT], wp3[NPT][NPT];
        OFN(spl)(v->x0, s0x); OFN(spl)(v->x1, s1x);
        OFN(spl)(v->y0, s0y); OFN(spl)(v->y1, s1y);
        OFN(spl)(v->z0, s0z); OFN(spl)(v->z1, s1z);
        OFN(wl)(v->q * jn[0], v->x0, v->x1, wl1);
        OFN(wl)(v->q * jn[1], v->y0, v->y1, wl2);
        OFN(wl)(v->q * jn[2], v->z0, v->z1, wl3);
        for (int b = 0; b < NPT; b++)
            for (int a = 0; a < NPT; a++) {
                R t1, t2;
                t1 = s0y[a] * s0z[b]; t2 = s0y[a] * s1z[b];
                t1 = FMA(s1y[a], s1z[b], t1); t2 = FMA(s1y[a], s0z[b], t2);
                wp1[b][a] = FMA(K(0.5), t2, t1);
                t1 = s0x[a] * s0z[b]; t2 = s0x[a] * s1z[b];
                t1 = FMA(s1x[a], s1z[b], t1); t2 = FMA(s1x[a], s0z[b], t2);
                wp2[b][a] = FMA(K(0.5), t2, t1);
                t1 = s0x[a] * s0y[b]; t2 = s0x[a] * s1y[b];
                t1 = FMA(s1x[a], s1y[b], t1); t2 = FMA(s1x[a], s0y[b], t2);
                wp3[b][a] = FMA(K(0.5), t2, t1);
            }
        R *p = pj + 3 * v->i + Dy * v->j + Dz * v->k;
        int lo = plane < 0 ? 0 : plane, hi = plane < 0 ? NPT : plane + 1;
        for (int k3 = lo; k3 < hi; k3++)
            for (int k2 = 0; k2 < NPT; k2++)
                for (int k1 = 0; k1 < ORD; k1++)
                    p[3 * k1 + Dy * k2 + Dz * k3 + 0] += wl1[k1] * wp1[k3][k2];
        for (int k3 = lo; k3 < hi; k3++)
            for (int k2 = 0; k2 < ORD; k2++)
                for (int k1 = 0; k1 < NPT; k1++)
                    p[3 * k1 + Dy * k2 + Dz * k3 + 1] += wl2[k2] * wp2[k3][k1];
        for (int k3 = lo; k3 < (hi < ORD ? hi : ORD); k3++)
            for (int k2 = 0; k2 < NPT; k2++)
                for (int k1 = 0; k1 < NPT; k1++)
                    p[3 * k1 + Dy * k2 + Dz * k3 + 2] += wl3[k3] * wp3[k2][k1];
    }
}

static void OFN(dep3d)(R *jf, const int *j_size, const int *j_off, const R *jn,
                        const OFN(vp3) *vp, int nvp)
{
    const int Dy = 3 * j_size[0], Dz = Dy * j_size[1];
    R *pj = jf + (j_off[0] - OFS) * 3 + (j_off[1] - OFS) * Dy + (j_off[2] - OFS) * Dz;
#if VW == 8
    for (int g0 = 0; g0 < nvp; g0 += VW) {
        int gn = nvp - g0 < VW ? nvp - g0 : VW;
        for (int k3 = 0; k3 < NPT; k3++)
            for (int n = 0; n < gn; n++) OFN(dep3d_one)(pj, Dy, Dz, jn, &vp[g0 + n], k3);
    }
#else
    for (int n = 0; n < nvp; n++) OFN(dep3d_one)(pj, Dy, Dz, jn, &vp[n], -1);
#endif
}

/* Split one segment that crosses a single cell face along axis a (0,1,2) at +-0.5.
 * Appends the second part at *w and shortens *v to the first part (split-vec.h single-axis
 * cases). */
static inline void OFN(cut3)(OFN(vp3) *v, OFN(vp3) *w, int a, int d)
{
    R *c0[3] = {&v->x0, &v->y0, &v->z0};
    R *c1[3] = {&v->x1, &v->y1, &v->z1};
    R cint = (R)(0.5 * d);
    R delta = (cint - *c0[a]) / (*c1[a] - *c0[a]);
    R in[3];
    for (int b = 0; b < 3; b++)
        in[b] = (b == a) ? cint : *c0[b] + (*c1[b] - *c0[b]) * delta;
    *w = *v;
    w->x0 = in[0]; w->y0 = in[1]; w->z0 = in[2];
    if (a == 0) { w->x0 = -cint; w->x1 = v->x1 - d; w->i = v->i + d; }
    if (a == 1) { w->y0 = -cint; w->y1 = v->y1 - d; w->j = v->j + d; }
    if (a == 2) { w->z0 = -cint; w->z1 = v->z1 - d; w->k = v->k + d; }
    v->x1 = in[0]; v->y1 = in[1]; v->z1 = in[2];
}

/* Two-axis crossing (axes a < b), split-vec.h cases 3, 5, 6 restated. */
static inline void OFN(cut3_two)(OFN(vp3) *v, OFN(vp3) *w0, OFN(vp3) *w1, int a, int b,
                                 int da, int db)
{
    R *c0[3] = {&v->x0, &v->y0, &v->z0};
    R *c1[3] = {&v->x1, &v->y1, &v->z1};
    int *ci[3] = {&v->i, &v->j, &v->k};
    int oth = 3 - a - b;
    R aint = (R)(0.5 * da);
    R delta = (aint - *c0[a]) / (*c1[a] - *c0[a]);
    R bint = *c0[b] + (*c1[b] - *c0[b]) * delta;
    R oint = *c0[oth] + (*c1[oth] - *c0[oth]) * delta;
    R a0[3], a1[3];
    int ii[3];
    if (bint >= -0.5 && bint < 0.5) {
        /* first segment reaches the a face without crossing b; split the remainder at b */
        R bint2 = (R)(0.5 * db);
        R del2 = (bint2 - bint) / (*c1[b] - bint);
        R aint2 = -aint + (*c1[a] - aint) * del2;
        R oint2 = oint + (*c1[oth] - oint) * del2;
        /* w0: from the a face to the b face, in the cell shifted along a */
        a0[a] = -aint; a1[a] = aint2; a0[b] = bint; a1[b] = bint2; a0[oth] = oint; a1[oth] = oint2;
        ii[0] = v->i; ii[1] = v->j; ii[2] = v->k; ii[a] += da;
        w0->x0 = a0[0]; w0->x1 = a1[0]; w0->y0 = a0[1]; w0->y1 = a1[1]; w0->z0 = a0[2]; w0->z1 = a1[2];
        w0->i = ii[0]; w0->j = ii[1]; w0->k = ii[2]; w0->q = v->q;
        /* w1: from the b face to the end, in the cell shifted along a and b */
        a0[a] = aint2; a1[a] = *c1[a] - da; a0[b] = -bint2; a1[b] = *c1[b] - db;
        a0[oth] = oint2; a1[oth] = *c1[oth];
        ii[b] += db;
        w1->x0 = a0[0]; w1->x1 = a1[0]; w1->y0 = a0[1]; w1->y1 = a1[1]; w1->z0 = a0[2]; w1->z1 = a1[2];
        w1->i = ii[0]; w1->j = ii[1]; w1->k = ii[2]; w1->q = v->q;
        *c1[a] = aint; *c1[b] = bint; *c1[oth] = oint;
    } else {
        /* the b face is crossed before the a face */
        R bint2 = (R)(0.5 * db);
        R del2 = (bint2 - *c0[b]) / (bint - *c0[b]);
        R aint2 = *c0[a] + (aint - *c0[a]) * del2;
        R oint2 = *c0[oth] + (oint - *c0[oth]) * del2;
        a0[a] = aint2; a1[a] = aint; a0[b] = -bint2; a1[b] = bint - db; a0[oth] = oint2; a1[oth] = oint;
        ii[0] = v->i; ii[1] = v->j; ii[2] = v->k; ii[b] += db;
        w0->x0 = a0[0]; w0->x1 = a1[0]; w0->y0 = a0[1]; w0->y1 = a1[1]; w0->z0 = a0[2]; w0->z1 = a1[2];
        w0->i = ii[0]; w0->j = ii[1]; w0->k = ii[2]; w0->q = v->q;
        a0[a] = -aint; a1[a] = *c1[a] - da; a0[b] = bint - db; a1[b] = *c1[b] - db;
        a0[oth] = oint; a1[oth] = *c1[oth];
        ii[a] += da;
        w1->x0 = a0[0]; w1->x1 = a1[0]; w1->y0 = a0[1]; w1->y1 = a1[1]; w1->z0 = a0[2]; w1->z1 = a1[2];
        w1->i = ii[0]; w1->j = ii[1]; w1->k = ii[2]; w1->q = v->q;
        *c1[a] = aint2; *c1[b] = bint2; *c1[oth] = oint2;
    }
    (void)ci;
}

static void OFN(split3d)(OFN(vp3) *buf, int base, int gn, const int *dix, const int *diy,
                          const int *diz, int *extra)
{
    int ne = *extra;
    for (int l = 0; l < gn; l++) {
        OFN(vp3) *v = &buf[base + l];
        int cross = (dix[l] != 0 ? 1 : 0) | (diy[l] != 0 ? 2 : 0) | (diz[l] != 0 ? 4 : 0);
        switch (cross) {
        case 0:
            break;
        case 1: OFN(cut3)(v, &buf[ne++], 0, dix[l]); break;
        case 2: OFN(cut3)(v, &buf[ne++], 1, diy[l]); break;
        case 4: OFN(cut3)(v, &buf[ne++], 2, diz[l]); break;
        case 3: OFN(cut3_two)(v, &buf[ne], &buf[ne + 1], 0, 1, dix[l], diy[l]); ne += 2; break;
        case 5: OFN(cut3_two)(v, &buf[ne], &buf[ne + 1], 0, 2, dix[l], diz[l]); ne += 2; break;
        case 6: OFN(cut3_two)(v, &buf[ne], &buf[ne + 1], 1, 2, diy[l], diz[l]); ne += 2; break;
        case 7: {
            /* x-y split first, then the one segment that still leaves the z cell is cut */
            OFN(cut3_two)(v, &buf[ne], &buf[ne + 1], 0, 1, dix[l], diy[l]);
            ne += 2;
            OFN(vp3) *seg[3] = {v, &buf[ne - 2], &buf[ne - 1]};
            R zint = (R)(0.5 * diz[l]);
            for (int s = 0; s < 3; s++) {
                OFN(vp3) *c = seg[s];
                if (c->z1 < -0.5 || c->z1 >= 0.5) {
                    R delta = (zint - c->z0) / (c->z1 - c->z0);
                    R xi = c->x0 + (c->x1 - c->x0) * delta;
                    R yi = c->y0 + (c->y1 - c->y0) * delta;
                    OFN(vp3) *w = &buf[ne++];
                    w->x0 = xi; w->x1 = c->x1; w->y0 = yi; w->y1 = c->y1;
                    w->z0 = -zint; w->z1 = c->z1 - diz[l];
                    w->i = c->i; w->j = c->j; w->k = c->k + diz[l]; w->q = c->q;
                    c->x1 = xi; c->y1 = yi; c->z1 = zint;
                    for (int t = s + 1; t < 3; t++) {
                        seg[t]->z0 -= diz[l];
                        seg[t]->z1 -= diz[l];
                        seg[t]->k += diz[l];
                    }
                    break;
                }
            }
        } break;
        }
    }
    *extra = ne;
}

void OFN(ora_vadvance_deposit_3d)(int *ix, R *x, R *u, R *q, int *i0, int *i1, R *rqm,
                                  R *e, R *b, int *emf_size, int *emf_off,
                                  R *j, int *j_size, int *j_off,
                                  double *dx, double *dt, double *ene)
{
    const R tem = (R)(0.5 * (*dt) / (*rqm));
    const R dtdx1 = (R)((*dt) / dx[0]), dtdx2 = (R)((*dt) / dx[1]), dtdx3 = (R)((*dt) / dx[2]);
    R jn[3];
    jn[0] = (R)(dx[0] / (*dt) / 3);
    jn[1] = (R)(dx[1] / (*dt) / 3);
    jn[2] = (R)(dx[2] / (*dt) / 3);
    const int Dy = 3 * emf_size[0], Dz = Dy * emf_size[1];
    const R *e0 = e + (emf_off[0] - OFS) * 3 + (emf_off[1] - OFS) * Dy + (emf_off[2] - OFS) * Dz;
    const R *b0 = b + (emf_off[0] - OFS) * 3 + (emf_off[1] - OFS) * Dy + (emf_off[2] - OFS) * Dz;
    const int first = *i0 - 1, np = *i1 - *i0 + 1;
    const int cache = 160;
    OFN(vp3) *buf = (OFN(vp3) *)malloc(sizeof(OFN(vp3)) * 4 * cache);

    for (int c0 = 0; c0 < np; c0 += cache) {
        int cn = np - c0 < cache ? np - c0 : cache;
        R acc[VW];
        double eacc = 0.0;
        for (int l = 0; l < VW; l++) acc[l] = K(0.0);
        int nvp = 0;
        for (int g = 0; g < cn; g += VW) {
            int gn = cn - g < VW ? cn - g : VW;
            int base = nvp, extra = base + VW;
            int dix[VW], diy[VW], diz[VW];
            for (int l = 0; l < gn; l++) {
                int p = first + c0 + g + l;
                R x0 = x[3 * p], y0 = x[3 * p + 1], z0 = x[3 * p + 2];
                int i = ix[3 * p], jj = ix[3 * p + 1], kk = ix[3 * p + 2];
                R wx[NPT], wy[NPT], wz[NPT], wxh[NPT], wyh[NPT], wzh[NPT];
                OFN(spl)(x0, wx); OFN(spl)(y0, wy); OFN(spl)(z0, wz);
                R hx = x0 < K(0.0) ? K(1.0) : K(0.0);
                R hy = y0 < K(0.0) ? K(1.0) : K(0.0);
                R hz = z0 < K(0.0) ? K(1.0) : K(0.0);
                int ih = i - (x0 < K(0.0) ? 1 : 0);
                int jh = jj - (y0 < K(0.0) ? 1 : 0);
                int kh = kk - (z0 < K(0.0) ? 1 : 0);
                OFN(splh)(x0, hx, wxh); OFN(splh)(y0, hy, wyh); OFN(splh)(z0, hz, wzh);
                /* E1 (ih,j,k) E2 (i,jh,k) E3 (i,j,kh); B1 (i,jh,kh) B2 (ih,j,kh) B3 (ih,jh,k) */
                R E1 = K(0.0), E2 = K(0.0), E3 = K(0.0);
                for (int k3 = 0; k3 < NPT; k3++) {
                    R g1 = K(0.0), g2 = K(0.0), g3 = K(0.0);
                    for (int k2 = 0; k2 < NPT; k2++) {
                        R f1 = K(0.0), f2 = K(0.0), f3 = K(0.0);
                        for (int k1 = 0; k1 < NPT; k1++) {
                            f1 = FMA(e0[3 * (ih + k1) + Dy * (jj + k2) + Dz * (kk + k3) + 0], wxh[k1], f1);
                            f2 = FMA(e0[3 * (i + k1) + Dy * (jh + k2) + Dz * (kk + k3) + 1], wx[k1], f2);
                            f3 = FMA(e0[3 * (i + k1) + Dy * (jj + k2) + Dz * (kh + k3) + 2], wx[k1], f3);
                        }
                        g1 = FMA(f1, wy[k2], g1);
                        g2 = FMA(f2, wyh[k2], g2);
                        g3 = FMA(f3, wy[k2], g3);
                    }
                    E1 = FMA(g1, wz[k3], E1);
                    E2 = FMA(g2, wz[k3], E2);
                    E3 = FMA(g3, wzh[k3], E3);
                }
                R B1 = K(0.0), B2 = K(0.0), B3 = K(0.0);
                for (int k3 = 0; k3 < NPT; k3++) {
                    R g1 = K(0.0), g2 = K(0.0), g3 = K(0.0);
                    for (int k2 = 0; k2 < NPT; k2++) {
                        R f1 = K(0.0), f2 = K(0.0), f3 = K(0.0);
                        for (int k1 = 0; k1 < NPT; k1++) {
                            f1 = FMA(b0[3 * (i + k1) + Dy * (jh + k2) + Dz * (kh + k3) + 0], wx[k1], f1);
                            f2 = FMA(b0[3 * (ih + k1) + Dy * (jj + k2) + Dz * (kh + k3) + 1], wxh[k1], f2);
                            f3 = FMA(b0[3 * (ih + k1) + Dy * (jh + k2) + Dz * (kk + k3) + 2], wxh[k1], f3);
                        }
                        g1 = FMA(f1, wyh[k2], g1);
                        g2 = FMA(f2, wy[k2], g2);
                        g3 = FMA(f3, wyh[k2], g3);
                    }
                    B1 = FMA(g1, wzh[k3], B1);
                    B2 = FMA(g2, wzh[k3], B2);
                    B3 = FMA(g3, wz[k3], B3);
                }
                R u1 = u[3 * p], u2 = u[3 * p + 1], u3 = u[3 * p + 2], en;
                OFN(dudt)(tem, *rqm, E1, E2, E3, B1, B2, B3, &u1, &u2, &u3, &en, q[p], &eacc);
                u[3 * p] = u1; u[3 * p + 1] = u2; u[3 * p + 2] = u3;
                R rg = OFN(rgamma)(u1, u2, u3);
                acc[l] = FMA(q[p], en, acc[l]);
                R x1 = FMA(u1 * rg, dtdx1, x0);
                R y1 = FMA(u2 * rg, dtdx2, y0);
                R z1 = FMA(u3 * rg, dtdx3, z0);
                OFN(vp3) *v = &buf[base + l];
                v->x0 = x0; v->x1 = x1; v->y0 = y0; v->y1 = y1; v->z0 = z0; v->z1 = z1;
                v->q = q[p]; v->i = i; v->j = jj; v->k = kk;
                R tx = OFN(trim)(x1), ty = OFN(trim)(y1), tz = OFN(trim)(z1);
                x[3 * p] = x1 - tx;
                x[3 * p + 1] = y1 - ty;
                x[3 * p + 2] = z1 - tz;
                dix[l] = (int)tx; diy[l] = (int)ty; diz[l] = (int)tz;
                ix[3 * p] = i + dix[l];
                ix[3 * p + 1] = jj + diy[l];
                ix[3 * p + 2] = kk + diz[l];
            }
            for (int l = gn; l < VW; l++) buf[base + l].i = SKIP_VP;
            OFN(split3d)(buf, base, gn, dix, diy, diz, &extra);
            nvp = extra;
        }
        OFN(dep3d)(j, j_size, j_off, jn, buf, nvp);
        *ene += (double)OFN(lane_reduce)(acc);
        *ene += eacc;
    }
    free(buf);
}

#undef OFN
#undef NPT
