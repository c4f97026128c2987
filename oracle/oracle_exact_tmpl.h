/*
 * oracle_exact_tmpl.h -- TEST INFRASTRUCTURE ONLY (parity checker, never shipped).
 *
 * Scalar CPU restatement of the OSIRIS "exact" momentum update (push_type = "exact",
 * dudt_exact, source/spec/os-spec-extpush.f03:40-348, after arXiv:2007.07556): the momentum
 * is advanced by the analytic solution of the Lorentz force in the fields seen by the
 * particle, held constant over the step, with the proper time of the step found by Newton
 * iterations (at most p_iter_max = 10, relative tolerance iter_tol, default 1e-3,
 * source/spec/os-spec-define.f03:471).  Helpers restated: get_t_light (:352-391), get_t
 * (:395-430), trig_func (:720-760), hyper_func (:763-803), dot4 (:806-814), get_fu
 * (:817-830).  The spin and radiation-reaction branches are not on this path.
 *
 * Included by pic_oracle.c once per precision with R / SFX / K / SQRT set.  The arithmetic
 * follows the Fortran source's precision rules: p_k_part expressions in R, every
 * `_p_double` literal and the internals of trig_func / hyper_func in double, a double value
 * assigned to a p_k_part variable rounded to R; Fortran evaluates a + b + c as (a + b) + c.
 */

#ifndef PASTE3
#define PASTE3_(a, b, c) a##b##c
#define PASTE3(a, b, c) PASTE3_(a, b, c)
#endif
#define EXN(name) PASTE3(name, _, SFX)

static inline R EXN(exabs)(R v) { return v < K(0.0) ? -v : v; }

/* F u for the field tensor F = (E, B) (already scaled by q/m) and a four-vector
 * u = (u1, u2, u3, u4 = gamma); get_fu (:817-830) */
static inline void EXN(exfu)(const R *ep, const R *bp, const R *u, R *f)
{
    f[3] = (ep[0] * u[0] + ep[1] * u[1]) + ep[2] * u[2];
    f[0] = (ep[0] * u[3] + bp[2] * u[1]) - bp[1] * u[2];
    f[1] = (ep[1] * u[3] - bp[2] * u[0]) + bp[0] * u[2];
    f[2] = (ep[2] * u[3] + bp[1] * u[0]) - bp[0] * u[1];
}

/* cos x, sin x / x, (cos x - 1) / x^2 (trig_func, :720-760) */
static inline void EXN(extrig)(R x, R *cn, R *snc, R *cnc)
{
    const double xd = (double)x, x2 = xd * xd;
    if (fabs(xd) < 0.007367081148666) {
        const double x4 = x2 * x2;
        *cn = (R)((1.0 - 0.5 * x2) + 0.041666666666667 * x4);
        *snc = (R)((1.0 - 0.166666666666667 * x2) + 0.008333333333333 * x4);
        *cnc = (R)((-0.5 + 0.041666666666667 * x2) - 0.001388888888889 * x4);
    } else {
        const double t1 = tan(0.5 * xd), t2 = t1 * t1, t3 = 1.0 / (1.0 + t2);
        const double cnd = (1.0 - t2) * t3;
        *cn = (R)cnd;
        *snc = (R)(((2.0 * t1) * t3) / xd);
        *cnc = (R)((cnd - 1.0) / x2);
    }
}

/* cosh x, sinh x / x, (cosh x - 1) / x^2 (hyper_func, :763-803) */
static inline void EXN(exhyp)(R x, R *ch, R *shc, R *chc)
{
    const double xd = (double)x, x2 = xd * xd;
    if (fabs(xd) < 0.007367081148666) {
        const double x4 = x2 * x2;
        *ch = (R)((1.0 + 0.5 * x2) + 0.041666666666667 * x4);
        *shc = (R)((1.0 + 0.166666666666667 * x2) + 0.008333333333333 * x4);
        *chc = (R)((0.5 + 0.041666666666667 * x2) + 0.001388888888889 * x4);
    } else {
        const double t1 = tanh(0.5 * xd), t2 = t1 * t1, t3 = 1.0 / (1.0 - t2);
        const double chd = (1.0 + t2) * t3;
        *ch = (R)chd;
        *shc = (R)(((2.0 * t1) * t3) / xd);
        *chc = (R)((chd - 1.0) / x2);
    }
}

/* Exact momentum update of one particle.  ep / bp: interpolated fields already multiplied by
 * qm = 1 / rqm (in R); u: momentum (in/out); dt: the double time step; tol: iter_tol.
 * Returns 1 when the particle was pushed, 0 in a weak field (e^2 + b^2 < 1e-12: the reference
 * leaves such a particle's momentum unchanged). */
static int EXN(ora_exact_u)(const R *ep, const R *bp, R *u, double dt, double tol)
{
    const double rel_tol = 1.0e-12, weak_fld_tol = 1.0e-12;
    const R e2 = (ep[0] * ep[0] + ep[1] * ep[1]) + ep[2] * ep[2];
    const R b2 = (bp[0] * bp[0] + bp[1] * bp[1]) + bp[2] * bp[2];
    if ((double)(e2 + b2) < weak_fld_tol) return 0;
    const R inv1 = e2 - b2;
    const R inv2 = (ep[0] * bp[0] + ep[1] * bp[1]) + ep[2] * bp[2];
    const R tmp = SQRT(inv1 * inv1 + (K(4.0) * inv2) * inv2);
    const R k2 = K(0.5) * (inv1 + tmp), kk = SQRT(k2);
    const R o2 = K(0.5) * (-inv1 + tmp), oo = SQRT(o2);
    R u0[4], fu0[4], f2u0[4];
    u0[0] = u[0];
    u0[1] = u[1];
    u0[2] = u[2];
    u0[3] = SQRT(((K(1.0) + u0[0] * u0[0]) + u0[1] * u0[1]) + u0[2] * u0[2]);
    EXN(exfu)(ep, bp, u0, fu0);
    EXN(exfu)(ep, bp, fu0, f2u0);
    if ((double)k2 < rel_tol && (double)o2 < rel_tol) {
        /* light-like field: get_t_light (:352-391) */
        R f3u0[4];
        EXN(exfu)(ep, bp, f2u0, f3u0);
        R t1 = (R)(dt / (double)u0[3]), t = t1, c1 = K(0.0), c2 = K(0.0);
        int iter = 0;
        for (;;) {
            const R t2 = t1 * t1, t3 = t2 * t1;
            c1 = (R)(0.5 * (double)t2);
            c2 = (R)(0.166666666666667 * (double)t3);
            const R fa = (t1 * u0[3] + c1 * fu0[3]) + c2 * f2u0[3];
            const double fb = ((0.041666666666667 * (double)t3) * (double)t1) * (double)f3u0[3];
            const R fun = (R)(((double)fa + fb) - dt);
            const R dfun = ((u0[3] + t1 * fu0[3]) + c1 * f2u0[3]) + c2 * f3u0[3];
            t = t1 - fun / dfun;
            iter++;
            if ((double)(EXN(exabs)(t - t1) / t1) < tol || iter > 10) break;
            t1 = t;
        }
        for (int c = 0; c < 3; c++) u[c] = ((u0[c] + t * fu0[c]) + c1 * f2u0[c]) + c2 * f3u0[c];
        return 1;
    }
    /* general field: subspace decomposition and get_t (:395-430) */
    const R k2o2 = k2 + o2;
    R uk0[4], uo0[4], fuk0[4], fuo0[4];
    for (int c = 0; c < 4; c++) {
        uk0[c] = (f2u0[c] + o2 * u0[c]) / k2o2;
        uo0[c] = u0[c] - uk0[c];
    }
    EXN(exfu)(ep, bp, uk0, fuk0);
    for (int c = 0; c < 4; c++) fuo0[c] = fu0[c] - fuk0[c];
    R t0 = (R)(dt / (double)(uk0[3] + uo0[3])), t = t0;
    R ch_k, shc_k, chc_k, cn_o, snc_o, cnc_o;
    int iter = 0;
    for (;;) {
        EXN(extrig)(oo * t0, &cn_o, &snc_o, &cnc_o);
        EXN(exhyp)(kk * t0, &ch_k, &shc_k, &chc_k);
        const R fa = (uk0[3] * shc_k + (fuk0[3] * chc_k) * t0) * t0 +
                     (uo0[3] * snc_o - (fuo0[3] * cnc_o) * t0) * t0;
        const R fun = (R)((double)fa - dt);
        const R dfun = ((uk0[3] * ch_k + (fuk0[3] * shc_k) * t0) + uo0[3] * cn_o) +
                       (fuo0[3] * snc_o) * t0;
        t = t0 - fun / dfun;
        iter++;
        if ((double)(EXN(exabs)(t - t0) / t0) < tol || iter > 10) break;
        t0 = t;
    }
    for (int c = 0; c < 3; c++) {
        const R uk = uk0[c] * ch_k + (fuk0[c] * shc_k) * t;
        const R uo = uo0[c] * cn_o + (fuo0[c] * snc_o) * t;
        u[c] = uk + uo;
    }
    return 1;
}

/* Vay pusher (dudt_vay, source/spec/os-spec-push.f03:636-796): tem = real(0.5 dt / rqm)
 * (:663); fields scaled by tem; returns q uc^2 / (gamma_c + 1) of the time-centred momentum
 * uc = (u_old + u_new) / 2 (:772-790).  x**2 of the Fortran is x * x. */
static R EXN(ora_vay_u)(R tem, const R *e, const R *b, R *u, R q)
{
    R ep[3], bp[3], tv[3], ut[3];
    for (int c = 0; c < 3; c++) {
        ep[c] = e[c] * tem;
        bp[c] = b[c] * tem;
    }
    R rgam = K(1.0) / SQRT(((K(1.0) + u[0] * u[0]) + u[1] * u[1]) + u[2] * u[2]);
    for (int c = 0; c < 3; c++) tv[c] = u[c] * rgam;
    const R bpsq = (bp[0] * bp[0] + bp[1] * bp[1]) + bp[2] * bp[2];
    ut[0] = ((u[0] + ep[0]) + tv[1] * bp[2]) - tv[2] * bp[1];
    ut[1] = ((u[1] + ep[1]) + tv[2] * bp[0]) - tv[0] * bp[2];
    ut[2] = ((u[2] + ep[2]) + tv[0] * bp[1]) - tv[1] * bp[0];
    for (int c = 0; c < 3; c++) tv[c] = ut[c] + ep[c];
    const R ustar = (tv[0] * bp[0] + tv[1] * bp[1]) + tv[2] * bp[2];
    const R sigma = (((K(1.0) + tv[0] * tv[0]) + tv[1] * tv[1]) + tv[2] * tv[2]) - bpsq;
    rgam = K(1.0) / SQRT(K(0.5) * (sigma + SQRT(sigma * sigma + K(4.0) * (bpsq + ustar * ustar))));
    for (int c = 0; c < 3; c++) bp[c] = bp[c] * rgam;
    const R spar = K(1.0) / (((K(1.0) + bp[0] * bp[0]) + bp[1] * bp[1]) + bp[2] * bp[2]);
    const R uptp = (tv[0] * bp[0] + tv[1] * bp[1]) + tv[2] * bp[2];
    const R uo[3] = {u[0], u[1], u[2]};
    u[0] = spar * (((tv[0] + uptp * bp[0]) + tv[1] * bp[2]) - tv[2] * bp[1]);
    u[1] = spar * (((tv[1] + uptp * bp[1]) + tv[2] * bp[0]) - tv[0] * bp[2]);
    u[2] = spar * (((tv[2] + uptp * bp[2]) + tv[0] * bp[1]) - tv[1] * bp[0]);
    R uc[3];
    for (int c = 0; c < 3; c++) uc[c] = K(0.5) * (uo[c] + u[c]);
    const R uc2 = (uc[0] * uc[0] + uc[1] * uc[1]) + uc[2] * uc[2];
    const R gc = SQRT(uc2 + K(1.0));
    return (q * uc2) / (gc + K(1.0));
}

/* Conditional Vay pusher (dudt_cond_vay, source/spec/os-spec-push.f03:800-1100): tem =
 * real(0.5 dt / rqm) (:835).  A particle whose gamma of the old momentum, sqrt(1 + p1**2 +
 * p2**2 + p3**2) left to right (:856), exceeds 5 takes the Vay update and its energy term
 * (:883-1007); the others the Boris loops of the same routine (:1011-1094): half kick,
 * energy q u2 / (gamma + 1) with the division in double, b scaled by tem / gamma, the
 * rotation written as two passes per cross product, 2 / (((1 + b1**2) + b2**2) + b3**2),
 * half kick. */
static double EXN(ora_cond_vay_u)(R tem, const R *e, const R *b, R *u, R q)
{
    const R g0 = SQRT(((K(1.0) + u[0] * u[0]) + u[1] * u[1]) + u[2] * u[2]);
    if (g0 > K(5.0)) return (double)EXN(ora_vay_u)(tem, e, b, u, q);
    R ep[3], bp[3], ut[3], pn[3];
    for (int c = 0; c < 3; c++) {
        ep[c] = e[c] * tem;
        ut[c] = u[c] + ep[c];
    }
    const R u2 = (ut[0] * ut[0] + ut[1] * ut[1]) + ut[2] * ut[2];
    const R gam = SQRT(u2 + K(1.0));
    const double ene = (double)(q * u2) / ((double)gam + 1.0);
    const R gt = tem / gam;
    for (int c = 0; c < 3; c++) bp[c] = b[c] * gt;
    pn[0] = ut[0] + ut[1] * bp[2];
    pn[1] = ut[1] + ut[2] * bp[0];
    pn[2] = ut[2] + ut[0] * bp[1];
    pn[0] = pn[0] - ut[2] * bp[1];
    pn[1] = pn[1] - ut[0] * bp[2];
    pn[2] = pn[2] - ut[1] * bp[0];
    const R otsq = K(2.0) / (((K(1.0) + bp[0] * bp[0]) + bp[1] * bp[1]) + bp[2] * bp[2]);
    for (int c = 0; c < 3; c++) bp[c] = bp[c] * otsq;
    ut[0] = ut[0] + pn[1] * bp[2];
    ut[1] = ut[1] + pn[2] * bp[0];
    ut[2] = ut[2] + pn[0] * bp[1];
    ut[0] = ut[0] - pn[2] * bp[1];
    ut[1] = ut[1] - pn[0] * bp[2];
    ut[2] = ut[2] - pn[1] * bp[0];
    for (int c = 0; c < 3; c++) u[c] = ut[c] + ep[c];
    return ene;
}

/* Higuera-Cary pusher (dudt_cary, source/spec/os-spec-push.f03:1104-1253): tem =
 * real(0.5 (dt / rqm)) (:1132); returns the energy term q u2 / (sqrt(gamma_minus^2) + 1)
 * accumulated in double (:1150-1153). */
static double EXN(ora_hc_u)(R tem, const R *e, const R *b, R *u, R q)
{
    R ep[3], bp[3], ut[3], pn[3];
    for (int c = 0; c < 3; c++) {
        ep[c] = e[c] * tem;
        bp[c] = b[c] * tem;
    }
    for (int c = 0; c < 3; c++) ut[c] = u[c] + ep[c];
    const R u2 = (ut[0] * ut[0] + ut[1] * ut[1]) + ut[2] * ut[2];
    const R gm = (R)((double)u2 + 1.0);
    const double ene = (double)(q * u2) / ((double)SQRT(gm) + 1.0);
    const R bpsq = (bp[0] * bp[0] + bp[1] * bp[1]) + bp[2] * bp[2];
    R bdu = (bp[0] * ut[0] + bp[1] * ut[1]) + bp[2] * ut[2];
    bdu = bdu * bdu;
    const R gmb = gm - bpsq;
    const R gam = SQRT(K(0.5) * (gmb + SQRT(gmb * gmb + K(4.0) * (bpsq + bdu))));
    for (int c = 0; c < 3; c++) bp[c] = bp[c] / gam;
    pn[0] = ut[0] + ut[1] * bp[2];
    pn[1] = ut[1] + ut[2] * bp[0];
    pn[2] = ut[2] + ut[0] * bp[1];
    pn[0] = pn[0] - ut[2] * bp[1];
    pn[1] = pn[1] - ut[0] * bp[2];
    pn[2] = pn[2] - ut[1] * bp[0];
    const R otsq = K(2.0) / (((K(1.0) + bp[0] * bp[0]) + bp[1] * bp[1]) + bp[2] * bp[2]);
    for (int c = 0; c < 3; c++) bp[c] = bp[c] * otsq;
    ut[0] = ut[0] + pn[1] * bp[2];
    ut[1] = ut[1] + pn[2] * bp[0];
    ut[2] = ut[2] + pn[0] * bp[1];
    ut[0] = ut[0] - pn[2] * bp[1];
    ut[1] = ut[1] - pn[0] * bp[2];
    ut[2] = ut[2] - pn[1] * bp[0];
    for (int c = 0; c < 3; c++) u[c] = ut[c] + ep[c];
    return ene;
}

/* Full-rotation pusher (dudt_fullrot, source/spec/os-spec-push.f03:83-231): Boris with the
 * rotation vector scaled by tan(b)/b, so a pure magnetic field turns the momentum by the exact
 * gyration angle.  tem = real(0.5 (dt / rqm)) (:112); tan(b)/b of b^2 by the reference's
 * rational approximation, evaluated in double from the float b^2 and rounded back (:166-178);
 * returns q u^2 / (gamma + 1) of the half-kicked momentum in double (:144-147). */
static double EXN(ora_fullrot_u)(R tem, const R *e, const R *b, R *u, R q)
{
    R ep[3], ut[3], bp[3], p[3];
    for (int c = 0; c < 3; c++) ep[c] = e[c] * tem;
    for (int c = 0; c < 3; c++) ut[c] = u[c] + ep[c];
    const R u2 = (ut[0] * ut[0] + ut[1] * ut[1]) + ut[2] * ut[2];
    const R gamma = SQRT(u2 + K(1.0));
    const double ene = (double)(q * u2) / ((double)gamma + 1.0);
    const R tg = tem / gamma;
    for (int c = 0; c < 3; c++) bp[c] = b[c] * tg;
    const R b2 = (bp[0] * bp[0] + bp[1] * bp[1]) + bp[2] * bp[2];
    const double d2 = (double)b2;
    const R r = (R)(2005892.32789228135999056 +
                    d2 * (-267559.850143894287032640 +
                          d2 * (6870.7950060474599763728 - 35.8427314349709199363798 * d2)));
    const R s = (R)(2005892.32789228136020125 +
                    d2 * (-936190.626107988089080768 +
                          d2 * (51482.0266564063006502261 + d2 * (d2 - 625.608053837898687047447))));
    const R t = s != K(0.0) ? r / s : K(1.0);
    for (int c = 0; c < 3; c++) bp[c] = bp[c] * t;
    p[0] = (ut[0] + ut[1] * bp[2]) - ut[2] * bp[1];
    p[1] = (ut[1] + ut[2] * bp[0]) - ut[0] * bp[2];
    p[2] = (ut[2] + ut[0] * bp[1]) - ut[1] * bp[0];
    const R sc = K(2.0) / (((K(1.0) + bp[0] * bp[0]) + bp[1] * bp[1]) + bp[2] * bp[2]);
    for (int c = 0; c < 3; c++) bp[c] = bp[c] * sc;
    ut[0] = (ut[0] + p[1] * bp[2]) - p[2] * bp[1];
    ut[1] = (ut[1] + p[2] * bp[0]) - p[0] * bp[2];
    ut[2] = (ut[2] + p[0] * bp[1]) - p[1] * bp[0];
    for (int c = 0; c < 3; c++) u[c] = ut[c] + ep[c];
    return ene;
}

/* Euler-rotation pusher (dudt_euler, :235-352): the magnetic rotation as an explicit rotation
 * matrix from the quaternion (cos(w/2), -sin(w/2) b/|b|), w = |b| dt / (rqm gamma) with
 * gam_tem = dt / (rqm gamma) in double from the float product rqm gamma (:289); tem as the
 * full-rotation pusher; same energy term. */
static double EXN(ora_euler_u)(R tem, R rqm, double dt, const R *e, const R *b, R *u, R q)
{
    R ep[3], ut[3], bp[3];
    for (int c = 0; c < 3; c++) ep[c] = e[c] * tem;
    for (int c = 0; c < 3; c++) ut[c] = u[c] + ep[c];
    const R u2 = (ut[0] * ut[0] + ut[1] * ut[1]) + ut[2] * ut[2];
    const R gamma = SQRT(u2 + K(1.0));
    const double ene = (double)(q * u2) / ((double)gamma + 1.0);
    const R gt = (R)(dt / (double)(rqm * gamma));
    for (int c = 0; c < 3; c++) bp[c] = b[c] * gt;
    const R b2 = (bp[0] * bp[0] + bp[1] * bp[1]) + bp[2] * bp[2];
    const R bn = SQRT(b2);
    R s = SIN(bn / K(2.0));
    const R a = COS(bn / K(2.0));
    s = b2 > K(0.0) ? -s / bn : K(-1.0);
    const R qb = bp[0] * s, qc = bp[1] * s, qd = bp[2] * s;
    const R r11 = ((a * a + qb * qb) - qc * qc) - qd * qd, r21 = K(2.0) * (qb * qc - a * qd),
            r31 = K(2.0) * (qb * qd + a * qc);
    const R r12 = K(2.0) * (qb * qc + a * qd), r22 = ((a * a + qc * qc) - qb * qb) - qd * qd,
            r32 = K(2.0) * (qc * qd - a * qb);
    const R r13 = K(2.0) * (qb * qd - a * qc), r23 = K(2.0) * (qc * qd + a * qb),
            r33 = ((a * a + qd * qd) - qb * qb) - qc * qc;
    const R pn[3] = {(r11 * ut[0] + r21 * ut[1]) + r31 * ut[2],
                     (r12 * ut[0] + r22 * ut[1]) + r32 * ut[2],
                     (r13 * ut[0] + r23 * ut[1]) + r33 * ut[2]};
    for (int c = 0; c < 3; c++) u[c] = pn[c] + ep[c];
    return ene;
}

/* Momentum update of n particles in given (unscaled) fields e(3,n), b(3,n) by pusher 1 (exact:
 * fields times qm = 1/rqm as dudt_exact, :76-86, energy q (gamma - 1) of the new momenta),
 * 2 (Vay), 3 (Higuera-Cary), 4 (full rotation), 5 (Euler rotation) or 6 (conditional Vay)
 * with their own tem and
 * energy terms; *ene += the double sum. */
void EXN(ora_dudt_pusher)(int pusher, int n, const R *e, const R *b, R *u, const R *q, R rqm,
                          double dt, double tol, double *ene)
{
    const R qm = K(1.0) / rqm;
    double loc = 0.0;
    for (int i = 0; i < n; i++) {
        if (pusher == 2) {
            loc += (double)EXN(ora_vay_u)((R)(0.5 * dt / (double)rqm), e + 3 * i, b + 3 * i,
                                          u + 3 * i, q[i]);
            continue;
        }
        if (pusher == 3) {
            loc += EXN(ora_hc_u)((R)(0.5 * (dt / (double)rqm)), e + 3 * i, b + 3 * i, u + 3 * i,
                                 q[i]);
            continue;
        }
        if (pusher == 4) {
            loc += EXN(ora_fullrot_u)((R)(0.5 * (dt / (double)rqm)), e + 3 * i, b + 3 * i,
                                      u + 3 * i, q[i]);
            continue;
        }
        if (pusher == 6) {
            loc += EXN(ora_cond_vay_u)((R)(0.5 * dt / (double)rqm), e + 3 * i, b + 3 * i,
                                       u + 3 * i, q[i]);
            continue;
        }
        if (pusher == 5) {
            loc += EXN(ora_euler_u)((R)(0.5 * (dt / (double)rqm)), rqm, dt, e + 3 * i, b + 3 * i,
                                    u + 3 * i, q[i]);
            continue;
        }
        R ep[3], bp[3];
        for (int c = 0; c < 3; c++) {
            ep[c] = e[3 * i + c] * qm;
            bp[c] = b[3 * i + c] * qm;
        }
        EXN(ora_exact_u)(ep, bp, u + 3 * i, dt, tol);
        const R g = SQRT(((K(1.0) + u[3 * i] * u[3 * i]) + u[3 * i + 1] * u[3 * i + 1]) +
                         u[3 * i + 2] * u[3 * i + 2]);
        loc += (double)(q[i] * (g - K(1.0)));
    }
    *ene += loc;
}

void EXN(ora_dudt_exact)(int n, const R *e, const R *b, R *u, const R *q, R rqm, double dt,
                         double tol, double *ene)
{
    EXN(ora_dudt_pusher)(1, n, e, b, u, q, rqm, dt, tol, ene);
}

/* Selected momentum update of the push restatement below (0 = Boris, 1 = exact, 2 = Vay,
 * 3 = Higuera-Cary, 4 = full rotation, 5 = Euler rotation), the exact pusher's tolerance and the double time step of the Fortran
 * pushers; set by ora_push_pusher_* around one call. */
static int EXN(ora_pusher) = 0;
static double EXN(ora_iter_tol) = 1.0e-3;
static double EXN(ora_push_dt) = 0.0;
