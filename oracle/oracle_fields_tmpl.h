/*
 * oracle_fields_tmpl.h -- TEST INFRASTRUCTURE ONLY (parity checker, never shipped).
 *
 * Scalar restatement of the grid phases of one OSIRIS time step on a single periodic node.
 * Included by pic_oracle.c with R (float|double) and SFX (f32|f64) defined.
 *
 * Grid layout (reference t_vdf, source/vdf/os-vdf-define.f03:35-116): component fastest,
 * f(3, 1-gcl:nx+gcu, ...) stored contiguously; here element (c, i1, i2, i3) with Fortran cell
 * indices lives at c + 3*((i1-1+gcl0) + size0*((i2-1+gcl1) + size1*(i3-1+gcl2))).
 *
 *   Yee B half step   source/emf/solver/os-emf-solver-yee.f03:102-138 (2D), :211-251 (3D)
 *   Yee E full step   source/emf/solver/os-emf-solver-yee.f03:287-326 (2D), :385-428 (3D)
 *   Yee advance       source/emf/solver/os-emf-solver-yee.f03:542-568
 *   periodic add/replace   source/vdf/os-vdf-comm.f90:142-326, direction loop :665-722
 *   particle periodic wrap source/spec/os-spec-boundary.f03:1280-1290
 *   counting sort     source/spec/os-species.f03:388-505 (index), :512- (rearrange)
 *   charge deposit    source/spec/os-spec-charge.f90:500-600
 *   divergence        source/vdf/os-vdf-math.f90:1013-1073
 *   field energy      source/emf/diagnostics/os-emf-diagnostics.f03:42-58 (0.5*dV*sum f^2)
 *   kinetic energy    source/spec/os-spec-define.f03:1030-1086
 *   smoothing         source/vdf/os-vdf-smooth.f90:639-1000 (filter_2d / filter_3d)
 */

#define FN(name) PASTE3(name, _, SFX)

typedef struct {
    int dim;
    int nx[3], gcl[3], gcu[3], size[3];
} FN(ora_grid);

static inline long FN(gidx)(const FN(ora_grid) *g, int c, int i1, int i2, int i3)
{
    long p = (long)(i1 - 1 + g->gcl[0]);
    if (g->dim > 1) p += (long)g->size[0] * (i2 - 1 + g->gcl[1]);
    if (g->dim > 2) p += (long)g->size[0] * g->size[1] * (i3 - 1 + g->gcl[2]);
    return c + 3 * p;
}

static void FN(grid_init)(FN(ora_grid) *g, int dim, const int *nx, const int *gcl,
                          const int *gcu)
{
    g->dim = dim;
    for (int d = 0; d < 3; d++) {
        g->nx[d] = d < dim ? nx[d] : 1;
        g->gcl[d] = d < dim ? gcl[d] : 0;
        g->gcu[d] = d < dim ? gcu[d] : 0;
        g->size[d] = g->nx[d] + g->gcl[d] + g->gcu[d];
    }
}

#define AT(f, c, a, b, cc) f[FN(gidx)(g, c, a, b, cc)]

static void FN(dbdt)(const FN(ora_grid) *g, R *bf, const R *ef, const double *dx, double dt)
{
    if (g->dim == 2) {
        const R d1 = (R)(dt / dx[0]), d2 = (R)(dt / dx[1]);
        for (int i2 = 0; i2 <= g->nx[1] + 1; i2++)
            for (int i1 = 0; i1 <= g->nx[0] + 1; i1++) {
                AT(bf, 0, i1, i2, 1) = AT(bf, 0, i1, i2, 1) - d2 * (AT(ef, 2, i1, i2 + 1, 1) - AT(ef, 2, i1, i2, 1));
                AT(bf, 1, i1, i2, 1) = AT(bf, 1, i1, i2, 1) + d1 * (AT(ef, 2, i1 + 1, i2, 1) - AT(ef, 2, i1, i2, 1));
                AT(bf, 2, i1, i2, 1) = AT(bf, 2, i1, i2, 1) - d1 * (AT(ef, 1, i1 + 1, i2, 1) - AT(ef, 1, i1, i2, 1))
                                       + d2 * (AT(ef, 0, i1, i2 + 1, 1) - AT(ef, 0, i1, i2, 1));
            }
    } else if (g->dim == 3) {
        const R d1 = (R)(dt / dx[0]), d2 = (R)(dt / dx[1]), d3 = (R)(dt / dx[2]);
        for (int i3 = 0; i3 <= g->nx[2] + 1; i3++)
            for (int i2 = 0; i2 <= g->nx[1] + 1; i2++)
                for (int i1 = 0; i1 <= g->nx[0] + 1; i1++) {
                    AT(bf, 0, i1, i2, i3) = AT(bf, 0, i1, i2, i3)
                        - d2 * (AT(ef, 2, i1, i2 + 1, i3) - AT(ef, 2, i1, i2, i3))
                        + d3 * (AT(ef, 1, i1, i2, i3 + 1) - AT(ef, 1, i1, i2, i3));
                    AT(bf, 1, i1, i2, i3) = AT(bf, 1, i1, i2, i3)
                        + d1 * (AT(ef, 2, i1 + 1, i2, i3) - AT(ef, 2, i1, i2, i3))
                        - d3 * (AT(ef, 0, i1, i2, i3 + 1) - AT(ef, 0, i1, i2, i3));
                    AT(bf, 2, i1, i2, i3) = AT(bf, 2, i1, i2, i3)
                        - d1 * (AT(ef, 1, i1 + 1, i2, i3) - AT(ef, 1, i1, i2, i3))
                        + d2 * (AT(ef, 0, i1, i2 + 1, i3) - AT(ef, 0, i1, i2, i3));
                }
    } else {
        const R d1 = (R)(dt / dx[0]);
        for (int i1 = 0; i1 <= g->nx[0] + 1; i1++) {
            AT(bf, 1, i1, 1, 1) = AT(bf, 1, i1, 1, 1) + d1 * (AT(ef, 2, i1 + 1, 1, 1) - AT(ef, 2, i1, 1, 1));
            AT(bf, 2, i1, 1, 1) = AT(bf, 2, i1, 1, 1) - d1 * (AT(ef, 1, i1 + 1, 1, 1) - AT(ef, 1, i1, 1, 1));
        }
    }
}

static void FN(dedt)(const FN(ora_grid) *g, R *ef, const R *bf, const R *jf, const double *dx,
                     double dt)
{
    const R dti = (R)dt;
    if (g->dim == 2) {
        const R d1 = (R)(dt / dx[0]), d2 = (R)(dt / dx[1]);
        for (int i2 = 1; i2 <= g->nx[1] + 1; i2++)
            for (int i1 = 1; i1 <= g->nx[0] + 1; i1++) {
                AT(ef, 0, i1, i2, 1) = AT(ef, 0, i1, i2, 1) - dti * AT(jf, 0, i1, i2, 1)
                                       + d2 * (AT(bf, 2, i1, i2, 1) - AT(bf, 2, i1, i2 - 1, 1));
                AT(ef, 1, i1, i2, 1) = AT(ef, 1, i1, i2, 1) - dti * AT(jf, 1, i1, i2, 1)
                                       - d1 * (AT(bf, 2, i1, i2, 1) - AT(bf, 2, i1 - 1, i2, 1));
                AT(ef, 2, i1, i2, 1) = AT(ef, 2, i1, i2, 1) - dti * AT(jf, 2, i1, i2, 1)
                                       + d1 * (AT(bf, 1, i1, i2, 1) - AT(bf, 1, i1 - 1, i2, 1))
                                       - d2 * (AT(bf, 0, i1, i2, 1) - AT(bf, 0, i1, i2 - 1, 1));
            }
    } else if (g->dim == 3) {
        const R d1 = (R)(dt / dx[0]), d2 = (R)(dt / dx[1]), d3 = (R)(dt / dx[2]);
        for (int i3 = 1; i3 <= g->nx[2] + 1; i3++)
            for (int i2 = 1; i2 <= g->nx[1] + 1; i2++)
                for (int i1 = 1; i1 <= g->nx[0] + 1; i1++) {
                    AT(ef, 0, i1, i2, i3) = AT(ef, 0, i1, i2, i3) - dti * AT(jf, 0, i1, i2, i3)
                        + d2 * (AT(bf, 2, i1, i2, i3) - AT(bf, 2, i1, i2 - 1, i3))
                        - d3 * (AT(bf, 1, i1, i2, i3) - AT(bf, 1, i1, i2, i3 - 1));
                    AT(ef, 1, i1, i2, i3) = AT(ef, 1, i1, i2, i3) - dti * AT(jf, 1, i1, i2, i3)
                        + d3 * (AT(bf, 0, i1, i2, i3) - AT(bf, 0, i1, i2, i3 - 1))
                        - d1 * (AT(bf, 2, i1, i2, i3) - AT(bf, 2, i1 - 1, i2, i3));
                    AT(ef, 2, i1, i2, i3) = AT(ef, 2, i1, i2, i3) - dti * AT(jf, 2, i1, i2, i3)
                        + d1 * (AT(bf, 1, i1, i2, i3) - AT(bf, 1, i1 - 1, i2, i3))
                        - d2 * (AT(bf, 0, i1, i2, i3) - AT(bf, 0, i1, i2 - 1, i3));
                }
    } else {
        const R d1 = (R)(dt / dx[0]);
        for (int i1 = 1; i1 <= g->nx[0] + 1; i1++) {
            AT(ef, 0, i1, 1, 1) = AT(ef, 0, i1, 1, 1) - dti * AT(jf, 0, i1, 1, 1);
            AT(ef, 1, i1, 1, 1) = AT(ef, 1, i1, 1, 1) - dti * AT(jf, 1, i1, 1, 1)
                                  - d1 * (AT(bf, 2, i1, 1, 1) - AT(bf, 2, i1 - 1, 1, 1));
            AT(ef, 2, i1, 1, 1) = AT(ef, 2, i1, 1, 1) - dti * AT(jf, 2, i1, 1, 1)
                                  + d1 * (AT(bf, 1, i1, 1, 1) - AT(bf, 1, i1 - 1, 1, 1));
        }
    }
}

/* B half step, E full step, B half step (periodic: no boundary work in between) */
void FN(ora_yee_advance)(int dim, const int *nx, const int *gcl, const int *gcu, R *e, R *b,
                         const R *j, const double *dx, double dt)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    FN(dbdt)(g, b, e, dx, dt / 2.0);
    FN(dedt)(g, e, b, j, dx, dt);
    FN(dbdt)(g, b, e, dx, dt / 2.0);
}

/* update_periodic_vdf for every direction in order; add = 1 folds guard cells (current),
 * add = 0 replaces guard cells by the periodic image (fields). ncomp components per point. */
void FN(ora_periodic)(int dim, const int *nx, const int *gcl, const int *gcu, R *f, int add)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    for (int d = 0; d < dim; d++) {
        int lo[3], hi[3], ulo[3], uhi[3], sh[3] = {0, 0, 0};
        for (int e = 0; e < 3; e++) {
            if (e == d) {
                lo[e] = 1 - g->gcl[e]; hi[e] = 0;
                ulo[e] = g->nx[e] + 1; uhi[e] = g->nx[e] + g->gcu[e];
                sh[e] = g->nx[e];
            } else if (e < dim) {
                lo[e] = ulo[e] = 1 - g->gcl[e];
                hi[e] = uhi[e] = g->nx[e] + g->gcu[e];
            } else {
                lo[e] = ulo[e] = hi[e] = uhi[e] = 1;
            }
        }
        for (int i3 = lo[2]; i3 <= hi[2]; i3++)
            for (int i2 = lo[1]; i2 <= hi[1]; i2++)
                for (int i1 = lo[0]; i1 <= hi[0]; i1++)
                    for (int c = 0; c < 3; c++) {
                        long a = FN(gidx)(g, c, i1, i2, i3);
                        long o = FN(gidx)(g, c, i1 + sh[0], i2 + sh[1], i3 + sh[2]);
                        if (add) {
                            R v = f[a] + f[o];
                            f[a] = v;
                            f[o] = v;
                        } else {
                            f[a] = f[o];
                        }
                    }
        for (int i3 = ulo[2]; i3 <= uhi[2]; i3++)
            for (int i2 = ulo[1]; i2 <= uhi[1]; i2++)
                for (int i1 = ulo[0]; i1 <= uhi[0]; i1++)
                    for (int c = 0; c < 3; c++) {
                        long a = FN(gidx)(g, c, i1, i2, i3);
                        long o = FN(gidx)(g, c, i1 - sh[0], i2 - sh[1], i3 - sh[2]);
                        if (add) {
                            R v = f[a] + f[o];
                            f[o] = v;
                            f[a] = v;
                        } else {
                            f[a] = f[o];
                        }
                    }
    }
}

/* 0.5 * dV * sum over the interior of each component squared; out[0..2] = B1..B3 style
 * per-component integrals of f (source/vdf/os-vdf-math.f90:625-736 with pow = 2). */
void FN(ora_field_energy)(int dim, const int *nx, const int *gcl, const int *gcu, const R *f,
                          const double *dx, double *out)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    double dv = 1.0;
    for (int d = 0; d < dim; d++) dv *= dx[d];
    for (int c = 0; c < 3; c++) {
        double s = 0.0;
        for (int i3 = 1; i3 <= g->nx[2]; i3++)
            for (int i2 = 1; i2 <= g->nx[1]; i2++)
                for (int i1 = 1; i1 <= g->nx[0]; i1++) {
                    double v = (double)AT(f, c, i1, i2, i3);
                    s += v * v;
                }
        out[c] = 0.5 * dv * s;
    }
}

/* charge deposit with the particle shape of the given order into rho (one component stored
 * in a 3-component grid at component 0), accumulation in double. */
void FN(ora_deposit_rho)(int dim, int order, const int *nx, const int *gcl, const int *gcu,
                         double *rho, int np, const int *ix, const R *x, const R *q)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    /* spline support starts at 1 - OFFSET: order 1 -> {0,1}, 2 -> {-1,0,1}, 3 -> {-1..2},
     * 4 -> {-2..2}; the same stencil origin as the current deposit */
    int lp;
    switch (order) {
    case 1: lp = 0; break;
    case 2: lp = -1; break;
    case 3: lp = -1; break;
    default: lp = -2; break;
    }
    for (int p = 0; p < np; p++) {
        double w[3][5];
        int ii[3] = {1, 1, 1};
        for (int d = 0; d < dim; d++) {
            double xx = (double)x[dim * p + d];
            ii[d] = ix[dim * p + d];
            ora_spline_weights_f64(order, xx, w[d]);
        }
        for (int d = dim; d < 3; d++) { w[d][0] = 1.0; }
        int n = order + 1;
        int n2 = dim > 1 ? n : 1, n3 = dim > 2 ? n : 1;
        int l2 = dim > 1 ? lp : 0, l3 = dim > 2 ? lp : 0;
        for (int k3 = 0; k3 < n3; k3++)
            for (int k2 = 0; k2 < n2; k2++)
                for (int k1 = 0; k1 < n; k1++) {
                    double wt = (double)q[p] * w[0][k1] * w[1][k2] * w[2][k3];
                    rho[FN(gidx)(g, 0, ii[0] + lp + k1, ii[1] + l2 + k2, ii[2] + l3 + k3)] += wt;
                }
    }
}

#undef AT

/* Separable smoothing in place, filter_2d / filter_3d restated: along axis d (order n = ord[d]
 * > 0, coefficients s[d][0 .. 2n] in R), every line of the array (all points of the other
 * axes, guard cells included) is filtered over [lb + n, ub - n] with a sliding window of the
 * original values: f = o(-n) s(-n); f = f + o(k) s(k), k = -n+1 .. n. */
void FN(ora_smooth)(int dim, const int *nx, const int *gcl, const int *gcu, R *f, const int *ord,
                    const R *coef /* [3][31] */)
{
    FN(ora_grid) g;
    FN(grid_init)(&g, dim, nx, gcl, gcu);
    for (int d = 0; d < dim; d++) {
        const int n = ord[d];
        if (n <= 0) continue;
        const R *s = coef + 31 * d;
        const long st = d == 0 ? 3 : (d == 1 ? 3L * g.size[0] : 3L * g.size[0] * g.size[1]);
        const int len = g.size[d];
        int others[2] = {0, 0}, k = 0;                      /* the other two axes */
        for (int e = 0; e < 3; e++)
            if (e != d && k < 2) others[k++] = e;
        const int n1 = g.size[others[0]], n2 = dim > 2 ? g.size[others[1]] : 1;
        R o[3][63];
        for (int a = 0; a < n1; a++)
            for (int b = 0; b < n2; b++) {
                int pos[3] = {0, 0, 0};
                pos[others[0]] = a;
                if (dim > 2) pos[others[1]] = b;
                const long base = 3L * (pos[0] + (long)g.size[0] * (pos[1] + (long)g.size[1] * pos[2]));
                for (int c = 0; c < 3; c++) {
                    for (int kk = -n; kk < n; kk++) o[c][kk + n] = f[base + c + (n + kk) * st];
                    for (int i = n; i <= len - 1 - n; i++) {
                        o[c][2 * n] = f[base + c + (i + n) * st];
                        R v = o[c][0] * s[0];
                        for (int kk = 1; kk <= 2 * n; kk++) v = v + o[c][kk] * s[kk];
                        for (int kk = 0; kk < 2 * n; kk++) o[c][kk] = o[c][kk + 1];
                        f[base + c + i * st] = v;
                    }
                }
            }
    }
}

/* smoothing applied after the current fold by the step below (order 0: none) */
static int FN(step_smooth_ord)[3] = {0, 0, 0};
static R FN(step_smooth_coef)[3 * 31];
void FN(ora_set_smooth)(const int *ord, const R *coef)
{
    for (int d = 0; d < 3; d++) FN(step_smooth_ord)[d] = ord ? ord[d] : 0;
    if (coef)
        for (int i = 0; i < 3 * 31; i++) FN(step_smooth_coef)[i] = coef[i];
}

#undef FN
