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
void FN(ora_periodic_skip)(int dim, const int *nx, const int *gcl, const int *gcu, R *f,
                           int add, int skip)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    for (int d = 0; d < dim; d++) {
        if (skip & (1 << d)) continue;
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

void FN(ora_periodic)(int dim, const int *nx, const int *gcl, const int *gcu, R *f, int add)
{
    FN(ora_periodic_skip)(dim, nx, gcl, gcu, f, add, 0);
}

/* Perfectly conducting walls bounding the axes in `walls` (bit d), restated from the
 * reference's tables (pec_bc_e/b_{1,2,3}d_odd/even, source/emf/boundary/os-emf-pec.f90;
 * spec_bc_{1,2,3}d, source/current/os-current-boundary.f03) as the image rule they follow:
 * along d a component sits at i - 1/2 (odd order) or i (even) when staggered along d (E_d,
 * J_d; B_c for c != d), else at i - 1 (odd) or i - 1/2 (even); its image is the point mirrored
 * about the wall (x_d = 0 below, x_d = nx_d above) with sign + for normal E and tangential
 * B, J and - for tangential E and normal B, J.  kind 0 (E) and 1 (B) set the guard points
 * from their images; kind 2 (J) adds the guard values into their images.  A point on the wall
 * is its own image: set with sign - zeroes it; add doubles it (+) or zeroes it (-).  Axes in
 * order, the lower wall before the upper, lines over the full extent of the other axes. */
static int FN(wall_mirror)(int i, int nx, int lower, int stag, int odd)
{
    if (lower) return stag ? (odd ? 1 - i : -i) : (odd ? 2 - i : 1 - i);
    return stag ? (odd ? 2 * nx + 1 - i : 2 * nx - i) : (odd ? 2 * nx + 2 - i : 2 * nx + 1 - i);
}

void FN(ora_walls)(int dim, const int *nx, const int *gcl, const int *gcu, R *f, int kind,
                   int walls, int order)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    const int odd = order & 1;
    /* kinds 3 and 4: E and B of a perfect magnetic conductor (pmc_bc_e/b_*d_odd/even,
     * source/emf/boundary/os-emf-pmc.f90), the same image points with the signs exchanged */
    const int fk = kind >= 3 ? kind - 3 : kind;
    const R flip = kind >= 3 ? K(-1.0) : K(1.0);
    for (int d = 0; d < dim; d++) {
        if (!(walls & (1 << d))) continue;
        const int n = g->nx[d];
        for (int side = 0; side < 2; side++) {
            const int lower = side == 0;
            int lo[3], hi[3];
            for (int a = 0; a < 3; a++) {
                if (a == d || a >= dim) {
                    lo[a] = hi[a] = 1;
                } else {
                    lo[a] = 1 - g->gcl[a];
                    hi[a] = g->nx[a] + g->gcu[a];
                }
            }
            const int i0 = lower ? 1 - g->gcl[d] : n + 1, i1 = lower ? 0 : n + g->gcu[d];
            for (int a3 = lo[2]; a3 <= hi[2]; a3++)
                for (int a2 = lo[1]; a2 <= hi[1]; a2++)
                    for (int a1 = lo[0]; a1 <= hi[0]; a1++)
                        for (int c = 0; c < 3; c++) {
                            const int normal = c == d;
                            const int stag = fk == 1 ? !normal : normal;
                            const R sg = (((fk == 0) == normal) ? K(1.0) : K(-1.0)) * flip;
                            int ic[3] = {a1, a2, a3};
                            for (int i = i0; i <= i1; i++) {
                                ic[d] = i;
                                const long pg = FN(gidx)(g, c, ic[0], ic[1], ic[2]);
                                const int m = FN(wall_mirror)(i, n, lower, stag, odd);
                                if (m == i) {
                                    f[pg] = fk == 2 ? (sg > 0 ? K(2.0) * f[pg] : K(0.0))
                                                      : (sg > 0 ? f[pg] : K(0.0));
                                    continue;
                                }
                                ic[d] = m;
                                const long pm = FN(gidx)(g, c, ic[0], ic[1], ic[2]);
                                if (fk == 2)
                                    f[pm] = f[pm] + sg * f[pg];
                                else
                                    f[pg] = sg * f[pm];
                            }
                            /* the wall point when it is inside the box */
                            const int iw = lower ? ((!stag && odd) ? 1 : -1000000)
                                                 : ((stag && !odd) ? n : -1000000);
                            if (iw != -1000000) {
                                ic[d] = iw;
                                const long pw = FN(gidx)(g, c, ic[0], ic[1], ic[2]);
                                f[pw] = fk == 2 ? (sg > 0 ? K(2.0) * f[pw] : K(0.0))
                                                  : (sg > 0 ? f[pw] : K(0.0));
                            }
                        }
        }
    }
}

/* the Yee advance bounded by conducting walls: the images after every partial step
 * (source/emf/solver/os-emf-solver-yee.f03:556-566) */
/* E (kind 0) or B (1) images of every walled axis in order, the axes in pmc as perfect
 * magnetic conductors */
static void FN(walls_em)(int dim, const int *nx, const int *gcl, const int *gcu, R *f, int kind,
                         int walls, int order, int pmc)
{
    for (int d = 0; d < dim; d++)
        if (walls & (1 << d))
            FN(ora_walls)(dim, nx, gcl, gcu, f, (pmc >> d) & 1 ? kind + 3 : kind, 1 << d, order);
}

static int FN(step_pmc) = 0;
void FN(ora_set_pmc)(int pmc) { FN(step_pmc) = pmc; }

void FN(ora_yee_advance_walls)(int dim, const int *nx, const int *gcl, const int *gcu, R *e,
                               R *b, const R *j, const double *dx, double dt, int walls,
                               int order)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    const int pmc = FN(step_pmc);
    FN(dbdt)(g, b, e, dx, dt / 2.0);
    FN(walls_em)(dim, nx, gcl, gcu, b, 1, walls, order, pmc);
    FN(dedt)(g, e, b, j, dx, dt);
    FN(walls_em)(dim, nx, gcl, gcu, e, 0, walls, order, pmc);
    FN(dbdt)(g, b, e, dx, dt / 2.0);
    FN(walls_em)(dim, nx, gcl, gcu, b, 1, walls, order, pmc);
}

/* Lindman open boundaries at both edges of axis d (p_bc_lindman; the reference admits them
 * along one axis only, source/emf/boundary/os-emf-boundary.f90:316-324), restated from
 * source/emf/boundary/os-emf-lindman.f90.  The state holds, per interior point of the other
 * axes (flat index m, the lower other axis fastest) and for 3 components, five buffer
 * columns along d: slot 0 E at i_d = 0, 1 E at i_d = 1, 2 B at i_d = 0 (the lower wall
 * buffers, range [0, 1], new_lindman :295-300) and 3 E at nx+1, 4 E at nx+2 (the upper one,
 * range [nx, nx+2]); every slot starts at zero (new_wall, source/vdf/os-wall.f90:198-210).
 *   E (after the E step, update_lindman_2d_e :454-535, 3d :604-750): for the two components
 *     other than d, E(0) = S1 + k (S0 - E(1)), then S0 = E(0), S1 = E(1); above,
 *     E(nx+2) = S3 + k (S4 - E(nx+1)), then S3 = E(nx+1), S4 = E(nx+2);
 *     k = (1 - dt/dx_d) / (1 + dt/dx_d) (disp_corr, new_lindman :237-238).
 *   B (after each B half step, update_lindman_2d_b :539-600, 3d :755-857): the lower B
 *     buffer takes the Yee increment of the point i_d = 0 from the grid's E with
 *     dt/dx * 0.5 (dtdxi, :236-241); nothing above.
 *   guard update (update_emfbound_lindman :861-1042, after the buffers' own periodic update
 *     along the other axes, update_boundary_lindman :352-368): E(0) and B(0), and E(nx+1),
 *     all three components, over the full extent of the other axes (guard points from the
 *     buffers' periodic images).  The normal component of a buffer is never written, so
 *     E_d(0) and E_d(nx+1) become 0. */
static int FN(step_open) = -1;
static R *FN(step_lind) = 0;
void FN(ora_set_open)(int axis, R *state)
{
    FN(step_open) = axis;
    FN(step_lind) = state;
}

static void FN(lind_axes)(const FN(ora_grid) *g, int d, int *pa, int *pb)
{
    int k = 0, o[2] = {3, 3};
    for (int a = 0; a < g->dim; a++)
        if (a != d) o[k++] = a;
    *pa = o[0];
    *pb = o[1];
}

#define LS(st, s, m, c) (st)[3 * ((long)(s) * nperp + (m)) + (c)]

static long FN(lind_nperp)(const FN(ora_grid) *g, int d)
{
    long n = 1;
    for (int a = 0; a < g->dim; a++)
        if (a != d) n *= g->nx[a];
    return n;
}

/* grid index of component c at coordinate i along d and interior point (ia, ib) */
static long FN(lind_at)(const FN(ora_grid) *g, int d, int pa, int pb, int c, int i, int ia, int ib)
{
    int ic[3] = {1, 1, 1};
    ic[d] = i;
    if (pa < 3) ic[pa] = ia;
    if (pb < 3) ic[pb] = ib;
    return FN(gidx)(g, c, ic[0], ic[1], ic[2]);
}

static void FN(lind_e)(const FN(ora_grid) *g, int d, R *e, R *st, R k)
{
    int pa, pb;
    FN(lind_axes)(g, d, &pa, &pb);
    const long nperp = FN(lind_nperp)(g, d);
    const int na = pa < 3 ? g->nx[pa] : 1, nb = pb < 3 ? g->nx[pb] : 1, n = g->nx[d];
    for (int ib = 1; ib <= nb; ib++)
        for (int ia = 1; ia <= na; ia++) {
            const long m = (ia - 1) + (long)na * (ib - 1);
            for (int c = 0; c < 3; c++) {
                if (c == d) continue;
                const long p0 = FN(lind_at)(g, d, pa, pb, c, 0, ia, ib);
                const long p1 = FN(lind_at)(g, d, pa, pb, c, 1, ia, ib);
                e[p0] = LS(st, 1, m, c) + k * (LS(st, 0, m, c) - e[p1]);
                LS(st, 0, m, c) = e[p0];
                LS(st, 1, m, c) = e[p1];
                const long q1 = FN(lind_at)(g, d, pa, pb, c, n + 1, ia, ib);
                const long q2 = FN(lind_at)(g, d, pa, pb, c, n + 2, ia, ib);
                e[q2] = LS(st, 3, m, c) + k * (LS(st, 4, m, c) - e[q1]);
                LS(st, 3, m, c) = e[q1];
                LS(st, 4, m, c) = e[q2];
            }
        }
}

static void FN(lind_b)(const FN(ora_grid) *g, int d, const R *e, R *st, const double *dx,
                       double dt)
{
    int pa, pb;
    FN(lind_axes)(g, d, &pa, &pb);
    const long nperp = FN(lind_nperp)(g, d);
    const int na = pa < 3 ? g->nx[pa] : 1, nb = pb < 3 ? g->nx[pb] : 1;
    R h[3] = {K(0.0), K(0.0), K(0.0)};
    for (int a = 0; a < g->dim; a++) h[a] = (R)(dt / dx[a]) * K(0.5);
    for (int ib = 1; ib <= nb; ib++)
        for (int ia = 1; ia <= na; ia++) {
            const long m = (ia - 1) + (long)na * (ib - 1);
            int ic[3] = {1, 1, 1};
            ic[d] = 0;
            if (pa < 3) ic[pa] = ia;
            if (pb < 3) ic[pb] = ib;
            /* E_c at the point and one cell up along axis a (a beyond dim: no derivative) */
#define EV(c) e[FN(gidx)(g, c, ic[0], ic[1], ic[2])]
#define EU(c, a) ((a) < g->dim ? e[FN(gidx)(g, c, ic[0] + ((a) == 0), ic[1] + ((a) == 1),     \
                                            ic[2] + ((a) == 2))] : EV(c))
            R *s = &LS(st, 2, m, 0);
            s[0] = s[0] - h[1] * (EU(2, 1) - EV(2)) + h[2] * (EU(1, 2) - EV(1));
            s[1] = s[1] - h[2] * (EU(0, 2) - EV(0)) + h[0] * (EU(2, 0) - EV(2));
            s[2] = s[2] - h[0] * (EU(1, 0) - EV(1)) + h[1] * (EU(0, 1) - EV(0));
#undef EV
#undef EU
        }
}

static void FN(lind_restore)(const FN(ora_grid) *g, int d, R *e, R *b, const R *st)
{
    int pa, pb;
    FN(lind_axes)(g, d, &pa, &pb);
    const long nperp = FN(lind_nperp)(g, d);
    const int na = pa < 3 ? g->nx[pa] : 1, nb = pb < 3 ? g->nx[pb] : 1, n = g->nx[d];
    const int la = pa < 3 ? 1 - g->gcl[pa] : 1, ua = pa < 3 ? na + g->gcu[pa] : 1;
    const int lb = pb < 3 ? 1 - g->gcl[pb] : 1, ub = pb < 3 ? nb + g->gcu[pb] : 1;
    for (int ib = lb; ib <= ub; ib++)
        for (int ia = la; ia <= ua; ia++) {
            const int wa = ((ia - 1) % na + na) % na, wb = ((ib - 1) % nb + nb) % nb;
            const long m = wa + (long)na * wb;
            for (int c = 0; c < 3; c++) {
                e[FN(lind_at)(g, d, pa, pb, c, 0, ia, ib)] = LS(st, 0, m, c);
                b[FN(lind_at)(g, d, pa, pb, c, 0, ia, ib)] = LS(st, 2, m, c);
                e[FN(lind_at)(g, d, pa, pb, c, n + 1, ia, ib)] = LS(st, 3, m, c);
            }
        }
}
#undef LS

/* the Yee advance with Lindman boundaries on axis d (update_boundary_b/e after every partial
 * step, source/emf/solver/os-emf-solver-yee.f03:556-566) */
void FN(ora_yee_advance_open)(int dim, const int *nx, const int *gcl, const int *gcu, R *e,
                              R *b, const R *j, const double *dx, double dt, int d, R *st)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    const R k = (R)((1.0 - dt / dx[d]) / (1.0 + dt / dx[d]));
    FN(dbdt)(g, b, e, dx, dt / 2.0);
    FN(lind_b)(g, d, e, st, dx, dt);
    FN(dedt)(g, e, b, j, dx, dt);
    FN(lind_e)(g, d, e, st, k);
    FN(dbdt)(g, b, e, dx, dt / 2.0);
    FN(lind_b)(g, d, e, st, dx, dt);
}

/* guard update of E and B with Lindman boundaries on axis d: periodic along the others, then
 * the boundary planes from the buffers */
void FN(ora_open_guards)(int dim, const int *nx, const int *gcl, const int *gcu, R *e, R *b,
                         int d, const R *st)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    FN(ora_periodic_skip)(dim, nx, gcl, gcu, e, 0, 1 << d);
    FN(ora_periodic_skip)(dim, nx, gcl, gcu, b, 0, 1 << d);
    FN(lind_restore)(g, d, e, b, st);
}

/* one phase of the Lindman boundaries on axis d (what 0: after the E step, 1: after a B half
 * step with the full dt, 2: the restore of the boundary planes) */
void FN(ora_lindman_phase)(int dim, const int *nx, const int *gcl, const int *gcu, int d,
                           int what, R *e, R *b, R *st, const double *dx, double dt)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    if (what == 0)
        FN(lind_e)(g, d, e, st, (R)((1.0 - dt / dx[d]) / (1.0 + dt / dx[d])));
    else if (what == 1)
        FN(lind_b)(g, d, e, st, dx, dt);
    else
        FN(lind_restore)(g, d, e, b, st);
}

/* PML (Vay's perfectly matched layer, "vpml") at both edges of the axes in a mask of a 2D box,
 * restated from source/emf/boundary/os-emf-vpml.f03 (Cartesian, no diffusion correction).
 * Each PML edge holds a wall of nb cells (vpml_bnd_size, default 8, source/emf/boundary/
 * os-emf-boundary.f90:30) along its axis a, range [2 - nb, 1] below and [nx + 1, nx + nb]
 * above (setup_vpml :361-368: two cells of overlap with the box), over [1 - g1, nt + g2] along
 * the other axis t (new_wall, source/vdf/os-wall.f90:188-195): g1 = max(gcl_t, c - 1),
 * g2 = max(gcu_t, c) with c = nb for the x1 walls when x2 has PML walls too (they cover the
 * corners, setup_vpml :382-398), else 2.  A wall point carries four split components
 * (:440-443): 0 X, 1 Y, 2 ZX (the z part driven by x1 derivatives), 3 ZY (by x2 derivatives).
 *
 * State layout (shared with the device engine): per PML axis a in increasing order, walls
 * (side, field), side 0 lower, 1 upper, field 0 E, 1 B, at base_a + (2 side + field) W_a,
 * W_a = nte_a nb 4 reals, nte_a = nt + g1 + g2; point (iw, it) component c at
 * 4 ((it - 1 + g1) nb + (iw - lo(side))) + c.  Then the attenuation tables of both axes: axis a,
 * table k (0 E lower, 1 E upper, 2 B lower, 3 B upper), coefficient m (0..2) of wall cell n
 * (1..nb) at T + ((4 a + k) 3 + m) nb + n - 1, T the walls' total.
 *
 * Per step: the walls' own periodic update along a periodic t at the guard update
 * (update_boundary_vpml :506-524, update_periodic_wall, source/vdf/os-wall-comm.f90:182-344);
 * after the first B half step the E walls advance (update_e_vpml_2d :598-722: first the
 * interfaces of every wall in setup order -- x1 lower, x1 upper, x2 lower, x2 upper -- then the
 * wall updates); after the E step the B walls likewise (update_b_vpml_2d :1742-1861); nothing
 * after the second B half step (source/emf/boundary/os-emf-boundary.f90:931-935, 1071-1074). */
static int FN(step_pml) = 0, FN(step_pml_nb) = 0;
static R *FN(step_pml_st) = 0;
void FN(ora_set_pml)(int mask, int nb, R *state)
{
    FN(step_pml) = mask;
    FN(step_pml_nb) = nb;
    FN(step_pml_st) = state;
}

typedef struct {
    int mask, nb, nx[2];
    int g1[2], g2[2], nte[2];   /* per wall axis a */
    long W[2], base[2], T;
} FN(pml_desc);

static FN(pml_desc) FN(pml_make)(const FN(ora_grid) *g, int mask, int nb)
{
    FN(pml_desc) P;
    P.mask = mask;
    P.nb = nb;
    long off = 0;
    for (int a = 0; a < 2; a++) {
        const int t = 1 - a;
        P.nx[a] = g->nx[a];
        const int c = (a == 0 && ((mask >> 1) & 1)) ? nb : 2;
        /* along x1 the lower corner count is one more (the reference's rule for a moving
           x1, setup_vpml :371-376, kept whether or not the window moves: the extra guard row
           never reaches the box) */
        const int cl = t == 0 ? c + 1 : c;
        P.g1[a] = g->gcl[t] > cl - 1 ? g->gcl[t] : cl - 1;
        P.g2[a] = g->gcu[t] > c ? g->gcu[t] : c;
        P.nte[a] = g->nx[t] + P.g1[a] + P.g2[a];
        P.W[a] = (long)P.nte[a] * nb * 4;
        P.base[a] = off;
        if ((mask >> a) & 1) off += 4 * P.W[a];
    }
    P.T = off;
    return P;
}

/* 3D PML walls at both edges of the axes in a mask, restated from update_e_x{1,2,3}_3d
 * (:1172-1704), update_b_x{1,2,3}_3d (:2311-2828) and update_interface_x{1,2,3}_3d
 * (:2997-3529).  A wall point holds six split components (:444-446): 2F + s for field component
 * F with s = 0 the part driven by the derivative along the lower of the two other axes (XY, YX,
 * ZX) and s = 1 the other (XZ, YZ, ZY).  Split (F, D) with G the third axis:
 * E_FD += sgn dt/dx_D (B_G(p) - B_G(p - e_D)), sgn = +1 when D follows F cyclically, -1
 * otherwise (the curl); B_FD -= sgn dt/dx_D (E_G(p + e_D) - E_G(p)); B_G / E_G the sum of G's
 * two splits.  Along D = a (the wall's axis) the update is the damped one with a's tables; the
 * walls of a lower axis than a PML axis D extend over D's edge regions (corner priority
 * x1 > x2 > x3, setup_vpml :382-430), where their D splits are damped with D's tables (the
 * corner branches).  The wall of axis a spans [1 - g1, n_t + g2] along each other axis t:
 * g1 = max(gcl_t, c - 1), g2 = max(gcu_t, c), c = nb when t has PML walls and a < t, else 2.
 * State layout: per PML axis a in increasing order, walls (side, field) at base_a + (2 side +
 * field) W_a, W_a = nte_a,t1 nte_a,t2 nb 6 (t1 < t2 the other axes); point (iw, i_t1, i_t2)
 * component c at 6 (((i_t2 - 1 + g1_t2) nte_t1 + i_t1 - 1 + g1_t1) nb + iw - lo(side)) + c;
 * then the tables of all three axes at T: axis x, table k, coefficient m, cell n at
 * T + ((4 x + k) 3 + m) nb + n - 1. */
typedef struct {
    int mask, nb, n[3];
    int g1[3][3], g2[3][3], nte[3][3];   /* [wall axis][other axis] */
    long W[3], base[3], T;
} FN(pml3_desc);

static FN(pml3_desc) FN(pml3_make)(const FN(ora_grid) *g, int mask, int nb)
{
    FN(pml3_desc) P;
    P.mask = mask;
    P.nb = nb;
    long off = 0;
    for (int d = 0; d < 3; d++) P.n[d] = g->nx[d];
    for (int a = 0; a < 3; a++) {
        long w = (long)nb * 6;
        for (int t = 0; t < 3; t++) {
            const int c = (((mask >> t) & 1) && a < t) ? nb : 2;
            const int cl = t == 0 ? c + 1 : c;   /* as in 2D: one more below along x1 */
            P.g1[a][t] = g->gcl[t] > cl - 1 ? g->gcl[t] : cl - 1;
            P.g2[a][t] = g->gcu[t] > c ? g->gcu[t] : c;
            P.nte[a][t] = g->nx[t] + P.g1[a][t] + P.g2[a][t];
            if (t != a) w *= P.nte[a][t];
        }
        P.W[a] = w;
        P.base[a] = off;
        if ((mask >> a) & 1) off += 4 * w;
    }
    P.T = off;
    return P;
}

static inline long FN(pml3_at)(const FN(pml3_desc) *P, int a, int side, int fld, int c,
                               const int *i)
{
    const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
    const int lo = side == 0 ? 2 - P->nb : P->n[a] + 1;
    return P->base[a] + (2 * side + fld) * P->W[a] +
           6 * ((((long)i[t2] - 1 + P->g1[a][t2]) * P->nte[a][t1] + i[t1] - 1 + P->g1[a][t1]) *
                    P->nb + i[a] - lo) + c;
}

#define P3COEF(x, k, m, nn) st[P.T + ((4 * (x) + (k)) * 3 + (m)) * P.nb + (nn) - 1]

/* the interfaces of the walls of axis a with the box (the box into the first split over
 * [1, n + 1] of the other axes, the second split 0; the wall's sums into the box over
 * [0, n + 2]), then their contacts with the walls of the higher PML axes: below, the other wall
 * takes this wall's plane 0 and gives it plane 1; above, this wall takes plane n_a + 1 and
 * gives n_a + 2, over the other wall's edge rows along its axis and, along the remaining axis,
 * [1 - g1, n + g2] of this wall for the x1 walls' x2 contacts, else [1, n + 1] */
static void FN(pml3_iface)(const FN(ora_grid) *g, const FN(pml3_desc) *Pp, R *st, R *f, int fld,
                           int a)
{
    const FN(pml3_desc) P = *Pp;
    const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
    for (int side = 0; side < 2; side++) {
        const int lo = side == 0 ? 2 - P.nb : P.n[a] + 1, hi = lo + P.nb - 1;
        const int to_w = side == 0 ? hi : lo, to_b = side == 0 ? hi - 1 : lo + 1;
        int i[3];
        i[a] = to_w;
        for (i[t2] = 1; i[t2] <= P.n[t2] + 1; i[t2]++)
            for (i[t1] = 1; i[t1] <= P.n[t1] + 1; i[t1]++)
                for (int F = 0; F < 3; F++) {
                    st[FN(pml3_at)(&P, a, side, fld, 2 * F, i)] = f[FN(gidx)(g, F, i[0], i[1], i[2])];
                    st[FN(pml3_at)(&P, a, side, fld, 2 * F + 1, i)] = K(0.0);
                }
        i[a] = to_b;
        for (i[t2] = 0; i[t2] <= P.n[t2] + 2; i[t2]++)
            for (i[t1] = 0; i[t1] <= P.n[t1] + 2; i[t1]++)
                for (int F = 0; F < 3; F++)
                    f[FN(gidx)(g, F, i[0], i[1], i[2])] = st[FN(pml3_at)(&P, a, side, fld, 2 * F, i)] +
                                                          st[FN(pml3_at)(&P, a, side, fld, 2 * F + 1, i)];
        for (int d = a + 1; d < 3; d++) {
            if (!((P.mask >> d) & 1)) continue;
            const int o = 3 - a - d;   /* the remaining axis */
            const int olo = (a == 0 && d == 1) ? 1 - P.g1[a][o] : 1;
            const int ohi = (a == 0 && d == 1) ? P.n[o] + P.g2[a][o] : P.n[o] + 1;
            for (int adj = 0; adj < 2; adj++) {
                const int r0 = adj == 0 ? 2 - P.nb : P.n[d] + 2, r1 = adj == 0 ? 0 : P.n[d] + P.nb;
                for (i[d] = r0; i[d] <= r1; i[d]++)
                    for (i[o] = olo; i[o] <= ohi; i[o]++)
                        for (int c = 0; c < 6; c++) {
                            if (side == 0) {
                                i[a] = 0;
                                st[FN(pml3_at)(&P, d, adj, fld, c, i)] = st[FN(pml3_at)(&P, a, 0, fld, c, i)];
                                i[a] = 1;
                                st[FN(pml3_at)(&P, a, 0, fld, c, i)] = st[FN(pml3_at)(&P, d, adj, fld, c, i)];
                            } else {
                                i[a] = P.n[a] + 1;
                                st[FN(pml3_at)(&P, a, 1, fld, c, i)] = st[FN(pml3_at)(&P, d, adj, fld, c, i)];
                                i[a] = P.n[a] + 2;
                                st[FN(pml3_at)(&P, d, adj, fld, c, i)] = st[FN(pml3_at)(&P, a, 1, fld, c, i)];
                            }
                        }
            }
        }
    }
}

/* one E (fld 0) or B (fld 1) update of the walls of axis a */
static void FN(pml3_update)(const FN(pml3_desc) *Pp, R *st, const double *dx, double dt, int fld,
                            int a)
{
    const FN(pml3_desc) P = *Pp;
    const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
    const int src = 1 - fld;
    for (int side = 0; side < 2; side++) {
        const int lo = side == 0 ? 2 - P.nb : P.n[a] + 1, hi = lo + P.nb - 1;
        const int r0 = fld == 0 ? lo + 1 : (side == 0 ? lo : lo + 1);
        const int r1 = fld == 0 ? (side == 0 ? hi - 1 : hi) : hi - 1;
        const int k = fld == 0 ? side : 2 + side;
        const int cofs = side == 0 ? (fld == 0 ? lo - 1 : lo - 2) : lo;
        const int t0 = fld == 0 ? 2 : 1, te = fld == 0 ? 0 : -1;   /* transverse ranges */
        int i[3];
        for (i[t2] = t0 - P.g1[a][t2]; i[t2] <= P.n[t2] + P.g2[a][t2] + te; i[t2]++)
            for (i[t1] = t0 - P.g1[a][t1]; i[t1] <= P.n[t1] + P.g2[a][t1] + te; i[t1]++)
                for (i[a] = r0; i[a] <= r1; i[a]++) {
                    const int ci = i[a] - cofs;
                    for (int F = 0; F < 3; F++)
                        for (int sp = 0; sp < 2; sp++) {
                            const int o1 = F == 0 ? 1 : 0, o2 = F == 2 ? 1 : 2;
                            const int D = sp == 0 ? o1 : o2, G = 3 - F - D;
                            /* E: +1 when D follows F cyclically; B: the opposite */
                            const int cyc = D == (F + 1) % 3;
                            const int sgn = fld == 0 ? (cyc ? 1 : -1) : (cyc ? -1 : 1);
                            int qa[3] = {i[0], i[1], i[2]}, qb[3] = {i[0], i[1], i[2]};
                            if (fld == 0) qb[D] -= 1;
                            else qa[D] += 1;
                            R *v = &st[FN(pml3_at)(&P, a, side, fld, 2 * F + sp, i)];
                            /* damped along D: the wall's own axis, or an edge region of a higher
                               PML axis D */
                            int dk = -1, dn = 0;
                            if (D == a) {
                                dk = k;
                                dn = ci;
                            } else if (((P.mask >> D) & 1) && a < D) {
                                if (i[D] <= 0) {
                                    dk = fld == 0 ? 0 : 2;
                                    dn = i[D] + P.g1[a][D] + (fld == 0 ? 0 : 1);
                                } else if (i[D] > P.n[D] + 1) {
                                    dk = fld == 0 ? 1 : 3;
                                    dn = i[D] - P.n[D] - 1;
                                }
                            }
                            if (dk >= 0) {
                                const R c1 = P3COEF(D, dk, 0, dn), c2 = P3COEF(D, dk, 1, dn),
                                        c3 = P3COEF(D, dk, 2, dn);
                                const R ga = st[FN(pml3_at)(&P, a, side, src, 2 * G, qa)] +
                                             st[FN(pml3_at)(&P, a, side, src, 2 * G + 1, qa)];
                                const R gb = st[FN(pml3_at)(&P, a, side, src, 2 * G, qb)] +
                                             st[FN(pml3_at)(&P, a, side, src, 2 * G + 1, qb)];
                                if (sgn > 0) *v = c1 * *v + c2 * ga - c3 * gb;
                                else *v = c1 * *v - c2 * ga + c3 * gb;
                            } else {
                                const R dtdx = (R)(dt / dx[D]);
                                const R d = st[FN(pml3_at)(&P, a, side, src, 2 * G, qa)] +
                                            st[FN(pml3_at)(&P, a, side, src, 2 * G + 1, qa)] -
                                            st[FN(pml3_at)(&P, a, side, src, 2 * G, qb)] -
                                            st[FN(pml3_at)(&P, a, side, src, 2 * G + 1, qb)];
                                if (sgn > 0) *v = *v + dtdx * d;
                                else *v = *v - dtdx * d;
                            }
                        }
                }
    }
}

/* the walls' periodic update along the periodic other axes (update_periodic_wall; the lower
 * axis first, then the higher over the full extent of the lower) */
static void FN(pml3_wall_guards)(const FN(pml3_desc) *Pp, R *st)
{
    const FN(pml3_desc) P = *Pp;
    for (int a = 0; a < 3; a++) {
        if (!((P.mask >> a) & 1)) continue;
        const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
        for (int side = 0; side < 2; side++) {
            const int lo = side == 0 ? 2 - P.nb : P.n[a] + 1;
            for (int pass = 0; pass < 2; pass++) {
                const int t = pass == 0 ? t1 : t2, o = pass == 0 ? t2 : t1;
                if (((P.mask >> t) & 1) || (t == 0 && ((P.mask >> 3) & 1))) continue;
                for (int fld = 0; fld < 2; fld++) {
                    int i[3], j[3];
                    for (i[a] = lo; i[a] < lo + P.nb; i[a]++)
                        for (i[o] = 1 - P.g1[a][o]; i[o] <= P.n[o] + P.g2[a][o]; i[o]++) {
                            j[a] = i[a];
                            j[o] = i[o];
                            for (i[t] = 1 - P.g1[a][t]; i[t] <= P.n[t] + P.g2[a][t]; i[t]++) {
                                if (i[t] >= 1 && i[t] <= P.n[t]) continue;
                                j[t] = i[t] < 1 ? i[t] + P.n[t] : i[t] - P.n[t];
                                for (int c = 0; c < 6; c++)
                                    st[FN(pml3_at)(&P, a, side, fld, c, i)] =
                                        st[FN(pml3_at)(&P, a, side, fld, c, j)];
                            }
                        }
                }
            }
        }
    }
}
#undef P3COEF

long FN(ora_pml_state_size)(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb)
{
    FN(ora_grid) G;
    FN(grid_init)(&G, dim, nx, gcl, gcu);
    if (dim == 3) return FN(pml3_make)(&G, mask, nb).T + 36L * nb;
    const FN(pml_desc) P = FN(pml_make)(&G, mask, nb);
    return P.T + 24L * nb;
}

static inline int FN(pml_lo)(const FN(pml_desc) *P, int a, int side)
{
    return side == 0 ? 2 - P->nb : P->nx[a] + 1;
}

/* component c of wall (a, side, fld) at box coordinates (i1, i2) (iw along a, it along t) */
#define PWX(a, side, fld, c, i1, i2)                                                           \
    st[P.base[a] + (2 * (side) + (fld)) * P.W[a] +                                            \
       4 * ((long)(((a) == 0 ? (i2) : (i1)) - 1 + P.g1[a]) * P.nb +                           \
            (((a) == 0 ? (i1) : (i2)) - FN(pml_lo)(&P, a, side))) + (c)]
#define PCOEF(a, k, m, n) st[P.T + ((4 * (a) + (k)) * 3 + (m)) * P.nb + (n) - 1]

/* attenuation tables (setup_att_coeff :3586-3684), computed in double and stored in R:
 * t(x) = exp(s1 (s2 x)^4), s1 = -0.8 (n + 1) / 2 with n = 4, s2 = 1 / (nb - 3); the power is
 * taken as an integer power (the reference's exponent is the real constant 4.0, whose base is
 * negative at the interface point of the lower edge).  Tables of both axes are kept. */
void FN(ora_pml_init)(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                      const double *dx, double dt, R *st)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    FN(pml_desc) P = FN(pml_make)(g, mask, nb);
    if (dim == 3) P.T = FN(pml3_make)(g, mask, nb).T;   /* the tables follow the walls */
    for (long i = 0; i < P.T + 12L * dim * nb; i++) st[i] = K(0.0);
    const double s1 = -(0.8 * (4.0 + 1.0)) / 2.0, s2 = 1.0 / (nb - 3);
#define ATT(x) exp(s1 * ((s2 * (x)) * (s2 * (x))) * ((s2 * (x)) * (s2 * (x))))
    for (int a = 0; a < dim; a++) {
        const double dtdx = dt / dx[a], dif = (1.0 - dtdx) / (1.0 + dtdx);
        for (int j = 0; j < nb; j++) {
            /* lower edge: B is the outer point; j = -1/2 is the interface */
            double tj = ATT(j - 0.5), tj12 = ATT((double)j), tj1 = ATT(j + 0.5);
            double b1e = dtdx * (1.0 + dif * (1.0 - tj12)), b1b = dtdx * (1.0 + dif * (1.0 - tj1));
            PCOEF(a, 0, 0, nb - j) = (R)(1.0 - b1e + tj12 * dtdx);
            PCOEF(a, 0, 1, nb - j) = (R)(tj * b1e);
            PCOEF(a, 0, 2, nb - j) = (R)dtdx;
            PCOEF(a, 2, 0, nb - j) = (R)(1.0 - b1b + tj1 * dtdx);
            PCOEF(a, 2, 1, nb - j) = (R)(tj12 * b1b);
            PCOEF(a, 2, 2, nb - j) = (R)dtdx;
            /* upper edge: E is the outer point; j = 0 is the interface */
            tj = ATT((double)j);
            tj12 = ATT(j + 0.5);
            tj1 = ATT(j + 1.0);
            b1e = dtdx * (1.0 + dif * (1.0 - tj12));
            b1b = dtdx * (1.0 + dif * (1.0 - tj1));
            PCOEF(a, 1, 0, j + 1) = (R)(1.0 - b1e + tj12 * dtdx);
            PCOEF(a, 1, 1, j + 1) = (R)dtdx;
            PCOEF(a, 1, 2, j + 1) = (R)(tj * b1e);
            PCOEF(a, 3, 0, j + 1) = (R)(1.0 - b1b + tj1 * dtdx);
            PCOEF(a, 3, 1, j + 1) = (R)dtdx;
            PCOEF(a, 3, 2, j + 1) = (R)(tj12 * b1b);
        }
    }
#undef ATT
}

/* interfaces of the walls of axis a with the box for field fld (0 E, 1 B)
 * (update_interface_x1_2d :2880-2993, update_interface_x2_2d :3190-3248): the box's point next
 * to the wall's inner end goes into the wall (ZX takes the box's z, ZY 0), and the wall's point
 * one cell further out goes into the box (z = ZX + ZY), for it = 0 .. nt + 2; then, for the x1
 * walls, the contact columns with the x2 walls over the corner rows (:2945-2988) */
static void FN(pml_iface)(const FN(ora_grid) *g, const FN(pml_desc) *Pp, R *st, R *f, int fld,
                          int a)
{
    const FN(pml_desc) P = *Pp;
    const int t = 1 - a, nt = P.nx[t];
    for (int side = 0; side < 2; side++) {
        const int lo = FN(pml_lo)(&P, a, side), hi = lo + P.nb - 1;
        const int to_w = side == 0 ? hi : lo, to_b = side == 0 ? hi - 1 : lo + 1;
        for (int it = 0; it <= nt + 2; it++) {
            const int w1 = a == 0 ? to_w : it, w2 = a == 0 ? it : to_w;
            for (int c = 0; c < 3; c++) PWX(a, side, fld, c, w1, w2) = f[FN(gidx)(g, c, w1, w2, 1)];
            PWX(a, side, fld, 3, w1, w2) = K(0.0);
        }
        for (int it = 0; it <= nt + 2; it++) {
            const int b1 = a == 0 ? to_b : it, b2 = a == 0 ? it : to_b;
            f[FN(gidx)(g, 0, b1, b2, 1)] = PWX(a, side, fld, 0, b1, b2);
            f[FN(gidx)(g, 1, b1, b2, 1)] = PWX(a, side, fld, 1, b1, b2);
            f[FN(gidx)(g, 2, b1, b2, 1)] = PWX(a, side, fld, 2, b1, b2) + PWX(a, side, fld, 3, b1, b2);
        }
        if (a == 0 && ((P.mask >> 1) & 1)) {
            for (int adj = 0; adj < 2; adj++) {
                /* the x2 wall below (rows 2 - nb .. 0) or above (nx2 + 2 .. nx2 + nb) */
                const int r0 = adj == 0 ? 2 - P.nb : P.nx[1] + 2;
                const int r1 = adj == 0 ? 0 : P.nx[1] + P.nb;
                for (int i2 = r0; i2 <= r1; i2++)
                    for (int c = 0; c < 4; c++) {
                        if (side == 0) {
                            PWX(1, adj, fld, c, 0, i2) = PWX(0, 0, fld, c, 0, i2);
                            PWX(0, 0, fld, c, 1, i2) = PWX(1, adj, fld, c, 1, i2);
                        } else {
                            const int i1 = P.nx[0] + 1;
                            PWX(0, 1, fld, c, i1, i2) = PWX(1, adj, fld, c, i1, i2);
                            PWX(1, adj, fld, c, i1 + 1, i2) = PWX(0, 1, fld, c, i1 + 1, i2);
                        }
                    }
            }
        }
    }
}

/* the E walls of axis a (update_e_x1_2d :925-1048 with its corner branch, update_e_x2_2d
 * :1369-1456) */
static void FN(pml_e)(const FN(pml_desc) *Pp, R *st, const double *dx, double dt, int a)
{
    const FN(pml_desc) P = *Pp;
    const int t = 1 - a, nt = P.nx[t];
    const R dtdx = (R)(dt / dx[t]);
    const int cor = a == 0 && ((P.mask >> 1) & 1);
    for (int side = 0; side < 2; side++) {
        const int lo = FN(pml_lo)(&P, a, side), hi = lo + P.nb - 1;
        const int r0 = lo + 1, r1 = side == 0 ? hi - 1 : hi;
        const int k = side == 0 ? 0 : 1, cofs = side == 0 ? lo - 1 : lo;
        if (a == 0) {
            for (int i2 = 2 - P.g1[0]; i2 <= nt + P.g2[0]; i2++) {
                /* corner rows (x2 walls below or above): damped along x2 as well */
                int cn = 0, ck = 0;
                if (cor && i2 <= 0) {
                    cn = i2 + P.g1[0];
                    ck = 0;
                } else if (cor && i2 > nt + 1) {
                    cn = i2 - nt - 1;
                    ck = 1;
                }
                for (int i1 = r0; i1 <= r1; i1++) {
                    const int ci = i1 - cofs;
                    const R c1 = PCOEF(0, k, 0, ci), c2 = PCOEF(0, k, 1, ci), c3 = PCOEF(0, k, 2, ci);
                    if ((P.mask >> 4) & 1) {
                        /* correction against noise from particles reaching the wall: the two
                           parts of B_z exchange 10% (p_difrate) at the point, before its E */
                        const R bzx = PWX(0, side, 1, 2, i1, i2);
                        PWX(0, side, 1, 2, i1, i2) = (K(1.0) - K(0.1)) * PWX(0, side, 1, 2, i1, i2) +
                                                     K(0.1) * PWX(0, side, 1, 3, i1, i2);
                        PWX(0, side, 1, 3, i1, i2) = (K(1.0) - K(0.1)) * PWX(0, side, 1, 3, i1, i2) +
                                                     K(0.1) * bzx;
                    }
                    if (cn) {
                        const R d1 = PCOEF(1, ck, 0, cn), d2 = PCOEF(1, ck, 1, cn), d3 = PCOEF(1, ck, 2, cn);
                        PWX(0, side, 0, 0, i1, i2) = d1 * PWX(0, side, 0, 0, i1, i2) +
                            d2 * (PWX(0, side, 1, 2, i1, i2) + PWX(0, side, 1, 3, i1, i2)) -
                            d3 * (PWX(0, side, 1, 2, i1, i2 - 1) + PWX(0, side, 1, 3, i1, i2 - 1));
                        PWX(0, side, 0, 3, i1, i2) = d1 * PWX(0, side, 0, 3, i1, i2) -
                            d2 * PWX(0, side, 1, 0, i1, i2) + d3 * PWX(0, side, 1, 0, i1, i2 - 1);
                    } else {
                        PWX(0, side, 0, 0, i1, i2) = PWX(0, side, 0, 0, i1, i2) +
                            dtdx * (PWX(0, side, 1, 2, i1, i2) + PWX(0, side, 1, 3, i1, i2) -
                                    PWX(0, side, 1, 2, i1, i2 - 1) - PWX(0, side, 1, 3, i1, i2 - 1));
                        PWX(0, side, 0, 3, i1, i2) = PWX(0, side, 0, 3, i1, i2) -
                            dtdx * (PWX(0, side, 1, 0, i1, i2) - PWX(0, side, 1, 0, i1, i2 - 1));
                    }
                    PWX(0, side, 0, 1, i1, i2) = c1 * PWX(0, side, 0, 1, i1, i2) -
                        c2 * (PWX(0, side, 1, 2, i1, i2) + PWX(0, side, 1, 3, i1, i2)) +
                        c3 * (PWX(0, side, 1, 2, i1 - 1, i2) + PWX(0, side, 1, 3, i1 - 1, i2));
                    PWX(0, side, 0, 2, i1, i2) = c1 * PWX(0, side, 0, 2, i1, i2) +
                        c2 * PWX(0, side, 1, 1, i1, i2) - c3 * PWX(0, side, 1, 1, i1 - 1, i2);
                }
            }
        } else {
            if ((P.mask >> 5) & 1)   /* the diffusion correction over the update range first */
                for (int i2 = r0; i2 <= r1; i2++)
                    for (int i1 = 2 - P.g1[1]; i1 <= nt + P.g2[1]; i1++) {
                        const R bzx = PWX(1, side, 1, 2, i1, i2);
                        PWX(1, side, 1, 2, i1, i2) = (K(1.0) - K(0.1)) * PWX(1, side, 1, 2, i1, i2) +
                                                     K(0.1) * PWX(1, side, 1, 3, i1, i2);
                        PWX(1, side, 1, 3, i1, i2) = (K(1.0) - K(0.1)) * PWX(1, side, 1, 3, i1, i2) +
                                                     K(0.1) * bzx;
                    }
            /* the wall's lowest row: Y and ZX by the plain Yee update */
            for (int i1 = 2 - P.g1[1]; i1 <= nt + P.g2[1]; i1++) {
                const int i2 = lo;
                PWX(1, side, 0, 1, i1, i2) = PWX(1, side, 0, 1, i1, i2) -
                    dtdx * (PWX(1, side, 1, 2, i1, i2) + PWX(1, side, 1, 3, i1, i2) -
                            PWX(1, side, 1, 2, i1 - 1, i2) - PWX(1, side, 1, 3, i1 - 1, i2));
                PWX(1, side, 0, 2, i1, i2) = PWX(1, side, 0, 2, i1, i2) +
                    dtdx * (PWX(1, side, 1, 1, i1, i2) - PWX(1, side, 1, 1, i1 - 1, i2));
            }
            for (int i2 = r0; i2 <= r1; i2++) {
                const int ci = i2 - cofs;
                const R c1 = PCOEF(1, k, 0, ci), c2 = PCOEF(1, k, 1, ci), c3 = PCOEF(1, k, 2, ci);
                for (int i1 = 2 - P.g1[1]; i1 <= nt + P.g2[1]; i1++) {
                    PWX(1, side, 0, 0, i1, i2) = c1 * PWX(1, side, 0, 0, i1, i2) +
                        c2 * (PWX(1, side, 1, 2, i1, i2) + PWX(1, side, 1, 3, i1, i2)) -
                        c3 * (PWX(1, side, 1, 2, i1, i2 - 1) + PWX(1, side, 1, 3, i1, i2 - 1));
                    PWX(1, side, 0, 1, i1, i2) = PWX(1, side, 0, 1, i1, i2) -
                        dtdx * (PWX(1, side, 1, 2, i1, i2) + PWX(1, side, 1, 3, i1, i2) -
                                PWX(1, side, 1, 2, i1 - 1, i2) - PWX(1, side, 1, 3, i1 - 1, i2));
                    PWX(1, side, 0, 2, i1, i2) = PWX(1, side, 0, 2, i1, i2) +
                        dtdx * (PWX(1, side, 1, 1, i1, i2) - PWX(1, side, 1, 1, i1 - 1, i2));
                    PWX(1, side, 0, 3, i1, i2) = c1 * PWX(1, side, 0, 3, i1, i2) -
                        c2 * PWX(1, side, 1, 0, i1, i2) + c3 * PWX(1, side, 1, 0, i1, i2 - 1);
                }
            }
        }
    }
}

/* the B walls of axis a (update_b_x1_2d :2066-2177 with its corner branch, update_b_x2_2d
 * :2512-2579) */
static void FN(pml_b)(const FN(pml_desc) *Pp, R *st, const double *dx, double dt, int a)
{
    const FN(pml_desc) P = *Pp;
    const int t = 1 - a, nt = P.nx[t];
    const R dtdx = (R)(dt / dx[t]);
    const int cor = a == 0 && ((P.mask >> 1) & 1);
    for (int side = 0; side < 2; side++) {
        const int lo = FN(pml_lo)(&P, a, side), hi = lo + P.nb - 1;
        const int r0 = side == 0 ? lo : lo + 1, r1 = hi - 1;
        const int k = side == 0 ? 2 : 3, cofs = side == 0 ? lo - 2 : lo;
        if (a == 0) {
            for (int i2 = 1 - P.g1[0]; i2 <= nt + P.g2[0] - 1; i2++) {
                int cn = 0, ck = 0;
                if (cor && i2 <= 0) {
                    cn = i2 + P.g1[0] + 1;
                    ck = 2;
                } else if (cor && i2 > nt + 1) {
                    cn = i2 - nt - 1;
                    ck = 3;
                }
                for (int i1 = r0; i1 <= r1; i1++) {
                    const int ci = i1 - cofs;
                    const R c1 = PCOEF(0, k, 0, ci), c2 = PCOEF(0, k, 1, ci), c3 = PCOEF(0, k, 2, ci);
                    if (cn) {
                        const R d1 = PCOEF(1, ck, 0, cn), d2 = PCOEF(1, ck, 1, cn), d3 = PCOEF(1, ck, 2, cn);
                        PWX(0, side, 1, 0, i1, i2) = d1 * PWX(0, side, 1, 0, i1, i2) -
                            d2 * (PWX(0, side, 0, 2, i1, i2 + 1) + PWX(0, side, 0, 3, i1, i2 + 1)) +
                            d3 * (PWX(0, side, 0, 2, i1, i2) + PWX(0, side, 0, 3, i1, i2));
                        PWX(0, side, 1, 3, i1, i2) = d1 * PWX(0, side, 1, 3, i1, i2) +
                            d2 * PWX(0, side, 0, 0, i1, i2 + 1) - d3 * PWX(0, side, 0, 0, i1, i2);
                    } else {
                        PWX(0, side, 1, 0, i1, i2) = PWX(0, side, 1, 0, i1, i2) -
                            dtdx * (PWX(0, side, 0, 2, i1, i2 + 1) + PWX(0, side, 0, 3, i1, i2 + 1) -
                                    PWX(0, side, 0, 2, i1, i2) - PWX(0, side, 0, 3, i1, i2));
                        PWX(0, side, 1, 3, i1, i2) = PWX(0, side, 1, 3, i1, i2) +
                            dtdx * (PWX(0, side, 0, 0, i1, i2 + 1) - PWX(0, side, 0, 0, i1, i2));
                    }
                    PWX(0, side, 1, 1, i1, i2) = c1 * PWX(0, side, 1, 1, i1, i2) +
                        c2 * (PWX(0, side, 0, 2, i1 + 1, i2) + PWX(0, side, 0, 3, i1 + 1, i2)) -
                        c3 * (PWX(0, side, 0, 2, i1, i2) + PWX(0, side, 0, 3, i1, i2));
                    PWX(0, side, 1, 2, i1, i2) = c1 * PWX(0, side, 1, 2, i1, i2) -
                        c2 * PWX(0, side, 0, 1, i1 + 1, i2) + c3 * PWX(0, side, 0, 1, i1, i2);
                }
            }
        } else {
            for (int i2 = r0; i2 <= r1; i2++) {
                const int ci = i2 - cofs;
                const R c1 = PCOEF(1, k, 0, ci), c2 = PCOEF(1, k, 1, ci), c3 = PCOEF(1, k, 2, ci);
                for (int i1 = 1 - P.g1[1]; i1 <= nt + P.g2[1] - 1; i1++) {
                    PWX(1, side, 1, 0, i1, i2) = c1 * PWX(1, side, 1, 0, i1, i2) -
                        c2 * (PWX(1, side, 0, 2, i1, i2 + 1) + PWX(1, side, 0, 3, i1, i2 + 1)) +
                        c3 * (PWX(1, side, 0, 2, i1, i2) + PWX(1, side, 0, 3, i1, i2));
                    PWX(1, side, 1, 1, i1, i2) = PWX(1, side, 1, 1, i1, i2) +
                        dtdx * (PWX(1, side, 0, 2, i1 + 1, i2) + PWX(1, side, 0, 3, i1 + 1, i2) -
                                PWX(1, side, 0, 2, i1, i2) - PWX(1, side, 0, 3, i1, i2));
                    PWX(1, side, 1, 2, i1, i2) = PWX(1, side, 1, 2, i1, i2) -
                        dtdx * (PWX(1, side, 0, 1, i1 + 1, i2) - PWX(1, side, 0, 1, i1, i2));
                    PWX(1, side, 1, 3, i1, i2) = c1 * PWX(1, side, 1, 3, i1, i2) +
                        c2 * PWX(1, side, 0, 0, i1, i2 + 1) - c3 * PWX(1, side, 0, 0, i1, i2);
                }
            }
            /* the wall's highest row: Y and ZX by the plain Yee update */
            for (int i1 = 1 - P.g1[1]; i1 <= nt + P.g2[1] - 1; i1++) {
                const int i2 = hi;
                PWX(1, side, 1, 1, i1, i2) = PWX(1, side, 1, 1, i1, i2) +
                    dtdx * (PWX(1, side, 0, 2, i1 + 1, i2) + PWX(1, side, 0, 3, i1 + 1, i2) -
                            PWX(1, side, 0, 2, i1, i2) - PWX(1, side, 0, 3, i1, i2));
                PWX(1, side, 1, 2, i1, i2) = PWX(1, side, 1, 2, i1, i2) -
                    dtdx * (PWX(1, side, 0, 1, i1 + 1, i2) - PWX(1, side, 0, 1, i1, i2));
            }
        }
    }
}

/* the walls' periodic update along t, when t is periodic (no PML walls along it): guard points
 * from the opposite interior points, all four components, the whole wall-normal range */
static void FN(pml_wall_guards)(const FN(pml_desc) *Pp, R *st)
{
    const FN(pml_desc) P = *Pp;
    for (int a = 0; a < 2; a++) {
        const int t = 1 - a, nt = P.nx[t];
        if (!((P.mask >> a) & 1) || ((P.mask >> t) & 1) || (t == 0 && ((P.mask >> 3) & 1)))
            continue;
        for (int side = 0; side < 2; side++) {
            const int lo = FN(pml_lo)(&P, a, side);
            for (int fld = 0; fld < 2; fld++)
                for (int iw = lo; iw < lo + P.nb; iw++)
                    for (int c = 0; c < 4; c++) {
                        for (int it = 1 - P.g1[a]; it <= 0; it++) {
                            if (a == 0) PWX(0, side, fld, c, iw, it) = PWX(0, side, fld, c, iw, it + nt);
                            else PWX(1, side, fld, c, it, iw) = PWX(1, side, fld, c, it + nt, iw);
                        }
                        for (int it = nt + 1; it <= nt + P.g2[a]; it++) {
                            if (a == 0) PWX(0, side, fld, c, iw, it) = PWX(0, side, fld, c, iw, it - nt);
                            else PWX(1, side, fld, c, it, iw) = PWX(1, side, fld, c, it - nt, iw);
                        }
                    }
        }
    }
}

/* one PML phase (what 0: the walls' guard update, 1: E walls after the first B half step,
 * interfaces with B first, 2: B walls after the E step, interfaces with E first) */
void FN(ora_pml_phase)(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                       int what, R *e, R *b, R *st, const double *dx, double dt)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    if (dim == 3) {
        const FN(pml3_desc) Q = FN(pml3_make)(g, mask, nb);
        if (what == 0) {
            FN(pml3_wall_guards)(&Q, st);
            return;
        }
        /* the interfaces of every wall in setup order (x1, x2, x3), then the wall updates */
        for (int a = 0; a < 3; a++)
            if ((mask >> a) & 1) FN(pml3_iface)(g, &Q, st, what == 1 ? b : e, what == 1 ? 1 : 0, a);
        for (int a = 0; a < 3; a++)
            if ((mask >> a) & 1) FN(pml3_update)(&Q, st, dx, dt, what == 1 ? 0 : 1, a);
        return;
    }
    const FN(pml_desc) P = FN(pml_make)(g, mask, nb);
    if (what == 0) {
        FN(pml_wall_guards)(&P, st);
        return;
    }
    for (int a = 0; a < 2; a++)
        if ((mask >> a) & 1) FN(pml_iface)(g, &P, st, what == 1 ? b : e, what == 1 ? 1 : 0, a);
    for (int a = 0; a < 2; a++) {
        if (!((mask >> a) & 1)) continue;
        if (what == 1) FN(pml_e)(&P, st, dx, dt, a);
        else FN(pml_b)(&P, st, dx, dt, a);
    }
}
#undef PWX
#undef PCOEF

/* window move: the walls of the axes other than x1 shift one cell down along x1, all
 * components, the last x1 plane becoming zero (move_window_vpml :478-494, move_window_wall,
 * source/vdf/os-wall-comm.f90:57-176) */
void FN(ora_pml_shift_x)(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                         R *st)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    if (dim == 2) {
        const FN(pml_desc) P = FN(pml_make)(g, mask, nb);
        if (!((mask >> 1) & 1)) return;
        /* x2 walls: point (iw, it) with it along x1, stride 4 nb */
        for (int w = 0; w < 4; w++) {
            R *f = st + P.base[1] + w * P.W[1];
            const long line = 4L * nb, nl = P.nte[1];
            for (long k = 0; k + 1 < nl; k++)
                for (long c = 0; c < line; c++) f[k * line + c] = f[(k + 1) * line + c];
            for (long c = 0; c < line; c++) f[(nl - 1) * line + c] = K(0.0);
        }
        return;
    }
    const FN(pml3_desc) P = FN(pml3_make)(g, mask, nb);
    for (int a = 1; a < 3; a++) {
        if (!((mask >> a) & 1)) continue;
        /* x1 is the walls' first other axis (t1): stride 6 nb, lines of nte_a,x1 points */
        const int t2 = a == 2 ? 1 : 2;
        const long line = 6L * nb, nl = P.nte[a][0];
        for (int w = 0; w < 4; w++)
            for (long o = 0; o < P.nte[a][t2]; o++) {
                R *f = st + P.base[a] + w * P.W[a] + o * nl * line;
                for (long k = 0; k + 1 < nl; k++)
                    for (long c = 0; c < line; c++) f[k * line + c] = f[(k + 1) * line + c];
                for (long c = 0; c < line; c++) f[(nl - 1) * line + c] = K(0.0);
            }
    }
}

/* the Yee advance with PML walls on the axes in mask */
void FN(ora_yee_advance_pml)(int dim, const int *nx, const int *gcl, const int *gcu, R *e, R *b,
                             const R *j, const double *dx, double dt, int mask, int nb, R *st)
{
    FN(ora_grid) G, *g = &G;
    FN(grid_init)(g, dim, nx, gcl, gcu);
    FN(dbdt)(g, b, e, dx, dt / 2.0);
    FN(ora_pml_phase)(dim, nx, gcl, gcu, mask, nb, 1, e, b, st, dx, dt);
    FN(dedt)(g, e, b, j, dx, dt);
    FN(ora_pml_phase)(dim, nx, gcl, gcu, mask, nb, 2, e, b, st, dx, dt);
    FN(dbdt)(g, b, e, dx, dt / 2.0);
}

/* guard update of E and B with PML walls on the axes in mask: the walls' own periodic update,
 * then the box periodic along the other axes only (along a PML axis its guard points keep what
 * the interfaces and the Yee steps left there, update_boundary_emf_bound,
 * source/emf/boundary/os-emf-boundary.f90:760-820) */
void FN(ora_pml_guards)(int dim, const int *nx, const int *gcl, const int *gcu, R *e, R *b,
                        int mask, int nb, R *st)
{
    const int skip = (mask & 7) | ((mask >> 3) & 1);   /* PML axes, and x1 when it moves */
    FN(ora_pml_phase)(dim, nx, gcl, gcu, mask, nb, 0, e, b, st, 0, 0.0);
    FN(ora_periodic_skip)(dim, nx, gcl, gcu, e, 0, skip);
    FN(ora_periodic_skip)(dim, nx, gcl, gcu, b, 0, skip);
}

/* absorbing particle boundary along axis d (p_bc_absorbing: a particle that left the box is
 * removed after its current was deposited, source/spec/os-spec-boundary.f03:501-511).  Here
 * it stays in the arrays with charge and momentum 0, at offset 0 of the edge cell it left
 * through; later steps still move it but, with charge 0, it deposits nothing. */
void FN(ora_particle_absorb)(int dim, const int *nx, int np, int *ix, R *x, R *u, R *q, int d)
{
    for (int p = 0; p < np; p++) {
        int *c = &ix[dim * p + d];
        if (*c >= 1 && *c <= nx[d]) continue;
        *c = *c < 1 ? 1 : nx[d];
        x[dim * p + d] = K(0.0);
        u[3 * p + 0] = u[3 * p + 1] = u[3 * p + 2] = K(0.0);
        q[p] = K(0.0);
    }
}

/* particle boundary after the push: periodic wrap, or along a walled axis specular
 * reflection (p_bc_specular, source/spec/os-spec-boundary.f03:1293-1310: u_d -> -u_d, the
 * particle to the edge cell at offset -x) */
void FN(ora_particle_bound)(int dim, const int *nx, int np, int *ix, R *x, R *u, int walls)
{
    for (int p = 0; p < np; p++)
        for (int d = 0; d < dim; d++) {
            int *c = &ix[dim * p + d];
            if (walls & (1 << d)) {
                if (*c < 1 || *c > nx[d]) {
                    *c = *c < 1 ? 1 : nx[d];
                    x[dim * p + d] = -x[dim * p + d];
                    u[3 * p + d] = -u[3 * p + d];
                }
            } else if (*c < 1) {
                *c += nx[d];
            } else if (*c > nx[d]) {
                *c -= nx[d];
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

/* conducting walls of the step below (bit d: axis d walled; 0: periodic box) */
static int FN(step_walls) = 0;
void FN(ora_set_walls)(int walls) { FN(step_walls) = walls; }

/* moving window along x1 for the step below (0: periodic x1): no guard update of E, B or J
 * along x1 (the p_bc_move_c boundary of the fields has no neighbour to exchange with,
 * source/emf/boundary/os-emf-boundary.f90:779-820; the current's boundary type is p_bc_none,
 * source/current/os-current-define.f03:240-251); particles are absorbed below cell 1 (:315 of
 * source/spec/os-spec-boundary.f03) and reflected specularly above nx (:1276, 1293-1310) */
static int FN(step_window) = 0;
void FN(ora_set_window)(int on) { FN(step_window) = on ? 1 : 0; }

/* the window's particle boundary along x1 on the pushed particles 1..np: above nx the particle
 * goes to cell nx with x1 and u1 negated; below 1 it is absorbed, marked by a cell index
 * ORA_GONE and zero charge and momentum (the caller removes it) */
#define ORA_GONE (-(1 << 28))
void FN(ora_particle_window)(int dim, const int *nx, int np, int *ix, R *x, R *u, R *q)
{
    for (int p = 0; p < np; p++) {
        int *c = &ix[dim * p];
        if (*c > nx[0]) {
            *c = nx[0];
            x[dim * p] = -x[dim * p];
            u[3 * p] = -u[3 * p];
        } else if (*c < 1) {
            *c = ORA_GONE;
            q[p] = K(0.0);
            u[3 * p] = u[3 * p + 1] = u[3 * p + 2] = K(0.0);
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

/* smoothing of the fields the particles see (e_part, b_part: copies of E and B after their
   guard update, smoothed; update_particle_fld_emf, source/emf/os-emf.f03:1065-1151,
   smooth_type "stand") applied by the step below (order 0: none) */
static int FN(step_esmooth_ord)[3] = {0, 0, 0};
static R FN(step_esmooth_coef)[3 * 31];
void FN(ora_set_emf_smooth)(const int *ord, const R *coef)
{
    for (int d = 0; d < 3; d++) FN(step_esmooth_ord)[d] = ord ? ord[d] : 0;
    if (coef)
        for (int i = 0; i < 3 * 31; i++) FN(step_esmooth_coef)[i] = coef[i];
}

#undef FN
