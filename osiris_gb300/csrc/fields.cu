// fields.cu -- grid kernels of the time step on the reference field layout (3 components
// fastest, guard cells included): Yee B half step / E full step, single-node periodic guard
// fold (current) and replace (fields), and the FP64 diagnostics (field energy, charge density
// deposit, divergence).
//
//   dbdt 2D/3D      source/emf/solver/os-emf-solver-yee.f03:102-138, :211-251
//   dedt 2D/3D      source/emf/solver/os-emf-solver-yee.f03:287-326, :385-428
//   advance_yee     source/emf/solver/os-emf-solver-yee.f03:542-568
//   periodic add / replace   source/vdf/os-vdf-comm.f90:142-326 (one direction per launch,
//                            directions in order as update_boundary_vdf :665-722)
//   field energy    source/emf/diagnostics/os-emf-diagnostics.f03:42-58
//   rho deposit     source/spec/os-spec-charge.f90:500-600
//   divergence      source/vdf/os-vdf-math.f90:1013-1073
#include <cuda_runtime.h>

#include <climits>

#include "common.cuh"
#include "fields.cuh"
#include "pic_math.cuh"

namespace osg {

template <typename T, int DIM>
__device__ __forceinline__ void dbdt_body(const GridDesc &g, const Box &box, T *__restrict__ b,
                                          const T *__restrict__ e, T d1, T d2, T d3)
{
    OSG_GRID_LOOP(n, box.n)
    {
        int i1, i2, i3;
        unflat(n, box.lo, box.ext, i1, i2, i3);
        const long p = pos(g, i1, i2, i3);
        const long sx = 3, sy = g.stride(1), sz = g.stride(2);
        if constexpr (DIM == 2) {
            b[p + 0] = b[p + 0] - d2 * (e[p + sy + 2] - e[p + 2]);
            b[p + 1] = b[p + 1] + d1 * (e[p + sx + 2] - e[p + 2]);
            b[p + 2] = b[p + 2] - d1 * (e[p + sx + 1] - e[p + 1]) + d2 * (e[p + sy + 0] - e[p + 0]);
        } else if constexpr (DIM == 3) {
            b[p + 0] = b[p + 0] - d2 * (e[p + sy + 2] - e[p + 2]) + d3 * (e[p + sz + 1] - e[p + 1]);
            b[p + 1] = b[p + 1] + d1 * (e[p + sx + 2] - e[p + 2]) - d3 * (e[p + sz + 0] - e[p + 0]);
            b[p + 2] = b[p + 2] - d1 * (e[p + sx + 1] - e[p + 1]) + d2 * (e[p + sy + 0] - e[p + 0]);
        } else {
            b[p + 1] = b[p + 1] + d1 * (e[p + sx + 2] - e[p + 2]);
            b[p + 2] = b[p + 2] - d1 * (e[p + sx + 1] - e[p + 1]);
        }
    }
}

template <typename T, int DIM>
__global__ void k_dbdt(GridDesc g, Box box, T *__restrict__ b, const T *__restrict__ e, T d1, T d2,
                       T d3)
{
    dbdt_body<T, DIM>(g, box, b, e, d1, d2, d3);
}

template <typename T, int DIM>
__device__ __forceinline__ void dedt_body(const GridDesc &g, const Box &box, T *__restrict__ e,
                                          const T *__restrict__ b, const T *__restrict__ j, T dti,
                                          T d1, T d2, T d3)
{
    OSG_GRID_LOOP(n, box.n)
    {
        int i1, i2, i3;
        unflat(n, box.lo, box.ext, i1, i2, i3);
        const long p = pos(g, i1, i2, i3);
        const long sx = 3, sy = g.stride(1), sz = g.stride(2);
        if constexpr (DIM == 2) {
            e[p + 0] = e[p + 0] - dti * j[p + 0] + d2 * (b[p + 2] - b[p - sy + 2]);
            e[p + 1] = e[p + 1] - dti * j[p + 1] - d1 * (b[p + 2] - b[p - sx + 2]);
            e[p + 2] = e[p + 2] - dti * j[p + 2] + d1 * (b[p + 1] - b[p - sx + 1]) -
                       d2 * (b[p + 0] - b[p - sy + 0]);
        } else if constexpr (DIM == 3) {
            e[p + 0] = e[p + 0] - dti * j[p + 0] + d2 * (b[p + 2] - b[p - sy + 2]) -
                       d3 * (b[p + 1] - b[p - sz + 1]);
            e[p + 1] = e[p + 1] - dti * j[p + 1] + d3 * (b[p + 0] - b[p - sz + 0]) -
                       d1 * (b[p + 2] - b[p - sx + 2]);
            e[p + 2] = e[p + 2] - dti * j[p + 2] + d1 * (b[p + 1] - b[p - sx + 1]) -
                       d2 * (b[p + 0] - b[p - sy + 0]);
        } else {
            e[p + 0] = e[p + 0] - dti * j[p + 0];
            e[p + 1] = e[p + 1] - dti * j[p + 1] - d1 * (b[p + 2] - b[p - sx + 2]);
            e[p + 2] = e[p + 2] - dti * j[p + 2] + d1 * (b[p + 1] - b[p - sx + 1]);
        }
    }
}

template <typename T, int DIM>
__global__ void k_dedt(GridDesc g, Box box, T *__restrict__ e, const T *__restrict__ b,
                       const T *__restrict__ j, T dti, T d1, T d2, T d3)
{
    dedt_body<T, DIM>(g, box, e, b, j, dti, d1, d2, d3);
}

template <typename T>
static void launch_dbdt(const GridDesc &g, T *b, const T *e, const double *dx, double dt,
                        cudaStream_t st)
{
    Box box = make_box(g, 0, 1);
    const T d1 = (T)(dt / dx[0]), d2 = g.dim > 1 ? (T)(dt / dx[1]) : T(0),
            d3 = g.dim > 2 ? (T)(dt / dx[2]) : T(0);
    const unsigned nb = blocks_for(box.n, 256);
    if (g.dim == 2) k_dbdt<T, 2><<<nb, 256, 0, st>>>(g, box, b, e, d1, d2, d3);
    else if (g.dim == 3) k_dbdt<T, 3><<<nb, 256, 0, st>>>(g, box, b, e, d1, d2, d3);
    else k_dbdt<T, 1><<<nb, 256, 0, st>>>(g, box, b, e, d1, d2, d3);
}

template <typename T>
static void launch_dedt(const GridDesc &g, T *e, const T *b, const T *j, const double *dx,
                        double dt, cudaStream_t st)
{
    Box box = make_box(g, 1, 1);
    const T dti = (T)dt, d1 = (T)(dt / dx[0]), d2 = g.dim > 1 ? (T)(dt / dx[1]) : T(0),
            d3 = g.dim > 2 ? (T)(dt / dx[2]) : T(0);
    const unsigned nb = blocks_for(box.n, 256);
    if (g.dim == 2) k_dedt<T, 2><<<nb, 256, 0, st>>>(g, box, e, b, j, dti, d1, d2, d3);
    else if (g.dim == 3) k_dedt<T, 3><<<nb, 256, 0, st>>>(g, box, e, b, j, dti, d1, d2, d3);
    else k_dedt<T, 1><<<nb, 256, 0, st>>>(g, box, e, b, j, dti, d1, d2, d3);
}

// ------------------------------------------------------------------------ conducting walls
// Image rule of a perfectly conducting wall at the lower (x_d = 0) or upper (x_d = nx_d) edge of
// axis d, for the field E (kind 0) and B (1), whose guard values are set from their mirror
// points, and for the current J (2), whose guard values are added to their mirror points
// (pec_bc_e/b_*d_odd/even, source/emf/boundary/os-emf-pec.f90; spec_bc_*d,
// source/current/os-current-boundary.f03).  Along d a component sits at cell positions i - 1/2
// (odd interpolation order) or i (even) when it is staggered along d (E_d, J_d, and B_c for
// c != d), else at i - 1 (odd) or i - 1/2 (even); its mirror point reflects the position
// about the wall.  The image carries sign + for normal E and tangential B and J, - for
// tangential E and normal B and J.  A point on the wall is its own image: a set with sign -
// zeroes it, an add doubles it (+) or zeroes it (-).  One thread per line along d (the full
// extent of the other axes, guard cells included), so every point of a line is handled in
// order by one thread.
template <typename T>
__device__ __forceinline__ int wall_mirror(int i, int nx, bool lower, bool stag, bool odd)
{
    if (lower) return stag ? (odd ? 1 - i : -i) : (odd ? 2 - i : 1 - i);
    return stag ? (odd ? 2 * nx + 1 - i : 2 * nx - i) : (odd ? 2 * nx + 2 - i : 2 * nx + 1 - i);
}

template <typename T>
__global__ void k_wall_dir(GridDesc g, int d, int side, int kind, int odd, T *__restrict__ f,
                           long nlines)
{
    OSG_GRID_LOOP(n, nlines)
    {
        int lo[3], ext[3];
        for (int a = 0; a < 3; a++) {
            if (a >= g.dim || a == d) {
                lo[a] = a == d ? 0 : 1;
                ext[a] = 1;
            } else {
                lo[a] = 1 - g.gcl[a];
                ext[a] = g.size[a];
            }
        }
        int ic[3];
        unflat(n, lo, ext, ic[0], ic[1], ic[2]);
        const bool lower = side == 0;
        const int nx = g.nx[d];
        const int i0 = lower ? 1 - g.gcl[d] : nx + 1, i1 = lower ? 0 : nx + g.gcu[d];
        // kinds 3 and 4: E and B of a perfect magnetic conductor, the same mirror points with
        // the signs of E and B exchanged (pmc_bc_e/b_*, source/emf/boundary/os-emf-pmc.f90)
        const int fk = kind >= 3 ? kind - 3 : kind;
        const T flip = kind >= 3 ? T(-1) : T(1);
        for (int c = 0; c < 3; c++) {
            const bool normal = c == d;
            const bool stag = fk == 1 ? !normal : normal;
            const T sg = ((fk == 0) == normal ? T(1) : T(-1)) * flip;
            // the wall point, when it is not a guard point (odd order, unstaggered, lower
            // wall: i = 1; even order, staggered, upper wall: i = nx)
            const int iw = lower ? (!stag && odd ? 1 : INT_MIN) : (stag && !odd ? nx : INT_MIN);
            for (int i = i0; i <= i1; i++) {
                ic[d] = i;
                const long pg = pos(g, ic[0], ic[1], ic[2]) + c;
                const int m = wall_mirror<T>(i, nx, lower, stag, odd != 0);
                if (m == i) {
                    f[pg] = kind == 2 ? (sg > T(0) ? T(2) * f[pg] : T(0))
                                      : (sg > T(0) ? f[pg] : T(0));
                    continue;
                }
                ic[d] = m;
                const long pm = pos(g, ic[0], ic[1], ic[2]) + c;
                if (kind == 2)
                    f[pm] += sg * f[pg];
                else
                    f[pg] = sg * f[pm];
            }
            if (iw != INT_MIN) {
                ic[d] = iw;
                const long pw = pos(g, ic[0], ic[1], ic[2]) + c;
                f[pw] = kind == 2 ? (sg > T(0) ? T(2) * f[pw] : T(0)) : (sg > T(0) ? f[pw] : T(0));
            }
        }
    }
}

template <typename T>
void wall_update(const GridDesc &g, T *f, int kind, int walls, int order, cudaStream_t st,
                 int pmc)
{
    for (int d = 0; d < g.dim; d++) {
        if (!(walls & (1 << d))) continue;
        long nlines = 1;
        for (int a = 0; a < g.dim; a++)
            if (a != d) nlines *= g.size[a];
        const int k = (kind < 2 && ((pmc >> d) & 1)) ? kind + 3 : kind;
        for (int side = 0; side < 2; side++)
            k_wall_dir<T><<<blocks_for(nlines, 256), 256, 0, st>>>(g, d, side, k, order & 1, f,
                                                                   nlines);
    }
}

// ------------------------------------------------------------------------ Lindman boundaries
// Both edges of axis d are open (update_lindman_{2,3}d_e/b and update_emfbound_lindman,
// source/emf/boundary/os-emf-lindman.f90:454-1042).  The state holds five buffer planes along
// d -- slot 0 E at i_d = 0, 1 E at 1, 2 B at 0 (the lower buffers, range [0, 1]), 3 E at
// nx+1, 4 E at nx+2 (the upper ones, range [nx, nx+2]) -- with 3 components per interior point
// m of the other axes (the lower other axis fastest); element (slot, m, c) at
// 3 * (slot * nperp + m) + c.  Only the components other than d of the E planes are ever
// written, so their normal component stays at the zero the buffers start with.
struct LindAxes {
    int d, pa, pb;        // the open axis and the other two (3: none)
    int na, nb;           // their interior extents (1 for none)
    long nperp;           // na * nb
};

static LindAxes lind_axes(const GridDesc &g, int d)
{
    LindAxes L;
    L.d = d;
    int o[2] = {3, 3}, k = 0;
    for (int a = 0; a < g.dim; a++)
        if (a != d) o[k++] = a;
    L.pa = o[0];
    L.pb = o[1];
    L.na = L.pa < 3 ? g.nx[L.pa] : 1;
    L.nb = L.pb < 3 ? g.nx[L.pb] : 1;
    L.nperp = (long)L.na * L.nb;
    return L;
}

long lindman_state_size(const GridDesc &g, int axis) { return 15L * lind_axes(g, axis).nperp; }

__device__ __forceinline__ long lind_pos(const GridDesc &g, const LindAxes &L, int i, int ia,
                                         int ib)
{
    int ic[3] = {1, 1, 1};
    ic[L.d] = i;
    if (L.pa < 3) ic[L.pa] = ia;
    if (L.pb < 3) ic[L.pb] = ib;
    return pos(g, ic[0], ic[1], ic[2]);
}

// after the E step: first-order Mur update of the two tangential components on the planes
// i_d = 0 (from i_d = 1) and i_d = nx+2 (from nx+1), with k = (1 - dt/dx_d) / (1 + dt/dx_d)
template <typename T>
__global__ void k_lindman_e(GridDesc g, LindAxes L, T *__restrict__ e, T *__restrict__ st, T k)
{
    OSG_GRID_LOOP(m, L.nperp)
    {
        const int ia = 1 + (int)(m % L.na), ib = 1 + (int)(m / L.na), n = g.nx[L.d];
        const long p0 = lind_pos(g, L, 0, ia, ib), p1 = lind_pos(g, L, 1, ia, ib);
        const long q1 = lind_pos(g, L, n + 1, ia, ib), q2 = lind_pos(g, L, n + 2, ia, ib);
        T *s0 = st + 3 * (0 * L.nperp + m), *s1 = st + 3 * (1 * L.nperp + m);
        T *s3 = st + 3 * (3 * L.nperp + m), *s4 = st + 3 * (4 * L.nperp + m);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            if (c == L.d) continue;
            const T e1 = e[p1 + c];
            const T e0 = s1[c] + k * (s0[c] - e1);
            e[p0 + c] = e0;
            s0[c] = e0;
            s1[c] = e1;
            const T f1 = e[q1 + c];
            const T f2 = s3[c] + k * (s4[c] - f1);
            e[q2 + c] = f2;
            s3[c] = f1;
            s4[c] = f2;
        }
    }
}

// after each B half step: the lower B buffer takes the Yee increment of the plane i_d = 0
// (h = dt / dx * 0.5 per axis, 0 beyond dim)
template <typename T>
__global__ void k_lindman_b(GridDesc g, LindAxes L, const T *__restrict__ e, T *__restrict__ st,
                            T h0, T h1, T h2)
{
    OSG_GRID_LOOP(m, L.nperp)
    {
        const int ia = 1 + (int)(m % L.na), ib = 1 + (int)(m / L.na);
        const long p = lind_pos(g, L, 0, ia, ib);
        const long u0 = p + 3, u1 = g.dim > 1 ? p + g.stride(1) : p,
                   u2 = g.dim > 2 ? p + g.stride(2) : p;
        T *s = st + 3 * (2 * L.nperp + m);
        s[0] = s[0] - h1 * (e[u1 + 2] - e[p + 2]) + h2 * (e[u2 + 1] - e[p + 1]);
        s[1] = s[1] - h2 * (e[u2 + 0] - e[p + 0]) + h0 * (e[u0 + 2] - e[p + 2]);
        s[2] = s[2] - h0 * (e[u0 + 1] - e[p + 1]) + h1 * (e[u1 + 0] - e[p + 0]);
    }
}

// the planes E(0), B(0) and E(nx+1), all components, over the full extent of the other axes;
// a guard point takes the buffer value of its periodic image (the buffers' own periodic
// update along the other axes, update_boundary_lindman :352-368)
template <typename T>
__global__ void k_lindman_restore(GridDesc g, LindAxes L, T *__restrict__ e, T *__restrict__ b,
                                  const T *__restrict__ st, long nfull)
{
    OSG_GRID_LOOP(m, nfull)
    {
        const int fa = L.pa < 3 ? g.size[L.pa] : 1;
        const int la = L.pa < 3 ? 1 - g.gcl[L.pa] : 1, lb = L.pb < 3 ? 1 - g.gcl[L.pb] : 1;
        const int ia = la + (int)(m % fa), ib = lb + (int)(m / fa);
        const int wa = ((ia - 1) % L.na + L.na) % L.na, wb = ((ib - 1) % L.nb + L.nb) % L.nb;
        const long w = wa + (long)L.na * wb;
        const long p0 = lind_pos(g, L, 0, ia, ib), q1 = lind_pos(g, L, g.nx[L.d] + 1, ia, ib);
        const T *s0 = st + 3 * (0 * L.nperp + w), *s2 = st + 3 * (2 * L.nperp + w),
                *s3 = st + 3 * (3 * L.nperp + w);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            e[p0 + c] = s0[c];
            b[p0 + c] = s2[c];
            e[q1 + c] = s3[c];
        }
    }
}

template <typename T>
static void launch_lindman_b(const GridDesc &g, const LindAxes &L, const T *e, T *lind,
                             const double *dx, double dt, cudaStream_t st)
{
    T h[3] = {T(0), T(0), T(0)};
    for (int a = 0; a < g.dim; a++) h[a] = (T)(dt / dx[a]) * T(0.5);
    k_lindman_b<T><<<blocks_for(L.nperp, 256), 256, 0, st>>>(g, L, e, lind, h[0], h[1], h[2]);
}

template <typename T>
void open_guards(const GridDesc &g, T *e, T *b, int axis, const T *lind, cudaStream_t st)
{
    periodic_update<T>(g, e, 0, st, 0, 1 << axis);
    periodic_update<T>(g, b, 0, st, 0, 1 << axis);
    const LindAxes L = lind_axes(g, axis);
    long nfull = 1;
    if (L.pa < 3) nfull *= g.size[L.pa];
    if (L.pb < 3) nfull *= g.size[L.pb];
    k_lindman_restore<T><<<blocks_for(nfull, 256), 256, 0, st>>>(g, L, e, b, lind, nfull);
}

template <typename T>
void lindman_phase(const GridDesc &g, int axis, int what, T *e, T *b, T *lind, const double *dx,
                   double dt, cudaStream_t st)
{
    const LindAxes L = lind_axes(g, axis);
    if (what == 0) {
        const T k = (T)((1.0 - dt / dx[axis]) / (1.0 + dt / dx[axis]));
        k_lindman_e<T><<<blocks_for(L.nperp, 256), 256, 0, st>>>(g, L, e, lind, k);
    } else if (what == 1) {
        launch_lindman_b(g, L, e, lind, dx, dt, st);
    } else {
        long nfull = 1;
        if (L.pa < 3) nfull *= g.size[L.pa];
        if (L.pb < 3) nfull *= g.size[L.pb];
        k_lindman_restore<T><<<blocks_for(nfull, 256), 256, 0, st>>>(g, L, e, b, lind, nfull);
    }
}

// ---------------------------------------------------------------------------- PML walls
// Vay's perfectly matched layer ("vpml", source/emf/boundary/os-emf-vpml.f03) at both edges of
// the axes in a mask of a 2D box (Cartesian, no diffusion correction).  Each PML edge is a wall
// of nb cells along its axis a -- range [2 - nb, 1] below, [nx + 1, nx + nb] above (setup_vpml
// :361-368, two cells of overlap with the box) -- over [1 - g1, nt + g2] along the other axis t
// (new_wall, source/vdf/os-wall.f90:188-195): g1 = max(gcl_t, c - 1), g2 = max(gcu_t, c), with
// c = nb for the x1 walls when x2 has PML walls too (they cover the corners, setup_vpml
// :382-398), else 2.  A wall point holds four split components: 0 X, 1 Y, 2 ZX (the z part
// driven by x1 derivatives), 3 ZY (by x2 derivatives); the box's z is ZX + ZY.
// State (pml_state_size reals): per PML axis a in increasing order, walls (side, field), side
// 0 lower / 1 upper, field 0 E / 1 B, at base_a + (2 side + field) W_a, W_a = nte_a nb 4,
// nte_a = nt + g1 + g2; point (iw, it) component c at 4 ((it - 1 + g1) nb + iw - lo(side)) + c.
// Then the attenuation tables of both axes at T (the walls' total): axis a, table k (0 E lower,
// 1 E upper, 2 B lower, 3 B upper), coefficient m (0..2) of wall cell n (1..nb) at
// T + ((4 a + k) 3 + m) nb + n - 1 (setup_att_coeff :3586-3684).
struct PmlDesc {
    int mask, nb, nx[2];
    int g1[2], g2[2], nte[2];
    long W[2], base[2], T;
};

static PmlDesc pml_desc(const GridDesc &g, int mask, int nb)
{
    PmlDesc P;
    P.mask = mask;
    P.nb = nb;
    long off = 0;
    for (int a = 0; a < 2; a++) {
        const int t = 1 - a;
        P.nx[a] = g.nx[a];
        const int c = (a == 0 && ((mask >> 1) & 1)) ? nb : 2;
        // along x1 the lower corner count is one more (the reference's rule for a moving x1,
        // setup_vpml :371-376, kept whether or not the window moves: the extra guard row never
        // reaches the box), so the state's layout does not depend on the window
        const int cl = t == 0 ? c + 1 : c;
        P.g1[a] = g.gcl[t] > cl - 1 ? g.gcl[t] : cl - 1;
        P.g2[a] = g.gcu[t] > c ? g.gcu[t] : c;
        P.nte[a] = g.nx[t] + P.g1[a] + P.g2[a];
        P.W[a] = (long)P.nte[a] * nb * 4;
        P.base[a] = off;
        if ((mask >> a) & 1) off += 4 * P.W[a];
    }
    P.T = off;
    return P;
}

// 3D walls at both edges of the axes in a mask: six split components per point, 2F + s for
// field component F, s = 0 the part driven by the derivative along the lower of the two other
// axes (XY, YX, ZX), s = 1 the other (XZ, YZ, ZY) (update_e_x{1,2,3}_3d, update_b_x{1,2,3}_3d,
// update_interface_x{1,2,3}_3d).  The walls of a lower axis than a PML axis D extend over D's
// edge regions (corner priority x1 > x2 > x3), where their D splits are damped with D's tables.
// The wall of axis a spans [1 - g1, n_t + g2] along each other axis t: g1 = max(gcl_t, c - 1),
// g2 = max(gcu_t, c), c = nb when t has PML walls and a < t, else 2.  Per PML axis a in
// increasing order, wall (side, field) at base_a + (2 side + field) W_a,
// W_a = nte_a,t1 nte_a,t2 nb 6 (t1 < t2); point (iw, i_t1, i_t2) component c at
// 6 (((i_t2 - 1 + g1_t2) nte_t1 + i_t1 - 1 + g1_t1) nb + iw - lo(side)) + c; the tables of all
// three axes follow at T (the walls' total).
struct Pml3Desc {
    int mask, nb, n[3];
    int g1[3][3], g2[3][3], nte[3][3];   // [wall axis][other axis]
    long W[3], base[3], T;
};

static Pml3Desc pml3_desc(const GridDesc &g, int mask, int nb)
{
    Pml3Desc P;
    P.mask = mask;
    P.nb = nb;
    long off = 0;
    for (int d = 0; d < 3; d++) P.n[d] = g.nx[d];
    for (int a = 0; a < 3; a++) {
        long w = (long)nb * 6;
        for (int t = 0; t < 3; t++) {
            const int c = (((mask >> t) & 1) && a < t) ? nb : 2;
            const int cl = t == 0 ? c + 1 : c;   // as in 2D: one more below along x1
            P.g1[a][t] = g.gcl[t] > cl - 1 ? g.gcl[t] : cl - 1;
            P.g2[a][t] = g.gcu[t] > c ? g.gcu[t] : c;
            P.nte[a][t] = g.nx[t] + P.g1[a][t] + P.g2[a][t];
            if (t != a) w *= P.nte[a][t];
        }
        P.W[a] = w;
        P.base[a] = off;
        if ((mask >> a) & 1) off += 4 * w;
    }
    P.T = off;
    return P;
}

__device__ __forceinline__ long pml3_at(const Pml3Desc &P, int a, int side, int fld, int c,
                                        const int *i)
{
    const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
    const int lo = side == 0 ? 2 - P.nb : P.n[a] + 1;
    return P.base[a] + (2 * side + fld) * P.W[a] +
           6 * ((((long)i[t2] - 1 + P.g1[a][t2]) * P.nte[a][t1] + i[t1] - 1 + P.g1[a][t1]) * P.nb +
                i[a] - lo) + c;
}

// interfaces of the walls of axis a: the box into the wall over [1, n + 1] of both other axes
// (first split the box's component, second 0), the wall's sums into the box over [0, n + 2];
// one thread per edge and transverse point of the larger range
template <typename T>
__global__ void k_pml3_iface(GridDesc g, Pml3Desc P, T *__restrict__ st, T *__restrict__ f, int fld,
                             int a)
{
    const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
    const int m1 = P.n[t1] + 3, m2 = P.n[t2] + 3;
    const long n = 2L * m1 * m2;
    OSG_GRID_LOOP(m, n)
    {
        const int side = (int)(m / ((long)m1 * m2));
        const int r = (int)(m % ((long)m1 * m2));
        const int lo = side == 0 ? 2 - P.nb : P.n[a] + 1, hi = lo + P.nb - 1;
        const int to_w = side == 0 ? hi : lo, to_b = side == 0 ? hi - 1 : lo + 1;
        int i[3];
        i[t1] = r % m1;
        i[t2] = r / m1;
        if (i[t1] >= 1 && i[t1] <= P.n[t1] + 1 && i[t2] >= 1 && i[t2] <= P.n[t2] + 1) {
            i[a] = to_w;
            const long pw = pos(g, i[0], i[1], i[2]);
            for (int F = 0; F < 3; F++) {
                st[pml3_at(P, a, side, fld, 2 * F, i)] = f[pw + F];
                st[pml3_at(P, a, side, fld, 2 * F + 1, i)] = T(0);
            }
        }
        i[a] = to_b;
        const long pb = pos(g, i[0], i[1], i[2]);
        for (int F = 0; F < 3; F++)
            f[pb + F] = st[pml3_at(P, a, side, fld, 2 * F, i)] +
                        st[pml3_at(P, a, side, fld, 2 * F + 1, i)];
    }
}

// contacts of the walls of axis a with the walls of a higher PML axis d (update_interface_x1_3d
// :3090-3180, update_interface_x2_3d :3370-3430): below, d's wall takes plane 0 of a's wall and
// gives it plane 1; above, a's wall takes plane n_a + 1 and gives n_a + 2; over d's edge rows
// and, along the remaining axis o, [1 - g1, n + g2] of a's wall for the x1 walls' x2 contacts,
// else [1, n + 1].  One thread per side of a, wall of d, edge row, point along o and component
template <typename T>
__global__ void k_pml3_contact(Pml3Desc P, T *__restrict__ st, int fld, int a, int d)
{
    const int o = 3 - a - d;
    const int olo = (a == 0 && d == 1) ? 1 - P.g1[a][o] : 1;
    const int ohi = (a == 0 && d == 1) ? P.n[o] + P.g2[a][o] : P.n[o] + 1;
    const int no = ohi - olo + 1, nr = P.nb - 1;
    const long n = 4L * nr * no * 6;
    OSG_GRID_LOOP(m, n)
    {
        const int c = (int)(m % 6);
        long r = m / 6;
        int i[3];
        i[o] = olo + (int)(r % no);
        r /= no;
        const int row = (int)(r % nr);
        r /= nr;
        const int adj = (int)(r % 2), side = (int)(r / 2);
        i[d] = adj == 0 ? 2 - P.nb + row : P.n[d] + 2 + row;
        if (side == 0) {
            i[a] = 0;
            st[pml3_at(P, d, adj, fld, c, i)] = st[pml3_at(P, a, 0, fld, c, i)];
            i[a] = 1;
            st[pml3_at(P, a, 0, fld, c, i)] = st[pml3_at(P, d, adj, fld, c, i)];
        } else {
            i[a] = P.n[a] + 1;
            st[pml3_at(P, a, 1, fld, c, i)] = st[pml3_at(P, d, adj, fld, c, i)];
            i[a] = P.n[a] + 2;
            st[pml3_at(P, d, adj, fld, c, i)] = st[pml3_at(P, a, 1, fld, c, i)];
        }
    }
}

// one E (fld 0) or B (fld 1) update of the walls of axis a: split (F, D) with G the third axis,
// E_FD += sgn dt/dx_D (E: G at p and p - e_D), B_FD -= sgn dt/dx_D (G at p + e_D and p), sgn +1
// when D follows F cyclically; damped along D = a with a's tables, and in the edge regions of a
// higher PML axis D with D's.  E reads only B and B only E: one thread per edge and wall point
template <typename T>
__global__ void k_pml3_update(Pml3Desc P, T *__restrict__ st, T dx0, T dx1, T dx2, int fld, int a)
{
    const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
    const long npl = (long)P.nte[a][t1] * P.nte[a][t2] * P.nb;
    const long n = 2 * npl;
    const T dtdx[3] = {dx0, dx1, dx2};
    OSG_GRID_LOOP(m, n)
    {
        const int side = (int)(m / npl);
        long r = m % npl;
        const int lo = side == 0 ? 2 - P.nb : P.n[a] + 1, hi = lo + P.nb - 1;
        int i[3];
        i[a] = lo + (int)(r % P.nb);
        r /= P.nb;
        i[t1] = 1 - P.g1[a][t1] + (int)(r % P.nte[a][t1]);
        i[t2] = 1 - P.g1[a][t2] + (int)(r / P.nte[a][t1]);
        const int r0 = fld == 0 ? lo + 1 : (side == 0 ? lo : lo + 1);
        const int r1 = fld == 0 ? (side == 0 ? hi - 1 : hi) : hi - 1;
        if (i[a] < r0 || i[a] > r1) continue;
        const int t0 = fld == 0 ? 2 : 1, te = fld == 0 ? 0 : -1;
        if (i[t1] < t0 - P.g1[a][t1] || i[t1] > P.n[t1] + P.g2[a][t1] + te) continue;
        if (i[t2] < t0 - P.g1[a][t2] || i[t2] > P.n[t2] + P.g2[a][t2] + te) continue;
        const int k = fld == 0 ? side : 2 + side;
        const int cofs = side == 0 ? (fld == 0 ? lo - 1 : lo - 2) : lo;
        const int ci = i[a] - cofs;
        const int src = 1 - fld;
#pragma unroll
        for (int F = 0; F < 3; F++)
#pragma unroll
            for (int sp = 0; sp < 2; sp++) {
                const int o1 = F == 0 ? 1 : 0, o2 = F == 2 ? 1 : 2;
                const int D = sp == 0 ? o1 : o2, G = 3 - F - D;
                const bool cyc = D == (F + 1) % 3;
                const int sgn = fld == 0 ? (cyc ? 1 : -1) : (cyc ? -1 : 1);
                int qa[3] = {i[0], i[1], i[2]}, qb[3] = {i[0], i[1], i[2]};
                if (fld == 0) qb[D] -= 1;
                else qa[D] += 1;
                T &v = st[pml3_at(P, a, side, fld, 2 * F + sp, i)];
                const T a0 = st[pml3_at(P, a, side, src, 2 * G, qa)];
                const T a1 = st[pml3_at(P, a, side, src, 2 * G + 1, qa)];
                const T b0 = st[pml3_at(P, a, side, src, 2 * G, qb)];
                const T b1 = st[pml3_at(P, a, side, src, 2 * G + 1, qb)];
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
                    const T *cf = st + P.T + (4 * D + dk) * 3 * P.nb + dn - 1;
                    const T c1 = cf[0], c2 = cf[P.nb], c3 = cf[2 * P.nb];
                    const T ga = a0 + a1, gb = b0 + b1;
                    if (sgn > 0) v = c1 * v + c2 * ga - c3 * gb;
                    else v = c1 * v - c2 * ga + c3 * gb;
                } else {
                    const T dd = a0 + a1 - b0 - b1;
                    if (sgn > 0) v = v + dtdx[D] * dd;
                    else v = v - dtdx[D] * dd;
                }
            }
    }
}

// the periodic update of the walls of axis a along the periodic other axis t, over the full
// extent of the remaining axis o (guards included)
template <typename T>
__global__ void k_pml3_guard(Pml3Desc P, T *__restrict__ st, int a, int t)
{
    const int o = 3 - a - t;
    const int ng = P.g1[a][t] + P.g2[a][t];
    const long n = 4L * P.nb * P.nte[a][o] * ng;
    OSG_GRID_LOOP(m, n)
    {
        long r = m;
        const int gi = (int)(r % ng);
        r /= ng;
        int i[3], j[3];
        i[o] = 1 - P.g1[a][o] + (int)(r % P.nte[a][o]);
        r /= P.nte[a][o];
        const int iw = (int)(r % P.nb), wall = (int)(r / P.nb);
        const int side = wall >> 1, fld = wall & 1;
        i[a] = (side == 0 ? 2 - P.nb : P.n[a] + 1) + iw;
        i[t] = gi < P.g1[a][t] ? 1 - P.g1[a][t] + gi : P.n[t] + 1 + (gi - P.g1[a][t]);
        j[a] = i[a];
        j[o] = i[o];
        j[t] = gi < P.g1[a][t] ? i[t] + P.n[t] : i[t] - P.n[t];
        for (int c = 0; c < 6; c++)
            st[pml3_at(P, a, side, fld, c, i)] = st[pml3_at(P, a, side, fld, c, j)];
    }
}

long pml_state_size(const GridDesc &g, int mask, int nb)
{
    if (g.dim == 3) return pml3_desc(g, mask, nb).T + 36L * nb;
    return pml_desc(g, mask, nb).T + 24L * nb;
}

template <typename T>
void pml_init_host(const GridDesc &g, int mask, int nb, const double *dx, double dt, T *st)
{
    // the tables follow the walls (2D: per PML axis; 3D: the one axis)
    const long tab = g.dim == 3 ? pml3_desc(g, mask, nb).T : pml_desc(g, mask, nb).T;
    const long n = tab + 12L * g.dim * nb;
    for (long i = 0; i < n; i++) st[i] = T(0);
    // t(x) = exp(s1 (s2 x)^4) with s1 = -0.8 (4 + 1) / 2, s2 = 1 / (nb - 3); the fourth power
    // as two squares (the reference's exponent is the real constant 4.0 and its base is
    // negative at the interface point of the lower edge)
    const double s1 = -(0.8 * (4.0 + 1.0)) / 2.0, s2 = 1.0 / (nb - 3);
    auto att = [&](double x) {
        const double y = s2 * x;
        return exp(s1 * (y * y) * (y * y));
    };
    for (int a = 0; a < g.dim; a++) {
        T *cf = st + tab + 12L * a * nb;
        auto at = [&](int k, int m, int c) -> T & { return cf[(3 * k + m) * nb + c - 1]; };
        const double dtdx = dt / dx[a], dif = (1.0 - dtdx) / (1.0 + dtdx);
        for (int j = 0; j < nb; j++) {
            // lower edge: B is the outer point, j = -1/2 the interface
            double tj = att(j - 0.5), tj12 = att((double)j), tj1 = att(j + 0.5);
            double b1e = dtdx * (1.0 + dif * (1.0 - tj12)), b1b = dtdx * (1.0 + dif * (1.0 - tj1));
            at(0, 0, nb - j) = (T)(1.0 - b1e + tj12 * dtdx);
            at(0, 1, nb - j) = (T)(tj * b1e);
            at(0, 2, nb - j) = (T)dtdx;
            at(2, 0, nb - j) = (T)(1.0 - b1b + tj1 * dtdx);
            at(2, 1, nb - j) = (T)(tj12 * b1b);
            at(2, 2, nb - j) = (T)dtdx;
            // upper edge: E is the outer point, j = 0 the interface
            tj = att((double)j);
            tj12 = att(j + 0.5);
            tj1 = att(j + 1.0);
            b1e = dtdx * (1.0 + dif * (1.0 - tj12));
            b1b = dtdx * (1.0 + dif * (1.0 - tj1));
            at(1, 0, j + 1) = (T)(1.0 - b1e + tj12 * dtdx);
            at(1, 1, j + 1) = (T)dtdx;
            at(1, 2, j + 1) = (T)(tj * b1e);
            at(3, 0, j + 1) = (T)(1.0 - b1b + tj1 * dtdx);
            at(3, 1, j + 1) = (T)dtdx;
            at(3, 2, j + 1) = (T)(tj12 * b1b);
        }
    }
}

__device__ __forceinline__ int pml_lo(const PmlDesc &P, int a, int side)
{
    return side == 0 ? 2 - P.nb : P.nx[a] + 1;
}

// component c of wall (a, side, fld) at box coordinates (i1, i2) (iw along a, it along t)
template <typename T>
__device__ __forceinline__ T &pml_at(const PmlDesc &P, T *st, int a, int side, int fld, int c,
                                     int i1, int i2)
{
    const int iw = a == 0 ? i1 : i2, it = a == 0 ? i2 : i1;
    return st[P.base[a] + (2 * side + fld) * P.W[a] +
              4 * ((long)(it - 1 + P.g1[a]) * P.nb + (iw - pml_lo(P, a, side))) + c];
}

template <typename T>
__device__ __forceinline__ T pml_coef(const PmlDesc &P, const T *st, int a, int k, int m, int n)
{
    return st[P.T + ((4 * a + k) * 3 + m) * P.nb + n - 1];
}

// interfaces of the walls of axis a with the box for field fld (update_interface_x1_2d
// :2880-2943, update_interface_x2_2d :3190-3248): the box point next to the wall's inner end
// goes into the wall (ZX takes the box's z, ZY 0), the wall point one cell further out goes
// into the box (z = ZX + ZY); one thread per edge and transverse point 0 .. nt + 2
template <typename T>
__global__ void k_pml_iface(GridDesc g, PmlDesc P, T *__restrict__ st, T *__restrict__ f, int fld,
                            int a)
{
    const int nt = P.nx[1 - a];
    const long n = 2L * (nt + 3);
    OSG_GRID_LOOP(m, n)
    {
        const int side = (int)(m / (nt + 3)), it = (int)(m % (nt + 3));
        const int lo = pml_lo(P, a, side), hi = lo + P.nb - 1;
        const int to_w = side == 0 ? hi : lo, to_b = side == 0 ? hi - 1 : lo + 1;
        const int w1 = a == 0 ? to_w : it, w2 = a == 0 ? it : to_w;
        const long pw = pos(g, w1, w2, 1);
        for (int c = 0; c < 3; c++) pml_at(P, st, a, side, fld, c, w1, w2) = f[pw + c];
        pml_at(P, st, a, side, fld, 3, w1, w2) = T(0);
        const int b1 = a == 0 ? to_b : it, b2 = a == 0 ? it : to_b;
        const long pb = pos(g, b1, b2, 1);
        f[pb + 0] = pml_at(P, st, a, side, fld, 0, b1, b2);
        f[pb + 1] = pml_at(P, st, a, side, fld, 1, b1, b2);
        f[pb + 2] = pml_at(P, st, a, side, fld, 2, b1, b2) + pml_at(P, st, a, side, fld, 3, b1, b2);
    }
}

// the x1 walls' contact columns with the x2 walls over the corner rows (update_interface_x1_2d
// :2945-2988): below, the x2 wall takes the x1 wall's column 0 and gives it column 1; above,
// the x1 wall takes column nx1 + 1 and gives column nx1 + 2.  One thread per x1 wall, x2 wall,
// corner row and component
template <typename T>
__global__ void k_pml_contact(PmlDesc P, T *__restrict__ st, int fld)
{
    const int nr = P.nb - 1;   // corner rows per x2 wall: 2 - nb .. 0 and nx2 + 2 .. nx2 + nb
    const long n = 2L * 2 * nr * 4;
    OSG_GRID_LOOP(m, n)
    {
        const int c = (int)(m % 4);
        const int r = (int)((m / 4) % nr), adj = (int)((m / (4 * nr)) % 2), side = (int)(m / (8 * nr));
        const int i2 = adj == 0 ? 2 - P.nb + r : P.nx[1] + 2 + r;
        if (side == 0) {
            pml_at(P, st, 1, adj, fld, c, 0, i2) = pml_at(P, st, 0, 0, fld, c, 0, i2);
            pml_at(P, st, 0, 0, fld, c, 1, i2) = pml_at(P, st, 1, adj, fld, c, 1, i2);
        } else {
            const int i1 = P.nx[0] + 1;
            pml_at(P, st, 0, 1, fld, c, i1, i2) = pml_at(P, st, 1, adj, fld, c, i1, i2);
            pml_at(P, st, 1, adj, fld, c, i1 + 1, i2) = pml_at(P, st, 0, 1, fld, c, i1 + 1, i2);
        }
    }
}

// the E walls of axis a (update_e_x1_2d :925-1048 with its corner branch, update_e_x2_2d
// :1369-1456): one thread per edge, wall row and transverse point; E reads only B, so the
// points are independent
template <typename T>
__global__ void k_pml_e(PmlDesc P, T *__restrict__ st, T dtdx, int a)
{
    const int nt = P.nx[1 - a], nte = P.nte[a];
    const long n = 2L * P.nb * nte;
    const bool cor = a == 0 && ((P.mask >> 1) & 1);
    OSG_GRID_LOOP(m, n)
    {
        const int side = (int)(m / ((long)P.nb * nte));
        const int rem = (int)(m % ((long)P.nb * nte));
        const int lo = pml_lo(P, a, side), hi = lo + P.nb - 1;
        const int iw = lo + rem % P.nb, it = 1 - P.g1[a] + rem / P.nb;
        if (it < 2 - P.g1[a]) continue;   // transverse range 2 - g1 .. nt + g2
        const int r0 = lo + 1, r1 = side == 0 ? hi - 1 : hi;
        const int k = side, cofs = side == 0 ? lo - 1 : lo;
        const bool lowest = a == 1 && iw == lo;
        if (!lowest && (iw < r0 || iw > r1)) continue;
        const int i1 = a == 0 ? iw : it, i2 = a == 0 ? it : iw;
#define WE(c, x, y) pml_at(P, st, a, side, 0, c, x, y)
#define WB(c, x, y) pml_at(P, st, a, side, 1, c, x, y)
        if (a == 0) {
            const int ci = i1 - cofs;
            const T c1 = pml_coef(P, st, 0, k, 0, ci), c2 = pml_coef(P, st, 0, k, 1, ci),
                    c3 = pml_coef(P, st, 0, k, 2, ci);
            // corner rows (x2 walls below or above): damped along x2 as well
            const int cn = !cor ? 0 : (i2 <= 0 ? i2 + P.g1[0] : (i2 > nt + 1 ? i2 - nt - 1 : 0));
            if (cn) {
                const int ck = i2 <= 0 ? 0 : 1;
                const T d1 = pml_coef(P, st, 1, ck, 0, cn), d2 = pml_coef(P, st, 1, ck, 1, cn),
                        d3 = pml_coef(P, st, 1, ck, 2, cn);
                WE(0, i1, i2) = d1 * WE(0, i1, i2) + d2 * (WB(2, i1, i2) + WB(3, i1, i2)) -
                                d3 * (WB(2, i1, i2 - 1) + WB(3, i1, i2 - 1));
                WE(3, i1, i2) = d1 * WE(3, i1, i2) - d2 * WB(0, i1, i2) + d3 * WB(0, i1, i2 - 1);
            } else {
                WE(0, i1, i2) = WE(0, i1, i2) + dtdx * (WB(2, i1, i2) + WB(3, i1, i2) -
                                                        WB(2, i1, i2 - 1) - WB(3, i1, i2 - 1));
                WE(3, i1, i2) = WE(3, i1, i2) - dtdx * (WB(0, i1, i2) - WB(0, i1, i2 - 1));
            }
            WE(1, i1, i2) = c1 * WE(1, i1, i2) - c2 * (WB(2, i1, i2) + WB(3, i1, i2)) +
                            c3 * (WB(2, i1 - 1, i2) + WB(3, i1 - 1, i2));
            WE(2, i1, i2) = c1 * WE(2, i1, i2) + c2 * WB(1, i1, i2) - c3 * WB(1, i1 - 1, i2);
        } else {
            if (!lowest) {
                const int ci = i2 - cofs;
                const T c1 = pml_coef(P, st, 1, k, 0, ci), c2 = pml_coef(P, st, 1, k, 1, ci),
                        c3 = pml_coef(P, st, 1, k, 2, ci);
                WE(0, i1, i2) = c1 * WE(0, i1, i2) + c2 * (WB(2, i1, i2) + WB(3, i1, i2)) -
                                c3 * (WB(2, i1, i2 - 1) + WB(3, i1, i2 - 1));
                WE(3, i1, i2) = c1 * WE(3, i1, i2) - c2 * WB(0, i1, i2) + c3 * WB(0, i1, i2 - 1);
            }
            // Y and ZX by the plain Yee update (also on the wall's lowest row)
            WE(1, i1, i2) = WE(1, i1, i2) - dtdx * (WB(2, i1, i2) + WB(3, i1, i2) -
                                                    WB(2, i1 - 1, i2) - WB(3, i1 - 1, i2));
            WE(2, i1, i2) = WE(2, i1, i2) + dtdx * (WB(1, i1, i2) - WB(1, i1 - 1, i2));
        }
    }
}

// the B walls of axis a (update_b_x1_2d :2066-2177 with its corner branch, update_b_x2_2d
// :2512-2579)
template <typename T>
__global__ void k_pml_b(PmlDesc P, T *__restrict__ st, T dtdx, int a)
{
    const int nt = P.nx[1 - a], nte = P.nte[a];
    const long n = 2L * P.nb * nte;
    const bool cor = a == 0 && ((P.mask >> 1) & 1);
    OSG_GRID_LOOP(m, n)
    {
        const int side = (int)(m / ((long)P.nb * nte));
        const int rem = (int)(m % ((long)P.nb * nte));
        const int lo = pml_lo(P, a, side), hi = lo + P.nb - 1;
        const int iw = lo + rem % P.nb, it = 1 - P.g1[a] + rem / P.nb;
        if (it > nt + P.g2[a] - 1) continue;   // transverse range 1 - g1 .. nt + g2 - 1
        const int r0 = side == 0 ? lo : lo + 1, r1 = hi - 1;
        const int k = 2 + side, cofs = side == 0 ? lo - 2 : lo;
        const bool highest = a == 1 && iw == hi;
        if (!highest && (iw < r0 || iw > r1)) continue;
        const int i1 = a == 0 ? iw : it, i2 = a == 0 ? it : iw;
        if (a == 0) {
            const int ci = i1 - cofs;
            const T c1 = pml_coef(P, st, 0, k, 0, ci), c2 = pml_coef(P, st, 0, k, 1, ci),
                    c3 = pml_coef(P, st, 0, k, 2, ci);
            const int cn = !cor ? 0 : (i2 <= 0 ? i2 + P.g1[0] + 1 : (i2 > nt + 1 ? i2 - nt - 1 : 0));
            if (cn) {
                const int ck = i2 <= 0 ? 2 : 3;
                const T d1 = pml_coef(P, st, 1, ck, 0, cn), d2 = pml_coef(P, st, 1, ck, 1, cn),
                        d3 = pml_coef(P, st, 1, ck, 2, cn);
                WB(0, i1, i2) = d1 * WB(0, i1, i2) - d2 * (WE(2, i1, i2 + 1) + WE(3, i1, i2 + 1)) +
                                d3 * (WE(2, i1, i2) + WE(3, i1, i2));
                WB(3, i1, i2) = d1 * WB(3, i1, i2) + d2 * WE(0, i1, i2 + 1) - d3 * WE(0, i1, i2);
            } else {
                WB(0, i1, i2) = WB(0, i1, i2) - dtdx * (WE(2, i1, i2 + 1) + WE(3, i1, i2 + 1) -
                                                        WE(2, i1, i2) - WE(3, i1, i2));
                WB(3, i1, i2) = WB(3, i1, i2) + dtdx * (WE(0, i1, i2 + 1) - WE(0, i1, i2));
            }
            WB(1, i1, i2) = c1 * WB(1, i1, i2) + c2 * (WE(2, i1 + 1, i2) + WE(3, i1 + 1, i2)) -
                            c3 * (WE(2, i1, i2) + WE(3, i1, i2));
            WB(2, i1, i2) = c1 * WB(2, i1, i2) - c2 * WE(1, i1 + 1, i2) + c3 * WE(1, i1, i2);
        } else {
            if (!highest) {
                const int ci = i2 - cofs;
                const T c1 = pml_coef(P, st, 1, k, 0, ci), c2 = pml_coef(P, st, 1, k, 1, ci),
                        c3 = pml_coef(P, st, 1, k, 2, ci);
                WB(0, i1, i2) = c1 * WB(0, i1, i2) - c2 * (WE(2, i1, i2 + 1) + WE(3, i1, i2 + 1)) +
                                c3 * (WE(2, i1, i2) + WE(3, i1, i2));
                WB(3, i1, i2) = c1 * WB(3, i1, i2) + c2 * WE(0, i1, i2 + 1) - c3 * WE(0, i1, i2);
            }
            // Y and ZX by the plain Yee update (also on the wall's highest row)
            WB(1, i1, i2) = WB(1, i1, i2) + dtdx * (WE(2, i1 + 1, i2) + WE(3, i1 + 1, i2) -
                                                    WE(2, i1, i2) - WE(3, i1, i2));
            WB(2, i1, i2) = WB(2, i1, i2) - dtdx * (WE(1, i1 + 1, i2) - WE(1, i1, i2));
        }
#undef WE
#undef WB
    }
}

// the diffusion correction of the walls of axis a (vpml_diffuse, 2D): over the points of the
// E update range the two parts of B_z exchange p_difrate = 0.1 (update_e_x1_2d :1001-1006,
// update_e_x2_2d :1399-1408), before the E walls advance (every point the reference's loop
// reads after diffusing it is diffused here first; the others are outside the range)
template <typename T>
__global__ void k_pml_diffuse(PmlDesc P, T *__restrict__ st, int a)
{
    const int nt = P.nx[1 - a], nte = P.nte[a];
    const long n = 2L * P.nb * nte;
    OSG_GRID_LOOP(m, n)
    {
        const int side = (int)(m / ((long)P.nb * nte));
        const int rem = (int)(m % ((long)P.nb * nte));
        const int lo = pml_lo(P, a, side), hi = lo + P.nb - 1;
        const int iw = lo + rem % P.nb, it = 1 - P.g1[a] + rem / P.nb;
        if (it < 2 - P.g1[a] || it > nt + P.g2[a]) continue;
        const int r0 = lo + 1, r1 = side == 0 ? hi - 1 : hi;
        if (iw < r0 || iw > r1) continue;
        const int i1 = a == 0 ? iw : it, i2 = a == 0 ? it : iw;
        T &zx = pml_at(P, st, a, side, 1, 2, i1, i2), &zy = pml_at(P, st, a, side, 1, 3, i1, i2);
        const T bzx = zx, rm = T(1) - T(0.1);
        zx = rm * zx + T(0.1) * zy;
        zy = rm * zy + T(0.1) * bzx;
    }
}

// the walls' periodic update along a periodic t (update_periodic_wall, source/vdf/
// os-wall-comm.f90:182-344): guard points from the opposite interior points, all components,
// the whole wall-normal range
template <typename T>
__global__ void k_pml_guard(PmlDesc P, T *__restrict__ st, int a)
{
    const int ng = P.g1[a] + P.g2[a], nt = P.nx[1 - a];
    const long n = 4L * P.nb * ng * 4;
    OSG_GRID_LOOP(m, n)
    {
        const int c = (int)(m % 4);
        long r = m / 4;
        const int gi = (int)(r % ng);
        r /= ng;
        const int iw_ofs = (int)(r % P.nb), wall = (int)(r / P.nb);   // wall = 2 side + fld
        const int side = wall >> 1, fld = wall & 1;
        const int iw = pml_lo(P, a, side) + iw_ofs;
        const int it = gi < P.g1[a] ? 1 - P.g1[a] + gi : nt + 1 + (gi - P.g1[a]);
        const int src = gi < P.g1[a] ? it + nt : it - nt;
        const int a1 = a == 0 ? iw : it, a2 = a == 0 ? it : iw;
        const int s1 = a == 0 ? iw : src, s2 = a == 0 ? src : iw;
        pml_at(P, st, a, side, fld, c, a1, a2) = pml_at(P, st, a, side, fld, c, s1, s2);
    }
}

template <typename T>
void pml_phase(const GridDesc &g, int mask, int nb, int what, T *e, T *b, T *pml,
               const double *dx, double dt, cudaStream_t st)
{
    if (g.dim == 3) {
        const Pml3Desc Q = pml3_desc(g, mask, nb);
        if (what == 0) {
            // the walls' periodic update along their periodic other axes, lower axis first
            for (int a = 0; a < 3; a++) {
                if (!((mask >> a) & 1)) continue;
                for (int t = 0; t < 3; t++) {
                    if (t == a || ((mask >> t) & 1) || (t == 0 && ((mask >> 3) & 1))) continue;
                    const long n = 4L * nb * Q.nte[a][3 - a - t] * (Q.g1[a][t] + Q.g2[a][t]);
                    k_pml3_guard<T><<<blocks_for(n, 256), 256, 0, st>>>(Q, pml, a, t);
                }
            }
            return;
        }
        const int fld = what == 1 ? 1 : 0;
        T *f = what == 1 ? b : e;
        // the interfaces of every wall in setup order (x1, x2, x3), each with its contacts with
        // the walls of the higher PML axes, then the wall updates
        for (int a = 0; a < 3; a++) {
            if (!((mask >> a) & 1)) continue;
            const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
            const long ni = 2L * (Q.n[t1] + 3) * (Q.n[t2] + 3);
            k_pml3_iface<T><<<blocks_for(ni, 256), 256, 0, st>>>(g, Q, pml, f, fld, a);
            for (int d = a + 1; d < 3; d++) {
                if (!((mask >> d) & 1)) continue;
                const int o = 3 - a - d;
                const int no = (a == 0 && d == 1) ? Q.n[o] + Q.g1[a][o] + Q.g2[a][o] : Q.n[o] + 1;
                const long nc = 4L * (nb - 1) * no * 6;
                k_pml3_contact<T><<<blocks_for(nc, 256), 256, 0, st>>>(Q, pml, fld, a, d);
            }
        }
        for (int a = 0; a < 3; a++) {
            if (!((mask >> a) & 1)) continue;
            const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
            const long nu = 2L * Q.nte[a][t1] * Q.nte[a][t2] * nb;
            k_pml3_update<T><<<blocks_for(nu, 256), 256, 0, st>>>(
                Q, pml, (T)(dt / dx[0]), (T)(dt / dx[1]), (T)(dt / dx[2]), what == 1 ? 0 : 1, a);
        }
        return;
    }
    const PmlDesc P = pml_desc(g, mask, nb);
    if (what == 0) {
        for (int a = 0; a < 2; a++) {
            const int t = 1 - a;
            if (!((mask >> a) & 1) || ((mask >> t) & 1) || (t == 0 && ((mask >> 3) & 1)))
                continue;
            const long n = 4L * nb * (P.g1[a] + P.g2[a]) * 4;
            k_pml_guard<T><<<blocks_for(n, 256), 256, 0, st>>>(P, pml, a);
        }
        return;
    }
    const int fld = what == 1 ? 1 : 0;
    T *f = what == 1 ? b : e;
    // the interfaces of every wall in the reference's order (x1 walls with their corner
    // contacts, then x2 walls), then the wall updates
    for (int a = 0; a < 2; a++) {
        if (!((mask >> a) & 1)) continue;
        k_pml_iface<T><<<blocks_for(2L * (g.nx[1 - a] + 3), 256), 256, 0, st>>>(g, P, pml, f,
                                                                                fld, a);
        if (a == 0 && ((mask >> 1) & 1))
            k_pml_contact<T><<<blocks_for(16L * (nb - 1), 256), 256, 0, st>>>(P, pml, fld);
    }
    for (int a = 0; a < 2; a++) {
        if (!((mask >> a) & 1)) continue;
        const T dtdx = (T)(dt / dx[1 - a]);
        const long n = 2L * nb * P.nte[a];
        if (what == 1 && ((mask >> (4 + a)) & 1))   // bits 4, 5: diffusion on the x1, x2 walls
            k_pml_diffuse<T><<<blocks_for(n, 256), 256, 0, st>>>(P, pml, a);
        if (what == 1) k_pml_e<T><<<blocks_for(n, 256), 256, 0, st>>>(P, pml, dtdx, a);
        else k_pml_b<T><<<blocks_for(n, 256), 256, 0, st>>>(P, pml, dtdx, a);
    }
}

template <typename T>
void pml_guards(const GridDesc &g, T *e, T *b, int mask, int nb, T *pml, cudaStream_t st)
{
    const int skip = (mask & 7) | ((mask >> 3) & 1);   // PML axes, and x1 when it moves
    pml_phase<T>(g, mask, nb, 0, e, b, pml, nullptr, 0.0, st);
    periodic_update<T>(g, e, 0, st, 0, skip);
    periodic_update<T>(g, b, 0, st, 0, skip);
}

// window move: the walls of the axes other than x1 shift one cell down along x1, all
// components, the last x1 plane becoming zero (move_window_vpml :478-494, move_window_wall,
// source/vdf/os-wall-comm.f90:57-176).  x1 is their first other axis, so a wall is lines of
// `line` reals (one x1 point) repeated nl times along x1, for each point of the remaining
// axes; out of place through tmp (at least as long as the largest wall)
template <typename T>
__global__ void k_pml_shift_x(const T *__restrict__ in, T *__restrict__ out, long line, long nl,
                              long n)
{
    OSG_GRID_LOOP(p, n)
    {
        const long k = (p / line) % nl;
        out[p] = k + 1 < nl ? in[p + line] : T(0);
    }
}

long pml_shift_scratch(const GridDesc &g, int mask, int nb)
{
    long w = 0;
    if (g.dim == 2) {
        const PmlDesc P = pml_desc(g, mask, nb);
        if ((mask >> 1) & 1) w = P.W[1];
    } else {
        const Pml3Desc P = pml3_desc(g, mask, nb);
        for (int a = 1; a < 3; a++)
            if (((mask >> a) & 1) && P.W[a] > w) w = P.W[a];
    }
    return w;
}

template <typename T>
void pml_shift_x(const GridDesc &g, int mask, int nb, T *pml, T *tmp, cudaStream_t st)
{
    for (int a = 1; a < g.dim; a++) {
        if (!((mask >> a) & 1)) continue;
        long base, W, line, nl;
        if (g.dim == 2) {
            const PmlDesc P = pml_desc(g, mask, nb);
            base = P.base[1];
            W = P.W[1];
            line = 4L * nb;
            nl = P.nte[1];
        } else {
            const Pml3Desc P = pml3_desc(g, mask, nb);
            base = P.base[a];
            W = P.W[a];
            line = 6L * nb;
            nl = P.nte[a][0];
        }
        for (int w = 0; w < 4; w++) {
            T *f = pml + base + w * W;
            unsigned blocks = blocks_for(W, 256);
            if (blocks > 152 * 32) blocks = 152 * 32;
            k_pml_shift_x<T><<<blocks, 256, 0, st>>>(f, tmp, line, nl, W);
            cudaMemcpyAsync(f, tmp, sizeof(T) * W, cudaMemcpyDeviceToDevice, st);
        }
    }
}

template <typename T>
void yee_advance(const GridDesc &g, T *e, T *b, const T *j, const double *dx, double dt,
                 cudaStream_t st, int walls, int order, int open_axis, T *lind, int pmc,
                 int pml_mask, int pml_nb, T *pml)
{
    if (pml_mask && pml) {
        // PML walls: their E after the first B half step, their B after the E step, nothing
        // after the second B half step (update_boundary_bfld step 1 / update_boundary_efld,
        // source/emf/boundary/os-emf-boundary.f90:931-935, 1071-1074)
        launch_dbdt(g, b, e, dx, dt / 2.0, st);
        pml_phase<T>(g, pml_mask, pml_nb, 1, e, b, pml, dx, dt, st);
        launch_dedt(g, e, b, j, dx, dt, st);
        pml_phase<T>(g, pml_mask, pml_nb, 2, e, b, pml, dx, dt, st);
        launch_dbdt(g, b, e, dx, dt / 2.0, st);
        return;
    }
    const bool open = open_axis >= 0 && lind;
    LindAxes L{};
    if (open) L = lind_axes(g, open_axis);
    launch_dbdt(g, b, e, dx, dt / 2.0, st);
    if (walls) wall_update(g, b, 1, walls, order, st, pmc);
    if (open) launch_lindman_b(g, L, e, lind, dx, dt, st);
    launch_dedt(g, e, b, j, dx, dt, st);
    if (walls) wall_update(g, e, 0, walls, order, st, pmc);
    if (open) {
        const T k = (T)((1.0 - dt / dx[open_axis]) / (1.0 + dt / dx[open_axis]));
        k_lindman_e<T><<<blocks_for(L.nperp, 256), 256, 0, st>>>(g, L, e, lind, k);
    }
    launch_dbdt(g, b, e, dx, dt / 2.0, st);
    if (walls) wall_update(g, b, 1, walls, order, st, pmc);
    if (open) launch_lindman_b(g, L, e, lind, dx, dt, st);
}

// One direction of the periodic update.  Thread n handles one guard point (lower or upper
// side along axis `d`, full range along the others) and its periodic image.
template <typename T>
__device__ __forceinline__ void periodic_body(const GridDesc &g, int d, int add,
                                              T *__restrict__ f, long n_lo, long n_all)
{
    OSG_GRID_LOOP(n, n_all)
    {
        const bool lower = n < n_lo;
        const long m = lower ? n : n - n_lo;
        int lo[3], ext[3];
        for (int a = 0; a < 3; a++) {
            if (a >= g.dim) {
                lo[a] = 1;
                ext[a] = 1;
            } else if (a == d) {
                lo[a] = lower ? 1 - g.gcl[a] : g.nx[a] + 1;
                ext[a] = lower ? g.gcl[a] : g.gcu[a];
            } else {
                lo[a] = 1 - g.gcl[a];
                ext[a] = g.size[a];
            }
        }
        int i[3];
        unflat(m, lo, ext, i[0], i[1], i[2]);
        const long pg = pos(g, i[0], i[1], i[2]);
        i[d] += lower ? g.nx[d] : -g.nx[d];
        const long pi = pos(g, i[0], i[1], i[2]);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            if (add) {
                const T v = f[pg + c] + f[pi + c];
                f[pg + c] = v;
                f[pi + c] = v;
            } else {
                f[pg + c] = f[pi + c];
            }
        }
    }
}

template <typename T>
__global__ void k_periodic_dir(GridDesc g, int d, int add, T *__restrict__ f, long n_lo, long n_all)
{
    periodic_body<T>(g, d, add, f, n_lo, n_all);
}

// Open boundary along axis d (moving window, x1): the guard slabs are zeroed, so fields see no
// periodic image and current deposited beyond the edge is dropped.
template <typename T>
__global__ void k_open_dir(GridDesc g, int d, T *__restrict__ f, long n_lo, long n_all)
{
    OSG_GRID_LOOP(n, n_all)
    {
        const bool lower = n < n_lo;
        const long m = lower ? n : n - n_lo;
        int lo[3], ext[3];
        for (int a = 0; a < 3; a++) {
            if (a >= g.dim) {
                lo[a] = 1;
                ext[a] = 1;
            } else if (a == d) {
                lo[a] = lower ? 1 - g.gcl[a] : g.nx[a] + 1;
                ext[a] = lower ? g.gcl[a] : g.gcu[a];
            } else {
                lo[a] = 1 - g.gcl[a];
                ext[a] = g.size[a];
            }
        }
        int i[3];
        unflat(m, lo, ext, i[0], i[1], i[2]);
        const long pg = pos(g, i[0], i[1], i[2]);
#pragma unroll
        for (int c = 0; c < 3; c++) f[pg + c] = T(0);
    }
}

template <typename T>
void periodic_update(const GridDesc &g, T *f, int add, cudaStream_t st, int open_mask,
                     int skip_mask)
{
    for (int d = 0; d < g.dim; d++) {
        if (skip_mask & (1 << d)) continue;
        long other = 1;
        for (int a = 0; a < g.dim; a++)
            if (a != d) other *= g.size[a];
        const long n_lo = other * g.gcl[d], n_all = n_lo + other * g.gcu[d];
        if (open_mask & (1 << d))
            k_open_dir<T><<<blocks_for(n_all, 256), 256, 0, st>>>(g, d, f, n_lo, n_all);
        else
            k_periodic_dir<T><<<blocks_for(n_all, 256), 256, 0, st>>>(g, d, add, f, n_lo, n_all);
    }
}

// Moving window: every point (guard cells included) takes the value one cell further along x1;
// the last x1 plane becomes zero (move_window_vdf, source/vdf/os-vdf.f03:56-205).  Out of place.
template <typename T>
__global__ void k_shift_x(GridDesc g, const T *__restrict__ in, T *__restrict__ out, long n)
{
    OSG_GRID_LOOP(p, n)
    {
        const long pt = p / 3;
        const int i1 = (int)(pt % g.size[0]);
        out[p] = i1 + 1 < g.size[0] ? in[p + 3] : T(0);
    }
}

template <typename T>
void shift_window_x(const GridDesc &g, T *f, T *tmp, cudaStream_t st)
{
    const long n = 3 * g.npoints();
    unsigned nb = blocks_for(n, 256);
    if (nb > 152 * 32) nb = 152 * 32;
    k_shift_x<T><<<nb, 256, 0, st>>>(g, f, tmp, n);
    cudaMemcpyAsync(f, tmp, sizeof(T) * n, cudaMemcpyDeviceToDevice, st);
}

// sum over the interior of each component squared, accumulated in double:
// out[c] += sum f_c^2 (caller applies 0.5 dV)
template <typename T>
__global__ void k_sumsq(GridDesc g, Box box, const T *__restrict__ f, double *out)
{
    double s0 = 0, s1 = 0, s2 = 0;
    OSG_GRID_LOOP(n, box.n)
    {
        int i1, i2, i3;
        unflat(n, box.lo, box.ext, i1, i2, i3);
        const long p = pos(g, i1, i2, i3);
        const double a = f[p], b = f[p + 1], c = f[p + 2];
        s0 += a * a;
        s1 += b * b;
        s2 += c * c;
    }
    s0 = block_sum(s0);
    s1 = block_sum(s1);
    s2 = block_sum(s2);
    if (threadIdx.x == 0) {
        atomicAdd(out + 0, s0);
        atomicAdd(out + 1, s1);
        atomicAdd(out + 2, s2);
    }
}

template <typename T>
void field_sumsq(const GridDesc &g, const T *f, double *d_out, cudaStream_t st)
{
    Box box = make_box(g, 1, 0);
    unsigned nb = blocks_for(box.n, 256);
    if (nb > 1216) nb = 1216;
    k_sumsq<T><<<nb, 256, 0, st>>>(g, box, f, d_out);
}

// charge density of particles (reference layout) into component 0 of a double grid with the
// same guard cells; shape of the interpolation order, support starting at 1 - OFFSET
template <typename T, int DIM, int ORD>
__global__ void k_rho(GridDesc g, const int *__restrict__ ix, const T *__restrict__ x,
                      const T *__restrict__ q, long np, double *rho, int *status)
{
    constexpr int NP = ORD + 1, LP = 1 - Stencil<ORD>::OFS;
    OSG_GRID_LOOP(p, np)
    {
        double w[3][NP];
        int c[3] = {1, 1, 1};
        bool ok = true;
        for (int d = 0; d < DIM; d++) {
            c[d] = ix[DIM * p + d];
            ok = ok && (c[d] + LP - 1 + g.gcl[d] >= 0) && (c[d] + LP + NP - 1 - 1 + g.gcl[d] < g.size[d]);
            const double xx = (double)x[DIM * p + d];
            const double a = 0.5 - xx, b = 0.5 + xx;
            if constexpr (ORD == 1) { w[d][0] = a; w[d][1] = b; }
            else if constexpr (ORD == 2) { w[d][0] = 0.5 * a * a; w[d][1] = fma(a, b, 0.5); w[d][2] = 0.5 * b * b; }
            else if constexpr (ORD == 3) {
                w[d][0] = a * a * a / 6.0; w[d][1] = fma(0.5, b * b * b, 2.0 / 3.0 - b * b);
                w[d][2] = fma(0.5, a * a * a, 2.0 / 3.0 - a * a); w[d][3] = b * b * b / 6.0;
            } else {
                const double ab = a * b;
                w[d][0] = a * a * a * a / 24.0; w[d][1] = fma(a, fma(a, 1.5 + ab, 1.0), 0.25) / 6.0;
                w[d][2] = fma(ab, fma(0.25, ab, 0.5), 11.0 / 24.0);
                w[d][3] = fma(b, fma(b, 1.5 + ab, 1.0), 0.25) / 6.0; w[d][4] = b * b * b * b / 24.0;
            }
        }
        if (!ok) {
            atomicOr(status, 1);
            continue;
        }
        const double qq = (double)q[p];
        const int n2 = DIM > 1 ? NP : 1, n3 = DIM > 2 ? NP : 1;
        for (int k3 = 0; k3 < n3; k3++)
            for (int k2 = 0; k2 < n2; k2++)
                for (int k1 = 0; k1 < NP; k1++) {
                    double wt = qq * w[0][k1];
                    if (DIM > 1) wt *= w[1][k2];
                    if (DIM > 2) wt *= w[2][k3];
                    const long pp = pos(g, c[0] + LP + k1, DIM > 1 ? c[1] + LP + k2 : 1,
                                        DIM > 2 ? c[2] + LP + k3 : 1);
                    atomicAdd(rho + pp, wt);
                }
    }
}

template <typename T>
int deposit_rho(const GridDesc &g, int order, const int *ix, const T *x, const T *q, long np,
                double *rho, int *status, cudaStream_t st)
{
    if (np <= 0) return OSG_OK;
    unsigned nb = blocks_for(np, 256);
    if (nb > 4096) nb = 4096;
#define OSG_CASE(D, O)                                                                        \
    if (g.dim == D && order == O) {                                                           \
        k_rho<T, D, O><<<nb, 256, 0, st>>>(g, ix, x, q, np, rho, status);                     \
        return OSG_OK;                                                                        \
    }
    OSG_CASE(2, 1) OSG_CASE(2, 2) OSG_CASE(2, 3) OSG_CASE(2, 4)
    OSG_CASE(3, 1) OSG_CASE(3, 2) OSG_CASE(3, 3) OSG_CASE(3, 4)
#undef OSG_CASE
    set_error("rho deposit: unsupported dim %d order %d", g.dim, order);
    return OSG_ERR_ARG;
}

// residual r = div E - (rho - rho_ref) on interior points; accumulates max |r| (as ordered
// bits) and sum r^2
template <typename T>
__global__ void k_gauss(GridDesc g, Box box, const T *__restrict__ e, const double *__restrict__ rho,
                        const double *__restrict__ rho_ref, double rdx0, double rdx1, double rdx2,
                        unsigned long long *maxbits, double *l2)
{
    double s = 0.0, m = 0.0;
    OSG_GRID_LOOP(n, box.n)
    {
        int i1, i2, i3;
        unflat(n, box.lo, box.ext, i1, i2, i3);
        const long p = pos(g, i1, i2, i3);
        double dv = ((double)e[p] - (double)e[p - 3]) * rdx0;
        if (g.dim > 1) dv += ((double)e[p + 1] - (double)e[p - g.stride(1) + 1]) * rdx1;
        if (g.dim > 2) dv += ((double)e[p + 2] - (double)e[p - g.stride(2) + 2]) * rdx2;
        const double r = dv - (rho[p] - (rho_ref ? rho_ref[p] : 0.0));
        s += r * r;
        m = fmax(m, fabs(r));
    }
    s = block_sum(s);
    // block max through the ordered bit pattern of non-negative doubles
    __shared__ double mx[32];
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) mx[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)((blockDim.x + 31) >> 5); w++) m = fmax(m, mx[w]);
        atomicAdd(l2, s);
        atomicMax(maxbits, (unsigned long long)__double_as_longlong(m));
    }
}

template <typename T>
void gauss_residual(const GridDesc &g, const T *e, const double *rho, const double *rho_ref,
                    const double *dx, unsigned long long *d_max, double *d_l2, cudaStream_t st)
{
    Box box = make_box(g, 1, 0);
    unsigned nb = blocks_for(box.n, 256);
    if (nb > 1216) nb = 1216;
    k_gauss<T><<<nb, 256, 0, st>>>(g, box, e, rho, rho_ref, 1.0 / dx[0],
                                   g.dim > 1 ? 1.0 / dx[1] : 0.0, g.dim > 2 ? 1.0 / dx[2] : 0.0,
                                   d_max, d_l2);
}



// ------------------------------------------------------------------------ batched boxes
FieldBox make_field_box(const GridDesc &g, float *e, float *b, float *j, const double *dx,
                        double dt)
{
    FieldBox f;
    f.g = g;
    f.e = e;
    f.b = b;
    f.j = j;
    const double h = dt / 2.0;
    f.d1h = (float)(h / dx[0]);
    f.d2h = g.dim > 1 ? (float)(h / dx[1]) : 0.0f;
    f.d3h = g.dim > 2 ? (float)(h / dx[2]) : 0.0f;
    f.dti = (float)dt;
    f.d1 = (float)(dt / dx[0]);
    f.d2 = g.dim > 1 ? (float)(dt / dx[1]) : 0.0f;
    f.d3 = g.dim > 2 ? (float)(dt / dx[2]) : 0.0f;
    return f;
}

template <int DIM>
__global__ void k_batch_periodic(const FieldBox *__restrict__ boxes, int d, int which, int add)
{
    const FieldBox &fb = boxes[blockIdx.y];
    float *f = which == 0 ? fb.e : (which == 1 ? fb.b : fb.j);
    long other = 1;
#pragma unroll
    for (int a = 0; a < DIM; a++)
        if (a != d) other *= fb.g.size[a];
    const long n_lo = other * fb.g.gcl[d], n_all = n_lo + other * fb.g.gcu[d];
    periodic_body<float>(fb.g, d, add, f, n_lo, n_all);
}

template <int DIM>
__global__ void k_batch_dbdt(const FieldBox *__restrict__ boxes)
{
    const FieldBox &fb = boxes[blockIdx.y];
    const Box box = make_box(fb.g, 0, 1);
    dbdt_body<float, DIM>(fb.g, box, fb.b, fb.e, fb.d1h, fb.d2h, fb.d3h);
}

template <int DIM>
__global__ void k_batch_dedt(const FieldBox *__restrict__ boxes)
{
    const FieldBox &fb = boxes[blockIdx.y];
    const Box box = make_box(fb.g, 1, 1);
    dedt_body<float, DIM>(fb.g, box, fb.e, fb.b, fb.j, fb.dti, fb.d1, fb.d2, fb.d3);
}

static unsigned batch_blocks(long n)
{
    long b = (n + 255) / 256;
    if (b > 1024) b = 1024;   // grid-stride beyond that
    return (unsigned)(b < 1 ? 1 : b);
}

void batch_periodic(const FieldBox *d_boxes, int nbox, int dim, int which, int add,
                    long max_side, cudaStream_t st)
{
    const dim3 grid(batch_blocks(max_side), (unsigned)nbox);
    for (int d = 0; d < dim; d++) {
        if (dim == 2) k_batch_periodic<2><<<grid, 256, 0, st>>>(d_boxes, d, which, add);
        else k_batch_periodic<3><<<grid, 256, 0, st>>>(d_boxes, d, which, add);
    }
}

void batch_yee(const FieldBox *d_boxes, int nbox, int dim, long max_points, cudaStream_t st)
{
    const dim3 grid(batch_blocks(max_points), (unsigned)nbox);
    if (dim == 2) {
        k_batch_dbdt<2><<<grid, 256, 0, st>>>(d_boxes);
        k_batch_dedt<2><<<grid, 256, 0, st>>>(d_boxes);
        k_batch_dbdt<2><<<grid, 256, 0, st>>>(d_boxes);
    } else {
        k_batch_dbdt<3><<<grid, 256, 0, st>>>(d_boxes);
        k_batch_dedt<3><<<grid, 256, 0, st>>>(d_boxes);
        k_batch_dbdt<3><<<grid, 256, 0, st>>>(d_boxes);
    }
}


// ------------------------------------------------------------------------ smoothing
// n 3-point kernels kern3[k] = {a, b, c} combined into one (2 nmax + 1)-point kernel
// (combine_kernel3, source/vdf/os-vdf-smooth.f90:151-183)
static void combine_kernel3(const double (*k3)[3], int n, int nmax, double *out)
{
    for (int i = 0; i < 2 * nmax + 1; i++) out[i] = 0.0;
    out[nmax] = 1.0;
    for (int k = 0; k < n; k++) {
        double f1 = 0.0;
        for (int j = nmax - k; j <= nmax + k + 1; j++) {
            out[j - 1] = k3[k][2] * out[j] + out[j - 1];
            const double f2 = k3[k][0] * out[j];
            out[j] = k3[k][1] * out[j] + f1;
            f1 = f2;
        }
    }
}

int smooth_coefficients(int type, int order, double *c, int *eff_order)
{
    double k3[15][3];
    int n = 0;
    switch (type) {
    case OSG_SMOOTH_NONE:
        *eff_order = 0;
        return OSG_OK;
    case OSG_SMOOTH_BINOMIAL:
        if (order < 1 || order > 15) return OSG_ERR_ARG;
        n = order;
        for (int j = 0; j < n; j++) k3[j][0] = 1.0, k3[j][1] = 2.0, k3[j][2] = 1.0;
        break;
    case OSG_SMOOTH_COMPENSATED: {
        n = order < 2 ? 2 : order;
        if (n > 15) return OSG_ERR_ARG;
        for (int j = 0; j < n - 1; j++) k3[j][0] = 1.0, k3[j][1] = 2.0, k3[j][2] = 1.0;
        // comp = (4.0 + 2.0 * (order - 1)) / (order - 1): default-real literals, so the
        // reference evaluates it in single precision (:418)
        const float comp = (4.0f + 2.0f * (float)(n - 1)) / (float)(n - 1);
        k3[n - 1][0] = -1.0, k3[n - 1][1] = (double)comp, k3[n - 1][2] = -1.0;
        break;
    }
    case OSG_SMOOTH_5PASS:
        n = 5;
        for (int j = 0; j < 4; j++) k3[j][0] = 1.0, k3[j][1] = 2.0, k3[j][2] = 1.0;
        k3[4][0] = -5.0, k3[4][1] = 15.0, k3[4][2] = -5.0;
        break;
    case OSG_SMOOTH_TRI6:
    case OSG_SMOOTH_TRI8:
        n = type == OSG_SMOOTH_TRI6 ? 3 : 4;
        break;
    default:
        return OSG_ERR_ARG;
    }
    if (type == OSG_SMOOTH_TRI6) {
        const double t[7] = {0.015625, -0.09375, 0.234375, 0.6875, 0.234375, -0.09375, 0.015625};
        for (int i = 0; i < 7; i++) c[i] = t[i];
    } else if (type == OSG_SMOOTH_TRI8) {
        const double t[9] = {-0.00390625, 0.03125, -0.109375, 0.21875, 0.7265625,
                             0.21875,     -0.109375, 0.03125, -0.00390625};
        for (int i = 0; i < 9; i++) c[i] = t[i];
    } else {
        combine_kernel3(k3, n, n, c);
    }
    // normalise (:452-464)
    double total = 0.0;
    for (int i = 0; i < 2 * n + 1; i++) total = total + c[i];
    for (int i = 0; i < 2 * n + 1; i++) c[i] = c[i] / total;
    *eff_order = n;
    return OSG_OK;
}

// one axis of the filter, out of place: points at least n from both ends of the axis (guard
// cells included) get sum_k c[k] f(i + k - n) summed in double in the reference's order
// (filter_2d/3d, :639-1000); the others are copied
template <typename T>
__global__ void k_smooth_dir(GridDesc g, int axis, int n, const T *__restrict__ in,
                             T *__restrict__ out, long npts, SmoothSpec sp)
{
    OSG_GRID_LOOP(q, npts)
    {
        const long pt = q / 3;
        const int j = (int)(axis == 0 ? pt % g.size[0]
                                      : (axis == 1 ? (pt / g.size[0]) % g.size[1]
                                                   : pt / ((long)g.size[0] * g.size[1])));
        if (j < n || j > g.size[axis] - 1 - n) {
            out[q] = in[q];
            continue;
        }
        const long st = g.stride(axis);
        const double *c = sp.c[axis];
        double f = (double)in[q - n * st] * c[0];
        for (int k = 1; k <= 2 * n; k++) f = f + (double)in[q + (k - n) * st] * c[k];
        out[q] = (T)f;
    }
}

template <typename T>
void smooth_field(const GridDesc &g, const SmoothSpec &sp, T *f, T *tmp, cudaStream_t st)
{
    const long n = 3 * g.npoints();
    unsigned nb = blocks_for(n, 256);
    if (nb > 152 * 32) nb = 152 * 32;
    for (int d = 0; d < g.dim; d++) {
        if (sp.order[d] <= 0) continue;
        k_smooth_dir<T><<<nb, 256, 0, st>>>(g, d, sp.order[d], f, tmp, n, sp);
        cudaMemcpyAsync(f, tmp, sizeof(T) * n, cudaMemcpyDeviceToDevice, st);
    }
}

template void yee_advance<float>(const GridDesc &, float *, float *, const float *,
                                 const double *, double, cudaStream_t, int, int, int, float *,
                                 int, int, int, float *);
template void yee_advance<double>(const GridDesc &, double *, double *, const double *,
                                  const double *, double, cudaStream_t, int, int, int,
                                  double *, int, int, int, double *);
template void pml_init_host<float>(const GridDesc &, int, int, const double *, double, float *);
template void pml_init_host<double>(const GridDesc &, int, int, const double *, double,
                                    double *);
template void pml_phase<float>(const GridDesc &, int, int, int, float *, float *, float *,
                               const double *, double, cudaStream_t);
template void pml_phase<double>(const GridDesc &, int, int, int, double *, double *, double *,
                                const double *, double, cudaStream_t);
template void pml_guards<float>(const GridDesc &, float *, float *, int, int, float *,
                                cudaStream_t);
template void pml_shift_x<float>(const GridDesc &, int, int, float *, float *, cudaStream_t);
template void pml_shift_x<double>(const GridDesc &, int, int, double *, double *, cudaStream_t);
template void pml_guards<double>(const GridDesc &, double *, double *, int, int, double *,
                                 cudaStream_t);
template void lindman_phase<float>(const GridDesc &, int, int, float *, float *, float *,
                                   const double *, double, cudaStream_t);
template void lindman_phase<double>(const GridDesc &, int, int, double *, double *, double *,
                                    const double *, double, cudaStream_t);
template void open_guards<float>(const GridDesc &, float *, float *, int, const float *,
                                 cudaStream_t);
template void open_guards<double>(const GridDesc &, double *, double *, int, const double *,
                                  cudaStream_t);
template void periodic_update<float>(const GridDesc &, float *, int, cudaStream_t, int, int);
template void periodic_update<double>(const GridDesc &, double *, int, cudaStream_t, int, int);
template void wall_update<float>(const GridDesc &, float *, int, int, int, cudaStream_t, int);
template void wall_update<double>(const GridDesc &, double *, int, int, int, cudaStream_t, int);
template void smooth_field<float>(const GridDesc &, const SmoothSpec &, float *, float *,
                                  cudaStream_t);
template void smooth_field<double>(const GridDesc &, const SmoothSpec &, double *, double *,
                                   cudaStream_t);
template void shift_window_x<float>(const GridDesc &, float *, float *, cudaStream_t);
template void shift_window_x<double>(const GridDesc &, double *, double *, cudaStream_t);
template void field_sumsq<float>(const GridDesc &, const float *, double *, cudaStream_t);
template void field_sumsq<double>(const GridDesc &, const double *, double *, cudaStream_t);
template int deposit_rho<float>(const GridDesc &, int, const int *, const float *,
                                const float *, long, double *, int *, cudaStream_t);
template int deposit_rho<double>(const GridDesc &, int, const int *, const double *,
                                 const double *, long, double *, int *, cudaStream_t);
template void gauss_residual<float>(const GridDesc &, const float *, const double *,
                                    const double *, const double *, unsigned long long *,
                                    double *, cudaStream_t);
template void gauss_residual<double>(const GridDesc &, const double *, const double *,
                                     const double *, const double *, unsigned long long *,
                                     double *, cudaStream_t);

} // namespace osg
