// fields.cuh -- grid kernels (Yee, periodic guard update, FP64 diagnostics).
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace osg {

// Fortran indices (i1,i2,i3) of flat point n of the box [lo, lo + ext) in each axis
__device__ __forceinline__ void unflat(long n, const int *lo, const int *ext, int &i1, int &i2,
                                       int &i3)
{
    i1 = lo[0] + (int)(n % ext[0]);
    long r = n / ext[0];
    i2 = lo[1] + (int)(r % ext[1]);
    i3 = lo[2] + (int)(r / ext[1]);
}

__device__ __forceinline__ long pos(const GridDesc &g, int i1, int i2, int i3)
{
    return 3L * ((long)(i1 - 1 + g.gcl[0]) +
                 (long)g.size[0] * ((i2 - 1 + g.gcl[1]) + (long)g.size[1] * (i3 - 1 + g.gcl[2])));
}

struct Box {
    int lo[3], ext[3];
    long n;
};

__host__ __device__ inline Box make_box(const GridDesc &g, int lo, int hi_off)
{
    // points lo .. nx + hi_off along active axes, single point 1 on inactive ones
    Box b;
    b.n = 1;
    for (int d = 0; d < 3; d++) {
        if (d < g.dim) {
            b.lo[d] = lo;
            b.ext[d] = g.nx[d] + hi_off - lo + 1;
        } else {
            b.lo[d] = 1;
            b.ext[d] = 1;
        }
        b.n *= b.ext[d];
    }
    return b;
}

// B half step, E full step, B half step; the axes in `walls` (bit d) are bounded by perfectly
// conducting walls, whose images are taken after every partial step as the reference's
// update_boundary_b / update_boundary_e (source/emf/solver/os-emf-solver-yee.f03:556-566)
// With open_axis >= 0 both edges of that axis are Lindman open boundaries whose state
// `lind` (lindman_state_size reals, zeroed before the first step) the E and B steps update
// (update_boundary_b / update_boundary_e, the same lines).
template <typename T>
void yee_advance(const GridDesc &g, T *e, T *b, const T *j, const double *dx, double dt,
                 cudaStream_t st, int walls = 0, int order = 2, int open_axis = -1,
                 T *lind = nullptr, int pmc = 0, int pml_mask = 0, int pml_nb = 0,
                 T *pml = nullptr);
// PML walls of nb cells at both edges of the axes in `mask` of a 2D box (Vay's perfectly
// matched layer, source/emf/boundary/os-emf-vpml.f03; the x1 walls cover the corners when both
// axes have walls).  The state: four split-field walls per PML axis (E and B per edge) and the
// attenuation tables, pml_state_size reals, set up on the host by pml_init_host (zeroed walls,
// tables from dt and dx).
long pml_state_size(const GridDesc &g, int mask, int nb);
template <typename T>
void pml_init_host(const GridDesc &g, int mask, int nb, const double *dx, double dt, T *st);
// one PML phase: 0 the walls' periodic update along a periodic other axis, 1 the E walls after
// the first B half step (interfaces with B first), 2 the B walls after the E step (interfaces
// with E first)
template <typename T>
void pml_phase(const GridDesc &g, int mask, int nb, int what, T *e, T *b, T *pml,
               const double *dx, double dt, cudaStream_t st);
// guard update of E and B with PML walls on the axes in `mask`: the walls' own update, then E
// and B periodic along the other axes only
template <typename T>
void pml_guards(const GridDesc &g, T *e, T *b, int mask, int nb, T *pml, cudaStream_t st);
// (bit 3 of `mask` in pml_phase / pml_guards: x1 is the axis of a moving window, so neither the
// walls nor the box take a periodic update along it; bits 4 and 5 in 2D: the x1 / x2 walls take
// the diffusion correction before their E update)
// window move: the PML walls of the axes other than x1 shift one cell down along x1, the last
// plane zero; tmp holds pml_shift_scratch reals
long pml_shift_scratch(const GridDesc &g, int mask, int nb);
template <typename T>
void pml_shift_x(const GridDesc &g, int mask, int nb, T *pml, T *tmp, cudaStream_t st);
// Lindman open boundaries at both edges of one axis (p_bc_lindman,
// source/emf/boundary/os-emf-lindman.f90).  Their state: 5 buffer planes along the axis
// (E at 0 and 1, B at 0, E at nx+1 and nx+2), 3 components, per interior point of the other
// axes.
long lindman_state_size(const GridDesc &g, int axis);
// guard update of E and B with Lindman boundaries on `axis`: periodic along the other axes,
// then the boundary planes E(0), B(0), E(nx+1) from the state (update_emfbound_lindman)
template <typename T>
void open_guards(const GridDesc &g, T *e, T *b, int axis, const T *lind, cudaStream_t st);
// one phase of the Lindman boundaries: 0 the Mur update of E and its planes after the E step,
// 1 the lower B buffer after a B half step (dt the full step), 2 the restore of E(0), B(0),
// E(nx+1) (guard points of the other axes from the state's periodic images)
template <typename T>
void lindman_phase(const GridDesc &g, int axis, int what, T *e, T *b, T *lind, const double *dx,
                   double dt, cudaStream_t st);
// conducting-wall images along the axes in `walls`: kind 0 E, 1 B (guards set), 2 J (guards
// added into the box); the axes in `pmc` are perfect magnetic instead of electric conductors
// for E and B (kinds 3 and 4 name those images directly)
template <typename T>
void wall_update(const GridDesc &g, T *f, int kind, int walls, int order, cudaStream_t st,
                 int pmc = 0);

// One box of a batch of independent periodic boxes (single precision): its fields and the
// Yee coefficients.  The batched launches take a device array of these, one box per
// blockIdx.y, and run the same per-point code as the single-box kernels.
struct FieldBox {
    GridDesc g;
    float *e, *b, *j;
    float d1h, d2h, d3h;      // dt / 2 / dx: the B half steps
    float dti, d1, d2, d3;    // dt and dt / dx: the E step
};
FieldBox make_field_box(const GridDesc &g, float *e, float *b, float *j, const double *dx,
                        double dt);
// periodic update of field `which` (0 = E, 1 = B, 2 = J) of every box, one launch per axis;
// max_side = the largest guard-slab point count over the boxes
void batch_periodic(const FieldBox *d_boxes, int nbox, int dim, int which, int add,
                    long max_side, cudaStream_t st);
// B half step, E step, B half step of every box; max_points = the largest box's point count
void batch_yee(const FieldBox *d_boxes, int nbox, int dim, long max_points, cudaStream_t st);

// add = 1: fold guard cells into their periodic images (current); add = 0: replace.  Axes set
// in open_mask (bit d) are open instead: their guard slabs are zeroed; axes in skip_mask
// (conducting walls) are left alone.
template <typename T>
void periodic_update(const GridDesc &g, T *f, int add, cudaStream_t st, int open_mask = 0,
                     int skip_mask = 0);

// Current smoothing (smooth_vdf, source/vdf/os-vdf-smooth.f90:514-540): a separable filter of
// 2 * order[d] + 1 points per axis with FP64 coefficients c[d][0 .. 2 order[d]].
struct SmoothSpec {
    int order[3];
    double c[3][31];
};
// coefficients of one axis (setup_smooth, :373-467): type OSG_SMOOTH_*, order as the deck's
int smooth_coefficients(int type, int order, double *c, int *eff_order);
// filter f in place along every axis with order > 0 (tmp: scratch array of the same size)
template <typename T>
void smooth_field(const GridDesc &g, const SmoothSpec &sp, T *f, T *tmp, cudaStream_t st);

// moving window: shift all of f one cell towards lower x1, zero the last x1 plane (tmp: a
// scratch array of the same size)
template <typename T> void shift_window_x(const GridDesc &g, T *f, T *tmp, cudaStream_t st);

// d_out[0..2] += sum over interior points of component^2 (double)
template <typename T>
void field_sumsq(const GridDesc &g, const T *f, double *d_out, cudaStream_t st);

template <typename T>
int deposit_rho(const GridDesc &g, int order, const int *ix, const T *x, const T *q, long np,
                double *rho, int *status, cudaStream_t st);

template <typename T>
void gauss_residual(const GridDesc &g, const T *e, const double *rho, const double *rho_ref,
                    const double *dx, unsigned long long *d_max, double *d_l2,
                    cudaStream_t st);

} // namespace osg
