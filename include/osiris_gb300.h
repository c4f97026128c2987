/*
 * osiris_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the OSIRIS particle-in-cell
 * time step: particle push (Boris), charge-conserving current deposition (orders 1-4), guard
 * cell fold/replace and the Yee field advance.
 *
 * Two layers:
 *
 *  1. Drop-in entry points with the reference's arguments and semantics, on HOST arrays in the
 *     reference memory layout.  They copy to the GPU, run the kernels and copy back, so a
 *     Fortran build of OSIRIS can call them in place of its SIMD kernels / Yee solver:
 *       osg_vadvance_deposit_{f32,f64}  replaces FNAME(vadvance_deposit_{1d,2d,3d}_s{1..4})
 *           source/simd/os-spec-push-avx2.c:255,471,1141 (single),
 *           source/simd/os-spec-push-avx2d.c:263,481,1127 (double);
 *           Fortran call sites source/spec/os-spec-vpush.f03:70-95,144-169,294-319.
 *           The exact reference symbol names (vadvance_deposit_2d_s2_ ...) are exported by the
 *           shim libraries libosiris_gb300_single.so / libosiris_gb300_double.so
 *           (include/osiris_gb300_fortran.h).
 *       osg_yee_advance_{f32,f64}       replaces advance_yee
 *           source/emf/solver/os-emf-solver-yee.f03:542-568 (dbdt/dedt :102-138,211-251,
 *           287-326,385-428)
 *       osg_periodic_{f32,f64}          replaces update_periodic_vdf (single-node periodic,
 *           p_vdf_add / p_vdf_replace) source/vdf/os-vdf-comm.f90:142-326, 665-722
 *
 *  2. A device-resident simulation handle (osg_sim_*): particles, fields and current stay in
 *     HBM between steps; one call advances N full time steps (phase order of iter_sim,
 *     source/os-simulation.f03:498-666); host copies happen only when the caller asks for
 *     state or diagnostics.  Two particle engines:
 *       OSG_ENGINE_PLAIN  reference particle layout, one thread per particle, global atomics
 *                         (the "plain" GPU form; used in FP64 and FP32)
 *       OSG_ENGINE_TILED  particles binned by spatial tile, fields staged in shared memory,
 *                         shared-memory current accumulation, per-step tile migration (FP32)
 *
 * All functions return OSG_OK (0) or a negative OSG_ERR_* code; osg_last_error() gives the
 * text of the calling thread's last error.  No function exits the process.
 */
#ifndef OSIRIS_GB300_H
#define OSIRIS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OSG_OK 0
#define OSG_ERR_ARG (-1)      /* invalid argument (dimension, order, sizes, pointers) */
#define OSG_ERR_CUDA (-2)     /* CUDA runtime error (no device, launch failure, ...) */
#define OSG_ERR_OVERFLOW (-3) /* a tile ran out of particle slots */
#define OSG_ERR_RANGE (-4)    /* a particle cell index left the valid range */
#define OSG_ERR_STATE (-5)    /* call out of sequence (e.g. no species) */
#define OSG_ERR_NOMEM (-6)    /* device or host allocation failed */

#define OSG_ENGINE_PLAIN 0
#define OSG_ENGINE_TILED 1

/* current smoothing types (the deck's smooth type, source/vdf/os-vdf-smooth.f90:27-38) */
#define OSG_SMOOTH_NONE 0
#define OSG_SMOOTH_BINOMIAL 2
#define OSG_SMOOTH_COMPENSATED 3
#define OSG_SMOOTH_5PASS 4
#define OSG_SMOOTH_TRI6 5
#define OSG_SMOOTH_TRI8 6

#define OSG_PUSHER_BORIS 0   /* push_type = "simd" / "standard" (Boris) */
#define OSG_PUSHER_EXACT 1   /* push_type = "exact" (analytic, source/spec/os-spec-extpush.f03) */
#define OSG_PUSHER_VAY 2     /* push_type = "vay" (dudt_vay, source/spec/os-spec-push.f03) */
#define OSG_PUSHER_HC 3      /* push_type = "cary" (Higuera-Cary, dudt_cary, same file) */
#define OSG_PUSHER_FULLROT 4 /* push_type = "fullrot" (dudt_fullrot, same file) */
#define OSG_PUSHER_EULER 5   /* push_type = "euler" (dudt_euler, same file) */
#define OSG_PUSHER_COND_VAY 6 /* push_type = "cond_vay" (dudt_cond_vay, same file: Vay when the
                                 particle's gamma exceeds 5, else Boris) */

const char *osg_last_error(void);
int osg_version(void);
int osg_device_count(void);
/* select the CUDA device used by the calling thread's subsequent calls */
int osg_set_device(int device);
/* free and total device memory of the current device, in bytes (cudaMemGetInfo); a
 * diagnostic with no counterpart in the reference */
int osg_device_memory(size_t *free_bytes, size_t *total_bytes);
/* page-locked host memory for the host-array entry points (fast copies); NULL on failure */
void *osg_host_alloc(size_t bytes);
int osg_host_free(void *p);

/* ---------------------------------------------------------------- drop-in, host arrays --- */

/* Push particles [i0, i1] (1-based, inclusive) of one species and ADD their current into j;
 * *ene += sum over particles of q * u^2/(gamma+1) at the half step.  ix/x/u/q: Fortran
 * ix(dim,N), x(dim,N), p(3,N), q(N); efield/bfield/j: f(3, size(1), size(2), size(3)) with
 * emf_offset / j_offset = number of lower guard cells.  dim 1..3, order 1..4.
 * Unlike the SIMD kernels, nothing is written past particle i1 (no padding contract). */
int osg_vadvance_deposit_f32(int dim, int order, int *ix, float *x, float *u, float *q,
                             int i0, int i1, float rqm, const float *efield,
                             const float *bfield, const int *emf_size, const int *emf_offset,
                             float *j, const int *j_size, const int *j_offset,
                             const double *dx, double dt, double *ene);
int osg_vadvance_deposit_f64(int dim, int order, int *ix, double *x, double *u, double *q,
                             int i0, int i1, double rqm, const double *efield,
                             const double *bfield, const int *emf_size, const int *emf_offset,
                             double *j, const int *j_size, const int *j_offset,
                             const double *dx, double dt, double *ene);

/* The 2D cylindrical push/deposit (x1 = z, x2 = r): replaces
 * FNAME(vadvance_deposit_2d_cyl_s{1..4}) (source/simd/os-spec-push-avx2.c:762-1092,
 * source/simd/os-spec-push-avx2d.c:777-1107), called from vadvance_deposit_2d_cyl
 * (source/spec/os-spec-vpush.f03:190-255) for coordinates = p_cylindrical_b (:424-425).  Same
 * arguments as osg_vadvance_deposit_* with dim = 2, plus ilb2 (after rqm, as the reference):
 * the lower global cell of the node along x2 (this%my_nx_p(p_lower, 2)).  The Boris update and
 * the axial move are the Cartesian ones; the radial move is done in double from the particle's
 * global radius, and p_r, p_theta are rotated onto the new radial direction with p_theta
 * scaled by r_old / r_new (angular momentum kept).  The current goes into j with the
 * Cartesian 2D charge-conserving deposit, as the reference's (its 1/r normalisation is a
 * later phase of the host). */
int osg_vadvance_deposit_cyl_f32(int order, int *ix, float *x, float *u, float *q, int i0,
                                 int i1, float rqm, int ilb2, const float *efield,
                                 const float *bfield, const int *emf_size,
                                 const int *emf_offset, float *j, const int *j_size,
                                 const int *j_offset, const double *dx, double dt, double *ene);
int osg_vadvance_deposit_cyl_f64(int order, int *ix, double *x, double *u, double *q, int i0,
                                 int i1, double rqm, int ilb2, const double *efield,
                                 const double *bfield, const int *emf_size,
                                 const int *emf_offset, double *j, const int *j_size,
                                 const int *j_offset, const double *dx, double dt, double *ene);

/* The same particle advance with the exact momentum update of push_type = "exact"
 * (dudt_exact, source/spec/os-spec-extpush.f03:40-348, reached through advance_deposit_{1d,2d,
 * 3d}, source/spec/os-spec-push.f03:1363-1605, with this%dudt => dudt_exact,
 * source/spec/os-species.f03:1432-1433): the Lorentz force in the interpolated fields is
 * integrated analytically over the step, its proper time found by at most 10 Newton
 * iterations to relative tolerance iter_tol (reference default 1e-3,
 * source/spec/os-spec-define.f03:471).  dt is the double time step (momentum and dt/dx, as
 * the Fortran path); position update, split and deposit as osg_vadvance_deposit_*.  *ene +=
 * sum of q (gamma - 1) of the new momenta (the energy dudt_exact reports). */
int osg_advance_deposit_exact_f32(int dim, int order, int *ix, float *x, float *u, float *q,
                                  int i0, int i1, float rqm, const float *efield,
                                  const float *bfield, const int *emf_size,
                                  const int *emf_offset, float *j, const int *j_size,
                                  const int *j_offset, const double *dx, double dt,
                                  double iter_tol, double *ene);
int osg_advance_deposit_exact_f64(int dim, int order, int *ix, double *x, double *u, double *q,
                                  int i0, int i1, double rqm, const double *efield,
                                  const double *bfield, const int *emf_size,
                                  const int *emf_offset, double *j, const int *j_size,
                                  const int *j_offset, const double *dx, double dt,
                                  double iter_tol, double *ene);

/* The particle advance of the Fortran path (advance_deposit_{1d,2d,3d},
 * source/spec/os-spec-push.f03:1363-1605) with any momentum update: pusher OSG_PUSHER_BORIS,
 * _EXACT (iter_tol), _VAY, _HC, _FULLROT or _EULER; dt is the double step (momentum and
 * dt/dx).  Position update, split and deposit as osg_vadvance_deposit_*; *ene += the energy the
 * chosen reference pusher reports (Boris and Vay: time-centred; exact: new momenta; HC, full
 * and Euler rotation: half-kicked). */
int osg_advance_deposit_f32(int dim, int order, int *ix, float *x, float *u, float *q, int i0,
                            int i1, float rqm, const float *efield, const float *bfield,
                            const int *emf_size, const int *emf_offset, float *j,
                            const int *j_size, const int *j_offset, const double *dx, double dt,
                            int pusher, double iter_tol, double *ene);
int osg_advance_deposit_f64(int dim, int order, int *ix, double *x, double *u, double *q,
                            int i0, int i1, double rqm, const double *efield,
                            const double *bfield, const int *emf_size, const int *emf_offset,
                            double *j, const int *j_size, const int *j_offset, const double *dx,
                            double dt, int pusher, double iter_tol, double *ene);

/* The same push for callers that cannot allocate device memory: hosts that give the whole GPU
 * to their own pool allocator at start-up and treat a foreign cudaMalloc as an error, and
 * stepping loops that budget device memory once and must not let a library allocate.  It has
 * no counterpart in the reference.  All device staging lives in one file-scope array of
 * OSG_NOALLOC_SCRATCH_BYTES, reserved on every GPU that loads the library until the process
 * exits; nothing is allocated or freed.  A call needs 8*dim + 16 bytes per particle (ix, x, u
 * and q: 32 B in 2D, 40 B in 3D), three copies of the grid (E, B, J) and under 2 KB of
 * alignment and counters; one that needs more than the array is rejected with OSG_ERR_ARG
 * (for a quadratic 256x256 grid the limit is about 446,000 2D particles per call); split the
 * particle range into smaller calls.  The first call on a device looks
 * up the array's address for that device; make it before any stream capture there.  Every
 * call shares the array, so calls that overlap on the GPU (several host threads at once) race;
 * each call clears what must start at zero and copies the rest in.  Runs on the calling
 * thread's default stream (cudaStreamPerThread) and returns when the results are on the host. */
#define OSG_NOALLOC_SCRATCH_BYTES (16u << 20)
int osg_vadvance_deposit_noalloc_f32(int dim, int order, int *ix, float *x, float *u, float *q,
                                     int i0, int i1, float rqm, const float *efield,
                                     const float *bfield, const int *emf_size,
                                     const int *emf_offset, float *j, const int *j_size,
                                     const int *j_offset, const double *dx, double dt,
                                     double *ene);

/* Same on arrays that already live in device memory, asynchronous on `stream`
 * (cudaStream_t, NULL = default stream).  d_ene is a device double that is incremented. */
int osg_vadvance_deposit_dev_f32(int dim, int order, int *ix, float *x, float *u,
                                 const float *q, long np, float rqm, const float *efield,
                                 const float *bfield, const int *emf_size,
                                 const int *emf_offset, float *j, const int *j_size,
                                 const int *j_offset, const double *dx, double dt,
                                 double *d_ene, void *stream);
int osg_vadvance_deposit_dev_f64(int dim, int order, int *ix, double *x, double *u,
                                 const double *q, long np, double rqm, const double *efield,
                                 const double *bfield, const int *emf_size,
                                 const int *emf_offset, double *j, const int *j_size,
                                 const int *j_offset, const double *dx, double dt,
                                 double *d_ene, void *stream);

/* Yee advance (B half step, E full step, B half step) on host arrays with guard cells. */
int osg_yee_advance_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *e,
                        float *b, const float *j, const double *dx, double dt);
int osg_yee_advance_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *e,
                        double *b, const double *j, const double *dx, double dt);

/* Single-node periodic guard update of a 3-component grid: add = 1 folds guard cells into
 * their periodic image and writes the sum to both (current); add = 0 copies the periodic
 * image into the guard cells (fields). */
int osg_periodic_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *f, int add);
/* Perfectly conducting walls bounding the axes in `walls` (bit d), on a HOST array: kind 0 E and
 * 1 B take their guard values from the image points (pec_bc_e/b_*d_odd/even,
 * source/emf/boundary/os-emf-pec.f90, odd or even by the interpolation order), kind 2 J adds
 * its guard values into the image points inside the box (spec_bc_*d,
 * source/current/os-current-boundary.f03).  The image of a component is the point mirrored
 * about the wall, with sign + for normal E and tangential B, J and - for tangential E and
 * normal B, J.  Kinds 3 (E) and 4 (B) are the walls of a perfect magnetic conductor
 * (pmc_bc_e/b_*d_odd/even, source/emf/boundary/os-emf-pmc.f90): the same image points with
 * the signs of E and B exchanged. */
/* Lindman open boundaries at both edges of `axis`, on HOST arrays (dim 2 or 3, gcl >= 1,
 * gcu >= 2), one phase per call: what 0 after the E step (update_lindman_{2,3}d_e,
 * source/emf/boundary/os-emf-lindman.f90:454-750: first-order Mur update of the tangential E on
 * the planes 0 and nx+2, the state's E planes refreshed), 1 after each B half step
 * (update_lindman_{2,3}d_b :539-857: the lower B buffer takes the Yee increment of the plane 0
 * from e; dt is the full step), 2 in the guard update (update_emfbound_lindman :861-1042:
 * E(0), B(0) and E(nx+1) from the state, guard points of the other axes from its periodic
 * images).  `state` holds 15 reals per interior point of the other axes, zeroed before the
 * first step: five planes (E at 0 and 1, B at 0, E at nx+1 and nx+2) of 3 components, the
 * point index with the lower other axis fastest. */
int osg_lindman_f32(int dim, const int *nx, const int *gcl, const int *gcu, int axis, int what,
                    float *e, float *b, float *state, const double *dx, double dt);
int osg_lindman_f64(int dim, const int *nx, const int *gcl, const int *gcu, int axis, int what,
                    double *e, double *b, double *state, const double *dx, double dt);
/* PML walls (Vay's split-field perfectly matched layer, source/emf/boundary/os-emf-vpml.f03) of
 * nb cells (>= 5) at both edges of the axes in `mask` (2D or 3D; gcl >= 1, gcu >= 2), on HOST
 * arrays, one phase per call: what 0 in the guard update (the walls' periodic update along their
 * periodic other axes, update_boundary_vpml :506-524), 1 after the first B half step (the B
 * interfaces, which write the box's B next to each wall, then the E walls, update_e_vpml_{2,3}d),
 * 2 after the E step (the E interfaces, which write the box's E, then the B walls,
 * update_b_vpml_{2,3}d).  `state` holds osg_pml_state_size reals: the split-field walls and the
 * attenuation tables, set up by osg_pml_init_* (walls zero, tables from dt and dx).  Flags above
 * the axes in `mask` for osg_pml_*: bit 3 x1 moves with a window (no periodic update of the
 * walls along it), bits 4 and 5 (2D) the diffusion correction of the x1 / x2 walls. */
long osg_pml_state_size(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb);
int osg_pml_init_f32(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                     const double *dx, double dt, float *state);
int osg_pml_init_f64(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                     const double *dx, double dt, double *state);
int osg_pml_f32(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb, int what,
                float *e, float *b, float *state, const double *dx, double dt);
int osg_pml_f64(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb, int what,
                double *e, double *b, double *state, const double *dx, double dt);
int osg_walls_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *f, int kind,
                  int walls, int order);
int osg_walls_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *f, int kind,
                  int walls, int order);
int osg_periodic_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *f,
                     int add);

/* Current smoothing of a 3-component grid on HOST arrays (smooth_vdf, source/vdf/
 * os-vdf-smooth.f90:514-540; applied to the current after its guard fold,
 * source/os-simulation.f03:651-657): along each axis d with type[d] != OSG_SMOOTH_NONE a
 * (2 n + 1)-point filter over the points at least n from both ends of the array (guard cells
 * included; the others are kept), axis after axis.  The coefficients are computed and kept in
 * FP64 (setup_smooth, :373-467) and the sums are taken in FP64.  The array needs gcl >= n and
 * gcu >= n + 1 guard cells for the filtered interior to be meaningful. */
int osg_smooth_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *f,
                   const int *type, const int *order);
int osg_smooth_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *f,
                   const int *type, const int *order);
/* the normalised FP64 coefficients of one axis: c[0 .. 2 n], *n = the filter's order */
int osg_smooth_coefficients(int type, int order, double *c, int *n);

/* Periodic particle boundary of a single node on HOST arrays: cell indices that left
 * [1, nx] are shifted by +-nx (replaces the periodic branch of phys_boundary_species,
 * source/spec/os-spec-boundary.f03:1280-1290; host code, no GPU). */
int osg_particle_wrap(int dim, const int *nx, long np, int *ix);

/* ---------------------------------------------------------------- seeded particle load --- */

/* Regular lattice load of one species over a periodic box, OSIRIS algorithm
 * (source/spec/psource/os-psource-std.f03:759-1120, source/spec/os-spec-udist.f03:452-850,
 * Mersenne Twister source/random/os-random-mt.f03:84-149, polar gaussian
 * source/random/os-random-class.f03:348-392).  The generator state lives in *rng (opaque,
 * OSG_RNG_BYTES bytes, initialised by osg_rng_seed); successive species share it like the
 * reference's global generator.  den(x1) = 1 + amp cos(2 pi kmode x1 / L1).
 * Writes nx.prod * ppc.prod particles; precision 32 or 64 selects float/double x, u, q. */
#define OSG_RNG_BYTES 2512
int osg_rng_seed(void *rng, int seed);
long osg_load_lattice(void *rng, int precision, int dim, const int *nx, const int *ppc,
                      const double *dx, double rqm, const double *uth, const double *ufl,
                      double amp, double kmode, int *ix, void *x, void *u, void *q);

/* ---------------------------------------------------------------- laser launch --------- */

/* A forward-propagating Gaussian laser pulse at t = 0: gaussian longitudinal envelope
 * exp(-2 ((x1 - lon_x0) / lon_duration)^2) cut at |x1 - lon_x0| <= lon_range / 2, Hermite-
 * Gaussian TEM00 transverse profile of waist per_w0 focused at x1 = per_focus around
 * per_center (x2[, x3]), peak field omega0 * a0, polarisation angle pol from x2 (zpulse with
 * lon_type = "gaussian", per_type = "gaussian", source/zpulse/os-zpulse-std.f03). */
typedef struct {
    double omega0, a0, pol;
    double lon_x0, lon_duration, lon_range;
    double per_w0, per_focus;
    double per_center[2];
} osg_zpulse;

/* Add the pulse to host field arrays (reference layout with guard cells; float for precision
 * 32, double for 64) of a box whose lower corner is xmin (launch_zpulse_2d/3d,
 * source/zpulse/os-zpulse-std.f03:1072-1390: in 2D the E/B components are set, in 3D added).
 * Host code only. */
int osg_zpulse_launch(int precision, int dim, int order, const int *nx, const int *gcl,
                      const int *gcu, const double *dx, const double *xmin, const osg_zpulse *zp,
                      void *e, void *b);

/* ---------------------------------------------------------------- device-resident sim --- */

typedef struct osg_sim osg_sim;

typedef struct {
    int dim;          /* 2 or 3 */
    int order;        /* interpolation order 1..4 */
    int precision;    /* 32 (mixed: FP32 particles/fields, FP64 diagnostics) or 64 */
    int engine;       /* OSG_ENGINE_PLAIN or OSG_ENGINE_TILED (TILED needs precision 32) */
    int nx[3];        /* cells per axis */
    double dx[3];     /* cell size */
    double dt;        /* time step (checked against the Courant limit) */
    int tile[3];      /* tile shape in cells (TILED; 0 = automatic) */
    int n_sort;       /* PLAIN: cell sort every n_sort steps (0 = never); TILED sorts every step */
    double capacity;  /* TILED: slots per tile as a multiple of the mean load (0 = 3.0) */
    int pusher;       /* OSG_PUSHER_BORIS (0), _EXACT (1), _VAY (2), _HC (3), _FULLROT (4),
                         _EULER (5), _COND_VAY (6) */
    double iter_tol;  /* exact pusher: Newton tolerance (0 = the reference default 1e-3) */
    int smooth_type;  /* current smoothing after the guard fold, OSG_SMOOTH_* (all axes) */
    int smooth_order; /* its order (binomial: passes; compensated: >= 2; others fixed) */
    int walls;        /* bit d set: axis d is bounded by perfectly conducting walls (PEC
                         fields, reflected current, specularly reflected particles); clear:
                         periodic */
    int open_fields;  /* bit d set (one axis at most): both edges of axis d are Lindman open
                         boundaries (first-order Mur update of the tangential E, the
                         reference's p_bc_lindman) and particles leaving through them are
                         absorbed; not with walls, smoothing or the moving window */
    int thermal;      /* bit d set (axis d walled or open): particles crossing its edges are
                         re-emitted from a thermal bath (the reference's p_bc_thermal) instead
                         of reflected or absorbed.  Both engines; the random stream is keyed by
                         the particle's index (PLAIN) or its tile slot (TILED) */
    unsigned int seed;      /* key of the re-emission random stream */
    double uth_bnd[3];      /* the bath's thermal momentum per component */
    double ufl_bnd[3];      /* its fluid momentum (added only when all three are non-zero) */
    int thermal_type; /* the bath's distribution (thermal_type): 0 "thermal" (Gaussian, normal
                         component half-Maxwellian), 1 "random dir" (|uth| in a random
                         direction), 2 "waterbag" (uniform in +-uth/2) */
    int pmc;          /* bit d set (d walled): the walls of axis d are perfect magnetic
                         conductors (the reference's p_bc_pmc, "reflecting") instead of
                         electric ones; the current and the particles are treated alike */
    int emf_smooth_type;  /* the fields the particles see (the reference's e_part/b_part,
                             smooth_type "stand" of the emf section): copies of E and B after
                             their guard update, filtered by OSG_SMOOTH_* (all axes); E and B
                             themselves are not changed.  Periodic boxes. */
    int emf_smooth_order; /* its order */
    int pml;          /* bit d set (2D, 3D): both edges of axis d are perfectly matched layers
                         (Vay's split-field PML, the reference's "vpml" field boundary) of
                         pml_cells cells each (the walls of a lower axis cover the edge regions
                         of the higher PML axes), and particles leaving through them are
                         absorbed; not with walls, Lindman boundaries, smoothing or a
                         thermal bath; with the moving window (along x1) on the other axes,
                         whose walls then move with the fields */
    int pml_cells;    /* PML thickness in cells (0 = the reference default 8; at least 5) */
    int pml_diffuse;  /* bit d set (d a PML axis of a 2D box): its walls take the reference's
                         diffusion correction (vpml_diffuse: the two parts of B_z exchange 10%
                         before every E update of the walls) */
} osg_config;

int osg_sim_create(const osg_config *cfg, osg_sim **out);
int osg_sim_destroy(osg_sim *s);
/* Add a species from host arrays (reference layout); x/u/q are float for precision 32 and
 * double for 64. Returns the species index (>= 0) or an error code. */
int osg_sim_add_species(osg_sim *s, double rqm, long np, const int *ix, const void *x,
                        const void *u, const void *q);
/* Guard-celled host fields (reference layout, precision of the sim); NULL leaves as is. */
int osg_sim_set_fields(osg_sim *s, const void *e, const void *b);
int osg_sim_get_fields(osg_sim *s, void *e, void *b, void *j);
int osg_sim_num_particles(osg_sim *s, int species, long *np);
/* Copy one species back to host arrays (tile order for the TILED engine). */
int osg_sim_get_species(osg_sim *s, int species, int *ix, void *x, void *u, void *q);
/* Advance n full time steps (captured once as a CUDA graph per step shape and replayed).
 * TILED: after every 8 steps, if any tile slab is more than 70% full, all species are re-binned
 * into larger slabs (a host round trip) so the following steps cannot overflow.
 * osg_sim_step_async makes no such check: a caller that times long runs with it checks
 * osg_sim_tile_occupancy between groups of steps. */
int osg_sim_step(osg_sim *s, int nsteps);
/* TILED: largest fraction of used particle slots over all tiles and species (0 for PLAIN). */
int osg_sim_tile_occupancy(osg_sim *s, double *max_frac);
/* Launch n steps without waiting for them (bench/timing); osg_sim_sync waits and reports
 * any error raised on the device. */
int osg_sim_step_async(osg_sim *s, int nsteps);
int osg_sim_sync(osg_sim *s);
void *osg_sim_stream(osg_sim *s);
/* FP64 diagnostics: kinetic[ns] kinetic energy of the last step (rqm * dV applied; Boris:
 * time-centred, exact pusher: of the new momenta, as each reference pusher reports it),
 * field[6] = 0.5 dV sum of E1..3^2 and B1..3^2. */
int osg_sim_energy(osg_sim *s, double *kinetic, double *field);
/* FP64 charge check: max over cells of |div E - rho| (rho of all species, order-matched
 * shape); the caller compares it with its value at t = 0 to verify conservation. */
int osg_sim_gauss_residual(osg_sim *s, double *max_abs, double *l2);
/* Average device time per launch of each phase over the last profiled steps (ms):
 * [0] push+deposit, [1] current fold, [2] Yee, [3] guard replace, [4] migration/sort. */
int osg_sim_profile(osg_sim *s, int nsteps, float *ms_phase);
/* Autotuner; call after the species are added and before the first step (not with the moving
 * window).  The state is put back after every trial.
 * TILED: times `steps` steps (after 2 untimed ones) for every candidate tile shape (2D: 8x8,
 * 16x8, 8x4, 16x16; 3D: 8x8x4, 8x4x4, 4x4x4, 8x8x8; those that divide the box and fit shared
 * memory) x push CTA size (256, 128), re-bins the particles for the fastest and returns it in
 * tile[3] and threads.  The tiled engine sorts every step inside its push (n_sort unchanged).
 * PLAIN: chooses the cell-sort interval n_sort (0 = never) from the measured cost of one sort C
 * and the growth g of the push time over `steps` unsorted steps: n = sqrt(2 C / g), the
 * interval with the least time per step; tile and threads are returned as 0. */
int osg_sim_autotune(osg_sim *s, int steps, int *tile, int *threads, int *n_sort);
/* Moving window along x1 at the speed of light (TILED engine; call before the first step):
 * every time the window has advanced one cell (the reference's move_boundary_space_global,
 * source/os-space.f90:508-566) the fields shift one cell towards lower x1 with the new plane
 * zeroed (move_window_vdf, source/vdf/os-vdf.f03:56-205), all cell indices shift by one and
 * particles leaving at x1 < 1 are dropped (move_window_species, source/spec/os-species.f03:
 * 171-229), and species `species` receives cold particles in the new x1 plane, ppc[d] per
 * cell on the OSIRIS lattice with the density of the piecewise-linear profile (nprof <= 8
 * points prof_x (global x1, increasing), prof_f; 0 outside) at the particle position
 * (inject_std, source/spec/psource/os-psource-std.f03:759-1120, :23).  x1 becomes an open
 * boundary: field guard cells zero, current beyond the edges dropped; x2 (x3) stay periodic. */
int osg_sim_set_window(osg_sim *s, int species, const int *ppc, int nprof, const double *prof_x,
                       const double *prof_f);
/* cell moves of the window so far */
int osg_sim_window_moves(osg_sim *s, long *moves);
/* guard cells per axis of the sim's grids (order-dependent, widened for smoothing) */
int osg_sim_guard_cells(osg_sim *s, int *gcl, int *gcu);
/* Checkpoint / restart of the device-resident state (the role of the reference's
 * write_restart / read_restart, source/os-main.f03:299-343, for the objects on this path):
 * the configuration, step count, moving-window state, every species' particles (reference
 * layout, the run's precision) and E, B are written to one binary file; osg_sim_restore
 * creates a simulation from it that continues the run.  The current is rebuilt by the next
 * step.  Returns OSG_ERR_ARG for a file that is missing, truncated or not a checkpoint. */
int osg_sim_checkpoint(osg_sim *s, const char *path);
int osg_sim_restore(const char *path, osg_sim **out);
/* the configuration a simulation runs with, its species count and their rqm (rqm may be
 * null; else room for OSG_MAX_SPECIES values) */
int osg_sim_get_config(osg_sim *s, osg_config *cfg, int *nspecies, double *rqm);
/* Number of kernel launches one step issues (for launch accounting). */
int osg_sim_launches_per_step(osg_sim *s);
/* Run n steps bracketed by CUDA events on the simulation's stream; *ms = device time. */
int osg_sim_time_steps(osg_sim *s, int nsteps, float *ms);

/* ------------------------------------------------------------ batched independent boxes --- */

/* Many independent periodic boxes of uneven size and particle load advanced together (mixed
 * precision, tiled engine, Boris pusher): one persistent push launch takes the tiles of all
 * boxes from a work list (heaviest boxes first), every field phase is one launch over all
 * boxes, and each full step is replayed from one CUDA graph.  Each box runs the time step of
 * osg_sim (phase order of iter_sim, source/os-simulation.f03:498-666) on its own fields.
 * A tile shape or CTA size left at 0 is chosen by the autotuner on the first step (or on
 * osg_batch_tuning): it times every candidate on a proxy batch of one box per distinct
 * (size, particles per cell) class and keeps the fastest. */
typedef struct osg_batch osg_batch;
typedef struct {
    int dim;          /* 2 or 3 */
    int order;        /* interpolation order 1..4 */
    double dt;        /* time step, shared by all boxes (Courant-checked per box) */
    int tile[3];      /* tile shape in cells; 0 = autotuned */
    int threads;      /* threads per push CTA (64..256, multiple of 32); 0 = autotuned */
    double capacity;  /* slots per tile as a multiple of the mean load (0 = 3.0) */
} osg_batch_config;

int osg_batch_create(const osg_batch_config *cfg, osg_batch **out);
int osg_batch_destroy(osg_batch *b);
/* add a box (cells and cell size per axis); returns its index (>= 0) or an error code */
int osg_batch_add_box(osg_batch *b, const int *nx, const double *dx);
/* add a species to a box from host arrays (reference layout, float); the data are copied.
 * Returns the species index (>= 0) or an error code.  Boxes and species come before the first
 * step. */
int osg_batch_add_species(osg_batch *b, int box, double rqm, long np, const int *ix,
                          const float *x, const float *u, const float *q);
/* builds the batch if needed (autotuning first when asked) and reports the tile shape and CTA
 * size in use */
int osg_batch_tuning(osg_batch *b, int *tile, int *threads);
int osg_batch_step(osg_batch *b, int nsteps);
/* n steps bracketed by CUDA events on the batch's stream; *ms = device time */
int osg_batch_time_steps(osg_batch *b, int nsteps, float *ms);
void *osg_batch_stream(osg_batch *b);
int osg_batch_num_boxes(osg_batch *b);
int osg_batch_launches_per_step(osg_batch *b);
/* FP64 diagnostics of one box, as osg_sim_energy */
int osg_batch_energy(osg_batch *b, int box, double *kinetic, double *field);
int osg_batch_get_fields(osg_batch *b, int box, float *e, float *bf, float *j);
int osg_batch_num_particles(osg_batch *b, int box, int species, long *np);
int osg_batch_get_species(osg_batch *b, int box, int species, int *ix, float *x, float *u,
                          float *q);

#ifdef __cplusplus
}
#endif

#endif
