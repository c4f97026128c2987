/*
 * pic_oracle.h -- TEST INFRASTRUCTURE ONLY: declarations of the CPU parity oracle
 * (pic_oracle.c).  Loaded from Python through ctypes by tests/, __graft_entry__.smoke() and
 * the CPU-baseline leg of bench.py; never linked by the product library.
 */
#ifndef PIC_ORACLE_H
#define PIC_ORACLE_H

#include <stdint.h>

typedef struct {
    uint32_t mt[624];
    int mti;
    int have_gauss;
    double gauss;
} ora_mt;

/* push + deposit with the reference argument conventions (1-based inclusive [i0, i1];
 * fields include guard cells; emf_off = lower guard-cell count) */
int ora_push_f32(int dim, int order, int *ix, float *x, float *u, float *q, int i0, int i1,
                 float rqm, float *e, float *b, int *emf_size, int *emf_off, float *j,
                 int *j_size, int *j_off, double *dx, double dt, double *ene);
int ora_push_f64(int dim, int order, int *ix, double *x, double *u, double *q, int i0, int i1,
                 double rqm, double *e, double *b, int *emf_size, int *emf_off, double *j,
                 int *j_size, int *j_off, double *dx, double dt, double *ene);

/* the 2D cylindrical push + deposit (vadvance_deposit_2d_cyl_sK: x1 = z, x2 = r; ilb2 = the
 * node's lower global cell along x2) */
int ora_push_cyl_f32(int order, int *ix, float *x, float *u, float *q, int i0, int i1,
                     float rqm, int ilb2, float *e, float *b, int *emf_size, int *emf_off,
                     float *j, int *j_size, int *j_off, double *dx, double dt, double *ene);
int ora_push_cyl_f64(int order, int *ix, double *x, double *u, double *q, int i0, int i1,
                     double rqm, int ilb2, double *e, double *b, int *emf_size, int *emf_off,
                     double *j, int *j_size, int *j_off, double *dx, double dt, double *ene);

/* the same with the exact momentum update (push_type = "exact", dudt_exact) at tolerance tol */
int ora_push_exact_f32(int dim, int order, int *ix, float *x, float *u, float *q, int i0, int i1,
                       float rqm, float *e, float *b, int *emf_size, int *emf_off, float *j,
                       int *j_size, int *j_off, double *dx, double dt, double tol, double *ene);
int ora_push_exact_f64(int dim, int order, int *ix, double *x, double *u, double *q, int i0,
                       int i1, double rqm, double *e, double *b, int *emf_size, int *emf_off,
                       double *j, int *j_size, int *j_off, double *dx, double dt, double tol,
                       double *ene);
/* momentum update of n particles in given fields e(3,n), b(3,n): pusher 1 exact, 2 Vay, 3 HC */
void ora_dudt_pusher_f32(int pusher, int n, const float *e, const float *b, float *u,
                         const float *q, float rqm, double dt, double tol, double *ene);
void ora_dudt_pusher_f64(int pusher, int n, const double *e, const double *b, double *u,
                         const double *q, double rqm, double dt, double tol, double *ene);
void ora_dudt_exact_f32(int n, const float *e, const float *b, float *u, const float *q,
                        float rqm, double dt, double tol, double *ene);
void ora_dudt_exact_f64(int n, const double *e, const double *b, double *u, const double *q,
                        double rqm, double dt, double tol, double *ene);

void ora_yee_advance_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *e,
                         float *b, const float *j, const double *dx, double dt);
void ora_yee_advance_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *e,
                         double *b, const double *j, const double *dx, double dt);
void ora_periodic_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *f, int add);
void ora_periodic_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *f, int add);
/* conducting walls on the axes in `walls`: kind 0 E / 1 B (guards set from images), 2 J (guards
 * added into the box); the step functions below use the walls set by ora_set_walls_* */
void ora_walls_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *f, int kind,
                   int walls, int order);
void ora_walls_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *f, int kind,
                   int walls, int order);
void ora_set_walls_f32(int walls);
/* the walled axes in `pmc` are perfect magnetic conductors in the steps below */
void ora_set_pmc_f32(int pmc);
void ora_set_pmc_f64(int pmc);
void ora_set_walls_f64(int walls);
/* moving window along x1 (on = 1) for the step functions below: no x1 guard update of E, B or
 * J, particles absorbed below cell 1 (cell index set to ORA_GONE, -2^28) and reflected above
 * nx */
void ora_set_window_f32(int on);
void ora_set_window_f64(int on);
/* Lindman open boundaries at both edges of `axis` (-1: none) for the step functions below;
 * `state` holds 15 reals per interior point of the other axes, zeroed before the first step
 * and kept between steps */
/* thermal-bath particle boundary on the axes in `mask` for the step functions below (mask 0:
 * none); `step` keys the random stream of the next step */
void ora_set_thermal(int mask, const double *uth, const double *ufl, uint32_t seed,
                     uint64_t step, int ttype);
void ora_lindman_phase_f32(int dim, const int *nx, const int *gcl, const int *gcu, int d,
                           int what, float *e, float *b, float *st, const double *dx, double dt);
void ora_lindman_phase_f64(int dim, const int *nx, const int *gcl, const int *gcu, int d,
                           int what, double *e, double *b, double *st, const double *dx,
                           double dt);
void ora_set_open_f32(int axis, float *state);
void ora_set_open_f64(int axis, double *state);
/* PML walls of nb cells at both edges of the axes in mask of a 2D box (corners covered by
 * the x1 walls); the state (walls and attenuation tables) is ora_pml_state_size reals, set up
 * by ora_pml_init */
long ora_pml_state_size_f32(int dim, const int *nx, const int *gcl, const int *gcu, int mask,
                            int nb);
long ora_pml_state_size_f64(int dim, const int *nx, const int *gcl, const int *gcu, int mask,
                            int nb);
void ora_pml_init_f32(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                      const double *dx, double dt, float *st);
void ora_pml_init_f64(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                      const double *dx, double dt, double *st);
void ora_pml_phase_f32(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                       int what, float *e, float *b, float *st, const double *dx, double dt);
void ora_pml_phase_f64(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                       int what, double *e, double *b, double *st, const double *dx, double dt);
void ora_pml_shift_x_f32(int dim, const int *nx, const int *gcl, const int *gcu, int mask,
                         int nb, float *st);
void ora_pml_shift_x_f64(int dim, const int *nx, const int *gcl, const int *gcu, int mask,
                         int nb, double *st);
void ora_set_pml_f32(int mask, int nb, float *state);
void ora_set_pml_f64(int mask, int nb, double *state);
void ora_field_energy_f32(int dim, const int *nx, const int *gcl, const int *gcu,
                          const float *f, const double *dx, double *out);
void ora_field_energy_f64(int dim, const int *nx, const int *gcl, const int *gcu,
                          const double *f, const double *dx, double *out);
void ora_deposit_rho_f32(int dim, int order, const int *nx, const int *gcl, const int *gcu,
                         double *rho, int np, const int *ix, const float *x, const float *q);
void ora_deposit_rho_f64(int dim, int order, const int *nx, const int *gcl, const int *gcu,
                         double *rho, int np, const int *ix, const double *x, const double *q);
void ora_div_f32(int dim, const int *nx, const int *gcl, const int *gcu, const float *f,
                 const double *dx, double *div);
void ora_div_f64(int dim, const int *nx, const int *gcl, const int *gcu, const double *f,
                 const double *dx, double *div);
void ora_spline_weights_f64(int order, double x, double *w);
void ora_smooth_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *f,
                    const int *ord, const float *coef);
void ora_smooth_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *f,
                    const int *ord, const double *coef);
void ora_set_smooth_f32(const int *ord, const float *coef);
void ora_set_smooth_f64(const int *ord, const double *coef);
void ora_set_emf_smooth_f32(const int *ord, const float *coef);
void ora_set_emf_smooth_f64(const int *ord, const double *coef);

void ora_wrap(int dim, const int *nx, int np, int *ix);
void ora_sort_index(int dim, const int *nx, int np, const int *ix, int *new_idx);

void ora_mt_seed(ora_mt *r, int seed);
int32_t ora_mt_int32(ora_mt *r);
double ora_gaussian(ora_mt *r);
int ora_load_f32(ora_mt *rng, int dim, const int *nx, const int *ppc_d, const double *dx,
                 double rqm, const double *uth, const double *ufl, double amp, double kmode,
                 int *ix, float *x, float *u, float *q);
int ora_load_f64(ora_mt *rng, int dim, const int *nx, const int *ppc_d, const double *dx,
                 double rqm, const double *uth, const double *ufl, double amp, double kmode,
                 int *ix, double *x, double *u, double *q);

int ora_step_f32(int dim, int order, const int *nx, const int *gcl, const int *gcu,
                 const double *dx, double dt, float *e, float *b, float *j, int nspec,
                 const int *np, int **ix, float **x, float **u, float **q, const float *rqm,
                 double *ene, int nthreads);
int ora_step_f64(int dim, int order, const int *nx, const int *gcl, const int *gcu,
                 const double *dx, double dt, double *e, double *b, double *j, int nspec,
                 const int *np, int **ix, double **x, double **u, double **q,
                 const double *rqm, double *ene, int nthreads);
int ora_step_pusher_f32(int pusher, int dim, int order, const int *nx, const int *gcl,
                        const int *gcu, const double *dx, double dt, float *e, float *b,
                        float *j, int nspec, const int *np, int **ix, float **x, float **u,
                        float **q, const float *rqm, double *ene, int nthreads, double tol);
int ora_step_pusher_f64(int pusher, int dim, int order, const int *nx, const int *gcl,
                        const int *gcu, const double *dx, double dt, double *e, double *b,
                        double *j, int nspec, const int *np, int **ix, double **x, double **u,
                        double **q, const double *rqm, double *ene, int nthreads, double tol);
int ora_push_pusher_f32(int pusher, int dim, int order, int *ix, float *x, float *u, float *q,
                        int i0, int i1, float rqm, float *e, float *b, int *emf_size,
                        int *emf_off, float *j, int *j_size, int *j_off, double *dx, double dt,
                        double tol, double *ene);
int ora_push_pusher_f64(int pusher, int dim, int order, int *ix, double *x, double *u,
                        double *q, int i0, int i1, double rqm, double *e, double *b,
                        int *emf_size, int *emf_off, double *j, int *j_size, int *j_off,
                        double *dx, double dt, double tol, double *ene);
int ora_max_threads(void);

#endif
