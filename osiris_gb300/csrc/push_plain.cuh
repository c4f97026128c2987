// push_plain.cuh -- launch interface of the plain (one thread per particle) push + deposit.
#pragma once

#include <cuda_runtime.h>

namespace osg {

// bits of the device status word shared by all kernels of a launch sequence
enum : int {
    OSG_STATUS_RANGE = 1,     // a particle cell index would reach outside the arrays
    OSG_STATUS_OVERFLOW = 2,  // a tile had no free particle slot
    OSG_STATUS_NAN = 4,       // non-finite value detected
};

template <typename T> struct PlainPushArgs {
    int *ix;
    T *x, *u;
    const T *q;
    long np;
    T tem;                 // dt / (2 rqm), rounded from double as the reference does
    T dtdx[3];             // dt / dx
    T jn[3];               // current normalisation dx / dt / dim
    const T *efield;       // shifted so that (cell, k) indexes the stencil directly
    const T *bfield;
    T *j;
    long emf_Dy, emf_Dz, j_Dy, j_Dz;
    int emf_off[3], emf_size[3], j_off[3], j_size[3];
    int wrap[3];           // > 0: periodic wrap of the stored cell index into [1, wrap[d]]
    int reflect[3];        // > 0: conducting walls at the edges of [1, reflect[d]]: specular
                           // reflection of a particle that crossed one
    int absorb[3];         // > 0: open edges of [1, absorb[d]]: a particle that crossed one is
                           // absorbed (charge and momentum set to 0 in q_absorb and u)
    T *q_absorb;           // the charges, writable (only with an absorbing axis)
    int thermal[3];        // > 0: thermal-bath edges of [1, thermal[d]]: a particle that crossed
                           // one is re-emitted with new momenta (thermal_reemit)
    T uth_bnd[3], ufl_bnd[3];   // the bath's thermal and fluid momenta
    int thermal_type;           // 0 thermal, 1 random dir, 2 waterbag
    const unsigned long long *step;   // device step counter (re-emission random stream)
    unsigned int rng_key[2];          // the stream's key: seed, species
    int pusher;            // OSG_PUSHER_*
    T qm;                  // 1 / rqm (exact pusher)
    T rqm;                 // the species' rqm (Euler-rotation pusher)
    double dt_full;        // the double time step (exact pusher, cylindrical radial move)
    int cyl;               // 1: 2D cylindrical (x1 = z, x2 = r): radial move and p_r, p_theta
                           // correction in double (vadvance_deposit_2d_cyl_sK)
    double cyl_gshift;     // global x2 cell of local cell 0: ilb2 - 2 (odd orders), - 2.5
    double cyl_dr, cyl_rdr;   // dx2 and 1 / dx2
    double iter_tol;       // Newton tolerance of the exact pusher
    double *ene;           // device accumulator (incremented)
    int *status;           // device status word (OR of OSG_STATUS_*)
};

template <typename T>
PlainPushArgs<T> make_plain_args(int dim, int order, int *ix, T *x, T *u, const T *q, long np,
                                 T rqm, const T *e, const T *b, const int *emf_size,
                                 const int *emf_off, T *j, const int *j_size, const int *j_off,
                                 const double *dx, double dt, double *d_ene, int *d_status);

template <typename T>
int launch_plain_push(int dim, int order, const PlainPushArgs<T> &a, cudaStream_t st);

} // namespace osg
