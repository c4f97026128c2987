/*
 * fortran_shim.c -- the reference-named push/deposit entry points (vadvance_deposit_Nd_sK_)
 * forwarding to the typed C ABI of libosiris_gb300.so.  Compiled twice, once per precision
 * (OSG_PRECISION_SINGLE / OSG_PRECISION_DOUBLE), like the reference's own SINGLE / DOUBLE
 * builds of source/simd/os-spec-push-c.c.
 */
#include <stdio.h>

#include "include/osiris_gb300.h"
#include "include/osiris_gb300_fortran.h"

static __thread int g_status = OSG_OK;

int osg_fortran_status(void) { return g_status; }

static void forward(int dim, int order, int *ix, osg_real *x, osg_real *u, osg_real *q,
                    int *i0, int *i1, osg_real *rqm, osg_real *efield, osg_real *bfield,
                    int *emf_size, int *emf_offset, osg_real *j, int *j_size, int *j_offset,
                    double *dx, double *dt, double *ene)
{
#if defined(OSG_PRECISION_SINGLE)
    g_status = osg_vadvance_deposit_f32(dim, order, ix, x, u, q, *i0, *i1, *rqm, efield, bfield,
                                        emf_size, emf_offset, j, j_size, j_offset, dx, *dt, ene);
#else
    g_status = osg_vadvance_deposit_f64(dim, order, ix, x, u, q, *i0, *i1, *rqm, efield, bfield,
                                        emf_size, emf_offset, j, j_size, j_offset, dx, *dt, ene);
#endif
    if (g_status != OSG_OK)
        fprintf(stderr, "(*error*) vadvance_deposit_%dd_s%d: %s\n", dim, order,
                osg_last_error());
}

#define OSG_FORTRAN_PUSH_DEF(name, D, O)                                                      \
    OSG_FORTRAN_PUSH_DECL(name)                                                               \
    {                                                                                         \
        forward(D, O, ix, x, u, q, i0, i1, rqm, efield, bfield, emf_size, emf_offset, j,       \
                j_size, j_offset, dx, dt, ene);                                               \
    }

OSG_FORTRAN_PUSH_DEF(vadvance_deposit_1d_s1_, 1, 1)
OSG_FORTRAN_PUSH_DEF(vadvance_deposit_1d_s2_, 1, 2)
OSG_FORTRAN_PUSH_DEF(vadvance_deposit_1d_s3_, 1, 3)
OSG_FORTRAN_PUSH_DEF(vadvance_deposit_1d_s4_, 1, 4)
OSG_FORTRAN_PUSH_DEF(vadvance_deposit_2d_s1_, 2, 1)
OSG_FORTRAN_PUSH_DEF(vadvance_deposit_2d_s2_, 2, 2)
OSG_FORTRAN_PUSH_DEF(vadvance_deposit_2d_s3_, 2, 3)
OSG_FORTRAN_PUSH_DEF(vadvance_deposit_2d_s4_, 2, 4)
OSG_FORTRAN_PUSH_DEF(vadvance_deposit_3d_s1_, 3, 1)
OSG_FORTRAN_PUSH_DEF(vadvance_deposit_3d_s2_, 3, 2)
OSG_FORTRAN_PUSH_DEF(vadvance_deposit_3d_s3_, 3, 3)
OSG_FORTRAN_PUSH_DEF(vadvance_deposit_3d_s4_, 3, 4)

static void forward_cyl(int order, int *ix, osg_real *x, osg_real *u, osg_real *q, int *i0,
                        int *i1, osg_real *rqm, int *ilb2, osg_real *efield, osg_real *bfield,
                        int *emf_size, int *emf_offset, osg_real *j, int *j_size, int *j_offset,
                        double *dx, double *dt, double *ene)
{
#if defined(OSG_PRECISION_SINGLE)
    g_status = osg_vadvance_deposit_cyl_f32(order, ix, x, u, q, *i0, *i1, *rqm, *ilb2, efield,
                                            bfield, emf_size, emf_offset, j, j_size, j_offset,
                                            dx, *dt, ene);
#else
    g_status = osg_vadvance_deposit_cyl_f64(order, ix, x, u, q, *i0, *i1, *rqm, *ilb2, efield,
                                            bfield, emf_size, emf_offset, j, j_size, j_offset,
                                            dx, *dt, ene);
#endif
    if (g_status != OSG_OK)
        fprintf(stderr, "(*error*) vadvance_deposit_2d_cyl_s%d: %s\n", order, osg_last_error());
}

#define OSG_FORTRAN_PUSH_CYL_DEF(name, O)                                                     \
    OSG_FORTRAN_PUSH_CYL_DECL(name)                                                           \
    {                                                                                         \
        forward_cyl(O, ix, x, u, q, i0, i1, rqm, ilb2, efield, bfield, emf_size, emf_offset,  \
                    j, j_size, j_offset, dx, dt, ene);                                        \
    }

OSG_FORTRAN_PUSH_CYL_DEF(vadvance_deposit_2d_cyl_s1_, 1)
OSG_FORTRAN_PUSH_CYL_DEF(vadvance_deposit_2d_cyl_s2_, 2)
OSG_FORTRAN_PUSH_CYL_DEF(vadvance_deposit_2d_cyl_s3_, 3)
OSG_FORTRAN_PUSH_CYL_DEF(vadvance_deposit_2d_cyl_s4_, 4)
