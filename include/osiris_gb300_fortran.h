/*
 * osiris_gb300_fortran.h -- the reference's own Fortran-callable push/deposit symbols, exported
 * by the shim libraries built with the native library:
 *
 *   libosiris_gb300_single.so   REAL = float   (reference PRECISION = SINGLE)
 *   libosiris_gb300_double.so   REAL = double  (reference PRECISION = DOUBLE)
 *
 * Linking an OSIRIS build against one of them in place of source/simd/os-spec-push-c.c +
 * os-spec-current-c.c routes every call of the Fortran bridge (source/spec/os-spec-vpush.f03:
 * 70-95, 144-169, 217-246, 294-319) to the GPU.  Names carry one trailing underscore (the
 * FORTRANSINGLEUNDERSCORE convention of source/simd/fortran.h:15-40); the argument list is the
 * reference's (source/simd/os-spec-push-avx2.c:471-475 / os-spec-push-avx2d.c:481-485).
 *
 * The reference signatures return nothing and the reference kernels exit the process on bad
 * input; here nothing exits: the status of the calling thread's last call is available from
 * osg_fortran_status() (OSG_OK or an OSG_ERR_* code of osiris_gb300.h).
 */
#ifndef OSIRIS_GB300_FORTRAN_H
#define OSIRIS_GB300_FORTRAN_H

#ifdef __cplusplus
extern "C" {
#endif

#if defined(OSG_PRECISION_SINGLE)
typedef float osg_real;
#elif defined(OSG_PRECISION_DOUBLE)
typedef double osg_real;
#else
#error "define OSG_PRECISION_SINGLE or OSG_PRECISION_DOUBLE"
#endif

#define OSG_FORTRAN_PUSH_DECL(name)                                                           \
    void name(int *ix, osg_real *x, osg_real *u, osg_real *q, int *i0, int *i1,              \
              osg_real *rqm, osg_real *efield, osg_real *bfield, int *emf_size,              \
              int *emf_offset, osg_real *j, int *j_size, int *j_offset, double *dx,           \
              double *dt, double *ene)

OSG_FORTRAN_PUSH_DECL(vadvance_deposit_1d_s1_);
OSG_FORTRAN_PUSH_DECL(vadvance_deposit_1d_s2_);
OSG_FORTRAN_PUSH_DECL(vadvance_deposit_1d_s3_);
OSG_FORTRAN_PUSH_DECL(vadvance_deposit_1d_s4_);
OSG_FORTRAN_PUSH_DECL(vadvance_deposit_2d_s1_);
OSG_FORTRAN_PUSH_DECL(vadvance_deposit_2d_s2_);
OSG_FORTRAN_PUSH_DECL(vadvance_deposit_2d_s3_);
OSG_FORTRAN_PUSH_DECL(vadvance_deposit_2d_s4_);
OSG_FORTRAN_PUSH_DECL(vadvance_deposit_3d_s1_);
OSG_FORTRAN_PUSH_DECL(vadvance_deposit_3d_s2_);
OSG_FORTRAN_PUSH_DECL(vadvance_deposit_3d_s3_);
OSG_FORTRAN_PUSH_DECL(vadvance_deposit_3d_s4_);

/* 2D cylindrical (source/simd/os-spec-push-avx2.c:762-766, os-spec-push-avx2d.c:777-782): the
 * node's lower global cell along x2 (ilb2) follows rqm */
#define OSG_FORTRAN_PUSH_CYL_DECL(name)                                                       \
    void name(int *ix, osg_real *x, osg_real *u, osg_real *q, int *i0, int *i1,              \
              osg_real *rqm, int *ilb2, osg_real *efield, osg_real *bfield, int *emf_size,   \
              int *emf_offset, osg_real *j, int *j_size, int *j_offset, double *dx,           \
              double *dt, double *ene)

OSG_FORTRAN_PUSH_CYL_DECL(vadvance_deposit_2d_cyl_s1_);
OSG_FORTRAN_PUSH_CYL_DECL(vadvance_deposit_2d_cyl_s2_);
OSG_FORTRAN_PUSH_CYL_DECL(vadvance_deposit_2d_cyl_s3_);
OSG_FORTRAN_PUSH_CYL_DECL(vadvance_deposit_2d_cyl_s4_);

/* status (OSG_OK / OSG_ERR_*) of the calling thread's last vadvance_deposit_* call */
int osg_fortran_status(void);

#ifdef __cplusplus
}
#endif

#endif
