// fields.cuh -- grid kernels (Yee, periodic guard update, FP64 diagnostics).
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace osg {

template <typename T>
void yee_advance(const GridDesc &g, T *e, T *b, const T *j, const double *dx, double dt,
                 cudaStream_t st);

// add = 1: fold guard cells into their periodic images (current); add = 0: replace
template <typename T> void periodic_update(const GridDesc &g, T *f, int add, cudaStream_t st);

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
