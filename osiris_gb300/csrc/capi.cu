// capi.cu -- drop-in C entry points on host arrays (reference layout and semantics) and the
// error / version helpers of the library.
//
//   osg_vadvance_deposit_*   replaces FNAME(vadvance_deposit_{1d,2d,3d}_s{1..4})
//                            (source/simd/os-spec-push-avx2.c:255,471,1141;
//                             source/simd/os-spec-push-avx2d.c:263,481,1127)
//   osg_yee_advance_*        replaces advance_yee (source/emf/solver/os-emf-solver-yee.f03:542)
//   osg_periodic_*           replaces update_periodic_vdf (source/vdf/os-vdf-comm.f90:142)
//
// The reference kernels are called concurrently from OpenMP threads on disjoint particle
// ranges with private current grids (source/particles/os-particles.f03:1423-1435), so every
// calling thread gets its own stream and its own grow-only set of device buffers.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "fields.cuh"
#include "push_plain.cuh"

namespace osg {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

// per-thread device staging for the host-array entry points
struct Staging {
    cudaStream_t stream = nullptr;
    void *buf[8] = {nullptr};
    size_t cap[8] = {0};
    ~Staging()
    {
        for (int i = 0; i < 8; i++)
            if (buf[i]) cudaFree(buf[i]);
        if (stream) cudaStreamDestroy(stream);
    }
    int get(int slot, size_t bytes, void **out)
    {
        if (!stream) OSG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        if (bytes == 0) bytes = 16;
        if (cap[slot] < bytes) {
            if (buf[slot]) OSG_CUDA(cudaFree(buf[slot]));
            buf[slot] = nullptr;
            cap[slot] = 0;
            OSG_CUDA(cudaMalloc(&buf[slot], bytes));
            cap[slot] = bytes;
        }
        *out = buf[slot];
        return OSG_OK;
    }
};
static thread_local Staging g_stage;

static long grid_points(int dim, const int *size)
{
    long n = 1;
    for (int d = 0; d < dim; d++) n *= size[d];
    return n;
}

template <typename T>
static int push_host(int dim, int order, int *ix, T *x, T *u, T *q, int i0, int i1, T rqm,
                     const T *e, const T *b, const int *emf_size, const int *emf_off, T *j,
                     const int *j_size, const int *j_off, const double *dx, double dt,
                     double *ene)
{
    OSG_CHECK(dim >= 1 && dim <= 3 && order >= 1 && order <= 4, OSG_ERR_ARG,
              "dim %d / order %d not supported", dim, order);
    OSG_CHECK(ix && x && u && q && e && b && j && emf_size && emf_off && j_size && j_off && dx &&
                  ene,
              OSG_ERR_ARG, "null argument");
    OSG_CHECK(dt > 0, OSG_ERR_ARG, "dt must be positive");
    const long np = (long)i1 - i0 + 1;
    if (np <= 0) return OSG_OK;
    OSG_CHECK(i0 >= 1, OSG_ERR_ARG, "i0 must be >= 1");
    const long ge = grid_points(dim, emf_size) * 3, gj = grid_points(dim, j_size) * 3;
    void *d_ix, *d_x, *d_u, *d_q, *d_e, *d_b, *d_j, *d_misc;
    int rc;
    if ((rc = g_stage.get(0, sizeof(int) * dim * np, &d_ix))) return rc;
    if ((rc = g_stage.get(1, sizeof(T) * dim * np, &d_x))) return rc;
    if ((rc = g_stage.get(2, sizeof(T) * 3 * np, &d_u))) return rc;
    if ((rc = g_stage.get(3, sizeof(T) * np, &d_q))) return rc;
    if ((rc = g_stage.get(4, sizeof(T) * ge, &d_e))) return rc;
    if ((rc = g_stage.get(5, sizeof(T) * ge, &d_b))) return rc;
    if ((rc = g_stage.get(6, sizeof(T) * gj, &d_j))) return rc;
    if ((rc = g_stage.get(7, 64, &d_misc))) return rc;
    cudaStream_t st = g_stage.stream;
    const long o = (long)i0 - 1;
    double *d_ene = (double *)d_misc;
    int *d_status = (int *)((char *)d_misc + 16);
    OSG_CUDA(cudaMemsetAsync(d_misc, 0, 64, st));
    OSG_CUDA(cudaMemcpyAsync(d_ix, ix + dim * o, sizeof(int) * dim * np, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_x, x + dim * o, sizeof(T) * dim * np, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_u, u + 3 * o, sizeof(T) * 3 * np, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_q, q + o, sizeof(T) * np, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_e, e, sizeof(T) * ge, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_b, b, sizeof(T) * ge, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_j, j, sizeof(T) * gj, cudaMemcpyHostToDevice, st));
    PlainPushArgs<T> a = make_plain_args<T>(dim, order, (int *)d_ix, (T *)d_x, (T *)d_u,
                                            (const T *)d_q, np, rqm, (const T *)d_e,
                                            (const T *)d_b, emf_size, emf_off, (T *)d_j, j_size,
                                            j_off, dx, dt, d_ene, d_status);
    if ((rc = launch_plain_push<T>(dim, order, a, st))) return rc;
    OSG_CUDA(cudaGetLastError());
    OSG_CUDA(cudaMemcpyAsync(ix + dim * o, d_ix, sizeof(int) * dim * np, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaMemcpyAsync(x + dim * o, d_x, sizeof(T) * dim * np, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaMemcpyAsync(u + 3 * o, d_u, sizeof(T) * 3 * np, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaMemcpyAsync(j, d_j, sizeof(T) * gj, cudaMemcpyDeviceToHost, st));
    double h_ene = 0.0;
    int h_status = 0;
    OSG_CUDA(cudaMemcpyAsync(&h_ene, d_ene, sizeof(double), cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaMemcpyAsync(&h_status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaStreamSynchronize(st));
    *ene += h_ene;
    OSG_CHECK(!(h_status & OSG_STATUS_RANGE), OSG_ERR_RANGE,
              "particle cell index outside the field arrays (particles left untouched)");
    return OSG_OK;
}

template <typename T>
static int push_dev(int dim, int order, int *ix, T *x, T *u, const T *q, long np, T rqm,
                    const T *e, const T *b, const int *emf_size, const int *emf_off, T *j,
                    const int *j_size, const int *j_off, const double *dx, double dt,
                    double *d_ene, void *stream)
{
    OSG_CHECK(dim >= 1 && dim <= 3 && order >= 1 && order <= 4, OSG_ERR_ARG,
              "dim %d / order %d not supported", dim, order);
    OSG_CHECK(dt > 0 && d_ene, OSG_ERR_ARG, "bad dt or energy pointer");
    if (np <= 0) return OSG_OK;
    void *d_misc;
    int rc;
    if ((rc = g_stage.get(7, 64, &d_misc))) return rc;
    int *d_status = (int *)((char *)d_misc + 16);
    cudaStream_t st = (cudaStream_t)stream;
    OSG_CUDA(cudaMemsetAsync(d_status, 0, sizeof(int), st));
    PlainPushArgs<T> a = make_plain_args<T>(dim, order, ix, x, u, q, np, rqm, e, b, emf_size,
                                            emf_off, j, j_size, j_off, dx, dt, d_ene, d_status);
    if ((rc = launch_plain_push<T>(dim, order, a, st))) return rc;
    OSG_CUDA(cudaGetLastError());
    return OSG_OK;
}

template <typename T>
static int yee_host(int dim, const int *nx, const int *gcl, const int *gcu, T *e, T *b,
                    const T *j, const double *dx, double dt)
{
    OSG_CHECK(dim >= 1 && dim <= 3 && nx && gcl && gcu && e && b && j && dx, OSG_ERR_ARG,
              "bad arguments");
    for (int d = 0; d < dim; d++)
        OSG_CHECK(gcl[d] >= 1 && gcu[d] >= 2 && nx[d] >= 1, OSG_ERR_ARG,
                  "Yee needs >= 1 lower and >= 2 upper guard cells");
    GridDesc g = make_grid(dim, nx, gcl, gcu);
    const long n = g.npoints() * 3;
    void *d_e, *d_b, *d_j;
    int rc;
    if ((rc = g_stage.get(4, sizeof(T) * n, &d_e))) return rc;
    if ((rc = g_stage.get(5, sizeof(T) * n, &d_b))) return rc;
    if ((rc = g_stage.get(6, sizeof(T) * n, &d_j))) return rc;
    cudaStream_t st = g_stage.stream;
    OSG_CUDA(cudaMemcpyAsync(d_e, e, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_b, b, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_j, j, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    yee_advance<T>(g, (T *)d_e, (T *)d_b, (const T *)d_j, dx, dt, st);
    OSG_CUDA(cudaGetLastError());
    OSG_CUDA(cudaMemcpyAsync(e, d_e, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaMemcpyAsync(b, d_b, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaStreamSynchronize(st));
    return OSG_OK;
}

template <typename T>
static int periodic_host(int dim, const int *nx, const int *gcl, const int *gcu, T *f, int add)
{
    OSG_CHECK(dim >= 1 && dim <= 3 && nx && gcl && gcu && f, OSG_ERR_ARG, "bad arguments");
    for (int d = 0; d < dim; d++)
        OSG_CHECK(gcl[d] >= 0 && gcu[d] >= 0 && nx[d] >= gcl[d] + gcu[d], OSG_ERR_ARG,
                  "periodic update needs nx >= gcl + gcu");
    GridDesc g = make_grid(dim, nx, gcl, gcu);
    const long n = g.npoints() * 3;
    void *d_f;
    int rc;
    if ((rc = g_stage.get(6, sizeof(T) * n, &d_f))) return rc;
    cudaStream_t st = g_stage.stream;
    OSG_CUDA(cudaMemcpyAsync(d_f, f, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    periodic_update<T>(g, (T *)d_f, add, st);
    OSG_CUDA(cudaGetLastError());
    OSG_CUDA(cudaMemcpyAsync(f, d_f, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaStreamSynchronize(st));
    return OSG_OK;
}

} // namespace osg

using namespace osg;

extern "C" {

const char *osg_last_error(void) { return g_err; }

int osg_version(void) { return 10000; }

void *osg_host_alloc(size_t bytes)
{
    void *p = nullptr;
    if (cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) {
        set_error("cudaHostAlloc of %zu bytes failed", bytes);
        return nullptr;
    }
    return p;
}

int osg_host_free(void *p)
{
    if (p) OSG_CUDA(cudaFreeHost(p));
    return OSG_OK;
}

int osg_set_device(int device)
{
    OSG_CUDA(cudaSetDevice(device));
    return OSG_OK;
}

int osg_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

int osg_vadvance_deposit_f32(int dim, int order, int *ix, float *x, float *u, float *q, int i0,
                             int i1, float rqm, const float *efield, const float *bfield,
                             const int *emf_size, const int *emf_offset, float *j,
                             const int *j_size, const int *j_offset, const double *dx,
                             double dt, double *ene)
{
    return push_host<float>(dim, order, ix, x, u, q, i0, i1, rqm, efield, bfield, emf_size,
                            emf_offset, j, j_size, j_offset, dx, dt, ene);
}

int osg_vadvance_deposit_f64(int dim, int order, int *ix, double *x, double *u, double *q,
                             int i0, int i1, double rqm, const double *efield,
                             const double *bfield, const int *emf_size, const int *emf_offset,
                             double *j, const int *j_size, const int *j_offset,
                             const double *dx, double dt, double *ene)
{
    return push_host<double>(dim, order, ix, x, u, q, i0, i1, rqm, efield, bfield, emf_size,
                             emf_offset, j, j_size, j_offset, dx, dt, ene);
}

int osg_vadvance_deposit_dev_f32(int dim, int order, int *ix, float *x, float *u,
                                 const float *q, long np, float rqm, const float *efield,
                                 const float *bfield, const int *emf_size,
                                 const int *emf_offset, float *j, const int *j_size,
                                 const int *j_offset, const double *dx, double dt,
                                 double *d_ene, void *stream)
{
    return push_dev<float>(dim, order, ix, x, u, q, np, rqm, efield, bfield, emf_size,
                           emf_offset, j, j_size, j_offset, dx, dt, d_ene, stream);
}

int osg_vadvance_deposit_dev_f64(int dim, int order, int *ix, double *x, double *u,
                                 const double *q, long np, double rqm, const double *efield,
                                 const double *bfield, const int *emf_size,
                                 const int *emf_offset, double *j, const int *j_size,
                                 const int *j_offset, const double *dx, double dt,
                                 double *d_ene, void *stream)
{
    return push_dev<double>(dim, order, ix, x, u, q, np, rqm, efield, bfield, emf_size,
                            emf_offset, j, j_size, j_offset, dx, dt, d_ene, stream);
}

int osg_yee_advance_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *e,
                        float *b, const float *j, const double *dx, double dt)
{
    return yee_host<float>(dim, nx, gcl, gcu, e, b, j, dx, dt);
}

int osg_yee_advance_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *e,
                        double *b, const double *j, const double *dx, double dt)
{
    return yee_host<double>(dim, nx, gcl, gcu, e, b, j, dx, dt);
}

int osg_particle_wrap(int dim, const int *nx, long np, int *ix)
{
    OSG_CHECK(dim >= 1 && dim <= 3 && nx && (np == 0 || ix), OSG_ERR_ARG, "bad arguments");
    for (long p = 0; p < np; p++)
        for (int d = 0; d < dim; d++) {
            int &c = ix[dim * p + d];
            if (c < 1) c += nx[d];
            else if (c > nx[d]) c -= nx[d];
        }
    return OSG_OK;
}

int osg_periodic_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *f, int add)
{
    return periodic_host<float>(dim, nx, gcl, gcu, f, add);
}

int osg_periodic_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *f,
                     int add)
{
    return periodic_host<double>(dim, nx, gcl, gcu, f, add);
}

} // extern "C"
