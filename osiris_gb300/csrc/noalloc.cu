// noalloc.cu -- the host-array push/deposit entry point for callers that must not allocate
// device memory (osg_vadvance_deposit_noalloc_f32).
//
// osg_vadvance_deposit_f32 stages its inputs and outputs in device buffers that it obtains with
// cudaMalloc on first use (and grows later).  Some hosts cannot tolerate that: programs that
// hand the whole GPU to their own pool allocator at start-up and treat any other allocation as
// an error, and time-stepping loops that budget device memory once and must not let a library
// allocate (cudaMalloc can synchronise the device and fragment a tightly packed memory plan).
// For them this file provides the same push with all its device staging inside one file-scope
// array of fixed size, reserved by the CUDA module when the library is loaded.
//
// Contract (also in include/osiris_gb300.h):
//   * the array holds OSG_NOALLOC_SCRATCH_BYTES (16 MiB) on every GPU that loads the library,
//     until the process exits;
//   * a call whose particles and fields do not fit is rejected with OSG_ERR_ARG and a message
//     giving the bytes it would need; split the particle range (i0..i1) into smaller calls;
//   * the first call on a device looks up the array's device address for that device (that
//     set-up should happen before any stream capture on the device);
//   * all calls share the one array: calls that overlap on the GPU (from several host threads
//     at once) race on it.  Each call clears the counters it needs and copies everything else
//     in fresh, so nothing carries over from a previous call.
// No cudaMalloc, cudaFree, stream creation or allocating library routine is called here.
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "push_plain.cuh"

namespace osg {

static __device__ __align__(256) unsigned char g_noalloc_scratch[OSG_NOALLOC_SCRATCH_BYTES];

// device address of g_noalloc_scratch per device ordinal, looked up once per device
static const int NOALLOC_MAX_DEVICES = 64;
static void *g_noalloc_ptr[NOALLOC_MAX_DEVICES];
static std::once_flag g_noalloc_once[NOALLOC_MAX_DEVICES];
static cudaError_t g_noalloc_err[NOALLOC_MAX_DEVICES];

static int noalloc_scratch(void **out)
{
    int dev = 0;
    OSG_CUDA(cudaGetDevice(&dev));
    OSG_CHECK(dev >= 0 && dev < NOALLOC_MAX_DEVICES, OSG_ERR_ARG, "device ordinal %d too large",
              dev);
    std::call_once(g_noalloc_once[dev], [dev]() {
        // the current device is `dev` here (same thread, just queried)
        g_noalloc_err[dev] = cudaGetSymbolAddress(&g_noalloc_ptr[dev], g_noalloc_scratch);
    });
    if (g_noalloc_err[dev] != cudaSuccess || !g_noalloc_ptr[dev]) {
        set_error("cudaGetSymbolAddress of the no-allocation scratch failed on device %d: %s",
                  dev, cudaGetErrorString(g_noalloc_err[dev]));
        return OSG_ERR_CUDA;
    }
    *out = g_noalloc_ptr[dev];
    return OSG_OK;
}

static size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

} // namespace osg

using namespace osg;

extern "C" int osg_vadvance_deposit_noalloc_f32(int dim, int order, int *ix, float *x,
                                                 float *u, float *q, int i0, int i1, float rqm,
                                                 const float *efield, const float *bfield,
                                                 const int *emf_size, const int *emf_offset,
                                                 float *j, const int *j_size,
                                                 const int *j_offset, const double *dx,
                                                 double dt, double *ene)
{
    OSG_CHECK(dim >= 1 && dim <= 3 && order >= 1 && order <= 4, OSG_ERR_ARG,
              "dim %d / order %d not supported", dim, order);
    OSG_CHECK(ix && x && u && q && efield && bfield && j && emf_size && emf_offset && j_size &&
                  j_offset && dx && ene,
              OSG_ERR_ARG, "null argument");
    OSG_CHECK(dt > 0, OSG_ERR_ARG, "dt must be positive");
    const long np = (long)i1 - i0 + 1;
    if (np <= 0) return OSG_OK;
    OSG_CHECK(i0 >= 1, OSG_ERR_ARG, "i0 must be >= 1");
    long ge = 3, gj = 3;
    for (int d = 0; d < dim; d++) {
        OSG_CHECK(emf_size[d] > 0 && j_size[d] > 0, OSG_ERR_ARG, "bad grid size");
        ge *= emf_size[d];
        gj *= j_size[d];
    }
    // scratch layout: [energy + status | E | B | J | ix | x | u | q], 256-byte aligned pieces
    const size_t b_misc = 256;
    const size_t b_e = align256(sizeof(float) * ge), b_j = align256(sizeof(float) * gj);
    const size_t b_ix = align256(sizeof(int) * dim * np), b_x = align256(sizeof(float) * dim * np);
    const size_t b_u = align256(sizeof(float) * 3 * np), b_q = align256(sizeof(float) * np);
    const size_t need = b_misc + 2 * b_e + b_j + b_ix + b_x + b_u + b_q;
    OSG_CHECK(need <= (size_t)OSG_NOALLOC_SCRATCH_BYTES, OSG_ERR_ARG,
              "this call needs %zu bytes of device scratch but the no-allocation entry point "
              "has %zu; push fewer particles per call (i1 - i0) or use osg_vadvance_deposit_f32",
              need, (size_t)OSG_NOALLOC_SCRATCH_BYTES);
    void *base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc) return rc;
    char *p = (char *)base;
    double *d_ene = (double *)p;
    int *d_status = (int *)(p + 16);
    float *d_e = (float *)(p + b_misc);
    float *d_b = (float *)((char *)d_e + b_e);
    float *d_j = (float *)((char *)d_b + b_e);
    int *d_ix = (int *)((char *)d_j + b_j);
    float *d_x = (float *)((char *)d_ix + b_ix);
    float *d_u = (float *)((char *)d_x + b_x);
    float *d_q = (float *)((char *)d_u + b_u);
    cudaStream_t st = cudaStreamPerThread;
    const long o = (long)i0 - 1;
    // the array keeps the previous call's contents: clear the accumulators, copy the rest in
    OSG_CUDA(cudaMemsetAsync(p, 0, b_misc, st));
    OSG_CUDA(cudaMemcpyAsync(d_ix, ix + dim * o, sizeof(int) * dim * np, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_x, x + dim * o, sizeof(float) * dim * np, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_u, u + 3 * o, sizeof(float) * 3 * np, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_q, q + o, sizeof(float) * np, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_e, efield, sizeof(float) * ge, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_b, bfield, sizeof(float) * ge, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_j, j, sizeof(float) * gj, cudaMemcpyHostToDevice, st));
    PlainPushArgs<float> a = make_plain_args<float>(dim, order, d_ix, d_x, d_u, d_q, np, rqm, d_e,
                                                    d_b, emf_size, emf_offset, d_j, j_size,
                                                    j_offset, dx, dt, d_ene, d_status);
    if ((rc = launch_plain_push<float>(dim, order, a, st))) return rc;
    OSG_CUDA(cudaGetLastError());
    OSG_CUDA(cudaMemcpyAsync(ix + dim * o, d_ix, sizeof(int) * dim * np, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaMemcpyAsync(x + dim * o, d_x, sizeof(float) * dim * np, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaMemcpyAsync(u + 3 * o, d_u, sizeof(float) * 3 * np, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaMemcpyAsync(j, d_j, sizeof(float) * gj, cudaMemcpyDeviceToHost, st));
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
