// capi.cu -- drop-in C entry points on host arrays (reference layout and semantics) and the
// error / version helpers of the library.
//
//   osg_vadvance_deposit_*   replaces FNAME(vadvance_deposit_{1d,2d,3d}_s{1..4})
//                            (source/simd/os-spec-push-avx2.c:255,471,1141;
//                             source/simd/os-spec-push-avx2d.c:263,481,1127)
//   osg_vadvance_deposit_cyl_*  replaces FNAME(vadvance_deposit_2d_cyl_s{1..4})
//                            (source/simd/os-spec-push-avx2.c:762;
//                             source/simd/os-spec-push-avx2d.c:777)
//   osg_yee_advance_*        replaces advance_yee (source/emf/solver/os-emf-solver-yee.f03:542)
//   osg_periodic_*           replaces update_periodic_vdf (source/vdf/os-vdf-comm.f90:142)
//
// The reference kernels are called concurrently from OpenMP threads on disjoint particle
// ranges with private current grids (source/particles/os-particles.f03:1423-1435), so every
// calling thread gets its own stream and its own grow-only set of device buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "fields.cuh"
#include "pic_math.cuh"
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
static const int SIDE_STREAMS = 3;
static const int MAX_PUSH_CHUNKS = 64;

// chunks of the staged host-array push (above 2 M particles): OSG_DROPIN_CHUNKS, default 16
static int push_chunks()
{
    static int n = 0;
    if (n == 0) {
        const char *ev = getenv("OSG_DROPIN_CHUNKS");
        const int v = ev ? atoi(ev) : 16;
        n = v < 1 ? 1 : (v > MAX_PUSH_CHUNKS ? MAX_PUSH_CHUNKS : v);
    }
    return n;
}

struct Staging {
    cudaStream_t stream = nullptr;
    // the chunked host-array push: copies in, pushes and copies out each on their own stream
    // (side[0..2]), chunk by chunk, joined by per-chunk events
    cudaStream_t side[SIDE_STREAMS] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev[2 + 2 * MAX_PUSH_CHUNKS] = {nullptr};
    void *buf[8] = {nullptr};
    size_t cap[8] = {0};
    ~Staging()
    {
        for (int i = 0; i < 8; i++)
            if (buf[i]) cudaFree(buf[i]);
        for (int i = 0; i < 2 + 2 * MAX_PUSH_CHUNKS; i++)
            if (ev[i]) cudaEventDestroy(ev[i]);
        for (int i = 0; i < SIDE_STREAMS; i++)
            if (side[i]) cudaStreamDestroy(side[i]);
        if (stream) cudaStreamDestroy(stream);
    }
    int streams()
    {
        if (!stream) OSG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        for (int i = 0; i < SIDE_STREAMS; i++)
            if (!side[i]) OSG_CUDA(cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking));
        for (int i = 0; i < 2 + 2 * MAX_PUSH_CHUNKS; i++)
            if (!ev[i]) OSG_CUDA(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
        return OSG_OK;
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

// Particle arrays the push kernel addresses in place, without staging copies: device or
// managed memory and -- on systems whose GPU reads and writes pageable host memory coherently
// through the host page tables (Grace with NVLink-C2C) -- pageable host memory.  nullptr: the
// array is staged through the copy pipeline.  Page-locked host memory is staged: on GB300 the
// copy engines' pipeline moved the 2D two-stream drop-in step at 2.8e9 particle-steps/s, the
// push kernel reading and writing the same page-locked arrays in place at 2.1e9.
// OSG_DROPIN_DIRECT=0 turns the in-place path off (every call stages).
static bool pageable_direct()
{
    static int ok = -1;
    if (ok < 0) {
        int dev = 0, a = 0, b = 0;
        const char *ev = getenv("OSG_DROPIN_DIRECT");
        ok = 0;
        if (!(ev && atoi(ev) == 0) && cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) ==
                cudaSuccess)
            ok = a == 1 && b == 1;
        cudaGetLastError();
    }
    return ok == 1;
}

template <typename P> static P *device_view(P *p)
{
    const char *ev = getenv("OSG_DROPIN_DIRECT");
    if (ev && atoi(ev) == 0) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, (const void *)p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    switch (at.type) {
    case cudaMemoryTypeDevice:
    case cudaMemoryTypeManaged: return p;
    case cudaMemoryTypeHost: return nullptr;
    default: return pageable_direct() ? p : nullptr;
    }
}

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
                     double *ene, int pusher = OSG_PUSHER_BORIS, double iter_tol = 1.0e-3,
                     int cyl = 0, int ilb2 = 0)
{
    OSG_CHECK(pusher >= OSG_PUSHER_BORIS && pusher <= OSG_PUSHER_COND_VAY &&
                  (pusher != OSG_PUSHER_EXACT || iter_tol > 0),
              OSG_ERR_ARG, "bad pusher / iteration tolerance");
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
    const long o = (long)i0 - 1;
    // in place when the GPU can address every particle array (the particles then cross the
    // host link inside the push kernel, reads and writes at once, with no staging pipeline)
    int *v_ix = device_view(ix + dim * o);
    T *v_x = device_view(x + dim * o), *v_u = device_view(u + 3 * o);
    const T *v_q = device_view((const T *)(q + o));
    const bool direct = v_ix && v_x && v_u && v_q;
    void *d_ix = nullptr, *d_x = nullptr, *d_u = nullptr, *d_q = nullptr;
    void *d_e, *d_b, *d_j, *d_misc;
    int rc;
    if (!direct) {
        if ((rc = g_stage.get(0, sizeof(int) * dim * np, &d_ix))) return rc;
        if ((rc = g_stage.get(1, sizeof(T) * dim * np, &d_x))) return rc;
        if ((rc = g_stage.get(2, sizeof(T) * 3 * np, &d_u))) return rc;
        if ((rc = g_stage.get(3, sizeof(T) * np, &d_q))) return rc;
    }
    if ((rc = g_stage.get(4, sizeof(T) * ge, &d_e))) return rc;
    if ((rc = g_stage.get(5, sizeof(T) * ge, &d_b))) return rc;
    if ((rc = g_stage.get(6, sizeof(T) * gj, &d_j))) return rc;
    if ((rc = g_stage.get(7, 64, &d_misc))) return rc;
    if ((rc = g_stage.streams())) return rc;
    cudaStream_t st = g_stage.stream;
    cudaStream_t s_in = g_stage.side[0], s_push = g_stage.side[1], s_out = g_stage.side[2];
    cudaEvent_t *ev = g_stage.ev;
    double *d_ene = (double *)d_misc;
    int *d_status = (int *)((char *)d_misc + 16);
    OSG_CUDA(cudaMemsetAsync(d_misc, 0, 64, st));
    OSG_CUDA(cudaMemcpyAsync(d_e, e, sizeof(T) * ge, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_b, b, sizeof(T) * ge, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_j, j, sizeof(T) * gj, cudaMemcpyHostToDevice, st));
    auto setup = [&](PlainPushArgs<T> &a) {
        a.pusher = pusher;
        a.iter_tol = iter_tol;
        if (cyl) {
            a.cyl = 1;
            a.cyl_gshift = (order == 1 || order == 3) ? (double)(ilb2 - 2)
                                                      : (double)(ilb2 - 2) - 0.5;
        }
        if (pusher >= OSG_PUSHER_VAY) a.tem = (T)pusher_tem(pusher, dt, (double)rqm);
    };
    if (direct) {
        PlainPushArgs<T> a = make_plain_args<T>(dim, order, v_ix, v_x, v_u, v_q, np, rqm,
                                                (const T *)d_e, (const T *)d_b, emf_size, emf_off,
                                                (T *)d_j, j_size, j_off, dx, dt, d_ene, d_status);
        setup(a);
        if ((rc = launch_plain_push<T>(dim, order, a, st))) return rc;
        OSG_CUDA(cudaGetLastError());
    } else {
        OSG_CUDA(cudaEventRecord(ev[0], st));
        OSG_CUDA(cudaStreamWaitEvent(s_in, ev[0], 0));
        OSG_CUDA(cudaStreamWaitEvent(s_push, ev[0], 0));
        OSG_CUDA(cudaStreamWaitEvent(s_out, ev[0], 0));
        // The particle range goes in chunks through a three-stage pipeline: the copies in of
        // chunk k + 1, the push of chunk k and the copies out of chunk k - 1 run at once, and
        // neither copy direction waits for the other (per-particle results do not depend on the
        // chunking; the current and energy sums are atomic either way).
        // chunk starts on a multiple of 4096 particles, so that every array's copy starts on a
        // 16 KB boundary of the (aligned) host array: copies of unaligned ranges measured ~20%
        // slower over the host link
        const long nck = np > (2L << 20) ? push_chunks() : 1;
        const long chunk = nck == 1 ? np : ((np + nck - 1) / nck + 4095) & ~4095L;
        for (long c0 = 0, k = 0; c0 < np; c0 += chunk, k++) {
            const long n = std::min(chunk, np - c0), h = o + c0;
            int *cix = (int *)d_ix + dim * c0;
            T *cx = (T *)d_x + dim * c0, *cu = (T *)d_u + 3 * c0, *cq = (T *)d_q + c0;
            OSG_CUDA(cudaMemcpyAsync(cix, ix + dim * h, sizeof(int) * dim * n,
                                     cudaMemcpyHostToDevice, s_in));
            OSG_CUDA(cudaMemcpyAsync(cx, x + dim * h, sizeof(T) * dim * n, cudaMemcpyHostToDevice,
                                     s_in));
            OSG_CUDA(cudaMemcpyAsync(cu, u + 3 * h, sizeof(T) * 3 * n, cudaMemcpyHostToDevice,
                                     s_in));
            OSG_CUDA(cudaMemcpyAsync(cq, q + h, sizeof(T) * n, cudaMemcpyHostToDevice, s_in));
            OSG_CUDA(cudaEventRecord(ev[2 + 2 * k], s_in));
            OSG_CUDA(cudaStreamWaitEvent(s_push, ev[2 + 2 * k], 0));
            PlainPushArgs<T> a = make_plain_args<T>(
                dim, order, cix, cx, cu, (const T *)cq, n, rqm, (const T *)d_e, (const T *)d_b,
                emf_size, emf_off, (T *)d_j, j_size, j_off, dx, dt, d_ene, d_status);
            setup(a);
            if ((rc = launch_plain_push<T>(dim, order, a, s_push))) return rc;
            OSG_CUDA(cudaGetLastError());
            OSG_CUDA(cudaEventRecord(ev[3 + 2 * k], s_push));
            OSG_CUDA(cudaStreamWaitEvent(s_out, ev[3 + 2 * k], 0));
            OSG_CUDA(cudaMemcpyAsync(ix + dim * h, cix, sizeof(int) * dim * n,
                                     cudaMemcpyDeviceToHost, s_out));
            OSG_CUDA(cudaMemcpyAsync(x + dim * h, cx, sizeof(T) * dim * n, cudaMemcpyDeviceToHost,
                                     s_out));
            OSG_CUDA(cudaMemcpyAsync(u + 3 * h, cu, sizeof(T) * 3 * n, cudaMemcpyDeviceToHost,
                                     s_out));
        }
        OSG_CUDA(cudaEventRecord(ev[1], s_out));
        OSG_CUDA(cudaStreamWaitEvent(st, ev[1], 0));
    }
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

static int smooth_spec(int dim, const int *type, const int *order, SmoothSpec *sp)
{
    memset(sp, 0, sizeof *sp);
    for (int d = 0; d < dim; d++) {
        int n = 0;
        OSG_CHECK(smooth_coefficients(type[d], order[d], sp->c[d], &n) == OSG_OK, OSG_ERR_ARG,
                  "bad smoothing type %d / order %d", type[d], order[d]);
        sp->order[d] = n;
    }
    return OSG_OK;
}

template <typename T>
static int smooth_host(int dim, const int *nx, const int *gcl, const int *gcu, T *f,
                       const int *type, const int *order)
{
    OSG_CHECK(dim >= 1 && dim <= 3 && nx && gcl && gcu && f && type && order, OSG_ERR_ARG,
              "bad arguments");
    SmoothSpec sp;
    int rc = smooth_spec(dim, type, order, &sp);
    if (rc) return rc;
    GridDesc g = make_grid(dim, nx, gcl, gcu);
    const long n = g.npoints() * 3;
    void *d_f, *d_t;
    if ((rc = g_stage.get(5, sizeof(T) * n, &d_f))) return rc;
    if ((rc = g_stage.get(6, sizeof(T) * n, &d_t))) return rc;
    cudaStream_t st = g_stage.stream;
    OSG_CUDA(cudaMemcpyAsync(d_f, f, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    smooth_field<T>(g, sp, (T *)d_f, (T *)d_t, st);
    OSG_CUDA(cudaGetLastError());
    OSG_CUDA(cudaMemcpyAsync(f, d_f, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaStreamSynchronize(st));
    return OSG_OK;
}

template <typename T>
static int lindman_host(int dim, const int *nx, const int *gcl, const int *gcu, int axis,
                        int what, T *e, T *b, T *state, const double *dx, double dt)
{
    OSG_CHECK(dim >= 2 && dim <= 3 && nx && gcl && gcu && e && state && dx && axis >= 0 &&
                  axis < dim && what >= 0 && what <= 2 && (what != 2 || b),
              OSG_ERR_ARG, "bad Lindman arguments");
    for (int d = 0; d < dim; d++)
        OSG_CHECK(nx[d] >= 1 && gcl[d] >= 1 && gcu[d] >= 2 && dx[d] > 0, OSG_ERR_ARG,
                  "the Lindman planes need gcl >= 1 and gcu >= 2");
    GridDesc g = make_grid(dim, nx, gcl, gcu);
    const long n = g.npoints() * 3, ns = lindman_state_size(g, axis);
    void *d_e, *d_b, *d_s;
    int rc;
    if ((rc = g_stage.get(4, sizeof(T) * n, &d_e))) return rc;
    if ((rc = g_stage.get(5, sizeof(T) * n, &d_b))) return rc;
    if ((rc = g_stage.get(6, sizeof(T) * ns, &d_s))) return rc;
    cudaStream_t st = g_stage.stream;
    OSG_CUDA(cudaMemcpyAsync(d_e, e, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    if (what == 2) OSG_CUDA(cudaMemcpyAsync(d_b, b, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(d_s, state, sizeof(T) * ns, cudaMemcpyHostToDevice, st));
    lindman_phase<T>(g, axis, what, (T *)d_e, (T *)d_b, (T *)d_s, dx, dt, st);
    OSG_CUDA(cudaGetLastError());
    if (what != 1) OSG_CUDA(cudaMemcpyAsync(e, d_e, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    if (what == 2) OSG_CUDA(cudaMemcpyAsync(b, d_b, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    if (what != 2)
        OSG_CUDA(cudaMemcpyAsync(state, d_s, sizeof(T) * ns, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaStreamSynchronize(st));
    return OSG_OK;
}

static int pml_check(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb)
{
    const int axes = mask & 7;
    OSG_CHECK(dim >= 2 && dim <= 3 && nx && gcl && gcu && axes > 0 && axes < (1 << dim) &&
                  nb >= 5 && (mask & ~63) == 0 && (dim == 2 || (mask >> 4) == 0),
              OSG_ERR_ARG, "bad PML arguments (2D/3D, a non-empty axis mask and its flags, "
                           "nb >= 5)");
    for (int d = 0; d < dim; d++)
        OSG_CHECK(nx[d] >= 6 && gcl[d] >= 1 && gcu[d] >= 2, OSG_ERR_ARG,
                  "PML walls need nx >= 6, gcl >= 1 and gcu >= 2 on every axis");
    return OSG_OK;
}

template <typename T>
static int pml_init_h(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                      const double *dx, double dt, T *state)
{
    int rc = pml_check(dim, nx, gcl, gcu, mask, nb);
    if (rc) return rc;
    OSG_CHECK(dx && state && dt > 0, OSG_ERR_ARG, "bad PML arguments");
    pml_init_host<T>(make_grid(dim, nx, gcl, gcu), mask, nb, dx, dt, state);
    return OSG_OK;
}

template <typename T>
static int pml_host(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                    int what, T *e, T *b, T *state, const double *dx, double dt)
{
    int rc = pml_check(dim, nx, gcl, gcu, mask, nb);
    if (rc) return rc;
    OSG_CHECK(state && what >= 0 && what <= 2 && (what == 0 || (e && b && dx)), OSG_ERR_ARG,
              "bad PML arguments");
    GridDesc g = make_grid(dim, nx, gcl, gcu);
    const long n = g.npoints() * 3, ns = pml_state_size(g, mask, nb);
    void *d_e = nullptr, *d_b = nullptr, *d_s;
    if (what > 0) {
        if ((rc = g_stage.get(4, sizeof(T) * n, &d_e))) return rc;
        if ((rc = g_stage.get(5, sizeof(T) * n, &d_b))) return rc;
    }
    if ((rc = g_stage.get(6, sizeof(T) * ns, &d_s))) return rc;
    cudaStream_t st = g_stage.stream;
    if (what > 0) {
        OSG_CUDA(cudaMemcpyAsync(d_e, e, sizeof(T) * n, cudaMemcpyHostToDevice, st));
        OSG_CUDA(cudaMemcpyAsync(d_b, b, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    }
    OSG_CUDA(cudaMemcpyAsync(d_s, state, sizeof(T) * ns, cudaMemcpyHostToDevice, st));
    pml_phase<T>(g, mask, nb, what, (T *)d_e, (T *)d_b, (T *)d_s, dx, dt, st);
    OSG_CUDA(cudaGetLastError());
    // what 1 writes the box's B next to the walls, what 2 its E
    if (what == 1) OSG_CUDA(cudaMemcpyAsync(b, d_b, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    if (what == 2) OSG_CUDA(cudaMemcpyAsync(e, d_e, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaMemcpyAsync(state, d_s, sizeof(T) * ns, cudaMemcpyDeviceToHost, st));
    OSG_CUDA(cudaStreamSynchronize(st));
    return OSG_OK;
}

template <typename T>
static int walls_host(int dim, const int *nx, const int *gcl, const int *gcu, T *f, int kind,
                      int walls, int order)
{
    OSG_CHECK(dim >= 1 && dim <= 3 && nx && gcl && gcu && f && kind >= 0 && kind <= 4 &&
                  walls >= 0 && walls < (1 << dim) && order >= 1 && order <= 4,
              OSG_ERR_ARG, "bad arguments");
    for (int d = 0; d < dim; d++)
        OSG_CHECK(gcl[d] >= 0 && gcu[d] >= 0 &&
                      (!((walls >> d) & 1) || (gcu[d] >= 1 && nx[d] >= gcl[d] + gcu[d] + 2)),
                  OSG_ERR_ARG, "a walled axis needs nx >= gcl + gcu + 2 and gcu >= 1");
    GridDesc g = make_grid(dim, nx, gcl, gcu);
    const long n = g.npoints() * 3;
    void *d_f;
    int rc;
    if ((rc = g_stage.get(6, sizeof(T) * n, &d_f))) return rc;
    cudaStream_t st = g_stage.stream;
    OSG_CUDA(cudaMemcpyAsync(d_f, f, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    wall_update<T>(g, (T *)d_f, kind, walls, order, st);
    OSG_CUDA(cudaGetLastError());
    OSG_CUDA(cudaMemcpyAsync(f, d_f, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
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

int osg_device_memory(size_t *free_bytes, size_t *total_bytes)
{
    OSG_CHECK(free_bytes && total_bytes, OSG_ERR_ARG, "null argument");
    OSG_CUDA(cudaMemGetInfo(free_bytes, total_bytes));
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

int osg_vadvance_deposit_cyl_f32(int order, int *ix, float *x, float *u, float *q, int i0,
                                 int i1, float rqm, int ilb2, const float *efield,
                                 const float *bfield, const int *emf_size,
                                 const int *emf_offset, float *j, const int *j_size,
                                 const int *j_offset, const double *dx, double dt, double *ene)
{
    OSG_CHECK(dx && dx[1] > 0, OSG_ERR_ARG, "dx[1] (the radial cell size) must be positive");
    return push_host<float>(2, order, ix, x, u, q, i0, i1, rqm, efield, bfield, emf_size,
                            emf_offset, j, j_size, j_offset, dx, dt, ene, OSG_PUSHER_BORIS,
                            1.0e-3, 1, ilb2);
}

int osg_vadvance_deposit_cyl_f64(int order, int *ix, double *x, double *u, double *q, int i0,
                                 int i1, double rqm, int ilb2, const double *efield,
                                 const double *bfield, const int *emf_size,
                                 const int *emf_offset, double *j, const int *j_size,
                                 const int *j_offset, const double *dx, double dt, double *ene)
{
    OSG_CHECK(dx && dx[1] > 0, OSG_ERR_ARG, "dx[1] (the radial cell size) must be positive");
    return push_host<double>(2, order, ix, x, u, q, i0, i1, rqm, efield, bfield, emf_size,
                             emf_offset, j, j_size, j_offset, dx, dt, ene, OSG_PUSHER_BORIS,
                             1.0e-3, 1, ilb2);
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

int osg_advance_deposit_exact_f32(int dim, int order, int *ix, float *x, float *u, float *q,
                                  int i0, int i1, float rqm, const float *efield,
                                  const float *bfield, const int *emf_size,
                                  const int *emf_offset, float *j, const int *j_size,
                                  const int *j_offset, const double *dx, double dt,
                                  double iter_tol, double *ene)
{
    return push_host<float>(dim, order, ix, x, u, q, i0, i1, rqm, efield, bfield, emf_size,
                            emf_offset, j, j_size, j_offset, dx, dt, ene, OSG_PUSHER_EXACT,
                            iter_tol);
}

int osg_advance_deposit_exact_f64(int dim, int order, int *ix, double *x, double *u, double *q,
                                  int i0, int i1, double rqm, const double *efield,
                                  const double *bfield, const int *emf_size,
                                  const int *emf_offset, double *j, const int *j_size,
                                  const int *j_offset, const double *dx, double dt,
                                  double iter_tol, double *ene)
{
    return push_host<double>(dim, order, ix, x, u, q, i0, i1, rqm, efield, bfield, emf_size,
                             emf_offset, j, j_size, j_offset, dx, dt, ene, OSG_PUSHER_EXACT,
                             iter_tol);
}

int osg_advance_deposit_f32(int dim, int order, int *ix, float *x, float *u, float *q, int i0,
                            int i1, float rqm, const float *efield, const float *bfield,
                            const int *emf_size, const int *emf_offset, float *j,
                            const int *j_size, const int *j_offset, const double *dx, double dt,
                            int pusher, double iter_tol, double *ene)
{
    return push_host<float>(dim, order, ix, x, u, q, i0, i1, rqm, efield, bfield, emf_size,
                            emf_offset, j, j_size, j_offset, dx, dt, ene, pusher, iter_tol);
}

int osg_advance_deposit_f64(int dim, int order, int *ix, double *x, double *u, double *q,
                            int i0, int i1, double rqm, const double *efield,
                            const double *bfield, const int *emf_size, const int *emf_offset,
                            double *j, const int *j_size, const int *j_offset, const double *dx,
                            double dt, int pusher, double iter_tol, double *ene)
{
    return push_host<double>(dim, order, ix, x, u, q, i0, i1, rqm, efield, bfield, emf_size,
                             emf_offset, j, j_size, j_offset, dx, dt, ene, pusher, iter_tol);
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

namespace {

// Host worker threads started once and reused by every call (a wrap of 16 M particles takes
// about a millisecond; starting threads per call would cost a sizeable part of it).  run(n, f)
// calls f(0..n-1) spread over the workers and the calling thread and returns when all are done.
class HostPool {
  public:
    static HostPool &get()
    {
        static HostPool pool;
        return pool;
    }
    int size() const { return (int)workers_.size() + 1; }
    void run(int n, const std::function<void(int)> &f)
    {
        std::lock_guard<std::mutex> one(call_);   // callers from several threads take turns
        std::unique_lock<std::mutex> lk(m_);
        job_ = &f;
        njobs_ = n;
        next_ = 0;
        done_ = 0;
        gen_++;
        cv_.notify_all();
        lk.unlock();
        work();
        lk.lock();
        fin_.wait(lk, [&] { return done_ == njobs_; });
        job_ = nullptr;
    }

  private:
    HostPool()
    {
        unsigned nt = std::thread::hardware_concurrency();
        if (nt == 0) nt = 1;
        if (nt > 32) nt = 32;
        for (unsigned t = 1; t < nt; t++) workers_.emplace_back([this] { loop(); });
    }
    ~HostPool()
    {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
            cv_.notify_all();
        }
        for (auto &w : workers_) w.join();
    }
    void work()
    {
        for (;;) {
            int i;
            const std::function<void(int)> *f;
            {
                std::lock_guard<std::mutex> lk(m_);
                if (!job_ || next_ >= njobs_) return;
                i = next_++;
                f = job_;
            }
            (*f)(i);
            std::lock_guard<std::mutex> lk(m_);
            if (++done_ == njobs_) fin_.notify_all();
        }
    }
    void loop()
    {
        long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
            }
            work();
        }
    }
    std::vector<std::thread> workers_;
    std::mutex call_, m_;
    std::condition_variable cv_, fin_;
    const std::function<void(int)> *job_ = nullptr;
    int njobs_ = 0, next_ = 0, done_ = 0;
    long gen_ = 0;
    bool stop_ = false;
};

} // namespace

int osg_particle_wrap(int dim, const int *nx, long np, int *ix)
{
    OSG_CHECK(dim >= 1 && dim <= 3 && nx && (np == 0 || ix), OSG_ERR_ARG, "bad arguments");
    // branch-free per axis so the loop vectorises; large arrays are split over host threads.
    // Only a few particles cross the box per step: a block of indices is first scanned
    // (read only) and rewritten only when one of them is out of range, so the unchanged
    // blocks cost a read and no write-back.
    const int n0 = nx[0], n1 = dim > 1 ? nx[1] : 1, n2 = dim > 2 ? nx[2] : 1;
    auto fix_range = [=](long p0, long p1) {
        int *c = ix + (long)dim * p0;
        const long m = (long)dim * (p1 - p0);
        if (dim == 1) {
            for (long k = 0; k < m; k++) c[k] += (c[k] < 1 ? n0 : 0) - (c[k] > n0 ? n0 : 0);
        } else if (dim == 2) {
            for (long k = 0; k < m; k += 2) {
                c[k] += (c[k] < 1 ? n0 : 0) - (c[k] > n0 ? n0 : 0);
                c[k + 1] += (c[k + 1] < 1 ? n1 : 0) - (c[k + 1] > n1 ? n1 : 0);
            }
        } else {
            for (long k = 0; k < m; k += 3) {
                c[k] += (c[k] < 1 ? n0 : 0) - (c[k] > n0 ? n0 : 0);
                c[k + 1] += (c[k + 1] < 1 ? n1 : 0) - (c[k + 1] > n1 ? n1 : 0);
                c[k + 2] += (c[k + 2] < 1 ? n2 : 0) - (c[k + 2] > n2 ? n2 : 0);
            }
        }
    };
    auto wrap_range = [=](long p0, long p1) {
        const long blk = 1024;   // particles per scanned block
        for (long b0 = p0; b0 < p1; b0 += blk) {
            const long b1 = std::min(p1, b0 + blk);
            const int *c = ix + (long)dim * b0;
            const long m = (long)dim * (b1 - b0);
            int out = 0;
            if (dim == 1) {
                for (long k = 0; k < m; k++) out |= (c[k] < 1) | (c[k] > n0);
            } else if (dim == 2) {
                for (long k = 0; k < m; k += 2)
                    out |= (c[k] < 1) | (c[k] > n0) | (c[k + 1] < 1) | (c[k + 1] > n1);
            } else {
                for (long k = 0; k < m; k += 3)
                    out |= (c[k] < 1) | (c[k] > n0) | (c[k + 1] < 1) | (c[k + 1] > n1) |
                           (c[k + 2] < 1) | (c[k + 2] > n2);
            }
            if (out) fix_range(b0, b1);
        }
    };
    if (np < (1L << 20)) {
        wrap_range(0, np);
        return OSG_OK;
    }
    HostPool &pool = HostPool::get();
    const int nparts = 4 * pool.size();
    const long chunk = (np + nparts - 1) / nparts;
    pool.run(nparts, [&](int t) {
        const long p0 = (long)t * chunk, p1 = std::min(np, p0 + chunk);
        if (p0 < p1) wrap_range(p0, p1);
    });
    return OSG_OK;
}

int osg_smooth_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *f,
                   const int *type, const int *order)
{
    return smooth_host<float>(dim, nx, gcl, gcu, f, type, order);
}

int osg_smooth_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *f,
                   const int *type, const int *order)
{
    return smooth_host<double>(dim, nx, gcl, gcu, f, type, order);
}

int osg_smooth_coefficients(int type, int order, double *c, int *n)
{
    OSG_CHECK(c && n, OSG_ERR_ARG, "null argument");
    OSG_CHECK(smooth_coefficients(type, order, c, n) == OSG_OK, OSG_ERR_ARG,
              "bad smoothing type %d / order %d", type, order);
    return OSG_OK;
}

long osg_pml_state_size(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb)
{
    if (pml_check(dim, nx, gcl, gcu, mask, nb)) return -1;
    return pml_state_size(make_grid(dim, nx, gcl, gcu), mask, nb);
}

int osg_pml_init_f32(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                     const double *dx, double dt, float *state)
{
    return pml_init_h<float>(dim, nx, gcl, gcu, mask, nb, dx, dt, state);
}

int osg_pml_init_f64(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb,
                     const double *dx, double dt, double *state)
{
    return pml_init_h<double>(dim, nx, gcl, gcu, mask, nb, dx, dt, state);
}

int osg_pml_f32(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb, int what,
                float *e, float *b, float *state, const double *dx, double dt)
{
    return pml_host<float>(dim, nx, gcl, gcu, mask, nb, what, e, b, state, dx, dt);
}

int osg_pml_f64(int dim, const int *nx, const int *gcl, const int *gcu, int mask, int nb, int what,
                double *e, double *b, double *state, const double *dx, double dt)
{
    return pml_host<double>(dim, nx, gcl, gcu, mask, nb, what, e, b, state, dx, dt);
}

int osg_lindman_f32(int dim, const int *nx, const int *gcl, const int *gcu, int axis, int what,
                    float *e, float *b, float *state, const double *dx, double dt)
{
    return lindman_host<float>(dim, nx, gcl, gcu, axis, what, e, b, state, dx, dt);
}

int osg_lindman_f64(int dim, const int *nx, const int *gcl, const int *gcu, int axis, int what,
                    double *e, double *b, double *state, const double *dx, double dt)
{
    return lindman_host<double>(dim, nx, gcl, gcu, axis, what, e, b, state, dx, dt);
}

int osg_walls_f32(int dim, const int *nx, const int *gcl, const int *gcu, float *f, int kind,
                  int walls, int order)
{
    return walls_host<float>(dim, nx, gcl, gcu, f, kind, walls, order);
}

int osg_walls_f64(int dim, const int *nx, const int *gcl, const int *gcu, double *f, int kind,
                  int walls, int order)
{
    return walls_host<double>(dim, nx, gcl, gcu, f, kind, walls, order);
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
