// sim.cu -- device-resident simulation handle (osg_sim_*): particles, fields and current stay
// in HBM; one call advances N time steps, each step replayed from a captured CUDA graph.
//
// Phase order of one step, as iter_sim (source/os-simulation.f03:498-666) on one periodic node:
//   1. E, B guard replace          emf%update_boundary (:561) -> update_periodic_vdf replace
//   2. J = 0; push + deposit       part%advance_deposit (:588), all species
//   3. periodic particle wrap      part%update_boundary (:593) -- fused into the push
//   4. cell sort every n_sort      sort_collide (:638) (plain engine) / tile migration, every
//                                  step, fused into the push (tiled engine)
//   5. J guard fold                jay%update_boundary (:652)
//   6. Yee B/2, E, B/2             emf%advance (:661)
#include <cuda_runtime.h>

#include <algorithm>
#include <array>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "fields.cuh"
#include "pic_math.cuh"
#include "push_plain.cuh"
#include "tiled.cuh"

namespace osg {

struct PlainSpecies {
    int *ix = nullptr;
    void *x = nullptr, *u = nullptr, *q = nullptr;
};

} // namespace osg

struct osg_sim {
    osg_config cfg;
    osg::GridDesc g;
    int gl = 0, gu = 0;
    int esz = 4;                 // bytes per real
    cudaStream_t st = nullptr;
    void *e = nullptr, *b = nullptr, *j = nullptr;
    double *d_ene = nullptr;     // [OSG_MAX_SPECIES] kinetic accumulators of the last step
    int *d_status = nullptr;
    double *d_diag = nullptr;    // 16 doubles of diagnostic scratch
    double *d_rho = nullptr, *d_rho0 = nullptr;
    long step_n = 0;
    int cur = 0;                 // tiled engine: particle buffer holding the current state
    std::vector<double> rqm;
    std::vector<long> np;
    std::vector<osg::PlainSpecies> plain;
    // plain-engine sort scratch
    int *d_cell_cnt = nullptr;
    int *d_scan_tmp = nullptr;
    void *d_sort_buf = nullptr;
    size_t sort_buf_bytes = 0;
    // tiled engine
    osg::TiledState *tiled = nullptr;
    // moving window along x1 (tiled engine)
    bool window = false;
    double xmoved = 0.0;         // window motion not yet turned into a cell move
    long moves = 0;              // cell moves so far
    void *shift_tmp = nullptr;   // scratch field array for the shift and the smoothing
    unsigned long long *d_step = nullptr;   // step counter of the thermal-bath random stream
    int open_axis = -1;          // Lindman open boundaries at both edges of this axis
    void *lind = nullptr;        // their state (lindman_state_size reals)
    int pml_mask = 0;            // PML walls at both edges of these axes
    int pml_flags = 0;           // bits 4, 5: the x1 / x2 walls' diffusion correction (2D)
    int pml_nb = 0;              // their thickness in cells
    void *pml = nullptr;         // their state (pml_state_size reals)
    void *pml_tmp = nullptr;     // scratch of the walls' shift with the moving window
    osg::SmoothSpec smooth;      // current smoothing (order 0 per axis: none)
    osg::SmoothSpec esmooth;     // smoothing of the fields the particles see (order 0: none)
    void *e_part = nullptr, *b_part = nullptr;   // those fields, when smoothed
    // graphs: [parity][sort (plain) / window move (tiled)]
    cudaGraphExec_t gexec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    bool graphs_dirty = true;
    int launches_per_step = 0;
};

namespace osg {

static const int MAX_SPECIES = 16;

// ------------------------------------------------------------------------ cell sort (plain)

template <int DIM>
__global__ void k_cell_count(const int *__restrict__ ix, long np, GridDesc g, int *cnt)
{
    OSG_GRID_LOOP(p, np)
    {
        long key = ix[DIM * p] - 1;
        if (DIM > 1) key += (long)g.nx[0] * (ix[DIM * p + 1] - 1);
        if (DIM > 2) key += (long)g.nx[0] * g.nx[1] * (ix[DIM * p + 2] - 1);
        atomicAdd(cnt + key, 1);
    }
}

// exclusive scan of n ints in place, three kernels: per-block scan, scan of block sums,
// add back
__global__ void k_scan_block(int *a, long n, int *block_sums)
{
    __shared__ int ws[32];
    const long i = (long)blockIdx.x * 1024 + threadIdx.x;
    int v = i < n ? a[i] : 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        ws[lane] = s;
    }
    __syncthreads();
    const int incl = x + (w > 0 ? ws[w - 1] : 0);
    if (i < n) a[i] = incl - v;
    if (threadIdx.x == 1023) block_sums[blockIdx.x] = incl;
}

__global__ void k_scan_sums(int *s, int nb)
{
    // single block of 1024 threads, sequential over chunks
    __shared__ int ws[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? s[i] : 0;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) ws[w] = x;
        __syncthreads();
        if (w == 0) {
            int t = ws[lane];
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            ws[lane] = t;
        }
        __syncthreads();
        const int incl = x + (w > 0 ? ws[w - 1] : 0);
        const int c = carry;
        if (i < nb) s[i] = c + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c + incl;
        __syncthreads();
    }
}

__global__ void k_scan_add(int *a, long n, const int *block_sums)
{
    const long i = (long)blockIdx.x * 1024 + threadIdx.x;
    if (i < n && blockIdx.x > 0) a[i] += block_sums[blockIdx.x];
}

void exclusive_scan(int *a, long n, int *tmp, cudaStream_t st)
{
    const int nb = (int)((n + 1023) / 1024);
    k_scan_block<<<nb, 1024, 0, st>>>(a, n, tmp);
    k_scan_sums<<<1, 1024, 0, st>>>(tmp, nb);
    k_scan_add<<<nb, 1024, 0, st>>>(a, n, tmp);
}

template <typename T, int DIM>
__global__ void k_cell_scatter(const int *__restrict__ ix, const T *__restrict__ x,
                               const T *__restrict__ u, const T *__restrict__ q, long np,
                               GridDesc g, int *next, int *ix2, T *x2, T *u2, T *q2)
{
    OSG_GRID_LOOP(p, np)
    {
        long key = ix[DIM * p] - 1;
        if (DIM > 1) key += (long)g.nx[0] * (ix[DIM * p + 1] - 1);
        if (DIM > 2) key += (long)g.nx[0] * g.nx[1] * (ix[DIM * p + 2] - 1);
        const long s = atomicAdd(next + key, 1);
        for (int d = 0; d < DIM; d++) {
            ix2[DIM * s + d] = ix[DIM * p + d];
            x2[DIM * s + d] = x[DIM * p + d];
        }
        u2[3 * s] = u[3 * p];
        u2[3 * s + 1] = u[3 * p + 1];
        u2[3 * s + 2] = u[3 * p + 2];
        q2[s] = q[p];
    }
}

long ncells(const GridDesc &g) { return (long)g.nx[0] * g.nx[1] * g.nx[2]; }

template <typename T>
static int sort_species(osg_sim *s, int k, cudaStream_t st)
{
    const long np = s->np[k];
    if (np <= 0) return OSG_OK;
    const int dim = s->cfg.dim;
    PlainSpecies &p = s->plain[k];
    const long nc = ncells(s->g);
    char *buf = (char *)s->d_sort_buf;
    int *ix2 = (int *)buf;
    T *x2 = (T *)(buf + sizeof(int) * dim * np);
    T *u2 = x2 + dim * np;
    T *q2 = u2 + 3 * np;
    OSG_CUDA(cudaMemsetAsync(s->d_cell_cnt, 0, sizeof(int) * nc, st));
    unsigned nb = blocks_for(np, 256);
    if (nb > 8192) nb = 8192;
    if (dim == 2) k_cell_count<2><<<nb, 256, 0, st>>>(p.ix, np, s->g, s->d_cell_cnt);
    else k_cell_count<3><<<nb, 256, 0, st>>>(p.ix, np, s->g, s->d_cell_cnt);
    exclusive_scan(s->d_cell_cnt, nc, s->d_scan_tmp, st);
    if (dim == 2)
        k_cell_scatter<T, 2><<<nb, 256, 0, st>>>(p.ix, (T *)p.x, (T *)p.u, (T *)p.q, np, s->g,
                                                 s->d_cell_cnt, ix2, x2, u2, q2);
    else
        k_cell_scatter<T, 3><<<nb, 256, 0, st>>>(p.ix, (T *)p.x, (T *)p.u, (T *)p.q, np, s->g,
                                                 s->d_cell_cnt, ix2, x2, u2, q2);
    OSG_CUDA(cudaMemcpyAsync(p.ix, ix2, sizeof(int) * dim * np, cudaMemcpyDeviceToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(p.x, x2, sizeof(T) * dim * np, cudaMemcpyDeviceToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(p.u, u2, sizeof(T) * 3 * np, cudaMemcpyDeviceToDevice, st));
    OSG_CUDA(cudaMemcpyAsync(p.q, q2, sizeof(T) * np, cudaMemcpyDeviceToDevice, st));
    return OSG_OK;
}

// ------------------------------------------------------------------------ one step

struct PhaseEvents {
    cudaEvent_t ev[8];
};

// the thermal-bath random stream's step counter, advanced at the end of every step
__global__ void k_step_tick(unsigned long long *step) { *step += 1; }

// with_sort: plain engine, cell sort after the push; shift: tiled engine with a moving
// window, the step ends with a one-cell window move (move_boundary_space_global,
// source/os-space.f90:508-566: in the reference the move opens the next step, whose push then
// sees the moved window; here the push of this step already stores the moved cell indices)
template <typename T>
static int enqueue_step(osg_sim *s, int parity, bool with_sort, bool shift, PhaseEvents *pe)
{
    cudaStream_t st = s->st;
    const osg_config &c = s->cfg;
    const int ns = (int)s->np.size();
    int emf_size[3], emf_off[3];
    for (int d = 0; d < 3; d++) {
        emf_size[d] = s->g.size[d];
        emf_off[d] = s->g.gcl[d];
    }
    int launches = 0;
    // the single-precision reference pushes with dt rounded to p_k_part
    // (dtcycle = real(dt, p_k_part), source/spec/os-spec-vpush.f03:365)
    // (the Fortran push the exact pusher runs in keeps the double dt,
    //  source/spec/os-spec-push.f03:1459-1460)
    const bool fortran_push = c.pusher != OSG_PUSHER_BORIS;
    const double push_dt = (sizeof(T) == 4 && !fortran_push) ? (double)(float)c.dt : c.dt;
    // moving window: the reference's x1 boundary (p_bc_move_c) updates no guard cells of E,
    // B or J (update_boundary_emf_bound, source/emf/boundary/os-emf-boundary.f90:779-820, has
    // no neighbour along x1; the current's boundary type is p_bc_none, source/current/
    // os-current-define.f03:240-251): the guards keep what the window shift and the Yee
    // update leave there
    const int win = s->window ? 1 : 0;
    // conducting walls: their guard cells hold the images set by the last field advance
    const int walls = c.walls;
    // Lindman open boundaries: no periodic update along their axis, the boundary planes come
    // from their state, the current beyond them is neither folded nor imaged
    const int oax = s->open_axis;
    // PML walls: the same, with the boundary points set by the walls' interfaces in the Yee
    // advance (no restore at the guard update)
    const int pml = s->pml_mask;
    const int skip = walls | (oax >= 0 ? 1 << oax : 0) | pml;
    if (pe) OSG_CUDA(cudaEventRecord(pe->ev[0], st));
    if (oax >= 0) {
        open_guards<T>(s->g, (T *)s->e, (T *)s->b, oax, (const T *)s->lind, st);
        launches += 2 * (c.dim - 1) + 1;
    } else if (pml) {
        // (bit 3: x1 is the moving window's axis, updated by neither the walls nor the box)
        pml_guards<T>(s->g, (T *)s->e, (T *)s->b, pml | (win ? 8 : 0), s->pml_nb, (T *)s->pml,
                      st);
        // one wall guard launch per PML axis and periodic other axis
        const int np_ = __builtin_popcount(pml);
        launches += 2 * (c.dim - np_) + np_ * (c.dim - np_);
    } else {
        periodic_update<T>(s->g, (T *)s->e, 0, st, 0, walls | win);
        periodic_update<T>(s->g, (T *)s->b, 0, st, 0, walls | win);
        launches += 2 * (c.dim - __builtin_popcount(walls | win));
    }
    // the fields the particles see (update_particle_fld_emf, source/emf/os-emf.f03:1065-1151):
    // E and B, or their smoothed copies (smooth_type "stand")
    const void *ep = s->e, *bp = s->b;
    if (s->esmooth.order[0] > 0) {
        const size_t gbytes = (size_t)s->esz * 3 * s->g.npoints();
        OSG_CUDA(cudaMemcpyAsync(s->e_part, s->e, gbytes, cudaMemcpyDeviceToDevice, st));
        OSG_CUDA(cudaMemcpyAsync(s->b_part, s->b, gbytes, cudaMemcpyDeviceToDevice, st));
        smooth_field<T>(s->g, s->esmooth, (T *)s->e_part, (T *)s->shift_tmp, st);
        smooth_field<T>(s->g, s->esmooth, (T *)s->b_part, (T *)s->shift_tmp, st);
        launches += 2 * c.dim;
        ep = s->e_part;
        bp = s->b_part;
    }
    if (pe) OSG_CUDA(cudaEventRecord(pe->ev[1], st));
    OSG_CUDA(cudaMemsetAsync(s->j, 0, (size_t)s->esz * 3 * s->g.npoints(), st));
    OSG_CUDA(cudaMemsetAsync(s->d_ene, 0, sizeof(double) * MAX_SPECIES, st));
    if (c.engine == OSG_ENGINE_TILED) {
        int rc = tiled_push(s->tiled, parity, (const float *)ep, (const float *)bp,
                            (float *)s->j, s->d_ene, s->d_status, st, &launches, shift ? 1 : 0);
        if (rc) return rc;
    } else {
        for (int k = 0; k < ns; k++) {
            if (s->np[k] <= 0) continue;
            PlainSpecies &p = s->plain[k];
            PlainPushArgs<T> a = make_plain_args<T>(
                c.dim, c.order, p.ix, (T *)p.x, (T *)p.u, (const T *)p.q, s->np[k],
                (T)s->rqm[k], (const T *)ep, (const T *)bp, emf_size, emf_off, (T *)s->j,
                emf_size, emf_off, c.dx, push_dt, s->d_ene + k, s->d_status);
            for (int d = 0; d < c.dim; d++) {
                a.wrap[d] = (skip >> d) & 1 ? 0 : c.nx[d];
                a.reflect[d] = (walls >> d) & 1 ? c.nx[d] : 0;
                a.absorb[d] = (d == oax || ((pml >> d) & 1)) ? c.nx[d] : 0;
            }
            a.q_absorb = (T *)p.q;
            if (c.thermal) {
                for (int d = 0; d < c.dim; d++) {
                    a.thermal[d] = (c.thermal >> d) & 1 ? c.nx[d] : 0;
                    if (a.thermal[d]) a.absorb[d] = a.reflect[d] = 0;
                }
                for (int d = 0; d < 3; d++) {
                    a.uth_bnd[d] = (T)c.uth_bnd[d];
                    a.ufl_bnd[d] = (T)c.ufl_bnd[d];
                }
                a.step = s->d_step;
                a.thermal_type = c.thermal_type;
                a.rng_key[0] = c.seed;
                a.rng_key[1] = (unsigned int)k;
            }
            a.pusher = c.pusher;
            a.iter_tol = c.iter_tol;
            if (c.pusher >= OSG_PUSHER_VAY)
                a.tem = (T)pusher_tem(c.pusher, push_dt, (double)(T)s->rqm[k]);
            int rc = launch_plain_push<T>(c.dim, c.order, a, st);
            if (rc) return rc;
            launches++;
        }
    }
    if (pe) OSG_CUDA(cudaEventRecord(pe->ev[2], st));
    if (with_sort && c.engine == OSG_ENGINE_PLAIN) {
        for (int k = 0; k < ns; k++) {
            int rc = sort_species<T>(s, k, st);
            if (rc) return rc;
            launches += 5;
        }
    }
    if (pe) OSG_CUDA(cudaEventRecord(pe->ev[3], st));
    periodic_update<T>(s->g, (T *)s->j, 1, st, 0, skip | win);
    launches += c.dim - __builtin_popcount(skip | win);
    if (walls) {
        // current deposited beyond a wall comes back as its image (update_boundary_current,
        // source/current/os-current-define.f03:683-725)
        wall_update<T>(s->g, (T *)s->j, 2, walls, c.order, st);
        launches += 2 * __builtin_popcount(walls);
    }
    if (s->smooth.order[0] > 0) {
        // smooth currents after the boundary update (source/os-simulation.f03:651-657)
        smooth_field<T>(s->g, s->smooth, (T *)s->j, (T *)s->shift_tmp, st);
        launches += c.dim;
    }
    if (pe) OSG_CUDA(cudaEventRecord(pe->ev[4], st));
    yee_advance<T>(s->g, (T *)s->e, (T *)s->b, (const T *)s->j, c.dx, c.dt, st, walls, c.order,
                   oax, (T *)s->lind, c.pmc, pml | s->pml_flags, s->pml_nb, (T *)s->pml);
    launches += 3 + (walls ? 6 * __builtin_popcount(walls) : 0) + (oax >= 0 ? 3 : 0) +
                (!pml ? 0
                      : __builtin_popcount(s->pml_flags) + 2 * (2 * __builtin_popcount(pml) +
                             (c.dim == 2 ? (pml == 3) : ((pml & 1) && (pml & 2)) +
                                                            ((pml & 1) && (pml & 4)) +
                                                            ((pml & 2) && (pml & 4)))));
    if (shift) {
        shift_window_x<T>(s->g, (T *)s->e, (T *)s->shift_tmp, st);
        shift_window_x<T>(s->g, (T *)s->b, (T *)s->shift_tmp, st);
        launches += 2;
        if (s->pml) {
            // the PML walls of the other axes move with the fields (move_window_vpml)
            pml_shift_x<T>(s->g, pml, s->pml_nb, (T *)s->pml, (T *)s->pml_tmp, st);
            launches += 4 * __builtin_popcount(pml & 6);
        }
        int rc = tiled_window_inject(s->tiled, parity, s->d_status, st, &launches);
        if (rc) return rc;
    }
    if (s->d_step) {
        k_step_tick<<<1, 1, 0, st>>>(s->d_step);
        launches++;
    }
    if (pe) OSG_CUDA(cudaEventRecord(pe->ev[5], st));
    OSG_CUDA(cudaGetLastError());
    s->launches_per_step = launches;
    return OSG_OK;
}

static int enqueue_step_any(osg_sim *s, int parity, bool with_sort, bool shift,
                            PhaseEvents *pe)
{
    return s->cfg.precision == 32 ? enqueue_step<float>(s, parity, with_sort, shift, pe)
                                  : enqueue_step<double>(s, parity, with_sort, shift, pe);
}

static void drop_graphs(osg_sim *s)
{
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++)
            if (s->gexec[a][b]) {
                cudaGraphExecDestroy(s->gexec[a][b]);
                s->gexec[a][b] = nullptr;
            }
    s->graphs_dirty = false;
}

// variant: the plain engine's cell sort or the tiled engine's window move
static int get_graph(osg_sim *s, int parity, int sort, cudaGraphExec_t *out)
{
    if (s->graphs_dirty) drop_graphs(s);
    if (!s->gexec[parity][sort]) {
        cudaGraph_t gr;
        OSG_CUDA(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
        const bool tiled = s->cfg.engine == OSG_ENGINE_TILED;
        int rc = enqueue_step_any(s, parity, !tiled && sort != 0, tiled && sort != 0, nullptr);
        cudaError_t ce = cudaStreamEndCapture(s->st, &gr);
        if (rc) {
            if (ce == cudaSuccess) cudaGraphDestroy(gr);
            return rc;
        }
        OSG_CUDA(ce);
        cudaError_t ie = cudaGraphInstantiate(&s->gexec[parity][sort], gr, 0);
        cudaGraphDestroy(gr);
        OSG_CUDA(ie);
    }
    *out = s->gexec[parity][sort];
    return OSG_OK;
}

// osg_sim_step checks the tiled engine's slab occupancy after every this many steps
static const int OCC_CHECK_STEPS = 8;

static bool sort_due(const osg_sim *s, long n)
{
    return s->cfg.engine == OSG_ENGINE_PLAIN && s->cfg.n_sort > 0 && n > 0 &&
           (n % s->cfg.n_sort) == 0;
}

// buffer bookkeeping of the tiled engine after one step (the push writes the other buffer)
static void advance_buffers(osg_sim *s)
{
    if (s->cfg.engine == OSG_ENGINE_TILED) s->cur ^= 1;
}

// Moving window: does the step about to run end with a cell move?  The reference adds dt to
// the window motion at the start of every step and moves one cell once it reaches dx
// (source/os-space.f90:529-550); xmoved here already holds the motion after the current
// step's start, so the move that opens the next step is decided now.
static bool window_move_next(osg_sim *s, bool commit)
{
    if (!s->window) return false;
    const double xm = s->xmoved + s->cfg.dt;
    const bool mv = xm >= s->cfg.dx[0];
    if (commit) {
        s->xmoved = mv ? xm - s->cfg.dx[0] : xm;
        if (mv) s->moves++;
    }
    return mv;
}

static int check_status(osg_sim *s)
{
    int h = 0;
    OSG_CUDA(cudaMemcpyAsync(&h, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    OSG_CUDA(cudaStreamSynchronize(s->st));
    if (h & OSG_STATUS_OVERFLOW) {
        set_error("a tile ran out of particle slots (raise osg_config.capacity)");
        return OSG_ERR_OVERFLOW;
    }
    if (h & OSG_STATUS_RANGE) {
        set_error("a particle cell index left the grid");
        return OSG_ERR_RANGE;
    }
    return OSG_OK;
}

template <typename T> static T *dalloc(size_t n, int *rc)
{
    void *p = nullptr;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
        set_error("cudaMalloc of %zu bytes failed", n * sizeof(T));
        *rc = OSG_ERR_NOMEM;
        return nullptr;
    }
    return (T *)p;
}

} // namespace osg

using namespace osg;

extern "C" {

int osg_sim_create(const osg_config *cfg, osg_sim **out)
{
    OSG_CHECK(cfg && out, OSG_ERR_ARG, "null argument");
    *out = nullptr;
    OSG_CHECK(cfg->dim == 2 || cfg->dim == 3, OSG_ERR_ARG, "dim must be 2 or 3");
    OSG_CHECK(cfg->order >= 1 && cfg->order <= 4, OSG_ERR_ARG, "order must be 1..4");
    OSG_CHECK(cfg->precision == 32 || cfg->precision == 64, OSG_ERR_ARG,
              "precision must be 32 or 64");
    OSG_CHECK(cfg->engine == OSG_ENGINE_PLAIN || cfg->engine == OSG_ENGINE_TILED, OSG_ERR_ARG,
              "unknown engine");
    OSG_CHECK(!(cfg->engine == OSG_ENGINE_TILED && cfg->precision != 32), OSG_ERR_ARG,
              "the tiled engine is single precision");
    OSG_CHECK(cfg->walls >= 0 && cfg->walls < (1 << cfg->dim), OSG_ERR_ARG,
              "walls: a bit mask of the axes");
    OSG_CHECK((cfg->walls == 0 && cfg->open_fields == 0) ||
                  cfg->emf_smooth_type == OSG_SMOOTH_NONE,
              OSG_ERR_ARG, "smoothing of the particles' fields runs on periodic boxes");
    OSG_CHECK(cfg->walls == 0 || cfg->smooth_type == OSG_SMOOTH_NONE, OSG_ERR_ARG,
              "current smoothing next to conducting walls is not supported");
    OSG_CHECK(cfg->open_fields >= 0 && cfg->open_fields < (1 << cfg->dim) &&
                  (cfg->open_fields & (cfg->open_fields - 1)) == 0,
              OSG_ERR_ARG, "open_fields: the bit of one axis (Lindman boundaries are admitted "
                           "along one axis)");
    OSG_CHECK(cfg->open_fields == 0 || (cfg->walls == 0 && cfg->smooth_type == OSG_SMOOTH_NONE),
              OSG_ERR_ARG, "open boundaries combine with neither walls nor smoothing");
    OSG_CHECK(cfg->pmc >= 0 && (cfg->pmc & ~cfg->walls) == 0, OSG_ERR_ARG,
              "pmc: a bit mask of walled axes");
    OSG_CHECK(cfg->pml >= 0 && cfg->pml < (1 << cfg->dim), OSG_ERR_ARG,
              "pml: a bit mask of the axes");
    OSG_CHECK(cfg->pml == 0 || cfg->dim >= 2, OSG_ERR_ARG, "PML walls: 2D and 3D boxes");
    OSG_CHECK(cfg->pml == 0 || (cfg->walls == 0 && cfg->open_fields == 0 &&
                                cfg->smooth_type == OSG_SMOOTH_NONE &&
                                cfg->emf_smooth_type == OSG_SMOOTH_NONE && cfg->thermal == 0),
              OSG_ERR_ARG, "PML walls combine with neither walls, Lindman boundaries, "
                           "smoothing nor a thermal bath");
    OSG_CHECK(cfg->pml_cells == 0 || cfg->pml_cells >= 5, OSG_ERR_ARG,
              "pml_cells: 0 (8) or at least 5");
    OSG_CHECK(cfg->pml_diffuse >= 0 && (cfg->pml_diffuse & ~cfg->pml) == 0 &&
                  (cfg->pml_diffuse == 0 || cfg->dim == 2),
              OSG_ERR_ARG, "pml_diffuse: a bit mask of PML axes of a 2D box");
    if (cfg->pml)
        for (int d = 0; d < cfg->dim; d++)
            OSG_CHECK(cfg->nx[d] >= 6, OSG_ERR_ARG, "PML walls need at least 6 cells per axis");
    OSG_CHECK(cfg->thermal >= 0 && (cfg->thermal & ~(cfg->walls | cfg->open_fields)) == 0,
              OSG_ERR_ARG, "thermal: a bit mask of walled or open axes");
    OSG_CHECK(cfg->thermal == 0 || cfg->engine == OSG_ENGINE_PLAIN ||
                  cfg->pusher == OSG_PUSHER_BORIS,
              OSG_ERR_ARG, "tiled engine: the thermal bath runs with the Boris pusher");
    OSG_CHECK(cfg->thermal_type >= 0 && cfg->thermal_type <= 2, OSG_ERR_ARG,
              "thermal_type: 0 thermal, 1 random dir, 2 waterbag");
    if (cfg->thermal)
        for (int d = 0; d < cfg->dim; d++)
            OSG_CHECK(!((cfg->thermal >> d) & 1) || cfg->uth_bnd[d] > 0, OSG_ERR_ARG,
                      "a thermal bath along axis %d needs uth_bnd[%d] > 0 (the reference's check)",
                      d, d);
    OSG_CHECK(cfg->pusher >= OSG_PUSHER_BORIS && cfg->pusher <= OSG_PUSHER_COND_VAY, OSG_ERR_ARG,
              "unknown pusher");
    OSG_CHECK(cfg->iter_tol >= 0, OSG_ERR_ARG, "iter_tol must be >= 0");
    double cour = 0.0;
    for (int d = 0; d < cfg->dim; d++) {
        OSG_CHECK(cfg->nx[d] >= 2 * cfg->order + 1 && cfg->dx[d] > 0, OSG_ERR_ARG,
                  "nx[%d] too small or dx <= 0", d);
        cour += 1.0 / (cfg->dx[d] * cfg->dx[d]);
    }
    // Courant condition of the Yee solver (source/emf/solver/os-emf-solver-yee.f03:430-456)
    OSG_CHECK(cfg->dt > 0 && cfg->dt <= std::sqrt(1.0 / cour), OSG_ERR_ARG,
              "dt violates the Yee Courant limit %g", std::sqrt(1.0 / cour));
    osg_sim *s = new osg_sim();
    s->cfg = *cfg;
    if (s->cfg.iter_tol <= 0) s->cfg.iter_tol = 1.0e-3;
    for (int d = cfg->dim; d < 3; d++) {
        s->cfg.nx[d] = 1;
        s->cfg.dx[d] = 1.0;
    }
    guard_cells(cfg->order, &s->gl, &s->gu);
    {
        int n = 0;
        memset(&s->smooth, 0, sizeof s->smooth);
        if (smooth_coefficients(cfg->smooth_type, cfg->smooth_order, s->smooth.c[0], &n)) {
            set_error("bad smoothing type %d / order %d", cfg->smooth_type, cfg->smooth_order);
            delete s;
            return OSG_ERR_ARG;
        }
        for (int d = 0; d < cfg->dim; d++) {
            s->smooth.order[d] = n;
            for (int k = 0; k < 2 * n + 1; k++) s->smooth.c[d][k] = s->smooth.c[0][k];
        }
        // the filter needs n lower and n + 1 upper guard cells (the first upper guard cell of
        // the current is used by the E advance), source/current/os-current-define.f03:198-206
        s->gl = std::max(s->gl, n);
        s->gu = std::max(s->gu, n + 1);
        // the particles' fields: the reference adds the filter's order to the field's guard
        // cells on both sides (source/emf/os-emf.f03:690-703), so that every point a particle
        // gathers from is filtered
        int ne = 0, gli = 0, gui = 0;
        memset(&s->esmooth, 0, sizeof s->esmooth);
        if (smooth_coefficients(cfg->emf_smooth_type, cfg->emf_smooth_order, s->esmooth.c[0],
                                &ne)) {
            set_error("bad field smoothing type %d / order %d", cfg->emf_smooth_type,
                      cfg->emf_smooth_order);
            delete s;
            return OSG_ERR_ARG;
        }
        for (int d = 0; d < cfg->dim; d++) {
            s->esmooth.order[d] = ne;
            for (int k = 0; k < 2 * ne + 1; k++) s->esmooth.c[d][k] = s->esmooth.c[0][k];
        }
        guard_cells(cfg->order, &gli, &gui);
        s->gl = std::max(s->gl, gli + ne);
        s->gu = std::max(s->gu, gui + ne);
    }
    int gcl[3] = {s->gl, s->gl, s->gl}, gcu[3] = {s->gu, s->gu, s->gu};
    s->g = make_grid(cfg->dim, s->cfg.nx, gcl, gcu);
    s->esz = cfg->precision == 32 ? 4 : 8;
    int rc = OSG_OK;
    if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("no CUDA device / stream creation failed");
        delete s;
        return OSG_ERR_CUDA;
    }
    const size_t gbytes = (size_t)s->esz * 3 * s->g.npoints();
    s->e = dalloc<char>(gbytes, &rc);
    s->b = rc ? nullptr : dalloc<char>(gbytes, &rc);
    s->j = rc ? nullptr : dalloc<char>(gbytes, &rc);
    s->d_ene = rc ? nullptr : dalloc<double>(MAX_SPECIES, &rc);
    s->d_status = rc ? nullptr : dalloc<int>(4, &rc);
    s->d_diag = rc ? nullptr : dalloc<double>(16, &rc);
    if (!rc && (s->smooth.order[0] > 0 || s->esmooth.order[0] > 0))
        s->shift_tmp = dalloc<char>(gbytes, &rc);
    if (!rc && s->esmooth.order[0] > 0) {
        s->e_part = dalloc<char>(gbytes, &rc);
        if (!rc) s->b_part = dalloc<char>(gbytes, &rc);
    }
    size_t lbytes = 0;
    if (!rc && cfg->thermal) s->d_step = dalloc<unsigned long long>(1, &rc);
    if (!rc && cfg->open_fields) {
        s->open_axis = __builtin_ctz(cfg->open_fields);
        lbytes = (size_t)s->esz * lindman_state_size(s->g, s->open_axis);
        s->lind = dalloc<char>(lbytes, &rc);
    }
    if (!rc && cfg->pml) {
        // the walls start at zero (new_wall, source/vdf/os-wall.f90:198-210); the attenuation
        // tables are computed on the host in double and stored in the field precision
        s->pml_mask = cfg->pml;
        s->pml_flags = (cfg->pml_diffuse & 3) << 4;
        s->pml_nb = cfg->pml_cells > 0 ? cfg->pml_cells : 8;
        const long n = pml_state_size(s->g, s->pml_mask, s->pml_nb);
        s->pml = dalloc<char>((size_t)s->esz * n, &rc);
        if (!rc) {
            std::vector<char> h((size_t)s->esz * n);
            if (s->esz == 4)
                pml_init_host<float>(s->g, s->pml_mask, s->pml_nb, cfg->dx, cfg->dt,
                                     (float *)h.data());
            else
                pml_init_host<double>(s->g, s->pml_mask, s->pml_nb, cfg->dx, cfg->dt,
                                      (double *)h.data());
            if (cudaMemcpy(s->pml, h.data(), h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
                rc = OSG_ERR_CUDA;
        }
    }
    if (rc) {
        osg_sim_destroy(s);
        return rc;
    }
    cudaMemsetAsync(s->e, 0, gbytes, s->st);
    cudaMemsetAsync(s->b, 0, gbytes, s->st);
    cudaMemsetAsync(s->j, 0, gbytes, s->st);
    if (s->lind) cudaMemsetAsync(s->lind, 0, lbytes, s->st);
    if (s->d_step) cudaMemsetAsync(s->d_step, 0, sizeof(unsigned long long), s->st);
    cudaMemsetAsync(s->d_status, 0, 4 * sizeof(int), s->st);
    cudaMemsetAsync(s->d_ene, 0, MAX_SPECIES * sizeof(double), s->st);
    if (cfg->engine == OSG_ENGINE_TILED) {
        rc = tiled_create(&s->tiled, s->cfg, s->g);
        if (rc) {
            osg_sim_destroy(s);
            return rc;
        }
        tiled_set_step(s->tiled, s->d_step);
    }
    if (cudaStreamSynchronize(s->st) != cudaSuccess) {
        set_error("initialisation failed");
        osg_sim_destroy(s);
        return OSG_ERR_CUDA;
    }
    *out = s;
    return OSG_OK;
}

int osg_sim_destroy(osg_sim *s)
{
    if (!s) return OSG_OK;
    if (s->st) cudaStreamSynchronize(s->st);
    drop_graphs(s);
    for (auto &p : s->plain) {
        cudaFree(p.ix);
        cudaFree(p.x);
        cudaFree(p.u);
        cudaFree(p.q);
    }
    if (s->tiled) tiled_destroy(s->tiled);
    cudaFree(s->e);
    cudaFree(s->b);
    cudaFree(s->j);
    cudaFree(s->shift_tmp);
    cudaFree(s->e_part);
    cudaFree(s->b_part);
    cudaFree(s->lind);
    cudaFree(s->pml);
    cudaFree(s->pml_tmp);
    cudaFree(s->d_step);
    cudaFree(s->d_ene);
    cudaFree(s->d_status);
    cudaFree(s->d_diag);
    cudaFree(s->d_rho);
    cudaFree(s->d_rho0);
    cudaFree(s->d_cell_cnt);
    cudaFree(s->d_scan_tmp);
    cudaFree(s->d_sort_buf);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
    return OSG_OK;
}

// plain-engine sort scratch, sized for the largest species
static int sort_scratch(osg_sim *s)
{
    const int dim = s->cfg.dim;
    size_t n = 1;
    for (long v : s->np) n = std::max(n, (size_t)v);
    const size_t need = ((size_t)sizeof(int) * dim + (size_t)s->esz * (dim + 4)) * n;
    int rc = OSG_OK;
    if (need > s->sort_buf_bytes) {
        cudaFree(s->d_sort_buf);
        s->sort_buf_bytes = 0;
        s->d_sort_buf = dalloc<char>(need, &rc);
        if (rc) return rc;
        s->sort_buf_bytes = need;
    }
    if (!s->d_cell_cnt) {
        const long nc = ncells(s->g);
        s->d_cell_cnt = dalloc<int>(nc, &rc);
        if (!rc) s->d_scan_tmp = dalloc<int>((nc + 1023) / 1024 + 1, &rc);
    }
    return rc;
}

int osg_sim_add_species(osg_sim *s, double rqm, long np, const int *ix, const void *x,
                        const void *u, const void *q)
{
    OSG_CHECK(s, OSG_ERR_ARG, "null sim");
    OSG_CHECK((int)s->np.size() < MAX_SPECIES, OSG_ERR_ARG, "too many species");
    OSG_CHECK(rqm != 0.0, OSG_ERR_ARG, "rqm must be non-zero");
    OSG_CHECK(np >= 0 && (np == 0 || (ix && x && u && q)), OSG_ERR_ARG, "bad particle arrays");
    const int dim = s->cfg.dim;
    for (long p = 0; p < np; p++)
        for (int d = 0; d < dim; d++)
            OSG_CHECK(ix[dim * p + d] >= 1 && ix[dim * p + d] <= s->cfg.nx[d], OSG_ERR_RANGE,
                      "particle %ld: cell index out of [1, nx]", p);
    const int k = (int)s->np.size();
    int rc = OSG_OK;
    if (s->cfg.engine == OSG_ENGINE_TILED) {
        OSG_CHECK(s->step_n == 0 && s->cur == 0, OSG_ERR_STATE,
                  "the tiled engine takes species only before the first step");
        rc = tiled_add_species(s->tiled, rqm, np, ix, (const float *)x, (const float *)u,
                               (const float *)q, s->st);
        if (rc) return rc;
        s->plain.emplace_back();
    } else {
        PlainSpecies p;
        const size_t n = np > 0 ? (size_t)np : 1;
        p.ix = dalloc<int>(n * dim, &rc);
        p.x = rc ? nullptr : dalloc<char>(n * dim * s->esz, &rc);
        p.u = rc ? nullptr : dalloc<char>(n * 3 * s->esz, &rc);
        p.q = rc ? nullptr : dalloc<char>(n * s->esz, &rc);
        if (rc) {
            cudaFree(p.ix);
            cudaFree(p.x);
            cudaFree(p.u);
            return rc;
        }
        if (np > 0) {
            OSG_CUDA(cudaMemcpyAsync(p.ix, ix, sizeof(int) * dim * np, cudaMemcpyHostToDevice, s->st));
            OSG_CUDA(cudaMemcpyAsync(p.x, x, (size_t)s->esz * dim * np, cudaMemcpyHostToDevice, s->st));
            OSG_CUDA(cudaMemcpyAsync(p.u, u, (size_t)s->esz * 3 * np, cudaMemcpyHostToDevice, s->st));
            OSG_CUDA(cudaMemcpyAsync(p.q, q, (size_t)s->esz * np, cudaMemcpyHostToDevice, s->st));
        }
        s->plain.push_back(p);
    }
    s->rqm.push_back(rqm);
    s->np.push_back(np);
    if (s->cfg.engine == OSG_ENGINE_PLAIN && s->cfg.n_sort > 0 && (rc = sort_scratch(s)))
        return rc;
    s->graphs_dirty = true;
    OSG_CUDA(cudaStreamSynchronize(s->st));
    return k;
}

int osg_sim_set_fields(osg_sim *s, const void *e, const void *b)
{
    OSG_CHECK(s, OSG_ERR_ARG, "null sim");
    const size_t n = (size_t)s->esz * 3 * s->g.npoints();
    if (e) OSG_CUDA(cudaMemcpyAsync(s->e, e, n, cudaMemcpyHostToDevice, s->st));
    if (b) OSG_CUDA(cudaMemcpyAsync(s->b, b, n, cudaMemcpyHostToDevice, s->st));
    OSG_CUDA(cudaStreamSynchronize(s->st));
    return OSG_OK;
}

int osg_sim_get_fields(osg_sim *s, void *e, void *b, void *j)
{
    OSG_CHECK(s, OSG_ERR_ARG, "null sim");
    const size_t n = (size_t)s->esz * 3 * s->g.npoints();
    if (e) OSG_CUDA(cudaMemcpyAsync(e, s->e, n, cudaMemcpyDeviceToHost, s->st));
    if (b) OSG_CUDA(cudaMemcpyAsync(b, s->b, n, cudaMemcpyDeviceToHost, s->st));
    if (j) OSG_CUDA(cudaMemcpyAsync(j, s->j, n, cudaMemcpyDeviceToHost, s->st));
    OSG_CUDA(cudaStreamSynchronize(s->st));
    return OSG_OK;
}

int osg_sim_num_particles(osg_sim *s, int k, long *np)
{
    OSG_CHECK(s && np && k >= 0 && k < (int)s->np.size(), OSG_ERR_ARG, "bad species");
    if (s->cfg.engine == OSG_ENGINE_TILED) return tiled_count(s->tiled, s->cur, k, np, s->st);
    *np = s->np[k];
    return OSG_OK;
}

int osg_sim_get_species(osg_sim *s, int k, int *ix, void *x, void *u, void *q)
{
    OSG_CHECK(s && k >= 0 && k < (int)s->np.size(), OSG_ERR_ARG, "bad species");
    if (s->cfg.engine == OSG_ENGINE_TILED)
        return tiled_get_species(s->tiled, s->cur, k, ix, (float *)x,
                                 (float *)u, (float *)q, s->st);
    const long np = s->np[k];
    const int dim = s->cfg.dim;
    PlainSpecies &p = s->plain[k];
    if (np > 0) {
        if (ix) OSG_CUDA(cudaMemcpyAsync(ix, p.ix, sizeof(int) * dim * np, cudaMemcpyDeviceToHost, s->st));
        if (x) OSG_CUDA(cudaMemcpyAsync(x, p.x, (size_t)s->esz * dim * np, cudaMemcpyDeviceToHost, s->st));
        if (u) OSG_CUDA(cudaMemcpyAsync(u, p.u, (size_t)s->esz * 3 * np, cudaMemcpyDeviceToHost, s->st));
        if (q) OSG_CUDA(cudaMemcpyAsync(q, p.q, (size_t)s->esz * np, cudaMemcpyDeviceToHost, s->st));
    }
    OSG_CUDA(cudaStreamSynchronize(s->st));
    return OSG_OK;
}

int osg_sim_step_async(osg_sim *s, int nsteps)
{
    OSG_CHECK(s && nsteps >= 0, OSG_ERR_ARG, "bad arguments");
    OSG_CHECK(!s->np.empty(), OSG_ERR_STATE, "no species");
    for (int i = 0; i < nsteps; i++) {
        const int parity = s->cfg.engine == OSG_ENGINE_TILED ? s->cur : 0;
        const int variant = (sort_due(s, s->step_n) || window_move_next(s, true)) ? 1 : 0;
        cudaGraphExec_t ge;
        int rc = get_graph(s, parity, variant, &ge);
        if (rc) return rc;
        OSG_CUDA(cudaGraphLaunch(ge, s->st));
        advance_buffers(s);
        s->step_n++;
    }
    return OSG_OK;
}

int osg_sim_sync(osg_sim *s)
{
    OSG_CHECK(s, OSG_ERR_ARG, "null sim");
    OSG_CUDA(cudaStreamSynchronize(s->st));
    return check_status(s);
}

int osg_sim_step(osg_sim *s, int nsteps)
{
    OSG_CHECK(s && nsteps >= 0, OSG_ERR_ARG, "bad arguments");
    // TILED: the steps go in groups of OCC_CHECK_STEPS; after each group, tile slabs filling
    // up (density bunching, injected plasma) are re-binned with room to spare before a tile can
    // overflow (particles move at most one cell per step, so a tile fills a little per step)
    const int group = s->cfg.engine == OSG_ENGINE_TILED ? OCC_CHECK_STEPS : nsteps;
    for (int done = 0; done < nsteps;) {
        const int n = std::min(group, nsteps - done);
        int rc = osg_sim_step_async(s, n);
        if (rc) return rc;
        rc = osg_sim_sync(s);
        if (rc) return rc;
        done += n;
        if (s->cfg.engine == OSG_ENGINE_TILED) {
            double m = 0.0;
            rc = tiled_occupancy(s->tiled, s->cur, &m, s->st);
            if (rc) return rc;
            if (m > 0.7) {
                rc = tiled_regrow(s->tiled, s->cur, s->st);
                if (rc) return rc;
                s->graphs_dirty = true;
            }
        }
    }
    return OSG_OK;
}

int osg_sim_set_window(osg_sim *s, int species, const int *ppc, int nprof, const double *prof_x,
                       const double *prof_f)
{
    OSG_CHECK(s, OSG_ERR_ARG, "null sim");
    OSG_CHECK(s->cfg.engine == OSG_ENGINE_TILED, OSG_ERR_ARG,
              "the moving window runs on the tiled engine");
    OSG_CHECK(s->step_n == 0, OSG_ERR_STATE, "set the window before the first step");
    OSG_CHECK(s->open_axis < 0 && (s->pml_mask & 1) == 0, OSG_ERR_ARG,
              "the moving window does not combine with Lindman boundaries or PML walls along x1");
    int rc = tiled_set_window(s->tiled, species, ppc, nprof, prof_x, prof_f);
    if (rc) return rc;
    if (!s->shift_tmp) {
        const size_t bytes = (size_t)s->esz * 3 * s->g.npoints();
        OSG_CUDA(cudaMalloc(&s->shift_tmp, bytes));
    }
    if (s->pml && !s->pml_tmp) {
        const size_t bytes = (size_t)s->esz * pml_shift_scratch(s->g, s->pml_mask, s->pml_nb);
        if (bytes) OSG_CUDA(cudaMalloc(&s->pml_tmp, bytes));
    }
    s->window = true;
    // the reference adds dt to the window motion at the start of step 1 (no move: dt < dx)
    s->xmoved = s->cfg.dt;
    s->moves = 0;
    s->graphs_dirty = true;
    return OSG_OK;
}

// ------------------------------------------------------------------------ checkpoint
// File layout (native byte order, as the reference's restart files): the tag "OSGCKPT2", the
// int size of osg_config and the struct, long step count, int window flag, double xmoved,
// long window moves, the window's injection parameters (int species, int ppc[3], int nprof,
// double prof_x[8], double prof_f[8]), int species count, then per species double rqm, long
// np and its arrays in reference layout (ix(dim,np) int, x(dim,np), u(3,np), q(np) in the
// run's precision), then long grid points and E(3,points), B(3,points) with guard cells, last,
// with Lindman open boundaries, their state (lindman_state_size reals; the reference stores
// its Lindman buffers in the restart file too, restart_write_lindman,
// source/emf/boundary/os-emf-lindman.f90:135-156), with PML walls theirs (pml_state_size
// reals: the walls, as restart_write_vpml stores its wall objects, source/emf/boundary/
// os-emf-vpml.f03:205-229, and the attenuation tables).  The current is rebuilt by the next
// step and is not stored.
namespace {

struct CkptFile {
    FILE *f = nullptr;
    ~CkptFile()
    {
        if (f) fclose(f);
    }
};

bool put(FILE *f, const void *p, size_t n) { return n == 0 || fwrite(p, 1, n, f) == n; }
bool get(FILE *f, void *p, size_t n) { return n == 0 || fread(p, 1, n, f) == n; }

const char CKPT_TAG[8] = {'O', 'S', 'G', 'C', 'K', 'P', 'T', '2'};

} // namespace

int osg_sim_checkpoint(osg_sim *s, const char *path)
{
    OSG_CHECK(s && path, OSG_ERR_ARG, "bad arguments");
    CkptFile cf;
    cf.f = fopen(path, "wb");
    OSG_CHECK(cf.f, OSG_ERR_ARG, "cannot open %s for writing", path);
    FILE *f = cf.f;
    const int csz = (int)sizeof(osg_config), win = s->window ? 1 : 0;
    int wsp = -1, wppc[3] = {1, 1, 1}, wn = 0;
    double wx[8] = {0}, wf[8] = {0};
    if (s->window) tiled_window_params(s->tiled, &wsp, wppc, &wn, wx, wf);
    const int ns = (int)s->np.size();
    bool ok = put(f, CKPT_TAG, 8) && put(f, &csz, sizeof csz) && put(f, &s->cfg, sizeof s->cfg) &&
              put(f, &s->step_n, sizeof s->step_n) && put(f, &win, sizeof win) &&
              put(f, &s->xmoved, sizeof s->xmoved) && put(f, &s->moves, sizeof s->moves) &&
              put(f, &wsp, sizeof wsp) && put(f, wppc, sizeof wppc) && put(f, &wn, sizeof wn) &&
              put(f, wx, sizeof wx) && put(f, wf, sizeof wf) && put(f, &ns, sizeof ns);
    const int dim = s->cfg.dim;
    for (int k = 0; ok && k < ns; k++) {
        long np = 0;
        int rc = osg_sim_num_particles(s, k, &np);
        if (rc) return rc;
        std::vector<int> ix((size_t)dim * np);
        std::vector<char> x((size_t)s->esz * dim * np), u((size_t)s->esz * 3 * np),
            q((size_t)s->esz * np);
        if (np > 0 && (rc = osg_sim_get_species(s, k, ix.data(), x.data(), u.data(), q.data())))
            return rc;
        ok = put(f, &s->rqm[k], sizeof(double)) && put(f, &np, sizeof np) &&
             put(f, ix.data(), ix.size() * sizeof(int)) && put(f, x.data(), x.size()) &&
             put(f, u.data(), u.size()) && put(f, q.data(), q.size());
    }
    const long npt = (long)s->g.npoints();
    std::vector<char> e((size_t)s->esz * 3 * npt), b(e.size());
    if (ok) {
        const int rc = osg_sim_get_fields(s, e.data(), b.data(), nullptr);
        if (rc) return rc;
        ok = put(f, &npt, sizeof npt) && put(f, e.data(), e.size()) && put(f, b.data(), b.size());
    }
    if (ok && s->lind) {
        std::vector<char> l((size_t)s->esz * lindman_state_size(s->g, s->open_axis));
        OSG_CUDA(cudaMemcpyAsync(l.data(), s->lind, l.size(), cudaMemcpyDeviceToHost, s->st));
        OSG_CUDA(cudaStreamSynchronize(s->st));
        ok = put(f, l.data(), l.size());
    }
    if (ok && s->pml) {
        std::vector<char> l((size_t)s->esz * pml_state_size(s->g, s->pml_mask, s->pml_nb));
        OSG_CUDA(cudaMemcpyAsync(l.data(), s->pml, l.size(), cudaMemcpyDeviceToHost, s->st));
        OSG_CUDA(cudaStreamSynchronize(s->st));
        ok = put(f, l.data(), l.size());
    }
    OSG_CHECK(ok && fflush(f) == 0, OSG_ERR_ARG, "write to %s failed", path);
    return OSG_OK;
}

int osg_sim_restore(const char *path, osg_sim **out)
{
    OSG_CHECK(path && out, OSG_ERR_ARG, "bad arguments");
    *out = nullptr;
    CkptFile cf;
    cf.f = fopen(path, "rb");
    OSG_CHECK(cf.f, OSG_ERR_ARG, "cannot open %s", path);
    FILE *f = cf.f;
    char tag[8];
    int csz = 0, win = 0, wsp = -1, wppc[3], wn = 0, ns = 0;
    osg_config cfg;
    long step_n = 0, moves = 0;
    double xmoved = 0.0, wx[8], wf[8];
    bool ok = get(f, tag, 8) && memcmp(tag, CKPT_TAG, 8) == 0 && get(f, &csz, sizeof csz) &&
              csz == (int)sizeof(osg_config) && get(f, &cfg, sizeof cfg) &&
              get(f, &step_n, sizeof step_n) && get(f, &win, sizeof win) &&
              get(f, &xmoved, sizeof xmoved) && get(f, &moves, sizeof moves) &&
              get(f, &wsp, sizeof wsp) && get(f, wppc, sizeof wppc) && get(f, &wn, sizeof wn) &&
              get(f, wx, sizeof wx) && get(f, wf, sizeof wf) && get(f, &ns, sizeof ns);
    OSG_CHECK(ok && ns >= 0 && ns <= MAX_SPECIES && step_n >= 0, OSG_ERR_ARG,
              "%s is not a checkpoint of this library", path);
    osg_sim *s = nullptr;
    int rc = osg_sim_create(&cfg, &s);
    if (rc) return rc;
    const int dim = cfg.dim, esz = s->esz;
    for (int k = 0; k < ns && rc == OSG_OK; k++) {
        double rqm = 0.0;
        long np = -1;
        if (!(get(f, &rqm, sizeof rqm) && get(f, &np, sizeof np) && np >= 0)) {
            rc = OSG_ERR_ARG;
            break;
        }
        std::vector<int> ix((size_t)dim * np);
        std::vector<char> x((size_t)esz * dim * np), u((size_t)esz * 3 * np), q((size_t)esz * np);
        if (!(get(f, ix.data(), ix.size() * sizeof(int)) && get(f, x.data(), x.size()) &&
              get(f, u.data(), u.size()) && get(f, q.data(), q.size()))) {
            rc = OSG_ERR_ARG;
            break;
        }
        rc = osg_sim_add_species(s, rqm, np, ix.data(), x.data(), u.data(), q.data());
        if (rc > 0) rc = OSG_OK;   // the species index
    }
    long npt = 0;
    if (rc == OSG_OK) {
        std::vector<char> e((size_t)esz * 3 * s->g.npoints()), b(e.size());
        if (!(get(f, &npt, sizeof npt) && npt == (long)s->g.npoints() && get(f, e.data(), e.size()) &&
              get(f, b.data(), b.size())))
            rc = OSG_ERR_ARG;
        else
            rc = osg_sim_set_fields(s, e.data(), b.data());
    }
    if (rc == OSG_OK && s->lind) {
        std::vector<char> l((size_t)esz * lindman_state_size(s->g, s->open_axis));
        if (!get(f, l.data(), l.size())) {
            rc = OSG_ERR_ARG;
        } else if (cudaMemcpyAsync(s->lind, l.data(), l.size(), cudaMemcpyHostToDevice, s->st) !=
                       cudaSuccess ||
                   cudaStreamSynchronize(s->st) != cudaSuccess) {
            set_error("upload of the Lindman state failed");
            rc = OSG_ERR_CUDA;
        }
    }
    if (rc == OSG_OK && s->pml) {
        std::vector<char> l((size_t)esz * pml_state_size(s->g, s->pml_mask, s->pml_nb));
        if (!get(f, l.data(), l.size())) {
            rc = OSG_ERR_ARG;
        } else if (cudaMemcpyAsync(s->pml, l.data(), l.size(), cudaMemcpyHostToDevice, s->st) !=
                       cudaSuccess ||
                   cudaStreamSynchronize(s->st) != cudaSuccess) {
            set_error("upload of the PML state failed");
            rc = OSG_ERR_CUDA;
        }
    }
    if (rc == OSG_OK && win) {
        rc = osg_sim_set_window(s, wsp, wppc, wn, wx, wf);
        if (rc == OSG_OK) rc = tiled_set_moves(s->tiled, moves, s->st);
        s->xmoved = xmoved;
        s->moves = moves;
    }
    if (rc != OSG_OK) {
        osg_sim_destroy(s);
        if (rc == OSG_ERR_ARG) set_error("%s: truncated or inconsistent checkpoint", path);
        return rc;
    }
    s->step_n = step_n;
    if (s->d_step) {
        const unsigned long long v = (unsigned long long)step_n;
        if (cudaMemcpy(s->d_step, &v, sizeof v, cudaMemcpyHostToDevice) != cudaSuccess) {
            osg_sim_destroy(s);
            set_error("upload of the step counter failed");
            return OSG_ERR_CUDA;
        }
    }
    *out = s;
    return OSG_OK;
}

int osg_sim_get_config(osg_sim *s, osg_config *cfg, int *nspecies, double *rqm)
{
    OSG_CHECK(s && cfg && nspecies, OSG_ERR_ARG, "bad arguments");
    *cfg = s->cfg;
    *nspecies = (int)s->np.size();
    if (rqm)
        for (int k = 0; k < *nspecies; k++) rqm[k] = s->rqm[k];
    return OSG_OK;
}

int osg_sim_guard_cells(osg_sim *s, int *gcl, int *gcu)
{
    OSG_CHECK(s && gcl && gcu, OSG_ERR_ARG, "bad arguments");
    for (int d = 0; d < s->cfg.dim; d++) {
        gcl[d] = s->g.gcl[d];
        gcu[d] = s->g.gcu[d];
    }
    return OSG_OK;
}

int osg_sim_window_moves(osg_sim *s, long *moves)
{
    OSG_CHECK(s && moves, OSG_ERR_ARG, "bad arguments");
    *moves = s->moves;
    return OSG_OK;
}

int osg_sim_tile_occupancy(osg_sim *s, double *max_frac)
{
    OSG_CHECK(s && max_frac, OSG_ERR_ARG, "bad arguments");
    *max_frac = 0.0;
    if (s->cfg.engine != OSG_ENGINE_TILED) return OSG_OK;
    return tiled_occupancy(s->tiled, s->cur, max_frac, s->st);
}

void *osg_sim_stream(osg_sim *s) { return s ? (void *)s->st : nullptr; }

int osg_sim_energy(osg_sim *s, double *kinetic, double *field)
{
    OSG_CHECK(s, OSG_ERR_ARG, "null sim");
    double dv = 1.0;
    for (int d = 0; d < s->cfg.dim; d++) dv *= s->cfg.dx[d];
    if (kinetic) {
        double h[MAX_SPECIES];
        OSG_CUDA(cudaMemcpyAsync(h, s->d_ene, sizeof(double) * MAX_SPECIES, cudaMemcpyDeviceToHost, s->st));
        OSG_CUDA(cudaStreamSynchronize(s->st));
        // get_energy normalisation, source/spec/os-spec-define.f03:1079-1084
        for (size_t k = 0; k < s->np.size(); k++) kinetic[k] = h[k] * s->rqm[k] * dv;
    }
    if (field) {
        OSG_CUDA(cudaMemsetAsync(s->d_diag, 0, 6 * sizeof(double), s->st));
        if (s->cfg.precision == 32) {
            field_sumsq<float>(s->g, (const float *)s->e, s->d_diag, s->st);
            field_sumsq<float>(s->g, (const float *)s->b, s->d_diag + 3, s->st);
        } else {
            field_sumsq<double>(s->g, (const double *)s->e, s->d_diag, s->st);
            field_sumsq<double>(s->g, (const double *)s->b, s->d_diag + 3, s->st);
        }
        OSG_CUDA(cudaGetLastError());
        double h[6];
        OSG_CUDA(cudaMemcpyAsync(h, s->d_diag, sizeof h, cudaMemcpyDeviceToHost, s->st));
        OSG_CUDA(cudaStreamSynchronize(s->st));
        for (int c = 0; c < 6; c++) field[c] = 0.5 * dv * h[c];
    }
    return OSG_OK;
}

int osg_sim_gauss_residual(osg_sim *s, double *max_abs, double *l2)
{
    OSG_CHECK(s, OSG_ERR_ARG, "null sim");
    OSG_CHECK(s->cfg.walls == 0 && s->cfg.open_fields == 0 && s->cfg.pml == 0, OSG_ERR_STATE,
              "the Gauss residual is taken on periodic boxes (no walls or open edges)");
    const size_t n = 3 * (size_t)s->g.npoints();
    int rc = OSG_OK;
    if (!s->d_rho) s->d_rho = dalloc<double>(n, &rc);
    if (rc) return rc;
    OSG_CUDA(cudaMemsetAsync(s->d_rho, 0, n * sizeof(double), s->st));
    for (size_t k = 0; k < s->np.size(); k++) {
        if (s->cfg.engine == OSG_ENGINE_TILED) {
            rc = tiled_deposit_rho(s->tiled, s->cur, (int)k, s->d_rho,
                                   s->d_status, s->st);
        } else if (s->cfg.precision == 32) {
            rc = deposit_rho<float>(s->g, s->cfg.order, s->plain[k].ix, (const float *)s->plain[k].x,
                                    (const float *)s->plain[k].q, s->np[k], s->d_rho, s->d_status, s->st);
        } else {
            rc = deposit_rho<double>(s->g, s->cfg.order, s->plain[k].ix, (const double *)s->plain[k].x,
                                     (const double *)s->plain[k].q, s->np[k], s->d_rho, s->d_status, s->st);
        }
        if (rc) return rc;
    }
    periodic_update<double>(s->g, s->d_rho, 1, s->st);
    // div E reads the lower neighbour of the first interior cell: refresh the E guard cells
    // (the next step starts with the same replace, so this changes nothing downstream)
    if (s->cfg.precision == 32) periodic_update<float>(s->g, (float *)s->e, 0, s->st);
    else periodic_update<double>(s->g, (double *)s->e, 0, s->st);
    OSG_CUDA(cudaMemsetAsync(s->d_diag, 0, 2 * sizeof(double), s->st));
    unsigned long long *dmax = (unsigned long long *)s->d_diag;
    if (s->cfg.precision == 32)
        gauss_residual<float>(s->g, (const float *)s->e, s->d_rho, nullptr, s->cfg.dx, dmax,
                              s->d_diag + 1, s->st);
    else
        gauss_residual<double>(s->g, (const double *)s->e, s->d_rho, nullptr, s->cfg.dx, dmax,
                               s->d_diag + 1, s->st);
    OSG_CUDA(cudaGetLastError());
    double h[2];
    OSG_CUDA(cudaMemcpyAsync(h, s->d_diag, sizeof h, cudaMemcpyDeviceToHost, s->st));
    OSG_CUDA(cudaStreamSynchronize(s->st));
    unsigned long long bits;
    memcpy(&bits, &h[0], sizeof bits);
    double m;
    memcpy(&m, &bits, sizeof m);
    if (max_abs) *max_abs = m;
    if (l2) *l2 = std::sqrt(h[1]);
    return check_status(s);
}

int osg_sim_profile(osg_sim *s, int nsteps, float *ms_phase)
{
    OSG_CHECK(s && ms_phase && nsteps > 0, OSG_ERR_ARG, "bad arguments");
    OSG_CHECK(!s->np.empty(), OSG_ERR_STATE, "no species");
    PhaseEvents pe;
    for (int i = 0; i < 6; i++) OSG_CUDA(cudaEventCreate(&pe.ev[i]));
    float acc[5] = {0, 0, 0, 0, 0};
    int rc = OSG_OK;
    for (int it = 0; it < nsteps && !rc; it++) {
        const int parity = s->cfg.engine == OSG_ENGINE_TILED ? s->cur : 0;
        const bool sort = sort_due(s, s->step_n);
        const bool move = window_move_next(s, true);
        rc = enqueue_step_any(s, parity, sort, move, &pe);
        if (rc) break;
        advance_buffers(s);
        s->step_n++;
        if (cudaEventSynchronize(pe.ev[5]) != cudaSuccess) {
            set_error("profiled step failed");
            rc = OSG_ERR_CUDA;
            break;
        }
        float t;
        cudaEventElapsedTime(&t, pe.ev[1], pe.ev[2]); acc[0] += t;   // push + deposit
        cudaEventElapsedTime(&t, pe.ev[3], pe.ev[4]); acc[1] += t;   // fold
        cudaEventElapsedTime(&t, pe.ev[4], pe.ev[5]); acc[2] += t;   // Yee
        cudaEventElapsedTime(&t, pe.ev[0], pe.ev[1]); acc[3] += t;   // replace
        cudaEventElapsedTime(&t, pe.ev[2], pe.ev[3]); acc[4] += t;   // sort
    }
    for (int i = 0; i < 6; i++) cudaEventDestroy(pe.ev[i]);
    if (rc) return rc;
    for (int i = 0; i < 5; i++) ms_phase[i] = acc[i] / nsteps;
    return check_status(s);
}

// ------------------------------------------------------------------------ autotuner
// Device state that trial steps change and the tuner puts back: fields, Lindman planes,
// thermal-bath step counter (the particles are either copied too, PLAIN, or live in a separate
// trial TiledState, TILED).
struct SavedState {
    std::vector<void *> buf;
    std::vector<std::pair<void *, size_t>> where;
    long step_n = 0;
    int cur = 0;
    ~SavedState()
    {
        for (void *p : buf) cudaFree(p);
    }
    int save(void *p, size_t bytes, cudaStream_t st)
    {
        if (!p || bytes == 0) return OSG_OK;
        void *c = nullptr;
        OSG_CUDA(cudaMalloc(&c, bytes));
        buf.push_back(c);
        where.push_back({p, bytes});
        OSG_CUDA(cudaMemcpyAsync(c, p, bytes, cudaMemcpyDeviceToDevice, st));
        return OSG_OK;
    }
    int restore(osg_sim *s)
    {
        for (size_t i = 0; i < buf.size(); i++)
            OSG_CUDA(cudaMemcpyAsync(where[i].first, buf[i], where[i].second,
                                     cudaMemcpyDeviceToDevice, s->st));
        OSG_CUDA(cudaMemsetAsync(s->d_ene, 0, MAX_SPECIES * sizeof(double), s->st));
        OSG_CUDA(cudaStreamSynchronize(s->st));
        s->step_n = step_n;
        s->cur = cur;
        s->graphs_dirty = true;
        return OSG_OK;
    }
};

static int save_fields(osg_sim *s, SavedState &sv)
{
    const size_t gbytes = (size_t)s->esz * 3 * s->g.npoints();
    int rc;
    if ((rc = sv.save(s->e, gbytes, s->st)) || (rc = sv.save(s->b, gbytes, s->st)) ||
        (rc = sv.save(s->j, gbytes, s->st)))
        return rc;
    if (s->lind &&
        (rc = sv.save(s->lind, (size_t)s->esz * lindman_state_size(s->g, s->open_axis), s->st)))
        return rc;
    if (s->pml &&
        (rc = sv.save(s->pml, (size_t)s->esz * pml_state_size(s->g, s->pml_mask, s->pml_nb),
                      s->st)))
        return rc;
    if (s->d_step && (rc = sv.save(s->d_step, sizeof(unsigned long long), s->st))) return rc;
    sv.step_n = s->step_n;
    sv.cur = s->cur;
    return OSG_OK;
}

// device ms of n steps (graph replays) after w untimed ones
static int time_trial(osg_sim *s, int w, int n, float *ms)
{
    int rc = osg_sim_step_async(s, w);
    if (rc) return rc;
    return osg_sim_time_steps(s, n, ms);
}

// TILED: every candidate tile shape x CTA size runs on a trial copy of the particles
static int tune_tiled(osg_sim *s, int steps, int *tile, int *threads)
{
    const int dim = s->cfg.dim;
    const int ns = (int)s->np.size();
    // the particles, once, on the host (the trial states are binned from them)
    std::vector<std::vector<int>> hix(ns);
    std::vector<std::vector<float>> hx(ns), hu(ns), hq(ns);
    std::vector<long> hnp(ns);
    int rc;
    for (int k = 0; k < ns; k++) {
        if ((rc = tiled_count(s->tiled, s->cur, k, &hnp[k], s->st))) return rc;
        const size_t n = (size_t)std::max(hnp[k], 1L);
        hix[k].resize(n * dim);
        hx[k].resize(n * dim);
        hu[k].resize(n * 3);
        hq[k].resize(n);
        if ((rc = tiled_get_species(s->tiled, s->cur, k, hix[k].data(), hx[k].data(),
                                    hu[k].data(), hq[k].data(), s->st)))
            return rc;
    }
    SavedState sv;
    if ((rc = save_fields(s, sv))) return rc;
    std::vector<std::array<int, 3>> tiles;
    if (dim == 2) tiles = {{8, 8, 1}, {16, 8, 1}, {8, 4, 1}, {16, 16, 1}};
    else tiles = {{8, 8, 4}, {8, 4, 4}, {4, 4, 4}, {8, 8, 8}};
    const int thr[2] = {256, 128};
    TiledState *orig = s->tiled;
    float best = 1e30f;
    int bestT[3] = {0, 0, 0}, best_th = 0;
    for (const auto &T : tiles) {
        bool fits = true;
        for (int d = 0; d < dim; d++) fits = fits && T[d] <= s->cfg.nx[d] && s->cfg.nx[d] % T[d] == 0;
        if (!fits) continue;
        for (int th : thr) {
            osg_config c = s->cfg;
            for (int d = 0; d < 3; d++) c.tile[d] = d < dim ? T[d] : 1;
            TiledState *tr = nullptr;
            rc = tiled_create(&tr, c, s->g);
            if (rc) continue;   // does not fit (shared memory, tile cells)
            tiled_set_step(tr, s->d_step);
            rc = tiled_set_threads(tr, th);
            for (int k = 0; k < ns && !rc; k++)
                rc = tiled_add_species(tr, s->rqm[k], hnp[k], hix[k].data(), hx[k].data(),
                                       hu[k].data(), hq[k].data(), s->st);
            float ms = 0.0f;
            if (!rc) {
                s->tiled = tr;
                s->cur = 0;
                s->graphs_dirty = true;
                rc = time_trial(s, 2, steps, &ms);
                if (!rc) rc = check_status(s);
                drop_graphs(s);
                s->tiled = orig;
            }
            tiled_destroy(tr);
            const int rs = sv.restore(s);
            if (rs) return rs;
            if (rc == OSG_ERR_CUDA) return rc;
            if (rc) continue;
            if (ms < best) {
                best = ms;
                for (int d = 0; d < 3; d++) bestT[d] = d < dim ? T[d] : 1;
                best_th = th;
            }
        }
    }
    OSG_CHECK(best_th > 0, OSG_ERR_ARG, "autotuner: no candidate tile shape fits the box");
    // rebuild the engine with the winner (from the host copy of the particles)
    bool same = best_th == tiled_threads(orig);
    for (int d = 0; d < dim; d++) same = same && bestT[d] == s->cfg.tile[d];
    if (!same) {
        osg_config c = s->cfg;
        for (int d = 0; d < 3; d++) c.tile[d] = bestT[d];
        TiledState *nt = nullptr;
        if ((rc = tiled_create(&nt, c, s->g))) return rc;
        tiled_set_step(nt, s->d_step);
        rc = tiled_set_threads(nt, best_th);
        for (int k = 0; k < ns && !rc; k++)
            rc = tiled_add_species(nt, s->rqm[k], hnp[k], hix[k].data(), hx[k].data(),
                                   hu[k].data(), hq[k].data(), s->st);
        if (rc) {
            tiled_destroy(nt);
            return rc;
        }
        drop_graphs(s);
        tiled_destroy(orig);
        s->tiled = nt;
        s->cur = 0;
        for (int d = 0; d < 3; d++) s->cfg.tile[d] = bestT[d];
        s->graphs_dirty = true;
    }
    for (int d = 0; d < 3; d++) tile[d] = bestT[d];
    *threads = best_th;
    return OSG_OK;
}

// PLAIN: the cell-sort interval from a cost model.  Unsorted steps get slower as the particles
// lose their cell order (scattered gathers and current atomics); a sort costs C once.  Sorting
// every n steps costs (C + g (0 + 1 + ... + (n - 1))) / n per step on top of a sorted step,
// g = the growth of the push time per unsorted step, minimal at n = sqrt(2 C / g).  The tuner
// measures g over `steps` unsorted steps from a sorted state (least-squares slope of the push
// times) and C as the sort phase of one step.
static int tune_sort(osg_sim *s, int steps, int *n_sort)
{
    SavedState sv;
    int rc = sort_scratch(s);
    if (rc) return rc;
    const int dim = s->cfg.dim;
    for (size_t k = 0; k < s->plain.size(); k++) {
        const size_t n = (size_t)std::max(s->np[k], 1L);
        PlainSpecies &p = s->plain[k];
        // the sort permutes every array, charges included
        if ((rc = sv.save(p.ix, sizeof(int) * dim * n, s->st)) ||
            (rc = sv.save(p.x, (size_t)s->esz * dim * n, s->st)) ||
            (rc = sv.save(p.u, (size_t)s->esz * 3 * n, s->st)) ||
            (rc = sv.save(p.q, (size_t)s->esz * n, s->st)))
            return rc;
    }
    if ((rc = save_fields(s, sv))) return rc;
    const int keep = s->cfg.n_sort;
    PhaseEvents pe;
    for (int i = 0; i < 6; i++) OSG_CUDA(cudaEventCreate(&pe.ev[i]));
    std::vector<double> push;
    float c_sort = 0.0f;
    // one sorted step first (the measurement starts from cell order), then `steps` unsorted
    for (int it = 0; it <= steps && !rc; it++) {
        rc = enqueue_step_any(s, 0, it == 0, false, &pe);
        if (rc) break;
        s->step_n++;
        if (cudaEventSynchronize(pe.ev[5]) != cudaSuccess) {
            set_error("tuning step failed");
            rc = OSG_ERR_CUDA;
            break;
        }
        float t = 0.0f;
        if (it == 0) {
            cudaEventElapsedTime(&t, pe.ev[2], pe.ev[3]);
            c_sort = t;
        } else {
            cudaEventElapsedTime(&t, pe.ev[1], pe.ev[2]);
            push.push_back(t);
        }
    }
    for (int i = 0; i < 6; i++) cudaEventDestroy(pe.ev[i]);
    if (!rc) rc = check_status(s);
    const int rs = sv.restore(s);
    s->cfg.n_sort = keep;
    if (rc) return rc;
    if (rs) return rs;
    // least-squares slope of the push time over the unsorted steps
    const int m = (int)push.size();
    double sx = 0, sy = 0, sxx = 0, sxy = 0;
    for (int i = 0; i < m; i++) {
        sx += i;
        sy += push[i];
        sxx += (double)i * i;
        sxy += i * push[i];
    }
    const double den = m * sxx - sx * sx;
    const double g = den > 0 ? (m * sxy - sx * sy) / den : 0.0;
    int n = 0;   // never: the push does not slow down measurably
    if (g > 1e-6 * std::max(sy / std::max(m, 1), 1e-6))
        n = (int)std::lround(std::sqrt(2.0 * c_sort / g));
    n = std::max(0, std::min(n, 100000));
    if (g > 0 && n == 0) n = 1;
    s->cfg.n_sort = n;
    s->graphs_dirty = true;
    *n_sort = n;
    return OSG_OK;
}

int osg_sim_autotune(osg_sim *s, int steps, int *tile, int *threads, int *n_sort)
{
    OSG_CHECK(s && tile && threads && n_sort && steps >= 2 && steps <= 1000, OSG_ERR_ARG,
              "bad arguments");
    OSG_CHECK(!s->np.empty(), OSG_ERR_STATE, "no species");
    OSG_CHECK(s->step_n == 0, OSG_ERR_STATE, "autotune before the first step");
    OSG_CHECK(!s->window, OSG_ERR_STATE, "the autotuner does not run with the moving window");
    for (int d = 0; d < 3; d++) tile[d] = 0;
    *threads = 0;
    *n_sort = s->cfg.n_sort;
    int rc = s->cfg.engine == OSG_ENGINE_TILED ? tune_tiled(s, steps, tile, threads)
                                               : tune_sort(s, steps, n_sort);
    if (rc) return rc;
    return check_status(s);
}

int osg_sim_launches_per_step(osg_sim *s) { return s ? s->launches_per_step : 0; }

int osg_sim_time_steps(osg_sim *s, int nsteps, float *ms)
{
    OSG_CHECK(s && ms && nsteps > 0, OSG_ERR_ARG, "bad arguments");
    cudaEvent_t a, b;
    OSG_CUDA(cudaEventCreate(&a));
    OSG_CUDA(cudaEventCreate(&b));
    int rc = OSG_OK;
    if (cudaEventRecord(a, s->st) != cudaSuccess) rc = OSG_ERR_CUDA;
    if (!rc) rc = osg_sim_step_async(s, nsteps);
    if (!rc && cudaEventRecord(b, s->st) != cudaSuccess) rc = OSG_ERR_CUDA;
    if (!rc && cudaEventSynchronize(b) != cudaSuccess) rc = OSG_ERR_CUDA;
    if (!rc) cudaEventElapsedTime(ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc == OSG_ERR_CUDA) set_error("timed steps failed");
    if (rc) return rc;
    return check_status(s);
}

} // extern "C"
